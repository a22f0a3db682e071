// iq_simulate: the iqsim driver (src/iqsim.jl:50-315) on the GPU.
//
// All realizations of a call share the tile path (genpath runs once per call,
// src/iqsim.jl:139), so every step processes one tile for the whole batch of realizations:
//   gather templates -> batched overlap distance -> [hard distance] -> pick (one CTA per
//   realization) -> graph cuts (one CTA per realization and slab) -> paste.
// The hard and soft distance terms do not depend on the realization; the soft maps of all
// tiles are computed up front in batches of 16 tiles and kept resident in HBM, the hard map
// of a data tile is computed once per step. Nothing is copied back to the host until the
// crop at the end.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <cmath>
#include <unordered_map>
#include <vector>

#include "iq_internal.h"

// ---------------------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------------------
namespace {

struct PathStream {
  uint64_t seed;
  uint32_t i = 0;
  explicit PathStream(uint64_t s) : seed(s) {}
  uint64_t below(uint64_t m) {
    uint64_t v = iq_rand64(seed, i++, 0u, 2u);
    return (uint64_t)(((unsigned __int128)v * m) >> 64);
  }
  void shuffle(std::vector<int64_t>& a) {
    for (int64_t i2 = (int64_t)a.size() - 1; i2 > 0; --i2) {
      int64_t j = (int64_t)below((uint64_t)i2 + 1);
      std::swap(a[i2], a[j]);
    }
  }
};

struct Grid3 {
  int64_t e[3];
  int64_t vol() const { return e[0] * e[1] * e[2]; }
};

// 3^N box dilation of a boolean grid (outside = false)
std::vector<uint8_t> dilate(const std::vector<uint8_t>& g, const Grid3& d) {
  std::vector<uint8_t> o(g.size(), 0);
  for (int64_t z = 0; z < d.e[2]; ++z)
    for (int64_t y = 0; y < d.e[1]; ++y)
      for (int64_t x = 0; x < d.e[0]; ++x) {
        uint8_t v = 0;
        for (int64_t dz = -1; dz <= 1 && !v; ++dz)
          for (int64_t dy = -1; dy <= 1 && !v; ++dy)
            for (int64_t dx = -1; dx <= 1 && !v; ++dx) {
              int64_t X = x + dx, Y = y + dy, Z = z + dz;
              if (X < 0 || Y < 0 || Z < 0 || X >= d.e[0] || Y >= d.e[1] || Z >= d.e[2]) continue;
              v = g[X + d.e[0] * (Y + d.e[1] * Z)];
            }
        o[x + d.e[0] * (y + d.e[1] * z)] = v;
      }
  return o;
}

void dilation_rings(std::vector<uint8_t>& grid, const Grid3& d, std::vector<int64_t>& path) {
  for (;;) {
    bool all = true;
    for (uint8_t v : grid) all = all && v;
    if (all) break;
    std::vector<uint8_t> dl = dilate(grid, d);
    for (int64_t i = 0; i < (int64_t)dl.size(); ++i)
      if (dl[i] && !grid[i]) path.push_back(i);
    grid.swap(dl);
  }
}

}  // namespace

// genpath (src/utils.jl:158-204) with the Philox path stream
static std::vector<int64_t> genpath_host(uint64_t seed, const Grid3& ext, int kind,
                                         std::vector<int64_t> datainds) {
  PathStream rs(seed);
  const int64_t n = ext.vol();
  std::vector<int64_t> path;
  path.reserve(n);
  if (datainds.empty()) {
    if (kind == IQ_PATH_RASTER) {
      for (int64_t i = 0; i < n; ++i) path.push_back(i);
    } else if (kind == IQ_PATH_RANDOM) {
      path.resize(n);
      for (int64_t i = 0; i < n; ++i) path[i] = i;
      rs.shuffle(path);
    } else {
      int64_t pivot = (int64_t)rs.below((uint64_t)n);
      std::vector<uint8_t> grid(n, 0);
      grid[pivot] = 1;
      path.push_back(pivot);
      dilation_rings(grid, ext, path);
    }
  } else {
    rs.shuffle(datainds);
    std::vector<uint8_t> grid(n, 0);
    for (int64_t p : datainds) {
      grid[p] = 1;
      path.push_back(p);
    }
    dilation_rings(grid, ext, path);
  }
  return path;
}

extern "C" int iq_genpath(uint64_t seed, int32_t ndim, const int64_t* extent, int32_t kind,
                          int64_t ndata, const int64_t* datainds, int64_t* path_out) {
  if (ndim < 1 || ndim > 3 || !extent || !path_out || ndata < 0 || (ndata > 0 && !datainds))
    return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (kind < 0 || kind > 2) return iq_set_error(IQ_ERR_ARG, "invalid simulation path");
  Grid3 g{{1, 1, 1}};
  for (int d = 0; d < ndim; ++d) {
    if (extent[d] <= 0) return iq_set_error(IQ_ERR_ARG, "extents must be positive");
    g.e[d] = extent[d];
  }
  std::vector<int64_t> di(datainds, datainds + ndata);
  for (int64_t v : di)
    if (v < 0 || v >= g.vol()) return iq_set_error(IQ_ERR_ARG, "data tile index out of range");
  std::vector<int64_t> p = genpath_host(seed, g, kind, di);
  std::copy(p.begin(), p.end(), path_out);
  return IQ_OK;
}

void iq_relax_sizes(int64_t npat, double tol, int64_t& dbnorm, int64_t& dbzero, int& nnorm,
                    int64_t* seqnorm, int& nzero, int64_t* seqzero) {
  auto seq = [&](int64_t dbsize, int64_t* out) {
    int n = 0;
    double frac = 0.1 * ((double)dbsize / (double)npat);
    for (;;) {
      out[n++] = (int64_t)std::ceil(frac * (double)npat);
      if (frac >= 1.0 || n >= IQ_MAX_SEQ) break;
      frac = std::min(frac + 0.1, 1.0);
    }
    return n;
  };
  dbnorm = (int64_t)std::ceil(tol * (double)npat);
  dbzero = npat;
  nnorm = seq(dbnorm, seqnorm);
  nzero = seq(dbzero, seqzero);
}

// ---------------------------------------------------------------------------------------
// iq_simulate
// ---------------------------------------------------------------------------------------
namespace {

struct Geo {
  int ndim;
  int64_t tile[3], ovl[3], spacing[3], ntiles[3], pad[3], sim[3], dist[3];
  int64_t ovlvol;
  int64_t ntot;
};

struct MaskCfg {
  int prev[3], next[3];
  int64_t lo[3], hi[3];
  int K;
  int id;
};

#define RET_IF(rc_expr)              \
  do {                               \
    int rc_ = (rc_expr);             \
    if (rc_) return rc_;             \
  } while (0)

}  // namespace

extern "C" int iq_simulate(iq_ctx* ctx, const iq_sim_params* p, const iq_hard_data* hard,
                           int32_t nsoft, const iq_soft_data* soft, float* reals, float* cuts,
                           double* voxs) {
  if (!ctx || !p || !reals) return iq_set_error(IQ_ERR_ARG, "null argument");
  if (!ctx->has_ti) return iq_set_error(IQ_ERR_STATE, "no training image set");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  const int N = p->ndim;
  if (N != ctx->ndim) return iq_set_error(IQ_ERR_ARG, "ndim differs from the training image");
  const int64_t TIe[3] = {ctx->ti.x, ctx->ti.y, ctx->ti.z};

  // ---- sanity checks (src/iqsim.jl:68-89) ----
  for (int d = 0; d < N; ++d)
    if (!(p->tilesize[d] > 0 && p->tilesize[d] <= TIe[d]))
      return iq_set_error(IQ_ERR_ARG, "invalid tile size");
  for (int d = 0; d < N; ++d)
    if (!(p->simsize[d] >= p->tilesize[d])) return iq_set_error(IQ_ERR_ARG, "invalid grid size");
  for (int d = 0; d < N; ++d)
    if (!(p->overlap[d] > 0 && p->overlap[d] < 1))
      return iq_set_error(IQ_ERR_ARG, "overlaps must be in range (0,1)");
  if (!(p->tol > 0 && p->tol <= 1)) return iq_set_error(IQ_ERR_ARG, "tolerance must be in range (0,1]");
  if (p->path < 0 || p->path > 2) return iq_set_error(IQ_ERR_ARG, "invalid simulation path");
  if (p->nreal <= 0) return iq_set_error(IQ_ERR_ARG, "invalid number of realizations");
  if (p->real0 < 0 || p->real0 + p->nreal > ((int64_t)1 << 32))
    return iq_set_error(IQ_ERR_ARG, "realization range outside [0, 2^32)");
  if (nsoft < 0 || (nsoft > 0 && !soft)) return iq_set_error(IQ_ERR_ARG, "invalid soft data");
  if (nsoft + 1 > IQ_MAX_AUX) return iq_set_error(IQ_ERR_LIMIT, "at most %d soft variables", IQ_MAX_AUX - 1);
  for (int s = 0; s < nsoft; ++s) {
    if (!soft[s].aux || !soft[s].auxti) return iq_set_error(IQ_ERR_ARG, "null soft data");
    for (int d = 0; d < N; ++d)
      if (!(soft[s].auxsize[d] >= p->simsize[d]))
        return iq_set_error(IQ_ERR_ARG, "soft data size < grid size");
  }
  for (int d = 0; d < N; ++d)
    if (p->tilesize[d] >= 1024) return iq_set_error(IQ_ERR_LIMIT, "tile extent >= 1024");

  // ---- geometry (src/iqsim.jl:91-115) ----
  Geo g;
  g.ndim = N;
  for (int d = 0; d < 3; ++d) {
    if (d < N) {
      g.tile[d] = p->tilesize[d];
      g.ovl[d] = (int64_t)std::ceil(p->overlap[d] * (double)p->tilesize[d]);
      g.spacing[d] = g.tile[d] - g.ovl[d];
      g.sim[d] = p->simsize[d];
      g.ntiles[d] = (int64_t)std::ceil((double)g.sim[d] / (double)std::max<int64_t>(g.spacing[d], 1));
      g.pad[d] = g.ntiles[d] * (g.tile[d] - g.ovl[d]) + g.ovl[d];
      if (g.pad[d] < g.sim[d])
        return iq_set_error(IQ_ERR_ARG, "tiles with zero spacing cannot cover the grid");
    } else {
      g.tile[d] = 1; g.ovl[d] = 0; g.spacing[d] = 1; g.sim[d] = 1; g.ntiles[d] = 1; g.pad[d] = 1;
    }
    g.dist[d] = TIe[d] - g.tile[d] + 1;
  }
  {
    int64_t a = 1, b = 1;
    for (int d = 0; d < 3; ++d) { a *= g.pad[d]; b *= g.pad[d] - (g.ntiles[d] - 1) * g.ovl[d]; }
    g.ovlvol = a - b;
  }
  g.ntot = g.ntiles[0] * g.ntiles[1] * g.ntiles[2];
  const Dim3 padD{g.pad[0], g.pad[1], g.pad[2]};
  const Dim3 tileD{g.tile[0], g.tile[1], g.tile[2]};
  const Dim3 distD{g.dist[0], g.dist[1], g.dist[2]};
  const Dim3 simD{g.sim[0], g.sim[1], g.sim[2]};
  const int64_t padvol = padD.vol(), T = tileD.vol(), P = distD.vol(), simvol = simD.vol();
  if (P >= ((int64_t)1 << 31)) return iq_set_error(IQ_ERR_LIMIT, "distance map above 2^31");
  const int R = p->nreal;
  cudaStream_t st = ctx->stream;

  // ---- hard data (src/utils.jl:18-55,131-156) ----
  int64_t nh = hard ? hard->n : 0;
  std::vector<int64_t> hcoord(nh * N);
  std::vector<double> hval(nh);
  if (nh > 0) {
    if (!hard->coords || !hard->values) return iq_set_error(IQ_ERR_ARG, "null hard data");
    IQ_CUDA_OK(cudaMemcpy(hcoord.data(), hard->coords, sizeof(int64_t) * nh * N, cudaMemcpyDefault));
    IQ_CUDA_OK(cudaMemcpy(hval.data(), hard->values, sizeof(double) * nh, cudaMemcpyDefault));
    for (int64_t i = 0; i < nh; ++i)
      for (int d = 0; d < N; ++d) {
        if (hcoord[i * N + d] >= g.sim[d]) return iq_set_error(IQ_ERR_ARG, "hard data coordinates outside of grid");
        if (hcoord[i * N + d] < 0) return iq_set_error(IQ_ERR_ARG, "hard data coordinates must be positive indices");
      }
  }
  // unique coordinates (the reference's Dict): last one wins
  std::unordered_map<int64_t, int64_t> hidx;
  std::vector<int64_t> hlin;
  std::vector<double> hv;
  for (int64_t i = 0; i < nh; ++i) {
    int64_t c[3] = {0, 0, 0};
    for (int d = 0; d < N; ++d) c[d] = hcoord[i * N + d];
    int64_t lin = c[0] + g.pad[0] * (c[1] + g.pad[1] * c[2]);
    auto it = hidx.find(lin);
    if (it == hidx.end()) {
      hidx[lin] = (int64_t)hlin.size();
      hlin.push_back(lin);
      hv.push_back(hval[i]);
    } else {
      hv[it->second] = hval[i];
    }
  }
  nh = (int64_t)hlin.size();
  std::vector<int64_t> nan_cnt(g.ntot, 0);
  std::vector<uint8_t> has_data(g.ntot, 0);
  std::vector<std::vector<std::pair<uint32_t, float>>> tile_hard(g.ntot);
  for (int64_t i = 0; i < nh; ++i) {
    int64_t c[3] = {hlin[i] % g.pad[0], (hlin[i] / g.pad[0]) % g.pad[1], hlin[i] / (g.pad[0] * g.pad[1])};
    int64_t lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      // tiles t with t*spacing <= c < t*spacing + tile
      const int64_t sp = std::max<int64_t>(g.spacing[d], 1);
      const int64_t num = c[d] - g.tile[d] + 1;
      lo[d] = num <= 0 ? 0 : (num + sp - 1) / sp;
      hi[d] = std::min<int64_t>(c[d] / sp, g.ntiles[d] - 1);
    }
    const bool isn = std::isnan(hv[i]);
    for (int64_t tz = lo[2]; tz <= hi[2]; ++tz)
      for (int64_t ty = lo[1]; ty <= hi[1]; ++ty)
        for (int64_t tx = lo[0]; tx <= hi[0]; ++tx) {
          const int64_t sx = tx * g.spacing[0], sy = ty * g.spacing[1], sz = tz * g.spacing[2];
          if (c[0] < sx || c[0] >= sx + g.tile[0] || c[1] < sy || c[1] >= sy + g.tile[1] ||
              c[2] < sz || c[2] >= sz + g.tile[2])
            continue;
          const int64_t t = tx + g.ntiles[0] * (ty + g.ntiles[1] * tz);
          if (isn) {
            nan_cnt[t]++;
          } else {
            has_data[t] = 1;
            tile_hard[t].push_back({kpack(c[0] - sx, c[1] - sy, c[2] - sz), (float)hv[i]});
          }
        }
  }
  std::vector<uint8_t> skipped(g.ntot, 0);
  std::vector<int64_t> datainds;
  for (int64_t t = 0; t < g.ntot; ++t) {
    int64_t ti3[3] = {t % g.ntiles[0], (t / g.ntiles[0]) % g.ntiles[1], t / (g.ntiles[0] * g.ntiles[1])};
    bool beyond = false;
    for (int d = 0; d < 3; ++d) beyond = beyond || ti3[d] * g.spacing[d] >= g.sim[d];
    if (beyond || nan_cnt[t] == T) skipped[t] = 1;
    else if (has_data[t]) datainds.push_back(t);
  }
  // hard offsets of a tile in column-major order
  for (auto& v : tile_hard)
    std::sort(v.begin(), v.end(), [](const std::pair<uint32_t, float>& a,
                                     const std::pair<uint32_t, float>& b) {
      const uint32_t ra = (uint32_t)kz_of(a.first) << 20 | (uint32_t)ky_of(a.first) << 10 | (uint32_t)kx_of(a.first);
      const uint32_t rb = (uint32_t)kz_of(b.first) << 20 | (uint32_t)ky_of(b.first) << 10 | (uint32_t)kx_of(b.first);
      return ra < rb;
    });

  // ---- path (src/utils.jl:158-204) ----
  Grid3 text{{g.ntiles[0], g.ntiles[1], g.ntiles[2]}};
  std::vector<int64_t> path = genpath_host(p->seed, text, p->path, datainds);

  // ---- disabled windows (src/utils.jl:115-129) ----
  uint8_t* d_dis = (uint8_t*)iq_scratch(ctx, S_DIS, (size_t)P);
  if (!d_dis) return IQ_ERR_ALLOC;
  RET_IF(iq_launch_disabled(ctx, ctx->d_nanii, ctx->ti, tileD, d_dis));
  int64_t npat = P;
  if (ctx->ti_nan > 0) {
    std::vector<uint8_t> hd(P);
    IQ_CUDA_OK(cudaMemcpyAsync(hd.data(), d_dis, (size_t)P, cudaMemcpyDeviceToHost, st));
    IQ_CUDA_OK(cudaStreamSynchronize(st));
    for (uint8_t v : hd) npat -= v;
  }

  // ---- step plan: neighbour flags per step, distinct masks (src/iqsim.jl:172-205) ----
  struct Step {
    int64_t tile; int64_t start[3]; int64_t startlin; int cfg; bool hardtile;
    int nslab; CutSlab slab[6]; int level; int64_t order;
  };
  std::vector<Step> steps;
  std::vector<MaskCfg> cfgs;
  std::vector<uint8_t> pasted(g.ntot, 0);
  for (int64_t ind : path) {
    if (skipped[ind]) continue;
    Step s;
    s.tile = ind;
    s.order = (int64_t)steps.size();
    int64_t ti3[3] = {ind % g.ntiles[0], (ind / g.ntiles[0]) % g.ntiles[1], ind / (g.ntiles[0] * g.ntiles[1])};
    MaskCfg m;
    s.nslab = 0;
    for (int d = 0; d < 3; ++d) {
      s.start[d] = ti3[d] * g.spacing[d];
      m.prev[d] = m.next[d] = 0;
      if (d < N && g.ovl[d] > 1) {
        int64_t pv[3] = {ti3[0], ti3[1], ti3[2]}, nx[3] = {ti3[0], ti3[1], ti3[2]};
        pv[d] -= 1;
        nx[d] += 1;
        if (pv[d] >= 0 && pasted[pv[0] + g.ntiles[0] * (pv[1] + g.ntiles[1] * pv[2])]) m.prev[d] = 1;
        if (nx[d] < g.ntiles[d] && pasted[nx[0] + g.ntiles[0] * (nx[1] + g.ntiles[1] * nx[2])]) m.next[d] = 1;
      }
      m.lo[d] = m.prev[d] ? g.ovl[d] : 0;
      m.hi[d] = m.next[d] ? g.spacing[d] : g.tile[d];
    }
    s.startlin = s.start[0] + padD.x * (s.start[1] + padD.y * s.start[2]);
    for (int d = 0; d < 3; ++d) {
      for (int side = 0; side < 2; ++side) {
        if (!(side ? m.next[d] : m.prev[d])) continue;
        CutSlab& c = s.slab[s.nslab++];
        c.dim = d;
        c.next = side;
        for (int e = 0; e < 3; ++e) { c.off[e] = 0; c.ext[e] = g.tile[e]; }
        c.off[d] = side ? g.spacing[d] : 0;
        c.ext[d] = side ? g.tile[d] - g.spacing[d] : g.ovl[d];
      }
    }
    int64_t inner = 1;
    for (int d = 0; d < 3; ++d) inner *= std::max<int64_t>(m.hi[d] - m.lo[d], 0);
    m.K = (int)(T - inner);
    int id = -1;
    for (auto& c : cfgs)
      if (!memcmp(c.prev, m.prev, sizeof(m.prev)) && !memcmp(c.next, m.next, sizeof(m.next))) id = c.id;
    if (id < 0) {
      m.id = (int)cfgs.size();
      cfgs.push_back(m);
      id = m.id;
    }
    s.cfg = id;
    s.hardtile = has_data[ind] != 0;
    steps.push_back(s);
    pasted[ind] = 1;
  }
  if (ctx->max_steps >= 0 && (int64_t)steps.size() > ctx->max_steps) steps.resize(ctx->max_steps);
  // Dependency levels: a step must follow every earlier step of the path whose tile region
  // overlaps its own (it reads what they paste and pastes over them). Steps of one level never
  // overlap, so each level runs as one batch with results identical to the path order.
  {
    int64_t rng3[3];
    for (int d = 0; d < 3; ++d)
      rng3[d] = g.spacing[d] > 0 ? (g.tile[d] + g.spacing[d] - 1) / g.spacing[d] - 1 : 0;
    std::vector<int> tile_level(g.ntot, -1);
    for (Step& s : steps) {
      const int64_t t3[3] = {s.tile % g.ntiles[0], (s.tile / g.ntiles[0]) % g.ntiles[1],
                             s.tile / (g.ntiles[0] * g.ntiles[1])};
      int lv = 0;
      for (int64_t oz = -rng3[2]; oz <= rng3[2]; ++oz)
        for (int64_t oy = -rng3[1]; oy <= rng3[1]; ++oy)
          for (int64_t ox = -rng3[0]; ox <= rng3[0]; ++ox) {
            const int64_t x = t3[0] + ox, y = t3[1] + oy, z = t3[2] + oz;
            if (x < 0 || y < 0 || z < 0 || x >= g.ntiles[0] || y >= g.ntiles[1] || z >= g.ntiles[2]) continue;
            const int l = tile_level[x + g.ntiles[0] * (y + g.ntiles[1] * z)];
            if (l >= 0) lv = std::max(lv, l + 1);
          }
      s.level = lv;
      tile_level[s.tile] = lv;
    }
    std::stable_sort(steps.begin(), steps.end(),
                     [](const Step& a, const Step& b) { return a.level < b.level; });
  }
  // offset lists: one block of T entries per mask configuration, plus the full tile
  const int ncfg = (int)cfgs.size();
  std::vector<uint32_t> klist((size_t)(ncfg + 1) * T);
  for (int c = 0; c <= ncfg; ++c) {
    int k = 0;
    for (int64_t z = 0; z < g.tile[2]; ++z)
      for (int64_t y = 0; y < g.tile[1]; ++y)
        for (int64_t x = 0; x < g.tile[0]; ++x) {
          bool in = true;
          if (c < ncfg) {
            const MaskCfg& m = cfgs[c];
            const bool inner = x >= m.lo[0] && x < m.hi[0] && y >= m.lo[1] && y < m.hi[1] &&
                               z >= m.lo[2] && z < m.hi[2];
            in = !inner;
          }
          if (in) klist[(size_t)c * T + k++] = kpack(x, y, z);
        }
  }
  const bool tc = ctx->corr_engine >= 1;
  // ---- exact re-rank: error coefficients of the maps (iq_map_kappa) ----
  // The simulation grid holds TI values, hard data and zeros only. The overlap maps come from
  // the tensor cores (FP16 halves when both ranges allow, else TF32 halves) or the SIMT kernel;
  // the hard maps from the SIMT kernel with A2 summed directly; the soft maps like the overlap
  // maps, from the auxiliary images (their statistics are known after the upload below).
  IqValueStats hard_stats;
  {
    std::vector<float> hvf(nh);
    for (int64_t i = 0; i < nh; ++i) hvf[i] = std::isnan(hv[i]) ? 0.f : (float)hv[i];
    hard_stats = iq_host_stats(hvf.data(), nh);
  }
  IqValueStats sim_stats = ctx->ti_stats;
  sim_stats.merge(hard_stats);
  const int ovl_form = !tc ? 0 : (ctx->corr_engine == 2 && ctx->ti_stats.fp16_range() &&
                                  sim_stats.fp16_range()) ? 1 : 2;
  const int64_t tivol_all = ctx->ti.vol();
  std::vector<double> cfg_kappa(ncfg);
  bool need_ref = nsoft > 0;
  for (int c = 0; c < ncfg; ++c) {
    cfg_kappa[c] = iq_map_kappa(ctx->ti_stats, sim_stats, cfgs[c].K, ovl_form);
    need_ref = need_ref || cfg_kappa[c] > 0.0;
  }
  const double ovl_eabs = iq_map_eabs(ctx->ti_stats, tivol_all);
  // hard lists of data tiles
  std::vector<int64_t> hoff(g.ntot + 1, 0);
  for (int64_t t = 0; t < g.ntot; ++t) hoff[t + 1] = hoff[t] + (int64_t)tile_hard[t].size();
  std::vector<uint32_t> hk(std::max<int64_t>(hoff[g.ntot], 1));
  std::vector<float> hkv(std::max<int64_t>(hoff[g.ntot], 1));
  for (int64_t t = 0; t < g.ntot; ++t)
    for (size_t i = 0; i < tile_hard[t].size(); ++i) {
      hk[hoff[t] + i] = tile_hard[t][i].first;
      hkv[hoff[t] + i] = tile_hard[t][i].second;
    }

  // ---- chunks: consecutive steps of one level, as many as memory allows ----
  const int rt = iq_register_tile(R);
  const int rpad = ((R + rt - 1) / rt) * rt;
  int64_t slabmax = 1;
  for (int d = 0; d < N; ++d) slabmax = std::max<int64_t>(slabmax, T / g.tile[d] * g.ovl[d]);
  int64_t cutscr_per = 0;
  {
    int dev = 0, lim = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    lim -= 1024;  // the cut kernel's static shared memory
    if ((int64_t)iq_cut_scratch_bytes(slabmax) > lim) cutscr_per = (int64_t)iq_cut_scratch_bytes(slabmax);
  }
  for (int64_t t = 0; t < g.ntot && !need_ref; ++t)
    if (!tile_hard[t].empty())
      need_ref = iq_map_kappa(ctx->ti_stats, hard_stats, (int64_t)tile_hard[t].size(), 0) > 0.0;
  const int64_t per_step = (int64_t)R * P * (4 + 4 + 16 + 16 + (need_ref ? 18 : 0)) + P * 4 +
                           T * (rpad + 1) * 4 + (int64_t)R * 6 * (slabmax + cutscr_per) + 4096;
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  // hard-data distance maps depend on the data only: one map per data tile, all held at once
  int64_t nhs = 0;
  for (const Step& s : steps) nhs += s.hardtile ? 1 : 0;
  const int64_t hard_bytes = nhs * (P + T) * 4;
  if ((size_t)hard_bytes > freeb / 2)
    return iq_set_error(IQ_ERR_LIMIT, "hard-data maps of %lld data tiles need %lld bytes",
                        (long long)nhs, (long long)hard_bytes);
  // soft-data maps: one map of P floats per (non-skipped tile, soft variable), all held for the
  // whole call (about 122 GB for a 5.7 M-position map over 5,324 tiles)
  if (nsoft > 0) {
    int64_t nlive = 0;
    for (int64_t t = 0; t < g.ntot; ++t) nlive += skipped[t] ? 0 : 1;
    const double soft_bytes = (double)nlive * nsoft * (double)P * 4.0;
    if (soft_bytes + (double)hard_bytes > (double)freeb * 0.75)
      return iq_set_error(IQ_ERR_LIMIT,
                          "soft-data maps of %lld tiles x %d variables need %.0f bytes, more than "
                          "three quarters of the %zu free bytes of the device",
                          (long long)nlive, nsoft, soft_bytes, freeb);
  }
  int64_t chunk_max = std::max<int64_t>(
      1, std::min<int64_t>(ctx->level_chunk, (int64_t)(freeb / 2 - hard_bytes) / per_step));
  std::vector<int64_t> cbeg;  // chunk boundaries into `steps`
  for (size_t i = 0; i < steps.size();) {
    size_t j = i + 1;
    while (j < steps.size() && steps[j].level == steps[i].level && (int64_t)(j - i) < chunk_max) ++j;
    cbeg.push_back((int64_t)i);
    i = j;
  }
  cbeg.push_back((int64_t)steps.size());
  const int64_t nchunk = (int64_t)cbeg.size() - 1;
  int64_t cmax = 1;
  for (int64_t c = 0; c < nchunk; ++c) cmax = std::max(cmax, cbeg[c + 1] - cbeg[c]);

  // Realization groups: realizations never read one another, so with `sim.streams` = 2 and
  // the tensor-core path two groups run on two streams, interleaved chunk by chunk. One
  // group's pick and cut then share the GPU with the other group's correlation, and the tail
  // of each launch is filled by the other stream's work. Group g holds realizations
  // [gb[g], gb[g+1]).
  const int ngrp = (tc && T > 0 && R >= 2 && ctx->sim_streams >= 2) ? 2 : 1;
  const int gb[3] = {0, ngrp == 2 ? (R + 1) / 2 : R, R};

  // ---- device buffers ----
  const bool debug = p->debug != 0 && (cuts || voxs);
  float* d_sim = (float*)iq_scratch(ctx, S_SIM, sizeof(float) * padvol * R);
  float* d_cut = debug ? (float*)iq_scratch(ctx, S_CUT, sizeof(float) * padvol * R) : nullptr;
  float* d_D = (float*)iq_scratch(ctx, S_D, sizeof(float) * P * R * cmax);
  float* d_Dh = (float*)iq_scratch(ctx, S_DHARD, sizeof(float) * P * std::max<int64_t>(nhs, 1));
  float* d_tv = (float*)iq_scratch(ctx, S_TV, sizeof(float) * T * (std::max(rpad, 16) * cmax + nhs));
  double* d_b2 = (double*)iq_scratch(ctx, S_B2, sizeof(double) * (std::max(rpad, 16) * cmax + nhs));
  uint32_t* d_kl = (uint32_t*)iq_scratch(ctx, S_KLIST, sizeof(uint32_t) * klist.size());
  unsigned* d_mm = (unsigned*)iq_scratch(ctx, S_MINMAX, sizeof(unsigned) * 2 * (R * cmax + nhs));
  uint32_t* d_hk = (uint32_t*)iq_scratch(ctx, S_HARDLIST, sizeof(uint32_t) * hk.size());
  float* d_hkv = (float*)iq_scratch(ctx, S_HARDPTS, sizeof(float) * hkv.size());
  const size_t pk = (size_t)P * R * cmax;
  int32_t* d_cand = (int32_t*)iq_scratch(ctx, S_PICK_CAND, sizeof(int32_t) * pk);
  uint32_t* d_k0 = (uint32_t*)iq_scratch(ctx, S_PICK_K0, sizeof(uint32_t) * pk);
  uint32_t* d_v0 = (uint32_t*)iq_scratch(ctx, S_PICK_V0, sizeof(uint32_t) * pk);
  uint32_t* d_k1 = (uint32_t*)iq_scratch(ctx, S_PICK_K1, sizeof(uint32_t) * pk);
  uint32_t* d_v1 = (uint32_t*)iq_scratch(ctx, S_PICK_V1, sizeof(uint32_t) * pk);
  double* d_w = (double*)iq_scratch(ctx, S_PICK_W, sizeof(double) * pk);
  double* d_prod = (double*)iq_scratch(ctx, S_PICK_PROD, sizeof(double) * pk);
  double* d_rv = need_ref ? (double*)iq_scratch(ctx, S_PICK_RV, sizeof(double) * pk) : nullptr;
  double* d_rr = need_ref ? (double*)iq_scratch(ctx, S_PICK_RR, sizeof(double) * pk) : nullptr;
  uint8_t* d_rl = need_ref ? (uint8_t*)iq_scratch(ctx, S_PICK_RL, 2 * pk) : nullptr;
  int64_t* d_rind = (int64_t*)iq_scratch(ctx, S_RIND, sizeof(int64_t) * R * cmax);
  int64_t* d_ncand = (int64_t*)iq_scratch(ctx, S_NCAND, sizeof(int64_t) * R * cmax);
  uint8_t* d_cutbuf = (uint8_t*)iq_scratch(ctx, S_CUTBUF, (size_t)R * cmax * 6 * slabmax);
  void* d_cutscr = cutscr_per ? iq_scratch(ctx, S_CUTSCR, (size_t)cutscr_per * 6 * R * cmax) : nullptr;
  if (!d_sim || (debug && !d_cut) || !d_D || !d_Dh || !d_tv || !d_b2 || !d_kl || !d_mm || !d_hk ||
      !d_hkv || !d_cand || !d_k0 || !d_v0 || !d_k1 || !d_v1 || !d_w || !d_prod || !d_rind ||
      !d_ncand || !d_cutbuf || (cutscr_per && !d_cutscr) || (need_ref && (!d_rv || !d_rr || !d_rl)))
    return IQ_ERR_ALLOC;
  float* d_tvh = d_tv + (size_t)T * std::max(rpad, 16) * cmax;  // hard templates (T x 1 each)
  // per-step scratch of group g starts at its first realization's share
  auto grp_pick = [&](int g) { return (size_t)gb[g] * cmax * P; };
  auto grp_rind = [&](int g) { return (size_t)gb[g] * cmax; };
  double* d_b2h = d_b2 + (size_t)std::max(rpad, 16) * cmax;
  unsigned* d_mmh = d_mm + 2 * R * cmax;
  IQ_CUDA_OK(cudaMemsetAsync(d_sim, 0, sizeof(float) * padvol * R, st));
  if (debug) IQ_CUDA_OK(cudaMemsetAsync(d_cut, 0, sizeof(float) * padvol * R, st));
  IQ_CUDA_OK(cudaMemcpyAsync(d_kl, klist.data(), sizeof(uint32_t) * klist.size(), cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemcpyAsync(d_hk, hk.data(), sizeof(uint32_t) * hk.size(), cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemcpyAsync(d_hkv, hkv.data(), sizeof(float) * hkv.size(), cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), st));
  IQ_CUDA_OK(cudaMemsetAsync(ctx->d_ties, 0, sizeof(unsigned long long), st));
  iq_lp_begin_call(ctx);
  // ---- tensor-core launches: union stage lists keyed by their set of masks ----
  // Mask configuration c < ncfg is "tile minus [lo, hi)"; c == ncfg is the full tile.
  auto cfg_box = [&](int c) {
    TcBox b{};
    if (c < ncfg)
      for (int d = 0; d < 3; ++d) { b.lo[d] = (int32_t)cfgs[c].lo[d]; b.hi[d] = (int32_t)cfgs[c].hi[d]; }
    return b;
  };
  // stage lists in both forms: TF32 (one row entry per stage) and FP16 (two per stage)
  struct TcStageRef { int64_t off; int nstage; int64_t nsteps; int64_t off16; int nstage16; int64_t nsteps16; };
  std::vector<uint32_t> tc_word, tc_pre, tc_w16;  // tc_w16: per list, w16a then w16b then pre16
  std::map<std::vector<int>, TcStageRef> tc_stage_of;
  auto stages_for = [&](const std::vector<int>& cfgset) -> TcStageRef {
    auto it = tc_stage_of.find(cfgset);
    if (it != tc_stage_of.end()) return it->second;
    std::vector<TcBox> bx;
    for (int c : cfgset) bx.push_back(cfg_box(c));
    TcStages st;
    iq_tc_stages(tileD, bx.data(), (int)bx.size(), st);
    TcStageRef r{(int64_t)tc_word.size(), (int)st.word.size(), st.nsteps,
                 (int64_t)tc_w16.size(), (int)st.w16a.size(), st.nsteps16};
    tc_word.insert(tc_word.end(), st.word.begin(), st.word.end());
    tc_pre.insert(tc_pre.end(), st.prefix.begin(), st.prefix.end());
    tc_w16.insert(tc_w16.end(), st.w16a.begin(), st.w16a.end());
    tc_w16.insert(tc_w16.end(), st.w16b.begin(), st.w16b.end());
    tc_w16.insert(tc_w16.end(), st.pre16.begin(), st.pre16.end());
    tc_stage_of[cfgset] = r;
    return r;
  };
  struct TcRun {
    int64_t chunk; size_t col0; int N; std::vector<int> cfgset; TcStageRef st; double flops;
  };
  std::vector<TcRun> tcruns;
  std::vector<TcCol> tccols;
  std::vector<int64_t> tcbeg(nchunk * ngrp + 1, 0);  // launches of (chunk c, group g): c * ngrp + g
  std::vector<uint8_t> chunk_tc(nchunk, 0);
  // Every chunk runs its overlap distances on the tensor cores: the (tile, realization)
  // columns of the chunk and group, grouped by mask, in launches of at most 256 columns and
  // 8 masks with balanced widths. A tile without pasted neighbours (mask box = the whole tile)
  // gets zero templates and A2 = B2 = 0, i.e. D = 0 like the reference's empty overlap.
  for (int64_t cg = 0; cg < nchunk * ngrp; ++cg) {
    const int64_t c = cg / ngrp;
    const int grp = (int)(cg % ngrp);
    const int Rg = gb[grp + 1] - gb[grp];
    const bool ok = tc && T > 0;
    chunk_tc[c] = ok;
    if (ok) {
      std::vector<std::pair<int, int64_t>> order;  // (cfg, step index in chunk) sorted by cfg
      for (int64_t k = cbeg[c]; k < cbeg[c + 1]; ++k) order.push_back({steps[k].cfg, k - cbeg[c]});
      std::stable_sort(order.begin(), order.end(),
                       [](const std::pair<int, int64_t>& x, const std::pair<int, int64_t>& y) { return x.first < y.first; });
      const int64_t ncols = (int64_t)order.size() * Rg;
      const int64_t nl = (ncols + IQ_TC_MAXN - 1) / IQ_TC_MAXN;
      const int64_t per = std::min<int64_t>(IQ_TC_MAXN, ((ncols + nl - 1) / nl + 15) / 16 * 16);
      int64_t q = 0;
      while (q < ncols) {
        TcRun run;
        run.chunk = c;
        run.col0 = tccols.size();
        int64_t cnt = 0;
        double fl = 0;
        while (q < ncols && cnt < per) {
          const int cf = order[q / Rg].first;
          int bid = -1;
          for (size_t j = 0; j < run.cfgset.size(); ++j) if (run.cfgset[j] == cf) bid = (int)j;
          if (bid < 0) {
            if ((int)run.cfgset.size() == IQ_TC_MAXBOX) break;
            run.cfgset.push_back(cf);
            bid = (int)run.cfgset.size() - 1;
          }
          const int64_t i = order[q / Rg].second, r = gb[grp] + q % Rg;
          tccols.push_back(TcCol{r * padvol + steps[cbeg[c] + i].startlin,
                                 d_D + ((size_t)i * R + r) * P, d_b2 + (size_t)i * rpad + r,
                                 d_mm + (size_t)i * R * 2 + 2 * r, bid, 0});
          fl += 2.0 * (double)P * (double)cfgs[cf].K;
          ++cnt;
          ++q;
        }
        for (; cnt % 16; ++cnt) tccols.push_back(TcCol{-1, nullptr, nullptr, nullptr, 0, 0});
        run.N = (int)cnt;
        run.st = stages_for(run.cfgset);
        run.flops = fl;
        tcruns.push_back(run);
      }
    }
    tcbeg[cg + 1] = (int64_t)tcruns.size();
  }
  const TcStageRef soft_st = (tc && nsoft > 0 && T > 0) ? stages_for(std::vector<int>{ncfg})
                                                         : TcStageRef{0, 0, 0, 0, 0, 0};
  uint32_t* d_tcst = nullptr;  // stage words of every list, then their prefixes
  void* d_tcb = nullptr;        // packed templates of one launch, per group
  size_t tcb_bytes = 0;
  double* d_tcb2 = nullptr;     // squared sums of the soft templates of one launch
  TcCol* d_tccols = nullptr;
  // (a simulation of one tile has columns but no stages: its launches only write D = 0)
  if (tc && (!tc_word.empty() || !tccols.empty())) {
    std::vector<uint32_t> both(tc_word);
    both.insert(both.end(), tc_pre.begin(), tc_pre.end());
    both.insert(both.end(), tc_w16.begin(), tc_w16.end());
    int64_t bmax = 1;
    for (const TcRun& u : tcruns)
      bmax = std::max<int64_t>(bmax, std::max(u.st.nsteps, u.st.nsteps16) * 64 * u.N);
    bmax = std::max<int64_t>(bmax, std::max(soft_st.nsteps, soft_st.nsteps16) * 64 * IQ_TC_MAXN);
    tcb_bytes = (size_t)(bmax + 255) / 256 * 256;  // one packed-template buffer per group
    d_tcst = (uint32_t*)iq_scratch(ctx, S_TCSTAGE, sizeof(uint32_t) * std::max<size_t>(both.size(), 1));
    d_tcb = iq_scratch(ctx, S_TCB, tcb_bytes * ngrp);
    d_tcb2 = (double*)iq_scratch(ctx, S_TCB2, sizeof(double) * IQ_TC_MAXN);
    if (!d_tcst || !d_tcb || !d_tcb2) return IQ_ERR_ALLOC;
    if (!both.empty()) {
      IQ_CUDA_OK(cudaMemcpyAsync(d_tcst, both.data(), sizeof(uint32_t) * both.size(),
                                 cudaMemcpyHostToDevice, st));
      IQ_CUDA_OK(cudaStreamSynchronize(st));  // `both` is a host vector
    }
    if (!tccols.empty()) {
      d_tccols = (TcCol*)iq_scratch(ctx, S_TCCOLS, sizeof(TcCol) * tccols.size());
      if (!d_tccols) return IQ_ERR_ALLOC;
      IQ_CUDA_OK(cudaMemcpyAsync(d_tccols, tccols.data(), sizeof(TcCol) * tccols.size(),
                                 cudaMemcpyHostToDevice, st));
    }
  }
  // one tensor-core launch over the columns cols[0..N) with the masks of `cfgset`
  auto tc_launch = [&](const std::vector<int>& cfgset, const TcStageRef& sr, const float* img,
                       const double* ii, const float* grid, Dim3 gdims, const TcCol* cols, int N,
                       const IqValueStats& img_stats, const IqValueStats& tmpl_stats,
                       double flops, void* B) -> int {
    TcCorrLaunch L;
    L.img = img; L.img_dims = ctx->ti; L.out_dims = distD; L.tile = tileD; L.ii = ii;
    L.nbox = (int)cfgset.size();
    for (int b = 0; b < L.nbox; ++b) L.box[b] = cfg_box(cfgset[b]);
    L.disabled = d_dis;
    L.stage_word = d_tcst + sr.off;
    L.stage_prefix = d_tcst + tc_word.size() + sr.off;
    L.nstage = sr.nstage;
    L.nsteps = sr.nsteps;
    L.stage16 = d_tcst + 2 * tc_word.size() + sr.off16;
    L.nstage16 = sr.nstage16;
    L.nsteps16 = sr.nsteps16;
    L.grid = grid; L.grid_dims = gdims; L.cols = cols; L.N = N; L.B = B;
    L.img_stats = img_stats; L.tmpl_stats = tmpl_stats; L.flops = flops;
    return iq_launch_corr_tc(ctx, L);
  };

  // ---- soft data: padded aux grids, auxTI integral images, per-tile distance maps ----
  std::vector<float*> d_aux(nsoft), d_auxti(nsoft);
  std::vector<double*> d_auxii(nsoft);
  std::vector<Dim3> aux_dims(nsoft);
  std::vector<double> soft_kappa(nsoft, 0.0), soft_eabs(nsoft, 0.0);
  double* d_softb2 = nullptr;  // sum of squared soft template values, per (variable, tile slot)
  float* d_soft = nullptr;
  unsigned* d_softmm = nullptr;  // [min, max finite] bits of each soft map
  std::vector<int64_t> slot_of(g.ntot, -1);
  int64_t nslot = 0;
  if (nsoft > 0) {
    for (int64_t t = 0; t < g.ntot; ++t)
      if (!skipped[t]) slot_of[t] = nslot++;
    const int64_t tivol = ctx->ti.vol();
    int64_t amax[3] = {1, 1, 1};
    for (int s = 0; s < nsoft; ++s)
      for (int d = 0; d < N; ++d) amax[d] = std::max(amax[d], std::max(soft[s].auxsize[d], g.pad[d]));
    const int64_t auxvol = amax[0] * amax[1] * amax[2];
    const int64_t iivol = (ctx->ti.x + 1) * (ctx->ti.y + 1) * (ctx->ti.z + 1);
    float* a_aux = (float*)iq_scratch(ctx, S_AUX, sizeof(float) * auxvol * nsoft);
    float* a_ti = (float*)iq_scratch(ctx, S_AUXTI, sizeof(float) * tivol * nsoft);
    double* a_ii = (double*)iq_scratch(ctx, S_AUXII, sizeof(double) * iivol * nsoft);
    float* a_raw = (float*)iq_scratch(ctx, S_TMP1, sizeof(float) * auxvol);
    d_soft = (float*)iq_scratch(ctx, S_SOFT, sizeof(float) * P * nslot * nsoft);
    d_softmm = (unsigned*)iq_scratch(ctx, S_SOFTMM, sizeof(unsigned) * 2 * nslot * nsoft);
    int64_t* d_starts = (int64_t*)iq_scratch(ctx, S_STARTS, sizeof(int64_t) * (nslot + 16));
    d_softb2 = (double*)iq_scratch(ctx, S_SOFTB2, sizeof(double) * (nslot * nsoft + 16));
    if (!a_aux || !a_ti || !a_ii || !a_raw || !d_soft || !d_softmm || !d_starts || !d_softb2)
      return IQ_ERR_ALLOC;
    std::vector<int64_t> tl;
    for (int64_t t = 0; t < g.ntot; ++t)
      if (!skipped[t]) tl.push_back(t);
    for (int s = 0; s < nsoft; ++s) {
      int64_t ae[3] = {1, 1, 1};
      for (int d = 0; d < N; ++d) ae[d] = soft[s].auxsize[d];
      const Dim3 asz{ae[0], ae[1], ae[2]};
      const Dim3 psz{std::max(ae[0], g.pad[0]), std::max(ae[1], g.pad[1]), std::max(ae[2], g.pad[2])};
      aux_dims[s] = psz;
      d_aux[s] = a_aux + auxvol * s;
      d_auxti[s] = a_ti + tivol * s;
      d_auxii[s] = a_ii + iivol * s;
      IQ_CUDA_OK(cudaMemcpyAsync(a_raw, soft[s].aux, sizeof(float) * asz.vol(), cudaMemcpyDefault, st));
      RET_IF(iq_launch_pad_symmetric(ctx, a_raw, asz, d_aux[s], psz));
      RET_IF(iq_launch_prepare(ctx, d_aux[s], psz.vol(), nullptr));  // NaN -> 0 (prepare(aux))
      IQ_CUDA_OK(cudaMemcpyAsync(d_auxti[s], soft[s].auxti, sizeof(float) * tivol, cudaMemcpyDefault, st));
      RET_IF(iq_launch_prepare(ctx, d_auxti[s], tivol, nullptr));
      RET_IF(iq_build_integrals(ctx, d_auxti[s], ctx->ti, d_auxii[s], nullptr, nullptr));
      std::vector<int64_t> starts(tl.size());
      for (size_t i = 0; i < tl.size(); ++i) {
        const int64_t t = tl[i];
        const int64_t sx = (t % g.ntiles[0]) * g.spacing[0];
        const int64_t sy = ((t / g.ntiles[0]) % g.ntiles[1]) * g.spacing[1];
        const int64_t sz = (t / (g.ntiles[0] * g.ntiles[1])) * g.spacing[2];
        starts[i] = sx + psz.x * (sy + psz.y * sz);
      }
      IQ_CUDA_OK(cudaMemcpyAsync(d_starts, starts.data(), sizeof(int64_t) * starts.size(),
                                 cudaMemcpyHostToDevice, st));
      IqValueStats aux_stats, auxti_stats;
      RET_IF(iq_value_stats(ctx, d_aux[s], psz.vol(), aux_stats));
      RET_IF(iq_value_stats(ctx, d_auxti[s], tivol, auxti_stats));
      {
        const int form = !(tc && T > 0) ? 0 : (ctx->corr_engine == 2 && auxti_stats.fp16_range() &&
                                                aux_stats.fp16_range()) ? 1 : 2;
        soft_kappa[s] = iq_map_kappa(auxti_stats, aux_stats, T, form);
        soft_eabs[s] = iq_map_eabs(auxti_stats, tivol);
      }
      if (tc && T > 0) {
        // per-tile soft distance maps on the tensor cores, up to 256 tiles per launch
        std::vector<TcCol> cols;
        std::vector<std::pair<size_t, int>> launches;  // (first column, N)
        for (size_t b0 = 0; b0 < tl.size(); b0 += IQ_TC_MAXN) {
          const int nb = (int)std::min<size_t>(IQ_TC_MAXN, tl.size() - b0);
          launches.push_back({cols.size(), (nb + 15) / 16 * 16});
          for (int i = 0; i < launches.back().second; ++i) {
            if (i < nb) {
              const int64_t slot = (int64_t)s * nslot + slot_of[tl[b0 + i]];
              cols.push_back(TcCol{starts[b0 + i], d_soft + slot * P, d_softb2 + slot,
                                   d_softmm + 2 * slot, 0, 0});
            } else {
              cols.push_back(TcCol{-1, nullptr, nullptr, nullptr, 0, 0});
            }
          }
        }
        TcCol* d_cols = (TcCol*)iq_scratch(ctx, S_TCSOFT, sizeof(TcCol) * cols.size());
        if (!d_cols) return IQ_ERR_ALLOC;
        IQ_CUDA_OK(cudaMemcpyAsync(d_cols, cols.data(), sizeof(TcCol) * cols.size(),
                                   cudaMemcpyHostToDevice, st));
        for (size_t l = 0; l < launches.size(); ++l) {
          const size_t b0 = l * IQ_TC_MAXN;
          const int nb = (int)std::min<size_t>(IQ_TC_MAXN, tl.size() - b0);
          const int64_t slot0 = (int64_t)s * nslot + slot_of[tl[b0]];
          GatherLaunch G;
          G.grid = d_aux[s]; G.grid_dims = psz; G.grid_stride = 0; G.starts = d_starts + b0;
          G.ntmpl = nb; G.rpad = nb;
          G.t0 = GatherTask{d_kl + (size_t)ncfg * T, (int)T, 0, nullptr, nullptr,
                            d_softb2 + slot0, d_softmm + 2 * slot0};
          RET_IF(iq_launch_gather(ctx, G));
          RET_IF(tc_launch(std::vector<int>{ncfg}, soft_st, d_auxti[s], d_auxii[s], d_aux[s], psz,
                           d_cols + launches[l].first, launches[l].second, auxti_stats, aux_stats,
                           2.0 * (double)P * (double)T * nb, d_tcb));
        }
        IQ_CUDA_OK(cudaStreamSynchronize(st));  // `cols` is a host vector
      } else {
        // per-tile soft distance maps, 16 tiles per launch
        for (size_t b0 = 0; b0 < tl.size(); b0 += 16) {
          const int nb = (int)std::min<size_t>(16, tl.size() - b0);
          const int64_t slot0 = (int64_t)s * nslot + slot_of[tl[b0]];
          GatherLaunch G;
          G.grid = d_aux[s]; G.grid_dims = psz; G.grid_stride = 0; G.starts = d_starts + b0;
          G.ntmpl = nb; G.rpad = 16;
          G.t0 = GatherTask{d_kl + (size_t)ncfg * T, (int)T, 0, nullptr, d_tv, d_softb2 + slot0,
                            d_softmm + 2 * slot0};
          RET_IF(iq_launch_gather(ctx, G));
          CorrLaunch C;
          C.img = d_auxti[s]; C.img_dims = ctx->ti; C.out_dims = distD; C.tile = tileD;
          C.rpad = 16; C.ntmpl = nb; C.out_stride = P; C.disabled = d_dis;
          C.t0 = CorrTask{d_kl + (size_t)ncfg * T, (int)T, d_tv, d_softb2 + slot0, d_auxii[s],
                          {0, 0, 0}, {0, 0, 0},
                          d_soft + slot0 * P, d_softmm + 2 * slot0};
          RET_IF(iq_launch_corr(ctx, C));
        }
      }
      IQ_CUDA_OK(cudaStreamSynchronize(st));  // `starts` is a host vector
    }
  }

  // ---- relaxation sizes; selection keys of the soft maps (shared by all realizations) for
  // the first steps of the softdbsize sequence, computed once instead of per realization ----
  int64_t dbn = 0, dbz = 0;
  int nsn = 0, nsz = 0;
  int64_t seqn[IQ_MAX_SEQ], seqz[IQ_MAX_SEQ];
  if (npat > 0) iq_relax_sizes(npat, p->tol, dbn, dbz, nsn, seqn, nsz, seqz);
  const int nkeys = std::min(nsn, IQ_PRE_KEYS);
  unsigned long long* d_softkeys = nullptr;
  PreBand* d_pb = nullptr;      // refined selections of the soft maps (maps with an error bound)
  int32_t* d_pbpool = nullptr;
  const int64_t pb_cap = 8192;  // listed band positions per selection
  if (nsoft > 0 && npat > 0 && nkeys > 0 && nslot > 0) {
    d_softkeys = (unsigned long long*)iq_scratch(ctx, S_SOFTKEYS,
                                                 sizeof(unsigned long long) * nslot * nsoft * nkeys);
    if (!d_softkeys) return IQ_ERR_ALLOC;
    RET_IF(iq_launch_select_keys(ctx, d_soft, d_softmm, nslot * nsoft, P, seqn, nkeys, d_softkeys));
    bool any_ref = false;
    for (int sv = 0; sv < nsoft; ++sv) any_ref = any_ref || soft_kappa[sv] > 0.0;
    if (any_ref) {
      // the re-evaluation of every soft map: the auxiliary TI against the padded auxiliary grid
      // at the tile, over the full tile
      std::vector<ExactSrc> xs((size_t)nslot * nsoft);
      for (int64_t t = 0; t < g.ntot; ++t) {
        if (slot_of[t] < 0) continue;
        const int64_t st3[3] = {(t % g.ntiles[0]) * g.spacing[0],
                                ((t / g.ntiles[0]) % g.ntiles[1]) * g.spacing[1],
                                (t / (g.ntiles[0] * g.ntiles[1])) * g.spacing[2]};
        for (int sv = 0; sv < nsoft; ++sv) {
          const int64_t slot = (int64_t)sv * nslot + slot_of[t];
          ExactSrc& x = xs[slot];
          if (!(soft_kappa[sv] > 0.0)) continue;
          const Dim3 ad = aux_dims[sv];
          x.img = d_auxti[sv]; x.isx = ctx->ti.x; x.isxy = ctx->ti.x * ctx->ti.y;
          x.klist = d_kl + (size_t)ncfg * T; x.K = (int)T;
          x.tmpl = d_aux[sv] + st3[0] + ad.x * (st3[1] + ad.y * st3[2]);
          x.tgx = ad.x; x.tgxy = ad.x * ad.y; x.tmpl_rs = 0;
          x.b2 = d_softb2 + slot; x.b2_rs = 0;
          x.kappa = soft_kappa[sv]; x.eabs = soft_eabs[sv];
        }
      }
      ExactSrc* d_xs = (ExactSrc*)iq_scratch(ctx, S_PB_SRC, sizeof(ExactSrc) * xs.size());
      d_pb = (PreBand*)iq_scratch(ctx, S_PB_OUT, sizeof(PreBand) * nslot * nsoft * nkeys);
      d_pbpool = (int32_t*)iq_scratch(ctx, S_PB_POOL, sizeof(int32_t) * nslot * nsoft * nkeys * pb_cap);
      if (!d_xs || !d_pb || !d_pbpool) return IQ_ERR_ALLOC;
      IQ_CUDA_OK(cudaMemcpyAsync(d_xs, xs.data(), sizeof(ExactSrc) * xs.size(),
                                 cudaMemcpyHostToDevice, st));
      RET_IF(iq_launch_select_bands(ctx, d_soft, d_softmm, d_xs, nslot * nsoft, P, distD.x,
                                    distD.x * distD.y, seqn, nkeys, d_pb, d_pbpool, pb_cap));
      IQ_CUDA_OK(cudaStreamSynchronize(st));  // `xs` is a host vector
    }
  }

  // ---- dbsize selections of the hard-data maps (one per data tile, shared by its
  // realizations), computed once after the maps below ----
  std::vector<ExactSrc> hard_x;   // re-evaluation of each hard map (kappa 0: exact)
  PreBand* d_pbh = nullptr;
  int32_t* d_pbhpool = nullptr;
  if (nhs > 0 && npat > 0) {
    d_pbh = (PreBand*)iq_scratch(ctx, S_PBH_OUT, sizeof(PreBand) * nhs);
    d_pbhpool = (int32_t*)iq_scratch(ctx, S_PBH_POOL, sizeof(int32_t) * nhs * pb_cap);
    if (!d_pbh || !d_pbhpool) return IQ_ERR_ALLOC;
    hard_x.resize(nhs);
  }
  // ---- task descriptors of every step, uploaded once ----
  // Gather and pick tasks point at per-realization slots: each group has its own copy, whose
  // pointers start at the group's first realization. Cut and paste tasks are shared.
  const int64_t nsteps = (int64_t)steps.size();
  std::vector<GatherTask> gt(nsteps * ngrp), hgt;
  std::vector<CorrTask> ct(nsteps), hct;
  std::vector<PickTask> pt(nsteps * ngrp);
  std::vector<StepTask> stk(nsteps);
  std::vector<double> cflops(nchunk, 0.0);
  std::vector<int> cslab(nchunk, 0), chard(nchunk, 0);
  int64_t hi = 0;  // slot of the next data tile's hard-data map
  for (int64_t c = 0; c < nchunk; ++c) {
    for (int64_t k = cbeg[c]; k < cbeg[c + 1]; ++k) {
      const Step& s = steps[k];
      const int64_t i = k - cbeg[c];
      const MaskCfg& m = cfgs[s.cfg];
      float* tv = d_tv + (size_t)i * T * rpad;
      double* b2 = d_b2 + (size_t)i * rpad;
      unsigned* mm = d_mm + (size_t)i * R * 2;
      float* D = d_D + (size_t)i * R * P;
      ct[k] = CorrTask{d_kl + (size_t)s.cfg * T, m.K, tv, b2, ctx->d_ti2ii,
                       {m.lo[0], m.lo[1], m.lo[2]}, {m.hi[0], m.hi[1], m.hi[2]}, D, mm};
      cflops[c] += 2.0 * (double)P * (double)m.K * (double)R;
      const float* Dh = nullptr;
      const unsigned* mmh = nullptr;
      if (s.hardtile) {
        const int64_t h0 = hoff[s.tile], hn = hoff[s.tile + 1] - hoff[s.tile];
        float* tvh = d_tvh + (size_t)hi * T;
        hgt.push_back(GatherTask{d_hk + h0, (int)hn, 0, d_hkv + h0, tvh, d_b2h + hi, d_mmh + 2 * hi});
        hct.push_back(CorrTask{d_hk + h0, (int)hn, tvh, d_b2h + hi, nullptr, {0, 0, 0}, {0, 0, 0},
                               d_Dh + (size_t)hi * P, d_mmh + 2 * hi});
        cflops[c] += 2.0 * (double)P * (double)hn;
        Dh = d_Dh + (size_t)hi * P;
        mmh = d_mmh + 2 * hi;
        ++hi;
        chard[c] = 1;
      }
      for (int grp = 0; grp < ngrp; ++grp) {
        const int64_t r0 = gb[grp];
        gt[grp * nsteps + k] = GatherTask{d_kl + (size_t)s.cfg * T, m.K, s.startlin, nullptr,
                                          chunk_tc[c] ? nullptr : tv, b2 + r0, mm + 2 * r0};
        PickTask& q = pt[grp * nsteps + k];
        memset(&q, 0, sizeof(q));
        q.tile = s.tile;
        // direct re-evaluation of the overlap map of realization r: the TI against the group's
        // simulation grid at the tile, over the mask's offsets
        ExactSrc xo{};
        if (cfg_kappa[s.cfg] > 0.0) {
          xo.img = ctx->d_ti; xo.isx = ctx->ti.x; xo.isxy = ctx->ti.x * ctx->ti.y;
          xo.klist = d_kl + (size_t)s.cfg * T; xo.K = m.K;
          xo.tmpl = d_sim + (size_t)r0 * padvol + s.startlin; xo.tgx = padD.x;
          xo.tgxy = padD.x * padD.y; xo.tmpl_rs = padvol;
          xo.b2 = b2 + r0; xo.b2_rs = 1;
          xo.kappa = cfg_kappa[s.cfg]; xo.eabs = ovl_eabs;
        }
        int na = 0;
        if (s.hardtile) {
          q.D0 = Dh; q.D0_rs = 0; q.mm0 = mmh; q.mm0_rs = 0;
          const int64_t h0 = hoff[s.tile], hn = hoff[s.tile + 1] - hoff[s.tile];
          const double hk_kappa = iq_map_kappa(ctx->ti_stats, hard_stats, hn, 0);
          if (d_pbh) {
            q.x0_pb = d_pbh + (hi - 1);
            q.x0_pool = d_pbhpool;
          }
          if (hk_kappa > 0.0) {
            ExactSrc& xh = q.x0;
            xh.img = ctx->d_ti; xh.isx = ctx->ti.x; xh.isxy = ctx->ti.x * ctx->ti.y;
            xh.klist = d_hk + h0; xh.K = (int)hn; xh.kval = d_hkv + h0;
            xh.b2 = Dh == nullptr ? nullptr : d_b2h + (hi - 1); xh.b2_rs = 0;
            xh.kappa = hk_kappa; xh.eabs = 0.0;
            if (!hard_x.empty()) hard_x[hi - 1] = xh;
          }
          q.aux[na] = D + r0 * P; q.aux_rs[na] = P; q.aux_mm[na] = mm + 2 * r0; q.aux_mm_rs[na] = 2;
          q.xa[na] = xo;
          ++na;
        } else {
          q.D0 = D + r0 * P; q.D0_rs = P; q.mm0 = mm + 2 * r0; q.mm0_rs = 2;
          q.x0 = xo;
        }
        for (int sv = 0; sv < nsoft; ++sv) {
          const int64_t slot = (int64_t)sv * nslot + slot_of[s.tile];
          q.aux[na] = d_soft + slot * P; q.aux_rs[na] = 0;
          q.aux_mm[na] = d_softmm + 2 * slot; q.aux_mm_rs[na] = 0;
          if (soft_kappa[sv] > 0.0) {
            if (d_pb) {  // refined selections shared by all realizations
              q.aux_pb[na] = d_pb + slot * nkeys;
              q.pb_pool = d_pbpool;
              q.nkeys = nkeys;
            }
            // the auxiliary TI against the padded auxiliary grid at the tile, full tile
            ExactSrc& xs = q.xa[na];
            xs.img = d_auxti[sv]; xs.isx = ctx->ti.x; xs.isxy = ctx->ti.x * ctx->ti.y;
            xs.klist = d_kl + (size_t)ncfg * T; xs.K = (int)T;
            const Dim3 ad = aux_dims[sv];
            xs.tmpl = d_aux[sv] + s.start[0] + ad.x * (s.start[1] + ad.y * s.start[2]);
            xs.tgx = ad.x; xs.tgxy = ad.x * ad.y; xs.tmpl_rs = 0;
            xs.b2 = d_softb2 + slot; xs.b2_rs = 0;
            xs.kappa = soft_kappa[sv]; xs.eabs = soft_eabs[sv];
          } else if (d_softkeys) {  // exact map: its keys are shared by all realizations
            q.aux_keys[na] = d_softkeys + slot * nkeys;
            q.nkeys = nkeys;
          }
          ++na;
        }
        q.naux = na;
      }
      StepTask& sk = stk[k];
      sk.start = s.startlin;
      sk.nslab = s.nslab;
      for (int j = 0; j < 6; ++j) sk.slab[j] = s.slab[j];
      cslab[c] = std::max(cslab[c], s.nslab);
    }
  }
  const size_t tbytes = sizeof(GatherTask) * (gt.size() + hgt.size()) + sizeof(CorrTask) * (nsteps + hct.size()) +
                        sizeof(PickTask) * pt.size() + sizeof(StepTask) * nsteps + 6 * 256;
  char* d_tasks = (char*)iq_scratch(ctx, S_TASKS, tbytes);
  if (!d_tasks) return IQ_ERR_ALLOC;
  size_t toff = 0;
  auto put = [&](const void* src, size_t bytes) -> char* {
    char* dst = d_tasks + toff;
    if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    toff += (bytes + 255) & ~(size_t)255;
    return dst;
  };
  const GatherTask* d_gt = (const GatherTask*)put(gt.data(), sizeof(GatherTask) * gt.size());
  const CorrTask* d_ct = (const CorrTask*)put(ct.data(), sizeof(CorrTask) * nsteps);
  const GatherTask* d_hgt = (const GatherTask*)put(hgt.data(), sizeof(GatherTask) * hgt.size());
  const CorrTask* d_hct = (const CorrTask*)put(hct.data(), sizeof(CorrTask) * hct.size());
  const PickTask* d_pt = (const PickTask*)put(pt.data(), sizeof(PickTask) * pt.size());
  const StepTask* d_st = (const StepTask*)put(stk.data(), sizeof(StepTask) * nsteps);
  IQ_CUDA_OK(cudaGetLastError());

  // ---- hard-data distance of every data tile: data values against the TI ----
  for (int64_t h = 0; h < (int64_t)hgt.size(); h += 32768) {
    const int nb = (int)std::min<int64_t>(32768, (int64_t)hgt.size() - h);
    GatherLaunch H;
    H.ntmpl = 1; H.rpad = 1; H.ntask = nb; H.tasks = d_hgt + h;
    RET_IF(iq_launch_gather(ctx, H));
    CorrLaunch Ch;
    Ch.img = ctx->d_ti; Ch.img_dims = ctx->ti; Ch.out_dims = distD; Ch.tile = tileD;
    Ch.rpad = 1; Ch.ntmpl = 1; Ch.out_stride = P; Ch.disabled = d_dis;
    Ch.ntask = nb; Ch.tasks = d_hct + h; Ch.flops = 1;
    RET_IF(iq_launch_corr(ctx, Ch));
  }
  if (d_pbh) {
    ExactSrc* d_hx = (ExactSrc*)iq_scratch(ctx, S_PBH_SRC, sizeof(ExactSrc) * nhs);
    if (!d_hx) return IQ_ERR_ALLOC;
    IQ_CUDA_OK(cudaMemcpyAsync(d_hx, hard_x.data(), sizeof(ExactSrc) * nhs, cudaMemcpyHostToDevice, st));
    const int64_t seq1[1] = {dbn};
    RET_IF(iq_launch_select_bands(ctx, d_Dh, d_mmh, d_hx, nhs, P, distD.x, distD.x * distD.y, seq1,
                                  1, d_pbh, d_pbhpool, pb_cap, 1));
    IQ_CUDA_OK(cudaStreamSynchronize(st));  // `hard_x` is a host vector
  }

  // ---- the tile loop (src/iqsim.jl:172-285), one dependency level chunk at a time ----
  // the learned proposal: applies to integer-valued data without hard or soft data
  int64_t maxK = 0;
  for (const MaskCfg& mc : cfgs) maxK = std::max<int64_t>(maxK, mc.K);
  const bool lp_on = iq_lp_applies(ctx, tileD, maxK, nh > 0 || nsoft > 0);
  const bool lp_cap = ctx->lp_capture > 0 && ctx->lp != nullptr;
  std::vector<int32_t> lc_lohi(6 * std::max(ncfg, 1)), lc_cfgK(std::max(ncfg, 1));
  for (int cf = 0; cf < ncfg; ++cf) {
    for (int d = 0; d < 3; ++d) {
      lc_lohi[6 * cf + d] = (int32_t)cfgs[cf].lo[d];
      lc_lohi[6 * cf + 3 + d] = (int32_t)cfgs[cf].hi[d];
    }
    lc_cfgK[cf] = cfgs[cf].K;
  }
  std::vector<int> lc_cfg, lc_rloc, lc_slot;
  std::vector<int64_t> lc_tile, lc_start, lc_real;
  cudaStream_t gstream[2] = {st, st};
  if (ngrp == 2) {
    if (!ctx->stream2) IQ_CUDA_OK(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
    if (!ctx->ev_fork) IQ_CUDA_OK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    if (!ctx->ev_join) IQ_CUDA_OK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    gstream[1] = ctx->stream2;
    IQ_CUDA_OK(cudaEventRecord(ctx->ev_fork, st));  // the second group follows the set-up
    IQ_CUDA_OK(cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0));
  }
  {
    // Launchers use the context stream, which is switched per group. On every way out of this
    // block it is restored and made to wait for the second group's stream.
    struct GroupJoin {
      iq_ctx* ctx;
      cudaStream_t main;
      bool on;
      ~GroupJoin() {
        ctx->stream = main;
        if (on && cudaEventRecord(ctx->ev_join, ctx->stream2) == cudaSuccess)
          cudaStreamWaitEvent(main, ctx->ev_join, 0);
      }
    } join{ctx, st, ngrp == 2};
    for (int64_t c = 0; c < nchunk; ++c)
      for (int grp = 0; grp < ngrp; ++grp) {
        ctx->stream = gstream[grp];
        const int64_t k0 = cbeg[c];
        const int m = (int)(cbeg[c + 1] - cbeg[c]);
        const int r0 = gb[grp], Rg = gb[grp + 1] - gb[grp];
        float* sim = d_sim + (size_t)r0 * padvol;
        int64_t* rind = d_rind + grp_rind(grp);
        uint8_t* cutbuf = d_cutbuf + grp_rind(grp) * 6 * slabmax;
        // The learned proposal: picks from shortlists instead of the full scan, where it applies.
        // Columns of the chunk in pick-CTA order: step i of the chunk, realization r of the group.
        const int ncol = m * Rg;
        if (lp_on || lp_cap) {
          lc_cfg.resize(ncol); lc_tile.resize(ncol); lc_start.resize(ncol); lc_real.resize(ncol);
          lc_rloc.resize(ncol); lc_slot.resize(ncol);
          for (int i = 0; i < m; ++i)
            for (int r = 0; r < Rg; ++r) {
              const Step& s = steps[k0 + i];
              const int col = i * Rg + r;
              lc_cfg[col] = s.cfg; lc_tile[col] = s.tile; lc_start[col] = s.startlin;
              lc_real[col] = p->real0 + r0 + r; lc_rloc[col] = r; lc_slot[col] = col;
            }
        }
        LpChunk lc{};
        lc.ncol = ncol; lc.cfg = lc_cfg.data(); lc.lohi = lc_lohi.data(); lc.d_klist = d_kl;
        lc.cfgK = lc_cfgK.data(); lc.T = T; lc.tile = lc_tile.data(); lc.start = lc_start.data();
        lc.real = lc_real.data(); lc.rloc = lc_rloc.data(); lc.slot = lc_slot.data();
        lc.sim = sim; lc.sim_rstride = padvol; lc.sim_dims = padD; lc.tile_dims = tileD;
        lc.dist = distD; lc.tol = p->tol; lc.seed = p->seed; lc.d_rind = rind;
        int lp_done = 0;
        if (lp_on) RET_IF(iq_lp_run_chunk(ctx, lc, c, &lp_done));
        if (!lp_done) {
        iq_lp_count_full(ctx, ncol);
        // overlap distance of every realization of the group for every tile of the chunk
        GatherLaunch G;
        G.grid = sim; G.grid_dims = padD; G.grid_stride = padvol; G.ntmpl = Rg;
        G.rpad = ngrp == 1 ? rpad : Rg;
        G.ntask = m; G.tasks = d_gt + grp * nsteps + k0;
        RET_IF(iq_launch_gather(ctx, G));
        if (chunk_tc[c]) {
          for (int64_t l = tcbeg[c * ngrp + grp]; l < tcbeg[c * ngrp + grp + 1]; ++l) {
            const TcRun& u = tcruns[l];
            RET_IF(tc_launch(u.cfgset, u.st, ctx->d_ti, ctx->d_ti2ii, d_sim, padD, d_tccols + u.col0,
                             u.N, ctx->ti_stats, sim_stats, u.flops, (char*)d_tcb + grp * tcb_bytes));
          }
        } else {  // one group
          CorrLaunch C;
          C.img = ctx->d_ti; C.img_dims = ctx->ti; C.out_dims = distD; C.tile = tileD;
          C.rpad = rpad; C.ntmpl = R; C.out_stride = P; C.disabled = d_dis;
          C.ntask = m; C.tasks = d_ct + k0; C.flops = cflops[c];
          RET_IF(iq_launch_corr(ctx, C));
        }
        // pick
        PickLaunch L;
        L.P = P; L.npat = npat; L.tol = p->tol; L.seed = p->seed; L.real0 = p->real0 + r0; L.nreal = Rg;
        L.ntask = m; L.tasks = d_pt + grp * nsteps + k0; L.naux_max = nsoft + chard[c];
        L.dbsize_norm = dbn; L.dbsize_zero = dbz; L.nseq_norm = nsn; L.nseq_zero = nsz;
        for (int q = 0; q < IQ_MAX_SEQ; ++q) { L.seq_norm[q] = q < nsn ? seqn[q] : 0; L.seq_zero[q] = q < nsz ? seqz[q] : 0; }
        const size_t po = grp_pick(grp);
        L.cand = d_cand + po; L.k0 = d_k0 + po; L.v0 = d_v0 + po; L.k1 = d_k1 + po; L.v1 = d_v1 + po;
        L.w = d_w + po; L.prod = d_prod + po;
        L.rv = d_rv ? d_rv + po : nullptr; L.rr = d_rr ? d_rr + po : nullptr;
        L.rl = d_rl ? d_rl + 2 * po : nullptr;
        L.dx = distD.x; L.dxy = distD.x * distD.y;
        L.ties = ctx->d_ties;
        L.rind = rind; L.ncand = d_ncand + grp_rind(grp); L.status = ctx->d_status;
        L.stats = ctx->prof ? ctx->d_stats : nullptr;
        RET_IF(iq_launch_pick(ctx, L));
        if (lp_cap) RET_IF(iq_lp_capture(ctx, lc, L.cand, L.ncand, P));
        }  // full scan
        // boundary cuts
        if (cslab[c] > 0) {
          CutLaunch K;
          K.nreal = Rg; K.ntask = m; K.nslab_max = cslab[c]; K.tasks = d_st + k0;
          K.sim = sim; K.sim_dims = padD; K.sim_rstride = padvol;
          K.ti = ctx->d_ti; K.ti_dims = ctx->ti; K.dist_dims = distD; K.rind = rind;
          K.out = cutbuf; K.slabmax = slabmax;
          K.scratch = d_cutscr ? (char*)d_cutscr + grp_rind(grp) * 6 * cutscr_per : nullptr;
          K.scratch_per_cta = cutscr_per;
          K.status = ctx->d_status;
          K.stats = ctx->prof ? ctx->d_stats : nullptr;
          K.gr_period = ctx->cut_gr_period;
          K.threads = ctx->cut_threads;
          RET_IF(iq_launch_cut(ctx, K));
        }
        // paste
        PasteLaunch Pl;
        Pl.nreal = Rg; Pl.ntask = m; Pl.tasks = d_st + k0;
        Pl.sim = sim; Pl.sim_dims = padD; Pl.sim_rstride = padvol;
        Pl.cut = d_cut ? d_cut + (size_t)r0 * padvol : nullptr;
        Pl.tile = tileD; Pl.ti = ctx->d_ti; Pl.ti_dims = ctx->ti; Pl.dist_dims = distD;
        Pl.rind = rind; Pl.cutbuf = cutbuf; Pl.slabmax = slabmax;
        RET_IF(iq_launch_paste(ctx, Pl));
      }
  }

  // ---- voxel reuse, hard overwrite, crop (src/iqsim.jl:287-307) ----
  double* d_vox = nullptr;
  if (debug && voxs) {
    d_vox = (double*)iq_scratch(ctx, S_VOX, sizeof(double) * R);
    if (!d_vox) return IQ_ERR_ALLOC;
    RET_IF(iq_launch_voxsum(ctx, R, d_cut, padvol, padvol, d_vox));
  }
  if (nh > 0) {
    std::vector<float> hvf(nh);
    for (int64_t i = 0; i < nh; ++i) hvf[i] = (float)hv[i];
    int64_t* d_hl = (int64_t*)iq_scratch(ctx, S_TMP0, sizeof(int64_t) * nh);
    float* d_hv = (float*)iq_scratch(ctx, S_TMP2, sizeof(float) * nh);
    if (!d_hl || !d_hv) return IQ_ERR_ALLOC;
    IQ_CUDA_OK(cudaMemcpyAsync(d_hl, hlin.data(), sizeof(int64_t) * nh, cudaMemcpyHostToDevice, st));
    IQ_CUDA_OK(cudaMemcpyAsync(d_hv, hvf.data(), sizeof(float) * nh, cudaMemcpyHostToDevice, st));
    RET_IF(iq_launch_hard_overwrite(ctx, R, d_sim, d_cut, padD, padvol, nh, d_hl, d_hv));
    IQ_CUDA_OK(cudaStreamSynchronize(st));  // host vectors above go out of scope
  }
  float* d_out = (float*)iq_scratch(ctx, S_OUT, sizeof(float) * simvol * R);
  if (!d_out) return IQ_ERR_ALLOC;
  RET_IF(iq_launch_crop(ctx, R, d_sim, padD, padvol, simD, d_out));
  IQ_CUDA_OK(cudaMemcpyAsync(reals, d_out, sizeof(float) * simvol * R, cudaMemcpyDefault, st));
  if (debug && cuts) {
    IQ_CUDA_OK(cudaStreamSynchronize(st));
    RET_IF(iq_launch_crop(ctx, R, d_cut, padD, padvol, simD, d_out));
    IQ_CUDA_OK(cudaMemcpyAsync(cuts, d_out, sizeof(float) * simvol * R, cudaMemcpyDefault, st));
  }
  std::vector<double> hvox(R, 0.0);
  if (d_vox) IQ_CUDA_OK(cudaMemcpyAsync(hvox.data(), d_vox, sizeof(double) * R, cudaMemcpyDeviceToHost, st));
  int status = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  IQ_CUDA_OK(cudaStreamSynchronize(st));
  if (d_vox)
    for (int r = 0; r < R; ++r) {
      double v = hvox[r] / (double)g.ovlvol;
      IQ_CUDA_OK(cudaMemcpy(voxs + r, &v, sizeof(double), cudaMemcpyDefault));
    }
  if (status == IQ_ERR_NOPATTERN) return iq_set_error(status, "every training-image pattern is disabled");
  if (status == IQ_ERR_CUTCAP) return iq_set_error(status, "graph cut hit its round limit");
  if (status) return iq_set_error(status, "kernel status %d", status);
  return IQ_OK;
}
