// Host side of the learned proposal (no counterpart in the reference): the encoder's parameters
// and Adam state, the cached window embeddings of the resident training image (one set per mask
// configuration), training pairs captured from full-scan simulations, the training loop, and the
// per-chunk path of iq_simulate -- template embeddings, shortlists, the shortlist pick, the
// recall monitor with its shortlist doubling, and the fall-back to the full scan.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "iq_internal.h"

namespace {

constexpr int NPOS = 8;  // positives kept per captured pair (candidates of its pick)
constexpr double kMonMinTrue = 1000;  // sampled candidates before the recall decides a fallback

struct LpCache {
  int32_t lohi[6];
  __nv_bfloat16* W = nullptr;  // [P][64]
  float* nW = nullptr;         // [P]
  __nv_bfloat16* Ws = nullptr; // sampled rows [IQ_LP_SAMPLES][64]
  float* nWs = nullptr;        // [IQ_LP_SAMPLES]
};

}  // namespace

struct IqLp {
  Dim3 tile{0, 0, 0};
  LpGeo g{};
  float* w = nullptr;     // FP32 parameters
  float* m = nullptr;     // Adam moments
  float* v = nullptr;
  float* grad = nullptr;
  double* loss = nullptr;
  int adam_step = 0;
  int64_t wversion = 0;   // bumped whenever the parameters change
  // training image side
  double* ii1 = nullptr;  // Float64 integral image of the values
  size_t ii1_bytes = 0;
  int64_t ii1_ti = -1;
  uint8_t* ti8 = nullptr;  // the image as bytes (the exact sums of the shortlist pick)
  size_t ti8_bytes = 0;
  int64_t ti8_ti = -1;
  bool ti8_ok = false;
  unsigned long long* ti2 = nullptr;  // plane form (codes 0..3)
  size_t ti2_words = 0;
  int64_t ti2_ntx = 0, ti2_nty = 0;
  bool ti2_ok = false;
  int* d_bad = nullptr;
  std::vector<LpCache> cache;
  int64_t cache_ti = -1, cache_w = -1;
  // captured pairs: features of the template, its mask box, NPOS candidate positions
  float* cap_feat = nullptr;
  int32_t* cap_box = nullptr;
  int32_t* cap_pos = nullptr;
  int64_t cap_n = 0, cap_max = 0;
  Dim3 cap_dist{0, 0, 0};
  // statistics of the current call
  int64_t cols_lp = 0, cols_full = 0, mon_cols = 0, short_total = 0;
  double mon_true = 0, mon_hit = 0;
  int64_t k_cur = 0;                  // shortlist length of the current phase of the call
  double ph_true = 0, ph_hit = 0;     // sampled candidates since k_cur was set
  bool off = false;       // sampled recall fell below 0.99: full scan for the rest of the call
  unsigned long long* d_counters = nullptr;
  unsigned* d_dmin = nullptr;
};

namespace {

void free_cache(IqLp* lp) {
  for (auto& c : lp->cache) {
    cudaFree(c.W);
    cudaFree(c.nW);
    cudaFree(c.Ws);
    cudaFree(c.nWs);
  }
  lp->cache.clear();
}

IqLp* lp_of(iq_ctx* ctx) {
  if (!ctx->lp) ctx->lp = new IqLp();
  return ctx->lp;
}

// Standard normal from the Philox stream (seed; i, 0, 3): Box-Muller on two 32-bit halves.
double philox_normal(uint64_t seed, uint32_t i) {
  const uint64_t r = iq_rand64(seed, i, 0u, 3u);
  const double u1 = ((double)(uint32_t)r + 1.0) / 4294967297.0;
  const double u2 = (double)(uint32_t)(r >> 32) / 4294967296.0;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

int alloc_params(IqLp* lp, Dim3 tile) {
  const LpGeo g = iq_lp_geo(tile);
  if (lp->w && lp->g.npar == g.npar) {
    lp->tile = tile;
    lp->g = g;
    return IQ_OK;
  }
  cudaFree(lp->w); cudaFree(lp->m); cudaFree(lp->v); cudaFree(lp->grad);
  lp->w = lp->m = lp->v = lp->grad = nullptr;
  const size_t b = sizeof(float) * g.npar;
  if (cudaMalloc(&lp->w, b) != cudaSuccess || cudaMalloc(&lp->m, b) != cudaSuccess ||
      cudaMalloc(&lp->v, b) != cudaSuccess || cudaMalloc(&lp->grad, b) != cudaSuccess ||
      (!lp->loss && cudaMalloc(&lp->loss, sizeof(double)) != cudaSuccess)) {
    cudaGetLastError();
    return iq_set_error(IQ_ERR_ALLOC, "proposal parameters: allocation failed");
  }
  lp->tile = tile;
  lp->g = g;
  return IQ_OK;
}

int reset_adam(iq_ctx* ctx, IqLp* lp) {
  IQ_CUDA_OK(cudaMemsetAsync(lp->m, 0, sizeof(float) * lp->g.npar, ctx->stream));
  IQ_CUDA_OK(cudaMemsetAsync(lp->v, 0, sizeof(float) * lp->g.npar, ctx->stream));
  lp->adam_step = 0;
  lp->wversion += 1;
  return IQ_OK;
}

Dim3 tile_of(int32_t ndim, const int64_t* t) {
  Dim3 d{1, 1, 1};
  if (ndim >= 1) d.x = t[0];
  if (ndim >= 2) d.y = t[1];
  if (ndim >= 3) d.z = t[2];
  return d;
}

int ensure_ii1(iq_ctx* ctx, IqLp* lp) {
  if (lp->ii1 && lp->ii1_ti == ctx->ti_version) return IQ_OK;
  const size_t bytes = sizeof(double) * (ctx->ti.x + 1) * (ctx->ti.y + 1) * (ctx->ti.z + 1);
  if (lp->ii1_bytes < bytes) {
    cudaFree(lp->ii1);
    lp->ii1 = nullptr;
    if (cudaMalloc(&lp->ii1, bytes) != cudaSuccess) {
      cudaGetLastError();
      return iq_set_error(IQ_ERR_ALLOC, "proposal: integral image allocation failed");
    }
    lp->ii1_bytes = bytes;
  }
  int rc = iq_build_value_integral(ctx, ctx->d_ti, ctx->ti, lp->ii1);
  if (rc) return rc;
  lp->ii1_ti = ctx->ti_version;
  return IQ_OK;
}

// The image as bytes, when every value is an integer in [0, 255] (categorical codes).
int ensure_ti8(iq_ctx* ctx, IqLp* lp) {
  if (lp->ti8_ti == ctx->ti_version) return IQ_OK;
  const int64_t n = ctx->ti.vol();
  const size_t bytes = (size_t)n + 16;
  if (lp->ti8_bytes < bytes || !lp->d_bad) {
    cudaFree(lp->ti8);
    lp->ti8 = nullptr;
    lp->ti8_bytes = 0;
    if (cudaMalloc(&lp->ti8, bytes) != cudaSuccess ||
        (!lp->d_bad && cudaMalloc(&lp->d_bad, sizeof(int)) != cudaSuccess)) {
      cudaGetLastError();
      return iq_set_error(IQ_ERR_ALLOC, "proposal: byte image allocation failed");
    }
    lp->ti8_bytes = bytes;
  }
  int rc = iq_lp_to_u8(ctx, ctx->d_ti, n, lp->ti8, lp->d_bad);
  if (rc) return rc;
  int bad = 1;
  IQ_CUDA_OK(cudaMemcpyAsync(&bad, lp->d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  lp->ti8_ok = bad == 0;
  // plane form when the codes are 0..3
  lp->ti2_ok = false;
  if (lp->ti8_ok) {
    const int64_t ntx = (ctx->ti.x + 31) / 32 + 1, nty = (ctx->ti.y + 15) / 16;
    const size_t words = (size_t)(ctx->ti.z * nty * ntx * 16);
    if (lp->ti2_words < words) {
      cudaFree(lp->ti2);
      lp->ti2 = nullptr;
      lp->ti2_words = 0;
      if (cudaMalloc(&lp->ti2, sizeof(unsigned long long) * words) != cudaSuccess) {
        cudaGetLastError();
        return iq_set_error(IQ_ERR_ALLOC, "proposal: plane image allocation failed");
      }
      lp->ti2_words = words;
    }
    rc = iq_lp_to_planes(ctx, ctx->d_ti, ctx->ti, ntx, nty, lp->ti2, lp->d_bad);
    if (rc) return rc;
    IQ_CUDA_OK(cudaMemcpyAsync(&bad, lp->d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    lp->ti2_ok = bad == 0 && words < ((size_t)1 << 31);
    lp->ti2_ntx = ntx;
    lp->ti2_nty = nty;
  }
  lp->ti8_ti = ctx->ti_version;
  return IQ_OK;
}

// The form the exact sums read: planes for codes 0..3 and tiles of x extent <= 32, else bytes.
LpImg lp_image(iq_ctx* ctx, IqLp* lp, Dim3 tile) {
  LpImg im{};
  im.b8 = lp->ti8;
  im.isx = ctx->ti.x;
  im.isxy = ctx->ti.x * ctx->ti.y;
  if (lp->ti2_ok && tile.x <= 32) {
    im.b2 = lp->ti2;
    im.ntx = lp->ti2_ntx;
    im.nty = lp->ti2_nty;
  }
  return im;
}

// Quads of the mask "tile minus box [lo, hi)": rows in (z, y, x) order, four x offsets from a
// multiple of 4, image strides (isx, isxy), template strides (tgx, tgxy).
void make_quads(Dim3 tile, const int32_t* lohi, int64_t isx, int64_t isxy, int64_t tgx,
                int64_t tgxy, std::vector<LpQuad>& out) {
  for (int64_t z = 0; z < tile.z; ++z)
    for (int64_t y = 0; y < tile.y; ++y)
      for (int64_t x4 = 0; x4 < tile.x; x4 += 4) {
        uint32_t m = 0;
        for (int b = 0; b < 4; ++b) {
          const int64_t x = x4 + b;
          if (x >= tile.x) break;
          const bool inner = x >= lohi[0] && x < lohi[3] && y >= lohi[1] && y < lohi[4] &&
                             z >= lohi[2] && z < lohi[5];
          if (!inner) m |= 0xFFu << (8 * b);
        }
        if (!m) continue;
        LpQuad q;
        q.off = (int32_t)(x4 + isx * y + isxy * z);
        q.tx = (int32_t)(x4 + tgx * y + tgxy * z);
        q.mask = m;
        q.pad_ = 0;
        out.push_back(q);
      }
}

Dim3 dist_of(iq_ctx* ctx, Dim3 tile) {
  return Dim3{ctx->ti.x - tile.x + 1, ctx->ti.y - tile.y + 1, ctx->ti.z - tile.z + 1};
}

// Window embeddings of every position under the mask box lohi (cached per training image and
// parameters).
int window_embeddings(iq_ctx* ctx, IqLp* lp, const int32_t* lohi, const LpCache** out) {
  if (lp->cache_ti != ctx->ti_version || lp->cache_w != lp->wversion) {
    free_cache(lp);
    lp->cache_ti = ctx->ti_version;
    lp->cache_w = lp->wversion;
  }
  for (const LpCache& c : lp->cache)
    if (!memcmp(c.lohi, lohi, sizeof(c.lohi))) { *out = &c; return IQ_OK; }
  int rc = ensure_ii1(ctx, lp);
  if (rc) return rc;
  const Dim3 dist = dist_of(ctx, lp->tile);
  const int64_t P = dist.vol();
  LpCache c;
  memcpy(c.lohi, lohi, sizeof(c.lohi));
  if (cudaMalloc(&c.W, sizeof(__nv_bfloat16) * P * IQ_LP_EMB) != cudaSuccess ||
      cudaMalloc(&c.nW, sizeof(float) * P) != cudaSuccess ||
      cudaMalloc(&c.Ws, sizeof(__nv_bfloat16) * IQ_LP_SAMPLES * IQ_LP_EMB) != cudaSuccess ||
      cudaMalloc(&c.nWs, sizeof(float) * IQ_LP_SAMPLES) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(c.W);
    cudaFree(c.nW);
    cudaFree(c.Ws);
    return iq_set_error(IQ_ERR_ALLOC, "proposal: window embeddings of %lld positions", (long long)P);
  }
  rc = iq_lp_encode_windows(ctx, lp->g, lp->w, lp->ii1, ctx->d_ti2ii, ctx->ti, dist, lohi,
                            lohi + 3, c.W, c.nW);
  if (!rc) rc = iq_lp_sample_rows(ctx, c.W, c.nW, P, c.Ws, c.nWs);
  if (rc) {
    cudaFree(c.W); cudaFree(c.nW); cudaFree(c.Ws); cudaFree(c.nWs);
    return rc;
  }
  lp->cache.push_back(c);
  *out = &lp->cache.back();
  return IQ_OK;
}

}  // namespace

void iq_lp_free(iq_ctx* ctx) {
  IqLp* lp = ctx->lp;
  if (!lp) return;
  free_cache(lp);
  cudaFree(lp->ti8); cudaFree(lp->ti2); cudaFree(lp->d_bad);
  cudaFree(lp->w); cudaFree(lp->m); cudaFree(lp->v); cudaFree(lp->grad); cudaFree(lp->loss);
  cudaFree(lp->ii1);
  cudaFree(lp->cap_feat); cudaFree(lp->cap_box); cudaFree(lp->cap_pos);
  cudaFree(lp->d_counters); cudaFree(lp->d_dmin);
  delete lp;
  ctx->lp = nullptr;
}

void iq_lp_begin_call(iq_ctx* ctx) {
  if (!ctx->lp) return;
  IqLp* lp = ctx->lp;
  lp->cols_lp = lp->cols_full = lp->mon_cols = lp->short_total = 0;
  lp->mon_true = lp->mon_hit = 0;
  lp->ph_true = lp->ph_hit = 0;
  lp->k_cur = ctx->lp_k;
  lp->off = false;
}

bool iq_lp_applies(iq_ctx* ctx, Dim3 tile, int64_t maxK, bool data) {
  IqLp* lp = ctx->lp;
  if (!ctx->lp_enable || !lp || !lp->w || data || ctx->ti_nan > 0) return false;
  if (lp->tile.x != tile.x || lp->tile.y != tile.y || lp->tile.z != tile.z) return false;
  // FP32 direct sums are exact: integer values whose squared sums stay below 2^24
  const IqValueStats& s = ctx->ti_stats;
  if (!s.narrow || s.lsbexp < 0) return false;
  const double m = (double)maxK * (double)s.amax * (double)s.amax * 4.0;
  if (!(m < 16777216.0)) return false;
  // byte-valued image (categorical codes): the exact sums read it as bytes
  if (ensure_ti8(ctx, lp) || !lp->ti8_ok) return false;
  return 16 * (maxK / 4 + 2 * tile.y * tile.z) <= 200 * 1024;
}

// ---------------------------------------------------------------------------------------------
// One chunk through the proposal
// ---------------------------------------------------------------------------------------------
int iq_lp_run_chunk(iq_ctx* ctx, const LpChunk& c, int64_t chunk_index, int* done) {
  *done = 0;
  IqLp* lp = ctx->lp;
  if (!lp || lp->off || c.ncol <= 0) return IQ_OK;
  for (int i = 0; i < c.ncol; ++i)
    if (c.cfgK[c.cfg[i]] <= 0) return IQ_OK;  // an empty mask: every position is a candidate
  cudaStream_t st = ctx->stream;
  const int N = c.ncol;
  const int64_t P = c.dist.vol();
  const int64_t kk = lp->k_cur > 0 ? lp->k_cur : ctx->lp_k;
  const int cap = (int)std::min<int64_t>(std::max<int64_t>(16384, 4 * kk), P);
  // columns in the order of their mask configuration
  std::vector<int> ord(N);
  for (int i = 0; i < N; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return c.cfg[x] < c.cfg[y]; });
  std::vector<int64_t> tsrc(N);
  std::vector<int32_t> tbox(6 * (size_t)N);
  std::vector<LpColumn> cols(N);
  // quad tables of the configurations present, one after another
  std::vector<LpQuad> quads;
  std::map<int, std::pair<size_t, int>> qcfg;  // configuration -> (first quad, count)
  for (int i = 0; i < N; ++i) {
    const int cf = c.cfg[i];
    if (qcfg.count(cf)) continue;
    const size_t q0 = quads.size();
    make_quads(c.tile_dims, c.lohi + 6 * cf, ctx->ti.x, ctx->ti.x * ctx->ti.y, c.sim_dims.x,
               c.sim_dims.x * c.sim_dims.y, quads);
    qcfg[cf] = {q0, (int)(quads.size() - q0)};
  }
  LpQuad* dquad = (LpQuad*)iq_scratch(ctx, S_LP_QUAD, sizeof(LpQuad) * std::max<size_t>(1, quads.size()));
  if (!dquad) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(dquad, quads.data(), sizeof(LpQuad) * quads.size(),
                             cudaMemcpyHostToDevice, st));
  int maxQ = 0;
  for (int q = 0; q < N; ++q) {
    const int i = ord[q];
    const int cf = c.cfg[i];
    tsrc[q] = (int64_t)c.rloc[i] * c.sim_rstride + c.start[i];
    for (int d = 0; d < 6; ++d) tbox[6 * q + d] = c.lohi[6 * cf + d];
    LpColumn& col = cols[q];
    col.klist = c.d_klist + (size_t)cf * c.T;
    col.K = c.cfgK[cf];
    col.quad = dquad + qcfg[cf].first;
    col.nq = qcfg[cf].second;
    for (int d = 0; d < 6; ++d) col.lohi[d] = c.lohi[6 * cf + d];
    col.tdim[0] = (int32_t)c.tile_dims.x;
    col.tdim[1] = (int32_t)c.tile_dims.y;
    col.tdim[2] = (int32_t)c.tile_dims.z;
    maxQ = std::max<int>(maxQ, (int)std::max<int64_t>(col.nq, c.tile_dims.y * c.tile_dims.z));
    col.tmpl = c.sim + tsrc[q];
    col.tgx = c.sim_dims.x;
    col.tgxy = c.sim_dims.x * c.sim_dims.y;
    col.tile = c.tile[i];
    col.real = c.real[i];
  }
  __nv_bfloat16* dT = (__nv_bfloat16*)iq_scratch(ctx, S_LP_T, sizeof(__nv_bfloat16) * N * IQ_LP_EMB);
  float* dnT = (float*)iq_scratch(ctx, S_LP_NT, sizeof(float) * N);
  float* dtau = (float*)iq_scratch(ctx, S_LP_TAU, sizeof(float) * N);
  float* ddense = (float*)iq_scratch(ctx, S_LP_DENSE, sizeof(float) * (size_t)N * IQ_LP_SAMPLES);
  int32_t* dlist = (int32_t*)iq_scratch(ctx, S_LP_LIST, sizeof(int32_t) * (size_t)N * cap);
  int32_t* dcnt = (int32_t*)iq_scratch(ctx, S_LP_CNT, sizeof(int32_t) * N);
  float* ddl = (float*)iq_scratch(ctx, S_LP_DL, sizeof(float) * (size_t)N * cap);
  LpColumn* dcols = (LpColumn*)iq_scratch(ctx, S_LP_COLS, sizeof(LpColumn) * N);
  int64_t* dtsrc = (int64_t*)iq_scratch(ctx, S_LP_TSRC, sizeof(int64_t) * N);
  int* dtbox = (int*)iq_scratch(ctx, S_LP_TBOX, sizeof(int32_t) * 6 * N);
  int64_t* drind = (int64_t*)iq_scratch(ctx, S_LP_RIND, sizeof(int64_t) * N);
  int64_t* dncand = (int64_t*)iq_scratch(ctx, S_LP_NCAND, sizeof(int64_t) * N);
  if (!dT || !dnT || !dtau || !ddense || !dlist || !dcnt || !ddl || !dcols || !dtsrc || !dtbox || !drind || !dncand)
    return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(dtsrc, tsrc.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemcpyAsync(dtbox, tbox.data(), sizeof(int32_t) * 6 * N, cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemcpyAsync(dcols, cols.data(), sizeof(LpColumn) * N, cudaMemcpyHostToDevice, st));
  int rc = iq_lp_encode_templates(ctx, lp->g, lp->w, c.sim, c.sim_dims, dtsrc, dtbox, N, dT, dnT);
  if (rc) return rc;
  // shortlists, one scan per mask configuration
  for (int q0 = 0; q0 < N;) {
    int q1 = q0 + 1;
    while (q1 < N && c.cfg[ord[q1]] == c.cfg[ord[q0]]) ++q1;
    const LpCache* wc = nullptr;
    rc = window_embeddings(ctx, lp, c.lohi + 6 * c.cfg[ord[q0]], &wc);
    if (rc) return rc;
    rc = iq_lp_shortlist(ctx, wc->W, wc->nW, P, wc->Ws, wc->nWs, dT + (size_t)q0 * IQ_LP_EMB,
                         dnT + q0, q1 - q0, kk, dtau + q0, ddense, dlist + (size_t)q0 * cap,
                         dcnt + q0, cap);
    if (rc) return rc;
    q0 = q1;
  }
  const LpImg im = lp_image(ctx, lp, c.tile_dims);
  rc = iq_lp_pick(ctx, im, c.dist, dcols, N, dlist, dcnt, cap, ddl, c.tol, c.seed,
                  drind, dncand, maxQ);
  if (rc) return rc;
  // recall of the first column against the full exact scan, every lp_monitor-th chunk
  const bool mon = ctx->lp_monitor > 0 && chunk_index % ctx->lp_monitor == 0;
  if (mon) {
    float* dD = (float*)iq_scratch(ctx, S_LP_D, sizeof(float) * P);
    uint32_t* dbits = (uint32_t*)iq_scratch(ctx, S_LP_BITS, sizeof(uint32_t) * ((P + 31) / 32));
    if (!dD || !dbits) return IQ_ERR_ALLOC;
    if (!lp->d_counters) {
      if (cudaMalloc(&lp->d_counters, 2 * sizeof(unsigned long long)) != cudaSuccess ||
          cudaMalloc(&lp->d_dmin, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return iq_set_error(IQ_ERR_ALLOC, "proposal: counters");
      }
    }
    IQ_CUDA_OK(cudaMemsetAsync(lp->d_counters, 0, 2 * sizeof(unsigned long long), st));
    rc = iq_lp_recall(ctx, im, c.dist, cols[0], dlist, dcnt, cap, c.tol, dD,
                      lp->d_dmin, dbits, lp->d_counters);
    if (rc) return rc;
  }
  std::vector<int64_t> hr(N), hn(N);
  std::vector<int32_t> hc(N);
  unsigned long long hcnt[2] = {0, 0};
  IQ_CUDA_OK(cudaMemcpyAsync(hr.data(), drind, sizeof(int64_t) * N, cudaMemcpyDeviceToHost, st));
  IQ_CUDA_OK(cudaMemcpyAsync(hc.data(), dcnt, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, st));
  if (mon)
    IQ_CUDA_OK(cudaMemcpyAsync(hcnt, lp->d_counters, sizeof(hcnt), cudaMemcpyDeviceToHost, st));
  IQ_CUDA_OK(cudaStreamSynchronize(st));
  if (mon) {
    lp->mon_cols += 1;
    lp->mon_true += (double)hcnt[0];
    lp->mon_hit += (double)hcnt[1];
    lp->ph_true += (double)hcnt[0];
    lp->ph_hit += (double)hcnt[1];
    // the sampled recall of the current shortlist length decides once it rests on enough
    // candidates (a standard error of about 0.003 at recall 0.99): below 0.99 the length
    // doubles (up to lp.kmax) and is judged afresh; at lp.kmax the call takes the full scan
    if (ctx->lp_fallback && lp->ph_true >= kMonMinTrue && lp->ph_hit < 0.99 * lp->ph_true) {
      if (2 * lp->k_cur <= ctx->lp_kmax) {
        lp->k_cur *= 2;
        lp->ph_true = lp->ph_hit = 0;
      } else {
        lp->off = true;
      }
    }
  }
  for (int q = 0; q < N; ++q)
    if (hr[q] < 0) return IQ_OK;  // a shortlist overflowed: the full scan takes this chunk
  // drawn positions into the chunk's rind slots
  int maxslot = 0;
  for (int i = 0; i < N; ++i) maxslot = std::max(maxslot, c.slot[i]);
  std::vector<int64_t> out((size_t)maxslot + 1, -1);
  for (int q = 0; q < N; ++q) out[c.slot[ord[q]]] = hr[q];
  IQ_CUDA_OK(cudaMemcpyAsync(c.d_rind, out.data(), sizeof(int64_t) * out.size(),
                             cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaStreamSynchronize(st));  // `out` is a host vector
  for (int q = 0; q < N; ++q) lp->short_total += std::min<int64_t>(hc[q], cap);
  lp->cols_lp += N;
  *done = 1;
  return IQ_OK;
}

// ---------------------------------------------------------------------------------------------
// Capture of training pairs from the full scan
// ---------------------------------------------------------------------------------------------
namespace {

__global__ void capture_pos_kernel(const int32_t* cand, const int64_t* ncand, const int* cta,
                                   int n, int64_t P, uint64_t seed, int64_t row0,
                                   int32_t* pos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * NPOS) return;
  const int col = i / NPOS, k = i % NPOS;
  const int64_t b = cta[col];
  const int64_t nc = ncand[b];
  int32_t p = -1;
  if (nc > 0) {
    const uint64_t r = iq_rand64(seed, (uint32_t)(row0 + col), (uint32_t)k, 4u);
    p = cand[b * P + (int64_t)(r % (uint64_t)nc)];
  }
  pos[(row0 + col) * NPOS + k] = p;
}

}  // namespace

int iq_lp_capture(iq_ctx* ctx, const LpChunk& c, const int32_t* d_cand, const int64_t* d_ncand,
                  int64_t P) {
  IqLp* lp = ctx->lp;
  if (!lp || !lp->w || lp->cap_n >= lp->cap_max) return IQ_OK;
  if (lp->tile.x != c.tile_dims.x || lp->tile.y != c.tile_dims.y || lp->tile.z != c.tile_dims.z)
    return IQ_OK;
  cudaStream_t st = ctx->stream;
  std::vector<int64_t> tsrc;
  std::vector<int32_t> tbox;
  std::vector<int> cta;
  for (int i = 0; i < c.ncol && lp->cap_n + (int64_t)tsrc.size() < lp->cap_max; ++i) {
    const int cf = c.cfg[i];
    if (c.cfgK[cf] <= 0) continue;
    tsrc.push_back((int64_t)c.rloc[i] * c.sim_rstride + c.start[i]);
    for (int d = 0; d < 6; ++d) tbox.push_back(c.lohi[6 * cf + d]);
    cta.push_back(c.slot[i]);
  }
  const int n = (int)tsrc.size();
  if (n == 0) return IQ_OK;
  int64_t* dtsrc = (int64_t*)iq_scratch(ctx, S_LP_TSRC, sizeof(int64_t) * n);
  int* dtbox = (int*)iq_scratch(ctx, S_LP_TBOX, sizeof(int32_t) * 6 * n);
  int* dcta = (int*)iq_scratch(ctx, S_LP_CNT, sizeof(int) * n);
  if (!dtsrc || !dtbox || !dcta) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(dtsrc, tsrc.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemcpyAsync(dtbox, tbox.data(), sizeof(int32_t) * 6 * n, cudaMemcpyHostToDevice, st));
  IQ_CUDA_OK(cudaMemcpyAsync(dcta, cta.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
  const int64_t row0 = lp->cap_n;
  int rc = iq_lp_template_features(ctx, lp->g, c.sim, c.sim_dims, dtsrc, dtbox, n,
                                   lp->cap_feat + row0 * 3 * lp->g.ng);
  if (rc) return rc;
  IQ_CUDA_OK(cudaMemcpyAsync(lp->cap_box + row0 * 6, dtbox, sizeof(int32_t) * 6 * n,
                             cudaMemcpyDeviceToDevice, st));
  capture_pos_kernel<<<(n * NPOS + 255) / 256, 256, 0, st>>>(d_cand, d_ncand, dcta, n, P,
                                                              c.seed ^ 0x5bd1e995ull, row0,
                                                              lp->cap_pos);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  IQ_CUDA_OK(cudaStreamSynchronize(st));  // host vectors above
  lp->cap_n += n;
  lp->cap_dist = c.dist;
  return IQ_OK;
}

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" int iq_lp_init(iq_ctx* ctx, int32_t ndim, const int64_t* tilesize, uint64_t seed) {
  if (!ctx || !tilesize || ndim < 1 || ndim > 3) return iq_set_error(IQ_ERR_ARG, "invalid argument");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  IqLp* lp = lp_of(ctx);
  int rc = alloc_params(lp, tile_of(ndim, tilesize));
  if (rc) return rc;
  // He initialization from the Philox stream, biases zero
  std::vector<float> h(lp->g.npar, 0.f);
  const LpGeo& g = lp->g;
  auto fill = [&](int off, int n, int fan_in) {
    const double s = std::sqrt(2.0 / fan_in);
    for (int i = 0; i < n; ++i) h[off + i] = (float)(s * philox_normal(seed, (uint32_t)(off + i)));
  };
  fill(LP_OFF_W1, IQ_LP_CH * 3, 3);
  fill(LP_OFF_W2, IQ_LP_CH * IQ_LP_CH * 27, IQ_LP_CH * 27);
  fill(LP_OFF_W3, IQ_LP_CH * IQ_LP_CH * 27, IQ_LP_CH * 27);
  fill(LP_OFF_W4, IQ_LP_EMB * g.nf, g.nf);
  IQ_CUDA_OK(cudaMemcpy(lp->w, h.data(), sizeof(float) * g.npar, cudaMemcpyHostToDevice));
  return reset_adam(ctx, lp);
}

extern "C" int iq_lp_params(iq_ctx* ctx, float* out, int64_t cap, int64_t* n) {
  if (!ctx || !n) return iq_set_error(IQ_ERR_ARG, "invalid argument");
  IqLp* lp = ctx->lp;
  if (!lp || !lp->w) return iq_set_error(IQ_ERR_STATE, "no proposal parameters (iq_lp_init)");
  *n = lp->g.npar;
  if (out && cap >= lp->g.npar) {
    IQ_CUDA_OK(cudaSetDevice(ctx->device));
    IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    IQ_CUDA_OK(cudaMemcpy(out, lp->w, sizeof(float) * lp->g.npar, cudaMemcpyDefault));
  }
  return IQ_OK;
}

extern "C" int iq_lp_set_params(iq_ctx* ctx, int32_t ndim, const int64_t* tilesize,
                                const float* in, int64_t n) {
  if (!ctx || !tilesize || !in || ndim < 1 || ndim > 3) return iq_set_error(IQ_ERR_ARG, "invalid argument");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  const LpGeo g = iq_lp_geo(tile_of(ndim, tilesize));
  if (n != g.npar)
    return iq_set_error(IQ_ERR_ARG, "the encoder of this tile has %d parameters, got %lld", g.npar,
                        (long long)n);
  IqLp* lp = lp_of(ctx);
  int rc = alloc_params(lp, tile_of(ndim, tilesize));
  if (rc) return rc;
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  IQ_CUDA_OK(cudaMemcpy(lp->w, in, sizeof(float) * g.npar, cudaMemcpyDefault));
  return reset_adam(ctx, lp);
}

// Window embeddings of the resident training image at `positions` under the mask "tile minus
// box" (box = lo[3], hi[3]): out is n x 64 floats (the BF16 values of the inference path).
extern "C" int iq_lp_embed(iq_ctx* ctx, int64_t n, const int64_t* positions, const int32_t* box,
                           float* out) {
  if (!ctx || n <= 0 || !positions || !box || !out) return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (!ctx->has_ti) return iq_set_error(IQ_ERR_STATE, "no training image set");
  IqLp* lp = ctx->lp;
  if (!lp || !lp->w) return iq_set_error(IQ_ERR_STATE, "no proposal parameters (iq_lp_init)");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  int rc = ensure_ii1(ctx, lp);
  if (rc) return rc;
  const Dim3 dist = dist_of(ctx, lp->tile);
  int64_t* dpos = (int64_t*)iq_scratch(ctx, S_LP_TSRC, sizeof(int64_t) * n);
  __nv_bfloat16* dW = (__nv_bfloat16*)iq_scratch(ctx, S_LP_T, sizeof(__nv_bfloat16) * n * IQ_LP_EMB);
  float* dn = (float*)iq_scratch(ctx, S_LP_NT, sizeof(float) * n);
  if (!dpos || !dW || !dn) return IQ_ERR_ALLOC;
  for (int64_t i = 0; i < n; ++i)
    if (positions[i] < 0 || positions[i] >= dist.vol()) return iq_set_error(IQ_ERR_ARG, "position out of range");
  IQ_CUDA_OK(cudaMemcpyAsync(dpos, positions, sizeof(int64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
  rc = iq_lp_encode_windows(ctx, lp->g, lp->w, lp->ii1, ctx->d_ti2ii, ctx->ti, dist, box, box + 3,
                            dW, dn, dpos, n);
  if (rc) return rc;
  std::vector<__nv_bfloat16> h((size_t)n * IQ_LP_EMB);
  IQ_CUDA_OK(cudaMemcpyAsync(h.data(), dW, sizeof(__nv_bfloat16) * h.size(), cudaMemcpyDeviceToHost,
                             ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < h.size(); ++i) out[i] = __bfloat162float(h[i]);
  return IQ_OK;
}

namespace {

// One training step's buffers and launch: anchor features rows feat_rows (from `feats`), window
// items at positions; items: anchors, positives, negatives (nA * nneg).
int train_step(iq_ctx* ctx, IqLp* lp, const float* feats, const int32_t* boxes,
               const std::vector<int32_t>& items, int nA, int nneg, double temp, double* loss) {
  const int64_t nitems = (int64_t)nA * (2 + nneg);
  const int G = lp->g.ng;
  int32_t* ditems = (int32_t*)iq_scratch(ctx, S_LP_ITEMS, sizeof(int32_t) * 4 * nitems);
  float* dX = (float*)iq_scratch(ctx, S_LP_X, sizeof(float) * 3 * G * nitems);
  float* dE = (float*)iq_scratch(ctx, S_LP_E, sizeof(float) * IQ_LP_EMB * nitems);
  float* dgE = (float*)iq_scratch(ctx, S_LP_GE, sizeof(float) * IQ_LP_EMB * nitems);
  if (!ditems || !dX || !dE || !dgE) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(ditems, items.data(), sizeof(int32_t) * 4 * nitems,
                             cudaMemcpyHostToDevice, ctx->stream));
  int rc = ensure_ii1(ctx, lp);
  if (rc) return rc;
  LpTrainBatch B;
  B.w = lp->w; B.items = ditems; B.nA = nA; B.nneg = nneg; B.temp = (float)temp;
  B.feats = feats; B.boxes = boxes; B.ii1 = lp->ii1; B.ii2 = ctx->d_ti2ii;
  B.img = ctx->ti; B.dist = dist_of(ctx, lp->tile);
  B.X = dX; B.E = dE; B.gE = dgE; B.grad = lp->grad; B.loss = lp->loss;
  return iq_lp_train_batch(ctx, lp->g, B, loss);  // synchronizes (host `items`)
}

}  // namespace

// Loss and parameter gradients of one batch (the gradient check): nA anchors given by their
// features (nA x 3 x cells), one positive and nneg negatives per anchor given by their positions,
// every window under the mask box (lo[3], hi[3]). Nothing is updated.
extern "C" int iq_lp_loss_grad(iq_ctx* ctx, int32_t nA, int32_t nneg, const float* anchor_feats,
                               const int64_t* pos_positions, const int64_t* neg_positions,
                               const int32_t* box, double temp, double* loss, float* grad) {
  if (!ctx || nA <= 0 || nneg < 0 || !anchor_feats || !pos_positions || !box || !loss || !grad ||
      (nneg > 0 && !neg_positions) || !(temp > 0))
    return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (!ctx->has_ti) return iq_set_error(IQ_ERR_STATE, "no training image set");
  IqLp* lp = ctx->lp;
  if (!lp || !lp->w) return iq_set_error(IQ_ERR_STATE, "no proposal parameters (iq_lp_init)");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  const int G = lp->g.ng;
  float* dfeat = (float*)iq_scratch(ctx, S_LP_FEAT, sizeof(float) * 3 * G * nA);
  int32_t* dbox = (int32_t*)iq_scratch(ctx, S_LP_TBOX, sizeof(int32_t) * 6);
  if (!dfeat || !dbox) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(dfeat, anchor_feats, sizeof(float) * 3 * G * nA, cudaMemcpyHostToDevice, ctx->stream));
  IQ_CUDA_OK(cudaMemcpyAsync(dbox, box, sizeof(int32_t) * 6, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<int32_t> items;
  for (int b = 0; b < nA; ++b) { items.push_back(b); items.push_back(-1); items.push_back(0); items.push_back(0); }
  for (int b = 0; b < nA; ++b) {
    items.push_back(-1); items.push_back((int32_t)pos_positions[b]); items.push_back(0); items.push_back(0);
  }
  for (int64_t i = 0; i < (int64_t)nA * nneg; ++i) {
    items.push_back(-1); items.push_back((int32_t)neg_positions[i]); items.push_back(0); items.push_back(0);
  }
  int rc = train_step(ctx, lp, dfeat, dbox, items, nA, nneg, temp, loss);
  if (rc) return rc;
  IQ_CUDA_OK(cudaMemcpy(grad, lp->grad, sizeof(float) * lp->g.npar, cudaMemcpyDefault));
  return IQ_OK;
}

// Trains the encoder on the captured pairs: `steps` Adam steps over batches of `batch` anchors,
// each with one of its captured candidates as the positive and `nneg` random positions as the
// negatives. loss_first / loss_last: batch losses of the first and last step.
extern "C" int iq_lp_train(iq_ctx* ctx, int32_t steps, int32_t batch, int32_t nneg, double lr,
                           double temp, uint64_t seed, double* loss_first, double* loss_last) {
  if (!ctx || steps <= 0 || batch <= 0 || nneg <= 0 || !(lr > 0) || !(temp > 0))
    return iq_set_error(IQ_ERR_ARG, "invalid argument");
  IqLp* lp = ctx->lp;
  if (!lp || !lp->w) return iq_set_error(IQ_ERR_STATE, "no proposal parameters (iq_lp_init)");
  if (lp->cap_n <= 0) return iq_set_error(IQ_ERR_STATE, "no captured training pairs");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  std::vector<int32_t> hpos((size_t)lp->cap_n * NPOS);
  IQ_CUDA_OK(cudaMemcpy(hpos.data(), lp->cap_pos, sizeof(int32_t) * hpos.size(), cudaMemcpyDeviceToHost));
  const int64_t P = lp->cap_dist.vol();
  uint32_t ctr = 0;
  auto rnd = [&](uint64_t m) { return (uint64_t)((unsigned __int128)iq_rand64(seed, ctr++, 1u, 5u) * m >> 64); };
  for (int s = 0; s < steps; ++s) {
    std::vector<int32_t> items;
    std::vector<int32_t> rows(batch), pos(batch);
    for (int b = 0; b < batch; ++b) {
      int32_t row = -1, p = -1;
      for (int tries = 0; tries < 64 && p < 0; ++tries) {
        row = (int32_t)rnd((uint64_t)lp->cap_n);
        p = hpos[(size_t)row * NPOS + rnd(NPOS)];
      }
      rows[b] = row;
      pos[b] = p < 0 ? 0 : p;
    }
    for (int b = 0; b < batch; ++b) { items.push_back(rows[b]); items.push_back(-1); items.push_back(rows[b]); items.push_back(0); }
    for (int b = 0; b < batch; ++b) { items.push_back(-1); items.push_back(pos[b]); items.push_back(rows[b]); items.push_back(0); }
    // negatives: random windows, and (lp.train_near of them) windows a few voxels from the
    // positive, which look alike but are rarely candidates: the ranking near the top
    const Dim3 dm = lp->cap_dist;
    const int nnear = std::min(nneg, ctx->lp_train_near);
    for (int b = 0; b < batch; ++b)
      for (int k = 0; k < nneg; ++k) {
        int64_t q = (int64_t)rnd((uint64_t)P);
        if (k < nnear) {
          const int64_t p = pos[b];
          const int64_t x = p % dm.x, y = (p / dm.x) % dm.y, z = p / (dm.x * dm.y);
          int64_t dx = 0, dy = 0, dz = 0;
          while (dx == 0 && dy == 0 && dz == 0) {
            dx = (int64_t)rnd(7) - 3;
            dy = (int64_t)rnd(7) - 3;
            dz = dm.z > 1 ? (int64_t)rnd(3) - 1 : 0;
          }
          const int64_t nx = std::min(std::max<int64_t>(x + dx, 0), dm.x - 1);
          const int64_t ny = std::min(std::max<int64_t>(y + dy, 0), dm.y - 1);
          const int64_t nz = std::min(std::max<int64_t>(z + dz, 0), dm.z - 1);
          q = nx + dm.x * (ny + dm.y * nz);
        }
        items.push_back(-1); items.push_back((int32_t)q); items.push_back(rows[b]); items.push_back(0);
      }
    double l = 0.0;
    const bool want = s == 0 || s == steps - 1;
    int rc = train_step(ctx, lp, lp->cap_feat, lp->cap_box, items, batch, nneg, temp, want ? &l : nullptr);
    if (rc) return rc;
    if (!want) IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));  // host `items`
    rc = iq_lp_adam(ctx, lp->w, lp->grad, lp->m, lp->v, lp->g.npar, (float)lr, ++lp->adam_step);
    if (rc) return rc;
    if (s == 0 && loss_first) *loss_first = l;
    if (s == steps - 1 && loss_last) *loss_last = l;
  }
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  lp->wversion += 1;
  return IQ_OK;
}

// Capacity for `n` captured pairs (0 frees them); capturing happens in iq_simulate while the
// option "lp.capture" is positive, for the tile shape of iq_lp_init.
int iq_lp_capture_reserve(iq_ctx* ctx, int64_t n) {
  IqLp* lp = lp_of(ctx);
  cudaFree(lp->cap_feat); cudaFree(lp->cap_box); cudaFree(lp->cap_pos);
  lp->cap_feat = nullptr; lp->cap_box = nullptr; lp->cap_pos = nullptr;
  lp->cap_n = 0;
  lp->cap_max = 0;
  if (n <= 0) return IQ_OK;
  if (!lp->w) return iq_set_error(IQ_ERR_STATE, "capture needs the proposal's tile (iq_lp_init)");
  if (cudaMalloc(&lp->cap_feat, sizeof(float) * 3 * lp->g.ng * n) != cudaSuccess ||
      cudaMalloc(&lp->cap_box, sizeof(int32_t) * 6 * n) != cudaSuccess ||
      cudaMalloc(&lp->cap_pos, sizeof(int32_t) * NPOS * n) != cudaSuccess) {
    cudaGetLastError();
    return iq_set_error(IQ_ERR_ALLOC, "capture buffers for %lld pairs", (long long)n);
  }
  lp->cap_max = n;
  return IQ_OK;
}

// Statistics of the last iq_simulate call: [0] columns picked from a shortlist, [1] columns of
// the full scan, [2] monitored columns, [3] their exact candidates, [4] of those shortlisted,
// [5] sampled recall (-1: none sampled), [6] 1 when the recall fell below 0.99 and the call
// fell back to the full scan, [7] mean shortlist length, [8] captured training pairs; with
// n >= 12 also [9] the shortlist length the call ended with, [10] the sampled recall at that
// length (-1: none sampled), [11] its sampled candidates.
extern "C" int iq_lp_stats(iq_ctx* ctx, double* out, int32_t n) {
  if (!ctx || !out || n < 9) return iq_set_error(IQ_ERR_ARG, "invalid argument");
  IqLp* lp = ctx->lp;
  for (int i = 0; i < n; ++i) out[i] = 0.0;
  if (!lp) {
    out[5] = -1.0;
    if (n >= 12) out[10] = -1.0;
    return IQ_OK;
  }
  out[0] = (double)lp->cols_lp;
  out[1] = (double)lp->cols_full;
  out[2] = (double)lp->mon_cols;
  out[3] = lp->mon_true;
  out[4] = lp->mon_hit;
  out[5] = lp->mon_true > 0 ? lp->mon_hit / lp->mon_true : -1.0;
  out[6] = lp->off ? 1.0 : 0.0;
  out[7] = lp->cols_lp > 0 ? (double)lp->short_total / (double)lp->cols_lp : 0.0;
  out[8] = (double)lp->cap_n;
  if (n >= 12) {
    out[9] = (double)(lp->k_cur > 0 ? lp->k_cur : ctx->lp_k);
    out[10] = lp->ph_true > 0 ? lp->ph_hit / lp->ph_true : -1.0;
    out[11] = lp->ph_true;
  }
  return IQ_OK;
}

void iq_lp_count_full(iq_ctx* ctx, int64_t ncol) {
  if (ctx->lp) ctx->lp->cols_full += ncol;
}
