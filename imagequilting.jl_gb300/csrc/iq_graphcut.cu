// Minimum-error boundary cut of the overlap slabs (src/graphcut.jl:5-84).
//
// One CTA per (realization, slab). The lattice graph, the capacities
//   c(u, v) = (|A-B|_u + |A-B|_v) / (|A_v-A_u| + |A_w-A_v| + |B_v-B_u| + |B_w-B_v| + eps())
// (Float32 differences and sums, Float64 division, as Julia does for Float32 arrays) and the
// infinite source/sink slices follow the reference. The max-flow is a synchronous
// push-relabel instead of Boykov-Kolmogorov:
//   * the first slice along the cut dimension is contracted into s, the last into t;
//   * capacities are rounded to multiples of q = 2^(ilogb(cmax) - 47), cmax the largest of
//     the slab, so that every residual (<= 2 cmax) and excess (<= 12 cmax) is a multiple of q
//     below 2^53 q and all flow arithmetic is exact (zero gradient sums give eps-denominator
//     capacities ~2^52 times the others, which unquantized Float64 flows cannot resolve);
//   * residuals are stored per directed arc in Float64; an arc is open when its residual is
//     positive (the oracle quantizes and tests the same way);
//   * each round: every active node pushes along its first admissible arc (h(u) = h(v) + 1),
//     then every node gathers the flow pushed into it in a fixed order and relabels if it
//     still has excess and no admissible arc -- deterministic, no atomics;
//   * a global relabel (BFS from t over open arcs) runs at the start, every GR rounds and at
//     the end; nodes that cannot reach t get height NH and stop being active.
// At the end the nodes that can reach t are the sink side of the canonical minimum cut (the
// same set for every maximum flow, which is what BK's sink tree holds at termination), and
// mask = not sink side (graphcut.jl:75-81). Excess arithmetic uses __dadd/__dsub; every
// comparison is done on the bit patterns of non-negative doubles (integer compares).
#include "iq_internal.h"

namespace {

constexpr int CUT_MAX_THREADS = 1024;

struct CutArgs {
  StepTask t0;                 // used when tasks is null
  const StepTask* tasks;
  int nreal;                   // CTA (s, y): slab s of realization y % nreal of task y / nreal
  const float* sim; int64_t sx, sy; int64_t sim_rs;
  const float* ti; int64_t tix, tiy; int64_t dx, dy;
  const int64_t* rind;
  const float* A; const float* B;
  uint8_t* out; int64_t slabmax;
  char* scratch; int64_t scratch_per_cta;
  int* status;
  int round_cap;
  unsigned long long* stats;
  int gr_period;
};

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

struct Graph {
  int n, ext[3], st[3];
  int d;          // cut dimension
  int L;          // extent along d
  int NH;         // height of s (= number of interior nodes + 2)
  double* rf[3];
  double* rb[3];
  double* ex;
  double* pamt;
  int* h[2];
  int* front[2];  // BFS frontier lists
  signed char* pdir;
  uint8_t* info;  // bits 0-5: neighbour exists in direction 0..5; bits 6-7: kind

  __device__ __forceinline__ int kind(int u) const { return info[u] >> 6; }  // 0 interior, 1 s, 2 t
  __device__ __forceinline__ bool nbr(int u, int dir, int& v) const {
    if (!(info[u] >> dir & 1)) return false;
    v = (dir & 1) ? u + st[dir >> 1] : u - st[dir >> 1];
    return true;
  }
  __device__ __forceinline__ int height(const int* hc, int v) const {
    int k = kind(v);
    return k == 1 ? NH : (k == 2 ? 0 : hc[v]);
  }
  // residual u->v (and pointers to both arc residuals) for direction dir
  __device__ __forceinline__ void arc(int u, int v, int dir, double*& ruv, double*& rvu) const {
    const int e = dir >> 1;
    if (dir & 1) { ruv = &rf[e][u]; rvu = &rb[e][u]; }
    else { ruv = &rb[e][v]; rvu = &rf[e][v]; }
  }
  __device__ __forceinline__ bool open(const double* ruv, const double*) const {
    return dbits(*ruv) > 0;  // residuals are non-negative; +0 and -0 are closed
  }
};

// Exact heights: breadth-first search from t over open arcs. Each level only examines the
// neighbours of the previous level's frontier (frontier lists fa/fb, counters cnt[2]), so the
// search costs O(edges) instead of O(nodes x levels). Heights are BFS distances, whatever
// order the frontier is filled in. Returns the number of levels.
__device__ int global_relabel(const Graph& g, int* hc, int* fa, int* fb, int* cnt) {
  if (threadIdx.x == 0) { cnt[0] = 0; cnt[1] = 0; }
  __syncthreads();
  const int dsink = 2 * g.d + 1;  // direction towards the sink slice
  for (int u = threadIdx.x; u < g.n; u += blockDim.x) {
    if (g.kind(u) != 0) continue;
    int h = g.NH;
    int v;
    if (g.nbr(u, dsink, v) && g.kind(v) == 2) {
      double *ruv, *rvu;
      g.arc(u, v, dsink, ruv, rvu);
      if (g.open(ruv, rvu)) h = 1;
    }
    hc[u] = h;
    if (h == 1) fa[atomicAdd(&cnt[0], 1)] = u;
  }
  __syncthreads();
  int level = 1, cur = 0;
  for (;;) {
    const int nf = cnt[cur];
    int* front = cur ? fb : fa;
    int* next = cur ? fa : fb;
    if (nf == 0) break;
    if (threadIdx.x == 0) cnt[cur ^ 1] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      const int v = front[i];
      for (int dir = 0; dir < 6; ++dir) {
        int u;
        if (!g.nbr(v, dir, u)) continue;
        if (g.kind(u) != 0 || hc[u] != g.NH) continue;
        double *ruv, *rvu;
        g.arc(u, v, dir ^ 1, ruv, rvu);  // arc u -> v
        if (!g.open(ruv, rvu)) continue;
        if (atomicCAS(&hc[u], g.NH, level + 1) == g.NH) next[atomicAdd(&cnt[cur ^ 1], 1)] = u;
      }
    }
    __syncthreads();
    cur ^= 1;
    ++level;
  }
  __syncthreads();
  return level;
}

__global__ void __launch_bounds__(CUT_MAX_THREADS) cut_kernel(const CutArgs a) {
  extern __shared__ __align__(16) char smem[];
  const int s_id = blockIdx.x;
  const int y = blockIdx.y;
  const int r = y % a.nreal;
  const StepTask& tk = a.tasks ? a.tasks[y / a.nreal] : a.t0;
  if (s_id >= tk.nslab) return;
  const CutSlab sl = tk.slab[s_id];
  const int64_t tile_start = tk.start;
  Graph g;
  g.ext[0] = (int)sl.ext[0]; g.ext[1] = (int)sl.ext[1]; g.ext[2] = (int)sl.ext[2];
  g.st[0] = 1; g.st[1] = g.ext[0]; g.st[2] = g.ext[0] * g.ext[1];
  g.n = g.ext[0] * g.ext[1] * g.ext[2];
  g.d = sl.dim;
  g.L = g.ext[g.d];
  g.NH = g.n / g.L * (g.L > 2 ? g.L - 2 : 0) + 2;
  const int n = g.n;

  char* base = a.scratch ? a.scratch + (int64_t)(blockIdx.y * gridDim.x + blockIdx.x) *
                                           a.scratch_per_cta
                         : smem;
  double* dp = reinterpret_cast<double*>(base);
  for (int e = 0; e < 3; ++e) { g.rf[e] = dp + (2 * e) * n; g.rb[e] = dp + (2 * e + 1) * n; }
  g.ex = dp + 6 * n;
  g.pamt = dp + 7 * n;
  int* ip = reinterpret_cast<int*>(dp + 8 * n);
  g.h[0] = ip;
  g.h[1] = ip + n;
  g.front[0] = ip + 2 * n;
  g.front[1] = ip + 3 * n;
  __shared__ int s_cnt[2];
  __shared__ unsigned long long s_cmax;  // bits of the largest capacity
  if (threadIdx.x == 0) s_cmax = 0ull;
  g.pdir = reinterpret_cast<signed char*>(ip + 4 * n);
  g.info = reinterpret_cast<uint8_t*>(g.pdir + n);
  float* Av = reinterpret_cast<float*>(g.pamt);  // A and B alias pamt during set-up
  float* Bv = Av + n;                            // (8n bytes = pamt)
  // ex holds nothing yet either; B needs n floats after A: pamt is n doubles = 2n floats

  // ---- load A (simulation grid) and B (training image at the drawn pattern) ----
  int64_t bstart = 0;
  if (!a.A) {
    const int64_t ri = a.rind[y];
    if (ri < 0) {  // pick failed: no cut (status already set)
      for (int u = threadIdx.x; u < n; u += blockDim.x)
        a.out[((int64_t)y * 6 + s_id) * a.slabmax + u] = 0;
      return;
    }
    const int64_t rx = ri % a.dx, rr = ri / a.dx, ry = rr % a.dy, rz = rr / a.dy;
    bstart = rx + a.tix * (ry + a.tiy * rz);
  }
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    const int x = u % g.ext[0], y = (u / g.ext[0]) % g.ext[1], z = u / g.st[2];
    const int c[3] = {x, y, z};
    uint8_t inf = 0;
    for (int e = 0; e < 3; ++e) {
      if (c[e] > 0) inf |= (uint8_t)(1u << (2 * e));
      if (c[e] + 1 < g.ext[e]) inf |= (uint8_t)(1u << (2 * e + 1));
    }
    const int cd = c[g.d];
    inf |= (uint8_t)((cd == 0 ? 1 : (cd == g.L - 1 ? 2 : 0)) << 6);
    g.info[u] = inf;
    if (a.A) {
      Av[u] = a.A[u];
      Bv[u] = a.B[u];
    } else {
      const int64_t lx = sl.off[0] + x, ly = sl.off[1] + y, lz = sl.off[2] + z;
      Av[u] = a.sim[(int64_t)r * a.sim_rs + tile_start + lx + a.sx * (ly + a.sy * lz)];
      Bv[u] = a.ti[bstart + lx + a.tix * (ly + a.tiy * lz)];
    }
  }
  __syncthreads();

  // ---- capacities (graphcut.jl:22-50) ----
  const double EPS = 2.220446049250313e-16;  // eps(Float64) = 2^-52
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    for (int e = 0; e < 3; ++e) {
      int v;
      if (!g.nbr(u, 2 * e + 1, v)) continue;
      const bool ok = (g.info[v] >> (2 * e + 1)) & 1;
      const int w = ok ? v + g.st[e] : v;
      const float Du = fabsf(__fsub_rn(Av[u], Bv[u]));
      const float Dv = fabsf(__fsub_rn(Av[v], Bv[v]));
      const float gAu = fabsf(__fsub_rn(Av[v], Av[u]));
      const float gBu = fabsf(__fsub_rn(Bv[v], Bv[u]));
      const float gAv = ok ? fabsf(__fsub_rn(Av[w], Av[v])) : gAu;
      const float gBv = ok ? fabsf(__fsub_rn(Bv[w], Bv[v])) : gBu;
      const float num = __fadd_rn(Du, Dv);
      float den = __fadd_rn(gAu, gAv);
      den = __fadd_rn(den, gBu);
      den = __fadd_rn(den, gBv);
      const double cap = __ddiv_rn((double)num, __dadd_rn((double)den, EPS));
      g.rf[e][u] = cap;
      g.rb[e][u] = cap;
      atomicMax(&s_cmax, (unsigned long long)dbits(cap));
    }
  }
  __syncthreads();
  // ---- round every capacity to a multiple of q = 2^(ilogb(cmax) - 47) (exact flows) ----
  if (s_cmax != 0ull) {
    int sh = ilogb(__longlong_as_double((long long)s_cmax)) - 47;
    if (sh < -1074) sh = -1074;
    for (int u = threadIdx.x; u < n; u += blockDim.x)
      for (int e = 0; e < 3; ++e) {
        int v;
        if (!g.nbr(u, 2 * e + 1, v)) continue;
        const double c = ldexp(rint(ldexp(g.rf[e][u], -sh)), sh);
        g.rf[e][u] = c;
        g.rb[e][u] = c;
      }
    __syncthreads();
  }

  // ---- saturate the source slice: push c(s, v) into every interior node of slice 1 ----
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    double e0 = 0.0;
    if (g.kind(u) == 0 && g.kind(u - g.st[g.d]) == 1) {
      const int sN = u - g.st[g.d];
      const double c = g.rf[g.d][sN];
      g.rf[g.d][sN] = 0.0;
      g.rb[g.d][sN] = __dadd_rn(c, c);
      e0 = c;
    }
    g.ex[u] = e0;
    g.pdir[u] = -1;
  }
  __syncthreads();

  int cur = 0;
  int round = 0, levels = 0;
  if (g.L > 2) {
    levels += global_relabel(g, g.h[cur], g.front[0], g.front[1], s_cnt);
    bool capped = false;
    for (;;) {
      int* hc = g.h[cur];
      int* hn = g.h[cur ^ 1];
      // push phase
      for (int u = threadIdx.x; u < n; u += blockDim.x) {
        signed char pd = -1;
        if (g.kind(u) == 0 && dbits(g.ex[u]) > 0 && hc[u] < g.NH) {
          const int hu = hc[u];
          for (int dir = 0; dir < 6; ++dir) {
            int v;
            if (!g.nbr(u, dir, v)) continue;
            if (hu != g.height(hc, v) + 1) continue;
            double *ruv, *rvu;
            g.arc(u, v, dir, ruv, rvu);
            if (!g.open(ruv, rvu)) continue;
            const double e = g.ex[u], rr = *ruv;
            const double delta = dbits(e) < dbits(rr) ? e : rr;
            *ruv = __dsub_rn(rr, delta);
            *rvu = __dadd_rn(*rvu, delta);
            g.ex[u] = __dsub_rn(e, delta);
            g.pamt[u] = delta;
            pd = (signed char)dir;
            break;
          }
        }
        g.pdir[u] = pd;
      }
      __syncthreads();
      // gather + relabel phase
      int active = 0;
      for (int u = threadIdx.x; u < n; u += blockDim.x) {
        if (g.kind(u) != 0) continue;
        double e = g.ex[u];
        for (int dir = 0; dir < 6; ++dir) {
          int v;
          if (!g.nbr(u, dir, v)) continue;
          if (g.pdir[v] == (dir ^ 1) && g.kind(v) == 0) e = __dadd_rn(e, g.pamt[v]);
        }
        g.ex[u] = e;
        int hu = hc[u];
        int hnew = hu;
        if (dbits(e) > 0 && hu < g.NH) {
          bool adm = false;
          int mh = 0x7fffffff;
          for (int dir = 0; dir < 6; ++dir) {
            int v;
            if (!g.nbr(u, dir, v)) continue;
            double *ruv, *rvu;
            g.arc(u, v, dir, ruv, rvu);
            if (!g.open(ruv, rvu)) continue;
            const int hv = g.height(hc, v);
            if (hu == hv + 1) { adm = true; break; }
            mh = min(mh, hv);
          }
          if (!adm) hnew = mh >= g.NH - 1 ? g.NH : mh + 1;
        }
        hn[u] = hnew;
        if (dbits(e) > 0 && hnew < g.NH) active = 1;
      }
      active = __syncthreads_or(active);
      cur ^= 1;
      ++round;
      if (!active) break;
      if (round >= a.round_cap) { capped = true; break; }
      if (round % a.gr_period == 0) {
        levels += global_relabel(g, g.h[cur], g.front[0], g.front[1], s_cnt);
        __syncthreads();
      }
    }
    levels += global_relabel(g, g.h[cur], g.front[0], g.front[1], s_cnt);
    __syncthreads();
    if (capped && threadIdx.x == 0) iq_dev_fail(a.status, IQ_ERR_CUTCAP);
  }

  if (a.stats && threadIdx.x == 0) {
    atomicAdd(a.stats + ST_CUT_ROUNDS, (unsigned long long)round);
    atomicAdd(a.stats + ST_CUT_LEVELS, (unsigned long long)levels);
    atomicAdd(a.stats + ST_CUT_CTAS, 1ull);
    atomicMax(a.stats + ST_CUT_MAXROUNDS, (unsigned long long)round);
    atomicMax(a.stats + ST_CUT_MAXLEVELS, (unsigned long long)levels);
  }
  // ---- mask: not sink side ----
  const int* hc = g.h[cur];
  uint8_t* out = a.out + ((int64_t)y * 6 + s_id) * a.slabmax;
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    const int k = g.kind(u);
    int M = k == 1 ? 1 : (k == 2 ? 0 : (hc[u] >= g.NH ? 1 : 0));
    out[u] = (uint8_t)(sl.next ? !M : M);
  }
}

}  // namespace

size_t iq_cut_scratch_bytes(int64_t nodes) {
  // rf, rb (6n doubles), ex, pamt (2n doubles), two heights and two BFS frontiers (4n ints),
  // push dir and node info (2n bytes)
  size_t b = (size_t)nodes * (8 * 8 + 4 * 4 + 2);
  return (b + 255) & ~(size_t)255;
}

int iq_launch_cut(iq_ctx* ctx, const CutLaunch& L) {
  const int nslab_max = L.tasks ? L.nslab_max : L.t0.nslab;
  if (nslab_max <= 0 || L.nreal <= 0 || L.ntask <= 0) return IQ_OK;
  CutArgs a;
  a.t0 = L.t0;
  a.tasks = L.tasks;
  a.nreal = L.nreal;
  a.sim = L.sim; a.sx = L.sim_dims.x; a.sy = L.sim_dims.y; a.sim_rs = L.sim_rstride;
  a.ti = L.ti; a.tix = L.ti_dims.x; a.tiy = L.ti_dims.y;
  a.dx = L.dist_dims.x; a.dy = L.dist_dims.y;
  a.rind = L.rind;
  a.A = L.A; a.B = L.B;
  a.out = L.out; a.slabmax = L.slabmax;
  a.status = L.status;
  a.round_cap = L.round_cap;
  a.stats = L.stats;
  a.gr_period = L.gr_period > 0 ? L.gr_period : 32;
  const int64_t nmax = L.slabmax;
  const size_t need = iq_cut_scratch_bytes(nmax);
  static int smem_limit = -1;
  if (smem_limit < 0) {
    // dynamic shared memory may use the opt-in maximum minus the kernel's static part
    int dev = 0, v = 0;
    IQ_CUDA_OK(cudaGetDevice(&dev));
    IQ_CUDA_OK(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    IQ_CUDA_OK(cudaFuncGetAttributes(&fa, cut_kernel));
    const int lim = v - (int)fa.sharedSizeBytes;
    IQ_CUDA_OK(cudaFuncSetAttribute(cut_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    smem_limit = lim;
  }
  size_t dyn = 0;
  if ((int64_t)need <= smem_limit) {
    a.scratch = nullptr;
    a.scratch_per_cta = 0;
    dyn = need;
  } else {
    if (!L.scratch || L.scratch_per_cta < (int64_t)need)
      return iq_set_error(IQ_ERR_LIMIT, "graph cut slab of %lld nodes needs global scratch",
                          (long long)nmax);
    a.scratch = (char*)L.scratch;
    a.scratch_per_cta = L.scratch_per_cta;
  }
  const int threads = (L.threads == 256 || L.threads == 1024) ? L.threads : 512;
  dim3 grid((unsigned)nslab_max, (unsigned)(L.ntask * L.nreal));
  iq_timer_start(ctx, "graphcut");
  cut_kernel<<<grid, threads, dyn, ctx->stream>>>(a);
  iq_timer_stop(ctx, "graphcut", 0);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
