// The pick of the learned proposal: exact distances at a column's shortlisted positions, then the
// pick of src/iqsim.jl:236-246 on them -- threshold (1 + tol) min D, tau-model weights
// (src/taumodel.jl:5-45, one source) and the StatsBase draw in the fixed summation order of the
// full pick (iq_pick.cu). The distances are integer sums (exact) over the categorical codes the
// proposal serves; whenever the shortlist holds the full candidate set the result equals the
// full scan's.
//
// Codes 0..3 with tiles of x extent <= 32: the training image as 2-bit planes and the template
// as staged rows, one row of 32 codes per lane step (iq_plane_ssd in iq_internal.h). Other byte
// codes: the image as bytes and the mask as quads of four consecutive x offsets of one row; a
// lane forms the four differences of a quad with one __vabsdiffu4 and adds their squares with
// one __dp4a. A sum stops early once it exceeds (1 + tol) x the running minimum x (1 + 2e-6).
#include "iq_internal.h"

namespace {

constexpr int LP_PT = 1024;
constexpr int LP_SORT = 8192;  // candidates a column's pick sorts in shared memory

struct LpPickArgs {
  LpImg im;                    // training image (plane or byte form)
  int64_t dx, dxy;             // distance-map strides
  const LpColumn* cols;        // per column: mask offsets, template, tile, realization
  const int32_t* list;         // shortlists [N][cap]
  const int32_t* cnt;
  int cap;
  float* dl;                   // distances of the shortlist entries [N][cap]
  double tol;
  uint64_t seed;
  int64_t* rind;               // per column: drawn position, -1 when the column must fall back
  int64_t* ncand;
  unsigned long long* ties;
};

__device__ __forceinline__ void lp_bitonic(unsigned long long* buf, int n) {
  int n2 = 2;
  while (n2 < n) n2 <<= 1;
  for (int i = n + threadIdx.x; i < n2; i += LP_PT) buf[i] = ~0ull;
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += LP_PT) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = buf[i], b = buf[l];
          if ((a > b) == ((i & k) == 0)) { buf[i] = b; buf[l] = a; }
        }
      }
      __syncthreads();
    }
}

__global__ void __launch_bounds__(LP_PT) lp_pick_kernel(const LpPickArgs a) {
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ float red[32];
  __shared__ unsigned long long ured[32];
  __shared__ int sflag;
  __shared__ unsigned smin;  // running minimum of the finished sums (bits of a non-negative float)
  const int c = blockIdx.x;
  const LpColumn col = a.cols[c];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = min(a.cnt[c], a.cap);
  if (a.cnt[c] > a.cap || n <= 0) {  // overflowed or empty shortlist: the column falls back
    if (threadIdx.x == 0) { a.rind[c] = -1; a.ncand[c] = 0; }
    return;
  }
  // the column's rows (plane form) or quads (byte form) in shared memory
  uint4* qd = reinterpret_cast<uint4*>(dyn);
  if (threadIdx.x == 0) smin = 0x7F7FFFFFu;
  const int nst = iq_stage(a.im, col, qd);
  if (nst < 0) {  // template values outside the form: the column falls back
    if (threadIdx.x == 0) { a.rind[c] = -1; a.ncand[c] = 0; }
    return;
  }
  // An entry is abandoned once a partial sum exceeds (1 + tol) * running minimum * (1 + 2e-6):
  // the terms are non-negative and the sums exact, so its full sum lies above the final
  // threshold by more than the near-tie band and it neither sets the minimum nor is a candidate.
  const float pf = (float)((1.0 + a.tol) * (1.0 + 2e-6));
  const int32_t* lst = a.list + (int64_t)c * a.cap;
  float* dl = a.dl + (int64_t)c * a.cap;
  float mloc = 3.4e38f;
  for (int i = warp; i < n; i += LP_PT / 32) {
    const int64_t p = lst[i];
    const int64_t z = p / a.dxy, r = p - z * a.dxy, y = r / a.dx, x = r - y * a.dx;
    const uint32_t s = iq_lp_ssd(a.im, qd, nst, x, y, z, [&] {
      return __uint_as_float(*(volatile unsigned*)&smin) * pf;
    });
    const bool pruned = s == 0xFFFFFFFFu;
    const float acc = pruned ? INFINITY : (float)s;
    if (lane == 0) {
      dl[i] = acc;
      if (!pruned) atomicMin(&smin, __float_as_uint(acc));
    }
    mloc = fminf(mloc, acc);
  }
  // minimum
  for (int o = 16; o > 0; o >>= 1) mloc = fminf(mloc, __shfl_xor_sync(0xffffffffu, mloc, o));
  if (lane == 0) red[warp] = mloc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float mm = red[0];
    for (int i = 1; i < LP_PT / 32; ++i) mm = fminf(mm, red[i]);
    red[0] = mm;
    sflag = 0;
  }
  __syncthreads();
  const double thr = __dmul_rn(__dadd_rn(1.0, a.tol), (double)red[0]);
  // candidates (position, value) and near-ties
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(dyn);
  unsigned long long nt = 0;
  // the Float64 tests d <= thr and |d - thr| <= 1e-6 thr as FP32 comparisons
  const float thr_f = f_dn(thr);
  float tlo = 1.f, thi = 0.f;
  if (thr > 0.0 && thr < 1e300) tie_window_f(thr, __dmul_rn(1e-6, thr), tlo, thi);
  for (int i = threadIdx.x; i < n; i += LP_PT) {
    const float d = dl[i];
    if (d >= tlo && d <= thi) nt++;
    if (d <= thr_f) {
      const int at = atomicAdd(&sflag, 1);
      if (at < LP_SORT) keys[at] = ((unsigned long long)(uint32_t)lst[i] << 32) | __float_as_uint(dl[i]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) nt += __shfl_xor_sync(0xffffffffu, nt, o);
  if (lane == 0) ured[warp] = nt;
  __syncthreads();
  const int nc = sflag;
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int i = 0; i < LP_PT / 32; ++i) t += ured[i];
    if (a.ties && t) atomicAdd(a.ties, t);
  }
  if (nc > LP_SORT) {
    if (threadIdx.x == 0) { a.rind[c] = -1; a.ncand[c] = nc; }
    return;
  }
  __syncthreads();
  lp_bitonic(keys, nc);  // ascending position: the candidate order of findall
  if (nc == 1) {
    if (threadIdx.x == 0) { a.rind[c] = (int64_t)(keys[0] >> 32); a.ncand[c] = 1; }
    return;
  }
  // dense ranks of D: sort (value bits, candidate index)
  unsigned long long* rk = keys + LP_SORT;
  for (int i = threadIdx.x; i < nc; i += LP_PT)
    rk[i] = ((unsigned long long)(uint32_t)keys[i] << 32) | (uint32_t)i;
  __syncthreads();
  lp_bitonic(rk, nc);
  double* w = reinterpret_cast<double*>(rk + LP_SORT);
  uint32_t* rank = reinterpret_cast<uint32_t*>(w + LP_SORT);
  if (threadIdx.x == 0) {
    uint32_t r = 0, prev = 0xFFFFFFFFu;
    unsigned long long S = 0;
    for (int i = 0; i < nc; ++i) {
      const uint32_t v = (uint32_t)(rk[i] >> 32);
      if (i == 0 || v != prev) ++r;
      prev = v;
      rank[(uint32_t)rk[i]] = r;
      S += (unsigned long long)(nc - r + 1);
    }
    ured[0] = S;
  }
  __syncthreads();
  // tau model with one source, the arithmetic of the full pick: P = (n - r + 1) / S,
  // X = (1 - P) / P, x = x0 * (1 * X / x0), p = 1 / (1 + x)
  const double dS = (double)ured[0];
  const double inv_n = __ddiv_rn(1.0, (double)nc);
  const double x0 = __ddiv_rn(__dsub_rn(1.0, inv_n), inv_n);
  for (int i = threadIdx.x; i < nc; i += LP_PT) {
    const double Pi = __ddiv_rn((double)(nc - (int64_t)rank[i] + 1), dS);
    const double X = __ddiv_rn(__dsub_rn(1.0, Pi), Pi);
    const double prod = __dmul_rn(1.0, __ddiv_rn(X, x0));
    w[i] = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(x0, prod)));
  }
  __syncthreads();
  // weighted draw: chunk sums left to right, then the chunk totals left to right
  double* csum = reinterpret_cast<double*>(rank + LP_SORT);
  const int nch = (nc + IQ_DRAW_CHUNK - 1) / IQ_DRAW_CHUNK;
  for (int ch = threadIdx.x; ch < nch; ch += LP_PT) {
    double run = 0.0;
    const int lo = ch * IQ_DRAW_CHUNK, hi = min(nc, lo + IQ_DRAW_CHUNK);
    for (int i = lo; i < hi; ++i) run = __dadd_rn(run, w[i]);
    csum[ch] = run;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int ch = 0; ch < nch; ++ch) { run = __dadd_rn(run, csum[ch]); csum[ch] = run; }
    const double u = iq_draw_uniform(a.seed, col.tile, col.real);
    const double t = __dmul_rn(u, run);
    int ch = 0;
    while (ch < nch - 1 && csum[ch] < t) ++ch;
    const double base = ch == 0 ? 0.0 : csum[ch - 1];
    const int lo = ch * IQ_DRAW_CHUNK, hi = min(nc, lo + IQ_DRAW_CHUNK);
    double part = 0.0;
    int pick = hi - 1;
    for (int i = lo; i < hi; ++i) {
      part = __dadd_rn(part, w[i]);
      if (__dadd_rn(base, part) >= t) { pick = i; break; }
    }
    a.rind[c] = (int64_t)(keys[pick] >> 32);
    a.ncand[c] = nc;
  }
}

}  // namespace

int iq_lp_pick(iq_ctx* ctx, const LpImg& im, Dim3 dist, const LpColumn* cols, int N,
               const int32_t* list, const int32_t* cnt, int cap, float* dl, double tol,
               uint64_t seed, int64_t* rind, int64_t* ncand, int maxQ) {
  if (N <= 0) return IQ_OK;
  LpPickArgs a{};
  a.im = im; a.dx = dist.x; a.dxy = dist.x * dist.y;
  a.cols = cols; a.list = list; a.cnt = cnt; a.cap = cap; a.dl = dl; a.tol = tol; a.seed = seed;
  a.rind = rind; a.ncand = ncand; a.ties = ctx->d_ties;
  // shared memory: the mask's rows or quads (16 bytes each; maxQ: the most of either), later
  // the sort buffers, weights and sums
  const size_t sm = std::max<size_t>((size_t)16 * maxQ,
                                     (size_t)LP_SORT * (8 + 8 + 8 + 4) +
                                         8 * ((LP_SORT + IQ_DRAW_CHUNK - 1) / IQ_DRAW_CHUNK)) + 64;
  if (sm > 227 * 1024)
    return iq_set_error(IQ_ERR_LIMIT, "proposal pick: a mask of %d quads is too large", maxQ);
  IQ_CUDA_OK(cudaFuncSetAttribute(lp_pick_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  iq_timer_start(ctx, "lp.pick");
  lp_pick_kernel<<<(unsigned)N, LP_PT, sm, ctx->stream>>>(a);
  iq_timer_stop(ctx, "lp.pick");
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
