// The pick of the learned proposal: exact distances at a column's shortlisted positions, then the
// pick of src/iqsim.jl:236-246 on them -- threshold (1 + tol) min D, tau-model weights
// (src/taumodel.jl:5-45, one source) and the StatsBase draw in the fixed summation order of the
// full pick (iq_pick.cu). The distances are FP32 direct sums, exact for the integer-valued
// (categorical) data the proposal serves; whenever the shortlist holds the full candidate set
// the result equals the full scan's.
#include "iq_internal.h"

namespace {

constexpr int LP_PT = 1024;
constexpr int LP_SORT = 8192;  // candidates a column's pick sorts in shared memory

struct LpPickArgs {
  const float* img;            // training image
  int64_t isx, isxy;
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
  // terms of the column's mask in shared memory
  int32_t* off = reinterpret_cast<int32_t*>(dyn);
  float* tv = reinterpret_cast<float*>(dyn + 4 * (size_t)col.K);
  for (int j = threadIdx.x; j < col.K; j += LP_PT) {
    const uint32_t k = col.klist[j];
    const int kx = kx_of(k), ky = ky_of(k), kz = kz_of(k);
    off[j] = (int32_t)(kx + a.isx * ky + a.isxy * kz);
    tv[j] = col.tmpl[kx + col.tgx * ky + col.tgxy * kz];
  }
  if (threadIdx.x == 0) smin = 0x7F7FFFFFu;
  __syncthreads();
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
    const float* base = a.img + x + a.isx * y + a.isxy * z;
    float acc = 0.f;
    int j = lane;
    bool pruned = false;
    for (int nx = 0; j + 96 < col.K; j += 128) {
      const float d0 = base[off[j]] - tv[j], d1 = base[off[j + 32]] - tv[j + 32];
      const float d2 = base[off[j + 64]] - tv[j + 64], d3 = base[off[j + 96]] - tv[j + 96];
      acc = fmaf(d0, d0, acc);
      acc = fmaf(d1, d1, acc);
      acc = fmaf(d2, d2, acc);
      acc = fmaf(d3, d3, acc);
      if (++nx == 4) {  // every 512 terms
        nx = 0;
        float part = acc;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        const float bound = __uint_as_float(*(volatile unsigned*)&smin) * pf;
        if (part > bound) { pruned = true; break; }
      }
    }
    if (!pruned)
      for (; j < col.K; j += 32) {
        const float d = base[off[j]] - tv[j];
        acc = fmaf(d, d, acc);
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (pruned) acc = INFINITY;
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
  const double tw = thr > 0.0 ? __dmul_rn(1e-6, thr) : -1.0;
  for (int i = threadIdx.x; i < n; i += LP_PT) {
    const double d = (double)dl[i];
    if (fabs(__dsub_rn(d, thr)) <= tw) nt++;
    if (d <= thr) {
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

int iq_lp_pick(iq_ctx* ctx, const float* img, Dim3 imgd, Dim3 dist, const LpColumn* cols, int N,
               const int32_t* list, const int32_t* cnt, int cap, float* dl, double tol,
               uint64_t seed, int64_t* rind, int64_t* ncand, int maxK) {
  if (N <= 0) return IQ_OK;
  LpPickArgs a{};
  a.img = img; a.isx = imgd.x; a.isxy = imgd.x * imgd.y; a.dx = dist.x; a.dxy = dist.x * dist.y;
  a.cols = cols; a.list = list; a.cnt = cnt; a.cap = cap; a.dl = dl; a.tol = tol; a.seed = seed;
  a.rind = rind; a.ncand = ncand; a.ties = ctx->d_ties;
  // shared memory: the mask's terms (8 bytes each), later the sort buffers, weights and sums
  const size_t sm = std::max<size_t>((size_t)8 * maxK,
                                     (size_t)LP_SORT * (8 + 8 + 8 + 4) +
                                         8 * ((LP_SORT + IQ_DRAW_CHUNK - 1) / IQ_DRAW_CHUNK)) + 64;
  if (sm > 227 * 1024)
    return iq_set_error(IQ_ERR_LIMIT, "proposal pick: a mask of %d offsets is too large", maxK);
  IQ_CUDA_OK(cudaFuncSetAttribute(lp_pick_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  iq_timer_start(ctx, "lp.pick");
  lp_pick_kernel<<<(unsigned)N, LP_PT, sm, ctx->stream>>>(a);
  iq_timer_stop(ctx, "lp.pick");
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
