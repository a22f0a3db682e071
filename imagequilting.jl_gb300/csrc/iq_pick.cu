// Pattern pick of one tile for a batch of realizations: one 1024-thread CTA per realization.
//
//   threshold pick  findall(D .<= (1 + tol) * minimum(D))           src/iqsim.jl:237
//   relaxation      top-dbsize of D intersected with growing top-s    src/relaxation.jl:5-39
//                   sets of each auxiliary distance
//   tau model       dense ranks per source, P = (n - r + 1)/sum,     src/taumodel.jl:5-45
//                   x = x0 * prod((1 - P)/P / x0), p = 1/(1 + x)
//   draw            t = u * sum(p), first i with cumsum(p)[i] >= t   src/iqsim.jl:243
//
// "Top-k" follows partialsortperm: order by (value, index). The k-th key is found by an MSD
// radix select on the value bits (non-negative floats order like their bits) and, among equal
// values, on the index. Candidate lists are compacted in ascending index order. Dense ranks
// come from a stable LSD radix sort of the candidates' values. All Float64 arithmetic uses
// explicit round-to-nearest intrinsics so that the weights equal the oracle's bit for bit;
// the draw sums in the fixed order of oracle/iqsim_oracle.sample_index.
#include "iq_internal.h"

namespace {

constexpr int PT = 1024;
constexpr int NW = PT / 32;

struct PickArgs {
  int64_t P, npat;
  double tol;
  uint64_t seed;
  int64_t tile, real0;
  const float* D0; int64_t D0_rs;
  const unsigned* mm0; int64_t mm0_rs;
  int naux;
  const float* aux[IQ_MAX_AUX];
  int64_t aux_rs[IQ_MAX_AUX];
  int64_t dbsize_norm, dbsize_zero;
  int nseq_norm, nseq_zero;
  int64_t seq_norm[IQ_MAX_SEQ], seq_zero[IQ_MAX_SEQ];
  int32_t* cand;
  uint32_t *k0, *v0, *k1, *v1;
  double* w;
  double* prod;
  int64_t* rind;
  int64_t* ncand;
  int* status;
  unsigned long long* stats;
};

struct Smem {
  uint32_t hist[256];
  uint32_t base[256];
  uint32_t wcnt[NW][256];
  uint32_t warp[NW];
  unsigned long long wred[NW];
  uint32_t sel, cnt;
  int64_t kk;
  int flag;
  double dval;
  int64_t ival;
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive block prefix sum of v; returns prefix, writes the block total to `total`.
__device__ uint32_t block_excl_sum(Smem& s, uint32_t v, uint32_t& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s.warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = s.warp[lane];
    uint32_t u = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
      if (lane >= o) u += y;
    }
    s.warp[lane] = u - t;  // exclusive warp offsets
    if (lane == 31) s.cnt = u;
  }
  __syncthreads();
  uint32_t res = s.warp[wid] + x - v;
  total = s.cnt;
  __syncthreads();
  return res;
}

__device__ unsigned long long block_sum_u64(Smem& s, unsigned long long v) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) s.wred[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int i = 0; i < NW; ++i) t += s.wred[i];
    s.wred[0] = t;
  }
  __syncthreads();
  unsigned long long r = s.wred[0];
  __syncthreads();
  return r;
}

// Histograms are counted per warp (s.wcnt[warp][digit], one leader per distinct digit of a
// warp after __match_any_sync) and summed into s.hist: no two warps touch the same counter,
// which matters because float bit patterns pile into a few high-order digits.
__device__ __forceinline__ void whist_zero(Smem& s) {
  for (int i = threadIdx.x; i < NW * 256; i += PT) (&s.wcnt[0][0])[i] = 0;
  __syncthreads();
}

__device__ __forceinline__ void whist_add(Smem& s, bool valid, uint32_t d) {
  const int lane = threadIdx.x & 31;
  uint32_t key = valid ? d : (0x10000u + lane);
  uint32_t peers = __match_any_sync(0xffffffffu, key);
  if (valid && lane == __ffs(peers) - 1)
    atomicAdd(&s.wcnt[threadIdx.x >> 5][d], (uint32_t)__popc(peers));
}

__device__ __forceinline__ void whist_reduce(Smem& s) {
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += PT) {
    uint32_t t = 0;
#pragma unroll 8
    for (int w = 0; w < NW; ++w) t += s.wcnt[w][d];
    s.hist[d] = t;
  }
  __syncthreads();
}

// Bucket holding the kk-th (1-based) element of s.hist; sets s.sel, s.cnt, s.kk (rank
// within the bucket). Called by all threads.
__device__ void find_bucket(Smem& s, int64_t kk) {
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    uint32_t c[8];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) { c[i] = s.hist[lane * 8 + i]; sum += c[i]; }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    uint32_t exc = inc - sum;
    bool here = (int64_t)exc < kk && (int64_t)inc >= kk;
    uint32_t b = __ballot_sync(0xffffffffu, here);
    if (b != 0 && lane == __ffs(b) - 1) {
      int64_t k = kk - exc;
      int sel = 0;
      for (int i = 0; i < 8; ++i) {
        if ((int64_t)c[i] >= k) { sel = i; break; }
        k -= c[i];
      }
      s.sel = lane * 8 + sel;
      s.cnt = c[sel];
      s.kk = k;
    }
    if (b == 0 && lane == 0) { s.sel = 255; s.cnt = 0; s.kk = 0; }
  }
  __syncthreads();
}

struct Key { uint32_t v; uint32_t i; };

__device__ __forceinline__ bool key_le(uint32_t b, uint32_t p, Key k) {
  return b < k.v || (b == k.v && p <= k.i);
}

// The kk-th smallest (value, index) key of src[0..P) (1 <= kk <= P).
__device__ Key select_kth(Smem& s, const float* __restrict__ src, int64_t P, int64_t kk) {
  uint32_t prefix = 0, mask = 0;
  const int64_t iters = (P + PT - 1) / PT;
  uint32_t cnt_eq = 0;
  for (int shift = 24; shift >= 0; shift -= 8) {
    whist_zero(s);
    for (int64_t it = 0; it < iters; ++it) {
      int64_t p = it * PT + threadIdx.x;
      bool valid = p < P;
      uint32_t b = valid ? fbits(src[p]) : 0u;
      valid = valid && (b & mask) == prefix;
      whist_add(s, valid, (b >> shift) & 255u);
    }
    whist_reduce(s);
    find_bucket(s, kk);
    prefix |= s.sel << shift;
    mask |= 255u << shift;
    kk = s.kk;
    cnt_eq = s.cnt;
  }
  Key k{prefix, 0xFFFFFFFFu};
  if (kk >= (int64_t)cnt_eq) return k;  // every index with this value is inside
  // select among equal values by index
  int topbit = 0;
  while (topbit < 31 && ((int64_t)1 << (topbit + 1)) <= P - 1) ++topbit;
  uint32_t ip = 0, im = 0;
  for (int shift = (topbit / 8) * 8; shift >= 0; shift -= 8) {
    whist_zero(s);
    for (int64_t it = 0; it < iters; ++it) {
      int64_t p = it * PT + threadIdx.x;
      bool valid = p < P;
      uint32_t b = valid ? fbits(src[p]) : 0u;
      valid = valid && b == prefix && ((uint32_t)p & im) == ip;
      whist_add(s, valid, ((uint32_t)p >> shift) & 255u);
    }
    whist_reduce(s);
    find_bucket(s, kk);
    ip |= s.sel << shift;
    im |= 255u << shift;
    kk = s.kk;
  }
  k.i = ip;
  return k;
}

// Predicates over a position p.
struct ThrPred {
  const float* D; double thr;
  __device__ bool operator()(int64_t p) const { return (double)D[p] <= thr; }
};
struct RelaxPred {
  const float* D; Key kD;
  int naux; const float* aux[IQ_MAX_AUX]; Key ka[IQ_MAX_AUX];
  __device__ bool operator()(int64_t p) const {
    if (!key_le(fbits(D[p]), (uint32_t)p, kD)) return false;
    for (int a = 0; a < naux; ++a)
      if (!key_le(fbits(aux[a][p]), (uint32_t)p, ka[a])) return false;
    return true;
  }
};

constexpr int CITEMS = 8;

// Ordered compaction of {p : pred(p)} into out (if non-null); returns the count.
template <typename Pred>
__device__ int64_t compact(Smem& s, const Pred& pred, int64_t P, int32_t* out) {
  int64_t base = 0;
  const int64_t tile = (int64_t)PT * CITEMS;
  for (int64_t t0 = 0; t0 < P; t0 += tile) {
    const int64_t p0 = t0 + (int64_t)threadIdx.x * CITEMS;
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) {
      int64_t p = p0 + i;
      if (p < P && pred(p)) bits |= 1u << i;
    }
    uint32_t total;
    uint32_t off = block_excl_sum(s, (uint32_t)__popc(bits), total);
    if (out) {
      int64_t o = base + off;
#pragma unroll
      for (int i = 0; i < CITEMS; ++i)
        if (bits >> i & 1u) out[o++] = (int32_t)(p0 + i);
    }
    base += total;
  }
  return base;
}

// Stable LSD radix sort of (keys, vals)[0..n) between the buffer pairs; returns 0 if the
// result is in (ka, va), 1 if in (kb, vb).
__device__ int radix_sort(Smem& s, uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb,
                          int64_t n) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int cur = 0;
  const int64_t ntiles = (n + PT - 1) / PT;
  for (int shift = 0; shift < 32; shift += 8) {
    uint32_t* ks = cur ? kb : ka; uint32_t* vs = cur ? vb : va;
    uint32_t* kd = cur ? ka : kb; uint32_t* vd = cur ? va : vb;
    whist_zero(s);
    for (int64_t t = 0; t < ntiles; ++t) {
      int64_t i = t * PT + threadIdx.x;
      bool valid = i < n;
      uint32_t d = valid ? (ks[i] >> shift) & 255u : 0u;
      whist_add(s, valid, d);
    }
    whist_reduce(s);
    // single-bucket pass: order unchanged, skip it
    int single = 0;
    if (threadIdx.x < 256 && (int64_t)s.hist[threadIdx.x] == n) single = 1;
    if (__syncthreads_or(single)) continue;
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      for (int d = 0; d < 256; ++d) { s.base[d] = run; run += s.hist[d]; }
    }
    __syncthreads();
    for (int64_t t = 0; t < ntiles; ++t) {
      for (int i = threadIdx.x; i < NW * 256; i += PT) (&s.wcnt[0][0])[i] = 0;
      __syncthreads();
      int64_t i = t * PT + threadIdx.x;
      bool valid = i < n;
      uint32_t k = valid ? ks[i] : 0u, v = valid ? vs[i] : 0u;
      uint32_t d = (k >> shift) & 255u;
      uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : (0x10000u + lane));
      uint32_t rank = __popc(peers & lanemask_lt());
      if (valid && lane == __ffs(peers) - 1) s.wcnt[wid][d] = __popc(peers);
      __syncthreads();
      if (threadIdx.x < 256) {
        uint32_t run = s.base[threadIdx.x];
        for (int w = 0; w < NW; ++w) {
          uint32_t c = s.wcnt[w][threadIdx.x];
          s.wcnt[w][threadIdx.x] = run;
          run += c;
        }
        s.base[threadIdx.x] = run;
      }
      __syncthreads();
      if (valid) {
        uint32_t dst = s.wcnt[wid][d] + rank;
        kd[dst] = k;
        vd[dst] = v;
      }
      __syncthreads();
    }
    cur ^= 1;
  }
  return cur;
}

// Dense ranks (1-based) of src[cand[i]], i < n, written to rank[i]; returns the sum of
// (n - rank + 1) over i.
__device__ unsigned long long dense_ranks(Smem& s, const float* __restrict__ src,
                                          const int32_t* __restrict__ cand, int64_t n,
                                          uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1,
                                          uint32_t** rank_out) {
  unsigned mn = 0xFFFFFFFFu, mx = 0u;
  for (int64_t i = threadIdx.x; i < n; i += PT) {
    uint32_t b = fbits(src[cand[i]]);
    k0[i] = b;
    v0[i] = (uint32_t)i;
    mn = min(mn, b);
    mx = max(mx, b);
  }
  mn = __reduce_min_sync(0xffffffffu, mn);
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0) { s.hist[threadIdx.x >> 5] = mn; s.base[threadIdx.x >> 5] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned a = 0xFFFFFFFFu, b = 0u;
    for (int w = 0; w < NW; ++w) { a = min(a, s.hist[w]); b = max(b, s.base[w]); }
    s.flag = (a == b) ? 1 : 0;
  }
  __syncthreads();
  const bool all_equal = s.flag != 0;
  __syncthreads();
  if (all_equal) {
    for (int64_t i = threadIdx.x; i < n; i += PT) k1[i] = 1u;
    __syncthreads();
    *rank_out = k1;
    return (unsigned long long)n * (unsigned long long)n;  // each term n - 1 + 1
  }
  int where = radix_sort(s, k0, v0, k1, v1, n);
  uint32_t* ks = where ? k1 : k0;
  uint32_t* vs = where ? v1 : v0;
  uint32_t* rk = where ? k0 : k1;  // free buffer receives ranks (indexed by candidate)
  // inclusive scan of "value changes" in sorted order
  uint32_t carry = 0;
  unsigned long long acc = 0;
  for (int64_t t0 = 0; t0 < n; t0 += PT) {
    int64_t i = t0 + threadIdx.x;
    uint32_t f = 0;
    if (i < n) f = (i == 0 || ks[i] != ks[i - 1]) ? 1u : 0u;
    uint32_t total;
    uint32_t ex = block_excl_sum(s, f, total);
    if (i < n) {
      uint32_t r = carry + ex + f;
      // the sort buffers are read before the rank buffer is written: rk aliases neither
      rk[vs[i]] = r;
      acc += (unsigned long long)(n - r + 1);
    }
    carry += total;
  }
  __syncthreads();
  *rank_out = rk;
  return block_sum_u64(s, acc);
}

__global__ void __launch_bounds__(PT) pick_kernel(const PickArgs a) {
  __shared__ Smem s;
  const int r = blockIdx.x;
  const int64_t P = a.P;
  const float* D = a.D0 + r * a.D0_rs;
  const unsigned* mm = a.mm0 + r * a.mm0_rs;
  int32_t* cand = a.cand + r * P;
  uint32_t* k0 = a.k0 + r * P;
  uint32_t* v0 = a.v0 + r * P;
  uint32_t* k1 = a.k1 + r * P;
  uint32_t* v1 = a.v1 + r * P;
  double* w = a.w + r * P;
  double* prod = a.prod + r * P;
  const float* aux[IQ_MAX_AUX];
  for (int j = 0; j < a.naux; ++j) aux[j] = a.aux[j] + r * a.aux_rs[j];

  int64_t n;
  if (a.naux == 0) {
    const float mn = __uint_as_float(mm[0]);
    const double thr = __dmul_rn(__dadd_rn(1.0, a.tol), (double)mn);
    ThrPred pr{D, thr};
    n = compact(s, pr, P, cand);
  } else {
    if (a.npat <= 0) {
      if (threadIdx.x == 0) { iq_dev_fail(a.status, IQ_ERR_NOPATTERN); a.rind[r] = -1; }
      return;
    }
    const bool allzero = mm[1] == 0u;
    const int64_t dbsize = allzero ? a.dbsize_zero : a.dbsize_norm;
    const int nseq = allzero ? a.nseq_zero : a.nseq_norm;
    RelaxPred pr;
    pr.D = D;
    pr.naux = a.naux;
    for (int j = 0; j < a.naux; ++j) pr.aux[j] = aux[j];
    pr.kD = select_kth(s, D, P, dbsize);
    n = 0;
    int q = 0;
    for (; q < nseq && n == 0; ++q) {
      const int64_t sz = allzero ? a.seq_zero[q] : a.seq_norm[q];
      for (int j = 0; j < a.naux; ++j) {
        if (sz >= P) pr.ka[j] = Key{0xFFFFFFFFu, 0xFFFFFFFFu};
        else if (sz <= 0) pr.ka[j] = Key{0u, 0u};  // nothing selected (never at valid sizes)
        else pr.ka[j] = select_kth(s, aux[j], P, sz);
      }
      // the compaction counts: an empty intersection moves on to the next softdbsize
      n = compact(s, pr, P, cand);
    }
    if (a.stats && threadIdx.x == 0) atomicAdd(a.stats + ST_PICK_ITERS, (unsigned long long)q);
  }
  if (n <= 0) {
    if (threadIdx.x == 0) { iq_dev_fail(a.status, IQ_ERR_NOPATTERN); a.rind[r] = -1; }
    return;
  }
  if (a.ncand && threadIdx.x == 0) a.ncand[r] = n;
  if (a.stats && threadIdx.x == 0) {
    atomicAdd(a.stats + ST_PICK_CAND, (unsigned long long)n);
    atomicAdd(a.stats + ST_PICK_CTAS, 1ull);
  }

  // ---- tau model weights ----
  if (n == 1) {
    if (threadIdx.x == 0) { w[0] = 1.0; a.rind[r] = cand[0]; }
    return;
  }
  const double dn = (double)n;
  const double inv_n = __ddiv_rn(1.0, dn);
  const double x0 = __ddiv_rn(__dsub_rn(1.0, inv_n), inv_n);
  for (int64_t i = threadIdx.x; i < n; i += PT) prod[i] = 1.0;
  const int nsrc = 1 + a.naux;
  for (int j = 0; j < nsrc; ++j) {
    const float* src = j == 0 ? D : aux[j - 1];
    __syncthreads();
    uint32_t* rank;
    unsigned long long S = dense_ranks(s, src, cand, n, k0, v0, k1, v1, &rank);
    const double dS = (double)S;
    for (int64_t i = threadIdx.x; i < n; i += PT) {
      const double Pi = __ddiv_rn((double)(n - (int64_t)rank[i] + 1), dS);
      const double X = __ddiv_rn(__dsub_rn(1.0, Pi), Pi);
      prod[i] = __dmul_rn(prod[i], __ddiv_rn(X, x0));
    }
    __syncthreads();
  }
  for (int64_t i = threadIdx.x; i < n; i += PT)
    w[i] = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(x0, prod[i])));
  __syncthreads();

  // ---- weighted draw ----
  const int64_t nch = (n + IQ_DRAW_CHUNK - 1) / IQ_DRAW_CHUNK;
  double* csum = prod;  // reuse
  for (int64_t c = threadIdx.x; c < nch; c += PT) {
    double run = 0.0;
    const int64_t lo = c * IQ_DRAW_CHUNK, hi = min(n, lo + IQ_DRAW_CHUNK);
    for (int64_t i = lo; i < hi; ++i) run = __dadd_rn(run, w[i]);
    csum[c] = run;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int64_t c = 0; c < nch; ++c) { run = __dadd_rn(run, csum[c]); csum[c] = run; }
    const double u = iq_draw_uniform(a.seed, a.tile, a.real0 + r);
    const double t = __dmul_rn(u, run);
    int64_t c = 0;
    while (c < nch - 1 && csum[c] < t) ++c;
    const double base = c == 0 ? 0.0 : csum[c - 1];
    const int64_t lo = c * IQ_DRAW_CHUNK, hi = min(n, lo + IQ_DRAW_CHUNK);
    double part = 0.0;
    int64_t pick = hi - 1;
    for (int64_t i = lo; i < hi; ++i) {
      part = __dadd_rn(part, w[i]);
      if (__dadd_rn(base, part) >= t) { pick = i; break; }
    }
    a.rind[r] = cand[pick];
  }
}

}  // namespace

int iq_launch_pick(iq_ctx* ctx, const PickLaunch& L) {
  if (L.naux > IQ_MAX_AUX) return iq_set_error(IQ_ERR_LIMIT, "too many auxiliary sources");
  PickArgs a;
  a.P = L.P; a.npat = L.npat; a.tol = L.tol; a.seed = L.seed; a.tile = L.tile;
  a.real0 = L.real0;
  a.D0 = L.D0; a.D0_rs = L.D0_rstride; a.mm0 = L.mm0; a.mm0_rs = L.mm0_rstride;
  a.naux = L.naux;
  for (int j = 0; j < IQ_MAX_AUX; ++j) { a.aux[j] = L.aux[j]; a.aux_rs[j] = L.aux_rstride[j]; }
  a.dbsize_norm = L.dbsize_norm; a.dbsize_zero = L.dbsize_zero;
  a.nseq_norm = L.nseq_norm; a.nseq_zero = L.nseq_zero;
  for (int q = 0; q < IQ_MAX_SEQ; ++q) { a.seq_norm[q] = L.seq_norm[q]; a.seq_zero[q] = L.seq_zero[q]; }
  a.cand = L.cand; a.k0 = L.k0; a.v0 = L.v0; a.k1 = L.k1; a.v1 = L.v1;
  a.w = L.w; a.prod = L.prod; a.rind = L.rind; a.ncand = L.ncand; a.status = L.status;
  a.stats = L.stats;
  iq_timer_start(ctx, "pick");
  pick_kernel<<<L.nreal, PT, 0, ctx->stream>>>(a);
  iq_timer_stop(ctx, "pick", 4.0 * (double)L.P * (double)(1 + L.naux) * (double)L.nreal);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
