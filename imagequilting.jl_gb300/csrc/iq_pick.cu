// Pattern pick of one tile for a batch of realizations: one 1024-thread CTA per realization.
//
//   threshold pick  findall(D .<= (1 + tol) * minimum(D))           src/iqsim.jl:237
//   relaxation      top-dbsize of D intersected with growing top-s    src/relaxation.jl:5-39
//                   sets of each auxiliary distance
//   tau model       dense ranks per source, P = (n - r + 1)/sum,     src/taumodel.jl:5-45
//                   x = x0 * prod((1 - P)/P / x0), p = 1/(1 + x)
//   draw            t = u * sum(p), first i with cumsum(p)[i] >= t   src/iqsim.jl:243
//
// "Top-k" follows partialsortperm: order by (value, index). The k-th (value, index) key is
// found by a histogram select: non-negative floats order like their bit patterns, so 4096
// bins over [bits(min), bits(max finite)] (the distance kernel supplies both) locate the bin
// that holds the k-th element in one pass over the map; a second pass collects that bin's
// (value, index) keys into shared memory and a bitonic sort gives the exact key. Bins too
// large to collect are narrowed by another histogram; a bin of one repeated value falls back
// to a radix select over the indices. The primary and one auxiliary source share passes.
// Candidate lists are compacted in ascending index order; dense ranks come from a
// shared-memory bitonic sort (a stable LSD radix sort in global memory above 8192
// candidates). All Float64 arithmetic uses explicit round-to-nearest intrinsics so that the
// weights equal the oracle's bit for bit; the draw sums in the fixed order of
// oracle/iqsim_oracle.sample_index.
#include "iq_internal.h"

namespace {

constexpr int PT = 1024;
constexpr int NW = PT / 32;
constexpr int NBIN = 4096;       // histogram bins per source
constexpr int SORT_CAP = 8192;   // 64-bit keys sorted in shared memory
constexpr int CITEMS = 8;        // positions per thread per compaction tile

struct PickArgs {
  int64_t P, npat;
  double tol;
  uint64_t seed;
  int64_t real0;
  int nreal;
  PickTask t0;
  const PickTask* tasks;
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

// small shared state (static); the large regions are dynamic shared memory:
//   hist : 2 x NBIN uint32 (32 KB)          histograms of up to two sources
//   sbuf : SORT_CAP uint64 (64 KB)          sort buffer; also the radix sort's per-warp
//                                           digit counters (NW x 256 uint32)
constexpr size_t DYN_BYTES = 2 * NBIN * 4 + SORT_CAP * 8;

struct Smem {
  uint32_t hist[256];
  uint32_t base[256];
  uint32_t warp[NW];
  unsigned long long wred[NW];
  uint32_t sel, cnt;
  int64_t kk;
  int flag;
  uint32_t ncol;
  int64_t bin[2], below[2], bcnt[2];
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
    s.warp[lane] = u - t;
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

// ---- per-warp 256-bin histograms (radix select over indices, radix sort) -----------------
__device__ __forceinline__ void whist_zero(uint32_t* wcnt) {
  for (int i = threadIdx.x; i < NW * 256; i += PT) wcnt[i] = 0;
  __syncthreads();
}

__device__ __forceinline__ void whist_add(uint32_t* wcnt, bool valid, uint32_t d) {
  const int lane = threadIdx.x & 31;
  uint32_t key = valid ? d : (0x10000u + lane);
  uint32_t peers = __match_any_sync(0xffffffffu, key);
  if (valid && lane == __ffs(peers) - 1)
    atomicAdd(&wcnt[(threadIdx.x >> 5) * 256 + d], (uint32_t)__popc(peers));
}

__device__ __forceinline__ void whist_reduce(Smem& s, const uint32_t* wcnt) {
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += PT) {
    uint32_t t = 0;
#pragma unroll 8
    for (int w = 0; w < NW; ++w) t += wcnt[w * 256 + d];
    s.hist[d] = t;
  }
  __syncthreads();
}

// Bucket of s.hist holding the kk-th (1-based) element; sets s.sel, s.cnt, s.kk.
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

// Radix select (MSD, 8-bit digits) of the kk-th smallest (value, index) key: the general
// fallback. With `fixed_value` set it only selects among the indices holding that value.
__device__ Key radix_select(Smem& s, uint32_t* wcnt, const float* __restrict__ src, int64_t P,
                            int64_t kk, bool fixed_value, uint32_t value) {
  uint32_t prefix = 0, mask = 0;
  const int64_t iters = (P + PT - 1) / PT;
  uint32_t cnt_eq = 0;
  if (!fixed_value) {
    for (int shift = 24; shift >= 0; shift -= 8) {
      whist_zero(wcnt);
      for (int64_t it = 0; it < iters; ++it) {
        int64_t p = it * PT + threadIdx.x;
        bool valid = p < P;
        uint32_t b = valid ? fbits(src[p]) : 0u;
        valid = valid && (b & mask) == prefix;
        whist_add(wcnt, valid, (b >> shift) & 255u);
      }
      whist_reduce(s, wcnt);
      find_bucket(s, kk);
      prefix |= s.sel << shift;
      mask |= 255u << shift;
      kk = s.kk;
      cnt_eq = s.cnt;
    }
    if (kk >= (int64_t)cnt_eq) return Key{prefix, 0xFFFFFFFFu};
  } else {
    prefix = value;
  }
  int topbit = 0;
  while (topbit < 31 && ((int64_t)1 << (topbit + 1)) <= P - 1) ++topbit;
  uint32_t ip = 0, im = 0;
  for (int shift = (topbit / 8) * 8; shift >= 0; shift -= 8) {
    whist_zero(wcnt);
    for (int64_t it = 0; it < iters; ++it) {
      int64_t p = it * PT + threadIdx.x;
      bool valid = p < P;
      uint32_t b = valid ? fbits(src[p]) : 0u;
      valid = valid && b == prefix && ((uint32_t)p & im) == ip;
      whist_add(wcnt, valid, ((uint32_t)p >> shift) & 255u);
    }
    whist_reduce(s, wcnt);
    find_bucket(s, kk);
    ip |= s.sel << shift;
    im |= 255u << shift;
    kk = s.kk;
  }
  return Key{prefix, ip};
}

// Bitonic sort of buf[0..n) ascending (n rounded up to a power of two, padded with ~0).
__device__ void bitonic_sort(unsigned long long* buf, int n) {
  int n2 = 2;
  while (n2 < n) n2 <<= 1;
  for (int i = n + threadIdx.x; i < n2; i += PT) buf[i] = ~0ull;
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += PT) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = buf[i], b = buf[l];
          const bool asc = (i & k) == 0;
          if ((a > b) == asc) { buf[i] = b; buf[l] = a; }
        }
      }
      __syncthreads();
    }
  }
}

// Histogram select of the k-th smallest (value, index) key of up to two sources at once.
// mn/mx: bits of the smallest value and of the largest finite value of each source.
struct SelReq {
  const float* src;
  uint32_t mn, mx;
  int64_t k;
};

__device__ __forceinline__ int bin_shift(uint32_t mn, uint32_t mx) {
  int sh = 0;
  while (((mx - mn) >> sh) >= (uint32_t)NBIN) ++sh;
  return sh;
}

constexpr int SEL_BATCH = 8;  // loads in flight per thread and source in the select passes

template <int NS>
__device__ void hist_select(Smem& s, uint32_t* hist, unsigned long long* sbuf, SelReq* req,
                            int64_t P, Key* out) {
  uint32_t lo[NS], hi[NS];
  int sh[NS];
  int64_t k[NS];
  bool pend[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    lo[j] = req[j].mn;
    hi[j] = req[j].mx;
    k[j] = req[j].k;
    pend[j] = true;
  }
  const int64_t iters = (P + PT - 1) / PT;
  for (int level = 0; level < 4; ++level) {
    bool any = false;
#pragma unroll
    for (int j = 0; j < NS; ++j) any = any || pend[j];
    if (!any) break;
#pragma unroll
    for (int j = 0; j < NS; ++j) sh[j] = pend[j] ? bin_shift(lo[j], hi[j]) : 0;
    for (int i = threadIdx.x; i < NS * NBIN; i += PT) hist[i] = 0;
    __syncthreads();
    for (int64_t it0 = 0; it0 < iters; it0 += SEL_BATCH) {
      // SEL_BATCH independent loads per source before the atomics (memory-level parallelism)
      uint32_t bv[NS][SEL_BATCH];
#pragma unroll
      for (int u = 0; u < SEL_BATCH; ++u) {
        const int64_t p = (it0 + u) * PT + threadIdx.x;
#pragma unroll
        for (int j = 0; j < NS; ++j)
          bv[j][u] = (p < P && pend[j]) ? fbits(req[j].src[p]) : 0xFFFFFFFFu;
      }
#pragma unroll
      for (int u = 0; u < SEL_BATCH; ++u)
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          const uint32_t b = bv[j][u];
          if (b >= lo[j] && b <= hi[j]) atomicAdd(&hist[j * NBIN + ((b - lo[j]) >> sh[j])], 1u);
        }
    }
    __syncthreads();
    // locate the bin of each pending source: warp j scans source j's 4096 bins
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (wid < NS && pend[wid]) {
      const int j = wid;
      uint32_t sum = 0;
      for (int i = 0; i < NBIN / 32; ++i) sum += hist[j * NBIN + lane * (NBIN / 32) + i];
      uint32_t inc = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      const uint32_t exc = inc - sum;
      const bool here = (int64_t)exc < k[j] && (int64_t)inc >= k[j];
      const uint32_t bal = __ballot_sync(0xffffffffu, here);
      if (bal == 0) {
        if (lane == 0) { s.bin[j] = -1; s.below[j] = 0; s.bcnt[j] = 0; }
      } else if (lane == __ffs(bal) - 1) {
        int64_t below = exc;
        int b = lane * (NBIN / 32);
        for (;; ++b) {
          const uint32_t c = hist[j * NBIN + b];
          if (below + c >= k[j]) break;
          below += c;
        }
        s.bin[j] = b;
        s.below[j] = below;
        s.bcnt[j] = hist[j * NBIN + b];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      if (!pend[j]) continue;
      const int64_t b = s.bin[j];
      const int64_t below = s.below[j];
      const int64_t cntb = s.bcnt[j];
      __syncthreads();
      if (b < 0) {  // k-th element lies above the largest finite value: general fallback
        out[j] = radix_select(s, reinterpret_cast<uint32_t*>(sbuf), req[j].src, P, req[j].k,
                              false, 0);
        pend[j] = false;
        continue;
      }
      const uint32_t blo = lo[j] + ((uint32_t)b << sh[j]);
      const uint32_t span = sh[j] >= 32 ? 0xFFFFFFFFu : ((1u << sh[j]) - 1u);
      const uint32_t bhi = (hi[j] - blo) < span ? hi[j] : blo + span;
      const int64_t kb = k[j] - below;
      if (cntb <= SORT_CAP) {
        // collect the bin's (value, index) keys and sort them
        if (threadIdx.x == 0) s.ncol = 0;
        __syncthreads();
        for (int64_t it0 = 0; it0 < iters; it0 += SEL_BATCH) {
          uint32_t vv[SEL_BATCH];
#pragma unroll
          for (int u = 0; u < SEL_BATCH; ++u) {
            const int64_t p = (it0 + u) * PT + threadIdx.x;
            vv[u] = p < P ? fbits(req[j].src[p]) : 0xFFFFFFFFu;
          }
#pragma unroll
          for (int u = 0; u < SEL_BATCH; ++u) {
            const uint32_t v = vv[u];
            if (v >= blo && v <= bhi) {
              const uint32_t at = atomicAdd(&s.ncol, 1u);
              sbuf[at] = ((unsigned long long)v << 32) | (uint32_t)((it0 + u) * PT + threadIdx.x);
            }
          }
        }
        __syncthreads();
        const int nc = (int)s.ncol;
        bitonic_sort(sbuf, nc);
        const unsigned long long key = sbuf[kb - 1];
        out[j] = Key{(uint32_t)(key >> 32), (uint32_t)key};
        __syncthreads();
        pend[j] = false;
      } else if (sh[j] == 0) {
        // one value repeated more than SORT_CAP times: select among its indices
        out[j] = radix_select(s, reinterpret_cast<uint32_t*>(sbuf), req[j].src, P, kb, true, blo);
        pend[j] = false;
      } else {
        lo[j] = blo;
        hi[j] = bhi;
        k[j] = kb;
      }
    }
  }
}

// Ordered compaction of {p : pred(p)} into out (if non-null); returns the count.
template <typename Pred>
__device__ int64_t compact(Smem& s, const Pred& pred, int64_t P, int32_t* out) {
  int64_t base = 0;
  const int64_t tile = (int64_t)PT * CITEMS;
  for (int64_t t0 = 0; t0 < P; t0 += tile) {
    const int64_t p0 = t0 + (int64_t)threadIdx.x * CITEMS;
    const uint32_t bits = pred.eval8(p0, P);
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

struct ThrPred {
  const float* D; double thr;
  // bit i set when D[p0 + i] <= thr (positions past P excluded)
  __device__ uint32_t eval8(int64_t p0, int64_t P) const {
    float v[CITEMS];
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) v[i] = p0 + i < P ? D[p0 + i] : __int_as_float(0x7F800000);
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i)
      if (p0 + i < P && (double)v[i] <= thr) bits |= 1u << i;
    return bits;
  }
};

template <int NAUX>
struct RelaxPred {
  const float* D; Key kD;
  int naux;  // <= NAUX
  const float* aux[NAUX > 0 ? NAUX : 1];
  Key ka[NAUX > 0 ? NAUX : 1];
  // bit i set when position p0 + i is in the top set of D and of every auxiliary source
  __device__ uint32_t eval8(int64_t p0, int64_t P) const {
    uint32_t b[CITEMS];
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) b[i] = p0 + i < P ? fbits(D[p0 + i]) : 0xFFFFFFFFu;
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i)
      if (p0 + i < P && key_le(b[i], (uint32_t)(p0 + i), kD)) bits |= 1u << i;
#pragma unroll
    for (int a = 0; a < NAUX; ++a) {
      if (a >= naux || !bits) continue;
      uint32_t c[CITEMS];
#pragma unroll
      for (int i = 0; i < CITEMS; ++i) c[i] = (bits >> i & 1u) ? fbits(aux[a][p0 + i]) : 0u;
#pragma unroll
      for (int i = 0; i < CITEMS; ++i)
        if ((bits >> i & 1u) && !key_le(c[i], (uint32_t)(p0 + i), ka[a])) bits &= ~(1u << i);
    }
    return bits;
  }
};

// Stable LSD radix sort of (keys, vals)[0..n) between the buffer pairs (global memory);
// returns 0 if the result is in (ka, va), 1 if in (kb, vb).
__device__ int radix_sort(Smem& s, uint32_t* wcnt, uint32_t* ka, uint32_t* va, uint32_t* kb,
                          uint32_t* vb, int64_t n) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int cur = 0;
  const int64_t ntiles = (n + PT - 1) / PT;
  for (int shift = 0; shift < 32; shift += 8) {
    uint32_t* ks = cur ? kb : ka; uint32_t* vs = cur ? vb : va;
    uint32_t* kd = cur ? ka : kb; uint32_t* vd = cur ? va : vb;
    whist_zero(wcnt);
    for (int64_t t = 0; t < ntiles; ++t) {
      int64_t i = t * PT + threadIdx.x;
      bool valid = i < n;
      uint32_t d = valid ? (ks[i] >> shift) & 255u : 0u;
      whist_add(wcnt, valid, d);
    }
    whist_reduce(s, wcnt);
    int single = 0;
    if (threadIdx.x < 256 && (int64_t)s.hist[threadIdx.x] == n) single = 1;
    if (__syncthreads_or(single)) continue;
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      for (int d = 0; d < 256; ++d) { s.base[d] = run; run += s.hist[d]; }
    }
    __syncthreads();
    for (int64_t t = 0; t < ntiles; ++t) {
      for (int i = threadIdx.x; i < NW * 256; i += PT) wcnt[i] = 0;
      __syncthreads();
      int64_t i = t * PT + threadIdx.x;
      bool valid = i < n;
      uint32_t k = valid ? ks[i] : 0u, v = valid ? vs[i] : 0u;
      uint32_t d = (k >> shift) & 255u;
      uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : (0x10000u + lane));
      uint32_t rank = __popc(peers & lanemask_lt());
      if (valid && lane == __ffs(peers) - 1) wcnt[wid * 256 + d] = __popc(peers);
      __syncthreads();
      if (threadIdx.x < 256) {
        uint32_t run = s.base[threadIdx.x];
        for (int w = 0; w < NW; ++w) {
          uint32_t c = wcnt[w * 256 + threadIdx.x];
          wcnt[w * 256 + threadIdx.x] = run;
          run += c;
        }
        s.base[threadIdx.x] = run;
      }
      __syncthreads();
      if (valid) {
        uint32_t dst = wcnt[wid * 256 + d] + rank;
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
// (n - rank + 1) over i. `rank` must not alias k0/v0/k1/v1.
__device__ unsigned long long dense_ranks(Smem& s, unsigned long long* sbuf,
                                          const float* __restrict__ src,
                                          const int32_t* __restrict__ cand, int64_t n,
                                          uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1,
                                          uint32_t* rank) {
  unsigned mn = 0xFFFFFFFFu, mx = 0u;
  const bool small = n <= SORT_CAP;
  for (int64_t i = threadIdx.x; i < n; i += PT) {
    const uint32_t b = fbits(src[cand[i]]);
    if (small) {
      sbuf[i] = ((unsigned long long)b << 32) | (uint32_t)i;
    } else {
      k0[i] = b;
      v0[i] = (uint32_t)i;
    }
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
    for (int64_t i = threadIdx.x; i < n; i += PT) rank[i] = 1u;
    __syncthreads();
    return (unsigned long long)n * (unsigned long long)n;  // each term n - 1 + 1
  }
  const uint32_t* ks = nullptr;
  const uint32_t* vs = nullptr;
  if (small) {
    bitonic_sort(sbuf, (int)n);
  } else {
    int where = radix_sort(s, reinterpret_cast<uint32_t*>(sbuf), k0, v0, k1, v1, n);
    ks = where ? k1 : k0;
    vs = where ? v1 : v0;
  }
  uint32_t carry = 0;
  unsigned long long acc = 0;
  for (int64_t t0 = 0; t0 < n; t0 += PT) {
    const int64_t i = t0 + threadIdx.x;
    uint32_t f = 0, idx = 0;
    if (i < n) {
      uint32_t cur, prev = 0;
      if (small) {
        cur = (uint32_t)(sbuf[i] >> 32);
        if (i) prev = (uint32_t)(sbuf[i - 1] >> 32);
        idx = (uint32_t)sbuf[i];
      } else {
        cur = ks[i];
        if (i) prev = ks[i - 1];
        idx = vs[i];
      }
      f = (i == 0 || cur != prev) ? 1u : 0u;
    }
    uint32_t total;
    const uint32_t ex = block_excl_sum(s, f, total);
    if (i < n) {
      const uint32_t r = carry + ex + f;
      rank[idx] = r;
      acc += (unsigned long long)(n - r + 1);
    }
    carry += total;
  }
  __syncthreads();
  return block_sum_u64(s, acc);
}

// One CTA per (task, realization): CTA b picks for realization b % nreal of task b / nreal.
// NAUX is the largest number of auxiliary sources of the launch's tasks.
template <int NAUX>
__global__ void __launch_bounds__(PT) pick_kernel(const PickArgs a) {
  __shared__ Smem s;
  extern __shared__ __align__(16) unsigned char dyn[];
  uint32_t* hist = reinterpret_cast<uint32_t*>(dyn);
  unsigned long long* sbuf = reinterpret_cast<unsigned long long*>(dyn + 2 * NBIN * 4);
  const int b = blockIdx.x;
  const int r = b % a.nreal;
  const PickTask& tk = a.tasks ? a.tasks[b / a.nreal] : a.t0;
  const int64_t P = a.P;
  const float* D = tk.D0 + r * tk.D0_rs;
  const unsigned* mm = tk.mm0 + r * tk.mm0_rs;
  const int naux = tk.naux < NAUX ? tk.naux : NAUX;
  int32_t* cand = a.cand + b * P;
  uint32_t* k0 = a.k0 + b * P;
  uint32_t* v0 = a.v0 + b * P;
  uint32_t* k1 = a.k1 + b * P;
  uint32_t* v1 = a.v1 + b * P;
  double* w = a.w + b * P;
  double* prod = a.prod + b * P;
  uint32_t* rankbuf = reinterpret_cast<uint32_t*>(w);  // ranks live in w until weights are made
  const float* aux[NAUX > 0 ? NAUX : 1];
  const unsigned* amm[NAUX > 0 ? NAUX : 1];
#pragma unroll
  for (int j = 0; j < NAUX; ++j) {
    aux[j] = j < naux ? tk.aux[j] + r * tk.aux_rs[j] : nullptr;
    amm[j] = j < naux ? tk.aux_mm[j] + r * tk.aux_mm_rs[j] : nullptr;
  }

  const bool prof = a.stats != nullptr && threadIdx.x == 0;
  const long long t0 = prof ? clock64() : 0;
  int64_t n;
  if (naux == 0) {
    const float mn = __uint_as_float(mm[0]);
    const double thr = __dmul_rn(__dadd_rn(1.0, a.tol), (double)mn);
    ThrPred pr{D, thr};
    n = compact(s, pr, P, cand);
  } else {
    if (a.npat <= 0) {
      if (threadIdx.x == 0) { iq_dev_fail(a.status, IQ_ERR_NOPATTERN); a.rind[b] = -1; }
      return;
    }
    const bool allzero = mm[1] == 0u;
    const int64_t dbsize = allzero ? a.dbsize_zero : a.dbsize_norm;
    const int nseq = allzero ? a.nseq_zero : a.nseq_norm;
    RelaxPred<NAUX> pr;
    pr.D = D;
    pr.naux = naux;
#pragma unroll
    for (int j = 0; j < NAUX; ++j) { pr.aux[j] = aux[j]; pr.ka[j] = Key{0xFFFFFFFFu, 0xFFFFFFFFu}; }
    n = 0;
    int q = 0;
    for (; q < nseq && n == 0; ++q) {
      const int64_t sz = allzero ? a.seq_zero[q] : a.seq_norm[q];
      // selections of this round: D (first round only) and every auxiliary source
      SelReq req[2];
      Key res[2];
      int j0 = 0;
      if (q == 0) {
        req[0] = SelReq{D, mm[0], mm[1], dbsize};
        const bool pre0 = !allzero && tk.aux_keys[0] && q < tk.nkeys;
        if (NAUX > 0 && naux > 0 && sz > 0 && sz < P && !pre0) {
          req[1] = SelReq{aux[0], amm[0][0], amm[0][1], sz};
          hist_select<2>(s, hist, sbuf, req, P, res);
          pr.ka[0] = res[1];
          j0 = 1;
        } else {
          hist_select<1>(s, hist, sbuf, req, P, res);
        }
        pr.kD = res[0];
      }
#pragma unroll
      for (int j = 0; j < NAUX; ++j) {
        if (j < j0 || j >= naux) continue;
        if (!allzero && tk.aux_keys[j] && q < tk.nkeys) {  // shared source: key precomputed
          const unsigned long long kk = tk.aux_keys[j][q];
          pr.ka[j] = Key{(uint32_t)(kk >> 32), (uint32_t)kk};
          continue;
        }
        if (sz >= P) { pr.ka[j] = Key{0xFFFFFFFFu, 0xFFFFFFFFu}; continue; }
        if (sz <= 0) { pr.ka[j] = Key{0u, 0u}; continue; }
        req[0] = SelReq{aux[j], amm[j][0], amm[j][1], sz};
        hist_select<1>(s, hist, sbuf, req, P, res);
        pr.ka[j] = res[0];
      }
      // the compaction counts: an empty intersection moves on to the next softdbsize
      n = compact(s, pr, P, cand);
    }
    if (a.stats && threadIdx.x == 0) atomicAdd(a.stats + ST_PICK_ITERS, (unsigned long long)q);
  }
  if (n <= 0) {
    if (threadIdx.x == 0) { iq_dev_fail(a.status, IQ_ERR_NOPATTERN); a.rind[b] = -1; }
    return;
  }
  if (a.ncand && threadIdx.x == 0) a.ncand[b] = n;
  if (a.stats && threadIdx.x == 0) {
    atomicAdd(a.stats + ST_PICK_CAND, (unsigned long long)n);
    atomicAdd(a.stats + ST_PICK_CTAS, 1ull);
  }
  const long long t1 = prof ? clock64() : 0;
  if (prof) atomicAdd(a.stats + ST_PICK_TSEL, (unsigned long long)(t1 - t0));

  // ---- tau model weights ----
  if (n == 1) {
    if (threadIdx.x == 0) { w[0] = 1.0; a.rind[b] = cand[0]; }
    return;
  }
  const double dn = (double)n;
  const double inv_n = __ddiv_rn(1.0, dn);
  const double x0 = __ddiv_rn(__dsub_rn(1.0, inv_n), inv_n);
  for (int64_t i = threadIdx.x; i < n; i += PT) prod[i] = 1.0;
#pragma unroll 1
  for (int j = 0; j <= naux; ++j) {
    const float* src = j == 0 ? D : aux[j > 0 ? j - 1 : 0];
    __syncthreads();
    const unsigned long long S = dense_ranks(s, sbuf, src, cand, n, k0, v0, k1, v1, rankbuf);
    const double dS = (double)S;
    for (int64_t i = threadIdx.x; i < n; i += PT) {
      const double Pi = __ddiv_rn((double)(n - (int64_t)rankbuf[i] + 1), dS);
      const double X = __ddiv_rn(__dsub_rn(1.0, Pi), Pi);
      prod[i] = __dmul_rn(prod[i], __ddiv_rn(X, x0));
    }
    __syncthreads();
  }
  for (int64_t i = threadIdx.x; i < n; i += PT)
    w[i] = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(x0, prod[i])));
  __syncthreads();

  const long long t2 = prof ? clock64() : 0;
  if (prof) atomicAdd(a.stats + ST_PICK_TW, (unsigned long long)(t2 - t1));
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
    const double u = iq_draw_uniform(a.seed, tk.tile, a.real0 + r);
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
    a.rind[b] = cand[pick];
    if (prof) atomicAdd(a.stats + ST_PICK_TDRAW, (unsigned long long)(clock64() - t2));
  }
}

// One CTA per (map, sequence step): the key of the k-th smallest (value, index) of the map, as
// the relaxation in pick_kernel computes it (k >= P: everything; k <= 0: nothing).
struct KeyArgs {
  const float* maps;
  const unsigned* mm;
  int64_t P;
  int nq;
  int64_t seq[IQ_PRE_KEYS];
  unsigned long long* keys;
};

__global__ void __launch_bounds__(PT) select_keys_kernel(const KeyArgs a) {
  __shared__ Smem s;
  extern __shared__ __align__(16) unsigned char dyn[];
  uint32_t* hist = reinterpret_cast<uint32_t*>(dyn);
  unsigned long long* sbuf = reinterpret_cast<unsigned long long*>(dyn + 2 * NBIN * 4);
  const int64_t m = blockIdx.x / a.nq;
  const int q = blockIdx.x % a.nq;
  const int64_t k = a.seq[q];
  Key key;
  if (k >= a.P) {
    key = Key{0xFFFFFFFFu, 0xFFFFFFFFu};
  } else if (k <= 0) {
    key = Key{0u, 0u};
  } else {
    SelReq req[1] = {SelReq{a.maps + m * a.P, a.mm[2 * m], a.mm[2 * m + 1], k}};
    Key res[1];
    hist_select<1>(s, hist, sbuf, req, a.P, res);
    key = res[0];
  }
  if (threadIdx.x == 0)
    a.keys[m * a.nq + q] = ((unsigned long long)key.v << 32) | key.i;
}

// The shared-memory attribute belongs to the current device, so it is set on every launch
// (a host call of a few microseconds) rather than once per process.
template <int NAUX>
cudaError_t launch_pick_t(const PickArgs& a, int nblocks, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(pick_kernel<NAUX>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)DYN_BYTES);
  if (e != cudaSuccess) return e;
  pick_kernel<NAUX><<<nblocks, PT, DYN_BYTES, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

int iq_launch_pick(iq_ctx* ctx, const PickLaunch& L) {
  if (L.naux_max > IQ_MAX_AUX || L.t0.naux > IQ_MAX_AUX)
    return iq_set_error(IQ_ERR_LIMIT, "too many auxiliary sources");
  if (L.ntask <= 0 || L.nreal <= 0) return IQ_OK;
  PickArgs a;
  a.P = L.P; a.npat = L.npat; a.tol = L.tol; a.seed = L.seed; a.real0 = L.real0;
  a.nreal = L.nreal;
  a.t0 = L.t0;
  a.tasks = L.tasks;
  a.dbsize_norm = L.dbsize_norm; a.dbsize_zero = L.dbsize_zero;
  a.nseq_norm = L.nseq_norm; a.nseq_zero = L.nseq_zero;
  for (int q = 0; q < IQ_MAX_SEQ; ++q) { a.seq_norm[q] = L.seq_norm[q]; a.seq_zero[q] = L.seq_zero[q]; }
  a.cand = L.cand; a.k0 = L.k0; a.v0 = L.v0; a.k1 = L.k1; a.v1 = L.v1;
  a.w = L.w; a.prod = L.prod; a.rind = L.rind; a.ncand = L.ncand; a.status = L.status;
  a.stats = L.stats;
  const int naux = L.tasks ? L.naux_max : L.t0.naux;
  const int nblocks = L.ntask * L.nreal;
  iq_timer_start(ctx, "pick");
  cudaError_t e;
  switch (naux) {
    case 0: e = launch_pick_t<0>(a, nblocks, ctx->stream); break;
    case 1: e = launch_pick_t<1>(a, nblocks, ctx->stream); break;
    case 2: e = launch_pick_t<2>(a, nblocks, ctx->stream); break;
    case 3: e = launch_pick_t<3>(a, nblocks, ctx->stream); break;
    case 4: e = launch_pick_t<4>(a, nblocks, ctx->stream); break;
    case 5: e = launch_pick_t<5>(a, nblocks, ctx->stream); break;
    case 6: e = launch_pick_t<6>(a, nblocks, ctx->stream); break;
    default: e = launch_pick_t<7>(a, nblocks, ctx->stream); break;
  }
  iq_timer_stop(ctx, "pick", 4.0 * (double)L.P * (double)(1 + naux) * (double)nblocks);
  iq_count(ctx);
  if (e != cudaSuccess) return iq_set_error(IQ_ERR_CUDA, "pick launch: %s", cudaGetErrorString(e));
  return IQ_OK;
}

int iq_launch_select_keys(iq_ctx* ctx, const float* maps, const unsigned* mm, int64_t nmaps,
                          int64_t P, const int64_t* seq, int nq, unsigned long long* keys) {
  if (nmaps <= 0 || nq <= 0) return IQ_OK;
  if (nq > IQ_PRE_KEYS) return iq_set_error(IQ_ERR_ARG, "too many precomputed keys");
  KeyArgs a;
  a.maps = maps; a.mm = mm; a.P = P; a.nq = nq; a.keys = keys;
  for (int q = 0; q < IQ_PRE_KEYS; ++q) a.seq[q] = q < nq ? seq[q] : 0;
  IQ_CUDA_OK(cudaFuncSetAttribute(select_keys_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)DYN_BYTES));
  iq_timer_start(ctx, "pick");
  select_keys_kernel<<<(unsigned)(nmaps * nq), PT, DYN_BYTES, ctx->stream>>>(a);
  iq_timer_stop(ctx, "pick", 0);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
