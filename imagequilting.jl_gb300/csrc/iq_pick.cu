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
  double* rv;
  double* rr;
  uint8_t* rl;
  int64_t dx, dxy;
  int64_t* rind;
  int64_t* ncand;
  int* status;
  unsigned long long* ties;
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
__device__ __noinline__ Key radix_select(Smem& s, uint32_t* wcnt, const float* __restrict__ src, int64_t P,
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

// Bitonic sort of (key, val) pairs by (key, val), n <= 8192 (key/val hold the next power of two).
__device__ void bitonic_sort_kv(unsigned long long* key, uint32_t* val, int n) {
  int n2 = 2;
  while (n2 < n) n2 <<= 1;
  for (int i = n + threadIdx.x; i < n2; i += PT) { key[i] = ~0ull; val[i] = 0xFFFFFFFFu; }
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += PT) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = key[i], b = key[l];
          const uint32_t va = val[i], vb = val[l];
          const bool gt = a > b || (a == b && va > vb);
          if (gt == ((i & k) == 0)) { key[i] = b; key[l] = a; val[i] = vb; val[l] = va; }
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
__device__ __noinline__ void hist_select(Smem& s, uint32_t* hist, unsigned long long* sbuf, SelReq* req,
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

constexpr double TIE_RTOL = 1e-6;                 // relative window of a reported near-tie

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
  const float* D;
  float thr;                          // f_dn of the Float64 threshold
  float tlo, thi;                     // near-ties |D - thr| <= 1e-6 thr (Float64): tlo <= D <= thi
  mutable unsigned long long nt = 0;  // this thread's near-ties
  __device__ ThrPred(const float* d, double t, bool ties) : D(d), thr(f_dn(t)), tlo(1.f), thi(0.f) {
    if (ties && t > 0.0 && t < 1e300) tie_window_f(t, __dmul_rn(TIE_RTOL, t), tlo, thi);
  }
  // bit i set when D[p0 + i] <= thr (positions past P excluded)
  __device__ uint32_t eval8(int64_t p0, int64_t P) const {
    float v[CITEMS];
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) v[i] = p0 + i < P ? D[p0 + i] : __int_as_float(0x7F800000);
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) {
      if (p0 + i < P && v[i] <= thr) bits |= 1u << i;
      if (p0 + i < P && v[i] >= tlo && v[i] <= thi) nt++;
    }
    return bits;
  }
};

// Band of one refined top-k selection: D < lo is in, D > hi is out, positions in between are
// listed (ascending, bit 31 set when in).
struct Band {
  double lo, hi;
  int32_t* list;
  int64_t n;
  float lof, hif;  // f_up(lo), f_dn(hi): the same tests on the FP32 values
};

__device__ __forceinline__ Band make_band(double lo, double hi, int32_t* list, int64_t n) {
  return Band{lo, hi, list, n, f_up(lo), f_dn(hi)};
}

__device__ __forceinline__ bool band_member(const Band& b, int64_t p, float d) {
  if (d < b.lof) return true;
  if (d > b.hif) return false;
  int64_t lo = 0, hi = b.n - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) >> 1;
    const int32_t e = b.list[mid];
    const int64_t q = e & 0x7FFFFFFF;
    if (q == p) return (e & (int32_t)0x80000000) != 0;
    if (q < p) lo = mid + 1; else hi = mid - 1;
  }
  return false;  // not reached for a position inside the band
}

template <int NAUX>
struct RelaxPred {
  const float* D; Key kD;
  const Band* bD;  // refined selection of D (nullable: the key decides)
  int naux;  // <= NAUX
  const float* aux[NAUX > 0 ? NAUX : 1];
  Key ka[NAUX > 0 ? NAUX : 1];
  const Band* ba[NAUX > 0 ? NAUX : 1];
  // bit i set when position p0 + i is in the top set of D and of every auxiliary source
  __device__ uint32_t eval8(int64_t p0, int64_t P) const {
    uint32_t b[CITEMS];
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) b[i] = p0 + i < P ? fbits(D[p0 + i]) : 0xFFFFFFFFu;
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) {
      if (p0 + i >= P) continue;
      const bool in = bD ? band_member(*bD, p0 + i, __uint_as_float(b[i]))
                         : key_le(b[i], (uint32_t)(p0 + i), kD);
      if (in) bits |= 1u << i;
    }
#pragma unroll
    for (int a = 0; a < NAUX; ++a) {
      if (a >= naux || !bits) continue;
      uint32_t c[CITEMS];
#pragma unroll
      for (int i = 0; i < CITEMS; ++i) c[i] = (bits >> i & 1u) ? fbits(aux[a][p0 + i]) : 0u;
#pragma unroll
      for (int i = 0; i < CITEMS; ++i) {
        if (!(bits >> i & 1u)) continue;
        const bool in = ba[a] ? band_member(*ba[a], p0 + i, __uint_as_float(c[i]))
                              : key_le(c[i], (uint32_t)(p0 + i), ka[a]);
        if (!in) bits &= ~(1u << i);
      }
    }
    return bits;
  }
};

// Stable LSD radix sort of (keys, vals)[0..n) between the buffer pairs (global memory);
// returns 0 if the result is in (ka, va), 1 if in (kb, vb).
__device__ __noinline__ int radix_sort(Smem& s, uint32_t* wcnt, uint32_t* ka, uint32_t* va, uint32_t* kb,
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
__device__ __noinline__ unsigned long long dense_ranks(Smem& s, unsigned long long* sbuf,
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

// =============================================================================================
// Exact re-rank (continuous data)
//
// The FP32 maps of the correlation kernels carry an error |D32 - D| <= kappa (A2 + B2) + eabs
// (cancellation in A2 - 2AB + B2). Decisions of the pick depend only on a few positions near
// their decision value (the threshold, a top-k boundary, the order of candidates for the tau
// model), so those positions are re-evaluated directly, D[p] = sum_k (img[p + k] - tmpl_k)^2 --
// a sum of non-negative terms without cancellation -- at increasing precision until every
// decision is certain:
//   level 1  FP32, 32 lanes each summing every 32nd offset, then a 5-step butterfly:
//            relative error <= (ceil(K/32) + 8) 2^-24
//   level 2  the same in double-float (pairs of FP32 numbers, error-free sums and products):
//            relative error <= 4.1 (ceil(K/32) + 8) 2^-48
//   level 3  the Float64 sequence of the oracle (oracle/direct.c): offsets in column-major
//            order, d = a - b, D = D + d * d, every operation rounded separately
// Each level gives an interval [v - r, v + r] that holds the level-3 value (the radius also
// covers the (K + 2) 2^-53 difference between the level-3 value and the exact sum), so a
// decision taken on disjoint intervals is the decision the Float64 distance would give.
// =============================================================================================
constexpr double RU32 = 5.9604644775390625e-08;  // 2^-24
constexpr double RU64 = 1.1102230246251565e-16;  // 2^-53
constexpr double TINY32 = 1.401298464324817e-45;  // smallest FP32 subnormal

// One map of one realization, as the re-rank reads it.
struct Ref {
  const float* img;
  int64_t isx, isxy;
  const uint32_t* kl;
  int K;
  const float* tm;
  int64_t tgx, tgxy;
  const float* kv;
  double b2, kappa, eabs;
  int64_t dx, dxy;
};

__device__ __forceinline__ bool ref_on(const ExactSrc& s) {
  return s.img != nullptr && s.kappa > 0.0;
}

__device__ Ref make_ref(const ExactSrc& s, int r, int64_t dx, int64_t dxy) {
  Ref f;
  f.img = s.img; f.isx = s.isx; f.isxy = s.isxy;
  f.kl = s.klist; f.K = s.K;
  f.tm = s.tmpl ? s.tmpl + r * s.tmpl_rs : nullptr;
  f.tgx = s.tgx; f.tgxy = s.tgxy;
  f.kv = s.kval;
  f.b2 = s.b2 ? s.b2[r * s.b2_rs] : 0.0;
  f.kappa = s.kappa; f.eabs = s.eabs;
  f.dx = dx; f.dxy = dxy;
  return f;
}

// image index of the window origin of map position p
__device__ __forceinline__ int64_t ref_base(const Ref& f, int64_t p) {
  const int64_t z = p / f.dxy, rem = p - z * f.dxy, y = rem / f.dx, x = rem - y * f.dx;
  return x + f.isx * y + f.isxy * z;
}

__device__ __forceinline__ void ref_term(const Ref& f, int64_t base, int j, float& a, float& b) {
  const uint32_t k = __ldg(f.kl + j);
  const int kx = kx_of(k), ky = ky_of(k), kz = kz_of(k);
  a = __ldg(f.img + base + kx + f.isx * ky + f.isxy * kz);
  b = f.kv ? __ldg(f.kv + j) : __ldg(f.tm + kx + f.tgx * ky + f.tgxy * kz);
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (h, l) += (x, y) in double-float arithmetic; symmetric in its two operands
__device__ __forceinline__ void df_add(float& h, float& l, float x, float y) {
  float s, e;
  two_sum(h, x, s, e);
  e = __fadd_rn(e, __fadd_rn(l, y));
  h = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(h, s));
}

// The terms of one map, staged in the CTA's dynamic shared memory for a batch of evaluations:
// off[j] = image offset of mask offset j from the window origin, tv[j] = its template value.
// (The region is free whenever entries are evaluated: histograms and sorts use it in between.)
constexpr int REF_CACHE = (2 * NBIN * 4 + SORT_CAP * 8) / 8;  // terms that fit: 12288

struct RefCache {
  const int32_t* off;
  const float* tv;
  bool on;
};

__device__ RefCache ref_cache_load(const Ref& f) {
  extern __shared__ __align__(16) unsigned char dyn[];
  int32_t* off = reinterpret_cast<int32_t*>(dyn);
  float* tv = reinterpret_cast<float*>(dyn + 4 * REF_CACHE);
  const bool on = f.K <= REF_CACHE && f.isxy * 1024 < ((int64_t)1 << 31);
  __syncthreads();  // earlier users of the region are done
  if (on) {
    for (int j = threadIdx.x; j < f.K; j += PT) {
      const uint32_t k = __ldg(f.kl + j);
      const int kx = kx_of(k), ky = ky_of(k), kz = kz_of(k);
      off[j] = (int32_t)(kx + f.isx * ky + f.isxy * kz);
      tv[j] = f.kv ? __ldg(f.kv + j) : __ldg(f.tm + kx + f.tgx * ky + f.tgxy * kz);
    }
  }
  __syncthreads();
  return RefCache{off, tv, on};
}

__device__ __forceinline__ void ref_term_c(const Ref& f, const RefCache& c, int64_t base, int j,
                                           float& a, float& b) {
  if (c.on) {
    a = __ldg(f.img + base + c.off[j]);
    b = c.tv[j];
  } else {
    ref_term(f, base, j, a, b);
  }
}

// Warp-collective: value and radius of D[p] at `level` (every lane gets the same result). The
// image is L2-resident and the loop is bound by the latency of its loads, so each lane issues
// four of them before it uses the first (sixteen measured slower on config 2: more registers,
// fewer resident warps).
__device__ __noinline__ void ref_eval(const Ref& f, const RefCache& c, int64_t p, int level,
                                      double& v, double& r) {
  const int lane = threadIdx.x & 31;
  const int64_t base = ref_base(f, p);
  const int nl = (f.K + 31) / 32;
  const double tail = (double)(f.K + 2) * RU64 * 1.02;   // level 3 vs the exact sum
  if (level <= 1) {
    float acc = 0.f;
    int j = lane;
    for (; j + 3 * 32 < f.K; j += 4 * 32) {
      float ta[4], tb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) ref_term_c(f, c, base, j + 32 * u, ta[u], tb[u]);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float d = __fsub_rn(ta[u], tb[u]);
        acc = __fmaf_rn(d, d, acc);
      }
    }
    for (; j < f.K; j += 32) {
      float a, b;
      ref_term_c(f, c, base, j, a, b);
      const float d = __fsub_rn(a, b);
      acc = __fmaf_rn(d, d, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    v = (double)acc;
    r = v * ((double)(nl + 8) * RU32 * 1.02 + tail) + (double)(f.K + 8) * TINY32 * 4.0;
  } else if (level == 2) {
    float h = 0.f, l = 0.f;
    int j = lane;
    for (; j < f.K; j += 128) {
      float ta[4], tb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        ta[u] = 0.f; tb[u] = 0.f;
        if (j + 32 * u < f.K) ref_term_c(f, c, base, j + 32 * u, ta[u], tb[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (j + 32 * u >= f.K) break;
        const float a = ta[u], b = tb[u];
        float dh, dl;
        two_sum(a, -b, dh, dl);                               // a - b = dh + dl exactly
        const float p2 = __fmul_rn(dh, dh);
        const float pe = __fmaf_rn(dh, dh, -p2);              // dh^2 = p2 + pe exactly
        const float q = __fmaf_rn(__fadd_rn(dh, dh), dl, pe);  // + 2 dh dl (dl^2 dropped)
        df_add(h, l, p2, q);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, h, o);
      const float l2 = __shfl_xor_sync(0xffffffffu, l, o);
      df_add(h, l, h2, l2);
    }
    v = (double)h + (double)l;
    r = v * ((double)(nl + 8) * 4.1 * RU32 * RU32 * 1.02 + tail + RU64) +
        (double)(f.K + 8) * TINY32 * 8.0;
  } else {
    // the oracle's sequence: lanes load and square 32 terms at a time, lane 0 adds them in
    // offset order
    double acc = 0.0;
    for (int j0 = 0; j0 < f.K; j0 += 32) {
      double t = 0.0;
      const int j = j0 + lane;
      if (j < f.K) {
        float a, b;
        ref_term_c(f, c, base, j, a, b);
        const double d = __dsub_rn((double)a, (double)b);
        t = __dmul_rn(d, d);
      }
      const int m = min(32, f.K - j0);
      for (int i = 0; i < m; ++i) {
        const double ti = __shfl_sync(0xffffffffu, t, i);
        acc = __dadd_rn(acc, ti);
      }
    }
    v = acc;
    r = 0.0;
  }
}

// Error bound of the map at positions whose distance is at most Dc:
// kappa (A2 + B2) + eabs with A2 <= (|b| + sqrt(Dc))^2 (triangle inequality).
__device__ __forceinline__ double tier0_bound(const Ref& f, double Dc) {
  const double sb = sqrt(fmax(f.b2, 0.0)), sd = sqrt(fmax(Dc, 0.0));
  return (f.kappa * ((sb + sd) * (sb + sd) + f.b2) + f.eabs) * 1.001 + 1e-300;
}

// Per-entry state of a refinement list, P entries per CTA.
struct RefArr {
  double* v;
  double* r;
  uint8_t* l;     // level (low 7 bits), 0x80 = to be raised
  uint8_t* link;  // 1 where sorted positions t and t + 1 were re-evaluated together
  unsigned* ev;   // shared-memory counts of evaluations per level [4] (nullable)
};

// Level 1 for entries [0, n) of pos (warp per entry).
__device__ __noinline__ void ref_init(const Ref& f, const int32_t* pos, int64_t n, RefArr a) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const RefCache c = ref_cache_load(f);
  for (int64_t i = warp; i < n; i += NW) {
    double v, r;
    ref_eval(f, c, pos[i] & 0x7FFFFFFF, 1, v, r);
    if (lane == 0) {
      a.v[i] = v; a.r[i] = r; a.l[i] = 1;
      if (a.ev) atomicAdd(a.ev + 1, 1u);
    }
  }
  __syncthreads();
}

// Raise every marked entry by one level, or to level 3 when `to3`.
__device__ __noinline__ void ref_raise(const Ref& f, const int32_t* pos, int64_t n, RefArr a, bool to3) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const RefCache c = ref_cache_load(f);
  for (int64_t i = warp; i < n; i += NW) {
    const uint8_t l = a.l[i];
    if (!(l & 0x80)) continue;
    const int nl = to3 ? 3 : min((l & 0x7F) + 1, 3);
    double v, r;
    ref_eval(f, c, pos[i] & 0x7FFFFFFF, nl, v, r);
    if (lane == 0) {
      a.v[i] = v; a.r[i] = r; a.l[i] = (uint8_t)nl;
      if (a.ev) atomicAdd(a.ev + nl, 1u);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ bool ref_exact(const RefArr& a, uint32_t i) { return (a.l[i] & 0x7F) == 3; }
__device__ __forceinline__ void ref_mark(RefArr& a, uint32_t i) {
  if ((a.l[i] & 0x7F) < 3) a.l[i] = (uint8_t)(a.l[i] | 0x80);  // racing writers store one value
}

// (value, position) order of entries i and j
__device__ __forceinline__ bool ref_less(const RefArr& a, const int32_t* pos, uint32_t i, uint32_t j) {
  const double vi = a.v[i], vj = a.v[j];
  return vi < vj || (vi == vj && (pos[i] & 0x7FFFFFFF) < (pos[j] & 0x7FFFFFFF));
}

// Sort entries [0, n) by (level-1 value, ordinal) into ord[0, n) (ordinals; ordinal order is
// position order): a bitonic sort in shared memory up to SORT_CAP, else the radix sort.
__device__ const uint32_t* ref_sort(Smem& s, unsigned long long* sbuf, int64_t n, RefArr a,
                                    uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1) {
  if (n <= SORT_CAP) {
    for (int64_t i = threadIdx.x; i < n; i += PT)
      sbuf[i] = ((unsigned long long)__float_as_uint((float)a.v[i]) << 32) | (uint32_t)i;
    __syncthreads();
    bitonic_sort(sbuf, (int)n);
    for (int64_t i = threadIdx.x; i < n; i += PT) v0[i] = (uint32_t)sbuf[i];
    __syncthreads();
    return v0;
  }
  for (int64_t i = threadIdx.x; i < n; i += PT) {
    k0[i] = __float_as_uint((float)a.v[i]);
    v0[i] = (uint32_t)i;
  }
  __syncthreads();
  const int where = radix_sort(s, reinterpret_cast<uint32_t*>(sbuf), k0, v0, k1, v1, n);
  return where ? v1 : v0;
}

// Make the order ord[0, n) exact: while two neighbours' intervals overlap (and are not both
// exact), raise both and re-sort the runs of raised neighbours by (value, position). At the
// end every adjacent pair is disjoint or both exact, so the order is the order of the Float64
// distances with ties broken by position.
__device__ __noinline__ void ref_resolve(Smem& s, const Ref& f, const int32_t* pos, int64_t n, uint32_t* ord,
                            RefArr a) {
  for (int round = 0; round < 64; ++round) {
    int any = 0;
    for (int64_t t = threadIdx.x; t < n; t += PT) a.link[t] = 0;
    __syncthreads();
    for (int64_t t = threadIdx.x; t + 1 < n; t += PT) {
      const uint32_t i = ord[t], j = ord[t + 1];
      if (ref_exact(a, i) && ref_exact(a, j)) continue;
      if (a.v[i] + a.r[i] >= a.v[j] - a.r[j]) {
        a.link[t] = 1;
        any = 1;
      }
    }
    if (!__syncthreads_or(any)) break;
    for (int64_t t = threadIdx.x; t + 1 < n; t += PT)
      if (a.link[t]) { ref_mark(a, ord[t]); ref_mark(a, ord[t + 1]); }
    __syncthreads();
    ref_raise(f, pos, n, a, round >= 3);
    if (n <= SORT_CAP) {
      // the whole order by (Float64 value, entry) in shared memory (values are >= 0, so their
      // bits order like the values)
      extern __shared__ __align__(16) unsigned char dyn[];
      uint32_t* val = reinterpret_cast<uint32_t*>(dyn);
      unsigned long long* key = reinterpret_cast<unsigned long long*>(dyn + 2 * NBIN * 4);
      for (int64_t t = threadIdx.x; t < n; t += PT) {
        const uint32_t i = ord[t];
        key[t] = (unsigned long long)__double_as_longlong(a.v[i]);
        val[t] = i;
      }
      __syncthreads();
      bitonic_sort_kv(key, val, (int)n);
      for (int64_t t = threadIdx.x; t < n; t += PT) ord[t] = val[t];
      __syncthreads();
      continue;
    }
    // runs of linked neighbours [t, e]: insertion sort by (value, position)
    for (int64_t t = threadIdx.x; t + 1 < n; t += PT) {
      if (!a.link[t] || (t > 0 && a.link[t - 1])) continue;
      int64_t e = t + 1;
      while (e + 1 < n && a.link[e]) ++e;
      for (int64_t x = t + 1; x <= e; ++x) {
        const uint32_t key = ord[x];
        int64_t y = x - 1;
        while (y >= t && ref_less(a, pos, key, ord[y])) {
          ord[y + 1] = ord[y];
          --y;
        }
        ord[y + 1] = key;
      }
    }
    __syncthreads();
  }
}

// Near-tie test |D - t| <= 1e-6 t (evaluated as the oracle does, in Float64) of entry i against
// the value t of entry b: 1 yes, 0 no, -1 undecided on the current intervals.
__device__ __forceinline__ int ref_tie(const RefArr& a, uint32_t i, double tv, double tr, bool texact) {
  const double vi = a.v[i], ri = a.r[i];
  if (ref_exact(a, i) && texact)
    return fabs(__dsub_rn(vi, tv)) <= __dmul_rn(TIE_RTOL, tv) ? 1 : 0;
  const double far = fmax(fabs(vi + ri - (tv - tr)), fabs(vi - ri - (tv + tr)));
  const double near = fmax(0.0, fmax((vi - ri) - (tv + tr), (tv - tr) - (vi + ri)));
  const double wlo = TIE_RTOL * (tv - tr), whi = TIE_RTOL * (tv + tr);
  if (far <= wlo * (1.0 - 1e-9)) return 1;
  if (near > whi * (1.0 + 1e-9)) return 0;
  return -1;
}

// Near-ties among entries [0, n) against the value of entry b (b itself excluded when
// skip_b): raises undecided entries (and b) until every test is decided.
__device__ __noinline__ unsigned long long ref_count_ties(Smem& s, const Ref& f, const int32_t* pos, int64_t n,
                                             RefArr a, int64_t b, bool skip_b, double tfix) {
  for (int round = 0; round < 8; ++round) {
    double tv, tr;
    bool tex;
    if (b >= 0) { tv = a.v[b]; tr = a.r[b]; tex = ref_exact(a, (uint32_t)b); }
    else { tv = tfix; tr = 0.0; tex = true; }
    if (tex && !(tv > 0.0 && tv < 1e300)) return 0;  // no relative window around 0 or Inf
    if (!tex && tv - tr <= 0.0) {  // the decision value may be 0: make it exact first
      if (threadIdx.x == 0) ref_mark(a, (uint32_t)b);
      __syncthreads();
      ref_raise(f, pos, n, a, true);
      continue;
    }
    unsigned long long cnt = 0;
    int und = 0;
    for (int64_t i = threadIdx.x; i < n; i += PT) {
      if (skip_b && i == b) continue;
      const int t = ref_tie(a, (uint32_t)i, tv, tr, tex);
      if (t > 0) cnt++;
      if (t < 0) { und = 1; ref_mark(a, (uint32_t)i); }
    }
    if (und && b >= 0 && threadIdx.x == 0) ref_mark(a, (uint32_t)b);
    if (!__syncthreads_or(und)) return block_sum_u64(s, cnt);
    ref_raise(f, pos, n, a, round >= 2);
  }
  return 0;  // not reached: level-3 tests always decide
}

__device__ double block_min_f64(Smem& s, double v) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  double* red = reinterpret_cast<double*>(s.wred);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int i = 1; i < NW; ++i) m = fmin(m, red[i]);
    red[0] = m;
  }
  __syncthreads();
  const double m = red[0];
  __syncthreads();
  return m;
}

__device__ double block_max_f64(Smem& s, double v) { return -block_min_f64(s, -v); }

__device__ unsigned long long block_max_u64(Smem& s, unsigned long long v) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = v > w ? v : w;
  }
  if (lane == 0) s.wred[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = s.wred[0];
    for (int i = 1; i < NW; ++i) m = m > s.wred[i] ? m : s.wred[i];
    s.wred[0] = m;
  }
  __syncthreads();
  const unsigned long long m = s.wred[0];
  __syncthreads();
  return m;
}

// Ordered compaction of the positions of `src` with lo <= D <= hi into out; `below` receives
// the count of positions with D < lo (Inf and NaN are neither).
__device__ __noinline__ int64_t band_collect(Smem& s, const float* __restrict__ src, int64_t P, double lo,
                                double hi, int32_t* out, int64_t& below) {
  int64_t base = 0;
  unsigned long long nb = 0;
  const int64_t tile = (int64_t)PT * CITEMS;
  const float lof = f_up(lo), hif = f_dn(hi);
  for (int64_t t0 = 0; t0 < P; t0 += tile) {
    const int64_t p0 = t0 + (int64_t)threadIdx.x * CITEMS;
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i) {
      if (p0 + i >= P) continue;
      const float d = src[p0 + i];
      if (d < lof) nb++;
      else if (d <= hif) bits |= 1u << i;
    }
    uint32_t total;
    const uint32_t off = block_excl_sum(s, (uint32_t)__popc(bits), total);
    int64_t o = base + off;
#pragma unroll
    for (int i = 0; i < CITEMS; ++i)
      if (bits >> i & 1u) out[o++] = (int32_t)(p0 + i);
    base += total;
  }
  below = (int64_t)block_sum_u64(s, nb);
  return base;
}

// The exact top-k set of a refined map, given the k-th (value, index) key of its FP32 values:
// fills `b` (list at `list`) and returns the near-ties at the boundary, or -1 when the bound
// failed (the FP32 k-th value lies outside the band: then the key is kept as it is).
__device__ __noinline__ long long band_topk(Smem& s, unsigned long long* sbuf, const Ref& f,
                               const float* __restrict__ src, int64_t P, int64_t k, Key kv,
                               int32_t* list, RefArr a, uint32_t* k0, uint32_t* v0, uint32_t* k1,
                               uint32_t* v1, Band& b) {
  const double v = (double)__uint_as_float(kv.v);
  if (!(v < 1e300)) return -1;  // Inf boundary: the key is exact
  // E0 valid up to Dc = v + 4E, E = E0 plus half the near-tie window
  double E0 = tier0_bound(f, v * 1.001), E = 0.0;
  for (int it = 0; it < 200; ++it) {
    E = E0 + 0.51 * TIE_RTOL * (v + E0);
    const double need = tier0_bound(f, v + 4.0 * E);
    if (need <= E0) break;
    E0 = fmax(need, 1.5 * E0);
  }
  b.lo = v - 2.0 * E;
  b.hi = v + 2.0 * E;
  b.lof = f_up(b.lo);
  b.hif = f_dn(b.hi);
  b.list = list;
  int64_t below = 0;
  b.n = band_collect(s, src, P, b.lo, b.hi, list, below);
  const int64_t kk = k - below;
  if (kk < 1 || kk > b.n) { b.n = 0; return -1; }
  ref_init(f, list, b.n, a);
  uint32_t* ord = const_cast<uint32_t*>(ref_sort(s, sbuf, b.n, a, k0, v0, k1, v1));
  // The set is the first kk entries of the order once every entry on the left lies below every
  // entry on the right: raise only the entries that may cross the split, else (equal values
  // across it) put the whole band in exact (value, position) order.
  bool split = false;
  for (int round = 0; round < 4; ++round) {
    double mh = -1e308, ml = 1e308;
    for (int64_t t = threadIdx.x; t < b.n; t += PT) {
      const uint32_t i = ord[t];
      if (t < kk) mh = fmax(mh, a.v[i] + a.r[i]);
      else ml = fmin(ml, a.v[i] - a.r[i]);
    }
    mh = block_max_f64(s, mh);
    ml = block_min_f64(s, ml);
    if (mh < ml) { split = true; break; }
    int any = 0;
    for (int64_t t = threadIdx.x; t < b.n; t += PT) {
      const uint32_t i = ord[t];
      const bool cross = t < kk ? a.v[i] + a.r[i] >= ml : a.v[i] - a.r[i] <= mh;
      if (cross && !ref_exact(a, i)) { ref_mark(a, i); any = 1; }
    }
    if (!__syncthreads_or(any)) break;
    ref_raise(f, list, b.n, a, round >= 1);
    ord = const_cast<uint32_t*>(ref_sort(s, sbuf, b.n, a, k0, v0, k1, v1));
  }
  if (!split) ref_resolve(s, f, list, b.n, ord, a);
  for (int64_t t = threadIdx.x; t < kk; t += PT) list[ord[t]] |= (int32_t)0x80000000;
  __syncthreads();
  // the boundary: the largest (value, position) of the set
  int64_t bi = split ? -1 : (int64_t)ord[kk - 1];
  for (int round = 0; bi < 0 && round < 8; ++round) {
    double mlo = -1e308;
    for (int64_t t = threadIdx.x; t < kk; t += PT) mlo = fmax(mlo, a.v[ord[t]] - a.r[ord[t]]);
    mlo = block_max_f64(s, mlo);
    unsigned long long cnt = 0, inexact = 0, best = 0;
    for (int64_t t = threadIdx.x; t < kk; t += PT) {
      const uint32_t i = ord[t];
      if (a.v[i] + a.r[i] >= mlo) {
        cnt++;
        if (!ref_exact(a, i)) inexact++;
      }
    }
    cnt = block_sum_u64(s, cnt);
    inexact = block_sum_u64(s, inexact);
    if (cnt == 1 || inexact == 0) {
      // unique candidate, or exact values: the largest (value, position)
      double vmax = -1e308;
      for (int64_t t = threadIdx.x; t < kk; t += PT) {
        const uint32_t i = ord[t];
        if (a.v[i] + a.r[i] >= mlo) vmax = fmax(vmax, a.v[i]);
      }
      vmax = block_max_f64(s, vmax);
      for (int64_t t = threadIdx.x; t < kk; t += PT) {
        const uint32_t i = ord[t];
        if (a.v[i] + a.r[i] >= mlo && (cnt == 1 || a.v[i] == vmax)) {
          const unsigned long long key =
              ((unsigned long long)(uint32_t)(list[i] & 0x7FFFFFFF) << 32) | i;
          best = best > key ? best : key;
        }
      }
      best = block_max_u64(s, best);
      bi = (int64_t)(uint32_t)best;
      break;
    }
    for (int64_t t = threadIdx.x; t < kk; t += PT) {
      const uint32_t i = ord[t];
      if (a.v[i] + a.r[i] >= mlo && !ref_exact(a, i)) ref_mark(a, i);
    }
    __syncthreads();
    ref_raise(f, list, b.n, a, round >= 1);
  }
  if (bi < 0) bi = ord[kk - 1];  // not reached: level-3 values decide within 3 rounds
  __syncthreads();
  return (long long)ref_count_ties(s, f, list, b.n, a, bi, true, 0.0);
}

// Near-ties of an exact map against t (Float64 test of the oracle), counted over all positions.
__device__ __noinline__ unsigned long long count_near(Smem& s, const float* __restrict__ src, int64_t P,
                                         double t) {
  unsigned long long c = 0;
  if (t > 0.0 && t < 1e300) {
    float lo, hi;
    tie_window_f(t, __dmul_rn(TIE_RTOL, t), lo, hi);
    for (int64_t p = threadIdx.x; p < P; p += PT) {
      const float d = src[p];
      if (d >= lo && d <= hi && d < __int_as_float(0x7F800000)) c++;
    }
  }
  return block_sum_u64(s, c);
}

// Dense ranks (1-based) of a refined source over the candidates cand[0, n), written to rank[i];
// returns the sum of (n - rank + 1). Ties of the Float64 distance share a rank.
// `have`: the intervals of the candidates are in `a` already (the refined threshold pick).
__device__ __noinline__ unsigned long long dense_ranks_refined(Smem& s, unsigned long long* sbuf, const Ref& f,
                                                  const int32_t* cand, int64_t n, RefArr a,
                                                  bool have, uint32_t* k0, uint32_t* v0,
                                                  uint32_t* k1, uint32_t* v1, uint32_t* rank) {
  if (!have) ref_init(f, cand, n, a);
  uint32_t* ord = const_cast<uint32_t*>(ref_sort(s, sbuf, n, a, k0, v0, k1, v1));
  ref_resolve(s, f, cand, n, ord, a);
  uint32_t carry = 0;
  unsigned long long acc = 0;
  for (int64_t t0 = 0; t0 < n; t0 += PT) {
    const int64_t t = t0 + threadIdx.x;
    uint32_t fl = 0, idx = 0;
    if (t < n) {
      idx = ord[t];
      if (t == 0) {
        fl = 1;
      } else {
        const uint32_t j = ord[t - 1];
        fl = (ref_exact(a, idx) && ref_exact(a, j) && a.v[idx] == a.v[j]) ? 0u : 1u;
      }
    }
    uint32_t total;
    const uint32_t ex = block_excl_sum(s, fl, total);
    if (t < n) {
      const uint32_t r = carry + ex + fl;
      rank[idx] = r;
      acc += (unsigned long long)(n - r + 1);
    }
    carry += total;
  }
  __syncthreads();
  return block_sum_u64(s, acc);
}

// Keep the entries i of (pos, a) with a.link[i] != 0, in order (in place); returns the count.
__device__ __noinline__ int64_t ref_filter(Smem& s, int32_t* pos, int64_t n, RefArr a) {
  int64_t base = 0;
  for (int64_t t0 = 0; t0 < n; t0 += PT) {
    const int64_t i = t0 + threadIdx.x;
    bool keep = false;
    int32_t pp = 0;
    double v = 0.0, r = 0.0;
    uint8_t l = 0;
    if (i < n && a.link[i]) {
      keep = true;
      pp = pos[i]; v = a.v[i]; r = a.r[i]; l = a.l[i];
    }
    uint32_t total;
    const uint32_t off = block_excl_sum(s, keep ? 1u : 0u, total);
    if (keep) {
      const int64_t o = base + off;
      pos[o] = pp; a.v[o] = v; a.r[o] = r; a.l[o] = l;
    }
    base += total;
    __syncthreads();
  }
  return base;
}

// Threshold pick of a refined map (src/iqsim.jl:237): the candidates D <= (1 + tol) min D of the
// Float64 distance, ascending in cand[0, n), with their intervals in `a`; `ties` receives the
// positions within 1e-6 of the threshold. m32 is the smallest FP32 value (finite).
__device__ __noinline__ int64_t thr_refined(Smem& s, const Ref& f, const float* __restrict__ D, int64_t P,
                               double m32, double tol, int32_t* cand, RefArr a,
                               unsigned long long& ties) {
  // every candidate, the minimum and every near-tie have D32 <= cut
  double E0 = tier0_bound(f, (1.0 + tol) * m32 * 1.01), cut = 0.0;
  for (int it = 0; it < 200; ++it) {
    cut = (1.0 + tol) * (m32 + E0) * (1.0 + 1.01 * TIE_RTOL) + E0;
    const double need = tier0_bound(f, cut + 2.0 * E0);
    if (need <= E0) break;
    E0 = fmax(need, 1.5 * E0);
  }
  int64_t below = 0;
  const int64_t n0 = band_collect(s, D, P, -1.0, cut, cand, below);
  ref_init(f, cand, n0, a);
  // the exact minimum: raise every entry whose interval reaches below the smallest upper bound
  double mhi = 0.0;
  for (int round = 0; round < 8; ++round) {
    double up = 1e308;
    for (int64_t i = threadIdx.x; i < n0; i += PT) up = fmin(up, a.v[i] + a.r[i]);
    mhi = block_min_f64(s, up);
    int any = 0;
    for (int64_t i = threadIdx.x; i < n0; i += PT)
      if (a.v[i] - a.r[i] <= mhi && !ref_exact(a, (uint32_t)i)) { ref_mark(a, (uint32_t)i); any = 1; }
    if (!__syncthreads_or(any)) break;
    ref_raise(f, cand, n0, a, round >= 1);
  }
  double mloc = 1e308;
  for (int64_t i = threadIdx.x; i < n0; i += PT)
    if (a.v[i] - a.r[i] <= mhi) mloc = fmin(mloc, a.v[i]);
  const double mstar = block_min_f64(s, mloc);
  const double thr = __dmul_rn(__dadd_rn(1.0, tol), mstar);
  ties += ref_count_ties(s, f, cand, n0, a, -1, false, thr);
  // membership D <= thr, raising undecided entries
  for (int round = 0; round < 8; ++round) {
    int und = 0;
    for (int64_t i = threadIdx.x; i < n0; i += PT) {
      const double v = a.v[i], r = a.r[i];
      uint8_t in = 0;
      if (ref_exact(a, (uint32_t)i)) in = v <= thr;
      else if (v + r <= thr) in = 1;
      else if (v - r > thr) in = 0;
      else { ref_mark(a, (uint32_t)i); und = 1; }
      a.link[i] = in;
    }
    if (!__syncthreads_or(und)) break;
    ref_raise(f, cand, n0, a, round >= 1);
  }
  return ref_filter(s, cand, n0, a);
}

// Whether every enabled position of a refined map has distance exactly 0 (the relaxation's
// all-zero case, src/relaxation.jl:11): impossible once the largest FP32 value exceeds the
// map's error bound at 0; otherwise every mask value is compared with its window.
__device__ __noinline__ bool all_zero_refined(const Ref& f, const float* __restrict__ D, int64_t P,
                                 unsigned mxbits) {
  if ((double)__uint_as_float(mxbits) > tier0_bound(f, 0.0)) return false;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t step = (int64_t)NW * 8;
  for (int64_t p0 = 0; p0 < P; p0 += step) {
    int bad = 0;
    for (int64_t p = p0 + warp; p < P && p < p0 + step; p += NW) {
      if (!(D[p] < __int_as_float(0x7F800000))) continue;
      const int64_t base = ref_base(f, p);
      int mis = 0;
      for (int j = lane; j < f.K; j += 32) {
        float x, y;
        ref_term(f, base, j, x, y);
        mis |= x != y;
      }
      if (__any_sync(0xffffffffu, mis)) bad = 1;
    }
    if (__syncthreads_or(bad)) return false;
  }
  return true;
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

  // exact re-rank state (used only for maps with kappa > 0)
  RefArr ra;
  ra.v = a.rv ? a.rv + b * P : nullptr;
  ra.r = a.rr ? a.rr + b * P : nullptr;
  ra.l = a.rl ? a.rl + 2 * b * P : nullptr;
  ra.link = a.rl ? a.rl + 2 * b * P + P : nullptr;
  const bool can_ref = a.rv != nullptr;
  __shared__ unsigned evc[4];
  __shared__ long long tband;
  ra.ev = a.stats ? evc : nullptr;
  if (threadIdx.x < 4) evc[threadIdx.x] = 0;
  if (threadIdx.x == 0) tband = 0;
  __syncthreads();
  __shared__ Band sband[1 + (NAUX > 0 ? NAUX : 1)];
  unsigned long long ties = 0;

  const bool prof = a.stats != nullptr && threadIdx.x == 0;
  const long long t0 = prof ? clock64() : 0;
  int64_t n;
  bool have0 = false;  // D's candidate intervals are in ra (refined threshold pick)
  if (naux == 0) {
    const float mn = __uint_as_float(mm[0]);
    if (can_ref && ref_on(tk.x0) && mn < __int_as_float(0x7F800000)) {
      const Ref f0 = make_ref(tk.x0, r, a.dx, a.dxy);
      n = thr_refined(s, f0, D, P, (double)mn, a.tol, cand, ra, ties);
      have0 = true;
    } else {
      const double thr = __dmul_rn(__dadd_rn(1.0, a.tol), (double)mn);
      ThrPred pr(D, thr, true);
      n = compact(s, pr, P, cand);
      ties += block_sum_u64(s, pr.nt);
    }
  } else {
    if (a.npat <= 0) {
      if (threadIdx.x == 0) { iq_dev_fail(a.status, IQ_ERR_NOPATTERN); a.rind[b] = -1; }
      return;
    }
    const bool ref0 = can_ref && ref_on(tk.x0);
    Ref f0;
    if (ref0) f0 = make_ref(tk.x0, r, a.dx, a.dxy);
    const bool allzero = ref0 ? all_zero_refined(f0, D, P, mm[1]) : mm[1] == 0u;
    const int64_t dbsize = allzero ? a.dbsize_zero : a.dbsize_norm;
    const int nseq = allzero ? a.nseq_zero : a.nseq_norm;
    RelaxPred<NAUX> pr;
    pr.D = D;
    pr.bD = nullptr;
    pr.naux = naux;
#pragma unroll
    for (int j = 0; j < NAUX; ++j) {
      pr.aux[j] = aux[j];
      pr.ka[j] = Key{0xFFFFFFFFu, 0xFFFFFFFFu};
      pr.ba[j] = nullptr;
    }
    // band lists of the refined selections live in `prod` (2P int32 entries), free until the
    // tau model
    int32_t* blist = reinterpret_cast<int32_t*>(prod);
    int64_t boff = 0;
    long long tiesD = -1;        // near-ties at D's boundary (refined), -1: count on the map
    long long tiesA[NAUX > 0 ? NAUX : 1];
    n = 0;
    int q = 0;
    for (; q < nseq && n == 0; ++q) {
      const int64_t sz = allzero ? a.seq_zero[q] : a.seq_norm[q];
      // selections of this round: D (first round only) and every auxiliary source
      SelReq req[2];
      Key res[2];
      int j0 = 0;
      // D's selection shared by all realizations of the tile (a hard-data map), precomputed
      const bool preD = q == 0 && !allzero && tk.x0_pb && tk.x0_pb->ok;
      if (preD) {
        const PreBand& pb = *tk.x0_pb;
        pr.kD = Key{(uint32_t)(pb.key >> 32), (uint32_t)pb.key};
        if (pb.ok == 1) {
          if (threadIdx.x == 0)
            sband[0] = make_band(pb.lo, pb.hi, const_cast<int32_t*>(tk.x0_pool) + pb.off, pb.n);
          __syncthreads();
          pr.bD = &sband[0];
          tiesD = pb.ties;
        }
      }
      if (q == 0 && !preD) {
        req[0] = SelReq{D, mm[0], mm[1], dbsize};
        const bool pre0 = !allzero && q < tk.nkeys &&
                          (tk.aux_keys[0] || (tk.aux_pb[0] && tk.aux_pb[0][q].ok == 1));
        if (NAUX > 0 && naux > 0 && sz > 0 && sz < P && !pre0) {
          req[1] = SelReq{aux[0], amm[0][0], amm[0][1], sz};
          hist_select<2>(s, hist, sbuf, req, P, res);
          pr.ka[0] = res[1];
          j0 = 1;
        } else {
          hist_select<1>(s, hist, sbuf, req, P, res);
        }
        pr.kD = res[0];
        if (ref0 && !allzero && dbsize < P) {
          const long long tb0 = prof ? clock64() : 0;
          const long long t = band_topk(s, sbuf, f0, D, P, dbsize, pr.kD, blist, ra, k0, v0, k1,
                                        v1, sband[0]);
          if (prof) tband += clock64() - tb0;
          if (t >= 0) {
            pr.bD = &sband[0];
            boff = sband[0].n;
            tiesD = t;
          }
        }
      }
      int64_t aoff = boff;  // auxiliary bands of this round follow D's band
#pragma unroll
      for (int j = 0; j < NAUX; ++j) {
        if (j >= naux) continue;
        tiesA[j] = -1;
        pr.ba[j] = nullptr;
        if (j >= j0 && !allzero && tk.aux_pb[j] && q < tk.nkeys && tk.aux_pb[j][q].ok == 1) {
          // shared source with an error bound: its refined selection is precomputed
          const PreBand& pb = tk.aux_pb[j][q];
          pr.ka[j] = Key{(uint32_t)(pb.key >> 32), (uint32_t)pb.key};
          if (threadIdx.x == 0)
            sband[1 + j] = make_band(pb.lo, pb.hi, const_cast<int32_t*>(tk.pb_pool) + pb.off, pb.n);
          __syncthreads();
          pr.ba[j] = &sband[1 + j];
          tiesA[j] = pb.ties;
          continue;
        }
        if (j >= j0) {
          if (!allzero && tk.aux_keys[j] && q < tk.nkeys) {  // shared source: key precomputed
            const unsigned long long kk = tk.aux_keys[j][q];
            pr.ka[j] = Key{(uint32_t)(kk >> 32), (uint32_t)kk};
          } else if (sz >= P) {
            pr.ka[j] = Key{0xFFFFFFFFu, 0xFFFFFFFFu};
          } else if (sz <= 0) {
            pr.ka[j] = Key{0u, 0u};
          } else {
            req[0] = SelReq{aux[j], amm[j][0], amm[j][1], sz};
            hist_select<1>(s, hist, sbuf, req, P, res);
            pr.ka[j] = res[0];
          }
        }
        if (can_ref && ref_on(tk.xa[j]) && sz > 0 && sz < P) {
          if (aoff + P > 2 * P) {  // no room for another band: the result would not be exact
            if (threadIdx.x == 0) iq_dev_fail(a.status, IQ_ERR_LIMIT);
            continue;
          }
          const Ref fa = make_ref(tk.xa[j], r, a.dx, a.dxy);
          const long long tb0 = prof ? clock64() : 0;
          const long long t = band_topk(s, sbuf, fa, aux[j], P, sz, pr.ka[j], blist + aoff, ra,
                                        k0, v0, k1, v1, sband[1 + j]);
          if (prof) tband += clock64() - tb0;
          if (t >= 0) {
            pr.ba[j] = &sband[1 + j];
            aoff += sband[1 + j].n;
            tiesA[j] = t;
          }
        }
      }
      // the compaction counts: an empty intersection moves on to the next softdbsize
      n = compact(s, pr, P, cand);
    }
    if (a.stats && threadIdx.x == 0) atomicAdd(a.stats + ST_PICK_ITERS, (unsigned long long)q);
    // near-ties at D's boundary and at each auxiliary boundary of the final round; exact maps
    // are counted on the map (the boundary position itself excluded)
    if (a.ties) {
      if (tiesD >= 0) {
        ties += (unsigned long long)tiesD;
      } else if (!allzero && dbsize < P) {
        const unsigned long long c = count_near(s, D, P, (double)__uint_as_float(pr.kD.v));
        ties += c > 0 ? c - 1 : 0;
      }
      const int64_t szf = q > 0 ? (allzero ? a.seq_zero[q - 1] : a.seq_norm[q - 1]) : 0;
#pragma unroll
      for (int j = 0; j < NAUX; ++j) {
        if (j >= naux || !(szf > 0 && szf < P)) continue;
        if (tiesA[j] >= 0) {
          ties += (unsigned long long)tiesA[j];
        } else {
          const unsigned long long c = count_near(s, aux[j], P, (double)__uint_as_float(pr.ka[j].v));
          ties += c > 0 ? c - 1 : 0;
        }
      }
    }
  }
  if (a.ties && threadIdx.x == 0 && ties) atomicAdd(a.ties, ties);
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
    const ExactSrc& xs = j == 0 ? tk.x0 : tk.xa[j > 0 ? j - 1 : 0];
    __syncthreads();
    unsigned long long S;
    if (can_ref && ref_on(xs)) {
      const Ref f = make_ref(xs, r, a.dx, a.dxy);
      S = dense_ranks_refined(s, sbuf, f, cand, n, ra, j == 0 && have0, k0, v0, k1, v1, rankbuf);
    } else {
      S = dense_ranks(s, sbuf, src, cand, n, k0, v0, k1, v1, rankbuf);
    }
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
  if (prof) {
    atomicAdd(a.stats + ST_PICK_TW, (unsigned long long)(t2 - t1));
    atomicAdd(a.stats + ST_PICK_TBAND, (unsigned long long)tband);
    for (int l = 1; l < 4; ++l) atomicAdd(a.stats + ST_PICK_EV1 + l - 1, (unsigned long long)evc[l]);
  }
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
  a.rv = L.rv; a.rr = L.rr; a.rl = L.rl; a.dx = L.dx; a.dxy = L.dxy;
  a.ties = L.ties;
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

// ---- refined selections of shared maps ---------------------------------------------------------
namespace {

struct BandArgs {
  const float* maps;
  const unsigned* mm;
  const ExactSrc* srcs;
  int64_t m0, nmaps;  // maps [m0, m0 + nmaps) of this launch
  int64_t P, dx, dxy;
  int nq;
  int64_t seq[IQ_PRE_KEYS];
  PreBand* out;
  int32_t* pool;
  int64_t cap;
  int keys_exact;     // exact maps get their key (ok = 2)
  // per-CTA scratch, P entries each
  double* rv;
  double* rr;
  uint8_t* rl;
  int32_t* list;
  uint32_t *k0, *v0, *k1, *v1;
};

// One CTA per (map, step): the key of the step's size, then, for a map with an error bound, the
// band of positions whose order against it is uncertain, resolved exactly (band_topk).
__global__ void __launch_bounds__(PT) select_bands_kernel(const BandArgs a) {
  __shared__ Smem s;
  extern __shared__ __align__(16) unsigned char dyn[];
  uint32_t* hist = reinterpret_cast<uint32_t*>(dyn);
  unsigned long long* sbuf = reinterpret_cast<unsigned long long*>(dyn + 2 * NBIN * 4);
  const int64_t b = blockIdx.x;
  const int64_t m = a.m0 + b / a.nq;
  const int q = (int)(b % a.nq);
  const int64_t k = a.seq[q];
  const int64_t P = a.P;
  PreBand* o = a.out + m * a.nq + q;
  const float* src = a.maps + m * P;
  Key key;
  if (k >= P) key = Key{0xFFFFFFFFu, 0xFFFFFFFFu};
  else if (k <= 0) key = Key{0u, 0u};
  else {
    SelReq req[1] = {SelReq{src, a.mm[2 * m], a.mm[2 * m + 1], k}};
    Key res[1];
    hist_select<1>(s, hist, sbuf, req, P, res);
    key = res[0];
  }
  int ok = 0;
  long long ties = 0;
  Band band{};
  if (k > 0 && k < P && ref_on(a.srcs[m])) {
    const Ref f = make_ref(a.srcs[m], 0, a.dx, a.dxy);
    RefArr ra;
    ra.v = a.rv + b * P;
    ra.r = a.rr + b * P;
    ra.l = a.rl + 2 * b * P;
    ra.link = ra.l + P;
    ra.ev = nullptr;
    int32_t* list = a.list + b * P;
    ties = band_topk(s, sbuf, f, src, P, k, key, list, ra, a.k0 + b * P, a.v0 + b * P,
                     a.k1 + b * P, a.v1 + b * P, band);
    if (ties >= 0 && band.n <= a.cap) {
      ok = 1;
      int32_t* dst = a.pool + (m * a.nq + q) * a.cap;
      for (int64_t i = threadIdx.x; i < band.n; i += PT) dst[i] = list[i];
    }
  }
  if (!ref_on(a.srcs[m]) && a.keys_exact) ok = 2;  // an exact map: its key decides
  if (threadIdx.x == 0) {
    o->lo = band.lo;
    o->hi = band.hi;
    o->off = (m * a.nq + q) * a.cap;
    o->n = band.n;
    o->key = ((unsigned long long)key.v << 32) | key.i;
    o->ties = ok ? ties : 0;
    o->ok = ok;
  }
}

}  // namespace

int iq_launch_select_bands(iq_ctx* ctx, const float* maps, const unsigned* mm,
                           const ExactSrc* srcs, int64_t nmaps, int64_t P, int64_t dx,
                           int64_t dxy, const int64_t* seq, int nq, PreBand* out, int32_t* pool,
                           int64_t cap, int keys_exact) {
  if (nmaps <= 0 || nq <= 0) return IQ_OK;
  if (nq > IQ_PRE_KEYS) return iq_set_error(IQ_ERR_ARG, "too many precomputed selections");
  // per-CTA scratch for a batch of CTAs (38 bytes per position each)
  const int64_t per = P * (8 + 8 + 2 + 4 + 16);
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  const int64_t batch = std::max<int64_t>(1, std::min<int64_t>(nmaps * nq, (int64_t)(freeb / 8) / per));
  // (slots of their own: the caller may hold pointers into the pick's scratch slots)
  double* rv = (double*)iq_scratch(ctx, S_PB_RV, sizeof(double) * P * batch);
  double* rr = (double*)iq_scratch(ctx, S_PB_RR, sizeof(double) * P * batch);
  uint8_t* rl = (uint8_t*)iq_scratch(ctx, S_PB_RL, 2 * P * batch);
  int32_t* list = (int32_t*)iq_scratch(ctx, S_PB_LIST, sizeof(int32_t) * P * batch);
  uint32_t* kk = (uint32_t*)iq_scratch(ctx, S_PB_K, 4 * sizeof(uint32_t) * P * batch);
  if (!rv || !rr || !rl || !list || !kk) return IQ_ERR_ALLOC;
  uint32_t* k0 = kk;
  uint32_t* v0 = kk + P * batch;
  uint32_t* k1 = kk + 2 * P * batch;
  uint32_t* v1 = kk + 3 * P * batch;
  IQ_CUDA_OK(cudaFuncSetAttribute(select_bands_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)DYN_BYTES));
  const int64_t mper = std::max<int64_t>(1, batch / nq);
  for (int64_t m0 = 0; m0 < nmaps; m0 += mper) {
    BandArgs a{};
    a.maps = maps; a.mm = mm; a.srcs = srcs; a.m0 = m0; a.nmaps = std::min(mper, nmaps - m0);
    a.P = P; a.dx = dx; a.dxy = dxy; a.nq = nq;
    for (int q = 0; q < IQ_PRE_KEYS; ++q) a.seq[q] = q < nq ? seq[q] : 0;
    a.out = out; a.pool = pool; a.cap = cap; a.keys_exact = keys_exact;
    a.rv = rv; a.rr = rr; a.rl = rl; a.list = list; a.k0 = k0; a.v0 = v0; a.k1 = k1; a.v1 = v1;
    iq_timer_start(ctx, "pick");
    select_bands_kernel<<<(unsigned)(a.nmaps * nq), PT, DYN_BYTES, ctx->stream>>>(a);
    iq_timer_stop(ctx, "pick", 0);
    iq_count(ctx);
    IQ_CUDA_OK(cudaGetLastError());
  }
  return IQ_OK;
}
