// Tensor-core distance maps (tcgen05, sm_103a) for masks of the form "tile minus a box": the
// overlap masks of the tile loop (src/iqsim.jl:184-200) and the full tile of soft data
// (src/iqsim.jl:160-169). Same maps as the SIMT kernel of iq_distance.cu,
//   D[n][p] = |A2(p) - 2 AB[n][p] + B2[n]|     (src/utils.jl:5-13, src/imfilter.jl:5-28),
// with AB computed as one GEMM per launch: M = TI positions, N = templates (every realization
// of every tile of one chunk of a dependency level, each column with its own mask box),
// K = the offsets of the union of the masks (a column's template is zero outside its own).
//
// A operand. Positions are taken as runs of consecutive LINEAR TI indices p (x fastest), so
// for a fixed (ky, kz) row of the mask A[p][kx] = TI[p + off(ky, kz) + kx] is a Hankel matrix.
// Its K-major core matrices (8 rows x 16 bytes) are all contained in one shared-memory
// "image" whose 16-byte row u = 8q + r holds TI[e0 + 4q + r + 0..3]: the core matrix of rows
// 8i.. and offsets 4j.. is image block 2i + j, i.e. a descriptor with leading (K) byte offset
// 128 and stride (M) byte offset 256, and advancing K by 8 offsets moves the start address by
// 256 bytes. The CTA's threads build the image from TI values they load one stage ahead
// (L2-resident rows); positions whose x lies past the valid extent are computed and dropped
// (a linear run wraps rows).
//
// B operand. tc_pack_kernel packs the templates per stage into the core-matrix layout (the
// TF32 high halves of all the stage's K-steps, then the low halves; per K-step: offset block
// j, template block i, row, 4 floats), and one cp.async.bulk per stage copies a stage to
// shared memory, completing on an mbarrier.
//
// Precision. FP32 inputs are split into two TF32 halves, v = hi + lo (both rounded to 11
// significant bits), and AB = hi*hi + hi*lo + lo*hi accumulates in FP32 in TMEM (three
// kind::tf32 MMAs per K-step), an error of order 2^-21 sum|A||B|. When the TI and every
// template are TF32 values (integer data below 2^11, for instance) lo = 0 and one MMA per
// K-step gives the same sums. The epilogue computes |(A2 + B2) - 2 AB| in FP32, exact for
// integer data below 2^24 like the rest of the product.
//
// Pipeline. 256 threads, 3 shared-memory stages, no CTA-wide barrier in the main loop:
//   * warp 0, one lane: waits for a stage's B (mbarrier with transaction count) and A
//     (mbarrier, one arrival per producer warp), issues its MMAs and commits them to the
//     stage's "done" mbarrier -- nothing else, since the rate at which this one thread issues
//     is what keeps the tensor pipe busy (a bulk-copy issue can stall it for hundreds of
//     cycles);
//   * warps 1-7: wait until the MMAs that last read a buffer are done; lane 0 of warp 1 starts
//     the bulk copy of the stage's B into it; all write the stage's A images from registers,
//     arrive, and load the TI values of the stage after next (two register sets, so the L2
//     latency of a load has two stages to pass).
// Each CTA owns 2 x 128 positions (two accumulators of N columns in TMEM); all 8 warps run
// the epilogue. Every mbarrier wait is bounded in time: on expiry the kernel records
// IQ_ERR_TIMEOUT, stops issuing work, waits (bounded) for what it issued, frees its TMEM and
// returns.
#include <float.h>

#include <algorithm>

#include "iq_internal.h"

namespace {

constexpr int TC_THREADS = 256;
constexpr int TC_PWARPS = 7;                   // producer warps (1..7)
constexpr int TC_PTHREADS = 32 * TC_PWARPS;
constexpr int TC_MB = 2;     // 128-position blocks per CTA
constexpr int TC_NST = 3;    // pipeline stages
constexpr int TC_STEPS = 3;  // 8-offset K-steps per stage (24 x-offsets)
constexpr int TC_NQ = 32 * TC_MB + 2 * (TC_STEPS - 1);  // 128-byte blocks of one image
constexpr int TC_UPT = (8 * TC_NQ + TC_PTHREADS - 1) / TC_PTHREADS;  // image rows per thread
constexpr int TC_GROUP = 8 * TC_STEPS;                  // x-offsets per stage
constexpr unsigned long long TC_WAIT_NS = 2000000000ull; // bound of every wait
constexpr int TC_SMW = 1024;  // stage words and prefixes kept in shared memory

struct TcArgs {
  const float* img;
  int64_t ix, iy, nimg;
  int64_t dx, dy, dz, Lp;  // valid extents; Lp = (dy - 1) * ix + dx linear span of a plane
  int bpp;                 // CTAs per z-plane
  int64_t tx, ty, tz;
  const double* ii;
  int nbox;
  TcBox box[IQ_TC_MAXBOX];
  const uint8_t* disabled;
  const uint32_t* word;
  const uint32_t* prefix;
  int nstage;
  const char* B;
  const TcCol* cols;
  int N;
  int exact;
  uint32_t tmem_cols;
  int* status;
  unsigned long long* stats;  // profiling counters (nullable)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared-memory matrix descriptor, no swizzle: start, leading (K) and stride (M/N) byte
// offsets in 16-byte units, descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for the phase of parity `parity` to complete; false after TC_WAIT_NS.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_test(bar, parity)) return true;
    if ((it & 63u) == 0 && globaltimer() - t0 > TC_WAIT_NS) return false;
  }
}

// mbar_wait that adds the cycles it spent to *acc when profiling
__device__ __forceinline__ bool mbar_wait_t(uint32_t bar, uint32_t parity, bool prof,
                                            long long& acc) {
  if (!prof) return mbar_wait(bar, parity);
  const long long t = clock64();
  const bool ok = mbar_wait(bar, parity);
  acc += clock64() - t;
  return ok;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// v = hi + lo with both halves rounded to TF32 (11 significant bits, ties away from zero).
__device__ __forceinline__ void tf32_split(float v, uint32_t& hi, uint32_t& lo) {
  hi = (__float_as_uint(v) + 0x1000u) & 0xFFFFE000u;
  const float r = __fsub_rn(v, __uint_as_float(hi));
  lo = (__float_as_uint(r) + 0x1000u) & 0xFFFFE000u;
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c,
                                             uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c),
               "r"(d)
               : "memory");
}

__device__ __forceinline__ int nth_bit(uint32_t mask, int n) {
  for (int s = 0; s < 32; ++s)
    if (mask >> s & 1u) {
      if (n == 0) return s;
      --n;
    }
  return 0;
}

__device__ __forceinline__ bool in_box(const TcBox& b, int64_t x, int64_t y, int64_t z) {
  return x >= b.lo[0] && x < b.hi[0] && y >= b.lo[1] && y < b.hi[1] && z >= b.lo[2] &&
         z < b.hi[2];
}

// ---- packing of the templates into the B core-matrix layout ----
struct PackArgs {
  const float* grid;
  int64_t gx, gy, tx;
  const TcCol* cols;
  int N;
  const uint32_t* word;
  const uint32_t* prefix;
  int nstage;
  TcBox box[IQ_TC_MAXBOX];
  char* B;
};

// Stage e occupies prefix[e] * 64N bytes from B: the high halves of its nact K-steps
// (32N bytes each: offset block jj = 0..1, template n, 4 floats), then the low halves.
__global__ void tc_pack_kernel(const PackArgs p) {
  const int N = p.N;
  for (int e = blockIdx.y; e < p.nstage; e += gridDim.y) {
    const uint32_t w = p.word[e];
    const int ky = (int)(w & 1023u), kz = (int)((w >> 10) & 1023u), g = (int)((w >> 20) & 63u);
    const uint32_t smask = w >> 26;
    const int nact = __popc(smask);
    const int units = nact * 2 * N;
    char* base = p.B + (size_t)p.prefix[e] * 64 * N;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < units; u += gridDim.x * blockDim.x) {
      const int a = u / (2 * N), rem = u - a * 2 * N;
      const int jj = rem / N, n = rem - jj * N;
      const int s = nth_bit(smask, a);
      const int64_t kx0 = (int64_t)TC_GROUP * g + 8 * s + 4 * jj;
      const TcCol col = p.cols[n];
      const TcBox bx = p.box[col.src >= 0 ? col.box : 0];
      uint32_t h[4], l[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int64_t kx = kx0 + c;
        float v = 0.f;
        if (col.src >= 0 && kx < p.tx && !in_box(bx, kx, ky, kz))
          v = p.grid[col.src + kx + p.gx * (ky + p.gy * (int64_t)kz)];
        tf32_split(v, h[c], l[c]);
      }
      uint4* hi = reinterpret_cast<uint4*>(base + (size_t)a * 32 * N + (size_t)rem * 16);
      uint4* lo = reinterpret_cast<uint4*>(base + (size_t)(nact + a) * 32 * N + (size_t)rem * 16);
      *hi = make_uint4(h[0], h[1], h[2], h[3]);
      *lo = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
}

// ---- the GEMM ----
struct StageInfo {
  int64_t e0;   // TI index of image row 0
  int nunits;   // 16-byte image rows to write
  uint32_t smask;
  uint32_t pre;
};

// stage e's word and prefix: from the shared-memory copy (first TC_SMW stages) or global
__device__ __forceinline__ uint32_t stage_word(const TcArgs& a, const uint32_t* sw, int e) {
  return e < TC_SMW ? sw[e] : __ldg(a.word + e);
}
__device__ __forceinline__ uint32_t stage_pre(const TcArgs& a, const uint32_t* sw, int e) {
  return e < TC_SMW ? sw[TC_SMW + e] : __ldg(a.prefix + e);
}

__device__ __forceinline__ StageInfo stage_info(const TcArgs& a, const uint32_t* sw, int e,
                                                int64_t p0) {
  StageInfo s;
  const uint32_t w = stage_word(a, sw, e);
  s.pre = stage_pre(a, sw, e);
  const int ky = (int)(w & 1023u), kz = (int)((w >> 10) & 1023u), g = (int)((w >> 20) & 63u);
  s.smask = w >> 26;
  const int smax = 31 - __clz((int)s.smask);
  s.e0 = p0 + (int64_t)TC_GROUP * g + a.ix * (ky + a.iy * (int64_t)kz);
  s.nunits = 8 * (32 * TC_MB + 2 * smax);
  return s;
}

__device__ __forceinline__ void stage_load(const TcArgs& a, const StageInfo& s, int ptid,
                                           float (&v)[TC_UPT][4]) {
#pragma unroll
  for (int i = 0; i < TC_UPT; ++i) {
    const int u = ptid + i * TC_PTHREADS;
    if (u < s.nunits) {
      const int64_t base = s.e0 + 4 * (u >> 3) + (u & 7);
#pragma unroll
      for (int c = 0; c < 4; ++c) v[i][c] = __ldg(a.img + min(base + c, a.nimg - 1));
    }
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1) corr_tc_kernel(const TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t s_tmem;
  const int N = a.N;
  const uint32_t bbytes = (uint32_t)TC_STEPS * 64u * (uint32_t)N;
  const uint32_t stage_bytes = bbytes + 2u * TC_NQ * 128u;
  unsigned char* colbase = smem + TC_NST * stage_bytes;
  float** s_out = reinterpret_cast<float**>(colbase);
  unsigned** s_mmp = reinterpret_cast<unsigned**>(colbase + 8 * N);
  float* s_b2 = reinterpret_cast<float*>(colbase + 16 * N);
  unsigned* s_mn = reinterpret_cast<unsigned*>(colbase + 20 * N);
  unsigned* s_mx = s_mn + N;
  int* s_box = reinterpret_cast<int*>(colbase + 28 * N);
  float* s_a2 = reinterpret_cast<float*>(colbase + 32 * N);  // [box][128 * TC_MB positions]
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_a2 + IQ_TC_MAXBOX * 128 * TC_MB);
  uint32_t* s_stage = reinterpret_cast<uint32_t*>(bars + 3 * TC_NST + 1);  // words, prefixes
  // full[NST] (B copies), done[NST] (MMA commits), afull[NST] (A images), fin
  const uint32_t bar_full = smem_u32(bars), bar_done = bar_full + 8 * TC_NST,
                 bar_afull = bar_full + 16 * TC_NST, bar_fin = bar_full + 24 * TC_NST;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int n = tid; n < N; n += TC_THREADS) {
    const TcCol c = a.cols[n];
    const bool live = c.src >= 0;
    s_out[n] = live ? c.out : nullptr;
    s_mmp[n] = live ? c.mm : nullptr;
    s_b2[n] = (live && c.b2) ? (float)*c.b2 : 0.f;
    s_box[n] = live ? c.box : 0;
    s_mn[n] = 0x7F800000u;
    s_mx[n] = 0u;
  }
  for (int e = tid; e < a.nstage && e < TC_SMW; e += TC_THREADS) {
    s_stage[e] = __ldg(a.word + e);
    s_stage[TC_SMW + e] = __ldg(a.prefix + e);
  }
  if (tid == 0) {
    for (int i = 0; i < 2 * TC_NST; ++i) mbar_init(bar_full + 8 * i, 1);
    for (int i = 0; i < TC_NST; ++i) mbar_init(bar_afull + 8 * i, TC_PWARPS);
    mbar_init(bar_fin, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s_tmem)),
                 "r"(a.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;

  const int64_t z = blockIdx.x / a.bpp;
  const int64_t zbase = z * a.ix * a.iy;
  const int64_t p0 = zbase + (int64_t)(blockIdx.x % a.bpp) * (128 * TC_MB);
  const uint32_t sbase = smem_u32(smem);
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
                         ((128u >> 4) << 24);

  int fail = 0;  // this thread saw a wait expire
  int aborted = 0;
  if (warp == 0) {
    if (lane == 0) {
      // ---- copies and MMAs ----
      // The issue rate of one thread bounds the tensor pipe, so the loop is lean: descriptors
      // of buffer 0 are built once (a buffer or K-step is an offset added to the start field),
      // the K-step and M-block loops are unrolled and the stage words sit in shared memory.
      const uint64_t dA0 = make_desc(sbase + bbytes, 128u, 256u);
      const uint64_t dL0 = make_desc(sbase + bbytes + TC_NQ * 128u, 128u, 256u);
      const uint64_t dB0 = make_desc(sbase, 16u * N, 128u);
      const uint32_t dbuf = stage_bytes >> 4, dstep = 2u * N;  // buffer, K-step B (16-byte units)
      int e = 0;
      int b = 0;
      uint32_t par = 0;
      const bool prof = a.stats != nullptr;
      long long t_full = 0, t_afull = 0, t_done = 0, t_issue = 0;  // t_done: unused now
      unsigned long long mmau = 0;
      const long long t_loop0 = prof ? clock64() : 0;
      for (; e < a.nstage; ++e) {
        if (!mbar_wait_t(bar_full + 8 * b, par, prof, t_full) ||
            !mbar_wait_t(bar_afull + 8 * b, par, prof, t_afull)) {
          fail = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const long long t_i0 = prof ? clock64() : 0;
        const uint32_t smask = stage_word(a, s_stage, e) >> 26;
        const uint32_t nact = (uint32_t)__popc(smask);
        const uint64_t dA = dA0 + (uint64_t)(b * dbuf), dL = dL0 + (uint64_t)(b * dbuf);
        const uint64_t dB = dB0 + (uint64_t)(b * dbuf);
        uint32_t act = 0;
        uint32_t acc = e > 0 ? 1u : 0u;
#pragma unroll
        for (int s = 0; s < TC_STEPS; ++s) {
          if (smask >> s & 1u) {
            const uint64_t bh = dB + (uint64_t)(act * dstep), bl = dB + (uint64_t)((nact + act) * dstep);
#pragma unroll
            for (int mb = 0; mb < TC_MB; ++mb) {
              const uint32_t ao = 8u * (32u * mb + 2u * s);  // 128 (32 mb + 2 s) bytes
              const uint32_t d = tmem + (uint32_t)(mb * N);
              mma_tf32(d, dA + ao, bh, idesc, acc);
              if (!a.exact) {
                mma_tf32(d, dA + ao, bl, idesc, 1u);
                mma_tf32(d, dL + ao, bh, idesc, 1u);
              }
            }
            ++act;
            acc = 1u;
          }
        }
        mma_commit(bar_done + 8 * b);
        if (prof) {
          t_issue += clock64() - t_i0;
          mmau += (unsigned long long)nact * TC_MB * (a.exact ? 1 : 3) * N;
        }
        if (++b == TC_NST) { b = 0; par ^= 1u; }
      }
      if (prof) {
        atomicAdd(a.stats + ST_TC_LOOP, (unsigned long long)(clock64() - t_loop0));
        atomicAdd(a.stats + ST_TC_WFULL, (unsigned long long)t_full);
        atomicAdd(a.stats + ST_TC_WAFULL, (unsigned long long)t_afull);
        atomicAdd(a.stats + ST_TC_WDONE, (unsigned long long)t_done);
        atomicAdd(a.stats + ST_TC_CTAS, 1ull);
        atomicAdd(a.stats + ST_TC_ISSUE, (unsigned long long)t_issue);
        atomicAdd(a.stats + ST_TC_MMAU, mmau);
      }
      // every MMA issued has completed (or the waits gave up)
      if (a.nstage > 0) mma_commit(bar_fin);
      else mbar_arrive(bar_fin);
    }
    __syncwarp();
  } else {
    // ---- A images (TI values loaded two stages ahead, in two register sets) ----
    const int ptid = tid - 32;
    float va[TC_UPT][4], vb[TC_UPT][4];
    StageInfo sa{}, sbi{};
    if (a.nstage > 0) {
      sa = stage_info(a, s_stage, 0, p0);
      stage_load(a, sa, ptid, va);
    }
    if (a.nstage > 1) {
      sbi = stage_info(a, s_stage, 1, p0);
      stage_load(a, sbi, ptid, vb);
    }
    const bool prof = a.stats != nullptr && warp == 1 && lane == 0;
    long long t_wait = 0;
    const long long t_p0 = prof ? clock64() : 0;
    // write stage e's images from v; false when the wait for the buffer gave up
    const bool copier = warp == 1 && lane == 0;  // issues the B copies
    int ncopied = 0;
    auto build = [&](int e, const StageInfo& si, float (&v)[TC_UPT][4]) -> bool {
      const int b = e % TC_NST;
      const uint32_t use = (uint32_t)(e / TC_NST);
      const bool ok = use == 0 || mbar_wait_t(bar_done + 8 * b, (use - 1) & 1u, prof, t_wait);
      if (__any_sync(0xffffffffu, !ok)) return false;  // the warp leaves together
      if (copier) {
        const uint32_t bytes = (uint32_t)__popc(si.smask) * (a.exact ? 32u : 64u) * (uint32_t)N;
        bulk_g2s(sbase + b * stage_bytes, a.B + (size_t)si.pre * 64 * N, bytes, bar_full + 8 * b);
        ncopied = e + 1;
      }
      const uint32_t sa_hi = sbase + b * stage_bytes + bbytes, sa_lo = sa_hi + TC_NQ * 128u;
#pragma unroll
      for (int i = 0; i < TC_UPT; ++i) {
        const int u = ptid + i * TC_PTHREADS;
        if (u < si.nunits) {
          uint32_t h[4], l[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) tf32_split(v[i][c], h[c], l[c]);
          st_shared_v4(sa_hi + 16u * u, h[0], h[1], h[2], h[3]);
          if (!a.exact) st_shared_v4(sa_lo + 16u * u, l[0], l[1], l[2], l[3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(bar_afull + 8 * b);
      return true;
    };
    for (int e = 0; e < a.nstage; e += 2) {
      if (!build(e, sa, va)) { fail = 1; break; }
      if (e + 2 < a.nstage) {
        sa = stage_info(a, s_stage, e + 2, p0);
        stage_load(a, sa, ptid, va);
      }
      if (e + 1 >= a.nstage) break;
      if (!build(e + 1, sbi, vb)) { fail = 1; break; }
      if (e + 3 < a.nstage) {
        sbi = stage_info(a, s_stage, e + 3, p0);
        stage_load(a, sbi, ptid, vb);
      }
    }
    if (copier)  // the last copies have landed (bounded waits) before the buffers go away
      for (int st = ncopied - 1; st >= 0 && st >= ncopied - TC_NST; --st)
        mbar_wait(bar_full + 8 * (st % TC_NST), (uint32_t)(st / TC_NST) & 1u);
    if (prof) {
      atomicAdd(a.stats + ST_TC_PWAIT, (unsigned long long)t_wait);
      atomicAdd(a.stats + ST_TC_PLOOP, (unsigned long long)(clock64() - t_p0));
    }
  }
  if (!mbar_wait(bar_fin, 0)) fail = 1;
  if (__syncthreads_or(fail)) aborted = 1;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  const long long t_epi0 = (a.stats && tid == 0) ? clock64() : 0;
  if (!aborted) {
    // A2 of each mask at each position, in FP64 from the integral image, stored as FP32
    const int lq = warp & 3, half = warp >> 2;
    const int64_t sx = a.ix + 1, sxy = (a.ix + 1) * (a.iy + 1);
#pragma unroll 1
    for (int mb = 0; mb < TC_MB; ++mb) {
      const int m = 128 * mb + 32 * lq + lane;
      const int64_t rel = p0 + m - zbase;
      const int64_t x = rel % a.ix, y = rel / a.ix;
      const bool valid = rel < a.Lp && x < a.dx;
      double full = 0.0;
      if (valid) full = iq_box_sum(a.ii, sx, sxy, x, y, z, a.tx, a.ty, a.tz);
      for (int bi = half; bi < a.nbox; bi += 2) {
        double A2 = full;
        const TcBox& bx = a.box[bi];
        if (valid && bx.hi[0] > bx.lo[0] && bx.hi[1] > bx.lo[1] && bx.hi[2] > bx.lo[2])
          A2 -= iq_box_sum(a.ii, sx, sxy, x + bx.lo[0], y + bx.lo[1], z + bx.lo[2],
                           bx.hi[0] - bx.lo[0], bx.hi[1] - bx.lo[1], bx.hi[2] - bx.lo[2]);
        s_a2[bi * 128 * TC_MB + m] = (float)A2;
      }
    }
    __syncthreads();
#pragma unroll 1
    for (int mb = 0; mb < TC_MB; ++mb) {
      const int m = 128 * mb + 32 * lq + lane;
      const int64_t rel = p0 + m - zbase;
      const int64_t x = rel % a.ix, y = rel / a.ix;
      const bool valid = rel < a.Lp && x < a.dx;
      const int64_t pout = valid ? x + a.dx * (y + a.dy * z) : 0;
      const bool dis = valid && a.disabled != nullptr && a.disabled[pout];
#pragma unroll 1
      for (int c0 = 16 * half; c0 < N; c0 += 32) {
        uint32_t r[16];
        if (a.nstage > 0) {
          tmem_ld16(tmem + ((uint32_t)(32 * lq) << 16) + (uint32_t)(mb * N + c0), r);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) r[j] = 0u;  // no offsets: AB = 0
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = c0 + j;
          float* o = s_out[n];
          unsigned mnb = 0x7F800000u, mxb = 0u;
          if (valid && o) {
            float df;
            if (dis) {
              df = __int_as_float(0x7F800000);
            } else {
              const float s2 = __fadd_rn(s_a2[s_box[n] * 128 * TC_MB + m], s_b2[n]);
              df = fabsf(__fmaf_rn(-2.f, __uint_as_float(r[j]), s2));
            }
            o[pout] = df;
            mnb = __float_as_uint(df);
            if (mnb < 0x7F800000u) mxb = mnb;
          }
          const unsigned m1 = __reduce_min_sync(0xffffffffu, mnb);
          const unsigned m2 = __reduce_max_sync(0xffffffffu, mxb);
          if (lane == 0 && o) {
            if (m1 != 0x7F800000u) atomicMin(s_mn + n, m1);
            if (m2 != 0u) atomicMax(s_mx + n, m2);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (a.stats && tid == 0) atomicAdd(a.stats + ST_TC_EPI, (unsigned long long)(clock64() - t_epi0));
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(a.tmem_cols));
  if (aborted) {
    if (tid == 0 && a.status) atomicCAS(a.status, 0, IQ_ERR_TIMEOUT);
    return;
  }
  for (int n = tid; n < N; n += TC_THREADS) {
    unsigned* mm = s_mmp[n];
    if (mm && s_mn[n] != 0x7F800000u) atomicMin(mm, s_mn[n]);
    if (mm && s_mx[n] != 0u) atomicMax(mm + 1, s_mx[n]);
  }
}

size_t tc_smem_bytes(int N) {
  return (size_t)TC_NST * ((size_t)TC_STEPS * 64 * N + 2 * TC_NQ * 128) + 32 * (size_t)N +
         4 * IQ_TC_MAXBOX * 128 * TC_MB + 8 * (3 * TC_NST + 1) + 8 * TC_SMW;
}

__global__ void tf32_check_kernel(const float* __restrict__ d, int64_t n, int* flag) {
  unsigned bad = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    bad |= __float_as_uint(d[i]) & 0x1FFFu;
  if (__syncthreads_or(bad != 0) && threadIdx.x == 0) atomicOr(flag, 1);
}

}  // namespace

void iq_tc_stages(Dim3 tile, const TcBox* boxes, int nbox, TcStages& out) {
  out.word.clear();
  out.prefix.clear();
  out.nsteps = 0;
  const int64_t ngroup = (tile.x + TC_GROUP - 1) / TC_GROUP;
  for (int64_t kz = 0; kz < tile.z; ++kz)
    for (int64_t ky = 0; ky < tile.y; ++ky)
      for (int64_t g = 0; g < ngroup; ++g) {
        uint32_t smask = 0;
        for (int s = 0; s < TC_STEPS; ++s) {
          const int64_t k0 = TC_GROUP * g + 8 * s, k1 = std::min(k0 + 8, tile.x);
          bool any = false;
          for (int b = 0; b < nbox && !any; ++b) {
            const TcBox& bx = boxes[b];
            const bool rowin = ky >= bx.lo[1] && ky < bx.hi[1] && kz >= bx.lo[2] && kz < bx.hi[2];
            for (int64_t kx = k0; kx < k1 && !any; ++kx)
              any = !(rowin && kx >= bx.lo[0] && kx < bx.hi[0]);
          }
          if (any) smask |= 1u << s;
        }
        if (!smask) continue;
        out.word.push_back((uint32_t)ky | ((uint32_t)kz << 10) | ((uint32_t)g << 20) | (smask << 26));
        out.prefix.push_back((uint32_t)out.nsteps);
        out.nsteps += __builtin_popcount(smask);
      }
}

int iq_tf32_exact(iq_ctx* ctx, const float* d, int64_t n, bool& exact) {
  exact = false;
  int* flag = (int*)iq_scratch(ctx, S_TCFLAG, sizeof(int));
  if (!flag) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
  if (n > 0) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    tf32_check_kernel<<<blocks, 256, 0, ctx->stream>>>(d, n, flag);
    iq_count(ctx);
    IQ_CUDA_OK(cudaGetLastError());
  }
  int h = 1;
  IQ_CUDA_OK(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  exact = h == 0;
  return IQ_OK;
}

int iq_launch_corr_tc(iq_ctx* ctx, const TcCorrLaunch& L) {
  if (L.N <= 0 || L.N % 16 || L.N > IQ_TC_MAXN || !L.ii || !L.cols || !L.B || L.nbox < 1 ||
      L.nbox > IQ_TC_MAXBOX)
    return iq_set_error(IQ_ERR_ARG, "tensor-core correlation: bad launch");
  if (L.tile.x / TC_GROUP >= 64 || L.tile.y >= 1024 || L.tile.z >= 1024)
    return iq_set_error(IQ_ERR_LIMIT, "tensor-core correlation: tile too large");
  const Dim3 od = L.out_dims;
  if (od.vol() <= 0) return IQ_OK;
  TcArgs a;
  a.img = L.img;
  a.ix = L.img_dims.x;
  a.iy = L.img_dims.y;
  a.nimg = L.img_dims.vol();
  a.dx = od.x; a.dy = od.y; a.dz = od.z;
  a.Lp = (od.y - 1) * a.ix + od.x;
  const int64_t bpp = (a.Lp + 128 * TC_MB - 1) / (128 * TC_MB);
  a.bpp = (int)bpp;
  a.tx = L.tile.x; a.ty = L.tile.y; a.tz = L.tile.z;
  a.ii = L.ii;
  a.nbox = L.nbox;
  for (int b = 0; b < IQ_TC_MAXBOX; ++b) a.box[b] = L.box[b];
  a.disabled = L.disabled;
  a.word = L.stage_word;
  a.prefix = L.stage_prefix;
  a.nstage = L.nstage;
  a.B = (const char*)L.B;
  a.cols = L.cols;
  a.N = L.N;
  a.exact = L.exact ? 1 : 0;
  uint32_t tc = 32;
  while (tc < (uint32_t)(TC_MB * L.N)) tc <<= 1;
  a.tmem_cols = tc;
  a.status = ctx->d_status;
  a.stats = ctx->prof ? ctx->d_stats : nullptr;

  iq_timer_start(ctx, "corr");
  if (L.nstage > 0) {  // no stages: every column's mask is empty and its products are zero
    PackArgs p;
    p.grid = L.grid; p.gx = L.grid_dims.x; p.gy = L.grid_dims.y; p.tx = L.tile.x;
    p.cols = L.cols; p.N = L.N;
    p.word = L.stage_word; p.prefix = L.stage_prefix; p.nstage = L.nstage;
    for (int b = 0; b < IQ_TC_MAXBOX; ++b) p.box[b] = L.box[b];
    p.B = (char*)L.B;
    dim3 grid((unsigned)((TC_STEPS * 2 * L.N + 255) / 256), (unsigned)std::min(L.nstage, 65535));
    tc_pack_kernel<<<grid, 256, 0, ctx->stream>>>(p);
    iq_count(ctx);
    IQ_CUDA_OK(cudaGetLastError());
  }
  const size_t smem = tc_smem_bytes(L.N);
  IQ_CUDA_OK(cudaFuncSetAttribute(corr_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  const int64_t nblk = od.z * bpp;
  if (ctx->prof) {
    ctx->prof_mma_flops += 2.0 * (double)nblk * 128 * TC_MB * (double)L.nsteps * 8 * L.N *
                           (L.exact ? 1 : 3);
    ctx->prof_mma_launches += 1;
    ctx->prof_tc_cols += L.N;
  }
  corr_tc_kernel<<<(unsigned)nblk, TC_THREADS, smem, ctx->stream>>>(a);
  iq_count(ctx);
  iq_timer_stop(ctx, "corr", L.flops);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
