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
#include <cuda_fp16.h>
#include <float.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "iq_internal.h"

namespace {

constexpr int TC_THREADS = 256;
constexpr int TC_PWARPS = 7;                   // producer warps (1..7)
constexpr int TC_PTHREADS = 32 * TC_PWARPS;
constexpr int TC_MB = 2;     // 128-position blocks per CTA
constexpr int TC_NST = 3;    // pipeline stages
constexpr int TC_STEPS = 3;  // 8-offset K-steps per stage (24 x-offsets)
constexpr int TC_NQ = 32 * TC_MB + 2 * (TC_STEPS - 1);  // 128-byte blocks of one TF32 image
constexpr int TC_GROUP = 8 * TC_STEPS;                  // x-offsets per row entry
constexpr unsigned long long TC_WAIT_NS = 2000000000ull; // bound of every wait
constexpr int TC_SMW = 512;   // stage words and prefixes kept in shared memory
// FP16 form: a stage is two row entries; an image row holds 8 halves, a row image has
// 16 * TC_MB + 3 blocks of 128 bytes (the last one only read by a K-step's unused half)
constexpr int F_CH = 3;                       // 8-offset chunks per row entry
constexpr int F_NQ = 16 * TC_MB + F_CH;       // blocks of one FP16 row image
constexpr int F_IMG = F_NQ * 128;             // bytes of one FP16 row image
constexpr int F_ROWU = 8 * F_NQ;              // image rows of one row entry

// A region of a stage: TF32 -> hi and lo images of one row entry; FP16 -> hi images of two
// row entries, then their lo images
template <bool F16> constexpr int a_region() { return F16 ? 4 * F_IMG : 2 * TC_NQ * 128; }
template <bool F16> constexpr int stage_units() { return F16 ? 2 * F_ROWU : 8 * TC_NQ; }
template <bool F16> constexpr int upt() {
  return (stage_units<F16>() + TC_PTHREADS - 1) / TC_PTHREADS;  // image rows per thread
}
template <bool F16> constexpr int vpu() { return F16 ? 8 : 4; }  // values per image row

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
  const uint32_t* wordb;      // FP16 form: second row entry of each stage (0 = none)
  const uint32_t* prefix;
  int nstage;
  const char* B;
  const TcCol* cols;
  int N;
  int exact;
  float scale_a;              // FP16 form: 2^-kA applied to the image values
  float ab2;                  // 2 * 2^(kA + kB): D = |A2 + B2 - ab2 * acc|
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

// two 16-column loads (columns taddr0.., taddr1..) and one wait
__device__ __forceinline__ void tmem_ld16x2(uint32_t taddr0, uint32_t taddr1, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr0));
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr1));
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
  int64_t e0a, e0b;  // TI index of image row 0 of the stage's row entries
  uint32_t ma, mb;   // their chunk masks (mb = 0: no second row entry)
  uint32_t pre;      // K-steps before the stage
  int nunits;        // 16-byte image rows to write
};

// stage e's words and prefix: from the shared-memory copy (first TC_SMW stages) or global
__device__ __forceinline__ uint32_t stage_word(const TcArgs& a, const uint32_t* sw, int e) {
  return e < TC_SMW ? sw[e] : __ldg(a.word + e);
}
__device__ __forceinline__ uint32_t stage_wordb(const TcArgs& a, const uint32_t* sw, int e) {
  return e < TC_SMW ? sw[2 * TC_SMW + e] : __ldg(a.wordb + e);
}
__device__ __forceinline__ uint32_t stage_pre(const TcArgs& a, const uint32_t* sw, int e) {
  return e < TC_SMW ? sw[TC_SMW + e] : __ldg(a.prefix + e);
}

__device__ __forceinline__ int64_t row_e0(const TcArgs& a, uint32_t w, int64_t p0) {
  const int ky = (int)(w & 1023u), kz = (int)((w >> 10) & 1023u), g = (int)((w >> 20) & 63u);
  return p0 + (int64_t)TC_GROUP * g + a.ix * (ky + a.iy * (int64_t)kz);
}

// K-steps of a stage: TF32 -> one per active 8-offset step; FP16 -> the active 8-offset
// chunks of the two row entries taken in pairs
template <bool F16>
__device__ __forceinline__ int stage_ksteps(uint32_t ma, uint32_t mb) {
  return F16 ? (__popc(ma) + __popc(mb) + 1) >> 1 : __popc(ma);
}

template <bool F16>
__device__ __forceinline__ StageInfo stage_info(const TcArgs& a, const uint32_t* sw, int e,
                                                int64_t p0) {
  StageInfo s;
  const uint32_t w = stage_word(a, sw, e);
  s.pre = stage_pre(a, sw, e);
  s.ma = w >> 26;
  s.e0a = row_e0(a, w, p0);
  if (F16) {
    const uint32_t wb = stage_wordb(a, sw, e);
    s.mb = wb >> 26;
    s.e0b = s.mb ? row_e0(a, wb, p0) : s.e0a;
    s.nunits = (s.mb ? 2 : 1) * F_ROWU;
  } else {
    s.mb = 0;
    s.e0b = s.e0a;
    const int smax = 31 - __clz((int)s.ma);
    s.nunits = 8 * (32 * TC_MB + 2 * smax);
  }
  return s;
}

// image row u of a stage: TF32 -> TI[e0 + 4 (u / 8) + u % 8 + 0..3]; FP16 -> row entry
// u / F_ROWU, TI[e0 + 8 (v / 8) + v % 8 + 0..7] with v = u % F_ROWU
template <bool F16>
__device__ __forceinline__ int64_t unit_base(const StageInfo& s, int u) {
  if (F16) {
    const bool second = u >= F_ROWU;
    const int v = second ? u - F_ROWU : u;
    return (second ? s.e0b : s.e0a) + 8 * (v >> 3) + (v & 7);
  }
  return s.e0a + 4 * (u >> 3) + (u & 7);
}

template <bool F16>
__device__ __forceinline__ void stage_load(const TcArgs& a, const StageInfo& s, int ptid,
                                           float (&v)[upt<F16>()][vpu<F16>()]) {
#pragma unroll
  for (int i = 0; i < upt<F16>(); ++i) {
    const int u = ptid + i * TC_PTHREADS;
    if (u < s.nunits) {
      const int64_t base = unit_base<F16>(s, u);
#pragma unroll
      for (int c = 0; c < vpu<F16>(); ++c) v[i][c] = __ldg(a.img + min(base + c, a.nimg - 1));
    }
  }
}

// v * scale = hi + lo, both FP16 (round to nearest even)
__device__ __forceinline__ void f16_split(float v, float scale, uint16_t& hi, uint16_t& lo) {
  const float x = v * scale;  // a power of two: exact
  const __half h = __float2half_rn(x);
  const __half l = __float2half_rn(__fsub_rn(x, __half2float(h)));
  hi = __half_as_ushort(h);
  lo = __half_as_ushort(l);
}

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// chunk idx of an FP16 stage: byte offset of its core-matrix column inside the A hi region
// (row entry a at 0, row entry b at F_IMG; chunk c is c blocks further)
__device__ __forceinline__ uint32_t f16_chunk_off(uint32_t ma, uint32_t mb, int idx) {
  const int na = __popc(ma);
  return idx < na ? 128u * (uint32_t)nth_bit(ma, idx)
                  : (uint32_t)F_IMG + 128u * (uint32_t)nth_bit(mb, idx - na);
}

template <bool F16>
__global__ void __launch_bounds__(TC_THREADS, 1) corr_tc_kernel(const TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t s_tmem;
  constexpr int UPT = upt<F16>(), VPU = vpu<F16>();
  const int N = a.N;
  const uint32_t bbytes = (uint32_t)TC_STEPS * 64u * (uint32_t)N;
  const uint32_t stage_bytes = bbytes + (uint32_t)a_region<F16>();
  unsigned char* colbase = smem + TC_NST * stage_bytes;
  float** s_out = reinterpret_cast<float**>(colbase);
  unsigned** s_mmp = reinterpret_cast<unsigned**>(colbase + 8 * N);
  float* s_b2 = reinterpret_cast<float*>(colbase + 16 * N);
  unsigned* s_mn = reinterpret_cast<unsigned*>(colbase + 20 * N);
  unsigned* s_mx = s_mn + N;
  int* s_box = reinterpret_cast<int*>(colbase + 28 * N);
  float* s_a2 = reinterpret_cast<float*>(colbase + 32 * N);  // [box][128 * TC_MB positions]
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_a2 + IQ_TC_MAXBOX * 128 * TC_MB);
  // stage words, prefixes, second words (FP16)
  uint32_t* s_stage = reinterpret_cast<uint32_t*>(bars + 3 * TC_NST + 1);
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
    if (F16) s_stage[2 * TC_SMW + e] = __ldg(a.wordb + e);
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
  // D F32; A, B: TF32 (2) or F16 (0); N >> 3 at bit 17, M >> 4 at bit 24
  const uint32_t ab_fmt = F16 ? 0u : 2u;
  const uint32_t idesc = (1u << 4) | (ab_fmt << 7) | (ab_fmt << 10) |
                         ((uint32_t)(N >> 3) << 17) | ((128u >> 4) << 24);

  int fail = 0;  // this thread saw a wait expire
  int aborted = 0;
  if (warp == 0) {
    if (lane == 0) {
      // ---- MMAs ----
      // The issue rate of one thread bounds the tensor pipe, so the loop is lean: the B
      // descriptor of buffer 0 is built once (a buffer or K-step is an offset added to the
      // start field), the loops are unrolled and the stage words sit in shared memory.
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
        const uint32_t ma = stage_word(a, s_stage, e) >> 26;
        const uint32_t mb2 = F16 ? stage_wordb(a, s_stage, e) >> 26 : 0u;
        const uint32_t nks = (uint32_t)stage_ksteps<F16>(ma, mb2);
        const uint32_t sA = sbase + b * stage_bytes + bbytes;  // A region of this buffer
        const uint64_t dB = dB0 + (uint64_t)(b * dbuf);
        uint32_t acc = e > 0 ? 1u : 0u;
        if (F16) {
          const int total = __popc(ma) + __popc(mb2);
#pragma unroll
          for (int t = 0; t < TC_STEPS; ++t) {
            if (t < (int)nks) {
              const uint64_t bh = dB + (uint64_t)(t * dstep), bl = dB + (uint64_t)((nks + t) * dstep);
              // two 8-offset chunks X, Y: the descriptor's leading offset joins them (the
              // unused half of an odd last K-step reads the next block, its B half is zero)
              const uint32_t ox = f16_chunk_off(ma, mb2, 2 * t);
              const uint32_t lbo = 2 * t + 1 < total ? f16_chunk_off(ma, mb2, 2 * t + 1) - ox : 128u;
#pragma unroll
              for (int mb = 0; mb < TC_MB; ++mb) {
                const uint32_t ao = ox + 128u * 16u * mb;
                const uint32_t d = tmem + (uint32_t)(mb * N);
                const uint64_t dah = make_desc(sA + ao, lbo, 128u);
                mma_f16(d, dah, bh, idesc, acc);
                if (!a.exact) {
                  const uint64_t dal = make_desc(sA + 2 * F_IMG + ao, lbo, 128u);
                  mma_f16(d, dah, bl, idesc, 1u);
                  mma_f16(d, dal, bh, idesc, 1u);
                }
              }
              acc = 1u;
            }
          }
        } else {
          const uint64_t dA = make_desc(sA, 128u, 256u);
          const uint64_t dL = make_desc(sA + TC_NQ * 128u, 128u, 256u);
          uint32_t act = 0;
#pragma unroll
          for (int s = 0; s < TC_STEPS; ++s) {
            if (ma >> s & 1u) {
              const uint64_t bh = dB + (uint64_t)(act * dstep), bl = dB + (uint64_t)((nks + act) * dstep);
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
        }
        mma_commit(bar_done + 8 * b);
        if (prof) {
          t_issue += clock64() - t_i0;
          mmau += (unsigned long long)nks * TC_MB * (a.exact ? 1 : 3) * N;
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
    float va[UPT][VPU], vb[UPT][VPU];
    StageInfo sa{}, sbi{};
    if (a.nstage > 0) {
      sa = stage_info<F16>(a, s_stage, 0, p0);
      stage_load<F16>(a, sa, ptid, va);
    }
    if (a.nstage > 1) {
      sbi = stage_info<F16>(a, s_stage, 1, p0);
      stage_load<F16>(a, sbi, ptid, vb);
    }
    const bool prof = a.stats != nullptr && warp == 1 && lane == 0;
    long long t_wait = 0;
    const long long t_p0 = prof ? clock64() : 0;
    // write stage e's images from v; false when the wait for the buffer gave up
    const bool copier = warp == 1 && lane == 0;  // issues the B copies
    int ncopied = 0;
    auto build = [&](int e, const StageInfo& si, float (&v)[UPT][VPU]) -> bool {
      const int b = e % TC_NST;
      const uint32_t use = (uint32_t)(e / TC_NST);
      const bool ok = use == 0 || mbar_wait_t(bar_done + 8 * b, (use - 1) & 1u, prof, t_wait);
      if (__any_sync(0xffffffffu, !ok)) return false;  // the warp leaves together
      if (copier) {
        const uint32_t bytes =
            (uint32_t)stage_ksteps<F16>(si.ma, si.mb) * (a.exact ? 32u : 64u) * (uint32_t)N;
        bulk_g2s(sbase + b * stage_bytes, a.B + (size_t)si.pre * 64 * N, bytes, bar_full + 8 * b);
        ncopied = e + 1;
      }
      const uint32_t sA = sbase + b * stage_bytes + bbytes;
#pragma unroll
      for (int i = 0; i < UPT; ++i) {
        const int u = ptid + i * TC_PTHREADS;
        if (u < si.nunits) {
          if (F16) {
            uint32_t h[4], l[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              uint16_t h0, l0, h1, l1;
              f16_split(v[i][2 * c], a.scale_a, h0, l0);
              f16_split(v[i][2 * c + 1], a.scale_a, h1, l1);
              h[c] = (uint32_t)h0 | ((uint32_t)h1 << 16);
              l[c] = (uint32_t)l0 | ((uint32_t)l1 << 16);
            }
            const bool second = u >= F_ROWU;
            const uint32_t off = (second ? (uint32_t)F_IMG : 0u) + 16u * (uint32_t)(second ? u - F_ROWU : u);
            st_shared_v4(sA + off, h[0], h[1], h[2], h[3]);
            if (!a.exact) st_shared_v4(sA + 2 * F_IMG + off, l[0], l[1], l[2], l[3]);
          } else {
            uint32_t h[4], l[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) tf32_split(v[i][c], h[c], l[c]);
            st_shared_v4(sA + 16u * u, h[0], h[1], h[2], h[3]);
            if (!a.exact) st_shared_v4(sA + TC_NQ * 128u + 16u * u, l[0], l[1], l[2], l[3]);
          }
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
        sa = stage_info<F16>(a, s_stage, e + 2, p0);
        stage_load<F16>(a, sa, ptid, va);
      }
      if (e + 1 >= a.nstage) break;
      if (!build(e + 1, sbi, vb)) { fail = 1; break; }
      if (e + 3 < a.nstage) {
        sbi = stage_info<F16>(a, s_stage, e + 3, p0);
        stage_load<F16>(a, sbi, ptid, vb);
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
      // this warp's 16-column chunks are c0 = 16 half + 32 k; two are loaded per wait
      int pbox = -1;
      float a2v = 0.f;
#pragma unroll 1
      for (int c0 = 16 * half; c0 < N; c0 += 64) {
        const bool two = c0 + 32 < N;
        uint32_t r[32];
        if (a.nstage > 0) {
          const uint32_t base = tmem + ((uint32_t)(32 * lq) << 16) + (uint32_t)(mb * N);
          tmem_ld16x2(base + (uint32_t)c0, base + (uint32_t)(two ? c0 + 32 : c0), r);
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) r[j] = 0u;  // no offsets: AB = 0
        }
        // per column: this lane's value, then a transpose-reduction over the warp (after the
        // 5 exchange steps lane c holds the min / max of column c of the group)
        unsigned vmn[32], vmx[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          vmn[j] = 0x7F800000u;
          vmx[j] = 0u;
          if (j >= 16 && !two) continue;
          const int n = j < 16 ? c0 + j : c0 + 16 + j;  // second load: columns c0 + 32..
          float* o = s_out[n];
          if (valid && o) {
            float df;
            if (dis) {
              df = __int_as_float(0x7F800000);
            } else {
              const int bx = s_box[n];
              if (bx != pbox) {  // columns are grouped by mask
                a2v = s_a2[bx * 128 * TC_MB + m];
                pbox = bx;
              }
              const float s2 = __fadd_rn(a2v, s_b2[n]);
              df = fabsf(__fmaf_rn(-a.ab2, __uint_as_float(r[j]), s2));
            }
            o[pout] = df;
            vmn[j] = __float_as_uint(df);
            if (vmn[j] < 0x7F800000u) vmx[j] = vmn[j];
          }
        }
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) {
#pragma unroll
          for (int i = 0; i < d; ++i) {
            const bool up = lane & d;
            const unsigned smn = up ? vmn[i] : vmn[i + d], kmn = up ? vmn[i + d] : vmn[i];
            const unsigned smx = up ? vmx[i] : vmx[i + d], kmx = up ? vmx[i + d] : vmx[i];
            vmn[i] = min(kmn, __shfl_xor_sync(0xffffffffu, smn, d));
            vmx[i] = max(kmx, __shfl_xor_sync(0xffffffffu, smx, d));
          }
        }
        {
          const int j = lane;  // the group's column this lane now holds
          if (j < 16 || two) {
            const int n = j < 16 ? c0 + j : c0 + 16 + j;
            if (s_out[n]) {
              if (vmn[0] != 0x7F800000u) atomicMin(s_mn + n, vmn[0]);
              if (vmx[0] != 0u) atomicMax(s_mx + n, vmx[0]);
            }
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

template <bool F16>
size_t tc_smem_bytes(int N) {
  return (size_t)TC_NST * ((size_t)TC_STEPS * 64 * N + a_region<F16>()) + 32 * (size_t)N +
         4 * IQ_TC_MAXBOX * 128 * TC_MB + 8 * (3 * TC_NST + 1) + 12 * TC_SMW;
}

// [largest magnitude bits, smallest exponent + 256 of a nonzero magnitude, OR of the low 13
// mantissa bits, smallest exponent + 256 of the lowest set bit of a nonzero value] over the
// finite values
__global__ void value_stats_kernel(const float* __restrict__ d, int64_t n, unsigned* out) {
  unsigned amax = 0, minx = 0xFFFFFFFFu, low = 0, lsb = 0xFFFFFFFFu;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned b = __float_as_uint(d[i]) & 0x7FFFFFFFu;
    if (b >= 0x7F800000u) continue;  // NaN, Inf
    amax = max(amax, b);
    if (b) {
      const unsigned ex = b >> 23;  // biased exponent; 0 for subnormals
      minx = min(minx, (ex ? ex : 1u) - 127u + 256u);
      const unsigned sig = ex ? ((b & 0x7FFFFFu) | 0x800000u) : (b & 0x7FFFFFu);
      lsb = min(lsb, (ex ? ex : 1u) + (unsigned)(__ffs(sig) - 1) - 150u + 256u);
    }
    low |= b & 0x1FFFu;
  }
  amax = __reduce_max_sync(0xffffffffu, amax);
  minx = __reduce_min_sync(0xffffffffu, minx);
  low = __reduce_or_sync(0xffffffffu, low);
  lsb = __reduce_min_sync(0xffffffffu, lsb);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, amax);
    atomicMin(out + 1, minx);
    atomicOr(out + 2, low);
    atomicMin(out + 3, lsb);
  }
}

// ---- packing of the templates, FP16 form ----
struct Pack16Args {
  const float* grid;
  int64_t gx, gy, tx;
  const TcCol* cols;
  int N;
  const uint32_t* wa;
  const uint32_t* wb;
  const uint32_t* prefix;
  int nstage;
  TcBox box[IQ_TC_MAXBOX];
  float scale_b;  // 2^-kB
  char* B;
};

// Stage e occupies prefix[e] * 64N bytes: the FP16 high halves of its nks K-steps (32N bytes
// each: chunk half jj = 0..1, template n, 8 halves), then the low halves. K-step t joins the
// stage's active chunks 2t and 2t + 1 (row entry a's chunks first); a missing second chunk
// is zero.
__global__ void tc_pack16_kernel(const Pack16Args p) {
  const int N = p.N;
  for (int e = blockIdx.y; e < p.nstage; e += gridDim.y) {
    const uint32_t wa = p.wa[e], wb = p.wb[e];
    const uint32_t ma = wa >> 26, mb = wb >> 26;
    const int na = __popc(ma), total = na + __popc(mb);
    const int nks = (total + 1) >> 1;
    const int units = nks * 2 * N;
    char* base = p.B + (size_t)p.prefix[e] * 64 * N;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < units; u += gridDim.x * blockDim.x) {
      const int t = u / (2 * N), rem = u - t * 2 * N;
      const int jj = rem / N, n = rem - jj * N;
      const int idx = 2 * t + jj;
      const TcCol col = p.cols[n];
      uint32_t h[4] = {0, 0, 0, 0}, l[4] = {0, 0, 0, 0};
      if (idx < total && col.src >= 0) {
        const bool second = idx >= na;
        const uint32_t w = second ? wb : wa;
        const int c = second ? nth_bit(mb, idx - na) : nth_bit(ma, idx);
        const int ky = (int)(w & 1023u), kz = (int)((w >> 10) & 1023u), g = (int)((w >> 20) & 63u);
        const TcBox bx = p.box[col.box];
        const int64_t kx0 = (int64_t)TC_GROUP * g + 8 * c;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int64_t kx = kx0 + q;
          float v = 0.f;
          if (kx < p.tx && !in_box(bx, kx, ky, kz))
            v = p.grid[col.src + kx + p.gx * (ky + p.gy * (int64_t)kz)];
          uint16_t hh, ll;
          f16_split(v, p.scale_b, hh, ll);
          h[q >> 1] |= (uint32_t)hh << (16 * (q & 1));
          l[q >> 1] |= (uint32_t)ll << (16 * (q & 1));
        }
      }
      uint4* hi = reinterpret_cast<uint4*>(base + (size_t)t * 32 * N + (size_t)rem * 16);
      uint4* lo = reinterpret_cast<uint4*>(base + (size_t)(nks + t) * 32 * N + (size_t)rem * 16);
      *hi = make_uint4(h[0], h[1], h[2], h[3]);
      *lo = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
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
  // FP16 form: consecutive row entries in pairs
  out.w16a.clear();
  out.w16b.clear();
  out.pre16.clear();
  out.nsteps16 = 0;
  for (size_t i = 0; i < out.word.size(); i += 2) {
    const uint32_t wa = out.word[i], wb = i + 1 < out.word.size() ? out.word[i + 1] : 0u;
    out.w16a.push_back(wa);
    out.w16b.push_back(wb);
    out.pre16.push_back((uint32_t)out.nsteps16);
    out.nsteps16 += (__builtin_popcount(wa >> 26) + __builtin_popcount(wb >> 26) + 1) / 2;
  }
}

int IqValueStats::maxexp() const { return amax > 0.f ? std::ilogb(amax) : 0; }
bool IqValueStats::fp16_range() const { return !(amax > 0.f) || minexp >= maxexp() - 17; }

IqValueStats iq_host_stats(const float* v, int64_t n) {
  IqValueStats s;
  for (int64_t i = 0; i < n; ++i) {
    if (!std::isfinite(v[i])) continue;
    const float a = std::fabs(v[i]);
    uint32_t b;
    memcpy(&b, &a, 4);
    s.amax = std::max(s.amax, a);
    if (a > 0.f) {
      s.minexp = std::min(s.minexp, std::max(std::ilogb(a), -126));
      const uint32_t ex = b >> 23;
      const uint32_t sig = ex ? ((b & 0x7FFFFFu) | 0x800000u) : (b & 0x7FFFFFu);
      s.lsbexp = std::min(s.lsbexp, (int)(ex ? ex : 1u) + __builtin_ctz(sig) - 150);
    }
    if (b & 0x1FFFu) s.narrow = false;
  }
  return s;
}

double iq_map_kappa(const IqValueStats& A, const IqValueStats& B, int64_t K, int form) {
  if (K <= 0) return 0.0;  // empty mask: every term is an exact zero
  const double u = std::ldexp(1.0, -24);
  if (!(A.amax > 0.f) || !(B.amax > 0.f)) {
    // one operand is all zeros: AB = 0 and D = A2 + B2, exact when the squares are
    const IqValueStats& Z = A.amax > 0.f ? A : B;
    if (!(Z.amax > 0.f)) return 0.0;
    const double m = (double)K * (double)Z.amax * (double)Z.amax;
    if (Z.narrow && m < std::ldexp(1.0, 24 + 2 * Z.lsbexp)) return 0.0;
  } else if (A.narrow && B.narrow) {
    // products exact (11-bit factors), all sums on the grid 2^g and below 2^(24 + g)
    const int g = 2 * std::min(A.lsbexp, B.lsbexp);
    const double m = (double)K * ((double)A.amax * A.amax + (double)B.amax * B.amax) * 1.001;
    if (m < std::ldexp(1.0, 24 + g)) return 0.0;
  }
  // one MMA adds its products to the FP32 accumulator with a relative error of at most 4u of
  // (|accumulator| + sum |products|); three MMAs per K-step (hi*hi + hi*lo + lo*hi) of 16
  // (FP16) or 8 (TF32) offsets; the SIMT kernel rounds once per fused multiply-add; the split
  // drops 12u |a||b|, the epilogue rounds A2, B2, their sum and the result (4u); and
  // sum |a||b| <= (A2 + B2) / 2
  const double nsteps = form == 1 ? std::ceil(K / 16.0) : form == 2 ? std::ceil(K / 8.0) : 0.0;
  const double acc = form == 0 ? (double)K : 3.0 * nsteps * 4.0;
  return (acc + 12.0 + 4.0 + 8.0) * u * 1.01;
}

double iq_map_eabs(const IqValueStats& A, int64_t n_img) {
  // A2 from a Float64 integral image: each prefix sum of at most n_img squares rounds n_img
  // times, and a box sum combines 8 of them
  const double total = (double)n_img * (double)A.amax * (double)A.amax;
  return 8.0 * (double)n_img * std::ldexp(1.0, -53) * total * 1.01;
}

int iq_value_stats(iq_ctx* ctx, const float* d, int64_t n, IqValueStats& out) {
  out = IqValueStats();
  unsigned* buf = (unsigned*)iq_scratch(ctx, S_TCFLAG, 4 * sizeof(unsigned));
  if (!buf) return IQ_ERR_ALLOC;
  const unsigned init[4] = {0u, 0xFFFFFFFFu, 0u, 0xFFFFFFFFu};
  IQ_CUDA_OK(cudaMemcpyAsync(buf, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
  if (n > 0) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    value_stats_kernel<<<blocks, 256, 0, ctx->stream>>>(d, n, buf);
    iq_count(ctx);
    IQ_CUDA_OK(cudaGetLastError());
  }
  unsigned h[4];
  IQ_CUDA_OK(cudaMemcpyAsync(h, buf, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  memcpy(&out.amax, &h[0], 4);
  out.minexp = h[1] == 0xFFFFFFFFu ? (1 << 30) : (int)h[1] - 256;
  out.narrow = h[2] == 0u;
  out.lsbexp = h[3] == 0xFFFFFFFFu ? (1 << 30) : (int)h[3] - 256;
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
  // FP16 halves when both operands' ranges allow them (engine 2), else TF32 halves; one MMA
  // per K-step when every value has at most 11 significant bits
  const bool f16 = ctx->corr_engine == 2 && L.stage16 && L.img_stats.fp16_range() &&
                   L.tmpl_stats.fp16_range();
  const bool exact = L.img_stats.narrow && L.tmpl_stats.narrow;
  const int ka = f16 && L.img_stats.amax > 0.f ? L.img_stats.maxexp() - 14 : 0;
  const int kb = f16 && L.tmpl_stats.amax > 0.f ? L.tmpl_stats.maxexp() - 14 : 0;
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
  const int nstage = f16 ? L.nstage16 : L.nstage;
  const int64_t nsteps = f16 ? L.nsteps16 : L.nsteps;
  if (f16) {
    a.word = L.stage16;
    a.wordb = L.stage16 + L.nstage16;
    a.prefix = L.stage16 + 2 * L.nstage16;
  } else {
    a.word = L.stage_word;
    a.wordb = nullptr;
    a.prefix = L.stage_prefix;
  }
  a.nstage = nstage;
  a.B = (const char*)L.B;
  a.cols = L.cols;
  a.N = L.N;
  a.exact = exact ? 1 : 0;
  a.scale_a = std::ldexp(1.f, -ka);
  a.ab2 = std::ldexp(1.f, ka + kb + 1);
  uint32_t tc = 32;
  while (tc < (uint32_t)(TC_MB * L.N)) tc <<= 1;
  a.tmem_cols = tc;
  a.status = ctx->d_status;
  a.stats = ctx->prof ? ctx->d_stats : nullptr;

  iq_timer_start(ctx, "corr");
  if (nstage > 0) {  // no stages: every column's mask is empty and its products are zero
    const dim3 grid((unsigned)((TC_STEPS * 2 * L.N + 255) / 256), (unsigned)std::min(nstage, 65535));
    if (f16) {
      Pack16Args p;
      p.grid = L.grid; p.gx = L.grid_dims.x; p.gy = L.grid_dims.y; p.tx = L.tile.x;
      p.cols = L.cols; p.N = L.N;
      p.wa = a.word; p.wb = a.wordb; p.prefix = a.prefix; p.nstage = nstage;
      for (int b = 0; b < IQ_TC_MAXBOX; ++b) p.box[b] = L.box[b];
      p.scale_b = std::ldexp(1.f, -kb);
      p.B = (char*)L.B;
      tc_pack16_kernel<<<grid, 256, 0, ctx->stream>>>(p);
    } else {
      PackArgs p;
      p.grid = L.grid; p.gx = L.grid_dims.x; p.gy = L.grid_dims.y; p.tx = L.tile.x;
      p.cols = L.cols; p.N = L.N;
      p.word = L.stage_word; p.prefix = L.stage_prefix; p.nstage = nstage;
      for (int b = 0; b < IQ_TC_MAXBOX; ++b) p.box[b] = L.box[b];
      p.B = (char*)L.B;
      tc_pack_kernel<<<grid, 256, 0, ctx->stream>>>(p);
    }
    iq_count(ctx);
    IQ_CUDA_OK(cudaGetLastError());
  }
  const size_t smem = f16 ? tc_smem_bytes<true>(L.N) : tc_smem_bytes<false>(L.N);
  auto kern = f16 ? corr_tc_kernel<true> : corr_tc_kernel<false>;
  IQ_CUDA_OK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t nblk = od.z * bpp;
  if (ctx->prof) {
    const double fl = 2.0 * (double)nblk * 128 * TC_MB * (double)nsteps * (f16 ? 16 : 8) * L.N *
                      (exact ? 1 : 3);
    ctx->prof_mma_flops += fl;
    if (f16) ctx->prof_mma_flops16 += fl;
    ctx->prof_mma_launches += 1;
    ctx->prof_tc_cols += L.N;
  }
  kern<<<(unsigned)nblk, TC_THREADS, smem, ctx->stream>>>(a);
  iq_count(ctx);
  iq_timer_stop(ctx, "corr", L.flops);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
