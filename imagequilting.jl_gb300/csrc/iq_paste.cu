// Paste of the drawn pattern and the per-realization finishing steps.
//   paste           simdev[.!cutmask] = TIdev[.!cutmask]          src/iqsim.jl:277-281
//   voxel reuse     sum(cutgrid) / ovlvol                          src/iqsim.jl:287-288
//   hard overwrite  simgrid[coord] = val (NaN too), cut NaN        src/iqsim.jl:290-300
//   crop            view(simgrid, CartesianIndices(simsize))      src/iqsim.jl:302-304
//   soft padding    padarray(aux, Pad(:symmetric, 0, append))      src/utils.jl:74-79
//   prepare         NaN -> 0                                       src/utils.jl:96-102
#include "iq_internal.h"

namespace {

struct PasteArgs {
  int nreal;
  StepTask t0;
  const StepTask* tasks;
  float* sim; int64_t sx, sy, srs;
  float* cut;
  int64_t tx, ty, tz;
  const float* ti; int64_t tix, tiy; int64_t dx, dy;
  const int64_t* rind;
  const uint8_t* cutbuf; int64_t slabmax;
};

// CTA row y: realization y % nreal of task y / nreal.
__global__ void paste_kernel(const PasteArgs a) {
  const int y = blockIdx.y;
  const int r = y % a.nreal;
  const StepTask& tk = a.tasks ? a.tasks[y / a.nreal] : a.t0;
  const int64_t T = a.tx * a.ty * a.tz;
  const int64_t ri = a.rind[y];
  if (ri < 0) return;
  const int64_t rx = ri % a.dx, rr = ri / a.dx, ry = rr % a.dy, rz = rr / a.dy;
  const int64_t bstart = rx + a.tix * (ry + a.tiy * rz);
  const int nslab = tk.nslab;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < T;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t kx = k % a.tx, kr = k / a.tx, ky = kr % a.ty, kz = kr / a.ty;
    bool keep = false;
    for (int s = 0; s < nslab; ++s) {
      const CutSlab& sl = tk.slab[s];
      const int64_t lx = kx - sl.off[0], ly = ky - sl.off[1], lz = kz - sl.off[2];
      if (lx < 0 || ly < 0 || lz < 0 || lx >= sl.ext[0] || ly >= sl.ext[1] || lz >= sl.ext[2])
        continue;
      const int64_t loc = lx + sl.ext[0] * (ly + sl.ext[1] * lz);
      keep |= a.cutbuf[((int64_t)y * 6 + s) * a.slabmax + loc] != 0;
    }
    const int64_t si = (int64_t)r * a.srs + tk.start + kx + a.sx * (ky + a.sy * kz);
    if (!keep) a.sim[si] = a.ti[bstart + kx + a.tix * (ky + a.tiy * kz)];
    if (a.cut) a.cut[si] = keep ? 1.f : 0.f;
  }
}

__global__ void hard_kernel(int nreal, float* sim, float* cut, int64_t srs, int64_t n,
                            const int64_t* lin, const float* val) {
  const int r = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = val[i];
    sim[(int64_t)r * srs + lin[i]] = v;
    if (cut && isnan(v)) cut[(int64_t)r * srs + lin[i]] = v;
  }
}

__global__ void crop_kernel(const float* src, int64_t sx, int64_t sy, int64_t srs, int64_t ox,
                            int64_t oy, int64_t oz, float* dst) {
  const int r = blockIdx.y;
  const int64_t n = ox * oy * oz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = i % ox, q = i / ox, y = q % oy, z = q / oy;
    dst[(int64_t)r * n + i] = src[(int64_t)r * srs + x + sx * (y + sy * z)];
  }
}

__global__ void voxsum_kernel(const float* cut, int64_t n, int64_t rs, double* out) {
  const int r = blockIdx.x;
  __shared__ unsigned long long s[32];
  unsigned long long c = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    c += cut[(int64_t)r * rs + i] == 1.f ? 1ull : 0ull;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
    out[r] = (double)t;
  }
}

__device__ __forceinline__ int64_t mirror(int64_t i, int64_t n) {
  const int64_t m = i % (2 * n);
  return m < n ? m : 2 * n - 1 - m;
}

__global__ void pad_kernel(const float* src, int64_t sx, int64_t sy, int64_t sz, float* dst,
                           int64_t dx, int64_t dy, int64_t dz) {
  const int64_t n = dx * dy * dz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = i % dx, q = i / dx, y = q % dy, z = q / dy;
    float v = src[mirror(x, sx) + sx * (mirror(y, sy) + sy * mirror(z, sz))];
    dst[i] = isnan(v) ? 0.f : v;
  }
}

// splitmix64 finalizer
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// NaN -> 0 with the NaN mask; `hash` (nullable) accumulates sum_i mix64(bits_i + i * phi), a
// content key of the values as given (independent of the summation order).
__global__ void prepare_kernel(float* data, int64_t n, uint8_t* nanmask, unsigned long long* hash) {
  unsigned long long h = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = data[i];
    h += mix64((unsigned long long)__float_as_uint(v) + (unsigned long long)i * 0x9E3779B97F4A7C15ull);
    const bool isn = isnan(v);
    if (nanmask) nanmask[i] = isn ? 1 : 0;
    if (isn) data[i] = 0.f;
  }
  if (hash) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(hash, h);
  }
}

__global__ void to_f32_kernel(const double* src, float* dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

inline unsigned blocks_for(int64_t n, int threads = 256, int64_t cap = 8192) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)(b > cap ? cap : b);
}

}  // namespace

int iq_launch_paste(iq_ctx* ctx, const PasteLaunch& L) {
  if (L.ntask <= 0 || L.nreal <= 0) return IQ_OK;
  PasteArgs a;
  a.nreal = L.nreal;
  a.t0 = L.t0;
  a.tasks = L.tasks;
  a.sim = L.sim; a.sx = L.sim_dims.x; a.sy = L.sim_dims.y; a.srs = L.sim_rstride;
  a.cut = L.cut;
  a.tx = L.tile.x; a.ty = L.tile.y; a.tz = L.tile.z;
  a.ti = L.ti; a.tix = L.ti_dims.x; a.tiy = L.ti_dims.y;
  a.dx = L.dist_dims.x; a.dy = L.dist_dims.y;
  a.rind = L.rind;
  a.cutbuf = L.cutbuf; a.slabmax = L.slabmax;
  dim3 grid(blocks_for(L.tile.vol(), 256, 64), (unsigned)(L.ntask * L.nreal));
  iq_timer_start(ctx, "paste");
  paste_kernel<<<grid, 256, 0, ctx->stream>>>(a);
  iq_timer_stop(ctx, "paste", 4.0 * (double)L.tile.vol() * L.nreal * L.ntask);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_hard_overwrite(iq_ctx* ctx, int nreal, float* sim, float* cut, Dim3,
                             int64_t sim_rstride, int64_t n, const int64_t* lin,
                             const float* val) {
  if (n <= 0) return IQ_OK;
  dim3 grid(blocks_for(n, 256, 1024), (unsigned)nreal);
  hard_kernel<<<grid, 256, 0, ctx->stream>>>(nreal, sim, cut, sim_rstride, n, lin, val);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_crop(iq_ctx* ctx, int nreal, const float* src, Dim3 src_dims, int64_t src_rstride,
                   Dim3 out_dims, float* dst) {
  dim3 grid(blocks_for(out_dims.vol(), 256, 4096), (unsigned)nreal);
  crop_kernel<<<grid, 256, 0, ctx->stream>>>(src, src_dims.x, src_dims.y, src_rstride,
                                             out_dims.x, out_dims.y, out_dims.z, dst);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_voxsum(iq_ctx* ctx, int nreal, const float* cut, int64_t n, int64_t rstride,
                     double* out) {
  voxsum_kernel<<<nreal, 1024, 0, ctx->stream>>>(cut, n, rstride, out);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_pad_symmetric(iq_ctx* ctx, const float* src, Dim3 src_dims, float* dst,
                            Dim3 dst_dims) {
  pad_kernel<<<blocks_for(dst_dims.vol()), 256, 0, ctx->stream>>>(
      src, src_dims.x, src_dims.y, src_dims.z, dst, dst_dims.x, dst_dims.y, dst_dims.z);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_prepare(iq_ctx* ctx, float* data, int64_t n, uint8_t* nanmask,
                      unsigned long long* hash) {
  prepare_kernel<<<blocks_for(n), 256, 0, ctx->stream>>>(data, n, nanmask, hash);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_to_f32(iq_ctx* ctx, const double* src, float* dst, int64_t n) {
  to_f32_kernel<<<blocks_for(n), 256, 0, ctx->stream>>>(src, dst, n);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
