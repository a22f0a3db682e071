// Distance maps of the quilting path (src/utils.jl:5-13, src/imfilter.jl:5-28).
//
// D[t][p] = |A2(p) - 2 * AB[t][p] + B2[t]| for a batch of templates t that share one mask:
//   * AB[t][p] = sum_k TI[p + k] * (w_k S_t[k]) is a batched masked cross-correlation, summed
//     directly (the reference uses FFTs): one thread owns PJ positions x RT templates in
//     registers, the template values of a chunk of offsets sit in shared memory and are read
//     as broadcasts, and the TI is read through L1 (its windows overlap heavily);
//   * A2(p) = sum_k w_k TI[p + k]^2 comes from a Float64 integral image when the mask is the
//     tile minus an inner box (overlap masks, unmasked soft data), or is summed in the same
//     loop for arbitrary masks (hard data);
//   * B2[t] = sum_k (w_k S_t[k])^2 in Float64.
// Windows that cover an inactive TI voxel get +Inf (src/iqsim.jl:207). The epilogue also
// folds each template's minimum and largest finite value into two atomics for the pick.
#include <float.h>

#include <algorithm>

#include "iq_internal.h"

namespace {

constexpr int CORR_THREADS = 128;
constexpr int CORR_KC = 128;  // offsets per shared-memory chunk

struct CorrArgs {
  const float* img;
  int64_t ix, iy;             // image extents (x, y)
  int64_t dx, dy, P;          // valid extents and their product
  int rpad, ntmpl;
  int64_t tx, ty, tz;         // tile
  const uint8_t* disabled;
  int64_t out_stride;
  CorrTask t0;                // used when tasks is null
  const CorrTask* tasks;      // one task per blockIdx.z
};

template <int RT, int PJ, int MINB>
__global__ void __launch_bounds__(CORR_THREADS, MINB) corr_kernel(const CorrArgs a) {
  __shared__ int32_t s_off[CORR_KC];
  __shared__ __align__(16) float s_tv[CORR_KC * RT];
  __shared__ unsigned s_min[CORR_THREADS / 32][RT], s_max[CORR_THREADS / 32][RT];

  const int tid = threadIdx.x;
  const int rg = blockIdx.y;
  const CorrTask t = a.tasks ? a.tasks[blockIdx.z] : a.t0;
  const bool direct = t.ii == nullptr;
  const int64_t pbase = (int64_t)blockIdx.x * (CORR_THREADS * PJ);

  const float* ptr[PJ];
  int64_t pos[PJ];
#pragma unroll
  for (int j = 0; j < PJ; ++j) {
    int64_t p = pbase + tid + (int64_t)j * CORR_THREADS;
    pos[j] = p;
    int64_t pc = p < a.P ? p : a.P - 1;
    int64_t x = pc % a.dx, row = pc / a.dx;
    int64_t y = row % a.dy, z = row / a.dy;
    ptr[j] = a.img + (x + a.ix * (y + a.iy * z));
  }

  float acc[PJ][RT];
  float a2d[PJ];
#pragma unroll
  for (int j = 0; j < PJ; ++j) {
    a2d[j] = 0.f;
#pragma unroll
    for (int r = 0; r < RT; ++r) acc[j][r] = 0.f;
  }

  for (int kc0 = 0; kc0 < t.K; kc0 += CORR_KC) {
    const int nk = min(CORR_KC, t.K - kc0);
    __syncthreads();
    for (int i = tid; i < nk; i += CORR_THREADS) {
      uint32_t k = t.klist[kc0 + i];
      s_off[i] = (int32_t)(kx_of(k) + a.ix * (ky_of(k) + a.iy * (int64_t)kz_of(k)));
    }
    for (int i = tid; i < nk * RT; i += CORR_THREADS) {
      int kk = i / RT, r = i % RT;
      s_tv[i] = t.tv[(int64_t)(kc0 + kk) * a.rpad + rg * RT + r];
    }
    __syncthreads();
#pragma unroll 2
    for (int i = 0; i < nk; ++i) {
      const int off = s_off[i];
      float t[RT];
      if constexpr (RT % 4 == 0) {
#pragma unroll
        for (int r4 = 0; r4 < RT / 4; ++r4) {
          float4 q = reinterpret_cast<const float4*>(s_tv + i * RT)[r4];
          t[4 * r4 + 0] = q.x; t[4 * r4 + 1] = q.y; t[4 * r4 + 2] = q.z; t[4 * r4 + 3] = q.w;
        }
      } else {
#pragma unroll
        for (int r = 0; r < RT; ++r) t[r] = s_tv[i * RT + r];
      }
#pragma unroll
      for (int j = 0; j < PJ; ++j) {
        const float v = __ldg(ptr[j] + off);
#pragma unroll
        for (int r = 0; r < RT; ++r) acc[j][r] = fmaf(v, t[r], acc[j][r]);
        if (direct) a2d[j] = fmaf(v, v, a2d[j]);
      }
    }
  }

  // epilogue
  unsigned mn[RT], mx[RT];
#pragma unroll
  for (int r = 0; r < RT; ++r) { mn[r] = 0x7F800000u; mx[r] = 0u; }
  const int64_t sx = a.ix + 1, sxy = (a.ix + 1) * (a.iy + 1);
  const bool inner = t.hi[0] > t.lo[0] && t.hi[1] > t.lo[1] && t.hi[2] > t.lo[2];
#pragma unroll
  for (int j = 0; j < PJ; ++j) {
    const int64_t p = pos[j];
    if (p >= a.P) continue;
    double A2;
    if (direct) {
      A2 = (double)a2d[j];
    } else {
      int64_t x = p % a.dx, row = p / a.dx;
      int64_t y = row % a.dy, z = row / a.dy;
      A2 = iq_box_sum(t.ii, sx, sxy, x, y, z, a.tx, a.ty, a.tz);
      if (inner)
        A2 -= iq_box_sum(t.ii, sx, sxy, x + t.lo[0], y + t.lo[1], z + t.lo[2], t.hi[0] - t.lo[0],
                      t.hi[1] - t.lo[1], t.hi[2] - t.lo[2]);
    }
    const bool dis = a.disabled != nullptr && a.disabled[p];
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      const int tt = rg * RT + r;
      if (tt >= a.ntmpl) continue;
      float df;
      if (dis) {
        df = __int_as_float(0x7F800000);
      } else {
        double d = A2 - 2.0 * (double)acc[j][r] + t.b2[tt];
        df = (float)fabs(d);
      }
      t.out[(int64_t)tt * a.out_stride + p] = df;
      unsigned b = __float_as_uint(df);
      mn[r] = min(mn[r], b);
      if (b < 0x7F800000u) mx[r] = max(mx[r], b);
    }
  }
  if (t.minmax == nullptr) return;
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int r = 0; r < RT; ++r) {
    unsigned m1 = __reduce_min_sync(0xffffffffu, mn[r]);
    unsigned m2 = __reduce_max_sync(0xffffffffu, mx[r]);
    if (lane == 0) { s_min[warp][r] = m1; s_max[warp][r] = m2; }
  }
  __syncthreads();
  if (tid < RT) {
    const int tt = rg * RT + tid;
    if (tt < a.ntmpl) {
      unsigned m1 = 0x7F800000u, m2 = 0u;
      for (int w = 0; w < CORR_THREADS / 32; ++w) {
        m1 = min(m1, s_min[w][tid]);
        m2 = max(m2, s_max[w][tid]);
      }
      atomicMin(t.minmax + 2 * tt, m1);
      atomicMax(t.minmax + 2 * tt + 1, m2);
    }
  }
}

template <int RT, int PJ, int MINB = 1>
void launch_corr_t(const CorrArgs& a, int ntask, cudaStream_t s) {
  dim3 grid((unsigned)((a.P + CORR_THREADS * PJ - 1) / (CORR_THREADS * PJ)),
            (unsigned)(a.rpad / RT), (unsigned)ntask);
  corr_kernel<RT, PJ, MINB><<<grid, CORR_THREADS, 0, s>>>(a);
}

// ---- gather of template values --------------------------------------------------------
struct GatherArgs {
  const float* grid;
  int64_t gx, gy;
  int64_t gstride;
  const int64_t* starts;
  int ntmpl, rpad;
  GatherTask t0;
  const GatherTask* tasks;
};

__global__ void gather_kernel(const GatherArgs g) {
  const int t = blockIdx.x;  // template (rpad blocks)
  const GatherTask k = g.tasks ? g.tasks[blockIdx.y] : g.t0;
  __shared__ double s_red[32];
  double sq = 0.0;
  if (t < g.ntmpl) {
    const int64_t st = g.starts ? g.starts[t] : k.start;
    const float* base = g.grid ? g.grid + (int64_t)t * g.gstride + st : nullptr;
    for (int i = threadIdx.x; i < k.K; i += blockDim.x) {
      float v;
      if (k.kval) {
        v = k.kval[i];
      } else {
        uint32_t kk = k.klist[i];
        v = base[kx_of(kk) + g.gx * (ky_of(kk) + g.gy * (int64_t)kz_of(kk))];
      }
      if (k.tv) k.tv[(int64_t)i * g.rpad + t] = v;
      sq += (double)v * (double)v;
    }
  } else if (k.tv) {
    for (int i = threadIdx.x; i < k.K; i += blockDim.x) k.tv[(int64_t)i * g.rpad + t] = 0.f;
  }
  // block reduction of the squares (fixed order: warp shuffles then warps in order)
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = sq;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += s_red[w];
    k.b2[t] = t < g.ntmpl ? s : 0.0;
    if (k.minmax && t < g.ntmpl) {
      k.minmax[2 * t] = 0x7F800000u;
      k.minmax[2 * t + 1] = 0u;
    }
  }
}

// ---- integral images -----------------------------------------------------------------
template <typename T>
__global__ void ii_fill_kernel(const float* __restrict__ img, const uint8_t* __restrict__ nan,
                               int64_t nx, int64_t ny, int64_t nz, T* __restrict__ ii, int mode) {
  // mode 0: v^2, mode 1: nan indicator, mode 2: v; writes the (x+1, y+1, z+1) cell
  const int64_t n = nx * ny * nz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t x = i % nx, r = i / nx, y = r % ny, z = r / ny;
    T v;
    if (mode == 0) {
      double f = (double)img[i];
      v = (T)(f * f);
    } else if (mode == 2) {
      v = (T)img[i];
    } else {
      v = (T)(nan[i] ? 1 : 0);
    }
    ii[(x + 1) + (nx + 1) * ((y + 1) + (ny + 1) * (z + 1))] = v;
  }
}

template <typename T>
__global__ void ii_scan_kernel(T* __restrict__ ii, int64_t sx, int64_t sy, int64_t sz, int axis) {
  // inclusive scan along `axis` of an (sx, sy, sz) array, one thread per line
  int64_t nlines, len, step;
  if (axis == 0) { nlines = sy * sz; len = sx; step = 1; }
  else if (axis == 1) { nlines = sx * sz; len = sy; step = sx; }
  else { nlines = sx * sy; len = sz; step = sx * sy; }
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nlines;
       l += (int64_t)gridDim.x * blockDim.x) {
    int64_t base;
    if (axis == 0) base = l * sx;
    else if (axis == 1) base = (l % sx) + sx * sy * (l / sx);
    else base = l;
    T run = 0;
    for (int64_t i = 0; i < len; ++i) {
      run += ii[base + i * step];
      ii[base + i * step] = run;
    }
  }
}

__global__ void disabled_kernel(const int32_t* __restrict__ ii, int64_t ix, int64_t iy,
                                int64_t dx, int64_t dy, int64_t P, int64_t tx, int64_t ty,
                                int64_t tz, uint8_t* __restrict__ out) {
  const int64_t sx = ix + 1, sxy = (ix + 1) * (iy + 1);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t x = p % dx, r = p / dx, y = r % dy, z = r / dy;
    const int64_t x1 = x + tx, y1 = y + ty, z1 = z + tz;
    int64_t s = (int64_t)ii[x1 + sx * y1 + sxy * z1] - ii[x + sx * y1 + sxy * z1] -
                ii[x1 + sx * y + sxy * z1] + ii[x + sx * y + sxy * z1] -
                ii[x1 + sx * y1 + sxy * z] + ii[x + sx * y1 + sxy * z] +
                ii[x1 + sx * y + sxy * z] - ii[x + sx * y + sxy * z];
    out[p] = s > 0 ? 1 : 0;
  }
}

}  // namespace

int iq_register_tile(int ntmpl) {
  if (ntmpl >= 16) return 16;
  if (ntmpl > 4) return 8;
  if (ntmpl > 2) return 4;
  if (ntmpl > 1) return 2;
  return 1;
}

int iq_launch_corr(iq_ctx* ctx, const CorrLaunch& L) {
  CorrArgs a;
  a.img = L.img;
  a.ix = L.img_dims.x;
  a.iy = L.img_dims.y;
  a.dx = L.out_dims.x;
  a.dy = L.out_dims.y;
  a.P = L.out_dims.vol();
  a.rpad = L.rpad;
  a.ntmpl = L.ntmpl;
  a.tx = L.tile.x; a.ty = L.tile.y; a.tz = L.tile.z;
  a.disabled = L.disabled;
  a.out_stride = L.out_stride;
  a.t0 = L.t0;
  a.tasks = L.tasks;
  if (a.P <= 0 || L.ntmpl <= 0 || L.ntask <= 0) return IQ_OK;
  const int rt = iq_register_tile(L.rpad);
  iq_timer_start(ctx, "corr");
  switch (rt) {
    case 16:
      // launch shapes of the 16-template tile (register budget vs positions per thread)
      switch (ctx->corr_variant) {
        case 1: launch_corr_t<16, 4, 3>(a, L.ntask, ctx->stream); break;
        case 2: launch_corr_t<16, 8, 2>(a, L.ntask, ctx->stream); break;
        case 3: launch_corr_t<16, 2, 4>(a, L.ntask, ctx->stream); break;
        default: launch_corr_t<16, 4>(a, L.ntask, ctx->stream); break;
      }
      break;
    case 8: launch_corr_t<8, 4>(a, L.ntask, ctx->stream); break;
    case 4: launch_corr_t<4, 8>(a, L.ntask, ctx->stream); break;
    case 2: launch_corr_t<2, 8>(a, L.ntask, ctx->stream); break;
    default: launch_corr_t<1, 8>(a, L.ntask, ctx->stream); break;
  }
  const double flops = L.flops > 0 ? L.flops
                                   : 2.0 * (double)a.P * (double)L.t0.K * (double)L.ntmpl;
  iq_timer_stop(ctx, "corr", flops);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_gather(iq_ctx* ctx, const GatherLaunch& G) {
  if (G.ntask <= 0) return IQ_OK;
  GatherArgs g;
  g.grid = G.grid;
  g.gx = G.grid_dims.x;
  g.gy = G.grid_dims.y;
  g.gstride = G.grid_stride;
  g.starts = G.starts;
  g.ntmpl = G.ntmpl;
  g.rpad = G.rpad;
  g.t0 = G.t0;
  g.tasks = G.tasks;
  dim3 grid((unsigned)G.rpad, (unsigned)G.ntask);
  gather_kernel<<<grid, 256, 0, ctx->stream>>>(g);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_build_value_integral(iq_ctx* ctx, const float* d_img, Dim3 dims, double* d_ii) {
  const int64_t sx = dims.x + 1, sy = dims.y + 1, sz = dims.z + 1;
  const int64_t n = dims.vol();
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  IQ_CUDA_OK(cudaMemsetAsync(d_ii, 0, sizeof(double) * sx * sy * sz, ctx->stream));
  ii_fill_kernel<double><<<blocks, 256, 0, ctx->stream>>>(d_img, nullptr, dims.x, dims.y, dims.z,
                                                         d_ii, 2);
  iq_count(ctx, 4);
  for (int ax = 0; ax < 3; ++ax) {
    const int64_t nl = ax == 0 ? sy * sz : ax == 1 ? sx * sz : sx * sy;
    ii_scan_kernel<double><<<(int)((nl + 127) / 128), 128, 0, ctx->stream>>>(d_ii, sx, sy, sz, ax);
  }
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_build_integrals(iq_ctx* ctx, const float* d_img, Dim3 dims, double* d_sqii,
                       int32_t* d_nanii, const uint8_t* d_nan) {
  const int64_t sx = dims.x + 1, sy = dims.y + 1, sz = dims.z + 1;
  const int64_t n = dims.vol();
  const int threads = 256;
  const int blocks = (int)std::min<int64_t>((n + threads - 1) / threads, 4096);
  if (d_sqii) {
    IQ_CUDA_OK(cudaMemsetAsync(d_sqii, 0, sizeof(double) * sx * sy * sz, ctx->stream));
    ii_fill_kernel<double><<<blocks, threads, 0, ctx->stream>>>(d_img, nullptr, dims.x, dims.y,
                                                                dims.z, d_sqii, 0);
    iq_count(ctx, 4);
    for (int ax = 0; ax < 3; ++ax) {
      int64_t nl = ax == 0 ? sy * sz : ax == 1 ? sx * sz : sx * sy;
      ii_scan_kernel<double><<<(int)((nl + 127) / 128), 128, 0, ctx->stream>>>(d_sqii, sx, sy,
                                                                              sz, ax);
    }
  }
  if (d_nanii) {
    IQ_CUDA_OK(cudaMemsetAsync(d_nanii, 0, sizeof(int32_t) * sx * sy * sz, ctx->stream));
    ii_fill_kernel<int32_t><<<blocks, threads, 0, ctx->stream>>>(nullptr, d_nan, dims.x, dims.y,
                                                                 dims.z, d_nanii, 1);
    iq_count(ctx, 4);
    for (int ax = 0; ax < 3; ++ax) {
      int64_t nl = ax == 0 ? sy * sz : ax == 1 ? sx * sz : sx * sy;
      ii_scan_kernel<int32_t><<<(int)((nl + 127) / 128), 128, 0, ctx->stream>>>(d_nanii, sx, sy,
                                                                               sz, ax);
    }
  }
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}

int iq_launch_disabled(iq_ctx* ctx, const int32_t* d_nanii, Dim3 dims, Dim3 tile, uint8_t* out) {
  Dim3 od{dims.x - tile.x + 1, dims.y - tile.y + 1, dims.z - tile.z + 1};
  const int64_t P = od.vol();
  if (P <= 0) return IQ_OK;
  const int blocks = (int)std::min<int64_t>((P + 255) / 256, 4096);
  disabled_kernel<<<blocks, 256, 0, ctx->stream>>>(d_nanii, dims.x, dims.y, od.x, od.y, P, tile.x,
                                                   tile.y, tile.z, out);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
