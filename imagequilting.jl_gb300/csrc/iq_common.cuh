// Shared definitions of the GB300 image-quilting library (libiqgpu.so).
//
// Layout conventions (same as the Julia reference, which is column-major):
//   * every grid is handled as 3-D (nx, ny, nz); 1-D and 2-D inputs get unit trailing extents;
//   * linear index = x + nx * (y + ny * z), 0-based;
//   * distance maps have the "valid" extent TIsize - tilesize + 1 (src/iqsim.jl:112).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/iqgpu.h"

#define IQ_HD __host__ __device__ __forceinline__

// Largest number of auxiliary distance sources a pick handles (ovl + soft variables).
#define IQ_MAX_AUX 7
// Length limit of the relaxation softdbsize sequence (frac grows by 0.1 up to 1).
#define IQ_MAX_SEQ 24
// Chunk length of the canonical summation order of the weighted draw.
#define IQ_DRAW_CHUNK 256

struct Dim3 {
  int64_t x, y, z;
  IQ_HD int64_t vol() const { return x * y * z; }
  IQ_HD int64_t lin(int64_t i, int64_t j, int64_t k) const { return i + x * (j + y * k); }
};

// ---------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). Streams (seed is the 64-bit key):
//   weighted draw of realization r at tile t : counter (t, r, 1, 0)
//   i-th integer of path generation          : counter (i, 0, 2, 0)
// The 64-bit value of a block is (x1 << 32) | x0.
// ---------------------------------------------------------------------------------------
IQ_HD void iq_philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += W0;
      k1 += W1;
    }
    uint64_t p0 = (uint64_t)M0 * c[0];
    uint64_t p1 = (uint64_t)M1 * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

IQ_HD uint64_t iq_rand64(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2) {
  uint32_t c[4] = {c0, c1, c2, 0u};
  iq_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return ((uint64_t)c[1] << 32) | c[0];
}

// u in [0,1) of the weighted draw: top 53 bits times 2^-53.
IQ_HD double iq_draw_uniform(uint64_t seed, int64_t tile, int64_t real) {
  uint64_t v = iq_rand64(seed, (uint32_t)tile, (uint32_t)real, 1u);
  return (double)(v >> 11) * (1.0 / 9007199254740992.0);
}

// Ordered bits of a non-negative float (NaN excluded): unsigned compare == float compare.
IQ_HD uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  union { float f; uint32_t u; } x; x.f = f; return x.u;
#endif
}

#define IQ_CUDA_OK(call)                                                              \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      iq_set_error(IQ_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,            \
                   cudaGetErrorString(e_));                                           \
      return IQ_ERR_CUDA;                                                             \
    }                                                                                 \
  } while (0)

// error reporting (iq_abi.cu): sets the thread-local message returned by iq_last_error
int iq_set_error(int code, const char* fmt, ...);

// Device status codes written by kernels (first error wins).
__device__ __forceinline__ void iq_dev_fail(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}
