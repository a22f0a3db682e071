// iq_pick_noalloc: the pattern pick of iq_pick for callers that cannot allocate device memory.
//
// Some hosts cannot call cudaMalloc from the code that drives this library: a framework whose
// device memory is owned by its own pool allocator and must not be fragmented from outside,
// or a latency-bound loop that cannot afford the device-wide synchronization a cudaMalloc
// may cause. This entry point allocates nothing: its scratch (the copies of the distance
// maps, the candidate list, the sort and weight buffers) lives in one file-scope __device__
// array, NOALLOC_BYTES bytes, that every GPU loading the library keeps until the process
// exits. It accepts at most NOALLOC_MAX_P positions and NOALLOC_MAX_AUX auxiliary maps.
//
// Set-up: the first call on a device (with that device current) looks up the array's
// device address with cudaGetSymbolAddress; make that first call before any stream capture.
// All calls share the array and it keeps the last call's contents; calls whose work overlaps
// on the GPU (other streams, other host threads) race on it and must be serialized by the
// caller.
#include <mutex>

#include "iq_internal.h"

namespace {

constexpr int64_t NOALLOC_MAX_P = 1 << 18;  // positions of a distance map
constexpr int NOALLOC_MAX_AUX = 3;          // auxiliary distance maps

// byte layout of the array
constexpr size_t OFF_SRC = 0;                                          // (1 + aux) x P floats
constexpr size_t OFF_CAND = OFF_SRC + 4 * (1 + NOALLOC_MAX_AUX) * NOALLOC_MAX_P;  // P int32
constexpr size_t OFF_K0 = OFF_CAND + 4 * NOALLOC_MAX_P;                // 4 x P uint32
constexpr size_t OFF_W = OFF_K0 + 16 * NOALLOC_MAX_P;                  // P doubles
constexpr size_t OFF_PROD = OFF_W + 8 * NOALLOC_MAX_P;                 // P doubles
constexpr size_t OFF_SMALL = OFF_PROD + 8 * NOALLOC_MAX_P;             // counters, outputs
constexpr size_t NOALLOC_BYTES = OFF_SMALL + 256;

// small region: [0..2*(1+aux)) min/max bits per source, then npat, rind, ncand, status
struct Small {
  unsigned mm[2 * (1 + NOALLOC_MAX_AUX)];
  unsigned long long npat;
  int64_t rind;
  int64_t ncand;
  int status;
};
static_assert(sizeof(Small) <= 256, "small region");

static __device__ __align__(256) unsigned char g_pick_scratch[NOALLOC_BYTES];

std::mutex g_mu;
void* g_ptr[64] = {};  // device address of g_pick_scratch, per device

// Min bits, largest finite bits of each source and the count of finite entries of source 0.
__global__ void noalloc_minmax_kernel(const float* src, int64_t P, int nsrc, Small* sm) {
  for (int j = 0; j < nsrc; ++j) {
    unsigned mn = 0x7F800000u, mx = 0u;
    unsigned long long fin = 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
         p += (int64_t)gridDim.x * blockDim.x) {
      const unsigned b = __float_as_uint(src[j * P + p]);
      mn = min(mn, b);
      if (b < 0x7F800000u) { mx = max(mx, b); ++fin; }
    }
    mn = __reduce_min_sync(0xffffffffu, mn);
    mx = __reduce_max_sync(0xffffffffu, mx);
    for (int o = 16; o > 0; o >>= 1) fin += __shfl_down_sync(0xffffffffu, fin, o);
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&sm->mm[2 * j], mn);
      atomicMax(&sm->mm[2 * j + 1], mx);
      if (j == 0) atomicAdd(&sm->npat, fin);
    }
  }
}

__global__ void noalloc_reset_kernel(Small* sm, int nsrc) {
  for (int j = threadIdx.x; j < nsrc; j += blockDim.x) {
    sm->mm[2 * j] = 0x7F800000u;
    sm->mm[2 * j + 1] = 0u;
  }
  if (threadIdx.x == 0) {
    sm->npat = 0;
    sm->rind = -1;
    sm->ncand = 0;
    sm->status = 0;
  }
}

// Device address of the array on the current device (looked up once per device).
int scratch_address(unsigned char** out) {
  int dev = 0;
  IQ_CUDA_OK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return iq_set_error(IQ_ERR_LIMIT, "device index above 63");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_pick_scratch);
    if (e != cudaSuccess || !p)
      return iq_set_error(IQ_ERR_CUDA, "cudaGetSymbolAddress of the pick scratch failed: %s",
                          cudaGetErrorString(e));
    g_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_ptr[dev]);
  return IQ_OK;
}

}  // namespace

extern "C" int iq_pick_noalloc(const float* D, int64_t P, int32_t naux, const float* const* Ds,
                               double tol, uint64_t seed, int64_t tile, int64_t real,
                               int64_t* out_index, int64_t* out_ncand, int64_t* out_cands,
                               double* out_weights, int64_t cap, void* stream) {
  if (!D || P <= 0 || naux < 0 || (naux > 0 && !Ds) || !out_index)
    return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (P > NOALLOC_MAX_P)
    return iq_set_error(IQ_ERR_LIMIT, "iq_pick_noalloc handles at most %lld positions (got %lld)",
                        (long long)NOALLOC_MAX_P, (long long)P);
  if (naux > NOALLOC_MAX_AUX)
    return iq_set_error(IQ_ERR_LIMIT, "iq_pick_noalloc handles at most %d auxiliary maps",
                        NOALLOC_MAX_AUX);
  if (!(tol > 0 && tol <= 1)) return iq_set_error(IQ_ERR_ARG, "tolerance must be in range (0,1]");
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* src = reinterpret_cast<float*>(base + OFF_SRC);
  Small* sm = reinterpret_cast<Small*>(base + OFF_SMALL);
  const int nsrc = 1 + naux;
  IQ_CUDA_OK(cudaMemcpyAsync(src, D, sizeof(float) * P, cudaMemcpyDefault, st));
  for (int j = 0; j < naux; ++j)
    IQ_CUDA_OK(cudaMemcpyAsync(src + (j + 1) * P, Ds[j], sizeof(float) * P, cudaMemcpyDefault, st));
  noalloc_reset_kernel<<<1, 32, 0, st>>>(sm, nsrc);
  noalloc_minmax_kernel<<<(unsigned)std::min<int64_t>((P + 255) / 256, 256), 256, 0, st>>>(
      src, P, nsrc, sm);
  IQ_CUDA_OK(cudaGetLastError());
  unsigned long long npat = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(&npat, &sm->npat, sizeof(npat), cudaMemcpyDeviceToHost, st));
  IQ_CUDA_OK(cudaStreamSynchronize(st));

  // the launch helpers only read the stream and the profiling switch of a context
  iq_ctx lc;
  lc.stream = st;
  PickLaunch L;
  L.P = P; L.npat = (int64_t)npat; L.tol = tol; L.seed = seed; L.real0 = real;
  L.nreal = 1; L.ntask = 1;
  L.t0.D0 = src; L.t0.D0_rs = 0; L.t0.mm0 = sm->mm; L.t0.mm0_rs = 0;
  L.t0.naux = naux;
  L.t0.tile = tile;
  for (int j = 0; j < naux; ++j) {
    L.t0.aux[j] = src + (j + 1) * P; L.t0.aux_rs[j] = 0;
    L.t0.aux_mm[j] = sm->mm + 2 * (j + 1); L.t0.aux_mm_rs[j] = 0;
  }
  L.naux_max = naux;
  if (naux > 0 && npat > 0)
    iq_relax_sizes((int64_t)npat, tol, L.dbsize_norm, L.dbsize_zero, L.nseq_norm, L.seq_norm,
                   L.nseq_zero, L.seq_zero);
  uint32_t* k = reinterpret_cast<uint32_t*>(base + OFF_K0);
  L.cand = reinterpret_cast<int32_t*>(base + OFF_CAND);
  L.k0 = k; L.v0 = k + NOALLOC_MAX_P; L.k1 = k + 2 * NOALLOC_MAX_P; L.v1 = k + 3 * NOALLOC_MAX_P;
  L.w = reinterpret_cast<double*>(base + OFF_W);
  L.prod = reinterpret_cast<double*>(base + OFF_PROD);
  L.rind = &sm->rind;
  L.ncand = &sm->ncand;
  L.status = &sm->status;
  if ((rc = iq_launch_pick(&lc, L))) return rc;
  int64_t hr[2];
  int status = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(hr, &sm->rind, sizeof(hr), cudaMemcpyDeviceToHost, st));
  IQ_CUDA_OK(cudaMemcpyAsync(&status, &sm->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  IQ_CUDA_OK(cudaStreamSynchronize(st));
  if (status) return iq_set_error(status, "pick failed (status %d): no enabled pattern", status);
  *out_index = hr[0];
  const int64_t n = hr[1];
  if (out_ncand) *out_ncand = n;
  const int64_t m = std::min(n, cap);
  if (m > 0 && (out_cands || out_weights)) {
    // Both read-backs run on the caller's stream, followed by one synchronization. The int32
    // candidate list lands in the front half of out_cands and is widened in place from the
    // last entry down: int32 entry i lies below int64 entry i, so every entry is read before
    // a wider write reaches it.
    if (out_cands)
      IQ_CUDA_OK(cudaMemcpyAsync(out_cands, L.cand, sizeof(int32_t) * m, cudaMemcpyDefault, st));
    if (out_weights)
      IQ_CUDA_OK(cudaMemcpyAsync(out_weights, L.w, sizeof(double) * m, cudaMemcpyDefault, st));
    IQ_CUDA_OK(cudaStreamSynchronize(st));
    if (out_cands) {
      const int32_t* narrow = reinterpret_cast<const int32_t*>(out_cands);
      for (int64_t i = m - 1; i >= 0; --i) out_cands[i] = (int64_t)narrow[i];
    }
  }
  return IQ_OK;
}
