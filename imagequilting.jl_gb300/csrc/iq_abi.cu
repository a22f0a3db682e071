// C ABI of libiqgpu.so: contexts, errors, the resident training image and the per-operation
// entry points (fastdistance, pick, graphcut, finddisabled, genpath). iq_simulate lives in
// iq_sim.cu.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "iq_internal.h"

static thread_local char g_err[1024] = "";

int iq_set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char* iq_last_error(void) { return g_err; }

extern "C" int iq_version(void) { return 100; }  // 0.1.0

void* iq_scratch(iq_ctx* ctx, int slot, size_t bytes) {
  if ((int)ctx->buf.size() <= slot) {
    ctx->buf.resize(slot + 1, nullptr);
    ctx->buf_bytes.resize(slot + 1, 0);
  }
  if (bytes == 0) bytes = 256;
  if (ctx->buf_bytes[slot] >= bytes) return ctx->buf[slot];
  if (ctx->buf[slot]) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->buf[slot]);
    ctx->buf[slot] = nullptr;
    ctx->buf_bytes[slot] = 0;
  }
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    iq_set_error(IQ_ERR_ALLOC, "device allocation of %zu bytes failed", bytes);
    return nullptr;
  }
  ctx->buf[slot] = p;
  ctx->buf_bytes[slot] = bytes;
  return p;
}

// ---- timers --------------------------------------------------------------------------
void iq_timer_start(iq_ctx* ctx, const char* name) {
  if (!ctx->prof) return;
  IqTimer& t = ctx->timers[name];
  if (t.ev.size() < 2 * (t.used + 1)) {
    for (int i = 0; i < 2; ++i) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      t.ev.push_back(e);
    }
  }
  cudaEventRecord(t.ev[2 * t.used], ctx->stream);
}

void iq_timer_stop(iq_ctx* ctx, const char* name, double work) {
  if (!ctx->prof) return;
  IqTimer& t = ctx->timers[name];
  cudaEventRecord(t.ev[2 * t.used + 1], ctx->stream);
  t.used++;
  t.work += work;
}

extern "C" int iq_profile(iq_ctx* ctx, int32_t enable) {
  if (!ctx) return iq_set_error(IQ_ERR_ARG, "null context");
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->timers) { kv.second.used = 0; kv.second.work = 0; }
  ctx->prof_mma_flops = 0;
  ctx->prof_mma_flops16 = 0;
  ctx->prof_mma_launches = 0;
  ctx->prof_tc_cols = 0;
  cudaMemsetAsync(ctx->d_stats, 0, sizeof(unsigned long long) * ST_COUNT, ctx->stream);
  ctx->prof = enable != 0;
  return IQ_OK;
}

extern "C" int64_t iq_ctx_launches(iq_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" int iq_profile_get(iq_ctx* ctx, const char* kernel, double* ms_total,
                              int64_t* launches, double* work) {
  if (!ctx || !kernel) return iq_set_error(IQ_ERR_ARG, "null argument");
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  double ms = 0, wk = 0;
  int64_t n = 0;
  // counters: "graphcut.rounds", "graphcut.levels" (work = total, launches = CTAs),
  // "pick.iterations", "pick.candidates" (work = total, launches = CTAs), "corr.mma" (work =
  // tensor-pipe FLOPs issued, with the TF32 split and the padded positions and offsets),
  // "corr.mma16" (the FP16 part of it), "corr.columns" (work = columns of the tensor-core
  // launches, launches = their count)
  if (!strcmp(kernel, "corr.mma") || !strcmp(kernel, "corr.mma16") ||
      !strcmp(kernel, "corr.columns")) {
    if (ms_total) *ms_total = 0;
    if (launches) *launches = ctx->prof_mma_launches;
    if (work)
      *work = !strcmp(kernel, "corr.mma") ? ctx->prof_mma_flops
              : !strcmp(kernel, "corr.mma16") ? ctx->prof_mma_flops16 : ctx->prof_tc_cols;
    return IQ_OK;
  }
  // "corr.loop", "corr.wait_full", "corr.wait_afull", "corr.wait_done", "corr.producer_wait",
  // "corr.producer_loop", "corr.epilogue" (work = SM cycles summed over CTAs, launches = CTAs)
  const char* names[27] = {"graphcut.rounds", "graphcut.levels", "pick.iterations",
                           "pick.candidates", "graphcut.max_rounds", "graphcut.max_levels",
                           "corr.loop", "corr.wait_full", "corr.wait_afull", "corr.wait_done",
                           "corr.producer_wait", "corr.producer_loop", "corr.epilogue",
                           "corr.issue", "corr.mma_units", "graphcut.setup_cycles",
                           "graphcut.round_cycles", "graphcut.relabel_cycles",
                           "pick.select_cycles", "pick.weight_cycles", "pick.draw_cycles",
                           "graphcut.active_nodes", "graphcut.nodes", "pick.band_cycles",
                           "pick.ev1", "pick.ev2", "pick.ev3"};
  const int idx[27][2] = {{ST_CUT_ROUNDS, ST_CUT_CTAS}, {ST_CUT_LEVELS, ST_CUT_CTAS},
                          {ST_PICK_ITERS, ST_PICK_CTAS}, {ST_PICK_CAND, ST_PICK_CTAS},
                          {ST_CUT_MAXROUNDS, ST_CUT_CTAS}, {ST_CUT_MAXLEVELS, ST_CUT_CTAS},
                          {ST_TC_LOOP, ST_TC_CTAS}, {ST_TC_WFULL, ST_TC_CTAS},
                          {ST_TC_WAFULL, ST_TC_CTAS}, {ST_TC_WDONE, ST_TC_CTAS},
                          {ST_TC_PWAIT, ST_TC_CTAS}, {ST_TC_PLOOP, ST_TC_CTAS},
                          {ST_TC_EPI, ST_TC_CTAS}, {ST_TC_ISSUE, ST_TC_CTAS},
                          {ST_TC_MMAU, ST_TC_CTAS}, {ST_CUT_TSETUP, ST_CUT_CTAS},
                          {ST_CUT_TROUNDS, ST_CUT_CTAS}, {ST_CUT_TGR, ST_CUT_CTAS},
                          {ST_PICK_TSEL, ST_PICK_CTAS}, {ST_PICK_TW, ST_PICK_CTAS},
                          {ST_PICK_TDRAW, ST_PICK_CTAS}, {ST_CUT_ACTIVE, ST_CUT_CTAS},
                          {ST_CUT_NODES, ST_CUT_CTAS}, {ST_PICK_TBAND, ST_PICK_CTAS},
                          {ST_PICK_EV1, ST_PICK_CTAS}, {ST_PICK_EV2, ST_PICK_CTAS},
                          {ST_PICK_EV3, ST_PICK_CTAS}};
  for (int i = 0; i < 27; ++i)
    if (!strcmp(kernel, names[i])) {
      unsigned long long h[ST_COUNT];
      IQ_CUDA_OK(cudaMemcpy(h, ctx->d_stats, sizeof(h), cudaMemcpyDeviceToHost));
      if (ms_total) *ms_total = 0;
      if (launches) *launches = (int64_t)h[idx[i][1]];
      if (work) *work = (double)h[idx[i][0]];
      return IQ_OK;
    }
  auto it = ctx->timers.find(kernel);
  if (it != ctx->timers.end()) {
    wk = it->second.work;
    for (size_t i = 0; i < it->second.used; ++i) {
      float f = 0;
      cudaEventElapsedTime(&f, it->second.ev[2 * i], it->second.ev[2 * i + 1]);
      ms += f;
    }
    n = (int64_t)it->second.used;
  }
  if (ms_total) *ms_total = ms;
  if (launches) *launches = n;
  if (work) *work = wk;
  return IQ_OK;
}

// ---- contexts ------------------------------------------------------------------------
extern "C" int iq_ctx_create(int device, iq_ctx** out) {
  if (!out) return iq_set_error(IQ_ERR_ARG, "null output pointer");
  *out = nullptr;
  IQ_CUDA_OK(cudaSetDevice(device));
  iq_ctx* c = new iq_ctx();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return iq_set_error(IQ_ERR_CUDA, "stream creation failed");
  }
  if (cudaMalloc(&c->d_status, sizeof(int)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return iq_set_error(IQ_ERR_ALLOC, "status word allocation failed");
  }
  cudaMemset(c->d_status, 0, sizeof(int));
  if (cudaMalloc(&c->d_stats, sizeof(unsigned long long) * ST_COUNT) != cudaSuccess) {
    cudaFree(c->d_status);
    cudaStreamDestroy(c->stream);
    delete c;
    return iq_set_error(IQ_ERR_ALLOC, "counter allocation failed");
  }
  cudaMemset(c->d_stats, 0, sizeof(unsigned long long) * ST_COUNT);
  if (cudaMalloc(&c->d_ties, sizeof(unsigned long long)) != cudaSuccess) {
    cudaFree(c->d_stats);
    cudaFree(c->d_status);
    cudaStreamDestroy(c->stream);
    delete c;
    return iq_set_error(IQ_ERR_ALLOC, "counter allocation failed");
  }
  cudaMemset(c->d_ties, 0, sizeof(unsigned long long));
  *out = c;
  return IQ_OK;
}

static void free_ti(iq_ctx* c) {
  cudaFree(c->d_ti);
  cudaFree(c->d_ti2ii);
  cudaFree(c->d_nanii);
  c->d_ti = nullptr;
  c->d_ti2ii = nullptr;
  c->d_nanii = nullptr;
  c->has_ti = false;
}

extern "C" int iq_ctx_destroy(iq_ctx* ctx) {
  if (!ctx) return IQ_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_ti(ctx);
  for (void* p : ctx->buf) cudaFree(p);
  for (auto& kv : ctx->timers)
    for (auto e : kv.second.ev) cudaEventDestroy(e);
  cudaFree(ctx->d_status);
  cudaFree(ctx->d_stats);
  cudaFree(ctx->d_ties);
  iq_lp_free(ctx);
  if (ctx->stream2) {
    cudaStreamSynchronize(ctx->stream2);
    cudaStreamDestroy(ctx->stream2);
  }
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return IQ_OK;
}

extern "C" void* iq_ctx_stream(iq_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" int iq_ties(iq_ctx* ctx, int64_t* out) {
  if (!ctx || !out) return iq_set_error(IQ_ERR_ARG, "null argument");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  unsigned long long v = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(&v, ctx->d_ties, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  *out = (int64_t)v;
  return IQ_OK;
}

extern "C" int iq_set_option(iq_ctx* ctx, const char* name, int64_t value) {
  if (!ctx || !name) return iq_set_error(IQ_ERR_ARG, "null argument");
  if (!strcmp(name, "graphcut.gr_period")) {
    if (value < 1 || value > 1 << 20) return iq_set_error(IQ_ERR_ARG, "gr_period out of range");
    ctx->cut_gr_period = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "graphcut.threads")) {
    if (value != 256 && value != 512 && value != 1024)
      return iq_set_error(IQ_ERR_ARG, "graphcut.threads must be 256, 512 or 1024");
    ctx->cut_threads = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "corr.variant")) {
    if (value < 0 || value > 3) return iq_set_error(IQ_ERR_ARG, "corr.variant must be 0..3");
    ctx->corr_variant = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "corr.engine")) {
    if (value < 0 || value > 2) return iq_set_error(IQ_ERR_ARG, "corr.engine must be 0, 1 or 2");
    ctx->corr_engine = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "sim.max_steps")) {
    ctx->max_steps = value < 0 ? -1 : value;
    return IQ_OK;
  }
  if (!strcmp(name, "sim.level_chunk")) {
    if (value < 1 || value > 4096) return iq_set_error(IQ_ERR_ARG, "level_chunk out of range");
    ctx->level_chunk = value;
    return IQ_OK;
  }
  if (!strcmp(name, "sim.streams")) {
    if (value < 1 || value > 2) return iq_set_error(IQ_ERR_ARG, "sim.streams must be 1 or 2");
    ctx->sim_streams = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.enable")) {
    if (value < 0 || value > 1) return iq_set_error(IQ_ERR_ARG, "lp.enable must be 0 or 1");
    ctx->lp_enable = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.k")) {
    if (value < 16 || value > (1 << 20)) return iq_set_error(IQ_ERR_ARG, "lp.k out of range");
    ctx->lp_k = value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.train_near")) {
    if (value < 0 || value > 4096) return iq_set_error(IQ_ERR_ARG, "lp.train_near out of range");
    ctx->lp_train_near = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.kmax")) {
    if (value < 16 || value > (1 << 22)) return iq_set_error(IQ_ERR_ARG, "lp.kmax out of range");
    ctx->lp_kmax = value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.monitor")) {
    if (value < 0 || value > (1 << 20)) return iq_set_error(IQ_ERR_ARG, "lp.monitor out of range");
    ctx->lp_monitor = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.fallback")) {
    if (value < 0 || value > 1) return iq_set_error(IQ_ERR_ARG, "lp.fallback must be 0 or 1");
    ctx->lp_fallback = (int)value;
    return IQ_OK;
  }
  if (!strcmp(name, "lp.capture")) {
    if (value < 0 || value > (1 << 24)) return iq_set_error(IQ_ERR_ARG, "lp.capture out of range");
    IQ_CUDA_OK(cudaSetDevice(ctx->device));
    const int rc = iq_lp_capture_reserve(ctx, value);
    if (rc) return rc;
    ctx->lp_capture = value;
    return IQ_OK;
  }
  return iq_set_error(IQ_ERR_ARG, "unknown option '%s'", name);
}

// ---- training image --------------------------------------------------------------------
static int read_dims(int32_t ndim, const int64_t* size, Dim3& d) {
  if (ndim < 1 || ndim > 3 || !size) return iq_set_error(IQ_ERR_ARG, "ndim must be 1, 2 or 3");
  int64_t e[3] = {1, 1, 1};
  for (int i = 0; i < ndim; ++i) {
    if (size[i] <= 0) return iq_set_error(IQ_ERR_ARG, "extents must be positive");
    if (size[i] > (1 << 20)) return iq_set_error(IQ_ERR_LIMIT, "extent above 2^20");
    e[i] = size[i];
  }
  d = Dim3{e[0], e[1], e[2]};
  return IQ_OK;
}

extern "C" int iq_set_ti(iq_ctx* ctx, const void* ti, int32_t dtype, int32_t ndim,
                         const int64_t* size) {
  if (!ctx || !ti) return iq_set_error(IQ_ERR_ARG, "null argument");
  if (dtype != IQ_F32 && dtype != IQ_F64) return iq_set_error(IQ_ERR_ARG, "dtype must be F32 or F64");
  Dim3 d;
  int rc = read_dims(ndim, size, d);
  if (rc) return rc;
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  const int64_t n = d.vol();
  if (n >= (int64_t)1 << 31) return iq_set_error(IQ_ERR_LIMIT, "training image above 2^31 voxels");
  const bool same = ctx->has_ti && ctx->ti.x == d.x && ctx->ti.y == d.y && ctx->ti.z == d.z;
  if (!same) {
    cudaStreamSynchronize(ctx->stream);
    free_ti(ctx);
    const int64_t nii = (d.x + 1) * (d.y + 1) * (d.z + 1);
    if (cudaMalloc(&ctx->d_ti, sizeof(float) * n) != cudaSuccess ||
        cudaMalloc(&ctx->d_ti2ii, sizeof(double) * nii) != cudaSuccess ||
        cudaMalloc(&ctx->d_nanii, sizeof(int32_t) * nii) != cudaSuccess) {
      cudaGetLastError();
      free_ti(ctx);
      return iq_set_error(IQ_ERR_ALLOC, "training image allocation failed");
    }
  }
  ctx->has_ti = false;
  uint8_t* nanm = (uint8_t*)iq_scratch(ctx, S_TMP0, (size_t)n);
  if (!nanm) return IQ_ERR_ALLOC;
  if (dtype == IQ_F32) {
    IQ_CUDA_OK(cudaMemcpyAsync(ctx->d_ti, ti, sizeof(float) * n, cudaMemcpyDefault, ctx->stream));
  } else {
    double* tmp = (double*)iq_scratch(ctx, S_TMP1, sizeof(double) * n);
    if (!tmp) return IQ_ERR_ALLOC;
    IQ_CUDA_OK(cudaMemcpyAsync(tmp, ti, sizeof(double) * n, cudaMemcpyDefault, ctx->stream));
    if ((rc = iq_launch_to_f32(ctx, tmp, ctx->d_ti, n))) return rc;
  }
  unsigned long long* dhash = (unsigned long long*)iq_scratch(ctx, S_TIHASH, 2 * sizeof(int64_t));
  if (!dhash) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemsetAsync(dhash, 0, sizeof(unsigned long long), ctx->stream));
  if ((rc = iq_launch_prepare(ctx, ctx->d_ti, n, nanm, dhash))) return rc;
  if ((rc = iq_build_integrals(ctx, ctx->d_ti, d, ctx->d_ti2ii, ctx->d_nanii, nanm))) return rc;
  int32_t total = 0;
  unsigned long long hash = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(&total, ctx->d_nanii + (d.x + 1) * (d.y + 1) * (d.z + 1) - 1,
                             sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaMemcpyAsync(&hash, dhash, sizeof(hash), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  IqValueStats st;
  if ((rc = iq_value_stats(ctx, ctx->d_ti, n, st))) return rc;
  ctx->ti = d;
  ctx->ndim = ndim;
  ctx->ti_nan = total;
  ctx->ti_stats = st;
  ctx->has_ti = true;
  hash ^= (unsigned long long)d.x * 0x100000001B3ull ^ (unsigned long long)d.y << 21 ^
          (unsigned long long)d.z << 42 ^ (unsigned long long)ndim << 60;
  if (!same || hash != ctx->ti_hash || ctx->ti_version == 0) ctx->ti_version += 1;
  ctx->ti_hash = hash;
  return IQ_OK;
}

// ---- fastdistance -----------------------------------------------------------------------
extern "C" int iq_fastdistance(iq_ctx* ctx, const int64_t* tilesize, int32_t ntmpl,
                               const float* tmpl, const uint8_t* weights, float* out) {
  if (!ctx || !tilesize || !tmpl || !out || ntmpl <= 0)
    return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (!ctx->has_ti) return iq_set_error(IQ_ERR_STATE, "no training image set");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  Dim3 t;
  int rc = read_dims(ctx->ndim, tilesize, t);
  if (rc) return rc;
  if (t.x > ctx->ti.x || t.y > ctx->ti.y || t.z > ctx->ti.z)
    return iq_set_error(IQ_ERR_ARG, "invalid tile size");
  if (t.x >= 1024 || t.y >= 1024 || t.z >= 1024) return iq_set_error(IQ_ERR_LIMIT, "tile extent >= 1024");
  const int64_t T = t.vol();
  Dim3 od{ctx->ti.x - t.x + 1, ctx->ti.y - t.y + 1, ctx->ti.z - t.z + 1};
  const int64_t P = od.vol();
  // mask -> offset list (host)
  std::vector<uint8_t> w(T, 1);
  if (weights) IQ_CUDA_OK(cudaMemcpy(w.data(), weights, T, cudaMemcpyDefault));
  std::vector<uint32_t> kl;
  for (int64_t k = 0; k < T; ++k)
    if (w[k]) kl.push_back(kpack(k % t.x, (k / t.x) % t.y, k / (t.x * t.y)));
  const int K = (int)kl.size();
  // Is the mask the tile minus one box (the shape of every overlap mask)? Then the tensor-core
  // kernel applies and A2 comes from the integral image.
  int64_t blo[3] = {0, 0, 0}, bhi[3] = {0, 0, 0};
  bool boxmask = true;
  {
    int64_t mn[3] = {t.x, t.y, t.z}, mx[3] = {-1, -1, -1}, nz = 0;
    for (int64_t k = 0; k < T; ++k)
      if (!w[k]) {
        const int64_t c3[3] = {k % t.x, (k / t.x) % t.y, k / (t.x * t.y)};
        for (int d = 0; d < 3; ++d) { mn[d] = std::min(mn[d], c3[d]); mx[d] = std::max(mx[d], c3[d]); }
        ++nz;
      }
    if (nz > 0) {
      const int64_t vol = (mx[0] - mn[0] + 1) * (mx[1] - mn[1] + 1) * (mx[2] - mn[2] + 1);
      boxmask = vol == nz;
      for (int d = 0; d < 3; ++d) { blo[d] = mn[d]; bhi[d] = mx[d] + 1; }
    }
  }
  const bool use_tc = ctx->corr_engine >= 1 && boxmask && K > 0;
  // A2 by integral image when the mask is all ones, else direct
  const bool full = K == T;
  const int rt = iq_register_tile(ntmpl);
  const int rpad = ((ntmpl + rt - 1) / rt) * rt;
  float* d_tmpl = (float*)iq_scratch(ctx, S_TMP2, sizeof(float) * T * ntmpl);
  uint32_t* d_kl = (uint32_t*)iq_scratch(ctx, S_KLIST, sizeof(uint32_t) * std::max(K, 1));
  float* d_tv = use_tc ? nullptr
                       : (float*)iq_scratch(ctx, S_TV, sizeof(float) * std::max<int64_t>(K, 1) * rpad);
  double* d_b2 = (double*)iq_scratch(ctx, S_B2, sizeof(double) * rpad);
  uint8_t* d_dis = (uint8_t*)iq_scratch(ctx, S_DIS, (size_t)P);
  float* d_out = (float*)iq_scratch(ctx, S_D, sizeof(float) * P * ntmpl);
  if (!d_tmpl || !d_kl || (!use_tc && !d_tv) || !d_b2 || !d_dis || !d_out) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(d_tmpl, tmpl, sizeof(float) * T * ntmpl, cudaMemcpyDefault, ctx->stream));
  if (K) IQ_CUDA_OK(cudaMemcpyAsync(d_kl, kl.data(), sizeof(uint32_t) * K, cudaMemcpyHostToDevice, ctx->stream));
  if ((rc = iq_launch_disabled(ctx, ctx->d_nanii, ctx->ti, t, d_dis))) return rc;
  GatherLaunch G;
  G.grid = d_tmpl; G.grid_dims = t; G.grid_stride = T;
  G.ntmpl = ntmpl; G.rpad = rpad;
  G.t0 = GatherTask{d_kl, K, 0, nullptr, d_tv, d_b2, nullptr};
  if ((rc = iq_launch_gather(ctx, G))) return rc;
  std::vector<TcCol> cols;
  std::vector<uint32_t> stw;
  if (use_tc) {
    IqValueStats tstats;
    if ((rc = iq_value_stats(ctx, d_tmpl, T * ntmpl, tstats))) return rc;
    TcBox box0;
    for (int d = 0; d < 3; ++d) { box0.lo[d] = (int32_t)blo[d]; box0.hi[d] = (int32_t)bhi[d]; }
    TcStages stg;
    iq_tc_stages(t, &box0, 1, stg);
    const size_t ns = stg.word.size(), n16 = stg.w16a.size();
    stw.resize(2 * ns + 3 * n16);
    for (size_t e = 0; e < ns; ++e) { stw[e] = stg.word[e]; stw[ns + e] = stg.prefix[e]; }
    for (size_t e = 0; e < n16; ++e) {
      stw[2 * ns + e] = stg.w16a[e];
      stw[2 * ns + n16 + e] = stg.w16b[e];
      stw[2 * ns + 2 * n16 + e] = stg.pre16[e];
    }
    for (int32_t c0 = 0; c0 < ntmpl; c0 += IQ_TC_MAXN) {
      const int nb = std::min<int32_t>(IQ_TC_MAXN, ntmpl - c0);
      const int Np = (nb + 15) / 16 * 16;
      for (int i = 0; i < Np; ++i)
        cols.push_back(i < nb ? TcCol{(int64_t)(c0 + i) * T, d_out + (size_t)(c0 + i) * P, d_b2 + c0 + i, nullptr, 0, 0}
                              : TcCol{-1, nullptr, nullptr, nullptr, 0, 0});
    }
    uint32_t* d_st = (uint32_t*)iq_scratch(ctx, S_TCSTAGE, sizeof(uint32_t) * std::max<size_t>(stw.size(), 1));
    TcCol* d_cols = (TcCol*)iq_scratch(ctx, S_TCCOLS, sizeof(TcCol) * cols.size());
    void* d_B = iq_scratch(ctx, S_TCB, (size_t)std::max<int64_t>(std::max(stg.nsteps, stg.nsteps16), 1) *
                                          64 * IQ_TC_MAXN);
    if (!d_st || !d_cols || !d_B) return IQ_ERR_ALLOC;
    IQ_CUDA_OK(cudaMemcpyAsync(d_st, stw.data(), sizeof(uint32_t) * stw.size(), cudaMemcpyHostToDevice, ctx->stream));
    IQ_CUDA_OK(cudaMemcpyAsync(d_cols, cols.data(), sizeof(TcCol) * cols.size(), cudaMemcpyHostToDevice, ctx->stream));
    size_t col0 = 0;
    for (int32_t c0 = 0; c0 < ntmpl; c0 += IQ_TC_MAXN) {
      const int nb = std::min<int32_t>(IQ_TC_MAXN, ntmpl - c0);
      TcCorrLaunch L;
      L.img = ctx->d_ti; L.img_dims = ctx->ti; L.out_dims = od; L.tile = t; L.ii = ctx->d_ti2ii;
      L.nbox = 1; L.box[0] = box0;
      L.disabled = d_dis;
      L.stage_word = d_st; L.stage_prefix = d_st + ns; L.nstage = (int)ns; L.nsteps = stg.nsteps;
      L.stage16 = d_st + 2 * ns; L.nstage16 = (int)n16; L.nsteps16 = stg.nsteps16;
      L.grid = d_tmpl; L.grid_dims = t; L.cols = d_cols + col0; L.N = (nb + 15) / 16 * 16;
      L.B = d_B; L.img_stats = ctx->ti_stats; L.tmpl_stats = tstats;
      L.flops = 2.0 * (double)P * (double)K * nb;
      if ((rc = iq_launch_corr_tc(ctx, L))) return rc;
      col0 += L.N;
    }
  } else {
    CorrLaunch C;
    C.img = ctx->d_ti; C.img_dims = ctx->ti; C.out_dims = od; C.tile = t;
    C.rpad = rpad; C.ntmpl = ntmpl; C.out_stride = P; C.disabled = d_dis;
    // all-ones mask: A^2 from the integral image (the full tile, no inner box); otherwise summed
    C.t0 = CorrTask{d_kl, K, d_tv, d_b2, full ? ctx->d_ti2ii : nullptr, {0, 0, 0}, {0, 0, 0},
                    d_out, nullptr};
    if ((rc = iq_launch_corr(ctx, C))) return rc;
  }
  IQ_CUDA_OK(cudaMemcpyAsync(out, d_out, sizeof(float) * P * ntmpl, cudaMemcpyDefault, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  return IQ_OK;
}

extern "C" int iq_finddisabled(iq_ctx* ctx, const int64_t* tilesize, uint8_t* out) {
  if (!ctx || !tilesize || !out) return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (!ctx->has_ti) return iq_set_error(IQ_ERR_STATE, "no training image set");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  Dim3 t;
  int rc = read_dims(ctx->ndim, tilesize, t);
  if (rc) return rc;
  if (t.x > ctx->ti.x || t.y > ctx->ti.y || t.z > ctx->ti.z)
    return iq_set_error(IQ_ERR_ARG, "invalid tile size");
  const int64_t P = (ctx->ti.x - t.x + 1) * (ctx->ti.y - t.y + 1) * (ctx->ti.z - t.z + 1);
  uint8_t* d = (uint8_t*)iq_scratch(ctx, S_DIS, (size_t)P);
  if (!d) return IQ_ERR_ALLOC;
  if ((rc = iq_launch_disabled(ctx, ctx->d_nanii, ctx->ti, t, d))) return rc;
  IQ_CUDA_OK(cudaMemcpyAsync(out, d, (size_t)P, cudaMemcpyDefault, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  return IQ_OK;
}

// ---- pick ------------------------------------------------------------------------------
extern "C" int iq_pick(iq_ctx* ctx, const float* D, int64_t P, int32_t naux,
                       const float* const* Ds, double tol, uint64_t seed, int64_t tile,
                       int64_t real, int64_t* out_index, int64_t* out_ncand, int64_t* out_cands,
                       double* out_weights, int64_t cap) {
  if (!ctx || !D || P <= 0 || naux < 0 || (naux > 0 && !Ds) || !out_index)
    return iq_set_error(IQ_ERR_ARG, "invalid argument");
  if (naux > IQ_MAX_AUX) return iq_set_error(IQ_ERR_LIMIT, "at most %d auxiliary distances", IQ_MAX_AUX);
  if (P >= ((int64_t)1 << 31)) return iq_set_error(IQ_ERR_LIMIT, "P above 2^31");
  if (!(tol > 0 && tol <= 1)) return iq_set_error(IQ_ERR_ARG, "tolerance must be in range (0,1]");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  const int nsrc = 1 + naux;
  float* d_src = (float*)iq_scratch(ctx, S_D, sizeof(float) * P * nsrc);
  unsigned* d_mm = (unsigned*)iq_scratch(ctx, S_MINMAX, sizeof(unsigned) * 2);
  int32_t* cand = (int32_t*)iq_scratch(ctx, S_PICK_CAND, sizeof(int32_t) * P);
  uint32_t* k0 = (uint32_t*)iq_scratch(ctx, S_PICK_K0, sizeof(uint32_t) * P);
  uint32_t* v0 = (uint32_t*)iq_scratch(ctx, S_PICK_V0, sizeof(uint32_t) * P);
  uint32_t* k1 = (uint32_t*)iq_scratch(ctx, S_PICK_K1, sizeof(uint32_t) * P);
  uint32_t* v1 = (uint32_t*)iq_scratch(ctx, S_PICK_V1, sizeof(uint32_t) * P);
  double* w = (double*)iq_scratch(ctx, S_PICK_W, sizeof(double) * P);
  double* prod = (double*)iq_scratch(ctx, S_PICK_PROD, sizeof(double) * P);
  int64_t* rind = (int64_t*)iq_scratch(ctx, S_RIND, sizeof(int64_t) * 2);
  if (!d_src || !d_mm || !cand || !k0 || !v0 || !k1 || !v1 || !w || !prod || !rind) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(d_src, D, sizeof(float) * P, cudaMemcpyDefault, ctx->stream));
  for (int j = 0; j < naux; ++j)
    IQ_CUDA_OK(cudaMemcpyAsync(d_src + (j + 1) * P, Ds[j], sizeof(float) * P, cudaMemcpyDefault,
                               ctx->stream));
  // min and max-finite bits of every source, and npatterns (finite entries of D)
  std::vector<float> hD(P);
  std::vector<unsigned> hmm(2 * nsrc);
  int64_t npat = 0;
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));  // the uploads above are on the ctx stream
  for (int j = 0; j < nsrc; ++j) {
    IQ_CUDA_OK(cudaMemcpy(hD.data(), d_src + j * P, sizeof(float) * P, cudaMemcpyDeviceToHost));
    unsigned mn = 0x7F800000u, mx = 0u;
    for (int64_t q = 0; q < P; ++q) {
      unsigned b = fbits(hD[q]);
      mn = std::min(mn, b);
      if (b < 0x7F800000u) { mx = std::max(mx, b); if (j == 0) ++npat; }
    }
    hmm[2 * j] = mn;
    hmm[2 * j + 1] = mx;
  }
  d_mm = (unsigned*)iq_scratch(ctx, S_MINMAX, sizeof(unsigned) * 2 * nsrc);
  if (!d_mm) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(d_mm, hmm.data(), sizeof(unsigned) * 2 * nsrc, cudaMemcpyHostToDevice, ctx->stream));
  IQ_CUDA_OK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  PickLaunch L;
  L.P = P; L.npat = npat; L.tol = tol; L.seed = seed; L.real0 = real; L.nreal = 1; L.ntask = 1;
  L.t0.D0 = d_src; L.t0.D0_rs = 0; L.t0.mm0 = d_mm; L.t0.mm0_rs = 0;
  L.t0.naux = naux;
  L.t0.tile = tile;
  for (int j = 0; j < naux; ++j) {
    L.t0.aux[j] = d_src + (j + 1) * P; L.t0.aux_rs[j] = 0;
    L.t0.aux_mm[j] = d_mm + 2 * (j + 1); L.t0.aux_mm_rs[j] = 0;
  }
  L.naux_max = naux;
  if (naux > 0 && npat > 0)
    iq_relax_sizes(npat, tol, L.dbsize_norm, L.dbsize_zero, L.nseq_norm, L.seq_norm, L.nseq_zero,
                   L.seq_zero);
  L.cand = cand; L.k0 = k0; L.v0 = v0; L.k1 = k1; L.v1 = v1; L.w = w; L.prod = prod;
  L.rind = rind; L.ncand = rind + 1; L.status = ctx->d_status;
  IQ_CUDA_OK(cudaMemsetAsync(ctx->d_ties, 0, sizeof(unsigned long long), ctx->stream));
  L.ties = ctx->d_ties;
  int rc = iq_launch_pick(ctx, L);
  if (rc) return rc;
  int64_t hr[2];
  int st = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(hr, rind, sizeof(hr), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  if (st) return iq_set_error(st, "pick failed (status %d): no enabled pattern", st);
  *out_index = hr[0];
  const int64_t n = hr[1];
  if (out_ncand) *out_ncand = n;
  if (out_cands && cap > 0) {
    std::vector<int32_t> c(std::min(n, cap));
    IQ_CUDA_OK(cudaMemcpy(c.data(), cand, sizeof(int32_t) * c.size(), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < c.size(); ++i) out_cands[i] = c[i];
  }
  if (out_weights && cap > 0)
    IQ_CUDA_OK(cudaMemcpy(out_weights, w, sizeof(double) * std::min(n, cap), cudaMemcpyDefault));
  return IQ_OK;
}

// ---- graph cut ---------------------------------------------------------------------------
extern "C" int iq_graphcut(iq_ctx* ctx, const float* A, const float* B, int32_t ndim,
                           const int64_t* size, int32_t dim, uint8_t* mask) {
  if (!ctx || !A || !B || !mask) return iq_set_error(IQ_ERR_ARG, "null argument");
  Dim3 d;
  int rc = read_dims(ndim, size, d);
  if (rc) return rc;
  if (dim < 0 || dim >= ndim) return iq_set_error(IQ_ERR_ARG, "invalid cut dimension");
  IQ_CUDA_OK(cudaSetDevice(ctx->device));
  const int64_t n = d.vol();
  if (n >= ((int64_t)1 << 24)) return iq_set_error(IQ_ERR_LIMIT, "slab above 2^24 nodes");
  float* dA = (float*)iq_scratch(ctx, S_TMP0, sizeof(float) * n * 2);
  uint8_t* dout = (uint8_t*)iq_scratch(ctx, S_CUTBUF, (size_t)n * 6);
  void* scr = iq_scratch(ctx, S_CUTSCR, iq_cut_scratch_bytes(n));
  if (!dA || !dout || !scr) return IQ_ERR_ALLOC;
  IQ_CUDA_OK(cudaMemcpyAsync(dA, A, sizeof(float) * n, cudaMemcpyDefault, ctx->stream));
  IQ_CUDA_OK(cudaMemcpyAsync(dA + n, B, sizeof(float) * n, cudaMemcpyDefault, ctx->stream));
  IQ_CUDA_OK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  CutLaunch L;
  L.t0.start = 0;
  L.t0.nslab = 1;
  L.t0.slab[0].dim = dim;
  L.t0.slab[0].next = 0;
  L.t0.slab[0].off[0] = L.t0.slab[0].off[1] = L.t0.slab[0].off[2] = 0;
  L.t0.slab[0].ext[0] = d.x; L.t0.slab[0].ext[1] = d.y; L.t0.slab[0].ext[2] = d.z;
  L.nreal = 1; L.ntask = 1;
  L.A = dA; L.B = dA + n;
  L.out = dout; L.slabmax = n;
  L.scratch = scr; L.scratch_per_cta = (int64_t)iq_cut_scratch_bytes(n);
  L.status = ctx->d_status;
  L.stats = ctx->prof ? ctx->d_stats : nullptr;
  L.gr_period = ctx->cut_gr_period;
  L.threads = ctx->cut_threads;
  if ((rc = iq_launch_cut(ctx, L))) return rc;
  int st = 0;
  IQ_CUDA_OK(cudaMemcpyAsync(mask, dout, (size_t)n, cudaMemcpyDefault, ctx->stream));
  IQ_CUDA_OK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  IQ_CUDA_OK(cudaStreamSynchronize(ctx->stream));
  if (st) return iq_set_error(st, "graph cut hit its round limit");
  return IQ_OK;
}
