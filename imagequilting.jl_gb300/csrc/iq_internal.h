// Internal declarations shared by the translation units of libiqgpu.so.
//
// Kernels work on batches of "tasks": all the tiles of one dependency level of the tile path
// (tiles whose regions do not overlap run together) times all realizations. A launch either
// carries one task by value (t0, for the per-operation entry points) or points at a device
// array of tasks uploaded once per simulation.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "iq_common.cuh"

// ---------------------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------------------
// Magnitude range and precision of an array of floats (NaN and Inf ignored), which decide how
// the tensor-core correlation may represent it: TF32 halves, or FP16 halves after a power-of-two
// scaling (only when the range keeps every half a normal FP16 number).
struct IqValueStats {
  float amax = 0.f;       // largest magnitude
  int minexp = 1 << 30;   // smallest binary exponent of a nonzero magnitude
  bool narrow = true;     // every value has at most 11 significant bits (a TF32 value)
  int lsbexp = 1 << 30;   // smallest binary exponent of the lowest set bit of a nonzero value
                          // (every value is a multiple of 2^lsbexp)
  void merge(const IqValueStats& o) {
    amax = amax > o.amax ? amax : o.amax;
    minexp = minexp < o.minexp ? minexp : o.minexp;
    narrow = narrow && o.narrow;
    lsbexp = lsbexp < o.lsbexp ? lsbexp : o.lsbexp;
  }
  int maxexp() const;      // binary exponent of amax (0 when amax == 0)
  bool fp16_range() const; // nonzero magnitudes within 2^17 of amax
};
IqValueStats iq_host_stats(const float* v, int64_t n);
// Error coefficient of a distance map of image values A against templates B over K offsets,
// |D32 - D| <= kappa (A2 + B2) + eabs: 0 when every product, partial sum and square is exact
// in FP32 (values on a common binary grid, sums below 2^24 of its step), else the bound of the
// form that computed it (form 1: tensor cores, FP16 halves; 2: tensor cores, TF32 halves;
// 0: SIMT FP32). n_img: image voxels, for the Float64 integral image behind A2.
double iq_map_kappa(const IqValueStats& A, const IqValueStats& B, int64_t K, int form);
double iq_map_eabs(const IqValueStats& A, int64_t n_img);

struct IqTimer {
  std::vector<cudaEvent_t> ev;  // start/stop pairs
  size_t used = 0;              // pairs recorded
  double work = 0;              // algorithmic work of the recorded launches
};

struct iq_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // resident training image
  bool has_ti = false;
  int ndim = 0;
  Dim3 ti{1, 1, 1};
  float* d_ti = nullptr;       // prepared TI, NaN -> 0 (float32)
  double* d_ti2ii = nullptr;   // integral image of TI^2, (x+1)(y+1)(z+1) doubles
  int32_t* d_nanii = nullptr;  // integral image of the NaN indicator
  int64_t ti_nan = 0;          // number of NaN voxels
  IqValueStats ti_stats;       // magnitude range and precision of the prepared TI
  int* d_status = nullptr;     // device status word (first kernel error)
  unsigned long long* d_ties = nullptr;  // near-tie count of the last pick or simulation
  // grow-only scratch buffers, by slot
  std::vector<void*> buf;
  std::vector<size_t> buf_bytes;
  // profiling
  bool prof = false;
  std::map<std::string, IqTimer> timers;
  int64_t launches = 0;         // kernels launched by this context
  // device counters filled while profiling: [0] cut rounds, [1] cut BFS levels, [2] cut CTAs,
  // [3] pick relaxation iterations, [4] pick candidates, [5] pick CTAs, [6] max cut rounds,
  // [7] max cut BFS levels
  unsigned long long* d_stats = nullptr;
  double prof_mma_flops = 0;    // tensor-pipe FLOPs issued by the correlation while profiling
  double prof_mma_flops16 = 0;  // the part issued as FP16 MMAs (bf16/fp16 rate; TF32: half)
  int64_t prof_mma_launches = 0;
  double prof_tc_cols = 0;      // columns (templates, with padding) of those launches
  // tuning knobs (iq_set_option)
  int cut_gr_period = 32;
  int cut_threads = 512;
  int64_t level_chunk = 64;     // most tiles of one dependency level launched together
  int corr_variant = 1;         // launch shape of the 16-template correlation
  int corr_engine = 2;          // box-mask distances: 2 tensor cores FP16 halves when the data's
                                // range allows (else TF32), 1 tensor cores TF32, 0 SIMT
  int64_t max_steps = -1;       // tiles simulated per realization (< 0: all)
  int sim_streams = 1;          // realization groups of iq_simulate, each on its own stream
  cudaStream_t stream2 = nullptr;  // stream of the second realization group (made on first use)
  struct IqLp* lp = nullptr;       // learned proposal state (iq_proposal_host.cu)
  int lp_enable = 0;               // iq_simulate shortlists with the proposal where it applies
  int64_t lp_k = 8192;             // shortlist size the proposal starts a call with
  int64_t lp_kmax = 65536;         // largest size the recall monitor may raise it to
  int lp_train_near = 16;          // training negatives per anchor drawn next to its positive
  int64_t lp_capture = 0;          // training pairs iq_simulate records (0: none)
  int lp_monitor = 16;             // every lp_monitor-th proposal chunk checks its recall
  int lp_fallback = 1;             // 0: keep the shortlists even below 0.99 recall (measuring)
  int64_t ti_version = 0;          // bumped by every iq_set_ti whose content differs from the
                                   // resident image's (keys the proposal's caches)
  unsigned long long ti_hash = 0;  // content key of the resident image (values and extents)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};
enum IqStat { ST_CUT_ROUNDS = 0, ST_CUT_LEVELS, ST_CUT_CTAS, ST_PICK_ITERS, ST_PICK_CAND,
              ST_PICK_CTAS, ST_CUT_MAXROUNDS, ST_CUT_MAXLEVELS,
              // tensor-core correlation, SM cycles summed over CTAs: issuer loop, issuer waits
              // for B copies / A images / MMA completion (refills), producer (warp 1) waits
              // and loop, epilogue; the CTA count; cycles inside the MMA issue blocks and the
              // MMAs issued in units of one M=128 N=256 K=8 MMA (x 256)
              ST_TC_LOOP, ST_TC_WFULL, ST_TC_WAFULL, ST_TC_WDONE, ST_TC_PWAIT, ST_TC_PLOOP,
              ST_TC_EPI, ST_TC_CTAS, ST_TC_ISSUE, ST_TC_MMAU,
              // graph cut, SM cycles summed over CTAs: set-up (loads, capacities), push and
              // relabel rounds, global relabels
              ST_CUT_TSETUP, ST_CUT_TROUNDS, ST_CUT_TGR,
              // pick, SM cycles summed over CTAs: selection + compaction, tau-model weights, draw
              ST_PICK_TSEL, ST_PICK_TW, ST_PICK_TDRAW, ST_PICK_TBAND, ST_PICK_EV1, ST_PICK_EV2,
              ST_PICK_EV3,
              // graph cut: active nodes summed over rounds, node count of the slabs
              ST_CUT_ACTIVE, ST_CUT_NODES, ST_COUNT };

// scratch slot ids
enum IqSlot {
  S_SIM = 0, S_CUT, S_D, S_DHARD, S_SOFT, S_TV, S_B2, S_KLIST, S_MINMAX, S_PICK_CAND,
  S_PICK_K0, S_PICK_V0, S_PICK_K1, S_PICK_V1, S_PICK_W, S_PICK_PROD, S_RIND, S_NCAND,
  S_CUTBUF, S_CUTSCR, S_DIS, S_AUX, S_AUXTI, S_AUXII, S_HARDLIST, S_HARDPTS, S_OUT,
  S_TMP0, S_TMP1, S_TMP2, S_TIHASH, S_STARTS, S_SOFTMM, S_TASKS, S_VOX, S_TCB, S_TCCOLS, S_TCSTAGE, S_TCB2, S_TCFLAG, S_TCSOFT, S_SOFTKEYS,
  S_PICK_RV, S_PICK_RR, S_PICK_RL, S_SOFTB2,
  S_PB_RV, S_PB_RR, S_PB_RL, S_PB_LIST, S_PB_K, S_PB_OUT, S_PB_POOL, S_PB_SRC,
  S_PBH_OUT, S_PBH_POOL, S_PBH_SRC,
  S_LP_T, S_LP_NT, S_LP_TAU, S_LP_LIST, S_LP_CNT, S_LP_DL, S_LP_COLS, S_LP_TSRC, S_LP_TBOX,
  S_LP_RIND, S_LP_NCAND, S_LP_D, S_LP_BITS, S_LP_ITEMS, S_LP_X, S_LP_E, S_LP_GE, S_LP_FEAT, S_LP_BH1, S_LP_BGZ1, S_LP_BH2, S_LP_DENSE, S_LP_QUAD,
  S_COUNT
};

// device scratch of at least `bytes` in slot `slot` (contents undefined); nullptr on failure
void* iq_scratch(iq_ctx* ctx, int slot, size_t bytes);

// ---------------------------------------------------------------------------------------
// Timing helpers (no-ops unless ctx->prof)
// ---------------------------------------------------------------------------------------
void iq_timer_start(iq_ctx* ctx, const char* name);
void iq_timer_stop(iq_ctx* ctx, const char* name, double work = 0);
// count a kernel launch of this context
inline void iq_count(iq_ctx* ctx, int n = 1) { ctx->launches += n; }

// ---------------------------------------------------------------------------------------
// Distance (iq_distance.cu)
// ---------------------------------------------------------------------------------------
// Packed template offset: kx | ky << 10 | kz << 20 (each < 1024).
IQ_HD uint32_t kpack(int64_t kx, int64_t ky, int64_t kz) {
  return (uint32_t)kx | ((uint32_t)ky << 10) | ((uint32_t)kz << 20);
}
IQ_HD int kx_of(uint32_t k) { return (int)(k & 1023u); }
IQ_HD int ky_of(uint32_t k) { return (int)((k >> 10) & 1023u); }
IQ_HD int kz_of(uint32_t k) { return (int)(k >> 20); }

// One batch of templates that share a mask (one tile of a level).
struct CorrTask {
  const uint32_t* klist;  // K packed offsets of the mask
  int K;
  const float* tv;        // K x rpad template values (weights applied)
  const double* b2;       // rpad: sum of squared template values
  const double* ii;       // integral image of img^2 (A^2 = full tile - inner box); nullptr:
                          // A^2 summed over the offset list
  int64_t lo[3], hi[3];   // inner box excluded from the full tile (empty if lo >= hi)
  float* out;             // ntmpl maps of out_stride floats
  unsigned* minmax;       // ntmpl x [min bits, max finite bits] (nullable)
};

struct CorrLaunch {
  const float* img = nullptr;  // image, extents `img_dims`
  Dim3 img_dims{1, 1, 1};
  Dim3 out_dims{1, 1, 1};      // valid extent
  Dim3 tile{1, 1, 1};
  int rpad = 0;                // row length of tv (multiple of the register tile)
  int ntmpl = 0;               // templates computed per task (<= rpad)
  int64_t out_stride = 0;      // floats between templates in `out`
  const uint8_t* disabled = nullptr;  // 1 -> +Inf (nullable)
  int ntask = 1;
  CorrTask t0{};               // the task when `tasks` is null
  const CorrTask* tasks = nullptr;  // device array of ntask tasks
  double flops = 0;            // algorithmic FLOPs of the launch (profiling)
};
int iq_launch_corr(iq_ctx* ctx, const CorrLaunch& L);

// Gather of template values tv[k][t] = grid_t[start + k] for the packed offsets.
struct GatherTask {
  const uint32_t* klist;
  int K;
  int64_t start;          // linear origin of the tile in the grid
  const float* kval;      // per-offset values instead of a grid (hard data); nullable
  float* tv;              // K x rpad
  double* b2;             // rpad
  unsigned* minmax;       // reset to [+Inf bits, 0] per template (nullable)
};
struct GatherLaunch {
  const float* grid = nullptr;      // base grid
  Dim3 grid_dims{1, 1, 1};
  int64_t grid_stride = 0;          // floats between consecutive templates' grids
  const int64_t* starts = nullptr;  // per template start (device), overrides task.start
  int ntmpl = 0;
  int rpad = 0;
  int ntask = 1;
  GatherTask t0{};
  const GatherTask* tasks = nullptr;
};
int iq_launch_gather(iq_ctx* ctx, const GatherLaunch& G);

int iq_register_tile(int ntmpl);  // register tile width used for `ntmpl` templates

// Sum over [x0, x0+ex) x [y0, y0+ey) x [z0, z0+ez) of an integral image with a zero border
// (row pitch sx, plane pitch sxy).
__device__ __forceinline__ double iq_box_sum(const double* __restrict__ ii, int64_t sx, int64_t sxy,
                                             int64_t x0, int64_t y0, int64_t z0, int64_t ex,
                                             int64_t ey, int64_t ez) {
  const int64_t x1 = x0 + ex, y1 = y0 + ey, z1 = z0 + ez;
  double s = ii[x1 + sx * y1 + sxy * z1];
  s -= ii[x0 + sx * y1 + sxy * z1];
  s -= ii[x1 + sx * y0 + sxy * z1];
  s += ii[x0 + sx * y0 + sxy * z1];
  s -= ii[x1 + sx * y1 + sxy * z0];
  s += ii[x0 + sx * y1 + sxy * z0];
  s += ii[x1 + sx * y0 + sxy * z0];
  s -= ii[x0 + sx * y0 + sxy * z0];
  return s;
}

// ---- tensor-core correlation (iq_corr_tc.cu) ----
constexpr int IQ_TC_MAXN = 256;   // columns (templates) per launch
constexpr int IQ_TC_MAXBOX = 8;   // distinct masks per launch

// A mask "tile minus the box [lo, hi)" (an empty box: the full tile).
struct TcBox {
  int32_t lo[3], hi[3];
};

// One column of the batched product: template n of a launch. Its values are read from
// `grid + src + kx + gx * (ky + gy * kz)` inside mask `box` (src < 0: a padding column).
struct TcCol {
  int64_t src;
  float* out;          // distance map of P floats
  const double* b2;    // sum of squared template values over the mask (from the gather)
  unsigned* mm;        // [min bits, max finite bits] (nullable)
  int32_t box;         // index into the launch's boxes
  int32_t pad_;
};

// Stage list of the union of some masks: one stage per (ky, kz) row and group of 24
// x-offsets that any of the masks touches, word = ky | kz << 10 | g << 20 | stepmask << 26
// (three 8-offset K-steps per group), prefix = K-steps before the stage.
struct TcStages {
  std::vector<uint32_t> word, prefix;
  int64_t nsteps = 0;  // K-steps of all stages
  // the FP16 form: consecutive rows in pairs (w16b = 0 when a row has no partner), each K-step
  // of 16 offsets made of two 8-offset chunks of the pair
  std::vector<uint32_t> w16a, w16b, pre16;
  int64_t nsteps16 = 0;
};
void iq_tc_stages(Dim3 tile, const TcBox* boxes, int nbox, TcStages& out);

struct TcCorrLaunch {
  const float* img = nullptr; Dim3 img_dims{1, 1, 1};
  Dim3 out_dims{1, 1, 1};
  Dim3 tile{1, 1, 1};
  const double* ii = nullptr;           // integral image of img^2 (required)
  int nbox = 1;
  TcBox box[IQ_TC_MAXBOX] = {};
  const uint8_t* disabled = nullptr;
  const uint32_t* stage_word = nullptr; // device copies of TcStages (TF32 form)
  const uint32_t* stage_prefix = nullptr;
  int nstage = 0;
  int64_t nsteps = 0;
  const uint32_t* stage16 = nullptr;    // FP16 form: w16a, w16b, pre16 of nstage16 each
  int nstage16 = 0;
  int64_t nsteps16 = 0;
  const float* grid = nullptr; Dim3 grid_dims{1, 1, 1};  // template source
  const TcCol* cols = nullptr;          // device array of N columns
  int N = 0;                            // multiple of 16, at most 256
  void* B = nullptr;                    // packed templates, max(nsteps, nsteps16) * 64 * N bytes
  IqValueStats img_stats, tmpl_stats;   // ranges of the image and of the templates
  double flops = 0;                     // algorithmic FLOPs (profiling)
};
int iq_launch_corr_tc(iq_ctx* ctx, const TcCorrLaunch& L);
// statistics of a device array of floats
int iq_value_stats(iq_ctx* ctx, const float* d, int64_t n, IqValueStats& out);

// integral images and disabled windows
int iq_build_integrals(iq_ctx* ctx, const float* d_img, Dim3 dims, double* d_sqii,
                       int32_t* d_nanii, const uint8_t* d_nan);
int iq_build_value_integral(iq_ctx* ctx, const float* d_img, Dim3 dims, double* d_ii);
int iq_launch_disabled(iq_ctx* ctx, const int32_t* d_nanii, Dim3 dims, Dim3 tile, uint8_t* out);

// ---------------------------------------------------------------------------------------
// Pick (iq_pick.cu)
// ---------------------------------------------------------------------------------------
// How the pick re-evaluates one distance map directly at chosen positions (the exact re-rank):
// D[p] = sum over the mask offsets k (klist order, column-major) of (img[p + k] - tmpl[k])^2.
// The map itself (FP32, from the tensor cores or the SIMT kernel) satisfies
// |D32[p] - D[p]| <= kappa * (A2[p] + B2) + eabs; kappa == 0 marks a map whose values are
// exact, which the pick then uses as they are.
struct ExactSrc {
  const float* img;       // image (TI or auxiliary TI, prepared: NaN -> 0)
  int64_t isx, isxy;      // image strides: x extent, x * y extents
  const uint32_t* klist;  // packed mask offsets, column-major order
  int K;
  const float* tmpl;      // template grid at the tile origin (realization 0), or nullptr
  int64_t tgx, tgxy;      // grid strides
  int64_t tmpl_rs;        // floats between consecutive realizations' grids (0: shared)
  const float* kval;      // per-offset template values instead of a grid (hard data)
  const double* b2;       // sum of squared template values (realization 0)
  int64_t b2_rs;
  double kappa, eabs;
};

// Refined top-k selection of a map shared by all realizations of a tile (a soft-data map),
// computed once per (map, relaxation step): positions with D < lo are in, D > hi out, and the
// positions in between are listed at pool + off (ascending, bit 31 set when in).
struct PreBand {
  double lo, hi;
  int64_t off, n;
  unsigned long long key;   // the FP32 (value, index) key of the selection
  long long ties;           // near-ties at its boundary (the boundary position excluded)
  int32_t ok;               // 0: not precomputed (the pick selects itself); 1: band; 2: the
                            // map is exact and the key alone decides
  int32_t pad_;
};

// Sources of one tile; realization r of the tile reads D0 + r * D0_rs etc.
struct PickTask {
  const float* D0; int64_t D0_rs;           // primary distance
  const unsigned* mm0; int64_t mm0_rs;      // its [min, max finite] bits
  int naux;                                 // 0: threshold pick, > 0: relaxation
  const float* aux[IQ_MAX_AUX];
  int64_t aux_rs[IQ_MAX_AUX];
  const unsigned* aux_mm[IQ_MAX_AUX];
  int64_t aux_mm_rs[IQ_MAX_AUX];
  // selection keys of aux j, (value bits << 32 | index), precomputed for the first nkeys steps
  // of the normal softdbsize sequence (sources shared by all realizations; nullable)
  const unsigned long long* aux_keys[IQ_MAX_AUX];
  const PreBand* aux_pb[IQ_MAX_AUX];        // refined selections of shared maps (nullable)
  const PreBand* x0_pb;                     // D's dbsize selection, shared (nullable)
  const int32_t* x0_pool;                   // its band list
  const int32_t* pb_pool;                   // their band lists
  int nkeys;
  int64_t tile;                             // Philox counter of the draw
  // direct re-evaluation of D0 and of each auxiliary map (kappa == 0, or img == nullptr:
  // the map's values are taken as exact)
  ExactSrc x0;
  ExactSrc xa[IQ_MAX_AUX];
};

struct PickLaunch {
  int64_t P = 0;           // positions
  int64_t npat = 0;        // enabled positions (finite D)
  double tol = 0.1;
  uint64_t seed = 0;
  int64_t real0 = 0;       // realization index of r = 0
  int nreal = 0;           // realizations per task; CTA b handles task b / nreal, r = b % nreal
  int ntask = 1;
  int naux_max = 0;        // largest naux of the tasks
  PickTask t0{};
  const PickTask* tasks = nullptr;
  // relaxation sizes (src/relaxation.jl:11-36): normal and all-zero cases
  int64_t dbsize_norm = 0, dbsize_zero = 0;
  int nseq_norm = 0, nseq_zero = 0;
  int64_t seq_norm[IQ_MAX_SEQ] = {}, seq_zero[IQ_MAX_SEQ] = {};
  // scratch, P entries per CTA
  int32_t* cand = nullptr;
  uint32_t *k0 = nullptr, *v0 = nullptr, *k1 = nullptr, *v1 = nullptr;
  double* w = nullptr;
  double* prod = nullptr;
  // exact re-rank scratch, P entries per CTA (needed when a task has a map with kappa > 0)
  double* rv = nullptr;       // refined values
  double* rr = nullptr;       // their error radii
  uint8_t* rl = nullptr;      // their levels
  int64_t dx = 0, dxy = 0;    // distance-map strides (x extent, x * y extents)
  // outputs, one per CTA
  int64_t* rind = nullptr;
  int64_t* ncand = nullptr;  // nullable
  int* status = nullptr;
  unsigned long long* ties = nullptr;   // near-tie counter (nullable)
  unsigned long long* stats = nullptr;  // profiling counters (nullable)
};
int iq_launch_pick(iq_ctx* ctx, const PickLaunch& L);
// an ExactSrc that marks a map as exact (no re-rank)
inline ExactSrc iq_exact_none() {
  ExactSrc s{};
  return s;
}

// Selection keys of nmaps maps of P floats (map m at maps + m * P, its [min, max finite] bits
// at mm + 2 m) for the sizes seq[0..nq): keys[m * nq + q] (iq_pick.cu)
constexpr int IQ_PRE_KEYS = 3;  // softdbsize steps precomputed per shared map
int iq_launch_select_keys(iq_ctx* ctx, const float* maps, const unsigned* mm, int64_t nmaps,
                          int64_t P, const int64_t* seq, int nq, unsigned long long* keys);
// Refined selections of nmaps shared maps (map m at maps + m * P, its re-evaluation srcs[m],
// a device array) for the sizes seq[0..nq): out[m * nq + q], lists in pool (cap entries each).
int iq_launch_select_bands(iq_ctx* ctx, const float* maps, const unsigned* mm,
                           const ExactSrc* srcs, int64_t nmaps, int64_t P, int64_t dx,
                           int64_t dxy, const int64_t* seq, int nq, PreBand* out, int32_t* pool,
                           int64_t cap, int keys_exact = 0);

// ---------------------------------------------------------------------------------------
// Graph cut (iq_graphcut.cu) and paste (iq_paste.cu)
// ---------------------------------------------------------------------------------------
struct CutSlab {
  int dim;          // cut dimension
  int next;         // 0: overlap with the previous tile (keep M), 1: with the next (keep !M)
  int64_t off[3];   // slab origin inside the tile
  int64_t ext[3];   // slab extents
};

// The overlap slabs of one tile.
struct StepTask {
  int64_t start;    // linear origin of the tile in the simulation grid
  int nslab;
  CutSlab slab[6];
};

struct CutLaunch {
  int nreal = 0;               // realizations per task; CTA y = task * nreal + r
  int ntask = 1;
  int nslab_max = 0;           // grid.x
  StepTask t0{};
  const StepTask* tasks = nullptr;
  // A: simulation grid of realization r at the tile; B: TI at rind[task * nreal + r]
  const float* sim = nullptr; Dim3 sim_dims{1, 1, 1}; int64_t sim_rstride = 0;
  const float* ti = nullptr;  Dim3 ti_dims{1, 1, 1};
  Dim3 dist_dims{1, 1, 1};
  const int64_t* rind = nullptr;
  // direct mode (iq_graphcut): A/B arrays of the slab itself
  const float* A = nullptr; const float* B = nullptr;
  uint8_t* out = nullptr;      // (ntask * nreal) x 6 x slabmax bytes: keep-old flags
  int64_t slabmax = 0;
  void* scratch = nullptr;     // global scratch for slabs too large for shared memory
  int64_t scratch_per_cta = 0;
  int* status = nullptr;
  int round_cap = 1 << 18;
  unsigned long long* stats = nullptr;  // profiling counters (nullable)
  int gr_period = 32;          // rounds between global relabels
  int threads = 512;           // threads per CTA
};
int iq_launch_cut(iq_ctx* ctx, const CutLaunch& L);
size_t iq_cut_scratch_bytes(int64_t nodes);

struct PasteLaunch {
  int nreal = 0;
  int ntask = 1;
  StepTask t0{};
  const StepTask* tasks = nullptr;
  float* sim = nullptr; Dim3 sim_dims{1, 1, 1}; int64_t sim_rstride = 0;
  float* cut = nullptr;       // debug cut grid (nullable)
  Dim3 tile{1, 1, 1};
  const float* ti = nullptr; Dim3 ti_dims{1, 1, 1}; Dim3 dist_dims{1, 1, 1};
  const int64_t* rind = nullptr;
  const uint8_t* cutbuf = nullptr; int64_t slabmax = 0;
};
int iq_launch_paste(iq_ctx* ctx, const PasteLaunch& L);

int iq_launch_hard_overwrite(iq_ctx* ctx, int nreal, float* sim, float* cut, Dim3 sim_dims,
                             int64_t sim_rstride, int64_t n, const int64_t* lin,
                             const float* val);
int iq_launch_crop(iq_ctx* ctx, int nreal, const float* src, Dim3 src_dims, int64_t src_rstride,
                   Dim3 out_dims, float* dst);
int iq_launch_voxsum(iq_ctx* ctx, int nreal, const float* cut, int64_t n, int64_t rstride,
                     double* out);
int iq_launch_pad_symmetric(iq_ctx* ctx, const float* src, Dim3 src_dims, float* dst,
                            Dim3 dst_dims);
int iq_launch_prepare(iq_ctx* ctx, float* data, int64_t n, uint8_t* nanmask,
                      unsigned long long* hash = nullptr);
int iq_launch_to_f32(iq_ctx* ctx, const double* src, float* dst, int64_t n);

// ---------------------------------------------------------------------------------------
// Learned proposal (iq_proposal.cu)
// ---------------------------------------------------------------------------------------
#define IQ_LP_CH 32      // channels of the encoder's convolutions
#define IQ_LP_EMB 64     // embedding width
#define IQ_LP_MAXG 256   // cells of the input grid (8 x 8 x 4)
#define IQ_LP_MAXG2 32   // after the first stride-2 convolution (4 x 4 x 2)
#define IQ_LP_MAXG3 4    // after the second (2 x 2 x 1)
// parameter offsets (floats): w1 [32][3], b1, w2 [32][32][27], b2, w3 [32][32][27], b3,
// w4 [64][nf], b4 (nf = 32 x cells of layer 3, channel fastest)
#define LP_OFF_W1 0
#define LP_OFF_B1 (LP_OFF_W1 + IQ_LP_CH * 3)
#define LP_OFF_W2 (LP_OFF_B1 + IQ_LP_CH)
#define LP_OFF_B2 (LP_OFF_W2 + IQ_LP_CH * IQ_LP_CH * 27)
#define LP_OFF_W3 (LP_OFF_B2 + IQ_LP_CH)
#define LP_OFF_B3 (LP_OFF_W3 + IQ_LP_CH * IQ_LP_CH * 27)
#define LP_OFF_W4 (LP_OFF_B3 + IQ_LP_CH)

struct LpGeo {
  int t[3];        // tile
  int g[3], c[3];  // cell grid and cell size
  int g2[3], g3[3];
  int ng, ng2, ng3, nf;
  int off_b4, npar;
};
LpGeo iq_lp_geo(Dim3 tile);

// One training step's data (device pointers): nA anchors with features feats[feat row], their
// positives and nneg negatives per anchor as windows of the image (integral images ii1, ii2);
// items: anchors, then positives, then negatives (iq_proposal.cu TrainItem layout, 16 bytes).
struct LpTrainBatch {
  const float* w;          // FP32 parameters
  const void* items;
  int nA, nneg;
  float temp;
  const float* feats;      // [rows][3 * ng]
  const int32_t* boxes;    // [rows][6]
  const double* ii1;
  const double* ii2;
  Dim3 img, dist;
  float* X;                // scratch [items][3 * ng]
  float* E;                // scratch [items][64]
  float* gE;               // scratch [items][64]
  float* grad;             // [npar]
  double* loss;            // device scalar
};
int iq_lp_train_batch(iq_ctx* ctx, const LpGeo& g, const LpTrainBatch& B, double* loss_out);
int iq_lp_adam(iq_ctx* ctx, float* p, const float* g, float* m, float* v, int n, float lr, int step);
struct __nv_bfloat16;
// Window embeddings of every distance-map position (pos == nullptr) or of pos[0, npos).
int iq_lp_encode_windows(iq_ctx* ctx, const LpGeo& g, const float* w, const double* ii1,
                         const double* ii2, Dim3 img, Dim3 dist, const int* lo, const int* hi,
                         __nv_bfloat16* out, float* norm, const int64_t* pos = nullptr,
                         int64_t npos = 0);
// One column of the proposal's pick: tile `tile` of global realization `real`, with the mask's
// offsets and the simulation grid at the tile.
// Quads of a mask: four consecutive x offsets of one (y, z) row starting at a multiple of 4,
// for byte-valued images (sums of squared differences with one dp4a per quad).
struct LpQuad {
  int32_t off;    // image offset of the quad's first voxel from the window origin
  int32_t tx;     // template offset of the same voxel
  uint32_t mask;  // 0xFF in each byte whose voxel is in the mask
  int32_t pad_;
};
struct LpColumn {
  const uint32_t* klist;
  int K;
  int nq;              // quads of the mask (quad)
  const LpQuad* quad;
  const float* tmpl;
  int64_t tgx, tgxy;
  int64_t tile, real;
  int32_t lohi[6];     // the mask: the tile minus the box [lo, hi)
  int32_t tdim[3];     // tile extents
  int32_t pad2_;
};
// The training image as the exact sums of the proposal read it. Plane form (codes 0..3, tiles
// of x extent <= 32): 2-bit codes in tiles of 32 (x) by 16 (y) voxels, one 64-bit word per tile
// row (bits 0-31: the low bit of each voxel's code, bits 32-63: the high bit), tiles ordered
// (x, y, z) with one extra column of zero tiles past the last in x; a window row of 32 voxels
// is then two words and a funnel shift. Byte form otherwise (quads).
struct LpImg {
  const uint8_t* b8;               // bytes, 16 bytes of padding past the end
  const unsigned long long* b2;    // plane form (nullptr: byte form)
  int64_t isx, isxy;               // byte image strides
  int64_t ntx, nty;                // plane tiles per row (x, including the zero column), per slice (y)
};
#ifdef __CUDACC__
// Comparisons of FP32 map values with Float64 bounds, made in FP32 (the FP64 pipe of this part
// is far narrower than its FP32 pipe): for a float d and a double x,
//   (double)d <  x  <=>  d <  f_up(x)     (f_up: the smallest float >= x)
//   (double)d <= x  <=>  d <= f_dn(x)     (f_dn: the largest float <= x)
__device__ __forceinline__ float f_up(double x) { return __double2float_ru(x); }
__device__ __forceinline__ float f_dn(double x) { return __double2float_rd(x); }

__device__ __forceinline__ float f_step(float v, bool up) {  // neighbour of a positive float
  const uint32_t b = __float_as_uint(v);
  return __uint_as_float(up ? b + 1u : b - 1u);
}

// FP32 bounds [lo, hi] of the floats v with fabs(rn((double)v - t)) <= w, the near-tie test
// as the oracle evaluates it (an interval, since rn is monotone); t > 0 finite, 0 <= w < t.
__device__ inline void tie_window_f(double t, double w, float& lo, float& hi) {
  lo = f_dn(t - w);
  hi = f_up(t + w);
  for (int i = 0; i < 8 && lo >= 0.f && !(__dsub_rn((double)lo, t) >= -w); ++i) lo = f_step(lo, true);
  for (int i = 0; i < 8 && lo > 0.f; ++i) {
    const float p = f_step(lo, false);
    if (p > 0.f && __dsub_rn((double)p, t) >= -w) lo = p; else break;
  }
  for (int i = 0; i < 8 && hi > 0.f && !(__dsub_rn((double)hi, t) <= w); ++i) hi = f_step(hi, false);
  for (int i = 0; i < 8 && hi < 3.0e38f; ++i) {
    const float p = f_step(hi, true);
    if (__dsub_rn((double)p, t) <= w) hi = p; else break;
  }
}

// The four bytes at image address p (any alignment): two aligned words and a byte permute.
__device__ __forceinline__ uint32_t iq_ld4(const uint8_t* p) {
  const uintptr_t u = reinterpret_cast<uintptr_t>(p);
  const uint32_t sh = (uint32_t)(u & 3u);
  const uint32_t* w = reinterpret_cast<const uint32_t*>(u - sh);
  return __byte_perm(__ldg(w), __ldg(w + 1), 0x3210u + 0x1111u * sh);
}

// Stage a column's quads in shared memory: (image offset, template bytes, byte mask) per quad.
// Returns false (for the whole block) when a template value in the mask is not a byte value.
__device__ inline bool iq_stage_quads(const LpColumn& col, uint4* q) {
  int bad = 0;
  for (int i = threadIdx.x; i < col.nq; i += blockDim.x) {
    const LpQuad e = col.quad[i];
    uint32_t t = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      if (!(e.mask >> (8 * b) & 0xFFu)) continue;
      const float v = col.tmpl[e.tx + b];
      if (!(v >= 0.f && v <= 255.f && v == floorf(v))) bad = 1;
      t |= ((uint32_t)v & 0xFFu) << (8 * b);
    }
    q[i] = make_uint4((uint32_t)e.off, t, e.mask, 0u);
  }
  return !__syncthreads_or(bad);
}

// Warp-collective: sum over the quads [0, nq) of the squared byte differences of the window at
// `base` (every lane gets the total). With `bound` finite, gives up (returns UINT32_MAX) as soon
// as a partial sum exceeds bound() -- a lower bound of the total, the terms being non-negative.
template <typename Bound>
__device__ __forceinline__ uint32_t iq_quad_ssd(const uint8_t* base, const uint4* q, int nq,
                                                const Bound& bound) {
  const int lane = threadIdx.x & 31;
  uint32_t acc = 0;
  int i = lane;
  for (; i + 7 * 32 < nq; i += 8 * 32) {
    uint32_t v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = iq_ld4(base + (int32_t)q[i + 32 * u].x);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint4 e = q[i + 32 * u];
      const uint32_t d = __vabsdiffu4(v[u], e.y) & e.z;
      acc = __dp4a(d, d, acc);
    }
    uint32_t part = acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((float)part > bound()) return 0xFFFFFFFFu;
  }
  for (; i < nq; i += 32) {
    const uint4 e = q[i];
    const uint32_t d = __vabsdiffu4(iq_ld4(base + (int32_t)e.x), e.y) & e.z;
    acc = __dp4a(d, d, acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// Plane form: stage a column's template rows (ty, tz) of the tile in shared memory as
// (low-bit plane, high-bit plane, mask bits, ty | tz << 16): the rows outside the box's (y, z)
// range (every x in the mask) first, then the rows through the box (x outside it only; left out
// when the box spans every x), so that partial sums grow fast for the early exit. Returns the
// number of rows staged, or -1 (for the whole block) when a template value in the mask is not
// one of 0, 1, 2, 3.
__device__ inline int iq_stage_rows(const LpColumn& col, uint4* rows) {
  const int R = col.tdim[1] * col.tdim[2];
  const int* lh = col.lohi;
  const int iy0 = max(lh[1], 0), iy1 = max(min(lh[4], col.tdim[1]), iy0);
  const int iz0 = max(lh[2], 0), iz1 = max(min(lh[5], col.tdim[2]), iz0);
  const int ny = iy1 - iy0, nz = iz1 - iz0;
  const int nouter = R - ny * nz;
  const bool inner_empty = lh[0] <= 0 && lh[3] >= col.tdim[0];
  int bad = 0;
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    const int ty = r % col.tdim[1], tz = r / col.tdim[1];
    const bool rin = ty >= iy0 && ty < iy1 && tz >= iz0 && tz < iz1;
    // box rows before r in (tz, ty) order
    const int before = (min(max(tz, iz0), iz1) - iz0) * ny +
                       (tz >= iz0 && tz < iz1 ? min(max(ty, iy0), iy1) - iy0 : 0);
    if (rin && inner_empty) continue;
    uint32_t p0 = 0, p1 = 0, m = 0;
    for (int x = 0; x < col.tdim[0]; ++x) {
      if (rin && x >= lh[0] && x < lh[3]) continue;
      const float v = col.tmpl[x + col.tgx * ty + col.tgxy * tz];
      if (!(v == 0.f || v == 1.f || v == 2.f || v == 3.f)) bad = 1;
      const uint32_t c = (uint32_t)v & 3u;
      m |= 1u << x;
      p0 |= (c & 1u) << x;
      p1 |= (c >> 1) << x;
    }
    rows[rin ? nouter + before : r - before] = make_uint4(p0, p1, m, (uint32_t)ty | ((uint32_t)tz << 16));
  }
  return __syncthreads_or(bad) ? -1 : (inner_empty ? nouter : R);
}

// Sum of (a - b)^2 over one row of 32 codes given as bit planes (a0, a1), (b0, b1) and mask m:
// with u = a1 - b1, v = a0 - b0 in {-1, 0, 1}, (a - b)^2 = 4u^2 + 4uv + v^2, u^2 = a1 ^ b1,
// v^2 = a0 ^ b0, and where both are nonzero uv = +1 exactly when a1 == a0 (then u and v have
// the sign of a1 - b1 = a0 - b0), so sum 4uv = 4 popc(y) - 8 popc(y & (a1 ^ a0)) with
// y = (a1 ^ b1) & (a0 ^ b0).
__device__ __forceinline__ int iq_row_ssd(uint32_t a0, uint32_t a1, const uint4& t) {
  const uint32_t m = t.z;
  const uint32_t x1 = (a1 ^ t.y) & m, x0 = (a0 ^ t.x) & m;
  const uint32_t y = x1 & x0;
  return __popc(x0) + 4 * (__popc(x1) + __popc(y)) - 8 * __popc(y & (a1 ^ a0));
}

// Warp-collective, plane form: sum over the R staged rows for the window at (x0, y0, z0), with
// the early exit of iq_quad_ssd.
// (The plane image has fewer than 2^31 words: 32-bit index arithmetic.)
template <typename Bound>
__device__ __forceinline__ uint32_t iq_plane_ssd(const LpImg& im, int64_t x0, int64_t y0,
                                                 int64_t z0, const uint4* rows, int R,
                                                 const Bound& bound) {
  const int lane = threadIdx.x & 31;
  const uint32_t s = (uint32_t)(x0 & 31);
  const uint32_t ntx16 = (uint32_t)im.ntx * 16u, zs = (uint32_t)im.nty * ntx16;
  const uint32_t base = (uint32_t)z0 * zs + ((uint32_t)x0 >> 5) * 16u;
  const uint32_t y0u = (uint32_t)y0;
  int acc = 0;
  int r = lane;
  for (; r + 3 * 32 < R; r += 4 * 32) {
    unsigned long long wa[4], wb[4];
    uint4 t[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      t[u] = rows[r + 32 * u];
      const uint32_t yy = y0u + (t[u].w & 0xFFFFu);
      const uint32_t i0 = base + (t[u].w >> 16) * zs + (yy >> 4) * ntx16 + (yy & 15u);
      wa[u] = __ldg(im.b2 + i0);
      wb[u] = __ldg(im.b2 + i0 + 16);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t a0 = __funnelshift_r((uint32_t)wa[u], (uint32_t)wb[u], s);
      const uint32_t a1 = __funnelshift_r((uint32_t)(wa[u] >> 32), (uint32_t)(wb[u] >> 32), s);
      acc += iq_row_ssd(a0, a1, t[u]);
    }
    int part = acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((float)part > bound()) return 0xFFFFFFFFu;
  }
  for (; r < R; r += 32) {
    const uint4 t = rows[r];
    const uint32_t yy = y0u + (t.w & 0xFFFFu);
    const uint32_t i0 = base + (t.w >> 16) * zs + (yy >> 4) * ntx16 + (yy & 15u);
    const unsigned long long a = __ldg(im.b2 + i0), b = __ldg(im.b2 + i0 + 16);
    acc += iq_row_ssd(__funnelshift_r((uint32_t)a, (uint32_t)b, s),
                      __funnelshift_r((uint32_t)(a >> 32), (uint32_t)(b >> 32), s), t);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return (uint32_t)acc;
}

// Stage a column for either form (rows or quads at `stage`): the number of staged items, or -1
// when the column cannot be summed in that form.
__device__ inline int iq_stage(const LpImg& im, const LpColumn& col, uint4* stage) {
  if (im.b2) return iq_stage_rows(col, stage);
  return iq_stage_quads(col, stage) ? col.nq : -1;
}

// Exact sum of the column at distance-map position (x, y, z), either form; n: staged items.
template <typename Bound>
__device__ __forceinline__ uint32_t iq_lp_ssd(const LpImg& im, const uint4* stage, int n,
                                              int64_t x, int64_t y, int64_t z, const Bound& bound) {
  if (im.b2) return iq_plane_ssd(im, x, y, z, stage, n, bound);
  return iq_quad_ssd(im.b8 + x + im.isx * y + im.isxy * z, stage, n, bound);
}
#endif
#define IQ_LP_SAMPLES 8192  // positions sampled per column for its shortlist threshold
// dst[0, n) = the image as bytes (dst holds n + 16 bytes; the 16 past the end are zeroed);
// *bad (device) = 1 when a value is not an integer in [0, 255].
int iq_lp_to_u8(iq_ctx* ctx, const float* src, int64_t n, uint8_t* dst, int* bad);
// The plane form of an image of codes 0..3 (LpImg; dst: d.z * nty * ntx * 16 words);
// *bad (device) = 1 when a value is not one of the four codes.
int iq_lp_to_planes(iq_ctx* ctx, const float* src, Dim3 d, int64_t ntx, int64_t nty,
                    unsigned long long* dst, int* bad);
// Rows i * ceil(P / IQ_LP_SAMPLES) of the window embeddings (the sampled positions).
int iq_lp_sample_rows(iq_ctx* ctx, const __nv_bfloat16* W, const float* nW, int64_t P,
                      __nv_bfloat16* Ws, float* nWs);
// Shortlists of N columns: per column the threshold of about k positions from the sampled
// rows' scores (dense: N x IQ_LP_SAMPLES scratch), then every position at or below it.
int iq_lp_shortlist(iq_ctx* ctx, const __nv_bfloat16* W, const float* nW, int64_t P,
                    const __nv_bfloat16* Ws, const float* nWs, const __nv_bfloat16* T,
                    const float* nT, int N, int64_t k, float* tau, float* dense, int32_t* list,
                    int32_t* cnt, int cap);
int iq_lp_pick(iq_ctx* ctx, const LpImg& im, Dim3 dist, const LpColumn* cols, int N,
               const int32_t* list, const int32_t* cnt, int cap, float* dl, double tol,
               uint64_t seed, int64_t* rind, int64_t* ncand, int maxK);
int iq_lp_template_features(iq_ctx* ctx, const LpGeo& g, const float* grid, Dim3 gdims,
                            const int64_t* tsrc, const int* tbox, int64_t n, float* out);
int iq_lp_recall(iq_ctx* ctx, const LpImg& im, Dim3 dist, const LpColumn& col,
                 const int32_t* list, const int32_t* cnt, int cap, double tol, float* Dbuf,
                 unsigned* dmin, uint32_t* bits, unsigned long long* counters);
void iq_lp_free(iq_ctx* ctx);
// The proposal's part of one dependency-level chunk of iq_simulate (iq_proposal_host.cu):
// columns = tiles of the chunk x realizations of the group.
struct LpChunk {
  int ncol;
  const int* cfg;                // per column: mask configuration
  const int32_t* lohi;           // per configuration: box lo[3], hi[3]
  const uint32_t* d_klist;       // device: offsets of configuration c at c * T
  const int* cfgK;               // per configuration: offsets of its mask
  int64_t T;
  const int64_t* tile;           // per column: tile index
  const int64_t* start;          // per column: linear start of the tile in a realization's grid
  const int64_t* real;           // per column: global realization index
  const int* rloc;               // per column: realization within the group
  const int* slot;               // per column: index into rind (step in chunk * R + realization)
  const float* sim;              // simulation grids of the group (its first realization at 0)
  int64_t sim_rstride;
  Dim3 sim_dims, tile_dims, dist;
  double tol;
  uint64_t seed;
  int64_t* d_rind;
};
// Whether iq_simulate may use the proposal for this call: parameters for the tile's shape,
// integer-valued data whose FP32 direct sums are exact, no hard or soft data.
bool iq_lp_applies(iq_ctx* ctx, Dim3 tile, int64_t maxK, bool data);
// Runs the proposal for a chunk; *done = 1 when every column was picked (else the caller runs
// the full scan for the chunk). Recall checks follow lp_monitor.
int iq_lp_run_chunk(iq_ctx* ctx, const LpChunk& c, int64_t chunk_index, int* done);
// Records training pairs from the full scan's picks of a chunk (when capturing).
int iq_lp_capture(iq_ctx* ctx, const LpChunk& c, const int32_t* d_cand, const int64_t* d_ncand,
                  int64_t P);
// Resets the per-call statistics of the proposal (start of iq_simulate).
void iq_lp_begin_call(iq_ctx* ctx);
void iq_lp_count_full(iq_ctx* ctx, int64_t ncol);
int iq_lp_capture_reserve(iq_ctx* ctx, int64_t n);
int iq_lp_encode_templates(iq_ctx* ctx, const LpGeo& g, const float* w, const float* grid,
                           Dim3 gdims, const int64_t* tsrc, const int* tbox, int64_t n,
                           __nv_bfloat16* out, float* norm);

// relaxation sizes of src/relaxation.jl:11-36 for a given npatterns (iq_sim.cu)
void iq_relax_sizes(int64_t npat, double tol, int64_t& dbnorm, int64_t& dbzero, int& nnorm,
                    int64_t* seqnorm, int& nzero, int64_t* seqzero);
