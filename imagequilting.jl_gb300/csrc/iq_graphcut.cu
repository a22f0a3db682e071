// Minimum-error boundary cut of the overlap slabs (src/graphcut.jl:5-84).
//
// One CTA per (realization, slab). The lattice graph, the capacities
//   c(u, v) = (|A-B|_u + |A-B|_v) / (|A_v-A_u| + |A_w-A_v| + |B_v-B_u| + |B_w-B_v| + eps())
// (Float32 differences and sums, Float64 division, as Julia does for Float32 arrays) and the
// infinite source/sink slices follow the reference. The max-flow is a synchronous
// push-relabel instead of Boykov-Kolmogorov:
//   * the first slice along the cut dimension is contracted into s, the last into t;
//   * capacities are rounded to multiples of q = 2^(ilogb(cmax) - 47), cmax the largest of
//     the slab, so that every residual (<= 2 cmax) and excess (<= 12 cmax) is a multiple of q
//     below 2^53 q and all flow arithmetic is exact (zero gradient sums give eps-denominator
//     capacities ~2^52 times the others, which unquantized Float64 flows cannot resolve);
//   * so residuals and excesses are kept as int64 counts of q (the same values as the exact
//     Float64 arithmetic, without GB300's narrow FP64 pipe); an arc is open when its residual
//     is positive (the oracle quantizes and tests the same way);
//   * each round: every node on the active list pushes along its admissible arcs
//     (h(u) = h(v) + 1) while it has excess, adding to the receivers' excesses with integer
//     atomics and listing them; then every listed node with excess and no admissible arc
//     relabels in place, and the nodes still active form the next list (a few percent of the
//     slab per round). The flow found depends on the order of the atomics, the cut does not:
//     integer sums are exact, and the set of nodes that can reach t is the same for every
//     maximum preflow;
//   * a global relabel (BFS from t over open arcs) runs at the start, every GR rounds and at
//     the end; nodes that cannot reach t get height NH and stop being active.
// At the end the nodes that can reach t are the sink side of the canonical minimum cut (the
// same set for every maximum flow, which is what BK's sink tree holds at termination), and
// mask = not sink side (graphcut.jl:75-81).
#include "iq_internal.h"

namespace {

constexpr int CUT_MAX_THREADS = 1024;

struct CutArgs {
  StepTask t0;                 // used when tasks is null
  const StepTask* tasks;
  int nreal;                   // CTA (s, y): slab s of realization y % nreal of task y / nreal
  const float* sim; int64_t sx, sy; int64_t sim_rs;
  const float* ti; int64_t tix, tiy; int64_t dx, dy;
  const int64_t* rind;
  const float* A; const float* B;
  uint8_t* out; int64_t slabmax;
  char* scratch; int64_t scratch_per_cta;
  int* status;
  int round_cap;
  unsigned long long* stats;
  int gr_period;
};

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// Slab graph in shared memory. Everything a lookup needs is a scalar or one base pointer:
// an array indexed by a run-time direction would live in local memory and cost a memory
// access per arc.
struct Graph {
  int n, s1, s2;  // nodes; strides of y and z (x has stride 1)
  int d;          // cut dimension
  int L;          // extent along d
  int NH;         // height of s (= number of interior nodes + 2)
  // residuals in units of q: R[2e n + u] for the arc u -> u + stride(e), R[(2e+1) n + u] for
  // the arc u + stride(e) -> u
  long long* R;
  long long* ex;  // excess
  uint8_t* info;  // bits 0-5: neighbour exists in direction 0..5; bits 6-7: kind

  __device__ __forceinline__ int stride(int e) const { return e == 0 ? 1 : (e == 1 ? s1 : s2); }
  __device__ __forceinline__ int kind(int u) const { return info[u] >> 6; }  // 0 interior, 1 s, 2 t
  __device__ __forceinline__ bool nbr(int u, int dir, int& v) const {
    if (!(info[u] >> dir & 1)) return false;
    v = (dir & 1) ? u + stride(dir >> 1) : u - stride(dir >> 1);
    return true;
  }
  template <typename HT>
  __device__ __forceinline__ int height(const HT* hc, int v) const {
    int k = kind(v);
    return k == 1 ? NH : (k == 2 ? 0 : (int)hc[v]);
  }
  __device__ __forceinline__ long long& rf(int e, int u) const { return R[(2 * e) * n + u]; }
  __device__ __forceinline__ long long& rb(int e, int u) const { return R[(2 * e + 1) * n + u]; }
  // residual u->v (and pointers to both arc residuals) for direction dir
  __device__ __forceinline__ void arc(int u, int v, int dir, long long*& ruv, long long*& rvu) const {
    const int e = dir >> 1;
    if (dir & 1) { ruv = R + (2 * e) * n + u; rvu = R + (2 * e + 1) * n + u; }
    else { ruv = R + (2 * e + 1) * n + v; rvu = R + (2 * e) * n + v; }
  }
  __device__ __forceinline__ bool open(const long long* ruv, const long long*) const {
    return *ruv > 0;
  }
};

// Exact heights: breadth-first search from t over open arcs. Each level only examines the
// neighbours of the previous level's frontier (frontier lists fa/fb, counters cnt[2]), so the
// search costs O(edges) instead of O(nodes x levels). Heights are BFS distances, whatever
// order the frontier is filled in. Returns the number of levels.
// heights and BFS frontier entries are HT: 16-bit for slabs below 32768 nodes (a smaller
// shared-memory footprint, two CTAs per SM), else 32-bit
__device__ __forceinline__ bool cas_height(short* p, int expect, int val) {
  return atomicCAS(reinterpret_cast<unsigned short*>(p), (unsigned short)expect,
                   (unsigned short)val) == (unsigned short)expect;
}
__device__ __forceinline__ bool cas_height(int* p, int expect, int val) {
  return atomicCAS(p, expect, val) == expect;
}

template <typename HT>
__device__ __forceinline__ int global_relabel(const Graph& g, HT* hc, HT* fa, HT* fb, int* cnt) {
  if (threadIdx.x == 0) { cnt[0] = 0; cnt[1] = 0; }
  __syncthreads();
  const int dsink = 2 * g.d + 1;  // direction towards the sink slice
  for (int u = threadIdx.x; u < g.n; u += blockDim.x) {
    if (g.kind(u) != 0) continue;
    int h = g.NH;
    int v;
    if (g.nbr(u, dsink, v) && g.kind(v) == 2) {
      long long *ruv, *rvu;
      g.arc(u, v, dsink, ruv, rvu);
      if (g.open(ruv, rvu)) h = 1;
    }
    hc[u] = (HT)h;
    if (h == 1) fa[atomicAdd(&cnt[0], 1)] = (HT)u;
  }
  __syncthreads();
  int level = 1, cur = 0;
  for (;;) {
    const int nf = cnt[cur];
    HT* front = cur ? fb : fa;
    HT* next = cur ? fa : fb;
    if (nf == 0) break;
    if (threadIdx.x == 0) cnt[cur ^ 1] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      const int v = front[i];
#pragma unroll
      for (int dir = 0; dir < 6; ++dir) {
        int u;
        if (!g.nbr(v, dir, u)) continue;
        if (g.kind(u) != 0 || hc[u] != g.NH) continue;
        long long *ruv, *rvu;
        g.arc(u, v, dir ^ 1, ruv, rvu);  // arc u -> v
        if (!g.open(ruv, rvu)) continue;
        if (cas_height(&hc[u], g.NH, level + 1)) next[atomicAdd(&cnt[cur ^ 1], 1)] = (HT)u;
      }
    }
    __syncthreads();
    cur ^= 1;
    ++level;
  }
  __syncthreads();
  return level;
}

// MODE 0: the slab lives in shared memory; the form derives every array from the shared window
// itself, so its loads, stores and atomics are shared-memory instructions rather than generic
// ones. MODE 1: everything in global scratch (too large for shared memory). MODE 2: the
// residuals, heights and node info (what every push and relabel reads) in shared memory, the
// excesses and the BFS frontiers in global scratch (slabs of 8 x 32 x 16 nodes, configs 3-4).
template <typename HT, int MODE>
__global__ void __launch_bounds__(CUT_MAX_THREADS, 1) cut_kernel(const CutArgs a) {
  extern __shared__ __align__(16) char smem[];
  const int s_id = blockIdx.x;
  const int y = blockIdx.y;
  const int r = y % a.nreal;
  const StepTask& tk = a.tasks ? a.tasks[y / a.nreal] : a.t0;
  if (s_id >= tk.nslab) return;
  const CutSlab sl = tk.slab[s_id];
  const int64_t tile_start = tk.start;
  const bool prof = a.stats != nullptr && threadIdx.x == 0;
  const long long t_start = prof ? clock64() : 0;
  long long t_gr = 0;
  Graph g;
  const int ex0 = (int)sl.ext[0], ex1 = (int)sl.ext[1], ex2 = (int)sl.ext[2];
  g.s1 = ex0; g.s2 = ex0 * ex1;
  g.n = ex0 * ex1 * ex2;
  g.d = sl.dim;
  g.L = g.d == 0 ? ex0 : (g.d == 1 ? ex1 : ex2);
  g.NH = g.n / g.L * (g.L > 2 ? g.L - 2 : 0) + 2;
  const int n = g.n;

  char* base = smem;
  char* gbase = a.scratch + (int64_t)(blockIdx.y * gridDim.x + blockIdx.x) * a.scratch_per_cta;
  if constexpr (MODE == 1) base = gbase;
  long long* dp = reinterpret_cast<long long*>(base);
  HT *h0, *h1, *fa, *fb;
  g.R = dp;
  if constexpr (MODE == 2) {
    HT* ip = reinterpret_cast<HT*>(dp + 6 * n);
    h0 = ip;        // heights, double-buffered
    h1 = ip + n;
    g.info = reinterpret_cast<uint8_t*>(ip + 2 * n);
    g.ex = reinterpret_cast<long long*>(gbase);
    fa = reinterpret_cast<HT*>(g.ex + n);  // BFS frontier lists
    fb = fa + n;
  } else {
    g.ex = dp + 6 * n;
    HT* ip = reinterpret_cast<HT*>(dp + 7 * n);
    h0 = ip;
    h1 = ip + n;
    fa = ip + 2 * n;
    fb = ip + 3 * n;
    g.info = reinterpret_cast<uint8_t*>(ip + 4 * n);
  }
  __shared__ int s_cnt[2];
  __shared__ unsigned long long s_cmax;  // bits of the largest capacity
  if (threadIdx.x == 0) s_cmax = 0ull;
  float* Av = reinterpret_cast<float*>(g.ex);  // A and B alias the excesses (8n bytes), which
  float* Bv = Av + n;                          // are first written after the capacities

  // ---- load A (simulation grid) and B (training image at the drawn pattern) ----
  int64_t bstart = 0;
  if (!a.A) {
    const int64_t ri = a.rind[y];
    if (ri < 0) {  // pick failed: no cut (status already set)
      for (int u = threadIdx.x; u < n; u += blockDim.x)
        a.out[((int64_t)y * 6 + s_id) * a.slabmax + u] = 0;
      return;
    }
    const int64_t rx = ri % a.dx, rr = ri / a.dx, ry = rr % a.dy, rz = rr / a.dy;
    bstart = rx + a.tix * (ry + a.tiy * rz);
  }
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    const int x = u % ex0, y = (u / ex0) % ex1, z = u / g.s2;
    uint8_t inf = 0;
    if (x > 0) inf |= 1u;
    if (x + 1 < ex0) inf |= 2u;
    if (y > 0) inf |= 4u;
    if (y + 1 < ex1) inf |= 8u;
    if (z > 0) inf |= 16u;
    if (z + 1 < ex2) inf |= 32u;
    const int cd = g.d == 0 ? x : (g.d == 1 ? y : z);
    inf |= (uint8_t)((cd == 0 ? 1 : (cd == g.L - 1 ? 2 : 0)) << 6);
    g.info[u] = inf;
    if (a.A) {
      Av[u] = a.A[u];
      Bv[u] = a.B[u];
    } else {
      const int64_t lx = sl.off[0] + x, ly = sl.off[1] + y, lz = sl.off[2] + z;
      Av[u] = a.sim[(int64_t)r * a.sim_rs + tile_start + lx + a.sx * (ly + a.sy * lz)];
      Bv[u] = a.ti[bstart + lx + a.tix * (ly + a.tiy * lz)];
    }
  }
  __syncthreads();

  // ---- capacities (graphcut.jl:22-50) ----
  const double EPS = 2.220446049250313e-16;  // eps(Float64) = 2^-52
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      int v;
      if (!g.nbr(u, 2 * e + 1, v)) continue;
      const bool ok = (g.info[v] >> (2 * e + 1)) & 1;
      const int w = ok ? v + g.stride(e) : v;
      const float Du = fabsf(__fsub_rn(Av[u], Bv[u]));
      const float Dv = fabsf(__fsub_rn(Av[v], Bv[v]));
      const float gAu = fabsf(__fsub_rn(Av[v], Av[u]));
      const float gBu = fabsf(__fsub_rn(Bv[v], Bv[u]));
      const float gAv = ok ? fabsf(__fsub_rn(Av[w], Av[v])) : gAu;
      const float gBv = ok ? fabsf(__fsub_rn(Bv[w], Bv[v])) : gBu;
      const float num = __fadd_rn(Du, Dv);
      float den = __fadd_rn(gAu, gAv);
      den = __fadd_rn(den, gBu);
      den = __fadd_rn(den, gBv);
      const double cap = __ddiv_rn((double)num, __dadd_rn((double)den, EPS));
      g.rf(e, u) = dbits(cap);  // the double's bits until the quantization below
      atomicMax(&s_cmax, (unsigned long long)dbits(cap));
    }
  }
  __syncthreads();
  // ---- capacities in units of q = 2^(ilogb(cmax) - 47), rounded half to even: the flows
  // are then exact integers (<= 2^49 per arc), the same numbers the oracle's quantized
  // Float64 arithmetic produces ----
  {
    int sh = s_cmax != 0ull ? ilogb(__longlong_as_double((long long)s_cmax)) - 47 : 0;
    if (sh < -1074) sh = -1074;
    for (int u = threadIdx.x; u < n; u += blockDim.x)
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        int v;
        if (!g.nbr(u, 2 * e + 1, v)) continue;
        const long long k = s_cmax != 0ull
                                ? (long long)rint(ldexp(__longlong_as_double(g.rf(e, u)), -sh))
                                : 0ll;
        g.rf(e, u) = k;
        g.rb(e, u) = k;
      }
    __syncthreads();
  }

  // ---- saturate the source slice: push c(s, v) into every interior node of slice 1 ----
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    long long e0 = 0;
    if (g.kind(u) == 0 && g.kind(u - g.stride(g.d)) == 1) {
      const int sN = u - g.stride(g.d);
      const long long c = g.rf(g.d, sN);
      g.rf(g.d, sN) = 0;
      g.rb(g.d, sN) = 2 * c;
      e0 = c;
    }
    g.ex[u] = e0;
  }
  __syncthreads();

  // heights live in h0 (relabels are in place: heights only grow, so a stale neighbour
  // height read by a concurrent relabel still gives a valid label); between global relabels
  // the BFS frontier lists hold the work lists and h1 the "listed" flags
  HT* const hc = h0;
  HT* const L = fa;     // nodes with excess and height below NH (pushed this round)
  HT* const Nl = fb;    // nodes to relabel: the pushers left with excess and the receivers
  HT* const flag = h1;  // 1 while a node is in Nl
  // list lengths, double-buffered by round parity `par`: a round reads |L| = s_cl[par] and
  // appends the receivers to Nl through s_cn[par], the next round's L through s_cl[par ^ 1];
  // the counters of the other parity are zeroed while nobody uses them, so a round needs only
  // a barrier after its push phase and one after its relabel phase
  __shared__ int s_cl[2], s_cn[2];
  int par = 0;
  int round = 0, levels = 0;
  long long nactive = 0;
  const long long t_setup = prof ? clock64() : 0;
  auto relabel_all = [&]() {
    const long long t = prof ? clock64() : 0;
    levels += global_relabel(g, hc, fa, fb, s_cnt);
    if (prof) t_gr += clock64() - t;
  };
  // the active list from scratch (after a global relabel, which used the lists as frontiers)
  auto rebuild = [&]() {
    par = 0;
    if (threadIdx.x == 0) { s_cl[0] = 0; s_cl[1] = 0; s_cn[0] = 0; s_cn[1] = 0; }
    __syncthreads();
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
      flag[u] = 0;
      if (g.kind(u) == 0 && g.ex[u] > 0 && (int)hc[u] < g.NH) L[atomicAdd(&s_cl[0], 1)] = (HT)u;
    }
    __syncthreads();
  };
  auto list_once = [&](int v) {  // append v to Nl unless it is there already
    if (cas_height(&flag[v], 0, 1)) Nl[atomicAdd(&s_cn[par], 1)] = (HT)v;
  };
  // push phase over L[0, A): every listed node pushes along its admissible arcs while it has
  // excess; the receivers' excesses are updated with integer atomics (exact in any order). Two
  // ends of one edge never push on it in the same round (that would need h(u) = h(v) + 1 and
  // h(v) = h(u) + 1), so each residual has one writer.
  auto push_phase = [&](int A, int t0, int step) {
    for (int i = t0; i < A; i += step) {
      const int u = L[i];
      const int hu = hc[u];
      long long e = g.ex[u];
      const long long e0 = e;
#pragma unroll
      for (int dir = 0; dir < 6; ++dir) {
        if (e <= 0) break;
        int v;
        if (!g.nbr(u, dir, v)) continue;
        if (hu != g.height(hc, v) + 1) continue;
        long long *ruv, *rvu;
        g.arc(u, v, dir, ruv, rvu);
        const long long rr = *ruv;
        if (rr <= 0) continue;
        const long long delta = e < rr ? e : rr;
        *ruv = rr - delta;
        *rvu += delta;
        e -= delta;
        if (g.kind(v) == 0) {
          atomicAdd(reinterpret_cast<unsigned long long*>(&g.ex[v]), (unsigned long long)delta);
          list_once(v);
        }
      }
      if (e != e0)
        atomicAdd(reinterpret_cast<unsigned long long*>(&g.ex[u]), (unsigned long long)(e - e0));
      if (e > 0) list_once(u);
    }
  };
  // relabel phase over Nl[0, B): a node left with excess and no admissible arc moves to 1 + the
  // lowest neighbour it still has residual capacity to; the nodes that stay active form the
  // next round's list
  auto relabel_phase = [&](int B, int t0, int step) {
    for (int i = t0; i < B; i += step) {
      const int u = Nl[i];
      flag[u] = 0;
      const long long e = g.ex[u];
      int hu = hc[u];
      if (e > 0 && hu < g.NH) {
        bool adm = false;
        int mh = 0x7fffffff;
#pragma unroll
        for (int dir = 0; dir < 6; ++dir) {
          int v;
          if (!g.nbr(u, dir, v)) continue;
          long long *ruv, *rvu;
          g.arc(u, v, dir, ruv, rvu);
          if (!g.open(ruv, rvu)) continue;
          const int hv = g.height(hc, v);
          if (hu == hv + 1) { adm = true; break; }
          mh = min(mh, hv);
        }
        if (!adm) {
          hu = mh >= g.NH - 1 ? g.NH : mh + 1;
          hc[u] = (HT)hu;
        }
        if (hu < g.NH) L[atomicAdd(&s_cl[par ^ 1], 1)] = (HT)u;
      }
    }
  };
  __shared__ int s_round, s_par;
  if (g.L > 2) {
    relabel_all();
    rebuild();
    bool capped = false;
    for (;;) {
      const int A = s_cl[par];
      if (A == 0) break;
      if (A <= 32) {
        // Rounds with at most 32 active nodes run on warp 0 alone, synchronised by __syncwarp,
        // until the list grows past 32 or empties, or the round cap or a global relabel is due
        // (the same rounds as the block form, without its barriers).
        __syncthreads();  // every thread has read A before warp 0 moves the counters on
        if (threadIdx.x < 32) {
          const int lane = threadIdx.x;
          int Aw = A;
          for (;;) {
            nactive += Aw;
            if (lane == 0) s_cn[par ^ 1] = 0;
            push_phase(Aw, lane, 32);
            __syncwarp();
            const int B = s_cn[par];
            if (lane == 0) s_cl[par] = 0;
            relabel_phase(B, lane, 32);
            __syncwarp();
            ++round;
            par ^= 1;
            Aw = s_cl[par];
            if (Aw == 0 || Aw > 32 || round >= a.round_cap || round % a.gr_period == 0) break;
          }
          if (lane == 0) { s_round = round; s_par = par; }
        }
        __syncthreads();
        round = s_round;
        par = s_par;
      } else {
        nactive += A;
        if (threadIdx.x == 0) s_cn[par ^ 1] = 0;
        push_phase(A, threadIdx.x, blockDim.x);
        __syncthreads();
        const int B = s_cn[par];
        if (threadIdx.x == 0) s_cl[par] = 0;
        relabel_phase(B, threadIdx.x, blockDim.x);
        __syncthreads();
        ++round;
        par ^= 1;
      }
      if (round >= a.round_cap && s_cl[par] > 0) { capped = true; break; }
      if (round % a.gr_period == 0) {
        relabel_all();
        rebuild();
      }
    }
    relabel_all();
    __syncthreads();
    if (capped && threadIdx.x == 0) iq_dev_fail(a.status, IQ_ERR_CUTCAP);
  }

  if (a.stats && threadIdx.x == 0) {
    const long long t_end = clock64();
    atomicAdd(a.stats + ST_CUT_TSETUP, (unsigned long long)(t_setup - t_start));
    atomicAdd(a.stats + ST_CUT_TGR, (unsigned long long)t_gr);
    atomicAdd(a.stats + ST_CUT_TROUNDS, (unsigned long long)(t_end - t_setup - t_gr));
    atomicAdd(a.stats + ST_CUT_ROUNDS, (unsigned long long)round);
    atomicAdd(a.stats + ST_CUT_NODES, (unsigned long long)n);
    atomicAdd(a.stats + ST_CUT_ACTIVE, (unsigned long long)nactive);
    atomicAdd(a.stats + ST_CUT_LEVELS, (unsigned long long)levels);
    atomicAdd(a.stats + ST_CUT_CTAS, 1ull);
    atomicMax(a.stats + ST_CUT_MAXROUNDS, (unsigned long long)round);
    atomicMax(a.stats + ST_CUT_MAXLEVELS, (unsigned long long)levels);
  }
  // ---- mask: not sink side ----
  uint8_t* out = a.out + ((int64_t)y * 6 + s_id) * a.slabmax;
  for (int u = threadIdx.x; u < n; u += blockDim.x) {
    const int k = g.kind(u);
    int M = k == 1 ? 1 : (k == 2 ? 0 : (hc[u] >= g.NH ? 1 : 0));
    out[u] = (uint8_t)(sl.next ? !M : M);
  }
}

}  // namespace

namespace {
size_t cut_bytes(int64_t nodes, int hbytes) {
  // residuals (6n int64), excess (n int64), two heights and two BFS frontiers (4n HT), node
  // info (n bytes)
  size_t b = (size_t)nodes * (7 * 8 + 4 * hbytes + 1);
  return (b + 255) & ~(size_t)255;
}
// MODE 2: shared part (residuals, two heights, node info) and global part (excess, frontiers)
size_t cut_bytes_shared2(int64_t nodes, int hbytes) {
  return ((size_t)nodes * (6 * 8 + 2 * hbytes + 1) + 255) & ~(size_t)255;
}
size_t cut_bytes_global2(int64_t nodes, int hbytes) {
  return ((size_t)nodes * (8 + 2 * hbytes) + 255) & ~(size_t)255;
}
constexpr int64_t CUT_SHORT_MAX = 32767;  // largest slab with 16-bit heights and indices
}  // namespace

size_t iq_cut_scratch_bytes(int64_t nodes) {
  return cut_bytes(nodes, nodes <= CUT_SHORT_MAX ? 2 : 4);
}

int iq_launch_cut(iq_ctx* ctx, const CutLaunch& L) {
  const int nslab_max = L.tasks ? L.nslab_max : L.t0.nslab;
  if (nslab_max <= 0 || L.nreal <= 0 || L.ntask <= 0) return IQ_OK;
  CutArgs a;
  a.t0 = L.t0;
  a.tasks = L.tasks;
  a.nreal = L.nreal;
  a.sim = L.sim; a.sx = L.sim_dims.x; a.sy = L.sim_dims.y; a.sim_rs = L.sim_rstride;
  a.ti = L.ti; a.tix = L.ti_dims.x; a.tiy = L.ti_dims.y;
  a.dx = L.dist_dims.x; a.dy = L.dist_dims.y;
  a.rind = L.rind;
  a.A = L.A; a.B = L.B;
  a.out = L.out; a.slabmax = L.slabmax;
  a.status = L.status;
  a.round_cap = L.round_cap;
  a.stats = L.stats;
  a.gr_period = L.gr_period > 0 ? L.gr_period : 32;
  const int64_t nmax = L.slabmax;
  const size_t need = iq_cut_scratch_bytes(nmax);
  const bool narrow = nmax <= CUT_SHORT_MAX;
  const int hb = narrow ? 2 : 4;
  // dynamic shared memory may use the opt-in maximum minus the kernel's static part
  auto limit_of = [&](void (*k)(CutArgs), int& lim) -> int {
    int dev = 0, v = 0;
    IQ_CUDA_OK(cudaGetDevice(&dev));
    IQ_CUDA_OK(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    IQ_CUDA_OK(cudaFuncGetAttributes(&fa, k));
    lim = v - (int)fa.sharedSizeBytes;
    IQ_CUDA_OK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    return IQ_OK;
  };
  void (*kern)(CutArgs) = narrow ? cut_kernel<short, 0> : cut_kernel<int, 0>;
  int smem_limit = 0;
  if (int rc = limit_of(kern, smem_limit)) return rc;
  size_t dyn = 0;
  a.scratch = nullptr;
  a.scratch_per_cta = 0;
  if ((int64_t)need <= smem_limit) {
    dyn = need;
  } else {
    if (!L.scratch || L.scratch_per_cta < (int64_t)need)
      return iq_set_error(IQ_ERR_LIMIT, "graph cut slab of %lld nodes needs global scratch",
                          (long long)nmax);
    a.scratch = (char*)L.scratch;
    a.scratch_per_cta = L.scratch_per_cta;
    void (*k2)(CutArgs) = narrow ? cut_kernel<short, 2> : cut_kernel<int, 2>;
    int lim2 = 0;
    if (int rc = limit_of(k2, lim2)) return rc;
    if ((int64_t)cut_bytes_shared2(nmax, hb) <= lim2 &&
        (int64_t)cut_bytes_global2(nmax, hb) <= L.scratch_per_cta) {
      kern = k2;
      dyn = cut_bytes_shared2(nmax, hb);
    } else {
      kern = narrow ? cut_kernel<short, 1> : cut_kernel<int, 1>;
    }
  }
  const int threads = (L.threads == 256 || L.threads == 1024) ? L.threads : 512;
  dim3 grid((unsigned)nslab_max, (unsigned)(L.ntask * L.nreal));
  iq_timer_start(ctx, "graphcut");
  kern<<<grid, threads, dyn, ctx->stream>>>(a);
  iq_timer_stop(ctx, "graphcut", 0);
  iq_count(ctx);
  IQ_CUDA_OK(cudaGetLastError());
  return IQ_OK;
}
