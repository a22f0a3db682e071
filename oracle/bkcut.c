/*
 * oracle/bkcut.c -- CPU oracle of the minimum-error boundary cut.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by oracle/iqsim_oracle.py for the tests, smoke() and the
 * CPU baseline of bench.py. It is never linked into the product library.
 *
 * Restates src/graphcut.jl:5-84 of ImageQuilting.jl v1.3.1:
 *   - lattice graph over the overlap slab, one undirected edge per pair (u, u+e_d)
 *     (graphcut.jl:22-50);
 *   - capacity (Du + Dv) / (dAu + dAv + dBu + dBv + eps()) with the border rule that repeats
 *     the u-gradient when u+2e_d falls outside (graphcut.jl:29-48);
 *   - source s -> every voxel of the first slice along `dim`, last slice -> sink t, both with
 *     infinite capacity (graphcut.jl:53-67);
 *   - Boykov-Kolmogorov max-flow (graphcut.jl:70, GraphsFlows 0.1 BoykovKolmogorovAlgorithm,
 *     not vendored: restated from Boykov & Kolmogorov, "An experimental comparison of
 *     min-cut/max-flow algorithms for energy minimization in vision", PAMI 2004);
 *   - mask = node label is "free" or "source tree", i.e. NOT in the sink tree
 *     (graphcut.jl:75-81).
 *
 * Arithmetic follows the element type of A and B like the Julia code does: the differences,
 * gradients and their sums are in the element type (float or double); the final sum with
 * eps() = 2^-52 and the division are in double (Julia promotes Float32 + Float64).
 *
 * Exact arithmetic. Where a gradient sum is zero the denominator is eps() and the capacity
 * is ~2^52 times larger than its neighbours', so a Float64 max-flow cannot resolve the small
 * arcs and different flow orders (BK here, push-relabel on the GPU, the Julia BK) stop at
 * different minimum cuts. Every capacity is therefore rounded to a multiple of
 * q = 2^(ilogb(cmax) - 47), cmax the largest capacity of the slab (round half to even). All
 * residuals (<= 2 cmax) and node excesses (<= 12 cmax) are then multiples of q below 2^53 q,
 * every push or augmentation is exact, an arc is open exactly when its residual is > 0, and
 * the set of nodes that can reach t is the same for every maximum flow (and preflow): BK's
 * sink tree at termination and the GPU's final breadth-first search both return it.
  */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define FREE 0
#define SRC 1
#define SNK 2

typedef struct {
    int a, b;         /* a = lower node, b = a + stride */
    double r_ab, r_ba;
} edge_t;

static inline uint64_t dbits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double bitsd(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

/* Round every capacity to a multiple of q = 2^(ilogb(cmax) - 47) (see the header). */
static void quantize_caps(double *c, long long n, long long stride) {
    double cmax = 0.0;
    for (long long i = 0; i < n; i++) if (c[i * stride] > cmax) cmax = c[i * stride];
    if (!(cmax > 0.0)) return;
    int sh = ilogb(cmax) - 47;
    if (sh < -1074) sh = -1074;
    for (long long i = 0; i < n; i++) c[i * stride] = ldexp(rint(ldexp(c[i * stride], -sh)), sh);
}

/* graph with explicit terminals s = nvox, t = nvox + 1 */
typedef struct {
    int nvox, n;
    int nedges;
    edge_t *edges;
    /* incidence: per node, list of (edge id << 1 | side), side 0 = node is a, 1 = node is b */
    int *inc_start, *inc;
    /* terminal arcs: s->u for first slice (infinite), u->t for last slice (infinite) */
    unsigned char *is_first, *is_last;
    double *r_su, *r_us, *r_ut, *r_tu;  /* per voxel */
} graph_t;

/* residual capacity of arc p->q given an incidence entry of p */
static inline double arc_res(const graph_t *g, int ent, int *q) {
    const edge_t *e = &g->edges[ent >> 1];
    if ((ent & 1) == 0) { *q = e->b; return e->r_ab; }
    *q = e->a; return e->r_ba;
}

/* BK state */
typedef struct {
    unsigned char *tree;
    int *parent;       /* parent node, -1 none */
    int *parent_ent;   /* how the parent link is stored: >=0 lattice incidence entry of child,
                          -2 terminal link */
    int *aq, ahead, atail, acap; unsigned char *inA;
    int *oq, ohead, otail, ocap;
} bk_t;

static void opush(bk_t *k, int v) {
    if (k->otail >= k->ocap) {
        k->ocap *= 2;
        k->oq = (int *)realloc(k->oq, sizeof(int) * (size_t)k->ocap);
    }
    k->oq[k->otail++] = v;
}

static void apush(bk_t *k, int v) {
    if (k->inA[v]) return;
    k->inA[v] = 1;
    k->aq[k->atail % k->acap] = v;
    k->atail++;
}

/* residual of the arc from x to y where y is a neighbour reached through x's entry ent */
static inline int lattice_open(const graph_t *g, int ent_of_x, int *y) {
    return arc_res(g, ent_of_x, y) > 0.0;
}
/* residual of the reverse arc (y -> x) for x's entry ent */
static inline int lattice_open_rev(const graph_t *g, int ent_of_x) {
    const edge_t *e = &g->edges[ent_of_x >> 1];
    double r = (ent_of_x & 1) == 0 ? e->r_ba : e->r_ab;
    return r > 0.0;
}

/* does node v trace back to its terminal through valid parent links? */
static int has_origin(const graph_t *g, const bk_t *k, int v) {
    int steps = 0;
    while (v != g->nvox && v != g->nvox + 1) {
        if (k->parent[v] < 0) return 0;
        v = k->parent[v];
        if (++steps > g->n + 2) return 0;
    }
    return 1;
}

static int run_bk(graph_t *g, bk_t *k, long long max_aug) {
    const int s = g->nvox, t = g->nvox + 1;
    k->tree[s] = SRC; k->tree[t] = SNK;
    apush(k, s); apush(k, t);
    long long naug = 0;
    for (;;) {
        /* ---- growth ---- */
        int found = 0, ps = -1, pt = -1;   /* meeting arc ps (S side) -> pt (T side) */
        while (k->ahead < k->atail && !found) {
            int p = k->aq[k->ahead % k->acap];
            if (!k->inA[p] || k->tree[p] == FREE) { k->ahead++; k->inA[p] = 0; continue; }
            if (p == s) {
                for (int v = 0; v < g->nvox && !found; v++) {
                    if (!g->is_first[v] || !(g->r_su[v] > 0)) continue;
                    if (k->tree[v] == FREE) { k->tree[v] = SRC; k->parent[v] = s; k->parent_ent[v] = -2; apush(k, v); }
                    else if (k->tree[v] == SNK) { found = 1; ps = s; pt = v; }
                }
            } else if (p == t) {
                for (int v = 0; v < g->nvox && !found; v++) {
                    if (!g->is_last[v] || !(g->r_ut[v] > 0)) continue;
                    if (k->tree[v] == FREE) { k->tree[v] = SNK; k->parent[v] = t; k->parent_ent[v] = -2; apush(k, v); }
                    else if (k->tree[v] == SRC) { found = 1; ps = v; pt = t; }
                }
            } else if (k->tree[p] == SRC) {
                for (int i = g->inc_start[p]; i < g->inc_start[p + 1] && !found; i++) {
                    int q;
                    if (!lattice_open(g, g->inc[i], &q)) continue;
                    if (k->tree[q] == FREE) { k->tree[q] = SRC; k->parent[q] = p; k->parent_ent[q] = -1; apush(k, q); }
                    else if (k->tree[q] == SNK) { found = 1; ps = p; pt = q; }
                }
                if (!found && g->is_last[p] && g->r_ut[p] > 0) {
                    found = 1; ps = p; pt = t;
                }
            } else { /* SNK: grow through arcs q -> p */
                for (int i = g->inc_start[p]; i < g->inc_start[p + 1] && !found; i++) {
                    int ent = g->inc[i];
                    const edge_t *e = &g->edges[ent >> 1];
                    int q = (ent & 1) == 0 ? e->b : e->a;
                    if (!lattice_open_rev(g, ent)) continue;
                    if (k->tree[q] == FREE) { k->tree[q] = SNK; k->parent[q] = p; k->parent_ent[q] = -1; apush(k, q); }
                    else if (k->tree[q] == SRC) { found = 1; ps = q; pt = p; }
                }
                if (!found && g->is_first[p] && g->r_su[p] > 0) { found = 1; ps = s; pt = p; }
            }
            if (!found) { k->inA[p] = 0; k->ahead++; }
        }
        if (!found) break;
        if (++naug > max_aug) return -1;

        /* ---- augmentation: path s ~> ps -> pt ~> t ---- */
        /* collect arcs as (from, to) pairs */
        int cap = g->n + 4;
        int *pf = (int *)malloc(sizeof(int) * cap * 2);
        int np = 0;
        /* S part: from ps back to s, stored reversed */
        int stackn = 0;
        int *stk = (int *)malloc(sizeof(int) * (g->n + 4));
        for (int v = ps; v != s; v = k->parent[v]) stk[stackn++] = v;
        int prev = s;
        for (int i = stackn - 1; i >= 0; i--) { pf[2 * np] = prev; pf[2 * np + 1] = stk[i]; np++; prev = stk[i]; }
        pf[2 * np] = ps; pf[2 * np + 1] = pt; np++;
        for (int v = pt; v != t; v = k->parent[v]) { pf[2 * np] = v; pf[2 * np + 1] = k->parent[v]; np++; }
        free(stk);

        /* residual access for a directed pair */
        double delta = INFINITY;
        for (int i = 0; i < np; i++) {
            int a = pf[2 * i], b = pf[2 * i + 1];
            double r;
            if (a == s) r = g->r_su[b];
            else if (b == t) r = g->r_ut[a];
            else {
                r = -1;
                for (int j = g->inc_start[a]; j < g->inc_start[a + 1]; j++) {
                    int q; double rr = arc_res(g, g->inc[j], &q);
                    if (q == b) { r = rr; break; }
                }
            }
            if (r < delta) delta = r;
        }
        for (int i = 0; i < np; i++) {
            int a = pf[2 * i], b = pf[2 * i + 1];
            if (a == s) {
                g->r_su[b] -= delta; g->r_us[b] += delta;
                if (!(g->r_su[b] > 0) && k->tree[b] == SRC && k->parent[b] == s) {
                    k->parent[b] = -1; opush(k, b);
                }
            } else if (b == t) {
                g->r_ut[a] -= delta; g->r_tu[a] += delta;
                if (!(g->r_ut[a] > 0) && k->tree[a] == SNK && k->parent[a] == t) {
                    k->parent[a] = -1; opush(k, a);
                }
            } else {
                for (int j = g->inc_start[a]; j < g->inc_start[a + 1]; j++) {
                    int ent = g->inc[j];
                    edge_t *e = &g->edges[ent >> 1];
                    int q = (ent & 1) == 0 ? e->b : e->a;
                    if (q != b) continue;
                    if ((ent & 1) == 0) { e->r_ab -= delta; e->r_ba += delta; }
                    else { e->r_ba -= delta; e->r_ab += delta; }
                    if (!lattice_open(g, ent, &q)) {
                        if (k->tree[a] == SRC && k->tree[b] == SRC && k->parent[b] == a) {
                            k->parent[b] = -1; opush(k, b);
                        }
                        if (k->tree[a] == SNK && k->tree[b] == SNK && k->parent[a] == b) {
                            k->parent[a] = -1; opush(k, a);
                        }
                    }
                    break;
                }
            }
        }
        free(pf);

        /* ---- adoption ---- */
        while (k->ohead < k->otail) {
            int p = k->oq[k->ohead++];
            if (k->parent[p] >= 0) continue;
            int tr = k->tree[p];
            int newpar = -1;
            /* candidate parents */
            if (tr == SRC) {
                if (g->is_first[p] && g->r_su[p] > 0) newpar = s;
                for (int i = g->inc_start[p]; i < g->inc_start[p + 1] && newpar < 0; i++) {
                    int ent = g->inc[i];
                    const edge_t *e = &g->edges[ent >> 1];
                    int q = (ent & 1) == 0 ? e->b : e->a;
                    if (k->tree[q] != SRC || !lattice_open_rev(g, ent)) continue;
                    if (has_origin(g, k, q)) newpar = q;
                }
            } else {
                if (g->is_last[p] && g->r_ut[p] > 0) newpar = t;
                for (int i = g->inc_start[p]; i < g->inc_start[p + 1] && newpar < 0; i++) {
                    int q;
                    if (!lattice_open(g, g->inc[i], &q)) continue;
                    if (k->tree[q] != SNK) continue;
                    if (has_origin(g, k, q)) newpar = q;
                }
            }
            if (newpar >= 0) { k->parent[p] = newpar; continue; }
            /* no valid parent: p becomes free */
            for (int i = g->inc_start[p]; i < g->inc_start[p + 1]; i++) {
                int ent = g->inc[i];
                const edge_t *e = &g->edges[ent >> 1];
                int q = (ent & 1) == 0 ? e->b : e->a;
                if (k->tree[q] != tr) continue;
                int qq;
                int open = (tr == SRC) ? lattice_open_rev(g, ent) : lattice_open(g, ent, &qq);
                if (open) apush(k, q);
                if (k->parent[q] == p) { k->parent[q] = -1; opush(k, q); }
            }
            if (tr == SRC && g->is_first[p]) apush(k, s);
            if (tr == SNK && g->is_last[p]) apush(k, t);
            k->tree[p] = FREE;
            k->inA[p] = 0;
        }
        k->ohead = k->otail = 0;
    }
    return 0;
}

/*
 * oracle_graphcut: A, B are column-major arrays of `nd` dims with extents sz[0..nd-1]
 * (dim 0 fastest); elem = 4 (float) or 8 (double). dim is 0-based. mask[v] = 1 when v is
 * not in the sink tree. Returns 0, or -1 when the augmentation cap was hit, -2 bad input.
 * If cut_cost != NULL it receives the sum of capacities of lattice edges from mask=1 to
 * mask=0 nodes.
 */
int oracle_graphcut(const void *A, const void *B, int elem, int nd, const long long *sz, int dim,
                    unsigned char *mask, double *cut_cost) {
    if (nd < 1 || nd > 3 || dim < 0 || dim >= nd || (elem != 4 && elem != 8)) return -2;
    long long ext[3] = {1, 1, 1}, stride[3];
    long long nv = 1;
    for (int d = 0; d < nd; d++) { ext[d] = sz[d]; nv *= sz[d]; }
    stride[0] = 1; stride[1] = ext[0]; stride[2] = ext[0] * ext[1];
    if (nv <= 0) return -2;
    graph_t g;
    memset(&g, 0, sizeof(g));
    g.nvox = (int)nv; g.n = (int)nv + 2;
    long long maxe = 3 * nv;
    g.edges = (edge_t *)malloc(sizeof(edge_t) * maxe);
    int *deg = (int *)calloc(g.n + 1, sizeof(int));
    const float *Af = (const float *)A, *Bf = (const float *)B;
    const double *Ad = (const double *)A, *Bd = (const double *)B;
    const double EPS = 2.220446049250313e-16; /* eps(Float64) = 2^-52 */
    for (int d = 0; d < 3; d++) {
        if (ext[d] < 2) continue;
        for (long long z = 0; z < ext[2]; z++)
            for (long long y = 0; y < ext[1]; y++)
                for (long long x = 0; x < ext[0]; x++) {
                    long long c[3] = {x, y, z};
                    if (c[d] + 1 >= ext[d]) continue;
                    long long u = x + stride[1] * y + stride[2] * z;
                    long long v = u + stride[d];
                    int ok = c[d] + 2 < ext[d];
                    long long w = v + stride[d];
                    double cap;
                    if (elem == 4) {
                        float Du = fabsf(Af[u] - Bf[u]);
                        float Dv = fabsf(Af[v] - Bf[v]);
                        float gAu = fabsf(Af[v] - Af[u]);
                        float gBu = fabsf(Bf[v] - Bf[u]);
                        float gAv = ok ? fabsf(Af[w] - Af[v]) : gAu;
                        float gBv = ok ? fabsf(Bf[w] - Bf[v]) : gBu;
                        float num = Du + Dv;
                        float den = gAu + gAv;
                        den = den + gBu;
                        den = den + gBv;
                        cap = (double)num / ((double)den + EPS);
                    } else {
                        double Du = fabs(Ad[u] - Bd[u]);
                        double Dv = fabs(Ad[v] - Bd[v]);
                        double gAu = fabs(Ad[v] - Ad[u]);
                        double gBu = fabs(Bd[v] - Bd[u]);
                        double gAv = ok ? fabs(Ad[w] - Ad[v]) : gAu;
                        double gBv = ok ? fabs(Bd[w] - Bd[v]) : gBu;
                        double num = Du + Dv;
                        double den = gAu + gAv;
                        den = den + gBu;
                        den = den + gBv;
                        cap = num / (den + EPS);
                    }
                    edge_t *e = &g.edges[g.nedges++];
                    e->a = (int)u; e->b = (int)v; e->r_ab = cap; e->r_ba = cap;
                    deg[u]++; deg[v]++;
                }
    }
    {
        double *caps = (double *)malloc(sizeof(double) * (g.nedges + 1));
        for (int i = 0; i < g.nedges; i++) caps[i] = g.edges[i].r_ab;
        quantize_caps(caps, g.nedges, 1);
        for (int i = 0; i < g.nedges; i++) { g.edges[i].r_ab = caps[i]; g.edges[i].r_ba = caps[i]; }
        free(caps);
    }
    g.inc_start = (int *)malloc(sizeof(int) * (g.n + 1));
    g.inc_start[0] = 0;
    for (int i = 0; i < g.n; i++) g.inc_start[i + 1] = g.inc_start[i] + deg[i];
    g.inc = (int *)malloc(sizeof(int) * (g.inc_start[g.n] + 1));
    memset(deg, 0, sizeof(int) * (g.n + 1));
    /* incidence in a fixed order: edges in creation order */
    for (int i = 0; i < g.nedges; i++) {
        int a = g.edges[i].a, b = g.edges[i].b;
        g.inc[g.inc_start[a] + deg[a]++] = (i << 1) | 0;
        g.inc[g.inc_start[b] + deg[b]++] = (i << 1) | 1;
    }
    free(deg);
    g.is_first = (unsigned char *)calloc(nv, 1);
    g.is_last = (unsigned char *)calloc(nv, 1);
    g.r_su = (double *)calloc(nv, sizeof(double));
    g.r_us = (double *)calloc(nv, sizeof(double));
    g.r_ut = (double *)calloc(nv, sizeof(double));
    g.r_tu = (double *)calloc(nv, sizeof(double));
    for (long long z = 0; z < ext[2]; z++)
        for (long long y = 0; y < ext[1]; y++)
            for (long long x = 0; x < ext[0]; x++) {
                long long c[3] = {x, y, z};
                long long u = x + stride[1] * y + stride[2] * z;
                if (c[dim] == 0) { g.is_first[u] = 1; g.r_su[u] = INFINITY; }
                if (c[dim] == ext[dim] - 1) { g.is_last[u] = 1; g.r_ut[u] = INFINITY; }
            }

    bk_t k;
    memset(&k, 0, sizeof(k));
    k.tree = (unsigned char *)calloc(g.n, 1);
    k.parent = (int *)malloc(sizeof(int) * g.n);
    k.parent_ent = (int *)malloc(sizeof(int) * g.n);
    for (int i = 0; i < g.n; i++) { k.parent[i] = -1; k.parent_ent[i] = -1; }
    k.acap = g.n + 8;
    k.aq = (int *)malloc(sizeof(int) * k.acap);
    k.inA = (unsigned char *)calloc(g.n, 1);
    k.ocap = 4 * g.n + 64;
    k.oq = (int *)malloc(sizeof(int) * (size_t)k.ocap);
    int rc = run_bk(&g, &k, 1000000000LL);

    if (rc == 0) {
        for (long long v = 0; v < nv; v++) mask[v] = k.tree[v] != SNK;
        if (cut_cost) {
            /* recompute capacities as half the residual sum (r_ab + r_ba = 2c) */
            double cc = 0;
            for (int i = 0; i < g.nedges; i++) {
                int a = g.edges[i].a, b = g.edges[i].b;
                double c = 0.5 * (g.edges[i].r_ab + g.edges[i].r_ba);
                if (mask[a] != mask[b]) cc += c;
            }
            *cut_cost = cc;
        }
    }
    free(g.edges); free(g.inc_start); free(g.inc); free(g.is_first); free(g.is_last);
    free(g.r_su); free(g.r_us); free(g.r_ut); free(g.r_tu);
    free(k.tree); free(k.parent); free(k.parent_ent); free(k.aq); free(k.inA); free(k.oq);
    return rc;
}

/* Capacities only (for tests): writes one quantized value per lattice edge in creation order
 * (dims 0,1,2; within a dim, column-major over the lower node). Returns the edge count. */
long long oracle_capacities(const void *A, const void *B, int elem, int nd, const long long *sz,
                            double *out) {
    long long ext[3] = {1, 1, 1}, stride[3];
    for (int d = 0; d < nd; d++) ext[d] = sz[d];
    stride[0] = 1; stride[1] = ext[0]; stride[2] = ext[0] * ext[1];
    const float *Af = (const float *)A, *Bf = (const float *)B;
    const double *Ad = (const double *)A, *Bd = (const double *)B;
    const double EPS = 2.220446049250313e-16;
    long long n = 0;
    for (int d = 0; d < 3; d++) {
        if (ext[d] < 2) continue;
        for (long long z = 0; z < ext[2]; z++)
            for (long long y = 0; y < ext[1]; y++)
                for (long long x = 0; x < ext[0]; x++) {
                    long long c[3] = {x, y, z};
                    if (c[d] + 1 >= ext[d]) continue;
                    long long u = x + stride[1] * y + stride[2] * z, v = u + stride[d], w = v + stride[d];
                    int ok = c[d] + 2 < ext[d];
                    double cap;
                    if (elem == 4) {
                        float Du = fabsf(Af[u] - Bf[u]), Dv = fabsf(Af[v] - Bf[v]);
                        float gAu = fabsf(Af[v] - Af[u]), gBu = fabsf(Bf[v] - Bf[u]);
                        float gAv = ok ? fabsf(Af[w] - Af[v]) : gAu;
                        float gBv = ok ? fabsf(Bf[w] - Bf[v]) : gBu;
                        float num = Du + Dv, den = gAu + gAv;
                        den = den + gBu; den = den + gBv;
                        cap = (double)num / ((double)den + EPS);
                    } else {
                        double Du = fabs(Ad[u] - Bd[u]), Dv = fabs(Ad[v] - Bd[v]);
                        double gAu = fabs(Ad[v] - Ad[u]), gBu = fabs(Bd[v] - Bd[u]);
                        double gAv = ok ? fabs(Ad[w] - Ad[v]) : gAu;
                        double gBv = ok ? fabs(Bd[w] - Bd[v]) : gBu;
                        double num = Du + Dv, den = gAu + gAv;
                        den = den + gBu; den = den + gBv;
                        cap = num / (den + EPS);
                    }
                    if (out) out[n] = cap;
                    n++;
                }
    }
    if (out) quantize_caps(out, n, 1);
    return n;
}
