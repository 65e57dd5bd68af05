/*
 * sph_oracle.c -- CPU oracle for the sphugo 2D SPH step (TEST INFRASTRUCTURE).
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 * Compile with -O2 -ffp-contract=off -fno-fast-math so that every a*b+c is two
 * roundings, as in the reference's Go code on amd64. Every function cites the
 * reference file:line it restates (paths within the bbeni/sphugo project).
 */
#include "sph_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Kernel prefactors, correctly rounded as Go folds the untyped constant
 * expressions of sim/sph.go:266,275,293,303 in exact arithmetic. */
static const double MONAHAN_PREF = 0x1.5d3b3e3583243p+3; /* 6*40/(pi*7) */
static const double WEND_FPREF = 0x1.1d34a60108f72p+1;   /* 4*7/(pi*4)  */
static const double WEND_DFPREF = 0x1.1d34a60108f72p+2;  /* 8*7/(pi*4)  */
#define MAX_PARTICLES_PER_CELL 8                        /* sim/core.go:11 */

/* One particle as in sim/core.go:17-42; the per-neighbour arrays are owned
 * by the particle so that Partition's swaps carry them along. */
typedef struct {
    double x, y, vx, vy, rho, c, e, edot, ax, ay, epred, vpx, vpy;
    double anorm, unorm;
    int64_t id;
    double *nnd;     /* NNDists: squared during the search, distances after */
    int32_t *nn;     /* NearestNeighbours as array positions, -1 = nil */
    double *nnx, *nny; /* NNPos */
    int32_t *nimg;   /* image code of each neighbour */
} P;

/* sim/core.go:46-60 Cell, children as indices into a node pool. */
typedef struct {
    int32_t lo, hi;            /* particle slice [lo, hi) */
    double llx, lly, urx, ury; /* LowerLeft, UpperRight */
    double bcx, bcy, br;       /* BCenter, BRadius */
    int32_t lower, upper;      /* -1 = nil */
} Node;

struct orc_sim {
    orc_params p;
    P *ps;
    double *blk_d;
    int32_t *blk_i;
    Node *nodes;
    int32_t nnodes, cap_nodes;
    int step;
    int check_tree;
    int64_t mismatches;
};

/* ------------------------------------------------------------------------ */
/* sim/linear-algebra.go:64-71 */
static inline double dist_sq(double ax, double ay, double bx, double by) {
    double dx = ax - bx, dy = ay - by;
    return dx * dx + dy * dy;
}

/* Go math.Hypot, pure-Go form: p*sqrt(1+(q/p)^2) with p >= q >= 0. */
double orc_hypot(double p, double q) {
    p = fabs(p);
    q = fabs(q);
    if (isinf(p) || isinf(q)) return INFINITY;
    if (isnan(p) || isnan(q)) return NAN;
    if (p < q) { double t = p; p = q; q = t; }
    if (p == 0) return 0;
    q = q / p;
    return p * sqrt(1 + q * q);
}

/* ------------------------------------------------------------------------ */
/* Kernels, sim/sph.go:258-304 */
double orc_kernel_f(int kernel, double q) {
    if (kernel == ORC_KERNEL_WENDLAND) {
        double a = 1 - q;
        return a * a * a * a * (1 + 4 * q);
    }
    if (q < 0.5) return q * q * q - q * q + 1.0 / 6;
    return (1 - q) * (1 - q) * (1 - q) / 3;
}
double orc_kernel_df(int kernel, double q) {
    if (kernel == ORC_KERNEL_WENDLAND) return -10 * q * (1 - q) * (1 - q) * (1 - q);
    if (q < 0.5) return (3 * q * q - 2 * q);
    return -(1 - q) * (1 - q);
}
double orc_kernel_fpref(int kernel) { return kernel == ORC_KERNEL_WENDLAND ? WEND_FPREF : MONAHAN_PREF; }
double orc_kernel_dfpref(int kernel) { return kernel == ORC_KERNEL_WENDLAND ? WEND_DFPREF : MONAHAN_PREF; }

/* ------------------------------------------------------------------------ */
/* sim/core.go:126-164 Partition. Vertical compares Y, Horizontal compares X;
 * the i==j fix-up sits inside the loop for Vertical and after it for
 * Horizontal, exactly as in the reference. Returns len(a). */
static inline void swap_p(P *a, P *b) { P t = *a; *a = *b; *b = t; }

static int partition_p(P *ps, int n, int orientation, double middle) {
    int i = 0, j = n - 1;
    if (orientation == 0) {
        while (i < j) {
            while (i < j && ps[i].y <= middle) i++;
            while (i < j && ps[j].y > middle) j--;
            if (ps[i].y > ps[j].y) swap_p(&ps[i], &ps[j]);
            if (i == j && middle > ps[i].y) i++;
        }
    } else {
        while (i < j) {
            while (i < j && ps[i].x <= middle) i++;
            while (i < j && ps[j].x > middle) j--;
            if (ps[i].x > ps[j].x) swap_p(&ps[i], &ps[j]);
        }
        if (i == j && middle > ps[i].x) i++;
    }
    return i;
}

int orc_partition(double *xs, double *ys, int n, int orientation, double middle) {
    P *ps = (P *)calloc(n > 0 ? (size_t)n : 1, sizeof(P));
    for (int i = 0; i < n; i++) { ps[i].x = xs[i]; ps[i].y = ys[i]; }
    int a = partition_p(ps, n, orientation, middle);
    for (int i = 0; i < n; i++) { xs[i] = ps[i].x; ys[i] = ps[i].y; }
    free(ps);
    return a;
}

/* ------------------------------------------------------------------------ */
static int32_t new_node(orc_sim *s, int32_t lo, int32_t hi, double llx, double lly,
                        double urx, double ury) {
    if (s->nnodes == s->cap_nodes) {
        s->cap_nodes = s->cap_nodes ? s->cap_nodes * 2 : 1024;
        s->nodes = (Node *)realloc(s->nodes, (size_t)s->cap_nodes * sizeof(Node));
    }
    Node *c = &s->nodes[s->nnodes];
    c->lo = lo; c->hi = hi;
    c->llx = llx; c->lly = lly; c->urx = urx; c->ury = ury;
    c->bcx = c->bcy = c->br = 0;
    c->lower = c->upper = -1;
    return s->nnodes++;
}

/* sim/core.go:172-224 Treebuild (SPLIT_FRACTION = 0.5). */
static void treebuild(orc_sim *s, int32_t ci, int orientation) {
    Node c = s->nodes[ci]; /* copy: the pool may move */
    if (c.lly == c.ury && c.llx == c.urx) return;
    double mid;
    if (orientation == 0) mid = 0.5 * c.lly + (1 - 0.5) * c.ury;
    else mid = 0.5 * c.llx + (1 - 0.5) * c.urx;
    int na = partition_p(s->ps + c.lo, c.hi - c.lo, orientation, mid);
    int nb = (c.hi - c.lo) - na;
    if (na > 0) {
        int32_t li = new_node(s, c.lo, c.lo + na, c.llx, c.lly, c.urx, c.ury);
        if (orientation == 0) s->nodes[li].ury = mid; else s->nodes[li].urx = mid;
        s->nodes[ci].lower = li;
        if (na > MAX_PARTICLES_PER_CELL) treebuild(s, li, 1 - orientation);
    }
    if (nb > 0) {
        int32_t ui = new_node(s, c.lo + na, c.hi, c.llx, c.lly, c.urx, c.ury);
        if (orientation == 0) s->nodes[ui].lly = mid; else s->nodes[ui].llx = mid;
        s->nodes[ci].upper = ui;
        if (nb > MAX_PARTICLES_PER_CELL) treebuild(s, ui, 1 - orientation);
    }
}

/* sim/core.go:229-312 BoundingSpheres. */
static void bounding_spheres(orc_sim *s, int32_t ci) {
    Node *c = &s->nodes[ci];
    if (c->upper < 0 && c->lower < 0) {
        P *ps = s->ps;
        if (c->hi - c->lo == 1) {
            c->bcx = ps[c->lo].x; c->bcy = ps[c->lo].y; c->br = 0;
        } else {
            double dmax = 0.0, pax = 0, pay = 0, pbx = 0, pby = 0;
            for (int a = c->lo; a < c->hi; a++)
                for (int b = c->lo; b < c->hi; b++) {
                    double xx = ps[b].x - ps[a].x, xy = ps[b].y - ps[a].y;
                    double dsq = xx * xx + xy * xy;
                    if (dsq > dmax) { dmax = dsq; pax = ps[a].x; pay = ps[a].y; pbx = ps[b].x; pby = ps[b].y; }
                }
            double rx = (pbx - pax) * 0.5, ry = (pby - pay) * 0.5;
            c->bcx = rx + pax; c->bcy = ry + pay;
            double brsq = rx * rx + ry * ry;
            for (int a = c->lo; a < c->hi; a++) {
                double xx = c->bcx - ps[a].x, xy = c->bcy - ps[a].y;
                double r = xx * xx + xy * xy;
                if (r > brsq) brsq = r;
            }
            c->br = sqrt(brsq);
        }
        return;
    }
    int32_t up = c->upper, lo = c->lower;
    if (up >= 0) bounding_spheres(s, up);
    if (lo >= 0) bounding_spheres(s, lo);
    c = &s->nodes[ci];
    if (up < 0) { c->br = s->nodes[lo].br; c->bcx = s->nodes[lo].bcx; c->bcy = s->nodes[lo].bcy; return; }
    if (lo < 0) { c->br = s->nodes[up].br; c->bcx = s->nodes[up].bcx; c->bcy = s->nodes[up].bcy; return; }
    Node *U = &s->nodes[up], *L = &s->nodes[lo];
    double abx = U->bcx - L->bcx, aby = U->bcy - L->bcy;
    double abn = sqrt(abx * abx + aby * aby);
    double ra = L->br, rb = U->br;
    double rc = (ra + rb + abn) * 0.5;
    double f = (rb - rc) / abn;
    double mx = abx * f, my = aby * f;
    c->bcx = mx + U->bcx; c->bcy = my + U->bcy;
    c->br = rc;
}

/* MakeCells (sim/core.go:93-105) over s->ps with root bounds [0,1]^2. */
static void make_cells(orc_sim *s) {
    s->nnodes = 0;
    new_node(s, 0, s->p.n, 0, 0, 1, 1);
    treebuild(s, 0, 0);
    bounding_spheres(s, 0);
}

/* ------------------------------------------------------------------------ */
/* sim/nearest-neighbour.go:139-153 NNQueueInsert. */
static inline void nn_insert(P *p, int k, double d, int32_t nb, double rx, double ry, int32_t img) {
    int i = 1;
    for (; i < k && p->nnd[i] > d; i++) {
        p->nnd[i - 1] = p->nnd[i];
        p->nn[i - 1] = p->nn[i];
        p->nnx[i - 1] = p->nnx[i];
        p->nny[i - 1] = p->nny[i];
        p->nimg[i - 1] = p->nimg[i];
    }
    p->nnd[i - 1] = d;
    p->nn[i - 1] = nb;
    p->nnx[i - 1] = rx;
    p->nny[i - 1] = ry;
    p->nimg[i - 1] = img;
}

/* sim/nearest-neighbour.go:70-119 findNNRec. */
static void find_nn_rec(const orc_sim *s, P *p, int32_t self, int32_t ci, double ox, double oy, int32_t img) {
    const Node *c = &s->nodes[ci];
    double px = p->x + ox, py = p->y + oy;
    if (c->upper < 0 && c->lower < 0) {
        for (int32_t j = c->lo; j < c->hi; j++) {
            const P *q = &s->ps[j];
            double d2 = dist_sq(px, py, q->x, q->y);
            if (d2 < p->nnd[0] && j != self)
                nn_insert(p, s->p.k, d2, j, q->x - ox, q->y - oy, img);
        }
        return;
    }
    if (c->upper >= 0 && c->lower >= 0) {
        const Node *U = &s->nodes[c->upper], *L = &s->nodes[c->lower];
        double du = orc_hypot(U->bcx - px, U->bcy - py);
        double dl = orc_hypot(L->bcx - px, L->bcy - py);
        double maxd = sqrt(p->nnd[0]);
        if (dl < du) {
            if (dl - L->br < maxd) find_nn_rec(s, p, self, c->lower, ox, oy, img);
            if (du - U->br < maxd) find_nn_rec(s, p, self, c->upper, ox, oy, img);
        } else {
            if (du - U->br < maxd) find_nn_rec(s, p, self, c->upper, ox, oy, img);
            if (dl - L->br < maxd) find_nn_rec(s, p, self, c->lower, ox, oy, img);
        }
        return;
    }
    if (c->upper >= 0) find_nn_rec(s, p, self, c->upper, ox, oy, img);
    if (c->lower >= 0) find_nn_rec(s, p, self, c->lower, ox, oy, img);
}

/* Image loop bounds of sim/nearest-neighbour.go:32-55. */
static int image_range(const double per[2], int *i0, int *i1, double *delta) {
    *i0 = -1; *i1 = 1;
    *delta = per[1] - per[0];
    if (per[0] == -DBL_MAX) {
        *i0 = 0; *i1 = 0; *delta = 0;
        if (per[1] != DBL_MAX) return ORC_ERR_OPEN_MIX;
    }
    return ORC_OK;
}

/* sim/nearest-neighbour.go:28-67 FindNearestNeighboursPeriodic + :155-165
 * NNQueueInitSentinel (the sentinel accumulates on the previous distances). */
static void knn_tree_one(const orc_sim *s, int32_t i) {
    P *p = &s->ps[i];
    int k = s->p.k;
    for (int a = 0; a < k; a++) { p->nnd[a] += 0.4; p->nn[a] = -1; p->nimg[a] = -1; }
    int i0, i1, j0, j1;
    double dX, dY;
    image_range(s->p.hor, &i0, &i1, &dX);
    image_range(s->p.vert, &j0, &j1, &dY);
    for (int a = i0; a <= i1; a++)
        for (int b = j0; b <= j1; b++)
            find_nn_rec(s, p, i, 0, (double)a * dX, (double)b * dY, (a + 1) * 3 + (b + 1));
    for (int a = 0; a < k; a++) p->nnd[a] = sqrt(p->nnd[a]);
}

/* ------------------------------------------------------------------------ */
/* Exact kNN: uniform grid, ring search with a rigorous stop rule, ties broken
 * by (squared distance, particle id, image code). Distances use the
 * reference's rounding: ((p + o) - q)^2 summed as dx*dx + dy*dy. */
typedef struct { double d2; int64_t id; int32_t img; int32_t j; } Cand;

static inline int cand_less(const Cand *a, const Cand *b) {
    if (a->d2 != b->d2) return a->d2 < b->d2;
    if (a->id != b->id) return a->id < b->id;
    return a->img < b->img;
}
/* bounded max-heap of the k best */
static inline void heap_push(Cand *h, int *cnt, int k, Cand c) {
    if (*cnt < k) {
        int i = (*cnt)++;
        h[i] = c;
        while (i > 0) {
            int pa = (i - 1) / 2;
            if (cand_less(&h[pa], &h[i])) { Cand t = h[pa]; h[pa] = h[i]; h[i] = t; i = pa; } else break;
        }
        return;
    }
    if (!cand_less(&c, &h[0])) return;
    h[0] = c;
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, r = l + 1, m = i;
        if (l < k && cand_less(&h[m], &h[l])) m = l;
        if (r < k && cand_less(&h[m], &h[r])) m = r;
        if (m == i) break;
        Cand t = h[m]; h[m] = h[i]; h[i] = t; i = m;
    }
}
static int cand_cmp(const void *a, const void *b) {
    const Cand *x = (const Cand *)a, *y = (const Cand *)b;
    if (cand_less(x, y)) return -1;
    if (cand_less(y, x)) return 1;
    return 0;
}

typedef struct {
    int G[2];
    double lo[2], s[2], inv_s[2], L[2], delta[2];
    int periodic[2];
    int32_t *start, *order;
} Grid;

static void grid_axis(Grid *g, int ax, const double per[2], const double *v, const P *ps, int n, int gdim) {
    if (per[0] == -DBL_MAX) {
        double mn = DBL_MAX, mx = -DBL_MAX;
        for (int i = 0; i < n; i++) {
            double t = ps ? (ax ? ps[i].y : ps[i].x) : v[i];
            if (t < mn) mn = t;
            if (t > mx) mx = t;
        }
        double w = mx - mn;
        if (!(w > 0)) w = 1;
        g->periodic[ax] = 0;
        g->lo[ax] = mn;
        g->L[ax] = w * (1 + 1e-9);
        g->delta[ax] = 0;
    } else {
        g->periodic[ax] = 1;
        g->lo[ax] = per[0];
        g->L[ax] = per[1] - per[0];
        double d = 0;
        for (int i = 0; i < n; i++) {
            double t = ps ? (ax ? ps[i].y : ps[i].x) : v[i];
            double o = fmax(per[0] - t, t - per[1]);
            if (o > d) d = o;
        }
        g->delta[ax] = d;
    }
    g->G[ax] = gdim;
    g->s[ax] = g->L[ax] / gdim;
    g->inv_s[ax] = gdim / g->L[ax];
}

static inline int cell_of(const Grid *g, int ax, double v) {
    double t = floor((v - g->lo[ax]) * g->inv_s[ax]);
    if (!(t >= 0)) return 0;
    if (t > g->G[ax] - 1) return g->G[ax] - 1;
    return (int)t;
}

static void grid_build_dim(Grid *g, const orc_params *p, const double *x, const double *y, const P *ps, int n,
                           int gd) {
    grid_axis(g, 0, p->hor, x, ps, n, gd);
    grid_axis(g, 1, p->vert, y, ps, n, gd);
    size_t nc = (size_t)g->G[0] * g->G[1];
    g->start = (int32_t *)calloc(nc + 1, sizeof(int32_t));
    g->order = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    int32_t *cell = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    for (int i = 0; i < n; i++) {
        double xi = ps ? ps[i].x : x[i], yi = ps ? ps[i].y : y[i];
        cell[i] = cell_of(g, 1, yi) * g->G[0] + cell_of(g, 0, xi);
        g->start[cell[i] + 1]++;
    }
    for (size_t c = 0; c < nc; c++) g->start[c + 1] += g->start[c];
    int32_t *fill = (int32_t *)malloc((nc + 1) * sizeof(int32_t));
    memcpy(fill, g->start, (nc + 1) * sizeof(int32_t));
    for (int i = 0; i < n; i++) g->order[fill[cell[i]]++] = i;
    free(fill);
    free(cell);
}

static void grid_free(Grid *g) { free(g->start); free(g->order); }

/* Uniform grids of every power-of-two resolution from 1 cell per axis up to
 * the first at or above 4 sqrt(n) (at most 4096) over the same points. A
 * query searches the finest grid whose cell around it holds at least k/4
 * points (the coarsest otherwise), so dense and sparse regions both see cells
 * of a few k points: one uniform grid sized by the mean density degenerates
 * on strongly clustered data (thousands of points per cell in a dense patch).
 * The exact result does not depend on the grid: the ring search's stop rule
 * holds for any cell size. */
#define PYR_LEVELS 13
typedef struct {
    int nl;
    Grid g[PYR_LEVELS]; /* g[0] finest */
} Pyramid;

static void pyramid_build(Pyramid *py, const orc_params *p, const double *x, const double *y, const P *ps, int n) {
    int top = 1;
    while (top < 4096 && (double)top < 4.0 * sqrt((double)n)) top <<= 1;
    py->nl = 0;
    for (int gd = top; gd >= 1 && py->nl < PYR_LEVELS; gd >>= 1) grid_build_dim(&py->g[py->nl++], p, x, y, ps, n, gd);
}

static void pyramid_free(Pyramid *py) {
    for (int l = 0; l < py->nl; l++) grid_free(&py->g[l]);
}

static const Grid *pyramid_pick(const Pyramid *py, double px, double py_, int k) {
    const int want = k / 4 > 0 ? k / 4 : 1;
    for (int l = 0; l < py->nl; l++) {
        const Grid *g = &py->g[l];
        const int c = cell_of(g, 1, py_) * g->G[0] + cell_of(g, 0, px);
        if (g->start[c + 1] - g->start[c] >= want) return g;
    }
    return &py->g[py->nl - 1];
}

/* Searches the k best candidates of query i; fills h[0..k) ascending.
 * Returns the number found (< k only if fewer candidates exist). */
static int knn_exact_query(const Grid *g, const orc_params *p, const double *x, const double *y,
                           const int64_t *ids, int n, int i, Cand *h) {
    int k = p->k, cnt = 0;
    double px = x[i], py = y[i];
    int cx = cell_of(g, 0, px), cy = cell_of(g, 1, py);
    double ex = fmin(px - (g->lo[0] + cx * g->s[0]), (g->lo[0] + (cx + 1) * g->s[0]) - px);
    double ey = fmin(py - (g->lo[1] + cy * g->s[1]), (g->lo[1] + (cy + 1) * g->s[1]) - py);
    double dmx = g->delta[0] > g->delta[1] ? g->delta[0] : g->delta[1];
    int rmax = 2 * (g->G[0] > g->G[1] ? g->G[0] : g->G[1]) + 2;
    for (int R = 0; R <= rmax; R++) {
        for (int b = -R; b <= R; b++) {
            for (int a = -R; a <= R; a++) {
                if (abs(a) != R && abs(b) != R) continue;
                int gx = cx + a, gy = cy + b;
                int wx = (int)floor((double)gx / g->G[0]), wy = (int)floor((double)gy / g->G[1]);
                if (g->periodic[0]) { if (wx < -1 || wx > 1) continue; } else if (wx != 0) continue;
                if (g->periodic[1]) { if (wy < -1 || wy > 1) continue; } else if (wy != 0) continue;
                int ia = -wx, ib = -wy; /* image multiples: o = (ia*dX, ib*dY) */
                double ox = g->periodic[0] ? (double)ia * g->L[0] : 0.0;
                double oy = g->periodic[1] ? (double)ib * g->L[1] : 0.0;
                int32_t img = (ia + 1) * 3 + (ib + 1);
                int c = (gy - wy * g->G[1]) * g->G[0] + (gx - wx * g->G[0]);
                double sx = px + ox, sy = py + oy;
                for (int t = g->start[c]; t < g->start[c + 1]; t++) {
                    int j = g->order[t];
                    if (j == i) continue;
                    Cand cd;
                    cd.d2 = dist_sq(sx, sy, x[j], y[j]);
                    cd.id = ids ? ids[j] : j;
                    cd.img = img;
                    cd.j = j;
                    heap_push(h, &cnt, k, cd);
                }
            }
        }
        if (cnt == k) {
            double bx = R * g->s[0] + ex - dmx, by = R * g->s[1] + ey - dmx;
            double bnd = bx < by ? bx : by;
            if (bnd > 0 && h[0].d2 < bnd * bnd * (1 - 1e-9)) break;
        }
    }
    qsort(h, cnt, sizeof(Cand), cand_cmp);
    return cnt;
}

static int knn_brute_query(const orc_params *p, const double *x, const double *y, const int64_t *ids,
                           int n, int i, Cand *h) {
    int i0, i1, j0, j1, cnt = 0;
    double dX, dY;
    image_range(p->hor, &i0, &i1, &dX);
    image_range(p->vert, &j0, &j1, &dY);
    for (int a = i0; a <= i1; a++)
        for (int b = j0; b <= j1; b++) {
            double sx = x[i] + (double)a * dX, sy = y[i] + (double)b * dY;
            for (int j = 0; j < n; j++) {
                if (j == i) continue;
                Cand cd;
                cd.d2 = dist_sq(sx, sy, x[j], y[j]);
                cd.id = ids ? ids[j] : j;
                cd.img = (a + 1) * 3 + (b + 1);
                cd.j = j;
                heap_push(h, &cnt, p->k, cd);
            }
        }
    qsort(h, cnt, sizeof(Cand), cand_cmp);
    return cnt;
}

static void set_threads(const orc_params *p) {
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#else
    (void)p;
#endif
}

static int knn_standalone(const orc_params *p, const double *x, const double *y,
                          int64_t *ids, double *d2, int32_t *img, int brute) {
    int n = p->n, k = p->k, rc = ORC_OK;
    int i0, i1;
    double d;
    if (image_range(p->hor, &i0, &i1, &d) || image_range(p->vert, &i0, &i1, &d)) return ORC_ERR_OPEN_MIX;
    if (k <= 0 || n <= k) return ORC_ERR_ARG;
    Pyramid py;
    memset(&py, 0, sizeof py);
    if (!brute) pyramid_build(&py, p, x, y, NULL, n);
    set_threads(p);
#pragma omp parallel
    {
        Cand *h = (Cand *)malloc((size_t)k * sizeof(Cand));
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < n; i++) {
            int cnt = brute ? knn_brute_query(p, x, y, NULL, n, i, h)
                            : knn_exact_query(pyramid_pick(&py, x[i], y[i], k), p, x, y, NULL, n, i, h);
            for (int a = 0; a < k; a++) {
                ids[(size_t)i * k + a] = a < cnt ? h[a].id : -1;
                if (d2) d2[(size_t)i * k + a] = a < cnt ? h[a].d2 : INFINITY;
                if (img) img[(size_t)i * k + a] = a < cnt ? h[a].img : -1;
            }
        }
        free(h);
    }
    if (!brute) pyramid_free(&py);
    return rc;
}

int orc_knn_exact(const orc_params *p, const double *x, const double *y, int64_t *ids, double *d2, int32_t *img) {
    return knn_standalone(p, x, y, ids, d2, img, 0);
}
int orc_knn_brute(const orc_params *p, const double *x, const double *y, int64_t *ids, double *d2, int32_t *img) {
    return knn_standalone(p, x, y, ids, d2, img, 1);
}

/* ------------------------------------------------------------------------ */
orc_sim *orc_create(const orc_params *p, const double *x, const double *y,
                    const double *vx, const double *vy, const double *u) {
    if (!p || p->n <= 0 || p->k <= 0) return NULL;
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    s->p = *p;
    int n = p->n, k = p->k;
    s->ps = (P *)calloc((size_t)n, sizeof(P));
    s->blk_d = (double *)calloc((size_t)n * k * 3, sizeof(double));
    s->blk_i = (int32_t *)calloc((size_t)n * k * 2, sizeof(int32_t));
    for (int i = 0; i < n; i++) {
        P *q = &s->ps[i];
        q->x = x[i]; q->y = y[i];
        q->vx = vx ? vx[i] : 0; q->vy = vy ? vy[i] : 0;
        q->e = u ? u[i] : 0;
        /* a fresh state counts as predicted with dt = 0, as Step 0 sets it
         * (sim/sph.go:96-100) before its first evaluation */
        q->vpx = q->vx; q->vpy = q->vy; q->epred = q->e;
        q->id = i;
        q->nnd = s->blk_d + (size_t)i * k * 3;
        q->nnx = q->nnd + k;
        q->nny = q->nnd + 2 * k;
        q->nn = s->blk_i + (size_t)i * k * 2;
        q->nimg = q->nn + k;
        for (int a = 0; a < k; a++) q->nn[a] = -1;
    }
    return s;
}

void orc_destroy(orc_sim *s) {
    if (!s) return;
    free(s->ps); free(s->blk_d); free(s->blk_i); free(s->nodes);
    free(s);
}

int orc_set_knn_mode(orc_sim *s, int mode) { s->p.knn_mode = mode; return ORC_OK; }
void orc_set_check_tree(orc_sim *s, int on) { s->check_tree = on; }
int64_t orc_tree_exact_mismatches(const orc_sim *s) { return s->mismatches; }
int orc_current_step(const orc_sim *s) { return s->step; }

/* Exact kNN into the particles' queues (same layout as the tree search). */
static int knn_exact_fill(orc_sim *s) {
    int n = s->p.n, k = s->p.k;
    double *x = (double *)malloc((size_t)n * sizeof(double));
    double *y = (double *)malloc((size_t)n * sizeof(double));
    int64_t *ids = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    for (int i = 0; i < n; i++) { x[i] = s->ps[i].x; y[i] = s->ps[i].y; ids[i] = s->ps[i].id; }
    Pyramid py;
    pyramid_build(&py, &s->p, x, y, NULL, n);
    int bad = 0;
#pragma omp parallel reduction(+ : bad)
    {
        Cand *h = (Cand *)malloc((size_t)k * sizeof(Cand));
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < n; i++) {
            P *p = &s->ps[i];
            int cnt = knn_exact_query(pyramid_pick(&py, x[i], y[i], k), &s->p, x, y, ids, n, i, h);
            if (cnt < k) { bad++; continue; }
            for (int a = 0; a < k; a++) {
                const Cand *c = &h[k - 1 - a]; /* slot 0 = farthest */
                int ia = c->img / 3 - 1, ib = c->img % 3 - 1;
                double ox = ia ? (double)ia * (s->p.hor[1] - s->p.hor[0]) : 0.0;
                double oy = ib ? (double)ib * (s->p.vert[1] - s->p.vert[0]) : 0.0;
                p->nnd[a] = c->d2;
                p->nn[a] = c->j;
                p->nnx[a] = s->ps[c->j].x - ox;
                p->nny[a] = s->ps[c->j].y - oy;
                p->nimg[a] = c->img;
            }
            /* the reference's queue only ever holds values below the 0.4 sentinel */
            if (!(h[k - 1].d2 < 0.4)) bad++;
            for (int a = 0; a < k; a++) p->nnd[a] = sqrt(p->nnd[a]);
        }
        free(h);
    }
    pyramid_free(&py);
    free(x); free(y); free(ids);
    return bad ? ORC_ERR_SENTINEL : ORC_OK;
}

/* sim/sph.go:306-323 Density2D */
static int density(P *p, const orc_params *pr) {
    double maxr = p->nnd[0], acc = 0.0;
    for (int i = 0; i < pr->k; i++) {
        double x = p->nnd[i] / maxr;
        if (x > 1 || x < 0) return ORC_ERR_Q_RANGE;
        acc += orc_kernel_f(pr->kernel, x);
    }
    p->rho = orc_kernel_fpref(pr->kernel) * pr->mass * acc / (maxr * maxr);
    return ORC_OK;
}

/* sim/sph.go:327-401 AccelerationAndEDot2D (alpha, beta, etaSq as params). */
static int accel_edot(P *p, const P *ps, const orc_params *pr) {
    double gamma = pr->gamma, maxr = p->nnd[0];
    double ca = p->c * p->c / (gamma * p->rho);
    double ax = 0.0, ay = 0.0, ed = 0.0, an = 0.0, un = 0.0;
    for (int i = 0; i < pr->k; i++) {
        if (p->nn[i] < 0) break;
        const P *nn = &ps[p->nn[i]];
        double q = p->nnd[i] / maxr;
        if (q > 1 || q < 0) return ORC_ERR_Q_RANGE;
        double drk = orc_kernel_df(pr->kernel, q);
        double cb = nn->c * nn->c / (gamma * nn->rho);
        double vabx = nn->vpx - p->vpx, vaby = nn->vpy - p->vpy;
        double rabx = p->nnx[i] - p->x, raby = p->nny[i] - p->y;
        double dot = vabx * rabx + vaby * raby;
        double piab = 0.0;
        if (dot < 0) {
            double cab = 0.5 * (p->c + nn->c);
            double rhoab = 0.5 * (p->rho + nn->rho);
            double hab = 0.5 * (p->nnd[0] + nn->nnd[0]);
            double mu = dot * hab / ((rabx * rabx + raby * raby) + pr->etasq);
            piab = (-pr->alpha * cab * mu + pr->beta * mu * mu) / rhoab;
        }
        ax += rabx * (piab + ca + cb) * drk / p->nnd[i];
        ay += raby * (piab + ca + cb) * drk / p->nnd[i];
        ed += dot * drk;
        an += sqrt(rabx * rabx + raby * raby) * fabs((piab + ca + cb) * drk / p->nnd[i]);
        un += fabs(dot * drk);
    }
    double f = pr->mass * orc_kernel_dfpref(pr->kernel) / (maxr * maxr * maxr);
    p->ax = ax * f + pr->accel[0];
    p->ay = ay * f + pr->accel[1];
    p->edot = ca * ed * pr->mass;
    p->anorm = an * fabs(f);
    p->unorm = un * fabs(ca * pr->mass);
    return ORC_OK;
}

static int same_set(const P *p, const P *ps, const int64_t *ids_exact, int k) {
    /* compare as multisets of (id, img) */
    for (int a = 0; a < k; a++) {
        int64_t id = ps[p->nn[a]].id;
        int found = 0;
        for (int b = 0; b < k; b++)
            if (ids_exact[2 * b] == id && ids_exact[2 * b + 1] == p->nimg[a]) { found = 1; break; }
        if (!found) return 0;
    }
    return 1;
}

/* sim/sph.go:403-435 CalculateForces */
static int calc_forces(orc_sim *s) {
    int n = s->p.n, k = s->p.k, rc = ORC_OK;
    int i0, i1;
    double d;
    if (image_range(s->p.hor, &i0, &i1, &d) || image_range(s->p.vert, &i0, &i1, &d)) return ORC_ERR_OPEN_MIX;
    set_threads(&s->p);
    if (s->p.knn_mode == ORC_KNN_TREE) {
        make_cells(s); /* Treebuild(Vertical) + BoundingSpheres on [0,1]^2 */
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : bad)
        for (int i = 0; i < n; i++) {
            knn_tree_one(s, i);
            for (int a = 0; a < k; a++) if (s->ps[i].nn[a] < 0) { bad++; break; }
        }
        if (bad) return ORC_ERR_SENTINEL;
        if (s->check_tree) {
            double *x = (double *)malloc((size_t)n * sizeof(double));
            double *y = (double *)malloc((size_t)n * sizeof(double));
            int64_t *ids = (int64_t *)malloc((size_t)n * sizeof(int64_t));
            for (int i = 0; i < n; i++) { x[i] = s->ps[i].x; y[i] = s->ps[i].y; ids[i] = s->ps[i].id; }
            Pyramid py;
            pyramid_build(&py, &s->p, x, y, NULL, n);
            int64_t mm = 0;
#pragma omp parallel reduction(+ : mm)
            {
                Cand *h = (Cand *)malloc((size_t)k * sizeof(Cand));
                int64_t *pairs = (int64_t *)malloc((size_t)k * 2 * sizeof(int64_t));
#pragma omp for schedule(dynamic, 64)
                for (int i = 0; i < n; i++) {
                    knn_exact_query(pyramid_pick(&py, x[i], y[i], k), &s->p, x, y, ids, n, i, h);
                    for (int a = 0; a < k; a++) { pairs[2 * a] = h[a].id; pairs[2 * a + 1] = h[a].img; }
                    if (!same_set(&s->ps[i], s->ps, pairs, k)) mm++;
                }
                free(h); free(pairs);
            }
            pyramid_free(&py);
            free(x); free(y); free(ids);
            s->mismatches = mm;
        }
    } else {
        rc = knn_exact_fill(s);
        if (rc) return rc;
    }
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int i = 0; i < n; i++) if (density(&s->ps[i], &s->p)) bad++;
    if (bad) return ORC_ERR_Q_RANGE;
    double factor = s->p.gamma * (s->p.gamma - 1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) s->ps[i].c = sqrt(factor * s->ps[i].epred);
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int i = 0; i < n; i++) if (accel_edot(&s->ps[i], s->ps, &s->p)) bad++;
    return bad ? ORC_ERR_Q_RANGE : ORC_OK;
}

int orc_forces(orc_sim *s) { return calc_forces(s); }

/* sim/sph.go:64-198 Step (sources are not part of this oracle). */
int orc_step(orc_sim *s, int nsteps) {
    int n = s->p.n, rc;
    double dth = s->p.dth;
    const orc_params *pr = &s->p;
    for (int st = 0; st < nsteps; st++) {
        if (s->step == 0) {
            for (int i = 0; i < n; i++) { P *p = &s->ps[i]; p->vpx = p->vx; p->vpy = p->vy; p->epred = p->e; }
            if ((rc = calc_forces(s))) return rc;
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) {
            P *p = &s->ps[i];
            double vdx = p->vx * dth, vdy = p->vy * dth;
            p->x = p->x + vdx; p->y = p->y + vdy;
            double adx = p->ax * dth, ady = p->ay * dth;
            p->vpx = p->vx + adx; p->vpy = p->vy + ady;
            p->epred = p->e + p->edot * dth;
        }
        if ((rc = calc_forces(s))) return rc;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) {
            P *p = &s->ps[i];
            double adx = p->ax * (2 * dth), ady = p->ay * (2 * dth);
            p->vx = p->vx + adx; p->vy = p->vy + ady;
            p->e = p->e + p->edot * 2 * dth;
            double vdx = p->vx * dth, vdy = p->vy * dth;
            p->x = p->x + vdx; p->y = p->y + vdy;
            /* periodic wrap: an if/continue chain, one axis at most */
            if (p->x < pr->hor[0]) { p->x += (pr->hor[1] - pr->hor[0]); }
            else if (p->x > pr->hor[1]) { p->x -= (pr->hor[1] - pr->hor[0]); }
            else if (p->y < pr->vert[0]) { p->y += (pr->vert[1] - pr->vert[0]); }
            else if (p->y > pr->vert[1]) { p->y -= (pr->vert[1] - pr->vert[0]); }
            /* reflections, sim/sph.go:170-193 */
            if (p->x < pr->refl[0]) { p->x -= p->x - pr->refl[0]; p->vx = -p->vx; }
            if (p->x > pr->refl[1]) { p->x -= p->x - pr->refl[1]; p->vx = -p->vx; }
            if (p->y < pr->refl[2]) { p->y -= p->y - pr->refl[2]; p->vy = -p->vy; }
            if (p->y > pr->refl[3]) { p->y -= p->y - pr->refl[3]; p->vy = -p->vy; }
        }
        s->step++;
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
void orc_get_state(const orc_sim *s, double *x, double *y, double *vx, double *vy,
                   double *u, double *ax, double *ay, double *udot,
                   double *rho, double *c, double *h) {
    for (int i = 0; i < s->p.n; i++) {
        const P *p = &s->ps[i];
        int64_t id = p->id;
        if (x) x[id] = p->x;
        if (y) y[id] = p->y;
        if (vx) vx[id] = p->vx;
        if (vy) vy[id] = p->vy;
        if (u) u[id] = p->e;
        if (ax) ax[id] = p->ax;
        if (ay) ay[id] = p->ay;
        if (udot) udot[id] = p->edot;
        if (rho) rho[id] = p->rho;
        if (c) c[id] = p->c;
        if (h) h[id] = p->nnd[0];
    }
}

void orc_get_pred(const orc_sim *s, double *vpx, double *vpy, double *upred) {
    for (int i = 0; i < s->p.n; i++) {
        const P *p = &s->ps[i];
        if (vpx) vpx[p->id] = p->vpx;
        if (vpy) vpy[p->id] = p->vpy;
        if (upred) upred[p->id] = p->epred;
    }
}

void orc_get_neighbours(const orc_sim *s, int64_t *ids, double *dist, int32_t *img) {
    int k = s->p.k;
    for (int i = 0; i < s->p.n; i++) {
        const P *p = &s->ps[i];
        size_t base = (size_t)p->id * k;
        for (int a = 0; a < k; a++) {
            if (ids) ids[base + a] = p->nn[a] >= 0 ? s->ps[p->nn[a]].id : -1;
            if (dist) dist[base + a] = p->nnd[a];
            if (img) img[base + a] = p->nimg[a];
        }
    }
}

void orc_get_norms(const orc_sim *s, double *anorm, double *unorm) {
    for (int i = 0; i < s->p.n; i++) {
        const P *p = &s->ps[i];
        if (anorm) anorm[p->id] = p->anorm;
        if (unorm) unorm[p->id] = p->unorm;
    }
}

/* sim/sph.go:441-463 */
void orc_diagnostics(const orc_sim *s, double out[3]) {
    double e = 0.0, r = 0.0, m = 0.0;
    for (int i = 0; i < s->p.n; i++) {
        const P *p = &s->ps[i];
        e += p->e;
        r += p->rho;
        m = sqrt(p->vx * p->vx + p->vy * p->vy);
    }
    out[0] = e; out[1] = r; out[2] = m;
}

/* sim/bounding-sphere_test.go:7-24 isInsideAny over the whole tree. */
static int inside_any(const orc_sim *s, int32_t ci, double x, double y) {
    const Node *c = &s->nodes[ci];
    double dx = x - c->bcx, dy = y - c->bcy;
    if (sqrt(dx * dx + dy * dy) <= c->br) return 1;
    if (c->upper >= 0 && inside_any(s, c->upper, x, y)) return 1;
    if (c->lower >= 0 && inside_any(s, c->lower, x, y)) return 1;
    return 0;
}

int orc_tree_count_outside(const double *x, const double *y, int n) {
    if (n <= 0) return 0;
    orc_params p;
    memset(&p, 0, sizeof p);
    p.n = n; p.k = 1;
    orc_sim *s = orc_create(&p, x, y, NULL, NULL, NULL);
    make_cells(s);
    int out = 0;
    for (int i = 0; i < n; i++) if (!inside_any(s, 0, s->ps[i].x, s->ps[i].y)) out++;
    orc_destroy(s);
    return out;
}

/* ------------------------------------------------------------------------ */
/* Particles spawned during a run (sim/sph.go:71-85: Spawn then append to
 * Root.Particles). Go zero values for everything the spawner does not set. */
int orc_append(orc_sim *s, int n_new, const double *x, const double *y, const double *vx,
               const double *vy, const double *u) {
    if (!s || n_new < 0) return ORC_ERR_ARG;
    if (n_new == 0) return ORC_OK;
    const int n0 = s->p.n, n1 = n0 + n_new, k = s->p.k;
    double *bd = (double *)calloc((size_t)n1 * k * 3, sizeof(double));
    int32_t *bi = (int32_t *)calloc((size_t)n1 * k * 2, sizeof(int32_t));
    P *ps = (P *)calloc((size_t)n1, sizeof(P));
    memcpy(ps, s->ps, (size_t)n0 * sizeof(P));
    memcpy(bd, s->blk_d, (size_t)n0 * k * 3 * sizeof(double));
    memcpy(bi, s->blk_i, (size_t)n0 * k * 2 * sizeof(int32_t));
    for (int i = 0; i < n0; i++) {  /* blocks keep their offsets */
        P *q = &ps[i];
        q->nnd = bd + (q->nnd - s->blk_d);
        q->nnx = bd + (q->nnx - s->blk_d);
        q->nny = bd + (q->nny - s->blk_d);
        q->nn = bi + (q->nn - s->blk_i);
        q->nimg = bi + (q->nimg - s->blk_i);
    }
    for (int i = n0; i < n1; i++) {
        P *q = &ps[i];
        const int a = i - n0;
        q->x = x[a]; q->y = y[a];
        q->vx = vx ? vx[a] : 0; q->vy = vy ? vy[a] : 0;
        q->e = u ? u[a] : 0;
        q->id = i;
        q->nnd = bd + (size_t)i * k * 3;
        q->nnx = q->nnd + k;
        q->nny = q->nnd + 2 * k;
        q->nn = bi + (size_t)i * k * 2;
        q->nimg = q->nn + k;
        for (int b = 0; b < k; b++) q->nn[b] = -1;
    }
    free(s->ps); free(s->blk_d); free(s->blk_i);
    s->ps = ps; s->blk_d = bd; s->blk_i = bi;
    s->p.n = n1;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* sim/heap.go:229-268 QuickSort / partitionQS on particle indices with the
 * comparison value -Z (sim/animator.go:65-70). */
static void quicksort_negz(int64_t *ps, int64_t len, const int64_t *z) {
    while (len > 0) {
        int64_t i = 0, j = len - 2;
        const int64_t pivot = -z[ps[len - 1]];
        while (i < j) {
            while (i < j && -z[ps[i]] <= pivot) i++;
            while (i < j && -z[ps[j]] > pivot) j--;
            if (-z[ps[i]] > -z[ps[j]]) { int64_t t = ps[i]; ps[i] = ps[j]; ps[j] = t; }
        }
        if (-z[ps[i]] > pivot) { int64_t t = ps[i]; ps[i] = ps[len - 1]; ps[len - 1] = t; }
        else i = len - 1;
        quicksort_negz(ps, i, z);          /* left: ps[:i] */
        ps += i + 1;                        /* right: ps[i+1:] */
        len -= i + 1;
    }
}

void orc_draw_order(int64_t n, const int64_t *z, int64_t *order) {
    for (int64_t i = 0; i < n; i++) order[i] = i;
    quicksort_negz(order, n, z);
}

/* gx/graphics.go:156-164 ParaRamp */
static void para_ramp(int index, uint8_t *rgb) {
    const double x = (double)index;
    const double r = fmin(215, fmax(0, -fabs((x - 60) * 31 / 17 - 232) + 245));
    const double g = fmin(190, fmax(0, -fabs(x * 31 / 17 - 232) + 245));
    const double b = fmin(215, fmax(0, -fabs((x + 70) * 31 / 17 - 232) + 245));
    rgb[0] = (uint8_t)r; rgb[1] = (uint8_t)g; rgb[2] = (uint8_t)b;
}

void orc_para_ramp(int index, uint8_t *rgb) { para_ramp(index, rgb); }

/* sim/animator.go:55-103 CurrentFrame: black canvas, then for each particle in
 * `order` a disk of radius 4 (gx/graphics.go:90-107 DrawDisk, float32 pixel
 * test) coloured by ParaRamp(uint8(min(rho/(m*N*10)*256, 255))). x, y, rho in
 * caller order. */
void orc_render(int64_t n, const double *x, const double *y, const double *rho, double mass,
                const int64_t *order, int W, int H, uint8_t *rgba) {
    for (int64_t p = 0; p < (int64_t)W * H; p++) {
        rgba[4 * p] = 0; rgba[4 * p + 1] = 0; rgba[4 * p + 2] = 0; rgba[4 * p + 3] = 255;
    }
    const double n10 = (double)(n * 10);
    for (int64_t o = 0; o < n; o++) {
        const int64_t i = order[o];
        const float cx = (float)x[i] * (float)W;
        const float cy = (float)y[i] * (float)H;
        const double cf = rho[i] / (mass * n10) * 256;
        const double mn = cf > 255 ? 255 : cf;  /* math.Min keeps a NaN; uint8(NaN) = 0 */
        const int idx = mn >= 0 ? (int)mn : 0;
        uint8_t rgb[3];
        para_ramp(idx, rgb);
        const float radius = 4;
        const double xa = floor((double)(cx - radius)), xb = ceil((double)(cx + radius));
        const double ya = floor((double)(cy - radius)), yb = ceil((double)(cy + radius));
        for (double fx = xa; fx <= xb; fx++) {
            for (double fy = ya; fy <= yb; fy++) {
                const int px = (int)fx, py = (int)fy;
                const float dx = (float)px - cx, dy = (float)py - cy;
                const float r2 = dx * dx + dy * dy;
                if (r2 <= radius * radius && px >= 0 && px < W && py >= 0 && py < H) {
                    uint8_t *d = rgba + 4 * ((int64_t)py * W + px);
                    d[0] = rgb[0]; d[1] = rgb[1]; d[2] = rgb[2]; d[3] = 255;
                }
            }
        }
    }
}
