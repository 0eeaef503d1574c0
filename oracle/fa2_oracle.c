/*
 * fa2_oracle.c -- ORACLE, test infrastructure only (see fa2_oracle.h).
 *
 * Part 1: the CPU engine of src/forceatlas2.c, restated in double. Each
 * function cites the reference lines whose arithmetic it repeats; the order
 * of every floating-point operation is kept, so that the results are the
 * reference's bit for bit when both are compiled without FMA contraction
 * (-ffp-contract=off, which the Makefile passes on every host).
 *
 * Part 2 (pipe_impl.h, included twice below) restates inst/opencl/pipeline.cl.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fa2_oracle.h"

#define ORC_LEAF 8 /* FA2_LEAF_SIZE, src/forceatlas2.c:40 */

/* ------------------------------------------------------------------------ */
/* Part 1                                                                   */
/* ------------------------------------------------------------------------ */

void orc_mass(int n, int m, const int *from, const int *to, double *mass,
              double *mean_mass)
{
    /* src/forceatlas2.c:592-603 */
    double mean = 0.0;
    for (int i = 0; i < n; i++) mass[i] = 1.0;
    for (int e = 0; e < m; e++) {
        mass[from[e]] += 1.0;
        mass[to[e]] += 1.0;
    }
    for (int i = 0; i < n; i++) mean += mass[i];
    if (mean_mass) *mean_mass = n > 0 ? mean / n : 0.0;
}

/* src/forceatlas2.c:265-275: force on the first node = (xd, yd) * factor. */
static inline double rep_factor(int adjust, double scaling, double d2,
                                double mm, double ss)
{
    if (adjust) {
        const double d = sqrt(d2) - ss;
        if (d > 0) return scaling * mm / (d * d);
        if (d < 0) return 100.0 * scaling * mm;
        return 0.0;
    }
    return d2 > 0 ? scaling * mm / d2 : 0.0;
}

void orc_repulse_exact(int n, const double *x, const double *y,
                       const double *mass, const double *size, int adjust,
                       double scaling, int threads, double *dx, double *dy)
{
    /* src/forceatlas2.c:278-294: j ascending, self skipped. */
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
    for (int i = 0; i < n; i++) {
        const double xi = x[i], yi = y[i], mi = mass[i];
        const double si = adjust ? size[i] : 0.0;
        double fx = 0.0, fy = 0.0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            const double xd = xi - x[j], yd = yi - y[j];
            const double f = rep_factor(adjust, scaling, xd * xd + yd * yd,
                                        mi * mass[j],
                                        adjust ? si + size[j] : 0.0);
            fx += xd * f;
            fy += yd * f;
        }
        dx[i] += fx;
        dy[i] += fy;
    }
    (void) threads;
}

/* Quadrant around (cx, cy): src/forceatlas2.c:43. */
static inline int quadrant(const fa2_node *p, double cx, double cy)
{
    return (p->x < cx ? 0 : 2) + (p->y < cy ? 0 : 1);
}

static inline int one_quadrant(const int *c, int count)
{
    return c[0] == count || c[1] == count || c[2] == count || c[3] == count;
}

void orc_tree_build(fa2_tree *t, int n, const double *x, const double *y,
                    const double *mass, const double *size)
{
    orc_tree_build_mt(t, n, x, y, mass, size, 1);
}

void orc_tree_build_mt(fa2_tree *t, int n, const double *x, const double *y,
                       const double *mass, const double *size, int threads)
{
    /* src/forceatlas2.c:64-239, breadth first, one level at a time; the
     * regions of a level in parallel as there (:104-108, :166-168,
     * :220-221): the tree does not depend on the number of threads. */
    fa2_region *R = t->reg;
#ifndef _OPENMP
    (void) threads;
#endif

    {   /* the root: every node, in index order (:74-97) */
        fa2_node *nd = t->buf[0];
        double msum = 0.0, sx = 0.0, sy = 0.0;
        for (int i = 0; i < n; i++) {
            nd[i].x = x[i];
            nd[i].y = y[i];
            nd[i].m = mass[i];
            nd[i].idx = i;
            msum += mass[i];
            sx += x[i] * mass[i];
            sy += y[i] * mass[i];
        }
        R[0].start = 0;
        R[0].count = n;
        R[0].skip = -1;
        R[0].buf = 0;
        R[0].child = -1;
        R[0].nchild = 0;
        R[0].mass = n > 1 ? msum : mass[0];
        R[0].cx = n > 1 ? sx / msum : x[0];
        R[0].cy = n > 1 ? sy / msum : y[0];
        R[0].size = 0.0;
        t->nreg = 1;
    }

    int lo = 0, hi = 1;
    while (lo < hi) {
#ifdef _OPENMP
        int chunk = (hi - lo) / (8 * (threads > 0 ? threads : 1));
        if (chunk < 1) chunk = 1;
#endif
        /* (1) size of each region and its quadrant counts (:106-126) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(dynamic, chunk) if (threads > 1 && hi - lo > 1)
#endif
        for (int r = lo; r < hi; r++) {
            int *c = t->cnt + 4 * (size_t) (r - lo);
            c[0] = c[1] = c[2] = c[3] = 0;
            if (R[r].count < 2) continue;
            const fa2_node *nd = t->buf[R[r].buf] + R[r].start;
            const double cx = R[r].cx, cy = R[r].cy;
            double d2max = 0.0;
            for (int k = 0; k < R[r].count; k++) {
                const double ex = nd[k].x - cx, ey = nd[k].y - cy;
                const double d2 = ex * ex + ey * ey;
                if (d2 > d2max) d2max = d2;
                c[quadrant(&nd[k], cx, cy)]++;
            }
            R[r].size = 2.0 * sqrt(d2max);
        }

        /* (2) the regions of the next level, in order (:128-164) */
        for (int r = lo; r < hi; r++) {
            const int *c = t->cnt + 4 * (size_t) (r - lo);
            const int start = R[r].start, count = R[r].count;
            if (count <= ORC_LEAF) continue;
            R[r].child = t->nreg;
            if (one_quadrant(c, count)) {
                /* coincident nodes: one leaf each, kept in place */
                R[r].nchild = count;
                for (int k = start; k < start + count; k++) {
                    fa2_region *ch = &R[t->nreg];
                    ch->start = k;
                    ch->count = 1;
                    ch->skip = k == start ? R[r].skip : t->nreg - 1;
                    ch->buf = R[r].buf;
                    ch->child = -1;
                    ch->nchild = 0;
                    t->nreg++;
                }
                continue;
            }
            int off = start;
            for (int q = 0; q < 4; q++) {
                if (c[q] == 0) continue;
                fa2_region *ch = &R[t->nreg];
                ch->start = off;
                ch->count = c[q];
                ch->skip = R[r].nchild == 0 ? R[r].skip : t->nreg - 1;
                ch->buf = 1 - R[r].buf;
                ch->child = -1;
                ch->nchild = 0;
                R[r].nchild++;
                t->nreg++;
                off += c[q];
            }
        }

        /* (3) move the nodes to their quadrant; masses and centres (:166-216) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(dynamic, chunk) if (threads > 1 && hi - lo > 1)
#endif
        for (int r = lo; r < hi; r++) {
            const int *c = t->cnt + 4 * (size_t) (r - lo);
            if (R[r].nchild == 0) continue;
            const fa2_node *nd = t->buf[R[r].buf] + R[r].start;
            if (!one_quadrant(c, R[r].count)) {
                fa2_node *out = t->buf[1 - R[r].buf];
                const double cx = R[r].cx, cy = R[r].cy;
                double qm[4] = {0, 0, 0, 0}, qx[4] = {0, 0, 0, 0},
                       qy[4] = {0, 0, 0, 0};
                int at[4];
                at[0] = R[r].start;
                for (int q = 1; q < 4; q++) at[q] = at[q - 1] + c[q - 1];
                for (int k = 0; k < R[r].count; k++) {
                    const int q = quadrant(&nd[k], cx, cy);
                    out[at[q]++] = nd[k];
                    qm[q] += nd[k].m;
                    qx[q] += nd[k].x * nd[k].m;
                    qy[q] += nd[k].y * nd[k].m;
                }
                fa2_region *ch = &R[R[r].child];
                for (int q = 0; q < 4; q++) {
                    if (c[q] == 0) continue;
                    ch->mass = qm[q];
                    ch->cx = qx[q] / qm[q];
                    ch->cy = qy[q] / qm[q];
                    ch->size = 0.0;
                    ch++;
                }
                nd = out + R[r].start;
            }
            /* a region of one node is exactly that node (:206-215) */
            for (int j = 0; j < R[r].nchild; j++) {
                fa2_region *ch = &R[R[r].child + j];
                if (ch->count > 1) continue;
                const fa2_node *p = nd + (ch->start - R[r].start);
                ch->mass = p->m;
                ch->cx = p->x;
                ch->cy = p->y;
                ch->size = 0.0;
            }
        }
        lo = hi;
        hi = t->nreg;
    }

    /* nodes in tree order, from the buffer that holds each leaf (:222-238) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
    for (int r = 0; r < t->nreg; r++) {
        if (R[r].nchild > 0) continue;
        const fa2_node *nd = t->buf[R[r].buf];
        for (int k = R[r].start; k < R[r].start + R[r].count; k++) {
            const int i = nd[k].idx;
            t->perm[k] = i;
            t->px[k] = nd[k].x;
            t->py[k] = nd[k].y;
            t->pm[k] = nd[k].m;
            if (size && t->ps) t->ps[k] = size[i];
        }
    }
}

/* One node's Barnes-Hut repulsion (src/forceatlas2.c:326-368). */
static void repulse_one_bh(const fa2_tree *t, int i, double xi, double yi,
                           double mi, double si, int adjust, double scaling,
                           double theta2, int *stack, double *fxo,
                           double *fyo)
{
    double fx = 0.0, fy = 0.0;
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const fa2_region *r = &t->reg[stack[--sp]];
        if (r->count > 1) {
            const double xd = xi - r->cx, yd = yi - r->cy;
            const double d2 = xd * xd + yd * yd;
            if (d2 * theta2 > r->size * r->size) {
                const double f = scaling * (mi * r->mass) / d2;
                fx += xd * f;
                fy += yd * f;
                continue;
            }
            if (r->nchild > 0) {
                for (int c = 0; c < r->nchild; c++) stack[sp++] = r->child + c;
                continue;
            }
        }
        const int end = r->start + r->count;
        for (int k = r->start; k < end; k++) {
            if (t->perm[k] == i) continue;
            const double xd = xi - t->px[k], yd = yi - t->py[k];
            const double f =
                rep_factor(adjust, scaling, xd * xd + yd * yd, mi * t->pm[k],
                           adjust ? si + t->ps[k] : 0.0);
            fx += xd * f;
            fy += yd * f;
        }
    }
    *fxo = fx;
    *fyo = fy;
}

void orc_repulse_bh(int n, const fa2_tree *t, const double *x,
                    const double *y, const double *mass, const double *size,
                    int adjust, double scaling, double theta, int threads,
                    double *dx, double *dy)
{
    const double theta2 = theta * theta;
    const size_t slen = 2 * (size_t) n + 4;
    int nthr = threads > 1 ? threads : 1;
    int *stacks = (int *) malloc(slen * (size_t) nthr * sizeof(int));
    if (!stacks) return;
    /* nodes in tree order, as the reference (src/forceatlas2.c:719-729) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 64) if (nthr > 1)
#endif
    for (int k = 0; k < n; k++) {
#ifdef _OPENMP
        int *stack = stacks + slen * (size_t) omp_get_thread_num();
#else
        int *stack = stacks;
#endif
        const int i = t->perm[k];
        double fx, fy;
        repulse_one_bh(t, i, x[i], y[i], mass[i], adjust ? size[i] : 0.0,
                       adjust, scaling, theta2, stack, &fx, &fy);
        dx[i] += fx;
        dy[i] += fy;
    }
    free(stacks);
}

void orc_gravity(int n, const double *x, const double *y, const double *mass,
                 double gravity, int strong, double *dx, double *dy)
{
    /* src/forceatlas2.c:371-381 */
    for (int i = 0; i < n; i++) {
        const double xi = x[i], yi = y[i];
        const double dist = sqrt(xi * xi + yi * yi);
        if (dist > 0) {
            const double f =
                strong ? gravity * mass[i] : gravity * mass[i] / dist;
            dx[i] -= xi * f;
            dy[i] -= yi * f;
        }
    }
}

/* src/forceatlas2.c:385-399 */
static inline double att_factor(const double *w, const double *mass,
                                const double *size, int a, int b, int e,
                                double coef, double xd, double yd, int linlog,
                                int outbound, int adjust)
{
    double f = -coef * w[e];
    if (adjust || linlog) {
        double dist = sqrt(xd * xd + yd * yd);
        if (adjust) dist -= size[a] + size[b];
        if (!(dist > 0)) return 0.0;
        if (linlog) f *= log1p(dist) / dist;
    }
    if (outbound) f /= mass[a];
    return f;
}

void orc_attract(int n, int m, const int *from, const int *to,
                 const double *w, const double *x, const double *y,
                 const double *mass, const double *size, double coef,
                 int linlog, int outbound, int adjust, double *dx, double *dy)
{
    /* src/forceatlas2.c:402-416 */
    (void) n;
    for (int e = 0; e < m; e++) {
        const int a = from[e], b = to[e];
        if (a == b) continue;
        const double xd = x[a] - x[b], yd = y[a] - y[b];
        const double f = att_factor(w, mass, size, a, b, e, coef, xd, yd,
                                    linlog, outbound, adjust);
        if (f == 0.0) continue;
        dx[a] += xd * f;
        dy[a] += yd * f;
        dx[b] -= xd * f;
        dy[b] -= yd * f;
    }
}

void orc_update_speed(int n, double total_swinging, double total_traction,
                      double jitter_tolerance, double *speed_,
                      double *speed_efficiency_)
{
    /* src/forceatlas2.c:445-485 */
    double speed = *speed_, eff = *speed_efficiency_;
    if (!(total_swinging > 0)) return;

    const double est = 0.05 * sqrt((double) n);
    const double min_jt = sqrt(est), max_jt = 10.0;
    double jt = est * total_traction / ((double) n * (double) n);
    if (jt > max_jt) jt = max_jt;
    if (jt < min_jt) jt = min_jt;
    jt *= jitter_tolerance;

    if (total_swinging > 2.0 * total_traction) {
        if (eff > 0.05) eff *= 0.5;
        if (jt < jitter_tolerance) jt = jitter_tolerance;
    }
    const double target = jt * eff * total_traction / total_swinging;
    if (total_swinging > jt * total_traction) {
        if (eff > 0.05) eff *= 0.7;
    } else if (speed < 1000) {
        eff *= 1.3;
    }
    const double rise = target - speed;
    speed += rise < 0.5 * speed ? rise : 0.5 * speed;
    *speed_ = speed;
    *speed_efficiency_ = eff;
}

/* Quadtree storage for n nodes; NULL on allocation failure. */
static int tree_alloc(fa2_tree *t, int n, int with_size)
{
    memset(t, 0, sizeof(*t));
    const size_t nn = (size_t) (n > 0 ? n : 1);
    t->reg = (fa2_region *) malloc(2 * nn * sizeof(fa2_region));
    t->perm = (int *) malloc(nn * sizeof(int));
    t->cnt = (int *) malloc(4 * nn * sizeof(int));
    t->buf[0] = (fa2_node *) malloc(nn * sizeof(fa2_node));
    t->buf[1] = (fa2_node *) malloc(nn * sizeof(fa2_node));
    t->px = (double *) malloc(nn * sizeof(double));
    t->py = (double *) malloc(nn * sizeof(double));
    t->pm = (double *) malloc(nn * sizeof(double));
    t->ps = with_size ? (double *) malloc(nn * sizeof(double)) : NULL;
    return t->reg && t->perm && t->cnt && t->buf[0] && t->buf[1] && t->px &&
           t->py && t->pm && (!with_size || t->ps);
}

static void tree_free(fa2_tree *t)
{
    free(t->reg);
    free(t->perm);
    free(t->cnt);
    free(t->buf[0]);
    free(t->buf[1]);
    free(t->px);
    free(t->py);
    free(t->pm);
    free(t->ps);
}

int orc_forces(int n, int m, const int *from, const int *to, const double *w,
               const double *pos, const double *size, const orc_opts *o,
               double *f)
{
    if (n < 1) return 1;
    double *mass = (double *) malloc((size_t) n * sizeof(double));
    if (!mass) return 1;
    double mean;
    orc_mass(n, m, from, to, mass, &mean);
    const double *x = pos, *y = pos + n;
    double *dx = f, *dy = f + n;
    memset(f, 0, 2 * (size_t) n * sizeof(double));
    const int thr = o->threads > 1 ? o->threads : 1;
    if (o->barnes_hut) {
        fa2_tree t;
        if (!tree_alloc(&t, n, o->adjust)) {
            tree_free(&t);
            free(mass);
            return 1;
        }
        orc_tree_build_mt(&t, n, x, y, mass, o->adjust ? size : NULL, thr);
        orc_repulse_bh(n, &t, x, y, mass, size, o->adjust, o->scaling,
                       o->theta, thr, dx, dy);
        tree_free(&t);
    } else {
        orc_repulse_exact(n, x, y, mass, size, o->adjust, o->scaling, thr, dx,
                          dy);
    }
    if (o->gravity != 0)
        orc_gravity(n, x, y, mass, o->gravity, o->strong, dx, dy);
    orc_attract(n, m, from, to, w, x, y, mass, size,
                o->outbound ? mean : 1.0, o->linlog, o->outbound, o->adjust,
                dx, dy);
    free(mass);
    return 0;
}

/* Node-wise attraction over the incidence list of C_forceatlas2
 * (src/forceatlas2.c:422-441); same results as orc_attract. */
static void attract_node(const int *from, const int *to, const double *w,
                         const double *x, const double *y, const double *mass,
                         const double *size, double coef, int linlog,
                         int outbound, int adjust, const int *off,
                         const int *inc, int i, double *dx, double *dy)
{
    double fx = dx[i], fy = dy[i];
    for (int k = off[i]; k < off[i + 1]; k++) {
        const int e = inc[k] >> 1;
        const int a = from[e], b = to[e];
        const double xd = x[a] - x[b], yd = y[a] - y[b];
        const double f = att_factor(w, mass, size, a, b, e, coef, xd, yd,
                                    linlog, outbound, adjust);
        if (f == 0.0) continue;
        if (inc[k] & 1) {
            fx -= xd * f;
            fy -= yd * f;
        } else {
            fx += xd * f;
            fy += yd * f;
        }
    }
    dx[i] = fx;
    dy[i] = fy;
}

static int layout_impl(int n, int m, const int *from, const int *to,
                       const double *w, double *pos, const double *size,
                       const int *fixed, int iterations, const orc_opts *o,
                       double *trace);

int orc_layout(int n, int m, const int *from, const int *to, const double *w,
               double *pos, const double *size, const int *fixed,
               int iterations, const orc_opts *o)
{
    return layout_impl(n, m, from, to, w, pos, size, fixed, iterations, o,
                       NULL);
}

int orc_layout_trace(int n, int m, const int *from, const int *to,
                     const double *w, double *pos, const double *size,
                     const int *fixed, int iterations, const orc_opts *o,
                     double *trace)
{
    return layout_impl(n, m, from, to, w, pos, size, fixed, iterations, o,
                       trace);
}

static int layout_impl(int n, int m, const int *from, const int *to,
                       const double *w, double *pos, const double *size,
                       const int *fixed, int iterations, const orc_opts *o,
                       double *trace)
{
    /* src/forceatlas2.c:521-803, the CPU branch (gpu = -1) */
    if (n < 0 || m < 0 || iterations < 0) return 1;
    for (int e = 0; e < m; e++)
        if (from[e] < 0 || from[e] >= n || to[e] < 0 || to[e] >= n) return 1;
    if (n == 0 || iterations == 0) return 0;
    const int threads = o->threads > 1 ? o->threads : 1;
    const size_t nn = (size_t) n;
    double *x = pos, *y = pos + n;
    double *mass = (double *) malloc(nn * sizeof(double));
    double *buf = (double *) calloc(6 * nn, sizeof(double));
    int *off = NULL, *inc = NULL;
    fa2_tree t;
    memset(&t, 0, sizeof(t));
    int status = 1;
    if (!mass || !buf) goto out;
    double *dx = buf, *dy = buf + nn, *odx = buf + 2 * nn, *ody = buf + 3 * nn;
    double *sw = buf + 4 * nn, *tr = buf + 5 * nn;
    double mean;
    orc_mass(n, m, from, to, mass, &mean);

    /* the incidence list for the node-wise attraction (:607-631) */
    if (threads > 1 && m > 0) {
        off = (int *) calloc(nn + 1, sizeof(int));
        inc = (int *) malloc(2 * (size_t) m * sizeof(int));
        if (!off || !inc) goto out;
        for (int e = 0; e < m; e++) {
            if (from[e] == to[e]) continue;
            off[from[e] + 1]++;
            off[to[e] + 1]++;
        }
        for (int i = 0; i < n; i++) off[i + 1] += off[i];
        for (int e = 0; e < m; e++) {
            if (from[e] == to[e]) continue;
            inc[off[from[e]]++] = 2 * e;
            inc[off[to[e]]++] = 2 * e + 1;
        }
        for (int i = n; i > 0; i--) off[i] = off[i - 1];
        off[0] = 0;
    }
    if (o->barnes_hut && !tree_alloc(&t, n, o->adjust)) goto out;

    const double coef = o->outbound ? mean : 1.0;
    double speed = 1.0, eff = 1.0;
    if (trace) memcpy(trace, pos, 2 * nn * sizeof(double));
    for (int it = 0; it < iterations; it++) {
        double *tmp = odx;
        odx = dx;
        dx = tmp;
        tmp = ody;
        ody = dy;
        dy = tmp;
        memset(dx, 0, nn * sizeof(double));
        memset(dy, 0, nn * sizeof(double));

        if (o->barnes_hut) {
            orc_tree_build_mt(&t, n, x, y, mass, o->adjust ? size : NULL, threads);
            orc_repulse_bh(n, &t, x, y, mass, size, o->adjust, o->scaling,
                           o->theta, threads, dx, dy);
        } else {
            orc_repulse_exact(n, x, y, mass, size, o->adjust, o->scaling,
                              threads, dx, dy);
        }
        if (o->gravity != 0) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
            for (int i = 0; i < n; i++) {
                const double dist = sqrt(x[i] * x[i] + y[i] * y[i]);
                if (dist > 0) {
                    const double f = o->strong
                                         ? o->gravity * mass[i]
                                         : o->gravity * mass[i] / dist;
                    dx[i] -= x[i] * f;
                    dy[i] -= y[i] * f;
                }
            }
        }
        if (inc) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
#endif
            for (int i = 0; i < n; i++)
                attract_node(from, to, w, x, y, mass, size, coef, o->linlog,
                             o->outbound, o->adjust, off, inc, i, dx, dy);
        } else {
            orc_attract(n, m, from, to, w, x, y, mass, size, coef, o->linlog,
                        o->outbound, o->adjust, dx, dy);
        }

        /* swinging and traction, sums in node order (:758-775) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
        for (int i = 0; i < n; i++) {
            const double sx = odx[i] - dx[i], sy = ody[i] - dy[i];
            const double tx = odx[i] + dx[i], ty = ody[i] + dy[i];
            sw[i] = mass[i] * sqrt(sx * sx + sy * sy);
            tr[i] = 0.5 * mass[i] * sqrt(tx * tx + ty * ty);
        }
        double tsw = 0.0, ttr = 0.0;
        for (int i = 0; i < n; i++) {
            if (fixed && fixed[i]) continue;
            tsw += sw[i];
            ttr += tr[i];
        }
        orc_update_speed(n, tsw, ttr, o->jitter_tolerance, &speed, &eff);

        /* displacement (:780-802) */
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
        for (int i = 0; i < n; i++) {
            if (fixed && fixed[i]) continue;
            double factor;
            if (o->adjust) {
                const double df = sqrt(dx[i] * dx[i] + dy[i] * dy[i]);
                factor = 0.1 * speed / (1.0 + sqrt(speed * sw[i]));
                if (df > 0) {
                    if (factor * df > 10.0) factor = 10.0 / df;
                } else {
                    factor = 0.0;
                }
            } else {
                factor = speed / (1.0 + sqrt(speed * sw[i]));
            }
            x[i] += dx[i] * factor;
            y[i] += dy[i] * factor;
        }
        if (trace)
            memcpy(trace + 2 * nn * (size_t) (it + 1), pos,
                   2 * nn * sizeof(double));
    }
    status = 0;
out:
    if (o->barnes_hut) tree_free(&t);
    free(mass);
    free(buf);
    free(off);
    free(inc);
    return status;
}

int orc_prepare_large(int n, int m, const int *from, const int *to,
                      const double *w, int outbound, double *mass, int *off,
                      int *inc_node, double *inc_coef)
{
    /* src/forceatlas2.c:870-902 */
    double mean;
    orc_mass(n, m, from, to, mass, &mean);
    const double coef = outbound ? mean : 1.0;
    memset(off, 0, ((size_t) n + 1) * sizeof(int));
    for (int e = 0; e < m; e++) {
        if (from[e] == to[e]) continue;
        off[from[e] + 1]++;
        off[to[e] + 1]++;
    }
    for (int i = 0; i < n; i++) off[i + 1] += off[i];
    for (int e = 0; e < m; e++) {
        if (from[e] == to[e]) continue;
        const double c =
            outbound ? coef * w[e] / mass[from[e]] : coef * w[e];
        inc_node[off[from[e]]] = to[e];
        inc_coef[off[from[e]]++] = c;
        inc_node[off[to[e]]] = from[e];
        inc_coef[off[to[e]]++] = c;
    }
    for (int i = n; i > 0; i--) off[i] = off[i - 1];
    off[0] = 0;
    return off[n];
}

/* ------------------------------------------------------------------------ */
/* Part 2: the pipeline, precision-independent pieces                       */
/* ------------------------------------------------------------------------ */

void orc_pipe_sort(int n, uint32_t *key, uint32_t *idx)
{
    /* Stable LSD radix sort, 4 passes of 8 bits (pipeline.cl:136-188). One
     * counting pass over the whole array gives the same order as the
     * reference's blocked histograms: blocks are consecutive and scattered
     * in block order. */
    uint32_t *k2 = (uint32_t *) malloc((size_t) (n > 0 ? n : 1) * 4);
    uint32_t *i2 = (uint32_t *) malloc((size_t) (n > 0 ? n : 1) * 4);
    if (!k2 || !i2) {
        free(k2);
        free(i2);
        return;
    }
    uint32_t *ka = key, *ia = idx, *kb = k2, *ib = i2;
    for (int pass = 0; pass < 4; pass++) {
        const int shift = 8 * pass;
        uint32_t cnt[256];
        memset(cnt, 0, sizeof(cnt));
        for (int i = 0; i < n; i++) cnt[(ka[i] >> shift) & 255u]++;
        uint32_t base = 0;
        for (int d = 0; d < 256; d++) {
            const uint32_t c = cnt[d];
            cnt[d] = base;
            base += c;
        }
        for (int i = 0; i < n; i++) {
            const uint32_t p = cnt[(ka[i] >> shift) & 255u]++;
            kb[p] = ka[i];
            ib[p] = ia[i];
        }
        uint32_t *t = ka;
        ka = kb;
        kb = t;
        t = ia;
        ia = ib;
        ib = t;
    }
    /* four passes: the result is back in key / idx */
    free(k2);
    free(i2);
}

static inline int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }

/* Common prefix of sorted keys i and j, -1 outside; equal keys are told
 * apart by their positions (pipeline.cl:209-217). */
static inline int prefix(const uint32_t *key, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = key[i], b = key[j];
    if (a == b) return 32 + clz32((uint32_t) (i ^ j));
    return clz32(a ^ b);
}

void orc_pipe_tree(int n, const uint32_t *key, int *child, int *range,
                   int *parent)
{
    /* Karras (2012) binary radix tree (pipeline.cl:219-270): internal nodes
     * 0 .. n-2, leaves n-1 .. 2n-2 in sorted order. */
    for (int i = 0; i < n - 1; i++) {
        const int d = prefix(key, n, i, i + 1) > prefix(key, n, i, i - 1)
                          ? 1 : -1;
        const int pmin = prefix(key, n, i, i - d);
        int lmax = 2;
        while (prefix(key, n, i, i + lmax * d) > pmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (prefix(key, n, i, i + (l + t) * d) > pmin) l += t;
        const int j = i + l * d;
        const int pnode = prefix(key, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (prefix(key, n, i, i + (s + t) * d) > pnode) s += t;
        } while (t > 1);
        const int split = i + s * d + (d < 0 ? d : 0);
        const int first = i < j ? i : j, last = i < j ? j : i;
        const int left = first == split ? n - 1 + split : split;
        const int right = last == split + 1 ? n - 1 + split + 1 : split + 1;
        child[2 * i] = left;
        child[2 * i + 1] = right;
        range[2 * i] = first;
        range[2 * i + 1] = last;
        parent[left] = i;
        parent[right] = i;
    }
    if (n >= 1) parent[0] = -1;
}

/* Part 2 in both precisions */
#define real float
#define S f
#include "pipe_impl.h"
#undef real
#undef S
#define real double
#define S d
#include "pipe_impl.h"
#undef real
#undef S

/* ------------------------------------------------------------------------ */
/* The construction of the FP32 path of libfa2cuda.so                       */
/* ------------------------------------------------------------------------ */

/* The float walk of that path: regions in float, but a region whose test
 * d^2 theta^2 > size^2 is within 1e-4 of the boundary is decided in double
 * from the double construction, so that the float path approximates the
 * regions the double path approximates. The forces of the far regions are
 * added in walk order, then those of the node pairs (the small regions too
 * close and the single nodes), in walk order: the order of the path's walk,
 * which queues the pairs (walk_deferred). */
static void repulse_mixed(const pipe_ws_f *w, const pipe_ws_d *wd,
                          float scaling, float theta2, double theta2d,
                          int adjust, float *f)
{
    const int n = w->n;
    const float *ps = w->psort, *ni = w->ni;
    int *pairs = (int *) malloc(2 * (size_t) n * 2 * sizeof(int));
    if (!pairs) return;
    for (int k = 0; k < n; k++) {
        const float xi = ps[4 * k], yi = ps[4 * k + 1];
        const float mi = ps[4 * k + 2], si = ps[4 * k + 3];
        const float smi = scaling * mi; /* a far region's pull: smi m / d^2 */
        float ax = 0.0f, ay = 0.0f;
        int np = 0; /* queued ranges (first, last) */
        int stack[160];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int r = stack[--sp];
            int first, last;
            if (r >= n - 1) {
                first = last = r - (n - 1);
            } else {
                const float xd = xi - ni[4 * r], yd = yi - ni[4 * r + 1];
                const float d2 = xd * xd + yd * yd;
                const float lhs = d2 * theta2;
                int far = lhs > ni[4 * r + 3];
                if (fabsf(lhs - ni[4 * r + 3]) <= 1e-4f * ni[4 * r + 3]) {
                    const double ex = (double) xi - wd->ni[4 * r];
                    const double ey = (double) yi - wd->ni[4 * r + 1];
                    far = (ex * ex + ey * ey) * theta2d > wd->ni[4 * r + 3];
                }
                if (far) {
                    const float g = smi * ni[4 * r + 2] / d2;
                    ax += xd * g;
                    ay += yd * g;
                    continue;
                }
                first = w->range[2 * r];
                last = w->range[2 * r + 1];
                if (last - first >= ORC_LEAF) {
                    stack[sp++] = w->child[2 * r + 1];
                    stack[sp++] = w->child[2 * r];
                    continue;
                }
            }
            pairs[2 * np] = first;
            pairs[2 * np + 1] = last;
            np++;
        }
        for (int b = 0; b < np; b++) {
            for (int j = pairs[2 * b]; j <= pairs[2 * b + 1]; j++) {
                if (j == k) continue;
                const float xd = xi - ps[4 * j], yd = yi - ps[4 * j + 1];
                const float g = rep_f(xd * xd + yd * yd, mi * ps[4 * j + 2],
                                      si + ps[4 * j + 3], scaling, adjust);
                ax += xd * g;
                ay += yd * g;
            }
        }
        const uint32_t i = w->order[k];
        f[2 * i] = ax;
        f[2 * i + 1] = ay;
    }
    free(pairs);
}

/* Its gravity and attraction, summed apart from the repulsion (the device
 * computes them beside the walk) and then added to it: from 0, the
 * gravity, then the incidences in edge order; a node of at least ORC_HEAVY
 * incidences starts from its attraction, as 32 interleaved partial sums
 * (incidence e to partial e mod 32, each in edge order) added pairwise
 * across distances 16, 8, 4, 2, 1 -- a warp's sum on the device -- and
 * adds its gravity. */
#define ORC_HEAVY 128
static void attract_mixed(int n, float gravity, int strong, int linlog,
                          int adjust, const float *p, const float *mass,
                          const float *size, const int *off,
                          const int *inc_node, const float *inc_coef, float *f)
{
    for (int i = 0; i < n; i++) {
        const float xi = p[2 * i], yi = p[2 * i + 1];
        const float si = adjust ? size[i] : 0.0f;
        const int heavy = off[i + 1] - off[i] >= ORC_HEAVY;
        float lx[32], ly[32];
        if (heavy) {
            for (int l = 0; l < 32; l++) {
                lx[l] = ly[l] = 0.0f;
                for (int e = off[i] + l; e < off[i + 1]; e += 32) {
                    const int j = inc_node[e];
                    const float xd = xi - p[2 * j], yd = yi - p[2 * j + 1];
                    float g = -inc_coef[e];
                    if (adjust || linlog) {
                        float dist = sqrtf(xd * xd + yd * yd);
                        if (adjust) dist -= si + size[j];
                        if (!(dist > 0.0f)) continue;
                        if (linlog) g *= log1pf(dist) / dist;
                    }
                    lx[l] += xd * g;
                    ly[l] += yd * g;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                float tx[32], ty[32];
                for (int l = 0; l < 32; l++) {
                    tx[l] = lx[l] + lx[l ^ o];
                    ty[l] = ly[l] + ly[l ^ o];
                }
                memcpy(lx, tx, sizeof(lx));
                memcpy(ly, ty, sizeof(ly));
            }
        }
        float ax = heavy ? lx[0] : 0.0f, ay = heavy ? ly[0] : 0.0f;
        if (gravity != 0.0f) {
            const float dist = sqrtf(xi * xi + yi * yi);
            if (dist > 0.0f) {
                const float g = strong ? gravity * mass[i] : gravity * mass[i] / dist;
                ax -= xi * g;
                ay -= yi * g;
            }
        }
        if (!heavy) {
            for (int e = off[i]; e < off[i + 1]; e++) {
                const int j = inc_node[e];
                const float xd = xi - p[2 * j], yd = yi - p[2 * j + 1];
                float g = -inc_coef[e];
                if (adjust || linlog) {
                    float dist = sqrtf(xd * xd + yd * yd);
                    if (adjust) dist -= si + size[j];
                    if (!(dist > 0.0f)) continue;
                    if (linlog) g *= log1pf(dist) / dist;
                }
                ax += xd * g;
                ay += yd * g;
            }
        }
        f[2 * i] += ax;
        f[2 * i + 1] += ay;
    }
}

/* Forces as that path computes them: the tree is built in double from the
 * positions and masses rounded to float (keys, order, regions: the double
 * construction of pipeline.cl), the regions' records are rounded to float,
 * and the walk (with the decisions above) and the attraction (with the
 * heavy nodes' order above) run in float (pipeline.cl:332-429). */
int orc_pipe_forces_m(const fa2_full_params *pp, const double *pos,
                      double *fout)
{
    const int n = pp->n;
    if (n < 2) return 1;
    pipe_ws_d wd;
    pipe_ws_f wf;
    pipe_graph_f gf;
    memset(&wd, 0, sizeof(wd));
    memset(&wf, 0, sizeof(wf));
    memset(&gf, 0, sizeof(gf));
    double *pr = (double *) malloc(2 * (size_t) n * sizeof(double));
    double *mr = (double *) malloc((size_t) n * sizeof(double));
    float *f = (float *) malloc(2 * (size_t) n * sizeof(float));
    int ok = pr && mr && f && ws_alloc_d(&wd, n) && ws_alloc_f(&wf, n) &&
             graph_load_f(&gf, pp, pos);
    if (ok) {
        for (int i = 0; i < n; i++) {
            pr[2 * i] = (double) gf.p[2 * i];
            pr[2 * i + 1] = (double) gf.p[2 * i + 1];
            mr[i] = (double) gf.mass[i];
        }
        build_core_d(&wd, pr, mr, NULL, 0);
        memcpy(wf.key, wd.key, (size_t) n * 4);
        memcpy(wf.order, wd.order, (size_t) n * 4);
        memcpy(wf.child, wd.child, 2 * (size_t) (n - 1) * sizeof(int));
        memcpy(wf.range, wd.range, 2 * (size_t) (n - 1) * sizeof(int));
        for (size_t r = 0; r < 4 * (size_t) (n - 1); r++)
            wf.ni[r] = (float) wd.ni[r];
        for (int k = 0; k < n; k++) {
            const uint32_t i = wf.order[k];
            wf.psort[4 * k] = gf.p[2 * i];
            wf.psort[4 * k + 1] = gf.p[2 * i + 1];
            wf.psort[4 * k + 2] = gf.mass[i];
            wf.psort[4 * k + 3] = pp->adjust ? gf.size[i] : 0.0f;
        }
        repulse_mixed(&wf, &wd, (float) pp->scaling,
                      (float) (pp->theta * pp->theta), pp->theta * pp->theta,
                      pp->adjust, f);
        attract_mixed(n, (float) pp->gravity, pp->strong, pp->linlog,
                      pp->adjust, gf.p, gf.mass, gf.size, pp->inc_off,
                      pp->inc_node, gf.coef, f);
        for (int i = 0; i < n; i++) {
            fout[i] = (double) f[2 * i];
            fout[n + i] = (double) f[2 * i + 1];
        }
    }
    ws_free_d(&wd);
    ws_free_f(&wf);
    graph_free_f(&gf);
    free(pr);
    free(mr);
    free(f);
    return ok ? 0 : 1;
}
