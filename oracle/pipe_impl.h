/*
 * pipe_impl.h -- ORACLE, test infrastructure only.
 *
 * Part 2 of fa2_oracle.c: the all-GPU construction of inst/opencl/pipeline.cl
 * restated for the CPU. Included twice, with `real` defined as float and as
 * double and S as f and d. Every arithmetic step is the reference's, in the
 * reference's order and precision, so that Morton codes, the sorted order
 * and the tree are bit-exact and the forces are those of the same
 * construction.
 */
#ifndef ORC_CAT
#define ORC_CAT_(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT_(a, b)
#define R_SQRT(x) _Generic((x), float: sqrtf, default: sqrt)(x)
#define R_LOG1P(x) _Generic((x), float: log1pf, default: log1p)(x)
#endif
#define PF(name) ORC_CAT(ORC_CAT(name, _), S)

/* OpenCL min/max/clamp on reals (no NaN input here). */
static inline real PF(rmin)(real a, real b) { return b < a ? b : a; }
static inline real PF(rmax)(real a, real b) { return a < b ? b : a; }

/* pipeline.cl:46-55 */
static inline real PF(rep)(real d2, real mm, real ss, real scaling,
                           int adjust)
{
    if (adjust) {
        const real d = R_SQRT(d2) - ss;
        if (d > (real) 0) return scaling * mm / (d * d);
        if (d < (real) 0) return (real) 100 * scaling * mm;
        return (real) 0;
    }
    return d2 > (real) 0 ? scaling * mm / d2 : (real) 0;
}

/* A zero bit inserted above each of the 16 low bits. */
static inline uint32_t PF(spread)(uint32_t v)
{
    v &= 0xFFFFu;
    v = (v ^ (v << 8)) & 0x00FF00FFu;
    v = (v ^ (v << 4)) & 0x0F0F0F0Fu;
    v = (v ^ (v << 2)) & 0x33333333u;
    v = (v ^ (v << 1)) & 0x55555555u;
    return v;
}

/* bbox (pipeline.cl:61-99; min and max are exact, so the blocking of the
 * reference does not matter) and Morton codes (pipeline.cl:116-130). */
static void PF(morton_core)(int n, const real *p, uint32_t *key,
                            uint32_t *idx, real *bb)
{
    real minx = p[0], maxx = p[0], miny = p[1], maxy = p[1];
    for (int i = 1; i < n; i++) {
        minx = PF(rmin)(minx, p[2 * i]);
        maxx = PF(rmax)(maxx, p[2 * i]);
        miny = PF(rmin)(miny, p[2 * i + 1]);
        maxy = PF(rmax)(maxy, p[2 * i + 1]);
    }
    const real extent = PF(rmax)(maxx - minx, maxy - miny);
    const real scale = extent > (real) 0 ? (real) 65535 / extent : (real) 0;
    for (int i = 0; i < n; i++) {
        const real fx = PF(rmin)(
            PF(rmax)((p[2 * i] - minx) * scale, (real) 0), (real) 65535);
        const real fy = PF(rmin)(
            PF(rmax)((p[2 * i + 1] - miny) * scale, (real) 0), (real) 65535);
        key[i] = PF(spread)((uint32_t) fx) | (PF(spread)((uint32_t) fy) << 1);
        idx[i] = (uint32_t) i;
    }
    if (bb) {
        bb[0] = minx;
        bb[1] = miny;
        bb[2] = maxx;
        bb[3] = maxy;
    }
}

void PF(orc_pipe_morton)(int n, const double *pos, uint32_t *key,
                         uint32_t *idx, double *bbox)
{
    real *p = (real *) malloc(2 * (size_t) n * sizeof(real));
    if (!p) return;
    for (int i = 0; i < n; i++) {
        p[2 * i] = (real) pos[i];
        p[2 * i + 1] = (real) pos[n + i];
    }
    real bb[4];
    PF(morton_core)(n, p, key, idx, bb);
    if (bbox)
        for (int c = 0; c < 4; c++) bbox[c] = (double) bb[c];
    free(p);
}

/* nd: bbox, mass, sum m*x, sum m*y for every tree node; the second child to
 * arrive computes its parent (pipeline.cl:276-305). ni: centre of mass, mass,
 * squared size of the regions (pipeline.cl:312-323). */
static void PF(aggregate_core)(int n, const real *psort, const int *child,
                               const int *parent, int *visits, real *nd,
                               real *ni)
{
    if (n < 2) return;
    memset(visits, 0, (size_t) (n - 1) * sizeof(int));
    for (int k = 0; k < n; k++) {
        const int leaf = n - 1 + k;
        const real x = psort[4 * k], y = psort[4 * k + 1],
                   m = psort[4 * k + 2];
        real *o = nd + 8 * (size_t) leaf;
        o[0] = x;
        o[1] = y;
        o[2] = x;
        o[3] = y;
        o[4] = m;
        o[5] = x * m;
        o[6] = y * m;
        o[7] = (real) 0;
        int r = parent[leaf];
        while (r >= 0) {
            if (visits[r]++ == 0) break;
            const real *a = nd + 8 * (size_t) child[2 * r];
            const real *b = nd + 8 * (size_t) child[2 * r + 1];
            real *q = nd + 8 * (size_t) r;
            q[0] = PF(rmin)(a[0], b[0]);
            q[1] = PF(rmin)(a[1], b[1]);
            q[2] = PF(rmax)(a[2], b[2]);
            q[3] = PF(rmax)(a[3], b[3]);
            q[4] = a[4] + b[4];
            q[5] = a[5] + b[5];
            q[6] = a[6] + b[6];
            q[7] = (real) 0;
            r = parent[r];
        }
    }
    for (int r = 0; r < n - 1; r++) {
        const real *q = nd + 8 * (size_t) r;
        const real m = q[4];
        const real w = q[2] - q[0];
        const real h = q[3] - q[1];
        ni[4 * r] = q[5] / m;
        ni[4 * r + 1] = q[6] / m;
        ni[4 * r + 2] = m;
        ni[4 * r + 3] = (real) 2 * (w * w + h * h);
    }
}

/* Work arrays of one construction. */
typedef struct {
    int n;
    uint32_t *key, *order;
    int *child, *range, *parent, *visits;
    real *psort, *nd, *ni;
} PF(pipe_ws);

static int PF(ws_alloc)(PF(pipe_ws) *w, int n)
{
    memset(w, 0, sizeof(*w));
    w->n = n;
    const size_t nn = (size_t) n;
    w->key = (uint32_t *) malloc(nn * 4);
    w->order = (uint32_t *) malloc(nn * 4);
    w->child = (int *) malloc(2 * nn * sizeof(int));
    w->range = (int *) malloc(2 * nn * sizeof(int));
    w->parent = (int *) malloc(2 * nn * sizeof(int));
    w->visits = (int *) malloc(nn * sizeof(int));
    w->psort = (real *) malloc(4 * nn * sizeof(real));
    w->nd = (real *) malloc(8 * 2 * nn * sizeof(real));
    w->ni = (real *) malloc(4 * nn * sizeof(real));
    return w->key && w->order && w->child && w->range && w->parent &&
           w->visits && w->psort && w->nd && w->ni;
}

static void PF(ws_free)(PF(pipe_ws) *w)
{
    free(w->key);
    free(w->order);
    free(w->child);
    free(w->range);
    free(w->parent);
    free(w->visits);
    free(w->psort);
    free(w->nd);
    free(w->ni);
}

/* Morton, sort, gather, tree, aggregate (src/gpu_full.c:413-443). */
static void PF(build_core)(PF(pipe_ws) *w, const real *p, const real *mass,
                           const real *size, int adjust)
{
    const int n = w->n;
    PF(morton_core)(n, p, w->key, w->order, NULL);
    orc_pipe_sort(n, w->key, w->order);
    for (int k = 0; k < n; k++) { /* gather, pipeline.cl:195-207 */
        const uint32_t i = w->order[k];
        w->psort[4 * k] = p[2 * i];
        w->psort[4 * k + 1] = p[2 * i + 1];
        w->psort[4 * k + 2] = mass[i];
        w->psort[4 * k + 3] = adjust ? size[i] : (real) 0;
    }
    orc_pipe_tree(n, w->key, w->child, w->range, w->parent);
    PF(aggregate_core)(n, w->psort, w->child, w->parent, w->visits, w->nd,
                       w->ni);
}

void PF(orc_pipe_build)(int n, const double *pos, const double *mass,
                        uint32_t *key, uint32_t *order, int *child,
                        int *range, int *parent, double *ni)
{
    if (n < 2) return;
    PF(pipe_ws) w;
    memset(&w, 0, sizeof(w));
    real *p = (real *) malloc(2 * (size_t) n * sizeof(real));
    real *m = (real *) malloc((size_t) n * sizeof(real));
    if (!p || !m || !PF(ws_alloc)(&w, n)) {
        free(p);
        free(m);
        PF(ws_free)(&w);
        return;
    }
    for (int i = 0; i < n; i++) {
        p[2 * i] = (real) pos[i];
        p[2 * i + 1] = (real) pos[n + i];
        m[i] = (real) mass[i];
    }
    PF(build_core)(&w, p, m, NULL, 0);
    memcpy(key, w.key, (size_t) n * 4);
    memcpy(order, w.order, (size_t) n * 4);
    memcpy(child, w.child, 2 * (size_t) (n - 1) * sizeof(int));
    memcpy(range, w.range, 2 * (size_t) (n - 1) * sizeof(int));
    memcpy(parent, w.parent, (2 * (size_t) n - 1) * sizeof(int));
    for (size_t r = 0; r < 4 * (size_t) (n - 1); r++) ni[r] = (double) w.ni[r];
    PF(ws_free)(&w);
    free(p);
    free(m);
}

/* Barnes-Hut over the Karras tree, left child first; f in original order
 * (pipeline.cl:332-383). */
static void PF(repulse_core)(const PF(pipe_ws) *w, real scaling, real theta2,
                             int adjust, real *f)
{
    const int n = w->n;
    const real *ps = w->psort, *ni = w->ni;
    for (int k = 0; k < n; k++) {
        const real xi = ps[4 * k], yi = ps[4 * k + 1];
        const real mi = ps[4 * k + 2], si = ps[4 * k + 3];
        real ax = (real) 0, ay = (real) 0;
        int stack[160];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int r = stack[--sp];
            int first, last;
            if (r >= n - 1) {
                first = last = r - (n - 1);
            } else {
                const real xd = xi - ni[4 * r], yd = yi - ni[4 * r + 1];
                const real d2 = xd * xd + yd * yd;
                if (d2 * theta2 > ni[4 * r + 3]) {
                    const real g = scaling * (mi * ni[4 * r + 2]) / d2;
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
            for (int j = first; j <= last; j++) {
                if (j == k) continue;
                const real xd = xi - ps[4 * j], yd = yi - ps[4 * j + 1];
                const real g = PF(rep)(xd * xd + yd * yd, mi * ps[4 * j + 2],
                                       si + ps[4 * j + 3], scaling, adjust);
                ax += xd * g;
                ay += yd * g;
            }
        }
        const uint32_t i = w->order[k];
        f[2 * i] = ax;
        f[2 * i + 1] = ay;
    }
}

/* Gravity and attraction over the symmetric CSR, added to f
 * (pipeline.cl:392-429). */
static void PF(attract_core)(int n, real gravity, int strong, int linlog,
                             int adjust, const real *p, const real *mass,
                             const real *size, const int *off,
                             const int *inc_node, const real *inc_coef,
                             real *f)
{
    for (int i = 0; i < n; i++) {
        const real xi = p[2 * i], yi = p[2 * i + 1];
        real ax = f[2 * i], ay = f[2 * i + 1];
        if (gravity != (real) 0) {
            const real dist = R_SQRT(xi * xi + yi * yi);
            if (dist > (real) 0) {
                const real g =
                    strong ? gravity * mass[i] : gravity * mass[i] / dist;
                ax -= xi * g;
                ay -= yi * g;
            }
        }
        const real si = adjust ? size[i] : (real) 0;
        for (int e = off[i]; e < off[i + 1]; e++) {
            const int j = inc_node[e];
            const real xd = xi - p[2 * j], yd = yi - p[2 * j + 1];
            real g = -inc_coef[e];
            if (adjust || linlog) {
                real dist = R_SQRT(xd * xd + yd * yd);
                if (adjust) dist -= si + size[j];
                if (!(dist > (real) 0)) continue;
                if (linlog) g *= R_LOG1P(dist) / dist;
            }
            ax += xd * g;
            ay += yd * g;
        }
        f[2 * i] = ax;
        f[2 * i + 1] = ay;
    }
}

/* Swinging of every node and the two totals over the nodes that can move
 * (pipeline.cl:438-474). fp64 = 0: block partials of S nodes and their sum
 * in `real`, blocking of src/gpu_full.c:193-198; fp64 = 1: double sums in
 * node order. */
static void PF(swing_core)(int n, const real *f, const real *fo,
                           const real *mass, const unsigned char *fixed,
                           real *sw, int fp64, double *tsw, double *ttr)
{
    if (fp64) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < n; i++) {
            const real sx = fo[2 * i] - f[2 * i];
            const real sy = fo[2 * i + 1] - f[2 * i + 1];
            const real tx = fo[2 * i] + f[2 * i];
            const real ty = fo[2 * i + 1] + f[2 * i + 1];
            const real s = mass[i] * R_SQRT(sx * sx + sy * sy);
            sw[i] = s;
            if (fixed && fixed[i]) continue;
            a += (double) s;
            b += (double) ((real) 0.5 * mass[i] * R_SQRT(tx * tx + ty * ty));
        }
        *tsw = a;
        *ttr = b;
        return;
    }
    int B = n / 256;
    if (B < 1) B = 1;
    if (B > 16384) B = 16384;
    const int Sz = (n + B - 1) / B;
    B = (n + Sz - 1) / Sz;
    real A = (real) 0, Bt = (real) 0;
    for (int b = 0; b < B; b++) {
        const int lo = b * Sz, hi = lo + Sz < n ? lo + Sz : n;
        real ps = (real) 0, pt = (real) 0;
        for (int i = lo; i < hi; i++) {
            const real sx = fo[2 * i] - f[2 * i];
            const real sy = fo[2 * i + 1] - f[2 * i + 1];
            const real tx = fo[2 * i] + f[2 * i];
            const real ty = fo[2 * i + 1] + f[2 * i + 1];
            const real s = mass[i] * R_SQRT(sx * sx + sy * sy);
            sw[i] = s;
            if (fixed && fixed[i]) continue;
            ps += s;
            pt += (real) 0.5 * mass[i] * R_SQRT(tx * tx + ty * ty);
        }
        A += ps;
        Bt += pt;
    }
    *tsw = (double) A;
    *ttr = (double) Bt;
}

/* Displacement; f_old takes f (pipeline.cl:480-506). */
static void PF(apply_core)(int n, real speed, int adjust,
                           const unsigned char *fixed, const real *f,
                           real *fo, const real *sw, real *p)
{
    for (int i = 0; i < n; i++) {
        const real fx = f[2 * i], fy = f[2 * i + 1];
        fo[2 * i] = fx;
        fo[2 * i + 1] = fy;
        if (fixed && fixed[i]) continue;
        real factor;
        if (adjust) {
            const real df = R_SQRT(fx * fx + fy * fy);
            factor = (real) 0.1 * speed / ((real) 1 + R_SQRT(speed * sw[i]));
            if (df > (real) 0) {
                if (factor * df > (real) 10) factor = (real) 10 / df;
            } else {
                factor = (real) 0;
            }
        } else {
            factor = speed / ((real) 1 + R_SQRT(speed * sw[i]));
        }
        p[2 * i] += fx * factor;
        p[2 * i + 1] += fy * factor;
    }
}

/* The graph of fa2_full_params in the device precision. */
typedef struct {
    real *p, *mass, *size, *coef;
    unsigned char *fixed;
} PF(pipe_graph);

static int PF(graph_load)(PF(pipe_graph) *g, const fa2_full_params *pp,
                          const double *pos)
{
    const int n = pp->n;
    const int ninc = pp->inc_off[n];
    memset(g, 0, sizeof(*g));
    g->p = (real *) malloc(2 * (size_t) n * sizeof(real));
    g->mass = (real *) malloc((size_t) n * sizeof(real));
    g->size = (real *) malloc((size_t) n * sizeof(real));
    g->coef = (real *) malloc((size_t) (ninc > 0 ? ninc : 1) * sizeof(real));
    if (!g->p || !g->mass || !g->size || !g->coef) return 0;
    for (int i = 0; i < n; i++) {
        g->p[2 * i] = (real) pos[i];
        g->p[2 * i + 1] = (real) pos[n + i];
        g->mass[i] = (real) pp->mass[i];
        g->size[i] = pp->adjust ? (real) pp->size[i] : (real) 0;
    }
    for (int e = 0; e < ninc; e++) g->coef[e] = (real) pp->inc_coef[e];
    if (pp->any_fixed) {
        g->fixed = (unsigned char *) malloc((size_t) n);
        if (!g->fixed) return 0;
        for (int i = 0; i < n; i++) g->fixed[i] = pp->fixed[i] != 0;
    }
    return 1;
}

static void PF(graph_free)(PF(pipe_graph) *g)
{
    free(g->p);
    free(g->mass);
    free(g->size);
    free(g->coef);
    free(g->fixed);
}

/* Repulsion then gravity and attraction at the current positions. */
static void PF(forces_core)(PF(pipe_ws) *w, const PF(pipe_graph) *g,
                            const fa2_full_params *pp, real *f)
{
    PF(build_core)(w, g->p, g->mass, g->size, pp->adjust);
    PF(repulse_core)(w, (real) pp->scaling, (real) (pp->theta * pp->theta),
                     pp->adjust, f);
    PF(attract_core)(pp->n, (real) pp->gravity, pp->strong, pp->linlog,
                     pp->adjust, g->p, g->mass, g->size, pp->inc_off,
                     pp->inc_node, g->coef, f);
}

int PF(orc_pipe_forces)(const fa2_full_params *pp, const double *pos,
                        double *fout)
{
    const int n = pp->n;
    if (n < 2) return 1;
    PF(pipe_ws) w;
    PF(pipe_graph) g;
    memset(&w, 0, sizeof(w));
    memset(&g, 0, sizeof(g));
    real *f = (real *) malloc(2 * (size_t) n * sizeof(real));
    int ok = f && PF(ws_alloc)(&w, n) && PF(graph_load)(&g, pp, pos);
    if (ok) {
        PF(forces_core)(&w, &g, pp, f);
        for (int i = 0; i < n; i++) {
            fout[i] = (double) f[2 * i];
            fout[n + i] = (double) f[2 * i + 1];
        }
    }
    PF(ws_free)(&w);
    PF(graph_free)(&g);
    free(f);
    return ok ? 0 : 1;
}

int PF(orc_pipe_run)(const fa2_full_params *pp, double *pos, int fp64)
{
    const int n = pp->n;
    if (n < 2) return 1;
    PF(pipe_ws) w;
    PF(pipe_graph) g;
    memset(&w, 0, sizeof(w));
    memset(&g, 0, sizeof(g));
    real *f = (real *) malloc(2 * (size_t) n * sizeof(real));
    real *fo = (real *) calloc(2 * (size_t) n, sizeof(real));
    real *sw = (real *) malloc((size_t) n * sizeof(real));
    int status = 1;
    if (!f || !fo || !sw || !PF(ws_alloc)(&w, n) ||
        !PF(graph_load)(&g, pp, pos))
        goto out;
    double speed = 1.0, eff = 1.0;
    for (int it = 0; it < pp->iterations; it++) {
        PF(forces_core)(&w, &g, pp, f);
        double tsw, ttr;
        PF(swing_core)(n, f, fo, g.mass, g.fixed, sw, fp64, &tsw, &ttr);
        if (!(tsw == tsw) || !(ttr == ttr)) {
            status = 2; /* "invalid numbers", src/gpu_full.c:486-491 */
            goto out;
        }
        orc_update_speed(n, tsw, ttr, pp->jitter_tolerance, &speed, &eff);
        PF(apply_core)(n, (real) speed, pp->adjust, g.fixed, f, fo, sw, g.p);
    }
    for (int i = 0; i < n; i++) {
        pos[i] = (double) g.p[2 * i];
        pos[n + i] = (double) g.p[2 * i + 1];
    }
    status = 0;
out:
    PF(ws_free)(&w);
    PF(graph_free)(&g);
    free(f);
    free(fo);
    free(sw);
    return status;
}

#undef PF
