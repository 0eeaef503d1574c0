/*
 * ref_harness.c -- ORACLE build only: compiles the package's own
 * src/forceatlas2.c (included from the reference checkout, never copied)
 * against a minimal stand-in for R's C API, and exposes
 *   - the static force functions of that file, for per-step forces;
 *   - C_forceatlas2 and C_forceatlas2_large, through stand-in SEXPs.
 * The result, oracle/_ref/libfa2ref.so, pins the oracle restatement
 * (fa2_oracle.c) and produces the golden fixtures under tests/golden/.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "forceatlas2.c" /* resolved through -I<reference>/src */

/* ------------------------------------------------------------------------ */
/* A stand-in R runtime: vectors in malloc'ed memory, freed after each call */
/* ------------------------------------------------------------------------ */

struct rstub_sexp {
    int type;
    R_xlen_t len;
    void *data;
    SEXP timings; /* the only attribute read back */
};

static void **arena = NULL;
static size_t arena_len = 0, arena_cap = 0;
static jmp_buf on_error;
static char error_message[1024];

static void *arena_alloc(size_t bytes)
{
    void *p = calloc(1, bytes ? bytes : 1);
    if (!p) abort();
    if (arena_len == arena_cap) {
        arena_cap = arena_cap ? 2 * arena_cap : 256;
        arena = (void **) realloc(arena, arena_cap * sizeof(void *));
        if (!arena) abort();
    }
    arena[arena_len++] = p;
    return p;
}

static void arena_release(void)
{
    for (size_t i = 0; i < arena_len; i++) free(arena[i]);
    arena_len = 0;
}

static size_t elt_size(int type)
{
    switch (type) {
    case REALSXP: return sizeof(double);
    case INTSXP:
    case LGLSXP: return sizeof(int);
    case STRSXP:
    case VECSXP: return sizeof(SEXP);
    default: return 1;
    }
}

SEXP Rf_allocVector(int type, R_xlen_t n)
{
    SEXP s = (SEXP) arena_alloc(sizeof(*s));
    s->type = type;
    s->len = n;
    s->data = arena_alloc((size_t) n * elt_size(type));
    return s;
}

SEXP Rf_duplicate(SEXP x)
{
    SEXP s = Rf_allocVector(x->type, x->len);
    memcpy(s->data, x->data, (size_t) x->len * elt_size(x->type));
    return s;
}

static struct rstub_sexp names_symbol = {SYMSXP, 0, NULL, NULL};
SEXP R_NamesSymbol = &names_symbol;
static struct rstub_sexp timings_symbol = {SYMSXP, 0, NULL, NULL};

SEXP Rf_install(const char *name)
{
    return strcmp(name, "timings") == 0 ? &timings_symbol : &names_symbol;
}

SEXP Rf_mkChar(const char *s)
{
    SEXP c = (SEXP) arena_alloc(sizeof(*c));
    c->type = CHARSXP;
    c->len = (R_xlen_t) strlen(s);
    c->data = arena_alloc(strlen(s) + 1);
    memcpy(c->data, s, strlen(s) + 1);
    return c;
}

SEXP Rf_mkNamed(int type, const char **names)
{
    R_xlen_t k = 0;
    while (names[k][0]) k++;
    return Rf_allocVector(type, k);
}

SEXP Rf_ScalarLogical(int v)
{
    SEXP s = Rf_allocVector(LGLSXP, 1);
    ((int *) s->data)[0] = v;
    return s;
}

SEXP Rf_setAttrib(SEXP x, SEXP name, SEXP value)
{
    if (name == &timings_symbol) x->timings = value;
    return value;
}

int Rf_asInteger(SEXP x)
{
    if (x->len < 1) return NA_INTEGER;
    if (x->type == INTSXP || x->type == LGLSXP) return ((int *) x->data)[0];
    if (x->type == REALSXP) return (int) ((double *) x->data)[0];
    return NA_INTEGER;
}

Rboolean Rf_isInteger(SEXP x) { return x->type == INTSXP ? TRUE : FALSE; }
Rboolean Rf_isReal(SEXP x) { return x->type == REALSXP ? TRUE : FALSE; }
Rboolean Rf_isLogical(SEXP x) { return x->type == LGLSXP ? TRUE : FALSE; }
Rboolean Rf_isString(SEXP x) { return x->type == STRSXP ? TRUE : FALSE; }

void Rf_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(error_message, sizeof(error_message), fmt, ap);
    va_end(ap);
    longjmp(on_error, 1);
}

int LENGTH(SEXP x) { return (int) x->len; }
R_xlen_t XLENGTH(SEXP x) { return x->len; }
int *INTEGER(SEXP x) { return (int *) x->data; }
int *LOGICAL(SEXP x) { return (int *) x->data; }
double *REAL(SEXP x) { return (double *) x->data; }
const char *R_CHAR(SEXP x) { return (const char *) x->data; }
SEXP STRING_ELT(SEXP x, R_xlen_t i) { return ((SEXP *) x->data)[i]; }
void SET_STRING_ELT(SEXP x, R_xlen_t i, SEXP v) { ((SEXP *) x->data)[i] = v; }
SEXP SET_VECTOR_ELT(SEXP x, R_xlen_t i, SEXP v)
{
    ((SEXP *) x->data)[i] = v;
    return v;
}
SEXP Rf_protect(SEXP x) { return x; }
void Rf_unprotect(int n) { (void) n; }
char *R_alloc(size_t n, int size) { return (char *) arena_alloc(n * size); }
void R_CheckUserInterrupt(void) {}
Rboolean R_ToplevelExec(void (*fun)(void *), void *data)
{
    fun(data);
    return TRUE;
}
int R_registerRoutines(DllInfo *info, const void *c, const R_CallMethodDef *call,
                       const void *fortran, const void *external)
{
    (void) info, (void) c, (void) call, (void) fortran, (void) external;
    return 1;
}
Rboolean R_useDynamicSymbols(DllInfo *info, Rboolean value)
{
    (void) info, (void) value;
    return TRUE;
}
Rboolean R_forceSymbols(DllInfo *info, Rboolean value)
{
    (void) info, (void) value;
    return TRUE;
}

/* ------------------------------------------------------------------------ */
/* Exported wrappers                                                        */
/* ------------------------------------------------------------------------ */

const char *ref_error(void) { return error_message; }

static SEXP int_vec(int n, const int *v)
{
    SEXP s = Rf_allocVector(INTSXP, n);
    if (n) memcpy(s->data, v, (size_t) n * sizeof(int));
    return s;
}

static SEXP lgl_vec(int n, const int *v)
{
    SEXP s = Rf_allocVector(LGLSXP, n);
    if (n) memcpy(s->data, v, (size_t) n * sizeof(int));
    return s;
}

static SEXP real_vec(R_xlen_t n, const double *v)
{
    SEXP s = Rf_allocVector(REALSXP, n);
    if (n) memcpy(s->data, v, (size_t) n * sizeof(double));
    return s;
}

/* C_forceatlas2 with gpu = c(-1, 0): the CPU engine. pos is x then y;
 * out receives the layout, timings (7 values) the timings attribute. */
int ref_C_forceatlas2(int n, int m, const int *from, const int *to,
                      const double *w, const double *pos, const double *size,
                      const int *fixed, int iterations, const double *dpar,
                      const int *flags5, int threads, double *out,
                      double *timings)
{
    int status = 1;
    if (setjmp(on_error) == 0) {
        const int gpu[2] = {-1, 0};
        SEXP ans = C_forceatlas2(
            int_vec(1, &n), int_vec(m, from), int_vec(m, to), real_vec(m, w),
            real_vec(2 * (R_xlen_t) n, pos), real_vec(n, size),
            lgl_vec(n, fixed), int_vec(1, &iterations), real_vec(4, dpar),
            lgl_vec(5, flags5), int_vec(1, &threads), int_vec(2, gpu));
        memcpy(out, ans->data, 2 * (size_t) n * sizeof(double));
        if (timings && ans->timings)
            memcpy(timings, ans->timings->data, 7 * sizeof(double));
        error_message[0] = 0;
        status = 0;
    }
    arena_release();
    return status;
}

/* C_forceatlas2_large: runs fa2_full_run of whichever library this harness
 * was linked with. Returns 0, or 1 with ref_error() set. */
int ref_C_forceatlas2_large(int n, int m, const int *from, const int *to,
                            const double *w, const double *pos,
                            const double *size, const int *fixed,
                            int iterations, const double *dpar,
                            const int *flags4, const int *gpu3, double *out)
{
    int status = 1;
    if (setjmp(on_error) == 0) {
        SEXP src = Rf_allocVector(STRSXP, 1);
        SET_STRING_ELT(src, 0, Rf_mkChar(""));
        SEXP ans = C_forceatlas2_large(
            int_vec(1, &n), int_vec(m, from), int_vec(m, to), real_vec(m, w),
            real_vec(2 * (R_xlen_t) n, pos), real_vec(n, size),
            lgl_vec(n, fixed), int_vec(1, &iterations), real_vec(4, dpar),
            lgl_vec(4, flags4), int_vec(3, gpu3), src);
        memcpy(out, ans->data, 2 * (size_t) n * sizeof(double));
        error_message[0] = 0;
        status = 0;
    }
    arena_release();
    return status;
}

/* Forces of one iteration with the reference's own static functions, in the
 * order of C_forceatlas2: repulsion, gravity, attraction. pos and f are
 * x then y. dpar = (scaling, gravity, jitter, theta); flags5 = (strong,
 * linlog, outbound, adjust, barnes_hut). */
int ref_forces(int n, int m, const int *from, const int *to, const double *w,
               const double *pos, const double *size, const double *dpar,
               const int *flags5, double *f)
{
    fa2_state s;
    memset(&s, 0, sizeof(s));
    double *mass = (double *) malloc((size_t) n * sizeof(double));
    double *xy = (double *) malloc(2 * (size_t) n * sizeof(double));
    if (!mass || !xy) return 1;
    memcpy(xy, pos, 2 * (size_t) n * sizeof(double));
    double mean = 0.0;
    for (int i = 0; i < n; i++) mass[i] = 1.0;
    for (int e = 0; e < m; e++) {
        mass[from[e]] += 1.0;
        mass[to[e]] += 1.0;
    }
    for (int i = 0; i < n; i++) mean += mass[i];
    mean /= n;
    s.n = n;
    s.m = m;
    s.x = xy;
    s.y = xy + n;
    s.dx = f;
    s.dy = f + n;
    s.mass = mass;
    s.size = size;
    s.from = from;
    s.to = to;
    s.w = w;
    s.scaling = dpar[0];
    s.gravity = dpar[1];
    s.theta = dpar[3];
    s.strong = flags5[0];
    s.linlog = flags5[1];
    s.outbound = flags5[2];
    s.adjust = flags5[3];
    memset(f, 0, 2 * (size_t) n * sizeof(double));
    if (flags5[4]) {
        fa2_tree t;
        memset(&t, 0, sizeof(t));
        t.reg = (fa2_region *) malloc(2 * (size_t) n * sizeof(fa2_region));
        t.perm = (int *) malloc((size_t) n * sizeof(int));
        t.cnt = (int *) malloc(4 * (size_t) n * sizeof(int));
        t.buf[0] = (fa2_node *) malloc((size_t) n * sizeof(fa2_node));
        t.buf[1] = (fa2_node *) malloc((size_t) n * sizeof(fa2_node));
        t.px = (double *) malloc((size_t) n * sizeof(double));
        t.py = (double *) malloc((size_t) n * sizeof(double));
        t.pm = (double *) malloc((size_t) n * sizeof(double));
        t.ps = s.adjust ? (double *) malloc((size_t) n * sizeof(double)) : NULL;
        int *stack = (int *) malloc(2 * (size_t) n * sizeof(int));
        tree_build(&t, n, s.x, s.y, mass, s.adjust ? s.size : NULL, 1);
        for (int k = 0; k < n; k++) repulse_node_bh(&s, &t, t.perm[k], stack);
        free(stack);
        free(t.reg);
        free(t.perm);
        free(t.cnt);
        free(t.buf[0]);
        free(t.buf[1]);
        free(t.px);
        free(t.py);
        free(t.pm);
        free(t.ps);
    } else {
        for (int i = 0; i < n; i++) repulse_node_exact(&s, i);
    }
    if (s.gravity != 0)
        for (int i = 0; i < n; i++) gravity_node(&s, i);
    attract_all(&s, s.outbound ? mean : 1.0);
    free(mass);
    free(xy);
    return 0;
}

/* The reference's quadtree: regions as 10 numbers each (mass, cx, cy, size,
 * start, count, child, nchild, skip, buf), perm and px/py/pm. Returns nreg. */
int ref_tree(int n, const double *pos, const double *mass, double *regs,
             int *perm, double *pxyz)
{
    fa2_tree t;
    memset(&t, 0, sizeof(t));
    t.reg = (fa2_region *) malloc(2 * (size_t) n * sizeof(fa2_region));
    t.perm = perm;
    t.cnt = (int *) malloc(4 * (size_t) n * sizeof(int));
    t.buf[0] = (fa2_node *) malloc((size_t) n * sizeof(fa2_node));
    t.buf[1] = (fa2_node *) malloc((size_t) n * sizeof(fa2_node));
    t.px = pxyz;
    t.py = pxyz + n;
    t.pm = pxyz + 2 * (size_t) n;
    t.ps = NULL;
    tree_build(&t, n, pos, pos + n, mass, NULL, 1);
    for (int r = 0; r < t.nreg; r++) {
        const fa2_region *g = &t.reg[r];
        double *o = regs + 10 * (size_t) r;
        o[0] = g->mass;
        o[1] = g->cx;
        o[2] = g->cy;
        o[3] = g->size;
        o[4] = g->start;
        o[5] = g->count;
        o[6] = g->child;
        o[7] = g->nchild;
        o[8] = g->skip;
        o[9] = g->buf;
    }
    const int nreg = t.nreg;
    free(t.reg);
    free(t.cnt);
    free(t.buf[0]);
    free(t.buf[1]);
    return nreg;
}

void ref_update_speed(int n, double sw, double tr, double jt, double *speed,
                      double *eff)
{
    fa2_update_speed(n, sw, tr, jt, speed, eff);
}
