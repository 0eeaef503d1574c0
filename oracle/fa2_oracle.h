/*
 * fa2_oracle.h -- ORACLE, test infrastructure only.
 *
 * CPU restatement of the ForceAtlas2 step of the forceatlas2r package. Only
 * tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
 * it, as the parity checker and as the timed CPU baseline ("port"). The
 * product (libfa2cuda.so) never links, loads or calls it.
 *
 * Part 1 (orc_*) restates the CPU engine of src/forceatlas2.c in double.
 * Part 2 (orc_pipe_*_f / _d) restates the all-GPU construction of
 * inst/opencl/pipeline.cl (Morton codes, stable radix order, Karras tree,
 * bottom-up centre of mass, Barnes-Hut traversal, attraction, swing, apply)
 * in float and in double.
 *
 * Positions cross this interface as in the package: x[0..n) then y[0..n)
 * (an R n x 2 matrix); forces likewise.
 */
#ifndef FA2_ORACLE_H
#define FA2_ORACLE_H

#include <stdint.h>
#include "../include/fa2.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Settings of one layout: dpar and flags of C_forceatlas2
 * (src/forceatlas2.c:491-506, 572-580). */
typedef struct {
    double scaling, gravity, jitter_tolerance, theta;
    int strong, linlog, outbound, adjust, barnes_hut;
    int threads;
} orc_opts;

/* ---- Part 1: src/forceatlas2.c ---------------------------------------- */

/* mass = 1 + degree, every edge end counted (src/forceatlas2.c:592-603). */
void orc_mass(int n, int m, const int *from, const int *to, double *mass,
              double *mean_mass);

/* Exact repulsion, ADDED to dx, dy (src/forceatlas2.c:265-294). size may be
 * NULL when adjust is 0. */
void orc_repulse_exact(int n, const double *x, const double *y,
                       const double *mass, const double *size, int adjust,
                       double scaling, int threads, double *dx, double *dy);

/* Gephi quadtree (src/forceatlas2.c:38-239). The caller allocates
 * t->reg (2n), t->perm (n), t->cnt (4n), t->buf[0..1] (n each),
 * t->px/py/pm (n) and t->ps (n, or NULL when size is NULL). */
void orc_tree_build(fa2_tree *t, int n, const double *x, const double *y,
                    const double *mass, const double *size);
/* The same with the regions of a level on `threads` OpenMP threads. */
void orc_tree_build_mt(fa2_tree *t, int n, const double *x, const double *y,
                       const double *mass, const double *size, int threads);

/* Barnes-Hut repulsion over that tree, ADDED to dx, dy
 * (src/forceatlas2.c:320-368). */
void orc_repulse_bh(int n, const fa2_tree *t, const double *x,
                    const double *y, const double *mass, const double *size,
                    int adjust, double scaling, double theta, int threads,
                    double *dx, double *dy);

/* Gravity, subtracted from dx, dy (src/forceatlas2.c:370-381). */
void orc_gravity(int n, const double *x, const double *y, const double *mass,
                 double gravity, int strong, double *dx, double *dy);

/* Attraction along the edges, edge by edge (src/forceatlas2.c:383-416). */
void orc_attract(int n, int m, const int *from, const int *to,
                 const double *w, const double *x, const double *y,
                 const double *mass, const double *size, double coef,
                 int linlog, int outbound, int adjust, double *dx, double *dy);

/* Gephi's adaptive speed (src/forceatlas2.c:443-485). */
void orc_update_speed(int n, double total_swinging, double total_traction,
                      double jitter_tolerance, double *speed,
                      double *speed_efficiency);

/* Forces of one iteration at the given positions: repulsion (exact or
 * Barnes-Hut), then gravity, then attraction, into fx, fy
 * (src/forceatlas2.c:683-756). */
int orc_forces(int n, int m, const int *from, const int *to, const double *w,
               const double *pos, const double *size, const orc_opts *o,
               double *f);

/* The iteration loop of C_forceatlas2 on the CPU, `threads` OpenMP threads
 * (src/forceatlas2.c:521-803). pos (x then y) is updated in place. Returns 0,
 * or 1 on invalid input. */
int orc_layout(int n, int m, const int *from, const int *to, const double *w,
               double *pos, const double *size, const int *fixed,
               int iterations, const orc_opts *o);

/* orc_layout that also records the positions before the first iteration
 * and after each one: trace holds (iterations + 1) * 2n doubles. */
int orc_layout_trace(int n, int m, const int *from, const int *to,
                     const double *w, double *pos, const double *size,
                     const int *fixed, int iterations, const orc_opts *o,
                     double *trace);

/* The symmetric CSR of C_forceatlas2_large with per-incidence coefficients
 * (src/forceatlas2.c:870-902). off has n+1 entries, inc_node and inc_coef
 * 2m. Returns the number of incidences. */
int orc_prepare_large(int n, int m, const int *from, const int *to,
                      const double *w, int outbound, double *mass, int *off,
                      int *inc_node, double *inc_coef);

/* ---- Part 2: inst/opencl/pipeline.cl, in float (_f) and double (_d) --- */

/* Stable order of the nodes by 32-bit key, LSD radix with 8-bit digits
 * (pipeline.cl:136-188): key and idx are sorted in place. */
void orc_pipe_sort(int n, uint32_t *key, uint32_t *idx);

/* Karras radix tree over sorted keys (pipeline.cl:209-270): child and range
 * have 2(n-1) entries, parent 2n-1. */
void orc_pipe_tree(int n, const uint32_t *key, int *child, int *range,
                   int *parent);

#define ORC_PIPE_DECLARE(real, S)                                             \
    /* bbox + Morton codes (pipeline.cl:61-130); pos is x then y. */          \
    void orc_pipe_morton_##S(int n, const double *pos, uint32_t *key,         \
                             uint32_t *idx, double *bbox);                    \
    /* Morton, order, tree, centre of mass and squared sizes of the regions  \
     * (pipeline.cl:195-323): keys and order n, child/range 2(n-1), parent    \
     * 2n-1, ni 4(n-1) as (cx, cy, m, size^2). */                            \
    void orc_pipe_build_##S(int n, const double *pos, const double *mass,     \
                            uint32_t *key, uint32_t *order, int *child,       \
                            int *range, int *parent, double *ni);             \
    /* Forces at the given positions: Barnes-Hut over the Karras tree, then  \
     * gravity and attraction (pipeline.cl:332-429). f is fx then fy. */      \
    int orc_pipe_forces_##S(const fa2_full_params *p, const double *pos,      \
                            double *f);                                       \
    /* fa2_full_run on the CPU (src/gpu_full.c:398-499). totals_fp64 = 0      \
     * sums swing and traction in `real` by blocks as the reference does;    \
     * 1 sums them in double in node order. */                                \
    int orc_pipe_run_##S(const fa2_full_params *p, double *pos,               \
                         int totals_fp64);

ORC_PIPE_DECLARE(float, f)
ORC_PIPE_DECLARE(double, d)

/* Forces of the FP32 path of libfa2cuda.so: tree of the double construction
 * over the float-rounded positions and masses, walk and attraction in float
 * (pipeline.cl:332-429). */
int orc_pipe_forces_m(const fa2_full_params *p, const double *pos,
                      double *f);

#ifdef __cplusplus
}
#endif

#endif
