/*
 * ref_pipeline.cpp -- ORACLE build only: compiles the package's own
 * inst/opencl/pipeline.cl (included from the reference checkout, never
 * copied) as C++ for the CPU, once in float and once in double, and drives
 * its kernels sequentially, one work item after the other, in the order and
 * with the blocking of src/gpu_full.c. The result pins the oracle's
 * restatement of the construction (Morton codes, stable order, Karras tree,
 * centres of mass) bit for bit.
 */
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" {
#include "fa2.h" /* the reference's, through -I<reference>/src */
}

/* What OpenCL C provides and C++ lacks. */
namespace clprelude {
typedef unsigned int uint;
typedef unsigned char uchar;
static size_t gid = 0;
static inline size_t get_global_id(int) { return gid; }
template <class T> static inline T min(T a, T b) { return b < a ? b : a; }
template <class T> static inline T max(T a, T b) { return a < b ? b : a; }
template <class T> static inline T clamp(T x, T lo, T hi)
{
    return min(max(x, lo), hi);
}
static inline int clz(uint v) { return v ? __builtin_clz(v) : 32; }
static inline int atomic_inc(volatile int *p)
{
    return __atomic_fetch_add((int *) p, 1, __ATOMIC_SEQ_CST);
}
using std::log1p;
using std::sqrt;
} // namespace clprelude

#define __kernel
#define __global

namespace cl_f {
using namespace clprelude;
#include "pipeline.cl"
} // namespace cl_f
#undef REAL
#undef FA2_LEAF_SIZE

#define FA2_DOUBLE
namespace cl_d {
using namespace clprelude;
#include "pipeline.cl"
} // namespace cl_d
#undef REAL
#undef FA2_LEAF_SIZE
#undef FA2_DOUBLE

/* One sequential sweep of a kernel over `count` work items. */
#define SWEEP(count, call)                                                    \
    for (size_t g_ = 0; g_ < (size_t) (count); g_++) {                        \
        clprelude::gid = g_;                                                  \
        call;                                                                 \
    }

template <class real, int DBL> struct Pipe {
    int n, B, S;
    std::vector<real> pos, mass, size, partial, bbox, psort, nd, ni, f, fold,
        sw, coef, total;
    std::vector<unsigned> keyA, idxA, keyB, idxB, hist, dtotal;
    std::vector<int> child, range, parent, visits;
    std::vector<unsigned char> fixed;

    explicit Pipe(int n_) : n(n_)
    {
        /* blocks of S nodes, src/gpu_full.c:193-198 */
        B = n / 256;
        if (B < 1) B = 1;
        if (B > 16384) B = 16384;
        S = (n + B - 1) / B;
        B = (n + S - 1) / S;
        pos.resize(2 * n);
        mass.resize(n);
        size.resize(n);
        partial.resize(4 * B);
        bbox.resize(4);
        psort.resize(4 * n);
        nd.resize(8 * (2 * n - 1));
        ni.resize(4 * (n - 1));
        f.resize(2 * n);
        fold.assign(2 * n, (real) 0);
        sw.resize(n);
        total.resize(2);
        keyA.resize(n);
        idxA.resize(n);
        keyB.resize(n);
        idxB.resize(n);
        hist.resize(256 * B);
        dtotal.resize(256);
        child.resize(2 * (n - 1));
        range.resize(2 * (n - 1));
        parent.resize(2 * n - 1);
        visits.resize(n - 1);
    }

    /* steps 1-4 of an iteration, src/gpu_full.c:413-443 */
    void build(int adjust)
    {
        if (DBL) {
            SWEEP(B, cl_d::bbox_partial(n, S, (const double *) pos.data(),
                                        (double *) partial.data()));
            SWEEP(1, cl_d::bbox_final(B, (const double *) partial.data(),
                                      (double *) bbox.data()));
            SWEEP(n, cl_d::morton(n, (const double *) pos.data(),
                                  (const double *) bbox.data(), keyA.data(),
                                  idxA.data()));
        } else {
            SWEEP(B, cl_f::bbox_partial(n, S, (const float *) pos.data(),
                                        (float *) partial.data()));
            SWEEP(1, cl_f::bbox_final(B, (const float *) partial.data(),
                                      (float *) bbox.data()));
            SWEEP(n, cl_f::morton(n, (const float *) pos.data(),
                                  (const float *) bbox.data(), keyA.data(),
                                  idxA.data()));
        }
        for (int pass = 0; pass < 4; pass++) {
            unsigned *kin = pass % 2 ? keyB.data() : keyA.data();
            unsigned *iin = pass % 2 ? idxB.data() : idxA.data();
            unsigned *kout = pass % 2 ? keyA.data() : keyB.data();
            unsigned *iout = pass % 2 ? idxA.data() : idxB.data();
            SWEEP(B, cl_f::sort_hist(n, S, B, 8 * pass, kin, hist.data()));
            SWEEP(256, cl_f::sort_scan(B, hist.data(), dtotal.data()));
            SWEEP(B, cl_f::sort_scatter(n, S, B, 8 * pass, kin, iin,
                                        hist.data(), dtotal.data(), kout,
                                        iout));
        }
        if (DBL) {
            SWEEP(n, cl_d::gather(n, adjust, idxA.data(),
                                  (const double *) pos.data(),
                                  (const double *) mass.data(),
                                  (const double *) size.data(),
                                  (double *) psort.data()));
            SWEEP(n - 1, cl_d::tree(n, keyA.data(), child.data(), range.data(),
                                    parent.data(), visits.data()));
            SWEEP(n, cl_d::aggregate(n, (const double *) psort.data(),
                                     child.data(), parent.data(), visits.data(),
                                     (double *) nd.data()));
            SWEEP(n - 1, cl_d::finalize(n, (const double *) nd.data(),
                                        (double *) ni.data()));
        } else {
            SWEEP(n, cl_f::gather(n, adjust, idxA.data(),
                                  (const float *) pos.data(),
                                  (const float *) mass.data(),
                                  (const float *) size.data(),
                                  (float *) psort.data()));
            SWEEP(n - 1, cl_f::tree(n, keyA.data(), child.data(), range.data(),
                                    parent.data(), visits.data()));
            SWEEP(n, cl_f::aggregate(n, (const float *) psort.data(),
                                     child.data(), parent.data(), visits.data(),
                                     (float *) nd.data()));
            SWEEP(n - 1, cl_f::finalize(n, (const float *) nd.data(),
                                        (float *) ni.data()));
        }
    }

    void load(const fa2_full_params *p, const double *xy)
    {
        for (int i = 0; i < n; i++) {
            pos[2 * i] = (real) xy[i];
            pos[2 * i + 1] = (real) xy[n + i];
            mass[i] = (real) p->mass[i];
            size[i] = p->adjust ? (real) p->size[i] : (real) 0;
        }
        const int ninc = p->inc_off[n];
        coef.resize(ninc > 0 ? ninc : 1);
        for (int e = 0; e < ninc; e++) coef[e] = (real) p->inc_coef[e];
        fixed.assign(n, 0);
        if (p->any_fixed)
            for (int i = 0; i < n; i++) fixed[i] = p->fixed[i] != 0;
    }

    /* steps 5-6: repulsion, then gravity and attraction */
    void forces(const fa2_full_params *p)
    {
        const real sc = (real) p->scaling, t2 = (real) (p->theta * p->theta);
        const real gr = (real) p->gravity;
        if (DBL) {
            SWEEP(n, cl_d::repulse(n, sc, t2, p->adjust,
                                   (const double *) psort.data(),
                                   (const double *) ni.data(), child.data(),
                                   range.data(), idxA.data(),
                                   (double *) f.data()));
            SWEEP(n, cl_d::attract(n, gr, p->strong, p->linlog, p->adjust,
                                   (const double *) pos.data(),
                                   (const double *) mass.data(),
                                   (const double *) size.data(), p->inc_off,
                                   p->inc_node, (const double *) coef.data(),
                                   (double *) f.data()));
        } else {
            SWEEP(n, cl_f::repulse(n, sc, t2, p->adjust,
                                   (const float *) psort.data(),
                                   (const float *) ni.data(), child.data(),
                                   range.data(), idxA.data(),
                                   (float *) f.data()));
            SWEEP(n, cl_f::attract(n, gr, p->strong, p->linlog, p->adjust,
                                   (const float *) pos.data(),
                                   (const float *) mass.data(),
                                   (const float *) size.data(), p->inc_off,
                                   p->inc_node, (const float *) coef.data(),
                                   (float *) f.data()));
        }
    }

    /* steps 7-8 with the host speed update, src/gpu_full.c:464-497 */
    int move(const fa2_full_params *p, double *speed, double *eff)
    {
        if (DBL) {
            SWEEP(B, cl_d::swing(n, S, p->any_fixed, (const double *) f.data(),
                                 (const double *) fold.data(),
                                 (const double *) mass.data(), fixed.data(),
                                 (double *) sw.data(),
                                 (double *) partial.data()));
            SWEEP(1, cl_d::sum2(B, (const double *) partial.data(),
                                (double *) total.data()));
        } else {
            SWEEP(B, cl_f::swing(n, S, p->any_fixed, (const float *) f.data(),
                                 (const float *) fold.data(),
                                 (const float *) mass.data(), fixed.data(),
                                 (float *) sw.data(),
                                 (float *) partial.data()));
            SWEEP(1, cl_f::sum2(B, (const float *) partial.data(),
                                (float *) total.data()));
        }
        const double tsw = (double) total[0], ttr = (double) total[1];
        if (!(tsw == tsw) || !(ttr == ttr)) return 1;
        fa2_update_speed(n, tsw, ttr, p->jitter_tolerance, speed, eff);
        if (DBL) {
            SWEEP(n, cl_d::apply(n, (double) *speed, p->adjust, p->any_fixed,
                                 (const double *) f.data(),
                                 (double *) fold.data(),
                                 (const double *) sw.data(), fixed.data(),
                                 (double *) pos.data()));
        } else {
            SWEEP(n, cl_f::apply(n, (float) *speed, p->adjust, p->any_fixed,
                                 (const float *) f.data(), (float *) fold.data(),
                                 (const float *) sw.data(), fixed.data(),
                                 (float *) pos.data()));
        }
        return 0;
    }
};

template <class real, int DBL>
static void build_out(int n, const double *xy, const double *mass,
                      uint32_t *key, uint32_t *order, int *child, int *range,
                      int *parent, double *ni)
{
    Pipe<real, DBL> P(n);
    for (int i = 0; i < n; i++) {
        P.pos[2 * i] = (real) xy[i];
        P.pos[2 * i + 1] = (real) xy[n + i];
        P.mass[i] = (real) mass[i];
        P.size[i] = (real) 0;
    }
    P.build(0);
    memcpy(key, P.keyA.data(), (size_t) n * 4);
    memcpy(order, P.idxA.data(), (size_t) n * 4);
    memcpy(child, P.child.data(), 2 * (size_t) (n - 1) * sizeof(int));
    memcpy(range, P.range.data(), 2 * (size_t) (n - 1) * sizeof(int));
    memcpy(parent, P.parent.data(), (2 * (size_t) n - 1) * sizeof(int));
    for (size_t r = 0; r < 4 * (size_t) (n - 1); r++) ni[r] = (double) P.ni[r];
}

template <class real, int DBL>
static int forces_out(const fa2_full_params *p, const double *xy, double *fo)
{
    const int n = p->n;
    Pipe<real, DBL> P(n);
    P.load(p, xy);
    P.build(p->adjust);
    P.forces(p);
    for (int i = 0; i < n; i++) {
        fo[i] = (double) P.f[2 * i];
        fo[n + i] = (double) P.f[2 * i + 1];
    }
    return 0;
}

template <class real, int DBL>
static int run_out(const fa2_full_params *p, double *xy)
{
    const int n = p->n;
    Pipe<real, DBL> P(n);
    P.load(p, xy);
    double speed = 1.0, eff = 1.0;
    for (int it = 0; it < p->iterations; it++) {
        P.build(p->adjust);
        P.forces(p);
        if (P.move(p, &speed, &eff)) return 2;
    }
    for (int i = 0; i < n; i++) {
        xy[i] = (double) P.pos[2 * i];
        xy[n + i] = (double) P.pos[2 * i + 1];
    }
    return 0;
}

extern "C" {
void ref_pipe_build_f(int n, const double *xy, const double *mass,
                      uint32_t *key, uint32_t *order, int *child, int *range,
                      int *parent, double *ni)
{
    build_out<float, 0>(n, xy, mass, key, order, child, range, parent, ni);
}
void ref_pipe_build_d(int n, const double *xy, const double *mass,
                      uint32_t *key, uint32_t *order, int *child, int *range,
                      int *parent, double *ni)
{
    build_out<double, 1>(n, xy, mass, key, order, child, range, parent, ni);
}
int ref_pipe_forces_f(const fa2_full_params *p, const double *xy, double *f)
{
    return forces_out<float, 0>(p, xy, f);
}
int ref_pipe_forces_d(const fa2_full_params *p, const double *xy, double *f)
{
    return forces_out<double, 1>(p, xy, f);
}
int ref_pipe_run_f(const fa2_full_params *p, double *xy)
{
    return run_out<float, 0>(p, xy);
}
int ref_pipe_run_d(const fa2_full_params *p, double *xy)
{
    return run_out<double, 1>(p, xy);
}
}
