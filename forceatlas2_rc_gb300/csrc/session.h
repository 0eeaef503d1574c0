// session.h -- the two kinds of device session behind the C interface:
//   Layout   a layout kept on the device between calls (fa2_full_run and
//            the fa2cu_layout_* entry points);
//   Repulse  the repulsion backend of fa2_gpu_open / fa2_gpu_repulse_*.
// Each has a float and a double implementation (inst_f32.cu, inst_f64.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fa2.h"

namespace fa2cu {

struct LayoutBase {
    virtual ~LayoutBase() {}
    virtual int iterate(int iterations) = 0;
    virtual int sync() = 0;
    virtual int positions(double *pos) = 0;
    virtual int set_positions(const double *pos) = 0;
    virtual int forces(const double *pos, double *f) = 0;
    virtual int speed(double state[4]) = 0;
    virtual cudaStream_t stream() = 0;
    virtual int phase_times(int iterations, double *ms) = 0;
    virtual int tree(const double *pos, uint32_t *key, uint32_t *order, int *child,
                     int *range, int *parent, double *ni) = 0;
    virtual int traversal_counts(double counts[2]) = 0;
    virtual int option(const char *name, double value) = 0;
    virtual int swing(double *sw, double *tr) = 0;
    virtual double info(const char *name) = 0;
    virtual double bytes() const = 0;
    int device = 0;
};

// How a layout gets its stream and memory: by default its own stream and
// cudaMalloc; a server passes a memory pool (stream-ordered allocation) and a
// stream priority.
struct LayoutOpts {
    cudaMemPool_t pool = nullptr;
    bool has_priority = false;
    int priority = 0;
};

// A graph given as its edge list (0-based ends, weights): the layout then
// prepares masses and incidence lists on the device, and p's inc_off,
// inc_node, inc_coef and mass are not read.
struct EdgeList {
    int m = 0;
    const int *from = nullptr, *to = nullptr;
    const double *w = nullptr;
    int outbound = 0;
};

// NULL on failure (message set). `pos` is x then y.
LayoutBase *make_layout_f32(const fa2_full_params *p, const double *pos, int repulsion,
                            const LayoutOpts *opts = nullptr, const EdgeList *edges = nullptr);
LayoutBase *make_layout_f64(const fa2_full_params *p, const double *pos, int repulsion,
                            const LayoutOpts *opts = nullptr, const EdgeList *edges = nullptr);
// Device bytes of a layout of n nodes and ninc incidences, staging included,
// on a device of `sms` SMs.
double layout_footprint_f32(int n, int ninc, int adjust, int any_fixed, int repulsion, int sms);
double layout_footprint_f64(int n, int ninc, int adjust, int any_fixed, int repulsion, int sms);

struct RepulseBase {
    virtual ~RepulseBase() {}
    virtual int exact(const double *x, const double *y, const double *mass,
                      const double *size, double scaling, double *dx, double *dy) = 0;
    virtual int bh(const fa2_tree *t, double scaling, double theta, double *dx,
                   double *dy) = 0;
    double t_send = 0.0, t_compute = 0.0, t_fetch = 0.0;
    int device = 0;
};

RepulseBase *make_repulse_f32(int device, int n, int adjust, int barnes_hut);
RepulseBase *make_repulse_f64(int device, int n, int adjust, int barnes_hut);

struct BatchBase {
    virtual ~BatchBase() {}
    virtual int iterate(int iterations) = 0;
    virtual int sync() = 0;
    virtual int positions(int g, double *pos) = 0;
    virtual int forces(int g, double *f) = 0;
    virtual int speed(int g, double state[4]) = 0;
    virtual cudaStream_t stream() = 0;
    virtual double bytes() const = 0;
    virtual int count() const = 0;
    virtual int phase_cycles(int iterations, double out[8]) = 0;
    int device = 0;
};

// NULL on failure (message set). exact_below: graphs of fewer nodes use the
// exact repulsion; threads: block size (256 or 512); npt: nodes per thread
// of the exact sum (1 or 2).
BatchBase *make_batch_f32(const fa2_full_params *ps, int count, const double *const *pos,
                          int exact_below, int threads, int npt);
BatchBase *make_batch_f64(const fa2_full_params *ps, int count, const double *const *pos,
                          int exact_below, int threads, int npt);
// Crossover, block size and tile shape measured on this device (0 on
// success).
int tune_batch_f32(int device, int *exact_below, int *threads, int *npt);
int tune_batch_f64(int device, int *exact_below, int *threads, int *npt);

// Host-side checks of caller data that the kernels index with: 0 if valid,
// otherwise 1 with the message set.
int check_csr(int n, const int *inc_off, const int *inc_node);
int check_quadtree(int n, const fa2_tree *t);

} // namespace fa2cu
