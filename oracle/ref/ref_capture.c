/* ref_capture.c -- ORACLE test infrastructure. A stand-in backend for the
 * package's .Call layer (src/forceatlas2.c) that records what
 * C_forceatlas2_large (src/forceatlas2.c:835-947) hands to fa2_full_run --
 * the masses and the symmetric incidence lists it prepared on the host --
 * instead of running a layout. Linked with ref_harness.o it lets the golden
 * fixtures pin the graph preparation on the reference's own code. Every
 * other backend entry point reports that there is no device. */
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fa2.h"

static int cap_n = 0, cap_ninc = 0;
static double *cap_mass = NULL, *cap_coef = NULL;
static int *cap_off = NULL, *cap_node = NULL;

int fa2_full_run(const fa2_full_params *p, double *pos, double *times)
{
    (void) pos;
    for (int k = 0; k < FA2_FULL_NTIMES; k++) times[k] = 0.0;
    free(cap_mass);
    free(cap_coef);
    free(cap_off);
    free(cap_node);
    cap_n = p->n;
    cap_ninc = p->inc_off[p->n];
    const size_t ni = cap_ninc > 0 ? (size_t) cap_ninc : 1;
    cap_mass = malloc((size_t) cap_n * sizeof(double));
    cap_off = malloc(((size_t) cap_n + 1) * sizeof(int));
    cap_node = malloc(ni * sizeof(int));
    cap_coef = malloc(ni * sizeof(double));
    if (!cap_mass || !cap_off || !cap_node || !cap_coef) return 1;
    memcpy(cap_mass, p->mass, (size_t) cap_n * sizeof(double));
    memcpy(cap_off, p->inc_off, ((size_t) cap_n + 1) * sizeof(int));
    if (cap_ninc > 0) {
        memcpy(cap_node, p->inc_node, (size_t) cap_ninc * sizeof(int));
        memcpy(cap_coef, p->inc_coef, (size_t) cap_ninc * sizeof(double));
    }
    return 0;
}

/* The last capture: sizes, then the arrays into caller buffers (each may be
 * NULL). */
int capture_get(int *n, int *ninc, double *mass, int *off, int *node, double *coef)
{
    *n = cap_n;
    *ninc = cap_ninc;
    if (mass && cap_mass) memcpy(mass, cap_mass, (size_t) cap_n * sizeof(double));
    if (off && cap_off) memcpy(off, cap_off, ((size_t) cap_n + 1) * sizeof(int));
    if (node && cap_node && cap_ninc > 0) memcpy(node, cap_node, (size_t) cap_ninc * sizeof(int));
    if (coef && cap_coef && cap_ninc > 0)
        memcpy(coef, cap_coef, (size_t) cap_ninc * sizeof(double));
    return 0;
}

const char *fa2_gpu_error(void) { return "the capture harness has no device"; }
int fa2_gpu_ndevices(void) { return 0; }
int fa2_gpu_device_info(int idx, fa2_gpu_devinfo *info)
{
    (void) idx;
    (void) info;
    return 1;
}
fa2_gpu *fa2_gpu_open(int device, int use_double, int n, int adjust, int barnes_hut,
                      int threads)
{
    (void) device;
    (void) use_double;
    (void) n;
    (void) adjust;
    (void) barnes_hut;
    (void) threads;
    return NULL;
}
void fa2_gpu_times(const fa2_gpu *g, double times[3])
{
    (void) g;
    times[0] = times[1] = times[2] = 0.0;
}
void fa2_gpu_close(fa2_gpu *g) { (void) g; }
int fa2_gpu_repulse_exact(fa2_gpu *g, const double *x, const double *y, const double *mass,
                          const double *size, double scaling, double *dx, double *dy)
{
    (void) g, (void) x, (void) y, (void) mass, (void) size, (void) scaling, (void) dx, (void) dy;
    return 1;
}
int fa2_gpu_repulse_bh(fa2_gpu *g, const fa2_tree *t, double scaling, double theta, double *dx,
                       double *dy)
{
    (void) g, (void) t, (void) scaling, (void) theta, (void) dx, (void) dy;
    return 1;
}
void fa2_gpu_shutdown(void) {}
double fa2_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}
