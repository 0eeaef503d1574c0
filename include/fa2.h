/*
 * fa2.h -- the C interface that the forceatlas2r package's .Call layer
 * (src/forceatlas2.c) links against, implemented here by libfa2cuda.so on
 * CUDA (sm_103a) instead of OpenCL.
 *
 * Every type and function below keeps the layout, signature and calling
 * convention of the reference interface (src/fa2.h:21-137), so that the
 * package's C code compiles and links against this library unchanged. The
 * reference file each entry point replaces is cited beside it.
 *
 * Conventions (unchanged from the reference):
 *   - functions return 0 on success (a NULL session for fa2_gpu_open) and a
 *     non-zero value on failure; the message is then read with
 *     fa2_gpu_error().  Nothing here longjmps, calls exit() or prints.
 *   - every pointer passed in belongs to the caller; host arrays are plain
 *     double / int arrays in the caller's memory.
 *   - the library is not thread safe: the reference calls it from R's main
 *     thread only.
 */
#ifndef FA2_H
#define FA2_H

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Barnes-Hut quadtree of the CPU engine (src/fa2.h:8-44). A region covers the
 * nodes perm[start .. start+count-1]; its children are the regions
 * child .. child+nchild-1.  `skip` is the next region of a depth-first walk
 * that is not a descendant: the previous sibling, else the parent's skip,
 * -1 at the end.  `size` is twice the largest distance between the centre
 * of mass and one of the region's nodes.
 */
typedef struct {
    double mass, cx, cy, size;
    int start, count;
    int child, nchild;
    int skip;
    int buf;
} fa2_region;

typedef struct {
    double x, y, m;
    int idx;
} fa2_node;

typedef struct {
    fa2_region *reg;
    int nreg;
    int *perm;
    int *cnt;
    fa2_node *buf[2];
    /* positions, masses and radii in the order of perm (radii may be NULL) */
    double *px, *py, *pm, *ps;
} fa2_tree;

/* Device description returned by fa2_gpu_device_info (src/fa2.h:50-58). */
typedef struct {
    char name[128];
    char vendor[128];
    char platform[128];
    char version[128];
    int is_gpu;
    int has_double;
    double memory; /* bytes */
} fa2_gpu_devinfo;

typedef struct fa2_gpu fa2_gpu;

/* Message of the last failure (src/gpu.c:129-131). */
const char *fa2_gpu_error(void);

/* Number of CUDA devices, 0 without a driver (src/gpu.c:156-187). */
int fa2_gpu_ndevices(void);

/* Description of device idx, 0-based; 0 on success (src/gpu.c:189-228). */
int fa2_gpu_device_info(int idx, fa2_gpu_devinfo *info);

/* Repulsion session for a layout of n nodes on device `device`
 * (src/gpu.c:393-475).  1 <= n <= 2^27.  `threads` sizes the host-side
 * conversion loops. */
fa2_gpu *fa2_gpu_open(int device, int use_double, int n, int adjust,
                      int barnes_hut, int threads);

/* Seconds spent since open: sending, computing, fetching (src/gpu.c:386). */
void fa2_gpu_times(const fa2_gpu *g, double times[3]);

/* Release a session; NULL is a no-op (src/gpu.c:368-384). */
void fa2_gpu_close(fa2_gpu *g);

/* Exact repulsion between every pair of nodes, ADDED to dx, dy
 * (src/gpu.c:582-637).  size may be NULL when radii are not used. */
int fa2_gpu_repulse_exact(fa2_gpu *g, const double *x, const double *y,
                          const double *mass, const double *size,
                          double scaling, double *dx, double *dy);

/* Barnes-Hut repulsion over a quadtree built on the host, ADDED to dx, dy in
 * the original node order through t->perm (src/gpu.c:639-704). */
int fa2_gpu_repulse_bh(fa2_gpu *g, const fa2_tree *t, double scaling,
                       double theta, double *dx, double *dy);

/* Release everything cached between calls (src/gpu.c:261-267). */
void fa2_gpu_shutdown(void);

/* Monotonic clock in seconds (src/ocl_loader.c:60-65). */
double fa2_now(void);

/* Parameters of the all-GPU layout (src/fa2.h:97-115).  Node i's edges are
 * inc_off[i] .. inc_off[i+1]-1 of inc_node (the other end) and inc_coef (the
 * attraction strength, outbound division already folded in). */
typedef struct {
    int n;
    const int *inc_off, *inc_node;
    const double *inc_coef;
    const double *mass;
    const double *size;
    const int *fixed;
    int any_fixed;
    double scaling, gravity, theta, jitter_tolerance;
    int strong, linlog, adjust;
    int iterations;
    int device, use_double;
    int profile;
    const char *source; /* accepted and ignored: the kernels are compiled in */
    int (*interrupted)(void);
} fa2_full_params;

/* Slots of the `times` array of fa2_full_run (src/fa2.h:117-126). */
enum {
    FA2_FULL_T_TOTAL,
    FA2_FULL_T_CODES,
    FA2_FULL_T_SORT,
    FA2_FULL_T_TREE,
    FA2_FULL_T_REPULSION,
    FA2_FULL_T_ATTRACTION,
    FA2_FULL_T_MOVE,
    FA2_FULL_NTIMES
};

/* The whole layout on the device (src/gpu_full.c:164-532).  pos holds the x
 * then the y coordinates (an R n x 2 matrix) and receives the result; times
 * receives FA2_FULL_NTIMES values in seconds.  2 <= n <= 2^26. */
int fa2_full_run(const fa2_full_params *p, double *pos, double *times);

/* Gephi's adaptive speed (src/forceatlas2.c:445-485).  It is defined by the
 * package's forceatlas2.c; libfa2cuda.so does not export it (the speed update
 * of fa2_full_run runs on the device) so that both link together. */
void fa2_update_speed(int n, double total_swinging, double total_traction,
                      double jitter_tolerance, double *speed,
                      double *speed_efficiency);

#ifdef __cplusplus
}
#endif

#endif
