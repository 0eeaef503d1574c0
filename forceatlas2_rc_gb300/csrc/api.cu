// api.cu -- the C interface of libfa2cuda.so: every entry point of the
// package's fa2.h (reference src/gpu.c, src/gpu_full.c, src/ocl_loader.c),
// implemented over the CUDA runtime, plus the fa2_cuda.h extensions.
//
// Like the reference, nothing here longjmps or prints: failures return a
// non-zero status (or NULL) and leave a message for fa2_gpu_error().
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <time.h>
#include <mutex>
#include <vector>

#include "session.h"
#include "prep.cuh"
#include "common.cuh"

// Opaque handles of the C interface.
struct fa2_gpu {
    fa2cu::RepulseBase *impl;
    int n;
};
struct fa2cu_layout {
    fa2cu::LayoutBase *impl;
    int n;
};
struct fa2cu_batch {
    fa2cu::BatchBase *impl;
};

namespace fa2cu {

// one message per host thread (the serving loop runs on threads of its own)
static thread_local char errbuf[2048] = "";

void set_message(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(errbuf, sizeof(errbuf), fmt, ap);
    va_end(ap);
}

void set_cuda_error(const char *what, cudaError_t e)
{
    snprintf(errbuf, sizeof(errbuf), "%s (CUDA error %d: %s)", what, (int) e,
             cudaGetErrorString(e));
    cudaGetLastError(); // clear a sticky launch error of this thread
}

int check_csr(int n, const int *off, const int *node)
{
    if (!off || off[0] != 0) {
        set_message("invalid incidence list: inc_off[0] must be 0");
        return 1;
    }
    for (int i = 0; i < n; i++)
        if (off[i + 1] < off[i]) {
            set_message("invalid incidence list: inc_off decreases at node %d", i + 1);
            return 1;
        }
    const int e1 = off[n];
    if (e1 > 0 && !node) {
        set_message("invalid incidence list: inc_node is missing");
        return 1;
    }
    for (int e = 0; e < e1; e++)
        if (node[e] < 0 || node[e] >= n) {
            set_message("invalid incidence list: entry %d refers to a node that does not exist",
                        e + 1);
            return 1;
        }
    return 0;
}

// The quadtree must be one the traversal can walk: regions in breadth-first
// order (children after their parent), node ranges inside [0, n), and skip
// links equal to the region that follows each subtree in the walk's order
// (last child first). This guarantees that every walk ends and stays in
// bounds, whatever the theta.
int check_quadtree(int n, const fa2_tree *t)
{
    const int nreg = t->nreg;
    if (nreg < 1 || nreg > 2 * n || !t->reg || !t->perm || !t->px || !t->py || !t->pm) {
        set_message("invalid Barnes-Hut tree");
        return 1;
    }
    const fa2_region *R = t->reg;
    std::vector<int> sz((size_t) nreg, 1);
    for (int r = nreg - 1; r >= 0; r--) {
        const fa2_region &g = R[r];
        if (g.start < 0 || g.count < 0 || g.start > n - g.count) {
            set_message("invalid Barnes-Hut tree: region %d covers missing nodes", r + 1);
            return 1;
        }
        if (g.nchild > 0) {
            if (g.child <= r || g.child > nreg - g.nchild) {
                set_message("invalid Barnes-Hut tree: region %d has invalid children", r + 1);
                return 1;
            }
            for (int c = 0; c < g.nchild; c++) sz[r] += sz[g.child + c];
        }
    }
    if (sz[0] != nreg) {
        set_message("invalid Barnes-Hut tree: not every region belongs to the tree");
        return 1;
    }
    // walk: position of each region in the order last-child-first
    std::vector<int> order;
    order.reserve((size_t) nreg);
    std::vector<int> stack;
    stack.push_back(0);
    while (!stack.empty()) {
        const int r = stack.back();
        stack.pop_back();
        order.push_back(r);
        if ((int) order.size() > nreg) break;
        for (int c = 0; c < R[r].nchild; c++) stack.push_back(R[r].child + c);
    }
    if ((int) order.size() != nreg) {
        set_message("invalid Barnes-Hut tree: a region is reached twice");
        return 1;
    }
    std::vector<int> at((size_t) nreg, -1);
    for (int k = 0; k < nreg; k++) {
        if (at[order[k]] >= 0) {
            set_message("invalid Barnes-Hut tree: a region is reached twice");
            return 1;
        }
        at[order[k]] = k;
    }
    for (int r = 0; r < nreg; r++) {
        const int next = at[r] + sz[r];
        const int want = next < nreg ? order[next] : -1;
        if (R[r].skip != want) {
            set_message("invalid Barnes-Hut tree: wrong skip link at region %d", r + 1);
            return 1;
        }
    }
    for (int k = 0; k < n; k++)
        if (t->perm[k] < 0 || t->perm[k] >= n) {
            set_message("invalid Barnes-Hut tree: perm refers to a node that does not exist");
            return 1;
        }
    return 0;
}

static int device_count()
{
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return nd;
}

static int check_device(int device)
{
    const int nd = device_count();
    if (nd < 0) {
        set_message("no CUDA device was found on this computer");
        return 1;
    }
    if (device < 0 || device >= nd) {
        set_message("there is no CUDA device %d", device + 1);
        return 1;
    }
    return 0;
}

} // namespace fa2cu

using namespace fa2cu;

extern "C" {

const char *fa2_gpu_error(void) { return errbuf; }

int fa2_gpu_ndevices(void)
{
    const int nd = device_count();
    if (nd < 0) {
        set_message("no CUDA device was found on this computer");
        return 0;
    }
    return nd;
}

int fa2_gpu_device_info(int idx, fa2_gpu_devinfo *info)
{
    if (idx < 0 || idx >= fa2_gpu_ndevices() || !info) return 1;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, idx) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    memset(info, 0, sizeof(*info));
    // the device name is cut to the interface's 128 bytes
    snprintf(info->name, sizeof(info->name), "%.*s", (int) sizeof(info->name) - 1, p.name);
    snprintf(info->vendor, sizeof(info->vendor), "NVIDIA Corporation");
    snprintf(info->platform, sizeof(info->platform), "CUDA");
    int rt = 0;
    cudaRuntimeGetVersion(&rt);
    snprintf(info->version, sizeof(info->version), "CUDA %d.%d sm_%d%d", rt / 1000,
             (rt % 1000) / 10, p.major, p.minor);
    info->is_gpu = 1;
    info->has_double = 1;
    info->memory = (double) p.totalGlobalMem;
    return 0;
}

fa2_gpu *fa2_gpu_open(int device, int use_double, int n, int adjust, int barnes_hut,
                      int threads)
{
    (void) threads; // conversions run on the device
    if (check_device(device)) return nullptr;
    if (n < 1 || n > (1 << 27)) {
        set_message("the GPU backend handles at most %d nodes", 1 << 27);
        return nullptr;
    }
    RepulseBase *impl = use_double ? make_repulse_f64(device, n, adjust, barnes_hut)
                                   : make_repulse_f32(device, n, adjust, barnes_hut);
    if (!impl) return nullptr;
    fa2_gpu *g = new fa2_gpu;
    g->impl = impl;
    g->n = n;
    return g;
}

void fa2_gpu_times(const fa2_gpu *g, double times[3])
{
    times[0] = g->impl->t_send;
    times[1] = g->impl->t_compute;
    times[2] = g->impl->t_fetch;
}

void fa2_gpu_close(fa2_gpu *g)
{
    if (!g) return;
    delete g->impl;
    delete g;
}

int fa2_gpu_repulse_exact(fa2_gpu *g, const double *x, const double *y, const double *mass,
                          const double *size, double scaling, double *dx, double *dy)
{
    return g->impl->exact(x, y, mass, size, scaling, dx, dy);
}

int fa2_gpu_repulse_bh(fa2_gpu *g, const fa2_tree *t, double scaling, double theta, double *dx,
                       double *dy)
{
    return g->impl->bh(t, scaling, theta, dx, dy);
}

void fa2_gpu_shutdown(void)
{
    // Nothing is cached between sessions: kernels are compiled in, and each
    // session owns its stream and memory.
}

double fa2_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

// ---- resident layouts -------------------------------------------------------

fa2cu_layout *fa2cu_layout_open(const fa2_full_params *p, const double *pos, int repulsion)
{
    if (!p || !pos) {
        set_message("invalid arguments");
        return nullptr;
    }
    if (repulsion != FA2CU_REPULSION_BH && repulsion != FA2CU_REPULSION_EXACT) {
        set_message("unknown repulsion %d", repulsion);
        return nullptr;
    }
    // the tree needs two nodes; the exact repulsion handles a single one
    const int nmin = repulsion == FA2CU_REPULSION_EXACT ? 1 : 2;
    if (p->n < nmin || p->n > (1 << 26)) {
        set_message("the all-GPU layout handles between 2 and 67 million nodes");
        return nullptr;
    }
    if (!p->mass || (p->adjust && !p->size)) {
        set_message("invalid arguments: masses (and radii with adjust) are required");
        return nullptr;
    }
    if (check_csr(p->n, p->inc_off, p->inc_node)) return nullptr;
    if (p->inc_off[p->n] > 0 && !p->inc_coef) {
        set_message("invalid incidence list: inc_coef is missing");
        return nullptr;
    }
    if (check_device(p->device)) return nullptr;
    LayoutBase *impl = p->use_double ? make_layout_f64(p, pos, repulsion)
                                     : make_layout_f32(p, pos, repulsion);
    if (!impl) return nullptr;
    fa2cu_layout *L = new fa2cu_layout;
    L->impl = impl;
    L->n = p->n;
    return L;
}

int fa2cu_layout_iterate(fa2cu_layout *L, int iterations)
{
    if (iterations < 0) {
        set_message("invalid number of iterations");
        return 1;
    }
    return L->impl->iterate(iterations);
}
int fa2cu_layout_sync(fa2cu_layout *L) { return L->impl->sync(); }
int fa2cu_layout_positions(fa2cu_layout *L, double *pos) { return L->impl->positions(pos); }
int fa2cu_layout_set_positions(fa2cu_layout *L, const double *pos)
{
    return L->impl->set_positions(pos);
}
int fa2cu_layout_forces(fa2cu_layout *L, const double *pos, double *f)
{
    return L->impl->forces(pos, f);
}
int fa2cu_layout_speed(fa2cu_layout *L, double state[4]) { return L->impl->speed(state); }
void *fa2cu_layout_stream(fa2cu_layout *L) { return (void *) L->impl->stream(); }
int fa2cu_layout_phase_times(fa2cu_layout *L, int iterations, double *ms)
{
    return L->impl->phase_times(iterations, ms);
}
int fa2cu_layout_tree(fa2cu_layout *L, const double *pos, uint32_t *key, uint32_t *order,
                      int *child, int *range, int *parent, double *ni)
{
    return L->impl->tree(pos, key, order, child, range, parent, ni);
}
int fa2cu_layout_traversal_counts(fa2cu_layout *L, double counts[2])
{
    return L->impl->traversal_counts(counts);
}
int fa2cu_layout_option(fa2cu_layout *L, const char *name, double value)
{
    if (!name) {
        set_message("invalid option");
        return 1;
    }
    return L->impl->option(name, value);
}
double fa2cu_layout_info(fa2cu_layout *L, const char *name)
{
    if (!name) {
        set_message("invalid layout information name");
        return -1.0;
    }
    return L->impl->info(name);
}
int fa2cu_layout_swing(fa2cu_layout *L, double *sw, double *tr)
{
    return L->impl->swing(sw, tr);
}
double fa2cu_layout_bytes(const fa2cu_layout *L) { return L->impl->bytes(); }
void fa2cu_layout_close(fa2cu_layout *L)
{
    if (!L) return;
    delete L->impl;
    delete L;
}

// ---- batched layouts ---------------------------------------------------------

// [device][double] -> exact_below, threads, nodes per thread (0: not yet);
// one tuning at a time (callers on several host threads wait for it)
static int tuned[64][2][3];
static std::mutex tune_lock;

int fa2cu_batch_tune(int device, int use_double, int *exact_below, int *threads,
                     int *nodes_per_thread)
{
    if (check_device(device)) return 1;
    if (device >= 64) {
        set_message("the autotuner supports devices 0 to 63");
        return 1;
    }
    std::lock_guard<std::mutex> hold(tune_lock);
    int *t = tuned[device][use_double ? 1 : 0];
    if (!t[1]) {
        const int rc = use_double ? tune_batch_f64(device, &t[0], &t[1], &t[2])
                                  : tune_batch_f32(device, &t[0], &t[1], &t[2]);
        if (rc) {
            t[0] = t[1] = t[2] = 0;
            return 1;
        }
    }
    *exact_below = t[0];
    *threads = t[1];
    if (nodes_per_thread) *nodes_per_thread = t[2];
    return 0;
}

fa2cu_batch *fa2cu_batch_open(const fa2_full_params *graphs, int count, const double *const *pos,
                              int exact_below, int threads, int nodes_per_thread)
{
    if (!graphs || !pos || count < 1) {
        set_message("invalid arguments: a batch needs at least one graph");
        return nullptr;
    }
    const int dev = graphs[0].device, dbl = graphs[0].use_double ? 1 : 0;
    if (check_device(dev)) return nullptr;
    for (int g = 0; g < count; g++) {
        const fa2_full_params &p = graphs[g];
        if (p.n < 1 || p.n > (1 << 26)) {
            set_message("graph %d of the batch: between 1 and 67 million nodes", g + 1);
            return nullptr;
        }
        if (!pos[g] || !p.mass || (p.adjust && !p.size)) {
            set_message("graph %d of the batch: missing positions, masses or radii", g + 1);
            return nullptr;
        }
        if (check_csr(p.n, p.inc_off, p.inc_node)) return nullptr;
        if (p.inc_off[p.n] > 0 && !p.inc_coef) {
            set_message("graph %d of the batch: inc_coef is missing", g + 1);
            return nullptr;
        }
        if (p.device != dev || (p.use_double ? 1 : 0) != dbl) {
            set_message("the graphs of a batch share one device and one precision");
            return nullptr;
        }
    }
    if (threads != 0 && threads != 256 && threads != 512) {
        set_message("threads must be 256 or 512 (0: tuned)");
        return nullptr;
    }
    if (nodes_per_thread != 0 && nodes_per_thread != 1 && nodes_per_thread != 2) {
        set_message("nodes_per_thread must be 1 or 2 (0: tuned)");
        return nullptr;
    }
    if (exact_below < 0 || threads == 0 || nodes_per_thread == 0) {
        int eb = 0, th = 0, np = 0;
        if (fa2cu_batch_tune(dev, dbl, &eb, &th, &np)) return nullptr;
        if (exact_below < 0) exact_below = eb;
        if (threads == 0) threads = th;
        if (nodes_per_thread == 0) nodes_per_thread = np;
    }
    BatchBase *impl =
        dbl ? make_batch_f64(graphs, count, pos, exact_below, threads, nodes_per_thread)
            : make_batch_f32(graphs, count, pos, exact_below, threads, nodes_per_thread);
    if (!impl) return nullptr;
    fa2cu_batch *B = new fa2cu_batch;
    B->impl = impl;
    return B;
}

int fa2cu_batch_iterate(fa2cu_batch *B, int iterations)
{
    if (iterations < 0) {
        set_message("invalid number of iterations");
        return 1;
    }
    return iterations ? B->impl->iterate(iterations) : 0;
}
int fa2cu_batch_sync(fa2cu_batch *B) { return B->impl->sync(); }
int fa2cu_batch_positions(fa2cu_batch *B, int g, double *pos) { return B->impl->positions(g, pos); }
int fa2cu_batch_forces(fa2cu_batch *B, int g, double *f) { return B->impl->forces(g, f); }
int fa2cu_batch_speed(fa2cu_batch *B, int g, double state[4]) { return B->impl->speed(g, state); }
void *fa2cu_batch_stream(fa2cu_batch *B) { return (void *) B->impl->stream(); }
int fa2cu_batch_phase_cycles(fa2cu_batch *B, int iterations, double cycles[8])
{
    if (iterations < 1) {
        set_message("invalid number of iterations");
        return 1;
    }
    return B->impl->phase_cycles(iterations, cycles);
}
double fa2cu_batch_bytes(const fa2cu_batch *B) { return B->impl->bytes(); }
void fa2cu_batch_close(fa2cu_batch *B)
{
    if (!B) return;
    delete B->impl;
    delete B;
}

const char *fa2cu_build_info(void)
{
    return "libfa2cuda: sm_103a; FP32 path -ftz -prec-div=false -prec-sqrt=false; "
           "FP64 path -fmad=false IEEE";
}

// ---- fa2_full_run (reference src/gpu_full.c:164-532) ------------------------

// The iterations of fa2_full_run on an open layout, then its positions.
// Interruptions are polled about every 10^6 units of work, as the reference
// (src/gpu_full.c:403-411): one chunk of iterations runs while the next is
// queued, and the host checks p->interrupted() each time a chunk ends.
static int run_full(fa2cu_layout *L, const fa2_full_params *p, int ninc, double *pos,
                    double *times)
{
    const double start = fa2_now();
    const int n = p->n;
    const double per_it = (double) n + (double) ninc;
    int chunk = (int) (1e6 / per_it);
    if (chunk < 1) chunk = 1;
    int status = 0;
    double ms[FA2_FULL_NTIMES] = {0, 0, 0, 0, 0, 0, 0};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (auto &e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            set_message("could not create a CUDA event");
            status = 1;
        }
    cudaStream_t s = L->impl->stream();
    long long c = 0;
    for (int it = 0; it < p->iterations && !status; c++) {
        const int k = p->iterations - it < chunk ? p->iterations - it : chunk;
        if (c >= 2 && cudaEventSynchronize(ev[c & 1]) != cudaSuccess) {
            set_message("the computation on the GPU failed");
            status = 1;
            break;
        }
        if (c >= 2 && p->interrupted && p->interrupted()) {
            L->impl->sync();
            set_message("the layout was interrupted");
            status = 1;
            break;
        }
        if (p->profile)
            status = L->impl->phase_times(k, ms);
        else
            status = L->impl->iterate(k);
        if (!status) cudaEventRecord(ev[c & 1], s);
        it += k;
    }
    if (!status) status = L->impl->sync();
    if (!status) status = L->impl->positions(pos);
    if (!status) {
        times[FA2_FULL_T_TOTAL] = fa2_now() - start;
        for (int k = 1; k < FA2_FULL_NTIMES; k++) times[k] = ms[k] / 1000.0;
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    return status;
}

int fa2_full_run(const fa2_full_params *p, double *pos, double *times)
{
    for (int i = 0; i < FA2_FULL_NTIMES; i++) times[i] = 0.0;
    if (p->iterations < 0) {
        set_message("invalid number of iterations");
        return 1;
    }
    fa2cu_layout *L = fa2cu_layout_open(p, pos, FA2CU_REPULSION_BH);
    if (!L) return 1;
    const int status = run_full(L, p, p->inc_off[p->n], pos, times);
    fa2cu_layout_close(L);
    return status;
}

// ---- graphs given as edge lists (preparation on the device) -------------------

// Largest edge count of the device preparation (its 2m sort entries and a
// sort tile stay within int indexing).
static const int PREP_MAX_EDGES = (1 << 30) - (1 << 20);

static int check_edges(int n, int m, const int *from, const int *to, const double *w)
{
    if (m < 0 || m > PREP_MAX_EDGES) {
        set_message("the edge list must have between 0 and %d edges", PREP_MAX_EDGES);
        return 1;
    }
    if (m > 0 && (!from || !to || !w)) {
        set_message("invalid arguments: the edge list is missing");
        return 1;
    }
    (void) n;
    return 0;
}

fa2cu_layout *fa2cu_layout_open_edges(const fa2_full_params *p, int m, const int *from,
                                      const int *to, const double *w, int outbound,
                                      const double *pos, int repulsion)
{
    if (!p || !pos) {
        set_message("invalid arguments");
        return nullptr;
    }
    if (repulsion != FA2CU_REPULSION_BH && repulsion != FA2CU_REPULSION_EXACT) {
        set_message("unknown repulsion %d", repulsion);
        return nullptr;
    }
    const int nmin = repulsion == FA2CU_REPULSION_EXACT ? 1 : 2;
    if (p->n < nmin || p->n > (1 << 26)) {
        set_message("the all-GPU layout handles between 2 and 67 million nodes");
        return nullptr;
    }
    if (p->adjust && !p->size) {
        set_message("invalid arguments: radii are required with adjust");
        return nullptr;
    }
    if (check_edges(p->n, m, from, to, w)) return nullptr;
    if (check_device(p->device)) return nullptr;
    EdgeList E;
    E.m = m;
    E.from = from;
    E.to = to;
    E.w = w;
    E.outbound = outbound ? 1 : 0;
    LayoutBase *impl = p->use_double ? make_layout_f64(p, pos, repulsion, nullptr, &E)
                                     : make_layout_f32(p, pos, repulsion, nullptr, &E);
    if (!impl) return nullptr;
    fa2cu_layout *L = new fa2cu_layout;
    L->impl = impl;
    L->n = p->n;
    return L;
}

int fa2cu_full_run_edges(const fa2_full_params *p, int m, const int *from, const int *to,
                         const double *w, int outbound, double *pos, double *times)
{
    for (int i = 0; i < FA2_FULL_NTIMES; i++) times[i] = 0.0;
    if (p->iterations < 0) {
        set_message("invalid number of iterations");
        return 1;
    }
    fa2cu_layout *L =
        fa2cu_layout_open_edges(p, m, from, to, w, outbound, pos, FA2CU_REPULSION_BH);
    if (!L) return 1;
    // incidences: at most 2m (self-loops have none); only the interrupt
    // polling interval depends on it
    const int status = run_full(L, p, 2 * m, pos, times);
    fa2cu_layout_close(L);
    return status;
}

long long fa2cu_graph_prep(int device, int n, int m, const int *from, const int *to,
                           const double *w, int outbound, double *mass, int *inc_off,
                           int *inc_node, double *inc_coef)
{
    if (n < 1 || n > (1 << 26)) {
        set_message("the graph must have between 1 and 67 million nodes");
        return -1;
    }
    if (check_edges(n, m, from, to, w)) return -1;
    if (check_device(device)) return -1;
    FA2_TRY(cudaSetDevice(device), "could not use the CUDA device", -1);
    cudaStream_t s = nullptr;
    FA2_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "could not create a CUDA stream",
            -1);
    DevMem mem;
    const size_t m1 = (size_t) (m > 0 ? m : 1);
    int *df = mem.get<int>(m1), *dt = mem.get<int>(m1);
    double *dw = mem.get<double>(m1), *dm = mem.get<double>((size_t) n);
    int *doff = mem.get<int>((size_t) n + 1), *dnode = mem.get<int>(2 * m1);
    double *dcoef = mem.get<double>(2 * m1);
    PrepScratch ws;
    prep_scratch(mem, n, m, ws);
    long long got = -1;
    if (mem.failed) {
        set_cuda_error("could not allocate memory on the device", mem.err);
    } else {
        int rc = 0;
        if (m > 0) {
            rc |= cudaMemcpyAsync(df, from, (size_t) m * sizeof(int), cudaMemcpyHostToDevice, s);
            rc |= cudaMemcpyAsync(dt, to, (size_t) m * sizeof(int), cudaMemcpyHostToDevice, s);
            rc |= cudaMemcpyAsync(dw, w, (size_t) m * sizeof(double), cudaMemcpyHostToDevice, s);
        }
        if (rc) set_message("could not send the graph to the device");
        else got = prep_graph(s, n, m, df, dt, dw, outbound, dm, doff, dnode, dcoef, ws);
        if (got >= 0) {
            rc = 0;
            rc |= cudaMemcpyAsync(mass, dm, (size_t) n * sizeof(double), cudaMemcpyDeviceToHost, s);
            rc |= cudaMemcpyAsync(inc_off, doff, ((size_t) n + 1) * sizeof(int),
                                  cudaMemcpyDeviceToHost, s);
            if (got > 0) {
                rc |= cudaMemcpyAsync(inc_node, dnode, (size_t) got * sizeof(int),
                                      cudaMemcpyDeviceToHost, s);
                rc |= cudaMemcpyAsync(inc_coef, dcoef, (size_t) got * sizeof(double),
                                      cudaMemcpyDeviceToHost, s);
            }
            rc |= cudaStreamSynchronize(s);
            if (rc) {
                set_message("could not fetch the prepared graph");
                got = -1;
            }
        }
    }
    cudaStreamSynchronize(s);
    mem.release();
    cudaStreamDestroy(s);
    return got;
}

} // extern "C"
