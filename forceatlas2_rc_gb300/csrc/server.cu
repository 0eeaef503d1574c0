// server.cu -- the layout server of fa2_cuda.h (fa2cu_server_*): continuous
// batching of layout jobs on one GPU.
//
// Three kinds of host thread meet here:
//   - callers: submit (the job's arrays are copied) and wait / collect;
//   - the admission thread: takes queued jobs (in arrival order, or least
//     work first) while fewer
//     than max_jobs are resident and their estimated device footprint fits
//     the budget, and opens each one (graph upload, buffers from the
//     server's memory pool, CUDA graphs of its iteration) on a stream of its
//     own;
//   - the scheduling thread: keeps up to two chunks of iterations in flight
//     per resident job (one CUDA event per chunk), so that the jobs'
//     kernels overlap on the device; when a job's last chunk has ended it
//     checks the job's status, fetches its positions and releases its
//     memory, which lets the admission thread bring in the next job.
//
// A job's computation reads and writes only its own buffers, on its own
// stream, with the single-layout path's kernels: its result is the same
// alone and beside any other jobs. Device memory comes from a pool with
// stream-ordered allocation (cudaMallocFromPoolAsync / cudaFreeAsync), so
// admitting or finishing a job never synchronises the device.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fa2_cuda.h"
#include "common.cuh"
#include "session.h"

namespace fa2cu {

struct Job {
    long long id = 0;
    fa2_full_params p{};
    int repulsion = 0;
    std::vector<int> off, node, fixed;
    std::vector<double> coef, mass, size, pos, result;
    double footprint = 0.0;
    int priority = 0;
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
    int state = 0; // 0 queued or running, 1 done, 2 failed
    bool claimed = false; // returned by a wait (then collected once)
    std::string message;
    LayoutBase *L = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int issued = 0, inflight = 0, head = 0;
    bool launch_failed = false;
    double speed = 0.0;

    void drop_inputs()
    {
        std::vector<int>().swap(off);
        std::vector<int>().swap(node);
        std::vector<int>().swap(fixed);
        std::vector<double>().swap(coef);
        std::vector<double>().swap(mass);
        std::vector<double>().swap(size);
        std::vector<double>().swap(pos);
    }
    void close_layout()
    {
        delete L; // synchronises the job's stream, frees into the pool
        L = nullptr;
        for (auto &e : ev)
            if (e) {
                cudaEventDestroy(e);
                e = nullptr;
            }
    }
};

struct Server {
    int device = 0, max_jobs = 16, chunk = 16, policy = FA2CU_ADMIT_ARRIVAL;
    static constexpr int DEPTH = 2; // chunks in flight per job
    double budget = 0.0;
    cudaMemPool_t pool = nullptr;
    int prio_least = 0, prio_greatest = 0;

    std::mutex mu;
    std::condition_variable cv_admit, cv_sched, cv_done;
    std::deque<Job *> queue;                   // submitted, not resident yet
    std::vector<Job *> ready;                  // resident, not scheduled yet
    std::unordered_map<long long, Job *> jobs; // every job not collected
    std::deque<long long> finished;            // ended, not claimed (in order)
    long long next_id = 0, unclaimed = 0;
    int resident = 0;
    double used = 0.0, peak_used = 0.0;
    long long n_done = 0, n_failed = 0;
    bool stop = false;
    std::thread admit_th, sched_th;

    void admit_loop();
    std::deque<Job *>::iterator next_job();
    void sched_loop();
    void finish(Job *j);
    int priority_of(const fa2_full_params &p) const;
};

// Stream priority from the job's work (nodes x iterations): 1e6 and less
// get the greatest priority, 2e9 and more the least, log-linear between.
int Server::priority_of(const fa2_full_params &p) const
{
    const double w = std::max(1.0, (double) p.n * (double) std::max(p.iterations, 1));
    double t = (std::log10(w) - 6.0) / (std::log10(2e9) - 6.0);
    t = std::min(1.0, std::max(0.0, t));
    return prio_greatest + (int) std::lround(t * (double) (prio_least - prio_greatest));
}

// The queued job to admit next: the first one, or the one of least work.
std::deque<Job *>::iterator Server::next_job()
{
    if (policy != FA2CU_ADMIT_LEAST_WORK) return queue.begin();
    auto best = queue.begin();
    double bw = 0.0;
    for (auto it = queue.begin(); it != queue.end(); ++it) {
        const double wk = (double) (*it)->p.n * (double) std::max((*it)->p.iterations, 1);
        if (it == queue.begin() || wk < bw) {
            best = it;
            bw = wk;
        }
    }
    return best;
}

void Server::admit_loop()
{
    cudaSetDevice(device);
    for (;;) {
        Job *j = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_admit.wait(lk, [&] {
                if (stop) return true;
                if (queue.empty() || resident >= max_jobs) return false;
                return used + (*next_job())->footprint <= budget;
            });
            if (stop) return;
            auto it = next_job();
            j = *it;
            queue.erase(it);
            resident++;
            used += j->footprint;
            peak_used = std::max(peak_used, used);
        }
        LayoutOpts o;
        o.pool = pool;
        o.has_priority = true;
        o.priority = j->priority;
        LayoutBase *L = j->p.use_double ? make_layout_f64(&j->p, j->pos.data(), j->repulsion, &o)
                                        : make_layout_f32(&j->p, j->pos.data(), j->repulsion, &o);
        std::string msg;
        if (L) {
            for (auto &e : j->ev)
                if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                    msg = "could not create a CUDA event";
                    break;
                }
        } else {
            msg = fa2_gpu_error();
        }
        j->L = L;
        j->drop_inputs();
        std::lock_guard<std::mutex> lk(mu);
        if (msg.empty()) {
            j->t_admit = fa2_now();
            ready.push_back(j);
            cv_sched.notify_one();
        } else {
            j->close_layout();
            j->state = 2;
            j->message = msg;
            j->t_admit = j->t_done = fa2_now();
            resident--;
            used -= j->footprint;
            n_failed++;
            finished.push_back(j->id);
            cv_done.notify_all();
        }
    }
}

void Server::finish(Job *j)
{
    std::string msg;
    if (j->launch_failed) msg = j->message;
    if (msg.empty() && j->L->sync()) msg = fa2_gpu_error();
    if (msg.empty()) {
        j->result.resize(2 * (size_t) j->p.n);
        if (j->L->positions(j->result.data())) msg = fa2_gpu_error();
        double st[4] = {0, 0, 0, 0};
        if (msg.empty() && !j->L->speed(st)) j->speed = st[0];
    }
    j->close_layout();
    std::lock_guard<std::mutex> lk(mu);
    j->t_done = fa2_now();
    if (msg.empty()) {
        j->state = 1;
        n_done++;
    } else {
        j->state = 2;
        j->message = msg;
        j->result.clear();
        n_failed++;
    }
    resident--;
    used -= j->footprint;
    finished.push_back(j->id);
    cv_done.notify_all();
    cv_admit.notify_one();
}

void Server::sched_loop()
{
    cudaSetDevice(device);
    std::vector<Job *> active;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            if (active.empty())
                cv_sched.wait(lk, [&] { return stop || !ready.empty(); });
            if (stop) break;
            active.insert(active.end(), ready.begin(), ready.end());
            ready.clear();
        }
        bool progressed = false;
        for (size_t k = 0; k < active.size();) {
            Job *j = active[k];
            // chunks that have ended (an error also ends the wait: the
            // status check at the end reports it)
            while (j->inflight > 0 && cudaEventQuery(j->ev[j->head]) != cudaErrorNotReady) {
                j->inflight--;
                j->head ^= 1;
                progressed = true;
            }
            if (j->issued >= j->p.iterations && j->inflight == 0) {
                finish(j);
                active[k] = active.back();
                active.pop_back();
                progressed = true;
                continue;
            }
            while (j->inflight < DEPTH && j->issued < j->p.iterations) {
                const int it = std::min(chunk, j->p.iterations - j->issued);
                if (j->L->iterate(it) ||
                    cudaEventRecord(j->ev[(j->head + j->inflight) & 1], j->L->stream()) !=
                        cudaSuccess) {
                    j->launch_failed = true;
                    j->message = fa2_gpu_error();
                    if (j->message.empty()) j->message = "the computation on the GPU failed";
                    j->issued = j->p.iterations;
                    break;
                }
                j->inflight++;
                j->issued += it;
                progressed = true;
            }
            k++;
        }
        if (!progressed) {
            std::unique_lock<std::mutex> lk(mu);
            cv_sched.wait_for(lk, std::chrono::microseconds(50),
                              [&] { return stop || !ready.empty(); });
        }
    }
    for (Job *j : active) j->close_layout();
}

} // namespace fa2cu

using namespace fa2cu;

struct fa2cu_server {
    Server *impl;
};

extern "C" {

static int device_sms(int device)
{
    int sms = 0;
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return sms > 0 ? sms : 1;
}

static double footprint_on(int device, int n, int ninc, int adjust, int any_fixed, int use_double,
                           int repulsion)
{
    if (n < 1 || ninc < 0) return 0.0;
    const int sms = device_sms(device);
    return use_double ? layout_footprint_f64(n, ninc, adjust, any_fixed, repulsion, sms)
                      : layout_footprint_f32(n, ninc, adjust, any_fixed, repulsion, sms);
}

double fa2cu_layout_footprint(int n, int ninc, int adjust, int any_fixed, int use_double,
                              int repulsion)
{
    return footprint_on(-1, n, ninc, adjust, any_fixed, use_double, repulsion);
}

fa2cu_server *fa2cu_server_open(const fa2cu_server_config *cfg)
{
    if (!cfg) {
        set_message("invalid arguments");
        return nullptr;
    }
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || cfg->device < 0 || cfg->device >= nd) {
        set_message("there is no CUDA device %d", cfg->device);
        return nullptr;
    }
    FA2_TRY(cudaSetDevice(cfg->device), "could not use the CUDA device", nullptr);
    Server *S = new Server();
    S->device = cfg->device;
    S->max_jobs = cfg->max_jobs > 0 ? cfg->max_jobs : 16;
    S->chunk = cfg->chunk > 0 ? cfg->chunk : 16;
    S->policy = cfg->policy == FA2CU_ADMIT_LEAST_WORK ? FA2CU_ADMIT_LEAST_WORK
                                                     : FA2CU_ADMIT_ARRIVAL;
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    S->budget = cfg->hbm_budget > 0 ? cfg->hbm_budget : 0.8 * (double) fr;
    cudaDeviceGetStreamPriorityRange(&S->prio_least, &S->prio_greatest);
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = cfg->device;
    cudaError_t e = cudaMemPoolCreate(&S->pool, &props);
    if (e != cudaSuccess) {
        set_cuda_error("could not create the device memory pool", e);
        delete S;
        return nullptr;
    }
    // keep freed memory in the pool for the next jobs
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    S->admit_th = std::thread([S] { S->admit_loop(); });
    S->sched_th = std::thread([S] { S->sched_loop(); });
    fa2cu_server *h = new fa2cu_server;
    h->impl = S;
    return h;
}

long long fa2cu_server_submit(fa2cu_server *h, const fa2_full_params *p, const double *pos,
                              int repulsion)
{
    if (!h || !p || !pos) {
        set_message("invalid arguments");
        return -1;
    }
    Server *S = h->impl;
    if (repulsion != FA2CU_REPULSION_BH && repulsion != FA2CU_REPULSION_EXACT) {
        set_message("unknown repulsion %d", repulsion);
        return -1;
    }
    const int nmin = repulsion == FA2CU_REPULSION_EXACT ? 1 : 2;
    if (p->n < nmin || p->n > (1 << 26)) {
        set_message("the all-GPU layout handles between 2 and 67 million nodes");
        return -1;
    }
    if (p->iterations < 0) {
        set_message("invalid number of iterations");
        return -1;
    }
    if (!p->mass || (p->adjust && !p->size)) {
        set_message("invalid arguments: masses (and radii with adjust) are required");
        return -1;
    }
    if (check_csr(p->n, p->inc_off, p->inc_node)) return -1;
    const int n = p->n, ninc = p->inc_off[n];
    if (ninc > 0 && !p->inc_coef) {
        set_message("invalid incidence list: inc_coef is missing");
        return -1;
    }
    for (int i = 0; i < 2 * n; i++)
        if (!std::isfinite(pos[i])) {
            set_message("the start positions must be finite");
            return -1;
        }
    int any_fixed = 0;
    if (p->fixed)
        for (int i = 0; i < n && !any_fixed; i++) any_fixed = p->fixed[i] != 0;
    const double fp =
        footprint_on(S->device, n, ninc, p->adjust, any_fixed, p->use_double, repulsion);
    if (fp > S->budget) {
        set_message("the job needs %.0f bytes of device memory, more than the server's "
                    "budget of %.0f",
                    fp, S->budget);
        return -1;
    }
    Job *j = new Job();
    j->repulsion = repulsion;
    j->footprint = fp;
    j->off.assign(p->inc_off, p->inc_off + n + 1);
    j->node.assign(p->inc_node, p->inc_node + ninc);
    if (ninc > 0) j->coef.assign(p->inc_coef, p->inc_coef + ninc);
    j->mass.assign(p->mass, p->mass + n);
    if (p->adjust) j->size.assign(p->size, p->size + n);
    if (any_fixed) j->fixed.assign(p->fixed, p->fixed + n);
    j->pos.assign(pos, pos + 2 * (size_t) n);
    j->p = *p;
    j->p.inc_off = j->off.data();
    j->p.inc_node = j->node.data();
    j->p.inc_coef = ninc > 0 ? j->coef.data() : nullptr;
    j->p.mass = j->mass.data();
    j->p.size = p->adjust ? j->size.data() : nullptr;
    j->p.fixed = any_fixed ? j->fixed.data() : nullptr;
    j->p.any_fixed = any_fixed;
    j->p.device = S->device;
    j->p.profile = 0;
    j->p.source = nullptr;
    j->p.interrupted = nullptr;
    j->priority = S->priority_of(j->p);
    j->t_submit = fa2_now();
    std::lock_guard<std::mutex> lk(S->mu);
    j->id = S->next_id++;
    S->unclaimed++;
    S->jobs[j->id] = j;
    S->queue.push_back(j);
    S->cv_admit.notify_one();
    return j->id;
}

long long fa2cu_server_wait(fa2cu_server *h, long long id, double timeout_s, double info[8])
{
    if (!h) {
        set_message("invalid arguments");
        return -2;
    }
    Server *S = h->impl;
    std::unique_lock<std::mutex> lk(S->mu);
    auto ended = [&] {
        if (id >= 0) {
            auto it = S->jobs.find(id);
            return it == S->jobs.end() || it->second->state != 0;
        }
        return !S->finished.empty() || S->unclaimed == 0;
    };
    if (timeout_s < 0)
        S->cv_done.wait(lk, ended);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ended))
        return -1;
    long long got = id;
    if (id >= 0) {
        if (!S->jobs.count(id)) {
            set_message("there is no job %lld (or it was collected)", id);
            return -2;
        }
        auto it = std::find(S->finished.begin(), S->finished.end(), id);
        if (it != S->finished.end()) S->finished.erase(it);
    } else {
        if (S->finished.empty()) {
            set_message("no job is pending");
            return -2;
        }
        got = S->finished.front();
        S->finished.pop_front();
    }
    Job *j = S->jobs[got];
    if (!j->claimed) {
        j->claimed = true;
        S->unclaimed--;
    }
    if (info) {
        info[0] = j->t_submit;
        info[1] = j->t_admit;
        info[2] = j->t_done;
        info[3] = j->state == 1 ? 0.0 : 1.0;
        info[4] = j->p.n;
        info[5] = j->p.iterations;
        info[6] = j->footprint;
        info[7] = j->speed;
    }
    return got;
}

int fa2cu_server_collect(fa2cu_server *h, long long id, double *pos)
{
    if (!h) {
        set_message("invalid arguments");
        return 1;
    }
    Server *S = h->impl;
    Job *j = nullptr;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->jobs.find(id);
        if (it == S->jobs.end() || it->second->state == 0) {
            set_message("job %lld has not ended (or was collected)", id);
            return 1;
        }
        j = it->second;
        S->jobs.erase(it);
        auto f = std::find(S->finished.begin(), S->finished.end(), id);
        if (f != S->finished.end()) S->finished.erase(f);
        if (!j->claimed) S->unclaimed--;
    }
    int rc = 0;
    if (j->state == 1) {
        if (pos) std::copy(j->result.begin(), j->result.end(), pos);
    } else {
        set_message("%s", j->message.c_str());
        rc = 1;
    }
    delete j;
    return rc;
}

int fa2cu_server_stats(fa2cu_server *h, double out[8])
{
    Server *S = h->impl;
    uint64_t reserved = 0;
    cudaMemPoolGetAttribute(S->pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    std::lock_guard<std::mutex> lk(S->mu);
    out[0] = (double) S->queue.size();
    out[1] = (double) S->resident;
    out[2] = (double) S->n_done;
    out[3] = (double) S->n_failed;
    out[4] = S->used;
    out[5] = S->peak_used;
    out[6] = S->budget;
    out[7] = (double) reserved;
    return 0;
}

void fa2cu_server_close(fa2cu_server *h)
{
    if (!h) return;
    Server *S = h->impl;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_admit.notify_all();
    S->cv_sched.notify_all();
    S->cv_done.notify_all();
    S->admit_th.join();
    S->sched_th.join();
    cudaSetDevice(S->device);
    for (Job *j : S->ready) j->close_layout();
    for (auto &kv : S->jobs) delete kv.second;
    // released once the jobs' frees have completed
    cudaMemPoolDestroy(S->pool);
    delete S;
    delete h;
}

} // extern "C"
