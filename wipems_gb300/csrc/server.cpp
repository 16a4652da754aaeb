// Continuous-batching job server (no counterpart in the reference, which
// runs one simulation per process through openEMS::RunFDTD).
//
// Requests (scenes) arrive at any time through fdtd_server_submit.  A pool
// of host threads builds and compresses their operators while the GPU
// works; one GPU thread runs scheduling rounds:
//
//   retire  jobs whose device end criterion fired (energy decay below
//           end_crit x the largest sampled energy, or the timestep cap):
//           samples (and optionally fields) are copied out, device memory
//           is freed;
//   admit   built jobs in arrival order while their device footprint fits
//           the HBM budget and the active-job cap (first fit: a large job
//           that does not fit yet does not block smaller ones behind it);
//   batch   (batch mode) on any change of the active set, a new batch over
//           the active engines (fdtd_batch_create) replaces the old one;
//   step    every idle resident job gets its next round_steps queued on
//           its own stream (fdtd_engine_iterate_async), so the GPU overlaps
//           all of them and a job that finishes is picked up, retired and
//           replaced without waiting for the others; or, with
//           batch_min_jobs set and at least that many jobs resident, one
//           persistent batch round (fdtd_batch_iterate) over all of them.
//
// Jobs stop on the device at exactly the timestep they would stop at when
// run alone (the kernels of a stopped job do nothing for the rest of the
// round), and the batched kernels apply the same per-node arithmetic as the
// single-job engine, so a job's result does not depend on what else ran.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cop.h"
#include "fdtd_host.h"

#define CK(call)                                                           \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
            return FDTD_ERR_CUDA;                                          \
        }                                                                  \
    } while (0)

namespace wipems {
namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    int state = FDTD_JOB_QUEUED;
    int error = FDTD_OK;
    std::string message;
    fdtd_scene_t scene = nullptr;
    fdtd_job_opts opts{};
    fdtd_cop_t cop = nullptr;
    std::vector<fdtd_probe_desc> probes;
    uint32_t interval = 0, max_ts = 0;
    uint64_t nodes = 0, footprint = 0;
    uint32_t N[3] = {0, 0, 0};   // device axes (tiling)
    uint32_t N0[3] = {0, 0, 0};  // the operator's axes (reported)
    double dT = 0;
    fdtd_engine_t eng = nullptr;
    uint32_t ts = 0;
    // results, filled at retirement
    std::vector<uint32_t> s_ts;
    std::vector<double> s_energy, s_vals;
    std::vector<float> volt, curr;
    double t_submit = 0, t_built = 0, t_admit = 0, t_done = 0;
};

}  // namespace
}  // namespace wipems

using namespace wipems;

struct fdtd_server_s {
    fdtd_server_opts opts{};
    uint64_t budget = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_build, cv_gpu, cv_done;
    std::map<uint64_t, std::unique_ptr<Job>> jobs;
    std::deque<Job*> build_q;
    std::vector<Job*> ready;  // built, waiting for admission (arrival order)
    uint64_t next_id = 1;
    bool stop = false;
    std::vector<std::thread> builders;
    std::thread gpu;
    // GPU-thread state
    std::vector<Job*> active;
    fdtd_batch_t batch = nullptr;
    std::vector<Job*> batch_jobs;  // the jobs the current batch was built over
    uint64_t used = 0;
    // statistics (under mu)
    fdtd_server_stats st{};

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace wipems {
namespace {

// Device bytes an engine over this operator will allocate (the allocations
// of fdtd_engine_create_compressed), rounded up per allocation.
// sample columns of a job: one per integral probe, three per field probe
size_t sample_columns(const Job* j) {
    size_t cols = 0;
    for (const fdtd_probe_desc& p : j->probes) cols += (p.type == 2 || p.type == 3) ? 3 : 1;
    return cols;
}

uint64_t engine_footprint(const fdtd_cop_s* c, uint32_t interval, uint32_t max_ts, size_t nprobe) {
    auto r = [](uint64_t b) { return (b + (2u << 20) - 1) / (2u << 20) * (2u << 20); };
    const uint64_t F = 3ull * (uint64_t)c->comp * 4;
    uint64_t b = 2 * r(F);
    if (c->E.any_upml || c->H.any_upml) b += 2 * r(F);
    b += (c->E.any_ade ? r(F) : 0) + (c->E.any_lor ? r(F) : 0) + (c->H.any_ade ? r(F) : 0) + (c->H.any_lor ? r(F) : 0);
    for (const HalfTables* T : {&c->E, &c->H})  // states of dispersion orders 1..3
        b += (T->adex_orders ? r(T->adex_orders * F) : 0) + (T->any_lorx ? r(T->adex_orders * F) : 0);
    for (const HalfTables* T : {&c->E, &c->H})
        b += r(T->idx_bytes) +
             r(4 * (T->main.size() + T->upml.size() + T->ade.size() + T->exc.size() + T->adex.size()));
    b += r(4 * c->geom.size()) + 2 * r(4 * std::max<uint32_t>(1, c->sig_len));
    const uint64_t cap = (interval ? max_ts / interval : 0) + 2;
    b += r(cap * (2 + nprobe) * 8) + 8 * (2u << 20);
    return b;
}

void build_one(fdtd_server_s* s, Job* j) {
    fdtd_operator_t op = nullptr;
    int rc = fdtd_operator_build(j->scene, s->opts.build_threads_per_job, &op);
    fdtd_cop_t cop = nullptr;
    std::vector<fdtd_probe_desc> probes;
    fdtd_operator_info info{};
    if (rc == FDTD_OK) rc = fdtd_operator_get_info(op, &info);
    if (rc == FDTD_OK) {
        probes.resize(info.num_probes);
        for (uint32_t p = 0; p < info.num_probes && rc == FDTD_OK; ++p) rc = fdtd_operator_get_probe(op, p, &probes[p]);
    }
    if (rc == FDTD_OK) {
        fdtd_op_desc d{};
        rc = fdtd_operator_describe(op, &d);
        if (rc == FDTD_OK) rc = fdtd_compress_ex(&d, 0, &cop);
    }
    std::string msg = rc ? last_error() : std::string();
    const uint32_t nr_ts = j->scene->nr_ts;
    if (op) fdtd_operator_destroy(op);
    fdtd_scene_destroy(j->scene);
    std::lock_guard<std::mutex> lock(s->mu);
    j->scene = nullptr;
    j->t_built = s->now();
    if (rc) {
        j->state = FDTD_JOB_FAILED;
        j->error = rc;
        j->message = "operator build: " + msg;
        j->t_done = j->t_built;
        s->st.jobs_failed++;
        s->cv_done.notify_all();
        return;
    }
    j->cop = cop;
    j->probes = std::move(probes);
    j->interval = j->opts.probe_interval ? j->opts.probe_interval : info.probe_interval;
    j->max_ts = j->opts.max_timesteps ? j->opts.max_timesteps : (nr_ts ? nr_ts : 100000);
    j->nodes = (uint64_t)cop->N[0] * cop->N[1] * cop->N[2];
    for (int a = 0; a < 3; ++a) {
        j->N[a] = cop->N[a];
        j->N0[a] = cop->N0[a];
    }
    j->dT = cop->dT;
    j->footprint = engine_footprint(cop, j->interval, j->max_ts, sample_columns(j));
    if (j->footprint > s->budget || (j->opts.end_crit > 0 && j->interval == 0)) {
        j->state = FDTD_JOB_FAILED;
        j->error = FDTD_ERR_ARG;
        j->message = j->footprint > s->budget
                         ? "the job's device footprint (" + std::to_string(j->footprint) +
                               " B) exceeds the server's HBM budget (" + std::to_string(s->budget) + " B)"
                         : "end_crit needs a probe interval (the scene has no excitation to derive one from)";
        j->t_done = j->t_built;
        s->st.jobs_failed++;
        fdtd_cop_destroy(cop);
        j->cop = nullptr;
        s->cv_done.notify_all();
        return;
    }
    j->state = FDTD_JOB_READY;
    s->ready.push_back(j);
    s->cv_gpu.notify_all();
}

void builder_loop(fdtd_server_s* s) {
    for (;;) {
        Job* j = nullptr;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_build.wait(lock, [&] { return s->stop || !s->build_q.empty(); });
            if (s->stop) return;
            j = s->build_q.front();
            s->build_q.pop_front();
            j->state = FDTD_JOB_BUILDING;
        }
        build_one(s, j);
    }
}

// copies a finished job's results to the host and frees its device state
void retire(fdtd_server_s* s, Job* j, int err, const std::string& msg) {
    uint32_t n = 0, ts = 0;
    int rc = err;
    if (rc == FDTD_OK) rc = fdtd_engine_num_timesteps(j->eng, &ts);
    if (rc == FDTD_OK) rc = fdtd_engine_num_samples(j->eng, &n);
    std::vector<uint32_t> sts(n);
    std::vector<double> se(n), sv((size_t)n * sample_columns(j));
    if (rc == FDTD_OK && n) rc = fdtd_engine_read_samples(j->eng, 0, n, sts.data(), sv.data(), se.data());
    std::vector<float> V, I;
    if (rc == FDTD_OK && j->opts.keep_fields) {
        const size_t cnt = 3 * (size_t)j->nodes;
        V.resize(cnt);
        I.resize(cnt);
        rc = fdtd_engine_get_fields(j->eng, V.data(), I.data());
    }
    const std::string m = rc ? (err ? msg : last_error()) : std::string();
    fdtd_engine_destroy(j->eng);
    std::lock_guard<std::mutex> lock(s->mu);
    j->eng = nullptr;
    j->ts = ts;
    j->s_ts = std::move(sts);
    j->s_energy = std::move(se);
    j->s_vals = std::move(sv);
    j->volt = std::move(V);
    j->curr = std::move(I);
    j->t_done = s->now();
    s->used -= j->footprint;
    if (rc) {
        j->state = FDTD_JOB_FAILED;
        j->error = rc;
        j->message = m;
        s->st.jobs_failed++;
    } else {
        j->state = FDTD_JOB_DONE;
        s->st.jobs_done++;
        s->st.node_steps += (double)j->nodes * ts;
    }
    s->cv_done.notify_all();
}

int admit(fdtd_server_s* s, Job* j) {
    fdtd_engine_opts o{};
    o.device = s->opts.device;
    o.max_timesteps = j->max_ts;
    o.probe_interval = j->interval;
    o.use_graphs = 1;  // interval graphs for rounds a job runs on its own
    o.kernel = 3;      // batched jobs run the two-pass kernels
    o.energy_on_probe = 1;
    o.end_crit = j->opts.end_crit;
    // jobs overlap on their own streams: tile each for its share of the SMs
    if (s->opts.tile_share != 1) o.x_chunk = engine_auto_x_chunk(j->N, o.device, s->opts.tile_share);
    fdtd_engine_t e = nullptr;
    int rc = fdtd_engine_create_compressed(j->cop, &o, &e);
    for (size_t p = 0; rc == FDTD_OK && p < j->probes.size(); ++p) rc = fdtd_engine_add_probe(e, &j->probes[p], nullptr);
    fdtd_cop_destroy(j->cop);
    std::lock_guard<std::mutex> lock(s->mu);
    j->cop = nullptr;
    if (rc) {
        if (e) fdtd_engine_destroy(e);
        j->state = FDTD_JOB_FAILED;
        j->error = rc;
        j->message = "engine create: " + last_error();
        j->t_done = s->now();
        s->used -= j->footprint;
        s->st.jobs_failed++;
        s->cv_done.notify_all();
        return rc;
    }
    j->eng = e;
    j->state = FDTD_JOB_RUNNING;
    j->t_admit = s->now();
    s->st.jobs_admitted++;
    return FDTD_OK;
}

void drop_batch(fdtd_server_s* s) {
    if (s->batch) fdtd_batch_destroy(s->batch);
    s->batch = nullptr;
    s->batch_jobs.clear();
}

// One persistent-batch round over `jobs` (batch mode); the batch is rebuilt
// when its membership changed.  Returns the jobs that are still running.
std::vector<Job*> batch_round(fdtd_server_s* s, const std::vector<Job*>& jobs) {
    if (!s->batch || jobs != s->batch_jobs) {
        drop_batch(s);
        std::vector<fdtd_engine_t> es;
        for (Job* j : jobs) es.push_back(j->eng);
        const int rc = fdtd_batch_create(es.data(), (uint32_t)es.size(), &s->opts.batch, &s->batch);
        std::lock_guard<std::mutex> lock(s->mu);
        s->st.rebuilds++;
        if (rc) {
            s->batch = nullptr;
            s->st.last_error = rc;
        } else {
            s->batch_jobs = jobs;
        }
    }
    int rc = s->batch ? fdtd_batch_iterate(s->batch, s->opts.round_steps) : FDTD_ERR_STATE;
    if (s->batch) {
        fdtd_batch_stats bs{};
        fdtd_batch_info(s->batch, &bs);
        std::lock_guard<std::mutex> lock(s->mu);
        s->st.rounds++;
        s->st.gpu_ms += bs.last_ms;
        s->st.kernel_launches += bs.last_launches;
    }
    if (!rc) return jobs;
    // find the failing jobs: each engine decodes its own error word
    const std::string msg = last_error();
    std::vector<Job*> ok;
    for (Job* j : jobs) {
        const int jr = s->batch ? fdtd_engine_iterate(j->eng, 0) : rc;
        if (jr) retire(s, j, jr, s->batch ? last_error() : msg);
        else ok.push_back(j);
    }
    if (ok.size() == jobs.size()) {  // not attributable to a job: fail them all
        for (Job* j : ok) retire(s, j, rc, msg);
        ok.clear();
    }
    drop_batch(s);
    return ok;
}

void gpu_loop(fdtd_server_s* s) {
    cudaSetDevice(s->opts.device);
    Clock::time_point busy_since{};
    bool busy = false;
    for (;;) {
        bool changed = false;
        // collect finished work, retire jobs whose end criterion fired
        std::vector<Job*> keep;
        bool any_pending = false;
        for (Job* j : s->active) {
            int ready = 1;
            if (fdtd_engine_query(j->eng, &ready) == FDTD_OK && !ready) {
                keep.push_back(j);
                any_pending = true;
                continue;
            }
            const int rc = fdtd_engine_wait(j->eng);
            if (rc) {
                retire(s, j, rc, last_error());
                changed = true;
                continue;
            }
            int done = 0;
            fdtd_engine_done(j->eng, &done);
            if (done) {
                retire(s, j, FDTD_OK, "");
                changed = true;
            } else {
                keep.push_back(j);
            }
        }
        s->active.swap(keep);
        // admit (first fit in arrival order)
        std::vector<Job*> take;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            if (busy && !any_pending) {  // time with concurrent-engine work in flight
                s->st.gpu_ms += std::chrono::duration<double, std::milli>(Clock::now() - busy_since).count();
                busy = false;
            }
            if (s->active.empty() && s->ready.empty()) {
                if (s->batch) {
                    lock.unlock();
                    drop_batch(s);
                    lock.lock();
                }
                s->cv_gpu.wait(lock, [&] { return s->stop || !s->ready.empty(); });
            } else if (any_pending && !changed && s->ready.empty()) {
                // every resident job is busy: sleep until a new job is built
                // or a short poll interval has passed
                s->cv_gpu.wait_for(lock, std::chrono::microseconds(50),
                                   [&] { return s->stop || !s->ready.empty(); });
            }
            if (s->stop) break;
            std::vector<Job*> rest;
            size_t n_active = s->active.size();
            for (Job* j : s->ready) {
                if (n_active < s->opts.max_active && s->used + j->footprint <= s->budget) {
                    s->used += j->footprint;
                    s->st.peak_bytes = std::max<uint64_t>(s->st.peak_bytes, s->used);
                    take.push_back(j);
                    ++n_active;
                } else {
                    rest.push_back(j);
                }
            }
            s->ready.swap(rest);
        }
        for (Job* j : take)
            if (admit(s, j) == FDTD_OK) {
                s->active.push_back(j);
                changed = true;
            }
        {
            std::lock_guard<std::mutex> lock(s->mu);
            s->st.active_jobs = (uint32_t)s->active.size();
        }
        if (s->active.empty()) continue;
        // batch mode: the jobs a batch can take run as one persistent batch
        // once there are batch_min_jobs of them; the others (Mur, lumped
        // RLC) run as concurrent engines beside it
        std::vector<Job*> bjobs, solo;
        if (s->opts.batch_min_jobs > 0) {
            for (Job* j : s->active) {
                // a batch steps its jobs together; a job without an energy
                // criterion is bounded by its timestep count alone, which the
                // host keeps (the rounds below), so it runs on its own
                int ok = 0;
                if (j->opts.end_crit > 0) fdtd_batch_accepts(j->eng, &ok);
                (ok ? bjobs : solo).push_back(j);
            }
            if (bjobs.size() < s->opts.batch_min_jobs) {
                solo = s->active;
                bjobs.clear();
            }
        } else {
            solo = s->active;
        }
        if (bjobs.empty() && s->batch) drop_batch(s);
        // concurrent engines: every idle job gets its next round_steps
        // queued on its own stream at once; finished jobs are picked up on
        // the next pass, so short and long jobs never wait for each other
        // (queued before a batch round, which runs synchronously, so the two
        // overlap on the device)
        std::vector<Job*> ok;
        uint64_t launches = 0;
        bool launched = false;
        for (Job* j : solo) {
            int ready = 1;
            if (fdtd_engine_query(j->eng, &ready) == FDTD_OK && !ready) {
                ok.push_back(j);
                continue;
            }
            int rc = fdtd_engine_wait(j->eng);  // collects steps that finished since the pass above
            int done = 0;
            uint32_t steps = s->opts.round_steps;
            if (!rc) fdtd_engine_done(j->eng, &done);
            if (!rc && !done && j->opts.end_crit <= 0) {
                // no energy criterion: the job ends after its max_ts
                // timesteps (NumberOfTimesteps), and no round passes them
                uint32_t ts = 0;
                fdtd_engine_num_timesteps(j->eng, &ts);
                if (ts >= j->max_ts) done = 1;
                else steps = std::min(steps, j->max_ts - ts);
            }
            if (!rc && done) {
                retire(s, j, FDTD_OK, "");
                continue;
            }
            if (!rc) rc = fdtd_engine_iterate_async(j->eng, steps);
            if (rc) {
                retire(s, j, rc, last_error());
                continue;
            }
            double ms = 0;
            uint64_t l = 0;
            fdtd_engine_last_timing(j->eng, &ms, &l);
            launches += l;
            launched = true;
            ok.push_back(j);
        }
        if (!bjobs.empty()) {
            bool idle = true;  // a batch needs every one of its engines idle
            for (Job* j : bjobs) {
                int ready = 1;
                if (fdtd_engine_query(j->eng, &ready) == FDTD_OK && !ready) idle = false;
            }
            const std::vector<Job*> left = idle ? batch_round(s, bjobs) : bjobs;  // else collected next pass
            ok.insert(ok.end(), left.begin(), left.end());
        }
        s->active.swap(ok);
        std::lock_guard<std::mutex> lock(s->mu);
        if (launched) {
            s->st.rounds++;
            s->st.kernel_launches += launches;
            if (!busy) {
                busy = true;
                busy_since = Clock::now();
            }
        }
    }
    // shutdown: free what is still resident
    drop_batch(s);
    for (Job* j : s->active) {
        fdtd_engine_wait(j->eng);
        fdtd_engine_destroy(j->eng);
        j->eng = nullptr;
    }
    s->active.clear();
}

Job* find(fdtd_server_s* s, uint64_t id) {
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? nullptr : it->second.get();
}

}  // namespace
}  // namespace wipems

extern "C" {

int fdtd_server_create(const fdtd_server_opts* opts, fdtd_server_t* out) {
    if (!out) return FDTD_ERR_ARG;
    auto s = std::make_unique<fdtd_server_s>();
    if (opts) s->opts = *opts;
    fdtd_server_opts& o = s->opts;
    if (o.max_active == 0) o.max_active = 256;
    if (o.round_steps == 0) o.round_steps = 128;
    if (o.tile_share == 0) o.tile_share = 4;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    // a few concurrent builds of a few threads each (measured on a 16-core
    // host: 4 builds finish the first large jobs sooner than 8 or 16 narrow
    // ones); one core is left to the GPU thread, which relaunches each job
    // as soon as its round completes
    if (o.build_workers <= 0) o.build_workers = (int)std::max(1u, hw / 4);
    if (o.build_threads_per_job <= 0)
        o.build_threads_per_job = (int)std::max(1u, (hw > 1 ? hw - 1 : 1) / (unsigned)o.build_workers);
    CK(cudaSetDevice(o.device));
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    s->budget = o.hbm_budget ? o.hbm_budget : (uint64_t)(0.9 * (double)free_b);
    if (s->budget > free_b) {
        set_error("fdtd_server_create: hbm_budget exceeds the free device memory");
        return FDTD_ERR_ARG;
    }
    s->st.budget_bytes = s->budget;
    s->t0 = Clock::now();
    fdtd_server_s* p = s.get();
    try {
        for (int k = 0; k < o.build_workers; ++k) p->builders.emplace_back(builder_loop, p);
        p->gpu = std::thread(gpu_loop, p);
    } catch (const std::exception& ex) {
        {
            std::lock_guard<std::mutex> lock(p->mu);
            p->stop = true;
        }
        p->cv_build.notify_all();
        p->cv_gpu.notify_all();
        for (auto& t : p->builders) t.join();
        if (p->gpu.joinable()) p->gpu.join();
        set_error(std::string("fdtd_server_create: cannot start threads: ") + ex.what());
        return FDTD_ERR_STATE;
    }
    *out = s.release();
    return FDTD_OK;
}

int fdtd_server_submit(fdtd_server_t s, fdtd_scene_t scene, const fdtd_job_opts* opts, uint64_t* id) {
    if (!s || !scene) {
        set_error("fdtd_server_submit: null argument");
        return FDTD_ERR_ARG;
    }
    auto j = std::make_unique<Job>();
    j->scene = scene;
    if (opts) j->opts = *opts;
    if (j->opts.end_crit < 0) {
        set_error("fdtd_server_submit: end_crit must be >= 0");
        return FDTD_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) {
        set_error("fdtd_server_submit: the server is shutting down");
        return FDTD_ERR_STATE;
    }
    j->id = s->next_id++;
    j->t_submit = s->now();
    if (id) *id = j->id;
    s->build_q.push_back(j.get());
    s->jobs.emplace(j->id, std::move(j));
    s->st.jobs_submitted++;
    s->cv_build.notify_one();
    return FDTD_OK;
}

int fdtd_server_job_status(fdtd_server_t s, uint64_t id, fdtd_job_status* st) {
    if (!s || !st) return FDTD_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    Job* j = find(s, id);
    if (!j) {
        set_error("fdtd_server_job_status: unknown job id");
        return FDTD_ERR_ARG;
    }
    std::memset(st, 0, sizeof(*st));
    st->state = j->state;
    st->error = j->error;
    st->timesteps = j->ts;
    st->num_samples = (uint32_t)j->s_ts.size();
    st->num_probes = (uint32_t)sample_columns(j);
    st->nodes = j->nodes;
    for (int a = 0; a < 3; ++a) st->num_lines[a] = j->N0[a];
    st->dT = j->dT;
    st->footprint = j->footprint;
    st->probe_interval = j->interval;
    st->t_submit = j->t_submit;
    st->t_built = j->t_built;
    st->t_admit = j->t_admit;
    st->t_done = j->t_done;
    if (j->state == FDTD_JOB_FAILED) set_error(j->message);
    return FDTD_OK;
}

int fdtd_server_probe_types(fdtd_server_t s, uint64_t id, int* types, uint32_t cap) {
    if (!s || !types) return FDTD_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    Job* j = find(s, id);
    if (!j) {
        set_error("fdtd_server_probe_types: unknown job id");
        return FDTD_ERR_ARG;
    }
    if (cap < sample_columns(j)) {
        set_error("fdtd_server_probe_types: buffer smaller than the job's sample columns");
        return FDTD_ERR_ARG;
    }
    uint32_t k = 0;
    for (const fdtd_probe_desc& p : j->probes)
        for (int c = 0; c < ((p.type == 2 || p.type == 3) ? 3 : 1); ++c) types[k++] = p.type;
    return FDTD_OK;
}

int fdtd_server_wait(fdtd_server_t s, uint64_t id, double timeout_s) {
    if (!s) return FDTD_ERR_ARG;
    std::unique_lock<std::mutex> lock(s->mu);
    auto finished = [&] {
        if (id == 0) {
            for (auto& kv : s->jobs)
                if (kv.second->state != FDTD_JOB_DONE && kv.second->state != FDTD_JOB_FAILED) return false;
            return true;
        }
        Job* j = find(s, id);
        return !j || j->state == FDTD_JOB_DONE || j->state == FDTD_JOB_FAILED;
    };
    if (id && !find(s, id)) {
        set_error("fdtd_server_wait: unknown job id");
        return FDTD_ERR_ARG;
    }
    if (timeout_s <= 0) {
        s->cv_done.wait(lock, finished);
        return FDTD_OK;
    }
    if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), finished)) {
        set_error("fdtd_server_wait: timed out");
        return FDTD_ERR_TIMEOUT;
    }
    return FDTD_OK;
}

int fdtd_server_read_samples(fdtd_server_t s, uint64_t id, uint32_t* ts, double* vals, double* energy) {
    if (!s) return FDTD_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    Job* j = find(s, id);
    if (!j || j->state != FDTD_JOB_DONE) {
        set_error("fdtd_server_read_samples: job unknown or not finished");
        return FDTD_ERR_STATE;
    }
    const size_t n = j->s_ts.size();
    if (ts) std::copy(j->s_ts.begin(), j->s_ts.end(), ts);
    if (energy) std::copy(j->s_energy.begin(), j->s_energy.end(), energy);
    if (vals) std::copy(j->s_vals.begin(), j->s_vals.begin() + n * sample_columns(j), vals);
    return FDTD_OK;
}

int fdtd_server_get_fields(fdtd_server_t s, uint64_t id, float* volt, float* curr) {
    if (!s) return FDTD_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    Job* j = find(s, id);
    if (!j || j->state != FDTD_JOB_DONE || j->volt.empty()) {
        set_error("fdtd_server_get_fields: job unknown, not finished or submitted without keep_fields");
        return FDTD_ERR_STATE;
    }
    if (volt) std::copy(j->volt.begin(), j->volt.end(), volt);
    if (curr) std::copy(j->curr.begin(), j->curr.end(), curr);
    return FDTD_OK;
}

int fdtd_server_release(fdtd_server_t s, uint64_t id) {
    if (!s) return FDTD_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    Job* j = find(s, id);
    if (!j || (j->state != FDTD_JOB_DONE && j->state != FDTD_JOB_FAILED)) {
        set_error("fdtd_server_release: job unknown or not finished");
        return FDTD_ERR_STATE;
    }
    s->jobs.erase(id);
    return FDTD_OK;
}

int fdtd_server_get_stats(fdtd_server_t s, fdtd_server_stats* st) {
    if (!s || !st) return FDTD_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    *st = s->st;
    st->used_bytes = s->used;
    st->elapsed_s = s->now();
    return FDTD_OK;
}

int fdtd_server_destroy(fdtd_server_t s) {
    if (!s) return FDTD_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_build.notify_all();
    s->cv_gpu.notify_all();
    for (auto& t : s->builders) t.join();
    if (s->gpu.joinable()) s->gpu.join();
    for (auto& kv : s->jobs) {
        Job* j = kv.second.get();
        if (j->scene) fdtd_scene_destroy(j->scene);
        if (j->cop) fdtd_cop_destroy(j->cop);
    }
    delete s;
    return FDTD_OK;
}

}  // extern "C"
