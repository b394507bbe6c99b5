// server.cuh -- continuous-batching request loop over the batch engine.
// Included by batch.cu after batch.cuh; implements the mpmgpu_server_*
// entry points of include/nairn_mpm_gpu.h.
//
// A server owns one batch per dimension (2D plane strain and 3D), sized at
// creation so that both together stay within the HBM budget, and one host
// thread that runs the loop
//
//     admit queued requests that fit (FIFO, least work first, or the
//     deadline order that bounds running requests' predicted slowdown)
//     enqueue `steps_per_round` batched steps on every batch with running runs
//     wait for them, retire finished and failed runs (results written back)
//
// The batches step on their own streams, so 2D and 3D work overlaps on the
// device.  Requests that arrive while others run join at the next round; a
// finished run's slots are compacted away by the next sort.  Each request's
// particle arrays are borrowed: they are read at admission and receive the
// results when the request completes.
#pragma once

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

namespace {

using ServerClock = std::chrono::steady_clock;

struct ServerRequest {
    int64_t id = 0;
    int dim = 2;
    MpmGpuGrid grid{};
    std::vector<double> xn, yn, zn;
    std::vector<MpmGpuMaterial> mats;
    std::vector<MpmGpuVelBC> bcs;
    MpmGpuContact contact{};
    MpmGpuParticles p{};  // borrowed caller arrays
    double dt = 0.;
    int nsteps = 0;
    int state = MPMGPU_REQ_QUEUED;
    int status = MPMGPU_OK;
    int run_id = -1;
    int steps_done = 0;
    std::string msg;
    ServerClock::time_point t_submit, t_admit, t_done;
};

double ms_between(ServerClock::time_point a, ServerClock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

// Step time of one batch as a + b R (ms per step, R resident particles): a
// least-squares line through the rounds' CUDA-event timings, each older round
// weighted down by kModelDecay, with priors until two different loads have
// been seen.
struct StepModel {
    static constexpr double kModelDecay = 0.95;
    double a = 0.1, b = 1e-6;  // priors, replaced by the fit
    double w = 0., sr = 0., srr = 0., st = 0., srt = 0.;
    void add(double R, double t) {
        w = w * kModelDecay + 1.;
        sr = sr * kModelDecay + R;
        srr = srr * kModelDecay + R * R;
        st = st * kModelDecay + t;
        srt = srt * kModelDecay + R * t;
        const double den = w * srr - sr * sr, tm = st / w, rm = sr / w;
        if (w > 2.5 && den > 1e-3 * w * srr) {
            b = (w * srt - sr * st) / den;
            a = (st - b * sr) / w;
        } else {
            a = std::min(a, tm);
            b = rm > 0. ? (tm - a) / rm : b;
        }
        a = std::min(std::max(a, kMinStepMs), tm);
        b = std::max(b, 0.);
    }
    // the resident load at which a step runs at kEfficiency of the batch's
    // asymptotic throughput 1/b: a + b R = b R / kEfficiency
    double efficient_load() const {
        return b > 0. ? a * kEfficiency / (1. - kEfficiency) / b : 1e300;
    }
    static constexpr double kMinStepMs = 0.05;  // a graph-launched step's launch floor
    static constexpr double kEfficiency = 0.9;
};

struct MpmGpuServer {
    MpmGpuServerOptions o{};
    StepModel model[2];
    cudaEvent_t ev[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int device = 0;
    MpmGpuBatch *batch[2] = {nullptr, nullptr};  // [0] 2D, [1] 3D
    int64_t reserved = 0;
    std::mutex mu;
    std::condition_variable wake, done;
    std::deque<ServerRequest *> queue;                                    // admission order
    std::unordered_map<int64_t, std::unique_ptr<ServerRequest>> reqs;   // every unreleased request
    std::vector<ServerRequest *> running[2];
    int64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    MpmGpuServerStats stats{};
    std::string msg;
    std::string loop_error;
};

namespace {

int serr(MpmGpuServer *s, int code, const std::string &m) {
    if (s) s->msg = m;
    else g_static_err = m;
    return code;
}

// largest particle capacity whose batch fits in `bytes`
int64_t server_capacity(MpmGpuBatchOptions o, int64_t bytes, double nodes_per_particle) {
    int64_t lo = 0, hi = (1LL << 31) - 1;
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo + 1) / 2;
        o.max_particles = mid;
        o.max_nodes = std::max<int64_t>(1, (int64_t)(nodes_per_particle * (double)mid));
        if (o.max_nodes > (1LL << 30)) {
            hi = mid - 1;
            continue;
        }
        const int64_t need = mpmgpu_batch_bytes(&o);
        if (need >= 0 && need <= bytes) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

double slowdown_target(const MpmGpuServerOptions &o) { return o.slowdown_target > 0. ? o.slowdown_target : 4.; }

// admission: FIFO per dimension; with backfill a request that does not fit
// now is passed by later ones of its dimension.  The deadline order (2) sorts
// by work with requests already past their bound first, and admits a request
// only while the running requests of its dimension stay within theirs.
void server_admit(MpmGpuServer *s, std::vector<ServerRequest *> &admitted, std::vector<ServerRequest *> &failed) {
    std::vector<ServerRequest *> cand;
    std::vector<MpmGpuRunLoad> load[2];
    const auto now = ServerClock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        cand.assign(s->queue.begin(), s->queue.end());
        for (int d = 0; d < 2; d++)
            for (const ServerRequest *q : s->running[d])
                load[d].push_back({q->p.n, q->nsteps - q->steps_done, q->nsteps, ms_between(q->t_submit, now)});
    }
    const bool deadline = s->o.order == 2;
    const double k = slowdown_target(s->o);
    auto alone_ms = [&](const ServerRequest *q) {
        const StepModel &m = s->model[q->dim == 3 ? 1 : 0];
        return q->nsteps * (m.a + m.b * (double)q->p.n);
    };
    auto late = [&](const ServerRequest *q) { return ms_between(q->t_submit, now) > (k - 1.) * alone_ms(q); };
    if (s->o.order == 1)
        std::stable_sort(cand.begin(), cand.end(), [](const ServerRequest *a, const ServerRequest *b) {
            return (double)a->p.n * a->nsteps < (double)b->p.n * b->nsteps;
        });
    else if (deadline)
        std::stable_sort(cand.begin(), cand.end(), [&](const ServerRequest *a, const ServerRequest *b) {
            const bool la = late(a), lb = late(b);
            if (la != lb) return la;
            if (la) return ms_between(a->t_submit, now) - k * alone_ms(a) > ms_between(b->t_submit, now) - k * alone_ms(b);
            return (double)a->p.n * a->nsteps < (double)b->p.n * b->nsteps;
        });
    int64_t resident = 0;
    for (int d = 0; d < 2; d++)
        for (const ServerRequest *q : s->running[d]) resident += q->p.n;
    bool blocked[2] = {false, false};
    bool capped = false;
    for (ServerRequest *q : cand) {
        const int d = q->dim == 3 ? 1 : 0;
        MpmGpuBatch *b = s->batch[d];
        if (blocked[d]) continue;
        if (deadline) {
            // admitted while the dimension's resident load stays within the
            // model's efficient load (whatever the request's size when nothing
            // runs) and the running requests within their bounds
            double R = 0.;
            for (const MpmGpuRunLoad &u : load[d]) R += (double)u.n;
            const bool fits = R == 0. || R + (double)q->p.n <= s->model[d].efficient_load();
            if (!fits || mpmgpu_server_admits(s->model[d].a, s->model[d].b, k, load[d].data(),
                                              (int32_t)load[d].size(), q->p.n, q->nsteps,
                                              ms_between(q->t_submit, now)) != 1) {
                // a request past its bound waits first: nothing later of its
                // dimension passes it, so the load drains until it fits
                if (late(q)) blocked[d] = true;
                continue;
            }
        }
        if (s->o.max_resident_particles > 0 && resident > 0 && resident + q->p.n > s->o.max_resident_particles) {
            // over the resident cap: wait (or let a smaller later request pass)
            if (!s->o.backfill) capped = true;
            if (capped) break;
            continue;
        }
        int32_t rid = -1;
        const int st = mpmgpu_batch_add_run(b, &q->grid, q->mats.data(), (int32_t)q->mats.size(),
                                            q->bcs.empty() ? nullptr : q->bcs.data(), (int32_t)q->bcs.size(),
                                            q->contact.enabled ? &q->contact : nullptr, &q->p, q->dt, q->nsteps,
                                            &rid);
        if (st == MPMGPU_OK) {
            q->run_id = rid;
            q->t_admit = ServerClock::now();
            admitted.push_back(q);
            resident += q->p.n;
            load[d].push_back({q->p.n, q->nsteps, q->nsteps, ms_between(q->t_submit, now)});
        } else if (st == MPMGPU_ERR_BUSY) {
            MpmGpuBatchInfo bi{};
            mpmgpu_batch_info(b, &bi);
            if (bi.runs == 0) {
                // the batch is empty and the request still does not fit
                q->status = MPMGPU_ERR_OOM;
                q->msg = "request needs more device memory than its share of the HBM budget";
                failed.push_back(q);
            } else if (!s->o.backfill) {
                blocked[d] = true;
            }
        } else {
            q->status = st;
            q->msg = mpmgpu_batch_last_error(b);
            failed.push_back(q);
        }
    }
}

void server_loop(MpmGpuServer *s) {
    cudaSetDevice(s->device);
    const int chunk = s->o.steps_per_round > 0 ? s->o.steps_per_round : 10;
    while (true) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop) break;
            if (s->queue.empty() && s->running[0].empty() && s->running[1].empty()) {
                s->wake.wait_for(lk, std::chrono::milliseconds(50));
                continue;
            }
        }
        std::vector<ServerRequest *> admitted, failed;
        server_admit(s, admitted, failed);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto drop = [&](ServerRequest *q) {
                for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
                    if (*it == q) {
                        s->queue.erase(it);
                        break;
                    }
            };
            for (ServerRequest *q : admitted) {
                drop(q);
                q->state = MPMGPU_REQ_RUNNING;
                s->running[q->dim == 3 ? 1 : 0].push_back(q);
            }
            for (ServerRequest *q : failed) {
                drop(q);
                q->state = MPMGPU_REQ_FAILED;
                q->t_done = ServerClock::now();
                s->stats.failed++;
            }
            if (!failed.empty()) s->done.notify_all();
        }
        bool any = false;
        const auto t0 = ServerClock::now();
        bool launched[2] = {false, false};
        int status[2] = {MPMGPU_OK, MPMGPU_OK};
        // enqueue on both batches first, then wait for both: their steps overlap.
        // Each batch's rounds are timed with events on its stream for the
        // step-time model.
        double load_now[2] = {0., 0.};
        for (int d = 0; d < 2; d++) {
            if (s->running[d].empty()) continue;
            for (const ServerRequest *q : s->running[d]) load_now[d] += (double)q->p.n;
            status[d] = batch_launch(s->batch[d], chunk, s->ev[d][0], &launched[d]);
            if (status[d] == MPMGPU_OK && launched[d] &&
                cudaEventRecord(s->ev[d][1], (cudaStream_t)mpmgpu_batch_stream(s->batch[d])) != cudaSuccess)
                status[d] = MPMGPU_ERR_CUDA;
        }
        for (int d = 0; d < 2; d++)
            if (status[d] == MPMGPU_OK && launched[d]) {
                status[d] = batch_collect(s->batch[d]);
                float ms = 0.f;
                if (status[d] == MPMGPU_OK && cudaEventElapsedTime(&ms, s->ev[d][0], s->ev[d][1]) == cudaSuccess)
                    s->model[d].add(load_now[d], (double)ms / chunk);
            }
        for (int d = 0; d < 2; d++) {
            if (status[d] != MPMGPU_OK) {
                // an error on this batch: its running requests fail.  Their
                // runs leave the batch, so their particle slots, nodes and
                // cells are free again; after a sticky CUDA error the removal
                // fails as well and the batch stays unusable
                const std::string why = mpmgpu_batch_last_error(s->batch[d]);
                for (ServerRequest *q : s->running[d])
                    if (q->run_id >= 0) mpmgpu_batch_remove_run(s->batch[d], q->run_id, nullptr);
                std::lock_guard<std::mutex> lk(s->mu);
                s->loop_error = why;
                for (ServerRequest *q : s->running[d]) {
                    q->state = MPMGPU_REQ_FAILED;
                    q->status = status[d];
                    q->msg = s->loop_error;
                    q->t_done = ServerClock::now();
                    s->stats.failed++;
                }
                s->running[d].clear();
                launched[d] = false;
                s->done.notify_all();
            }
            any = any || launched[d];
        }
        // retire finished and failed runs: results go back into the caller's arrays
        for (int d = 0; d < 2; d++) {
            std::vector<ServerRequest *> keep;
            for (ServerRequest *q : s->running[d]) {
                int32_t st = 0, steps = 0;
                mpmgpu_batch_run_state(s->batch[d], q->run_id, &st, &steps);
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    q->steps_done = steps;
                }
                if (st == MPMGPU_RUN_RUNNING) {
                    keep.push_back(q);
                    continue;
                }
                const int rs = mpmgpu_batch_remove_run(s->batch[d], q->run_id, &q->p);
                std::lock_guard<std::mutex> lk(s->mu);
                q->t_done = ServerClock::now();
                if (st == MPMGPU_RUN_FINISHED && rs == MPMGPU_OK) {
                    q->state = MPMGPU_REQ_DONE;
                    s->stats.completed++;
                    s->stats.particle_steps += q->p.n * (int64_t)q->steps_done;
                } else {
                    q->state = MPMGPU_REQ_FAILED;
                    q->status = rs != MPMGPU_OK ? rs : -st;
                    q->msg = rs != MPMGPU_OK ? mpmgpu_batch_last_error(s->batch[d]) : "run failed on the device";
                    s->stats.failed++;
                }
                s->done.notify_all();
            }
            std::lock_guard<std::mutex> lk(s->mu);
            s->running[d].swap(keep);
        }
        std::lock_guard<std::mutex> lk(s->mu);
        if (any) {
            s->stats.rounds++;
            s->stats.busy_ms += ms_between(t0, ServerClock::now());
        }
    }
    // stopping: requests still queued or running end as failed, and every
    // waiter is woken before the server goes away
    std::lock_guard<std::mutex> lk(s->mu);
    auto stopped = [&](ServerRequest *q) {
        q->state = MPMGPU_REQ_FAILED;
        q->status = MPMGPU_ERR_BUSY;
        q->msg = "server stopped before the request finished";
        q->t_done = ServerClock::now();
        s->stats.failed++;
    };
    for (ServerRequest *q : s->queue) stopped(q);
    s->queue.clear();
    for (int d = 0; d < 2; d++) {
        for (ServerRequest *q : s->running[d]) stopped(q);
        s->running[d].clear();
    }
    s->done.notify_all();
}

// the server's batches and events (not the server itself)
void server_free(MpmGpuServer *s) {
    for (auto *&b : s->batch) {
        mpmgpu_batch_destroy(b);
        b = nullptr;
    }
    for (auto &pair : s->ev)
        for (auto &e : pair)
            if (e) {
                cudaEventDestroy(e);
                e = nullptr;
            }
}

}  // namespace

extern "C" {

int mpmgpu_server_admits(double a_ms, double b_ms, double k, const MpmGpuRunLoad *running, int32_t nrunning,
                         int64_t cand_n, int32_t cand_steps, double cand_waited_ms) {
    if (!(a_ms >= 0.) || !(b_ms >= 0.) || !(k >= 1.) || nrunning < 0 || (nrunning > 0 && !running) || cand_n <= 0 ||
        cand_steps <= 0 || !(cand_waited_ms >= 0.))
        return -MPMGPU_ERR_INVALID;
    if (nrunning == 0) return 1;
    double R = 0.;
    for (int32_t r = 0; r < nrunning; r++) R += (double)running[r].n;
    const double t_now = a_ms + b_ms * R, t_with = a_ms + b_ms * (R + (double)cand_n);
    for (int32_t r = 0; r < nrunning; r++) {
        const MpmGpuRunLoad &u = running[r];
        const double bound = k * u.steps_total * (a_ms + b_ms * (double)u.n);
        if (u.elapsed_ms + u.steps_left * t_now > bound) continue;  // past its bound already: does not block
        if (u.elapsed_ms + u.steps_left * t_with > bound) return 0;
    }
    return 1;
}

int mpmgpu_server_create(const MpmGpuServerOptions *o, MpmGpuServer **out) {
    if (!o || !out) return serr(nullptr, MPMGPU_ERR_INVALID, "mpmgpu_server_create: null argument");
    *out = nullptr;
    if (o->hbm_budget_bytes <= 0 || o->max_runs <= 0 || !(o->frac_3d >= 0. && o->frac_3d <= 1.))
        return serr(nullptr, MPMGPU_ERR_INVALID, "server needs a positive HBM budget, run slots and 0 <= frac_3d <= 1");
    if (o->order < 0 || o->order > 2 || !(o->slowdown_target == 0. || o->slowdown_target >= 1.))
        return serr(nullptr, MPMGPU_ERR_INVALID, "server order must be 0, 1 or 2 and slowdown_target 0 or >= 1");
    auto s = std::make_unique<MpmGpuServer>();
    s->o = *o;
    if (!(s->o.nodes_per_particle > 0.)) s->o.nodes_per_particle = 0.5;
    cudaGetDevice(&s->device);
    // priors of the step-time model until rounds have been timed
    s->model[0].b = 0.7e-6;
    s->model[1].b = 2.0e-6;
    for (auto &pair : s->ev)
        for (auto &e : pair)
            if (cudaEventCreate(&e) != cudaSuccess) {
                for (auto &pr : s->ev)
                    for (auto &x : pr)
                        if (x) cudaEventDestroy(x);
                return serr(nullptr, MPMGPU_ERR_CUDA, "server: cudaEventCreate failed");
            }
    const double frac[2] = {1. - o->frac_3d, o->frac_3d};
    const int np[2] = {MPMGPU_PLANE_STRAIN, MPMGPU_THREED};
    for (int d = 0; d < 2; d++) {
        const int64_t bytes = (int64_t)(frac[d] * (double)o->hbm_budget_bytes);
        if (frac[d] <= 0.) continue;
        MpmGpuBatchOptions bo{};
        bo.np = np[d];
        bo.method = o->method;
        bo.shape = o->shape;
        bo.precision = o->precision;
        bo.sort_interval = o->sort_interval > 0 ? o->sort_interval : 1;
        bo.block = o->block;
        bo.max_runs = o->max_runs;
        bo.max_materials = 4 * o->max_runs;
        bo.max_fields = o->max_fields;
        bo.lr_links = o->lr_links > 0 ? std::min(o->lr_links, d == 1 ? 64 : 16) : 0;
        bo.xpic_order = o->xpic_order;
        bo.xpic_fmpm = o->xpic_fmpm;
        bo.xpic_period = o->xpic_period;
        bo.fraction_usf = o->fraction_usf;
        const int64_t P = server_capacity(bo, bytes, s->o.nodes_per_particle);
        if (P < 1000) {
            server_free(s.get());
            return serr(nullptr, MPMGPU_ERR_INVALID, "HBM budget too small for a batch");
        }
        bo.max_particles = P;
        bo.max_nodes = std::max<int64_t>(1, (int64_t)(s->o.nodes_per_particle * (double)P));
        const int st = mpmgpu_batch_create(&bo, &s->batch[d]);
        if (st != MPMGPU_OK) {
            std::string m = mpmgpu_batch_last_error(nullptr);
            server_free(s.get());
            return serr(nullptr, st, "server batch: " + m);
        }
        s->reserved += mpmgpu_batch_bytes(&bo);
    }
    s->stats.reserved_bytes = s->reserved;
    MpmGpuServer *raw = s.release();
    raw->worker = std::thread(server_loop, raw);
    *out = raw;
    return MPMGPU_OK;
}

int mpmgpu_server_submit(MpmGpuServer *s, const MpmGpuGrid *grid, const MpmGpuMaterial *mats, int32_t nmat,
                         const MpmGpuVelBC *bcs, int32_t nbc, const MpmGpuContact *contact, MpmGpuParticles *p,
                         double timestep, int32_t nsteps, int64_t *request_id) {
    if (!s || !grid || !mats || nmat <= 0 || !p || p->n <= 0 || nbc < 0 || (nbc > 0 && !bcs) || !request_id ||
        nsteps <= 0 || !(timestep > 0.))
        return serr(s, MPMGPU_ERR_INVALID, "mpmgpu_server_submit: bad argument");
    if (grid->dim != 2 && grid->dim != 3) return serr(s, MPMGPU_ERR_INVALID, "grid dim must be 2 or 3");
    if (!s->batch[grid->dim == 3 ? 1 : 0])
        return serr(s, MPMGPU_ERR_UNSUPPORTED, "the server holds no batch for this dimension");
    if (grid->nx < 1 || grid->ny < 1 || (grid->dim == 3 && grid->nz < 1) || !grid->xnodes || !grid->ynodes ||
        (grid->dim == 3 && !grid->znodes))
        return serr(s, MPMGPU_ERR_INVALID, "grid needs element counts and node coordinates");
    auto q = std::make_unique<ServerRequest>();
    q->dim = grid->dim;
    q->grid = *grid;
    q->xn.assign(grid->xnodes, grid->xnodes + grid->nx + 1);
    q->yn.assign(grid->ynodes, grid->ynodes + grid->ny + 1);
    if (grid->dim == 3) q->zn.assign(grid->znodes, grid->znodes + grid->nz + 1);
    q->grid.xnodes = q->xn.data();
    q->grid.ynodes = q->yn.data();
    q->grid.znodes = grid->dim == 3 ? q->zn.data() : nullptr;
    q->mats.assign(mats, mats + nmat);
    if (nbc) q->bcs.assign(bcs, bcs + nbc);
    if (contact) q->contact = *contact;
    q->p = *p;
    q->dt = timestep;
    q->nsteps = nsteps;
    q->t_submit = ServerClock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    q->id = s->next_id++;
    *request_id = q->id;
    s->queue.push_back(q.get());
    s->reqs[q->id] = std::move(q);
    s->stats.submitted++;
    s->wake.notify_all();
    return MPMGPU_OK;
}

int mpmgpu_server_poll(MpmGpuServer *s, int64_t id, MpmGpuRequestInfo *info) {
    if (!s || !info) return MPMGPU_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return serr(s, MPMGPU_ERR_INVALID, "unknown request");
    const ServerRequest &q = *it->second;
    const auto now = ServerClock::now();
    const bool ended = q.state == MPMGPU_REQ_DONE || q.state == MPMGPU_REQ_FAILED;
    const auto end = ended ? q.t_done : now;
    info->state = q.state;
    info->status = q.status;
    info->steps_done = q.steps_done;
    info->pad = 0;
    info->queue_ms = q.state == MPMGPU_REQ_QUEUED || q.run_id < 0 ? ms_between(q.t_submit, end)
                                                                  : ms_between(q.t_submit, q.t_admit);
    info->run_ms = q.run_id >= 0 ? ms_between(q.t_admit, end) : 0.;
    info->total_ms = ms_between(q.t_submit, end);
    return MPMGPU_OK;
}

int mpmgpu_server_wait(MpmGpuServer *s, int64_t id, double timeout_s) {
    if (!s) return MPMGPU_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return serr(s, MPMGPU_ERR_INVALID, "unknown request");
    ServerRequest *q = it->second.get();
    const auto limit = ServerClock::now() + std::chrono::duration_cast<ServerClock::duration>(
                                                std::chrono::duration<double>(std::max(0., timeout_s)));
    const bool ok = s->done.wait_until(lk, limit, [&] {
        return q->state == MPMGPU_REQ_DONE || q->state == MPMGPU_REQ_FAILED;
    });
    if (!ok) return serr(s, MPMGPU_ERR_TIMEOUT, "request not finished within the timeout");
    if (q->state == MPMGPU_REQ_FAILED) {
        s->msg = q->msg;
        return q->status != MPMGPU_OK ? q->status : MPMGPU_ERR_INVALID;
    }
    return MPMGPU_OK;
}

int mpmgpu_server_drain(MpmGpuServer *s, double timeout_s) {
    if (!s) return MPMGPU_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto limit = ServerClock::now() + std::chrono::duration_cast<ServerClock::duration>(
                                                std::chrono::duration<double>(std::max(0., timeout_s)));
    const bool ok = s->done.wait_until(lk, limit, [&] {
        return s->queue.empty() && s->running[0].empty() && s->running[1].empty();
    });
    return ok ? MPMGPU_OK : serr(s, MPMGPU_ERR_TIMEOUT, "requests still pending after the timeout");
}

int mpmgpu_server_release(MpmGpuServer *s, int64_t id) {
    if (!s) return MPMGPU_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return serr(s, MPMGPU_ERR_INVALID, "unknown request");
    if (it->second->state != MPMGPU_REQ_DONE && it->second->state != MPMGPU_REQ_FAILED)
        return serr(s, MPMGPU_ERR_BUSY, "request still queued or running");
    s->reqs.erase(it);
    return MPMGPU_OK;
}

int mpmgpu_server_stats(MpmGpuServer *s, MpmGpuServerStats *out) {
    if (!s || !out) return MPMGPU_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->queued = (int64_t)s->queue.size();
    out->running = (int64_t)(s->running[0].size() + s->running[1].size());
    return MPMGPU_OK;
}

const char *mpmgpu_server_last_error(const MpmGpuServer *s) {
    if (!s) return g_static_err.c_str();
    return !s->loop_error.empty() && s->msg.empty() ? s->loop_error.c_str() : s->msg.c_str();
}

void mpmgpu_server_destroy(MpmGpuServer *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->wake.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    server_free(s);
    delete s;
}

}  // extern "C"
