// Serving loop: Poisson solves and NSCube advances admitted by device-memory
// budget, run concurrently on a set of lanes (CUDA streams), with
// same-geometry solves that wait together merged into one launch sequence
// (continuous batching).  The reference has no counterpart: it solves one
// LaplCube at a time on the caller's thread (src/lapl_cube.h:58-102) and
// steps one NSCube (src/ns_cube.cpp:27-62).
//
// Threads.  Callers submit, poll, wait and cancel from any thread; one
// scheduler thread owns the lanes, the plan pool and every CUDA call on the
// serving path.  A lane's work ends with a host callback that stamps the
// completion time and hands the lane back.  The queue mutex is never held
// across a CUDA call, so a callback never waits on a thread that waits on
// the device.
//
// Memory.  used = staging of the requests in flight (FP64 in + out) + the
// scratch of pooled solver plans + resident session state; a request is
// admitted only if its bytes fit under the budget.  Admission is first come
// first served: a solve that does not fit holds back the requests behind it
// (idle plans are released first), so large requests do not starve.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>
#include <algorithm>

#include "internal.h"
#include "poisson.h"

namespace fdmgpu {
namespace serve {

static double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// solves share a plan (and may share a launch) when their geometry and
// refinement class agree; tol <= 0 selects the plain FP64 form
struct PlanKey {
    int n[3];
    double h[3], l[3];
    int sweeps;  // -1 plain FP64, else mixed refinement sweeps
    bool operator<(const PlanKey& o) const {
        return std::tie(n[0], n[1], n[2], h[0], h[1], h[2], l[0], l[1], l[2], sweeps) <
               std::tie(o.n[0], o.n[1], o.n[2], o.h[0], o.h[1], o.h[2], o.l[0], o.l[1], o.l[2], o.sweeps);
    }
    bool operator==(const PlanKey& o) const { return !(*this < o) && !(o < *this); }
};

// refinement sweeps of the mixed form for a tolerance (as CubePlan)
static int sweeps_for(double tol) { return tol <= 0 ? -1 : (tol >= 1e-5 ? 0 : (tol >= 1e-11 ? 1 : 2)); }

// the tolerance a plan of a sweep class is configured with
static double tol_for(int sweeps) { return sweeps == 0 ? 1e-5 : (sweeps == 1 ? 1e-10 : 1e-13); }

struct Request {
    unsigned long long id = 0;
    int kind = FDMGPU_REQ_SOLVE;
    int state = FDMGPU_REQ_QUEUED;
    int status = FDMGPU_OK;
    std::string error;
    // solve
    PlanKey key{};
    long long vol = 0;
    const double* rhs = nullptr;
    double* ans = nullptr;
    // advance
    int session = -1;
    int steps = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int batch = 1;  // requests in the launch this one ran in
    double err_est = -1.0;  // solves: estimated relative error of the answer (-1: none)
};

struct Plan {
    PlanKey key;
    fdmgpu_lapl_cube* h = nullptr;
    size_t bytes = 0;
    double last_used = 0;
    ~Plan() {
        if (h) fdmgpu_lapl_cube_destroy(h);
    }
};

struct Session {
    fdmgpu_nscube* h = nullptr;
    cudaStream_t st = nullptr;  // the session's own stream: its steps stay in order
    size_t bytes = 0;
    bool busy = false;
    bool closing = false;
    long long steps_done = 0;
    ~Session() {
        if (st) cudaStreamSynchronize(st);
        if (h) fdmgpu_nscube_destroy(h);
        if (st) cudaStreamDestroy(st);
    }
};

struct Server;

struct Lane {
    Server* srv = nullptr;
    int index = 0;
    cudaStream_t st = nullptr;
    bool busy = false;
    std::vector<Request*> reqs;
    std::unique_ptr<Plan> plan;  // plan in use (solves)
    size_t staged = 0;           // staging bytes reserved by this launch
    double t_done = 0;
    double* norms_host = nullptr;  // page-locked copy of the launch's refinement norms
    cudaEvent_t ev = nullptr;      // orders shared cavity steps against the sessions' streams
    int sweeps = 0;                // sweeps of the launch's solve (0: none, -1: FP64)
};

struct Server {
    double budget = 0;
    int max_batch = 8;
    std::vector<Lane> lanes;
    cudaMemPool_t pool = nullptr;
    int device = 0;

    std::mutex mq;
    std::condition_variable cv_sched, cv_done;
    std::deque<Request*> pending;
    std::unordered_map<unsigned long long, std::unique_ptr<Request>> reqs;
    std::vector<Lane*> completed;
    std::deque<unsigned long long> finished;  // finished request ids, in completion order
    std::map<int, std::unique_ptr<Session>> sessions;
    std::multimap<PlanKey, std::unique_ptr<Plan>> idle;
    int next_session = 0;
    unsigned long long next_id = 1;
    bool stop = false;
    std::thread thread;

    // accounting (under mq)
    double used = 0, peak = 0, plan_bytes = 0, session_bytes = 0, staged_bytes = 0;
    int running = 0;
    unsigned long long n_submitted = 0, n_completed = 0, n_failed = 0, n_cancelled = 0, n_rejected = 0;
    unsigned long long n_shed = 0;
    int max_queued = 0;      // > 0: submits find the queue full at this length (EBUSY)
    double max_wait_ms = 0;  // > 0: queued requests are shed after this wait (EBUSY)
    unsigned long long n_batches = 0, n_batched = 0;
    std::vector<float> lat_solve, lat_advance;
    double queue_sum = 0;
    unsigned long long queue_n = 0;

    void account(double delta) {
        used += delta;
        if (used > peak) peak = used;
    }

    static void CUDART_CB on_done(void* p) {
        Lane* L = (Lane*)p;
        Server* s = L->srv;
        std::lock_guard<std::mutex> g(s->mq);
        L->t_done = now_ms();
        s->completed.push_back(L);
        s->cv_sched.notify_one();
    }

    // staging bytes of a solve: the FP64 input and output volumes
    static double staging_bytes(const Request& r) { return 16.0 * (double)r.vol; }

    // scratch a plan of this key needs for nrhs volumes (FP32 work, high
    // and low parts of the FP32 solution; plain FP64 solves in place)
    static double plan_need(const PlanKey& k, long long vol, int nrhs) {
        if (k.sweeps < 0) return 0.0;
        const double per = k.sweeps == 0 ? 4.0 : (k.sweeps == 1 ? 8.0 : 12.0);
        return per * (double)vol * nrhs + 64.0 * 1024 * 1024;  // + tables, norms
    }

    void finish_lane(Lane* L) {  // under mq; no CUDA calls
        // per-request error estimates of a solve launch from the norms the
        // lane copied back (host arithmetic)
        if (L->plan && !L->reqs.empty() && L->reqs[0]->kind == FDMGPU_REQ_SOLVE) {
            const int nb = (int)L->reqs.size();
            if (L->sweeps > 0) {
                std::vector<double> est((size_t)nb);
                cube_estimates(L->plan->h, L->norms_host, L->sweeps, nb, est.data());
                for (int i = 0; i < nb; i++) L->reqs[i]->err_est = est[i];
            } else {
                // FP64 solves (tol <= 0, or a mixed plan beyond its
                // conditioning limit) carry no refinement error
                for (Request* r : L->reqs) r->err_est = (r->key.sweeps < 0 || L->sweeps < 0) ? 0.0 : -1.0;
            }
        }
        for (Request* r : L->reqs) {
            r->t_done = L->t_done;
            finished.push_back(r->id);
            if (r->state == FDMGPU_REQ_RUNNING) {
                r->state = FDMGPU_REQ_DONE;
                n_completed++;
                const float lat = (float)(r->t_done - r->t_submit);
                (r->kind == FDMGPU_REQ_SOLVE ? lat_solve : lat_advance).push_back(lat);
            }
            if (r->kind == FDMGPU_REQ_ADVANCE) {
                auto it = sessions.find(r->session);
                if (it != sessions.end()) {
                    it->second->busy = false;
                    if (r->state == FDMGPU_REQ_DONE) it->second->steps_done += r->steps;
                }
            }
        }
        account(-(double)L->staged);
        staged_bytes -= (double)L->staged;
        L->staged = 0;
        if (L->plan) {
            L->plan->last_used = now_ms();
            PlanKey k = L->plan->key;
            idle.emplace(k, std::move(L->plan));
        }
        L->reqs.clear();
        L->busy = false;
        running--;
        cv_done.notify_all();
    }

    void fail(Request* r, int code, const std::string& msg) {  // under mq
        r->state = FDMGPU_REQ_FAILED;
        r->status = code;
        r->error = msg;
        n_failed++;
    }

    // Sheds the queued requests that waited past max_wait_ms (under mq).
    // The queue is in submission order, so the expired ones lead it.
    // Returns the ms until the next one expires (< 0: none queued).
    double shed_expired() {
        if (max_wait_ms <= 0) return -1.0;
        const double t = now_ms();
        while (!pending.empty() && t - pending.front()->t_submit >= max_wait_ms) {
            Request* r = pending.front();
            pending.pop_front();
            r->state = FDMGPU_REQ_FAILED;
            r->status = FDMGPU_EBUSY;
            r->error = "shed: not started within the queue deadline";
            r->t_done = t;
            n_shed++;
            finished.push_back(r->id);
        }
        if (pending.empty()) return -1.0;
        return pending.front()->t_submit + max_wait_ms - t;
    }

    // What the scheduler does next (chosen under mq, carried out without it)
    struct Action {
        Lane* lane = nullptr;
        std::vector<Request*> batch;
        std::unique_ptr<Plan> plan;  // pooled plan to reuse (solves)
        std::vector<fdmgpu_nscube*> cavities;  // advances: the sessions' cavities
        std::vector<cudaStream_t> streams;     // and their streams
        std::vector<std::unique_ptr<Plan>> evict;
        double plan_grow = 0;
    };

    Lane* free_lane() {
        for (auto& L : lanes)
            if (!L.busy) return &L;
        return nullptr;
    }

    // Picks the next launch: the oldest admissible request, plus for a
    // solve the later waiting solves of the same plan key (up to max_batch)
    // that still fit, and for an advance the first waiting advance of each
    // other idle session of the same cavity geometry (up to max_batch): their
    // steps share launches.  Returns false when nothing can start now.
    bool pick(Action& a) {
        Lane* L = free_lane();
        if (!L) return false;
        for (auto it = pending.begin(); it != pending.end(); ++it) {
            Request* r = *it;
            if (r->kind == FDMGPU_REQ_ADVANCE) {
                auto s = sessions.find(r->session);
                if (s == sessions.end()) {
                    fail(r, FDMGPU_EINVAL, "session was closed");
                    finished.push_back(r->id);
                    pending.erase(it);
                    cv_done.notify_all();
                    return pick(a);
                }
                if (s->second->busy) continue;  // keeps the session's order
                s->second->busy = true;
                a.lane = L;
                a.batch.push_back(r);
                a.cavities.push_back(s->second->h);
                auto next = pending.erase(it);
                for (auto j = next; j != pending.end() && (int)a.batch.size() < max_batch;) {
                    Request* q = *j;
                    auto t = q->kind == FDMGPU_REQ_ADVANCE ? sessions.find(q->session) : sessions.end();
                    if (t == sessions.end() || t->second->busy || !nscube_mergeable(a.cavities[0], t->second->h)) {
                        ++j;
                        continue;
                    }
                    t->second->busy = true;  // one advance per session and launch
                    a.batch.push_back(q);
                    a.cavities.push_back(t->second->h);
                    a.streams.push_back(t->second->st);
                    j = pending.erase(j);
                }
                a.streams.insert(a.streams.begin(), s->second->st);
                return true;
            }
            // solve: first come first served on memory
            double need = staging_bytes(*r);
            auto pit = idle.find(r->key);
            const double have = pit != idle.end() ? (double)pit->second->bytes : 0.0;
            double grow = std::max(0.0, plan_need(r->key, r->vol, 1) - have);
            if (used + need + grow > budget) {
                // release idle plans (least recently used first) of other keys
                std::vector<std::multimap<PlanKey, std::unique_ptr<Plan>>::iterator> cand;
                for (auto i = idle.begin(); i != idle.end(); ++i)
                    if (!(i->first == r->key)) cand.push_back(i);
                std::sort(cand.begin(), cand.end(),
                          [](const auto& x, const auto& y) { return x->second->last_used < y->second->last_used; });
                double freed = 0;
                for (auto& i : cand) {
                    if (used - freed + need + grow <= budget) break;
                    freed += (double)i->second->bytes;
                    a.evict.push_back(std::move(i->second));
                    idle.erase(i);
                }
                plan_bytes -= freed;
                account(-freed);
                if (used + need + grow > budget) return !a.evict.empty();  // wait for running work
            }
            a.lane = L;
            a.batch.push_back(r);
            auto next = pending.erase(it);
            if (pit != idle.end()) {
                a.plan = std::move(pit->second);
                idle.erase(pit);
            }
            // continuous batching: later solves of the same key join
            double total = need;
            int nb = 1;
            for (auto j = next; j != pending.end() && nb < max_batch;) {
                Request* q = *j;
                if (q->kind == FDMGPU_REQ_SOLVE && q->key == r->key) {
                    const double g2 = std::max(0.0, plan_need(r->key, r->vol, nb + 1) - have);
                    if (used + total + staging_bytes(*q) + g2 > budget) break;
                    total += staging_bytes(*q);
                    grow = g2;
                    a.batch.push_back(q);
                    nb++;
                    j = pending.erase(j);
                } else {
                    ++j;
                }
            }
            a.plan_grow = grow;
            L->staged = (size_t)total;
            staged_bytes += total;
            account(total + grow);  // plan growth is corrected after the launch
            plan_bytes += grow;
            return true;
        }
        return false;
    }

    // Issues one launch on its lane (scheduler thread, mq not held).
    void issue(Action& a) {
        Lane* L = a.lane;
        const double t = now_ms();
        for (Request* r : a.batch) {
            r->t_start = t;
            r->batch = (int)a.batch.size();
        }
        std::string err;
        int code = FDMGPU_OK;
        cudaStream_t cb = L->st;
        if (a.batch[0]->kind == FDMGPU_REQ_ADVANCE && a.batch.size() == 1) {
            // the session's own stream; the lane is the concurrency slot
            cb = a.streams[0];
            code = fdmgpu_nscube_step(a.cavities[0], a.batch[0]->steps);
            if (code) err = fdmgpu_last_error();
        } else if (a.batch[0]->kind == FDMGPU_REQ_ADVANCE) {
            code = run_advances(a, err);
        } else {
            code = run_solves(a, err);
        }
        size_t plan_real = 0;
        if (a.plan) fdmgpu_lapl_cube_scratch_bytes(a.plan->h, &plan_real);
        if (!code) {
            cudaError_t e = cudaLaunchHostFunc(cb, on_done, L);
            if (e != cudaSuccess) {
                code = FDMGPU_ECUDA;
                err = std::string("cudaLaunchHostFunc failed: ") + cudaGetErrorString(e);
            }
        }
        // a failed launch completes through no callback: drain its stream
        // before the lane is handed back (outside the lock: callbacks of
        // other lanes take it)
        if (code) cudaStreamSynchronize(cb);
        std::lock_guard<std::mutex> g(mq);
        L->busy = true;
        running++;
        L->reqs = a.batch;
        if (a.plan) {
            // the plan's real scratch replaces the estimate
            const double est = (double)a.plan->bytes + a.plan_grow;
            plan_bytes += (double)plan_real - est;
            account((double)plan_real - est);
            a.plan->bytes = plan_real;
            L->plan = std::move(a.plan);
        } else {
            plan_bytes -= a.plan_grow;
            account(-a.plan_grow);
        }
        if (a.batch[0]->kind == FDMGPU_REQ_SOLVE) {
            n_batches++;
            n_batched += a.batch.size();
        }
        for (Request* r : a.batch) r->state = FDMGPU_REQ_RUNNING;
        if (code) {
            // nothing of this launch completes through the callback: the
            // lane's stream is drained before the lane is handed back
            for (Request* r : a.batch) fail(r, code, err);
            L->t_done = now_ms();
            finish_lane(L);
        }
    }

    // Advances of several sessions of one cavity geometry: each step's
    // kernels take all the cavities that still have steps to go, on the
    // lane's stream, ordered after and before the sessions' own streams.
    int run_advances(Action& a, std::string& err) {
        Lane* L = a.lane;
        const int n = (int)a.batch.size();
        std::vector<int> steps((size_t)n);
        for (int i = 0; i < n; i++) steps[i] = a.batch[i]->steps;
        cudaError_t e = cudaSuccess;
        for (int i = 0; e == cudaSuccess && i < n; i++) {
            e = cudaEventRecord(L->ev, a.streams[i]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(L->st, L->ev, 0);
        }
        if (e != cudaSuccess) {
            err = std::string("ordering the sessions' streams failed: ") + cudaGetErrorString(e);
            return FDMGPU_ECUDA;
        }
        int code = FDMGPU_OK;
        try {
            nscube_step_many(a.cavities.data(), steps.data(), n, L->st, pool);
        } catch (const Error& x) {
            err = fdmgpu_last_error();
            code = x.code;
        } catch (const std::bad_alloc&) {
            err = "host allocation failed";
            code = FDMGPU_ENOMEM;
        }
        // the sessions' later work follows the shared steps
        e = cudaEventRecord(L->ev, L->st);
        for (int i = 0; e == cudaSuccess && i < n; i++) e = cudaStreamWaitEvent(a.streams[i], L->ev, 0);
        if (e != cudaSuccess && !code) {
            err = std::string("ordering the sessions' streams failed: ") + cudaGetErrorString(e);
            code = FDMGPU_ECUDA;
        }
        return code;
    }

    int run_solves(Action& a, std::string& err) {
        Lane* L = a.lane;
        Request* r0 = a.batch[0];
        const PlanKey& k = r0->key;
        const int nb = (int)a.batch.size();
        int code = FDMGPU_OK;
        if (!a.plan) {
            std::unique_ptr<Plan> p(new Plan());
            p->key = k;
            code = fdmgpu_lapl_cube_create(&p->h, FDMGPU_F64, FDMGPU_DIRICHLET, k.h[0], k.h[1], k.h[2], k.l[0],
                                           k.l[1], k.l[2], k.n[0], k.n[1], k.n[2]);
            if (!code)
                code = fdmgpu_lapl_cube_set_precision(p->h, k.sweeps < 0 ? FDMGPU_PLAIN : FDMGPU_MIXED,
                                                      tol_for(k.sweeps), 3);
            if (code) {
                err = fdmgpu_last_error();
                return code;
            }
            a.plan = std::move(p);
        }
        const size_t vb = (size_t)r0->vol * sizeof(double);
        void *din = nullptr, *dout = nullptr;
        cudaError_t e = cudaMallocFromPoolAsync(&din, vb * nb, pool, L->st);
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&dout, vb * nb, pool, L->st);
        for (int i = 0; e == cudaSuccess && i < nb; i++)
            e = cudaMemcpyAsync((char*)din + vb * i, a.batch[i]->rhs, vb, cudaMemcpyHostToDevice, L->st);
        if (e != cudaSuccess) {
            err = std::string("staging failed: ") + cudaGetErrorString(e);
            if (din) cudaFreeAsync(din, L->st);
            if (dout) cudaFreeAsync(dout, L->st);
            return e == cudaErrorMemoryAllocation ? FDMGPU_ENOMEM : FDMGPU_ECUDA;
        }
        code = fdmgpu_lapl_cube_solve_device(a.plan->h, dout, din, nb, L->st);
        if (code) err = fdmgpu_last_error();
        L->sweeps = 0;
        if (!code) {
            try {
                L->sweeps = cube_norms_async(a.plan->h, L->norms_host, nb, L->st);
            } catch (const Error& ex) {
                code = ex.code;
                err = fdmgpu_last_error();
            }
        }
        for (int i = 0; !code && i < nb; i++) {
            e = cudaMemcpyAsync(a.batch[i]->ans, (char*)dout + vb * i, vb, cudaMemcpyDeviceToHost, L->st);
            if (e != cudaSuccess) {
                code = FDMGPU_ECUDA;
                err = std::string("copy-out failed: ") + cudaGetErrorString(e);
            }
        }
        cudaFreeAsync(din, L->st);
        cudaFreeAsync(dout, L->st);
        return code;
    }

    void loop() {
        std::unique_lock<std::mutex> lk(mq);
        while (true) {
            while (!completed.empty()) {
                Lane* L = completed.back();
                completed.pop_back();
                finish_lane(L);
            }
            if (stop && running == 0) break;
            const size_t nfin = finished.size();
            const double next_expiry = shed_expired();
            if (finished.size() != nfin) cv_done.notify_all();
            Action a;
            if (!stop && pick(a)) {
                lk.unlock();
                a.evict.clear();  // destroys released plans (CUDA frees) outside the lock
                if (a.lane && !a.batch.empty()) issue(a);
                lk.lock();
                continue;
            }
            if (next_expiry >= 0)
                cv_sched.wait_for(lk, std::chrono::microseconds((long long)(next_expiry * 1e3) + 1));
            else
                cv_sched.wait(lk);
        }
    }

    void start(int nlanes) {
        FDM_CUDA(cudaGetDevice(&device));
        cudaMemPoolProps props;
        memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        FDM_CUDA(cudaMemPoolCreate(&pool, &props));
        // freed staging stays cached in the pool up to the budget
        unsigned long long keep = (unsigned long long)budget;
        FDM_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        lanes.resize(nlanes);
        for (int i = 0; i < nlanes; i++) {
            lanes[i].srv = this;
            lanes[i].index = i;
            FDM_CUDA(cudaStreamCreateWithFlags(&lanes[i].st, cudaStreamNonBlocking));
            // refinement norms of one launch: 2 doubles per right-hand side
            // per sweep (at most 3 sweeps)
            FDM_CUDA(cudaHostAlloc(&lanes[i].norms_host, sizeof(double) * 2 * 3 * (size_t)max_batch,
                                   cudaHostAllocDefault));
            FDM_CUDA(cudaEventCreateWithFlags(&lanes[i].ev, cudaEventDisableTiming));
        }
        thread = std::thread([this] { loop(); });
    }

    void shutdown() {
        {
            std::lock_guard<std::mutex> g(mq);
            stop = true;
            for (Request* r : pending) {
                r->state = FDMGPU_REQ_CANCELLED;
                n_cancelled++;
                finished.push_back(r->id);
            }
            pending.clear();
            cv_sched.notify_one();
        }
        if (thread.joinable()) thread.join();
        idle.clear();
        sessions.clear();
        for (auto& L : lanes) {
            if (L.st) cudaStreamDestroy(L.st);
            if (L.norms_host) cudaFreeHost(L.norms_host);
            if (L.ev) cudaEventDestroy(L.ev);
        }
        if (pool) cudaMemPoolDestroy(pool);
    }

    static void percentiles(std::vector<float> v, double* p50, double* p99) {
        if (v.empty()) {
            *p50 = *p99 = 0;
            return;
        }
        std::sort(v.begin(), v.end());
        auto q = [&](double f) {
            size_t i = (size_t)std::ceil(f * v.size());
            return (double)v[std::min(v.size() - 1, i > 0 ? i - 1 : 0)];
        };
        *p50 = q(0.50);
        *p99 = q(0.99);
    }
};

}  // namespace serve
}  // namespace fdmgpu

using namespace fdmgpu;
using namespace fdmgpu::serve;

struct fdmgpu_server {
    Server s;
};

static void read_request(const Request& r, int* state, int* status, double* latency_ms, double* queue_ms,
                         int* batch, double* err_est) {
    if (err_est) *err_est = r.state == FDMGPU_REQ_DONE ? r.err_est : -1.0;
    if (state) *state = r.state;
    if (status) *status = r.status;
    const bool fin = r.state == FDMGPU_REQ_DONE || r.state == FDMGPU_REQ_FAILED;
    if (latency_ms) *latency_ms = fin ? r.t_done - r.t_submit : -1.0;
    if (queue_ms) *queue_ms = r.t_start > 0 ? r.t_start - r.t_submit : -1.0;
    if (batch) *batch = r.batch;
}

static bool final_state(int st) {
    return st == FDMGPU_REQ_DONE || st == FDMGPU_REQ_FAILED || st == FDMGPU_REQ_CANCELLED;
}

// hands a finished request's record back (under mq)
static void retire(Server& s, unsigned long long id) {
    auto it = s.reqs.find(id);
    if (it == s.reqs.end()) return;
    if (it->second->t_start > 0) {
        s.queue_sum += it->second->t_start - it->second->t_submit;
        s.queue_n++;
    }
    if (it->second->state == FDMGPU_REQ_FAILED) set_error("%s", it->second->error.c_str());
    s.reqs.erase(it);
}

// blocks until the session has no queued or running advance, then runs fn
template <typename Fn>
static int with_idle_session(Server& s, int session, double timeout_ms, Fn fn) {
    std::unique_lock<std::mutex> lk(s.mq);
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double, std::milli>(timeout_ms);
    while (true) {
        auto it = s.sessions.find(session);
        if (it == s.sessions.end()) FDM_FAIL(FDMGPU_EINVAL, "no session %d", session);
        bool queued = false;
        for (Request* r : s.pending)
            if (r->kind == FDMGPU_REQ_ADVANCE && r->session == session) queued = true;
        if (!it->second->busy && !queued) return fn(*it->second, lk);
        if (s.cv_done.wait_until(lk, until) == std::cv_status::timeout)
            FDM_FAIL(FDMGPU_ETIMEOUT, "session %d still busy after %.0f ms", session, timeout_ms);
    }
}

extern "C" {

int fdmgpu_server_create(fdmgpu_server** h, double budget_bytes, int lanes, int max_batch) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (!(budget_bytes > 0) || lanes < 1 || lanes > 64 || max_batch < 1 || max_batch > 64)
        FDM_FAIL(FDMGPU_EINVAL, "budget must be positive, lanes and max_batch in [1, 64]");
    std::unique_ptr<fdmgpu_server> p(new fdmgpu_server());
    p->s.budget = budget_bytes;
    p->s.max_batch = max_batch;
    p->s.start(lanes);
    *h = p.release();
    FDM_API_END
}

int fdmgpu_server_submit_solve(fdmgpu_server* h, unsigned long long* id, const int* n3, const double* h3,
                               const double* l3, double tol, const double* rhs, double* ans) {
    FDM_API_BEGIN
    if (!h || !id || !n3 || !h3 || !l3 || !rhs || !ans) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    Server& s = h->s;
    std::unique_ptr<Request> r(new Request());
    r->kind = FDMGPU_REQ_SOLVE;
    r->vol = 1;
    for (int a = 0; a < 3; a++) {
        const int n = n3[a];
        if (n < 1 || n > FDMGPU_MAX_N || ((n + 1) & n))
            FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: n=%d on axis %d", n, a);
        if (!(h3[a] > 0 && l3[a] > 0)) FDM_FAIL(FDMGPU_EINVAL, "spacings and lengths must be positive");
        r->key.n[a] = n;
        r->key.h[a] = h3[a];
        r->key.l[a] = l3[a];
        r->vol *= n;
    }
    r->key.sweeps = sweeps_for(tol);
    for (const void* p : {(const void*)rhs, (const void*)ans}) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            FDM_FAIL(FDMGPU_EINVAL, "request buffers must be page-locked host memory (cudaHostAlloc / cudaHostRegister)");
        }
    }
    r->rhs = rhs;
    r->ans = ans;
    const double need = Server::staging_bytes(*r) + Server::plan_need(r->key, r->vol, 1);
    std::lock_guard<std::mutex> g(s.mq);
    if (s.stop) FDM_FAIL(FDMGPU_EINVAL, "server is shutting down");
    if (s.max_queued > 0 && (int)s.pending.size() >= s.max_queued) {
        s.n_shed++;
        FDM_FAIL(FDMGPU_EBUSY, "queue full (%d requests)", s.max_queued);
    }
    if (need + s.session_bytes > s.budget) {
        s.n_rejected++;
        FDM_FAIL(FDMGPU_EBUDGET, "request needs %.0f bytes, budget %.0f (%.0f held by sessions)", need, s.budget,
                 s.session_bytes);
    }
    r->id = s.next_id++;
    r->t_submit = now_ms();
    *id = r->id;
    s.pending.push_back(r.get());
    s.reqs.emplace(r->id, std::move(r));
    s.n_submitted++;
    s.cv_sched.notify_one();
    FDM_API_END
}

int fdmgpu_server_session_create(fdmgpu_server* h, int* session, int nx, int nz, double x1, double y1, double z1,
                                 double x2, double y2, double z2, double u0, double Re, double dt) {
    FDM_API_BEGIN
    if (!h || !session) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    Server& s = h->s;
    // nine fields and the pressure solve's work volume, plus the work volume
    // of steps shared with other sessions
    const double bytes = 11.0 * (nx + 3.0) * (nx + 3.0) * (nz + 3.0) * sizeof(double);
    {
        std::lock_guard<std::mutex> g(s.mq);
        if (s.used + bytes > s.budget) FDM_FAIL(FDMGPU_EBUDGET, "session state does not fit in the budget");
        s.account(bytes);
        s.session_bytes += bytes;
    }
    std::unique_ptr<Session> ss(new Session());
    ss->bytes = (size_t)bytes;
    int rc = fdmgpu_nscube_create(&ss->h, FDMGPU_F64, nx, nz, x1, y1, z1, x2, y2, z2, u0, Re, dt);
    if (!rc) {
        if (cudaStreamCreateWithFlags(&ss->st, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaStreamCreateWithFlags failed");
            rc = FDMGPU_ECUDA;
        } else {
            rc = fdmgpu_nscube_set_stream(ss->h, ss->st);
        }
    }
    std::lock_guard<std::mutex> g(s.mq);
    if (rc) {
        s.account(-bytes);
        s.session_bytes -= bytes;
        return rc;
    }
    const int id = s.next_session++;
    s.sessions.emplace(id, std::move(ss));
    *session = id;
    FDM_API_END
}

int fdmgpu_server_submit_advance(fdmgpu_server* h, unsigned long long* id, int session, int steps) {
    FDM_API_BEGIN
    if (!h || !id) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (steps < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
    Server& s = h->s;
    std::lock_guard<std::mutex> g(s.mq);
    if (s.stop) FDM_FAIL(FDMGPU_EINVAL, "server is shutting down");
    auto it = s.sessions.find(session);
    if (it == s.sessions.end() || it->second->closing) FDM_FAIL(FDMGPU_EINVAL, "no session %d", session);
    if (s.max_queued > 0 && (int)s.pending.size() >= s.max_queued) {
        s.n_shed++;
        FDM_FAIL(FDMGPU_EBUSY, "queue full (%d requests)", s.max_queued);
    }
    std::unique_ptr<Request> r(new Request());
    r->kind = FDMGPU_REQ_ADVANCE;
    r->session = session;
    r->steps = steps;
    r->id = s.next_id++;
    r->t_submit = now_ms();
    *id = r->id;
    s.pending.push_back(r.get());
    s.reqs.emplace(r->id, std::move(r));
    s.n_submitted++;
    s.cv_sched.notify_one();
    FDM_API_END
}

int fdmgpu_server_poll(fdmgpu_server* h, unsigned long long id, int* state, int* status, double* latency_ms,
                       double* queue_ms, int* batch, double* err_est) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    Server& s = h->s;
    std::lock_guard<std::mutex> g(s.mq);
    auto it = s.reqs.find(id);
    if (it == s.reqs.end()) FDM_FAIL(FDMGPU_EINVAL, "no request %llu (finished requests are reported once)", id);
    read_request(*it->second, state, status, latency_ms, queue_ms, batch, err_est);
    if (final_state(it->second->state)) retire(s, id);
    FDM_API_END
}

int fdmgpu_server_wait(fdmgpu_server* h, unsigned long long id, double timeout_ms, int* state, int* status,
                       double* latency_ms, double* queue_ms, int* batch, double* err_est) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    Server& s = h->s;
    std::unique_lock<std::mutex> lk(s.mq);
    auto it = s.reqs.find(id);
    if (it == s.reqs.end()) FDM_FAIL(FDMGPU_EINVAL, "no request %llu (finished requests are reported once)", id);
    Request* r = it->second.get();
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double, std::milli>(timeout_ms);
    while (!final_state(r->state)) {
        if (s.cv_done.wait_until(lk, until) == std::cv_status::timeout && !final_state(r->state)) {
            read_request(*r, state, status, latency_ms, queue_ms, batch, err_est);
            FDM_FAIL(FDMGPU_ETIMEOUT, "request %llu not finished after %.0f ms", id, timeout_ms);
        }
    }
    read_request(*r, state, status, latency_ms, queue_ms, batch, err_est);
    retire(s, id);
    FDM_API_END
}

int fdmgpu_server_cancel(fdmgpu_server* h, unsigned long long id) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    Server& s = h->s;
    std::lock_guard<std::mutex> g(s.mq);
    auto it = s.reqs.find(id);
    if (it == s.reqs.end()) FDM_FAIL(FDMGPU_EINVAL, "no request %llu", id);
    Request* r = it->second.get();
    if (r->state != FDMGPU_REQ_QUEUED) FDM_FAIL(FDMGPU_EINVAL, "request %llu already started", id);
    s.pending.erase(std::find(s.pending.begin(), s.pending.end(), r));
    r->state = FDMGPU_REQ_CANCELLED;
    s.n_cancelled++;
    s.finished.push_back(id);
    s.cv_done.notify_all();
    FDM_API_END
}

int fdmgpu_server_next_done(fdmgpu_server* h, double timeout_ms, unsigned long long* id, int* state, int* status,
                            double* latency_ms, double* queue_ms, int* batch, double* err_est) {
    FDM_API_BEGIN
    if (!h || !id) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    Server& s = h->s;
    std::unique_lock<std::mutex> lk(s.mq);
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double, std::milli>(timeout_ms);
    while (true) {
        while (!s.finished.empty()) {
            const unsigned long long f = s.finished.front();
            s.finished.pop_front();
            auto it = s.reqs.find(f);
            if (it == s.reqs.end()) continue;  // already reported by poll or wait
            *id = f;
            read_request(*it->second, state, status, latency_ms, queue_ms, batch, err_est);
            retire(s, f);
            return FDMGPU_OK;
        }
        if (s.cv_done.wait_until(lk, until) == std::cv_status::timeout && s.finished.empty())
            FDM_FAIL(FDMGPU_ETIMEOUT, "no request finished within %.0f ms", timeout_ms);
    }
    FDM_API_END
}

int fdmgpu_server_session_get_field(fdmgpu_server* h, int session, int field, double* out, size_t count,
                                    long long* steps_done, double timeout_ms) {
    FDM_API_BEGIN
    if (!h || !out) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    int rc = with_idle_session(h->s, session, timeout_ms, [&](Session& ss, std::unique_lock<std::mutex>&) {
        if (steps_done) *steps_done = ss.steps_done;
        ss.busy = true;  // no advance starts while the field is read
        return 0;
    });
    if (rc) return rc;
    fdmgpu_nscube* nh = nullptr;
    {
        std::lock_guard<std::mutex> g(h->s.mq);
        nh = h->s.sessions[session]->h;
    }
    rc = fdmgpu_nscube_get_field(nh, field, out, count);
    std::lock_guard<std::mutex> g(h->s.mq);
    h->s.sessions[session]->busy = false;
    h->s.cv_sched.notify_one();
    if (rc) return rc;
    FDM_API_END
}

int fdmgpu_server_session_close(fdmgpu_server* h, int session, double timeout_ms) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    std::unique_ptr<Session> gone;
    int rc = with_idle_session(h->s, session, timeout_ms, [&](Session& ss, std::unique_lock<std::mutex>&) {
        auto it = h->s.sessions.find(session);
        gone = std::move(it->second);
        h->s.sessions.erase(it);
        h->s.account(-(double)ss.bytes);
        h->s.session_bytes -= (double)gone->bytes;
        return 0;
    });
    if (rc) return rc;
    gone.reset();  // frees the device state outside the lock
    FDM_API_END
}

int fdmgpu_server_stats(fdmgpu_server* h, fdmgpu_server_stats_t* out) {
    FDM_API_BEGIN
    if (!h || !out) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    Server& s = h->s;
    std::vector<float> a, b;
    {
        std::lock_guard<std::mutex> g(s.mq);
        memset(out, 0, sizeof(*out));
        out->submitted = s.n_submitted;
        out->completed = s.n_completed;
        out->failed = s.n_failed;
        out->cancelled = s.n_cancelled;
        out->rejected = s.n_rejected;
        out->shed = s.n_shed;
        out->queued = (int)s.pending.size();
        out->running = s.running;
        out->batches = s.n_batches;
        out->batched_requests = s.n_batched;
        out->used_bytes = s.used;
        out->peak_bytes = s.peak;
        out->budget_bytes = s.budget;
        out->plan_bytes = s.plan_bytes;
        out->session_bytes = s.session_bytes;
        out->mean_queue_ms = s.queue_n ? s.queue_sum / s.queue_n : 0.0;
        a = s.lat_solve;
        b = s.lat_advance;
    }
    Server::percentiles(a, &out->p50_solve_ms, &out->p99_solve_ms);
    Server::percentiles(b, &out->p50_advance_ms, &out->p99_advance_ms);
    std::vector<float> all(a);
    all.insert(all.end(), b.begin(), b.end());
    Server::percentiles(all, &out->p50_ms, &out->p99_ms);
    FDM_API_END
}

int fdmgpu_server_stats_reset(fdmgpu_server* h) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    Server& s = h->s;
    std::lock_guard<std::mutex> g(s.mq);
    s.n_submitted = s.n_completed = s.n_failed = s.n_cancelled = s.n_rejected = s.n_shed = 0;
    s.n_batches = s.n_batched = 0;
    s.lat_solve.clear();
    s.lat_advance.clear();
    s.queue_sum = 0;
    s.queue_n = 0;
    s.peak = s.used;
    FDM_API_END
}

int fdmgpu_server_set_admission(fdmgpu_server* h, int max_queued, double max_wait_ms) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (max_queued < 0 || !(max_wait_ms >= 0)) FDM_FAIL(FDMGPU_EINVAL, "negative admission limit");
    Server& s = h->s;
    std::lock_guard<std::mutex> g(s.mq);
    s.max_queued = max_queued;
    s.max_wait_ms = max_wait_ms;
    s.cv_sched.notify_one();  // the scheduler picks up the new deadline
    FDM_API_END
}

int fdmgpu_server_destroy(fdmgpu_server* h) {
    FDM_API_BEGIN
    if (!h) return FDMGPU_OK;
    h->s.shutdown();
    delete h;
    FDM_API_END
}

}  // extern "C"
