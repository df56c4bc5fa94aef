// Request server: continuous batching of steady transport solves and of
// the correction solves of Euler time loops.
//
// Transport: one worker thread owns a BatchRun.  Between restart cycles it
// admits waiting requests (FIFO) while their device footprint (the
// system's arrays and its Krylov workspace) fits the HBM budget, assembles
// each admitted system on the device, and runs one cycle for all admitted
// solves; converged solves leave the batch immediately and their results
// are published with submit / admit / done times.  Because every system's
// reductions use only its own parts, a result does not depend on which
// other requests shared its cycles.
//
// Euler: a pool of request threads runs admitted Euler time loops
// (Predictor_Old, 00_CommonFiles/Time_Integration/Predictor_Old.c:53-123:
// assembly, preconditioner set-up and the update on each system's own
// stream).  Each correction solve of a loop is handed to a second batch
// thread, which keeps its own BatchRun of every Euler correction currently
// waiting: corrections of different requests join and leave it between
// restart cycles, exactly as transport solves do, so the Euler loops share
// GMRES cycles instead of queueing behind one another.  A loop's result is
// the same as its solo run (same kernels, per-system reductions).  Euler
// requests are admitted against the same HBM budget.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <set>
#include <string>
#include <thread>

#include "system.h"

namespace fg {

struct Request {
    fg_system *s;
    fg_transport_coeffs c;
    unsigned long long tag;
    double t_submit, t_admit;
    size_t bytes;
    const double *hA = nullptr, *hF = nullptr;   // host-buffer request: blocks and right-hand side
    double *hX = nullptr;                         // and its solution
};

struct EulerRequest {
    fg_system *s;
    fg_euler_coeffs c;
    fg_time_opts t;
    double *u;
    unsigned long long tag;
    double t_submit;
    size_t bytes;
};

// One correction solve waiting for the Euler batch.
struct EulerSolve {
    fg_system *s;
    fg_solve_stats *stats;
    bool done;
    int rc;
};

constexpr int kEulerWorkers = 16;      // Euler time loops in flight at most

}  // namespace fg

using namespace fg;

struct fg_server {
    fg_server_opts o{};
    SolveConfig cfg;
    int device = 0;
    cudaStream_t st = nullptr;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> queue;
    std::deque<EulerRequest> queue_eu;
    std::condition_variable cv_work_eu;
    std::vector<fg_server_result> done;
    std::vector<Request> active;   // parallel to the batch members (transport thread only)
    std::set<fg_system *> busy;
    size_t in_use = 0;             // admitted bytes (transport + Euler)
    int tr_active = 0, eu_active = 0;   // admitted requests
    bool stop = false;
    int error = FG_OK;
    std::string error_text;
    std::thread worker, worker_eub;
    std::vector<std::thread> workers_eu;
    // Euler correction batch
    SolveConfig cfg_eu;
    cudaStream_t st_eu = nullptr;
    std::deque<EulerSolve *> eu_pending;
    std::condition_variable cv_eu_batch, cv_eu_solved;
    bool stop_eub = false;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    // a request of `bytes` may start: it fits the budget, or nothing else is
    // admitted (one oversized request still runs alone)
    bool fits(size_t bytes, int extra) const
    {
        return o.hbm_budget_bytes == 0 || in_use + bytes <= o.hbm_budget_bytes || tr_active + eu_active + extra == 0;
    }
    void run();
    void run_euler();
    void run_euler_batch();
    int solve_correction(fg_system *s, const SolveConfig &c, fg_solve_stats *st);
    void fail(int code)
    {
        std::lock_guard<std::mutex> l(mu);
        error = code;
        error_text = fg_last_error();
        cv_done.notify_all();
        cv_eu_solved.notify_all();
    }
};

void fg_server::run()
{
    cudaSetDevice(device);
    BatchRun batch(cfg, st);
    std::vector<int> live;
    for (;;) {
        // admission
        std::vector<Request> admit;
        {
            std::unique_lock<std::mutex> l(mu);
            if (active.empty() && queue.empty() && !stop)
                cv_work.wait(l, [&] { return stop || !queue.empty(); });
            if (active.empty() && !queue.empty() && !stop && !fits(queue.front().bytes, 0))
                cv_work.wait_for(l, std::chrono::milliseconds(2),
                                 [&] { return stop || queue.empty() || fits(queue.front().bytes, 0); });
            if (stop && queue.empty() && active.empty()) return;
            if (stop) { queue.clear(); }
            for (auto it = queue.begin(); it != queue.end();) {
                const bool room = fits(it->bytes, (int)admit.size());
                const bool slot = o.max_active <= 0 || (int)(active.size() + admit.size()) < o.max_active;
                if (!room || !slot) break;              // FIFO: the head waits for room
                if (busy.count(it->s)) { ++it; continue; }
                busy.insert(it->s);
                in_use += it->bytes;
                ++tr_active;
                admit.push_back(*it);
                it = queue.erase(it);
            }
        }
        if (!admit.empty()) {
            for (auto &r : admit) {
                int rc = r.hA ? prepare_host_request(r.s, r.hA, r.hF) : fg_transport_prepare(r.s, &r.c, nullptr);
                if (rc == FG_OK && cudaStreamSynchronize(r.s->stream) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "prepare");
                if (rc == FG_OK) rc = batch.stage({r.s, r.s->rhs_b.as<double>(), r.s->rhs_f.as<double>(), nullptr});
                if (rc != FG_OK) { fail(rc); return; }
                r.t_admit = now();
                active.push_back(r);
            }
            int rc = batch.commit();
            if (rc != FG_OK) { fail(rc); return; }
        }
        if (active.empty()) continue;
        int rc = batch.cycle(false, live);
        if (rc != FG_OK) { fail(rc); return; }
        std::vector<int> fin;
        for (size_t i = 0; i < live.size(); ++i)
            if (!live[i]) fin.push_back((int)i);
        if (fin.empty()) continue;
        std::vector<SysState> sts;
        if ((rc = batch.finish(fin, sts)) != FG_OK) { fail(rc); return; }
        for (int i : fin)                                // host-buffer requests: X before the result
            if (active[i].hX && (rc = download_solution(active[i].s, active[i].hX, st)) != FG_OK) { fail(rc); return; }
        double t = now();
        {
            std::lock_guard<std::mutex> l(mu);
            for (size_t q = 0; q < fin.size(); ++q) {
                const Request &r = active[fin[q]];
                fg_server_result res{};
                res.tag = r.tag;
                fill_stats(sts[q], t - r.t_admit, res.stats);
                res.t_submit = r.t_submit;
                res.t_admit = r.t_admit;
                res.t_done = t;
                done.push_back(res);
                busy.erase(r.s);
                in_use -= r.bytes;
                --tr_active;
            }
            cv_done.notify_all();
        }
        cv_work_eu.notify_all();                      // room for waiting Euler loops
        batch.remove(fin);
        std::vector<int> sorted = fin;
        std::sort(sorted.rbegin(), sorted.rend());
        for (int i : sorted) active.erase(active.begin() + i);
        if ((rc = batch.commit()) != FG_OK) { fail(rc); return; }
    }
}

// A correction solve of an Euler loop: joins the Euler batch when its
// configuration is the batch's (the server's solver options with
// BlockDiag), else runs alone on the system's stream.
int fg_server::solve_correction(fg_system *s, const SolveConfig &c, fg_solve_stats *st)
{
    if (c.precond != cfg_eu.precond || c.kmax != cfg_eu.kmax || c.lmax != cfg_eu.lmax || c.tol != cfg_eu.tol ||
        c.mixed != cfg_eu.mixed || c.vhalf != cfg_eu.vhalf || c.inner_tol != cfg_eu.inner_tol) {
        std::vector<BatchMember> mem{{s, s->rhs_b.as<double>(), s->rhs_f.as<double>(), nullptr}};
        return solve_batch(mem, c, st, s->stream);
    }
    FG_CUDA(cudaStreamSynchronize(s->stream));        // assembly and set-up finished before the batch reads them
    EulerSolve job{s, st, false, FG_OK};
    {
        std::lock_guard<std::mutex> l(mu);
        eu_pending.push_back(&job);
    }
    cv_eu_batch.notify_one();
    std::unique_lock<std::mutex> l(mu);
    cv_eu_solved.wait(l, [&] { return job.done; });    // the batch thread completes every job it takes
    return job.rc;
}

void fg_server::run_euler_batch()
{
    cudaSetDevice(device);
    BatchRun batch(cfg_eu, st_eu);
    std::vector<EulerSolve *> act;                    // parallel to the batch members
    std::vector<int> live;
    auto give_up = [&](int rc) {
        fail(rc);
        std::lock_guard<std::mutex> l(mu);
        for (auto *a : act) { a->rc = rc; a->done = true; }
        for (auto *a : eu_pending) { a->rc = rc; a->done = true; }
        eu_pending.clear();
        cv_eu_solved.notify_all();
    };
    for (;;) {
        std::deque<EulerSolve *> add;
        {
            std::unique_lock<std::mutex> l(mu);
            if (act.empty()) cv_eu_batch.wait(l, [&] { return stop_eub || !eu_pending.empty(); });
            if (stop_eub && act.empty() && eu_pending.empty()) return;
            add.swap(eu_pending);
        }
        int rc = FG_OK;
        for (auto *a : add) {
            act.push_back(a);
            if ((rc = batch.stage({a->s, a->s->rhs_b.as<double>(), a->s->rhs_f.as<double>(), nullptr}))) {
                give_up(rc);
                return;
            }
        }
        if (!add.empty() && (rc = batch.commit())) { give_up(rc); return; }
        if (act.empty()) continue;
        if ((rc = batch.cycle(false, live))) { give_up(rc); return; }
        std::vector<int> fin;
        for (size_t i = 0; i < live.size(); ++i)
            if (!live[i]) fin.push_back((int)i);
        if (fin.empty()) continue;
        std::vector<SysState> sts;
        if ((rc = batch.finish(fin, sts))) { give_up(rc); return; }
        {
            std::lock_guard<std::mutex> l(mu);
            for (size_t q = 0; q < fin.size(); ++q) {
                EulerSolve *a = act[fin[q]];
                fill_stats(sts[q], 0.0, *a->stats);
                a->rc = FG_OK;
                a->done = true;
            }
            cv_eu_solved.notify_all();
        }
        batch.remove(fin);
        std::vector<int> sorted = fin;
        std::sort(sorted.rbegin(), sorted.rend());
        for (int i : sorted) act.erase(act.begin() + i);
        if ((rc = batch.commit())) { give_up(rc); return; }
    }
}

void fg_server::run_euler()
{
    cudaSetDevice(device);
    fg_solver_opts so{cfg.kmax, cfg.lmax, cfg.tol, o.precision, o.inner_tol};
    const CorrectionSolve hook = [this](fg_system *s, const SolveConfig &c, fg_solve_stats *st) {
        return solve_correction(s, c, st);
    };
    for (;;) {
        EulerRequest r;
        {
            std::unique_lock<std::mutex> l(mu);
            cv_work_eu.wait(l, [&] { return stop || (!queue_eu.empty() && fits(queue_eu.front().bytes, 0)); });
            if (stop) { queue_eu.clear(); return; }
            r = queue_eu.front();
            queue_eu.pop_front();
            in_use += r.bytes;
            ++eu_active;
        }
        const double t_admit = now();
        fg_time_stats ts{};
        int rc = euler_predictor_hooked(r.s, &r.c, &so, &r.t, r.u, nullptr, &ts, &hook);
        if (rc != FG_OK) { fail(rc); return; }
        const double t = now();
        {
            std::lock_guard<std::mutex> l(mu);
            fg_server_result res{};
            res.tag = r.tag;
            res.stats.iterations = ts.gmres_iterations;
            res.stats.cycles = ts.corrections;
            res.stats.converged = ts.true_rel_residual <= cfg.tol ? 1 : 0;
            res.stats.status = FG_OK;
            res.stats.eps = cfg.tol;
            res.stats.true_rel_residual = ts.true_rel_residual;
            res.stats.seconds = t - t_admit;
            res.t_submit = r.t_submit;
            res.t_admit = t_admit;
            res.t_done = t;
            done.push_back(res);
            busy.erase(r.s);
            in_use -= r.bytes;
            --eu_active;
            cv_done.notify_all();
        }
        cv_work.notify_all();                         // room for waiting transport requests
        cv_work_eu.notify_all();
    }
}

extern "C" {

int fg_server_create(fg_server **out, const fg_server_opts *opts)
{
    if (!out || !opts) { set_error("NULL argument"); return FG_ERR_ARG; }
    *out = nullptr;
    if (opts->precision != FG_PREC_MIXED && opts->precision != FG_PREC_FP64 && opts->precision != FG_PREC_MIXED16) {
        set_error("precision must be FG_PREC_FP64, FG_PREC_MIXED or FG_PREC_MIXED16"); return FG_ERR_ARG;
    }
    if (opts->precision == FG_PREC_MIXED16 && opts->kmax > 32) {
        set_error("FG_PREC_MIXED16 needs kmax <= 32"); return FG_ERR_ARG;
    }
    if (opts->kmax < 2 || opts->kmax > kPartStride - 4 || opts->lmax < 1) {
        set_error("kmax must be in [2, 60] and lmax >= 1"); return FG_ERR_ARG;
    }
    fg_server *sv = new (std::nothrow) fg_server();
    if (!sv) { set_error("host allocation failed"); return FG_ERR_NOMEM; }
    sv->o = *opts;
    sv->cfg.kmax = opts->kmax;
    sv->cfg.lmax = opts->lmax;
    sv->cfg.tol = opts->tol;
    sv->cfg.mixed = opts->precision == FG_PREC_FP64 ? 0 : 1;
    sv->cfg.vhalf = opts->precision == FG_PREC_MIXED16 ? 1 : 0;
    sv->cfg.inner_tol = opts->inner_tol > 0 ? opts->inner_tol : 1e-5;
    sv->cfg.precond = FG_PRECOND_DIAG;
    sv->cfg.device_io = 1;
    sv->cfg.use_graph = 0;
    sv->cfg_eu = sv->cfg;
    sv->cfg_eu.precond = FG_PRECOND_BLOCKDIAG;
    cudaError_t ce = cudaGetDevice(&sv->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&sv->st, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&sv->st_eu, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { delete sv; return cuda_fail(ce, "fg_server_create"); }
    if (sv->o.hbm_budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) sv->o.hbm_budget_bytes = (size_t)(0.8 * fr);
    }
    sv->t0 = std::chrono::steady_clock::now();
    sv->worker = std::thread([sv] { sv->run(); });
    sv->worker_eub = std::thread([sv] { sv->run_euler_batch(); });
    for (int i = 0; i < kEulerWorkers; ++i) sv->workers_eu.emplace_back([sv] { sv->run_euler(); });
    *out = sv;
    return FG_OK;
}

int fg_server_submit_host(fg_server *sv, fg_system *s, const double *A, const double *F, double *X,
                          unsigned long long tag)
{
    if (!sv || !s || !A || !F || !X) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (s->topo.S != 3) { set_error("fg_server_submit_host: 3x3 element blocks (ndof == 1)"); return FG_ERR_UNSUPPORTED; }
    if (s->device != sv->device) { set_error("fg_server_submit_host: system on another device"); return FG_ERR_ARG; }
    Request r{s, fg_transport_coeffs{}, tag, sv->now(), 0.0, request_bytes(s, sv->cfg.kmax, sv->cfg.mixed, false)};
    r.hA = A;
    r.hF = F;
    r.hX = X;
    {
        std::lock_guard<std::mutex> l(sv->mu);
        if (sv->error) { set_error(sv->error_text); return sv->error; }
        if (sv->stop) { set_error("server is stopping"); return FG_ERR_STATE; }
        sv->queue.push_back(r);
    }
    sv->cv_work.notify_one();
    return FG_OK;
}

int fg_server_submit(fg_server *sv, fg_system *s, const fg_transport_coeffs *c, unsigned long long tag)
{
    if (!sv || !s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (!s->geometry_ok) { set_error("fg_server_submit: the system has no geometry (fg_set_geometry)"); return FG_ERR_STATE; }
    if (s->topo.ndof != 1) { set_error("fg_server_submit: transport systems have ndof == 1"); return FG_ERR_UNSUPPORTED; }
    if (s->device != sv->device) { set_error("fg_server_submit: system on another device"); return FG_ERR_ARG; }
    Request r{s, *c, tag, sv->now(), 0.0, request_bytes(s, sv->cfg.kmax, sv->cfg.mixed, false)};
    {
        std::lock_guard<std::mutex> l(sv->mu);
        if (sv->error) { set_error(sv->error_text); return sv->error; }
        if (sv->stop) { set_error("server is stopping"); return FG_ERR_STATE; }
        sv->queue.push_back(r);
    }
    sv->cv_work.notify_one();
    return FG_OK;
}

int fg_server_submit_euler(fg_server *sv, fg_system *s, const fg_euler_coeffs *c, const fg_time_opts *t,
                           double *u, unsigned long long tag)
{
    if (!sv || !s || !c || !t || !u) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (!s->eu_geometry_ok || s->topo.ndof != 4) {
        set_error("fg_server_submit_euler: the system has no Euler geometry (fg_euler_set_geometry)");
        return FG_ERR_STATE;
    }
    if (s->device != sv->device) { set_error("fg_server_submit_euler: system on another device"); return FG_ERR_ARG; }
    size_t bytes = request_bytes(s, sv->cfg.kmax, sv->cfg.mixed, true);
    // element state the loop allocates: the DD bubbles and delta, and the
    // Predictor2 bubble planes
    if (c->form == FG_EULER_DD && s->shock_state.bytes < 40 * (size_t)s->nel_pad) bytes += 40 * (size_t)s->nel_pad;
    if (t->scheme >= FG_TIME_PREDICTOR2 && s->bubble_nb != 4) bytes += 8 * (size_t)kBubblePlanesEuler * s->nel_pad;
    EulerRequest r{s, *c, *t, u, tag, sv->now(), bytes};
    {
        std::lock_guard<std::mutex> l(sv->mu);
        if (sv->error) { set_error(sv->error_text); return sv->error; }
        if (sv->stop) { set_error("server is stopping"); return FG_ERR_STATE; }
        if (sv->busy.count(s)) { set_error("fg_server_submit_euler: the system is in use by another request"); return FG_ERR_STATE; }
        sv->busy.insert(s);
        sv->queue_eu.push_back(r);
    }
    sv->cv_work_eu.notify_one();
    return FG_OK;
}

int fg_server_poll(fg_server *sv, fg_server_result *out, int max, int *count)
{
    if (!sv || !count || (max > 0 && !out)) { set_error("NULL argument"); return FG_ERR_ARG; }
    std::lock_guard<std::mutex> l(sv->mu);
    int n = std::min<int>(max, (int)sv->done.size());
    for (int i = 0; i < n; ++i) out[i] = sv->done[i];
    sv->done.erase(sv->done.begin(), sv->done.begin() + n);
    *count = n;
    if (sv->error) { set_error(sv->error_text); return sv->error; }
    return FG_OK;
}

int fg_server_wait(fg_server *sv, int n, double timeout_s)
{
    if (!sv) { set_error("NULL argument"); return FG_ERR_ARG; }
    std::unique_lock<std::mutex> l(sv->mu);
    sv->cv_done.wait_for(l, std::chrono::duration<double>(timeout_s),
                         [&] { return sv->error || (int)sv->done.size() >= n; });
    if (sv->error) { set_error(sv->error_text); return sv->error; }
    return FG_OK;
}

double fg_server_now(const fg_server *sv) { return sv ? sv->now() : 0.0; }

int fg_server_destroy(fg_server *sv)
{
    if (!sv) return FG_OK;
    {
        std::lock_guard<std::mutex> l(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    sv->cv_work_eu.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    for (auto &w : sv->workers_eu)
        if (w.joinable()) w.join();                   // running loops finish first
    {
        std::lock_guard<std::mutex> l(sv->mu);
        sv->stop_eub = true;
    }
    sv->cv_eu_batch.notify_all();
    if (sv->worker_eub.joinable()) sv->worker_eub.join();
    cudaStreamSynchronize(sv->st);
    cudaStreamDestroy(sv->st);
    cudaStreamSynchronize(sv->st_eu);
    cudaStreamDestroy(sv->st_eu);
    delete sv;
    return FG_OK;
}

}  // extern "C"
