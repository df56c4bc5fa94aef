// Request server: continuous batching of steady transport solves, and
// Euler time loops beside them.
//
// Transport: one worker thread owns a BatchRun.  Between restart cycles it admits
// waiting requests (FIFO) while their Krylov workspace fits the HBM budget,
// assembles each admitted system on the device, and runs one cycle for all
// admitted solves; converged solves leave the batch immediately and their
// results are published with submit / admit / done times.  Because every
// system's reductions use only its own parts, a result does not depend on
// which other requests shared its cycles.
//
// Euler: a second worker thread takes Euler requests (a system with Euler
// geometry, coefficients, time-stepping controls and a host state) in FIFO
// order and runs each request's Predictor_Old loop (fg_euler_predictor: the
// loop's assembly, preconditioner set-up and solves stay on the device, on
// the system's own stream), so Euler loops overlap with the transport
// batch on the GPU.
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
};

struct EulerRequest {
    fg_system *s;
    fg_euler_coeffs c;
    fg_time_opts t;
    double *u;
    unsigned long long tag;
    double t_submit;
};

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
    std::vector<Request> active;   // parallel to the batch members
    std::set<fg_system *> busy;
    size_t in_use = 0;
    bool stop = false;
    int error = FG_OK;
    std::string error_text;
    std::thread worker, worker_eu;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    void run();
    void run_euler();
    void fail(int code)
    {
        std::lock_guard<std::mutex> l(mu);
        error = code;
        error_text = fg_last_error();
        cv_done.notify_all();
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
            if (stop && queue.empty() && active.empty()) return;
            if (stop) { queue.clear(); }
            for (auto it = queue.begin(); it != queue.end();) {
                bool fits = o.hbm_budget_bytes == 0 || in_use + it->bytes <= o.hbm_budget_bytes || active.empty();
                bool slot = o.max_active <= 0 || (int)(active.size() + admit.size()) < o.max_active;
                if (!fits || !slot) break;              // FIFO: the head waits for room
                if (busy.count(it->s)) { ++it; continue; }
                busy.insert(it->s);
                in_use += it->bytes;
                admit.push_back(*it);
                it = queue.erase(it);
            }
        }
        if (!admit.empty()) {
            for (auto &r : admit) {
                int rc = fg_transport_prepare(r.s, &r.c, nullptr);
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
            }
            cv_done.notify_all();
        }
        batch.remove(fin);
        std::vector<int> sorted = fin;
        std::sort(sorted.rbegin(), sorted.rend());
        for (int i : sorted) active.erase(active.begin() + i);
        if ((rc = batch.commit()) != FG_OK) { fail(rc); return; }
    }
}

void fg_server::run_euler()
{
    cudaSetDevice(device);
    fg_solver_opts so{cfg.kmax, cfg.lmax, cfg.tol, o.precision, o.inner_tol};
    for (;;) {
        EulerRequest r;
        {
            std::unique_lock<std::mutex> l(mu);
            cv_work_eu.wait(l, [&] { return stop || !queue_eu.empty(); });
            if (stop) { queue_eu.clear(); return; }
            r = queue_eu.front();
            queue_eu.pop_front();
        }
        const double t_admit = now();
        fg_time_stats ts{};
        int rc = fg_euler_predictor(r.s, &r.c, &so, &r.t, r.u, nullptr, &ts);
        if (rc != FG_OK) { fail(rc); return; }
        const double t = now();
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
        cv_done.notify_all();
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
    cudaError_t ce = cudaGetDevice(&sv->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&sv->st, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { delete sv; return cuda_fail(ce, "fg_server_create"); }
    if (sv->o.hbm_budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) sv->o.hbm_budget_bytes = (size_t)(0.8 * fr);
    }
    sv->t0 = std::chrono::steady_clock::now();
    sv->worker = std::thread([sv] { sv->run(); });
    sv->worker_eu = std::thread([sv] { sv->run_euler(); });
    *out = sv;
    return FG_OK;
}

int fg_server_submit(fg_server *sv, fg_system *s, const fg_transport_coeffs *c, unsigned long long tag)
{
    if (!sv || !s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (!s->geometry_ok) { set_error("fg_server_submit: the system has no geometry (fg_set_geometry)"); return FG_ERR_STATE; }
    if (s->topo.ndof != 1) { set_error("fg_server_submit: transport systems have ndof == 1"); return FG_ERR_UNSUPPORTED; }
    if (s->device != sv->device) { set_error("fg_server_submit: system on another device"); return FG_ERR_ARG; }
    Request r{s, *c, tag, sv->now(), 0.0, workspace_bytes(s, sv->cfg.kmax, sv->cfg.mixed)};
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
    EulerRequest r{s, *c, *t, u, tag, sv->now()};
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
    if (sv->worker_eu.joinable()) sv->worker_eu.join();
    cudaStreamSynchronize(sv->st);
    cudaStreamDestroy(sv->st);
    delete sv;
    return FG_OK;
}

}  // extern "C"
