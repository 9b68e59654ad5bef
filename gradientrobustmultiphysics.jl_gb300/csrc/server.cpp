// Serving engine: continuous admission of assembly + solve requests of mixed
// size and element type under an HBM budget.
//
// A server owns `nslots` worker threads; each worker owns a library context
// (its own CUDA stream) on the same GPU.  Submitted requests are copied and
// queued; the admission loop hands a request to an idle worker as soon as its
// estimated device footprint fits under the budget, so requests that arrive
// while others run are admitted as slots and memory free up, and their kernels
// overlap on the device (different streams).  A request's computation depends
// only on the request (launch shapes are chosen from its own sizes), so its
// result is bit-identical whether it runs alone or in the mix.
//
// No counterpart in the reference (it is single-process, one solve at a time);
// each request is one solve_direct! (src/solvers.jl:622-686) of a linear
// problem with the operators of include/grmp.h.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <thread>

#include "grmp_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    // copies of the caller's data
    int dim = 0, fe = 0, ncomp = 1;
    int32_t nverts = 0, ncells = 0, ndofs = 0;
    std::vector<double> coords;
    std::vector<int32_t> cells, celldofs, fixed;
    std::vector<grmp_bilinear_term> terms;
    std::vector<std::vector<double>> term_coef;
    grmp_rhs rhs{};
    std::vector<double> rhs_params;
    grmp_solve_params solve{};
    size_t bytes = 0;   // admission estimate
    // results
    std::vector<double> x;
    grmp_request_stats stats{};
    bool done = false;
    Clock::time_point t_submit, t_start, t_end;
};

struct Worker {
    grmp_context ctx = nullptr;
    std::thread th;
    std::shared_ptr<Request> job;
    bool has_job = false;
};

}  // namespace

struct grmp_server_s {
    int device = 0;
    size_t budget = 0, in_use = 0;
    std::mutex mu;
    std::condition_variable cv_admit, cv_done, cv_work;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<int64_t, std::shared_ptr<Request>> all;
    std::vector<Worker> workers;
    int64_t next_id = 1;
    bool stop = false;
    std::thread admitter;
    std::string last_error;
};

namespace {

size_t estimate_bytes(const Request &r) {
    // per-DoF nonzeros bound of the element / dimension, matrix in both precisions,
    // cols, slot map, incidence, mesh, vectors and solver workspace
    int ld = grmp_fe_ldofs(r.fe, r.dim, r.ncomp);
    double nnz_per_row = r.fe == GRMP_FE_H1P1 ? (r.dim == 2 ? 8 : 16) : (r.dim == 2 ? 14 : 30);
    nnz_per_row *= r.ncomp;
    double nnz = nnz_per_row * r.ndofs;
    double b = nnz * (8 + 4 + 4) + (double)r.ncells * ld * (4 + 1 + 4 + 2 * ld + 8) +
               (double)r.nverts * r.dim * 8 + (double)r.ncells * (r.dim + 1) * 4 + (double)r.ndofs * 120.0 +
               (double)r.ncells * 16 * 8;
    return (size_t)(1.25 * b) + (16u << 20);
}

// One request, synchronously, on a worker's context.
int run_request(grmp_context ctx, Request &r) {
    grmp_mesh mesh = nullptr;
    grmp_space space = nullptr;
    grmp_matrix A = nullptr;
    grmp_vector b = nullptr, x = nullptr;
    int rc = grmp_mesh_upload(ctx, r.dim, r.nverts, r.coords.data(), r.ncells, r.cells.data(), &mesh);
    if (!rc) rc = grmp_space_create(mesh, r.fe, r.ncomp, r.celldofs.data(), r.ndofs, &space);
    for (size_t i = 0; i < r.terms.size(); i++)
        r.terms[i].cell_coef = r.term_coef[i].empty() ? nullptr : r.term_coef[i].data();
    r.rhs.params = r.rhs_params.data();
    r.rhs.cell_group = nullptr;
    if (!rc) rc = grmp_pattern_build(space, (int)r.terms.size(), r.terms.data(), &A);
    const bool mixed = r.solve.mode == GRMP_SOLVE_MIXED;
    // one walk of the incidence lists fills both precisions (bit-identical to two passes)
    if (!rc) rc = grmp_assemble_bilinear(A, (int)r.terms.size(), r.terms.data(), mixed ? GRMP_FP64_FP32 : GRMP_FP64);
    if (!rc) rc = grmp_vector_create(ctx, r.ndofs, &b);
    if (!rc) rc = grmp_vector_create(ctx, r.ndofs, &x);
    if (!rc) rc = grmp_assemble_linear(space, &r.rhs, b);
    if (!rc)
        rc = grmp_apply_dirichlet(A, b, (int32_t)r.fixed.size(), r.fixed.empty() ? nullptr : r.fixed.data(), nullptr,
                                  GRMP_DIRICHLET_ELIMINATE, 1e60);
    grmp_solve_stats st{};
    // the SpMV configuration comes from the request's own sizes, never from
    // timings taken while other requests share the GPU
    if (r.solve.spmv_config == 0) r.solve.spmv_config = -1;
    if (!rc) rc = grmp_solve(A, b, x, &r.solve, &st);
    if (!rc || rc == GRMP_ERR_NOT_CONVERGED) {
        r.x.resize(r.ndofs);
        int rc2 = grmp_vector_download(x, r.x.data());
        if (!rc) rc = rc2;
    }
    r.stats.iterations = st.iterations;
    r.stats.outer_iterations = st.outer_iterations;
    r.stats.final_relres = st.final_relres;
    r.stats.solve_ms = st.solve_ms;
    if (x) grmp_vector_destroy(x);
    if (b) grmp_vector_destroy(b);
    if (A) grmp_matrix_destroy(A);
    if (space) grmp_space_destroy(space);
    if (mesh) grmp_mesh_destroy(mesh);
    grmp_synchronize(ctx);
    return rc;
}

void worker_loop(grmp_server srv, int w) {
    Worker &me = srv->workers[w];
    while (true) {
        std::shared_ptr<Request> job;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            srv->cv_work.wait(lk, [&] { return srv->stop || me.has_job; });
            if (!me.has_job && srv->stop) return;
            job = me.job;
        }
        job->t_start = Clock::now();
        int rc = run_request(me.ctx, *job);
        job->t_end = Clock::now();
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            job->stats.status = rc;
            job->stats.slot = w;
            job->stats.queue_ms = std::chrono::duration<double, std::milli>(job->t_start - job->t_submit).count();
            job->stats.run_ms = std::chrono::duration<double, std::milli>(job->t_end - job->t_start).count();
            job->stats.latency_ms = std::chrono::duration<double, std::milli>(job->t_end - job->t_submit).count();
            job->done = true;
            srv->in_use -= job->bytes;
            me.job.reset();
            me.has_job = false;
        }
        srv->cv_done.notify_all();
        srv->cv_admit.notify_all();
    }
}

void admit_loop(grmp_server srv) {
    std::unique_lock<std::mutex> lk(srv->mu);
    while (true) {
        srv->cv_admit.wait(lk, [&] {
            if (srv->stop) return true;
            if (srv->queue.empty()) return false;
            bool idle = false;
            for (auto &w : srv->workers) idle = idle || !w.has_job;
            return idle && (srv->in_use + srv->queue.front()->bytes <= srv->budget || srv->in_use == 0);
        });
        if (srv->stop) return;
        // first come, first served; the head waits for memory (no starvation)
        auto job = srv->queue.front();
        srv->queue.pop_front();
        for (auto &w : srv->workers)
            if (!w.has_job) {
                w.job = job;
                w.has_job = true;
                srv->in_use += job->bytes;
                break;
            }
        srv->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int grmp_server_create(int device, size_t hbm_budget_bytes, int nslots, grmp_server *out) {
    if (!out || nslots <= 0 || nslots > 64) return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    auto srv = new (std::nothrow) grmp_server_s();
    if (!srv) return GRMP_ERR_OUT_OF_MEMORY;
    srv->device = device;
    srv->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)-1;
    srv->workers.resize(nslots);
    for (int w = 0; w < nslots; w++) {
        int rc = grmp_create_context(device, 0, &srv->workers[w].ctx);
        if (rc) {
            for (int k = 0; k < w; k++) grmp_destroy_context(srv->workers[k].ctx);
            delete srv;
            return rc;
        }
    }
    for (int w = 0; w < nslots; w++) srv->workers[w].th = std::thread(worker_loop, srv, w);
    srv->admitter = std::thread(admit_loop, srv);
    *out = srv;
    return GRMP_OK;
}

int grmp_server_request_bytes(const grmp_request *q, size_t *bytes) {
    if (!q || !bytes) return GRMP_ERR_INVALID_ARG;
    if ((q->dim != 2 && q->dim != 3) || q->nverts <= 0 || q->ncells <= 0 || q->ndofs <= 0) return GRMP_ERR_INVALID_ARG;
    if (grmp_fe_ldofs(q->fe_kind, q->dim, q->ncomponents) <= 0) return GRMP_ERR_UNSUPPORTED;
    Request r;
    r.dim = q->dim;
    r.fe = q->fe_kind;
    r.ncomp = q->ncomponents;
    r.nverts = q->nverts;
    r.ncells = q->ncells;
    r.ndofs = q->ndofs;
    *bytes = estimate_bytes(r);
    return GRMP_OK;
}

int grmp_server_submit(grmp_server srv, const grmp_request *q, int64_t *id) {
    if (!srv || !q || !id || !q->coords || !q->cells || !q->celldofs || q->nterms <= 0 || q->nterms > GRMP_MAX_TERMS ||
        !q->terms)
        return GRMP_ERR_INVALID_ARG;
    if ((q->dim != 2 && q->dim != 3) || q->nverts <= 0 || q->ncells <= 0 || q->ndofs <= 0 || q->nfixed < 0)
        return GRMP_ERR_INVALID_ARG;
    int ld = grmp_fe_ldofs(q->fe_kind, q->dim, q->ncomponents);
    if (ld <= 0) return GRMP_ERR_UNSUPPORTED;
    auto r = std::make_shared<Request>();
    r->dim = q->dim;
    r->fe = q->fe_kind;
    r->ncomp = q->ncomponents;
    r->nverts = q->nverts;
    r->ncells = q->ncells;
    r->ndofs = q->ndofs;
    r->coords.assign(q->coords, q->coords + (size_t)q->nverts * q->dim);
    r->cells.assign(q->cells, q->cells + (size_t)q->ncells * (q->dim + 1));
    r->celldofs.assign(q->celldofs, q->celldofs + (size_t)q->ncells * ld);
    if (q->nfixed) r->fixed.assign(q->fixed, q->fixed + q->nfixed);
    r->terms.assign(q->terms, q->terms + q->nterms);
    r->term_coef.resize(q->nterms);
    for (int i = 0; i < q->nterms; i++) {
        if (q->terms[i].cell_coef && q->terms[i].coef_on_device) return GRMP_ERR_INVALID_ARG;
        if (q->terms[i].cell_coef) r->term_coef[i].assign(q->terms[i].cell_coef, q->terms[i].cell_coef + q->ncells);
    }
    r->rhs = q->rhs;
    if (q->rhs.nparams < 0 || (q->rhs.nparams > 0 && !q->rhs.params) || q->rhs.cell_group) return GRMP_ERR_INVALID_ARG;
    r->rhs_params.assign(q->rhs.params, q->rhs.params + q->rhs.nparams);
    r->solve = q->solve;
    r->bytes = estimate_bytes(*r);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (r->bytes > srv->budget) {
            srv->last_error = "request exceeds the server's HBM budget";
            return GRMP_ERR_BUDGET;
        }
        r->id = srv->next_id++;
        srv->all[r->id] = r;
        srv->queue.push_back(r);
        *id = r->id;
    }
    srv->cv_admit.notify_all();
    return GRMP_OK;
}

int grmp_server_wait(grmp_server srv, int64_t id, double timeout_s, double *x_out, grmp_request_stats *stats) {
    if (!srv) return GRMP_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->all.find(id);
    if (it == srv->all.end()) return GRMP_ERR_INVALID_ARG;
    auto r = it->second;
    auto pred = [&] { return r->done; };
    if (timeout_s >= 0) {
        if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return GRMP_ERR_TIMEOUT;
    } else {
        srv->cv_done.wait(lk, pred);
    }
    if (x_out && !r->x.empty()) std::memcpy(x_out, r->x.data(), r->x.size() * sizeof(double));
    if (stats) *stats = r->stats;
    srv->all.erase(it);
    return r->stats.status;
}

int grmp_server_destroy(grmp_server srv) {
    if (!srv) return GRMP_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_admit.notify_all();
    srv->cv_work.notify_all();
    if (srv->admitter.joinable()) srv->admitter.join();
    for (auto &w : srv->workers)
        if (w.th.joinable()) w.th.join();
    for (auto &w : srv->workers) grmp_destroy_context(w.ctx);
    delete srv;
    return GRMP_OK;
}

}  // extern "C"
