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
// Residency: a request with a non-zero mesh_key leaves its mesh, DoF map,
// sparsity pattern (with the solver workspace and tuned state) and vectors
// on the device, in the slot that ran it (an LRU list of kSlotResident
// entries per slot); a later request with the same key and operator
// structure runs there and skips the upload and setup.  Resident entries
// count against the budget; when the head of the queue does not fit, the
// admission loop drops least recently used entries of idle slots.
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

constexpr int kSlotResident = 4;   // resident problems kept per slot

struct Request {
    int64_t id = 0;
    // copies of the caller's data
    int dim = 0, fe = 0, ncomp = 1;
    int32_t nverts = 0, ncells = 0, ndofs = 0;
    std::vector<double> coords;
    std::vector<int32_t> cells, celldofs, fixed;
    bool device_dofmap = false;     // celldofs built on the device
    bool all_boundary = false;      // fixed = every boundary DoF (device)
    uint64_t key = 0, sig = 0;      // residency key and operator-structure signature
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

// Device data of one problem, reused by later requests with its key.
struct Resident {
    uint64_t key = 0, sig = 0;
    grmp_mesh mesh = nullptr;
    grmp_space space = nullptr;
    grmp_matrix A = nullptr;
    grmp_vector b = nullptr, x = nullptr;
    std::vector<int32_t> fixed;
    int32_t ndofs = 0;
    size_t bytes = 0;        // counted against the budget
    uint64_t last_use = 0;
};

void destroy_resident(Resident &r) {
    if (r.x) grmp_vector_destroy(r.x);
    if (r.b) grmp_vector_destroy(r.b);
    if (r.A) grmp_matrix_destroy(r.A);
    if (r.space) grmp_space_destroy(r.space);
    if (r.mesh) grmp_mesh_destroy(r.mesh);
    r = Resident();
}

struct Worker {
    grmp_context ctx = nullptr;
    std::thread th;
    std::shared_ptr<Request> job;
    bool has_job = false;
    bool hit = false;                 // the job's key is resident here
    std::vector<Resident> cache;      // touched by the worker while it has a job, by the admitter otherwise
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
    uint64_t clock = 0;      // LRU stamps
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
    // a device-built DoF map: vertices plus (P2) edges / faces, bounded from the cell count
    const double nd = r.ndofs > 0 ? (double)r.ndofs
                                  : (double)r.ncomp * (r.nverts + (r.fe == GRMP_FE_H1P2
                                                                       ? (r.dim == 2 ? 1.5 : 1.25) * r.ncells + r.nverts
                                                                       : 0.0));
    double nnz = nnz_per_row * nd;
    double b = nnz * (8 + 4 + 4) + (double)r.ncells * ld * (4 + 1 + 4 + 2 * ld + 8) +
               (double)r.nverts * r.dim * 8 + (double)r.ncells * (r.dim + 1) * 4 + nd * 120.0 +
               (double)r.ncells * 16 * 8;
    return (size_t)(1.25 * b) + (16u << 20);
}

// Mesh, DoF map, pattern, vectors and Dirichlet DoFs of a request.
int build_resident(grmp_context ctx, Request &r, Resident &res) {
    int rc = grmp_mesh_upload(ctx, r.dim, r.nverts, r.coords.data(), r.ncells, r.cells.data(), &res.mesh);
    if (!rc) {
        if (r.device_dofmap) {
            rc = grmp_space_create_on_device(res.mesh, r.fe, r.ncomp, &res.space, &res.ndofs);
        } else {
            rc = grmp_space_create(res.mesh, r.fe, r.ncomp, r.celldofs.data(), r.ndofs, &res.space);
            res.ndofs = r.ndofs;
        }
    }
    if (!rc) {
        // A resident pattern serves later coefficients too: it is built with
        // unit factors and no cell coefficients, so it drops only the entries
        // whose contributions vanish for the operator kinds themselves (the
        // reference likewise keeps a matrix's pattern when it refills it with
        // zeros and assembles again, src/fematrix.jl:220-232,
        // src/solvers.jl:556).  A one-off request uses its own coefficients.
        std::vector<grmp_bilinear_term> pt = r.terms;
        if (r.key != 0)
            for (auto &t : pt) {
                t.factor = 1.0;
                t.cell_coef = nullptr;
                t.coef_on_device = 0;
                if (t.op_kind == GRMP_OP_HOOKE) {
                    t.param[0] = 1.0;
                    t.param[1] = 1.6180339887498949;   // no coincidental cancellation of mu and lambda parts
                }
            }
        else
            for (size_t i = 0; i < pt.size(); i++)
                pt[i].cell_coef = r.term_coef[i].empty() ? nullptr : r.term_coef[i].data();
        rc = grmp_pattern_build(res.space, (int)pt.size(), pt.data(), &res.A);
        // no timed choice of the assembly's block shape for served requests:
        // a request's latency must not pay trial launches (nor depend on the
        // other requests sharing the GPU while they run)
        if (!rc)
            for (int &t : res.A->asm_tpb) t = -1;
    }
    if (!rc) rc = grmp_vector_create(ctx, res.ndofs, &res.b);
    if (!rc) rc = grmp_vector_create(ctx, res.ndofs, &res.x);
    if (!rc) {
        if (r.all_boundary) {
            int32_t nb = 0;
            rc = grmp_space_boundary_dofs(res.space, 0, nullptr, &nb);
            if (!rc) {
                res.fixed.resize(nb);
                rc = grmp_space_boundary_dofs(res.space, nb, res.fixed.data(), &nb);
            }
        } else {
            res.fixed = r.fixed;
        }
    }
    res.key = r.key;
    res.sig = r.sig;
    res.bytes = r.bytes;
    if (rc) destroy_resident(res);
    return rc;
}

// Assembly with the request's coefficients, its right-hand side, Dirichlet
// elimination and the solve on resident (or freshly built) data.
int run_on(grmp_context ctx, Request &r, Resident &res) {
    for (size_t i = 0; i < r.terms.size(); i++)
        r.terms[i].cell_coef = r.term_coef[i].empty() ? nullptr : r.term_coef[i].data();
    r.rhs.params = r.rhs_params.data();
    r.rhs.cell_group = nullptr;
    const bool mixed = r.solve.mode == GRMP_SOLVE_MIXED;
    // one walk of the incidence lists fills both precisions (bit-identical to two passes)
    int rc = grmp_assemble_bilinear(res.A, (int)r.terms.size(), r.terms.data(), mixed ? GRMP_FP64_FP32 : GRMP_FP64);
    if (!rc) rc = grmp_vector_fill(res.b, 0.0);
    if (!rc) rc = grmp_vector_fill(res.x, 0.0);   // the same zero start as a fresh request
    if (!rc) rc = grmp_assemble_linear(res.space, &r.rhs, res.b);
    if (!rc)
        rc = grmp_apply_dirichlet(res.A, res.b, (int32_t)res.fixed.size(), res.fixed.empty() ? nullptr : res.fixed.data(),
                                  nullptr, GRMP_DIRICHLET_ELIMINATE, 1e60);
    grmp_solve_stats st{};
    // the SpMV configuration comes from the request's own sizes, never from
    // timings taken while other requests share the GPU
    if (r.solve.spmv_config == 0) r.solve.spmv_config = -1;
    if (!rc) rc = grmp_solve(res.A, res.b, res.x, &r.solve, &st);
    if (!rc || rc == GRMP_ERR_NOT_CONVERGED) {
        r.x.resize(res.ndofs);
        int rc2 = grmp_vector_download(res.x, r.x.data());
        if (!rc) rc = rc2;
    }
    r.stats.iterations = st.iterations;
    r.stats.outer_iterations = st.outer_iterations;
    r.stats.final_relres = st.final_relres;
    r.stats.solve_ms = st.solve_ms;
    r.stats.ndofs = res.ndofs;
    return rc;
}

// One request, synchronously, on a worker's context: on its resident entry
// (a hit), or on data built for it and then kept (key != 0, least recently
// used entry of the slot dropped when full) or freed.  *freed receives the
// bytes released from the budget.
int run_request(grmp_server srv, Worker &me, Request &r, size_t *freed) {
    grmp_context ctx = me.ctx;
    *freed = 0;
    if (me.hit) {
        for (auto &e : me.cache)
            if (e.key == r.key && e.sig == r.sig) {
                r.stats.resident = 1;
                if (!r.all_boundary) e.fixed = r.fixed;   // the request's own Dirichlet DoFs
                {
                    std::lock_guard<std::mutex> lk(srv->mu);
                    e.last_use = ++srv->clock;
                }
                int rc = run_on(ctx, r, e);
                grmp_synchronize(ctx);
                return rc;
            }
    }
    Resident res;
    int rc = build_resident(ctx, r, res);
    if (!rc) rc = run_on(ctx, r, res);
    if (!rc && r.key != 0) {
        std::lock_guard<std::mutex> lk(srv->mu);
        if ((int)me.cache.size() >= kSlotResident) {   // drop the slot's least recently used entry
            size_t lru = 0;
            for (size_t i = 1; i < me.cache.size(); i++)
                if (me.cache[i].last_use < me.cache[lru].last_use) lru = i;
            *freed += me.cache[lru].bytes;
            destroy_resident(me.cache[lru]);
            me.cache.erase(me.cache.begin() + lru);
        }
        res.last_use = ++srv->clock;
        me.cache.push_back(res);   // its bytes stay counted
    } else {
        destroy_resident(res);
        *freed += r.bytes;
    }
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
        size_t freed = 0;
        int rc = run_request(srv, me, *job, &freed);
        job->t_end = Clock::now();
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            job->stats.status = rc;
            job->stats.slot = w;
            job->stats.queue_ms = std::chrono::duration<double, std::milli>(job->t_start - job->t_submit).count();
            job->stats.run_ms = std::chrono::duration<double, std::milli>(job->t_end - job->t_start).count();
            job->stats.latency_ms = std::chrono::duration<double, std::milli>(job->t_end - job->t_submit).count();
            job->done = true;
            srv->in_use -= freed;
            me.job.reset();
            me.has_job = false;
            me.hit = false;
        }
        srv->cv_done.notify_all();
        srv->cv_admit.notify_all();
    }
}

// the idle slot holding the request's key, or -1
int resident_slot(grmp_server srv, const Request &q) {
    if (q.key == 0) return -1;
    for (size_t w = 0; w < srv->workers.size(); w++) {
        const Worker &wk = srv->workers[w];
        if (wk.has_job) continue;
        for (const auto &e : wk.cache)
            if (e.key == q.key && e.sig == q.sig) return (int)w;
    }
    return -1;
}

// Drops the least recently used resident entry of an idle slot (not the one
// `keep` names); false when there is none.  Called with srv->mu held.
bool evict_one(grmp_server srv, int keep_w, uint64_t keep_key) {
    int bw = -1;
    size_t bi = 0;
    uint64_t best = UINT64_MAX;
    for (size_t w = 0; w < srv->workers.size(); w++) {
        Worker &wk = srv->workers[w];
        if (wk.has_job) continue;
        for (size_t i = 0; i < wk.cache.size(); i++) {
            if ((int)w == keep_w && wk.cache[i].key == keep_key) continue;
            if (wk.cache[i].last_use < best) {
                best = wk.cache[i].last_use;
                bw = (int)w;
                bi = i;
            }
        }
    }
    if (bw < 0) return false;
    Worker &wk = srv->workers[bw];
    srv->in_use -= wk.cache[bi].bytes;
    destroy_resident(wk.cache[bi]);   // the slot is idle: its context is not in use
    wk.cache.erase(wk.cache.begin() + bi);
    return true;
}

void admit_loop(grmp_server srv) {
    std::unique_lock<std::mutex> lk(srv->mu);
    while (true) {
        srv->cv_admit.wait(lk, [&] {
            if (srv->stop) return true;
            if (srv->queue.empty()) return false;
            bool idle = false;
            for (auto &w : srv->workers) idle = idle || !w.has_job;
            if (!idle) return false;
            const auto &q = *srv->queue.front();
            if (resident_slot(srv, q) >= 0) return true;   // runs on its resident data: no new memory
            while (srv->in_use + q.bytes > srv->budget && evict_one(srv, -1, 0)) {
            }
            return srv->in_use + q.bytes <= srv->budget || srv->in_use == 0;
        });
        if (srv->stop) return;
        // first come, first served; the head waits for memory (no starvation)
        auto job = srv->queue.front();
        srv->queue.pop_front();
        const int rw = resident_slot(srv, *job);
        int chosen = rw;
        if (chosen < 0)
            for (size_t w = 0; w < srv->workers.size(); w++)
                if (!srv->workers[w].has_job) {
                    chosen = (int)w;
                    break;
                }
        Worker &wk = srv->workers[chosen];
        wk.job = job;
        wk.has_job = true;
        wk.hit = rw >= 0;
        if (rw < 0) srv->in_use += job->bytes;
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
    if ((q->dim != 2 && q->dim != 3) || q->nverts <= 0 || q->ncells <= 0 || q->ndofs < 0) return GRMP_ERR_INVALID_ARG;
    if (grmp_fe_ldofs(q->fe_kind, q->dim, q->ncomponents) <= 0) return GRMP_ERR_UNSUPPORTED;
    if (q->ndofs == 0 && q->fe_kind != GRMP_FE_H1P1 && q->fe_kind != GRMP_FE_H1P2) return GRMP_ERR_INVALID_ARG;
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
    if (!srv || !q || !id || !q->coords || !q->cells || q->nterms <= 0 || q->nterms > GRMP_MAX_TERMS || !q->terms)
        return GRMP_ERR_INVALID_ARG;
    if ((q->dim != 2 && q->dim != 3) || q->nverts <= 0 || q->ncells <= 0 || q->nfixed < -1)
        return GRMP_ERR_INVALID_ARG;
    if (q->celldofs ? q->ndofs <= 0 : (q->fe_kind != GRMP_FE_H1P1 && q->fe_kind != GRMP_FE_H1P2))
        return GRMP_ERR_INVALID_ARG;   // a device-built DoF map: H1P1 / H1P2
    if (q->nfixed > 0 && !q->fixed) return GRMP_ERR_INVALID_ARG;
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
    r->device_dofmap = q->celldofs == nullptr;
    if (q->celldofs) r->celldofs.assign(q->celldofs, q->celldofs + (size_t)q->ncells * ld);
    else r->ndofs = 0;
    r->all_boundary = q->nfixed == -1;
    if (q->nfixed > 0) r->fixed.assign(q->fixed, q->fixed + q->nfixed);
    r->key = q->mesh_key;
    // operator structure: the pattern depends on it (and on the mesh / element the key stands for)
    uint64_t sig = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { sig = (sig ^ v) * 1099511628211ull; };
    mix((uint64_t)q->dim);
    mix((uint64_t)q->fe_kind);
    mix((uint64_t)q->ncomponents);
    mix((uint64_t)q->nverts);
    mix((uint64_t)q->ncells);
    mix((uint64_t)(q->celldofs != nullptr));
    mix((uint64_t)q->ndofs);
    mix((uint64_t)q->nterms);
    for (int i = 0; i < q->nterms; i++) {
        mix((uint64_t)q->terms[i].op_kind);
        mix((uint64_t)q->terms[i].symmetric);
        mix((uint64_t)q->terms[i].bonus_quadorder);
    }
    r->sig = sig;
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
    if (stats) *stats = r->stats;
    if (!x_out) return r->stats.status;   // a query: the result stays for a later wait
    if (!r->x.empty()) std::memcpy(x_out, r->x.data(), r->x.size() * sizeof(double));
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
    for (auto &w : srv->workers) {
        for (auto &e : w.cache) destroy_resident(e);
        w.cache.clear();
        grmp_destroy_context(w.ctx);
    }
    delete srv;
    return GRMP_OK;
}

}  // extern "C"
