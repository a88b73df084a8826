// server.cu -- request server with continuous batching (serving extension;
// no counterpart in the reference, where one ogs process runs one deck).
//
// Flow and transport solve requests arrive at any time.  Each request
// belongs to a class (mesh, kind, Dirichlet set) registered once; its own
// data is a conductivity field on the device, a tolerance and an output
// array.  The server keeps a pool of equation systems ("slots") per class,
// each with its own CUDA stream, matrices and Krylov state resident on the
// device, and walks one scheduling round per ogs_gpu_server_progress call:
//
//   * every running request is polled without blocking (ogs_gpu_solve_poll:
//     the next chunk of iterations is enqueued as soon as the GPU reached the
//     previous decision point), finished ones release their slot;
//   * queued requests are admitted in arrival order as slots free up: an
//     idle slot of the class is reused, or a new one is created while the
//     device bytes of all slots stay within the HBM budget (idle slots of
//     other classes are released, least recently used first, to make room);
//   * admission enqueues the whole request -- initial guess, assembly,
//     Dirichlet elimination, (for transport) Gauss-point flux, start of the
//     solve -- on the slot's stream with no host wait.
//
// So requests that arrive while others run join at the next round, and the
// work of all admitted requests overlaps on the GPU (one stream each).  A
// request runs exactly the kernels, launch shapes and order of the
// single-system API on a system of its own, so its result does not depend on
// what else is in flight.
//
// Dynamic batching (OGS_SERVER_BATCH): steady flow classes on a regular hex
// lattice with heads given on the two x faces are the Monte-Carlo batch's
// problem (batch.cu).  When two or more queued requests of such a class
// with the same tolerance wait at admission, up to kMaxServerBatch of them
// are assembled and solved together by one persistent batch launch (the
// batch object of that class, size and tolerance is kept for reuse).
//
// FP32-inner requests are solved to a tenth of their tolerance: two solves
// stopped at |r|/|b| < tol differ by up to cond(A) tol, and the tighter
// internal stop keeps a served result within the FP64 path's accuracy.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "common.cuh"

namespace ogs {
constexpr double kServedTolFactor = 0.1;  // internal stop of FP32-inner requests, times the tolerance
constexpr int kMaxServerBatch = 32;       // requests per batch launch at most
cudaStream_t system_stream(ogs_system* s);
int64_t system_rows(const ogs_system* s);
size_t system_bytes(const ogs_mesh* m, bool fp32);
void system_reset_request(ogs_system* s, double tol);
ogs_status system_upload_dirichlet(ogs_system* s, const int64_t* rows, const double* vals, int64_t n, int32_t mode);
ogs_status system_enqueue_assembly(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                   const double* u0, const double* gpv);
ogs_status system_enqueue_velocity(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                   const double* u, double* q);
ogs_status system_element_status(const ogs_system* s);
}  // namespace ogs

using namespace ogs;

namespace {

using Clock = std::chrono::steady_clock;

struct SrvClass
{
    ogs_server_class c;
    std::vector<int64_t> bc_rows;
    std::vector<double> bc_vals;
    double* x0 = nullptr;      // initial guess (Dirichlet values, else 0), device
    double* u_flow = nullptr;  // transport: head field of the Gauss-point flux, device
    size_t bytes = 0;          // device bytes of one slot
    int64_t n = 0, ngp = 0, ne = 0;
    int priority = 0;          // CUDA stream priority of its slots
    bool fp64_only = false;    // an FP32-inner solve of the class fell back to FP64
    // the Monte-Carlo batch's problem (steady flow on a hex lattice, heads on
    // the two x faces): lattice, cells, spacing and face heads
    bool batchable = false;
    int gx = 0, gy = 0, gz = 0;
    int64_t cells = 0;
    double hx = 0.0, hy = 0.0, hz = 0.0, h_left = 0.0, h_right = 0.0;
};

// a batch object kept for reuse: class, size, tolerance
struct SrvBatch
{
    int cls = -1, count = 0;
    double tol = 0.0;
    ogs_batch* b = nullptr;
    double* k_all = nullptr;   // gathered conductivities, device
    double* heads = nullptr;   // heads of all realisations, device
    size_t bytes = 0;
};

struct SrvSlot
{
    int cls = -1;
    ogs_system* sys = nullptr;
    double* q = nullptr;       // transport: Gauss-point flux
    cudaStream_t stream = nullptr;  // owned by the server, priority by class size
    int precision = -1;        // OGS_PRECISION_* its system is configured for
    bool busy = false;
    int64_t last_used = 0;
};

struct SrvReq
{
    int cls = 0;
    const double* elem_k = nullptr;
    double* out = nullptr;
    double tol = 0.0;
    int state = 0;             // 0 queued, 1 running, 2 done
    int slot = -1;
    ogs_status status = OGS_OK;
    ogs_solve_stats st{};
    int batch_size = 0;        // requests of the batch launch that served it (0: a slot)
    int precision = -1;        // OGS_PRECISION_* it was solved in
    Clock::time_point t_submit, t_admit, t_done;
};

}  // namespace

struct ogs_server
{
    size_t budget = 0, used = 0;
    int max_active = 0;
    int flags = 0;             // OGS_SERVER_* policy bits
    std::vector<SrvClass> classes;
    std::vector<SrvSlot> slots;
    std::vector<SrvBatch> batches;
    std::vector<SrvReq> reqs;
    std::deque<int64_t> queue;
    std::vector<int64_t> running;
    int64_t tick = 0;
    int64_t completed = 0;
    int64_t batched = 0;       // requests served by batch launches
    cudaStream_t batch_stream = nullptr;  // every batch object's copies and launches
};

namespace {

void release_slot(ogs_server* S, size_t k)
{
    SrvSlot& sl = S->slots[k];
    if (sl.sys) ogs_gpu_system_destroy(sl.sys);
    cudaFree(sl.q);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    S->used -= S->classes[sl.cls].bytes;
    S->slots.erase(S->slots.begin() + k);
    for (int64_t id : S->running)
        if (S->reqs[id].slot > (int)k) S->reqs[id].slot -= 1;
}

// the solver configuration of a class's slots: the class's own, or FP64 CG
// of the same method once an FP32-inner solve of the class fell back
ogs_status configure_slot(SrvSlot& sl, const SrvClass& C)
{
    ogs_solver_config cfg = C.c.solver;
    if (C.fp64_only) cfg.precision = OGS_PRECISION_FP64;
    if (sl.precision == cfg.precision) return OGS_OK;
    const ogs_status st = ogs_gpu_configure(sl.sys, &cfg);
    if (st == OGS_OK) sl.precision = cfg.precision;
    return st;
}

// a slot of class c, while fewer than max_active requests run: an idle
// one, or a new one within the budget
int acquire_slot(ogs_server* S, int c)
{
    if ((int)S->running.size() >= S->max_active) return -1;
    for (size_t k = 0; k < S->slots.size(); k++)
        if (!S->slots[k].busy && S->slots[k].cls == c) return (int)k;
    const SrvClass& C = S->classes[c];
    while (S->used + C.bytes > S->budget)
    {
        int lru = -1;
        for (size_t k = 0; k < S->slots.size(); k++)
            if (!S->slots[k].busy && (lru < 0 || S->slots[k].last_used < S->slots[lru].last_used)) lru = (int)k;
        if (lru < 0) return -1;
        release_slot(S, lru);
    }
    SrvSlot sl;
    sl.cls = c;
    if (cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, C.priority) != cudaSuccess)
    {
        cudaGetLastError();
        set_error("server: stream creation failed");
        return -2;
    }
    if (ogs_gpu_system_create(C.c.mesh, sl.stream, &sl.sys))
    {
        cudaStreamDestroy(sl.stream);
        return -2;
    }
    if (configure_slot(sl, C) ||
        system_upload_dirichlet(sl.sys, C.bc_rows.data(), C.bc_vals.data(), (int64_t)C.bc_rows.size(),
                                C.c.bc_mode))
    {
        ogs_gpu_system_destroy(sl.sys);
        cudaStreamDestroy(sl.stream);
        return -2;
    }
    if (C.c.kind == OGS_REQUEST_TRANSPORT && cudaMalloc(&sl.q, (size_t)C.ne * C.ngp * 3 * sizeof(double)) != cudaSuccess)
    {
        cudaGetLastError();
        ogs_gpu_system_destroy(sl.sys);
        cudaStreamDestroy(sl.stream);
        set_error("server: no device memory for a transport slot");
        return -2;
    }
    S->used += C.bytes;
    S->slots.push_back(sl);
    return (int)S->slots.size() - 1;
}

ogs_status start(ogs_server* S, int64_t id, int k)
{
    SrvReq& R = S->reqs[id];
    SrvSlot& sl = S->slots[k];
    const SrvClass& C = S->classes[R.cls];
    ogs_system* s = sl.sys;
    cudaStream_t st = system_stream(s);
    ogs_status e = configure_slot(sl, C);
    if (e) return e;
    R.precision = sl.precision;
    // FP32 classes stop at a tenth of the tolerance, also when served in FP64
    // after a fallback, so their heads stay as close to the converged ones
    system_reset_request(s, C.c.solver.precision != OGS_PRECISION_FP64 ? R.tol * kServedTolFactor : R.tol);
    OGS_CUDA_TRY(cudaMemcpyAsync(R.out, C.x0, C.n * sizeof(double), cudaMemcpyDefault, st));
    if (C.c.kind == OGS_REQUEST_TRANSPORT)
    {
        if ((e = system_enqueue_velocity(s, &C.c.flow_params, R.elem_k, C.u_flow, sl.q))) return e;
        if ((e = system_enqueue_assembly(s, &C.c.params, nullptr, C.x0, sl.q))) return e;
    }
    else if ((e = system_enqueue_assembly(s, &C.c.params, R.elem_k, C.x0, nullptr)))
        return e;
    return ogs_gpu_solve_begin(s, R.out);
}

// Smaller systems get higher stream priorities: their short kernels are
// scheduled ahead of the blocks of large solves, so a small request is not
// time-sliced behind every large one in flight (shortest job first at the
// block scheduler).  Classes are ranked by rows, spread over the device's
// priority range in factors of four.
void assign_priorities(ogs_server* S)
{
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
    {
        cudaGetLastError();
        return;
    }
    const int levels = least - greatest + 1;  // greatest is the most negative
    int64_t nmin = INT64_MAX;
    for (const SrvClass& C : S->classes) nmin = std::min(nmin, C.n);
    nmin = std::max<int64_t>(1, nmin);
    for (SrvClass& C : S->classes)
    {
        // factors of four above the smallest class; the smallest get the
        // greatest priority
        int step = 0;
        for (int64_t v = C.n; v >= 4 * nmin && step < levels - 1; v /= 4) step++;
        C.priority = greatest + step;
    }
}

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Is the class the Monte-Carlo batch's problem?  Steady GROUNDWATER_FLOW
// (no storage) solved by FP32-inner CG + Jacobi on a regular hex lattice,
// symmetric Dirichlet on exactly the nodes of the x = 0 and x = max faces
// with one head per face.
void detect_batchable(SrvClass& C, const ogs_mesh* m)
{
    const ogs_server_class& c = C.c;
    C.batchable = false;
    if (c.kind != OGS_REQUEST_FLOW || c.params.pcs_type != OGS_PCS_GROUNDWATER_FLOW || c.params.storage != 0.0 ||
        c.solver.precision != OGS_PRECISION_FP32_REFINED || c.solver.method != OGS_LS_CG ||
        c.solver.precond != OGS_PRECOND_JACOBI || c.bc_mode != OGS_DIRICHLET_SYMMETRIC || !m->grid ||
        m->gx < 3 || m->gy < 3 || m->gz < 3)
        return;
    const int64_t face = (int64_t)m->gy * m->gz;
    if ((int64_t)C.bc_rows.size() != 2 * face) return;
    std::vector<unsigned char> seen((size_t)C.n, 0);
    double hl = 0.0, hr = 0.0;
    bool have_l = false, have_r = false;
    for (size_t q = 0; q < C.bc_rows.size(); q++)
    {
        const int64_t r = C.bc_rows[q];
        if (r < 0 || r >= C.n || seen[r]) return;
        seen[r] = 1;
        const int64_t ix = r % m->gx;
        if (ix != 0 && ix != m->gx - 1) return;
        double& h = ix == 0 ? hl : hr;
        bool& have = ix == 0 ? have_l : have_r;
        if (have && h != C.bc_vals[q]) return;
        h = C.bc_vals[q];
        have = true;
    }
    if (!have_l || !have_r) return;
    C.gx = m->gx; C.gy = m->gy; C.gz = m->gz;
    C.cells = (int64_t)(m->gx - 1) * (m->gy - 1) * (m->gz - 1);
    C.hx = m->ghx; C.hy = m->ghy; C.hz = m->ghz;
    C.h_left = hl;
    C.h_right = hr;
    C.batchable = true;
}

void release_batch(SrvBatch& B)
{
    if (B.b) ogs_gpu_batch_destroy(B.b);
    cudaFree(B.k_all);
    cudaFree(B.heads);
    B = SrvBatch();
}

// the batch object of (class, count, tol): kept one, or a new one within the
// budget (idle slots released, least recently used first, to make room).
// Returns -1 when it does not fit.
int acquire_batch(ogs_server* S, int c, int count, double tol, const std::vector<int64_t>& ids)
{
    for (size_t k = 0; k < S->batches.size(); k++)
    {
        const SrvBatch& B = S->batches[k];
        if (B.cls == c && B.count == count && B.tol == tol) return (int)k;
    }
    const SrvClass& C = S->classes[c];
    const size_t rows = (size_t)C.n * count, elems = (size_t)C.cells * count;
    const size_t bytes = rows * (14 * 8 + 3 * 8 + 21 * 4 + 8) + 2 * elems * 8;
    while (S->used + bytes > S->budget)
    {
        int lru = -1;
        for (size_t k = 0; k < S->slots.size(); k++)
            if (!S->slots[k].busy && (lru < 0 || S->slots[k].last_used < S->slots[lru].last_used)) lru = (int)k;
        if (lru < 0) return -1;
        release_slot(S, lru);
    }
    ogs_batch_config cfg;
    std::memset(&cfg, 0, sizeof cfg);
    cfg.hx = C.hx; cfg.hy = C.hy; cfg.hz = C.hz;
    cfg.time_unit_factor = C.c.params.time_unit_factor;
    cfg.tol = tol * kServedTolFactor;
    cfg.inner_tol = C.c.solver.inner_tol;
    cfg.max_iter = C.c.solver.max_iter;
    std::vector<ogs_batch_realisation> reals(count);
    for (int r = 0; r < count; r++)
    {
        std::memset(&reals[r], 0, sizeof reals[r]);
        reals[r].nx = C.gx; reals[r].ny = C.gy; reals[r].nz = C.gz;
        reals[r].elem_k = S->reqs[ids[r]].elem_k;
        reals[r].h_left = C.h_left;
        reals[r].h_right = C.h_right;
    }
    SrvBatch B;
    B.cls = c;
    B.count = count;
    B.tol = tol;
    B.bytes = bytes;
    if (!S->batch_stream)
    {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (cudaStreamCreateWithPriority(&S->batch_stream, cudaStreamNonBlocking, greatest) != cudaSuccess)
        {
            cudaGetLastError();
            S->batch_stream = nullptr;
            return -1;
        }
    }
    if (ogs_gpu_batch_create(&cfg, reals.data(), count, S->batch_stream, &B.b) != OGS_OK) return -1;
    if (cudaMalloc(&B.k_all, elems * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&B.heads, rows * sizeof(double)) != cudaSuccess)
    {
        cudaGetLastError();
        release_batch(B);
        return -1;
    }
    S->used += bytes;
    S->batches.push_back(B);
    return (int)S->batches.size() - 1;
}

// one batch launch for the requests ids (same class and tolerance): their
// conductivities gathered, assembly and solve, heads scattered to their
// outputs, every copy on the server's batch stream (the batch object's
// own), so the gather is complete before the batch reads it and the
// scatter before the next batch overwrites its heads.  Blocks until done.
ogs_status run_batch(ogs_server* S, int k, const std::vector<int64_t>& ids)
{
    SrvBatch& B = S->batches[k];
    const SrvClass& C = S->classes[B.cls];
    cudaStream_t st = S->batch_stream;
    for (size_t r = 0; r < ids.size(); r++)
        OGS_CUDA_TRY(cudaMemcpyAsync(B.k_all + r * C.cells, S->reqs[ids[r]].elem_k, C.cells * sizeof(double),
                                     cudaMemcpyDefault, st));
    ogs_status e = ogs_gpu_batch_set_k(B.b, B.k_all);
    if (e) return e;
    std::vector<ogs_batch_stats> bs(ids.size());
    const ogs_status sst = ogs_gpu_batch_solve(B.b, bs.data());
    if (sst != OGS_OK && sst != OGS_NOT_CONVERGED && sst != OGS_NONFINITE && sst != OGS_BREAKDOWN) return sst;
    if ((e = ogs_gpu_batch_get_heads(B.b, B.heads))) return e;
    for (size_t r = 0; r < ids.size(); r++)
        OGS_CUDA_TRY(cudaMemcpyAsync(S->reqs[ids[r]].out, B.heads + r * C.n, C.n * sizeof(double),
                                     cudaMemcpyDefault, st));
    OGS_CUDA_TRY(cudaStreamSynchronize(st));
    for (size_t r = 0; r < ids.size(); r++)
    {
        SrvReq& R = S->reqs[ids[r]];
        std::memset(&R.st, 0, sizeof R.st);
        R.st.iterations = bs[r].iterations;
        R.st.status = bs[r].status;
        R.st.refinements = bs[r].refinements;
        R.st.rel_residual = bs[r].rel_residual;
        R.st.solve_ms = bs[r].finish_ms;
        R.st.fp32_operator = 0;
        R.status = (ogs_status)bs[r].status;
        R.precision = OGS_PRECISION_FP32_REFINED;
    }
    return OGS_OK;
}

}  // namespace

extern "C" ogs_status ogs_gpu_server_create(int64_t hbm_budget_bytes, int32_t max_active, int32_t flags,
                                            ogs_server** out)
{
    if (!out || max_active <= 0) { set_error("server_create: bad arguments"); return OGS_BAD_ARG; }
    ogs_server* S = new ogs_server;
    if (hbm_budget_bytes <= 0)
    {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { delete S; set_error("server_create: no device"); return OGS_CUDA_ERROR; }
        S->budget = (size_t)(0.8 * (double)fr);
    }
    else
        S->budget = (size_t)hbm_budget_bytes;
    S->max_active = max_active;
    S->flags = flags;
    *out = S;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_destroy(ogs_server* S)
{
    if (!S) return OGS_OK;
    for (SrvSlot& sl : S->slots)
    {
        if (sl.sys) ogs_gpu_system_destroy(sl.sys);
        cudaFree(sl.q);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (SrvBatch& B : S->batches) release_batch(B);
    if (S->batch_stream) cudaStreamDestroy(S->batch_stream);
    for (SrvClass& C : S->classes)
    {
        cudaFree(C.x0);
        cudaFree(C.u_flow);
    }
    delete S;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_add_class(ogs_server* S, const ogs_server_class* c, int32_t* class_id)
{
    if (!S || !c || !c->mesh || !class_id || c->n_bc < 0 || (c->n_bc && (!c->bc_rows || !c->bc_values)))
    {
        set_error("server_add_class: bad arguments");
        return OGS_BAD_ARG;
    }
    if (c->kind != OGS_REQUEST_FLOW && c->kind != OGS_REQUEST_TRANSPORT)
    {
        set_error("server_add_class: kind %d", c->kind);
        return OGS_BAD_ARG;
    }
    SrvClass C;
    C.c = *c;
    int64_t n = 0, nnz = 0;
    ogs_gpu_mesh_info(c->mesh, &n, &nnz);
    C.n = n;
    C.ngp = ogs_gpu_mesh_gauss_points(c->mesh);
    C.ne = c->n_elements;
    C.bc_rows.assign(c->bc_rows, c->bc_rows + c->n_bc);
    C.bc_vals.assign(c->bc_values, c->bc_values + c->n_bc);
    std::vector<double> x0(n, 0.0);
    for (int64_t q = 0; q < c->n_bc; q++)
        if (c->bc_rows[q] >= 0 && c->bc_rows[q] < n) x0[c->bc_rows[q]] = c->bc_values[q];
    OGS_CUDA_TRY(cudaMalloc(&C.x0, std::max<int64_t>(1, n) * sizeof(double)));
    OGS_CUDA_TRY(cudaMemcpy(C.x0, x0.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    if (c->kind == OGS_REQUEST_TRANSPORT)
    {
        if (!c->flow_head || C.ne <= 0)
        {
            cudaFree(C.x0);
            set_error("server_add_class: transport needs flow_head and n_elements");
            return OGS_BAD_ARG;
        }
        OGS_CUDA_TRY(cudaMalloc(&C.u_flow, std::max<int64_t>(1, n) * sizeof(double)));
        OGS_CUDA_TRY(cudaMemcpy(C.u_flow, c->flow_head, n * sizeof(double), cudaMemcpyDefault));
        // a device-to-device copy returns before it completes: finish it
        // before slots on other streams read the field
        OGS_CUDA_TRY(cudaStreamSynchronize(cudaStreamLegacy));
    }
    C.bytes = system_bytes(c->mesh, c->solver.precision != OGS_PRECISION_FP64);
    detect_batchable(C, c->mesh);
    if (c->kind == OGS_REQUEST_TRANSPORT) C.bytes += (size_t)C.ne * C.ngp * 3 * sizeof(double);
    C.c.bc_rows = nullptr;
    C.c.bc_values = nullptr;
    C.c.flow_head = nullptr;
    S->classes.push_back(std::move(C));
    *class_id = (int32_t)S->classes.size() - 1;
    if (S->flags & OGS_SERVER_PRIORITY) assign_priorities(S);
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_reserve(ogs_server* S, int32_t class_id, int32_t n_slots)
{
    if (!S || class_id < 0 || class_id >= (int32_t)S->classes.size() || n_slots < 0)
    {
        set_error("server_reserve: bad arguments");
        return OGS_BAD_ARG;
    }
    int have = 0;
    for (const SrvSlot& sl : S->slots) have += sl.cls == class_id;
    std::vector<int> made;
    for (; have < n_slots; have++)
    {
        const int k = acquire_slot(S, class_id);
        if (k == -2) return OGS_OOM;
        if (k < 0) break;  // budget reached
        S->slots[k].busy = true;  // keep acquire_slot from handing it out again in this loop
        made.push_back(k);
    }
    for (int k : made) S->slots[k].busy = false;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_submit(ogs_server* S, int32_t class_id, const double* elem_k, double tol,
                                            double* out, int64_t* request_id)
{
    if (!S || !out || !request_id || class_id < 0 || class_id >= (int32_t)S->classes.size() || !(tol > 0.0) ||
        !elem_k)
    {
        set_error("server_submit: bad arguments");
        return OGS_BAD_ARG;
    }
    SrvReq R;
    R.cls = class_id;
    R.elem_k = elem_k;
    R.out = out;
    R.tol = tol;
    R.t_submit = Clock::now();
    S->reqs.push_back(R);
    *request_id = (int64_t)S->reqs.size() - 1;
    S->queue.push_back(*request_id);
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_progress(ogs_server* S, int32_t* n_running, int32_t* n_queued)
{
    if (!S) { set_error("server_progress: NULL server"); return OGS_BAD_ARG; }
    S->tick += 1;
    // running requests: non-blocking polls
    for (size_t q = 0; q < S->running.size();)
    {
        const int64_t id = S->running[q];
        SrvReq& R = S->reqs[id];
        SrvSlot& sl = S->slots[R.slot];
        int32_t fin = 0;
        ogs_status st = ogs_gpu_solve_poll(sl.sys, &fin);
        if (st == OGS_OK && !fin)
        {
            q++;
            continue;
        }
        ogs_status es = ogs_gpu_solve_end(sl.sys, &R.st);
        R.status = st != OGS_OK ? st : es;
        if (R.status == OGS_OK || R.status == OGS_NONFINITE)
        {
            const ogs_status ef = system_element_status(sl.sys);
            if (ef) R.status = ef;
        }
        R.t_done = Clock::now();
        R.state = 2;
        if ((S->flags & OGS_SERVER_PRECISION_FALLBACK) && R.st.fp64_fallback)
            S->classes[R.cls].fp64_only = true;
        sl.busy = false;
        sl.last_used = S->tick;
        S->completed += 1;
        S->running.erase(S->running.begin() + q);
    }
    // admission: arrival order, or smallest class first (arrival order
    // among equals) with OGS_SERVER_SJF
    while (!S->queue.empty())
    {
        size_t pick = 0;
        if (S->flags & OGS_SERVER_SJF)
            for (size_t q = 1; q < S->queue.size(); q++)
                if (S->classes[S->reqs[S->queue[q]].cls].n < S->classes[S->reqs[S->queue[pick]].cls].n) pick = q;
        const int64_t id = S->queue[pick];
        SrvReq& R = S->reqs[id];
        if ((S->flags & OGS_SERVER_BATCH) && S->classes[R.cls].batchable && !S->classes[R.cls].fp64_only)
        {
            // same class and tolerance, in queue order from the picked one
            std::vector<size_t> at;
            for (size_t q = pick; q < S->queue.size() && (int)at.size() < kMaxServerBatch; q++)
            {
                const SrvReq& O = S->reqs[S->queue[q]];
                if (O.cls == R.cls && O.tol == R.tol) at.push_back(q);
            }
            if (at.size() >= 2)
            {
                std::vector<int64_t> ids;
                for (size_t q : at) ids.push_back(S->queue[q]);
                const int bk = acquire_batch(S, R.cls, (int)ids.size(), R.tol, ids);
                if (bk >= 0)
                {
                    for (size_t j = at.size(); j-- > 0;) S->queue.erase(S->queue.begin() + at[j]);
                    const Clock::time_point ta = Clock::now();
                    for (int64_t q : ids)
                    {
                        S->reqs[q].state = 1;
                        S->reqs[q].t_admit = ta;
                    }
                    const ogs_status bst = run_batch(S, bk, ids);
                    const Clock::time_point td = Clock::now();
                    for (int64_t q : ids)
                    {
                        SrvReq& Q = S->reqs[q];
                        if (bst) Q.status = bst;
                        Q.state = 2;
                        Q.t_done = td;
                        Q.batch_size = (int)ids.size();
                    }
                    S->completed += (int64_t)ids.size();
                    S->batched += (int64_t)ids.size();
                    continue;
                }
            }
        }
        const int k = acquire_slot(S, R.cls);
        if (k == -2) return OGS_OOM;
        if (k < 0) break;
        S->queue.erase(S->queue.begin() + pick);
        S->slots[k].busy = true;
        R.slot = k;
        R.state = 1;
        R.t_admit = Clock::now();
        ogs_status st = start(S, id, k);
        if (st)
        {
            // the request fails on its own; its slot goes back to the pool
            R.status = st;
            R.state = 2;
            R.t_done = Clock::now();
            S->slots[k].busy = false;
            S->completed += 1;
            cudaStreamSynchronize(system_stream(S->slots[k].sys));
            continue;
        }
        S->running.push_back(id);
    }
    if (n_running) *n_running = (int32_t)S->running.size();
    if (n_queued) *n_queued = (int32_t)S->queue.size();
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_result(const ogs_server* S, int64_t request_id, ogs_server_result* r)
{
    if (!S || !r || request_id < 0 || request_id >= (int64_t)S->reqs.size())
    {
        set_error("server_result: bad arguments");
        return OGS_BAD_ARG;
    }
    const SrvReq& R = S->reqs[request_id];
    std::memset(r, 0, sizeof *r);
    r->state = R.state;
    r->status = R.status;
    if (R.state == 2)
    {
        r->iterations = R.st.iterations;
        r->refinements = R.st.refinements;
        r->rel_residual = R.st.rel_residual;
        r->latency_ms = ms_between(R.t_submit, R.t_done);
        r->queue_ms = R.slot >= 0 || R.batch_size ? ms_between(R.t_submit, R.t_admit) : r->latency_ms;
        r->solve_ms = R.st.solve_ms;
        r->batch_size = R.batch_size;
        r->precision = R.precision;
        r->fp64_fallback = R.st.fp64_fallback;
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_server_info(const ogs_server* S, ogs_server_info* info)
{
    if (!S || !info) { set_error("server_info: bad arguments"); return OGS_BAD_ARG; }
    std::memset(info, 0, sizeof *info);
    info->slots = (int32_t)S->slots.size();
    info->running = (int32_t)S->running.size();
    info->queued = (int32_t)S->queue.size();
    info->completed = S->completed;
    info->batched = S->batched;
    for (const SrvClass& C : S->classes) info->fp64_classes += C.fp64_only ? 1 : 0;
    info->bytes_used = (int64_t)S->used;
    info->bytes_budget = (int64_t)S->budget;
    return OGS_OK;
}
