// C ABI of libspicier_gb300 (declarations and reference citations in
// include/spicier_gb300.h).  Host-side orchestration only: argument checks,
// the device copy of a circuit, scratch management and kernel launches.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "internal.h"
#include "ladder.cuh"
#include "transient_fixed.cuh"
#include "ac.cuh"
#include "powergrid.cuh"

using namespace sp;

namespace {

int fail(sp_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

int cuda_fail(sp_ctx* ctx, cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? SP_ERR_MEMORY_ALLOC : SP_ERR_BACKEND;
    return fail(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

#define SP_CUDA(ctx, expr, what)                           \
    do {                                                   \
        cudaError_t e_ = (expr);                           \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int ensure_scratch(sp_ctx* ctx, size_t bytes) {
    return ::grow_buffer(ctx, &ctx->scratch, &ctx->scratch_bytes, bytes, "scratch");
}

// Threads per block of the thread-per-sample kernels: the largest multiple of
// 32 up to 128 whose shared-memory work area stays within ~110 KB (two blocks
// per SM on a 228 KB SM).
int pick_block(size_t per_thread, int max_smem) {
    int block = 128;
    while (block > 32 && per_thread * block > 110 * 1024) block -= 32;
    if (per_thread * block > (size_t)max_smem) return 0;
    return block;
}


}  // namespace

// Grow a context-owned device buffer (grow-only).  Inside a call's ordering
// guard the old buffer is freed and the new one allocated in the calling
// stream's order (cudaFreeAsync / cudaMallocAsync): the stream already waits
// for every earlier user of the context's buffers, so nothing else on the
// device is stalled.  A stream being captured into a CUDA graph cannot grow
// them (the allocation would belong to the graph); outside a guard the growth
// waits for the device.
int grow_buffer(sp_ctx* ctx, void** buf, size_t* have, size_t bytes, const char* what) {
    if (bytes <= *have) return SP_OK;
    if (ctx->order_active && ctx->order_capturing)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT,
                    "the context's %s must grow to %zu bytes while the stream is being captured: make the same "
                    "call once before the capture",
                    what, bytes);
    const size_t want = align256(bytes + bytes / 4);
    void* p = nullptr;
    cudaError_t e;
    if (ctx->order_active) {
        if (*buf) {
            e = cudaFreeAsync(*buf, ctx->order_stream);
            if (e != cudaSuccess) return cuda_fail(ctx, e, what);
        }
        *buf = nullptr;
        *have = 0;
        e = cudaMallocAsync(&p, want, ctx->order_stream);
    } else {
        if (*buf) {
            e = cudaDeviceSynchronize();
            if (e != cudaSuccess) return cuda_fail(ctx, e, what);
            cudaFreeAsync(*buf, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
        }
        *buf = nullptr;
        *have = 0;
        e = cudaMallocAsync(&p, want, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    *buf = p;
    *have = want;
    return SP_OK;
}

int tune_get(sp_ctx* ctx, const char* name, long long n, int dflt) {
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    if (ctx->tune.empty()) return dflt;
    auto it = ctx->tune.find(std::string(name) + "@" + std::to_string(tune_bucket(n)));
    return it == ctx->tune.end() ? dflt : it->second;
}

extern "C" {

const char* sp_version(void) { return "spicier-gb300 0.1.0 sm_103a"; }

int sp_backend_type(void) { return SP_BACKEND_GB300; }

int sp_ctx_create(int device, sp_ctx** out) {
    if (!out) return SP_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SP_ERR_NO_BACKEND;
    if (device < 0 || device >= ndev) return SP_ERR_INVALID_ARGUMENT;
    sp_ctx* ctx = new sp_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->scratch_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = prepare_exact_kernels(ctx->max_smem);
    if (e == cudaSuccess) e = prepare_fast_kernels(ctx->max_smem);
    if (e != cudaSuccess) {
        delete ctx;
        return SP_ERR_BACKEND_INIT;
    }
    *out = ctx;
    return SP_OK;
}

int sp_ctx_destroy(sp_ctx* ctx) {
    if (!ctx) return SP_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaDeviceSynchronize();
    // both buffers come from the stream-ordered allocator
    if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->stream);
    if (ctx->aux) cudaFreeAsync(ctx->aux, ctx->stream);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->scratch_done) cudaEventDestroy(ctx->scratch_done);
    for (auto& r : ctx->recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    for (auto& kv : ctx->host_topos) sp_topology_destroy(kv.second);
    ctx->host_topos.clear();
    spec_release_all(ctx);
    delete ctx;
    return SP_OK;
}

const char* sp_ctx_last_error(const sp_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int sp_should_use_gpu(const sp_ctx* ctx, size_t matrix_size, size_t batch_size) {
    if (!ctx) return 0;
    return matrix_size >= ctx->cfg.min_matrix_size && batch_size >= ctx->cfg.min_batch_size;
}

int sp_get_config(const sp_ctx* ctx, sp_batch_config* out) {
    if (!ctx || !out) return SP_ERR_INVALID_ARGUMENT;
    *out = ctx->cfg;
    return SP_OK;
}

int sp_set_config(sp_ctx* ctx, const sp_batch_config* cfg) {
    if (!ctx || !cfg) return SP_ERR_INVALID_ARGUMENT;
    if (cfg->max_batch_per_launch == 0) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "max_batch_per_launch == 0");
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->cfg = *cfg;
    return SP_OK;
}

void sp_grid_config_default(sp_grid_config* c) {
    if (!c) return;
    *c = sp_grid_config{};
    c->rows = c->cols = 64;
    c->num_sinks = 512;
    c->max_newton = 30;
    c->restart = 30;
    c->max_krylov = 20000;
    c->precision = SP_PREC_FP64;
    c->r_lo = 0.5;
    c->r_hi = 2.0;
    c->r_scale_lo = 0.9;
    c->r_scale_hi = 1.1;
    c->vto_shift = 0.05;
    c->vdd = 1.0;
    c->strap_g = 1e3;
    c->vgs_lo = 0.8;
    c->vgs_hi = 1.2;
    c->vto = 0.7;
    c->kp = 110e-6;
    c->lambda = 0.04;
    c->w = 5e-6;
    c->l = 0.5e-6;
    c->v_reltol = 1e-3;
    c->v_abstol = 1e-6;
    c->i_abstol = 1e-12;
    c->krylov_tol = 1e-9;
    c->resid_target = 1e-9;
}

void sp_ladder_config_default(sp_ladder_config* c) {
    if (!c) return;
    *c = sp_ladder_config{};
    c->tstop = 100e-9;
    c->h_init = 1e-9;
    c->h_min = 1e-15;
    c->h_max = c->tstop / 100.0;  // AdaptiveTransientParams::for_tstop
    c->lte_reltol = 1e-3;
    c->lte_abstol = 1e-6;
    c->v_reltol = 1e-3;
    c->v_abstol = 1e-6;
    c->i_abstol = 1e-12;
    c->r_lo = 100.0;
    c->r_hi = 10e3;
    c->c_lo = 1e-12;
    c->c_hi = 100e-12;
    c->diode_is = 1e-14;
    c->diode_n = 1.0;
    c->pulse = sp_pulse{0.0, 1.8, 0.0, 1e-9, 1e-9, 10e-9, 20e-9};
    c->min_sections = 8;
    c->max_sections = 512;
    c->max_iterations = 50;
    c->max_steps = 200000;
    c->precision = SP_PREC_FP64;
    c->num_probe = 101;
}

void sp_newton_config_default(sp_newton_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->v_abstol = 1e-6;
    c->v_reltol = 1e-3;
    c->i_abstol = 1e-12;
    c->gmin = 1e-12;
    c->max_iterations = 50;
    c->precision = SP_PREC_FP64;
    c->fallback = SP_FALLBACK_GMIN | SP_FALLBACK_SOURCE;
    c->refine_steps = 0;
    c->gmin_initial = 1e-3;
    c->gmin_final = 1e-12;
    c->gmin_reduction = 10.0;
    c->gmin_max_attempts = 5;
    c->src_max_attempts = 5;
    c->src_initial = 0.1;
    c->src_step = 0.1;
    c->src_min_step = 0.01;
}

// ---------------------------------------------------------------------------
// solve_batch
// ---------------------------------------------------------------------------
static int ensure_aux(sp_ctx* ctx, size_t bytes) {
    return ::grow_buffer(ctx, &ctx->aux, &ctx->aux_bytes, bytes, "second buffer");
}

static int solve_batch_device_locked(sp_ctx* ctx, const double* d_m, const double* d_r, size_t n,
                                     size_t batch, double* d_x, uint8_t* d_s, int precision,
                                     int refine_steps, cudaStream_t st) {
    if (batch == 0) return SP_OK;
    if (n == 0) return fail(ctx, SP_ERR_INVALID_DIMENSION, "Expected n > 0, got 0");
    if (batch > ctx->cfg.max_batch_per_launch)
        return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %zu exceeds maximum %llu", batch,
                    (unsigned long long)ctx->cfg.max_batch_per_launch);
    if (n > (size_t)kMaxBatchLuN)
        return fail(ctx, SP_ERR_INVALID_DIMENSION, "n = %zu exceeds the batched dense LU limit %d", n,
                    kMaxBatchLuN);
    // one thread per system up to kMaxDenseN unknowns unless the tuner chose
    // the CTA-per-system kernel for this size (setting "lu.cta", 1 = CTA)
    const bool cta = n > (size_t)kMaxDenseN || tune_get(ctx, "lu.cta", (long long)n, 0) == 1;
    if (cta) {
        // one CTA per system, FP64 in the reference's order (both precisions)
        ProfScope prof(ctx, "lu_batch_cta", st);
        double* work = nullptr;
        int grid = (int)std::min<size_t>(batch, (size_t)ctx->num_sms * 8);
        if (lu_batch_cta_smem((int)n) > (size_t)ctx->max_smem - 1024) {
            const size_t per = lu_batch_cta_smem((int)n);
            grid = (int)std::max<size_t>(1, std::min<size_t>({batch, (size_t)ctx->num_sms * 2, ((size_t)4 << 30) / per}));
            int rc = ensure_aux(ctx, per * grid);
            if (rc) return rc;
            work = (double*)ctx->aux;
        }
        cudaError_t e = launch_lu_batch_cta(d_m, d_r, (int)n, batch, d_x, d_s, work, grid, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "solve_batch launch");
        return SP_OK;
    }
    ProfScope prof(ctx, precision == SP_PREC_MIXED ? "lu_batch_mixed" : "lu_batch_fp64", st);
    cudaError_t e = (precision == SP_PREC_MIXED)
                        ? launch_lu_batch_mixed(d_m, d_r, (int)n, batch, d_x, d_s, refine_steps, st)
                        : launch_lu_batch_exact(d_m, d_r, (int)n, batch, d_x, d_s, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "solve_batch launch");
    return SP_OK;
}

int sp_solve_batch_device(sp_ctx* ctx, const double* d_matrices, const double* d_rhs, size_t n,
                          size_t batch, double* d_solutions, uint8_t* d_singular_flags, int precision,
                          int refine_steps, void* stream) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    if (batch && (!d_matrices || !d_rhs || !d_solutions || !d_singular_flags))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return solve_batch_device_locked(ctx, d_matrices, d_rhs, n, batch, d_solutions, d_singular_flags,
                                     precision, refine_steps, (cudaStream_t)stream);
}

int sp_solve_batch(sp_ctx* ctx, const double* matrices, const double* rhs, size_t n, size_t batch,
                   double* solutions, uint64_t* singular_indices, uint64_t* num_singular) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    if (num_singular) *num_singular = 0;
    if (batch == 0) return SP_OK;
    if (!matrices || !rhs || !solutions) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    if (n == 0) return fail(ctx, SP_ERR_INVALID_DIMENSION, "Expected n > 0, got 0");
    size_t bm = align256(batch * n * n * 8), br = align256(batch * n * 8), bs = align256(batch);
    int rc = ensure_scratch(ctx, bm + 2 * br + bs);
    if (rc) return rc;
    ScratchOrder order(ctx, ctx->stream);
    char* base = (char*)ctx->scratch;
    double* d_m = (double*)base;
    double* d_r = (double*)(base + bm);
    double* d_x = (double*)(base + bm + br);
    uint8_t* d_s = (uint8_t*)(base + bm + 2 * br);
    cudaStream_t st = ctx->stream;
    SP_CUDA(ctx, cudaMemcpyAsync(d_m, matrices, batch * n * n * 8, cudaMemcpyHostToDevice, st), "H2D matrices");
    SP_CUDA(ctx, cudaMemcpyAsync(d_r, rhs, batch * n * 8, cudaMemcpyHostToDevice, st), "H2D rhs");
    rc = solve_batch_device_locked(ctx, d_m, d_r, n, batch, d_x, d_s, SP_PREC_FP64, 0, st);
    if (rc) return rc;
    std::vector<uint8_t> flags(batch);
    SP_CUDA(ctx, cudaMemcpyAsync(solutions, d_x, batch * n * 8, cudaMemcpyDeviceToHost, st), "D2H solutions");
    SP_CUDA(ctx, cudaMemcpyAsync(flags.data(), d_s, batch, cudaMemcpyDeviceToHost, st), "D2H flags");
    SP_CUDA(ctx, cudaStreamSynchronize(st), "solve_batch");
    uint64_t ns = 0;
    for (size_t i = 0; i < batch; ++i)
        if (flags[i]) {
            if (singular_indices) singular_indices[ns] = i;
            ++ns;
        }
    if (num_singular) *num_singular = ns;
    return SP_OK;
}

// ---------------------------------------------------------------------------
// Topology
// ---------------------------------------------------------------------------
static int validate_circuit(sp_ctx* ctx, const sp_circuit* c) {
    if (!c || c->num_nodes < 0 || c->num_branches < 0 || c->num_elements < 0 || c->num_params < 0 ||
        c->num_pulses < 0)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad circuit header");
    if (c->num_elements && !c->elements) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null elements");
    if (c->num_params && !c->params) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null params");
    const int nn = c->num_nodes;
    for (int e = 0; e < c->num_elements; ++e) {
        const sp_element& el = c->elements[e];
        if (el.kind < SP_EL_R || el.kind > SP_EL_BSIM3P)
            return fail(ctx, SP_ERR_INVALID_ARGUMENT, "element %d: bad kind %d", e, el.kind);
        const int terms = terminal_count(el.kind);
        for (int t = 0; t < terms; ++t)
            if (el.node[t] < -1 || el.node[t] >= nn)
                return fail(ctx, SP_ERR_INVALID_DIMENSION, "element %d: node %d out of range", e, el.node[t]);
        if (!element_slots_ok(el, c->num_params))
            return fail(ctx, SP_ERR_INVALID_DIMENSION, "element %d: parameter slot out of range", e);
        bool needs_branch = el.kind == SP_EL_V || el.kind == SP_EL_L;
        if (needs_branch && (el.branch < 0 || el.branch >= c->num_branches))
            return fail(ctx, SP_ERR_INVALID_DIMENSION, "element %d: branch %d out of range", e, el.branch);
        if (el.wave >= c->num_pulses)
            return fail(ctx, SP_ERR_INVALID_DIMENSION, "element %d: pulse %d out of range", e, el.wave);
    }
    for (int k = 0; k < c->num_params; ++k)
        if (c->params[k].kind < SP_DRAW_FIXED || c->params[k].kind > SP_DRAW_TABLE)
            return fail(ctx, SP_ERR_INVALID_ARGUMENT, "param %d: bad draw kind", k);
    return SP_OK;
}

int sp_topology_create(sp_ctx* ctx, const sp_circuit* c, sp_topology** out) {
    if (!ctx || !out) return SP_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int rc = validate_circuit(ctx, c);
    if (rc) return rc;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    sp_topology* t = new sp_topology();
    t->ctx = ctx;
    t->num_nodes = c->num_nodes;
    t->num_branches = c->num_branches;
    t->n = c->num_nodes + c->num_branches;
    t->num_elements = c->num_elements;
    t->num_params = c->num_params;
    t->num_pulses = c->num_pulses;
    std::vector<int> doff(c->num_elements);
    int nd = 0;
    for (int e = 0; e < c->num_elements; ++e) {
        doff[e] = nd;
        nd += derived_count(c->elements[e].kind);
    }
    t->num_derived = nd;
    for (int k = 0; k < c->num_params; ++k)
        if (c->params[k].kind == SP_DRAW_TABLE) {
            t->has_table = true;
            t->min_table_cols = std::max(t->min_table_cols, c->params[k].rng_index + 1);
        }
    size_t be = align256(sizeof(sp_element) * c->num_elements);
    size_t bp = align256(sizeof(sp_param) * c->num_params);
    size_t bu = align256(sizeof(sp_pulse) * c->num_pulses);
    size_t bo = align256(sizeof(int) * c->num_elements);
    size_t bn = align256(sizeof(double) * t->n);
    std::vector<int> drawn;
    for (int k = 0; k < c->num_params; ++k)
        if (c->params[k].kind != SP_DRAW_FIXED) drawn.push_back(k);
    size_t bw = align256(sizeof(int) * drawn.size());
    cudaError_t e = cudaMalloc(&t->dev, be + bp + bu + bo + bn + bw + 256);
    if (e != cudaSuccess) {
        delete t;
        return cuda_fail(ctx, e, "topology allocation");
    }
    char* b = (char*)t->dev;
    sp_element* del = (sp_element*)b;
    sp_param* dpar = (sp_param*)(b + be);
    sp_pulse* dpul = (sp_pulse*)(b + be + bp);
    int* ddoff = (int*)(b + be + bp + bu);
    double* dns = (double*)(b + be + bp + bu + bo);
    int* ddrawn = (int*)(b + be + bp + bu + bo + bn);
    if (c->num_elements) e = cudaMemcpy(del, c->elements, sizeof(sp_element) * c->num_elements, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !drawn.empty())
        e = cudaMemcpy(ddrawn, drawn.data(), sizeof(int) * drawn.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && c->num_params)
        e = cudaMemcpy(dpar, c->params, sizeof(sp_param) * c->num_params, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && c->num_pulses)
        e = cudaMemcpy(dpul, c->pulses, sizeof(sp_pulse) * c->num_pulses, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && c->num_elements)
        e = cudaMemcpy(ddoff, doff.data(), sizeof(int) * c->num_elements, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && c->nodeset) e = cudaMemcpy(dns, c->nodeset, sizeof(double) * t->n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(t->dev);
        delete t;
        return cuda_fail(ctx, e, "topology upload");
    }
    t->dc = DevCircuit{c->num_nodes, c->num_branches, t->n, c->num_elements, c->num_params, nd,
                       del, dpar, dpul, ddoff, c->nodeset ? dns : nullptr};
    t->d_drawn = ddrawn;
    t->num_drawn = (int)drawn.size();
    t->h_elements.assign(c->elements, c->elements + c->num_elements);
    t->h_params.assign(c->params, c->params + c->num_params);
    if (c->nodeset) t->h_nodeset.assign(c->nodeset, c->nodeset + t->n);
    *out = t;
    return SP_OK;
}

int sp_topology_specialize(sp_ctx* ctx, sp_topology* t, int precision, int enable, char* log, size_t log_len) {
    if (!ctx || !t) return SP_ERR_INVALID_ARGUMENT;
    if (t->ctx != ctx) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "topology belongs to another context");
    if (precision != SP_PREC_MIXED && precision != SP_PREC_FP64)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "specialisation exists for SP_PREC_MIXED and SP_PREC_FP64");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    const int sidx = precision == SP_PREC_MIXED ? 0 : 1;
    if (!enable) {
        t->spec_enabled[sidx] = false;
        return SP_OK;
    }
    std::string why;
    int rc = spec_prepare(t, precision, why);
    const std::string& msg = rc == SP_OK ? t->spec_log[sidx] : why;
    if (log && log_len) {
        std::strncpy(log, msg.c_str(), log_len - 1);
        log[log_len - 1] = '\0';
    }
    if (rc != SP_OK) return fail(ctx, rc, "specialisation failed: %s", why.c_str());
    t->spec_enabled[sidx] = true;
    return SP_OK;
}

int sp_topology_destroy(sp_topology* t) {
    if (!t) return SP_OK;
    cudaSetDevice(t->ctx->device);
    cudaDeviceSynchronize();
    if (t->dev) cudaFree(t->dev);
    delete t;
    return SP_OK;
}

int sp_topology_size(const sp_topology* t) { return t ? t->n : 0; }

// ---------------------------------------------------------------------------
// Batched DC operating points
// ---------------------------------------------------------------------------
struct NewtonScratch {
    double* params;
    double* derived;
    uint32_t* fail_list;
    unsigned int* counters;  // [0] fail count, [1] undecided roundings, [2..3] work counter,
                             // [4] draw groups, [6..7] draw items
    sp_moments* partial;
    uint32_t moment_blocks;
    double* x0;   // learned warm starts [count][n] (when requested)
    size_t used;  // bytes of the context scratch this layout occupies
};

static int newton_scratch(sp_ctx* ctx, const sp_topology* t, uint64_t count, NewtonScratch& s,
                          bool want_x0 = false) {
    size_t bp = align256(8 * (size_t)t->num_params * count);
    size_t bd = align256(8 * (size_t)t->num_derived * count);
    size_t bl = align256(4 * count);
    size_t bc = 256;
    uint32_t mb = (uint32_t)std::max<uint64_t>(1216, (count + 511) / 512);  // partials per column
    size_t bm = align256(sizeof(sp_moments) * mb * (size_t)t->n);
    size_t bx = want_x0 ? align256(8 * (size_t)t->n * count) : 0;
    int rc = ensure_scratch(ctx, bp + bd + bl + bc + bm + bx);
    if (rc) return rc;
    char* b = (char*)ctx->scratch;
    s.params = (double*)b;
    s.derived = (double*)(b + bp);
    s.fail_list = (uint32_t*)(b + bp + bd);
    s.counters = (unsigned int*)(b + bp + bd + bl);
    s.partial = (sp_moments*)(b + bp + bd + bl + bc);
    s.moment_blocks = mb;
    s.x0 = want_x0 ? (double*)(b + bp + bd + bl + bc + bm) : nullptr;
    s.used = bp + bd + bl + bc + bm + bx;
    return SP_OK;
}

static int newton_dc_locked(sp_ctx* ctx, const sp_topology* t, const sp_newton_config* cfg, uint64_t seed,
                            uint64_t first_index, uint64_t count, const double* d_table, uint32_t table_cols,
                            const double* d_x0, double* d_x, int32_t* d_iters, uint8_t* d_status,
                            double* d_resid, double* d_params, sp_moments* d_moments, cudaStream_t st,
                            sp_mlp* warm = nullptr) {
    if (count == 0) return SP_OK;
    if (!d_x) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null output x");
    if (count > ctx->cfg.max_batch_per_launch)
        return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %llu exceeds maximum %llu",
                    (unsigned long long)count, (unsigned long long)ctx->cfg.max_batch_per_launch);
    if (count > 0xffffffffull)
        return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %llu exceeds maximum %llu", (unsigned long long)count,
                    0xffffffffull);
    if (first_index + count > 0x100000000ull)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "sweep index beyond u32 (rng.rs keys sweeps by u32)");
    if (t->has_table && !d_table) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "circuit needs a parameter table");
    if (t->has_table && table_cols < t->min_table_cols)
        return fail(ctx, SP_ERR_INVALID_DIMENSION, "table has %u columns, circuit reads %u", table_cols,
                    t->min_table_cols);
    if (t->n == 0) return fail(ctx, SP_ERR_INVALID_DIMENSION, "empty circuit");
    if (t->n > kMaxDenseN)
        return fail(ctx, SP_ERR_INVALID_DIMENSION, "MNA size %d exceeds the dense Newton limit %d", t->n,
                    kMaxDenseN);
    const int prec = cfg->precision;
    if (prec != SP_PREC_FP64 && prec != SP_PREC_MIXED && prec != SP_PREC_FP64_EXACT)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad precision %d", prec);
    if (cfg->max_iterations <= 0) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "max_iterations <= 0");
    if (warm) {
        if (mlp_ctx(warm) != ctx) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "network belongs to another context");
        if (!mlp_io_ready(warm)) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "network inputs/outputs not set");
        if (mlp_outputs(warm) != t->n)
            return fail(ctx, SP_ERR_INVALID_DIMENSION, "network has %d outputs, circuit %d unknowns",
                        mlp_outputs(warm), t->n);
        if (mlp_max_slot(warm) >= t->num_params)
            return fail(ctx, SP_ERR_INVALID_DIMENSION, "network input slot %d beyond the circuit's %d parameters",
                        mlp_max_slot(warm), t->num_params);
        if (count > mlp_max_rows())
            return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %llu exceeds maximum %llu",
                        (unsigned long long)count, (unsigned long long)mlp_max_rows());
    }
    NewtonScratch s;
    int rc = newton_scratch(ctx, t, count, s, warm != nullptr);
    if (rc) return rc;
    // counters: [0] miss count, [1] undecided roundings, [2..3] work counter (u64),
    // [4] draw group counter, [6..7] draw item counter (u64)
    SP_CUDA(ctx, cudaMemsetAsync(s.counters, 0, 32, st), "clear counters");
    DrawLaunch D{t->dc, seed, first_index, count, d_table, table_cols, s.params, s.derived, d_params,
                 s.counters + 1, t->d_drawn, t->num_drawn, s.counters + 4};
    // topology-specialised primary kernel when enabled and buildable
    const int sidx = prec == SP_PREC_MIXED ? 0 : (prec == SP_PREC_FP64 ? 1 : -1);
    bool use_spec = false;
    if (sidx >= 0 && t->spec_enabled[sidx] && !std::getenv("SPICIER_GB300_GENERIC")) {
        std::string why;
        use_spec = spec_prepare(const_cast<sp_topology*>(t), prec, why) == SP_OK;
    }
    // the double-float specialised kernel computes its constants from the
    // parameters: the draw kernel skips the derived constants
    const bool pmode = use_spec && spec_params_mode(t, prec);
    D.derive = !pmode;
    // a linear warm start is evaluated by the specialised kernel from each
    // sample's parameters, or by the draw kernel into x0 for the generic kernels
    DrawLaunch lin{};
    const bool linear_warm = warm && mlp_linear_only(warm, &lin);
    if (linear_warm && !use_spec) {
        D.lin = lin.lin;
        D.lin_io = lin.lin_io;
        D.lin_slots = lin.lin_slots;
        D.lin_nin = lin.lin_nin;
        D.lin_nout = lin.lin_nout;
        D.x0_out = s.x0;
    }
    // with nothing reading a sample's parameters together inside the draw
    // kernel, the draws run as per-warp items; the fixed slots then stay
    // unwritten, so the warm start's inputs must all be drawn slots
    if (!D.derive && !D.x0_out && !D.params_out &&
        (!warm || mlp_inputs_drawn(warm, t->h_params.data(), t->num_params)))
        D.next_items = reinterpret_cast<unsigned long long*>(s.counters + 6);
    {
        ProfScope prof(ctx, "draw_params", st);
        SP_CUDA(ctx, launch_draw(D, st), "draw launch");
    }
    if (linear_warm) {
        if (!use_spec) d_x0 = s.x0;
    } else if (warm) {
        ProfScope prof(ctx, "mlp_warm_start", st);
        SP_CUDA(ctx, mlp_warm_start(warm, s.params, (size_t)count, (int)count, s.x0, st), "network warm start");
        d_x0 = s.x0;
    }
    NewtonLaunch L;
    L.c = t->dc;
    L.cfg = *cfg;
    L.dv = SoA{s.derived, (size_t)count};
    L.count = count;
    L.x0 = d_x0;
    L.x = d_x;
    L.iters = d_iters;
    L.status = d_status;
    L.resid = d_resid;
    L.fail_list = s.fail_list;
    L.fail_count = s.counters;
    L.work_next = reinterpret_cast<unsigned long long*>(s.counters + 2);
    L.cold_max_iterations = cfg->max_iterations;
    if (linear_warm && use_spec) {
        mlp_linear_host(warm, &L.lin_host, &L.lin_io_host, &L.lin_slots_host);
        L.lin_params = s.params;
        L.lin_pstride = count;
        L.lin = lin.lin;
        L.lin_io = lin.lin_io;
        L.lin_slots = lin.lin_slots;
        L.lin_nin = lin.lin_nin;
    }
    if (pmode) {
        L.params = s.params;
        L.params_stride = count;
        L.derived_out = s.derived;
    }
    // with one sample per thread the specialised kernel reduces its blocks'
    // moments itself; a final kernel merges them (replacing the rows pass)
    const bool fused_moments = d_moments && d_status && use_spec && spec_one_sample_per_thread(t, prec, count);
    const bool warm_start = d_x0 || L.lin;
    const int kprec = prec == SP_PREC_MIXED ? SP_PREC_MIXED : SP_PREC_FP64;
    size_t per = kprec == SP_PREC_MIXED ? work_bytes_per_thread<SP_PREC_MIXED>(t->n)
                                        : work_bytes_per_thread<SP_PREC_FP64>(t->n);
    int block = pick_block(per, ctx->max_smem);
    if (!block) return fail(ctx, SP_ERR_INVALID_DIMENSION, "MNA size %d does not fit shared memory", t->n);
    {
        // tuned threads per block (setting "newton.block.<precision>"), within what shared memory allows
        static const char* bname[3] = {"newton.block.fp64", "newton.block.mixed", "newton.block.exact"};
        const int tb = tune_get(ctx, bname[prec], t->n, 0);
        if (tb >= 32 && tb % 32 == 0 && tb <= 1024 && per * tb <= (size_t)ctx->max_smem) block = tb;
    }
    size_t smem = per * block;
    int grid = (int)((count + block - 1) / block);
    static const char* kname[3] = {"newton_primary_fp64", "newton_primary_mixed", "newton_primary_fp64_exact"};
    static const char* fname[3] = {"newton_fallback_fp64", "newton_fallback_mixed", "newton_fallback_fp64_exact"};
    static const char* sname[2] = {"newton_primary_mixed_spec", "newton_primary_fp64_spec"};
    // the attempt from a warm start may carry its own iteration cap
    NewtonLaunch Lp = L;
    if (fused_moments) Lp.moments_partial = s.partial;
    if (warm_start && cfg->warm_max_iterations > 0 && cfg->warm_max_iterations < cfg->max_iterations)
        Lp.cfg.max_iterations = cfg->warm_max_iterations;
    cudaError_t e;
    {
        ProfScope prof(ctx, use_spec ? sname[sidx] : kname[prec], st);
        if (use_spec)
            e = spec_launch(t, prec, Lp, st);
        else
            e = prec == SP_PREC_FP64_EXACT ? launch_newton_exact(Lp, false, grid, block, smem, st)
                                           : launch_newton_fast(kprec, Lp, false, grid, block, smem, st);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "newton launch");
    const bool any_fallback = warm_start || (cfg->fallback & (SP_FALLBACK_GMIN | SP_FALLBACK_SOURCE));
    if (any_fallback) {
        // one-warp blocks (a few KB of shared memory each) fit beside the
        // primary kernel's blocks, so under programmatic dependent launch they
        // are resident while it drains; two per SM: the chained op-amp step
        // measured 94.4 us with two, 95.7 with one, ~98-100 with four and
        // 93.9 with no fallback launch at all (an empty miss list is the
        // common case; a long list gets 64 threads per SM)
        const int fblock = 32;
        const int fgrid = std::max(1, std::min(ctx->num_sms * 2, (int)((count + fblock - 1) / fblock)));
        const size_t fsmem = per * fblock;
        ProfScope prof(ctx, fname[prec], st);
        e = prec == SP_PREC_FP64_EXACT ? launch_newton_exact(L, true, fgrid, fblock, fsmem, st)
                                       : launch_newton_fast(kprec, L, true, fgrid, fblock, fsmem, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "fallback launch");
    }
    if (d_moments && fused_moments) {
        ProfScope prof(ctx, "moments", st);
        e = launch_moments_from_partials(s.partial, (uint32_t)((count + 127) / 128), s.counters, d_x, count,
                                         (uint32_t)t->n, d_status, d_moments, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "moments launch");
    } else if (d_moments) {
        ProfScope prof(ctx, "moments", st);
        e = launch_moments(d_x, count, (uint32_t)t->n, (uint32_t)t->n, d_status, s.partial, s.moment_blocks,
                           d_moments, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "moments launch");
    }
    return SP_OK;
}

int sp_newton_dc_device(sp_ctx* ctx, const sp_topology* topo, const sp_newton_config* cfg, uint64_t seed,
                        uint64_t first_index, uint64_t num_samples, const double* d_table, uint32_t table_cols,
                        const double* d_x0, double* d_x, int32_t* d_iters, uint8_t* d_status, double* d_resid,
                        double* d_params, sp_moments* d_moments, void* stream) {
    if (!ctx || !topo || !cfg) return SP_ERR_INVALID_ARGUMENT;
    if (topo->ctx != ctx) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "topology belongs to another context");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return newton_dc_locked(ctx, topo, cfg, seed, first_index, num_samples, d_table, table_cols, d_x0, d_x,
                            d_iters, d_status, d_resid, d_params, d_moments, (cudaStream_t)stream);
}

int sp_newton_dc_learned_device(sp_ctx* ctx, const sp_topology* topo, sp_mlp* mlp, const sp_newton_config* cfg,
                                uint64_t seed, uint64_t first_index, uint64_t num_samples, const double* d_table,
                                uint32_t table_cols, double* d_x, int32_t* d_iters, uint8_t* d_status,
                                double* d_resid, sp_moments* d_moments, void* stream) {
    if (!ctx || !topo || !cfg || !mlp) return SP_ERR_INVALID_ARGUMENT;
    if (topo->ctx != ctx) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "topology belongs to another context");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return newton_dc_locked(ctx, topo, cfg, seed, first_index, num_samples, d_table, table_cols, nullptr, d_x,
                            d_iters, d_status, d_resid, nullptr, d_moments, (cudaStream_t)stream, mlp);
}

// The topology of `c` for a host-buffer call: created on first use and kept
// by the context (at most 16 circuits; the 17th clears the cache).
static int host_topology(sp_ctx* ctx, const sp_circuit* c, sp_topology** out) {
    std::string key;
    auto put = [&](const void* p, size_t n) { key.append((const char*)p, n); };
    put(&c->num_nodes, sizeof(int));
    put(&c->num_branches, sizeof(int));
    put(&c->num_elements, sizeof(int));
    put(&c->num_params, sizeof(int));
    put(&c->num_pulses, sizeof(int));
    if (c->num_elements > 0 && c->elements) put(c->elements, sizeof(sp_element) * c->num_elements);
    if (c->num_params > 0 && c->params) put(c->params, sizeof(sp_param) * c->num_params);
    if (c->num_pulses > 0 && c->pulses) put(c->pulses, sizeof(sp_pulse) * c->num_pulses);
    const char has_ns = c->nodeset ? 1 : 0;
    put(&has_ns, 1);
    if (c->nodeset && c->num_nodes + c->num_branches > 0)
        put(c->nodeset, sizeof(double) * (size_t)(c->num_nodes + c->num_branches));
    std::lock_guard<std::mutex> g(ctx->topo_mu);
    auto it = ctx->host_topos.find(key);
    if (it != ctx->host_topos.end()) {
        *out = it->second;
        return SP_OK;
    }
    if (ctx->host_topos.size() >= 16) {
        for (auto& kv : ctx->host_topos) sp_topology_destroy(kv.second);
        ctx->host_topos.clear();
    }
    sp_topology* t = nullptr;
    int rc = sp_topology_create(ctx, c, &t);
    if (rc) return rc;
    ctx->host_topos[key] = t;
    *out = t;
    return SP_OK;
}

static int newton_dc_host(sp_ctx* ctx, const sp_circuit* circuit, const sp_newton_config* cfg, uint64_t seed,
                          uint64_t first_index, uint64_t count, const double* table, uint32_t table_cols,
                          const double* x0, double* x, int32_t* iters, uint8_t* status, double* resid,
                          double* params, sp_moments* moments, sp_mlp* warm) {
    if (!ctx || !circuit || !cfg) return SP_ERR_INVALID_ARGUMENT;
    if (count == 0) return SP_OK;
    if (!x) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null output x");
    sp_topology* t = nullptr;
    int rc = host_topology(ctx, circuit, &t);
    if (rc) return rc;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    const int n = t->n;
    // The device buffers of this call sit after the Newton scratch; size both.
    NewtonScratch ns;
    rc = newton_scratch(ctx, t, count, ns, warm != nullptr);
    if (rc) return rc;
    size_t inner = ns.used;
    size_t bx = align256(8 * count * n), bi = align256(4 * count), bs = align256(count), br = align256(8 * count);
    size_t bpar = align256(8 * count * (size_t)t->num_params), bm = align256(sizeof(sp_moments) * n);
    size_t btab = table ? align256(8 * count * (size_t)table_cols) : 0;
    size_t bx0 = x0 ? bx : 0;
    rc = ensure_scratch(ctx, inner + bx + bi + bs + br + bpar + bm + btab + bx0);
    if (rc) return rc;
    rc = newton_scratch(ctx, t, count, ns, warm != nullptr);  // pointers may have moved
    if (rc) return rc;
    char* b = (char*)ctx->scratch + inner;
    double* d_x = (double*)b;
    int32_t* d_it = (int32_t*)(b + bx);
    uint8_t* d_st = (uint8_t*)(b + bx + bi);
    double* d_res = (double*)(b + bx + bi + bs);
    double* d_par = (double*)(b + bx + bi + bs + br);
    sp_moments* d_mom = (sp_moments*)(b + bx + bi + bs + br + bpar);
    double* d_tab = table ? (double*)(b + bx + bi + bs + br + bpar + bm) : nullptr;
    double* d_x0 = x0 ? (double*)(b + bx + bi + bs + br + bpar + bm + btab) : nullptr;
    cudaStream_t st = ctx->stream;
    if (table) SP_CUDA(ctx, cudaMemcpyAsync(d_tab, table, 8 * count * table_cols, cudaMemcpyHostToDevice, st), "H2D table");
    if (x0) SP_CUDA(ctx, cudaMemcpyAsync(d_x0, x0, 8 * count * n, cudaMemcpyHostToDevice, st), "H2D x0");
    rc = newton_dc_locked(ctx, t, cfg, seed, first_index, count, d_tab, table_cols, d_x0, d_x, d_it, d_st,
                          resid ? d_res : nullptr, params ? d_par : nullptr, moments ? d_mom : nullptr, st, warm);
    if (rc) return rc;
    SP_CUDA(ctx, cudaMemcpyAsync(x, d_x, 8 * count * n, cudaMemcpyDeviceToHost, st), "D2H x");
    if (iters) SP_CUDA(ctx, cudaMemcpyAsync(iters, d_it, 4 * count, cudaMemcpyDeviceToHost, st), "D2H iters");
    if (status) SP_CUDA(ctx, cudaMemcpyAsync(status, d_st, count, cudaMemcpyDeviceToHost, st), "D2H status");
    if (resid) SP_CUDA(ctx, cudaMemcpyAsync(resid, d_res, 8 * count, cudaMemcpyDeviceToHost, st), "D2H resid");
    if (params)
        SP_CUDA(ctx, cudaMemcpyAsync(params, d_par, 8 * count * t->num_params, cudaMemcpyDeviceToHost, st),
                "D2H params");
    if (moments) SP_CUDA(ctx, cudaMemcpyAsync(moments, d_mom, sizeof(sp_moments) * n, cudaMemcpyDeviceToHost, st),
                         "D2H moments");
    SP_CUDA(ctx, cudaStreamSynchronize(st), "newton_dc");
    return SP_OK;
}

int sp_newton_dc(sp_ctx* ctx, const sp_circuit* circuit, const sp_newton_config* cfg, uint64_t seed,
                 uint64_t first_index, uint64_t count, const double* table, uint32_t table_cols,
                 const double* x0, double* x, int32_t* iters, uint8_t* status, double* resid, double* params,
                 sp_moments* moments) {
    return newton_dc_host(ctx, circuit, cfg, seed, first_index, count, table, table_cols, x0, x, iters, status,
                          resid, params, moments, nullptr);
}

int sp_newton_dc_learned(sp_ctx* ctx, const sp_circuit* circuit, sp_mlp* mlp, const sp_newton_config* cfg,
                         uint64_t seed, uint64_t first_index, uint64_t count, const double* table,
                         uint32_t table_cols, double* x, int32_t* iters, uint8_t* status, double* resid,
                         sp_moments* moments) {
    if (!mlp) return SP_ERR_INVALID_ARGUMENT;
    return newton_dc_host(ctx, circuit, cfg, seed, first_index, count, table, table_cols, nullptr, x, iters,
                          status, resid, nullptr, moments, mlp);
}

int sp_draw_params_device(sp_ctx* ctx, const sp_topology* t, uint64_t seed, uint64_t first_index,
                          uint64_t num_samples, const double* d_table, uint32_t table_cols, double* d_params,
                          void* stream) {
    if (!ctx || !t || !d_params) return SP_ERR_INVALID_ARGUMENT;
    if (t->has_table && !d_table) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "circuit needs a parameter table");
    if (t->has_table && table_cols < t->min_table_cols)
        return fail(ctx, SP_ERR_INVALID_DIMENSION, "table has %u columns, circuit reads %u", table_cols,
                    t->min_table_cols);
    if (num_samples == 0) return SP_OK;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    NewtonScratch s;
    int rc = newton_scratch(ctx, t, num_samples, s);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    ScratchOrder order(ctx, st);
    SP_CUDA(ctx, cudaMemsetAsync(s.counters, 0, 32, st), "clear counters");
    DrawLaunch D{t->dc, seed, first_index, num_samples, d_table, table_cols, s.params, s.derived, d_params,
                 s.counters + 1, t->d_drawn, t->num_drawn, s.counters + 4};
    SP_CUDA(ctx, launch_draw(D, st), "draw launch");
    return SP_OK;
}

int sp_rng_fill_device(sp_ctx* ctx, int kind, uint64_t seed, uint64_t first_index, uint32_t param_index,
                       uint64_t count, double* d_out, void* stream) {
    if (!ctx || !d_out) return SP_ERR_INVALID_ARGUMENT;
    if (kind < 0 || kind > 3) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad rng kind %d", kind);
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ProfScope prof(ctx, "rng_fill", (cudaStream_t)stream);
    SP_CUDA(ctx, launch_rng_fill(kind, seed, first_index, param_index, count, d_out, (cudaStream_t)stream),
            "rng launch");
    return SP_OK;
}

int sp_moments_device(sp_ctx* ctx, const double* d_values, uint64_t rows, uint32_t ld, uint32_t cols,
                      const uint8_t* d_status, sp_moments* d_out, void* stream) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    if (!d_out || (rows && !d_values)) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null buffer");
    if (cols > ld) return fail(ctx, SP_ERR_INVALID_DIMENSION, "cols > ld");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    uint32_t mb = (uint32_t)std::max<uint64_t>(1216, (rows + 511) / 512);  // partials per column
    int rc = ensure_scratch(ctx, align256(sizeof(sp_moments) * mb * (size_t)cols));
    if (rc) return rc;
    ScratchOrder order(ctx, (cudaStream_t)stream);
    SP_CUDA(ctx, launch_moments(d_values, rows, ld, cols, d_status, (sp_moments*)ctx->scratch, mb, d_out,
                                (cudaStream_t)stream),
            "moments launch");
    return SP_OK;
}

int sp_tune_set(sp_ctx* ctx, const char* key, int value) {
    if (!ctx || !key || !*key) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    if (value <= 0)
        ctx->tune.erase(key);
    else
        ctx->tune[key] = value;
    return SP_OK;
}

int sp_tune_get(sp_ctx* ctx, const char* key, int* value) {
    if (!ctx || !key || !value) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    auto it = ctx->tune.find(key);
    *value = it == ctx->tune.end() ? 0 : it->second;
    return it == ctx->tune.end() ? 0 : 1;
}

int sp_tune_bucket(long long n) { return tune_bucket(n); }

int sp_moments_merge_device(sp_ctx* ctx, sp_moments* d_acc, const sp_moments* d_other, uint32_t n, void* stream) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    if (n && (!d_acc || !d_other)) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "null buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    SP_CUDA(ctx, launch_moments_merge(d_acc, d_other, n, (cudaStream_t)stream), "moments merge launch");
    return SP_OK;
}

int sp_moments_merge(sp_moments* acc, const sp_moments* other, uint32_t n) {
    if (n && (!acc || !other)) return SP_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; ++i) {
        acc[i].count += other[i].count;
        acc[i].sum += other[i].sum;
        acc[i].sum_sq += other[i].sum_sq;
        acc[i].min = std::fmin(acc[i].min, other[i].min);  // f64::min: a NaN operand gives the other
        acc[i].max = std::fmax(acc[i].max, other[i].max);
    }
    return SP_OK;
}

int sp_profile_enable(sp_ctx* ctx, int on) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->profiling = on != 0;
    return SP_OK;
}

int sp_profile_read(sp_ctx* ctx, sp_kernel_time* out, int cap, int* count) {
    if (!ctx || !count || (cap > 0 && !out)) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    int k = 0;
    for (auto& r : ctx->recs) {
        cudaError_t e = cudaEventSynchronize(r.b);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "profile synchronise");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        int j = 0;
        while (j < k && std::strncmp(out[j].name, r.name, sizeof out[j].name) != 0) ++j;
        if (j == k) {
            if (k >= cap) continue;
            std::memset(&out[k], 0, sizeof out[k]);
            std::strncpy(out[k].name, r.name, sizeof out[k].name - 1);
            ++k;
        }
        out[j].launches += 1;
        out[j].total_ms += ms;
    }
    for (auto& r : ctx->recs) {
        ctx->event_pool.push_back(r.a);
        ctx->event_pool.push_back(r.b);
    }
    ctx->recs.clear();
    *count = k;
    return SP_OK;
}


// ---------------------------------------------------------------------------
// Batched RC-diode ladder transients (ladder.cuh)
// ---------------------------------------------------------------------------
static int ladder_validate(sp_ctx* ctx, const sp_ladder_config* c, uint64_t count) {
    if (!c) return SP_ERR_INVALID_ARGUMENT;
    if (c->min_sections < 2 || c->max_sections < c->min_sections || c->max_sections > 4000)
        return fail(ctx, SP_ERR_INVALID_DIMENSION, "sections must satisfy 2 <= min <= max <= 4000");
    if (!(c->tstop > 0) || !(c->h_min > 0) || !(c->h_max >= c->h_min) || !(c->h_init > 0))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad time-step settings");
    if (!(c->r_lo > 0) || !(c->r_hi >= c->r_lo) || !(c->c_lo > 0) || !(c->c_hi >= c->c_lo) || !(c->diode_is > 0) ||
        !(c->diode_n > 0))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad element ranges");
    if (c->max_iterations < 1 || c->max_steps < 1 || c->num_probe < 0)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad iteration, step or probe counts");
    if (c->precision < SP_PREC_FP64 || c->precision > SP_PREC_FP64_EXACT)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "unknown precision");
    if (count > 0xffffffffull)
        return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %llu exceeds maximum %llu", (unsigned long long)count,
                    0xffffffffull);
    return SP_OK;
}

struct LadderPlan {
    int stride;
    size_t smem;
    uint64_t blocks;
    size_t bh, bo, bn, bw;
    size_t bytes() const { return bh + bo + bn + bw; }
};

static LadderPlan ladder_plan(const sp_ctx* ctx, const sp_ladder_config* c, uint64_t count) {
    LadderPlan p;
    p.stride = (c->max_sections + 2 + 31) & ~31;
    // four warps x (diag, rhs, c', d', block unknowns): FP64 elements, or FP32 in
    // the mixed mode, whose smaller footprint leaves the SM's L1 to the
    // per-ladder arrays
    p.smem = (size_t)4 * ladder_warp_doubles(p.stride, c->precision) * 8;
    // resident blocks per SM: the kernel's launch bounds allow two (registers), shared memory may allow fewer
    int bpsm = std::max(1, std::min(2, (int)((228 * 1024 - 1024) / (p.smem + 1024))));
    // tuned resident blocks per SM (setting "ladder.bpsm"), never above what fits
    const int tb = tune_get(const_cast<sp_ctx*>(ctx), "ladder.bpsm", c->max_sections, 0);
    if (tb >= 1 && tb < bpsm) bpsm = tb;
    p.blocks = std::min<uint64_t>((count + 3) / 4, (uint64_t)ctx->num_sms * bpsm);
    const int bins = c->max_sections - c->min_sections + 1;
    p.bh = align256(4 * (size_t)bins);
    p.bo = align256(4 * count);
    p.bn = 256;
    p.bw = align256((size_t)p.blocks * 4 * LA_COUNT * p.stride * 8);
    return p;
}

static int ladder_locked(sp_ctx* ctx, const sp_ladder_config* c, uint64_t seed, uint64_t first, uint64_t count,
                         double* d_x, int32_t* d_n, int32_t* d_acc, int32_t* d_rej, int32_t* d_it, uint8_t* d_st,
                         double* d_probe, size_t extra, cudaStream_t st, double* d_steps = nullptr,
                         int max_rec = 0) {
    const LadderPlan p = ladder_plan(ctx, c, count);
    if (p.smem > (size_t)ctx->max_smem) return fail(ctx, SP_ERR_INVALID_DIMENSION, "ladder too long for shared memory");
    const int stride = p.stride;
    const size_t smem = p.smem, bh = p.bh, bo = p.bo, bn = p.bn;
    const uint64_t blocks = p.blocks;
    int rc = ensure_scratch(ctx, extra + p.bytes());
    if (rc) return rc;
    char* b = (char*)ctx->scratch + extra;
    LadderLaunch L{};
    L.cfg = *c;
    L.seed = seed;
    L.first = first;
    L.count = count;
    unsigned int* hist = (unsigned int*)b;
    L.order = (const uint32_t*)(b + bh);
    L.next = (unsigned int*)(b + bh + bo);
    L.ws = (double*)(b + bh + bo + bn);
    L.stride = stride;
    L.slots = (int)(blocks * 4);
    L.x_final = d_x;
    L.n = d_n;
    L.accepted = d_acc;
    L.rejected = d_rej;
    L.iters = d_it;
    L.status = d_st;
    L.probe = d_probe;
    L.steps = max_rec > 0 ? d_steps : nullptr;
    L.max_rec = max_rec;
    SP_CUDA(ctx, launch_ladder_prelude(*c, seed, first, count, hist, (uint32_t*)L.order, L.next, st), "ladder order");
    static const char* names[3] = {"ladder_transient_fp64", "ladder_transient_mixed", "ladder_transient_fp64_exact"};
    ProfScope prof(ctx, names[c->precision], st);
    if (c->precision == SP_PREC_FP64_EXACT)
        SP_CUDA(ctx, launch_ladder_exact(L, (int)blocks, smem, st), "ladder launch");
    else
        SP_CUDA(ctx, launch_ladder_fast(L, c->precision, (int)blocks, smem, st), "ladder launch");
    return SP_OK;
}

int sp_ladder_transient_device(sp_ctx* ctx, const sp_ladder_config* cfg, uint64_t seed, uint64_t first_index,
                               uint64_t count, double* d_x_final, int32_t* d_n, int32_t* d_accepted,
                               int32_t* d_rejected, int32_t* d_iters, uint8_t* d_status, double* d_probe,
                               void* stream) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    int rc = ladder_validate(ctx, cfg, count);
    if (rc) return rc;
    if (count == 0) return SP_OK;
    if (!d_x_final || !d_n || !d_accepted || !d_rejected || !d_iters || !d_status || (cfg->num_probe && !d_probe))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "missing output buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return ladder_locked(ctx, cfg, seed, first_index, count, d_x_final, d_n, d_accepted, d_rejected, d_iters,
                         d_status, cfg->num_probe ? d_probe : nullptr, 0, (cudaStream_t)stream);
}

int sp_ladder_transient_steps_device(sp_ctx* ctx, const sp_ladder_config* cfg, uint64_t seed, uint64_t first_index,
                                     uint64_t count, double* d_x_final, int32_t* d_n, int32_t* d_accepted,
                                     int32_t* d_rejected, int32_t* d_iters, uint8_t* d_status, double* d_probe,
                                     double* d_steps, int32_t max_steps_recorded, void* stream) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    int rc = ladder_validate(ctx, cfg, count);
    if (rc) return rc;
    if (max_steps_recorded < 0 || (max_steps_recorded > 0 && !d_steps))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad step record buffer");
    if (count == 0) return SP_OK;
    if (!d_x_final || !d_n || !d_accepted || !d_rejected || !d_iters || !d_status || (cfg->num_probe && !d_probe))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "missing output buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return ladder_locked(ctx, cfg, seed, first_index, count, d_x_final, d_n, d_accepted, d_rejected, d_iters,
                         d_status, cfg->num_probe ? d_probe : nullptr, 0, (cudaStream_t)stream, d_steps,
                         max_steps_recorded);
}

int sp_ladder_transient(sp_ctx* ctx, const sp_ladder_config* cfg, uint64_t seed, uint64_t first_index,
                        uint64_t count, double* x_final, int32_t* n, int32_t* accepted, int32_t* rejected,
                        int32_t* iters, uint8_t* status, double* probe) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    int rc = ladder_validate(ctx, cfg, count);
    if (rc) return rc;
    if (count == 0) return SP_OK;
    if (!x_final || !n || !accepted || !rejected || !iters || !status || (cfg->num_probe && !probe))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "missing output buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    ScratchOrder order(ctx, st);
    const size_t ld = (size_t)cfg->max_sections + 2, np = (size_t)cfg->num_probe;
    const size_t bx = align256(8 * ld * count), bi = align256(4 * count), bs = align256(count),
                 bp = align256(8 * np * count);
    const size_t extra = bx + 4 * bi + bs + bp;
    rc = ensure_scratch(ctx, extra + ladder_plan(ctx, cfg, count).bytes());  // once: the pointers below stay valid
    if (rc) return rc;
    char* b = (char*)ctx->scratch;
    double* dx = (double*)b;
    int32_t* dn = (int32_t*)(b + bx);
    int32_t* da = (int32_t*)(b + bx + bi);
    int32_t* dr = (int32_t*)(b + bx + 2 * bi);
    int32_t* di = (int32_t*)(b + bx + 3 * bi);
    uint8_t* ds = (uint8_t*)(b + bx + 4 * bi);
    double* dp = np ? (double*)(b + bx + 4 * bi + bs) : nullptr;
    rc = ladder_locked(ctx, cfg, seed, first_index, count, dx, dn, da, dr, di, ds, dp, extra, st);
    if (rc) return rc;
    SP_CUDA(ctx, cudaMemcpyAsync(x_final, b, 8 * ld * count, cudaMemcpyDeviceToHost, st), "D2H x");
    SP_CUDA(ctx, cudaMemcpyAsync(n, b + bx, 4 * count, cudaMemcpyDeviceToHost, st), "D2H n");
    SP_CUDA(ctx, cudaMemcpyAsync(accepted, b + bx + bi, 4 * count, cudaMemcpyDeviceToHost, st), "D2H accepted");
    SP_CUDA(ctx, cudaMemcpyAsync(rejected, b + bx + 2 * bi, 4 * count, cudaMemcpyDeviceToHost, st), "D2H rejected");
    SP_CUDA(ctx, cudaMemcpyAsync(iters, b + bx + 3 * bi, 4 * count, cudaMemcpyDeviceToHost, st), "D2H iterations");
    SP_CUDA(ctx, cudaMemcpyAsync(status, b + bx + 4 * bi, count, cudaMemcpyDeviceToHost, st), "D2H status");
    if (np) SP_CUDA(ctx, cudaMemcpyAsync(probe, b + bx + 4 * bi + bs, 8 * np * count, cudaMemcpyDeviceToHost, st), "D2H probe");
    SP_CUDA(ctx, cudaStreamSynchronize(st), "ladder transient");
    return SP_OK;
}


// ---------------------------------------------------------------------------
// Power-grid corner sweep (powergrid.cuh)
// ---------------------------------------------------------------------------
static int grid_validate(sp_ctx* ctx, const sp_grid_config* c, uint64_t count) {
    if (!c) return SP_ERR_INVALID_ARGUMENT;
    if (c->rows < 2 || c->cols < 2 || (uint64_t)c->rows * c->cols + 1 > (uint64_t)kGridThreads * kGridRowsPerThread)
        return fail(ctx, SP_ERR_INVALID_DIMENSION, "grid must be at least 2 x 2 with at most %d unknowns",
                    kGridThreads * kGridRowsPerThread);
    if (c->restart < 1 || c->restart > kGridMaxRestart)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "restart must be 1..%d", kGridMaxRestart);
    if (c->num_sinks < 0 || c->max_newton < 1 || c->max_krylov < 1)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad sink, Newton or Krylov counts");
    if (c->precision != SP_PREC_FP64 && c->precision != SP_PREC_MIXED)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "precision must be SP_PREC_FP64 or SP_PREC_MIXED");
    if (!(c->r_lo > 0) || !(c->r_hi >= c->r_lo) || !(c->krylov_tol > 0))
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad resistance range or tolerance");
    if (count > 0x7fffffffull)
        return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %llu exceeds maximum %llu", (unsigned long long)count,
                    0x7fffffffull);
    const size_t smem = grid_smem_bytes(*c, c->precision == SP_PREC_MIXED ? 4 : 8);
    if (smem > (size_t)ctx->max_smem) return fail(ctx, SP_ERR_INVALID_DIMENSION, "grid too large for shared memory");
    return SP_OK;
}

static int grid_locked(sp_ctx* ctx, const sp_grid_config* c, uint64_t seed, uint64_t first, uint64_t count, double* d_x,
                       int32_t* d_newton, int32_t* d_krylov, uint8_t* d_status, double* d_resid, size_t extra,
                       cudaStream_t st) {
    const GridWs W = grid_ws(*c, c->precision == SP_PREC_MIXED ? 4 : 8);
    int rc = ensure_scratch(ctx, extra + W.total * count);
    if (rc) return rc;
    GridLaunch L{};
    L.cfg = *c;
    L.seed = seed;
    L.first = first;
    L.count = count;
    L.ws = (char*)ctx->scratch + extra;
    L.ws_stride = W.total;
    L.x = d_x;
    L.newton = d_newton;
    L.krylov = d_krylov;
    L.status = d_status;
    L.resid = d_resid;
    ProfScope prof(ctx, c->precision == SP_PREC_MIXED ? "grid_newton_gmres_mixed" : "grid_newton_gmres_fp64", st);
    SP_CUDA(ctx, launch_grid(L, c->precision, st), "grid launch");
    return SP_OK;
}

int sp_grid_solve_device(sp_ctx* ctx, const sp_grid_config* cfg, uint64_t seed, uint64_t first_index, uint64_t count,
                         double* d_x, int32_t* d_newton, int32_t* d_krylov, uint8_t* d_status, double* d_resid,
                         void* stream) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    int rc = grid_validate(ctx, cfg, count);
    if (rc) return rc;
    if (count == 0) return SP_OK;
    if (!d_x || !d_newton || !d_krylov || !d_status || !d_resid)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "missing output buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return grid_locked(ctx, cfg, seed, first_index, count, d_x, d_newton, d_krylov, d_status, d_resid, 0,
                       (cudaStream_t)stream);
}

int sp_grid_solve(sp_ctx* ctx, const sp_grid_config* cfg, uint64_t seed, uint64_t first_index, uint64_t count,
                  double* x, int32_t* newton, int32_t* krylov, uint8_t* status, double* resid) {
    if (!ctx) return SP_ERR_INVALID_ARGUMENT;
    int rc = grid_validate(ctx, cfg, count);
    if (rc) return rc;
    if (count == 0) return SP_OK;
    if (!x || !newton || !krylov || !status || !resid) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "missing output buffer");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    ScratchOrder order(ctx, st);
    const size_t n = (size_t)cfg->rows * cfg->cols + 1;
    const size_t bx = align256(8 * n * count), bi = align256(4 * count), bs = align256(count), br = align256(8 * count);
    const size_t extra = bx + 2 * bi + bs + br;
    const GridWs W = grid_ws(*cfg, cfg->precision == SP_PREC_MIXED ? 4 : 8);
    rc = ensure_scratch(ctx, extra + W.total * count);  // once: the pointers below stay valid
    if (rc) return rc;
    char* b = (char*)ctx->scratch;
    rc = grid_locked(ctx, cfg, seed, first_index, count, (double*)b, (int32_t*)(b + bx), (int32_t*)(b + bx + bi),
                     (uint8_t*)(b + bx + 2 * bi), (double*)(b + bx + 2 * bi + bs), extra, st);
    if (rc) return rc;
    SP_CUDA(ctx, cudaMemcpyAsync(x, b, 8 * n * count, cudaMemcpyDeviceToHost, st), "D2H x");
    SP_CUDA(ctx, cudaMemcpyAsync(newton, b + bx, 4 * count, cudaMemcpyDeviceToHost, st), "D2H newton");
    SP_CUDA(ctx, cudaMemcpyAsync(krylov, b + bx + bi, 4 * count, cudaMemcpyDeviceToHost, st), "D2H krylov");
    SP_CUDA(ctx, cudaMemcpyAsync(status, b + bx + 2 * bi, count, cudaMemcpyDeviceToHost, st), "D2H status");
    SP_CUDA(ctx, cudaMemcpyAsync(resid, b + bx + 2 * bi + bs, 8 * count, cudaMemcpyDeviceToHost, st), "D2H resid");
    SP_CUDA(ctx, cudaStreamSynchronize(st), "grid solve");
    return SP_OK;
}


// ---------------------------------------------------------------------------
// Histogram and yield (statistics.rs)
// ---------------------------------------------------------------------------
int sp_bsim3_eval_device(sp_ctx* ctx, int pmos, const double* d_card, const double* d_bias, uint64_t count,
                         double* d_out, uint8_t* d_region, void* stream) {
    if (!ctx || (count && (!d_card || !d_bias || !d_out))) return SP_ERR_INVALID_ARGUMENT;
    if (count > ((uint64_t)1 << 40))
        return fail(ctx, SP_ERR_BATCH_TOO_LARGE, "Batch size %llu exceeds maximum %llu", (unsigned long long)count,
                    1ull << 40);
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ProfScope prof(ctx, "bsim3_eval", (cudaStream_t)stream);
    SP_CUDA(ctx, launch_bsim3_eval(pmos, d_card, d_bias, count, d_out, d_region, (cudaStream_t)stream),
            "bsim3 evaluation launch");
    return SP_OK;
}

int sp_histogram_device(sp_ctx* ctx, const double* d_values, uint64_t rows, uint32_t ld, uint32_t col,
                        const uint8_t* d_status, double min, double max, uint32_t num_bins, uint64_t* d_bins,
                        void* stream) {
    if (!ctx || !d_bins || (rows && !d_values)) return SP_ERR_INVALID_ARGUMENT;
    if (num_bins == 0 || num_bins > 12288) return fail(ctx, SP_ERR_INVALID_DIMENSION, "num_bins must be 1..12288");
    if (!(max > min)) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "max must be > min");
    if (col >= ld) return fail(ctx, SP_ERR_INVALID_DIMENSION, "column outside the row");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ProfScope prof(ctx, "histogram", (cudaStream_t)stream);
    SP_CUDA(ctx, launch_histogram(d_values, rows, ld, col, d_status, min, max, num_bins, d_bins, ctx->num_sms,
                                  (cudaStream_t)stream),
            "histogram launch");
    return SP_OK;
}

int sp_yield_device(sp_ctx* ctx, const double* d_values, uint64_t rows, uint32_t ld, const uint8_t* d_status,
                    const sp_yield_spec* specs, uint32_t num_specs, uint64_t* d_pass, void* stream) {
    if (!ctx || !d_pass || (rows && !d_values) || (num_specs && !specs)) return SP_ERR_INVALID_ARGUMENT;
    if (num_specs > 4096) return fail(ctx, SP_ERR_INVALID_DIMENSION, "at most 4096 specifications");
    for (uint32_t k = 0; k < num_specs; ++k)
        if (specs[k].col >= ld) return fail(ctx, SP_ERR_INVALID_DIMENSION, "specification %u: column outside the row", k);
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    ScratchOrder order(ctx, st);
    int rc = ensure_scratch(ctx, sizeof(sp_yield_spec) * ((size_t)num_specs + 1));
    if (rc) return rc;
    sp_yield_spec* d_specs = (sp_yield_spec*)ctx->scratch;
    if (num_specs)
        SP_CUDA(ctx, cudaMemcpyAsync(d_specs, specs, sizeof(sp_yield_spec) * num_specs, cudaMemcpyHostToDevice, st),
                "H2D specifications");
    ProfScope prof(ctx, "yield", st);
    SP_CUDA(ctx, launch_yield(d_values, rows, ld, d_status, d_specs, num_specs, d_pass, ctx->num_sms, st), "yield launch");
    return SP_OK;
}


// ---------------------------------------------------------------------------
// Fixed-step linear transients (transient_fixed.cuh)
// ---------------------------------------------------------------------------
static int transient_locked(sp_ctx* ctx, sp_topology* t, const sp_newton_config* dc_cfg,
                            const sp_transient_config* tc, uint64_t seed, uint64_t first, uint64_t count,
                            const double* d_table, uint32_t cols, double* d_x, double* d_probe, uint8_t* d_status,
                            cudaStream_t st) {
    int nv = 0, ncap = 0, nind = 0;
    for (const sp_element& el : t->h_elements) {
        const int k = el.kind;
        if (k != SP_EL_R && k != SP_EL_C && k != SP_EL_L && k != SP_EL_V && k != SP_EL_I)
            return fail(ctx, SP_ERR_INVALID_ARGUMENT, "fixed-step transients take linear circuits (R, C, L, V, I), as "
                                                      "solve_transient");
        nv += k == SP_EL_V;
        ncap += k == SP_EL_C;
        nind += k == SP_EL_L;
    }
    const int nt = t->num_nodes + nv;
    const long steps = (long)std::ceil(tc->tstop / tc->tstep);
    const size_t words = transient_words(nt, ncap, nind);
    int block = 128;
    while (block > 1 && words * 8 * block > 110 * 1024) block >>= 1;
    if (words * 8 * block > (size_t)ctx->max_smem) return fail(ctx, SP_ERR_INVALID_DIMENSION, "circuit too large");
    const int ndc = t->n, np = t->num_params;
    const size_t bx = align256(8 * (size_t)ndc * count), bp = align256(8 * (size_t)std::max(np, 1) * count);
    int rc = ensure_aux(ctx, bx + bp);
    if (rc) return rc;
    double* x_dc = (double*)ctx->aux;
    double* params = (double*)((char*)ctx->aux + bx);
    sp_newton_config dcc = *dc_cfg;
    dcc.precision = tc->precision;
    rc = newton_dc_locked(ctx, t, &dcc, seed, first, count, d_table, cols, nullptr, x_dc, nullptr, d_status, nullptr,
                          params, nullptr, st);
    if (rc) return rc;
    TransientLaunch L{};
    L.c = t->dc;
    L.params = params;
    L.np = np;
    L.x_dc = x_dc;
    L.count = count;
    L.method = tc->method;
    L.h = tc->tstep;
    L.tstop = tc->tstop;
    L.steps = steps;
    L.nt = nt;
    L.num_caps = ncap;
    L.num_inds = nind;
    L.probe_idx = tc->probe;
    L.x = d_x;
    L.probe = d_probe;
    L.status = d_status;
    ProfScope prof(ctx, tc->precision == SP_PREC_FP64_EXACT ? "transient_fixed_exact" : "transient_fixed_fp64", st);
    const size_t smem = words * 8 * block;
    if (tc->precision == SP_PREC_FP64_EXACT) SP_CUDA(ctx, launch_transient_exact(L, block, smem, st), "transient launch");
    else SP_CUDA(ctx, launch_transient_fast(L, block, smem, st), "transient launch");
    return SP_OK;
}

static int transient_validate(sp_ctx* ctx, const sp_transient_config* tc) {
    if (!tc) return SP_ERR_INVALID_ARGUMENT;
    if (!(tc->tstep > 0) || !(tc->tstop > 0) || tc->tstop / tc->tstep > 1e8)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad tstep/tstop");
    if (tc->method < SP_TRAN_BE || tc->method > SP_TRAN_TRBDF2) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "unknown method");
    if (tc->precision != SP_PREC_FP64 && tc->precision != SP_PREC_FP64_EXACT)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "precision must be SP_PREC_FP64 or SP_PREC_FP64_EXACT");
    return SP_OK;
}

int sp_transient_device(sp_ctx* ctx, const sp_topology* topo, const sp_newton_config* dc_cfg,
                        const sp_transient_config* tc, uint64_t seed, uint64_t first_index, uint64_t count,
                        const double* d_table, uint32_t table_cols, double* d_x, double* d_probe, uint8_t* d_status,
                        void* stream) {
    if (!ctx || !topo || !dc_cfg || !d_x || !d_status) return SP_ERR_INVALID_ARGUMENT;
    if (topo->ctx != ctx) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "topology belongs to another context");
    int rc = transient_validate(ctx, tc);
    if (rc) return rc;
    if (tc->probe >= 0 && !d_probe) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "probe requested without a buffer");
    if (count == 0) return SP_OK;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return transient_locked(ctx, const_cast<sp_topology*>(topo), dc_cfg, tc, seed, first_index, count, d_table,
                            table_cols, d_x, tc->probe >= 0 ? d_probe : nullptr, d_status, (cudaStream_t)stream);
}

int sp_transient(sp_ctx* ctx, const sp_circuit* circuit, const sp_newton_config* dc_cfg,
                 const sp_transient_config* tc, uint64_t seed, uint64_t first_index, uint64_t count,
                 const double* table, uint32_t table_cols, double* x, double* probe, uint8_t* status) {
    if (!ctx || !circuit || !dc_cfg || !x || !status) return SP_ERR_INVALID_ARGUMENT;
    int rc = transient_validate(ctx, tc);
    if (rc) return rc;
    if (tc->probe >= 0 && !probe) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "probe requested without a buffer");
    if (count == 0) return SP_OK;
    sp_topology* t = nullptr;
    rc = host_topology(ctx, circuit, &t);
    if (rc) return rc;
    int nv = 0;
    for (int e = 0; e < circuit->num_elements; ++e) nv += circuit->elements[e].kind == SP_EL_V;
    const size_t nt = (size_t)circuit->num_nodes + nv;
    const long steps = (long)std::ceil(tc->tstop / tc->tstep);
    double *dx = nullptr, *dp = nullptr, *dt = nullptr;
    uint8_t* ds = nullptr;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMalloc(&dx, 8 * nt * count);
    if (e == cudaSuccess) e = cudaMalloc(&ds, count);
    if (e == cudaSuccess && tc->probe >= 0) e = cudaMalloc(&dp, 8 * (size_t)(steps + 1) * count);
    if (e == cudaSuccess && table) e = cudaMalloc(&dt, 8 * (size_t)table_cols * count);
    if (e == cudaSuccess && table) e = cudaMemcpy(dt, table, 8 * (size_t)table_cols * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> g(ctx->mu);
        ScratchOrder order(ctx, ctx->stream);
        rc = transient_locked(ctx, t, dc_cfg, tc, seed, first_index, count, dt, table_cols, dx, dp, ds, ctx->stream);
        if (rc == SP_OK) {
            e = cudaMemcpyAsync(x, dx, 8 * nt * count, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(status, ds, count, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess && dp)
                e = cudaMemcpyAsync(probe, dp, 8 * (size_t)(steps + 1) * count, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        }
    }
    for (void* p : {(void*)dx, (void*)dp, (void*)dt, (void*)ds})
        if (p) cudaFree(p);
    if (rc) return rc;
    return e == cudaSuccess ? SP_OK : cuda_fail(ctx, e, "transient copies");
}


// ---------------------------------------------------------------------------
// AC small-signal sweeps (ac.cuh)
// ---------------------------------------------------------------------------
static std::vector<double> ac_grid(const sp_ac_config* c) {
    std::vector<double> f;
    if (c->sweep == SP_AC_LIN) {
        if (c->num_points <= 1) return {c->fstart};
        const double step = (c->fstop - c->fstart) / ((double)c->num_points - 1.0);
        for (int i = 0; i < c->num_points; ++i) f.push_back(c->fstart + step * (double)i);
        return f;
    }
    const double base = c->sweep == SP_AC_DEC ? 10.0 : 2.0;
    const double span = c->sweep == SP_AC_DEC ? std::log10(c->fstop / c->fstart) : std::log2(c->fstop / c->fstart);
    const long total = (long)std::ceil((double)c->num_points * span) + 1;
    for (long i = 0; i < total && i < (1L << 20); ++i) {
        const double v = c->fstart * std::pow(base, (double)i / (double)c->num_points);
        if (v <= c->fstop * 1.001) f.push_back(v);
    }
    return f;
}

static int ac_validate(sp_ctx* ctx, const sp_ac_config* c, int n, int num_elements) {
    if (!c) return SP_ERR_INVALID_ARGUMENT;
    if (c->sweep < SP_AC_LIN || c->sweep > SP_AC_OCT) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "unknown sweep type");
    if (!(c->fstart > 0) || !(c->fstop >= c->fstart) || c->num_points < 1)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "need 0 < fstart <= fstop and num_points >= 1");
    if (c->num_probe < 1 || c->num_probe > 8) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "num_probe must be 1..8");
    for (int k = 0; k < c->num_probe; ++k)
        if (c->probe[k] < 0 || c->probe[k] >= n) return fail(ctx, SP_ERR_INVALID_DIMENSION, "probe %d out of range", k);
    if (c->source < -1 || c->source >= num_elements) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "bad AC source");
    if (c->precision != SP_PREC_FP64 && c->precision != SP_PREC_MIXED)
        return fail(ctx, SP_ERR_INVALID_ARGUMENT, "AC precision must be SP_PREC_FP64 or SP_PREC_MIXED");
    if (c->refine < 0 || c->refine > 8) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "refine must be 0..8");
    return SP_OK;
}

int sp_ac_frequencies(const sp_ac_config* cfg, double* freqs, int cap) {
    if (!cfg) return SP_ERR_INVALID_ARGUMENT;
    const std::vector<double> f = ac_grid(cfg);
    for (int i = 0; i < (int)f.size() && i < cap && freqs; ++i) freqs[i] = f[i];
    return (int)f.size();
}

static int ac_locked(sp_ctx* ctx, sp_topology* t, const sp_newton_config* dc_cfg, const sp_ac_config* ac, uint64_t seed,
                     uint64_t first, uint64_t count, const double* d_table, uint32_t cols, double* d_probe,
                     uint8_t* d_status, cudaStream_t st) {
    const std::vector<double> freqs = ac_grid(ac);
    const int nf = (int)freqs.size();
    if (nf < 1) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "empty frequency grid");
    const int n = t->n, np = std::max(t->num_params, 1);
    const bool mixed = ac->precision == SP_PREC_MIXED;
    const size_t per = ac_work_bytes(n, mixed);  // per-thread work area
    int block = 128;
    while (block > 32 && per * block > 110 * 1024) block >>= 1;
    const bool shared = per * block <= 110 * 1024;
    const uint64_t units = count * (uint64_t)nf;
    int grid = (int)std::min<uint64_t>((units + block - 1) / block,
                                       (uint64_t)ctx->num_sms * (shared ? std::max<size_t>(1, (220 * 1024) / (per * block)) : 2));
    grid = std::max(grid, 1);
    const size_t bx = align256(8 * (size_t)n * count), bp = align256(8 * (size_t)np * count),
                 bf = align256(8 * (size_t)nf), bs = align256(4 * count),
                 bw = shared ? 0 : align256(per * (size_t)grid * block);
    int rc = ensure_aux(ctx, bx + bp + bf + bs + bw);
    if (rc) return rc;
    char* base = (char*)ctx->aux;
    double* x_dc = (double*)base;
    double* params = (double*)(base + bx);
    double* d_freqs = (double*)(base + bx + bp);
    unsigned int* singular = (unsigned int*)(base + bx + bp + bf);
    double* work = shared ? nullptr : (double*)(base + bx + bp + bf + bs);
    SP_CUDA(ctx, cudaMemcpyAsync(d_freqs, freqs.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice, st), "H2D freqs");
    SP_CUDA(ctx, cudaMemsetAsync(singular, 0, 4 * count, st), "clear flags");
    rc = newton_dc_locked(ctx, t, dc_cfg, seed, first, count, d_table, cols, nullptr, x_dc, nullptr, d_status,
                          nullptr, params, nullptr, st);
    if (rc) return rc;
    AcLaunch L{};
    L.c = t->dc;
    L.params = params;
    L.np = t->num_params;
    L.x_dc = x_dc;
    L.dc_status = d_status;
    L.count = count;
    L.freqs = d_freqs;
    L.nf = nf;
    L.source = ac->source;
    L.num_probe = ac->num_probe;
    for (int k = 0; k < 8; ++k) L.probe[k] = k < ac->num_probe ? ac->probe[k] : 0;
    L.out = d_probe;
    L.singular = singular;
    L.work = work;
    L.refine = ac->refine > 0 ? ac->refine : 3;
    {
        NewtonScratch ns;  // the DC pass's layout: its derived constants are still in place
        rc = newton_scratch(ctx, t, count, ns);
        if (rc) return rc;
        L.dv = SoA{ns.derived, (size_t)count};
    }
    ProfScope prof(ctx, mixed ? "ac_sweep_mixed" : "ac_sweep_fp64", st);
    if (mixed) SP_CUDA(ctx, launch_ac_mixed(L, grid, block, shared ? per * block : 0, st), "AC launch");
    else SP_CUDA(ctx, launch_ac(L, grid, block, shared ? per * block : 0, st), "AC launch");
    return SP_OK;
}

int sp_ac_sweep_device(sp_ctx* ctx, const sp_topology* topo, const sp_newton_config* dc_cfg, const sp_ac_config* ac,
                       uint64_t seed, uint64_t first_index, uint64_t count, const double* d_table,
                       uint32_t table_cols, double* d_probe, uint8_t* d_status, void* stream) {
    if (!ctx || !topo || !dc_cfg || !d_probe || !d_status) return SP_ERR_INVALID_ARGUMENT;
    if (topo->ctx != ctx) return fail(ctx, SP_ERR_INVALID_ARGUMENT, "topology belongs to another context");
    int rc = ac_validate(ctx, ac, topo->n, topo->num_elements);
    if (rc) return rc;
    if (count == 0) return SP_OK;
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    ScratchOrder order(ctx, (cudaStream_t)stream);
    return ac_locked(ctx, const_cast<sp_topology*>(topo), dc_cfg, ac, seed, first_index, count, d_table, table_cols,
                     d_probe, d_status, (cudaStream_t)stream);
}

int sp_ac_sweep(sp_ctx* ctx, const sp_circuit* circuit, const sp_newton_config* dc_cfg, const sp_ac_config* ac,
                uint64_t seed, uint64_t first_index, uint64_t count, const double* table, uint32_t table_cols,
                double* probe, uint8_t* status) {
    if (!ctx || !circuit || !dc_cfg || !probe || !status) return SP_ERR_INVALID_ARGUMENT;
    int rc = ac_validate(ctx, ac, circuit->num_nodes + circuit->num_branches, circuit->num_elements);
    if (rc) return rc;
    if (count == 0) return SP_OK;
    sp_topology* t = nullptr;
    rc = host_topology(ctx, circuit, &t);
    if (rc) return rc;
    const size_t nf = ac_grid(ac).size();
    const size_t pbytes = 16 * nf * (size_t)ac->num_probe * count;
    double *dp = nullptr, *dt = nullptr;
    uint8_t* ds = nullptr;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMalloc(&dp, pbytes);
    if (e == cudaSuccess) e = cudaMalloc(&ds, count);
    if (e == cudaSuccess && table) e = cudaMalloc(&dt, 8 * (size_t)table_cols * count);
    if (e == cudaSuccess && table) e = cudaMemcpy(dt, table, 8 * (size_t)table_cols * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> g(ctx->mu);
        ScratchOrder order(ctx, ctx->stream);
        rc = ac_locked(ctx, t, dc_cfg, ac, seed, first_index, count, dt, table_cols, dp, ds, ctx->stream);
        if (rc == SP_OK) {
            e = cudaMemcpyAsync(probe, dp, pbytes, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(status, ds, count, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        }
    }
    for (void* p : {(void*)dp, (void*)dt, (void*)ds})
        if (p) cudaFree(p);
    if (rc) return rc;
    return e == cudaSuccess ? SP_OK : cuda_fail(ctx, e, "AC copies");
}

}  // extern "C"
