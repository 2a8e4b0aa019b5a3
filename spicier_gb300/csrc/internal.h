// Internal launchers shared by the translation units of libspicier_gb300.
//
// Kernels whose results must reproduce the reference's IEEE operation
// sequence live in kernels_exact.cu, compiled with --fmad=false; kernels
// free to contract a*b+c into FMA live in kernels_fast.cu.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/spicier_gb300.h"
#include "newton_dense.cuh"
#include "pdl.cuh"

namespace sp {

struct DrawLaunch {
    DevCircuit c;
    uint64_t seed;
    uint64_t first_index;
    uint64_t count;
    const double* table;  // [count][table_cols] or nullptr
    uint32_t table_cols;
    double* params_soa;   // [num_params][count]
    double* derived_soa;  // [num_derived][count]
    double* params_out;   // [count][num_params] or nullptr
    unsigned int* hard;   // count of draws whose rounding was undecided (or nullptr)
    const int* drawn;     // [num_drawn] slots whose kind is not SP_DRAW_FIXED (device), ascending
    int num_drawn;
    unsigned int* next;   // zeroed group counter of the persistent draw kernel, or nullptr
    // optional linear warm start (SP_MLP_KERNEL_LINEAR): x0_out[s][lin_nout] =
    // lin_io[2 nin + k] + sum_j lin[k][j] (p[lin_slots[j]] - lin_io[j])
    const float* lin = nullptr;
    const float* lin_io = nullptr;  // in_mean[nin], in_scale[nin], out_mean[nout], out_scale[nout]
    const int* lin_slots = nullptr;
    int lin_nin = 0, lin_nout = 0;
    double* x0_out = nullptr;
    // false: skip the derived constants (the consumer, the double-float
    // specialised kernel, computes its constants from the parameters)
    bool derive = true;
    // zeroed item counter: with no per-group consumer (derive false, no
    // x0_out, no params_out) the draws run as (group, drawn slot) items taken
    // by warps, and the fixed slots are not written to params_soa (every
    // consumer of that mode reads fixed values from the circuit)
    unsigned long long* next_items = nullptr;
};

cudaError_t launch_bsim3_eval(int pmos, const double* card, const double* bias, uint64_t count, double* out,
                              uint8_t* region, cudaStream_t st);
cudaError_t launch_histogram(const double* v, uint64_t rows, uint32_t ld, uint32_t col, const uint8_t* status,
                             double mn, double mx, uint32_t nb, uint64_t* bins, int num_sms, cudaStream_t st);
cudaError_t launch_yield(const double* v, uint64_t rows, uint32_t ld, const uint8_t* status,
                         const sp_yield_spec* d_specs, uint32_t ns, uint64_t* pass, int num_sms, cudaStream_t st);
struct TransientLaunch;
cudaError_t launch_transient_exact(const TransientLaunch& L, int block, size_t smem, cudaStream_t st);
cudaError_t launch_transient_fast(const TransientLaunch& L, int block, size_t smem, cudaStream_t st);
struct LadderLaunch;
struct GridLaunch;
cudaError_t launch_grid(const GridLaunch& L, int precision, cudaStream_t st);
// Ladder transient launchers (ladder.cuh): 128-thread blocks, one warp per instance.
cudaError_t launch_ladder_exact(const LadderLaunch& L, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_ladder_fast(const LadderLaunch& L, int precision, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_ladder_prelude(const sp_ladder_config& c, uint64_t seed, uint64_t first, uint64_t count,
                                  unsigned int* hist, uint32_t* order, unsigned int* next, cudaStream_t st);

// kernels_exact.cu (no FMA contraction)
cudaError_t launch_draw(const DrawLaunch& L, cudaStream_t st);
cudaError_t launch_newton_exact(const NewtonLaunch& L, bool fallback, int grid, int block, size_t smem,
                                cudaStream_t st);
cudaError_t launch_rng_fill(int kind, uint64_t seed, uint64_t first, uint32_t param, uint64_t count,
                            double* out, cudaStream_t st);
cudaError_t launch_lu_batch_exact(const double* mats, const double* rhs, int n, uint64_t batch,
                                  double* sol, uint8_t* sing, cudaStream_t st);
cudaError_t prepare_exact_kernels(int max_smem);
// Opt kernel f in to the device's whole shared memory per block less its own
// static shared memory (cudaFuncSetAttribute rejects a larger dynamic size).
inline cudaError_t allow_dynamic_smem(const void* f, int max_smem) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, f);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - (int)a.sharedSizeBytes);
}
struct AcLaunch;
cudaError_t launch_ac(const AcLaunch& L, int grid, int block, size_t smem, cudaStream_t st);
cudaError_t launch_ac_mixed(const AcLaunch& L, int grid, int block, size_t smem, cudaStream_t st);
// solve_batch for n > kMaxDenseN: one CTA per system (shared memory when
// lu_batch_cta_smem(n) fits, else work = grid slices of n*n + n doubles)
constexpr int kMaxBatchLuN = 4096;
size_t lu_batch_cta_smem(int n);
cudaError_t launch_lu_batch_cta(const double* mats, const double* rhs, int n, uint64_t batch, double* sol,
                                uint8_t* sing, double* work, int grid, cudaStream_t st);

// kernels_fast.cu (FMA allowed)
cudaError_t launch_newton_fast(int prec, const NewtonLaunch& L, bool fallback, int grid, int block,
                               size_t smem, cudaStream_t st);
cudaError_t launch_lu_batch_mixed(const double* mats, const double* rhs, int n, uint64_t batch,
                                  double* sol, uint8_t* sing, int refine_steps, cudaStream_t st);
cudaError_t launch_moments(const double* values, uint64_t rows, uint32_t ld, uint32_t cols,
                           const uint8_t* status, sp_moments* partial, uint32_t nblocks, sp_moments* out,
                           cudaStream_t st);
cudaError_t launch_moments_merge(sp_moments* acc, const sp_moments* other, uint32_t n, cudaStream_t st);
// Moments from the specialised kernel's per-block partials ([cols][nblocks]),
// merged in a fixed order; when the fallback changed samples (*fail_count > 0)
// the moments are computed from the values instead (same order for any run).
cudaError_t launch_moments_from_partials(const sp_moments* partial, uint32_t nblocks, const unsigned int* fail_count,
                                         const double* values, uint64_t rows, uint32_t cols, const uint8_t* status,
                                         sp_moments* out, cudaStream_t st);
cudaError_t prepare_fast_kernels(int max_smem);

// Largest dense size of the thread-per-sample Newton kernels.
constexpr int kMaxDenseN = 28;

// mlp.cu: warm start x0[rows][n_out] from parameters in SoA layout.
cudaError_t mlp_warm_start(sp_mlp* m, const double* params_soa, size_t stride, int rows, double* x0,
                           cudaStream_t st);
int mlp_outputs(const sp_mlp* m);
// True when the warm start is the linear term alone (SP_MLP_KERNEL_LINEAR);
// then fills the draw launch's linear-warm-start fields (x0_out left to the caller).
bool mlp_linear_only(const sp_mlp* m, DrawLaunch* d);
int mlp_max_slot(const sp_mlp* m);
// Host copies of the linear term [n_out][n_in] (FP32), io and the input slots;
// false when they are not all set.
bool mlp_linear_host(const sp_mlp* m, const float** lin, const float** io, const int** slots);
// True when every input slot of the warm start is a drawn (not fixed) parameter.
bool mlp_inputs_drawn(const sp_mlp* m, const sp_param* params, int num_params);
uint64_t mlp_max_rows();
bool mlp_io_ready(const sp_mlp* m);
sp_ctx* mlp_ctx(const sp_mlp* m);

}  // namespace sp

// The context: one per device per caller; a mutex serialises host calls.
struct sp_ctx {
    int device = 0;
    sp_batch_config cfg{16, 1, 1ull << 26};
    std::string last_error;
    std::mutex mu;
    cudaStream_t stream = nullptr;  // used by the host-buffer entry points
    cudaEvent_t scratch_done = nullptr;  // last enqueued user of the scratch
    int max_smem = 0;
    int num_sms = 0;
    // grow-only device scratch of the host-buffer entry points and of the
    // Newton launches (parameters, derived constants, fallback list)
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    // stream of the call that holds the scratch (set by the call's ordering
    // guard): growth frees and allocates in that stream's order, after every
    // earlier user, instead of synchronising the device
    cudaStream_t order_stream = nullptr;
    bool order_active = false;
    bool order_capturing = false;
    // kernel timing records (sp_profile_enable)
    bool profiling = false;
    struct Rec {
        const char* name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> event_pool;
    // topology-specialised kernels, keyed by circuit structure + nominal values
    struct Spec {
        cudaLibrary_t lib = nullptr;
        cudaKernel_t kernel = nullptr;
        std::string log;
        int nnz = 0;
        int blocks_per_sm = 1;  // resident 128-thread blocks (the persistent grid)
    };
    std::map<std::string, Spec> spec_cache;
    // topologies of the host-buffer entry points, keyed by the circuit's bytes,
    // so repeated calls on one circuit upload and specialise it once
    std::mutex topo_mu;
    std::map<std::string, sp_topology*> host_topos;
    // second grow-only buffer for entry points that run the Newton path (which
    // owns `scratch`) and keep their own data across it
    void* aux = nullptr;
    size_t aux_bytes = 0;
    // launch settings chosen by the autotuner (sp_tune_set), keyed
    // "<setting>@<size bucket>"; absent keys keep the built-in heuristics
    std::mutex tune_mu;
    std::map<std::string, int> tune;
};

// Size bucket of a tuning key: the smallest power of two >= n (at least 4).
inline int tune_bucket(long long n) {
    int b = 4;
    while (b < n && b < (1 << 30)) b <<= 1;
    return b;
}
// The tuned value of setting `name` at size n, or dflt when none was set.
int tune_get(sp_ctx* ctx, const char* name, long long n, int dflt);

// Grow a context-owned device buffer (*buf, *have bytes) to at least `bytes`;
// see api.cu.  Returns an SP_* status.
int grow_buffer(sp_ctx* ctx, void** buf, size_t* have, size_t bytes, const char* what);

// Calls on different streams share the context's buffers (scratch, second
// buffer, network workspaces): each call orders itself after the previous user
// (skipped while the stream is being captured into a CUDA graph, where the
// caller orders the work), and buffer growth inside the guard is ordered on
// the call's stream.
struct ScratchOrder {
    sp_ctx* ctx;
    cudaStream_t st;
    bool capturing = false;
    cudaStream_t prev_stream;
    bool prev_active, prev_capturing;
    ScratchOrder(sp_ctx* c, cudaStream_t s)
        : ctx(c), st(s), prev_stream(c->order_stream), prev_active(c->order_active),
          prev_capturing(c->order_capturing) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cs);
        capturing = cs != cudaStreamCaptureStatusNone;
        if (!capturing) cudaStreamWaitEvent(st, ctx->scratch_done, 0);
        ctx->order_stream = st;
        ctx->order_active = true;
        ctx->order_capturing = capturing;
    }
    ~ScratchOrder() {
        if (!capturing) cudaEventRecord(ctx->scratch_done, st);
        ctx->order_stream = prev_stream;
        ctx->order_active = prev_active;
        ctx->order_capturing = prev_capturing;
    }
};

// Brackets one kernel launch with events when the context is profiling.
struct ProfScope {
    sp_ctx* ctx;
    cudaStream_t st;
    sp_ctx::Rec rec{};
    ProfScope(sp_ctx* c, const char* name, cudaStream_t s) : ctx(c), st(s) {
        if (!ctx->profiling) return;
        rec.name = name;
        rec.a = take();
        rec.b = take();
        cudaEventRecord(rec.a, st);
    }
    ~ProfScope() {
        if (!ctx->profiling || !rec.a) return;
        cudaEventRecord(rec.b, st);
        ctx->recs.push_back(rec);
    }
    cudaEvent_t take() {
        if (!ctx->event_pool.empty()) {
            cudaEvent_t e = ctx->event_pool.back();
            ctx->event_pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
};

struct sp_topology {
    sp_ctx* ctx = nullptr;
    int n = 0;
    int num_nodes = 0, num_branches = 0, num_elements = 0, num_params = 0, num_derived = 0;
    int num_pulses = 0;
    bool has_table = false;
    uint32_t min_table_cols = 0;  // 1 + largest table column any parameter reads
    void* dev = nullptr;  // one allocation: elements, params, pulses, doff, nodeset, drawn slots
    sp::DevCircuit dc{};
    int* d_drawn = nullptr;  // slots whose kind is not SP_DRAW_FIXED, ascending (inside `dev`)
    int num_drawn = 0;
    // host copy of the description (for the specialiser)
    std::vector<sp_element> h_elements;
    std::vector<sp_param> h_params;
    std::vector<double> h_nodeset;
    // topology-specialised kernels: [0] SP_PREC_MIXED, [1] SP_PREC_FP64
    bool spec_tried[2] = {false, false};
    bool spec_enabled[2] = {true, false};
    cudaKernel_t spec_kernel[2] = {nullptr, nullptr};  // owned by the context's cache
    std::string spec_log[2];
    int spec_nnz[2] = {0, 0};
    int spec_bpsm[2] = {1, 1};
};

namespace sp {
int spec_prepare(sp_topology* t, int prec, std::string& err);
// True when the specialised kernel of t at `prec` reads each sample's
// parameters (and computes its constants) rather than the derived constants.
bool spec_params_mode(const sp_topology* t, int prec);
// True when the specialised kernel's grid gives every sample its own thread
// (then it can reduce its blocks' moments itself).
bool spec_one_sample_per_thread(const sp_topology* t, int prec, uint64_t count);
cudaError_t spec_launch(const sp_topology* t, int prec, const NewtonLaunch& L, cudaStream_t st);
void spec_release_all(sp_ctx* ctx);
}  // namespace sp
