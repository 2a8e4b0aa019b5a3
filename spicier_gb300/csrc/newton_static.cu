// sp_newton_dc_static: the batched DC operating-point sweep without any
// device allocation.
//
// Some callers cannot let a library call cudaMalloc: a host application whose
// device memory is owned by its own pool, reserved at start-up and handed out
// by its allocator; a process running under a hard device-memory cap; a
// latency-bound loop where cudaMalloc/cudaFree's implicit device
// synchronisation is not allowed.  This entry point keeps every intermediate
// of the sweep (the circuit description, the drawn parameters, the derived
// device constants, the miss list of the fallback chain and its counter) in
// one file-scope __device__ array of fixed size, kStaticScratchBytes.  Every
// GPU that loads this library holds that array until the process exits.
//
// Rules of use:
//  * The first call on a device performs the one-time set-up for that
//    device (it looks up the array's device address with
//    cudaGetSymbolAddress and sets the kernels' shared-memory limits), so
//    make the first call before any stream capture.
//  * All calls on a device share the one array, which keeps the contents of
//    the last call.  Calls whose work overlaps on the GPU (different streams,
//    or different host threads without ordering) race on it; order them.
//  * Every call copies the circuit from pageable host memory, so a call
//    whose stream is capturing returns SP_ERR_INVALID_ARGUMENT and enqueues
//    nothing.
//  * The set-up is kept per device ordinal for the life of the process;
//    cudaDeviceReset after the first call is not supported (the cached
//    symbol address and kernel attributes belong to the destroyed context).
//  * The caller passes inputs and outputs (device pointers) as for
//    sp_newton_dc_device; sweeps that need more scratch than the array holds
//    are rejected with SP_ERR_BATCH_TOO_LARGE and a message giving the limit.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "internal.h"

using namespace sp;

namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

struct DeviceSetup {
    bool done = false;
    unsigned char* scratch = nullptr;  // device address of g_static_scratch
    int max_smem = 0;
    int num_sms = 0;
};

std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

int report(char* err, size_t err_len, int code, const char* fmt, ...) {
    if (err && err_len) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, err_len, fmt, ap);
        va_end(ap);
    }
    return code;
}

// One-time set-up of the current device.  In host code g_static_scratch names
// a host-side stand-in, not device memory; the kernels get the address that
// cudaGetSymbolAddress returns for the current device.
int setup_current_device(DeviceSetup** out, char* err, size_t err_len) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return report(err, err_len, SP_ERR_NO_BACKEND, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return report(err, err_len, SP_ERR_BACKEND_INIT, "device ordinal %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> g(g_setup_mu);
    DeviceSetup& s = g_setup[dev];
    if (!s.done) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return report(err, err_len, SP_ERR_BACKEND_INIT, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s.max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = prepare_exact_kernels(s.max_smem);
        if (e == cudaSuccess) e = prepare_fast_kernels(s.max_smem);
        if (e != cudaSuccess)
            return report(err, err_len, SP_ERR_BACKEND_INIT, "device set-up: %s", cudaGetErrorString(e));
        s.scratch = static_cast<unsigned char*>(p);
        s.done = true;
    }
    *out = &s;
    return SP_OK;
}

bool check_circuit(const sp_circuit* c, char* err, size_t err_len, int* code) {
    *code = SP_OK;
    if (!c || c->num_nodes < 0 || c->num_branches < 0 || c->num_elements < 0 || c->num_params < 0 ||
        c->num_pulses < 0 || (c->num_elements && !c->elements) || (c->num_params && !c->params) ||
        (c->num_pulses && !c->pulses)) {
        *code = report(err, err_len, SP_ERR_INVALID_ARGUMENT, "bad circuit description");
        return false;
    }
    for (int e = 0; e < c->num_elements; ++e) {
        const sp_element& el = c->elements[e];
        if (el.kind < SP_EL_R || el.kind > SP_EL_BSIM3P) {
            *code = report(err, err_len, SP_ERR_INVALID_ARGUMENT, "element %d: bad kind %d", e, el.kind);
            return false;
        }
        const int terms = terminal_count(el.kind);
        for (int t = 0; t < terms; ++t)
            if (el.node[t] < -1 || el.node[t] >= c->num_nodes) {
                *code = report(err, err_len, SP_ERR_INVALID_DIMENSION, "element %d: node out of range", e);
                return false;
            }
        if (!element_slots_ok(el, c->num_params)) {
            *code = report(err, err_len, SP_ERR_INVALID_DIMENSION, "element %d: field slot out of range", e);
            return false;
        }
        if ((el.kind == SP_EL_V || el.kind == SP_EL_L) && (el.branch < 0 || el.branch >= c->num_branches)) {
            *code = report(err, err_len, SP_ERR_INVALID_DIMENSION, "element %d: branch out of range", e);
            return false;
        }
        if (el.wave >= c->num_pulses) {
            *code = report(err, err_len, SP_ERR_INVALID_DIMENSION, "element %d: pulse out of range", e);
            return false;
        }
    }
    for (int k = 0; k < c->num_params; ++k)
        if (c->params[k].kind < SP_DRAW_FIXED || c->params[k].kind > SP_DRAW_TABLE) {
            *code = report(err, err_len, SP_ERR_INVALID_ARGUMENT, "param %d: bad draw kind", k);
            return false;
        }
    return true;
}

}  // namespace

extern "C" int sp_newton_dc_static(const sp_circuit* circuit, const sp_newton_config* cfg, uint64_t seed,
                                   uint64_t first_index, uint64_t num_samples, const double* d_table,
                                   uint32_t table_cols, const double* d_x0, double* d_x, int32_t* d_iters,
                                   uint8_t* d_status, double* d_resid, void* stream, char* err,
                                   size_t err_len) {
    if (err && err_len) err[0] = '\0';
    if (!cfg) return report(err, err_len, SP_ERR_INVALID_ARGUMENT, "null config");
    int code;
    if (!check_circuit(circuit, err, err_len, &code)) return code;
    if (num_samples == 0) return SP_OK;
    if (!d_x) return report(err, err_len, SP_ERR_INVALID_ARGUMENT, "null output x");
    const int n = circuit->num_nodes + circuit->num_branches;
    if (n == 0) return report(err, err_len, SP_ERR_INVALID_DIMENSION, "empty circuit");
    if (n > kMaxDenseN)
        return report(err, err_len, SP_ERR_INVALID_DIMENSION, "MNA size %d exceeds the dense Newton limit %d", n,
                      kMaxDenseN);
    const int prec = cfg->precision;
    if (prec != SP_PREC_FP64 && prec != SP_PREC_MIXED && prec != SP_PREC_FP64_EXACT)
        return report(err, err_len, SP_ERR_INVALID_ARGUMENT, "bad precision %d", prec);
    if (cfg->max_iterations <= 0) return report(err, err_len, SP_ERR_INVALID_ARGUMENT, "max_iterations <= 0");
    if (first_index + num_samples > 0x100000000ull)
        return report(err, err_len, SP_ERR_INVALID_ARGUMENT, "sweep index beyond u32");
    uint32_t need_cols = 0;
    for (int k = 0; k < circuit->num_params; ++k)
        if (circuit->params[k].kind == SP_DRAW_TABLE)
            need_cols = std::max(need_cols, circuit->params[k].rng_index + 1);
    if (need_cols && (!d_table || table_cols < need_cols))
        return report(err, err_len, SP_ERR_INVALID_DIMENSION, "circuit reads %u table columns, got %u",
                      need_cols, d_table ? table_cols : 0);

    // scratch plan: circuit copy, then per-sample arrays
    int nd = 0;
    for (int e = 0; e < circuit->num_elements; ++e) nd += derived_count(circuit->elements[e].kind);
    const size_t be = a256(sizeof(sp_element) * circuit->num_elements);
    const size_t bp = a256(sizeof(sp_param) * circuit->num_params);
    const size_t bu = a256(sizeof(sp_pulse) * circuit->num_pulses);
    const size_t bo = a256(sizeof(int) * circuit->num_elements);
    const size_t bn = a256(sizeof(double) * n);
    const size_t bc = 256;  // counters: [0] miss count, [1] undecided roundings, [4] draw groups
    const size_t bw = a256(sizeof(int) * circuit->num_params);  // drawn (non-fixed) slots
    const size_t fixed = be + bp + bu + bo + bn + bc + bw;
    const size_t per_sample = 8 * (size_t)(circuit->num_params + nd) + 4;
    const uint64_t max_samples = fixed + 3 * 256 < kStaticScratchBytes
                                     ? (kStaticScratchBytes - fixed - 3 * 256) / per_sample : 0;
    if (num_samples > max_samples)
        return report(err, err_len, SP_ERR_BATCH_TOO_LARGE,
                      "Batch size %llu exceeds maximum %llu for this circuit: the static scratch holds %zu bytes",
                      (unsigned long long)num_samples, (unsigned long long)max_samples, kStaticScratchBytes);

    cudaStream_t st = (cudaStream_t)stream;
    // Every call copies the circuit from pageable host memory (partly from
    // this stack frame); a graph recorded from such copies would replay them
    // from memory that no longer holds the circuit, so a capturing stream is
    // refused before anything is enqueued.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(st, &cap);
    if (ce != cudaSuccess)
        return report(err, err_len, SP_ERR_BACKEND, "cudaStreamIsCapturing: %s", cudaGetErrorString(ce));
    if (cap != cudaStreamCaptureStatusNone)
        return report(err, err_len, SP_ERR_INVALID_ARGUMENT,
                      "the stream is capturing: sp_newton_dc_static copies the circuit from host memory on every "
                      "call and cannot be recorded into a CUDA graph");

    DeviceSetup* dev = nullptr;
    int rc = setup_current_device(&dev, err, err_len);
    if (rc) return rc;
    unsigned char* base = dev->scratch;
    sp_element* del = (sp_element*)base;
    sp_param* dpar = (sp_param*)(base + be);
    sp_pulse* dpul = (sp_pulse*)(base + be + bp);
    int* ddoff = (int*)(base + be + bp + bu);
    double* dns = (double*)(base + be + bp + bu + bo);
    unsigned int* counters = (unsigned int*)(base + be + bp + bu + bo + bn);
    int* ddrawn = (int*)(base + be + bp + bu + bo + bn + bc);
    unsigned char* dyn = base + fixed;
    double* params_soa = (double*)dyn;
    double* derived_soa = (double*)(dyn + a256(8 * (size_t)circuit->num_params * num_samples));
    uint32_t* fail_list = (uint32_t*)((unsigned char*)derived_soa + a256(8 * (size_t)nd * num_samples));

    int doff[1024];
    if (circuit->num_elements > 1024)
        return report(err, err_len, SP_ERR_INVALID_DIMENSION, "more than 1024 elements");
    int drawn[1024];
    int num_drawn = 0;
    if (circuit->num_params > 1024)
        return report(err, err_len, SP_ERR_INVALID_DIMENSION, "more than 1024 parameters");
    for (int k = 0; k < circuit->num_params; ++k)
        if (circuit->params[k].kind != SP_DRAW_FIXED) drawn[num_drawn++] = k;
    for (int e = 0, o = 0; e < circuit->num_elements; ++e) {
        doff[e] = o;
        o += derived_count(circuit->elements[e].kind);
    }
    cudaError_t e = cudaSuccess;
    if (circuit->num_elements)
        e = cudaMemcpyAsync(del, circuit->elements, sizeof(sp_element) * circuit->num_elements,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && circuit->num_params)
        e = cudaMemcpyAsync(dpar, circuit->params, sizeof(sp_param) * circuit->num_params, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && circuit->num_pulses)
        e = cudaMemcpyAsync(dpul, circuit->pulses, sizeof(sp_pulse) * circuit->num_pulses, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && circuit->num_elements)
        e = cudaMemcpyAsync(ddoff, doff, sizeof(int) * circuit->num_elements, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && circuit->nodeset)
        e = cudaMemcpyAsync(dns, circuit->nodeset, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && num_drawn)
        e = cudaMemcpyAsync(ddrawn, drawn, sizeof(int) * num_drawn, cudaMemcpyHostToDevice, st);
    // the counters (misses, undecided roundings, draw groups) start at zero on every call
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 32, st);
    if (e != cudaSuccess)
        return report(err, err_len, SP_ERR_TRANSFER, "circuit upload: %s", cudaGetErrorString(e));

    DevCircuit dc{circuit->num_nodes, circuit->num_branches, n, circuit->num_elements, circuit->num_params, nd,
                  del, dpar, dpul, ddoff, circuit->nodeset ? dns : nullptr};
    DrawLaunch D{dc, seed, first_index, num_samples, d_table, table_cols, params_soa, derived_soa, nullptr,
                 counters + 1, ddrawn, num_drawn, counters + 4};
    e = launch_draw(D, st);
    if (e != cudaSuccess) return report(err, err_len, SP_ERR_BACKEND, "draw launch: %s", cudaGetErrorString(e));

    NewtonLaunch L;
    L.c = dc;
    L.cfg = *cfg;
    L.dv = SoA{derived_soa, (size_t)num_samples};
    L.count = num_samples;
    L.x0 = d_x0;
    L.x = d_x;
    L.iters = d_iters;
    L.status = d_status;
    L.resid = d_resid;
    L.fail_list = fail_list;
    L.fail_count = counters;
    const int kprec = prec == SP_PREC_MIXED ? SP_PREC_MIXED : SP_PREC_FP64;
    const size_t per = kprec == SP_PREC_MIXED ? work_bytes_per_thread<SP_PREC_MIXED>(n)
                                              : work_bytes_per_thread<SP_PREC_FP64>(n);
    int block = 128;
    while (block > 32 && per * block > 110 * 1024) block -= 32;
    if (per * block > (size_t)dev->max_smem)
        return report(err, err_len, SP_ERR_INVALID_DIMENSION, "MNA size %d does not fit shared memory", n);
    const size_t smem = per * block;
    const int grid = (int)((num_samples + block - 1) / block);
    NewtonLaunch Lp = L;
    if (d_x0 && cfg->warm_max_iterations > 0 && cfg->warm_max_iterations < cfg->max_iterations)
        Lp.cfg.max_iterations = cfg->warm_max_iterations;
    e = prec == SP_PREC_FP64_EXACT ? launch_newton_exact(Lp, false, grid, block, smem, st)
                                   : launch_newton_fast(kprec, Lp, false, grid, block, smem, st);
    if (e != cudaSuccess) return report(err, err_len, SP_ERR_BACKEND, "newton launch: %s", cudaGetErrorString(e));
    if (d_x0 || (cfg->fallback & (SP_FALLBACK_GMIN | SP_FALLBACK_SOURCE))) {
        const int fgrid = std::min(grid, std::max(1, dev->num_sms * 2));
        e = prec == SP_PREC_FP64_EXACT ? launch_newton_exact(L, true, fgrid, block, smem, st)
                                       : launch_newton_fast(kprec, L, true, fgrid, block, smem, st);
        if (e != cudaSuccess)
            return report(err, err_len, SP_ERR_BACKEND, "fallback launch: %s", cudaGetErrorString(e));
    }
    return SP_OK;
}
