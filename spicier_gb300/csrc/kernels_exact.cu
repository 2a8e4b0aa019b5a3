// Kernels that reproduce the reference's IEEE operation sequence.
// Compiled with --fmad=false: no a*b+c is fused, as in the Rust reference.
#define SP_KERNEL_NS kexact
#include "internal.h"
#include <math_constants.h>

#include "rng.cuh"
#include "ladder.cuh"
#include "transient_fixed.cuh"
#define SP_AC_KERNELS
#include "ac.cuh"

namespace sp {

// Per-sample parameter draw (sp_draw_kind) and derived constants.
// gaussian_scaled = mean + z * sigma (rng.rs:148-150), two roundings.
__device__ inline double draw_one(const sp_param& p, uint64_t seed, uint32_t sweep,
                                  const double* row, unsigned* hard) {
    switch (p.kind) {
        case SP_DRAW_FIXED: return p.a;
        case SP_DRAW_GAUSS: return p.a + rng_gaussian(seed, sweep, p.rng_index, hard) * p.b;
        case SP_DRAW_UNIFORM: return p.a + rng_uniform(seed, sweep, p.rng_index) * (p.b - p.a);
        case SP_DRAW_LOGUNIFORM:
            return p.a * cr_exp(rng_uniform(seed, sweep, p.rng_index) * cr_log(p.b / p.a, hard), hard);
        case SP_DRAW_TABLE: return row ? row[p.rng_index] : CUDART_NAN;
    }
    return CUDART_NAN;
}

// Persistent draw kernel: each block takes groups of 32 samples from a
// device counter (a static stride without one) and, per group,
//
//   draws     warp w draws the non-fixed slots drawn[w], drawn[w + 8], ...
//             of the 32 samples (one distribution per warp), then writes
//             its share of the fixed slots;
//   derives   after the block barrier, lane y derives the constants of
//             elements y, y + 8, ... of each sample (fixed slots read from
//             the circuit, drawn ones from the values just written).
//
// A Gaussian is about a thousand integer instructions plus a few FP64 ones
// (the products and the square root), so the kernel is bound by the integer
// ALU pipe; taking groups from a counter keeps every SM busy to the end,
// where a fixed grid of short blocks would leave its last partial wave.
constexpr int kDrawSamples = 32, kDrawLanes = 8;

__global__ void __launch_bounds__(kDrawSamples * kDrawLanes, 4) draw_kernel(DrawLaunch L) {
    pdl_wait();
    pdl_trigger();
    __shared__ unsigned int group_s;
    // linear warm start (x0_out set): weights lin[nout][nin], in_mean[nin],
    // out_mean[nout], then the group's centred inputs pin[nin][32]
    extern __shared__ float lsm[];
    const int nin = L.lin_nin, nout = L.lin_nout;
    float* lin_s = lsm;
    float* inm_s = lsm + nout * nin;
    float* outm_s = inm_s + nin;
    float* pin_s = outm_s + nout;
    const DevCircuit& c = L.c;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int tid = warp * kDrawSamples + lane;
    if (L.x0_out) {
        for (int i = tid; i < nout * nin; i += kDrawSamples * kDrawLanes) lin_s[i] = L.lin[i];
        for (int i = tid; i < nin; i += kDrawSamples * kDrawLanes) inm_s[i] = L.lin_io[i];
        for (int i = tid; i < nout; i += kDrawSamples * kDrawLanes) outm_s[i] = L.lin_io[2 * nin + i];
    }
    const uint64_t groups = (L.count + kDrawSamples - 1) / kDrawSamples;
    unsigned hard = 0;
    for (uint64_t it = 0;; ++it) {
        if (lane == 0 && warp == 0) group_s = L.next ? atomicAdd(L.next, 1u) : (unsigned)(blockIdx.x + it * gridDim.x);
        __syncthreads();
        const uint64_t g = L.next ? (uint64_t)group_s : blockIdx.x + it * gridDim.x;
        if (g >= groups) break;  // the same value in every thread of the block
        const uint64_t s = g * kDrawSamples + (uint64_t)lane;
        const bool live = s < L.count;
        const uint32_t sweep = (uint32_t)(L.first_index + s);
        if (live) {
            const double* row = L.table ? L.table + s * L.table_cols : nullptr;
            for (int d = warp; d < L.num_drawn; d += kDrawLanes) {
                const int k = L.drawn[d];
                const double v = draw_one(c.par[k], L.seed, sweep, row, &hard);
                L.params_soa[(size_t)k * L.count + s] = v;
                if (L.params_out) L.params_out[s * c.num_params + k] = v;
            }
            for (int k = warp; k < c.num_params; k += kDrawLanes) {
                const sp_param p = c.par[k];
                if (p.kind != SP_DRAW_FIXED) continue;
                L.params_soa[(size_t)k * L.count + s] = p.a;
                if (L.params_out) L.params_out[s * c.num_params + k] = p.a;
            }
        }
        __syncthreads();  // this group's parameter slots are written (group_s is read by all)
        auto P = [&](int slot) {
            const sp_param& p = c.par[slot];
            return p.kind == SP_DRAW_FIXED ? p.a : L.params_soa[(size_t)slot * L.count + s];
        };
        if (L.x0_out) {  // the group's centred warm-start inputs, input j by warp j % 8
            for (int j = warp; j < nin; j += kDrawLanes)
                pin_s[j * kDrawSamples + lane] = live ? __double2float_rn(P(L.lin_slots[j])) - inm_s[j] : 0.f;
            __syncthreads();
        }
        if (!live) continue;
        if (L.derive)
            for (int e = warp; e < c.num_elements; e += kDrawLanes) {
                const sp_element el = c.el[e];
                double* out = L.derived_soa + (size_t)c.doff[e] * L.count + s;
                const size_t st = L.count;
                derive_element(el, P, [&](int k, double v) { out[k * st] = v; });
            }
        // linear warm start: lane y evaluates unknowns y, y + 8, ... in FP32 (as
        // the network kernels' linear term), inputs and weights from shared memory
        if (L.x0_out)
            for (int k = warp; k < nout; k += kDrawLanes) {
                float x = outm_s[k];
                for (int j = 0; j < nin; ++j) x = fmaf(lin_s[k * nin + j], pin_s[j * kDrawSamples + lane], x);
                L.x0_out[s * nout + k] = (double)x;
            }
    }
    if (hard && L.hard) atomicAdd(L.hard, hard);
}

// The draws alone, as work items of one warp each: item i is drawn slot
// drawn[i % num_drawn] of the 32-sample group i / num_drawn, taken from a
// device counter by the warp's lane 0.  Used when nothing in this kernel
// consumes a group's parameters together (no derived constants, no warm
// start, no row-major copy), so no block barrier is needed and every warp
// stays busy to the end, where whole groups per block spread a group's drawn
// slots unevenly over the 8 warps (17 slots: one warp draws three, the others
// two, and the block waits for it).  Fixed slots are not written (their
// consumers read them from the circuit).
__global__ void __launch_bounds__(kDrawSamples * kDrawLanes, 4) draw_items_kernel(DrawLaunch L) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const DevCircuit& c = L.c;
    const uint64_t groups = (L.count + kDrawSamples - 1) / kDrawSamples;
    const uint64_t items = groups * (uint64_t)L.num_drawn;
    unsigned hard = 0;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(L.next_items, 1ULL);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= items) break;
        const uint64_t g = item / (uint64_t)L.num_drawn;
        const int k = L.drawn[(int)(item - g * (uint64_t)L.num_drawn)];
        const uint64_t s = g * kDrawSamples + (uint64_t)lane;
        if (s >= L.count) continue;
        const double* row = L.table ? L.table + s * L.table_cols : nullptr;
        L.params_soa[(size_t)k * L.count + s] = draw_one(c.par[k], L.seed, (uint32_t)(L.first_index + s), row, &hard);
    }
    if (hard && L.hard) atomicAdd(L.hard, hard);
}

cudaError_t launch_draw(const DrawLaunch& L, cudaStream_t st) {
    if (L.count == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const uint64_t groups = (L.count + kDrawSamples - 1) / kDrawSamples;
    if (L.next_items && !L.derive && !L.x0_out && !L.params_out) {
        if (L.num_drawn == 0) return cudaSuccess;
        const uint64_t warps = groups * (uint64_t)L.num_drawn;
        const uint64_t grid = std::min<uint64_t>((warps + kDrawLanes - 1) / kDrawLanes, (uint64_t)sms * 4);
        return launch_chained(draw_items_kernel, dim3((unsigned)grid), dim3(kDrawSamples * kDrawLanes), 0, st, L);
    }
    // resident blocks (four per SM at 64 registers); without a counter one block per group
    const uint64_t grid = L.next ? std::min<uint64_t>(groups, (uint64_t)sms * 4) : groups;
    const size_t smem = L.x0_out ? sizeof(float) * ((size_t)L.lin_nout * L.lin_nin + L.lin_nin + L.lin_nout +
                                                    (size_t)L.lin_nin * kDrawSamples)
                                 : 0;
    return launch_chained(draw_kernel, dim3((unsigned)grid), dim3(kDrawSamples, kDrawLanes), smem, st, L);
}

// Batched Bsim3Mosfet::evaluate (one thread per device): the per-sample
// constants from the device's card, then the evaluation at its bias.
__global__ void bsim3_eval_kernel(int pmos, const double* __restrict__ card, const double* __restrict__ bias,
                                  uint64_t count, double* __restrict__ out, uint8_t* __restrict__ region) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double* c = card + i * SP_B3_CARD;
    double k[B3C_COUNT];
    bsim3_constants([&](int j) { return c[j]; }, [&](int j, double v) { k[j] = v; });
    const Bsim3Out r = bsim3_eval(pmos != 0, [&](int j) { return k[j]; }, bias[3 * i], bias[3 * i + 1], bias[3 * i + 2]);
    double* o = out + 6 * i;
    o[0] = r.ids;
    o[1] = r.gds;
    o[2] = r.gm;
    o[3] = r.gmbs;
    o[4] = r.vth;
    o[5] = r.vdsat;
    if (region) region[i] = (uint8_t)r.region;
}

cudaError_t launch_bsim3_eval(int pmos, const double* card, const double* bias, uint64_t count, double* out,
                              uint8_t* region, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const int block = 128;
    bsim3_eval_kernel<<<(unsigned)((count + block - 1) / block), block, 0, st>>>(pmos, card, bias, count, out,
                                                                                region);
    return cudaGetLastError();
}

__global__ void rng_fill_kernel(int kind, uint64_t seed, uint64_t first, uint32_t param, uint64_t count,
                                double* out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t s = (uint32_t)(first + i);
    unsigned hard = 0;
    switch (kind) {
        case 0: out[i] = rng_uniform(seed, s, param); break;
        case 1: out[i] = rng_gaussian(seed, s, param, &hard); break;
        case 2: out[i] = (double)rng_uniform_f32(seed, s, param); break;
        default: out[i] = (double)rng_gaussian_f32(seed, s, param); break;
    }
}

cudaError_t launch_rng_fill(int kind, uint64_t seed, uint64_t first, uint32_t param, uint64_t count,
                            double* out, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const int block = 256;
    rng_fill_kernel<<<(unsigned)((count + block - 1) / block), block, 0, st>>>(kind, seed, first, param,
                                                                              count, out);
    return cudaGetLastError();
}

cudaError_t launch_newton_exact(const NewtonLaunch& L, bool fallback, int grid, int block, size_t smem,
                                cudaStream_t st) {
    if (fallback) return launch_chained(SP_KERNEL_NS::newton_fallback_kernel<SP_PREC_FP64>, dim3(grid), dim3(block), smem, st, L);
    return launch_chained(SP_KERNEL_NS::newton_primary_kernel<SP_PREC_FP64>, dim3(grid), dim3(block), smem, st, L);
}

// BatchedLuSolver::solve_batch in FP64 with the reference's LU
// (CpuBatchedSolver, solver.rs:326-384): one thread per system, column-major
// input copied into interleaved shared memory; singular -> zero solution.
__global__ void lu_batch_fp64_kernel(const double* __restrict__ mats, const double* __restrict__ rhs,
                                     int n, uint64_t batch, double* __restrict__ sol,
                                     uint8_t* __restrict__ sing) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= batch) return;
    double* base = reinterpret_cast<double*>(smem);
    Il<double> A{base + threadIdx.x, (int)blockDim.x};
    Il<double> b{base + (size_t)n * n * blockDim.x + threadIdx.x, (int)blockDim.x};
    const double* m = mats + s * n * n;
    for (int i = 0; i < n * n; ++i) A[i] = m[i];
    for (int i = 0; i < n; ++i) b[i] = rhs[s * n + i];
    bool ok = lu_solve_fp64(n, A, b);
    for (int i = 0; i < n; ++i) sol[s * n + i] = ok ? b[i] : 0.0;
    sing[s] = ok ? 0 : 1;
}

cudaError_t launch_lu_batch_exact(const double* mats, const double* rhs, int n, uint64_t batch,
                                  double* sol, uint8_t* sing, cudaStream_t st) {
    if (batch == 0) return cudaSuccess;
    size_t per = (size_t)(n * n + n) * 8;
    int block = 128;
    while (block > 32 && per * block > 110 * 1024) block -= 32;
    size_t smem = per * block;
    lu_batch_fp64_kernel<<<(unsigned)((batch + block - 1) / block), block, smem, st>>>(mats, rhs, n, batch,
                                                                                     sol, sing);
    return cudaGetLastError();
}

// The same solve for n beyond the one-thread-per-system limit: one CTA per
// system.  Each step's pivot search (warp 0: first index of the largest
// |a|, NaN never chosen, the diagonal kept when it is NaN), row swap,
// scaling and rank-1 update touch every element in the order and with the
// operations of lu_solve_fp64, only spread over threads, so the solution is
// bit-identical.  A and b live in shared memory when they fit, else in a
// per-CTA slice of global memory (work).
__global__ void __launch_bounds__(256) lu_batch_cta_kernel(const double* __restrict__ mats,
                                                           const double* __restrict__ rhs, int n, uint64_t batch,
                                                           double* __restrict__ sol, uint8_t* __restrict__ sing,
                                                           double* __restrict__ work) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_piv[2];
    __shared__ double s_diag[2];
    __shared__ int s_bad;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    const size_t nn = (size_t)n * n;
    double* A = work ? work + (size_t)blockIdx.x * (nn + n) : reinterpret_cast<double*>(smem);
    double* b = A + nn;
    for (uint64_t s = blockIdx.x; s < batch; s += gridDim.x) {
        const double* m = mats + s * nn;
        for (size_t k = tid; k < nn; k += blockDim.x) A[k] = m[k];
        for (int k = tid; k < n; k += blockDim.x) b[k] = rhs[s * n + k];
        __syncthreads();
        for (int i = 0; i < n; ++i) {
            double* col = A + (size_t)i * n;  // column i: entries (r, i), r = 0..n-1
            if (wid == 0) {
                int piv = i;
                if (!isnan(col[i])) {
                    double best = -1.0;
                    int bi = n;
                    for (int r = i + lane; r < n; r += 32) {
                        const double v = fabs(col[r]);
                        if (v > best) {
                            best = v;
                            bi = r;
                        }
                    }
#pragma unroll
                    for (int o = 16; o; o >>= 1) {
                        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                        if (ob > best || (ob == best && oi < bi)) {
                            best = ob;
                            bi = oi;
                        }
                    }
                    piv = bi;
                }
                if (lane == 0) {
                    s_piv[i & 1] = piv;
                    s_diag[i & 1] = col[piv];
                }
            }
            __syncthreads();
            const int piv = s_piv[i & 1];
            const double diag = s_diag[i & 1];
            if (diag == 0.0) continue;
            if (piv != i) {
                for (int c = tid; c < n; c += blockDim.x) {
                    double* cc = A + (size_t)c * n;
                    const double t = cc[i];
                    cc[i] = cc[piv];
                    cc[piv] = t;
                }
                if (tid == 0) {
                    const double t = b[i];
                    b[i] = b[piv];
                    b[piv] = t;
                }
                __syncthreads();
            }
            const double inv = 1.0 / diag;
            for (int r = i + 1 + tid; r < n; r += blockDim.x) col[r] = col[r] * inv;
            __syncthreads();
            for (int c = i + 1 + wid; c < n; c += nw) {
                double* cc = A + (size_t)c * n;
                const double p = cc[i];
                for (int r = i + 1 + lane; r < n; r += 32) cc[r] = -p * col[r] + cc[r];
            }
            __syncthreads();
        }
        // substitutions by warp 0 (warp-synchronous)
        if (wid == 0) {
            for (int i = 0; i < n; ++i) {
                const double coeff = b[i];
                const double* col = A + (size_t)i * n;
                for (int r = i + 1 + lane; r < n; r += 32) b[r] = -coeff * col[r] + b[r];
                __syncwarp();
            }
            bool ok = true;
            for (int i = n - 1; i >= 0; --i) {
                const double* col = A + (size_t)i * n;
                const double diag = col[i];
                if (diag == 0.0) {
                    ok = false;
                    break;
                }
                const double coeff = b[i] / diag;
                __syncwarp();
                if (lane == 0) b[i] = coeff;
                for (int r = lane; r < i; r += 32) b[r] = -coeff * col[r] + b[r];
                __syncwarp();
            }
            if (lane == 0) s_bad = ok ? 0 : 1;
        }
        __syncthreads();
        const bool bad = s_bad != 0;
        for (int k = tid; k < n; k += blockDim.x) sol[s * n + k] = bad ? 0.0 : b[k];
        if (tid == 0) sing[s] = bad ? 1 : 0;
        __syncthreads();  // before the next system overwrites A and b
    }
}

size_t lu_batch_cta_smem(int n) { return ((size_t)n * n + n) * 8; }

cudaError_t launch_lu_batch_cta(const double* mats, const double* rhs, int n, uint64_t batch, double* sol,
                                uint8_t* sing, double* work, int grid, cudaStream_t st) {
    if (batch == 0) return cudaSuccess;
    const size_t smem = work ? 0 : lu_batch_cta_smem(n);
    lu_batch_cta_kernel<<<grid, 256, smem, st>>>(mats, rhs, n, batch, sol, sing, work);
    return cudaGetLastError();
}

cudaError_t launch_ac(const AcLaunch& L, int grid, int block, size_t smem, cudaStream_t st) {
    ac_kernel<<<grid, block, smem, st>>>(L);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    ac_status_kernel<<<(unsigned)((L.count + 255) / 256), 256, 0, st>>>(L.count, L.dc_status, L.singular,
                                                                       const_cast<uint8_t*>(L.dc_status));
    return cudaGetLastError();
}

cudaError_t launch_ladder_exact(const LadderLaunch& L, int grid, size_t smem, cudaStream_t st) {
    SP_KERNEL_NS::ladder_kernel<SP_PREC_FP64_EXACT><<<grid, 128, smem, st>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_transient_exact(const TransientLaunch& L, int block, size_t smem, cudaStream_t st) {
    const unsigned grid = (unsigned)((L.count + block - 1) / block);
    SP_KERNEL_NS::transient_fixed_kernel<<<grid, block, smem, st>>>(L);
    return cudaGetLastError();
}

cudaError_t prepare_exact_kernels(int max_smem) {
    const void* fns[] = {(const void*)SP_KERNEL_NS::newton_primary_kernel<SP_PREC_FP64>,
                         (const void*)SP_KERNEL_NS::newton_fallback_kernel<SP_PREC_FP64>,
                         (const void*)SP_KERNEL_NS::transient_fixed_kernel,
                         (const void*)SP_KERNEL_NS::ladder_kernel<SP_PREC_FP64_EXACT>, (const void*)ac_kernel,
                         (const void*)lu_batch_fp64_kernel, (const void*)lu_batch_cta_kernel};
    for (const void* f : fns) {
        cudaError_t e = allow_dynamic_smem(f, max_smem);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sp
