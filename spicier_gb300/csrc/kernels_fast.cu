// Kernels free to use FMA: the mixed-precision Newton path, the FMA build
// of the FP64 Newton path (the fastest plain-FP64 form), the mixed-precision
// batched LU and the statistics reductions.
#include <math_constants.h>

#include <cfloat>

#define SP_KERNEL_NS kfast
#include "internal.h"
#define SP_AC_MIXED_KERNELS
#include "ac.cuh"
#include "ladder.cuh"
#include "transient_fixed.cuh"
#include "powergrid.cuh"
#include <algorithm>

namespace sp {

cudaError_t launch_newton_fast(int prec, const NewtonLaunch& L, bool fallback, int grid, int block,
                               size_t smem, cudaStream_t st) {
    using namespace SP_KERNEL_NS;
    const dim3 g(grid), b(block);
    if (prec == SP_PREC_MIXED)
        return fallback ? launch_chained(newton_fallback_kernel<SP_PREC_MIXED>, g, b, smem, st, L)
                        : launch_chained(newton_primary_kernel<SP_PREC_MIXED>, g, b, smem, st, L);
    return fallback ? launch_chained(newton_fallback_kernel<SP_PREC_FP64>, g, b, smem, st, L)
                    : launch_chained(newton_primary_kernel<SP_PREC_FP64>, g, b, smem, st, L);
}

// Mixed-precision BatchedLuSolver::solve_batch: FP32 partial-pivot LU in
// shared memory, then refine_steps sweeps of FP64 iterative refinement
// (r = b - A x from the FP64 matrix in HBM, d = LU32 \ r, x += d).  A system
// whose final FP64 residual is not at FP64 level (||r|| > 64 eps ||A|| ||x||)
// is refactorised in FP64 with the reference's algorithm.
__global__ void lu_batch_mixed_kernel(const double* __restrict__ mats, const double* __restrict__ rhs,
                                      int n, uint64_t batch, double* __restrict__ sol,
                                      uint8_t* __restrict__ sing, int refine_steps) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= batch) return;
    const int bs = blockDim.x;
    double* dbase = reinterpret_cast<double*>(smem);
    Il<double> x{dbase + threadIdx.x, bs};
    Il<double> r{dbase + (size_t)n * bs + threadIdx.x, bs};
    float* fbase = reinterpret_cast<float*>(dbase + (size_t)2 * n * bs);
    Il<float> A{fbase + threadIdx.x, bs};
    Il<float> d{fbase + (size_t)n * n * bs + threadIdx.x, bs};
    int* ibase = reinterpret_cast<int*>(fbase + (size_t)(n * n + n) * bs);
    Il<int> perm{ibase + threadIdx.x, bs};
    const double* M = mats + s * n * n;
    const double* b = rhs + s * n;
    double anorm = 0.0;
    for (int i = 0; i < n * n; ++i) {
        double v = M[i];
        A[i] = (float)v;
        anorm = fmax(anorm, fabs(v));
    }
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
        int piv = i;
        float best = fabsf(A[i * n + i]);
        for (int q = i + 1; q < n; ++q) {
            float v = fabsf(A[i * n + q]);
            if (v > best) {
                best = v;
                piv = q;
            }
        }
        perm[i] = piv;
        float diag = A[i * n + piv];
        if (diag == 0.0f) {
            ok = false;
            break;
        }
        if (piv != i)
            for (int c = 0; c < n; ++c) {
                float t = A[c * n + i];
                A[c * n + i] = A[c * n + piv];
                A[c * n + piv] = t;
            }
        float inv = 1.0f / diag;
        for (int q = i + 1; q < n; ++q) A[i * n + q] *= inv;
        for (int c = i + 1; c < n; ++c) {
            float p = A[c * n + i];
            for (int q = i + 1; q < n; ++q) A[c * n + q] = fmaf(-p, A[i * n + q], A[c * n + q]);
        }
    }
    double xnorm = 0.0, rnorm = 0.0;
    if (ok) {
        for (int i = 0; i < n; ++i) {
            x[i] = 0.0;
            r[i] = b[i];
        }
        for (int sweep = 0; sweep <= refine_steps; ++sweep) {
            for (int i = 0; i < n; ++i) d[i] = (float)r[i];
            for (int i = 0; i < n; ++i) {
                int p = perm[i];
                if (p != i) {
                    float t = d[i];
                    d[i] = d[p];
                    d[p] = t;
                }
            }
            for (int i = 0; i < n; ++i) {
                float cf = d[i];
                for (int q = i + 1; q < n; ++q) d[q] = fmaf(-cf, A[i * n + q], d[q]);
            }
            for (int i = n - 1; i >= 0; --i) {
                float cf = d[i] / A[i * n + i];
                d[i] = cf;
                for (int q = 0; q < i; ++q) d[q] = fmaf(-cf, A[i * n + q], d[q]);
            }
            xnorm = 0.0;
            for (int i = 0; i < n; ++i) {
                x[i] = x[i] + (double)d[i];
                xnorm = fmax(xnorm, fabs(x[i]));
            }
            for (int i = 0; i < n; ++i) r[i] = b[i];
            for (int c = 0; c < n; ++c) {
                double xc = x[c];
                for (int q = 0; q < n; ++q) r[q] = fma(-M[c * n + q], xc, r[q]);
            }
            rnorm = 0.0;
            for (int i = 0; i < n; ++i) rnorm = fmax(rnorm, fabs(r[i]));
        }
        if (!(rnorm <= 64.0 * DBL_EPSILON * anorm * xnorm * n) || !isfinite(rnorm)) ok = false;
    }
    if (!ok) {
        // FP32 pivot breakdown or refinement short of FP64 accuracy: mark the
        // system for lu_batch_escalate_kernel (FP64 factorisation).
        sing[s] = 2;
        return;
    }
    for (int i = 0; i < n; ++i) sol[s * n + i] = x[i];
    sing[s] = 0;
}

// Re-solve the systems flagged 2 by the mixed kernel in FP64.
__global__ void lu_batch_escalate_kernel(const double* __restrict__ mats, const double* __restrict__ rhs,
                                         int n, uint64_t batch, double* __restrict__ sol,
                                         uint8_t* __restrict__ sing) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= batch) return;
    if (sing[s] != 2) return;
    double* base = reinterpret_cast<double*>(smem);
    Il<double> A{base + threadIdx.x, (int)blockDim.x};
    Il<double> b{base + (size_t)n * n * blockDim.x + threadIdx.x, (int)blockDim.x};
    for (int i = 0; i < n * n; ++i) A[i] = mats[s * n * n + i];
    for (int i = 0; i < n; ++i) b[i] = rhs[s * n + i];
    bool ok = lu_solve_fp64(n, A, b);
    for (int i = 0; i < n; ++i) sol[s * n + i] = ok ? b[i] : 0.0;
    sing[s] = ok ? 0 : 1;
}

cudaError_t launch_lu_batch_mixed(const double* mats, const double* rhs, int n, uint64_t batch,
                                  double* sol, uint8_t* sing, int refine_steps, cudaStream_t st) {
    if (batch == 0) return cudaSuccess;
    size_t per = (size_t)2 * n * 8 + (size_t)(n * n + n) * 4 + (size_t)n * 4;
    int block = 128;
    while (block > 32 && per * block > 110 * 1024) block -= 32;
    lu_batch_mixed_kernel<<<(unsigned)((batch + block - 1) / block), block, per * block, st>>>(
        mats, rhs, n, batch, sol, sing, refine_steps);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    size_t per64 = (size_t)(n * n + n) * 8;
    int b64 = 128;
    while (b64 > 32 && per64 * b64 > 110 * 1024) b64 -= 32;
    lu_batch_escalate_kernel<<<(unsigned)((batch + b64 - 1) / b64), b64, per64 * b64, st>>>(mats, rhs, n,
                                                                                          batch, sol, sing);
    return cudaGetLastError();
}

// Moments of `cols` columns over rows (StatisticsAccumulator::add/merge,
// statistics.rs:127-155).  Pass 1: each block reduces a contiguous row range
// per column in a fixed tree order; pass 2: one block merges the partials in
// block order.  The order is fixed, so reruns are bit-identical.
// min / max by the order-preserving integer keys of the doubles (integer pipe;
// no NaN reaches the accumulators)
__device__ __forceinline__ long long mom_key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b) - 1;
}

__device__ inline void mom_merge(sp_moments& a, const sp_moments& b) {
    a.count += b.count;
    a.sum += b.sum;
    a.sum_sq += b.sum_sq;
    a.min = mom_key(b.min) < mom_key(a.min) ? b.min : a.min;
    a.max = mom_key(b.max) > mom_key(a.max) ? b.max : a.max;
}

__global__ void moments_partial_kernel(const double* __restrict__ v, uint64_t rows, uint32_t ld,
                                       uint32_t cols, const uint8_t* __restrict__ status,
                                       sp_moments* __restrict__ partial) {
    __shared__ sp_moments sh[256];
    const uint32_t col = blockIdx.y;
    const uint64_t per_block = (rows + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = (uint64_t)blockIdx.x * per_block;
    const uint64_t hi = min(rows, lo + per_block);
    sp_moments m{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
    for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
        double x = v[i * ld + col];
        m.count += 1;
        m.sum += x;
        m.sum_sq += x * x;
        m.min = fmin(m.min, x);
        m.max = fmax(m.max, x);
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) mom_merge(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)col * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void moments_final_kernel(const sp_moments* __restrict__ partial, uint32_t nblocks,
                                     uint32_t cols, sp_moments* __restrict__ out) {
    const uint32_t col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= cols) return;
    sp_moments m{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
    for (uint32_t b = 0; b < nblocks; ++b) mom_merge(m, partial[(size_t)col * nblocks + b]);
    out[col] = m;
}

// Narrow tables (cols <= 32): thread t of a block accumulates column t % cp
// (cp = cols rounded up to a power of two) over rows t / cp, t / cp + 256 / cp,
// ... of the block's chunk, so a warp reads whole rows (coalesced); the
// groups of a column are then merged in a fixed order, and the chunks'
// partials by the tree kernel.  The chunk length is a function of rows alone
// (about eight chunks per SM, one batch of loads per thread), so the result
// depends only on rows and cols.
constexpr int kMomChunkMin = 64;

__host__ __device__ inline uint64_t moments_chunk(uint64_t rows, uint32_t max_blocks) {
    const uint64_t target = max_blocks < 1216 ? max_blocks : 1216;  // about eight blocks per SM
    uint64_t chunk = (rows + target - 1) / target;
    chunk = (chunk + kMomChunkMin - 1) / kMomChunkMin * kMomChunkMin;
    return chunk < kMomChunkMin ? kMomChunkMin : chunk;
}

// Order-preserving integer key of a double (IEEE bits with the negative half
// reflected): min/max run on the integer pipe; NaN never reaches here.
__device__ __forceinline__ long long order_key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b) - 1;
}
__device__ __forceinline__ double from_key(long long k) {
    return __longlong_as_double(k >= 0 ? k : (long long)(0x8000000000000000ULL - (unsigned long long)(k + 1)));
}

__global__ void __launch_bounds__(256) moments_rows_kernel(const double* __restrict__ v, uint64_t rows, uint32_t ld,
                                                           uint32_t cols, uint32_t cp, uint64_t chunk,
                                                           const uint8_t* __restrict__ status,
                                                           sp_moments* __restrict__ partial) {
    __shared__ sp_moments sh[256];
    pdl_wait();
    pdl_trigger();
    const uint32_t c = threadIdx.x % cp, g = threadIdx.x / cp, groups = 256 / cp;
    const uint64_t lo = (uint64_t)blockIdx.x * chunk, hi = min(rows, lo + chunk);
    sp_moments m{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
    long long kmin = order_key(CUDART_INF), kmax = order_key(-CUDART_INF);
    if (c < cols) {
        // loads first (four rows in flight per thread), then the fixed-order accumulation
        for (uint64_t i0 = lo + g; i0 < hi; i0 += 4 * (uint64_t)groups) {
            double xs[4];
            bool ok[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint64_t i = i0 + (uint64_t)u * groups;
                ok[u] = i < hi && (!status || (status[i] & SP_ST_MASK) == SP_ST_CONVERGED);
                xs[u] = ok[u] ? v[i * ld + c] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!ok[u]) continue;
                const double x = xs[u];
                m.count += 1;
                m.sum += x;
                m.sum_sq += x * x;
                const long long k = order_key(x);
                kmin = k < kmin ? k : kmin;
                kmax = k > kmax ? k : kmax;
            }
        }
    }
    m.min = from_key(kmin);
    m.max = from_key(kmax);
    sh[threadIdx.x] = m;
    __syncthreads();
    // pairwise tree over the groups (fixed order)
    for (uint32_t w = groups / 2; w >= 1; w >>= 1) {
        if (g < w) mom_merge(sh[threadIdx.x], sh[threadIdx.x + w * cp]);
        __syncthreads();
    }
    if (threadIdx.x < cols) partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = sh[threadIdx.x];
}

// One block per column: each thread merges partials t, t + 256, ... in order,
// then a pairwise tree; deterministic for a given partial count.
__global__ void __launch_bounds__(256) moments_tree_kernel(const sp_moments* __restrict__ partial, uint32_t nblocks,
                                                           sp_moments* __restrict__ out) {
    __shared__ sp_moments sh[256];
    pdl_wait();
    pdl_trigger();
    const uint32_t col = blockIdx.x;
    sp_moments m{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
    for (uint32_t b0 = threadIdx.x; b0 < nblocks; b0 += 4 * 256) {  // four partials in flight, merged in order
        sp_moments q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t b = b0 + (uint32_t)u * 256;
            q[u] = b < nblocks ? partial[(size_t)col * nblocks + b] : sp_moments{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (b0 + (uint32_t)u * 256 < nblocks) mom_merge(m, q[u]);
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w) mom_merge(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[col] = sh[0];
}

__global__ void ac_status_kernel_fast(uint64_t count, const unsigned int* singular, uint8_t* status) {
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count || !singular[s]) return;
    status[s] = (uint8_t)((status[s] & ~SP_ST_MASK) | SP_ST_SINGULAR);
}

cudaError_t launch_ac_mixed(const AcLaunch& L, int grid, int block, size_t smem, cudaStream_t st) {
    ac_mixed_kernel<<<grid, block, smem, st>>>(L);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    ac_status_kernel_fast<<<(unsigned)((L.count + 255) / 256), 256, 0, st>>>(L.count, L.singular,
                                                                            const_cast<uint8_t*>(L.dc_status));
    return cudaGetLastError();
}

// StatisticsAccumulator::merge per unknown (statistics.rs:148-155): acc[i] += other[i].
__global__ void moments_merge_kernel(sp_moments* __restrict__ acc, const sp_moments* __restrict__ other,
                                     uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    sp_moments a = acc[i];
    mom_merge(a, other[i]);
    acc[i] = a;
}

// One block per column: the specialised kernel's block partials merged in
// block order (four in flight per thread, then a pairwise tree), or, when the
// fallback kernel changed samples after those partials were formed, the
// column's moments over every converged row (rows t, t + 256, ... per thread,
// then the same tree).
__global__ void __launch_bounds__(256) moments_partials_kernel(const sp_moments* __restrict__ partial,
                                                                uint32_t nblocks,
                                                                const unsigned int* __restrict__ fail_count,
                                                                const double* __restrict__ v, uint64_t rows,
                                                                uint32_t ld, const uint8_t* __restrict__ status,
                                                                sp_moments* __restrict__ out) {
    __shared__ sp_moments sh[256];
    pdl_wait();
    pdl_trigger();
    const uint32_t col = blockIdx.x;
    sp_moments m{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
    if (*fail_count == 0) {
        for (uint32_t b0 = threadIdx.x; b0 < nblocks; b0 += 4 * 256) {
            sp_moments q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t b = b0 + (uint32_t)u * 256;
                q[u] = b < nblocks ? partial[(size_t)col * nblocks + b] : sp_moments{0, 0.0, 0.0, CUDART_INF, -CUDART_INF};
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (b0 + (uint32_t)u * 256 < nblocks) mom_merge(m, q[u]);
        }
    } else {
        long long kmin = order_key(CUDART_INF), kmax = order_key(-CUDART_INF);
        for (uint64_t i = threadIdx.x; i < rows; i += 256) {
            if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
            const double x = v[i * ld + col];
            m.count += 1;
            m.sum += x;
            m.sum_sq += x * x;
            const long long k = order_key(x);
            kmin = k < kmin ? k : kmin;
            kmax = k > kmax ? k : kmax;
        }
        m.min = from_key(kmin);
        m.max = from_key(kmax);
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w) mom_merge(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[col] = sh[0];
}

cudaError_t launch_moments_from_partials(const sp_moments* partial, uint32_t nblocks, const unsigned int* fail_count,
                                         const double* values, uint64_t rows, uint32_t cols, const uint8_t* status,
                                         sp_moments* out, cudaStream_t st) {
    if (cols == 0) return cudaSuccess;
    return launch_chained(moments_partials_kernel, dim3(cols), dim3(256), 0, st, partial, nblocks, fail_count, values,
                          rows, cols, status, out);
}

cudaError_t launch_moments_merge(sp_moments* acc, const sp_moments* other, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    moments_merge_kernel<<<(n + 127) / 128, 128, 0, st>>>(acc, other, n);
    return cudaGetLastError();
}

cudaError_t launch_moments(const double* values, uint64_t rows, uint32_t ld, uint32_t cols,
                           const uint8_t* status, sp_moments* partial, uint32_t nblocks, sp_moments* out,
                           cudaStream_t st) {
    if (cols == 0) return cudaSuccess;
    if (rows == 0) {  // empty accumulators (count 0, min +inf, max -inf)
        moments_tree_kernel<<<cols, 256, 0, st>>>(partial, 0, out);
        return cudaGetLastError();
    }
    const uint64_t chunk = moments_chunk(rows, nblocks);
    if (cols <= 32 && (rows + chunk - 1) / chunk <= nblocks) {
        uint32_t cp = 1;
        while (cp < cols) cp <<= 1;
        const uint32_t nb = (uint32_t)((rows + chunk - 1) / chunk);
        cudaError_t e = launch_chained(moments_rows_kernel, dim3(nb), dim3(256), 0, st, values, rows, ld, cols, cp,
                                       chunk, status, partial);
        if (e != cudaSuccess) return e;
        return launch_chained(moments_tree_kernel, dim3(cols), dim3(256), 0, st, partial, nb, out);
    }
    nblocks = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(nblocks, 256), std::max<uint64_t>(1, rows / 1024));
    dim3 grid(nblocks, cols);
    moments_partial_kernel<<<grid, 256, 0, st>>>(values, rows, ld, cols, status, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    moments_final_kernel<<<(cols + 127) / 128, 128, 0, st>>>(partial, nblocks, cols, out);
    return cudaGetLastError();
}

// Ladder order, largest first: a histogram of the section counts, its
// exclusive scan from the largest count down, and a scatter.
__global__ void ladder_hist_kernel(sp_ladder_config c, uint64_t seed, uint64_t first, uint64_t count,
                                   unsigned int* hist) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int N = ladder_sections(c, seed, (uint32_t)(first + i));
    atomicAdd(&hist[c.max_sections - N], 1u);
}

__global__ void ladder_scan_kernel(unsigned int* hist, int bins) {
    unsigned int acc = 0;
    for (int b = 0; b < bins; ++b) {
        const unsigned int v = hist[b];
        hist[b] = acc;
        acc += v;
    }
}

__global__ void ladder_order_kernel(sp_ladder_config c, uint64_t seed, uint64_t first, uint64_t count,
                                    unsigned int* offsets, uint32_t* order) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int N = ladder_sections(c, seed, (uint32_t)(first + i));
    order[atomicAdd(&offsets[c.max_sections - N], 1u)] = (uint32_t)i;
}

cudaError_t launch_ladder_prelude(const sp_ladder_config& c, uint64_t seed, uint64_t first, uint64_t count,
                                  unsigned int* hist, uint32_t* order, unsigned int* next, cudaStream_t st) {
    const int bins = c.max_sections - c.min_sections + 1;
    cudaError_t e = cudaMemsetAsync(hist, 0, 4 * (size_t)bins, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(next, 0, 4, st);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((count + 255) / 256);
    ladder_hist_kernel<<<grid, 256, 0, st>>>(c, seed, first, count, hist);
    ladder_scan_kernel<<<1, 1, 0, st>>>(hist, bins);
    ladder_order_kernel<<<grid, 256, 0, st>>>(c, seed, first, count, hist, order);
    return cudaGetLastError();
}

cudaError_t launch_ladder_fast(const LadderLaunch& L, int precision, int grid, size_t smem, cudaStream_t st) {
    if (precision == SP_PREC_MIXED)
        SP_KERNEL_NS::ladder_kernel<SP_PREC_MIXED><<<grid, 128, smem, st>>>(L);
    else
        SP_KERNEL_NS::ladder_kernel<SP_PREC_FP64><<<grid, 128, smem, st>>>(L);
    return cudaGetLastError();
}

// Histogram: per-block shared counts, then one atomic add per bin and block
// (integer counts: the result does not depend on the order).
__global__ void histogram_kernel(const double* __restrict__ v, uint64_t rows, uint32_t ld, uint32_t col,
                                 const uint8_t* __restrict__ status, double mn, double width, uint32_t nb,
                                 unsigned long long* __restrict__ bins) {
    extern __shared__ unsigned int hsm[];
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) hsm[b] = 0;
    __syncthreads();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (uint64_t)gridDim.x * blockDim.x) {
        if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
        const double f = floor((v[i * ld + col] - mn) / width);
        // Rust's `as isize`: NaN -> 0, out of range saturates; then clamp
        long long b = f != f ? 0 : (f < 0.0 ? -1 : (f >= (double)nb ? (long long)nb : (long long)f));
        b = b < 0 ? 0 : (b > (long long)nb - 1 ? (long long)nb - 1 : b);
        atomicAdd(&hsm[b], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x)
        if (hsm[b]) atomicAdd(&bins[b], (unsigned long long)hsm[b]);
}

cudaError_t launch_histogram(const double* v, uint64_t rows, uint32_t ld, uint32_t col, const uint8_t* status,
                             double mn, double mx, uint32_t nb, uint64_t* bins, int num_sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(bins, 0, 8 * (size_t)nb, st);
    if (e != cudaSuccess || rows == 0) return e;
    const unsigned grid = (unsigned)std::min<uint64_t>((rows + 255) / 256, (uint64_t)num_sms * 8);
    histogram_kernel<<<grid, 256, 4 * (size_t)nb, st>>>(v, rows, ld, col, status, mn, (mx - mn) / (double)nb, nb,
                                                        (unsigned long long*)bins);
    return cudaGetLastError();
}

__global__ void yield_kernel(const double* __restrict__ v, uint64_t rows, uint32_t ld,
                             const uint8_t* __restrict__ status, const sp_yield_spec* __restrict__ specs, uint32_t ns,
                             unsigned long long* __restrict__ pass) {
    extern __shared__ unsigned int ysm[];  // [ns + 1]
    for (uint32_t k = threadIdx.x; k <= ns; k += blockDim.x) ysm[k] = 0;
    __syncthreads();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (uint64_t)gridDim.x * blockDim.x) {
        if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
        bool all = true;
        for (uint32_t k = 0; k < ns; ++k) {
            const double x = v[i * ld + specs[k].col];
            const bool ok = x >= specs[k].lower && x <= specs[k].upper;  // YieldSpec::passes
            all = all && ok;
            if (ok) atomicAdd(&ysm[k], 1u);
        }
        if (all) atomicAdd(&ysm[ns], 1u);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k <= ns; k += blockDim.x)
        if (ysm[k]) atomicAdd(&pass[k], (unsigned long long)ysm[k]);
}

cudaError_t launch_yield(const double* v, uint64_t rows, uint32_t ld, const uint8_t* status, const sp_yield_spec* d_specs,
                         uint32_t ns, uint64_t* pass, int num_sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(pass, 0, 8 * ((size_t)ns + 1), st);
    if (e != cudaSuccess || rows == 0) return e;
    const unsigned grid = (unsigned)std::min<uint64_t>((rows + 255) / 256, (uint64_t)num_sms * 8);
    yield_kernel<<<grid, 256, 4 * ((size_t)ns + 1), st>>>(v, rows, ld, status, d_specs, ns, (unsigned long long*)pass);
    return cudaGetLastError();
}

cudaError_t launch_grid(const GridLaunch& L, int precision, cudaStream_t st) {
    if (precision == SP_PREC_MIXED)
        SP_KERNEL_NS::grid_kernel<SP_PREC_MIXED><<<(unsigned)L.count, kGridThreads, grid_smem_bytes(L.cfg, 4), st>>>(L);
    else
        SP_KERNEL_NS::grid_kernel<SP_PREC_FP64><<<(unsigned)L.count, kGridThreads, grid_smem_bytes(L.cfg, 8), st>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_transient_fast(const TransientLaunch& L, int block, size_t smem, cudaStream_t st) {
    const unsigned grid = (unsigned)((L.count + block - 1) / block);
    SP_KERNEL_NS::transient_fixed_kernel<<<grid, block, smem, st>>>(L);
    return cudaGetLastError();
}

cudaError_t prepare_fast_kernels(int max_smem) {
    const void* fns[] = {
        (const void*)SP_KERNEL_NS::grid_kernel<SP_PREC_MIXED>, (const void*)SP_KERNEL_NS::grid_kernel<SP_PREC_FP64>,
        (const void*)SP_KERNEL_NS::transient_fixed_kernel, (const void*)ac_mixed_kernel,
        (const void*)SP_KERNEL_NS::ladder_kernel<SP_PREC_MIXED>, (const void*)SP_KERNEL_NS::ladder_kernel<SP_PREC_FP64>,
        (const void*)SP_KERNEL_NS::newton_primary_kernel<SP_PREC_MIXED>, (const void*)SP_KERNEL_NS::newton_fallback_kernel<SP_PREC_MIXED>,
        (const void*)SP_KERNEL_NS::newton_primary_kernel<SP_PREC_FP64>, (const void*)SP_KERNEL_NS::newton_fallback_kernel<SP_PREC_FP64>,
        (const void*)lu_batch_mixed_kernel, (const void*)lu_batch_escalate_kernel};
    for (const void* f : fns) {
        cudaError_t e = allow_dynamic_smem(f, max_smem);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sp
