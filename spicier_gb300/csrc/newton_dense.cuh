// Batched dense Newton-Raphson DC operating points, one thread per sample.
//
// Follows solve_newton_raphson (crates/spicier-solver/src/newton.rs:70-131):
// restamp at the current iterate, solve the linearised system, test the step
// with check_convergence (newton.rs:134-159), take the full step; gmin and
// source stepping (newton.rs:261-459) are the fallback chain.
//
// Work layout: every per-sample array lives in shared memory, interleaved
// across the threads of the block (element i of thread t at
// base[i * blockDim + t]), so each warp-wide access touches 32 consecutive
// words: no bank conflicts for FP32 and two wavefronts for FP64.
//
// Precision modes (template PREC):
//   SP_PREC_FP64  — the reference's arithmetic: the FP64 system A x_new = b
//                   is factorised with the same partial-pivot LU as
//                   nalgebra's LU::new/solve (column icamax pivot, multipliers
//                   scaled by 1/diag, column-oriented axpy updates).  Built
//                   without FMA contraction it is bit-identical to the
//                   reference on circuits without transcendental models.
//   SP_PREC_MIXED — correction form: the FP64 KCL residual F(x) = A(x)x - b(x)
//                   is accumulated from the stamps, the Jacobian A(x) is
//                   stored and factorised in FP32, delta = -A32^-1 F is taken
//                   in FP32 and the update x += delta, the convergence test
//                   and the device models stay FP64.  Newton itself is the
//                   FP64 iterative refinement: the fixed point is the FP64
//                   root of F, independent of the FP32 factorisation error.
#pragma once
#include "circuit_dev.cuh"
#include "pdl.cuh"

namespace sp {

template <class T>
struct Il {  // interleaved per-thread array view
    T* base;
    int bs;
    __device__ T& operator[](int i) const { return base[(size_t)i * bs]; }
};

struct PlainSink {
    Il<double> A, b, xs;
    int n;
    __device__ double x(int i) const { return xs[i]; }
    __device__ void add(int r, int c, double v) { A[c * n + r] += v; }
    __device__ void rhs_add(int r, double v) { b[r] += v; }
    __device__ void rhs_set(int r, double v) { b[r] = v; }
};

// Jacobian in FP32, residual F = A x - b in FP64 (only one element writes a
// branch row's RHS, so rhs_set is a subtraction from zero).
struct MixedSink {
    Il<float> J;
    Il<double> F, xs;
    int n;
    __device__ double x(int i) const { return xs[i]; }
    __device__ void add(int r, int c, double v) {
        J[c * n + r] += (float)v;
        F[r] += v * xs[c];
    }
    __device__ void rhs_add(int r, double v) { F[r] -= v; }
    __device__ void rhs_set(int r, double v) { F[r] -= v; }
};

struct ResidSink {
    Il<double> F, xs;
    __device__ double x(int i) const { return xs[i]; }
    __device__ void add(int r, int c, double v) { F[r] += v * xs[c]; }
    __device__ void rhs_add(int r, double v) { F[r] -= v; }
    __device__ void rhs_set(int r, double v) { F[r] -= v; }
};

// nalgebra-order partial-pivot LU solve of A (column-major, A[c*n+r]) with
// b overwritten by x.  The row permutation is applied to b as it is found,
// which is the order in which LU::solve replays it.  Returns false on a zero
// pivot (the system is singular).
__device__ inline bool lu_solve_fp64(int n, Il<double> A, Il<double> b) {
    for (int i = 0; i < n; ++i) {
        int piv = i;
        double best = fabs(A[i * n + i]);
        for (int r = i + 1; r < n; ++r) {
            double v = fabs(A[i * n + r]);
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        double diag = A[i * n + piv];
        if (diag == 0.0) continue;
        if (piv != i) {
            for (int c = 0; c < n; ++c) {
                double t = A[c * n + i];
                A[c * n + i] = A[c * n + piv];
                A[c * n + piv] = t;
            }
            double t = b[i];
            b[i] = b[piv];
            b[piv] = t;
        }
        double inv = 1.0 / diag;
        for (int r = i + 1; r < n; ++r) A[i * n + r] = A[i * n + r] * inv;
        for (int c = i + 1; c < n; ++c) {
            double p = A[c * n + i];
            for (int r = i + 1; r < n; ++r) A[c * n + r] = -p * A[i * n + r] + A[c * n + r];
        }
    }
    for (int i = 0; i < n; ++i) {
        double coeff = b[i];
        for (int r = i + 1; r < n; ++r) b[r] = -coeff * A[i * n + r] + b[r];
    }
    for (int i = n - 1; i >= 0; --i) {
        double diag = A[i * n + i];
        if (diag == 0.0) return false;
        double coeff = b[i] / diag;
        b[i] = coeff;
        for (int r = 0; r < i; ++r) b[r] = -coeff * A[i * n + r] + b[r];
    }
    return true;
}

// FP32 partial-pivot LU solve (same algorithm, FMA allowed).
__device__ inline bool lu_solve_fp32(int n, Il<float> A, Il<float> b) {
    for (int i = 0; i < n; ++i) {
        int piv = i;
        float best = fabsf(A[i * n + i]);
        for (int r = i + 1; r < n; ++r) {
            float v = fabsf(A[i * n + r]);
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        float diag = A[i * n + piv];
        if (diag == 0.0f) continue;
        if (piv != i) {
            for (int c = 0; c < n; ++c) {
                float t = A[c * n + i];
                A[c * n + i] = A[c * n + piv];
                A[c * n + piv] = t;
            }
            float t = b[i];
            b[i] = b[piv];
            b[piv] = t;
        }
        float inv = 1.0f / diag;
        for (int r = i + 1; r < n; ++r) A[i * n + r] *= inv;
        for (int c = i + 1; c < n; ++c) {
            float p = A[c * n + i];
            for (int r = i + 1; r < n; ++r) A[c * n + r] = fmaf(-p, A[i * n + r], A[c * n + r]);
        }
    }
    for (int i = 0; i < n; ++i) {
        float coeff = b[i];
        for (int r = i + 1; r < n; ++r) b[r] = fmaf(-coeff, A[i * n + r], b[r]);
    }
    for (int i = n - 1; i >= 0; --i) {
        float diag = A[i * n + i];
        if (diag == 0.0f) return false;
        float coeff = b[i] / diag;
        b[i] = coeff;
        for (int r = 0; r < i; ++r) b[r] = fmaf(-coeff, A[i * n + r], b[r]);
    }
    return true;
}

// Shared-memory work area of one thread.
struct Work {
    Il<double> x;   // current iterate [n]
    Il<double> v;   // FP64: RHS / new iterate [n];  MIXED: residual F [n]
    Il<double> A;   // FP64 matrix [n*n]               (PREC FP64)
    Il<float> J;    // FP32 Jacobian [n*n]             (PREC MIXED)
    Il<float> d;    // FP32 RHS / step [n]             (PREC MIXED)
};

template <int PREC>
__host__ __device__ inline size_t work_bytes_per_thread(int n) {
    if (PREC == SP_PREC_FP64) return (size_t)(2 * n + n * n) * 8;
    // doubles first (x, F), then floats (J, d): 8-byte alignment preserved
    return (size_t)(2 * n) * 8 + (size_t)(n * n + n) * 4;
}

template <int PREC>
__device__ inline Work make_work(unsigned char* smem, int n, int bs, int tid) {
    Work w;
    double* dp = reinterpret_cast<double*>(smem);
    w.x = Il<double>{dp + tid, bs};
    w.v = Il<double>{dp + (size_t)n * bs + tid, bs};
    if (PREC == SP_PREC_FP64) {
        w.A = Il<double>{dp + (size_t)2 * n * bs + tid, bs};
        w.J = Il<float>{nullptr, bs};
        w.d = Il<float>{nullptr, bs};
    } else {
        float* fp = reinterpret_cast<float*>(dp + (size_t)2 * n * bs);
        w.A = Il<double>{nullptr, bs};
        w.J = Il<float>{fp + tid, bs};
        w.d = Il<float>{fp + (size_t)n * n * bs + tid, bs};
    }
    return w;
}

enum NrResultCode { NR_CONVERGED = 0, NR_MAXITER = 1, NR_SINGULAR = 2 };

// check_convergence (newton.rs:134-159) for old x and new xn.
__device__ inline bool step_ok(double old, double nw, double reltol, double abstol) {
    double delta = fabs(nw - old);
    double tol = reltol * fmax(fabs(nw), fabs(old)) + abstol;
    return !(delta > tol);
}

// One solve_newton_raphson from w.x; w.x holds the last iterate on return.
template <int PREC>
__device__ inline int newton_run(const DevCircuit& c, const SoA& dv, size_t s,
                                 const sp_newton_config& cfg, int mode, double aux, Work& w,
                                 int& iters) {
    const int n = c.n;
    const int nn = c.num_nodes;
    for (int it = 0; it < cfg.max_iterations; ++it) {
        if (PREC == SP_PREC_FP64) {
            for (int i = 0; i < n * n; ++i) w.A[i] = 0.0;
            for (int i = 0; i < n; ++i) w.v[i] = 0.0;
            PlainSink k{w.A, w.v, w.x, n};
            stamp_all(c, dv, s, k, mode, aux);
            if (!lu_solve_fp64(n, w.A, w.v)) {
                iters = it + 1;
                return NR_SINGULAR;
            }
            bool conv = true;
            for (int i = 0; i < n; ++i) {
                double xo = w.x[i], xn = w.v[i];
                conv = conv && step_ok(xo, xn, cfg.v_reltol, i < nn ? cfg.v_abstol : cfg.i_abstol);
                w.x[i] = xn;
            }
            if (conv) {
                iters = it + 1;
                return NR_CONVERGED;
            }
        } else {
            for (int i = 0; i < n * n; ++i) w.J[i] = 0.0f;
            for (int i = 0; i < n; ++i) w.v[i] = 0.0;
            MixedSink k{w.J, w.v, w.x, n};
            stamp_all(c, dv, s, k, mode, aux);
            for (int i = 0; i < n; ++i) w.d[i] = (float)(-w.v[i]);
            if (!lu_solve_fp32(n, w.J, w.d)) {
                iters = it + 1;
                return NR_SINGULAR;
            }
            bool conv = true;
            for (int i = 0; i < n; ++i) {
                double xo = w.x[i];
                double xn = xo + (double)w.d[i];
                conv = conv && step_ok(xo, xn, cfg.v_reltol, i < nn ? cfg.v_abstol : cfg.i_abstol);
                w.x[i] = xn;
            }
            if (conv) {
                iters = it + 1;
                return NR_CONVERGED;
            }
        }
    }
    iters = cfg.max_iterations;
    return NR_MAXITER;
}

// max_i<num_nodes |F_i| of the FP64 KCL residual at w.x (uses w.v as scratch).
__device__ inline double kcl_residual(const DevCircuit& c, const SoA& dv, size_t s, Work& w) {
    for (int i = 0; i < c.n; ++i) w.v[i] = 0.0;
    ResidSink k{w.v, w.x};
    stamp_all(c, dv, s, k, STAMP_PLAIN, 0.0);
    double r = 0.0;
    for (int i = 0; i < c.num_nodes; ++i) r = fmax(r, fabs(w.v[i]));
    return r;
}

struct NewtonLaunch {
    DevCircuit c;
    sp_newton_config cfg;
    SoA dv;                 // derived constants [num_derived][stride]
    uint64_t count;         // samples in this call
    const double* x0;       // [count][n] warm starts or nullptr
    double* x;              // [count][n] output
    int32_t* iters;         // [count]
    uint8_t* status;        // [count]
    double* resid;          // [count] or nullptr
    uint32_t* fail_list;    // [count]
    unsigned int* fail_count;
    unsigned long long* work_next = nullptr;  // zeroed work counter of the persistent kernels
    // learned linear warm start evaluated by the topology-specialised kernel
    // (x0 == nullptr): x0[k] = lin_io[2 nin + k] + sum_j lin[k][j] (p[lin_slots[j]] - lin_io[j])
    // with p the sample's parameters at lin_params[slot * lin_pstride + s]
    const double* lin_params = nullptr;
    uint64_t lin_pstride = 0;
    const float* lin = nullptr;
    const float* lin_io = nullptr;
    const int* lin_slots = nullptr;
    int lin_nin = 0;
    // host copies of lin, lin_io and lin_slots (the specialised kernel takes the
    // linear term as a launch parameter when its inputs allow)
    const float* lin_host = nullptr;
    const float* lin_io_host = nullptr;
    const int* lin_slots_host = nullptr;
    // per-sample parameters [slot][params_stride] for the specialised kernel's
    // parameters mode, which writes the FP64 derived constants of the samples it
    // lists for the fallback into derived_out (same layout as dv)
    const double* params = nullptr;
    uint64_t params_stride = 0;
    double* derived_out = nullptr;
    // per-block moments of the specialised kernel (one sample per thread), [n][grid]
    sp_moments* moments_partial = nullptr;
    // iteration limit of the specialised kernel's cold restart of a sample
    // whose warm start missed (the full limit; cfg may hold the warm cap)
    int cold_max_iterations = 0;
};

__device__ inline void load_start(const NewtonLaunch& L, size_t s, Work& w, bool warm) {
    const int n = L.c.n;
    if (warm) {
        for (int i = 0; i < n; ++i) w.x[i] = L.x0[s * n + i];
    } else if (L.c.nodeset) {
        for (int i = 0; i < n; ++i) w.x[i] = L.c.nodeset[i];
    } else {
        for (int i = 0; i < n; ++i) w.x[i] = 0.0;
    }
}

__device__ inline uint8_t finish_status(int code, const Work& w, int n) {
    for (int i = 0; i < n; ++i)
        if (!isfinite(w.x[i])) return SP_ST_NONFINITE;
    if (code == NR_CONVERGED) return SP_ST_CONVERGED;
    return code == NR_SINGULAR ? SP_ST_SINGULAR : SP_ST_FAILED;
}

// The __global__ templates below are instantiated by two translation units
// compiled with different FMA settings; each unit picks its own namespace
// (SP_KERNEL_NS) so that the two instantiations are distinct kernels.
#ifndef SP_KERNEL_NS
#define SP_KERNEL_NS kdefault
#endif
namespace SP_KERNEL_NS {

// Phase 1: Newton from the warm start (or the circuit's nodeset, or zero)
// for every sample; misses go to the fallback list.
template <int PREC>
__global__ void newton_primary_kernel(NewtonLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_wait();
    pdl_trigger();
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.count) return;
    Work w = make_work<PREC>(smem, L.c.n, blockDim.x, threadIdx.x);
    const int n = L.c.n;
    const bool warm = L.x0 != nullptr;
    load_start(L, s, w, warm);
    int it = 0;
    int code = newton_run<PREC>(L.c, L.dv, s, L.cfg, STAMP_PLAIN, 0.0, w, it);
    uint8_t st = finish_status(code, w, n) | (warm ? SP_ST_FLAG_WARM : 0);
    for (int i = 0; i < n; ++i) L.x[s * n + i] = w.x[i];
    if (L.iters) L.iters[s] = it;
    bool need_fallback = (st & SP_ST_MASK) != SP_ST_CONVERGED &&
                         (warm || (L.cfg.fallback & (SP_FALLBACK_GMIN | SP_FALLBACK_SOURCE)));
    if (need_fallback) {
        unsigned int slot = atomicAdd(L.fail_count, 1u);
        L.fail_list[slot] = (uint32_t)s;
    } else if (L.resid) {
        L.resid[s] = kcl_residual(L.c, L.dv, s, w);
    }
    if (L.status) L.status[s] = st;
}

}  // namespace SP_KERNEL_NS

// gmin stepping (newton.rs:373-459).  The level solution lives in the
// output row (global), the trial iterate in shared memory.  A failed attempt
// is repeated by the reference with the identical initial guess and stamper,
// so its outcome repeats; those repeats are accounted without recomputation.
template <int PREC>
__device__ inline int gmin_stepping(const NewtonLaunch& L, size_t s, Work& w, int& total) {
    const int n = L.c.n;
    const sp_newton_config& cfg = L.cfg;
    double* sol = L.x + s * n;
    for (int i = 0; i < n; ++i) sol[i] = 0.0;
    double g = cfg.gmin_initial;
    int levels = 0;
    while (g >= cfg.gmin_final * 0.99 && levels < 4096) {
        ++levels;
        for (int i = 0; i < n; ++i) w.x[i] = sol[i];
        int it = 0;
        int code = newton_run<PREC>(L.c, L.dv, s, cfg, STAMP_GMIN, g, w, it);
        total += it;
        if (code == NR_SINGULAR) return NR_SINGULAR;
        if (code != NR_CONVERGED) {
            total += (cfg.gmin_max_attempts - 1) * it;
            return NR_MAXITER;
        }
        for (int i = 0; i < n; ++i) sol[i] = w.x[i];
        if (g <= cfg.gmin_final) break;
        g /= cfg.gmin_reduction;
        if (g < cfg.gmin_final) g = cfg.gmin_final;
    }
    return NR_CONVERGED;
}

// source stepping (newton.rs:261-356).
template <int PREC>
__device__ inline int source_stepping(const NewtonLaunch& L, size_t s, Work& w, int& total) {
    const int n = L.c.n;
    const sp_newton_config& cfg = L.cfg;
    double* sol = L.x + s * n;
    for (int i = 0; i < n; ++i) sol[i] = 0.0;
    double factor = cfg.src_initial;
    double step = cfg.src_step;
    int guard = 0;
    while (factor <= 1.0 + 1e-9 && guard < 100000) {
        ++guard;
        double cur = fmin(factor, 1.0);
        for (int i = 0; i < n; ++i) w.x[i] = sol[i];
        int it = 0;
        int code = newton_run<PREC>(L.c, L.dv, s, cfg, STAMP_SCALED, cur, w, it);
        total += it;
        if (code == NR_SINGULAR) return NR_SINGULAR;
        if (code != NR_CONVERGED) {
            total += (cfg.src_max_attempts - 1) * it;
            if (step > cfg.src_min_step) {
                step /= 2.0;
                factor -= step;
                continue;
            }
            return NR_MAXITER;
        }
        for (int i = 0; i < n; ++i) sol[i] = w.x[i];
        if (fabs(cur - 1.0) < 1e-9) break;
        factor += step;
        if (step < cfg.src_step) step = fmin(step * 1.5, cfg.src_step);
    }
    return NR_CONVERGED;
}

namespace SP_KERNEL_NS {

// Phase 2: the fallback chain for the samples phase 1 missed (grid-stride
// over the miss list, whose length is only known on the device).
template <int PREC>
__global__ void newton_fallback_kernel(NewtonLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_wait();
    pdl_trigger();
    Work w = make_work<PREC>(smem, L.c.n, blockDim.x, threadIdx.x);
    const int n = L.c.n;
    const bool warm = L.x0 != nullptr || L.lin != nullptr;  // listed samples started warm
    const unsigned int misses = *L.fail_count;
    for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < misses; j += gridDim.x * blockDim.x) {
        const size_t s = L.fail_list[j];
        int total = L.iters ? L.iters[s] : 0;
        uint8_t flags = warm ? SP_ST_FLAG_WARM : 0;
        // A stage succeeds only if it converged with a finite iterate (the
        // reference's convergence test passes NaN iterates).
        auto ok = [&](int code) {
            if (code != NR_CONVERGED) return false;
            for (int i = 0; i < n; ++i)
                if (!isfinite(L.x[s * n + i])) return false;
            return true;
        };
        int code = NR_MAXITER;
        // the specialised kernel has already restarted this sample cold (status
        // flag), so the chain continues with gmin stepping
        const bool cold_done = warm && L.status && (L.status[s] & SP_ST_FLAG_COLD);
        if (cold_done) flags |= SP_ST_FLAG_COLD;
        if (warm && !cold_done) {
            flags |= SP_ST_FLAG_COLD;
            load_start(L, s, w, false);
            int it = 0;
            code = newton_run<PREC>(L.c, L.dv, s, L.cfg, STAMP_PLAIN, 0.0, w, it);
            total += it;
            for (int i = 0; i < n; ++i) L.x[s * n + i] = w.x[i];
        }
        if (!ok(code) && (L.cfg.fallback & SP_FALLBACK_GMIN)) {
            flags |= SP_ST_FLAG_GMIN;
            code = gmin_stepping<PREC>(L, s, w, total);
        }
        if (!ok(code) && (L.cfg.fallback & SP_FALLBACK_SOURCE)) {
            flags |= SP_ST_FLAG_SOURCE;
            code = source_stepping<PREC>(L, s, w, total);
        }
        for (int i = 0; i < n; ++i) w.x[i] = L.x[s * n + i];
        uint8_t st = finish_status(code, w, n) | flags;
        if (L.iters) L.iters[s] = total;
        if (L.status) L.status[s] = st;
        if (L.resid) L.resid[s] = kcl_residual(L.c, L.dv, s, w);
    }
}

}  // namespace SP_KERNEL_NS
}  // namespace sp
