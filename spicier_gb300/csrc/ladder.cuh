// Batched nonlinear transient of RC-diode ladders on the GPU.
//
// One warp integrates one ladder from t = 0 to tstop; warps take ladders
// from a work counter in order of decreasing size (the longest first), so a
// single persistent launch covers instances of 10 to 514 unknowns.  Inside a
// warp, lane l owns sections k = 1 + l + 32 j: it draws their R and C, keeps
// their capacitor states, evaluates their diodes and assembles their rows;
// the tridiagonal solve of each Newton iteration runs in the warp's shared
// memory.  The algorithm (step, controller, Newton per stage) is the one
// stated in oracle/transient.hpp, which cites the reference for every piece.
//
// Precisions:
//   SP_PREC_FP64_EXACT  the oracle's operation sequence (full-step Newton,
//                       divisions, sequential elimination by lane 0); with
//                       the portable transcendentals it is bit-identical to
//                       the oracle in its "cr" mode;
//   SP_PREC_FP64        the same with FMA contraction and one reciprocal per
//                       eliminated row;
//   SP_PREC_MIXED       correction form: FP64 KCL residual of the linearised
//                       stage (diode current linearised at the limited
//                       voltage, as the full-step form), FP32 Jacobian and
//                       FP32 elimination, FP64 update and convergence test.
#pragma once
#include "internal.h"
#include "rng.cuh"
#include "fpconv.cuh"

namespace sp {

// Arrays of one instance in the global workspace, each `stride` doubles.
enum LadderArray {
    LA_G, LA_C, LA_VP, LA_IP, LA_VPP, LA_SVP, LA_SIP, LA_SVPP, LA_X, LA_XS, LA_GEQ, LA_IEQ, LA_COUNT
};

// Shared doubles of one warp's solver scratch: four stride-long arrays of the
// element type (FP32 in the mixed mode) and 64 block unknowns.
__host__ __device__ inline int ladder_warp_doubles(int stride, int prec) {
    return prec == SP_PREC_MIXED ? 2 * stride + 64 : 4 * stride + 64;
}

struct LadderLaunch {
    sp_ladder_config cfg;
    uint64_t seed, first, count;
    const uint32_t* order;  // [count] instance order (largest first)
    unsigned int* next;     // work counter (zero before the launch)
    double* ws;             // [slots][LA_COUNT][stride]
    int stride;             // >= max_sections + 2
    int slots;              // workspace slots (one per resident warp)
    double* x_final;        // [count][max_sections + 2]
    int32_t* n;
    int32_t* accepted;
    int32_t* rejected;
    int32_t* iters;
    uint8_t* status;
    double* probe;          // [count][num_probe] or nullptr
    double* steps;          // [count][max_rec] accepted step sizes, or nullptr
    int max_rec;            // steps recorded per instance (the first max_rec)
};

__host__ __device__ inline int ladder_sections(const sp_ladder_config& c, uint64_t seed, uint32_t inst) {
    const double span = (double)(c.max_sections - c.min_sections + 1);
    return c.min_sections + (int)floor(span * rng_uniform(seed, inst, 0));
}

__host__ __device__ inline double ladder_pulse(const sp_pulse& p, double t) {
    if (t < p.td) return p.v1;
    const double t_rel = p.per > 0.0 ? fmod(t - p.td, p.per) : t - p.td;
    if (t_rel < p.tr) return p.v1 + (p.v2 - p.v1) * t_rel / p.tr;
    if (t_rel < p.tr + p.pw) return p.v2;
    if (t_rel < p.tr + p.pw + p.tf) return p.v2 - (p.v2 - p.v1) * (t_rel - p.tr - p.pw) / p.tf;
    return p.v1;
}

#ifdef SP_KERNEL_NS
namespace SP_KERNEL_NS {

// Warp-parallel solve of the chain's tridiagonal system (rows 1..N, sub-diagonal
// -g_i, super-diagonal -g_{i+1}, diagonal B, right-hand side D; diagonally
// dominant, so no pivoting): the partition method.  The rows are split into P
// contiguous blocks (P = min(32, N/2), one per lane); each lane eliminates
// inside its block downwards and upwards, so that every row i reads
//   L_i x_{lo-1} + B_i x_i + R_i x_{hi} = D_i,
// lane 0 solves the 2P-unknown system of the blocks' first and last rows
// (an affine recurrence over the blocks), and every lane then recovers its
// rows.  On exit D[i] = x_i.  L, R: scratch rows; fl: 2 x 32 scratch values.
template <class T>
__device__ __forceinline__ T from_f64(double v) { return v; }
template <>
__device__ __forceinline__ float from_f64<float>(double v) { return f64_to_f32_int(v); }

template <class T>
__device__ inline void warp_partition_solve(int N, int lane, const double* g, T* B, T* D, T* L, T* R, T* fl) {
    const int P = N / 2 < 32 ? N / 2 : 32;
    int lo = 0, hi = 0;
    if (lane < P) {
        lo = 1 + (int)(((long long)lane * N) / P);
        hi = 1 + (int)(((long long)(lane + 1) * N) / P);
        // downward: move the sub-diagonal into the left spike L
        L[lo] = lo > 1 ? -from_f64<T>(g[lo]) : (T)0;
        for (int i = lo + 1; i < hi; ++i) {
            const T a = -from_f64<T>(g[i]), cprev = -from_f64<T>(g[i]);  // c_{i-1} = -g_i = a_i
            const T f = a / B[i - 1];
            L[i] = -f * L[i - 1];
            B[i] = B[i] - f * cprev;
            D[i] = D[i] - f * D[i - 1];
        }
        // upward: move the super-diagonal into the right spike R
        R[hi - 1] = hi - 1 < N ? -from_f64<T>(g[hi]) : (T)0;
        for (int i = hi - 2; i >= lo; --i) {
            const T cc = -from_f64<T>(g[i + 1]);
            const T f = cc / B[i + 1];
            L[i] = L[i] - f * L[i + 1];
            R[i] = -f * R[i + 1];
            D[i] = D[i] - f * D[i + 1];
        }
    }
    __syncwarp();
    if (lane == 0) {
        // forward over blocks: l_{j-1} = al + be f_j;  f_j = p_j + q_j f_{j+1};  l_j = al_j + be_j f_{j+1}
        T al = 0, be = 0;
        T pq[2 * 32];
        for (int j = 0; j < P; ++j) {
            const int l0 = 1 + (int)(((long long)j * N) / P), h1 = (int)(((long long)(j + 1) * N) / P);  // h1 = hi - 1
            const T den = B[l0] + L[l0] * be;
            const T pj = (D[l0] - L[l0] * al) / den, qj = -R[l0] / den;
            const T nal = (D[h1] - L[h1] * al - L[h1] * be * pj) / B[h1];
            const T nbe = (-L[h1] * be * qj - R[h1]) / B[h1];
            pq[2 * j] = pj;
            pq[2 * j + 1] = qj;
            fl[2 * j] = nbe;  // al_j, be_j kept for the back pass
            fl[2 * j + 1] = nal;
            al = nal;
            be = nbe;
        }
        // backward: f_P = 0
        T fnext = 0;
        for (int j = P - 1; j >= 0; --j) {
            const T fj = pq[2 * j] + pq[2 * j + 1] * fnext;
            const T lj = fl[2 * j + 1] + fl[2 * j] * fnext;
            fl[2 * j] = fj;
            fl[2 * j + 1] = lj;
            fnext = fj;
        }
    }
    __syncwarp();
    if (lane < P) {
        const T xl = lane > 0 ? fl[2 * (lane - 1) + 1] : (T)0;  // last of the previous block
        const T xr = lane + 1 < P ? fl[2 * (lane + 1)] : (T)0;  // first of the next block
        for (int i = lo; i < hi; ++i) D[i] = (D[i] - L[i] * xl - R[i] * xr) / B[i];
    }
    __syncwarp();
}

template <int PREC>
struct LadderWarp {
    const LadderLaunch& L;
    const sp_ladder_config& c;
    double* A[LA_COUNT];
    double* sdiag;  // shared: diag / rhs / c' / d' of the elimination
    double* srhs;
    double* scp;
    double* sdp;
    double* sfl;  // 64 values: the partition solve's block unknowns
    int N, lane;
    double nvt, inv_nvt, vcrit;
    unsigned hard;

    __device__ double limit(double vd) {
        if (vd > vcrit) {
            if (PREC == SP_PREC_FP64_EXACT) {
                const double arg = (vd - vcrit) / nvt;
                return vcrit + nvt * (1.0 + pm_log1p(arg, &hard));
            }
            return vcrit + nvt * (1.0 + log1p((vd - vcrit) * inv_nvt));
        }
        return vd;
    }

    // exp of the diode: the portable correctly rounded one for the exact mode,
    // the device's (shorter dependency chain) otherwise
    __device__ double dexp(double v) {
        if (PREC == SP_PREC_FP64_EXACT) return cr_exp(v / nvt, &hard);
        return exp(v * inv_nvt);
    }

    // One Newton iteration of a stage on xs; writes the new iterate into xs
    // and returns whether every unknown passed the convergence test.
    __device__ bool iterate(double V, bool* finite) {
        double* g = A[LA_G];
        double* xs = A[LA_XS];
        const double* geq = A[LA_GEQ];
        const double* ieq = A[LA_IEQ];
        bool ok = true, fin = true;
        if (PREC != SP_PREC_MIXED) {
            // full-step form: diag and rhs of the linearised stage (oracle order)
            for (int k = 1 + lane; k <= N; k += 32) {
                const double vl1 = limit(xs[k]);
                const double vl2 = limit(vl1);
                const double e = dexp(vl2);
                const double id = c.diode_is * (e - 1.0);
                const double gd = PREC == SP_PREC_FP64_EXACT ? fmax(c.diode_is * e / nvt, 1e-12)
                                                             : fmax(c.diode_is * e * inv_nvt, 1e-12);
                const double ieq_d = id - gd * vl1;
                const double gk1 = k < N ? g[k + 1] : 0.0;
                sdiag[k] = ((g[k] + gk1) + geq[k]) + gd;
                double r = (0.0 + ieq[k]) - ieq_d;
                if (k == 1) r = r - (-g[1]) * V;
                srhs[k] = r;
            }
            __syncwarp();
            if (PREC == SP_PREC_FP64_EXACT && lane == 0) {
                {
                    scp[1] = (N > 1 ? -g[2] : 0.0) / sdiag[1];
                    sdp[1] = srhs[1] / sdiag[1];
                    for (int k = 2; k <= N; ++k) {
                        const double sub = -g[k];
                        const double m = sdiag[k] - sub * scp[k - 1];
                        scp[k] = (k < N ? -g[k + 1] : 0.0) / m;
                        sdp[k] = (srhs[k] - sub * sdp[k - 1]) / m;
                    }
                    // back substitution into srhs (the new iterate of nodes 1..N)
                    srhs[N] = sdp[N];
                    for (int k = N - 1; k >= 1; --k) srhs[k] = sdp[k] - scp[k] * srhs[k + 1];
                }
            }
            if (PREC != SP_PREC_FP64_EXACT) warp_partition_solve<double>(N, lane, g, sdiag, srhs, scp, sdp, sfl);
            __syncwarp();
            for (int k = 1 + lane; k <= N; k += 32) {
                const double nw = srhs[k], old = xs[k];
                const double tol = c.v_reltol * fmax(fabs(nw), fabs(old)) + c.v_abstol;
                ok = ok && fabs(nw - old) <= tol;
                fin = fin && isfinite(nw);
                xs[k] = nw;
            }
        } else {
            // correction form: FP64 residual of the linearised stage, FP32 solve
            float* jd = reinterpret_cast<float*>(sdiag);
            float* jr = reinterpret_cast<float*>(srhs);
            float* jc = reinterpret_cast<float*>(scp);
            float* jp = reinterpret_cast<float*>(sdp);
            // exp(a) = expf(ah) (1 + al), a = ah + al split at FP32 (relative error
            // ~1e-7, far inside the stage tolerances), conductance and Jacobian in
            // FP32, conversions on the integer pipe: the FP64 pipe keeps only the
            // residual (what the refinement needs) and the update
            const float inv_nvt_f = f64_to_f32_int(inv_nvt), is_f = f64_to_f32_int(c.diode_is);
            for (int k = 1 + lane; k <= N; k += 32) {
                const double xk = xs[k];
                const double vl1 = limit(xk);
                const double vl2 = limit(vl1);
                const double a = vl2 * inv_nvt;
                const float ah = f64_to_f32_int(a);
                const float ef = expf(ah);
                const double e = f32_to_f64_int(ef) * (1.0 + (a - f32_to_f64_int(ah)));
                const double id = c.diode_is * (e - 1.0);
                const float gdf = fmaxf(is_f * ef * inv_nvt_f, 1e-12f);
                const double xl = k == 1 ? V : xs[k - 1];
                const double xr = k < N ? xs[k + 1] : 0.0;
                const double gk1 = k < N ? g[k + 1] : 0.0;
                // KCL: currents leaving node k (R left, R right, C companion, diode linearised at vl1)
                const double F = g[k] * (xk - xl) + gk1 * (xk - xr) + (geq[k] * xk - ieq[k]) + (id + f32_to_f64_int(gdf) * (xk - vl1));
                jd[k] = f64_to_f32_int((g[k] + gk1) + geq[k]) + gdf;
                jr[k] = __uint_as_float(__float_as_uint(f64_to_f32_int(F)) ^ 0x80000000u);
            }
            __syncwarp();
            warp_partition_solve<float>(N, lane, g, jd, jr, jc, jp, reinterpret_cast<float*>(sfl));
            const float vrel = f64_to_f32_int(c.v_reltol), vabs = f64_to_f32_int(c.v_abstol);
            for (int k = 1 + lane; k <= N; k += 32) {
                const double old = xs[k];
                const float dy = jr[k];
                const double nw = old + f32_to_f64_int(dy);
                const float nwf = f64_to_f32_int(nw), oldf = f64_to_f32_int(old);
                ok = ok && !(fabsf(dy) > vrel * fmaxf(fabsf(nwf), fabsf(oldf)) + vabs);
                fin = fin && isfinite(nwf);
                xs[k] = nw;
            }
        }
        __syncwarp();
        if (lane == 0) {
            // source node and branch current (KCL of node in)
            const double v0 = xs[0], i0 = xs[N + 1];
            const double inew = -(g[1] * V + (-g[1]) * xs[1]);
            ok = ok && fabs(V - v0) <= c.v_reltol * fmax(fabs(V), fabs(v0)) + c.v_abstol;
            ok = ok && fabs(inew - i0) <= c.v_reltol * fmax(fabs(inew), fabs(i0)) + c.i_abstol;
            fin = fin && isfinite(inew);
            xs[0] = V;
            xs[N + 1] = inew;
        }
        *finite = __all_sync(0xffffffffu, fin);
        return __all_sync(0xffffffffu, ok);
    }

    // Newton solve of a stage from xs: iterations (> 0), -1 on a miss, -2 on NaN/Inf.
    __device__ int newton(double V) {
        for (int it = 1; it <= c.max_iterations; ++it) {
            bool fin;
            const bool ok = iterate(V, &fin);
            if (!fin) return -2;
            if (ok) return it;
        }
        return -1;
    }
};

__device__ inline double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int PREC>
__global__ void __launch_bounds__(128, 2) ladder_kernel(LadderLaunch L) {
    extern __shared__ __align__(16) unsigned char lsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int slot = blockIdx.x * (blockDim.x >> 5) + wib;
    if (slot >= L.slots) return;
    const sp_ladder_config& c = L.cfg;
    const int wd = ladder_warp_doubles(L.stride, PREC);
    double* sm = reinterpret_cast<double*>(lsm) + (size_t)wib * wd;
    LadderWarp<PREC> W{L, c};
    for (int a = 0; a < LA_COUNT; ++a) W.A[a] = L.ws + ((size_t)slot * LA_COUNT + a) * L.stride;
    const int ast = PREC == SP_PREC_MIXED ? L.stride / 2 : L.stride;  // doubles per scratch array
    W.sdiag = sm;
    W.srhs = sm + ast;
    W.scp = sm + 2 * ast;
    W.sdp = sm + 3 * ast;
    W.sfl = sm + 4 * ast;
    W.lane = lane;
    W.hard = 0;
    W.nvt = c.diode_n * thermal_voltage_300();
    W.inv_nvt = 1.0 / W.nvt;
    W.vcrit = W.nvt * cr_log(W.nvt / (1.4142135623730951 * 1e-14), &W.hard);
    const double gamma = 2.0 - 1.4142135623730951;
    const int ldx = c.max_sections + 2;
    while (true) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(L.next, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= L.count) break;
        const uint32_t i = L.order[idx];
        const uint32_t inst = (uint32_t)(L.first + i);
        const int N = ladder_sections(c, L.seed, inst);
        W.N = N;
        double *g = W.A[LA_G], *C = W.A[LA_C], *vp = W.A[LA_VP], *ip = W.A[LA_IP], *vpp = W.A[LA_VPP];
        double *svp = W.A[LA_SVP], *sip = W.A[LA_SIP], *svpp = W.A[LA_SVPP], *x = W.A[LA_X], *xs = W.A[LA_XS];
        double *geq = W.A[LA_GEQ], *ieq = W.A[LA_IEQ];
        // draws (a exp(u ln(b/a)), the log-uniform rule of the parameter draws) and the DC start (all zero)
        const double lr = cr_log(c.r_hi / c.r_lo, &W.hard), lc = cr_log(c.c_hi / c.c_lo, &W.hard);
        for (int k = 1 + lane; k <= N; k += 32) {
            const double R = c.r_lo * cr_exp(rng_uniform(L.seed, inst, 2u * k - 1u) * lr, &W.hard);
            C[k] = c.c_lo * cr_exp(rng_uniform(L.seed, inst, 2u * k) * lc, &W.hard);
            g[k] = 1.0 / R;
            vp[k] = ip[k] = vpp[k] = 0.0;
            x[k] = 0.0;
        }
        if (lane == 0) {
            x[0] = 0.0;
            x[N + 1] = 0.0;
        }
        __syncwarp();
        double t = 0.0, h = c.h_init;
        int accepted = 0, rejected = 0, iterations = 0, steps = 0, next_probe = 0;
        uint8_t status = SP_ST_CONVERGED;
        double* probe = L.probe ? L.probe + (size_t)i * c.num_probe : nullptr;
        const int owner = (N - 1) & 31;  // lane holding node N
        auto record = [&](double t0, double xa, double t1, double xb) {
            while (next_probe < c.num_probe) {
                const double tp = c.num_probe > 1 ? c.tstop * (double)next_probe / (double)(c.num_probe - 1) : 0.0;
                if (tp > t1) break;
                if (probe && lane == owner) probe[next_probe] = t1 > t0 ? xa + (xb - xa) * ((tp - t0) / (t1 - t0)) : xb;
                ++next_probe;
            }
        };
        record(0.0, 0.0, 0.0, 0.0);
        while (t < c.tstop) {
            if (++steps > c.max_steps) {
                status = SP_ST_FAILED;
                break;
            }
            h = fmin(fmax(h, c.h_min), c.h_max);
            if (t + h > c.tstop) h = c.tstop - t;
            const double V = ladder_pulse(c.pulse, t + h);
            const double hg = gamma * h;
            // MIXED: one reciprocal per step instead of a divide per node (GB300's
            // FP64 divide is a long FP64-pipe sequence); the other modes keep the
            // reference's 2 C / (gamma h) per node
            const bool mx = PREC == SP_PREC_MIXED;
            const double r_hg = 2.0 / hg;
            for (int k = 1 + lane; k <= N; k += 32) {
                svp[k] = vp[k];
                sip[k] = ip[k];
                svpp[k] = vpp[k];
                geq[k] = mx ? C[k] * r_hg : 2.0 * C[k] / hg;
                ieq[k] = geq[k] * vp[k] + ip[k];
            }
            for (int k = lane; k <= N + 1; k += 32) xs[k] = x[k];
            __syncwarp();
            const int it1 = W.newton(V);
            int it2 = -1;
            if (it1 > 0) {
                iterations += it1;
                const double h2 = (1.0 - gamma) * h, h1 = gamma * h, rho = h2 / h1;
                const double denom = 1.0 + 2.0 * rho;
                const double a1 = (1.0 + rho) * (1.0 + rho) / denom, a2 = -rho * rho / denom,
                             b0 = (1.0 + rho) / denom;
                const double r_b0h2 = 1.0 / (b0 * h2);
                for (int k = 1 + lane; k <= N; k += 32) {
                    vpp[k] = vp[k];
                    ip[k] = (mx ? C[k] * r_hg : 2.0 * C[k] / hg) * (xs[k] - vpp[k]) - ip[k];
                    vp[k] = xs[k];
                    geq[k] = mx ? C[k] * r_b0h2 : C[k] / (b0 * h2);
                    ieq[k] = geq[k] * (a1 * vp[k] + a2 * vpp[k]);
                }
                __syncwarp();
                it2 = W.newton(V);
                if (it2 > 0) iterations += it2;
            }
            if (it1 == -2 || it2 == -2) {
                status = SP_ST_NONFINITE;
                break;
            }
            if (it1 < 0 || it2 < 0) {
                for (int k = 1 + lane; k <= N; k += 32) {
                    vp[k] = svp[k];
                    ip[k] = sip[k];
                    vpp[k] = svpp[k];
                }
                __syncwarp();
                ++rejected;
                if (h <= c.h_min) {
                    status = SP_ST_FAILED;
                    break;
                }
                h *= 0.25;
                continue;
            }
            double lte = 0.0, ref = 0.0;
            const double r_h = 1.0 / h, r_2h = 2.0 / h;
            for (int k = 1 + lane; k <= N; k += 32) {
                const double v_new = xs[k];
                const double i_trap = (mx ? C[k] * r_2h : 2.0 * C[k] / h) * (v_new - svp[k]) - sip[k];
                const double i_be = (mx ? C[k] * r_h : C[k] / h) * (v_new - svp[k]);
                lte = fmax(lte, mx ? fabs(i_trap - i_be) * (1.0 / 3.0) : fabs(i_trap - i_be) / 3.0);
                ref = fmax(ref, fabs(v_new));
            }
            const double max_lte = warp_max(lte), max_ref = warp_max(ref);
            const double tol = fmax(c.lte_abstol, c.lte_reltol * max_ref);
            if (max_lte > tol && h > c.h_min) {
                for (int k = 1 + lane; k <= N; k += 32) {
                    vp[k] = svp[k];
                    ip[k] = sip[k];
                    vpp[k] = svpp[k];
                }
                __syncwarp();
                ++rejected;
                h *= fmax(fmin(sqrt(tol / max_lte), 0.5), 0.1);
                continue;
            }
            const double xa = __shfl_sync(0xffffffffu, x[N], owner), xb = __shfl_sync(0xffffffffu, xs[N], owner);
            for (int k = 1 + lane; k <= N; k += 32) {
                ip[k] = geq[k] * xs[k] - ieq[k];
                vpp[k] = vp[k];
                vp[k] = xs[k];
            }
            for (int k = lane; k <= N + 1; k += 32) x[k] = xs[k];
            __syncwarp();
            record(t, xa, t + h, xb);
            if (L.steps && lane == 0 && accepted < L.max_rec) L.steps[(size_t)i * L.max_rec + accepted] = h;
            t += h;
            ++accepted;
            if (max_lte < tol * 0.5 && h < c.h_max) h *= fmin(fmin(sqrt(tol / fmax(max_lte, 1e-20)), 2.0), 1.5);
        }
        const double xN = __shfl_sync(0xffffffffu, x[N], owner);
        while (next_probe < c.num_probe) {
            if (probe && lane == owner) probe[next_probe] = xN;
            ++next_probe;
        }
        double* xf = L.x_final + (size_t)i * ldx;
        for (int k = lane; k < ldx; k += 32) xf[k] = k <= N + 1 ? x[k] : 0.0;
        if (lane == 0) {
            L.n[i] = N + 2;
            L.accepted[i] = accepted;
            L.rejected[i] = rejected;
            L.iters[i] = iterations;
            L.status[i] = status;
        }
        __syncwarp();
    }
}

}  // namespace SP_KERNEL_NS
#endif  // SP_KERNEL_NS

}  // namespace sp
