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

namespace sp {

// Arrays of one instance in the global workspace, each `stride` doubles.
enum LadderArray {
    LA_G, LA_C, LA_VP, LA_IP, LA_VPP, LA_SVP, LA_SIP, LA_SVPP, LA_X, LA_XS, LA_GEQ, LA_IEQ, LA_COUNT
};

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

template <int PREC>
struct LadderWarp {
    const LadderLaunch& L;
    const sp_ladder_config& c;
    double* A[LA_COUNT];
    double* sdiag;  // shared: diag / rhs / c' / d' of the elimination
    double* srhs;
    double* scp;
    double* sdp;
    int N, lane;
    double nvt, vcrit;
    unsigned hard;

    __device__ double limit(double vd) {
        if (vd > vcrit) {
            const double arg = (vd - vcrit) / nvt;
            return vcrit + nvt * (1.0 + pm_log1p(arg, &hard));
        }
        return vd;
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
                const double e = cr_exp(vl2 / nvt, &hard);
                const double id = c.diode_is * (e - 1.0);
                const double gd = fmax(c.diode_is * e / nvt, 1e-12);
                const double ieq_d = id - gd * vl1;
                const double gk1 = k < N ? g[k + 1] : 0.0;
                sdiag[k] = ((g[k] + gk1) + geq[k]) + gd;
                double r = (0.0 + ieq[k]) - ieq_d;
                if (k == 1) r = r - (-g[1]) * V;
                srhs[k] = r;
            }
            __syncwarp();
            if (lane == 0) {
                if (PREC == SP_PREC_FP64_EXACT) {
                    scp[1] = (N > 1 ? -g[2] : 0.0) / sdiag[1];
                    sdp[1] = srhs[1] / sdiag[1];
                    for (int k = 2; k <= N; ++k) {
                        const double sub = -g[k];
                        const double m = sdiag[k] - sub * scp[k - 1];
                        scp[k] = (k < N ? -g[k + 1] : 0.0) / m;
                        sdp[k] = (srhs[k] - sub * sdp[k - 1]) / m;
                    }
                } else {
                    double r = 1.0 / sdiag[1];
                    scp[1] = (N > 1 ? -g[2] : 0.0) * r;
                    sdp[1] = srhs[1] * r;
                    for (int k = 2; k <= N; ++k) {
                        const double sub = -g[k];
                        r = 1.0 / (sdiag[k] - sub * scp[k - 1]);
                        scp[k] = (k < N ? -g[k + 1] : 0.0) * r;
                        sdp[k] = (srhs[k] - sub * sdp[k - 1]) * r;
                    }
                }
                // back substitution into srhs (the new iterate of nodes 1..N)
                srhs[N] = sdp[N];
                for (int k = N - 1; k >= 1; --k) srhs[k] = sdp[k] - scp[k] * srhs[k + 1];
            }
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
            for (int k = 1 + lane; k <= N; k += 32) {
                const double xk = xs[k];
                const double vl1 = limit(xk);
                const double vl2 = limit(vl1);
                const double e = cr_exp(vl2 / nvt, &hard);
                const double id = c.diode_is * (e - 1.0);
                const double gd = fmax(c.diode_is * e / nvt, 1e-12);
                const double xl = k == 1 ? V : xs[k - 1];
                const double xr = k < N ? xs[k + 1] : 0.0;
                const double gk1 = k < N ? g[k + 1] : 0.0;
                // KCL: currents leaving node k (R left, R right, C companion, diode linearised at vl1)
                const double F = g[k] * (xk - xl) + gk1 * (xk - xr) + (geq[k] * xk - ieq[k]) + (id + gd * (xk - vl1));
                jd[k] = (float)(((g[k] + gk1) + geq[k]) + gd);
                jr[k] = (float)(-F);
            }
            __syncwarp();
            if (lane == 0) {
                float r = 1.0f / jd[1];
                jc[1] = (N > 1 ? -(float)g[2] : 0.0f) * r;
                jp[1] = jr[1] * r;
                for (int k = 2; k <= N; ++k) {
                    const float sub = -(float)g[k];
                    r = 1.0f / (jd[k] - sub * jc[k - 1]);
                    jc[k] = (k < N ? -(float)g[k + 1] : 0.0f) * r;
                    jp[k] = (jr[k] - sub * jp[k - 1]) * r;
                }
                jr[N] = jp[N];
                for (int k = N - 1; k >= 1; --k) jr[k] = jp[k] - jc[k] * jr[k + 1];
            }
            __syncwarp();
            for (int k = 1 + lane; k <= N; k += 32) {
                const double old = xs[k];
                const double nw = old + (double)jr[k];
                const double tol = c.v_reltol * fmax(fabs(nw), fabs(old)) + c.v_abstol;
                ok = ok && fabs(nw - old) <= tol;
                fin = fin && isfinite(nw);
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
    double* sm = reinterpret_cast<double*>(lsm) + (size_t)wib * 4 * L.stride;
    LadderWarp<PREC> W{L, c};
    for (int a = 0; a < LA_COUNT; ++a) W.A[a] = L.ws + ((size_t)slot * LA_COUNT + a) * L.stride;
    W.sdiag = sm;
    W.srhs = sm + L.stride;
    W.scp = sm + 2 * L.stride;
    W.sdp = sm + 3 * L.stride;
    W.lane = lane;
    W.hard = 0;
    W.nvt = c.diode_n * thermal_voltage_300();
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
            for (int k = 1 + lane; k <= N; k += 32) {
                svp[k] = vp[k];
                sip[k] = ip[k];
                svpp[k] = vpp[k];
                geq[k] = 2.0 * C[k] / hg;
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
                for (int k = 1 + lane; k <= N; k += 32) {
                    vpp[k] = vp[k];
                    ip[k] = 2.0 * C[k] / hg * (xs[k] - vpp[k]) - ip[k];
                    vp[k] = xs[k];
                    geq[k] = C[k] / (b0 * h2);
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
            for (int k = 1 + lane; k <= N; k += 32) {
                const double v_new = xs[k];
                const double i_trap = 2.0 * C[k] / h * (v_new - svp[k]) - sip[k];
                const double i_be = C[k] / h * (v_new - svp[k]);
                lte = fmax(lte, fabs(i_trap - i_be) / 3.0);
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
