// Batched AC small-signal sweep: one thread per (sample, frequency).
//
// From each sample's DC operating point (the Newton path's output), the
// devices' small-signal conductances (ac_info_at: diode.rs:202-220,
// mosfet/level1.rs:307-331, bjt.rs:404-427) and the reactive terms at
// w = 2 pi f are stamped into a complex MNA matrix exactly as the netlist AC
// stamper does (crates/spicier-cli/src/stampers.rs:94-330, ComplexMna in
// crates/spicier-solver/src/ac.rs:121-240), then solved by the dense complex
// LU of solve_complex (nalgebra LU on num_complex numbers, linear.rs:557-583):
// pivot = first maximum of |re| + |im| in the column, num_complex's operation
// order for products and quotients.  In the exact build (no FMA contraction)
// the result is the oracle's bit for bit wherever the DC point is.
//
// Real contributions accumulate in element order, then the imaginary ones
// (capacitors, inductors) in element order: each component's sum has the
// order of the reference's triplet sum.  The matrix and right-hand side live
// interleaved per thread ([element][thread]) in shared memory, or in a global
// work buffer with the same layout when n is too large for shared memory.
#pragma once
#include "circuit_dev.cuh"
#include "internal.h"

namespace sp {

struct AcLaunch {
    DevCircuit c;
    const double* params;  // [count][np] the DC pass's drawn parameters
    int np;
    const double* x_dc;     // [count][n]
    const uint8_t* dc_status;
    uint64_t count;
    const double* freqs;    // [nf]
    int nf;
    int source;             // -1: every V source at magnitude 1; else the element index of the stimulus
    int num_probe;
    int probe[8];
    double* out;            // [count][nf][num_probe][2]
    unsigned int* singular; // [count] set when a frequency's matrix was singular
    double* work;           // global interleaved work area, or nullptr (shared memory)
    int refine;             // mixed kernel: FP64 residual refinement steps
    SoA dv;                 // the DC pass's per-sample derived constants (BSIM3 elements)
};

// BSIM3 small-signal values at the operating point x (ac_info_at,
// mosfet/bsim3/mod.rs:296-342): g = gds, gm, gmbs, then cgs, cgd, cgb, cbs, cbd.
__device__ inline void bsim3_ac_values(const AcLaunch& L, uint64_t s, int e, const sp_element& el, const double* P,
                                       const double* x, double* g) {
    auto V = [&](int i) { return i >= 0 ? x[i] : 0.0; };
    const int off = L.c.doff[e];
    const auto K = [&](int i) { return L.dv(off + i, s); };
    const auto C = [&](int k) { return P[el.field[0] + k]; };
    const bool pm = el.kind == SP_EL_BSIM3P;
    const double vs = V(el.node[2]);
    const double vgs = V(el.node[1]) - vs, vds = V(el.node[0]) - vs, vbs = V(el.node[3]) - vs;
    const Bsim3Out r = bsim3_eval(pm, K, vgs, vds, vbs);
    g[0] = r.gds, g[1] = r.gm, g[2] = r.gmbs;
    bsim3_caps(pm, K, C, vds, vbs, r.region, g + 3);
}

// Per-thread work bytes: exact kernel (FP64 complex matrix + rhs), mixed
// kernel (FP32 complex matrix + rhs, FP64 x and residual).
__host__ __device__ inline size_t ac_work_bytes(int n, bool mixed) {
    return mixed ? (size_t)8 * ((size_t)n * n + n) + (size_t)32 * n : (size_t)16 * ((size_t)n * n + n);
}

#if defined(SP_AC_KERNELS) || defined(SP_AC_MIXED_KERNELS)
// bjt.rs:176-259 evaluate at (vbe, vce): o[3..5] = gm, gpi, go (floored at 1e-12).
__device__ inline void bjt_eval_ac(bool pnp, double is, double bf, double br, double nf_vt, double nr_vt, double vaf,
                                   double vbe, double vce, double o[6]) {
    if (pnp) {
        vbe = -vbe;
        vce = -vce;
    }
    const double vbc = vbe - vce;
    const double vbe_l = limit_voltage(vbe, nf_vt, diode_vcrit(nf_vt));
    const double vbc_l = limit_voltage(vbc, nr_vt, diode_vcrit(nr_vt));
    const double exp_be = exp(vbe_l / nf_vt), exp_bc = exp(vbc_l / nr_vt);
    const double i_f = is * (exp_be - 1.0), i_r = is * (exp_bc - 1.0);
    const bool vfin = isfinite(vaf) && vaf > 0.0;
    const double early = (vfin && vce > 0.0) ? 1.0 + vce / vaf : 1.0;
    const double ic = (i_f - i_r / br) * early;
    const double gm = (i_f > 1e-20) ? (is * exp_be / nf_vt) * early : 1e-12;
    const double gpi = gm / bf;
    const double go_early = (vfin && fabs(ic) > 1e-20) ? fabs(ic) / vaf : 0.0;
    const double go = fmax(go_early + is * exp_bc / nr_vt / br * early, 1e-12);
    o[3] = fmax(gm, 1e-12);
    o[4] = fmax(gpi, 1e-12);
    o[5] = fmax(go, 1e-12);
}

#endif

#ifdef SP_AC_KERNELS  // the kernels: only in the translation unit that builds them (no FMA contraction)
// complex number stored at p[0], p[stride] (re, im) of an interleaved array
struct CxRef {
    double* p;
    int64_t stride;
    __device__ double& re() const { return p[0]; }
    __device__ double& im() const { return p[stride]; }
};

struct CxArr {
    double* base;
    int64_t stride;  // distance between consecutive doubles of one thread
    __device__ CxRef operator[](int k) const { return CxRef{base + (int64_t)(2 * k) * stride, stride}; }
};

__device__ inline void ac_add_re(CxArr A, int n, int r, int c, double v) {
    if (r >= 0 && c >= 0) A[c * n + r].re() += v;
}
__device__ inline void ac_add_im(CxArr A, int n, int r, int c, double v) {
    if (r >= 0 && c >= 0) A[c * n + r].im() += v;
}

// nalgebra LU + solve on the interleaved complex matrix (column-major), b -> x.
__device__ inline bool ac_lu_solve(int n, CxArr A, CxArr b, int8_t* swap_with) {
    for (int i = 0; i < n; ++i) {
        int piv = i;
        double best = fabs(A[i * n + i].re()) + fabs(A[i * n + i].im());
        for (int r = i + 1; r < n; ++r) {
            const double v = fabs(A[i * n + r].re()) + fabs(A[i * n + r].im());
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        swap_with[i] = -1;
        const double dre = A[i * n + piv].re(), dim = A[i * n + piv].im();
        if (dre == 0.0 && dim == 0.0) continue;
        if (piv != i) {
            swap_with[i] = (int8_t)piv;
            for (int c = 0; c < n; ++c) {
                const double tr = A[c * n + i].re(), ti = A[c * n + i].im();
                A[c * n + i].re() = A[c * n + piv].re();
                A[c * n + i].im() = A[c * n + piv].im();
                A[c * n + piv].re() = tr;
                A[c * n + piv].im() = ti;
            }
        }
        // inv = 1 / diag (num_complex: (1 re + 0 im) / d)
        const double ns = dre * dre + dim * dim;
        const double ire = (1.0 * dre + 0.0 * dim) / ns, iim = (0.0 * dre - 1.0 * dim) / ns;
        for (int r = i + 1; r < n; ++r) {
            const double ar = A[i * n + r].re(), ai = A[i * n + r].im();
            A[i * n + r].re() = ar * ire - ai * iim;
            A[i * n + r].im() = ar * iim + ai * ire;
        }
        for (int c = i + 1; c < n; ++c) {
            const double pr = -A[c * n + i].re(), pi = -A[c * n + i].im();
            for (int r = i + 1; r < n; ++r) {
                const double ar = A[i * n + r].re(), ai = A[i * n + r].im();
                const double mr = pr * ar - pi * ai, mi = pr * ai + pi * ar;
                A[c * n + r].re() = mr + A[c * n + r].re();
                A[c * n + r].im() = mi + A[c * n + r].im();
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        const int p = swap_with[i];
        if (p >= 0) {
            const double tr = b[i].re(), ti = b[i].im();
            b[i].re() = b[p].re();
            b[i].im() = b[p].im();
            b[p].re() = tr;
            b[p].im() = ti;
        }
    }
    for (int i = 0; i < n; ++i) {
        const double cr = -b[i].re(), ci = -b[i].im();
        for (int r = i + 1; r < n; ++r) {
            const double ar = A[i * n + r].re(), ai = A[i * n + r].im();
            const double mr = cr * ar - ci * ai, mi = cr * ai + ci * ar;
            b[r].re() = mr + b[r].re();
            b[r].im() = mi + b[r].im();
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        const double dr = A[i * n + i].re(), di = A[i * n + i].im();
        if (dr == 0.0 && di == 0.0) return false;
        const double ns = dr * dr + di * di;
        const double br = b[i].re(), bi = b[i].im();
        const double qr = (br * dr + bi * di) / ns, qi = (bi * dr - br * di) / ns;
        b[i].re() = qr;
        b[i].im() = qi;
        const double cr = -qr, ci = -qi;
        for (int r = 0; r < i; ++r) {
            const double ar = A[i * n + r].re(), ai = A[i * n + r].im();
            const double mr = cr * ar - ci * ai, mi = cr * ai + ci * ar;
            b[r].re() = mr + b[r].re();
            b[r].im() = mi + b[r].im();
        }
    }
    return true;
}

// One (sample, frequency) unit u = s * nf + f with the work area A.
__device__ inline void ac_unit(const AcLaunch& L, uint64_t u, CxArr A) {
    const uint64_t s = u / (uint64_t)L.nf;
    const int f = (int)(u % (uint64_t)L.nf);
    const DevCircuit& c = L.c;
    const int n = c.n, nn = c.num_nodes;
    double* out = L.out + (u * (uint64_t)L.num_probe) * 2;
    if ((L.dc_status[s] & SP_ST_MASK) != SP_ST_CONVERGED) {
        for (int k = 0; k < 2 * L.num_probe; ++k) out[k] = CUDART_NAN;
        return;
    }
    const CxArr b{A.base + (int64_t)(2 * n * n) * A.stride, A.stride};
    for (int k = 0; k < n * n; ++k) A[k].re() = 0.0, A[k].im() = 0.0;
    for (int k = 0; k < n; ++k) b[k].re() = 0.0, b[k].im() = 0.0;
    const double* P = L.params + s * (uint64_t)L.np;
    const double* x = L.x_dc + s * (uint64_t)n;
    auto V = [&](int i) { return i >= 0 ? x[i] : 0.0; };
    auto cond = [&](int i, int j, double g) {
        ac_add_re(A, n, i, i, g), ac_add_re(A, n, j, j, g), ac_add_re(A, n, i, j, -g), ac_add_re(A, n, j, i, -g);
    };
    auto vccs = [&](int op, int on, int cp, int cn, double gm) {
        ac_add_re(A, n, op, cp, gm), ac_add_re(A, n, op, cn, -gm), ac_add_re(A, n, on, cp, -gm),
            ac_add_re(A, n, on, cn, gm);
    };
    const double vt = thermal_voltage_300();
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element el = c.el[e];
        const int a0 = el.node[0], a1 = el.node[1], a2 = el.node[2];
        switch (el.kind) {
            case SP_EL_R: cond(a0, a1, 1.0 / P[el.field[0]]); break;
            case SP_EL_V:
            case SP_EL_L: {
                const int br = nn + el.branch;
                ac_add_re(A, n, a0, br, 1.0), ac_add_re(A, n, br, a0, 1.0);
                ac_add_re(A, n, a1, br, -1.0), ac_add_re(A, n, br, a1, -1.0);
                if (el.kind == SP_EL_V && (L.source < 0 || L.source == e)) b[br].re() += 1.0;
                break;
            }
            case SP_EL_D: {  // diode.rs evaluate at vd (it limits once)
                const double nvt = P[el.field[1]] * vt;
                const double vd = V(a0) - V(a1);
                const double vl = limit_voltage(vd, nvt, diode_vcrit(nvt));
                const double g = P[el.field[0]] * exp(vl / nvt) / nvt;
                cond(a0, a1, fmax(g, 1e-12));
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS: {
                const double kp = P[el.field[1]], w = P[el.field[3]], l = P[el.field[4]], nf = P[el.field[5]];
                double ids, gds, gm;
                mos_eval(el.kind == SP_EL_PMOS, fabs(P[el.field[0]]), kp * nf * w / l, P[el.field[2]],
                         V(a1) - V(a2), V(a0) - V(a2), ids, gds, gm);
                cond(a0, a2, gds);
                vccs(a0, a2, a1, a2, gm);
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {
                double o[6];
                bjt_eval_ac(el.kind == SP_EL_PNP, P[el.field[0]], P[el.field[1]], P[el.field[2]],
                            P[el.field[3]] * vt, P[el.field[4]] * vt, P[el.field[5]], V(a1) - V(a2),
                            V(a0) - V(a2), o);
                cond(a1, a2, o[4]);
                cond(a0, a2, o[5]);
                vccs(a0, a2, a1, a2, o[3]);
                break;
            }
            case SP_EL_BSIM3N:
            case SP_EL_BSIM3P: {  // stampers.rs:423-470: gds, gm and gmbs VCCSs (capacitances below)
                double g[8];
                bsim3_ac_values(L, s, e, el, P, x, g);
                cond(a0, a2, g[0]);
                vccs(a0, a2, a1, a2, g[1]);
                vccs(a0, a2, el.node[3], a2, g[2]);
                break;
            }
            default:
                break;
        }
    }
    const double wv = 2.0 * 3.141592653589793 * L.freqs[f];
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element el = c.el[e];
        if (el.kind == SP_EL_C) {
            const double y = wv * P[el.field[0]];
            const int i = el.node[0], j = el.node[1];
            ac_add_im(A, n, i, i, y), ac_add_im(A, n, j, j, y), ac_add_im(A, n, i, j, -y), ac_add_im(A, n, j, i, -y);
        } else if (el.kind == SP_EL_L) {
            const int br = nn + el.branch;
            A[br * n + br].im() -= wv * P[el.field[0]];
        } else if (el.kind == SP_EL_BSIM3N || el.kind == SP_EL_BSIM3P) {
            double g[8];
            bsim3_ac_values(L, s, e, el, P, x, g);
            const int d = el.node[0], gt = el.node[1], so = el.node[2], b = el.node[3];
            const int pr[5][2] = {{gt, so}, {gt, d}, {gt, b}, {b, so}, {b, d}};
            for (int k = 0; k < 5; ++k) {
                if (!(g[3 + k] > 0.0)) continue;
                const double y = wv * g[3 + k];
                const int i = pr[k][0], j = pr[k][1];
                ac_add_im(A, n, i, i, y), ac_add_im(A, n, j, j, y), ac_add_im(A, n, i, j, -y), ac_add_im(A, n, j, i, -y);
            }
        }
    }
    int8_t swap_with[64];
    const bool ok = ac_lu_solve(n, A, b, swap_with);
    if (!ok) atomicOr(L.singular + s, 1u);
    for (int k = 0; k < L.num_probe; ++k) {
        out[2 * k] = ok ? b[L.probe[k]].re() : CUDART_NAN;
        out[2 * k + 1] = ok ? b[L.probe[k]].im() : CUDART_NAN;
    }
}

// Grid-stride over the units; thread t's work area is column t of the
// interleaved shared (blockDim threads) or global (gridDim * blockDim) array.
__global__ void __launch_bounds__(128) ac_kernel(AcLaunch L) {
    extern __shared__ __align__(16) unsigned char ac_smem[];
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
    const CxArr A = L.work ? CxArr{L.work + t, (int64_t)nthreads}
                           : CxArr{reinterpret_cast<double*>(ac_smem) + threadIdx.x, (int64_t)blockDim.x};
    const uint64_t total = L.count * (uint64_t)L.nf;
    for (uint64_t u = t; u < total; u += nthreads) ac_unit(L, u, A);
}

__global__ void ac_status_kernel(uint64_t count, const uint8_t* dc_status, const unsigned int* singular,
                                 uint8_t* status) {
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    const uint8_t st = dc_status[s];
    status[s] = singular[s] ? (uint8_t)((st & ~SP_ST_MASK) | SP_ST_SINGULAR) : st;
}

#endif  // SP_AC_KERNELS


#ifdef SP_AC_MIXED_KERNELS  // built in the translation unit with FMA contraction
// Mixed-precision AC: the complex matrix in FP32 (factorised once per
// frequency, same pivoting rule), the solution in FP64 refined `refine` times
// with the residual b - A x evaluated element by element in FP64 from the
// small-signal values (which the FP64 path stamps into its matrix).  The
// FP64 pipe sees only the residuals and updates (~20 n per step) instead of
// the 8 n^3 / 3 of the FP64 factorisation.
struct CxfArr {
    float* base;
    int64_t stride;  // distance between consecutive floats of one thread
    __device__ float& re(int k) const { return base[(int64_t)(2 * k) * stride]; }
    __device__ float& im(int k) const { return base[(int64_t)(2 * k + 1) * stride]; }
};
struct DvArr {
    double* base;
    int64_t stride;
    __device__ double& re(int k) const { return base[(int64_t)(2 * k) * stride]; }
    __device__ double& im(int k) const { return base[(int64_t)(2 * k + 1) * stride]; }
};

// small-signal element values at the operating point: one visit per element
// (the same evaluation the FP64 path stamps), through the callback
template <class F>
__device__ inline void ac_elements(const AcLaunch& L, uint64_t s, F visit) {
    const DevCircuit& c = L.c;
    const double* P = L.params + s * (uint64_t)L.np;
    const double* x = L.x_dc + s * (uint64_t)c.n;
    auto V = [&](int i) { return i >= 0 ? x[i] : 0.0; };
    const double vt = thermal_voltage_300();
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element el = c.el[e];
        const int a0 = el.node[0], a1 = el.node[1], a2 = el.node[2];
        double g[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        double& g0 = g[0];
        double& g1 = g[1];
        double& g2 = g[2];
        switch (el.kind) {
            case SP_EL_R: g0 = 1.0 / P[el.field[0]]; break;
            case SP_EL_C:
            case SP_EL_L: g0 = P[el.field[0]]; break;
            case SP_EL_D: {
                const double nvt = P[el.field[1]] * vt;
                const double vl = limit_voltage(V(a0) - V(a1), nvt, diode_vcrit(nvt));
                g0 = fmax(P[el.field[0]] * exp(vl / nvt) / nvt, 1e-12);
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS: {
                const double kp = P[el.field[1]], w = P[el.field[3]], l = P[el.field[4]], nf = P[el.field[5]];
                double ids;
                mos_eval(el.kind == SP_EL_PMOS, fabs(P[el.field[0]]), kp * nf * w / l, P[el.field[2]], V(a1) - V(a2),
                         V(a0) - V(a2), ids, g0, g1);  // g0 = gds, g1 = gm
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {
                double o[6];
                bjt_eval_ac(el.kind == SP_EL_PNP, P[el.field[0]], P[el.field[1]], P[el.field[2]], P[el.field[3]] * vt,
                            P[el.field[4]] * vt, P[el.field[5]], V(a1) - V(a2), V(a0) - V(a2), o);
                g0 = o[4], g1 = o[5], g2 = o[3];  // gpi, go, gm
                break;
            }
            case SP_EL_BSIM3N:
            case SP_EL_BSIM3P: bsim3_ac_values(L, s, e, el, P, x, g); break;  // gds gm gmbs cgs cgd cgb cbs cbd
            default:
                break;
        }
        visit(el, e, (const double*)g);
    }
}

__device__ inline void ac_mixed_unit(const AcLaunch& L, uint64_t u, float* fbase, double* dbase, int64_t stride) {
    const uint64_t s = u / (uint64_t)L.nf;
    const int f = (int)(u % (uint64_t)L.nf);
    const DevCircuit& c = L.c;
    const int n = c.n, nn = c.num_nodes;
    double* out = L.out + (u * (uint64_t)L.num_probe) * 2;
    if ((L.dc_status[s] & SP_ST_MASK) != SP_ST_CONVERGED) {
        for (int k = 0; k < 2 * L.num_probe; ++k) out[k] = CUDART_NAN;
        return;
    }
    const CxfArr A{fbase, stride}, bf{fbase + (int64_t)(2 * n * n) * stride, stride};
    const DvArr x{dbase, stride}, r{dbase + (int64_t)(2 * n) * stride, stride};
    const double wv = 2.0 * 3.141592653589793 * L.freqs[f];
    // FP32 matrix
    for (int k = 0; k < n * n; ++k) A.re(k) = 0.f, A.im(k) = 0.f;
    auto are = [&](int i, int j, float v) {
        if (i >= 0 && j >= 0) A.re(j * n + i) += v;
    };
    auto aim = [&](int i, int j, float v) {
        if (i >= 0 && j >= 0) A.im(j * n + i) += v;
    };
    ac_elements(L, s, [&](const sp_element& el, int, const double* g) {
        const double g0 = g[0], g1 = g[1], g2 = g[2];
        const int a0 = el.node[0], a1 = el.node[1], a2 = el.node[2];
        switch (el.kind) {
            case SP_EL_R:
            case SP_EL_D: {
                const float g = (float)g0;
                are(a0, a0, g), are(a1, a1, g), are(a0, a1, -g), are(a1, a0, -g);
                break;
            }
            case SP_EL_C: {
                const float y = (float)(wv * g0);
                aim(a0, a0, y), aim(a1, a1, y), aim(a0, a1, -y), aim(a1, a0, -y);
                break;
            }
            case SP_EL_V:
            case SP_EL_L: {
                const int br = nn + el.branch;
                are(a0, br, 1.f), are(br, a0, 1.f), are(a1, br, -1.f), are(br, a1, -1.f);
                if (el.kind == SP_EL_L) aim(br, br, (float)(-wv * g0));
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS: {  // d = a0, g = a1, s = a2: gds (d, s), gm VCCS d <- (g, s)
                const float gd = (float)g0, gm = (float)g1;
                are(a0, a0, gd), are(a2, a2, gd), are(a0, a2, -gd), are(a2, a0, -gd);
                are(a0, a1, gm), are(a0, a2, -gm), are(a2, a1, -gm), are(a2, a2, gm);
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {  // c = a0, b = a1, e = a2
                const float gp = (float)g0, go = (float)g1, gm = (float)g2;
                are(a1, a1, gp), are(a2, a2, gp), are(a1, a2, -gp), are(a2, a1, -gp);
                are(a0, a0, go), are(a2, a2, go), are(a0, a2, -go), are(a2, a0, -go);
                are(a0, a1, gm), are(a0, a2, -gm), are(a2, a1, -gm), are(a2, a2, gm);
                break;
            }
            case SP_EL_BSIM3N:
            case SP_EL_BSIM3P: {  // d = a0, g = a1, s = a2, b = node[3]
                const int a3 = el.node[3];
                const float gd = (float)g0, gm = (float)g1, gb = (float)g2;
                are(a0, a0, gd), are(a2, a2, gd), are(a0, a2, -gd), are(a2, a0, -gd);
                are(a0, a1, gm), are(a0, a2, -gm), are(a2, a1, -gm), are(a2, a2, gm);
                are(a0, a3, gb), are(a0, a2, -gb), are(a2, a3, -gb), are(a2, a2, gb);
                const int pr[5][2] = {{a1, a2}, {a1, a0}, {a1, a3}, {a3, a2}, {a3, a0}};
                for (int k = 0; k < 5; ++k) {
                    if (!(g[3 + k] > 0.0)) continue;
                    const float y = (float)(wv * g[3 + k]);
                    const int i = pr[k][0], j = pr[k][1];
                    aim(i, i, y), aim(j, j, y), aim(i, j, -y), aim(j, i, -y);
                }
                break;
            }
            default:
                break;
        }
    });
    // FP32 LU, pivot = first maximum of |re| + |im|
    int8_t piv_of[64];
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
        int piv = i;
        float best = fabsf(A.re(i * n + i)) + fabsf(A.im(i * n + i));
        for (int q = i + 1; q < n; ++q) {
            const float v = fabsf(A.re(i * n + q)) + fabsf(A.im(i * n + q));
            if (v > best) best = v, piv = q;
        }
        piv_of[i] = (int8_t)piv;
        const float dr = A.re(i * n + piv), di = A.im(i * n + piv);
        if (!(fabsf(dr) + fabsf(di) > 0.f)) {
            ok = false;
            break;
        }
        if (piv != i)
            for (int cc = 0; cc < n; ++cc) {
                const float tr = A.re(cc * n + i), ti = A.im(cc * n + i);
                A.re(cc * n + i) = A.re(cc * n + piv), A.im(cc * n + i) = A.im(cc * n + piv);
                A.re(cc * n + piv) = tr, A.im(cc * n + piv) = ti;
            }
        const float ns = dr * dr + di * di, ir = dr / ns, ii = -di / ns;
        for (int q = i + 1; q < n; ++q) {
            const float ar = A.re(i * n + q), ai = A.im(i * n + q);
            A.re(i * n + q) = ar * ir - ai * ii;
            A.im(i * n + q) = ar * ii + ai * ir;
        }
        for (int cc = i + 1; cc < n; ++cc) {
            const float pr = A.re(cc * n + i), pi = A.im(cc * n + i);
            for (int q = i + 1; q < n; ++q) {
                const float ar = A.re(i * n + q), ai = A.im(i * n + q);
                A.re(cc * n + q) -= pr * ar - pi * ai;
                A.im(cc * n + q) -= pr * ai + pi * ar;
            }
        }
    }
    // forward / back substitution of the FP32 right-hand side in bf
    auto lu_solve32 = [&]() {
        for (int i = 0; i < n; ++i) {
            const int p = piv_of[i];
            if (p != i) {
                const float tr = bf.re(i), ti = bf.im(i);
                bf.re(i) = bf.re(p), bf.im(i) = bf.im(p);
                bf.re(p) = tr, bf.im(p) = ti;
            }
        }
        for (int i = 0; i < n; ++i) {
            const float cr = bf.re(i), ci = bf.im(i);
            for (int q = i + 1; q < n; ++q) {
                const float ar = A.re(i * n + q), ai = A.im(i * n + q);
                bf.re(q) -= cr * ar - ci * ai;
                bf.im(q) -= cr * ai + ci * ar;
            }
        }
        for (int i = n - 1; i >= 0; --i) {
            const float dr = A.re(i * n + i), di = A.im(i * n + i), ns = dr * dr + di * di;
            const float br = bf.re(i), bi = bf.im(i);
            const float qr = (br * dr + bi * di) / ns, qi = (bi * dr - br * di) / ns;
            bf.re(i) = qr, bf.im(i) = qi;
            for (int q = 0; q < i; ++q) {
                const float ar = A.re(i * n + q), ai = A.im(i * n + q);
                bf.re(q) -= qr * ar - qi * ai;
                bf.im(q) -= qr * ai + qi * ar;
            }
        }
    };
    // right-hand side (V sources' AC magnitudes on their branch rows)
    auto rhs = [&](int i) -> double {
        int k = -1;
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            if (el.kind == SP_EL_V && nn + el.branch == i && (L.source < 0 || L.source == e)) k = e;
        }
        return k >= 0 ? 1.0 : 0.0;
    };
    if (ok) {
        for (int i = 0; i < n; ++i) {
            x.re(i) = 0.0, x.im(i) = 0.0;
            r.re(i) = rhs(i), r.im(i) = 0.0;
        }
        for (int step = 0; step <= L.refine; ++step) {
            // scale the residual into FP32 range, solve, accumulate in FP64
            double m = 0.0;
            for (int i = 0; i < n; ++i) m = fmax(m, fmax(fabs(r.re(i)), fabs(r.im(i))));
            if (!(m > 0.0)) break;
            const double sc = 1.0 / m;
            for (int i = 0; i < n; ++i) bf.re(i) = (float)(r.re(i) * sc), bf.im(i) = (float)(r.im(i) * sc);
            lu_solve32();
            for (int i = 0; i < n; ++i) x.re(i) += (double)bf.re(i) * m, x.im(i) += (double)bf.im(i) * m;
            if (step == L.refine) break;
            // r = b - A x in FP64, element by element
            for (int i = 0; i < n; ++i) r.re(i) = rhs(i), r.im(i) = 0.0;
            auto xr = [&](int i) { return i >= 0 ? x.re(i) : 0.0; };
            auto xi = [&](int i) { return i >= 0 ? x.im(i) : 0.0; };
            auto sub = [&](int i, double vr, double vi) {
                if (i >= 0) r.re(i) -= vr, r.im(i) -= vi;
            };
            ac_elements(L, s, [&](const sp_element& el, int, const double* g) {
        const double g0 = g[0], g1 = g[1], g2 = g[2];
                const int a0 = el.node[0], a1 = el.node[1], a2 = el.node[2];
                switch (el.kind) {
                    case SP_EL_R:
                    case SP_EL_D: {
                        const double ir = g0 * (xr(a0) - xr(a1)), ii = g0 * (xi(a0) - xi(a1));
                        sub(a0, ir, ii), sub(a1, -ir, -ii);
                        break;
                    }
                    case SP_EL_C: {  // j w C (v0 - v1)
                        const double y = wv * g0;
                        const double ir = -y * (xi(a0) - xi(a1)), ii = y * (xr(a0) - xr(a1));
                        sub(a0, ir, ii), sub(a1, -ir, -ii);
                        break;
                    }
                    case SP_EL_V:
                    case SP_EL_L: {
                        const int br = nn + el.branch;
                        sub(a0, x.re(br), x.im(br)), sub(a1, -x.re(br), -x.im(br));
                        sub(br, xr(a0) - xr(a1), xi(a0) - xi(a1));
                        if (el.kind == SP_EL_L) {  // -j w L on the branch diagonal
                            const double z = wv * g0;
                            sub(br, z * x.im(br), -z * x.re(br));
                        }
                        break;
                    }
                    case SP_EL_NMOS:
                    case SP_EL_PMOS: {
                        const double ir = g0 * (xr(a0) - xr(a2)) + g1 * (xr(a1) - xr(a2));
                        const double ii = g0 * (xi(a0) - xi(a2)) + g1 * (xi(a1) - xi(a2));
                        sub(a0, ir, ii), sub(a2, -ir, -ii);
                        break;
                    }
                    case SP_EL_NPN:
                    case SP_EL_PNP: {
                        const double ibr = g0 * (xr(a1) - xr(a2)), ibi = g0 * (xi(a1) - xi(a2));
                        const double icr = g1 * (xr(a0) - xr(a2)) + g2 * (xr(a1) - xr(a2));
                        const double ici = g1 * (xi(a0) - xi(a2)) + g2 * (xi(a1) - xi(a2));
                        sub(a1, ibr, ibi), sub(a2, -ibr, -ibi);
                        sub(a0, icr, ici), sub(a2, -icr, -ici);
                        break;
                    }
                    case SP_EL_BSIM3N:
                    case SP_EL_BSIM3P: {  // channel current, then j w C (v_i - v_j) of each capacitance
                        const int a3 = el.node[3];
                        const double ir = g0 * (xr(a0) - xr(a2)) + g1 * (xr(a1) - xr(a2)) + g2 * (xr(a3) - xr(a2));
                        const double ii = g0 * (xi(a0) - xi(a2)) + g1 * (xi(a1) - xi(a2)) + g2 * (xi(a3) - xi(a2));
                        sub(a0, ir, ii), sub(a2, -ir, -ii);
                        const int pr[5][2] = {{a1, a2}, {a1, a0}, {a1, a3}, {a3, a2}, {a3, a0}};
                        for (int k = 0; k < 5; ++k) {
                            if (!(g[3 + k] > 0.0)) continue;
                            const double y = wv * g[3 + k];
                            const int i = pr[k][0], j = pr[k][1];
                            const double cr = -y * (xi(i) - xi(j)), ci = y * (xr(i) - xr(j));
                            sub(i, cr, ci), sub(j, -cr, -ci);
                        }
                        break;
                    }
                    default:
                        break;
                }
            });
        }
    }
    if (!ok) atomicOr(L.singular + s, 1u);
    for (int k = 0; k < L.num_probe; ++k) {
        out[2 * k] = ok ? x.re(L.probe[k]) : CUDART_NAN;
        out[2 * k + 1] = ok ? x.im(L.probe[k]) : CUDART_NAN;
    }
}

__global__ void __launch_bounds__(128) ac_mixed_kernel(AcLaunch L) {
    extern __shared__ __align__(16) unsigned char ac_smem[];
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
    const int n = L.c.n;
    float* fb;
    double* db;
    int64_t stride;
    if (L.work) {  // [2 n^2 + 2 n floats][threads], then [4 n doubles][threads]
        stride = (int64_t)nthreads;
        fb = reinterpret_cast<float*>(L.work) + t;
        db = reinterpret_cast<double*>(reinterpret_cast<float*>(L.work) + (size_t)(2 * n * n + 2 * n + 1) / 2 * 2 * nthreads) + t;
    } else {
        stride = blockDim.x;
        fb = reinterpret_cast<float*>(ac_smem) + threadIdx.x;
        db = reinterpret_cast<double*>(ac_smem + (size_t)((2 * n * n + 2 * n + 1) / 2 * 2) * 4 * blockDim.x) + threadIdx.x;
    }
    const uint64_t total = L.count * (uint64_t)L.nf;
    for (uint64_t u = t; u < total; u += nthreads) ac_mixed_unit(L, u, fb, db, stride);
}
#endif  // SP_AC_MIXED_KERNELS

}  // namespace sp
