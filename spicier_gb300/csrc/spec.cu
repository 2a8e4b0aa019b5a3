// Topology-specialised Newton kernels, generated and compiled at run time.
//
// For one circuit the generic kernels interpret the element list and keep the
// dense Jacobian in shared memory.  Here the element list, the MNA sparsity
// pattern and the elimination order are constants: the host generates CUDA
// source in which every stamp is a named register update, the factorisation
// is straight-line code over the structural nonzeros plus their fill, and the
// whole Newton iteration of one sample stays in registers.  The pivot order
// is the partial-pivoting order of the Jacobian at the circuit's nominal
// operating point (parameters at their distribution centres, x at the
// nodeset), chosen once and cached with the symbolic fill pattern — the
// numeric factorisation of every iteration of every sample reuses it (the
// cached symbolic factorisation of CachedSparseLu, linear.rs:334-410, taken
// to compile time).  A zero or non-finite pivot marks the sample singular, and
// it goes to the generic fallback chain.
//
// The iteration is the correction form of the mixed-precision kernel: FP64
// device currents and KCL residual F(x) (current form: each element adds
// its current, not G*x - b), FP32 Jacobian (device conductances evaluated
// from an FP32 shadow of x) and LU for the step, FP64 update, and the
// convergence test of check_convergence (newton.rs:134-159) on the FP32 step.
// GB300's FP64 pipe is the bound of this kernel, so nothing that does not
// need 53 bits runs on it: the region tests are sign-bit tests and the
// FP64 <-> FP32 conversions run on the integer pipe.  With precision
// SP_PREC_FP64 the Jacobian, LU and test are FP64 instead.
#include <nvrtc.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

namespace sp {

namespace {

struct Pattern {
    int n = 0;
    std::vector<int> perm, iperm;  // permuted row k holds original row perm[k]
    std::vector<int> slot;         // [k*n + j] -> J slot or -1 (permuted rows)
    int nnz = 0;
    bool has(int k, int j) const { return slot[k * n + j] >= 0; }
    int at(int orig_row, int col) const { return slot[iperm[orig_row] * n + col]; }
};

double nominal_value(const sp_param& p) {
    switch (p.kind) {
        case SP_DRAW_FIXED: return p.a;
        case SP_DRAW_GAUSS: return p.a;
        case SP_DRAW_UNIFORM: return 0.5 * (p.a + p.b);
        case SP_DRAW_LOGUNIFORM: return std::sqrt(p.a * p.b);
        default: return 1.0;
    }
}

struct HostSink {
    std::vector<double>& A;
    std::vector<double>& b;
    const std::vector<double>& xs;
    int n;
    double x(int i) const { return xs[i]; }
    void add(int r, int c, double v) { A[(size_t)c * n + r] += v; }
    void rhs_add(int r, double v) { b[r] += v; }
    void rhs_set(int r, double v) { b[r] = v; }
};

// Structural nonzeros of the MNA Jacobian of the element list.
std::vector<char> structure(const std::vector<sp_element>& els, int nn, int n) {
    std::vector<char> S((size_t)n * n, 0);
    auto put = [&](int r, int c) {
        if (r >= 0 && c >= 0) S[(size_t)r * n + c] = 1;
    };
    for (const sp_element& e : els) {
        const int a = e.node[0], b = e.node[1], c = e.node[2];
        switch (e.kind) {
            case SP_EL_R:
            case SP_EL_D:
                put(a, a), put(b, b), put(a, b), put(b, a);
                break;
            case SP_EL_V:
            case SP_EL_L: {
                const int br = nn + e.branch;
                put(a, br), put(br, a), put(b, br), put(br, b);
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS:  // d = a, g = b, s = c
                put(a, a), put(c, c), put(a, c), put(c, a), put(a, b), put(c, b);
                break;
            case SP_EL_NPN:
            case SP_EL_PNP:  // c = a, b = b, e = c
                put(b, b), put(c, c), put(b, c), put(c, b), put(a, a), put(a, c), put(c, a), put(a, b);
                break;
            default:
                break;
        }
    }
    return S;
}

// Partial pivoting (column icamax over structural candidates) at the
// nominal Jacobian, then the symbolic fill of the permuted pattern.
bool plan(const sp_topology* t, Pattern& P, std::string& why) {
    const int n = t->n, nn = t->num_nodes;
    // nominal parameters and derived constants
    std::vector<double> prm(t->num_params);
    for (int k = 0; k < t->num_params; ++k) prm[k] = nominal_value(t->h_params[k]);
    std::vector<double> der(t->num_derived, 0.0);
    std::vector<int> doff(t->num_elements);
    for (int e = 0, o = 0; e < t->num_elements; ++e) {
        doff[e] = o;
        const sp_element& el = t->h_elements[e];
        derive_element(el, [&](int s) { return prm[s]; }, [&](int k, double v) { der[o + k] = v; });
        o += derived_count(el.kind);
    }
    DevCircuit hc{nn, t->num_branches, n, t->num_elements, t->num_params, t->num_derived,
                  t->h_elements.data(), t->h_params.data(), nullptr, doff.data(), nullptr};
    std::vector<double> x(n, 0.0);
    if (!t->h_nodeset.empty()) x = t->h_nodeset;
    std::vector<double> A((size_t)n * n, 0.0), b(n, 0.0);
    HostSink sink{A, b, x, n};
    stamp_all(hc, SoA{der.data(), 1}, 0, sink, STAMP_PLAIN, 0.0);
    std::vector<char> S = structure(t->h_elements, nn, n);
    // work on a row-major copy with row swaps tracked in perm
    std::vector<double> M((size_t)n * n);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) M[(size_t)r * n + c] = A[(size_t)c * n + r];
    std::vector<char> Sp = S;
    P.n = n;
    P.perm.resize(n);
    for (int i = 0; i < n; ++i) P.perm[i] = i;
    for (int k = 0; k < n; ++k) {
        int piv = -1;
        double best = -1.0;
        for (int r = k; r < n; ++r) {
            if (!Sp[(size_t)r * n + k]) continue;
            double v = std::fabs(M[(size_t)r * n + k]);
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        if (piv < 0) {
            why = "structurally singular column " + std::to_string(k);
            return false;
        }
        if (piv != k) {
            for (int c = 0; c < n; ++c) {
                std::swap(M[(size_t)k * n + c], M[(size_t)piv * n + c]);
                std::swap(Sp[(size_t)k * n + c], Sp[(size_t)piv * n + c]);
            }
            std::swap(P.perm[k], P.perm[piv]);
        }
        const double d = M[(size_t)k * n + k];
        for (int r = k + 1; r < n; ++r) {
            if (!Sp[(size_t)r * n + k]) continue;
            const double l = d != 0.0 ? M[(size_t)r * n + k] / d : 0.0;
            for (int c = k + 1; c < n; ++c)
                if (Sp[(size_t)k * n + c]) {
                    M[(size_t)r * n + c] -= l * M[(size_t)k * n + c];
                    Sp[(size_t)r * n + c] = 1;  // fill
                }
        }
    }
    P.iperm.resize(n);
    for (int k = 0; k < n; ++k) P.iperm[P.perm[k]] = k;
    P.slot.assign((size_t)n * n, -1);
    P.nnz = 0;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            if (Sp[(size_t)k * n + j]) P.slot[k * n + j] = P.nnz++;
    return true;
}

const char* kPreamble = R"SRC(
typedef unsigned long long u64;
// Per-block moments of the converged samples (the layout of sp_moments).
struct spx_mom { u64 count; double sum, sum_sq, mn, mx; };
struct SpecArgs {
    const double* dv; u64 stride; u64 count;
    const double* x0; const double* nodeset;
    double* x; int* iters; unsigned char* status; double* resid;
    unsigned int* fail_list; unsigned int* fail_count;
    double reltol, vabstol, iabstol; int max_it; int fallback_any;
    u64* next;
    const double* lp; u64 lpstride; const float* lw; const float* lio; const int* lslots; int lnin;
    double* dvo;
    spx_mom* mom;
    int cold_max_it;
};
__device__ __forceinline__ bool spx_fin(double v) {  // not Inf / NaN, on the integer pipe
    return ((unsigned int)(__double_as_longlong(v) >> 32) & 0x7ff00000u) != 0x7ff00000u;
}
__device__ __forceinline__ bool spx_bad(float p, float iv) { return !(fabsf(p) > 0.f) || !(fabsf(iv) <= 3.0e38f); }
__device__ __forceinline__ bool spx_bad(double p, double iv) { return !(fabs(p) > 0.0) || !(fabs(iv) <= 1.0e308); }
// FP64 <-> FP32 conversions entirely on the integer pipe (GB300's FP64 pipe
// issues conversions at the FP64 rate), round to nearest even, with zeros,
// subnormals, overflow, Inf and NaN handled by integer code too: a fallback
// to the hardware conversion would be if-converted into every call.
__device__ __forceinline__ float spx_f(double x) {
    const u64 b = (u64)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ff);
    const u64 m = (b & ((1ULL << 52) - 1)) | (ex ? (1ULL << 52) : 0ULL);  // 53-bit significand
    const int e = ex - 1023 + 127;                                         // biased float exponent
    // normal results keep 24 bits (drop 29); subnormal ones drop 29 + 1 - e
    int sh = e >= 1 ? 29 : 30 - e;
    sh = sh > 63 ? 63 : sh;
    const u64 q = m >> sh, rem = m & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    unsigned int f = (unsigned int)q + (unsigned int)(rem > half || (rem == half && (q & 1)));
    // f counts in units of the result's last place: for normal results add the
    // exponent field minus the implicit bit (a carry rounds into the exponent)
    f = e >= 1 ? f + ((unsigned int)(e - 1) << 23) : f;
    f = (e >= 255 || f >= 0x7f800000u) ? 0x7f800000u : f;                   // overflow -> Inf
    f = ex == 0x7ff ? (0x7f800000u | (unsigned int)(m >> 29) | ((b & ((1ULL << 52) - 1)) ? 0x400000u : 0u)) : f;
    return __uint_as_float(sign | f);
}
__device__ __forceinline__ float spx_fneg(double x) { return __uint_as_float(__float_as_uint(spx_f(x)) ^ 0x80000000u); }
__device__ __forceinline__ double spx_d(float x) {
    const unsigned int f = __float_as_uint(x);
    const u64 sign = (u64)(f & 0x80000000u) << 32;
    const unsigned int e = (f >> 23) & 0xff, m = f & 0x7fffffu;
    // subnormal floats: normalise the 23-bit significand (m != 0); zero stays zero
    const int lz = __clz(m) - 8;  // m < 2^23: shift that brings its top bit to bit 23
    const u64 sub = m ? ((u64)(1023 - 126 - lz) << 52) | ((u64)((m << lz) & 0x7fffffu) << 29) : 0ULL;
    const u64 nrm = ((u64)(e - 127 + 1023) << 52) | ((u64)m << 29);
    const u64 inf = (0x7ffULL << 52) | ((u64)m << 29);
    return __longlong_as_double((long long)(sign | (e == 0 ? sub : (e == 255 ? inf : nrm))));
}
// Double-float (an FP32 pair h + l, |l| <= ulp(h) / 2, about 48 bits) for the
// KCL residual and device currents of the mixed kernel on topologies whose
// elements allow it: GB300 issues FP32 at 64 times its FP64 rate.  Every
// operation is written with the _rn intrinsics and fmaf so that the compiler
// contracts nothing (the error terms must be the exact rounding errors).
struct spx_df { float h, l; };
__device__ __forceinline__ spx_df spx_two(float s, float e) {  // |s| >= |e|, or s == 0
    const float h = __fadd_rn(s, e);
    return spx_df{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ spx_df spx_add(spx_df a, spx_df b) {
    const float s = __fadd_rn(a.h, b.h), bb = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    return spx_two(s, e);
}
__device__ __forceinline__ spx_df spx_addf(spx_df a, float b) {
    const float s = __fadd_rn(a.h, b), bb = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    e = __fadd_rn(e, a.l);
    return spx_two(s, e);
}
__device__ __forceinline__ spx_df spx_neg2(spx_df a) { return spx_df{-a.h, -a.l}; }
__device__ __forceinline__ spx_df spx_sub(spx_df a, spx_df b) { return spx_add(a, spx_neg2(b)); }
__device__ __forceinline__ spx_df spx_mulf(spx_df a, float b) {
    const float p = __fmul_rn(a.h, b);
    float e = fmaf(a.h, b, -p);
    e = fmaf(a.l, b, e);
    return spx_two(p, e);
}
__device__ __forceinline__ spx_df spx_mul(spx_df a, spx_df b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return spx_two(p, e);
}
__device__ __forceinline__ bool spx_finf(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }
// Order-preserving integer keys of doubles (min and max of the block moments).
__device__ __forceinline__ long long spx_key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b) - 1;
}
__device__ __forceinline__ double spx_unkey(long long k) {
    return __longlong_as_double(k >= 0 ? k : (long long)(0x8000000000000000ULL - (unsigned long long)(k + 1)));
}
// v < 0 from the sign bit (integer pipe); -0 is not negative
__device__ __forceinline__ bool spx_neg(double v) {
    const long long b = __double_as_longlong(v);
    return b < 0 && (b << 1) != 0;
}
__device__ __forceinline__ double spx_lim(double vd, double nvt, double vcrit) {
    if (vd > vcrit) { double arg = (vd - vcrit) / nvt; return vcrit + nvt * (1.0 + log1p(arg)); }
    return vd;
}
__device__ __forceinline__ void spx_mos(bool pmos, double vth, double beta, double lam, double vgs, double vds,
                                        double& ids, double& gds, double& gm) {
    if (pmos) { vgs = -vgs; vds = -vds; }
    if (vgs < vth) { ids = 0.0; gds = 1e-12; gm = 0.0; }
    else if (vds < vgs - vth) {
        double vov = vgs - vth;
        double i = beta * (vov * vds - 0.5 * vds * vds) * (1.0 + lam * vds);
        double g = beta * (vov - vds) * (1.0 + lam * vds) + beta * (vov * vds - 0.5 * vds * vds) * lam;
        double m = beta * vds * (1.0 + lam * vds);
        ids = pmos ? -i : i; gds = fmax(g, 1e-12); gm = m;
    } else {
        double vov = vgs - vth;
        double i = 0.5 * beta * vov * vov * (1.0 + lam * vds);
        double g = 0.5 * beta * vov * vov * lam;
        double m = beta * vov * (1.0 + lam * vds);
        ids = pmos ? -i : i; gds = fmax(g, 1e-12); gm = m;
    }
}
)SRC";

std::string V(int node) { return node >= 0 ? "x[" + std::to_string(node) + "]" : "0.0"; }

// Element currents into F (and, when jac, conductances into J).
// mixed: the Jacobian in FP32 — MOSFET conductances from the FP32 shadow xf
// of x and FP32 copies of the constants, other conversions on the integer pipe.
void emit_elements(std::ostringstream& o, const sp_topology* t, const Pattern& P, const std::vector<int>& doff,
                   bool jac, bool mixed = false) {
    const int nn = t->num_nodes;
    auto cst = [&](int e, int k) { return "c" + std::to_string(doff[e] + k); };
    auto cstf = [&](int e, int k) { return "cf" + std::to_string(doff[e] + k); };
    auto VF = [&](int node) { return node >= 0 ? "xf[" + std::to_string(node) + "]" : std::string("0.f"); };
    const char* cvt = mixed ? "spx_f" : "(JT)";
    auto J = [&](int r, int c, const std::string& expr, bool neg) {
        if (r < 0 || c < 0 || !jac) return;
        o << "    J[" << P.at(r, c) << "] " << (neg ? "-=" : "+=") << " " << expr << ";\n";
    };
    auto F = [&](int r, const std::string& expr, bool neg) {
        if (r < 0) return;
        o << "    F[" << r << "] " << (neg ? "-=" : "+=") << " " << expr << ";\n";
    };
    for (int e = 0; e < t->num_elements; ++e) {
        const sp_element& el = t->h_elements[e];
        const int a = el.node[0], b = el.node[1], c = el.node[2];
        o << "  { // element " << e << "\n";
        switch (el.kind) {
            case SP_EL_R:
                o << "    double i = " << cst(e, 0) << " * (" << V(a) << " - " << V(b) << ");\n";
                F(a, "i", false), F(b, "i", true);
                break;  // linear J: emit_linear_jacobian
            case SP_EL_V:
            case SP_EL_L: {
                const int br = nn + el.branch;
                F(a, "x[" + std::to_string(br) + "]", false);
                F(b, "x[" + std::to_string(br) + "]", true);
                std::string val = el.kind == SP_EL_V ? cst(e, 0) : std::string("0.0");
                o << "    F[" << br << "] += " << V(a) << " - " << V(b) << " - " << val << ";\n";
                break;
            }
            case SP_EL_I:
                F(a, cst(e, 0), false), F(b, cst(e, 0), true);
                break;
            case SP_EL_C:
                break;
            case SP_EL_D:
                o << "    double vd = " << V(a) << " - " << V(b) << ";\n"
                  << "    double vl = spx_lim(vd, " << cst(e, 1) << ", " << cst(e, 2) << ");\n"
                  << "    double vl2 = spx_lim(vl, " << cst(e, 1) << ", " << cst(e, 2) << ");\n"
                  << "    double ex = exp(vl2 / " << cst(e, 1) << ");\n"
                  << "    double id = " << cst(e, 0) << " * (ex - 1.0);\n"
                  << "    double gd = fmax(" << cst(e, 0) << " * ex / " << cst(e, 1) << ", 1e-12);\n"
                  << "    double i = id + gd * (vd - vl);\n";
                F(a, "i", false), F(b, "i", true);
                if (jac) {
                    o << "    JT g = " << cvt << "(gd);\n";
                    J(a, a, "g", false), J(b, b, "g", false), J(a, b, "g", true), J(b, a, "g", true);
                }
                break;
            case SP_EL_NMOS:
            case SP_EL_PMOS: {
                const int d = a, g = b, s = c;
                const bool pm = el.kind == SP_EL_PMOS;
                if (mixed) {
                    // level1.rs:154-248 with the drain current in FP64 (it enters F) and
                    // gds, gm in FP32 from the shadow of x.  The region comes from the
                    // FP32 voltages: ids is continuous across both region boundaries
                    // (a misread region changes it by O(delta^2)), and one formula
                    // serves both conducting regions: ids = beta u (vov - u/2) q with
                    // u = vds in the linear region and u = vov in saturation.
                    auto dif = [&](int p, int q) { return pm ? V(q) + " - " + V(p) : V(p) + " - " + V(q); };
                    auto diff = [&](int p, int q) { return pm ? VF(q) + " - " + VF(p) : VF(p) + " - " + VF(q); };
                    o << "    float vgsf = " << diff(g, s) << ", vdsf = " << diff(d, s) << ";\n"
                      << "    float vovf = vgsf - " << cstf(e, 0) << ", qf = 1.f + " << cstf(e, 2) << " * vdsf;\n"
                      << "    bool on = vovf >= 0.f, lin = on && vdsf < vovf;\n"
                      << "    double vds = " << dif(d, s) << ", vov = (" << dif(g, s) << ") - " << cst(e, 0) << ";\n"
                      << "    double u = lin ? vds : vov;\n"
                      << "    double ids = on ? " << cst(e, 1) << " * u * fma(-0.5, u, vov) * fma(" << cst(e, 2)
                      << ", vds, 1.0) : 0.0;\n";
                    if (pm) o << "    ids = -ids;\n";
                    F(d, "ids", false), F(s, "ids", true);
                    o << "    float gdf = 1e-12f, gmf = 0.f;\n"
                      << "    if (lin) { gdf = " << cstf(e, 1) << " * (vovf - vdsf) * qf + " << cstf(e, 1)
                      << " * (vovf * vdsf - 0.5f * vdsf * vdsf) * " << cstf(e, 2) << "; gmf = " << cstf(e, 1)
                      << " * vdsf * qf; }\n"
                      << "    else if (on) { gdf = 0.5f * " << cstf(e, 1) << " * vovf * vovf * " << cstf(e, 2)
                      << "; gmf = " << cstf(e, 1) << " * vovf * qf; }\n"
                      << "    gdf = fmaxf(gdf, 1e-12f);\n";
                } else {
                    o << "    double ids, gds, gm;\n"
                      << "    spx_mos(" << (pm ? "true" : "false") << ", " << cst(e, 0) << ", " << cst(e, 1) << ", "
                      << cst(e, 2) << ", " << V(g) << " - " << V(s) << ", " << V(d) << " - " << V(s)
                      << ", ids, gds, gm);\n";
                    F(d, "ids", false), F(s, "ids", true);
                    if (jac) o << "    JT gdf = (JT)gds, gmf = (JT)gm;\n";
                }
                if (jac) {
                    J(d, d, "gdf", false), J(s, s, "gdf", false), J(d, s, "gdf", true), J(s, d, "gdf", true);
                    J(d, g, "gmf", false), J(d, s, "gmf", true), J(s, g, "gmf", true), J(s, s, "gmf", false);
                }
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {
                const int cn = a, bn = b, en = c;
                const bool pnp = el.kind == SP_EL_PNP;
                o << "    double vbe = " << V(bn) << " - " << V(en) << ", vce = " << V(cn) << " - " << V(en) << ";\n"
                  << "    double is = " << cst(e, 0) << ", bf = " << cst(e, 1) << ", br = " << cst(e, 2)
                  << ", nfv = " << cst(e, 3) << ", nrv = " << cst(e, 4) << ", vaf = " << cst(e, 5)
                  << ", vcf = " << cst(e, 6) << ", vcr = " << cst(e, 7) << ";\n"
                  << "    double vbe_lim = spx_lim(" << (pnp ? "-vbe" : "vbe") << ", nfv, vcf);\n"
                  << "    double vbe_ieq = " << (pnp ? "-vbe_lim" : "vbe_lim") << ";\n"
                  << "    double sgn = " << (pnp ? "-1.0" : "1.0") << ";\n"
                  << "    double ibe = sgn * vbe, ice = sgn * vce, vbc = ibe - ice;\n"
                  << "    double exb = exp(spx_lim(ibe, nfv, vcf) / nfv), exc = exp(spx_lim(vbc, nrv, vcr) / nrv);\n"
                  << "    double i_f = is * (exb - 1.0), i_r = is * (exc - 1.0);\n"
                  << "    bool vfin = spx_fin(vaf) && vaf > 0.0;\n"
                  << "    double early = (vfin && ice > 0.0) ? 1.0 + ice / vaf : 1.0;\n"
                  << "    double ic = (i_f - i_r / br) * early, ib = i_f / bf + i_r / br;\n"
                  << "    double gmv = (i_f > 1e-20) ? (is * exb / nfv) * early : 1e-12;\n"
                  << "    double gpi = gmv / bf;\n"
                  << "    double go_e = (vfin && fabs(ic) > 1e-20) ? fabs(ic) / vaf : 0.0;\n"
                  << "    double go = fmax(go_e + is * exc / nrv / br * early, 1e-12);\n"
                  << "    ic = sgn * ic; ib = sgn * ib;\n"
                  << "    double gm = fmax(gmv, 1e-12); gpi = fmax(gpi, 1e-12); go = fmax(go, 1e-12);\n"
                  << "    double fc = ic + gm * (vbe - vbe_ieq), fb = ib + gpi * (vbe - vbe_ieq);\n";
                F(cn, "fc", false), F(bn, "fb", false), F(en, "(fc + fb)", true);
                if (jac) {
                    o << "    JT gpf = " << cvt << "(gpi), gof = " << cvt << "(go), gmf = " << cvt << "(gm);\n";
                    J(bn, bn, "gpf", false), J(en, en, "gpf", false), J(bn, en, "gpf", true), J(en, bn, "gpf", true);
                    J(cn, cn, "gof", false), J(en, en, "gof", false), J(cn, en, "gof", true), J(en, cn, "gof", true);
                    J(cn, bn, "gmf", false), J(cn, en, "gmf", true), J(en, bn, "gmf", true), J(en, en, "gmf", false);
                }
                break;
            }
            default:
                break;
        }
        o << "  }\n";
    }
}

// Linear (per-sample constant) Jacobian entries, stamped into J at the start
// of every iteration: the +-1 entries of sources and inductors are literals
// the compiler folds, and only the resistor conductances (g<e>, converted
// once per sample) occupy registers.
void emit_linear_jacobian(std::ostringstream& o, const sp_topology* t, const Pattern& P) {
    const int nn = t->num_nodes;
    o << "    #pragma unroll\n    for (int k = 0; k < " << P.nnz << "; ++k) J[k] = (JT)0;\n";
    for (int e = 0; e < t->num_elements; ++e) {
        const sp_element& el = t->h_elements[e];
        const int a = el.node[0], b = el.node[1];
        if (el.kind == SP_EL_R) {
            const std::string g = "g" + std::to_string(e);
            if (a >= 0) o << "    J[" << P.at(a, a) << "] += " << g << ";\n";
            if (b >= 0) o << "    J[" << P.at(b, b) << "] += " << g << ";\n";
            if (a >= 0 && b >= 0) o << "    J[" << P.at(a, b) << "] -= " << g << "; J[" << P.at(b, a) << "] -= " << g << ";\n";
        } else if (el.kind == SP_EL_V || el.kind == SP_EL_L) {
            const int br = nn + el.branch;
            if (a >= 0) o << "    J[" << P.at(a, br) << "] += (JT)1; J[" << P.at(br, a) << "] += (JT)1;\n";
            if (b >= 0) o << "    J[" << P.at(b, br) << "] -= (JT)1; J[" << P.at(br, b) << "] -= (JT)1;\n";
        }
    }
}

// The kernel is persistent: each thread iterates one sample at a time and,
// when its sample has converged (or failed), takes the next one from a
// global counter (warp-aggregated atomics), so lanes whose samples converge
// early do not idle while others iterate: the warp executes about the mean
// iteration count per sample, not the maximum over its 32 lanes.  Which
// thread solves a sample does not change the sample's arithmetic.
// Per-thread shared memory of the per-sample constants (0: they stay in
// registers).  Shared memory frees ~3 registers per constant, so more warps
// stay resident to hide the latency of the next sample's loads.
// The mixed kernel keeps its state, KCL residual and device currents in
// double-float when every element is linear or a Level-1 MOSFET (the diode
// and BJT limiters and exponentials stay in FP64).
bool df_supported(const sp_topology* t) {
    for (const sp_element& el : t->h_elements)
        switch (el.kind) {
            case SP_EL_R: case SP_EL_C: case SP_EL_L: case SP_EL_V: case SP_EL_I: case SP_EL_NMOS: case SP_EL_PMOS:
                break;
            default:
                return false;
        }
    return true;
}

// Derived constants that the mixed kernel also keeps in FP32 (cf<k>): the
// MOSFET constants (for the FP32 Jacobian, and the currents in double-float
// mode) and, in double-float mode, the source values.
std::vector<int> fp32_constants(const sp_topology* t, bool fp32_jac) {
    std::vector<int> fcs;
    if (!fp32_jac) return fcs;
    const bool dfm = df_supported(t);
    for (int e = 0, o = 0; e < t->num_elements; ++e) {
        const int kind = t->h_elements[e].kind;
        if (kind == SP_EL_NMOS || kind == SP_EL_PMOS)
            for (int k = 0; k < 3; ++k) fcs.push_back(o + k);
        else if (dfm && (kind == SP_EL_V || kind == SP_EL_I))
            fcs.push_back(o);
        o += derived_count(kind);
    }
    return fcs;
}

size_t spec_smem_bytes(const sp_topology* t, bool fp32_jac) {
    const size_t nfc = fp32_constants(t, fp32_jac).size();
    const size_t bytes = ((size_t)t->num_derived * 8 + nfc * 4) * 128;
    return bytes <= 48 * 1024 ? bytes : 0;
}

// Element currents into the double-float residual F (state X, double-float)
// and conductances into the FP32 Jacobian J (from X[].h, as in
// emit_elements' mixed mode): the same formulas, with the constants in FP32
// (a relative change of at most 2^-24 in a device parameter or source value,
// far inside the SPICE tolerances the mixed precision is held to).
void emit_elements_df(std::ostringstream& o, const sp_topology* t, const Pattern& P, const std::vector<int>& doff) {
    const int nn = t->num_nodes;
    auto cf = [&](int e, int k) { return "cf" + std::to_string(doff[e] + k); };
    auto XV = [&](int node) { return node >= 0 ? "X[" + std::to_string(node) + "]" : std::string("spx_df{0.f, 0.f}"); };
    auto XF = [&](int node) { return node >= 0 ? "X[" + std::to_string(node) + "].h" : std::string("0.f"); };
    auto J = [&](int r, int c, const std::string& expr, bool neg) {
        if (r < 0 || c < 0) return;
        o << "    J[" << P.at(r, c) << "] " << (neg ? "-=" : "+=") << " " << expr << ";\n";
    };
    auto F = [&](int r, const std::string& expr, bool neg) {
        if (r < 0) return;
        o << "    F[" << r << "] = spx_add(F[" << r << "], " << (neg ? "spx_neg2(" + expr + ")" : expr) << ");\n";
    };
    for (int e = 0; e < t->num_elements; ++e) {
        const sp_element& el = t->h_elements[e];
        const int a = el.node[0], b = el.node[1], c = el.node[2];
        o << "  { // element " << e << "\n";
        switch (el.kind) {
            case SP_EL_R:
                o << "    const spx_df i = spx_mulf(spx_sub(" << XV(a) << ", " << XV(b) << "), g" << e << ");\n";
                F(a, "i", false), F(b, "i", true);
                break;
            case SP_EL_V:
            case SP_EL_L: {
                const int br = nn + el.branch;
                F(a, "X[" + std::to_string(br) + "]", false);
                F(b, "X[" + std::to_string(br) + "]", true);
                o << "    F[" << br << "] = spx_add(F[" << br << "], ";
                if (el.kind == SP_EL_V)
                    o << "spx_addf(spx_sub(" << XV(a) << ", " << XV(b) << "), -" << cf(e, 0) << "));\n";
                else
                    o << "spx_sub(" << XV(a) << ", " << XV(b) << "));\n";
                break;
            }
            case SP_EL_I:
                if (a >= 0) o << "    F[" << a << "] = spx_addf(F[" << a << "], " << cf(e, 0) << ");\n";
                if (b >= 0) o << "    F[" << b << "] = spx_addf(F[" << b << "], -" << cf(e, 0) << ");\n";
                break;
            case SP_EL_C:
                break;
            case SP_EL_NMOS:
            case SP_EL_PMOS: {
                const int d = a, g = b, s = c;
                const bool pm = el.kind == SP_EL_PMOS;
                auto dv = [&](int p, int q) { return pm ? "spx_sub(" + XV(q) + ", " + XV(p) + ")" : "spx_sub(" + XV(p) + ", " + XV(q) + ")"; };
                auto df32 = [&](int p, int q) { return pm ? XF(q) + " - " + XF(p) : XF(p) + " - " + XF(q); };
                o << "    float vgsf = " << df32(g, s) << ", vdsf = " << df32(d, s) << ";\n"
                  << "    float vovf = vgsf - " << cf(e, 0) << ", qf = 1.f + " << cf(e, 2) << " * vdsf;\n"
                  << "    bool on = vovf >= 0.f, lin = on && vdsf < vovf;\n"
                  << "    const spx_df vds = " << dv(d, s) << ";\n"
                  << "    const spx_df vov = spx_addf(" << dv(g, s) << ", -" << cf(e, 0) << ");\n"
                  << "    const spx_df u = lin ? vds : vov;\n"
                  << "    const spx_df t1 = spx_sub(vov, spx_df{0.5f * u.h, 0.5f * u.l});\n"
                  << "    const spx_df t2 = spx_addf(spx_mulf(vds, " << cf(e, 2) << "), 1.f);\n"
                  << "    spx_df ids = on ? spx_mul(spx_mul(spx_mulf(u, " << cf(e, 1) << "), t1), t2) : spx_df{0.f, 0.f};\n";
                if (pm) o << "    ids = spx_neg2(ids);\n";
                F(d, "ids", false), F(s, "ids", true);
                o << "    float gdf = 1e-12f, gmf = 0.f;\n"
                  << "    if (lin) { gdf = " << cf(e, 1) << " * (vovf - vdsf) * qf + " << cf(e, 1)
                  << " * (vovf * vdsf - 0.5f * vdsf * vdsf) * " << cf(e, 2) << "; gmf = " << cf(e, 1)
                  << " * vdsf * qf; }\n"
                  << "    else if (on) { gdf = 0.5f * " << cf(e, 1) << " * vovf * vovf * " << cf(e, 2)
                  << "; gmf = " << cf(e, 1) << " * vovf * qf; }\n"
                  << "    gdf = fmaxf(gdf, 1e-12f);\n";
                J(d, d, "gdf", false), J(s, s, "gdf", false), J(d, s, "gdf", true), J(s, d, "gdf", true);
                J(d, g, "gmf", false), J(d, s, "gmf", true), J(s, g, "gmf", true), J(s, s, "gmf", false);
                break;
            }
            default:
                break;
        }
        o << "  }\n";
    }
}

// C++ literal of a double (exact, hexadecimal) and of its FP32 rounding.
std::string lit64(double v) {
    char b[64];
    snprintf(b, sizeof b, "%a", v);
    return std::string("(") + b + ")";
}
std::string lit32(double v) {
    char b[64];
    snprintf(b, sizeof b, "%af", (double)(float)v);
    return std::string("(") + b + ")";
}

// Parameters mode of the double-float kernel: the per-sample constants are
// computed from the sample's parameters (drawn slots loaded, fixed slots
// compiled in as literals) instead of read from the draw kernel's derived
// constants, so that kernel skips its derivation.  pd<slot> is the loaded
// FP64 value of drawn slot `slot`.
struct ParamExpr {
    const sp_topology* t;
    std::string d(int slot) const {  // FP64 value
        const sp_param& p = t->h_params[slot];
        return p.kind == SP_DRAW_FIXED ? lit64(p.a) : "pd" + std::to_string(slot);
    }
    std::string f(int slot) const {  // FP32 value
        const sp_param& p = t->h_params[slot];
        return p.kind == SP_DRAW_FIXED ? lit32(p.a) : "pf" + std::to_string(slot);
    }
};

// Drawn parameter slots that the elements of t read (parameters mode loads these).
std::vector<int> drawn_slots_used(const sp_topology* t) {
    std::vector<int> out;
    auto use = [&](int slot) {
        if (slot >= 0 && slot < t->num_params && t->h_params[slot].kind != SP_DRAW_FIXED &&
            std::find(out.begin(), out.end(), slot) == out.end())
            out.push_back(slot);
    };
    for (const sp_element& el : t->h_elements) {
        if (el.kind == SP_EL_NMOS || el.kind == SP_EL_PMOS)
            for (int k : {0, 1, 2, 3, 4, 5}) use(el.field[k]);
        else if (el.kind == SP_EL_R || el.kind == SP_EL_C || el.kind == SP_EL_L || el.kind == SP_EL_V ||
                 el.kind == SP_EL_I)
            use(el.field[0]);
    }
    return out;
}

// The linear warm start as a launch parameter of the double-float kernel
// (SpecLin): for each drawn slot the elements read, in ascending slot order,
// its weights for the n unknowns, then the slots' input means, then the n
// output means; mask bit k set where the k-th slot is an input.  The kernel
// evaluates out + sum_k w_k (p_k - m_k) over the set bits in slot order with
// the weights as constant-bank operands, which is the standalone evaluation's
// order when the inputs are ascending slots.
struct LinLayout {
    std::vector<int> slots;  // ascending
    int nw = 1;              // floats of SpecLin::w
    bool usable = false;     // the kernel carries the parameter-order path
};
LinLayout lin_layout(const sp_topology* t, bool dfm) {
    LinLayout l;
    if (!dfm) return l;
    l.slots = drawn_slots_used(t);
    std::sort(l.slots.begin(), l.slots.end());
    const int ps = (int)l.slots.size();
    if (ps == 0 || ps > 64 || (size_t)(ps * t->n + ps + t->n) * 4 > 3072) return l;
    l.nw = ps * t->n + ps + t->n;
    l.usable = true;
    return l;
}

// FP64 derived constants of element e (derive_element's operations in its
// order: IEEE division and products, so the values equal the draw kernel's).
void emit_derive64(std::ostringstream& o, const sp_topology* t, const std::vector<int>& doff, const ParamExpr& pe,
                   const char* indent) {
    for (int e = 0; e < t->num_elements; ++e) {
        const sp_element& el = t->h_elements[e];
        const int d0 = doff[e];
        switch (el.kind) {
            case SP_EL_R:
                o << indent << "c" << d0 << " = 1.0 / " << pe.d(el.field[0]) << ";\n";
                break;
            case SP_EL_NMOS:
            case SP_EL_PMOS:
                o << indent << "c" << d0 << " = fabs(" << pe.d(el.field[0]) << ");\n"
                  << indent << "c" << d0 + 1 << " = ((" << pe.d(el.field[1]) << " * " << pe.d(el.field[5]) << ") * "
                  << pe.d(el.field[3]) << ") / " << pe.d(el.field[4]) << ";\n"
                  << indent << "c" << d0 + 2 << " = " << pe.d(el.field[2]) << ";\n";
                break;
            default:  // C, L, V, I
                o << indent << "c" << d0 << " = " << pe.d(el.field[0]) << ";\n";
                break;
        }
    }
}

std::string generate(const sp_topology* t, const Pattern& P, bool fp32_jac) {
    const int n = t->n, nn = t->num_nodes;
    std::vector<int> doff(t->num_elements);
    for (int e = 0, o = 0; e < t->num_elements; ++e) {
        doff[e] = o;
        o += derived_count(t->h_elements[e].kind);
    }
    const bool sm = spec_smem_bytes(t, fp32_jac) > 0;
    const std::vector<int> fcs = fp32_constants(t, fp32_jac);
    const bool dfm = fp32_jac && df_supported(t);  // double-float state and residual
    std::ostringstream o;
    o << kPreamble << "typedef " << (fp32_jac ? "float" : "double") << " JT;\n";
    if (sm) {  // constant k of this thread at [k][threadIdx.x]; volatile keeps them out of registers
        for (int k = 0; k < t->num_derived; ++k) o << "#define c" << k << " (spx_cd[" << k << " * 128])\n";
        for (size_t j = 0; j < fcs.size(); ++j) o << "#define cf" << fcs[j] << " (spx_cf[" << j << " * 128])\n";
    }
    const LinLayout ll = lin_layout(t, dfm);
    o << "struct SpecLin { unsigned long long mask; int on; int pad; float w[" << ll.nw << "]; };\n";
    o << "extern \"C\" __global__ void __launch_bounds__(128, " << (sm ? (fp32_jac ? 4 : 2) : 1)
      << ") spec_newton(SpecArgs a, SpecLin lk) {\n"
      << "  asm volatile(\"griddepcontrol.wait;\" ::: \"memory\");  // chained launch: predecessor complete\n"
      << "  asm volatile(\"griddepcontrol.launch_dependents;\" ::: \"memory\");\n"
      << "  const u64 nthreads = (u64)gridDim.x * blockDim.x;\n"
      << "  u64 s = (u64)blockIdx.x * blockDim.x + threadIdx.x;\n"
      << "  extern __shared__ __align__(16) unsigned char spx_smem[];\n"
      // learned linear warm start: weights lw[n][lnin], in_mean, out_mean and the input slots,
      // staged by the block (behind the per-thread constants) before any thread leaves
      << "  float* const spx_lw = reinterpret_cast<float*>(spx_smem + " << spec_smem_bytes(t, fp32_jac) << ");\n"
      << "  float* const spx_linm = spx_lw + " << n << " * a.lnin;\n"
      << "  float* const spx_lout = spx_linm + a.lnin;\n"
      << "  int* const spx_lslot = reinterpret_cast<int*>(spx_lout + " << n << ");\n"
      << "  if (a.lw && !lk.on) {\n"
      << "    for (int i = threadIdx.x; i < " << n << " * a.lnin; i += blockDim.x) spx_lw[i] = a.lw[i];\n"
      << "    for (int i = threadIdx.x; i < a.lnin; i += blockDim.x) { spx_linm[i] = a.lio[i]; spx_lslot[i] = a.lslots[i]; }\n"
      << "    for (int i = threadIdx.x; i < " << n << "; i += blockDim.x) spx_lout[i] = a.lio[2 * a.lnin + i];\n"
      << "    __syncthreads();\n"
      << "  }\n"
      << "  unsigned char spx_st = 0xff;  // status of the thread's (last) sample\n"
      << "  if (s < a.count) {\n"
      << "  const u64 st = a.stride;\n"
      << "  const bool warm = a.x0 != 0 || a.lw != 0;\n";
    if (sm) {
        o << "  volatile double* const spx_cd = reinterpret_cast<volatile double*>(spx_smem) + threadIdx.x;\n"
          << "  volatile float* const spx_cf = reinterpret_cast<volatile float*>(spx_smem + " << t->num_derived * 8 * 128
          << ") + threadIdx.x;\n";
    } else {
        for (int k = 0; k < t->num_derived; ++k) o << "  double c" << k << ";\n";
        for (int k : fcs) o << "  float cf" << k << ";\n";
    }
    for (int e = 0; e < t->num_elements; ++e)
        if (t->h_elements[e].kind == SP_EL_R) o << "  JT g" << e << ";\n";
    if (dfm)
        o << "  spx_df X[" << n << "];\n";
    else
        o << "  double x[" << n << "];\n";
    if (fp32_jac && !dfm) o << "  float xf[" << n << "];\n";
    if (fp32_jac)
        o << "  const float reltolf = spx_f(a.reltol), vabstolf = spx_f(a.vabstol), iabstolf = spx_f(a.iabstol);\n";
    // it: iterations of the current attempt; spx_itlim its limit; spx_it0 the
    // iterations of a missed warm attempt; spx_cold: the attempt is the cold restart
    o << "  int it, code, spx_itlim, spx_it0;\n  bool spx_cold;\n";
    // per-sample set-up: constants, linear Jacobian, start point
    std::ostringstream ld;
    const ParamExpr pe{t};
    const std::vector<int> pslots = drawn_slots_used(t);
    if (dfm) {
        // parameters mode: the drawn parameters (loads issued together), then the
        // FP32 constants: |VTO|, ((KP NF) W) / L and LAMBDA, 1 / R, source values
        // (at most a few FP32 roundings from the FP64 constants rounded to FP32)
        ld << "  {\n";
        for (int slot : pslots)
            ld << "  const double pd" << slot << " = __ldg(a.lp + (u64)" << slot << " * a.lpstride + s);\n";
        for (int slot : pslots) ld << "  const float pf" << slot << " = __double2float_rn(pd" << slot << ");\n";
        for (int e = 0; e < t->num_elements; ++e) {
            const sp_element& el = t->h_elements[e];
            const int d0 = doff[e];
            switch (el.kind) {
                case SP_EL_R:
                    ld << "  g" << e << " = __fdiv_rn(1.f, " << pe.f(el.field[0]) << ");\n";
                    break;
                case SP_EL_NMOS:
                case SP_EL_PMOS:
                    ld << "  cf" << d0 << " = fabsf(" << pe.f(el.field[0]) << ");\n"
                       << "  cf" << d0 + 1 << " = __fdiv_rn(__fmul_rn(__fmul_rn(" << pe.f(el.field[1]) << ", "
                       << pe.f(el.field[5]) << "), " << pe.f(el.field[3]) << "), " << pe.f(el.field[4]) << ");\n"
                       << "  cf" << d0 + 2 << " = " << pe.f(el.field[2]) << ";\n";
                    break;
                case SP_EL_V:
                case SP_EL_I:
                    ld << "  cf" << d0 << " = " << pe.f(el.field[0]) << ";\n";
                    break;
                default:
                    break;
            }
        }
    } else {
        ld << "  {\n  const double* dv = a.dv + s;\n";
        for (int k = 0; k < t->num_derived; ++k) ld << "  c" << k << " = __ldg(dv + " << k << " * st);\n";
        for (int k : fcs) ld << "  cf" << k << " = spx_f(c" << k << ");\n";
        for (int e = 0; e < t->num_elements; ++e)
            if (t->h_elements[e].kind == SP_EL_R)
                ld << "  g" << e << " = " << (fp32_jac ? "spx_f(c" : "(JT)(c") << doff[e] << ");\n";
    }
    // the learned linear warm start of sample s into xl[] in FP32, the same
    // operations in the same order as its standalone evaluation: from the launch
    // parameter (lk.on: weights as constant-bank operands, inputs the parameters
    // converted above) or from memory (inputs eight at a time with their loads
    // in flight together, weights staged in shared memory)
    ld << "  float xl[" << n << "];\n";
    if (ll.usable) {
        const int ps = (int)ll.slots.size();
        ld << "  if (lk.on) {\n"
           << "    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) xl[i] = lk.w[" << ps * n + ps << " + i];\n";
        for (int k = 0; k < ps; ++k)
            ld << "    if ((lk.mask >> " << k << ") & 1ull) {\n"
               << "      const float v = pf" << ll.slots[k] << " - lk.w[" << ps * n + k << "];\n"
               << "      #pragma unroll\n      for (int i = 0; i < " << n << "; ++i) xl[i] = fmaf(lk.w[" << k * n
               << " + i], v, xl[i]);\n    }\n";
        ld << "  } else\n";
    }
    ld << "  if (a.lw) {\n"
       << "    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) xl[i] = spx_lout[i];\n"
       << "    for (int j0 = 0; j0 < a.lnin; j0 += 8) {\n"
       << "      float pv[8];\n"
       << "      #pragma unroll\n      for (int u = 0; u < 8; ++u)\n"
       << "        pv[u] = j0 + u < a.lnin ? __double2float_rn(__ldg(a.lp + (u64)spx_lslot[j0 + u] * a.lpstride + s))"
          " - spx_linm[j0 + u] : 0.f;\n"
       << "      #pragma unroll\n      for (int u = 0; u < 8; ++u)\n"
       << "        if (j0 + u < a.lnin) {\n"
       << "          #pragma unroll\n          for (int i = 0; i < " << n << "; ++i) xl[i] = fmaf(spx_lw[i * a.lnin + j0 + u], pv[u], xl[i]);\n"
       << "        }\n    }\n  }\n";
    if (dfm)  // the start point rounded to FP32 (a starting guess: its low part is not needed)
        ld << "  #pragma unroll\n  for (int i = 0; i < " << n << "; ++i)\n"
           << "    X[i] = spx_df{a.lw ? xl[i] : (a.x0 ? __double2float_rn(a.x0[s * " << n
           << " + i]) : (a.nodeset ? __double2float_rn(a.nodeset[i]) : 0.f)), 0.f};\n";
    else
        ld << "  if (a.lw) {\n    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) x[i] = (double)xl[i];\n"
           << "  } else if (a.x0) {\n    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) x[i] = a.x0[s * " << n
           << " + i];\n"
           << "  } else if (a.nodeset) {\n    #pragma unroll\n    for (int i = 0; i < " << n
           << "; ++i) x[i] = a.nodeset[i];\n"
           << "  } else {\n    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) x[i] = 0.0;\n  }\n";
    if (fp32_jac && !dfm) ld << "  #pragma unroll\n  for (int i = 0; i < " << n << "; ++i) xf[i] = spx_f(x[i]);\n";
    ld << "  it = 0; code = 1; spx_itlim = a.max_it; spx_it0 = 0; spx_cold = false;\n  }\n";
    o << ld.str();
    o << "  while (true) {\n    ++it;\n";
    if (dfm)
        o << "    spx_df F[" << n << "];\n    #pragma unroll\n    for (int i = 0; i < " << n
          << "; ++i) F[i] = spx_df{0.f, 0.f};\n";
    else
        o << "    double F[" << n << "];\n    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) F[i] = 0.0;\n";
    o << "    JT J[" << P.nnz << "];\n";
    emit_linear_jacobian(o, t, P);
    if (dfm)
        emit_elements_df(o, t, P, doff);
    else
        emit_elements(o, t, P, doff, true, fp32_jac);
    // factorisation over the static pattern
    o << "    bool sing = false;\n";
    for (int k = 0; k < n; ++k) {
        o << "    const JT iv" << k << " = (JT)1 / J[" << P.slot[k * n + k] << "];\n"
          << "    sing = sing || spx_bad(J[" << P.slot[k * n + k] << "], iv" << k << ");\n";
        for (int i = k + 1; i < n; ++i) {
            if (!P.has(i, k)) continue;
            const int lik = P.slot[i * n + k];
            o << "    J[" << lik << "] *= iv" << k << ";\n";
            for (int j = k + 1; j < n; ++j)
                if (P.has(k, j)) o << "    J[" << P.slot[i * n + j] << "] -= J[" << lik << "] * J[" << P.slot[k * n + j] << "];\n";
        }
    }
    // forward and back substitution on -F (rows permuted)
    o << "    JT y[" << n << "];\n";
    for (int i = 0; i < n; ++i) {
        if (dfm)
            o << "    y[" << i << "] = -__fadd_rn(F[" << P.perm[i] << "].h, F[" << P.perm[i] << "].l)";
        else
            o << "    y[" << i << "] = " << (fp32_jac ? "spx_fneg(F[" : "(JT)(-F[") << P.perm[i] << "])";
        for (int k = 0; k < i; ++k)
            if (P.has(i, k)) o << " - J[" << P.slot[i * n + k] << "] * y[" << k << "]";
        o << ";\n";
    }
    for (int i = n - 1; i >= 0; --i) {
        o << "    y[" << i << "] = (y[" << i << "]";
        for (int j = i + 1; j < n; ++j)
            if (P.has(i, j)) o << " - J[" << P.slot[i * n + j] << "] * y[" << j << "]";
        o << ") * iv" << i << ";\n";
    }
    o << "    bool conv = true;\n";
    for (int i = 0; i < n; ++i) {
        if (dfm)  // double-float update; the same test on the FP32 step and the high parts
            o << "    { const float xof = X[" << i << "].h; X[" << i << "] = spx_addf(X[" << i << "], y[" << i << "]);\n"
              << "      conv = conv && !(fabsf(y[" << i << "]) > reltolf * fmaxf(fabsf(X[" << i << "].h), fabsf(xof)) + "
              << (i < nn ? "vabstolf" : "iabstolf") << "); }\n";
        else if (fp32_jac)  // FP64 update; the test (newton.rs:134-159) on the FP32 step and shadows
            o << "    { double xn = x[" << i << "] + spx_d(y[" << i << "]); float xnf = spx_f(xn);\n"
              << "      conv = conv && !(fabsf(y[" << i << "]) > reltolf * fmaxf(fabsf(xnf), fabsf(xf[" << i
              << "])) + " << (i < nn ? "vabstolf" : "iabstolf") << ");\n      x[" << i << "] = xn; xf[" << i
              << "] = xnf; }\n";
        else
            o << "    { double xo = x[" << i << "], xn = xo + (double)y[" << i << "];\n"
              << "      conv = conv && !(fabs(xn - xo) > a.reltol * fmax(fabs(xn), fabs(xo)) + "
              << (i < nn ? "a.vabstol" : "a.iabstol") << ");\n      x[" << i << "] = xn; }\n";
    }
    o << "    code = sing ? 2 : (conv ? 0 : 1);\n"
      << "    if (sing || conv || it >= spx_itlim) {\n";
    // status, outputs, miss list, residual of sample s
    if (dfm)
        o << "    double x[" << n << "];\n    #pragma unroll\n    for (int i = 0; i < " << n
          << "; ++i) x[i] = (double)X[i].h + (double)X[i].l;\n";
    o << "    bool fin = true;\n    #pragma unroll\n    for (int i = 0; i < " << n
      << "; ++i) fin = fin && spx_fin(x[i]);\n"
      << "    unsigned char st8 = !fin ? 3 : (unsigned char)code;\n";
    // a warm start that missed restarts here from the nodeset (zero without
    // one) with the full iteration limit: the fallback chain's first stage
    // (warm -> cold), in this kernel's precision, without waiting for the
    // fallback launch, where one sample's serial FP64 Newton would take
    // longer than this whole kernel; the fallback kernel skips that stage
    // for samples whose status carries the cold flag
    o << "    if ((st8 & 15) != 0 && warm && !spx_cold && a.cold_max_it > 0) {\n"
      << "      spx_cold = true; spx_it0 = it; it = 0; spx_itlim = a.cold_max_it;\n";
    if (dfm)
        o << "      #pragma unroll\n      for (int i = 0; i < " << n
          << "; ++i) X[i] = spx_df{a.nodeset ? __double2float_rn(a.nodeset[i]) : 0.f, 0.f};\n";
    else {
        o << "      #pragma unroll\n      for (int i = 0; i < " << n << "; ++i) x[i] = a.nodeset ? a.nodeset[i] : 0.0;\n";
        if (fp32_jac) o << "      #pragma unroll\n      for (int i = 0; i < " << n << "; ++i) xf[i] = spx_f(x[i]);\n";
    }
    o << "      continue;\n    }\n"
      << "    if (warm) st8 |= spx_cold ? 0x30 : 0x10;\n"
      << "    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) a.x[s * " << n << " + i] = x[i];\n"
      << "    if (a.iters) a.iters[s] = spx_it0 + it;\n"
      << "    const bool spx_miss = (st8 & 15) != 0 && (warm || a.fallback_any);\n";
    if (dfm) {
        // parameters mode: the FP64 constants of a listed sample (for the generic
        // fallback) or of a residual, from the sample's parameters
        o << "    if (spx_miss || a.resid) {\n";
        for (int slot : pslots)
            o << "      const double pd" << slot << " = __ldg(a.lp + (u64)" << slot << " * a.lpstride + s);\n";
        emit_derive64(o, t, doff, pe, "      ");
        o << "    }\n";
    }
    o << "    if (spx_miss) {\n"
      << "      unsigned int k = atomicAdd(a.fail_count, 1u); a.fail_list[k] = (unsigned int)s;\n";
    if (dfm)
        for (int k = 0; k < t->num_derived; ++k) o << "      a.dvo[" << k << " * st + s] = c" << k << ";\n";
    o << "    } else if (a.resid) {\n"
      << "    double F[" << n << "];\n    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) F[i] = 0.0;\n";
    emit_elements(o, t, P, doff, false);
    o << "    double r = 0.0;\n";
    for (int i = 0; i < nn; ++i) o << "    r = fmax(r, fabs(F[" << i << "]));\n";
    o << "    a.resid[s] = r;\n    }\n    if (a.status) a.status[s] = st8;\n    spx_st = st8;\n";
    // next sample: warp-aggregated fetch from the counter
    o << "    {\n      const unsigned m = __activemask();\n      const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;\n"
      << "      u64 base = 0;\n      if (lane == lead) base = atomicAdd(a.next, (u64)__popc(m));\n"
      << "      base = __shfl_sync(m, base, lead);\n"
      << "      s = nthreads + base + (u64)__popc(m & ((1u << lane) - 1u));\n    }\n"
      << "    if (s >= a.count) break;\n";
    o << ld.str();
    o << "    }\n  }\n  }\n";
    // moments of the block's samples (the host enables this only when every
    // thread has exactly one sample, s = blockIdx.x * 128 + threadIdx.x): its
    // converged unknowns in shared memory, T threads per unknown (T the largest
    // power of two with T n <= 128) over 128 / T rows each in row order, then
    // the T partials in order: a fixed order, so the result does not depend on
    // scheduling
    int T = 1;
    while (T * 2 * n <= 128 && T < 32) T *= 2;
    const int R = 128 / T;
    o << "  if (a.mom) {\n"
      << "    __syncthreads();\n"
      << "    double* const xs = reinterpret_cast<double*>(spx_smem);\n"
      << "    unsigned char* const oks = spx_smem + 128 * " << n << " * 8;\n"
      << "    spx_mom* const pm = reinterpret_cast<spx_mom*>(spx_smem + 128 * " << n << " * 8 + 128);\n"
      << "    const u64 s0 = (u64)blockIdx.x * blockDim.x + threadIdx.x;\n"
      << "    const bool okm = s0 < a.count && (spx_st & 15) == 0;\n"
      << "    #pragma unroll\n    for (int i = 0; i < " << n << "; ++i) xs[threadIdx.x * " << n
      << " + i] = okm ? a.x[s0 * " << n << " + i] : 0.0;\n"
      << "    oks[threadIdx.x] = okm ? 1 : 0;\n"
      << "    __syncthreads();\n"
      << "    if (threadIdx.x < " << T * n << ") {\n"
      << "      const int col = threadIdx.x / " << T << ", q = threadIdx.x % " << T << ";\n"
      << "      u64 cnt = 0; double sm = 0.0, sq = 0.0;\n"
      << "      long long kmin = spx_key(__longlong_as_double(0x7ff0000000000000LL));\n"
      << "      long long kmax = spx_key(__longlong_as_double((long long)0xfff0000000000000ULL));\n"
      << "      for (int r = " << R << " * q; r < " << R << " * q + " << R << "; ++r) {\n"
      << "        if (!oks[r]) continue;\n"
      << "        const double v = xs[r * " << n << " + col];\n"
      << "        ++cnt; sm += v; sq += v * v;\n"
      << "        const long long k = spx_key(v); kmin = k < kmin ? k : kmin; kmax = k > kmax ? k : kmax;\n"
      << "      }\n"
      << "      pm[threadIdx.x] = spx_mom{cnt, sm, sq, spx_unkey(kmin), spx_unkey(kmax)};\n"
      << "    }\n"
      << "    __syncthreads();\n"
      << "    if (threadIdx.x < " << n << ") {\n"
      << "      spx_mom m = pm[threadIdx.x * " << T << "];\n"
      << "      for (int q = 1; q < " << T << "; ++q) {\n"
      << "        const spx_mom b = pm[threadIdx.x * " << T << " + q];\n"
      << "        m.count += b.count; m.sum += b.sum; m.sum_sq += b.sum_sq;\n"
      << "        m.mn = spx_key(b.mn) < spx_key(m.mn) ? b.mn : m.mn;\n"
      << "        m.mx = spx_key(b.mx) > spx_key(m.mx) ? b.mx : m.mx;\n"
      << "      }\n"
      << "      a.mom[(u64)threadIdx.x * gridDim.x + blockIdx.x] = m;\n"
      << "    }\n"
      << "  }\n"
      << "}\n";
    return o.str();
}

}  // namespace

struct SpecArgsHost {
    const double* dv;
    unsigned long long stride, count;
    const double* x0;
    const double* nodeset;
    double* x;
    int* iters;
    unsigned char* status;
    double* resid;
    unsigned int* fail_list;
    unsigned int* fail_count;
    double reltol, vabstol, iabstol;
    int max_it;
    int fallback_any;
    unsigned long long* next;
    // learned linear warm start (lw != nullptr): see NewtonLaunch
    const double* lp;
    unsigned long long lpstride;
    const float* lw;
    const float* lio;
    const int* lslots;
    int lnin;
    double* dvo;  // parameters mode: FP64 derived constants of the samples put on the miss list
    sp_moments* mom;  // per-block moments [n][grid] (one sample per thread), or nullptr
    int cold_max_it;  // iteration limit of the cold restart of a warm-start miss (0: none)
};

bool spec_params_mode(const sp_topology* t, int prec) { return prec == SP_PREC_MIXED && df_supported(t); }

// Build (once) the specialised kernel of topology t for `prec` (MIXED: FP32
// Jacobian; FP64: FP64 Jacobian).  Returns SP_OK or an error with the reason.
int spec_prepare(sp_topology* t, int prec, std::string& err) {
    const int slot = prec == SP_PREC_MIXED ? 0 : 1;
    if (t->spec_tried[slot]) {
        if (!t->spec_kernel[slot]) err = t->spec_log[slot];
        return t->spec_kernel[slot] ? SP_OK : SP_ERR_BACKEND;
    }
    t->spec_tried[slot] = true;
    for (const sp_element& el : t->h_elements)
        if (el.kind == SP_EL_BSIM3N || el.kind == SP_EL_BSIM3P) {
            t->spec_log[slot] = err = "BSIM3 elements run in the generic kernels";
            return SP_ERR_BACKEND;
        }
    // cache key: precision, sizes, element list, parameter specs, nodeset
    std::string key;
    key.push_back((char)slot);
    key.append((const char*)&t->num_nodes, sizeof(int));
    key.append((const char*)&t->num_branches, sizeof(int));
    key.append((const char*)t->h_elements.data(), sizeof(sp_element) * t->h_elements.size());
    key.append((const char*)t->h_params.data(), sizeof(sp_param) * t->h_params.size());
    key.append((const char*)t->h_nodeset.data(), sizeof(double) * t->h_nodeset.size());
    auto hit = t->ctx->spec_cache.find(key);
    if (hit != t->ctx->spec_cache.end()) {
        t->spec_kernel[slot] = hit->second.kernel;
        t->spec_log[slot] = hit->second.log;
        t->spec_nnz[slot] = hit->second.nnz;
        t->spec_bpsm[slot] = hit->second.blocks_per_sm;
        if (!t->spec_kernel[slot]) err = t->spec_log[slot];
        return t->spec_kernel[slot] ? SP_OK : SP_ERR_BACKEND;
    }
    sp_ctx::Spec& entry = t->ctx->spec_cache[key];
    Pattern P;
    std::string why;
    if (!plan(t, P, why)) {
        entry.log = t->spec_log[slot] = err = "no static pivot order: " + why;
        return SP_ERR_SOLVER;
    }
    entry.nnz = t->spec_nnz[slot] = P.nnz;
    std::string src = generate(t, P, prec == SP_PREC_MIXED);
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "spec_newton.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        entry.log = t->spec_log[slot] = err = "nvrtcCreateProgram failed";
        return SP_ERR_BACKEND;
    }
    const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "--fmad=true", "-lineinfo"};
    nvrtcResult r = nvrtcCompileProgram(prog, 4, opts);
    size_t logsz = 0;
    nvrtcGetProgramLogSize(prog, &logsz);
    std::string log(logsz, '\0');
    if (logsz) nvrtcGetProgramLog(prog, &log[0]);
    if (r != NVRTC_SUCCESS) {
        entry.log = t->spec_log[slot] = err = "NVRTC: " + log.substr(0, 2000);
        nvrtcDestroyProgram(&prog);
        return SP_ERR_BACKEND;
    }
    size_t cubin_sz = 0;
    nvrtcGetCUBINSize(prog, &cubin_sz);
    std::vector<char> cubin(cubin_sz);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    cudaKernel_t k = nullptr;
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&k, lib, "spec_newton");
    if (e != cudaSuccess) {
        entry.log = t->spec_log[slot] = err = std::string("module load: ") + cudaGetErrorString(e);
        return SP_ERR_BACKEND;
    }
    int bpsm = 0;
    const size_t smem = spec_smem_bytes(t, prec == SP_PREC_MIXED);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bpsm, (const void*)k, 128, smem) != cudaSuccess || bpsm < 1)
        bpsm = 1;
    entry.blocks_per_sm = t->spec_bpsm[slot] = bpsm;
    entry.lib = lib;
    entry.kernel = t->spec_kernel[slot] = k;
    entry.log = t->spec_log[slot] = log;
    return SP_OK;
}

cudaError_t spec_launch(const sp_topology* t, int prec, const NewtonLaunch& L, cudaStream_t st) {
    const int slot = prec == SP_PREC_MIXED ? 0 : 1;
    SpecArgsHost a{};
    a.dv = L.dv.p;
    a.stride = L.dv.stride;
    a.count = L.count;
    a.x0 = L.x0;
    a.nodeset = L.c.nodeset;
    a.x = L.x;
    a.iters = L.iters;
    a.status = L.status;
    a.resid = L.resid;
    a.fail_list = L.fail_list;
    a.fail_count = L.fail_count;
    a.reltol = L.cfg.v_reltol;
    a.vabstol = L.cfg.v_abstol;
    a.iabstol = L.cfg.i_abstol;
    a.max_it = L.cfg.max_iterations;
    // (the fallback kernel learns of the restart from the status byte)
    a.cold_max_it = (L.x0 || L.lin) && L.status ? L.cold_max_iterations : 0;
    a.fallback_any = (L.cfg.fallback & (SP_FALLBACK_GMIN | SP_FALLBACK_SOURCE)) ? 1 : 0;
    a.next = L.work_next;
    if (!a.next) return cudaErrorInvalidValue;
    a.lp = L.params ? L.params : L.lin_params;
    a.lpstride = L.params ? L.params_stride : L.lin_pstride;
    a.dvo = L.derived_out;
    a.mom = L.moments_partial;
    if (spec_params_mode(t, prec) && (!a.lp || !a.dvo)) return cudaErrorInvalidValue;
    a.lw = L.lin;
    a.lio = L.lin_io;
    a.lslots = L.lin_slots;
    a.lnin = L.lin_nin;
    // SpecLin: the linear term in the kernel's parameter order when its inputs
    // are ascending slots that the elements read (otherwise on = 0 and the
    // kernel reads the term from memory)
    const LinLayout ll = lin_layout(t, prec == SP_PREC_MIXED && df_supported(t));
    std::vector<unsigned long long> lkbuf((16 + 4 * (size_t)ll.nw + 7) / 8, 0ull);
    if (ll.usable && L.lin && L.lin_host && L.lin_io_host && L.lin_slots_host) {
        const int ps = (int)ll.slots.size(), n = t->n, nin = L.lin_nin;
        std::vector<int> at(nin, -1);
        bool ok = nin > 0;
        for (int j = 0; ok && j < nin; ++j) {
            ok = j == 0 || L.lin_slots_host[j] > L.lin_slots_host[j - 1];
            for (int k = 0; ok && k < ps; ++k)
                if (ll.slots[k] == L.lin_slots_host[j]) at[j] = k;
            ok = ok && at[j] >= 0;
        }
        if (ok) {
            unsigned long long mask = 0;
            float* w = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(lkbuf.data()) + 16);
            for (int j = 0; j < nin; ++j) {
                mask |= 1ull << at[j];
                for (int i = 0; i < n; ++i) w[at[j] * n + i] = L.lin_host[(size_t)i * nin + j];
                w[ps * n + at[j]] = L.lin_io_host[j];
            }
            for (int i = 0; i < n; ++i) w[ps * n + ps + i] = L.lin_io_host[2 * nin + i];
            lkbuf[0] = mask;
            reinterpret_cast<int*>(lkbuf.data())[2] = 1;
        }
    }
    void* args[] = {&a, lkbuf.data()};
    // tuned resident blocks per SM (setting "spec.bpsm.<precision>"), never above the occupancy limit
    int bpsm = t->spec_bpsm[slot];
    const int tb = tune_get(t->ctx, prec == SP_PREC_MIXED ? "spec.bpsm.mixed" : "spec.bpsm.fp64", t->n, 0);
    if (tb >= 1 && tb < bpsm) bpsm = tb;
    const uint64_t resident = (uint64_t)t->ctx->num_sms * (uint64_t)bpsm;
    const unsigned grid = (unsigned)std::min<uint64_t>((L.count + 127) / 128, resident);
    const size_t lin_bytes = L.lin ? sizeof(float) * ((size_t)t->n * L.lin_nin + 2 * (size_t)L.lin_nin + t->n) : 0;
    size_t smem = spec_smem_bytes(t, prec == SP_PREC_MIXED) + lin_bytes;
    if (L.moments_partial) {  // the moments epilogue reuses the block's shared memory
        if ((L.count + 127) / 128 > grid) return cudaErrorInvalidValue;  // needs one sample per thread
        smem = std::max(smem, (size_t)128 * t->n * 8 + 128 + (size_t)128 * sizeof(sp_moments));
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)t->spec_kernel[slot],
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    ChainedLaunch cl(dim3(grid), dim3(128), smem, st);
    return cudaLaunchKernelExC(&cl.cfg, (const void*)t->spec_kernel[slot], args);
}

bool spec_one_sample_per_thread(const sp_topology* t, int prec, uint64_t count) {
    const int slot = prec == SP_PREC_MIXED ? 0 : 1;
    int bpsm = t->spec_bpsm[slot];
    const int tb = tune_get(t->ctx, prec == SP_PREC_MIXED ? "spec.bpsm.mixed" : "spec.bpsm.fp64", t->n, 0);
    if (tb >= 1 && tb < bpsm) bpsm = tb;
    return (count + 127) / 128 <= (uint64_t)t->ctx->num_sms * (uint64_t)bpsm;
}

void spec_release_all(sp_ctx* ctx) {
    for (auto& kv : ctx->spec_cache)
        if (kv.second.lib) cudaLibraryUnload(kv.second.lib);
    ctx->spec_cache.clear();
}

}  // namespace sp

extern "C" int sp_specialize_source(const sp_circuit* c, int precision, int compile, char* src, size_t src_len,
                                    int* nnz) {
    using namespace sp;
    if (!c || (c->num_elements && !c->elements) || (c->num_params && !c->params)) return SP_ERR_INVALID_ARGUMENT;
    if (precision != SP_PREC_MIXED && precision != SP_PREC_FP64) return SP_ERR_INVALID_ARGUMENT;
    for (int e = 0; e < c->num_elements; ++e) {
        const sp_element& el = c->elements[e];
        if (el.kind < SP_EL_R || el.kind > SP_EL_PNP) return SP_ERR_INVALID_ARGUMENT;  // no BSIM3 here
        const int terms = terminal_count(el.kind);
        for (int k = 0; k < terms; ++k)
            if (el.node[k] < -1 || el.node[k] >= c->num_nodes) return SP_ERR_INVALID_DIMENSION;
        if (!element_slots_ok(el, c->num_params)) return SP_ERR_INVALID_DIMENSION;
        if ((el.kind == SP_EL_V || el.kind == SP_EL_L) && (el.branch < 0 || el.branch >= c->num_branches))
            return SP_ERR_INVALID_DIMENSION;
    }
    sp_topology t;
    t.num_nodes = c->num_nodes;
    t.num_branches = c->num_branches;
    t.n = c->num_nodes + c->num_branches;
    t.num_elements = c->num_elements;
    t.num_params = c->num_params;
    for (int e = 0; e < c->num_elements; ++e) t.num_derived += derived_count(c->elements[e].kind);
    t.h_elements.assign(c->elements, c->elements + c->num_elements);
    t.h_params.assign(c->params, c->params + c->num_params);
    if (c->nodeset) t.h_nodeset.assign(c->nodeset, c->nodeset + t.n);
    Pattern P;
    std::string why;
    auto put = [&](const std::string& s) {
        if (src && src_len) {
            std::strncpy(src, s.c_str(), src_len - 1);
            src[src_len - 1] = '\0';
        }
    };
    if (!plan(&t, P, why)) {
        put(why);
        return SP_ERR_SOLVER;
    }
    if (nnz) *nnz = P.nnz;
    std::string code = generate(&t, P, precision == SP_PREC_MIXED);
    put(code);
    if (!compile) return SP_OK;
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, code.c_str(), "spec_newton.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        return SP_ERR_BACKEND;
    const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "--fmad=true", "-lineinfo"};
    nvrtcResult r = nvrtcCompileProgram(prog, 4, opts);
    if (r != NVRTC_SUCCESS) {
        size_t logsz = 0;
        nvrtcGetProgramLogSize(prog, &logsz);
        std::string log(logsz, '\0');
        if (logsz) nvrtcGetProgramLog(prog, &log[0]);
        put(log);
    }
    nvrtcDestroyProgram(&prog);
    return r == NVRTC_SUCCESS ? SP_OK : SP_ERR_BACKEND;
}
