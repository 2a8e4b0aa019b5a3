// Oracle core: FP64 CPU restatement of Spicier's Newton sweep path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU backend:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// it.  The product library never links it.
//
// Every function follows a reference function (paths relative to the Spicier
// repository) operation for operation, in the same evaluation order, so that
// with -ffp-contract=off it reproduces the reference's IEEE results.  The
// reference is Rust; Rust never contracts a*b+c into an FMA.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/spicier_gb300.h"
#include "../spicier_gb300/csrc/cr_math.cuh"
#include "bsim3.hpp"

namespace oracle {

// ---------------------------------------------------------------------------
// Hash RNG (crates/spicier-batched-sweep/src/rng.rs)
// ---------------------------------------------------------------------------

// rng.rs:39-44
inline uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

// rng.rs:51-56
inline uint64_t combine_indices(uint64_t seed, uint32_t sweep, uint32_t param) {
    return seed ^ ((uint64_t)sweep * 0x517cc1b727220a95ULL) ^
           ((uint64_t)param * 0x5851f42d4c957f2dULL);
}

// rng.rs:80-85
inline double uniform(uint64_t seed, uint32_t sweep, uint32_t param) {
    uint64_t h = splitmix64(combine_indices(seed, sweep, param));
    return (double)(h >> 11) * (1.0 / (double)(1ULL << 53));
}

// rng.rs:90-95
inline float uniform_f32(uint64_t seed, uint32_t sweep, uint32_t param) {
    uint64_t h = splitmix64(combine_indices(seed, sweep, param));
    return (float)(h >> 40) * (1.0f / (float)(1ULL << 24));
}

constexpr double PI = 3.14159265358979323846;  // std::f64::consts::PI

// ln and cos of the Gaussian draw.  Mode 0 (default): the host libm, as
// Rust's f64::ln/cos call it (glibc on Linux), i.e. the reference's own bits.
// Mode 1: the correctly rounded integer fixed-point functions the GPU kernels
// use (cr_math.cuh, pinned against 400-bit mpmath by the tests), which agree
// with glibc wherever glibc rounds correctly.
inline int& math_mode() {
    static int mode = 0;
    return mode;
}

// rng.rs:120-131
inline double gaussian(uint64_t seed, uint32_t sweep, uint32_t param) {
    double u1 = uniform(seed, sweep, param * 2u);
    double u2 = uniform(seed, sweep, param * 2u + 1u);
    u1 = std::fmax(u1, 1e-10);
    const double t = 2.0 * PI * u2;
    if (math_mode() == 1) return std::sqrt(-2.0 * sp::cr_log(u1, nullptr)) * sp::cr_cos(t, nullptr);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(t);
}

// rng.rs:138-145
inline float gaussian_f32(uint64_t seed, uint32_t sweep, uint32_t param) {
    float u1 = uniform_f32(seed, sweep, param * 2u);
    float u2 = uniform_f32(seed, sweep, param * 2u + 1u);
    u1 = std::fmax(u1, 1e-7f);
    return std::sqrt(-2.0f * std::log(u1)) * std::cos(2.0f * 3.14159265f * u2);
}

// rng.rs:148-150
inline double gaussian_scaled(uint64_t seed, uint32_t sweep, uint32_t param, double mean,
                              double sigma) {
    return mean + gaussian(seed, sweep, param) * sigma;
}

// One per-sample parameter (sp_draw_kind in spicier_gb300.h).
inline double draw_param(const sp_param& p, uint64_t seed, uint32_t sweep, const double* table_row) {
    switch (p.kind) {
        case SP_DRAW_FIXED: return p.a;
        case SP_DRAW_GAUSS: return gaussian_scaled(seed, sweep, p.rng_index, p.a, p.b);
        case SP_DRAW_UNIFORM: return p.a + uniform(seed, sweep, p.rng_index) * (p.b - p.a);
        case SP_DRAW_LOGUNIFORM:
            if (math_mode() == 1)
                return p.a * sp::cr_exp(uniform(seed, sweep, p.rng_index) * sp::cr_log(p.b / p.a, nullptr), nullptr);
            return p.a * std::exp(uniform(seed, sweep, p.rng_index) * std::log(p.b / p.a));
        case SP_DRAW_TABLE: return table_row ? table_row[p.rng_index] : NAN;
    }
    return NAN;
}

// ---------------------------------------------------------------------------
// Dense MNA accumulator (crates/spicier-core/src/mna.rs).  Entries are summed
// straight into a column-major dense matrix in stamping order, which is the
// same sequence of additions as to_dense_matrix over the triplet list
// (mna.rs:64-71).
// ---------------------------------------------------------------------------
struct Mna {
    int num_nodes = 0, num_branches = 0, n = 0;
    std::vector<double> A;  // column-major n*n
    std::vector<double> b;

    void init(int nn, int nb) {
        num_nodes = nn;
        num_branches = nb;
        n = nn + nb;
        A.assign((size_t)n * n, 0.0);
        b.assign(n, 0.0);
    }
    void clear() {  // mna.rs:47-50
        std::fill(A.begin(), A.end(), 0.0);
        std::fill(b.begin(), b.end(), 0.0);
    }
    void add(int r, int c, double v) { A[(size_t)c * n + r] += v; }
    // mna.rs:87-99
    void conductance(int i, int j, double g) {
        if (i >= 0) add(i, i, g);
        if (j >= 0) add(j, j, g);
        if (i >= 0 && j >= 0) {
            add(i, j, -g);
            add(j, i, -g);
        }
    }
    // mna.rs:104-116
    void current_source(int i, int j, double cur) {
        if (i >= 0) b[i] += -cur;
        if (j >= 0) b[j] += cur;
    }
    // mna.rs:125-146
    void voltage_source(int pos, int neg, int branch, double v) {
        int row = num_nodes + branch;
        if (pos >= 0) {
            add(pos, row, 1.0);
            add(row, pos, 1.0);
        }
        if (neg >= 0) {
            add(neg, row, -1.0);
            add(row, neg, -1.0);
        }
        b[row] = v;
    }
    // mna.rs:164-168
    void gmin(double g) {
        for (int i = 0; i < num_nodes; ++i) add(i, i, g);
    }
};

// ---------------------------------------------------------------------------
// Devices
// ---------------------------------------------------------------------------

// diode.rs:41-45
inline double thermal_voltage(double temp_k) {
    const double K = 1.380649e-23;
    const double Q = 1.602176634e-19;
    return K * temp_k / Q;
}

// diode.rs:138-148 (the same limiter is restated in bjt.rs:334-343)
inline double limit_voltage(double vd, double nvt) {
    double vcrit = nvt * std::log(nvt / (1.4142135623730951 * 1e-14));
    if (vd > vcrit) {
        double arg = (vd - vcrit) / nvt;
        return vcrit + nvt * (1.0 + std::log1p(arg));
    }
    return vd;
}

// diode.rs:91-106
inline void diode_evaluate(double is, double n, double vd, double* id, double* gd) {
    double vt = thermal_voltage(300.15);
    double nvt = n * vt;
    double vl = limit_voltage(vd, nvt);
    double e = std::exp(vl / nvt);
    *id = is * (e - 1.0);
    double g = is * e / nvt;
    *gd = std::fmax(g, 1e-12);
}

// MOSFET Level 1: mosfet/level1.rs:154-191.  Returns region 0 cutoff,
// 1 linear, 2 saturation.
struct MosParams {
    double vto, kp, lambda, w, l, nf;
    double beta() const { return kp * nf * w / l; }  // level1.rs:68-70
};

inline int mos_evaluate(bool pmos, const MosParams& p, double vgs, double vds, double* ids,
                        double* gds, double* gm) {
    if (pmos) {
        vgs = -vgs;
        vds = -vds;
    }
    double vth = std::fabs(p.vto);
    double beta = p.beta();
    double lambda = p.lambda;
    if (vgs < vth) {
        *ids = 0.0;
        *gds = 1e-12;
        *gm = 0.0;
        return 0;
    } else if (vds < vgs - vth) {
        double vov = vgs - vth;
        double i = beta * (vov * vds - 0.5 * vds * vds) * (1.0 + lambda * vds);
        double g = beta * (vov - vds) * (1.0 + lambda * vds) +
                   beta * (vov * vds - 0.5 * vds * vds) * lambda;
        double m = beta * vds * (1.0 + lambda * vds);
        *ids = pmos ? -i : i;
        *gds = std::fmax(g, 1e-12);
        *gm = m;
        return 1;
    } else {
        double vov = vgs - vth;
        double i = 0.5 * beta * vov * vov * (1.0 + lambda * vds);
        double g = 0.5 * beta * vov * vov * lambda;
        double m = beta * vov * (1.0 + lambda * vds);
        *ids = pmos ? -i : i;
        *gds = std::fmax(g, 1e-12);
        *gm = m;
        return 2;
    }
}

struct BjtParams {
    double is, bf, br, nf, nr, vaf;  // vaf <= 0 or inf: no Early effect
};

// bjt.rs:176-259.  Outputs ic, ib, ie, gm, gpi, go (already sign-applied / floored).
inline void bjt_evaluate(bool pnp, const BjtParams& p, double vbe, double vce, double out[6]) {
    double sign = 1.0;
    if (pnp) {
        vbe = -vbe;
        vce = -vce;
        sign = -1.0;
    }
    double vbc = vbe - vce;
    double vt = thermal_voltage(300.15);
    double nf_vt = p.nf * vt;
    double nr_vt = p.nr * vt;
    double vbe_l = limit_voltage(vbe, nf_vt);
    double vbc_l = limit_voltage(vbc, nr_vt);
    double exp_be = std::exp(vbe_l / nf_vt);
    double exp_bc = std::exp(vbc_l / nr_vt);
    double i_f = p.is * (exp_be - 1.0);
    double i_r = p.is * (exp_bc - 1.0);
    bool vaf_finite = std::isfinite(p.vaf) && p.vaf > 0.0;
    double early = (vaf_finite && vce > 0.0) ? 1.0 + vce / p.vaf : 1.0;
    double ic = (i_f - i_r / p.br) * early;
    double ie = i_f / p.bf + i_r;
    double ib = i_f / p.bf + i_r / p.br;
    double gm = (i_f > 1e-20) ? (p.is * exp_be / nf_vt) * early : 1e-12;
    double gpi = gm / p.bf;
    double go_early = (vaf_finite && std::fabs(ic) > 1e-20) ? std::fabs(ic) / p.vaf : 0.0;
    double gbc = p.is * exp_bc / nr_vt;
    double go_rev = gbc / p.br * early;
    double go = std::fmax(go_early + go_rev, 1e-12);
    out[0] = sign * ic;
    out[1] = sign * ib;
    out[2] = sign * ie;
    out[3] = std::fmax(gm, 1e-12);
    out[4] = std::fmax(gpi, 1e-12);
    out[5] = std::fmax(go, 1e-12);
}

inline double node_v(const double* x, int i) { return i >= 0 ? x[i] : 0.0; }

// Stamp every element linearised at x (Netlist::stamp_nonlinear_into,
// netlist.rs:441-445, or stamp_nonlinear_into_scaled, netlist.rs:452-461,
// when source_factor is given; scaled = false reproduces the unscaled stamps
// exactly).  P is the per-sample parameter vector.
inline void stamp_dc(const sp_circuit& c, const double* P, const double* x, Mna& m, bool scaled,
                     double source_factor) {
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element& el = c.elements[e];
        const int* nd = el.node;
        switch (el.kind) {
            case SP_EL_R:  // passive.rs:53-59
                m.conductance(nd[0], nd[1], 1.0 / P[el.field[0]]);
                break;
            case SP_EL_C:  // open at DC (passive.rs:232-240)
                break;
            case SP_EL_L:  // 0 V source at DC (passive.rs:318-325)
                m.voltage_source(nd[0], nd[1], el.branch, 0.0);
                break;
            case SP_EL_V: {  // sources.rs:96-101, 148-157
                double v = P[el.field[0]];
                m.voltage_source(nd[0], nd[1], el.branch, scaled ? v * source_factor : v);
                break;
            }
            case SP_EL_I: {  // sources.rs:230-236, 270-279
                double i = P[el.field[0]];
                m.current_source(nd[0], nd[1], scaled ? i * source_factor : i);
                break;
            }
            case SP_EL_D: {  // diode.rs:113-131, 191-200
                double vd = node_v(x, nd[0]) - node_v(x, nd[1]);
                double is = P[el.field[0]], n = P[el.field[1]];
                double nvt = n * thermal_voltage(300.15);
                double vl = limit_voltage(vd, nvt);
                double id, gd;
                diode_evaluate(is, n, vl, &id, &gd);
                double ieq = id - gd * vl;
                m.conductance(nd[0], nd[1], gd);
                m.current_source(nd[0], nd[1], ieq);
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS: {  // level1.rs:202-248, 291-305
                int d = nd[0], g = nd[1], s = nd[2];
                double vg = node_v(x, g), vd = node_v(x, d), vs = node_v(x, s);
                double vgs = vg - vs, vds = vd - vs;
                MosParams mp{P[el.field[0]], P[el.field[1]], P[el.field[2]],
                             P[el.field[3]], P[el.field[4]], P[el.field[5]]};
                double ids, gds, gm;
                mos_evaluate(el.kind == SP_EL_PMOS, mp, vgs, vds, &ids, &gds, &gm);
                m.conductance(d, s, gds);
                if (d >= 0) {
                    if (g >= 0) m.add(d, g, gm);
                    if (s >= 0) m.add(d, s, -gm);
                }
                if (s >= 0) {
                    if (g >= 0) m.add(s, g, -gm);
                    m.add(s, s, gm);
                }
                double ieq = ids - gds * vds - gm * vgs;
                m.current_source(d, s, ieq);
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {  // bjt.rs:268-330
                int cn = nd[0], bn = nd[1], en = nd[2];
                double vb = node_v(x, bn), vc = node_v(x, cn), ve = node_v(x, en);
                double vbe = vb - ve, vce = vc - ve;
                bool pnp = el.kind == SP_EL_PNP;
                BjtParams bp{P[el.field[0]], P[el.field[1]], P[el.field[2]],
                             P[el.field[3]], P[el.field[4]], P[el.field[5]]};
                double nf_vt = bp.nf * thermal_voltage(300.15);
                double vbe_int = pnp ? -vbe : vbe;
                double vbe_lim = limit_voltage(vbe_int, nf_vt);
                double vbe_ieq = pnp ? -vbe_lim : vbe_lim;
                double o[6];
                bjt_evaluate(pnp, bp, vbe, vce, o);
                double ic = o[0], ib = o[1], gm = o[3], gpi = o[4], go = o[5];
                m.conductance(bn, en, gpi);
                m.conductance(cn, en, go);
                if (cn >= 0) {
                    if (bn >= 0) m.add(cn, bn, gm);
                    if (en >= 0) m.add(cn, en, -gm);
                }
                if (en >= 0) {
                    if (bn >= 0) m.add(en, bn, -gm);
                    m.add(en, en, gm);
                }
                double ic_eq = ic - gm * vbe_ieq - go * vce;
                m.current_source(cn, en, ic_eq);
                double ib_eq = ib - gpi * vbe_ieq;
                m.current_source(bn, en, ib_eq);
                break;
            }
            case SP_EL_BSIM3N:
            case SP_EL_BSIM3P: {  // bsim3/mod.rs:176-227, 275-294: no limiting
                int d = nd[0], g = nd[1], s = nd[2], b = nd[3];
                const double* card = P + el.field[0];
                const bool cr = math_mode() == 1;
                const Bsim3Derived dv = bsim3_derive(card, cr);
                double vg = node_v(x, g), vd = node_v(x, d), vs = node_v(x, s), vb = node_v(x, b);
                double vgs = vg - vs, vds = vd - vs, vbs = vb - vs;
                const Bsim3Eval r = bsim3_evaluate(el.kind == SP_EL_BSIM3P, card, dv, vgs, vds, vbs, cr);
                m.conductance(d, s, r.gds);
                if (d >= 0) {
                    if (g >= 0) m.add(d, g, r.gm);
                    if (s >= 0) m.add(d, s, -r.gm);
                }
                if (s >= 0) {
                    if (g >= 0) m.add(s, g, -r.gm);
                    m.add(s, s, r.gm);
                }
                if (d >= 0) {
                    if (b >= 0) m.add(d, b, r.gmbs);
                    if (s >= 0) m.add(d, s, -r.gmbs);
                }
                if (s >= 0) {
                    if (b >= 0) m.add(s, b, -r.gmbs);
                    m.add(s, s, r.gmbs);
                }
                double ieq = r.ids - r.gds * vds - r.gm * vgs - r.gmbs * vbs;
                m.current_source(d, s, ieq);
                break;
            }
            default:
                break;
        }
    }
}

// ---------------------------------------------------------------------------
// Dense LU with partial pivoting, restating nalgebra 0.33 LU::new + solve
// (call site crates/spicier-solver/src/linear.rs:506): column icamax pivot
// (first maximum), multipliers scaled by 1/diag, column-oriented axpy
// updates, zero pivot skipped at factor time and reported as singular by the
// back substitution.  A is column-major and overwritten; b becomes x.
// Returns false when singular.
// ---------------------------------------------------------------------------
inline bool lu_solve(int n, double* A, double* b) {
    std::vector<int> swap_with(n, -1);
    for (int i = 0; i < n; ++i) {
        int piv = i;
        double best = std::fabs(A[(size_t)i * n + i]);
        for (int r = i + 1; r < n; ++r) {
            double v = std::fabs(A[(size_t)i * n + r]);
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        double diag = A[(size_t)i * n + piv];
        if (diag == 0.0) continue;
        if (piv != i) {
            swap_with[i] = piv;
            for (int c = 0; c < n; ++c) std::swap(A[(size_t)c * n + i], A[(size_t)c * n + piv]);
        }
        double inv = 1.0 / diag;
        for (int r = i + 1; r < n; ++r) A[(size_t)i * n + r] *= inv;
        for (int c = i + 1; c < n; ++c) {
            double p = A[(size_t)c * n + i];
            for (int r = i + 1; r < n; ++r)
                A[(size_t)c * n + r] = -p * A[(size_t)i * n + r] + A[(size_t)c * n + r];
        }
    }
    for (int i = 0; i < n; ++i)
        if (swap_with[i] >= 0) std::swap(b[i], b[swap_with[i]]);
    for (int i = 0; i < n; ++i) {
        double coeff = b[i];
        for (int r = i + 1; r < n; ++r) b[r] = -coeff * A[(size_t)i * n + r] + b[r];
    }
    for (int i = n - 1; i >= 0; --i) {
        double diag = A[(size_t)i * n + i];
        if (diag == 0.0) return false;
        double coeff = b[i] / diag;
        b[i] = coeff;
        for (int r = 0; r < i; ++r) b[r] = -coeff * A[(size_t)i * n + r] + b[r];
    }
    return true;
}

// ---------------------------------------------------------------------------
// Newton-Raphson (crates/spicier-solver/src/newton.rs)
// ---------------------------------------------------------------------------
struct NrOutcome {
    bool converged = false;
    bool singular = false;
    int iterations = 0;
};

// newton.rs:134-159
inline bool check_convergence(const double* old, const double* nw, int num_nodes, int n,
                              const sp_newton_config& c) {
    for (int i = 0; i < num_nodes; ++i) {
        double delta = std::fabs(nw[i] - old[i]);
        double tol = c.v_reltol * std::fmax(std::fabs(nw[i]), std::fabs(old[i])) + c.v_abstol;
        if (delta > tol) return false;
    }
    for (int i = num_nodes; i < n; ++i) {
        double delta = std::fabs(nw[i] - old[i]);
        double tol = c.v_reltol * std::fmax(std::fabs(nw[i]), std::fabs(old[i])) + c.i_abstol;
        if (delta > tol) return false;
    }
    return true;
}

enum class StampMode { Plain, Gmin, Scaled };

// newton.rs:70-131 (dense path; size < SPARSE_THRESHOLD = 50).  x holds the
// initial guess on entry and the last iterate on exit.  A singular system
// returns immediately (the reference propagates Err(SingularMatrix)).
inline NrOutcome newton(const sp_circuit& c, const double* P, const sp_newton_config& cfg,
                        StampMode mode, double aux, double* x, Mna& m) {
    NrOutcome out;
    int n = m.n;
    std::vector<double> xn(n);
    for (int it = 0; it < cfg.max_iterations; ++it) {
        m.clear();
        stamp_dc(c, P, x, m, mode == StampMode::Scaled, aux);
        if (mode == StampMode::Gmin) m.gmin(aux);
        std::copy(m.b.begin(), m.b.end(), xn.begin());
        if (!lu_solve(n, m.A.data(), xn.data())) {
            out.singular = true;
            out.iterations = it + 1;
            return out;
        }
        bool conv = check_convergence(x, xn.data(), c.num_nodes, n, cfg);
        std::copy(xn.begin(), xn.end(), x);
        if (conv) {
            out.converged = true;
            out.iterations = it + 1;
            return out;
        }
    }
    out.iterations = cfg.max_iterations;
    return out;
}

struct SteppingOutcome {
    bool converged = false;
    bool singular = false;
    int total_iterations = 0;
    int num_levels = 0;
};

// newton.rs:373-459.  x: solution (starts at zero as in the reference).
inline SteppingOutcome gmin_stepping(const sp_circuit& c, const double* P,
                                     const sp_newton_config& cfg, double* x, Mna& m) {
    SteppingOutcome out;
    int n = m.n;
    std::vector<double> sol(n, 0.0), trial(n);
    double g = cfg.gmin_initial;
    while (g >= cfg.gmin_final * 0.99) {
        int attempts = 0;
        bool level_ok = false;
        while (attempts < cfg.gmin_max_attempts && !level_ok) {
            trial = sol;
            NrOutcome r = newton(c, P, cfg, StampMode::Gmin, g, trial.data(), m);
            out.total_iterations += r.iterations;
            if (r.singular) {
                out.singular = true;
                std::copy(sol.begin(), sol.end(), x);
                return out;
            }
            if (r.converged) {
                sol = trial;
                level_ok = true;
            } else {
                attempts += 1;
            }
        }
        if (!level_ok) {
            std::copy(sol.begin(), sol.end(), x);
            return out;
        }
        out.num_levels += 1;
        if (g <= cfg.gmin_final) break;
        g /= cfg.gmin_reduction;
        if (g < cfg.gmin_final) g = cfg.gmin_final;
    }
    out.converged = true;
    std::copy(sol.begin(), sol.end(), x);
    return out;
}

// newton.rs:261-356
inline SteppingOutcome source_stepping(const sp_circuit& c, const double* P,
                                       const sp_newton_config& cfg, double* x, Mna& m) {
    SteppingOutcome out;
    int n = m.n;
    std::vector<double> sol(n, 0.0), trial(n);
    double factor = cfg.src_initial;
    double step = cfg.src_step;
    while (factor <= 1.0 + 1e-9) {
        double cur = std::fmin(factor, 1.0);
        int attempts = 0;
        bool level_ok = false;
        while (attempts < cfg.src_max_attempts && !level_ok) {
            trial = sol;
            NrOutcome r = newton(c, P, cfg, StampMode::Scaled, cur, trial.data(), m);
            out.total_iterations += r.iterations;
            if (r.singular) {
                out.singular = true;
                std::copy(sol.begin(), sol.end(), x);
                return out;
            }
            if (r.converged) {
                sol = trial;
                level_ok = true;
            } else {
                attempts += 1;
            }
        }
        if (!level_ok) {
            if (step > cfg.src_min_step) {
                step /= 2.0;
                factor -= step;
                continue;
            }
            std::copy(sol.begin(), sol.end(), x);
            return out;
        }
        out.num_levels += 1;
        if (std::fabs(cur - 1.0) < 1e-9) break;
        factor += step;
        if (step < cfg.src_step && level_ok) step = std::fmin(step * 1.5, cfg.src_step);
    }
    out.converged = true;
    std::copy(sol.begin(), sol.end(), x);
    return out;
}

inline bool all_finite(const double* x, int n) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(x[i])) return false;
    return true;
}

// The per-sample DC pipeline a Spicier user runs: Newton from the guess (or
// zero); on a miss, Newton from zero when a guess was used; then gmin
// stepping, then source stepping, as enabled by cfg.fallback.  Returns the
// sp_sample_status byte; *iters is the total Newton iteration count.
// A stage succeeds only if it converged with a finite iterate: the
// reference's check_convergence passes a NaN iterate (every comparison with
// NaN is false), which would otherwise end the chain on a NaN "solution".
inline uint8_t dc_pipeline(const sp_circuit& c, const double* P, const sp_newton_config& cfg,
                           const double* x0, double* x, int* iters, Mna& m) {
    int n = c.num_nodes + c.num_branches;
    int total = 0;
    uint8_t flags = 0;
    bool last_singular = false;
    // Start: the warm start, else the circuit's nodeset, else zero.
    auto cold_start = [&] {
        if (c.nodeset) std::copy(c.nodeset, c.nodeset + n, x);
        else std::fill(x, x + n, 0.0);
    };
    sp_newton_config first = cfg;  // the warm attempt may have its own cap
    if (x0) {
        std::copy(x0, x0 + n, x);
        flags |= SP_ST_FLAG_WARM;
        if (cfg.warm_max_iterations > 0 && cfg.warm_max_iterations < cfg.max_iterations)
            first.max_iterations = cfg.warm_max_iterations;
    } else {
        cold_start();
    }
    NrOutcome r = newton(c, P, first, StampMode::Plain, 0.0, x, m);
    total += r.iterations;
    last_singular = r.singular;
    bool ok = r.converged && all_finite(x, n);
    if (!ok && x0) {
        flags |= SP_ST_FLAG_COLD;
        cold_start();
        r = newton(c, P, cfg, StampMode::Plain, 0.0, x, m);
        total += r.iterations;
        last_singular = r.singular;
        ok = r.converged && all_finite(x, n);
    }
    if (!ok && (cfg.fallback & SP_FALLBACK_GMIN)) {
        flags |= SP_ST_FLAG_GMIN;
        SteppingOutcome s = gmin_stepping(c, P, cfg, x, m);
        total += s.total_iterations;
        last_singular = s.singular;
        ok = s.converged && all_finite(x, n);
    }
    if (!ok && (cfg.fallback & SP_FALLBACK_SOURCE)) {
        flags |= SP_ST_FLAG_SOURCE;
        SteppingOutcome s = source_stepping(c, P, cfg, x, m);
        total += s.total_iterations;
        last_singular = s.singular;
        ok = s.converged && all_finite(x, n);
    }
    *iters = total;
    uint8_t st;
    if (!all_finite(x, n)) st = SP_ST_NONFINITE;
    else if (ok) st = SP_ST_CONVERGED;
    else st = last_singular ? SP_ST_SINGULAR : SP_ST_FAILED;
    return st | flags;
}

}  // namespace oracle
