// Oracle (test infrastructure, never the product path): batched AC
// small-signal sweeps from each sample's DC operating point.
//
// Restates crates/spicier-solver/src/ac.rs (generate_frequencies :258-287,
// ComplexMna stamps :121-240, solve_ac :357-400 with the dense complex LU of
// linear.rs:557-583, nalgebra 0.33 LU on num_complex numbers) and the
// netlist AC stamper crates/spicier-cli/src/stampers.rs:94-330 with the
// devices' ac_info / ac_info_at (sources.rs:135-142, 258-264; diode.rs:202-220;
// mosfet/level1.rs:307-331; bjt.rs:404-427):
//   R: conductance; C: admittance j w C; L: branch with -j w L on its diagonal;
//   V: branch, right-hand side = AC magnitude (ac_info gives every voltage
//   source magnitude 1; here `source` = -1 keeps that, an element index makes
//   that source the only stimulus); I: no AC stimulus (ac_mag 0);
//   D: gd at the operating point; MOSFET: gds and the gm VCCS; BJT: gpi, go
//   and the gm VCCS (evaluate at the operating point, no limiting beyond
//   what evaluate does); BSIM3 (mosfet/bsim3/mod.rs:296-342, stamper
//   stampers.rs:423-470): gds, the gm and gmbs VCCSs, and j w C for each of
//   Cgs (g, s), Cgd (g, d), Cgb (g, b), Cbs (b, s), Cbd (b, d) that is > 0.
#pragma once
#include <cmath>
#include <complex>
#include <vector>

#include "oracle_core.hpp"

namespace oracle {

struct Cx {
    double re, im;
};
// num_complex 0.4 operation order
inline Cx cmul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cx cadd(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
inline Cx cdiv(Cx a, Cx b) {
    const double ns = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / ns, (a.im * b.re - a.re * b.im) / ns};
}
inline Cx cneg(Cx a) { return {-a.re, -a.im}; }
inline double norm1(Cx a) { return std::fabs(a.re) + std::fabs(a.im); }

// ac.rs:258-287
inline std::vector<double> ac_frequencies(double fstart, double fstop, int num_points, int sweep) {
    std::vector<double> f;
    if (sweep == 0) {
        if (num_points <= 1) return {fstart};
        const double step = (fstop - fstart) / ((double)num_points - 1.0);
        for (int i = 0; i < num_points; ++i) f.push_back(fstart + step * (double)i);
        return f;
    }
    const double base = sweep == 1 ? 10.0 : 2.0;
    const double span = sweep == 1 ? std::log10(fstop / fstart) : std::log2(fstop / fstart);
    const long total = (long)std::ceil((double)num_points * span) + 1;
    for (long i = 0; i < total; ++i) {
        const double v = fstart * std::pow(base, (double)i / (double)num_points);
        if (v <= fstop * 1.001) f.push_back(v);
    }
    return f;
}

// nalgebra LU (column icamax on norm1, zero pivot skipped) and LU::solve,
// column-major A (n x n), b overwritten by x; false when singular.
inline bool lu_solve_complex(int n, Cx* A, Cx* b) {
    std::vector<int> swap_with(n, -1);
    for (int i = 0; i < n; ++i) {
        int piv = i;
        double best = norm1(A[(size_t)i * n + i]);
        for (int r = i + 1; r < n; ++r) {
            const double v = norm1(A[(size_t)i * n + r]);
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        const Cx diag = A[(size_t)i * n + piv];
        if (diag.re == 0.0 && diag.im == 0.0) continue;
        if (piv != i) {
            swap_with[i] = piv;
            for (int c = 0; c < n; ++c) std::swap(A[(size_t)c * n + i], A[(size_t)c * n + piv]);
        }
        const Cx inv = cdiv({1.0, 0.0}, diag);
        for (int r = i + 1; r < n; ++r) A[(size_t)i * n + r] = cmul(A[(size_t)i * n + r], inv);
        for (int c = i + 1; c < n; ++c) {
            const Cx p = cneg(A[(size_t)c * n + i]);
            for (int r = i + 1; r < n; ++r)
                A[(size_t)c * n + r] = cadd(cmul(p, A[(size_t)i * n + r]), A[(size_t)c * n + r]);
        }
    }
    for (int i = 0; i < n; ++i)
        if (swap_with[i] >= 0) std::swap(b[i], b[swap_with[i]]);
    for (int i = 0; i < n; ++i) {
        const Cx coeff = cneg(b[i]);
        for (int r = i + 1; r < n; ++r) b[r] = cadd(cmul(coeff, A[(size_t)i * n + r]), b[r]);
    }
    for (int i = n - 1; i >= 0; --i) {
        const Cx diag = A[(size_t)i * n + i];
        if (diag.re == 0.0 && diag.im == 0.0) return false;
        const Cx coeff = cdiv(b[i], diag);
        b[i] = coeff;
        const Cx nc = cneg(coeff);
        for (int r = 0; r < i; ++r) b[r] = cadd(cmul(nc, A[(size_t)i * n + r]), b[r]);
    }
    return true;
}

// Small-signal stamps at the operating point x into the real part G (the
// frequency-independent conductances) and the AC right-hand side; the
// reactive terms are added per frequency by ac_matrix.
struct AcLinear {
    int n = 0;
    std::vector<double> G;  // column-major, real
    std::vector<double> rhs;
    std::vector<double> caps;  // BSIM3 elements: cgs, cgd, cgb, cbs, cbd at element index * 5
};

inline AcLinear ac_linearise(const sp_circuit& c, const double* P, const double* x, int source) {
    AcLinear L;
    const int nn = c.num_nodes;
    L.n = nn + c.num_branches;
    L.G.assign((size_t)L.n * L.n, 0.0);
    L.rhs.assign(L.n, 0.0);
    L.caps.assign((size_t)c.num_elements * 5, 0.0);
    auto add = [&](int r, int col, double v) {
        if (r >= 0 && col >= 0) L.G[(size_t)col * L.n + r] += v;
    };
    auto cond = [&](int i, int j, double g) {
        add(i, i, g), add(j, j, g), add(i, j, -g), add(j, i, -g);
    };
    auto vccs = [&](int op, int on, int cp, int cn, double gm) {
        add(op, cp, gm), add(op, cn, -gm), add(on, cp, -gm), add(on, cn, gm);
    };
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element& el = c.elements[e];
        const int* nd = el.node;
        switch (el.kind) {
            case SP_EL_R: cond(nd[0], nd[1], 1.0 / P[el.field[0]]); break;
            case SP_EL_V:
            case SP_EL_L: {
                const int br = nn + el.branch;
                add(nd[0], br, 1.0), add(br, nd[0], 1.0), add(nd[1], br, -1.0), add(br, nd[1], -1.0);
                if (el.kind == SP_EL_V && (source < 0 || source == e)) L.rhs[br] += 1.0;
                break;
            }
            case SP_EL_D: {
                const double vd = node_v(x, nd[0]) - node_v(x, nd[1]);
                double id, gd;
                diode_evaluate(P[el.field[0]], P[el.field[1]], vd, &id, &gd);
                cond(nd[0], nd[1], gd);
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS: {
                const int d = nd[0], g = nd[1], s = nd[2];
                const double vgs = node_v(x, g) - node_v(x, s), vds = node_v(x, d) - node_v(x, s);
                MosParams mp{P[el.field[0]], P[el.field[1]], P[el.field[2]],
                             P[el.field[3]], P[el.field[4]], P[el.field[5]]};
                double ids, gds, gm;
                mos_evaluate(el.kind == SP_EL_PMOS, mp, vgs, vds, &ids, &gds, &gm);
                cond(d, s, gds);
                vccs(d, s, g, s, gm);
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {
                const int cn = nd[0], bn = nd[1], en = nd[2];
                const double vbe = node_v(x, bn) - node_v(x, en), vce = node_v(x, cn) - node_v(x, en);
                BjtParams bp{P[el.field[0]], P[el.field[1]], P[el.field[2]],
                             P[el.field[3]], P[el.field[4]], P[el.field[5]]};
                double o[6];
                bjt_evaluate(el.kind == SP_EL_PNP, bp, vbe, vce, o);
                cond(bn, en, o[4]);
                cond(cn, en, o[5]);
                vccs(cn, en, bn, en, o[3]);
                break;
            }
            case SP_EL_BSIM3N:
            case SP_EL_BSIM3P: {
                const int d = nd[0], g = nd[1], s = nd[2], b = nd[3];
                const bool pm = el.kind == SP_EL_BSIM3P;
                const double* card = P + el.field[0];
                const bool cr = math_mode() == 1;
                const Bsim3Derived dv = bsim3_derive(card, cr);
                const double vgs = node_v(x, g) - node_v(x, s), vds = node_v(x, d) - node_v(x, s);
                const double vbs = node_v(x, b) - node_v(x, s);
                const Bsim3Eval r = bsim3_evaluate(pm, card, dv, vgs, vds, vbs, cr);
                cond(d, s, r.gds);
                vccs(d, s, g, s, r.gm);
                vccs(d, s, b, s, r.gmbs);
                bsim3_capacitances(pm, card, dv, vds, vbs, r.region, &L.caps[(size_t)e * 5]);
                break;
            }
            default:
                break;
        }
    }
    return L;
}

// The complex MNA matrix at angular frequency w (column-major).
inline void ac_matrix(const sp_circuit& c, const double* P, const AcLinear& L, double w, Cx* A, Cx* b) {
    const int n = L.n, nn = c.num_nodes;
    for (size_t k = 0; k < (size_t)n * n; ++k) A[k] = {L.G[k], 0.0};
    for (int i = 0; i < n; ++i) b[i] = {L.rhs[i], 0.0};
    auto addc = [&](int r, int col, double im) {
        if (r >= 0 && col >= 0) A[(size_t)col * n + r].im += im;
    };
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element& el = c.elements[e];
        if (el.kind == SP_EL_C) {
            const double y = w * P[el.field[0]];
            const int i = el.node[0], j = el.node[1];
            addc(i, i, y), addc(j, j, y), addc(i, j, -y), addc(j, i, -y);
        } else if (el.kind == SP_EL_L) {
            const int br = nn + el.branch;
            A[(size_t)br * n + br].im -= w * P[el.field[0]];
        } else if (el.kind == SP_EL_BSIM3N || el.kind == SP_EL_BSIM3P) {
            const int d = el.node[0], g = el.node[1], s = el.node[2], b = el.node[3];
            const int pr[5][2] = {{g, s}, {g, d}, {g, b}, {b, s}, {b, d}};
            for (int k = 0; k < 5; ++k) {
                const double cap = L.caps[(size_t)e * 5 + k];
                if (!(cap > 0.0)) continue;
                const double y = w * cap;
                const int i = pr[k][0], j = pr[k][1];
                addc(i, i, y), addc(j, j, y), addc(i, j, -y), addc(j, i, -y);
            }
        }
    }
}

}  // namespace oracle
