// Device-side interpretation of an sp_circuit: per-sample derived constants,
// device models and MNA stamping into a "sink".
//
// Every model follows its reference function operation for operation
// (paths relative to the Spicier repository), so that a translation unit
// compiled without FMA contraction reproduces the reference's IEEE results:
//   Level-1 MOSFET ...... crates/spicier-devices/src/mosfet/level1.rs:154-248
//   Shockley diode ...... crates/spicier-devices/src/diode.rs:41-148
//   Ebers-Moll BJT ...... crates/spicier-devices/src/bjt.rs:176-343
//   MNA stamps .......... crates/spicier-core/src/mna.rs:87-169
//
// Layout in HBM: all per-sample arrays are structure-of-arrays with the
// sample index fastest ("[slot][sample]"), so the 32 threads of a warp (32
// consecutive samples) read 32 consecutive doubles per slot.
#pragma once
#include <stdint.h>

#include "../../include/spicier_gb300.h"
#include "cr_math.cuh"

namespace sp {

// Number of derived per-sample constants an element kind keeps.
__host__ __device__ inline int derived_count(int kind) {
    switch (kind) {
        case SP_EL_D: return 3;     // is, nvt, vcrit
        case SP_EL_NMOS:
        case SP_EL_PMOS: return 3;  // vth, beta, lambda
        case SP_EL_NPN:
        case SP_EL_PNP: return 8;   // is, bf, br, nf_vt, nr_vt, vaf, vcrit_f, vcrit_r
        default: return 1;          // R: g = 1/R; C, L, V, I: value
    }
}

struct DevCircuit {
    int num_nodes, num_branches, n, num_elements, num_params, num_derived;
    const sp_element* el;    // [num_elements]
    const sp_param* par;     // [num_params]
    const sp_pulse* pulses;  // [num_pulses]
    const int* doff;         // [num_elements] offset of each element's derived block
    const double* nodeset;   // [n] or nullptr
};

// Thermal voltage at 300.15 K, k*T/q with CODATA constants (diode.rs:41-45).
__host__ __device__ inline double thermal_voltage_300() {
    const double K = 1.380649e-23;
    const double Q = 1.602176634e-19;
    return K * 300.15 / Q;
}

// nvt * ln(nvt / (sqrt(2) * 1e-14)) — the critical voltage of the diode
// limiter (diode.rs:139).  The saturation current in it is the literal 1e-14.
__host__ __device__ inline double diode_vcrit(double nvt) { return nvt * log(nvt / (1.4142135623730951 * 1e-14)); }

// diode.rs:138-148 with vcrit precomputed (the same value the reference
// recomputes on every call).
__host__ __device__ inline double limit_voltage(double vd, double nvt, double vcrit) {
    if (vd > vcrit) {
        double arg = (vd - vcrit) / nvt;
        return vcrit + nvt * (1.0 + log1p(arg));
    }
    return vd;
}

// Level-1 evaluate (level1.rs:154-191); vth = |VTO|, beta = KP*NF*W/L.
__host__ __device__ inline void mos_eval(bool pmos, double vth, double beta, double lambda, double vgs,
                                double vds, double& ids, double& gds, double& gm) {
    if (pmos) {
        vgs = -vgs;
        vds = -vds;
    }
    if (vgs < vth) {
        ids = 0.0;
        gds = 1e-12;
        gm = 0.0;
    } else if (vds < vgs - vth) {
        double vov = vgs - vth;
        double i = beta * (vov * vds - 0.5 * vds * vds) * (1.0 + lambda * vds);
        double g = beta * (vov - vds) * (1.0 + lambda * vds) +
                   beta * (vov * vds - 0.5 * vds * vds) * lambda;
        double m = beta * vds * (1.0 + lambda * vds);
        ids = pmos ? -i : i;
        gds = fmax(g, 1e-12);
        gm = m;
    } else {
        double vov = vgs - vth;
        double i = 0.5 * beta * vov * vov * (1.0 + lambda * vds);
        double g = 0.5 * beta * vov * vov * lambda;
        double m = beta * vov * (1.0 + lambda * vds);
        ids = pmos ? -i : i;
        gds = fmax(g, 1e-12);
        gm = m;
    }
}

// Derived per-sample constants of one element from its parameters
// (P(slot) -> value; out(k, value) stores derived constant k).  The same
// operation order as the reference's per-call computations, done once.
template <class PF, class OF>
__host__ __device__ inline void derive_element(const sp_element& el, PF P, OF out) {
    const double vt = thermal_voltage_300();
    switch (el.kind) {
        case SP_EL_R: out(0, ieee_div(1.0, P(el.field[0]))); break;  // passive.rs:48-50
        case SP_EL_D: {
            double nvt = P(el.field[1]) * vt;
            out(0, P(el.field[0]));
            out(1, nvt);
            out(2, diode_vcrit(nvt));
            break;
        }
        case SP_EL_NMOS:
        case SP_EL_PMOS: {
            // vth = |VTO| (level1.rs:164); beta = kp * nf * w / l (level1.rs:68-70)
            double kp = P(el.field[1]), w = P(el.field[3]), l = P(el.field[4]), nf = P(el.field[5]);
            out(0, fabs(P(el.field[0])));
            out(1, ieee_div(ieee_mul(ieee_mul(kp, nf), w), l));  // ((kp nf) w) / l
            out(2, P(el.field[2]));
            break;
        }
        case SP_EL_NPN:
        case SP_EL_PNP: {
            double nf_vt = P(el.field[3]) * vt, nr_vt = P(el.field[4]) * vt;
            out(0, P(el.field[0]));
            out(1, P(el.field[1]));
            out(2, P(el.field[2]));
            out(3, nf_vt);
            out(4, nr_vt);
            out(5, P(el.field[5]));
            out(6, diode_vcrit(nf_vt));
            out(7, diode_vcrit(nr_vt));
            break;
        }
        default: out(0, P(el.field[0])); break;  // C, L, V, I
    }
}

// Reader of per-sample SoA arrays.
struct SoA {
    const double* __restrict__ p;
    size_t stride;  // number of samples
    __host__ __device__ double operator()(int slot, size_t s) const {
#ifdef __CUDA_ARCH__
        return __ldg(p + (size_t)slot * stride + s);
#else
        return p[(size_t)slot * stride + s];
#endif
    }
};

// Mode of a stamping pass (Netlist::stamp_nonlinear_into, _scaled, + gmin).
enum StampMode { STAMP_PLAIN = 0, STAMP_GMIN = 1, STAMP_SCALED = 2 };

// Stamp every element linearised at the sink's current x.
// Sink API: double x(int i); void add(int r, int c, double v);
//           void rhs_add(int r, double v); void rhs_set(int r, double v).
template <class Sink>
__host__ __device__ inline void stamp_all(const DevCircuit& c, const SoA& dv, size_t s, Sink& k, int mode,
                                 double aux) {
    const bool scaled = (mode == STAMP_SCALED);
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element el = c.el[e];
        const int off = c.doff[e];
        const int n0 = el.node[0], n1 = el.node[1], n2 = el.node[2];
        switch (el.kind) {
            case SP_EL_R: {
                double g = dv(off, s);
                if (n0 >= 0) k.add(n0, n0, g);
                if (n1 >= 0) k.add(n1, n1, g);
                if (n0 >= 0 && n1 >= 0) {
                    k.add(n0, n1, -g);
                    k.add(n1, n0, -g);
                }
                break;
            }
            case SP_EL_C:
                break;
            case SP_EL_L:
            case SP_EL_V: {
                double v = (el.kind == SP_EL_L) ? 0.0 : dv(off, s);
                if (scaled && el.kind == SP_EL_V) v = v * aux;
                int row = c.num_nodes + el.branch;
                if (n0 >= 0) {
                    k.add(n0, row, 1.0);
                    k.add(row, n0, 1.0);
                }
                if (n1 >= 0) {
                    k.add(n1, row, -1.0);
                    k.add(row, n1, -1.0);
                }
                k.rhs_set(row, v);
                break;
            }
            case SP_EL_I: {
                double i = dv(off, s);
                if (scaled) i = i * aux;
                if (n0 >= 0) k.rhs_add(n0, -i);
                if (n1 >= 0) k.rhs_add(n1, i);
                break;
            }
            case SP_EL_D: {
                double vp = n0 >= 0 ? k.x(n0) : 0.0;
                double vn = n1 >= 0 ? k.x(n1) : 0.0;
                double vd = vp - vn;
                double is = dv(off, s), nvt = dv(off + 1, s), vcrit = dv(off + 2, s);
                double vl = limit_voltage(vd, nvt, vcrit);
                // evaluate() limits a second time (diode.rs:97, 118-121)
                double vl2 = limit_voltage(vl, nvt, vcrit);
                double ex = exp(vl2 / nvt);
                double id = is * (ex - 1.0);
                double gd = fmax(is * ex / nvt, 1e-12);
                double ieq = id - gd * vl;
                if (n0 >= 0) k.add(n0, n0, gd);
                if (n1 >= 0) k.add(n1, n1, gd);
                if (n0 >= 0 && n1 >= 0) {
                    k.add(n0, n1, -gd);
                    k.add(n1, n0, -gd);
                }
                if (n0 >= 0) k.rhs_add(n0, -ieq);
                if (n1 >= 0) k.rhs_add(n1, ieq);
                break;
            }
            case SP_EL_NMOS:
            case SP_EL_PMOS: {
                const int d = n0, g = n1, so = n2;
                double vg = g >= 0 ? k.x(g) : 0.0;
                double vd = d >= 0 ? k.x(d) : 0.0;
                double vs = so >= 0 ? k.x(so) : 0.0;
                double vgs = vg - vs, vds = vd - vs;
                double ids, gds, gm;
                mos_eval(el.kind == SP_EL_PMOS, dv(off, s), dv(off + 1, s), dv(off + 2, s), vgs, vds,
                         ids, gds, gm);
                if (d >= 0) k.add(d, d, gds);
                if (so >= 0) k.add(so, so, gds);
                if (d >= 0 && so >= 0) {
                    k.add(d, so, -gds);
                    k.add(so, d, -gds);
                }
                if (d >= 0) {
                    if (g >= 0) k.add(d, g, gm);
                    if (so >= 0) k.add(d, so, -gm);
                }
                if (so >= 0) {
                    if (g >= 0) k.add(so, g, -gm);
                    k.add(so, so, gm);
                }
                double ieq = ids - gds * vds - gm * vgs;
                if (d >= 0) k.rhs_add(d, -ieq);
                if (so >= 0) k.rhs_add(so, ieq);
                break;
            }
            case SP_EL_NPN:
            case SP_EL_PNP: {
                const int cn = n0, bn = n1, en = n2;
                const bool pnp = el.kind == SP_EL_PNP;
                double vb = bn >= 0 ? k.x(bn) : 0.0;
                double vc = cn >= 0 ? k.x(cn) : 0.0;
                double ve = en >= 0 ? k.x(en) : 0.0;
                double vbe = vb - ve, vce = vc - ve;
                double is = dv(off, s), bf = dv(off + 1, s), br = dv(off + 2, s);
                double nf_vt = dv(off + 3, s), nr_vt = dv(off + 4, s), vaf = dv(off + 5, s);
                double vcf = dv(off + 6, s), vcr = dv(off + 7, s);
                // stamp_linearized_at: limited vbe for the equivalent sources (bjt.rs:270-293)
                double vbe_int = pnp ? -vbe : vbe;
                double vbe_lim = limit_voltage(vbe_int, nf_vt, vcf);
                double vbe_ieq = pnp ? -vbe_lim : vbe_lim;
                // evaluate (bjt.rs:176-259)
                double sgn = 1.0, ve_be = vbe, ve_ce = vce;
                if (pnp) {
                    ve_be = -vbe;
                    ve_ce = -vce;
                    sgn = -1.0;
                }
                double vbc = ve_be - ve_ce;
                double vbe_l = limit_voltage(ve_be, nf_vt, vcf);
                double vbc_l = limit_voltage(vbc, nr_vt, vcr);
                double exp_be = exp(vbe_l / nf_vt);
                double exp_bc = exp(vbc_l / nr_vt);
                double i_f = is * (exp_be - 1.0);
                double i_r = is * (exp_bc - 1.0);
                bool vaf_fin = isfinite(vaf) && vaf > 0.0;
                double early = (vaf_fin && ve_ce > 0.0) ? 1.0 + ve_ce / vaf : 1.0;
                double ic = (i_f - i_r / br) * early;
                double ib = i_f / bf + i_r / br;
                double gmv = (i_f > 1e-20) ? (is * exp_be / nf_vt) * early : 1e-12;
                double gpi = gmv / bf;
                double go_e = (vaf_fin && fabs(ic) > 1e-20) ? fabs(ic) / vaf : 0.0;
                double gbc = is * exp_bc / nr_vt;
                double go_r = gbc / br * early;
                double go = fmax(go_e + go_r, 1e-12);
                ic = sgn * ic;
                ib = sgn * ib;
                double gm = fmax(gmv, 1e-12);
                gpi = fmax(gpi, 1e-12);
                go = fmax(go, 1e-12);
                // stamps (bjt.rs:295-329)
                if (bn >= 0) k.add(bn, bn, gpi);
                if (en >= 0) k.add(en, en, gpi);
                if (bn >= 0 && en >= 0) {
                    k.add(bn, en, -gpi);
                    k.add(en, bn, -gpi);
                }
                if (cn >= 0) k.add(cn, cn, go);
                if (en >= 0) k.add(en, en, go);
                if (cn >= 0 && en >= 0) {
                    k.add(cn, en, -go);
                    k.add(en, cn, -go);
                }
                if (cn >= 0) {
                    if (bn >= 0) k.add(cn, bn, gm);
                    if (en >= 0) k.add(cn, en, -gm);
                }
                if (en >= 0) {
                    if (bn >= 0) k.add(en, bn, -gm);
                    k.add(en, en, gm);
                }
                double ic_eq = ic - gm * vbe_ieq - go * vce;
                if (cn >= 0) k.rhs_add(cn, -ic_eq);
                if (en >= 0) k.rhs_add(en, ic_eq);
                double ib_eq = ib - gpi * vbe_ieq;
                if (bn >= 0) k.rhs_add(bn, -ib_eq);
                if (en >= 0) k.rhs_add(en, ib_eq);
                break;
            }
            default:
                break;
        }
    }
    if (mode == STAMP_GMIN)
        for (int i = 0; i < c.num_nodes; ++i) k.add(i, i, aux);  // mna.rs:164-168
}

}  // namespace sp
