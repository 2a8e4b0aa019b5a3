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
        case SP_EL_BSIM3N:
        case SP_EL_BSIM3P: return 37;  // Bsim3Const (B3C_COUNT)
        default: return 1;          // R: g = 1/R; C, L, V, I: value
    }
}

// Terminals of an element kind (node[0..terms-1]).
__host__ __device__ inline int terminal_count(int kind) {
    return kind >= SP_EL_BSIM3N ? 4 : (kind >= SP_EL_NMOS ? 3 : 2);
}

// Whether every parameter slot the element reads lies in [0, num_params):
// fields 0..k-1 of the kind, or the SP_B3_CARD slots from field[0] of a BSIM3.
__host__ __device__ inline bool element_slots_ok(const sp_element& el, int num_params) {
    if (el.kind == SP_EL_BSIM3N || el.kind == SP_EL_BSIM3P)
        return el.field[0] >= 0 && el.field[0] <= num_params - SP_B3_CARD;
    const int nf = el.kind == SP_EL_D ? 2 : (el.kind >= SP_EL_NMOS ? 6 : 1);
    for (int f = 0; f < nf; ++f)
        if (el.field[f] < 0 || el.field[f] >= num_params) return false;
    return true;
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

// ---------------------------------------------------------------------------
// BSIM3v3.3 DC model (the reference's "BSIM3-lite"):
//   derived values ....... crates/spicier-devices/src/mosfet/bsim3/derived.rs:81-196
//   evaluate ............. crates/spicier-devices/src/mosfet/bsim3/evaluate.rs:171-598
//   stamps ............... crates/spicier-devices/src/mosfet/bsim3/mod.rs:176-227
// Everything that does not depend on the bias (the derived values at TNOM and
// the length / width factors of the threshold) is computed once per sample
// into these constants, in the reference's operation order, so that the
// per-iteration evaluation repeats only the bias-dependent operations.
enum Bsim3Const {
    B3C_VTH0ABS = 0, B3C_K1, B3C_K2, B3C_PHI, B3C_SQRTPHI,
    B3C_SCE,       // (-DVT0 theta) vt
    B3C_DVT2, B3C_NWE_ON, B3C_K3TW, B3C_K3B, B3C_WEFF,
    B3C_SCEW,      // (-DVT0W theta_w) vt
    B3C_DVT2W, B3C_ETA0, B3C_ETAB, B3C_THETA_DIBL, B3C_KT2,
    B3C_NVT, B3C_I0, B3C_VT, B3C_C32, B3C_TOX, B3C_UA, B3C_UC, B3C_UB, B3C_U0SI,
    B3C_SCEF,      // 1 - 0.3 min(lt / leff, 1)
    B3C_VSAT, B3C_LEFF,
    B3C_VABASE,    // leff (2 vsat / u0_si) 4 / max(pclm, 0.1)
    B3C_PDIBLC1, B3C_PDIBLCB, B3C_PDIBLC2, B3C_DROUT, B3C_PVAG,
    B3C_WL,        // weff / leff
    B3C_COX,
    B3C_COUNT
};

// Per-sample constants from the card (C(k) = slot k of sp_bsim3_card).  The
// logarithm and exponentials are the correctly rounded ones, so these
// constants do not depend on a math library.
template <class CF, class OF>
__host__ __device__ inline void bsim3_constants(CF C, OF out) {
    const double Q = 1.602176634e-19, KB = 1.380649e-23;
    const double EPS_SI = 1.03594e-10, EPS_OX = 3.45314e-11, NI = 1.45e10;
    const double tox = C(SP_B3_TOX);
    const double leff = C(SP_B3_L) - 2.0 * C(SP_B3_LINT);
    const double weff = (C(SP_B3_W) - 2.0 * C(SP_B3_WINT)) * C(SP_B3_NF);
    const double cox = EPS_OX / tox;
    const double vt = KB * C(SP_B3_TNOM) / Q;
    const double phi = 2.0 * vt * cr_log(C(SP_B3_NCH) / NI, nullptr);
    const double sqrt_phi = sqrt(phi);
    const double u0_si = C(SP_B3_U0) * 1e-4;
    const double xdep = sqrt(2.0 * EPS_SI * phi / (Q * C(SP_B3_NCH) * 1e6));
    const double lt = sqrt(EPS_SI * xdep * tox / EPS_OX);
    // calc_threshold's length and width factors
    const double lt_ratio = C(SP_B3_DVT1) * leff / (2.0 * lt);
    const double e1 = cr_exp(-fmin(lt_ratio, 20.0), nullptr);
    const double theta = e1 / (1.0 + 2.0 * e1);
    const double wt = sqrt(EPS_SI * tox / EPS_OX);
    const double wt_ratio = C(SP_B3_DVT1W) * weff / (2.0 * wt + C(SP_B3_W0));
    const double ew = cr_exp(-fmin(wt_ratio, 20.0), nullptr);
    const double theta_w = ew / (1.0 + 2.0 * ew);
    const double dibl_ratio = C(SP_B3_DSUB) * leff / (2.0 * lt);
    const double nvt = C(SP_B3_NFACTOR) * vt;
    const double vth0_abs = fabs(C(SP_B3_VTH0));
    out(B3C_VTH0ABS, vth0_abs);
    out(B3C_K1, C(SP_B3_K1));
    out(B3C_K2, C(SP_B3_K2));
    out(B3C_PHI, phi);
    out(B3C_SQRTPHI, sqrt_phi);
    out(B3C_SCE, -C(SP_B3_DVT0) * theta * vt);
    out(B3C_DVT2, C(SP_B3_DVT2));
    out(B3C_NWE_ON, weff > 1e-9 ? 1.0 : 0.0);
    out(B3C_K3TW, C(SP_B3_K3) * (tox / weff));
    out(B3C_K3B, C(SP_B3_K3B));
    out(B3C_WEFF, weff);
    out(B3C_SCEW, -C(SP_B3_DVT0W) * theta_w * vt);
    out(B3C_DVT2W, C(SP_B3_DVT2W));
    out(B3C_ETA0, C(SP_B3_ETA0));
    out(B3C_ETAB, C(SP_B3_ETAB));
    out(B3C_THETA_DIBL, cr_exp(-fmin(dibl_ratio, 20.0), nullptr));
    out(B3C_KT2, C(SP_B3_KT2));
    out(B3C_NVT, nvt);
    out(B3C_I0, (weff / leff) * u0_si * cox * nvt * nvt);
    out(B3C_VT, vt);
    out(B3C_C32, 3.2 * vth0_abs);
    out(B3C_TOX, tox);
    out(B3C_UA, C(SP_B3_UA));
    out(B3C_UC, C(SP_B3_UC));
    out(B3C_UB, C(SP_B3_UB));
    out(B3C_U0SI, u0_si);
    out(B3C_SCEF, 1.0 - 0.3 * fmin(lt / leff, 1.0));
    out(B3C_VSAT, C(SP_B3_VSAT));
    out(B3C_LEFF, leff);
    out(B3C_VABASE, leff * (2.0 * C(SP_B3_VSAT) / u0_si) * 4.0 / fmax(C(SP_B3_PCLM), 0.1));
    out(B3C_PDIBLC1, C(SP_B3_PDIBLC1));
    out(B3C_PDIBLCB, C(SP_B3_PDIBLCB));
    out(B3C_PDIBLC2, C(SP_B3_PDIBLC2));
    out(B3C_DROUT, C(SP_B3_DROUT));
    out(B3C_PVAG, C(SP_B3_PVAG));
    out(B3C_WL, weff / leff);
    out(B3C_COX, cox);
}

struct Bsim3Out {
    double ids, gds, gm, gmbs, vth, vdsat;
    int region;  // 0 subthreshold, 1 linear, 2 saturation
};

// f64::clamp: bounds applied in turn, NaN kept.
__host__ __device__ inline double rs_clamp(double x, double lo, double hi) {
    x = x < lo ? lo : x;
    return x > hi ? hi : x;
}

// Bsim3Mosfet::evaluate at terminal voltages (vgs, vds, vbs); K(i) reads
// constant i of Bsim3Const.
template <class KF>
__host__ __device__ inline Bsim3Out bsim3_eval(bool pmos, KF K, double vgs, double vds, double vbs) {
    Bsim3Out r;
    double sign = 1.0;
    if (pmos) {
        vgs = -vgs;
        vds = -vds;
        vbs = -vbs;
        sign = -1.0;
    }
    const bool swap = vds < 0.0;  // source/drain exchange, the old vds in every term
    if (swap) {
        vgs = vgs - vds;
        vbs = vbs - vds;
        vds = -vds;
    }
    // calc_threshold
    const double phi_vbs = fmax(K(B3C_PHI) - vbs, 0.01);
    const double sq = sqrt(phi_vbs);
    const double body = K(B3C_K1) * (sq - K(B3C_SQRTPHI)) - K(B3C_K2) * vbs;
    const double sce = K(B3C_SCE) * (1.0 + K(B3C_DVT2) * vbs);
    const double nwe = K(B3C_NWE_ON) != 0.0 ? K(B3C_K3TW) * sq + K(B3C_K3B) * vbs / K(B3C_WEFF) : 0.0;
    const double nwe_sce = K(B3C_SCEW) * (1.0 + K(B3C_DVT2W) * vbs);
    const double dibl = -(K(B3C_ETA0) + K(B3C_ETAB) * vbs) * vds * K(B3C_THETA_DIBL);
    const double temp = 0.0 + K(B3C_KT2) * vbs * 0.0;  // vth0_temp + KT2 vbs (T/TNOM - 1) at TNOM
    const double vth = K(B3C_VTH0ABS) + body + sce + nwe + nwe_sce + dibl + temp;
    const double vgst = vgs - vth;
    r.vth = sign * vth;
    if (vgst < 0.0) {  // calc_subthreshold
        const double nvt = K(B3C_NVT);
        const double ids_sub = K(B3C_I0) * exp(fmin(vgst / nvt, 20.0)) * (1.0 - exp(-vds / K(B3C_VT)));
        r.ids = sign * ids_sub;
        r.gds = fmax(ids_sub * 0.01, 1e-12);
        r.gm = swap ? 0.0 : ids_sub / nvt;
        r.gmbs = 0.0;
        r.vdsat = 0.0;
        r.region = 0;
        return r;
    }
    // calc_mobility
    const double eeff = (fmax(vgst, 0.01) + K(B3C_C32)) / K(B3C_TOX);
    const double degr = 1.0 + (K(B3C_UA) + K(B3C_UC) * vbs) * eeff + K(B3C_UB) * eeff * eeff;
    const double ueff = K(B3C_U0SI) / fmax(degr, 0.1);
    // calc_abulk
    const double abulk = rs_clamp((1.0 + K(B3C_K1) / (2.0 * sq) - K(B3C_K2)) * K(B3C_SCEF), 1.0, 2.5);
    // calc_vdsat (VSAT at TNOM) and the esat of the region functions
    const double esat_l = 2.0 * K(B3C_VSAT) / ueff * K(B3C_LEFF);
    const double vge = fmax(vgst, 0.001);
    const double vdsat = fmax(vge / (abulk + vge / esat_l), 0.001);
    // calc_early_voltage
    const double pdiblc_eff = fabs(K(B3C_PDIBLC1) + K(B3C_PDIBLCB) * vbs) + K(B3C_PDIBLC2);
    const double f_dibl = 1.0 / (1.0 + pdiblc_eff * (vds / (vdsat + 0.1)));
    const double f_drout = 1.0 / (1.0 + K(B3C_DROUT) * vds / (vgst + 0.1));
    const double f_pvag = 1.0 + K(B3C_PVAG) * vgst / (vdsat + 0.1);
    const double va = rs_clamp(K(B3C_VABASE) * f_dibl * f_drout * f_pvag, 0.5, 10.0);
    const double beta = K(B3C_WL) * ueff * K(B3C_COX);
    double ids, gm, gds, gmbs;
    if (vds < vdsat) {  // calc_linear
        const double vgl = fmax(vge - abulk * vds / 2.0, 0.001);
        const double vsf = 1.0 + vds / esat_l;
        const double ids_base = beta * vgl * vds / vsf;
        const double clm = 1.0 + vds / va * 0.1;
        const double m = beta * vds / vsf * clm;
        const double g = beta * (vge - abulk * vds) / vsf + beta * vgl * vds / (vsf * esat_l * vsf) + ids_base / va * 0.1;
        gmbs = fabs(m * fabs(K(B3C_K1) / (2.0 * sq) - K(B3C_K2)) * 0.5);
        ids = fmax(ids_base * clm, 0.0);
        gm = fmax(m, 0.0);
        gds = fmax(g, 1e-12);
        r.region = 1;
    } else {  // calc_saturation
        const double t = abulk + vge / esat_l;
        const double ids_dsat = beta * vge * vge / (2.0 * t);
        const double clm = 1.0 + fmax(vds - vdsat, 0.0) / va;
        const double m = beta * vge * (2.0 * abulk + vge / esat_l) / (2.0 * (t * t)) * clm;
        gmbs = fabs(m * fabs(K(B3C_K1) / (2.0 * sq) - K(B3C_K2) - K(B3C_ETAB) * vds));
        ids = fmax(ids_dsat * clm, 0.0);
        gm = fmax(m, 0.0);
        gds = fmax(ids_dsat / va, 1e-12);
        r.region = 2;
    }
    r.ids = sign * ids;
    r.gds = gds;  // already >= 1e-12
    r.gm = swap ? gm - gds : gm;
    r.gmbs = gmbs;
    r.vdsat = vdsat;
    return r;
}

// Bsim3Derived::junction_cap (derived.rs:323-345), FC = 0.5.
__host__ __device__ inline double bsim3_junction_cap(double cj0, double v, double pb, double mj) {
    if (cj0 <= 0.0) return 0.0;
    v = fmin(v, pb * 0.95);
    if (v < 0.5 * pb) return cj0 / pow(1.0 - v / pb, mj);
    const double f1 = pow(1.0 - 0.5, 1.0 + mj), f2 = 1.0 + mj, f3 = 1.0 - 0.5 * (1.0 + mj);
    return cj0 / f1 * (f3 + mj * v / pb / f2);
}

// evaluate_capacitances (evaluate.rs:82-158) at the terminal voltages and the
// region evaluate returned: out = (cgs, cgd, cgb, cbs, cbd).  K reads the
// per-sample constants, C the card slots.
template <class KF, class CF>
__host__ __device__ inline void bsim3_caps(bool pmos, KF K, CF C, double vds, double vbs, int region,
                                           double* out) {
    if (pmos) {
        vds = -vds;
        vbs = -vbs;
    }
    const double weff = K(B3C_WEFF), leff = K(B3C_LEFF);
    const double cox_total = K(B3C_COX) * weff * leff;
    double cgs = 0.0, cgd = 0.0, cgb = 0.0;
    if (region == 0) {
        cgb = cox_total;
    } else if (region == 1) {
        cgs = cox_total / 2.0;
        cgd = cgs;
    } else {
        cgs = cox_total * 2.0 / 3.0;
    }
    out[0] = cgs + C(SP_B3_CGSO) * weff;
    out[1] = cgd + C(SP_B3_CGDO) * weff;
    out[2] = cgb + C(SP_B3_CGBO) * leff;
    const double vbd = vbs - vds, diff = 0.5e-6;
    const double as_e = C(SP_B3_AS) > 0.0 ? C(SP_B3_AS) : weff * diff;
    const double ad_e = C(SP_B3_AD) > 0.0 ? C(SP_B3_AD) : weff * diff;
    const double ps_e = C(SP_B3_PS) > 0.0 ? C(SP_B3_PS) : 2.0 * (weff + diff);
    const double pd_e = C(SP_B3_PD) > 0.0 ? C(SP_B3_PD) : 2.0 * (weff + diff);
    out[3] = bsim3_junction_cap(C(SP_B3_CJ) * as_e, vbs, C(SP_B3_PB), C(SP_B3_MJ)) +
             bsim3_junction_cap(C(SP_B3_CJSW) * ps_e, vbs, C(SP_B3_PBSW), C(SP_B3_MJSW)) +
             bsim3_junction_cap(C(SP_B3_CJSWG) * weff, vbs, C(SP_B3_PBSWG), C(SP_B3_MJSWG));
    out[4] = bsim3_junction_cap(C(SP_B3_CJ) * ad_e, vbd, C(SP_B3_PB), C(SP_B3_MJ)) +
             bsim3_junction_cap(C(SP_B3_CJSW) * pd_e, vbd, C(SP_B3_PBSW), C(SP_B3_MJSW)) +
             bsim3_junction_cap(C(SP_B3_CJSWG) * weff, vbd, C(SP_B3_PBSWG), C(SP_B3_MJSWG));
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
        case SP_EL_BSIM3N:
        case SP_EL_BSIM3P: {
            const int base = el.field[0];
            bsim3_constants([&](int k) { return P(base + k); }, out);
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
            case SP_EL_BSIM3N:
            case SP_EL_BSIM3P: {  // mod.rs:176-227, at the unlimited terminal voltages
                const int d = n0, g = n1, so = n2, b = el.node[3];
                const double vg = g >= 0 ? k.x(g) : 0.0;
                const double vd = d >= 0 ? k.x(d) : 0.0;
                const double vs = so >= 0 ? k.x(so) : 0.0;
                const double vb = b >= 0 ? k.x(b) : 0.0;
                const double vgs = vg - vs, vds = vd - vs, vbs = vb - vs;
                const Bsim3Out r = bsim3_eval(el.kind == SP_EL_BSIM3P, [&](int i) { return dv(off + i, s); },
                                              vgs, vds, vbs);
                if (d >= 0) k.add(d, d, r.gds);
                if (so >= 0) k.add(so, so, r.gds);
                if (d >= 0 && so >= 0) {
                    k.add(d, so, -r.gds);
                    k.add(so, d, -r.gds);
                }
                if (d >= 0) {
                    if (g >= 0) k.add(d, g, r.gm);
                    if (so >= 0) k.add(d, so, -r.gm);
                }
                if (so >= 0) {
                    if (g >= 0) k.add(so, g, -r.gm);
                    k.add(so, so, r.gm);
                }
                if (d >= 0) {
                    if (b >= 0) k.add(d, b, r.gmbs);
                    if (so >= 0) k.add(d, so, -r.gmbs);
                }
                if (so >= 0) {
                    if (b >= 0) k.add(so, b, -r.gmbs);
                    k.add(so, so, r.gmbs);
                }
                const double ieq = r.ids - r.gds * vds - r.gm * vgs - r.gmbs * vbs;
                if (d >= 0) k.rhs_add(d, -ieq);
                if (so >= 0) k.rhs_add(so, ieq);
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
