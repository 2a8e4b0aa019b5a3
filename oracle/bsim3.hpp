// Oracle (test infrastructure, never the product path): the BSIM3v3.3 DC
// model of the reference ("BSIM3-lite", LEVEL=49 / 8), restated from
//   crates/spicier-devices/src/mosfet/bsim3/params.rs   (card, defaults :160-310,
//                                                       vt/cox/leff/weff :440-470)
//   crates/spicier-devices/src/mosfet/bsim3/derived.rs  (from_params :81-196)
//   crates/spicier-devices/src/mosfet/bsim3/evaluate.rs (evaluate :171-265,
//                                                       calc_* :268-598)
//   crates/spicier-devices/src/mosfet/bsim3/mod.rs      (stamp_linearized_at :176-227,
//                                                       stamp_nonlinear :275-294)
// in the reference's operation order (Rust evaluates a * b / c left to
// right; f64::max/min ignore a NaN operand; clamp keeps a NaN).  Derived
// values are computed at TNOM (Bsim3Derived::from_params, what with_params
// uses), so the temperature terms reduce to their nominal values.
//
// Parity with the reference is anchored on its own evaluate tests
// (evaluate.rs:600-…: regions, signs, orderings, the ngspice comparison
// within its stated tolerances) and on the netlist golden data
// crates/spicier-parser/tests/golden_data/dc_bsim3.json (ngspice-45, within
// the tolerances stored in that file); no bit-level vectors of the reference
// exist for this model.
#pragma once
#include <algorithm>
#include <cmath>

#include "../include/spicier_gb300.h"

namespace oracle {

namespace b3 {
constexpr double Q = 1.602176634e-19;
constexpr double KB = 1.380649e-23;
constexpr double EPS_SI = 1.03594e-10;
constexpr double EPS_OX = 3.45314e-11;
constexpr double NI = 1.45e10;

inline double rmax(double a, double b) { return std::fmax(a, b); }  // f64::max
inline double rmin(double a, double b) { return std::fmin(a, b); }  // f64::min
inline double rclamp(double x, double lo, double hi) {              // f64::clamp
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
}  // namespace b3

// Bsim3Params::{nmos,pmos}_default in sp_bsim3_card order.
inline void bsim3_default_card(bool pmos, double* card) {
    double* c = card;
    c[SP_B3_TOX] = 9e-9, c[SP_B3_LINT] = 0.0, c[SP_B3_WINT] = 0.0;
    c[SP_B3_VTH0] = pmos ? -0.4 : 0.4, c[SP_B3_K1] = 0.5, c[SP_B3_K2] = 0.0;
    c[SP_B3_DVT0] = 2.2, c[SP_B3_DVT1] = 0.53, c[SP_B3_DVT2] = -0.032, c[SP_B3_NFACTOR] = 1.0;
    c[SP_B3_K3] = 0.0, c[SP_B3_K3B] = 0.0, c[SP_B3_W0] = 0.0;
    c[SP_B3_DVT0W] = 0.0, c[SP_B3_DVT1W] = 0.0, c[SP_B3_DVT2W] = 0.0;
    c[SP_B3_U0] = pmos ? 250.0 : 670.0, c[SP_B3_UA] = 2.25e-9, c[SP_B3_UB] = 5.87e-19;
    c[SP_B3_UC] = -4.65e-11, c[SP_B3_VSAT] = pmos ? 1.0e5 : 1.5e5;
    c[SP_B3_PCLM] = 1.3, c[SP_B3_PDIBLC1] = 0.39, c[SP_B3_PDIBLC2] = 0.0086, c[SP_B3_DROUT] = 0.56;
    c[SP_B3_ETA0] = 0.08, c[SP_B3_ETAB] = -0.07, c[SP_B3_DSUB] = 0.56;
    c[SP_B3_PDIBLCB] = 0.0, c[SP_B3_PVAG] = 1.0;
    c[SP_B3_NCH] = 1.7e17, c[SP_B3_TNOM] = 300.15, c[SP_B3_KT2] = 0.022;
    c[SP_B3_W] = 1e-6, c[SP_B3_L] = 100e-9, c[SP_B3_NF] = 1.0;
    c[SP_B3_CGSO] = 0.0, c[SP_B3_CGDO] = 0.0, c[SP_B3_CGBO] = 0.0;
    c[SP_B3_CJ] = 5e-4, c[SP_B3_CJSW] = 5e-10, c[SP_B3_CJSWG] = 0.0;
    c[SP_B3_MJ] = 0.5, c[SP_B3_MJSW] = 0.33, c[SP_B3_MJSWG] = 0.33;
    c[SP_B3_PB] = 1.0, c[SP_B3_PBSW] = 1.0, c[SP_B3_PBSWG] = 1.0;
    c[SP_B3_AS] = 0.0, c[SP_B3_AD] = 0.0, c[SP_B3_PS] = 0.0, c[SP_B3_PD] = 0.0;
}

// Bsim3Derived (the fields evaluate reads), derived.rs:81-196.
struct Bsim3Derived {
    double leff, weff, cox, vt, phi, sqrt_phi, u0_si, lt;
    double temp_ratio, vth0_temp, vsat_temp, ua_temp, ub_temp, uc_temp;
};

inline Bsim3Derived bsim3_derive(const double* p, bool cr) {
    using namespace b3;
    Bsim3Derived d;
    d.leff = p[SP_B3_L] - 2.0 * p[SP_B3_LINT];
    d.weff = (p[SP_B3_W] - 2.0 * p[SP_B3_WINT]) * p[SP_B3_NF];
    d.cox = EPS_OX / p[SP_B3_TOX];
    d.vt = KB * p[SP_B3_TNOM] / Q;
    const double ln_nch = cr ? sp::cr_log(p[SP_B3_NCH] / NI, nullptr) : std::log(p[SP_B3_NCH] / NI);
    d.phi = 2.0 * d.vt * ln_nch;
    d.sqrt_phi = std::sqrt(d.phi);
    d.u0_si = p[SP_B3_U0] * 1e-4;
    const double xdep = std::sqrt(2.0 * EPS_SI * d.phi / (Q * p[SP_B3_NCH] * 1e6));
    d.lt = std::sqrt(EPS_SI * xdep * p[SP_B3_TOX] / EPS_OX);
    d.temp_ratio = 1.0;
    d.vth0_temp = 0.0;
    d.vsat_temp = p[SP_B3_VSAT];
    d.ua_temp = p[SP_B3_UA];
    d.ub_temp = p[SP_B3_UB];
    d.uc_temp = p[SP_B3_UC];
    return d;
}

struct Bsim3Eval {
    double ids, gds, gm, gmbs, vth, vdsat;
    int region;  // 0 subthreshold, 1 linear, 2 saturation
};

// evaluate.rs:268-326
inline double bsim3_threshold(const double* p, const Bsim3Derived& d, double vds, double vbs, bool cr) {
    using namespace b3;
    auto ex = [&](double v) { return cr ? sp::cr_exp(v, nullptr) : std::exp(v); };
    const double phi_vbs = rmax(d.phi - vbs, 0.01);
    const double body = p[SP_B3_K1] * (std::sqrt(phi_vbs) - d.sqrt_phi) - p[SP_B3_K2] * vbs;
    const double lt_ratio = p[SP_B3_DVT1] * d.leff / (2.0 * d.lt);
    const double e1 = ex(-rmin(lt_ratio, 20.0));
    const double theta = e1 / (1.0 + 2.0 * e1);
    const double sce = -p[SP_B3_DVT0] * theta * d.vt * (1.0 + p[SP_B3_DVT2] * vbs);
    double nwe = 0.0;
    if (d.weff > 1e-9) {
        const double tox_weff = p[SP_B3_TOX] / d.weff;
        nwe = p[SP_B3_K3] * tox_weff * std::sqrt(phi_vbs) + p[SP_B3_K3B] * vbs / d.weff;
    }
    const double wt = std::sqrt(EPS_SI * p[SP_B3_TOX] / EPS_OX);
    const double wt_ratio = p[SP_B3_DVT1W] * d.weff / (2.0 * wt + p[SP_B3_W0]);
    const double ew = ex(-rmin(wt_ratio, 20.0));
    const double theta_w = ew / (1.0 + 2.0 * ew);
    const double nwe_sce = -p[SP_B3_DVT0W] * theta_w * d.vt * (1.0 + p[SP_B3_DVT2W] * vbs);
    const double dibl_ratio = p[SP_B3_DSUB] * d.leff / (2.0 * d.lt);
    const double theta_dibl = ex(-rmin(dibl_ratio, 20.0));
    const double dibl = -(p[SP_B3_ETA0] + p[SP_B3_ETAB] * vbs) * vds * theta_dibl;
    const double temp = d.vth0_temp + p[SP_B3_KT2] * vbs * (d.temp_ratio - 1.0);
    const double vth0_abs = std::fabs(p[SP_B3_VTH0]);
    return vth0_abs + body + sce + nwe + nwe_sce + dibl + temp;
}

// evaluate.rs:171-265 with calc_subthreshold :328-356, calc_mobility :359-382,
// calc_abulk :385-404, calc_vdsat :407-430, calc_early_voltage :433-492,
// calc_linear :495-546, calc_saturation :549-598.
inline Bsim3Eval bsim3_evaluate(bool pmos, const double* p, const Bsim3Derived& d, double vgs, double vds,
                                double vbs, bool cr) {
    using namespace b3;
    auto ex = [&](double v) { return cr ? sp::cr_exp(v, nullptr) : std::exp(v); };
    double sign = 1.0;
    if (pmos) vgs = -vgs, vds = -vds, vbs = -vbs, sign = -1.0;
    bool swap = false;
    if (vds < 0.0) {
        const double v0 = vds;
        vgs = vgs - v0, vds = -v0, vbs = vbs - v0, swap = true;
    }
    Bsim3Eval r{};
    const double vth = bsim3_threshold(p, d, vds, vbs, cr);
    const double vgst = vgs - vth;
    if (vgst < 0.0) {
        const double nvt = p[SP_B3_NFACTOR] * d.vt;
        const double i0 = (d.weff / d.leff) * d.u0_si * d.cox * nvt * nvt;
        const double exp_factor = ex(rmin(vgst / nvt, 20.0));
        const double vds_factor = 1.0 - ex(-vds / d.vt);
        const double ids_sub = i0 * exp_factor * vds_factor;
        const double gm_sub = ids_sub / (p[SP_B3_NFACTOR] * d.vt);
        const double gds_sub = ids_sub * 0.01;
        r.ids = sign * ids_sub;
        r.gds = rmax(gds_sub, 1e-12);
        r.gm = (swap ? 0.0 : gm_sub) * std::fabs(sign);
        r.gmbs = 0.0;
        r.vth = sign * vth;
        r.vdsat = 0.0;
        r.region = 0;
        return r;
    }
    // mobility
    const double vgst_m = rmax(vgst, 0.01);
    const double eeff = (vgst_m + 3.2 * std::fabs(p[SP_B3_VTH0])) / p[SP_B3_TOX];
    const double degr = 1.0 + (d.ua_temp + d.uc_temp * vbs) * eeff + d.ub_temp * eeff * eeff;
    const double ueff = d.u0_si / rmax(degr, 0.1);
    // abulk
    const double phi_vbs = rmax(d.phi - vbs, 0.01);
    const double abulk_base = 1.0 + p[SP_B3_K1] / (2.0 * std::sqrt(phi_vbs)) - p[SP_B3_K2];
    const double sce_factor = 1.0 - 0.3 * rmin(d.lt / d.leff, 1.0);
    const double abulk = rclamp(abulk_base * sce_factor, 1.0, 2.5);
    // vdsat
    const double esat_v = 2.0 * d.vsat_temp / ueff;
    const double esat_lv = esat_v * d.leff;
    const double vg_v = rmax(vgst, 0.001);
    const double vdsat = rmax(vg_v / (abulk + vg_v / esat_lv), 0.001);
    // early voltage
    const double esat0 = 2.0 * p[SP_B3_VSAT] / d.u0_si;
    const double va_base = d.leff * esat0 * 4.0 / rmax(p[SP_B3_PCLM], 0.1);
    const double pdiblc_eff = std::fabs(p[SP_B3_PDIBLC1] + p[SP_B3_PDIBLCB] * vbs) + p[SP_B3_PDIBLC2];
    const double va_dibl = 1.0 / (1.0 + pdiblc_eff * (vds / (vdsat + 0.1)));
    const double drout = 1.0 / (1.0 + p[SP_B3_DROUT] * vds / (vgst + 0.1));
    const double pvag = 1.0 + p[SP_B3_PVAG] * vgst / (vdsat + 0.1);
    const double va = rclamp(va_base * va_dibl * drout * pvag, 0.5, 10.0);

    const double vge = rmax(vgst, 0.001);
    const double beta = (d.weff / d.leff) * ueff * d.cox;
    const double esat = 2.0 * p[SP_B3_VSAT] / ueff;
    const double esat_l = esat * d.leff;
    double ids, gm, gds, gmbs;
    if (vds < vdsat) {
        const double vge_lin = rmax(vge - abulk * vds / 2.0, 0.001);
        const double vs_factor = 1.0 + vds / esat_l;
        const double ids_base = beta * vge_lin * vds / vs_factor;
        const double i = ids_base * (1.0 + vds / va * 0.1);
        const double m = beta * vds / vs_factor * (1.0 + vds / va * 0.1);
        const double g = beta * (vge - abulk * vds) / vs_factor +
                         beta * vge_lin * vds / (vs_factor * esat_l * vs_factor) + ids_base / va * 0.1;
        const double dvth_dvbs = p[SP_B3_K1] / (2.0 * std::sqrt(phi_vbs)) - p[SP_B3_K2];
        gmbs = std::fabs(m * std::fabs(dvth_dvbs) * 0.5);
        ids = rmax(i, 0.0), gm = rmax(m, 0.0), gds = rmax(g, 1e-12);
        r.region = 1;
    } else {
        const double denom = 2.0 * (abulk + vge / esat_l);
        const double ids_dsat = beta * vge * vge / denom;
        const double clm = 1.0 + rmax(vds - vdsat, 0.0) / va;
        const double i = ids_dsat * clm;
        const double t = abulk + vge / esat_l;
        const double denom_sq = t * t;
        const double m = beta * vge * (2.0 * abulk + vge / esat_l) / (2.0 * denom_sq) * clm;
        const double g = ids_dsat / va;
        const double dvth_dvbs = p[SP_B3_K1] / (2.0 * std::sqrt(phi_vbs)) - p[SP_B3_K2] - p[SP_B3_ETAB] * vds;
        gmbs = std::fabs(m * std::fabs(dvth_dvbs));
        ids = rmax(i, 0.0), gm = rmax(m, 0.0), gds = rmax(g, 1e-12);
        r.region = 2;
    }
    if (swap) gm = gm - gds;
    r.ids = sign * ids;
    r.gds = rmax(gds, 1e-12);
    r.gm = gm * std::fabs(sign);
    r.gmbs = gmbs * std::fabs(sign);
    r.vth = sign * vth;
    r.vdsat = vdsat;
    return r;
}

// Bsim3Derived::junction_cap, derived.rs:323-345
inline double bsim3_junction_cap(double cj0, double v, double pb, double mj) {
    const double FC = 0.5;
    if (cj0 <= 0.0) return 0.0;
    v = std::fmin(v, pb * 0.95);
    if (v < FC * pb) {
        const double ratio = 1.0 - v / pb;
        return cj0 / std::pow(ratio, mj);
    }
    const double f1 = std::pow(1.0 - FC, 1.0 + mj);
    const double f2 = 1.0 + mj;
    const double f3 = 1.0 - FC * (1.0 + mj);
    return cj0 / f1 * (f3 + mj * v / pb / f2);
}

// evaluate_capacitances, evaluate.rs:82-158 (with derived.rs:122-163 for the
// overlap capacitances and diffusion estimates): c = cgs, cgd, cgb, cbs, cbd.
inline void bsim3_capacitances(bool pmos, const double* p, const Bsim3Derived& d, double vds, double vbs,
                               int region, double* c) {
    if (pmos) vds = -vds, vbs = -vbs;
    const double cox_total = d.cox * d.weff * d.leff;
    double cgs_int = 0.0, cgd_int = 0.0, cgb_int = 0.0;
    if (region == 0) {
        cgb_int = cox_total;
    } else if (region == 1) {
        const double c_half = cox_total / 2.0;
        cgs_int = c_half, cgd_int = c_half;
    } else {
        cgs_int = cox_total * 2.0 / 3.0;
    }
    c[0] = cgs_int + p[SP_B3_CGSO] * d.weff;
    c[1] = cgd_int + p[SP_B3_CGDO] * d.weff;
    c[2] = cgb_int + p[SP_B3_CGBO] * d.leff;
    const double vbd = vbs - vds;
    const double diff_length = 0.5e-6;
    const double as_eff = p[SP_B3_AS] > 0.0 ? p[SP_B3_AS] : d.weff * diff_length;
    const double ad_eff = p[SP_B3_AD] > 0.0 ? p[SP_B3_AD] : d.weff * diff_length;
    const double ps_eff = p[SP_B3_PS] > 0.0 ? p[SP_B3_PS] : 2.0 * (d.weff + diff_length);
    const double pd_eff = p[SP_B3_PD] > 0.0 ? p[SP_B3_PD] : 2.0 * (d.weff + diff_length);
    c[3] = bsim3_junction_cap(p[SP_B3_CJ] * as_eff, vbs, p[SP_B3_PB], p[SP_B3_MJ]) +
           bsim3_junction_cap(p[SP_B3_CJSW] * ps_eff, vbs, p[SP_B3_PBSW], p[SP_B3_MJSW]) +
           bsim3_junction_cap(p[SP_B3_CJSWG] * d.weff, vbs, p[SP_B3_PBSWG], p[SP_B3_MJSWG]);
    c[4] = bsim3_junction_cap(p[SP_B3_CJ] * ad_eff, vbd, p[SP_B3_PB], p[SP_B3_MJ]) +
           bsim3_junction_cap(p[SP_B3_CJSW] * pd_eff, vbd, p[SP_B3_PBSW], p[SP_B3_MJSW]) +
           bsim3_junction_cap(p[SP_B3_CJSWG] * d.weff, vbd, p[SP_B3_PBSWG], p[SP_B3_MJSWG]);
}

}  // namespace oracle
