// Oracle of the batched RC-diode ladder transient — TEST INFRASTRUCTURE ONLY.
//
// The reference's transient solvers are linear (solve_transient, TR-BDF2 at a
// fixed step; solve_transient_adaptive, trapezoidal).  The ladder workload
// combines their pieces into a nonlinear adaptive TR-BDF2 integration, and
// this file is the CPU statement of that combination, in the operation order
// the GPU kernel follows:
//   * section draws: N = min + floor((max-min+1) u_0), R_k and C_k log-uniform
//     a exp(u ln(b/a)) with u = uniform(seed, instance, 2k-1 / 2k)
//     (rng.rs:80-85 for u);
//   * MNA unknowns [v_in, v_1..v_N, I_src]: the PULSE source (waveforms.rs:
//     159-182) at node in, R_k between nodes k-1 and k, C_k and the diode
//     (diode.rs:91-131: double limiting, Ieq at the once-limited voltage)
//     from node k to ground;
//   * one step = the reference's TR-BDF2 (solver.rs:186-251): stage 1
//     stamp_trap at gamma h, update_trbdf2_intermediate, stage 2
//     stamp_trbdf2_bdf2, update(TrBdf2) on acceptance (companion.rs:41-150),
//     both stages with the source at the step's end time as in solver.rs:110;
//     one deviation: after the BDF2 stage the capacitor current is the
//     current of the BDF2 companion at the solution, geq v - ieq, where
//     update(TrBdf2) (companion.rs:75-84) uses C/h ((1+a) v - (1+2a) v_gamma
//     + a v_0), which is that current only for gamma = 1/2 (for a linear
//     ramp it gives a third of C dv/dt); the reference's fixed-step RC test
//     tolerates 0.6 V of error at one time constant, but the adaptive
//     controller's LTE (the mismatch of that current against the next step)
//     would then never fall with h and the step size collapses;
//     each stage is a Newton solve (full step, newton.rs:70-131 and the
//     convergence test of newton.rs:134-159) from the previous stage's result;
//   * step control = solve_transient_adaptive (solver.rs:548-671): h clamped to
//     [h_min, h_max] and to tstop; LTE = max over capacitors of estimate_lte
//     (companion.rs:137-150) against the step-start state; reject when
//     LTE > max(abstol, reltol max|v|) and h > h_min (restore the capacitor
//     states, h *= max(0.1, min(0.5, sqrt(tol/LTE)))); on acceptance grow by
//     min(1.5, sqrt(tol/LTE), 2) when LTE < tol/2.  A stage whose Newton solve
//     fails rejects the step with h *= 1/4 (the linear reference cannot fail
//     there); at h_min the instance ends FAILED;
//   * linear solves: v_in = V(t), then the tridiagonal system of the chain by
//     forward elimination and back substitution (the symbolic factorisation of
//     this pattern has no fill), then I_src from the KCL of node in.
// Transcendentals: math_mode() 0 = host libm (std::exp, std::log,
// std::log1p), 1 = the portable set the GPU uses (cr_exp, cr_log, pm_log1p).
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "oracle_core.hpp"

namespace oracle {

constexpr double kTrbdf2Gamma = 2.0 - 1.4142135623730951;  // types.rs:11, 2 - SQRT_2

inline double m_exp(double x) { return math_mode() == 1 ? sp::cr_exp(x, nullptr) : std::exp(x); }
inline double m_log(double x) { return math_mode() == 1 ? sp::cr_log(x, nullptr) : std::log(x); }
inline double m_log1p(double x) { return math_mode() == 1 ? sp::pm_log1p(x, nullptr) : std::log1p(x); }

// waveforms.rs:159-182
inline double eval_pulse(const sp_pulse& p, double t) {
    if (t < p.td) return p.v1;
    const double t_rel = p.per > 0.0 ? std::fmod(t - p.td, p.per) : t - p.td;
    if (t_rel < p.tr) return p.v1 + (p.v2 - p.v1) * t_rel / p.tr;
    if (t_rel < p.tr + p.pw) return p.v2;
    if (t_rel < p.tr + p.pw + p.tf) return p.v2 - (p.v2 - p.v1) * (t_rel - p.tr - p.pw) / p.tf;
    return p.v1;
}

struct Ladder {
    int N = 0;
    std::vector<double> g, C;  // g[k] = 1/R_k, C[k] for k = 1..N (index 0 unused)
};

inline Ladder ladder_draw(const sp_ladder_config& c, uint64_t seed, uint32_t inst) {
    Ladder L;
    const double span = (double)(c.max_sections - c.min_sections + 1);
    L.N = c.min_sections + (int)std::floor(span * uniform(seed, inst, 0));
    L.g.assign(L.N + 1, 0.0);
    L.C.assign(L.N + 1, 0.0);
    const double lr = m_log(c.r_hi / c.r_lo), lc = m_log(c.c_hi / c.c_lo);
    for (int k = 1; k <= L.N; ++k) {
        const double R = c.r_lo * m_exp(uniform(seed, inst, 2u * k - 1u) * lr);
        L.C[k] = c.c_lo * m_exp(uniform(seed, inst, 2u * k) * lc);
        L.g[k] = 1.0 / R;  // passive.rs:48-50
    }
    return L;
}

struct LadderOutcome {
    uint8_t status = SP_ST_CONVERGED;
    int32_t accepted = 0, rejected = 0, iterations = 0;
    std::vector<double> steps;  // accepted step sizes, in order
};

struct LadderSolver {
    const sp_ladder_config& c;
    const Ladder& L;
    double nvt, vcrit;
    std::vector<double> diag, sup, rhs, cp, dp;

    LadderSolver(const sp_ladder_config& cfg, const Ladder& lad) : c(cfg), L(lad) {
        nvt = c.diode_n * thermal_voltage(300.15);
        vcrit = nvt * m_log(nvt / (1.4142135623730951 * 1e-14));
        diag.resize(L.N + 2);
        sup.resize(L.N + 2);
        rhs.resize(L.N + 2);
        cp.resize(L.N + 2);
        dp.resize(L.N + 2);
    }

    // diode.rs:138-148 with vcrit computed once (the same value every call)
    double limit(double vd) const {
        if (vd > vcrit) {
            const double arg = (vd - vcrit) / nvt;
            return vcrit + nvt * (1.0 + m_log1p(arg));
        }
        return vd;
    }

    // One linearised solve of a stage: x -> xn.  geq/ieq: capacitor companions.
    void linear_solve(const double* x, const double* geq, const double* ieq, double V, double* xn) {
        const int N = L.N;
        for (int k = 1; k <= N; ++k) {
            // diode.rs:113-131: limit once for Ieq, evaluate (limits again)
            const double vl1 = limit(x[k]);
            const double vl2 = limit(vl1);
            const double e = m_exp(vl2 / nvt);
            const double id = c.diode_is * (e - 1.0);
            const double gd = std::fmax(c.diode_is * e / nvt, 1e-12);
            const double ieq_d = id - gd * vl1;
            // stamping order: resistors, source, capacitors, diodes
            const double gk1 = k < N ? L.g[k + 1] : 0.0;
            diag[k] = ((L.g[k] + gk1) + geq[k]) + gd;
            sup[k] = -gk1;
            rhs[k] = (0.0 + ieq[k]) - ieq_d;
        }
        // v_in = V; the chain with -g_1 v_in moved to the right-hand side
        rhs[1] = rhs[1] - (-L.g[1]) * V;
        cp[1] = sup[1] / diag[1];
        dp[1] = rhs[1] / diag[1];
        for (int k = 2; k <= N; ++k) {
            const double sub = -L.g[k];
            const double m = diag[k] - sub * cp[k - 1];
            cp[k] = sup[k] / m;
            dp[k] = (rhs[k] - sub * dp[k - 1]) / m;
        }
        xn[N] = dp[N];
        for (int k = N - 1; k >= 1; --k) xn[k] = dp[k] - cp[k] * xn[k + 1];
        xn[0] = V;
        // KCL of node in: g_1 v_in - g_1 v_1 + I = 0
        xn[N + 1] = -(L.g[1] * V + (-L.g[1]) * xn[1]);
    }

    bool converged(const double* old, const double* nw) const {
        const int n = L.N + 2;
        for (int i = 0; i < n; ++i) {
            const double delta = std::fabs(nw[i] - old[i]);
            const double tol = c.v_reltol * std::fmax(std::fabs(nw[i]), std::fabs(old[i])) +
                               (i < L.N + 1 ? c.v_abstol : c.i_abstol);
            if (delta > tol) return false;
        }
        return true;
    }

    // Newton solve of a stage from x (updated in place); returns iterations or -1.
    int newton(double* x, const double* geq, const double* ieq, double V, std::vector<double>& work) {
        const int n = L.N + 2;
        work.resize(n);
        for (int it = 1; it <= c.max_iterations; ++it) {
            linear_solve(x, geq, ieq, V, work.data());
            const bool ok = converged(x, work.data());
            bool finite = true;
            for (int i = 0; i < n; ++i) {
                x[i] = work[i];
                finite = finite && std::isfinite(x[i]);
            }
            if (!finite) return -2;
            if (ok) return it;
        }
        return -1;
    }
};

// One instance: x_final[N+2], probe[num_probe] of v_N.
// Replay (forced != nullptr): the step sizes are forced[0..nforced-1], taken in
// order with no clamping and no LTE test, every step accepted; everything else
// is the adaptive run's arithmetic, so a GPU run's recorded accepted steps
// replayed here give the oracle's result along the GPU's own step sequence.
// A stage that fails in a replay ends the instance FAILED (a replay cannot
// retry with a smaller step).
inline LadderOutcome ladder_transient(const sp_ladder_config& c, const Ladder& L, double* x_final, double* probe,
                                      const double* forced = nullptr, int nforced = 0) {
    LadderSolver S(c, L);
    const int N = L.N, n = N + 2;
    LadderOutcome out;
    std::vector<double> x(n, 0.0), x1(n), x2(n), work;
    // capacitor states (companion.rs CapacitorState): v_prev, i_prev, v_prev_prev; DC start: all zero
    std::vector<double> vp(N + 1, 0.0), ip(N + 1, 0.0), vpp(N + 1, 0.0);
    std::vector<double> svp(N + 1), sip(N + 1), svpp(N + 1), geq(N + 1), ieq(N + 1);
    const double gamma = kTrbdf2Gamma;
    double t = 0.0, h = c.h_init;
    int next_probe = 0;
    auto record = [&](double t0, const double* xa, double t1, const double* xb) {
        while (next_probe < c.num_probe) {
            const double tp = c.num_probe > 1 ? c.tstop * (double)next_probe / (double)(c.num_probe - 1) : 0.0;
            if (tp > t1) break;
            probe[next_probe++] = t1 > t0 ? xa[N] + (xb[N] - xa[N]) * ((tp - t0) / (t1 - t0)) : xb[N];
        }
    };
    record(0.0, x.data(), 0.0, x.data());
    int steps = 0;
    while (forced ? out.accepted < nforced : t < c.tstop) {
        if (++steps > c.max_steps) {
            out.status = SP_ST_FAILED;
            break;
        }
        if (forced) {
            h = forced[out.accepted];
        } else {
            h = std::min(std::max(h, c.h_min), c.h_max);  // h.clamp(h_min, h_max)
            if (t + h > c.tstop) h = c.tstop - t;
        }
        const double V = eval_pulse(c.pulse, t + h);
        svp = vp;
        sip = ip;
        svpp = vpp;
        // stage 1: trapezoidal over gamma h (stamp_trap with h_gamma)
        const double hg = gamma * h;
        for (int k = 1; k <= N; ++k) {
            geq[k] = 2.0 * L.C[k] / hg;
            ieq[k] = geq[k] * vp[k] + ip[k];
        }
        x1 = x;
        int it1 = S.newton(x1.data(), geq.data(), ieq.data(), V, work);
        int it2 = -1;
        if (it1 > 0) {
            out.iterations += it1;
            // update_trbdf2_intermediate(v_gamma, h)
            for (int k = 1; k <= N; ++k) {
                vpp[k] = vp[k];
                ip[k] = 2.0 * L.C[k] / hg * (x1[k] - vpp[k]) - ip[k];
                vp[k] = x1[k];
            }
            // stage 2: BDF2 over (1 - gamma) h (stamp_trbdf2_bdf2)
            const double h2 = (1.0 - gamma) * h, h1 = gamma * h, rho = h2 / h1;
            const double denom = 1.0 + 2.0 * rho;
            const double a1 = (1.0 + rho) * (1.0 + rho) / denom, a2 = -rho * rho / denom, b0 = (1.0 + rho) / denom;
            for (int k = 1; k <= N; ++k) {
                geq[k] = L.C[k] / (b0 * h2);
                ieq[k] = geq[k] * (a1 * vp[k] + a2 * vpp[k]);
            }
            x2 = x1;
            it2 = S.newton(x2.data(), geq.data(), ieq.data(), V, work);
            if (it2 > 0) out.iterations += it2;
        }
        if (it1 == -2 || it2 == -2) {
            out.status = SP_ST_NONFINITE;
            break;
        }
        if ((it1 < 0 || it2 < 0) && forced) {
            out.status = SP_ST_FAILED;
            break;
        }
        if (it1 < 0 || it2 < 0) {  // a stage's Newton solve failed
            vp = svp;
            ip = sip;
            vpp = svpp;
            ++out.rejected;
            if (h <= c.h_min) {
                out.status = SP_ST_FAILED;
                break;
            }
            h *= 0.25;
            continue;
        }
        // LTE: estimate_lte(v_new, h) against the step-start state
        double max_lte = 0.0, max_ref = 0.0;
        for (int k = 1; k <= N; ++k) {
            const double v_new = x2[k];
            const double i_trap = 2.0 * L.C[k] / h * (v_new - svp[k]) - sip[k];
            const double i_be = L.C[k] / h * (v_new - svp[k]);
            const double lte = std::fabs(i_trap - i_be) / 3.0;
            max_lte = std::fmax(max_lte, lte);
            max_ref = std::fmax(max_ref, std::fabs(v_new));
        }
        const double tol = std::fmax(c.lte_abstol, c.lte_reltol * max_ref);
        if (!forced && max_lte > tol && h > c.h_min) {
            vp = svp;
            ip = sip;
            vpp = svpp;
            ++out.rejected;
            const double factor = std::fmin(std::sqrt(tol / max_lte), 0.5);
            h *= std::fmax(factor, 0.1);
            continue;
        }
        // accept: the capacitor current the BDF2 companion carries at the
        // solution, geq v_new - ieq (see the header: update(TrBdf2)'s own
        // formula is not this current for gamma != 1/2)
        for (int k = 1; k <= N; ++k) {
            const double v_new = x2[k];
            ip[k] = geq[k] * v_new - ieq[k];
            vpp[k] = vp[k];
            vp[k] = v_new;
        }
        record(t, x.data(), t + h, x2.data());
        out.steps.push_back(h);
        x = x2;
        t += h;
        ++out.accepted;
        if (max_lte < tol * 0.5 && h < c.h_max) {
            const double factor = std::fmin(std::sqrt(tol / std::fmax(max_lte, 1e-20)), 2.0);
            h *= std::fmin(factor, 1.5);
        }
    }
    while (next_probe < c.num_probe) probe[next_probe++] = x[N];  // t reached tstop
    for (int i = 0; i < n; ++i) x_final[i] = x[i];
    return out;
}

}  // namespace oracle

namespace oracle {

// ---------------------------------------------------------------------------
// Fixed-step linear transient, solve_transient (solver.rs:41-252): the
// circuit's R, V and I stamped at t = step h (stamp_at_time, element order),
// then the capacitor and inductor companions (companion.rs, capacitors
// first), one dense solve per step (two for TR-BDF2), the states updated with
// the reference's own update rules (update, update_trbdf2_intermediate —
// including the TR-BDF2 inductor update's v_prev term as written).
// Unknowns: nodes + V-source currents (inductors carry no branch variable);
// the capacitor voltages, inductor currents and the initial solution come
// from the DC operating point dc[] (nodes + every DC branch, V and L).
// ---------------------------------------------------------------------------
struct TranState {
    double v_prev = 0, i_prev = 0, pp = 0;  // pp: v_prev_prev (C) or i_prev_prev (L)
};

inline double wave_value(const sp_circuit& c, const sp_element& el, const double* P, double t) {
    if (el.wave >= 0 && el.wave < c.num_pulses) return eval_pulse(c.pulses[el.wave], t);
    return P[el.field[0]];
}

// Transient-MNA branch index of V source element e (order among V sources).
inline int vsource_index(const sp_circuit& c, int e) {
    int k = 0;
    for (int i = 0; i < e; ++i) k += c.elements[i].kind == SP_EL_V;
    return k;
}

inline int num_vsources(const sp_circuit& c) { return vsource_index(c, c.num_elements); }

inline void stamp_static(const sp_circuit& c, const double* P, double t, Mna& m) {
    for (int e = 0; e < c.num_elements; ++e) {
        const sp_element& el = c.elements[e];
        const int* nd = el.node;
        if (el.kind == SP_EL_R) m.conductance(nd[0], nd[1], 1.0 / P[el.field[0]]);
        else if (el.kind == SP_EL_V) m.voltage_source(nd[0], nd[1], vsource_index(c, e), wave_value(c, el, P, t));
        else if (el.kind == SP_EL_I) m.current_source(nd[0], nd[1], wave_value(c, el, P, t));
    }
}

// method: 0 BE, 1 TRAP, 2 TR-BDF2.  x[n_t] = state at tstop; probe[steps + 1]
// = unknown `probe_idx` at every step (nullptr or probe_idx < 0: none).
// Returns false when a solve hit a zero pivot.
inline bool linear_transient(const sp_circuit& c, const double* P, const double* dc, int method, double h,
                             double tstop, double* x, int probe_idx, double* probe) {
    const int nn = c.num_nodes, nt = nn + num_vsources(c);
    std::vector<int> cap_el, ind_el;
    for (int e = 0; e < c.num_elements; ++e) {
        if (c.elements[e].kind == SP_EL_C) cap_el.push_back(e);
        if (c.elements[e].kind == SP_EL_L) ind_el.push_back(e);
    }
    auto node = [&](const double* v, int i) { return i >= 0 ? v[i] : 0.0; };
    std::vector<TranState> cs(cap_el.size()), is(ind_el.size());
    for (size_t k = 0; k < cap_el.size(); ++k) {
        const sp_element& el = c.elements[cap_el[k]];
        cs[k].v_prev = node(dc, el.node[0]) - node(dc, el.node[1]);
    }
    for (size_t k = 0; k < ind_el.size(); ++k) {
        const sp_element& el = c.elements[ind_el[k]];
        is[k].v_prev = node(dc, el.node[0]) - node(dc, el.node[1]);
        is[k].i_prev = dc[nn + el.branch];
    }
    for (int i = 0; i < nn; ++i) x[i] = dc[i];
    for (int e = 0; e < c.num_elements; ++e)
        if (c.elements[e].kind == SP_EL_V) x[nn + vsource_index(c, e)] = dc[nn + c.elements[e].branch];
    const long steps = (long)std::ceil(tstop / h);
    if (probe && probe_idx >= 0) probe[0] = x[probe_idx];
    Mna m;
    m.init(nn, nt - nn);
    const double gamma = kTrbdf2Gamma;
    auto vc = [&](const sp_element& el, const double* s) { return node(s, el.node[0]) - node(s, el.node[1]); };
    auto stamp_cap = [&](int kind, double hh) {  // 0 BE, 1 TRAP, 2 BDF2 stage
        for (size_t k = 0; k < cap_el.size(); ++k) {
            const sp_element& el = c.elements[cap_el[k]];
            const double C = P[el.field[0]];
            double geq, ieq;
            if (kind == 0) {
                geq = C / hh;
                ieq = geq * cs[k].v_prev;
            } else if (kind == 1) {
                geq = 2.0 * C / hh;
                ieq = geq * cs[k].v_prev + cs[k].i_prev;
            } else {
                const double h2 = (1.0 - gamma) * hh, h1 = gamma * hh, rho = h2 / h1, denom = 1.0 + 2.0 * rho;
                const double a1 = (1.0 + rho) * (1.0 + rho) / denom, a2 = -rho * rho / denom, b0 = (1.0 + rho) / denom;
                geq = C / (b0 * h2);
                ieq = geq * (a1 * cs[k].v_prev + a2 * cs[k].pp);
            }
            m.conductance(el.node[0], el.node[1], geq);
            m.current_source(el.node[1], el.node[0], ieq);
        }
        for (size_t k = 0; k < ind_el.size(); ++k) {
            const sp_element& el = c.elements[ind_el[k]];
            const double L = P[el.field[0]];
            double geq, ieq;
            if (kind == 0) {
                geq = hh / L;
                ieq = is[k].i_prev;
            } else if (kind == 1) {
                geq = hh / (2.0 * L);
                ieq = is[k].i_prev + geq * is[k].v_prev;
            } else {
                const double h2 = (1.0 - gamma) * hh, h1 = gamma * hh, rho = h2 / h1, denom = 1.0 + 2.0 * rho;
                const double a1 = (1.0 + rho) * (1.0 + rho) / denom, a2 = -rho * rho / denom, b0 = (1.0 + rho) / denom;
                geq = b0 * h2 / L;
                ieq = a1 * is[k].i_prev + a2 * is[k].pp;
            }
            m.conductance(el.node[0], el.node[1], geq);
            m.current_source(el.node[0], el.node[1], ieq);
        }
    };
    auto solve = [&](double* out) {
        std::vector<double> A = m.A, b = m.b;
        if (!lu_solve(nt, A.data(), b.data())) return false;
        for (int i = 0; i < nt; ++i) out[i] = b[i];
        return true;
    };
    auto update = [&](const double* s, double hh, int meth) {  // CapacitorState/InductorState::update
        const double alpha = (1.0 - gamma) / (gamma * (2.0 - gamma));
        for (size_t k = 0; k < cap_el.size(); ++k) {
            const double C = P[c.elements[cap_el[k]].field[0]], v = vc(c.elements[cap_el[k]], s);
            TranState& q = cs[k];
            if (meth == 0) q.i_prev = C / hh * (v - q.v_prev);
            else if (meth == 1) q.i_prev = 2.0 * C / hh * (v - q.v_prev) - q.i_prev;
            else q.i_prev = C / hh * ((1.0 + alpha) * v - (1.0 + 2.0 * alpha) * q.v_prev + alpha * q.pp);
            q.pp = q.v_prev;
            q.v_prev = v;
        }
        for (size_t k = 0; k < ind_el.size(); ++k) {
            const double L = P[c.elements[ind_el[k]].field[0]], v = vc(c.elements[ind_el[k]], s);
            TranState& q = is[k];
            if (meth == 0) q.i_prev += hh / L * v;
            else if (meth == 1) q.i_prev += hh / (2.0 * L) * (v + q.v_prev);
            else q.i_prev += hh / L * ((1.0 + alpha) * v - (1.0 + 2.0 * alpha) * q.v_prev + alpha * q.v_prev);
            q.pp = q.i_prev;
            q.v_prev = v;
        }
    };
    std::vector<double> sg(nt);
    for (long step = 1; step <= steps; ++step) {
        const double t = (double)step * h;
        m.clear();
        stamp_static(c, P, t, m);
        if (method == 2) {
            const double hg = gamma * h;
            stamp_cap(1, hg);
            if (!solve(sg.data())) return false;
            for (size_t k = 0; k < cap_el.size(); ++k) {  // update_trbdf2_intermediate
                const double C = P[c.elements[cap_el[k]].field[0]], v = vc(c.elements[cap_el[k]], sg.data());
                TranState& q = cs[k];
                q.pp = q.v_prev;
                q.i_prev = 2.0 * C / hg * (v - q.pp) - q.i_prev;
                q.v_prev = v;
            }
            for (size_t k = 0; k < ind_el.size(); ++k) {
                const double L = P[c.elements[ind_el[k]].field[0]], v = vc(c.elements[ind_el[k]], sg.data());
                TranState& q = is[k];
                q.pp = q.i_prev;
                q.i_prev += hg / (2.0 * L) * (v + q.v_prev);
                q.v_prev = v;  // solver.rs:214: ind.v_prev = v after the intermediate update
            }
            m.clear();
            stamp_static(c, P, t, m);
            stamp_cap(2, h);
        } else {
            stamp_cap(method, h);
        }
        if (!solve(x)) return false;
        update(x, h, method);
        if (probe && probe_idx >= 0) probe[step] = x[probe_idx];
    }
    return true;
}

}  // namespace oracle
