// Batched fixed-step linear transients (solve_transient, solver.rs:41-252),
// one thread per sample, after the DC operating point of the same samples.
//
// Per step the circuit's R, V and I are stamped at t = step h in element
// order, then the capacitor and inductor companions (companion.rs: BE, TRAP,
// or the TR-BDF2 pair of stages), and the dense system is solved with the
// nalgebra-order LU of the DC path; the states follow the reference's update
// rules, including its TR-BDF2 updates as written.  Unknowns: nodes + V-source
// currents (inductors carry no branch variable in the transient MNA).  In the
// exact translation unit (no FMA) a run is bit-identical to the oracle's
// linear_transient.
#pragma once
#include <math_constants.h>

#include "newton_dense.cuh"

namespace sp {

struct TransientLaunch {
    DevCircuit c;
    const double* params;      // [count][np] (the DC pass's drawn parameters)
    int np;
    const double* x_dc;        // [count][n_dc]
    uint64_t count;
    int method;                // 0 BE, 1 TRAP, 2 TR-BDF2
    double h, tstop;
    long steps;
    int nt;                    // transient unknowns
    int num_caps, num_inds;
    int probe_idx;
    double* x;                 // [count][nt]
    double* probe;             // [count][steps + 1] or nullptr
    uint8_t* status;           // in: DC status; out: transient status
};

__host__ __device__ inline size_t transient_words(int nt, int caps, int inds) {
    return (size_t)nt * nt + 3 * (size_t)nt + 3 * (size_t)(caps + inds);
}

#ifdef SP_KERNEL_NS
namespace SP_KERNEL_NS {

__device__ inline double tr_pulse(const sp_pulse& p, double t) {
    if (t < p.td) return p.v1;
    const double t_rel = p.per > 0.0 ? fmod(t - p.td, p.per) : t - p.td;
    if (t_rel < p.tr) return p.v1 + (p.v2 - p.v1) * t_rel / p.tr;
    if (t_rel < p.tr + p.pw) return p.v2;
    if (t_rel < p.tr + p.pw + p.tf) return p.v2 - (p.v2 - p.v1) * (t_rel - p.tr - p.pw) / p.tf;
    return p.v1;
}

__global__ void transient_fixed_kernel(TransientLaunch L) {
    extern __shared__ __align__(16) double tsm[];
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = s < L.count;
    if (!live) return;  // no block-wide synchronisation below
    const DevCircuit& c = L.c;
    const int nt = L.nt, nn = c.num_nodes, bs = blockDim.x;
    double* base = tsm + threadIdx.x;
    Il<double> A{base, bs};
    Il<double> b{base + (size_t)nt * nt * bs, bs};
    Il<double> xs{base + ((size_t)nt * nt + nt) * bs, bs};
    Il<double> sg{base + ((size_t)nt * nt + 2 * nt) * bs, bs};
    Il<double> st{base + ((size_t)nt * nt + 3 * nt) * bs, bs};  // [3 per cap][3 per ind]: v_prev, i_prev, pp
    auto P = [&](int slot) { return L.params[s * L.np + slot]; };
    auto wave = [&](const sp_element& el, double t) {
        return (el.wave >= 0) ? tr_pulse(c.pulses[el.wave], t) : P(el.field[0]);
    };
    const int ndc = nn + c.num_branches;
    const double* dc = L.x_dc + s * ndc;
    double* xo = L.x + s * nt;
    if ((L.status[s] & SP_ST_MASK) != SP_ST_CONVERGED) {
        for (int i = 0; i < nt; ++i) xo[i] = CUDART_NAN;
        return;  // keeps the DC status
    }
    auto nv = [&](const double* v, int i) { return i >= 0 ? v[i] : 0.0; };
    auto nvi = [&](Il<double> v, int i) { return i >= 0 ? v[i] : 0.0; };
    // initial states and solution from the DC operating point
    {
        int kc = 0, kl = 0, kv = 0;
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            if (el.kind == SP_EL_C) {
                st[3 * kc] = nv(dc, el.node[0]) - nv(dc, el.node[1]);
                st[3 * kc + 1] = 0.0;
                st[3 * kc + 2] = 0.0;
                ++kc;
            } else if (el.kind == SP_EL_L) {
                const int o = 3 * (L.num_caps + kl);
                st[o] = nv(dc, el.node[0]) - nv(dc, el.node[1]);
                st[o + 1] = dc[nn + el.branch];
                st[o + 2] = 0.0;
                ++kl;
            } else if (el.kind == SP_EL_V) {
                xs[nn + kv] = dc[nn + el.branch];
                ++kv;
            }
        }
        for (int i = 0; i < nn; ++i) xs[i] = dc[i];
    }
    double* pr = L.probe ? L.probe + s * (L.steps + 1) : nullptr;
    if (pr && L.probe_idx >= 0) pr[0] = xs[L.probe_idx];
    const double gamma = 2.0 - 1.4142135623730951;
    auto clear = [&]() {
        for (int i = 0; i < nt * nt; ++i) A[i] = 0.0;
        for (int i = 0; i < nt; ++i) b[i] = 0.0;
    };
    auto add = [&](int r, int col, double v) { A[col * nt + r] += v; };
    auto cond = [&](int i, int j, double g) {
        if (i >= 0) add(i, i, g);
        if (j >= 0) add(j, j, g);
        if (i >= 0 && j >= 0) {
            add(i, j, -g);
            add(j, i, -g);
        }
    };
    auto isrc = [&](int i, int j, double cur) {
        if (i >= 0) b[i] += -cur;
        if (j >= 0) b[j] += cur;
    };
    auto stamp_static = [&](double t) {
        int kv = 0;
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            const int n0 = el.node[0], n1 = el.node[1];
            if (el.kind == SP_EL_R) {
                cond(n0, n1, 1.0 / P(el.field[0]));
            } else if (el.kind == SP_EL_V) {
                const int row = nn + kv;
                if (n0 >= 0) {
                    add(n0, row, 1.0);
                    add(row, n0, 1.0);
                }
                if (n1 >= 0) {
                    add(n1, row, -1.0);
                    add(row, n1, -1.0);
                }
                b[row] = wave(el, t);
                ++kv;
            } else if (el.kind == SP_EL_I) {
                isrc(n0, n1, wave(el, t));
            }
        }
    };
    auto stamp_comp = [&](int kind, double hh) {
        int kc = 0, kl = 0;
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            if (el.kind != SP_EL_C) continue;
            const double C = P(el.field[0]);
            const int o = 3 * kc++;
            double geq, ieq;
            if (kind == 0) {
                geq = C / hh;
                ieq = geq * st[o];
            } else if (kind == 1) {
                geq = 2.0 * C / hh;
                ieq = geq * st[o] + st[o + 1];
            } else {
                const double h2 = (1.0 - gamma) * hh, h1 = gamma * hh, rho = h2 / h1, denom = 1.0 + 2.0 * rho;
                const double a1 = (1.0 + rho) * (1.0 + rho) / denom, a2 = -rho * rho / denom, b0 = (1.0 + rho) / denom;
                geq = C / (b0 * h2);
                ieq = geq * (a1 * st[o] + a2 * st[o + 2]);
            }
            cond(el.node[0], el.node[1], geq);
            isrc(el.node[1], el.node[0], ieq);
        }
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            if (el.kind != SP_EL_L) continue;
            const double Lv = P(el.field[0]);
            const int o = 3 * (L.num_caps + kl++);
            double geq, ieq;
            if (kind == 0) {
                geq = hh / Lv;
                ieq = st[o + 1];
            } else if (kind == 1) {
                geq = hh / (2.0 * Lv);
                ieq = st[o + 1] + geq * st[o];
            } else {
                const double h2 = (1.0 - gamma) * hh, h1 = gamma * hh, rho = h2 / h1, denom = 1.0 + 2.0 * rho;
                const double a1 = (1.0 + rho) * (1.0 + rho) / denom, a2 = -rho * rho / denom, b0 = (1.0 + rho) / denom;
                geq = b0 * h2 / Lv;
                ieq = a1 * st[o + 1] + a2 * st[o + 2];
            }
            cond(el.node[0], el.node[1], geq);
            isrc(el.node[0], el.node[1], ieq);
        }
    };
    auto vacross = [&](const sp_element& el, Il<double> v) { return nvi(v, el.node[0]) - nvi(v, el.node[1]); };
    const double alpha = (1.0 - gamma) / (gamma * (2.0 - gamma));
    uint8_t status = SP_ST_CONVERGED;
    long done = 0;  // last completed step
    for (long step = 1; step <= L.steps && status == SP_ST_CONVERGED; ++step) {
        const double t = (double)step * L.h;
        clear();
        stamp_static(t);
        if (L.method == 2) {
            const double hg = gamma * L.h;
            stamp_comp(1, hg);
            if (!lu_solve_fp64(nt, A, b)) {
                status = SP_ST_SINGULAR;
                break;
            }
            for (int i = 0; i < nt; ++i) sg[i] = b[i];
            int kc = 0, kl = 0;
            for (int e = 0; e < c.num_elements; ++e) {
                const sp_element& el = c.el[e];
                if (el.kind == SP_EL_C) {
                    const int o = 3 * kc++;
                    const double C = P(el.field[0]), v = vacross(el, sg);
                    st[o + 2] = st[o];
                    st[o + 1] = 2.0 * C / hg * (v - st[o + 2]) - st[o + 1];
                    st[o] = v;
                }
            }
            for (int e = 0; e < c.num_elements; ++e) {
                const sp_element& el = c.el[e];
                if (el.kind == SP_EL_L) {
                    const int o = 3 * (L.num_caps + kl++);
                    const double Lv = P(el.field[0]), v = vacross(el, sg);
                    st[o + 2] = st[o + 1];
                    st[o + 1] += hg / (2.0 * Lv) * (v + st[o]);
                    st[o] = v;
                }
            }
            clear();
            stamp_static(t);
            stamp_comp(2, L.h);
        } else {
            stamp_comp(L.method, L.h);
        }
        if (!lu_solve_fp64(nt, A, b)) {
            status = SP_ST_SINGULAR;
            break;
        }
        for (int i = 0; i < nt; ++i) xs[i] = b[i];
        int kc = 0, kl = 0;
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            if (el.kind == SP_EL_C) {
                const int o = 3 * kc++;
                const double C = P(el.field[0]), v = vacross(el, xs);
                if (L.method == 0) st[o + 1] = C / L.h * (v - st[o]);
                else if (L.method == 1) st[o + 1] = 2.0 * C / L.h * (v - st[o]) - st[o + 1];
                else st[o + 1] = C / L.h * ((1.0 + alpha) * v - (1.0 + 2.0 * alpha) * st[o] + alpha * st[o + 2]);
                st[o + 2] = st[o];
                st[o] = v;
            }
        }
        for (int e = 0; e < c.num_elements; ++e) {
            const sp_element& el = c.el[e];
            if (el.kind == SP_EL_L) {
                const int o = 3 * (L.num_caps + kl++);
                const double Lv = P(el.field[0]), v = vacross(el, xs);
                if (L.method == 0) st[o + 1] += L.h / Lv * v;
                else if (L.method == 1) st[o + 1] += L.h / (2.0 * Lv) * (v + st[o]);
                else st[o + 1] += L.h / Lv * ((1.0 + alpha) * v - (1.0 + 2.0 * alpha) * st[o] + alpha * st[o]);
                st[o + 2] = st[o + 1];
                st[o] = v;
            }
        }
        if (pr && L.probe_idx >= 0) pr[step] = xs[L.probe_idx];
        done = step;
    }
    if (status != SP_ST_CONVERGED && pr && L.probe_idx >= 0)
        for (long k = done + 1; k <= L.steps; ++k) pr[k] = CUDART_NAN;  // steps after a singular solve
    for (int i = 0; i < nt; ++i) xo[i] = xs[i];
    L.status[s] = status;
}

}  // namespace SP_KERNEL_NS
#endif  // SP_KERNEL_NS

}  // namespace sp
