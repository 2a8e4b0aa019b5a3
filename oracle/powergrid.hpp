// Oracle of the power-grid corner sweep — TEST INFRASTRUCTURE ONLY.
//
// Per instance: full-step Newton (newton.rs:70-131, check_convergence
// newton.rs:134-159) from x = 0, each linearised system A x_new = b solved by
// solve_gmres_real_preconditioned (gmres/real.rs:218-397: right Jacobi
// preconditioning, restarted Arnoldi with modified Gram-Schmidt, Givens
// rotations gmres/helpers.rs:40-48, convergence on |g_{k+1}| / |b|, the
// final true residual check after each cycle) with the Jacobi preconditioner
// of preconditioner.rs:43-101 (1/diag, 1 where |diag| < 1e-30, i.e. on the
// VDD branch row).  Dot products are the scalar sequential sums of
// spicier-simd real_dot_scalar (real_dot.rs:70-76); the SIMD variants sum in
// other orders, so bitwise results of the reference are platform-dependent.
//
// Circuit (unknowns [v_0 .. v_{R C - 1}, I_vdd], node p = r C + j):
//   edges: horizontal (r,j)-(r,j+1) and vertical (r,j)-(r+1,j) resistors,
//     R = r_lo exp(u ln(r_hi/r_lo)) times the corner's scale;
//   VDD: a voltage source from node 0 to ground (mna.rs stamp_voltage_source);
//   straps: conductance strap_g from node 0 to each other corner;
//   sinks: Level-1 NMOS (level1.rs:154-191) drain at a drawn node, source at
//     ground, gate at an ideal drive VGS: the linearised current
//     ids + gds (v' - vds) is stamped as gds on the diagonal and
//     -(ids - gds vds) on the right-hand side (the gm term vanishes because
//     the gate voltage is fixed).
// Draw order (sweep index = layout = instance / 4): edges horizontal then
// vertical, row-major; then per sink its node floor(R C u) and its VGS.
#pragma once

#include <cmath>
#include <vector>

#include "oracle_core.hpp"

namespace oracle {

struct Grid {
    int R = 0, Cn = 0, n = 0;
    std::vector<double> gh, gv;  // [R][Cn-1], [R-1][Cn]
    std::vector<int> sink;
    std::vector<double> vgs;
    double vto = 0.0;
};

inline Grid grid_draw(const sp_grid_config& c, uint64_t seed, uint32_t inst) {
    Grid G;
    G.R = c.rows;
    G.Cn = c.cols;
    G.n = c.rows * c.cols + 1;
    const uint32_t layout = inst / 4, corner = inst % 4;
    const double scale = (corner & 1) ? c.r_scale_hi : c.r_scale_lo;
    G.vto = (corner & 2) ? c.vto + c.vto_shift : c.vto - c.vto_shift;
    const double lr = math_mode() == 1 ? sp::cr_log(c.r_hi / c.r_lo, nullptr) : std::log(c.r_hi / c.r_lo);
    auto rdraw = [&](uint32_t idx) {
        const double u = uniform(seed, layout, idx);
        const double e = math_mode() == 1 ? sp::cr_exp(u * lr, nullptr) : std::exp(u * lr);
        return 1.0 / (c.r_lo * e * scale);
    };
    uint32_t idx = 0;
    G.gh.resize((size_t)c.rows * (c.cols - 1));
    G.gv.resize((size_t)(c.rows - 1) * c.cols);
    for (auto& g : G.gh) g = rdraw(idx++);
    for (auto& g : G.gv) g = rdraw(idx++);
    G.sink.resize(c.num_sinks);
    G.vgs.resize(c.num_sinks);
    for (int s = 0; s < c.num_sinks; ++s) {
        G.sink[s] = (int)std::floor((double)(c.rows * c.cols) * uniform(seed, layout, idx++));
        G.vgs[s] = c.vgs_lo + uniform(seed, layout, idx++) * (c.vgs_hi - c.vgs_lo);
    }
    return G;
}

// Linearisation at x: diagonal of A and right-hand side b.
struct GridSystem {
    const sp_grid_config& c;
    const Grid& G;
    std::vector<double> diag, b;

    GridSystem(const sp_grid_config& cfg, const Grid& g) : c(cfg), G(g), diag(g.n), b(g.n) {}

    bool is_corner(int p) const {
        const int last = G.R * G.Cn - 1;
        return p == G.Cn - 1 || p == (G.R - 1) * G.Cn || p == last;
    }

    void linearise(const double* x) {
        const int R = G.R, Cn = G.Cn, nn = R * Cn;
        for (int r = 0; r < R; ++r)
            for (int j = 0; j < Cn; ++j) {
                const int p = r * Cn + j;
                double d = 0.0;
                if (j > 0) d += G.gh[r * (Cn - 1) + j - 1];
                if (j < Cn - 1) d += G.gh[r * (Cn - 1) + j];
                if (r > 0) d += G.gv[(r - 1) * Cn + j];
                if (r < R - 1) d += G.gv[r * Cn + j];
                if (p == 0) d += 3.0 * c.strap_g;
                else if (is_corner(p)) d += c.strap_g;
                diag[p] = d;
                b[p] = 0.0;
            }
        diag[nn] = 0.0;
        b[nn] = c.vdd;
        const MosParams mp{G.vto, c.kp, c.lambda, c.w, c.l, 1.0};
        for (int s = 0; s < c.num_sinks; ++s) {
            const int p = G.sink[s];
            double ids, gds, gm;
            const double vds = x[p];
            mos_evaluate(false, mp, G.vgs[s], vds, &ids, &gds, &gm);
            diag[p] += gds;
            b[p] -= ids - gds * vds;
        }
    }

    // y = A z
    void apply(const double* z, double* y) const {
        const int R = G.R, Cn = G.Cn, nn = R * Cn;
        const int c1 = Cn - 1, c2 = (R - 1) * Cn, c3 = nn - 1;
        for (int r = 0; r < R; ++r)
            for (int j = 0; j < Cn; ++j) {
                const int p = r * Cn + j;
                double v = diag[p] * z[p];
                if (j > 0) v -= G.gh[r * (Cn - 1) + j - 1] * z[p - 1];
                if (j < Cn - 1) v -= G.gh[r * (Cn - 1) + j] * z[p + 1];
                if (r > 0) v -= G.gv[(r - 1) * Cn + j] * z[p - Cn];
                if (r < R - 1) v -= G.gv[r * Cn + j] * z[p + Cn];
                if (p == 0) {
                    v -= c.strap_g * z[c1];
                    v -= c.strap_g * z[c2];
                    v -= c.strap_g * z[c3];
                    v += z[nn];
                } else if (p == c1 || p == c2 || p == c3) {
                    v -= c.strap_g * z[0];
                }
                y[p] = v;
            }
        y[nn] = z[0];
    }
};

inline double dot(const double* a, const double* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

struct GmresOutcome {
    int iterations = 0;
    bool converged = false;
    double residual = 0.0;
};

// solve_gmres_real_preconditioned (gmres/real.rs:218-397) with Jacobi.
inline GmresOutcome gmres(const GridSystem& S, const double* b, double* x, int restart, int max_iter, double tol) {
    const int n = S.G.n;
    GmresOutcome out;
    std::vector<double> inv(n);
    for (int i = 0; i < n; ++i) inv[i] = std::fabs(S.diag[i]) < 1e-30 ? 1.0 : 1.0 / S.diag[i];
    const double b_norm = std::sqrt(dot(b, b, n));
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    if (b_norm < 1e-30) {
        out.converged = true;
        return out;
    }
    const int m = std::min(restart, n);
    std::vector<std::vector<double>> v(m + 1, std::vector<double>(n)), z(m, std::vector<double>(n));
    std::vector<std::vector<double>> h(m, std::vector<double>(m + 1));
    std::vector<double> ax(n), w(n), g(m + 1), cs(m), sn(m), y(m);
    int total = 0;
    for (int cycle = 0; cycle < max_iter; ++cycle) {
        S.apply(x, ax.data());
        for (int i = 0; i < n; ++i) v[0][i] = b[i] - ax[i];
        const double r_norm = std::sqrt(dot(v[0].data(), v[0].data(), n));
        if (r_norm / b_norm < tol) {
            out.converged = true;
            out.residual = r_norm / b_norm;
            out.iterations = total;
            return out;
        }
        const double inv_r = 1.0 / r_norm;
        for (int i = 0; i < n; ++i) v[0][i] *= inv_r;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = r_norm;
        int k = 0;
        while (k < m) {
            ++total;
            if (total > max_iter) break;
            for (int i = 0; i < n; ++i) z[k][i] = v[k][i] * inv[i];
            S.apply(z[k].data(), w.data());
            for (int j = 0; j <= k; ++j) {
                const double hij = dot(v[j].data(), w.data(), n);
                h[k][j] = hij;
                for (int i = 0; i < n; ++i) w[i] -= hij * v[j][i];
            }
            const double w_norm = std::sqrt(dot(w.data(), w.data(), n));
            h[k][k + 1] = w_norm;
            if (w_norm < 1e-30) {
                ++k;
                break;
            }
            const double inv_w = 1.0 / w_norm;
            for (int i = 0; i < n; ++i) v[k + 1][i] = w[i] * inv_w;
            for (int j = 0; j < k; ++j) {
                const double temp = cs[j] * h[k][j] + sn[j] * h[k][j + 1];
                h[k][j + 1] = -sn[j] * h[k][j] + cs[j] * h[k][j + 1];
                h[k][j] = temp;
            }
            double cc = 1.0, ss = 0.0;  // real_givens_rotation (helpers.rs:40-48)
            if (std::fabs(h[k][k + 1]) >= 1e-30) {
                const double r = std::sqrt(h[k][k] * h[k][k] + h[k][k + 1] * h[k][k + 1]);
                cc = h[k][k] / r;
                ss = h[k][k + 1] / r;
            }
            cs[k] = cc;
            sn[k] = ss;
            const double temp = cc * h[k][k] + ss * h[k][k + 1];
            h[k][k + 1] = 0.0;
            h[k][k] = temp;
            const double tg = cc * g[k] + ss * g[k + 1];
            g[k + 1] = -ss * g[k] + cc * g[k + 1];
            g[k] = tg;
            const double rel = std::fabs(g[k + 1]) / b_norm;
            ++k;
            if (rel < tol) break;
        }
        for (int i = k - 1; i >= 0; --i) {
            double sum = g[i];
            for (int j = i + 1; j < k; ++j) sum -= h[j][i] * y[j];
            y[i] = std::fabs(h[i][i]) > 1e-30 ? sum / h[i][i] : 0.0;
        }
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < n; ++j) x[j] += z[i][j] * y[i];
        S.apply(x, ax.data());
        double fr = 0.0;
        for (int i = 0; i < n; ++i) fr += (b[i] - ax[i]) * (b[i] - ax[i]);
        fr = std::sqrt(fr);
        out.residual = fr / b_norm;
        out.iterations = total;
        if (fr / b_norm < tol) {
            out.converged = true;
            return out;
        }
        if (total >= max_iter) return out;
    }
    return out;
}

struct GridOutcome {
    uint8_t status = SP_ST_FAILED;
    int newton = 0, krylov = 0;
    double resid = 0.0;  // max |KCL residual| at the final iterate (A)
};

inline GridOutcome grid_solve(const sp_grid_config& c, const Grid& G, double* x) {
    GridSystem S(c, G);
    GridOutcome out;
    const int n = G.n, nn = n - 1;
    std::vector<double> xn(n), Ax(n);
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    for (int it = 1; it <= c.max_newton; ++it) {
        S.linearise(x);
        GmresOutcome go = gmres(S, S.b.data(), xn.data(), c.restart, c.max_krylov, c.krylov_tol);
        out.krylov += go.iterations;
        bool conv = true, fin = true;
        for (int i = 0; i < n; ++i) {
            const double tol = c.v_reltol * std::fmax(std::fabs(xn[i]), std::fabs(x[i])) + (i < nn ? c.v_abstol : c.i_abstol);
            conv = conv && std::fabs(xn[i] - x[i]) <= tol;
            fin = fin && std::isfinite(xn[i]);
            x[i] = xn[i];
        }
        out.newton = it;
        if (!fin) {
            out.status = SP_ST_NONFINITE;
            break;
        }
        if (conv) {
            out.status = SP_ST_CONVERGED;
            break;
        }
    }
    // KCL residual of the nonlinear circuit at x: A(x) x - b(x)
    S.linearise(x);
    S.apply(x, Ax.data());
    double r = 0.0;
    for (int i = 0; i < nn; ++i) r = std::fmax(r, std::fabs(Ax[i] - S.b[i]));
    out.resid = r;
    return out;
}

}  // namespace oracle
