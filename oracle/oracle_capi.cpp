// C ABI of the CPU oracle (TEST INFRASTRUCTURE ONLY; see oracle_core.hpp).
//
// Loaded with ctypes by tests/ and by bench.py's CPU-baseline leg.  The
// multi-sample entry points spread samples over a pool of std::threads with
// an atomic work counter, the shape of solve_batched_sweep_parallel's rayon
// par_iter (crates/spicier-batched-sweep/src/parallel.rs:142-156): one
// independent solver state per worker, samples handed out in small chunks.
#include <algorithm>
#include <climits>
#include <atomic>
#include <thread>

#include "oracle_core.hpp"
#include "transient.hpp"
#include "ac.hpp"
#include "powergrid.hpp"


using namespace oracle;

namespace {

template <class F>
void parallel_for(uint64_t count, int threads, F&& body) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (threads == 1 || count < 2) {
        body(0, 0, count);
        return;
    }
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = 16;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&, t] {
            for (;;) {
                uint64_t lo = next.fetch_add(chunk);
                if (lo >= count) break;
                body(t, lo, std::min(count, lo + chunk));
            }
        });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

uint64_t or_splitmix64(uint64_t x) { return splitmix64(x); }
uint64_t or_combine_indices(uint64_t seed, uint32_t s, uint32_t p) { return combine_indices(seed, s, p); }
double or_uniform(uint64_t seed, uint32_t s, uint32_t p) { return uniform(seed, s, p); }
float or_uniform_f32(uint64_t seed, uint32_t s, uint32_t p) { return uniform_f32(seed, s, p); }
double or_gaussian(uint64_t seed, uint32_t s, uint32_t p) { return gaussian(seed, s, p); }
float or_gaussian_f32(uint64_t seed, uint32_t s, uint32_t p) { return gaussian_f32(seed, s, p); }
void or_set_math_mode(int mode) { math_mode() = mode; }
int or_get_math_mode() { return math_mode(); }
double or_cr_log(double x, unsigned* hard) { return sp::cr_log(x, hard); }
double or_cr_cos(double x, unsigned* hard) { return sp::cr_cos(x, hard); }
void or_cr_log_batch(const double* x, uint64_t n, double* y, unsigned* hard) {
    for (uint64_t i = 0; i < n; ++i) y[i] = sp::cr_log(x[i], hard);
}
void or_cr_cos_batch(const double* x, uint64_t n, double* y, unsigned* hard) {
    for (uint64_t i = 0; i < n; ++i) y[i] = sp::cr_cos(x[i], hard);
}
void or_cr_exp_batch(const double* x, uint64_t n, double* y, unsigned* hard) {
    for (uint64_t i = 0; i < n; ++i) y[i] = sp::cr_exp(x[i], hard);
}
// the 128-bit evaluations alone (no 64-bit fast path), to check the fast paths against
void or_cr_log_full_batch(const double* x, uint64_t n, double* y, unsigned* hard) {
    for (uint64_t i = 0; i < n; ++i) y[i] = sp::cr_log_impl(x[i], hard, false);
}
void or_cr_cos_full_batch(const double* x, uint64_t n, double* y, unsigned* hard) {
    for (uint64_t i = 0; i < n; ++i) y[i] = sp::cr_cos_impl(x[i], hard, false);
}
// the integer multiply / divide / square root of cr_math.cuh against the
// host's IEEE operators on n random normal operands (mismatches returned)
uint64_t or_ieee_int_mismatches(uint64_t seed, uint64_t n) {
    uint64_t st = seed, bad = 0;
    auto next = [&]() { st = oracle::splitmix64(st); return st; };
    auto rnd = [&](int elo, int ehi) {
        const uint64_t m = next() & ((1ULL << 52) - 1);
        const int e = elo + (int)(next() % (uint64_t)(ehi - elo + 1));
        return sp::cr::bdouble(((uint64_t)(e + 1023) << 52) | m);
    };
    for (uint64_t i = 0; i < n; ++i) {
        const double a = rnd(-400, 400), b = rnd(-400, 400), sa = (next() & 1) ? -a : a;
        bad += sp::cr::dbits(sp::cr::mul_rn(sa, b)) != sp::cr::dbits(sa * b);
        bad += sp::cr::dbits(sp::cr::div_pos(a, b)) != sp::cr::dbits(a / b);
        bad += sp::cr::dbits(sp::cr::sqrt_pos(a)) != sp::cr::dbits(std::sqrt(a));
    }
    return bad;
}

// how often the ln fast path hands over to the 128-bit evaluation
uint64_t or_cr_fast_misses(int fn, const double* x, uint64_t n) {
    uint64_t miss = 0;
    for (uint64_t i = 0; i < n && fn == 0; ++i) {
        double r;
        const uint64_t b = sp::cr::dbits(x[i]);
        const int bexp = (int)(b >> 52);
        if (bexp < 1023 - 360 || bexp > 1023 + 359) continue;
        if (b > 0x3FEFFFE000000000ULL && b < 0x3FF0001000000000ULL) continue;
        miss += sp::cr::ln_fast(bexp - 1023, b & ((1ULL << 52) - 1), &r) ? 0 : 1;
    }
    return miss;
}

// kind: 0 uniform, 1 gaussian, 2 uniform_f32, 3 gaussian_f32 (sp_rng_fill_device).
void or_rng_fill(int kind, uint64_t seed, uint64_t first, uint32_t param, uint64_t count,
                 double* out) {
    for (uint64_t i = 0; i < count; ++i) {
        uint32_t s = (uint32_t)(first + i);
        switch (kind) {
            case 0: out[i] = uniform(seed, s, param); break;
            case 1: out[i] = gaussian(seed, s, param); break;
            case 2: out[i] = (double)uniform_f32(seed, s, param); break;
            default: out[i] = (double)gaussian_f32(seed, s, param); break;
        }
    }
}

int or_mos_evaluate(int pmos, const double* p6, double vgs, double vds, double* out3) {
    MosParams mp{p6[0], p6[1], p6[2], p6[3], p6[4], p6[5]};
    return mos_evaluate(pmos != 0, mp, vgs, vds, &out3[0], &out3[1], &out3[2]);
}

// Bsim3Mosfet::evaluate for `count` devices: card[i][SP_B3_CARD], bias[i][3] =
// (vgs, vds, vbs); out[i][6] = (ids, gds, gm, gmbs, vth, vdsat), region[i].
void or_bsim3_evaluate(int pmos, const double* card, const double* bias, uint64_t count, double* out,
                       uint8_t* region) {
    const bool cr = math_mode() == 1;
    for (uint64_t i = 0; i < count; ++i) {
        const double* c = card + i * SP_B3_CARD;
        const Bsim3Eval r = bsim3_evaluate(pmos != 0, c, bsim3_derive(c, cr), bias[3 * i], bias[3 * i + 1],
                                           bias[3 * i + 2], cr);
        double* o = out + 6 * i;
        o[0] = r.ids, o[1] = r.gds, o[2] = r.gm, o[3] = r.gmbs, o[4] = r.vth, o[5] = r.vdsat;
        if (region) region[i] = (uint8_t)r.region;
    }
}
void or_bsim3_default_card(int pmos, double* card) { bsim3_default_card(pmos != 0, card); }

void or_diode_evaluate(double is, double n, double vd, double* out2) {
    diode_evaluate(is, n, vd, &out2[0], &out2[1]);
}

double or_limit_voltage(double vd, double nvt) { return limit_voltage(vd, nvt); }
double or_thermal_voltage(double t) { return thermal_voltage(t); }

void or_bjt_evaluate(int pnp, const double* p6, double vbe, double vce, double* out6) {
    BjtParams bp{p6[0], p6[1], p6[2], p6[3], p6[4], p6[5]};
    bjt_evaluate(pnp != 0, bp, vbe, vce, out6);
}

// mode: 0 plain, 1 gmin (aux = gmin), 2 source-scaled (aux = factor).
// A receives the column-major dense matrix, b the RHS.
int or_stamp_dc(const sp_circuit* c, const double* P, const double* x, int mode, double aux,
                double* A, double* b) {
    Mna m;
    m.init(c->num_nodes, c->num_branches);
    stamp_dc(*c, P, x, m, mode == 2, aux);
    if (mode == 1) m.gmin(aux);
    std::copy(m.A.begin(), m.A.end(), A);
    std::copy(m.b.begin(), m.b.end(), b);
    return 0;
}

// nalgebra-style LU solve in place; returns 1 when singular.
int or_lu_solve(int n, double* A, double* b) { return lu_solve(n, A, b) ? 0 : 1; }

// CpuBatchedSolver::solve_batch (crates/spicier-batched-sweep/src/solver.rs:326-384):
// singular systems get zero solutions and singular[i] = 1.
void or_solve_batch(const double* mats, const double* rhs, uint64_t n, uint64_t batch,
                    double* sol, uint8_t* singular, int threads) {
    parallel_for(batch, threads, [&](int, uint64_t lo, uint64_t hi) {
        std::vector<double> A(n * n);
        for (uint64_t i = lo; i < hi; ++i) {
            std::copy(mats + i * n * n, mats + (i + 1) * n * n, A.begin());
            double* x = sol + i * n;
            std::copy(rhs + i * n, rhs + (i + 1) * n, x);
            bool ok = lu_solve((int)n, A.data(), x);
            if (!ok) std::fill(x, x + n, 0.0);
            singular[i] = ok ? 0 : 1;
        }
    });
}

int or_draw_params(const sp_circuit* c, uint64_t seed, uint64_t first, uint64_t count,
                   const double* table, uint32_t cols, double* out) {
    for (uint64_t i = 0; i < count; ++i) {
        const double* row = table ? table + i * cols : nullptr;
        for (int k = 0; k < c->num_params; ++k)
            out[i * c->num_params + k] = draw_param(c->params[k], seed, (uint32_t)(first + i), row);
    }
    return 0;
}

// One Newton-Raphson solve (mode 0 plain, 1 gmin with aux, 2 scaled with aux).
// Returns bit0 converged, bit1 singular; *iters iterations.  x: guess in, result out.
int or_newton_single(const sp_circuit* c, const double* P, const sp_newton_config* cfg, int mode,
                     double aux, double* x, int* iters) {
    Mna m;
    m.init(c->num_nodes, c->num_branches);
    StampMode sm = mode == 1 ? StampMode::Gmin : mode == 2 ? StampMode::Scaled : StampMode::Plain;
    NrOutcome r = newton(*c, P, *cfg, sm, aux, x, m);
    *iters = r.iterations;
    return (r.converged ? 1 : 0) | (r.singular ? 2 : 0);
}

// which: 0 gmin stepping, 1 source stepping.  out3 = {converged, total_iterations, num_levels}.
int or_stepping(const sp_circuit* c, const double* P, const sp_newton_config* cfg, int which,
                double* x, int* out3) {
    Mna m;
    m.init(c->num_nodes, c->num_branches);
    SteppingOutcome s =
        which == 0 ? gmin_stepping(*c, P, *cfg, x, m) : source_stepping(*c, P, *cfg, x, m);
    out3[0] = s.converged;
    out3[1] = s.total_iterations;
    out3[2] = s.num_levels;
    return s.singular ? 1 : 0;
}

// Batched DC operating points: the CPU restatement of sp_newton_dc.
int or_newton_dc(const sp_circuit* c, const sp_newton_config* cfg, uint64_t seed, uint64_t first,
                 uint64_t count, const double* table, uint32_t cols, const double* x0, double* x,
                 int32_t* iters, uint8_t* status, double* params, int threads) {
    const int n = c->num_nodes + c->num_branches;
    const int np = c->num_params;
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        Mna m;
        m.init(c->num_nodes, c->num_branches);
        std::vector<double> P(np);
        for (uint64_t i = lo; i < hi; ++i) {
            const double* row = table ? table + i * cols : nullptr;
            for (int k = 0; k < np; ++k)
                P[k] = draw_param(c->params[k], seed, (uint32_t)(first + i), row);
            if (params) std::copy(P.begin(), P.end(), params + i * np);
            int it = 0;
            uint8_t st = dc_pipeline(*c, P.data(), *cfg, x0 ? x0 + i * n : nullptr, x + i * n, &it, m);
            if (iters) iters[i] = it;
            if (status) status[i] = st;
        }
    });
    return 0;
}

// AC frequency grid (ac.rs:258-287): writes up to cap values, returns the count.
int or_ac_frequencies(double fstart, double fstop, int num_points, int sweep, double* out, int cap) {
    const std::vector<double> f = ac_frequencies(fstart, fstop, num_points, sweep);
    for (int i = 0; i < (int)f.size() && i < cap; ++i) out[i] = f[i];
    return (int)f.size();
}

// Batched AC sweep: per sample the draws, the DC pipeline, then the complex
// solve at every frequency; probe[count][nf][np] complex (re, im) values of
// the given unknowns; status: the DC status, or SP_ST_SINGULAR when a
// frequency's matrix was singular (its probes NaN).
int or_ac_sweep(const sp_circuit* c, const sp_newton_config* cfg, uint64_t seed, uint64_t first, uint64_t count,
                const double* table, uint32_t cols, const double* freqs, int nf, int source, const int* probes,
                int np, double* probe, uint8_t* status, int threads) {
    const int n = c->num_nodes + c->num_branches;
    const int npar = c->num_params;
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        Mna m;
        m.init(c->num_nodes, c->num_branches);
        std::vector<double> P(npar), x(n);
        std::vector<Cx> A((size_t)n * n), b(n);
        for (uint64_t i = lo; i < hi; ++i) {
            const double* row = table ? table + i * cols : nullptr;
            for (int k = 0; k < npar; ++k) P[k] = draw_param(c->params[k], seed, (uint32_t)(first + i), row);
            int it = 0;
            uint8_t st = dc_pipeline(*c, P.data(), *cfg, nullptr, x.data(), &it, m);
            double* out = probe + i * (size_t)nf * np * 2;
            if ((st & SP_ST_MASK) != SP_ST_CONVERGED) {
                for (size_t k = 0; k < (size_t)nf * np * 2; ++k) out[k] = NAN;
                status[i] = st;
                continue;
            }
            const AcLinear L = ac_linearise(*c, P.data(), x.data(), source);
            for (int f = 0; f < nf; ++f) {
                const double w = 2.0 * 3.141592653589793 * freqs[f];
                ac_matrix(*c, P.data(), L, w, A.data(), b.data());
                const bool ok = lu_solve_complex(n, A.data(), b.data());
                if (!ok) st = (uint8_t)((st & ~SP_ST_MASK) | SP_ST_SINGULAR);
                for (int k = 0; k < np; ++k) {
                    out[((size_t)f * np + k) * 2] = ok ? b[probes[k]].re : NAN;
                    out[((size_t)f * np + k) * 2 + 1] = ok ? b[probes[k]].im : NAN;
                }
            }
            status[i] = st;
        }
    });
    return 0;
}

// StatisticsAccumulator over column `col` (statistics.rs:113-160), samples in
// index order, optionally restricted to converged status bytes.
void or_moments(const double* values, uint64_t rows, uint32_t ld, uint32_t col,
                const uint8_t* status, sp_moments* out) {
    sp_moments m{0, 0.0, 0.0, INFINITY, -INFINITY};
    for (uint64_t i = 0; i < rows; ++i) {
        if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
        double v = values[i * ld + col];
        m.count += 1;
        m.sum += v;
        m.sum_sq += v * v;
        m.min = std::fmin(m.min, v);
        m.max = std::fmax(m.max, v);
    }
    *out = m;
}

// Histogram::new (statistics.rs:243-268) over column `col`, converged rows only
// when status is given.  Rust's `as isize` saturates and maps NaN to 0.
void or_histogram(const double* v, uint64_t rows, uint32_t ld, uint32_t col, const uint8_t* status, double mn,
                  double mx, uint32_t nb, uint64_t* bins) {
    const double width = (mx - mn) / (double)nb;
    for (uint32_t b = 0; b < nb; ++b) bins[b] = 0;
    for (uint64_t i = 0; i < rows; ++i) {
        if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
        const double f = std::floor((v[i * ld + col] - mn) / width);
        long long b = std::isnan(f) ? 0 : (f < -9.2e18 ? LLONG_MIN : (f > 9.2e18 ? LLONG_MAX : (long long)f));
        b = std::min<long long>(std::max<long long>(b, 0), (long long)nb - 1);
        bins[b] += 1;
    }
}

// YieldSpec::passes / YieldAnalysis::all_pass (statistics.rs:347-428).
void or_yield(const double* v, uint64_t rows, uint32_t ld, const uint8_t* status, const sp_yield_spec* specs,
              uint32_t ns, uint64_t* pass) {
    for (uint32_t k = 0; k <= ns; ++k) pass[k] = 0;
    for (uint64_t i = 0; i < rows; ++i) {
        if (status && (status[i] & SP_ST_MASK) != SP_ST_CONVERGED) continue;
        bool all = true;
        for (uint32_t k = 0; k < ns; ++k) {
            const double x = v[i * ld + specs[k].col];
            const bool ok = x >= specs[k].lower && x <= specs[k].upper;
            all = all && ok;
            pass[k] += ok ? 1 : 0;
        }
        pass[ns] += all ? 1 : 0;
    }
}

// Power-grid corner instances first..first+count-1: x[count][rows*cols+1].
void or_grid_solve(const sp_grid_config* c, uint64_t seed, uint64_t first, uint64_t count, double* x,
                   int32_t* newton, int32_t* krylov, uint8_t* status, double* resid, int threads) {
    const int n = c->rows * c->cols + 1;
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            Grid G = grid_draw(*c, seed, (uint32_t)(first + i));
            GridOutcome o = grid_solve(*c, G, x + i * n);
            newton[i] = o.newton;
            krylov[i] = o.krylov;
            status[i] = o.status;
            resid[i] = o.resid;
        }
    });
}

// Sink nodes and gate drives of instance `inst` (arrays of num_sinks).
void or_grid_sinks(const sp_grid_config* c, uint64_t seed, uint32_t inst, int32_t* node, double* vgs) {
    Grid G = grid_draw(*c, seed, inst);
    for (int s = 0; s < c->num_sinks; ++s) {
        node[s] = G.sink[s];
        vgs[s] = G.vgs[s];
    }
}

// Fixed-step linear transients of samples first..first+count-1: the DC
// operating point by the DC pipeline, then solve_transient.  x[count][nt],
// probe[count][steps + 1] (probe_idx < 0: none), status SP_ST_*.
void or_transient(const sp_circuit* c, const sp_newton_config* cfg, uint64_t seed, uint64_t first, uint64_t count,
                  const double* table, uint32_t cols, int method, double h, double tstop, int probe_idx, double* x,
                  double* probe, uint8_t* status, int threads) {
    const int n = c->num_nodes + c->num_branches, np = c->num_params;
    const int nt = c->num_nodes + num_vsources(*c);
    const long steps = (long)std::ceil(tstop / h);
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        Mna m;
        m.init(c->num_nodes, c->num_branches);
        std::vector<double> P(np), dc(n);
        for (uint64_t i = lo; i < hi; ++i) {
            const double* row = table ? table + i * cols : nullptr;
            for (int k = 0; k < np; ++k) P[k] = draw_param(c->params[k], seed, (uint32_t)(first + i), row);
            int it = 0;
            uint8_t st = dc_pipeline(*c, P.data(), *cfg, nullptr, dc.data(), &it, m);
            if ((st & SP_ST_MASK) == SP_ST_CONVERGED &&
                !linear_transient(*c, P.data(), dc.data(), method, h, tstop, x + i * nt, probe_idx,
                                  probe ? probe + i * (steps + 1) : nullptr))
                st = SP_ST_SINGULAR;
            status[i] = st;
        }
    });
}

// Section draws of ladder instance `inst` (R, C with room for max_sections).
int or_ladder_draw(const sp_ladder_config* c, uint64_t seed, uint32_t inst, double* R, double* C) {
    Ladder L = ladder_draw(*c, seed, inst);
    for (int k = 1; k <= L.N; ++k) {
        R[k - 1] = 1.0 / L.g[k];
        C[k - 1] = L.C[k];
    }
    return L.N;
}

// Ladder transients of instances first..first+count-1: x_final[count][max_sections+2],
// probe[count][num_probe].
void or_ladder_transient(const sp_ladder_config* c, uint64_t seed, uint64_t first, uint64_t count,
                         double* x_final, int32_t* n, int32_t* accepted, int32_t* rejected, int32_t* iters,
                         uint8_t* status, double* probe, int threads) {
    const int ld = c->max_sections + 2;
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        std::vector<double> pr(std::max(c->num_probe, 1));
        for (uint64_t i = lo; i < hi; ++i) {
            Ladder L = ladder_draw(*c, seed, (uint32_t)(first + i));
            LadderOutcome o = ladder_transient(*c, L, x_final + i * ld, pr.data());
            for (int k = L.N + 2; k < ld; ++k) x_final[i * ld + k] = 0.0;
            if (probe) std::copy(pr.begin(), pr.begin() + c->num_probe, probe + i * c->num_probe);
            n[i] = L.N + 2;
            accepted[i] = o.accepted;
            rejected[i] = o.rejected;
            iters[i] = o.iterations;
            status[i] = o.status;
        }
    });
}

// The accepted step sizes of the adaptive runs of ladders first .. first +
// count - 1: steps[i][0..min(nsteps[i], max_rec)-1].
void or_ladder_steps(const sp_ladder_config* c, uint64_t seed, uint64_t first, uint64_t count, double* steps,
                     int max_rec, int32_t* nsteps, int threads) {
    const int ld = c->max_sections + 2;
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        std::vector<double> pr(std::max(c->num_probe, 1)), x(ld);
        for (uint64_t i = lo; i < hi; ++i) {
            Ladder L = ladder_draw(*c, seed, (uint32_t)(first + i));
            LadderOutcome o = ladder_transient(*c, L, x.data(), pr.data());
            nsteps[i] = (int32_t)o.steps.size();
            for (int k = 0; k < max_rec; ++k) steps[i * (uint64_t)max_rec + k] = k < nsteps[i] ? o.steps[k] : 0.0;
        }
    });
}

// The ladders first .. first + count - 1 replayed along recorded step
// sequences: steps[i][0..nsteps[i]-1] (row stride max_rec) are instance i's
// accepted step sizes; outputs as or_ladder_transient (rejected stays 0).
void or_ladder_replay(const sp_ladder_config* c, uint64_t seed, uint64_t first, uint64_t count, const double* steps,
                      int max_rec, const int32_t* nsteps, double* x_final, int32_t* iters, uint8_t* status,
                      double* probe, int threads) {
    const int ld = c->max_sections + 2;
    parallel_for(count, threads, [&](int, uint64_t lo, uint64_t hi) {
        std::vector<double> pr(std::max(c->num_probe, 1));
        for (uint64_t i = lo; i < hi; ++i) {
            Ladder L = ladder_draw(*c, seed, (uint32_t)(first + i));
            const int ns = std::min(std::max(nsteps[i], 0), max_rec);
            LadderOutcome o = ladder_transient(*c, L, x_final + i * ld, pr.data(), steps + i * (uint64_t)max_rec, ns);
            for (int k = L.N + 2; k < ld; ++k) x_final[i * ld + k] = 0.0;
            if (probe) std::copy(pr.begin(), pr.begin() + c->num_probe, probe + i * c->num_probe);
            iters[i] = o.iterations;
            status[i] = o.status;
        }
    });
}

}  // extern "C"
