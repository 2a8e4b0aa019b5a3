// sp_draw_params_host: the per-sample parameter draws computed on the host
// with the C library's ln, cos and exp, as the reference draws them.
//
// The reference evaluates its Gaussian draws on the host
// (crates/spicier-batched-sweep/src/rng.rs:120-131: Box-Muller with Rust's
// f64::ln and f64::cos, which call the platform's libm).  Those functions are
// not correctly rounded, so the reference's draws are the host libm's bits,
// and they differ between platforms.  The device draw kernel returns the
// correctly rounded Box-Muller value, which equals the libm's wherever the
// libm rounds correctly (about 99.8 % of draws on glibc).  A caller that needs
// the reference's exact bits on this host draws here instead and passes the
// result to a sweep as its parameter table (every slot a table column).
//
// Operation order (no contraction: this file is compiled with
// -ffp-contract=off, and Rust never fuses a * b + c):
//   GAUSS       a + (sqrt(-2 ln(max(u1, 1e-10))) * cos(2 pi u2)) * b  (rng.rs:120-150)
//   UNIFORM     a + u * (b - a)
//   LOGUNIFORM  a * exp(u * ln(b / a))
//   FIXED       a;   TABLE  table[i][col]  (NaN without a table)
// with u, u1, u2 the hash RNG's uniforms (rng.rs:39-95), integer-exact.
#include <cmath>
#include <thread>
#include <vector>

#include "internal.h"
#include "rng.cuh"

namespace {

double host_draw(const sp_param& p, uint64_t seed, uint32_t sweep, const double* row) {
    switch (p.kind) {
        case SP_DRAW_FIXED: return p.a;
        case SP_DRAW_GAUSS: {
            double u1 = sp::rng_uniform(seed, sweep, p.rng_index * 2u);
            const double u2 = sp::rng_uniform(seed, sweep, p.rng_index * 2u + 1u);
            u1 = std::fmax(u1, 1e-10);
            const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
            return p.a + z * p.b;
        }
        case SP_DRAW_UNIFORM: return p.a + sp::rng_uniform(seed, sweep, p.rng_index) * (p.b - p.a);
        case SP_DRAW_LOGUNIFORM:
            return p.a * std::exp(sp::rng_uniform(seed, sweep, p.rng_index) * std::log(p.b / p.a));
        case SP_DRAW_TABLE: return row ? row[p.rng_index] : NAN;
    }
    return NAN;
}

}  // namespace

extern "C" int sp_draw_params_host(const sp_circuit* circuit, uint64_t seed, uint64_t first_index,
                                   uint64_t num_samples, const double* table, uint32_t table_cols, double* out,
                                   int threads) {
    if (!circuit || (num_samples && !out) || circuit->num_params < 0 || (circuit->num_params && !circuit->params))
        return SP_ERR_INVALID_ARGUMENT;
    if (first_index + num_samples > 0x100000000ull) return SP_ERR_INVALID_ARGUMENT;
    const int np = circuit->num_params;
    for (int k = 0; k < np; ++k) {
        const sp_param& p = circuit->params[k];
        if (p.kind < SP_DRAW_FIXED || p.kind > SP_DRAW_TABLE) return SP_ERR_INVALID_ARGUMENT;
        if (p.kind == SP_DRAW_TABLE && table && p.rng_index >= table_cols) return SP_ERR_INVALID_DIMENSION;
    }
    if (num_samples == 0 || np == 0) return SP_OK;
    unsigned nt = threads > 0 ? (unsigned)threads : std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    if ((uint64_t)nt > num_samples) nt = (unsigned)num_samples;
    auto body = [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            const double* row = table ? table + i * table_cols : nullptr;
            for (int k = 0; k < np; ++k)
                out[i * np + k] = host_draw(circuit->params[k], seed, (uint32_t)(first_index + i), row);
        }
    };
    if (nt == 1) {
        body(0, num_samples);
        return SP_OK;
    }
    std::vector<std::thread> pool;
    const uint64_t chunk = (num_samples + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t lo = t * chunk, hi = std::min<uint64_t>(num_samples, lo + chunk);
        if (lo < hi) pool.emplace_back(body, lo, hi);
    }
    for (auto& th : pool) th.join();
    return SP_OK;
}
