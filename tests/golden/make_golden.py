#!/usr/bin/env python3
"""Writes the golden vectors of tests/golden/ (run from the repository root):

    python tests/golden/make_golden.py

rng_golden.json   hash-RNG draws computed here in pure Python (integers) and
                  mpmath (ln, cos at 300 bits, rounded to nearest double):
                  SplitMix64 values, uniform draws and Box-Muller Gaussian
                  draws z = sqrt(-2 ln max(u1, 1e-10)) cos(2pi_d u2), the
                  formula of crates/spicier-batched-sweep/src/rng.rs:120-131
                  with correctly rounded ln and cos.
cr_math_golden.json  correctly rounded ln, cos and exp at inputs chosen to be
                  hard for fixed-precision evaluation: ln(1 - k 2^-53), ln(1 +
                  k 2^-52), u1 grid values, cos next to multiples of pi/2, exp
                  of k 2^-53 and of log-uniform exponents.

No reference code runs here: the SplitMix64 finaliser and the index mixing
are restated from the reference's rng.rs (lines 39-56, 80-85), and every
other value comes from mpmath.
"""
import json
import math
import os
import random
import struct

import mpmath as mp
from mpmath.libmp import to_float

mp.mp.prec = 300
HERE = os.path.dirname(os.path.abspath(__file__))
M64 = (1 << 64) - 1
TWO_PI = 6.283185307179586  # 2.0 * std::f64::consts::PI, exact product


def hexbits(x: float) -> str:
    return struct.pack(">d", x).hex()


def splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def combine(seed: int, sweep: int, param: int) -> int:
    return (seed ^ ((sweep * 0x517CC1B727220A95) & M64) ^ ((param * 0x5851F42D4C957F2D) & M64)) & M64


def uniform(seed, sweep, param) -> float:
    return float(splitmix64(combine(seed, sweep, param)) >> 11) * 2.0 ** -53


def cr(fn, x: float) -> float:
    return to_float(fn(mp.mpf(x))._mpf_, rnd="n")


def gaussian(seed, sweep, param) -> float:
    u1 = max(uniform(seed, sweep, 2 * param), 1e-10)
    u2 = uniform(seed, sweep, 2 * param + 1)
    return math.sqrt(-2.0 * cr(mp.log, u1)) * cr(mp.cos, TWO_PI * u2)


def rng_golden():
    rnd = random.Random(20260101)
    cases = [(1, 0, 0), (1, 1, 3), (7, 123456, 13), (12345, 2 ** 32 - 1, 2 ** 31 - 1), (0, 0, 0)]
    cases += [(rnd.getrandbits(64), rnd.getrandbits(32), rnd.getrandbits(20)) for _ in range(251)]
    out = {"splitmix64": [[f"{v:016x}", f"{splitmix64(v):016x}"] for v in
                          [0, 1, 0x9E3779B97F4A7C15, M64] + [rnd.getrandbits(64) for _ in range(12)]],
           "uniform": [], "gaussian": []}
    for seed, sweep, param in cases:
        out["uniform"].append([f"{seed:016x}", sweep, param, hexbits(uniform(seed, sweep, param))])
    # a contiguous block too (the GPU fill kernel draws sweeps first..first+n)
    for s in range(4096):
        out["gaussian"].append([f"{1:016x}", s, 3, hexbits(gaussian(1, s, 3))])
    for seed, sweep, param in cases:
        param &= (1 << 30) - 1
        out["gaussian"].append([f"{seed:016x}", sweep, param, hexbits(gaussian(seed, sweep, param))])
    return out


def cr_golden():
    rnd = random.Random(7)
    logs = [1.0 - k * 2.0 ** -53 for k in range(1, 400)]
    logs += [1.0 + k * 2.0 ** -52 for k in range(1, 200)]
    logs += [1.0 - k * 2.0 ** -30 for k in range(1, 200)]
    logs += [max(rnd.getrandbits(53) * 2.0 ** -53, 1e-10) for _ in range(2000)]
    logs += [1e-10, 0.5, 0.25, 2.0 ** -33, 0.7071067811865476, 0.9999847412109375]
    coss = [0.0, 1e-9, 2.0 ** -27, 2.0 ** -26]
    for k in range(1, 5):
        c = float(mp.pi / 2 * k)
        v = c
        for _ in range(40):
            v = math.nextafter(v, -math.inf)
        for _ in range(81):
            coss.append(v)
            v = math.nextafter(v, math.inf)
    coss += [TWO_PI * (rnd.getrandbits(53) * 2.0 ** -53) for _ in range(2000)]
    exps = [k * 2.0 ** -53 for k in range(-100, 101) if k] + [k * 2.0 ** -40 for k in range(1, 100)]
    exps += [rnd.uniform(0, 1) * math.log(100.0) for _ in range(1000)]             # log-uniform draws
    exps += [math.log(1e-12) + rnd.uniform(0, 1) * math.log(100.0) for _ in range(500)]
    exps += [rnd.uniform(-708, 709) for _ in range(500)] + [-708.0, 709.0, 0.5, -0.5, 1.0]
    return {"log": [[hexbits(x), hexbits(cr(mp.log, x))] for x in logs],
            "cos": [[hexbits(x), hexbits(cr(mp.cos, x))] for x in coss if x < 8.0],
            "exp": [[hexbits(x), hexbits(cr(mp.exp, x))] for x in exps]}


def main():
    json.dump(rng_golden(), open(os.path.join(HERE, "rng_golden.json"), "w"), separators=(",", ":"))
    json.dump(cr_golden(), open(os.path.join(HERE, "cr_math_golden.json"), "w"), separators=(",", ":"))


if __name__ == "__main__":
    main()
