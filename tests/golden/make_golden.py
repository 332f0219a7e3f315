"""Generates tests/golden/resample_kat.json: known-answer vectors of the
reference's real(16) residual-systematic resampling recurrence
(smc_slip.f90:572-589, smc_fault.f90:572-590), evaluated with mpmath at
113-bit precision, which rounds every +, -, *, / to nearest-even like IEEE
binary128.  Run: python tests/golden/make_golden.py
"""
import json
import math
import os

import mpmath
import numpy as np

mpmath.mp.prec = 113


def recurrence(w, u_hi, u_lo, count_n=None):
    n = len(w)
    dn = mpmath.mpf(count_n or n)
    u = mpmath.mpf(u_hi) + mpmath.mpf(u_lo)
    u = u / dn
    out = []
    for wi in w:
        wq = mpmath.mpf(float(wi))
        a = int(mpmath.floor((wq - u) * dn)) + 1
        out.append(a)
        u = u + mpmath.mpf(a) / dn - wq
    return out


def hexd(x):
    return float(x).hex()


def case(name, w, u_hi, u_lo):
    return {"name": name, "w": [hexd(v) for v in w], "u_hi": hexd(u_hi), "u_lo": hexd(u_lo),
            "counts": recurrence(w, u_hi, u_lo)}


def main():
    rng = np.random.default_rng(20240611)
    cases = []
    for n in (1, 2, 5, 64, 500, 2048):
        for rep in range(2):
            w = np.exp(rng.normal(0, 2, n))
            w = w / w.sum()
            u_hi = float(rng.integers(0, 2**53)) * 2.0**-53
            u_lo = float(rng.integers(0, 2**53)) * 2.0**-106
            cases.append(case(f"lognormal-{n}-{rep}", w, u_hi, u_lo))
    w = np.full(500, 1.0 / 500)
    cases.append(case("uniform-500-clipped-u", w, 1e-5, 0.0))
    w = np.zeros(100); w[37] = 1.0
    cases.append(case("degenerate-100", w, 0.5, 0.0))
    w = np.exp(rng.normal(0, 1, 300)); w[::7] = 0.0; w /= w.sum()
    cases.append(case("zeros-300", w, 0.25, 2.0**-80))
    # near ties: u0 placed within ~1e-27 of frac(N W_k) so that N W_k - u0 is
    # a hair away from an integer; the binary128 recurrence decides the side
    for n, k, eps in ((64, 20, 1e-27), (500, 123, -1e-27), (2048, 1500, 3e-30)):
        w = np.exp(rng.normal(0, 1, n)); w /= w.sum()
        W = mpmath.fsum([mpmath.mpf(float(v)) for v in w[: k + 1]])
        x = mpmath.mpf(n) * W
        frac = x - mpmath.floor(x)
        target = frac - mpmath.mpf(eps)
        u_hi = float(target)
        u_lo = float(target - mpmath.mpf(u_hi))
        cases.append(case(f"near-tie-{n}-{k}", w, u_hi, u_lo))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "resample_kat.json")
    with open(out, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "precision_bits": 113, "cases": cases}, f)
    print(out, len(cases))


if __name__ == "__main__":
    main()
