"""Device resampling counts against the binary128 known-answer vectors and
the oracle (bit-exact)."""
import json
import os

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import preset

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_device_resample_matches_golden(smcgpu, orc):
    with open(os.path.join(ROOT, "tests/golden/resample_kat.json")) as f:
        cases = json.load(f)["cases"]
    g = smcgpu.SmcGpu(preset("tiny").settings)
    for c in cases:
        w = np.array([float.fromhex(x) for x in c["w"]])
        uh, ul = float.fromhex(c["u_hi"]), float.fromhex(c["u_lo"])
        got = g.resample_counts(w, uh, ul)
        assert list(got) == c["counts"], c["name"]


def test_device_resample_matches_oracle_random(smcgpu, orc):
    g = smcgpu.SmcGpu(preset("tiny").settings)
    rng = np.random.default_rng(5)
    for n in (3, 31, 32, 33, 1023, 1024, 1025, 4096, 20000):
        w = np.exp(rng.normal(0, 3, n))
        w /= w.sum()
        uh, ul = orc.quad_uniform(9, n, 8, 1)
        assert np.array_equal(g.resample_counts(w, uh, ul), orc.resample(w, uh, ul)), n
