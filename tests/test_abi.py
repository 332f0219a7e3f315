"""The C-ABI library builds, loads without a GPU and exports every entry
point declared in include/smcgpu.h."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "smcgpu.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(smcgpu_\w+)\s*\(", txt)))


def test_header_symbols_exported(smcgpu):
    lib = ctypes.CDLL(smcgpu.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert set(smcgpu.EXPORTED_SYMBOLS) <= set(names)


def test_create_rejects_bad_config(smcgpu):
    from smc_inversion_fort_gb300.configs import SmcSettings
    import pytest
    with pytest.raises(Exception):
        smcgpu.SmcGpu(SmcSettings(nxi=(1,), neta=(4,)))
