"""The committed engine table (written by smc_inversion_fort_gb300.autotune on
a GB300, loaded into SMCGPU_ENGINE_AUTO contexts): well formed and within each
engine's slip-dimension limit, so that no row asks an engine for a size it
hands on.  CPU only."""
import smc_inversion_fort_gb300 as pkg

LIMITS = {("mixed", pkg.ENGINE_MMA): 256, ("mixed", pkg.ENGINE_CUDA): 192, ("mixed", pkg.ENGINE_TCGEN05): 128,
          ("mixed", pkg.ENGINE_GLOBAL): 1024, ("fp64", pkg.ENGINE_CUDA): 128, ("fp64", pkg.ENGINE_GLOBAL): 1024}


def test_engine_table_rows_are_valid():
    tab = pkg.load_engine_table()
    assert tab is not None, "engine_table.json is committed next to the package"
    for key in ("mixed", "fp64"):
        rows = tab[key]
        assert rows, key
        dmax = [r[0] for r in rows]
        assert dmax == sorted(set(dmax)), (key, dmax)          # strictly ascending
        assert dmax[-1] >= 576                                  # covers the uneven-mesh sizes (D <= 576)
        for d, eng, warps in rows:
            assert (key, eng) in LIMITS, (key, d, eng)
            assert d <= LIMITS[(key, eng)], (key, d, eng)
            assert warps in (0, 1, 2, 4, 8)
            assert warps == 0 or eng == pkg.ENGINE_CUDA         # warps only for the CUDA-core engine
