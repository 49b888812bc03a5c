"""Host-side helpers: block lengths, wormlike-chain Rg, bench workload."""
import math

import wlc


def test_even_block_lengths():
    assert wlc.even_block_lengths((0.33, 0.33, 0.34), 100) == (34, 32, 34)
    assert wlc.even_block_lengths((0.25, 0.50, 0.25), 200) == (50, 100, 50)
    assert wlc.even_block_lengths((0.3, 0.4, 0.3), 400) == (120, 160, 120)
    for fa in (0.2, 0.27, 0.33, 0.4):
        for fc in (0.2, 0.31, 0.4):
            na, nb, nc = wlc.even_block_lengths((fa, 1 - fa - fc, fc), 128)
            assert na % 2 == nb % 2 == nc % 2 == 0 and na + nb + nc == 128


def test_wlc_radius_of_gyration_limits():
    # rod limit L/lp -> 0: Rg^2 = L^2/12 ; coil limit: Rg^2 -> L lp / 3
    assert abs(wlc.wlc_radius_of_gyration(1e-3) - math.sqrt(1 / 12.0)) < 1e-3
    x = 200.0
    assert abs(wlc.wlc_radius_of_gyration(x) ** 2 / (1.0 / (3 * x)) - 1) < 2e-2
    assert abs(wlc.wlc_radius_of_gyration(2.0) - 0.24203) < 1e-4


def test_bench_workload_matches_headline_config():
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    wl = bench.workload("fp64")
    assert (wl["n"], wl["L"], wl["nmax"], wl["ns"]) == (64, 10, 200, (50, 100, 50))
    assert abs(wl["box"] - 5.0 * wlc.wlc_radius_of_gyration(2.0)) < 1e-12
    assert abs(wl["loa"] / wl["kappa"][0] - 2.0) < 1e-12
    assert bench.algorithmic_bytes(wl, 8) == 4 * 121 * 64 ** 3 * 8 + 8 * 64 ** 3
