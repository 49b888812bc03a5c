"""Host-side pieces of the learned warm start (wlc.warmstart), on CPU:
parameter draws and network inputs, the instance specification, and the
band-limited resampling that carries a G^3 prediction to another grid."""
import numpy as np

from wlc import warmstart as ws


def _field(n, fx=1, fy=2, fz=1):
    x = np.arange(n) / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    return (np.cos(2 * np.pi * fx * X) + 0.3 * np.sin(2 * np.pi * fy * Y) * np.cos(2 * np.pi * fz * Z)).reshape(-1)


def test_fourier_resample_is_exact_for_band_limited_fields():
    f16, f32, f64 = _field(16), _field(32), _field(64)
    up = ws.fourier_resample(np.stack([f16, 2 * f16]), 32)
    assert np.abs(up[0] - f32).max() < 1e-13 and np.abs(up[1] - 2 * f32).max() < 1e-13
    assert np.abs(ws.fourier_resample(f32[None], 64)[0] - f64).max() < 1e-13
    assert np.abs(ws.fourier_resample(f64[None], 16)[0] - f16).max() < 1e-13
    # the mean (the gauge of each block field) is kept
    g = np.random.default_rng(1).normal(size=(3, 16 ** 3))
    assert np.allclose(ws.fourier_resample(g, 32).mean(axis=1), g.mean(axis=1), atol=1e-14)


def test_draws_inputs_and_specs():
    draws = ws.draw_params(50, 3)
    for d in draws:
        for k, (lo, hi) in ws.RANGES.items():
            assert lo <= d[k] <= hi
        x = ws.net_input(d)
        assert x.shape == (6, ws.GRID ** 3)
        assert np.all(np.abs(x[1:]) <= 1.0 + 1e-12)
        s = ws.instance_spec(d)
        assert sum(s["ns"]) == ws.NMAX and all(v % 2 == 0 for v in s["ns"])
        assert abs(s["dx"] * ws.GRID - ws.box_length(d)) < 1e-12
    # the noise field repeats the 16^3 seed field on 2^3 blocks
    xi = ws.noise_field(draws[0]["noise_seed"]).reshape(32, 32, 32)
    assert np.array_equal(xi[::2, ::2, ::2], xi[1::2, 1::2, 1::2])
    # targets drop the gauge and the chiN scale, outputs restore the scale
    w = np.random.default_rng(2).normal(size=(3, 8))
    t = ws.to_target(w, 15.0)
    assert np.allclose(t.mean(axis=1), 0.0) and np.allclose(ws.from_output(t, 15.0), w - w.mean(axis=1, keepdims=True))


def test_tiling_and_range_clipping():
    f = np.random.default_rng(5).normal(size=(3, 8 ** 3))
    t = ws.tile_periodic(f, 2).reshape(3, 16, 16, 16)
    g = f.reshape(3, 8, 8, 8)
    for dz in (0, 8):
        for dy in (0, 8):
            for dx in (0, 8):
                assert np.array_equal(t[:, dz:dz + 8, dy:dy + 8, dx:dx + 8], g)
    e = ws.clamp_to_ranges(dict(fa=0.1, fc=0.3, chi=30.0, x=4.0, box=4.0, noise_seed=1))
    assert e["fa"] == 0.2 and e["chi"] == 24.0 and e["x"] == 3.0 and e["box"] == 4.0 and e["fc"] == 0.3
