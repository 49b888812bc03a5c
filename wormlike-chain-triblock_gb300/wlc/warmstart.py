"""Learned warm start of the SCFT field iteration: solver-generated data,
training and use of the network (wlc.WarmStartNet) on the device.

No counterpart in the reference, which starts every run from analytic or
random fields or from a W_dump restart (init_array_2dcomp_mod.f90:843-1107;
SCFT_dump.f90:273-337).  Here the solver itself generates converged fields
over a parameter range; the network learns the map

    (f_A, f_C, chiN, L/lp, box edge, 16^3 seeded noise) -> (w_A, w_B, w_C)

on a G^3 grid, and its prediction replaces the random start.  The plain
cold start stays the fallback.  Fields of other grids are obtained by
band-limited (Fourier) resampling of the G^3 prediction: the box is the
same physical box, only the grid spacing changes.

Targets are (w_K - <w_K>) / chiN: the mean of each block field is a gauge
freedom (it changes neither phi nor F), and chiN sets the field scale.
"""
import time

import numpy as np

from . import Batch, mix_params, even_block_lengths, wlc_radius_of_gyration, WlcError

# data set: 32^3 grid, l <= 6, Ns = 100, parameter ranges of the batched sweep
GRID, LMAX, NMAX = 32, 6, 100
RANGES = {"fa": (0.2, 0.4), "fc": (0.2, 0.4), "chi": (12.0, 24.0), "x": (0.5, 3.0), "box": (3.5, 5.5)}


def draw_params(count, seed):
    """`count` instance parameter draws: f_A, f_C ~ U(0.2, 0.4) (f_B the
    rest), chiN ~ U(12, 24), contour/persistence x ~ U(0.5, 3.0), box edge
    ~ U(3.5, 5.5) Rg, and the seed of each instance's noise field."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = {k: float(rng.uniform(*RANGES[k])) for k in ("fa", "fc", "chi", "x", "box")}
        d["noise_seed"] = int(rng.integers(1 << 31))
        out.append(d)
    return out


def noise_field(seed, grid=GRID):
    """16^3 N(0, 1) noise ([z][y][x]), nearest-upsampled to grid^3."""
    xi = np.random.default_rng(seed).normal(size=(16, 16, 16))
    f = grid // 16
    return xi.repeat(f, 0).repeat(f, 1).repeat(f, 2).reshape(-1)


def box_length(d):
    """box edge in units of the contour length (Rg from the wormlike-chain relation)"""
    return d["box"] * wlc_radius_of_gyration(d["x"])


def instance_spec(d, grid=GRID, lmax=LMAX, nmax=NMAX):
    """make_params keywords of one draw (kappa = 0.5 for every block, so
    Loa = x / 2 gives contour/persistence x)."""
    ns = even_block_lengths((d["fa"], 1.0 - d["fa"] - d["fc"], d["fc"]), nmax)
    return dict(n=grid, lmax=lmax, nmax=nmax, ns=ns, dx=box_length(d) / grid, loa=0.5 * d["x"],
                kappa=(0.5, 0.5, 0.5), chi=(d["chi"],) * 3)


def net_input(d, grid=GRID):
    """Network input (6, grid^3): the noise field and the five parameters,
    scaled to [-1, 1] over their ranges, as constant fields."""
    par = [2.0 * (d[k] - RANGES[k][0]) / (RANGES[k][1] - RANGES[k][0]) - 1.0 for k in ("fa", "fc", "chi", "x", "box")]
    P = grid ** 3
    return np.concatenate([noise_field(d["noise_seed"], grid)[None, :], np.repeat(np.array(par)[:, None], P, axis=1)])


def cold_start(d, grid=GRID):
    """The method without the network: A and B fields from the same noise,
    in antiphase, amplitude 0.3; C flat."""
    xi = noise_field(d["noise_seed"], grid)
    return 0.3 * np.stack([xi, -xi, np.zeros_like(xi)])


def to_target(w, chi):
    return (w - w.mean(axis=1, keepdims=True)) / chi


def from_output(y, chi):
    return np.asarray(y, dtype=np.float64) * chi


def fourier_resample(f, n_out):
    """Band-limited resampling of periodic fields f (..., n^3, [z][y][x]
    flattened) to n_out^3: zero-padding (or truncation) of the spectrum."""
    f = np.asarray(f, dtype=np.float64)
    lead = f.shape[:-1]
    n = round(f.shape[-1] ** (1.0 / 3.0))
    if n == n_out:
        return f.copy()
    F = np.fft.fftn(f.reshape(lead + (n, n, n)), axes=(-3, -2, -1))
    m = min(n, n_out)
    idx = np.r_[0:(m + 1) // 2, -(m // 2):0] if m > 1 else np.r_[0:1]
    G = np.zeros(lead + (n_out, n_out, n_out), dtype=complex)
    G[..., idx[:, None, None], idx[None, :, None], idx[None, None, :]] = \
        F[..., idx[:, None, None], idx[None, :, None], idx[None, None, :]]
    g = np.fft.ifftn(G, axes=(-3, -2, -1)).real * (n_out / n) ** 3
    return g.reshape(lead + (n_out ** 3,))


def data_mixing():
    """Field-update settings of the data generation and evaluation: the
    reference's constants (20 simple-mixing iterations with lambda 0.1, then
    Anderson mixing of depth 5 with lambda_A 0.1).  Measured on 48 cold
    32^3 draws over 400 iterations they converge more draws than depth 10
    with lambda_A 0.5 or ramped towards 1, which diverge more often.  The
    `ramp` key (0: off) ramps lambda_A = max(lambda_A, 1 - ramp^(n - 20))."""
    return dict(anderson_depth=5, lambda_anderson=0.1, ramp=0.0)


def solve_batch(draws, w0s, max_iter, tol, mixing=None, grid=GRID, lmax=LMAX, nmax=NMAX, log=None):
    """SCFT of every draw from the given fields in one batch (FP32
    propagators, FP64 densities / F / field update on the device) until every
    block residual is below tol or max_iter.  Returns a list of dicts
    (fields, iterations to tol or None, final residual, F, residual history);
    instances whose iteration diverges (non-finite density) get fields None."""
    mixing = dict(mixing or data_mixing())
    ramp = mixing.pop("ramp", 0.0)
    b = Batch([instance_spec(d, grid, lmax, nmax) for d in draws])
    for inst, w0 in zip(b.instances, w0s):
        inst.set_fields(w0)
    b.autotune()
    mp = mix_params(relax_iter=0, tol=tol, **mixing)
    lam0 = mp.lambda_anderson
    nd = len(draws)
    hist = [[] for _ in range(nd)]
    done = [None] * nd
    bad = [False] * nd
    fe = [np.nan] * nd
    fields = [None] * nd
    t0 = time.perf_counter()
    for it in range(1, max_iter + 1):
        if ramp and it > mp.num_simple:
            mp.lambda_anderson = max(lam0, 1.0 - ramp ** (it - mp.num_simple))
        b.propagate()
        for j, inst in enumerate(b.instances):
            if bad[j] or done[j] is not None:
                continue
            try:
                inst.density(want_junction=False)
                fe[j] = inst.free_energy()
                err, conv = inst.iterate(mp)
            except WlcError:
                bad[j] = True
                continue
            r = float(max(err[:3]))
            hist[j].append(r)
            if not np.isfinite(r):
                bad[j] = True
            elif conv:
                done[j] = it
                fields[j] = inst.get_fields()
        if all(bad[j] or done[j] is not None for j in range(nd)):
            break
        if log and it % 50 == 0:
            log("  iteration %d: %d converged, %d diverged, %.1f s" % (it, sum(v is not None for v in done),
                                                                       sum(bad), time.perf_counter() - t0))
    out = []
    for j, inst in enumerate(b.instances):
        w = fields[j] if fields[j] is not None else (None if bad[j] else inst.get_fields())
        out.append(dict(fields=w, iterations=done[j], residual=hist[j][-1] if hist[j] else np.nan, F=fe[j],
                        history=hist[j], diverged=bad[j]))
    b.close()
    return out


def tile_periodic(f, reps):
    """Periodic fields f (..., n^3, [z][y][x] flattened) repeated reps times
    along every axis: the fields of a box reps times larger."""
    f = np.asarray(f)
    lead = f.shape[:-1]
    n = round(f.shape[-1] ** (1.0 / 3.0))
    g = np.tile(f.reshape(lead + (n, n, n)), (1,) * len(lead) + (reps, reps, reps))
    return g.reshape(lead + ((n * reps) ** 3,))


def clamp_to_ranges(d):
    """The draw with every parameter clipped to the training ranges (the
    network is not asked to extrapolate)."""
    e = dict(d)
    for k, (lo, hi) in RANGES.items():
        e[k] = float(min(max(e[k], lo), hi))
    return e


def predict_large(net, d, grid_out, reps):
    """Warm start of a box `reps` times the predicted one along each axis:
    the network's fields for the box d["box"] / reps (clipped to the
    training ranges), tiled reps^3 times and Fourier-resampled to grid_out^3."""
    e = clamp_to_ranges(dict(d, box=d["box"] / reps))
    w = from_output(net.forward(net_input(e, net.G)), d["chi"])
    return fourier_resample(tile_periodic(w, reps), grid_out)


def predict(net, draws, grid_out=None):
    """Warm-start fields of each draw from the network (grid_out^3 by
    Fourier resampling when it differs from the network's grid)."""
    out = []
    for d in draws:
        w = from_output(net.forward(net_input(d, net.G)), d["chi"])
        if grid_out and grid_out != net.G:
            w = fourier_resample(w, grid_out)
        out.append(w)
    return out


def generate_dataset(target, seed, tol=1e-4, max_iter_cold=400, max_iter_warm=250, chunk=96, budget_s=1800.0,
                     bootstrap_after=24, epochs_bootstrap=30, width=32, log=print):
    """Converged training fields generated by the solver, bootstrapped:
    draws start cold until `bootstrap_after` have converged; then a network
    trained on the fields so far warm-starts the next draws (its prediction
    skips most of a cold start's morphology search, the slow part of the
    iteration), and is trained further after every chunk.  Stops at
    `target` converged fields or after budget_s seconds.  Returns (draws,
    targets (n, 3, G^3) float32, per-draw records)."""
    from . import WarmStartNet
    t0 = time.perf_counter()
    rng_seed = seed
    kept_d, kept_t, records = [], [], []
    net = None
    while len(kept_d) < target and time.perf_counter() - t0 < budget_s:
        draws = draw_params(chunk, rng_seed)
        rng_seed += 1
        warm = net is not None
        w0s = predict(net, draws) if warm else [cold_start(d) for d in draws]
        res = []
        for c0 in range(0, chunk, 48):
            res += solve_batch(draws[c0:c0 + 48], w0s[c0:c0 + 48], max_iter_warm if warm else max_iter_cold, tol)
        for d, r in zip(draws, res):
            records.append(dict(start="warm" if warm else "cold", iterations=r["iterations"], residual=r["residual"],
                                diverged=r["diverged"]))
            if r["iterations"] is not None and r["fields"] is not None and np.isfinite(r["fields"]).all():
                kept_d.append(d)
                kept_t.append(to_target(r["fields"], d["chi"]).astype(np.float32))
        if log:
            log("dataset: %d converged after %d draws (%s chunk), %.0f s" %
                (len(kept_d), len(records), "warm" if warm else "cold", time.perf_counter() - t0))
        if len(kept_d) >= bootstrap_after and len(kept_d) < target:
            if net is None:
                net = WarmStartNet(GRID, width, seed=1)
            # continue training the same network; a few thousand sample
            # passes per chunk keep the training short next to the solves
            X = np.stack([net_input(d) for d in kept_d]).astype(np.float32)
            ep = max(2, min(epochs_bootstrap, 3000 // len(kept_d)))
            net.train(X, np.stack(kept_t), batch=8, epochs=ep, lr=3e-4, seed=len(kept_d))
    if net is not None:
        net.close()
    return kept_d[:target], np.stack(kept_t[:target]) if kept_t else None, records


def train(draws, targets, epochs=20, lr=3e-4, width=32, seed=1, batch=8):
    """A network trained on (draws, targets); returns (net, loss history)."""
    from . import WarmStartNet
    net = WarmStartNet(GRID, width, seed=seed)
    X = np.stack([net_input(d) for d in draws]).astype(np.float32)
    hist = net.train(X, np.asarray(targets, dtype=np.float32), batch=batch, epochs=epochs, lr=lr, seed=seed + 1)
    return net, hist


def evaluate(net, draws, tol=2e-6, max_iter=400, thresholds=(1e-2, 1e-3, 1e-4, 1e-5), log=None):
    """Cold start against the network's warm start on the same held-out
    draws (same batches, same mixing): iterations to each residual
    threshold, wall time, final residuals and free energies."""
    out = {}
    for kind in ("cold", "warm"):
        w0s = [cold_start(d) for d in draws] if kind == "cold" else predict(net, draws)
        t0 = time.perf_counter()
        res = []
        for c0 in range(0, len(draws), 48):
            res += solve_batch(draws[c0:c0 + 48], w0s[c0:c0 + 48], max_iter, tol, log=log)
        out[kind] = dict(results=res, seconds=time.perf_counter() - t0)
    summary = {}
    for thr in tuple(thresholds) + (tol,):
        row = {}
        for kind in ("cold", "warm"):
            its = []
            for r in out[kind]["results"]:
                k = [i for i, v in enumerate(r["history"]) if v < thr]
                its.append(k[0] + 1 if k else None)
            ok = [v for v in its if v is not None]
            row[kind] = {"reached": len(ok), "median_iterations": float(np.median(ok)) if ok else None,
                         "mean_iterations_capped": float(np.mean([v if v is not None else max_iter for v in its]))}
            out[kind]["its_%g" % thr] = its
        both = [(a, b) for a, b in zip(out["cold"]["its_%g" % thr], out["warm"]["its_%g" % thr])
                if a is not None and b is not None]
        row["both_reached"] = len(both)
        row["median_ratio_cold_over_warm"] = float(np.median([a / b for a, b in both])) if both else None
        summary["%g" % thr] = row
    return out, summary
