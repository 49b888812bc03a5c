"""Batched instances (wlc_batch_*) and launch autotuning.

A batch advances several independent FP32 instances with one launch per
pass per grid-size group and replays the contour loop as a CUDA graph.  Each
instance must give what the same instance gives on its own (the batched
kernels are the single-instance kernels reading their arguments from a
device array; 1e-6 relative covers a different FP32 instruction schedule of
the batched instantiation, bit-identical is expected and reported), and
every launch configuration the autotuner may pick must give identical
results."""
import numpy as np
import pytest

import oracle
import wlc

pytestmark = pytest.mark.gpu

SPECS = [
    dict(n=16, lmax=3, nmax=12, ns=(4, 4, 4), dx=0.07, loa=1.0, kappa=(0.5, 0.5, 0.5), chi=(15.0, 12.0, 18.0),
         store_qstar=0),
    dict(n=24, lmax=3, nmax=12, ns=(2, 6, 4), dx=0.05, loa=1.5, kappa=(0.5, 0.6, 0.7), chi=(12.0, 20.0, 14.0),
         store_qstar=2),
    dict(n=16, lmax=3, nmax=12, ns=(6, 0, 6), dx=0.09, loa=0.7, kappa=(0.5, 0.5, 0.5), chi=(18.0, 18.0, 18.0),
         store_qstar=1),
    dict(n=24, lmax=3, nmax=12, ns=(4, 2, 6), dx=0.06, loa=2.5, kappa=(0.5, 0.8, 0.5), chi=(13.0, 16.0, 22.0),
         store_qstar=0),
]


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _fields(spec, seed):
    return np.random.default_rng(seed).normal(0.0, 0.3, size=(3, spec["n"] ** 3))


def _single(spec, w, dx=None):
    kw = dict(spec)
    kw["precision"] = wlc.WLC_FP32
    if dx is not None:
        kw["dx"] = dx
    g = wlc.Instance(**kw)
    g.set_fields(w)
    g.MDE_q()
    g.MDE_qstar()
    d = g.density(want_s=spec["store_qstar"] != 0)
    fe = g.free_energy()
    g.close()
    return d, fe


def _check(inst, spec, ref, fref, exact):
    d = inst.density(want_s=spec["store_qstar"] != 0)
    fe = inst.free_energy()
    same = d["lnQ"] == ref["lnQ"] and np.array_equal(d["phi"], ref["phi"]) and fe == fref
    exact.append(same)
    assert abs(d["lnQ"] - ref["lnQ"]) <= 1e-6 * max(1.0, abs(ref["lnQ"]))
    assert _rel(d["phi"], ref["phi"]) < 1e-6
    assert _rel(d["junction"], ref["junction"]) < 1e-6
    assert abs(fe - fref) <= 1e-6 * abs(fref)
    if spec["store_qstar"] != 0:
        assert _rel(d["S"], ref["S"]) < 1e-5


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_single_instances(graph):
    b = wlc.Batch(SPECS)
    b.use_graph(graph)
    ws = [_fields(s, 40 + i) for i, s in enumerate(SPECS)]
    for inst, w in zip(b.instances, ws):
        inst.set_fields(w)
    exact = []
    for rep in range(2):  # second pass replays the captured graph
        b.propagate()
        for inst, spec, w in zip(b.instances, SPECS, ws):
            ref, fref = _single(spec, w)
            _check(inst, spec, ref, fref, exact)
    print("bit-identical to single-instance runs:", all(exact))
    b.close()


def test_batch_after_field_update_and_box_change():
    """Fields updated in place by wlc_iterate replay through the same graph;
    a box change of one member rebuilds the arguments and re-captures."""
    b = wlc.Batch(SPECS)
    ws = [_fields(s, 60 + i) for i, s in enumerate(SPECS)]
    for inst, w in zip(b.instances, ws):
        inst.set_fields(w)
    b.propagate()
    mp = wlc.mix_params(anderson_depth=2, num_simple=1)
    for inst in b.instances:
        inst.density(want_junction=False)
        inst.iterate(mp)  # simple mixing step on the device
    b.instances[1].init_inverse_sparse_GAB(0.055)
    b.propagate()
    exact = []
    for i, (inst, spec) in enumerate(zip(b.instances, SPECS)):
        w_now = inst.get_fields()
        ref, fref = _single(spec, w_now, dx=0.055 if i == 1 else None)
        _check(inst, spec, ref, fref, exact)
    b.close()


def test_batch_autotune_keeps_results():
    b = wlc.Batch(SPECS)
    ws = [_fields(s, 80 + i) for i, s in enumerate(SPECS)]
    for inst, w in zip(b.instances, ws):
        inst.set_fields(w)
    b.propagate()
    before = [inst.density(want_junction=False) for inst in b.instances]
    cfg = b.autotune()
    assert sorted(c[0] for c in cfg) == [16, 24] and all(c[3] in (256, 512) and 0 <= c[4] <= 3 for c in cfg)
    b.propagate()
    for inst, d0 in zip(b.instances, before):
        d = inst.density(want_junction=False)
        assert d["lnQ"] == d0["lnQ"] and np.array_equal(d["phi"], d0["phi"])
    b.close()


def test_batch_rejects_unsupported_members():
    with pytest.raises(wlc.WlcError):
        wlc.Batch([dict(SPECS[0]), dict(SPECS[1], nmax=14, ns=(4, 4, 6))])  # two nmax
    with pytest.raises(wlc.WlcError):
        wlc.Batch([dict(SPECS[0], n=12)])  # no batched kernels for N = 12
    with pytest.raises(wlc.WlcError):
        wlc.Batch([dict(SPECS[0], precision=wlc.WLC_FP64)])


@pytest.mark.parametrize("precision", [wlc.WLC_FP64, wlc.WLC_FP32])
def test_single_autotune_keeps_results(precision):
    n, L, nmax, ns = 16, 4, 10, (4, 2, 4)
    g = wlc.Instance(n, L, nmax, ns, 0.08, 1.2, (0.5, 0.6, 0.7), (15.0, 12.0, 18.0), precision=precision)
    w = np.random.default_rng(3).normal(0.0, 0.4, size=(3, n ** 3))
    g.set_fields(w)
    g.MDE_q()
    g.MDE_qstar()
    d0 = g.density()
    a_var, threads, xy, xv = g.autotune()
    assert a_var in (1, 2) and threads % n == 0 and 0 < threads <= 256 and xy in (256, 512) and 0 <= xv <= 3
    g.MDE_q()
    g.MDE_qstar()
    d = g.density()
    assert d["lnQ"] == d0["lnQ"] and np.array_equal(d["phi"], d0["phi"])
    for cfg in ((1, n, 512, 1), (2, 2 * n, 256, 0), (1, 3 * n, 512, 2), (1, 2 * n, 256, 3), (0, 0, 0, 0)):
        g.set_launch_config(*cfg)
        g.MDE_q()
        g.MDE_qstar()
        d = g.density()
        assert d["lnQ"] == d0["lnQ"] and np.array_equal(d["phi"], d0["phi"]), cfg
    if precision == wlc.WLC_FP64:
        o = oracle.Oracle((n, n, n), L, nmax, ns, (0.08,) * 3, 1.2, (0.5, 0.6, 0.7), (15.0, 12.0, 18.0))
        o.set_fields(w)
        o.propagate(1)
        o.propagate(-1)
        od = o.density(want_s=False)
        assert abs(d["lnQ"] - od["lnQ"]) <= 1e-10 * max(1.0, abs(od["lnQ"]))
        assert _rel(d["phi"], od["phi"]) < 1e-10
