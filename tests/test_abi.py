"""The C ABI library builds, loads and exports every symbol include/wlc.h
declares; parameter validation works without a GPU (no compute calls)."""
import ctypes
import os
import re

import pytest

import wlc

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "wlc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(wlc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = wlc.load()
    names = declared_symbols()
    assert len(names) >= 17
    for name in names:
        assert hasattr(lib, name), "libwlc.so does not export %s" % name
    assert set(wlc.SYMBOLS) <= set(names)


def test_abi_version():
    assert wlc.load().wlc_abi_version() == 1


def test_params_struct_layout():
    # int32 n[3], lmax, nmax, ns[3]; double dx[3], loa, kappa[3], chi[3], nmu;
    # int32 precision, literals, store_qstar, q_checkpoint, reserved[4]
    assert ctypes.sizeof(wlc.Params) == 152
    assert wlc.Params.dx.offset == 32 and wlc.Params.precision.offset == 120
    assert wlc.Params.q_checkpoint.offset == 132


def test_mix_params_struct_layout():
    # int32 anderson_depth, num_simple; double lambda_simple, lambda_anderson, tol;
    # int32 min_iter, relax_iter; double relax_tol, lambda_m; int32 reserved[2]
    assert ctypes.sizeof(wlc.MixParams) == 64
    assert wlc.MixParams.tol.offset == 24 and wlc.MixParams.relax_tol.offset == 40
    assert wlc.MixParams.lambda_m.offset == 48


def _create(**kw):
    lib = wlc.load()
    p = wlc.Params()
    p.n[:] = kw.get("n", [8, 8, 8])
    p.lmax = kw.get("lmax", 2)
    p.nmax = kw.get("nmax", 6)
    p.ns[:] = kw.get("ns", [2, 2, 2])
    p.dx[:] = [0.1, 0.1, 0.1]
    p.loa = 1.0
    p.kappa[:] = [0.5, 0.5, 0.5]
    p.chi[:] = [15.0, 15.0, 15.0]
    p.precision = kw.get("precision", 0)
    p.literals = 0
    p.store_qstar = kw.get("store_qstar", 1)
    p.q_checkpoint = kw.get("q_checkpoint", 0)
    h = ctypes.c_void_p()
    rc = lib.wlc_create(ctypes.byref(p), ctypes.byref(h))
    msg = lib.wlc_last_error(h).decode() if h else ""
    lib.wlc_destroy(h)
    return rc, msg


@pytest.mark.parametrize("kw,code,text", [
    (dict(ns=[3, 1, 2]), -1, "even"),             # odd block (initialize_mod.f90:190-195)
    (dict(ns=[2, 2, 4]), -1, "equal nmax"),       # NA+NB+NC != Nmax
    (dict(n=[8, 8, 16]), -6, "cubic"),
    (dict(n=[10, 10, 10]), -6, "compiled"),
    (dict(lmax=20), -1, "lmax"),
    (dict(precision=7), -1, "precision"),
    (dict(lmax=13), -1, "lmax"),                  # rotation codelets cover l <= 12
    (dict(store_qstar=3), -1, "store_qstar"),
    (dict(q_checkpoint=4), -1, "q_checkpoint"),   # checkpointing needs streamed densities
    (dict(q_checkpoint=2, store_qstar=0), -1, "q_checkpoint"),
    (dict(q_checkpoint=7, store_qstar=0), -1, "q_checkpoint"),  # > nmax
])
def test_invalid_parameters_are_rejected_before_any_device_work(kw, code, text):
    rc, msg = _create(**kw)
    assert rc == code
    assert text in msg
