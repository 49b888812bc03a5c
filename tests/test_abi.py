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
    # int32 precision, literals, store_qstar, reserved[5]
    assert ctypes.sizeof(wlc.Params) == 152
    assert wlc.Params.dx.offset == 32 and wlc.Params.precision.offset == 120


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
])
def test_invalid_parameters_are_rejected_before_any_device_work(kw, code, text):
    rc, msg = _create(**kw)
    assert rc == code
    assert text in msg
