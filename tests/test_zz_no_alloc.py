"""The allocation-free one-step entry point (wlc_mde_one_step_noalloc).

It serves callers that cannot call cudaMalloc -- code that only receives
device pointers from its framework or must not grow a fixed memory pool --
so it keeps its k-space scratch in a static device array instead of
allocating.  This test calls it through the C ABI with device buffers and
checks it against the allocating entry point (wlc_mde_one_step) at the
FP64 parity tolerance, on two calls in a row, and checks that a size above
the static limit is refused with a message.  It lives in its own file that
pytest collects last.
"""
import ctypes

import numpy as np
import pytest

import wlc

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _bind(lib):
    f = lib.wlc_mde_one_step_noalloc
    f.argtypes = [ctypes.POINTER(wlc.Params), ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_char_p, ctypes.c_int32]
    f.restype = ctypes.c_int
    return f


def test_noalloc_matches_allocating_step_twice():
    import torch
    lib = wlc.load()
    noalloc = _bind(lib)
    n, L, nmax, ns = 16, 4, 10, (4, 2, 4)
    dx = 1.1 / n
    kappa, chi = (0.5, 0.6, 0.7), (15.0, 15.0, 15.0)
    inst = wlc.Instance(n, L, nmax, ns, dx, 1.3, kappa, chi)
    p = inst.params
    rng = np.random.default_rng(2024)
    err = ctypes.create_string_buffer(256)
    for g_index in (3, 7):  # two calls in a row, different operators and inputs
        pr = rng.standard_normal((inst.M, inst.nr))  # [i][r]
        ref = inst.mde_one_step(g_index, pr.T.copy()).T  # existing entry point, host buffers
        d_pr = torch.from_numpy(pr).cuda()
        d_q = torch.empty_like(d_pr)
        rc = noalloc(ctypes.byref(p), g_index, d_pr.data_ptr(), d_q.data_ptr(), None, err, 256)
        torch.cuda.synchronize()
        assert rc == 0, err.value.decode()
        out = d_q.cpu().numpy()
        e = np.abs(out - ref).max() / np.abs(ref).max()
        assert e < TOL, "G_index %d: rel err %.3e" % (g_index, e)
    inst.close()


def test_noalloc_rejects_sizes_above_static_limit():
    import torch
    lib = wlc.load()
    noalloc = _bind(lib)
    p = wlc.Params()
    p.n[:] = [64, 64, 64]
    p.lmax = 10
    p.nmax = 200
    p.ns[:] = [50, 100, 50]
    p.dx[:] = [0.02, 0.02, 0.02]
    p.loa = 1.0
    p.kappa[:] = [0.5, 0.5, 0.5]
    p.chi[:] = [18.0, 18.0, 18.0]
    err = ctypes.create_string_buffer(256)
    # the size check refuses before any launch; the small buffers are never touched
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = noalloc(ctypes.byref(p), 3, buf.data_ptr(), buf.data_ptr(), None, err, 256)
    torch.cuda.synchronize()
    assert rc == -6  # WLC_E_UNSUPPORTED
    assert b"static limit" in err.value
