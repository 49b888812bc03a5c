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


def test_noalloc_in_place_against_oracle_alternating_L():
    """In place (q_out_dev == pr_dev, which the header allows) against the
    CPU oracle, with (L, literals) changing between calls so that the
    tables in the static array are replaced and then replaced back."""
    import torch
    import oracle
    lib = wlc.load()
    noalloc = _bind(lib)
    n, nmax, ns = 12, 10, (4, 2, 4)
    dx = 1.2 / n
    kappa, chi = (0.5, 0.6, 0.7), (15.0, 15.0, 15.0)
    rng = np.random.default_rng(77)
    err = ctypes.create_string_buffer(256)
    table = {3: (3, 1, 0), 5: (3, 1, 2), 8: (3, -1, 2)}
    for L, lit, g_index in ((4, wlc.WLC_LIT_REAL4, 3), (6, wlc.WLC_LIT_REAL8, 8), (4, wlc.WLC_LIT_REAL4, 5)):
        p = wlc.make_params(n, L, nmax, ns, dx, 1.3, kappa, chi, literals=lit)
        o = oracle.Oracle((n, n, n), L, nmax, ns, (dx, dx, dx), 1.3, kappa, chi,
                          real4=1 if lit == wlc.WLC_LIT_REAL4 else 0)
        M = (L + 1) ** 2
        pr = rng.standard_normal((M, n ** 3))
        order, sigma, blk = table[g_index]
        ref = o.one_step(order, sigma, blk, pr)
        o.close()
        d = torch.from_numpy(pr.copy()).cuda()
        rc = noalloc(ctypes.byref(p), g_index, d.data_ptr(), d.data_ptr(), None, err, 256)
        torch.cuda.synchronize()
        assert rc == 0, err.value.decode()
        out = d.cpu().numpy()
        e = np.abs(out - ref).max() / np.abs(ref).max()
        assert e < TOL, "L=%d G_index %d in place: rel err %.3e" % (L, g_index, e)


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
