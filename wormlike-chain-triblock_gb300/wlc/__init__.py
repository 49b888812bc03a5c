"""Python host mirror of the reference's propagator / density entry points,
bound through the C ABI of libwlc.so (include/wlc.h) with ctypes.

The reference (tjz2026/wormlike-chain-triblock) keeps its state in Fortran
module globals and calls, per SCFT iteration (SCFT_control.f90:237-273):
    calc_THETAij(); MDE_q(); MDE_qstar(); density(); free_energy()
and, inside the ABC draft driver, init_pr(...) / mde_one_step(...)
(MDE_ABC.f90:8-383) and init_inverse_sparse_GAB() on every box change
(Gmatrix_2dcomp_mod.f90:222).  `Instance` exposes the same names on one
GPU-resident instance.  There is no CPU fallback: if libwlc.so cannot be
built or loaded, or no CUDA device exists, every call raises.

Array layouts follow the reference's Fortran arrays (documented in wlc.h):
propagator slices / right-hand sides are (nr, M) C arrays (coefficient
fastest, as q_f(0:M-1, 0:LS, s)); fields are (3, nr); the Maier-Saupe
tensor M_OP(0:LS,0:2,0:2) is a (3, 3, nr) C array indexed [b][a][r].
Grid point r = x + nx*(y + ny*z).
"""
import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

WLC_FP64, WLC_FP32 = 0, 1
WLC_LIT_REAL4, WLC_LIT_REAL8 = 0, 1
WLC_SCHEME_BDF, WLC_SCHEME_SPLIT = 0, 1
ERRORS = {-1: "WLC_E_PARAM", -2: "WLC_E_ALLOC", -3: "WLC_E_CUDA", -4: "WLC_E_STATE",
          -5: "WLC_E_NONFINITE", -6: "WLC_E_UNSUPPORTED", -7: "WLC_E_SELFTEST", -8: "WLC_E_IO"}

# exported symbols declared in include/wlc.h
SYMBOLS = ["wlc_abi_version", "wlc_create", "wlc_destroy", "wlc_last_error", "wlc_set_box",
           "wlc_set_fields", "wlc_propagate", "wlc_density", "wlc_free_energy", "wlc_get_q",
           "wlc_set_q", "wlc_init_pr", "wlc_mde_one_step", "wlc_launch_count", "wlc_stream",
           "wlc_enable_timing", "wlc_last_timing", "wlc_iterate", "wlc_reset_mixing", "wlc_get_fields",
           "wlc_set_precision", "wlc_get_mop", "wlc_autotune", "wlc_set_launch_config", "wlc_batch_create",
           "wlc_batch_destroy", "wlc_batch_last_error", "wlc_batch_size", "wlc_batch_groups", "wlc_batch_get",
           "wlc_batch_propagate", "wlc_batch_autotune", "wlc_batch_use_graph", "wlc_batch_stream",
           "wlc_batch_launch_count", "wlc_io_write_w", "wlc_io_read_w", "wlc_io_write_mop", "wlc_io_read_mop",
           "wlc_io_write_rho", "wlc_io_append_free_energy", "wlc_io_append_errors", "wlc_net_create",
           "wlc_net_destroy", "wlc_net_last_error", "wlc_net_param_count", "wlc_net_get_params",
           "wlc_net_set_params", "wlc_net_forward", "wlc_net_loss_grad", "wlc_net_train"]


class WlcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32 * 3), ("lmax", ctypes.c_int32), ("nmax", ctypes.c_int32),
                ("ns", ctypes.c_int32 * 3), ("dx", ctypes.c_double * 3), ("loa", ctypes.c_double),
                ("kappa", ctypes.c_double * 3), ("chi", ctypes.c_double * 3), ("nmu", ctypes.c_double),
                ("precision", ctypes.c_int32), ("literals", ctypes.c_int32),
                ("store_qstar", ctypes.c_int32), ("q_checkpoint", ctypes.c_int32), ("scheme", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 3)]


class MixParams(ctypes.Structure):
    """wlc_mix_params: the reference's iteration constants
    (global_parameters.f90:69,126-139, SCFT_main.f90:41)."""
    _fields_ = [("anderson_depth", ctypes.c_int32), ("num_simple", ctypes.c_int32),
                ("lambda_simple", ctypes.c_double), ("lambda_anderson", ctypes.c_double),
                ("tol", ctypes.c_double), ("min_iter", ctypes.c_int32), ("relax_iter", ctypes.c_int32),
                ("relax_tol", ctypes.c_double), ("lambda_m", ctypes.c_double), ("reserved", ctypes.c_int32 * 2)]


def mix_params(anderson_depth=5, num_simple=20, lambda_simple=0.1, lambda_anderson=0.1, tol=1e-4,
               min_iter=20, relax_iter=150, relax_tol=5e-4, lambda_m=0.08):
    m = MixParams()
    m.anderson_depth, m.num_simple = int(anderson_depth), int(num_simple)
    m.lambda_simple, m.lambda_anderson, m.tol = float(lambda_simple), float(lambda_anderson), float(tol)
    m.min_iter, m.relax_iter, m.relax_tol = int(min_iter), int(relax_iter), float(relax_tol)
    m.lambda_m = float(lambda_m)
    return m


def lib_path():
    return os.path.join(_HERE, "_lib", "libwlc.so")


def load(build_if_missing=True):
    """Load libwlc.so (building it in-tree when missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_wlc_build", os.path.join(os.path.dirname(_HERE), "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = ctypes.CDLL(path)
    P, I, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_double
    Dp = ctypes.POINTER(ctypes.c_double)
    lib.wlc_abi_version.restype = ctypes.c_int
    lib.wlc_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(P)]
    lib.wlc_destroy.argtypes = [P]
    lib.wlc_last_error.argtypes = [P]
    lib.wlc_last_error.restype = ctypes.c_char_p
    lib.wlc_set_box.argtypes = [P, D, D, D]
    lib.wlc_set_fields.argtypes = [P, Dp, Dp]
    lib.wlc_propagate.argtypes = [P, I]
    lib.wlc_density.argtypes = [P, Dp, Dp, Dp, Dp]
    lib.wlc_free_energy.argtypes = [P, Dp]
    lib.wlc_get_q.argtypes = [P, I, I, Dp]
    lib.wlc_set_q.argtypes = [P, I, I, Dp]
    lib.wlc_init_pr.argtypes = [P, I, I, Dp]
    lib.wlc_mde_one_step.argtypes = [P, I, Dp, Dp]
    lib.wlc_launch_count.argtypes = [P]
    lib.wlc_launch_count.restype = ctypes.c_int64
    lib.wlc_stream.argtypes = [P]
    lib.wlc_stream.restype = P
    lib.wlc_enable_timing.argtypes = [P, I]
    lib.wlc_last_timing.argtypes = [P, Dp]
    lib.wlc_iterate.argtypes = [P, ctypes.POINTER(MixParams), Dp, ctypes.POINTER(ctypes.c_int32)]
    lib.wlc_reset_mixing.argtypes = [P]
    lib.wlc_get_fields.argtypes = [P, Dp]
    lib.wlc_set_precision.argtypes = [P, I]
    lib.wlc_get_mop.argtypes = [P, Dp]
    C = ctypes.c_char_p
    L64 = ctypes.c_int64
    lib.wlc_io_write_w.argtypes = [C, Dp, L64]
    lib.wlc_io_read_w.argtypes = [C, Dp, L64]
    lib.wlc_io_write_mop.argtypes = [C, Dp, L64, Dp]
    lib.wlc_io_read_mop.argtypes = [C, Dp, L64]
    lib.wlc_io_write_rho.argtypes = [C, Dp, ctypes.POINTER(ctypes.c_int32), Dp]
    lib.wlc_io_append_free_energy.argtypes = [C, I, D, D, D, Dp, ctypes.POINTER(ctypes.c_int32), I]
    lib.wlc_io_append_errors.argtypes = [C, I, Dp, I]
    Fp = ctypes.POINTER(ctypes.c_float)
    lib.wlc_net_create.argtypes = [I, I, ctypes.c_uint64, ctypes.POINTER(P)]
    lib.wlc_net_destroy.argtypes = [P]
    lib.wlc_net_last_error.argtypes = [P]
    lib.wlc_net_last_error.restype = ctypes.c_char_p
    lib.wlc_net_param_count.argtypes = [P]
    lib.wlc_net_param_count.restype = ctypes.c_int64
    lib.wlc_net_get_params.argtypes = [P, Fp]
    lib.wlc_net_set_params.argtypes = [P, Fp]
    lib.wlc_net_forward.argtypes = [P, Fp, Fp]
    lib.wlc_net_loss_grad.argtypes = [P, Fp, Fp, Dp, Fp]
    lib.wlc_net_train.argtypes = [P, Fp, Fp, I, I, I, ctypes.c_float, ctypes.c_uint64, Dp]
    Ip = ctypes.POINTER(ctypes.c_int32)
    lib.wlc_autotune.argtypes = [P, Ip]
    lib.wlc_set_launch_config.argtypes = [P, I, I, I, I]
    lib.wlc_batch_create.argtypes = [ctypes.POINTER(Params), I, ctypes.POINTER(P)]
    lib.wlc_batch_destroy.argtypes = [P]
    lib.wlc_batch_last_error.argtypes = [P]
    lib.wlc_batch_last_error.restype = ctypes.c_char_p
    lib.wlc_batch_size.argtypes = [P]
    lib.wlc_batch_groups.argtypes = [P]
    lib.wlc_batch_get.argtypes = [P, I, ctypes.POINTER(P)]
    lib.wlc_batch_propagate.argtypes = [P]
    lib.wlc_batch_autotune.argtypes = [P, Ip]
    lib.wlc_batch_use_graph.argtypes = [P, I]
    lib.wlc_batch_stream.argtypes = [P]
    lib.wlc_batch_stream.restype = P
    lib.wlc_batch_launch_count.argtypes = [P]
    lib.wlc_batch_launch_count.restype = ctypes.c_int64
    _LIB = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def even_block_lengths(f, nmax):
    """Block lengths NA, NB, NC from fractions: the reference uses
    NINT(f*Nmax) and stops unless all three are even
    (initialize_mod.f90:142-144,190-195); here each of NA and NC is rounded
    to the nearest even integer and NB takes the remainder (also even when
    Nmax is even)."""
    def ev(x):
        return int(2 * math.floor(x / 2.0 + 0.5))
    na = ev(f[0] * nmax)
    nc = ev(f[2] * nmax) if len(f) > 2 else ev((1.0 - f[0] - f[1]) * nmax)
    nb = nmax - na - nc
    return na, nb, nc


def wlc_radius_of_gyration(x):
    """Rg / L for a wormlike chain of contour/persistence ratio x = L/lp."""
    return math.sqrt(1.0 / (3.0 * x) - 1.0 / x ** 2 + 2.0 / x ** 3 - 2.0 / x ** 4 * (1.0 - math.exp(-x)))


def make_params(n, lmax, nmax, ns, dx, loa, kappa, chi, nmu=0.0, precision=WLC_FP64, literals=WLC_LIT_REAL4,
                store_qstar=1, q_checkpoint=0, scheme=WLC_SCHEME_BDF):
    """wlc_params of one instance (kappa, chi: 3-tuples; n, dx: scalar or 3-tuple)."""
    p = Params()
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    dx = (dx, dx, dx) if np.isscalar(dx) else tuple(dx)
    p.n[:] = [int(v) for v in n]
    p.lmax = int(lmax)
    p.nmax = int(nmax)
    p.ns[:] = [int(v) for v in ns]
    p.dx[:] = [float(v) for v in dx]
    p.loa = float(loa)
    p.kappa[:] = [float(v) for v in kappa]
    p.chi[:] = [float(v) for v in chi]
    p.nmu = float(nmu)
    p.precision = int(precision)
    p.literals = int(literals)
    p.store_qstar = int(store_qstar)
    p.q_checkpoint = int(q_checkpoint)
    p.scheme = int(scheme)
    return p


class Instance:
    """One ABC-triblock instance on the current CUDA device."""

    def __init__(self, n, lmax, nmax, ns, dx, loa, kappa, chi, nmu=0.0, precision=WLC_FP64,
                 literals=WLC_LIT_REAL4, store_qstar=1, q_checkpoint=0, scheme=WLC_SCHEME_BDF):
        self.lib = load()
        p = make_params(n, lmax, nmax, ns, dx, loa, kappa, chi, nmu, precision, literals, store_qstar, q_checkpoint,
                        scheme)
        self._init_from(p)
        self.owned = True
        self.h = ctypes.c_void_p()
        rc = self.lib.wlc_create(ctypes.byref(p), ctypes.byref(self.h))
        if rc != 0:
            msg = self.lib.wlc_last_error(self.h).decode() if self.h else ""
            self.lib.wlc_destroy(self.h)
            self.h = None
            raise WlcError(rc, msg)

    def _init_from(self, p):
        self.params = p
        self.n = tuple(p.n)
        self.nr = self.n[0] * self.n[1] * self.n[2]
        self.M = (p.lmax + 1) ** 2
        self.nmax = p.nmax

    @classmethod
    def _wrap(cls, lib, h, p, owner):
        """A batch member: the handle belongs to the batch (owner)."""
        self = cls.__new__(cls)
        self.lib = lib
        self._init_from(p)
        self.owned = False
        self.h = h
        self._owner = owner
        return self

    def _check(self, rc):
        if rc != 0:
            raise WlcError(rc, self.lib.wlc_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None) and getattr(self, "owned", True):
            self.lib.wlc_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def volume(self):
        d = self.params.dx
        return d[0] * d[1] * d[2] * self.nr

    @property
    def launch_count(self):
        return self.lib.wlc_launch_count(self.h)

    @property
    def stream(self):
        return self.lib.wlc_stream(self.h)

    # -------------------------------------------------- reference entry points
    def init_inverse_sparse_GAB(self, dx=None):
        """Box change: Gmatrix_2dcomp_mod.f90:222 (the k-space operator is
        rebuilt from the new spacing)."""
        if dx is not None:
            d = (dx, dx, dx) if np.isscalar(dx) else tuple(dx)
            self.params.dx[:] = [float(v) for v in d]
        d = self.params.dx
        self._check(self.lib.wlc_set_box(self.h, d[0], d[1], d[2]))

    def set_fields(self, w, m_op=None):
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(3, self.nr)
        self._w = w
        if m_op is None:
            self._check(self.lib.wlc_set_fields(self.h, _dp(w), None))
        else:
            m = np.ascontiguousarray(m_op, dtype=np.float64).reshape(9, self.nr)
            self._m = m
            self._check(self.lib.wlc_set_fields(self.h, _dp(w), _dp(m)))

    def calc_THETAij(self):
        """Theta(r) is built from M_OP inside every step on the device
        (wormlike_MDE_2dcomp_mod.f90:5-110); nothing to precompute."""
        return None

    def MDE_q(self):
        self._check(self.lib.wlc_propagate(self.h, 1))

    def MDE_qstar(self):
        self._check(self.lib.wlc_propagate(self.h, -1))

    def ABC_melt_driver(self):
        self.MDE_q()
        self.MDE_qstar()

    def density(self, want_s=False, want_junction=True):
        phi = np.empty((3, self.nr))
        junc = np.empty((3, self.nr)) if want_junction else None
        sop = np.empty((3, 3, 3, self.nr)) if want_s else None
        lnq = np.zeros(1)
        self._check(self.lib.wlc_density(self.h, _dp(phi), _dp(junc) if want_junction else None,
                                         _dp(sop) if want_s else None, _dp(lnq)))
        out = dict(lnQ=float(lnq[0]), phi=phi)
        if want_junction:
            out["junction"] = junc
        if want_s:
            # sop[blk][b][a][r] = S_OP_blk(r, a, b, blk)
            out["S"] = sop
        return out

    def free_energy(self):
        fe = np.zeros(1)
        self._check(self.lib.wlc_free_energy(self.h, _dp(fe)))
        return float(fe[0])

    def get_q(self, direction, s):
        out = np.empty((self.nr, self.M))
        self._check(self.lib.wlc_get_q(self.h, int(direction), int(s), _dp(out)))
        return out

    def set_q(self, direction, s, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.nr, self.M)
        self._check(self.lib.wlc_set_q(self.h, int(direction), int(s), _dp(q)))

    def init_pr(self, direction, s):
        out = np.empty((self.nr, self.M))
        self._check(self.lib.wlc_init_pr(self.h, int(direction), int(s), _dp(out)))
        return out

    def mde_one_step(self, g_index, pr, out=None):
        pr = np.ascontiguousarray(pr, dtype=np.float64).reshape(self.nr, self.M)
        if out is None:
            out = np.empty((self.nr, self.M))
        self._check(self.lib.wlc_mde_one_step(self.h, int(g_index), _dp(pr), _dp(out)))
        return out

    def enable_timing(self, on=True):
        self._check(self.lib.wlc_enable_timing(self.h, 1 if on else 0))

    def last_timing(self):
        t = np.zeros(4)
        self._check(self.lib.wlc_last_timing(self.h, _dp(t)))
        return t

    # ---------------------------------------------------------- SCFT loop
    def iterate(self, mix=None, **kw):
        """iterate(converge) (SCFT_iterate.f90:27-334, three-block form) on the
        device; returns (err[5], converged).  err[0..2] block errors, err[3]
        max |sum_K phi_K - 1|, err[4] the Maier-Saupe tensor error (nmu != 0)."""
        mp = mix if mix is not None else mix_params(**kw)
        err = np.zeros(5)
        conv = ctypes.c_int32(0)
        self._check(self.lib.wlc_iterate(self.h, ctypes.byref(mp), _dp(err), ctypes.byref(conv)))
        return err, bool(conv.value)

    def set_precision(self, precision):
        """WLC_FP64 or WLC_FP32 propagators from the next sweep on."""
        self._check(self.lib.wlc_set_precision(self.h, int(precision)))
        self.params.precision = int(precision)

    def autotune(self):
        """Time the launch configurations of a contour step on this
        instance's data and keep the fastest; returns (a_variant,
        solve_threads, xy_threads, xy_variant)."""
        cfg = (ctypes.c_int32 * 4)()
        self._check(self.lib.wlc_autotune(self.h, cfg))
        return tuple(int(v) for v in cfg)

    def set_launch_config(self, a_variant=0, solve_threads=0, xy_threads=0, xy_variant=0):
        self._check(self.lib.wlc_set_launch_config(self.h, int(a_variant), int(solve_threads), int(xy_threads),
                                                   int(xy_variant)))

    def reset_mixing(self):
        self._check(self.lib.wlc_reset_mixing(self.h))

    def W_dump(self, directory=".", rank=0):
        """W_dump (SCFT_dump.f90:273-308): W<rank>.dat and M_OP<rank>.dat."""
        box = [self.params.dx[a] * self.n[a] for a in range(3)]
        io.write_w(os.path.join(directory, "W%d.dat" % rank), self.get_fields())
        io.write_mop(os.path.join(directory, "M_OP%d.dat" % rank), self.get_mop(), box)

    def readW(self, directory=".", rank=0):
        """readW (init_array_2dcomp_mod.f90:1070-1106): fields and M_OP from
        W<rank>.dat / M_OP<rank>.dat (M_OP optional)."""
        w = io.read_w(os.path.join(directory, "W%d.dat" % rank), self.nr)
        mpath = os.path.join(directory, "M_OP%d.dat" % rank)
        self.set_fields(w, io.read_mop(mpath, self.nr) if os.path.exists(mpath) else None)

    def get_mop(self):
        """M_OP as a (3, 3, nr) array [b][a][r] (symmetric)."""
        m = np.empty((3, 3, self.nr))
        self._check(self.lib.wlc_get_mop(self.h, _dp(m)))
        return m

    def get_fields(self):
        w = np.empty((3, self.nr))
        self._check(self.lib.wlc_get_fields(self.h, _dp(w)))
        return w

    def cal_scft(self, max_iter=5000, mix=None, callback=None, **kw):
        """The SCFT loop of cal_scft (SCFT_control.f90:237-273): propagators,
        density, free energy and field update until converged or max_iter
        (MAXITS = 5000, global_parameters.f90:69) iterations.  Returns
        dict(F, lnQ, n_iter, converged, history=[(F, err)])."""
        mp = mix if mix is not None else mix_params(**kw)
        hist = []
        conv, n, d, fe = False, 0, None, float("nan")
        while not conv and n < max_iter:
            n += 1
            self.MDE_q()
            self.MDE_qstar()
            d = self.density(want_junction=False)
            fe = self.free_energy()
            err, conv = self.iterate(mp)
            hist.append((fe, err.copy()))
            if callback is not None:
                callback(n, fe, err)
        return dict(F=fe, lnQ=d["lnQ"] if d else float("nan"), n_iter=n, converged=conv, history=hist)


class Batch:
    """Independent FP32 instances advanced together (wlc_batch_*): batched
    launches per grid-size group, the contour loop replayed as a CUDA graph.
    `specs` is a list of make_params keyword dicts; members are Instance
    objects (self.instances) for fields, densities, free energy and mixing."""

    def __init__(self, specs):
        self.lib = load()
        arr = (Params * len(specs))()
        for i, kw in enumerate(specs):
            kw = dict(kw)
            kw.setdefault("precision", WLC_FP32)
            kw.setdefault("store_qstar", 0)
            arr[i] = make_params(**kw)
        self.h = ctypes.c_void_p()
        rc = self.lib.wlc_batch_create(arr, len(specs), ctypes.byref(self.h))
        if rc != 0:
            msg = self.lib.wlc_batch_last_error(self.h).decode() if self.h else ""
            self.lib.wlc_batch_destroy(self.h)
            self.h = None
            raise WlcError(rc, msg)
        self.instances = []
        for i in range(len(specs)):
            hi = ctypes.c_void_p()
            self._check(self.lib.wlc_batch_get(self.h, i, ctypes.byref(hi)))
            self.instances.append(Instance._wrap(self.lib, hi, arr[i], self))

    def _check(self, rc):
        if rc != 0:
            raise WlcError(rc, self.lib.wlc_batch_last_error(self.h).decode())

    def __len__(self):
        return len(self.instances)

    def __getitem__(self, i):
        return self.instances[i]

    def propagate(self):
        """MDE_q and MDE_qstar of every instance."""
        self._check(self.lib.wlc_batch_propagate(self.h))

    def autotune(self):
        g = self.lib.wlc_batch_groups(self.h)
        cfg = (ctypes.c_int32 * (5 * max(1, g)))()
        self._check(self.lib.wlc_batch_autotune(self.h, cfg))
        return [tuple(int(cfg[5 * i + k]) for k in range(5)) for i in range(g)]

    def use_graph(self, on=True):
        self._check(self.lib.wlc_batch_use_graph(self.h, 1 if on else 0))

    @property
    def stream(self):
        return self.lib.wlc_batch_stream(self.h)

    @property
    def launch_count(self):
        return self.lib.wlc_batch_launch_count(self.h)

    def close(self):
        if getattr(self, "h", None):
            for inst in getattr(self, "instances", []):
                inst.h = None
            self.lib.wlc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class io:
    """The reference's files (W<rank>.dat, M_OP<rank>.dat, RHO_total.dat,
    FreeEG.dat, error.dat) through libwlc's host-side readers and writers."""

    @staticmethod
    def _rc(rc, what):
        if rc != 0:
            raise WlcError(rc, what)

    @staticmethod
    def write_w(path, w):
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(3, -1)
        io._rc(load().wlc_io_write_w(os.fsencode(path), _dp(w), w.shape[1]), "write " + str(path))

    @staticmethod
    def read_w(path, nr):
        w = np.empty((3, nr))
        io._rc(load().wlc_io_read_w(os.fsencode(path), _dp(w), nr), "read " + str(path))
        return w

    @staticmethod
    def write_mop(path, m_op, box):
        m = np.ascontiguousarray(m_op, dtype=np.float64).reshape(9, -1)
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(3)
        io._rc(load().wlc_io_write_mop(os.fsencode(path), _dp(m), m.shape[1], _dp(b)), "write " + str(path))

    @staticmethod
    def read_mop(path, nr):
        m = np.empty((3, 3, nr))
        io._rc(load().wlc_io_read_mop(os.fsencode(path), _dp(m), nr), "read " + str(path))
        return m

    @staticmethod
    def write_rho(path, phi, n, dx):
        phi = np.ascontiguousarray(phi, dtype=np.float64).reshape(3, -1)
        nn = (ctypes.c_int32 * 3)(*[int(v) for v in n])
        d = np.ascontiguousarray(dx, dtype=np.float64).reshape(3)
        io._rc(load().wlc_io_write_rho(os.fsencode(path), _dp(phi), nn, _dp(d)), "write " + str(path))

    @staticmethod
    def append_free_energy(path, n_iter, fe, lnq, box, chi, ns, nmax):
        c = np.ascontiguousarray(chi, dtype=np.float64).reshape(3)
        nn = (ctypes.c_int32 * 3)(*[int(v) for v in ns])
        io._rc(load().wlc_io_append_free_energy(os.fsencode(path), int(n_iter), float(fe), float(lnq), float(box),
                                                _dp(c), nn, int(nmax)), "append " + str(path))

    @staticmethod
    def append_errors(path, n_iter, err):
        e = np.ascontiguousarray(err, dtype=np.float64).reshape(-1)
        io._rc(load().wlc_io_append_errors(os.fsencode(path), int(n_iter), _dp(e), len(e)), "append " + str(path))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class WarmStartNet:
    """Learned warm start (wlc_net_*): a 3D conv encoder-decoder on a G^3
    grid, BF16 tensor-core kernels with FP32 accumulation, trained on the
    device.  Input (6, G^3): a noise field and five instance parameters as
    constant fields; output (3, G^3): normalised block fields."""

    def __init__(self, grid=32, width=32, seed=1):
        self.lib = load()
        self.G, self.C = int(grid), int(width)
        self.h = ctypes.c_void_p()
        rc = self.lib.wlc_net_create(self.G, self.C, int(seed), ctypes.byref(self.h))
        if rc != 0:
            msg = self.lib.wlc_net_last_error(self.h).decode() if self.h else ""
            self.lib.wlc_net_destroy(self.h)
            self.h = None
            raise WlcError(rc, msg)
        self.np = self.lib.wlc_net_param_count(self.h)

    def _check(self, rc):
        if rc != 0:
            raise WlcError(rc, self.lib.wlc_net_last_error(self.h).decode())

    @property
    def npts(self):
        return self.G ** 3

    def params(self):
        p = np.empty(self.np, dtype=np.float32)
        self._check(self.lib.wlc_net_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32).reshape(self.np)
        self._check(self.lib.wlc_net_set_params(self.h, _fp(p)))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(6, self.npts)
        out = np.empty((3, self.npts), dtype=np.float32)
        self._check(self.lib.wlc_net_forward(self.h, _fp(x), _fp(out)))
        return out

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(6, self.npts)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(3, self.npts)
        loss = np.zeros(1)
        g = np.empty(self.np, dtype=np.float32)
        self._check(self.lib.wlc_net_loss_grad(self.h, _fp(x), _fp(t), _dp(loss), _fp(g)))
        return float(loss[0]), g

    def train(self, inputs, targets, batch=8, epochs=10, lr=1e-3, seed=7):
        x = np.ascontiguousarray(inputs, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        n = x.shape[0]
        hist = np.zeros(epochs)
        self._check(self.lib.wlc_net_train(self.h, _fp(x.reshape(-1)), _fp(t.reshape(-1)), n, int(batch),
                                           int(epochs), float(lr), int(seed), _dp(hist)))
        return hist

    def close(self):
        if getattr(self, "h", None):
            self.lib.wlc_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
