#!/usr/bin/env python3
"""Benchmark of the wormlike-chain MDE hot path on GB300.

Workload (the single-GPU configuration of the headline metric): one ABC
triblock instance, 64^3 grid, box edge 5.0 Rg, l <= 10 (121 real-harmonic
coefficients), Ns = 200 (blocks 50/100/50), chiN = 18 for all pairs,
contour/persistence = 2.0, seeded random fields w ~ N(0, 0.5^2).

One bench step = one SCFT iteration's hot path: forward propagator sweep
(MDE_q), backward sweep (MDE_qstar), densities + Q (density) and the free
energy -- 2*Ns = 400 contour steps.  `value` is contour steps/s with the
fields resident on the device; `e2e` is the same metric through the C ABI
with the fields copied host->device (pinned) and the block densities copied
back every step.  The propagator history (51 GB per direction in FP64) is far
larger than L2, so no L2 flush is needed between steps.

--impl reference times the CPU restatement of the reference's step (the
reference itself cannot be built: no Fortran/MPI/FFTW/MKL and undefined
routines) on the host cores, on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "wormlike-chain-triblock_gb300"))

import numpy as np  # noqa: E402

PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def workload(precision):
    import wlc
    x = 2.0  # contour / persistence
    rg = wlc.wlc_radius_of_gyration(x)  # Rg / L
    box = 5.0 * rg
    n, L, nmax = 64, 10, 200
    ns = wlc.even_block_lengths((0.25, 0.50, 0.25), nmax)
    kappa = 0.5  # kapa_A of the reference; Loa/kappa = L/lp
    return dict(n=n, L=L, nmax=nmax, ns=ns, dx=box / n, loa=x * kappa, kappa=(kappa,) * 3,
                chi=(18.0, 18.0, 18.0), box=box, precision=precision, w_sigma=0.5)


def algorithmic_bytes(wl, bq):
    """Per contour step: BDF3 history read (3 slices) + one slice written +
    the block field: (3+1)*M*N^3*b_q + 8*N^3."""
    M = (wl["L"] + 1) ** 2
    nr = wl["n"] ** 3
    return 4 * M * nr * bq + 8 * nr


def pass_bytes(wl, bq):
    """Minimal DRAM bytes of each pass of one step: A reads the history and
    writes the k-space planes, B reads and writes them, C reads them and
    writes the new slice."""
    M = (wl["L"] + 1) ** 2
    n = wl["n"]
    nr = n ** 3
    nk = (n // 2 + 1) * n * n
    kspace = M * nk * 2 * bq
    return {"A": 3 * M * nr * bq + 8 * nr + kspace, "B": 2 * kspace, "C": kspace + M * nr * bq}


class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_throughput(units_local, seconds_local, group=None):
    """Whole-job throughput of independent replicas: units summed over
    ranks divided by the slowest rank's time (max over ranks)."""
    import torch
    import torch.distributed as dist
    if group is None and not (dist.is_available() and dist.is_initialized()):
        return units_local / seconds_local, units_local, seconds_local
    u = torch.tensor([float(units_local)], dtype=torch.float64)
    t = torch.tensor([float(seconds_local)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        u, t = u.cuda(), t.cuda()
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()) / float(t.item()), float(u.item()), float(t.item())


WORKLOAD_SINGLE = ("ABC triblock 64^3, box 5.0 Rg, L=10 (M=121), Ns=200 (50/100/50), chiN=18, L/lp=2.0; "
                   "metric unit: one contour step (BDF3 RHS, R2C FFTs, per-k G solve, C2R FFTs, density "
                   "contribution of the slice)")


class CpuArm:
    """The CPU restatement of the reference's step (the oracle, test
    infrastructure; the reference itself cannot be built) at this workload,
    on all host cores: whole BDF3 contour steps -- every wavevector's solve
    and the slice's density contribution -- with the LU factors of G(k)
    built once before the clock starts, as the reference precomputes G^-1."""

    def __init__(self, wl, nthreads=None):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        self.nthreads = nthreads or os.cpu_count() or 1
        n = wl["n"]
        self.o = oracle.Oracle((n, n, n), wl["L"], 4, (2, 2, 0), (wl["dx"],) * 3, wl["loa"], wl["kappa"], wl["chi"],
                               nthreads=self.nthreads)
        rng = np.random.default_rng(11)
        self.o.set_fields(rng.normal(0.0, wl["w_sigma"], size=(3, n ** 3)))
        M = (wl["L"] + 1) ** 2
        for s in range(4):
            self.o.set_q(1, s, rng.random((M, n ** 3)))
        self.o.set_q(-1, 0, rng.random((M, n ** 3)))
        self.setup_s = None

    def steps(self, nsteps):
        """Time nsteps whole contour steps; returns seconds per step."""
        setup, timed, per = self.o.bench_steps(nsteps)
        if self.setup_s is None:
            self.setup_s = setup
        return per

    def close(self):
        self.o.close()


def cpu_sample(wl, nsteps=4):
    """cpu_baseline of the default run: `nsteps` whole contour steps."""
    arm = CpuArm(wl)
    per = arm.steps(nsteps)
    out = dict(steps_per_s=1.0 / per, cores=arm.nthreads, setup_s=arm.setup_s, nsteps=nsteps)
    arm.close()
    return out


def cpu_sample_text(nsteps, setup_s):
    return ("%d whole BDF3 contour steps of the 64^3, L=10 workload (RHS, R2C FFTs of all 121 coefficients, dense "
            "LU solve at every one of the 135168 wavevectors, C2R FFTs, density contribution of the slice); LU "
            "factors built once before timing (%.1f s, as the reference precomputes G^-1)" % (nsteps, setup_s))


def run_reference(args, wl):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    arm = CpuArm(wl)
    per_step_contour = 2  # contour steps timed per bench step
    for _ in range(args.warmup):
        arm.steps(per_step_contour)
    t = 0.0
    for _ in range(args.steps):
        t += arm.steps(per_step_contour) * per_step_contour
    arm.close()
    v = args.steps * per_step_contour / t
    sample = cpu_sample_text(per_step_contour, arm.setup_s) + " per bench step"
    line = {"impl": "reference", "metric": "MDE contour steps/s (64^3, L=10, Ns=200, ABC)", "value": v,
            "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded N(0,0.5^2) fields)",
            "config": {"workload": WORKLOAD_SINGLE, "precision": "fp64"},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": arm.nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, wl):
    import torch
    import wlc
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    inst = wlc.Instance(wl["n"], wl["L"], wl["nmax"], wl["ns"], wl["dx"], wl["loa"], wl["kappa"], wl["chi"],
                        precision=wlc.WLC_FP64 if wl["precision"] == "fp64" else wlc.WLC_FP32)
    nr = wl["n"] ** 3
    rng = np.random.default_rng(1234 + rank)
    tuned = None
    w_host = torch.empty((3, nr), dtype=torch.float64).pin_memory()
    w_host.numpy()[:] = rng.normal(0.0, wl["w_sigma"], size=(3, nr))
    phi_host = torch.empty((3, nr), dtype=torch.float64).pin_memory()
    stream = torch.cuda.ExternalStream(inst.stream, device=dev)
    import ctypes
    lib = inst.lib
    h = inst.h
    wp = ctypes.cast(w_host.data_ptr(), ctypes.POINTER(ctypes.c_double))
    php = ctypes.cast(phi_host.data_ptr(), ctypes.POINTER(ctypes.c_double))
    lnq = np.zeros(1)
    lnqp = lnq.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    fe = np.zeros(1)
    fep = fe.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def check(rc):
        if rc != 0:
            raise RuntimeError(lib.wlc_last_error(h).decode())

    def device_step():
        check(lib.wlc_propagate(h, 1))
        check(lib.wlc_propagate(h, -1))
        check(lib.wlc_density(h, None, None, None, lnqp))

    def e2e_step():
        check(lib.wlc_set_fields(h, wp, None))
        check(lib.wlc_propagate(h, 1))
        check(lib.wlc_propagate(h, -1))
        check(lib.wlc_density(h, php, None, None, lnqp))
        check(lib.wlc_free_energy(h, fep))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    check(lib.wlc_set_fields(h, wp, None))
    if not args.no_autotune:
        tuned = inst.autotune()
    for _ in range(args.warmup):
        device_step()
    barrier()
    # ---- timed: device-resident
    inst.enable_timing(True)
    clk = ClockSampler(local)
    clk.start()
    l0 = inst.launch_count
    ev = []
    pass_ms = np.zeros(4)
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        device_step()
        e.record(stream)
        ev.append((s, e))
        pass_ms += inst.last_timing()  # per-sweep sums of the last (backward) sweep only
    barrier()
    t_wall = time.perf_counter() - t_wall0
    clocks = clk.stop()
    launches = inst.launch_count - l0
    ms = [s.elapsed_time(e) for s, e in ev]
    ms_total = float(sum(ms))
    inst.enable_timing(False)
    steps_per_bench = 2 * wl["nmax"]
    value, _, t_max = replica_throughput(steps_per_bench * args.steps, ms_total / 1000.0)
    ms_total = t_max * 1000.0
    # ---- timed: end to end through the C ABI with host buffers
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e, _, e2e_s = replica_throughput(steps_per_bench * args.steps, e2e_s)
    # ---- roofline of the dominant pass (pass times are of one sweep of Ns steps)
    bq = 8 if wl["precision"] == "fp64" else 4
    pb = pass_bytes(wl, bq)
    per_pass = {"A": pass_ms[0], "B": pass_ms[1], "C": pass_ms[2]}
    dom = max(per_pass, key=per_pass.get)
    launches_per_sweep = args.steps * wl["nmax"]
    avg_ms = per_pass[dom] / launches_per_sweep
    peak, peak_kind = load_peaks()
    achieved = pb[dom] / (avg_ms / 1000.0) / 1e9
    step_ms = ms_total / (args.steps * steps_per_bench)
    b_step = algorithmic_bytes(wl, bq)
    pass_names = {"A": "rhs_fft_xy", "B": "zfft_solve", "C": "ifft_xy"}
    share = {pass_names[k]: per_pass[k] / max(1e-9, sum(per_pass.values())) for k in per_pass}
    traffic = None
    tfile = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tfile):
        try:
            with open(tfile) as f:
                tj = json.load(f)
            traffic = tj.get(wl["precision"], {}).get(pass_names[dom])
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": pass_names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                "bytes_per_launch": pb[dom], "avg_launch_ms": avg_ms, "kernel_share": share,
                "binding_limit": ("FP64 pipe: 75-84 % active in every pass (ncu); the HBM fraction is"
                                  " reported alongside") if bq == 8 else
                                 "latency-bound shared-memory FFT stages (ncu: 8-18 % DRAM, ~10 % FMA pipe)",
                "step": {"algorithmic_bytes": b_step, "ms": step_ms,
                         "achieved_gbs": b_step / (step_ms / 1000.0) / 1e9,
                         "frac": b_step / (step_ms / 1000.0) / 1e9 / peak}}
    h2d = 3 * nr * 8
    d2h = 3 * nr * 8 + 16
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        r = cpu_sample(wl)
        cpu = {"value": r["steps_per_s"], "unit": "steps/s", "cores": r["cores"], "kind": "port",
               "sample": cpu_sample_text(r["nsteps"], r["setup_s"])}
    forms = None
    if wl["precision"] == "fp64" and not args.no_fp32:
        # the FP32 form of the same workload, measured the same way (device-resident)
        inst.close()
        torch.cuda.synchronize()
        i32 = wlc.Instance(wl["n"], wl["L"], wl["nmax"], wl["ns"], wl["dx"], wl["loa"], wl["kappa"], wl["chi"],
                           precision=wlc.WLC_FP32)
        i32.set_fields(w_host.numpy())
        t32 = None if args.no_autotune else i32.autotune()
        s32 = torch.cuda.ExternalStream(i32.stream, device=dev)
        for _ in range(args.warmup):
            i32.MDE_q()
            i32.MDE_qstar()
            i32.density(want_junction=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s32)
        for _ in range(args.steps):
            i32.MDE_q()
            i32.MDE_qstar()
            i32.density(want_junction=False)
        e1.record(s32)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1)
        v32 = steps_per_bench * args.steps / (ms32 / 1000.0)
        b32 = algorithmic_bytes(wl, 4)
        st32 = ms32 / (args.steps * steps_per_bench)
        forms = {"fp32": {"value": v32, "unit": "steps/s", "ms_per_step": ms32 / args.steps,
                          "step_hbm_frac": b32 / (st32 / 1000.0) / 1e9 / peak,
                          "launch_config": list(t32) if t32 else "default",
                          "note": "FP32 propagators, FP64 densities/Q; same workload and timing"}}
        i32.close()
        inst = None
    if rank == 0:
        line = {"metric": "MDE contour steps/s (64^3, L=10, Ns=200, ABC)", "value": value, "unit": "steps/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_total / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if wl["precision"] == "fp64" else "f32",
                "data": "synthetic (seeded N(0,0.5^2) fields)",
                "config": {"workload": WORKLOAD_SINGLE, "precision": wl["precision"],
                           "bench_step": "forward + backward sweep + densities (400 contour steps)", "l2": "inputs larger than L2 (51 GB history/direction)",
                           "parallelism": "replicas" if world > 1 else "single",
                           "launch_config": {"a_variant": tuned[0], "solve_threads": tuned[1],
                                             "xy_threads": tuned[2], "xy_variant": tuned[3]} if tuned else
                           "default"},
                "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "wall_s": t_wall, "other_forms": forms}
        print(json.dumps(line))
    if inst is not None:
        inst.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_profile_case(args):
    """Small-footprint case for ncu captures: the headline kernels (64^3,
    L=10) on a 6-step chain (2/2/2), two forward and one backward sweep, a
    density pass; a few GB of device memory."""
    import wlc
    wl = workload(args.precision)
    if args.workload == "large":  # the large workload's grid and L on a 6-step chain, K = 3
        n = 128
        inst = wlc.Instance(n, 12, 6, (2, 2, 2), 8.0 * wlc.wlc_radius_of_gyration(4.0) / n, 2.0, (0.5, 0.5, 0.5),
                            (20.0, 20.0, 20.0), nmu=5.0, precision=wlc.WLC_FP32, store_qstar=2, q_checkpoint=3)
        rng = np.random.default_rng(5)
        inst.set_fields(rng.normal(0.0, 0.5, size=(3, n ** 3)), rng.normal(0.0, 0.1, size=(3, 3, n ** 3)))
        if args.launch_config:
            inst.set_launch_config(*(int(v) for v in args.launch_config.split(",")))
        inst.MDE_q()
        inst.MDE_qstar()
        d = inst.density(want_junction=False)
        inst.free_energy()
        inst.iterate(wlc.mix_params())
        print(json.dumps({"profile_case": "large", "lnQ": d["lnQ"], "launches": inst.launch_count}))
        inst.close()
        return
    inst = wlc.Instance(wl["n"], wl["L"], 6, (2, 2, 2), wl["dx"], wl["loa"], wl["kappa"], wl["chi"],
                        precision=wlc.WLC_FP64 if args.precision == "fp64" else wlc.WLC_FP32)
    rng = np.random.default_rng(5)
    inst.set_fields(rng.normal(0.0, wl["w_sigma"], size=(3, wl["n"] ** 3)))
    if args.launch_config:
        inst.set_launch_config(*(int(v) for v in args.launch_config.split(",")))
    inst.MDE_q()
    inst.MDE_q()
    inst.MDE_qstar()
    d = inst.density()
    print(json.dumps({"profile_case": args.precision, "lnQ": d["lnQ"], "launches": inst.launch_count}))
    inst.close()


def c2_draw(seed):
    """The headline instance as a warm-start draw (64^3 run, box 5.0 Rg)."""
    return dict(fa=0.25, fc=0.25, chi=18.0, x=2.0, box=5.0, noise_seed=int(seed))


def converge_form(wl, w0, form, args):
    """One SCFT run to residual <= args.tol from fields w0 (wall time
    includes everything: propagators, densities copied back, free energy,
    field update on the device).  form 'fp64': FP64 propagators throughout;
    'fp32': FP32 propagators until the residual falls below --switch-tol or
    stops improving for --stall iterations (FP32's floor), then FP64 with a
    fresh Anderson history (one simple-mixing iteration, then Anderson)."""
    import torch
    import wlc
    prec = wlc.WLC_FP32 if form == "fp32" else wlc.WLC_FP64
    inst = wlc.Instance(wl["n"], wl["L"], wl["nmax"], wl["ns"], wl["dx"], wl["loa"], wl["kappa"], wl["chi"],
                        precision=prec, store_qstar=1 if args.stored else 0)
    inst.set_fields(w0)
    if not args.no_autotune:
        inst.autotune()
    mp = wlc.mix_params(anderson_depth=args.depth, num_simple=20, lambda_anderson=args.lambda_a, tol=args.tol,
                        min_iter=20, relax_iter=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    inst.set_fields(w0)
    hist, n, conv = [], 0, False
    switched, t_switch, best, since = None, None, np.inf, 0
    while not conv and n < args.max_iter and time.perf_counter() - t0 < args.budget:
        n += 1
        inst.MDE_q()
        inst.MDE_qstar()
        d = inst.density(want_junction=False)
        fe = inst.free_energy()
        err, conv = inst.iterate(mp)
        r = float(max(err[:3]))
        hist.append([n, fe, d["lnQ"], r])
        if not np.isfinite(r):
            break
        if args.lambda_late > 0 and n > 20 and r < args.late_below:
            mp.lambda_anderson = args.lambda_late  # larger Anderson weight close to the solution
        if form == "fp32" and switched is None and not conv:
            if r < 0.98 * best:
                best, since = r, 0
            else:
                since += 1
            if n > 20 and (r < args.switch_tol or (since >= args.stall and best < 1e-3)):
                inst.set_precision(wlc.WLC_FP64)
                inst.reset_mixing()
                mp.num_simple, mp.min_iter = 1, 2
                switched, t_switch = n, time.perf_counter() - t0
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    w_fin = inst.get_fields()
    inst.close()
    res = {"converged": bool(conv), "iterations": n, "seconds": secs, "F": hist[-1][1], "lnQ": hist[-1][2],
           "residual": hist[-1][3], "s_per_iteration": secs / max(1, n), "switched_at": switched,
           "switch_seconds": t_switch, "residual_every_10": [h[3] for h in hist[::10]]}
    if args.history:
        res["history"] = hist
    return res, w_fin


def run_converge(args):
    """Time to converged F at the 64^3, L=10, Ns=200 workload (residual <=
    --tol in every block), through the public API:
      fp64_cold  plain FP64 from the seeded random fields N(0, 0.5^2)
                 (capped at --budget seconds);
      fp64_warm  plain FP64 from the learned warm start;
      fp32_warm  FP32 propagators (FP64 Q, F, densities, residuals and
                 Anderson least squares) from the learned warm start, FP64
                 for the last iterations (FP32's residual floor is above 1e-6).
    The warm start is the network (--ws-load) evaluated at this instance's
    parameters on its 32^3 grid and Fourier-resampled to 64^3; one run per
    noise seed (--seeds)."""
    import wlc
    from wlc import warmstart as ws
    wl = workload("fp64")
    nr = wl["n"] ** 3
    w_cold = np.random.default_rng(2024).normal(0.0, wl["w_sigma"], size=(3, nr))
    net = None
    forms = args.forms.split(",")
    if any(f.endswith("_warm") for f in forms):
        if not args.ws_load:
            raise SystemExit("warm forms need --ws-load (parameters saved by --workload warmstart --ws-save)")
        net = wlc.WarmStartNet(ws.GRID, 32, seed=1)
        net.set_params(np.load(args.ws_load))
    out = {"metric": "time-to-converged F (64^3, L=10, Ns=200, ABC; residual <= %g)" % args.tol,
           "config": {"workload": WORKLOAD_SINGLE, "tol": args.tol, "switch_tol": args.switch_tol,
                      "stall": args.stall, "budget_s": args.budget,
                      "mixing": {"anderson_depth": args.depth, "num_simple": 20, "lambda_simple": 0.1,
                                 "lambda_anderson": args.lambda_a, "lambda_late": args.lambda_late,
                                 "late_below": args.late_below}},
           "runs": []}
    cold = None
    if "fp64_cold" in forms:
        cold, _ = converge_form(wl, w_cold, "fp64", args)
        out["fp64_cold"] = cold
        print(json.dumps({"form": "fp64_cold", **{k: v for k, v in cold.items() if k != "history"}}), flush=True)
    for seed in [int(v) for v in args.seeds.split(",")]:
        run = {"seed": seed}
        w_warm = None
        if net is not None:
            tp = time.perf_counter()
            w_warm = ws.predict(net, [c2_draw(seed)], grid_out=wl["n"])[0]
            run["predict_seconds"] = time.perf_counter() - tp
        for f in forms:
            if f == "fp64_cold":
                continue
            r, _ = converge_form(wl, w_warm, "fp32" if f == "fp32_warm" else "fp64", args)
            if f == "fp32_warm":
                r["seconds"] += run.get("predict_seconds", 0.0)  # the prediction is part of this form's time
            run[f] = r
            print(json.dumps({"form": f, "seed": seed, **{k: v for k, v in r.items() if k != "history"}}),
                  flush=True)
        if "fp32_warm" in run and "fp64_warm" in run:
            a, b = run["fp32_warm"], run["fp64_warm"]
            run["F_rel_diff_fp32_warm_vs_fp64_warm"] = abs(a["F"] - b["F"]) / abs(b["F"])
            run["speedup_vs_fp64_warm"] = b["seconds"] / a["seconds"]
        if "fp32_warm" in run and cold is not None:
            run["speedup_vs_fp64_cold"] = cold["seconds"] / run["fp32_warm"]["seconds"]
            run["speedup_vs_fp64_cold_is_lower_bound"] = not cold["converged"]
        out["runs"].append(run)
    if net is not None:
        net.close()
    if out["runs"] and "fp32_warm" in out["runs"][0]:
        med = statistics.median([r["fp32_warm"]["seconds"] for r in out["runs"]])
        out["value"] = med
        out["unit"] = "s (median over seeds, fp32_warm)"
        out["e2e"] = {"value": med, "unit": "s", "h2d_bytes_per_step": 3 * nr * 8,
                      "d2h_bytes_per_step": 3 * nr * 8 + 24}
    print(json.dumps(out))


def batch_specs(count=48, seed=3):
    """The batched sweep workload: `count` independent instances, grid edge
    drawn from {24, 32, 40, 48}, l <= 8, Ns = 128, fA, fC ~ U(0.2, 0.4),
    fB = 1 - fA - fC, chiN ~ U(12, 24) for all pairs, contour/persistence
    ~ U(0.5, 3.0), box edge 5.0 Rg; FP32 propagators, streamed densities."""
    import wlc
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        n = int(rng.choice([24, 32, 40, 48]))
        fa, fc = rng.uniform(0.2, 0.4), rng.uniform(0.2, 0.4)
        chi = float(rng.uniform(12.0, 24.0))
        x = float(rng.uniform(0.5, 3.0))
        box = 5.0 * wlc.wlc_radius_of_gyration(x)
        specs.append(dict(n=n, lmax=8, nmax=128, ns=wlc.even_block_lengths((fa, 1.0 - fa - fc, fc), 128),
                          dx=box / n, loa=x * 0.5, kappa=(0.5, 0.5, 0.5), chi=(chi, chi, chi),
                          precision=wlc.WLC_FP32, store_qstar=0, seed=1000 + i))
    return specs


def run_batch(args):
    """Batched sweep: all instances' forward + backward sweeps per bench
    step (one graph replay), against the same instances swept one by one."""
    import torch
    import wlc
    specs = batch_specs(args.count)
    seeds = [s.pop("seed") for s in specs]
    b = wlc.Batch(specs)
    for inst, spec, sd in zip(b.instances, specs, seeds):
        inst.set_fields(np.random.default_rng(sd).normal(0.0, 0.3, size=(3, spec["n"] ** 3)))
    stream = torch.cuda.ExternalStream(b.stream)
    cfg = None if args.no_autotune else b.autotune()
    for _ in range(args.warmup):
        b.propagate()
    torch.cuda.synchronize()
    clk = ClockSampler(0)
    clk.start()
    l0 = b.launch_count
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        b.propagate()
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = ev0.elapsed_time(ev1)
    launches = b.launch_count - l0
    steps = 2 * 128 * len(specs) * args.steps
    value = steps / (ms / 1000.0)
    # the same batched launches issued directly instead of replayed as a graph
    b.use_graph(False)
    ev0.record(stream)
    for _ in range(args.steps):
        b.propagate()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_direct = ev0.elapsed_time(ev1)
    b.use_graph(True)
    # the same instances swept one by one (no batching, no graph)
    ev0.record(stream)
    for _ in range(args.steps):
        for inst in b.instances:
            inst.MDE_q()
            inst.MDE_qstar()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_seq = ev0.elapsed_time(ev1)
    # end to end: fields in from the host, densities and free energies out
    w_host = [np.random.default_rng(sd).normal(0.0, 0.3, size=(3, sp["n"] ** 3)) for sp, sd in zip(specs, seeds)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(args.steps):
        for inst, w in zip(b.instances, w_host):
            inst.set_fields(w)
            h2d += w.nbytes
        b.propagate()
        for inst in b.instances:
            d = inst.density(want_junction=False)
            inst.free_energy()
            d2h += d["phi"].nbytes + 16
    torch.cuda.synchronize()
    e2e = steps / (time.perf_counter() - t0)
    groups = {}
    for sp in specs:
        groups[sp["n"]] = groups.get(sp["n"], 0) + 1
    line = {"metric": "MDE contour steps/s, %d batched ABC instances (l<=8, Ns=128)" % len(specs),
            "value": value, "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (per-instance seeded N(0,0.3^2) fields)",
            "config": {"workload": "%d instances, N in {24,32,40,48} (%s), L=8, Ns=128, fA,fC~U(.2,.4), "
                                   "chiN~U(12,24), L/lp~U(.5,3), box 5 Rg; FP32 propagators, streamed densities; one "
                                   "bench step = forward + backward sweep of every instance" % (
                                       len(specs), ", ".join("%d x %d^3" % (v, k) for k, v in sorted(groups.items()))),
                       "l2": "inputs larger than L2 (the stored forward propagators total ~110 GB)",
                       "autotuned": cfg},
            "unbatched": {"value": steps / (ms_seq / 1000.0), "unit": "steps/s",
                          "note": "same instances swept one after another, one launch per pass per instance"},
            "graph": {"ms_per_propagate": ms / args.steps, "direct_ms_per_propagate": ms_direct / args.steps,
                      "launches_per_propagate": launches / args.steps,
                      "note": "one propagate = forward + backward sweep of every instance; direct = the same "
                              "batched launches issued one by one instead of replayed as a CUDA graph"},
            "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps},
            "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(line))
    b.close()


def run_large(args):
    """Large single instance with contour checkpointing: 128^3, box 8.0 Rg,
    l <= 12 (169 coefficients), Ns = 400 (120/160/120), chiN = 20,
    contour/persistence = 4.0, Maier-Saupe muN = 5, gyroid-like start (sum
    of sin.cos terms, amplitude 1.0, plus N(0, 0.05^2)); FP32 propagators,
    FP64 reductions; q kept at every K-th slice (K ~ sqrt(3 Ns)) and
    recomputed per segment in the backward sweep, densities and the
    orientation tensor streamed.  One bench step = forward sweep + backward
    sweep with segment recompute + densities + free energy + field update
    (3 Ns contour steps, 2 Ns of them the MDE sweeps proper)."""
    import torch
    import wlc
    x = 4.0
    n, L, nmax = 128, 12, 400
    box = 8.0 * wlc.wlc_radius_of_gyration(x)
    ns = wlc.even_block_lengths((0.3, 0.4, 0.3), nmax)
    K = args.checkpoint or int(round((3 * nmax) ** 0.5))
    inst = wlc.Instance(n, L, nmax, ns, box / n, x * 0.5, (0.5, 0.5, 0.5), (20.0, 20.0, 20.0), nmu=5.0,
                        precision=wlc.WLC_FP32, store_qstar=2, q_checkpoint=K)
    if args.ws_load:
        # learned warm start: the 32^3 network's fields for a 4 Rg box at these
        # parameters (contour/persistence clipped to the training range),
        # tiled 2 x 2 x 2 and resampled to 128^3
        from wlc import warmstart as ws
        net = wlc.WarmStartNet(ws.GRID, 32, seed=1)
        net.set_params(np.load(args.ws_load))
        w = ws.predict_large(net, dict(fa=0.3, fc=0.3, chi=20.0, x=x, box=8.0, noise_seed=77), n, 2)
        net.close()
        start = "learned warm start (32^3 network, 4 Rg box tiled 2x2x2, resampled)"
    else:
        g = 2 * np.pi * np.arange(n) / n
        X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
        gyr = (np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X)).transpose(2, 1, 0).reshape(-1)
        rng = np.random.default_rng(77)
        w = np.stack([gyr, -gyr, 0.5 * gyr]) + rng.normal(0.0, 0.05, size=(3, n ** 3))
        start = "gyroid-like seeded start"
    inst.set_fields(w)
    tuned = None if args.no_autotune else inst.autotune()
    stream = torch.cuda.ExternalStream(inst.stream)
    mp = wlc.mix_params(anderson_depth=5)

    def step():
        inst.MDE_q()
        inst.MDE_qstar()
        inst.density(want_junction=False)
        fe = inst.free_energy()
        err, _ = inst.iterate(mp)
        return fe, err

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(0)
    clk.start()
    l0 = inst.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        fe, err = step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    mde_steps = 2 * nmax * args.steps
    free, total = torch.cuda.mem_get_info()
    line = {"metric": "MDE contour steps/s (128^3, L=12, Ns=400, sqrt(Ns) checkpointing, Maier-Saupe)",
            "value": mde_steps / (ms / 1000.0), "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (%s)" % start,
            "config": {"workload": "ABC triblock 128^3, box 8.0 Rg, L=12 (M=169), Ns=400 (%d/%d/%d), chiN=20, "
                                   "L/lp=4.0, muN=5; q checkpoint every %d slices, recompute per segment; one bench "
                                   "step = one SCFT iteration (%d MDE steps + %d recompute steps)" % (
                                       ns[0], ns[1], ns[2], K, 2 * nmax, nmax - nmax // K),
                       "l2": "inputs larger than L2 (1.4 GB per slice)",
                       "launch_config": tuned},
            "device_memory_used_gb": (total - free) / 1e9, "F": fe, "residual": float(max(err[:3])),
            "gpu_launches": int(inst.launch_count - l0), "clocks": clocks}
    print(json.dumps(line))
    inst.close()


def run_warmstart(args):
    """Learned warm start at 32^3, l <= 6, Ns = 100 over the batched
    sweep's parameter ranges (box 3.5-5.5 Rg): solver-generated converged
    fields (bootstrapped, wlc.warmstart.generate_dataset), network training
    on the device, then cold against warm starts on held-out draws (same
    batches and mixing), and the final free energy of converged warm-started
    draws re-evaluated with FP64 propagators."""
    import torch
    import wlc
    from wlc import warmstart as ws
    t0 = time.perf_counter()
    out = {"metric": "learned warm start: iterations to a residual, warm vs cold (32^3, L=6, Ns=100)"}
    if args.ws_load:
        net = wlc.WarmStartNet(ws.GRID, 32, seed=1)
        net.set_params(np.load(args.ws_load))
        out["network"] = {"loaded": os.path.basename(args.ws_load)}
    else:
        draws, targets, recs = ws.generate_dataset(args.ws_target, seed=1000, tol=args.ws_tol,
                                                   budget_s=args.ws_budget, log=lambda m: print(m, flush=True))
        t_data = time.perf_counter() - t0
        cold = [r for r in recs if r["start"] == "cold"]
        warm = [r for r in recs if r["start"] == "warm"]

        def med(rs):
            v = [r["iterations"] for r in rs if r["iterations"] is not None]
            return float(np.median(v)) if v else None
        out["dataset"] = {"converged_fields": len(draws), "tolerance": args.ws_tol, "seconds": t_data,
                          "cold_draws": len(cold), "cold_converged": sum(r["iterations"] is not None for r in cold),
                          "warm_draws": len(warm), "warm_converged": sum(r["iterations"] is not None for r in warm),
                          "median_iterations_cold": med(cold), "median_iterations_warm": med(warm)}
        print(json.dumps(out["dataset"]), flush=True)
        t1 = time.perf_counter()
        net, hist = ws.train(draws, targets, epochs=args.ws_epochs, lr=args.ws_lr)
        torch.cuda.synchronize()
        out["network"] = {"params": int(net.np), "train_samples": len(draws), "epochs": args.ws_epochs,
                          "lr": args.ws_lr, "seconds": time.perf_counter() - t1,
                          "loss_first_last": [float(hist[0]), float(hist[-1])]}
        if args.ws_save:
            np.save(args.ws_save, net.params())
        print(json.dumps(out["network"]), flush=True)
    test = ws.draw_params(args.ws_test, 777)
    res, summary = ws.evaluate(net, test, tol=args.ws_eval_tol, max_iter=args.ws_eval_iters)
    out["evaluation"] = {"held_out_draws": len(test), "max_iterations": args.ws_eval_iters, "thresholds": summary,
                         "seconds": {k: res[k]["seconds"] for k in ("cold", "warm")},
                         "diverged": {k: sum(r["diverged"] for r in res[k]["results"]) for k in ("cold", "warm")},
                         "median_final_residual": {k: float(np.nanmedian([r["residual"] for r in res[k]["results"]]))
                                                   for k in ("cold", "warm")}}
    # converged warm-started draws: F of the FP32 run against FP64 propagators at the same fields
    checks = []
    for d, r in zip(test, res["warm"]["results"]):
        if r["iterations"] is None or len(checks) >= args.ws_f_checks:
            continue
        vals = {}
        for prec in (wlc.WLC_FP32, wlc.WLC_FP64):
            inst = wlc.Instance(precision=prec, store_qstar=1, **ws.instance_spec(d))
            inst.set_fields(r["fields"])
            inst.MDE_q()
            inst.MDE_qstar()
            dd = inst.density(want_junction=False)
            vals[prec] = (inst.free_energy(), dd["lnQ"])
            inst.close()
        f32, f64 = vals[wlc.WLC_FP32][0], vals[wlc.WLC_FP64][0]
        checks.append({"F_fp32": f32, "F_fp64": f64, "rel": abs(f32 - f64) / abs(f64),
                       "lnQ_fp64": vals[wlc.WLC_FP64][1], "residual": r["residual"]})
    out["evaluation"]["F_fp32_vs_fp64_at_converged_fields"] = checks
    out["seconds_total"] = time.perf_counter() - t0
    print(json.dumps(out))
    net.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--profile", action="store_true", help="small-footprint case for ncu captures")
    ap.add_argument("--converge", action="store_true", help="time-to-converged F instead of steps/s")
    ap.add_argument("--workload", default="single", choices=["single", "batch", "large", "warmstart"])
    ap.add_argument("--ws-target", type=int, default=2000, help="warm start: converged training fields wanted")
    ap.add_argument("--ws-budget", type=float, default=1800.0, help="warm start: data generation seconds at most")
    ap.add_argument("--ws-tol", type=float, default=1e-4, help="warm start: residual of a converged training field")
    ap.add_argument("--ws-test", type=int, default=200, help="warm start: held-out draws")
    ap.add_argument("--ws-epochs", type=int, default=20)
    ap.add_argument("--ws-eval-iters", type=int, default=400)
    ap.add_argument("--ws-eval-tol", type=float, default=2e-6)
    ap.add_argument("--ws-lr", type=float, default=3e-4)
    ap.add_argument("--ws-save", default="", help="warm start: save the trained parameters (.npy)")
    ap.add_argument("--ws-load", default="", help="warm start: load parameters instead of generating and training")
    ap.add_argument("--ws-f-checks", type=int, default=8)
    ap.add_argument("--checkpoint", type=int, default=0, help="large workload: q checkpoint interval")
    ap.add_argument("--count", type=int, default=48, help="instances of the batched workload")
    ap.add_argument("--no-autotune", action="store_true", help="default launch configuration")
    ap.add_argument("--no-fp32", action="store_true", help="fp64 run: skip the FP32 form's line entry")
    ap.add_argument("--launch-config", default="", help="profile case: a_variant,solve_threads[,xy_threads[,xy_variant]]")
    ap.add_argument("--forms", default="fp32_warm,fp64_warm,fp64_cold")
    ap.add_argument("--seeds", default="1,2,3", help="converge: noise seeds of the warm start")
    ap.add_argument("--stall", type=int, default=30, help="converge: FP32 iterations without progress before FP64")
    ap.add_argument("--stored", action="store_true", help="converge: keep every slice (overlapped sweeps)")
    ap.add_argument("--lambda-late", type=float, default=0.0, help="converge: Anderson weight once the residual "
                    "is below --late-below (0: keep --lambda-a)")
    ap.add_argument("--late-below", type=float, default=1e-3)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--switch-tol", type=float, default=1e-5)
    ap.add_argument("--depth", type=int, default=5)
    ap.add_argument("--max-iter", type=int, default=2000)
    ap.add_argument("--budget", type=float, default=900.0, help="wall-time cap per form, seconds")
    ap.add_argument("--history", action="store_true")
    ap.add_argument("--lambda-a", type=float, default=0.1, help="Anderson mixing parameter")
    args = ap.parse_args()
    if args.profile:
        run_profile_case(args)
        return
    if args.converge:
        run_converge(args)
        return
    if args.workload == "batch" and args.impl == "ours":
        run_batch(args)
        return
    if args.workload == "large" and args.impl == "ours":
        run_large(args)
        return
    if args.workload == "warmstart" and args.impl == "ours":
        run_warmstart(args)
        return
    wl = workload(args.precision)
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
