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


def run_converge(args):
    """Time-to-converged F at the bench workload: the SCFT loop (propagators,
    densities, free energy, field update on the device) from the same seeded
    cold start until every block residual is <= tol, for each form:
      fp64       plain FP64 propagators throughout (the drop-in);
      fp32sched  FP32 propagators until the residual falls below
                 --switch-tol, then FP64 to the end (same fields and
                 mixing history);
      fp32       FP32 propagators throughout (reports where FP32 stalls).
    FP64 Q, F, residuals and the Anderson least squares in every form.
    Wall time includes everything; capped by --budget seconds per form."""
    import torch
    import wlc
    wl = workload("fp64")
    nr = wl["n"] ** 3
    rng = np.random.default_rng(2024)
    w0 = rng.normal(0.0, wl["w_sigma"], size=(3, nr))
    if args.seed_kind == "lamellar":
        # lamellar start: A and C stripes in antiphase along x, B between them,
        # amplitude 1.0, plus seeded N(0, 0.1^2) noise
        n = wl["n"]
        x = (np.arange(nr) % n) / n
        c1, c2 = np.cos(2 * np.pi * x), np.cos(4 * np.pi * x)
        w0 = np.stack([c1, c2, -c1]) + rng.normal(0.0, 0.1, size=(3, nr))
    if args.init_w:  # restart from saved fields (the reference's readW restart)
        w0 = np.load(args.init_w)
    mp = wlc.mix_params(anderson_depth=args.depth, num_simple=20, lambda_anderson=args.lambda_a, tol=args.tol,
                        min_iter=20, relax_iter=0)
    out = {"metric": "time-to-converged F (64^3, L=10, Ns=200, ABC; residual <= %g)" % args.tol,
           "mixing": {"anderson_depth": args.depth, "num_simple": 20, "lambda_simple": 0.1,
                      "lambda_anderson": args.lambda_a, "ramp": args.ramp}, "forms": {}}
    for form in args.forms.split(","):
        prec = wlc.WLC_FP64 if form == "fp64" else wlc.WLC_FP32
        inst = wlc.Instance(wl["n"], wl["L"], wl["nmax"], wl["ns"], wl["dx"], wl["loa"], wl["kappa"], wl["chi"],
                            precision=prec)
        inst.set_fields(w0)
        mp.lambda_anderson = args.lambda_a
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hist, switched, n, conv = [], None, 0, False
        t_switch = None
        while not conv and n < args.max_iter and time.perf_counter() - t0 < args.budget:
            if args.stop_at > 0 and hist and max(hist[-1][3:6]) < args.stop_at and n > 20:
                break
            n += 1
            if args.ramp and n > 20:  # lambda_A = max(lambda_a, 1 - 0.9^(n - 20))
                mp.lambda_anderson = max(args.lambda_a, 1.0 - 0.9 ** (n - 20))
            inst.MDE_q()
            inst.MDE_qstar()
            d = inst.density(want_junction=False)
            fe = inst.free_energy()
            err, conv = inst.iterate(mp)
            hist.append([n, fe, d["lnQ"]] + [float(e) for e in err])
            if form == "fp32sched" and switched is None and max(err[:3]) < args.switch_tol and n > 20:
                inst.set_precision(wlc.WLC_FP64)
                switched = n
                t_switch = time.perf_counter() - t0
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        if args.save_w:
            np.save(args.save_w, inst.get_fields())
        fp32_err = None
        if prec == wlc.WLC_FP32 and switched is None:
            # the FP32 form's error at its final fields: the same fields
            # evaluated by the FP64 propagators
            w_fin = inst.get_fields()
            vals = {}
            for pr in (wlc.WLC_FP32, wlc.WLC_FP64):
                inst.set_precision(pr)
                inst.set_fields(w_fin)
                inst.MDE_q()
                inst.MDE_qstar()
                dd = inst.density(want_junction=False)
                vals[pr] = (dd["lnQ"], inst.free_energy(), dd["phi"])
            a32, a64 = vals[wlc.WLC_FP32], vals[wlc.WLC_FP64]
            fp32_err = {"lnQ_abs": abs(a32[0] - a64[0]), "F_rel": abs(a32[1] - a64[1]) / abs(a64[1]),
                        "phi_max_rel": float(np.abs(a32[2] - a64[2]).max() / np.abs(a64[2]).max())}
        out["forms"][form] = {"converged": bool(conv), "iterations": n, "seconds": secs, "F": hist[-1][1],
                              "fp32_error_vs_fp64": fp32_err,
                              "lnQ": hist[-1][2], "residual": max(hist[-1][3:6]), "incompressibility": hist[-1][6],
                              "switched_at": switched, "switch_seconds": t_switch,
                              "s_per_iteration": secs / max(1, n)}
        if args.history:
            out["forms"][form]["history"] = hist
        inst.close()
        print(json.dumps({"form": form, **{k: v for k, v in out["forms"][form].items() if k != "history"}}),
              flush=True)
    f = out["forms"]
    if "fp64" in f:
        for k, v in f.items():
            if k != "fp64":
                v["F_rel_err_vs_fp64"] = abs(v["F"] - f["fp64"]["F"]) / abs(f["fp64"]["F"])
                v["speedup_vs_fp64"] = f["fp64"]["seconds"] / v["seconds"]
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
    g = 2 * np.pi * np.arange(n) / n
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    gyr = (np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X)).transpose(2, 1, 0).reshape(-1)
    rng = np.random.default_rng(77)
    w = np.stack([gyr, -gyr, 0.5 * gyr]) + rng.normal(0.0, 0.05, size=(3, n ** 3))
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
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (gyroid-like seeded start)",
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


WS_G, WS_NMAX, WS_L = 32, 100, 6


def ws_draws(count, seed):
    """Instance parameters of the warm-start data set (the batched sweep's
    ranges): fA, fC ~ U(0.2, 0.4), chiN ~ U(12, 24), L/lp ~ U(0.5, 3.0),
    box 4.0 Rg; and the 16^3 noise seed of each instance."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        out.append(dict(fa=rng.uniform(0.2, 0.4), fc=rng.uniform(0.2, 0.4), chi=rng.uniform(12.0, 24.0),
                        x=rng.uniform(0.5, 3.0), noise_seed=int(rng.integers(1 << 31))))
    return out


def ws_noise(seed):
    """16^3 N(0, 1) noise, nearest-upsampled to the 32^3 grid."""
    xi = np.random.default_rng(seed).normal(size=(16, 16, 16))  # [z][y][x]
    return xi.repeat(2, 0).repeat(2, 1).repeat(2, 2).reshape(-1)


def ws_spec(d):
    import wlc
    box = 4.0 * wlc.wlc_radius_of_gyration(d["x"])
    return dict(n=WS_G, lmax=WS_L, nmax=WS_NMAX, ns=wlc.even_block_lengths((d["fa"], 1 - d["fa"] - d["fc"], d["fc"]),
                                                                          WS_NMAX),
                dx=box / WS_G, loa=d["x"] * 0.5, kappa=(0.5, 0.5, 0.5), chi=(d["chi"],) * 3)


def ws_input(d):
    """network input (6, G^3): the noise field and the five parameters
    (scaled to about [-1, 1]) as constant fields"""
    import wlc
    box = 4.0 * wlc.wlc_radius_of_gyration(d["x"])
    par = [(d["fa"] - 0.3) / 0.1, (d["fc"] - 0.3) / 0.1, (d["chi"] - 18.0) / 6.0, (d["x"] - 1.75) / 1.25,
           box - 1.0]
    P = WS_G ** 3
    return np.concatenate([ws_noise(d["noise_seed"])[None, :], np.repeat(np.array(par)[:, None], P, axis=1)])


def ws_cold(d):
    xi = ws_noise(d["noise_seed"])
    return 0.3 * np.stack([xi, -xi, np.zeros_like(xi)])


def ws_solve(draws, w0s, iters, tol=0.0):
    """SCFT of all draws together (one batch, FP32 propagators, field update
    on the device) from the given fields; returns final fields and the
    per-iteration max block residual of every instance."""
    import wlc
    b = wlc.Batch([ws_spec(d) for d in draws])
    for inst, w0 in zip(b.instances, w0s):
        inst.set_fields(w0)
    b.autotune()
    mp = wlc.mix_params(anderson_depth=5)
    res = np.full((len(draws), iters), np.nan)
    fe = np.full((len(draws), iters), np.nan)
    bad = np.zeros(len(draws), dtype=bool)  # iteration diverged (non-finite density): frozen
    for it in range(iters):
        b.propagate()
        for j, inst in enumerate(b.instances):
            if bad[j]:
                continue
            try:
                inst.density(want_junction=False)
                fe[j, it] = inst.free_energy()
                err, conv = inst.iterate(mp)
                res[j, it] = max(err[:3])
            except wlc.WlcError:
                bad[j] = True
        if tol > 0 and (res[~bad, it] < tol).all():
            res, fe = res[:, :it + 1], fe[:, :it + 1]
            break
    ws = [None if bad[j] else inst.get_fields() for j, inst in enumerate(b.instances)]
    b.close()
    return ws, res, fe


def run_warmstart(args):
    """Learned warm start: solver-generated training fields (32^3, l <= 6,
    Ns = 100, the batched sweep's parameter ranges, fields after
    --ws-iters iterations from the cold start), network training on the
    device, then warm vs cold starts on held-out draws."""
    import torch
    import wlc
    t0 = time.perf_counter()
    ntr, nte = args.ws_train, args.ws_test
    draws = ws_draws(ntr + nte, 11)
    train, test = draws[:ntr], draws[ntr:]
    # training data: the solver's fields after ws_iters iterations
    targets, kept = [], []
    chunk = 64
    for c0 in range(0, ntr, chunk):
        part = train[c0:c0 + chunk]
        ws, _, _ = ws_solve(part, [ws_cold(d) for d in part], args.ws_iters)
        for d, w in zip(part, ws):
            if w is None or not np.isfinite(w).all():
                continue
            targets.append((w - w.mean(axis=1, keepdims=True)) / d["chi"])
            kept.append(d)
    n_diverged_train = ntr - len(kept)
    train = kept
    t_data = time.perf_counter() - t0
    X = np.stack([ws_input(d) for d in train]).astype(np.float32)
    T = np.stack(targets).astype(np.float32)
    net = wlc.WarmStartNet(WS_G, 32, seed=1)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    hist = net.train(X, T, batch=8, epochs=args.ws_epochs, lr=args.ws_lr)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    # held-out draws: cold start vs the network's fields
    Xte = np.stack([ws_input(d) for d in test]).astype(np.float32)
    t2 = time.perf_counter()
    warm0 = [net.forward(x).astype(np.float64) * d["chi"] for x, d in zip(Xte, test)]
    t_pred = time.perf_counter() - t2
    wc, res_c, fe_c = ws_solve(test, [ws_cold(d) for d in test], args.ws_eval_iters)
    # held-out error of the network against the solver's fields after as many iterations
    ok = [j for j, w in enumerate(wc) if w is not None and np.isfinite(w).all()]
    tt = {j: (wc[j] - wc[j].mean(axis=1, keepdims=True)) / test[j]["chi"] for j in ok}
    test_mse = float(np.mean([np.mean((net.forward(Xte[j]) - tt[j]) ** 2) for j in ok]))
    test_var = float(np.mean([np.mean(tt[j] ** 2) for j in ok]))
    _, res_w, fe_w = ws_solve(test, warm0, args.ws_eval_iters)
    both_ok = [j for j in range(len(test)) if np.isfinite(res_c[j, -1]) and np.isfinite(res_w[j, -1])]
    n_div_cold = int(sum(not np.isfinite(res_c[j, -1]) for j in range(len(test))))
    n_div_warm = int(sum(not np.isfinite(res_w[j, -1]) for j in range(len(test))))
    res_c, res_w, fe_c, fe_w = res_c[both_ok], res_w[both_ok], fe_c[both_ok], fe_w[both_ok]

    def first_below(res, thr):
        out = []
        for r in res:
            k = np.nonzero(r < thr)[0]
            out.append(int(k[0]) + 1 if k.size else None)
        return out

    summary = {}
    for thr in (1e-1, 3e-2, 1e-2, 3e-3, 1e-3):
        c, w = first_below(res_c, thr), first_below(res_w, thr)
        both = [(a, b) for a, b in zip(c, w) if a is not None and b is not None]
        summary["%g" % thr] = {"cold_reached": sum(a is not None for a in c), "warm_reached": sum(b is not None for b in w),
                               "median_cold_iters": float(np.median([a for a, _ in both])) if both else None,
                               "median_warm_iters": float(np.median([b for _, b in both])) if both else None}
    line = {"metric": "learned warm start: iterations to a residual, warm vs cold (32^3, L=6, Ns=100)",
            "train_instances": len(train), "train_diverged": n_diverged_train, "test_instances": nte,
            "test_diverged": {"cold": n_div_cold, "warm": n_div_warm}, "data_iterations": args.ws_iters,
            "params": int(net.np), "epochs": args.ws_epochs, "lr": args.ws_lr,
            "train_loss_first_last": [float(hist[0]), float(hist[-1])], "train_loss": [float(v) for v in hist],
            "test_mse": test_mse, "test_target_mean_square": test_var,
            "seconds": {"data": t_data, "train": t_train, "predict_all": t_pred},
            "eval_iterations": args.ws_eval_iters, "thresholds": summary,
            "median_final_residual": {"cold": float(np.median(res_c[:, -1])), "warm": float(np.median(res_w[:, -1]))},
            "median_residual_at_50": {"cold": float(np.median(res_c[:, min(49, res_c.shape[1] - 1)])),
                                      "warm": float(np.median(res_w[:, min(49, res_w.shape[1] - 1)]))},
            "median_abs_F_diff_final": float(np.median(np.abs(fe_c[:, -1] - fe_w[:, -1])))}
    print(json.dumps(line))
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
    ap.add_argument("--ws-train", type=int, default=128)
    ap.add_argument("--ws-test", type=int, default=32)
    ap.add_argument("--ws-iters", type=int, default=250)
    ap.add_argument("--ws-epochs", type=int, default=40)
    ap.add_argument("--ws-eval-iters", type=int, default=250)
    ap.add_argument("--ws-lr", type=float, default=1e-4)
    ap.add_argument("--checkpoint", type=int, default=0, help="large workload: q checkpoint interval")
    ap.add_argument("--count", type=int, default=48, help="instances of the batched workload")
    ap.add_argument("--no-autotune", action="store_true", help="default launch configuration")
    ap.add_argument("--no-fp32", action="store_true", help="fp64 run: skip the FP32 form's line entry")
    ap.add_argument("--launch-config", default="", help="profile case: a_variant,solve_threads[,xy_threads[,xy_variant]]")
    ap.add_argument("--forms", default="fp32sched,fp64")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--switch-tol", type=float, default=1e-4)
    ap.add_argument("--depth", type=int, default=5)
    ap.add_argument("--max-iter", type=int, default=2000)
    ap.add_argument("--budget", type=float, default=900.0, help="wall-time cap per form, seconds")
    ap.add_argument("--history", action="store_true")
    ap.add_argument("--lambda-a", type=float, default=0.1, help="Anderson mixing parameter")
    ap.add_argument("--init-w", default="", help="start from fields saved with --save-w (.npy)")
    ap.add_argument("--seed-kind", default="random", choices=["random", "lamellar"])
    ap.add_argument("--save-w", default="", help="save the final fields (.npy)")
    ap.add_argument("--stop-at", type=float, default=0.0, help="stop once the residual is below this")
    ap.add_argument("--ramp", action="store_true", help="ramp lambda_A towards 1 after the simple phase")
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
