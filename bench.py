"""Benchmark of the split-operator step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload 2d4096|2d1024|1d4096|batch1d|serving|born2d|3d256]
                    [--precision mixed|fp64]

Default workload: the large 2D configuration -- 4096x4096 periodic grid on
[-200,200)^2, double-slit wall (V=10 on |x|<1 except openings of width 2 at
y=+-6) plus seeded U[-0.01,0.01] noise, Gaussian packet k=(2,0), s=10 at
(-60,0), dt=0.01, O4, complex64-mixed.  Synthetic seeded inputs; the
complex128 plain path runs the same steps beside it for the error figures.

A "step" is one O4 time step of the whole grid.  K steps are timed as one
qsg_step(K) call (launches queued back to back on the context stream),
bracketed by CUDA events on that stream.  psi (128 MiB) plus its phase tables
(256 MiB) exceed the 129 MB L2, so no flush is needed between steps.

Multi-GPU: the workload is one grid; the path does not shard (no collective),
so --gpus N runs N independent replicas ("replicas only"), value = total
site-steps over the slowest rank's time.

--impl reference times the reference's CPU path (the oracle: the reference
compiled from its own sources when that build is present, otherwise the C
restatement of the same algorithm) on this host, one core (the reference's
CPU path is single-threaded for one grid), on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from tests.workloads import double_slit_2d, gauss_packet_1d, gauss_packet_2d, gaussian_bumps_2d  # noqa: E402

WORKLOADS = {
    "2d4096": dict(desc="2D 4096x4096 double slit, O4, dt=0.01", dim=2, nx=4096, ny=4096, half=200.0,
                   k=(2.0, 0.0), c=(-60.0, 0.0), s=10.0, dt=0.01, order=4, full_steps=2000),
    "2d1024": dict(desc="2D 1024x1024 16 Gaussian bumps (seed 0), O4, dt=0.02", dim=2, nx=1024, ny=1024,
                   half=100.0, k=(1.5, 0.0), c=(-40.0, 0.0), s=8.0, dt=0.02, order=4, full_steps=1000),
    "1d4096": dict(desc="1D N=4096 barrier 0.5 exp(-x^2/2), O2, dt=0.05", dim=1, n=4096, dt=0.05, order=2,
                   full_steps=2000),
    "batch1d": dict(desc="batched 1D: 2048 instances, N=2^e e~U{10..17} (seed 0), 8 bumps, O2, dt=0.01",
                    dim=0, count=2048, dt=0.01, order=2, full_steps=500),
    "born2d": dict(desc="Born series 2D: 2048x2048 on [-150,150)^2, E=2 (21 points per wavelength), Gaussian "
                        "well 0.3 exp(-r^2/4) with a weak absorbing spot, preconditioned (Vellekoop), order 20 "
                        "updates per Compute, incident along x", dim=-2, nx=2048, ny=2048, half=150.0, en=2.0,
                   order=20, preconditioner=1),
    "3d256": dict(desc="3D 256^3 on [-25.6,25.6)^3, Gaussian packet k=(1.5,-0.5,0.8), s=2 at the origin, "
                       "Gaussian bump 0.8 exp(-|r-c|^2/2) (seed 0), dt=0.01, O4", dim=-3, n=256, half=25.6,
                  dt=0.01, order=4),
    "serving": dict(desc="serving: seeded Poisson arrivals; 70% 1D N log-uniform 2^10..2^18, 30% 2D side "
                         "log-uniform 256..2048 (both rounded to powers of two); steps U{100..5000}; O2/O4 50/50; "
                         "complex64; 120 GB budget", dim=-1),
}


def make_inputs(w):
    if w["dim"] == 1:
        psi, V, dx = gauss_packet_1d(w["n"], -200.0, 200.0, 1.0, -50.0, 10.0, barrier=0.5)
        return psi, V, (dx,)
    h = w["half"]
    psi, dx, dy = gauss_packet_2d(w["nx"], w["ny"], -h, h, -h, h, w["k"][0], w["k"][1], w["c"][0], w["c"][1],
                                  w["s"])
    if w["nx"] == 4096:
        V, _, _ = double_slit_2d(w["nx"], w["ny"], h, seed=0)
    else:
        V = gaussian_bumps_2d(w["nx"], w["ny"], -h, h, -h, h, nbumps=16, seed=0, spread=30.0)
    return psi, V, (dx, dy)


def algorithmic_bytes(w, precision, form="direct"):
    """Minimal-fused-schedule HBM bytes per site-step (psi in and out per pass,
    one V table read per real-space pass): 2D O4 = 6 passes x 2 psi + 3 tables,
    O2 = 2 passes x 2 psi + 1 table; 1D resident = one round trip per call.
    The momentum form's column passes also read and write the stored state
    (4 psi-sized transfers instead of 2)."""
    sc = 8 if precision == "mixed" else 16
    cp = 4 if form == "momentum" else 2
    if w["dim"] == 2:
        return (3 * 2 * sc + 3 * cp * sc + 3 * sc) if w["order"] == 4 else (2 * sc + cp * sc + sc)
    return None


def kernel_bytes_per_site(name, precision, form="direct"):
    sc = 8 if precision == "mixed" else 16
    return {"row_pass": 3 * sc, "col_pass": (4 if form == "momentum" else 2) * sc}.get(name)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # wait for nvidia-smi's first line, then count only the lines that arrive
        # after this point (the timed region)
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5.0:
            time.sleep(0.01)
        self.first = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines[getattr(self, "first", 0):]:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def clocks_over(run_once, device, timed_ms, clk, min_s=1.5):
    """The timed region's clock record, or, when it was too short for the
    sampler (fewer than 3 samples at 200 ms), a record taken over untimed
    repeats of the same work lasting min_s, marked as such."""
    if clk.get("samples", 0) >= 3 or "nvidia-smi unavailable" in clk.get("reasons", []):
        clk["window"] = "the timed region"
        return clk
    cs = ClockSampler(device)
    cs.start()
    t0, reps = time.perf_counter(), 0
    while time.perf_counter() - t0 < min_s:
        run_once()
        reps += 1
    el = time.perf_counter() - t0
    c2 = cs.stop()
    c2["window"] = (f"{reps} untimed repeats of the timed work ({el:.2f} s) right after it: the timed region "
                    f"itself ({timed_ms:.1f} ms) is shorter than the sampler's 200 ms period")
    c2["timed_region_samples"] = clk.get("samples", 0)
    return c2


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(kernel):
    """DRAM bytes per site of one launch of `kernel` from the committed ncu summary, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


SERIAL_NOTE = ("one core: the reference's CPU path for one grid is serial (its CPU_PAR device falls back to "
               "libstdc++'s serial parallel-STL backend without TBB, and its FFT plans are single-threaded)")


def oracle_2d_rows(w, per_step_s, calib_rows=256):
    """Rows of the workload's own grid (its own psi0 and V, full-length rows)
    whose O4 step the oracle finishes in about per_step_s on this host: the full
    grid when it fits, else the largest power-of-two slab around the centre.
    Returns (rows, seconds per full-grid step, measured)."""
    from oracle import oracle as orc
    o = orc.Oracle()
    psi, V, (dx, dy) = make_inputs(w)
    nx = w["nx"]
    r0 = (nx - calib_rows) // 2
    st = orc.Stepper2D(o, psi[r0:r0 + calib_rows], V[r0:r0 + calib_rows], dx, dy, w["dt"], order=w["order"])
    st.step(1)
    t0 = time.perf_counter()
    st.step(1)
    per_row = (time.perf_counter() - t0) / calib_rows
    st.close()
    rows = nx
    while rows > 32 and per_row * rows > per_step_s:
        rows //= 2
    return rows, per_row * nx


def oracle_2d_slab(w, rows):
    """The oracle stepper on `rows` full-length rows of the workload's own inputs."""
    from oracle import oracle as orc
    psi, V, (dx, dy) = make_inputs(w)
    r0 = (w["nx"] - rows) // 2
    return orc.Stepper2D(orc.Oracle(), psi[r0:r0 + rows], V[r0:r0 + rows], dx, dy, w["dt"], order=w["order"])


def cpu_sample(w, budget_s=15.0):
    """Time the oracle on a bounded sample of the workload on this host (1 core)."""
    from oracle import oracle as orc
    if not os.path.exists(orc.ORACLE_SO):
        orc.build()
    o = orc.Oracle()
    kind = "port"
    if w["dim"] == 1:
        psi, V, (dx,) = make_inputs(w)
        st = orc.Stepper1D(o, psi, V, dx, w["dt"], order=w["order"])
        st.step(5)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < budget_s:
            st.step(50)
            n += 50
        el = time.perf_counter() - t0
        st.close()
        return dict(value=w["n"] * n / el, unit="site-steps/s", cores=1, kind=kind,
                    sample=f"{n} steps of the N={w['n']} workload, single thread")
    # 2D: O4 steps of the workload's own grid (a slab of full-length rows of its
    # own inputs only when one full step would not fit the budget)
    ny = w["ny"]
    rows, _ = oracle_2d_rows(w, budget_s * 0.5)
    st = oracle_2d_slab(w, rows)
    n, t0 = 0, time.perf_counter()
    while True:
        st.step(1)
        n += 1
        if time.perf_counter() - t0 > budget_s * 0.5:
            break
    el = time.perf_counter() - t0
    st.close()
    what = f"the full {w['nx']}x{ny} grid" if rows == w["nx"] else f"a {rows}x{ny} slab (full-length rows)"
    return dict(value=rows * ny * n / el, unit="site-steps/s", cores=1, kind=kind,
                sample=f"{n} O4 step(s) of {what} of the workload's own inputs; " + SERIAL_NOTE,
                host_cores=os.cpu_count())


def world_max(x: float, world: int, device: str = "cuda") -> float:
    """The maximum of x over the ranks (the slowest rank's time), or x alone."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units all ranks processed per second of the slowest rank (weak scaling)."""
    return units_per_rank * world / seconds


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def born_inputs(w):
    from tests.workloads import born_potential_2d
    h = w["half"]
    V, _, _ = born_potential_2d(w["nx"], w["ny"], -h, h, -h, h)
    return V


def born_cpu_sample(budget_s, order):
    """The oracle's preconditioned Born series (1 core) on a 640x640 grid of the
    workload's wavelength and potential: site-updates/s."""
    from oracle import oracle as orc
    from tests.workloads import born_potential_2d
    if not os.path.exists(orc.ORACLE_SO):
        orc.build()
    o = orc.Oracle()
    n = 640  # the smallest box of >= 24 wavelengths at this grid spacing, 5 x 2^7 points
    h = 150.0 * n / 2048
    V, _, _ = born_potential_2d(n, n, -h, h, -h, h)
    done, t0 = 0, time.perf_counter()
    while True:
        o.born2d(V, -h, h, -h, h, 2.0, 0.0, order=order, preconditional=True, preconditioner=1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return dict(value=n * n * order * done / el, unit="site-updates/s", cores=1, kind="port",
                sample=f"{done} x (init + one Compute of {order} preconditioned updates) on a {n}x{n} grid with "
                       "the workload's grid spacing and potential, single thread")


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if w["dim"] == -3:
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no 3D evolver (only the 3D "
                          "transform); its 2D/1D step formulas extended to three axes are the oracle's"}), flush=True)
        return
    if w["dim"] == -2:
        cpu = born_cpu_sample(120.0 / max(1, args.steps + args.warmup) * args.steps, 2)
        v = cpu["value"]
        line = {"metric": "site-updates/s", "value": v, "unit": "site-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic", "impl": "reference",
                "config": {"workload": w["desc"], "precision": "fp64"}, "cpu_baseline": cpu,
                "e2e": {"value": v, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    from oracle import oracle as orc
    if not os.path.exists(orc.ORACLE_SO):
        orc.build()
    o = orc.Oracle()
    kind = "port"
    if w["dim"] == 1:
        psi, V, (dx,) = make_inputs(w)
        st = orc.Stepper1D(o, psi, V, dx, w["dt"], order=w["order"])
        st.step(args.warmup)
        t0 = time.perf_counter()
        st.step(args.steps)
        el = time.perf_counter() - t0
        sites, sample = w["n"], f"full N={w['n']} grid, K={args.steps} steps"
    else:
        # each step: one O4 step of the workload's own grid and inputs; a slab of
        # full-length rows of them only when the whole run would not end within
        # a few minutes
        ny = w["ny"]
        per_step_budget = 240.0 / max(1, args.steps + args.warmup)
        rows, full_s = oracle_2d_rows(w, per_step_budget)
        st = oracle_2d_slab(w, rows)
        st.step(args.warmup)
        t0 = time.perf_counter()
        st.step(args.steps)
        el = time.perf_counter() - t0
        sites = rows * ny
        what = f"the full {w['nx']}x{ny} grid" if rows == w["nx"] else f"a {rows}x{ny} slab (full-length rows)"
        sample = f"each step: one O4 step of {what} of the workload's own inputs"
    st.close()
    v = sites * args.steps / el
    line = {"metric": "site-steps/s", "value": v, "unit": "site-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": w["desc"], "precision": "fp64", "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": "site-steps/s", "cores": 1, "kind": kind,
                             "sample": sample + "; " + SERIAL_NOTE, "host_cores": os.cpu_count()},
            "e2e": {"value": v, "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batch_cpu_sample(psis, Vs, dxs, w, threads, budget_s=12.0, steps=20):
    """The oracle on the batch's instances, one instance per host thread at a
    time (instances are independent; the oracle's C calls release the GIL):
    `steps` O2 steps of each instance taken from a shared queue in batch order
    until budget_s has passed."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as orc
    o = orc.Oracle()
    lock = threading.Lock()
    state = {"next": 0, "sites": 0, "instances": 0}
    t0 = time.perf_counter()

    def worker():
        while time.perf_counter() - t0 < budget_s:
            with lock:
                i = state["next"]
                state["next"] += 1
            if i >= len(psis):
                return
            st = orc.Stepper1D(o, psis[i], Vs[i], dxs[i], w["dt"], order=w["order"])
            st.step(steps)
            st.close()
            with lock:
                state["sites"] += psis[i].size * steps
                state["instances"] += 1

    with ThreadPoolExecutor(threads) as ex:
        for f in [ex.submit(worker) for _ in range(threads)]:
            f.result()
    el = time.perf_counter() - t0
    return {"value": state["sites"] / el, "unit": "site-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} O2 steps of each of {state['instances']} instances of the batch (in batch order), "
                      f"one instance per thread at a time, {threads} thread(s)", "host_cores": os.cpu_count()}


def time_batch(q, ctx, psis, Vs, dxs, w, args, local, plans=None):
    """K steps of a freshly built batch in ctx (on `plans` {n: Plan1D} where
    given), timed with events on its stream."""
    import torch
    s = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    b = q.Batch(ctx, psis, Vs, dxs, [w["dt"]] * len(psis), order=w["order"], precision=args.precision)
    for n, p in (plans or {}).items():
        if p.kind == 1:
            b.set_plan(n, p)
    b.step(args.warmup)
    b.sync()
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(s)
    b.step(args.steps)
    h1.record(s)
    h1.synchronize()
    ms = h0.elapsed_time(h1)
    sites = b.sites()
    b.close()
    return {"value": sites * args.steps / (ms / 1e3), "unit": "site-steps/s", "ms_per_step": ms / args.steps}


def run_batch(args, w):
    """The batched 1D configuration: every instance advances K steps per timed call."""
    from tests.workloads import batch_1d
    import tempfile
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    import qusim_gb300 as q
    psis, Vs, dxs = batch_1d(w["count"], seed=rank)
    # no plan cache entries from elsewhere: the batch starts on the default plans
    os.environ["QSG_PLAN_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="qsg_plans_"), "plans.tsv")
    ctx = q.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    b = q.Batch(ctx, psis, Vs, dxs, [w["dt"]] * len(psis), order=w["order"], precision=args.precision)
    tuned, tune_ms = (None, None) if args.no_tune else b.autotune(trial_steps=8)
    sites = b.sites()
    b.step(args.warmup)
    b.sync()
    torch.cuda.synchronize()
    ctx.profile(2)  # launch counts only inside the timed region
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    counts = ctx.profile_read()
    ctx.profile(False)

    def repeat_timed_work():
        b.step(args.steps)
        b.sync()

    clk = clocks_over(repeat_timed_work, local, ms, clk)
    ctx.profile(True)  # per-kernel event times: the same K steps again
    b.step(args.steps)
    b.sync()
    prof = ctx.profile_read()
    ctx.profile(False)
    value = sites * args.steps * world / (ms / 1e3)
    # the same batch with one launch per resident size class instead of the
    # tile-queue launch (QSG_BATCH_QUEUE=0, read when a context is created)
    per_class = None
    if args.precision == "mixed" and not args.no_plain:
        os.environ["QSG_BATCH_QUEUE"] = "0"
        try:
            ctx2 = q.Context(local)
        finally:
            del os.environ["QSG_BATCH_QUEUE"]
        per_class = time_batch(q, ctx2, psis, Vs, dxs, w, args, local, plans=tuned)
        per_class["value"] *= world
        per_class["launch"] = ("one launch per resident size class (QSG_BATCH_QUEUE=0), the same plans; the states "
                               "are bitwise those of the tile-queue launch (tests/test_gpu_parity.py)")
        ctx2.close()
    # the same batch on the default plans
    default_plans = None
    if tuned:
        ctx3 = q.Context(local)
        default_plans = time_batch(q, ctx3, psis, Vs, dxs, w, args, local)
        default_plans["value"] *= world
        ctx3.close()
    # four-step instances (N > one CTA) move 2 HBM round trips of psi plus one
    # V table and one K table entry per site-step (O2): 6 complex elements
    peak, peak_kind = measured_peaks()
    fs_sites = sum(p.size for p in psis if p.size > (8192 if args.precision == "mixed" else 4096))
    cs = 8 if args.precision == "mixed" else 16
    fs_gbs = 6 * cs * fs_sites * args.steps / (ms / 1e3) / 1e9
    fs_roof = {"four_step_sites": fs_sites, "algorithmic_bytes_per_site_step": 6 * cs,
               "achieved_gbs": fs_gbs, "peak": peak, "peak_source": peak_kind, "frac": fs_gbs / peak,
               "note": "four-step bytes over the whole batch time (resident classes run beside them)"}
    acc = None
    if not args.no_plain and args.precision == "mixed":
        # every instance of the batch over the configuration's full step count,
        # complex64 against complex128 (each batched the same way)
        nacc = args.accuracy_steps if args.accuracy_steps is not None else w["full_steps"]
        bm = q.Batch(ctx, psis, Vs, dxs, [w["dt"]] * len(psis), order=w["order"], precision="mixed")
        bp = q.Batch(ctx, psis, Vs, dxs, [w["dt"]] * len(psis), order=w["order"], precision="fp64")
        n0 = [bp.instance(k).norm2() for k in range(len(psis))]
        bm.step(nacc)
        bp.step(nacc)
        errs, drifts = [], []
        for k in range(len(psis)):
            a, r = bm.instance(k).get_psi(), bp.instance(k).get_psi()
            errs.append(float(np.linalg.norm(a - r) / np.linalg.norm(r)))
            drifts.append(abs(bm.instance(k).norm2() - n0[k]))
        bm.close()
        bp.close()
        acc = {"steps": nacc, "instances": len(psis), "rel_l2_vs_fp64_max": max(errs),
               "rel_l2_vs_fp64_median": float(np.median(errs)), "norm_drift_mixed_max": float(max(drifts))}
    # the complex128 path instance by instance (one qsg_step per instance), on
    # the first 256 instances of the batch
    plain = None
    if not args.no_plain and args.precision == "mixed":
        sub = list(range(min(256, len(psis))))
        solo = [q.Instance.create_1d(ctx, psis[i], Vs[i], dxs[i], w["dt"], order=w["order"], precision="fp64")
                for i in sub]
        for s_ in solo:
            s_.step(2)
        solo[0].sync()
        torch.cuda.synchronize()
        psteps = 10
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for s_ in solo:
            s_.step(psteps)
        f1.record(stream)
        f1.synchronize()
        pms = f0.elapsed_time(f1)
        psites = sum(psis[i].size for i in sub)
        plain = {"value": psites * psteps / (pms / 1e3), "unit": "site-steps/s", "steps": psteps,
                 "instances": len(sub), "dtype": "c128", "launch": "one qsg_step per instance"}
        for s_ in solo:
            s_.close()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = batch_cpu_sample(psis, Vs, dxs, w, os.cpu_count() or 1)
        cpu["one_core"] = batch_cpu_sample(psis, Vs, dxs, w, 1)
    if rank == 0:
        line = {"metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c64" if args.precision == "mixed" else "c128", "data": "synthetic",
                "config": {"workload": w["desc"], "precision": args.precision, "sites": sites,
                           "instances": len(psis), "parallelism": f"replicas x{world}",
                           "l2": "2.2 GB of state and tables, larger than L2"},
                "roofline": {"bound": "on-chip", "note": "resident sizes keep psi in shared memory for all "
                             "K steps; four-step sizes make 2 HBM passes per step"},
                "step_roofline": fs_roof, "plain_fp64": plain, "resident_per_class_launches": per_class,
                "plans_1d": {"tuned": {str(k): list(v.as_tuple()) for k, v in (tuned or {}).items()},
                             "tuned_classes_ms_per_step": tune_ms, "default_plans": default_plans,
                             "default": {str(n): list(q.candidate_plans_1d(args.precision, n)[0].as_tuple())
                                         for n in sorted({p.size for p in psis})},
                             "note": "qsg_batch_autotune: each four-step size class timed alone in the batch on "
                                     "every four-step plan of its length (kind, n1, tma), keeping its fastest; "
                                     "default_plans = the same batch on the default plans"},
                "accuracy": acc, "gpu_launches": int(sum(v[0] for v in counts.values())),
                "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()},
                "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)


def born_bytes_per_site(order, precision, needs_old=True):
    """Algorithmic HBM bytes per site of one Compute of `order` updates: the
    first row pass reads dpsi and V and writes the scratch (3 elements); each
    later one reads the scratch, V and (post-updates that need it) dpsi, and
    writes dpsi and the scratch (5); the last reads the scratch, V, dpsi and
    dpsi at the start of the Compute and writes dpsi (5); each column pass
    reads and writes the scratch (2)."""
    cs = 8 if precision == "mixed" else 16
    mid = 5 if needs_old else 3
    row = 3 + (order - 1) * mid + 5
    return cs * (row + 2 * order), cs * row, cs * 2 * order


def run_born(args, w):
    """The Born-series 2D workload: a step is one Compute (``order`` updates)."""
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import qusim_gb300 as q
    V = born_inputs(w)
    nx, ny, h, K = w["nx"], w["ny"], w["half"], w["order"]
    sites = nx * ny
    ctx = q.default_context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    def solver(precision):
        per = q.QuPerturbation2D()
        per.init(V, -h, h, nx, -h, h, ny, w["en"], 0.0, 1.0, 0.0, q.SolverMethod.BornSerise, 1.0, 1.0,
                 q.Options().Gb300().Order(K).Preconditional(True).VellekoopPreconditioner().Precision(precision))
        return per

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    per = solver(args.precision)
    for _ in range(args.warmup):
        per.Compute()
    per.GetDeltaPsiNorm()
    torch.cuda.synchronize()
    ctx.profile(2)
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        per.Compute()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    ms = world_max(e0.elapsed_time(e1), world)
    counts = ctx.profile_read()
    ctx.profile(False)
    ctx.profile(True)
    for _ in range(args.steps):
        per.Compute()
    per.GetDeltaPsiNorm()
    prof = ctx.profile_read()
    ctx.profile(False)
    value = whole_job_rate(sites * K * args.steps, world, ms / 1e3)
    peak, peak_kind = measured_peaks()
    total_b, row_b, col_b = born_bytes_per_site(K, args.precision)
    roof = None
    if "born_row_pass" in prof:
        nl, tot = prof["born_row_pass"]
        avg = tot / nl
        per_launch = row_b / (K + 1) * sites
        ach = per_launch / (avg / 1e3) / 1e9
        tr = profile_traffic(f"born_row_pass_{args.precision}")
        roof = {"bound": "hbm", "kernel": "born_row_pass", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_source": peak_kind, "avg_launch_ms": avg,
                "algorithmic_bytes_per_launch": per_launch, "traffic": (tr * sites) if tr else None,
                "share": tot / sum(v[1] for v in prof.values())}
    step_roof = {"algorithmic_bytes_per_site_update": total_b / K,
                 "achieved_gbs": total_b / K * value / world / 1e9,
                 "frac": total_b / K * value / world / 1e9 / peak}
    # accuracy of the mixed form against the complex128 path, and its speed
    acc = plain = None
    if not args.no_plain and args.precision == "mixed":
        p64 = solver("fp64")
        p64.Compute()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        p64.Compute()
        f1.record(stream)
        f1.synchronize()
        plain = {"value": sites * K / (f0.elapsed_time(f1) / 1e3), "unit": "site-updates/s", "dtype": "c128"}
        m = solver("mixed")
        m.Compute()
        m.Compute()
        a, b = m.GetPsi(), p64.GetPsi()
        cs = [(np.cos(t), np.sin(t)) for t in np.linspace(0, 2 * np.pi, 16, endpoint=False)]
        xa, xb = m.ComputeXSections(cs), p64.ComputeXSections(cs)
        acc = {"computes": 2, "updates": 2 * K, "rel_l2_vs_fp64": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
               "xsection_max_rel_vs_fp64": float(np.max(np.abs(xa - xb) / np.abs(xb))),
               "delta_norm_mixed": m.GetDeltaPsiNorm(), "delta_norm_fp64": p64.GetDeltaPsiNorm()}
        m.close()
        p64.close()
    # end to end through the public API: init (H2D of V from pinned memory),
    # K x (Compute + GetDeltaPsiNorm read back), GetPsi and 16 cross sections
    import torch as _t
    pin_V = _t.from_numpy(np.ascontiguousarray(V).view(np.float64).copy()).pin_memory()
    V_pinned = pin_V.numpy().view(np.complex128).reshape(V.shape)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    e2 = q.QuPerturbation2D()
    e2.init(V_pinned, -h, h, nx, -h, h, ny, w["en"], 0.0, 1.0, 0.0, q.SolverMethod.BornSerise, 1.0, 1.0,
            q.Options().Gb300().Order(K).Preconditional(True).VellekoopPreconditioner().Precision(args.precision))
    for _ in range(args.steps):
        e2.Compute()
        e2.GetDeltaPsiNorm()
    e2.GetPsi()
    xs16 = e2.ComputeXSections([(np.cos(t), np.sin(t)) for t in np.linspace(0, 2 * np.pi, 16, endpoint=False)])
    e2.close()
    el = world_max(time.perf_counter() - t0, world)
    e2e = {"value": whole_job_rate(sites * K * args.steps, world, el), "unit": "site-updates/s",
           "h2d_bytes_per_step": V.nbytes / args.steps, "d2h_bytes_per_step": V.nbytes / args.steps + 16,
           "includes": "init (V upload, tables), K x (Compute + delta-psi norm read back), GetPsi, 16 cross sections",
           "xsection_theta0": float(xs16[0])}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = born_cpu_sample(15.0, 2)
    per.close()
    if rank == 0:
        line = {"metric": "site-updates/s", "value": value, "unit": "site-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c64" if args.precision == "mixed" else "c128", "data": "synthetic",
                "config": {"workload": w["desc"], "precision": args.precision, "sites": sites,
                           "updates_per_step": K, "parallelism": f"replicas x{world}",
                           "l2": "dpsi x2, V and the scratch (128 MiB in complex64) exceed L2"},
                "roofline": roof, "step_roofline": step_roof, "plain_fp64": plain, "accuracy": acc, "e2e": e2e,
                "gpu_launches": int(sum(v[0] for v in counts.values())),
                "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()},
                "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)


def inputs_3d(n, half, seed=0):
    xs = -half + 2 * half / n * np.arange(n)
    X, Y, Z = np.meshgrid(xs, xs, xs, indexing="ij")
    psi = np.exp(1j * (1.5 * X - 0.5 * Y + 0.8 * Z)) * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (4 * 2.0 ** 2))
    c = np.random.default_rng(seed).uniform(-3, 3, size=3)
    V = 0.8 * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / 2.0)
    d = 2 * half / n
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * d ** 3)
    return psi.astype(np.complex128), V, d


def run_3d(args, w):
    """The 3D split-operator: a step is one O4 step of the 256^3 grid."""
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import qusim_gb300 as q
    n, h = w["n"], w["half"]
    psi0, V, d = inputs_3d(n, h)
    sites = psi0.size
    ctx = q.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    inst = q.Instance.create_3d(ctx, psi0, V, d, d, d, w["dt"], order=w["order"], precision=args.precision)
    inst.step(args.warmup)
    inst.sync()
    ctx.profile(2)
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    inst.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    ms = world_max(e0.elapsed_time(e1), world)
    counts = ctx.profile_read()
    ctx.profile(False)
    ctx.profile(True)
    inst.step(args.steps)
    inst.sync()
    prof = ctx.profile_read()
    ctx.profile(False)
    value = whole_job_rate(sites * args.steps, world, ms / 1e3)
    sc = 8 if args.precision == "mixed" else 16
    # O4: 9 line passes of psi in and out, 3 of them also read a V table
    step_b = (9 * 2 + 3) * sc if w["order"] == 4 else (3 * 2 + 1) * sc
    peak, peak_kind = measured_peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    nl, tot = dom[1]
    # x passes: 3 per step, two of them with a V table
    per_launch = (2 * sc + (2 * sc / 3 if dom[0] == "pass3_x" else 0)) * sites
    ach = per_launch / (tot / nl / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": dom[0], "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
            "peak_source": peak_kind, "avg_launch_ms": tot / nl, "algorithmic_bytes_per_launch": per_launch,
            "traffic": None, "share": tot / sum(v[1] for v in prof.values())}
    step_roof = {"algorithmic_bytes_per_site_step": step_b, "achieved_gbs": step_b * value / world / 1e9,
                 "frac": step_b * value / world / 1e9 / peak}
    acc = plain = None
    if not args.no_plain and args.precision == "mixed":
        p64 = q.Instance.create_3d(ctx, psi0, V, d, d, d, w["dt"], order=w["order"], precision="fp64")
        p64.step(2)
        p64.sync()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        p64.step(10)
        f1.record(stream)
        f1.synchronize()
        plain = {"value": sites * 10 / (f0.elapsed_time(f1) / 1e3), "unit": "site-steps/s", "dtype": "c128"}
        m = q.Instance.create_3d(ctx, psi0, V, d, d, d, w["dt"], order=w["order"], precision="mixed")
        p64.close()
        p64 = q.Instance.create_3d(ctx, psi0, V, d, d, d, w["dt"], order=w["order"], precision="fp64")
        nacc = args.accuracy_steps if args.accuracy_steps is not None else 500
        m.step(nacc)
        p64.step(nacc)
        a, b = m.get_psi(), p64.get_psi()
        acc = {"steps": nacc, "rel_l2_vs_fp64": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
               "norm_mixed": m.norm2(), "norm_fp64": p64.norm2()}
        m.close()
        p64.close()
    # end to end: create (H2D psi0 + V from pinned memory), K x (step + Norm2 read back), psi read back
    import torch as _t
    pin_psi = _t.from_numpy(psi0.view(np.float64).copy()).pin_memory()
    pin_V = _t.from_numpy(np.ascontiguousarray(V, dtype=np.float64)).pin_memory()
    out = _t.empty(psi0.size * 2, dtype=_t.float64).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2 = q.Instance.create_3d(ctx, pin_psi.numpy().view(np.complex128).reshape(psi0.shape),
                              pin_V.numpy().reshape(V.shape), d, d, d, w["dt"], order=w["order"],
                              precision=args.precision)
    prev = None
    for _ in range(args.steps):
        e2.step(1)
        t = e2.post_step_norm2()
        if prev is not None:
            e2.get_step_norm2(prev)
        prev = t
    e2.get_step_norm2(prev)
    e2.get_psi(out.numpy().view(np.complex128).reshape(psi0.shape))
    e2.close()
    el = world_max(time.perf_counter() - t0, world)
    e2e = {"value": whole_job_rate(sites * args.steps, world, el), "unit": "site-steps/s",
           "h2d_bytes_per_step": (psi0.nbytes + V.nbytes) / args.steps, "d2h_bytes_per_step": psi0.nbytes / args.steps + 8,
           "includes": "instance creation (H2D psi0+V, tables), K x (qsg_step(1) + Norm2 posted behind the step and "
                       "read while the next step runs), final psi read back"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as orc
        o = orc.Oracle()
        m_ = 64
        ps, Vs, ds = inputs_3d(m_, h * m_ / n)
        o.evolve3d(ps, Vs, ds, ds, ds, w["dt"], 1, order=w["order"])
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < 15.0:
            o.evolve3d(ps, Vs, ds, ds, ds, w["dt"], 2, order=w["order"])
            k += 2
        cpu = {"value": ps.size * k / (time.perf_counter() - t0), "unit": "site-steps/s", "cores": 1, "kind": "port",
               "sample": f"{k} O4 steps (in calls of 2, tables rebuilt per call) of a 64^3 grid with the workload's "
                         "spacing, single thread"}
    inst.close()
    if rank == 0:
        line = {"metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c64" if args.precision == "mixed" else "c128", "data": "synthetic",
                "config": {"workload": w["desc"], "precision": args.precision, "sites": sites,
                           "parallelism": f"replicas x{world}", "l2": "psi + V tables exceed L2"},
                "roofline": roof, "step_roofline": step_roof, "plain_fp64": plain, "accuracy": acc, "e2e": e2e,
                "gpu_launches": int(sum(v[0] for v in counts.values())),
                "kernels": {k_: {"launches": v[0], "ms": v[1]} for k_, v in prof.items()},
                "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)


def serving_inputs(seed=0):
    """A pool of seeded inputs per power-of-two size (4 variants each): a packet
    and an 8-bump potential as in the batched configuration."""
    from tests.workloads import gaussian_bumps_1d, grid
    rng = np.random.default_rng(seed)
    pool = {}
    for e in range(10, 19):
        n = 1 << e
        half = 0.05 * n
        xs, dx = grid(n, -half, half)
        lst = []
        for _ in range(4):
            k0, s0 = rng.uniform(0.5, 3.0), rng.uniform(2.0, 20.0)
            p = np.exp(1j * k0 * xs) * np.exp(-((xs + 0.25 * half) ** 2) / (4 * s0 * s0))
            p /= np.sqrt(np.sum(np.abs(p) ** 2) * dx)
            lst.append((p, gaussian_bumps_1d(xs, 8, rng, -half, half), dx))
        pool[(1, n)] = lst
    for e in range(8, 12):
        side = 1 << e
        h = 0.05 * side
        lst = []
        for v in range(2):
            p, dx, dy = gauss_packet_2d(side, side, -h, h, -h, h, rng.uniform(0.5, 3), 0.0, -0.25 * h, 0.0,
                                        rng.uniform(2, 20))
            V = gaussian_bumps_2d(side, side, -h, h, -h, h, nbumps=8, seed=int(rng.integers(1 << 30)),
                                  spread=0.8 * h)
            lst.append((p, V, dx))
        pool[(2, side)] = lst
    return pool


def serving_fp64_one_at_a_time(q, device, reqs, arrivals):
    """The same request stream run one request at a time in complex128.

    Every request kind (dimension, size, order) is measured once alone in
    complex128 on this GPU: instance creation from a device-sampled spec, a few
    steps (site-steps/s of the kind), the result read back.  Each request's
    service time is then creation + read + its steps at its kind's rate, and
    the stream's arrival times are replayed through a first-in first-out
    single server (one request on the GPU at a time).  Returns the throughput
    and the latency percentiles of that replay."""
    from tests.workloads import grid
    ctx = q.Context(device)
    kinds = sorted({(key, order) for key, _, _, order in reqs})
    rate, fixed = {}, {}
    for (dim, n), order in kinds:
        half = 0.05 * n
        _, dx = grid(n, -half, half)
        sp = q.Spec.make(x0=-half, y0=-half, s=5.0, kx=1.0, cx=-0.25 * half,
                         bumps=[(0.5, 0.0, 0.0, 2.0)])
        sites = n if dim == 1 else n * n
        steps = int(max(4, min(200, 3e8 / sites)))
        t0 = time.perf_counter()
        if dim == 1:
            inst = q.Instance.create_1d_spec(ctx, sp, n, dx, 0.01, order=order, precision="fp64")
        else:
            inst = q.Instance.create_2d_spec(ctx, sp, n, n, dx, dx, 0.01, order=order, precision="fp64")
        inst.sync()
        t1 = time.perf_counter()
        inst.step(2)
        inst.sync()
        t2 = time.perf_counter()
        inst.step(steps)
        inst.sync()
        t3 = time.perf_counter()
        inst.get_psi()
        t4 = time.perf_counter()
        inst.close()
        rate[((dim, n), order)] = sites * steps / (t3 - t2)
        fixed[((dim, n), order)] = (t1 - t0) + (t4 - t3)
    ctx.close()
    free_at, lat, work, busy = 0.0, [], 0.0, 0.0
    for i, (key, _, steps, order) in enumerate(reqs):
        sites = key[1] if key[0] == 1 else key[1] * key[1]
        service = fixed[(key, order)] + sites * steps / rate[(key, order)]
        start = max(arrivals[i], free_at)
        free_at = start + service
        lat.append(free_at - arrivals[i])
        work += sites * steps
        busy += service
    lat = np.array(lat)
    return {"value": work / free_at, "unit": "site-steps/s", "dtype": "c128",
            "busy_value": work / busy, "makespan_s": free_at,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                          "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
            "kinds_measured": len(kinds),
            "method": "each request kind measured alone in complex128 on this GPU (creation + read back + steps at "
                      "the kind's site-steps/s); the stream's arrivals replayed through a FIFO single server with "
                      "those service times"}


def run_serving(args, w):
    """Requests arrive at Poisson times; the server admits them against its HBM
    budget and batches them continuously.  Reports latency percentiles and the
    aggregate site-steps/s from first submit to last completion."""
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    import qusim_gb300 as q
    from tests.workloads import grid
    pool = serving_inputs(seed=rank) if args.serve_inputs == "arrays" else None
    rng = np.random.default_rng(1000 + rank)
    nreq = int(args.serve_rate * args.serve_seconds)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, size=nreq))
    reqs = []
    for i in range(nreq):
        if rng.uniform() < 0.7:
            n = 1 << int(np.clip(np.round(rng.uniform(10, 18)), 10, 18))
            key = (1, n)
        else:
            side = 1 << int(np.clip(np.round(rng.uniform(8, 11)), 8, 11))
            key = (2, side)
        reqs.append((key, int(rng.integers(0, len(pool[key]))) if pool else 0, int(rng.integers(100, 5001)),
                     2 if rng.uniform() < 0.5 else 4))
    srv = q.Server(local, hbm_budget=120 << 30, max_running=256)

    def spec_for(key):
        # a fresh seeded packet and 8 bumps per request, sampled on the device
        dim, n = key
        half = 0.05 * n
        _, dx = grid(n, -half, half)
        if dim == 1:
            bumps = [(rng.uniform(-1, 1), rng.uniform(-half, half), 0.0, rng.uniform(1, 5)) for _ in range(8)]
            sp = q.Spec.make(x0=-half, s=rng.uniform(2, 20), kx=rng.uniform(0.5, 3), cx=-0.25 * half, bumps=bumps)
        else:
            bumps = [(rng.uniform(-1, 1), rng.uniform(-0.8 * half, 0.8 * half), rng.uniform(-0.8 * half, 0.8 * half),
                      rng.uniform(1, 5)) for _ in range(8)]
            sp = q.Spec.make(x0=-half, y0=-half, s=rng.uniform(2, 20), kx=rng.uniform(0.5, 3), cx=-0.25 * half,
                             bumps=bumps)
        return sp, dx

    def submit(key, var, steps, order):
        dim, n = key
        shape = (n,) if dim == 1 else (n, n)
        if args.serve_inputs == "spec":
            sp, dx = spec_for(key)
            return srv.submit_spec(sp, shape, dx, 0.01, steps, order=order, precision="mixed", dy=dx)
        p, V, dx = pool[key][var]
        return srv.submit(p, V, dx, 0.01, steps, order=order, precision="mixed", dy=dx)

    # warm-up: one small request of each kind, so module loading is not in the latencies
    for key in [(1, 1024), (1, 65536), (2, 256)]:
        rid = submit(key, 0, 10, 2)
        srv.wait(rid, 120)
        srv.take(rid)
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    ids = []
    site_steps = 0
    for i, (key, var, steps, order) in enumerate(reqs):
        now = time.perf_counter() - t0
        if arrivals[i] > now:
            time.sleep(arrivals[i] - now)
        ids.append(submit(key, var, steps, order))
        site_steps += (key[1] if key[0] == 1 else key[1] * key[1]) * steps
    lats = []
    for rid in ids:
        srv.wait(rid, 3600)
        lats.append(srv.take(rid)[1])
    t_end = time.perf_counter() - t0
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    lats = np.array(lats)
    solo = None
    if rank == 0 and not args.no_plain:
        solo = serving_fp64_one_at_a_time(q, local, reqs, arrivals)
    if rank == 0:
        value = site_steps * world / t_end
        line = {"metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
                "steps": nreq, "warmup": 3, "ms_per_step": 1e3 * t_end / max(1, nreq),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
                "data": "synthetic",
                "config": {"workload": w["desc"], "rate_per_s": args.serve_rate, "seconds": args.serve_seconds,
                           "requests": nreq, "budget_bytes": 120 << 30, "parallelism": f"replicas x{world}",
                           "inputs": ("packet-plus-bumps specs sampled on the device, one seeded spec per request"
                                      if args.serve_inputs == "spec" else "host arrays from a seeded pool"),
                           "l2": "requests' state far larger than L2"},
                "latency_s": {"p50": float(np.percentile(lats, 50)), "p90": float(np.percentile(lats, 90)),
                              "p99": float(np.percentile(lats, 99)), "max": float(lats.max())},
                "offered_site_steps_per_s": site_steps / max(arrivals[-1], 1e-9),
                "makespan_s": t_end, "peak_device_bytes": st["peak_device_bytes"],
                "completed": st["completed"], "failed": st["failed"], "clocks": clk,
                "admitted_mid_flight": st["admitted_mid_flight"], "max_in_flight": st["max_in_flight"],
                "fp64_one_at_a_time": solo,
                "note": "a 'step' here is one request; ms_per_step = makespan / requests"}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="2d4096", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--form", default="momentum", choices=["momentum", "direct"],
                    help="2D complex64: state in momentum space with potential increments (default), or direct")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the fp64 comparison runs")
    ap.add_argument("--accuracy-steps", type=int, default=None,
                    help="steps of the mixed-vs-fp64 accuracy run (default: the configuration's own count)")
    ap.add_argument("--no-tune", action="store_true", help="use the default plan instead of autotuning")
    ap.add_argument("--plan", default=None,
                    help="2D plan g,row_e,row_nt,col_e,col_w[,row_kind] for the timed precision (no autotuning)")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serving: requests per second")
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="serving: length of the arrival stream")
    ap.add_argument("--serve-inputs", default="spec", choices=["spec", "arrays"],
                    help="serving: psi0 / V as device-sampled specs or as host arrays")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args, w)
    if w["dim"] == 0:
        return run_batch(args, w)
    if w["dim"] == -1:
        return run_serving(args, w)
    if w["dim"] == -2:
        return run_born(args, w)
    if w["dim"] == -3:
        return run_3d(args, w)

    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import qusim_gb300 as q

    psi0, V, d = make_inputs(w)
    sites = psi0.size
    ctx = q.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    form = args.form if (w["dim"] == 2 and args.precision == "mixed") else "direct"
    other = {"momentum": "direct", "direct": "momentum"}[form]

    def create(precision, frm=None):
        if w["dim"] == 1:
            return q.Instance.create_1d(ctx, psi0, V, d[0], w["dt"], order=w["order"], precision=precision)
        i = q.Instance.create_2d(ctx, psi0, V, d[0], d[1], w["dt"], order=w["order"], precision=precision)
        if precision == "mixed":
            i.form = frm or form
        return i

    tuned = {}

    def tuned_instance(precision, frm=None):
        i = create(precision, frm)
        if w["dim"] == 2 and args.plan and precision == args.precision:
            p = [int(v) for v in args.plan.split(",")]
            i.set_plan(p)
            tuned[precision] = {"plan": list(i.plan().as_tuple()), "trial_ms_per_step": None}
        elif w["dim"] == 2 and not args.no_tune:
            if precision not in tuned:
                p, ms_tr = i.autotune(trial_steps=3, persist=True)
                tuned[precision] = {"plan": list(p.as_tuple()), "trial_ms_per_step": ms_tr}
            else:
                i.set_plan(tuned[precision]["plan"])
        return i

    inst = tuned_instance(args.precision)
    inst.step(args.warmup)
    inst.sync()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # timed region: launch counts only (per-launch events would add gaps
    # between the launches, ~20% of a step at 1024^2)
    ctx.profile(2)
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        inst.step(args.steps)
        e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    ms = e0.elapsed_time(e1)
    counts = ctx.profile_read()
    ctx.profile(False)

    def repeat_timed_work():
        inst.step(args.steps)
        inst.sync()

    clk = clocks_over(repeat_timed_work, local, ms, clk)
    # per-kernel CUDA-event times for the roofline: the same K steps again,
    # every launch bracketed by events on the context stream
    ctx.profile(True)
    inst.step(args.steps)
    inst.sync()
    prof = ctx.profile_read()
    ctx.profile(False)
    ms = world_max(ms, world)
    value = whole_job_rate(sites * args.steps, world, ms / 1e3)

    # dominant kernel and its roofline
    peak, peak_kind = measured_peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else None
    roof = None
    if dom:
        name, (nl, tot) = dom
        bps = kernel_bytes_per_site(name, args.precision, form)
        avg_ms = tot / nl
        if bps:
            ach = bps * sites / (avg_ms / 1e3) / 1e9
            tr = profile_traffic(f"{name}_{args.precision}" + ("_momentum" if form == "momentum" and name == "col_pass"
                                                               else ""))
            roof = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak, "peak_source": peak_kind, "avg_launch_ms": avg_ms,
                    "algorithmic_bytes_per_launch": bps * sites,
                    "traffic": (tr * sites) if tr else None,
                    "share": tot / sum(v[1] for v in prof.values())}
        else:
            roof = {"bound": "fp64" if args.precision == "fp64" else "on-chip", "kernel": name,
                    "avg_launch_ms": avg_ms, "achieved": None, "peak": peak, "unit": "GB/s", "frac": None,
                    "traffic": None}
    launches = int(sum(v[0] for v in counts.values()))
    # the minimal fused schedule's bytes (the same for both forms) give `frac`;
    # the momentum form's own traffic (its column passes also read and write the
    # stored state) is reported beside it
    ab = algorithmic_bytes(w, args.precision)
    fb = algorithmic_bytes(w, args.precision, form)
    step_roof = {"algorithmic_bytes_per_site_step": ab, "achieved_gbs": ab * value / world / 1e9,
                 "frac": ab * value / world / 1e9 / peak, "form": form,
                 "form_bytes_per_site_step": fb, "form_gbs": fb * value / world / 1e9,
                 "form_frac": fb * value / world / 1e9 / peak} if ab else None

    # the fp64 path on the same workload (site-steps/s), and the accuracy of the
    # mixed form against it over the configuration's full step count
    acc = None
    plain = None
    if not args.no_plain and args.precision == "mixed":
        ref = tuned_instance("fp64")
        ref.step(args.warmup)
        ref.sync()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        psteps = max(1, min(args.steps, 20))
        with torch.cuda.stream(stream):
            f0.record(stream)
            ref.step(psteps)
            f1.record(stream)
        f1.synchronize()
        pms = f0.elapsed_time(f1)
        plain = {"value": sites * psteps / (pms / 1e3), "unit": "site-steps/s", "steps": psteps,
                 "dtype": "c128", "plan": tuned.get("fp64", {}).get("plan")}
        ref.close()
        nacc = args.accuracy_steps if args.accuracy_steps is not None else w["full_steps"]
        a_m, a_p = tuned_instance("mixed"), tuned_instance("fp64")
        # 2D: the other complex64 form beside it, against the same complex128 run
        a_o = tuned_instance("mixed", other) if w["dim"] == 2 else None
        k0, p0 = a_p.energies()
        n0 = a_p.norm2()
        chunk = 250
        done = 0
        while done < nacc:
            c = min(chunk, nacc - done)
            a_m.step(c)
            a_p.step(c)
            if a_o is not None:
                a_o.step(c)
            done += c
        a, b = a_m.get_psi(), a_p.get_psi()
        km, pm = a_m.energies()
        kr, pr = a_p.energies()
        acc = {"steps": nacc, "form": form, "rel_l2_vs_fp64": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
               "norm_drift_mixed": float(a_m.norm2() - n0), "norm_drift_fp64": float(a_p.norm2() - n0),
               "energy_drift_mixed": float((km + pm) - (k0 + p0)),
               "energy_drift_fp64": float((kr + pr) - (k0 + p0)),
               "energy_mixed_minus_fp64": float((km + pm) - (kr + pr)), "energy_start": float(k0 + p0)}
        if a_o is not None:
            o = a_o.get_psi()
            ko, po = a_o.energies()
            acc["other_form"] = {"form": other, "rel_l2_vs_fp64": float(np.linalg.norm(o - b) / np.linalg.norm(b)),
                                 "norm_drift_mixed": float(a_o.norm2() - n0),
                                 "energy_mixed_minus_fp64": float((ko + po) - (kr + pr))}
            a_o.close()
        a_m.close()
        a_p.close()

    # 2D complex64: the other form's speed on the same plan (same event timing)
    other_speed = None
    if w["dim"] == 2 and args.precision == "mixed" and not args.no_plain:
        io = create("mixed", other)
        io.set_plan(inst.plan())
        io.step(args.warmup)
        io.sync()
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            g0.record(stream)
            io.step(args.steps)
            g1.record(stream)
        g1.synchronize()
        oms = g0.elapsed_time(g1)
        ov = sites * args.steps / (oms / 1e3)
        other_speed = {"form": other, "value": ov, "unit": "site-steps/s", "ms_per_step": oms / args.steps,
                       "step_roofline_frac": algorithmic_bytes(w, "mixed") * ov / 1e9 / peak,
                       "form_bytes_per_site_step": algorithmic_bytes(w, "mixed", other)}
        io.close()

    # end to end through the public API: H2D of psi0 and V from pinned memory,
    # K x (step + the step's Norm2 read back), final psi read back
    import torch as _t
    pin_psi = _t.from_numpy(psi0.view(np.float64).copy()).pin_memory()
    pin_V = _t.from_numpy(np.ascontiguousarray(V, dtype=np.float64)).pin_memory()
    out = _t.empty(psi0.size * 2, dtype=_t.float64).pin_memory()
    psi_pinned = pin_psi.numpy().view(np.complex128).reshape(psi0.shape)
    V_pinned = pin_V.numpy().reshape(V.shape)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    if w["dim"] == 1:
        e2 = q.Instance.create_1d(ctx, psi_pinned, V_pinned, d[0], w["dt"], order=w["order"],
                                  precision=args.precision)
    else:
        # a new instance picks up the plan tuned above (the context remembers it)
        e2 = q.Instance.create_2d(ctx, psi_pinned, V_pinned, d[0], d[1], w["dt"], order=w["order"],
                                  precision=args.precision)
        if args.precision == "mixed":
            e2.form = form
    # each step's Norm2 is posted behind the step and read while the next step runs
    norms = []
    prev = None
    for _ in range(args.steps):
        e2.step(1)
        t = e2.post_step_norm2()
        if prev is not None:
            norms.append(e2.get_step_norm2(prev))
        prev = t
    norms.append(e2.get_step_norm2(prev))
    e2.get_psi(out.numpy().view(np.complex128).reshape(psi0.shape))
    final_norm = e2.norm2()
    e2.close()
    el = time.perf_counter() - t0
    el = world_max(el, world)
    e2e = {"value": whole_job_rate(sites * args.steps, world, el), "unit": "site-steps/s",
           "h2d_bytes_per_step": (psi0.nbytes + V.nbytes) / args.steps,
           "d2h_bytes_per_step": psi0.nbytes / args.steps + 8,
           "includes": "instance creation (H2D psi0+V, phase tables), K x (qsg_step(1) + the step's Norm2 "
                       "read back: posted behind the step (qsg_step_norm2_post, summed by the step itself in 2D and in 1D one-CTA instances) "
                       "and read on the host while the next step runs), final psi read back",
           "norm_first_step": norms[0] if norms else None, "norm_last_step": norms[-1] if norms else None,
           "norm2_of_final_psi": final_norm}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(w)

    if rank == 0:
        line = {"metric": "site-steps/s", "value": value, "unit": "site-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c64" if args.precision == "mixed" else "c128", "data": "synthetic",
                "config": {"workload": w["desc"], "precision": args.precision, "form": form, "sites": sites,
                           "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (no flush)"},
                "roofline": roof, "step_roofline": step_roof, "accuracy": acc, "plain_fp64": plain,
                "other_form": other_speed, "plan": tuned.get(args.precision),
                "e2e": e2e, "gpu_launches": launches, "kernels": {k: {"launches": v[0], "ms": v[1]}
                                                                  for k, v in prof.items()},
                "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
