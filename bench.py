#!/usr/bin/env python3
"""Element-updates/s of DynELA's explicit step on GB300 (libdnlgpu, FP64).

Workload (default): the 3D Taylor impact bar of ElHex8n3D -- a 40x40 cross-section grid clipped
to the radius, 400 layers (505,600 elements, 539,345 nodes), copper J2 material
(A 90 MPa, B 292 MPa, n 0.31), impact speed 227 m/s, Chung-Hulbert explicit integration with the
Pulse critical time step.  A step is one full explicit increment: element pass (kinematics, polar
decomposition, radial return, forces), CSR assembly, nodal update and the time-step logic
(Pulse power iteration every 10 increments).  An element-update is one element through one step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config hex|axi]

The timed window starts at t = 10 us of the 80 us impact (reached untimed), when the elastic
wave has crossed the bar and the impact end is plastic.
`value` is measured with device-resident state (CUDA events on the library's stream);
`e2e` goes through the C ABI with page-locked host buffers: each step uploads the nodal state the
caller owns (coordinates, delta_disp, velocity, acceleration, displacement), advances one step and
reads it back in one dnl_step_host call (v, a and disp travel beside the element pass), over the
same increments as `value` (a second handle brought to the same state).  The reference arm (--impl reference) times the oracle's CPU restatement of the
reference (oracle/dnl_oracle.c, OpenMP on all host cores) on a bounded slice of the same bar.
Multi-GPU: independent replicas, one per rank (the explicit step has no cross-replica exchange).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from redynela_gb300 import meshes  # noqa: E402

# dram__bytes_read.sum + dram__bytes_write.sum of one k_elem<ElHex8n3D> launch per element,
# measured by ncu on the 126,400-element bar's mid-run window (308.85 MB); scaled by the elements
# of the workload
ELEM_TRAFFIC_BYTES_PER_ELEMENT = 308.85e6 / 126400

# FP64 thread-instructions of one k_elem<ElHex8n3D> launch per Gauss point in the timed window of
# the 505,600-element bar (t = 10 us, increment 1,553), from ncu's
# sm__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum counters of that launch
# (2,145,155,470 / 573,527,287 / 914,639,971 over the launch's 4,044,800 points, one counter per
# capture, each a one-pass capture)
HEX_FP64_INSTR_PER_POINT = {"dfma": 2145155470 / 4044800, "dadd": 573527287 / 4044800,
                            "dmul": 914639971 / 4044800}
HEX_FP64_SOURCE = "the 505,600-element bar's timed window (t = 10 us, increment 1,553)"


def hex_fp64_flops_per_point() -> float:
    """FP64 flops per Gauss point (a DFMA counted as two)."""
    c = HEX_FP64_INSTR_PER_POINT
    return 2 * c["dfma"] + c["dadd"] + c["dmul"]


def hex_fp64_instr_per_point() -> float:
    c = HEX_FP64_INSTR_PER_POINT
    return c["dfma"] + c["dadd"] + c["dmul"]


def workload(name: str, layers: int = 400):
    if name == "hex":
        return meshes.taylor_hex(40, layers), f"taylor_hex_40x40x{layers}"
    if name == "axi":
        return meshes.taylor_axi(20, 200), "taylor_axi_20x200"
    if name == "hex1pt":  # not the reference's formulation (see meshes.taylor_hex_1pt)
        return meshes.taylor_hex_1pt(40, layers), f"taylor_hex_1pt_40x40x{layers}"
    raise SystemExit(f"unknown config {name}")


def cpu_sample(name: str, layers: int = 400):
    """CPU sample: the same bar, timed over a bounded number of steps after its prologue."""
    m, wname = workload(name, layers)
    return m, f"{wname} ({m.E:,} elements)"


def elem_bytes(m) -> float:
    """Compulsory HBM bytes of one k_elem launch: integration-point state read (S, Eps, EpsPlas, p,
    evp, evp^n) and written (S, Eps, EpsPlas, p; evp and evp^n only where plastic, not counted),
    connectivity, element forces written, node coordinates and delta_disp read once."""
    ns = 6 if m.dim == 3 else 4
    ncomp = 3 * ns + 3
    per_elem = m.nip * (ncomp * 8 + (3 * ns + 1) * 8) + m.nen * 4 + m.nen * m.dim * 8
    return m.E * per_elem + m.N * 2 * m.dim * 8


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for ln in open(self.path):
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        load = [s for s in sm if mx and s > 0.3 * max(mx)] or sm
        return {"sm_mhz": float(np.median(load)) if load else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def peak_hbm():
    """(HBM GB/s, "measured" | "fallback"): the copy bandwidth in MEASURED_PEAKS.json, else 6.8 TB/s."""
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(pk)) if os.path.exists(pk) else {}
    if "hbm_gbs" in peaks:
        return float(peaks["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_and_max(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units: float, seconds: float, world: int) -> float:
    """Whole-job rate of independent replicas: the units every rank processed, summed, over the
    slowest rank's time."""
    if world == 1:
        return units / seconds
    import torch
    import torch.distributed as dist
    u = torch.tensor([units], dtype=torch.float64)
    t = torch.tensor([seconds], dtype=torch.float64)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()) / float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def hex_config(model, name: str, args, world: int) -> dict:
    """The `config` of the element-update line, identical for both arms (it names the workload)."""
    ns = 4 if model.dim == 2 else 6
    return {"workload": name, "elements": model.E, "nodes": model.N,
            "time_step": ("Pulse" if model.method == meshes.PULSE else "Courant")
                         + f" every {model.freq} increments",
            "formulation": ("one Gauss point + viscous hourglass control (not the reference's "
                            "2x2x2-point ElHex8n3D)" if model.etype == meshes.ELHEX8N3D_1PT
                            else "the reference's"),
            "window": f"{args.steps} steps from t = {args.start_us:g} us of the impact, reached "
                      "untimed",
            "l2": "inputs larger than L2 (integration-point state "
                  f"{model.E * model.nip * (3 * ns + 3) * 8 / 1e6:.0f} MB)",
            "parallelism": f"replicas x{world}"}


def sm_count(device: int = 0) -> int:
    import torch
    return int(torch.cuda.get_device_properties(device).multi_processor_count)


def fp64_roofline(model, launch_s, clocks, device: int = 0):
    """Roofline of one k_elem launch of `model` taking `launch_s` seconds (CUDA events).

    Bound: the FP64 pipe.  achieved = FP64 flops per launch (the counted mix per Gauss point, a
    DFMA as two) / launch time, against the DFMA peak measured at the start of this run on this
    GPU (`dnl_measure_fp64_peak`: independent DFMA chains on every SM); the same launch as FP64
    instructions issued per second against the pipe's issue ceiling (2 FP64 thread-instructions per
    SM per cycle at the sampled SM clock).  HBM: the algorithmic bytes per launch over the launch
    time against the measured copy bandwidth, and the DRAM traffic ncu counted."""
    from redynela_gb300 import dynela
    hbm_peak, peak_src = peak_hbm()
    bytes_per_launch = elem_bytes(model)
    traffic = (ELEM_TRAFFIC_BYTES_PER_ELEMENT * model.E) if model.etype == meshes.ELHEX8N3D else None
    hbm = {"achieved": bytes_per_launch / launch_s / 1e9 if launch_s else None, "peak": hbm_peak,
           "unit": "GB/s", "peak_source": peak_src, "algorithmic_bytes_per_launch": bytes_per_launch,
           "traffic": traffic}
    hbm["frac"] = hbm["achieved"] / hbm_peak if hbm["achieved"] else None
    kernel = {meshes.ELHEX8N3D: "k_elem<ElHex8n3D>", meshes.ELQUA4NAX: "k_elem<ElQua4nAx>",
              meshes.ELHEX8N3D_1PT: "k_elem<ElHex8n3D at one point + hourglass>"}.get(model.etype, "k_elem")
    if model.etype != meshes.ELHEX8N3D or not launch_s:
        return dict(hbm, bound="hbm", kernel=kernel, avg_launch_ms=launch_s * 1e3 if launch_s else None)
    points = model.E * model.nip
    dfma_peak = dynela.fp64_peak_tflops()
    achieved = hex_fp64_flops_per_point() * points / launch_s / 1e12
    sms = sm_count(device)
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 0.0
    ceiling = sms * 2.0 * mhz * 1e6  # FP64 thread-instructions per second
    issued = hex_fp64_instr_per_point() * points / launch_s
    return {"bound": "fp64", "achieved": achieved, "peak": dfma_peak, "unit": "TFLOP/s",
            "frac": achieved / dfma_peak if dfma_peak else None, "traffic": traffic,
            "kernel": kernel, "avg_launch_ms": launch_s * 1e3,
            "peak_source": "measured on this GPU at the start of the run (DFMA loop); "
                           "MEASURED_PEAKS.json has no FP64 figure",
            "flops_per_gauss_point": hex_fp64_flops_per_point(),
            "fp64_instructions_per_gauss_point": dict(HEX_FP64_INSTR_PER_POINT),
            "counted_on": HEX_FP64_SOURCE,
            "issue": {"achieved_instr_per_s": issued, "ceiling_instr_per_s": ceiling,
                      "frac": issued / ceiling if ceiling else None, "sms": sms,
                      "sm_mhz": mhz, "per_sm_per_cycle": 2},
            "hbm": hbm}


def run_cpu_baseline(model, sample_desc, min_seconds=10.0, max_steps=400, threads=None,
                     start=None, start_us=0.0):
    """The oracle on the host cores.  `start` = (state, time info) of the GPU run at the window
    start, injected after the oracle's own prologue (which computes the lumped mass on the
    undeformed mesh, as the reference does once); otherwise the oracle advances to start_us."""
    from oracle.oracle import Oracle
    threads = threads or os.cpu_count() or 1
    o = Oracle(model, threads=threads)
    o.prologue()
    if start is not None:
        st, info = start
        o.inject(coords=st["coords"], du=st["du"], v=st["v"], a=st["a"], disp=st["disp"],
                 S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"],
                 dt=info["time_step"])
        o.set("time", info["time"])
        o.set("increment", info["increment"])
        o.set("computed_dt", info["computed_step"])
        o.set("last_dt", info["computed_step"])
        o.set("ts_date", info["time"])
        o.set("last_ts_date", info["time"])
        o.internal_matrices()
        if model.method == meshes.PULSE:
            o.max_frequency()  # warm the power-iteration vector like the GPU's
    else:
        while o.get("time") < start_us * 1e-6:
            if o.steps(50) == 0:
                break
    o.steps(2)  # warm-up
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        steps += o.steps(1)
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    rate = model.E * steps / dt
    return {"value": rate, "unit": "element-updates/s", "cores": threads, "kind": "port",
            "sample": f"{sample_desc}, {steps} explicit steps after the prologue, {dt:.1f} s"}


def main_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    model, sample = cpu_sample(args.config, args.layers)
    from oracle.oracle import Oracle
    threads = os.cpu_count() or 1
    o = Oracle(model, threads=threads)
    o.prologue()
    while o.get("time") < args.start_us * 1e-6:  # untimed, to the window start
        if o.steps(50) == 0:
            break
    t_start, inc_start = o.get("time"), int(o.get("increment"))
    if args.warmup:
        o.steps(args.warmup)
    t0 = time.perf_counter()
    done = o.steps(args.steps)
    dt = time.perf_counter() - t0
    rate = model.E * done / dt
    name = workload(args.config, args.layers)[1]
    line = {"impl": "reference", "metric": "element-updates/s", "value": rate,
            "unit": "element-updates/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": hex_config(model, name, args, args.gpus),
            "window_start": {"time_us": t_start * 1e6, "increment": inc_start},
            "cpu_baseline": {"value": rate, "unit": "element-updates/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{sample}; the oracle's C restatement of the reference "
                                       "(the reference's own build needs its sources, absent on "
                                       "this host)"},
            "e2e": {"value": rate, "unit": "element-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main_ours(args):
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from redynela_gb300 import build, dynela
    build.build()
    dynela.set_device(local)
    model, name = workload(args.config, args.layers)

    def to_window(dom):
        # advance, untimed, to the start of the measured window (runs are bitwise deterministic,
        # so every handle advanced this way holds the same state)
        dom.prologue()
        while dom.time_info()["time"] < args.start_us * 1e-6:
            if dom.step(50) == 0:
                break

    d = dynela.GpuDomain(model)
    to_window(d)
    window = d.time_info()
    snapshot = None
    if rank == 0 and not args.no_cpu:
        snapshot = d.get_state("coords", "du", "v", "a", "disp", "S", "Eps", "EpsPlas", "p", "evp")
    d.step(args.warmup)

    # ---- device-resident timed region
    barrier(world)
    with ClockSampler(local) as clk:
        launches0 = dynela.kernel_launches()
        d.profile_begin()
        dynela.range_push("window")
        d.timer_mark(0)
        done = d.step(args.steps)
        d.timer_mark(1)
        dynela.range_pop()
        ms = d.timer_elapsed_ms(0, 1)
        prof = d.profile_end()
        launches = dynela.kernel_launches() - launches0
    clocks = clk.summary()
    barrier(world)
    ms_max = barrier_and_max(ms, world)
    value = aggregate_rate(model.E * done, ms * 1e-3, world)

    # ---- roofline of the dominant kernel (k_elem): the FP64 pipe binds it, HBM is reported beside
    elem_ms, elem_n = prof["elem"]
    launch_s = elem_ms / elem_n * 1e-3 if elem_n else None
    roofline = fp64_roofline(model, launch_s, clocks, local)
    kernel_share = {k: round(v[0] / ms, 4) for k, v in prof.items() if v[1]}

    # ---- end to end through the C ABI with page-locked host buffers, over the same increments as
    # the timed region: a second handle brought to the same state (the cost of a step, and of the
    # Pulse iteration most of all, grows as the impact proceeds, so a later window would not compare)
    e2e_steps = args.steps
    N = model.N
    d.close()
    d = dynela.GpuDomain(model)
    to_window(d)
    d.step(args.warmup)
    host = {k: dynela.PinnedArray((N, 3)) for k in ("coords", "du", "v", "a", "disp")}
    st = d.get_state(*host.keys())
    for k, pa in host.items():
        pa.array[:] = st[k]
    # one view for both directions, built once: the loop is the C call itself
    sv = dynela.StateView()
    for k, pa in host.items():
        setattr(sv, k, pa.array.ctypes.data_as(dynela._dp))
    stepped = dynela.C.c_int(0)
    d.timer_mark(2)
    e2e_done = 0
    for _ in range(e2e_steps):
        d._check_run(d.L.dnl_step_host(d.h, dynela.C.byref(sv), 1, dynela.C.byref(sv), dynela.C.byref(stepped)))
        e2e_done += stepped.value
    d.timer_mark(3)
    e2e_ms = d.timer_elapsed_ms(2, 3)
    e2e_rate = aggregate_rate(model.E * e2e_done, e2e_ms * 1e-3, world)
    e2e_ms = barrier_and_max(e2e_ms, world)
    nodal_bytes = 5 * N * 3 * 8
    e2e = {"value": e2e_rate, "unit": "element-updates/s",
           "h2d_bytes_per_step": nodal_bytes, "d2h_bytes_per_step": nodal_bytes,
           "steps": e2e_done, "path": "dnl_step_host(in, 1, out) per step: the five nodal fields in, "
           "one step, the five out"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cm, sample = cpu_sample(args.config, args.layers)
        cpu = run_cpu_baseline(cm, sample, min_seconds=args.cpu_seconds,
                               start=(snapshot, window))

    if rank == 0:
        line = {"metric": "element-updates/s", "value": value, "unit": "element-updates/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_max / max(done, 1), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator of the reference Taylor deck's geometry)",
                "config": hex_config(model, name, args, world),
                "window_start": {"time_us": window["time"] * 1e6, "increment": window["increment"]},
                "gpu_launches": launches, "kernel_time_share": kernel_share,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks}
    d.close()
    if rank == 0 and world == 1 and not args.no_extras and args.config == "hex":
        # the batched, the gradient and the batched-gradient workloads, timed in the same run:
        # their own lines, kept under three keys of this one
        line["batched"] = batch_line(argparse.Namespace(**dict(vars(args), steps=20, warmup=3)))
        line["gradients"] = sens_line(argparse.Namespace(**dict(vars(args), steps=3, warmup=3,
                                                                no_cpu=True)), fd_steps=(1e-5,))
        line["necking"] = necking_line(argparse.Namespace(**dict(vars(args), steps=3, warmup=3,
                                                                 no_cpu=True)))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def batch_line(args) -> dict:
    """Batched mode: 256 seeded axisymmetric Taylor bars (radial x axial divisions 4-40 x 40-400,
    v 150-300 m/s, A 60-150 MPa, B 200-400 MPa, n 0.2-0.5), every instance advancing K steps with
    its own time step in one graph-captured launch sequence per step, against the same bars run
    one after another through the single-mesh path on the same GPU."""
    from redynela_gb300 import build, dynela
    build.build()
    models = meshes.taylor_batch(args.instances, seed=0)
    E = sum(m.E for m in models)
    b = dynela.BatchDomain(models)
    b.prologue()
    block = b.autotune(steps=3)
    mode = ("persistent kernel per step" if b.tuning()[0] == dynela.BATCH_PERSISTENT
            else "launch sequence per step")
    # every arm is timed over the same increments [S, S + K) of each bar, S = --batch-start (400:
    # every bar still running, the impact wave across most of them, their impact ends plastic; a
    # run's cost per step grows as the wave spreads and points yield).  The batch, back at t = 0
    # after the tuning: S - W K launch-sequence steps, W graph replays of K steps (the first
    # captures), then the timed replay.
    K, W = args.steps, max(1, args.warmup)
    start = max(args.batch_start, W * K)
    b.reset()
    b.prologue()
    if start > W * K:
        b.step(start - W * K)
    for _ in range(W):
        b.step_graph(K)
    inc0 = [b.time_info(i)["increment"] for i in range(len(models))]
    hv = b.handle_view()
    with ClockSampler(0) as clk:
        launches0 = dynela.kernel_launches()
        dynela.range_push("batch_window")  # the timed region, for a profiler's NVTX filter
        hv.timer_mark(0)
        active = b.step_graph(K)
        hv.timer_mark(1)
        dynela.range_pop()
        ms = hv.timer_elapsed_ms(0, 1)
        launches = dynela.kernel_launches() - launches0
    clocks = clk.summary()
    # element-updates: each bar's elements times the increments it made (a bar at its end time
    # makes none)
    done = sum(m.E * (b.time_info(i)["increment"] - inc0[i]) for i, m in enumerate(models))
    value = done / (ms * 1e-3)
    # the same bars one at a time through the single-mesh path, state resident, over the same
    # increments: stream launches (dnl_step) and graph replay (dnl_step_graph; the faster of the two
    # is the ratio's denominator)
    plain_ms = plain_graph_ms = 0.0
    plain_done = plain_graph_done = 0
    for m in models:
        d = dynela.GpuDomain(m)
        d.prologue()
        d.step(start)
        i0 = d.time_info()["increment"]
        d.timer_mark(0)
        d.step(K)
        d.timer_mark(1)
        plain_ms += d.timer_elapsed_ms(0, 1)
        plain_done += m.E * (d.time_info()["increment"] - i0)
        d.reset()
        d.prologue()
        if start > W * K:
            d.step(start - W * K)
        for _ in range(W):
            d.step_graph(K)  # the first captures
        i0 = d.time_info()["increment"]
        d.timer_mark(0)
        d.step_graph(K)
        d.timer_mark(1)
        plain_graph_ms += d.timer_elapsed_ms(0, 1)
        plain_graph_done += m.E * (d.time_info()["increment"] - i0)
        d.close()
    plain = plain_done / (plain_ms * 1e-3)
    plain_graph = plain_graph_done / (plain_graph_ms * 1e-3)
    line = {"metric": "element-updates/s (batched)", "value": value, "unit": "element-updates/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, numpy default_rng(0))",
            "config": {"workload": f"taylor_axi_batch_{args.instances}", "elements": E,
                       "instances": args.instances, "block": block, "mode": mode,
                       "window": f"increments {start} to {start + K} of every bar, "
                                 "the same for the batch and the bars run alone",
                       "element_updates_timed": done,
                       "active_after": active,
                       "l2": "inputs larger than L2 (integration-point state "
                             f"{E * 4 * 15 * 8 / 1e6:.0f} MB)"},
            "plain_instance_by_instance": {"value": max(plain, plain_graph),
                                           "ms_per_step": min(plain_ms, plain_graph_ms) / args.steps,
                                           "stream_launches": {"value": plain,
                                                               "ms_per_step": plain_ms / args.steps},
                                           "graph_replay": {"value": plain_graph,
                                                            "ms_per_step": plain_graph_ms / args.steps}},
            "batched_over_plain": value / max(plain, plain_graph), "gpu_launches": launches,
            "clocks": clocks}
    return line


def main_batch(args):
    print(json.dumps(batch_line(args)), flush=True)


def sens_line(args, fd_steps=(1e-5, 1e-6, 1e-7)) -> dict:
    """Gradient workload: the 20x200 axisymmetric Taylor bar (4,000 ElQua4nAx elements) advanced
    with a fixed step-size schedule -- the nominal run's own Courant steps, at most 4,000 -- and
    L = |x_final(p) - x_target|^2 with x_target the final shape for (A, B, n) = (110 MPa, 310 MPa,
    0.28).  One gradient = dL/d(A, B, n, |v0|) at the nominal parameters: dnl_reset with the
    parameters, one forward-mode run (dnl_sens_run: the explicit run plus four tangent copies) and
    the contraction with dL/dx.  `value`: gradients/s from CUDA events around the device work;
    `e2e`: wall clock of the whole call sequence a user makes (reset, run, copies, contraction)."""
    from redynela_gb300 import build, dynela
    build.build()
    m = meshes.taylor_axi(20, 200)
    v0 = float(np.linalg.norm(m.v0))
    sched = dynela.GpuDomain(m)
    sched.prologue()
    dts = []
    while len(dts) < args.sens_steps:
        info = sched.time_info()
        if info["done"]:
            break
        dts.append(info["time_step"])
        if sched.step(1) == 0:
            break
    sched.close()
    dts = np.array(dts)
    nst = len(dts)
    target = dynela.model_with_params(m, 110e6, 310e6, 0.28, v0)
    xt, _ = dynela.GpuDomain(target).sensitivities(dts)
    d = dynela.GpuDomain(m)
    surf = meshes.taylor_axi_free_surface(20, 200)  # outer radius and top face nodes
    w = np.zeros((m.N, 3))

    def gradient():
        # L = mean over the free-surface nodes of |x - x_target|^2
        d.reset(m)
        x, dx = d.sensitivities(dts)
        w[:] = 0.
        w[surf] = 2.0 * (x[surf] - xt[surf]) / len(surf)
        return np.einsum("pnj,nj->p", dx, w), x

    for _ in range(args.warmup):
        gradient()
    launches0 = dynela.kernel_launches()
    dev_ms = 0.0
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            d.timer_mark(0)
            g, x = gradient()
            d.timer_mark(1)
            dev_ms += d.timer_elapsed_ms(0, 1)
        wall = time.perf_counter() - t0
    launches = (dynela.kernel_launches() - launches0) // args.steps
    value = args.steps / (dev_ms * 1e-3)
    # the forward cost: the same schedule as a plain run (Courant steps recomputed, as the schedule
    # was made) from the same initial state, graph-replayed; the mean of K runs
    fwd_ms = 0.0
    for _ in range(args.steps):
        d.reset(m)
        d.prologue()
        d.timer_mark(0)
        k = 0
        while k < nst:
            k += d.step_graph(min(100, nst - k))
        d.timer_mark(1)
        fwd_ms += d.timer_elapsed_ms(0, 1) / args.steps
    grad_ms = dev_ms / args.steps
    e2e = args.steps / wall
    # central differences of L over the same fixed schedule, h = 1e-5, 1e-6, 1e-7 relative per
    # parameter: the difference quotient carries the run's rounding noise in L divided by 2h, so
    # its distance from the derivative growing as h shrinks shows that noise, not the derivative
    pv = np.array([m.A, m.B, m.n, v0])

    def loss_at(q):
        d.reset(dynela.model_with_params(m, *q))
        x, _ = d.sensitivities(dts)
        return float(np.mean(np.sum((x[surf] - xt[surf]) ** 2, axis=1)))

    fd_rel = {}
    for hrel in fd_steps:
        errs = []
        for p in range(4):
            h = hrel * pv[p]
            lp, lm = (loss_at(pv + s * h * np.eye(4)[p]) for s in (1.0, -1.0))
            errs.append(float(abs((lp - lm) / (2 * h) - g[p]) / abs(g[p])))
        fd_rel[f"{hrel:.0e}"] = errs
    # the quotients at h = 1e-6 with the two iterations' stopping tests tightened
    # (dnl_set_stop_tolerances): with the reference's tolerances a change of 1e-6 in a parameter
    # can add or remove an iteration somewhere in the run, a jump of the tolerance's order in L
    # that the quotient divides by h; with tight ones the run's map is smooth at that scale and the
    # quotients meet the derivative (recomputed under the same tolerances)
    tight = {"polar": 1e-15, "radial_return": 1e-13}
    dynela.set_stop_tolerances(tight["polar"], tight["radial_return"])
    try:
        d.reset(m)
        xs, dxs = d.sensitivities(dts)
        ws = np.zeros((m.N, 3))
        ws[surf] = 2.0 * (xs[surf] - xt[surf]) / len(surf)
        gs = np.einsum("pnj,nj->p", dxs, ws)
        errs = []
        for p in range(4):
            h = 1e-6 * pv[p]
            lp, lm = (loss_at(pv + s * h * np.eye(4)[p]) for s in (1.0, -1.0))
            errs.append(float(abs((lp - lm) / (2 * h) - gs[p]) / abs(gs[p])))
    finally:
        dynela.set_stop_tolerances()
    fd_tight = {"h": 1e-6, "relative_error": errs, "stop_tolerances": tight,
                "derivative_change_vs_reference_tolerances": float(np.max(np.abs(gs - g) / np.abs(g)))}
    # reverse mode: the same gradient by dnl_adjoint_forward (the run with a checkpoint every
    # ceil(sqrt(steps)) steps, the final shape), the loss's dL/dx on the host, then
    # dnl_adjoint_backward (the reverse sweep); CUDA events around the whole sequence
    def gradient_reverse():
        d.reset(m)
        x = d.adjoint_forward(dts, 0)
        w[:] = 0.
        w[surf] = 2.0 * (x[surf] - xt[surf]) / len(surf)
        return d.adjoint_backward(w)

    for _ in range(args.warmup):
        gradient_reverse()
    rev_ms = 0.0
    with ClockSampler(0) as clk_rev:
        launches0 = dynela.kernel_launches()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            d.timer_mark(0)
            g_rev = gradient_reverse()
            d.timer_mark(1)
            rev_ms += d.timer_elapsed_ms(0, 1)
        rev_wall = time.perf_counter() - t0
        rev_launches = (dynela.kernel_launches() - launches0) // args.steps
    rev_ms /= args.steps
    ast = d.adjoint_stats()
    # kernel shares of one more reverse-mode gradient with CUDA events around every launch
    # (untimed; profiled sweeps launch step by step instead of replaying their graphs)
    d.profile_begin()
    gradient_reverse()
    prof_rev = d.profile_end()
    # the device memory a stored trajectory would take: every step's state record
    per_record = ast["record_bytes"] / max(ast["stride"], 1)
    checkpointing = {"checkpoints": ast["checkpoints"], "steps_per_checkpoint": ast["stride"],
                     "recomputed_steps": ast["recomputed_steps"], "device_bytes": ast["bytes"],
                     "checkpoint_bytes": ast["checkpoint_bytes"],
                     "segment_record_bytes": ast["record_bytes"],
                     "kept_per_point_record_bytes": ast["kept_record_bytes"],
                     "stored_trajectory_bytes": int(per_record * nst)}
    forward_mode = {"value": value, "unit": "gradients/s", "gradient_ms": grad_ms,
                    "gradient_cost_vs_forward": grad_ms / fwd_ms,
                    "gradient": [float(v) for v in g], "gpu_launches": launches,
                    "e2e": e2e,
                    "path": "dnl_reset + dnl_sens_run (the run with four tangent copies) + contraction"}
    # the reverse sweep's dominant kernel, the element pass's adjoint (profiled as "tangent")
    adj_ms, adj_n = prof_rev["tangent"]
    total_ms = sum(v[0] for v in prof_rev.values())
    # agreement with the sensitivity oracle (FP64 dual numbers) over a bounded prefix, which is
    # also the CPU baseline's sample
    cpu = None
    agree = None
    if not args.no_cpu:
        from oracle.oracle import Oracle, SensOracle
        threads = os.cpu_count() or 1
        o = Oracle(m, threads=threads)
        o.prologue()
        mass = o.array("mass").copy()
        probe = 20
        so = SensOracle(m, mass=mass, threads=threads)
        t1 = time.perf_counter()
        so.run(dts[:probe])
        per_step = (time.perf_counter() - t1) / probe
        k = int(min(nst, max(probe, args.cpu_seconds / max(per_step, 1e-9))))
        so = SensOracle(m, mass=mass, threads=threads)
        t1 = time.perf_counter()
        so.run(dts[:k])
        tc = time.perf_counter() - t1
        _, dxo = so.coords()
        d.reset(m)
        _, dxg = d.sensitivities(dts[:k])
        agree = max(float(np.linalg.norm(dxg[p] - dxo[p]) / np.linalg.norm(dxo[p])) for p in range(4))
        cpu = {"value": 1.0 / (tc * nst / k), "unit": "gradients/s", "cores": threads, "kind": "port",
               "sample": f"the sensitivity oracle (FP64 dual numbers, OpenMP) over the first {k} of "
                         f"the {nst} steps, {tc:.1f} s, scaled to the full schedule"}
    # adjoint element pass: compulsory bytes per launch -- the step's per-point record (64 doubles,
    # axisymmetric) and the integration-point state read, the state adjoints (15 doubles per point)
    # read and written, the parameter adjoints (4 per point) accumulated, the element-node adjoints
    # of coordinates and delta_disp written -- over its mean launch time
    nip, nt = 4, 64
    adj_bytes = m.E * nip * 8 * (nt + 15 + 2 * 15 + 2 * 4) + m.E * 4 * 2 * 8 * 2
    line = {"metric": "adjoint gradients/s", "value": 1e3 / rev_ms, "unit": "gradients/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": rev_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the reference Taylor deck's geometry)",
            "config": {"workload": "taylor_axi_20x200_sensitivities", "elements": m.E,
                       "explicit_steps": nst, "parameters": ["A", "B", "n", "|v0|"],
                       "loss": "mean over the free-surface nodes (outer radius, impact-free end) of "
                               "|x_final - x_final(A=110 MPa, B=310 MPa, n=0.28)|^2",
                       "step": "one gradient = dnl_reset + dnl_adjoint_forward (the run, a "
                               "checkpoint every ceil(sqrt(steps)) steps, made even) + dL/dx on "
                               "the host + dnl_adjoint_backward (the reverse sweep)",
                       "l2": "state of 4,000 elements fits L2; each gradient is a 4,000-step run"},
            "gradient": [float(v) for v in g_rev],
            "forward_run_ms": fwd_ms, "gradient_ms": rev_ms,
            "gradient_cost_vs_forward": rev_ms / fwd_ms,
            "checkpointing": checkpointing,
            "agreement_vs_forward_mode": float(np.max(np.abs(g_rev - g) / np.abs(g))),
            "agreement_vs_dual_oracle": agree,
            "agreement_vs_central_differences": {"relative_error_by_relative_h": fd_rel,
                                                 "with_tight_stopping_tests": fd_tight,
                                                 "of": "the forward-mode gradient"},
            "forward_mode": forward_mode,
            "gpu_launches": rev_launches,
            "kernel_time_share": {k: round(v[0] / total_ms, 4) for k, v in prof_rev.items()} if total_ms else None,
            "roofline": {"bound": "hbm", "achieved": adj_bytes / (adj_ms / max(adj_n, 1) * 1e-3) / 1e9,
                         "peak": peak_hbm()[0], "unit": "GB/s",
                         "frac": adj_bytes / (adj_ms / max(adj_n, 1) * 1e-3) / 1e9 / peak_hbm()[0],
                         "avg_launch_ms": adj_ms / max(adj_n, 1), "algorithmic_bytes_per_launch": adj_bytes,
                         "traffic": None, "kernel": "k_elem_adj<ElQua4nAx>",
                         "peak_source": peak_hbm()[1],
                         "note": "4,000 elements: launch-latency bound; the adjoint pass is FP64 work"},
            "cpu_baseline": cpu,
            "e2e": {"value": args.steps / rev_wall, "unit": "gradients/s",
                    "h2d_bytes_per_step": 8 * (nst + 3 * m.N), "d2h_bytes_per_step": 8 * (3 * m.N + 4)},
            "clocks": clk_rev.summary()}
    return line


def main_sens(args):
    print(json.dumps(sens_line(args)), flush=True)


def main_necking(args):
    print(json.dumps(necking_line(args)), flush=True)


def necking_line(args) -> dict:
    """Batched sensitivities: 32 parameter sets (A, B, n drawn as for the batched Taylor bars) of
    the tensile necking bar (ElHex8n3D, gauge radius 6.4 mm, length 53.3 mm, 209,824 elements each,
    6.7 M in the batch; clamped end, the other pulled at 1 m/s, mass scaling x100) run as one batch
    with their forward-mode derivatives, over a 30,000-step schedule of 3.55e-7 s.  The timed window
    is K steps of that schedule from its middle, where the bar is plastic: one bar is run to step
    15,000 (the plain scheduled run, untimed), its state is copied into every instance
    (dnl_batch_broadcast_state) and the batched tangent run is timed from there.  `value` = instances
    / (time per step of the window x 30,000).  Loss: the mid-length cross-section, mean over its
    nodes of x^2 + y^2 (the necking measure)."""
    from redynela_gb300 import build, dynela
    build.build()
    nz = 166
    models = meshes.necking_batch(args.necking_instances, seed=0, nz=nz)
    total_steps = 30000
    start_step = args.necking_start
    dt = models[0].tend / total_steps
    probe = dynela.GpuDomain(models[0])
    probe.prologue()
    dt_stable = probe.time_step()
    probe.close()
    # the window's starting state: one bar run plainly to mid-schedule
    src = dynela.GpuDomain(models[0])
    t0 = time.perf_counter()
    src.run_schedule(np.full(start_step, dt))
    advance_s = time.perf_counter() - t0
    evp_mid = src.get_state("evp")["evp"]
    plastic_frac = float(np.mean(evp_mid > 1e-9))
    E = sum(m.E for m in models)
    b = dynela.BatchDomain(models)
    dts = np.full(max(args.warmup, args.steps), dt)
    b.broadcast_state(src)
    b.sensitivities(dts[:args.warmup], outputs=False)  # allocations, first launches
    b.reset()
    b.broadcast_state(src)
    src.close()
    hv = b.handle_view()
    launches0 = dynela.kernel_launches()
    hv.profile_begin()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        hv.timer_mark(0)
        b.sensitivities(dts[:args.steps], outputs=False)
        hv.timer_mark(1)
        wall = time.perf_counter() - t0
    ms = hv.timer_elapsed_ms(0, 1)
    prof = hv.profile_end()
    launches = dynela.kernel_launches() - launches0
    clocks = clk.summary()
    per_step = ms * 1e-3 / args.steps
    value = len(models) / (per_step * total_steps)
    tan_ms, tan_n = prof["tangent"]
    total_ms = sum(v[0] for v in prof.values())
    nip, ns, nt = 8, 6, 76  # the per-point record of a hex8 Gauss point: 76 doubles
    tan_bytes = E * nip * 8 * (nt + 3 * ns + 1 + 4 * 2 * (3 * ns + 2)) + E * 8 * 3 * 8 * 4
    achieved = tan_bytes / (tan_ms / max(tan_n, 1) * 1e-3) / 1e9 if tan_n else None
    cpu = None
    agree = None
    if not args.no_cpu:
        from oracle.oracle import SensOracle
        threads = os.cpu_count() or 1
        m0 = models[0]
        g = dynela.GpuDomain(m0)
        g.prologue()
        mass = g.get_state("mass")["mass"].ravel().copy()  # lumped mass, bit-exact with the oracle's
        g.close()
        k = 2
        so = SensOracle(m0, mass=mass, threads=threads)
        t1 = time.perf_counter()
        so.run(dts[:k])
        tc = (time.perf_counter() - t1) / k
        _, dxo = so.coords()
        g = dynela.GpuDomain(m0)
        _, dxg = g.sensitivities(dts[:k])
        agree = max(float(np.linalg.norm(dxg[p] - dxo[p]) / np.linalg.norm(dxo[p]))
                    for p in range(3) if np.linalg.norm(dxo[p]) > 0) if any(
            np.linalg.norm(dxo[p]) > 0 for p in range(3)) else None
        cpu = {"value": 1.0 / (tc * total_steps), "unit": "gradients/s", "cores": threads,
               "kind": "port",
               "sample": f"the sensitivity oracle (FP64 dual numbers, OpenMP) on one bar "
                         f"({m0.E:,} elements), its first {k} steps, {tc:.2f} s per step, scaled to one "
                         f"gradient of the 30,000-step schedule"}
    line = {"metric": "gradients/s (batched, 3D)", "value": value, "unit": "gradients/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded parameter sets, numpy default_rng(0))",
            "config": {"workload": f"necking_hex_batch_{len(models)}", "elements": E,
                       "instances": len(models), "elements_per_instance": models[0].E,
                       "schedule": f"{total_steps} steps of {dt:.4g} s (stable step at t=0: "
                                   f"{dt_stable:.4g} s)",
                       "timed": f"{args.steps} steps of the schedule from step {start_step} "
                                f"(the state one bar reached there, {plastic_frac:.0%} of its Gauss "
                                f"points plastic, copied into every instance; reached in "
                                f"{advance_s:.0f} s untimed), extrapolated to {total_steps}",
                       "parameters": ["A", "B", "n", "|v0| (0: starts at rest)"],
                       "l2": "inputs larger than L2 (tangent state "
                             f"{E * 8 * 4 * 20 * 8 / 1e9:.0f} GB)"},
            "element_updates_per_s_with_tangents": E / per_step,
            "agreement_vs_dual_oracle": agree,
            "gpu_launches": launches,
            "kernel_time_share": {k: round(v[0] / total_ms, 4) for k, v in prof.items()} if total_ms else None,
            "roofline": {"bound": "fp64", "achieved": None, "peak": None, "unit": "TFLOP/s",
                         "frac": None, "traffic": None,
                         "kernel": "k_elem_tan<ElHex8n3D>",
                         "avg_launch_ms": tan_ms / max(tan_n, 1),
                         "hbm": {"achieved": achieved, "peak": peak_hbm()[0], "unit": "GB/s",
                                 "frac": achieved / peak_hbm()[0] if achieved else None,
                                 "peak_source": peak_hbm()[1],
                                 "algorithmic_bytes_per_launch": tan_bytes},
                         "note": "the tangent pass is FP64-pipe bound; no FP64 count is taken here"},
            "cpu_baseline": cpu,
            "e2e": {"value": 1.0 / (wall / args.steps * total_steps) * len(models), "unit": "gradients/s",
                    "h2d_bytes_per_step": 8, "d2h_bytes_per_step": 0},
            "clocks": clocks}
    return line


def main_fd_sweep(args):
    """Forward-mode tangents against central differences, every element type: a small bar of each
    (and a domain of two, and the tensile bar pulled by an imposed speed) over its own plain run's
    step sizes, L = a seeded random linear functional of the final coordinates, the largest
    relative distance over A, B, n, |v0| of the central quotient of L (dnl_run_schedule at
    p +- h p) from the tangent, at h = 1e-5, 1e-6, 1e-7 relative; with the reference's stopping
    tests and with them tightened (dnl_set_stop_tolerances 1e-15, 1e-13).  One JSON line; not a
    throughput measurement."""
    from redynela_gb300 import build, dynela
    build.build()
    bars = {"axi_4x30": (meshes.taylor_axi(4, 30), 120), "plane_4x30": (meshes.taylor_plane(4, 30), 120),
            "hex_4x4x10_pulse": (meshes.taylor_hex(4, 10), 80), "tet4_6x6x8": (meshes.taylor_tet(6, 8), 80),
            "hex1pt_6x6x10": (meshes.taylor_hex_1pt(6, 10), 80),
            "tensile_4x4x12_speed": (meshes.necking_bar(4, 12, speed=5.0), 60),
            "hex_tet_4x4x8": (meshes.taylor_mixed(4, 8, lower=meshes.ELHEX8N3D, upper=meshes.ELTET4N3D), 60)}
    steps = (1e-5, 1e-6, 1e-7)
    out = {}
    try:
        for tight in (False, True):
            dynela.set_stop_tolerances(*((1e-15, 1e-13) if tight else (-1.0, -1.0)))
            for name, (m, n) in bars.items():
                d = dynela.GpuDomain(m)
                d.prologue()
                dts = []
                for _ in range(n):
                    dts.append(d.time_info()["time_step"])
                    d.step(1)
                dts = np.array(dts)
                w = np.zeros((m.N, 3))
                w[:, :m.dim] = np.random.default_rng(3).normal(size=(m.N, m.dim))
                _, dx = dynela.GpuDomain(m).sensitivities(dts)
                g = np.einsum("pnj,nj->p", dx, w)
                pv = np.array([m.A, m.B, m.n, np.linalg.norm(m.v0)])
                e = dynela.GpuDomain(m)
                worst = {}
                for hrel in steps:
                    errs = []
                    for p in range(4):
                        if pv[p] == 0.0 or g[p] == 0.0:
                            continue
                        h = hrel * pv[p]
                        ls = []
                        for sgn in (1.0, -1.0):
                            e.reset(dynela.model_with_params(m, *(pv + sgn * h * np.eye(4)[p])))
                            ls.append(float(np.sum(e.run_schedule(dts) * w)))
                        errs.append(abs((ls[0] - ls[1]) / (2 * h) - g[p]) / abs(g[p]))
                    worst[f"{hrel:.0e}"] = max(errs)
                out.setdefault(name, {})["tight" if tight else "reference"] = worst
    finally:
        dynela.set_stop_tolerances()
    print(json.dumps({"metric": "max relative distance of central differences from the tangents",
                      "stop_tolerances": {"reference": [1e-9, 1e-8], "tight": [1e-15, 1e-13]},
                      "by_bar": out}), flush=True)


def main_full_run(args):
    """The whole run of a bar (`--config hex` or `hex1pt`) from t = 0 to its end time (80 us), not a
    window: the prologue, then dnl_run, CUDA events on the library's stream around the run.
    `value` = elements x increments / run time; the early elastic steps are cheaper per element
    than the window of the default line, the late ones dearer (the impact end crushed, the Pulse
    iteration longer)."""
    from redynela_gb300 import build, dynela
    build.build()
    model, name = workload(args.config, args.layers)
    d = dynela.GpuDomain(model)
    d.prologue()
    with ClockSampler(0) as clk:
        launches0 = dynela.kernel_launches()
        d.timer_mark(0)
        n = d.run()
        d.timer_mark(1)
        launches = dynela.kernel_launches() - launches0
    ms = d.timer_elapsed_ms(0, 1)
    info = d.time_info()
    line = {"metric": "element-updates/s (full run)", "value": model.E * n / (ms * 1e-3),
            "unit": "element-updates/s", "n_gpus": 1, "steps": n, "warmup": 0,
            "ms_per_step": ms / max(n, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator of the "
            "reference Taylor deck's geometry)",
            "config": {"workload": name, "elements": model.E, "nodes": model.N,
                       "run": f"t = 0 to {model.tend * 1e6:g} us, {n} increments",
                       "end_time_us": info["time"] * 1e6, "status": info["status"]},
            "run_s": ms * 1e-3, "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="hex",
                    choices=["hex", "hex1pt", "axi", "batch", "sens", "necking", "fdsweep"])
    ap.add_argument("--necking-instances", type=int, default=32)
    ap.add_argument("--necking-start", type=int, default=15000,
                    help="schedule step at which the necking window starts (reached untimed)")
    ap.add_argument("--sens-steps", type=int, default=4000,
                    help="explicit steps of the gradient workload's schedule")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--batch-start", type=int, default=400,
                    help="increment at which the batched line's timed window starts")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--start-us", type=float, default=10.0,
                    help="simulated time at which the timed window starts (reached untimed), so "
                         "the window sees the deformed, partly plastic bar of a real run")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--full-run", action="store_true",
                    help="time the bar's whole run to its end time instead of a window")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched, gradient and necking workloads that the default line "
                         "also reports")
    ap.add_argument("--layers", type=int, default=400,
                    help="axial layers of the hex bar (400 = the benchmark workload; fewer for "
                         "profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        main_reference(args)
    elif args.config == "batch":
        main_batch(args)
    elif args.config == "sens":
        main_sens(args)
    elif args.config == "necking":
        main_necking(args)
    elif args.config == "fdsweep":
        main_fd_sweep(args)
    elif args.full_run:
        main_full_run(args)
    else:
        main_ours(args)


if __name__ == "__main__":
    main()
