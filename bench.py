#!/usr/bin/env python
"""Benchmark of the linear-solve hot path on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): the 256^3
Poisson system on the uniform unit-cube hex mesh (16,777,216 cells,
50,135,040 internal faces), fixed value on x = 0, zero gradient elsewhere,
RHS U[-1, 1] (seed 2), solved by PCG + DIC to a 1e-10 relative residual.

One step = one solve from a freshly set matrix: coefficient packing, DIC
factorisation and the Krylov iterations of the mixed-precision refined PCG
(FP32 inner iterations, FP64 reliable updates).  ``value`` is seconds per
solve with the system resident in HBM (inputs of ~1.9 GB are far larger than
the 129 MB L2, so no flush is needed between steps).  The FP64 PCG solve of
the same system is timed once beside it for the speed-up.

``e2e`` repeats the step through the public API with HOST buffers: the
page-locked host coefficients and RHS go to the LduMatrix setters and
``to_device`` (which move them with the SMs over NVLink-C2C) and x is read
back with ``to_host``, all inside the timed region; the same loop with
copy-engine copies is timed beside it (``e2e.copy_engine_loop``).

``roofline``: the dominant kernel is the FP32 Amul + p.Ap reduction of the
inner iteration.  ``achieved`` is the bytes that kernel moves per launch in
its own layout -- p, diagonal and Ap (4 B per cell each), the off-diagonal
slots (4 B per slot, both sides) and the per-slice {offset, mask} entries
(8 B per slot column); no per-face index is read, the offsets replace them
-- divided by the launch durations recorded with CUDA events on the
launching stream during the timed steps.  ``frac_survey_bytes`` states the
same durations against B_amul(4) = 12n + 16F, which also counts int32
owner and neighbour arrays this kernel never reads.  ``traffic`` is the DRAM
bytes per launch of a small-case ncu capture of the same kernel, scaled to
this workload by its layout bytes.

``--impl reference`` times the reference algorithm on the host cores
instead: the CPU restatement of the reference's PCG+DIC (the reference is
pure Python on PyTorch and cannot run here), threaded over all host cores.
It first runs one full FP64 solve to the tolerance (its iteration count and
time are reported), then each step is a bounded sample (DIC factorisation
+ 20 iterations) extrapolated to that iteration count.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to 1e-10 rel. residual: mixed-prec refined vs FP64 PCG on GPU; Amul HBM GB/s"
WORKLOAD = "256^3 Poisson (unit-cube hex, x0 fixed value), PCG+DIC to 1e-10 relative residual"
# ncu summary of the small-case capture whose DRAM bytes per launch give
# ``roofline.traffic`` (scaled by layout bytes to the bench's size)
TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "mp_ap_stream_kernel_192cube_dram.md")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", "--size", type=int, default=256, dest="n",
                   help="cells per direction (--size under torchrun, whose own options "
                        "--n would abbreviate)")
    p.add_argument("--rel-tol", type=float, default=1e-10)
    p.add_argument("--delta", type=float, default=0.1)
    p.add_argument("--storage", choices=["auto", "full", "symmetric"], default="auto",
                   help="inner FP32 Amul of the mixed PCG: both coefficient sides, the "
                        "owner-side half of a symmetric matrix, or the solver's default")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison solve")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    p.add_argument("--ref-sample-only", action="store_true",
                   help="--impl reference: skip the full solve that sets the iteration count")
    p.add_argument("--workload", choices=["poisson256", "poisson256_renumbered", "poisson32",
                                          "convdiff128", "batch64", "adjoint96", "next",
                                          "assembly"],
                   default="poisson256",
                   help="poisson256 (default, the headline): 256^3 mixed vs FP64 PCG; "
                        "poisson32: 32^3 PCG+DIC to 1e-6; convdiff128: 128^3 jittered "
                        "convection-diffusion with PBiCGStab+DILU; batch64: 64 uneven Poisson "
                        "systems, batched; adjoint96: adjoint gradient of 20 implicit steps at 96^3; "
                        "next: geometry, correctors, GAMG and smoothers")
    p.add_argument("--convdiff-legs", default="standard,reference,mixed,mixed_kernels,mixed_gather,"
                                              "mixed_fused,standard_1e-10,mixed_1e-10",
                   help="convdiff128: comma-separated solver legs to run")
    p.add_argument("--fd-faces", type=int, default=32, help="adjoint96: faces checked by central "
                                                            "differences")
    return p.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
def b_amul(s: int, n: int, F: int) -> int:
    return 3 * s * n + 2 * s * F + 8 * F


def design_bytes_ap(n: int, n_slots: int, sym: bool) -> int:
    """Bytes the staged FP32 K_ap moves in its own layout: p, diagonal and
    Ap (4 B each per cell), the off-diagonal slots (4 B per slot on both
    sides; for the half storage of a symmetric matrix only the owner-side
    half, plus a 1 B mirror entry per neighbour-side slot column) and one
    8 B {offset, mask} entry per slot column of 32 slots.  No per-face index
    bytes: the offsets replace them."""
    cols = n_slots // 32
    if sym:
        return 12 * n + 2 * n_slots + cols * 8 + cols // 2
    return 12 * n + 4 * n_slots + cols * 8


def layout_bytes(s: int, n: int, n_slots: int, n_slices: int, kind: str) -> int:
    """Bytes one Amul moves in a given layout, element size s: x, diagonal
    and y (s B per cell each) and one coefficient per slot (s B), plus the
    addressing the layout reads -- an 8 B {offset, mask} entry per column of
    32 slots (offset-compressed), with the per-slice start and width (4 + 4
    B per slice) when the width is not fixed, or an int32 column per slot
    (explicit columns)."""
    base = 3 * s * n + s * n_slots
    if kind == "compressed":
        return base + 8 * (n_slots // 32)
    if kind == "variable_width":
        return base + 8 * (n_slots // 32) + 8 * n_slices
    if kind == "explicit_columns":
        return base + 4 * n_slots + 8 * n_slices
    raise ValueError(kind)


def traffic_from_profile(design_bytes: int) -> dict | None:
    """DRAM bytes per launch of K_ap from the committed small-case capture,
    scaled to this workload by layout bytes.  The summary holds one line
    ``traffic: <dram read+write bytes per launch> <layout bytes per launch>``."""
    try:
        with open(TRAFFIC_PROFILE) as f:
            for line in f:
                if line.startswith("traffic:"):
                    dram, lay = (float(v) for v in line.split()[1:3])
                    return {"bytes": dram / lay * design_bytes, "ratio_to_layout_bytes": dram / lay,
                            "captured_dram_bytes": dram, "captured_layout_bytes": lay,
                            "source": os.path.relpath(TRAFFIC_PROFILE, ROOT)}
    except (OSError, ValueError):
        pass
    return None


def load_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def make_matrix(sysd, dev):
    from pyopenfoam_gb300 import LduMatrix

    m = LduMatrix(sysd["n"], torch.as_tensor(sysd["owner"]), torch.as_tensor(sysd["neighbour"]),
                  device=dev)
    m.diag = torch.as_tensor(sysd["diag"])
    m.lower = torch.as_tensor(sysd["lower"])
    m.upper = torch.as_tensor(sysd["upper"])
    m.topology()
    return m


def true_rel_residual(m, x, b) -> float:
    r = b - m.Ax(x)
    return float(torch.linalg.vector_norm(r) / torch.linalg.vector_norm(b))


def time_amul(m, dev, reps=20):
    from pyopenfoam_gb300 import _lib

    n, F = m.n_cells, m.n_internal_faces
    x = torch.rand(n, dtype=torch.float64, device=dev)
    topo = m.topology()
    L = _lib.lib()
    st = torch.cuda.current_stream(dev)
    out = {}
    y64 = torch.empty_like(x)
    coef64 = m.packed()
    coef32 = m.packed(dtype=torch.float32)
    d32, x32 = m.diag.float(), x.float()
    y32 = torch.empty_like(x32)
    import ctypes

    plain = topo.uncompressed_layout()
    var = topo.variable_width_layout()
    fns = {
        "f64": lambda: L.gbf_amul_f64(topo.layout_ref, coef64.data_ptr(), m.diag.data_ptr(),
                                      x.data_ptr(), y64.data_ptr(), 0, st.cuda_stream),
        "f32": lambda: L.gbf_amul_f32(topo.layout_ref, coef32.data_ptr(), d32.data_ptr(),
                                      x32.data_ptr(), y32.data_ptr(), 0, st.cuda_stream),
        "f32_explicit_columns": lambda: L.gbf_amul_f32(ctypes.byref(plain), coef32.data_ptr(),
                                                       d32.data_ptr(), x32.data_ptr(),
                                                       y32.data_ptr(), 0, st.cuda_stream),
        "f32_variable_width": lambda: L.gbf_amul_f32(ctypes.byref(var), coef32.data_ptr(),
                                                     d32.data_ptr(), x32.data_ptr(),
                                                     y32.data_ptr(), 0, st.cuda_stream),
    }
    kinds = {"f64": "compressed", "f32": "compressed", "f32_explicit_columns": "explicit_columns",
             "f32_variable_width": "variable_width"}
    for name, fn in fns.items():
        s = 8 if name == "f64" else 4
        moved = layout_bytes(s, n, topo.n_slots, topo.n_slices, kinds[name])
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"us": ms * 1e3, "layout": kinds[name], "bytes": moved,
                     "GBs": moved / (ms * 1e-3) / 1e9,
                     "GBs_survey_bytes": b_amul(s, n, F) / (ms * 1e-3) / 1e9}
    return out


def cpu_sample(sysd, iters=20, threads=None):
    """Reference algorithm on the host: DIC build + PCG iterations, threaded
    over all host cores (oracle restatement of the reference).  Two solves,
    of 2 and 2 + `iters` iterations, separate the cost of an iteration from
    the per-call set-up (work vectors allocated and first touched, the
    initial residual), which a single short solve would spread over its few
    iterations.  Returns (DIC s, s per iteration, set-up s, threads)."""
    from oracle import oracle as O

    threads = threads or len(os.sched_getaffinity(0))
    own, nei = sysd["owner"], sysd["neighbour"]
    t0 = time.perf_counter()
    pd = O.dic_build(own, nei, sysd["diag"], sysd["upper"])
    t_dic = time.perf_counter() - t0
    x0 = np.zeros(sysd["n"])

    def solve(k):
        t = time.perf_counter()
        O.pcg(own, nei, sysd["diag"], sysd["lower"], sysd["upper"], sysd["b"], x0, pd, 0.0, 0.0,
              k, threads=threads)
        return time.perf_counter() - t

    t_short = solve(2)
    t_long = solve(2 + iters)
    t_it = max(t_long - t_short, 0.0) / iters
    t_setup = max(t_short - 2 * t_it, 0.0)
    return t_dic, t_it, t_setup, threads


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


# --------------------------------------------------------------------------
def headline_config(args, n: int, F: int, world: int) -> dict:
    """The workload both arms report, key for key."""
    return {"workload": WORKLOAD.replace("256^3", f"{args.n}^3"), "n_cells": n, "n_faces": F,
            "rel_tol": args.rel_tol, "rhs_seed": 2,
            "l2": "no flush: resident inputs (~1.9 GB at 256^3) exceed the 129 MB L2",
            "parallelism": f"replicas x{world}"}


def run_reference(args, rank, world):
    from oracle import oracle as O
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    if rank != 0:
        return
    sysd = hex_poisson(args.n, seed=2)
    threads = len(os.sched_getaffinity(0))
    full = None
    if not args.ref_sample_only:
        # one full FP64 solve to the tolerance: the iteration count the
        # samples extrapolate to, and a measured total to check them against
        t0 = time.perf_counter()
        pd = O.dic_build(sysd["owner"], sysd["neighbour"], sysd["diag"], sysd["upper"])
        o = O.pcg(sysd["owner"], sysd["neighbour"], sysd["diag"], sysd["lower"], sysd["upper"],
                  sysd["b"], np.zeros(sysd["n"]), pd, 0.0, args.rel_tol, 50000, threads=threads)
        full = {"s": time.perf_counter() - t0, "iterations": o.iterations,
                "converged": bool(o.converged)}
    samples = []
    for i in range(args.warmup + args.steps):
        t_dic, t_it, t_setup, threads = cpu_sample(sysd, iters=20)
        if i >= args.warmup:
            samples.append((t_dic, t_it, t_setup))
    t_dic = statistics.median(s[0] for s in samples)
    t_it = statistics.median(s[1] for s in samples)
    t_setup = statistics.median(s[2] for s in samples)
    n_it = full["iterations"] if full else None
    value = t_dic + t_setup + t_it * (n_it or 1)
    sample = (f"DIC factorisation + solves of 2 and 22 PCG iterations of the {args.n}^3 system "
              "per step (their difference gives the cost per iteration, the rest the per-call "
              "set-up), " + (f"extrapolated to the {n_it} iterations of one full solve of the "
                             "same port run first" if n_it else
                             "not extrapolated (--ref-sample-only): one iteration"))
    n, F = sysd["n"], int(sysd["owner"].shape[0])
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": headline_config(args, n, F, world),
        "solver": "oracle port of the reference PCG+DIC (FP64), all host cores",
        "extrapolated": bool(n_it), "sampled_iterations": 20,
        "timed_s_per_step": t_dic + 2 * t_setup + 24 * t_it,
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                         "sample": sample, "cpu": cpu_model(), "dic_build_s": t_dic,
                         "s_per_iteration": t_it, "setup_s": t_setup},
        "full_solve": full,
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if full:
        line["full_solve"]["extrapolation_rel_err"] = value / full["s"] - 1.0
    print(json.dumps(line), flush=True)


def _pinned_link_probe(dev, nbytes: int = 1 << 28, reps: int = 3) -> float:
    """GB/s of one pinned host -> device copy of ``nbytes`` (best of
    ``reps``), the link rate the e2e copies can reach on this machine."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    best = float("inf")
    for _ in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        d.copy_(h, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return nbytes / best / 1e9


def _host_placement(dev) -> dict:
    """Where this process runs relative to the GPU: the host CPUs it may use,
    the GPU's PCI NUMA node and the CPUs local to it (sysfs; empty where the
    platform does not say)."""
    out = {"cpus": len(os.sched_getaffinity(0))}
    try:
        p = torch.cuda.get_device_properties(dev)
        bus = f"{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
        base = f"/sys/bus/pci/devices/{bus}"
        with open(f"{base}/numa_node") as f:
            out["gpu_numa_node"] = int(f.read())
        with open(f"{base}/local_cpulist") as f:
            out["gpu_local_cpulist"] = f.read().strip()
    except (AttributeError, OSError, ValueError):
        pass
    return out


def run_ours(args, rank, world, local):
    import ctypes

    from pyopenfoam_gb300 import MixedPrecisionPCGSolver, PCGSolver, _lib
    from pyopenfoam_gb300.core.device import to_device, to_host
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    dev = torch.device("cuda", local)
    sysd = hex_poisson(args.n, seed=2)
    n, F = sysd["n"], int(sysd["owner"].shape[0])
    m = make_matrix(sysd, dev)
    b = torch.as_tensor(sysd["b"]).to(dev)
    x0 = torch.zeros(n, dtype=torch.float64, device=dev)
    L = _lib.lib()
    extra = {}

    kw = {} if args.storage == "auto" else {"symmetric_storage": args.storage == "symmetric"}
    mixed = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=args.rel_tol, max_iter=50000,
                                    preconditioner="DIC", delta=args.delta, **kw)

    def step():
        m.invalidate_cache()  # re-pack + re-factorise each solve, like the reference
        return mixed(m, b, x0)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    L.gbf_timing_enable(1, 100000)
    launches = 0
    iters = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            x, it, res = step()
            r = mixed.last_result
            iters.append(it)
            launches += r.launches
        e1.record()
        torch.cuda.synchronize()
    ms_total = e0.elapsed_time(e1)
    cnt, tot = ctypes.c_int32(), ctypes.c_double()
    _lib.check(L.gbf_timing_read(1, ctypes.byref(cnt), ctypes.byref(tot)))
    L.gbf_timing_enable(0, 0)
    # launches outside the solver loop: pack f64 + pack f32 + the DIC
    # factorisation (one cooperative launch)
    launches += args.steps * 3
    sec = max_over_ranks(ms_total / 1e3 / args.steps, world)
    barrier(world)

    # --- end to end through the public API with host buffers (right after
    # the device-timed steps, before the auxiliary measurements allocate) ---
    names = ("diag", "lower", "upper", "b")
    host = {k: torch.as_tensor(sysd[k]).pin_memory() for k in names}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = n * 8
    xs_host = torch.empty(n, dtype=torch.float64).pin_memory()
    link = None if args.no_e2e else _pinned_link_probe(dev)
    # each step hands the page-locked host arrays to the public API: the
    # LduMatrix setters and to_device upload them (by the SMs, over
    # NVLink-C2C; each returns when its copy is done), the solver runs, and
    # to_host reads x back into page-locked memory
    e2e_times, h2d_times, d2h_times = [], [], []
    per_copy, host_setters = {k: [] for k in names}, []
    for i in range(0 if args.no_e2e else args.warmup + args.steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 3)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev[0].record()
        m.diag = host["diag"]
        ev[1].record()  # stream-ordered after upload j: its device time alone
        m.lower = host["lower"]
        ev[2].record()
        m.upper = host["upper"]
        ev[3].record()
        bd = to_device(host["b"], dev, torch.float64)
        ev[4].record()
        t1 = time.perf_counter()
        xe, _, _ = mixed(m, bd, x0)
        ev[5].record()
        to_host(xe, xs_host)
        ev[6].record()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
            h2d_times.append(ev[0].elapsed_time(ev[4]) / 1e3)
            d2h_times.append(ev[5].elapsed_time(ev[6]) / 1e3)
            for j, k in enumerate(names):
                per_copy[k].append(ev[j].elapsed_time(ev[j + 1]) / 1e3)
            host_setters.append(t1 - t0)
    # median over the steps (one slow step -- a host-side stall -- moved the
    # mean by up to 10 %); the mean is reported beside it
    e2e = max_over_ranks(statistics.median(e2e_times), world) if e2e_times else None
    e2e_mean = max_over_ranks(statistics.mean(e2e_times), world) if e2e_times else None
    # the same loop with the copy engines (device buffers kept across steps,
    # torch copy_ from the same page-locked arrays), for comparison
    ce_times, ce_h2d = [], []
    if not args.no_e2e:
        dbuf = {k: torch.empty_like(t, device=dev) for k, t in host.items()}
        for i in range(1 + min(args.steps, 3)):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ev0.record()
            for k in names:
                dbuf[k].copy_(host[k], non_blocking=True)
            ev1.record()
            m.diag, m.lower, m.upper = dbuf["diag"], dbuf["lower"], dbuf["upper"]
            xe, _, _ = mixed(m, dbuf["b"], x0)
            xs_host.copy_(xe, non_blocking=True)
            torch.cuda.synchronize()
            if i > 0:
                ce_times.append(time.perf_counter() - t0)
                ce_h2d.append(ev0.elapsed_time(ev1) / 1e3)
        del dbuf

    # --- FP64 comparison: the same system, the same API, the same K steps ---
    x64 = None
    if not args.no_fp64:
        fp64 = PCGSolver(tolerance=0.0, rel_tol=args.rel_tol, max_iter=50000,
                         preconditioner="DIC")
        m.invalidate_cache()
        fp64(m, b, x0)  # one untimed solve (first launches, lazy module loading)
        f_times = []
        for _ in range(args.steps):
            m.invalidate_cache()
            torch.cuda.synchronize()
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record()
            x64, it64, res64 = fp64(m, b, x0)
            f1.record()
            torch.cuda.synchronize()
            f_times.append(f0.elapsed_time(f1) / 1e3)
        extra["fp64_pcg_s"] = statistics.mean(f_times)
        extra["fp64_pcg_s_min_max"] = [min(f_times), max(f_times)]
        extra["fp64_steps"] = len(f_times)
        extra["fp64_iterations"] = it64
        extra["fp64_true_rel_residual"] = true_rel_residual(m, x64, b)

    peaks = load_peaks()
    avg_ms = tot.value / max(cnt.value, 1)
    sym = mixed._symmetric_storage and m.packed_sym32() is not None
    topo = m.topology()
    design = design_bytes_ap(n, topo.n_slots, sym)
    achieved = design / (avg_ms * 1e-3) / 1e9
    survey = b_amul(4, n, F) / (avg_ms * 1e-3) / 1e9
    traffic = traffic_from_profile(design)
    extra["iterations"] = iters[-1]
    extra["inner_iterations_per_s"] = iters[-1] / sec
    extra["outer_updates"] = mixed.last_result.outer_updates
    extra["true_rel_residual"] = true_rel_residual(m, x, b)
    if x64 is not None:
        extra["x_rel_err_vs_fp64"] = float(torch.linalg.vector_norm(x - x64) /
                                           torch.linalg.vector_norm(x64))
        extra["speedup_vs_fp64"] = extra["fp64_pcg_s"] / sec
        extra["fp64_iterations_per_s"] = extra["fp64_iterations"] / extra["fp64_pcg_s"]
    extra["amul"] = time_amul(m, dev)

    cpu = None
    if rank == 0 and world >= 1 and not args.no_cpu:
        t_dic, t_it, t_setup, threads = cpu_sample(sysd, iters=20)
        n_it = extra.get("fp64_iterations") or iters[-1]
        cpu = {"value": t_dic + t_setup + t_it * n_it, "unit": "s", "cores": threads,
               "kind": "port",
               "sample": (f"oracle restatement of the reference PCG+DIC: DIC factorisation + "
                          f"threaded solves of 2 and 22 iterations at {args.n}^3 (cost per "
                          f"iteration from their difference), extrapolated to the {n_it} "
                          f"iterations of this run's FP64 GPU solve"),
               "extrapolated": True, "cpu": cpu_model(), "dic_build_s": t_dic,
               "s_per_iteration": t_it, "setup_s": t_setup}

    if rank == 0:
        line = {
            "metric": METRIC, "value": sec, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": headline_config(args, n, F, world),
            "solver": f"mixed FP32/FP64 reliable-update PCG+DIC, delta={args.delta}",
            "roofline": {"bound": "hbm",
                         "kernel": ("mp_ap_stream_kernel<%s> (FP32 Amul + p.Ap, bulk-copy "
                                    "staged)" % ("true: owner-side half of the symmetric matrix"
                                                 if sym else "false: both sides")),
                         "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                         "bytes_per_launch": design,
                         "bytes_formula": ("12n + 2*n_slots + 8.5*n_slots/32 (p, diag, Ap; "
                                           "owner-side slots; offset and mirror entries)" if sym
                                           else "12n + 4*n_slots + 8*n_slots/32 (p, diag, Ap; "
                                                "both slot sides; one {offset, mask} entry per "
                                                "32-slot column)"),
                         "n_slots": topo.n_slots,
                         "traffic": traffic["bytes"] if traffic else None,
                         "traffic_source": traffic,
                         "frac_survey_bytes": survey / peaks["hbm_gbs"],
                         "survey_bytes_per_launch": b_amul(4, n, F),
                         "survey_bytes_formula": "B_amul(4) = 12n + 16F (diag, x, y; lower, "
                                                 "upper; int32 owner, neighbour -- not read by "
                                                 "this kernel)",
                         "timed_launches": cnt.value, "avg_launch_us": avg_ms * 1e3},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "s", "statistic": "median of the timed steps",
                    "mean": e2e_mean, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "h2d_s_median": statistics.median(h2d_times) if h2d_times else None,
                    "h2d_s_per_array_median": {k: statistics.median(v) for k, v in
                                               per_copy.items()} if h2d_times else None,
                    "h2d_GBs": h2d / statistics.median(h2d_times) / 1e9 if h2d_times else None,
                    "d2h_s_median": statistics.median(d2h_times) if d2h_times else None,
                    "copies": "by the SMs over NVLink-C2C (gbf_copy_from_host / "
                              "gbf_copy_to_host) through the LduMatrix setters, to_device and "
                              "to_host, from and into page-locked host arrays",
                    "uploads_host_s_median": (statistics.median(host_setters)
                                              if host_setters else None),
                    "copy_engine_loop": {
                        "s_median": statistics.median(ce_times) if ce_times else None,
                        "h2d_s_median": statistics.median(ce_h2d) if ce_h2d else None,
                        "steps": len(ce_times),
                        "what": "the same loop with torch copy_ (copy engines) into kept "
                                "device buffers"},
                    "link_probe_GBs": link,
                    "link_probe": "one 256 MB copy-engine copy from page-locked memory, best "
                                  "of 4",
                    "host": _host_placement(dev)},
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "extra": extra,
        }
        print(json.dumps(line), flush=True)


def renumbered_system(N: int, seed: int = 2, perm_seed: int = 5) -> dict:
    """The N^3 Poisson system of the headline under a seeded random cell
    renumbering: cell c becomes perm[c]; every face is re-oriented so that
    owner < neighbour (lower and upper swapped with it) and the faces are
    re-sorted into upper-triangular (owner, neighbour) order.  The same
    matrix up to a symmetric permutation, but neighbour offsets are no longer
    uniform per slice, so the offset compression and the fixed 3 + 3 gather
    do not apply: the Amul reads an explicit int32 column per slot."""
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    d = hex_poisson(N, seed=seed)
    n = d["n"]
    perm = np.random.default_rng(perm_seed).permutation(n)
    own, nei = perm[d["owner"]], perm[d["neighbour"]]
    lo, up = d["lower"].copy(), d["upper"].copy()
    swap = own > nei
    own[swap], nei[swap] = nei[swap], own[swap]
    lo[swap], up[swap] = d["upper"][swap], d["lower"][swap]
    order = np.lexsort((nei, own))
    diag, b = np.empty(n), np.empty(n)
    diag[perm], b[perm] = d["diag"], d["b"]
    return {"n": n, "owner": np.ascontiguousarray(own[order]),
            "neighbour": np.ascontiguousarray(nei[order]),
            "lower": np.ascontiguousarray(lo[order]), "upper": np.ascontiguousarray(up[order]),
            "diag": diag, "b": b, "perm": perm}


def generic_layout_bytes(topo, s: int) -> int:
    """Bytes one Amul moves on a generic (not offset-uniform) layout: x,
    diagonal, y (s B per cell), one coefficient and one int32 column per
    slot, the 8 B {offset, mask} entry per 32-slot column (read to learn that
    the column is explicit) and the per-slice start and width."""
    return 3 * s * topo.n_cells + (s + 4) * topo.n_slots + 8 * (topo.n_slots // 32) \
        + 8 * topo.n_slices


def run_poisson256_renumbered(args, rank, world, local):
    """The headline system under a random cell renumbering: mixed-precision
    PCG+DIC to 1e-10 on the general gather path, with the Amul's roofline on
    the bytes that path moves."""
    import ctypes

    from pyopenfoam_gb300 import MixedPrecisionPCGSolver, PCGSolver, _lib

    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    sysd = renumbered_system(args.n)
    t_setup = time.perf_counter() - t0
    n, F = sysd["n"], int(sysd["owner"].shape[0])
    m = make_matrix(sysd, dev)
    b = torch.as_tensor(sysd["b"]).to(dev)
    x0 = torch.zeros(n, dtype=torch.float64, device=dev)
    topo = m.topology()
    L = _lib.lib()
    mixed = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=args.rel_tol, max_iter=50000,
                                    preconditioner="DIC", delta=args.delta)

    def step():
        m.invalidate_cache()
        return mixed(m, b, x0)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    L.gbf_timing_enable(1, 100000)
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            x, it, _ = step()
        e1.record()
        torch.cuda.synchronize()
    sec = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, world)
    cnt, tot = ctypes.c_int32(), ctypes.c_double()
    _lib.check(L.gbf_timing_read(1, ctypes.byref(cnt), ctypes.byref(tot)))
    L.gbf_timing_enable(0, 0)
    avg_s = tot.value / max(cnt.value, 1) / 1e3
    moved = generic_layout_bytes(topo, 4)
    peaks = load_peaks()
    extra = {"iterations": it, "outer_updates": mixed.last_result.outer_updates,
             "true_rel_residual": true_rel_residual(m, x, b), "setup_s": t_setup,
             "layout": {"n_slots": topo.n_slots, "slots_per_face": topo.n_slots / (2 * F),
                        "n_slices": topo.n_slices, "max_width": topo.max_width,
                        "offset_uniform_entries": topo.n_uniform_entries,
                        "slot_columns": topo.n_slots // 32,
                        "dic_levels": topo.dic_schedule().n_levels},
             "amul": time_amul(m, dev)}
    if not args.no_fp64:
        fp64 = PCGSolver(tolerance=0.0, rel_tol=args.rel_tol, max_iter=50000,
                         preconditioner="DIC")
        m.invalidate_cache()
        fp64(m, b, x0)
        m.invalidate_cache()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record()
        x64, it64, _ = fp64(m, b, x0)
        f1.record()
        torch.cuda.synchronize()
        extra.update(fp64_pcg_s=f0.elapsed_time(f1) / 1e3, fp64_iterations=it64,
                     speedup_vs_fp64=f0.elapsed_time(f1) / 1e3 / sec,
                     x_rel_err_vs_fp64=float(torch.linalg.vector_norm(x - x64) /
                                             torch.linalg.vector_norm(x64)))
    if rank == 0:
        _line(args, world, f"{args.n}^3 Poisson, random cell renumbering: mixed PCG+DIC to "
              f"{args.rel_tol:g} relative, time", sec, "s", False,
              {"workload": f"{args.n}^3 Poisson (unit-cube hex, x0 fixed value) under a seeded "
                           "random cell permutation (seed 5), faces in upper-triangular order",
               "n_cells": n, "n_faces": F, "rel_tol": args.rel_tol,
               "l2": "no flush: resident inputs exceed the 129 MB L2"},
              extra,
              roofline={"bound": "hbm", "kernel": "mp_ap_kernel<generic> (FP32 Amul + p.Ap, "
                                                  "explicit columns)",
                        "achieved": moved / avg_s / 1e9, "peak": peaks["hbm_gbs"],
                        "unit": "GB/s", "frac": moved / avg_s / 1e9 / peaks["hbm_gbs"],
                        "peak_source": peaks["source"], "bytes_per_launch": moved,
                        "bytes_formula": "12n + 8*n_slots + 8*n_slots/32 + 8*n_slices",
                        "traffic": None, "timed_launches": cnt.value,
                        "avg_launch_us": avg_s * 1e6},
              clocks=clk.summary())


def _line(args, world, metric, value, unit, hib, workload, extra, **kw):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
         "warmup": args.warmup, "ms_per_step": value * 1e3 if unit == "s" else None,
         "higher_is_better": hib, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
         "data": "synthetic", "config": workload}
    d.update(kw)
    d["extra"] = extra
    print(json.dumps(d), flush=True)


def run_poisson32(args, rank, world, local):
    """32^3 Poisson, PCG+DIC to 1e-6 relative (the reference's CPU case)."""
    from oracle import oracle as O
    from pyopenfoam_gb300 import PCGSolver
    from pyopenfoam_gb300.mesh.poisson import hex_poisson

    dev = torch.device("cuda", local)
    sysd = hex_poisson(32, seed=0)
    m = make_matrix(sysd, dev)
    b = torch.as_tensor(sysd["b"]).to(dev)
    x0 = torch.zeros_like(b)
    s = PCGSolver(tolerance=0.0, rel_tol=1e-6, max_iter=1000, preconditioner="DIC")
    ts = []
    for i in range(args.warmup + args.steps):
        m.invalidate_cache()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, it, res = s(m, b, x0)
        torch.cuda.synchronize()
        if i >= args.warmup:
            ts.append(time.perf_counter() - t0)
    gpu = max_over_ranks(statistics.median(ts), world)
    cpu = None
    if rank == 0:
        own, nei = sysd["owner"], sysd["neighbour"]
        t0 = time.perf_counter()
        pd = O.dic_build(own, nei, sysd["diag"], sysd["upper"])
        o = O.pcg(own, nei, sysd["diag"], sysd["lower"], sysd["upper"], sysd["b"],
                  np.zeros(sysd["n"]), pd, 0.0, 1e-6, 1000, threads=len(os.sched_getaffinity(0)))
        cpu = time.perf_counter() - t0
        _line(args, world, "32^3 Poisson PCG+DIC to 1e-6 relative residual, time",
              gpu, "s", False,
              {"workload": "32^3 Poisson (unit-cube hex, x0 fixed value), PCG+DIC to 1e-6",
               "n_cells": sysd["n"]},
              {"iterations": it, "oracle_iterations": o.iterations,
               "x_rel_err_vs_oracle": float(np.abs(x.cpu().numpy() - o.x).max() /
                                            np.abs(o.x).max())},
              cpu_baseline={"value": cpu, "unit": "s", "cores": len(os.sched_getaffinity(0)),
                            "kind": "port", "sample": "full solve"})


def convdiff_system(N: int, dev):
    """The convection-diffusion system: N^3 hex mesh with +-20 % jitter (seed 1), face diffusivity
    LogNormal(0, 1), upwind convection of u = (1, 0.5, 0.25) scaled to a cell
    Peclet number of ~10, fixed value on x = 0.  The flux uses the nominal
    (unjittered) face areas, so it is positive on every internal face and
    divergence free; the outflow boundary faces add F_b/V_P to the diagonal
    (what a zero-gradient outflow condition contributes to an upwind
    convection matrix -- the reference's fvm.div itself skips boundary
    faces, which leaves a closed box)."""
    from pyopenfoam_gb300 import LduMatrix
    from pyopenfoam_gb300.discretisation import fvm
    from pyopenfoam_gb300.mesh import HexMesh

    mesh = HexMesh(N, jitter=0.2, seed=1, device=dev)
    nominal = HexMesh(N)
    rng = np.random.default_rng(1)
    gamma = rng.lognormal(0.0, 1.0, mesh.n_faces)
    b = rng.uniform(-1.0, 1.0, mesh.n_cells)
    u = np.array([1.0, 0.5, 0.25])
    phi = (nominal.numpy("face_areas") * u).sum(axis=1) * (10.0 * N / np.linalg.norm(u))
    nint = mesh.n_internal_faces
    Lap = fvm.laplacian(torch.as_tensor(gamma), torch.zeros(1), mesh=mesh)
    Dv = fvm.div(torch.as_tensor(phi), torch.zeros(1), "Gauss upwind", mesh=mesh)
    own_b = mesh.numpy("owner")[nint:]
    V = mesh.numpy("cell_volumes")
    out_b = np.zeros(mesh.n_cells)
    np.add.at(out_b, own_b, np.where(phi[nint:] > 0.0, phi[nint:], 0.0) / V[own_b])
    A = LduMatrix(mesh.n_cells, Lap.owner, Lap.neighbour, device=dev)
    A.diag = Lap.diag - Dv.diag + torch.as_tensor(out_b).to(dev)
    A.lower = Lap.lower - Dv.lower
    A.upper = Lap.upper - Dv.upper
    return mesh, A, torch.as_tensor(b).to(dev)


def run_convdiff128(args, rank, world, local):
    """128^3 jittered convection-diffusion, PBiCGStab+DILU to 1e-8."""
    import ctypes

    from oracle import oracle as O
    from pyopenfoam_gb300 import MixedPrecisionPBiCGSTABSolver, PBiCGSTABSolver, _lib

    dev = torch.device("cuda", local)
    N = 128 if args.n == 256 else args.n
    t0 = time.perf_counter()
    mesh, A, b = convdiff_system(N, dev)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    L = _lib.lib()

    def timed(s):
        ts = []
        for i in range(args.warmup + args.steps):
            A.invalidate_cache()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            x, it, r = s(A, b, torch.zeros_like(b))
            torch.cuda.synchronize()
            if i >= args.warmup:
                ts.append(time.perf_counter() - t0)
        return x, it, statistics.median(ts)

    res = {}
    solvers = {
        "standard": PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-8, max_iter=4000, omega="standard"),
        "reference": PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-8, max_iter=4000,
                                     omega="reference"),
        "mixed": MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-8, max_iter=4000),
        "mixed_kernels": MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-8,
                                                       max_iter=4000, form="kernels"),
        "mixed_gather": MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-8, max_iter=4000,
                                                      form="gather"),
        "mixed_fused": MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-8, max_iter=4000,
                                                     form="fused"),
        "standard_1e-10": PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10, max_iter=4000,
                                          omega="standard"),
        "mixed_1e-10": MixedPrecisionPBiCGSTABSolver(tolerance=0.0, rel_tol=1e-10,
                                                     max_iter=4000),
    }
    wanted = [k for k in args.convdiff_legs.split(",") if k]
    for key in wanted:
        if key not in solvers:
            raise SystemExit(f"--convdiff-legs: unknown leg {key!r} (known: {', '.join(solvers)})")
    for key, s in solvers.items():
        if key not in wanted:
            continue
        mixed = key.startswith("mixed")
        if mixed:
            _lib.check(L.gbf_timing_enable(1, 4096))
        x, it, t = timed(s)
        res[key] = {"s": t, "converged": s.last_info.converged,
                    "true_rel_residual": true_rel_residual(A, x, b), "x": x}
        if mixed:
            R = s.last_result
            cnt, tot = ctypes.c_int32(0), ctypes.c_double(0.0)
            _lib.check(L.gbf_timing_read(4, ctypes.byref(cnt), ctypes.byref(tot)))
            _lib.check(L.gbf_timing_enable(0, 0))
            res[key].update(inner_iterations=R.inner_iterations, fp64_updates=R.outer_updates,
                            inner_iterations_per_s=R.inner_iterations / t,
                            k_v_us=(tot.value * 1e3 / cnt.value) if cnt.value else None)
        else:
            res[key].update(checks=it, iterations=(it - 1) / 2, iterations_per_s=(it - 1) / 2 / t)
    for key, ref in (("mixed", "standard"), ("mixed_kernels", "standard"),
                     ("mixed_gather", "standard"), ("mixed_fused", "standard"),
                     ("mixed_1e-10", "standard_1e-10")):
        if key not in res or ref not in res:
            continue
        res[key]["speedup_vs_fp64"] = res[ref]["s"] / res[key]["s"]
        res[key]["x_rel_err_vs_fp64"] = float(torch.linalg.vector_norm(res[key]["x"] - res[ref]["x"])
                                              / torch.linalg.vector_norm(res[ref]["x"]))
    head = "standard" if "standard" in res else wanted[0]
    cpu = None
    if rank == 0 and not args.no_cpu:
        own = A.owner.cpu().numpy()
        nei = A.neighbour.cpu().numpy()
        d, lo, up = A.diag.cpu().numpy(), A.lower.cpu().numpy(), A.upper.cpu().numpy()
        threads = len(os.sched_getaffinity(0))
        t0 = time.perf_counter()
        pd = O.dilu_build(own, nei, d, lo, up)
        o = O.pbicgstab(own, nei, d, lo, up, b.cpu().numpy(), np.zeros(mesh.n_cells), pd, 0.0,
                        1e-8, 4000, threads=threads, omega="standard")
        t_cpu = time.perf_counter() - t0
        xs = res[head]["x"].cpu().numpy()
        cpu = {"value": t_cpu, "unit": "s", "cores": threads, "kind": "port",
               "sample": "full solve (oracle PBiCGStab+DILU, standard omega)",
               "checks": o.iterations, "converged": o.converged,
               "x_rel_err_gpu_vs_oracle": float(np.abs(xs - o.x).max() / np.abs(o.x).max())}
        # at 1e-8 the GPU and the oracle stop on different trajectories (their
        # dot products round differently), so x agrees only to ~cond * 1e-8;
        # driven to 1e-14 both converge to the same x to ~1e-13
        tight = PBiCGSTABSolver(tolerance=0.0, rel_tol=1e-14, max_iter=4000, omega="standard")
        A.invalidate_cache()
        xt, itt, _ = tight(A, b, torch.zeros_like(b))
        ot = O.pbicgstab(own, nei, d, lo, up, b.cpu().numpy(), np.zeros(mesh.n_cells), pd, 0.0,
                         1e-14, 4000, threads=threads, omega="standard")
        cpu["x_rel_err_gpu_vs_oracle_both_at_1e-14"] = float(
            np.abs(xt.cpu().numpy() - ot.x).max() / np.abs(ot.x).max())
        cpu["converged_at_1e-14"] = [bool(tight.last_info.converged), bool(ot.converged)]
    for v in res.values():
        v.pop("x")
    if rank == 0:
        names = {"standard": "omega_standard", "reference": "omega_reference",
                 "mixed": "mixed_fp32_fp64", "mixed_kernels": "mixed_six_kernels_staged",
                 "mixed_gather": "mixed_six_kernels_gather",
                 "mixed_fused": "mixed_three_kernels_fused", "standard_1e-10": "fp64_to_1e-10",
                 "mixed_1e-10": "mixed_to_1e-10"}
        extra = {names[k]: v for k, v in res.items()}
        extra["setup_s"] = t_setup
        _line(args, world, f"128^3 jittered convection-diffusion, PBiCGStab+DILU "
              f"({head} leg) to 1e-{10 if head.endswith('1e-10') else 8} relative, time",
              res[head]["s"], "s", False,
              {"workload": f"{N}^3 hex, +-20% jitter, log-normal gamma, upwind Pe~10, outflow "
                           "boundary term", "n_cells": mesh.n_cells,
               "n_faces": mesh.n_internal_faces}, extra, cpu_baseline=cpu)


def run_batch64(args, rank, world, local):
    """64 independent Poisson systems (sides U{16..96}, seed 3), mixed
    FP32/FP64 refined PCG+DIC to 1e-8: the batched solve in its two forms --
    CUDA-graph replay of per-phase kernels and one persistent cooperative
    launch -- each with the autotuner's block and tile, against 64 sequential
    single-system solves; every system's x against an FP64 GPU PCG+DIC solve
    of the same system."""
    import ctypes

    from pyopenfoam_gb300 import MixedPrecisionPCGSolver, PCGSolver, _lib
    from pyopenfoam_gb300.mesh.batch import poisson_batch
    from pyopenfoam_gb300.solvers.batched import BatchedPCGSolver

    import tempfile

    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    mats, rhs, sides = poisson_batch(64, 16, 96, sigma=0.5, seed=3, device=dev)
    t_setup = time.perf_counter() - t0
    n_total = sum(m.n_cells for m in mats)
    # tune afresh in every run (a private cache file), so the timings are this box's
    os.environ["GBFOAM_AUTOTUNE_CACHE"] = os.path.join(tempfile.mkdtemp(), "autotune.json")
    auto = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=20000)
    t0 = time.perf_counter()
    auto.solve(mats, rhs)  # autotune (cached) + warm-up
    torch.cuda.synchronize()
    t_tune = time.perf_counter() - t0
    tuned = dict(auto.last_config)
    timings = tuned.pop("timings", None)

    forms = {}
    for form in ("graph", "persistent"):
        # the autotuner's best block and tile for this form (short fixed-iteration runs)
        cand = {k.split(":", 1)[1]: v for k, v in (timings or {}).items()
                if k.startswith(form + ":")}
        blk, tl, tpc = ((int(v) for v in min(cand, key=cand.get).split("x")) if cand
                        else (256, 4096, 1))
        bs = BatchedPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=20000, form=form,
                              block_size=blk, tile_cells=tl, wavefront=tuned["wavefront"],
                              threads_per_cell=tpc)
        bs.solve(mats, rhs)  # per-form tuning of block and tile (cached), warm-up
        for _ in range(max(args.warmup - 1, 0)):
            bs.solve(mats, rhs)
        ts = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = bs.solve(mats, rhs)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        cfg = {k: v for k, v in bs.last_config.items() if k != "timings"}
        forms[form] = {"s": max_over_ranks(statistics.median(ts), world), "config": cfg,
                       "out": out, "results": bs.last_results,
                       "converged": sum(i.converged for i in bs.last_infos)}
    head = tuned["form"] if tuned.get("form") in forms else "graph"
    t_batch = forms[head]["s"]
    out = forms[head]["out"]
    res = forms[head]["results"]
    same_bits = all(bool(torch.equal(a[0], b[0])) for a, b in
                    zip(forms["graph"]["out"], forms["persistent"]["out"])) \
        if all(forms["graph"]["config"][k] == forms["persistent"]["config"][k]
               for k in ("block", "tile", "tpc")) else None

    # every system against the FP64 GPU solver: same tolerance, and 1e-12
    errs, errs_tight, worst_true = [], [], 0.0
    f64 = PCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=20000, preconditioner="DIC")
    f64t = PCGSolver(tolerance=0.0, rel_tol=1e-12, max_iter=20000, preconditioner="DIC")
    for (x, _, _), m, b in zip(out, mats, rhs):
        xr, _, _ = f64(m, b, torch.zeros_like(b))
        xt, _, _ = f64t(m, b, torch.zeros_like(b))
        nr, nt = torch.linalg.vector_norm(xr), torch.linalg.vector_norm(xt)
        errs.append(float(torch.linalg.vector_norm(x - xr) / nr))
        errs_tight.append(float(torch.linalg.vector_norm(x - xt) / nt))
        worst_true = max(worst_true, true_rel_residual(m, x, b))

    # batched Amul roofline: plain launches with the timing probe, a fixed 64
    # iterations during which every system is still running
    L = _lib.lib()
    rb = BatchedPCGSolver(tolerance=0.0, rel_tol=0.0, max_iter=64, form="plain",
                          block_size=forms["graph"]["config"]["block"],
                          tile_cells=forms["graph"]["config"]["tile"],
                          wavefront=tuned["wavefront"],
                          threads_per_cell=forms["graph"]["config"]["tpc"])
    rb.solve(mats, rhs)
    _lib.check(L.gbf_timing_enable(1, 100000))
    rb.solve(mats, rhs)
    cnt, tot = ctypes.c_int32(), ctypes.c_double()
    _lib.check(L.gbf_timing_read(5, ctypes.byref(cnt), ctypes.byref(tot)))
    _lib.check(L.gbf_timing_enable(0, 0))
    topo = rb.layout(mats).matrix.topology()
    moved = design_bytes_ap(topo.n_cells, topo.n_slots, False)
    avg_s = tot.value / max(cnt.value, 1) / 1e3
    peaks = load_peaks()
    roof = {"bound": "hbm", "kernel": "bmp_ap_kernel (batched FP32 Amul + p.Ap, one tile per "
                                      "CTA, unstaged gather)",
            "achieved": moved / avg_s / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": moved / avg_s / 1e9 / peaks["hbm_gbs"], "peak_source": peaks["source"],
            "bytes_per_launch": moved,
            "bytes_formula": "12n + 4*n_slots + 8*n_slots/32 over the padded batch layout",
            "n_cells_padded": topo.n_cells, "n_slots": topo.n_slots, "traffic": None,
            "timed_launches": cnt.value, "avg_launch_us": avg_s * 1e6}

    single = MixedPrecisionPCGSolver(tolerance=0.0, rel_tol=1e-8, max_iter=20000)
    for m, b in zip(mats[:4], rhs[:4]):
        single(m, b, torch.zeros_like(b))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for m, b in zip(mats, rhs):
        m.invalidate_cache()
        single(m, b, torch.zeros_like(b))
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O

        threads = len(os.sched_getaffinity(0))
        host = [(m.owner.cpu().numpy(), m.neighbour.cpu().numpy(), m.diag.cpu().numpy(),
                 m.lower.cpu().numpy(), m.upper.cpu().numpy(), b.cpu().numpy())
                for m, b in zip(mats, rhs)]
        t0 = time.perf_counter()
        its = 0
        for own, nei, d, lo, up, bb in host:
            o = O.pcg(own, nei, d, lo, up, bb, np.zeros_like(bb), O.dic_build(own, nei, d, up),
                      0.0, 1e-8, 20000, threads=threads)
            its += o.iterations
        cpu = {"value": time.perf_counter() - t0, "unit": "s", "cores": threads, "kind": "port",
               "sample": "all 64 systems, one after another: the oracle's threaded FP64 "
                         "PCG+DIC (the reference's algorithm) to 1e-8, DIC factorisation "
                         "included", "iterations_total": its}
    if rank == 0:
        its = [r.iterations for r in res]
        _line(args, world, "64 uneven Poisson systems, batched mixed PCG+DIC to 1e-8, "
              "time", t_batch, "s", False,
              {"workload": "64 uniform hex Poisson systems, sides U{16..96} (seed 3), gamma "
                           "LogNormal(0,0.5), mixed FP32/FP64 refined to 1e-8",
               "n_cells": n_total, "sides": sides,
               "l2": "no flush: the batch (~1.2 GB of matrix and vectors) exceeds the 129 MB L2"},
              {"form": head, "autotuned": tuned, "autotune_timings": timings,
               "graph_replay_s": forms["graph"]["s"], "persistent_s": forms["persistent"]["s"],
               "graph_config": forms["graph"]["config"],
               "persistent_config": forms["persistent"]["config"],
               "forms_same_bits": same_bits,
               "sequential_s": t_seq, "speedup_vs_sequential": t_seq / t_batch,
               "converged": forms[head]["converged"], "worst_true_rel_residual": worst_true,
               "x_rel_err_vs_fp64_same_tol_max": max(errs),
               "x_rel_err_vs_fp64_same_tol_median": statistics.median(errs),
               "x_rel_err_vs_fp64_1e-12_max": max(errs_tight),
               "iterations_min_max": [min(its), max(its)],
               "setup_s": t_setup, "first_solve_incl_autotune_s": t_tune},
              roofline=roof, cpu_baseline=cpu)


def reference_gradient_24cube(dev) -> dict:
    """The 24^3 case of the adjoint workload against the gradient the
    reference itself computed (tests/golden/reference_unroll24.npz: its
    fvm.laplacian under autograd and DifferentiableLinearSolve per step, PCG
    to 1e-13 without preconditioner).  Inputs come from the same seeded
    draws; the target x_T(gamma') is computed here by the GPU solver."""
    from pyopenfoam_gb300 import PCGSolver
    from pyopenfoam_gb300.differentiable.unrolled import UnrolledImplicitDiffusion
    from pyopenfoam_gb300.mesh import HexMesh

    path = os.path.join(ROOT, "tests", "golden", "reference_unroll24.npz")
    if not os.path.exists(path):
        return {"unavailable": "fixture missing"}
    R = np.load(path)
    h = HexMesh(24)
    rng = np.random.default_rng(4)
    gamma = rng.lognormal(0.0, 1.0, h.n_faces)
    gamma2 = rng.lognormal(0.0, 1.0, h.n_faces)
    x0 = rng.uniform(0.0, 1.0, h.n_cells)
    sol = PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=5000, preconditioner="none")
    model = UnrolledImplicitDiffusion(h.to(dev), dt=1e-3, steps=20, checkpoint_every=5,
                                      solver=sol)
    T = lambda a: torch.as_tensor(a).to(dev)  # noqa: E731
    target = model.final_state(T(gamma2), T(x0))
    loss, grad = model.loss_and_grad(T(gamma), T(x0), target)
    g = grad.cpu().numpy()
    ref = R["grad_at_faces"]
    return {"n_cells": h.n_cells, "sampled_faces": int(R["faces"].shape[0]),
            "max_rel_err_sampled_faces": float(np.abs(g[R["faces"]] - ref).max()
                                               / np.abs(ref).max()),
            "grad_norm_rel_err": float(abs(np.linalg.norm(g) - float(R["grad_norm"]))
                                       / float(R["grad_norm"])),
            "loss_rel_err": float(abs(loss - float(R["loss"])) / float(R["loss"])),
            "reference_solver": "PCGSolver(tolerance=0, rel_tol=1e-13, preconditioner='none')"}


def reference_gradient_full_size(N: int, g: np.ndarray, loss: float) -> dict:
    """This run's gradient and loss against the gradient the reference itself
    computed on the same N^3 case (tests/golden/reference_unroll96.npz,
    sampled faces, norm and loss: its fvm.laplacian under autograd and
    DifferentiableLinearSolve per step, PCG to 1e-13 without
    preconditioner, on a target from the oracle)."""
    path = os.path.join(ROOT, "tests", "golden", f"reference_unroll{N}.npz")
    if not os.path.exists(path):
        return {"unavailable": f"no reference gradient fixture at {N}^3"}
    R = np.load(path)
    ref = R["grad_at_faces"]
    return {"n_cells": N ** 3, "sampled_faces": int(R["faces"].shape[0]),
            "max_rel_err_sampled_faces": float(np.abs(g[R["faces"]] - ref).max()
                                               / np.abs(ref).max()),
            "grad_norm_rel_err": float(abs(np.linalg.norm(g) - float(R["grad_norm"]))
                                       / float(R["grad_norm"])),
            "loss_rel_err": float(abs(loss - float(R["loss"])) / float(R["loss"])),
            "reference_solver": "PCGSolver(tolerance=0, rel_tol=1e-13, preconditioner='none')"}


def run_adjoint96(args, rank, world, local):
    """Adjoint gradient through 20 implicit diffusion steps at 96^3."""
    from pyopenfoam_gb300 import PCGSolver
    from pyopenfoam_gb300.differentiable.unrolled import UnrolledImplicitDiffusion
    from pyopenfoam_gb300.mesh import HexMesh

    dev = torch.device("cuda", local)
    N = 96 if args.n == 256 else args.n
    hm = HexMesh(N)
    mesh = hm.to(dev)
    rng = np.random.default_rng(4)
    gamma_h = rng.lognormal(0.0, 1.0, mesh.n_faces)
    gamma2_h = rng.lognormal(0.0, 1.0, mesh.n_faces)
    x0_h = rng.uniform(0.0, 1.0, mesh.n_cells)
    gamma, gamma2, x0 = (torch.as_tensor(a).to(dev) for a in (gamma_h, gamma2_h, x0_h))
    solver = PCGSolver(tolerance=0.0, rel_tol=1e-14, max_iter=50000, preconditioner="DIC")
    model = UnrolledImplicitDiffusion(mesh, dt=1e-3, steps=20, checkpoint_every=5, solver=solver)
    target = model.final_state(gamma2, x0)
    for _ in range(args.warmup):
        model.loss_and_grad(gamma, x0, target)
    fw, bw, peak = [], [], []
    for _ in range(args.steps):
        loss, grad = model.loss_and_grad(gamma, x0, target)
        fw.append(model.stats.forward_s)
        bw.append(model.stats.backward_s)
        peak.append(model.stats.peak_bytes)
    iters = model.stats.iterations
    full = UnrolledImplicitDiffusion(mesh, dt=1e-3, steps=20, checkpoint_every=1, solver=solver)
    full.loss_and_grad(gamma, x0, target)
    peak_all = full.stats.peak_bytes
    faces = rng.choice(mesh.n_faces, args.fd_faces, replace=False)
    errs = []
    t0 = time.perf_counter()
    for f in faces:
        fd = model.central_difference(gamma, x0, target, int(f), 1e-6)
        g = float(grad[f])
        errs.append(abs(fd - g) / max(abs(g), 1e-300))
    t_fd = time.perf_counter() - t0
    f_s, b_s = statistics.median(fw), statistics.median(bw)
    ref24 = reference_gradient_24cube(dev)
    ref_full = reference_gradient_full_size(N, grad.cpu().numpy(), loss)
    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = len(os.sched_getaffinity(0))
        from oracle.adjoint import unrolled_adjoint

        c_loss, c_grad, c_f, c_b = unrolled_adjoint(
            hm, gamma_h, x0_h, target.cpu().numpy(), 1e-3, 20, threads)
        gh = grad.cpu().numpy()
        cpu = {"value": c_f + c_b, "unit": "s", "cores": threads, "kind": "port",
               "sample": "full forward + backward (20 steps, all states kept) by the oracle's "
                         "threaded PCG+DIC and a numpy face gradient",
               "forward_s": c_f, "backward_s": c_b,
               "grad_rel_err_gpu_vs_cpu": float(np.abs(gh - c_grad).max() / np.abs(c_grad).max()),
               "loss_rel_err_gpu_vs_cpu": abs(loss - c_loss) / c_loss}
    if rank == 0:
        _line(args, world, "adjoint gradient of 20 implicit steps (96^3), "
              "forward + backward time", f_s + b_s, "s", False,
              {"workload": f"{N}^3 uniform hex, dt=1e-3, 20 steps, gamma ~ LogNormal(0,1) "
                           "per face, checkpoint every 5", "n_cells": mesh.n_cells,
               "n_faces": mesh.n_faces},
              {"forward_s": f_s, "backward_s": b_s, "backward_over_forward": b_s / f_s,
               "peak_bytes_checkpointed": statistics.median(peak),
               "peak_bytes_all_states": peak_all, "loss": loss,
               "solver_iterations_per_solve": statistics.mean(iters),
               "fd_faces": len(errs), "fd_h": 1e-6, "fd_max_rel_err": max(errs),
               "fd_median_rel_err": statistics.median(errs), "fd_seconds": t_fd,
               "reference_gradient_24cube": ref24, f"reference_gradient_{N}cube": ref_full},
              cpu_baseline=cpu)


def _event_time(fn, reps: int = 5, warmup: int = 2) -> float:
    """Mean seconds of fn() over `reps` calls, CUDA events on the current
    stream after `warmup` calls."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def run_next(args, rank, world, local):
    """The rows either side of the solve on one mesh: GPU FvMesh geometry
    of a jittered N^3 polyMesh (default 128^3) against the vectorised numpy
    restatement of the same formulas; the pressure correctors and Rhie-Chow
    fluxes on that mesh; GAMG and SmoothSolver on an N/2 cube Poisson
    system.  Times are CUDA-event means; bytes are the arrays each kernel
    reads and writes once (gathers of neighbour values counted once)."""
    from pyopenfoam_gb300 import LduMatrix
    from pyopenfoam_gb300.mesh import FvMesh, HexMesh
    from pyopenfoam_gb300.mesh.poisson import hex_poisson
    from pyopenfoam_gb300.solvers import GAMGSolver, SmoothSolver, rhie_chow
    from pyopenfoam_gb300.solvers.pressure_equation import correct_face_flux, correct_velocity

    dev = torch.device("cuda", local)
    N = 128 if args.n == 256 else args.n
    h = HexMesh(N, jitter=0.2, seed=1, geometry=False)
    d = h.polymesh()
    nf, ni, n = d["face_ptr"].shape[0] - 1, d["neighbour"].shape[0], h.n_cells
    out = {"n_cells": n, "n_faces": nf, "n_internal_faces": ni}
    m = FvMesh(d["points"], (d["face_ptr"], d["face_pts"]), d["owner"], d["neighbour"],
               d["boundary"], device=dev)
    m.compute_geometry()  # warm (addressing upload, module load)

    def geo():
        m._geo.clear()
        m.compute_geometry()

    t_geo = _event_time(geo, reps=3, warmup=1)
    geo_bytes = nf * (8 + 16 + 48) + d["points"].shape[0] * 24 + n * (24 + 32) + nf * 16
    t0 = time.perf_counter()
    HexMesh(N, jitter=0.2, seed=1)  # numpy restatement of the geometry formulas
    t_np = time.perf_counter() - t0
    out["geometry"] = {"gpu_s": t_geo, "cpu_numpy_s": t_np, "speedup": t_np / t_geo,
                       "bytes": geo_bytes, "GBs": geo_bytes / t_geo / 1e9}
    rng = np.random.default_rng(5)
    HbyA = torch.as_tensor(rng.normal(size=(n, 3))).to(dev)
    p = torch.as_tensor(rng.uniform(-1, 1, n)).to(dev)
    A = torch.as_tensor(rng.uniform(0.5, 2.0, n)).to(dev)
    phi = torch.as_tensor(rng.normal(size=nf)).to(dev)
    w = m.face_weights
    t_cv = _event_time(lambda: correct_velocity(HbyA, HbyA, p, A, m))
    t_cf = _event_time(lambda: correct_face_flux(phi, p, A, m, face_weights=w))
    own, nei, S, dl, V = m.owner, m.neighbour, m.face_areas, m.delta_coefficients, m.cell_volumes
    t_rc = _event_time(lambda: rhie_chow.compute_face_flux(HbyA, p, A, S, dl, own, nei, ni, V, w))
    cv_bytes = n * (24 + 8 + 8 + 8 + 24) + 2 * ni * (24 + 8) + (nf - ni) * 24
    ff_bytes = nf * (8 + 24 + 8 + 8 + 8) + n * (8 + 8)
    rc_bytes = nf * (8 + 24 + 8 + 8 + 8) + n * (24 + 8 + 8)
    out["correct_velocity"] = {"s": t_cv, "bytes": cv_bytes, "GBs": cv_bytes / t_cv / 1e9}
    out["correct_face_flux"] = {"s": t_cf, "bytes": ff_bytes, "GBs": ff_bytes / t_cf / 1e9}
    out["rhie_chow_face_flux"] = {"s": t_rc, "bytes": rc_bytes, "GBs": rc_bytes / t_rc / 1e9}
    if rank == 0 and not args.no_cpu:
        # the oracle's serial C restatement of the same formulas beside each
        # kernel (one core), and the GPU result against it bit for bit
        from oracle import oracle as O

        own_h, nei_h = own.cpu().numpy(), nei.cpu().numpy()
        S_h, dl_h, V_h, w_h = (a.cpu().numpy() for a in (S, dl, V, w))
        p_h, A_h, H_h, phi_h = (a.cpu().numpy() for a in (p, A, HbyA, phi))
        bits = lambda a: np.ascontiguousarray(a, np.float64).view(np.int64)  # noqa: E731
        legs = {
            "correct_velocity": (
                lambda: O.correct_velocity(n, own_h, nei_h, S_h, w_h, V_h, p_h, A_h, H_h),
                lambda: correct_velocity(HbyA, HbyA, p, A, m)),
            "correct_face_flux": (
                lambda: O.correct_face_flux(own_h, nei_h, phi_h, p_h, A_h, S_h, dl_h, w_h),
                lambda: correct_face_flux(phi, p, A, m, face_weights=w)),
            "rhie_chow_face_flux": (
                lambda: O.face_flux(own_h, nei_h, H_h, S_h, w_h, p_h, A_h, dl_h),
                lambda: rhie_chow.compute_face_flux(HbyA, p, A, S, dl, own, nei, ni, V, w)),
        }
        for key, (cpu_fn, gpu_fn) in legs.items():
            t0 = time.perf_counter()
            ref = cpu_fn()
            t_c = time.perf_counter() - t0
            out[key].update(cpu_oracle_s=t_c, cpu_cores=1, speedup_vs_cpu=t_c / out[key]["s"],
                            bitwise_vs_oracle=bool((bits(gpu_fn().cpu().numpy())
                                                    == bits(ref)).all()))

    Nm = max(N // 2, 8)
    sd = hex_poisson(Nm, seed=2)
    mm = LduMatrix(sd["n"], torch.as_tensor(sd["owner"]), torch.as_tensor(sd["neighbour"]),
                   device=dev)
    mm.diag, mm.lower, mm.upper = (torch.as_tensor(sd[k]) for k in ("diag", "lower", "upper"))
    b = torch.as_tensor(sd["b"]).to(dev)
    # a fixed number of V-cycles: the reference's GAMG (aggregation, smoother,
    # restriction -- reproduced here bit for bit) reduces the residual slowly
    # on this system (run on the CPU: 60 cycles reach 1.2e-3 at 8^3 and
    # 7.2e-3 at 16^3), so the leg reports time per cycle and the reduction
    g = GAMGSolver(tolerance=0.0, rel_tol=0.0, max_iter=50)
    t0 = time.perf_counter()
    g(mm, b, torch.zeros_like(b))
    torch.cuda.synchronize()
    t_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    x, it, res = g(mm, b, torch.zeros_like(b))
    torch.cuda.synchronize()
    t_g = time.perf_counter() - t0
    h = g.last_info.residual_history
    gamg_cpu = {}
    if rank == 0 and not args.no_cpu:
        # the oracle's serial restatement: hierarchy + the same 50 V-cycles
        from oracle import oracle as O

        t0 = time.perf_counter()
        xo, _, _ = O.gamg(sd["owner"], sd["neighbour"], sd["diag"], sd["lower"], sd["upper"],
                          sd["b"], np.zeros(sd["n"]), 50)
        t_o = time.perf_counter() - t0
        gamg_cpu = {"cpu_oracle_s_incl_hierarchy": t_o, "cpu_cores": 1,
                    "speedup_vs_cpu": t_o / t_first,
                    "bitwise_vs_oracle": bool((x.cpu().numpy().view(np.int64)
                                               == xo.view(np.int64)).all())}
    out["gamg"] = {"n_cells": sd["n"], "levels": [lv.n_cells for lv in g.last_levels],
                   # the monitor's first check follows the first cycle (as the reference's)
                   "v_cycles": it, "residual_reduction_after_cycle1": h[-1] / h[0],
                   "reduction_per_cycle": (h[-1] / h[0]) ** (1.0 / max(len(h) - 1, 1)),
                   "solve_s": t_g, "s_per_v_cycle": t_g / max(it, 1),
                   "first_solve_incl_hierarchy_s": t_first, **gamg_cpu}
    gs_cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O

        t0 = time.perf_counter()
        xg = O.gauss_seidel(sd["owner"], sd["neighbour"], sd["diag"], sd["lower"], sd["upper"],
                            sd["b"], np.zeros(sd["n"]), n_sweeps=1)
        gs_cpu = time.perf_counter() - t0
        from pyopenfoam_gb300.solvers.smoothers import gs_sweep

        xd = torch.zeros_like(b)
        gs_sweep(mm, xd, b)
        gs_bitwise = bool((xd.cpu().numpy().view(np.int64) == xg.view(np.int64)).all())
    sm = SmoothSolver(tolerance=0.0, rel_tol=0.0, max_iter=5, smoother="GaussSeidel",
                      n_sweeps=2)
    sm(mm, b, torch.zeros_like(b))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sm(mm, b, torch.zeros_like(b))
    torch.cuda.synchronize()
    t_s = time.perf_counter() - t0
    from pyopenfoam_gb300.solvers.smoothers import gs_sweep

    xs = torch.zeros_like(b)
    t_sw = _event_time(lambda: gs_sweep(mm, xs, b))
    out["smooth_gauss_seidel"] = {"n_cells": sd["n"], "sweeps": 10,
                                  "s_per_sweep_incl_checks": t_s / 10,
                                  "gpu_s_per_forward_sweep": t_sw}
    if gs_cpu is not None:
        out["smooth_gauss_seidel"].update(cpu_oracle_s_per_sweep=gs_cpu, cpu_cores=1,
                                          speedup_vs_cpu=gs_cpu / t_sw,
                                          bitwise_vs_oracle=gs_bitwise)
    if rank == 0:
        _line(args, world, f"rows next to the solve: GPU geometry, correctors, GAMG, smoothers "
              f"({N}^3 mesh)", t_geo, "s", False,
              {"workload": f"jittered {N}^3 hex polyMesh (geometry, correctors); {Nm}^3 Poisson "
                           "(GAMG, SmoothSolver)", "n_cells": n},
              out, cpu_baseline={"value": t_np, "unit": "s", "cores": 1, "kind": "port",
                                 "sample": "numpy restatement of the geometry formulas, same "
                                           "mesh (the reference's Python loops take hours)"})


def run_assembly(args, rank, world, local):
    """The operators on the path around the solve, each timed on the GPU
    (CUDA events) beside the oracle's serial C restatement of the same
    formulas (one core), with the GPU result compared bit for bit, on the
    jittered N^3 mesh (default 128^3): fvm.laplacian, fvm.div (upwind), the
    pressure-equation assembly, the DIC and DILU factorisations, the
    DifferentiableLaplacian forward + backward and the DifferentiableLinear-
    Solve gradient kernel.  Bytes are the arrays each operator reads and
    writes once."""
    from oracle import oracle as O
    from pyopenfoam_gb300 import DICPreconditioner, DILUPreconditioner, LduMatrix
    from pyopenfoam_gb300.differentiable import DifferentiableLaplacian, dls_grads
    from pyopenfoam_gb300.discretisation import fvm
    from pyopenfoam_gb300.mesh import HexMesh
    from pyopenfoam_gb300.solvers import assemble_pressure_equation

    dev = torch.device("cuda", local)
    N = 128 if args.n == 256 else args.n
    h = HexMesh(N, jitter=0.2, seed=1)
    m = h.to(dev)
    n, nf, ni = h.n_cells, h.n_faces, h.n_internal_faces
    own, nei = h.numpy("owner"), h.numpy("neighbour")
    S, dl, V = h.numpy("face_areas"), h.numpy("delta_coefficients"), h.numpy("cell_volumes")
    rng = np.random.default_rng(1)
    gamma = rng.lognormal(0.0, 1.0, nf)
    nominal = HexMesh(N)
    u = np.array([1.0, 0.5, 0.25])
    flux = (nominal.numpy("face_areas") * u).sum(axis=1) * (10.0 * N / np.linalg.norm(u))
    A_p = rng.uniform(0.5, 3.0, n)
    phiHbyA = rng.normal(0.0, 1.0, nf)
    w = O.centre_weights(own, nei, h.numpy("cell_centres"), h.numpy("face_centres"))
    phi_c, g_c = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    T = lambda a: torch.as_tensor(a).to(dev)  # noqa: E731
    bits = lambda a: np.ascontiguousarray(a, np.float64).view(np.int64)  # noqa: E731
    out = {"n_cells": n, "n_faces": nf, "n_internal_faces": ni}

    def leg(name, gpu_fn, cpu_fn, nbytes):
        t_g = _event_time(gpu_fn, reps=5, warmup=2)
        got = gpu_fn()
        rec = {"gpu_s": t_g, "bytes": nbytes, "GBs": nbytes / t_g / 1e9}
        if rank == 0 and not args.no_cpu:
            t0 = time.perf_counter()
            ref = cpu_fn()
            t_c = time.perf_counter() - t0
            same = all(bool((bits(a.detach().cpu().numpy()) == bits(b)).all())
                       for a, b in zip(got, ref))
            rec.update(cpu_oracle_s=t_c, cpu_cores=1, speedup_vs_cpu=t_c / t_g,
                       bitwise_vs_oracle=same)
        out[name] = rec

    gam = T(gamma)
    lap = lambda: fvm.laplacian(gam, torch.zeros(1), mesh=m)  # noqa: E731
    leg("fvm_laplacian", lambda: (lambda A: (A.lower, A.upper, A.diag))(lap()),
        lambda: O.laplacian(n, own, nei, S, dl, gamma, V),
        nf * (24 + 8 + 8 + 8) + ni * (8 + 8 + 16) + n * (8 + 8))
    fl = T(flux)
    leg("fvm_div_upwind",
        lambda: (lambda A: (A.lower, A.upper, A.diag))(fvm.div(fl, torch.zeros(1),
                                                                "Gauss upwind", mesh=m)),
        lambda: O.div_upwind(n, own[:ni], nei, flux[:ni], V),
        ni * (8 + 8 + 16 + 16) + n * (8 + 8))
    Ap, ph, wt = T(A_p), T(phiHbyA), T(w)
    leg("pressure_assembly",
        lambda: (lambda P: (P.lower, P.upper, P.diag, P.source))(
            assemble_pressure_equation(ph, Ap, m, face_weights=wt)),
        lambda: O.pressure_assemble(n, own, nei, S, dl, w, A_p, V, phiHbyA),
        nf * (24 + 8 + 8 + 8 + 8) + ni * (8 + 8 + 16 + 16) + n * (8 + 8 + 16))

    A = lap()
    own_i = own[:ni]
    lo_h, up_h, dg_h = (t.cpu().numpy() for t in (A.lower, A.upper, A.diag))
    def fresh(mat, cls):
        # drop the cached factorisation (kept per matrix) so that every call builds it
        for k in [k for k in mat._csr_cache if k[0] == cls.kind]:
            del mat._csr_cache[k]
        return (cls(mat).precond_diag,)

    # the default dataflow walk, and the barrier-per-level walk it replaced
    DICLevels = type("DICLevels", (DICPreconditioner,), {"factor_form": "levels"})
    DILULevels = type("DILULevels", (DILUPreconditioner,), {"factor_form": "levels"})
    leg("dic_factorisation", lambda: fresh(A, DICPreconditioner),
        lambda: (O.dic_build(own_i, nei, dg_h, up_h),), 16 * n + 16 * ni)
    leg("dic_factorisation_levels", lambda: fresh(A, DICLevels),
        lambda: (O.dic_build(own_i, nei, dg_h, up_h),), 16 * n + 16 * ni)
    D = fvm.div(fl, torch.zeros(1), "Gauss upwind", mesh=m)
    M = LduMatrix(n, A.owner, A.neighbour, device=dev)
    M.diag, M.lower, M.upper = A.diag - D.diag, A.lower - D.lower, A.upper - D.upper
    md, ml, mu = (t.cpu().numpy() for t in (M.diag, M.lower, M.upper))
    leg("dilu_factorisation", lambda: fresh(M, DILUPreconditioner),
        lambda: (O.dilu_build(own_i, nei, md, ml, mu),), 16 * n + 48 * ni)
    leg("dilu_factorisation_levels", lambda: fresh(M, DILULevels),
        lambda: (O.dilu_build(own_i, nei, md, ml, mu),), 16 * n + 48 * ni)

    def dlap():
        p_ = T(phi_c).requires_grad_(True)
        d_ = T(gamma).requires_grad_(True)
        y = DifferentiableLaplacian.apply(p_, d_, m)
        (y * T(g_c)).sum().backward()
        return y.detach(), p_.grad, d_.grad

    leg("differentiable_laplacian_fwd_bwd", dlap,
        lambda: (O.explicit_laplacian(n, own, nei, S, dl, gamma, V, phi_c),
                 O.explicit_laplacian(n, own, nei, S, dl, gamma, V, g_c),
                 O.explicit_laplacian_grad_d(own, nei, S, dl, V, phi_c, g_c)),
        3 * (nf * (24 + 8 + 8 + 16) + ni * 16) + n * 48)
    lam_h, x_h = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    lam, xx = T(lam_h), T(x_h)
    leg("dls_gradients", lambda: dls_grads(M, lam, xx),
        lambda: O.dls_grads(own_i, nei, lam_h, x_h), 24 * n + 48 * ni)
    if rank == 0:
        _line(args, world, f"operators around the solve on the {N}^3 jittered mesh: "
              f"fvm.laplacian time", out["fvm_laplacian"]["gpu_s"], "s", False,
              {"workload": f"{N}^3 hex, +-20% jitter: fvm.laplacian, fvm.div, pressure "
                           "assembly, DIC / DILU factorisation, DifferentiableLaplacian, "
                           "DLS gradients", "n_cells": n},
              out, cpu_baseline={"value": out["fvm_laplacian"].get("cpu_oracle_s"),
                                 "unit": "s", "cores": 1, "kind": "port",
                                 "sample": "the oracle's serial C restatement of each "
                                           "operator, same inputs (per-operator times in "
                                           "extra)"})


def main():
    args = parse()
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "poisson32":
        run_poisson32(args, rank, world, local)
    elif args.workload == "poisson256_renumbered":
        run_poisson256_renumbered(args, rank, world, local)
    elif args.workload == "convdiff128":
        run_convdiff128(args, rank, world, local)
    elif args.workload == "batch64":
        run_batch64(args, rank, world, local)
    elif args.workload == "adjoint96":
        run_adjoint96(args, rank, world, local)
    elif args.workload == "next":
        run_next(args, rank, world, local)
    elif args.workload == "assembly":
        run_assembly(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
