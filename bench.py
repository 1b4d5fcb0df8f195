"""Benchmark of the TeaLeaf implicit solve on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload ppcg4096|cheby4096|cg4096|cg512]

A step is one TeaLeaf timestep (one tea_leaf call: set-up, the solve to
tl_eps, finalise) of a synthetic five-state problem with the reference's
deck layout.  The default workload is 4096^2 cells, PPCG with the 4-row
block-Jacobi preconditioner, 10 inner steps, halo depth 2, 20 CG steps
before the switch, tl_eps 1e-15, FP64.  W untimed steps run first (the
first contains the CG steps and the eigenvalue estimate); K steps are timed
with CUDA events on the library's stream.

value : cell-iterations/s (interior cells x solver iterations / s, counting
        outer plus PPCG inner iterations as the reference's "Total" count
        does) with the fields resident in HBM, through the library's
        fastest driver mode.
e2e   : the same metric through the per-call C ABI (two host round trips
        per CG iteration, as the reference's Fortran makes them), with each
        step's input fields (density, energy1) copied host->device from
        pinned memory and the result field (energy1) copied back inside the
        timed region.
mixed : FP64 CG and FP32-inner / FP64-refined CG to the same 1e-10
        relative FP64 residual at 4096^2 (diagonal Jacobi), 3 timesteps:
        their wall times and ratio, final recomputed residuals and the
        field_summary difference (--no-mixed leaves it out).
--impl reference times the CPU restatement of the reference (oracle/) on
the host cores, all threads, on bounded samples of the same workload: the
first (warm-up) step runs its CG iterations to the switch and the
eigenvalue estimate, and every PPCG or Chebyshev step ends
--cpu-cap-after-switch iterations after its switch, so the timed steps
are PPCG outer iterations with their inner steps, as on the GPU (CG
workloads: each step capped at --cpu-cap iterations).

Multi-GPU (torchrun): every rank solves its own copy of the problem
(replicas; the solve is not sharded), value = all ranks' cell-iterations /
max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (cells, solver, prec, halo, inner, presteps, eps, dominant kernel,
    #        algorithmic bytes per cell of one launch of it)
    "ppcg4096": (4096, "ppcg", "jac_block", 2, 10, 20, 1e-15,
                 "tea_leaf_ppcg_solve_inner_step", 112),
    "cheby4096": (4096, "chebyshev", "jac_block", 2, 10, 20, 1e-15,
                  "tea_leaf_cheby_solve_calc_p_u", 104),
    "cg4096": (4096, "cg", "jac_block", 2, 10, 20, 1e-15,
               "tea_leaf_cg_solve_calc_ur", 88),
    "cg512": (512, "cg", "jac_diag", 1, 10, 25, 1e-15,
              "tea_leaf_cg_solve_calc_ur", 64),
}


ARITHMETIC = "chain"  # set from --arithmetic in main()

# FP64-pipe instructions per interior cell of one launch of the dominant
# kernel, counted from its source (products done on the integer pipes are
# not counted): update_r is r - A sd plus u + sd (chain: 5 fused
# multiply-adds and an add; fused: 4 + 1 + 1; exact: 7 + 1 + 1); calc_ur
# with diagonal Jacobi is u + alpha p, r - alpha w, z = Mi r, r.z (4 when
# fused, 7 when exact) and with block Jacobi adds 2.5 for the strip sweep
# instead of 1 for z (5.5 when fused).  These kernels are bound by GB300's
# FP64 pipe, not by HBM.
FP64_PER_CELL = {
    # two inner steps of update_r + calc_sd (6 + 2.5 each in the fused forms)
    ("tea_leaf_ppcg_solve_inner_pair", "jac_block", "chain"): 17,
    ("tea_leaf_ppcg_solve_inner_pair", "jac_block", "fused"): 17,
    # one inner step in one pass: update_r 6 + calc_sd 3.5
    ("tea_leaf_ppcg_solve_inner_step", "jac_block", "chain"): 9.5,
    ("tea_leaf_ppcg_solve_inner_step", "jac_block", "fused"): 9.5,
    ("tea_leaf_ppcg_solve_update_r", "jac_block", "chain"): 6,
    ("tea_leaf_ppcg_solve_update_r", "jac_block", "fused"): 6,
    ("tea_leaf_ppcg_solve_update_r", "jac_block", "exact"): 9,
    ("tea_leaf_cg_solve_calc_ur", "jac_diag", "chain"): 4,
    ("tea_leaf_cg_solve_calc_ur", "jac_diag", "fused"): 4,
    ("tea_leaf_cg_solve_calc_ur", "jac_diag", "exact"): 7,
    ("tea_leaf_cg_solve_calc_ur", "jac_block", "chain"): 5.5,
    ("tea_leaf_cg_solve_calc_ur", "jac_block", "fused"): 5.5,
    # the Chebyshev step: operator 5 (chain) or 6 (fused), r = u0 - w 1,
    # strip sweep 2.5, alpha p + beta z 1 (beta z on the integer pipes)
    ("tea_leaf_cheby_solve_calc_p", "jac_block", "chain"): 9.5,
    ("tea_leaf_cheby_solve_calc_p", "jac_block", "fused"): 10.5,
    # the same with calc_u's u + p folded in
    ("tea_leaf_cheby_solve_calc_p_u", "jac_block", "chain"): 10.5,
    ("tea_leaf_cheby_solve_calc_p_u", "jac_block", "fused"): 11.5,
}


def deck_for(name, steps):
    from tealeaf_opencl_gb300 import decks
    cells, solver, prec, halo, inner, presteps, eps = WORKLOADS[name][:7]
    # the 512^2 CG configuration names tl_max_iters 5000; the 4096^2 one
    # names none, so the reference's default of 1000 (read_input.f90:59)
    # applies
    max_iters = 5000 if cells <= 512 else 1000
    return decks.five_state_deck(cells, solver=solver, prec=prec, steps=steps,
                                 eps=eps, max_iters=max_iters, halo=halo,
                                 inner_steps=inner, presteps=presteps,
                                 summary_frequency=0,
                                 extra="tl_arithmetic %s" % ARITHMETIC)


def config_for(name):
    cells, solver, prec, halo, inner, presteps, eps = WORKLOADS[name][:7]
    cfg = {"workload": "%s: %dx%d five-state TeaLeaf, %s + %s, FP64, tl_eps %g"
                       % (name, cells, cells, solver, prec, eps),
           "cells": cells * cells, "solver": solver, "preconditioner": prec,
           "halo_depth": halo, "tl_eps": eps, "dt": 0.004,
           "domain": "[0,10]^2, five reference states",
           "l2": "inputs larger than L2: each FP64 field is %.0f MB, the "
                 "solve touches about 12 of them" % (cells * cells * 8 / 1e6),
           "arithmetic": ARITHMETIC,
           "iteration_count": "outer + PPCG inner (the reference's 'Total')",
           "parallelism": "replicas",
           "tl_max_iters": 5000 if cells <= 512 else 1000}
    if solver == "ppcg":
        cfg["inner_steps"] = inner
    if solver in ("ppcg", "chebyshev"):
        cfg["cg_presteps"] = presteps
    return cfg


# ---------------------------------------------------------------------------
# distributed helpers (replicas)
# ---------------------------------------------------------------------------

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            backend = os.environ.get("TEA_DIST_BACKEND", "gloo")
            td.init_process_group(backend=backend)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        return self.reduce(v, "max")

    def sum(self, v):
        return self.reduce(v, "sum")

    def reduce(self, v, op):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def step_bytes_per_cell_iteration(name):
    """Algorithmic HBM bytes per cell-iteration of a whole solver iteration:
    the fields the reference's kernels read and write, each once
    (KERNEL_BYTES), summed over the kernels of one iteration and divided by
    the cell-iterations it counts (PPCG: one outer plus its inner steps)."""
    cells, solver, prec, halo, inner = WORKLOADS[name][:5]
    kb = lambda k: KERNEL_BYTES[k][prec] if isinstance(KERNEL_BYTES[k], dict) else KERNEL_BYTES[k]
    cg = kb("tea_leaf_cg_solve_calc_w") + kb("tea_leaf_cg_solve_calc_ur") + \
        kb("tea_leaf_cg_solve_calc_p")
    if solver == "cg":
        return cg
    if solver == "chebyshev":
        return kb("tea_leaf_cheby_solve_calc_p") + kb("tea_leaf_cheby_solve_calc_u")
    # PPCG: calc_w, calc_ur, init_sd, the inner steps, r.z, calc_p
    outer = cg + kb("tea_leaf_ppcg_solve_init_sd") + kb("tea_leaf_calc_2norm") + inner * (
        kb("tea_leaf_ppcg_solve_update_r") + kb("tea_leaf_ppcg_solve_calc_sd"))
    return outer / (1 + inner)


def whole_job_rate(dist, cell_iters, seconds):
    """Cell-iterations per second of the whole job: every rank's count
    summed, over the slowest rank's time (replicas run the same work)."""
    return dist.sum(cell_iters) / dist.max(seconds)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------

class Clocks:
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.loads(Path(path).read_text())["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel, workload):
    """DRAM bytes per launch of the kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        return json.loads(Path(path).read_text())[workload][kernel]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def run_ours(args, dist):
    import ctypes
    import numpy as np
    from tealeaf_opencl_gb300 import lib

    L = lib.load()
    L.tea_gb300_set_inner_pairs(args.inner_pairs)
    name = args.workload
    cells = WORKLOADS[name][0]
    ncell = cells * cells
    kernel, bytes_per_cell = WORKLOADS[name][7], WORKLOADS[name][8]
    if args.inner_pairs and WORKLOADS[name][1] == "ppcg" and WORKLOADS[name][2] == "jac_block":
        # two inner steps per launch: reads u r sd Kx Ky diag cp bfp, writes u r sd
        kernel, bytes_per_cell = "tea_leaf_ppcg_solve_inner_pair", 88
    steps_total = args.warmup + args.steps
    deck = deck_for(name, steps_total)

    # ---- value: fields resident in HBM, fastest driver mode ----
    drv = lib.Driver(deck, mode=lib.DRIVER_RESIDENT, max_iters_cap=args.cap)
    for _ in range(args.warmup):
        drv.step()
    clocks = Clocks(0)
    dist.barrier()
    L.tea_gb300_synchronize()
    launches0 = L.tea_gb300_kernel_launches()
    clocks.start()
    t0 = time.perf_counter()
    L.tea_gb300_event_record(0)
    infos = [drv.step() for _ in range(args.steps)]
    L.tea_gb300_event_record(1)
    L.tea_gb300_synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dist.barrier()
    ms = float(L.tea_gb300_event_elapsed_ms(0, 1))
    launches = L.tea_gb300_kernel_launches() - launches0
    drv.close()
    outer = sum(i.iterations for i in infos)
    inner = sum(i.inner_iterations for i in infos)
    ms_max = dist.max(ms)
    value = whole_job_rate(dist, (outer + inner) * ncell, ms / 1e3)

    # ---- e2e: per-call C ABI, host buffers, copies inside the timed region ----
    drv = lib.Driver(deck, mode=lib.DRIVER_PER_CALL, max_iters_cap=args.cap)
    for _ in range(args.warmup):
        drv.step()
    nbytes = ncell * 8
    bufs = [L.tea_gb300_host_alloc(nbytes) for _ in range(3)]
    host = [np.ctypeslib.as_array(ctypes.cast(b, ctypes.POINTER(ctypes.c_double)),
                                  shape=(cells, cells)) for b in bufs]
    chunk_read = lambda f, a: L.tea_gb300_read_field(lib.FIELD[f], a.ctypes.data_as(lib.PD))
    chunk_write = lambda f, a: L.tea_gb300_write_field(lib.FIELD[f], a.ctypes.data_as(lib.PD))
    chunk_read("density", host[0])
    chunk_read("energy1", host[1])
    # the dominant kernel's launches are timed with CUDA events during this
    # pass: the per-call path launches it on its own (the resident loop
    # replays it inside graphs)
    L.tea_gb300_kernel_timer_select(kernel.encode())
    dist.barrier()
    L.tea_gb300_synchronize()
    t0 = time.perf_counter()
    e2e_outer = 0
    for _ in range(args.steps):
        chunk_write("density", host[0])
        chunk_write("energy1", host[1])
        info = drv.step()
        chunk_read("energy1", host[2])
        host[1][...] = host[2]
        e2e_outer += info.iterations + info.inner_iterations
    L.tea_gb300_synchronize()
    e2e_s = time.perf_counter() - t0
    kms, kn = ctypes.c_double(), ctypes.c_longlong()
    L.tea_gb300_kernel_timer_read(ctypes.byref(kms), ctypes.byref(kn))
    L.tea_gb300_kernel_timer_select(b"")
    dist.barrier()
    drv.close()
    for b in bufs:
        L.tea_gb300_host_free(b)
    e2e_value = whole_job_rate(dist, e2e_outer * ncell, e2e_s)

    peak, peak_kind = measured_peak_hbm()
    avg_launch_ms = kms.value / kn.value if kn.value else None
    achieved = (bytes_per_cell * ncell / (avg_launch_ms / 1e3) / 1e9
                if avg_launch_ms else None)
    traffic = ncu_traffic(kernel, name)
    fp64_n = FP64_PER_CELL.get((kernel, WORKLOADS[name][2], ARITHMETIC))
    fp64 = None
    if fp64_n is not None and avg_launch_ms:
        rate = float(L.tea_gb300_fp64_rate())  # measured FP64 FMA/s, after the timed regions
        done = fp64_n * ncell / (avg_launch_ms / 1e3)
        fp64 = {"instructions_per_cell": fp64_n, "achieved_per_s": done,
                "peak_per_s": rate, "peak_kind": "measured: 8 independent FMA chains per thread",
                "frac": done / rate if rate > 0 else None}
    out = {
        "metric": "TeaLeaf %s cell-iterations/s at %dx%d (FP64)" % (WORKLOADS[name][1].upper(), cells, cells),
        "value": value,
        "unit": "cell-iters/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: five-state layout of the reference's decks",
        "config": config_for(name),
        "iterations": {"outer": outer, "ppcg_inner": inner,
                       "per_step": [i.iterations for i in infos]},
        "outer_cell_iters_per_s": dist.sum(outer) * ncell / (ms_max / 1e3),
        "wall_s": wall,
        "e2e": {"value": e2e_value, "unit": "cell-iters/s",
                "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": nbytes,
                "path": "per-call C ABI (host scalars), pinned host fields"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": kernel,
                     "achieved": achieved, "peak": peak,
                     "peak_kind": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind
                     if peak_kind == "measured" else "fallback",
                     "unit": "GB/s",
                     "frac": achieved / peak if achieved else None,
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": bytes_per_cell * ncell,
                     "avg_launch_ms": avg_launch_ms, "launches_timed": kn.value,
                     "fp64_pipe": fp64},
        "clocks": clk,
    }
    bpc = step_bytes_per_cell_iteration(name)
    out["step_hbm"] = {
        "algorithmic_bytes_per_cell_iteration": bpc,
        "gbs": value * bpc / 1e9, "peak": peak,
        "frac": value * bpc / 1e9 / peak if peak else None,
        "unit": "GB/s",
        "basis": "the reference kernels' fields per solver iteration, each once, "
                 "over the resident timed region"}
    return out


# algorithmic bytes per interior cell of each entry point's kernels: the
# fields the reference kernel reads and writes, each once, FP64
KERNEL_BYTES = {
    "tea_leaf_cg_solve_calc_w": 32,       # r p Kx Ky, w w
    "tea_leaf_cg_solve_calc_ur": {"jac_diag": 64, "jac_block": 88, "none": 56},
    "tea_leaf_cg_solve_calc_p": 24,       # r z p, w p
    "tea_leaf_calc_2norm": 16,
    "tea_leaf_ppcg_solve_update_r": 56,   # r u r Kx Ky sd, w u r
    # update_r and calc_sd in one pass (block Jacobi): the two kernels' fields
    "tea_leaf_ppcg_solve_inner_step": {"jac_diag": 88, "jac_block": 112, "none": 80},
    "tea_leaf_ppcg_solve_inner_pair": 88,  # two steps: r u r sd Kx Ky diag cp bfp, w u r sd
    "tea_leaf_ppcg_solve_calc_sd": {"jac_diag": 32, "jac_block": 56, "none": 24},
    "tea_leaf_cheby_solve_calc_p": {"jac_diag": 80, "jac_block": 96, "none": 72},
    "tea_leaf_cheby_solve_calc_u": 24,
    # calc_p and calc_u in one pass (block Jacobi): calc_p's fields and u written
    "tea_leaf_cheby_solve_calc_p_u": {"jac_diag": 88, "jac_block": 104, "none": 80},
    "tea_leaf_calc_residual": 48,         # u0 u Kx Ky (diag), r
    "tea_leaf_cg_solve_init_p": {"jac_diag": 32, "jac_block": 56, "none": 24},
    "tea_leaf_ppcg_solve_init_sd": {"jac_diag": 24, "jac_block": 48, "none": 16},
    "tea_leaf_cheby_solve_init_p": {"jac_diag": 72, "jac_block": 88, "none": 64},
    "tea_leaf_jacobi_copy_u": 16,         # u, un
    "tea_leaf_jacobi_solve": 48,          # u0 un Kx Ky, u
    "tea_leaf_finalise": 24,              # u density, energy1
    "field_summary": 32,                  # volume density energy1 u
    "tea_leaf_init_common": 24,           # density, Kx Ky
    "tea_leaf_init_diag": 24,             # Kx Ky, diag
    "generate_chunk_init_u": 32,          # energy1 density, u u0
    "tea_leaf_block_init": 40,            # Kx Ky diag, cp bfp
    "update_halo": 0,                     # halo cells only
}


def run_kernels(args):
    """Each hot entry point called repeatedly on the workload's grid; every
    kernel timed with CUDA events (non-serialising)."""
    import ctypes
    from tealeaf_opencl_gb300 import decks, lib
    L = lib.load()
    L.tea_gb300_set_inner_pairs(args.inner_pairs)
    name = args.workload
    cells, solver, prec, halo = WORKLOADS[name][:4]
    ch = lib.Chunk(cells, cells, halo, "ppcg", prec)
    ch.set_arithmetic(ARITHMETIC)
    decks.setup_five_state(ch, cells)
    ch.common_init(1, 0.004)
    ch.calc_residual()
    reps = args.reps
    L.tea_gb300_kernel_timer_select(b"*")
    rro = ch.cg_init()
    for _ in range(reps):
        pw = ch.cg_calc_w()
        rrn = ch.cg_calc_ur(rro / pw)
        ch.cg_calc_p(rrn / rro)
        rro = rrn
        ch.calc_2norm(2)
    a, b_, theta = decks.chebyshev_coefficients(1.0, 60.0, reps + 1)
    ch.ppcg_init(a, b_, theta)
    ch.ppcg_init_sd()
    for s in range(1, reps + 1):
        ch.ppcg_inner(s)
    ch.cheby_init(a, b_, theta)
    for s in range(1, reps + 1):
        ch.cheby_iterate(s)
    for _ in range(reps):
        ch.calc_residual()
        ch.jacobi_solve()
        ch.finalise()
        ch.field_summary()
        ch.update_halo([1, 1, 1, 0, 0, 0, 0], halo)
        ch.common_init(1, 0.004)
        ch.cg_init()
    L.tea_gb300_synchronize()
    peak, kind = measured_peak_hbm()
    ncell = cells * cells
    out = {"mode": "kernels", "workload": name, "cells": ncell, "reps": reps,
           "arithmetic": ARITHMETIC, "peak_gbs": peak, "peak_kind": kind,
           "fp64_fma_per_s": L.tea_gb300_fp64_rate(), "kernels": {}}
    for kname, per in KERNEL_BYTES.items():
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        L.tea_gb300_kernel_timer_read_name(kname.encode(), ctypes.byref(ms), ctypes.byref(n))
        if not n.value:
            continue
        bpc = per[prec] if isinstance(per, dict) else per
        avg = ms.value / n.value
        gbs = bpc * ncell / (avg / 1e3) / 1e9 if bpc else None  # update_halo: halo only
        out["kernels"][kname] = {"launches": n.value, "avg_us": 1e3 * avg,
                                 "bytes_per_cell": bpc, "achieved_gbs": gbs,
                                 "frac": gbs / peak if gbs else None}
    L.tea_gb300_kernel_timer_select(b"")
    return out


def lognormal_factor(n, sigma=0.5, corr=8.0, seed=2024):
    """exp(sigma g) for a unit-variance Gaussian field g with correlation
    exp(-d^2 / (2 corr^2)): seeded white noise filtered by a Gaussian of
    width corr/sqrt(2) (spectrally), then renormalised."""
    import numpy as np
    rng = np.random.Generator(np.random.Philox(seed))
    w = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n)
    s = corr / np.sqrt(2.0)
    gk = np.exp(-2.0 * (np.pi * s) ** 2 * (k[:, None] ** 2 + k[None, :] ** 2))
    g = np.fft.ifft2(np.fft.fft2(w) * gk).real
    g = (g - g.mean()) / g.std()
    return np.exp(sigma * g)


def run_mixed(args):
    """FP64 CG and FP32-inner/FP64-refined CG to the same true relative
    FP64 residual (1e-10), on the same problem; wall time per timestep."""
    return mixed_compare(args.cells, args.steps, args.lognormal, args.mixed_solver,
                         args.inner_steps, args.presteps)


MIXED_DEFAULT_STEPS = 3


def mixed_summary(args):
    """The mixed-precision comparison on the default line: 4096^2, the
    five-state problem, CG + diagonal Jacobi, both solves to a 1e-10
    relative FP64 residual, MIXED_DEFAULT_STEPS timesteps (the full
    precision configuration is --mode mixed --cells 8192 --lognormal
    --steps 10)."""
    r = mixed_compare(4096, MIXED_DEFAULT_STEPS, False, "cg", 10, 25)
    return {"cells": r["cells"], "steps": r["steps"], "tol": r["tol"],
            "solver": "CG + jac_diag; mixed: FP32 inner CG in FP64 defect correction",
            "fp64_seconds": r["fp64"]["seconds"], "mixed_seconds": r["mixed"]["seconds"],
            "time_ratio_mixed_over_fp64": r["time_ratio_mixed_over_fp64"],
            "fp64_final_relative_residual": r["fp64"]["relative_residual"],
            "mixed_final_relative_residual": r["mixed"]["relative_residual"],
            "field_summary_rel_diff": r["field_summary_rel_diff"],
            "fp64_iterations": r["fp64"]["iterations"],
            "mixed_fp32_iterations": r["mixed"]["iterations"],
            "mixed_corrections": r["mixed"]["corrections"],
            "fp64_arithmetic": r["fp64_arithmetic"],
            "timing": "wall time per timestep, CUDA-synchronised, summed"}


def deck_rate(deck, warm_steps, timed_steps, mode):
    """Runs warm_steps untimed then timed_steps timesteps of a deck on the
    GPU driver; cell-iterations/s (outer + inner) with CUDA events."""
    from tealeaf_opencl_gb300 import lib
    L = lib.load()
    drv = lib.Driver(deck, mode=mode)
    for _ in range(warm_steps):
        drv.step()
    L.tea_gb300_synchronize()
    L.tea_gb300_event_record(2)
    infos = [drv.step() for _ in range(timed_steps)]
    L.tea_gb300_event_record(3)
    L.tea_gb300_synchronize()
    ms = float(L.tea_gb300_event_elapsed_ms(2, 3))
    x, y = lib.chunk_shape()[:2]
    drv.close()
    L.tea_gb300_finalise()
    its = sum(i.iterations + i.inner_iterations for i in infos)
    return {"cell_iters_per_s": its * x * y / (ms / 1e3), "ms_per_step": ms / timed_steps,
            "iterations": [i.iterations for i in infos],
            "inner_iterations": [i.inner_iterations for i in infos],
            "warm_steps": warm_steps, "timed_steps": timed_steps}


def other_workloads(args):
    """The benchmark set's other workloads, each measured compactly so that
    the default line carries them all: 512^2 CG + diagonal Jacobi (10 timed
    steps after 10), the Chebyshev solve at 4096^2 (block Jacobi, 2 timed
    steps after the one with the eigenvalue estimate), both through the
    resident driver, the 512-problem batch (autotuned, 5 steps) and the adjoint at
    2048^2 (20 steps, checked on 2 finite-difference directions here, 16
    with --mode adjoint, and on the FP64 reference gradient at 32^2)."""
    from tealeaf_opencl_gb300 import lib
    out = {}
    c1 = deck_rate(deck_for("cg512", 20), 10, 10, lib.DRIVER_RESIDENT)
    c1["workload"] = "512^2 five-state, CG + jac_diag, tl_eps 1e-15, 10 timed steps after 10"
    out["cg512"] = c1
    c2 = deck_rate(deck_for("cheby4096", 3), 1, 2, lib.DRIVER_RESIDENT)
    c2["workload"] = ("4096^2 five-state, Chebyshev + block Jacobi, 20 CG presteps, "
                      "tl_eps 1e-15, 2 timed steps after the first")
    out["cheby4096"] = c2
    batch = run_batch(argparse.Namespace(problems=512, seed=0, steps=5, reps=1, sequential=0,
                                         batch_launch="auto"))
    out["batch512"] = {k: batch[k] for k in ("problems", "cells", "steps", "launch",
                                            "cell_iters_per_s", "solve_gbs",
                                            "solve_frac_of_measured_hbm",
                                            "iterations_per_step")}
    adj = run_adjoint(argparse.Namespace(cells=2048, steps=20, eps=1e-12, directions=2,
                                         fd_step=1e-6, seed=0, ref_cells=32))
    out["adjoint2048"] = {"cells": adj["cells"], "steps": adj["steps"],
                         "forward_ms": adj["forward_ms"], "backward_ms": adj["backward_ms"],
                         "backward_over_forward": adj["backward_over_forward"],
                         "fd_max_rel_err": adj["finite_differences"]["max_rel_err"],
                         "fd_directions": adj["finite_differences"]["directions"],
                         "fp64_reference": adj["fp64_reference"]}
    return out


def mixed_compare(cells, steps, lognormal, mixed_solver, inner_steps, presteps):
    from tealeaf_opencl_gb300 import decks, lib
    L = lib.load()
    factor = lognormal_factor(cells) if lognormal else None
    out = {"mode": "mixed", "cells": cells * cells, "steps": steps,
           "lognormal": bool(lognormal), "tol": 1e-10}
    out["mixed_inner_solver"] = mixed_solver
    out["fp64_arithmetic"] = ARITHMETIC
    for name, extra, mode in (("fp64", "tl_exit_true_residual\ntl_arithmetic %s" % ARITHMETIC,
                               lib.DRIVER_RESIDENT),
                              ("mixed", "tl_mixed_precision\ntl_mixed_inner_eps 1e-5\n"
                               "tl_arithmetic %s" % ARITHMETIC, lib.DRIVER_PER_CALL)):
        solver = mixed_solver if name == "mixed" else "cg"
        deck = decks.five_state_deck(cells, solver=solver, prec="jac_diag",
                                     steps=steps, eps=1e-10, max_iters=100000,
                                     summary_frequency=0, check_result=True, extra=extra,
                                     inner_steps=inner_steps if solver == "ppcg" else None,
                                     presteps=presteps if solver == "ppcg" else None)
        drv = lib.Driver(deck, mode=mode)
        if factor is not None:
            lib.write_field("density", lib.read_field("density") * factor)
        L.tea_gb300_synchronize()
        times, infos = [], []
        for _ in range(steps):
            t0 = time.perf_counter()
            infos.append(drv.step())
            L.tea_gb300_synchronize()
            times.append(time.perf_counter() - t0)
        drv.close()
        last = infos[-1]
        out[name] = {"seconds": sum(times), "step_seconds": times,
                     "iterations": [i.iterations for i in infos],
                     "ppcg_inner_steps": [i.inner_iterations for i in infos],
                     "corrections": [i.outer_corrections for i in infos],
                     "relative_residual": [i.relative_residual if name == "mixed"
                                           else i.exact_error for i in infos],
                     "field_summary": {"vol": last.vol, "mass": last.mass,
                                       "ie": last.ie, "temp": last.temp}}
    a, b = out["fp64"]["field_summary"], out["mixed"]["field_summary"]
    out["field_summary_rel_diff"] = {k: abs(a[k] - b[k]) / abs(a[k]) for k in a}
    out["time_ratio_mixed_over_fp64"] = out["mixed"]["seconds"] / out["fp64"]["seconds"]
    return out


BATCH_BYTES_PER_CELL_ITER = 128  # CG with jac_diag: calc_w 40, calc_ur 64, calc_p 24


def run_batch(args):
    """Many independent problems solved together (tea_gb300_batch_*): seeded
    problems of uneven size, FP64 CG with diagonal Jacobi, tl_eps 1e-12,
    args.steps timesteps each.  Reports the batch's cell-iterations/s with the
    fields reset before every timed run, and the same problems solved one
    after another by the single-chunk resident driver on a sample."""
    import numpy as np
    from tealeaf_opencl_gb300 import decks, lib
    L = lib.load()
    L.tea_gb300_set_arithmetic(lib.arithmetic_form(ARITHMETIC))
    problems = decks.batch_problems(args.problems, seed=args.seed)
    t0 = time.perf_counter()
    fields = [decks.paint(p) for p in problems]
    paint_s = time.perf_counter() - t0
    b = lib.Batch([(p["x"], p["y"]) for p in problems], prec="jac_diag")
    cells = sum(p["x"] * p["y"] for p in problems)

    def reset():
        for i, (d, e) in enumerate(fields):
            b.set_fields(i, d, e)

    reset()
    t0 = time.perf_counter()
    tuned = b.autotune()
    tune_s = time.perf_counter() - t0
    if args.batch_launch != "auto":
        # the tuned geometry with the launch mode forced
        tuned["persistent"] = 1 if args.batch_launch == "persistent" else 0
        b.set_launch(tuned["blocks_per_sm"], tuned["graph_iterations"],
                     tuned["supertiles_per_unit"], tuned["persistent"])
        tuned = b.launch()
    runs = []
    for rep in range(max(1, args.reps)):
        reset()
        t0 = time.perf_counter()
        st = b.run(args.steps, 0.004, 1e-12, 5000)
        runs.append((time.perf_counter() - t0, st.as_dict()))
    wall, st = min(runs, key=lambda r: r[1]["total_ms"])
    iters = np.array([b.iterations(i) for i in range(len(problems))])
    peak, peak_kind = measured_peak_hbm()
    rate = st["cell_iterations"] / (st["total_ms"] * 1e-3)
    out = {"mode": "batch", "problems": len(problems), "seed": args.seed,
           "cells": cells, "steps": args.steps, "eps": 1e-12, "prec": "jac_diag",
           "dtype": "f64", "launch": tuned, "autotune_seconds": tune_s,
           "paint_seconds": paint_s, "stats": st, "wall_seconds": wall,
           "cell_iters_per_s": rate,
           "solve_gbs": st["cell_iterations"] * BATCH_BYTES_PER_CELL_ITER / (st["solve_ms"] * 1e-3) / 1e9,
           "hbm_peak_gbs": peak, "hbm_peak_kind": peak_kind,
           "iterations_per_step": {"min": int(iters.min()), "median": float(np.median(iters)),
                                   "max": int(iters.max())}}
    out["solve_frac_of_measured_hbm"] = out["solve_gbs"] / peak if peak else None
    b.free()
    # the same problems one by one through the single-chunk resident driver
    k = min(args.sequential, len(problems))
    if k > 0:
        seq_s, seq_ci = 0.0, 0.0
        for p in problems[:k]:
            deck = decks.batch_deck(p, steps=args.steps, eps=1e-12, prec="jac_diag",
                                    arithmetic=ARITHMETIC)
            drv = lib.Driver(deck, mode=lib.DRIVER_RESIDENT)
            L.tea_gb300_synchronize()
            t0 = time.perf_counter()
            its = 0
            while True:
                info = drv.step()
                if info is None:
                    break
                its += info.iterations
                if info.complete:
                    break
            L.tea_gb300_synchronize()
            seq_s += time.perf_counter() - t0
            seq_ci += p["x"] * p["y"] * its
            drv.close()
        sub = lib.Batch([(p["x"], p["y"]) for p in problems[:k]], prec="jac_diag")
        for i in range(k):
            sub.set_fields(i, *fields[i])
        sub.autotune()
        for i in range(k):
            sub.set_fields(i, *fields[i])
        t0 = time.perf_counter()
        sst = sub.run(args.steps, 0.004, 1e-12, 5000)
        sub_s = time.perf_counter() - t0
        sub.free()
        out["sequential_sample"] = {
            "problems": k, "single_chunk_seconds": seq_s,
            "single_chunk_cell_iters_per_s": seq_ci / seq_s,
            "batch_seconds": sub_s, "batch_cell_iters_per_s": sst.cell_iterations / sub_s,
            "speedup": seq_s / sub_s}
    return out


def run_adjoint(args):
    """Gradient of 0.5*||u_T - u_obs||^2 w.r.t. per-cell log-density through
    args.steps implicit CG timesteps (jac_diag, FP64) on the five-state
    problem at args.cells^2, with u_obs from a forward run whose density is
    perturbed by a seeded smooth log-normal field.  Times the forward pass
    (with checkpoints every 4 steps) and the adjoint pass, then checks the
    gradient against central finite differences on args.directions random
    directions, and against the FP64 torch-autograd reference gradient on a
    small problem (args.ref_cells^2)."""
    import numpy as np
    import torch
    from tealeaf_opencl_gb300 import adjoint, decks, lib
    from tests import adjoint_reference as ref
    L = lib.load()
    n, steps, dt = args.cells, args.steps, 0.004
    deck = decks.five_state_deck(n, solver="cg", prec="jac_diag", steps=1,
                                 summary_frequency=0)
    drv = lib.Driver(deck)
    dens = lib.read_field("density")
    en = lib.read_field("energy1")
    drv.close()
    L.tea_gb300_finalise()
    L.tea_gb300_set_arithmetic(lib.arithmetic_form(ARITHMETIC))
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    adj = lib.Adjoint(n, n)
    d, e = dev(dens), dev(en)
    cfg = adj.config(steps, dt, args.eps, 20000, 4)
    u_obs = torch.empty_like(d)
    adj.forward(dev(dens * np.exp(ref.smooth_field((n, n), 2024, sigma=0.3, corr=16.0))), e,
                u_final=u_obs, cfg=cfg)
    loss, fst = adj.forward(d, e, u_obs, cfg=cfg)
    g = torch.empty_like(d)
    bst = adj.backward(g)
    out = {"mode": "adjoint", "cells": n * n, "steps": steps, "dt": dt, "eps": args.eps,
           "checkpoint_every": 4, "dtype": "f64", "loss": loss,
           "forward_ms": fst.forward_ms, "backward_ms": bst.backward_ms,
           "backward_over_forward": bst.backward_ms / fst.forward_ms,
           "iterations": {"forward": fst.forward_iterations,
                          "recompute": bst.recompute_iterations,
                          "adjoint": bst.adjoint_iterations},
           "checkpoints": bst.checkpoints,
           "grad_norm": float(g.norm())}
    theta = torch.log(d)
    gen = torch.Generator(device="cuda").manual_seed(args.seed)
    h = args.fd_step
    errs = []
    t0 = time.perf_counter()
    for _ in range(args.directions):
        v = torch.randn(theta.shape, dtype=torch.float64, device="cuda", generator=gen)
        lp = adjoint.time_stepped_loss(theta + h * v, e, u_obs, adj, cfg)
        lm = adjoint.time_stepped_loss(theta - h * v, e, u_obs, adj, cfg)
        fd = float((lp - lm) / (2 * h))
        gv = float((g * v).sum())
        errs.append({"fd": fd, "adjoint": gv, "rel_err": abs(fd - gv) / abs(fd)})
    out["finite_differences"] = {"directions": args.directions, "step": h,
                                 "max_rel_err": max(x["rel_err"] for x in errs),
                                 "seconds": time.perf_counter() - t0, "each": errs}
    adj.free()
    # the FP64 reference gradient (dense direct solves, torch autograd)
    m = args.ref_cells
    deck = decks.five_state_deck(m, solver="cg", prec="jac_diag", steps=1, summary_frequency=0)
    drv = lib.Driver(deck)
    dens_s, en_s = lib.read_field("density"), lib.read_field("energy1")
    drv.close()
    L.tea_gb300_finalise()
    L.tea_gb300_set_arithmetic(lib.arithmetic_form(ARITHMETIC))
    adj = lib.Adjoint(m, m)
    cfg_s = adj.config(steps, dt, 1e-15, 20000, 4)
    uo = torch.empty((m, m), dtype=torch.float64, device="cuda")
    adj.forward(dev(dens_s * np.exp(ref.smooth_field((m, m), 7, sigma=0.3, corr=4.0))),
                dev(en_s), u_final=uo, cfg=cfg_s)
    loss_s, _ = adj.forward(dev(dens_s), dev(en_s), uo, cfg=cfg_s)
    gs = torch.empty_like(uo)
    adj.backward(gs)
    adj.free()
    loss_r, g_r = ref.loss_and_gradient(dens_s, en_s, uo.cpu().numpy(), steps, dt)
    out["fp64_reference"] = {
        "cells": m * m, "eps": 1e-15,
        "loss_rel_err": abs(loss_s - loss_r) / abs(loss_r),
        "grad_max_abs_err_over_max": float(np.abs(gs.cpu().numpy() - g_r).max() / np.abs(g_r).max())}
    return out


def oracle_sample(name, steps, first_timed, cap, cap_after_switch):
    """The oracle on the workload's deck for `steps` timesteps, bounded:
    CG workloads cap every step at `cap` outer iterations; Chebyshev and
    PPCG steps end `cap_after_switch` iterations after their switch from CG,
    so the first step runs its CG iterations to the switch and the
    eigenvalue estimate (as on the GPU), and every later PPCG step is one CG
    iteration and then PPCG outer iterations with their inner steps.  Steps
    first_timed.. are measured.  Returns (value, description, threads)."""
    from oracle import oracle
    cells = WORKLOADS[name][0]
    solver = WORKLOADS[name][1]
    deck = deck_for(name, steps)
    if solver == "cg":
        res = oracle.run_deck(deck, max_solver_iters=cap)
        bound = "each step capped at %d CG iterations" % cap
    else:
        res = oracle.run_deck(deck, max_after_switch=cap_after_switch)
        bound = ("each step ended %d iterations after its switch from CG (step 1 "
                 "switched after %d CG iterations)" % (cap_after_switch,
                                                      res.switch_iteration[0] - 1))
    sl = slice(first_timed, steps)
    outer, inner = sum(res.iterations[sl]), sum(res.inner_iterations[sl])
    cg = sum(max(0, s - 1) if s else it for s, it in
             zip(res.switch_iteration[sl], res.iterations[sl]))
    secs = sum(res.step_seconds[sl])
    value = (outer + inner) * cells * cells / secs
    desc = ("oracle (C/OpenMP restatement of the reference) on the same deck, "
            "timesteps %d-%d timed of %d, %s: %d outer iterations (%d CG, %d %s) "
            "+ %d PPCG inner steps, %.1f s"
            % (first_timed + 1, steps, steps, bound, outer, cg, outer - cg,
               solver.upper(), inner, secs))
    return value, desc, oracle.lib().oracle_num_threads(), secs


def cpu_sample(name, args):
    """Our arm's cpu_baseline: the oracle, step 2 of a two-step run."""
    return oracle_sample(name, 2, 1, args.cpu_cap, args.cpu_cap_after_switch)[:3]


def run_reference(args, dist):
    """The CPU restatement of the reference on the host cores."""
    name = args.workload
    cells = WORKLOADS[name][0]
    w, k = args.warmup, args.steps
    t0 = time.perf_counter()
    value, sample, threads, secs = oracle_sample(name, w + k, w, args.cpu_cap,
                                                 args.cpu_cap_after_switch)
    wall = time.perf_counter() - t0
    return {
        "impl": "reference",
        "metric": "TeaLeaf %s cell-iterations/s at %dx%d (FP64)" % (WORKLOADS[name][1].upper(), cells, cells),
        "value": value, "unit": "cell-iters/s", "n_gpus": dist.world,
        "steps": k, "warmup": w, "ms_per_step": 1e3 * secs / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic: five-state layout of the reference's decks",
        "config": config_for(name),
        "cpu_baseline": {"value": value, "unit": "cell-iters/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cell-iters/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ppcg4096", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-cap", type=int, default=24,
                    help="CG workloads: outer iterations per CPU sample step")
    ap.add_argument("--cpu-cap-after-switch", type=int, default=9,
                    help="PPCG/Chebyshev workloads: iterations per CPU sample step "
                         "from the switch from CG on")
    ap.add_argument("--inner-pairs", type=int, default=0, choices=[0, 1],
                    help="PPCG inner steps two at a time in one TMA-fed pass (1) or one "
                         "one-pass update_r + calc_sd per step (0, the faster on GB300)")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="leave out the compact cg512 / cheby4096 / batch / adjoint measurements "
                         "of the default line")
    ap.add_argument("--no-mixed", action="store_true",
                    help="leave out the mixed-precision comparison of the default line")
    ap.add_argument("--cap", type=int, default=0,
                    help="limit solver iterations per GPU step (profiling runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="run",
                    choices=["run", "kernels", "mixed", "batch", "adjoint"],
                    help="kernels: time each hot entry point on the workload's grid; "
                         "mixed: FP64 vs FP32-inner/FP64-refined CG to 1e-10")
    ap.add_argument("--cells", type=int, default=4096, help="grid side for --mode mixed")
    ap.add_argument("--mixed-solver", default="cg", choices=["cg", "ppcg"],
                    help="--mode mixed: FP32 inner solver")
    ap.add_argument("--presteps", type=int, default=25,
                    help="--mode mixed --mixed-solver ppcg: CG presteps")
    ap.add_argument("--inner-steps", type=int, default=10,
                    help="--mode mixed --mixed-solver ppcg: Chebyshev steps per iteration")
    ap.add_argument("--lognormal", action="store_true",
                    help="--mode mixed: density times a seeded log-normal field")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--arithmetic", default="chain", choices=["exact", "fused", "chain"],
                    help="arithmetic form of the FP64 kernels (tl_arithmetic)")
    ap.add_argument("--problems", type=int, default=512, help="--mode batch: problem count")
    ap.add_argument("--seed", type=int, default=0, help="--mode batch: problem seed")
    ap.add_argument("--directions", type=int, default=16,
                    help="--mode adjoint: finite-difference directions")
    ap.add_argument("--fd-step", type=float, default=1e-6,
                    help="--mode adjoint: central-difference step in log-density")
    ap.add_argument("--eps", type=float, default=1e-12, help="--mode adjoint: CG tolerance")
    ap.add_argument("--ref-cells", type=int, default=32,
                    help="--mode adjoint: side of the FP64 reference-gradient problem")
    ap.add_argument("--batch-launch", default="auto", choices=["auto", "kernels", "persistent"],
                    help="--mode batch: the autotuner's launch mode, or three kernels per "
                         "CG iteration, or one persistent launch per graph replay")
    ap.add_argument("--sequential", type=int, default=32,
                    help="--mode batch: problems also run one by one for comparison")
    args = ap.parse_args()
    global ARITHMETIC
    ARITHMETIC = args.arithmetic
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")

    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")

    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        out = run_reference(args, _Solo())
        print(json.dumps(out))
        return

    if args.mode == "kernels":
        print(json.dumps(run_kernels(args)))
        return
    if args.mode == "mixed":
        print(json.dumps(run_mixed(args)))
        return
    if args.mode == "batch":
        print(json.dumps(run_batch(args)))
        return
    if args.mode == "adjoint":
        print(json.dumps(run_adjoint(args)))
        return

    dist = Dist()
    out = run_ours(args, dist)
    if dist.world == 1 and not args.no_mixed:
        out["mixed"] = mixed_summary(args)
    if dist.world == 1 and not args.no_other_workloads:
        out["other_workloads"] = other_workloads(args)
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        value, sample, threads = cpu_sample(args.workload, args)
        out["cpu_baseline"] = {"value": value, "unit": "cell-iters/s", "cores": threads,
                               "kind": "port", "sample": sample}
    if dist.rank == 0:
        print(json.dumps(out))
    dist.close()


class _Solo:
    world = 1
    rank = 0


if __name__ == "__main__":
    main()
