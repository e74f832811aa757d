#!/usr/bin/env python
"""CG time-to-solution on one GB300: the 8192^2 seeded random-rectangle deck.

Workload (one "step" = one diffuse! timestep of the deck): halo of energy and
density, the CG solve to 1e-10 relative residual (||u0 - A u|| / ||u0||, the
true residual checked in FP64 on the device), solvefinished!.  The deck is
synthetic and seeded: background rho=100 e=1e-4 plus 4-8 axis-aligned
rectangles with corners uniform in [0,10]^2, rho log-uniform in [0.1, 100],
e uniform in [0.1, 25]; dt = 0.004.  The K timed steps are timesteps 1..K of
the deck: the W warm-up timesteps run first on the same context, which is
then put back to the deck's initial state.  Every field (537 MB) is larger
than L2, so no flush is needed between timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` is the device time of one timestep (ms, lower
is better) of the headline variant (learned warm start + FP32 refinement);
`variants` gives every variant with its final-field error against plain FP64
CG; `e2e` repeats the timesteps through the C ABI with the inputs uploaded
from pinned host memory and the result downloaded inside the timed region.
The reference arm times the CPU restatement of the reference solver (OpenMP
over all host cores) on a bounded sample of the same solve.
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG_DIR = ROOT / "tealeaf.jl_gb300"
METRIC = "CG time-to-solution @1e-10 rel resid, HBM GB/s: learned+FP32-IR vs plain FP64"
DECK_SEED = 2024
# FP64 CG iterations to 1e-10 relative residual of timesteps 1, 2, ... of the
# 8192^2 deck (seed 2024), measured on a GB300 with the fused kernels.  The
# reference arm, which runs without a GPU, scales its CPU sample by the mean
# over the timed timesteps; the GPU arm uses the counts it measures.
FP64_ITERS_8192 = [4122, 3884, 3643, 3403, 3190, 2993, 2822, 2681, 2531, 2429, 2322, 2220, 2175, 2065, 2016, 1966,
                   1899, 1849, 1783, 1758, 1693, 1642, 1610, 1647, 1615]
BYTES_PER_CELL_ITER = 104    # 13 FP64 words: stencil 4 + u/r update 6 + p update 3
W_STEP_BYTES = 48            # fused p-update + stencil + p.w: read p, r, kx, ky; write p, w
UR_STEP_BYTES = 48           # u/r update + r.r: read u, p, r, w; write u, r


def load_package():
    if "tealeaf_gb300" in sys.modules:
        return sys.modules["tealeaf_gb300"]
    spec = importlib.util.spec_from_file_location("tealeaf_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["tealeaf_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    spec = importlib.util.spec_from_file_location("tealeaf_oracle_py", ROOT / "oracle" / "oracle.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_deck(n: int, seed: int = DECK_SEED, steps: int = 20, eps: float = 1e-10, maxiters: int = 40000) -> str:
    rng = np.random.default_rng(seed)
    nrect = int(rng.integers(4, 9))
    lines = ["state 1 density=100.0 energy=0.0001"]
    for k in range(nrect):
        x0, x1 = sorted(float(v) for v in rng.uniform(0, 10, 2))
        y0, y1 = sorted(float(v) for v in rng.uniform(0, 10, 2))
        rho = float(10 ** rng.uniform(-1, 2))
        e = float(rng.uniform(0.1, 25))
        lines.append(f"state {k + 2} density={rho!r} energy={e!r} geometry=rectangle xmin={x0!r} xmax={x1!r} "
                     f"ymin={y0!r} ymax={y1!r}")
    lines += [f"x_cells={n}", f"y_cells={n}", "xmin=0.0", "ymin=0.0", "xmax=10.0", "ymax=10.0",
              "initial_timestep=0.004", f"end_step={steps}", f"max_iters={maxiters}", "use_cg", f"eps={eps!r}",
              "halo_depth=2", "coefficient=1", "summary_frequency=10"]
    return "\n".join(lines) + "\n"


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"tealeaf_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.path.read_text().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------

# bench variants: (precision, warm start)
# learned: the A-norm projection onto u^n, the last six increments and the
# network's correction; history: the same projection without the network;
# extrap: u^n + (u^n - u^{n-1})
VARIANTS = {"learned_fp32_ir": (1, 1), "fp32_ir": (1, 0), "history_fp32_ir": (1, 3), "extrap_fp32_ir": (1, 2),
            "fp64": (0, 0)}
HEADLINE = "learned_fp32_ir"
# plain FP64 runs first: every other variant's final field is compared with it
RUN_ORDER = ["fp64", "learned_fp32_ir", "fp32_ir", "history_fp32_ir", "extrap_fp32_ir"]


def gpu_setup(tl, n, precision, maxiters=40000, warm=0):
    s = tl.Settings.from_text(make_deck(n, maxiters=maxiters), mode=1, exact=False, criterion=1,
                              precision=precision, warmstart=warm)
    chunk = tl.initialiseapp(s)
    if warm == tl._abi.WARM_NETWORK:
        chunk.warm_load(tl.warmstart.load_params())
    return s, chunk


def restart_deck(tl, chunk, s):
    """Puts the context back to the deck's initial state (initialiseapp!: the
    states, the halo of density, energy0, energy, energy = energy0) and clears
    the warm start's history, keeping the tuned layouts and the instantiated
    graphs: the next timestep is timestep 1 of the deck."""
    arr = tl._state_array(s, chunk.mode)
    chunk.check(chunk.lib.tl_initialise(chunk.ctx, arr, len(s.states)))
    s.resettoexchange()
    for f in ("density", "energy0", "energy"):
        s.toexchange[f] = True
    chunk.warm_reset()


def timestep(tl, chunk, s):
    rx = s.dtinit / s.dx ** 2
    ry = s.dtinit / s.dy ** 2
    tl.haloupdate(chunk, s, 1, ["energy", "density"])
    res = tl.SOLVERS[s.solver].solve(chunk, s, rx, ry)
    tl.solvefinished(chunk, s)
    return res


def run_variant(tl, n, precision, steps, warmup, warm=0):
    """W untimed warm-up timesteps, then the deck restarted and timesteps
    1..K timed, each bracketed by device events on the library's stream."""
    s, chunk = gpu_setup(tl, n, precision, warm=warm)
    lib = chunk.lib
    for _ in range(warmup):
        r = timestep(tl, chunk, s)
        if not r.converged:
            raise RuntimeError(f"warm-up solve did not converge: {r}")
    restart_deck(tl, chunk, s)
    times, results = [], []
    for _ in range(steps):
        chunk.check(lib.tl_synchronize(chunk.ctx))
        chunk.check(lib.tl_timer_start(chunk.ctx))
        r = timestep(tl, chunk, s)
        ms = C.c_double()
        chunk.check(lib.tl_timer_stop(chunk.ctx, C.byref(ms)))
        if not r.converged:
            raise RuntimeError(f"timed solve did not converge: {r}")
        times.append(ms.value)
        results.append(r)
    return s, chunk, times, results


def run_e2e(tl, n, precision, steps, warmup, warm=0):
    """The same timesteps through the C ABI with host buffers: each step uploads
    energy and density from pinned memory, solves, runs solvefinished and
    downloads energy.  The W warm-up steps go through the same path untimed;
    the deck is then restarted and timesteps 1..K are timed."""
    import torch
    s, chunk = gpu_setup(tl, n, precision, warm=warm)
    lib = chunk.lib
    X, Y = chunk.size()
    pinned = {nm: torch.empty((Y, X), dtype=torch.float64, pin_memory=True) for nm in ("energy", "density")}
    out = torch.empty((Y, X), dtype=torch.float64, pin_memory=True)

    def load_initial():
        for nm in pinned:
            pinned[nm].numpy()[...] = chunk.field(nm).T

    load_initial()
    # host-side check of the staging buffers: pinned, and a plain copy's rate
    dev = torch.empty((Y, X), dtype=torch.float64, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dev.copy_(pinned["energy"], non_blocking=True)
    e0.record()
    dev.copy_(pinned["energy"], non_blocking=True)
    e1.record()
    e1.synchronize()
    probe = {"pinned": all(t.is_pinned() for t in list(pinned.values()) + [out]),
             "torch_h2d_gbs": X * Y * 8 / (e0.elapsed_time(e1) * 1e-3) / 1e9}
    del dev
    fidx = {"energy": 3, "density": 1}
    dptr = C.POINTER(C.c_double)
    times, results, phases = [], [], []
    for k in range(warmup + steps):
        if k == warmup:
            restart_deck(tl, chunk, s)
            load_initial()
        chunk.check(lib.tl_synchronize(chunk.ctx))
        chunk.check(lib.tl_timer_start(chunk.ctx))
        w0 = time.perf_counter()
        for nm in ("energy", "density"):
            chunk.check(lib.tl_upload(chunk.ctx, fidx[nm], C.cast(pinned[nm].data_ptr(), dptr), X))
        w1 = time.perf_counter()
        r = timestep(tl, chunk, s)
        chunk.check(lib.tl_synchronize(chunk.ctx))
        w2 = time.perf_counter()
        chunk.check(lib.tl_download(chunk.ctx, fidx["energy"], C.cast(out.data_ptr(), dptr), X))
        w3 = time.perf_counter()
        ms = C.c_double()
        chunk.check(lib.tl_timer_stop(chunk.ctx, C.byref(ms)))
        pinned["energy"].copy_(out)     # the next step starts from this step's result, as diffuse! does
        if k >= warmup:
            times.append(ms.value)
            results.append(r)
            phases.append({"upload": (w1 - w0) * 1e3, "step": (w2 - w1) * 1e3, "download": (w3 - w2) * 1e3})
    chunk.close()
    phases.append(probe)
    return statistics.mean(times), 2 * X * Y * 8, X * Y * 8, times, results, phases


# FP32 CG iteration: the direction step (read p, r, iw; write p': 16 B) and
# the update step (read p', iw, x, r; write x, r: 24 B)
IR_ITER_BYTES = 40
KERNELS = {"fp64": ((0, "cg_w_step", W_STEP_BYTES + 8), (1, "cg_ur_step", UR_STEP_BYTES)),
           "fp32_ir": ((8, "ir_dir_step", 16), (9, "ir_update_step", 24))}
# DRAM bytes (read + write) per interior cell of one launch, from ncu
# captures at 4096^2; traffic grows with the cells, so a full launch moves
# this times n^2.
TRAFFIC_BYTES_PER_CELL = {"ir_dir_step": 247.4e6 / 4096 ** 2, "ir_update_step": 362.5e6 / 4096 ** 2,
                          "cg_w_step": 923.7e6 / 4096 ** 2}


def kernel_roofline(tl, chunk, kind, peak):
    """Average duration of the two iteration kernels of one precision, each
    launched 20 times back to back on the library's stream and timed with
    CUDA events; algorithmic bytes = compulsory reads + writes per interior
    cell (the FP64 stencil step also reads the stored diagonal: 56 B)."""
    lib = chunk.lib
    cells = chunk.settings.xcells * chunk.settings.ycells
    out = {}
    for k, name, b in KERNELS[kind]:
        ms = C.c_double()
        chunk.check(lib.tl_bench_kernel(chunk.ctx, k, 20, C.byref(ms)))
        gbs = b * cells / (ms.value * 1e-3) / 1e9
        out[name] = {"ms": ms.value, "bytes_per_cell": b, "gbs": gbs, "frac": gbs / peak}
    return out


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_sample(oracle, n, iters_full, threads, small=10, large=330):
    """The oracle's tealeaf-mode CG (OpenMP over `threads`, relative
    criterion) on timestep 1 of the same deck: two bounded solves (small and
    large iteration caps) give the per-iteration time and the set-up cost;
    the time-to-solution is scaled to `iters_full` iterations."""
    text = make_deck(n)
    s = oracle.parse_deck(text)
    o = oracle.make_opts(mode=oracle.MODE_TEALEAF, order=oracle.ORDER_THREADS, nthreads=threads, criterion=1)
    ch = oracle.OracleChunk(s, o)
    ch.initialise()
    rx = s.dtinit / s.dx ** 2
    ry = s.dtinit / s.dy ** 2
    t = {}
    for cap in (small, large):
        s.maxiters = cap
        ch.halo(1, ["energy", "density"])
        t0 = time.perf_counter()
        ch.solve(rx, ry)
        t[cap] = time.perf_counter() - t0
    per_iter = (t[large] - t[small]) / (large - small)
    setup = max(t[small] - small * per_iter, 0.0)
    return (setup + iters_full * per_iter) * 1e3, per_iter * 1e3, t[small] + t[large]


def cpu_single_thread(oracle, n, iters_full):
    """The same scaled time-to-solution with one host thread (3- and
    13-iteration solves: about 15 s of CPU work at 8192^2)."""
    v, pi, wall = cpu_sample(oracle, n, iters_full, 1, small=3, large=13)
    return {"value": v, "unit": "ms", "cores": 1, "ms_per_iteration": pi,
            "sample": f"3- and 13-iteration solves, one thread ({wall:.1f} s)"}


def oracle_iters(oracle, n, steps, threads):
    """FP64 CG iteration counts of timesteps 1..steps of the n^2 deck, solved
    to 1e-10 relative by the oracle itself (small decks only)."""
    s = oracle.parse_deck(make_deck(n))
    ch = oracle.OracleChunk(s, oracle.make_opts(mode=oracle.MODE_TEALEAF, order=oracle.ORDER_THREADS,
                                                nthreads=threads, criterion=1))
    ch.initialise()
    out = []
    for _ in range(steps):
        ch.halo(1, ["energy", "density"])
        out.append(ch.solve(s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2).iters)
        ch.solve_finished()
    return out


def fp64_iters_of_window(steps):
    """The committed FP64 iteration counts of timesteps 1..K, or None."""
    if FP64_ITERS_8192 is None or len(FP64_ITERS_8192) < steps:
        return None
    return FP64_ITERS_8192[:steps]


def reference_arm(args):
    """--impl reference: the CPU restatement of the reference solver (the
    reference itself is Julia and cannot run here) on the machine's host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    oracle = load_oracle()
    oracle.build()
    threads = os.cpu_count() or 1
    window = fp64_iters_of_window(args.steps) if args.size == 8192 else None
    if window is None and args.size <= 1024:
        window = oracle_iters(oracle, args.size, args.steps, threads)
    if window is None:
        print(json.dumps({"impl": "reference", "unavailable": f"no FP64 iteration counts committed for "
                                                              f"timesteps 1..{args.steps} of the {args.size}^2 deck"}))
        return
    iters = statistics.mean(window)
    vals, per_it, walls = [], [], []
    for k in range(args.warmup + args.steps):
        v, pi, wall = cpu_sample(oracle, args.size, iters, threads)
        if k >= args.warmup:
            vals.append(v)
            per_it.append(pi)
            walls.append(wall)
    value = statistics.mean(vals)
    sample = (f"tealeaf-mode CG of the oracle (relative criterion) on timestep 1 of the {args.size}^2 deck: 10- and "
              f"330-iteration solves per step ({statistics.mean(walls):.1f} s of CPU work each), time-to-solution "
              f"scaled to {iters:.0f} iterations, the mean FP64 CG count of timesteps 1..{args.steps}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.size}^2 seeded random-rectangle deck, CG to 1e-10 relative residual, "
                                   f"timesteps 1..{args.steps}", "n": args.size, "seed": DECK_SEED},
            "cpu_baseline": {"value": value, "unit": "ms", "cores": threads, "kind": "port", "sample": sample,
                             "ms_per_iteration": statistics.mean(per_it), "sample_seconds": sum(walls),
                             "iterations_scaled_to": iters},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_single:
        line["cpu_baseline"]["single_thread"] = cpu_single_thread(oracle, args.size, iters)
    print(json.dumps(line))


def final_field(tl, chunk, s):
    """Host copies of the interior of u and of the field summary."""
    hd = s.halodepth
    u = np.ascontiguousarray(chunk.field("u")[hd:-hd, hd:-hd])
    return u, tl.fieldsummary(chunk, s, problemfile=None)


def accuracy_against(u, summ, u64, summ64):
    """Final-field error against plain FP64 CG: max |u - u64| / max |u64| over
    the interior, and each field-summary component's relative difference."""
    ref = float(np.max(np.abs(u64)))
    return {"u_max_rel_diff": float(np.max(np.abs(u - u64))) / ref,
            "summary_rel_diff": {k: abs(a - b) / max(abs(b), 1e-300)
                                 for k, a, b in zip(("vol", "mass", "ie", "temp"), summ, summ64)}}


def gpu_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("gloo")
    else:
        torch.cuda.set_device(0)
    tl = load_package()
    peak, peak_kind = measured_peaks()
    n = args.size
    variants = {}
    roof = {}
    headline_res = None
    u64 = summ64 = None
    order = RUN_ORDER if args.variant == "all" else [args.variant]
    with ClockSampler(local) as clk:
        for name in order:
            try:
                if dist:
                    dist.barrier()
                prec, warm = VARIANTS[name]
                s, chunk, times, results = run_variant(tl, n, prec, args.steps, args.warmup, warm=warm)
            except tl.TeaLeafError as e:
                variants[name] = {"error": str(e)}
                continue
            ms = max(times)
            if dist:
                t = torch.tensor([statistics.mean(times)], dtype=torch.float64)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                mean_ms = float(t[0])
            else:
                mean_ms = statistics.mean(times)
            iters = [r.iters for r in results]
            loop_ms = [r.solve_ms for r in results]
            variants[name] = {"ms_per_step": mean_ms, "max_ms": ms, "ms": times, "iters": iters,
                              "timesteps": f"1..{args.steps}",
                              "rel_residual": [r.rel_residual for r in results],
                              "loop_ms": loop_ms, "launches": [r.launches for r in results],
                              "ms_per_iteration": statistics.mean(loop_ms) / statistics.mean(iters),
                              "algorithmic_gbs_per_iteration": (BYTES_PER_CELL_ITER if name == "fp64" else IR_ITER_BYTES) *
                              n * n * statistics.mean(iters) / (statistics.mean(loop_ms) * 1e-3) / 1e9,
                              "warm": [r.warm for r in results], "r0_plain": [r.r0_plain for r in results],
                              "r0_pred": [r.r0_pred for r in results],
                              "warm_coef": [list(r.warm_coef) for r in results],
                              "refinements": [r.refinements for r in results]}
            u, summ = final_field(tl, chunk, s)
            if name == "fp64":
                u64, summ64 = u, summ
                variants[name]["final_summary"] = summ
            elif u64 is not None:
                variants[name]["final_field_vs_fp64"] = accuracy_against(u, summ, u64, summ64)
            del u
            if name == "fp64" or name == HEADLINE:
                roof.update(kernel_roofline(tl, chunk, "fp64" if name == "fp64" else "fp32_ir", peak))
            if name == HEADLINE:
                headline_res = results
            chunk.close()
    clocks = clk.summary()
    if headline_res is None:
        print(json.dumps({"metric": METRIC, "error": variants}))
        return
    e2e_ms, h2d, d2h, e2e_times, e2e_res, e2e_phases = run_e2e(tl, n, VARIANTS[HEADLINE][0], args.steps, args.warmup,
                                                               warm=VARIANTS[HEADLINE][1])
    value = variants[HEADLINE]["ms_per_step"]
    line = {"metric": METRIC, "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (bf16 network)", "data": "synthetic",
            "config": {"workload": f"{n}^2 seeded random-rectangle deck, CG to 1e-10 relative residual, timesteps "
                                   f"1..{args.steps} (halo, solve, solvefinished per step)", "n": n,
                       "seed": DECK_SEED, "variant": HEADLINE,
                       "warmup": f"{args.warmup} timesteps on the same context, then the deck restarted",
                       "l2": "every field (537 MB at 8192^2) is larger than L2; no flush"},
            "clocks": clocks,
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms": e2e_times, "iters": [r.iters for r in e2e_res], "warm": [r.warm for r in e2e_res],
                    "host_wall_ms": e2e_phases},
            # the solve's own launches plus the halo and solvefinished! kernels of each step
            "gpu_launches": int(sum(r.launches for r in headline_res) + 4 * len(headline_res)),
            "variants": variants,
            "vs_fp64_gpu": {k: variants["fp64"]["ms_per_step"] / v["ms_per_step"] for k, v in variants.items()
                            if "ms_per_step" in v and "ms_per_step" in variants.get("fp64", {})}}
    if roof:
        dom = max((v for k, v in roof.items() if k.startswith("ir_")), key=lambda d: d["ms"], default=None)
        if dom is not None:
            dname = [k for k, v in roof.items() if v is dom][0]
            tpc = TRAFFIC_BYTES_PER_CELL.get(dname)
            line["roofline"] = {"bound": "hbm", "kernel": dname, "achieved": dom["gbs"], "peak": peak,
                                "unit": "GB/s", "frac": dom["gbs"] / peak,
                                "traffic": tpc * n * n if tpc else None,
                                "traffic_source": "ncu capture at 4096^2 scaled by cells" if tpc else None,
                                "algorithmic_bytes": dom["bytes_per_cell"] * n * n,
                                "peak_kind": peak_kind, "kernels": roof}
    if rank == 0 and world == 1 and not args.no_config4:
        line["config4"] = config4_leg(tl)
    if rank == 0 and world == 1 and not args.no_cpu:
        oracle = load_oracle()
        oracle.build()
        threads = os.cpu_count() or 1
        iters = statistics.mean(variants["fp64"]["iters"]) if "iters" in variants.get("fp64", {}) \
            else statistics.mean(fp64_iters_of_window(args.steps) or [3000])
        v, pi, wall = cpu_sample(oracle, n, iters, threads)
        line["cpu_baseline"] = {"value": v, "unit": "ms", "cores": threads, "kind": "port",
                                "sample": f"oracle tealeaf-mode CG (relative criterion), timestep 1 of the {n}^2 deck, "
                                          f"10- and 330-iteration solves ({wall:.1f} s), scaled to {iters:.0f} "
                                          f"iterations (the mean FP64 CG count of timesteps 1..{args.steps})",
                                "ms_per_iteration": pi, "sample_seconds": wall, "iterations_scaled_to": iters}
        if not args.no_single:
            line["cpu_baseline"]["single_thread"] = cpu_single_thread(oracle, n, iters)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def config4_leg(tl):
    """The batched workload beside the headline: 128 decks of uneven sizes,
    10 timesteps each, one batched graph launch per timestep against the same
    decks solved one after another, FP64 and FP32-refined CG to 1e-10."""
    sizes, texts = config4_decks(128)
    out = {"workload": "128 random-rectangle decks, nx, ny in 256..2048 step 128, 10 steps, CG to 1e-10 relative",
           "cells": sum(a * b for a, b in sizes)}
    for prec, pname in ((0, "fp64"), (1, "fp32_ir")):
        r = run_config4_precision(tl, texts, 10, prec)
        out[pname] = {"batched_s": r["batched"]["seconds"], "sequential_s": r["sequential"]["seconds"],
                      "batched_loop_ms": r["batched"]["loop_ms"], "sequential_loop_ms": r["sequential"]["loop_ms"],
                      "iterations": {m: r[m]["iterations"] for m in ("batched", "sequential")},
                      "speedup": r["sequential"]["seconds"] / r["batched"]["seconds"],
                      "loop_speedup": r["sequential"]["loop_ms"] / r["batched"]["loop_ms"]}
    out["fp32_ir_batched_vs_fp64_sequential"] = out["fp64"]["sequential_s"] / out["fp32_ir"]["batched_s"]
    return out


CONFIG2_STATES = """state 1 density=100.0 energy=0.0001
state 2 density=0.1 energy=25.0 geometry=rectangle xmin=0.0 xmax=1.0 ymin=1.0 ymax=2.0
state 3 density=0.1 energy=0.1 geometry=rectangle xmin=1.0 xmax=6.0 ymin=1.0 ymax=2.0
state 4 density=0.1 energy=0.1 geometry=rectangle xmin=5.0 xmax=6.0 ymin=1.0 ymax=8.0
state 5 density=0.1 energy=0.1 geometry=rectangle xmin=5.0 xmax=10.0 ymin=7.0 ymax=8.0
"""
# algorithmic bytes per interior cell of each timed kernel
CONFIG2_KERNELS = ((0, "cg_w_step", 48), (1, "cg_ur_step", 48), (4, "cheby_step", 72), (5, "ppcg_inner_sweep", 64),
                   (6, "cheby32_step", 24), (7, "ppcg32_inner_sweep", 28))


def config2_deck(n: int, solver: str) -> str:
    return CONFIG2_STATES + (f"x_cells={n}\ny_cells={n}\nxmin=0.0\nymin=0.0\nxmax=10.0\nymax=10.0\n"
                             f"initial_timestep=0.004\nend_step=10\nmax_iters=40000\nuse_{solver}\neps=1e-10\n"
                             "halo_depth=2\ncoefficient=1\nsummary_frequency=10\npresteps=30\nppcg_inner_steps=10\n")


def run_config2(args):
    """The 5-state geometry of the 10x10 deck on 4096^2 cells: CG, Chebyshev
    (30 CG presteps) and PPCG (10 inner steps), 10 timesteps each at eps 1e-10
    with each solver's own convergence test, three runs of each; per-kernel
    HBM GB/s of the fused kernels on the solved fields; the CPU path's CG
    per-iteration time beside it."""
    import torch
    torch.cuda.set_device(0)
    tl = load_package()
    n = args.size if args.size != 8192 else 4096
    peak, peak_kind = measured_peaks()
    out = {"workload": f"config2: 5-state geometry on {n}^2, 10 steps, eps 1e-10", "n": n, "solvers": {}}
    chosen = [x for x in args.solvers.split(",") if x]
    for solver in [x for x in ("cg", "cheby", "ppcg") if x in chosen]:
        runs = []
        chunk = None
        for run in range(3):
            if chunk is not None:
                chunk.close()
            s = tl.Settings.from_text(config2_deck(n, solver), mode=1, exact=False)
            chunk = tl.initialiseapp(s)
            lib = chunk.lib
            chunk.check(lib.tl_synchronize(chunk.ctx))
            chunk.check(lib.tl_timer_start(chunk.ctx))
            steps, sums = tl.diffuse(chunk, s, problemfile=None)
            ms = C.c_double()
            chunk.check(lib.tl_timer_stop(chunk.ctx, C.byref(ms)))
            runs.append({"ms": ms.value, "iters": [r.iters for r in steps], "cg_iters": [r.cg_iters for r in steps],
                         "inner_iters": [r.inner_iters for r in steps], "summary": sums[-1]})
        kern = {}
        for k, name, b in CONFIG2_KERNELS:
            kms = C.c_double()
            chunk.check(chunk.lib.tl_bench_kernel(chunk.ctx, k, 10, C.byref(kms)))
            kern[name] = {"ms": kms.value, "gbs": b * n * n / (kms.value * 1e-3) / 1e9,
                          "frac": b * n * n / (kms.value * 1e-3) / 1e9 / peak}
        chunk.close()
        out["solvers"][solver] = {"runs": runs, "ms_per_run": statistics.mean(r["ms"] for r in runs),
                                  "kernels_after_solve": kern}
    # the same decks to the relative true residual 1e-10: FP64 and FP32 inside
    # FP64 refinement, each solver (one run each)
    out["relative"] = {}
    for solver in [x for x in ("cg", "cheby", "ppcg") if x in chosen]:
        for prec, pname in ((0, "fp64"), (1, "fp32_refined")):
            s = tl.Settings.from_text(config2_deck(n, solver), mode=1, exact=False, criterion=1, precision=prec)
            chunk = tl.initialiseapp(s)
            lib = chunk.lib
            chunk.check(lib.tl_synchronize(chunk.ctx))
            chunk.check(lib.tl_timer_start(chunk.ctx))
            steps, sums = tl.diffuse(chunk, s, problemfile=None)
            ms = C.c_double()
            chunk.check(lib.tl_timer_stop(chunk.ctx, C.byref(ms)))
            out["relative"][f"{solver}_{pname}"] = {
                "ms": ms.value, "iters": [r.iters for r in steps], "inner_iters": [r.inner_iters for r in steps],
                "refinements": [r.refinements for r in steps], "rel_residual_max": max(r.rel_residual for r in steps),
                "converged": all(r.converged for r in steps), "summary": sums[-1]}
            chunk.close()
    out["peak_gbs"] = peak
    out["peak_kind"] = peak_kind
    if not args.no_cpu:
        oracle = load_oracle()
        oracle.build()
        threads = os.cpu_count() or 1
        s = oracle.parse_deck(config2_deck(n, "cg"))
        ch = oracle.OracleChunk(s, oracle.make_opts(mode=oracle.MODE_TEALEAF, order=oracle.ORDER_THREADS,
                                                    nthreads=threads))
        ch.initialise()
        t = {}
        for cap in (5, 25):
            s.maxiters = cap
            ch.halo(1, ["energy", "density"])
            t0 = time.perf_counter()
            ch.solve(s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
            t[cap] = time.perf_counter() - t0
        per_iter = (t[25] - t[5]) / 20
        cg_iters = sum(out["solvers"]["cg"]["runs"][0]["iters"]) if "cg" in out["solvers"] else 0
        out["cpu_cg"] = {"ms_per_iteration": per_iter * 1e3, "cores": threads, "kind": "port",
                         "estimated_ms_per_run": per_iter * 1e3 * cg_iters}
    print(json.dumps(out))


def config4_decks(count: int = 128, seed: int = DECK_SEED + 4):
    """Seeded random-rectangle decks with nx, ny drawn from 256..2048 in steps of 128."""
    rng = np.random.default_rng(seed)
    sizes = [(int(rng.integers(2, 17)) * 128, int(rng.integers(2, 17)) * 128) for _ in range(count)]
    texts = []
    for k, (nx, ny) in enumerate(sizes):
        t = make_deck(nx, seed=seed * 1000 + k, steps=10, maxiters=40000)
        texts.append(t.replace(f"y_cells={nx}", f"y_cells={ny}"))
    return sizes, texts


def run_config4(args):
    """128 independent decks of uneven sizes, 10 timesteps each, CG to 1e-10
    relative residual, FP64 and FP32-refined: one batched graph launch per
    timestep against the same decks solved one after another by the
    single-deck solver of the same precision."""
    import torch
    torch.cuda.set_device(0)
    tl = load_package()
    sizes, texts = config4_decks(args.decks)
    steps = 10
    out = {"workload": f"config4: {len(texts)} random-rectangle decks, nx, ny in 256..2048 step 128, {steps} steps, "
                       "CG to 1e-10 relative", "cells": sum(a * b for a, b in sizes)}
    for prec, pname in ((0, "fp64"), (1, "fp32_ir")):
        out[pname] = run_config4_precision(tl, texts, steps, prec)
        # wall clock (the sequential wall includes each deck's first-use FP32
        # set-up, layout tuning included) and device loop time
        out[pname]["speedup"] = out[pname]["sequential"]["seconds"] / out[pname]["batched"]["seconds"]
        out[pname]["loop_speedup"] = out[pname]["sequential"]["loop_ms"] / out[pname]["batched"]["loop_ms"]
    print(json.dumps(out))


def run_config4_precision(tl, texts, steps, precision):
    out = {}
    for mode in ("batched", "sequential"):
        sets = [tl.Settings.from_text(t, mode=1, criterion=1, precision=precision) for t in texts]
        chunks = [tl.initialiseapp(s) for s in sets]
        lib = chunks[0].lib
        batch = tl.Batch(chunks) if mode == "batched" else None  # the batch tables: set-up, not timed
        for c in chunks:
            c.check(lib.tl_synchronize(c.ctx))
        t0 = time.perf_counter()
        iters, loop_ms, first_loop_ms = 0, 0.0, 0.0
        if mode == "batched":
            for step in range(steps):
                for c, s in zip(chunks, sets):
                    tl.haloupdate(c, s, 1, ["energy", "density"])
                res = batch.solve(sets)
                iters += sum(r.iters for r in res)
                loop_ms += res[0].solve_ms
                if step == 0:
                    first_loop_ms = res[0].solve_ms
                for c, s in zip(chunks, sets):
                    tl.solvefinished(c, s)
            batch.close()
        else:
            for c, s in zip(chunks, sets):
                for step in range(steps):
                    tl.haloupdate(c, s, 1, ["energy", "density"])
                    r = tl.CG.solve(c, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
                    iters += r.iters
                    loop_ms += r.solve_ms
                    if step == 0:
                        first_loop_ms += r.solve_ms
                    tl.solvefinished(c, s)
        for c in chunks:
            c.check(lib.tl_synchronize(c.ctx))
        wall = time.perf_counter() - t0
        summ = [tl.fieldsummary(c, s, problemfile=None)[3] for c, s in zip(chunks, sets)]
        out[mode] = {"seconds": wall, "iterations": iters, "loop_ms": loop_ms, "first_step_loop_ms": first_loop_ms,
                     "temp_summaries_first4": summ[:4]}
        for c in chunks:
            c.close()
    return out


def conv_kernel_rates(tl, n, reps=10):
    """Each convolution shape of the network (forward; and the input-gradient
    mode) on one n x n image of random BF16 activations, timed with CUDA
    events on torch's stream; FLOPs = 2 * 9 * cin * cout per pixel."""
    import torch
    lib = tl._abi.load()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}
    for ci, co, mode in ((16, 32, 1), (32, 32, 1), (32, 16, 0), (32, 32, 2)):
        x = torch.randn((1, n, n, ci), device="cuda").to(torch.bfloat16)
        w = (0.05 * torch.randn(co * 9 * ci, device="cuda")).to(torch.bfloat16)
        b = torch.zeros(co, device="cuda")
        y = torch.empty((1, n, n, co), device="cuda", dtype=torch.bfloat16)
        gz = torch.randn((1, n, n, co), device="cuda").to(torch.bfloat16) if mode == 2 else None
        g32 = torch.empty((1, n, n), device="cuda") if mode == 0 else None
        args = (x.data_ptr(), w.data_ptr(), b.data_ptr() if mode != 2 else None,
                gz.data_ptr() if gz is not None else None, None, y.data_ptr() if mode != 0 else None,
                g32.data_ptr() if g32 is not None else None, 1, n, n, ci, co, mode, st)
        for _ in range(2):
            assert lib.tl_conv3x3_forward(*args) == 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            lib.tl_conv3x3_forward(*args)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        flops = 2.0 * 9 * ci * co * n * n
        name = f"conv{ci}x{co}" + {0: "_out", 1: "_gelu", 2: "_input_grad"}[mode]
        out[name] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12,
                     "bytes": n * n * 2 * (ci + (co if mode else 2) + (co if mode == 2 else 0))}
        out[name]["gbs"] = out[name]["bytes"] / (ms * 1e-3) / 1e9
    return out


def run_config5(args):
    """The learned warm start: convolution kernel rates at n^2, one training
    step (forward + residual loss + backward + Adam on 32 crops of 128^2) and
    the A/B evaluation (plain start, network, extrapolation) on a held-out
    random deck for FP64 CG and FP32 refinement."""
    import torch
    torch.cuda.set_device(0)
    tl = load_package()
    n = args.size if args.size != 8192 else 2048
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    rates = conv_kernel_rates(tl, n)
    line = {"metric": "learned warm start: CG iterations and time to 1e-10 with and without the prediction",
            "unit": "ms", "config": {"workload": f"{n}^2 held-out random-rectangle deck", "n": n,
                                     "steps": args.steps, "seed": 900001},
            "conv_kernels": rates, "bf16_peak_tflops": bf16_peak,
            "conv_frac_of_bf16_peak": {k: v["tflops"] / bf16_peak for k, v in rates.items()}}
    params = tl.warmstart.load_params()
    traj = tl.warmstart.generate(tl, 512, [4242], 6)
    pairs, scales = tl.warmstart._pairs(traj)
    trn = tl.warmstart.Trainer(params, 32, 128, 128)
    rng = np.random.default_rng(0)
    for it in range(25):
        if it == 5:
            torch.cuda.synchronize()
            t0 = time.time()
        trn.step(tl.warmstart._random_crops(rng, traj, pairs, scales, 32, 128), 1e-6)
    torch.cuda.synchronize()
    line["train_step_ms"] = (time.time() - t0) * 1e3 / 20
    if not args.no_eval:
        ev = {}
        for prec, pname in ((0, "fp64"), (1, "fp32_ir")):
            r = tl.warmstart.evaluate(tl, params, n, 900001, args.steps, prec)
            ev[pname] = {k: {"iters": sum(v["iters"]), "ms": sum(v["ms"]),
                             "predictions_used": sum(1 for u in v["used"] if u == 1),
                             "final_rel_diff": v.get("final_rel_diff"), "iters_per_step": v["iters"],
                             "network_weight": [c[-1] for c in v["coef"]]}
                         for k, v in r.items()}
        line["eval"] = ev
        line["value"] = ev["fp32_ir"]["network"]["ms"] / args.steps
    print(json.dumps(line))


# Kernels timed by --workload kernels: (tl_bench_kernel id, name, algorithmic
# bytes per interior cell, FP64 (or FP32) arithmetic instructions per cell of
# the fused form).  FP64: the stencil w = diag p - sum k p_nbr is 5 (1 DMUL +
# 4 DFMA), each axpy-like update 1, each dot term 1.
KERNEL_TABLE = (
    (0, "cg_w_step", 56, 7),           # p' = beta p + r (1), w = A p' (5), p'.w (1); read p r kx ky diag, write p' w
    (1, "cg_ur_step", 48, 3),          # u += a p (1), r -= a w (1), r.r (1); read u p r w, write u r
    (4, "cheby_step", 80, 10),         # w = A u (5), r = u0 - w (1), p = a p + b r (2), u' = u + p (1), r.r (1)
    (5, "ppcg_inner_sweep", 64, 9),    # w = A sd (5), r -= w (1), u += sd (1), sd' = a sd + b r (2)
    (12, "ppcg_outer_update", 56, 3),  # u += a p, r -= a w (2), sd = r / theta (1 division)
    (10, "jacobi_sweep", 48, 10),      # u' = (u0 + sum k u_nbr) / (1 + sum k): 4 DFMA, 4 DADD, 1 DDIV, |u'-u| sum
    (11, "halo_u_p", None, 0),         # four face strips of two fields
    (6, "cheby32_step", 24, None),
    (7, "ppcg32_inner_sweep", 28, None),
    (8, "ir_dir_step", 16, None),
    (9, "ir_update_step", 24, None),
)


def run_kernels(args):
    """Every fused iteration kernel launched from the host (`--reps` back to
    back launches each, CUDA events on the library's stream) on the fields of
    the 5-state deck at n^2 (4096 by default) after a short FP64 and a short
    FP32-refined CG solve: per kernel the time, the algorithmic GB/s and its
    fraction of the measured HBM peak.  Also the launch source for per-kernel
    ncu captures (-k regex:<Op name> -c 1)."""
    import torch
    torch.cuda.set_device(0)
    tl = load_package()
    n = args.size if args.size != 8192 else 4096
    peak, peak_kind = measured_peaks()
    out = {"workload": f"5-state deck on {n}^2 after 60 FP64 and 60 FP32-refined CG iterations, "
                       f"{args.reps} launches per kernel", "n": n, "peak_gbs": peak, "peak_kind": peak_kind,
           "kernels": {}}
    s = tl.Settings.from_text(config2_deck(n, "cg"), mode=1, exact=False, criterion=1)
    chunk = tl.initialiseapp(s)
    s.maxiters = 60
    tl.haloupdate(chunk, s, 1, ["energy", "density"])
    tl.CG.solve(chunk, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    s.precision = 1
    tl.CG.solve(chunk, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    cells = n * n
    for k, name in ((0, "cg_w_step"), (1, "cg_ur_step"), (8, "ir_dir_step"), (9, "ir_update_step")):
        w, r, blk = C.c_int(), C.c_int(), C.c_int()
        chunk.check(chunk.lib.tl_get_layout(chunk.ctx, k, C.byref(w), C.byref(r), C.byref(blk)))
        out.setdefault("layouts", {})[name] = {"warps": w.value, "rows": r.value, "blocks": blk.value}
    for k, name, b, ops in KERNEL_TABLE:
        ms = C.c_double()
        chunk.check(chunk.lib.tl_bench_kernel(chunk.ctx, k, args.reps, C.byref(ms)))
        d = {"ms": ms.value}
        if b is not None:
            d["bytes_per_cell"] = b
            d["gbs"] = b * cells / (ms.value * 1e-3) / 1e9
            d["frac"] = d["gbs"] / peak
        if ops:
            d["fp64_ops_per_cell"] = ops
            d["fp64_gops"] = ops * cells / (ms.value * 1e-3) / 1e9
        out["kernels"][name] = d
    chunk.close()
    print(json.dumps(out))


def run_cpucheck(args):
    """Checks the CPU baseline's linear model: timestep 1 of the deck solved
    to convergence (1e-10 relative residual) by the oracle's tealeaf-mode CG
    on all host cores, beside the time the bounded 10- and 330-iteration
    sample predicts for the same iteration count."""
    oracle = load_oracle()
    oracle.build()
    threads = os.cpu_count() or 1
    n = args.size
    s = oracle.parse_deck(make_deck(n))
    o = oracle.make_opts(mode=oracle.MODE_TEALEAF, order=oracle.ORDER_THREADS, nthreads=threads, criterion=1)
    ch = oracle.OracleChunk(s, o)
    ch.initialise()
    ch.halo(1, ["energy", "density"])
    t0 = time.perf_counter()
    r = ch.solve(s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    full_ms = (time.perf_counter() - t0) * 1e3
    del ch
    pred, pi, wall = cpu_sample(oracle, n, r.iters, threads)
    out = {"workload": f"timestep 1 of the {n}^2 deck, oracle CG to 1e-10 relative, {threads} threads",
           "iterations": r.iters, "rel_residual": r.rel_residual, "converged": bool(r.converged),
           "measured_ms": full_ms, "sample_predicted_ms": pred, "sample_ms_per_iteration": pi,
           "sample_seconds": wall, "predicted_over_measured": pred / full_ms}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--variant", default="all", choices=["all"] + list(VARIANTS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-single", action="store_true", help="skip the single-thread CPU sample")
    ap.add_argument("--no-config4", action="store_true", help="skip the batched 128-deck leg of the headline run")
    ap.add_argument("--workload", default="timestep", choices=["timestep", "config2", "config4", "config5", "cpucheck", "kernels"],
                    help="timestep: the headline line; config2: the 4096^2 CG/Cheby/PPCG suite; "
                         "config4: 128 uneven decks, batched against sequential; config5: the learned warm "
                         "start (kernel rates, training step, A/B evaluation; --size, --steps); cpucheck: one "
                         "converged CPU timestep against the CPU sample's prediction; kernels: every fused "
                         "kernel launched from the host on the 4096^2 deck (--reps), for per-kernel rates and ncu")
    ap.add_argument("--no-eval", action="store_true", help="config5: kernel rates and training step only")
    ap.add_argument("--solvers", default="cg,cheby,ppcg", help="config2: the solvers to run (comma list)")
    ap.add_argument("--decks", type=int, default=128)
    ap.add_argument("--reps", type=int, default=20, help="kernels: launches per kernel")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.workload == "config2":
        run_config2(args)
    elif args.workload == "config4":
        run_config4(args)
    elif args.workload == "config5":
        run_config5(args)
    elif args.workload == "cpucheck":
        run_cpucheck(args)
    elif args.workload == "kernels":
        run_kernels(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
