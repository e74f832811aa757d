"""Helpers shared by the parity tests: run one deck through the CUDA library
(via the host mirror and the C ABI) and through the CPU oracle."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
CONFIG1 = (GOLDEN / "tea_config1.in").read_text()

FIELDS = ["density", "energy0", "energy", "u", "u0", "p", "r", "w", "kx", "ky", "sd"]
SOLVER_CODES = {"cg": 0, "cheby": 1, "ppcg": 2, "jacobi": 3}


def deck_text(base: str = CONFIG1, **kv) -> str:
    """The config-1 deck with keys replaced or added (key=value lines)."""
    lines = []
    seen = set()
    for ln in base.split("\n"):
        s = ln.strip()
        if "=" in s and not s.startswith("state") and not s.startswith("*"):
            key = s.split("=")[0].strip()
            if key in kv:
                lines.append(f"{key}={kv[key]}")
                seen.add(key)
                continue
        if s.startswith("use_") and "solver" in kv:
            lines.append(f"use_{kv['solver']}")
            seen.add("solver")
            continue
        lines.append(ln)
    extra = [f"{k}={v}" for k, v in kv.items() if k not in seen and k != "solver"]
    if "solver" in kv and "solver" not in seen:
        extra.append(f"use_{kv['solver']}")
    return "\n".join(extra + lines)


def random_deck(n: int, seed: int, nrect: int = 6, steps: int = 2, eps: float = 1e-15, ny: int | None = None,
                solver: str = "cg", **kv) -> str:
    """Seeded random-rectangle deck: background rho=100 e=1e-4 plus rectangles
    with corners in [0,10]^2, rho log-uniform in [0.1, 100], e in [0.1, 25]."""
    rng = np.random.default_rng(seed)
    lines = ["state 1 density=100.0 energy=0.0001"]
    for k in range(nrect):
        x0, x1 = sorted(float(v) for v in rng.uniform(0, 10, 2))
        y0, y1 = sorted(float(v) for v in rng.uniform(0, 10, 2))
        rho = float(10 ** rng.uniform(-1, 2))
        e = float(rng.uniform(0.1, 25))
        lines.append(f"state {k + 2} density={rho!r} energy={e!r} geometry=rectangle xmin={x0!r} xmax={x1!r} "
                     f"ymin={y0!r} ymax={y1!r}")
    lines += [f"x_cells={n}", f"y_cells={ny or n}", "xmin=0.0", "ymin=0.0", "xmax=10.0", "ymax=10.0",
              "initial_timestep=0.004", f"end_step={steps}", "max_iters=5000", f"use_{solver}", f"eps={eps!r}",
              "halo_depth=2", "coefficient=1", "summary_frequency=10"]
    lines += [f"{k}={v}" for k, v in kv.items()]
    return "\n".join(lines) + "\n"


def gpu_run(tl, text: str, mode: int, exact: bool = False, steps_fields: bool = False, **overrides):
    """diffuse! on the GPU; returns (chunk, per-step results, summaries, per-step fields)."""
    s = tl.Settings.from_text(text, mode=mode, exact=exact, **overrides)
    chunk = tl.initialiseapp(s)
    per_step = []
    results = []
    summaries = []
    solver = tl.SOLVERS[s.solver]
    for tt in range(1, s.endstep + 1):
        rx = s.dtinit / s.dx ** 2
        ry = s.dtinit / s.dy ** 2
        tl.haloupdate(chunk, s, 1, ["energy", "density"])
        results.append(solver.solve(chunk, s, rx, ry))
        tl.solvefinished(chunk, s)
        if tt % s.summaryfrequency == 0:
            summaries.append(tl.fieldsummary(chunk, s, problemfile=None))
        if steps_fields:
            per_step.append({f: chunk.field(f).copy() for f in FIELDS})
    summaries.append(tl.fieldsummary(chunk, s, problemfile=None))
    return chunk, results, summaries, per_step


def oracle_run(text: str, mode: int, order: int = O.ORDER_REFERENCE, layout=None, steps_fields=False,
               solver: str | None = None, criterion: int = 0, nthreads: int = 1):
    s = O.parse_deck(text)
    if solver:
        s.solver = SOLVER_CODES[solver]
    o = O.make_opts(mode=mode, order=order, layout=layout, criterion=criterion, nthreads=nthreads)
    ch = O.OracleChunk(s, o)
    ch.initialise()
    if not steps_fields:
        steps, sums = ch.diffuse()
        return ch, steps, sums, []
    # step by step, mirroring diffuse! (TeaLeaf.jl:67-80)
    per_step, results, sums = [], [], []
    rx = s.dtinit / s.dx ** 2
    ry = s.dtinit / s.dy ** 2
    for tt in range(1, s.endstep + 1):
        ch.halo(1, ["energy", "density"])
        results.append(ch.solve(rx, ry))
        ch.solve_finished()
        if tt % s.summaryfrequency == 0:
            sums.append(ch.summary())
        per_step.append({f: ch.field(f).copy() for f in FIELDS})
    sums.append(ch.summary())
    return ch, results, sums, per_step


def rel(a, b):
    a, b = float(a), float(b)
    if a == b:
        return 0.0
    return abs(a - b) / max(abs(a), abs(b), 1e-300)
