"""tealeaf_gb300 -- host-side mirror of TeaLeaf.jl's solve interface, backed by
the sm_103a CUDA library libtealeaf_gb300.so.

The names follow the reference (Julia's `!` dropped):

    set = Settings.from_file("tea.in")          # Settings(infile)      settings.jl:90
    chunk = initialiseapp(set)                  # initialiseapp!        TeaLeaf.jl:35
    diffuse(chunk, set)                         # diffuse!              TeaLeaf.jl:62
    CG.solve(chunk, set, rx, ry)                # solve! plugin         CG.jl:7
    haloupdate(chunk, set, 1, ["u", "p"])       # haloupdate!           kernels.jl:146
    solvefinished(chunk, set)                   # solvefinished!        kernels.jl:166
    fieldsummary(chunk, set)                    # fieldsummary          kernels.jl:119

A Chunk owns a device context: every field stays resident in HBM across
timesteps; `chunk.field(name)` downloads a copy in the reference's
column-major (X, Y) layout, `chunk.set_field` uploads one.
"""
from __future__ import annotations

import ctypes as C
import logging
import os
from dataclasses import dataclass
from typing import Iterable, List, Optional

import numpy as np

from . import _abi
from ._abi import TeaLeafError
from .settings import (CIRCULAR, CONDUCTIVITY, POINT, RECIP_CONDUCTIVITY, RECTANGULAR, Settings, State,
                       checkingvalue, qa_passes)

log = logging.getLogger("tealeaf_gb300")

__all__ = ["Settings", "State", "Chunk", "initialiseapp", "diffuse", "haloupdate", "solvefinished",
           "fieldsummary", "copyu", "residual", "finalise", "CG", "Cheby", "PPCG", "Jacobi", "SolveResult",
           "TeaLeafError", "CONDUCTIVITY", "RECIP_CONDUCTIVITY", "debugrecord"]

ERROR_START = 1e10


@dataclass
class SolveResult:
    iters: int
    cg_iters: int
    inner_iters: int
    est_iters: int
    error: float
    eigmin: float
    eigmax: float
    converged: bool
    refinements: int
    rel_residual: float
    solve_ms: float
    launches: int
    warm: int = 0              # 0 plain start, 1 the prediction was used, 2 it lost to the plain start
    r0_plain: float = -1.0     # initial relative residual of the plain start (warm start asked)
    r0_pred: float = -1.0      # the same for the prediction (-1: none made)
    warm_coef: tuple = ()      # the prediction's weights on u^n, u^{n-1}, ..., u^{n-6}, network term


class Chunk:
    """Chunk(settings) (src/chunk.jl:68-89) on the GPU."""

    def __init__(self, settings: Settings, mode: Optional[int] = None):
        self.lib = _abi.load()
        self.settings = settings
        self.mode = settings.mode if mode is None else mode
        self.halodepth = settings.halodepth
        self.x = settings.xcells + 2 * settings.halodepth
        self.y = settings.ycells + 2 * settings.halodepth
        cfg = _abi.Config(settings.xcells, settings.ycells, settings.halodepth, settings.maxiters, settings.xmin,
                          settings.ymin, settings.dx, settings.dy, self.mode)
        self._ctx = C.c_void_p()
        rc = self.lib.tl_create(C.byref(self._ctx), C.byref(cfg))
        if rc:
            msg = self.lib.tl_last_error(self._ctx)
            self.lib.tl_destroy(self._ctx)
            self._ctx = None
            raise TeaLeafError(rc, msg.decode() if msg else f"tl_create status {rc}")

    @property
    def ctx(self):
        return self._ctx

    def close(self):
        if getattr(self, "_ctx", None):
            self.lib.tl_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()

    def check(self, rc: int):
        _abi.check(self.lib, self._ctx, rc)

    def size(self):
        return self.x, self.y

    def field(self, name: str) -> np.ndarray:
        """A host copy of one field as an (X, Y) array (index [i, j])."""
        k = _abi.FIELDS.index(name)
        buf = np.empty((self.y, self.x), dtype=np.float64)   # C order: column j of (X, Y) is row j
        self.check(self.lib.tl_download(self._ctx, k, buf.ctypes.data_as(C.POINTER(C.c_double)), self.x))
        return buf.T

    def set_field(self, name: str, a: np.ndarray):
        k = _abi.FIELDS.index(name)
        a = np.asarray(a, dtype=np.float64)
        if a.shape != (self.x, self.y):
            raise ValueError(f"field shape {a.shape} != {(self.x, self.y)}")
        buf = np.ascontiguousarray(a.T)
        self.check(self.lib.tl_upload(self._ctx, k, buf.ctypes.data_as(C.POINTER(C.c_double)), self.x))

    def cg_coefficients(self, n: int):
        al = np.zeros(n)
        be = np.zeros(n)
        self.check(self.lib.tl_get_cg_coefficients(self._ctx, al.ctypes.data_as(C.POINTER(C.c_double)),
                                                    be.ctypes.data_as(C.POINTER(C.c_double)), n))
        return al, be

    def reduction_layout(self):
        w, r, b = C.c_int(), C.c_int(), C.c_int()
        self.check(self.lib.tl_reduction_layout(self._ctx, C.byref(w), C.byref(r), C.byref(b)))
        return w.value, r.value, b.value

    def set_states(self, settings: Settings):
        arr = _state_array(settings, self.mode)
        self.check(self.lib.tl_set_states(self._ctx, arr, len(settings.states)))

    def warm_load(self, params: np.ndarray):
        """Loads a warm-start network (FP32 vector of _abi.WARM_NPARAMS values)."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        self.check(self.lib.tl_warm_load(self._ctx, p.ctypes.data_as(C.POINTER(C.c_float)), p.size))

    def warm_reset(self):
        """Forgets the previous step: the next warm-start solve makes no prediction."""
        self.check(self.lib.tl_warm_reset(self._ctx))


def _state_array(settings: Settings, mode: int):
    n = len(settings.states)
    arr = (_abi.State * max(n, 1))()
    for k, st in enumerate(settings.states):
        xmin, ymin, xmax, ymax = st.bounds(settings, mode)
        arr[k] = _abi.State(st.density, st.energy, xmin, ymin, xmax, ymax, st.radius, st.geometry)
    return arr


def setchunkstate(chunk: Chunk, settings: Settings):
    """setchunkstate! (src/chunk.jl:122-151)."""
    chunk.set_states(settings)


def initialiseapp(settings: Settings, mode: Optional[int] = None) -> Chunk:
    """initialiseapp! (src/TeaLeaf.jl:35-44)."""
    chunk = Chunk(settings, mode)
    arr = _state_array(settings, chunk.mode)
    chunk.check(chunk.lib.tl_initialise(chunk.ctx, arr, len(settings.states)))
    # the reference marks density, energy0, energy for exchange here
    settings.resettoexchange()
    for f in ("density", "energy0", "energy"):
        settings.toexchange[f] = True
    return chunk


def haloupdate(chunk: Chunk, settings: Settings, depth: int, toex: Optional[Iterable[str]] = None,
               reset: bool = True):
    """haloupdate!(chunk, set, depth[, toex][, reset]) (src/kernels.jl:146-159)."""
    if toex is not None:
        toex = list(toex)
        idx = (C.c_int * max(len(toex), 1))(*[_abi.EXCHANGE_FIELDS.index(f) for f in toex])
        chunk.check(chunk.lib.tl_halo_update(chunk.ctx, depth, idx, len(toex), int(reset)))
        if reset:
            settings.resettoexchange()
        for f in toex:
            settings.toexchange[f] = True
    else:
        marked = [f for f in _abi.EXCHANGE_FIELDS if settings.toexchange[f]]
        idx = (C.c_int * max(len(marked), 1))(*[_abi.EXCHANGE_FIELDS.index(f) for f in marked])
        chunk.check(chunk.lib.tl_halo_update(chunk.ctx, depth, idx, len(marked), 1))


def copyu(chunk: Chunk, settings: Settings = None):
    chunk.check(chunk.lib.tl_copy_u(chunk.ctx))


def residual(chunk: Chunk, settings: Settings = None):
    chunk.check(chunk.lib.tl_residual(chunk.ctx))


def finalise(chunk: Chunk, settings: Settings = None):
    chunk.check(chunk.lib.tl_finalise(chunk.ctx))


def solvefinished(chunk: Chunk, settings: Settings):
    """solvefinished! (src/kernels.jl:166-170)."""
    chunk.check(chunk.lib.tl_solve_finished(chunk.ctx, int(settings.checkresult)))
    settings.toexchange["energy"] = True


def fieldsummary(chunk: Chunk, settings: Settings, problemfile: Optional[str] = None):
    """fieldsummary (src/kernels.jl:119-133).  Returns (vol, mass, ie, temp),
    or None when checkresult is off; logs the QA verdict when a tea.problems
    file is given or present."""
    if not settings.checkresult:
        return None
    out = (C.c_double * 4)()
    chunk.check(chunk.lib.tl_field_summary(chunk.ctx, out))
    vol, mass, ie, temp = out[0], out[1], out[2], out[3]
    pf = problemfile if problemfile is not None else ("tea.problems" if os.path.exists("tea.problems") else None)
    if pf is not None:
        cv = checkingvalue(settings, pf)
        log.info("Checking results... cv=%r actual=%r", cv, temp)
        if qa_passes(temp, cv):
            log.info("This run PASSED qa_diff=%r", abs(100 * temp / cv - 100.0))
        else:
            log.warning("This run FAILED qa_diff=%r", abs(100 * temp / cv - 100.0))
    return vol, mass, ie, temp


def _params(settings: Settings, solver: int) -> _abi.Params:
    return _abi.Params(solver, settings.coefficient, settings.maxiters, settings.presteps,
                       settings.ppcginnersteps, int(settings.errorswitch), settings.eps, settings.epslim,
                       settings.criterion, settings.precision, int(settings.exact), int(settings.warmstart))


def _solve(chunk: Chunk, settings: Settings, rx: float, ry: float, solver: int) -> SolveResult:
    prm = _params(settings, solver)
    res = _abi.Result()
    rc = chunk.lib.tl_solve(chunk.ctx, rx, ry, C.byref(prm), C.byref(res))
    chunk.check(rc)
    ms = C.c_double()
    chunk.lib.tl_last_solve_ms(chunk.ctx, C.byref(ms))
    # the exchange marks the solver leaves behind (CG.jl:11, Cheby.jl:78, PPCG.jl:92, Jacobi.jl:54)
    settings.resettoexchange()
    if solver == _abi.SOLVER_CG:
        settings.toexchange["u"] = settings.toexchange["p"] = True
    elif solver == _abi.SOLVER_CHEBY:
        settings.toexchange["u"] = True
        if res.inner_iters == 0:
            settings.toexchange["p"] = True
    elif solver == _abi.SOLVER_PPCG:
        settings.toexchange["p"] = True
        if res.inner_iters == 0:
            settings.toexchange["u"] = True
    else:
        settings.toexchange["u"] = True
    r = SolveResult(res.iters, res.cg_iters, res.inner_iters, res.est_iters, res.error, res.eigmin, res.eigmax,
                    bool(res.converged), res.refinements, res.rel_residual, ms.value, res.launches, res.warm,
                    res.r0_plain, res.r0_pred, tuple(res.warm_coef))
    log.info("solve complete iters=%d error=%r", r.iters, r.error)
    return r


class _SolverModule:
    """A solver plugin: `solve(chunk, settings, rx, ry)` like the reference's modules."""

    def __init__(self, name: str, code: int):
        self.__name__ = name
        self.code = code

    def solve(self, chunk: Chunk, settings: Settings, rx: float, ry: float) -> SolveResult:
        return _solve(chunk, settings, rx, ry, self.code)

    def __repr__(self):
        return f"<solver {self.__name__}>"


CG = _SolverModule("CG", _abi.SOLVER_CG)
Cheby = _SolverModule("Cheby", _abi.SOLVER_CHEBY)
PPCG = _SolverModule("PPCG", _abi.SOLVER_PPCG)
Jacobi = _SolverModule("Jacobi", _abi.SOLVER_JACOBI)
SOLVERS = {_abi.SOLVER_CG: CG, _abi.SOLVER_CHEBY: Cheby, _abi.SOLVER_PPCG: PPCG, _abi.SOLVER_JACOBI: Jacobi}


def diffuse(chunk: Chunk, settings: Settings, problemfile: Optional[str] = None):
    """diffuse! (src/TeaLeaf.jl:62-83).  Returns the per-step solve results and
    the field summaries taken (every summaryfrequency steps and at the end)."""
    if settings.debugfile and os.path.isfile(settings.debugfile):
        os.remove(settings.debugfile)
    steps: List[SolveResult] = []
    summaries = []
    solver = SOLVERS[settings.solver]
    for tt in range(1, settings.endstep + 1):
        debugrecord(settings, chunk)
        rx = settings.dtinit / settings.dx ** 2
        ry = settings.dtinit / settings.dy ** 2
        haloupdate(chunk, settings, 1, ["energy", "density"])
        steps.append(solver.solve(chunk, settings, rx, ry))
        solvefinished(chunk, settings)
        if tt % settings.summaryfrequency == 0:
            s = fieldsummary(chunk, settings, problemfile)
            if s is not None:
                summaries.append(s)
        log.info("Timestep %d finished", tt)
    s = fieldsummary(chunk, settings, problemfile)
    if s is not None:
        summaries.append(s)
    return steps, summaries


class Batch:
    """Many independent decks (tealeaf-mode Chunks of any sizes) whose CG
    solves run together in one graph launch (tl_batch_*)."""

    def __init__(self, chunks):
        self.lib = _abi.load()
        self.chunks = list(chunks)
        arr = (C.c_void_p * len(self.chunks))(*[c.ctx.value for c in self.chunks])
        self._b = C.c_void_p()
        rc = self.lib.tl_batch_create(C.byref(self._b), arr, len(self.chunks))
        if rc:
            msg = self.lib.tl_batch_last_error(self._b).decode()
            self.lib.tl_batch_destroy(self._b)
            self._b = None
            raise TeaLeafError(rc, msg)

    def close(self):
        if getattr(self, "_b", None):
            self.lib.tl_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()

    def solve(self, settings_list) -> List[SolveResult]:
        """CG.solve!(chunk, set, rx, ry) for every deck at once; the solver
        parameters (eps, maxiters, coefficient, criterion, precision: FP64 or
        FP32-refined) come from the first deck's settings, rx/ry from each
        deck's own."""
        n = len(self.chunks)
        rx = (C.c_double * n)(*[s.dtinit / s.dx ** 2 for s in settings_list])
        ry = (C.c_double * n)(*[s.dtinit / s.dy ** 2 for s in settings_list])
        prm = _params(settings_list[0], _abi.SOLVER_CG)
        prm.exact = 0
        prm.warmstart = 0
        res = (_abi.Result * n)()
        rc = self.lib.tl_batch_solve(self._b, rx, ry, C.byref(prm), res)
        if rc:
            raise TeaLeafError(rc, self.lib.tl_batch_last_error(self._b).decode())
        ms = C.c_double()
        self.lib.tl_batch_last_ms(self._b, C.byref(ms))
        out = []
        for k, s in enumerate(settings_list):
            s.resettoexchange()
            s.toexchange["u"] = s.toexchange["p"] = True
            r = res[k]
            out.append(SolveResult(r.iters, r.cg_iters, r.inner_iters, r.est_iters, r.error, r.eigmin, r.eigmax,
                                   bool(r.converged), r.refinements, r.rel_residual, ms.value, r.launches))
        return out


def diffuse_batch(chunks, settings_list, steps: Optional[int] = None):
    """diffuse! over many decks with batched CG solves: per timestep the halo
    of energy and density of every deck, one batched solve, solvefinished!.
    Returns per step the list of per-deck results and the batch's loop time."""
    batch = Batch(chunks)
    history = []
    try:
        nsteps = steps if steps is not None else min(s.endstep for s in settings_list)
        for _ in range(nsteps):
            for c, s in zip(chunks, settings_list):
                haloupdate(c, s, 1, ["energy", "density"])
            history.append(batch.solve(settings_list))
            for c, s in zip(chunks, settings_list):
                solvefinished(c, s)
    finally:
        batch.close()
    return history


_CHUNK_DUMP_FIELDS = ["density0", "density", "energy0", "energy", "u", "u0", "p", "r", "mi", "w", "kx", "ky",
                      "sd"]


def debugrecord(settings: Settings, chunk: Chunk):
    """debugrecord (src/TeaLeaf.jl:90-107): appends every field to
    settings.debugfile, each column of the (X, Y) array on one line."""
    if not settings.debugfile:
        return
    with open(settings.debugfile, "a") as fh:
        for name in _CHUNK_DUMP_FIELDS:
            a = chunk.field(name)
            fh.write(name + "\n")
            fh.write("\n".join(" ".join(_julia_repr(v) for v in a[:, j]) for j in range(a.shape[1])) + "\n")
            fh.write("\n")
        fh.write("\n\n")


def _julia_repr(v: float) -> str:
    """Julia's `print` of a Float64: the shortest round-trip digits (the same
    digits Python's repr finds), written in fixed form when the decimal point
    falls at -4 < pt <= 6 digits from the first digit (and the value is not an
    integer whose exact value differs from its shortest digits), otherwise as
    d.ddde<exp>."""
    import decimal
    import math
    v = float(v)
    if v != v:
        return "NaN"
    if math.isinf(v):
        return "Inf" if v > 0 else "-Inf"
    sign = "-" if math.copysign(1.0, v) < 0 else ""
    if v == 0:
        return sign + "0.0"
    t = decimal.Decimal(repr(abs(v))).normalize().as_tuple()
    digits = "".join(str(d) for d in t.digits)
    olength = len(digits)
    pt = t.exponent + olength
    fixed = -4 < pt <= 6
    if fixed and pt >= olength:
        fixed = not abs(math.fmod(abs(v) + 0.05, 10.0 ** (pt - olength)) - 0.05) > 0.05
    if fixed:
        if pt <= 0:
            body = "0." + "0" * (-pt) + digits
        elif pt >= olength:
            body = digits + "0" * (pt - olength) + ".0"
        else:
            body = digits[:pt] + "." + digits[pt:]
    else:
        body = digits[0] + "." + (digits[1:] or "0") + "e" + str(pt - 1)
    return sign + body


from . import warmstart  # noqa: E402  (learned warm start: network file, training, evaluation)
