"""ctypes binding of the CPU oracle (tealeaf_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline leg
of the benchmark use this module as the checker.  The product never imports
it.  Parity is unpinned: the restated reference is Julia code that cannot run
on these machines and ships no golden data (see tealeaf_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libtealeaf_oracle.so"

MAX_STATES = 64
FIELDS = ["density0", "density", "energy0", "energy", "u", "u0", "p", "r", "mi", "w", "kx", "ky", "sd",
          "volume"]
EXCHANGE = ["density", "p", "energy0", "energy", "u", "sd"]   # src/chunk.jl:12
SOLVERS = {"cg": 0, "cheby": 1, "ppcg": 2, "jacobi": 3}
MODE_REFERENCE, MODE_TEALEAF = 0, 1
ORDER_REFERENCE, ORDER_DEVICE, ORDER_THREADS = 0, 1, 2
ERR_REFERENCE_THROWS = 5


class State(C.Structure):
    _fields_ = [("density", C.c_double), ("energy", C.c_double), ("xmin", C.c_double), ("ymin", C.c_double),
                ("xmax", C.c_double), ("ymax", C.c_double), ("radius", C.c_double), ("geometry", C.c_int),
                ("given", C.c_int), ("pdx", C.c_double), ("pdy", C.c_double)]


class Settings(C.Structure):
    _fields_ = [("endstep", C.c_longlong), ("presteps", C.c_int), ("maxiters", C.c_int),
                ("coefficient", C.c_int), ("ppcginnersteps", C.c_int), ("summaryfrequency", C.c_int),
                ("halodepth", C.c_int), ("errorswitch", C.c_int), ("checkresult", C.c_int),
                ("eps", C.c_double), ("dtinit", C.c_double), ("endtime", C.c_double), ("epslim", C.c_double),
                ("solver", C.c_int), ("xcells", C.c_int), ("ycells", C.c_int),
                ("xmin", C.c_double), ("ymin", C.c_double), ("xmax", C.c_double), ("ymax", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("nstates", C.c_int),
                ("states", State * MAX_STATES), ("toexchange", C.c_int * 6)]


class Opts(C.Structure):
    _fields_ = [("mode", C.c_int), ("order", C.c_int), ("dev_warps", C.c_int), ("dev_rows", C.c_int),
                ("dev_blocks", C.c_int), ("nthreads", C.c_int), ("criterion", C.c_int)]


class Chunk(C.Structure):
    _fields_ = [("f", C.POINTER(C.c_double) * 14), ("vertexx", C.POINTER(C.c_double)),
                ("vertexy", C.POINTER(C.c_double)), ("cellx", C.POINTER(C.c_double)),
                ("celly", C.POINTER(C.c_double)), ("theta", C.c_double), ("eigmin", C.c_double),
                ("eigmax", C.c_double), ("cgalpha", C.POINTER(C.c_double)), ("cgbeta", C.POINTER(C.c_double)),
                ("chebyalpha", C.POINTER(C.c_double)), ("chebybeta", C.POINTER(C.c_double)),
                ("x", C.c_int), ("y", C.c_int), ("hd", C.c_int), ("maxiters", C.c_int)]


class Result(C.Structure):
    _fields_ = [("iters", C.c_int), ("cg_iters", C.c_int), ("inner_iters", C.c_int), ("est_iters", C.c_int),
                ("error", C.c_double), ("eigmin", C.c_double), ("eigmax", C.c_double), ("status", C.c_int),
                ("converged", C.c_int), ("rel_residual", C.c_double)]


class Summary(C.Structure):
    _fields_ = [("vol", C.c_double), ("mass", C.c_double), ("ie", C.c_double), ("temp", C.c_double)]


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (no FMA contraction, OpenMP for the baseline)."""
    src = HERE / "tealeaf_oracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(src.stat().st_mtime,
                                                                (HERE / "tealeaf_oracle.h").stat().st_mtime):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-o", str(tmp),
                           str(src), "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.POINTER
        L.tlo_parse_deck.argtypes = [C.c_char_p, P(Settings), C.c_char_p, C.c_int]
        L.tlo_chunk_create.argtypes = [P(Settings), P(Opts), P(C.c_int)]
        L.tlo_chunk_create.restype = P(Chunk)
        L.tlo_chunk_free.argtypes = [P(Chunk)]
        L.tlo_initialise_app.argtypes = [P(Chunk), P(Settings), P(Opts)]
        L.tlo_set_chunk_state.argtypes = [P(Chunk), P(Settings), P(Opts)]
        L.tlo_halo_update.argtypes = [P(Chunk), P(Settings), P(Opts), C.c_int, P(C.c_int), C.c_int, C.c_int]
        L.tlo_solve.argtypes = [P(Chunk), P(Settings), P(Opts), C.c_double, C.c_double, P(Result)]
        L.tlo_solve_finished.argtypes = [P(Chunk), P(Settings), P(Opts)]
        L.tlo_field_summary.argtypes = [P(Chunk), P(Opts), P(Summary)]
        L.tlo_diffuse.argtypes = [P(Chunk), P(Settings), P(Opts), P(Result), C.c_int, P(Summary), C.c_int,
                                  P(C.c_int)]
        L.tlo_cg_init.argtypes = [P(Chunk), C.c_int, C.c_double, C.c_double, P(Opts), P(C.c_double)]
        L.tlo_cg_calc_w.argtypes = [P(Chunk), P(Opts)]
        L.tlo_cg_calc_w.restype = C.c_double
        L.tlo_cg_calc_ur.argtypes = [P(Chunk), C.c_double, P(Opts)]
        L.tlo_cg_calc_ur.restype = C.c_double
        L.tlo_cg_calc_p.argtypes = [P(Chunk), C.c_double, P(Opts)]
        L.tlo_copy_u.argtypes = [P(Chunk), P(Opts)]
        L.tlo_residual.argtypes = [P(Chunk), P(Opts)]
        L.tlo_finalise.argtypes = [P(Chunk), P(Opts)]
        L.tlo_pairwise_sum.argtypes = [P(C.c_double), C.c_longlong]
        L.tlo_pairwise_sum.restype = C.c_double
        L.tlo_device_sum.argtypes = [P(C.c_double), C.c_int, C.c_int, P(Opts)]
        L.tlo_device_sum.restype = C.c_double
        L.tlo_last_message.restype = C.c_char_p
        L.tlo_effective_bounds.argtypes = [P(Settings), P(State), C.c_int, P(C.c_double)]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oracle error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc:
        raise OracleError(rc, lib().tlo_last_message().decode())


def parse_deck(text: str) -> Settings:
    s = Settings()
    msg = C.create_string_buffer(512)
    _check(lib().tlo_parse_deck(text.encode(), C.byref(s), msg, 512))
    return s


def make_opts(mode=MODE_TEALEAF, order=ORDER_REFERENCE, layout=None, nthreads=1, criterion=0) -> Opts:
    """criterion 1: CG's relative test on the recursive then the true residual
    (the GPU library's TL_CRIT_RELATIVE); 0: the reference's own test."""
    o = Opts()
    o.mode, o.order, o.nthreads, o.criterion = mode, order, nthreads, criterion
    if layout is not None:
        o.dev_warps, o.dev_rows, o.dev_blocks = layout
    return o


class OracleChunk:
    """The reference's Chunk + driver calls, on the CPU oracle."""

    def __init__(self, settings: Settings, opts: Opts):
        self.s = settings
        self.o = opts
        st = C.c_int(0)
        self.c = lib().tlo_chunk_create(C.byref(self.s), C.byref(self.o), C.byref(st))
        if not self.c:
            raise OracleError(st.value, lib().tlo_last_message().decode())
        self.X, self.Y = self.c.contents.x, self.c.contents.y

    def __del__(self):
        if getattr(self, "c", None):
            lib().tlo_chunk_free(self.c)
            self.c = None

    def field(self, name: str) -> np.ndarray:
        """Column-major (X, Y) view, returned as a numpy array indexed [i, j]."""
        k = FIELDS.index(name)
        ptr = self.c.contents.f[k]
        a = np.ctypeslib.as_array(ptr, shape=(self.Y, self.X))  # row j holds column j of the (X,Y) array
        return a.T

    def set_field(self, name, arr):
        self.field(name)[...] = arr

    def initialise(self):
        _check(lib().tlo_initialise_app(self.c, C.byref(self.s), C.byref(self.o)))

    def halo(self, depth, fields=None, reset=True):
        if fields is None:
            _check(lib().tlo_halo_update(self.c, C.byref(self.s), C.byref(self.o), depth, None, -1, int(reset)))
        else:
            arr = (C.c_int * len(fields))(*[EXCHANGE.index(f) for f in fields])
            _check(lib().tlo_halo_update(self.c, C.byref(self.s), C.byref(self.o), depth, arr, len(fields),
                                         int(reset)))

    def solve(self, rx, ry) -> Result:
        r = Result()
        rc = lib().tlo_solve(self.c, C.byref(self.s), C.byref(self.o), rx, ry, C.byref(r))
        if rc:
            raise OracleError(rc, lib().tlo_last_message().decode())
        return r

    def solve_finished(self):
        _check(lib().tlo_solve_finished(self.c, C.byref(self.s), C.byref(self.o)))

    def summary(self):
        out = Summary()
        lib().tlo_field_summary(self.c, C.byref(self.o), C.byref(out))
        return out.vol, out.mass, out.ie, out.temp

    def diffuse(self):
        n = int(self.s.endstep)
        steps = (Result * n)()
        sums = (Summary * (n + 1))()
        ns = C.c_int(0)
        rc = lib().tlo_diffuse(self.c, C.byref(self.s), C.byref(self.o), steps, n, sums, n + 1, C.byref(ns))
        if rc:
            raise OracleError(rc, lib().tlo_last_message().decode())
        return list(steps), [(x.vol, x.mass, x.ie, x.temp) for x in sums[:ns.value]]

    def cg_alpha(self, n):
        return np.array([self.c.contents.cgalpha[k] for k in range(1, n + 1)])

    def cg_beta(self, n):
        return np.array([self.c.contents.cgbeta[k] for k in range(1, n + 1)])


def effective_bounds(s: Settings, k: int, mode: int):
    out = (C.c_double * 4)()
    lib().tlo_effective_bounds(C.byref(s), C.byref(s.states[k]), mode, out)
    return tuple(out)


def pairwise_sum(a: np.ndarray) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    return lib().tlo_pairwise_sum(a.ctypes.data_as(C.POINTER(C.c_double)), a.size)


def device_sum(v: np.ndarray, layout) -> float:
    """v indexed [i, j] over the interior (nx, ny)."""
    nx, ny = v.shape
    flat = np.ascontiguousarray(v.T, dtype=np.float64)   # i fastest
    o = make_opts(order=ORDER_DEVICE, layout=layout)
    return lib().tlo_device_sum(flat.ctypes.data_as(C.POINTER(C.c_double)), nx, ny, C.byref(o))
