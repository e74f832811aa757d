"""ctypes binding of libtealeaf_gb300.so (include/tealeaf_gb300.h).

The library is the product: every solve runs in its sm_103a kernels.  There is
no CPU fallback; loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libtealeaf_gb300.so"

# status codes
OK, ERR_ARG, ERR_CUDA, ERR_COEF, ERR_EIGEN, ERR_REFERENCE_THROWS, ERR_NOMEM, ERR_STATE = range(8)
FIELDS = ["density0", "density", "energy0", "energy", "u", "u0", "p", "r", "mi", "w", "kx", "ky", "sd",
          "volume"]
EXCHANGE_FIELDS = ["density", "p", "energy0", "energy", "u", "sd"]   # src/chunk.jl:12
MODE_REFERENCE, MODE_TEALEAF = 0, 1
SOLVER_CG, SOLVER_CHEBY, SOLVER_PPCG, SOLVER_JACOBI = 0, 1, 2, 3
CRIT_REFERENCE, CRIT_RELATIVE = 0, 1
PREC_FP64, PREC_FP32_IR = 0, 1
GEOM_RECTANGULAR, GEOM_CIRCULAR, GEOM_POINT = 0, 1, 2
WARM_OFF, WARM_NETWORK, WARM_EXTRAPOLATE, WARM_HISTORY = 0, 1, 2, 3
WARM_HIST = 6          # TL_WARM_HIST: earlier right-hand sides of the warm-start projection


class Config(C.Structure):
    _fields_ = [("xcells", C.c_int), ("ycells", C.c_int), ("halodepth", C.c_int), ("maxiters", C.c_int),
                ("xmin", C.c_double), ("ymin", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("mode", C.c_int)]


class State(C.Structure):
    _fields_ = [("density", C.c_double), ("energy", C.c_double), ("xmin", C.c_double), ("ymin", C.c_double),
                ("xmax", C.c_double), ("ymax", C.c_double), ("radius", C.c_double), ("geometry", C.c_int)]


class Params(C.Structure):
    _fields_ = [("solver", C.c_int), ("coefficient", C.c_int), ("maxiters", C.c_int), ("presteps", C.c_int),
                ("ppcginnersteps", C.c_int), ("errorswitch", C.c_int), ("eps", C.c_double),
                ("epslim", C.c_double), ("criterion", C.c_int), ("precision", C.c_int), ("exact", C.c_int),
                ("warmstart", C.c_int)]


class Result(C.Structure):
    _fields_ = [("iters", C.c_int), ("cg_iters", C.c_int), ("inner_iters", C.c_int), ("est_iters", C.c_int),
                ("error", C.c_double), ("eigmin", C.c_double), ("eigmax", C.c_double), ("converged", C.c_int),
                ("refinements", C.c_int), ("rel_residual", C.c_double), ("launches", C.c_int), ("warm", C.c_int),
                ("r0_plain", C.c_double), ("r0_pred", C.c_double), ("warm_coef", C.c_double * (WARM_HIST + 2))]


class Deck(C.Structure):
    """tl_deck: the Settings fields the library's tea.in reader returns."""
    _fields_ = [("endstep", C.c_longlong)] + [(k, C.c_int) for k in (
        "presteps", "maxiters", "coefficient", "ppcginnersteps", "summaryfrequency", "halodepth", "xcells", "ycells",
        "errorswitch", "checkresult", "solver")] + [(k, C.c_double) for k in (
        "eps", "dtinit", "endtime", "epslim", "xmin", "ymin", "xmax", "ymax", "dx", "dy")] + [
        ("nstates", C.c_int), ("warnings", C.c_int)]


class WarmCrop(C.Structure):
    """tl_warm_crop: a crop of a deck's device fields for the network kernels."""
    _fields_ = [("u", C.c_void_p), ("uprev", C.c_void_p), ("rho", C.c_void_p), ("pitch", C.c_longlong),
                ("nx", C.c_int), ("ny", C.c_int), ("ox", C.c_int), ("oy", C.c_int), ("rx", C.c_double),
                ("ry", C.c_double), ("inv_su", C.c_double), ("inv_sd", C.c_double)]


# the warm-start network: (cin, cout) per layer; parameters W[cout][9][cin], b[cout]
WARM_LAYERS = [(16, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 16)]
WARM_NPARAMS = sum(co * 9 * ci + co for ci, co in WARM_LAYERS)


# every symbol the header declares, with its ctypes signature
_P = C.POINTER
_CTX = C.c_void_p
SIGNATURES = {
    "tl_create": ([_P(_CTX), _P(Config)], C.c_int),
    "tl_destroy": ([_CTX], C.c_int),
    "tl_last_error": ([_CTX], C.c_char_p),
    "tl_upload": ([_CTX, C.c_int, _P(C.c_double), C.c_int], C.c_int),
    "tl_download": ([_CTX, C.c_int, _P(C.c_double), C.c_int], C.c_int),
    "tl_set_states": ([_CTX, _P(State), C.c_int], C.c_int),
    "tl_initialise": ([_CTX, _P(State), C.c_int], C.c_int),
    "tl_halo_update": ([_CTX, C.c_int, _P(C.c_int), C.c_int, C.c_int], C.c_int),
    "tl_solve": ([_CTX, C.c_double, C.c_double, _P(Params), _P(Result)], C.c_int),
    "tl_solve_finished": ([_CTX, C.c_int], C.c_int),
    "tl_field_summary": ([_CTX, _P(C.c_double)], C.c_int),
    "tl_copy_u": ([_CTX], C.c_int),
    "tl_residual": ([_CTX], C.c_int),
    "tl_finalise": ([_CTX], C.c_int),
    "tl_get_cg_coefficients": ([_CTX, _P(C.c_double), _P(C.c_double), C.c_int], C.c_int),
    "tl_reduction_layout": ([_CTX, _P(C.c_int), _P(C.c_int), _P(C.c_int)], C.c_int),
    "tl_synchronize": ([_CTX], C.c_int),
    "tl_get_layout": ([_CTX, C.c_int, _P(C.c_int), _P(C.c_int), _P(C.c_int)], C.c_int),
    "tl_set_layout": ([_CTX, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
    "tl_last_solve_ms": ([_CTX, _P(C.c_double)], C.c_int),
    "tl_timer_start": ([_CTX], C.c_int),
    "tl_timer_stop": ([_CTX, _P(C.c_double)], C.c_int),
    "tl_bench_kernel": ([_CTX, C.c_int, C.c_int, _P(C.c_double)], C.c_int),
    "tl_diffuse": ([_CTX, _P(Params), C.c_double, C.c_int, C.c_int, C.c_int, _P(Result), _P(C.c_double), C.c_int,
                    _P(C.c_int)], C.c_int),
    "tl_batch_create": ([_P(C.c_void_p), _P(C.c_void_p), C.c_int], C.c_int),
    "tl_batch_destroy": ([C.c_void_p], C.c_int),
    "tl_batch_last_error": ([C.c_void_p], C.c_char_p),
    "tl_batch_solve": ([C.c_void_p, _P(C.c_double), _P(C.c_double), _P(Params), _P(Result)], C.c_int),
    "tl_batch_last_ms": ([C.c_void_p, _P(C.c_double)], C.c_int),
    "tl_field_summary_noalloc": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                  C.c_longlong, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int], C.c_int),
    "tl_parse_deck": ([C.c_char_p, C.c_int, _P(Deck), _P(State), C.c_int, C.c_char_p, C.c_int], C.c_int),
    "tl_warm_load": ([_CTX, _P(C.c_float), C.c_int], C.c_int),
    "tl_warm_reset": ([_CTX], C.c_int),
    "tl_conv3x3_forward": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p], C.c_int),
    "tl_conv3x3_weight_grad": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                C.c_int, C.c_int, C.c_void_p], C.c_int),
    "tl_conv3x3_flip": ([C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p], C.c_int),
    "tl_conv_status": ([C.POINTER(C.c_int)], C.c_int),
    "tl_adam_step": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float,
                      C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "tl_warm_features": ([C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "tl_warm_loss": ([C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                      C.c_int, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
}

_lib = None


class TeaLeafError(RuntimeError):
    """A non-zero status from the library (the reference's `throw`s map here)."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def load(path: Path | None = None):
    """Load the CUDA library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with tealeaf.jl_gb300/build.py (the solve path has no "
                           "CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def check(lib, ctx, rc: int):
    if rc:
        msg = lib.tl_last_error(ctx)
        raise TeaLeafError(rc, msg.decode() if msg else f"status {rc}")
