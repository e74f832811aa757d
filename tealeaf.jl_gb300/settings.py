"""Settings and the tea.in deck reader (src/settings.jl), kept on the host.

The reader follows Settings(infile) (settings.jl:90-135) and readstate
(settings.jl:142-173): keys lose their underscores, `initial_timestep` is an
alias of `dtinit`, `use_*` lines pick the solver, unknown keys and values
that do not parse are skipped with a warning, and each state's bounds are
inset by dx/100 (dy/100) with dx, dy as they stand when the state line is
read (the default 10 unless the deck sets dx itself).  dx and dy are computed
from the domain once the whole file is read (settings.jl:132-133).
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass, field
from typing import Dict, List

from . import _abi

CONDUCTIVITY = 1          # settings.jl:13
RECIP_CONDUCTIVITY = 2    # settings.jl:14
RECTANGULAR, CIRCULAR, POINT = _abi.GEOM_RECTANGULAR, _abi.GEOM_CIRCULAR, _abi.GEOM_POINT


@dataclass
class State:
    """A `state` line (settings.jl:20-29).  Bounds are kept as written; `given`
    marks which were present and pdx/pdy record dx/dy at parse time."""
    density: float = 0.0
    energy: float = 0.0
    xmin: float = 0.0
    ymin: float = 0.0
    xmax: float = 0.0
    ymax: float = 0.0
    radius: float = 0.0
    geometry: int = RECTANGULAR
    given: int = 0
    pdx: float = 10.0
    pdy: float = 10.0

    def bounds(self, settings: "Settings", mode: int):
        """Bounds setchunkstate! tests.  Reference mode: the parse-time inset
        (settings.jl:159-162).  Tealeaf mode: inset by the deck's final dx/100."""
        ix = self.pdx if mode == _abi.MODE_REFERENCE else settings.dx
        iy = self.pdy if mode == _abi.MODE_REFERENCE else settings.dy
        return (self.xmin + ix / 100 if self.given & 1 else self.xmin,
                self.ymin + iy / 100 if self.given & 2 else self.ymin,
                self.xmax - ix / 100 if self.given & 4 else self.xmax,
                self.ymax - iy / 100 if self.given & 8 else self.ymax)


SOLVER_NAMES = {"cg": _abi.SOLVER_CG, "ppcg": _abi.SOLVER_PPCG, "cheby": _abi.SOLVER_CHEBY,
                "jacobi": _abi.SOLVER_JACOBI}

_INT_KEYS = {"endstep", "presteps", "maxiters", "coefficient", "ppcginnersteps", "summaryfrequency", "halodepth",
             "xcells", "ycells"}
_BOOL_KEYS = {"errorswitch", "checkresult"}
_F64_KEYS = {"eps", "dtinit", "endtime", "epslim", "xmin", "ymin", "xmax", "ymax", "dx", "dy"}


@dataclass
class Settings:
    """The reference's Settings struct (settings.jl:39-78)."""
    endstep: int = 2 ** 63 - 1
    presteps: int = 30
    maxiters: int = 10_000
    coefficient: int = CONDUCTIVITY
    ppcginnersteps: int = 10
    summaryfrequency: int = 10
    halodepth: int = 2
    toexchange: Dict[str, bool] = field(default_factory=lambda: {f: False for f in _abi.EXCHANGE_FIELDS})
    errorswitch: bool = False
    checkresult: bool = True
    eps: float = 1e-15
    dtinit: float = 0.1
    endtime: float = 10.0
    epslim: float = 1e-5
    solver: int = _abi.SOLVER_CG
    xcells: int = 10
    ycells: int = 10
    xmin: float = 0.0
    ymin: float = 0.0
    xmax: float = 100.0
    ymax: float = 100.0
    dx: float = 10.0
    dy: float = 10.0
    states: List[State] = field(default_factory=list)
    debugfile: str = ""
    # build-side choices (not in the reference): semantics, precision, criterion
    mode: int = _abi.MODE_TEALEAF
    precision: int = _abi.PREC_FP64
    criterion: int = _abi.CRIT_REFERENCE
    exact: bool = False
    warmstart: bool = False    # CG from the learned prediction when it beats the plain start

    def resettoexchange(self):        # settings.jl:80
        for k in self.toexchange:
            self.toexchange[k] = False

    @classmethod
    def from_file(cls, path, **overrides) -> "Settings":
        with open(path) as fh:
            return cls.from_text(fh.read(), **overrides)

    @classmethod
    def from_text(cls, text: str, **overrides) -> "Settings":
        s = cls()
        for raw in text.split("\n"):
            line = raw.strip()
            if line.startswith("state"):
                s.states.append(_read_state(line, s))
                continue
            if line.startswith("use_"):
                name = line[4:]
                if name in SOLVER_NAMES:
                    s.solver = SOLVER_NAMES[name]
                else:
                    warnings.warn(f"Unknown setting {line!r}")
                continue
            if line.startswith("*") or "=" not in line:
                continue
            parts = line.split("=")
            key = parts[0].replace("_", "").strip()
            val = parts[1]
            if key == "initialtimestep":
                key = "dtinit"
            try:
                if key in _INT_KEYS:
                    setattr(s, key, _parse_int(val))
                elif key in _BOOL_KEYS:
                    setattr(s, key, _parse_bool(val))
                elif key in _F64_KEYS:
                    setattr(s, key, _parse_f64(val))
                else:
                    raise ValueError(key)
            except ValueError:
                warnings.warn(f"Unknown setting {line!r} (key {key!r})")
        s.dx = (s.xmax - s.xmin) / s.xcells      # settings.jl:132-133
        s.dy = (s.ymax - s.ymin) / s.ycells
        for k, v in overrides.items():
            setattr(s, k, v)
        return s


def _parse_int(v: str) -> int:
    t = v.strip()
    body = t[1:] if t[:1] in "+-" else t
    if not body.isdigit():
        raise ValueError(v)
    return int(t)


def _parse_bool(v: str) -> bool:
    t = v.strip()
    if t in ("true", "1"):
        return True
    if t in ("false", "0"):
        return False
    raise ValueError(v)


def _parse_f64(v: str) -> float:
    t = v.strip()
    if not t:
        raise ValueError(v)
    x = float(t)
    return x


def _read_state(line: str, s: Settings) -> State:
    """readstate (settings.jl:142-173)."""
    pieces = line.split(" ")
    num = _parse_int(pieces[1])
    st = State(pdx=s.dx, pdy=s.dy)
    for pair in pieces[2:]:
        kv = pair.split("=")
        if len(kv) < 2:
            raise ValueError(f"state item {pair!r} has no '=' (src/settings.jl:148)")
        key, val = kv[0], kv[1]
        if key == "density":
            st.density = _parse_f64(val)
        elif key == "energy":
            st.energy = _parse_f64(val)
        if num == 1:
            continue
        if key in ("xmin", "ymin", "xmax", "ymax"):
            setattr(st, key, _parse_f64(val))
            st.given |= {"xmin": 1, "ymin": 2, "xmax": 4, "ymax": 8}[key]
        elif key == "radius":
            st.radius = _parse_f64(val)
        elif key == "geometry":
            geo = {"rectangle": RECTANGULAR, "circular": CIRCULAR, "point": POINT}
            if val not in geo:
                raise ValueError(f"unknown geometry {val!r}")
            st.geometry = geo[val]
    return st


def checkingvalue(settings: Settings, problemfile="tea.problems") -> float:
    """checkingvalue (settings.jl:180-196): the QA value for (xcells, ycells,
    endstep), 1.0 with a warning when the file has no such line."""
    with open(problemfile) as fh:
        for ln in fh:
            parts = ln.split(" ")
            if len(parts) < 4:
                continue
            params = [int(x) for x in parts[:3]]
            value = float(parts[3])
            if params == [settings.xcells, settings.ycells, settings.endstep]:
                return value
    warnings.warn("Problem was not found in the test problems file.")
    return 1.0


def qa_passes(actual: float, checking: float) -> bool:
    """The PASS rule of fieldsummary (kernels.jl:127-128)."""
    return abs(100 * actual / checking - 100.0) < 0.001 if checking != 0 and math.isfinite(actual) else False
