"""Generates tests/golden/oracle_golden.json: per-step iteration counts and
errors, field summaries and a checksum of the final u field from the CPU
oracle (reference summation order) on the config-1 deck in both semantics and
with every solver, plus seeded random decks.

These fixtures pin the oracle against accidental change; they were not
produced by the reference itself (Julia is absent on every machine here, and
the reference ships no golden data).  Regenerate with
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1] / "oracle"))
sys.path.insert(0, str(HERE.parent))

import oracle as O  # noqa: E402
from parity_util import CONFIG1, deck_text, random_deck  # noqa: E402

SOLVERS = ["cg", "cheby", "ppcg", "jacobi"]


def run_case(deck: str, mode: int, solver: str) -> dict:
    s = O.parse_deck(deck)
    s.solver = O.SOLVERS[solver]
    ch = O.OracleChunk(s, O.make_opts(mode=mode))
    ch.initialise()
    try:
        steps, sums = ch.diffuse()
        status = 0
    except O.OracleError as e:
        return {"status": e.code, "steps": [], "summaries": [], "u_checksum": ""}
    u = ch.field("u").T.copy().tobytes()
    return {
        "status": status,
        "steps": [[r.iters, r.cg_iters, r.inner_iters, r.error.hex()] for r in steps],
        "summaries": [[v.hex() for v in sm] for sm in sums],
        "u_checksum": hashlib.sha256(u).hexdigest(),
    }


def cases():
    out = []
    for mode, mname in ((O.MODE_REFERENCE, "reference"), (O.MODE_TEALEAF, "tealeaf")):
        for solver in SOLVERS:
            out.append((f"config1-{mname}-{solver}", CONFIG1, mode, solver))
    for solver in SOLVERS:
        deck = random_deck(32, 101, steps=3, eps=1e-12, solver=solver, presteps=8)
        out.append((f"random32-tealeaf-{solver}", deck, O.MODE_TEALEAF, solver))
    out.append(("config1-tealeaf-cg-recip", deck_text(coefficient=2), O.MODE_TEALEAF, "cg"))
    return out


def main():
    res = []
    for name, deck, mode, solver in cases():
        r = run_case(deck, mode, solver)
        r.update({"name": name, "deck": deck, "mode": mode, "solver": solver})
        res.append(r)
        print(name, r["status"], [s[0] for s in r["steps"]][:5])
    (HERE / "oracle_golden.json").write_text(json.dumps({"generator": "tests/golden/make_golden.py", "cases": res},
                                                        indent=1))


if __name__ == "__main__":
    main()
