"""GPU parity of the Chebyshev, PPCG and Jacobi solver plugins, through the C
ABI, against the CPU oracle.

`exact` tealeaf mode and reference mode are bit-identical to the oracle
summing in the device order (same reduction tree): every field after every
step, iteration counts, errors and eigenvalue estimates.  The fused FMA
kernels agree to the tolerances written in each test.  Where the reference
raises (Cheby's minmax, PPCG's `++`, Jacobi's missing solve!), both raise.
"""
import numpy as np
import pytest

import oracle as O
from parity_util import CONFIG1, FIELDS, deck_text, gpu_run, oracle_run, random_deck, rel

pytestmark = pytest.mark.gpu
REF, TEA = O.MODE_REFERENCE, O.MODE_TEALEAF
SUMMARY_RTOL = 1e-12


def _cases():
    return [("cheby", 128, 40, dict(presteps=20)), ("cheby", 96, 41, dict(presteps=30)),
            ("ppcg", 128, 42, dict(presteps=20)), ("ppcg", 96, 43, dict(presteps=30, ppcg_inner_steps=5)),
            ("jacobi", 64, 44, {}), ("jacobi", 48, 45, {})]


@pytest.mark.parametrize("solver,n,seed,kv", _cases())
def test_exact_device_order(tl, built_lib, solver, n, seed, kv):
    text = random_deck(n, seed, steps=2, eps=1e-12, solver=solver, **kv)
    chunk, res, sums, per = gpu_run(tl, text, TEA, exact=True, steps_fields=True)
    _, ores, osums, oper = oracle_run(text, TEA, O.ORDER_DEVICE, chunk.reduction_layout(), steps_fields=True)
    for tt, (g, o) in enumerate(zip(res, ores)):
        assert (g.iters, g.cg_iters, g.inner_iters) == (o.iters, o.cg_iters, o.inner_iters), f"step {tt + 1}"
        assert g.error == o.error, f"step {tt + 1}"
        if solver != "jacobi":
            assert g.eigmin == o.eigmin and g.eigmax == o.eigmax
        for f in FIELDS:
            np.testing.assert_array_equal(per[tt][f], oper[tt][f], err_msg=f"step {tt + 1} field {f}")
    for g, o in zip(sums, osums):
        assert tuple(g) == tuple(o)
    if solver != "jacobi":
        assert res[0].inner_iters > 0, "the deck must reach the switch"


@pytest.mark.parametrize("solver,n,seed,kv", _cases())
def test_reference_order(tl, built_lib, solver, n, seed, kv):
    """Against the reference's own summation order: equal iteration counts,
    field summary within 1e-12 relative."""
    text = random_deck(n, seed, steps=2, eps=1e-12, solver=solver, **kv)
    _, res, sums, _ = gpu_run(tl, text, TEA, exact=True)
    _, ores, osums, _ = oracle_run(text, TEA, O.ORDER_REFERENCE)
    assert [(r.iters, r.inner_iters) for r in res] == [(r.iters, r.inner_iters) for r in ores]
    for g, o in zip(sums, osums):
        for a, b in zip(g, o):
            assert rel(a, b) <= SUMMARY_RTOL


@pytest.mark.parametrize("solver,n,seed,kv", _cases())
def test_fused_kernels(tl, built_lib, solver, n, seed, kv):
    """Fused FMA Chebyshev/PPCG/Jacobi kernels: iteration counts within 2,
    summary within 1e-12 relative, u within 1e-9 relative of its maximum."""
    text = random_deck(n, seed, steps=2, eps=1e-12, solver=solver, **kv)
    _, res, sums, per = gpu_run(tl, text, TEA, exact=False, steps_fields=True)
    _, ores, osums, oper = oracle_run(text, TEA, O.ORDER_REFERENCE, steps_fields=True)
    for g, o in zip(res, ores):
        assert abs(g.iters - o.iters) <= 2, (g.iters, o.iters)
    for g, o in zip(sums, osums):
        for a, b in zip(g, o):
            assert rel(a, b) <= SUMMARY_RTOL
    u, ou = per[-1]["u"], oper[-1]["u"]
    assert np.max(np.abs(u - ou)) <= 1e-9 * np.max(np.abs(ou))


@pytest.mark.parametrize("solver", ["cheby", "ppcg"])
def test_reference_mode_config1(tl, built_lib, solver):
    """Reference mode on config 1: Cheby's stale rro turns the fields to NaN and
    runs to max_iters; PPCG converges in its CG presteps.  Bit-identical to the
    oracle in device order (NaN compares equal to NaN here)."""
    text = deck_text(solver=solver)
    chunk, res, sums, per = gpu_run(tl, text, REF, exact=True, steps_fields=True)
    _, ores, osums, oper = oracle_run(text, REF, O.ORDER_DEVICE, chunk.reduction_layout(), steps_fields=True)
    assert [r.iters for r in res] == [r.iters for r in ores]
    for tt in range(len(res)):
        for f in FIELDS:
            np.testing.assert_array_equal(per[tt][f], oper[tt][f], err_msg=f"step {tt + 1} field {f}")


@pytest.mark.parametrize("solver,msg,n,seed,pre", [("cheby", "minmax", 24, 0, 1), ("ppcg", "++", 64, 7, 5),
                                                   ("jacobi", "solve!", 64, 7, 5)])
def test_reference_mode_raises(tl, built_lib, solver, msg, n, seed, pre):
    """Where the reference raises, reference mode raises at the same point
    (decks chosen so that the presteps reach the switch)."""
    text = random_deck(n, seed, steps=1, eps=1e-30, solver=solver, presteps=pre)
    s = tl.Settings.from_text(text, mode=REF, exact=True)
    chunk = tl.initialiseapp(s)
    tl.haloupdate(chunk, s, 1, ["energy", "density"])
    with pytest.raises(tl.TeaLeafError) as e:
        tl.SOLVERS[s.solver].solve(chunk, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    assert e.value.code == 5 and msg in str(e.value)
    och = O.OracleChunk(O.parse_deck(text), O.make_opts(mode=REF))
    och.initialise()
    och.halo(1, ["energy", "density"])
    with pytest.raises(O.OracleError) as oe:
        och.solve(s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    assert oe.value.code == O.ERR_REFERENCE_THROWS


@pytest.mark.parametrize("n,seed,pre", [(128, 50, 20), (200, 51, 30)])
def test_cheby_fp32_refined(tl, built_lib, n, seed, pre):
    """Chebyshev in FP32 inside FP64 refinement, the CG presteps included:
    every step meets the 1e-10 relative true residual, with at least one
    refinement, and the final u matches FP64 Chebyshev to 1e-8 of its
    maximum.  The FP32 presteps record the CG coefficients for the
    eigenvalue estimate and switch within a few iterations of FP64's (the
    switch test reads the FP32 recurrence r.r); at the same switch the
    estimates agree to 1e-4 relative, and the Chebyshev iteration counts to
    25 % (FP64 tests the norm every 10th step past its estimate, FP32 every
    step)."""
    text = random_deck(n, seed, steps=3, eps=1e-10, solver="cheby", presteps=pre)
    _, r64, _, per64 = gpu_run(tl, text, TEA, exact=False, steps_fields=True, criterion=1, precision=0)
    _, r32, _, per32 = gpu_run(tl, text, TEA, exact=False, steps_fields=True, criterion=1, precision=1)
    for tt, (a, b) in enumerate(zip(r32, r64)):
        assert a.converged and 0 <= a.rel_residual < 1e-10, (tt, a)
        assert b.converged
        assert a.refinements >= 1
        assert abs(a.cg_iters - b.cg_iters) <= 0.05 * b.cg_iters + 2, (tt, a.cg_iters, b.cg_iters)
        if a.inner_iters:
            assert a.cg_iters >= pre
            if a.cg_iters == b.cg_iters:
                for x, y in ((a.eigmin, b.eigmin), (a.eigmax, b.eigmax)):
                    assert abs(x - y) <= 1e-4 * abs(y), (tt, a.eigmin, a.eigmax, b.eigmin, b.eigmax)
            assert abs(a.inner_iters - b.inner_iters) <= 0.25 * b.inner_iters + 10, (tt, a.inner_iters, b.inner_iters)
    u32, u64 = per32[-1]["u"], per64[-1]["u"]
    assert np.max(np.abs(u32 - u64)) <= 1e-8 * np.max(np.abs(u64))


@pytest.mark.parametrize("n,ny,seed,pre,inner", [(200, 200, 53, 30, 5), (243, 150, 56, 15, 10), (77, 131, 54, 20, 3)])
def test_ppcg_fp32_refined(tl, built_lib, n, ny, seed, pre, inner):
    """PPCG in FP32 inside FP64 refinement, the CG presteps included: every
    step meets the 1e-10 relative true residual, with at least one
    refinement, and the final u matches FP64 PPCG to 1e-8 of its maximum.
    The switch falls within a few iterations of FP64's; the outer PPCG step
    counts agree to 25 % (FP64 tests |r.r| < eps, FP32 the relative true
    residual after each refinement)."""
    text = random_deck(n, seed, steps=3, eps=1e-10, ny=ny, solver="ppcg", presteps=pre, ppcg_inner_steps=inner)
    _, r64, _, per64 = gpu_run(tl, text, TEA, exact=False, steps_fields=True, criterion=1, precision=0)
    _, r32, _, per32 = gpu_run(tl, text, TEA, exact=False, steps_fields=True, criterion=1, precision=1)
    for tt, (a, b) in enumerate(zip(r32, r64)):
        assert a.converged and 0 <= a.rel_residual < 1e-10, (tt, a)
        assert b.converged
        assert a.refinements >= 1
        assert abs(a.cg_iters - b.cg_iters) <= 0.05 * b.cg_iters + 2, (tt, a.cg_iters, b.cg_iters)
        if a.inner_iters:
            assert a.cg_iters >= pre
            assert abs(a.inner_iters - b.inner_iters) <= 0.25 * b.inner_iters + 3, (tt, a.inner_iters, b.inner_iters)
    assert any(a.inner_iters for a in r32), "the deck must reach the switch"
    # interior only: FP64 PPCG leaves u's halo from the last CG prestep (its
    # steps exchange p alone, PPCG.jl:31), the FP32 refinements refresh it
    u32, u64 = per32[-1]["u"][2:-2, 2:-2], per64[-1]["u"][2:-2, 2:-2]
    assert np.max(np.abs(u32 - u64)) <= 1e-8 * np.max(np.abs(u64))
