"""GPU: CG with FP32 inner sweeps inside FP64 refinement.

The refined solve must reach the same 1e-10 relative true residual as the
FP64 solve, and its final field must agree with the oracle's FP64 solution to
the tolerance stated in each test (a relative residual of 1e-10 bounds the
solution error by the condition number times 1e-10).
"""
import numpy as np
import pytest

import oracle as O
from parity_util import gpu_run, oracle_run, random_deck, rel

pytestmark = pytest.mark.gpu
TEA = O.MODE_TEALEAF


@pytest.mark.parametrize("nx,ny,seed", [(64, 64, 31), (256, 256, 32), (130, 70, 33), (33, 257, 34)])
def test_ir_converges_and_matches_fp64(tl, built_lib, nx, ny, seed):
    text = random_deck(nx, seed, ny=ny, steps=2, eps=1e-10)
    _, res, sums, per = gpu_run(tl, text, TEA, steps_fields=True, criterion=1, precision=1)
    _, res64, sums64, per64 = gpu_run(tl, text, TEA, steps_fields=True, criterion=1, precision=0)
    for r, r64 in zip(res, res64):
        assert r.converged and r.rel_residual < 1e-10
        assert r.refinements >= 1
        # refinement restarts cost some iterations; bound the overhead
        assert r.iters <= 1.5 * r64.iters + 20
    # the oracle's FP64 CG run to a tighter absolute tolerance is the reference solution
    tight = random_deck(nx, seed, ny=ny, steps=2, eps=1e-14)
    _, ores, osums, oper = oracle_run(tight, TEA, O.ORDER_REFERENCE, steps_fields=True)
    u, ou = per[-1]["u"], oper[-1]["u"]
    err = np.max(np.abs(u - ou)) / np.max(np.abs(ou))
    assert err <= 1e-8, err
    for a, b in zip(sums[-1], osums[-1]):
        assert rel(a, b) <= 1e-9


def test_ir_reference_mode_rejected(tl, built_lib):
    text = random_deck(32, 1, steps=1)
    s = tl.Settings.from_text(text, mode=O.MODE_REFERENCE, precision=1)
    chunk = tl.initialiseapp(s)
    with pytest.raises(tl.TeaLeafError):
        tl.CG.solve(chunk, s, 0.004, 0.004)
