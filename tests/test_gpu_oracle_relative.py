"""GPU against the CPU oracle under the relative criterion ||u0 - A u|| / ||u0||
< eps, the test of the mixed-precision and batched measurements.

The oracle's CG carries the same criterion (its tlo_opts.criterion 1): the
loop tests the recursive residual, then the true residual, restarting from
it while it is above eps.  With it:

* exact FP64 CG is bit-identical to the oracle in the device order, the
  true-residual checks and restarts included;
* the fused FP64 kernels agree in iteration count to within one;
* FP32 inner sweeps inside FP64 refinement (CG, Chebyshev, PPCG) and the
  batched decks (FP64 and FP32-refined) are compared with the oracle's FP64
  solution of the same timesteps, not with the GPU's own FP64 runs.

Solutions that each meet the 1e-10 relative residual differ by the
conditioning of the system times that residual; the tolerance written in
each test (1e-9 or 1e-8 of max |u|) covers it.
"""
import os

import numpy as np
import pytest

import oracle as O
from parity_util import FIELDS, gpu_run, oracle_run, random_deck, rel

pytestmark = pytest.mark.gpu

TEA = O.MODE_TEALEAF
SUMMARY_RTOL = 1e-12
FP64_U_RTOL = 1e-9
FP32_U_RTOL = 1e-8
THREADS = os.cpu_count() or 1


def _oracle_fp64(text, steps_fields=True):
    """The oracle's FP64 CG, relative criterion, on the deck (solver forced to CG)."""
    return oracle_run(text, TEA, O.ORDER_REFERENCE, steps_fields=steps_fields, solver="cg", criterion=1,
                      nthreads=THREADS)


def _u_close(u, ou, rtol, what):
    hd = 2
    d = np.max(np.abs(u[hd:-hd, hd:-hd] - ou[hd:-hd, hd:-hd]))
    assert d <= rtol * np.max(np.abs(ou)), (what, d, np.max(np.abs(ou)))


@pytest.mark.parametrize("nx,ny,seed", [(64, 64, 71), (130, 70, 72), (257, 191, 73)])
def test_relative_cg_exact_bit_exact(tl, built_lib, nx, ny, seed):
    """Exact FP64 CG under the relative criterion: every field after every
    step, the iteration counts and the final relative residuals identical to
    the oracle summing in the device order."""
    text = random_deck(nx, seed, ny=ny, steps=3, eps=1e-10)
    chunk, res, sums, per = gpu_run(tl, text, TEA, exact=True, steps_fields=True, criterion=1)
    _, ores, osums, oper = oracle_run(text, TEA, O.ORDER_DEVICE, chunk.reduction_layout(), steps_fields=True,
                                      criterion=1, nthreads=THREADS)
    for tt, (g, o) in enumerate(zip(res, ores)):
        assert g.converged and o.converged, tt
        assert g.iters == o.iters, (tt, g.iters, o.iters)
        assert g.rel_residual == o.rel_residual, (tt, g.rel_residual, o.rel_residual)
        for f in FIELDS:
            np.testing.assert_array_equal(per[tt][f], oper[tt][f], err_msg=f"step {tt + 1} field {f}")
    for g, o in zip(sums, osums):
        assert tuple(g) == tuple(o)


@pytest.mark.parametrize("nx,ny,seed", [(64, 64, 71), (130, 70, 72), (257, 191, 73)])
def test_relative_cg_fused(tl, built_lib, nx, ny, seed):
    """The fused FP64 kernels under the relative criterion: iteration counts
    within one of the oracle's, both below 1e-10, summary within 1e-12, u
    within 1e-9 of its maximum."""
    text = random_deck(nx, seed, ny=ny, steps=3, eps=1e-10)
    _, res, sums, per = gpu_run(tl, text, TEA, exact=False, steps_fields=True, criterion=1)
    _, ores, osums, oper = _oracle_fp64(text)
    for tt, (g, o) in enumerate(zip(res, ores)):
        assert g.converged and 0 <= g.rel_residual < 1e-10 and o.rel_residual < 1e-10, tt
        assert abs(g.iters - o.iters) <= 1, (tt, g.iters, o.iters)
    for g, o in zip(sums, osums):
        for a, b in zip(g, o):
            assert rel(a, b) <= SUMMARY_RTOL
    _u_close(per[-1]["u"], oper[-1]["u"], FP64_U_RTOL, "fused FP64")


@pytest.mark.parametrize("solver,nx,ny,seed,kv", [
    ("cg", 200, 200, 74, {}),
    ("cg", 243, 150, 75, {}),
    ("cheby", 128, 128, 50, dict(presteps=20)),
    ("cheby", 200, 200, 51, dict(presteps=30)),
    ("ppcg", 200, 200, 53, dict(presteps=30, ppcg_inner_steps=5)),
    ("ppcg", 243, 150, 56, dict(presteps=15, ppcg_inner_steps=10)),
])
def test_fp32_refined_vs_oracle(tl, built_lib, solver, nx, ny, seed, kv):
    """FP32 inner sweeps inside FP64 refinement (CG, Chebyshev, PPCG, their
    presteps included): every step meets 1e-10 on the true residual, and u
    after each step is within 1e-8 of its maximum of the oracle's FP64
    solution of the same timesteps."""
    text = random_deck(nx, seed, ny=ny, steps=3, eps=1e-10, solver=solver, **kv)
    _, res, _, per = gpu_run(tl, text, TEA, exact=False, steps_fields=True, criterion=1, precision=1)
    _, ores, _, oper = _oracle_fp64(text)
    for tt, (g, o) in enumerate(zip(res, ores)):
        assert g.converged and 0 <= g.rel_residual < 1e-10 and g.refinements >= 1, (tt, g)
        assert o.converged, tt
        _u_close(per[tt]["u"], oper[tt]["u"], FP32_U_RTOL, f"{solver} step {tt + 1}")


SIZES = [(64, 64), (130, 70), (33, 257), (256, 256), (100, 100), (17, 19)]


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_vs_oracle(tl, built_lib, precision):
    """Decks of uneven sizes solved together (one graph launch, per-deck
    convergence masks), FP64 and FP32-refined, against the oracle's FP64 CG
    of each deck: every deck converged to 1e-10 at every step; FP64:
    iteration counts within one of the oracle's, u within 1e-9; FP32-refined:
    u within 1e-8."""
    texts = [random_deck(nx, 400 + k, ny=ny, steps=3, eps=1e-10) for k, (nx, ny) in enumerate(SIZES)]
    sets = [tl.Settings.from_text(t, mode=1, criterion=1, precision=precision) for t in texts]
    chunks = [tl.initialiseapp(s) for s in sets]
    hist = tl.diffuse_batch(chunks, sets, steps=3)
    for k, t in enumerate(texts):
        _, ores, _, oper = _oracle_fp64(t)
        for step in range(3):
            b, o = hist[step][k], ores[step]
            assert b.converged and 0 <= b.rel_residual < 1e-10, (k, step, b)
            if precision == 0:
                assert abs(b.iters - o.iters) <= 1, (k, step, b.iters, o.iters)
        _u_close(chunks[k].field("u"), oper[-1]["u"], FP64_U_RTOL if precision == 0 else FP32_U_RTOL, f"deck {k}")
