"""GPU edge cases of the solve path against the CPU oracle: one-cell and
one-cell-wide decks, halo depths other than 2, iteration caps that end the
loop, and a tolerance met at once.  Bit-identical to the oracle in the device
order where the kernels take the reference operation order (`exact`).

A one-cell deck is exact at the start: r = 0 and CG's alpha is 0/0, so the
reference's loop (and both semantics with its own test) runs to max_iters
on NaN; that is compared as it is.  The relative test stops before the first
iteration instead (see test_fp32_refined_tiny_decks)."""
import numpy as np
import pytest

import oracle as O
from parity_util import FIELDS, gpu_run, oracle_run, random_deck

pytestmark = pytest.mark.gpu
REF, TEA = O.MODE_REFERENCE, O.MODE_TEALEAF


def _deck(nx, ny, seed=9, **kv):
    return random_deck(nx, seed, ny=ny, nrect=3, steps=2, eps=1e-12, **kv)


def _eq(a, b):
    """Equal, with NaN equal to NaN."""
    return np.array_equal(np.asarray(a, dtype=float), np.asarray(b, dtype=float), equal_nan=True)


def _same(tl, text, mode):
    chunk, res, sums, per = gpu_run(tl, text, mode, exact=True, steps_fields=True)
    _, ores, osums, oper = oracle_run(text, mode, O.ORDER_DEVICE, chunk.reduction_layout(), steps_fields=True)
    assert [r.iters for r in res] == [r.iters for r in ores]
    assert _eq([r.error for r in res], [r.error for r in ores])
    for f in FIELDS:
        np.testing.assert_array_equal(per[-1][f], oper[-1][f], err_msg=f)
    for g, o in zip(sums, osums):
        assert _eq(g, o)
    return res


@pytest.mark.parametrize("nx,ny", [(1, 1), (1, 7), (7, 1), (2, 2), (3, 130)])
def test_tiny_and_thin_decks(tl, built_lib, nx, ny):
    _same(tl, _deck(nx, ny), TEA)
    if nx == ny:
        _same(tl, _deck(nx, ny), REF)


@pytest.mark.parametrize("hd", [1, 3, 4])
def test_halo_depths_tealeaf(tl, built_lib, hd):
    """Tealeaf mode computes w over the whole array, so halo depth 1 keeps
    Kx, Ky at the domain edge finite (the reference's 2:X-1 range does not)."""
    res = _same(tl, _deck(24, 20, halo_depth=hd), TEA)
    assert all(r.converged and np.isfinite(r.error) for r in res)


def test_halo_depth_1_reference_raises(tl, built_lib):
    """halodepth 1 in the reference's updateface! indexes column 0: BoundsError (src/kernels.jl:196)."""
    s = tl.Settings.from_text(_deck(12, 12, halo_depth=1), mode=REF)
    with pytest.raises(tl.TeaLeafError) as e:
        chunk = tl.initialiseapp(s)
        tl.haloupdate(chunk, s, 1, ["energy", "density"])
    assert e.value.code == tl._abi.ERR_REFERENCE_THROWS


@pytest.mark.parametrize("mode", [REF, TEA])
@pytest.mark.parametrize("maxiters", [1, 2, 5])
def test_iteration_cap(tl, built_lib, mode, maxiters):
    """A tolerance out of reach: the loop ends on max_iters, like CG.jl's for loop."""
    res = _same(tl, _deck(16, 16, seed=3).replace("eps=1e-12", "eps=1e-300").replace("max_iters=5000",
                                                                                       f"max_iters={maxiters}"), mode)
    assert all(r.iters == maxiters and not r.converged for r in res)


@pytest.mark.parametrize("mode", [REF, TEA])
def test_tolerance_met_at_once(tl, built_lib, mode):
    res = _same(tl, _deck(16, 16, seed=4).replace("eps=1e-12", "eps=1e300"), mode)
    assert all(r.converged for r in res)


@pytest.mark.parametrize("nx,ny", [(1, 1), (5, 1), (1, 9), (33, 3)])
def test_fp32_refined_tiny_decks(tl, built_lib, nx, ny):
    """FP32 refinement on decks narrower than one lane's four cells: the
    1e-10 relative true residual is met and u matches FP64 CG."""
    text = random_deck(nx, 12, ny=ny, nrect=2, steps=2, eps=1e-10)
    _, r32, _, p32 = gpu_run(tl, text, TEA, steps_fields=True, criterion=1, precision=1)
    _, r64, _, p64 = gpu_run(tl, text, TEA, steps_fields=True, criterion=1, precision=0)
    assert all(r.converged and r.rel_residual < 1e-10 for r in r32)
    u32, u64 = p32[-1]["u"], p64[-1]["u"]
    assert np.max(np.abs(u32 - u64)) <= 1e-8 * max(np.max(np.abs(u64)), 1e-300)


@pytest.mark.parametrize("solver", ["cg", "cheby", "ppcg"])
@pytest.mark.parametrize("nx,ny,hd", [(2, 40, 2), (3, 33, 1), (6, 17, 3), (7, 129, 1), (131, 9, 4)])
def test_fp32_sweeps_ragged_widths_and_halo_depths(tl, built_lib, solver, nx, ny, hd):
    """Every FP32 sweep kernel on widths that leave a lane with 2, 3 or 1
    cells (and a ragged last warp strip at 131), with halo depths 1, 3 and 4:
    the 1e-10 relative true residual is met and u matches FP64 on the
    interior.  Cheby and PPCG switch after 5 CG presteps, so the Chebyshev
    and PPCG sweeps run."""
    text = random_deck(nx, 21, ny=ny, nrect=3, steps=2, eps=1e-10, solver=solver, halo_depth=hd, presteps=5,
                       ppcg_inner_steps=4)
    _, r32, _, p32 = gpu_run(tl, text, TEA, steps_fields=True, criterion=1, precision=1)
    _, r64, _, p64 = gpu_run(tl, text, TEA, steps_fields=True, criterion=1, precision=0)
    assert all(r.converged and 0 <= r.rel_residual < 1e-10 for r in r32), r32
    assert all(r.converged for r in r64)
    u32, u64 = p32[-1]["u"][hd:-hd, hd:-hd], p64[-1]["u"][hd:-hd, hd:-hd]
    assert np.max(np.abs(u32 - u64)) <= 1e-8 * np.max(np.abs(u64))
