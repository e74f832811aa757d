"""GPU: many decks of uneven sizes solved by the batched CG (one graph launch
with per-deck convergence masks), against the same decks solved one at a
time by the fused CG.  The batched reduction splits each deck over a
different number of blocks, so sums agree to rounding: iteration counts
within one, field summaries within 1e-12 relative, u within 1e-9 of its
maximum."""
import numpy as np
import pytest

from parity_util import random_deck, rel

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (130, 70), (33, 257), (256, 256), (100, 100), (17, 19)]


def _decks():
    return [random_deck(nx, 300 + k, ny=ny, steps=3, eps=1e-10) for k, (nx, ny) in enumerate(SIZES)]


def test_batch_matches_single_solves(tl, built_lib):
    texts = _decks()
    sets = [tl.Settings.from_text(t, mode=1) for t in texts]
    chunks = [tl.initialiseapp(s) for s in sets]
    hist = tl.diffuse_batch(chunks, sets, steps=3)
    for k, t in enumerate(texts):
        s1 = tl.Settings.from_text(t, mode=1)
        c1 = tl.initialiseapp(s1)
        single = []
        for _ in range(3):
            tl.haloupdate(c1, s1, 1, ["energy", "density"])
            single.append(tl.CG.solve(c1, s1, s1.dtinit / s1.dx ** 2, s1.dtinit / s1.dy ** 2))
            tl.solvefinished(c1, s1)
        for step in range(3):
            b, o = hist[step][k], single[step]
            assert b.converged
            assert abs(b.iters - o.iters) <= 1, (k, step, b.iters, o.iters)
        for a, o in zip(tl.fieldsummary(chunks[k], sets[k], problemfile=None),
                        tl.fieldsummary(c1, s1, problemfile=None)):
            assert rel(a, o) <= 1e-12
        u, ou = chunks[k].field("u"), c1.field("u")
        assert np.max(np.abs(u - ou)) <= 1e-9 * np.max(np.abs(ou))


def test_batch_rejects_reference_mode(tl, built_lib):
    s = tl.Settings.from_text(random_deck(16, 1, steps=1), mode=0)
    c = tl.initialiseapp(s)
    with pytest.raises(tl.TeaLeafError):
        tl.Batch([c])


def test_batch_fp32_refined_matches_single_solves(tl, built_lib):
    """FP32 inner sweeps with FP64 refinement, batched: every deck meets the
    1e-10 relative true residual; iteration counts within 5 % of the deck's
    own FP32-refined solve (the FP32 sums differ in rounding, which moves the
    refinement points); u within 1e-8 of its maximum."""
    texts = _decks()
    kw = dict(mode=1, criterion=1, precision=1)
    sets = [tl.Settings.from_text(t, **kw) for t in texts]
    chunks = [tl.initialiseapp(s) for s in sets]
    hist = tl.diffuse_batch(chunks, sets, steps=3)
    for k, t in enumerate(texts):
        s1 = tl.Settings.from_text(t, **kw)
        c1 = tl.initialiseapp(s1)
        single = []
        for _ in range(3):
            tl.haloupdate(c1, s1, 1, ["energy", "density"])
            single.append(tl.CG.solve(c1, s1, s1.dtinit / s1.dx ** 2, s1.dtinit / s1.dy ** 2))
            tl.solvefinished(c1, s1)
        for step in range(3):
            b, o = hist[step][k], single[step]
            assert b.converged and 0 <= b.rel_residual < 1e-10, (k, step, b)
            assert b.refinements >= 1
            assert abs(b.iters - o.iters) <= max(3, 0.05 * o.iters), (k, step, b.iters, o.iters)
        u, ou = chunks[k].field("u"), c1.field("u")
        assert np.max(np.abs(u - ou)) <= 1e-8 * np.max(np.abs(ou))
