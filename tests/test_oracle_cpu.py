"""CPU tests of the oracle (the checker): known answers derived by hand from
the reference's source, a cross-check against an independent Python
transliteration of the Julia code, the reduction restatements, and the
committed golden fixtures (tests/golden/make_golden.py)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import julia_transliteration as JT
import oracle as O
from parity_util import CONFIG1, deck_text, random_deck

GOLDEN = Path(__file__).resolve().parent / "golden"


def _host_settings(text, **kw):
    from conftest import load_package
    return load_package().Settings.from_text(text, **kw)


# ---------------------------------------------------------------------------
# known answers
# ---------------------------------------------------------------------------

def test_reference_halo_indices():
    """updateface! with hd=2, depth=1 on a 3x3 interior (X = Y = 7), 1-based:
    left b[1,j] <- b[3,j], right b[6,j] <- b[3,j], top b[i,6] <- b[i,3],
    bottom b[i,1] <- b[i,3], for i, j in 3:5; b[2,*], b[7,*], corners kept."""
    text = deck_text(x_cells=3, y_cells=3)
    s = O.parse_deck(text)
    ch = O.OracleChunk(s, O.make_opts(mode=O.MODE_REFERENCE))
    pat = np.arange(49, dtype=float).reshape(7, 7).T + 1.0     # pat[i, j], 0-based
    ch.set_field("sd", pat)
    ch.halo(1, ["sd"])
    got = ch.field("sd")
    exp = pat.copy()
    for j in range(2, 5):              # 0-based interior rows 2..4
        exp[0, j] = pat[2, j]          # 1-based b[1] <- b[3]
        exp[5, j] = pat[2, j]          # 1-based b[6] <- b[3]  (X-1 <- X-4)
    for i in range(2, 5):
        exp[i, 5] = pat[i, 2]
        exp[i, 0] = pat[i, 2]
    np.testing.assert_array_equal(got, exp)


def test_reflective_halo_indices():
    text = deck_text(x_cells=3, y_cells=4)
    s = O.parse_deck(text)
    ch = O.OracleChunk(s, O.make_opts(mode=O.MODE_TEALEAF))
    X, Y = 7, 8
    pat = np.arange(X * Y, dtype=float).reshape(Y, X).T + 1.0
    ch.set_field("sd", pat)
    ch.halo(2, ["sd"])
    got = ch.field("sd")
    exp = pat.copy()
    for j in range(2, Y - 2):
        exp[1, j], exp[0, j] = pat[2, j], pat[3, j]
        exp[X - 2, j], exp[X - 1, j] = pat[X - 3, j], pat[X - 4, j]
    for i in range(2, X - 2):
        exp[i, 1], exp[i, 0] = pat[i, 2], pat[i, 3]
        exp[i, Y - 2], exp[i, Y - 1] = pat[i, Y - 3], pat[i, Y - 4]
    np.testing.assert_array_equal(got, exp)


def test_config1_initial_density_transposed():
    """setchunkstate! in the reference writes [j, k] (dim 1 = y-vertex index):
    state 2 (x 0..1, y 1..2, inset 0.1) lands on 0-based [3, 2], state 3
    (x 1..6, y 1..2) on [3, 3..7]; the halo update then copies [3, 2] into
    [3, 0] (bottom face, 1-based b[i,1] <- b[i,3])."""
    s = O.parse_deck(CONFIG1)
    ch = O.OracleChunk(s, O.make_opts(mode=O.MODE_REFERENCE))
    ch.initialise()
    rho = ch.field("density")
    assert rho[3, 2] == 0.1 and all(rho[3, k] == 0.1 for k in range(3, 8))
    assert rho[3, 0] == 0.1 and rho[3, 1] == 100.0
    assert rho[2, 3] == 100.0      # the untransposed position stays background
    tea = O.OracleChunk(O.parse_deck(CONFIG1), O.make_opts(mode=O.MODE_TEALEAF))
    tea.initialise()
    trho = tea.field("density")   # tealeaf mode: dim 1 = x index, so state 2 sits at [2, 3]
    assert trho[2, 3] == 0.1 and trho[3, 3] == 0.1 and trho[3, 2] == 100.0


def test_diagonal_operator_one_iteration():
    """With kx = ky = 0 (rx = ry = 0) the operator is the identity: r = u - u =
    0 at init, so CG stops after one iteration with error 0 (CG.jl:24)."""
    s = O.parse_deck(CONFIG1)
    for mode in (O.MODE_REFERENCE, O.MODE_TEALEAF):
        ch = O.OracleChunk(s, O.make_opts(mode=mode))
        ch.initialise()
        ch.halo(1, ["energy", "density"])
        r = ch.solve(0.0, 0.0)
        assert r.iters == 1 and r.error == 0.0 or math.isnan(r.error)


def test_state_inset_uses_parse_time_dx():
    """readstate insets by dx/100 with dx still the default (100-0)/10 = 10
    while the file is read (settings.jl:72, 159-162)."""
    s = O.parse_deck(CONFIG1)
    assert s.states[1].pdx == 10.0
    assert O.effective_bounds(s, 1, O.MODE_REFERENCE) == (0.1, 1.1, 0.9, 1.9)
    assert O.effective_bounds(s, 1, O.MODE_TEALEAF) == (0.01, 1.01, 0.99, 1.99)
    assert s.dx == 1.0 and s.dy == 1.0


# ---------------------------------------------------------------------------
# the reductions
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("n", [0, 1, 2, 15, 16, 17, 1023, 1024, 1025, 5000])
def test_pairwise_sum_matches_transliteration(n):
    rng = np.random.default_rng(n)
    v = rng.standard_normal(n) * 10.0 ** rng.integers(-8, 8, n)
    assert O.pairwise_sum(v) == JT.julia_sum([float(x) for x in v])


def _device_tree(v, warps, rows, blocks):
    """A direct Python statement of the device reduction tree."""
    nx, ny = v.shape
    TW = 64 * warps
    ntx, nty = -(-nx // TW), -(-ny // rows)
    T = ntx * nty

    def bfly(lanes):
        for off in (16, 8, 4, 2, 1):
            lanes = [lanes[l] + lanes[l ^ off] for l in range(32)]
        return lanes[0]

    partial = []
    for b in range(blocks):
        acc = [0.0] * (32 * warps)
        for t in range(b, T, blocks):
            tx, ty = t % ntx, t // ntx
            for w in range(warps):
                for l in range(32):
                    i0 = tx * TW + 64 * w + 2 * l
                    a = acc[32 * w + l]
                    for j in range(ty * rows, min(ty * rows + rows, ny)):
                        if i0 < nx:
                            a = a + float(v[i0, j])
                        if i0 + 1 < nx:
                            a = a + float(v[i0 + 1, j])
                    acc[32 * w + l] = a
        tot = None
        for w in range(warps):
            s = bfly(acc[32 * w:32 * w + 32])
            tot = s if tot is None else tot + s
        partial.append(tot)
    F = 32 * warps
    acc = [0.0] * F
    for t in range(F):
        a = 0.0
        for k in range(t, blocks, F):
            a = a + partial[k]
        acc[t] = a
    tot = None
    for w in range(warps):
        s = bfly(acc[32 * w:32 * w + 32])
        tot = s if tot is None else tot + s
    return tot


@pytest.mark.parametrize("shape,layout", [((10, 10), (4, 8, 2)), ((37, 53), (4, 8, 5)), ((300, 7), (2, 3, 3))])
def test_device_sum_tree(shape, layout):
    rng = np.random.default_rng(7)
    v = rng.standard_normal(shape) * 1e3
    assert O.device_sum(v, layout) == _device_tree(v, *layout)
    ints = rng.integers(-1000, 1000, shape).astype(float)
    assert O.device_sum(ints, layout) == float(ints.sum())


# ---------------------------------------------------------------------------
# the oracle against the independent transliteration
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("mode", [O.MODE_REFERENCE, O.MODE_TEALEAF])
@pytest.mark.parametrize("text", [CONFIG1, random_deck(12, 3, steps=3, eps=1e-13)],
                         ids=["config1", "random12"])
def test_oracle_matches_transliteration(mode, text):
    s = _host_settings(text, mode=mode)
    jch, jsteps, jsums = JT.run(s, intended=mode == O.MODE_TEALEAF)
    och = O.OracleChunk(O.parse_deck(text), O.make_opts(mode=mode))
    och.initialise()
    osteps, osums = och.diffuse()
    assert [(r.iters, r.error) for r in osteps] == [(i, e) for i, e in jsteps]
    assert [x[3] for x in osums] == jsums
    for f in ("density", "energy0", "energy", "u", "u0", "p", "r", "w", "kx", "ky"):
        a = np.array(getattr(jch, f).a).reshape(jch.y, jch.x).T
        np.testing.assert_array_equal(och.field(f), a, err_msg=f)


# ---------------------------------------------------------------------------
# golden fixtures
# ---------------------------------------------------------------------------

def _golden_cases():
    return json.loads((GOLDEN / "oracle_golden.json").read_text())["cases"]


@pytest.mark.parametrize("case", _golden_cases(), ids=lambda c: c["name"])
def test_golden(case):
    from make_golden import run_case
    got = run_case(case["deck"], case["mode"], case["solver"])
    assert got["status"] == case["status"]
    assert got["steps"] == case["steps"]
    assert got["summaries"] == case["summaries"]
    assert got["u_checksum"] == case["u_checksum"]


# ---------------------------------------------------------------------------
# the relative criterion against a direct sparse solve
# ---------------------------------------------------------------------------

def _operator_from_fields(kx, ky, hd):
    """The tealeaf-mode 5-point operator of the oracle's Kx, Ky (interior
    cells, reflective boundary: a neighbour across the edge is the cell
    itself, so that coupling drops out) as a scipy sparse matrix."""
    import scipy.sparse as sp
    X, Y = kx.shape
    nx, ny = X - 2 * hd, Y - 2 * hd
    idx = np.arange(nx * ny).reshape(ny, nx).T          # idx[i, j], i fastest
    rows, cols, vals = [], [], []
    diag = np.ones((nx, ny))
    for di, dj, k in ((1, 0, kx[hd + 1:X - hd + 1, hd:Y - hd]), (-1, 0, kx[hd:X - hd, hd:Y - hd]),
                      (0, 1, ky[hd:X - hd, hd + 1:Y - hd + 1]), (0, -1, ky[hd:X - hd, hd:Y - hd])):
        ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        ni, nj = ii + di, jj + dj
        inside = (ni >= 0) & (ni < nx) & (nj >= 0) & (nj < ny)
        diag += np.where(inside, k, 0.0)
        rows.append(idx[inside])
        cols.append(idx[ni[inside], nj[inside]])
        vals.append(-k[inside])
    rows.append(idx.ravel())
    cols.append(idx.ravel())
    vals.append(diag.ravel())
    n = nx * ny
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


@pytest.mark.parametrize("nx,ny,seed", [(40, 40, 3), (57, 31, 4)])
def test_relative_criterion_against_direct_solve(nx, ny, seed):
    """CG with the relative criterion (the GPU library's TL_CRIT_RELATIVE)
    stops with ||u0 - A u|| / ||u0|| < eps, checked on the true residual, and
    its u equals scipy's direct sparse solve of the same 5-point system
    to the accuracy that residual allows."""
    import scipy.sparse.linalg as spla
    text = random_deck(nx, seed, ny=ny, steps=1, eps=1e-10)
    s = O.parse_deck(text)
    ch = O.OracleChunk(s, O.make_opts(mode=O.MODE_TEALEAF, criterion=1))
    ch.initialise()
    ch.halo(1, ["energy", "density"])
    r = ch.solve(s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    assert r.converged and 0 <= r.rel_residual < 1e-10
    hd = s.halodepth
    A = _operator_from_fields(ch.field("kx"), ch.field("ky"), hd)
    u0 = ch.field("u0")[hd:-hd, hd:-hd]
    u = ch.field("u")[hd:-hd, hd:-hd]
    exact = spla.spsolve(A.tocsc(), u0.T.ravel()).reshape(ny, nx).T
    true_rel = np.linalg.norm(u0.T.ravel() - A @ u.T.ravel()) / np.linalg.norm(u0)
    assert abs(true_rel - r.rel_residual) <= 1e-3 * r.rel_residual + 1e-16
    assert np.max(np.abs(u - exact)) <= 1e-8 * np.max(np.abs(exact))


def test_relative_criterion_edges():
    """Near the rounding floor (eps 1e-14) the loop ends converged on the true
    residual or out of restarts with it measured; a tolerance the start
    already meets stops before the first iteration (no 0/0 alpha)."""
    text = random_deck(48, 9, steps=1, eps=1e-14)
    s = O.parse_deck(text)
    ch = O.OracleChunk(s, O.make_opts(mode=O.MODE_TEALEAF, criterion=1))
    ch.initialise()
    ch.halo(1, ["energy", "density"])
    r = ch.solve(s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    assert r.rel_residual >= 0 and (bool(r.converged) == (r.rel_residual < 1e-14))
    s2 = O.parse_deck(random_deck(48, 9, steps=1, eps=10.0))
    ch2 = O.OracleChunk(s2, O.make_opts(mode=O.MODE_TEALEAF, criterion=1))
    ch2.initialise()
    ch2.halo(1, ["energy", "density"])
    r2 = ch2.solve(s2.dtinit / s2.dx ** 2, s2.dtinit / s2.dy ** 2)
    assert r2.converged and r2.iters == 0 and 0 <= r2.rel_residual < 10.0
