"""CPU checks of the warm-start oracle: BF16 rounding, the backward pass
against finite differences (float64), the parameter layout shared with the C
ABI, and the committed network file."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import warmstart_oracle as W

ROOT = Path(__file__).resolve().parents[1]


def small_deck(n=24, seed=0):
    """Fields of a small random deck: u^n, u^{n-1} (smooth + rectangle), density."""
    rng = np.random.default_rng(seed)
    rho = np.full((n, n), 100.0)
    for _ in range(3):
        x0, y0 = rng.integers(0, n - 6, 2)
        rho[y0:y0 + 6, x0:x0 + 6] = 10 ** rng.uniform(-1, 2)
    yy, xx = np.mgrid[0:n, 0:n]
    base = 1.0 + np.sin(xx / 5.0) * np.cos(yy / 7.0)
    u = base + 0.1 * rng.standard_normal((n, n))
    up = u - 0.05 * base - 0.01 * rng.standard_normal((n, n))
    return u, up, rho


def crops_of(u, up, rho, rx=3.0):
    return [W.Crop(u, up, rho, 2, 3, 16, 16, rx, rx), W.Crop(u, up, rho, 8, 0, 16, 16, rx, rx)]


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9])
    got = W.bf16(v)
    # BF16 spacing at 1 is 2^-7; 1 + 2^-8 is a tie -> even (1), 1 + 3*2^-8 is a tie -> even (1 + 2^-6)
    assert list(got) == [1.0, 1.0, 1.0 + 2 ** -7, -2.5, 1.0 + 2 ** -6, 1.0]
    torch = pytest.importorskip("torch")
    ref = torch.tensor(v, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(got, ref)


def test_param_layout_matches_header(tl):
    hdr = (ROOT / "include" / "tealeaf_gb300.h").read_text()
    m = re.search(r"#define TL_WARM_NPARAMS \((.*)\)", hdr)
    assert m and eval(m.group(1)) == W.NPARAMS == tl._abi.WARM_NPARAMS
    assert W.LAYERS == tl._abi.WARM_LAYERS
    assert C.sizeof(tl._abi.WarmCrop) == 80


def test_backward_matches_finite_differences():
    u, up, rho = small_deck()
    crops = crops_of(u, up, rho)
    rng = np.random.default_rng(1)
    p = W.init_params(3, out_scale=0.05).astype(np.float64)
    p += 0.01 * rng.standard_normal(p.size) * (p != 0)
    feat = W.features(crops, rounded=False)
    margin = 3

    def L(params):
        g, _ = W.forward(params, feat, rounded=False)
        return W.loss(crops, g, margin)[0]

    g, saved = W.forward(p, feat, rounded=False)
    _, _, dg = W.loss(crops, g, margin)
    grad = W.backward(p, saved, dg, rounded=False)
    # probe coordinates in every layer's weights and biases (used channels)
    offs, k = [], 0
    for ci, co in W.LAYERS:
        used = 3 if k == 0 else ci
        offs += [k + (o * 9 + t) * ci + c for o, t, c in ((0, 4, 0), (co - 1 if co < 16 else 1, 0, used - 1))]
        offs.append(k + co * 9 * ci)   # bias 0
        k += co * 9 * ci + co
    for i in offs:
        h = 1e-5 * max(1.0, abs(p[i]))
        e = np.zeros_like(p)
        e[i] = h
        fd = (L(p + e) - L(p - e)) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-5 * max(abs(fd), 1e-3 * np.max(np.abs(grad))), (i, fd, grad[i])


def test_loss_gradient_matches_finite_differences():
    u, up, rho = small_deck(seed=4)
    crops = crops_of(u, up, rho, rx=11.0)
    rng = np.random.default_rng(2)
    g = 0.1 * rng.standard_normal((2, 16, 16))
    L0, terms, dg = W.loss(crops, g, 3)
    assert all(t[1] > 0 for t in terms)
    for b, y, x in ((0, 8, 8), (1, 2, 5), (0, 3, 12), (1, 13, 13)):
        e = np.zeros_like(g)
        e[b, y, x] = 1e-6
        fd = (W.loss(crops, g + e, 3)[0] - W.loss(crops, g - e, 3)[0]) / 2e-6
        assert abs(fd - dg[b, y, x]) <= 1e-6 * max(abs(fd), 1e-8), (b, y, x, fd, dg[b, y, x])


def test_plain_start_loss_is_one_per_unit():
    """g = -1 (x = u^n, the plain start): r = d, so each crop's term equals its plain value."""
    u, up, rho = small_deck(seed=5)
    crops = crops_of(u, up, rho)
    L, terms, _ = W.loss(crops, -np.ones((2, 16, 16)), 3)
    for a, b in terms:
        assert a == pytest.approx(b, rel=1e-14)


def test_committed_network_file(tl):
    path = ROOT / "tealeaf.jl_gb300" / "warmstart_net.bin"
    if not path.exists():
        pytest.skip("no trained network committed")
    p = tl.warmstart.load_params(path)
    assert p.dtype == np.float32 and p.size == W.NPARAMS and np.all(np.isfinite(p))


def test_log_ratio_gradient_matches_finite_differences():
    u, up, rho = small_deck(seed=6)
    crops = crops_of(u, up, rho, rx=7.0)
    g = 0.1 * np.random.default_rng(3).standard_normal((2, 16, 16))
    _, _, dg = W.loss(crops, g, 3, objective=1)
    for b, y, x in ((0, 8, 8), (1, 4, 9)):
        e = np.zeros_like(g)
        e[b, y, x] = 1e-6
        fd = (W.loss(crops, g + e, 3, objective=1)[0] - W.loss(crops, g - e, 3, objective=1)[0]) / 2e-6
        assert abs(fd - dg[b, y, x]) <= 1e-6 * max(abs(fd), 1e-8), (b, y, x, fd, dg[b, y, x])
