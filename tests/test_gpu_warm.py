"""GPU checks of the warm-start network kernels against the CPU oracle
(oracle/warmstart_oracle.py), the trainer, and the warm start inside CG.

Per-kernel checks feed the oracle the same BF16 inputs the kernels read, so
each comparison isolates one kernel: BF16 outputs agree to one BF16 unit in
the last place (at most 2^-7 relative: a different FP32 summation order or
tanh can move a value across a rounding boundary) plus FP32 accumulation, FP32 outputs to 1e-5, the FP64 loss to
1e-10.  The end-to-end gradient (oracle forward + backward with BF16 rounding
at the same points) agrees per layer to 5e-2 in norm: a different FP32
summation order can flip a BF16 rounding, which then propagates.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import warmstart_oracle as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
ULP = 2.0 ** -7


def deck_arrays(ny=40, nx=56, seed=0):
    rng = np.random.default_rng(seed)
    rho = np.full((ny, nx), 100.0)
    for _ in range(4):
        x0, y0 = rng.integers(0, nx - 10), rng.integers(0, ny - 10)
        rho[y0:y0 + 10, x0:x0 + 14] = 10 ** rng.uniform(-1, 2)
    yy, xx = np.mgrid[0:ny, 0:nx]
    base = 1.0 + np.sin(xx / 6.0) * np.cos(yy / 9.0)
    u = base + 0.2 * (rho < 50) + 0.05 * rng.standard_normal((ny, nx))
    up = u - 0.03 * base - 0.01 * rng.standard_normal((ny, nx))
    return u, up, rho


def setup(tl, B_crops, H, W_, params, margin=3, rx=5.0, objective=0):
    u, up, rho = deck_arrays()
    dev = {k: torch.tensor(v, dtype=torch.float64, device="cuda") for k, v in (("u", u), ("up", up), ("rho", rho))}
    ocrops = [W.Crop(u, up, rho, ox, oy, H, W_, rx, rx) for ox, oy in B_crops]
    ny, nx = u.shape
    gcrops = [tl._abi.WarmCrop(dev["u"].data_ptr(), dev["up"].data_ptr(), dev["rho"].data_ptr(), nx, nx, ny, c.ox,
                               c.oy, rx, rx, c.inv_su, c.inv_sd) for c in ocrops]
    tr = tl.warmstart.Trainer(params, len(ocrops), H, W_, margin=margin, keep_grads=True, objective=objective)
    tr.set_crops(gcrops)
    return tr, ocrops, dev


def f64(t):
    return t.detach().float().cpu().numpy().astype(np.float64)


def close_bf16(gpu, ref, what):
    tol = ULP * np.abs(ref) + 1e-5 * max(np.max(np.abs(ref)), 1e-30)
    bad = np.abs(gpu - ref) > tol
    assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} beyond one BF16 rounding, max {np.max(np.abs(gpu - ref))}"


@pytest.fixture(scope="module")
def run(tl, built_lib):
    rng = np.random.default_rng(7)
    p = W.init_params(11, out_scale=0.05)
    p = (p + 0.02 * rng.standard_normal(p.size).astype(np.float32) * (p != 0)).astype(np.float32)
    tr, ocrops, dev = setup(tl, [(3, 2), (12, 14)], 24, 40, p)
    tr.forward()
    tr.loss()
    tr.backward()
    torch.cuda.synchronize()
    return tr, ocrops, p, dev


def test_features(run):
    tr, ocrops, p, _ = run
    ref = W.features(ocrops, rounded=True)
    close_bf16(f64(tr.feat), ref, "features")


def test_forward_layers(run):
    tr, ocrops, p, _ = run
    layers = W.unpack(p.astype(np.float64))
    x = f64(tr.feat)
    for l in range(5):
        w, b = layers[l]
        z = W.conv(x, W.bf16(w)) + b
        close_bf16(f64(tr.z[l]), W.bf16(z), f"z{l}")
        close_bf16(f64(tr.a[l]), W.bf16(W.gelu(z)), f"a{l}")
        x = f64(tr.a[l])
    w, b = layers[5]
    g = (W.conv(x, W.bf16(w)) + b)[..., 0]
    gg = tr.g.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(gg - g)) <= 1e-5 * np.max(np.abs(g))


def test_loss_and_output_gradient(run):
    tr, ocrops, p, _ = run
    g = tr.g.cpu().numpy().astype(np.float64)
    L, terms, dg = W.loss(ocrops, g, tr.margin)
    cl = tr.crop_loss.cpu().numpy()
    for b, (a, plain) in enumerate(terms):
        assert cl[b, 0] == pytest.approx(a, rel=1e-10)
        assert cl[b, 1] == pytest.approx(plain, rel=1e-10)
    dz = f64(tr.dz_out)
    assert np.all(dz[..., 1:] == 0)
    close_bf16(dz[..., 0], W.bf16(np.float32(dg)), "dL/dg")


def test_weight_and_input_gradients(run):
    tr, ocrops, p, _ = run
    layers = W.unpack(p.astype(np.float64))
    grad = tr.grad.cpu().numpy().astype(np.float64)
    offs = [o for o in __import__("itertools").accumulate([0] + [co * 9 * ci + co for ci, co in W.LAYERS])]
    for l in range(6):
        ci, co = W.LAYERS[l]
        x = f64(tr.feat) if l == 0 else f64(tr.a[l - 1])
        dz = f64(tr.dz_out) if l == 5 else f64(tr.dz[l])
        dw, db = W.conv_weight_grad(x, dz)
        ref = np.concatenate([dw.ravel(), db])
        got = grad[offs[l]:offs[l + 1]]
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref) + 1e-30, f"weight grad {l}"
        if l > 0:
            dx = W.conv_input_grad(dz, W.bf16(layers[l][0]))
            ref_dz = W.bf16(dx * W.gelu_grad(f64(tr.z[l - 1])))
            close_bf16(f64(tr.dz[l - 1]), ref_dz, f"input grad {l}")


def test_log_ratio_objective_gradient(tl, built_lib):
    """Objective 1 (mean log(term / plain)): the output gradient against the oracle."""
    p = W.init_params(3, out_scale=0.05)
    tr, ocrops, dev = setup(tl, [(3, 2), (12, 14)], 24, 40, p, objective=1)
    tr.forward()
    tr.loss()
    torch.cuda.synchronize()
    g = tr.g.cpu().numpy().astype(np.float64)
    L, terms, dg = W.loss(ocrops, g, tr.margin, objective=1)
    assert tl.warmstart.batch_objective(tr) == pytest.approx(L, rel=1e-9)
    close_bf16(f64(tr.dz_out)[..., 0], W.bf16(np.float32(dg)), "dlog/dg")


def test_end_to_end_gradient(run):
    tr, ocrops, p, _ = run
    feat = W.features(ocrops, rounded=True)
    g, saved = W.forward(p.astype(np.float64), feat, rounded=True)
    _, _, dg = W.loss(ocrops, g, tr.margin)
    ref = W.backward(p.astype(np.float64), saved, dg, rounded=True)
    got = tr.grad.cpu().numpy().astype(np.float64)
    k = 0
    for l, (ci, co) in enumerate(W.LAYERS):
        n = co * 9 * ci + co
        r, gg = ref[k:k + n], got[k:k + n]
        assert np.linalg.norm(gg - r) <= 5e-2 * np.linalg.norm(r), f"layer {l}"
        k += n


def test_training_reduces_loss_on_a_fixed_batch(tl, built_lib):
    p = W.init_params(5)
    tr, ocrops, dev = setup(tl, [(3, 2), (12, 14), (0, 0), (16, 16)], 24, 40, p)
    first = None
    for it in range(120):
        tr.forward()
        tr.loss()
        if it == 0:
            first = tr.crop_loss[:, 0].mean().item()
        tr.backward()
        tr.adam(2e-3)
    tr.forward()
    tr.loss()
    last = tr.crop_loss[:, 0].mean().item()
    assert np.isfinite(last) and last < 0.5 * first, (first, last)


@pytest.mark.parametrize("precision", [0, 1])
def test_warm_start_judge_and_accuracy(tl, built_lib, precision):
    """CG from the projected start: every solve meets eps on the true
    residual, the prediction is used exactly when its initial residual is
    below the plain start's, and the final field matches the plain-start run."""
    params = W.init_params(0)
    if (tl.warmstart.NET_FILE).exists():
        params = tl.warmstart.load_params()
    ev = tl.warmstart.evaluate(tl, params, 128, 424242, 12, precision)
    for name in ("network", "history", "extrapolate"):
        w = ev[name]
        assert w["used"][0] == 0                       # no previous step yet
        for k in range(1, 12):
            used, a, b = w["used"][k], w["r0_pred"][k], w["r0_plain"][k]
            assert used in ((1, 2, 3) if name == "network" else (1, 2))
            assert (used in (1, 3)) == (a < b), (name, k, a, b)
            if used == 3:                              # the network's term lost its judge
                assert w["coef"][k][tl._abi.WARM_HIST + 1] == 0.0
        assert w["final_rel_diff"] < 1e-7


def _operator(kx, ky, hd):
    """The tealeaf-mode 5-point operator of Kx, Ky on the interior (reflective
    boundary) as a scipy sparse matrix, cells ordered i fastest."""
    sp = pytest.importorskip("scipy.sparse")
    X, Y = kx.shape
    nx, ny = X - 2 * hd, Y - 2 * hd
    idx = np.arange(nx * ny).reshape(ny, nx).T
    rows, cols, vals = [], [], []
    diag = np.ones((nx, ny))
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    for di, dj, k in ((1, 0, kx[hd + 1:X - hd + 1, hd:Y - hd]), (-1, 0, kx[hd:X - hd, hd:Y - hd]),
                      (0, 1, ky[hd:X - hd, hd + 1:Y - hd + 1]), (0, -1, ky[hd:X - hd, hd:Y - hd])):
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


def test_history_projection_is_the_a_norm_optimum(tl, built_lib):
    """The projected start against a CPU restatement of the projection: with
    the same right-hand sides u^n (the u0 field of each step), A from the
    context's Kx, Ky, the optimal weights c minimise ||V c - A^{-1} u^n||_A
    over V = [u^n, u^n - u^{n-1}, u^{n-1} - u^{n-2}, ...] with the increments
    that exist (at most TL_WARM_HIST).  The GPU's weights give an A-norm error
    within 1e-6 of the optimum's, and its weights on u^n, u^{n-1}, ... agree
    to 1e-5 of the largest."""
    spla = pytest.importorskip("scipy.sparse.linalg")
    from parity_util import random_deck
    nhist = tl._abi.WARM_HIST
    steps = nhist + 4
    s = tl.Settings.from_text(random_deck(96, 515, steps=steps, eps=1e-10), mode=1, criterion=1,
                              warmstart=tl._abi.WARM_HISTORY)
    chunk = tl.initialiseapp(s)
    hd = s.halodepth
    rhs, res = [], []
    for _ in range(steps):
        tl.haloupdate(chunk, s, 1, ["energy", "density"])
        res.append(tl.CG.solve(chunk, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2))
        rhs.append(chunk.field("u0")[hd:-hd, hd:-hd].T.ravel().copy())
        tl.solvefinished(chunk, s)
    A = _operator(chunk.field("kx"), chunk.field("ky"), hd)
    lu = spla.splu(A.tocsc())
    checked = 0
    for k in range(3, steps):
        if res[k].warm != 1:
            continue                                             # the plain start won its judge
        nh = min(k, nhist)
        b = rhs[k]
        H = [rhs[k - j] for j in range(nh + 1)]                  # u^n, u^{n-1}, ..., u^{n-nh}
        V = np.array([H[0]] + [H[j - 1] - H[j] for j in range(1, nh + 1)]).T
        AV = A @ V
        G = V.T @ AV
        d = 1 / np.sqrt(np.diag(G))
        c = d * np.linalg.lstsq(d[:, None] * G * d[None, :], d * (V.T @ b), rcond=1e-12)[0]
        w_np = np.zeros(nh + 1)
        w_np[0] = c[0] + c[1]
        for q in range(1, nh + 1):
            w_np[q] = (c[q + 1] if q < nh else 0.0) - c[q]
        w_gpu = np.array(res[k].warm_coef[:nh + 1])
        xstar = lu.solve(b)
        err = lambda x: float(np.sqrt((x - xstar) @ (A @ (x - xstar))))   # noqa: E731
        e_gpu = err(np.array(H).T @ w_gpu)
        e_np = err(np.array(H).T @ w_np)
        assert e_gpu <= e_np * (1 + 1e-6) + 1e-14 * np.linalg.norm(b), (k, e_gpu, e_np)
        assert np.max(np.abs(w_gpu - w_np)) <= 1e-5 * np.max(np.abs(w_np)), (k, w_gpu, w_np)
        assert res[k].warm_coef[nhist + 1] == 0.0
        # never farther than the plain start or the extrapolation
        assert e_gpu <= err(H[0]) and e_gpu <= err(2 * H[0] - H[1])
        checked += 1
    assert checked >= 4, [r.warm for r in res]


def test_trained_network_gain(tl, built_lib):
    """What the committed network gains over the method without it, on a
    held-out 512^2 deck over 24 steps (FP64 CG to 1e-10): total iterations
    from the plain start, from linear extrapolation, from the projection onto
    the history alone and from the projection with the network's term.  The
    projections contain the plain start and the extrapolation, so they need
    fewer iterations than both; the network's term is kept only with the
    weight the A-norm gives it."""
    if not tl.warmstart.NET_FILE.exists():
        pytest.skip("no trained network committed")
    params = tl.warmstart.load_params()
    ev = tl.warmstart.evaluate(tl, params, 512, 777001, 24, 0)
    tot = {k: sum(v["iters"]) for k, v in ev.items()}
    print("iterations over 24 steps:", tot)
    for k in ("network", "history", "extrapolate"):
        assert ev[k]["final_rel_diff"] < 1e-8
    assert tot["network"] < tot["extrapolate"] < tot["plain"]
    assert tot["history"] < tot["extrapolate"]


@pytest.mark.parametrize("N,H,Wd", [(2, 37, 150), (3, 131, 300), (1, 1040, 1000)])
@pytest.mark.parametrize("cin,cout,mode", [(16, 32, 1), (32, 32, 1), (32, 16, 0), (32, 32, 2), (16, 32, 0)])
def test_conv_forward_ragged_shapes(tl, built_lib, cin, cout, mode, N, H, Wd):
    """The forward kernel on images whose width spans 128-pixel columns with
    a ragged end, several images, every mode, against the oracle's
    convolution.  The two small shapes get short tiles (one row on 37 x 150 x
    2), 1040 x 1000 the 16-row tiles with some blocks taking two; the rows
    are ragged at the bottom of each image."""
    rng = np.random.default_rng(cin * 7 + cout + mode)
    x = W.bf16(rng.standard_normal((N, H, Wd, cin)))
    w = W.bf16(0.1 * rng.standard_normal((cout, 9, cin)))
    b = rng.standard_normal(cout).astype(np.float32).astype(np.float64)
    gz = W.bf16(rng.standard_normal((N, H, Wd, cout)))
    dev = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda").to(torch.bfloat16)  # noqa: E731
    xd, wd, gzd = dev(x), dev(w.reshape(-1)), dev(gz)
    bd = torch.tensor(b, dtype=torch.float32, device="cuda")
    out = torch.zeros((N, H, Wd, cout), dtype=torch.bfloat16, device="cuda")
    zd = torch.zeros_like(out)
    g32 = torch.zeros((N, H, Wd), dtype=torch.float32, device="cuda")
    lib = tl._abi.load()
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.tl_conv3x3_forward(xd.data_ptr(), wd.data_ptr(), bd.data_ptr() if mode != 2 else None,
                                gzd.data_ptr() if mode == 2 else None, zd.data_ptr() if mode == 1 else None,
                                out.data_ptr(), g32.data_ptr(), N, H, Wd, cin, cout, mode, st)
    assert rc == 0
    torch.cuda.synchronize()
    z = W.conv(x, w) + (b if mode != 2 else 0.0)
    ref = {0: z, 1: W.gelu(z), 2: z * W.gelu_grad(gz)}[mode]
    close_bf16(f64(out), W.bf16(ref), f"conv {cin}->{cout} mode {mode}")
    if mode == 1:
        close_bf16(f64(zd), W.bf16(z), "pre-activation")
    gg = g32.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(gg - z[..., 0])) <= 1e-5 * np.max(np.abs(z[..., 0]))
    timeouts = ctypes.c_int(-1)
    assert lib.tl_conv_status(ctypes.byref(timeouts)) == 0 and timeouts.value == 0


def test_conv_forward_at_the_measured_size(tl, built_lib):
    """The 32->32 GELU layer on one 2048 x 2048 image, the size whose rate
    the bench reports (16-row tiles, several per block), against the
    oracle's convolution: every output within one BF16 rounding."""
    n, ci, co = 2048, 32, 32
    rng = np.random.default_rng(2048)
    x = W.bf16(rng.standard_normal((1, n, n, ci)).astype(np.float32))
    w = W.bf16(0.05 * rng.standard_normal((co, 9, ci)))
    b = rng.standard_normal(co).astype(np.float32).astype(np.float64)
    dev = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda").to(torch.bfloat16)  # noqa: E731
    xd, wd = dev(x), dev(w.reshape(-1))
    bd = torch.tensor(b, dtype=torch.float32, device="cuda")
    out = torch.zeros((1, n, n, co), dtype=torch.bfloat16, device="cuda")
    lib = tl._abi.load()
    st = torch.cuda.current_stream().cuda_stream
    assert lib.tl_conv3x3_forward(xd.data_ptr(), wd.data_ptr(), bd.data_ptr(), None, None, out.data_ptr(), None,
                                  1, n, n, ci, co, 1, st) == 0
    torch.cuda.synchronize()
    close_bf16(f64(out), W.bf16(W.gelu(W.conv(x, w) + b)), "conv 32->32 GELU at 2048^2")
    timeouts = ctypes.c_int(-1)
    assert lib.tl_conv_status(ctypes.byref(timeouts)) == 0 and timeouts.value == 0


@pytest.mark.parametrize("knob,value", [("TEALEAF_GB300_CONV_WS", "1"), ("TEALEAF_GB300_CONV_WS", "2"),
                                        ("TEALEAF_GB300_CONV_ROWS", "1"), ("TEALEAF_GB300_CONV_ROWS", "16")])
def test_conv_forward_other_producers(built_lib, knob, value):
    """The same ragged-shape checks in a child process (the choices are read
    once per process): tensor-copy rows with every epilogue warp on every
    row at three blocks per SM in every mode (CONV_WS 1), the cp.async
    producer (CONV_WS 2), one-row tiles (several per block, streamed back to
    back) and 16-row tiles on every shape."""
    env = dict(os.environ, **{knob: value})
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-m", "gpu",
                        f"{__file__}::test_conv_forward_ragged_shapes"], env=env, capture_output=True, text=True,
                       timeout=600, cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]


def test_warm_context_destroy_leaves_no_error(tl, built_lib, monkeypatch):
    """A context whose warm start rotated its history buffers frees them
    cleanly: the next context is created without a stale CUDA error (with the
    layout tuner off, nothing would clear one before tl_create checks)."""
    from parity_util import random_deck
    s = tl.Settings.from_text(random_deck(64, 77, steps=9, eps=1e-10), mode=1, criterion=1,
                              warmstart=tl._abi.WARM_HISTORY)
    chunk = tl.initialiseapp(s)
    for _ in range(9):
        tl.haloupdate(chunk, s, 1, ["energy", "density"])
        tl.CG.solve(chunk, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
        tl.solvefinished(chunk, s)
    chunk.close()
    monkeypatch.setenv("TEALEAF_GB300_TUNE", "0")
    s2 = tl.Settings.from_text(random_deck(64, 78, steps=1, eps=1e-10), mode=1)
    tl.initialiseapp(s2).close()
