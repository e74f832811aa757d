"""Learned warm start: trajectories from the FP64 solver, training on the GPU
with the library's kernels (tl_conv3x3_*, tl_warm_*, tl_adam_step), the
network file, and the A/B evaluation against the plain start.

No counterpart in the reference.  The network (six 3x3 convolutions, 32
channels, GELU, BF16 weights, FP32 accumulation) maps per-cell features of
step n -- u^n, log(rx / density), u^n - u^{n-1} -- to a factor g; the
prediction of u^{n+1} is u^n + (1 + g)(u^n - u^{n-1}).  It is trained to
minimise the residual the solver's judge compares, ||u^n - A x||^2 in units of
the deck's rms increment, where u^n - A u^n = u^n - u^{n-1} holds to the solve
tolerance because u^n solved A u^n = u^{n-1}.  So a training sample is a pair
of consecutive solutions and the density; no u^{n+1} is needed.

PyTorch provides device memory and the stream only; every operation of the
forward pass, the loss, the backward pass and the optimiser runs in the
library.  Run as a script to train:
    python tealeaf.jl_gb300/warmstart.py train --out net.bin
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import struct
import sys
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

if __name__ == "__main__" and not __package__:
    # run as a script: load the package (its directory name is not an
    # importable identifier) and run this module's main from inside it
    import importlib.util
    _dir = Path(__file__).resolve().parent
    _spec = importlib.util.spec_from_file_location("tealeaf_gb300", _dir / "__init__.py",
                                                   submodule_search_locations=[str(_dir)])
    _mod = importlib.util.module_from_spec(_spec)
    sys.modules["tealeaf_gb300"] = _mod
    _spec.loader.exec_module(_mod)
    sys.exit(_mod.warmstart.main())

from . import _abi  # noqa: E402

MAGIC = b"TLWS"
VERSION = 1
NET_FILE = Path(__file__).resolve().parent / "warmstart_net.bin"


# ---------------------------------------------------------------------------
# the network file: "TLWS", version, count (little-endian int32), FP32 values
# ---------------------------------------------------------------------------

def save_params(path, params: np.ndarray, meta: dict | None = None):
    p = np.ascontiguousarray(params, dtype="<f4")
    if p.size != _abi.WARM_NPARAMS:
        raise ValueError(f"{p.size} parameters, expected {_abi.WARM_NPARAMS}")
    with open(path, "wb") as fh:
        fh.write(MAGIC + struct.pack("<ii", VERSION, p.size) + p.tobytes())
    if meta is not None:
        Path(str(path) + ".json").write_text(json.dumps(meta, indent=1) + "\n")


def load_params(path=NET_FILE) -> np.ndarray:
    raw = Path(path).read_bytes()
    if raw[:4] != MAGIC:
        raise ValueError(f"{path}: not a warm-start network file")
    version, n = struct.unpack("<ii", raw[4:12])
    if version != VERSION or n != _abi.WARM_NPARAMS:
        raise ValueError(f"{path}: version {version}, {n} parameters")
    return np.frombuffer(raw[12:12 + 4 * n], dtype="<f4").astype(np.float32)


def layer_offsets():
    """(weight offset, bias offset, cin, cout) of each layer in the parameter vector."""
    out, off = [], 0
    for ci, co in _abi.WARM_LAYERS:
        out.append((off, off + co * 9 * ci, ci, co))
        off += co * 9 * ci + co
    return out


def init_params(seed: int = 0, out_scale: float = 1e-3) -> np.ndarray:
    """He-normal weights on the used channels, zero biases, a small last layer
    (g ~ 0 at the start: the prediction starts as linear extrapolation)."""
    rng = np.random.default_rng(seed)
    parts = []
    for k, (ci, co) in enumerate(_abi.WARM_LAYERS):
        used_in = 3 if k == 0 else ci
        w = np.zeros((co, 9, ci))
        if k == len(_abi.WARM_LAYERS) - 1:
            w[0, :, :used_in] = rng.standard_normal((9, used_in)) * out_scale
        else:
            w[:, :, :used_in] = rng.standard_normal((co, 9, used_in)) * np.sqrt(2.0 / (9 * used_in))
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)


# ---------------------------------------------------------------------------
# decks and trajectories
# ---------------------------------------------------------------------------

def deck_text(n: int, seed: int, steps: int = 20, eps: float = 1e-10, maxiters: int = 40000) -> str:
    """A random-rectangle deck: background density 100, energy 1e-4, and 4-8
    rectangles with corners uniform in [0, 10]^2, density log-uniform in
    [0.1, 100], energy uniform in [0.1, 25]."""
    rng = np.random.default_rng(seed)
    lines = ["state 1 density=100.0 energy=0.0001"]
    for k in range(int(rng.integers(4, 9))):
        x0, x1 = sorted(float(v) for v in rng.uniform(0, 10, 2))
        y0, y1 = sorted(float(v) for v in rng.uniform(0, 10, 2))
        rho = float(10 ** rng.uniform(-1, 2))
        e = float(rng.uniform(0.1, 25))
        lines.append(f"state {k + 2} density={rho!r} energy={e!r} geometry=rectangle xmin={x0!r} xmax={x1!r} "
                     f"ymin={y0!r} ymax={y1!r}")
    lines += [f"x_cells={n}", f"y_cells={n}", "xmin=0.0", "ymin=0.0", "xmax=10.0", "ymax=10.0",
              "initial_timestep=0.004", f"end_step={steps}", f"max_iters={maxiters}", "use_cg", f"eps={eps!r}",
              "halo_depth=2", "coefficient=1", "summary_frequency=10"]
    return "\n".join(lines) + "\n"


@dataclass
class Trajectory:
    """Consecutive interior solutions u[0..T] (device, float64 [T+1, ny, nx])
    and the density (device [ny, nx]) of one deck."""
    u: object
    rho: object
    rx: float
    ry: float
    n: int
    seed: int


def _interior(chunk, name, hd):
    return chunk.field(name)[hd:-hd, hd:-hd].T    # [ny, nx], x contiguous


def generate(tl, n: int, seeds, steps: int, device="cuda", log=None):
    """Runs the FP64 CG (tealeaf semantics, 1e-10 relative) on each seed's
    deck and keeps u after every step."""
    import torch
    out = []
    for seed in seeds:
        s = tl.Settings.from_text(deck_text(n, seed, steps), mode=_abi.MODE_TEALEAF, exact=False,
                                  criterion=_abi.CRIT_RELATIVE, precision=_abi.PREC_FP64)
        chunk = tl.initialiseapp(s)
        hd = s.halodepth
        rx, ry = s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2
        us = torch.empty((steps + 1, s.ycells, s.xcells), dtype=torch.float64, device=device)
        e0, d0 = _interior(chunk, "energy", hd), _interior(chunk, "density", hd)
        us[0] = torch.from_numpy(np.ascontiguousarray(e0 * d0))
        for k in range(steps):
            tl.haloupdate(chunk, s, 1, ["energy", "density"])
            r = tl.CG.solve(chunk, s, rx, ry)
            if not r.converged:
                raise RuntimeError(f"deck {seed} step {k + 1} did not converge")
            us[k + 1] = torch.from_numpy(np.ascontiguousarray(_interior(chunk, "u", hd)))
            tl.solvefinished(chunk, s)
        rho = torch.from_numpy(np.ascontiguousarray(d0)).to(device)
        chunk.close()
        out.append(Trajectory(us, rho, rx, ry, n, seed))
        if log:
            log(f"trajectory n={n} seed={seed} steps={steps}")
    return out


def crop_struct(traj: Trajectory, k: int, ox: int, oy: int, scales) -> _abi.WarmCrop:
    """The crop descriptor of pair (u[k-1], u[k]) of a trajectory."""
    ny, nx = traj.u.shape[1:]
    plane = ny * nx * 8
    base = traj.u.data_ptr()
    inv_su, inv_sd = scales
    return _abi.WarmCrop(base + k * plane, base + (k - 1) * plane, traj.rho.data_ptr(), nx, nx, ny, ox, oy,
                         traj.rx, traj.ry, inv_su, inv_sd)


def pair_scales(traj: Trajectory, k: int):
    """1 / rms(u^k) and 1 / rms(u^k - u^{k-1}) over the deck (as the solver computes them)."""
    u, d = traj.u[k], traj.u[k] - traj.u[k - 1]
    su = float((u * u).mean().sqrt())
    sd = float((d * d).mean().sqrt())
    return 1.0 / su, (1.0 / sd if sd > 0 else 0.0)


# ---------------------------------------------------------------------------
# training
# ---------------------------------------------------------------------------

class Trainer:
    """Forward, loss, backward and Adam for B crops of H x W, all in the library."""

    def __init__(self, params: np.ndarray, B: int, H: int, W: int, margin: int = 7, keep_grads: bool = False,
                 objective: int = 1, device="cuda"):
        import torch
        self.torch = torch
        self.lib = _abi.load()
        self.B, self.H, self.W, self.margin, self.objective = B, H, W, margin, objective
        dev = torch.device(device)
        n = _abi.WARM_NPARAMS
        self.p = torch.tensor(np.asarray(params, dtype=np.float32), device=dev)
        self.pbf = self.p.to(torch.bfloat16)
        self.m = torch.zeros(n, device=dev)
        self.v = torch.zeros(n, device=dev)
        self.grad = torch.zeros(n, device=dev)
        self.offs = layer_offsets()
        bf = torch.bfloat16
        self.feat = torch.zeros((B, H, W, 16), dtype=bf, device=dev)
        self.z = [torch.zeros((B, H, W, 32), dtype=bf, device=dev) for _ in range(5)]
        self.a = [torch.zeros((B, H, W, 32), dtype=bf, device=dev) for _ in range(5)]
        self.g = torch.zeros((B, H, W), dtype=torch.float32, device=dev)
        self.dz_out = torch.zeros((B, H, W, 16), dtype=bf, device=dev)
        nd = 5 if keep_grads else 2
        self.dz = [torch.zeros((B, H, W, 32), dtype=bf, device=dev) for _ in range(nd)]
        self.keep_grads = keep_grads
        self.wt = [torch.zeros(ci * 9 * co, dtype=bf, device=dev) for ci, co in _abi.WARM_LAYERS]
        self.nparts = 2 * torch.cuda.get_device_properties(dev).multi_processor_count
        maxw = max(co * 9 * ci + co for ci, co in _abi.WARM_LAYERS)
        self.partials = torch.zeros(self.nparts * maxw, device=dev)
        self.resid = torch.zeros((B, H, W), dtype=torch.float64, device=dev)
        self.nblk = 32
        self.sums = torch.zeros((B, self.nblk, 2), dtype=torch.float64, device=dev)
        self.crop_loss = torch.zeros((B, 2), dtype=torch.float64, device=dev)
        self.crops = torch.zeros(B * C.sizeof(_abi.WarmCrop), dtype=torch.uint8, device=dev)
        self.step_count = 0

    # pointers -------------------------------------------------------------
    def _st(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _chk(self, rc, what):
        if rc:
            raise _abi.TeaLeafError(rc, f"{what} failed with status {rc}")

    def _wbf(self, l):
        return self.pbf.data_ptr() + 2 * self.offs[l][0]

    def _b32(self, l):
        return self.p.data_ptr() + 4 * self.offs[l][1]

    def set_crops(self, crops):
        arr = (_abi.WarmCrop * self.B)(*crops)
        host = self.torch.frombuffer(bytearray(bytes(arr)), dtype=self.torch.uint8)
        self.crops.copy_(host)

    # passes ---------------------------------------------------------------
    def forward(self):
        lib, B, H, W, st = self.lib, self.B, self.H, self.W, self._st()
        self._chk(lib.tl_warm_features(self.crops.data_ptr(), B, H, W, self.feat.data_ptr(), st), "features")
        x = self.feat
        for l, (ci, co) in enumerate(_abi.WARM_LAYERS):
            if l < 5:
                rc = lib.tl_conv3x3_forward(x.data_ptr(), self._wbf(l), self._b32(l), None, self.z[l].data_ptr(),
                                            self.a[l].data_ptr(), None, B, H, W, ci, co, 1, st)
                x = self.a[l]
            else:
                rc = lib.tl_conv3x3_forward(x.data_ptr(), self._wbf(l), self._b32(l), None, None, None,
                                            self.g.data_ptr(), B, H, W, ci, co, 0, st)
            self._chk(rc, f"conv layer {l}")

    def loss(self):
        rc = self.lib.tl_warm_loss(self.crops.data_ptr(), self.B, self.H, self.W, self.margin, self.objective,
                                   self.g.data_ptr(),
                                   self.resid.data_ptr(), self.sums.data_ptr(), self.nblk, self.crop_loss.data_ptr(),
                                   self.dz_out.data_ptr(), self._st())
        self._chk(rc, "loss")

    def backward(self):
        lib, B, H, W, st = self.lib, self.B, self.H, self.W, self._st()
        dz = self.dz_out
        for l in range(5, -1, -1):
            ci, co = _abi.WARM_LAYERS[l]
            x = self.feat if l == 0 else self.a[l - 1]
            rc = lib.tl_conv3x3_weight_grad(x.data_ptr(), dz.data_ptr(), self.partials.data_ptr(), self.nparts,
                                            self.grad.data_ptr() + 4 * self.offs[l][0], B, H, W, ci, co, st)
            self._chk(rc, f"weight grad {l}")
            if l > 0:
                self._chk(lib.tl_conv3x3_flip(self._wbf(l), self.wt[l].data_ptr(), ci, co, st), "flip")
                nxt = self.dz[l - 1] if self.keep_grads else self.dz[l % 2]
                rc = lib.tl_conv3x3_forward(dz.data_ptr(), self.wt[l].data_ptr(), None, self.z[l - 1].data_ptr(),
                                            None, nxt.data_ptr(), None, B, H, W, co, ci, 2, st)
                self._chk(rc, f"input grad {l}")
                dz = nxt

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8, clip=1.0):
        self.step_count += 1
        rc = self.lib.tl_adam_step(self.p.data_ptr(), self.m.data_ptr(), self.v.data_ptr(), self.grad.data_ptr(),
                                   self.pbf.data_ptr(), _abi.WARM_NPARAMS, lr, b1, b2, eps, self.step_count, clip,
                                   1.0, self._st())
        self._chk(rc, "adam")

    def step(self, crops, lr):
        self.set_crops(crops)
        self.forward()
        self.loss()
        self.backward()
        self.adam(lr)

    def params(self) -> np.ndarray:
        return self.p.detach().cpu().numpy().copy()


def _random_crops(rng, trajs, pairs, scales, B, size):
    crops = []
    for _ in range(B):
        t, k = pairs[rng.integers(len(pairs))]
        ny, nx = trajs[t].u.shape[1:]
        oy, ox = int(rng.integers(0, ny - size + 1)), int(rng.integers(0, nx - size + 1))
        crops.append(crop_struct(trajs[t], k, ox, oy, scales[t, k]))
    return crops


def _pairs(trajs):
    pairs = [(t, k) for t in range(len(trajs)) for k in range(1, trajs[t].u.shape[0])]
    scales = {pk: pair_scales(trajs[pk[0]], pk[1]) for pk in pairs}
    return [pk for pk in pairs if scales[pk][1] > 0], scales


def batch_objective(tr: Trainer) -> float:
    """The trainer's objective on its current batch (after forward and loss)."""
    cl = tr.crop_loss.detach().cpu().numpy()
    if tr.objective == 1:
        ok = (cl[:, 0] > 0) & (cl[:, 1] > 0)
        return float(np.mean(np.log(cl[ok, 0] / cl[ok, 1]))) if ok.any() else 0.0
    return float(cl[:, 0].mean())


def validation_loss(tr: Trainer, batches) -> float:
    """The objective of the current parameters over fixed batches of crops."""
    tot = 0.0
    for crops in batches:
        tr.set_crops(crops)
        tr.forward()
        tr.loss()
        tot += batch_objective(tr)
    return tot / len(batches)


def train(trajs, steps: int, B: int = 16, size: int = 128, lr: float = 1e-4, seed: int = 0, params=None,
          log=None, margin: int = 7, val_trajs=None, val_batches: int = 8, val_every: int = 250, objective: int = 1):
    """Adam on random crops of random consecutive pairs, cosine learning-rate
    decay.  With `val_trajs`, the loss on fixed held-out crops is measured at
    the start and every `val_every` steps and the best parameters are kept
    (the start, g = 0, is linear extrapolation).  Returns (params, history of
    (step, mean term, mean plain value, mean log ratio, best validation), selection)."""
    import torch
    rng = np.random.default_rng(seed)
    pairs, scales = _pairs(trajs)
    tr = Trainer(init_params(seed, out_scale=0.0) if params is None else params, B, size, size, margin,
                 objective=objective)
    val = None
    if val_trajs:
        vpairs, vscales = _pairs(val_trajs)
        vrng = np.random.default_rng(seed + 1)
        val = [_random_crops(vrng, val_trajs, vpairs, vscales, B, size) for _ in range(val_batches)]
    best = (validation_loss(tr, val) if val else float("inf"), tr.params(), 0)
    hist, acc = [], []
    t0 = time.time()
    for it in range(steps):
        cur_lr = lr * 0.5 * (1 + np.cos(np.pi * it / steps))
        tr.step(_random_crops(rng, trajs, pairs, scales, B, size), cur_lr)
        if it % 50 == 0 or it == steps - 1:
            acc.append(tr.crop_loss.detach().clone())
        last = it == steps - 1
        if val and ((it + 1) % val_every == 0 or last):
            v = validation_loss(tr, val)
            if v < best[0]:
                best = (v, tr.params(), it + 1)
        if ((it + 1) % 1000 == 0 or last) and acc:
            cl = torch.cat(acc).cpu().numpy()
            acc = []
            ok = (cl[:, 0] > 0) & (cl[:, 1] > 0)
            lr_mean = float(np.mean(np.log(cl[ok, 0] / cl[ok, 1]))) if ok.any() else 0.0
            hist.append((it + 1, float(cl[:, 0].mean()), float(cl[:, 1].mean()), lr_mean, best[0]))
            if log:
                log(f"step {it + 1}: term {hist[-1][1]:.3e} plain {hist[-1][2]:.3e} mean log ratio {lr_mean:.3f} "
                    f"best validation {best[0]:.4f} at step {best[2]} ({time.time() - t0:.1f} s)")
    if val:
        return best[1], hist, {"val_objective": best[0], "val_step": best[2], "objective": objective}
    return tr.params(), hist, {}


# ---------------------------------------------------------------------------
# A/B evaluation through the solver
# ---------------------------------------------------------------------------

MODES = {"plain": _abi.WARM_OFF, "network": _abi.WARM_NETWORK, "extrapolate": _abi.WARM_EXTRAPOLATE,
         "history": _abi.WARM_HISTORY}


def evaluate(tl, params, n: int, seed: int, steps: int, precision: int,
             modes=("plain", "extrapolate", "history", "network"), log=None):
    """The same deck solved from the plain start u^n, from the linear
    extrapolation 2u^n - u^{n-1}, from the A-norm projection onto the history
    (u^n and the last six increments) and from the projection with the
    network's correction added: iterations, device time, warm-start decision
    and weights per step, and the final u of each relative to the plain-start
    run."""
    out, fields = {}, {}
    for name in modes:
        s = tl.Settings.from_text(deck_text(n, seed, steps), mode=_abi.MODE_TEALEAF, exact=False,
                                  criterion=_abi.CRIT_RELATIVE, precision=precision, warmstart=MODES[name])
        chunk = tl.initialiseapp(s)
        if MODES[name] == _abi.WARM_NETWORK:
            chunk.warm_load(params)
        rx, ry = s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2
        iters, ms, used, r0p, r0q, coef = [], [], [], [], [], []
        for k in range(steps):
            chunk.check(chunk.lib.tl_synchronize(chunk.ctx))
            chunk.check(chunk.lib.tl_timer_start(chunk.ctx))
            tl.haloupdate(chunk, s, 1, ["energy", "density"])
            r = tl.CG.solve(chunk, s, rx, ry)
            tl.solvefinished(chunk, s)
            t = C.c_double()
            chunk.check(chunk.lib.tl_timer_stop(chunk.ctx, C.byref(t)))
            if not r.converged:
                raise RuntimeError(f"step {k + 1} ({name}) did not converge: {r}")
            iters.append(r.iters)
            ms.append(t.value)
            used.append(r.warm)
            r0p.append(r.r0_plain)
            r0q.append(r.r0_pred)
            coef.append(list(r.warm_coef))
        hd = s.halodepth
        out[name] = {"iters": iters, "ms": ms, "used": used, "r0_plain": r0p, "r0_pred": r0q, "coef": coef}
        fields[name] = chunk.field("u")[hd:-hd, hd:-hd].copy()
        chunk.close()
        if log:
            log(f"n={n} seed={seed} prec={precision} {name}: iters {sum(iters)} time {sum(ms):.1f} ms "
                f"predictions used {sum(1 for x in used if x == 1)}/{steps}")
    if "plain" in fields:
        ref = fields["plain"]
        for name, u in fields.items():
            out[name]["final_rel_diff"] = float(np.linalg.norm(u - ref) / np.linalg.norm(ref))
    return out


def main(argv=None):
    import torch
    import tealeaf_gb300 as tl
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default="warmstart_net.bin")
    t.add_argument("--decks512", type=int, default=192)
    t.add_argument("--decks2048", type=int, default=16)
    t.add_argument("--steps512", type=int, default=40)
    t.add_argument("--steps2048", type=int, default=24)
    t.add_argument("--iters", type=int, default=4000)
    t.add_argument("--batch", type=int, default=16)
    t.add_argument("--crop", type=int, default=128)
    t.add_argument("--lr", type=float, default=1e-4)
    t.add_argument("--eval-n", type=int, default=2048)
    t.add_argument("--eval-steps", type=int, default=40)
    t.add_argument("--eval-seeds", type=int, nargs="*", default=[900001])
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)   # noqa: E731
    t0 = time.time()
    trajs = generate(tl, 512, range(1000, 1000 + a.decks512), a.steps512, log=None)
    val = generate(tl, 512, range(5000, 5004), a.steps512, log=None)
    log(f"generated {a.decks512} trajectories at 512^2 ({time.time() - t0:.1f} s)")
    t1 = time.time()
    trajs += generate(tl, 2048, range(2000, 2000 + a.decks2048), a.steps2048, log=None)
    val += generate(tl, 2048, range(6000, 6002), a.steps2048, log=None)
    log(f"generated {a.decks2048} trajectories at 2048^2 ({time.time() - t1:.1f} s)")
    t2 = time.time()
    params, hist, sel = train(trajs, a.iters, a.batch, a.crop, a.lr, log=log, val_trajs=val)
    log(f"selected parameters: {sel}")
    torch.cuda.synchronize()
    log(f"trained {a.iters} steps ({time.time() - t2:.1f} s)")
    del trajs, val
    torch.cuda.empty_cache()
    evals = []
    for sd in a.eval_seeds:
        for prec in (_abi.PREC_FP64, _abi.PREC_FP32_IR):
            evals.append({"seed": sd, "n": a.eval_n, "precision": prec,
                          "runs": evaluate(tl, params, a.eval_n, sd, a.eval_steps, prec, log=log)})
    meta = {"decks512": a.decks512, "decks2048": a.decks2048, "steps512": a.steps512, "steps2048": a.steps2048,
            "iters": a.iters, "batch": a.batch, "crop": a.crop, "lr": a.lr, "history": hist, "selection": sel,
            "eval": evals}
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    save_params(a.out, params, meta)
    log(f"saved {a.out}")
    return 0
