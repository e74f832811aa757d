"""A second, independent restatement of the reference's CG path, written as a
near line-by-line transliteration of the Julia source with 1-based indexing
helpers, in pure Python (IEEE doubles, no FMA).  Test infrastructure: it
cross-checks the C oracle on small decks (bit-for-bit in the reference's
summation order), so that a transcription slip in either one shows up.

Covers: Chunk (src/chunk.jl:68-89), setchunkstate! (:122-151), haloupdate! /
updateface! (src/kernels.jl:146-159, 191-210), CG.init!/w!/ur!/p!/solve!
(src/solvers/CG.jl), residual!/finalise!/solvefinished!/fieldsummary
(src/kernels.jl), diffuse! (src/TeaLeaf.jl:62-83).  `intended=True` swaps in
the 5-point operator and the reflective halo.
"""
from __future__ import annotations

import math

EXCHANGE_FIELDS = ["density", "p", "energy0", "energy", "u", "sd"]


def julia_sum(vals):
    """Julia Base sum over a dense vector: _mapreduce + mapreduce_impl
    (pairwise, 1024-element sequential leaves)."""
    n = len(vals)
    if n == 0:
        return 0.0
    if n == 1:
        return vals[0]
    if n < 16:
        s = vals[0] + vals[1]
        for v in vals[2:]:
            s = s + v
        return s

    def impl(lo, hi):  # inclusive, 0-based
        if lo == hi:
            return vals[lo]
        if hi - lo < 1024:
            v = vals[lo] + vals[lo + 1]
            for i in range(lo + 2, hi + 1):
                v = v + vals[i]
            return v
        mid = lo + ((hi - lo) >> 1)
        return impl(lo, mid) + impl(mid + 1, hi)

    return impl(0, n - 1)


class Field:
    """A column-major (x, y) Float64 matrix with 1-based access."""

    def __init__(self, x, y, v=0.0):
        self.x, self.y = x, y
        self.a = [v] * (x * y)

    def __getitem__(self, ij):
        i, j = ij
        return self.a[(i - 1) + (j - 1) * self.x]

    def __setitem__(self, ij, v):
        i, j = ij
        self.a[(i - 1) + (j - 1) * self.x] = v


class Chunk:
    FIELDS = ["density0", "density", "energy0", "energy", "u", "u0", "p", "r", "mi", "w", "kx", "ky", "sd"]

    def __init__(self, s, intended):
        hd = s.halodepth
        self.x = x = s.xcells + 2 * hd
        self.y = y = s.ycells + 2 * hd
        for f in self.FIELDS:
            setattr(self, f, Field(x, y))
        self.vertexx = [s.xmin + s.dx * (k - hd - 1) for k in range(1, x + 2)]
        self.vertexy = [s.ymin + s.dy * (k - hd - 1) for k in range(1, y + 2)]
        self.volume = Field(x, y, s.dx * s.dy)
        self.cga = [0.0] * (s.maxiters + 2)
        self.cgb = [0.0] * (s.maxiters + 2)


def haloa(c, hd):
    return range(1 + hd, c.x - hd + 1), range(1 + hd, c.y - hd + 1)


def setchunkstate(ch, s, intended):
    mode = 1 if intended else 0
    states = s.states
    for k in range(len(ch.energy0.a)):
        ch.energy0.a[k] = states[0].energy
        ch.density.a[k] = states[0].density
    x, y = ch.x, ch.y
    for st in states:
        xmin, ymin, xmax, ymax = st.bounds(s, mode)
        for j in range(1, y + 1):
            for k in range(1, x + 1):
                # Rectangular arm for every state (Match.jl binds the bare symbol)
                apply = (ch.vertexx[k] >= xmin and ch.vertexx[k - 1] < xmax and ch.vertexy[j] >= ymin
                         and ch.vertexy[j - 1] < ymax)
                if not apply:
                    continue
                if intended:
                    ch.energy0[k, j] = st.energy
                    ch.density[k, j] = st.density
                else:
                    ch.energy0[j, k] = st.energy
                    ch.density[j, k] = st.density
    for j in range(2, y):
        for i in range(2, x):
            ch.u[i, j] = ch.energy0[i, j] * ch.density[i, j]


def updateface(ch, hd, depth, b, intended):
    x, y = ch.x, ch.y
    xs, ys = haloa(ch, hd)
    if not intended:
        for kk in range(1, depth + 1):
            for j in ys:
                b[hd - kk, j] = b[hd + kk, j]
        for kk in range(1, depth + 1):
            for j in ys:
                b[x - hd + kk, j] = b[x - hd - 1 - kk, j]
        for jj in range(1, depth + 1):
            for i in xs:
                b[i, y - hd + jj] = b[i, y - hd - 1 - jj]
        for jj in range(1, depth + 1):
            for i in xs:
                b[i, hd - jj] = b[i, hd + jj]
    else:  # reflective, 1-based: hd+1-kk <- hd+kk, x-hd+kk <- x-hd+1-kk (kk = 1:depth)
        for kk in range(1, depth + 1):
            for j in ys:
                b[hd + 1 - kk, j] = b[hd + kk, j]
        for kk in range(1, depth + 1):
            for j in ys:
                b[x - hd + kk, j] = b[x - hd + 1 - kk, j]
        for jj in range(1, depth + 1):
            for i in xs:
                b[i, y - hd + jj] = b[i, y - hd + 1 - jj]
        for jj in range(1, depth + 1):
            for i in xs:
                b[i, hd + 1 - jj] = b[i, hd + jj]


def haloupdate(ch, s, depth, intended, toex=None, reset=True):
    if toex is not None:
        if reset:
            s.resettoexchange()
        for f in toex:
            s.toexchange[f] = True
        fields = toex
    else:
        fields = [f for f in EXCHANGE_FIELDS if s.toexchange[f]]
    for f in fields:
        updateface(ch, s.halodepth, depth, getattr(ch, f), intended)


def smvp(ch, a, i, j, intended):
    consum = (((1 + ch.kx[i + 1, j]) + ch.kx[i, j]) + ch.ky[i, j + 1]) + ch.ky[i, j]
    v = consum * a[i, j]
    if not intended:
        return v
    v = v - (ch.kx[i + 1, j] * a[i + 1, j] + ch.kx[i, j] * a[i - 1, j])
    v = v - (ch.ky[i, j + 1] * a[i, j + 1] + ch.ky[i, j] * a[i, j - 1])
    return v


def cg_init(ch, hd, coef, rx, ry, intended):
    for k in range(len(ch.u.a)):
        ch.u.a[k] = ch.energy.a[k] * ch.density.a[k]
        ch.p.a[k] = 0.0
        ch.r.a[k] = 0.0
    # CG.jl:57-60 fills w on 2:X-1 x 2:Y-1; the intended algorithm fills the
    # whole array (with halo depth 1 the 2:X-1 range leaves w = 0 in the halo
    # and Kx, Ky at the domain edge infinite)
    lo, hi_x, hi_y = (1, ch.x + 1, ch.y + 1) if intended else (2, ch.x, ch.y)
    for j in range(lo, hi_y):
        for i in range(lo, hi_x):
            ch.w[i, j] = ch.density[i, j] if coef == 1 else 1.0 / ch.density[i, j]
    for jj in range(hd + 1, ch.y):
        for kk in range(hd + 1, ch.x):
            wl, wc, wd = ch.w[kk - 1, jj], ch.w[kk, jj], ch.w[kk, jj - 1]
            ch.kx[kk, jj] = rx * (wl + wc) / (2 * wl * wc)
            ch.ky[kk, jj] = ry * (wd + wc) / (2 * wd * wc)
    temp = 0.0
    xs, ys = haloa(ch, hd)
    for jj in ys:
        for kk in xs:
            ch.w[kk, jj] = smvp(ch, ch.u, kk, jj, intended)
            ch.r[kk, jj] = ch.u[kk, jj] - ch.w[kk, jj]
            ch.p[kk, jj] = ch.r[kk, jj]
            temp += ch.r[kk, jj] * ch.r[kk, jj]
    return temp


def cg_w(ch, hd, intended):
    temp = 0.0
    xs, ys = haloa(ch, hd)
    for jj in ys:
        for kk in xs:
            ch.w[kk, jj] = smvp(ch, ch.p, kk, jj, intended)
            temp += ch.w[kk, jj] * ch.p[kk, jj]
    return temp


def cg_ur(ch, hd, alpha):
    xs, ys = haloa(ch, hd)
    for jj in ys:
        for kk in xs:
            ch.u[kk, jj] = ch.u[kk, jj] + alpha * ch.p[kk, jj]
    for jj in ys:
        for kk in xs:
            ch.r[kk, jj] = ch.r[kk, jj] - alpha * ch.w[kk, jj]
    return julia_sum([v * v for v in ch.r.a])


def cg_p(ch, hd, beta):
    xs, ys = haloa(ch, hd)
    for jj in ys:
        for kk in xs:
            ch.p[kk, jj] = beta * ch.p[kk, jj] + ch.r[kk, jj]


def cg_solve(ch, s, rx, ry, intended):
    hd = s.halodepth
    rro = cg_init(ch, hd, s.coefficient, rx, ry, intended)
    haloupdate(ch, s, 1, intended, ["u", "p"])
    xs, ys = haloa(ch, hd)
    for jj in ys:
        for kk in xs:
            ch.u0[kk, jj] = ch.u[kk, jj]
    error = 1e10
    iters = 0
    for tt in range(1, s.maxiters + 1):
        iters = tt
        pw = cg_w(ch, hd, intended)
        alpha = rro / pw
        ch.cga[tt] = alpha
        rrn = cg_ur(ch, hd, alpha)
        beta = rrn / rro
        ch.cgb[tt] = beta
        cg_p(ch, hd, beta)
        rro = error = rrn
        haloupdate(ch, s, 1, intended)
        if math.sqrt(abs(error)) < s.eps:
            break
    return iters, error


def solvefinished(ch, s, intended):
    hd = s.halodepth
    xs, ys = haloa(ch, hd)
    if s.checkresult:
        for jj in ys:
            for kk in xs:
                ch.r[kk, jj] = ch.u0[kk, jj] - smvp(ch, ch.u, kk, jj, intended)
    for jj in ys:
        for kk in xs:
            ch.energy[kk, jj] = ch.u[kk, jj] / ch.density[kk, jj]
    haloupdate(ch, s, 1, intended, ["energy"], False)


def fieldsummary(ch, s):
    xs, ys = haloa(ch, s.halodepth)
    vals = [ch.volume[i, j] * ch.density[i, j] * ch.u[i, j] for j in ys for i in xs]
    return julia_sum(vals)


def run(s, intended):
    """initialiseapp! then diffuse! with CG; returns (chunk, per-step (iters,
    error), summaries of temperature)."""
    ch = Chunk(s, intended)
    setchunkstate(ch, s, intended)
    haloupdate(ch, s, 1, intended, ["density", "energy0", "energy"])
    ch.energy.a = list(ch.energy0.a)
    steps, sums = [], []
    for tt in range(1, s.endstep + 1):
        rx = s.dtinit / s.dx ** 2
        ry = s.dtinit / s.dy ** 2
        haloupdate(ch, s, 1, intended, ["energy", "density"])
        steps.append(cg_solve(ch, s, rx, ry, intended))
        solvefinished(ch, s, intended)
        if tt % s.summaryfrequency == 0:
            sums.append(fieldsummary(ch, s))
    sums.append(fieldsummary(ch, s))
    return ch, steps, sums
