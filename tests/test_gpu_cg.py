"""GPU parity of the CG solve path, through the C ABI, against the CPU oracle.

Reference mode and tealeaf `exact` mode reproduce the oracle bit for bit when
the oracle sums in the device order (same reduction tree); against the
reference's own summation order the iteration counts are equal and the field
summary agrees to 1e-12 relative.  The fused FMA kernels (tealeaf, exact off)
agree with the oracle to the tolerances written in each test.
"""
import numpy as np
import pytest

import oracle as O
from parity_util import CONFIG1, FIELDS, deck_text, gpu_run, oracle_run, random_deck, rel

pytestmark = pytest.mark.gpu

REF, TEA = O.MODE_REFERENCE, O.MODE_TEALEAF
SUMMARY_RTOL = 1e-12          # field_summary tolerance, relative (FP64)


def _layout(chunk):
    return chunk.reduction_layout()


@pytest.mark.parametrize("mode", [REF, TEA])
def test_config1_bit_exact_device_order(tl, built_lib, mode):
    """Config 1 (10x10, 5 states, 10 steps, eps 1e-15): every field after
    every step, every iteration count and error, bit-identical to the oracle
    summing in the device order."""
    chunk, res, sums, per = gpu_run(tl, CONFIG1, mode, exact=True, steps_fields=True)
    _, ores, osums, oper = oracle_run(CONFIG1, mode, O.ORDER_DEVICE, _layout(chunk), steps_fields=True)
    assert len(res) == len(ores) == 10
    for tt, (g, o) in enumerate(zip(res, ores)):
        assert g.iters == o.iters, f"step {tt + 1}"
        assert g.error == o.error, f"step {tt + 1}"
        for f in FIELDS:
            np.testing.assert_array_equal(per[tt][f], oper[tt][f], err_msg=f"step {tt + 1} field {f}")
    for g, o in zip(sums, osums):
        assert tuple(g) == tuple(o)
    al, be = chunk.cg_coefficients(res[-1].iters)
    assert np.all(np.isfinite(al)) and np.all(np.isfinite(be))


@pytest.mark.parametrize("mode", [REF, TEA])
def test_config1_reference_order(tl, built_lib, mode):
    """Against the reference's own summation order: iteration counts equal,
    field summary (vol, mass, ie, temp) within 1e-12 relative."""
    _, res, sums, _ = gpu_run(tl, CONFIG1, mode, exact=True)
    _, ores, osums, _ = oracle_run(CONFIG1, mode, O.ORDER_REFERENCE)
    assert [r.iters for r in res] == [r.iters for r in ores]
    for g, o in zip(sums, osums):
        for a, b in zip(g, o):
            assert rel(a, b) <= SUMMARY_RTOL


def test_config1_fused_kernels(tl, built_lib):
    """The fused FMA CG kernels on config 1 (tealeaf mode)."""
    _, res, sums, _ = gpu_run(tl, CONFIG1, TEA, exact=False)
    _, ores, osums, _ = oracle_run(CONFIG1, TEA, O.ORDER_REFERENCE)
    assert [r.iters for r in res] == [r.iters for r in ores]
    for g, o in zip(sums, osums):
        for a, b in zip(g, o):
            assert rel(a, b) <= SUMMARY_RTOL


@pytest.mark.parametrize("n,seed", [(17, 1), (64, 2), (97, 3)])
def test_random_decks_exact(tl, built_lib, n, seed):
    """Odd and even random-rectangle decks: bit-exact in device order."""
    text = random_deck(n, seed, steps=2, eps=1e-12)
    for mode in (REF, TEA):
        chunk, res, sums, per = gpu_run(tl, text, mode, exact=True, steps_fields=True)
        _, ores, osums, oper = oracle_run(text, mode, O.ORDER_DEVICE, _layout(chunk), steps_fields=True)
        assert [r.iters for r in res] == [r.iters for r in ores]
        for f in FIELDS:
            np.testing.assert_array_equal(per[-1][f], oper[-1][f], err_msg=f"mode {mode} field {f}")


@pytest.mark.parametrize("nx,ny,seed", [(64, 64, 5), (130, 70, 6), (33, 257, 7)])
def test_fused_vs_oracle(tl, built_lib, nx, ny, seed):
    """Fused FMA kernels on square and non-square tealeaf decks converging to
    1e-10 relative: equal iteration counts, summary within 1e-12 relative,
    u within 1e-9 relative of its maximum."""
    text = random_deck(nx, seed, ny=ny, steps=2, eps=1e-10)
    chunk, res, sums, per = gpu_run(tl, text, TEA, exact=False, steps_fields=True)
    _, ores, osums, oper = oracle_run(text, TEA, O.ORDER_REFERENCE, steps_fields=True)
    for g, o in zip(res, ores):
        assert abs(g.iters - o.iters) <= 1
    for g, o in zip(sums, osums):
        for a, b in zip(g, o):
            assert rel(a, b) <= SUMMARY_RTOL
    u, ou = per[-1]["u"], oper[-1]["u"]
    assert np.max(np.abs(u - ou)) <= 1e-9 * np.max(np.abs(ou))


def test_halo_both_modes(tl, built_lib):
    """updateface! index math: quirky in reference mode, reflective in tealeaf
    mode, corners untouched; compared with the oracle on a patterned field."""
    for mode in (REF, TEA):
        text = random_deck(12, 11, steps=1)
        s = tl.Settings.from_text(text, mode=mode)
        chunk = tl.initialiseapp(s)
        X, Y = chunk.size()
        pat = np.arange(X * Y, dtype=np.float64).reshape(Y, X).T + 0.5
        chunk.set_field("sd", pat)
        tl.haloupdate(chunk, s, 1, ["sd"])
        os_ = O.parse_deck(text)
        och = O.OracleChunk(os_, O.make_opts(mode=mode))
        och.set_field("sd", pat)
        och.halo(1, ["sd"])
        np.testing.assert_array_equal(chunk.field("sd"), och.field("sd"))


@pytest.mark.parametrize("mode", [REF, TEA])
def test_native_diffuse_matches_host_driver(tl, built_lib, mode):
    """tl_diffuse (the timestep loop inside the library) against the host
    mirror's diffuse, which calls the same entry points one by one."""
    import ctypes as C
    s1 = tl.Settings.from_text(CONFIG1, mode=mode, exact=True)
    c1 = tl.initialiseapp(s1)
    steps, sums = tl.diffuse(c1, s1, problemfile=None)
    s2 = tl.Settings.from_text(CONFIG1, mode=mode, exact=True)
    c2 = tl.initialiseapp(s2)
    prm = tl._params(s2, tl._abi.SOLVER_CG)
    res = (tl._abi.Result * s2.endstep)()
    out = (C.c_double * 8)()
    ns = C.c_int()
    c2.check(c2.lib.tl_diffuse(c2.ctx, C.byref(prm), s2.dtinit, s2.endstep, s2.summaryfrequency, 1, res, out, 2,
                               C.byref(ns)))
    assert [r.iters for r in res] == [r.iters for r in steps]
    assert ns.value == 2 and tuple(out[4:8]) == tuple(sums[-1])
    for f in FIELDS:
        np.testing.assert_array_equal(c1.field(f), c2.field(f), err_msg=f)


def test_coefficient_error(tl, built_lib):
    """An invalid coefficient raises like CG.jl:48-50."""
    s = tl.Settings.from_text(deck_text(coefficient=3), mode=TEA)
    chunk = tl.initialiseapp(s)
    with pytest.raises(tl.TeaLeafError) as e:
        tl.CG.solve(chunk, s, 0.004, 0.004)
    assert e.value.code == 3


GEOMETRY_DECK = """state 1 density=100.0 energy=0.0001
state 2 density=0.5 energy=20.0 geometry=circular xmin=4.0 ymin=5.0 radius=2.2
state 3 density=2.0 energy=5.0 geometry=rectangle xmin=6.0 xmax=9.0 ymin=1.0 ymax=3.0
state 4 density=1.5 energy=8.0 geometry=point xmin=2.5 ymin=7.5
x_cells=32
y_cells=32
xmin=0.0
ymin=0.0
xmax=10.0
ymax=10.0
initial_timestep=0.004
end_step=2
max_iters=5000
use_cg
eps=1e-12
halo_depth=2
coefficient=1
summary_frequency=10
"""


@pytest.mark.parametrize("mode", [REF, TEA])
def test_circular_and_point_states(tl, built_lib, mode):
    """setchunkstate! with circular and point states (chunk.jl:138-140; in
    reference mode every state takes the rectangle arm), then two CG steps:
    bit-identical to the oracle in device order."""
    chunk, res, sums, per = gpu_run(tl, GEOMETRY_DECK, mode, exact=True, steps_fields=True)
    _, ores, osums, oper = oracle_run(GEOMETRY_DECK, mode, O.ORDER_DEVICE, _layout(chunk), steps_fields=True)
    assert [r.iters for r in res] == [r.iters for r in ores]
    for f in FIELDS:
        np.testing.assert_array_equal(per[-1][f], oper[-1][f], err_msg=f)
    if mode == TEA:
        assert np.any(chunk.field("density") == 0.5)    # the circle was drawn


def test_debugrecord_dump(tl, built_lib, tmp_path):
    """debugrecord (src/TeaLeaf.jl:90-107): each field's name, then each column
    of the (X, Y) array on one line, then a blank line; the printed values
    read back to the device values exactly."""
    s = tl.Settings.from_text(CONFIG1, mode=TEA)
    chunk = tl.initialiseapp(s)
    s.debugfile = str(tmp_path / "dump.txt")
    tl.debugrecord(s, chunk)
    lines = (tmp_path / "dump.txt").read_text().split("\n")
    X, Y = chunk.size()
    pos = 0
    for name in tl._CHUNK_DUMP_FIELDS:
        assert lines[pos] == name
        a = chunk.field(name)
        for j in range(Y):
            vals = [float(t) for t in lines[pos + 1 + j].split(" ")]
            assert vals == list(a[:, j])
        assert lines[pos + 1 + Y] == ""
        pos += Y + 2


@pytest.mark.parametrize("mode,precision,criterion", [(REF, 0, 0), (TEA, 0, 0), (TEA, 1, 1)])
def test_c_driver_matches_host_mirror(tl, built_lib, tmp_path, mode, precision, criterion):
    """The plain C driver (tests/c_driver.c: the library's deck reader, then
    tl_diffuse) on config 1 gives the host mirror's summaries and iteration
    counts: bit-identical in FP64, within the refinement's tolerance in FP32."""
    import shutil
    import subprocess
    from pathlib import Path
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    root = Path(__file__).resolve().parents[1]
    lib = Path(built_lib)
    exe = tmp_path / "c_driver"
    subprocess.run(["gcc", "-std=c99", "-O1", "-I", str(root / "include"), str(root / "tests" / "c_driver.c"),
                    "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"], check=True)
    deck = tmp_path / "tea.in"
    text = CONFIG1 if precision == 0 else deck_text(eps=1e-10)
    deck.write_text(text)
    out = subprocess.run([str(exe), str(deck), str(mode), str(precision), str(criterion), "0"], check=True,
                         capture_output=True, text=True).stdout.split("\n")
    sums = [tuple(float(x) for x in ln.split()[1:]) for ln in out if ln.startswith("summary")]
    iters = [int(x) for ln in out if ln.startswith("iters") for x in ln.split()[1:]]
    s = tl.Settings.from_text(text, mode=mode, precision=precision, criterion=criterion)
    chunk = tl.initialiseapp(s)
    steps, hsums = tl.diffuse(chunk, s, problemfile=None)
    assert len(iters) == len(steps) and sums
    if precision == 0:
        assert iters == [r.iters for r in steps]
        assert sums[-1] == tuple(hsums[-1])
    else:
        assert all(abs(a - b) <= max(3, 0.05 * b) for a, b in zip(iters, [r.iters for r in steps]))
        for x, y in zip(sums[-1], hsums[-1]):
            assert rel(x, y) <= 1e-9


@pytest.mark.parametrize("ld_extra", [0, 3])
def test_upload_download_pinned_and_pageable(tl, built_lib, ld_extra):
    """tl_upload / tl_download move the same bits through both paths: pinned
    (mapped) host memory, copied by a kernel over the host link, and pageable
    memory, copied by cudaMemcpy2DAsync; with a leading dimension equal to X
    and larger than X."""
    import ctypes as C
    import torch
    s = tl.Settings.from_text(random_deck(37, 5, ny=29, steps=1), mode=TEA)
    chunk = tl.initialiseapp(s)
    X, Y = chunk.size()
    ld = X + ld_extra
    rng = np.random.default_rng(ld_extra)
    src = rng.standard_normal((Y, ld))
    dptr = C.POINTER(C.c_double)
    lib, ctx = chunk.lib, chunk.ctx
    k = tl._abi.FIELDS.index("sd")
    pinned = torch.from_numpy(src.copy()).pin_memory()
    back_pinned = torch.zeros((Y, ld), dtype=torch.float64).pin_memory()
    back_pageable = np.zeros((Y, ld))
    chunk.check(lib.tl_upload(ctx, k, C.cast(pinned.data_ptr(), dptr), ld))
    chunk.check(lib.tl_download(ctx, k, C.cast(back_pinned.data_ptr(), dptr), ld))
    chunk.check(lib.tl_download(ctx, k, back_pageable.ctypes.data_as(dptr), ld))
    np.testing.assert_array_equal(back_pinned.numpy()[:, :X], src[:, :X])
    np.testing.assert_array_equal(back_pageable[:, :X], src[:, :X])
    assert not back_pinned.numpy()[:, X:].any() and not back_pageable[:, X:].any()  # columns past X untouched
    pageable = np.ascontiguousarray(src[::-1])
    chunk.check(lib.tl_upload(ctx, k, pageable.ctypes.data_as(dptr), ld))
    chunk.check(lib.tl_download(ctx, k, C.cast(back_pinned.data_ptr(), dptr), ld))
    np.testing.assert_array_equal(back_pinned.numpy()[:, :X], pageable[:, :X])
    chunk.close()
