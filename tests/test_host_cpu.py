"""CPU tests of the host side: the deck reader of the host mirror against the
oracle's restatement of src/settings.jl, and the C ABI library's exports
(every entry point declared in include/tealeaf_gb300.h) without compute calls."""
import ctypes as C
import re
from pathlib import Path

import pytest

import oracle as O
from conftest import load_package
from parity_util import CONFIG1, random_deck

ROOT = Path(__file__).resolve().parents[1]

DECKS = [
    CONFIG1,
    random_deck(64, 3, ny=40, steps=4, eps=1e-9, solver="ppcg", presteps=12),
    # underscores stripped, the initial_timestep alias, a comment, unknown and malformed keys
    "*tea\nx_cells = 20\ny_cells=20\nxmax=5.0\nymax=5.0\ninitial_timestep=0.01\nend_step=3\n"
    "tl_max_iters=77\nmax_iters=500\nbogus=3\neps=1e-12\nerror_switch=true\neps_lim=1e-4\nuse_cheby\n"
    "pres_teps=7\nhalo_depth=2\ncoefficient=2\ncheck_result=0\n"
    "state 1 density=1.0 energy=1.0\n"
    "state 2 density=2.5 energy=3.0 geometry=circular xmin=2.5 ymin=2.5 radius=1.0\n"
    "state 3 density=0.5 energy=9.0 geometry=point xmin=1.0 ymin=1.0\n"
    "max_iters=12.5\n",
    # states after the size keys: the inset still uses the default dx
    "x_cells=50\ny_cells=50\nxmax=10.0\nymax=10.0\nend_step=1\n"
    "state 1 density=100.0 energy=0.0001\nstate 2 density=0.1 energy=25 geometry=rectangle xmin=1 xmax=3 "
    "ymin=2 ymax=4\nuse_jacobi\n",
]

INT_KEYS = ["endstep", "presteps", "maxiters", "coefficient", "ppcginnersteps", "summaryfrequency", "halodepth",
            "xcells", "ycells"]
F_KEYS = ["eps", "dtinit", "endtime", "epslim", "xmin", "ymin", "xmax", "ymax", "dx", "dy"]


@pytest.mark.parametrize("text", DECKS)
def test_host_reader_matches_oracle(text):
    tl = load_package()
    h = tl.Settings.from_text(text)
    o = O.parse_deck(text)
    for k in INT_KEYS + F_KEYS:
        assert getattr(h, k) == getattr(o, k), k
    assert int(h.errorswitch) == o.errorswitch and int(h.checkresult) == o.checkresult
    assert h.solver == o.solver
    assert len(h.states) == o.nstates
    for k, st in enumerate(h.states):
        os = o.states[k]
        for f in ("density", "energy", "xmin", "ymin", "xmax", "ymax", "radius", "geometry", "given", "pdx", "pdy"):
            assert getattr(st, f) == getattr(os, f), (k, f)
        for mode in (0, 1):
            assert st.bounds(h, mode) == O.effective_bounds(o, k, mode)


def test_reader_rejects_malformed_state():
    tl = load_package()
    bad = "state 1 density=1.0 energy\n"
    with pytest.raises(ValueError):
        tl.Settings.from_text(bad)
    with pytest.raises(O.OracleError):
        O.parse_deck(bad)


def test_checkingvalue(tmp_path):
    tl = load_package()
    p = tmp_path / "tea.problems"
    p.write_text("10 10 10 77.4067653961985\n4096 4096 10 1.0\n")
    s = tl.Settings.from_text(CONFIG1)
    from tealeaf_gb300.settings import checkingvalue, qa_passes
    assert checkingvalue(s, str(p)) == 77.4067653961985
    assert qa_passes(77.4067653961985 * (1 + 1e-6), 77.4067653961985)
    assert not qa_passes(77.5, 77.4067653961985)


def _declared_functions():
    hdr = (ROOT / "include" / "tealeaf_gb300.h").read_text()
    body = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(tl_\w+)\s*\(", body, flags=re.M)))


def test_library_exports_every_declared_symbol(built_lib):
    names = _declared_functions()
    assert len(names) >= 20
    lib = C.CDLL(str(built_lib))
    for n in names:
        assert hasattr(lib, n), n
    tl = load_package()
    assert set(names) == set(tl._abi.SIGNATURES), set(names) ^ set(tl._abi.SIGNATURES)


def test_library_loads_through_binding(built_lib):
    tl = load_package()
    lib = tl._abi.load()
    assert lib.tl_last_error(None) == b"null context"
    assert lib.tl_destroy(None) == 0
    ctx = C.c_void_p()
    assert lib.tl_create(C.byref(ctx), None) == 1       # null configuration: rejected before any CUDA call


@pytest.mark.parametrize("v,text", [(1.0, "1.0"), (0.5, "0.5"), (0.1, "0.1"), (100000.0, "100000.0"),
                                    (1e6, "1.0e6"), (1234567.0, "1.234567e6"), (0.0001, "0.0001"),
                                    (1e-5, "1.0e-5"), (2.5e-7, "2.5e-7"), (-3.25, "-3.25"), (123.456, "123.456"),
                                    (0.0, "0.0"), (-0.0, "-0.0"), (1e16, "1.0e16"), (120000.0, "120000.0"),
                                    (0.00012, "0.00012"), (float("nan"), "NaN"), (float("-inf"), "-Inf")])
def test_julia_float_print(tl, v, text):
    """debugrecord writes floats the way Julia's print does (src/TeaLeaf.jl:90-107)."""
    assert tl._julia_repr(v) == text


@pytest.mark.parametrize("text", DECKS)
@pytest.mark.parametrize("mode", [0, 1])
def test_native_deck_reader_matches_host_reader(tl, built_lib, text, mode):
    """tl_parse_deck (the tea.in reader inside the library, no device work)
    against the host reader: every Settings field, the warning count, and
    each state's inset bounds as the given semantics tests them."""
    import warnings as W
    lib = tl._abi.load()
    deck = tl._abi.Deck()
    states = (tl._abi.State * 16)()
    err = C.create_string_buffer(256)
    assert lib.tl_parse_deck(text.encode(), mode, C.byref(deck), states, 16, err, 256) == 0, err.value
    with W.catch_warnings(record=True) as caught:
        W.simplefilter("always")
        s = tl.Settings.from_text(text)
    assert deck.warnings == len(caught)
    for k in INT_KEYS + ["coefficient", "solver"]:
        assert getattr(deck, k) == getattr(s, k), k
    assert bool(deck.errorswitch) == s.errorswitch and bool(deck.checkresult) == s.checkresult
    for k in F_KEYS:
        assert getattr(deck, k) == getattr(s, k), k
    assert deck.nstates == len(s.states)
    for k, st in enumerate(s.states):
        b = st.bounds(s, mode)
        got = states[k]
        assert (got.density, got.energy, got.radius, got.geometry) == (st.density, st.energy, st.radius, st.geometry)
        assert (got.xmin, got.ymin, got.xmax, got.ymax) == b


def test_native_deck_reader_rejects_malformed_state(tl, built_lib):
    lib = tl._abi.load()
    deck = tl._abi.Deck()
    err = C.create_string_buffer(256)
    for bad in ("state 2 density=1.0 energy 3\n", "state 2 density=1.0 geometry=hexagon\n", "state x density=1\n"):
        assert lib.tl_parse_deck(bad.encode(), 1, C.byref(deck), None, 0, err, 256) == tl._abi.ERR_ARG
        assert err.value


def test_c_driver_compiles_against_the_header(built_lib, tmp_path):
    """The header is plain C: a C driver that uses the deck reader, the
    context, tl_diffuse and the summaries compiles and links with gcc."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    lib = Path(built_lib)
    exe = tmp_path / "c_driver"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_driver.c"), "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"],
                   check=True)
    assert exe.exists()


@pytest.mark.parametrize("cfg,code", [((0, 10, 2, 100, 0), 1), ((10, 10, 0, 100, 1), 1), ((10, 10, 2, 0, 1), 1),
                                       ((10, 10, 2, 100, 7), 1), ((10, 12, 2, 100, 0), 5)])
def test_create_rejects_invalid_configurations(tl, built_lib, cfg, code):
    """tl_create validates before touching the device: non-positive sizes,
    halo depth or table length, an unknown mode (TL_ERR_ARG); a non-square
    deck in reference mode raises like Chunk (src/chunk.jl:44)."""
    lib = tl._abi.load()
    nx, ny, hd, maxiters, mode = cfg
    c = tl._abi.Config(nx, ny, hd, maxiters, 0.0, 0.0, 1.0, 1.0, mode)
    ctx = C.c_void_p()
    rc = lib.tl_create(C.byref(ctx), C.byref(c))
    msg = lib.tl_last_error(ctx)
    lib.tl_destroy(ctx)
    assert rc == code and msg


# Fake device addresses: the argument checks of tl_conv3x3_forward run before
# any CUDA call, so nothing here touches a device.
_A = 1 << 20          # 16-byte aligned
_CONV_OK = dict(x=_A, w=_A, b=_A, gz=None, z=None, out=_A, out32=None, N=1, H=8, W=8, cin=32, cout=32, mode=1)


@pytest.mark.parametrize("change", [
    dict(x=None), dict(w=None), dict(out=None, out32=None), dict(mode=3), dict(mode=-1), dict(mode=2, gz=None),
    dict(N=0), dict(H=0), dict(W=0), dict(x=_A + 2), dict(w=_A + 8), dict(out=_A + 4), dict(gz=_A + 1, mode=2),
    dict(z=_A + 8), dict(out32=_A + 2), dict(cin=16, cout=16), dict(cin=8, cout=32), dict(cin=32, cout=64),
])
def test_conv_forward_rejects_invalid_arguments(tl, built_lib, change):
    """tl_conv3x3_forward returns TL_ERR_ARG, before any launch, for null or
    misaligned buffers (activations and weights 16-byte, out32 4-byte), an
    unknown mode, mode 2 without gz, empty images and channel counts outside
    (16, 32), (32, 32), (32, 16)."""
    lib = tl._abi.load()
    a = dict(_CONV_OK, **change)
    rc = lib.tl_conv3x3_forward(a["x"], a["w"], a["b"], a["gz"], a["z"], a["out"], a["out32"], a["N"], a["H"], a["W"],
                                a["cin"], a["cout"], a["mode"], None)
    assert rc == tl._abi.ERR_ARG, change


@pytest.mark.parametrize("change", [dict(x=None), dict(x=_A + 2), dict(dz=_A + 8), dict(partials=_A + 2),
                                    dict(dw=_A + 1), dict(nparts=0), dict(N=0), dict(cin=16, cout=16)])
def test_conv_weight_grad_rejects_invalid_arguments(tl, built_lib, change):
    """tl_conv3x3_weight_grad returns TL_ERR_ARG, before any launch, for null
    or misaligned buffers, no partials, an empty image and unsupported
    channel counts."""
    lib = tl._abi.load()
    a = dict(dict(x=_A, dz=_A, partials=_A, nparts=4, dw=_A, N=1, H=8, W=8, cin=32, cout=32), **change)
    rc = lib.tl_conv3x3_weight_grad(a["x"], a["dz"], a["partials"], a["nparts"], a["dw"], a["N"], a["H"], a["W"],
                                    a["cin"], a["cout"], None)
    assert rc == tl._abi.ERR_ARG, change
