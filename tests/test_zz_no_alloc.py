"""tl_field_summary_noalloc: the field summary for callers that cannot let the
library allocate device memory (a framework that owns every device buffer
through its own pool, or a driver that cannot afford cudaFree's implicit
device synchronisation).  Its reduction scratch is a static device array
instead of context memory; these tests call it through the C ABI on
caller-owned buffers and compare it with tl_field_summary of the same fields,
twice in a row, since every call reuses the same scratch.  The rejection
cases are host-side checks and launch nothing."""
import ctypes as C

import numpy as np
import pytest

from parity_util import random_deck, rel

pytestmark = pytest.mark.gpu
SUMMARY_RTOL = 1e-12          # the tolerance of the other field-summary tests
NAMES = ("volume", "density", "energy", "u")
TL_ERR_ARG = 1


def _fields(tl):
    import torch
    s = tl.Settings.from_text(random_deck(96, 21, steps=1, eps=1e-10), mode=1)
    chunk = tl.initialiseapp(s)
    tl.haloupdate(chunk, s, 1, ["energy", "density"])
    tl.CG.solve(chunk, s, s.dtinit / s.dx ** 2, s.dtinit / s.dy ** 2)
    tl.solvefinished(chunk, s)
    expected = tl.fieldsummary(chunk, s, problemfile=None)
    X, Y = chunk.size()
    pitch = X + 3              # a pitch wider than X
    dev = {}
    for name in NAMES:
        host = np.zeros((Y, pitch))
        host[:, :X] = chunk.field(name).T
        dev[name] = torch.tensor(host, device="cuda")
    return s, chunk, expected, dev, pitch


def _noalloc_layout(chunk, s):
    """The walk the entry point uses: 4 warps, 8 rows, min(tiles, 2 x SMs, 1024) blocks."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    tiles = ((s.xcells + 255) // 256) * ((s.ycells + 7) // 8)
    return 4, 8, min(tiles, 2 * sms, 1024)


def test_noalloc_summary_matches(tl, built_lib):
    import torch
    lib = tl._abi.load()
    s, chunk, expected, dev, pitch = _fields(tl)
    same_tree = chunk.reduction_layout() == _noalloc_layout(chunk, s)
    out = torch.empty(4, dtype=torch.float64, device="cuda")
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out.fill_(float("nan"))
        rc = lib.tl_field_summary_noalloc(*(C.c_void_p(dev[n].data_ptr()) for n in NAMES), s.xcells, s.ycells,
                                          s.halodepth, pitch, C.c_void_p(out.data_ptr()), C.c_void_p(stream),
                                          err, 256)
        assert rc == 0, err.value
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        if same_tree:
            # the same tile walk and reduction tree: the same bits
            assert tuple(got) == tuple(expected), (call, got, expected)
        for a, b in zip(got, expected):
            assert rel(a, b) <= SUMMARY_RTOL, (call, got, expected)


@pytest.mark.parametrize("case,xcells,ycells,hd,pitch,null,msg", [
    ("cells", 1 << 16, 1 << 16, 2, (1 << 16) + 4, False, b"maximum"),
    ("thin_strip_x", (1 << 31) - 1, 1, 2, (1 << 31) + 3, False, b"per dimension"),
    ("thin_strip_y", 1, (1 << 31) - 8, 2, 5, False, b"per dimension"),
    ("halo_depth", 8, 8, 1 << 21, 8 + (1 << 22), False, b"halodepth"),
    ("null_pointer", 8, 8, 2, 12, True, b"null"),
    ("pitch_too_small", 8, 8, 2, 11, False, b"pitch"),
    ("halo_zero", 8, 8, 0, 12, False, b"halo depth"),
])
def test_noalloc_rejects(tl, built_lib, case, xcells, ycells, hd, pitch, null, msg):
    import torch
    lib = tl._abi.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    err = C.create_string_buffer(256)
    arrays = (None if null else p, p, p, p)
    rc = lib.tl_field_summary_noalloc(*arrays, xcells, ycells, hd, pitch, p, None, err, 256)
    assert rc == TL_ERR_ARG, (case, rc)
    assert err.value, case
    assert msg in err.value, (case, err.value)
