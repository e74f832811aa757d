"""tl_field_summary_noalloc: the field summary for callers that cannot let the
library allocate device memory (a framework that owns every device buffer
through its own pool, or a driver that cannot afford cudaFree's implicit
device synchronisation).  Its reduction scratch is a static device array
instead of context memory; these tests call it through the C ABI on
caller-owned buffers and compare it with tl_field_summary of the same fields,
twice in a row, since every call reuses the same scratch."""
import ctypes as C

import numpy as np
import pytest

from parity_util import random_deck, rel

pytestmark = pytest.mark.gpu
SUMMARY_RTOL = 1e-12          # the tolerance of the other field-summary tests
NAMES = ("volume", "density", "energy", "u")


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
    return s, expected, dev, pitch


def test_noalloc_summary_matches(tl, built_lib):
    import torch
    lib = tl._abi.load()
    s, expected, dev, pitch = _fields(tl)
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
        for a, b in zip(got, expected):
            assert rel(a, b) <= SUMMARY_RTOL, (call, got, expected)


def test_noalloc_rejects_oversize(tl, built_lib):
    import torch
    lib = tl._abi.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    err = C.create_string_buffer(256)
    n = 1 << 16
    rc = lib.tl_field_summary_noalloc(p, p, p, p, n, n, 2, n + 4, p, None, err, 256)
    assert rc == 1
    assert b"maximum" in err.value
