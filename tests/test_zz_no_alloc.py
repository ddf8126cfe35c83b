"""The statistics entry point that allocates nothing.

Callers that cannot allocate device memory themselves (their device memory
belongs to another allocator or runtime, or they run in a loop that must not
pay cudaMalloc's implicit synchronisation) call
ludwig_gb_field_stats_noalloc with their own device array; its partial sums
live in a static device array inside the library.  This test allocates the
input itself (through torch) and checks two calls in a row against
stats_field_q, the entry point that uses a library-allocated scratch
buffer.  The file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-13, 1e-19          # as the other statistics tests


def _noalloc(lib):
    fn = lib.ludwig_gb_field_stats_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("nf", [1, 5])
def test_noalloc_matches_stats_field_q(gb, nf):
    torch = pytest.importorskip("torch")
    L = (24, 20, 16)
    rng = np.random.default_rng(99 + nf)
    pe = gb.PE(0)
    cs = gb.Coords(pe, L)
    field = gb.Field(cs, nf=nf, name="q")
    fn = _noalloc(gb.lib())

    for call in range(2):
        data = rng.uniform(-1.0, 1.0, (nf,) + L)
        field.set(data)
        ref = np.array([field.stats(n) for n in range(nf)]).reshape(-1)

        dev = torch.from_numpy(data.reshape(-1).copy()).to("cuda:0")
        torch.cuda.synchronize()
        out = np.zeros(5 * nf)
        rc = fn(ctypes.c_void_p(dev.data_ptr()), int(np.prod(L)), nf,
                out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
        assert rc == 0, "call %d returned %d" % (call, rc)
        np.testing.assert_allclose(out, ref, rtol=RTOL, atol=ATOL)
        del dev


def test_noalloc_rejects_too_many_components(gb):
    fn = _noalloc(gb.lib())
    out = np.zeros(5 * 6)
    rc = fn(ctypes.c_void_p(1), 8, 6,
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    assert rc == 1                  # LUDWIG_GB_EINVAL: beyond the scratch
