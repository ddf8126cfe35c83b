"""The statistics entry point that allocates nothing.

Callers that cannot allocate device memory themselves (their device memory
belongs to another allocator or runtime, or they run in a loop that must not
pay cudaMalloc's implicit synchronisation) call
ludwig_gb_field_stats_noalloc with their own device array; its partial sums
live in a static device array inside the library.  This test allocates the
input itself (through torch) and checks two calls in a row against
stats_field_q, the entry point that uses a library-allocated scratch
buffer, and against numpy's sum, mean, variance, minimum and maximum of the
same values; that the calls leave the device's free memory unchanged; and
that a call on a non-default stream gives the same result.  The file is
named so that pytest collects it last.
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


def _numpy_stats(data):
    """{total, mean, variance, min, max} of each component, in numpy."""
    out = []
    for comp in data.reshape(data.shape[0], -1):
        out += [comp.sum(), comp.mean(), comp.var(), comp.min(), comp.max()]
    return np.array(out)


def _call(fn, dev, nsites, nf, stream=None):
    out = np.zeros(5 * nf)
    rc = fn(ctypes.c_void_p(dev.data_ptr()), nsites, nf,
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), stream)
    return rc, out


@pytest.mark.parametrize("nf", [1, 5])
def test_noalloc_matches_stats_field_q(gb, nf):
    torch = pytest.importorskip("torch")
    L = (24, 20, 16)
    nsites = int(np.prod(L))
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
        rc, out = _call(fn, dev, nsites, nf)
        assert rc == 0, "call %d returned %d: %s" % (
            call, rc, gb.lib().ludwig_gb_last_error())
        np.testing.assert_allclose(out, ref, rtol=RTOL, atol=ATOL)
        np.testing.assert_allclose(out, _numpy_stats(data), rtol=1e-12,
                                   atol=1e-15)
        del dev


def test_noalloc_allocates_nothing_and_honours_the_stream(gb):
    """After the first call on the device (which looks up the static
    array's address), further calls leave the free device memory as it was,
    and a call on a non-default stream returns what the default stream
    does."""
    torch = pytest.importorskip("torch")
    nf, L = 5, (32, 24, 16)
    nsites = int(np.prod(L))
    rng = np.random.default_rng(7)
    data = rng.standard_normal((nf,) + L)
    dev = torch.from_numpy(data.reshape(-1).copy()).to("cuda:0")
    torch.cuda.synchronize()
    fn = _noalloc(gb.lib())
    # First calls: the one on the device looks up the static array's
    # address; the stream's own first use may make the driver set up
    # per-stream resources.  Neither belongs to the calls measured below.
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    rc, first = _call(fn, dev, nsites, nf)
    assert rc == 0
    rc, _ = _call(fn, dev, nsites, nf, ctypes.c_void_p(side.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()

    free0, _ = torch.cuda.mem_get_info(0)
    results = []
    for _ in range(2):
        rc, out = _call(fn, dev, nsites, nf)
        assert rc == 0
        results.append(out)
    rc, on_side = _call(fn, dev, nsites, nf, ctypes.c_void_p(side.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, "free device memory changed by %d bytes" % (
        free0 - free1)

    for out in results + [on_side]:
        np.testing.assert_array_equal(out, first)      # deterministic
    np.testing.assert_allclose(first, _numpy_stats(data), rtol=1e-12,
                               atol=1e-15)


def test_noalloc_rejects_too_many_components(gb):
    fn = _noalloc(gb.lib())
    out = np.zeros(5 * 6)
    rc = fn(ctypes.c_void_p(1), 8, 6,
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    assert rc == 1                  # LUDWIG_GB_EINVAL: beyond the scratch
    msg = gb.lib().ludwig_gb_last_error()
    assert b"ncomp = 6" in msg
