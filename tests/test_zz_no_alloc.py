"""gb_pdma_batch_noalloc, the pentadiagonal batch for callers that cannot
allocate device memory when they call (a Fortran driver with only static
storage and no way to handle an allocation failure mid-step, or a program
whose device memory belongs to its own pool or budget), against the
allocating entry point gb_pdma_batch through the C ABI.

Both run the same per-line elimination, so the results must be identical
(the bit-for-bit bar the other banded-solver tests use), on two calls in a
row that share the fixed scratch array, and a request larger than the
scratch must be refused without a launch.  This file is collected last and
passes alone in a fresh process as well as after the other tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lines(rng, nl, n):
    a, b, d, e, r = (rng.standard_normal((nl, n)) for _ in range(5))
    c = rng.standard_normal((nl, n)) + 8.0
    return [a, b, c, d, e, r]


def _solve(fn, arrs, n, nl):
    import torch
    dv = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in arrs]
    y = torch.full((nl, n), np.nan, dtype=torch.float64, device="cuda")
    st = fn(*[t.data_ptr() for t in dv], y.data_ptr(), n, nl, n, 1, None)
    return st, y.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(gblib):
    from codesthesis_dir_gb300 import lib
    rng = np.random.default_rng(2024)
    # two calls in a row with different shapes: the second reuses the scratch
    # the first left behind
    for n, nl in ((64, 512), (17, 1000)):
        arrs = _lines(rng, nl, n)
        st_ref, ref = _solve(gblib.gb_pdma_batch, arrs, n, nl)
        st_new, got = _solve(gblib.gb_pdma_batch_noalloc, arrs, n, nl)
        assert st_ref == lib.GB_OK and st_new == lib.GB_OK, lib.last_error()
        np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_requests_beyond_its_scratch(gblib):
    from codesthesis_dir_gb300 import lib
    n = 100
    nl = 524288 // (5 * n) + 1          # one line more than the fixed scratch holds
    rng = np.random.default_rng(7)
    st, out = _solve(gblib.gb_pdma_batch_noalloc, _lines(rng, nl, n), n, nl)
    assert st == lib.GB_ERR_INVALID
    assert "exceeds the fixed scratch" in lib.last_error()
    assert np.all(np.isnan(out))        # nothing was launched


def _cudart():
    """The CUDA runtime as a shared library (the toolkit's, else none): the
    default memory pool it reports is the device's own, shared with the
    library's statically linked runtime."""
    import ctypes
    import ctypes.util
    for name in (ctypes.util.find_library("cudart"), "/usr/local/cuda/lib64/libcudart.so",
                 "libcudart.so.13", "libcudart.so"):
        if not name:
            continue
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    return None


def test_noalloc_draws_nothing_from_the_device_memory_pool(gblib):
    """The defining property: a call takes no memory from the device's
    stream-ordered pool (which gb_pdma_batch's scratch comes from).  The
    pool's high-water mark is reset before each call and read after it: the
    allocating entry point raises it, the no-allocation one leaves it and
    the pool's reserved memory untouched."""
    import ctypes as C
    import torch
    rt = _cudart()
    if rt is None:
        pytest.skip("no shared CUDA runtime library to read the memory pool from")
    dev = torch.cuda.current_device()
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    USED_HIGH, RESERVED_CUR = 0x8, 0x5

    def attr(a):
        v = C.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, a, C.byref(v)) == 0
        return v.value

    def reset_high():
        z = C.c_uint64(0)
        assert rt.cudaMemPoolSetAttribute(pool, USED_HIGH, C.byref(z)) == 0

    from codesthesis_dir_gb300 import lib
    rng = np.random.default_rng(99)
    n, nl = 64, 512
    arrs = _lines(rng, nl, n)
    torch.cuda.synchronize()
    reset_high()
    st, _ = _solve(gblib.gb_pdma_batch, arrs, n, nl)
    assert st == lib.GB_OK
    assert attr(USED_HIGH) >= 5 * n * nl * 8          # the control: its scratch came from the pool
    torch.cuda.synchronize()
    reserved = attr(RESERVED_CUR)
    reset_high()
    st, _ = _solve(gblib.gb_pdma_batch_noalloc, arrs, n, nl)
    assert st == lib.GB_OK
    assert attr(USED_HIGH) == 0
    assert attr(RESERVED_CUR) == reserved
