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
