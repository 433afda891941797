"""Batched banded solvers (gb_tdma_batch / gb_ptdma_batch / gb_pdma_batch)
against the oracle's restatement of tdma/ptdma/pdma, bit for bit, on
randomly perturbed diagonally dominant lines of varying length."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("kind", ["tdma", "ptdma", "pdma"])
@pytest.mark.parametrize("n", [3, 4, 17, 129])
def test_banded_batch(oracle, gblib, kind, n):
    import torch
    rng = np.random.default_rng(n)
    nl = 37
    a, b, c, d, e, r = (rng.standard_normal((nl, n)) for _ in range(6))
    b += 6.0 if kind != "pdma" else 0.0
    c += 8.0 if kind == "pdma" else 0.0
    arrs = [a, b, c] + ([d, e] if kind == "pdma" else []) + [r]
    dv = [_dev(x) for x in arrs]
    y = torch.zeros((nl, n), dtype=torch.float64, device="cuda")
    fn = getattr(gblib, "gb_%s_batch" % kind)
    st = fn(*[t.data_ptr() for t in dv], y.data_ptr(), n, nl, n, 1, None)
    assert st == 0
    got = y.cpu().numpy()
    for l in range(nl):
        if kind == "tdma":
            ref = oracle.tdma(a[l], b[l], c[l], r[l])
        elif kind == "ptdma":
            ref = oracle.ptdma(a[l], b[l], c[l], r[l])
        else:
            ref = oracle.pdma(a[l], b[l], c[l], d[l], e[l], r[l])
        np.testing.assert_array_equal(got[l], ref)
    # inputs preserved
    for t, x in zip(dv, arrs):
        np.testing.assert_array_equal(t.cpu().numpy(), x)
