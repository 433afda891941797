"""The mixed batched solve keeps f and psi as FP32 float pairs (hi, lo)
and forms its outer residual in pair arithmetic.  On the CPU (the oracle
performs the device's operations in the device's order): over right-hand
sides scaled across the range the pairs cover, every problem stops at
relative residual <= 1e-10 measured independently in FP64, and its
solution agrees with the plain FP64 solve far inside the 1e-6 field
tolerance."""
import numpy as np
import pytest

SIZES = [65, 33, 129, 9]


def fp64_relres(sizes, f, psi):
    out, off = [], 0
    for n in sizes:
        F = f[off:off + n * n].reshape(n, n)
        X = psi[off:off + n * n].reshape(n, n)
        h2 = (1.0 / (n - 1)) ** 2
        lap = (X[1:-1, :-2] + X[1:-1, 2:] + X[:-2, 1:-1] + X[2:, 1:-1] - 4 * X[1:-1, 1:-1]) / h2
        out.append(np.linalg.norm(F[1:-1, 1:-1] - lap) / np.linalg.norm(F[1:-1, 1:-1]))
        off += n * n
    return np.array(out)


@pytest.mark.parametrize("scale", [1e-25, 1e-8, 1.0, 1e12, 1e30])
def test_pair_residual_reaches_tolerance_across_magnitudes(oracle, scale):
    rng = np.random.default_rng(7)
    f = np.concatenate([rng.standard_normal(n * n) for n in SIZES]) * scale
    st, psi, cyc, rr = oracle.batch_solve(SIZES, f, precision=1, inner=3)
    assert st == 0 and np.all(rr <= 1e-10)
    assert np.all(fp64_relres(SIZES, f, psi) <= 2e-10)
    st64, psi64, _, _ = oracle.batch_solve(SIZES, f, precision=0)
    assert st64 == 0
    assert np.linalg.norm(psi - psi64) / np.linalg.norm(psi64) <= 1e-9


def test_pair_solution_is_exact_sum_of_halves(oracle):
    """psi comes back as hi + lo in FP64; a pair spans at most 48 bits, so
    every value is a double whose rounding to FP32 is its high half."""
    rng = np.random.default_rng(3)
    f = np.concatenate([rng.standard_normal(n * n) for n in SIZES])
    st, psi, _, _ = oracle.batch_solve(SIZES, f, precision=1, inner=3)
    hi = psi.astype(np.float32).astype(np.float64)
    lo = (psi - hi).astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(hi + lo, psi)


@pytest.mark.parametrize("scale", [1e-25, 1e-8, 1.0, 1e12, 1e30])
def test_f64_outer_and_pair_outer_agree_across_magnitudes(oracle, scale):
    """The FP64-outer defect correction (GB_BATCH_MIXED_F64OUTER) and the
    float-pair one (GB_BATCH_MIXED) both stop at relative residual <= 1e-10,
    checked independently in FP64; their solutions agree with each other and
    with the plain FP64 solve far inside the 1e-6 field tolerance, and their
    final relative residuals are both below the stopping tolerance with the
    FP64-outer one measured against an FP64 residual."""
    rng = np.random.default_rng(11)
    f = np.concatenate([rng.standard_normal(n * n) for n in SIZES]) * scale
    st2, psi2, cyc2, rr2 = oracle.batch_solve(SIZES, f, precision=2, inner=3)
    st1, psi1, cyc1, rr1 = oracle.batch_solve(SIZES, f, precision=1, inner=3)
    st0, psi0, _, _ = oracle.batch_solve(SIZES, f, precision=0)
    assert st2 == st1 == st0 == 0
    assert np.all(rr2 <= 1e-10) and np.all(rr1 <= 1e-10)
    ind2, ind1 = fp64_relres(SIZES, f, psi2), fp64_relres(SIZES, f, psi1)
    assert np.all(ind2 <= 1.0001e-10) and np.all(ind1 <= 2e-10)
    # the FP64-outer relres is the FP64 residual itself, up to the order of
    # the operations (at ~1e-12 the residual is near its FP64 rounding floor)
    np.testing.assert_allclose(rr2, ind2, rtol=1e-3)
    assert np.linalg.norm(psi2 - psi0) / np.linalg.norm(psi0) <= 1e-9
    assert np.linalg.norm(psi2 - psi1) / np.linalg.norm(psi0) <= 1e-9


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_nan_rhs_stops_that_problem_only(oracle, precision):
    """A NaN in one problem's right-hand side stops that problem at its
    first residual with status 2; the other problems solve as they would
    alone."""
    rng = np.random.default_rng(5)
    f = np.concatenate([rng.standard_normal(n * n) for n in SIZES])
    g = f.copy()
    g[SIZES[0] ** 2 + 4 * SIZES[1] + 3] = np.nan        # problem 1
    st, psi, cyc, rr = oracle.batch_solve(SIZES, g, precision=precision, inner=3 if precision else 1)
    st_a, psi_a, cyc_a, _ = oracle.batch_solve(SIZES, f, precision=precision, inner=3 if precision else 1)
    assert st == 2 and st_a == 0
    assert cyc[1] == 0
    off = np.concatenate([[0], np.cumsum(np.array(SIZES) ** 2)])
    for p in (0, 2, 3):
        assert cyc[p] == cyc_a[p]
        np.testing.assert_array_equal(psi[off[p]:off[p + 1]], psi_a[off[p]:off[p + 1]])
