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
