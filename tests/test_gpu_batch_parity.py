"""Batched Poisson solve on the device against the oracle.

The smoothing, residual and transfer kernels round exactly as the oracle's
loops; only the order of the residual-norm sums differs, so the solutions
agree bit for bit whenever the V-cycle counts agree (they do for these
seeds), and the relative residuals to ~1e-15."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def grf(rng, n, corr=0.05):
    """Seeded zero-mean, unit-variance Gaussian random field on an n x n grid
    with squared-exponential correlation length corr (FFT filtering of white
    noise); boundary values zeroed."""
    w = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n, d=1.0 / (n - 1))
    kx, ky = np.meshgrid(k, k, indexing="ij")
    filt = np.exp(-((2 * np.pi) ** 2) * (kx ** 2 + ky ** 2) * corr ** 2 / 4.0)
    g = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    g = (g - g.mean()) / g.std()
    g[0, :] = g[-1, :] = g[:, 0] = g[:, -1] = 0.0
    return g


def make_batch(sizes, seed):
    rng = np.random.default_rng(seed)
    return np.concatenate([-grf(rng, n).ravel() for n in sizes])


def independent_relres(sizes, f, psi):
    out, off = [], 0
    for n in sizes:
        F = f[off:off + n * n].reshape(n, n)
        X = psi[off:off + n * n].reshape(n, n)
        h2 = (1.0 / (n - 1)) ** 2
        lap = (X[1:-1, :-2] + X[1:-1, 2:] + X[:-2, 1:-1] + X[2:, 1:-1] - 4 * X[1:-1, 1:-1]) / h2
        r = F[1:-1, 1:-1] - lap
        fn = np.linalg.norm(F[1:-1, 1:-1])
        out.append(np.linalg.norm(r) / fn if fn > 0 else 0.0)
        off += n * n
    return np.array(out)


SMALL = [3, 5, 9, 17, 33, 65, 129, 257, 65, 129, 3, 33, 513]


@pytest.mark.parametrize("exec_mode", [0, 1], ids=["graph", "persistent"])
@pytest.mark.parametrize("precision,inner", [(0, 1), (1, 1), (1, 2), (1, 3), (2, 1), (2, 3), (2, 4)],
                         ids=["fp64", "mixed", "mixed-inner2", "mixed-inner3", "f64outer", "f64outer-inner3",
                              "f64outer-inner4"])
def test_batch_matches_oracle(oracle, gblib, precision, inner, exec_mode):
    from codesthesis_dir_gb300.batch import BatchPoisson
    f = make_batch(SMALL, 7)
    st_o, psi_o, cyc_o, rr_o = oracle.batch_solve(SMALL, f, precision=precision, inner=inner)
    bp = BatchPoisson(SMALL, precision=precision, inner=inner, exec_mode=exec_mode)
    st, psi, cyc, rr = bp.solve_host(f)
    assert st == 0 and st_o == 0
    np.testing.assert_array_equal(cyc, cyc_o)
    np.testing.assert_array_equal(psi, psi_o)
    np.testing.assert_allclose(rr, rr_o, rtol=1e-9, atol=1e-25)
    assert np.all(rr <= 1e-10)
    assert np.all(independent_relres(SMALL, f, psi) <= 2e-10)


def test_batch_fp64_vs_mixed(gblib):
    """The mixed path reaches the same 1e-10 relative residual and the same
    solution to well within the 1e-6 field tolerance."""
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = [513, 257, 129, 65, 257, 513]
    f = make_batch(sizes, 11)
    _, p64, c64, r64 = BatchPoisson(sizes, precision=0).solve_host(f)
    for prec in (1, 2):
        _, pmx, cmx, rmx = BatchPoisson(sizes, precision=prec, inner=3).solve_host(f)
        assert np.all(r64 <= 1e-10) and np.all(rmx <= 1e-10)
        assert np.linalg.norm(pmx - p64) / np.linalg.norm(p64) <= 1e-9


def test_batch_edge_cases(oracle, gblib):
    """A zero right-hand side converges in zero cycles; a single-point grid
    is solved exactly; repeated solves on one handle give identical results."""
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = [33, 3, 65]
    f = make_batch(sizes, 5)
    f[: 33 * 33] = 0.0
    bp = BatchPoisson(sizes, precision=0)
    st1, psi1, cyc1, rr1 = bp.solve_host(f)
    st2, psi2, cyc2, rr2 = bp.solve_host(f)
    assert st1 == 0 and cyc1[0] == 0 and np.all(psi1[: 33 * 33] == 0)
    assert cyc1[1] == 1
    np.testing.assert_array_equal(psi1, psi2)
    np.testing.assert_array_equal(cyc1, cyc2)


@pytest.mark.parametrize("exec_mode", [0, 1], ids=["graph", "persistent"])
def test_batch_max_cycles_status(gblib, exec_mode):
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = [129, 65]
    f = make_batch(sizes, 2)
    st, psi, cyc, rr = BatchPoisson(sizes, precision=0, max_cycles=2, rtol=1e-14, exec_mode=exec_mode).solve_host(f)
    assert st == 1 and np.all(cyc == 2)


def test_graph_and_persistent_agree_on_workload_sizes(gblib):
    """The two execution modes run the same operations: identical results on
    a batch with every size of the benchmark workload."""
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = [513, 65, 257, 129, 513, 129, 65, 257, 3, 17]
    f = make_batch(sizes, 21)
    for prec in (1, 2):
        out = []
        for mode in (0, 1):
            st, psi, cyc, rr = BatchPoisson(sizes, precision=prec, inner=3, exec_mode=mode).solve_host(f)
            assert st == 0
            out.append((psi, cyc))
        np.testing.assert_array_equal(out[0][0], out[1][0])
        np.testing.assert_array_equal(out[0][1], out[1][1])


def test_integer_conversions_match_hardware(gblib):
    """The mixed solve converts the defect to FP32 and the correction back
    to FP64 with integer operations; over every float bit pattern and 2^26
    seeded double patterns (ties, denormals, overflow, NaN and infinity
    included) they equal the hardware conversions."""
    import ctypes as C
    f2d, d2f = C.c_longlong(-1), C.c_longlong(-1)
    assert gblib.gb_check_conversions(1 << 26, 20261203, C.byref(f2d), C.byref(d2f)) == 0
    assert (f2d.value, d2f.value) == (0, 0)


@pytest.mark.parametrize("precision", [0, 1, 2], ids=["fp64", "mixed", "f64outer"])
def test_pipelined_stream_matches_single_calls(gblib, precision):
    """A stream of different right-hand sides through the pipelined calls
    (upload of call k and download of call k-1 overlapping the solves) gives
    each call exactly what a lone host-buffer solve gives, including a
    maximum-cycle failure in the middle of the stream; the handle solves
    plainly again after the drain."""
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = [257, 65, 129, 513, 33]
    fs = [make_batch(sizes, 40 + i) for i in range(5)]
    fs[2] = fs[2] * 1e30          # large magnitudes (still inside the FP32 range in the inner cycles)
    bp = BatchPoisson(sizes, precision=precision)
    ref = [bp.solve_host(f) for f in fs]
    got = bp.solve_stream(fs)
    assert len(got) == len(fs)
    for (st, psi, cyc, rr), (st0, psi0, cyc0, rr0) in zip(got, ref):
        assert st == st0 == 0
        np.testing.assert_array_equal(psi, psi0)
        np.testing.assert_array_equal(cyc, cyc0)
        np.testing.assert_array_equal(rr, rr0)
    assert gblib.gb_batch_drain(bp._h) == 0          # nothing pending
    st, psi, cyc, rr = bp.solve_host(fs[0])
    np.testing.assert_array_equal(psi, ref[0][1])
    short = BatchPoisson(sizes, precision=precision, max_cycles=2, rtol=1e-14)
    res = short.solve_stream(fs[:3])
    assert [r[0] for r in res] == [1, 1, 1] and all(np.all(r[2] == 2) for r in res)
