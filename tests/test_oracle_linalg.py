"""The oracle's restated LAPACK solves against scipy's LAPACK, and the Differentiate1D
stencils (SolidSolver.f90:1085-1233) against polynomials they differentiate exactly."""
import ctypes as C

import numpy as np
import pytest

scipy_lapack = pytest.importorskip("scipy.linalg.lapack")

dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731


def test_tridiagonal_matches_scipy_dgttrf_dgttrs(oracle):
    L = oracle.lib()
    rng = np.random.default_rng(7)
    for n in (8, 17, 64):
        dl, d, du = rng.standard_normal(n - 1), rng.standard_normal(n), rng.standard_normal(n - 1)
        d[::3] *= 0.05  # force row interchanges
        b = rng.standard_normal(n)
        x = b.copy()
        assert L.orc_gttrf_solve(n, dp(dl.copy()), dp(d.copy()), dp(du.copy()), dp(x)) == 0
        dl2, d2, du2, du22, ipiv, info = scipy_lapack.dgttrf(dl, d, du)
        xs, info2 = scipy_lapack.dgttrs(dl2, d2, du2, du22, ipiv, b)
        assert info == 0 and info2 == 0
        assert np.abs(x - xs).max() <= 1e-13 * np.abs(xs).max()


def test_dense_lu_matches_scipy_dgetrf_dgetrs(oracle):
    L = oracle.lib()
    rng = np.random.default_rng(8)
    for n in (10, 36, 132):
        A = rng.standard_normal((n, n))
        b = rng.standard_normal(n)
        x = b.copy()
        assert L.orc_getrf_solve(n, dp(np.ascontiguousarray(A)), dp(x)) == 0
        lu, piv, info = scipy_lapack.dgetrf(A)
        xs, info2 = scipy_lapack.dgetrs(lu, piv, b)
        assert np.abs(x - xs).max() <= 1e-11 * np.abs(xs).max()


def test_singular_matrix_is_reported(oracle):
    L = oracle.lib()
    A = np.zeros((4, 4))
    b = np.ones(4)
    assert L.orc_getrf_solve(4, dp(A), dp(b)) == 1


@pytest.mark.parametrize("order,deg", [(1, 2), (2, 3), (3, 3), (4, 4)])
def test_differentiate1d_is_exact_on_low_degree_polynomials(oracle, order, deg):
    L = oracle.lib()
    n, dx = 24, 0.1
    s = np.arange(n) * dx
    f = sum(((k + 1.0) * 0.3) * s ** k for k in range(deg + 1))
    coef = [((k + 1.0) * 0.3) for k in range(deg + 1)]
    dpoly = np.polynomial.polynomial.polyder(coef, order)
    exact = np.polynomial.polynomial.polyval(s, dpoly)
    out = np.zeros(n)
    L.orc_differentiate1d(dp(f), dp(out), n, dx, order)
    assert np.abs(out - exact).max() < 1e-7 * max(1.0, np.abs(exact).max())
