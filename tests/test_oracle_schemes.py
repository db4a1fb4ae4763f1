"""The oracle's SBP 1-2, 2-4 and 3-6 operators (setupOperator,
src/StencilOperatorImpl.f90:1164-1585) against the reference's own Python
derivative (golden vectors, tests/golden/sbp_first_derivative_schemes.npz
from make_sbp_golden.py) and the reference's operator property tests:
SBP identity H D + (H D)^T = diag(-1, 0, ..., 0, 1) (test/SBP_property.f90),
exactness on polynomials up to the boundary order
(test/stencil_coefficients.f90), self-adjoint composite dissipation
(test/dissipation_self_adjoint.f90) and the non-composite dissipation's
transpose pair."""
import os

import numpy as np
import pytest

import oracle_lib
from magudi_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "sbp_first_derivative_schemes.npz")
SCHEMES = {capi.SBP_12: ("12", 1), capi.SBP_24: ("24", 2), capi.SBP_36: ("36", 3), capi.SBP_48: ("48", 4)}


def dense(which, n, scheme):
    M = np.zeros((n, n))
    for k in range(n):
        e = np.zeros((1, n))
        e[0, k] = 1.0
        M[:, k] = oracle_lib.apply_operator(which, e, (n, 1, 1), 0, scheme=scheme)[0]
    return M


def norm_diag(n, scheme):
    _, _, _, h = oracle_lib.operator(0, scheme)
    H = np.ones(n)
    H[: len(h)] = h
    H[n - len(h):] = h[::-1]
    return H


@pytest.mark.parametrize("scheme", [capi.SBP_12, capi.SBP_24, capi.SBP_36])
def test_first_derivative_matches_reference_python(scheme):
    g = np.load(GOLDEN)
    tag = SCHEMES[scheme][0]
    for n in (24, 37):
        x, d = g[f"s{tag}_x_{n}"], g[f"s{tag}_dx_{n}"]
        y = oracle_lib.apply_operator(0, x.T.copy(), (n, 1, 1), 0, scheme=scheme)
        assert np.max(np.abs(y - d.T)) <= 1e-14 * max(1.0, np.max(np.abs(d)))


@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_sbp_identity_and_polynomial_exactness(scheme):
    n = 41
    D = dense(0, n, scheme)
    H = np.diag(norm_diag(n, scheme))
    Q = H @ D
    B = np.zeros((n, n))
    B[0, 0], B[-1, -1] = -1.0, 1.0
    assert np.max(np.abs(Q + Q.T - B)) < 10 * np.finfo(float).eps * n
    # boundary order s = interior order / 2 (1 for SBP 1-2): exact on x^k, k <= s
    s = SCHEMES[scheme][1]
    x = np.arange(n, dtype=float)
    for k in range(0, s + 1):
        exact = k * x ** (k - 1) if k > 0 else np.zeros(n)
        assert np.max(np.abs(D @ (x ** k) - exact)) <= 1e-9 * max(1.0, np.max(np.abs(exact)))


@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_adjoint_operator_is_the_h_adjoint(scheme):
    n = 43
    D, A = dense(0, n, scheme), dense(1, n, scheme)
    H = norm_diag(n, scheme)
    assert np.max(np.abs(A - (D.T * H[None, :]) / H[:, None])) < 1e-13


@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_composite_dissipation_is_self_adjoint_and_dissipative(scheme):
    n = 45
    Dc = dense(4, n, scheme)
    H = norm_diag(n, scheme)
    HD = H[:, None] * Dc
    assert np.max(np.abs(HD - HD.T)) < 1e-12 * np.max(np.abs(HD))
    assert np.max(np.linalg.eigvalsh(0.5 * (HD + HD.T))) < 1e-12
    assert np.max(np.abs(Dc @ np.ones(n))) < 1e-12  # constants are not damped


@pytest.mark.parametrize("scheme", [capi.SBP_24, capi.SBP_36, capi.SBP_48])
def test_noncomposite_dissipation_transpose_pair(scheme):
    """The dissipation transpose operator is the transpose of the dissipation
    operator. One exception is restated as the reference defines it: the
    SBP 3-6 transpose's right closure ("SBP 3-6 dissipation transpose",
    src/StencilOperatorImpl.f90:1579-1584) has the opposite sign in the last
    two columns of its last four rows."""
    n = 47
    Dd, Dt = dense(2, n, scheme), dense(3, n, scheme)
    expected = Dd.T.copy()
    if scheme == capi.SBP_36:
        expected[-4:, -2:] *= -1.0
    assert np.max(np.abs(Dt - expected)) < 1e-13
