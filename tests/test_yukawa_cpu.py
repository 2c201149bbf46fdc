"""Range-separated (Yukawa-screened) exchange, CPU side: the oracle against
an analytic known answer, and the product's host tabulation against the
oracle's.

Known answer: for the hydrogen 1s orbital (computed in the FE basis, energy
-0.5 to 1e-12) the screened exchange energy tr(P K) of its one-electron
density equals -int int rho rho exp(-lambda r12)/r12, which the Fourier
transform of rho reduces to a one-dimensional integral (5/8 at lambda = 0).
This pins the normalisation of the screened kernel (the factor 4 pi lambda
and the Bessel functions i_L, k_L) independently of the reference's code."""
import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import FockOracle
from oracle import tabulate as tab
from oracle.yukawa import hydrogenic_yukawa_self_energy, yukawa_tables


def hydrogen_1s():
    b = tab.get_grid(40.0, 12, 4, 2.0)
    A = tab.build_atom(1, 15, b, 0, 0)
    X = tab.invh(A.S)
    e, U = np.linalg.eigh(X.T @ (A.T + A.V) @ X)
    c = X @ U[:, 0]
    return A, b, e[0], np.outer(c, c)


@pytest.mark.parametrize("lam", [1e-3, 0.3, 1.0, 2.5])
def test_oracle_matches_analytic_hydrogen(lam):
    A, _, e1s, P = hydrogen_1s()
    assert abs(e1s + 0.5) < 1e-12
    Ex = float(np.sum(P * FockOracle(yukawa_tables(A, lam)).exchange(P)))
    assert abs(Ex + hydrogenic_yukawa_self_energy(1.0, lam)) < 1e-11, (Ex, lam)


def test_small_lambda_limit_is_bare_exchange():
    """exp(-lambda r12)/r12 = 1/r12 - lambda + O(lambda^2): K(lambda) - K(0)
    is linear in lambda for small lambda."""
    b = tab.get_grid(40.0, 6, 4, 2.0)
    A = tab.build_atom(8, 15, b, 1, 1)
    rng = np.random.default_rng(3)
    C = rng.standard_normal((A.nbf, 4))
    P = C @ C.T * 1e-2
    K0 = FockOracle(A).exchange(P)
    # second order relative to first ~ lambda r / 2 over a basis reaching 40 bohr
    d1 = FockOracle(yukawa_tables(A, 1e-5)).exchange(P) - K0
    d2 = FockOracle(yukawa_tables(A, 2e-5)).exchange(P) - K0
    assert np.abs(d2 - 2 * d1).max() < 1e-3 * np.abs(d1).max()


def test_host_tabulation_matches_oracle():
    """The product's screened disjoint factors against the oracle's
    (independent Bessel functions and quadrature orders)."""
    b = tab.get_grid(40.0, 5, 4, 2.0)
    A = tab.build_atom(10, 15, b, 2, 0)
    a = hg.Atom(10, b, *hg.angular_basis(2, 0), host_only=True)
    for lam in (0.2, 1.5):
        a.compute_yukawa(lam)
        Y = yukawa_tables(A, lam)
        for L in range(A.NL):
            for e in range(A.rad.nel):
                rs, rb, tk = a.yukawa_tables(L, e)
                p0 = 1 if e == 0 else 0
                n = A.rs[L][e].shape[0]
                ref = Y.rs[L][e]
                got = rs[p0:p0 + n, p0:p0 + n]
                assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), (lam, L, e)
                if e > 0:
                    refb = Y.rb[L][e]
                    gotb = rb[:n, :n]
                    assert np.abs(gotb - refb).max() <= 1e-12 * np.abs(refb).max(), (lam, L, e)
                # in-element tensor: the exchange-ordered table against chol chol^T
                ch = Y.chol[L][e]
                T = ch @ ch.T  # (ab|cd) with pair index a + b*n
                nn = a.nnodes
                idx = np.arange(n) + p0
                # tk[(a + c nn), (b + d nn)] = (ab|cd)
                got4 = tk.reshape(nn, nn, nn, nn, order="F")[np.ix_(idx, idx, idx, idx)]  # [a, c, b, d]
                ref4 = T.reshape(n, n, n, n, order="F").transpose(0, 2, 1, 3)      # [a, c, b, d]
                assert np.abs(got4 - ref4).max() <= 1e-11 * np.abs(ref4).max(), (lam, L, e)


def test_rs_exchange_requires_tables():
    a = hg.Atom(2, tab.get_grid(40.0, 3, 4, 2.0), *hg.angular_basis(0, 0), host_only=True)
    with pytest.raises(RuntimeError):
        a.yukawa_tables(0, 0)
