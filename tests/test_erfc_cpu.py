"""The erfc kernel of the range-separated exchange on the host: the
Angyan-Gerber-Marsman expansion against a direct Legendre projection of
erfc(mu r12)/r12, the host pair tables against the numpy restatement, and
the mu -> 0 limit of the exchange against the bare exchange (oracle)."""
import numpy as np
import pytest
from scipy.special import erfc, eval_legendre

import helfem_gb300 as hg
from oracle import FockOracle, gaunt_table
from oracle import erfc as E
from oracle import tabulate as tab


def phi_projected(n, X, x):
    """Legendre coefficient of erfc(r12)/r12 at r1 = X, r2 = x (mu = 1)."""
    t, w = np.polynomial.legendre.leggauss(600)
    r12 = np.sqrt(X * X + x * x - 2 * X * x * t)
    return (2 * n + 1) / 2 * np.sum(w * erfc(r12) / r12 * eval_legendre(n, t))


ARGS = [(0.3, 0.1), (0.45, 0.3), (0.8, 0.35), (1.5, 0.3), (0.7, 0.6), (2.0, 1.2), (3.0, 1.0), (3.0, 0.3)]


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4])
def test_phi_exact_rule_matches_projection(n):
    for X, x in ARGS:
        ref = phi_projected(n, X, x)
        got = E.phi(n, X, x, binomial="exact")
        assert abs(got - ref) <= 1e-9 * abs(ref), (n, X, x, got, ref)


def test_phi_reference_rule_deviation_is_bounded_and_real():
    """The reference's binomial rule for negative arguments changes the
    short-range series: below 1e-5 relative for arguments below 1, but
    visible (above 1e-9) there, and ~1e-3 at mu r> = 5, mu r< = 0.39
    (where the kernel itself is small)."""
    small = max(abs(E.phi(n, X, x) / phi_projected(n, X, x) - 1.0)
                for n in range(4) for X, x in [(0.45, 0.3), (0.8, 0.35), (0.7, 0.6)])
    assert 1e-9 < small < 1e-5, small
    big = abs(E.phi(0, 5.0, 0.39) / phi_projected(0, 5.0, 0.39) - 1.0)
    assert 1e-4 < big < 1e-2, big


def _padded(rad, ktei, iel, kel):
    nn = rad.nnodes
    n2 = nn * nn
    out = np.zeros((n2, n2))
    ei, ek = rad.enabled(iel), rad.enabled(kel)
    Ni = len(ei)
    for kk, pk in enumerate(ek):
        for jj, pj in enumerate(ei):
            for ll, pl in enumerate(ek):
                for ii, pi in enumerate(ei):
                    out[pj + pk * nn, pi + pl * nn] = ktei[kk * Ni + jj, ll * Ni + ii]
    return out


@pytest.mark.parametrize("nn,nel,mu,exact", [(5, 3, 0.7, False), (7, 3, 1.3, False), (5, 3, 0.7, True)])
def test_host_tables_match_oracle(nn, nel, mu, exact):
    b = tab.get_grid(20.0, nel, 4, 2.0)
    lv, mv = hg.angular_basis(1, 0)
    atom = hg.Atom(4, b, lv, mv, nnodes=nn, host_only=True)
    atom.compute_erfc(mu, exact_binomial=exact)
    rad = tab.RadialBasis(nn, b)
    worst = 0.0
    for L in range(3):
        for i in range(nel):
            for k in range(nel):
                ref = E.exchange_order(E.erfc_integral(rad, L, mu, i, k, "exact" if exact else "reference"),
                                       rad.nprim(i), rad.nprim(k))
                got = atom.erfc_table(L, i, k) / mu
                worst = max(worst, np.abs(got - _padded(rad, ref, i, k)).max() / np.abs(ref).max())
    assert worst < 1e-10, worst


def test_erfc_exchange_small_mu_limit():
    """erfc(mu r12)/r12 = 1/r12 - 2 mu / sqrt(pi) + O(mu^2 r12): the erfc
    exchange approaches the bare one linearly in mu (the oracle's own
    tables; the intra-element cusp quadrature leaves a small offset)."""
    b = tab.get_grid(20.0, 3, 4, 2.0)
    A = tab.build_atom(4, 5, b, 1, 0)
    rng = np.random.default_rng(3)
    C = rng.standard_normal((A.nbf, 3))
    P = C @ C.T
    Kb = FockOracle(A).exchange(P)
    G = gaunt_table(2)
    d = {}
    for mu in (1e-3, 2e-3):
        d[mu] = E.rs_exchange_erfc(A, mu, P, G) - Kb
    s = np.abs(Kb).max()
    assert np.abs(d[1e-3]).max() < 1e-2 * s
    # linear in mu: the mu^1 term dominates
    ratio = np.abs(d[2e-3]).max() / np.abs(d[1e-3]).max()
    assert 1.9 < ratio < 2.1, ratio
