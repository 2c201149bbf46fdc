"""Oracle (test infrastructure only): the Yukawa-screened exchange tables of
HelFEM's range-separated exchange, restated in numpy.

The GPU product is compared against it. Only tests, the smoke check and
the CPU-baseline leg of the benchmark may import it.

Restated (paths inside the HelFEM project):

* ``src/atomic/TwoDBasis.cpp:736-758`` compute_yukawa: the disjoint factors
  int B_a B_b i_L(lambda r) dr and int B_a B_b k_L(lambda r) dr
  (``libhelfemqc/include/CoulombExchangeFE.h:175-217``,
  ``libhelfem/src/RadialBasis.cpp:321-330``) and the pivoted-Cholesky factor
  of the in-element tensor of the kernel i_L(lambda r<) k_L(lambda r>)
  (``RadialBasis.cpp:719-737``, ``quadrature.cpp:163-197``).
* ``src/atomic/TwoDBasis.cpp:1001-1131`` rs_exchange: the bare exchange
  assembly with the multipole factor 4 pi lambda instead of 4 pi/(2L+1).
* ``libhelfem/include/math.h:48-110``: i_L(x) = sqrt(pi/2x) I_{L+1/2}(x),
  k_L(x) = sqrt(2/(pi x)) K_{L+1/2}(x).

The Bessel functions come from SciPy (``spherical_in``, ``spherical_kn``;
SciPy's k_n is sqrt(pi/2x) K, so k_L = (2/pi) k_n), and the quadratures use
higher orders than the product's tabulation, so agreement also checks
convergence. The tables are returned scaled so that the bare exchange
restatement (factor 4 pi/(2L+1)) evaluates the screened one: r_small and the
in-element factor carry (2L+1) lambda and sqrt((2L+1) lambda).
"""
from __future__ import annotations

import math
from dataclasses import replace

import numpy as np
from scipy.special import spherical_in, spherical_kn

from .tabulate import AtomTables, gauss_legendre, pivoted_cholesky


def i_L(x, L):
    return spherical_in(L, x)


def k_L(x, L):
    return (2.0 / math.pi) * spherical_kn(L, x)


def _weighted(rad, f, iel, ngl=160):
    x, w = gauss_legendre(ngl)
    r = rad.coord(x, iel)
    B = rad.B(x, iel)
    wt = w * rad.sf(iel) * f(r)
    return (B * wt[:, None]).T @ B


def _twoe(rad, fin, fout, iel, n_out=160, n_in=64):
    """(ij|kl) = int int B_iB_j(r) B_kB_l(r') fin(r<) fout(r>), pair index
    a + b*Ni (the structure of tabulate.RadialBasis.twoe_integral)."""
    rmin = rad.bval[iel]
    xo, wo = gauss_legendre(n_out)
    xi, wi = gauss_legendre(n_in)
    ro = rad.coord(xo, iel)
    Bo = rad.B(xo, iel)
    half = 0.5 * (ro - rmin)
    rin = rmin + half[:, None] * (xi[None, :] + 1.0)
    xin = (rin - rad.mid(iel)) / rad.sf(iel)
    Bin = rad.B(xin.ravel(), iel).reshape(n_out, n_in, -1)
    win = (half[:, None] * wi[None, :]) * fin(rin)
    G = np.einsum("pq,pqk,pql->pkl", win, Bin, Bin)
    wout = wo * rad.sf(iel) * fout(ro)
    T = np.einsum("p,pi,pj,pkl->ijkl", wout, Bo, Bo, G)
    ni = Bo.shape[1]
    Tm = T.transpose(1, 0, 3, 2).reshape(ni * ni, ni * ni)
    return Tm + Tm.T


def yukawa_tables(A: AtomTables, lam: float, chol_tol: float = 1e-12) -> AtomTables:
    """A copy of A whose rs, rb, chol give the Yukawa-screened exchange when
    fed to the bare exchange restatement (FockOracle(...).exchange)."""
    rad = A.rad
    rs, rb, chol = [], [], []
    for L in range(A.NL):
        s = (2 * L + 1) * lam
        rs.append([s * _weighted(rad, lambda r: i_L(lam * r, L), e) for e in range(rad.nel)])
        rb.append([None if e == 0 else _weighted(rad, lambda r: k_L(lam * r, L), e) for e in range(rad.nel)])
        chol.append([math.sqrt(s) * pivoted_cholesky(_twoe(rad, lambda r: i_L(lam * r, L),
                                                            lambda r: k_L(lam * r, L), e), chol_tol)
                     for e in range(rad.nel)])
    return replace(A, rs=rs, rb=rb, chol=chol)


def hydrogenic_yukawa_self_energy(zeta: float, lam: float) -> float:
    """int int rho(1) rho(2) exp(-lam r12)/r12 for the 1s density
    rho = zeta^3/pi exp(-2 zeta r), from its Fourier transform
    rho^(k) = 16 zeta^4/(4 zeta^2 + k^2)^2:
    (2/pi) int_0^inf rho^(k)^2 k^2/(k^2 + lam^2) dk (the one-dimensional
    integral by adaptive quadrature; lam -> 0 gives 5 zeta/8)."""
    from scipy.integrate import quad
    if lam == 0.0:
        return 5.0 * zeta / 8.0
    a2 = 4.0 * zeta * zeta
    f = lambda k: (16.0 * zeta ** 4 / (a2 + k * k) ** 2) ** 2 * k * k / (k * k + lam * lam)
    val, err = quad(f, 0.0, np.inf, epsabs=1e-16, epsrel=1e-13, limit=400)
    return 2.0 / math.pi * val
