"""Oracle (test infrastructure only): HelFEM's range-separated exchange with
the erfc kernel, restated in numpy.

The GPU product is compared against it. Only tests, the smoke check and the
CPU-baseline leg of the benchmark may import it.

Restated (paths inside the HelFEM project):

* ``libhelfem/src/erfc_expn.cpp``: the Angyan-Gerber-Marsman expansion
  (J. Phys. A 39, 8613 (2006)) of erfc(mu r12)/r12 in Legendre polynomials,
  mu Phi_L(mu r>, mu r<) per multipole L: the general form (their eqs. 21,
  22, 24) and the short-range Taylor series (eqs. 28-30), chosen as the
  reference chooses (series when xi < 0.4 or Xi < 0.5).
* ``libhelfem/src/RadialBasis.cpp:742-811`` erfc_integral and
  ``libhelfem/src/quadrature.cpp:203-249``: the pair tables
  (ij|kl) = int int B_iB_j(r) mu Phi_L B_kB_l(r') on the modified
  Gauss-Chebyshev rule of the radial basis, the inner element split into as
  many sub-intervals as points when both functions share the element, the
  result symmetrised there.
* ``libhelfemqc/include/CoulombExchangeFE.h:275-295`` compute_erfc_ktei and
  ``libhelfem/src/utils.cpp:54-80`` exchange_tei: the exchange ordering
  (ij|kl) -> [(j,k), (i,l)] of every element pair.
* ``src/atomic/TwoDBasis.cpp:1001-1131`` rs_exchange and
  ``CoulombExchangeFE.h:396-422``: the Gaunt recoupling with the factor
  4 pi mu / (2L+1) and the pairwise assembly.

The reference's short-range series uses a binomial coefficient for negative
upper arguments that is not the generalised binomial (its recursion
C(n, m) = (-1)^m C(n+m-1, m) for n < -1); ``binomial="reference"`` keeps
that rule (parity), ``binomial="exact"`` uses n(n-1)...(n-m+1)/m!. Against
a direct Legendre projection of erfc(mu r12)/r12 the exact rule agrees to
~1e-12 relative and the reference rule deviates by up to ~1.5e-6 for
arguments below 1 and by ~1e-3 at Xi = 5-6 with xi near 0.4, where the
kernel itself is small (tests).
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erfc

from .tabulate import chebyshev


def _dfact(n: int) -> float:
    v = 1.0
    while n >= 2:
        v *= n
        n -= 2
    return v


def binomial_reference(n: int, m: int) -> float:
    """The reference's choose(n, m) (erfc_expn.cpp), negative n included."""
    if n == -1:
        return (-1.0) ** m
    if n == 0:
        return 1.0 if m == 0 else 0.0
    if m == 0:
        return 1.0
    if m == 1:
        return float(n)
    if n > 0 and m > n:
        return 0.0
    if n < 0:
        return binomial_reference(n + m - 1, m) * (-1.0) ** m
    v = 1.0
    for i in range(min(m, n - m)):
        v *= (n - i) / (i + 1)
    return v


def binomial_exact(n: int, m: int) -> float:
    v = 1.0
    for i in range(m):
        v *= (n - i) / (i + 1)
    return v


def _Fn(n, X, x):
    """AGM eq. 22 (summed from p = 0, as the reference does)."""
    ep = np.exp(-(X + x) ** 2)
    em = np.exp(-(X - x) ** 2)
    pre = -1.0 / (4.0 * X * x)
    F = np.zeros_like(X)
    for p in range(n + 1):
        c = math.factorial(n + p) / (math.factorial(p) * math.factorial(n - p))
        F = F + pre ** (p + 1) * c * ((-1.0) ** (n - p) * ep - em)
    return 2.0 / math.sqrt(math.pi) * F


def _Hn(n, X, x):
    """AGM eq. 24 (X >= x)."""
    a = X ** (2 * n + 1)
    b = x ** (2 * n + 1)
    return ((a + b) * erfc(X + x) - (a - b) * erfc(X - x)) / (2.0 * (x * X) ** (n + 1))


def phi_general(n, X, x):
    """AGM eq. 21, X >= x > 0."""
    s = _Fn(n, X, x) + _Hn(n, X, x)
    for m in range(1, n + 1):
        s = s + _Fn(n - m, X, x) * ((X ** m) ** 2 + (x ** m) ** 2) / (X ** m * x ** m)
    return s


def _Dnk(n, k, X, binom):
    """AGM eqs. 28, 29."""
    pre = np.exp(-X * X) / math.sqrt(math.pi) * 2.0 ** (n + 1) * X ** (2 * n + 1)
    if k == 0:
        s = sum(1.0 / (_dfact(2 * (n - m) + 1) * (2.0 * X * X) ** m) for m in range(1, n + 1))
        return erfc(X) + pre * s
    s = sum(binom(m - k - 1, m - 1) * (2.0 * X * X) ** (k - m) / _dfact(2 * (n + k - m) + 1)
            for m in range(1, k + 1))
    return pre * (2 * n + 1) / (math.factorial(k) * (2 * n + 2 * k + 1)) * s


def phi_short(n, X, x, binom=binomial_reference):
    """AGM eq. 30, the series in x to FP64 precision (X >= x, X > 0)."""
    X = float(X)
    x = float(x)
    if x == 0.0 and n > 0:
        return 0.0
    if n == 0 and x == 0.0 and X == 0.0:
        return 1.0
    P = 0.0
    for k in range(0, 201, 2):
        d = _Dnk(n, k, X, binom) * x ** (n + 2 * k) + _Dnk(n, k + 1, X, binom) * x ** (n + 2 * (k + 1))
        P += d
        if abs(d) < np.finfo(float).eps * max(abs(P), 1.0):
            return P / X ** (n + 1)
    raise RuntimeError(f"phi_short did not converge: n={n} X={X} x={x}")


def phi(n, X, x, binomial="reference"):
    """Phi_n(X, x) for scalar arguments, the reference's choice of form."""
    if X < x:
        X, x = x, X
    binom = binomial_reference if binomial == "reference" else binomial_exact
    if x < 0.4 or X < 0.5:
        return phi_short(n, X, x, binom)
    return float(phi_general(n, np.float64(X), np.float64(x)))


def phi_array(n, A, B, binomial="reference"):
    """Phi_n elementwise over arrays of arguments (either order): the
    series where the reference takes it, each element summed until its own
    increment falls below eps of max(|sum|, 1), the general form elsewhere."""
    A = np.asarray(A, float)
    B = np.asarray(B, float)
    X = np.maximum(A, B)
    x = np.minimum(A, B)
    out = np.empty(X.shape)
    short = (x < 0.4) | (X < 0.5)
    gen = ~short
    if gen.any():
        out[gen] = phi_general(n, X[gen], x[gen])
    if short.any():
        binom = binomial_reference if binomial == "reference" else binomial_exact
        Xs, xs = X[short], x[short]
        res = np.zeros(Xs.shape)
        zero = (xs == 0.0)
        work = ~zero
        P = np.zeros(Xs.shape)
        done = np.zeros(Xs.shape, bool)
        done[zero] = True
        for k in range(0, 201, 2):
            idx = np.nonzero(~done)[0]
            if idx.size == 0:
                break
            Xi, xi = Xs[idx], xs[idx]
            d = _Dnk(n, k, Xi, binom) * xi ** (n + 2 * k) + _Dnk(n, k + 1, Xi, binom) * xi ** (n + 2 * (k + 1))
            P[idx] += d
            conv = np.abs(d) < np.finfo(float).eps * np.maximum(np.abs(P[idx]), 1.0)
            done[idx[conv]] = True
        if not done.all():
            raise RuntimeError("phi_array: series did not converge")
        res[work] = P[work] / Xs[work] ** (n + 1)
        res[zero] = 1.0 if n == 0 else 0.0
        # (n = 0, x = 0, X > 0: the series is D_00(X) / X)
        z0 = zero & (Xs > 0.0)
        if n == 0 and z0.any():
            res[z0] = _Dnk(0, 0, Xs[z0], binom) / Xs[z0]
        out[short] = res
    return out


def _pairprod(B, w):
    """bfprod with column fi*N + fj, weighted by w (quadrature.cpp make_bfprod)."""
    n = B.shape[1]
    P = (B[:, :, None] * B[:, None, :]).reshape(B.shape[0], n * n)
    return P * w[:, None]


def erfc_integral(rad, L: int, mu: float, iel: int, kel: int, binomial="reference"):
    """(ij|kl) of the erfc kernel for multipole L, i,j in element iel and
    k,l in element kel: Ni^2 x Nk^2."""
    nq = rad.nquad
    xq, wq = chebyshev(nq)
    nint = nq if iel == kel else 1
    xk = np.concatenate([(ii * 2.0 / nint - 1.0 + (ii + 1) * 2.0 / nint - 1.0) / 2.0 + xq * (1.0 / nint)
                         for ii in range(nint)])
    wk = np.concatenate([wq * (1.0 / nint) for _ in range(nint)])
    ri = rad.coord(xq, iel)
    rk = rad.coord(xk, kel)
    Fn = phi_array(L, mu * ri[:, None] * np.ones((1, len(rk))), mu * rk[None, :] * np.ones((len(ri), 1)), binomial)
    Bi = _pairprod(rad.B(xq, iel), wq * rad.sf(iel))
    Bk = _pairprod(rad.B(xk, kel), wk * rad.sf(kel))
    tei = Bi.T @ Fn @ Bk
    if iel == kel:
        tei = 0.5 * (tei + tei.T)
    return tei


def exchange_order(tei, ni: int, nk: int):
    """(ij|kl) with pair indices j*Ni + i and l*Nk + k -> ktei[(k*Ni + j),
    (l*Ni + i)] (utils.cpp exchange_tei with Ni = Nj, Nk = Nl)."""
    T = tei.reshape(ni, ni, nk, nk)  # [j, i, l, k] from rows jj*Ni+ii, cols ll*Nk+kk
    K = np.transpose(T, (3, 0, 2, 1))  # [k, j, l, i]
    return K.reshape(nk * ni, nk * ni)


def erfc_ktei(rad, NL: int, mu: float, binomial="reference"):
    """ktei[L][iel][jel], exchange-ordered."""
    nel = rad.nel
    out = [[[None] * nel for _ in range(nel)] for _ in range(NL)]
    for L in range(NL):
        for i in range(nel):
            for j in range(nel):
                out[L][i][j] = exchange_order(erfc_integral(rad, L, mu, i, j, binomial),
                                              rad.nprim(i), rad.nprim(j))
    return out


def rs_exchange_erfc(A, mu: float, P: np.ndarray, gaunt_table, ktei=None, binomial="reference"):
    """K of the erfc kernel (signed as the reference's rs_exchange: the
    matrix added to the Fock matrix), dense P of the atom A (AtomTables)."""
    rad = A.rad
    nrad, nang, nel, NL = A.nrad, A.nang, rad.nel, A.NL
    if ktei is None:
        ktei = erfc_ktei(rad, NL, mu, binomial)
    g = (gaunt_table.shape[1] - 1) // 2
    lv, mv = A.lval, A.mval
    K = np.zeros((nrad * nang, nrad * nang))
    thr = 10.0 * np.finfo(float).eps
    for ja in range(nang):
        for ka in range(nang):
            R = [np.zeros((nrad, nrad)) for _ in range(NL)]
            used = [False] * NL
            for ia in range(nang):
                for la in range(nang):
                    M, Mp = mv[ja] - mv[ia], mv[ka] - mv[la]
                    if M != Mp:
                        continue
                    blk = P[ia * nrad:(ia + 1) * nrad, la * nrad:(la + 1) * nrad]
                    if np.linalg.norm(blk) < thr:
                        continue
                    Lmin = max(abs(lv[ia] - lv[ja]), abs(lv[ka] - lv[la]), abs(M))
                    Lmax = min(lv[ia] + lv[ja], lv[ka] + lv[la])
                    for L in range(Lmin, Lmax + 1):
                        c = (gaunt_table[lv[ja], mv[ja] + g, L, M + g, lv[ia]] *
                             gaunt_table[lv[ka], mv[ka] + g, L, M + g, lv[la]])
                        if c == 0.0:
                            continue
                        R[L] += (4.0 * math.pi * mu / (2 * L + 1) * c) * blk
                        used[L] = True
            Kb = np.zeros((nrad, nrad))
            for L in range(NL):
                if not used[L]:
                    continue
                for i in range(nel):
                    fi, ni = rad.first[i], rad.nprim(i)
                    for j in range(nel):
                        fj, nj = rad.first[j], rad.nprim(j)
                        Ps = R[L][fi:fi + ni, fj:fj + nj]
                        Ks = ktei[L][i][j] @ Ps.ravel(order="F")
                        Kb[fi:fi + ni, fj:fj + nj] += Ks.reshape(ni, nj, order="F")
            K[ja * nrad:(ja + 1) * nrad, ka * nrad:(ka + 1) * nrad] -= Kb
    return K
