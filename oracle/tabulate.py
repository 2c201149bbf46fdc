"""Oracle (test infrastructure only): numpy restatement of HelFEM's atomic
finite-element radial basis and of the tabulated quantities the Fock build
consumes.

The GPU product is compared against it. Only tests, the smoke check and
the CPU-baseline leg of the benchmark may import it. It is written
independently of the product's C++ tabulation (different quadrature rules,
vectorised numpy) so that agreement between the two is evidence, not an echo.

Reference files restated here (paths inside the HelFEM project):

* ``libhelfem/include/lobatto.h:35-108``      Gauss-Lobatto rule (Newton on
  Chebyshev-Gauss-Lobatto guesses).
* ``libhelfem/include/chebyshev.h:31-55``     modified Gauss-Chebyshev rule.
* ``libhelfem/include/grid.h:37-101``         element boundary grids 1-5.
* ``libhelfem/include/LIPBasis.h:30-105`` and ``LIPBasis_eval.h:29-100``
  Lagrange interpolating polynomials on the nodes, derivatives, and the
  deflated B/r form on the first element.
* ``libhelfem/src/FiniteElementBasis.cpp:51-64,158-161,183,305-320``
  element bookkeeping: shared boundary functions, dropped first/last function.
* ``libhelfem/src/RadialBasis.cpp:245-257,868-926`` radial integrals in the
  R = B/r representation, R and dR/dr on a grid.
* ``libhelfem/src/quadrature.cpp:36-161``     in-element 2e tensor
  (r_<^L / r_>^{L+1}), symmetrised.
* ``libhelfem/src/RadialBasis.cpp:670-716``   pivoted Cholesky, tol 1e-12.
* ``libhelfemqc/include/CoulombExchangeFE.h:180-217`` disjoint factors
  r_small = int B B r^L, r_big = int B B r^{-L-1} (not on element 0).
* ``src/general/gaunt.cpp:77-84,201-251``     Gaunt coefficients
  int Y_L^M* Y_l^m Y_l'^{M-m}, from Racah's closed form for the Wigner 3j
  symbol in exact rational arithmetic (the reference calls the wignernj
  library, which also rounds an exact rational once).
* ``src/atomic/basis.cpp:179-203``            angular basis ordering.
* ``src/general/angular.cpp:21-70``           Chebyshev x uniform-phi
  angular rule for the DFT grid.

Integrals that the reference converges adaptively with Gauss-Lobatto rules
are evaluated here with fixed high-order Gauss-Legendre rules; every one of
them is either a polynomial integrated exactly or an analytic integrand whose
singularity lies outside the element, so both routes converge to the same
value to within a few ulps.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from decimal import Decimal, getcontext
from fractions import Fraction
from functools import lru_cache

import numpy as np

# ---------------------------------------------------------------------------
# 1-D quadrature rules
# ---------------------------------------------------------------------------


def lobatto(n: int):
    """Gauss-Lobatto nodes/weights on [-1,1] (lobatto.h:35-108)."""
    if n < 2:
        raise ValueError("Lobatto rule needs n >= 2")
    x = np.cos(np.pi * np.arange(n) / (n - 1))
    tol = 100 * np.finfo(float).eps
    while True:
        xold = x.copy()
        p = np.zeros((n, n))
        p[:, 0] = 1.0
        p[:, 1] = x
        for j in range(2, n):
            p[:, j] = ((2 * j - 1) * x * p[:, j - 1] - (j - 1) * p[:, j - 2]) / j
        x = xold - (x * p[:, n - 1] - p[:, n - 2]) / (n * p[:, n - 1])
        if np.max(np.abs(x - xold)) <= tol:
            break
    x = x[::-1].copy()
    pn = np.ones(n)
    pnm1 = np.ones(n)
    pn = x.copy()
    for j in range(2, n):
        pnm2 = pnm1
        pnm1 = pn
        pn = ((2 * j - 1) * x * pnm1 - (j - 1) * pnm2) / j
    w = 2.0 / ((n - 1) * n * pn * pn)
    return x, w


def chebyshev(n: int):
    """Modified Gauss-Chebyshev rule of the second kind (chebyshev.h:31-55)."""
    i = np.arange(1, n + 1, dtype=float)
    ang = i * np.pi / (n + 1)
    s = np.sin(ang)
    c = np.cos(ang)
    s2 = s * s
    w = 16.0 / 3.0 / (n + 1) * s2 * s2
    x = 1.0 - 2.0 * i / (n + 1) + 2.0 / np.pi * (1.0 + 2.0 / 3.0 * s2) * c * s
    return x[::-1].copy(), w[::-1].copy()


@lru_cache(maxsize=None)
def gauss_legendre(n: int):
    x, w = np.polynomial.legendre.leggauss(n)
    x.setflags(write=False)
    w.setflags(write=False)
    return x, w


def get_grid(rmax: float, num_el: int, igrid: int, zexp: float) -> np.ndarray:
    """Element boundaries (grid.h:37-101)."""
    if igrid == 1:
        b = np.linspace(0.0, rmax, num_el + 1)
    elif igrid == 2:
        i = np.arange(num_el + 1, dtype=float)
        b = i * i * rmax / (num_el * num_el)
    elif igrid == 3:
        b = rmax * (np.arange(num_el + 1) / num_el) ** zexp
    elif igrid == 4:
        upper = math.log(rmax + 1.0) ** (1.0 / zexp)
        t = np.linspace(0.0, upper, num_el + 1)
        b = np.exp(t ** zexp) - 1.0
    elif igrid == 5:
        if not (0.0 < zexp < 1.0):
            raise ValueError("invalid s parameter")
        hk = np.zeros(num_el)
        hk[-1] = (1 - zexp) / (1 - zexp ** num_el) * rmax
        for iel in range(num_el - 2, -1, -1):
            hk[iel] = zexp * hk[iel + 1]
        b = np.concatenate([[0.0], np.cumsum(hk)])
    else:
        raise ValueError("invalid grid")
    b = np.array(b, dtype=float)
    b[0] = 0.0
    b[-1] = rmax
    return b


# ---------------------------------------------------------------------------
# Lagrange interpolating polynomials (primitive basis 4)
# ---------------------------------------------------------------------------


def lip_eval(x: np.ndarray, x0: np.ndarray, nder: int) -> np.ndarray:
    """d^n L_i / dx^n at points x for nodes x0; shape (len(x), len(x0)).

    Sum-of-products form (LIPBasis_eval.h): valid at the nodes themselves.
    """
    x = np.asarray(x, dtype=float)
    n = len(x0)
    out = np.zeros((len(x), n))
    diff = x[:, None] - x0[None, :]  # (npts, n)
    for fi in range(n):
        den = x0[fi] - x0  # (n,)
        others = [p for p in range(n) if p != fi]
        if nder == 0:
            v = np.ones(len(x))
            for p in others:
                v = v * diff[:, p] / den[p]
            out[:, fi] = v
        elif nder == 1:
            acc = np.zeros(len(x))
            for d1 in others:
                v = np.ones(len(x))
                for p in others:
                    if p != d1:
                        v = v * diff[:, p] / den[p]
                acc += v / den[d1]
            out[:, fi] = acc
        elif nder == 2:
            acc = np.zeros(len(x))
            for a, d1 in enumerate(others):
                for d2 in others[:a]:
                    v = np.ones(len(x))
                    for p in others:
                        if p != d1 and p != d2:
                            v = v * diff[:, p] / den[p]
                    acc += v / (den[d1] * den[d2])
            out[:, fi] = 2.0 * acc
        else:
            raise ValueError("nder <= 2 supported")
    return out


# ---------------------------------------------------------------------------
# Finite-element radial basis
# ---------------------------------------------------------------------------


@dataclass
class RadialBasis:
    """FE radial basis: LIP on Gauss-Lobatto nodes, Dirichlet at r=0 and Rmax.

    Function layout follows FiniteElementBasis.cpp:51-64 (consecutive
    elements share one function) and :305-313 (element 0 drops its x=-1
    function; the last element drops its x=+1 function).
    """

    nnodes: int
    bval: np.ndarray
    nquad: int = 0
    x0: np.ndarray = field(init=False)
    nel: int = field(init=False)
    first: np.ndarray = field(init=False)
    last: np.ndarray = field(init=False)
    nbf: int = field(init=False)

    def __post_init__(self):
        self.bval = np.asarray(self.bval, dtype=float)
        self.x0, _ = lobatto(self.nnodes)
        self.nel = len(self.bval) - 1
        if self.nquad == 0:
            self.nquad = 5 * self.nnodes
        first = np.zeros(self.nel, dtype=int)
        last = np.zeros(self.nel, dtype=int)
        for iel in range(self.nel):
            first[iel] = 0 if iel == 0 else last[iel - 1]
            last[iel] = first[iel] + len(self.enabled(iel)) - 1
        self.first, self.last = first, last
        self.nbf = int(last[-1] + 1)

    # --- element geometry --------------------------------------------------
    def enabled(self, iel: int) -> np.ndarray:
        idx = np.arange(self.nnodes)
        if iel == 0:
            idx = idx[1:]
        if iel == self.nel - 1:
            idx = idx[:-1]
        return idx

    def nprim(self, iel: int) -> int:
        return len(self.enabled(iel))

    def sf(self, iel: int) -> float:
        return 0.5 * (self.bval[iel + 1] - self.bval[iel])

    def mid(self, iel: int) -> float:
        return 0.5 * (self.bval[iel] + self.bval[iel + 1])

    def coord(self, x, iel):
        return self.mid(iel) + self.sf(iel) * np.asarray(x)

    # --- basis values -------------------------------------------------------
    def B(self, x, iel, nder=0):
        """d^n B / dr^n at reference points x (RadialBasis: eval_dnf)."""
        v = lip_eval(x, self.x0, nder)[:, self.enabled(iel)]
        return v / self.sf(iel) ** nder

    def R(self, x, iel):
        """R = B / r; analytic deflation on element 0 (LIPBasis.h:74-101)."""
        if iel == 0:
            return self._over_r(x, 0)
        return self.B(x, iel) / self.coord(x, iel)[:, None]

    def dR(self, x, iel):
        """dR/dr (RadialBasis.cpp:887-901)."""
        if iel == 0:
            return self._over_r(x, 1)
        r = self.coord(x, iel)[:, None]
        return (-self.B(x, iel) / r + self.B(x, iel, 1)) / r

    def _over_r(self, x, nder):
        # B_u(r)/r on element 0, r = sf (x+1): deflate the (x+1) factor.
        sf = self.sf(0)
        red = lip_eval(x, self.x0[1:], nder)  # drops node x0[0] = -1
        en = self.enabled(0)
        out = np.empty((len(np.atleast_1d(x)), len(en)))
        for k, ifull in enumerate(en):
            out[:, k] = red[:, ifull - 1] / (self.x0[ifull] + 1.0)
        return out / sf ** (nder + 1)

    # --- one-electron radial integrals --------------------------------------
    def radial_integral(self, rexp: int, iel: int, ngl: int = 128):
        """int R_a R_b r^{rexp+2} dr over element iel (RadialBasis.cpp:245-257)."""
        x, w = gauss_legendre(ngl)
        r = self.coord(x, iel)
        R = self.R(x, iel)
        wt = w * self.sf(iel) * r ** (rexp + 2)
        return (R * wt[:, None]).T @ R

    def kinetic(self, iel: int, ngl: int = 64):
        x, w = gauss_legendre(ngl)
        dB = self.B(x, iel, 1)
        return 0.5 * (dB * (w * self.sf(iel))[:, None]).T @ dB

    def assemble(self, blocks) -> np.ndarray:
        M = np.zeros((self.nbf, self.nbf))
        for iel, blk in enumerate(blocks):
            f, l = self.first[iel], self.last[iel] + 1
            M[f:l, f:l] += blk
        return M

    # --- in-element two-electron tensor --------------------------------------
    def twoe_integral(self, L: int, iel: int, n_out: int = 128, n_in: int = 48):
        """(ij|kl)_L = int int B_iB_j(r) B_kB_l(r') r_<^L / r_>^{L+1}.

        Returned as a (Ni^2 x Ni^2) matrix with pair index a + b*Ni
        (quadrature.cpp:136-161; CoulombExchangeFE.h:471-477).
        """
        rmin, rmax = self.bval[iel], self.bval[iel + 1]
        xo, wo = gauss_legendre(n_out)
        xi, wi = gauss_legendre(n_in)
        ro = self.coord(xo, iel)
        Bo = self.B(xo, iel)  # (n_out, Ni)
        # inner: G_kl(p) = int_{rmin}^{r_p} B_k B_l r'^L dr'   (exact)
        half = 0.5 * (ro - rmin)  # (n_out,)
        rin = rmin + half[:, None] * (xi[None, :] + 1.0)  # (n_out, n_in)
        xin = (rin - self.mid(iel)) / self.sf(iel)
        Bin = self.B(xin.ravel(), iel).reshape(n_out, n_in, -1)
        win = (half[:, None] * wi[None, :]) * rin ** L
        G = np.einsum("pq,pqk,pql->pkl", win, Bin, Bin)
        wout = wo * self.sf(iel) * ro ** (-L - 1.0)
        T = np.einsum("p,pi,pj,pkl->ijkl", wout, Bo, Bo, G)
        ni = Bo.shape[1]
        # pair index a + b*Ni  -> Fortran-order reshape of (a,b)
        Tm = T.transpose(1, 0, 3, 2).reshape(ni * ni, ni * ni)
        return Tm + Tm.T

    def dft_points(self, iel: int):
        """Chebyshev radial points and weights of element iel
        (RadialBasis.cpp:178-188,928-946)."""
        xq, wq = chebyshev(self.nquad)
        return self.coord(xq, iel), self.sf(iel) * wq, xq


def pivoted_cholesky(A: np.ndarray, tol: float = 1e-12) -> np.ndarray:
    """Greedy pivoted Cholesky with absolute residual-diagonal tolerance
    (RadialBasis.cpp:670-709). Returns L (n x r), L L^T ~ A."""
    n = A.shape[0]
    D = np.diag(A).copy()
    done = np.zeros(n, dtype=bool)
    cols = []
    for _ in range(n):
        cand = np.where(~done & (D > tol), D, -np.inf)
        piv = int(np.argmax(cand))
        if not np.isfinite(cand[piv]):
            break
        done[piv] = True
        s = math.sqrt(D[piv])
        col = A[:, piv].copy()
        for c in cols:
            col -= c * c[piv]
        col /= s
        col[done] = 0.0
        col[piv] = s
        cols.append(col)
        D[~done] -= col[~done] ** 2
    return np.stack(cols, axis=1) if cols else np.zeros((n, 0))


# ---------------------------------------------------------------------------
# Angular basis and Gaunt coefficients
# ---------------------------------------------------------------------------


def angular_basis(lmax: int, mmax: int):
    """(l, m) list: |m| outer, l inner, +m before -m (basis.cpp:179-203)."""
    lval, mval = [], []
    for mabs in range(mmax + 1):
        for l in range(mabs, lmax + 1):
            lval.append(l)
            mval.append(mabs)
            if mabs > 0:
                lval.append(l)
                mval.append(-mabs)
    return np.array(lval, dtype=int), np.array(mval, dtype=int)


def _assoc_legendre_norm(l: int, m: int, x: np.ndarray) -> np.ndarray:
    """Theta_l^m(x) with Y_l^m = Theta_l^m(cos th) e^{i m phi}; Condon-Shortley
    phase included, m >= 0, normalised over the sphere."""
    # normalised recurrences: start at P_m^m
    somx2 = np.sqrt(np.maximum((1 - x) * (1 + x), 0.0))
    # N_mm P_mm = (-1)^m sqrt((2m+1)/(4pi) (2m-1)!!^2/(2m)!) (1-x^2)^{m/2}
    c = math.sqrt((2 * m + 1) / (4 * math.pi))
    for k in range(1, m + 1):
        c *= math.sqrt((2 * k - 1) / (2 * k))
    pmm = ((-1) ** m) * c * somx2 ** m
    if l == m:
        return pmm
    # Theta_{m+1}^m
    pm1 = x * math.sqrt(2 * m + 3) * pmm
    if l == m + 1:
        return pm1
    p2, p1 = pmm, pm1
    for ll in range(m + 2, l + 1):
        a = math.sqrt((4 * ll * ll - 1) / (ll * ll - m * m))
        b = math.sqrt(((ll - 1) ** 2 - m * m) / (4 * (ll - 1) ** 2 - 1))
        p = a * (x * p1 - b * p2)
        p2, p1 = p1, p
    return p1


def theta_lm(l: int, m: int, x: np.ndarray) -> np.ndarray:
    if abs(m) > l:
        return np.zeros_like(x)
    if m >= 0:
        return _assoc_legendre_norm(l, m, x)
    return ((-1) ** abs(int(m))) * _assoc_legendre_norm(l, -m, x)


def _pi_decimal():
    """pi to ~60 digits (Machin's formula), for the exact Gaunt rounding."""
    getcontext().prec = 70

    def arctan_inv(x):
        x = Decimal(x)
        term = 1 / x
        total, n, sign, x2 = term, 1, 1, x * x
        while True:
            term /= x2
            n += 2
            sign = -sign
            t = term / n
            if t < Decimal(10) ** -68:
                break
            total += sign * t
        return total

    return 4 * (4 * arctan_inv(5) - arctan_inv(239))


_PI = None


def _fact(n):
    return math.factorial(n)


def _threej_sq(j1, j2, j3, m1, m2, m3):
    """(j1 j2 j3; m1 m2 m3) as (sign, Fraction value of the square root's
    argument times the Racah sum squared): returns Fraction v with
    3j = sign(v) * sqrt(|v|). Exact integer arithmetic (Racah formula)."""
    if m1 + m2 + m3 != 0:
        return Fraction(0)
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return Fraction(0)
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return Fraction(0)
    pre = Fraction(_fact(j1 + j2 - j3) * _fact(j1 - j2 + j3) * _fact(-j1 + j2 + j3),
                   _fact(j1 + j2 + j3 + 1))
    pre *= (_fact(j1 + m1) * _fact(j1 - m1) * _fact(j2 + m2) * _fact(j2 - m2)
            * _fact(j3 + m3) * _fact(j3 - m3))
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        den = (_fact(k) * _fact(j3 - j2 + k + m1) * _fact(j3 - j1 + k - m2)
               * _fact(j1 + j2 - j3 - k) * _fact(j1 - k - m1) * _fact(j2 - k + m2))
        s += Fraction((-1) ** k, den)
    phase = -1 if (j1 - j2 - m3) % 2 else 1
    v = pre * s * s
    return v if (phase * s) >= 0 else -v


def gaunt(L: int, M: int, l: int, m: int, lp: int) -> float:
    """coeff(L,M,l,m,lp) = int Y_L^M* Y_l^m Y_lp^{M-m} dOmega (gaunt.cpp:77-84,
    201-251), correctly rounded: exact rationals (Racah's formula for the two
    Wigner 3j symbols) and a 60-digit square root."""
    global _PI
    mp = M - m
    if L < 0 or l < 0 or lp < 0:
        return 0.0
    if abs(M) > L or abs(m) > l or abs(mp) > lp:
        return 0.0
    if (L + l + lp) % 2 or lp < abs(L - l) or lp > L + l:
        return 0.0
    # Y_L^M* = (-1)^M Y_L^{-M}:  (-1)^M int Y_L^{-M} Y_l^m Y_lp^mp
    a = _threej_sq(L, l, lp, 0, 0, 0)
    b = _threej_sq(L, l, lp, -M, m, mp)
    v = a * b * (2 * L + 1) * (2 * l + 1) * (2 * lp + 1)
    if v == 0:
        return 0.0
    sign = (1 if v > 0 else -1) * (-1 if M % 2 else 1)
    if _PI is None:
        _PI = _pi_decimal()
    getcontext().prec = 60
    val = (Decimal(abs(v.numerator)) / Decimal(v.denominator) / (4 * _PI)).sqrt()
    return sign * float(val)


# ---------------------------------------------------------------------------
# Atomic two-dimensional basis (TwoDBasis restated as plain data)
# ---------------------------------------------------------------------------


@dataclass
class AtomTables:
    """Everything the atomic Fock build consumes, in FP64."""

    Z: int
    rad: RadialBasis
    lval: np.ndarray
    mval: np.ndarray
    NL: int
    rs: list  # rs[L][iel]  (Ni x Ni)
    rb: list  # rb[L][iel]  (Ni x Ni), rb[L][0] empty
    chol: list  # chol[L][iel] (Ni^2 x r)
    S: np.ndarray
    T: np.ndarray
    V: np.ndarray

    @property
    def nrad(self):
        return self.rad.nbf

    @property
    def nang(self):
        return len(self.lval)

    @property
    def nbf(self):
        return self.nrad * self.nang


def build_atom(Z: int, nnodes: int, bval, lmax: int, mmax: int = None,
               lval=None, mval=None, nquad: int = 0, chol_tol: float = 1e-12) -> AtomTables:
    """compute_tei plus one-electron matrices (TwoDBasis.cpp:66-94, 350-374,
    708-735)."""
    rad = RadialBasis(nnodes, np.asarray(bval, float), nquad)
    if lval is None:
        lval, mval = angular_basis(lmax, lmax if mmax is None else mmax)
    lval = np.asarray(lval, int)
    mval = np.asarray(mval, int)
    NL = 2 * int(lval.max()) + 1
    rs = [[rad.radial_integral(L, e) for e in range(rad.nel)] for L in range(NL)]
    rb = [[None if e == 0 else rad.radial_integral(-L - 1, e) for e in range(rad.nel)]
          for L in range(NL)]
    chol = [[pivoted_cholesky(rad.twoe_integral(L, e), chol_tol) for e in range(rad.nel)]
            for L in range(NL)]
    Srad = rad.assemble([rad.radial_integral(0, e) for e in range(rad.nel)])
    Trad = rad.assemble([rad.kinetic(e) for e in range(rad.nel)])
    Tl = rad.assemble([0.5 * rad.radial_integral(-2, e) for e in range(rad.nel)])
    Vrad = rad.assemble([rad.radial_integral(-1, e) for e in range(rad.nel)])
    n = rad.nbf
    nang = len(lval)
    S = np.zeros((n * nang, n * nang))
    T = np.zeros_like(S)
    V = np.zeros_like(S)
    for ia in range(nang):
        sl = slice(ia * n, (ia + 1) * n)
        S[sl, sl] = Srad
        T[sl, sl] = Trad + lval[ia] * (lval[ia] + 1) * Tl
        V[sl, sl] = -Z * Vrad
    return AtomTables(Z, rad, lval, mval, NL, rs, rb, chol, S, T, V)


def invh(S: np.ndarray) -> np.ndarray:
    """Symmetric orthonormaliser with diagonal pre-normalisation
    (utils.cpp:120-159, chol=false)."""
    d = np.diag(S) ** -0.5
    Sn = d[:, None] * S * d[None, :]
    ev, evec = np.linalg.eigh(Sn)
    X = evec @ np.diag(ev ** -0.5) @ evec.T
    return d[:, None] * X
