"""Oracle (test infrastructure only): numpy restatement of HelFEM's diatomic
two-dimensional basis in prolate spheroidal coordinates (mu, nu, phi) and of
the tables its Coulomb and exchange builds consume.

The GPU product is compared against it. Only tests, the smoke check and
the CPU-baseline leg of the benchmark may import it. It is written
independently of the product's C++ tabulation: the associated Legendre
functions are evaluated from mu (not from cosh mu), the angular couplings of
the cos(nu) powers come from the three-term recurrence of Y_l^m rather than
from Gaunt expansions, and the quadratures are fixed high-order Gauss-Legendre
rules with a cubic change of variable on the element that touches mu = 0.

Reference files restated here (paths inside the HelFEM project):

* ``src/legendre/Legendre.h:30-330``  P_L^M(x), Q_L^M(x) for x > 1 in the
  Hobson convention (no Condon-Shortley phase): P_1^1 = sqrt(x^2-1),
  Q_0^0 = 1/2 ln((x+1)/(x-1)), Q_0^1 = -1/sqrt(x^2-1); three-term recurrences
  in L, and in M for Q. Here Q_L^0, Q_L^1 come from Christoffel's closed form
  near x = 1 and from Miller's backward recurrence elsewhere.
* ``src/diatomic/basis.cpp:522-540``  radial FE basis in mu: the mu = 0
  function is kept, the mu_max function dropped (Nrad = Nel (Nnodes-1)).
* ``src/diatomic/basis.cpp:712-736``  pure functions: m != 0 shells drop their
  first (mu = 0) radial function.
* ``src/diatomic/basis.cpp:253-290,350-395`` one-electron radial integrals
  int B_a B_b sinh^m cosh^n dmu, the kinetic block int B'_a B'_b sinh dmu,
  and the disjoint factors int B_a B_b sinh cosh^k P_L^|M| (cosh mu) dmu
  (and Q_L^|M|).
* ``src/diatomic/quadrature.cpp:175-255``  in-element kernel
  T_kl[(cd),(ab)] = int int f^k_cd(mu1) f^l_ab(mu2) P(mu_<) Q(mu_>),
  f^k = B B sinh cosh^k.
* ``src/diatomic/basis.cpp:1382-1548``  compute_tei: the 2-channel kernel
  W = [[T00, -T02], [-T02', T22]] factorised W = B diag(sigma) B' by a
  diagonal-pivoted, sign-carrying Cholesky with relative threshold 1e-12.
* ``src/diatomic/basis.cpp:1549-1560``  LMfac = (-1)^M 4 pi Rhalf^5
  (L-|M|)! / (L+|M|)!.
* ``src/diatomic/basis.cpp:1033-1140``  overlap, kinetic, nuclear attraction.
* ``src/general/gaunt.cpp:254-290``  mod_coeff = int Y_lj^mj* cos^2(nu)
  Y_L^M Y_li^mi, cosine / cosine^2 couplings.
* ``src/diatomic/basis.cpp:1621-1815`` Coulomb (two channels: P0 with the
  cos^2-weighted coupling, P2 with the plain Gaunt coupling).
* ``src/diatomic/basis.cpp:1817-2061`` exchange (four channel pairs, signs
  +, -, -, +; RI-K contraction on the in-element blocks).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from functools import lru_cache

import numpy as np

from .tabulate import gauss_legendre, get_grid, gaunt, lip_eval, lobatto

# ---------------------------------------------------------------------------
# Associated Legendre functions of x = cosh(mu) > 1 (Hobson convention)
# ---------------------------------------------------------------------------


def legendre_pq(Lmax: int, Mmax: int, mu: np.ndarray):
    """P[M, L, i] and Q[M, L, i] for x = cosh(mu[i]), mu > 0.

    Non-finite and subnormal values are returned as 0, as the reference's
    Legendre cache does (diatomic/quadrature.h:45-52)."""
    mu = np.atleast_1d(np.asarray(mu, dtype=float))
    n = mu.size
    x = np.cosh(mu)
    w = np.sinh(mu)
    P = np.zeros((Mmax + 1, Lmax + 1, n))
    Q = np.zeros((Mmax + 1, Lmax + 1, n))
    # ---- P: diagonal seed, first off-diagonal, upward recurrence in L
    for M in range(Mmax + 1):
        if M > Lmax:
            break
        dfac = 1.0
        for k in range(1, 2 * M, 2):
            dfac *= k
        P[M, M] = dfac * w ** M
        if M + 1 <= Lmax:
            P[M, M + 1] = (2 * M + 1) * x * P[M, M]
        for L in range(M + 1, Lmax):
            P[M, L + 1] = ((2 * L + 1) * x * P[M, L] - (L + M) * P[M, L - 1]) / (L + 1 - M)
    # ---- Q_L^0 and Q_L^1
    q00 = -np.log(np.tanh(0.5 * mu))  # 1/2 ln((x+1)/(x-1)), exact in mu
    mu_sw = 1.0 / max(Lmax, 1)
    near = mu < mu_sw
    if near.any():
        # Christoffel: Q_L = P_L Q_0 - W_L, W obeys the Legendre recurrence
        # with W_0 = 0, W_1 = 1; M = 1 from the x-derivative, times w.
        xs, ws, q0 = x[near], w[near], q00[near]
        m = xs.size
        Pl = np.zeros((Lmax + 1, m))
        Wl = np.zeros((Lmax + 1, m))
        dP = np.zeros((Lmax + 1, m))
        dW = np.zeros((Lmax + 1, m))
        Pl[0] = 1.0
        if Lmax >= 1:
            Pl[1] = xs
            Wl[1] = 1.0
            dP[1] = 1.0
        for k in range(1, Lmax):
            Pl[k + 1] = ((2 * k + 1) * xs * Pl[k] - k * Pl[k - 1]) / (k + 1)
            Wl[k + 1] = ((2 * k + 1) * xs * Wl[k] - k * Wl[k - 1]) / (k + 1)
            dP[k + 1] = ((2 * k + 1) * (Pl[k] + xs * dP[k]) - k * dP[k - 1]) / (k + 1)
            dW[k + 1] = ((2 * k + 1) * (Wl[k] + xs * dW[k]) - k * dW[k - 1]) / (k + 1)
        Q[0, :, near] = (Pl * q0 - Wl).T
        if Mmax >= 1:
            Q[1, :, near] = (ws * dP * q0 - Pl / ws - ws * dW).T
    far = ~near
    if far.any():
        # Miller: backward recurrence from N well past Lmax (the minimal
        # solution dominates downward), normalised on Q_0^0 resp. Q_0^1.
        xs, ws, ms = x[far], w[far], mu[far]
        N = Lmax + int(math.ceil(37.0 / ms.min())) + 20
        for M in range(min(Mmax, 1) + 1):
            nxt = np.zeros_like(xs)
            cur = np.full_like(xs, 1e-280)
            vals = np.zeros((Lmax + 1, xs.size))
            for L in range(N, 0, -1):
                # (L-M+1) Q_{L+1} = (2L+1) x Q_L - (L+M) Q_{L-1}
                prev = ((2 * L + 1) * xs * cur - (L - M + 1) * nxt) / (L + M)
                nxt, cur = cur, prev
                if L - 1 <= Lmax:
                    vals[L - 1] = cur
                big = np.abs(cur) > 1e250
                if big.any():
                    cur = np.where(big, cur * 1e-250, cur)
                    nxt = np.where(big, nxt * 1e-250, nxt)
                    vals = np.where(big[None, :], vals * 1e-250, vals)
            if M == 0:
                vals *= q00[far] / vals[0]
            else:
                vals *= (-1.0 / ws) / vals[0]
            Q[M, :, far] = vals.T
    # ---- Q for M >= 2: upward recurrence in M
    #   Q_L^{M+1} = -2 M x / w Q_L^M + (L+M)(L-M+1) Q_L^{M-1}
    for M in range(1, Mmax):
        for L in range(Lmax + 1):
            Q[M + 1, L] = -2.0 * M * x / w * Q[M, L] + (L + M) * (L - M + 1) * Q[M - 1, L]
    for A in (P, Q):
        bad = ~np.isfinite(A) | ((A != 0.0) & (np.abs(A) < np.finfo(float).tiny))
        A[bad] = 0.0
    return P, Q


# ---------------------------------------------------------------------------
# Angular couplings
# ---------------------------------------------------------------------------


def _cos_matrix(lmax: int, m: int) -> np.ndarray:
    """C[l', l] = int Y_l'^m* cos(nu) Y_l^m for l, l' in |m|..lmax+2 (index l)."""
    n = lmax + 3
    C = np.zeros((n, n))
    for l in range(abs(m), n - 1):
        a = math.sqrt(((l + 1) ** 2 - m * m) / ((2 * l + 1) * (2 * l + 3)))
        C[l + 1, l] = a
        C[l, l + 1] = a
    return C


@lru_cache(maxsize=None)
def _cos2(lmax: int, m: int) -> np.ndarray:
    C = _cos_matrix(lmax + 2, m)
    return C @ C


def cosine_coupling(lj, mj, li, mi) -> float:
    if mi != mj:
        return 0.0
    return float(_cos_matrix(max(lj, li) + 1, mi)[lj, li])


def cosine2_coupling(lj, mj, li, mi) -> float:
    if mi != mj:
        return 0.0
    return float(_cos2(max(lj, li) + 2, mi)[lj, li])


@lru_cache(maxsize=None)
def coeff(L, M, l, m, lp) -> float:
    """int Y_L^M* Y_l^m Y_lp^{M-m}: the reference's Gaunt coeff()."""
    return gaunt(L, M, l, m, lp)


@lru_cache(maxsize=None)
def mod_coeff(lj, mj, L, M, li, mi) -> float:
    """int Y_lj^mj* cos^2(nu) Y_L^M Y_li^mi, with cos^2 applied to Y_li^mi
    through the l-recurrence: sum_l' (C^2)[l', li] coeff(lj, mj, l', mi, L)."""
    if mj != M + mi:
        return 0.0
    C2 = _cos2(li + 2, mi)
    s = 0.0
    for lp in (li - 2, li, li + 2):
        if lp < abs(mi) or lp < 0:
            continue
        c = C2[lp, li]
        if c != 0.0:
            s += c * coeff(lj, mj, lp, mi, L)
    return s


def lmfac(L: int, M: int, Rhalf: float) -> float:
    """(-1)^M 4 pi Rhalf^5 (L-|M|)!/(L+|M|)!  (basis.cpp:1549-1560)."""
    Ma = abs(M)
    fr = 1.0
    for p in range(L + Ma, L - Ma, -1):
        fr *= p
    return (-1.0 if M % 2 else 1.0) * 4.0 * math.pi * Rhalf ** 5 / fr


def lm_maps(lval, mval):
    """(L,|M|) list ordered |M|-major then L, and (L,M) list ordered by (L,M),
    of every multipole the angular basis couples (basis.cpp:553-620)."""
    lm, LM = set(), set()
    for li, mi in zip(lval, mval):
        for lj, mj in zip(lval, mval):
            M = mj - mi
            for L in range(max(abs(lj - li) - 2, abs(M)), lj + li + 3):
                lm.add((L, abs(M)))
                LM.add((L, M))
    lm = sorted(lm, key=lambda p: (p[1], p[0]))
    LM = sorted(LM)
    return lm, LM


def lm_to_l_m(lmmax):
    """Angular basis from lmax per |m| (basis.cpp:456-471)."""
    lv, mv = [], []
    for mabs, lmx in enumerate(lmmax):
        for l in range(mabs, lmx + 1):
            lv.append(l)
            mv.append(mabs)
            if mabs > 0:
                lv.append(l)
                mv.append(-mabs)
    return np.array(lv, int), np.array(mv, int)


# ---------------------------------------------------------------------------
# Radial FE basis in mu
# ---------------------------------------------------------------------------


def _sign_cholesky(W: np.ndarray, thresh: float = 1e-12):
    """Diagonal-pivoted, sign-carrying Cholesky W ~ B diag(sigma) B'
    (basis.cpp:1497-1535): pivot on the largest |residual diagonal|, stop
    when it drops to thresh * max|diag(W)|."""
    N = W.shape[0]
    d = np.diag(W).copy()
    dmax0 = np.max(np.abs(d)) if N else 0.0
    cols, sg = [], []
    for _ in range(N):
        piv = int(np.argmax(np.abs(d)))
        dp = d[piv]
        if dmax0 <= 0.0 or abs(dp) <= thresh * dmax0:
            break
        s = 1.0 if dp >= 0.0 else -1.0
        col = W[:, piv].copy()
        for c, sq in zip(cols, sg):
            col -= sq * c[piv] * c
        col /= math.sqrt(abs(dp))
        d -= s * col * col
        d[piv] = 0.0
        cols.append(col)
        sg.append(s)
    if not cols:
        return np.zeros((N, 0)), np.zeros(0)
    return np.stack(cols, axis=1), np.array(sg)


@dataclass
class DiatomicTables:
    """Everything the diatomic Fock build consumes (FP64, compact per element)."""

    Z1: int
    Z2: int
    Rhalf: float
    nnodes: int
    bval: np.ndarray
    lval: np.ndarray
    mval: np.ndarray
    nrad: int
    first: np.ndarray        # first global radial function of each element
    ni: np.ndarray           # functions per element
    lm: list                 # (L,|M|)
    LM: list                 # (L,M)
    P0: list                 # [ilm][iel] Ni x Ni
    P2: list
    Q0: list
    Q2: list
    cdB: list                # [ilm][iel] (2 Ni^2 x r)
    cds: list                # [ilm][iel] (r,)
    S: np.ndarray = None     # pure-basis one-electron matrices
    T: np.ndarray = None
    V: np.ndarray = None

    @property
    def nel(self):
        return len(self.bval) - 1

    @property
    def nang(self):
        return len(self.lval)

    @property
    def ndummy(self):
        return self.nang * self.nrad

    def pure_indices(self) -> np.ndarray:
        idx = []
        for ia, m in enumerate(self.mval):
            start = 0 if m == 0 else 1
            idx.extend(ia * self.nrad + j for j in range(start, self.nrad))
        return np.array(idx, dtype=np.int64)

    @property
    def nbf(self):
        return len(self.pure_indices())

    def expand(self, Ppure: np.ndarray) -> np.ndarray:
        idx = self.pure_indices()
        Pd = np.zeros((self.ndummy, self.ndummy))
        Pd[np.ix_(idx, idx)] = Ppure
        return Pd

    def remove(self, Fd: np.ndarray) -> np.ndarray:
        idx = self.pure_indices()
        return Fd[np.ix_(idx, idx)]

    def sym_blocks(self):
        """Per-m blocks over the pure functions, unique m ascending
        (basis.cpp:876-918, symmetry 1)."""
        idx = self.pure_indices()
        ang = idx // self.nrad
        mv = self.mval[ang]
        return [(m, np.where(mv == m)[0]) for m in sorted(set(int(x) for x in self.mval))]

    def lmind(self, L, M):
        return self._lmidx[(L, abs(M))]

    def __post_init__(self):
        self._lmidx = {p: i for i, p in enumerate(self.lm)}


class MuBasis:
    """LIP radial basis in mu; element iel spans [bval[iel], bval[iel+1]]."""

    def __init__(self, nnodes: int, bval):
        self.nn = nnodes
        self.bval = np.asarray(bval, float)
        self.nel = len(self.bval) - 1
        self.x0, _ = lobatto(nnodes)
        self.nrad = self.nel * (nnodes - 1)

    def enabled(self, iel):
        idx = np.arange(self.nn)
        if iel == self.nel - 1:
            idx = idx[:-1]
        return idx

    def first(self, iel):
        return iel * (self.nn - 1)

    def sf(self, iel):
        return 0.5 * (self.bval[iel + 1] - self.bval[iel])

    def mid(self, iel):
        return 0.5 * (self.bval[iel + 1] + self.bval[iel])

    def B(self, x, iel, nder=0):
        return lip_eval(np.asarray(x, float), self.x0, nder)[:, self.enabled(iel)] / self.sf(iel) ** nder

    def rule(self, iel, n):
        """Gauss-Legendre points (mu, x, w) on element iel."""
        x, w = gauss_legendre(n)
        return self.mid(iel) + self.sf(iel) * x, x, w * self.sf(iel)

    def weighted(self, iel, wfun, n=96, nder=0):
        mu, x, w = self.rule(iel, n)
        B = self.B(x, iel, nder)
        wt = w * wfun(mu)
        return (B * wt[:, None]).T @ B

    def assemble(self, blocks):
        M = np.zeros((self.nrad, self.nrad))
        for iel, blk in enumerate(blocks):
            f = self.first(iel)
            n = blk.shape[0]
            M[f:f + n, f:f + n] += blk
        return M

    def twoe(self, iel, Lmax_leg, M, Ls, n_out=64, n_in=64):
        """In-element kernels T_kl[(cd),(ab)] for k,l in {0,2}, every L in Ls,
        pair index a + b*Ni. Returns {L: (T00, T02, T22)}."""
        mus, mue = self.bval[iel], self.bval[iel + 1]
        xo, wo = gauss_legendre(n_out)
        if iel == 0:
            # cubic map mu = mue t^3 smooths the log / mu^-M endpoint of Q at 0
            t = 0.5 * (xo + 1.0)
            mu1 = mus + (mue - mus) * t ** 3
            w1 = 0.5 * wo * 3.0 * (mue - mus) * t * t
        else:
            mu1 = 0.5 * (mus + mue) + 0.5 * (mue - mus) * xo
            w1 = 0.5 * (mue - mus) * wo
        xi, wi = gauss_legendre(n_in)
        half = 0.5 * (mu1 - mus)
        mu2 = mus + half[:, None] * (xi[None, :] + 1.0)      # (n_out, n_in)
        w2 = half[:, None] * wi[None, :]
        ref = lambda mu: (mu - self.mid(iel)) / self.sf(iel)
        B1 = self.B(ref(mu1), iel)                            # (n_out, Ni)
        B2 = self.B(ref(mu2.ravel()), iel).reshape(n_out, n_in, -1)
        P1, Q1 = legendre_pq(Lmax_leg, M, mu1)
        P2, _ = legendre_pq(Lmax_leg, M, mu2.ravel())
        P2 = P2.reshape(M + 1, Lmax_leg + 1, n_out, n_in)
        ni = B1.shape[1]
        pr1 = (B1[:, :, None] * B1[:, None, :]).reshape(n_out, ni * ni, order="C")
        out = {}
        sh1, ch1 = np.sinh(mu1), np.cosh(mu1)
        sh2, ch2 = np.sinh(mu2), np.cosh(mu2)
        for L in Ls:
            inner = {}
            for l in (0, 2):
                wq = w2 * sh2 * ch2 ** l * P2[M, L]
                G = np.einsum("pq,pqa,pqb->pab", wq, B2, B2)  # (n_out, Ni, Ni)
                # pair index a + b*Ni: column-major vec of (a,b)
                inner[l] = G.transpose(0, 2, 1).reshape(n_out, ni * ni)
            res = {}
            for k in (0, 2):
                wk = w1 * sh1 * ch1 ** k * Q1[M, L]
                outerk = pr1 * wk[:, None]  # (n_out, pairs), symmetric in (c,d)
                for l in (0, 2):
                    res[(k, l)] = outerk.T @ inner[l]
            T00 = res[(0, 0)] + res[(0, 0)].T
            T02 = res[(0, 2)] + res[(2, 0)].T
            T22 = res[(2, 2)] + res[(2, 2)].T
            out[L] = (T00, T02, T22)
        return out


def build_diatomic(Z1: int, Z2: int, Rbond: float, nnodes: int, nelem: int, lmmax, Rmax: float = 40.0,
                   igrid: int = 4, zexp: float = 1.0, bval=None, cd_thresh: float = 1e-12,
                   one_electron: bool = True) -> DiatomicTables:
    """compute_tei plus the one-electron matrices (basis.cpp:522-645,
    1033-1140, 1382-1548)."""
    Rhalf = 0.5 * Rbond
    if bval is None:
        mumax = math.acosh(Rmax / Rhalf)
        bval = get_grid(mumax, nelem, igrid, zexp)
    rb = MuBasis(nnodes, bval)
    lval, mval = lm_to_l_m(lmmax)
    lm, LM = lm_maps(lval, mval)
    Lmax = max(L for L, _ in lm)
    Mmax = max(M for _, M in lm)
    nel = rb.nel
    first = np.array([rb.first(e) for e in range(nel)])
    ni = np.array([len(rb.enabled(e)) for e in range(nel)])
    nlm = len(lm)
    P0 = [[None] * nel for _ in range(nlm)]
    P2 = [[None] * nel for _ in range(nlm)]
    Q0 = [[None] * nel for _ in range(nlm)]
    Q2 = [[None] * nel for _ in range(nlm)]
    cdB = [[None] * nel for _ in range(nlm)]
    cds = [[None] * nel for _ in range(nlm)]
    for e in range(nel):
        mu, x, w = rb.rule(e, 96)
        B = rb.B(x, e)
        Pl, Ql = legendre_pq(Lmax, Mmax, mu)
        sh, ch = np.sinh(mu), np.cosh(mu)
        for i, (L, M) in enumerate(lm):
            for dst, fun, k in ((P0, Pl, 0), (P2, Pl, 2), (Q0, Ql, 0), (Q2, Ql, 2)):
                wt = w * sh * ch ** k * fun[M, L]
                dst[i][e] = (B * wt[:, None]).T @ B
        for M in range(Mmax + 1):
            Ls = [L for (L, Ma) in lm if Ma == M]
            Tt = rb.twoe(e, Lmax, M, Ls)
            for L in Ls:
                T00, T02, T22 = Tt[L]
                W = np.block([[T00, -T02], [-T02.T, T22]])
                W = 0.5 * (W + W.T)
                Bc, sg = _sign_cholesky(W, cd_thresh)
                i = lm.index((L, M))
                cdB[i][e] = Bc
                cds[i][e] = sg
    tab = DiatomicTables(Z1, Z2, Rhalf, nnodes, np.asarray(bval, float), lval, mval, rb.nrad, first, ni,
                         lm, LM, P0, P2, Q0, Q2, cdB, cds)
    if one_electron:
        _one_electron(tab, rb)
    return tab


def _one_electron(tab: DiatomicTables, rb: MuBasis):
    nel = rb.nel
    sh = np.sinh
    ch = np.cosh
    I10 = rb.assemble([rb.weighted(e, lambda m: sh(m)) for e in range(nel)])
    I11 = rb.assemble([rb.weighted(e, lambda m: sh(m) * ch(m)) for e in range(nel)])
    I12 = rb.assemble([rb.weighted(e, lambda m: sh(m) * ch(m) ** 2) for e in range(nel)])
    Im1 = rb.assemble([rb.weighted(e, lambda m: 1.0 / sh(m)) for e in range(nel)])
    Trad = rb.assemble([rb.weighted(e, lambda m: sh(m), nder=1) for e in range(nel)])
    n, nang = rb.nrad, tab.nang
    S = np.zeros((n * nang, n * nang))
    T = np.zeros_like(S)
    V = np.zeros_like(S)
    Rh = tab.Rhalf
    for ia in range(nang):
        li, mi = int(tab.lval[ia]), int(tab.mval[ia])
        si = slice(ia * n, (ia + 1) * n)
        T[si, si] = Trad + li * (li + 1) * I10 + (mi * mi) * Im1 if mi else Trad + li * (li + 1) * I10
        for ja in range(nang):
            lj, mj = int(tab.lval[ja]), int(tab.mval[ja])
            if mi != mj:
                continue
            sj = slice(ja * n, (ja + 1) * n)
            blk = I12 if li == lj else 0.0
            c2 = cosine2_coupling(lj, mj, li, mi)
            S[si, sj] = blk - c2 * I10
            vb = (tab.Z1 + tab.Z2) * I11 if li == lj else np.zeros((n, n))
            if tab.Z1 != tab.Z2:
                c1 = cosine_coupling(lj, mj, li, mi)
                vb = vb + (tab.Z2 - tab.Z1) * c1 * I10
            V[si, sj] = vb
    tab.S = tab.remove(S * Rh ** 3)
    tab.T = tab.remove(T * Rh / 2.0)
    tab.V = tab.remove(-V * Rh ** 2)


# ---------------------------------------------------------------------------
# Coulomb (numpy, follows basis.cpp:1621-1815)
# ---------------------------------------------------------------------------


def coulomb(tab: DiatomicTables, Ppure: np.ndarray) -> np.ndarray:
    P = tab.expand(Ppure)
    n, nang, nel = tab.nrad, tab.nang, tab.nel
    lv, mv = tab.lval, tab.mval
    J = np.zeros_like(P)
    for (L, M) in tab.LM:
        ilm = tab.lmind(L, M)
        fac = lmfac(L, M, tab.Rhalf)
        Pa0 = np.zeros((n, n))
        Pa2 = np.zeros((n, n))
        any_ket = False
        for k in range(nang):
            for l in range(nang):
                if mv[k] - mv[l] != M:
                    continue
                c0 = mod_coeff(lv[k], mv[k], L, M, lv[l], mv[l])
                c2 = coeff(lv[k], mv[k], L, M, lv[l])
                if c0 == 0.0 and c2 == 0.0:
                    continue
                blk = P[k * n:(k + 1) * n, l * n:(l + 1) * n]
                Pa0 += c0 * blk
                Pa2 += c2 * blk
                any_ket = True
        Ja0 = np.zeros((n, n))
        Ja2 = np.zeros((n, n))
        if any_ket:
            for je in range(nel):
                f, m_ = tab.first[je], tab.ni[je]
                s0 = Pa0[f:f + m_, f:f + m_]
                s2 = Pa2[f:f + m_, f:f + m_]
                js0 = fac * np.sum(tab.P0[ilm][je] * s0.T)
                jb0 = fac * np.sum(tab.Q0[ilm][je] * s0.T)
                js2 = fac * np.sum(tab.P2[ilm][je] * s2.T)
                jb2 = fac * np.sum(tab.Q2[ilm][je] * s2.T)
                for ie in range(nel):
                    fi, mi_ = tab.first[ie], tab.ni[ie]
                    if ie < je:
                        Ja0[fi:fi + mi_, fi:fi + mi_] += (jb0 - jb2) * tab.P0[ilm][ie]
                        Ja2[fi:fi + mi_, fi:fi + mi_] += (-jb0 + jb2) * tab.P2[ilm][ie]
                    elif ie > je:
                        Ja0[fi:fi + mi_, fi:fi + mi_] += (js0 - js2) * tab.Q0[ilm][ie]
                        Ja2[fi:fi + mi_, fi:fi + mi_] += (-js0 + js2) * tab.Q2[ilm][ie]
                Bc, sg = tab.cdB[ilm][je], tab.cds[ilm][je]
                pv = np.concatenate([s0.ravel(order="F"), s2.ravel(order="F")])
                jv = fac * (Bc @ (sg * (Bc.T @ pv)))
                nn2 = m_ * m_
                Ja0[f:f + m_, f:f + m_] += jv[:nn2].reshape(m_, m_, order="F")
                Ja2[f:f + m_, f:f + m_] += jv[nn2:].reshape(m_, m_, order="F")
        for i in range(nang):
            for j in range(nang):
                if mv[j] - mv[i] != M:
                    continue
                c0 = mod_coeff(lv[j], mv[j], L, M, lv[i], mv[i])
                c2 = coeff(lv[j], mv[j], L, M, lv[i])
                if c0 != 0.0:
                    J[i * n:(i + 1) * n, j * n:(j + 1) * n] += c0 * Ja0
                if c2 != 0.0:
                    J[i * n:(i + 1) * n, j * n:(j + 1) * n] += c2 * Ja2
    return tab.remove(J)


# ---------------------------------------------------------------------------
# Tables for the compiled exchange oracle (dfock_ref.cpp)
# ---------------------------------------------------------------------------


def gaunt_tables(tab: DiatomicTables):
    """Dense coupling tables over the basis: coef[(j, L, Midx, i)] =
    coeff(lj,mj,L,M,li) and modc[...] = mod_coeff(lj,mj,L,M,li,mi) with
    M = mj - mi, Midx = M + 2 mmax."""
    nang = tab.nang
    Lmax = max(L for L, _ in tab.lm)
    mmax = int(np.max(np.abs(tab.mval)))
    nM = 4 * mmax + 1
    co = np.zeros((nang, Lmax + 1, nM, nang))
    mo = np.zeros_like(co)
    for j in range(nang):
        lj, mj = int(tab.lval[j]), int(tab.mval[j])
        for i in range(nang):
            li, mi = int(tab.lval[i]), int(tab.mval[i])
            M = mj - mi
            for L in range(max(abs(lj - li) - 2, abs(M)), lj + li + 3):
                co[j, L, M + 2 * mmax, i] = coeff(lj, mj, L, M, li)
                mo[j, L, M + 2 * mmax, i] = mod_coeff(lj, mj, L, M, li, mi)
    return co, mo, Lmax, mmax
