"""Oracle (test infrastructure only): exchange-correlation functionals and the
atomic DFT-grid Vxc build, restated in numpy.

Functionals are restated from the published papers (libxc is not present and
its source is not used):

* Slater/Dirac exchange (``lda_x``).
* VWN5 correlation (``lda_c_vwn``): S. H. Vosko, L. Wilk, M. Nusair,
  Can. J. Phys. 58, 1200 (1980), parametrisation 5 with the spin-stiffness
  interpolation.
* PW92 correlation (``lda_c_pw``): J. P. Perdew, Y. Wang, PRB 45, 13244
  (1992); the ``pw_mod`` digits are used inside PBE correlation.
* PBE exchange and correlation (``gga_x_pbe``, ``gga_c_pbe``):
  J. P. Perdew, K. Burke, M. Ernzerhof, PRL 77, 3865 (1996).

Potentials (v_rho, v_sigma) are obtained by complex-step differentiation of
the energy density, which is exact to rounding for these analytic forms and
independent of the hand-derived derivatives in the CUDA kernels.

The grid build restates ``src/atomic/dftgrid.cpp:51-128,304-359,470-576``
(density and gradient on the per-element grid, LDA and GGA Fock terms) and
``src/general/dftgrid_common.h:128-217`` (split real/imaginary accumulation),
with the element loop of ``DFTGrid::eval_Fxc`` (dftgrid.cpp:591-712).
"""
from __future__ import annotations

import math

import numpy as np

from . import tabulate as tab

H_STEP = 1e-40

# --------------------------------------------------------------------------
# energy densities e(rho, sigma) per volume; spin-resolved inputs
# --------------------------------------------------------------------------


def _fzeta(opz, omz):
    # opz = 1 + zeta = 2 rho_a / n, omz = 1 - zeta = 2 rho_b / n, formed from the
    # spin densities (1 - zeta by subtraction loses a minority spin's precision)
    return (opz ** (4.0 / 3.0) + omz ** (4.0 / 3.0) - 2.0) / (2.0 ** (4.0 / 3.0) - 2.0)


FPP0 = 4.0 / (9.0 * (2.0 ** (1.0 / 3.0) - 1.0))


def slater_x(ra, rb):
    c = -0.75 * (6.0 / np.pi) ** (1.0 / 3.0)
    return c * (ra ** (4.0 / 3.0) + rb ** (4.0 / 3.0))


def _vwn_eps(x, A, b, c, x0):
    X = x * x + b * x + c
    X0 = x0 * x0 + b * x0 + c
    Q = math.sqrt(4 * c - b * b)
    at = np.arctan(Q / (2 * x + b))
    return A * (np.log(x * x / X) + 2 * b / Q * at
                - b * x0 / X0 * (np.log((x - x0) ** 2 / X) + 2 * (b + 2 * x0) / Q * at))


VWN5_P = (0.0310907, 3.72744, 12.9352, -0.10498)
VWN5_F = (0.01554535, 7.06042, 18.0578, -0.32500)
VWN5_A = (-1.0 / (6.0 * np.pi ** 2), 1.13107, 13.0045, -0.0047584)


def _rs(n):
    return (3.0 / (4.0 * np.pi * n)) ** (1.0 / 3.0)


def vwn5_c(ra, rb):
    n = ra + rb
    z = (ra - rb) / n
    x = np.sqrt(_rs(n))
    eP = _vwn_eps(x, *VWN5_P)
    eF = _vwn_eps(x, *VWN5_F)
    ac = _vwn_eps(x, *VWN5_A)
    f = _fzeta(2 * ra / n, 2 * rb / n)
    z4 = z ** 4
    eps = eP + ac * f / FPP0 * (1 - z4) + (eF - eP) * f * z4
    return n * eps


def _pw_G(rs, A, a1, b1, b2, b3, b4):
    den = 2 * A * (b1 * np.sqrt(rs) + b2 * rs + b3 * rs ** 1.5 + b4 * rs * rs)
    return -2 * A * (1 + a1 * rs) * np.log(1 + 1 / den)


PW92 = dict(
    P=(0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294),
    F=(0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517),
    A=(0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671),
    fpp=1.709921,
)
PW92_MOD = dict(
    P=(0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294),
    F=(0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517),
    A=(0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671),
    fpp=1.709920934161365617563962776245,
)


def _pw_eps(n, z, opz, omz, par):
    rs = _rs(n)
    eP = _pw_G(rs, *par["P"])
    eF = _pw_G(rs, *par["F"])
    ac = -_pw_G(rs, *par["A"])
    f = _fzeta(opz, omz)
    z4 = z ** 4
    return eP + ac * f / par["fpp"] * (1 - z4) + (eF - eP) * f * z4


def pw92_c(ra, rb):
    n = ra + rb
    return n * _pw_eps(n, (ra - rb) / n, 2 * ra / n, 2 * rb / n, PW92)


PBE_KAPPA = 0.804
PBE_MU = 0.2195149727645171
PBE_BETA = 0.06672455060314922
PBE_GAMMA = (1.0 - math.log(2.0)) / np.pi ** 2


def _pbe_x_unpol(n, s2n):
    # exchange of an unpolarised density n with |grad n|^2 = s2n
    kf = (3 * np.pi ** 2 * n) ** (1.0 / 3.0)
    ex_unif = -0.75 / np.pi * kf * n
    s2 = s2n / (2 * kf * n) ** 2
    Fx = 1 + PBE_KAPPA - PBE_KAPPA / (1 + PBE_MU * s2 / PBE_KAPPA)
    return ex_unif * Fx


def pbe_x(ra, rb, saa, sab, sbb):
    # spin scaling E_x[a,b] = (E_x[2a] + E_x[2b]) / 2
    return 0.5 * (_pbe_x_unpol(2 * ra, 4 * saa) + _pbe_x_unpol(2 * rb, 4 * sbb))


def pbe_c(ra, rb, saa, sab, sbb):
    n = ra + rb
    z = (ra - rb) / n
    opz, omz = 2 * ra / n, 2 * rb / n
    ec = _pw_eps(n, z, opz, omz, PW92_MOD)
    phi = 0.5 * (opz ** (2.0 / 3.0) + omz ** (2.0 / 3.0))
    kf = (3 * np.pi ** 2 * n) ** (1.0 / 3.0)
    ks = np.sqrt(4 * kf / np.pi)
    sig = saa + 2 * sab + sbb
    t2 = sig / (2 * phi * ks * n) ** 2
    g3 = PBE_GAMMA * phi ** 3
    A = PBE_BETA / PBE_GAMMA / (np.exp(-ec / g3) - 1)
    At2 = A * t2
    H = g3 * np.log(1 + PBE_BETA / PBE_GAMMA * t2 * (1 + At2) / (1 + At2 + At2 * At2))
    return n * (ec + H)


FUNCTIONALS = {
    "lda_x": ("lda", slater_x),
    "lda_c_vwn": ("lda", vwn5_c),
    "lda_c_pw": ("lda", pw92_c),
    "gga_x_pbe": ("gga", pbe_x),
    "gga_c_pbe": ("gga", pbe_c),
}


def parse_method(method: str):
    """'hf' or 'lda_x-lda_c_vwn' style strings (dftfuncs.cpp:94-143)."""
    if method.lower() == "hf":
        return []
    return [p for p in method.split("-") if p]


def eval_functionals(names, ra, rb, saa=None, sab=None, sbb=None, thr=1e-12):
    """Return e (per volume), v_rho_a, v_rho_b, v_saa, v_sab, v_sbb at every
    point. Points with total density below thr contribute nothing, as libxc's
    density threshold does."""
    n = ra + rb
    ok = n >= thr
    npts = len(ra)
    out = [np.zeros(npts) for _ in range(6)]
    if not ok.any():
        return out
    ra_, rb_ = np.maximum(ra[ok], thr / 2), np.maximum(rb[ok], thr / 2)
    gga = any(FUNCTIONALS[f][0] == "gga" for f in names)
    if gga:
        sa, sx, sb = saa[ok], sab[ok], sbb[ok]
    else:
        sa = sx = sb = np.zeros_like(ra_)
    args = [ra_, rb_, sa, sx, sb]
    for f in names:
        kind, fn = FUNCTIONALS[f]
        nargs = 2 if kind == "lda" else 5
        e = np.real(fn(*args[:nargs]))
        out[0][ok] += e
        for k in range(nargs):
            a = [x.astype(complex) for x in args[:nargs]]
            a[k] = a[k] + 1j * H_STEP
            out[1 + k][ok] += np.imag(fn(*a)) / H_STEP
    return out


# --------------------------------------------------------------------------
# atomic DFT grid
# --------------------------------------------------------------------------


def _ylm(l, m, cth, phi):
    return tab.theta_lm(l, m, cth) * np.exp(1j * m * phi)


class AtomGrid:
    """Per-element (radial Chebyshev x angular Chebyshev x uniform phi) grid
    (dftgrid.cpp:470-576, angular.cpp:21-70)."""

    def __init__(self, atom: tab.AtomTables, ldft: int = 0, mdft: int = 0):
        self.atom = atom
        lmax, mmax = int(atom.lval.max()), int(np.abs(atom.mval).max())
        self.ldft = ldft or 4 * lmax + 12
        self.mdft = mdft or 4 * mmax + 12
        xc, wc = tab.chebyshev(self.ldft)
        dphi = 2 * np.pi / self.mdft
        self.cth = np.repeat(xc, self.mdft)
        self.phi = np.tile(np.arange(self.mdft) * dphi, self.ldft)
        self.wang = np.repeat(wc * dphi, self.mdft)
        self._cache = {}

    def element(self, iel):
        if iel in self._cache:
            return self._cache[iel]
        A, rad = self.atom, self.atom.rad
        r, wrad, xq = rad.dft_points(iel)
        R = rad.R(xq, iel)  # (nrad, ni)
        dR = rad.dR(xq, iel)
        nr, na = len(r), len(self.wang)
        sth = np.sqrt(1 - self.cth ** 2)
        cot = self.cth / sth
        Y = np.array([_ylm(l, m, self.cth, self.phi) for l, m in zip(A.lval, A.mval)])  # (nang, na)
        dY = np.array([m * cot * _ylm(l, m, self.cth, self.phi)
                       + (math.sqrt((l - m) * (l + m + 1)) * np.exp(-1j * self.phi)
                          * _ylm(l, m + 1, self.cth, self.phi) if m < l else 0.0)
                       for l, m in zip(A.lval, A.mval)])
        mfac = np.array([1j * m for m in A.mval])[:, None] * Y
        # basis values: functions f = (iang, irad) ; points p = ia*nr + ir
        def outer(ang, radv):
            # (nang, na) x (nr, ni) -> (nang*ni, na*nr); stored conjugated
            v = np.einsum("ka,ri->kiar", ang, radv).reshape(len(A.lval) * radv.shape[1], na * nr)
            return np.conj(v)
        bf = outer(Y, R)
        bfr = outer(Y, dR)
        bft = outer(dY, R)
        bfp = outer(mfac, R)
        scale_t = np.tile(r, na)
        scale_p = np.repeat(sth, nr) * np.tile(r, na)
        wtot = np.repeat(self.wang, nr) * np.tile(wrad * r * r, na)
        ni = R.shape[1]
        f0 = rad.first[iel]
        idx = np.concatenate([ia * rad.nbf + f0 + np.arange(ni) for ia in range(len(A.lval))])
        res = dict(bf=bf, grads=(bfr, bft, bfp), scales=(np.ones_like(scale_t), scale_t, scale_p),
                   w=wtot, idx=idx)
        self._cache[iel] = res
        return res

    def eval_Fxc(self, names, Pa, Pb, thr=1e-12):
        """Return (Ha, Hb, Exc, Nel) for spin densities Pa, Pb."""
        gga = any(FUNCTIONALS[f][0] == "gga" for f in names)
        nbf = Pa.shape[0]
        Ha = np.zeros((nbf, nbf))
        Hb = np.zeros((nbf, nbf))
        Exc = 0.0
        Nel = 0.0
        for iel in range(self.atom.rad.nel):
            E = self.element(iel)
            idx, bf, w = E["idx"], E["bf"], E["w"]
            pa = Pa[np.ix_(idx, idx)]
            pb = Pb[np.ix_(idx, idx)]

            def dens(P, g):
                return np.real(np.einsum("ab,ap,bp->p", P, bf, np.conj(g)))

            ra, rb = dens(pa, bf), dens(pb, bf)
            Nel += np.sum(w * (ra + rb))
            if gga:
                ga = [2 * dens(pa, g) / s for g, s in zip(E["grads"], E["scales"])]
                gb = [2 * dens(pb, g) / s for g, s in zip(E["grads"], E["scales"])]
                saa = sum(x * x for x in ga)
                sab = sum(x * y for x, y in zip(ga, gb))
                sbb = sum(x * x for x in gb)
            else:
                saa = sab = sbb = None
            e, va, vb, vaa, vab, vbb = eval_functionals(names, ra, rb, saa, sab, sbb, thr)
            Exc += np.sum(w * e)
            for H, v, own, oth, vs_own in ((Ha, va, "a", "b", vaa), (Hb, vb, "b", "a", vbb)):
                M = np.real(np.einsum("p,ap,bp->ab", w * v, bf, np.conj(bf)))
                if gga:
                    gown = ga if own == "a" else gb
                    goth = gb if own == "a" else ga
                    X = np.zeros_like(M)
                    for c, (g, s) in enumerate(zip(E["grads"], E["scales"])):
                        coef = w * (2 * vs_own * gown[c] + vab * goth[c]) / s
                        X += np.real(np.einsum("p,ap,bp->ab", coef, g, np.conj(bf)))
                    M += X + X.T
                H[np.ix_(idx, idx)] += M
        return Ha, Hb, Exc, Nel
