"""Oracle (test infrastructure only): numpy restatement of HelFEM's pure-m
diatomic DFT grid, the XC potential of a diatomic whose orbitals do not mix
m (symmetry >= 1).

The GPU product is compared against it. Only tests, the smoke check and
the CPU-baseline leg of the benchmark may import it.

Reference files restated here (paths inside the HelFEM project):

* ``src/diatomic/dftgrid_purem.cpp:34-80``  nu rule: modified Gauss-Chebyshev
  in cos(nu) of order lang (default 4 lmax + 12, ``src/diatomic/main.cpp:316``);
  angular factors Y_l^m(nu, phi = 0) and
  dY/dnu = m cot(nu) Y_l^m + sqrt((l-m)(l+m+1)) Y_l^{m+1}.
* ``src/diatomic/dftgrid_purem.cpp:83-199``  per radial point: the element's
  Chebyshev rule of 5 Nnodes points in mu (``main.cpp:191``, radial weight
  wr = element half-length x wq, ``basis.cpp:496-503``), scale factor
  h = Rhalf sqrt(sinh^2 mu + sin^2 nu) and weight
  w = 2 pi wang wr Rhalf^3 sinh mu (sinh^2 mu + sin^2 nu); basis values per
  m block over the dummy functions of the element (``basis.cpp:2379-2397``).
* ``src/diatomic/dftgrid_purem.cpp:213-291,306-369``  density of each m block
  from the (m, m) sub-block of the dummy-expanded density; gradient
  components along mu and nu, divided by h.
* ``src/diatomic/dftgrid_purem.cpp:480-530,575-650``  the Fock increments
  w v_rho B B' (LDA) and X + X' with X = sum_c dB_c diag(w (2 v_ss g_c +
  v_ab g'_c) / h) B' (GGA); only (m, m) blocks are non-zero.
* ``src/diatomic/dftgrid_purem.cpp:668-712``  element/radial loop, energy and
  electron count, and the removal of the boundary functions.

The +m/-m mirroring of the reference is an optimisation that does not change
the numbers; every m block is evaluated here.
"""
from __future__ import annotations

import math

import numpy as np

from . import xc as xcmod
from .diatomic import DiatomicTables, MuBasis, get_grid, lm_maps, lm_to_l_m
from .tabulate import chebyshev, lip_eval, lobatto, theta_lm


def grid_tables(Z1: int, Z2: int, Rbond: float, nnodes: int, nelem: int, lmmax, Rmax: float = 40.0,
                igrid: int = 4, zexp: float = 1.0) -> DiatomicTables:
    """The basis geometry alone (no integrals): enough for the XC grid, whose
    inputs are the element boundaries, the angular functions and Rhalf."""
    Rhalf = 0.5 * Rbond
    bval = get_grid(math.acosh(Rmax / Rhalf), nelem, igrid, zexp)
    rb = MuBasis(nnodes, bval)
    lval, mval = lm_to_l_m(lmmax)
    lm, LM = lm_maps(lval, mval)
    first = np.array([rb.first(e) for e in range(rb.nel)])
    ni = np.array([len(rb.enabled(e)) for e in range(rb.nel)])
    return DiatomicTables(Z1, Z2, Rhalf, nnodes, np.asarray(bval, float), lval, mval, rb.nrad, first, ni, lm, LM,
                          [], [], [], [], [], [])


class PureMGrid:
    """(mu, nu) product grid per radial element with the phi integral done
    analytically (2 pi)."""

    def __init__(self, tab: DiatomicTables, lang: int = 0, nquad: int = 0):
        self.tab = tab
        self.lang = lang or 4 * int(np.max(tab.lval)) + 12
        self.nquad = nquad or 5 * tab.nnodes
        self.cth, self.wang = chebyshev(self.lang)
        self.xq, self.wq = chebyshev(self.nquad)
        self.x0, _ = lobatto(tab.nnodes)
        self.mlist = sorted(set(int(m) for m in tab.mval))
        c = self.cth
        sth = np.sqrt(np.maximum((1.0 - c) * (1.0 + c), 0.0))
        cot = np.where(sth > 0, c / np.where(sth > 0, sth, 1.0), 0.0)
        self.sth = sth
        self.Y = {}
        self.dY = {}
        for m in self.mlist:
            sh = [ia for ia in range(tab.nang) if int(tab.mval[ia]) == m]
            Y, dY = [], []
            for ia in sh:
                l = int(tab.lval[ia])
                y = theta_lm(l, m, c)
                d = m * cot * y
                if m < l:
                    d = d + math.sqrt((l - m) * (l + m + 1.0)) * theta_lm(l, m + 1, c)
                Y.append(y)
                dY.append(d)
            self.Y[m] = (sh, np.array(Y), np.array(dY))
        self._cache = {}

    def element(self, iel):
        if iel in self._cache:
            return self._cache[iel]
        tab = self.tab
        nn = tab.nnodes
        b0, b1 = tab.bval[iel], tab.bval[iel + 1]
        sf, mid = 0.5 * (b1 - b0), 0.5 * (b1 + b0)
        mu = mid + sf * self.xq
        wr = sf * self.wq
        en = np.arange(nn) if iel < tab.nel - 1 else np.arange(nn - 1)
        B = lip_eval(self.xq, self.x0, 0)[:, en]
        dB = lip_eval(self.xq, self.x0, 1)[:, en] / sf
        shmu = np.sinh(mu)
        s2 = shmu[:, None] ** 2 + self.sth[None, :] ** 2          # (nq, na)
        Rh = tab.Rhalf
        h = Rh * np.sqrt(s2)
        w = 2 * np.pi * self.wang[None, :] * wr[:, None] * Rh ** 3 * shmu[:, None] * s2
        first = int(tab.first[iel])
        blocks = []
        for m in self.mlist:
            sh, Y, dY = self.Y[m]
            # functions (shell s, radial j) x points (q, a)
            bf = np.einsum("sa,qj->sjqa", Y, B).reshape(len(sh) * len(en), -1)
            dr = np.einsum("sa,qj->sjqa", Y, dB).reshape(len(sh) * len(en), -1)
            dt = np.einsum("sa,qj->sjqa", dY, B).reshape(len(sh) * len(en), -1)
            idx = np.concatenate([ia * tab.nrad + first + en for ia in sh])
            blocks.append((m, idx, bf, dr, dt))
        res = dict(w=w.ravel(), h=h.ravel(), blocks=blocks)
        # keep small grids; large ones are rebuilt element by element
        if sum(b[2].nbytes for b in blocks) * 3 * tab.nel < 2e9:
            self._cache[iel] = res
        return res

    def mblocks(self):
        """{m: (pure positions, dummy indices)} of every symmetry block."""
        tab = self.tab
        pidx = tab.pure_indices()
        mv = tab.mval[pidx // tab.nrad]
        return {m: (np.where(mv == m)[0], pidx[mv == m]) for m in self.mlist}

    def eval_Fxc_blocks(self, names, Pa, Pb, thr=1e-12):
        """The (m, m) blocks only: Pa, Pb map m -> the block of the spin
        density over the block's pure functions (ascending pure index).
        Returns ({m: Ha_m}, {m: Hb_m}, Exc, Nel)."""
        tab = self.tab
        gga = any(xcmod.FUNCTIONALS[f][0] == "gga" for f in names)
        mb = self.mblocks()
        loc, Pae, Pbe, Hae, Hbe = {}, {}, {}, {}, {}
        for m, (_, dum) in mb.items():
            n = len(dum)
            lm = np.full(tab.ndummy, n)  # dropped boundary functions -> a zero row
            lm[dum] = np.arange(n)
            loc[m] = lm
            for src, dst in ((Pa, Pae), (Pb, Pbe)):
                X = np.zeros((n + 1, n + 1))
                X[:n, :n] = src[m]
                dst[m] = X
            Hae[m] = np.zeros((n + 1, n + 1))
            Hbe[m] = np.zeros((n + 1, n + 1))
        Exc = Nel = 0.0
        for iel in range(tab.nel):
            E = self.element(iel)
            w, h = E["w"], E["h"]
            ra = np.zeros_like(w)
            rb = np.zeros_like(w)
            ga = [np.zeros_like(w), np.zeros_like(w)]
            gb = [np.zeros_like(w), np.zeros_like(w)]
            for m, idx, bf, dr, dt in E["blocks"]:
                li = loc[m][idx]
                for P, rho, g in ((Pae[m], ra, ga), (Pbe[m], rb, gb)):
                    Pv = P[np.ix_(li, li)] @ bf
                    rho += np.sum(Pv * bf, axis=0)
                    if gga:
                        g[0] += 2 * np.sum(Pv * dr, axis=0) / h
                        g[1] += 2 * np.sum(Pv * dt, axis=0) / h
            Nel += float(np.sum(w * (ra + rb)))
            if gga:
                saa = ga[0] ** 2 + ga[1] ** 2
                sab = ga[0] * gb[0] + ga[1] * gb[1]
                sbb = gb[0] ** 2 + gb[1] ** 2
            else:
                saa = sab = sbb = None
            e, va, vb, vaa, vab, vbb = xcmod.eval_functionals(names, ra, rb, saa, sab, sbb, thr)
            Exc += float(np.sum(w * e))
            for H, v, gown, goth, vss in ((Hae, va, ga, gb, vaa), (Hbe, vb, gb, ga, vbb)):
                for m, idx, bf, dr, dt in E["blocks"]:
                    M = (bf * (w * v)) @ bf.T
                    if gga:
                        X = np.zeros_like(M)
                        for c, dbf in enumerate((dr, dt)):
                            coef = w * (2 * vss * gown[c] + vab * goth[c]) / h
                            X += (dbf * coef) @ bf.T
                        M += X + X.T
                    li = loc[m][idx]
                    H[m][np.ix_(li, li)] += M
        strip = lambda H: {m: X[:-1, :-1] for m, X in H.items()}
        return strip(Hae), strip(Hbe), Exc, Nel

    def eval_Fxc(self, names, Pa, Pb, thr=1e-12):
        """Return (Ha, Hb, Exc, Nel) in the pure basis for spin densities
        Pa, Pb given in the pure basis (only their (m, m) blocks enter)."""
        mb = self.mblocks()
        blk = lambda P: {m: P[np.ix_(pos, pos)] for m, (pos, _) in mb.items()}
        Hab, Hbb, Exc, Nel = self.eval_Fxc_blocks(names, blk(Pa), blk(Pb), thr)
        Ha = np.zeros_like(Pa)
        Hb = np.zeros_like(Pb)
        for m, (pos, _) in mb.items():
            Ha[np.ix_(pos, pos)] = Hab[m]
            Hb[np.ix_(pos, pos)] = Hbb[m]
        return Ha, Hb, Exc, Nel
