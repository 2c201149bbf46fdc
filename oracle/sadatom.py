"""Oracle (test infrastructure, never product code) for the Fock build of
the spherically averaged atom, src/sadatom/basis.cpp:186-429.

Two independent routes, both in FP64:

* a restatement of the reference's formulas on the radial tables of
  `tabulate.build_atom` (rs, rb and the pivoted-Cholesky factors per
  multipole and element):
    J       = 4 pi J_0[P]                                   basis.cpp:186-207
    K[lout] = -sum_L K_L[sum_lin (4 pi/(2L+1)) c(lout, lin, L) P[lin]]
              c = (2 lout + 1)^-1 sum_{mout, min} Gaunt(lout, mout, L, mout - min, lin)^2
                                                            basis.cpp:209-312
  with the single-multipole assemblies J_L, K_L of
  libhelfemqc/include/CoulombExchangeFE.h:432-530;
* the atomic oracle (`FockOracle`, pinned to the reference's goldens) on a
  full (l, m) basis: K[l] is the m-average of the diagonal (l m, l m) blocks
  of the atomic K of the density that repeats P[l] on every m, and J is 4 pi
  times the atomic J of an s-only basis.
"""
from __future__ import annotations

import math

import numpy as np

from . import FockOracle
from . import tabulate as tab


def channel_average(lout: int, lin: int, L: int) -> float:
    """c(lout, lin, L) of basis.cpp:246-268."""
    c = 0.0
    for mo in range(-lout, lout + 1):
        for mi in range(-lin, lin + 1):
            M = mo - mi
            if abs(M) > L:
                continue
            g = tab.gaunt(lout, mo, L, M, lin)
            c += g * g
    return c / (2 * lout + 1)


def _blocks(A: tab.AtomTables):
    rad = A.rad
    return [(int(rad.first[e]), int(rad.last[e]) + 1) for e in range(rad.nel)]


def J_L(A: tab.AtomTables, L: int, X: np.ndarray) -> np.ndarray:
    """Single-multipole Coulomb assembly (CoulombExchangeFE.h:432-482)."""
    blk = _blocks(A)
    nel = len(blk)
    out = np.zeros_like(X)
    for j, (f, l) in enumerate(blk):
        Xs = X[f:l, f:l]
        small = float(np.trace(A.rs[L][j] @ Xs))
        big = float(np.trace(A.rb[L][j] @ Xs)) if j > 0 else 0.0
        for i in range(j):
            fi, li = blk[i]
            out[fi:li, fi:li] += big * A.rs[L][i]
        for i in range(j + 1, nel):
            fi, li = blk[i]
            out[fi:li, fi:li] += small * A.rb[L][i]
        C = A.chol[L][j]
        n = l - f
        out[f:l, f:l] += (C @ (C.T @ Xs.ravel(order="F"))).reshape((n, n), order="F")
    return out


def K_L(A: tab.AtomTables, L: int, X: np.ndarray) -> np.ndarray:
    """Single-multipole exchange assembly (CoulombExchangeFE.h:484-530)."""
    blk = _blocks(A)
    out = np.zeros_like(X)
    for i, (fi, li) in enumerate(blk):
        for j, (fj, lj) in enumerate(blk):
            Xs = X[fi:li, fj:lj]
            if i == j:
                C = A.chol[L][i]
                n = li - fi
                acc = np.zeros_like(Xs)
                for p in range(C.shape[1]):
                    Mp = C[:, p].reshape((n, n), order="F")
                    acc += Mp @ (Xs @ Mp.T)
                out[fi:li, fj:lj] += acc
            else:
                a = A.rb[L][i] if i > j else A.rs[L][i]
                b = A.rs[L][j] if i > j else A.rb[L][j]
                out[fi:li, fj:lj] += a @ (Xs @ b.T)
    return out


def coulomb(A: tab.AtomTables, P: np.ndarray) -> np.ndarray:
    """sadatom TwoDBasis::coulomb (basis.cpp:186-207)."""
    return 4.0 * math.pi * J_L(A, 0, P)


def exchange(A: tab.AtomTables, P: list) -> list:
    """sadatom TwoDBasis::exchange (basis.cpp:209-312); P is one nrad x nrad
    matrix per l = 0..lmax. With A's tables replaced by screened ones
    (`yukawa.yukawa_tables`) this is rs_exchange (basis.cpp:314-429)."""
    lmax = len(P) - 1
    nrad = P[0].shape[0]
    K = []
    for lout in range(lmax + 1):
        Prad = {}
        for lin in range(lmax + 1):
            if np.linalg.norm(P[lin]) == 0.0:
                continue
            for L in range(abs(lin - lout), lin + lout + 1):
                c = channel_average(lout, lin, L)
                if c == 0.0:
                    continue
                Prad[L] = Prad.get(L, np.zeros((nrad, nrad))) + (4.0 * math.pi / (2 * L + 1) * c) * P[lin]
        Kl = np.zeros((nrad, nrad))
        for L, X in sorted(Prad.items()):
            Kl -= K_L(A, L, X)
        K.append(Kl)
    return K


def coulomb_via_atomic(A_s: tab.AtomTables, P: np.ndarray) -> np.ndarray:
    """4 pi times the atomic J of an s-only basis (the same radial tables)."""
    return 4.0 * math.pi * FockOracle(A_s).coulomb(P)


def exchange_via_atomic(A_full: tab.AtomTables, P: list) -> list:
    """m-average of the diagonal blocks of the atomic K of the density that
    repeats P[l] on every m of the full (l, m) basis A_full."""
    nrad = P[0].shape[0]
    lv = np.asarray(A_full.lval)
    nbf = nrad * len(lv)
    Pf = np.zeros((nbf, nbf))
    for ia, l in enumerate(lv):
        s = slice(ia * nrad, (ia + 1) * nrad)
        Pf[s, s] = P[l]
    Kf = FockOracle(A_full).exchange(Pf)
    out = []
    for l in range(len(P)):
        acc = np.zeros((nrad, nrad))
        for ia in np.where(lv == l)[0]:
            s = slice(ia * nrad, (ia + 1) * nrad)
            acc += Kf[s, s]
        out.append(acc / (2 * l + 1))
    return out


def channel_densities(A_full: tab.AtomTables, P: np.ndarray, lmax: int) -> list:
    """P_l = sum over the m of l of the diagonal blocks of a full-basis
    density (the reference SCF's per-channel density, scf.cpp:125-136)."""
    nrad = A_full.nrad
    lv = np.asarray(A_full.lval)
    out = []
    for l in range(lmax + 1):
        acc = np.zeros((nrad, nrad))
        for ia in np.where(lv == l)[0]:
            s = slice(ia * nrad, (ia + 1) * nrad)
            acc += P[s, s]
        out.append(acc)
    return out


def fock_energies(J_fn, K_fn, T: list, V: np.ndarray, Pl: list, restricted: bool = True) -> dict:
    """Energy terms of the reference's spherically averaged Fock build
    (src/sadatom/scf.cpp:155-233) for channel densities Pl (total
    electrons per channel): J from Prad / 4 pi, K from Pl / (2 (2l+1)),
    Ekin from the channel kinetic matrices T[l] (with l(l+1) Tl included)."""
    Prad = sum(Pl)
    J = J_fn(Prad / (4.0 * math.pi))
    ang = [Pl[l] / ((2.0 if restricted else 1.0) * (2 * l + 1)) for l in range(len(Pl))]
    K = K_fn(ang)
    e = {"Ekin": sum(float(np.sum(Pl[l] * T[l])) for l in range(len(Pl))),
         "Enuc": float(np.sum(Prad * V)),
         "Ecoul": 0.5 * float(np.sum(Prad * J)),
         "Exx": 0.5 * sum(float(np.sum(K[l] * Pl[l])) for l in range(len(Pl)))}
    e["Etot"] = e["Ekin"] + e["Enuc"] + e["Ecoul"] + e["Exx"]
    return e
