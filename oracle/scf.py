"""Oracle (test infrastructure only): atomic SCF driver.

Restates the caller pattern of the reference's Fock builder
(``src/atomic/main.cpp:369-470``): density assembly per symmetry block
(``src/general/scf_driver_common.h:406-425``), J from the total density, K
from the spin densities with the restricted shortcut
(``scf_driver_common.h:459-474``), XC from the DFT grid, the energy
decomposition (``main.cpp:410-446``) and per-block orthonormal Fock matrices
(``scf_driver_common.h:432-445,489-520``) built with ``utils::invh``
orthonormalisers (``scf_driver_common.h:176-187``).

The reference hands the state machine to OpenOrbitalOptimizer (DIIS, ODA,
CG). Converged energies do not depend on the convergence accelerator, so the
oracle uses plain Pulay DIIS with Aufbau occupations (or fixed per-block
occupations, the reference's ``--readocc``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import FockOracle
from . import tabulate as tab
from . import xc as xcmod


@dataclass
class SCFResult:
    Etot: float
    Ekin: float
    Enuc: float
    Ecoul: float
    Exx: float
    Exc: float
    iterations: int
    converged: bool
    Pa: np.ndarray
    Pb: np.ndarray
    eps: list


def sym_blocks(atom: tab.AtomTables):
    """Per-m blocks, unique m ascending (TwoDBasis.cpp:218-232, symmetry=1;
    diatomic: basis.cpp:906-918 over the pure functions)."""
    if hasattr(atom, "sym_blocks"):
        return atom.sym_blocks()
    n = atom.nrad
    out = []
    for m in sorted(set(int(x) for x in atom.mval)):
        idx = np.concatenate([ia * n + np.arange(n) for ia in range(atom.nang) if atom.mval[ia] == m])
        out.append((m, idx))
    return out


def _occupy(eps_blocks, nel, maxocc, fixed=None):
    """Aufbau over all blocks (or within blocks for fixed counts)."""
    occ = [np.zeros(len(e)) for e in eps_blocks]
    if fixed is not None:
        for k, nk in enumerate(fixed):
            left = nk
            for i in range(len(eps_blocks[k])):
                o = min(maxocc, left)
                occ[k][i] = o
                left -= o
                if left <= 0:
                    break
        return occ
    allv = sorted((e, k, i) for k, ev in enumerate(eps_blocks) for i, e in enumerate(ev))
    left = nel
    for e, k, i in allv:
        if left <= 0:
            break
        o = min(maxocc, left)
        occ[k][i] = o
        left -= o
    return occ


def run_scf(atom: tab.AtomTables, nela: int, nelb: int, method: str = "hf",
            restricted: bool = True, fixed_occ=None, fock: FockOracle = None,
            grid: xcmod.AtomGrid = None, maxiter: int = 200, conv: float = 1e-10,
            thr: float = 1e-12, verbose: bool = False, guess_H: np.ndarray = None,
            l_occ=None, gtol: float = 1e-7) -> SCFResult:
    """fixed_occ: dict m -> (nocc_alpha, nocc_beta) (restricted: total/2 each).
    guess_H: one-electron Hamiltonian whose orbitals start the SCF (default
    the core Hamiltonian T + V; T + a screened-nucleus model potential is
    the reference's iguess 1-3, src/atomic/main.cpp:474-511).
    l_occ: [(n_alpha, n_beta) per l] switches to one block per angular
    function with fixed occupations: the electrons of each l shared equally
    over its 2l+1 m blocks and filled lowest-first within a block (the
    spherically averaged occupations of the engine's batch and serving
    solves; symmetry 2 of the reference's atomic driver).
    Converged when the energy change is below conv and the largest element
    of the orthonormal-basis commutator F P S - S P F is below gtol."""
    fock = fock or FockOracle(atom)
    names = xcmod.parse_method(method)
    have_xc = bool(names)
    have_exx = not have_xc
    if have_xc and grid is None:
        grid = xcmod.AtomGrid(atom)
    H = atom.T + atom.V
    S = atom.S
    if l_occ is not None:
        n = atom.nrad
        blocks = [(ia, ia * n + np.arange(n)) for ia in range(atom.nang)]
    else:
        blocks = sym_blocks(atom)
    X = [tab.invh(S[np.ix_(idx, idx)]) for _, idx in blocks]
    nspin = 1 if restricted else 2
    maxocc = 2.0 if restricted else 1.0
    nel_spin = [nela + nelb] if restricted else [nela, nelb]
    fixed = None
    if l_occ is not None:
        per = [[l_occ[atom.lval[ia]][sp] / (2 * atom.lval[ia] + 1) if atom.lval[ia] < len(l_occ) else 0.0
                for ia in range(atom.nang)] for sp in range(2)]
        fixed = [[a + b for a, b in zip(per[0], per[1])]] if restricted else per
    elif fixed_occ is not None:
        if restricted:
            fixed = [[fixed_occ.get(m, (0, 0))[0] + fixed_occ.get(m, (0, 0))[1] for m, _ in blocks]]
        else:
            fixed = [[fixed_occ.get(m, (0, 0))[s] for m, _ in blocks] for s in range(2)]

    def diag(F):
        eps, C = [], []
        for (m, idx), Xk in zip(blocks, X):
            Fo = Xk.T @ F[np.ix_(idx, idx)] @ Xk
            e, v = np.linalg.eigh(Fo)
            eps.append(e)
            C.append(Xk @ v)
        return eps, C

    def density(eps, C, s):
        occ = _occupy(eps, nel_spin[s], maxocc, None if fixed is None else fixed[s])
        P = np.zeros_like(S)
        for (m, idx), Ck, ok in zip(blocks, C, occ):
            P[np.ix_(idx, idx)] += (Ck * ok) @ Ck.T
        return P

    eps0, C0 = diag(H if guess_H is None else guess_H)
    state = [(eps0, C0)] * nspin
    diis_F, diis_e = [], []
    Eold = 0.0
    converged = False
    res = None
    for it in range(1, maxiter + 1):
        Ps = [density(*state[s], s) for s in range(nspin)]
        if restricted:
            P = Ps[0]
            Pa = Pb = 0.5 * P
        else:
            Pa, Pb = Ps
            P = Pa + Pb
        J = fock.coulomb(P)
        Ekin = float(np.sum(P * atom.T))
        Enuc = float(np.sum(P * atom.V))
        Ecoul = 0.5 * float(np.sum(P * J))
        Exx = Exc = 0.0
        Fa = H + J
        Fb = H + J
        if have_exx:
            Ka = fock.exchange(Pa)
            Exx = 0.5 * float(np.sum(Pa * Ka))
            if restricted:
                Exx *= 2
                Kb = Ka
            else:
                Kb = fock.exchange(Pb)
                Exx += 0.5 * float(np.sum(Pb * Kb))
            Fa = Fa + Ka
            Fb = Fb + Kb
        if have_xc:
            XCa, XCb, Exc, _ = grid.eval_Fxc(names, Pa, Pb, thr)
            Fa = Fa + XCa
            Fb = Fb + XCb
        E = Ekin + Enuc + Ecoul + Exx + Exc
        res = SCFResult(E, Ekin, Enuc, Ecoul, Exx, Exc, it, False, Pa, Pb, [s[0] for s in state])
        Fs = [Fa] if restricted else [Fa, Fb]
        Pspin = [P] if restricted else [Pa, Pb]
        errs = []
        for F, Pk in zip(Fs, Pspin):
            comm = F @ Pk @ S - S @ Pk @ F
            errs.append(np.concatenate([(Xk.T @ comm[np.ix_(idx, idx)] @ Xk).ravel()
                                        for (m, idx), Xk in zip(blocks, X)]))
        err = np.concatenate(errs)
        emax = float(np.max(np.abs(err)))
        if verbose:
            print(f"it {it:3d} E {E:.12f} dE {E - Eold: .3e} err {emax:.3e}")
        if it > 1 and abs(E - Eold) < conv and emax < gtol:
            converged = True
            res.converged = True
            break
        Eold = E
        diis_F.append([F.copy() for F in Fs])
        diis_e.append(err)
        if len(diis_F) > 10:
            diis_F.pop(0)
            diis_e.pop(0)
        n = len(diis_F)
        B = -np.ones((n + 1, n + 1))
        B[n, n] = 0.0
        for i in range(n):
            for j in range(n):
                B[i, j] = diis_e[i] @ diis_e[j]
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        try:
            c = np.linalg.solve(B, rhs)[:n]
        except np.linalg.LinAlgError:
            c = np.zeros(n)
            c[-1] = 1.0
        Fext = [sum(c[i] * diis_F[i][s] for i in range(n)) for s in range(nspin)]
        state = [diag(Fext[s]) for s in range(nspin)]
    return res
