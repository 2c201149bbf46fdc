"""Spherically averaged atom (src/sadatom/basis.cpp:186-429) on the CPU:
the oracle's restatement of the reference's J and K against the atomic
oracle through exact identities, the reference's Ne Hartree-Fock energy
(tests/README.md, -128.5470981094 Eh) recovered from the restated Fock
build at the converged closed-shell density, and the product's host-side
handle (dimensions, argument checks)."""
import math

import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import sadatom as sad
from oracle import scf as oscf
from oracle import tabulate as tab

NE_GOLDEN = -128.5470981094


def channel_density(nrad, nocc, seed):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((nrad, nocc))
    return C @ C.T


@pytest.mark.parametrize("lmax", [0, 1, 2, 3])
def test_restatement_matches_atomic_identities(lmax):
    bval = tab.get_grid(30.0, 3, 4, 2.0)
    A = tab.build_atom(8, 6, bval, lmax, 0)           # (l, 0) channels
    Af = tab.build_atom(8, 6, bval, lmax, lmax)       # full (l, m) basis
    As = tab.build_atom(8, 6, bval, 0, 0)             # s only
    P = [channel_density(A.nrad, 3, 10 + l) for l in range(lmax + 1)]
    J1 = sad.coulomb(A, sum(P))
    J2 = sad.coulomb_via_atomic(As, sum(P))
    assert np.abs(J1 - J2).max() <= 1e-12 * np.abs(J2).max()
    K1 = sad.exchange(A, P)
    K2 = sad.exchange_via_atomic(Af, P)
    scale = max(np.abs(k).max() for k in K2)
    for l in range(lmax + 1):
        assert np.abs(K1[l] - K2[l]).max() <= 1e-12 * scale, l


def test_channel_average_sum_rule():
    # closure of the Gaunt coefficients: sum_{L, M} G(lout, mout, L, M, lin)^2
    # = (2 lin + 1)/(4 pi) for every mout, hence for the m-average too
    for lout in range(4):
        for lin in range(4):
            tot = sum(sad.channel_average(lout, lin, L) for L in range(abs(lout - lin), lout + lin + 1))
            assert abs(tot - (2 * lin + 1) / (4 * math.pi)) < 1e-14


def test_restated_fock_build_recovers_ne_energy():
    bval = tab.get_grid(40.0, 5, 4, 2.0)
    Af = tab.build_atom(10, 15, bval, 1, 1)
    res = oscf.run_scf(Af, 5, 5, "hf")
    assert res.converged and abs(res.Etot - NE_GOLDEN) < 1e-8
    A = tab.build_atom(10, 15, bval, 1, 0)
    nr = A.nrad
    Pl = sad.channel_densities(Af, res.Pa + res.Pb, 1)
    T = [A.T[l * nr:(l + 1) * nr, l * nr:(l + 1) * nr] for l in range(2)]
    V = A.V[:nr, :nr]
    e = sad.fock_energies(lambda P: sad.coulomb(A, P), lambda P: sad.exchange(A, P), T, V, Pl)
    for k in ("Ekin", "Enuc", "Ecoul", "Exx", "Etot"):
        assert abs(e[k] - getattr(res, k)) < 1e-9 * max(1.0, abs(getattr(res, k))), k
    assert abs(e["Etot"] - NE_GOLDEN) < 1e-8


def test_sadatom_handle_host_side():
    a = hg.SadAtom.from_grid(10, 5, 40.0, 2, host_only=True)
    assert (a.nang, a.NL, a.nbf) == (3, 5, 3 * a.nrad)
    assert list(a.lval) == [0, 1, 2] and not a.mval.any()
    with pytest.raises(hg.HfgError):
        a.coulomb_host(np.zeros((a.nrad, a.nrad)))  # host-only handle
    with pytest.raises(hg.HfgError):
        hg.SadAtom.from_grid(10, 5, 40.0, 4, host_only=True)  # lmax above 3
    with pytest.raises(ValueError):
        hg.SadAtom.from_grid(10, 5, 40.0, 1, tabulate="gpu")
    b = hg.Atom.from_grid(10, 5, 40.0, 1, 1, host_only=True)
    with pytest.raises(hg.HfgError):
        hg._check(hg._lib.hfg_sadatom_coulomb_host(b._h, hg._dptr(np.zeros(1)), hg._dptr(np.zeros(1))))
