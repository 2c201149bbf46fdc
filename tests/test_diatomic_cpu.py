"""Diatomic host side of the product (no GPU): its Legendre functions and
cos^2 couplings against the reference's goldens, and its tabulation (disjoint
P/Q integrals, in-element factor, one-electron matrices) against the oracle's
independent tabulation."""
import json
import math
import os

import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import diatomic as dia

HERE = os.path.dirname(os.path.abspath(__file__))
G = json.load(open(os.path.join(HERE, "golden", "diatomic.json")))
GAUNT = json.load(open(os.path.join(HERE, "golden", "gaunt.json")))


def test_product_legendre_golden():
    byx = {}
    for e in G["legendre"]:
        byx.setdefault(e["x"], []).append(e)
    for xs, es in byx.items():
        P, Q = hg.legendre_pq(40, 8, math.acosh(float(xs)))
        for e in es:
            p, q = float(e["P"]), float(e["Q"])
            assert abs(P[e["m"], e["l"]] - p) <= 1e-12 * abs(p) + 1e-300, (xs, e)
            if abs(q) > 1e-280:
                assert abs(Q[e["m"], e["l"]] - q) <= 1e-12 * abs(q), (xs, e)


def test_product_mod_coeff_golden():
    for g in GAUNT:
        if g["fn"] == "mod_coeff":
            v = hg.gaunt_mod(*g["args"])
            assert abs(v - g["ref"]) <= 8 * 2.2e-16 * (1 + abs(g["ref"])), g


@pytest.mark.parametrize("case", [(1, 1, 1.4, [4]), (7, 8, 2.17, [4, 3, 2])])
def test_tabulation_matches_oracle(case):
    Z1, Z2, R, lm = case
    d = hg.Diatomic.from_grid(Z1, Z2, R, 3, lm, host_only=True)
    D = dia.build_diatomic(Z1, Z2, R, 15, 3, lm)
    assert d.nbf == D.nbf and d.dims["nlm"] == len(D.lm)
    assert np.array_equal(d.pure_indices(), D.pure_indices())
    nn = 15
    for ilm, (L, M) in enumerate(D.lm):
        for e in range(D.nel):
            ni = D.ni[e]
            for which, name in enumerate(["P0", "P2", "Q0", "Q2"]):
                if e == 0 and which >= 2:
                    continue  # never used (element 0 is never the outer one)
                L2, M2, t = d.tables(which, ilm, e)
                assert (L2, M2) == (L, M)
                ref = getattr(D, name)[ilm][e]
                assert np.abs(t[:ni, :ni] - ref).max() <= 1e-12 * np.abs(ref).max()
            _, _, B, s = d.tables(4, ilm, e)
            Bo, so = D.cdB[ilm][e], D.cds[ilm][e]
            assert B.shape[1] == Bo.shape[1]
            idx = np.array([a + b * nn for b in range(ni) for a in range(ni)])
            full = np.concatenate([idx, nn * nn + idx])
            W = (B @ np.diag(s) @ B.T)[np.ix_(full, full)]
            Wo = Bo @ np.diag(so) @ Bo.T
            assert np.abs(W - Wo).max() <= 1e-12 * np.abs(Wo).max()
    for mine, ref in ((d.overlap(), D.S), (d.kinetic(), D.T), (d.nuclear(), D.V)):
        assert np.abs(mine - ref).max() <= 1e-12 * np.abs(ref).max()
    for m in sorted(set(int(x) for x in D.mval)):
        (_, idx), = [(mm, ix) for mm, ix in D.sym_blocks() if mm == m]
        Sb = d.one_electron_block("S", m)
        assert np.abs(Sb - D.S[np.ix_(idx, idx)]).max() <= 1e-12 * np.abs(D.S).max()


def test_diatomic_bad_arguments():
    with pytest.raises(hg.HfgError):
        hg.Diatomic(1, 1, 0.7, [0.0, 1.0], [0], [0], host_only=True)  # one element
    with pytest.raises(hg.HfgError):
        hg.Diatomic(1, 1, 0.7, [0.1, 1.0, 2.0], [0], [0], host_only=True)  # first boundary not 0
    with pytest.raises(hg.HfgError):
        hg.Diatomic(1, 1, 0.7, [0.0, 1.0, 2.0], [1], [2], host_only=True)  # |m| > l
    d = hg.Diatomic(1, 1, 0.7, [0.0, 1.0, 2.0], [0], [0], host_only=True)
    with pytest.raises(hg.HfgError):
        d.coulomb_host(np.zeros((d.nbf, d.nbf)))  # host-only handle


def test_diatomic_tabulation_mode_checked():
    import ctypes
    with pytest.raises(ValueError):
        hg.Diatomic(1, 1, 0.7, [0.0, 1.0, 2.0], [0], [0], tabulate="gpu")
    # the C ABI refuses an unknown host_only mode before any device work
    b = np.array([0.0, 1.0, 2.0])
    lv = np.array([0], np.int32)
    mv = np.array([0], np.int32)
    desc = hg._DDesc(1, 1, 0.7, 5, 2, hg._dptr(b), 1, lv.ctypes.data_as(hg._I), mv.ctypes.data_as(hg._I), 0.0, 3)
    h = hg._P()
    assert hg._lib.hfg_diatomic_create(ctypes.byref(desc), ctypes.byref(h)) != 0
    assert not h.value
