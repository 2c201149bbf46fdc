"""CPU-side checks of the product library (no GPU compute calls):
exported symbols, Gaunt goldens through the C ABI, host tabulation against
the independent oracle tabulation, and error reporting."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import tabulate as tab

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def declared_symbols():
    syms = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            syms |= set(re.findall(r"\b(hfg_\w+)\s*\(", src))
    return syms


def test_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) > 10
    missing = [s for s in sorted(syms) if not hasattr(hg.lib(), s)]
    assert not missing, missing


def test_gaunt_golden_through_capi():
    eps = np.finfo(float).eps
    for g in json.load(open(os.path.join(HERE, "golden", "gaunt.json"))):
        if g["fn"] != "coeff":
            continue
        L, M, l, m, lp, mp = g["args"]
        v = hg.gaunt(L, M, l, m, lp) if mp == M - m else 0.0
        assert abs(v - g["ref"]) < eps * (1 + abs(g["ref"])), (g, v)


@pytest.mark.parametrize("Z,lmax,mmax,nelem,nnodes", [(10, 1, 1, 5, 15), (36, 2, 2, 6, 10), (4, 0, 0, 3, 17)])
def test_host_tabulation_matches_oracle(Z, lmax, mmax, nelem, nnodes):
    b = tab.get_grid(40.0, nelem, 4, 2.0)
    lv, mv = hg.angular_basis(lmax, mmax)
    A = hg.Atom(Z, b, lv, mv, nnodes=nnodes, host_only=True)
    O = tab.build_atom(Z, nnodes, b, lmax, mmax)
    assert (A.nrad, A.nbf) == (O.nrad, O.nbf)
    for L in range(O.NL):
        for e in range(O.rad.nel):
            rs, rb, ch = A.radial_tables(L, e)
            assert np.allclose(rs, O.rs[L][e], rtol=0, atol=1e-12 * np.abs(rs).max())
            if e > 0:
                assert np.allclose(rb, O.rb[L][e], rtol=0, atol=1e-12 * np.abs(rb).max())
            T = ch @ ch.T
            To = O.chol[L][e] @ O.chol[L][e].T
            assert np.abs(T - To).max() < 1e-11 * np.abs(To).max()
    for f, ref in ((A.overlap, O.S), (A.kinetic, O.T), (A.nuclear, O.V)):
        M = f()
        assert np.abs(M - ref).max() < 1e-11 * np.abs(ref).max()


def test_grid_and_angular_basis_match_reference_conventions():
    for igrid, z in ((1, 1.0), (2, 1.0), (3, 2.0), (4, 2.0), (4, 1.0), (5, 0.5)):
        assert np.allclose(hg.get_grid(40.0, 7, igrid, z), tab.get_grid(40.0, 7, igrid, z), rtol=1e-14, atol=0)
    lv, mv = hg.angular_basis(3, 2)
    lo, mo = tab.angular_basis(3, 2)
    assert list(lv) == list(lo) and list(mv) == list(mo)


def test_errors_are_status_codes():
    b = tab.get_grid(40.0, 3, 4, 2.0)
    with pytest.raises(hg.HfgError) as e:
        hg.Atom(2, b, [0], [1], host_only=True)  # |m| > l
    assert e.value.status == hg.HFG_ERR_ARG
    with pytest.raises(hg.HfgError) as e:
        hg.Atom(2, b[:1], [0], [0], host_only=True)
    assert e.value.status == hg.HFG_ERR_ARG
    with pytest.raises(hg.HfgError) as e:
        hg.Atom(2, b, [0], [0], nnodes=40, host_only=True)
    assert e.value.status == hg.HFG_ERR_ARG
    A = hg.Atom(2, b, [0], [0], host_only=True)
    with pytest.raises(hg.HfgError) as e:
        A.coulomb(0, 0, 0)
    assert e.value.status in (hg.HFG_ERR_ARG, hg.HFG_ERR_STATE)
    with pytest.raises(hg.HfgError) as e:
        A.coulomb(1 << 20, 1 << 21, 0)
    assert e.value.status == hg.HFG_ERR_STATE


def test_creation_modes_are_validated():
    """host_only selects the tabulation: 0 device, 1 host-only handle, 2 host
    tables uploaded; anything else is an argument error before any work."""
    b = tab.get_grid(40.0, 3, 4, 2.0)
    lv = np.array([0], dtype=np.int32)
    d = hg._Desc(2, 15, 0, len(b) - 1, hg._dptr(b), 1, lv.ctypes.data_as(hg._I), lv.ctypes.data_as(hg._I),
                 0.0, 3)
    h = hg._P()
    assert hg._lib.hfg_atom_create(ctypes.byref(d), ctypes.byref(h)) == hg.HFG_ERR_ARG
    assert "host_only" in hg._lib.hfg_last_error().decode()
    with pytest.raises(ValueError):
        hg.Atom(2, b, [0], [0], tabulate="gpu")
    A = hg.Atom(2, b, [0], [0], host_only=True, tabulate="host")  # host-only wins
    rs, rb, ch = A.radial_tables(0, 1)
    assert ch.shape[1] >= 1 and np.isfinite(ch).all()


def test_madelung_l_occupations():
    from helfem_gb300 import workloads as wl
    occ = wl.l_occupations(13, 13, 2)  # Fe: [Ar] 4s2 3d6 restricted-averaged -> 13 per spin
    assert occ.tolist() == [[4, 4], [6, 6], [3, 3]]
    occ = wl.l_occupations(5, 3, 1)  # O
    assert occ.tolist() == [[2, 2], [3, 1]]
    assert wl.l_occupations(1, 0, 0).tolist() == [[1, 0]]
