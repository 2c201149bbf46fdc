"""The diatomic oracle against the reference's own numbers: Maple values of
the associated Legendre functions for x > 1, the modified Gaunt goldens of
src/general/gaunt_test.cpp, and converged diatomic HF energies recorded by
the reference's test harness (tests/refs/ci.json)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import DiatomicOracle
from oracle import diatomic as dia
from oracle import scf

HERE = os.path.dirname(os.path.abspath(__file__))
G = json.load(open(os.path.join(HERE, "golden", "diatomic.json")))
GAUNT = json.load(open(os.path.join(HERE, "golden", "gaunt.json")))
SCF = {c["name"]: c for c in G["scf"]}


def test_legendre_golden():
    byx = {}
    for e in G["legendre"]:
        byx.setdefault(e["x"], []).append(e)
    for xs, es in byx.items():
        P, Q = dia.legendre_pq(40, 8, np.array([math.acosh(float(xs))]))
        for e in es:
            p, q = float(e["P"]), float(e["Q"])
            assert abs(P[e["m"], e["l"], 0] - p) <= 1e-12 * abs(p) + 1e-300, (xs, e)
            if abs(q) > 1e-280:
                assert abs(Q[e["m"], e["l"], 0] - q) <= 1e-12 * abs(q), (xs, e)


def test_mod_coeff_golden():
    for g in GAUNT:
        if g["fn"] != "mod_coeff":
            continue
        v = dia.mod_coeff(*g["args"])
        assert abs(v - g["ref"]) <= 2.2e-16 * (1 + abs(g["ref"])) * 8, g


def run_case(name):
    a = SCF[name]["args"]
    lm = [int(x) for x in a["lmax"].split(",")]
    Z1, Z2, R = int(a["Z1"]), int(a["Z2"]), float(a["Rbond"])
    D = dia.build_diatomic(Z1, Z2, R, int(a["nnodes"]), int(a["nelem"]), lm)
    restricted = a.get("restricted", "1") != "0"
    r = scf.run_scf(D, int(a["nela"]), int(a["nelb"]), "hf", restricted=restricted, fock=DiatomicOracle(D),
                    conv=1e-12, maxiter=80)
    return r, Z1 * Z2 / R


@pytest.mark.parametrize("name", ["diatomic-H2-hf-r", "diatomic-H2-hf-u", "diatomic-He-dummy-hf"])
def test_diatomic_hf_energy(name):
    r, enuc = run_case(name)
    ref = SCF[name]["ref"]
    assert r.converged
    assert abs(r.Etot + enuc - ref["total"]) < 2e-9, (r.Etot + enuc, ref["total"])
    # the recorded components carry the reference's SCF stopping error
    # (its own restricted/unrestricted and symmetry variants differ at 1e-5)
    for k, v in (("kinetic", r.Ekin), ("nuclear", r.Enuc), ("Coulomb", r.Ecoul), ("Exx", r.Exx)):
        assert abs(v - ref[k]) < 1e-5 * max(1.0, abs(ref[k])), (k, v, ref[k])


@pytest.mark.slow
def test_diatomic_ne_dummy_hf_energy():
    r, enuc = run_case("diatomic-Ne-dummy-hf")
    assert abs(r.Etot + enuc - SCF["diatomic-Ne-dummy-hf"]["ref"]["total"]) < 2e-9


def test_in_element_factor_reproduces_kernel():
    """B diag(sigma) B' reproduces the 2-channel in-element kernel W to the
    1e-12 relative threshold, and the quadrature is converged."""
    rb = dia.MuBasis(15, dia.get_grid(math.acosh(40 / 0.7), 3, 4, 1.0))
    for e in range(3):
        for M in (0, 1, 3):
            T = rb.twoe(e, 10, M, [M + 2, 9])
            T2 = rb.twoe(e, 10, M, [M + 2, 9], n_out=96, n_in=96)
            for L in (M + 2, 9):
                W = np.block([[T[L][0], -T[L][1]], [-T[L][1].T, T[L][2]]])
                W2 = np.block([[T2[L][0], -T2[L][1]], [-T2[L][1].T, T2[L][2]]])
                assert np.abs(W - W2).max() < 1e-13 * np.abs(W).max()
                W = 0.5 * (W + W.T)
                B, s = dia._sign_cholesky(W)
                assert np.abs(B @ np.diag(s) @ B.T - W).max() < 1e-11 * np.abs(W).max()
