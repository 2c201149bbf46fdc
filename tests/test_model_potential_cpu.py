"""Screened-nucleus model potential (the reference's TwoDBasisT::
model_potential with TFAtom, iguess 3) through the product's host tables
against the oracle's independent quadrature, and the Thomas-Fermi guess in
the oracle's SCF: it starts elsewhere but converges to the reference's
pinned energies."""
import json
import os

import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import guess, scf
from oracle import tabulate as tab

HERE = os.path.dirname(os.path.abspath(__file__))
CI = {c["name"]: c for c in json.load(open(os.path.join(HERE, "golden", "ci_energies.json")))}


@pytest.mark.parametrize("Z,lmax,nelem,nnodes", [(2, 0, 5, 15), (10, 1, 8, 15), (36, 2, 12, 13), (54, 2, 6, 17)])
def test_thomas_fermi_matrix_matches_oracle(Z, lmax, nelem, nnodes):
    b = tab.get_grid(40.0, nelem, 4, 2.0)
    lv, mv = hg.angular_basis(lmax, lmax)
    A = hg.Atom(Z, b, lv, mv, nnodes=nnodes, host_only=True)
    V = A.model_potential(3)
    O = tab.build_atom(Z, nnodes, b, lmax, lmax)
    Vo = guess.thomas_fermi_matrix(O)
    assert np.abs(V - Vo).max() <= 1e-12 * np.abs(Vo).max()
    # screening: between the bare nucleus and zero, on the diagonal
    Vn = A.nuclear()
    d, dn = np.diag(V), np.diag(Vn)
    assert np.all(d <= 0) and np.all(d >= dn - 1e-12 * np.abs(dn).max())


def test_thomas_fermi_charge_limits():
    r = np.array([1e-12, 1e-6, 1.0, 10.0, 100.0])
    for Z in (1, 10, 86):
        z = guess.thomas_fermi_charge(r, Z)
        assert abs(z[0] - Z) < 1e-4 * Z and np.all(np.diff(z) < 0) and z[-1] < 1e-3 * Z


def test_unavailable_models_are_argument_errors():
    b = tab.get_grid(40.0, 3, 4, 2.0)
    A = hg.Atom(2, b, [0], [0], host_only=True)
    for model in (0, 1, 2, 4):
        with pytest.raises(hg.HfgError) as e:
            A.model_potential(model)
        assert e.value.status == hg.HFG_ERR_ARG


@pytest.mark.parametrize("name,Z", [("atomic-He-hf-r", 2), ("atomic-Be-hf-r", 4)])
def test_thomas_fermi_guess_reaches_pinned_energy(name, Z):
    b = tab.get_grid(40.0, 5, 4, 2.0)
    O = tab.build_atom(Z, 15, b, 0, 0)
    Vg = guess.thomas_fermi_matrix(O)
    r = scf.run_scf(O, Z // 2, Z // 2, "hf", guess_H=O.T + Vg)
    assert r.converged
    assert abs(r.Etot - CI[name]["total"]) < 1e-8
