"""The oracle's SCF with spherically averaged per-l occupations on one block
per angular function (the occupations the engine's batch and serving solves
use): for closed shells it must reproduce the per-m Aufbau solution, and
for Be the reference's pinned energy."""
import json
import os

import pytest

from oracle import scf
from oracle import tabulate as tab

HERE = os.path.dirname(os.path.abspath(__file__))
CI = {c["name"]: c for c in json.load(open(os.path.join(HERE, "golden", "ci_energies.json")))}


def test_be_pinned_energy():
    b = tab.get_grid(40.0, 5, 4, 2.0)
    A = tab.build_atom(4, 15, b, 0, 0)
    r = scf.run_scf(A, 2, 2, "hf", l_occ=[(2, 2)])
    assert r.converged and abs(r.Etot - CI["atomic-Be-hf-r"]["total"]) < 1e-8


@pytest.mark.parametrize("Z,lmax,l_occ,method,nelem", [
    (10, 1, [(2, 2), (3, 3)], "hf", 8),
    (18, 1, [(3, 3), (6, 6)], "hf", 8),
    (4, 0, [(2, 2)], "lda_x-lda_c_pw", 4),
])
def test_closed_shell_equals_aufbau(Z, lmax, l_occ, method, nelem):
    b = tab.get_grid(40.0, nelem, 4, 2.0)
    A = tab.build_atom(Z, 15, b, lmax, lmax)
    ra = scf.run_scf(A, Z // 2, Z // 2, method)
    rl = scf.run_scf(A, Z // 2, Z // 2, method, l_occ=l_occ)
    assert ra.converged and rl.converged
    assert abs(ra.Etot - rl.Etot) < 1e-9, (ra.Etot, rl.Etot)


def test_open_shell_fractional_occupation_converges():
    """C (1s2 2s2 2p2), the two p electrons shared over the three m blocks
    (2/3 each, restricted): converges, and lies above the integer-occupation
    (symmetry-broken) Aufbau solution of the same basis."""
    b = tab.get_grid(40.0, 6, 4, 2.0)
    A = tab.build_atom(6, 15, b, 1, 1)
    r = scf.run_scf(A, 3, 3, "hf", l_occ=[(2, 2), (1, 1)])
    assert r.converged
    ru = scf.run_scf(A, 4, 2, "hf", restricted=False)
    assert ru.converged and ru.Etot < r.Etot
