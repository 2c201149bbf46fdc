"""Whole atomic SCF on the GPU (J, K, XC, orthonormalisation, diagonalisation
all on the device) against the reference's own recorded energies
(tests/refs/ci.json, tests/README.md) at the harness tolerance, 1e-8 Eh."""
import json
import os

import numpy as np
import pytest

import helfem_gb300 as hg
from gpu_util import torch_cuda
from oracle import tabulate as tab

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CI = {c["name"]: c for c in json.load(open(os.path.join(HERE, "golden", "ci_energies.json")))}
SYMBOL = {"H": 1, "He": 2, "Be": 4, "O": 8, "Ne": 10}


def run_case(name, symmetry=1):
    c = CI[name]
    a = c["args"]
    Z = SYMBOL[a["Z"]]
    atom = hg.Atom.from_grid(Z, int(a["nelem"]), 40.0, int(a["lmax"]), int(a["mmax"]), igrid=4, zexp=2.0,
                             nnodes=int(a.get("nnodes", 15)))
    M = int(a.get("M", 1))
    nela, nelb = (Z + M - 1) // 2, (Z - M + 1) // 2
    restricted = a.get("restricted", "1" if nela == nelb else "0") == "1"
    fixed = None
    if c["occs"]:
        fixed = {}
        for line in c["occs"].strip().splitlines():
            na, nb, m = (int(x) for x in line.split())
            fixed[m] = (na, nb)
        restricted = False
    return atom.scf(nela, nelb, a.get("method", "hf"), restricted=restricted, symmetry=symmetry, fixed_occ=fixed)


CASES = ["atomic-He-hf-r", "atomic-He-hf-u", "atomic-Be-hf-r", "atomic-H-hf-u", "atomic-He-lda-r",
         "atomic-Be-lda-u", "atomic-He-gga-r", "atomic-He-gga-u", "atomic-O-3P-p0-hf", "atomic-O-3P-pplus-hf",
         "atomic-Ne-hf-r", "atomic-Be-nop-l0"]


@pytest.mark.parametrize("name", CASES)
def test_gpu_scf_matches_reference_energy(name):
    torch_cuda()
    r = run_case(name)
    assert r["converged"], r
    assert abs(r["Etot"] - CI[name]["total"]) < 1e-8, (r["Etot"], CI[name]["total"])


@pytest.mark.parametrize("name,damped", [("atomic-Ne-hf-r", True), ("atomic-O-3P-p0-hf", True),
                                         ("atomic-Be-hf-r", False), ("atomic-Be-lda-u", None),
                                         ("atomic-He-gga-u", None)])
def test_optimal_damping_reaches_reference_energy(name, damped, monkeypatch, capfd):
    """Optimal damping (ODA) started at the first iteration (it otherwise
    starts only when DIIS stalls under the full level shift): the line-search
    steps, then DIIS, reach the reference's energy at 1e-8 Eh. Ne and O take
    at least one damped step (lambda < 1); for Be the full Roothaan step is
    optimal from the core guess on, and two full steps end the damping. The
    LDA and GGA runs take the curvature from the energy at the Aufbau
    density and evaluate the XC potential again at each damped density."""
    torch_cuda()
    monkeypatch.setenv("HFG_SCF_ODA", "first")
    monkeypatch.setenv("HFG_SCF_VERBOSE", "1")
    r = run_case(name)
    err = capfd.readouterr().err
    lams = [float(l.split("lambda")[1]) for l in err.splitlines() if "ODA s" in l]
    print("ODA lambdas", lams)
    assert lams, err[-2000:]
    if damped is not None:
        assert (min(lams) < 1.0) == damped, lams
    assert r["converged"], r
    assert abs(r["Etot"] - CI[name]["total"]) < 1e-8, (r["Etot"], CI[name]["total"])


def test_symmetry_blocks_agree():
    """Per-(l,m) blocks give the per-m energy for a closed-shell atom."""
    torch_cuda()
    a = run_case("atomic-Ne-hf-r", symmetry=1)
    b = run_case("atomic-Ne-hf-r", symmetry=2)
    assert abs(a["Etot"] - b["Etot"]) < 1e-9


def _tight_pair(Z, nelem, lmax, mmax, zexp, nel, monkeypatch):
    """One GPU SCF and one oracle SCF of the same atom, both converged to an
    orbital gradient (largest orthonormal-basis commutator element) below
    1e-10 from the core-Hamiltonian guess, with full eigensolves on the GPU
    so that the gradient can fall below the refinement's residual floor."""
    from oracle import scf as oscf
    monkeypatch.setenv("HFG_SCF_EIGENSOLVER", "full")
    atom = hg.Atom.from_grid(Z, nelem, 40.0, lmax, mmax, igrid=4, zexp=zexp)
    r = atom.scf(nel, nel, "hf", restricted=True, symmetry=1, e_tol=1e-12, diis_tol=1e-10, maxiter=300)
    A = tab.build_atom(Z, 15, tab.get_grid(40.0, nelem, 4, zexp), lmax, mmax)
    o = oscf.run_scf(A, nel, nel, "hf", True, conv=1e-12, gtol=1e-10, maxiter=300)
    return r, o


def _check_spectrum(r, o, nocc, atol):
    """SCF-converged orbital energies: the occupied and the first virtual,
    within atol (both solves stop at an orbital gradient of 1e-10, which
    leaves orbital energies uncertain at that level: they are first order
    in the density error, unlike the total energy)."""
    e_gpu = np.sort(r["orbital_energies"])[:nocc + 1]
    e_ora = np.sort(np.concatenate([np.ravel(x) for x in o.eps]))[:nocc + 1]
    d = np.abs(e_gpu - e_ora)
    print("orbital energies", e_gpu, "max |d|", d.max())
    assert (d <= atol).all(), (e_gpu, e_ora, d)


def _same_input_spectrum(atom, A, o, nocc):
    """Orbital energies from the same input: the oracle's converged density
    gives the Fock matrix on both sides (GPU J and K, oracle J and K), whose
    generalised eigenvalues in the S metric are compared per m block."""
    import scipy.linalg
    from gpu_util import from_dev, to_dev
    from oracle import FockOracle
    torch = torch_cuda()
    P = o.Pa + o.Pb
    F = FockOracle(A)
    Fo = A.T + A.V + F.coulomb(P) + F.exchange(o.Pa)
    Pd = to_dev(torch, P)
    Jd, Kd = torch.empty_like(Pd), torch.empty_like(Pd)
    atom.coulomb(Pd, Jd)
    atom.exchange(0.5 * Pd, Kd)
    Fg = atom.kinetic() + atom.nuclear() + from_dev(Jd) + from_dev(Kd)
    Fd = to_dev(torch, Fg)
    Cd = torch.zeros_like(Fd)
    ed = torch.zeros(atom.nbf, dtype=torch.float64, device="cuda")
    atom.fock_diag(Fd, Cd, ed, symmetry=1)
    torch.cuda.synchronize()
    e_gpu = np.sort(ed.cpu().numpy())[:nocc + 1]
    e_ora = np.sort(scipy.linalg.eigh(Fo, A.S, eigvals_only=True))[:nocc + 1]
    d = np.abs(e_gpu - e_ora)
    rel = d / np.abs(e_ora)
    print("same-input orbital energies", e_gpu, "max |d|", d.max(), "max rel", rel.max())
    return e_gpu, e_ora, d, rel


def test_orbital_energies_match_oracle(monkeypatch):
    """He (the reference's CI geometry): total energy at 1e-10 relative;
    SCF-converged orbital energies within 1e-9 Eh; the same-input occupied
    orbital energy at 1e-10 relative."""
    torch_cuda()
    r, o = _tight_pair(2, 5, 0, 0, 2.0, 1, monkeypatch)
    assert r["converged"] and o.converged
    assert abs(r["Etot"] - o.Etot) < 1e-10 * abs(o.Etot), (r["Etot"], o.Etot)
    _check_spectrum(r, o, 1, 1e-9)
    atom = hg.Atom.from_grid(2, 5, 40.0, 0, 0, igrid=4, zexp=2.0)
    A = tab.build_atom(2, 15, tab.get_grid(40.0, 5, 4, 2.0), 0, 0)
    e_gpu, e_ora, d, rel = _same_input_spectrum(atom, A, o, 1)
    assert rel[0] < 1e-10, (e_gpu, e_ora)


def test_ne_config1_matches_oracle(monkeypatch):
    """Ne as the first benchmark configuration states it: Z = 10 restricted
    HF, 10 elements with r_i = 41^(i/10) - 1 (zexp = 1, Rmax = 40), 15-node
    LIP, l = 0..1 with m = 0 only (Nbf = 278), L = 0..2, core-Hamiltonian
    guess. The default SCF path to the configuration's own criterion gives
    the oracle's total energy at 1e-10 relative; converged tightly, the
    energy components agree at 1e-9 relative and the orbital energies within
    1e-9 Eh; from the same density, the five occupied orbital energies agree
    at 1e-10 relative and the first virtual (3.6e-3 Eh, near zero in the
    40-bohr box) within 1e-11 Eh, the FP64 eigensolver's resolution for this
    spectrum (its largest eigenvalue is ~5e4 Eh)."""
    torch_cuda()
    from oracle import scf as oscf
    atom = hg.Atom.from_grid(10, 10, 40.0, 1, 0, igrid=4, zexp=1.0)
    assert atom.nbf == 278
    r0 = atom.scf(5, 5, "hf", restricted=True, symmetry=1)
    A = tab.build_atom(10, 15, tab.get_grid(40.0, 10, 4, 1.0), 1, 0)
    o0 = oscf.run_scf(A, 5, 5, "hf", True)
    assert r0["converged"] and o0.converged
    assert abs(r0["Etot"] - o0.Etot) < 1e-10 * abs(o0.Etot), (r0["Etot"], o0.Etot)
    r, o = _tight_pair(10, 10, 1, 0, 1.0, 5, monkeypatch)
    assert r["converged"] and o.converged
    assert abs(r["Etot"] - o.Etot) < 1e-10 * abs(o.Etot), (r["Etot"], o.Etot)
    for k in ("Ekin", "Enuc", "Ecoul", "Exx"):
        assert abs(r[k] - getattr(o, k)) < 1e-9 * abs(o.Etot), (k, r[k], getattr(o, k))
    _check_spectrum(r, o, 5, 1e-9)
    e_gpu, e_ora, d, rel = _same_input_spectrum(atom, A, o, 5)
    assert (rel[:5] < 1e-10).all(), (e_gpu, e_ora, rel)
    assert d[5] < 1e-11, (e_gpu, e_ora, d)


@pytest.mark.parametrize("symmetry", [1, 2])
def test_fock_diag_matches_generalized_eigenproblem(symmetry):
    """hfg_fock_diag: per-block generalized eigenpairs of F (here the core
    Hamiltonian, block diagonal in (l,m)) in the S metric."""
    import scipy.linalg
    from gpu_util import to_dev, from_dev
    torch = torch_cuda()
    b = tab.get_grid(40.0, 5, 4, 2.0)
    lv, mv = hg.angular_basis(1, 1)
    A = hg.Atom(8, b, lv, mv)
    S, H = A.overlap(), A.kinetic() + A.nuclear()
    Fd = to_dev(torch, H)
    Cd = torch.zeros_like(Fd)
    ed = torch.zeros(A.nbf, dtype=torch.float64, device="cuda")
    A.fock_diag(Fd, Cd, ed, symmetry=symmetry)
    torch.cuda.synchronize()
    C, eps = from_dev(Cd), ed.cpu().numpy()
    n = A.nbf // len(lv)
    if symmetry == 1:
        groups = [[i for i in range(len(mv)) if mv[i] == m] for m in sorted(set(mv.tolist()))]
    else:
        groups = [[i] for i in range(len(lv))]
    col = 0
    for g in groups:
        idx = np.concatenate([np.arange(i * n, (i + 1) * n) for i in g])
        w = scipy.linalg.eigh(H[np.ix_(idx, idx)], S[np.ix_(idx, idx)], eigvals_only=True)
        e = eps[col:col + len(idx)]
        assert np.allclose(e, w, rtol=1e-10, atol=1e-10 * np.abs(w).max())
        col += len(idx)
    # S-orthonormal eigenvectors of H
    assert np.abs(C.T @ S @ C - np.eye(A.nbf)).max() < 1e-9
    R = H @ C - S @ C * eps[None, :]
    assert np.abs(R).max() < 1e-8 * np.abs(H).max()


@pytest.mark.parametrize("case", ["Kr-hf-spherical", "Kr-pw92-spherical", "Ne-hf-aufbau"])
def test_davidson_refinement_matches_full_eigensolves(case, monkeypatch):
    """The refined eigensolves (Davidson from the previous orbitals after two
    full solves) converge to the same SCF solution as full eigensolves every
    iteration: total energy to 1e-8 Eh, every orbital energy to 1e-6 Eh
    (the final spectrum comes from one full solve of the last Fock blocks)."""
    torch_cuda()
    from helfem_gb300 import workloads as wl
    if case.startswith("Kr"):
        atom = hg.Atom(36, wl.grid(60.0, 40, zexp=1.0), *wl.angular(2, 2))
        kw = dict(symmetry=2, l_occ=wl.l_occupations(18, 18, 2))
        method = "hf" if "hf" in case else "lda_x-lda_c_pw"
        nel = (18, 18)
    else:  # per-m blocks with Aufbau occupations
        atom = hg.Atom.from_grid(10, 12, 40.0, 1, 1, igrid=4, zexp=2.0)
        kw = dict(symmetry=1)
        method = "hf"
        nel = (5, 5)
    runs = {}
    for mode in ("full", "davidson"):
        monkeypatch.setenv("HFG_SCF_EIGENSOLVER", mode)
        runs[mode] = atom.scf(*nel, method=method, restricted=True, **kw)
    f, d = runs["full"], runs["davidson"]
    assert f["converged"] and d["converged"]
    assert abs(f["Etot"] - d["Etot"]) < 1e-8, (f["Etot"], d["Etot"])
    ef, ed = np.sort(f["orbital_energies"]), np.sort(d["orbital_energies"])
    assert np.abs(ef - ed).max() < 1e-6 * max(1.0, np.abs(ef).max() / 1e3)
    # the refinement is what the default path runs: it must be cheaper
    assert d["phase_ms"]["eigh_occupy"] < f["phase_ms"]["eigh_occupy"]
    if case.endswith("spherical"):
        # the opt-in banded shift-invert preconditioner (refinement from the
        # second iteration on) reaches the same solution
        monkeypatch.setenv("HFG_SCF_EIGENSOLVER", "davidson")
        monkeypatch.setenv("HFG_SCF_PRECOND", "banded")
        b = atom.scf(*nel, method=method, restricted=True, **kw)
        assert b["converged"] and abs(b["Etot"] - f["Etot"]) < 1e-8, (b["Etot"], f["Etot"])
        eb = np.sort(b["orbital_energies"])
        assert np.abs(ef - eb).max() < 1e-6 * max(1.0, np.abs(ef).max() / 1e3)
