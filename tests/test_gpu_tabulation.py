"""Device tabulation of the atomic in-element two-electron tables.

A device handle (the default, tabulate="device") forms the in-element tensor
of r<^L/r>^(L+1), its pivoted Cholesky factor and the exchange-ordered tensor
on the GPU. Checked against
  * the oracle's independently tabulated tensors (reconstructed L L^T,
    <= 1e-11 relative, the bar of the host tabulation),
  * the host tabulation of the same basis (tabulate="host"): tensors within
    1e-13 relative and the same ranks, J and K within 1e-12 relative,
  * an SCF energy through the engine with either tabulation (1e-9 Eh).
"""
import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import tabulate as tab
from gpu_util import from_dev, random_density, relerr, to_dev, torch_cuda

pytestmark = pytest.mark.gpu

CASES = [
    # Z, lmax, mmax, nelem, nnodes
    (2, 0, 0, 5, 15),
    (36, 2, 2, 8, 15),
    (20, 3, 1, 4, 10),
    (4, 0, 0, 2, 3),
    (6, 1, 1, 3, 17),
    (54, 2, 0, 6, 13),
]


def _pair(Z, lmax, mmax, nelem, nnodes):
    b = tab.get_grid(40.0, nelem, 4, 2.0)
    lv, mv = hg.angular_basis(lmax, mmax)
    Ad = hg.Atom(Z, b, lv, mv, nnodes=nnodes)
    Ah = hg.Atom(Z, b, lv, mv, nnodes=nnodes, tabulate="host")
    return b, Ad, Ah


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"Z{c[0]}_l{c[1]}m{c[2]}_e{c[3]}_n{c[4]}")
def test_device_tensors_match_oracle_and_host(case):
    torch_cuda()
    Z, lmax, mmax, nelem, nnodes = case
    b, Ad, Ah = _pair(*case)
    O = tab.build_atom(Z, nnodes, b, lmax, mmax)
    assert Ad.rmax >= 1
    for L in range(Ad.NL):
        for e in range(Ad.nel):
            rs_d, rb_d, C_d = Ad.radial_tables(L, e)
            rs_h, rb_h, C_h = Ah.radial_tables(L, e)
            assert np.array_equal(rs_d, rs_h) and np.array_equal(rb_d, rb_h)
            assert C_d.shape == C_h.shape, (L, e, C_d.shape, C_h.shape)
            Td, Th = C_d @ C_d.T, C_h @ C_h.T
            To = O.chol[L][e] @ O.chol[L][e].T
            assert np.abs(Td - Th).max() <= 1e-13 * np.abs(Th).max(), (L, e)
            assert np.abs(Td - To).max() < 1e-11 * np.abs(To).max(), (L, e)


@pytest.mark.parametrize("case", CASES[:3] + CASES[4:5], ids=lambda c: f"Z{c[0]}_l{c[1]}m{c[2]}_n{c[4]}")
def test_device_tabulated_jk_match_host_tabulated(case):
    torch = torch_cuda()
    b, Ad, Ah = _pair(*case)
    O = tab.build_atom(case[0], case[4], b, case[1], case[2])
    P = random_density(Ad.nbf, min(7, Ad.nbf), seed=case[0], S=O.S)
    Pd = to_dev(torch, P)
    out = {}
    for name, A in (("dev", Ad), ("host", Ah)):
        J = torch.full_like(Pd, np.nan)
        K = torch.full_like(Pd, np.nan)
        Ks = torch.full_like(Pd, np.nan)
        A.coulomb(Pd, J)
        A.exchange(Pd, K)
        A.exchange(Pd, Ks, split=True)
        torch.cuda.synchronize()
        out[name] = [from_dev(x) for x in (J, K, Ks)]
    for x, y in zip(out["dev"], out["host"]):
        assert np.isfinite(x).all()
        assert relerr(x, y) < 1e-12


def test_engine_energy_identical_with_either_tabulation():
    """Ne HF (l <= 1, all m, 5 elements) through the engine."""
    torch_cuda()
    b = tab.get_grid(40.0, 5, 4, 2.0)
    lv, mv = hg.angular_basis(1, 1)
    eng = hg.Engine(n_workers=2, hbm_budget_gb=8.0)
    ids = [eng.submit(10, b, lv, mv, 5, 5, "hf", True, nnodes=15, tabulate=t) for t in ("device", "host")]
    r = [eng.wait(i) for i in ids]
    eng.close()
    assert all(x["status"] == 2 and x["converged"] for x in r)
    assert abs(r[0]["Etot"] - r[1]["Etot"]) < 1e-9
