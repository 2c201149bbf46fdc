"""GPU parity of the pure-m diatomic XC potential (hfg_diatomic_xc) against the
oracle grid, and the reference's converged diatomic DFT energies reproduced
with the GPU Coulomb and XC builds inside the oracle's SCF driver.

Bars: max|GPU - oracle| <= 1e-10 * max|oracle| for the XC matrices (FP64,
same quadrature, different summation order and transcendental
implementations), |dExc| <= 1e-11 |Exc|, electron count to 1e-11; energies
as in tests/test_oracle_diatomic_xc.py.
"""
import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import diatomic as dia
from oracle.diatomic_xc import PureMGrid
from gpu_util import from_dev, relerr, to_dev, torch_cuda
from test_gpu_diatomic import CASES, bound_density
from test_oracle_diatomic_xc import BAR, SCF, run_case

pytestmark = pytest.mark.gpu
TOL = 1e-10
FUNCS = {"lda": ["lda_x", "lda_c_vwn"], "gga": ["gga_x_pbe", "gga_c_pbe"], "pw": ["lda_x", "lda_c_pw"]}


def pair(case):
    Z1, Z2, R, nel, lm = case
    return hg.Diatomic.from_grid(Z1, Z2, R, nel, lm), dia.build_diatomic(Z1, Z2, R, 15, nel, lm)


@pytest.mark.parametrize("func", sorted(FUNCS))
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"Z{c[0]}-{c[1]}_e{c[3]}_m{len(c[4]) - 1}")
def test_diatomic_xc_matches_oracle(case, func):
    torch = torch_cuda()
    d, D = pair(case)
    g = PureMGrid(D)
    names = FUNCS[func]
    x, c = hg.parse_xc("-".join(names))
    Pa = bound_density(D, 2, seed=0, blockdiag=True)
    # beta keeps at least half the alpha density everywhere: where one spin
    # density falls below half the density threshold it is clamped while its
    # gradient is not, and the GGA potential of that spin is ill-conditioned
    # in any implementation (|w v_sigma| ~ 1e16 at such tail points)
    Pb = 0.5 * Pa + 0.5 * bound_density(D, 1, seed=0, blockdiag=True)
    # restricted: total density Pa + Pb split evenly
    P = Pa + Pb
    Hr, _, Er, Nr = g.eval_Fxc(names, 0.5 * P, 0.5 * P)
    H, _, E, N = d.xc_host(x, c, P)
    assert relerr(H, Hr) < TOL, relerr(H, Hr)
    assert abs(E - Er) < 1e-11 * abs(Er) and abs(N - Nr) < 1e-11 * Nr, (E, Er, N, Nr)
    # unrestricted
    Ha_r, Hb_r, Eu_r, Nu_r = g.eval_Fxc(names, Pa, Pb)
    Ha, Hb, Eu, Nu = d.xc_host(x, c, Pa, Pb)
    assert relerr(Ha, Ha_r) < TOL and relerr(Hb, Hb_r) < TOL, (relerr(Ha, Ha_r), relerr(Hb, Hb_r))
    assert abs(Eu - Eu_r) < 1e-11 * abs(Eu_r) and abs(Nu - Nu_r) < 1e-11 * Nu_r
    # device entry point on torch buffers, energies in device memory
    Pd = to_dev(torch, Pa)
    Qd = to_dev(torch, Pb)
    Had = torch.full_like(Pd, np.nan)
    Hbd = torch.full_like(Pd, np.nan)
    en = torch.zeros(2, dtype=torch.float64, device="cuda")
    d.xc(x, c, Pd, Had, Qd, Hbd, energies=en)
    torch.cuda.synchronize()
    assert relerr(from_dev(Had), Ha_r) < TOL and relerr(from_dev(Hbd), Hb_r) < TOL
    assert abs(float(en[0]) - Eu_r) < 1e-11 * abs(Eu_r)


def test_diatomic_xc_grid_rebuild():
    """A finer nu rule changes the potential by the quadrature error only, and
    the default rule is restored by dft_grid(0)."""
    torch_cuda()
    d, D = pair(CASES[1])
    P = bound_density(D, 2, seed=0, blockdiag=True)
    x, c = hg.parse_xc("lda_x-lda_c_vwn")
    H0, _, E0, N0 = d.xc_host(x, c, P)
    d.dft_grid(4 * 4 + 24)
    H1, _, E1, N1 = d.xc_host(x, c, P)
    assert abs(E1 - E0) < 1e-4 * abs(E0) and abs(N1 - N0) < 1e-4 * N0
    g = PureMGrid(D, lang=4 * 4 + 24)
    Hr, _, Er, _ = g.eval_Fxc(["lda_x", "lda_c_vwn"], 0.5 * P, 0.5 * P)
    assert relerr(H1, Hr) < TOL and abs(E1 - Er) < 1e-11 * abs(Er)
    d.dft_grid(0)
    H2, _, E2, _ = d.xc_host(x, c, P)
    assert relerr(H2, H0) < 1e-14 and E2 == E0


class _GpuJ:
    def __init__(self, d):
        self.d = d

    def coulomb(self, P):
        return self.d.coulomb_host(P)


class _GpuXC:
    """eval_Fxc on the GPU; the restricted driver passes Pa is Pb = P/2."""

    def __init__(self, d):
        self.d = d

    def eval_Fxc(self, names, Pa, Pb, thr=1e-12):
        x, c = hg.parse_xc("-".join(names))
        if Pa is Pb:
            H, _, E, N = self.d.xc_host(x, c, Pa + Pb, thr=thr)
            return H, H, E, N
        Ha, Hb, E, N = self.d.xc_host(x, c, Pa, Pb, thr=thr)
        return Ha, Hb, E, N


@pytest.mark.parametrize("name", ["diatomic-H2-purem-on", "diatomic-Ne-dummy-lda", "diatomic-Ne-dummy-gga",
                                  "diatomic-NH-lda-u"])
def test_pure_m_dft_energy_through_gpu(name):
    """The reference's converged diatomic DFT energies with J and V_xc from the
    GPU: the oracle's SCF driver, the product's Coulomb and XC builds."""
    torch_cuda()
    a = SCF[name]["args"]
    lm = [int(v) for v in a["lmax"].split(",")]
    d = hg.Diatomic.from_grid(int(a["Z1"]), int(a["Z2"]), float(a["Rbond"]), int(a["nelem"]), lm,
                              nnodes=int(a["nnodes"]))
    r, ref = run_case(name, fock=lambda D: _GpuJ(d), grid=lambda D: _GpuXC(d))
    assert r.converged
    assert abs(r.Etot + ref["Enucr"] - ref["total"]) < BAR.get(name, 2e-9), (r.Etot + ref["Enucr"], ref["total"])


def test_n2_full_size_xc_parity():
    """The N2 benchmark basis and density (30 mu-elements, l <= 12 for
    |m| <= 3, 33114 functions): every (m, m) block of the GPU PBE potential
    against the oracle grid at full size, with Exc and the electron count."""
    import bench
    from oracle.diatomic_xc import grid_tables
    torch = torch_cuda()
    d, P, _ = bench.n2_setup(hg)
    D = grid_tables(7, 7, 2.074, 15, 30, [12] * 4)
    g = PureMGrid(D)
    mb = g.mblocks()
    blk = {m: 0.5 * P[np.ix_(pos, pos)] for m, (pos, _) in mb.items()}
    Hr, _, Er, Nr = g.eval_Fxc_blocks(["gga_x_pbe", "gga_c_pbe"], blk, blk)
    nbf = d.nbf
    Pd = torch.zeros((nbf, nbf), dtype=torch.float64, device="cuda")
    for m, (pos, _) in mb.items():
        ix = torch.from_numpy(pos).cuda()
        Pd[ix[:, None], ix[None, :]] = torch.from_numpy(2.0 * blk[m]).cuda()  # symmetric: layout-free
    Hd = torch.empty_like(Pd)
    en = torch.zeros(2, dtype=torch.float64, device="cuda")
    x, c = hg.parse_xc("gga_x_pbe-gga_c_pbe")
    d.xc(x, c, Pd, Hd, energies=en)
    torch.cuda.synchronize()
    del Pd
    assert abs(float(en[0]) - Er) < 1e-11 * abs(Er) and abs(float(en[1]) - Nr) < 1e-11 * Nr, (en, Er, Nr)
    for m, (pos, _) in mb.items():
        ix = torch.from_numpy(pos).cuda()
        got = Hd[ix[:, None], ix[None, :]].cpu().numpy().T
        assert relerr(got, Hr[m]) < TOL, (m, relerr(got, Hr[m]))
