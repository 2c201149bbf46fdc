"""GPU parity of the XC potential (separable DFT-grid kernels) against the
oracle's dense restatement of DFTGrid::eval_Fxc. Bar: Vxc matrices and Exc
within 1e-10 relative."""
import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import tabulate as tab
from oracle import xc as oxc
from gpu_util import random_density, relerr, torch_cuda

pytestmark = pytest.mark.gpu
TOL = 1e-10

CASES = [
    # Z, lmax, mmax, nelem, nnodes, method, polarized
    (2, 0, 0, 4, 15, "lda_x-lda_c_vwn", False),
    (2, 0, 0, 4, 15, "gga_x_pbe-gga_c_pbe", False),
    (10, 1, 0, 4, 12, "lda_x-lda_c_pw", False),
    (8, 1, 1, 3, 10, "gga_x_pbe-gga_c_pbe", True),
    (8, 1, 1, 3, 10, "lda_x-lda_c_vwn", True),
    (36, 2, 2, 3, 8, "gga_x_pbe", False),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"Z{c[0]}_l{c[1]}m{c[2]}_{c[5]}_{'u' if c[6] else 'r'}")
def test_xc_matches_oracle(case):
    torch_cuda()
    Z, lmax, mmax, nelem, nn, method, pol = case
    b = tab.get_grid(40.0, nelem, 4, 2.0)
    lv, mv = hg.angular_basis(lmax, mmax)
    A = hg.Atom(Z, b, lv, mv, nnodes=nn)
    O = tab.build_atom(Z, nn, b, lmax, mmax)
    G = oxc.AtomGrid(O)
    names = oxc.parse_method(method)
    x, c = hg.parse_xc(method)
    S = O.S
    if pol:
        Pa = random_density(O.nbf, 3, seed=Z, S=S)
        Pb = random_density(O.nbf, 2, seed=Z + 1, S=S)
        Ha, Hb, E, N = A.xc_host(x, c, Pa, Pb)
        Ra, Rb, Er, Nr = G.eval_Fxc(names, Pa, Pb)
        assert relerr(Hb, Rb) < TOL
    else:
        P = random_density(O.nbf, 2, seed=Z, S=S) * 2.0
        Ha, _, E, N = A.xc_host(x, c, P)
        Ra, _, Er, Nr = G.eval_Fxc(names, 0.5 * P, 0.5 * P)
    assert relerr(Ha, Ra) < TOL
    assert abs(E - Er) < TOL * abs(Er)
    assert abs(N - Nr) < TOL * abs(Nr)


def test_xc_device_entry_and_zero_density():
    torch = torch_cuda()
    A = hg.Atom.from_grid(2, 3, 40.0, 0, 0)
    P = torch.zeros((A.nbf, A.nbf), dtype=torch.float64, device="cuda")
    H = torch.full_like(P, 3.0)
    e = torch.full((2,), 9.0, dtype=torch.float64, device="cuda")
    A.xc(1, 7, P, H, energies=e)
    torch.cuda.synchronize()
    assert float(H.abs().max()) == 0.0
    assert float(e.abs().max()) == 0.0


def test_xc_rejects_unknown_functional():
    torch_cuda()
    A = hg.Atom.from_grid(2, 3, 40.0, 0, 0)
    with pytest.raises(hg.HfgError) as err:
        A.xc_host(999, 0, np.zeros((A.nbf, A.nbf)))
    assert err.value.status == hg.HFG_ERR_ARG
