"""Range-separated exchange with the erfc kernel on the GPU (hfg_atom_compute_erfc,
hfg_rs_exchange) against the numpy restatement of the reference's
compute_erfc / rs_exchange (oracle/erfc.py), on the same quadrature.

Bar: max|GPU - oracle| <= 1e-10 max|oracle| (FP64 both; the general form of
the expansion carries ~1e-10 relative rounding noise at higher multipoles
whose contributions to K are small)."""
import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import FockOracle, gaunt_table
from oracle import erfc as E
from oracle import tabulate as tab
from gpu_util import from_dev, random_density, relerr, to_dev, torch_cuda

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [(4, 1, 0, 3, 5, 0.7), (8, 1, 1, 3, 7, 1.3), (10, 2, 1, 3, 5, 0.4)],
                         ids=lambda c: f"Z{c[0]}_l{c[1]}m{c[2]}_e{c[3]}_n{c[4]}_mu{c[5]}")
def test_erfc_exchange_matches_oracle(case):
    torch = torch_cuda()
    Z, lmax, mmax, nel, nn, mu = case
    b = tab.get_grid(20.0, nel, 4, 2.0)
    lv, mv = hg.angular_basis(lmax, mmax)
    A = hg.Atom(Z, b, lv, mv, nnodes=nn)
    O = tab.build_atom(Z, nn, b, lmax, mmax)
    with pytest.raises(Exception):  # before compute_erfc: the reference's logic_error
        A.rs_exchange_host(np.eye(A.nbf))
    A.compute_erfc(mu)
    P = random_density(O.nbf, 4, seed=Z, S=O.S)
    ref = E.rs_exchange_erfc(O, mu, P, gaunt_table(2 * lmax))
    assert relerr(A.rs_exchange_host(P), ref) < 1e-10
    Pd = to_dev(torch, P)
    Kd = torch.full_like(Pd, np.nan)
    A.rs_exchange(Pd, Kd)
    torch.cuda.synchronize()
    K = from_dev(Kd)
    err = relerr(K, ref)
    print(f"erfc K {case}: max rel err {err:.2e}")
    assert np.isfinite(K).all() and err < 1e-10
    # the split form is refused; the bare exchange is unchanged
    with pytest.raises(Exception):
        A.rs_exchange_host(P, split=True)
    assert relerr(A.exchange_host(P), FockOracle(O).exchange(P)) < 1e-10


def test_erfc_exact_binomial_and_mode_switch():
    """The exact-binomial tables give the exact-rule oracle; compute_yukawa
    afterwards switches hfg_rs_exchange back to the Yukawa kernel."""
    torch_cuda()
    from oracle.yukawa import yukawa_tables
    b = tab.get_grid(20.0, 3, 4, 2.0)
    lv, mv = hg.angular_basis(1, 0)
    A = hg.Atom(6, b, lv, mv, nnodes=5)
    O = tab.build_atom(6, 5, b, 1, 0)
    P = random_density(O.nbf, 3, seed=5, S=O.S)
    A.compute_erfc(0.9, exact_binomial=True)
    ref = E.rs_exchange_erfc(O, 0.9, P, gaunt_table(2), binomial="exact")
    assert relerr(A.rs_exchange_host(P), ref) < 1e-10
    A.compute_yukawa(0.5)
    assert relerr(A.rs_exchange_host(P), FockOracle(yukawa_tables(O, 0.5)).exchange(P)) < 1e-10
