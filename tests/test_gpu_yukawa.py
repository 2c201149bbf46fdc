"""Range-separated (Yukawa-screened) exchange on the GPU (hfg_rs_exchange)
against the oracle's screened exchange and the analytic hydrogenic integral.

Bars as for the bare exchange: FP64 max|GPU - oracle| <= 1e-10 max|oracle|,
split precision 1e-12 relative; the hydrogen 1s screened exchange energy to
1e-11 Eh of the analytic value."""
import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import FockOracle
from oracle import tabulate as tab
from oracle.yukawa import hydrogenic_yukawa_self_energy, yukawa_tables
from gpu_util import from_dev, make_pair, random_density, relerr, to_dev, torch_cuda
from test_yukawa_cpu import hydrogen_1s

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [(10, 1, 1, 5, 0.4), (36, 2, 2, 8, 1.0), (8, 3, 0, 4, 0.1)],
                         ids=lambda c: f"Z{c[0]}_l{c[1]}m{c[2]}_e{c[3]}_lam{c[4]}")
def test_rs_exchange_matches_oracle(case):
    torch = torch_cuda()
    Z, lmax, mmax, nel, lam = case
    A, O = make_pair(Z, lmax, mmax, nel)
    with pytest.raises(Exception):  # before compute_yukawa: the reference's logic_error
        A.rs_exchange_host(np.eye(A.nbf))
    A.compute_yukawa(lam)
    P = random_density(O.nbf, 4, seed=Z, S=O.S)
    ref = FockOracle(yukawa_tables(O, lam)).exchange(P)
    assert relerr(A.rs_exchange_host(P), ref) < 1e-10
    assert relerr(A.rs_exchange_host(P, symmetric=True), ref) < 1e-10
    assert relerr(A.rs_exchange_host(P, symmetric=True, split=True), ref) < 1e-12
    # device entry point on torch buffers; the bare exchange is unchanged
    Pd = to_dev(torch, P)
    Kd = torch.full_like(Pd, np.nan)
    A.rs_exchange(Pd, Kd, symmetric=True)
    torch.cuda.synchronize()
    assert relerr(from_dev(Kd), ref) < 1e-10
    assert relerr(A.exchange_host(P), FockOracle(O).exchange(P)) < 1e-10


def test_rs_exchange_hydrogen_analytic():
    torch_cuda()
    O, b, e1s, P = hydrogen_1s()
    a = hg.Atom(1, b, *hg.angular_basis(0, 0))
    for lam in (0.05, 0.5, 2.0):
        a.compute_yukawa(lam)  # replaces the previous screening parameter
        for split in (False, True):
            Ex = float(np.sum(P * a.rs_exchange_host(P, symmetric=True, split=split)))
            assert abs(Ex + hydrogenic_yukawa_self_energy(1.0, lam)) < 1e-11, (lam, split, Ex)
