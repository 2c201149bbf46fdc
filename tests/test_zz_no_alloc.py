"""The allocation-free Coulomb entry point (hfg_coulomb_noalloc).

Callers that cannot allocate device memory on their per-call path (hosts
that own every device allocation and give the library a fixed budget, loops
that must not risk an allocation's synchronisation) use this variant; its scratch is a fixed 4 MiB array in the library's static device
memory. It must give the same J as hfg_coulomb, call after call (the shared
array keeps the previous call's contents), and must refuse atoms whose
scratch does not fit. This file is named to be collected last.
"""
import numpy as np
import pytest

import helfem_gb300 as hg
from gpu_util import from_dev, random_density, relerr, to_dev, torch_cuda

pytestmark = pytest.mark.gpu
TOL = 1e-10


def test_noalloc_matches_coulomb_twice():
    torch = torch_cuda()
    A = hg.Atom.from_grid(36, 12, 40.0, 2, 2)
    P1 = random_density(A.nbf, 9, seed=21, S=A.overlap())
    P2 = random_density(A.nbf, 4, seed=22)
    for P in (P1, P2):  # two calls in a row, different densities
        Pd = to_dev(torch, P)
        Jref = torch.empty_like(Pd)
        Jna = torch.full_like(Pd, np.nan)
        A.coulomb(Pd, Jref)
        A.coulomb_noalloc(Pd, Jna)
        torch.cuda.synchronize()
        ref, got = from_dev(Jref), from_dev(Jna)
        assert np.isfinite(got).all()
        assert relerr(got, ref) < TOL


def test_noalloc_rejects_oversized_atom():
    torch = torch_cuda()
    # 49 (L,M) channels x 50 elements x (15^2 + 2) doubles > 4 MiB
    A = hg.Atom.from_grid(54, 50, 60.0, 3, 3, zexp=1.0)
    # real, correctly sized buffers: the call must fail on the size check alone
    Pd = torch.zeros((A.nbf, A.nbf), dtype=torch.float64, device="cuda")
    Jd = torch.zeros_like(Pd)
    with pytest.raises(hg.HfgError) as e:
        A.coulomb_noalloc(Pd, Jd)
    assert e.value.status == hg.HFG_ERR_ARG
    assert "static array" in str(e.value)
    # the handle's own path still serves this atom
    A.coulomb(Pd, Jd)
    torch.cuda.synchronize()
    assert float(Jd.abs().max()) == 0.0
