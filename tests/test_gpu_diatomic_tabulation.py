"""Device tabulation of the diatomic two-electron primitives
(src/diatomic/basis.cpp:1382-1547: the disjoint Plm/Qlm integrals and the
sign-carrying pivoted factor of the two-channel in-element kernel) against
the host tabulation of the same basis.

Bars: every disjoint table within 1e-13 of the largest entry of its kind,
except the Q tables of the first element (reported, not bounded: they are
never read, since the first element is never the outer element of a
disjoint pair; there sinh Q_L^M with M >= 2 grows like 1/mu, the
Gauss-Legendre sums are dominated by the innermost node, and two roundings
of the same sum differ by a few 1e-13 of the largest entry);
every reconstructed in-element kernel B diag(sigma) B^T within 1e-12 of its
largest entry (the factor is truncated at 1e-12 of the largest diagonal, so
two roundings of the same kernel may stop one pivot apart); J and K built
from either handle within 1e-12. The host tabulation itself is pinned to the
oracle (tests/test_oracle_diatomic.py, tests/test_gpu_diatomic.py).
"""
import time

import numpy as np
import pytest

import helfem_gb300 as hg
from gpu_util import from_dev, relerr, to_dev, torch_cuda

pytestmark = pytest.mark.gpu

BASES = [
    # Z1, Z2, Rbond, nelem, lmax per |m|, nnodes
    (1, 1, 1.4, 4, [2, 1], 5),
    (2, 1, 1.46, 5, [3, 2, 1], 7),
    (7, 7, 2.074, 6, [6, 4, 2], 15),
    (3, 1, 3.0, 3, [4, 3, 2, 1], 17),
]


def compare_tables(dd, dh, ilms=None, elems=None):
    """Largest differences between the tables of a device- and a
    host-tabulated handle: disjoint kinds relative to the kind's largest
    entry (the first element's unused Q tables apart, as a fifth figure),
    kernels relative to each tile's largest entry; rank mismatches."""
    nlm, nel = dd.dims["nlm"], dd.dims["nel"]
    ilms = range(nlm) if ilms is None else ilms
    elems = range(nel) if elems is None else elems
    dmax = [0.0] * 5
    smax = [0.0] * 5
    werr, rank_diff, ntile = 0.0, 0, 0
    for ilm in ilms:
        for e in elems:
            for w in range(4):
                _, _, A = dd.tables(w, ilm, e)
                _, _, B = dh.tables(w, ilm, e)
                k = 4 if (e == 0 and w >= 2) else w
                dmax[k] = max(dmax[k], float(np.abs(A - B).max()))
                smax[k] = max(smax[k], float(np.abs(B).max()))
            _, _, Bd, sd = dd.tables(4, ilm, e)
            _, _, Bh, sh = dh.tables(4, ilm, e)
            Wd = (Bd * sd) @ Bd.T
            Wh = (Bh * sh) @ Bh.T
            werr = max(werr, float(np.abs(Wd - Wh).max() / max(np.abs(Wh).max(), 1e-300)))
            rank_diff += int(Bd.shape[1] != Bh.shape[1])
            ntile += 1
    return [dmax[w] / max(smax[w], 1e-300) for w in range(5)], werr, rank_diff, ntile


@pytest.mark.parametrize("case", BASES)
def test_device_tables_match_host(case):
    Z1, Z2, R, nel, lm, nn = case
    dd = hg.Diatomic.from_grid(Z1, Z2, R, nel, lm, nnodes=nn)
    dh = hg.Diatomic.from_grid(Z1, Z2, R, nel, lm, nnodes=nn, host_only=True)
    assert dd.dims == dh.dims or {k: v for k, v in dd.dims.items() if k != "rmax"} == \
        {k: v for k, v in dh.dims.items() if k != "rmax"}
    disj, werr, rank_diff, ntile = compare_tables(dd, dh)
    print(f"nn={nn} tiles={ntile}: disjoint {['%.1e' % x for x in disj]}, kernel {werr:.1e}, "
          f"rank mismatches {rank_diff}")
    assert max(disj[:4]) <= 1e-13
    assert disj[4] <= 1e-10
    assert werr <= 1e-12
    assert rank_diff <= max(1, ntile // 100)
    dd.close()
    dh.close()


@pytest.mark.parametrize("case", BASES[1:3])
def test_fock_from_device_tables_matches_host_tables(case):
    torch = torch_cuda()
    Z1, Z2, R, nel, lm, nn = case
    dd = hg.Diatomic.from_grid(Z1, Z2, R, nel, lm, nnodes=nn)
    dh = hg.Diatomic.from_grid(Z1, Z2, R, nel, lm, nnodes=nn, tabulate="host")
    rng = np.random.default_rng(7)
    C = rng.standard_normal((dd.nbf, 4))
    P = C @ C.T
    Pd = to_dev(torch, P)
    out = {}
    for name, d in (("dev", dd), ("host", dh)):
        J, K, Ks = torch.empty_like(Pd), torch.empty_like(Pd), torch.empty_like(Pd)
        d.coulomb(Pd, J)
        d.exchange(Pd, K, symmetric=True)
        d.exchange(Pd, Ks, symmetric=True, split=True)
        torch.cuda.synchronize()
        out[name] = (from_dev(J), from_dev(K), from_dev(Ks))
    for i, what in enumerate(("J", "K", "split K")):
        err = relerr(out["dev"][i], out["host"][i])
        print(f"{what}: {err:.2e}")
        assert err <= 1e-12, what
    dd.close()
    dh.close()


def test_n2_device_tabulation_full_size():
    """The N2 benchmark basis (30 mu elements, l <= 12 for m = 0..3, 168
    multipoles): device and host tabulation side by side, a sample of the
    tables compared, and J and K of a bound density from both handles."""
    torch = torch_cuda()
    args = (7, 7, 2.074, 30, [12] * 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dd = hg.Diatomic.from_grid(*args)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    dh = hg.Diatomic.from_grid(*args, tabulate="host")
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    print(f"N2 handle set-up: device tabulation {t1 - t0:.2f} s, host tabulation {t2 - t1:.2f} s")
    nlm = dd.dims["nlm"]
    disj, werr, rank_diff, ntile = compare_tables(dd, dh, ilms=range(0, nlm, 11))
    print(f"N2 sample ({ntile} tiles): disjoint {['%.1e' % x for x in disj]}, kernel {werr:.1e}, "
          f"rank mismatches {rank_diff}")
    assert max(disj[:4]) <= 1e-13
    assert disj[4] <= 1e-10
    assert werr <= 1e-12
    assert rank_diff <= max(1, ntile // 100)
    idx = dd.pure_indices()
    mv = dd.mval[idx // dd.nrad]
    rng = np.random.default_rng(12345)
    P = np.zeros((dd.nbf, dd.nbf), order="F")
    for m, nocc in ((0, 5), (1, 1), (-1, 1)):
        sel = np.where(mv == m)[0]
        S = dd.one_electron_block("S", m)
        C = rng.standard_normal((len(sel), nocc))
        w, v = np.linalg.eigh(C.T @ S @ C)
        C = C @ (v @ np.diag(w ** -0.5) @ v.T)
        P[np.ix_(sel, sel)] = 2.0 * (C @ C.T)
    # one handle's device state at a time from here (each holds ~26 GB)
    Pd = torch.from_numpy(P.ravel(order="F")).cuda()
    Pa = 0.5 * Pd
    Jd, Kd = torch.empty_like(Pd), torch.empty_like(Pd)
    dd.coulomb(Pd, Jd)
    dd.exchange(Pa, Kd, symmetric=True)
    torch.cuda.synchronize()
    dd.close()
    J, K = torch.empty_like(Pd), torch.empty_like(Pd)
    dh.coulomb(Pd, J)
    dh.exchange(Pa, K, symmetric=True)
    torch.cuda.synchronize()
    dh.close()
    for what, A, B in (("J", Jd, J), ("K", Kd, K)):
        err = float((A - B).abs().max() / B.abs().max())
        print(f"N2 {what} device vs host tables: {err:.2e}")
        assert err <= 1e-12, what
    del Pd, Pa, Jd, Kd, J, K
