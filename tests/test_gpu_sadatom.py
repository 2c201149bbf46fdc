"""GPU parity of the spherically averaged atom's Fock build
(src/sadatom/basis.cpp:186-429: coulomb, exchange, rs_exchange; the XC of
src/sadatom/dftgrid.cpp) through hfg_sadatom_*.

Bars: J and K within 1e-10 of the largest entry against the oracle's
restatement (oracle/sadatom.py, which tabulates its own integrals); the
split exchange within 1e-12; the host entries equal to the device ones bit
for bit; the reference's Ne Hartree-Fock energy (tests/README.md) recovered
to 1e-8 Eh from the device J and K at the converged closed-shell density;
the reference's He LDA total and components (tests/refs/ci.json) to 1e-8 Eh
from the device J and XC; the XC block equal to the m-resolved atom's at a
spherical density (LDA and PBE) to 1e-10.
"""
import math

import numpy as np
import pytest

import helfem_gb300 as hg
from oracle import sadatom as sad
from oracle import scf as oscf
from oracle import tabulate as tab
from oracle.yukawa import yukawa_tables
from gpu_util import from_dev, to_dev, torch_cuda

pytestmark = pytest.mark.gpu
TOL = 1e-10

CASES = [
    # Z, lmax, nelem, nnodes
    (2, 0, 4, 15),
    (10, 1, 5, 15),
    (26, 2, 6, 10),
    (54, 3, 5, 7),
]


def channel_density(nrad, nocc, seed):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((nrad, nocc))
    return C @ C.T


def stack(torch, mats):
    return torch.stack([to_dev(torch, M) for M in mats]).contiguous()


def rel(A, B):
    return float(np.abs(A - B).max() / np.abs(B).max())


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"Z{c[0]}_l{c[1]}")
def test_sadatom_jk_match_oracle(case):
    torch = torch_cuda()
    Z, lmax, nel, nn = case
    bval = tab.get_grid(40.0, nel, 4, 2.0)
    a = hg.SadAtom(Z, bval, lmax, nnodes=nn)
    A = tab.build_atom(Z, nn, bval, lmax, 0)
    assert a.nrad == A.nrad
    P = [channel_density(A.nrad, 3, 20 + l) for l in range(lmax + 1)]
    Prad = sum(P)
    # J of the radial density
    Pd = to_dev(torch, Prad)
    Jd = torch.full_like(Pd, np.nan)
    a.coulomb(Pd, Jd)
    torch.cuda.synchronize()
    Jref = sad.coulomb(A, Prad)
    assert rel(from_dev(Jd), Jref) < TOL
    assert np.array_equal(a.coulomb_host(Prad), from_dev(Jd))
    # K of the channel densities: general and symmetric, FP64 and split
    Kref = sad.exchange(A, P)
    scale = max(np.abs(k).max() for k in Kref)
    Pc = stack(torch, P)
    for symmetric in (False, True):
        for split in (False, True):
            Kd = torch.full_like(Pc, np.nan)
            a.exchange(Pc, Kd, symmetric=symmetric, split=split)
            torch.cuda.synchronize()
            tol = 1e-12 if split else TOL
            for l in range(lmax + 1):
                err = float(np.abs(from_dev(Kd[l]) - Kref[l]).max() / scale)
                assert err < tol, (symmetric, split, l, err)
            Kh = a.exchange_host(P, symmetric=symmetric, split=split)
            for l in range(lmax + 1):
                assert np.array_equal(Kh[l], from_dev(Kd[l])), (symmetric, split, l)
    a.close()


def test_sadatom_yukawa_exchange_matches_oracle():
    torch = torch_cuda()
    Z, lmax, nel, nn, lam = 10, 2, 4, 15, 0.7
    bval = tab.get_grid(40.0, nel, 4, 2.0)
    a = hg.SadAtom(Z, bval, lmax, nnodes=nn)
    a.compute_yukawa(lam)
    A = yukawa_tables(tab.build_atom(Z, nn, bval, lmax, 0), lam)
    P = [channel_density(a.nrad, 4, 40 + l) for l in range(lmax + 1)]
    Kref = sad.exchange(A, P)
    scale = max(np.abs(k).max() for k in Kref)
    Kd = torch.full_like(stack(torch, P), np.nan)
    a.rs_exchange(stack(torch, P), Kd, symmetric=True)
    torch.cuda.synchronize()
    for l in range(lmax + 1):
        assert float(np.abs(from_dev(Kd[l]) - Kref[l]).max() / scale) < TOL, l
    Kh = a.rs_exchange_host(P, symmetric=True)
    for l in range(lmax + 1):
        assert np.array_equal(Kh[l], from_dev(Kd[l]))
    a.close()


def test_sadatom_fock_build_recovers_ne_energy():
    """The reference's Ne HF total (lmax = mmax = 1, 5 elements, zexp 2,
    Rmax 40) from the spherically averaged Fock build run on the GPU, at the
    closed-shell density the oracle SCF converges to: Ekin and Enuc from the
    handle's one-electron blocks, Ecoul and Exx from hfg_sadatom_coulomb /
    hfg_sadatom_exchange with the reference SCF's density scaling."""
    torch_cuda()
    bval = tab.get_grid(40.0, 5, 4, 2.0)
    Af = tab.build_atom(10, 15, bval, 1, 1)
    res = oscf.run_scf(Af, 5, 5, "hf")
    assert res.converged and abs(res.Etot - -128.5470981094) < 1e-8
    a = hg.SadAtom(10, bval, 1)
    nr = a.nrad
    T, V = a.kinetic(), a.nuclear()
    Pl = sad.channel_densities(Af, res.Pa + res.Pb, 1)
    e = sad.fock_energies(a.coulomb_host, a.exchange_host,
                          [T[l * nr:(l + 1) * nr, l * nr:(l + 1) * nr] for l in range(2)], V[:nr, :nr], Pl)
    print("sadatom Ne energies from the GPU J/K:", e)
    for k in ("Ecoul", "Exx", "Etot"):
        assert abs(e[k] - getattr(res, k)) < 1e-9 * max(1.0, abs(getattr(res, k))), k
    assert abs(e["Etot"] - -128.5470981094) < 1e-8
    a.close()


def test_sadatom_refuses_driver_and_xc():
    torch_cuda()
    a = hg.SadAtom(2, tab.get_grid(40.0, 3, 4, 2.0), 0)
    with pytest.raises(hg.HfgError):
        a.scf(1, 1, "hf")
    with pytest.raises(hg.HfgError):
        a.dft_grid()
    a.close()


def test_sadatom_lda_recovers_he_golden():
    """He LDA (Slater + VWN5, lmax = 0, 5 elements, zexp 2, Rmax 40): the
    reference's total (tests/refs/ci.json) from the spherically averaged
    Fock build at the density the oracle SCF converges to, its components
    equal to the oracle's at that density (ci.json's components carry the
    reference run's own convergence, linear in the density error, while the
    total is variational), and that density stationary under the Fock
    matrix T + V + J + Vxc the handle builds (the commutator F P S - S P F
    vanishes)."""
    torch_cuda()
    golden = -2.8348356241
    bval = tab.get_grid(40.0, 5, 4, 2.0)
    A = tab.build_atom(2, 15, bval, 0, 0)
    res = oscf.run_scf(A, 1, 1, "lda_x-lda_c_vwn", conv=1e-12, gtol=1e-10)
    assert res.converged and abs(res.Etot - golden) < 1e-8
    a = hg.SadAtom(2, bval, 0)
    P = res.Pa + res.Pb
    T, V, S = a.kinetic(), a.nuclear(), a.overlap()
    J = a.coulomb_host(P / (4.0 * math.pi))
    H, _, exc, nel = a.xc_host(1, 7, P)
    e = {"Ekin": float(np.sum(P * T)), "Enuc": float(np.sum(P * V)), "Ecoul": 0.5 * float(np.sum(P * J)),
         "Exc": exc}
    e["Etot"] = sum(e.values())
    print("sadatom He LDA from the GPU:", e, "electrons on the grid", nel)
    assert abs(e["Etot"] - golden) < 1e-8
    for k in ("Ekin", "Enuc", "Ecoul", "Exc"):
        ref = getattr(res, k)
        assert abs(e[k] - ref) < 1e-9 * max(1.0, abs(ref)), (k, e[k], ref)
    assert abs(nel - 2.0) < 1e-6
    F = T + V + J + H
    C = F @ P @ S - S @ P @ F
    assert np.abs(C).max() < 1e-7 * np.abs(F).max()
    a.close()


@pytest.mark.parametrize("funcs", [(1, 7), (101, 130)], ids=["lda", "pbe"])
def test_sadatom_xc_matches_m_resolved_atom(funcs):
    """At a spherical density the XC block of the spherically averaged
    handle gives every diagonal (l m, l m) block of the m-resolved atom's XC
    matrix, with the same XC energy: Ne (lmax = mmax = 1) channel densities
    from the converged closed-shell solution, spread as P_l / (2l+1) over the
    m of each l (exactly spherical at every grid point). The radial handle
    integrates the angular part exactly; the m-resolved grid's modified
    Gauss-Chebyshev rule in cos(theta) (16 points for lmax = 1) integrates
    |Y_1m|^2 to 1 + O(1e-9), so its p blocks are the radial block times that
    rule's integral, which the test restates."""
    torch_cuda()
    bval = tab.get_grid(40.0, 5, 4, 2.0)
    Af = tab.build_atom(10, 15, bval, 1, 1)
    res = oscf.run_scf(Af, 5, 5, "hf")
    Pl = sad.channel_densities(Af, res.Pa + res.Pb, 1)
    lv, mv = hg.angular_basis(1, 1)
    nr = Af.nrad
    P = np.zeros((nr * len(lv), nr * len(lv)))
    for ia, l in enumerate(lv):
        P[ia * nr:(ia + 1) * nr, ia * nr:(ia + 1) * nr] = Pl[l] / (2 * l + 1)
    full = hg.Atom(10, bval, lv, mv)
    Hf, _, exc_f, _ = full.xc_host(funcs[0], funcs[1], P)
    a = hg.SadAtom(10, bval, 1)
    Hs, _, exc_s, _ = a.xc_host(funcs[0], funcs[1], sum(Pl))
    assert abs(exc_s - exc_f) < 1e-10 * abs(exc_f)
    n = 4 * 1 + 12  # cos(theta) points of the m-resolved grid (src/atomic/main.cpp:329-331)
    t = np.arange(1, n + 1) * np.pi / (n + 1)
    x = 1 + 2 / np.pi * ((1 + 2 / 3 * np.sin(t) ** 2) * np.cos(t) * np.sin(t)) - 2 * np.arange(1, n + 1) / (n + 1)
    w = 16 / (3 * (n + 1)) * np.sin(t) ** 4
    ang = {(0, 0): 0.5 * w.sum(), (1, 0): 1.5 * (w * x * x).sum(), (1, 1): 0.75 * (w * (1 - x * x)).sum()}
    for ia in range(len(lv)):
        blk = Hf[ia * nr:(ia + 1) * nr, ia * nr:(ia + 1) * nr]
        f = ang[(int(lv[ia]), abs(int(mv[ia])))]
        assert np.abs(blk - f * Hs).max() < 1e-12 * np.abs(Hs).max(), (ia, f)
    full.close()
    a.close()


@pytest.mark.parametrize("split", [False, True], ids=["fp64", "split"])
def test_sadatom_fock_build_cost_against_m_resolved(split):
    """On the Kr benchmark grid (40 elements, r_i = 61^(i/40) - 1, l <= 2) the
    spherically averaged Fock build (3 channels, nbf 1677) against the
    m-resolved one of the same atom (9 angular functions, nbf 5031): J + K
    of a spherical density, CUDA events over 10 builds after 2 warm-up
    builds, printed; the averaged build must be the cheaper one."""
    torch = torch_cuda()
    b = hg.get_grid(60.0, 40, 4, 1.0)
    lv, mv = hg.angular_basis(2, 2)
    full = hg.Atom(36, b, lv, mv)
    s = hg.SadAtom(36, b, 2)
    nr = s.nrad
    Pl = [channel_density(nr, 4, 60 + l) for l in range(3)]
    Pf = np.zeros((full.nbf, full.nbf))
    for ia, l in enumerate(lv):
        Pf[ia * nr:(ia + 1) * nr, ia * nr:(ia + 1) * nr] = Pl[l] / (2 * l + 1)
    st = torch.cuda.current_stream()

    def timed(step):
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(10):
            step()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 10

    Pfd = to_dev(torch, Pf)
    Jf, Kf = torch.empty_like(Pfd), torch.empty_like(Pfd)

    def full_step():
        full.coulomb(Pfd, Jf, stream=st)
        full.exchange(Pfd, Kf, symmetric=True, split=split, stream=st)

    Prd = to_dev(torch, sum(Pl))
    Pcd = stack(torch, Pl)
    Js, Ks = torch.empty_like(Prd), torch.empty_like(Pcd)

    def sad_step():
        s.coulomb(Prd, Js, stream=st)
        s.exchange(Pcd, Ks, symmetric=True, split=split, stream=st)

    t_full, t_sad = timed(full_step), timed(sad_step)
    print(f"Kr grid J+K ({'split' if split else 'fp64'}): m-resolved {t_full:.3f} ms, "
          f"spherically averaged {t_sad:.3f} ms ({t_full / t_sad:.1f}x)")
    assert t_sad < t_full
    full.close()
    s.close()
