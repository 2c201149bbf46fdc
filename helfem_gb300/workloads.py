"""Seeded synthetic atom workloads for the batched and streaming benchmarks.

Batch (many atomic SCF solves): Z uniform in 1..zmax, element count uniform
in a range, nodes per element from {10, 13, 15, 17}, Rmax uniform in
[40, 80] bohr, lmax from the occupied shells, HF or LDA (Slater + PW92)
50/50. Stream: Poisson arrivals; Z in 1..zmax with charge -1..+3,
spin-restricted or unrestricted, HF / LDA / PBE, 15-node elements.

Occupations are fixed per angular momentum from Madelung-order filling of
each spin and shared equally over the 2l+1 m components (spherically
averaged open shells), which makes per-(l,m) symmetry blocks exact and the
solves robust.
"""
from __future__ import annotations

import numpy as np

# Madelung (n + l, n) filling order
_ORDER = [(1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (4, 0), (3, 2), (4, 1), (5, 0), (4, 2), (5, 1), (6, 0), (4, 3),
          (5, 2), (6, 1), (7, 0), (5, 3), (6, 2), (7, 1)]


def occupied_lmax(nel: int) -> int:
    """Largest l among the subshells occupied by nel electrons (Madelung)."""
    left, lmax = nel, 0
    for n, l in _ORDER:
        if left <= 0:
            break
        lmax = max(lmax, l)
        left -= 2 * (2 * l + 1)
    return lmax


def l_occupations(nela: int, nelb: int, lmax: int) -> np.ndarray:
    """Alpha/beta electrons per l from Madelung-order filling of each spin,
    [lmax+1][2]; used as spherically averaged fixed occupations."""
    out = np.zeros((lmax + 1, 2))
    for s, n in enumerate((nela, nelb)):
        left = n
        for _, l in _ORDER:
            if left <= 0:
                break
            take = min(left, 2 * l + 1)
            out[l, s] += take
            left -= take
    return out


def grid(rmax: float, nelem: int, zexp: float = 2.0) -> np.ndarray:
    up = np.log(rmax + 1.0) ** (1.0 / zexp)
    t = np.linspace(0.0, up, nelem + 1)
    b = np.exp(t ** zexp) - 1.0
    b[0], b[-1] = 0.0, rmax
    return b


def angular(lmax: int, mmax: int):
    lv, mv = [], []
    for mabs in range(mmax + 1):
        for l in range(mabs, lmax + 1):
            lv.append(l)
            mv.append(mabs)
            if mabs > 0:
                lv.append(l)
                mv.append(-mabs)
    return np.array(lv, np.int32), np.array(mv, np.int32)


def batch_atoms(n: int, seed: int = 2024, zmax: int = 86, nel_range=(10, 60), nodes=(10, 13, 15, 17),
                rmax_range=(40.0, 80.0)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        Z = int(rng.integers(1, zmax + 1))
        lmax = occupied_lmax(Z)
        nelem = int(rng.integers(nel_range[0], nel_range[1] + 1))
        nn = int(rng.choice(nodes))
        rmax = float(rng.uniform(*rmax_range))
        method = "hf" if rng.random() < 0.5 else "lda_x-lda_c_pw"
        lv, mv = angular(lmax, lmax)
        nela, nelb = (Z + 1) // 2, Z // 2
        out.append(dict(Z=Z, nela=nela, nelb=nelb, restricted=True, method=method, nnodes=nn,
                        bval=grid(rmax, nelem), lval=lv, mval=mv, l_occ=l_occupations(nela, nelb, lmax)))
    return out


def stream_atoms(n: int, seed: int = 7, zmax: int = 86, nel_range=(10, 80)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        Z = int(rng.integers(1, zmax + 1))
        q = int(rng.integers(-1, 4))
        nel = max(Z - q, 1)
        lmax = occupied_lmax(nel)
        nelem = int(rng.integers(nel_range[0], nel_range[1] + 1))
        method = ["hf", "lda_x-lda_c_vwn", "gga_x_pbe-gga_c_pbe"][int(rng.integers(0, 3))]
        restricted = bool(rng.random() < 0.5)
        lv, mv = angular(lmax, lmax)
        nela, nelb = (nel + 1) // 2, nel // 2
        out.append(dict(Z=Z, nela=nela, nelb=nelb, restricted=restricted, method=method, nnodes=15,
                        bval=grid(40.0, nelem), lval=lv, mval=mv, l_occ=l_occupations(nela, nelb, lmax)))
    return out
