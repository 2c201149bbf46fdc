"""Helpers shared by the GPU parity tests (device buffers through torch)."""
import numpy as np

import helfem_gb300 as hg
from oracle import FockOracle
from oracle import tabulate as tab


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch


def to_dev(torch, M: np.ndarray):
    """Column-major nbf x nbf host matrix -> device buffer with the same layout."""
    return torch.from_numpy(np.ascontiguousarray(M.T)).cuda()  # row-major of M^T == col-major of M


def from_dev(t) -> np.ndarray:
    return t.cpu().numpy().T.copy()


def relerr(A, B):
    return float(np.abs(A - B).max() / max(np.abs(B).max(), 1e-300))


def make_pair(Z, lmax, mmax, nelem, nnodes=15, rmax=40.0, zexp=2.0):
    b = tab.get_grid(rmax, nelem, 4, zexp)
    lv, mv = hg.angular_basis(lmax, mmax)
    A = hg.Atom(Z, b, lv, mv, nnodes=nnodes)
    O = tab.build_atom(Z, nnodes, b, lmax, mmax)
    return A, O


def random_density(nbf, nocc, seed, S=None):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((nbf, nocc))
    if S is not None:  # Loewdin-orthonormalise in the metric S
        M = C.T @ S @ C
        w, v = np.linalg.eigh(M)
        C = C @ (v @ np.diag(w ** -0.5) @ v.T)
    return C @ C.T
