"""Oracle (test infrastructure only): screened-nucleus model potentials for
the SCF guess, restated in numpy.

The product is compared against it. Only tests, the smoke check and the
CPU-baseline leg of the benchmark may import it.

Restated (paths inside the HelFEM project):

* ``src/general/gsz.cpp:51-58`` Z_thomasfermi: the Thomas-Fermi screening
  function as fitted by Oulne (arXiv physics/0511017),
  Z(r) = Z (1 + a sqrt(x) + b x exp(-g sqrt(x)))^2 exp(-2 a sqrt(x)),
  x = r (128 Z / (9 pi^2))^(1/3).
* ``src/general/model_potential.cpp:53-55`` TFAtom::V = -Z(r)/r.
* ``src/atomic/TwoDBasis.cpp:444-455`` model_potential: the element
  integrals int B_a B_b V(r) dr (``libhelfem/src/RadialBasis.cpp:605-619``)
  assembled like the nuclear attraction, one radial block per angular
  function.
"""
from __future__ import annotations

import numpy as np

from . import tabulate as tab

TF_A, TF_B, TF_G = 0.7280642371, -0.5430794693, 0.3612163121


def thomas_fermi_charge(r, Z: int):
    x = np.asarray(r, float) * np.cbrt(128.0 * Z / (9.0 * np.pi ** 2))
    sx = np.sqrt(x)
    return Z * (1.0 + TF_A * sx + TF_B * x * np.exp(-TF_G * sx)) ** 2 * np.exp(-2.0 * TF_A * sx)


def thomas_fermi_matrix(atom: tab.AtomTables, ngl: int = 400) -> np.ndarray:
    """nbf x nbf matrix of V = -Z_TF(r)/r in the atom's basis (R = B/r form,
    so the element integrand is R_a R_b (-Z_TF(r)) r). Z_TF has a sqrt(r)
    term, so on the element at the nucleus a Gauss rule converges only
    algebraically: a plain high-order rule (converged to ~2e-14 relative at
    400 points) keeps this check independent of the product's graded rule."""
    rad = atom.rad
    x, w = tab.gauss_legendre(ngl)
    blocks = []
    for e in range(rad.nel):
        r = rad.coord(x, e)
        R = rad.R(x, e)
        wt = -w * rad.sf(e) * r * thomas_fermi_charge(r, atom.Z)
        blocks.append((R * wt[:, None]).T @ R)
    Vr = rad.assemble(blocks)
    n = rad.nbf
    V = np.zeros((n * atom.nang, n * atom.nang))
    for ia in range(atom.nang):
        V[ia * n:(ia + 1) * n, ia * n:(ia + 1) * n] = Vr
    return V
