"""Oracle: CPU restatement of HelFEM's atomic Fock-build path.

TEST INFRASTRUCTURE ONLY. The product (``helfem_gb300``) never imports,
links or executes anything in this package; only ``tests/``, the smoke check
in ``__graft_entry__.py`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` use it, and there only as the checker or as the timed CPU
baseline.

Parity pins: ``tests/test_oracle_golden.py`` checks this oracle against the
reference's own recorded SCF energies (``tests/refs/ci.json``,
``tests/README.md``) and Gaunt goldens (``src/general/gaunt_test.cpp``),
copied as small fixtures into ``tests/golden/`` by ``tests/golden/make_golden.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

from . import tabulate  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libfock_ref.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the C++ oracle (plain g++, OpenMP)."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    src = os.path.join(_HERE, "fock_ref.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        tmp = _LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                               src, "-o", tmp])
        os.replace(tmp, _LIB)
    return _LIB


class _OraAtom(ctypes.Structure):
    _fields_ = [
        ("nrad", ctypes.c_int), ("nang", ctypes.c_int), ("nel", ctypes.c_int), ("NL", ctypes.c_int),
        ("gmax", ctypes.c_int),
        ("lval", ctypes.c_void_p), ("mval", ctypes.c_void_p),
        ("first", ctypes.c_void_p), ("ni", ctypes.c_void_p),
        ("rs", ctypes.c_void_p), ("rs_off", ctypes.c_void_p),
        ("rb", ctypes.c_void_p), ("rb_off", ctypes.c_void_p),
        ("chol", ctypes.c_void_p), ("chol_off", ctypes.c_void_p), ("chol_rank", ctypes.c_void_p),
        ("gaunt", ctypes.c_void_p),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            for fn in ("ora_coulomb", "ora_exchange"):
                getattr(_lib, fn).argtypes = [ctypes.POINTER(_OraAtom), ctypes.c_void_p, ctypes.c_void_p]
                getattr(_lib, fn).restype = None
            _lib.ora_num_threads.restype = ctypes.c_int
    return _lib


def gaunt_table(gmax: int) -> np.ndarray:
    """Dense table g[a, ma, b, mb, c] = coeff(a, ma, b, mb, c)."""
    w = 2 * gmax + 1
    G = np.zeros((gmax + 1, w, gmax + 1, w, gmax + 1))
    for a in range(gmax + 1):
        for ma in range(-a, a + 1):
            for b in range(gmax + 1):
                for mb in range(-b, b + 1):
                    for c in range(abs(a - b), min(a + b, gmax) + 1):
                        G[a, ma + gmax, b, mb + gmax, c] = tabulate.gaunt(a, ma, b, mb, c)
    return G


class FockOracle:
    """Packs the tables of one atom for the C++ J/K restatement.

    ``tables`` may come from ``tabulate.build_atom`` or from any object with
    the same fields (the parity tests feed the product's own tables here so
    that J/K are compared on identical integrals).
    """

    def __init__(self, A, gaunt=None):
        self.A = A
        rad = A.rad
        nel, NL = rad.nel, A.NL
        self.nrad, self.nang = A.nrad, A.nang
        self.nbf = self.nrad * self.nang
        keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(np.asarray(x, dtype=dt))
            keep.append(a)
            return a.ctypes.data

        rs, rb, ch = [], [], []
        rs_off, rb_off, ch_off, rank = [], [], [], []
        o1 = o2 = o3 = 0
        for L in range(NL):
            for e in range(nel):
                m = np.asarray(A.rs[L][e])
                rs_off.append(o1); rs.append(m.ravel(order="F")); o1 += m.size
                mb = A.rb[L][e]
                rb_off.append(o2)
                if mb is not None:
                    mb = np.asarray(mb); rb.append(mb.ravel(order="F")); o2 += mb.size
                c = np.asarray(A.chol[L][e])
                ch_off.append(o3); ch.append(c.ravel(order="F")); o3 += c.size
                rank.append(c.shape[1])
        gmax = 2 * int(np.max(A.lval))
        if gaunt is None:
            gaunt = gaunt_table(gmax)
        self.gaunt = gaunt
        self.s = _OraAtom(
            self.nrad, self.nang, nel, NL, gmax,
            arr(A.lval, np.int32), arr(A.mval, np.int32),
            arr(rad.first, np.int32), arr([rad.nprim(e) for e in range(nel)], np.int32),
            arr(np.concatenate(rs), np.float64), arr(rs_off, np.int64),
            arr(np.concatenate(rb) if rb else np.zeros(1), np.float64), arr(rb_off, np.int64),
            arr(np.concatenate(ch), np.float64), arr(ch_off, np.int64), arr(rank, np.int32),
            arr(gaunt, np.float64),
        )
        self._keep = keep

    def coulomb(self, P: np.ndarray) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros((self.nbf, self.nbf), order="F")
        lib().ora_coulomb(ctypes.byref(self.s), P.ctypes.data, J.ctypes.data)
        return J

    def exchange(self, P: np.ndarray) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        K = np.zeros((self.nbf, self.nbf), order="F")
        lib().ora_exchange(ctypes.byref(self.s), P.ctypes.data, K.ctypes.data)
        return K
