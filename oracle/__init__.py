"""Oracle: CPU restatement of HelFEM's atomic Fock-build path.

TEST INFRASTRUCTURE ONLY. The product (``helfem_gb300``) never imports,
links or executes anything in this package; only ``tests/``, the smoke check
in ``__graft_entry__.py`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` use it, and there only as the oracle or as the timed CPU
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
_DLIB = os.path.join(_HERE, "_build", "libdfock_ref.so")
_lock = threading.Lock()
_lib = None
_dlib = None


def _compile(src_name: str, out: str, force: bool) -> str:
    os.makedirs(os.path.dirname(out), exist_ok=True)
    src = os.path.join(_HERE, src_name)
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        tmp = out + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                               src, "-o", tmp])
        os.replace(tmp, out)
    return out


def build(force: bool = False) -> str:
    """Compile the C++ oracles (plain g++, OpenMP): atomic and diatomic."""
    _compile("dfock_ref.cpp", _DLIB, force)
    return _compile("fock_ref.cpp", _LIB, force)


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
            _lib.ora_set_threads.argtypes = [ctypes.c_int]
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


# ---------------------------------------------------------------------------
# Diatomic (prolate spheroidal) basis
# ---------------------------------------------------------------------------


class _OraDiatomic(ctypes.Structure):
    _fields_ = [
        ("nrad", ctypes.c_int), ("nang", ctypes.c_int), ("nel", ctypes.c_int), ("nn", ctypes.c_int),
        ("nlm", ctypes.c_int), ("Lmax", ctypes.c_int), ("mmax", ctypes.c_int), ("Rhalf", ctypes.c_double),
        ("lval", ctypes.c_void_p), ("mval", ctypes.c_void_p), ("first", ctypes.c_void_p), ("ni", ctypes.c_void_p),
        ("lm_L", ctypes.c_void_p), ("lm_M", ctypes.c_void_p),
        ("P0", ctypes.c_void_p), ("P2", ctypes.c_void_p), ("Q0", ctypes.c_void_p), ("Q2", ctypes.c_void_p),
        ("cdB", ctypes.c_void_p), ("cdB_off", ctypes.c_void_p), ("cds", ctypes.c_void_p),
        ("cds_off", ctypes.c_void_p), ("cd_rank", ctypes.c_void_p),
        ("coef", ctypes.c_void_p), ("modc", ctypes.c_void_p),
    ]


def dlib():
    global _dlib
    with _lock:
        if _dlib is None:
            _dlib = ctypes.CDLL(_compile("dfock_ref.cpp", _DLIB, False))
            _dlib.ora_dexchange.argtypes = [ctypes.POINTER(_OraDiatomic), ctypes.c_void_p, ctypes.c_void_p]
            _dlib.ora_dexchange.restype = None
            _dlib.ora_dexchange_blocks.argtypes = [ctypes.POINTER(_OraDiatomic), ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_int]
            _dlib.ora_dexchange_blocks.restype = None
            _dlib.ora_num_threads_d.restype = ctypes.c_int
    return _dlib


class DiatomicOracle:
    """J (numpy) and K (compiled, OpenMP) of a diatomic basis from
    ``diatomic.build_diatomic`` tables; inputs and outputs are pure-basis
    (boundary-removed) matrices, as the reference's coulomb/exchange take."""

    def __init__(self, D):
        from . import diatomic as dia
        self.D = D
        nel, nlm, nn = D.nel, len(D.lm), D.nnodes
        keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(np.asarray(x, dtype=dt))
            keep.append(a)
            return a.ctypes.data

        pads = {}
        for name in ("P0", "P2", "Q0", "Q2"):
            buf = np.zeros((nlm, nel, nn, nn))
            src = getattr(D, name)
            for i in range(nlm):
                for e in range(nel):
                    m = src[i][e]
                    buf[i, e, :m.shape[0], :m.shape[1]] = m.T  # row-major (c, r) -> column-major tile
            pads[name] = buf
        cb, cs, boff, soff, rank = [], [], [], [], []
        ob = os_ = 0
        for i in range(nlm):
            for e in range(nel):
                B = D.cdB[i][e]
                boff.append(ob); cb.append(B.ravel(order="F")); ob += B.size
                soff.append(os_); cs.append(D.cds[i][e]); os_ += D.cds[i][e].size
                rank.append(B.shape[1])
        co, mo, Lmax, mmax = dia.gaunt_tables(D)
        self.s = _OraDiatomic(
            D.nrad, D.nang, nel, nn, nlm, Lmax, mmax, D.Rhalf,
            arr(D.lval, np.int32), arr(D.mval, np.int32), arr(D.first, np.int32), arr(D.ni, np.int32),
            arr([L for L, _ in D.lm], np.int32), arr([M for _, M in D.lm], np.int32),
            arr(pads["P0"], np.float64), arr(pads["P2"], np.float64), arr(pads["Q0"], np.float64),
            arr(pads["Q2"], np.float64),
            arr(np.concatenate(cb) if cb else np.zeros(1), np.float64), arr(boff, np.int64),
            arr(np.concatenate(cs) if cs else np.zeros(1), np.float64), arr(soff, np.int64),
            arr(rank, np.int32), arr(co, np.float64), arr(mo, np.float64))
        self._keep = keep

    def coulomb(self, Ppure: np.ndarray) -> np.ndarray:
        from . import diatomic as dia
        return dia.coulomb(self.D, np.asarray(Ppure, dtype=np.float64))

    def exchange(self, Ppure: np.ndarray) -> np.ndarray:
        Pd = np.asfortranarray(self.D.expand(np.asarray(Ppure, dtype=np.float64)))
        Kd = np.zeros_like(Pd, order="F")
        dlib().ora_dexchange(ctypes.byref(self.s), Pd.ctypes.data, Kd.ctypes.data)
        return self.D.remove(Kd)

    def exchange_dummy_blocks(self, Pdummy: np.ndarray, jk) -> np.ndarray:
        """K over the dummy basis restricted to the output blocks jk (j + k*nang),
        from an already expanded (Fortran-ordered) density: a bounded sample
        of the full build for CPU timing."""
        Pd = np.asfortranarray(Pdummy, dtype=np.float64)
        Kd = np.zeros_like(Pd, order="F")
        jk = np.ascontiguousarray(jk, dtype=np.int32)
        dlib().ora_dexchange_blocks(ctypes.byref(self.s), Pd.ctypes.data, Kd.ctypes.data, jk.ctypes.data, len(jk))
        return Kd
