"""helfem_gb300: GB300 Fock-build engine for HelFEM's atomic finite-element basis.

Python mirror of the C ABI in ``include/helfem_gb300.h`` (ctypes). The
compute path is the in-tree CUDA library ``libhelfem_gb300.so``; there is no
CPU fallback: importing this package without the built library raises.

Reference interfaces mirrored (HelFEM project paths):
  ``TwoDBasisT::coulomb / exchange / compute_tei``  src/atomic/TwoDBasis.h:180-227
  ``TwoDBasisT::overlap / kinetic / nuclear``       src/atomic/TwoDBasis.h:201-207
  ``atomic::basis::angular_basis``                  src/atomic/basis.cpp:179-203
  ``grid::get_grid``                                libhelfem/include/grid.h:37-101
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhelfem_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA extension first "
        "(python helfem_gb300/build.py or __graft_entry__.build())")

_lib = ctypes.CDLL(LIB_PATH)

HFG_OK, HFG_ERR_ARG, HFG_ERR_CUDA, HFG_ERR_STATE, HFG_ERR_NOMEM, HFG_ERR_INTERNAL = range(6)


class HfgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"helfem_gb300 error {status}: {msg}")
        self.status = status


class _Desc(ctypes.Structure):
    _fields_ = [("Z", ctypes.c_int), ("nnodes", ctypes.c_int), ("nquad", ctypes.c_int),
                ("nelem", ctypes.c_int), ("bval", ctypes.POINTER(ctypes.c_double)),
                ("nang", ctypes.c_int), ("lval", ctypes.POINTER(ctypes.c_int)),
                ("mval", ctypes.POINTER(ctypes.c_int)), ("chol_tol", ctypes.c_double),
                ("host_only", ctypes.c_int)]


class _Dims(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nrad", "nang", "nbf", "nelem", "nnodes", "NL", "rmax")]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_SIGS = {
    "hfg_last_error": ([], ctypes.c_char_p),
    "hfg_grid": ([ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, _D], ctypes.c_int),
    "hfg_angular_basis": ([ctypes.c_int, ctypes.c_int, _I, _I, _I], ctypes.c_int),
    "hfg_atom_create": ([ctypes.POINTER(_Desc), ctypes.POINTER(_P)], ctypes.c_int),
    "hfg_atom_destroy": ([_P], ctypes.c_int),
    "hfg_tc_selftest": ([ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                         ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         ctypes.c_int], ctypes.c_int),
    "hfg_tc_peak": ([ctypes.c_int, ctypes.c_int, _D, _D], ctypes.c_int),
    "hfg_atom_tc_work": ([_P, ctypes.c_int, _D], ctypes.c_int),
    "hfg_atom_get_dims": ([_P, ctypes.POINTER(_Dims)], ctypes.c_int),
    "hfg_overlap": ([_P, _D], ctypes.c_int),
    "hfg_kinetic": ([_P, _D], ctypes.c_int),
    "hfg_nuclear": ([_P, _D], ctypes.c_int),
    "hfg_atom_radial_tables": ([_P, ctypes.c_int, ctypes.c_int, _I, _D, _D, _I, _D], ctypes.c_int),
    "hfg_gaunt": ([ctypes.c_int] * 5 + [_D], ctypes.c_int),
    "hfg_coulomb": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_coulomb_acc": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_exchange": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_exchange_ex": ([_P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_coulomb_ex": ([_P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_jk": ([_P, _P, _P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_coulomb_noalloc": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_coulomb_host": ([_P, _D, _D], ctypes.c_int),
    "hfg_exchange_host": ([_P, _D, _D], ctypes.c_int),
    "hfg_exchange_host_ex": ([_P, _D, _D, ctypes.c_int], ctypes.c_int),
    "hfg_jk_host": ([_P, _D, _D, _D, _D, ctypes.c_int], ctypes.c_int),
    "hfg_host_copy_bytes": ([_P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "hfg_sadatom_create": ([ctypes.c_void_p, ctypes.POINTER(_P)], ctypes.c_int),
    "hfg_sadatom_coulomb": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_sadatom_exchange": ([_P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_sadatom_rs_exchange": ([_P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_sadatom_coulomb_host": ([_P, _D, _D], ctypes.c_int),
    "hfg_sadatom_exchange_host": ([_P, _D, _D, ctypes.c_int], ctypes.c_int),
    "hfg_sadatom_rs_exchange_host": ([_P, _D, _D, ctypes.c_int], ctypes.c_int),
    "hfg_sadatom_xc": ([_P, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_double, _P], ctypes.c_int),
    "hfg_sadatom_xc_host": ([_P, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, _D, _D, ctypes.c_double],
                            ctypes.c_int),
    "hfg_fock_diag": ([_P, _P, ctypes.c_int, _P, _P, _P], ctypes.c_int),
    "hfg_atom_autotune": ([_P, ctypes.c_int, _I, _D], ctypes.c_int),
    "hfg_atom_set_partition": ([_P, ctypes.c_int], ctypes.c_int),
    "hfg_atom_compute_yukawa": ([_P, ctypes.c_double], ctypes.c_int),
    "hfg_atom_compute_erfc": ([_P, ctypes.c_double, ctypes.c_int], ctypes.c_int),
    "hfg_atom_erfc_table": ([_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D], ctypes.c_int),
    "hfg_atom_yukawa_tables": ([_P, ctypes.c_int, ctypes.c_int, _D, _D, _D], ctypes.c_int),
    "hfg_rs_exchange": ([_P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_rs_exchange_host": ([_P, _D, _D, ctypes.c_int], ctypes.c_int),
    "hfg_atom_work": ([_P, _P], ctypes.c_int),
    "hfg_dft_grid": ([_P, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "hfg_xc": ([_P, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_double, _P], ctypes.c_int),
    "hfg_xc_host": ([_P, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, _D, _D, ctypes.c_double], ctypes.c_int),
    "hfg_scf_run": ([_P, _P, _P, _D, _P], ctypes.c_int),
    "hfg_engine_create": ([ctypes.c_int, ctypes.c_double, ctypes.POINTER(_P)], ctypes.c_int),
    "hfg_engine_submit": ([_P, _P, _P, ctypes.POINTER(ctypes.c_ulonglong)], ctypes.c_int),
    "hfg_engine_wait": ([_P, ctypes.c_ulonglong, ctypes.c_double, _P], ctypes.c_int),
    "hfg_engine_stats": ([_P, _I, _I, _D], ctypes.c_int),
    "hfg_engine_destroy": ([_P], ctypes.c_int),
    "hfg_profile_enable": ([_P, ctypes.c_int], ctypes.c_int),
    "hfg_profile_classes": ([_P, ctypes.c_uint], ctypes.c_int),
    "hfg_profile_read": ([_P, _P, ctypes.c_int], ctypes.c_int),
    "hfg_diatomic_create": ([_P, ctypes.POINTER(_P)], ctypes.c_int),
    "hfg_diatomic_destroy": ([_P], ctypes.c_int),
    "hfg_diatomic_get_dims": ([_P, _P], ctypes.c_int),
    "hfg_diatomic_pure_indices": ([_P, _I], ctypes.c_int),
    "hfg_diatomic_overlap": ([_P, _D], ctypes.c_int),
    "hfg_diatomic_kinetic": ([_P, _D], ctypes.c_int),
    "hfg_diatomic_nuclear": ([_P, _D], ctypes.c_int),
    "hfg_diatomic_one_electron_block": ([_P, ctypes.c_int, ctypes.c_int, _D, _I], ctypes.c_int),
    "hfg_diatomic_tables": ([_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, _I, _D, _D], ctypes.c_int),
    "hfg_legendre_pq": ([ctypes.c_int, ctypes.c_int, ctypes.c_double, _D, _D], ctypes.c_int),
    "hfg_gaunt_mod": ([ctypes.c_int] * 6 + [_D], ctypes.c_int),
    "hfg_diatomic_coulomb": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_diatomic_exchange": ([_P, _P, _P, ctypes.c_int, _P], ctypes.c_int),
    "hfg_diatomic_coulomb_host": ([_P, _D, _D], ctypes.c_int),
    "hfg_diatomic_exchange_host": ([_P, _D, _D, ctypes.c_int], ctypes.c_int),
    "hfg_diatomic_work": ([_P, _P, _P, _P], ctypes.c_int),
    "hfg_diatomic_dft_grid": ([_P, ctypes.c_int], ctypes.c_int),
    "hfg_diatomic_xc": ([_P, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_double, _P], ctypes.c_int),
    "hfg_diatomic_xc_host": ([_P, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, _D, _D, ctypes.c_double],
                             ctypes.c_int),
}
KERNEL_CLASSES = ("j_contract", "j_scatter", "k_block_norms", "k_tiles", "k_fixup")
XC_IDS = {"lda_x": 1, "lda_c_vwn": 7, "lda_c_pw": 12, "gga_x_pbe": 101, "gga_c_pbe": 130}


def parse_xc(method: str):
    """'lda_x-lda_c_vwn' style names -> (x_id, c_id) (dftfuncs.cpp:94-143)."""
    parts = [p for p in method.split("-") if p]
    ids = [XC_IDS[p] for p in parts]
    return (ids + [0, 0])[:2]
EXCHANGE_SYMMETRIC = 1
EXCHANGE_SPLIT = 2
COULOMB_SPLIT = 4
EXCHANGE_ITEMWISE = 4  # diatomic split form: diagonal tiles one output block per item (comparison schedule)




class _Work(ctypes.Structure):
    _fields_ = [("k_offdiag_flops", ctypes.c_double), ("k_diag_flops", ctypes.c_double),
                ("k_offdiag_sym_flops", ctypes.c_double), ("k_diag_sym_flops", ctypes.c_double),
                ("k_bytes", ctypes.c_double), ("j_flops", ctypes.c_double), ("j_bytes", ctypes.c_double),
                ("n_k_entries", ctypes.c_int), ("n_k_terms", ctypes.c_int)]


class _ScfDesc(ctypes.Structure):
    _fields_ = [("nela", ctypes.c_int), ("nelb", ctypes.c_int), ("restricted", ctypes.c_int),
                ("symmetry", ctypes.c_int), ("x_func", ctypes.c_int), ("c_func", ctypes.c_int),
                ("kfrac", ctypes.c_double), ("maxiter", ctypes.c_int), ("e_tol", ctypes.c_double),
                ("diis_tol", ctypes.c_double), ("fixed_occ", _I), ("n_fixed_blocks", ctypes.c_int),
                ("dftthr", ctypes.c_double), ("frac_aufbau", ctypes.c_int), ("split_exchange", ctypes.c_int),
                ("l_occ", _D), ("n_l_occ", ctypes.c_int)]


class _ScfRes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("Etot", "Ekin", "Enuc", "Ecoul", "Exx", "Exc", "Nel_grid")] + \
               [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("phase_ms", ctypes.c_double * 6)]


PHASES = ("fock", "energies", "ortho_errors", "diis", "eigh_occupy", "density")


class _JobRes(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("scf", _ScfRes), ("queue_ms", ctypes.c_double),
                ("setup_ms", ctypes.c_double), ("scf_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("footprint_bytes", ctypes.c_double), ("error", ctypes.c_char * 256)]


class _Prof(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int * 5), ("ms", ctypes.c_double * 5)]


for _name, (_args, _res) in _SIGS.items():
    _f = getattr(_lib, _name)
    _f.argtypes = _args
    _f.restype = _res


def lib():
    return _lib


def _check(status: int):
    if status != HFG_OK:
        raise HfgError(status, _lib.hfg_last_error().decode())


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def get_grid(rmax: float, nelem: int, igrid: int = 4, zexp: float = 2.0) -> np.ndarray:
    b = np.zeros(nelem + 1)
    _check(_lib.hfg_grid(rmax, nelem, igrid, zexp, _dptr(b)))
    return b


def angular_basis(lmax: int, mmax: int):
    n = ctypes.c_int()
    _check(_lib.hfg_angular_basis(lmax, mmax, ctypes.byref(n), None, None))
    lv = np.zeros(n.value, dtype=np.int32)
    mv = np.zeros(n.value, dtype=np.int32)
    _check(_lib.hfg_angular_basis(lmax, mmax, ctypes.byref(n), lv.ctypes.data_as(_I), mv.ctypes.data_as(_I)))
    return lv, mv


def tc_selftest(A: np.ndarray, B: np.ndarray, a_mn_major: bool = False, b_mn_major: bool = False,
                swap_offsets: bool = False) -> np.ndarray:
    """D = A B^T through the library's tcgen05 operand layouts (A: 128 x K,
    B: N x K, K a multiple of 16; operands rounded to bf16, FP32 sums)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    assert A.shape[0] == 128 and A.shape[1] == B.shape[1] and A.shape[1] % 16 == 0
    D = np.zeros((128, B.shape[0]), dtype=np.float32)
    f = ctypes.POINTER(ctypes.c_float)
    _check(_lib.hfg_tc_selftest(A.ctypes.data_as(f), B.ctypes.data_as(f), D.ctypes.data_as(f), B.shape[0],
                                A.shape[1] // 16, int(a_mn_major), int(b_mn_major), int(swap_offsets)))
    return D


def tc_peak(ctas_per_sm: int = 2, iters: int = 4096) -> dict:
    """Dense bf16 tcgen05 MMA rate of this GPU (M = 128, N = 256, K = 16)."""
    tf, ms = ctypes.c_double(), ctypes.c_double()
    _check(_lib.hfg_tc_peak(ctas_per_sm, iters, ctypes.byref(tf), ctypes.byref(ms)))
    return {"tflops": tf.value, "ms": ms.value, "ctas_per_sm": ctas_per_sm, "iters": iters}


def gaunt(L: int, M: int, l: int, m: int, lp: int) -> float:
    v = ctypes.c_double()
    _check(_lib.hfg_gaunt(L, M, l, m, lp, ctypes.byref(v)))
    return v.value


def _ptr(x):
    """Device pointer of a torch tensor (or an int address)."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous (column-major matrices: pass M.T.contiguous().T)")
        return x.data_ptr()
    raise TypeError("expected a torch CUDA tensor or a device address")


def _stream(stream):
    if stream is None:
        try:
            import torch
            return torch.cuda.current_stream().cuda_stream
        except Exception:  # pragma: no cover
            return 0
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


class Atom:
    """One atomic basis with its cached two-electron tables (FP64) and their
    device copies. Mirrors TwoDBasisT construction + compute_tei.

    tabulate="device" (default) forms the in-element two-electron factors and
    the exchange tensor on the GPU; "host" tabulates everything on the host
    and uploads it. host_only=True builds the host tables only (no GPU)."""

    def __init__(self, Z: int, bval, lval, mval, nnodes: int = 15, nquad: int = 0,
                 chol_tol: float = 0.0, host_only: bool = False, tabulate: str = "device"):
        if tabulate not in ("device", "host"):
            raise ValueError("tabulate must be 'device' or 'host'")
        self.Z = int(Z)
        self.bval = np.ascontiguousarray(bval, dtype=np.float64)
        self.lval = np.ascontiguousarray(lval, dtype=np.int32)
        self.mval = np.ascontiguousarray(mval, dtype=np.int32)
        mode = 1 if host_only else (2 if tabulate == "host" else 0)
        d = _Desc(self.Z, nnodes, nquad, len(self.bval) - 1, _dptr(self.bval), len(self.lval),
                  self.lval.ctypes.data_as(_I), self.mval.ctypes.data_as(_I), chol_tol, mode)
        h = _P()
        _check(_lib.hfg_atom_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        dims = _Dims()
        _check(_lib.hfg_atom_get_dims(h, ctypes.byref(dims)))
        for n, _ in _Dims._fields_:
            setattr(self, n, getattr(dims, n))
        self.nel = self.nelem

    @classmethod
    def from_grid(cls, Z, nelem, rmax, lmax, mmax, igrid=4, zexp=2.0, nnodes=15, **kw):
        lv, mv = angular_basis(lmax, mmax)
        return cls(Z, get_grid(rmax, nelem, igrid, zexp), lv, mv, nnodes=nnodes, **kw)

    def close(self):
        if getattr(self, "_h", None):
            _lib.hfg_atom_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- one-electron (host) ----
    def _full(self, fn):
        M = np.zeros((self.nbf, self.nbf), order="F")
        _check(fn(self._h, _dptr(M)))
        return M

    def overlap(self):
        return self._full(_lib.hfg_overlap)

    def kinetic(self):
        return self._full(_lib.hfg_kinetic)

    def nuclear(self):
        return self._full(_lib.hfg_nuclear)

    def radial_tables(self, L: int, iel: int):
        ni, rank = ctypes.c_int(), ctypes.c_int()
        _check(_lib.hfg_atom_radial_tables(self._h, L, iel, ctypes.byref(ni), None, None, ctypes.byref(rank), None))
        n = ni.value
        rs = np.zeros((n, n), order="F")
        rb = np.zeros((n, n), order="F")
        ch = np.zeros((n * n, rank.value), order="F")
        _check(_lib.hfg_atom_radial_tables(self._h, L, iel, None, _dptr(rs), _dptr(rb), None, _dptr(ch)))
        return rs, rb, ch

    # ---- hot path: device pointers ----
    def coulomb(self, P, J, stream=None, split: bool = False):
        if split:
            _check(_lib.hfg_coulomb_ex(self._h, _ptr(P), _ptr(J), COULOMB_SPLIT, _stream(stream)))
        else:
            _check(_lib.hfg_coulomb(self._h, _ptr(P), _ptr(J), _stream(stream)))

    def jk(self, PJ, J, K, PK=None, stream=None, symmetric: bool = False, split: bool = False,
           split_j: bool = False):
        """J(PJ) and K(PK) (PK defaults to PJ) in one call, J on the handle's
        second stream concurrently with K, joined back into `stream`."""
        PK = PJ if PK is None else PK
        flags = ((EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0) |
                 (COULOMB_SPLIT if split_j else 0))
        _check(_lib.hfg_jk(self._h, _ptr(PJ), _ptr(PK), _ptr(J), _ptr(K), flags, _stream(stream)))

    def coulomb_acc(self, P, F, stream=None):
        _check(_lib.hfg_coulomb_acc(self._h, _ptr(P), _ptr(F), _stream(stream)))

    def coulomb_noalloc(self, P, J, stream=None):
        _check(_lib.hfg_coulomb_noalloc(self._h, _ptr(P), _ptr(J), _stream(stream)))

    def exchange(self, P, K, stream=None, symmetric: bool = False, split: bool = False):
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        if flags:
            _check(_lib.hfg_exchange_ex(self._h, _ptr(P), _ptr(K), flags, _stream(stream)))
        else:
            _check(_lib.hfg_exchange(self._h, _ptr(P), _ptr(K), _stream(stream)))

    def tc_work(self, symmetric: bool = True) -> float:
        """bf16 MMA FLOPs of one split-precision exchange (all entries active)."""
        f = ctypes.c_double()
        _check(_lib.hfg_atom_tc_work(self._h, int(symmetric), ctypes.byref(f)))
        return f.value

    def work(self) -> dict:
        w = _Work()
        _check(_lib.hfg_atom_work(self._h, ctypes.byref(w)))
        return {n: getattr(w, n) for n, _ in _Work._fields_}

    # ---- XC ----
    def dft_grid(self, ldft: int = 0, mdft: int = 0):
        _check(_lib.hfg_dft_grid(self._h, ldft, mdft))

    def xc(self, x_func, c_func, Pa, Ha, Pb=None, Hb=None, energies=None, thr=1e-12, stream=None):
        _check(_lib.hfg_xc(self._h, x_func, c_func, _ptr(Pa), _ptr(Pb) if Pb is not None else None,
                           _ptr(Ha), _ptr(Hb) if Hb is not None else None,
                           _ptr(energies) if energies is not None else None, thr, _stream(stream)))

    def xc_host(self, x_func, c_func, Pa, Pb=None, thr=1e-12):
        """Returns (Ha, Hb or None, Exc, Nel)."""
        Pa = np.asfortranarray(Pa, dtype=np.float64)
        Ha = np.zeros_like(Pa, order="F")
        Pb_ = Hb = None
        if Pb is not None:
            Pb_ = np.asfortranarray(Pb, dtype=np.float64)
            Hb = np.zeros_like(Pa, order="F")
        exc, nel = ctypes.c_double(), ctypes.c_double()
        _check(_lib.hfg_xc_host(self._h, x_func, c_func, _dptr(Pa), _dptr(Pb_) if Pb_ is not None else None,
                                _dptr(Ha), _dptr(Hb) if Hb is not None else None,
                                ctypes.byref(exc), ctypes.byref(nel), thr))
        return Ha, Hb, exc.value, nel.value

    # ---- SCF ----
    def scf(self, nela: int, nelb: int, method: str = "hf", restricted: bool = True, symmetry: int = 1,
            fixed_occ=None, maxiter: int = 0, e_tol: float = 0.0, diis_tol: float = 0.0, stream=None,
            frac_aufbau: bool = False, split: bool = False, l_occ=None) -> dict:
        """Atomic SCF on the device. fixed_occ: dict m -> (n_alpha, n_beta) (symmetry 1);
        l_occ: [lmax+1][2] alpha/beta electrons per l shared equally over m (symmetry 2)."""
        x, c = (0, 0) if method.lower() == "hf" else parse_xc(method)
        occ = None
        nfix = 0
        if fixed_occ is not None:
            ms = sorted(set(int(m) for m in self.mval))
            occ = np.array([v for m in ms for v in fixed_occ.get(m, (0, 0))], dtype=np.int32)
            nfix = len(ms)
        lo = None if l_occ is None else np.ascontiguousarray(np.asarray(l_occ, dtype=np.float64).ravel())
        d = _ScfDesc(nela, nelb, int(restricted), symmetry, x, c, -1.0, maxiter, e_tol, diis_tol,
                     occ.ctypes.data_as(_I) if occ is not None else None, nfix, 0.0, int(frac_aufbau),
                     int(split), lo.ctypes.data_as(_D) if lo is not None else None,
                     len(lo) // 2 if lo is not None else 0)
        r = _ScfRes()
        nspin = 1 if restricted else 2
        eps = np.zeros(self.nbf * nspin)
        _check(_lib.hfg_scf_run(self._h, ctypes.byref(d), ctypes.byref(r), _dptr(eps),
                                _stream(stream) if stream is not None else None))
        out = {n: getattr(r, n) for n, _ in _ScfRes._fields_ if n != "phase_ms"}
        out["phase_ms"] = dict(zip(PHASES, list(r.phase_ms)))
        out["orbital_energies"] = eps
        return out

    # ---- per-kernel timing ----
    def profile_enable(self, capacity: int = 4096):
        _check(_lib.hfg_profile_enable(self._h, capacity))

    def profile_classes(self, names=None):
        """Bracket only these kernel classes (names from KERNEL_CLASSES; None: all)."""
        mask = 0xFFFFFFFF if names is None else sum(1 << KERNEL_CLASSES.index(n) for n in names)
        _check(_lib.hfg_profile_classes(self._h, mask))

    def profile_read(self, reset: bool = True) -> dict:
        pr = _Prof()
        _check(_lib.hfg_profile_read(self._h, ctypes.byref(pr), int(reset)))
        return {n: (pr.launches[i], pr.ms[i]) for i, n in enumerate(KERNEL_CLASSES)}

    # ---- hot path: host arrays (drop-in value semantics) ----
    def coulomb_host(self, P: np.ndarray, out: np.ndarray = None) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros_like(P, order="F") if out is None else out
        assert J.flags.f_contiguous and J.shape == P.shape
        _check(_lib.hfg_coulomb_host(self._h, _dptr(P), _dptr(J)))
        return J

    def exchange_host(self, P: np.ndarray, out: np.ndarray = None, symmetric: bool = False,
                      split: bool = False) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        K = np.zeros_like(P, order="F") if out is None else out
        assert K.flags.f_contiguous and K.shape == P.shape
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        if flags:
            _check(_lib.hfg_exchange_host_ex(self._h, _dptr(P), _dptr(K), flags))
        else:
            _check(_lib.hfg_exchange_host(self._h, _dptr(P), _dptr(K)))
        return K

    def autotune(self, symmetric: bool = True, split: bool = False) -> dict:
        """Pick the exchange work partition by timing candidates (kept for
        later calls on this handle)."""
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        ns, ms = ctypes.c_int(), ctypes.c_double()
        _check(_lib.hfg_atom_autotune(self._h, flags, ctypes.byref(ns), ctypes.byref(ms)))
        return {"nsplit": ns.value, "ms": ms.value}

    # ---- range-separated (Yukawa-screened) exchange ----
    def compute_yukawa(self, lam: float):
        """Screened radial tables for the kernel exp(-lam r12)/r12."""
        _check(_lib.hfg_atom_compute_yukawa(self._h, lam))

    def compute_erfc(self, mu: float, exact_binomial: bool = False):
        """Pair tables of the erfc kernel erfc(mu r12)/r12 (the reference's
        series rule unless exact_binomial); rs_exchange then uses them."""
        _check(_lib.hfg_atom_compute_erfc(self._h, mu, 1 if exact_binomial else 0))

    def erfc_table(self, L: int, iel: int, kel: int):
        """mu (ij|kl) of the element pair, exchange-ordered, (nn^2 x nn^2)."""
        nn = self.nnodes
        out = np.zeros((nn * nn, nn * nn), order="F")
        _check(_lib.hfg_atom_erfc_table(self._h, L, iel, kel, _dptr(out)))
        return out

    def yukawa_tables(self, L: int, iel: int):
        """(r_small, r_big, tk) of the screened tables as stored (padded)."""
        nn = self.nnodes
        rs = np.zeros((nn, nn), order="F")
        rb = np.zeros((nn, nn), order="F")
        tk = np.zeros((nn * nn, nn * nn), order="F")
        _check(_lib.hfg_atom_yukawa_tables(self._h, L, iel, _dptr(rs), _dptr(rb), _dptr(tk)))
        return rs, rb, tk

    def rs_exchange(self, P, K, stream=None, symmetric: bool = False, split: bool = False):
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        _check(_lib.hfg_rs_exchange(self._h, _ptr(P), _ptr(K), flags, _stream(stream)))

    def rs_exchange_host(self, P: np.ndarray, symmetric: bool = False, split: bool = False) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        K = np.zeros_like(P, order="F")
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        _check(_lib.hfg_rs_exchange_host(self._h, _dptr(P), _dptr(K), flags))
        return K

    def set_partition(self, nsplit: int = 0):
        """Exchange work partition as the autotuner would set it (0 = automatic)."""
        _check(_lib.hfg_atom_set_partition(self._h, nsplit))

    def fock_diag(self, F, C, eps, symmetry: int = 1, stream=None):
        """Orbital energies eps (nbf) and AO coefficients C (nbf x nbf) of
        the Fock matrix F per symmetry block (device buffers)."""
        _check(_lib.hfg_fock_diag(self._h, _ptr(F), symmetry, _ptr(C), _ptr(eps), _stream(stream)))

    def jk_host(self, PJ: np.ndarray, PK: np.ndarray = None, J: np.ndarray = None, K: np.ndarray = None,
                symmetric: bool = False, split: bool = False, split_j: bool = False):
        """J(PJ) and K(PK) (PK defaults to PJ: one staging of the density);
        split: K in the split form, split_j: J in float pairs."""
        PJ = np.asfortranarray(PJ, dtype=np.float64)
        PK = PJ if PK is None else np.asfortranarray(PK, dtype=np.float64)
        J = np.zeros_like(PJ, order="F") if J is None else J
        K = np.zeros_like(PJ, order="F") if K is None else K
        assert J.flags.f_contiguous and K.flags.f_contiguous and J.shape == K.shape == PJ.shape
        flags = ((EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0) |
                 (COULOMB_SPLIT if split_j else 0))
        _check(_lib.hfg_jk_host(self._h, _dptr(PJ), _dptr(PK), _dptr(J), _dptr(K), flags))
        return J, K

    def host_copy_bytes(self):
        """(host-to-device, device-to-host) bytes of the last host-pointer
        J/K call on this handle (a symmetric density crosses the link as its
        lower column blocks)."""
        h2d, d2h = ctypes.c_size_t(), ctypes.c_size_t()
        _check(_lib.hfg_host_copy_bytes(self._h, ctypes.byref(h2d), ctypes.byref(d2h)))
        return h2d.value, d2h.value


class _SadDesc(ctypes.Structure):
    _fields_ = [("Z", ctypes.c_int), ("nnodes", ctypes.c_int), ("nquad", ctypes.c_int),
                ("nelem", ctypes.c_int), ("bval", ctypes.POINTER(ctypes.c_double)), ("lmax", ctypes.c_int),
                ("chol_tol", ctypes.c_double), ("host_only", ctypes.c_int)]


class SadAtom(Atom):
    """Spherically averaged atom: the reference's sadatom::basis::TwoDBasis
    (src/sadatom/basis.h) after compute_tei, one radial channel per
    l = 0..lmax. coulomb / exchange / rs_exchange take and return l-channel
    matrices: J of the radial density (nrad x nrad), and K of the channel
    densities as an (lmax+1, nrad, nrad) stack (basis.cpp:186-429). Device
    buffers hold the slices one after the other, each column-major; the
    host methods take and return lists of matrices; xc / xc_host give the
    XC block of every channel from the radial density. compute_yukawa /
    compute_erfc work as for atoms; scf() and dft_grid() are refused."""

    def __init__(self, Z: int, bval, lmax: int, nnodes: int = 15, nquad: int = 0, chol_tol: float = 0.0,
                 host_only: bool = False, tabulate: str = "device"):
        if tabulate not in ("device", "host"):
            raise ValueError("tabulate must be 'device' or 'host'")
        self.Z = int(Z)
        self.lmax = int(lmax)
        self.bval = np.ascontiguousarray(bval, dtype=np.float64)
        self.lval = np.arange(self.lmax + 1, dtype=np.int32)
        self.mval = np.zeros(self.lmax + 1, dtype=np.int32)
        mode = 1 if host_only else (2 if tabulate == "host" else 0)
        d = _SadDesc(self.Z, nnodes, nquad, len(self.bval) - 1, _dptr(self.bval), self.lmax, chol_tol, mode)
        h = _P()
        _check(_lib.hfg_sadatom_create(ctypes.addressof(d), ctypes.byref(h)))
        self._h = h
        dims = _Dims()
        _check(_lib.hfg_atom_get_dims(h, ctypes.byref(dims)))
        for n, _ in _Dims._fields_:
            setattr(self, n, getattr(dims, n))
        self.nel = self.nelem

    @classmethod
    def from_grid(cls, Z, nelem, rmax, lmax, igrid=4, zexp=2.0, nnodes=15, **kw):
        return cls(Z, get_grid(rmax, nelem, igrid, zexp), lmax, nnodes=nnodes, **kw)

    # ---- device pointers ----
    def coulomb(self, P, J, stream=None):
        _check(_lib.hfg_sadatom_coulomb(self._h, _ptr(P), _ptr(J), _stream(stream)))

    def exchange(self, P, K, stream=None, symmetric: bool = False, split: bool = False):
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        _check(_lib.hfg_sadatom_exchange(self._h, _ptr(P), _ptr(K), flags, _stream(stream)))

    def rs_exchange(self, P, K, stream=None, symmetric: bool = False, split: bool = False):
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        _check(_lib.hfg_sadatom_rs_exchange(self._h, _ptr(P), _ptr(K), flags, _stream(stream)))

    # ---- host arrays ----
    def _stack(self, mats):
        mats = list(mats)
        if len(mats) != self.lmax + 1:
            raise ValueError(f"need {self.lmax + 1} channel matrices")
        buf = np.empty((len(mats), self.nrad, self.nrad))
        for l, M in enumerate(mats):
            buf[l] = np.asarray(M, dtype=np.float64).T  # slice memory = column-major M
        return buf

    def coulomb_host(self, P: np.ndarray) -> np.ndarray:
        Pb = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros_like(Pb, order="F")
        _check(_lib.hfg_sadatom_coulomb_host(self._h, _dptr(Pb), _dptr(J)))
        return J

    def _k_host(self, fn, P, symmetric, split):
        buf = self._stack(P)
        out = np.zeros_like(buf)
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        _check(fn(self._h, _dptr(buf), _dptr(out), flags))
        return [np.asfortranarray(out[l].T) for l in range(len(out))]

    def exchange_host(self, P, symmetric: bool = False, split: bool = False):
        return self._k_host(_lib.hfg_sadatom_exchange_host, P, symmetric, split)

    def rs_exchange_host(self, P, symmetric: bool = False, split: bool = False):
        return self._k_host(_lib.hfg_sadatom_rs_exchange_host, P, symmetric, split)

    def xc(self, x_func, c_func, Pa, Ha, Pb=None, Hb=None, energies=None, thr=1e-12, stream=None):
        """XC block of every channel from the radial density (device
        buffers, nrad x nrad column-major); Pb None: Pa is the total."""
        _check(_lib.hfg_sadatom_xc(self._h, x_func, c_func, _ptr(Pa), _ptr(Pb) if Pb is not None else None,
                                   _ptr(Ha), _ptr(Hb) if Hb is not None else None,
                                   _ptr(energies) if energies is not None else None, thr, _stream(stream)))

    def xc_host(self, x_func, c_func, Pa, Pb=None, thr=1e-12):
        """Returns (Ha, Hb or None, Exc, Nel) for the radial density."""
        Pa = np.asfortranarray(Pa, dtype=np.float64)
        Ha = np.zeros_like(Pa, order="F")
        Pb_ = Hb = None
        if Pb is not None:
            Pb_ = np.asfortranarray(Pb, dtype=np.float64)
            Hb = np.zeros_like(Pa, order="F")
        exc, nel = ctypes.c_double(), ctypes.c_double()
        _check(_lib.hfg_sadatom_xc_host(self._h, x_func, c_func, _dptr(Pa), _dptr(Pb_) if Pb_ is not None else None,
                                        _dptr(Ha), _dptr(Hb) if Hb is not None else None,
                                        ctypes.byref(exc), ctypes.byref(nel), thr))
        return Ha, Hb, exc.value, nel.value


def _scf_desc(nela, nelb, method="hf", restricted=True, symmetry=1, fixed=None, nblocks=0, e_tol=0.0,
              diis_tol=0.0, maxiter=0, frac_aufbau=False, split=False, l_occ=None):
    x, c = (0, 0) if method.lower() == "hf" else parse_xc(method)
    return _ScfDesc(nela, nelb, int(restricted), symmetry, x, c, -1.0, maxiter, e_tol, diis_tol,
                    fixed.ctypes.data_as(_I) if fixed is not None else None, nblocks, 0.0, int(frac_aufbau),
                    int(split), l_occ.ctypes.data_as(_D) if l_occ is not None else None,
                    len(l_occ) // 2 if l_occ is not None else 0)


class Engine:
    """Concurrent atomic SCF solves (hfg_engine_*): submit() returns a job id
    at once; wait() returns the result dict (energies, timings)."""

    def __init__(self, n_workers: int = 4, hbm_budget_gb: float = 180.0):
        h = _P()
        _check(_lib.hfg_engine_create(n_workers, hbm_budget_gb, ctypes.byref(h)))
        self._h = h

    def submit(self, Z, bval, lval, mval, nela, nelb, method="hf", restricted=True, nnodes=15, symmetry=1,
               fixed_occ=None, e_tol=0.0, diis_tol=0.0, frac_aufbau=False, split=False, l_occ=None,
               maxiter=0, tabulate="device") -> int:
        if tabulate not in ("device", "host"):
            raise ValueError("tabulate must be 'device' or 'host'")
        bval = np.ascontiguousarray(bval, dtype=np.float64)
        lval = np.ascontiguousarray(lval, dtype=np.int32)
        mval = np.ascontiguousarray(mval, dtype=np.int32)
        ad = _Desc(int(Z), nnodes, 0, len(bval) - 1, _dptr(bval), len(lval), lval.ctypes.data_as(_I),
                   mval.ctypes.data_as(_I), 0.0, 2 if tabulate == "host" else 0)
        occ, nfix = None, 0
        if fixed_occ is not None:
            ms = sorted(set(int(m) for m in mval))
            occ = np.array([v for m in ms for v in fixed_occ.get(m, (0, 0))], dtype=np.int32)
            nfix = len(ms)
        lo = None if l_occ is None else np.ascontiguousarray(np.asarray(l_occ, dtype=np.float64).ravel())
        sd = _scf_desc(nela, nelb, method, restricted, symmetry, occ, nfix, e_tol, diis_tol, maxiter=maxiter,
                       frac_aufbau=frac_aufbau, split=split, l_occ=lo)
        jid = ctypes.c_ulonglong()
        _check(_lib.hfg_engine_submit(self._h, ctypes.byref(ad), ctypes.byref(sd), ctypes.byref(jid)))
        return jid.value

    def wait(self, job_id: int, timeout_s: float = -1.0) -> dict:
        r = _JobRes()
        _check(_lib.hfg_engine_wait(self._h, job_id, timeout_s, ctypes.byref(r)))
        out = {n: getattr(r.scf, n) for n, _ in _ScfRes._fields_ if n != "phase_ms"}
        out["phase_ms"] = dict(zip(PHASES, list(r.scf.phase_ms)))
        out.update(status=r.status, queue_ms=r.queue_ms, setup_ms=r.setup_ms, scf_ms=r.scf_ms,
                   total_ms=r.total_ms, footprint_bytes=r.footprint_bytes, error=r.error.decode())
        return out

    def stats(self):
        q, r, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(_lib.hfg_engine_stats(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(g)))
        return {"queued": q.value, "running": r.value, "in_use_gb": g.value}

    def close(self):
        if getattr(self, "_h", None):
            _check(_lib.hfg_engine_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Diatomic molecules (prolate spheroidal coordinates)
# ---------------------------------------------------------------------------


class _DDesc(ctypes.Structure):
    _fields_ = [("Z1", ctypes.c_int), ("Z2", ctypes.c_int), ("Rhalf", ctypes.c_double), ("nnodes", ctypes.c_int),
                ("nelem", ctypes.c_int), ("bval", _D), ("nang", ctypes.c_int), ("lval", _I), ("mval", _I),
                ("cd_thresh", ctypes.c_double), ("host_only", ctypes.c_int)]


class _DDims(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nrad", "nang", "nel", "nnodes", "ndummy", "nbf", "nlm", "Lmax",
                                             "rmax", "nchan", "nent")]


class _DWork(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("k_offdiag_flops", "k_diag_flops", "k_recouple_flops", "n_entries",
                                                "k_offdiag_sym_flops", "k_diag_sym_flops",
                                                "k_recouple_sym_flops", "n_entries_sym")]


def lm_to_l_m(lmmax):
    """Angular basis of a diatomic from lmax per |m| (the reference's
    lm_to_l_m, src/diatomic/basis.cpp:456-471)."""
    lv, mv = [], []
    for mabs, lmx in enumerate(lmmax):
        for l in range(mabs, int(lmx) + 1):
            lv.append(l)
            mv.append(mabs)
            if mabs > 0:
                lv.append(l)
                mv.append(-mabs)
    return np.array(lv, np.int32), np.array(mv, np.int32)


def legendre_pq(Lmax: int, Mmax: int, mu: float):
    """P[M, L], Q[M, L] of cosh(mu) (Hobson convention), the product's own
    evaluation."""
    P = np.zeros((Mmax + 1) * (Lmax + 1))
    Q = np.zeros_like(P)
    _check(_lib.hfg_legendre_pq(Lmax, Mmax, mu, _dptr(P), _dptr(Q)))
    return P.reshape(Mmax + 1, Lmax + 1), Q.reshape(Mmax + 1, Lmax + 1)


def gaunt_mod(lj, mj, L, M, li, mi) -> float:
    v = ctypes.c_double()
    _check(_lib.hfg_gaunt_mod(lj, mj, L, M, li, mi, ctypes.byref(v)))
    return v.value


class Diatomic:
    """One diatomic basis (the reference's diatomic TwoDBasis after
    compute_tei): Z1 at one end of the bond and Z2 at the other, half bond
    length Rhalf, LIP elements in mu with boundaries ``bval`` and angular
    functions (lval, mval). Matrices are over the pure basis.
    host_only=True builds the host tables only (no GPU); otherwise the
    two-electron primitives are tabulated on the device (tabulate="device")
    or on the host and uploaded (tabulate="host")."""

    def __init__(self, Z1: int, Z2: int, Rhalf: float, bval, lval, mval, nnodes: int = 15,
                 cd_thresh: float = 1e-12, host_only: bool = False, tabulate: str = "device"):
        if tabulate not in ("device", "host"):
            raise ValueError("tabulate must be 'device' or 'host'")
        self._bval = np.ascontiguousarray(bval, dtype=np.float64)
        self._lval = np.ascontiguousarray(lval, dtype=np.int32)
        self._mval = np.ascontiguousarray(mval, dtype=np.int32)
        mode = 1 if host_only else (2 if tabulate == "host" else 0)
        d = _DDesc(Z1, Z2, Rhalf, nnodes, len(self._bval) - 1, _dptr(self._bval), len(self._lval),
                   self._lval.ctypes.data_as(_I), self._mval.ctypes.data_as(_I), cd_thresh, mode)
        h = _P()
        _check(_lib.hfg_diatomic_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        dims = _DDims()
        _check(_lib.hfg_diatomic_get_dims(h, ctypes.byref(dims)))
        self.dims = {n: getattr(dims, n) for n, _ in _DDims._fields_}
        self.nbf = dims.nbf
        self.nrad = dims.nrad
        self.nang = dims.nang
        self.ndummy = dims.ndummy
        self.Z1, self.Z2, self.Rhalf = Z1, Z2, Rhalf
        self.lval, self.mval = self._lval, self._mval

    @classmethod
    def from_grid(cls, Z1, Z2, Rbond, nelem, lmmax, Rmax=40.0, igrid=4, zexp=1.0, nnodes=15, **kw):
        """The reference's diatomic driver set-up (src/diatomic/main.cpp:
        195-217): mu_max = arccosh(Rmax / Rhalf), element grid in mu."""
        import math
        Rhalf = 0.5 * Rbond
        bval = get_grid(math.acosh(Rmax / Rhalf), nelem, igrid, zexp)
        lv, mv = lm_to_l_m(lmmax)
        return cls(Z1, Z2, Rhalf, bval, lv, mv, nnodes=nnodes, **kw)

    def close(self):
        if getattr(self, "_h", None):
            _lib.hfg_diatomic_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pure_indices(self) -> np.ndarray:
        idx = np.zeros(self.nbf, dtype=np.int32)
        _check(_lib.hfg_diatomic_pure_indices(self._h, idx.ctypes.data_as(_I)))
        return idx

    def _one(self, fn):
        M = np.zeros((self.nbf, self.nbf), order="F")
        _check(fn(self._h, _dptr(M)))
        return M

    def overlap(self):
        return self._one(_lib.hfg_diatomic_overlap)

    def kinetic(self):
        return self._one(_lib.hfg_diatomic_kinetic)

    def nuclear(self):
        return self._one(_lib.hfg_diatomic_nuclear)

    def one_electron_block(self, which: str, m: int) -> np.ndarray:
        w = {"S": 0, "T": 1, "V": 2}[which]
        n = ctypes.c_int()
        _check(_lib.hfg_diatomic_one_electron_block(self._h, w, m, None, ctypes.byref(n)))
        M = np.zeros((n.value, n.value), order="F")
        _check(_lib.hfg_diatomic_one_electron_block(self._h, w, m, _dptr(M), ctypes.byref(n)))
        return M

    def tables(self, which: int, ilm: int, iel: int):
        """(L, |M|, padded table) for which 0..3 (P0, P2, Q0, Q2), or
        (L, |M|, factor, sigma) for which 4."""
        L, M, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        nn = self.dims["nnodes"]
        _check(_lib.hfg_diatomic_tables(self._h, which, ilm, iel, ctypes.byref(L), ctypes.byref(M),
                                        ctypes.byref(r), None, None))
        if which < 4:
            out = np.zeros((nn, nn), order="F")
            _check(_lib.hfg_diatomic_tables(self._h, which, ilm, iel, None, None, None, _dptr(out), None))
            return L.value, M.value, out
        out = np.zeros((2 * nn * nn, r.value), order="F")
        sg = np.zeros(r.value)
        _check(_lib.hfg_diatomic_tables(self._h, which, ilm, iel, None, None, None, _dptr(out), _dptr(sg)))
        return L.value, M.value, out, sg

    # ---- hot path: device pointers ----
    def coulomb(self, P, J, stream=None):
        _check(_lib.hfg_diatomic_coulomb(self._h, _ptr(P), _ptr(J), _stream(stream)))

    def exchange(self, P, K, symmetric: bool = False, stream=None, split: bool = False,
                 itemwise: bool = False):
        flags = ((EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
                 | (EXCHANGE_ITEMWISE if itemwise else 0))
        _check(_lib.hfg_diatomic_exchange(self._h, _ptr(P), _ptr(K), flags, _stream(stream)))

    # ---- hot path: host arrays (drop-in value semantics) ----
    def coulomb_host(self, P: np.ndarray, out: np.ndarray = None) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros_like(P, order="F") if out is None else out
        _check(_lib.hfg_diatomic_coulomb_host(self._h, _dptr(P), _dptr(J)))
        return J

    def exchange_host(self, P: np.ndarray, out: np.ndarray = None, symmetric: bool = False,
                      split: bool = False) -> np.ndarray:
        P = np.asfortranarray(P, dtype=np.float64)
        K = np.zeros_like(P, order="F") if out is None else out
        flags = (EXCHANGE_SYMMETRIC if symmetric else 0) | (EXCHANGE_SPLIT if split else 0)
        _check(_lib.hfg_diatomic_exchange_host(self._h, _dptr(P), _dptr(K), flags))
        return K

    # ---- XC on the pure-m grid ----
    def dft_grid(self, lang: int = 0):
        """(Re)build the pure-m grid: lang cos(nu) points (0 -> 4 lmax + 12)."""
        _check(_lib.hfg_diatomic_dft_grid(self._h, lang))

    def xc(self, x_func, c_func, Pa, Ha, Pb=None, Hb=None, energies=None, thr=1e-12, stream=None):
        """Device pointers (torch tensors, column-major pure-basis matrices);
        Pb None: restricted, Pa the total density."""
        _check(_lib.hfg_diatomic_xc(self._h, x_func, c_func, _ptr(Pa), _ptr(Pb) if Pb is not None else None,
                                    _ptr(Ha), _ptr(Hb) if Hb is not None else None,
                                    _ptr(energies) if energies is not None else None, thr, _stream(stream)))

    def xc_host(self, x_func, c_func, Pa, Pb=None, thr=1e-12):
        """Returns (Ha, Hb or None, Exc, Nel)."""
        Pa = np.asfortranarray(Pa, dtype=np.float64)
        Ha = np.zeros_like(Pa, order="F")
        Pb_ = Hb = None
        if Pb is not None:
            Pb_ = np.asfortranarray(Pb, dtype=np.float64)
            Hb = np.zeros_like(Pa, order="F")
        exc, nel = ctypes.c_double(), ctypes.c_double()
        _check(_lib.hfg_diatomic_xc_host(self._h, x_func, c_func, _dptr(Pa), _dptr(Pb_) if Pb_ is not None else None,
                                         _dptr(Ha), _dptr(Hb) if Hb is not None else None,
                                         ctypes.byref(exc), ctypes.byref(nel), thr))
        return Ha, Hb, exc.value, nel.value

    def work(self, act: np.ndarray = None, jk_mask: np.ndarray = None) -> dict:
        """Exchange work model (flops) for a density-block activity mask
        act[i + l*nang] and an optional output-block mask jk_mask[j + k*nang]."""
        w = _DWork()
        a = None if act is None else np.ascontiguousarray(act, dtype=np.uint8)
        m = None if jk_mask is None else np.ascontiguousarray(jk_mask, dtype=np.uint8)
        _check(_lib.hfg_diatomic_work(self._h, None if a is None else a.ctypes.data,
                                      None if m is None else m.ctypes.data, ctypes.byref(w)))
        return {n: getattr(w, n) for n, _ in _DWork._fields_}
