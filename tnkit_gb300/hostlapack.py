"""The host half of the device truncation routes: eigenvalues and eigenvectors of the symmetric
tridiagonal matrices that the Gram route's device reduction (tnk_sytrd_batched_f64) leaves, by
LAPACK's divide and conquer (dstedc, COMPZ='I'), and singular values and vectors of the upper
bidiagonal matrices that the exact route's device reduction (tnk_gebrd_batched_f64) leaves
(dbdsdc, COMPQ='I'). The work is O(n^2) per sector when the spectrum deflates (a DMRG spectrum
spans ~20 decades, and most of its merges deflate): ~3 ms at n = 522, against the O(n^3)
reductions and back-transformations that stay on the GPU.

dstedc and dbdsdc are called through the function pointers that scipy exports for Cython
(scipy.linalg.cython_lapack), from ctypes, which releases the interpreter lock for the call: the
sectors of a bond run side by side in a thread pool. scipy's own Python wrappers hold the lock.
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes as C
import glob
import os
from typing import List, Sequence, Tuple

import numpy as np

_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
_STATE = {"stedc": None, "bdsdc": None, "threads": None, "tried_threads": False, "pools": {}}


def _capsule_fn(name: str, proto):
    import scipy.linalg.cython_lapack as cl
    cap = cl.__pyx_capi__[name]
    api = C.pythonapi
    api.PyCapsule_GetName.restype = C.c_char_p
    api.PyCapsule_GetName.argtypes = [C.py_object]
    api.PyCapsule_GetPointer.restype = C.c_void_p
    api.PyCapsule_GetPointer.argtypes = [C.py_object, C.c_char_p]
    ptr = api.PyCapsule_GetPointer(cap, api.PyCapsule_GetName(cap))
    if not ptr:
        raise RuntimeError(f"scipy.linalg.cython_lapack exports no {name}")
    return proto(ptr)


def _stedc():
    if _STATE["stedc"] is None:
        proto = C.CFUNCTYPE(None, C.c_char_p, _IP, _DP, _DP, _DP, _IP, _DP, _IP, _IP, _IP, _IP)
        _STATE["stedc"] = _capsule_fn("dstedc", proto)
    return _STATE["stedc"]


def available() -> bool:
    """Whether the host tridiagonal solver can be called (scipy with its Cython LAPACK)."""
    try:
        _stedc()
        return True
    except Exception:
        return False


def _thread_control():
    """(set, get) of the thread count of the BLAS under scipy's LAPACK, or None."""
    if not _STATE["tried_threads"]:
        _STATE["tried_threads"] = True
        try:
            import scipy
            base = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
            for path in sorted(glob.glob(os.path.join(base, "libscipy_openblas*.so*"))):
                lib = C.CDLL(path)
                set_ = getattr(lib, "scipy_openblas_set_num_threads", None)
                get_ = getattr(lib, "scipy_openblas_get_num_threads", None)
                if set_ is not None and get_ is not None:
                    set_.argtypes, set_.restype = [C.c_int], None
                    get_.argtypes, get_.restype = [], C.c_int
                    _STATE["threads"] = (set_, get_)
                    break
        except Exception:
            _STATE["threads"] = None
    return _STATE["threads"]


def tridiag_eigh(d: np.ndarray, e: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Eigenvalues (ascending) and orthonormal eigenvectors (the columns of a Fortran-ordered
    n x n array) of the symmetric tridiagonal matrix with diagonal d (n) and off-diagonal
    e[:n-1]. Raises numpy.linalg.LinAlgError when dstedc reports a failure."""
    n = int(d.shape[0])
    if n == 0:
        return np.zeros(0), np.zeros((0, 0), order="F")
    D = np.array(d[:n], dtype=np.float64, copy=True)
    E = np.zeros(max(n, 1))
    E[:n - 1] = e[:n - 1]
    Z = np.zeros((n, n), order="F")
    lwork = 1 + 4 * n + n * n
    liwork = 3 + 5 * n
    W = np.empty(lwork)
    IW = np.empty(liwork, dtype=np.int32)
    info = C.c_int(0)
    ci = lambda v: C.byref(C.c_int(v))
    _stedc()(b"I", ci(n), D.ctypes.data_as(_DP), E.ctypes.data_as(_DP), Z.ctypes.data_as(_DP),
             ci(max(n, 1)), W.ctypes.data_as(_DP), ci(lwork), IW.ctypes.data_as(_IP),
             ci(liwork), C.byref(info))
    if info.value != 0:
        raise np.linalg.LinAlgError(f"dstedc failed (info {info.value}, n {n})")
    return D, Z


def _bdsdc():
    if _STATE.get("bdsdc") is None:
        proto = C.CFUNCTYPE(None, C.c_char_p, C.c_char_p, _IP, _DP, _DP, _DP, _IP, _DP, _IP, _DP,
                            _IP, _DP, _IP, _IP)
        _STATE["bdsdc"] = _capsule_fn("dbdsdc", proto)
    return _STATE["bdsdc"]


def bidiag_svd(d: np.ndarray, e: np.ndarray) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Singular values (descending) and vectors of the upper bidiagonal matrix with diagonal d
    (n) and superdiagonal e[:n-1], by LAPACK's divide and conquer (dbdsdc, COMPQ='I'):
    B = U diag(s) VT, U and VT Fortran-ordered n x n. Raises numpy.linalg.LinAlgError when
    dbdsdc reports a failure."""
    n = int(d.shape[0])
    if n == 0:
        return np.zeros(0), np.zeros((0, 0), order="F"), np.zeros((0, 0), order="F")
    D = np.array(d[:n], dtype=np.float64, copy=True)
    E = np.zeros(max(n, 1))
    E[:n - 1] = e[:n - 1]
    U = np.zeros((n, n), order="F")
    VT = np.zeros((n, n), order="F")
    W = np.empty(3 * n * n + 4 * n + 1)
    IW = np.empty(8 * n + 1, dtype=np.int32)
    q = np.zeros(1)
    iq = np.zeros(1, dtype=np.int32)
    info = C.c_int(0)
    ci = lambda v: C.byref(C.c_int(v))
    _bdsdc()(b"U", b"I", ci(n), D.ctypes.data_as(_DP), E.ctypes.data_as(_DP),
             U.ctypes.data_as(_DP), ci(max(n, 1)), VT.ctypes.data_as(_DP), ci(max(n, 1)),
             q.ctypes.data_as(_DP), iq.ctypes.data_as(_IP), W.ctypes.data_as(_DP),
             IW.ctypes.data_as(_IP), C.byref(info))
    if info.value != 0:
        raise np.linalg.LinAlgError(f"dbdsdc failed (info {info.value}, n {n})")
    return D, U, VT


def _many(fn, probs, lanes):
    if len(probs) <= 1 or lanes <= 1:
        return [fn(*p) for p in probs]
    pool = _STATE["pools"].get(lanes)
    if pool is None:
        pool = _STATE["pools"][lanes] = cf.ThreadPoolExecutor(lanes,
                                                               thread_name_prefix="tnk-lapack")
    order = sorted(range(len(probs)), key=lambda i: -probs[i][0].shape[0])
    ctl = _thread_control()
    prev = None
    if ctl is not None:
        prev = ctl[1]()
        ctl[0](max(1, (os.cpu_count() or lanes) // lanes))
    try:
        futs = {i: pool.submit(fn, *probs[i]) for i in order}
        return [futs[i].result() for i in range(len(probs))]
    finally:
        if ctl is not None and prev is not None:
            ctl[0](prev)


def bidiag_svd_many(des: Sequence[Tuple[np.ndarray, np.ndarray]],
                    lanes: int = 4) -> List[Tuple[np.ndarray, np.ndarray, np.ndarray]]:
    """bidiag_svd of several problems, the largest first, over `lanes` threads."""
    return _many(bidiag_svd, des, lanes)


def tridiag_eigh_many(des: Sequence[Tuple[np.ndarray, np.ndarray]],
                      lanes: int = 4) -> List[Tuple[np.ndarray, np.ndarray]]:
    """tridiag_eigh of several problems, the largest first, over `lanes` threads; the BLAS
    under LAPACK gets cores / lanes threads meanwhile."""
    return _many(tridiag_eigh, des, lanes)
