"""ctypes loader for the CPU oracle (oracle/h2w_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py as the checker, never by the GPU library.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

LISTS = {"charge": 0, "nbr": 1, "il": 2, "isvertex": 3, "far_check": 4, "far_charge": 5,
         "ver_check": 6, "ver_charge": 7, "sn_row": 8, "sn_col": 9, "uv_rank": 10}


def build():
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = ctypes.CDLL(_LIB)
        P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        L.h2wo_create.restype = P
        L.h2wo_create.argtypes = [I, I, I64, P, I, I, I, I64, I64]
        L.h2wo_destroy.argtypes = [P]
        L.h2wo_assemble.argtypes = [P]
        L.h2wo_matvec.argtypes = [P, P, P]
        L.h2wo_dense_matvec.argtypes = [P, P, P]
        L.h2wo_gmres.argtypes = [P, P, P, I, I, P, P]
        L.h2wo_memory.restype = ctypes.c_double
        L.h2wo_memory.argtypes = [P]
        L.h2wo_kii.restype = ctypes.c_double
        L.h2wo_kii.argtypes = [P]
        L.h2wo_entries.argtypes = [P, P, I64, P, I64, P]
        L.h2wo_list.restype = I64
        L.h2wo_list.argtypes = [P, I, P, P]
        L.h2wo_list_nptr.restype = I64
        L.h2wo_list_nptr.argtypes = [P, I]
        L.h2wo_is_complex.argtypes = [P]
        L.h2wo_is_complex.restype = I
        L.h2wo_set_sum_order.argtypes = [I]
        L.h2wo_set_sum_order.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_sum_order(reverse):
    """Sum every block product of every oracle in descending order (True) or in
    the reference build's ascending order (False, the default)."""
    lib().h2wo_set_sum_order(1 if reverse else 0)


class Oracle:
    """One compressed operator, built and assembled on the host."""

    def __init__(self, dim, form, points, nlevels, tol_pow, choice, kernel_n=None, diag_n=None,
                 assemble=True):
        L = lib()
        self.points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, dim)
        self.N = self.points.shape[0]
        self.dim = dim
        kn = self.N if kernel_n is None else kernel_n
        dn = self.N if diag_n is None else diag_n
        self.h = L.h2wo_create(dim, form, self.N, _p(self.points), nlevels, tol_pow, choice, kn, dn)
        if not self.h:
            raise ValueError("bad oracle arguments")
        # the complex Helmholtz kernel (choice 2): complex128 vectors
        self.dtype = np.complex128 if L.h2wo_is_complex(self.h) else np.float64
        if assemble:
            L.h2wo_assemble(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().h2wo_destroy(self.h)
            self.h = None

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.empty(self.N, dtype=self.dtype)
        lib().h2wo_matvec(self.h, _p(x), _p(y))
        return y

    def dense_matvec(self, x):
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.empty(self.N, dtype=self.dtype)
        lib().h2wo_dense_matvec(self.h, _p(x), _p(y))
        return y

    def gmres(self, b, x0=None, max_iter=500, tol_pow=10):
        b = np.ascontiguousarray(b, dtype=self.dtype)
        x = np.ones(self.N, dtype=self.dtype) if x0 is None else np.array(x0, dtype=self.dtype)
        it = ctypes.c_int(0)
        res = ctypes.c_double(0)
        lib().h2wo_gmres(self.h, _p(b), _p(x), max_iter, tol_pow, ctypes.byref(it), ctypes.byref(res))
        return x, it.value, res.value

    def memory(self):
        return lib().h2wo_memory(self.h)

    def kii(self):
        return lib().h2wo_kii(self.h)

    def entries(self, rows, cols):
        r = np.ascontiguousarray(rows, dtype=np.int32)
        c = np.ascontiguousarray(cols, dtype=np.int32)
        out = np.empty((len(r), len(c)), dtype=self.dtype)
        lib().h2wo_entries(self.h, _p(r), len(r), _p(c), len(c), _p(out))
        return out

    def csr(self, name):
        w = LISTS[name]
        L = lib()
        nv = L.h2wo_list(self.h, w, None, None)
        npt = L.h2wo_list_nptr(self.h, w)
        ptr = np.empty(npt, dtype=np.int64)
        val = np.empty(max(nv, 1), dtype=np.int32)
        L.h2wo_list(self.h, w, _p(ptr), _p(val))
        return ptr, val[:nv]
