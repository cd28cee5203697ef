"""GB300-native H2* / (H2+H)* HODLRdD operator and GMRES (sm_103a).

Host-side Python mirror of the reference's operator interface. Everything
runs through the C ABI of libh2w.so (include/h2w.h): the tree and plan are
built by native host code, the compression, every matvec pass and GMRES run
as CUDA kernels on the GPU. There is no CPU fallback: without the built
library or a GPU the calls raise.

Reference interface mirrored here (paths within the reference project):
  initialisation(...)          {1D,2D,3D}/codes/matvec.hpp  (tree_initialisation, mat_vec_prod)
  iterative_solver(...)        {1D,2D,3D}/codes/gmres.hpp   (GMRES, resid, max_iter)
"""
import ctypes
import math
import os

import numpy as np

from . import synth  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libh2w.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_RANK, ERR_NOT_CONVERGED, ERR_STATE = -1, -2, -3, -4, -5, -6
FORM_NESTED, FORM_SEMINESTED, FORM_NONNESTED = 0, 1, 2
KERNEL_IE, KERNEL_RBF, KERNEL_HELMHOLTZ, KERNEL_HANKEL = 0, 1, 2, 10
ASSEMBLE_NCA, ASSEMBLE_IMPORT, ASSEMBLE_LEARNED = 0, 1, 2
PREC_FP64, PREC_FP32, PREC_DF64 = 0, 1, 2
HOST, DEVICE = 0, 1
OPT_GRAPH, OPT_COOP, OPT_IR_RESIDUAL, OPT_MULTI_XW, OPT_ROW_SPLIT, OPT_IR_UPDATE, OPT_TENSOR, OPT_F32_BASIS = (
    0, 1, 2, 3, 4, 5, 6, 7)
OPT_DATAFLOW = 8
OPT_PRODUCER_WARP = 9
OPT_SPIN_LIMIT = 10
OPT_FAR_ON_THE_FLY = 11
OPT_NCA_DF = 12
OPT_COMPLEX_ARNOLDI = 13
TUNE_IR_MIX = 16
LISTS = {"charge": 0, "nbr": 1, "il": 2, "isvertex": 3, "far_check": 4, "far_charge": 5,
         "ver_check": 6, "ver_charge": 7, "sn_row": 8, "sn_col": 9}

EXPORTS = ["h2w_create", "h2w_destroy", "h2w_last_error", "h2w_set_points", "h2w_gen_grid", "h2w_gen_uniform",
           "h2w_get_points", "h2w_num_points", "h2w_build_tree", "h2w_get_list", "h2w_import_list",
           "h2w_assemble", "h2w_storage_entries", "h2w_operator_bytes", "h2w_matvec", "h2w_gmres",
           "h2w_gmres_ir", "h2w_dense_matvec", "h2w_total_error", "h2w_profile", "h2w_profile_phases", "h2w_launch_count"]


class H2WError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("h2w error %d: %s" % (code, msg))
        self.code = code


class _Config(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("form", ctypes.c_int), ("choice", ctypes.c_int),
                ("tol_pow", ctypes.c_int), ("nlevels", ctypes.c_int), ("rank_cap", ctypes.c_int),
                ("kernel_n", ctypes.c_int64), ("diag_n", ctypes.c_int64), ("device", ctypes.c_int)]


_lib = None


def build(force=False):
    from . import buildlib
    return buildlib.build(force=force)


def lib():
    """Load libh2w.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    sig = {
        "h2w_create": [ctypes.POINTER(_Config), ctypes.POINTER(P)],
        "h2w_destroy": [P],
        "h2w_set_points": [P, P, I64],
        "h2w_gen_grid": [P, I64],
        "h2w_gen_uniform": [P, ctypes.c_uint64, I64],
        "h2w_get_points": [P, P],
        "h2w_num_points": [P, ctypes.POINTER(I64)],
        "h2w_build_tree": [P],
        "h2w_get_list": [P, I, P, P, ctypes.POINTER(I64), ctypes.POINTER(I64)],
        "h2w_import_list": [P, I, P, P, I64],
        "h2w_assemble": [P, I],
        "h2w_storage_entries": [P, ctypes.POINTER(D)],
        "h2w_operator_bytes": [P, I, ctypes.POINTER(I64)],
        "h2w_matvec": [P, P, P, I, I, I, P],
        "h2w_matvec_static": [P, P, P, I, P],
        "h2w_gmres": [P, P, P, I, I, I, ctypes.POINTER(I), ctypes.POINTER(D)],
        "h2w_gmres_ir": [P, P, P, I, I, I, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(D)],
        "h2w_gmres_batch": [P, P, P, I, I, I, I, P, P],
        "h2w_gmres_ir_batch": [P, P, P, I, I, I, I, I, ctypes.POINTER(I), ctypes.POINTER(I), P],
        "h2w_dense_matvec": [P, P, P, I64, I64, I],
        "h2w_total_error": [P, P, I64, I, ctypes.POINTER(D)],
        "h2w_save_operator": [P, ctypes.c_char_p],
        "h2w_open_operator": [ctypes.c_char_p, I, ctypes.POINTER(P)],
        "h2w_get_config": [P, ctypes.POINTER(_Config)],
        "h2w_profile": [P, I],
        "h2w_profile_multi": [P, I, ctypes.POINTER(I64), ctypes.POINTER(D), ctypes.POINTER(D)],
        "h2w_profile_fly": [P, I, ctypes.POINTER(I64), ctypes.POINTER(D), ctypes.POINTER(I64)],
        "h2w_plan_stats": [P, P, I],
        "h2w_set_option": [P, I, I64],
        "h2w_learn_record": [P, I],
        "h2w_learn_data": [P, P, P, ctypes.POINTER(I64)],
        "h2w_learn_set_model": [P, P, ctypes.c_float, I],
        "h2w_learn_stats": [P, ctypes.POINTER(I64), ctypes.POINTER(I64)],
        "h2w_learn_detail": [P, P, ctypes.POINTER(D), ctypes.POINTER(D)],
        "h2w_mlp_forward": [P, P, I64, P, P],
        "h2w_mlp_grad": [P, P, P, I64, ctypes.c_float, P, P, P],
        "h2w_mlp_adam": [P, P, P, P, I, ctypes.c_float, P],
        "h2w_batch_create": [P, I, ctypes.POINTER(P)],
        "h2w_batch_destroy": [P],
        "h2w_batch_offsets": [P, P],
        "h2w_batch_matvec": [P, P, P, I, I],
        "h2w_batch_gmres": [P, P, P, I, I, I, P, P],
        "h2w_batch_gmres_ir": [P, P, P, I, I, I, I, ctypes.POINTER(I), ctypes.POINTER(I), P],
        "h2w_autotune": [P, I, I, I, ctypes.POINTER(I64), ctypes.POINTER(D)],
        "h2w_get_option": [P, I, ctypes.POINTER(I64)],
        "h2w_profile_phases": [P, I, I, P, P, P, ctypes.POINTER(I)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = I
    L.h2w_mlp_nparam.argtypes = []
    L.h2w_mlp_nparam.restype = I
    L.h2w_launch_count.argtypes = []
    L.h2w_launch_count.restype = I64
    L.h2w_batch_last_error.argtypes = [P]
    L.h2w_batch_last_error.restype = ctypes.c_char_p
    L.h2w_last_error.argtypes = [P]
    L.h2w_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def launch_count():
    """Kernel launches this library has issued since it was loaded."""
    return int(lib().h2w_launch_count())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def levels_for(dim, n_param, leaf_param):
    """Tree depth exactly as the reference drivers compute it
    (1D/codes/main.cpp:13, 2D/codes/main.cpp:13, 3D/codes/main.cpp:11)."""
    if dim == 1:
        return int(math.ceil(math.log(float(n_param) / leaf_param) / math.log(2)))
    if dim == 2:
        return int(math.ceil(2.0 * math.log(float(n_param) / leaf_param) / math.log(4)))
    return int(math.ceil(3 * math.log(float(n_param) / leaf_param) / math.log(8)))


class H2Operator:
    """One compressed kernel matrix on one GPU (a handle of the C ABI)."""

    def __init__(self, dim, form, choice, tol_pow, nlevels, rank_cap=0, kernel_n=0, diag_n=0, device=0):
        L = lib()
        cfg = _Config(dim, form, choice, tol_pow, nlevels, rank_cap, kernel_n, diag_n, device)
        h = ctypes.c_void_p()
        rc = L.h2w_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != OK:
            raise H2WError(rc, "h2w_create failed (no CUDA device or bad configuration)")
        self.h = h
        self.dim, self.form, self.choice, self.tol_pow, self.nlevels = dim, form, choice, tol_pow, nlevels
        # the Helmholtz kernels are complex: vectors are complex128 (interleaved (re, im) doubles in the C ABI)
        self.complex = choice in (KERNEL_HELMHOLTZ, KERNEL_HANKEL)

    @classmethod
    def open(cls, path, device=0):
        """A handle from an operator file (h2w_open_operator): the saved
        operator formed from its pivots on `device` (-1: host-only)."""
        h = ctypes.c_void_p()
        rc = lib().h2w_open_operator(os.fsencode(path), device, ctypes.byref(h))
        if rc != OK:
            raise H2WError(rc, "h2w_open_operator failed for %s (missing, corrupted or not an operator file)" % path)
        self = cls.__new__(cls)
        self.h = h
        cfg = _Config()
        self._ck(lib().h2w_get_config(self.h, ctypes.byref(cfg)))
        self.dim, self.form, self.choice, self.tol_pow, self.nlevels = (cfg.dim, cfg.form, cfg.choice, cfg.tol_pow,
                                                                        cfg.nlevels)
        self.complex = cfg.choice in (KERNEL_HELMHOLTZ, KERNEL_HANKEL)
        return self

    def save(self, path):
        """Write the operator file of this assembled operator (h2w_save_operator)."""
        self._ck(lib().h2w_save_operator(self.h, os.fsencode(path)))

    def close(self):
        if getattr(self, "h", None):
            lib().h2w_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, allow=()):
        if rc != OK and rc not in allow:
            raise H2WError(rc, lib().h2w_last_error(self.h).decode())
        return rc

    # points and tree
    def set_points(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, self.dim)
        self._ck(lib().h2w_set_points(self.h, _ptr(p), p.shape[0]))

    def gen_grid(self, n_per_axis):
        self._ck(lib().h2w_gen_grid(self.h, n_per_axis))

    def gen_uniform(self, seed, n):
        self._ck(lib().h2w_gen_uniform(self.h, seed, n))

    @property
    def N(self):
        n = ctypes.c_int64()
        self._ck(lib().h2w_num_points(self.h, ctypes.byref(n)))
        return n.value

    def points(self):
        out = np.empty((self.N, self.dim))
        self._ck(lib().h2w_get_points(self.h, _ptr(out)))
        return out

    def build_tree(self):
        self._ck(lib().h2w_build_tree(self.h))

    def get_list(self, name):
        w = LISTS[name]
        npt, nv = ctypes.c_int64(), ctypes.c_int64()
        self._ck(lib().h2w_get_list(self.h, w, None, None, ctypes.byref(npt), ctypes.byref(nv)))
        ptr = np.empty(npt.value, dtype=np.int64)
        val = np.empty(max(nv.value, 1), dtype=np.int32)
        self._ck(lib().h2w_get_list(self.h, w, _ptr(ptr), _ptr(val), None, None))
        return ptr, val[:nv.value]

    def import_list(self, name, ptr, val):
        p = np.ascontiguousarray(ptr, dtype=np.int64)
        v = np.ascontiguousarray(val, dtype=np.int32)
        if v.size == 0:
            v = np.zeros(1, dtype=np.int32)
        self._ck(lib().h2w_import_list(self.h, LISTS[name], _ptr(p), _ptr(v), p.size))

    def assemble(self, mode=ASSEMBLE_NCA):
        self._ck(lib().h2w_assemble(self.h, mode))

    def storage_entries(self):
        e = ctypes.c_double()
        self._ck(lib().h2w_storage_entries(self.h, ctypes.byref(e)))
        return e.value

    def operator_bytes(self, precision=PREC_FP64):
        b = ctypes.c_int64()
        self._ck(lib().h2w_operator_bytes(self.h, precision, ctypes.byref(b)))
        return b.value

    # instrumentation
    # learned NCA proposals
    def learn_record(self, enable=True):
        self._ck(lib().h2w_learn_record(self.h, 1 if enable else 0))

    def learn_data(self):
        """Recorded (features n x 16 float32, labels n uint8) of plain NCA assemblies."""
        n = ctypes.c_int64()
        self._ck(lib().h2w_learn_data(self.h, None, None, ctypes.byref(n)))
        X = np.empty((n.value, 16), dtype=np.float32)
        y = np.empty(n.value, dtype=np.uint8)
        self._ck(lib().h2w_learn_data(self.h, _ptr(X), _ptr(y), ctypes.byref(n)))
        return X, y

    def learn_set_model(self, params, calib=1.0, margin=2):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._ck(lib().h2w_learn_set_model(self.h, _ptr(p), float(calib), int(margin)))

    def learn_detail(self):
        """(rejections: no pivots / non-finite / test failed, mean proposal size, mean pivots kept)."""
        r = np.zeros(3, dtype=np.int64)
        a, b = ctypes.c_double(), ctypes.c_double()
        self._ck(lib().h2w_learn_detail(self.h, _ptr(r), ctypes.byref(a), ctypes.byref(b)))
        return r, a.value, b.value

    def learn_stats(self):
        """(blocks proposed, blocks accepted) since the last call."""
        b, a = ctypes.c_int64(), ctypes.c_int64()
        self._ck(lib().h2w_learn_stats(self.h, ctypes.byref(b), ctypes.byref(a)))
        return b.value, a.value

    def autotune(self, nrhs=64, precision=PREC_FP32, reps=3):
        """Time each candidate target granularity and keep the fastest;
        returns (chosen value, ms per repetition)."""
        c, ms = ctypes.c_int64(), ctypes.c_double()
        self._ck(lib().h2w_autotune(self.h, nrhs, precision, reps, ctypes.byref(c), ctypes.byref(ms)))
        return c.value, ms.value

    def set_option(self, option, value):
        self._ck(lib().h2w_set_option(self.h, option, int(value)))

    def get_option(self, option):
        v = ctypes.c_int64()
        self._ck(lib().h2w_get_option(self.h, option, ctypes.byref(v)))
        return v.value

    def profile_multi(self, precision=PREC_FP32):
        """(launches, total ms, algorithmic bytes per launch) of the multi-vector kernel."""
        la, ms, by = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        self._ck(lib().h2w_profile_multi(self.h, precision, ctypes.byref(la), ctypes.byref(ms), ctypes.byref(by)))
        return la.value, ms.value, by.value

    def profile_fly(self, precision=PREC_FP32):
        """(launches, total ms, kernel entries per launch) of the far-field M2L
        kernel of products with the far field on the fly."""
        la, ms, en = ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
        self._ck(lib().h2w_profile_fly(self.h, precision, ctypes.byref(la), ctypes.byref(ms), ctypes.byref(en)))
        return la.value, ms.value, en.value

    def plan_stats(self):
        """Multi-vector plan: targets, panels, operator entries per column, entries
        the kernel multiplies per column (with its row and column padding),
        atomically accumulated targets, entries spanned by the 64-row tiles."""
        st = np.zeros(6, dtype=np.int64)
        self._ck(lib().h2w_plan_stats(self.h, _ptr(st), 6))
        return dict(zip(("targets", "panels", "entries", "multiplied", "atomic_targets", "tile_span"), st.tolist()))

    def profile(self, enable):
        self._ck(lib().h2w_profile(self.h, 1 if enable else 0))

    def profile_phases(self, precision=PREC_FP64):
        n = ctypes.c_int()
        self._ck(lib().h2w_profile_phases(self.h, precision, 0, None, None, None, ctypes.byref(n)))
        la = np.zeros(n.value, dtype=np.int64)
        ms = np.zeros(n.value)
        by = np.zeros(n.value)
        self._ck(lib().h2w_profile_phases(self.h, precision, n.value, _ptr(la), _ptr(ms), _ptr(by), None))
        return la, ms, by

    # products
    def matvec(self, x, precision=PREC_FP64):
        if self.complex:
            x = np.ascontiguousarray(x, dtype=np.complex128)
            y = np.empty_like(x)
            self._ck(lib().h2w_matvec(self.h, ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(y.ctypes.data), 1,
                                      precision, HOST, None))
            return y
        x = np.ascontiguousarray(x, dtype=np.float64)
        nrhs = 1 if x.ndim == 1 else x.shape[1]
        xc = np.asfortranarray(x.reshape(self.N, nrhs)) if x.ndim > 1 else x
        y = np.empty_like(xc)
        self._ck(lib().h2w_matvec(self.h, ctypes.c_void_p(xc.ctypes.data), ctypes.c_void_p(y.ctypes.data), nrhs,
                                  precision, HOST, None))
        return y

    def matvec_device(self, x_ptr, y_ptr, nrhs=1, precision=PREC_FP64, stream=0):
        self._ck(lib().h2w_matvec(self.h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), nrhs, precision, DEVICE,
                                  ctypes.c_void_p(stream) if stream else None))

    def dense_matvec(self, x, row0=0, nrows=None):
        dt = np.complex128 if self.complex else np.float64
        x = np.ascontiguousarray(x, dtype=dt)
        n = self.N - row0 if nrows is None else nrows
        y = np.empty(n, dtype=dt)
        self._ck(lib().h2w_dense_matvec(self.h, _ptr(x), _ptr(y), row0, n, HOST))
        return y

    def total_error(self, x, nrows=0):
        """||y_dense - A x|| / ||y_dense|| with the exact dense product on the
        GPU (compute_total_error); nrows > 0 samples that many evenly spaced rows."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        e = ctypes.c_double()
        self._ck(lib().h2w_total_error(self.h, _ptr(x), int(nrows), HOST, ctypes.byref(e)))
        return e.value

    def gmres_device(self, b_ptr, x_ptr, max_iter=500, tol_pow=10):
        it, res = ctypes.c_int(), ctypes.c_double()
        rc = lib().h2w_gmres(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), max_iter, tol_pow, DEVICE,
                             ctypes.byref(it), ctypes.byref(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return it.value, res.value

    def gmres_ir_device(self, b_ptr, x_ptr, max_outer=20, inner_iter=100, tol_pow=10, where=DEVICE):
        oi, ii, res = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        rc = lib().h2w_gmres_ir(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), max_outer, inner_iter,
                                tol_pow, where, ctypes.byref(oi), ctypes.byref(ii), ctypes.byref(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return oi.value, ii.value, res.value

    def gmres_host_ptr(self, b_ptr, x_ptr, max_iter=500, tol_pow=10):
        it, res = ctypes.c_int(), ctypes.c_double()
        rc = lib().h2w_gmres(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), max_iter, tol_pow, HOST,
                             ctypes.byref(it), ctypes.byref(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return it.value, res.value

    def gmres(self, b, x0=None, max_iter=500, tol_pow=10):
        dt = np.complex128 if self.complex else np.float64
        b = np.ascontiguousarray(b, dtype=dt)
        x = np.ones(self.N, dtype=dt) if x0 is None else np.array(x0, dtype=dt)
        it, res = ctypes.c_int(), ctypes.c_double()
        rc = lib().h2w_gmres(self.h, _ptr(b), _ptr(x), max_iter, tol_pow, HOST, ctypes.byref(it), ctypes.byref(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return x, it.value, res.value

    def gmres_ir(self, b, x0=None, max_outer=20, inner_iter=100, tol_pow=10):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ones(self.N) if x0 is None else np.array(x0, dtype=np.float64)
        oi, ii, res = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        rc = lib().h2w_gmres_ir(self.h, _ptr(b), _ptr(x), max_outer, inner_iter, tol_pow, HOST, ctypes.byref(oi),
                                ctypes.byref(ii), ctypes.byref(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return x, oi.value, ii.value, res.value


    # many right-hand sides (columns of an N x nrhs array)
    def _cols(self, a):
        a = np.asarray(a, dtype=np.float64)
        return np.asfortranarray(a.reshape(self.N, -1))

    def gmres_batch(self, B, X0=None, max_iter=200, tol_pow=10):
        """Per-column GMRES on all columns of B at once (one multi-vector
        product per Arnoldi step). Returns X, iterations and residuals per column."""
        B = self._cols(B)
        X = np.asfortranarray(np.ones_like(B)) if X0 is None else self._cols(np.array(X0, dtype=np.float64))
        k = B.shape[1]
        it = np.zeros(k, dtype=np.int32)
        res = np.zeros(k)
        rc = lib().h2w_gmres_batch(self.h, _ptr(B), _ptr(X), k, max_iter, tol_pow, HOST, _ptr(it), _ptr(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return X, it, res

    def gmres_batch_device(self, b_ptr, x_ptr, nrhs, max_iter=200, tol_pow=10):
        it = np.zeros(nrhs, dtype=np.int32)
        res = np.zeros(nrhs)
        rc = lib().h2w_gmres_batch(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), nrhs, max_iter, tol_pow,
                                   DEVICE, _ptr(it), _ptr(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return it, res

    def gmres_ir_batch(self, B, X0=None, max_outer=20, inner_iter=100, tol_pow=10):
        """FP32-operator batched inner GMRES inside FP64 iterative refinement,
        all columns of B at once. Returns X, outer steps, inner steps, residuals."""
        B = self._cols(B)
        X = np.asfortranarray(np.ones_like(B)) if X0 is None else self._cols(np.array(X0, dtype=np.float64))
        k = B.shape[1]
        oi, ii = ctypes.c_int(), ctypes.c_int()
        res = np.zeros(k)
        rc = lib().h2w_gmres_ir_batch(self.h, _ptr(B), _ptr(X), k, max_outer, inner_iter, tol_pow, HOST,
                                      ctypes.byref(oi), ctypes.byref(ii), _ptr(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return X, oi.value, ii.value, res

    def gmres_ir_batch_device(self, b_ptr, x_ptr, nrhs, max_outer=20, inner_iter=100, tol_pow=10, where=DEVICE):
        oi, ii = ctypes.c_int(), ctypes.c_int()
        res = np.zeros(nrhs)
        rc = lib().h2w_gmres_ir_batch(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), nrhs, max_outer,
                                      inner_iter, tol_pow, where, ctypes.byref(oi), ctypes.byref(ii), _ptr(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return oi.value, ii.value, res


class Batch:
    """Many assembled operators run together (one cooperative launch per
    product, lockstep solvers over concatenated vectors)."""

    def __init__(self, ops):
        self.ops = list(ops)  # keeps the handles alive
        arr = (ctypes.c_void_p * len(self.ops))(*[o.h.value for o in self.ops])
        b = ctypes.c_void_p()
        rc = lib().h2w_batch_create(arr, len(self.ops), ctypes.byref(b))
        if rc != OK:
            raise H2WError(rc, "h2w_batch_create failed (handles must be assembled, on one device)")
        self.b = b
        self.off = np.zeros(len(self.ops) + 1, dtype=np.int64)
        self._ck(lib().h2w_batch_offsets(self.b, _ptr(self.off)))
        self.N = int(self.off[-1])

    def _ck(self, rc, allow=()):
        if rc != OK and rc not in allow:
            raise H2WError(rc, lib().h2w_batch_last_error(self.b).decode())

    def close(self):
        if getattr(self, "b", None):
            lib().h2w_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def split(self, v):
        return [v[self.off[p]:self.off[p + 1]] for p in range(len(self.ops))]

    def matvec(self, x, precision=PREC_FP64):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self._ck(lib().h2w_batch_matvec(self.b, _ptr(x), _ptr(y), precision, HOST))
        return y

    def matvec_device(self, x_ptr, y_ptr, precision=PREC_FP64):
        self._ck(lib().h2w_batch_matvec(self.b, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), precision, DEVICE))

    def gmres(self, b, x0=None, max_iter=200, tol_pow=10):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ones(self.N) if x0 is None else np.array(x0, dtype=np.float64)
        it = np.zeros(len(self.ops), dtype=np.int32)
        res = np.zeros(len(self.ops))
        rc = lib().h2w_batch_gmres(self.b, _ptr(b), _ptr(x), max_iter, tol_pow, HOST, _ptr(it), _ptr(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return x, it, res

    def gmres_ir(self, b, x0=None, max_outer=20, inner_iter=100, tol_pow=10, where=HOST, b_ptr=None, x_ptr=None):
        oi, ii = ctypes.c_int(), ctypes.c_int()
        res = np.zeros(len(self.ops))
        if b_ptr is not None:
            rc = lib().h2w_batch_gmres_ir(self.b, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), max_outer,
                                          inner_iter, tol_pow, where, ctypes.byref(oi), ctypes.byref(ii), _ptr(res))
            self._ck(rc, allow=(ERR_NOT_CONVERGED,))
            return None, oi.value, ii.value, res
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ones(self.N) if x0 is None else np.array(x0, dtype=np.float64)
        rc = lib().h2w_batch_gmres_ir(self.b, _ptr(b), _ptr(x), max_outer, inner_iter, tol_pow, HOST,
                                      ctypes.byref(oi), ctypes.byref(ii), _ptr(res))
        self._ck(rc, allow=(ERR_NOT_CONVERGED,))
        return x, oi.value, ii.value, res


class _TreeView:
    """The few members of the reference's tree object that callers read
    (K->N, K->memory, findMemory_*, getTruePoten)."""

    def __init__(self, op):
        self._op = op
        self.N = op.N
        self.memory = 0.0
        self.collective_charge = None  # the charge of the last mat_vec_prod

    def findMemory(self):
        self.memory = self._op.storage_entries()
        return self.memory

    findMemory_n = findMemory
    findMemory_sn = findMemory

    def getTruePoten(self, charge):
        return self._op.dense_matvec(charge)

    def compute_total_error(self, nrows=0):
        """Error of the last mat_vec_prod against the exact dense product
        (compute_total_error, 3D/codes/HODLR3Dtree.hpp:2645-2662)."""
        if self.collective_charge is None:
            raise RuntimeError("no mat_vec_prod has run yet")
        return self._op.total_error(self.collective_charge, nrows)


class initialisation:
    """Mirror of the reference's operator facade (class initialisation,
    1D/codes/matvec.hpp:73-181, 2D/codes/matvec.hpp:106-173,
    3D/codes/matvec.hpp:6-180): constructor arguments as the reference's,
    tree_initialisation() assembles, mat_vec_prod(charge, output) fills
    output in original point order. dim and form replace the compile-time
    -DUSE_* choice; points (optional) replaces the uniform grid. Kernel_Choice
    2 (3D) / 10 (2D) are the complex Helmholtz kernels of the reference's
    USE_Helm / USE_Hankel builds: charge and output are then complex128."""

    def __init__(self, n_param, nLevels, nParticlesInLeaf, L, TOL_POW, Kernel_Choice, dim=1, form=FORM_NESTED,
                 points=None, device=0, rank_cap=0):
        if L != 1:
            raise ValueError("the reference's grids and trees are defined for L = 1")
        self.dim, self.form = dim, form
        self.N_param, self.nLevels, self.nParticlesInLeaf = n_param, nLevels, nParticlesInLeaf
        self.TOL_POW, self.Kernel_Choice, self.points = TOL_POW, Kernel_Choice, points
        self.device, self.rank_cap = device, rank_cap
        self.op = None
        self.K = None

    def tree_initialisation(self, mode=ASSEMBLE_NCA, skeleton=None):
        if self.points is None:
            N = self.N_param ** self.dim
        else:
            N = int(np.asarray(self.points).reshape(-1, self.dim).shape[0])
        # 1D drivers push the grid twice before evaluating entries, so the
        # RBF diagonal there is sqrt(2N) (1D/codes/matvec.hpp:102-106, kernel.hpp:180)
        diag_n = 2 * N if self.dim == 1 else N
        op = H2Operator(self.dim, self.form, self.Kernel_Choice, self.TOL_POW, self.nLevels, self.rank_cap,
                        kernel_n=N, diag_n=diag_n, device=self.device)
        if self.points is None:
            op.gen_grid(self.N_param)
        else:
            op.set_points(self.points)
        op.build_tree()
        if skeleton is not None:
            for name, (p, v) in skeleton.items():
                op.import_list(name, p, v)
            mode = ASSEMBLE_IMPORT
        op.assemble(mode)
        self.op = op
        self.K = _TreeView(op)

    def mat_vec_prod(self, charge, output=None):
        y = self.op.matvec(charge)
        self.K.collective_charge = np.array(charge, dtype=np.complex128 if self.op.complex else np.float64)
        if output is not None:
            output.resize(y.shape, refcheck=False)
            output[...] = y
        return y


class iterative_solver:
    """Mirror of the reference's GMRES driver (class iterative_solver,
    {1D,2D,3D}/codes/gmres.hpp:14-201): unrestarted FP64 GMRES on the GPU;
    after GMRES() the members resid and max_iter hold the final residual
    and the iteration count, as in the reference."""

    def __init__(self, max_iter, gmres_tol_pow):
        self.restart = max_iter
        self.max_iter = max_iter
        self.gmres_tol_pow = gmres_tol_pow
        self.gmres_tol = 10.0 ** (-gmres_tol_pow)
        self.resid = 0.0

    def GMRES(self, A, x, b):
        xs, it, res = A.op.gmres(b, x0=x, max_iter=self.max_iter, tol_pow=self.gmres_tol_pow)
        x[...] = xs
        self.resid = res
        self.max_iter = it
        return x
