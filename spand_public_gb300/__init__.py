"""spaND factorization and solve on GB300: Python binding of the C ABI.

``Tree`` mirrors ``spaND::Tree`` of leopoldcambier/spaND_public (include/tree.h:133-197:
set_* options, partition, assemble, factorize, solve) and ``cg`` mirrors its CG driver
(include/is.h:12).  Every call goes through ``lib/libspand_gb300.so`` (include/spand_gb300.h);
there is no CPU fallback: a missing library or a missing GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libspand_gb300.so")

# ScalingKind / SymmKind / PartKind enumerators of include/spaND.h:19-21
SVD, PLU, PLUQ, EVD, LLT, LDLT = range(6)
SPD, SYM, GEN = range(3)
MND, RB = range(2)

OP_NAMES = {0: "ScalingLLT", 1: "GemmSymmOut", 2: "GemmSymmIn", 3: "Orthogonal", 4: "Merge", 5: "Split",
            6: "GemmOut", 7: "GemmIn", 8: "ScalingPLUQ", 9: "ScalingLDLT"}

_lib = None


class SpandError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


_PROTOS = {
    "spand_last_error": (C.c_char_p, []),
    "spand_tree_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "spand_tree_destroy": (C.c_int, [C.c_void_p]),
    "spand_tree_set_verb": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_use_geo": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_Xcoo": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "spand_tree_set_tol": (C.c_int, [C.c_void_p, C.c_double]),
    "spand_tree_set_skip": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_scaling_kind": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_symm_kind": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_part_kind": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_use_sparsify": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_fp32": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_preserve": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_set_phi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "spand_tree_partition": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "spand_tree_partition_lorasp": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "spand_tree_factorize_lorasp": (C.c_int, [C.c_void_p]),
    "spand_tree_assemble": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "spand_tree_factorize": (C.c_int, [C.c_void_p]),
    "spand_tree_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "spand_tree_solve_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "spand_tree_solve_device_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "spand_cg": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                           C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_gmres": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int,
                              C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_gmres_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                     C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_fgmres": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int,
                               C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_ir": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                           C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_cg_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                  C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_adjoint_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "spand_batch_factorize": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "spand_forest_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_int]),
    "spand_forest_destroy": (C.c_int, [C.c_void_p]),
    "spand_forest_offsets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "spand_forest_assemble_values": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int]),
    "spand_forest_factorize": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_forest_solve_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_forest_cg": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p,
                                  C.c_void_p]),
    "spand_forest_cg_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p,
                                         C.c_void_p]),
    "spand_forest_num_ranks": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_forest_get_ranks": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_forest_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.c_int]),
    "spand_forest_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_forest_profile_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_forest_profile_entry": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.POINTER(C.c_longlong),
                                             C.POINTER(C.c_double)]),
    "spand_forest_profile_reset": (C.c_int, [C.c_void_p]),
    "spand_batch_cg": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p,
                                 C.c_void_p]),
    "spand_batch_cg_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                        C.c_void_p, C.c_void_p]),
    "spand_tree_assemble_values": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int]),
    "spand_cg_multi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                 C.c_void_p, C.c_void_p]),
    "spand_cg_multi_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                        C.c_void_p, C.c_void_p]),
    "spand_tree_get_N": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_tree_get_perm": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_tree_nnz": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "spand_tree_get_stop": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_tree_level_log": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_tree_num_ranks": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_tree_get_ranks": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_tree_num_ops": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_tree_get_ops": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_tree_get_op_matrix": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "spand_tree_get_op_tau": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "spand_tree_get_op_perm": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "spand_tree_get_op_signs": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "spand_tree_timings": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spand_tree_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.c_int]),
    "spand_tree_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "spand_tree_bench_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                        C.c_void_p]),
    "spand_tree_assembled_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "spand_tree_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "spand_tree_profile_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_tree_profile_entry": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.POINTER(C.c_longlong),
                                           C.POINTER(C.c_double)]),
    "spand_tree_profile_reset": (C.c_int, [C.c_void_p]),
    "spand_tree_qrcp_wave_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "spand_tree_qrcp_wave": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "spand_tree_qrcp_wave_candidate": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int),
                                                 C.POINTER(C.c_double)]),
    "spand_tree_work_count": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "spand_tree_work_entry": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]),
}


def exported_symbols():
    return list(_PROTOS)


def lib():
    """Load the in-tree C-ABI library; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise SpandError(rc, lib().spand_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _csc(A):
    A = A.tocsc()
    cp = np.ascontiguousarray(A.indptr, dtype=np.int32)
    rv = np.ascontiguousarray(A.indices, dtype=np.int32)
    vv = np.ascontiguousarray(A.data, dtype=np.float64)
    return A.shape[0], cp, rv, vv


LOG_KEYS = ["dofs_nd", "dofs_left_nd", "dofs_left_elim", "dofs_left_spars", "rank_before_sum", "rank_after_sum",
            "rank_after_count", "ignored", "nbrs_sum", "nbrs_count", "fact_nnz"]


class Tree:
    """spaND::Tree on one GB300 (include/tree.h:133-197)."""

    def __init__(self, nlevels: int):
        self.L = lib()
        h = C.c_void_p()
        _check(self.L.spand_tree_create(C.byref(h), int(nlevels)))
        self.h = h
        self.nlevels = int(nlevels)
        self._A = None

    def close(self):
        if getattr(self, "h", None):
            self.L.spand_tree_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # setters (include/tree.h:133-147)
    def set_verb(self, v): _check(self.L.spand_tree_set_verb(self.h, int(bool(v))))
    def set_use_geo(self, g): _check(self.L.spand_tree_set_use_geo(self.h, int(bool(g))))
    def set_tol(self, tol): _check(self.L.spand_tree_set_tol(self.h, float(tol)))
    def set_skip(self, s): _check(self.L.spand_tree_set_skip(self.h, int(s)))
    def set_scaling_kind(self, k): _check(self.L.spand_tree_set_scaling_kind(self.h, int(k)))
    def set_symm_kind(self, k): _check(self.L.spand_tree_set_symm_kind(self.h, int(k)))
    def set_part_kind(self, k): _check(self.L.spand_tree_set_part_kind(self.h, int(k)))
    def set_use_sparsify(self, u): _check(self.L.spand_tree_set_use_sparsify(self.h, int(bool(u))))
    def set_fp32(self, f): _check(self.L.spand_tree_set_fp32(self.h, int(bool(f))))
    def set_preserve(self, p): _check(self.L.spand_tree_set_preserve(self.h, int(bool(p))))

    def set_phi(self, phi):
        """Vectors to preserve (include/tree.h:136): N x nphi (or N), natural ordering; copied."""
        phi = np.asarray(phi, dtype=np.float64)
        if phi.ndim == 1:
            phi = phi[:, None]
        phi = np.asfortranarray(phi)
        _check(self.L.spand_tree_set_phi(self.h, phi.ctypes.data, phi.shape[0], phi.shape[1]))

    def set_Xcoo(self, X):
        X = np.asfortranarray(X, dtype=np.float64)
        self._X = X
        _check(self.L.spand_tree_set_Xcoo(self.h, _ptr(X), X.shape[0], X.shape[1]))

    def partition(self, A):
        n, cp, rv, _ = _csc(A)
        out = np.zeros((n, 6), dtype=np.int32)
        _check(self.L.spand_tree_partition(self.h, n, _ptr(cp), _ptr(rv), _ptr(out)))
        self.n = n
        return out

    def partition_lorasp(self, A):
        """LoRaSp ordering (include/tree.h:177): returns the part of every dof."""
        n, cp, rv, _ = _csc(A)
        out = np.zeros(n, dtype=np.int32)
        _check(self.L.spand_tree_partition_lorasp(self.h, n, _ptr(cp), _ptr(rv), _ptr(out)))
        self.n = n
        return out

    def factorize_lorasp(self):
        """include/tree.h:187 (SPD / LLT)."""
        _check(self.L.spand_tree_factorize_lorasp(self.h))

    def assemble(self, A):
        n, cp, rv, vv = _csc(A)
        _check(self.L.spand_tree_assemble(self.h, n, _ptr(cp), _ptr(rv), _ptr(vv)))
        self._A = A

    def factorize(self):
        _check(self.L.spand_tree_factorize(self.h))

    def solve(self, x):
        """Return M^{-1} x for a vector or an (n, nrhs) array (src/tree.cpp:1610-1635)."""
        y = np.array(x, dtype=np.float64, order="F", copy=True)
        nrhs = 1 if y.ndim == 1 else y.shape[1]
        _check(self.L.spand_tree_solve(self.h, _ptr(y), nrhs, y.shape[0]))
        return y

    def solve_device(self, ptr: int, nrhs: int, ld: int):
        _check(self.L.spand_tree_solve_device(self.h, C.c_void_p(ptr), int(nrhs), int(ld)))

    def cg(self, b, iters=100, tol=1e-12, x0=None, verb=False):
        if np.ndim(b) == 2:
            return self.cg_multi(b, iters, tol, x0)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_cg(self.h, _ptr(b), _ptr(x), int(iters), float(tol), int(bool(verb)), C.byref(it),
                               C.byref(rr)))
        return x, it.value, rr.value

    def gmres(self, b, iters=100, restart=None, tol=1e-12, x0=None, verb=False):
        """Restarted GMRES (is.cpp:123-300) preconditioned by this tree, on the device
        (restart defaults to iters, as the reference's driver passes it).  Returns
        (x, iterations, |w_k| / |M^{-1} r_0|)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        restart = iters if restart is None else restart
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_gmres(self.h, _ptr(b), _ptr(x), int(iters), int(restart), float(tol), int(bool(verb)),
                                  C.byref(it), C.byref(rr)))
        return x, it.value, rr.value

    def gmres_device(self, b_ptr: int, x_ptr: int, iters=100, restart=None, tol=1e-12):
        restart = iters if restart is None else restart
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_gmres_device(self.h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), int(iters), int(restart),
                                         float(tol), C.byref(it), C.byref(rr)))
        return it.value, rr.value

    def fgmres(self, b, iters=100, restart=None, tol=1e-12, x0=None, verb=False):
        """Flexible (right-preconditioned) GMRES: stops on the true |b - Ax| < tol |b| also
        with an FP32 factor.  Returns (x, iterations, |b - Ax| / |b|)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        restart = iters if restart is None else restart
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_fgmres(self.h, _ptr(b), _ptr(x), int(iters), int(restart), float(tol), int(bool(verb)),
                                   C.byref(it), C.byref(rr)))
        return x, it.value, rr.value

    def ir(self, b, iters=100, tol=1e-12, x0=None, verb=False):
        """Iterative refinement (is.cpp:12-37) on the device.  Returns (x, iterations, |b - Ax|/|b|)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_ir(self.h, _ptr(b), _ptr(x), int(iters), float(tol), int(bool(verb)), C.byref(it),
                               C.byref(rr)))
        return x, it.value, rr.value

    def assemble_values(self, vals, on_device=False):
        """New values on the pattern of the last assemble() (CSC order).  vals: numpy array,
        or (on_device=True) the address of nnz doubles in device memory."""
        if on_device:
            _check(self.L.spand_tree_assemble_values(self.h, C.c_void_p(int(vals[0])), int(vals[1]), 1))
        else:
            v = np.ascontiguousarray(vals, dtype=np.float64)
            _check(self.L.spand_tree_assemble_values(self.h, _ptr(v), int(v.size), 0))

    def cg_multi(self, B, iters=100, tol=1e-12, X0=None):
        """Independent CGs on the columns of B (n x k) in lockstep (one multi-right-hand-side
        preconditioner application per iteration).  Returns X (n x k), the iteration count
        and the recurrence residual |r|/|b| of every column."""
        B = np.asfortranarray(B, dtype=np.float64)
        n, k = B.shape
        X = np.zeros((n, k), dtype=np.float64, order="F") if X0 is None else \
            np.array(X0, dtype=np.float64, order="F", copy=True)
        its = np.zeros(k, dtype=np.int32)
        rr = np.zeros(k, dtype=np.float64)
        _check(self.L.spand_cg_multi(self.h, _ptr(B), _ptr(X), int(k), int(n), int(iters), float(tol), _ptr(its),
                                     _ptr(rr)))
        return X, its, rr

    def cg_device(self, b_ptr: int, x_ptr: int, iters=100, tol=1e-12):
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_cg_device(self.h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), int(iters), float(tol),
                                      C.byref(it), C.byref(rr)))
        return it.value, rr.value

    def adjoint_device(self, g_ptr: int, x_ptr: int, lam_ptr: int, grad_ptr: int, iters=100, tol=1e-12):
        """lambda = A^{-T} g by PCG with this factor, grad[k] = -lambda[row_k] x[col_k] over
        the stored entries (CSC order); device addresses.  Returns (iterations, |r|/|g|)."""
        it = C.c_int()
        rr = C.c_double()
        _check(self.L.spand_adjoint_device(self.h, C.c_void_p(g_ptr), C.c_void_p(x_ptr), C.c_void_p(lam_ptr),
                                           C.c_void_p(grad_ptr), int(iters), float(tol), C.byref(it), C.byref(rr)))
        return it.value, rr.value

    # introspection
    def get_N(self):
        n = C.c_int()
        _check(self.L.spand_tree_get_N(self.h, C.byref(n)))
        return n.value

    def get_assembly_perm(self):
        p = np.zeros(self.get_N(), dtype=np.int32)
        _check(self.L.spand_tree_get_perm(self.h, _ptr(p)))
        return p

    def nnz(self):
        v = C.c_longlong()
        _check(self.L.spand_tree_nnz(self.h, C.byref(v)))
        return v.value

    def get_stop(self):
        v = C.c_int()
        _check(self.L.spand_tree_get_stop(self.h, C.byref(v)))
        return v.value

    def level_log(self):
        out = np.zeros((self.nlevels, 11), dtype=np.int64)
        _check(self.L.spand_tree_level_log(self.h, _ptr(out)))
        return [dict(zip(LOG_KEYS, map(int, r))) for r in out]

    def ranks(self):
        n = C.c_int()
        _check(self.L.spand_tree_num_ranks(self.h, C.byref(n)))
        out = np.zeros((n.value, 4), dtype=np.int32)
        if n.value:
            _check(self.L.spand_tree_get_ranks(self.h, _ptr(out)))
        return out

    def ops(self):
        n = C.c_int()
        _check(self.L.spand_tree_num_ops(self.h, C.byref(n)))
        out = np.zeros((n.value, 8), dtype=np.int32)
        if n.value:
            _check(self.L.spand_tree_get_ops(self.h, _ptr(out)))
        return out

    def op_matrix(self, idx, rows, cols):
        buf = np.zeros(max(rows * cols, 1))
        _check(self.L.spand_tree_get_op_matrix(self.h, int(idx), _ptr(buf)))
        return buf[: rows * cols].reshape((cols, rows)).T

    def op_signs(self, idx, n):
        """sign(D) of a ScalingLDLT op (n entries)."""
        buf = np.zeros(max(n, 1))
        _check(self.L.spand_tree_get_op_signs(self.h, int(idx), _ptr(buf)))
        return buf[:n]

    def op_perm(self, idx, n):
        """Row permutation of a ScalingPLUQ / ScalingLDLT op (n entries)."""
        buf = np.zeros(max(n, 1), dtype=np.int32)
        _check(self.L.spand_tree_get_op_perm(self.h, int(idx), _ptr(buf)))
        return buf[:n]

    def op_tau(self, idx, k):
        buf = np.zeros(max(k, 1))
        _check(self.L.spand_tree_get_op_tau(self.h, int(idx), _ptr(buf)))
        return buf[:k]

    def timings(self):
        out = np.zeros(3)
        _check(self.L.spand_tree_timings(self.h, _ptr(out)))
        return dict(partition=out[0], assemble=out[1], factorize=out[2])

    def launches(self, reset=False):
        v = C.c_longlong()
        _check(self.L.spand_tree_launches(self.h, C.byref(v), int(bool(reset))))
        return v.value

    def bench_step(self, b_ptr: int, x_ptr: int, iters=200, tol=1e-10, nrhs=1):
        """factorize + device CG (nrhs columns of n doubles each), timed with CUDA events on
        the tree's stream."""
        out = np.zeros(4)
        _check(self.L.spand_tree_bench_step(self.h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), int(nrhs), int(iters),
                                            float(tol), _ptr(out)))
        return dict(factor_ms=out[0], pcg_ms=out[1], iterations=int(out[2]), relres=out[3])

    def assembled_bytes(self):
        v = C.c_longlong()
        _check(self.L.spand_tree_assembled_bytes(self.h, C.byref(v)))
        return v.value

    def set_profiling(self, on: bool):
        _check(self.L.spand_tree_set_profiling(self.h, int(bool(on))))

    def profile(self, reset=True):
        n = C.c_int()
        _check(self.L.spand_tree_profile_count(self.h, C.byref(n)))
        out = {}
        for i in range(n.value):
            name = C.create_string_buffer(64)
            la = C.c_longlong()
            ms = C.c_double()
            _check(self.L.spand_tree_profile_entry(self.h, i, name, C.byref(la), C.byref(ms)))
            out[name.value.decode()] = dict(launches=la.value, ms=ms.value)
        if reset:
            _check(self.L.spand_tree_profile_reset(self.h))
        return out

    def qrcp_waves(self):
        """The QRCP launch of every sparsification wave: a list of dicts (level, wave, items,
        cap_rows, rpl, cs, threads, smem, vec_rows) with 'timed': [(conf dict, ms), ...], the
        configurations the measuring factorization timed for the wave."""
        n = C.c_int()
        _check(self.L.spand_tree_qrcp_wave_count(self.h, C.byref(n)))
        keys = ("level", "wave", "items", "cap_rows", "rpl", "cs", "threads", "smem", "vec_rows")
        ckeys = ("rpl", "cs", "threads", "smem", "vec_rows")
        out = []
        for i in range(n.value):
            conf = (C.c_int * 9)()
            nc = C.c_int()
            _check(self.L.spand_tree_qrcp_wave(self.h, i, conf, C.byref(nc)))
            d = dict(zip(keys, list(conf)))
            d["timed"] = []
            for k in range(nc.value):
                c5 = (C.c_int * 5)()
                ms = C.c_double()
                _check(self.L.spand_tree_qrcp_wave_candidate(self.h, i, k, c5, C.byref(ms)))
                d["timed"].append((dict(zip(ckeys, list(c5))), ms.value))
            out.append(d)
        return out

    def work(self, which: str = "factor"):
        w = 0 if which == "factor" else 1
        n = C.c_int()
        _check(self.L.spand_tree_work_count(self.h, w, C.byref(n)))
        out = {}
        for i in range(n.value):
            name = C.create_string_buffer(64)
            b = C.c_double()
            f = C.c_double()
            _check(self.L.spand_tree_work_entry(self.h, w, i, name, C.byref(b), C.byref(f)))
            out[name.value.decode()] = dict(bytes=b.value, flops=f.value)
        return out

    def device_bytes(self):
        v = C.c_longlong()
        _check(self.L.spand_tree_device_bytes(self.h, C.byref(v)))
        return v.value


def batch_factorize(trees):
    """Factorize many trees at once (every tree's launches queued on its own stream before
    the first wait).  Returns the status of every tree (0: factored)."""
    L = lib()
    hs = (C.c_void_p * len(trees))(*[t.h for t in trees])
    st = np.zeros(len(trees), dtype=np.int32)
    rc = L.spand_batch_factorize(hs, len(trees), _ptr(st))
    if rc not in (0, 4):
        _check(rc)
    return st


def batch_cg(trees, bs, iters=100, tol=1e-12):
    """cg on many independent systems in lockstep: tree k solves with bs[k].  Returns
    ([x_k], iterations, recurrence residuals)."""
    L = lib()
    k = len(trees)
    bs = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
    xs = [np.zeros_like(b) for b in bs]
    hs = (C.c_void_p * k)(*[t.h for t in trees])
    bp = (C.c_void_p * k)(*[b.ctypes.data for b in bs])
    xp = (C.c_void_p * k)(*[x.ctypes.data for x in xs])
    its = np.zeros(k, dtype=np.int32)
    rr = np.zeros(k, dtype=np.float64)
    _check(L.spand_batch_cg(hs, k, bp, xp, int(iters), float(tol), _ptr(its), _ptr(rr)))
    return xs, its, rr


def batch_cg_device(trees, b_ptrs, x_ptrs, iters=100, tol=1e-12):
    """batch_cg on device vectors (addresses of FP64 arrays of each tree's size)."""
    L = lib()
    k = len(trees)
    hs = (C.c_void_p * k)(*[t.h for t in trees])
    bp = (C.c_void_p * k)(*[int(p) for p in b_ptrs])
    xp = (C.c_void_p * k)(*[int(p) for p in x_ptrs])
    its = np.zeros(k, dtype=np.int32)
    rr = np.zeros(k, dtype=np.float64)
    _check(L.spand_batch_cg_device(hs, k, bp, xp, int(iters), float(tol), _ptr(its), _ptr(rr)))
    return its, rr


class Forest:
    """Many independent SPD systems factored and solved as one block-diagonal matrix
    (C ABI ``spand_forest_*``).  ``trees``: partitioned and assembled Trees with one
    tolerance, skip and precision; each keeps its own ordering and hierarchy.  Vectors are
    stacked: system k at ``offsets[k]:offsets[k+1]``."""

    def __init__(self, trees):
        self.L = lib()
        k = len(trees)
        hs = (C.c_void_p * k)(*[t.h for t in trees])
        h = C.c_void_p()
        _check(self.L.spand_forest_create(C.byref(h), hs, k))
        self.h = h
        self.count = k
        self.offsets = np.zeros(k + 1, dtype=np.int64)
        self.value_offsets = np.zeros(k + 1, dtype=np.int64)
        _check(self.L.spand_forest_offsets(self.h, _ptr(self.offsets), _ptr(self.value_offsets)))
        self.N = int(self.offsets[-1])

    def close(self):
        if getattr(self, "h", None):
            self.L.spand_forest_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def assemble_values(self, vals, on_device=False):
        """All systems' values, stacked (numpy array, or (address, nnz) of device memory)."""
        if on_device:
            _check(self.L.spand_forest_assemble_values(self.h, C.c_void_p(int(vals[0])), int(vals[1]), 1))
        else:
            v = np.ascontiguousarray(vals, dtype=np.float64)
            _check(self.L.spand_forest_assemble_values(self.h, _ptr(v), int(v.size), 0))

    def factorize(self):
        """Raises SpandError when a pivot fails; ``failed_system`` names the system."""
        f = C.c_int(-1)
        rc = self.L.spand_forest_factorize(self.h, C.byref(f))
        self.failed_system = f.value
        _check(rc)

    def solve_device(self, x_ptr: int):
        _check(self.L.spand_forest_solve_device(self.h, C.c_void_p(int(x_ptr))))

    def stack(self, bs):
        return np.concatenate([np.ascontiguousarray(b, dtype=np.float64) for b in bs])

    def split(self, x):
        return [x[self.offsets[k]:self.offsets[k + 1]] for k in range(self.count)]

    def cg(self, bs, iters=100, tol=1e-12):
        """cg on every system (bs: list of right-hand sides, or one stacked vector).
        Returns ([x_k], iterations, recurrence residuals)."""
        b = self.stack(bs) if isinstance(bs, (list, tuple)) else np.ascontiguousarray(bs, dtype=np.float64)
        x = np.zeros_like(b)
        its = np.zeros(self.count, dtype=np.int32)
        rr = np.zeros(self.count)
        _check(self.L.spand_forest_cg(self.h, _ptr(b), _ptr(x), int(iters), float(tol), _ptr(its), _ptr(rr)))
        return self.split(x), its, rr

    def cg_device(self, b_ptr: int, x_ptr: int, iters=100, tol=1e-12):
        """Stacked device vectors (x: initial guess).  Returns (iterations, residuals)."""
        its = np.zeros(self.count, dtype=np.int32)
        rr = np.zeros(self.count)
        _check(self.L.spand_forest_cg_device(self.h, C.c_void_p(int(b_ptr)), C.c_void_p(int(x_ptr)), int(iters),
                                             float(tol), _ptr(its), _ptr(rr)))
        return its, rr

    def ranks(self):
        n = C.c_int()
        _check(self.L.spand_forest_num_ranks(self.h, C.byref(n)))
        out = np.zeros((n.value, 5), dtype=np.int32)
        if n.value:
            _check(self.L.spand_forest_get_ranks(self.h, _ptr(out)))
        return out  # system, level, cluster order, rows, rank

    def launches(self, reset=False):
        n = C.c_longlong()
        _check(self.L.spand_forest_launches(self.h, C.byref(n), int(bool(reset))))
        return n.value

    def set_profiling(self, on: bool):
        _check(self.L.spand_forest_set_profiling(self.h, int(bool(on))))

    def profile(self, reset=True):
        n = C.c_int()
        _check(self.L.spand_forest_profile_count(self.h, C.byref(n)))
        out = {}
        for i in range(n.value):
            name = C.create_string_buffer(64)
            la = C.c_longlong()
            ms = C.c_double()
            _check(self.L.spand_forest_profile_entry(self.h, i, name, C.byref(la), C.byref(ms)))
            out[name.value.decode()] = dict(launches=la.value, ms=ms.value)
        if reset:
            _check(self.L.spand_forest_profile_reset(self.h))
        return out
