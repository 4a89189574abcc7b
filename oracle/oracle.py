"""ctypes front-end of the CPU oracle (test infrastructure only).

The oracle restates the reference's Tree (partition / assemble / factorize / solve) and
its CG / IR drivers in plain C++ (``oracle/spand_oracle.cpp``).  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use it, always as
the checker: the product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "spand_oracle.cpp")
LIB = os.path.join(HERE, "build", "libspand_oracle.so")

OP_NAMES = {0: "ScalingLLT", 1: "GemmSymmOut", 2: "GemmSymmIn", 3: "Orthogonal", 4: "Merge", 5: "Split",
            6: "GemmOut", 7: "GemmIn", 8: "ScalingPLUQ"}


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (a few seconds)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        tmp = LIB + ".tmp"
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-o", tmp, SRC, "-ldl"])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        P, I, D, LL = C.c_void_p, C.c_int, C.c_double, C.c_longlong
        pi, pd, pll = C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_longlong)
        sig = {
            "orc_create": (P, [I]), "orc_destroy": (None, [P]), "orc_error": (C.c_char_p, [P]),
            "orc_set_tol": (None, [P, D]), "orc_set_skip": (None, [P, I]),
            "orc_set_symm_kind": (None, [P, I]), "orc_set_scaling_kind": (None, [P, I]),
            "orc_set_use_sparsify": (None, [P, I]), "orc_set_Xcoo": (None, [P, pd, I, I]),
            "orc_partition": (I, [P, I, pi, pi]), "orc_get_partition": (None, [P, pi]),
            "orc_get_perm": (None, [P, pi]), "orc_num_clusters": (I, [P, I]),
            "orc_get_clusters": (None, [P, I, pi]),
            "orc_assemble": (I, [P, I, pi, pi, pd]), "orc_trailing": (I, [P, pi, pi, pd]),
            "orc_factorize": (I, [P]), "orc_solve": (None, [P, pd]),
            "orc_solve_multi": (None, [P, pd, I, I]),
            "orc_cg": (I, [P, pd, pd, I, D, pd]), "orc_ir": (I, [P, pd, pd, I, D]),
            "orc_nnz": (LL, [P]), "orc_get_stop": (I, [P]), "orc_get_log": (None, [P, pll]),
            "orc_get_prof": (None, [P, pd]), "orc_get_times": (None, [P, pd]),
            "orc_num_ranks": (I, [P]), "orc_get_ranks": (None, [P, pi]),
            "orc_num_ops": (I, [P]), "orc_get_ops": (None, [P, pi]),
            "orc_get_op_matrix": (LL, [P, I, pd]), "orc_get_op_tau": (I, [P, I, pd]),
            "orc_dense_potf": (I, [I, pd]), "orc_dense_geqp3": (None, [I, I, pd, pi, pd]),
            "orc_dense_getf": (I, [I, pd, pi]), "orc_choose_rank": (I, [pd, I, D]),
            "orc_spmv": (None, [P, pd, pd]),
            "orc_gmres": (I, [P, pd, pd, I, I, D, pd]),
            "orc_get_op_u": (C.c_longlong, [P, I, pd]), "orc_get_op_perm": (I, [P, I, pi]),
            "orc_get_op_signs": (I, [P, I, pd]),
            "orc_set_preserve": (None, [P, I]), "orc_set_phi": (None, [P, pd, I, I]),
            "orc_use_lapack": (I, [C.c_char_p, C.c_char_p, I]),
            "orc_partition_lorasp": (I, [P, I, pi, pi]), "orc_get_rb_parts": (None, [P, pi]),
            "orc_factorize_lorasp": (I, [P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def use_lapack(threads=0):
    """Route the oracle's dense kernels through the CBLAS / LAPACKE of scipy's bundled
    OpenBLAS, as the reference calls them (timing only: LAPACK's dgeqp3 pivots without the
    oracle's tie rule).  threads > 0 sets OpenBLAS's thread count.  Returns the library path,
    or None when no such library is found (the restated kernels stay in use)."""
    import glob
    try:
        import scipy
    except ImportError:
        return None
    base = os.path.dirname(scipy.__file__)
    for path in sorted(glob.glob(os.path.join(base, "..", "scipy.libs", "libscipy_openblas*.so*")) +
                       glob.glob(os.path.join(base, ".libs", "libscipy_openblas*.so*"))):
        if lib().orc_use_lapack(path.encode(), b"scipy_", int(threads)) == 0:
            return os.path.realpath(path)
    return None


def use_restated():
    """Back to the restated kernels (the default)."""
    lib().orc_use_lapack(None, None, 0)


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleTree:
    """Mirror of the reference ``spaND::Tree`` API (include/tree.h:133-197) on the CPU oracle."""

    SPD, SYM, GEN = 0, 1, 2
    LLT, PLU, PLUQ, LDLT = 0, 3, 4, 5

    def __init__(self, nlevels: int):
        self.L = lib()
        self.h = self.L.orc_create(nlevels)
        self.nlevels = nlevels
        self.n = 0
        self._keep = []

    def __del__(self):
        try:
            if self.h:
                self.L.orc_destroy(self.h)
        except Exception:
            pass

    # setters (tree.h:133-147)
    def set_tol(self, tol): self.L.orc_set_tol(self.h, float(tol))
    def set_skip(self, skip): self.L.orc_set_skip(self.h, int(skip))
    def set_symm_kind(self, k): self.L.orc_set_symm_kind(self.h, int(k))
    def set_scaling_kind(self, k): self.L.orc_set_scaling_kind(self.h, int(k))
    def set_use_sparsify(self, u): self.L.orc_set_use_sparsify(self.h, int(bool(u)))
    def set_preserve(self, on): self.L.orc_set_preserve(self.h, int(bool(on)))

    def set_phi(self, phi):
        """Vectors to preserve (tree.h:136): N x nphi, natural ordering (copied)."""
        phi = np.asfortranarray(np.atleast_2d(np.asarray(phi, dtype=np.float64).T).T)
        self.L.orc_set_phi(self.h, _dp(phi), phi.shape[0], phi.shape[1])

    def set_Xcoo(self, X):
        X = np.asfortranarray(X, dtype=np.float64)
        self._keep.append(X)
        self.L.orc_set_Xcoo(self.h, _dp(X), X.shape[0], X.shape[1])

    def _err(self):
        return self.L.orc_error(self.h).decode()

    def partition(self, A):
        A = A.tocsc()
        self.n = A.shape[0]
        cp = np.ascontiguousarray(A.indptr, dtype=np.int32)
        rv = np.ascontiguousarray(A.indices, dtype=np.int32)
        if self.L.orc_partition(self.h, self.n, _ip(cp), _ip(rv)) != 0:
            raise RuntimeError(self._err())
        out = np.zeros((self.n, 6), dtype=np.int32)
        self.L.orc_get_partition(self.h, _ip(out))
        return out

    def assemble(self, A):
        A = A.tocsc()
        cp = np.ascontiguousarray(A.indptr, dtype=np.int32)
        rv = np.ascontiguousarray(A.indices, dtype=np.int32)
        vv = np.ascontiguousarray(A.data, dtype=np.float64)
        if self.L.orc_assemble(self.h, A.shape[0], _ip(cp), _ip(rv), _dp(vv)) != 0:
            raise RuntimeError(self._err())

    def factorize(self):
        if self.L.orc_factorize(self.h) != 0:
            raise RuntimeError(self._err())

    def partition_lorasp(self, A):
        """LoRaSp ordering (tree.cpp:421-503): recursive bisection; returns the part of every dof."""
        A = A.tocsc()
        self.n = A.shape[0]
        cp = np.ascontiguousarray(A.indptr, dtype=np.int32)
        rv = np.ascontiguousarray(A.indices, dtype=np.int32)
        if self.L.orc_partition_lorasp(self.h, self.n, _ip(cp), _ip(rv)) != 0:
            raise RuntimeError(self._err())
        out = np.zeros(self.n, dtype=np.int32)
        self.L.orc_get_rb_parts(self.h, _ip(out))
        return out

    def factorize_lorasp(self):
        """tree.cpp:1553-1608 (SPD / LLT)."""
        if self.L.orc_factorize_lorasp(self.h) != 0:
            raise RuntimeError(self._err())

    def solve(self, x):
        x = np.array(x, dtype=np.float64, order="F", copy=True)
        if x.ndim == 1:
            self.L.orc_solve(self.h, _dp(x))
        else:
            self.L.orc_solve_multi(self.h, _dp(x), x.shape[1], x.shape[0])
        return x

    def cg(self, b, iters=100, tol=1e-12, x0=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        rr = np.zeros(1)
        it = self.L.orc_cg(self.h, _dp(b), _dp(x), int(iters), float(tol), _dp(rr))
        return x, it

    def gmres(self, b, iters=100, restart=None, tol=1e-12, x0=None):
        """Restarted GMRES (is.cpp:123-300); returns (x, iterations, preconditioned
        residual estimate |w_k| / |M^{-1} r_0|)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        rr = np.zeros(1)
        restart = iters if restart is None else restart
        it = self.L.orc_gmres(self.h, _dp(b), _dp(x), int(iters), int(restart), float(tol), _dp(rr))
        return x, it, float(rr[0])

    def ir(self, b, iters=100, tol=1e-12):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        it = self.L.orc_ir(self.h, _dp(b), _dp(x), int(iters), float(tol))
        return x, it

    def get_assembly_perm(self):
        p = np.zeros(self.n, dtype=np.int32)
        self.L.orc_get_perm(self.h, _ip(p))
        return p

    def clusters(self, lvl):
        k = self.L.orc_num_clusters(self.h, lvl)
        out = np.zeros((k, 6), dtype=np.int32)
        self.L.orc_get_clusters(self.h, lvl, _ip(out))
        return out

    def trailing(self):
        import scipy.sparse as sp
        k = self.L.orc_trailing(self.h, None, None, None)
        I = np.zeros(k, dtype=np.int32)
        J = np.zeros(k, dtype=np.int32)
        V = np.zeros(k)
        self.L.orc_trailing(self.h, _ip(I), _ip(J), _dp(V))
        return sp.csc_matrix((V, (I, J)), shape=(self.n, self.n))

    def nnz(self): return self.L.orc_nnz(self.h)
    def get_stop(self): return self.L.orc_get_stop(self.h)

    def level_log(self):
        out = np.zeros((self.nlevels, 11), dtype=np.int64)
        self.L.orc_get_log(self.h, out.ctypes.data_as(C.POINTER(C.c_longlong)))
        keys = ["dofs_nd", "dofs_left_nd", "dofs_left_elim", "dofs_left_spars", "rank_before_sum",
                "rank_after_sum", "rank_after_count", "ignored", "nbrs_sum", "nbrs_count", "fact_nnz"]
        return [dict(zip(keys, map(int, row))) for row in out]

    def prof(self):
        out = np.zeros((self.nlevels, 8))
        self.L.orc_get_prof(self.h, _dp(out))
        return out

    def times(self):
        out = np.zeros(3)
        self.L.orc_get_times(self.h, _dp(out))
        return dict(partition=out[0], assemble=out[1], factorize=out[2])

    def ranks(self):
        k = self.L.orc_num_ranks(self.h)
        out = np.zeros((k, 4), dtype=np.int32)
        if k:
            self.L.orc_get_ranks(self.h, _ip(out))
        return out  # (level, cluster order, rows, rank)

    def ops(self):
        k = self.L.orc_num_ops(self.h)
        out = np.zeros((k, 8), dtype=np.int32)
        if k:
            self.L.orc_get_ops(self.h, _ip(out))
        return out  # kind, level, self order, nbr order, ns, nn, rows, cols

    def op_matrix(self, idx, rows, cols):
        buf = np.zeros(rows * cols)
        self.L.orc_get_op_matrix(self.h, idx, _dp(buf))
        return buf.reshape((cols, rows)).T

    def op_u(self, idx, n):
        buf = np.zeros(n * n)
        self.L.orc_get_op_u(self.h, idx, _dp(buf))
        return buf.reshape((n, n)).T

    def op_signs(self, idx, n):
        buf = np.zeros(max(n, 1))
        self.L.orc_get_op_signs(self.h, idx, _dp(buf))
        return buf[:n]

    def op_perm(self, idx, n):
        buf = np.zeros(max(n, 1), dtype=np.int32)
        self.L.orc_get_op_perm(self.h, idx, _ip(buf))
        return buf[:n]

    def op_tau(self, idx, k):
        buf = np.zeros(max(k, 1))
        self.L.orc_get_op_tau(self.h, idx, _dp(buf))
        return buf[:k]


def dense_potf(A):
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    info = lib().orc_dense_potf(A.shape[0], _dp(A))
    return np.tril(A), info


def dense_geqp3(A):
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    jp = np.zeros(n, dtype=np.int32)
    tau = np.zeros(min(m, n))
    lib().orc_dense_geqp3(m, n, _dp(A), _ip(jp), _dp(tau))
    return A, jp, tau


def dense_getf(A):
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    p = np.zeros(A.shape[0], dtype=np.int32)
    info = lib().orc_dense_getf(A.shape[0], _dp(A), _ip(p))
    return A, p, info


def choose_rank(s, tol):
    s = np.ascontiguousarray(s, dtype=np.float64)
    return lib().orc_choose_rank(_dp(s), s.size, float(tol))
