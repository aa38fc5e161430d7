"""ORACLE - TEST INFRASTRUCTURE ONLY.

ctypes front end of the CPU restatement of the reference DAFMM + GMRES path
(oracle/ls_oracle.cpp). Only tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py import this module, and only as the checker or as
the timed CPU baseline. The reference needs Eigen and Boost.Math, which are
absent, so it cannot be compiled and run here; the oracle is pinned to the
assembly log the reference's README publishes through the adaptive-tree
restatement (oracle/ls_oracle_adaptive.cpp, tests/test_oracle_pinned.py).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libls_oracle.so")
MAX_BUMPS = 8


class OraCfg(ctypes.Structure):
    _fields_ = [
        ("nCones_LFR", ctypes.c_int),
        ("nChebNodes", ctypes.c_int),
        ("yes2DFMM", ctypes.c_int),
        ("TOL_POW", ctypes.c_int),
        ("degreeOfBases", ctypes.c_int),
        ("nLevelsUniform", ctypes.c_int),
        ("Qchoice", ctypes.c_int),
        ("findPhi", ctypes.c_int),
        ("reference_rounding", ctypes.c_int),
        ("n_bumps", ctypes.c_int),
        ("L", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("bump_cx", ctypes.c_double * MAX_BUMPS),
        ("bump_cy", ctypes.c_double * MAX_BUMPS),
        ("bump_a", ctypes.c_double * MAX_BUMPS),
        ("bump_w", ctypes.c_double * MAX_BUMPS),
    ]


def build():
    """Compiles the oracle with its Makefile (g++, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.ora_create.restype = vp
        L.ora_create.argtypes = [ctypes.POINTER(OraCfg), ctypes.c_char_p, ctypes.c_int]
        L.ora_destroy.argtypes = [vp]
        for name in ("ora_N", "ora_nlevels", "ora_level_lfr", "ora_rank"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = [vp]
        for name in ("ora_points", "ora_contrast", "ora_rhs", "ora_get_M", "ora_get_near"):
            getattr(L, name).argtypes = [vp, dp]
        L.ora_skeleton_dump.restype = ctypes.c_long
        L.ora_skeleton_dump.argtypes = [vp, ip, ctypes.c_long]
        L.ora_matvec.argtypes = [vp, dp, dp]
        L.ora_dense_matvec.argtypes = [vp, dp, dp]
        L.ora_gmres.restype = ctypes.c_int
        L.ora_gmres.argtypes = [vp, dp, ctypes.c_int, ctypes.c_double, dp, dp, ip]
        L.ora_gmres_restarted.restype = ctypes.c_int
        L.ora_gmres_restarted.argtypes = [vp, dp, ctypes.c_int, ctypes.c_int, dp]
        L.ora_set_threads.argtypes = [ctypes.c_int]
        L.ora_gauss_legendre.argtypes = [ctypes.c_int, dp, dp]
        L.ora_bessel_jy.argtypes = [ctypes.c_int, ctypes.c_double, dp, dp]
        L.ora_colpiv_solve.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp]
        L.ora_adaptive_report.restype = ctypes.c_int
        L.ora_adaptive_report.argtypes = [ctypes.POINTER(OraCfg), ctypes.c_int, ip, ip, ctypes.c_int]
        L.ora_bessel_jy_orders.argtypes = [ctypes.c_int, ctypes.c_double, dp, dp]
        L.ora_adaptive_create.restype = vp
        L.ora_adaptive_create.argtypes = [ctypes.POINTER(OraCfg), ctypes.c_int]
        L.ora_adaptive_destroy.argtypes = [vp]
        for name in ("ora_adaptive_N", "ora_adaptive_unmatched_neighbors"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = [vp]
        for name in ("ora_adaptive_points", "ora_adaptive_rhs"):
            getattr(L, name).argtypes = [vp, dp]
        L.ora_adaptive_matvec.argtypes = [vp, dp, dp]
        L.ora_adaptive_gmres_restarted.argtypes = [vp, dp, ctypes.c_int, ctypes.c_int, dp]
        L.ora_adaptive_set_per_order_bessel.argtypes = [ctypes.c_int]
        L.ora_bessel_jy_orders.restype = None
        L.ora_adaptive_set_per_order_bessel.argtypes = [ctypes.c_int]
        L.ora_adaptive_set_per_order_bessel.restype = None
        L.ora_adaptive_skeletons.restype = ctypes.c_long
        L.ora_adaptive_skeletons.argtypes = [ctypes.POINTER(OraCfg), ctypes.c_int, ip, ctypes.c_long]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_cfg(d):
    """Builds an OraCfg from a plain dict of the same field names."""
    c = OraCfg()
    for name, _ in OraCfg._fields_:
        if name.startswith("bump_"):
            vals = list(d.get(name, []))
            arr = (ctypes.c_double * MAX_BUMPS)(*(vals + [0.0] * (MAX_BUMPS - len(vals))))
            setattr(c, name, arr)
        elif name in d:
            setattr(c, name, d[name])
    return c


def set_threads(n):
    lib().ora_set_threads(int(n))


class Oracle:
    """The reference DAFMM operator restated on the CPU (one per config)."""

    def __init__(self, cfg):
        L = lib()
        self._cfg = make_cfg(cfg)
        err = ctypes.create_string_buffer(256)
        self._h = L.ora_create(ctypes.byref(self._cfg), err, 256)
        if not self._h:
            raise ValueError("oracle: " + err.value.decode())
        self.N = L.ora_N(self._h)
        self.nlevels = L.ora_nlevels(self._h)
        self.level_lfr = L.ora_level_lfr(self._h)
        self.rank = L.ora_rank(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().ora_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def points(self):
        a = np.empty((self.N, 2))
        lib().ora_points(self._h, _dp(a))
        return a

    def contrast(self):
        a = np.empty(self.N)
        lib().ora_contrast(self._h, _dp(a))
        return a

    def rhs(self):
        a = np.empty(self.N, dtype=np.complex128)
        lib().ora_rhs(self._h, _dp(a))
        return a

    def far_moments(self):
        """M at the leaf level, shape (rank, 31): M[i, n + 15] (column i)."""
        a = np.empty((self.rank, 31), dtype=np.complex128)
        lib().ora_get_M(self._h, _dp(a))
        return a

    def near_blocks(self):
        """Colleague blocks, shape (9, rank, rank) in (row, col) order."""
        a = np.empty((9, self.rank, self.rank), dtype=np.complex128)
        lib().ora_get_near(self._h, _dp(a))
        return np.ascontiguousarray(a.transpose(0, 2, 1))

    def skeleton_dump(self):
        n = lib().ora_skeleton_dump(self._h, None, 0)
        a = np.empty(n, dtype=np.int32)
        lib().ora_skeleton_dump(self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
        return a

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        lib().ora_matvec(self._h, _dp(x), _dp(y))
        return y

    def dense_matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        lib().ora_dense_matvec(self._h, _dp(x), _dp(y))
        return y

    def gmres(self, b, max_iter=400, tol=1e-10):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        hist = np.zeros(max_iter + 2)
        it = ctypes.c_int(0)
        lib().ora_gmres(self._h, _dp(b), max_iter, tol, _dp(x), _dp(hist), ctypes.byref(it))
        return x, hist[: it.value + 1], it.value

    def gmres_restarted(self, b, m, restarts):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        lib().ora_gmres_restarted(self._h, _dp(b), m, restarts, _dp(x))
        return x


class AdaptiveOracle:
    """The adaptive-tree restatement with its full operator: createTree with
    resolveContrast, the 2:1 level restriction, mixed-level interaction lists,
    NCA, the ten matvec phases with leaves on several levels and the
    colleague / fine / separated-fine / coarse near blocks, and the
    reference's RestartedGMRES (oracle/ls_oracle_adaptive.cpp).
    treeAdaptivity >= 0: the adaptive tree with epsilonTree 10^-treeAdaptivity
    (the reference's default path); < 0: the uniform tree of nLevelsUniform
    levels."""

    def __init__(self, cfg, treeAdaptivity=5, per_order_bessel=False):
        lib().ora_adaptive_set_per_order_bessel(1 if per_order_bessel else 0)
        c = make_cfg(cfg)
        self._h = lib().ora_adaptive_create(ctypes.byref(c), int(treeAdaptivity))
        if not self._h:
            raise ValueError("bad configuration")
        self.N = lib().ora_adaptive_N(self._h)
        self.unmatched_neighbors = lib().ora_adaptive_unmatched_neighbors(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().ora_adaptive_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def points(self):
        a = np.empty((self.N, 2))
        lib().ora_adaptive_points(self._h, _dp(a))
        return a

    def rhs(self):
        b = np.empty(self.N, dtype=np.complex128)
        lib().ora_adaptive_rhs(self._h, _dp(b))
        return b

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        lib().ora_adaptive_matvec(self._h, _dp(x), _dp(y))
        return y

    def gmres_restarted(self, b, m, restarts):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        lib().ora_adaptive_gmres_restarted(self._h, _dp(b), int(m), int(restarts), _dp(x))
        return x


def gauss_legendre(n):
    nodes, w = np.empty(n), np.empty(n)
    lib().ora_gauss_legendre(n, _dp(nodes), _dp(w))
    return nodes, w


def bessel_jy(n, x):
    j, y = ctypes.c_double(), ctypes.c_double()
    lib().ora_bessel_jy(n, x, ctypes.byref(j), ctypes.byref(y))
    return j.value, y.value


def colpiv_solve(A, b):
    A = np.asfortranarray(A, dtype=np.complex128)
    m, n = A.shape
    b = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.empty(n, dtype=np.complex128)
    Af = np.ascontiguousarray(A.T).reshape(-1)  # column-major flat
    lib().ora_colpiv_solve(m, n, _dp(Af), _dp(b), _dp(x))
    return x


def adaptive_report(cfg, tree_adaptivity, per_order_bessel=True):
    """Adaptive-tree assembly statistics (ls_oracle_adaptive.cpp).

    Returns {"nLevels", "level_LFR", "N", "levels": [...]}; each level entry
    is one line the reference prints while choosing NCA skeletons
    (GMRES/G_FMM2DTree.hpp:2238, 2384, 3418, 3570): direction "O"/"I",
    level j, Nboxes, k (HFR levels only, else None), rows, cols, Crank.
    per_order_bessel: far-field Bessel orders from one library call each, as
    the reference calls Boost (default), or from the recurrence that the
    uniform oracle and the library use."""
    c = make_cfg(cfg)
    head = (ctypes.c_int * 4)()
    cap = 7 * 64
    rec = (ctypes.c_int * cap)()
    lib().ora_adaptive_set_per_order_bessel(1 if per_order_bessel else 0)
    try:
        n = lib().ora_adaptive_report(ctypes.byref(c), int(tree_adaptivity), head, rec, cap)
    finally:
        lib().ora_adaptive_set_per_order_bessel(0)
    if n < 0:
        raise ValueError("ora_adaptive_report: invalid configuration")
    levels = []
    for r in range(min(n, cap) // 7):
        d, j, nb, k, rows, cols, rk = rec[7 * r:7 * r + 7]
        levels.append({"dir": "OI"[d], "j": j, "Nboxes": nb, "k": None if k < 0 else k,
                       "rows": rows, "cols": cols, "Crank": rk})
    return {"nLevels": head[0], "level_LFR": head[1], "N": head[2], "levels": levels}


def _parse_skeletons(buf, n_lists, skip):
    out, p = {}, 0
    while p < len(buf):
        key = (int(buf[p]), int(buf[p + 1]), int(buf[p + 2]))
        p += 3 + skip
        lists = []
        for _ in range(n_lists):
            m = int(buf[p])
            lists.append(buf[p + 1:p + 1 + m].tolist())
            p += 1 + m
        out[key] = lists
    return out


def adaptive_skeletons(cfg, tree_adaptivity, per_order_bessel=False):
    """{(j, k, cone): [out_charge, out_check, in_charge, in_check]} of the
    adaptive restatement; tree_adaptivity < 0 builds the uniform tree.
    per_order_bessel as in adaptive_report (default: the shared recurrence,
    the method of the uniform oracle)."""
    c = make_cfg(cfg)
    lib().ora_adaptive_set_per_order_bessel(1 if per_order_bessel else 0)
    try:
        n = lib().ora_adaptive_skeletons(ctypes.byref(c), int(tree_adaptivity), None, 0)
        if n < 0:
            raise ValueError("ora_adaptive_skeletons: invalid configuration")
        buf = np.empty(n, dtype=np.int32)
        lib().ora_adaptive_skeletons(ctypes.byref(c), int(tree_adaptivity),
                                     buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
    finally:
        lib().ora_adaptive_set_per_order_bessel(0)
    return _parse_skeletons(buf, 4, 0)


def bessel_jy_orders(nmax, x):
    """J_0..J_nmax(x), Y_0..Y_nmax(x) by the far-field recurrences."""
    J = np.empty(nmax + 1)
    Y = np.empty(nmax + 1)
    lib().ora_bessel_jy_orders(int(nmax), float(x), _dp(J), _dp(Y))
    return J, Y
