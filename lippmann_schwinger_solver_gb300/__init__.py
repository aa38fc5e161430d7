"""GB300 DAFMM matvec + GMRES for the 2-D Lippmann-Schwinger equation.

Python front end of liblsdafmm.so (C ABI in include/ls_dafmm.h). The
classes mirror the reference's operator interface
(vaishna77/Lippmann_Schwinger_Solver, GMRES/GMRES.cpp):

* ``DFMM(inputs)`` with ``FMMTreeInitialisation()`` and
  ``MatVecProduct(b)`` (GMRES/GMRES.cpp:140-255);
* ``classGMRES().gmres(M, b, maxIterations, threshold)``
  (GMRES_Hybrid/include/gmres.hpp:54-119);
* ``RestartedGMRES(restart, S, m, inputs, b)`` (GMRES/GMRES.cpp:307-319);
* ``userkernel`` contrast / incident / right-hand-side functions
  (GMRES/GMRES.cpp:100-127).

Every numerical call runs on the GPU through the CUDA library; there is no
CPU implementation here. If the library is missing or no GPU is present the
calls raise instead of falling back.
"""
import ctypes
import dataclasses
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblsdafmm.so")
MAX_BUMPS = 8

LS_OK = 0
LS_E_INVALID = -1
LS_E_CUDA = -2
LS_E_NOMEM = -3
LS_E_NOT_CONVERGED = -4
LS_E_STATE = -5
LS_E_TIMEOUT = -6
LS_PREC_F64 = 0
LS_PREC_F32 = 1
LS_F64_NATIVE = 0
LS_F64_DOUBLE_FLOAT = 1
LS_INNER_BASIS_F64 = 0
LS_INNER_BASIS_F32 = 1

# Every symbol declared in include/ls_dafmm.h.
EXPORTED_SYMBOLS = (
    "ls_op_create", "ls_op_destroy", "ls_op_info", "ls_op_points", "ls_op_contrast", "ls_op_rhs", "ls_op_rhs_angles",
    "ls_matvec", "ls_matvec_f32", "ls_op_enable_f32", "ls_matvec_host", "ls_gmres", "ls_gmres_restarted",
    "ls_gmres_mixed", "ls_time_matvec", "ls_op_skeleton_dump", "ls_op_precomputations", "ls_last_error",
    "ls_version", "ls_matvec_noalloc", "ls_op_set_f64_kernels", "ls_gmres_mixed_batched", "ls_op_interpolate",
    "ls_write_result", "ls_set_pdl", "ls_get_pdl", "ls_time_matvec_phases", "ls_measure_fma_peak", "ls_op_set_inner_basis",
    "ls_op_set_batch_width", "ls_matvec_f32_many", "ls_time_block_apply", "ls_op_tc_stages", "ls_measure_mma_issue",
    "ls_tc_wait_probe", "ls_set_near_overlap", "ls_get_near_overlap", "ls_set_precompute_cache",
    "ls_precompute_cache_stats",
)
# Every symbol declared in include/ls_fno.h (learned preconditioner).
FNO_SYMBOLS = (
    "ls_fno_create", "ls_fno_destroy", "ls_fno_num_params", "ls_fno_get_params", "ls_fno_set_params",
    "ls_fno_get_grads", "ls_fno_forward", "ls_fno_loss_grad", "ls_fno_adam_step", "ls_fno_make_batch",
    "ls_op_grid_sample", "ls_op_grid_weights", "ls_op_grid_contrast", "ls_fgmres_nn",
)
LS_NN_GUESS = 1
LS_NN_PRECOND = 2
FNO_IN_CHANNELS = 6
FNO_OUT_CHANNELS = 2
FNO_WIDTH = 32
FNO_KAPPA_SCALE = 40.0


class LSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} (status {code})")
        self.code = code


class _Config(ctypes.Structure):
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
        ("tree_adaptive", ctypes.c_int),
        ("treeAdaptivity", ctypes.c_int),
        ("precompute_on_gpu", ctypes.c_int),
        ("far_on_gpu", ctypes.c_int),
    ]


class _Info(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("n_leaves", ctypes.c_int),
        ("n_levels", ctypes.c_int),
        ("level_LFR", ctypes.c_int),
        ("rank", ctypes.c_int),
        ("far_entries", ctypes.c_longlong),
        ("near_entries", ctypes.c_longlong),
        ("matvec_bytes", ctypes.c_longlong),
        ("matvec_flops", ctypes.c_longlong),
        ("device_bytes", ctypes.c_longlong),
        ("assemble_seconds", ctypes.c_double),
        ("max_rank", ctypes.c_int),
        ("n_kernels_per_matvec", ctypes.c_int),
        ("m2l_entries", ctypes.c_longlong),
        ("m2l_bytes", ctypes.c_longlong),
        ("m2l_flops", ctypes.c_longlong),
        ("assemble_stage_seconds", ctypes.c_double * 6),
    ]


class _FnoConfig(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_int), ("modes", ctypes.c_int), ("layers", ctypes.c_int),
                ("proj_width", ctypes.c_int)]


class _NnReport(ctypes.Structure):
    _fields_ = [("n_matvec", ctypes.c_int), ("n_precond", ctypes.c_int), ("outer", ctypes.c_int),
                ("fell_back", ctypes.c_int), ("guess_residual", ctypes.c_double), ("rel_residual", ctypes.c_double)]


@dataclasses.dataclass
class Config:
    """Problem description (ls_config). Defaults follow GMRES/Readme.md:43."""
    nCones_LFR: int = 16
    nChebNodes: int = 6
    yes2DFMM: int = 1
    TOL_POW: int = 8
    degreeOfBases: int = 6
    nLevelsUniform: int = 4
    Qchoice: int = 0
    findPhi: int = 1
    reference_rounding: int = 1
    L: float = 1.0
    kappa: float = 10.0
    bumps: tuple = ()  # ((cx, cy, a, w), ...) for Qchoice 6
    tree_adaptive: int = 0   # 1: the reference's adaptive quadtree (createAdaptiveTree + 2:1 balance)
    treeAdaptivity: int = 5  # adaptive: boxes split until q is resolved to 10^-treeAdaptivity
    precompute_on_gpu: int = 0  # 1: precomputation quadratures on the operator's GPU (not bit-exact with the host)
    far_on_gpu: int = 0  # 1: far-field sum table on the GPU; 2: and the NCA; 3: and the M2L block fill (uniform trees)

    def to_c(self):
        c = _Config()
        for f in ("nCones_LFR", "nChebNodes", "yes2DFMM", "TOL_POW", "degreeOfBases", "nLevelsUniform",
                  "Qchoice", "findPhi", "reference_rounding", "tree_adaptive", "treeAdaptivity",
                  "precompute_on_gpu", "far_on_gpu"):
            setattr(c, f, int(getattr(self, f)))
        c.L = float(self.L)
        c.kappa = float(self.kappa)
        c.n_bumps = len(self.bumps)
        for k, (bx, by, a, w) in enumerate(self.bumps):
            c.bump_cx[k], c.bump_cy[k], c.bump_a[k], c.bump_w[k] = bx, by, a, w
        return c

    def as_dict(self):
        d = {f.name: getattr(self, f.name) for f in dataclasses.fields(self) if f.name != "bumps"}
        d["n_bumps"] = len(self.bumps)
        d["bump_cx"] = [b[0] for b in self.bumps]
        d["bump_cy"] = [b[1] for b in self.bumps]
        d["bump_a"] = [b[2] for b in self.bumps]
        d["bump_w"] = [b[3] for b in self.bumps]
        return d


def seeded_bumps(seed, n=3):
    """Gaussian bumps q(x) = sum_k a_k exp(-|x-c_k|^2 / w_k^2) with centres
    U[-0.6, 0.6]^2, amplitudes U[0.5, 1.5] and widths U[0.05, 0.2] drawn from
    numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.6, 0.6, size=(n, 2))
    a = rng.uniform(0.5, 1.5, size=n)
    w = rng.uniform(0.05, 0.2, size=n)
    return tuple((float(c[k, 0]), float(c[k, 1]), float(a[k]), float(w[k])) for k in range(n))


_lib = None


def skeleton_nodes(dump):
    """Per-node skeletons of an ls_op_skeleton_dump array: {(level, box,
    cone or -1): (out_active, in_active, out_charge, out_check, in_charge,
    in_check, user_check)} with the lists as tuples of point indices."""
    d = [int(v) for v in dump]
    out, p = {}, 0
    while p < len(d):
        key, flags = (d[p], d[p + 1], d[p + 2]), (d[p + 3], d[p + 4])
        p += 5
        lists = []
        for _ in range(5):
            n = d[p]
            lists.append(tuple(d[p + 1:p + 1 + n]))
            p += 1 + n
        out[key] = flags + tuple(lists)
    return out


def skeleton_agreement(dump_a, dump_b):
    """Fraction of the nodes of dump_b whose skeletons (flags and all five
    lists) are the same in dump_a."""
    a, b = skeleton_nodes(dump_a), skeleton_nodes(dump_b)
    return sum(1 for k, v in b.items() if a.get(k) == v) / max(1, len(b))


def build(verbose=False):
    """Compiles liblsdafmm.so in-tree (nvcc for sm_103a + g++)."""
    from . import _build
    return _build.build(verbose=verbose)


def lib():
    """Loads liblsdafmm.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run lippmann_schwinger_solver_gb300.build() first")
        L = ctypes.CDLL(LIB_PATH)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.ls_op_create.argtypes = [ctypes.POINTER(_Config), ctypes.c_int, ctypes.POINTER(vp)]
        L.ls_op_destroy.argtypes = [vp]
        L.ls_op_info.argtypes = [vp, ctypes.POINTER(_Info)]
        for n in ("ls_op_points", "ls_op_contrast", "ls_op_rhs"):
            getattr(L, n).argtypes = [vp, dp]
        L.ls_op_rhs_angles.argtypes = [vp, dp, ctypes.c_int, dp]
        for n in ("ls_matvec", "ls_matvec_f32", "ls_matvec_noalloc"):
            getattr(L, n).argtypes = [vp, vp, vp, vp]
        L.ls_op_enable_f32.argtypes = [vp]
        L.ls_op_set_f64_kernels.argtypes = [vp, ctypes.c_int]
        L.ls_gmres_mixed_batched.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp,
                                             ip, dp]
        L.ls_matvec_host.argtypes = [vp, dp, dp]
        L.ls_gmres.argtypes = [vp, dp, ctypes.c_int, ctypes.c_double, dp, dp, ip, dp]
        L.ls_gmres_restarted.argtypes = [vp, dp, ctypes.c_int, ctypes.c_int, dp]
        L.ls_gmres_mixed.argtypes = [vp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, dp, ip, dp]
        L.ls_time_matvec.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.ls_op_skeleton_dump.restype = ctypes.c_long
        L.ls_op_skeleton_dump.argtypes = [vp, ip, ctypes.c_long]
        L.ls_op_precomputations.argtypes = [vp, dp, dp]
        L.ls_op_interpolate.argtypes = [vp, ctypes.c_int, dp, dp, dp]
        L.ls_write_result.argtypes = [ctypes.c_char_p, ctypes.c_int, dp]
        L.ls_last_error.restype = ctypes.c_char_p
        L.ls_version.restype = ctypes.c_char_p
        L.ls_set_pdl.argtypes = [ctypes.c_int]
        L.ls_op_set_inner_basis.argtypes = [vp, ctypes.c_int]
        L.ls_op_set_batch_width.argtypes = [vp, ctypes.c_int]
        L.ls_matvec_f32_many.argtypes = [vp, ctypes.c_int, dp, dp]
        L.ls_time_block_apply.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.ls_time_matvec_phases.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.ls_measure_fma_peak.argtypes = [ctypes.c_int, ctypes.c_int, dp]
        L.ls_measure_mma_issue.argtypes = [ctypes.c_int, ctypes.c_int, dp]
        L.ls_op_tc_stages.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.ls_tc_wait_probe.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.POINTER(ctypes.c_int)]
        L.ls_get_pdl.argtypes = []
        L.ls_set_near_overlap.argtypes = [ctypes.c_int]
        L.ls_set_precompute_cache.argtypes = [ctypes.c_char_p]
        L.ls_precompute_cache_stats.argtypes = [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
        L.ls_get_near_overlap.argtypes = []
        fp = ctypes.POINTER(ctypes.c_float)
        L.ls_fno_create.argtypes = [ctypes.POINTER(_FnoConfig), ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(vp)]
        L.ls_fno_destroy.argtypes = [vp]
        L.ls_fno_num_params.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        for n in ("ls_fno_get_params", "ls_fno_set_params", "ls_fno_get_grads"):
            getattr(L, n).argtypes = [vp, fp]
        L.ls_fno_forward.argtypes = [vp, ctypes.c_int, vp, vp, vp]
        L.ls_fno_loss_grad.argtypes = [vp, ctypes.c_int, vp, vp, fp, vp]
        L.ls_fno_adam_step.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, vp]
        L.ls_fno_make_batch.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 9
        L.ls_op_grid_sample.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp]
        L.ls_op_grid_weights.argtypes = [vp, ctypes.c_int, fp, ip]
        L.ls_op_grid_contrast.argtypes = [vp, ctypes.c_int, fp]
        L.ls_fgmres_nn.argtypes = [vp, vp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, dp,
                                   ctypes.POINTER(_NnReport)]
        for n in EXPORTED_SYMBOLS + FNO_SYMBOLS:
            if n not in ("ls_op_skeleton_dump", "ls_last_error", "ls_version"):
                getattr(L, n).restype = ctypes.c_int
        _lib = L
    return _lib


def measure_fma_peak(device=0, kind="fp64"):
    """Measured FMA throughput of the device in TFLOP/s (ls_measure_fma_peak):
    kind "fp64" (DFMA) or "fp32" (FFMA)."""
    v = ctypes.c_double()
    _check(lib().ls_measure_fma_peak(int(device), 0 if kind == "fp64" else 1, ctypes.byref(v)),
           "ls_measure_fma_peak")
    return v.value


def measure_mma_issue(device=0, n=48):
    """SM cycles per TF32 tensor-core MMA (M = 128, N = n, K = 8) issued back to
    back (ls_measure_mma_issue): the floor of the tensor-core block apply."""
    v = ctypes.c_double()
    _check(lib().ls_measure_mma_issue(int(device), int(n), ctypes.byref(v)), "ls_measure_mma_issue")
    return v.value


def tc_wait_probe(device=0, polls=100000):
    """Runs the tensor-core kernels' bounded mbarrier wait on a barrier that
    nothing arrives on (ls_tc_wait_probe); True when the wait gave up and
    recorded it."""
    v = ctypes.c_int()
    _check(lib().ls_tc_wait_probe(int(device), int(polls), ctypes.byref(v)), "ls_tc_wait_probe")
    return bool(v.value)


def set_near_overlap(on):
    """Run the native FP64 matvec's near field beside its far-field chain
    (1, the default) or after it (0) (ls_set_near_overlap); bitwise identical."""
    lib().ls_set_near_overlap(1 if on else 0)


def set_precompute_cache(dir):
    """Cache of the assembly's precomputations (ls_set_precompute_cache):
    None off, "" in memory, a directory path also as binary files there."""
    lib().ls_set_precompute_cache(None if dir is None else os.fsencode(dir))


def precompute_cache_stats():
    """(hits, misses) of the precomputation cache since the process started."""
    h, m = ctypes.c_longlong(), ctypes.c_longlong()
    _check(lib().ls_precompute_cache_stats(ctypes.byref(h), ctypes.byref(m)), "ls_precompute_cache_stats")
    return h.value, m.value


def get_near_overlap():
    return bool(lib().ls_get_near_overlap())


def set_pdl(on):
    """Launch the matvec and Krylov kernel chains with programmatic dependent
    launch (True, the default) or as plain stream-ordered launches
    (ls_set_pdl). Results are bitwise identical either way."""
    _check(lib().ls_set_pdl(1 if on else 0), "ls_set_pdl")


def get_pdl():
    return bool(lib().ls_get_pdl())


def _check(code, what):
    if code != LS_OK:
        raise LSError(code, f"{what}: {lib().ls_last_error().decode()}")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Operator:
    """An assembled DAFMM operator resident on one GPU (ls_op)."""

    def __init__(self, cfg, device=0):
        if isinstance(cfg, dict):
            cfg = Config(**cfg)
        self.cfg = cfg
        self._c = cfg.to_c()
        h = ctypes.c_void_p()
        _check(lib().ls_op_create(ctypes.byref(self._c), int(device), ctypes.byref(h)), "ls_op_create")
        self._h = h
        self.info = self._info()
        self.N = self.info["N"]

    def _info(self):
        i = _Info()
        _check(lib().ls_op_info(self._h, ctypes.byref(i)), "ls_op_info")
        out = {f: getattr(i, f) for f, _ in _Info._fields_}
        out["assemble_stage_seconds"] = list(out["assemble_stage_seconds"])
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().ls_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # geometry / plugin
    def points(self):
        a = np.empty((self.N, 2))
        _check(lib().ls_op_points(self._h, _dp(a)), "ls_op_points")
        return a

    def contrast(self):
        a = np.empty(self.N)
        _check(lib().ls_op_contrast(self._h, _dp(a)), "ls_op_contrast")
        return a

    def rhs(self):
        a = np.empty(self.N, dtype=np.complex128)
        _check(lib().ls_op_rhs(self._h, _dp(a)), "ls_op_rhs")
        return a

    # products
    def matvec(self, x):
        """y = A x for host vectors (copies in, computes on the GPU, copies out)."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if x.shape != (self.N,):
            raise ValueError(f"x must have shape ({self.N},)")
        y = np.empty_like(x)
        _check(lib().ls_matvec_host(self._h, _dp(x), _dp(y)), "ls_matvec_host")
        return y

    def matvec_device(self, x_ptr, y_ptr, stream=0, precision=LS_PREC_F64):
        """y = A x for device pointers (e.g. torch complex128 tensors' data_ptr())."""
        f = lib().ls_matvec if precision == LS_PREC_F64 else lib().ls_matvec_f32
        _check(f(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), ctypes.c_void_p(stream)), "ls_matvec")

    def matvec_device_noalloc(self, x_ptr, y_ptr, stream=0):
        """y = A x for device pointers with the matvec scratch taken from the
        library's static device array (no device allocation per call)."""
        _check(lib().ls_matvec_noalloc(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr),
                                       ctypes.c_void_p(stream)), "ls_matvec_noalloc")

    def enable_f32(self):
        _check(lib().ls_op_enable_f32(self._h), "ls_op_enable_f32")

    def set_batch_width(self, width):
        """Right-hand sides per block of gmres_mixed_batched: 64 (tensor-core
        block apply, the default) or 8 (CUDA-core block kernels)."""
        _check(lib().ls_op_set_batch_width(self._h, int(width)), "ls_op_set_batch_width")

    def matvec_f32_many(self, X):
        """Y = A32 X for the columns of X (N x nrhs), 64 per pass on the
        tensor cores (ls_matvec_f32_many)."""
        X = np.asfortranarray(X, dtype=np.complex128)
        if X.ndim != 2 or X.shape[0] != self.N:
            raise ValueError(f"X must have shape ({self.N}, nrhs)")
        Y = np.empty_like(X, order="F")
        _check(lib().ls_matvec_f32_many(self._h, X.shape[1], _dp(X), _dp(Y)), "ls_matvec_f32_many")
        return Y

    def tc_stages(self):
        """Stages of one 64-wide tensor-core block apply (12 MMAs each); 0
        before the first 64-wide apply builds the tensor-core form."""
        v = ctypes.c_longlong()
        _check(lib().ls_op_tc_stages(self._h, ctypes.byref(v)), "ls_op_tc_stages")
        return v.value

    def time_block_apply(self, width=64, warmup=3, iters=10):
        """Mean ms of one FP32 block apply of `width` resident right-hand sides
        (8: CUDA cores, 64: tensor cores)."""
        ms = ctypes.c_float()
        _check(lib().ls_time_block_apply(self._h, int(width), int(warmup), int(iters), ctypes.byref(ms)),
               "ls_time_block_apply")
        return ms.value

    def set_inner_basis(self, basis):
        """Inner Krylov basis of the mixed-precision solvers: LS_INNER_BASIS_F64
        (default: FP64 Gram-Schmidt and Givens) or LS_INNER_BASIS_F32."""
        _check(lib().ls_op_set_inner_basis(self._h, int(basis)), "ls_op_set_inner_basis")

    def set_f64_kernels(self, kernels):
        """LS_F64_NATIVE or LS_F64_DOUBLE_FLOAT behind every FP64 entry point."""
        _check(lib().ls_op_set_f64_kernels(self._h, int(kernels)), "ls_op_set_f64_kernels")

    def gmres(self, b, max_iter=400, tol=1e-10, raise_on_fail=False):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        hist = np.full(max_iter + 1, np.nan)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        code = lib().ls_gmres(self._h, _dp(b), int(max_iter), float(tol), _dp(x), _dp(hist), ctypes.byref(it),
                              ctypes.byref(rr))
        if code not in (LS_OK, LS_E_NOT_CONVERGED) or (raise_on_fail and code != LS_OK):
            _check(code, "ls_gmres")
        return x, hist[: it.value + 1], it.value, rr.value, code

    def gmres_restarted(self, b, m, restarts):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        _check(lib().ls_gmres_restarted(self._h, _dp(b), int(m), int(restarts), _dp(x)), "ls_gmres_restarted")
        return x

    def gmres_mixed(self, b, max_outer=10, inner_iter=200, tol=1e-8):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        hist = np.full(max_outer + 1, np.nan)
        nmv = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        code = lib().ls_gmres_mixed(self._h, _dp(b), int(max_outer), int(inner_iter), float(tol), _dp(x), _dp(hist),
                                    ctypes.byref(nmv), ctypes.byref(rr))
        if code not in (LS_OK, LS_E_NOT_CONVERGED):
            _check(code, "ls_gmres_mixed")
        return x, hist[~np.isnan(hist)], nmv.value, rr.value, code

    def gmres_mixed_batched(self, B, max_outer=10, inner_iter=100, tol=1e-8):
        """Solves A X = B for the columns of B (N x nrhs) with the batched
        mixed-precision refinement (needs enable_f32()). Returns (X, number of
        FP32 block applies + FP64 residual products, per-column FP64 relative
        residuals, status)."""
        B = np.asfortranarray(B, dtype=np.complex128)
        if B.ndim != 2 or B.shape[0] != self.N:
            raise ValueError("B must be N x nrhs")
        nrhs = B.shape[1]
        X = np.empty_like(B, order="F")
        rr = np.empty(nrhs)
        nmv = ctypes.c_int(0)
        code = lib().ls_gmres_mixed_batched(self._h, int(nrhs), _dp(B), int(max_outer), int(inner_iter), float(tol),
                                            _dp(X), ctypes.byref(nmv), rr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if code not in (LS_OK, LS_E_NOT_CONVERGED):
            _check(code, "ls_gmres_mixed_batched")
        return X, nmv.value, rr, code

    def rhs_angles(self, thetas):
        """Right-hand sides -kappa^2 q exp(i kappa (x cos t + y sin t)) for the
        incidence directions t (GMRES/GMRES.cpp:119-126 for t = 0), N x len(t),
        formed by ls_op_rhs_angles on the host threads."""
        t = np.ascontiguousarray(np.asarray(thetas, dtype=float).ravel())
        B = np.empty((self.N, len(t)), dtype=np.complex128, order="F")
        _check(lib().ls_op_rhs_angles(self._h, _dp(t), len(t), _dp(B)), "ls_op_rhs_angles")
        return B

    def time_matvec(self, warmup=3, iters=20, precision=LS_PREC_F64):
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(lib().ls_time_matvec(self._h, int(precision), int(warmup), int(iters), ctypes.byref(a),
                                    ctypes.byref(b)), "ls_time_matvec")
        return a.value, b.value

    def time_matvec_phases(self, warmup=3, iters=20, precision=LS_PREC_F64):
        """Mean ms per matvec by phase: dict with total, up, m2l, down, near."""
        ms = (ctypes.c_float * 5)()
        _check(lib().ls_time_matvec_phases(self._h, int(precision), int(warmup), int(iters), ms),
               "ls_time_matvec_phases")
        return dict(zip(("total", "up", "m2l", "down", "near"), (float(v) for v in ms)))

    def interpolate(self, xy, phi):
        """The density phi (nodes) at the points xy (n x 2) by the
        reference's Chebyshev-Q+ interpolation (ls_op_interpolate)."""
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        if phi.shape != (self.N,):
            raise ValueError(f"phi must have shape ({self.N},)")
        out = np.empty(len(xy), dtype=np.complex128)
        _check(lib().ls_op_interpolate(self._h, len(xy), _dp(xy), _dp(phi), _dp(out)), "ls_op_interpolate")
        return out

    # grid resampling and the learned preconditioner (include/ls_fno.h)
    def grid_weights(self, grid):
        """Host weight rows [G*G, rank] and leaf [G*G] of the nodes -> grid map."""
        w = np.empty((grid * grid, self.info["rank"]), dtype=np.float32)
        leaf = np.empty(grid * grid, dtype=np.int32)
        _check(lib().ls_op_grid_weights(self._h, int(grid), w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                        leaf.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), "ls_op_grid_weights")
        return w, leaf

    def grid_contrast(self, grid):
        q = np.empty(grid * grid, dtype=np.float32)
        _check(lib().ls_op_grid_contrast(self._h, int(grid), q.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
               "ls_op_grid_contrast")
        return q

    def grid_sample_device(self, grid, nvec, x_ptr, out_ptr, stream=0):
        """out[v][G*G] (complex64) from nvec complex128 vectors at x_ptr (device)."""
        _check(lib().ls_op_grid_sample(self._h, int(grid), int(nvec), ctypes.c_void_p(x_ptr), ctypes.c_void_p(out_ptr),
                                       ctypes.c_void_p(stream)), "ls_op_grid_sample")

    def fgmres_nn(self, net, b, flags=LS_NN_GUESS | LS_NN_PRECOND, max_outer=10, inner_iter=100, tol=1e-8):
        """Mixed-precision flexible GMRES with the network as initial guess
        and right preconditioner (ls_fgmres_nn). Returns (x, FP64 residual
        history, report dict, status)."""
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.empty_like(b)
        hist = np.full(max_outer + 2, np.nan)
        rep = _NnReport()
        code = lib().ls_fgmres_nn(self._h, net._h if net is not None else None, _dp(b), int(flags), int(max_outer),
                                  int(inner_iter), float(tol), _dp(x), _dp(hist), ctypes.byref(rep))
        if code not in (LS_OK, LS_E_NOT_CONVERGED):
            _check(code, "ls_fgmres_nn")
        return x, hist[~np.isnan(hist)], {f: getattr(rep, f) for f, _ in _NnReport._fields_}, code

    # inspection
    def skeleton_dump(self):
        n = lib().ls_op_skeleton_dump(self._h, None, 0)
        a = np.empty(n, dtype=np.int32)
        lib().ls_op_skeleton_dump(self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
        return a

    def precomputations(self):
        r = self.info["rank"]
        M = np.empty((r, 31), dtype=np.complex128)
        B = np.empty((9, r, r), dtype=np.complex128)
        _check(lib().ls_op_precomputations(self._h, _dp(M), _dp(B)), "ls_op_precomputations")
        return M, B


# --------------------------------------------------------------------------
# Reference-shaped interface (GMRES/GMRES.cpp, GMRES_Hybrid/include/gmres.hpp)


@dataclasses.dataclass
class inputsToDFMM:  # noqa: N801 - reference name (GMRES/GMRES.cpp:129-138)
    nCones_LFR: int = 16
    nChebNodes: int = 6
    L: float = 1.0
    yes2DFMM: int = 1
    TOL_POW: int = 8
    degreeOfBases: int = 6
    treeAdaptivity: int = 5
    nLevelsUniform: int = 4
    # 1: the adaptive quadtree GMRES/GMRES.cpp:164-165 builds; 0: the uniform
    # tree (createUniformTree) of the benchmark workloads.
    treeAdaptive: int = 0


class userkernel:  # noqa: N801 - reference name (GMRES/GMRES.cpp:100-127)
    """Contrast / incidence / right-hand side plugin. Qchoice 0..5 are the
    reference contrasts; Qchoice 6 are Gaussian bumps."""

    def __init__(self, kappa, Qchoice=0, bumps=()):
        self.kappa, self.Qchoice, self.bumps = kappa, Qchoice, tuple(bumps)

    def IncidenceFunction(self, xy):
        return np.exp(1j * self.kappa * np.asarray(xy)[..., 0])


class DFMM:
    """Drop-in for the reference's DFMM adapter (GMRES/GMRES.cpp:140-255)."""

    def __init__(self, inputs, kernel, findPhi=True, reference_rounding=True, device=0):
        self.inputs, self.mykernel = inputs, kernel
        self.cfg = Config(nCones_LFR=inputs.nCones_LFR, nChebNodes=inputs.nChebNodes, yes2DFMM=inputs.yes2DFMM,
                          TOL_POW=inputs.TOL_POW, degreeOfBases=inputs.degreeOfBases,
                          nLevelsUniform=inputs.nLevelsUniform, Qchoice=kernel.Qchoice, findPhi=int(findPhi),
                          reference_rounding=int(reference_rounding), L=inputs.L, kappa=kernel.kappa,
                          bumps=kernel.bumps, tree_adaptive=int(inputs.treeAdaptive),
                          treeAdaptivity=int(inputs.treeAdaptivity))
        self.device = device
        self.K = None

    def FMMTreeInitialisation(self):
        self.K = Operator(self.cfg, self.device)
        self.N = self.K.N
        self.gridPoints = self.K.points()

    def MatVecProduct(self, b):
        return self.K.matvec(b)

    def RHS(self):
        return self.K.rhs()


class classGMRES:  # noqa: N801 - reference name
    def gmres(self, M, b, maxIterations, threshold):
        """Returns (x, error, noOfIterations, e) like classGMRES::gmres."""
        x, hist, it, _, _ = M.K.gmres(b, maxIterations, threshold)
        return x, float(hist[-1]), it, list(hist)


def RestartedGMRES(restart, S, m, inputs, b):  # noqa: N802 - reference name
    return S.K.gmres_restarted(b, m, restart)


def write_result(path, v):
    """Writes complex values one per line as "(re,im)" with six significant
    digits, the reference's result-file text (GMRES/GMRES.cpp:391-397)."""
    v = np.ascontiguousarray(v, dtype=np.complex128)
    _check(lib().ls_write_result(os.fsencode(path), len(v), _dp(v)), "ls_write_result")


def scattered_field(cfg, phi, device=0):
    """Scattered and total field from the solved density (GMRES/GMRES.cpp:581-597).

    A second operator with findPhi = 0 (the bare volume potential G, no
    q scaling and no identity) is assembled on the same tree. It gives
    u_scat = G phi and u_tot = u_inc + u_scat, where u_inc = exp(i kappa x1).
    It also returns the residual of the Lippmann-Schwinger identity
    phi / kappa^2 + q u_tot = 0, the check that
    GMRES_Hybrid/LippmannSchwinger/main/hybridTrueValidation_gmres.cpp:227-232
    prints, as an absolute 2-norm.
    """
    if isinstance(cfg, dict):
        cfg = Config(**cfg)
    g = Config(**{**dataclasses.asdict(cfg), "findPhi": 0})
    with Operator(g, device) as op2:
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        u_scat = op2.matvec(phi)
        pts = op2.points()
        q = op2.contrast()
    u_inc = np.exp(1j * cfg.kappa * pts[:, 0])
    u_tot = u_inc + u_scat
    err = np.linalg.norm(phi / cfg.kappa ** 2 + q * u_tot)
    return u_scat, u_tot, float(err)


# ---------------------------------------------------------------- learned preconditioner

def fno_layout(grid=128, modes=24, layers=4, proj_width=128):
    """Offsets of the parameter groups in the flat FP32 vector (include/ls_fno.h)."""
    W, o, lay = FNO_WIDTH, 0, {}

    def take(name, n):
        nonlocal o
        lay[name] = (o, n)
        o += n
    take("lift_w", W * FNO_IN_CHANNELS)
    take("lift_b", W)
    for l in range(layers):
        take(f"spec{l}", 2 * (2 * modes) * modes * W * W)
        take(f"pw_w{l}", W * W)
        take(f"pw_b{l}", W)
    take("p1_w", proj_width * W)
    take("p1_b", proj_width)
    take("p2_w", FNO_OUT_CHANNELS * proj_width)
    take("p2_b", FNO_OUT_CHANNELS)
    lay["total"] = o
    return lay


_FNO_MAGIC = b"LSFNO001"


class FNO:
    """Spectral neural operator on one GPU (ls_fno): hand-written CUDA
    forward, backward and Adam. Device buffers are passed as integer
    addresses (e.g. torch tensors' data_ptr())."""

    def __init__(self, grid=128, modes=24, layers=4, proj_width=128, device=0, seed=0):
        self.shape = dict(grid=grid, modes=modes, layers=layers, proj_width=proj_width)
        c = _FnoConfig(grid, modes, layers, proj_width)
        h = ctypes.c_void_p()
        _check(lib().ls_fno_create(ctypes.byref(c), int(device), int(seed), ctypes.byref(h)), "ls_fno_create")
        self._h = h
        n = ctypes.c_longlong()
        _check(lib().ls_fno_num_params(self._h, ctypes.byref(n)), "ls_fno_num_params")
        self.n_params = n.value
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            lib().ls_fno_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _fp(self, a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def get_params(self):
        p = np.empty(self.n_params, dtype=np.float32)
        _check(lib().ls_fno_get_params(self._h, self._fp(p)), "ls_fno_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (self.n_params,):
            raise ValueError(f"expected {self.n_params} parameters")
        _check(lib().ls_fno_set_params(self._h, self._fp(p)), "ls_fno_set_params")

    def get_grads(self):
        g = np.empty(self.n_params, dtype=np.float32)
        _check(lib().ls_fno_get_grads(self._h, self._fp(g)), "ls_fno_get_grads")
        return g

    def forward_device(self, batch, in_ptr, out_ptr, stream=0):
        _check(lib().ls_fno_forward(self._h, int(batch), ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr),
                                    ctypes.c_void_p(stream)), "ls_fno_forward")

    def loss_grad_device(self, batch, in_ptr, target_ptr, want_loss=True, stream=0):
        loss = ctypes.c_float(float("nan"))
        _check(lib().ls_fno_loss_grad(self._h, int(batch), ctypes.c_void_p(in_ptr), ctypes.c_void_p(target_ptr),
                                      ctypes.byref(loss) if want_loss else None, ctypes.c_void_p(stream)),
               "ls_fno_loss_grad")
        return loss.value if want_loss else None

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=0):
        _check(lib().ls_fno_adam_step(self._h, float(lr), float(beta1), float(beta2), float(eps),
                                      ctypes.c_void_p(stream)), "ls_fno_adam_step")

    def make_batch_device(self, batch, n_basis, n_scatterers, F, PHI, Q, kappa, scatterer, coef, inp, target,
                          stream=0):
        args = [ctypes.c_void_p(a) for a in (F, PHI, Q, kappa, scatterer, coef, inp, target, stream)]
        _check(lib().ls_fno_make_batch(self._h, int(batch), int(n_basis), int(n_scatterers), *args),
               "ls_fno_make_batch")

    def save(self, path, half=True):
        """Weights file: magic, 5 int32 (grid, modes, layers, proj_width,
        dtype 0 = float32 / 1 = float16), then the flat parameters."""
        p = self.get_params()
        hdr = np.array([self.shape["grid"], self.shape["modes"], self.shape["layers"], self.shape["proj_width"],
                        1 if half else 0], dtype="<i4")
        with open(path, "wb") as f:
            f.write(_FNO_MAGIC)
            f.write(hdr.tobytes())
            f.write(p.astype("<f2" if half else "<f4").tobytes())

    @classmethod
    def load(cls, path, device=0):
        with open(path, "rb") as f:
            if f.read(8) != _FNO_MAGIC:
                raise ValueError(f"{path}: not a network weights file")
            g, m, l, pw, dt = np.frombuffer(f.read(20), dtype="<i4")
            p = np.frombuffer(f.read(), dtype="<f2" if dt == 1 else "<f4").astype(np.float32)
        net = cls(grid=int(g), modes=int(m), layers=int(l), proj_width=int(pw), device=device)
        net.set_params(p)
        return net
