"""GB300-native multiwavelet apply engine: Python mirror of the mrcpp:: call surface.

The compute path is libmwgb300.so (CUDA sm_103a kernels + host C++ driver),
loaded from the package's _lib/ directory through its C ABI
(include/mw_gb300.h).  There is no host fallback: if the library is missing or
no CUDA device is usable, the calls raise.

Names and argument meaning follow the MRCPP calls MRChem makes on this path:
    mrcpp::MultiResolutionAnalysis<3>      src/mrenv.cpp:105-122
    mrcpp::PoissonOperator(MRA, prec)       src/driver.cpp:1131,1283
    mrcpp::HelmholtzOperator(MRA, mu, prec) src/scf_solver/HelmholtzVector.cpp:144
    mrcpp::apply(prec, out, oper, inp[, precTrees], maxIter, absPrec)
                                            src/qmoperators/two_electron/CoulombPotential.cpp:131
    mrcpp::multiply / square / add          src/qmoperators/QMPotential.cpp:147,
                                            src/qmfunctions/density_utils.cpp:73,86
    mrcpp::build_grid / copy_grid / copy_func / clear
                                            src/qmfunctions/density_utils.cpp:72,85,87
"""
import ctypes as C
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmwgb300.so")

MW_OK = 0
MW_ERR_ARG, MW_ERR_OOM, MW_ERR_CUDA, MW_ERR_TIMEOUT, MW_ERR_STATE = 1, 2, 3, 4, 5
PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_NEARFP64 = 2
PREC_MIXED_FP32 = 3
PREC_DF = 4
_PREC = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "mixed-near64": PREC_MIXED_NEARFP64,
         "mixed-fp32": PREC_MIXED_FP32, "df": PREC_DF}


class MWError(RuntimeError):
    """Raised when an engine call returns a non-zero status."""

    def __init__(self, code, msg):
        super().__init__("mw error %d: %s" % (code, msg))
        self.code = code


class GTerm(C.Structure):
    _fields_ = [("coef", C.c_double), ("alpha", C.c_double), ("pos", C.c_double * 3),
                ("pw", C.c_int * 3), ("pad", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("out_nodes", C.c_longlong), ("items", C.c_longlong), ("items_fp64", C.c_longlong),
                ("items_fp32", C.c_longlong), ("items_tf32", C.c_longlong), ("generated", C.c_longlong),
                ("levels", C.c_longlong), ("launches", C.c_longlong), ("flops", C.c_double),
                ("flops_issued", C.c_double), ("bytes", C.c_double), ("kernel_ms", C.c_double),
                ("host_ms", C.c_double), ("flops_fp64", C.c_double), ("flops_fp32", C.c_double),
                ("kernel_ms_fp64", C.c_double), ("kernel_ms_fp32", C.c_double), ("host_enum_ms", C.c_double),
                ("host_items_ms", C.c_double), ("host_wait_ms", C.c_double), ("flops_tf32", C.c_double),
                ("kernel_ms_tf32", C.c_double), ("items_df", C.c_longlong), ("flops_df", C.c_double),
                ("kernel_ms_df", C.c_double), ("host_gen_ms", C.c_double), ("host_launch_ms", C.c_double),
                ("host_refine_ms", C.c_double), ("gpu_levels_ms", C.c_double), ("gpu_post_ms", C.c_double),
                ("screen_regrows", C.c_longlong), ("rows_fp64", C.c_longlong), ("rows_fp32", C.c_longlong),
                ("rows_tf32", C.c_longlong), ("rows_df", C.c_longlong), ("host_io_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

EXPORTS = [
    "mw_ctx_create", "mw_ctx_destroy", "mw_last_error", "mw_ctx_basis", "mw_ctx_last_stats", "mw_ctx_synchronize",
    "mw_tree_create", "mw_tree_destroy", "mw_tree_nnodes", "mw_tree_nleaves", "mw_tree_depth", "mw_tree_upload",
    "mw_tree_download", "mw_tree_squared_norm", "mw_tree_integrate", "mw_tree_rescale", "mw_tree_eval",
    "mw_tree_clear", "mw_project_gauss", "mw_project_hydrogen", "mw_copy_grid", "mw_build_grid", "mw_copy_func",
    "mw_crop", "mw_dot", "mw_op_create_poisson", "mw_op_create_helmholtz", "mw_op_destroy", "mw_op_nterms",
    "mw_op_terms", "mw_op_band", "mw_op_block", "mw_apply", "mw_apply_batch", "mw_apply_fixed", "mw_apply_adjoint", "mw_multiply_adjoint", "mw_apply_batch_host",
    "mw_multiply", "mw_multiply_batch", "mw_square", "mw_add", "mw_probe_fma_peak", "mw_density", "mw_rotate",
    "mw_tree_save", "mw_tree_load", "mw_probe_mma_peak", "mw_dot_noalloc", "mw_ctx_set_overlap", "mw_ctx_set_groups", "mw_ctx_set_screening", "mw_apply_batch_autotune", "mw_op_create_helmholtz_batch",
    "mw_tree_upload_batch", "mw_tree_download_batch", "mw_pin_host", "mw_unpin_host",
]


def load_library(path=None):
    """Loads libmwgb300.so (build it first with mrchem_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libmwgb300.so not built: run `python -m mrchem_gb300.build` (or __graft_entry__.build())")
    L = C.CDLL(path)
    P, I, D = C.c_void_p, C.c_int, C.c_double
    ip, dp, pp = C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_void_p)
    sig = {
        "mw_ctx_create": [I, I, ip, ip, I, I, I, pp],
        "mw_ctx_destroy": [P],
        "mw_ctx_basis": [P, dp, dp, dp, dp, dp],
        "mw_ctx_last_stats": [P, C.POINTER(Stats)],
        "mw_ctx_synchronize": [P],
        "mw_ctx_set_overlap": [P, I],
        "mw_ctx_set_groups": [P, I],
        "mw_ctx_set_screening": [P, I],
        "mw_tree_create": [P, pp],
        "mw_tree_destroy": [P],
        "mw_tree_nnodes": [P, ip],
        "mw_tree_nleaves": [P, ip],
        "mw_tree_depth": [P, ip],
        "mw_tree_upload": [P, I, ip, dp],
        "mw_tree_download": [P, ip, dp, C.POINTER(C.c_ubyte)],
        "mw_tree_upload_batch": [I, pp, ip, pp, pp],
        "mw_pin_host": [P, P, C.c_size_t],
        "mw_unpin_host": [P, P],
        "mw_tree_download_batch": [I, pp, pp, pp, pp],
        "mw_tree_squared_norm": [P, dp],
        "mw_tree_integrate": [P, dp],
        "mw_tree_rescale": [P, D],
        "mw_tree_eval": [P, I, dp, dp],
        "mw_tree_clear": [P],
        "mw_project_gauss": [D, P, I, C.POINTER(GTerm), I],
        "mw_project_hydrogen": [D, P, I, I, I, D, dp, I],
        "mw_copy_grid": [P, P],
        "mw_build_grid": [P, I, pp],
        "mw_copy_func": [P, P],
        "mw_crop": [P, D, I],
        "mw_dot": [P, P, dp],
        "mw_dot_noalloc": [P, P, dp],
        "mw_op_create_poisson": [P, D, pp],
        "mw_op_create_helmholtz": [P, D, D, pp],
        "mw_op_destroy": [P],
        "mw_op_nterms": [P, ip],
        "mw_op_terms": [P, dp, dp],
        "mw_op_band": [P, I, I, ip],
        "mw_op_block": [P, I, I, I, dp, dp],
        "mw_apply": [D, P, P, P, I, pp, I, I, I],
        "mw_apply_batch": [I, dp, pp, pp, pp, ip, pp, I, I, I],
        "mw_op_create_helmholtz_batch": [P, I, dp, D, pp],
        "mw_apply_batch_autotune": [I, dp, pp, pp, pp, I, I, I, ip, C.POINTER(C.c_longlong), dp],
        "mw_multiply_batch": [I, dp, pp, dp, pp, pp, I, I, I],
        "mw_apply_fixed": [D, P, P, P, I, I],
        "mw_apply_adjoint": [D, P, P, P, P, I],
        "mw_multiply_adjoint": [D, P, D, P, P, P],
        "mw_apply_batch_host": [I, P, P, P, P, P, P, P, I, I, I, P, P, P, P, P],
        "mw_multiply": [D, P, D, P, P, I, I, I],
        "mw_square": [D, P, P, I, I],
        "mw_add": [D, P, I, dp, pp, I],
        "mw_probe_fma_peak": [P, I, dp],
        "mw_probe_mma_peak": [P, I, dp],
        "mw_density": [D, P, I, pp, dp, I],
        "mw_rotate": [I, pp, I, pp, dp],
        "mw_tree_save": [P, C.c_char_p],
        "mw_tree_load": [P, C.c_char_p],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.mw_last_error.argtypes = [P]
    L.mw_last_error.restype = C.c_char_p
    _lib = L
    return L


def _check(rc, ctx=None):
    if rc != MW_OK:
        msg = _lib.mw_last_error(ctx).decode() if _lib is not None else ""
        raise MWError(rc, msg)


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class MultiResolutionAnalysis:
    """World box [corner, corner + boxes] * 2^-root_scale with a scaling basis of the given order.

    Mirrors mrcpp::MultiResolutionAnalysis<3>(BoundingBox<3>(root_scale, corner, boxes), Basis(order), max_depth)
    (src/mrenv.cpp:105-122); the reference test fixture is order 5 interpolating on [-32,32]^3
    (tests/unit_tests.cpp:66-84).
    """

    def __init__(self, order, root_scale=-5, corner=(-1, -1, -1), boxes=(2, 2, 2), basis="interpolating",
                 max_depth=25, device=0):
        L = load_library()
        self.order, self.K = order, order + 1
        self.root_scale, self.corner, self.boxes = root_scale, tuple(corner), tuple(boxes)
        self.basis, self.max_depth = basis, max_depth
        c = np.ascontiguousarray(corner, dtype=np.int32)
        b = np.ascontiguousarray(boxes, dtype=np.int32)
        h = C.c_void_p()
        _check(L.mw_ctx_create(device, root_scale, _ip(c), _ip(b), order, 1 if basis == "interpolating" else 0,
                               max_depth, C.byref(h)))
        self.ptr = h.value
        self._owned = weakref.WeakSet()  # trees and operators, released before the context

    def close(self):
        if getattr(self, "ptr", None):
            for obj in list(self._owned):
                obj.close()
            _lib.mw_ctx_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def basis_data(self):
        K = self.K
        qx, qw, W = np.zeros(K), np.zeros(K), np.zeros((2 * K, 2 * K))
        c2v, v2c = np.zeros((K, K)), np.zeros((K, K))
        _check(_lib.mw_ctx_basis(self.ptr, _dp(qx), _dp(qw), _dp(W), _dp(c2v), _dp(v2c)), self.ptr)
        return dict(qx=qx, qw=qw, W=W, c2v=c2v, v2c=v2c)

    def last_stats(self):
        st = Stats()
        _check(_lib.mw_ctx_last_stats(self.ptr, C.byref(st)), self.ptr)
        return st.as_dict()

    def synchronize(self):
        _check(_lib.mw_ctx_synchronize(self.ptr), self.ptr)

    def set_overlap(self, on=True):
        """Pipelined job groups in batched applies (default on); off gives exclusive kernel times."""
        _check(_lib.mw_ctx_set_overlap(self.ptr, int(bool(on))), self.ptr)

    def set_groups(self, n):
        """Number of pipelined job groups (1..8) that batched applies split into (default 4)."""
        _check(_lib.mw_ctx_set_groups(self.ptr, int(n)), self.ptr)

    def set_screening(self, where="gpu"):
        """Where applies enumerate, screen and list their items: "gpu" (the default) or "host"
        (OpenMP).  Both give the same items in the same order (bit-identical results)."""
        if where not in ("host", "gpu"):
            raise ValueError("screening must be 'host' or 'gpu'")
        _check(_lib.mw_ctx_set_screening(self.ptr, 1 if where == "gpu" else 0), self.ptr)

    def probe_fma_peak(self, fp64=True):
        """Measured FMA throughput of this GPU in TFLOP/s (FP64 or FP32 CUDA cores)."""
        v = C.c_double()
        _check(_lib.mw_probe_fma_peak(self.ptr, int(fp64), C.byref(v)), self.ptr)
        return v.value

    def probe_mma_peak(self, kind="tf32"):
        """Measured dense tensor-core throughput in TFLOP/s: "tf32" / "bf16" = warp-level mma.sync
        (m16n8k8 / m16n8k16), "tc05" = tcgen05.mma TF32 M128 N256 K8 (the dense TF32 rate),
        "tc05_n32" = tcgen05.mma TF32 M128 N32 K8 (the TF32 apply tier's shape)."""
        v = C.c_double()
        code = {"tf32": 0, "bf16": 1, "tc05": 2, "tc05_n32": 3}[kind]
        _check(_lib.mw_probe_mma_peak(self.ptr, code, C.byref(v)), self.ptr)
        return v.value


class FunctionTree:
    """Device-resident adaptive function tree (mrcpp::FunctionTree<3>)."""

    def __init__(self, mra):
        self.mra = mra
        h = C.c_void_p()
        _check(_lib.mw_tree_create(mra.ptr, C.byref(h)), mra.ptr)
        self.ptr = h.value
        mra._owned.add(self)

    def close(self):
        if getattr(self, "ptr", None):
            _lib.mw_tree_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _int(self, fn):
        v = C.c_int()
        _check(fn(self.ptr, C.byref(v)), self.mra.ptr)
        return v.value

    @property
    def nnodes(self):
        return self._int(_lib.mw_tree_nnodes)

    def getNNodes(self):
        return self.nnodes

    @property
    def nleaves(self):
        return self._int(_lib.mw_tree_nleaves)

    @property
    def depth(self):
        return self._int(_lib.mw_tree_depth)

    def squared_norm(self):
        v = C.c_double()
        _check(_lib.mw_tree_squared_norm(self.ptr, C.byref(v)), self.mra.ptr)
        return v.value

    def norm(self):
        return float(np.sqrt(self.squared_norm()))

    def integrate(self):
        v = C.c_double()
        _check(_lib.mw_tree_integrate(self.ptr, C.byref(v)), self.mra.ptr)
        return v.value

    def rescale(self, c):
        _check(_lib.mw_tree_rescale(self.ptr, float(c)), self.mra.ptr)

    def evalf(self, points):
        pts = np.ascontiguousarray(np.atleast_2d(points), dtype=np.float64)
        out = np.zeros(pts.shape[0])
        _check(_lib.mw_tree_eval(self.ptr, pts.shape[0], _dp(pts), _dp(out)), self.mra.ptr)
        return out

    def clear(self):
        _check(_lib.mw_tree_clear(self.ptr), self.mra.ptr)

    def crop(self, prec, abs_prec=False):
        _check(_lib.mw_crop(self.ptr, prec, int(abs_prec)), self.mra.ptr)

    def download(self, out=None):
        """(keys[n,4] int32, coefs[n, 8K^3] float64, is_leaf[n] uint8) in canonical order.

        out: optional (keys, coefs, is_leaf) arrays of exactly these shapes and types to fill
        instead of new ones (saves allocating and first-touching tens of MB per tree).
        """
        n = self.nnodes
        shapes = ((n, 4), (n, 8 * self.mra.K ** 3), (n,))
        dtypes = (np.int32, np.float64, np.uint8)
        if out is not None and all(a.shape == s and a.dtype == d and a.flags.c_contiguous
                                   for a, s, d in zip(out, shapes, dtypes)):
            keys, coefs, leaf = out
        else:
            keys, coefs, leaf = (np.empty(s, dtype=d) for s, d in zip(shapes, dtypes))
        _check(_lib.mw_tree_download(self.ptr, _ip(keys), _dp(coefs), leaf.ctypes.data_as(C.POINTER(C.c_ubyte))),
               self.mra.ptr)
        return keys, coefs, leaf

    def upload(self, keys, coefs):
        keys = np.ascontiguousarray(keys, dtype=np.int32)
        coefs = np.ascontiguousarray(coefs, dtype=np.float64)
        _check(_lib.mw_tree_upload(self.ptr, keys.shape[0], _ip(keys), _dp(coefs)), self.mra.ptr)
        return self


def pin_host(mra, arr):
    """Page-locks a NumPy array for the GPU (mw_pin_host); batched transfers then copy it directly."""
    _check(_lib.mw_pin_host(mra.ptr, arr.ctypes.data, arr.nbytes), mra.ptr)
    return arr


def unpin_host(mra, arr):
    _check(_lib.mw_unpin_host(mra.ptr, arr.ctypes.data), mra.ptr)


def upload_batch(trees, inputs):
    """tree.upload(keys, coefs) for every (tree, (keys, coefs, ...)) pair with one synchronisation."""
    n = len(trees)
    ks = [np.ascontiguousarray(x[0], dtype=np.int32) for x in inputs]
    cs = [np.ascontiguousarray(x[1], dtype=np.float64) for x in inputs]
    nn = np.ascontiguousarray([k.shape[0] for k in ks], dtype=np.int32)
    kp = (C.c_void_p * n)(*[k.ctypes.data for k in ks])
    cp = (C.c_void_p * n)(*[c.ctypes.data for c in cs])
    _check(_lib.mw_tree_upload_batch(n, _ptrs(trees), _ip(nn), kp, cp), trees[0].mra.ptr)
    return trees


def download_batch(trees, outs=None):
    """[tree.download() for tree in trees] with one synchronisation; outs as in download(out=)."""
    n = len(trees)
    res = []
    for i, t in enumerate(trees):
        m = t.nnodes
        shapes = ((m, 4), (m, 8 * t.mra.K ** 3), (m,))
        dtypes = (np.int32, np.float64, np.uint8)
        o = outs[i] if outs is not None else None
        if o is not None and all(a.shape == s and a.dtype == d and a.flags.c_contiguous
                                 for a, s, d in zip(o, shapes, dtypes)):
            res.append(tuple(o))
        else:
            res.append(tuple(np.empty(s, dtype=d) for s, d in zip(shapes, dtypes)))
    kp = (C.c_void_p * n)(*[r[0].ctypes.data for r in res])
    cp = (C.c_void_p * n)(*[r[1].ctypes.data for r in res])
    lp = (C.c_void_p * n)(*[r[2].ctypes.data for r in res])
    _check(_lib.mw_tree_download_batch(n, _ptrs(trees), kp, cp, lp), trees[0].mra.ptr)
    return res


def _gterms(terms):
    arr = (GTerm * len(terms))()
    for i, (c, a, pos, pw) in enumerate(terms):
        arr[i].coef, arr[i].alpha = c, a
        for d in range(3):
            arr[i].pos[d] = pos[d]
            arr[i].pw[d] = pw[d]
    return arr


def project(prec, tree, terms, abs_prec=False):
    """mrcpp::project of a Gaussian expansion: terms = [(coef, alpha, (X,Y,Z), (px,py,pz)), ...]."""
    arr = _gterms(terms)
    _check(_lib.mw_project_gauss(prec, tree.ptr, len(terms), arr, int(abs_prec)), tree.mra.ptr)
    return tree


def project_hydrogen(prec, tree, n, l, m, Z=1.0, origin=(0.0, 0.0, 0.0), abs_prec=False):
    """Projects the hydrogen-like orbital (n, l, m) of src/analyticfunctions/HydrogenFunction.cpp."""
    o = np.ascontiguousarray(origin, dtype=np.float64)
    _check(_lib.mw_project_hydrogen(prec, tree.ptr, n, l, m, Z, _dp(o), int(abs_prec)), tree.mra.ptr)
    return tree


class ConvolutionOperator:
    def __init__(self, mra, ptr):
        self.mra, self.ptr = mra, ptr
        mra._owned.add(self)

    def close(self):
        if getattr(self, "ptr", None):
            _lib.mw_op_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nterms(self):
        v = C.c_int()
        _check(_lib.mw_op_nterms(self.ptr, C.byref(v)), self.mra.ptr)
        return v.value

    def terms(self):
        T = self.nterms
        c, a = np.zeros(T), np.zeros(T)
        _check(_lib.mw_op_terms(self.ptr, _dp(c), _dp(a)), self.mra.ptr)
        return c, a

    def band(self, term, scale):
        v = C.c_int()
        _check(_lib.mw_op_band(self.ptr, term, scale, C.byref(v)), self.mra.ptr)
        return v.value

    def block(self, term, scale, l):
        K = self.mra.K
        b, nr = np.zeros((2 * K, 2 * K)), np.zeros(4)
        _check(_lib.mw_op_block(self.ptr, term, scale, l, _dp(b), _dp(nr)), self.mra.ptr)
        return b, nr


class PoissonOperator(ConvolutionOperator):
    """Separated Gaussian-sum expansion of 1/r (mrcpp::PoissonOperator(MRA, prec))."""

    def __init__(self, mra, prec):
        h = C.c_void_p()
        _check(_lib.mw_op_create_poisson(mra.ptr, prec, C.byref(h)), mra.ptr)
        super().__init__(mra, h.value)


class HelmholtzOperator(ConvolutionOperator):
    """Separated Gaussian-sum expansion of exp(-mu r)/r (mrcpp::HelmholtzOperator(MRA, mu, prec))."""

    def __init__(self, mra, mu, prec, _handle=None):
        if _handle is None:
            h = C.c_void_p()
            _check(_lib.mw_op_create_helmholtz(mra.ptr, mu, prec, C.byref(h)), mra.ptr)
            _handle = h.value
        self.mu = mu
        super().__init__(mra, _handle)

    @classmethod
    def batch(cls, mra, mus, prec):
        """One operator per mu, built together (shared GPU launches for their NS blocks)."""
        mus = np.ascontiguousarray(mus, dtype=np.float64)
        hs = (C.c_void_p * len(mus))()
        _check(_lib.mw_op_create_helmholtz_batch(mra.ptr, len(mus), _dp(mus), float(prec), hs), mra.ptr)
        return [cls(mra, float(m), prec, _handle=h) for m, h in zip(mus, hs)]


def _ptrs(trees):
    return (C.c_void_p * max(1, len(trees)))(*[t.ptr for t in trees])


def apply(prec, out, oper, inp, prec_trees=(), max_iter=-1, abs_prec=False, precision="fp64"):
    """mrcpp::apply(prec, out, oper, inp[, precTrees], maxIter, absPrec); returns the call's statistics."""
    _check(_lib.mw_apply(prec, out.ptr, oper.ptr, inp.ptr, len(prec_trees), _ptrs(prec_trees), max_iter,
                         int(abs_prec), _PREC[precision]), out.mra.ptr)
    return out.mra.last_stats()


def apply_batch(precs, outs, opers, inps, prec_trees=None, max_iter=-1, abs_prec=False, precision="fp64"):
    """Independent applies (own operator, input, output) run level-synchronously in shared launches.

    prec_trees: optional list (one entry per job) of lists of precision-steering trees.
    """
    n = len(outs)
    p = np.ascontiguousarray(precs if np.ndim(precs) else [precs] * n, dtype=np.float64)
    if prec_trees is None:
        npr, flat = None, []
    else:
        npr = np.ascontiguousarray([len(pt) for pt in prec_trees], dtype=np.int32)
        flat = [t for pt in prec_trees for t in pt]
    _check(_lib.mw_apply_batch(n, _dp(p), _ptrs(outs), _ptrs(opers), _ptrs(inps),
                               _ip(npr) if npr is not None else None, _ptrs(flat), max_iter, int(abs_prec),
                               _PREC[precision]), outs[0].mra.ptr)
    return outs[0].mra.last_stats()


def autotune_batch(precs, outs, opers, inps, abs_prec=False, precision="mixed", repeats=3):
    """Pick the batched apply's launch settings for this batch shape by timing it (job groups 2..6,
    then the chunk size of each reduced tier); later apply_batch calls with the same order, batch
    size and precision use them.  Leaves the batch's result in outs.  Returns the settings."""
    n = len(outs)
    p = np.ascontiguousarray(precs if np.ndim(precs) else [precs] * n, dtype=np.float64)
    g = np.zeros(1, dtype=np.int32)
    ch = (C.c_longlong * 4)()
    ms = np.zeros(1, dtype=np.float64)
    _check(_lib.mw_apply_batch_autotune(n, _dp(p), _ptrs(outs), _ptrs(opers), _ptrs(inps), int(abs_prec),
                                        _PREC[precision], int(repeats), _ip(g), ch, _dp(ms)), outs[0].mra.ptr)
    return {"groups": int(g[0]), "chunk": {"fp64": ch[0], "fp32": ch[1], "tf32": ch[2], "df32": ch[3]},
            "ms": float(ms[0])}


def apply_batch_host(precs, outs, opers, inps, inputs, max_iter=-1, abs_prec=False, precision="fp64", outputs=None):
    """upload_batch(inps, inputs), apply_batch(...) and, with `outputs`, download_batch(outs) as one
    call (mw_apply_batch_host): each job group's inputs go up on its own stream and the group
    starts once they have landed; its outputs go down as soon as its post-processing is queued.
    inputs: (keys, coefs, ...) per job, coefs pinned with pin_host for the overlap.  outputs: per
    job (keys, coefs, leaf) arrays as download_batch returns them (coefs pinned), filled in place
    where the output fits; the returned stats hold "outputs_filled" (one bool per job)."""
    n = len(outs)
    p = np.ascontiguousarray(precs if np.ndim(precs) else [precs] * n, dtype=np.float64)
    ks = [np.ascontiguousarray(x[0], dtype=np.int32) for x in inputs]
    cs = [np.ascontiguousarray(x[1], dtype=np.float64) for x in inputs]
    nn = np.ascontiguousarray([k.shape[0] for k in ks], dtype=np.int32)
    kp = (C.c_void_p * n)(*[k.ctypes.data for k in ks])
    cp = (C.c_void_p * n)(*[c.ctypes.data for c in cs])
    ocap = okp = ocp = olp = onn = None
    if outputs is not None:
        bs = 8 * outs[0].mra.K ** 3
        for k, c, l in outputs:
            if not (k.dtype == np.int32 and c.dtype == np.float64 and l.dtype == np.uint8 and k.flags.c_contiguous
                    and c.flags.c_contiguous and l.flags.c_contiguous and k.ndim == 2 and k.shape[1] == 4
                    and c.ndim == 2 and c.shape[1] == bs and l.ndim == 1):
                raise ValueError("outputs: (n, 4) int32 keys, (n, 8K^3) float64 coefs and (n,) uint8 leaf "
                                 "arrays, C-contiguous")
        ocap = np.ascontiguousarray([min(k.shape[0], c.shape[0], l.shape[0]) for k, c, l in outputs], dtype=np.int32)
        okp = (C.c_void_p * n)(*[o[0].ctypes.data for o in outputs])
        ocp = (C.c_void_p * n)(*[o[1].ctypes.data for o in outputs])
        olp = (C.c_void_p * n)(*[o[2].ctypes.data for o in outputs])
        onn = np.zeros(n, dtype=np.int32)
    _check(_lib.mw_apply_batch_host(n, _dp(p), _ptrs(outs), _ptrs(opers), _ptrs(inps), _ip(nn), kp, cp, max_iter,
                                    int(abs_prec), _PREC[precision], _ip(ocap) if ocap is not None else None, okp,
                                    ocp, olp, _ip(onn) if onn is not None else None), outs[0].mra.ptr)
    st = outs[0].mra.last_stats()
    if onn is not None:
        st["outputs_filled"] = [bool(v > 0) for v in onn]
    return st


def multiply_batch(precs, outs, coefs, as_, bs_, max_iter=-1, abs_prec=False, use_max_norms=False):
    """Independent products out_i = coef_i a_i b_i, refined level-synchronously in shared launches."""
    n = len(outs)
    p = np.ascontiguousarray(precs if np.ndim(precs) else [precs] * n, dtype=np.float64)
    c = np.ascontiguousarray(coefs if np.ndim(coefs) else [coefs] * n, dtype=np.float64)
    _check(_lib.mw_multiply_batch(n, _dp(p), _ptrs(outs), _dp(c), _ptrs(as_), _ptrs(bs_), max_iter, int(abs_prec),
                                  int(use_max_norms)), outs[0].mra.ptr)
    return outs[0].mra.last_stats()


def apply_fixed(prec, out, oper, inp, abs_prec=False, precision="fp64"):
    """apply on out's current grid (no refinement)."""
    _check(_lib.mw_apply_fixed(prec, out.ptr, oper.ptr, inp.ptr, int(abs_prec), _PREC[precision]), out.mra.ptr)
    return out.mra.last_stats()


def apply_adjoint(prec, out, oper, x, seed):
    """L2-adjoint of the fixed-grid FP64 apply on seed's grid (absolute precision): out <- A^T seed on x's grid."""
    _check(_lib.mw_apply_adjoint(prec, out.ptr, oper.ptr, x.ptr, seed.ptr, 1), out.mra.ptr)
    return out.mra.last_stats()


def multiply_adjoint(prec, out, coef, a, b, seed):
    """L2-adjoint of the fixed-grid product h = coef a b in a: out <- coef P_a(seed b) on a's grid
    (seed on h's grid), so that <seed, coef a b> = <out, a>."""
    _check(_lib.mw_multiply_adjoint(prec, out.ptr, coef, a.ptr, b.ptr, seed.ptr), out.mra.ptr)
    return out.mra.last_stats()


def multiply(prec, out, coef, a, b, max_iter=-1, abs_prec=False, use_max_norms=False):
    """mrcpp::multiply(prec, out, coef, a, b, maxIter, absPrec, useMaxNorms); out's grid is the start grid."""
    _check(_lib.mw_multiply(prec, out.ptr, coef, a.ptr, b.ptr, max_iter, int(abs_prec), int(use_max_norms)),
           out.mra.ptr)
    return out.mra.last_stats()


def square(prec, out, inp, max_iter=-1, abs_prec=False):
    """mrcpp::square(prec, out, inp)."""
    _check(_lib.mw_square(prec, out.ptr, inp.ptr, max_iter, int(abs_prec)), out.mra.ptr)
    return out.mra.last_stats()


def add(prec, out, vec, max_iter=-1):
    """mrcpp::add(prec, out, FunctionTreeVector, maxIter); vec = [(coef, tree), ...], union grid."""
    coefs = np.ascontiguousarray([c for c, _ in vec], dtype=np.float64)
    trees = [t for _, t in vec]
    _check(_lib.mw_add(prec, out.ptr, len(trees), _dp(coefs), _ptrs(trees), max_iter), out.mra.ptr)
    return out.mra.last_stats()


def build_grid(out, trees):
    """mrcpp::build_grid(out, vec): extend out's grid by the union of the trees' grids."""
    if isinstance(trees, FunctionTree):
        trees = [trees]
    trees = [t[1] if isinstance(t, tuple) else t for t in trees]
    _check(_lib.mw_build_grid(out.ptr, len(trees), _ptrs(trees)), out.mra.ptr)


def copy_grid(out, inp):
    """mrcpp::copy_grid(out, inp)."""
    _check(_lib.mw_copy_grid(out.ptr, inp.ptr), out.mra.ptr)


def copy_func(out, inp):
    """mrcpp::copy_func(out, inp): inp's coefficients on out's grid."""
    _check(_lib.mw_copy_func(out.ptr, inp.ptr), out.mra.ptr)


def clear(trees, dealloc=False):
    """mrcpp::clear(vec, dealloc)."""
    for t in trees:
        t = t[1] if isinstance(t, tuple) else t
        if dealloc:
            t.close()
        else:
            t.clear()


def density(prec, rho, orbitals, occupations, crop=True):
    """rho <- sum_i occ_i |phi_i|^2 on the device (density::compute, src/qmfunctions/density_utils.cpp:64-150)."""
    occ = np.ascontiguousarray(occupations, dtype=np.float64)
    _check(_lib.mw_density(prec, rho.ptr, len(orbitals), _ptrs(orbitals), _dp(occ), int(crop)), rho.mra.ptr)
    return rho.mra.last_stats()


def rotate(outs, ins, U):
    """out_i <- sum_j U[i, j] in_j on the inputs' union grid (orbital rotation)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    if U.shape != (len(outs), len(ins)):
        raise ValueError("U must be len(outs) x len(ins)")
    _check(_lib.mw_rotate(len(outs), _ptrs(outs), len(ins), _ptrs(ins), _dp(U)), outs[0].mra.ptr)
    return outs[0].mra.last_stats()


def save_tree(tree, path):
    _check(_lib.mw_tree_save(tree.ptr, os.fsencode(path)), tree.mra.ptr)


def load_tree(tree, path):
    _check(_lib.mw_tree_load(tree.ptr, os.fsencode(path)), tree.mra.ptr)
    return tree


def dot(a, b):
    """mrcpp::dot(a, b) = <a|b>."""
    v = C.c_double()
    _check(_lib.mw_dot(a.ptr, b.ptr, C.byref(v)), a.mra.ptr)
    return v.value


def dot_noalloc(a, b):
    """<a|b> without allocating anything, for callers that cannot allocate GPU memory at that point.

    Uses a fixed 1 MiB device array, reserved when the context was created and held for the life
    of the process: at most 32768 nodes common to both trees; calls that overlap race on that
    array.  Blocks until the result is on the host, so not callable during stream capture.
    """
    v = C.c_double()
    _check(_lib.mw_dot_noalloc(a.ptr, b.ptr, C.byref(v)), a.mra.ptr)
    return v.value


def cuda_available():
    """True when the engine can create a context on device 0."""
    try:
        load_library()
        MultiResolutionAnalysis(order=5, max_depth=4).close()
        return True
    except (MWError, ImportError, OSError):
        return False
