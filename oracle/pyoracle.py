"""ctypes wrapper of the CPU oracle (oracle/_build/libmworacle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, as the CPU result the GPU path is compared
with.  The product package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmworacle.so")
_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


class GTerm(C.Structure):
    _fields_ = [("coef", C.c_double), ("alpha", C.c_double), ("pos", C.c_double * 3),
                ("pw", C.c_int * 3), ("pad", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("out_nodes", C.c_longlong), ("items", C.c_longlong), ("pairs", C.c_longlong),
                ("generated", C.c_longlong), ("flops", C.c_double), ("seconds", C.c_double),
                ("bound_hist", C.c_longlong * 32)]


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(_LIB_PATH)
    P, D, I = C.c_void_p, C.c_double, C.c_int
    ip = C.POINTER(C.c_int)
    dp = C.POINTER(C.c_double)
    sig = {
        "orc_mra_create": (P, [I, ip, ip, I, I, I]),
        "orc_mra_free": (None, [P]),
        "orc_mra_basis": (None, [P, dp, dp, dp, dp, dp]),
        "orc_tree_create": (P, [P]),
        "orc_tree_free": (None, [P]),
        "orc_tree_nnodes": (I, [P]),
        "orc_tree_nleaves": (I, [P]),
        "orc_tree_depth": (I, [P]),
        "orc_tree_export": (None, [P, ip, dp, C.POINTER(C.c_ubyte)]),
        "orc_tree_import": (P, [P, I, ip, dp]),
        "orc_tree_norm": (D, [P]),
        "orc_tree_sqnorm": (D, [P]),
        "orc_tree_integrate": (D, [P]),
        "orc_tree_eval": (D, [P, dp]),
        "orc_tree_rescale": (None, [P, D]),
        "orc_dot": (D, [P, P]),
        "orc_project_gauss": (I, [D, P, I, C.POINTER(GTerm), I]),
        "orc_project_hydrogen": (I, [D, P, I, I, I, D, dp, I]),
        "orc_copy_grid": (None, [P, P]),
        "orc_build_grid": (None, [P, I, C.POINTER(P)]),
        "orc_clear": (None, [P]),
        "orc_oper_poisson": (P, [P, D]),
        "orc_oper_helmholtz": (P, [P, D, D]),
        "orc_oper_free": (None, [P]),
        "orc_oper_nterms": (I, [P]),
        "orc_oper_terms": (None, [P, dp, dp]),
        "orc_oper_band": (I, [P, I, I]),
        "orc_oper_block": (I, [P, I, I, I, dp, dp]),
        "orc_oper_kernel_eval": (D, [P, D]),
        "orc_apply": (I, [D, P, P, P, I, I, I, C.POINTER(P), C.POINTER(Stats)]),
        "orc_multiply": (I, [D, P, D, P, P, I, I, I]),
        "orc_add": (I, [D, P, I, dp, C.POINTER(P), I]),
        "orc_crop": (None, [P, D, I]),
        "orc_set_threads": (None, [I]),
        "orc_get_threads": (I, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class MRA:
    """World box [corner, corner+boxes] * 2^-root_scale, order k, basis 'interpolating'|'legendre'."""

    def __init__(self, order, root_scale=-5, corner=(-1, -1, -1), boxes=(2, 2, 2), basis="interpolating",
                 max_depth=25):
        L = lib()
        self.order = order
        self.K = order + 1
        self.root_scale = root_scale
        self.corner = tuple(corner)
        self.boxes = tuple(boxes)
        self.basis = basis
        self.max_depth = max_depth
        c = np.array(corner, dtype=np.int32)
        b = np.array(boxes, dtype=np.int32)
        self.ptr = L.orc_mra_create(root_scale, _iptr(c), _iptr(b), order, 1 if basis == "interpolating" else 0,
                                    max_depth)
        if not self.ptr:
            raise ValueError("invalid MRA parameters")

    def basis_data(self):
        K = self.K
        qx, qw = np.zeros(K), np.zeros(K)
        W = np.zeros((2 * K, 2 * K))
        c2v, v2c = np.zeros((K, K)), np.zeros((K, K))
        lib().orc_mra_basis(self.ptr, _dptr(qx), _dptr(qw), _dptr(W), _dptr(c2v), _dptr(v2c))
        return dict(qx=qx, qw=qw, W=W, c2v=c2v, v2c=v2c)

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.orc_mra_free(self.ptr)
            self.ptr = None


class Tree:
    def __init__(self, mra, ptr=None):
        self.mra = mra
        self.ptr = ptr if ptr else lib().orc_tree_create(mra.ptr)

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.orc_tree_free(self.ptr)
            self.ptr = None

    @property
    def nnodes(self):
        return lib().orc_tree_nnodes(self.ptr)

    @property
    def nleaves(self):
        return lib().orc_tree_nleaves(self.ptr)

    @property
    def depth(self):
        return lib().orc_tree_depth(self.ptr)

    def export(self):
        n = self.nnodes
        K = self.mra.K
        keys = np.zeros((n, 4), dtype=np.int32)
        coefs = np.zeros((n, 8 * K ** 3))
        leaf = np.zeros(n, dtype=np.uint8)
        lib().orc_tree_export(self.ptr, _iptr(keys), _dptr(coefs), leaf.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return keys, coefs, leaf

    @classmethod
    def from_arrays(cls, mra, keys, coefs):
        keys = np.ascontiguousarray(keys, dtype=np.int32)
        coefs = np.ascontiguousarray(coefs, dtype=np.float64)
        p = lib().orc_tree_import(mra.ptr, keys.shape[0], _iptr(keys), _dptr(coefs))
        if not p:
            raise ValueError("keys do not form a complete tree")
        return cls(mra, p)

    def norm(self):
        return lib().orc_tree_norm(self.ptr)

    def sqnorm(self):
        return lib().orc_tree_sqnorm(self.ptr)

    def integrate(self):
        return lib().orc_tree_integrate(self.ptr)

    def eval(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        return lib().orc_tree_eval(self.ptr, _dptr(r))

    def rescale(self, c):
        lib().orc_tree_rescale(self.ptr, float(c))

    def crop(self, prec, abs_prec=False):
        lib().orc_crop(self.ptr, prec, int(abs_prec))

    def clear(self):
        lib().orc_clear(self.ptr)


def dot(a, b):
    return lib().orc_dot(a.ptr, b.ptr)


def gterms(terms):
    """terms: list of (coef, alpha, (X,Y,Z), (px,py,pz))."""
    arr = (GTerm * len(terms))()
    for i, (c, a, pos, pw) in enumerate(terms):
        arr[i].coef = c
        arr[i].alpha = a
        for d in range(3):
            arr[i].pos[d] = pos[d]
            arr[i].pw[d] = pw[d]
    return arr


def project_gauss(prec, tree, terms, abs_prec=False):
    arr = gterms(terms)
    rc = lib().orc_project_gauss(prec, tree.ptr, len(terms), arr, int(abs_prec))
    if rc != 0:
        raise RuntimeError("projection failed")
    return tree


def project_hydrogen(prec, tree, n, l, m, Z=1.0, origin=(0.0, 0.0, 0.0), abs_prec=False):
    o = np.array(origin, dtype=np.float64)
    rc = lib().orc_project_hydrogen(prec, tree.ptr, n, l, m, Z, _dptr(o), int(abs_prec))
    if rc != 0:
        raise ValueError("unsupported hydrogen orbital")
    return tree


def copy_grid(out, inp):
    lib().orc_copy_grid(out.ptr, inp.ptr)


def build_grid(out, trees):
    arr = (C.c_void_p * len(trees))(*[t.ptr for t in trees])
    lib().orc_build_grid(out.ptr, len(trees), arr)


class Operator:
    def __init__(self, mra, ptr):
        self.mra = mra
        self.ptr = ptr
        if not ptr:
            raise ValueError("operator construction failed")

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.orc_oper_free(self.ptr)
            self.ptr = None

    @property
    def nterms(self):
        return lib().orc_oper_nterms(self.ptr)

    def terms(self):
        T = self.nterms
        c, a = np.zeros(T), np.zeros(T)
        lib().orc_oper_terms(self.ptr, _dptr(c), _dptr(a))
        return c, a

    def band(self, t, n):
        return lib().orc_oper_band(self.ptr, t, n)

    def block(self, t, n, l):
        K = self.mra.K
        b = np.zeros((2 * K, 2 * K))
        nr = np.zeros(4)
        if lib().orc_oper_block(self.ptr, t, n, l, _dptr(b), _dptr(nr)) != 0:
            raise IndexError("no block")
        return b, nr

    def kernel(self, r):
        return lib().orc_oper_kernel_eval(self.ptr, float(r))


def poisson(mra, prec):
    return Operator(mra, lib().orc_oper_poisson(mra.ptr, prec))


def helmholtz(mra, mu, prec):
    return Operator(mra, lib().orc_oper_helmholtz(mra.ptr, mu, prec))


def apply(prec, out, op, inp, max_iter=-1, abs_prec=False, prec_trees=()):
    st = Stats()
    arr = (C.c_void_p * max(1, len(prec_trees)))(*[t.ptr for t in prec_trees])
    rc = lib().orc_apply(prec, out.ptr, op.ptr, inp.ptr, max_iter, int(abs_prec), len(prec_trees), arr, C.byref(st))
    if rc != 0:
        raise RuntimeError("apply failed")
    return dict(out_nodes=st.out_nodes, items=st.items, pairs=st.pairs, generated=st.generated, flops=st.flops,
                seconds=st.seconds, bound_hist=list(st.bound_hist))


def multiply(prec, out, coef, a, b, max_iter=-1, abs_prec=False, use_max_norms=False):
    rc = lib().orc_multiply(prec, out.ptr, coef, a.ptr, b.ptr, max_iter, int(abs_prec), int(use_max_norms))
    if rc != 0:
        raise RuntimeError("multiply failed")


def add(prec, out, coefs, trees, max_iter=-1):
    c = np.ascontiguousarray(coefs, dtype=np.float64)
    arr = (C.c_void_p * len(trees))(*[t.ptr for t in trees])
    rc = lib().orc_add(prec, out.ptr, len(trees), _dptr(c), arr, max_iter)
    if rc != 0:
        raise RuntimeError("add failed")


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()
