"""ctypes binding of the CPU oracle (oracle/liboracle.so) for the tests and for
bench.py's CPU-baseline leg. The oracle is the checker, never the thing
measured on the GPU path."""
import ctypes
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
LIB = os.path.join(ORACLE_DIR, "liboracle.so")

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double

_SIGS = {
    "or_restriction_build": [_I, _I, _I, _P, _P, _P, _P, _P],
    "or_restriction_mult": [_I, _I, _P, _P, _P],
    "or_restriction_mult_transpose": [_I, _I, _P, _P, _P, _P, _I],
    "or_restriction_abs_mult_transpose": [_I, _I, _P, _P, _P, _P],
    "or_gauss_legendre": [_I, _P, _P],
    "or_gauss_lobatto": [_I, _P],
    "or_basis_tables": [_I, _P, _I, _P, _P, _P],
    "or_geom_jacobians3d": [_I, _I, _I, _P, _P, _P, _P],
    "or_geom_det3d": [_I, _P, _I, _P],
    "or_diffusion_setup3d": [_I, _I, _I, _P, _P, _P, _L, _P],
    "or_diffusion_apply3d": [_I, _I, _I, _I, _P, _P, _P, _P, _P],
    "or_diffusion_diagonal3d": [_I, _I, _I, _I, _P, _P, _P, _P],
    "or_mass_setup3d": [_I, _I, _P, _P, _P, _L, _I, _P],
    "or_mass_apply3d": [_I, _I, _I, _P, _P, _P, _P],
    "or_mass_diagonal3d": [_I, _I, _I, _P, _P, _P],
    "or_pa_mult": [_I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "or_pa_mult_markers": [_I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "or_pcg_diffusion": [_I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _I,
                         _P, _P, _P, _D, _D, _I, _I, _P, _P],
    "or_num_threads": [],
    "or_set_num_threads": [_I],
    "or_boolean_mask": [_I, _I, _P, _P, _P],
    "or_ptransfer_mult": [_P, _P, _P, _P],
    "or_ptransfer_mult_transpose": [_P, _P, _P, _P],
    "or_chebyshev_coeffs": [_I, _D, _P],
    "or_chebyshev_mult": [_P, _I, _P, _P],
    "or_power_method": [_P, _I, _D, ctypes.c_ulonglong],
    "or_mg_mult": [_P, _I, _I, _D, _I, _P, _P],
    "or_mg_pcg": [_P, _I, _I, _D, _I, _P, _P, _D, _D, _I, _P, _P],
    "or_domain_lf3d": [_I, _I, _I, _P, _P, _P, _P, _L, _I, _P, _P, _P],
}
_RESTYPES = {"or_pcg_diffusion": ctypes.c_int, "or_num_threads": ctypes.c_int,
             "or_power_method": ctypes.c_double, "or_mg_pcg": ctypes.c_int}


class MGLevel(ctypes.Structure):
    """One level of the p-multigrid hierarchy (or_mg_level in gbpa_oracle.h).
    The numpy arrays it points to are kept alive in `keep`."""
    _fields_ = [("ne", _I), ("ndofs", _I), ("d1d", _I), ("q1d", _I), ("gather_map", _P),
                ("offsets", _P), ("indices", _P), ("B", _P), ("G", _P), ("qdata", _P), ("ess", _P),
                ("n_ess", _I), ("diag", _P), ("lambda_", _D), ("Bi", _P)]


def mg_level(ne, ndofs, d1d, q1d, gm, off, ind, B, G, qd, ess, diag=None, lam=0.0, Bi=None):
    arrs = dict(gm=np.ascontiguousarray(gm, np.int32), off=np.ascontiguousarray(off, np.int32),
                ind=np.ascontiguousarray(ind, np.int32), B=np.ascontiguousarray(B, np.float64),
                G=np.ascontiguousarray(G, np.float64), qd=np.ascontiguousarray(qd, np.float64),
                ess=np.ascontiguousarray(ess, np.int32),
                diag=None if diag is None else np.ascontiguousarray(diag, np.float64),
                Bi=None if Bi is None else np.ascontiguousarray(Bi, np.float64))
    lv = MGLevel(ne, ndofs, d1d, q1d, _ptr(arrs["gm"]), _ptr(arrs["off"]), _ptr(arrs["ind"]),
                 _ptr(arrs["B"]), _ptr(arrs["G"]), _ptr(arrs["qd"]), _ptr(arrs["ess"]), arrs["ess"].size,
                 _ptr(arrs["diag"]), lam, _ptr(arrs["Bi"]))
    lv.keep = arrs
    return lv


def build():
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR])


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Oracle:
    def __init__(self, lib):
        self.lib = lib

    def restriction_build(self, ne, dof, ndofs, elem_dofs, dof_map):
        off = np.zeros(ndofs + 1, np.int32)
        ind = np.zeros(ne * dof, np.int32)
        gm = np.zeros(ne * dof, np.int32)
        ed = np.ascontiguousarray(elem_dofs, np.int32)
        dm = None if dof_map is None else np.ascontiguousarray(dof_map, np.int32)
        self.lib.or_restriction_build(ne, dof, ndofs, _ptr(ed), _ptr(dm), _ptr(off), _ptr(ind), _ptr(gm))
        return off, ind, gm

    def restriction_mult(self, ne, nd, gm, x):
        y = np.zeros(ne * nd)
        self.lib.or_restriction_mult(ne, nd, _ptr(gm), _ptr(x), _ptr(y))
        return y

    def restriction_mult_transpose(self, nd, ndofs, off, ind, x, y=None, add=False):
        y = np.zeros(ndofs) if y is None else y
        self.lib.or_restriction_mult_transpose(nd, ndofs, _ptr(off), _ptr(ind), _ptr(x), _ptr(y), int(add))
        return y

    def restriction_abs_mult_transpose(self, nd, ndofs, off, ind, x):
        y = np.zeros(ndofs)
        self.lib.or_restriction_abs_mult_transpose(nd, ndofs, _ptr(off), _ptr(ind), _ptr(x), _ptr(y))
        return y

    def gauss_legendre(self, n):
        x = np.zeros(n); w = np.zeros(n)
        self.lib.or_gauss_legendre(n, _ptr(x), _ptr(w))
        return x, w

    def gauss_lobatto(self, n):
        x = np.zeros(n)
        self.lib.or_gauss_lobatto(n, _ptr(x))
        return x

    def basis_tables(self, nodes, xq):
        D, Q = len(nodes), len(xq)
        B = np.zeros(Q * D); G = np.zeros(Q * D)
        self.lib.or_basis_tables(D, _ptr(np.ascontiguousarray(nodes)), Q,
                                 _ptr(np.ascontiguousarray(xq)), _ptr(B), _ptr(G))
        return B, G

    def geom_jacobians3d(self, ne, dg, q1d, Bg, Gg, nodesE):
        J = np.zeros(q1d ** 3 * 9 * ne)
        self.lib.or_geom_jacobians3d(ne, dg, q1d, _ptr(Bg), _ptr(Gg), _ptr(nodesE), _ptr(J))
        return J

    def geom_det3d(self, ne, J, q3):
        d = np.zeros(q3 * ne)
        self.lib.or_geom_det3d(ne, _ptr(J), q3, _ptr(d))
        return d

    def diffusion_setup3d(self, ne, q1d, coeff_dim, W, J, C):
        S = 9 if coeff_dim == 9 else 6
        D = np.zeros(q1d ** 3 * S * ne)
        C = np.ascontiguousarray(C, np.float64)
        self.lib.or_diffusion_setup3d(ne, q1d, coeff_dim, _ptr(W), _ptr(J), _ptr(C), C.size, _ptr(D))
        return D

    def diffusion_apply3d(self, ne, symm, d1d, q1d, B, G, D, x, y=None):
        y = np.zeros(ne * d1d ** 3) if y is None else y
        self.lib.or_diffusion_apply3d(ne, int(symm), d1d, q1d, _ptr(B), _ptr(G), _ptr(D), _ptr(x), _ptr(y))
        return y

    def diffusion_diagonal3d(self, ne, symm, d1d, q1d, B, G, D):
        y = np.zeros(ne * d1d ** 3)
        self.lib.or_diffusion_diagonal3d(ne, int(symm), d1d, q1d, _ptr(B), _ptr(G), _ptr(D), _ptr(y))
        return y

    def mass_setup3d(self, ne, nq, W, detJ, C, by_val=True):
        D = np.zeros(nq * ne)
        C = np.ascontiguousarray(C, np.float64)
        self.lib.or_mass_setup3d(ne, nq, _ptr(W), _ptr(detJ), _ptr(C), C.size, int(by_val), _ptr(D))
        return D

    def mass_apply3d(self, ne, d1d, q1d, B, D, x, y=None):
        y = np.zeros(ne * d1d ** 3) if y is None else y
        self.lib.or_mass_apply3d(ne, d1d, q1d, _ptr(B), _ptr(D), _ptr(x), _ptr(y))
        return y

    def mass_diagonal3d(self, ne, d1d, q1d, B, D):
        y = np.zeros(ne * d1d ** 3)
        self.lib.or_mass_diagonal3d(ne, d1d, q1d, _ptr(B), _ptr(D), _ptr(y))
        return y

    def pa_mult(self, kind, ne, ndofs, symm, d1d, q1d, gm, off, ind, B, G, D, x):
        y = np.zeros(ndofs)
        work = np.zeros(2 * ne * d1d ** 3)
        self.lib.or_pa_mult(kind, ne, ndofs, int(symm), d1d, q1d, _ptr(gm), _ptr(off), _ptr(ind),
                            _ptr(B), _ptr(G), _ptr(D), _ptr(x), _ptr(y), _ptr(work))
        return y

    def pa_mult_markers(self, kind, ne, ndofs, symm, d1d, q1d, gm, off, ind, B, G, D, attributes, markers, x):
        y = np.zeros(ndofs)
        work = np.zeros(3 * ne * d1d ** 3)
        a = np.ascontiguousarray(attributes, np.int32)
        m = np.ascontiguousarray(markers, np.int32)
        self.lib.or_pa_mult_markers(kind, ne, ndofs, int(symm), d1d, q1d, _ptr(gm), _ptr(off), _ptr(ind),
                                    _ptr(B), _ptr(G), _ptr(D), _ptr(a), _ptr(m), _ptr(x), _ptr(y), _ptr(work))
        return y

    def pcg_diffusion(self, ne, ndofs, symm, d1d, q1d, gm, off, ind, B, G, D, ess, dinv, b,
                      rel_tol=1e-12, abs_tol=0.0, max_it=500, x0=None):
        x = np.zeros(ndofs) if x0 is None else x0.copy()
        fn = ctypes.c_double(0.0); conv = ctypes.c_int(0)
        ess = np.ascontiguousarray(ess, np.int32)
        it = self.lib.or_pcg_diffusion(ne, ndofs, int(symm), d1d, q1d, _ptr(gm), _ptr(off), _ptr(ind),
                                       _ptr(B), _ptr(G), _ptr(D), _ptr(ess), ess.size, _ptr(dinv),
                                       _ptr(b), _ptr(x), rel_tol, abs_tol, max_it, int(x0 is not None),
                                       ctypes.byref(fn), ctypes.byref(conv))
        return x, it, fn.value, bool(conv.value)

    def num_threads(self):
        return self.lib.or_num_threads()

    def set_num_threads(self, n):
        self.lib.or_set_num_threads(int(n))

    def domain_lf3d(self, ne, d1d, q1d, B, W, detJ, f, ndofs, off, ind):
        b = np.zeros(ndofs)
        f = np.ascontiguousarray(f, np.float64)
        self.lib.or_domain_lf3d(ne, d1d, q1d, _ptr(np.ascontiguousarray(B)), _ptr(np.ascontiguousarray(W)),
                                _ptr(np.ascontiguousarray(detJ)), _ptr(f), f.size, ndofs,
                                _ptr(np.ascontiguousarray(off, np.int32)), _ptr(np.ascontiguousarray(ind, np.int32)),
                                _ptr(b))
        return b

    # ---- p-multigrid (levels: list of MGLevel, coarsest first)
    @staticmethod
    def _levels(levels):
        arr = (MGLevel * len(levels))(*levels)
        return arr

    def ptransfer_mult(self, c, f, x):
        y = np.zeros(f.ndofs)
        self.lib.or_ptransfer_mult(ctypes.byref(c), ctypes.byref(f), _ptr(np.ascontiguousarray(x)), _ptr(y))
        return y

    def ptransfer_mult_transpose(self, c, f, x):
        y = np.zeros(c.ndofs)
        self.lib.or_ptransfer_mult_transpose(ctypes.byref(c), ctypes.byref(f),
                                             _ptr(np.ascontiguousarray(x)), _ptr(y))
        return y

    def chebyshev_coeffs(self, order, lam):
        c = np.zeros(order)
        self.lib.or_chebyshev_coeffs(order, lam, _ptr(c))
        return c

    def chebyshev_mult(self, lv, order, x):
        y = np.zeros(lv.ndofs)
        self.lib.or_chebyshev_mult(ctypes.byref(lv), order, _ptr(np.ascontiguousarray(x)), _ptr(y))
        return y

    def power_method(self, lv, steps=10, tol=1e-8, seed=12345):
        return self.lib.or_power_method(ctypes.byref(lv), steps, tol, seed)

    def mg_mult(self, levels, x, order=2, coarse_tol=1e-2, coarse_max=200):
        arr = self._levels(levels)
        y = np.zeros(levels[-1].ndofs)
        self.lib.or_mg_mult(arr, len(levels), order, coarse_tol, coarse_max,
                            _ptr(np.ascontiguousarray(x)), _ptr(y))
        return y

    def mg_pcg(self, levels, b, order=2, coarse_tol=1e-2, coarse_max=200, rel_tol=1e-10, abs_tol=0.0,
               max_it=200):
        arr = self._levels(levels)
        x = np.zeros(levels[-1].ndofs)
        fn = ctypes.c_double(0.0); conv = ctypes.c_int(0)
        it = self.lib.or_mg_pcg(arr, len(levels), order, coarse_tol, coarse_max,
                                _ptr(np.ascontiguousarray(b)), _ptr(x), rel_tol, abs_tol, max_it,
                                ctypes.byref(fn), ctypes.byref(conv))
        return x, it, fn.value, bool(conv.value)


_cached = None


def load():
    global _cached
    if _cached is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        for name, args in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = _RESTYPES.get(name)
        _cached = Oracle(lib)
    return _cached
