"""ORACLE -- test infrastructure only.

ctypes bindings to the reference's own compiled functions in
oracle/_ref/libxyst_ref.so (built from the unmodified reference sources by
oracle/build_ref.sh).  Available only where the reference sources exist;
callers skip when :func:`available` is false.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import REF_LIB, _c, _p

_i64 = C.c_int64
_dbl = C.c_double
_vp = C.c_void_p
_lib = None


def available() -> bool:
    return os.path.exists(REF_LIB)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(REF_LIB)
        _lib.ref_last_error.restype = C.c_char_p
        _lib.ref_set_config.argtypes = [_dbl, C.c_char_p, C.c_int, _dbl, C.c_char_p, C.c_int]
        _lib.ref_set_problem_params.argtypes = [_dbl] * 8
        _lib.ref_riemann_grad.argtypes = [_i64, _vp, _i64] + [_i64, _vp, _vp] * 3 + [_i64, _vp, _vp, _vp]
        _lib.ref_riemann_rhs.argtypes = ([_i64, _vp, _i64] + [_i64, _vp, _vp] * 3 +
                                         [_i64, _vp, _vp, _vp, _vp, _vp, _dbl, _vp])
        _lib.ref_kozak_rhs.argtypes = [_i64, _vp, _i64, _vp, _i64, _dbl, _dbl, _vp, _vp]
        _lib.ref_chorin_div.argtypes = [_i64, _vp, _i64, _vp, _vp, _i64, _vp, _dbl, _vp, _vp, _vp,
                                        C.c_int, _vp]
        _lib.ref_chorin_grad.argtypes = [_i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp]
        _lib.ref_genpsup.argtypes = [_i64, _vp, _vp, _vp, _vp, _vp]
        _lib.ref_set_chorin.argtypes = [_dbl, C.c_int]
        _lib.ref_chorin_vgrad.argtypes = [_i64, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp]
        _lib.ref_chorin_flux.argtypes = [_i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, _vp]
        _lib.ref_chorin_rhs.argtypes = [_i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _dbl, _vp, _vp,
                                        _vp, _vp]
        _lib.ref_csr_pressure.argtypes = [_i64, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp,
                                          _vp, _vp]
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().ref_last_error().decode())


def set_config(gamma=1.4, flux="rusanov", stab2=False, stab2coef=0.2, problem="userdef",
               ncomp=5):
    lib().ref_set_config(gamma, flux.encode(), int(stab2), stab2coef, problem.encode(), ncomp)


def set_problem_params(alpha=0.0, beta=(0.0, 0.0, 0.0), kappa=0.0, r0=0.0, p0=0.0, ce=0.0):
    """The manufactured-solution parameters of the control file."""
    lib().ref_set_problem_params(alpha, beta[0], beta[1], beta[2], kappa, r0, p0, ce)


def _sup(sup):
    """sup: list of three (ids, ints) pairs; missing groups may be None."""
    out = []
    sizes = (4, 3, 2)
    for k in range(3):
        if sup[k] is None:
            out.append((0, None, None))
        else:
            ids = _c(sup[k][0], np.int64)
            ints = _c(sup[k][1], np.float64)
            out.append((ids.size // sizes[k], ids, ints))
    return out


def riemann_grad(coord, sup, tri, U):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    U = _c(U, np.float64)
    tri = _c(tri, np.int64)
    s = _sup(sup)
    G = np.zeros((n, 15))
    args = [n, _p(coord), 5]
    for cnt, ids, ints in s:
        args += [cnt, _p(ids), _p(ints)]
    args += [tri.shape[0], _p(tri), _p(U), _p(G)]
    _check(lib().ref_riemann_grad(*args))
    return G


def riemann_rhs(coord, sup, tri, besym, G, U, vol, t=0.0):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    U = _c(U, np.float64)
    G = _c(G, np.float64)
    vol = _c(vol, np.float64)
    tri = _c(tri, np.int64)
    besym = _c(besym, np.uint8)
    s = _sup(sup)
    R = np.zeros((n, 5))
    args = [n, _p(coord), 5]
    for cnt, ids, ints in s:
        args += [cnt, _p(ids), _p(ints)]
    args += [tri.shape[0], _p(tri), _p(besym), _p(G), _p(U), _p(vol), t, _p(R)]
    _check(lib().ref_riemann_rhs(*args))
    return R


def kozak_rhs(coord, inpoel, U, t, dt):
    coord = _c(coord, np.float64)
    inpoel = _c(inpoel, np.int64)
    U = _c(U, np.float64)
    n = coord.shape[1]
    R = np.zeros((n, 5))
    _check(lib().ref_kozak_rhs(inpoel.shape[0], _p(inpoel), n, _p(coord), 5, t, dt, _p(U), _p(R)))
    return R


def chorin_grad(coord, edge, dedge5, tri, S):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    edge = _c(edge, np.int64)
    dedge5 = _c(dedge5, np.float64)
    tri = _c(tri, np.int64)
    S = _c(S, np.float64)
    G = np.zeros((n, 3))
    _check(lib().ref_chorin_grad(n, _p(coord), edge.shape[0], _p(edge), _p(dedge5), tri.shape[0],
                                 _p(tri), _p(S), _p(G)))
    return G


def chorin_div(coord, edge, dedge5, tri, dt, P, PG, Uvel, stab):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    edge = _c(edge, np.int64)
    dedge5 = _c(dedge5, np.float64)
    tri = _c(tri, np.int64)
    P = _c(P, np.float64)
    PG = _c(PG, np.float64)
    Uvel = _c(Uvel, np.float64)
    D = np.zeros(n)
    _check(lib().ref_chorin_div(n, _p(coord), edge.shape[0], _p(edge), _p(dedge5), tri.shape[0],
                                _p(tri), dt, _p(P), _p(PG), _p(Uvel), int(stab), _p(D)))
    return D


def genpsup(inpoel):
    inpoel = _c(inpoel, np.int64)
    n1 = np.zeros(1, np.int64)
    n2 = np.zeros(1, np.int64)
    _check(lib().ref_genpsup(inpoel.shape[0], _p(inpoel), _p(n1), _p(n2), None, None))
    p1 = np.zeros(int(n1[0]), np.int64)
    p2 = np.zeros(int(n2[0]), np.int64)
    _check(lib().ref_genpsup(inpoel.shape[0], _p(inpoel), _p(n1), _p(n2), _p(p1), _p(p2)))
    return p1, p2


def csr_pressure(coord, inpoel, dirnodes=(), dirvals=(), x=None):
    """Reference pressure matrix (1-based CSR), A*x and the Dirichlet rhs shift."""
    coord = _c(coord, np.float64)
    inpoel = _c(inpoel, np.int64)
    n = coord.shape[1]
    dn = _c(np.asarray(dirnodes, dtype=np.int64), np.int64)
    dv = _c(np.asarray(dirvals, dtype=np.float64), np.float64)
    nnz = np.zeros(1, np.int64)
    _check(lib().ref_csr_pressure(inpoel.shape[0], _p(inpoel), n, _p(coord), dn.size, _p(dn),
                                  _p(dv), None, _p(nnz), None, None, None, None, None))
    k = int(nnz[0])
    ia = np.zeros(n + 1, np.int64)
    ja = np.zeros(k, np.int64)
    a = np.zeros(k)
    ax = np.zeros(n)
    bmod = np.zeros(n)
    xx = None if x is None else _c(x, np.float64)
    _check(lib().ref_csr_pressure(inpoel.shape[0], _p(inpoel), n, _p(coord), dn.size, _p(dn),
                                  _p(dv), _p(xx), _p(nnz), _p(ia), _p(ja), _p(a),
                                  _p(ax) if xx is not None else None, _p(bmod)))
    return ia, ja, a, (ax if xx is not None else None), bmod


def set_chorin(mu=0.0, stab=True):
    lib().ref_set_chorin(mu, int(stab))


def chorin_vgrad(coord, edge, dedge5, tri, U):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    edge, dedge5, tri = _c(edge, np.int64), _c(dedge5, np.float64), _c(tri, np.int64)
    U = _c(U, np.float64)
    nc = U.shape[1]
    G = np.zeros((n, 3 * nc))
    _check(lib().ref_chorin_vgrad(n, _p(coord), edge.shape[0], _p(edge), _p(dedge5),
                                  tri.shape[0], _p(tri), nc, _p(U), _p(G)))
    return G


def chorin_flux(coord, edge, dedge5, tri, U, G):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    edge, dedge5, tri = _c(edge, np.int64), _c(dedge5, np.float64), _c(tri, np.int64)
    U, G = _c(U, np.float64), _c(G, np.float64)
    F = np.zeros((n, 3))
    _check(lib().ref_chorin_flux(n, _p(coord), edge.shape[0], _p(edge), _p(dedge5), tri.shape[0],
                                 _p(tri), _p(U), _p(G), _p(F)))
    return F


def chorin_rhs(coord, edge, dedge5, tri, vol, P, U, G, t=0.0):
    coord = _c(coord, np.float64)
    n = coord.shape[1]
    edge, dedge5, tri = _c(edge, np.int64), _c(dedge5, np.float64), _c(tri, np.int64)
    vol, P, U, G = _c(vol, np.float64), _c(P, np.float64), _c(U, np.float64), _c(G, np.float64)
    R = np.zeros((n, 3))
    _check(lib().ref_chorin_rhs(n, _p(coord), edge.shape[0], _p(edge), _p(dedge5), tri.shape[0],
                                _p(tri), _p(vol), t, _p(P), _p(U), _p(G), _p(R)))
    return R
