"""ORACLE -- test infrastructure only.

ctypes bindings to the serial C++ restatement of the reference's CPU arithmetic
(oracle/xg_oracle.cpp) and, where it has been built, to the reference's own
compiled functions (oracle/_ref/libxyst_ref.so, see oracle/build_ref.sh).

Only tests/, the smoke check and the CPU-baseline leg of bench.py import this
package, and only as the checker.  The product library never loads it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libxyst_ref.so")

_i64 = C.c_int64
_dbl = C.c_double
_vp = C.c_void_p


def build(force: bool = False) -> str:
    """Compile the restatement (seconds).  Flags follow the reference's build:
    no FP contraction, so the arithmetic matches operation by operation."""
    src = os.path.join(HERE, "xg_oracle.cpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                           src, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


def reference_root() -> str | None:
    """Where the reference's sources are: $XYST_REFERENCE if set, else a
    checkout named ``reference`` beside this repository; None when neither
    holds the reference's src/Physics."""
    cands = [os.environ.get("XYST_REFERENCE"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "src", "Physics")):
            return c
    return None


def build_ref(root: str | None = None) -> str | None:
    """Build oracle/_ref from the reference sources when they are present."""
    src = root or reference_root()
    if src is None or not os.path.isdir(os.path.join(src, "src", "Physics")):
        return None
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), src])
    return REF_LIB


def _p(a):
    return a.ctypes.data_as(_vp) if a is not None else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_vol.restype = _i64
        L.orc_domint.restype = _i64
        L.orc_bnorm.restype = C.c_int
        L.orc_riecg_create.restype = _vp
        L.orc_riecg_create.argtypes = [_i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _dbl,
                                       C.c_int, C.c_int, _dbl, _dbl, _dbl]
        L.orc_riecg_destroy.argtypes = [_vp]
        L.orc_riecg_set_sym.argtypes = [_vp, _i64, _vp, _vp]
        L.orc_riecg_set_far.argtypes = [_vp, _i64, _vp, _vp, _dbl, _dbl, _dbl, _dbl, _dbl]
        L.orc_riecg_set_dir.argtypes = [_vp, _i64, _vp, _vp, _vp]
        L.orc_riecg_set_pre.argtypes = [_vp, _i64, _vp, _vp]
        L.orc_riecg_set_state.argtypes = [_vp, _vp, _dbl]
        L.orc_riecg_get_state.argtypes = [_vp, _vp]
        L.orc_riecg_grad.argtypes = [_vp, _vp, _vp]
        L.orc_riecg_rhs.argtypes = [_vp, _vp, _vp, _vp]
        L.orc_riecg_bc.argtypes = [_vp]
        L.orc_riecg_dt.argtypes = [_vp]
        L.orc_riecg_dt.restype = _dbl
        L.orc_riecg_run.argtypes = [_vp, _i64, _vp]
        L.orc_riecg_run.restype = _dbl
        L.orc_riecg_stage.argtypes = [_vp, C.c_int, _dbl]
        L.orc_riecg_set_source.argtypes = [_vp, C.c_int, _vp]
        L.orc_kozcg_create.restype = _vp
        L.orc_kozcg_create.argtypes = [_i64, _vp, _vp, _i64, _vp, _dbl, _dbl, _dbl, C.c_int,
                                       _dbl, C.c_int, C.c_int, _vp]
        L.orc_kozcg_destroy.argtypes = [_vp]
        L.orc_kozcg_set_sym.argtypes = [_vp, _i64, _vp, _vp]
        L.orc_kozcg_set_dir.argtypes = [_vp, _i64, _vp, _vp, _vp]
        L.orc_kozcg_set_state.argtypes = [_vp, _vp, _dbl]
        L.orc_kozcg_set_source.argtypes = [_vp, C.c_int, _vp]
        L.orc_kozcg_step.argtypes = [_vp, _dbl]
        L.orc_kozcg_dt.argtypes = [_vp]
        L.orc_kozcg_dt.restype = _dbl
        L.orc_kozcg_get_state.argtypes = [_vp, _vp]
        L.orc_kozcg_rhs.argtypes = [_vp, _vp, _dbl, _vp]
        L.orc_kozcg_run.argtypes = [_vp, _i64, _vp]
        L.orc_kozcg_run.restype = _dbl
        L.orc_pressure_matrix.restype = _i64
        L.orc_csr_dirichlet.argtypes = [_i64, _vp, _vp, _vp, _vp, _i64, _vp, _vp]
        L.orc_pcg.restype = _i64
        L.orc_pcg.argtypes = [_i64, _vp, _vp, _vp, _vp, _vp, _i64, _dbl, C.c_int, _vp, _vp, _vp]
        L.orc_csr_mult.argtypes = [_i64, _vp, _vp, _vp, _vp, _vp]
        L.orc_chocg_create.restype = _vp
        L.orc_chocg_create.argtypes = ([_i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, _vp,
                                        _dbl, _dbl, _dbl] + [C.c_int] * 3 +
                                       [_dbl, C.c_int, C.c_int, _dbl, _i64])
        L.orc_chocg_destroy.argtypes = [_vp]
        L.orc_chocg_set_bc.argtypes = [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _i64,
                                       _vp, _vp]
        L.orc_chocg_set_state.argtypes = [_vp, _vp, _vp, _dbl]
        L.orc_chocg_get.argtypes = [_vp, C.c_int, _vp]
        L.orc_chocg_init.argtypes = [_vp]
        L.orc_chocg_init.restype = _i64
        L.orc_chocg_step.argtypes = [_vp, _vp]
        L.orc_chocg_step.restype = _dbl
        L.orc_chocg_set_theta.argtypes = [_vp, _dbl, _i64, _vp, C.c_int, _i64, _dbl]
        L.orc_chocg_momentum_its.argtypes = [_vp]
        L.orc_chocg_momentum_its.restype = _i64
        L.orc_chocg_div.argtypes = [_vp, _vp, _vp, _vp, _dbl, C.c_int, _vp]
        L.orc_chocg_vgrad.argtypes = [_vp, _vp, C.c_int, _vp]
        L.orc_chocg_flux.argtypes = [_vp, _vp, _vp, _vp]
        L.orc_chocg_rhs.argtypes = [_vp, _vp, _vp, _vp, _vp]
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ---------------------------------------------------------------- mesh setup

def vol(coord, inpoel):
    coord = _c(coord, np.float64)
    inpoel = _c(inpoel, np.int64)
    n = coord.shape[1]
    v = np.zeros(n)
    bad = lib().orc_vol(_i64(n), _p(coord), _i64(inpoel.shape[0]), _p(inpoel), _p(v))
    if bad:
        raise ValueError(f"{bad} elements with non-positive Jacobian")
    return v


def domint(coord, inpoel, gid=None, ncoef=3):
    """Edge list (E,2) in (smaller, larger global id) orientation and D (E,ncoef)."""
    coord = _c(coord, np.float64)
    inpoel = _c(inpoel, np.int64)
    n = coord.shape[1]
    g = None if gid is None else _c(gid, np.int64)
    ne = lib().orc_domint(_i64(n), _p(coord), _i64(inpoel.shape[0]), _p(inpoel), _p(g),
                          C.c_int(ncoef), _i64(0), None, None)
    edge = np.zeros((ne, 2), np.int64)
    d = np.zeros((ne, ncoef))
    lib().orc_domint(_i64(n), _p(coord), _i64(inpoel.shape[0]), _p(inpoel), _p(g),
                     C.c_int(ncoef), _i64(ne), _p(edge), _p(d))
    return edge, d


def bnorm(coord, faces, nodes):
    coord = _c(coord, np.float64)
    faces = _c(faces, np.int64)
    nodes = _c(nodes, np.int64)
    out = np.zeros((nodes.size, 3))
    rc = lib().orc_bnorm(_i64(coord.shape[1]), _p(coord), _i64(faces.shape[0]), _p(faces),
                         _i64(nodes.size), _p(nodes), _p(out))
    if rc:
        raise ValueError(lib().orc_last_error())
    return out


def sym_bc(coord, bface, sym_sets, far_sets=()):
    """Symmetry BC node list and normals in the reference's layout
    (src/Inciter/RieCG.cpp:109-245, 527-618): every node on a face of a
    symmetry side set (minus farfield nodes) gets one entry per symmetry set
    that contains it, in the configured set order."""
    far = set()
    for s in far_sets:
        if s in bface:
            far.update(np.unique(bface[s]).tolist())
    symset = set()
    for s in sym_sets:
        if s in bface:
            symset.update(np.unique(bface[s]).tolist())
    symset -= far
    nodes, norms = [], []
    per_set = {}
    for s in sym_sets:
        if s not in bface:
            continue
        sn = np.unique(bface[s])
        per_set[s] = (set(sn.tolist()), dict(zip(sn.tolist(), bnorm(coord, bface[s], sn))))
    for p in sorted(symset):
        for s in sym_sets:
            if s in per_set and p in per_set[s][0]:
                nodes.append(p)
                norms.append(per_set[s][1][p])
    return (np.array(nodes, dtype=np.int64), np.array(norms, dtype=np.float64).reshape(-1, 3),
            symset)


# ---------------------------------------------------------------- RieCG

# problems with a manufactured source term in riemann::rhs (codes of the C ABI)
SOURCES = {"none": 0, "taylor_green": 1, "vortical_flow": 2, "nonlinear_energy_growth": 3,
           "rayleigh_taylor": 4}


class RieCG:
    """Serial RieCG restatement over a plain edge list (canonical orientation)."""

    def __init__(self, coord, vol, edge, dedge, tri, besym, gamma=1.4, flux="rusanov",
                 stab2=False, stab2coef=0.2, cfl=0.5, const_dt=0.0):
        self.coord = _c(coord, np.float64)
        self.n = self.coord.shape[1]
        self._keep = [self.coord, _c(vol, np.float64), _c(edge, np.int64), _c(dedge, np.float64),
                      _c(tri, np.int64), _c(besym, np.uint8)]
        c, v, e, d, t, b = self._keep
        self.h = lib().orc_riecg_create(self.n, _p(c), _p(v), e.shape[0], _p(e), _p(d),
                                        t.shape[0], _p(t), _p(b), gamma,
                                        1 if flux == "hllc" else 0, int(stab2), stab2coef, cfl,
                                        const_dt)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_riecg_destroy(self.h)
            self.h = None

    def set_sym(self, nodes, norms):
        nodes = _c(nodes, np.int64)
        norms = _c(norms, np.float64)
        self._sym = (nodes, norms)
        lib().orc_riecg_set_sym(self.h, nodes.size, _p(nodes), _p(norms))

    def set_far(self, nodes, norms, r, u, v, w, p):
        nodes = _c(nodes, np.int64)
        norms = _c(norms, np.float64)
        self._far = (nodes, norms)
        lib().orc_riecg_set_far(self.h, nodes.size, _p(nodes), _p(norms), r, u, v, w, p)

    def set_dir(self, nodes, mask, vals):
        nodes = _c(nodes, np.int64)
        mask = _c(mask, np.int32)
        vals = _c(vals, np.float64)
        self._dir = (nodes, mask, vals)
        lib().orc_riecg_set_dir(self.h, nodes.size, _p(nodes), _p(mask), _p(vals))

    def set_pre(self, nodes, vals):
        nodes = _c(nodes, np.int64)
        vals = _c(vals, np.float64)
        self._pre = (nodes, vals)
        lib().orc_riecg_set_pre(self.h, nodes.size, _p(nodes), _p(vals))

    def set_state(self, U, t=0.0):
        U = _c(U, np.float64)
        lib().orc_riecg_set_state(self.h, _p(U), t)

    def state(self):
        U = np.zeros((self.n, 5))
        lib().orc_riecg_get_state(self.h, _p(U))
        return U

    def grad(self, U):
        U = _c(U, np.float64)
        G = np.zeros((self.n, 15))
        lib().orc_riecg_grad(self.h, _p(U), _p(G))
        return G

    def rhs(self, G, U):
        G = _c(G, np.float64)
        U = _c(U, np.float64)
        R = np.zeros((self.n, 5))
        lib().orc_riecg_rhs(self.h, _p(G), _p(U), _p(R))
        return R

    def set_source(self, problem, prm=None):
        """The manufactured source of riemann::rhs (SOURCES names the
        problems), evaluated at the state's time; prm = alpha, beta[3], kappa,
        r0, p0, ce."""
        self._src = None if prm is None else _c(np.asarray(prm, dtype=np.float64), np.float64)
        lib().orc_riecg_set_source(self.h, SOURCES[problem],
                                   None if self._src is None else _p(self._src))

    def bc(self):
        lib().orc_riecg_bc(self.h)

    def dt(self):
        return lib().orc_riecg_dt(self.h)

    def run(self, nstep):
        dts = np.zeros(nstep)
        lib().orc_riecg_run(self.h, nstep, _p(dts))
        return dts

    def stage(self, stage, dt):
        lib().orc_riecg_stage(self.h, stage, dt)


# ---------------------------------------------------------------- KozCG

class KozCG:
    def __init__(self, coord, vol, inpoel, gamma=1.4, cfl=0.5, const_dt=0.0, fct=True,
                 ctau=1.0, fctclip=False, fctsys=()):
        self.coord = _c(coord, np.float64)
        self.n = self.coord.shape[1]
        sys_ = _c(np.asarray(fctsys, dtype=np.int32), np.int32)
        self._keep = [self.coord, _c(vol, np.float64), _c(inpoel, np.int64), sys_]
        c, v, e, s = self._keep
        self.h = lib().orc_kozcg_create(self.n, _p(c), _p(v), e.shape[0], _p(e), gamma, cfl,
                                        const_dt, int(fct), ctau, int(fctclip), s.size, _p(s))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_kozcg_destroy(self.h)
            self.h = None

    def set_sym(self, nodes, norms):
        nodes = _c(nodes, np.int64)
        norms = _c(norms, np.float64)
        self._sym = (nodes, norms)
        lib().orc_kozcg_set_sym(self.h, nodes.size, _p(nodes), _p(norms))

    def set_dir(self, nodes, mask, vals):
        nodes = _c(nodes, np.int64)
        mask = _c(mask, np.int32)
        vals = _c(vals, np.float64)
        self._dir = (nodes, mask, vals)
        lib().orc_kozcg_set_dir(self.h, nodes.size, _p(nodes), _p(mask), _p(vals))

    def set_state(self, U, t=0.0):
        U = _c(U, np.float64)
        lib().orc_kozcg_set_state(self.h, _p(U), t)

    def set_source(self, problem, prm=None):
        """The manufactured source of kozak::rhs (SOURCES names the problems;
        prm: alpha, beta[3], kappa, r0, p0, ce)."""
        self._src = None if prm is None else _c(np.asarray(prm, dtype=np.float64).reshape(8),
                                                  np.float64)
        lib().orc_kozcg_set_source(self.h, SOURCES[problem],
                                   None if self._src is None else _p(self._src))

    def dt(self):
        return lib().orc_kozcg_dt(self.h)

    def step(self, dt):
        """One step of the given dt."""
        lib().orc_kozcg_step(self.h, dt)

    def state(self):
        U = np.zeros((self.n, 5))
        lib().orc_kozcg_get_state(self.h, _p(U))
        return U

    def rhs(self, U, dt):
        U = _c(U, np.float64)
        R = np.zeros((self.n, 5))
        lib().orc_kozcg_rhs(self.h, _p(U), dt, _p(R))
        return R

    def run(self, nstep):
        dts = np.zeros(nstep)
        lib().orc_kozcg_run(self.h, nstep, _p(dts))
        return dts


# ---------------------------------------------------------------- CSR / PCG

def pressure_matrix(coord, inpoel):
    coord = _c(coord, np.float64)
    inpoel = _c(inpoel, np.int64)
    n = coord.shape[1]
    nnz = lib().orc_pressure_matrix(_i64(n), _p(coord), _i64(inpoel.shape[0]), _p(inpoel),
                                    _i64(0), None, None, None)
    ia = np.zeros(n + 1, np.int64)
    ja = np.zeros(nnz, np.int64)
    a = np.zeros(nnz)
    lib().orc_pressure_matrix(_i64(n), _p(coord), _i64(inpoel.shape[0]), _p(inpoel), _i64(nnz),
                              _p(ia), _p(ja), _p(a))
    return ia, ja, a


def csr_dirichlet(ia, ja, a, b, nodes, vals):
    """In place on a and b (copies returned)."""
    a = _c(a, np.float64).copy()
    b = _c(b, np.float64).copy()
    ia = _c(ia, np.int64)
    ja = _c(ja, np.int64)
    nodes = _c(nodes, np.int64)
    vals = _c(vals, np.float64)
    lib().orc_csr_dirichlet(ia.size - 1, _p(ia), _p(ja), _p(a), _p(b), nodes.size, _p(nodes),
                            _p(vals))
    return a, b


def pcg(ia, ja, a, b, x0, maxit, tol, pc="jacobi"):
    ia = _c(ia, np.int64)
    ja = _c(ja, np.int64)
    a = _c(a, np.float64)
    b = _c(b, np.float64)
    x = _c(x0, np.float64).copy()
    nr = np.zeros(1)
    nb = np.zeros(1)
    conv = np.zeros(1, np.int32)
    it = lib().orc_pcg(ia.size - 1, _p(ia), _p(ja), _p(a), _p(b), _p(x), maxit, tol,
                       1 if pc == "jacobi" else 0, _p(nr), _p(nb), _p(conv))
    return x, int(it), float(nr[0]), float(nb[0]), bool(conv[0])


def csr_mult(ia, ja, a, x):
    ia = _c(ia, np.int64)
    ja = _c(ja, np.int64)
    a = _c(a, np.float64)
    x = _c(x, np.float64)
    r = np.zeros(ia.size - 1)
    lib().orc_csr_mult(ia.size - 1, _p(ia), _p(ja), _p(a), _p(x), _p(r))
    return r


# ---------------------------------------------------------------- ChoCG

class ChoCG:
    """Serial ChoCG (src/Inciter/ChoCG.cpp, src/Physics/Chorin.cpp) over plain
    edges with ChoCG's five integrals per edge; pressure matrix zero-based."""

    def __init__(self, coord, vol, edge, dint5, tri, ia, ja, a, mu=0.0, cfl=0.5, const_dt=0.0,
                 flux="damp2", stab=True, stab2=False, stab2coef=0.2, rk=1, pc="jacobi",
                 ptol=1e-3, pmaxit=10):
        self._k = [_c(coord, np.float64), _c(vol, np.float64), _c(edge, np.int64),
                   _c(dint5, np.float64), _c(tri, np.int64), _c(ia, np.int64), _c(ja, np.int64),
                   _c(a, np.float64)]
        c, v, e, d, t, i, j, aa = self._k
        self.n = c.shape[1]
        self.h = lib().orc_chocg_create(self.n, _p(c), _p(v), e.shape[0], _p(e), _p(d),
                                        t.shape[0], _p(t), _p(i), _p(j), _p(aa), mu, cfl,
                                        const_dt, 1 if flux == "damp4" else 0, int(stab),
                                        int(stab2), stab2coef, rk,
                                        1 if pc == "jacobi" else 0, ptol, pmaxit)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_chocg_destroy(self.h)
            self.h = None

    def set_bc(self, dir=None, sym=None, noslip=(), pdir=None):
        """dir: (nodes, mask (n,3), values (n,3)); sym: (nodes, normals);
        noslip: nodes; pdir: (nodes, values of the initial solves)."""
        z = np.zeros(0, np.int64)
        dn, dm, dv = dir if dir is not None else (z, np.zeros((0, 3)), np.zeros((0, 3)))
        sn, snv = sym if sym is not None else (z, np.zeros((0, 3)))
        pn, pv = pdir if pdir is not None else (z, np.zeros(0))
        k = [_c(dn, np.int64), _c(dm, np.int32), _c(dv, np.float64), _c(sn, np.int64),
             _c(snv, np.float64), _c(np.asarray(noslip), np.int64), _c(pn, np.int64),
             _c(pv, np.float64)]
        self._bc = k
        lib().orc_chocg_set_bc(self.h, k[0].size, _p(k[0]), _p(k[1]), _p(k[2]), k[3].size,
                               _p(k[3]), _p(k[4]), k[5].size, _p(k[5]), k[6].size, _p(k[6]),
                               _p(k[7]))

    def set_state(self, u, p=None, t=0.0):
        u = _c(u, np.float64)
        pp = None if p is None else _c(p, np.float64)
        lib().orc_chocg_set_state(self.h, _p(u), _p(pp), t)

    def get(self, what):
        shape = {0: (self.n, 3), 1: (self.n, 3), 2: (self.n,), 3: (self.n, 3), 4: (self.n, 9),
                 5: (self.n,), 6: (self.n,)}[what]
        out = np.zeros(shape)
        lib().orc_chocg_get(self.h, what, _p(out))
        return out

    def init(self):
        return int(lib().orc_chocg_init(self.h))

    def set_theta(self, theta, inpoel, mom_pc="none", mom_iter=10, mom_tol=1e-3):
        """theta-implicit momentum prediction on the tetrahedra inpoel."""
        self._tets = _c(inpoel, np.int64)
        lib().orc_chocg_set_theta(self.h, theta, self._tets.size // 4, _p(self._tets),
                                  1 if mom_pc == "jacobi" else 0, mom_iter, mom_tol)

    def momentum_its(self):
        return int(lib().orc_chocg_momentum_its(self.h))

    def step(self):
        it = np.zeros(1, np.int64)
        dt = lib().orc_chocg_step(self.h, _p(it))
        return dt, int(it[0])

    def div(self, U, P, G, dt, stab):
        D = np.zeros(self.n)
        U, P, G = _c(U, np.float64), _c(P, np.float64), _c(G, np.float64)
        lib().orc_chocg_div(self.h, _p(U), _p(P), _p(G), dt, int(stab), _p(D))
        return D

    def vgrad(self, U, ncomp):
        G = np.zeros((self.n, 3 * ncomp))
        U = _c(U, np.float64)
        lib().orc_chocg_vgrad(self.h, _p(U), ncomp, _p(G))
        return G

    def flux(self, U, G):
        F = np.zeros((self.n, 3))
        U, G = _c(U, np.float64), _c(G, np.float64)
        lib().orc_chocg_flux(self.h, _p(U), _p(G), _p(F))
        return F

    def rhs(self, U, G, P):
        R = np.zeros((self.n, 3))
        U, G, P = _c(U, np.float64), _c(G, np.float64), _c(P, np.float64)
        lib().orc_chocg_rhs(self.h, _p(U), _p(G), _p(P), _p(R))
        return R
