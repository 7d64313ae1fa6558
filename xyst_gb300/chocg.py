"""ChoCG (projection scheme for incompressible flow) on the GPU, behind the
reference's own function boundaries.

:class:`ChoCG` mirrors what the reference's ChoCG chare does
(src/Inciter/ChoCG.cpp): ``init`` is the start-up sequence of
``ChoCG::merge`` (projection of the initial velocity, initial pressure),
``run`` chains time steps (``dt -> rhs/solve/pred/corr -> div -> pinit ->
psolve -> sgrad -> psolved -> pgrad``) with the pressure Poisson solve on the
context's CG system, and ``div``/``grad``/``vgrad``/``flux``/``rhs`` are the
``chorin::`` passes (src/Physics/Chorin.hpp:19-70) as drop-ins on host arrays.

:func:`operators` is the host side that produces the operator and BC arrays
from a mesh the way ``ChoCG::feop``/``setupDirBC``/``streamable`` and
``ChoCG::prelhs`` do (with plain edges in place of superedge groups), using
the C++ setup routines of libxg.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import riecg as _r
from .lib import ChocgParams, Context, f64, i32, p, u64

FLUX = {"damp2": 0, "damp4": 1}
PC = {"none": 0, "jacobi": 1, "factor": 2}


def _nodes(bface, sets):
    out = [np.unique(bface[s]) for s in sets if s in bface]
    return np.unique(np.concatenate(out)) if out else np.zeros(0, np.int64)


def operators(mesh, sym_sets=(), noslip_sets=(), dir_bcs=(), pdir_bcs=(), hydrostat=None,
              renumber=True):
    """ChoCG operators for a mesh dict (see xyst_gb300.mesh).

    dir_bcs: (side set, mask[3], value[3]) velocity Dirichlet entries
      (bc_dir/bc_dirval; a node on several sets takes the union of the masks
      and the values of the last set, ChoCG::setupDirBC,
      src/Inciter/ChoCG.cpp:207-275);
    pdir_bcs: (side set, value) pressure Dirichlet entries for the initial
      solves (pressure.bc_dir with its values);
    hydrostat: input id of a node pinned to pressure 0 unless already
      Dirichlet (pressure.hydrostat, src/Inciter/ChoCG.cpp:1095-1106).
    Returns the (possibly renumbered) mesh with vol, edges, dint (5 per
    edge), tri, the BC lists in local ids and the pressure matrix."""
    import scipy  # noqa: F401  (the pressure matrix comes back as CSR arrays)
    from . import cg as _cg

    coord = f64(mesh["coord"])
    inpoel = np.asarray(mesh["inpoel"], dtype=np.int64)
    bface = dict(mesh["bface"])
    npoin = coord.shape[1]
    new_of_old = None
    gid = None
    if renumber:
        new_of_old = _r.rcm(inpoel, npoin)
        c2 = np.empty_like(coord)
        c2[:, new_of_old] = coord
        coord = c2
        inpoel = new_of_old[inpoel]
        bface = {s: new_of_old[f] for s, f in bface.items()}
        gid = np.empty(npoin, np.int64)
        gid[new_of_old] = np.arange(npoin)
    used = (set(sym_sets) | set(noslip_sets) | {s for s, *_ in dir_bcs} |
            {s for s, _ in pdir_bcs})
    kept = _r.boundary_sets(bface, used)
    tri = np.concatenate([bface[s] for s in kept]) if kept else np.zeros((0, 3), np.int64)
    vol = _r.volumes(coord, inpoel)
    e, d = _r.edges(coord, inpoel, gid=gid, ncoef=5)
    # velocity Dirichlet: union of masks, values of the last set holding a node
    mask, val = {}, {}
    for s, m3, v3 in dir_bcs:
        for q in _nodes(bface, [s]).tolist():
            mk = mask.setdefault(q, [0, 0, 0])
            for c in range(3):
                if not mk[c]:
                    mk[c] = int(m3[c] != 0)
            val[q] = list(v3)
    dn = np.array(sorted(mask), dtype=np.int64)
    dirbc = (dn, np.array([mask[q] for q in dn.tolist()], dtype=np.int32).reshape(-1, 3),
             np.array([val[q] for q in dn.tolist()], dtype=np.float64).reshape(-1, 3))
    # symmetry: one normal per (node, set), in configured set order
    sn, snv = [], []
    per = {}
    for s in sym_sets:
        if s in bface and s not in per:
            nodes = np.unique(bface[s])
            per[s] = dict(zip(nodes.tolist(), _r.bnorm(coord, bface[s], nodes)))
    for q in sorted(set().union(*[set(v) for v in per.values()]) if per else []):
        for s in sym_sets:
            if s in per and q in per[s]:
                sn.append(q)
                snv.append(per[s][q])
    sym = (np.array(sn, dtype=np.int64), np.array(snv, dtype=np.float64).reshape(-1, 3))
    noslip = _nodes(bface, noslip_sets)
    # pressure Dirichlet and hydrostat
    pv = {}
    for s, v in pdir_bcs:
        for q in _nodes(bface, [s]).tolist():
            pv[q] = float(v)
    if hydrostat is not None:
        h = int(new_of_old[hydrostat]) if new_of_old is not None else int(hydrostat)
        pv.setdefault(h, 0.0)
    pn = np.array(sorted(pv), dtype=np.int64)
    pdir = (pn, np.array([pv[q] for q in pn.tolist()], dtype=np.float64))
    ia, ja, a = _cg.pressure_matrix(coord, inpoel)
    return {"coord": coord, "inpoel": inpoel, "bface": bface, "vol": vol, "edges": e, "dint": d,
            "tri": tri, "dir": dirbc, "sym": sym, "noslip": noslip, "pdir": pdir,
            "matrix": (ia, ja, a), "new_of_old": new_of_old, "gid": gid}


class ChoCG:
    def __init__(self, ctx: Context, ops, mu=0.0, cfl=0.5, const_dt=0.0, flux="damp2",
                 stab=True, stab2=False, stab2coef=0.2, rk=1, pc="jacobi", ptol=1e-3,
                 pmaxit=10, mixed=False, inner_tol=0.1, guard="reference", matrix=True):
        """ops: :func:`operators` output.  The pressure matrix goes to the
        context's CG system unless matrix is False (already set up).  guard:
        "reference" keeps the reference's absolute (p,q) breakdown test,
        "underflow" lets the FP64 solve run to its relative tolerance.
        inner_tol: residual reduction of the mixed solve's FP32 iteration
        between true-residual replacements (0.1 measured fastest on the 129^3
        Taylor-Green pressure systems; 1e-2 let the FP32 recursion stagnate)."""
        from . import cg as _cg

        self.ctx = ctx
        self.lib = ctx.lib
        coord = f64(ops["coord"])
        self.n = coord.shape[1]
        if matrix:
            self.cg = _cg.ConjugateGradients(ctx, *ops["matrix"])
        prm = ChocgParams(mu, cfl, const_dt, FLUX[flux], int(stab), int(stab2), stab2coef, rk,
                          PC[pc], ptol, pmaxit, int(mixed), inner_tol,
                          {"reference": 0, "underflow": 1}[guard])
        self.prm = prm
        e = u64(ops["edges"]).reshape(-1)
        dd = f64(ops["dint"]).reshape(-1)
        tri = u64(ops["tri"]).reshape(-1)
        v = f64(ops["vol"])
        self._keep = [coord, e, dd, tri, v]
        ctx.check(self.lib.xg_chocg_setup(ctx.h, C.byref(prm), self.n, p(coord), p(v), 0, None,
                                          None, 0, None, None, e.size // 2, p(e), p(dd),
                                          tri.size // 3, p(tri) if tri.size else None))
        self.set_bc(ops["dir"], ops["sym"], ops["noslip"], ops["pdir"])

    def set_bc(self, dirbc, sym, noslip, pdir):
        dn, dm, dv = u64(dirbc[0]), i32(dirbc[1]), f64(dirbc[2])
        sn, snv = u64(sym[0]), f64(sym[1])
        ns = u64(noslip)
        pn, pv = u64(pdir[0]), f64(pdir[1])
        self._bc = [dn, dm, dv, sn, snv, ns, pn, pv]
        z = lambda a: p(a) if a.size else None  # noqa: E731
        self.ctx.check(self.lib.xg_chocg_set_bc(self.ctx.h, dn.size, z(dn), z(dm), z(dv), sn.size,
                                                z(sn), z(snv), ns.size, z(ns), pn.size, z(pn),
                                                z(pv)))

    def set_state(self, u, pr=None, t=0.0):
        u = f64(u)
        pp = None if pr is None else f64(pr)
        self.ctx.check(self.lib.xg_chocg_set_state(self.ctx.h, p(u), p(pp), t))

    def state(self):
        u = np.zeros((self.n, 3))
        pr = np.zeros(self.n)
        t = C.c_double()
        self.ctx.check(self.lib.xg_chocg_get_state(self.ctx.h, p(u), p(pr), C.byref(t)))
        return u, pr, t.value

    def init(self):
        it = C.c_int64()
        self.ctx.check(self.lib.xg_chocg_init(self.ctx.h, C.byref(it)))
        return it.value

    def set_theta(self, theta, inpoel, mom_pc="none", mom_iter=10, mom_tol=1e-3):
        """theta-implicit momentum prediction (the control file's theta and
        momentum solver iter / tol / pc) on the tetrahedra inpoel (ntet, 4)."""
        self._tets = u64(inpoel).reshape(-1)
        self.ctx.check(self.lib.xg_chocg_set_theta(self.ctx.h, float(theta), self._tets.size // 4,
                                                   p(self._tets), 1 if mom_pc == "jacobi" else 0,
                                                   int(mom_iter), float(mom_tol)))

    def momentum_its(self):
        it = C.c_int64()
        self.ctx.check(self.lib.xg_chocg_momentum_its(self.ctx.h, C.byref(it)))
        return it.value

    def run(self, nstep, check=True):
        """Returns (dts, pressure iterations per step, device ms, status)."""
        dts = np.zeros(nstep)
        its = np.zeros(nstep, np.int64)
        ms = C.c_float()
        rc = self.lib.xg_chocg_run(self.ctx.h, nstep, p(dts), p(its), C.byref(ms))
        if check:
            self.ctx.check(rc)
        return dts, its, ms.value, rc

    def field(self, what):
        nc = {0: 3, 1: 3, 2: 9, 3: 1, 4: 1}[what]
        out = np.zeros((self.n, nc)) if nc > 1 else np.zeros(self.n)
        self.ctx.check(self.lib.xg_chocg_fields(self.ctx.h, what, p(out)))
        return out

    # drop-ins for the chorin:: passes (raw weak sums)
    def div(self, U, P, G, dt, stab):
        D = np.zeros(self.n)
        U, P, G = f64(U), f64(P), f64(G)
        self.ctx.check(self.lib.xg_chorin_div(self.ctx.h, p(U), p(P), p(G), dt, int(stab), p(D)))
        return D

    def grad(self, S):
        G = np.zeros((self.n, 3))
        S = f64(S)
        self.ctx.check(self.lib.xg_chorin_grad(self.ctx.h, p(S), p(G)))
        return G

    def vgrad(self, U):
        G = np.zeros((self.n, 9))
        U = f64(U)
        self.ctx.check(self.lib.xg_chorin_vgrad(self.ctx.h, p(U), p(G)))
        return G

    def flux(self, U, G):
        F = np.zeros((self.n, 3))
        U, G = f64(U), f64(G)
        self.ctx.check(self.lib.xg_chorin_flux(self.ctx.h, p(U), p(G), p(F)))
        return F

    def rhs(self, P, U, G):
        R = np.zeros((self.n, 3))
        P, U, G = f64(P), f64(U), f64(G)
        self.ctx.check(self.lib.xg_chorin_rhs(self.ctx.h, p(P), p(U), p(G), p(R)))
        return R


def taylor_green(coord):
    """Taylor-Green vortex on [0, 2 pi]^3 mapped to the unit cube:
    u = sin x cos y cos z, v = -cos x sin y cos z, w = 0 (x = 2 pi X)."""
    X, Y, Z = 2 * np.pi * np.asarray(coord)
    u = np.zeros((X.size, 3))
    u[:, 0] = np.sin(X) * np.cos(Y) * np.cos(Z)
    u[:, 1] = -np.cos(X) * np.sin(Y) * np.cos(Z)
    return u
