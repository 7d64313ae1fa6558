"""RieCG hot path on the GPU, behind the reference's own function boundaries.

:class:`RieCG` mirrors what the reference's RieCG chare calls
(src/Inciter/RieCG.cpp): ``grad`` is ``riemann::grad``, ``rhs`` is
``riemann::rhs``, ``bc`` is ``RieCG::BC``, ``dt`` is ``RieCG::dt``, ``stage``
is one ``grad -> rhs -> solve`` pass and ``run`` chains whole time steps on the
device.  Arrays use the reference layouts: U is (npoin, 5) node-major, G is
(npoin, 15), superedges are the three ``m_dsupedge``/``m_dsupint`` groups.

:func:`operators` is the host side that produces those operator arrays from a
mesh the way ``RieCG::feop``/``setupBC``/``streamable`` do (with edges in
place of tet/triangle superedge groups), using the C++ setup routines of
libxg.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import Context, RiecgParams, f64, i32, load, p, u64, u8

# problems with a manufactured source term (enum xg_source)
SOURCES = {"none": 0, "taylor_green": 1, "vortical_flow": 2, "nonlinear_energy_growth": 3,
           "rayleigh_taylor": 4}

FLUX = {"rusanov": 0, "hllc": 1}
PRECISION = {"fp64": 0, "fp32": 1}


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


# ---------------------------------------------------------------- host setup

def rcm(inpoel, npoin):
    lib = load()
    ip = u64(inpoel)
    out = np.zeros(npoin, np.uint64)
    _check(lib.xg_mesh_rcm(npoin, ip.shape[0], p(ip), p(out)), "xg_mesh_rcm")
    return out.astype(np.int64)


def volumes(coord, inpoel):
    lib = load()
    c = f64(coord)
    ip = u64(inpoel)
    v = np.zeros(c.shape[1])
    rc = lib.xg_mesh_vol(c.shape[1], p(c), ip.shape[0], p(ip), p(v))
    if rc != 0:
        raise ValueError("Element Jacobian non-positive")
    return v


def edges(coord, inpoel, gid=None, ncoef=3):
    lib = load()
    c = f64(coord)
    ip = u64(inpoel)
    g = None if gid is None else u64(gid)
    ne = C.c_int64()
    _check(lib.xg_mesh_edges(c.shape[1], p(c), ip.shape[0], p(ip), p(g), ncoef, 0, C.byref(ne),
                             None, None), "xg_mesh_edges")
    e = np.zeros((ne.value, 2), np.uint64)
    d = np.zeros((ne.value, ncoef))
    _check(lib.xg_mesh_edges(c.shape[1], p(c), ip.shape[0], p(ip), p(g), ncoef, ne.value,
                             C.byref(ne), p(e), p(d)), "xg_mesh_edges")
    return e.astype(np.int64), d


def bnorm(coord, faces, nodes):
    lib = load()
    c = f64(coord)
    f = u64(faces)
    nd = u64(nodes)
    out = np.zeros((nd.size, 3))
    _check(lib.xg_mesh_bnorm(c.shape[1], p(c), f.shape[0], p(f), nd.size, p(nd), p(out)),
           "xg_mesh_bnorm")
    return out


def boundary_sets(bface, used):
    """Side sets whose faces enter the boundary integrals.

    The reference matches the configured side sets first against the side-set
    node lists and only when that finds none against the face lists
    (``bcs_set = matchsets(bnode) || matchsets(bface)``,
    src/Inciter/Transporter.cpp:347-350).  Every side set of an ExodusII mesh
    has a node list, so as soon as one configured set exists the face lists
    are left unfiltered and all side sets contribute boundary faces; with no
    configured set present none do."""
    if any(s in bface for s in used):
        return sorted(bface)
    return []


def operators(mesh, sym_sets=(), far_sets=(), dir_sets=(), pre_sets=(), extra_sets=(),
              renumber=True):
    """RieCG operators for a mesh dict (see xyst_gb300.mesh).

    Boundary triangles come from the side sets :func:`boundary_sets` selects.
    Returns a dict with the (possibly renumbered) mesh and: vol, edges, dint,
    tri, besym, sym (nodes, norms), far (nodes, norms), dirnodes, prenodes,
    new_of_old and gid (the input id of each local node; None without
    renumbering).
    """
    coord = f64(mesh["coord"])
    inpoel = np.asarray(mesh["inpoel"], dtype=np.int64)
    bface = dict(mesh["bface"])
    npoin = coord.shape[1]
    new_of_old = None
    gid = None
    if renumber:
        new_of_old = rcm(inpoel, npoin)
        c2 = np.empty_like(coord)
        c2[:, new_of_old] = coord
        coord = c2
        inpoel = new_of_old[inpoel]
        bface = {s: new_of_old[f] for s, f in bface.items()}
        gid = np.empty(npoin, np.int64)  # caller's (global) id of each local node
        gid[new_of_old] = np.arange(npoin)
    used = set(sym_sets) | set(far_sets) | set(dir_sets) | set(pre_sets) | set(extra_sets)
    kept = boundary_sets(bface, used)
    tri = (np.concatenate([bface[s] for s in kept]) if kept else np.zeros((0, 3), np.int64))
    vol = volumes(coord, inpoel)
    # edges are oriented from the smaller to the larger global id, as the
    # reference keys its edge integrals (src/Inciter/RieCG.cpp:369-380)
    e, d = edges(coord, inpoel, gid=gid)

    def nodes_of(sets):
        out = set()
        for s in sets:
            if s in bface:
                out.update(np.unique(bface[s]).tolist())
        return out

    far = nodes_of(far_sets)
    sym = nodes_of(sym_sets) - far
    besym = np.isin(tri, np.fromiter(sym, dtype=np.int64, count=len(sym))).astype(np.uint8)
    # per set normals, one entry per (node, set) in configured set order
    norms = {}
    for s in list(sym_sets) + list(far_sets):
        if s in bface and s not in norms:
            sn = np.unique(bface[s])
            norms[s] = (sn, bnorm(coord, bface[s], sn))

    def entries(nodeset, sets):
        nodes, nv = [], []
        for s in sets:
            if s not in norms:
                continue
            sn, nn = norms[s]
            m = np.isin(sn, np.fromiter(nodeset, dtype=np.int64, count=len(nodeset)))
            nodes.append(sn[m])
            nv.append(nn[m])
        if not nodes:
            return np.zeros(0, np.int64), np.zeros((0, 3))
        nodes = np.concatenate(nodes)
        nv = np.concatenate(nv)
        order = np.argsort(nodes, kind="stable")
        return nodes[order], nv[order]

    return {"coord": coord, "inpoel": inpoel, "bface": bface, "vol": vol, "edges": e, "dint": d,
            "tri": tri, "besym": besym, "sym": entries(sym, sym_sets),
            "far": entries(far, far_sets),
            "dirnodes": np.array(sorted(nodes_of(dir_sets)), dtype=np.int64),
            "prenodes": np.array(sorted(nodes_of(pre_sets)), dtype=np.int64),
            "new_of_old": new_of_old, "gid": gid, "symset": sym}


# ---------------------------------------------------------------- device path

class RieCG:
    def __init__(self, ctx: Context, coord, vol, dsupedge, dsupint, triinpoel, besym,
                 gamma=1.4, flux="rusanov", stab2=False, stab2coef=0.2, cfl=0.5, const_dt=0.0,
                 precision="fp64"):
        """dsupedge/dsupint: three groups (tets, triangles, edges); a group may
        be None.  Ids are zero-based local node ids."""
        self.ctx = ctx
        self.lib = ctx.lib
        coord = f64(coord)
        self.n = coord.shape[1]
        prm = RiecgParams(gamma, FLUX[flux], int(stab2), stab2coef, cfl, const_dt,
                          PRECISION[precision])
        sizes = (4, 3, 2)
        ints = (18, 9, 3)
        grp = []
        for k in range(3):
            if dsupedge[k] is None or len(dsupedge[k]) == 0:
                grp += [0, None, None]
            else:
                ids = u64(dsupedge[k]).reshape(-1)
                it = f64(dsupint[k]).reshape(-1)
                cnt = ids.size // sizes[k]
                assert it.size == cnt * ints[k], "superedge integral size mismatch"
                grp += [cnt, ids, it]
        tri = u64(triinpoel).reshape(-1)
        bs = u8(besym).reshape(-1)
        v = f64(vol)
        self._keep = [coord, v, tri, bs] + [g for g in grp if isinstance(g, np.ndarray)]
        args = [ctx.h, C.byref(prm), self.n, p(coord), p(v)]
        for k in range(3):
            cnt, ids, it = grp[3 * k:3 * k + 3]
            args += [cnt, p(ids), p(it)]
        args += [tri.size // 3, p(tri), p(bs)]
        ctx.check(self.lib.xg_riecg_setup(*args))

    def set_bc(self, sym=None, far=None, far_state=None, dir=None, pre=None):
        """sym/far: (nodes, normals); dir: (nodes, mask (n,5), values (n,5));
        pre: (nodes, values (n,2)); far_state: (density, u, v, w, pressure)."""
        def two(x, w):
            if x is None:
                return 0, None, None
            n = u64(x[0])
            return n.size, n, f64(x[1]).reshape(-1)
        ns, sn, sv = two(sym, 3)
        nf, fn, fv = two(far, 3)
        f5 = f64(far_state if far_state is not None else (1, 0, 0, 0, 1))
        if dir is None:
            nd, dn, dm, dv = 0, None, None, None
        else:
            dn = u64(dir[0])
            nd = dn.size
            dm = i32(dir[1]).reshape(-1)
            dv = f64(dir[2]).reshape(-1)
        npr, pn, pv = two(pre, 2)
        self._bc = [sn, sv, fn, fv, f5, dn, dm, dv, pn, pv]
        self.ctx.check(self.lib.xg_riecg_set_bc(self.ctx.h, ns, p(sn), p(sv), nf, p(fn), p(fv),
                                                p(f5), nd, p(dn), p(dm), p(dv), npr, p(pn),
                                                p(pv)))

    def grad(self, U):
        U = f64(U)
        G = np.zeros((self.n, 15))
        self.ctx.check(self.lib.xg_riecg_grad(self.ctx.h, p(U), p(G)))
        return G

    def rhs(self, G, U):
        G = f64(G)
        U = f64(U)
        R = np.zeros((self.n, 5))
        self.ctx.check(self.lib.xg_riecg_rhs(self.ctx.h, p(G), p(U), p(R)))
        return R

    def set_source(self, problem, prm=None):
        """The manufactured source of riemann::rhs (SOURCES names the
        problems; src/Physics/Riemann.cpp:880-907) with the control-file
        parameters prm = alpha, beta[3], kappa, r0, p0, ce, evaluated at the
        context's time (the start of each step)."""
        self._src = None if prm is None else f64(np.asarray(prm, dtype=np.float64).reshape(8))
        self.ctx.check(self.lib.xg_riecg_set_source(self.ctx.h, SOURCES[problem],
                                                    None if self._src is None else p(self._src)))

    def rhs_coloured(self, G, U):
        """rhs() by the edge-coloured scatter (FP32 mode): (R, colours)."""
        G = f64(G)
        U = f64(U)
        R = np.zeros((self.n, 5))
        k = C.c_int(0)
        self.ctx.check(self.lib.xg_riecg_rhs_coloured(self.ctx.h, p(G), p(U), p(R), C.byref(k)))
        return R, k.value

    def set_state(self, U, t=0.0):
        U = f64(U)
        assert U.shape == (self.n, 5)
        self.ctx.check(self.lib.xg_riecg_set_state(self.ctx.h, p(U), t))

    def state(self, out=None):
        """(U, t); U node-major (n, 5).  ``out``: a C-contiguous float64
        (n, 5) array to download into (pinned host memory for a DMA copy)."""
        if out is None:
            U = np.zeros((self.n, 5))
        else:
            if out.shape != (self.n, 5) or out.dtype != np.float64 or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float64 (n, 5) array")
            U = out
        t = C.c_double()
        self.ctx.check(self.lib.xg_riecg_get_state(self.ctx.h, p(U), C.byref(t)))
        return U, t.value

    def bc(self):
        self.ctx.check(self.lib.xg_riecg_bc(self.ctx.h))

    def dt(self):
        d = C.c_double()
        self.ctx.check(self.lib.xg_riecg_dt(self.ctx.h, C.byref(d)))
        return d.value

    def stage(self, stage, dt):
        self.ctx.check(self.lib.xg_riecg_stage(self.ctx.h, stage, dt))

    def run(self, nstep):
        dts = np.zeros(nstep)
        ms = C.c_float()
        self.ctx.check(self.lib.xg_riecg_run(self.ctx.h, nstep, p(dts), C.byref(ms)))
        return dts, ms.value

    def profile(self, enable=True):
        self.ctx.check(self.lib.xg_riecg_profile(self.ctx.h, int(enable)))

    def kernel_times(self):
        n = C.c_int()
        cap = 16
        names = (C.c_char_p * cap)()
        ms = np.zeros(cap)
        la = np.zeros(cap, np.int64)
        self.ctx.check(self.lib.xg_riecg_kernel_times(self.ctx.h, cap, names, p(ms), p(la),
                                                      C.byref(n)))
        return {names[i].decode(): (float(ms[i]), int(la[i])) for i in range(n.value)}


def from_operators(ctx, ops, **kw):
    """Build a RieCG from :func:`operators` output (all edges as the edge group)."""
    r = RieCG(ctx, ops["coord"], ops["vol"], [None, None, ops["edges"]],
              [None, None, ops["dint"]], ops["tri"], ops["besym"], **kw)
    sym = ops["sym"] if ops["sym"][0].size else None
    far = ops["far"] if ops["far"][0].size else None
    if sym is not None or far is not None:
        r.set_bc(sym=sym, far=far)
    return r
