"""Tetrahedron meshes for the edge-based solvers.

Two sources of meshes:

* :func:`cube` -- a structured unit cube of ``n**3`` nodes, each hexahedral cell
  split into six tetrahedra around its main diagonal (Kuhn split), with
  optional seeded jitter of interior nodes and a seeded relabelling of nodes.
  This is the synthetic stand-in for the cube meshes the solver is benchmarked
  on (``N = n**3``, ``T = 6 (n-1)**3``, ``B = 12 (n-1)**2`` boundary triangles).
* :func:`read_exo` -- reads an ExodusII (NetCDF classic) mesh: coordinates,
  tetrahedra and the triangle faces of its side sets, following how the
  reference's ExodusII reader turns side sets into boundary triangles
  (src/IO/ExodusIIMeshReader.cpp:639-835: triangle-block sides take the
  triangle's own connectivity, tetrahedron sides take the ExodusII face-node
  table).

A mesh is a plain dict: ``coord`` (3, N) float64, ``inpoel`` (T, 4) int64,
``bface`` {side set id: (F, 3) int64 triangles with outward normals}.
"""

from __future__ import annotations

import numpy as np

# ExodusII tetrahedron side -> local nodes, already reordered so that the
# triangle normal (b-a)x(c-a) points out of the element
# (src/Mesh/DerivedData.hpp expofa with the 0,2,1 switch noted at
# src/IO/ExodusIIMeshReader.cpp:807-813).
_EXO_TET_SIDE = np.array([[0, 1, 3], [1, 2, 3], [0, 3, 2], [0, 2, 1]], dtype=np.int64)


def _kuhn_cells(m: int, k0: int = 0, k1: int | None = None) -> np.ndarray:
    """Six tets per cell, ids in the lexicographic (i fastest) numbering;
    only the cell layers k0 <= k < k1 (all by default)."""
    n = m + 1
    k1 = m if k1 is None else k1
    i, j, k = np.meshgrid(np.arange(m), np.arange(m), np.arange(k0, k1), indexing="ij")
    base = (i + n * j + n * n * k).transpose(2, 1, 0).reshape(-1)  # i fastest
    step = {0: 1, 1: n, 2: n * n}
    tets = []
    for a, b, c in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        v0 = base
        v1 = base + step[a]
        v2 = v1 + step[b]
        v3 = v2 + step[c]
        tets.append(np.stack([v0, v1, v2, v3], axis=1))
    # interleave so the six tets of one cell are contiguous
    return np.stack(tets, axis=1).reshape(-1, 4).astype(np.int64)


def _orient_positive(coord: np.ndarray, inpoel: np.ndarray) -> np.ndarray:
    x = coord[:, inpoel]  # (3, T, 4)
    ba = x[:, :, 1] - x[:, :, 0]
    ca = x[:, :, 2] - x[:, :, 0]
    da = x[:, :, 3] - x[:, :, 0]
    J = np.einsum("it,it->t", ba, np.cross(ca.T, da.T).T)
    neg = J < 0
    out = inpoel.copy()
    out[neg, 1], out[neg, 2] = inpoel[neg, 2], inpoel[neg, 1]
    return out


def _cube_faces(n: int) -> dict[int, np.ndarray]:
    """Boundary triangles of the Kuhn-split cube, consistent with its tets.

    On every face plane the quad diagonal joins the corner with the smallest
    coordinate sum to the opposite one, which is the diagonal the six-tet
    split induces.  Side sets: 1 x=0, 2 y=0, 3 z=0, 4 x=1, 5 y=1, 6 z=1.
    """
    m = n - 1
    s = np.arange(m)
    u, v = np.meshgrid(s, s, indexing="ij")
    u = u.reshape(-1)
    v = v.reshape(-1)
    faces = {}
    for sid, (axis, side) in enumerate(((0, 0), (1, 0), (2, 0), (0, 1), (1, 1), (2, 1)), start=1):
        ax = [a for a in range(3) if a != axis]

        def nid(a_val, b_val):
            ijk = [None, None, None]
            ijk[axis] = np.full_like(a_val, side * m)
            ijk[ax[0]] = a_val
            ijk[ax[1]] = b_val
            return ijk[0] + n * ijk[1] + n * n * ijk[2]

        p00 = nid(u, v)
        p10 = nid(u + 1, v)
        p11 = nid(u + 1, v + 1)
        p01 = nid(u, v + 1)
        t1 = np.stack([p00, p10, p11], axis=1)
        t2 = np.stack([p00, p11, p01], axis=1)
        tri = np.concatenate([t1, t2]).astype(np.int64)
        # orientation: (b-a)x(c-a) along ax0 x ax1; make it point outward
        e = np.zeros(3)
        e[ax[0]] = 1
        f = np.zeros(3)
        f[ax[1]] = 1
        nrm = np.cross(e, f)[axis]
        outward = 1.0 if side == 1 else -1.0
        if nrm * outward < 0:
            tri = tri[:, [0, 2, 1]]
        faces[sid] = tri
    return faces


def _cube_coord(n: int, jitter: float, seed: int) -> np.ndarray:
    """Node coordinates of the n**3 cube (lexicographic ids), interior nodes
    jittered by U(-jitter*h, +jitter*h) per coordinate (seeded)."""
    m = n - 1
    h = 1.0 / m
    g = np.arange(n, dtype=np.float64) * h
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    coord = np.stack([X.transpose(2, 1, 0).reshape(-1), Y.transpose(2, 1, 0).reshape(-1),
                      Z.transpose(2, 1, 0).reshape(-1)])
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        idx = np.arange(n)
        I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
        interior = ((I > 0) & (I < m) & (J > 0) & (J < m) & (K > 0) & (K < m))
        interior = interior.transpose(2, 1, 0).reshape(-1)
        d = rng.uniform(-jitter * h, jitter * h, size=(3, int(interior.sum())))
        coord[:, interior] += d
    return coord


def cube_slab(n: int, k0: int, k1: int, jitter: float = 0.0, seed: int = 0) -> dict:
    """The part of ``cube(n, jitter, seed)`` (lexicographic numbering) made of
    the cell layers k0 <= k < k1 along z: a partition of the cube as a
    domain-decomposed solver holds it (the node planes k0..k1, the shared
    planes duplicated in the neighbouring slabs), with the cube's own
    boundary triangles that lie in it.  Node ids are local (global id minus
    k0 * n**2); ``owned`` counts the nodes the slab owns when every shared
    plane belongs to the slab below it (the slabs' counts sum to n**3)."""
    m = n - 1
    if not (0 <= k0 < k1 <= m):
        raise ValueError("slab layers out of range")
    coord = _cube_coord(n, jitter, seed)
    lo, hi = k0 * n * n, (k1 + 1) * n * n
    coord = coord[:, lo:hi].copy()
    inpoel = _orient_positive(coord, _kuhn_cells(m, k0, k1) - lo)
    faces = {}
    for sid, tri in _cube_faces(n).items():
        keep = np.all((tri >= lo) & (tri < hi), axis=1)
        if keep.any():
            faces[sid] = tri[keep] - lo
    bface = faces_from_tets(inpoel, faces)
    owned = (k1 - k0) * n * n + (n * n if k1 == m else 0)
    return {"coord": coord, "inpoel": inpoel, "bface": bface, "h": 1.0 / m, "owned": owned}


def cube(n: int, jitter: float = 0.0, seed: int = 0, numbering: str = "lex",
         perm_seed: int | None = None, faces: bool = True) -> dict:
    """Unit cube [0,1]^3 with n**3 nodes, Kuhn-split into 6 (n-1)**3 tets.

    jitter: interior nodes move by U(-jitter*h, +jitter*h) per coordinate
    (seeded by ``seed``); boundary nodes stay on the cube faces.
    numbering: "lex" (i fastest), "random" (seeded permutation, ``perm_seed``)
    or "rcm" (reverse Cuthill-McKee of the lexicographic graph).
    faces: False leaves the side sets out (bface empty), for uses that need
    the volume mesh only.
    """
    if n < 2:
        raise ValueError("cube needs at least 2 nodes per side")
    m = n - 1
    h = 1.0 / m
    coord = _cube_coord(n, jitter, seed)
    inpoel = _orient_positive(coord, _kuhn_cells(m))
    bface = faces_from_tets(inpoel, _cube_faces(n)) if faces else {}
    mesh = {"coord": coord, "inpoel": inpoel, "bface": bface, "h": h}
    if numbering == "lex":
        return mesh
    if numbering == "random":
        rng = np.random.default_rng(0 if perm_seed is None else perm_seed)
        new_of_old = rng.permutation(coord.shape[1]).astype(np.int64)
    elif numbering == "rcm":
        new_of_old = rcm_order(inpoel, coord.shape[1])
    else:
        raise ValueError(f"unknown numbering {numbering!r}")
    return relabel(mesh, new_of_old)


def relabel(mesh: dict, new_of_old: np.ndarray) -> dict:
    """Renumber nodes: node i becomes new_of_old[i]."""
    N = mesh["coord"].shape[1]
    coord = np.empty_like(mesh["coord"])
    coord[:, new_of_old] = mesh["coord"]
    out = dict(mesh)
    out["coord"] = coord
    out["inpoel"] = new_of_old[mesh["inpoel"]]
    out["bface"] = {s: new_of_old[f] for s, f in mesh["bface"].items()}
    assert len(np.unique(new_of_old)) == N
    return out


def rcm_order(inpoel: np.ndarray, npoin: int) -> np.ndarray:
    """Reverse Cuthill-McKee new-of-old permutation of the node graph."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    i = np.repeat(inpoel, 4, axis=1).reshape(-1)
    j = np.tile(inpoel, (1, 4)).reshape(-1)
    A = sp.coo_matrix((np.ones(i.size, dtype=np.int8), (i, j)), shape=(npoin, npoin)).tocsr()
    order = reverse_cuthill_mckee(A, symmetric_mode=True)  # old ids in new order
    new_of_old = np.empty(npoin, dtype=np.int64)
    new_of_old[order] = np.arange(npoin)
    return new_of_old


def read_exo(path: str) -> dict:
    """Read coordinates, tetrahedra and side-set triangles of an ExodusII file."""
    from scipy.io import netcdf_file

    f = netcdf_file(path, "r", mmap=False)
    v = f.variables
    coord = np.stack([np.asarray(v["coordx"][:], dtype=np.float64),
                      np.asarray(v["coordy"][:], dtype=np.float64),
                      np.asarray(v["coordz"][:], dtype=np.float64)])
    blocks = []
    b = 1
    while f"connect{b}" in v:
        conn = np.asarray(v[f"connect{b}"][:], dtype=np.int64) - 1
        blocks.append(conn)
        b += 1
    tets = [c for c in blocks if c.shape[1] == 4]
    inpoel = np.concatenate(tets) if tets else np.zeros((0, 4), np.int64)
    # file-internal element id -> (kind, block-relative row)
    starts = np.cumsum([0] + [c.shape[0] for c in blocks])
    ssids = np.asarray(v["ss_prop1"][:]) if "ss_prop1" in v else np.zeros(0, np.int64)
    bface = {}
    ntet_before = np.cumsum([0] + [c.shape[0] if c.shape[1] == 4 else 0 for c in blocks])
    for k, sid in enumerate(ssids, start=1):
        if f"elem_ss{k}" not in v:
            continue
        elem = np.asarray(v[f"elem_ss{k}"][:], dtype=np.int64) - 1
        side = np.asarray(v[f"side_ss{k}"][:], dtype=np.int64) - 1
        tri = np.empty((elem.size, 3), dtype=np.int64)
        for t, (e, s) in enumerate(zip(elem, side)):
            blk = int(np.searchsorted(starts, e, side="right") - 1)
            row = e - starts[blk]
            conn = blocks[blk]
            if conn.shape[1] == 3:
                tri[t] = conn[row]
            else:
                tri[t] = conn[row][_EXO_TET_SIDE[s]]
        bface[int(sid)] = tri
    f.close()
    return {"coord": coord, "inpoel": inpoel, "bface": faces_from_tets(inpoel, bface)}


def faces_from_tets(inpoel: np.ndarray, bface: dict) -> dict:
    """Re-derive side-set triangles from the tetrahedra, as the reference's
    partitioner does (src/Inciter/Partitioner.cpp:578-587): every tet, in
    order, offers its faces {t0,t2,t1}, {t0,t1,t3}, {t0,t3,t2}, {t1,t2,t3}
    (outward for positive tets); a face found (in any node order) in a side
    set is appended to that set with the tet's node order.  The triangle node
    order matters: the boundary term of the gradient pairs node j's value with
    normal component j (src/Physics/Riemann.cpp:347-358)."""
    inpoel = np.asarray(inpoel, dtype=np.int64)
    key_of = {}
    for s in sorted(bface):
        for f in np.asarray(bface[s], dtype=np.int64):
            key_of[tuple(sorted(f.tolist()))] = s
    local = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]])
    faces = inpoel[:, local]  # (T, 4, 3)
    skey = np.sort(faces, axis=2).reshape(-1, 3)
    flat = faces.reshape(-1, 3)
    out = {s: [] for s in bface}
    # only boundary candidates: faces whose sorted key is in the side sets
    keys = np.array(list(key_of.keys()), dtype=np.int64) if key_of else np.zeros((0, 3), np.int64)
    if keys.size:
        big = int(max(inpoel.max(), keys.max())) + 1
        enc = (skey[:, 0] * big + skey[:, 1]) * big + skey[:, 2]
        kenc = (keys[:, 0] * big + keys[:, 1]) * big + keys[:, 2]
        hit = np.nonzero(np.isin(enc, kenc))[0]
        for i in hit:
            s = key_of[tuple(skey[i].tolist())]
            out[s].append(flat[i])
    return {s: (np.array(v, dtype=np.int64).reshape(-1, 3)) for s, v in out.items()}


def counts(n: int) -> dict:
    """Closed-form sizes of the Kuhn-split cube with n nodes per side."""
    m = n - 1
    return {"N": n ** 3, "E": 3 * m * n * n + 3 * m * m * n + m ** 3, "T": 6 * m ** 3,
            "B": 12 * m * m}
