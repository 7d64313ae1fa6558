"""On-disk formats around the path: the diagnostics text file and ExodusII
(NetCDF classic) field output.

* :class:`DiagWriter` writes the reference's ``diag`` file
  (tk::DiagWriter, src/IO/DiagWriter.cpp:25-101): a ``#``-prefixed header of
  numbered column names, then one row per diagnostics step: the iteration in
  10 columns, t, dt and the norms in columns of width max(20, precision + 8),
  scientific notation by default.
* :func:`riecg_diagnostics` / :func:`chocg_diagnostics` are the norms the
  reference puts in those rows (NodeDiagnostics::compute/precompute,
  src/Inciter/NodeDiagnostics.cpp:46-246, finished by
  Transporter::diagnostics/prediagnostics, src/Inciter/Transporter.cpp:
  1436-1575): volume-weighted L2 norms sqrt(sum_i f_i^2 V_i / V) of the
  solution and of its change over the last step.
* :func:`write_exo` writes a tetrahedral mesh, its side sets and node fields
  over time as an ExodusII file (the layout tk::ExodusIIMeshWriter produces,
  src/IO/ExodusIIMeshWriter.cpp), readable by :func:`xyst_gb300.mesh.read_exo`
  and by ExodusII tools.
"""

from __future__ import annotations

import numpy as np

from .mesh import _EXO_TET_SIDE


class DiagWriter:
    def __init__(self, path: str, names, precision: int = 12, fmt: str = "scientific",
                 append: bool = False):
        if fmt not in ("scientific", "fixed"):
            raise ValueError("Text floating-point format not recognized.")
        self.precision = int(precision)
        self.width = max(20, self.precision + 8)
        self.fmt = "e" if fmt == "scientific" else "f"
        self.f = open(path, "a" if append else "w")
        if not append:
            head = "#" + "1:it".rjust(9) + "2:t".rjust(self.width) + "3:dt".rjust(self.width)
            for k, n in enumerate(names, start=4):
                head += f"{k}:{n}".rjust(self.width)
            self.f.write(head + "\n")

    def write(self, it: int, t: float, dt: float, diag) -> int:
        num = f"{{:.{self.precision}{self.fmt}}}"
        row = str(int(it)).rjust(10) + num.format(t).rjust(self.width) + \
            num.format(dt).rjust(self.width)
        for d in diag:
            row += num.format(float(d)).rjust(self.width)
        self.f.write(row + "\n")
        self.f.flush()
        return len(diag)

    def close(self):
        self.f.close()


def read_diag(path: str) -> np.ndarray:
    """Rows of a diag file as floats (the header skipped)."""
    rows = [ln.split() for ln in open(path) if ln.strip() and not ln.startswith("#")]
    return np.array([[float(x) for x in r] for r in rows])


RIECG_DIAG = ["L2(r)", "L2(ru)", "L2(rv)", "L2(rw)", "L2(rE)",
              "L2(dr)", "L2(dru)", "L2(drv)", "L2(drw)", "L2(drE)"]
CHOCG_DIAG = ["L2(p)", "L2(u)", "L2(v)", "L2(w)", "L2(dp)", "L2(du)", "L2(dv)", "L2(dw)"]


def _l2(f, vol, vt):
    f = np.asarray(f, dtype=np.float64)
    if f.ndim == 1:
        return np.sqrt((f * f * vol).sum() / vt)
    return np.sqrt((f * f * vol[:, None]).sum(0) / vt)


def riecg_diagnostics(U, Un, vol):
    """L2 of the conserved variables and of their change over the step."""
    vt = float(np.sum(vol))
    return np.concatenate([_l2(U, vol, vt), _l2(np.asarray(U) - np.asarray(Un), vol, vt)])


def chocg_diagnostics(u, un, p, dp, vol):
    """L2 of the pressure and velocity, of the pressure increment and of the
    velocity change over the step."""
    vt = float(np.sum(vol))
    return np.concatenate([[_l2(p, vol, vt)], _l2(u, vol, vt), [_l2(dp, vol, vt)],
                           _l2(np.asarray(u) - np.asarray(un), vol, vt)])


def _tet_sides(inpoel, tri):
    """(element, side) pairs, both one-based, of boundary triangles on tets."""
    inpoel = np.asarray(inpoel, dtype=np.int64)
    lookup = {}
    for side in range(4):
        faces = np.sort(inpoel[:, _EXO_TET_SIDE[side]], axis=1)
        for e, f in enumerate(faces.tolist()):
            lookup.setdefault(tuple(f), (e + 1, side + 1))
    out = np.zeros((len(tri), 2), dtype=np.int64)
    for k, f in enumerate(np.sort(np.asarray(tri, dtype=np.int64), axis=1).tolist()):
        out[k] = lookup[tuple(f)]
    return out


def _chars(strings, width):
    a = np.zeros((len(strings), width), dtype="S1")
    for i, s in enumerate(strings):
        b = s.encode()[:width]
        a[i, :len(b)] = [bytes([c]) for c in b]
    return a


def write_exo(path: str, mesh: dict, steps, title: str = "xyst_gb300"):
    """mesh: coord (3, N), inpoel (T, 4) zero-based, optional bface
    {side set id: (k, 3) triangles}; steps: list of (time, {name: (N,)
    array}) with the same names every step."""
    from scipy.io import netcdf_file

    coord = np.asarray(mesh["coord"], dtype=np.float64)
    inpoel = np.asarray(mesh["inpoel"], dtype=np.int64)
    bface = mesh.get("bface", {}) or {}
    names = list(steps[0][1].keys()) if steps else []
    f = netcdf_file(path, "w", version=2)
    f.api_version = np.float32(5.22)
    f.version = np.float32(5.22)
    f.floating_point_word_size = np.int32(8)
    f.file_size = np.int32(1)
    f.title = title
    f.createDimension("time_step", None)  # the record dimension comes first here
    f.createDimension("len_string", 33)
    f.createDimension("len_line", 81)
    f.createDimension("four", 4)
    f.createDimension("len_name", 33)
    f.createDimension("num_dim", 3)
    f.createDimension("num_nodes", coord.shape[1])
    f.createDimension("num_elem", inpoel.shape[0])
    f.createDimension("num_el_blk", 1)
    f.createDimension("num_el_in_blk1", inpoel.shape[0])
    f.createDimension("num_nod_per_el1", 4)
    if bface:
        f.createDimension("num_side_sets", len(bface))
    if names:
        f.createDimension("num_nod_var", len(names))
    tw = f.createVariable("time_whole", "d", ("time_step",))
    ebs = f.createVariable("eb_status", "i", ("num_el_blk",))
    ebs[:] = [1]
    ebp = f.createVariable("eb_prop1", "i", ("num_el_blk",))
    ebp[:] = [1]
    ebp.name = "ID"
    for k, x in enumerate(("coordx", "coordy", "coordz")):
        v = f.createVariable(x, "d", ("num_nodes",))
        v[:] = coord[k]
    cn = f.createVariable("coor_names", "c", ("num_dim", "len_name"))
    cn[:] = _chars(["x", "y", "z"], 33)
    conn = f.createVariable("connect1", "i", ("num_el_in_blk1", "num_nod_per_el1"))
    conn[:] = (inpoel + 1).astype(np.int32)
    conn.elem_type = "TETRA4"
    if bface:
        sids = sorted(bface)
        sst = f.createVariable("ss_status", "i", ("num_side_sets",))
        sst[:] = [1] * len(sids)
        ssp = f.createVariable("ss_prop1", "i", ("num_side_sets",))
        ssp[:] = sids
        ssp.name = "ID"
        for k, s in enumerate(sids, start=1):
            es = _tet_sides(inpoel, bface[s])
            f.createDimension(f"num_side_ss{k}", es.shape[0])
            ve = f.createVariable(f"elem_ss{k}", "i", (f"num_side_ss{k}",))
            ve[:] = es[:, 0].astype(np.int32)
            vs = f.createVariable(f"side_ss{k}", "i", (f"num_side_ss{k}",))
            vs[:] = es[:, 1].astype(np.int32)
    if names:
        nn = f.createVariable("name_nod_var", "c", ("num_nod_var", "len_name"))
        nn[:] = _chars(names, 33)
        vals = [f.createVariable(f"vals_nod_var{k + 1}", "d", ("time_step", "num_nodes"))
                for k in range(len(names))]
        for ts, (t, flds) in enumerate(steps):
            tw[ts] = t
            for k, nm in enumerate(names):
                vals[k][ts, :] = np.asarray(flds[nm], dtype=np.float64)
    f.close()


def read_exo_fields(path: str):
    """Times, field names and the (steps, N) arrays of an ExodusII file."""
    from scipy.io import netcdf_file

    f = netcdf_file(path, "r", mmap=False)
    v = f.variables
    names = ["".join(c.decode() for c in row if c) for row in v["name_nod_var"][:]] \
        if "name_nod_var" in v else []
    times = np.array(v["time_whole"][:], dtype=np.float64)
    fields = {nm: np.array(v[f"vals_nod_var{k + 1}"][:], dtype=np.float64)
              for k, nm in enumerate(names)}
    f.close()
    return times, names, fields
