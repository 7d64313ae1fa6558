"""Formats around the path (CPU): the diag text file and ExodusII output.

The diag file is checked against the reference's own baseline of the RieCG
Sod regression (tests/regression/inciter/RieCG/Sod/diag.std): the norms the
oracle's ten Sod steps produce, written by DiagWriter and read back, agree
with the baseline within its numdiff tolerances.  The ExodusII writer is
checked by a round trip through the same reader that reads the reference's
meshes and baselines."""

import numpy as np

import oracle
from common import sod_ic, sod_mesh
from xyst_gb300 import io, mesh


def test_diag_file_matches_reference_sod_baseline(tmp_path):
    m, d = sod_mesh("RieCG")
    coord, inpoel = m["coord"], m["inpoel"]
    tri = np.concatenate([m["bface"][s] for s in sorted(m["bface"])])
    v = oracle.vol(coord, inpoel)
    e, de = oracle.domint(coord, inpoel)
    nodes, norms, symset = oracle.sym_bc(coord, m["bface"], [2, 4, 5, 6])
    besym = np.isin(tri, list(symset)).astype(np.uint8)
    o = oracle.RieCG(coord, v, e, de, tri, besym, cfl=0.5)
    o.set_sym(nodes, norms)
    o.set_state(sod_ic(coord))
    o.bc()
    path = str(tmp_path / "diag")
    w = io.DiagWriter(path, io.RIECG_DIAG, precision=8)
    t = 0.0
    for k in range(10):
        Un = o.state()
        dt = o.run(1)[0]
        t += dt
        w.write(k + 1, t, dt, io.riecg_diagnostics(o.state(), Un, v))
    w.close()
    head = open(path).readline()
    assert head.startswith("#     1:it") and "13:L2(drE)" in head
    got = io.read_diag(path)
    exp = d["diag"]
    assert got.shape == exp[:, :13].shape
    tol = np.where(np.arange(13) < 8, np.maximum(2e-4, 1e-5 * np.abs(exp[:, :13])),
                   np.maximum(3e-4, 1e-7 * np.abs(exp[:, :13])))
    assert np.all(np.abs(got - exp[:, :13]) <= tol)


def test_exo_round_trip(tmp_path):
    m = mesh.cube(5, jitter=0.2, seed=3)
    path = str(tmp_path / "out.exo")
    rng = np.random.default_rng(0)
    n = m["coord"].shape[1]
    steps = [(0.0, {"density": rng.random(n), "pressure": rng.random(n)}),
             (0.25, {"density": rng.random(n), "pressure": rng.random(n)})]
    io.write_exo(path, m, steps)
    back = mesh.read_exo(path)
    assert np.array_equal(back["coord"], m["coord"])
    assert np.array_equal(back["inpoel"], m["inpoel"])
    assert sorted(back["bface"]) == sorted(m["bface"])
    for s in m["bface"]:
        a = np.sort(np.sort(back["bface"][s], axis=1), axis=0)
        b = np.sort(np.sort(m["bface"][s], axis=1), axis=0)
        assert np.array_equal(np.unique(a, axis=0), np.unique(b, axis=0))
    times, names, fields = io.read_exo_fields(path)
    assert np.array_equal(times, [0.0, 0.25]) and names == ["density", "pressure"]
    for ts, (_, flds) in enumerate(steps):
        for nm in names:
            assert np.array_equal(fields[nm][ts], flds[nm])
