"""ChoCG (projection scheme) on the GPU against the oracle and the
reference's ChoCG regression baselines.  FP64 throughout; node-owned gathers
sum each node's edges in neighbour order, so results agree with the oracle up
to summation order (drop-ins 1e-12 relative; whole runs, whose pressure
solves amplify rounding by the condition number, 1e-9)."""

import numpy as np
import pytest

import oracle
from common import chocg_mesh
from gpu_util import ctx, relerr
from test_chocg_oracle import FIELD_TOL, _by_coord
from xyst_gb300 import chocg, io, mesh

pytestmark = pytest.mark.gpu


def _cube_ops(n=9, seed=1):
    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed + 3)
    return chocg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], hydrostat=0)


def same_its(a, b):
    """Pressure-solve iteration counts agree (negated counts: stopped short)."""
    return (a > 0) == (b > 0) and abs(abs(a) - abs(b)) <= 1


def _oracle(ops, **kw):
    ia, ja, a = ops["matrix"]
    o = oracle.ChoCG(ops["coord"], ops["vol"], ops["edges"], ops["dint"], ops["tri"], ia, ja, a,
                     **kw)
    o.set_bc(dir=ops["dir"], sym=ops["sym"], noslip=ops["noslip"], pdir=ops["pdir"])
    return o


@pytest.mark.parametrize("flux,mu", [("damp2", 0.0), ("damp4", 0.01)])
def test_dropins(flux, mu):
    ops = _cube_ops()
    n = ops["coord"].shape[1]
    rng = np.random.default_rng(3)
    U, P = rng.standard_normal((n, 3)), rng.standard_normal(n)
    PG, G = rng.standard_normal((n, 3)), rng.standard_normal((n, 9))
    d = chocg.ChoCG(ctx(), ops, mu=mu, flux=flux)
    o = _oracle(ops, mu=mu, flux=flux)
    for stab in (False, True):
        assert relerr(d.div(U, P, PG, 2.3e-2, stab), o.div(U, P, PG, 2.3e-2, stab)) < 1e-12
    assert relerr(d.grad(P), o.vgrad(P[:, None], 1)) < 1e-12
    assert relerr(d.vgrad(U), o.vgrad(U, 3)) < 1e-12
    assert relerr(d.flux(U, G), o.flux(U, G)) < 1e-12
    assert relerr(d.rhs(P, U, G), o.rhs(U, G, P)) < 1e-12


@pytest.mark.parametrize("flux,rk", [("damp2", 1), ("damp4", 1), ("damp2", 3)])
def test_run_matches_oracle(flux, rk):
    """Taylor-Green vortex with symmetry on all faces and the hydrostat node:
    start-up and six steps, pressure PCG to 1e-10 (iteration counts within one
    of the oracle's, including the solves the (p,q) breakdown guard ends)."""
    ops = _cube_ops(11)
    kw = dict(mu=0.01, cfl=0.5, flux=flux, rk=rk, pc="jacobi", ptol=1e-10, pmaxit=2000)
    d = chocg.ChoCG(ctx(), ops, **kw)
    o = _oracle(ops, **kw)
    u0 = chocg.taylor_green(ops["coord"])
    d.set_state(u0)
    o.set_state(u0, np.zeros(u0.shape[0]))
    assert same_its(d.init(), o.init())
    dts, its, _, _ = d.run(6)
    for k in range(6):
        dto, ito = o.step()
        assert abs(dts[k] / dto - 1) < 1e-12
        assert same_its(its[k], ito)
    u, p, _ = d.state()
    assert relerr(u, o.get(0)) < 1e-9
    assert relerr(p, o.get(2)) < 1e-9
    assert relerr(d.field(4), o.get(6)) < 1e-8


@pytest.mark.parametrize("mom_pc,mom_iter,mom_tol,rk", [("jacobi", 200, 1e-10, 1),
                                                          ("none", 10, 1e-3, 3)])
def test_theta_implicit_matches_oracle(mom_pc, mom_iter, mom_tol, rk):
    """theta-implicit momentum prediction (theta = 0.5): the last stage
    solves -(M/dt + theta mu K) du = R on a second CG system of 3n rows,
    warm-started from the previous increment; converged (Jacobi, 1e-10) and
    with the reference's defaults (no preconditioner, 10 iterations, 1e-3,
    stopping at the limit).  Four steps against the oracle: dt, pressure and
    momentum iteration counts, fields."""
    ops = _cube_ops(9)
    kw = dict(mu=0.05, cfl=0.5, flux="damp2", rk=rk, pc="jacobi", ptol=1e-10, pmaxit=2000)
    d = chocg.ChoCG(ctx(), ops, **kw)
    o = _oracle(ops, **kw)
    for s in (d, o):
        s.set_theta(0.5, ops["inpoel"], mom_pc=mom_pc, mom_iter=mom_iter, mom_tol=mom_tol)
    u0 = chocg.taylor_green(ops["coord"])
    d.set_state(u0)
    o.set_state(u0, np.zeros(u0.shape[0]))
    assert same_its(d.init(), o.init())
    dts, its, _, _ = d.run(4)
    for k in range(4):
        dto, ito = o.step()
        assert abs(dts[k] / dto - 1) < 1e-12
        assert same_its(its[k], ito)
    assert same_its(d.momentum_its(), o.momentum_its())
    u, p, _ = d.state()
    assert relerr(u, o.get(0)) < 1e-9
    assert relerr(p, o.get(2)) < 1e-9


def test_theta_implicit_lid_dirichlet_rows():
    """The lid-driven cavity (noslip walls, lid velocity Dirichlet) with the
    theta-implicit prediction: the momentum system's zero rows at the noslip
    and Dirichlet components; three steps against the oracle."""
    m, data, ops, kw, nstep, _ = _regression_ops("lid")
    kw = dict(kw, ptol=1e-8)
    d = chocg.ChoCG(ctx(), ops, **kw)
    o = _oracle(ops, **kw)
    for s in (d, o):
        s.set_theta(1.0, ops["inpoel"], mom_pc="jacobi", mom_iter=100, mom_tol=1e-8)
    n = ops["coord"].shape[1]
    d.set_state(np.zeros((n, 3)))
    o.set_state(np.zeros((n, 3)), np.zeros(n))
    assert same_its(d.init(), o.init())
    dts, its, _, _ = d.run(3)
    for k in range(3):
        dto, ito = o.step()
        assert abs(dts[k] / dto - 1) < 1e-12
        assert same_its(its[k], ito)
    u, p, _ = d.state()
    assert relerr(u, o.get(0)) < 1e-9
    assert relerr(p, o.get(2)) < 1e-9


def _regression_ops(name):
    m, data = chocg_mesh(name)
    u0 = (0.0, 0.0, 0.0)
    if name == "lid":
        ops = chocg.operators(m, noslip_sets=[1, 2, 3, 5, 6],
                              dir_bcs=[(4, (1, 1, 1), (1.0, 0.0, 0.0))], hydrostat=0)
        kw = dict(mu=0.01, cfl=0.9, flux="damp4", pc="jacobi", ptol=1e-3, pmaxit=500)
        nstep = 10
    elif name == "inviscid_sphere":
        ops = chocg.operators(m, sym_sets=[1, 4], dir_bcs=[(2, (1, 0, 0), (1.0, 0.0, 0.0))],
                              pdir_bcs=[(3, 0.0)])
        kw = dict(mu=0.0, cfl=0.5, flux="damp2", pc="jacobi", ptol=1e-3, pmaxit=300)
        nstep = 10
        u0 = (1.0, 0.0, 0.0)
    elif name == "viscous_sphere":
        ops = chocg.operators(m, noslip_sets=[1], dir_bcs=[(2, (1, 0, 0), (1.0, 0.0, 0.0)),
                                                           (4, (1, 1, 1), (1.0, 0.0, 0.0))],
                              pdir_bcs=[(3, 0.0)])
        kw = dict(mu=1.0 / 40.0, cfl=0.3, flux="damp4", rk=4, pc="jacobi", ptol=1e-3,
                  pmaxit=300)
        nstep = 20
        u0 = (1.0, 0.0, 0.0)
    else:
        ops = chocg.operators(m, noslip_sets=[3, 4],
                              dir_bcs=[(1, (0, 1, 1), (0.0, 0.0, 0.0)),
                                       (5, (0, 1, 1), (0.0, 0.0, 0.0))],
                              pdir_bcs=[(1, 2.4), (2, 0.0)])
        kw = dict(mu=0.01, cfl=0.05, flux="damp2", pc="jacobi", ptol=1e-3, pmaxit=500)
        nstep = 20
    return m, data, ops, kw, nstep, u0


@pytest.mark.parametrize("name", ["lid", "poiseuille", "inviscid_sphere", "viscous_sphere"])
def test_reference_regression_on_gpu(name, tmp_path):
    """The reference's lid-driven cavity, Poiseuille and inviscid sphere
    regressions run through the C ABI on renumbered (RCM) meshes: the diag
    file written by DiagWriter matches the reference's diag baseline within
    its numdiff tolerances, and the final fields match its exodiff
    tolerances."""
    m, data, ops, kw, nstep, u0 = _regression_ops(name)
    d = chocg.ChoCG(ctx(), ops, **kw)
    n = ops["coord"].shape[1]
    d.set_state(np.tile(np.asarray(u0), (n, 1)))
    d.init()
    v = ops["vol"]
    t = 0.0
    path = str(tmp_path / "diag")
    w = io.DiagWriter(path, io.CHOCG_DIAG, precision=12)
    for k in range(nstep):
        dts, its, _, _ = d.run(1)
        t += dts[0]
        u, pr, _ = d.state()
        w.write(k + 1, t, dts[0], io.chocg_diagnostics(u, d.field(0), pr, d.field(4), v))
    w.close()
    got, exp = io.read_diag(path)[:, :11], data["diag"][:, :11]
    # diag.ndiff.cfg: t, dt and every L2 norm abs 1e-7 or rel 1e-7
    assert np.all(np.abs(got - exp) <= np.maximum(1e-7, 1e-7 * np.abs(exp)))
    names = [str(x) for x in data["out_names"]]
    idx = _by_coord(ops["coord"], data["out_coord"])
    u, pr, _ = d.state()
    got = {"velocityx": u[idx, 0], "velocityy": u[idx, 1], "velocityz": u[idx, 2],
           "pressure": pr[idx]}
    tol = FIELD_TOL.get(name, {})
    for fname, val in got.items():
        exp = data["out_fields"][names.index(fname)]
        rel = tol.get(fname, 1e-7)
        big = np.abs(exp) > 1e-8
        err = np.abs(val - exp)
        assert np.all(err[big] <= rel * np.abs(exp[big]) + tol.get("abs", 1e-12)), (
            fname, err.max())
        assert np.all(err[~big] <= 1e-8), fname
