"""Parity on the benchmark workloads' own mesh sizes (not toy meshes).

Each test runs the GPU path and the oracle (the serial restatement of the
reference's loops, pinned bit-for-bit to the reference's compiled physics)
on the same mesh and inputs and compares every field:

* RieCG Sod shock tube on the 33^3-node unit cube (196,608 tets), FP64,
  symmetry on all faces, RK3 at CFL 0.5, 100 steps (RieCG::solve,
  src/Inciter/RieCG.cpp:992-1057): dt history and fields within 1e-12.
* RieCG smooth density wave on the 129^3-node jittered cube (2,146,689
  nodes), FP64, one full 3-stage step.  At this size the reference
  arithmetic itself is order-sensitive at a few nodes: the oracle run with
  its edges in reverse order differs from the oracle by up to 7.7e-12 in
  the max norm (9e-15 in the L2 norm) after one step.  The GPU must be as
  close to the oracle as that (max norm within twice the oracle's own
  reordering difference, or 1e-12) and within 1e-13 in the L2 norm.
* KozCG smooth density wave on the same 129^3 cube, FP64 Taylor-Galerkin +
  FCT, one step (KozCG.cpp:613-1197): fields within 1e-12.
* ChoCG Taylor-Green vortex on the 65^3-node cube (1,572,864 tets), Re 100,
  damp2, Jacobi PCG to 1e-10 with the reference's breakdown test, start-up
  and 10 time steps (ChoCG.cpp:1357-1695): every dt within 1e-12, pressure
  iteration counts within one, fields within 1e-9 (the pressure solves
  amplify summation-order rounding by the condition number).

Sizes are the full ones; the step counts are what the single-threaded
oracle finishes in about a minute each.
"""

import numpy as np
import pytest

import oracle
from common import sod_ic, wave_ic
from gpu_util import ctx, pair, relerr
from xyst_gb300 import chocg, kozcg, mesh, riecg

pytestmark = pytest.mark.gpu

FIELDS = ("density", "x-momentum", "y-momentum", "z-momentum", "total energy")


def _per_field(a, b):
    return {f: relerr(a[:, k], b[:, k]) for k, f in enumerate(FIELDS)}


def test_riecg_sod_33cube_100_steps_fp64():
    m = mesh.cube(33)
    ops = riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=True)
    assert ops["coord"].shape[1] == 35937 and m["inpoel"].shape[0] == 196608
    d, o = pair(ops)
    U0 = sod_ic(ops["coord"])
    d.set_state(U0)
    o.set_state(U0)
    d.bc()
    o.bc()
    dts, _ = d.run(100)
    dto = o.run(100)
    assert np.allclose(dts, dto, rtol=1e-12, atol=0)
    U, _ = d.state()
    Uo = o.state()
    errs = _per_field(U, Uo)
    assert max(errs.values()) < 1e-12, errs
    assert relerr(U, Uo) < 1e-12


def _wave_129():
    m = mesh.cube(129, jitter=0.2, seed=0, numbering="random", perm_seed=1)
    return riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=True)


def _l2(a, b):
    return {f: float(np.linalg.norm(a[:, k] - b[:, k]) / np.linalg.norm(b[:, k]))
            for k, f in enumerate(FIELDS)}


def test_riecg_wave_129cube_fp64_one_step():
    ops = _wave_129()
    assert ops["coord"].shape[1] == 2146689
    d, o = pair(ops)
    U0 = wave_ic(ops["coord"])
    d.set_state(U0)
    o.set_state(U0)
    d.bc()
    o.bc()
    dts, _ = d.run(1)
    dto = o.run(1)
    assert np.allclose(dts, dto, rtol=1e-12, atol=0)
    Ud, Uo = d.state()[0], o.state()
    # the oracle against itself with the edges summed in reverse order
    rev = oracle.RieCG(ops["coord"], ops["vol"], ops["edges"][::-1].copy(),
                       ops["dint"][::-1].copy(), ops["tri"], ops["besym"])
    rev.set_sym(*ops["sym"])
    rev.set_state(U0)
    rev.bc()
    rev.run(1)
    own = _per_field(rev.state(), Uo)
    errs = _per_field(Ud, Uo)
    for f in FIELDS:
        assert errs[f] <= max(1e-12, 2.0 * own[f]), (f, errs[f], own[f])
    l2 = _l2(Ud, Uo)
    assert max(l2.values()) < 1e-13, l2


def test_kozcg_wave_129cube_fp64_one_step():
    m = mesh.cube(129, jitter=0.2, seed=0, numbering="random", perm_seed=1)
    m = mesh.relabel(m, riecg.rcm(m["inpoel"], m["coord"].shape[1]))
    v = riecg.volumes(m["coord"], m["inpoel"])
    sym = oracle.sym_bc(m["coord"], m["bface"], [1, 2, 3, 4, 5, 6])
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], fct=True)
    o = oracle.KozCG(m["coord"], v, m["inpoel"], fct=True)
    d.set_bc(sym=sym[:2])
    o.set_sym(*sym[:2])
    U0 = wave_ic(m["coord"])
    d.set_state(U0)
    o.set_state(U0)
    dts, _ = d.run(1)
    dto = o.run(1)
    assert np.allclose(dts, dto, rtol=1e-12, atol=0)
    errs = _per_field(d.state()[0], o.state())
    assert max(errs.values()) < 1e-12, errs


def _same_its(a, b):
    """Iteration counts agree within one (negative: ended by the (p,q)
    breakdown test before the tolerance, on both sides)."""
    return (a > 0) == (b > 0) and abs(abs(a) - abs(b)) <= 1


def test_chocg_taylor_green_65cube_jacobi_1e10():
    m = mesh.cube(65)
    ops = chocg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], hydrostat=0)
    assert ops["coord"].shape[1] == 274625
    kw = dict(mu=0.01, cfl=0.5, flux="damp2", pc="jacobi", ptol=1e-10, pmaxit=50000)
    d = chocg.ChoCG(ctx(), ops, **kw)
    ia, ja, a = ops["matrix"]
    o = oracle.ChoCG(ops["coord"], ops["vol"], ops["edges"], ops["dint"], ops["tri"], ia, ja, a,
                     **kw)
    o.set_bc(dir=ops["dir"], sym=ops["sym"], noslip=ops["noslip"], pdir=ops["pdir"])
    u0 = chocg.taylor_green(ops["coord"])
    d.set_state(u0)
    o.set_state(u0, np.zeros(u0.shape[0]))
    assert _same_its(d.init(), o.init())
    nstep = 10
    dts, its, _, _ = d.run(nstep)
    for k in range(nstep):
        dto, ito = o.step()
        assert abs(dts[k] / dto - 1) < 1e-12
        assert _same_its(its[k], ito), (k, its[k], ito)
    u, p, _ = d.state()
    assert relerr(u, o.get(0)) < 1e-9
    assert relerr(p, o.get(2)) < 1e-9
