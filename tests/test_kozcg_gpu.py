"""KozCG (Taylor-Galerkin + FCT) on the GPU against the oracle and the
reference's KozCG Sod baseline.  In FP64 each node sums its element
contributions in ascending element order (the oracle's order), with no
atomics, so a run gives the same bits every time; it agrees with the oracle
to 1e-12 relative (contracted multiply-adds round differently).  The FP32
element path (element terms in FP32, nodal sums and update in FP64) is held
to stated error bounds against the same FP64 oracle."""

import numpy as np
import pytest

import oracle
from common import random_state, sod_mesh, wave_ic
from gpu_util import ctx, relerr
from test_oracle_pins import (KOZCG_GOLDEN, SOURCE_CASES, _by_coord, _fields,
                              check_golden, golden_case, golden_run, kozcg_sod_setup,
                              source_prm)
from xyst_gb300 import kozcg, mesh, riecg

pytestmark = pytest.mark.gpu


def _cube(n=8, seed=1):
    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed)
    v = riecg.volumes(m["coord"], m["inpoel"])
    return m, v


def test_dropin_rhs():
    m, v = _cube()
    U = random_state(m["coord"].shape[1], 5)
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"])
    o = oracle.KozCG(m["coord"], v, m["inpoel"])
    assert relerr(d.rhs(U, 2.5e-3), o.rhs(U, 2.5e-3)) < 1e-12


@pytest.mark.parametrize("problem", sorted(SOURCE_CASES))
def test_dropin_rhs_with_source(problem):
    """kozak::rhs with a manufactured source at the context's time t = 0.3
    (nodes' sources at t, centroids' at t + dt/2): FP64 against the oracle,
    itself pinned bit for bit to the reference's compiled function."""
    m, v = _cube()
    U = random_state(m["coord"].shape[1], 6)
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"])
    o = oracle.KozCG(m["coord"], v, m["inpoel"])
    for s in (d, o):
        s.set_source(problem, source_prm(problem))
        s.set_state(U, 0.3)
    R = d.rhs(U, 2.5e-3)
    Ro = o.rhs(U, 2.5e-3)
    assert relerr(R, Ro) < 1e-12
    d.set_source("none")
    assert relerr(d.rhs(U, 2.5e-3), Ro) > 1e-10  # the source was on


@pytest.mark.parametrize("name", KOZCG_GOLDEN)
def test_manufactured_solution_baselines_on_gpu(name):
    """The reference's KozCG manufactured-solution regressions (Taylor-Green,
    vortical flow, nonlinear energy growth, Rayleigh-Taylor) on the GPU in
    FP64 (no FCT, the problem's source, its analytic state as Dirichlet
    values at each step's end time, steps given their dt by xg_kozcg_step):
    every diagnostics row and the fields at every output time within the
    reference's numdiff and exodiff tolerances."""
    m, dd, case, state = golden_case(name)
    coord, inpoel = m["coord"], m["inpoel"]
    v = riecg.volumes(coord, inpoel)
    d = kozcg.KozCG(ctx(), coord, v, inpoel, gamma=5.0 / 3.0, cfl=case["cfl"], fct=False)
    U0 = state(coord)
    dn = np.unique(np.concatenate([m["bface"][s] for s in sorted(m["bface"])]))
    d.set_bc(dir=(dn, np.ones((dn.size, 5), np.int32), U0[dn]))
    d.set_source(case["problem"], case["prm"])
    d.set_state(U0, 0.0)
    rows, states = golden_run(d, case, v)
    check_golden(name, rows, states, coord, dd)
    assert abs(d.state()[1] - rows[-1, 1]) < 1e-15


def test_dropin_rhs_fp32_bound():
    """FP32 element residual: within 2e-6 of the FP64 oracle's largest entry."""
    m, v = _cube()
    U = random_state(m["coord"].shape[1], 5)
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], precision="fp32")
    o = oracle.KozCG(m["coord"], v, m["inpoel"])
    e = relerr(d.rhs(U, 2.5e-3), o.rhs(U, 2.5e-3))
    assert 0 < e < 2e-6


@pytest.mark.parametrize("fct", [False, True])
def test_run_fp32_bound(fct):
    """FP32 element terms, FP64 state: 8 steps of the smooth wave (symmetry
    walls, FCT on and off) stay within 1e-5 of the FP64 oracle; time steps,
    formed from the FP64 state, within 1e-6."""
    m, v = _cube(9)
    sym = oracle.sym_bc(m["coord"], m["bface"], [1, 2, 3, 4, 5, 6])
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], fct=fct, precision="fp32")
    o = oracle.KozCG(m["coord"], v, m["inpoel"], fct=fct)
    d.set_bc(sym=sym[:2])
    o.set_sym(*sym[:2])
    U0 = wave_ic(m["coord"])
    d.set_state(U0)
    o.set_state(U0)
    dts, _ = d.run(8)
    dto = o.run(8)
    assert np.allclose(dts, dto, rtol=1e-6)
    assert relerr(d.state()[0], o.state()) < 1e-5


def test_fp64_runs_are_bit_identical():
    """FP64 with FCT on a 17^3 cube in random node order (many elements per
    node, every order of arrival possible): two set-ups, the same state and
    steps, give bit-identical states, time steps and right-hand sides."""
    m, v = _cube(17, seed=3)
    sym = oracle.sym_bc(m["coord"], m["bface"], [1, 2, 3, 4, 5, 6])
    U0 = wave_ic(m["coord"])
    out = []
    for _ in range(2):
        d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], fct=True)
        d.set_bc(sym=sym[:2])
        rhs = d.rhs(U0, 1.0e-3)
        d.set_state(U0)
        dts, _ = d.run(10)
        out.append((rhs, dts, d.state()[0]))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    o = oracle.KozCG(m["coord"], v, m["inpoel"], fct=True)
    o.set_sym(*sym[:2])
    o.set_state(U0)
    o.run(10)
    assert relerr(out[0][2], o.state()) < 1e-12


def test_bad_precision_rejected():
    m, v = _cube(4)
    prm = kozcg.KozcgParams(1.4, 0.5, 0.0, 1, 1.0, 0, 0, 7)
    c = ctx()
    ip = np.ascontiguousarray(m["inpoel"].astype(np.uint64).reshape(-1))
    co = np.ascontiguousarray(m["coord"], dtype=np.float64)
    vv = np.ascontiguousarray(v, dtype=np.float64)
    rc = c.lib.xg_kozcg_setup(c.h, kozcg.C.byref(prm), co.shape[1], co.ctypes.data,
                              vv.ctypes.data, ip.size // 4, ip.ctypes.data)
    assert rc != 0


@pytest.mark.parametrize("fct,clip,sys", [(False, False, ()), (True, False, ()),
                                          (True, True, (0, 1, 4))])
def test_run_matches_oracle(fct, clip, sys):
    m, v = _cube(9)
    sym = oracle.sym_bc(m["coord"], m["bface"], [1, 2, 3, 4, 5, 6])
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], fct=fct, fctclip=clip, fctsys=sys)
    o = oracle.KozCG(m["coord"], v, m["inpoel"], fct=fct, fctclip=clip, fctsys=sys)
    d.set_bc(sym=sym[:2])
    o.set_sym(*sym[:2])
    U0 = wave_ic(m["coord"])
    d.set_state(U0)
    o.set_state(U0)
    dts, _ = d.run(8)
    dto = o.run(8)
    assert np.allclose(dts, dto, rtol=1e-12)
    assert relerr(d.state()[0], o.state()) < 1e-12


def test_sod_reference_baseline_on_gpu():
    m, dd = sod_mesh("KozCG")
    v = riecg.volumes(m["coord"], m["inpoel"])
    sym, dirbc, U0 = kozcg_sod_setup(m)
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], cfl=0.5, fct=True, fctclip=True,
                    fctsys=[0, 1, 4])
    d.set_bc(sym=sym, dir=dirbc)
    d.set_state(U0)
    dts, _ = d.run(10)
    assert np.all(np.abs(dts / dd["diag"][:, 2] - 1) < 1e-8)
    f = _fields(d.state()[0])[:, _by_coord(m["coord"], dd["out_coord"])]
    ref_f = dd["out_fields"]
    for i in range(6):
        if i in (1, 2, 3):
            big = np.abs(ref_f[i]) > 1e-7
            assert np.all(np.abs(f[i] - ref_f[i])[big] <= 1e-8), i
        else:
            big = np.abs(ref_f[i]) > 1e-8
            assert np.all(np.abs(f[i] - ref_f[i])[big] <= 1e-7 * np.abs(ref_f[i][big])), i


def test_sod_reference_baseline_fp32_on_gpu():
    """FP32 element terms through the FCT Sod problem (discontinuous data,
    limiter switching): density and energy within 1e-4 relative of the
    reference's baseline where they exceed 1e-8, velocity within 1e-5."""
    m, dd = sod_mesh("KozCG")
    v = riecg.volumes(m["coord"], m["inpoel"])
    sym, dirbc, U0 = kozcg_sod_setup(m)
    d = kozcg.KozCG(ctx(), m["coord"], v, m["inpoel"], cfl=0.5, fct=True, fctclip=True,
                    fctsys=[0, 1, 4], precision="fp32")
    d.set_bc(sym=sym, dir=dirbc)
    d.set_state(U0)
    dts, _ = d.run(10)
    assert np.all(np.abs(dts / dd["diag"][:, 2] - 1) < 1e-5)
    f = _fields(d.state()[0])[:, _by_coord(m["coord"], dd["out_coord"])]
    ref_f = dd["out_fields"]
    for i in range(6):
        if i in (1, 2, 3):
            assert np.all(np.abs(f[i] - ref_f[i]) <= 1e-5), i
        else:
            big = np.abs(ref_f[i]) > 1e-8
            assert np.all(np.abs(f[i] - ref_f[i])[big] <= 1e-4 * np.abs(ref_f[i][big])), i
