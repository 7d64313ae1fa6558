"""RieCG on the GPU against the oracle (and the reference's Sod baseline).

Tolerances: the FP64 path must agree with the oracle to 1e-12 relative (the
only differences are summation order); the FP32-flux path (FP32 gradients and
fluxes, FP64 state and update) is held to the bound stated in each test."""

import numpy as np
import pytest

from common import golden, problem_state, random_state, sod_ic, sod_mesh, wave_ic
from gpu_util import cube_ops, ctx, pair, relerr
from test_oracle_pins import (FLOW_CASES, RIECG_GOLDEN, SOURCE_CASES, check_golden,
                              golden_case, golden_run, pressure_bc, source_prm)
from xyst_gb300 import lib, riecg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flux,stab2", [("rusanov", False), ("hllc", True)])
def test_dropin_grad_rhs_fp64(flux, stab2):
    ops = cube_ops(8)
    d, o = pair(ops, flux=flux, stab2=stab2)
    U = random_state(ops["coord"].shape[1], 7)
    G = d.grad(U)
    Go = o.grad(U)
    assert relerr(G, Go) < 1e-12
    Gv = Go / ops["vol"][:, None]
    R = d.rhs(Gv, U)
    assert relerr(R, o.rhs(Gv, U)) < 1e-12


def test_dropin_fp32_bound():
    ops = cube_ops(8)
    d, o = pair(ops, precision="fp32")
    U = random_state(ops["coord"].shape[1], 8)
    Go = o.grad(U)
    assert relerr(d.grad(U), Go) < 1e-5
    Gv = Go / ops["vol"][:, None]
    assert relerr(d.rhs(Gv, U), o.rhs(Gv, U)) < 1e-4


@pytest.mark.parametrize("flux,stab2", [("rusanov", False), ("hllc", True)])
def test_dropin_rhs_edge_coloured(flux, stab2):
    """The edge-coloured scatter (one launch per class of node-disjoint edges,
    both ends updated in place) gives the owner/deposit residual up to FP32
    summation order, within the FP32 bound of the oracle; the colouring is a
    proper one (checked on the host from the class count: at least the
    largest node degree)."""
    ops = cube_ops(9)
    d, o = pair(ops, precision="fp32", flux=flux, stab2=stab2)
    U = random_state(ops["coord"].shape[1], 9)
    Gv = o.grad(U) / ops["vol"][:, None]
    Ro = o.rhs(Gv, U)
    R = d.rhs(Gv, U)
    Rc, ncol = d.rhs_coloured(Gv, U)
    assert relerr(Rc, Ro) < 1e-4
    assert relerr(Rc, R) < 1e-5
    deg = np.bincount(np.asarray(ops["edges"]).ravel()).max()
    assert deg <= ncol <= 128


@pytest.mark.parametrize("problem", sorted(SOURCE_CASES))
def test_dropin_rhs_with_source_fp64(problem):
    """riemann::rhs with a manufactured source (riemann::src): the GPU
    evaluates the problem's s(x, t) V per node at the context's time and
    subtracts it after the domain and boundary sums; against the oracle
    (pinned bit for bit to the reference's Problems.cpp) at t = 0.3."""
    ops = cube_ops(8)
    d, o = pair(ops)
    U = random_state(ops["coord"].shape[1], 11)
    Gv = o.grad(U) / ops["vol"][:, None]
    for s in (d, o):
        s.set_source(problem, source_prm(problem))
        s.set_state(U, 0.3)
    R = d.rhs(Gv, U)
    Ro = o.rhs(Gv, U)
    assert relerr(R, Ro) < 1e-12
    d.set_source("none")
    assert relerr(d.rhs(Gv, U), Ro) > 1e-8  # the source was on


@pytest.mark.parametrize("problem", ["taylor_green", "rayleigh_taylor"])
def test_run_with_source_fp64(problem):
    """Whole RK3 steps with a source, time-dependent for rayleigh_taylor:
    each step's three stages use the source at the step's start time (as
    RieCG::rhs passes it); 4 steps from t = 0.1 (rayleigh_taylor from its
    manufactured state: the symmetry walls do not hold that flow, and its
    pressure falls towards zero after about five steps) against the oracle,
    and the time the context ends at."""
    ops = cube_ops(9)
    d, o = pair(ops)
    if problem == "rayleigh_taylor":
        U0 = problem_state(problem, source_prm(problem), ops["coord"], 0.1, gamma=1.4)
    else:
        U0 = wave_ic(ops["coord"])
    for s in (d, o):
        s.set_source(problem, source_prm(problem))
        s.set_state(U0, 0.1)
    dts, _ = d.run(4)
    dto = o.run(4)
    assert np.allclose(dts, dto, rtol=1e-12, atol=0)
    U, t = d.state()
    assert relerr(U, o.state()) < 1e-12
    assert abs(t - (0.1 + dts.sum())) < 1e-14


def test_dropin_rhs_with_source_fp32_bound():
    ops = cube_ops(8)
    d, o = pair(ops, precision="fp32")
    U = random_state(ops["coord"].shape[1], 12)
    Gv = o.grad(U) / ops["vol"][:, None]
    for s in (d, o):
        s.set_source("nonlinear_energy_growth", source_prm("nonlinear_energy_growth"))
        s.set_state(U, 0.3)
    assert relerr(d.rhs(Gv, U), o.rhs(Gv, U)) < 1e-4


def test_superedge_groups_expand_like_reference():
    """Tet and triangle superedge groups are evaluated edge by edge in the
    reference's orientation; equal to the same edges passed as a plain list."""
    ops = cube_ops(6)
    inpoel = ops["inpoel"]
    e = ops["edges"]
    key = {(int(a), int(b)): k for k, (a, b) in enumerate(e)}
    lpoed = [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]
    used = np.zeros(len(e), bool)
    sup0, int0 = [], []
    for t in inpoel:
        ks, sg = [], []
        for a, b in lpoed:
            p, q = int(t[a]), int(t[b])
            k = key.get((p, q), key.get((q, p)))
            ks.append(k)
            sg.append(1.0 if (p, q) in key else -1.0)
        if not any(used[k] for k in ks):
            for k in ks:
                used[k] = True
            sup0.append(t)
            int0.append(np.concatenate([s * ops["dint"][k] for k, s in zip(ks, sg)]))
    rest = ~used
    d = riecg.RieCG(ctx(), ops["coord"], ops["vol"], [np.array(sup0), None, e[rest]],
                    [np.array(int0), None, ops["dint"][rest]], ops["tri"], ops["besym"])
    # the same edges, as a plain list with the group orientation
    ee, dd = [], []
    for t, it in zip(sup0, int0):
        for k, (a, b) in enumerate(lpoed):
            ee.append((t[a], t[b]))
            dd.append(it[3 * k:3 * k + 3])
    ee = np.concatenate([np.array(ee), e[rest]])
    dd = np.concatenate([np.array(dd), ops["dint"][rest]])
    import oracle
    o = oracle.RieCG(ops["coord"], ops["vol"], ee, dd, ops["tri"], ops["besym"])
    U = random_state(ops["coord"].shape[1], 9)
    Go = o.grad(U)
    assert relerr(d.grad(U), Go) < 1e-12
    Gv = Go / ops["vol"][:, None]
    assert relerr(d.rhs(Gv, U), o.rhs(Gv, U)) < 1e-12


@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
def test_run_fp64_matches_oracle(flux):
    ops = cube_ops(9)
    d, o = pair(ops, flux=flux)
    U0 = wave_ic(ops["coord"])
    d.set_state(U0)
    o.set_state(U0)
    d.bc()
    o.bc()
    assert abs(d.dt() / o.dt() - 1) < 1e-14
    dts, ms = d.run(12)
    dto = o.run(12)
    assert np.allclose(dts, dto, rtol=1e-12, atol=0)
    U, t = d.state()
    assert relerr(U, o.state()) < 1e-12
    assert abs(t - dto.sum()) < 1e-15


def test_single_stages_match_oracle():
    ops = cube_ops(7)
    d, o = pair(ops)
    U0 = random_state(ops["coord"].shape[1], 2)
    d.set_state(U0)
    o.set_state(U0)
    for st in range(3):
        d.stage(st, 1.0e-4)
        o.stage(st, 1.0e-4)
        assert relerr(d.state()[0], o.state()) < 1e-12


def test_run_fp32_bound():
    """FP32 fluxes and gradients, FP64 state: fields within 1e-5 relative of the
    FP64 oracle after 12 steps of the smooth wave."""
    ops = cube_ops(9)
    d, o = pair(ops, precision="fp32")
    U0 = wave_ic(ops["coord"])
    d.set_state(U0)
    o.set_state(U0)
    d.bc()
    o.bc()
    dts, _ = d.run(12)
    dto = o.run(12)
    assert np.allclose(dts, dto, rtol=1e-6)
    assert relerr(d.state()[0], o.state()) < 1e-5


def test_farfield_dirichlet_pressure_bcs():
    ops = cube_ops(7, sym=(2, 5), far=(1,), dirs=(3,), pres=(6,))
    d, o = pair(ops, far_state=(1.2, 0.3, 0.0, 0.0, 1.1),
                dir_vals=lambda x: np.column_stack([np.ones(x.shape[1]), 0.1 * np.ones(x.shape[1]),
                                                    np.zeros(x.shape[1]), np.zeros(x.shape[1]),
                                                    2.6 * np.ones(x.shape[1])]),
                pre_vals=(0.9, 0.95))
    U0 = wave_ic(ops["coord"])
    d.set_state(U0)
    o.set_state(U0)
    d.bc()
    o.bc()
    assert relerr(d.state()[0], o.state()) < 1e-14
    dts, _ = d.run(6)
    assert np.allclose(dts, o.run(6), rtol=1e-12)
    assert relerr(d.state()[0], o.state()) < 1e-12


def test_sod_reference_baseline_on_gpu():
    """The reference's RieCG Sod regression run on the GPU: dt history and final
    fields within the reference's exodiff/numdiff tolerances."""
    from test_oracle_pins import _by_coord, _fields
    m, dd = sod_mesh("RieCG")
    ops = riecg.operators(m, sym_sets=[2, 4, 5, 6], renumber=True)
    d, o = pair(ops)
    U0 = sod_ic(ops["coord"])
    d.set_state(U0)
    d.bc()
    dts, _ = d.run(10)
    assert np.allclose(dts, dd["diag"][:, 2], rtol=1e-8, atol=0)
    f = _fields(d.state()[0])[:, _by_coord(ops["coord"], dd["out_coord"])]
    ref_f = dd["out_fields"]
    for i in range(6):
        if i in (1, 2, 3):
            big = np.abs(ref_f[i]) > 1e-7
            assert np.all(np.abs(f[i] - ref_f[i])[big] <= 1e-8)
        else:
            big = np.abs(ref_f[i]) > 1e-8
            assert np.all(np.abs(f[i] - ref_f[i])[big] <= 1e-7 * np.abs(ref_f[i][big]))


@pytest.mark.parametrize("name", RIECG_GOLDEN)
def test_manufactured_solution_baselines_on_gpu(name):
    """The reference's RieCG manufactured-solution regressions (Taylor-Green,
    vortical flow with and without stab2, nonlinear energy growth,
    Rayleigh-Taylor) on the GPU in FP64 mode: the problem's source, its
    analytic state as Dirichlet values on all six side sets at each stage's
    time, gamma 5/3; every diagnostics row and the fields at every output
    time within the reference's numdiff and exodiff tolerances."""
    m, dd, case, state = golden_case(name)
    ops = riecg.operators(m, dir_sets=[1, 2, 3, 4, 5, 6], renumber=True)
    d = riecg.RieCG(ctx(), ops["coord"], ops["vol"], [None, None, ops["edges"]],
                    [None, None, ops["dint"]], ops["tri"], ops["besym"], gamma=5.0 / 3.0,
                    cfl=case["cfl"], stab2=case.get("stab2", False))
    U0 = state(ops["coord"])
    dn = ops["dirnodes"]
    d.set_bc(dir=(dn, np.ones((dn.size, 5), np.int32), U0[dn]))
    d.set_source(case["problem"], case["prm"])
    d.set_state(U0, 0.0)
    d.bc()
    rows, states = golden_run(d, case, ops["vol"])
    check_golden(name, rows, states, ops["coord"], dd)


@pytest.mark.parametrize("name", sorted(FLOW_CASES))
def test_flow_baselines_on_gpu(name):
    """The reference's RieCG Sedov and Pipe regressions on the GPU in FP64
    mode (symmetry and pressure side sets as their control files set them):
    every diagnostics row and (Pipe) the fields at every output time within
    the tolerances the oracle meets."""
    case = FLOW_CASES[name]
    d = golden(name)
    m = {"coord": d["coord"], "inpoel": d["inpoel"],
         "bface": {int(k[5:]): d[k] for k in d.files if k.startswith("bface")}}
    ops = riecg.operators(m, sym_sets=list(case["sym"]), pre_sets=list(case["pre"]),
                          renumber=True)
    dev = riecg.RieCG(ctx(), ops["coord"], ops["vol"], [None, None, ops["edges"]],
                      [None, None, ops["dint"]], ops["tri"], ops["besym"], gamma=case["gamma"],
                      cfl=case["cfl"])
    pn, pv = pressure_bc(ops["bface"], case["pre"])
    dev.set_bc(sym=ops["sym"], pre=(pn, pv) if pn.size else None)
    dev.set_state(case["state"](ops["coord"]), 0.0)
    dev.bc()
    rows, states = golden_run(dev, case, ops["vol"])
    check_golden(name, rows, states, ops["coord"], d)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pinned_host_buffers_match_pageable(precision):
    """set_state / state with a pinned host buffer (read and written by the
    kernels over the host link) give the same bits as with pageable memory,
    on a node count that is not a multiple of the block size."""
    torch = pytest.importorskip("torch")
    ops = cube_ops(10)
    n = ops["coord"].shape[1]
    assert n % 256 != 0
    a, _ = pair(ops, precision=precision)
    b, _ = pair(ops, precision=precision, context=lib.Context(0))
    U0 = wave_ic(ops["coord"])
    pinned = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    assert pinned.ctypes.data % 8 == 0
    pinned[:] = U0
    a.set_state(U0.copy())
    b.set_state(pinned)
    assert a.dt() == b.dt()
    a.run(2)
    b.run(2)
    out = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    out[:] = np.nan
    Ua, ta = a.state()
    Ub, tb = b.state(out=out)
    assert Ub is out
    assert np.array_equal(Ua, Ub) and ta == tb


def test_profile_counts_launches():
    ops = cube_ops(6)
    d, _ = pair(ops)
    d.set_state(wave_ic(ops["coord"]))
    d.profile(True)
    d.run(3)
    kt = d.kernel_times()
    assert kt["riecg_grad"][1] == 9 and kt["riecg_rhs_update"][1] == 9
    assert kt["riecg_flux"][1] == 9
    assert kt["riecg_step_begin"][1] == 3
    d.profile(False)


def test_fp32_graph_profile_and_stage_paths_agree():
    """FP32 steps through the captured graphs and through the kernel-by-
    kernel profiling path give the same bits, and so do single stages."""
    ops = cube_ops(7)
    a, _ = pair(ops, precision="fp32")
    b, _ = pair(ops, precision="fp32", context=lib.Context(0))
    for d in (a, b):
        d.set_state(wave_ic(ops["coord"]))
    a.run(4)
    b.run(2)
    b.profile(True)
    b.run(1)
    b.profile(False)
    b.run(1)
    assert np.array_equal(a.state()[0], b.state()[0])
    dt = a.dt()
    assert dt == b.dt()
    b.profile(True)
    for st in range(3):
        a.stage(st, dt)
        b.stage(st, dt)
    assert np.array_equal(a.state()[0], b.state()[0])
    b.profile(False)


def test_errors_are_status_codes():
    ops = cube_ops(4)
    d, _ = pair(ops)
    with pytest.raises(RuntimeError):
        d.stage(3, 1e-3)
    with pytest.raises(RuntimeError):
        riecg.RieCG(ctx(), ops["coord"], ops["vol"], [None, None, ops["edges"] + 10 ** 6],
                    [None, None, ops["dint"]], ops["tri"], ops["besym"])
