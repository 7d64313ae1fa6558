"""Benchmark: RieCG node-updates/s on one GB300 (and N independent replicas).

Workload (one "step" = one full 3-stage RieCG time step over the whole mesh):
unit cube with 129^3 nodes (2,146,689 nodes, 12,582,912 tets), interior nodes
jittered by a seeded U(-0.2h, 0.2h), seeded random input numbering renumbered
by reverse Cuthill-McKee, smooth density wave rho = 1 + 0.2 sin sin sin,
u = (1, 0.5, 0.25), p = 1, gamma 1.4, Rusanov flux with MUSCL, symmetry BCs on
all six faces, CFL 0.5.  Synthetic data: the mesh and state are generated.

  value  node-updates/s = nodes x steps / device time (state resident in HBM)
  e2e    the same through the C ABI with host buffers: every step uploads U
         from pinned host memory, advances one step and downloads U
  roofline  for the dominant kernel (the one with the largest device time),
         algorithmic bytes per launch / mean launch time from CUDA events
         taken inside the timed region, against the measured HBM copy
         bandwidth
  cpu_baseline  the oracle (serial C++ restatement of the reference loops) on
         one host core, on a bounded sample of the same workload (eight cell
         layers from the middle of the cube, ten steps)
  chocg  the metric's second half: ChoCG s/step on the same cube (Taylor-Green
         vortex, Re 100), every pressure solve to 1e-8 relative residual, FP64
         Jacobi PCG against the learned factor with mixed precision

--impl reference runs the reference's CPU arithmetic (the oracle port; the
reference itself needs Charm++ and cannot be built on the GPU machine) on the same
n^3 workload: the cube cut into one z-slab per host core, one single-threaded
process per slab, --warmup real warm-up steps and --steps timed steps.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RieCG node-updates/s"
UNIT = "node-updates/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks

class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


# ------------------------------------------------------------------ workload

def wave_state(coord, gamma=1.4):
    x, y, z = coord
    r = 1.0 + 0.2 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)
    u = np.array([1.0, 0.5, 0.25])
    U = np.empty((coord.shape[1], 5))
    U[:, 0] = r
    U[:, 1:4] = r[:, None] * u[None, :]
    U[:, 4] = 1.0 / (gamma - 1.0) + 0.5 * r * (u @ u)
    return U


def build_ops(n, seed=0):
    from xyst_gb300 import mesh, riecg

    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed + 1)
    return riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=True)


def kernel_bytes(n, nedge, nbtri, fp32):
    """Algorithmic bytes per launch of the time loop's kernels, by the
    reference's dataflow per RK stage (each array read or written once per
    pass; node arrays 8 B per value, halved for the G, D and coordinate terms
    in FP32-flux mode; int32 ids): riemann::grad reads U and writes G, with
    the edge ids and D (160 N + 32 E in FP64, 100 N + 20 E in FP32);
    riemann::rhs reads U, G and coordinates and writes R, with the edge ids
    and D (224 N + 32 E, or 152 N + 20 E) -- the flux kernel; the update
    reads R, Un and Vol and writes U (128 N) -- the residual-and-update
    kernel; each boundary integral 15 B per boundary triangle.  Per stage
    that is 512 N + 64 E + 30 B (FP64) or 380 N + 40 E + 30 B (FP32), and
    the step adds a dt pass and the Un copy (128 N).

    `own` is what each kernel itself must move per launch (each array it
    reads or writes once; gathered neighbour records excluded): the
    gradient pass both ends of every edge in the adjacency; the flux pass
    the owned half (neighbour, D and the slot of the edge in the other end's
    list, where it deposits that end's flux) and the deposits; the
    residual-and-update pass the deposits and the node state."""
    F = 4 if fp32 else 8
    Wb, Gb, Db = 8 * F, 16 * F, 4 + 3 * F
    if fp32:
        grad, flux = 100 * n + 20 * nedge, 152 * n + 20 * nedge
    else:
        grad, flux = 160 * n + 32 * nedge, 224 * n + 32 * nedge
    upd = 128 * n
    bnd = 15 * nbtri
    own_rhs = n * (5 * F + Wb + 8 + 4 + 40 + Wb) + nedge * 5 * F
    own = {"riecg_grad": n * (Wb + 8 + 4 + Gb) + 2 * nedge * Db,
           "riecg_flux": n * (Wb + Gb + 5 * F) + nedge * (Db + 4 + 5 * F),
           "riecg_rhs_update": own_rhs + n * 40 / 3.0}
    return {"riecg_grad": grad, "riecg_flux": flux, "riecg_rhs_update": upd,
            "riecg_grad_bnd": bnd, "riecg_rhs_bnd": bnd,
            "step": 3 * (grad + flux + upd + 2 * bnd) + 128 * n, "own": own}


# the learned preconditioner's training corpus (cube size, jitter seed) and
# its evaluation systems (unseen seeds)
CORPUS = ([(33, s) for s in range(10, 16)] + [(49, s) for s in range(20, 24)] +
          [(65, s) for s in range(30, 33)] + [(81, 40), (97, 50)])
EVAL = [(129, 98), (193, 99)]


def lpc_eval(model, n, seed, tol=1e-8):
    """One ChoCG pressure system (n^3 jittered cube, unseen jitter seed,
    hydrostat node, smooth right-hand side) solved to tol relative residual
    by FP64 Jacobi PCG (the reference's algorithm, underflow guard) and by
    the mixed-precision solve with the first-order and the learned factor:
    iterations and wall seconds per solve (x0 = 0, device sync included)."""
    from xyst_gb300 import cg, lib, lpc

    t0 = time.perf_counter()
    sysd = lpc.chocg_system(None, n, seed, rhs="smooth")
    ctx = lib.Context(0)
    s = cg.ConjugateGradients(ctx, sysd["ia"], sysd["ja"], sysd["a"])
    s.set_guard("underflow")
    out = {"nodes": int(n ** 3), "jitter_seed": seed, "tol": tol,
           "setup_s": time.perf_counter() - t0}
    dirbc = (sysd["dirnodes"], sysd["dirvals"])
    for name, pc, mdl in (("fp64_jacobi", "jacobi", None), ("mixed_first_order", "factor", "none"),
                          ("mixed_learned", "factor", model)):
        if pc == "factor":
            s.set_factor(None if mdl == "none" else mdl, 1.0)
        runs = []
        for rep in range(2):  # the first solve also builds the factor
            s.init(x=np.zeros(s.n), b=sysd["b"], dirbc=dirbc, apply=True, pc=pc)
            t1 = time.perf_counter()
            if pc == "jacobi":
                s.solve(50000, tol)
            else:
                s.solve_mixed(1000, tol, inner_tol=0.1, inner_maxit=50000)
            runs.append(time.perf_counter() - t1)
        out[name] = {"iterations": int(s.it()), "converged": bool(s.converged()),
                     "s_per_solve": runs[-1],
                     "rel_residual": float(s.normr / max(s.normb, 1e-300))}
    out["speedup_learned_mixed_vs_fp64_jacobi"] = (out["fp64_jacobi"]["s_per_solve"] /
                                                   out["mixed_learned"]["s_per_solve"])
    ctx.close()
    return out


def run_chocg(n=129, steps=5, warm=2, tol=1e-8, train_steps=300, seed=0):
    """ChoCG s/step on the n^3 jittered cube (Taylor-Green vortex on
    [0, 2 pi]^3 mapped to the unit cube, mu = 1/Re = 0.01, damp2, CFL 0.5,
    symmetry on every face, hydrostat node), every pressure-increment solve to
    tol relative residual: FP64 Jacobi PCG (the reference's algorithm)
    against the learned factor with the mixed-precision solve, plus the
    factor without the network; fields after the timed steps compared with
    the FP64 Jacobi run.  Every solve runs to the tolerance: the reference's
    absolute (p,q) breakdown test would end these small-rhs increment solves
    near 1e-6, so the FP64 solver guards underflow only (as the FP32 one)."""
    from xyst_gb300 import chocg, lib, lpc, mesh

    t_setup = time.perf_counter()
    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed + 1)
    ops = chocg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], hydrostat=0)
    u0 = chocg.taylor_green(ops["coord"])
    t_setup = time.perf_counter() - t_setup
    tctx = lib.Context(0)
    t0 = time.perf_counter()
    systems = [lpc.training_system(tctx, lpc.chocg_system(tctx, k, sd)) for k, sd in CORPUS]
    t_corpus = time.perf_counter() - t0
    model = lpc.LearnedPreconditioner(tctx, precision="bf16", seed=0)
    t0 = time.perf_counter()
    hist = model.train(systems, train_steps, lr=1e-3)
    t_train = time.perf_counter() - t0
    out = {"workload": f"ChoCG Taylor-Green, {n}^3 jittered cube, Re 100, damp2, CFL 0.5, "
                       "symmetry on all faces, hydrostat node",
           "nodes": int(ops["coord"].shape[1]), "tol": tol, "steps_timed": steps,
           "setup_s": t_setup,
           "training": {"s": t_train, "corpus_setup_s": t_corpus, "steps": train_steps,
                        "loss_first_last": [hist[0], hist[-1]],
                        "systems": f"{len(CORPUS)} ChoCG pressure matrices (hydrostat) of "
                                   f"33^3-97^3 jittered cubes, jitter seeds 10-50 (the matrix, "
                                   f"not the Reynolds number, is all the trace loss reads); "
                                   f"{sum(k ** 3 for k, _ in CORPUS)} rows in all",
                        "dense_layers": "BF16 tcgen05 tensor-core GEMMs, forward and backward"}}
    modes = {"fp64_jacobi": ("jacobi", None, False),
             "mixed_first_order": ("factor", "none", True),
             "mixed_learned": ("factor", model, True)}
    fields = {}
    for name, (pc, mdl, mixed) in modes.items():
        ctx = lib.Context(0)
        d = chocg.ChoCG(ctx, ops, mu=0.01, cfl=0.5, flux="damp2", pc=pc, ptol=tol,
                        pmaxit=50000, mixed=mixed, inner_tol=0.1, guard="underflow")
        if pc == "factor":
            d.cg.set_factor(None if mdl == "none" else mdl, 1.0)
        d.set_state(u0)
        init_it = d.init()
        d.run(warm)
        t0 = time.perf_counter()
        dts, its, ms, _ = d.run(steps)
        wall = time.perf_counter() - t0
        u, pr, t = d.state()
        fields[name] = (u, pr)
        out[name] = {"s_per_step": wall / steps, "device_ms_per_step": ms / steps,
                     "pressure_iterations": [int(i) for i in its], "init_iterations": init_it,
                     "dt_last": float(dts[-1])}
        ctx.close()
    ref_u, ref_p = fields["fp64_jacobi"]
    for name in ("mixed_first_order", "mixed_learned"):
        u, pr = fields[name]
        out[name]["u_rel_err_vs_fp64"] = float(np.linalg.norm(u - ref_u) / np.linalg.norm(ref_u))
        out[name]["p_rel_err_vs_fp64"] = float(np.linalg.norm(pr - ref_p) /
                                               max(np.linalg.norm(ref_p), 1e-300))
    out["speedup_learned_mixed_vs_fp64_jacobi"] = (out["fp64_jacobi"]["s_per_step"] /
                                                   out["mixed_learned"]["s_per_step"])
    out["pressure_solve_eval"] = [lpc_eval(model, k, sd, tol) for k, sd in EVAL]
    model.close()
    for s_ in systems:
        s_.ctx.close()
    tctx.close()
    return out


# ------------------------------------------------------------------ CPU leg

def _ref_partition(n, k0, k1, warmup, steps, barrier, queue):
    """One reference-arm process: the oracle RieCG (FP64, the reference's
    arithmetic, one thread) on the z-slab k0 <= k < k1 of the n^3 jittered
    cube, as one partition of a domain-decomposed run without its halo
    exchange: warmup untimed steps, then steps timed between two barriers
    shared by all partitions."""
    os.environ["OMP_NUM_THREADS"] = "1"
    import oracle
    from xyst_gb300 import mesh

    m = mesh.cube_slab(n, k0, k1, jitter=0.2, seed=0)
    c, ip = m["coord"], m["inpoel"]
    v = oracle.vol(c, ip)
    e, d = oracle.domint(c, ip)
    tri = np.concatenate([m["bface"][s_] for s_ in sorted(m["bface"])])
    nodes, norms, symset = oracle.sym_bc(c, m["bface"], [1, 2, 3, 4, 5, 6])
    besym = np.isin(tri, list(symset)).astype(np.uint8)
    o = oracle.RieCG(c, v, e, d, tri, besym)
    o.set_sym(nodes, norms)
    o.set_state(wave_state(c))
    o.bc()
    if warmup:
        o.run(warmup)
    barrier.wait()
    t0 = time.perf_counter()
    if steps:
        o.run(steps)
    t1 = time.perf_counter()
    barrier.wait()
    queue.put({"k0": k0, "k1": k1, "owned": int(m["owned"]), "nodes": int(c.shape[1]),
               "s": t1 - t0})


def reference_arm(n, steps, warmup, procs=None, one_slab=None):
    """The reference's CPU arithmetic on the n^3 workload itself: the cube cut
    into P z-slabs (P = host cores, at most n-1), one single-threaded oracle
    process per slab, all timed over the same `steps` steps after `warmup`
    real warm-up steps.  node-updates/s = n^3 * steps / the slowest slab's
    time (an upper bound of the reference's parallel model: each slab does a
    Charm++ chare's work without the halo exchange).

    one_slab=(k0, k1): time only that slab, on one core (a bounded sample of
    the same workload: node-updates/s per core)."""
    import multiprocessing as mp

    import oracle
    oracle.build()
    if one_slab is None:
        P = max(1, min(procs or os.cpu_count() or 1, n - 1))
        cuts = np.linspace(0, n - 1, P + 1).round().astype(int)
        slabs = [(int(cuts[j]), int(cuts[j + 1])) for j in range(P)]
    else:
        P, slabs = 1, [tuple(one_slab)]
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(P)
    queue = ctx.Queue()
    ps = [ctx.Process(target=_ref_partition, args=(n, k0, k1, warmup, steps, barrier, queue))
          for k0, k1 in slabs]
    t0 = time.perf_counter()
    for pr in ps:
        pr.start()
    res = [queue.get() for _ in range(P)]
    for pr in ps:
        pr.join()
    wall = time.perf_counter() - t0
    owned = sum(r["owned"] for r in res)
    worst = max(r["s"] for r in res)
    value = owned * steps / worst if steps and worst > 0 else 0.0
    if one_slab is not None:
        r = res[0]
        return {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                "ms_per_step": worst / max(steps, 1) * 1e3,
                "sample": f"z-slab layers {r['k0']}-{r['k1']} of the {n}^3 workload "
                          f"({r['nodes']} nodes, {owned} owned), {warmup} warm-up + {steps} "
                          f"timed steps, oracle C++ restatement (FP64), 1 thread, {worst:.2f} s",
                "wall_s": wall}
    assert owned == n ** 3
    return {"value": value, "unit": UNIT, "cores": P, "kind": "port",
            "ms_per_step": worst / max(steps, 1) * 1e3,
            "sample": f"the whole {n}^3 workload ({owned} nodes) in {P} z-slab partitions "
                      f"({min(r['nodes'] for r in res)}-{max(r['nodes'] for r in res)} nodes "
                      f"each, shared planes duplicated), one single-threaded oracle (C++ "
                      f"restatement, FP64) process per partition and core, {warmup} warm-up + "
                      f"{steps} timed steps between barriers, no halo exchange (upper bound); "
                      f"slowest partition {worst:.2f} s",
            "wall_s": wall}


def _oracle_proc(code):
    """Run a timing snippet in a fresh single-threaded process; its JSON line."""
    import oracle
    oracle.build()
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run([sys.executable, "-c", code], stdout=subprocess.PIPE, text=True,
                         env=env, check=True).stdout
    return json.loads(out.strip().splitlines()[-1])


def cpu_kozcg(n=49, steps=6):
    """Oracle KozCG (Taylor-Galerkin + FCT) node-updates/s on one core."""
    code = r"""
import sys, time, json
sys.path.insert(0, %r)
import oracle
from xyst_gb300 import mesh
from bench import wave_state
m = mesh.cube(%d, jitter=0.2, seed=0)
c, ip = m["coord"], m["inpoel"]
v = oracle.vol(c, ip)
nodes, norms, _ = oracle.sym_bc(c, m["bface"], [1,2,3,4,5,6])
k = oracle.KozCG(c, v, ip)
k.set_sym(nodes, norms); k.set_state(wave_state(c))
t0 = time.perf_counter(); k.run(%d); t1 = time.perf_counter()
print(json.dumps({"n": c.shape[1], "s": t1 - t0}))
""" % (ROOT, n, steps)
    r = _oracle_proc(code)
    return {"value": r["n"] * steps / r["s"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n}^3 cube ({r['n']} nodes), {steps} KozCG steps, oracle C++ "
                      f"restatement, 1 thread, {r['s']:.2f} s"}


def cpu_chocg(n=49, steps=3):
    """Oracle ChoCG s/step (FP64 Jacobi PCG to 1e-8, the reference's breakdown
    test) on one core."""
    code = r"""
import sys, time, json
sys.path.insert(0, %r)
import numpy as np, oracle
from xyst_gb300 import mesh, chocg
m = mesh.cube(%d, jitter=0.2, seed=0, numbering="random", perm_seed=1)
ops = chocg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], hydrostat=0)
ia, ja, a = ops["matrix"]
o = oracle.ChoCG(ops["coord"], ops["vol"], ops["edges"], ops["dint"], ops["tri"], ia, ja, a,
                 mu=0.01, cfl=0.5, flux="damp2", pc="jacobi", ptol=1e-8, pmaxit=50000)
o.set_bc(dir=ops["dir"], sym=ops["sym"], noslip=ops["noslip"], pdir=ops["pdir"])
u0 = chocg.taylor_green(ops["coord"]); o.set_state(u0, np.zeros(u0.shape[0])); o.init()
its = []
t0 = time.perf_counter()
for _ in range(%d): its.append(o.step()[1])
t1 = time.perf_counter()
print(json.dumps({"n": u0.shape[0], "s": t1 - t0, "its": its}))
""" % (ROOT, n, steps)
    r = _oracle_proc(code)
    return {"value": r["s"] / steps, "unit": "s/step", "cores": 1, "kind": "port",
            "sample": f"{n}^3 cube ({r['n']} nodes), {steps} ChoCG steps, FP64 Jacobi PCG to "
                      f"1e-8 with the reference's breakdown test (iterations {r['its']}, "
                      "negative: stopped by the test), oracle C++ restatement, 1 thread"}


def run_kozcg(n=129, steps=10, warm=2, seed=0):
    """KozCG (FP64 Taylor-Galerkin + FCT) node-updates/s on the n^3 jittered
    cube with the smooth density wave and symmetry on every face."""
    from xyst_gb300 import kozcg, lib, mesh, riecg

    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed + 1)
    new_of_old = riecg.rcm(m["inpoel"], m["coord"].shape[1])
    m = mesh.relabel(m, new_of_old)
    coord, inpoel = m["coord"], m["inpoel"]
    v = riecg.volumes(coord, inpoel)
    ops = riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=False)
    ctx = lib.Context(0)
    U0 = wave_state(coord)
    nn = coord.shape[1]
    res = {}
    for fct in (True, False):
        for prec in ("fp64", "fp32"):
            k = kozcg.KozCG(ctx, coord, v, inpoel, fct=fct, precision=prec)
            k.set_bc(sym=ops["sym"])
            k.set_state(U0)
            k.run(warm)
            k.set_state(U0)
            dts, ms = k.run(steps)
            res[prec, fct] = (ms, k.state()[0])
            if prec == "fp64" and fct:
                # the same steps again: FP64 sums in a fixed order, same bits
                k.set_state(U0)
                k.run(steps)
                rerun_same = bool(np.array_equal(k.state()[0], res[prec, fct][1]))
            del k
    ctx.close()

    def dev(fct):
        a, b = res["fp32", fct][1], res["fp64", fct][1]
        return float(np.abs(a - b).max() / np.abs(b).max())

    ms, ms32 = res["fp64", True][0], res["fp32", True][0]
    return {"workload": f"KozCG Euler, {n}^3 jittered cube (RCM), smooth density wave, "
                        "Taylor-Galerkin + FCT, symmetry on all faces, CFL 0.5, FP64",
            "nodes": int(nn), "steps": steps, "ms_per_step": ms / steps,
            "value": nn * steps / (ms / 1e3), "unit": UNIT,
            "fp64_rerun_bit_identical": rerun_same,
            "fp32_elements": {"ms_per_step": ms32 / steps,
                              "value": nn * steps / (ms32 / 1e3), "unit": UNIT,
                              "max_rel_dev_vs_fp64": dev(True),
                              "max_rel_dev_vs_fp64_without_fct": dev(False)}}


# ------------------------------------------------------------------ GPU leg

def run_gpu(args, rank, world):
    from xyst_gb300 import lib, riecg

    t_setup = time.perf_counter()
    ops = build_ops(args.n, seed=rank)
    n = ops["coord"].shape[1]
    U0 = wave_state(ops["coord"])
    ctx = lib.Context(args.device if world == 1 else int(os.environ.get("LOCAL_RANK", 0)))
    prec = args.precision
    r = riecg.from_operators(ctx, ops, precision=prec)
    t_setup = time.perf_counter() - t_setup
    nedge = ops["edges"].shape[0]
    nbtri = ops["tri"].shape[0]
    r.set_state(U0)
    r.bc()
    # warm-up
    r.run(args.warmup)
    barrier(world)
    # timed region: device-resident state, per-kernel events on the ctx stream
    r.set_state(U0)
    r.bc()
    r.profile(True)
    with Clocks(int(os.environ.get("LOCAL_RANK", args.device))) as ck:
        barrier(world)
        dts, ms = r.run(args.steps)
        barrier(world)
    r.profile(False)
    kt = r.kernel_times()
    # the same step count without events (the headline device time)
    r.set_state(U0)
    r.bc()
    barrier(world)
    dts2, ms_plain = r.run(args.steps)
    barrier(world)
    # e2e through the C ABI with host buffers
    e2e = e2e_run(r, U0, args.steps, world)
    dev_bytes = ctx.device_bytes()
    # the same workload in FP64 (the reference's arithmetic on the GPU), and
    # every field of the benchmark's mode against it after the workload's
    # 200 steps
    fp64 = accuracy = None
    if rank == 0 and not args.no_fp64:
        fp64, accuracy = fp64_leg(ctx, ops, r, U0, prec, args)
    ctx.close()
    cho = run_chocg(n=args.n) if (rank == 0 and not args.no_pcg) else None
    koz = run_kozcg(n=args.n) if (rank == 0 and not args.no_pcg) else None
    out = {"chocg": cho, "kozcg": koz, "fp64": fp64, "accuracy": accuracy,
           "n": n, "nedge": nedge, "nbtri": nbtri, "ms": ms_plain, "ms_events": ms, "kt": kt,
           "clocks": ck.summary(), "e2e_ms": e2e, "setup_s": t_setup, "dts": dts2,
           "dev_bytes": dev_bytes}
    return out


FIELDS = ("density", "x-momentum", "y-momentum", "z-momentum", "total energy")


def fp64_leg(ctx, ops, r, U0, prec, args, acc_steps=200):
    """RieCG in FP64 mode on the same workload (device-resident, per-kernel
    events) and, for the FP32-flux mode, the error of every conserved field
    after acc_steps steps against the FP64 run from the same initial state:
    max |U32 - U64| / max |U64| per field, and the dt history's largest
    relative difference."""
    from xyst_gb300 import lib, riecg

    ctx64 = lib.Context(ctx.device)  # a context holds one RieCG state
    r64 = riecg.from_operators(ctx64, ops, precision="fp64")
    r64.set_state(U0)
    r64.bc()
    r64.run(2)
    k64 = max(3, min(args.steps, 20))
    r64.set_state(U0)
    r64.bc()
    r64.profile(True)
    _, ms_ev = r64.run(k64)
    r64.profile(False)
    kt = r64.kernel_times()
    r64.set_state(U0)
    r64.bc()
    _, ms = r64.run(k64)
    n = U0.shape[0]
    nedge = ops["edges"].shape[0]
    out = {"workload": "the same cube, state and steps in FP64 mode (gradients, fluxes and "
                       "update in FP64, the reference's operation order apart from the van "
                       "Leer limiter in an algebraically equal form with one division for its "
                       "ten quotients, and the sound speed times |D| as one root)",
           "steps": k64, "ms_per_step": ms / k64, "value": n * k64 / (ms / 1e3), "unit": UNIT,
           "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in kt.items()}}
    # FP64 roofline of the flux kernel: its operation count per edge from the
    # source (10 three-term projections 50; MUSCL 5 x 25 + 28, the ten
    # quotients from one division by batch inversion; Rusanov 93 with 2 square
    # roots; the two residual shares 15: 311 FP64 operations, a multiply-add
    # counted as two, each division or square root once) against the FP64
    # peak measured here (cuBLAS DGEMM), and its bytes against HBM
    if "riecg_flux" in kt:
        fl_ms = kt["riecg_flux"][0] / kt["riecg_flux"][1]
        peak64 = fp64_peak_tflops()
        flops = 311.0 * nedge
        kb = kernel_bytes(n, nedge, ops["tri"].shape[0], False)
        hbm, kind = peaks()
        out["flux_roofline"] = {
            "kernel": "riecg_flux (FP64)", "mean_launch_ms": fl_ms,
            "flops_per_launch": flops, "achieved_tflops": flops / (fl_ms / 1e3) / 1e12,
            "fp64_peak_tflops": peak64, "fp64_peak_kind": "measured: cuBLAS DGEMM 4096^3",
            "frac_fp64": flops / (fl_ms / 1e3) / 1e12 / peak64 if peak64 else None,
            "algorithmic_bytes_per_launch": kb["riecg_flux"],
            "frac_hbm": kb["riecg_flux"] / (fl_ms / 1e3) / 1e9 / hbm,
            "bound": "fp64"}
    acc = None
    if prec == "fp32":
        r64.set_state(U0)
        r64.bc()
        d64, _ = r64.run(acc_steps)
        U64 = r64.state()[0]
        r.set_state(U0)
        r.bc()
        d32, _ = r.run(acc_steps)
        U32 = r.state()[0]
        acc = {"steps": acc_steps, "reference": "FP64 mode on the GPU (equal to the oracle to "
                                                "1e-12 on the same mesh)",
               "max_rel_dev_vs_fp64": {f: float(np.abs(U32[:, k] - U64[:, k]).max() /
                                               np.abs(U64[:, k]).max())
                                       for k, f in enumerate(FIELDS)},
               "dt_max_rel_dev": float(np.abs(d32 / d64 - 1).max())}
    del r64
    ctx64.close()
    return out, acc


def fp64_peak_tflops(m=4096, reps=5):
    """FP64 throughput of a cuBLAS DGEMM (m^3, best of reps, CUDA events):
    the measured FP64 roof of this GPU."""
    try:
        import torch
        a = torch.randn(m, m, dtype=torch.float64, device="cuda")
        b = torch.randn(m, m, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1e3
            best = t if best is None else min(best, t)
        del a, b
        return 2.0 * m ** 3 / best / 1e12
    except Exception:
        return None


def e2e_run(r, U0, steps, world):
    try:
        import torch
        host = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        host = np.empty_like(U0)
    host[:] = U0
    r.set_state(host)
    r.run(1)
    r.state()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        r.set_state(host)  # H2D of the step's input state (pinned)
        r.run(1)
        r.state(out=host)  # D2H of the step's result into the same pinned buffer
    t1 = time.perf_counter()
    barrier(world)
    return (t1 - t0) * 1e3


_dist = None


def barrier(world):
    if world > 1 and _dist is not None:
        _dist.barrier()


def max_over_ranks(vals, world):
    """Element-wise maximum of a few floats over the replica ranks (the
    slowest rank's times define the whole job's)."""
    if world <= 1 or _dist is None:
        return [float(v) for v in vals]
    import torch
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64)
    _dist.all_reduce(t, op=_dist.ReduceOp.MAX)
    return [float(x) for x in t]


def _cuda_profiler(on):
    """cudaProfilerStart/Stop through the CUDA runtime, so that
    `ncu --profile-from-start off` captures exactly the bracketed region."""
    import ctypes
    import glob
    rt = None
    for name in ["libcudart.so", "libcudart.so.13"] + sorted(
            glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    if rt is None:
        raise RuntimeError("CUDA runtime library not found")
    (rt.cudaProfilerStart if on else rt.cudaProfilerStop)()


def scatter_designs(n=81, reps=20):
    """The two scatters of the RieCG edge fluxes on the same n^3 FP32 Rusanov
    residual (drop-in riemann::rhs with host G and U): owner half-edges with
    deposit slots (k_flux1 + k_rhs2 + k_rhs_bnd) against edge colouring (one
    k_flux_colour launch per class of node-disjoint edges + the node
    epilogue).  Per-kernel CUDA-event times over reps calls of each."""
    from xyst_gb300 import lib, riecg

    ops = build_ops(n, seed=0)
    ctx = lib.Context(0)
    r = riecg.from_operators(ctx, ops, precision="fp32")
    U = wave_state(ops["coord"])
    Gv = r.grad(U) / ops["vol"][:, None]
    R0 = r.rhs(Gv, U)
    Rc, ncol = r.rhs_coloured(Gv, U)
    out = {"n": n, "nodes": int(ops["coord"].shape[1]), "edges": int(ops["edges"].shape[0]),
           "colours": ncol, "reps": reps,
           "max_rel_diff": float(np.abs(Rc - R0).max() / np.abs(R0).max())}
    for name, call in (("owner_deposit", r.rhs), ("edge_colouring", r.rhs_coloured)):
        r.profile(True)
        for _ in range(reps):
            call(Gv, U)
        r.profile(False)
        kt = r.kernel_times()
        out[name] = {k: {"ms_per_call": v[0] / reps, "launches_per_call": v[1] / reps}
                     for k, v in kt.items()}
        out[name]["total_ms_per_call"] = sum(v[0] for v in kt.values()) / reps
    ctx.close()
    return out


def profile_step(what, n):
    """One warm step of a workload bracketed by the profiler range (for
    `ncu --profile-from-start off`): chocg-fp64 (Jacobi PCG), chocg-mixed
    (first-order factor, mixed solve), kozcg-fp64, kozcg-fp32, and one FP32
    RieCG residual by each flux scatter, riecg-rhs-owner and
    riecg-rhs-colour."""
    from xyst_gb300 import chocg, kozcg, lib, mesh, riecg

    ctx = lib.Context(0)
    if what.startswith("riecg-rhs"):
        ops = build_ops(n, seed=0)
        r = riecg.from_operators(ctx, ops, precision="fp32")
        U = wave_state(ops["coord"])
        Gv = r.grad(U) / ops["vol"][:, None]
        call = r.rhs if what == "riecg-rhs-owner" else (lambda g, u: r.rhs_coloured(g, u)[0])
        call(Gv, U)
        _cuda_profiler(True)
        call(Gv, U)
        _cuda_profiler(False)
        out = {"profile": what, "n": n}
    elif what.startswith("chocg"):
        m = mesh.cube(n, jitter=0.2, seed=0, numbering="random", perm_seed=1)
        ops = chocg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], hydrostat=0)
        if what == "chocg-fp64":
            d = chocg.ChoCG(ctx, ops, mu=0.01, cfl=0.5, flux="damp2", pc="jacobi", ptol=1e-8,
                            pmaxit=50000, guard="underflow")
        else:
            d = chocg.ChoCG(ctx, ops, mu=0.01, cfl=0.5, flux="damp2", pc="factor", ptol=1e-8,
                            pmaxit=50000, mixed=True, inner_tol=0.1, guard="underflow")
            d.cg.set_factor(None, 1.0)
        d.set_state(chocg.taylor_green(ops["coord"]))
        d.init()
        d.run(1)
        _cuda_profiler(True)
        _, its, ms, _ = d.run(1)
        _cuda_profiler(False)
        out = {"profile": what, "n": n, "iterations": [int(i) for i in its], "ms": ms}
    else:
        m = mesh.cube(n, jitter=0.2, seed=0, numbering="random", perm_seed=1)
        m = mesh.relabel(m, riecg.rcm(m["inpoel"], m["coord"].shape[1]))
        v = riecg.volumes(m["coord"], m["inpoel"])
        ops = riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=False)
        k = kozcg.KozCG(ctx, m["coord"], v, m["inpoel"],
                        precision="fp32" if what == "kozcg-fp32" else "fp64")
        k.set_bc(sym=ops["sym"])
        k.set_state(wave_state(m["coord"]))
        k.run(1)
        _cuda_profiler(True)
        _, ms = k.run(1)
        _cuda_profiler(False)
        out = {"profile": what, "n": n, "ms": ms}
    ctx.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xg", choices=["xg", "reference"])
    ap.add_argument("--n", type=int, default=129)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-pcg", action="store_true", help="skip the ChoCG leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-mode RieCG leg")
    ap.add_argument("--profile-step", default=None,
                    choices=["chocg-fp64", "chocg-mixed", "kozcg-fp64", "kozcg-fp32",
                             "riecg-rhs-owner", "riecg-rhs-colour"],
                    help="run one warm step of that workload (side --n) inside a profiler "
                         "range and exit")
    ap.add_argument("--scatter-designs", action="store_true",
                    help="time the owner/deposit and edge-colouring flux scatters on the "
                         "--n cube and exit")
    args = ap.parse_args()
    if args.profile_step:
        profile_step(args.profile_step, args.n)
        return
    if args.scatter_designs:
        print(json.dumps(scatter_designs(args.n)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    global _dist
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        _dist = dist
    config = {"workload": f"RieCG Euler, {args.n}^3-node jittered cube (Kuhn 6-tet split), "
                          "smooth density wave, Rusanov+MUSCL, symmetry BCs, CFL 0.5, 3-stage RK",
              "nodes": args.n ** 3, "precision": ("FP32 gradients/fluxes, FP64 state/update"
                                                  if args.precision == "fp32" else "FP64"),
              "l2": "no flush needed: working set > 129 MB L2",
              "parallelism": f"replicas x{args.gpus}"}
    if args.impl == "reference":
        if rank != 0:
            return
        cb = reference_arm(args.n, args.steps, args.warmup)
        ms_step = cb.pop("ms_per_step")
        wall = cb.pop("wall_s")
        rconfig = dict(config, precision="FP64 (the reference's arithmetic)")
        line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": rconfig, "impl": "reference",
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "wall_s": wall}
        print(json.dumps(line))
        return
    cpu = cpu_koz = cpu_cho = None
    if rank == 0 and not args.no_cpu:
        # before any GPU work in this process: one slab of eight cell layers
        # from the middle of the same cube, ten steps on one core
        mid = (args.n - 1) // 2
        cpu = reference_arm(args.n, 10, 1, one_slab=(max(0, mid - 4), min(args.n - 1, mid + 4)))
        cpu.pop("ms_per_step")
        cpu.pop("wall_s")
        if not args.no_pcg:
            cpu_koz = cpu_kozcg()
            cpu_cho = cpu_chocg()
    res = run_gpu(args, rank, world)
    # max over ranks
    ms, e2e_ms = max_over_ranks([res["ms"], res["e2e_ms"]], world)
    if rank != 0:
        return
    n = res["n"]
    value = world * n * args.steps / (ms / 1e3)
    e2e_val = world * n * args.steps / (e2e_ms / 1e3)
    kb = kernel_bytes(n, res["nedge"], res["nbtri"], args.precision == "fp32")
    kt = res["kt"]
    dom = max((k for k in kt if k in kb), key=lambda k: kt[k][0])
    avg_ms = kt[dom][0] / kt[dom][1]
    peak, kind = peaks()
    achieved = kb[dom] / (avg_ms / 1e3) / 1e9
    own = kb["own"].get(dom)
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(f"{dom}:{args.precision}:{args.n}")
    except Exception:
        pass
    launches = int(sum(v[1] for v in kt.values()))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": config,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_kind": kind, "algorithmic_bytes_per_launch": kb[dom],
                         "mean_launch_ms": avg_ms,
                         "own_bytes_per_launch": own,
                         "own_frac": None if own is None else own / (avg_ms / 1e3) / 1e9 / peak},
            "step_roofline": {"algorithmic_bytes_per_step": kb["step"],
                              "achieved": kb["step"] / (ms / args.steps / 1e3) / 1e9,
                              "frac": kb["step"] / (ms / args.steps / 1e3) / 1e9 / peak},
            "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in kt.items()},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": n * 5 * 8,
                    "d2h_bytes_per_step": n * 5 * 8},
            "gpu_launches": launches,
            "clocks": res["clocks"],
            "cpu_baseline": cpu,
            "setup_s": res["setup_s"], "device_bytes": res["dev_bytes"],
            "dt_first_last": [float(res["dts"][0]), float(res["dts"][-1])],
            "riecg_fp64": res["fp64"], "accuracy": res["accuracy"],
            "chocg": res["chocg"], "kozcg": res["kozcg"]}
    if line["chocg"] is not None:
        line["chocg"]["cpu_baseline"] = cpu_cho
    if line["kozcg"] is not None:
        line["kozcg"]["cpu_baseline"] = cpu_koz
    print(json.dumps(line))


if __name__ == "__main__":
    main()
