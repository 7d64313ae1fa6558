"""Learned preconditioner for the pressure-Poisson CG (device network of
libxg's xg_lpc_* entry points): training on solved systems and attachment to
a ConjugateGradients as its "factor" preconditioner.

There is no counterpart in the reference, whose ConjugateGradients offers the
"none" and "jacobi" preconditioners only
(src/LinearSolver/ConjugateGradients.cpp:213-259).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import cg, mesh
from .lib import Context

PRECISION = {"fp32": 0, "bf16": 1}


class LearnedPreconditioner:
    """One network on the device of ``ctx``; precision "bf16" runs its dense
    layers as BF16 tensor-core GEMMs (FP32 accumulation), "fp32" on CUDA cores."""

    def __init__(self, ctx: Context, precision: str = "bf16", params=None, seed: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        self.n = int(self.lib.xg_lpc_nparams())
        h = C.c_void_p()
        ctx.check(self.lib.xg_lpc_create(ctx.h, PRECISION[precision], C.byref(h)))
        self.h = h
        self.set_params(init_params(seed) if params is None else params)

    def close(self):
        if self.h:
            self.lib.xg_lpc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, theta):
        t = np.ascontiguousarray(theta, dtype=np.float32)
        if t.size != self.n:
            raise ValueError(f"expected {self.n} parameters, got {t.size}")
        self._check(self.lib.xg_lpc_set_params(self.h, t.ctypes.data_as(C.c_void_p)))

    def params(self):
        t = np.zeros(self.n, np.float32)
        self._check(self.lib.xg_lpc_get_params(self.h, t.ctypes.data_as(C.c_void_p)))
        return t

    def zero_grads(self):
        self._check(self.lib.xg_lpc_zero_grads(self.h))

    def grads(self):
        g = np.zeros(self.n, np.float32)
        self._check(self.lib.xg_lpc_get_grads(self.h, g.ctypes.data_as(C.c_void_p)))
        return g

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"xg_lpc error {rc}: "
                               f"{self.lib.xg_lpc_last_error(self.h).decode()}")

    def grad(self, system: "cg.ConjugateGradients"):
        """Accumulate d loss / d theta on the matrix of an initialised system
        (Dirichlet rows eliminated); returns the loss."""
        loss = C.c_double()
        system.ctx.check(self.lib.xg_lpc_grad(self.h, system.ctx.h, C.byref(loss)))
        return loss.value

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self._check(self.lib.xg_lpc_adam(self.h, lr, beta1, beta2, eps))

    def train(self, systems, steps, lr=1e-3, log=None):
        """Adam on the mean loss over ``systems`` (initialised ConjugateGradients)."""
        hist = []
        for k in range(steps):
            self.zero_grads()
            tot = 0.0
            for s in systems:
                tot += self.grad(s)
            # Adam is invariant to a constant gradient scale: the summed
            # gradient stands for the mean
            self.adam(lr=lr)
            hist.append(tot / len(systems))
            if log is not None and (k % 20 == 0 or k == steps - 1):
                log(k, hist[-1])
        return hist


H = 64
SHAPES = [("W0", (4, H)), ("b0", (H,)), ("W1", (2 * H, H)), ("b1", (H,)),
          ("W2", (2 * H, H)), ("b2", (H,)), ("W3", (2 * H, H)), ("b3", (H,)),
          ("Wo", (H, 2 * H)), ("c", (H,)), ("c2", (H,)), ("d", (H,)), ("w", (H,)),
          ("ob", (1,))]


def init_params(seed=0, wscale=0.0):
    """He-initialised weights, zero biases; w = wscale * N(0, 1/H) (0: the
    network starts as the second-order factor N = e + t)."""
    rng = np.random.default_rng(seed)
    out = []
    for name, shp in SHAPES:
        if name.startswith("W"):
            out.append(rng.standard_normal(shp) * np.sqrt(2.0 / shp[0]))
        elif name == "w":
            out.append(rng.standard_normal(shp) * wscale / np.sqrt(H))
        else:
            out.append(np.zeros(shp))
    return np.concatenate([o.reshape(-1) for o in out]).astype(np.float32)


def pressure_system(ctx: Context, n: int, seed: int, jitter: float = 0.2, dir_sets=(4,),
                    numbering: str = "rcm", smooth: bool = True):
    """A ChoCG-like pressure system on an n^3 jittered cube: Laplacian of
    ChoCG::prelhs, Dirichlet p = 0 on the given side sets, a random smooth
    right-hand side (sum of a few low Fourier modes plus noise)."""
    m = mesh.cube(n, jitter=jitter, seed=seed, numbering=numbering, perm_seed=seed + 7)
    ia, ja, a = cg.pressure_matrix(m["coord"], m["inpoel"])
    dn = np.unique(np.concatenate([m["bface"][s] for s in dir_sets])) if dir_sets else \
        np.zeros(0, np.int64)
    rng = np.random.default_rng(seed + 1000)
    x, y, z = m["coord"]
    if smooth:
        b = np.zeros(x.size)
        for _ in range(4):
            k = rng.integers(1, 4, size=3)
            ph = rng.uniform(0, 2 * np.pi, size=3)
            b += rng.standard_normal() * (np.sin(np.pi * k[0] * x + ph[0]) *
                                          np.sin(np.pi * k[1] * y + ph[1]) *
                                          np.sin(np.pi * k[2] * z + ph[2]))
        b += 0.1 * rng.standard_normal(x.size)
    else:
        b = rng.standard_normal(x.size)
    # ChoCG's rhs is a divergence times nodal volume: scale to that magnitude
    b *= np.abs(a).max() * 1e2
    return dict(mesh=m, ia=ia, ja=ja, a=a, dirnodes=dn, dirvals=np.zeros(dn.size), b=b)


def chocg_system(ctx: Context, n: int, seed: int, jitter: float = 0.2, rhs: str = "random"):
    """The pressure system ChoCG assembles for the Taylor-Green setup on an
    n^3 jittered cube (symmetry on every face), nodes in reverse
    Cuthill-McKee order: the ChoCG::prelhs matrix with the hydrostat node as
    its only Dirichlet row.  The trace loss reads the matrix only; b is a
    right-hand side for iteration counts: "random" (white noise) or
    "smooth" (a few low Fourier modes plus 10 % noise, the character of a
    pressure increment's divergence source), scaled like ChoCG's."""
    from . import riecg
    m = mesh.cube(n, jitter=jitter, seed=seed, numbering="lex", faces=False)
    m = mesh.relabel(m, riecg.rcm(m["inpoel"], m["coord"].shape[1]))
    ia, ja, a = cg.pressure_matrix(m["coord"], m["inpoel"])
    rng = np.random.default_rng(seed + 1000)
    if rhs == "smooth":
        x, y, z = m["coord"]
        b = np.zeros(x.size)
        for _ in range(4):
            k = rng.integers(1, 4, size=3)
            ph = rng.uniform(0, 2 * np.pi, size=3)
            b += rng.standard_normal() * (np.sin(np.pi * k[0] * x + ph[0]) *
                                          np.sin(np.pi * k[1] * y + ph[1]) *
                                          np.sin(np.pi * k[2] * z + ph[2]))
        b += 0.1 * rng.standard_normal(x.size)
    else:
        b = rng.standard_normal(ia.size - 1)
    b *= np.abs(a).max() * 1e2
    b[0] = 0.0  # the hydrostat row
    return dict(mesh=m, ia=ia, ja=ja, a=a, dirnodes=np.array([0]), dirvals=np.zeros(1), b=b)


def training_system(ctx: Context, sysd):
    """A ConjugateGradients holding sysd with its Dirichlet rows eliminated
    (what the trace loss reads), on a context of its own (a context holds
    one CG system) on ctx's device."""
    own = Context(ctx.device)
    s = cg.ConjugateGradients(own, sysd["ia"], sysd["ja"], sysd["a"])
    s.init(x=np.zeros(s.n), b=sysd["b"], dirbc=(sysd["dirnodes"], sysd["dirvals"]), apply=True,
           pc="jacobi")
    return s


def iterations(s: "cg.ConjugateGradients", sysd, pc, model=None, scale=1.0, tol=1e-8,
               maxit=20000):
    """PCG iterations to tol with the given preconditioner on sysd (x0 = 0)."""
    if pc == "factor":
        s.set_factor(model, scale)
    s.init(x=np.zeros(s.n), b=sysd["b"], dirbc=(sysd["dirnodes"], sysd["dirvals"]), apply=True,
           pc=pc)
    s.solve(maxit, tol)
    return s.it(), s.converged()
