"""ConjugateGradients on the GPU, mirroring tk::ConjugateGradients
(src/LinearSolver/ConjugateGradients.hpp:89-161): ``init`` sets the initial
guess, right-hand side and boundary conditions, ``solve`` iterates, and
``solution``/``it``/``converged`` report, with the same argument meaning."""

from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import Context, f64, load, p, u64

# "factor": M^-1 = -S (I+N)(I+N)^T S with N from set_factor (no counterpart
# in the reference, whose ConjugateGradients offers "none" and "jacobi")
PC = {"none": 0, "jacobi": 1, "factor": 2}


class ConjugateGradients:
    def __init__(self, ctx: Context, ia, ja, a, base=0):
        """ia/ja/a: scalar CSR (rows sorted by column, diagonal present);
        base=1 for the reference's one-based tk::CSR arrays."""
        self.ctx = ctx
        self.lib = ctx.lib
        ia = u64(ia)
        ja = u64(ja)
        a = f64(a)
        self.n = ia.size - 1
        self._keep = (ia, ja, a)
        ctx.check(self.lib.xg_cg_setup(ctx.h, self.n, p(ia), p(ja), p(a), base))
        self._it = 0
        self._conv = False
        self.normr = None
        self.normb = None

    def mult(self, x):
        x = f64(x)
        y = np.zeros(self.n)
        self.ctx.check(self.lib.xg_cg_mult(self.ctx.h, p(x), p(y)))
        return y

    def init(self, x=None, b=None, neubc=None, dirbc=None, apply=False, pc="jacobi"):
        """dirbc: dict node -> value (or (nodes, values))."""
        xx = None if x is None else f64(x)
        bb = None if b is None else f64(b)
        nb = None if neubc is None else f64(neubc)
        if dirbc is None:
            nodes, vals = np.zeros(0, np.uint64), np.zeros(0)
        elif isinstance(dirbc, dict):
            nodes = u64(np.array(list(dirbc.keys()), dtype=np.int64))
            vals = f64(np.array(list(dirbc.values()), dtype=np.float64))
        else:
            nodes, vals = u64(dirbc[0]), f64(dirbc[1])
        self.ctx.check(self.lib.xg_cg_init(self.ctx.h, p(xx), p(bb), p(nb), nodes.size,
                                           p(nodes) if nodes.size else None,
                                           p(vals) if vals.size else None, int(apply), PC[pc]))

    def solve(self, maxit, tol):
        it = C.c_int64()
        nr = C.c_double()
        nb = C.c_double()
        cv = C.c_int()
        self.ctx.check(self.lib.xg_cg_solve(self.ctx.h, maxit, tol, C.byref(it), C.byref(nr),
                                            C.byref(nb), C.byref(cv)))
        self._it, self._conv = it.value, bool(cv.value)
        self.normr, self.normb = nr.value, nb.value
        return self.normr

    def solve_mixed(self, maxit, tol, inner_tol=1e-3, inner_maxit=2000):
        o = C.c_int64()
        i = C.c_int64()
        nr = C.c_double()
        nb = C.c_double()
        cv = C.c_int()
        self.ctx.check(self.lib.xg_cg_solve_mixed(self.ctx.h, maxit, tol, inner_tol, inner_maxit,
                                                  C.byref(o), C.byref(i), C.byref(nr),
                                                  C.byref(nb), C.byref(cv)))
        self._it, self._conv = i.value, bool(cv.value)
        self.normr, self.normb = nr.value, nb.value
        self.outer = o.value
        return self.normr

    def set_factor(self, model=None, scale=1.0):
        """Source of N for pc="factor": a LearnedPreconditioner, or None for
        N = scale * e (scale 1: the first-order factor, 0: Jacobi)."""
        self._model = model  # keep the model alive while it is attached
        h = None if model is None else model.h
        self.ctx.check(self.lib.xg_cg_set_factor(self.ctx.h, h, float(scale)))

    def set_guard(self, guard="reference"):
        """(p,q) breakdown test of the FP64 solver: "reference" (absolute
        epsilon, ConjugateGradients.cpp:681-690) or "underflow"."""
        self.ctx.check(self.lib.xg_cg_set_guard(self.ctx.h,
                                                {"reference": 0, "underflow": 1}[guard]))

    def precondition(self, r):
        """z = M^-1 r with the preconditioner of the last init."""
        r = f64(r)
        z = np.zeros(self.n)
        self.ctx.check(self.lib.xg_cg_precondition(self.ctx.h, p(r), p(z)))
        return z

    def solution(self):
        x = np.zeros(self.n)
        self.ctx.check(self.lib.xg_cg_solution(self.ctx.h, p(x)))
        return x

    def it(self):
        return self._it

    def converged(self):
        return self._conv


def pressure_matrix(coord, inpoel):
    """ChoCG::prelhs on the host (C++): zero-based CSR (ia, ja, a)."""
    lib = load()
    c = f64(coord)
    ip = u64(inpoel)
    n = c.shape[1]
    nnz = C.c_int64()
    rc = lib.xg_mesh_pressure_matrix(n, p(c), ip.shape[0], p(ip), 0, C.byref(nnz), None, None,
                                     None)
    if rc != 0:
        raise ValueError("xg_mesh_pressure_matrix failed")
    ia = np.zeros(n + 1, np.uint64)
    ja = np.zeros(nnz.value, np.uint64)
    a = np.zeros(nnz.value)
    rc = lib.xg_mesh_pressure_matrix(n, p(c), ip.shape[0], p(ip), nnz.value, C.byref(nnz), p(ia),
                                     p(ja), p(a))
    if rc != 0:
        raise ValueError("xg_mesh_pressure_matrix failed")
    return ia.astype(np.int64), ja.astype(np.int64), a
