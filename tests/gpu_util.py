"""Helpers for GPU parity tests: one set of operators fed to both the oracle
and the device path."""

from __future__ import annotations

import numpy as np

import oracle
from xyst_gb300 import lib, mesh, riecg

_ctx = None


def ctx():
    global _ctx
    if _ctx is None:
        _ctx = lib.Context(0)
    return _ctx


def cube_ops(n, jitter=0.2, seed=1, sym=(1, 2, 3, 4, 5, 6), far=(), dirs=(), pres=(),
             numbering="random"):
    m = mesh.cube(n, jitter=jitter, seed=seed, numbering=numbering, perm_seed=seed + 11)
    return riecg.operators(m, sym_sets=sym, far_sets=far, dir_sets=dirs, pre_sets=pres)


def pair(ops, precision="fp64", flux="rusanov", stab2=False, cfl=0.5, const_dt=0.0,
         far_state=None, dir_vals=None, pre_vals=None, context=None):
    """(device RieCG, oracle RieCG) on the same operators and BCs.  A context
    holds one RieCG: two device solvers alive at once need two contexts."""
    d = riecg.RieCG(context or ctx(), ops["coord"], ops["vol"], [None, None, ops["edges"]],
                    [None, None, ops["dint"]], ops["tri"], ops["besym"], flux=flux, stab2=stab2,
                    cfl=cfl, const_dt=const_dt, precision=precision)
    o = oracle.RieCG(ops["coord"], ops["vol"], ops["edges"], ops["dint"], ops["tri"],
                     ops["besym"], flux=flux, stab2=stab2, cfl=cfl, const_dt=const_dt)
    kw = {}
    if ops["sym"][0].size:
        kw["sym"] = ops["sym"]
        o.set_sym(*ops["sym"])
    if ops["far"][0].size:
        kw["far"] = ops["far"]
        kw["far_state"] = far_state
        o.set_far(*ops["far"], *far_state)
    if dir_vals is not None and ops["dirnodes"].size:
        nd = ops["dirnodes"]
        mask = np.ones((nd.size, 5), np.int32)
        vals = dir_vals(ops["coord"][:, nd])
        kw["dir"] = (nd, mask, vals)
        o.set_dir(nd, mask, vals)
    if pre_vals is not None and ops["prenodes"].size:
        npn = ops["prenodes"]
        vals = np.tile(np.asarray(pre_vals, dtype=np.float64), (npn.size, 1))
        kw["pre"] = (npn, vals)
        o.set_pre(npn, vals)
    if kw:
        d.set_bc(**kw)
    return d, o


def relerr(a, b):
    """max |a-b| / max |b| (scale-aware for fields that pass through zero)."""
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
