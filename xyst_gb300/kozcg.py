"""KozCG hot path on the GPU: ``rhs`` is ``kozak::rhs``, ``bc`` is
``KozCG::BC``, ``dt`` is ``KozCG::dt`` and ``run`` chains whole KozCG steps
(residual, flux-corrected transport, BCs) on the device
(src/Inciter/KozCG.cpp, src/Physics/Kozak.cpp).  U is (npoin, 5) node-major."""

from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import Context, KozcgParams, f64, i32, p, u64


class KozCG:
    def __init__(self, ctx: Context, coord, vol, inpoel, gamma=1.4, cfl=0.5, const_dt=0.0,
                 fct=True, ctau=1.0, fctclip=False, fctsys=(), precision="fp64"):
        """fctsys: zero-based component ids limited as a system.  precision
        "fp32" forms the element terms in FP32 and sums them into FP64 nodes."""
        self.ctx = ctx
        self.lib = ctx.lib
        coord = f64(coord)
        self.n = coord.shape[1]
        mask = 0
        for c in fctsys:
            mask |= 1 << int(c)
        prec = {"fp64": 0, "fp32": 1}[precision]
        prm = KozcgParams(gamma, cfl, const_dt, int(fct), ctau, int(fctclip), mask, prec)
        v = f64(vol)
        ip = u64(inpoel).reshape(-1)
        self._keep = (coord, v, ip)
        ctx.check(self.lib.xg_kozcg_setup(ctx.h, C.byref(prm), self.n, p(coord), p(v),
                                          ip.size // 4, p(ip)))

    def set_bc(self, sym=None, dir=None):
        ns, sn, sv = 0, None, None
        if sym is not None and len(sym[0]):
            sn, sv = u64(sym[0]), f64(sym[1]).reshape(-1)
            ns = sn.size
        nd, dn, dm, dv = 0, None, None, None
        if dir is not None and len(dir[0]):
            dn, dm, dv = u64(dir[0]), i32(dir[1]).reshape(-1), f64(dir[2]).reshape(-1)
            nd = dn.size
        self._bc = (sn, sv, dn, dm, dv)
        self.ctx.check(self.lib.xg_kozcg_set_bc(self.ctx.h, ns, p(sn), p(sv), nd, p(dn), p(dm),
                                                p(dv)))

    def set_state(self, U, t=0.0):
        U = f64(U)
        self.ctx.check(self.lib.xg_kozcg_set_state(self.ctx.h, p(U), t))

    def state(self):
        U = np.zeros((self.n, 5))
        t = C.c_double()
        self.ctx.check(self.lib.xg_kozcg_get_state(self.ctx.h, p(U), C.byref(t)))
        return U, t.value

    def rhs(self, U, dt):
        U = f64(U)
        R = np.zeros((self.n, 5))
        self.ctx.check(self.lib.xg_kozcg_rhs(self.ctx.h, p(U), dt, p(R)))
        return R

    def bc(self):
        self.ctx.check(self.lib.xg_kozcg_bc(self.ctx.h))

    def dt(self):
        d = C.c_double()
        self.ctx.check(self.lib.xg_kozcg_dt(self.ctx.h, C.byref(d)))
        return d.value

    def run(self, nstep):
        dts = np.zeros(nstep)
        ms = C.c_float()
        self.ctx.check(self.lib.xg_kozcg_run(self.ctx.h, nstep, p(dts), C.byref(ms)))
        return dts, ms.value

    def step(self, dt):
        """One step of the given dt (the last step cut to the final time)."""
        self.ctx.check(self.lib.xg_kozcg_step(self.ctx.h, float(dt)))

    def set_source(self, problem, prm=None):
        """The manufactured source of kozak::rhs (riecg.SOURCES names the
        problems; src/Physics/Kozak.cpp:125-132, 161-170) with the
        control-file parameters prm = alpha, beta[3], kappa, r0, p0, ce."""
        from .riecg import SOURCES
        self._src = None if prm is None else f64(np.asarray(prm, dtype=np.float64).reshape(8))
        self.ctx.check(self.lib.xg_kozcg_set_source(self.ctx.h, SOURCES[problem],
                                                    None if self._src is None else p(self._src)))
