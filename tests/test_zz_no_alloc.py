"""xg_riecg_dt_noalloc: the allocation-free CFL time step, for callers that
cannot allocate device memory (their own pool owns the GPU's memory, or
cudaMalloc is not allowed where they run) and keep the RieCG state in device
buffers of their own.  Its answer must equal the context-based xg_riecg_dt of
an FP64 context on the same state, call after call: consecutive no-alloc
calls share the library's fixed scratch array (the context's dt uses its own
allocation), so a second call must not see the first call's block minima."""

import ctypes as C

import numpy as np
import pytest

from common import wave_ic
from gpu_util import cube_ops, pair

pytestmark = pytest.mark.gpu


def _noalloc_dt(lib, torch, U, vol, cfl=0.5, gamma=1.4, const_dt=0.0):
    Ud = torch.as_tensor(np.ascontiguousarray(U), device="cuda")
    vd = torch.as_tensor(np.ascontiguousarray(vol), device="cuda")
    torch.cuda.synchronize()
    out = C.c_double(-1.0)
    rc = lib.xg_riecg_dt_noalloc(C.c_void_p(Ud.data_ptr()), C.c_void_p(vd.data_ptr()),
                                 U.shape[0], gamma, cfl, const_dt,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                 C.byref(out))
    return rc, out.value


@pytest.mark.parametrize("n", [9, 41])
def test_dt_noalloc_matches_context_dt_twice(n):
    """9^3 = 729 nodes (3 blocks) and 41^3 = 68,921 nodes (270 blocks: the
    final pass strides over more than one sweep of block minima)."""
    torch = pytest.importorskip("torch")
    ops = cube_ops(n)
    d, _ = pair(ops)
    lib = d.lib
    states = [wave_ic(ops["coord"])]
    U2 = wave_ic(ops["coord"])
    U2[:, 1:4] *= 3.0  # faster flow: a different minimum than the first call
    U2[:, 4] += 0.5 * (U2[:, 1:4] ** 2).sum(1) / U2[:, 0]
    states.append(U2)
    for U in states:
        d.set_state(U)
        expect = d.dt()
        rc, got = _noalloc_dt(lib, torch, U, ops["vol"])
        assert rc == 0
        assert abs(got / expect - 1.0) < 1e-14


def test_dt_noalloc_rejects_oversize_and_const_dt():
    torch = pytest.importorskip("torch")
    ops = cube_ops(4)
    d, _ = pair(ops)
    lib = d.lib
    U = wave_ic(ops["coord"])
    Ud = torch.as_tensor(U, device="cuda")
    vd = torch.as_tensor(ops["vol"], device="cuda")
    out = C.c_double(-1.0)
    rc = lib.xg_riecg_dt_noalloc(C.c_void_p(Ud.data_ptr()), C.c_void_p(vd.data_ptr()),
                                 16_777_217, 1.4, 0.5, 0.0, None, C.byref(out))
    assert rc == 1 and out.value == -1.0  # XG_ERR_ARG before touching the device
    rc, got = _noalloc_dt(lib, torch, U, ops["vol"], const_dt=2.5e-3)
    assert rc == 0 and got == 2.5e-3


def test_dt_noalloc_fp64_formula_against_fp32_context():
    """An FP32-flux context forms its dt in FP32 arithmetic; the no-alloc call
    always uses the FP64 formula, so the two agree to FP32 rounding only."""
    torch = pytest.importorskip("torch")
    ops = cube_ops(9)
    d, _ = pair(ops, precision="fp32")
    U = wave_ic(ops["coord"])
    d.set_state(U)
    expect = d.dt()
    rc, got = _noalloc_dt(d.lib, torch, U, ops["vol"])
    assert rc == 0
    assert abs(got / expect - 1.0) < 1e-6
