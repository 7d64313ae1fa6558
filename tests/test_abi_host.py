"""CPU checks of the product library: it builds and loads without a GPU,
exports every symbol include/xg.h declares, and its host-side operator setup
matches the oracle's restatement bit for bit."""

import os
import re

import numpy as np
import pytest

import oracle
from xyst_gb300 import lib, mesh, riecg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            out += re.findall(r"\b(xg_\w+)\s*\(", text)
    return sorted(set(out))


def test_library_exports_all_declared_symbols():
    L = lib.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(syms) <= set(lib.SIGNATURES)


def test_no_gpu_create_fails_cleanly():
    import ctypes as C
    L = lib.load()
    h = C.c_void_p()
    rc = L.xg_create(12345, C.byref(h))
    assert rc != 0 and not h.value


@pytest.mark.parametrize("numbering", ["lex", "random"])
def test_host_setup_matches_oracle(numbering):
    m = mesh.cube(7, jitter=0.2, seed=3, numbering=numbering, perm_seed=5)
    ops = riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=True)
    coord, inpoel = ops["coord"], ops["inpoel"]
    assert np.array_equal(oracle.vol(coord, inpoel), ops["vol"])
    e2, d2 = oracle.domint(coord, inpoel, gid=ops["gid"])
    assert np.array_equal(e2, ops["edges"]) and np.array_equal(d2, ops["dint"])
    n2, nn2, ss = oracle.sym_bc(coord, ops["bface"], [1, 2, 3, 4, 5, 6])
    assert np.array_equal(n2, ops["sym"][0]) and np.array_equal(nn2, ops["sym"][1])
    assert ss == ops["symset"]
    # ChoCG coefficients
    e5, d5 = riecg.edges(coord, inpoel, gid=ops["gid"], ncoef=5)
    o5, od5 = oracle.domint(coord, inpoel, gid=ops["gid"], ncoef=5)
    assert np.array_equal(e5, o5) and np.array_equal(d5, od5)


@pytest.mark.parametrize("ncoef", [3, 5])
def test_threaded_edge_integrals_match_oracle(ncoef):
    """Large enough (15,625 nodes) for the row-parallel edge integrals: still
    the oracle's serial element-order sums, bit for bit."""
    m = mesh.cube(25, jitter=0.2, seed=4, numbering="random", perm_seed=6)
    ops = riecg.operators(m, sym_sets=[1, 2, 3, 4, 5, 6], renumber=True)
    e, d = riecg.edges(ops["coord"], ops["inpoel"], gid=ops["gid"], ncoef=ncoef)
    eo, do = oracle.domint(ops["coord"], ops["inpoel"], gid=ops["gid"], ncoef=ncoef)
    assert np.array_equal(e, eo) and np.array_equal(d, do)


def test_threaded_pressure_matrix_matches_oracle():
    """The row-parallel ChoCG::prelhs matrix (15,625 rows): the oracle's
    serial element-order sums, bit for bit."""
    from xyst_gb300 import cg
    m = mesh.cube(25, jitter=0.2, seed=4, numbering="random", perm_seed=6)
    ia, ja, a = cg.pressure_matrix(m["coord"], m["inpoel"])
    io, jo, ao = oracle.pressure_matrix(m["coord"], m["inpoel"])
    assert np.array_equal(np.asarray(ia, np.int64), np.asarray(io, np.int64))
    assert np.array_equal(np.asarray(ja, np.int64), np.asarray(jo, np.int64))
    assert np.array_equal(a, ao)


def test_rcm_is_permutation_and_reduces_bandwidth():
    m = mesh.cube(9, numbering="random", perm_seed=1)
    perm = riecg.rcm(m["inpoel"], m["coord"].shape[1])
    assert np.array_equal(np.sort(perm), np.arange(perm.size))
    def bw(ip):
        return np.abs(ip[:, :, None] - ip[:, None, :]).max()
    assert bw(perm[m["inpoel"]]) < bw(m["inpoel"]) / 4


def test_nonpositive_jacobian_rejected():
    m = mesh.cube(3)
    ip = m["inpoel"].copy()
    ip[0, [1, 2]] = ip[0, [2, 1]]
    with pytest.raises(ValueError):
        riecg.volumes(m["coord"], ip)


def test_boundary_sets_short_circuit():
    bface = {1: 0, 2: 0, 3: 0}
    assert riecg.boundary_sets(bface, {2}) == [1, 2, 3]
    assert riecg.boundary_sets(bface, {7}) == []
    assert riecg.boundary_sets(bface, set()) == []


def test_pressure_matrix_matches_oracle():
    from xyst_gb300 import cg
    m = mesh.cube(6, jitter=0.2, seed=4, numbering="random", perm_seed=3)
    ia, ja, a = cg.pressure_matrix(m["coord"], m["inpoel"])
    oia, oja, oa = oracle.pressure_matrix(m["coord"], m["inpoel"])
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja) and np.array_equal(a, oa)


def test_header_is_c_and_links_from_c(tmp_path):
    """include/xg.h is plain C99: a C translation unit that includes it, links
    against libxg and calls the host entry points (mesh volumes, the error
    path of xg_create without a GPU) builds and runs."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    so = lib.load()._name
    src = tmp_path / "c_abi.c"
    src.write_text(r'''
#include <stdio.h>
#include "xg.h"
int main(void) {
  /* one right tetrahedron of volume 1/6 */
  const double coord[12] = {0, 1, 0, 0,  0, 0, 1, 0,  0, 0, 0, 1};
  const uint64_t inpoel[4] = {0, 1, 2, 3};
  double vol[4] = {0, 0, 0, 0};
  if (xg_mesh_vol(4, coord, 1, inpoel, vol) != XG_OK) return 1;
  for (int i = 0; i < 4; ++i)
    if (vol[i] < 1.0 / 24 - 1e-15 || vol[i] > 1.0 / 24 + 1e-15) return 2;
  xg_ctx* ctx = 0;
  if (xg_create(12345, &ctx) == XG_OK || ctx != 0) return 3;
  printf("ok\n");
  return 0;
}
''')
    exe = tmp_path / "c_abi"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), so, "-Wl,-rpath," + os.path.dirname(so), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)


# ---------------------------------------------------------------- edge cases

# one tetrahedron with unit legs along the axes (J = 1, volume 1/6)
TET_COORD = np.array([[0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]])
TET = np.array([[0, 1, 2, 3]])


def test_host_setup_rejects_bad_input():
    """Node ids past the node count, an empty node set and a degenerate tet
    come back as status codes (the wrappers raise), never as a crash."""
    bad = np.array([[0, 1, 2, 4]])
    with pytest.raises(RuntimeError):
        riecg.rcm(bad, 4)
    with pytest.raises(ValueError):
        riecg.volumes(TET_COORD, bad)
    with pytest.raises(RuntimeError):
        riecg.edges(TET_COORD, bad)
    with pytest.raises(RuntimeError):
        riecg.rcm(TET, 0)
    flat = TET_COORD.copy()
    flat[2, 3] = 0.0  # all four nodes in one plane: J = 0
    with pytest.raises(ValueError):
        riecg.volumes(flat, TET)
    from xyst_gb300 import cg
    with pytest.raises(ValueError):
        cg.pressure_matrix(TET_COORD, bad)


def test_single_tet_operators():
    """The operators of one tetrahedron against their closed forms: nodal
    volumes J/24 each, six edges oriented from the smaller id, and the
    pressure matrix -grad_a.grad_b V (symmetric, zero row sums)."""
    v = riecg.volumes(TET_COORD, TET)
    assert np.allclose(v, 1.0 / 24.0, rtol=0, atol=1e-16)
    e, d = riecg.edges(TET_COORD, TET)
    assert e.shape == (6, 2) and d.shape == (6, 3)
    assert np.all(e[:, 0] < e[:, 1])
    from xyst_gb300 import cg
    ia, ja, a = cg.pressure_matrix(TET_COORD, TET)
    A = np.zeros((4, 4))
    for i in range(4):
        A[i, ja[ia[i]:ia[i + 1]]] = a[ia[i]:ia[i + 1]]
    grads = np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    assert np.allclose(A, -grads @ grads.T / 6.0, rtol=0, atol=1e-15)
    assert np.allclose(A.sum(1), 0.0, atol=1e-15)


def test_rcm_disconnected_and_isolated_nodes():
    """Two separate tetrahedra and a node that no element uses: the
    renumbering is still a permutation of all nine nodes, and each connected
    piece takes consecutive numbers."""
    ip = np.array([[0, 1, 2, 3], [4, 5, 6, 7]])
    r = riecg.rcm(ip, 9)
    assert sorted(r) == list(range(9))
    for piece in ([0, 1, 2, 3], [4, 5, 6, 7]):
        nums = np.sort(r[piece])
        assert nums[-1] - nums[0] == 3


def test_bnorm_rejects_nodes_off_the_faces():
    faces = np.array([[0, 2, 1]])  # the z = 0 face of the tetrahedron
    n = riecg.bnorm(TET_COORD, faces, np.array([0, 1, 2]))
    assert np.allclose(np.abs(n[:, 2]), 1.0) and np.allclose(n[:, :2], 0.0)
    with pytest.raises(RuntimeError):
        riecg.bnorm(TET_COORD, faces, np.array([3]))
