"""ConjugateGradients on the GPU against the oracle and the reference's
unit-test known answers."""

import numpy as np
import pytest

import oracle
from common import (POISSON_PROBLEMS, check_poisson, dirichlet_matrix_only, golden, laplacian_14,
                    poisson_case)
from gpu_util import ctx, relerr
from xyst_gb300 import cg, mesh

pytestmark = pytest.mark.gpu


def _system(n=9, seed=2, ndir_face=1):
    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed)
    ia, ja, a = cg.pressure_matrix(m["coord"], m["inpoel"])
    dn = np.unique(m["bface"][ndir_face])
    rng = np.random.default_rng(seed)
    # scaled well above the solver's absolute (p,q) breakdown guard
    # (src/LinearSolver/ConjugateGradients.cpp:681-690)
    dv = rng.standard_normal(dn.size) * 1e3
    b = rng.standard_normal(ia.size - 1) * 1e4
    return m, ia, ja, a, dn, dv, b


def test_mult_matches_oracle():
    m, ia, ja, a, *_ = _system()
    A = cg.ConjugateGradients(ctx(), ia, ja, a)
    x = np.random.default_rng(1).standard_normal(ia.size - 1)
    assert relerr(A.mult(x), oracle.csr_mult(ia, ja, a, x)) < 1e-14


def test_onebased_reference_layout():
    m, ia, ja, a, *_ = _system(6)
    A = cg.ConjugateGradients(ctx(), ia + 1, ja + 1, a, base=1)
    x = np.arange(ia.size - 1, dtype=np.float64)
    assert relerr(A.mult(x), oracle.csr_mult(ia, ja, a, x)) < 1e-14


@pytest.mark.parametrize("case", ["dof1", "dof3"])
def test_laplace_golden(case):
    d = golden("cg_laplace")
    maxit, tol, normb_ex, normres_ex = d[case]
    ia, ja, a = laplacian_14(d)
    n = ia.size - 1
    a = dirichlet_matrix_only(ia, ja, a, 0)
    if case == "dof3":
        import scipy.sparse as sp
        A = sp.kron(sp.csr_matrix((a, ja, ia), shape=(n, n)), sp.eye(3)).tocsr()
        A.sort_indices()
        ia, ja, a = A.indptr.astype(np.int64), A.indices.astype(np.int64), A.data
        n *= 3
    s = cg.ConjugateGradients(ctx(), ia, ja, a)
    s.init(x=np.zeros(n), b=np.ones(n), pc="none")
    s.solve(int(maxit), float(tol))
    assert abs(s.normb - normb_ex) < 1e-12
    assert abs(s.normr - normres_ex) < 1e-12
    assert s.converged()


@pytest.mark.parametrize("pc", ["jacobi", "none"])
def test_pcg_dirichlet_matches_oracle(pc):
    m, ia, ja, a, dn, dv, b = _system()
    n = ia.size - 1
    a2, b2 = oracle.csr_dirichlet(ia, ja, a, b, dn, dv)
    x0 = np.zeros(n)
    xo, ito, nro, nbo, co = oracle.pcg(ia, ja, a2, b2, x0, 2000, 1e-10, pc=pc)
    s = cg.ConjugateGradients(ctx(), ia, ja, a)
    s.init(x=x0, b=b, dirbc=(dn, dv), apply=True, pc=pc)
    s.solve(2000, 1e-10)
    assert s.converged() and co
    assert abs(s.it() - ito) <= max(2, 0.02 * ito)  # reduction order differs
    assert abs(s.normb / nbo - 1) < 1e-13
    x = s.solution()
    assert relerr(x, xo) < 1e-8
    # residual of the eliminated system, evaluated by the oracle
    res = b2 - oracle.csr_mult(ia, ja, a2, x)
    assert np.linalg.norm(res) < 1e-10 * nbo
    # the stored matrix is restored: plain products are unaffected
    assert relerr(s.mult(x), oracle.csr_mult(ia, ja, a, x)) < 1e-14


@pytest.mark.parametrize("name", sorted(POISSON_PROBLEMS))
def test_poisson_reference_baselines_on_gpu(name):
    """The reference's ChoCG Poisson regressions through the ConjugateGradients
    drop-in on the GPU: ChoCG::prelhs's matrix, the problem's right-hand
    side pr V and Dirichlet values, FP64 PCG without preconditioner to 1e-6
    (at most 100 iterations): the reference's diagnostics within 1e-8 and,
    for poisson_const, its pressure field."""
    d, coord, inpoel, v, b, dn, dv, exact, neu = poisson_case(name, oracle.vol)
    ia, ja, a = oracle.pressure_matrix(coord, inpoel)
    s = cg.ConjugateGradients(ctx(), ia, ja, a)
    s.init(x=np.zeros(coord.shape[1]), b=b, neubc=neu, dirbc=(dn, dv), apply=True, pc="none")
    s.solve(100, 1e-6)
    assert s.converged()
    check_poisson(name, s.solution(), v, exact, d, coord)


def test_warm_start_and_maxit():
    m, ia, ja, a, dn, dv, b = _system()
    n = ia.size - 1
    s = cg.ConjugateGradients(ctx(), ia, ja, a)
    s.init(x=np.zeros(n), b=b, dirbc=(dn, dv), apply=True)
    s.solve(5, 1e-12)
    assert s.it() == 5 and not s.converged()
    a2, b2 = oracle.csr_dirichlet(ia, ja, a, b, dn, dv)
    xo, ito, *_ = oracle.pcg(ia, ja, a2, b2, np.zeros(n), 5, 1e-12)
    assert relerr(s.solution(), xo) < 1e-10
    # warm start from the previous solution (x omitted), as ChoCG does
    s.init(b=b, dirbc=(dn, dv), apply=True)
    s.solve(2000, 1e-10)
    assert s.converged()


def test_mixed_precision_refinement():
    m, ia, ja, a, dn, dv, b = _system(11)
    n = ia.size - 1
    a2, b2 = oracle.csr_dirichlet(ia, ja, a, b, dn, dv)
    s = cg.ConjugateGradients(ctx(), ia, ja, a)
    s.init(x=np.zeros(n), b=b, dirbc=(dn, dv), apply=True)
    s.solve_mixed(50, 1e-8, inner_tol=1e-3)
    assert s.converged() and s.outer >= 2
    x = s.solution()
    res = b2 - oracle.csr_mult(ia, ja, a2, x)
    assert np.linalg.norm(res) < 1e-8 * np.linalg.norm(b2)


def test_breakdown_guard_modes():
    """A small right-hand side (ChoCG's pressure increments on fine meshes):
    with the reference's absolute (p,q) test the FP64 solve stops short of the
    tolerance exactly where the oracle does; with the underflow-only guard it
    runs to the tolerance."""
    m, ia, ja, a, dn, dv, b = _system(9)
    b = b * 1e-9
    dv = np.zeros_like(dv)
    A = cg.ConjugateGradients(ctx(), ia, ja, a)
    aa, bb = oracle.csr_dirichlet(ia, ja, a, b, dn, dv)
    _, ito, _, _, conv_o = oracle.pcg(ia, ja, aa, bb, np.zeros(ia.size - 1), 5000, 1e-10)
    A.init(x=np.zeros(A.n), b=b, dirbc=(dn, dv), apply=True, pc="jacobi")
    A.solve(5000, 1e-10)
    assert not conv_o and not A.converged() and abs(A.it() - ito) <= 1
    A.set_guard("underflow")
    A.init(x=np.zeros(A.n), b=b, dirbc=(dn, dv), apply=True, pc="jacobi")
    A.solve(5000, 1e-10)
    assert A.converged() and A.normr < 1e-10 * A.normb
    A.set_guard("reference")
