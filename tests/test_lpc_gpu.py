"""The factored and learned preconditioners on the GPU against the oracle
(oracle/lpc.py): preconditioner application, the network's loss and
gradient, and the iteration gain over Jacobi PCG."""

import numpy as np
import pytest

import oracle
from oracle import lpc as olpc
from gpu_util import ctx, relerr
from xyst_gb300 import cg, lpc, mesh

pytestmark = pytest.mark.gpu


def _system(n=9, seed=2, numbering="random"):
    m = mesh.cube(n, jitter=0.2, seed=seed, numbering=numbering, perm_seed=seed)
    ia, ja, a = cg.pressure_matrix(m["coord"], m["inpoel"])
    dn = np.unique(m["bface"][4])
    rng = np.random.default_rng(seed)
    dv = rng.standard_normal(dn.size) * 1e3
    b = rng.standard_normal(ia.size - 1) * 1e4
    a2, b2 = oracle.csr_dirichlet(ia, ja, a, b, dn, dv)
    mask = np.zeros(ia.size - 1, bool)
    mask[dn] = True
    return dict(ia=ia, ja=ja, a=a, a2=a2, b=b, b2=b2, dn=dn, dv=dv, mask=mask)


def _cg(S, pc, model=None, scale=1.0):
    s = cg.ConjugateGradients(ctx(), S["ia"], S["ja"], S["a"])
    if pc == "factor":
        s.set_factor(model, scale)
    s.init(x=np.zeros(s.n), b=S["b"], dirbc=(S["dn"], S["dv"]), apply=True, pc=pc)
    return s


def _random_params(seed):
    rng = np.random.default_rng(seed)
    t = lpc.init_params(seed, wscale=1.0).astype(np.float64)
    return (t + 0.05 * rng.standard_normal(t.size)).astype(np.float32)


@pytest.mark.parametrize("scale", [0.0, 1.0, 0.7])
def test_scaled_factor_matches_oracle(scale):
    S = _system()
    s = _cg(S, "factor", scale=scale)
    g = olpc.Graph(S["ia"], S["ja"], S["a2"], S["mask"])
    r = np.random.default_rng(4).standard_normal(s.n)
    z = s.precondition(r)
    zo = olpc.precondition(g, scale * g.le, r)
    assert relerr(z, zo) < 2e-6  # N and s in FP32


def test_factor_pcg_converges_with_fewer_iterations():
    S = _system(n=17, seed=4, numbering="rcm")
    sj = _cg(S, "jacobi")
    sj.solve(5000, 1e-10)
    sf = _cg(S, "factor")
    sf.solve(5000, 1e-10)
    assert sj.converged() and sf.converged()
    assert sf.it() < 0.7 * sj.it()
    x = sf.solution()
    res = S["b2"] - oracle.csr_mult(S["ia"], S["ja"], S["a2"], x)
    assert np.linalg.norm(res) < 1e-10 * np.linalg.norm(S["b2"])
    assert relerr(x, sj.solution()) < 1e-7


def test_factor_mixed_precision():
    S = _system(n=13, seed=6, numbering="rcm")
    s = _cg(S, "factor")
    s.solve_mixed(50, 1e-8, inner_tol=1e-3)
    assert s.converged()
    x = s.solution()
    res = S["b2"] - oracle.csr_mult(S["ia"], S["ja"], S["a2"], x)
    assert np.linalg.norm(res) < 1e-8 * np.linalg.norm(S["b2"])


@pytest.mark.parametrize("precision,tol", [("fp32", 2e-5), ("bf16", 3e-2)])
def test_network_factor_matches_oracle(precision, tol):
    S = _system()
    theta = _random_params(3)
    model = lpc.LearnedPreconditioner(ctx(), precision=precision, params=theta)
    s = _cg(S, "factor", model=model)
    g = olpc.Graph(S["ia"], S["ja"], S["a2"], S["mask"])
    nval, _ = olpc.forward(theta.astype(np.float64), g)
    assert np.abs(nval - g.le).max() > 0.05 * np.abs(g.le).max()  # the network does something
    r = np.random.default_rng(5).standard_normal(s.n)
    assert relerr(s.precondition(r), olpc.precondition(g, nval, r)) < tol
    model.close()


def test_network_gradient_matches_oracle():
    S = _system(n=7, seed=8)
    s = _cg(S, "jacobi")
    theta = _random_params(9)
    model = lpc.LearnedPreconditioner(ctx(), precision="fp32", params=theta)
    model.zero_grads()
    loss = model.grad(s)
    gg = model.grads().astype(np.float64)
    g = olpc.Graph(S["ia"], S["ja"], S["a2"], S["mask"])
    lo, go, _ = olpc.loss_grad(theta.astype(np.float64), g)
    assert abs(loss - lo) < 1e-5 * abs(lo)
    k = 0
    for name, shp in olpc.SHAPES:
        m = int(np.prod(shp))
        a, b = gg[k:k + m], go[k:k + m]
        assert np.abs(a - b).max() <= 1e-3 * np.abs(go).max() + 1e-4 * np.abs(b).max(), name
        k += m
    # accumulation: a second call doubles the gradient, bit for bit
    model.grad(s)
    assert np.array_equal(model.grads().astype(np.float64), 2 * gg)
    model.close()


def test_network_gradient_tensor_cores_matches_oracle():
    """The BF16 path: forward layers, the backward data products dY W^T and
    the weight gradients X^T dY on the 5th-generation tensor cores
    (tcgen05.mma, BF16 operands, FP32 accumulation in TMEM).  Against the
    FP64 oracle: loss within 1e-2 relative; every parameter group's
    gradient within 3e-2 of the largest oracle gradient entry (BF16 rounds
    each operand to 8 significant bits); the whole gradient vector's cosine
    similarity above 0.999; the second call doubles the gradient bit for
    bit (fixed-order partials)."""
    S = _system(n=13, seed=8)
    s = _cg(S, "jacobi")
    theta = _random_params(9)
    model = lpc.LearnedPreconditioner(ctx(), precision="bf16", params=theta)
    model.zero_grads()
    loss = model.grad(s)
    gg = model.grads().astype(np.float64)
    g = olpc.Graph(S["ia"], S["ja"], S["a2"], S["mask"])
    lo, go, _ = olpc.loss_grad(theta.astype(np.float64), g)
    assert abs(loss - lo) < 1e-2 * abs(lo)
    scale = np.abs(go).max()
    k = 0
    for name, shp in olpc.SHAPES:
        m = int(np.prod(shp))
        assert np.abs(gg[k:k + m] - go[k:k + m]).max() <= 3e-2 * scale, name
        k += m
    cos = gg @ go / (np.linalg.norm(gg) * np.linalg.norm(go))
    assert cos > 0.999, cos
    model.grad(s)
    assert np.array_equal(model.grads().astype(np.float64), 2 * gg)
    model.close()


def test_adam_matches_oracle():
    """Two device Adam steps against the oracle's FP64 Adam (Kingma and Ba,
    Algorithm 1) on the same gradient: parameters within FP32 rounding."""
    S = _system(n=7, seed=8)
    s = _cg(S, "jacobi")
    theta = _random_params(11)
    model = lpc.LearnedPreconditioner(ctx(), precision="fp32", params=theta)
    t = theta.astype(np.float64)
    m = np.zeros_like(t)
    v = np.zeros_like(t)
    for step in (1, 2):
        model.zero_grads()
        model.grad(s)
        grad = model.grads().astype(np.float64)
        model.adam(lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8)
        t, m, v = olpc.adam(t, grad, m, v, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8)
        got = model.params().astype(np.float64)
        assert np.abs(got - t).max() <= 1e-6 * np.abs(t).max() + 2e-6
    model.close()


def test_mixed_solve_smooth_rhs_tracks_fp64():
    """The mixed-precision solve on a ChoCG pressure system with a smooth
    right-hand side (its solution dominated by A's smoothest modes): the FP32
    inner iteration forms A p' as sum a_ij (p'_j - p'_i) + rowsum p'_i and
    accumulates the correction in FP64, so it converges like the FP64 PCG
    with the same factor (at most 30 % more iterations) to the same
    solution.  A plain FP32 row sum or an FP32 correction made the solve
    stall on such systems."""
    c = ctx()
    sysd = lpc.chocg_system(None, 49, 5, rhs="smooth")
    s = cg.ConjugateGradients(c, sysd["ia"], sysd["ja"], sysd["a"])
    s.set_guard("underflow")
    dirbc = (sysd["dirnodes"], sysd["dirvals"])
    s.set_factor(None, 1.0)
    s.init(x=np.zeros(s.n), b=sysd["b"], dirbc=dirbc, apply=True, pc="factor")
    s.solve(20000, 1e-10)
    it64, x64 = s.it(), s.solution()
    assert s.converged()
    s.init(x=np.zeros(s.n), b=sysd["b"], dirbc=dirbc, apply=True, pc="factor")
    s.solve_mixed(1000, 1e-10, inner_tol=0.1, inner_maxit=20000)
    assert s.converged()
    assert s.it() <= 1.3 * it64, (s.it(), it64)
    assert relerr(s.solution(), x64) < 1e-7


def test_training_lowers_loss_and_beats_first_order():
    c = ctx()
    train = [lpc.training_system(c, lpc.pressure_system(c, n, seed))
             for n, seed in ((9, 1), (11, 2))]
    model = lpc.LearnedPreconditioner(c, precision="bf16", seed=0)
    hist = model.train(train, 60, lr=2e-3)
    assert hist[-1] < hist[0]
    test = lpc.pressure_system(c, 15, 77)
    s = cg.ConjugateGradients(c, test["ia"], test["ja"], test["a"])
    itj, cj = lpc.iterations(s, test, "jacobi")
    itf, cf = lpc.iterations(s, test, "factor")
    itl, cl = lpc.iterations(s, test, "factor", model=model)
    assert cj and cf and cl
    assert itl < 0.6 * itj
    assert itl < itf  # better than the first-order factor N = e
    model.close()
