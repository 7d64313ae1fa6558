"""The learned-preconditioner oracle (oracle/lpc.py) on the CPU: its backward
pass against finite differences, the factor's algebra, and the first-order
factor's iteration gain over Jacobi in a plain PCG."""

import numpy as np

import oracle
from oracle import lpc
from xyst_gb300 import mesh


def _graph(n=4, seed=3):
    m = mesh.cube(n, jitter=0.2, seed=seed, numbering="random", perm_seed=seed)
    ia, ja, a = oracle.pressure_matrix(m["coord"], m["inpoel"])
    dn = np.unique(m["bface"][4])
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(ia.size - 1)
    a2, b2 = oracle.csr_dirichlet(ia, ja, a, b, dn, np.zeros(dn.size))
    mask = np.zeros(ia.size - 1, bool)
    mask[dn] = True
    return ia, ja, a2, b2, mask


def _dense(ia, ja, a):
    n = ia.size - 1
    A = np.zeros((n, n))
    for i in range(n):
        A[i, ja[ia[i]:ia[i + 1]]] = a[ia[i]:ia[i + 1]]
    return A


def test_backward_matches_finite_differences():
    ia, ja, a2, b2, mask = _graph()
    g = lpc.Graph(ia, ja, a2, mask)
    rng = np.random.default_rng(0)
    theta = lpc.init_params(1) + 0.05 * rng.standard_normal(lpc.nparams())
    loss, grad, _ = lpc.loss_grad(theta, g)
    # central differences along random directions and single coordinates
    h = 1e-6
    scale = np.abs(grad).max()
    for k in range(4):
        v = rng.standard_normal(theta.size)
        lp, _, _ = lpc.loss_grad(theta + h * v, g)
        lm, _, _ = lpc.loss_grad(theta - h * v, g)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grad @ v) < 1e-6 * max(scale, abs(fd))
    for idx in (0, 300, 5000, 20000, 25000, 33000, theta.size - 1):
        e = np.zeros(theta.size)
        e[idx] = 1.0
        lp, _, _ = lpc.loss_grad(theta + h * e, g)
        lm, _, _ = lpc.loss_grad(theta - h * e, g)
        assert abs((lp - lm) / (2 * h) - grad[idx]) < 1e-6 * scale


def test_trace_loss_is_the_kaporin_functional():
    """loss = (tr(L^T A^ L) - n) / n, checked with dense matrices."""
    ia, ja, a2, b2, mask = _graph()
    g = lpc.Graph(ia, ja, a2, mask)
    n = g.n
    nval = g.le * np.random.default_rng(2).uniform(-1, 3, g.le.size)
    L = np.eye(n)
    L[g.li, g.lj] = nval
    E = np.zeros((n, n))
    E[g.r, g.c] = g.e
    Ah = np.eye(n) - E
    loss, dn = lpc.kaporin(g, nval)
    assert abs(loss - (np.trace(L.T @ Ah @ L) - n) / n) < 1e-13
    # its minimiser on the lower pattern (a factorised sparse approximate
    # inverse) has zero gradient
    nf = np.zeros_like(nval)
    for j in range(n):
        sel = np.nonzero(g.lj == j)[0]
        if sel.size:
            P = g.li[sel]
            nf[sel] = np.linalg.solve(Ah[np.ix_(P, P)], g.le[sel])
    _, dnf = lpc.kaporin(g, nf)
    assert np.abs(dnf).max() < 1e-12


def test_factor_algebra():
    """M^-1 is symmetric, the identity on Dirichlet rows, Jacobi for N = 0."""
    ia, ja, a2, b2, mask = _graph()
    g = lpc.Graph(ia, ja, a2, mask)
    n = g.n
    rng = np.random.default_rng(1)
    nval = g.le * rng.uniform(0, 2, g.le.size)
    M = np.stack([lpc.precondition(g, nval, np.eye(n)[k]) for k in range(n)], axis=1)
    assert np.abs(M - M.T).max() < 1e-14 * np.abs(M).max()
    r = rng.standard_normal(n)
    assert np.array_equal(lpc.precondition(g, nval, r)[mask], r[mask])
    d = np.array([a2[ia[i] + np.searchsorted(ja[ia[i]:ia[i + 1]], i)] for i in range(n)])
    zj = lpc.precondition(g, np.zeros_like(nval), r)
    assert np.abs(zj[~mask] - r[~mask] / d[~mask]).max() < 1e-12 * np.abs(zj).max()
    # M^-1 A is positive definite on the interior block
    A = _dense(ia, ja, a2)
    ev = np.linalg.eigvals(M @ A)
    assert ev.real.min() > 0


def _pcg(A, b, apply_m, tol=1e-8, maxit=5000):
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_m(r)
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for it in range(1, maxit + 1):
        q = A @ p
        al = rz / (p @ q)
        x += al * p
        r -= al * q
        if np.linalg.norm(r) < tol * nb:
            return it
        z = apply_m(r)
        rz2 = r @ z
        p = z + rz2 / rz * p
        rz = rz2
    return maxit


def test_first_order_factor_beats_jacobi():
    ia, ja, a2, b2, mask = _graph(n=9, seed=5)
    g = lpc.Graph(ia, ja, a2, mask)
    A = _dense(ia, ja, a2)
    itj = _pcg(A, b2, lambda r: lpc.precondition(g, np.zeros_like(g.le), r))
    itf = _pcg(A, b2, lambda r: lpc.precondition(g, g.le, r))
    assert itf < 0.7 * itj


def _pcg_its(A, b, apply_m, tol=1e-8, maxit=5000):
    """Iterations of a plain PCG (x0 = 0) to ||r|| < tol ||b||."""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_m(r)
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for k in range(1, maxit + 1):
        q = A @ p
        al = rz / (p @ q)
        x += al * p
        r -= al * q
        if np.linalg.norm(r) < tol * nb:
            return k
        z = apply_m(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return maxit


def test_pattern_optimal_factor_bounds_the_learned_one():
    """The trace loss the network is trained on, minimised exactly on the
    factor's pattern (strictly lower part of A, column by column: the
    factorised sparse approximate inverse), is the best a learned N of that
    pattern can reach.  On a ChoCG pressure system (hydrostat node) it gains
    only ~10 % of PCG iterations over the first-order factor N = E, which in
    turn halves Jacobi's: the pattern, not the network, bounds the learned
    preconditioner."""
    m = mesh.cube(11, jitter=0.2, seed=3, numbering="rcm", perm_seed=10)
    ia, ja, a = oracle.pressure_matrix(m["coord"], m["inpoel"])
    A = _dense(ia, ja, a)
    n = A.shape[0]
    A[0, :] = 0.0
    A[:, 0] = 0.0
    A[0, 0] = A[1, 1]
    A *= np.sign(A[1, 1])  # positive definite
    s = 1.0 / np.sqrt(np.abs(np.diag(A)))
    Ah = s[:, None] * A * s[None, :]
    E = np.eye(n) - Ah
    pattern = np.tril(A != 0.0, -1)
    N1 = np.where(pattern, E, 0.0)
    Nf = np.zeros((n, n))
    for j in range(n):
        P = np.nonzero(pattern[:, j])[0]
        if P.size:
            Nf[P, j] = np.linalg.solve(Ah[np.ix_(P, P)], -Ah[P, j])

    def loss(N):
        L = np.eye(n) + N
        return (np.trace(L.T @ Ah @ L) - n) / n

    assert loss(Nf) < loss(N1) < 0.0
    rng = np.random.default_rng(1)
    b = rng.standard_normal(n)
    b[0] = 0.0
    d = np.diag(A)

    def factor(N):
        L = np.eye(n) + N
        return lambda r: s * (L @ (L.T @ (s * r)))

    its_j = _pcg_its(A, b, lambda r: r / d)
    its_1 = _pcg_its(A, b, factor(N1))
    its_f = _pcg_its(A, b, factor(Nf))
    assert its_1 < 0.7 * its_j
    assert its_f < its_1
    assert its_f > 0.8 * its_1
