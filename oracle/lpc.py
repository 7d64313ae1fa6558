"""ORACLE -- test infrastructure only.

FP64 numpy restatement of the learned preconditioner (no reference
counterpart: the reference's ConjugateGradients offers "none" and "jacobi"
only, src/LinearSolver/ConjugateGradients.cpp:213-259).  Used to check the
GPU network's loss and gradients; its own backward pass is checked against
finite differences in tests/test_lpc_oracle.py.

The preconditioned system.  For a matrix A with Dirichlet rows eliminated
(identity rows, decoupled) and a negative-definite remainder (ChoCG's
-K), let s_i = 1/sqrt|a_ii| and, off the diagonal and away from Dirichlet
nodes, e_ij = a_ij s_i s_j, so that A_hat = I - E = -S A S is the SPD
Jacobi-scaled matrix.  With t_ij = sum_{k > j, k != i} e_ik e_kj (the
second-order term of the factorised sparse approximate inverse on A's lower
pattern), the network emits, for every lower edge (i > j),
n_ij = (e_ij + t_ij) * (1 + tanh(o_ij)); with L = I + N (strictly lower N),

    z = M^-1 r:  z_i = r_i (Dirichlet), z_i = -s_i (L L^T (s o r))_i (others),

which is Jacobi for N = 0 and symmetric (negative definite on the -K block)
for any N.

The network.  Node features x_i = [dirichlet_i, sum_j e_ij, sum_j e_ij^2,
degree_i/16]; h0 = relu(x W0 + b0); three message-passing layers
h_l = relu([h_{l-1}, E h_{l-1}] W_l + b_l) (64 wide); a = h3 P, b = h3 Q;
per lower edge z = relu(a_i + b_j + c e_ij + c2 t_ij + d), o_ij = w . z + ob.

The loss is Kaporin's trace functional of the factorised approximate inverse
(the objective that factorised sparse approximate inverses minimise): with
unit-diagonal L, det(L^T A_hat L) = det(A_hat) is fixed, so minimising the
Kaporin condition number of L^T A_hat L is minimising its trace,

    loss = (tr(L^T A_hat L) - n) / n
         = (1/n) sum_j [ -2 sum_i n_ij e_ij + sum_i n_ij^2 - sum_{i != k} n_ij n_kj e_ik ],

d loss / d n_ij = (2/n) (n_ij - e_ij - sum_{k != i} e_ik n_kj).  It needs no
solution of the system, and its minimiser over N on A's lower pattern is the
factorised sparse approximate inverse with unit diagonal.
"""

from __future__ import annotations

import numpy as np

H = 64

SHAPES = [("W0", (4, H)), ("b0", (H,)), ("W1", (2 * H, H)), ("b1", (H,)),
          ("W2", (2 * H, H)), ("b2", (H,)), ("W3", (2 * H, H)), ("b3", (H,)),
          ("Wo", (H, 2 * H)), ("c", (H,)), ("c2", (H,)), ("d", (H,)), ("w", (H,)),
          ("ob", (1,))]


def nparams():
    return int(sum(np.prod(s) for _, s in SHAPES))


def unflatten(theta):
    out, k = {}, 0
    for name, shp in SHAPES:
        m = int(np.prod(shp))
        out[name] = theta[k:k + m].reshape(shp)
        k += m
    return out


def flatten(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("W"):
            d[name] = rng.standard_normal(shp) * np.sqrt(2.0 / shp[0])
        else:
            d[name] = np.zeros(shp)
    d["w"] = np.zeros(H)  # o = 0 at start: n = e + t (second-order factor)
    return flatten(d)


class Graph:
    """Matrix graph of a CSR system (zero-based, full rows) with a Dirichlet mask."""

    def __init__(self, ia, ja, a, dirmask):
        n = ia.size - 1
        self.n = n
        rows = np.repeat(np.arange(n), np.diff(ia))
        diag = a[(rows == ja)]
        self.s = 1.0 / np.sqrt(np.abs(a[ia[:-1] + np.array([np.searchsorted(ja[ia[i]:ia[i + 1]], i)
                                                           for i in range(n)])]))
        self.dir = dirmask.astype(bool)
        off = rows != ja
        keep = off & ~self.dir[rows] & ~self.dir[ja]
        self.r = rows[keep]
        self.c = ja[keep]
        self.e = a[keep] * self.s[self.r] * self.s[self.c]
        lo = self.r > self.c
        self.li, self.lj, self.le = self.r[lo], self.c[lo], self.e[lo]
        self.deg = np.bincount(rows[off], minlength=n).astype(np.float64)
        del diag
        self.lt = self.cross(self.le)

    def cross(self, nval):
        """sum_{k != i} e_ik n_kj at every lower edge (i, j), N strictly lower."""
        import scipy.sparse as sp
        n = self.n
        N = sp.csr_matrix((nval, (self.li, self.lj)), shape=(n, n))
        E = sp.csr_matrix((self.e, (self.r, self.c)), shape=(n, n))
        EN = (E @ N).tocsr()
        return np.asarray(EN[self.li, self.lj]).ravel()

    def E(self, v):
        out = np.zeros((self.n,) + v.shape[1:])
        np.add.at(out, self.r, self.e.reshape((-1,) + (1,) * (v.ndim - 1)) * v[self.c])
        return out

    def features(self):
        rs = np.zeros(self.n)
        np.add.at(rs, self.r, self.e)
        r2 = np.zeros(self.n)
        np.add.at(r2, self.r, self.e * self.e)
        return np.stack([self.dir.astype(np.float64), rs, r2, self.deg / 16.0], axis=1)


def relu(x):
    return np.maximum(x, 0.0)


def forward(theta, g):
    p = unflatten(theta)
    x = g.features()
    cache = {"x": x}
    h = relu(x @ p["W0"] + p["b0"])
    cache["h0"] = h
    for l in (1, 2, 3):
        m = g.E(h)
        inp = np.concatenate([h, m], axis=1)
        h = relu(inp @ p[f"W{l}"] + p[f"b{l}"])
        cache[f"in{l}"] = inp
        cache[f"h{l}"] = h
    ab = h @ p["Wo"]
    a, b = ab[:, :H], ab[:, H:]
    z = a[g.li] + b[g.lj] + np.outer(g.le, p["c"]) + np.outer(g.lt, p["c2"]) + p["d"]
    zr = relu(z)
    o = zr @ p["w"] + p["ob"][0]
    t = np.tanh(o)
    nval = (g.le + g.lt) * (1.0 + t)
    cache.update(a=a, b=b, z=z, zr=zr, t=t)
    return nval, cache


def apply_L(g, nval, v, transpose):
    """(I + N) v or (I + N)^T v, N strictly lower with entries nval at (li, lj)."""
    out = v.copy()
    if transpose:
        np.add.at(out, g.lj, nval * v[g.li])
    else:
        np.add.at(out, g.li, nval * v[g.lj])
    return out


def apply_Mhat(g, nval, v):
    return apply_L(g, nval, apply_L(g, nval, v, True), False)


def Ahat(g, v):
    return v - g.E(v)


def precondition(g, nval, r):
    """z = M^-1 r in the unscaled space."""
    z = -g.s * apply_Mhat(g, nval, g.s * r)
    z[g.dir] = r[g.dir]
    return z


def kaporin(g, nval):
    """Trace loss and its derivative with respect to each lower n_ij."""
    n = g.n
    cross = g.cross(nval)
    loss = float(-2.0 * nval @ g.le + nval @ nval - nval @ cross) / n
    dn = 2.0 * (nval - g.le - cross) / n
    return loss, dn


def loss_grad(theta, g):
    """Loss and d loss / d theta (FP64)."""
    p = unflatten(theta)
    nval, cache = forward(theta, g)
    loss, dn = kaporin(g, nval)
    grads = {k: np.zeros_like(v) for k, v in p.items()}
    do = dn * (g.le + g.lt) * (1.0 - cache["t"] ** 2)
    grads["ob"][0] = do.sum()
    grads["w"] = cache["zr"].T @ do
    dz = np.outer(do, p["w"]) * (cache["z"] > 0)
    grads["c"] = dz.T @ g.le
    grads["c2"] = dz.T @ g.lt
    grads["d"] = dz.sum(0)
    da = np.zeros((g.n, H))
    db = np.zeros((g.n, H))
    np.add.at(da, g.li, dz)
    np.add.at(db, g.lj, dz)
    dab = np.concatenate([da, db], axis=1)
    h3 = cache["h3"]
    grads["Wo"] = h3.T @ dab
    dh = dab @ p["Wo"].T
    for l in (3, 2, 1):
        du = dh * (cache[f"h{l}"] > 0)
        grads[f"W{l}"] = cache[f"in{l}"].T @ du
        grads[f"b{l}"] = du.sum(0)
        dinp = du @ p[f"W{l}"].T
        dh = dinp[:, :H] + g.E(dinp[:, H:])  # E symmetric
    du = dh * (cache["h0"] > 0)
    grads["W0"] = cache["x"].T @ du
    grads["b0"] = du.sum(0)
    return loss, flatten(grads), nval


def adam(theta, grad, m, v, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (Kingma and Ba, "Adam: A Method for Stochastic
    Optimization", ICLR 2015, Algorithm 1) in FP64: the first and second
    moment estimates, their bias corrections 1 - beta^step, and
    theta -= lr * m_hat / (sqrt(v_hat) + eps).  Returns (theta, m, v)."""
    m = beta1 * m + (1.0 - beta1) * grad
    v = beta2 * v + (1.0 - beta2) * grad * grad
    mh = m / (1.0 - beta1 ** step)
    vh = v / (1.0 - beta2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
