"""Shared test inputs: reference golden fixtures and seeded cube problems."""

from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def sod_mesh(scheme="RieCG"):
    d = golden("riecg_sod" if scheme == "RieCG" else "kozcg_sod")
    bface = {int(k[5:]): d[k] for k in d.files if k.startswith("bface")}
    return {"coord": d["coord"], "inpoel": d["inpoel"], "bface": bface}, d


def sod_ic(coord, gamma=1.4):
    """Sod shock tube IC (problems::sod::ic, src/Physics/Problems.cpp:371-404)."""
    x = coord[0]
    r = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    U = np.zeros((coord.shape[1], 5))
    U[:, 0] = r
    U[:, 4] = p / (gamma - 1.0)
    return U


def problem_state(problem, prm, coord, t=0.0, gamma=5.0 / 3.0):
    """A manufactured-solution problem's analytic state at time t, conserved
    variables (the problems' ic functions, src/Physics/Problems.cpp:
    nonlinear_energy_growth 117-151, rayleigh_taylor 226-258, taylor_green
    409-428, vortical_flow 453-478); prm = alpha, beta[3], kappa, r0, p0, ce."""
    a, b0, b1, b2, k, r0, p0, ce = prm
    x, y, z = coord
    n = x.size
    r = np.ones(n)
    u = np.zeros(n)
    v = np.zeros(n)
    w = np.zeros(n)
    if problem == "taylor_green":
        p = 10.0 + r / 4.0 * (np.cos(2.0 * np.pi * x) + np.cos(2.0 * np.pi * y))
        u = np.sin(np.pi * x) * np.cos(np.pi * y)
        v = -np.cos(np.pi * x) * np.sin(np.pi * y)
        rE = p / (gamma - 1.0) + 0.5 * r * (u * u + v * v)
    elif problem == "vortical_flow":
        u, v, w = a * x - k * y, k * x + a * y, -2.0 * a * z
        rE = (u * u + v * v + w * w) / 2.0 + (p0 - 2.0 * a * a * z * z) / (gamma - 1.0)
    elif problem == "nonlinear_energy_growth":
        h = np.cos(b0 * np.pi * x) * np.cos(b1 * np.pi * y) * np.cos(b2 * np.pi * z)
        r = r0 + np.exp(-a * t) * (1.0 - x * x - y * y - z * z)
        rE = r * (-3.0 * (ce + k * h * h * t)) ** (-1.0 / 3.0)
    else:  # rayleigh_taylor
        gx = b0 * x * x + b1 * y * y + b2 * z * z
        r = r0 - gx
        ft = np.cos(k * np.pi * t)
        u = ft * z * np.sin(np.pi * x)
        v = ft * z * np.cos(np.pi * y)
        w = ft * (-0.5 * np.pi * z * z * (np.cos(np.pi * x) - np.sin(np.pi * y)))
        rE = (p0 + a * gx) / (gamma - 1.0) + 0.5 * r * (u * u + v * v + w * w)
    return np.stack([r, r * u, r * v, r * w, rE], axis=1)


def wave_ic(coord, gamma=1.4):
    """Smooth density wave rho = 1 + 0.2 sin(2 pi x) sin(2 pi y) sin(2 pi z),
    u = (1, 0.5, 0.25), p = 1."""
    x, y, z = coord
    r = 1.0 + 0.2 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)
    u = np.array([1.0, 0.5, 0.25])
    U = np.zeros((coord.shape[1], 5))
    U[:, 0] = r
    U[:, 1:4] = r[:, None] * u[None, :]
    U[:, 4] = 1.0 / (gamma - 1.0) + 0.5 * r * (u @ u)
    return U


def random_state(n, seed=0):
    rng = np.random.default_rng(seed)
    U = np.zeros((n, 5))
    U[:, 0] = 1.0 + 0.2 * rng.random(n)
    U[:, 1:4] = 0.2 * rng.standard_normal((n, 3))
    U[:, 4] = 2.5 + 0.5 * rng.random(n) + 0.5 * (U[:, 1:4] ** 2).sum(1) / U[:, 0]
    return U


def laplacian_14(d):
    """The positive Laplacian the reference unit tests assemble on their 14-node
    mesh (tests/unit/LinearSolver/TestCSR.cpp:309-333): A += J/6 grad_a.grad_b
    with grad = crossdiv(., J), on the psup sparsity; zero-based CSR."""
    ip = d["inpoel_1based"] - 1
    X, Y, Z = d["coord"]
    n = X.size
    rows = [set([i]) for i in range(n)]
    for t in ip:
        for a in t:
            rows[a].update(t.tolist())
    ia = np.zeros(n + 1, np.int64)
    ja = []
    for i in range(n):
        c = sorted(rows[i])
        ja += c
        ia[i + 1] = ia[i] + len(c)
    ja = np.array(ja, np.int64)
    a = np.zeros(ja.size)
    for N in ip:
        ba = np.array([X[N[1]] - X[N[0]], Y[N[1]] - Y[N[0]], Z[N[1]] - Z[N[0]]])
        ca = np.array([X[N[2]] - X[N[0]], Y[N[2]] - Y[N[0]], Z[N[2]] - Z[N[0]]])
        da = np.array([X[N[3]] - X[N[0]], Y[N[3]] - Y[N[0]], Z[N[3]] - Z[N[0]]])
        J = ba @ np.cross(ca, da)
        g = np.zeros((4, 3))
        g[1] = np.cross(ca, da) / J
        g[2] = np.cross(da, ba) / J
        g[3] = np.cross(ba, ca) / J
        g[0] = -g[1] - g[2] - g[3]
        for i in range(4):
            for k in range(3):
                for j in range(4):
                    r = N[i]
                    pos = ia[r] + np.searchsorted(ja[ia[r]:ia[r + 1]], N[j])
                    a[pos] += J / 6 * g[i][k] * g[j][k]
    return ia, ja, a


def dirichlet_matrix_only(ia, ja, a, i):
    """tk::CSR::dirichlet with value 0 in serial (src/LinearSolver/CSR.cpp:
    106-152): zero column i and row i, 1 on the diagonal (b unchanged)."""
    a = a.copy()
    a[ja == i] = 0.0
    for j in range(ia[i], ia[i + 1]):
        a[j] = 1.0 if ja[j] == i else 0.0
    return a


def chocg_mesh(name):
    """ChoCG regression fixture ("lid" or "poiseuille"): mesh dict and data."""
    d = golden("chocg_" + name)
    bface = {int(k[5:]): d[k] for k in d.files if k.startswith("bface")}
    return {"coord": d["coord"], "inpoel": d["inpoel"], "bface": bface}, d


def nodes_of(bface, sets):
    out = [np.unique(bface[s]) for s in sets if s in bface]
    return np.unique(np.concatenate(out)) if out else np.zeros(0, np.int64)


def chocg_regression_setup(name, m):
    """Boundary conditions and settings of the reference's ChoCG regressions
    (tests/regression/inciter/ChoCG/Lid/ldc.q, Poiseuille/poiseuille_damp2.q,
    Sphere/inviscid_sphere.q and Sphere/sphere_chocg_viscous_test.q) as
    per-node lists in the mesh file's
    numbering: velocity Dirichlet (nodes, mask, values), noslip nodes,
    pressure Dirichlet (nodes, values of the initial solves), the solver
    settings, the step count, the symmetry side sets and the initial
    velocity."""
    bf = m["bface"]
    sym, u0 = (), (0.0, 0.0, 0.0)
    if name == "lid":
        dn = nodes_of(bf, [4])
        dirbc = (dn, np.ones((dn.size, 3), np.int32), np.tile([1.0, 0.0, 0.0], (dn.size, 1)))
        noslip = nodes_of(bf, [1, 2, 3, 5, 6])
        pdir = (np.array([0]), np.array([0.0]))  # hydrostat = 0, userdef pressure IC 0
        prm = dict(mu=0.01, cfl=0.9, flux="damp4", pc="jacobi", ptol=1e-3, pmaxit=500)
        nstep = 10
    elif name == "inviscid_sphere":
        dn = nodes_of(bf, [2])
        dirbc = (dn, np.tile([1, 0, 0], (dn.size, 1)).astype(np.int32),
                 np.tile([1.0, 0.0, 0.0], (dn.size, 1)))  # mask 1: the IC value u = 1
        noslip = np.zeros(0, np.int64)
        p3 = nodes_of(bf, [3])
        pdir = (p3, np.zeros(p3.size))
        prm = dict(mu=0.0, cfl=0.5, flux="damp2", pc="jacobi", ptol=1e-3, pmaxit=300)
        nstep = 10
        sym, u0 = (1, 4), (1.0, 0.0, 0.0)
    elif name == "viscous_sphere":
        # a node on both velocity sets takes the union of their masks
        d2, d4 = nodes_of(bf, [2]), nodes_of(bf, [4])
        dn = np.union1d(d2, d4)
        mask = np.zeros((dn.size, 3), np.int32)
        mask[np.isin(dn, d2), 0] = 1
        mask[np.isin(dn, d4)] = 1
        dirbc = (dn, mask, np.tile([1.0, 0.0, 0.0], (dn.size, 1)))
        noslip = nodes_of(bf, [1])
        p3 = nodes_of(bf, [3])
        pdir = (p3, np.zeros(p3.size))
        prm = dict(mu=1.0 / 40.0, cfl=0.3, flux="damp4", rk=4, pc="jacobi", ptol=1e-3,
                   pmaxit=300)
        nstep = 20
        u0 = (1.0, 0.0, 0.0)
    else:
        dn = nodes_of(bf, [1, 5])
        mask = np.tile([0, 1, 1], (dn.size, 1)).astype(np.int32)
        dirbc = (dn, mask, np.zeros((dn.size, 3)))  # mask 1: the IC value, 0
        noslip = nodes_of(bf, [3, 4])
        p1, p2 = nodes_of(bf, [1]), nodes_of(bf, [2])
        pn = np.concatenate([p1, p2])
        pv = np.concatenate([np.full(p1.size, 2.4), np.zeros(p2.size)])
        order = np.argsort(pn, kind="stable")
        pdir = (pn[order], pv[order])
        prm = dict(mu=0.01, cfl=0.05, flux="damp2", pc="jacobi", ptol=1e-3, pmaxit=500)
        nstep = 20
    return dirbc, noslip, pdir, prm, nstep, sym, u0


# The ChoCG Poisson problems' right-hand sides and solutions (poisson_const,
# poisson_sine, poisson_sine3: src/Physics/Problems.cpp:841-954).
POISSON_PROBLEMS = {
    "const": (lambda x, y, z: 6.0 + 0.0 * x, lambda x, y, z: x * x + y * y + z * z),
    "sine": (lambda x, y, z: -np.pi * np.pi * x * y * np.sin(np.pi * z),
             lambda x, y, z: x * y * np.sin(np.pi * z)),
    "sine3": (lambda x, y, z: -3.0 * np.pi * np.pi * np.sin(np.pi * x) * np.sin(np.pi * y) *
              np.sin(np.pi * z),
              lambda x, y, z: np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)),
    "neumann": (lambda x, y, z: -3.0 * np.cos(2.0 * x) * np.exp(y),
                lambda x, y, z: np.cos(2.0 * x) * np.exp(y)),
}


def _neumann_gradient(x, y, z):
    """poisson_neumann's pressure gradient (Problems.cpp:966-972)."""
    return np.array([-2.0 * np.sin(2.0 * x) * np.exp(y), np.cos(2.0 * x) * np.exp(y), 0.0 * x])


def poisson_case(name, vol_of):
    """A Poisson regression's system as ChoCG's start-up sets it up
    (ChoCG.cpp:1046-1118): the pressure matrix's right-hand side pr V, the
    solution's values as Dirichlet data (on all six side sets; for
    poisson_neumann on 1-3, with Neumann data on 4-6).  Returns the fixture,
    coordinates, tetrahedra, volumes, b, Dirichlet nodes and values, the
    exact solution at the nodes and the Neumann data."""
    d = golden("chocg_poisson")
    pre = "neumann_" if name == "neumann" else ""
    coord, inpoel = d[pre + "coord"], d[pre + "inpoel"]
    x, y, z = coord
    v = vol_of(coord, inpoel)
    pr, sol = POISSON_PROBLEMS[name]
    bface = {int(k[len(pre) + 5:]): d[k] for k in d.files
             if k.startswith(pre + "bface") and k[len(pre) + 5:].isdigit()}
    dirsets, neusets = ((1, 2, 3), (4, 5, 6)) if name == "neumann" else ((1, 2, 3, 4, 5, 6), ())
    dn = np.unique(np.concatenate([bface[s] for s in dirsets]).ravel())
    # Neumann data of the symmetry sets (ChoCG.cpp:1071-1092): each triangle
    # takes n . grad p at its nodes off them, n = (b - a) x (c - a) / 6
    neu = np.zeros(x.size)
    for s in neusets:
        for N in bface[s]:
            n = np.cross(coord[:, N[1]] - coord[:, N[0]], coord[:, N[2]] - coord[:, N[0]]) / 6.0
            for p in N:
                neu[p] -= n @ _neumann_gradient(x[p], y[p], z[p])
    return (d, coord, inpoel, v, pr(x, y, z) * v, dn, sol(x[dn], y[dn], z[dn]), sol(x, y, z),
            neu)


def check_poisson(name, p, v, exact, d, coord):
    """L2(p), L2(dp) (the change from zero), L2 and L1 of the error against
    diag_poisson_<name>.std within its numdiff tolerance (abs or rel 1e-8),
    and for poisson_const the pressure field against poisson_const.std.exo
    (exodiff: relative 1e-7, floor 1e-8)."""
    V = v.sum()
    l2 = np.sqrt((p * p * v).sum() / V)
    got = np.array([l2, l2, np.sqrt(((p - exact) ** 2 * v).sum() / V),
                    (np.abs(p - exact) * v).sum() / V])
    exp = d["diag_" + name][0, 3:7]
    assert np.all(np.abs(got - exp) <= np.maximum(1e-8, 1e-8 * np.abs(exp))), (got, exp)
    if name == "const":
        from scipy.spatial import cKDTree
        dist, idx = cKDTree(coord.T).query(d["out_coord"].T)
        assert dist.max() < 1e-12
        ref = d["const_pressure"]
        m = np.maximum(np.abs(p[idx]), np.abs(ref))
        big = m > 1e-8
        assert np.all(np.abs(p[idx] - ref)[big] <= 1e-7 * m[big])
