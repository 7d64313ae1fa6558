"""Extract the reference's own golden vectors for the accelerated path into
small committed fixtures (tests/golden/*.npz).

Run where the reference sources are readable (the root given as the argument,
else $XYST_REFERENCE, else a checkout named "reference" beside this repository):

    python tests/golden/make_golden.py [reference-root]

Sources, all read as data (nothing is executed):
  * tests/unit/LinearSolver/TestCSR.cpp: the 14-node tet mesh and the
    expected Laplacian matrix-vector product (test 9);
  * tests/unit/LinearSolver/TestConjugateGradients.cpp: its 14-node mesh and
    the expected ||b|| and final residual of the 1-DOF and 3-DOF serial solves
    (tests 1 and 3);
  * tests/regression/inciter/RieCG/Sod: the input mesh, the final nodal
    fields (sod.std.exo) and the per-step diagnostics (diag.std) of the RieCG
    Sod shock tube (10 steps, CFL 0.5, symmetry on side sets 2,4,5,6);
  * tests/regression/inciter/KozCG/Sod: the same for KozCG;
  * tests/regression/inciter/ChoCG/Lid: the lid-driven cavity (damp4, CFL
    0.9, Re 100, Jacobi PCG to 1e-3, hydrostat node 0, noslip on side sets
    1,2,3,5,6, lid velocity (1,0,0) on side set 4, 10 steps): input mesh,
    final nodal fields (ldc.std.exo) and per-step diagnostics (diag_ldc.std);
  * tests/regression/inciter/ChoCG/Poiseuille: the damp2 Poiseuille flow
    (CFL 0.05, mu 0.01, pressure 2.4 / 0 on side sets 1 / 2, noslip on 3,4,
    v = w = 0 on 1 and 5, 20 steps): the same three files;
  * tests/regression/inciter/RieCG/TaylorGreen: the stationary Taylor-Green
    vortex with its manufactured energy source (gamma 5/3, CFL 0.8, the
    analytic state as Dirichlet values on all six side sets, to t = 1 in 68
    steps): input mesh, nodal fields at every output time
    (taylor_green.std.exo) and the diagnostics of every second step
    (diag.std);
  * tests/regression/inciter/KozCG/TaylorGreen: the same problem with KozCG
    (no FCT), the same three files;
  * tests/regression/inciter/{RieCG,KozCG}/VorticalFlow: the vortical flow
    with its manufactured source (alpha 0.1, kappa 1, p0 10, gamma 5/3, CFL
    0.8, the analytic state as Dirichlet values on all six side sets, to
    t = 1), RieCG with and without stab2 and KozCG without FCT: the same
    three files each;
  * tests/regression/inciter/{RieCG,KozCG}/{NonlinearEnergyGrowth,
    RayleighTaylor}: the time-dependent manufactured solutions (Dirichlet
    values of the analytic state at each BC's time; nleg.q to t = 1 at CFL
    0.8, rayleigh_taylor.q 50 steps at CFL 0.5): the same three files each;
  * tests/regression/inciter/ChoCG/Poisson: the pressure Poisson problems
    poisson_const, poisson_sine and poisson_sine3 (right-hand side and
    Dirichlet values from the problem's formulas on all six side sets, PCG
    without preconditioner to 1e-6, at most 100 iterations) and
    poisson_neumann (Dirichlet on side sets 1-3, the solution's gradient as
    Neumann data on 4-6): the meshes, the four diagnostics files and the
    poisson_const pressure field;
  * tests/regression/inciter/RieCG/Sedov: the Sedov blast on sedov_coarse.exo
    (p0 4.86e3 at the origin node, gamma 5/3, CFL 0.5, symmetry on side sets
    1-3, 10 steps): the mesh and the diagnostics (the checkout holds no
    single-process field baseline);
  * tests/regression/inciter/RieCG/Pipe: flow between pressure boundaries
    (1e5 at side set 1, 99900 at 3, density 1, symmetry on 2, 4, 5, 6,
    CFL 0.5, 20 steps): the mesh, the fields (pipe.std.exo) and the
    diagnostics;
  * tests/regression/inciter/ChoCG/Sphere: the inviscid flow past a sphere
    (inviscid_sphere.q on sphere2_5K.exo: damp2, CFL 0.5, velocity (1, 0, 0)
    held in x on side set 2, symmetry on 1 and 4, pressure 0 on 3, Jacobi
    PCG to 1e-3, 10 steps): the mesh, the final fields and the diagnostics;
    and the viscous flow (sphere_chocg_viscous_test.q: Re 40, damp4, 4-stage
    RK, CFL 0.3, noslip on the sphere, u = 1 held on the inflow set and all
    of (1, 0, 0) on the far field, pressure 0 on the outflow, 20 steps): the
    same three files.
"""

from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _block(text: str, start_pat: str) -> str:
    i = text.index(start_pat)
    j = text.index("};", i)
    return text[i + len(start_pat):j]


def _numbers(s: str, kind=float):
    s = re.sub(r"//[^\n]*", "", s)
    toks = re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", s)
    return np.array([kind(t) if kind is float else int(float(t)) for t in toks])


def _mesh14(text: str, test_marker: str):
    part = text[text.index(test_marker):] if test_marker else text
    ip = _numbers(_block(part, "inpoel {"), int).reshape(-1, 4)
    cb = _block(part, "coord {{")
    rows = re.findall(r"\{\{([^{}]*)\}\}", cb)
    coord = np.array([_numbers(r) for r in rows[:3]])
    return ip, coord


def csr_fixture(ref: str):
    t = open(os.path.join(ref, "tests/unit/LinearSolver/TestCSR.cpp")).read()
    ip, coord = _mesh14(t, "")
    m = t[t.index("test_name( \"matrix-vector multiply\" )"):]
    correct = _numbers(_block(m, "std::vector< tk::real > correct{"))
    return {"inpoel_1based": ip, "coord": coord, "mult_correct": correct,
            "prec": np.float64(np.finfo(np.float64).eps * 100)}


def cg_fixture(ref: str):
    t = open(os.path.join(ref, "tests/unit/LinearSolver/TestConjugateGradients.cpp")).read()
    ip, coord = _mesh14(t, "Laplace eq 1DOF 1PE setup")

    def expected(marker):
        part = t[t.index(marker):]
        blk = part[part.index("CProxy_CGReceiver::ckNew"):]
        blk = blk[:blk.index(");")]
        vals = {}
        for key in ("maxit", "tol", "normb_ex", "normres_ex"):
            mm = re.search(r"/\*\s*" + key + r"\s*=\s*\*?\s*\*/\s*([-+0-9.eE]+)", blk)
            vals[key] = float(mm.group(1))
        return vals

    e1 = expected("Laplace eq 1DOF 1PE setup")
    e3 = expected("Laplace eq 3DOF 1PE setup")
    return {"inpoel_1based": ip, "coord": coord,
            "dof1": np.array([e1["maxit"], e1["tol"], e1["normb_ex"], e1["normres_ex"]]),
            "dof3": np.array([e3["maxit"], e3["tol"], e3["normb_ex"], e3["normres_ex"]])}


def _diag(path):
    rows = [ln.split() for ln in open(path) if ln.strip() and not ln.startswith("#")]
    return np.array([[float(x) for x in r] for r in rows])


def sod_fixture(ref: str, scheme: str):
    from xyst_gb300 import mesh as M
    from scipy.io import netcdf_file

    base = os.path.join(ref, "tests/regression/inciter", scheme, "Sod")
    m = M.read_exo(os.path.join(base, "rectangle_01_1.5k.exo"))
    f = netcdf_file(os.path.join(base, "sod.std.exo"), "r", mmap=False)
    names = ["".join(c.decode() for c in row if c) for row in f.variables["name_nod_var"][:]]
    times = np.array(f.variables["time_whole"][:], dtype=np.float64)
    fields = np.array([np.array(f.variables[f"vals_nod_var{i + 1}"][:][-1], dtype=np.float64)
                       for i in range(len(names))])
    ocoord = np.stack([np.asarray(f.variables[k][:], dtype=np.float64)
                       for k in ("coordx", "coordy", "coordz")])
    f.close()
    out = {"coord": m["coord"], "inpoel": m["inpoel"], "final_time": times[-1],
           "out_coord": ocoord, "out_fields": fields, "out_names": np.array(names),
           "diag": _diag(os.path.join(base, "diag.std"))}
    for s, tri in m["bface"].items():
        out[f"bface{s}"] = tri
    return out


def regression_fixture(ref: str, scheme: str, case: str, meshfile: str, outfile: str,
                       diagfile: str, all_times: bool = False):
    """Input mesh, output fields (the last time, or every time) and
    diagnostics of one regression case of a scheme."""
    from xyst_gb300 import mesh as M
    from scipy.io import netcdf_file

    base = os.path.join(ref, "tests/regression/inciter", scheme, case)
    m = M.read_exo(os.path.join(base, meshfile))
    if outfile is None:  # diagnostics only
        out = {"coord": m["coord"], "inpoel": m["inpoel"],
               "diag": _diag(os.path.join(base, diagfile))}
        for s, tri in m["bface"].items():
            out[f"bface{s}"] = tri
        return out
    f = netcdf_file(os.path.join(base, outfile), "r", mmap=False)
    names = ["".join(c.decode() for c in row if c) for row in f.variables["name_nod_var"][:]]
    times = np.array(f.variables["time_whole"][:], dtype=np.float64)
    allf = np.array([np.array(f.variables[f"vals_nod_var{i + 1}"][:], dtype=np.float64)
                     for i in range(len(names))])  # [field][time][node]
    ocoord = np.stack([np.asarray(f.variables[k][:], dtype=np.float64)
                       for k in ("coordx", "coordy", "coordz")])
    f.close()
    out = {"coord": m["coord"], "inpoel": m["inpoel"], "final_time": times[-1],
           "out_coord": ocoord, "out_fields": allf[:, -1], "out_names": np.array(names),
           "diag": _diag(os.path.join(base, diagfile))}
    if all_times:
        out["out_times"] = times
        out["out_fields_all"] = allf
    for s, tri in m["bface"].items():
        out[f"bface{s}"] = tri
    return out


def poisson_fixture(ref: str):
    """The ChoCG Poisson regressions' meshes, the diagnostics of the
    poisson_const, poisson_sine, poisson_sine3 and poisson_neumann runs, and
    the pressure of the single-process poisson_const run
    (poisson_const.std.exo)."""
    from xyst_gb300 import mesh as M
    from scipy.io import netcdf_file

    base = os.path.join(ref, "tests/regression/inciter/ChoCG/Poisson")
    m = M.read_exo(os.path.join(base, "unitcube_01_1k.exo"))
    out = {"coord": m["coord"], "inpoel": m["inpoel"]}
    for s, tri in m["bface"].items():
        out[f"bface{s}"] = tri
    for name in ("const", "sine", "sine3"):
        out["diag_" + name] = _diag(os.path.join(base, f"diag_poisson_{name}.std"))
    out["diag_neumann"] = _diag(os.path.join(base, "diag_poisson_neumann.std"))
    m2 = M.read_exo(os.path.join(base, "unitcube_0pidiv4_1k.exo"))
    out["neumann_coord"] = m2["coord"]
    out["neumann_inpoel"] = m2["inpoel"]
    for s, tri in m2["bface"].items():
        out[f"neumann_bface{s}"] = tri
    f = netcdf_file(os.path.join(base, "poisson_const.std.exo"), "r", mmap=False)
    names = ["".join(c.decode() for c in row if c) for row in f.variables["name_nod_var"][:]]
    k = names.index("pressure")
    out["const_pressure"] = np.array(f.variables[f"vals_nod_var{k + 1}"][:][-1], dtype=np.float64)
    out["out_coord"] = np.stack([np.asarray(f.variables[c][:], dtype=np.float64)
                                 for c in ("coordx", "coordy", "coordz")])
    f.close()
    return out


def chocg_fixture(ref: str, case: str, meshfile: str, outfile: str, diagfile: str):
    return regression_fixture(ref, "ChoCG", case, meshfile, outfile, diagfile)


def main(ref: str):
    np.savez_compressed(os.path.join(HERE, "csr_mult.npz"), **csr_fixture(ref))
    np.savez_compressed(os.path.join(HERE, "cg_laplace.npz"), **cg_fixture(ref))
    np.savez_compressed(os.path.join(HERE, "riecg_sod.npz"), **sod_fixture(ref, "RieCG"))
    np.savez_compressed(os.path.join(HERE, "kozcg_sod.npz"), **sod_fixture(ref, "KozCG"))
    np.savez_compressed(os.path.join(HERE, "chocg_lid.npz"),
                        **chocg_fixture(ref, "Lid", "unitcube_1k.exo", "ldc.std.exo",
                                        "diag_ldc.std"))
    np.savez_compressed(os.path.join(HERE, "chocg_poiseuille.npz"),
                        **chocg_fixture(ref, "Poiseuille", "poiseuille1tetz.exo",
                                        "poiseuille_damp2.std.exo",
                                        "diag_poiseuille_damp2.std"))
    np.savez_compressed(os.path.join(HERE, "riecg_taylor_green.npz"),
                        **regression_fixture(ref, "RieCG", "TaylorGreen", "unitcube_1k.exo",
                                             "taylor_green.std.exo", "diag.std", all_times=True))
    np.savez_compressed(os.path.join(HERE, "kozcg_taylor_green.npz"),
                        **regression_fixture(ref, "KozCG", "TaylorGreen", "unitcube_1k.exo",
                                             "taylor_green.std.exo", "diag.std", all_times=True))
    for scheme, name, out, diag in (("RieCG", "riecg_vortical_flow", "vortical_flow.std.exo",
                                     "diag.std"),
                                    ("RieCG", "riecg_vortical_flow_stab2",
                                     "vortical_flow_stab2.std.exo", "diag_stab2.std"),
                                    ("KozCG", "kozcg_vortical_flow", "vortical_flow.std.exo",
                                     "diag.std")):
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            **regression_fixture(ref, scheme, "VorticalFlow", "unitcube_1k.exo",
                                                 out, diag, all_times=True))
    for scheme in ("RieCG", "KozCG"):
        low = scheme.lower()
        np.savez_compressed(os.path.join(HERE, low + "_nonlinear_energy_growth.npz"),
                            **regression_fixture(ref, scheme, "NonlinearEnergyGrowth",
                                                 "unitcube_1k.exo", "nleg.std.exo", "diag.std",
                                                 all_times=True))
        np.savez_compressed(os.path.join(HERE, low + "_rayleigh_taylor.npz"),
                            **regression_fixture(ref, scheme, "RayleighTaylor", "unitcube_1k.exo",
                                                 "rayleigh_taylor.std.exo", "diag.std",
                                                 all_times=True))
    np.savez_compressed(os.path.join(HERE, "chocg_poisson.npz"), **poisson_fixture(ref))
    np.savez_compressed(os.path.join(HERE, "chocg_inviscid_sphere.npz"),
                        **chocg_fixture(ref, "Sphere", "sphere2_5K.exo", "inviscid_sphere.std.exo",
                                        "diag_inviscid_sphere.std"))
    np.savez_compressed(os.path.join(HERE, "chocg_viscous_sphere.npz"),
                        **chocg_fixture(ref, "Sphere", "sphere2_5K.exo",
                                        "sphere_chocg_viscous_test.std.exo",
                                        "diag_sphere_chocg_viscous_test.std"))
    np.savez_compressed(os.path.join(HERE, "riecg_sedov.npz"),
                        **regression_fixture(ref, "RieCG", "Sedov", "sedov_coarse.exo", None,
                                             "diag.std"))
    np.savez_compressed(os.path.join(HERE, "riecg_pipe.npz"),
                        **regression_fixture(ref, "RieCG", "Pipe", "rectangle_01_1.5k.exo",
                                             "pipe.std.exo", "diag.std", all_times=True))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    default = os.environ.get("XYST_REFERENCE") or os.path.join(
        os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")
    main(sys.argv[1] if len(sys.argv) > 1 else default)
