// Test-only C shim over the reference's own compiled physics functions.
//
// This file is part of the oracle (test infrastructure), never of the product.
// It is compiled together with the reference's unmodified sources
// (src/Physics/{Riemann,Kozak,Chorin,Problems,Box,BC}.cpp,
// src/LinearSolver/CSR.cpp, src/Mesh/{DerivedData,Reorder}.cpp,
// src/Base/Exception.cpp) by oracle/build_ref.sh into oracle/_ref/, and is
// used only to pin the C++ restatement in oracle/xg_oracle.cpp and to generate
// golden fixtures.  Each entry point forwards plain arrays into the reference
// function it names; nothing here re-implements reference arithmetic.

#include <array>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "Fields.hpp"
#include "Riemann.hpp"
#include "Kozak.hpp"
#include "Chorin.hpp"
#include "CSR.hpp"
#include "DerivedData.hpp"
#include "InciterConfig.hpp"
#include "Vector.hpp"

namespace inciter {
ctr::Config g_cfg;
}

using inciter::g_cfg;

namespace {

using Coord = std::array<std::vector<tk::real>, 3>;

Coord make_coord(int64_t npoin, const double* xyz) {
  Coord c;
  for (int d = 0; d < 3; ++d) c[d].assign(xyz + d * npoin, xyz + (d + 1) * npoin);
  return c;
}

tk::Fields make_fields(int64_t nunk, int64_t nprop, const double* v) {
  tk::Fields f(static_cast<std::size_t>(nunk), static_cast<std::size_t>(nprop));
  if (v)
    for (int64_t i = 0; i < nunk; ++i)
      for (int64_t c = 0; c < nprop; ++c) f(i, c) = v[i * nprop + c];
  return f;
}

void read_fields(const tk::Fields& f, double* out) {
  for (std::size_t i = 0; i < f.nunk(); ++i)
    for (std::size_t c = 0; c < f.nprop(); ++c) out[i * f.nprop() + c] = f(i, c);
}

std::vector<std::size_t> ids(const int64_t* p, int64_t n) {
  std::vector<std::size_t> v(static_cast<std::size_t>(n));
  for (int64_t i = 0; i < n; ++i) v[i] = static_cast<std::size_t>(p[i]);
  return v;
}

std::string g_err;

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Configure the handful of global settings the hot-path functions read.
int ref_set_config(double gamma, const char* flux, int stab2, double stab2coef,
                   const char* problem, int ncomp) {
  g_cfg.get<tag::mat_spec_heat_ratio>() = gamma;
  g_cfg.get<tag::flux>() = flux;
  g_cfg.get<tag::stab2>() = stab2 != 0;
  g_cfg.get<tag::stab2coef>() = stab2coef;
  g_cfg.get<tag::problem>() = problem;
  g_cfg.get<tag::problem_ncomp>() = static_cast<uint64_t>(ncomp);
  g_cfg.get<tag::steady>() = false;
  return 0;
}

// The manufactured-solution parameters the problems' source terms read
// (problem_alpha, problem_beta[3], problem_kappa, problem_r0, problem_p0,
// problem_ce of the control file).
int ref_set_problem_params(double alpha, double b0, double b1, double b2, double kappa,
                           double r0, double p0, double ce) {
  g_cfg.get<tag::problem_alpha>() = alpha;
  g_cfg.get<tag::problem_beta>() = std::vector<double>{b0, b1, b2};
  g_cfg.get<tag::problem_kappa>() = kappa;
  g_cfg.get<tag::problem_r0>() = r0;
  g_cfg.get<tag::problem_p0>() = p0;
  g_cfg.get<tag::problem_ce>() = ce;
  return 0;
}

// riemann::grad (src/Physics/Riemann.cpp:229-367).  Superedge counts are in
// groups (tets: 4 ids + 18 reals, tris: 3 ids + 9 reals, edges: 2 ids + 3).
int ref_riemann_grad(int64_t npoin, const double* xyz, int64_t ncomp,
                     int64_t n0, const int64_t* e0, const double* i0,
                     int64_t n1, const int64_t* e1, const double* i1,
                     int64_t n2, const int64_t* e2, const double* i2,
                     int64_t ntri, const int64_t* tri, const double* U,
                     double* G) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{ids(e0, n0 * 4), ids(e1, n1 * 3),
                                                ids(e2, n2 * 2)};
    std::array<std::vector<tk::real>, 3> sint{
        std::vector<tk::real>(i0, i0 + n0 * 18),
        std::vector<tk::real>(i1, i1 + n1 * 9),
        std::vector<tk::real>(i2, i2 + n2 * 3)};
    auto coord = make_coord(npoin, xyz);
    auto u = make_fields(npoin, ncomp, U);
    tk::Fields g(static_cast<std::size_t>(npoin), static_cast<std::size_t>(ncomp * 3));
    riemann::grad(sup, sint, coord, ids(tri, ntri * 3), u, g);
    read_fields(g, G);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// riemann::rhs (src/Physics/Riemann.cpp:909-946).
int ref_riemann_rhs(int64_t npoin, const double* xyz, int64_t ncomp,
                    int64_t n0, const int64_t* e0, const double* i0,
                    int64_t n1, const int64_t* e1, const double* i1,
                    int64_t n2, const int64_t* e2, const double* i2,
                    int64_t ntri, const int64_t* tri, const uint8_t* besym,
                    const double* G, const double* U, const double* vol,
                    double t, double* R) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{ids(e0, n0 * 4), ids(e1, n1 * 3),
                                                ids(e2, n2 * 2)};
    std::array<std::vector<tk::real>, 3> sint{
        std::vector<tk::real>(i0, i0 + n0 * 18),
        std::vector<tk::real>(i1, i1 + n1 * 9),
        std::vector<tk::real>(i2, i2 + n2 * 3)};
    auto coord = make_coord(npoin, xyz);
    auto u = make_fields(npoin, ncomp, U);
    auto g = make_fields(npoin, ncomp * 3, G);
    tk::Fields r(static_cast<std::size_t>(npoin), static_cast<std::size_t>(ncomp));
    std::vector<std::uint8_t> bs(besym, besym + ntri * 3);
    std::vector<tk::real> v(vol, vol + npoin);
    std::vector<tk::real> tp(static_cast<std::size_t>(npoin), t);
    riemann::rhs(sup, sint, coord, ids(tri, ntri * 3), bs, g, u, v, t, tp, r);
    read_fields(r, R);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// kozak::rhs (src/Physics/Kozak.cpp:29-180).
int ref_kozak_rhs(int64_t nelem, const int64_t* inpoel, int64_t npoin,
                  const double* xyz, int64_t ncomp, double t, double dt,
                  const double* U, double* R) {
  try {
    auto coord = make_coord(npoin, xyz);
    auto u = make_fields(npoin, ncomp, U);
    tk::Fields r(static_cast<std::size_t>(npoin), static_cast<std::size_t>(ncomp));
    std::vector<tk::real> tp(static_cast<std::size_t>(npoin), t), dtp(tp.size(), dt);
    kozak::rhs(ids(inpoel, nelem * 4), coord, t, dt, tp, dtp, u, r);
    read_fields(r, R);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// chorin::div and chorin::grad (src/Physics/Chorin.cpp:85-209, 336-449) over
// edge groups only (2 ids + 5 reals per edge), as ChoCG stores them.
int ref_chorin_div(int64_t npoin, const double* xyz, int64_t n2, const int64_t* e2,
                   const double* i2, int64_t ntri, const int64_t* tri, double dt,
                   const double* P, const double* PG, const double* Uvel,
                   int stab, double* D) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{{{}, {}, ids(e2, n2 * 2)}};
    std::array<std::vector<tk::real>, 3> sint{{{}, {}, std::vector<tk::real>(i2, i2 + n2 * 5)}};
    auto coord = make_coord(npoin, xyz);
    std::vector<tk::real> p(P, P + npoin), d(static_cast<std::size_t>(npoin), 0.0);
    auto g = make_fields(npoin, 3, PG);
    auto u = make_fields(npoin, 3, Uvel);
    chorin::div(sup, sint, coord, ids(tri, ntri * 3), dt, p, g, u, d, stab != 0);
    std::memcpy(D, d.data(), sizeof(double) * d.size());
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

int ref_chorin_grad(int64_t npoin, const double* xyz, int64_t n2, const int64_t* e2,
                    const double* i2, int64_t ntri, const int64_t* tri,
                    const double* S, double* G) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{{{}, {}, ids(e2, n2 * 2)}};
    std::array<std::vector<tk::real>, 3> sint{{{}, {}, std::vector<tk::real>(i2, i2 + n2 * 5)}};
    auto coord = make_coord(npoin, xyz);
    std::vector<tk::real> s(S, S + npoin);
    tk::Fields g(static_cast<std::size_t>(npoin), 3);
    g.fill(0.0);
    chorin::grad(sup, sint, coord, ids(tri, ntri * 3), s, g);
    read_fields(g, G);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// The viscosity and advection stabilisation switch chorin::rhs/flux read.
int ref_set_chorin(double mu, int stab) {
  g_cfg.get<tag::mat_dyn_viscosity>() = mu;
  g_cfg.get<tag::stab>() = stab != 0;
  return 0;
}

// chorin::vgrad (src/Physics/Chorin.cpp:211-334) over edge groups only.
int ref_chorin_vgrad(int64_t npoin, const double* xyz, int64_t n2, const int64_t* e2,
                     const double* i2, int64_t ntri, const int64_t* tri, int64_t ncomp,
                     const double* U, double* G) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{{{}, {}, ids(e2, n2 * 2)}};
    std::array<std::vector<tk::real>, 3> sint{{{}, {}, std::vector<tk::real>(i2, i2 + n2 * 5)}};
    auto coord = make_coord(npoin, xyz);
    auto u = make_fields(npoin, ncomp, U);
    tk::Fields g(static_cast<std::size_t>(npoin), static_cast<std::size_t>(ncomp * 3));
    g.fill(0.0);
    chorin::vgrad(sup, sint, coord, ids(tri, ntri * 3), u, g);
    read_fields(g, G);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// chorin::flux (src/Physics/Chorin.cpp:509-638) over edge groups only.
int ref_chorin_flux(int64_t npoin, const double* xyz, int64_t n2, const int64_t* e2,
                    const double* i2, int64_t ntri, const int64_t* tri, const double* U,
                    const double* G, double* F) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{{{}, {}, ids(e2, n2 * 2)}};
    std::array<std::vector<tk::real>, 3> sint{{{}, {}, std::vector<tk::real>(i2, i2 + n2 * 5)}};
    auto coord = make_coord(npoin, xyz);
    auto u = make_fields(npoin, 3, U);
    auto g = make_fields(npoin, 9, G);
    tk::Fields f(static_cast<std::size_t>(npoin), 3);
    f.fill(0.0);
    chorin::flux(sup, sint, coord, ids(tri, ntri * 3), u, g, f);
    read_fields(f, F);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// chorin::rhs (src/Physics/Chorin.cpp:1010-1044) over edge groups only.
int ref_chorin_rhs(int64_t npoin, const double* xyz, int64_t n2, const int64_t* e2,
                   const double* i2, int64_t ntri, const int64_t* tri, const double* vol,
                   double t, const double* P, const double* U, const double* G, double* R) {
  try {
    std::array<std::vector<std::size_t>, 3> sup{{{}, {}, ids(e2, n2 * 2)}};
    std::array<std::vector<tk::real>, 3> sint{{{}, {}, std::vector<tk::real>(i2, i2 + n2 * 5)}};
    auto coord = make_coord(npoin, xyz);
    auto u = make_fields(npoin, 3, U);
    auto g = make_fields(npoin, 9, G);
    tk::Fields r(static_cast<std::size_t>(npoin), 3);
    std::vector<tk::real> v(vol, vol + npoin), p(P, P + npoin);
    chorin::rhs(sup, sint, coord, ids(tri, ntri * 3), v, t, p, u, g, r);
    read_fields(r, R);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// tk::genPsup (src/Mesh/DerivedData.cpp:132-250): returns sizes first when the
// output pointers are null.
int ref_genpsup(int64_t nelem, const int64_t* inpoel, int64_t* n1, int64_t* n2,
                int64_t* psup1, int64_t* psup2) {
  try {
    auto ip = ids(inpoel, nelem * 4);
    auto psup = tk::genPsup(ip, 4, tk::genEsup(ip, 4));
    *n1 = static_cast<int64_t>(psup.first.size());
    *n2 = static_cast<int64_t>(psup.second.size());
    if (psup1)
      for (std::size_t i = 0; i < psup.first.size(); ++i) psup1[i] = static_cast<int64_t>(psup.first[i]);
    if (psup2)
      for (std::size_t i = 0; i < psup.second.size(); ++i) psup2[i] = static_cast<int64_t>(psup.second[i]);
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// The pressure matrix exactly as ChoCG::prelhs builds it
// (src/Inciter/ChoCG.cpp:146-188), stored in tk::CSR (src/LinearSolver/CSR.cpp),
// then optionally Dirichlet rows eliminated with tk::CSR::dirichlet
// (CSR.cpp:106-152) in decreasing node order as ConjugateGradients::apply
// does (src/LinearSolver/ConjugateGradients.cpp:475-485).  Outputs the 1-based
// ia/ja/a arrays, the product A*x, and the rhs modification vector.
int ref_csr_pressure(int64_t nelem, const int64_t* inpoel, int64_t npoin,
                     const double* xyz, int64_t ndir, const int64_t* dirnodes,
                     const double* dirvals, const double* x, int64_t* nnz_out,
                     int64_t* ia, int64_t* ja, double* a, double* ax, double* bmod) {
  try {
    auto ip = ids(inpoel, nelem * 4);
    auto psup = tk::genPsup(ip, 4, tk::genEsup(ip, 4));
    tk::CSR A(1, psup);
    const double* X = xyz;
    const double* Y = xyz + npoin;
    const double* Z = xyz + 2 * npoin;
    for (int64_t e = 0; e < nelem; ++e) {
      const auto N = ip.data() + e * 4;
      std::array<tk::real, 3> ba{{X[N[1]] - X[N[0]], Y[N[1]] - Y[N[0]], Z[N[1]] - Z[N[0]]}},
          ca{{X[N[2]] - X[N[0]], Y[N[2]] - Y[N[0]], Z[N[2]] - Z[N[0]]}},
          da{{X[N[3]] - X[N[0]], Y[N[3]] - Y[N[0]], Z[N[3]] - Z[N[0]]}};
      const auto J = tk::triple(ba, ca, da) * 6.0;
      std::array<std::array<tk::real, 3>, 4> grad;
      grad[1] = tk::cross(ca, da);
      grad[2] = tk::cross(da, ba);
      grad[3] = tk::cross(ba, ca);
      for (std::size_t i = 0; i < 3; ++i) grad[0][i] = -grad[1][i] - grad[2][i] - grad[3][i];
      for (std::size_t aa = 0; aa < 4; ++aa)
        for (std::size_t b = 0; b < 4; ++b) A(N[aa], N[b]) -= tk::dot(grad[aa], grad[b]) / J;
    }
    std::vector<tk::real> r(static_cast<std::size_t>(npoin), 0.0);
    for (int64_t k = ndir - 1; k >= 0; --k) A.dirichlet(static_cast<std::size_t>(dirnodes[k]), dirvals[k], r);
    // Walk rows with operator() over psup neighbours to extract entries.
    std::vector<int64_t> cia(static_cast<std::size_t>(npoin) + 1, 1);
    std::vector<int64_t> cja;
    std::vector<double> ca_;
    for (int64_t i = 0; i < npoin; ++i) {
      std::vector<std::size_t> cols{static_cast<std::size_t>(i)};
      for (auto j = psup.second[i] + 1; j <= psup.second[i + 1]; ++j) cols.push_back(psup.first[j]);
      std::sort(cols.begin(), cols.end());
      for (auto c : cols) {
        cja.push_back(static_cast<int64_t>(c) + 1);
        ca_.push_back(A(static_cast<std::size_t>(i), c, 0));
      }
      cia[i + 1] = cia[i] + static_cast<int64_t>(cols.size());
    }
    std::size_t nnz = cja.size();
    *nnz_out = static_cast<int64_t>(nnz);
    if (ia) std::memcpy(ia, cia.data(), sizeof(int64_t) * cia.size());
    if (ja) std::memcpy(ja, cja.data(), sizeof(int64_t) * nnz);
    if (a) std::memcpy(a, ca_.data(), sizeof(double) * nnz);
    if (ax && x) {
      std::vector<tk::real> xv(x, x + npoin), rv(static_cast<std::size_t>(npoin));
      A.mult(xv, rv);
      std::memcpy(ax, rv.data(), sizeof(double) * rv.size());
    }
    if (bmod) std::memcpy(bmod, r.data(), sizeof(double) * r.size());
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

}  // extern "C"
