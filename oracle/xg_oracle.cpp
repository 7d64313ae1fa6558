// ORACLE -- test infrastructure only.
//
// A plain, serial C++ restatement of the reference's CPU arithmetic on the
// accelerated path, used exclusively as the checker by tests/, by
// __graft_entry__.smoke() and by the CPU-baseline leg of bench.py.  No product
// code links, loads or calls this file.  Every function cites the reference
// lines it follows (paths relative to the reference project root).
//
// Parity of this restatement is pinned against the reference itself: the
// reference's own compiled functions (oracle/_ref, built by
// oracle/build_ref.sh from the unmodified sources) and the reference's
// golden vectors (tests/golden/).
//
// Conventions shared with the reference:
//   * fields are node-major: U[i*ncomp + c] (tk::Data<UnkEqComp>,
//     src/Base/Data.hpp:419-426);
//   * coordinates are SoA: xyz[0..n) = x, [n..2n) = y, [2n..3n) = z;
//   * an edge (p,q) with its dual-face integral D is evaluated with p as the
//     left state and contributes -f to p and +f to q (src/Physics/Riemann.cpp:
//     745-759).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <set>
#include <string>
#include <vector>

extern "C" {
void orc_csr_dirichlet(int64_t n, const int64_t* ia, const int64_t* ja, double* a, double* b,
                       int64_t ndir, const int64_t* nodes, const double* vals);
int64_t orc_pcg(int64_t n, const int64_t* ia, const int64_t* ja, const double* a,
                const double* b, double* x, int64_t maxit, double tol, int pc,
                double* normr_out, double* normb_out, int* converged);
}

namespace {

using real = double;

// --------------------------------------------------------------------------
// vector helpers (src/Base/Vector.hpp:35-176)
inline void cross(real ax, real ay, real az, real bx, real by, real bz, real& rx,
                  real& ry, real& rz) {
  rx = ay * bz - by * az;
  ry = az * bx - bz * ax;
  rz = ax * by - bx * ay;
}
inline real triple(const real a[3], const real b[3], const real c[3]) {
  real cx, cy, cz;
  cross(b[0], b[1], b[2], c[0], c[1], c[2], cx, cy, cz);
  return a[0] * cx + a[1] * cy + a[2] * cz;
}

// Tet edge and face tables (src/Mesh/DerivedData.hpp:35-44).
const int lpoed[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};

struct Tet {
  real J;            // triple product, 6V
  real grad[4][3];   // J * shape-function gradients
};

// Element geometry as computed in RieCG::domint (src/Inciter/RieCG.cpp:357-368)
// and kozak::rhs (src/Physics/Kozak.cpp:76-89).
Tet tetgeo(const real* x, const real* y, const real* z, const int64_t* N) {
  Tet t;
  real ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
  real ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
  real da[3] = {x[N[3]] - x[N[0]], y[N[3]] - y[N[0]], z[N[3]] - z[N[0]]};
  t.J = triple(ba, ca, da);
  cross(ca[0], ca[1], ca[2], da[0], da[1], da[2], t.grad[1][0], t.grad[1][1], t.grad[1][2]);
  cross(da[0], da[1], da[2], ba[0], ba[1], ba[2], t.grad[2][0], t.grad[2][1], t.grad[2][2]);
  cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], t.grad[3][0], t.grad[3][1], t.grad[3][2]);
  for (int i = 0; i < 3; ++i) t.grad[0][i] = -t.grad[1][i] - t.grad[2][i] - t.grad[3][i];
  return t;
}

std::string g_err;

// --------------------------------------------------------------------------
// RieCG state
struct RieCG {
  int64_t npoin = 0;
  std::vector<real> x, y, z, vol;
  std::vector<int64_t> edge;   // 2 per edge, canonical orientation
  std::vector<real> dedge;     // 3 per edge
  std::vector<int64_t> tri;    // 3 per boundary triangle
  std::vector<uint8_t> besym;  // 3 per boundary triangle
  std::vector<int64_t> symnode;
  std::vector<real> symnorm;
  std::vector<int64_t> farnode;
  std::vector<real> farnorm;
  real far_r = 1, far_u[3] = {0, 0, 0}, far_p = 1;
  std::vector<int64_t> dirnode;
  std::vector<int32_t> dirmask;  // 5 per node: 0 keep, otherwise set dirval
  std::vector<real> dirval;      // 5 per node
  std::vector<int64_t> prenode;
  std::vector<real> preval;      // density, pressure per node
  real gamma = 1.4, stab2coef = 0.2, cfl = 0.5, const_dt = 0.0;
  int flux = 0;  // 0 rusanov, 1 hllc
  int stab2 = 0;
  std::vector<real> U, Un, G, R;
  real t = 0, dt = 0;
  int stage = 0;
  int64_t it = 0;
  // manufactured source (riemann::src): problem 0 none, 1 taylor_green,
  // 2 vortical_flow, 3 nonlinear_energy_growth, 4 rayleigh_taylor; prm =
  // alpha, beta[3], kappa, r0, p0, ce
  int src = 0;
  real sprm[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

// EOS (src/Physics/EOS.hpp:29-56)
inline real pressure(const RieCG& s, real re) { return re * (s.gamma - 1.0); }
inline real soundspeed(const RieCG& s, real r, real p) { return std::sqrt(s.gamma * p / r); }
inline real totalenergy(const RieCG& s, real r, real u, real v, real w, real p) {
  return p / (s.gamma - 1.0) + 0.5 * r * (u * u + v * v + w * w);
}

// primitive() (src/Physics/Riemann.cpp:211-227)
inline void primitive(const real* U, int64_t i, real u[5]) {
  u[0] = U[i * 5 + 0];
  u[1] = U[i * 5 + 1] / u[0];
  u[2] = U[i * 5 + 2] / u[0];
  u[3] = U[i * 5 + 3] / u[0];
  u[4] = U[i * 5 + 4] / u[0] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]);
}

// muscl() for the five flow variables (src/Physics/Riemann.cpp:34-143):
// van Leer limited reconstruction with eps 1e-9 and k = 1/3, falling back to
// first order when density or internal energy could turn negative.
void muscl(const RieCG& s, int64_t p, int64_t q, const real* G, real l[5], real r[5]) {
  const real eps = 1.0e-9, k = 1.0 / 3.0;
  real vw[3] = {s.x[q] - s.x[p], s.y[q] - s.y[p], s.z[q] - s.z[p]};
  real d1[5], d2[5], d3[5], ls[5], rs[5], url[5], urr[5];
  for (int c = 0; c < 5; ++c) {
    ls[c] = url[c] = l[c];
    rs[c] = urr[c] = r[c];
  }
  for (int c = 0; c < 5; ++c) {
    real g1 = G[p * 15 + c * 3 + 0] * vw[0] + G[p * 15 + c * 3 + 1] * vw[1] + G[p * 15 + c * 3 + 2] * vw[2];
    real g2 = G[q * 15 + c * 3 + 0] * vw[0] + G[q * 15 + c * 3 + 1] * vw[1] + G[q * 15 + c * 3 + 2] * vw[2];
    d2[c] = rs[c] - ls[c];
    d1[c] = 2.0 * g1 - d2[c];
    d3[c] = 2.0 * g2 - d2[c];
    real rcL = (d2[c] + eps) / (d1[c] + eps);
    real rcR = (d2[c] + eps) / (d3[c] + eps);
    real rLinv = (d1[c] + eps) / (d2[c] + eps);
    real rRinv = (d3[c] + eps) / (d2[c] + eps);
    real phiL = (std::abs(rcL) + rcL) / (std::abs(rcL) + 1.0);
    real phiR = (std::abs(rcR) + rcR) / (std::abs(rcR) + 1.0);
    real phiLi = (std::abs(rLinv) + rLinv) / (std::abs(rLinv) + 1.0);
    real phiRi = (std::abs(rRinv) + rRinv) / (std::abs(rRinv) + 1.0);
    url[c] += 0.25 * (d1[c] * (1.0 - k) * phiL + d2[c] * (1.0 + k) * phiLi);
    urr[c] -= 0.25 * (d3[c] * (1.0 - k) * phiR + d2[c] * (1.0 + k) * phiRi);
  }
  if (ls[0] < d1[0] || ls[4] < d1[4])
    for (int c = 0; c < 5; ++c) url[c] = ls[c];
  if (rs[0] < -d3[0] || rs[4] < -d3[4])
    for (int c = 0; c < 5; ++c) urr[c] = rs[c];
  for (int c = 0; c < 5; ++c) {
    l[c] = url[c];
    r[c] = urr[c];
  }
}

// rusanov() (src/Physics/Riemann.cpp:369-478), flow variables only.
void rusanov(const RieCG& s, const real* G, const real* d, int64_t p, int64_t q,
             const real L[5], const real R[5], real f[5]) {
  real l[5], r[5];
  for (int c = 0; c < 5; ++c) {
    l[c] = L[c];
    r[c] = R[c];
  }
  muscl(s, p, q, G, l, r);
  real pL = pressure(s, l[0] * l[4]);
  real pR = pressure(s, r[0] * r[4]);
  real nx = d[0], ny = d[1], nz = d[2];
  real vnL = l[1] * nx + l[2] * ny + l[3] * nz;
  real vnR = r[1] * nx + r[2] * ny + r[3] * nz;
  l[4] = (l[4] + 0.5 * (l[1] * l[1] + l[2] * l[2] + l[3] * l[3])) * l[0];
  l[1] *= l[0];
  l[2] *= l[0];
  l[3] *= l[0];
  r[4] = (r[4] + 0.5 * (r[1] * r[1] + r[2] * r[2] + r[3] * r[3])) * r[0];
  r[1] *= r[0];
  r[2] *= r[0];
  r[3] *= r[0];
  real len = std::sqrt(nx * nx + ny * ny + nz * nz);
  real sl = std::abs(vnL) + soundspeed(s, l[0], pL) * len;
  real sr = std::abs(vnR) + soundspeed(s, r[0], pR) * len;
  real fw = std::max(sl, sr);
  f[0] = l[0] * vnL + r[0] * vnR + fw * (r[0] - l[0]);
  f[1] = l[1] * vnL + r[1] * vnR + (pL + pR) * nx + fw * (r[1] - l[1]);
  f[2] = l[2] * vnL + r[2] * vnR + (pL + pR) * ny + fw * (r[2] - l[2]);
  f[3] = l[3] * vnL + r[3] * vnR + (pL + pR) * nz + fw * (r[3] - l[3]);
  f[4] = (l[4] + pL) * vnL + (r[4] + pR) * vnR + fw * (r[4] - l[4]);
  if (s.stab2) {
    real fws = s.stab2coef * fw;
    for (int c = 0; c < 5; ++c) f[c] -= fws * (l[c] - r[c]);
  }
}

// hllc() (src/Physics/Riemann.cpp:480-650), flow variables only.
void hllc(const RieCG& s, const real* G, const real* d, int64_t p, int64_t q,
          const real L[5], const real R[5], real f[5]) {
  real l[5], r[5];
  for (int c = 0; c < 5; ++c) {
    l[c] = L[c];
    r[c] = R[c];
  }
  muscl(s, p, q, G, l, r);
  real nx = -d[0], ny = -d[1], nz = -d[2];
  real len = std::sqrt(nx * nx + ny * ny + nz * nz);
  nx /= len;
  ny /= len;
  nz /= len;
  real qL = l[1] * nx + l[2] * ny + l[3] * nz;
  real qR = r[1] * nx + r[2] * ny + r[3] * nz;
  real pL = pressure(s, l[0] * l[4]);
  real pR = pressure(s, r[0] * r[4]);
  l[4] = (l[4] + 0.5 * (l[1] * l[1] + l[2] * l[2] + l[3] * l[3])) * l[0];
  l[1] *= l[0];
  l[2] *= l[0];
  l[3] *= l[0];
  r[4] = (r[4] + 0.5 * (r[1] * r[1] + r[2] * r[2] + r[3] * r[3])) * r[0];
  r[1] *= r[0];
  r[2] *= r[0];
  r[3] *= r[0];
  real cL = soundspeed(s, l[0], pL);
  real cR = soundspeed(s, r[0], pR);
  real sL = std::fmin(qL - cL, qR - cR);
  real sR = std::fmax(qL + cL, qR + cR);
  real tL = sL - qL;
  real tR = sR - qR;
  real sM = (r[0] * qR * tR - l[0] * qL * tL + pL - pR) / (r[0] * tR - l[0] * tL);
  real pS = pL - l[0] * tL * (qL - sM);
  real uL[5], uR[5];
  real sd = sL - sM;
  uL[0] = tL * l[0] / sd;
  uL[1] = (tL * l[1] + (pS - pL) * nx) / sd;
  uL[2] = (tL * l[2] + (pS - pL) * ny) / sd;
  uL[3] = (tL * l[3] + (pS - pL) * nz) / sd;
  uL[4] = (tL * l[4] - pL * qL + pS * sM) / sd;
  sd = sR - sM;
  uR[0] = tR * r[0] / sd;
  uR[1] = (tR * r[1] + (pS - pR) * nx) / sd;
  uR[2] = (tR * r[2] + (pS - pR) * ny) / sd;
  uR[3] = (tR * r[3] + (pS - pR) * nz) / sd;
  uR[4] = (tR * r[4] - pR * qR + pS * sM) / sd;
  real L2 = -2.0 * len;
  nx *= L2;
  ny *= L2;
  nz *= L2;
  if (sL > 0.0) {
    real qL2 = qL * L2;
    f[0] = l[0] * qL2;
    f[1] = l[1] * qL2 + pL * nx;
    f[2] = l[2] * qL2 + pL * ny;
    f[3] = l[3] * qL2 + pL * nz;
    f[4] = (l[4] + pL) * qL2;
  } else if (sL <= 0.0 && sM > 0.0) {
    real qL2 = qL * L2, sL2 = sL * L2;
    f[0] = l[0] * qL2 + sL2 * (uL[0] - l[0]);
    f[1] = l[1] * qL2 + pL * nx + sL2 * (uL[1] - l[1]);
    f[2] = l[2] * qL2 + pL * ny + sL2 * (uL[2] - l[2]);
    f[3] = l[3] * qL2 + pL * nz + sL2 * (uL[3] - l[3]);
    f[4] = (l[4] + pL) * qL2 + sL2 * (uL[4] - l[4]);
  } else if (sM <= 0.0 && sR >= 0.0) {
    real qR2 = qR * L2, sR2 = sR * L2;
    f[0] = r[0] * qR2 + sR2 * (uR[0] - r[0]);
    f[1] = r[1] * qR2 + pR * nx + sR2 * (uR[1] - r[1]);
    f[2] = r[2] * qR2 + pR * ny + sR2 * (uR[2] - r[2]);
    f[3] = r[3] * qR2 + pR * nz + sR2 * (uR[3] - r[3]);
    f[4] = (r[4] + pR) * qR2 + sR2 * (uR[4] - r[4]);
  } else {
    real qR2 = qR * L2;
    f[0] = r[0] * qR2;
    f[1] = r[1] * qR2 + pR * nx;
    f[2] = r[2] * qR2 + pR * ny;
    f[3] = r[3] * qR2 + pR * nz;
    f[4] = (r[4] + pR) * qR2;
  }
  if (s.stab2) {
    real sl = std::abs(qL) + cL;
    real sr = std::abs(qR) + cR;
    real fws = s.stab2coef * std::max(sl, sr) * len;
    for (int c = 0; c < 5; ++c) f[c] -= fws * (l[c] - r[c]);
  }
}

// riemann::grad (src/Physics/Riemann.cpp:229-367) over plain edges.
void riecg_grad(const RieCG& s, const real* U, real* G) {
  const int64_t n = s.npoin;
  std::fill(G, G + n * 15, 0.0);
  const int64_t ne = static_cast<int64_t>(s.edge.size() / 2);
  for (int64_t e = 0; e < ne; ++e) {
    int64_t N0 = s.edge[e * 2], N1 = s.edge[e * 2 + 1];
    real u0[5], u1[5];
    primitive(U, N0, u0);
    primitive(U, N1, u1);
    const real* d = &s.dedge[e * 3];
    for (int c = 0; c < 5; ++c)
      for (int j = 0; j < 3; ++j) {
        real f = d[j] * (u1[c] + u0[c]);
        G[N0 * 15 + c * 3 + j] -= f;
        G[N1 * 15 + c * 3 + j] += f;
      }
  }
  const int64_t nt = static_cast<int64_t>(s.tri.size() / 3);
  for (int64_t e = 0; e < nt; ++e) {
    const int64_t* N = &s.tri[e * 3];
    real u[3][5];
    for (int a = 0; a < 3; ++a) primitive(U, N[a], u[a]);
    real ba[3] = {s.x[N[1]] - s.x[N[0]], s.y[N[1]] - s.y[N[0]], s.z[N[1]] - s.z[N[0]]};
    real ca[3] = {s.x[N[2]] - s.x[N[0]], s.y[N[2]] - s.y[N[0]], s.z[N[2]] - s.z[N[0]]};
    real nn[3];
    cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], nn[0], nn[1], nn[2]);
    for (int j = 0; j < 3; ++j) nn[j] /= 12.0;
    for (int c = 0; c < 5; ++c) {
      real uab = (u[0][c] + u[1][c]) / 4.0;
      real ubc = (u[1][c] + u[2][c]) / 4.0;
      real uca = (u[2][c] + u[0][c]) / 4.0;
      real g[3] = {uab + uca + u[0][c], uab + ubc + u[1][c], ubc + uca + u[2][c]};
      for (int j = 0; j < 3; ++j)
        for (int a = 0; a < 3; ++a) G[N[a] * 15 + c * 3 + j] += g[j] * nn[j];
    }
  }
}

// Source terms of the manufactured-solution problems at (x, y, z, t), the
// problems' src functions (src/Physics/Problems.cpp: nonlinear_energy_growth
// 163-220, rayleigh_taylor 261-332, taylor_green 433-449, vortical_flow
// 481-508), restated from their formulas.
// src: 0 none, 1 taylor_green, 2 vortical_flow, 3 nonlinear_energy_growth,
// 4 rayleigh_taylor; sprm: alpha, beta[3], kappa, r0, p0, ce.
void problem_source(int src, const real* sprm, real gamma, real x, real y, real z, real t,
                    real o[5]) {
  const real pi = M_PI, g = gamma;
  const real a = sprm[0], b0 = sprm[1], b1 = sprm[2], b2 = sprm[3];
  const real kap = sprm[4], r0 = sprm[5], p0 = sprm[6], ce = sprm[7];
  for (int c = 0; c < 5; ++c) o[c] = 0.0;
  if (src == 1) {  // taylor_green: energy only
    o[4] = 3.0 * pi / 8.0 *
           (std::cos(3.0 * pi * x) * std::cos(pi * y) - std::cos(3.0 * pi * y) * std::cos(pi * x));
  } else if (src == 2) {  // vortical_flow: rho = 1, linear velocity field
    const real rho = 1.0;
    const real mx = a * x - kap * y, my = kap * x + a * y;
    o[1] = a * mx / rho - kap * my / rho;
    o[2] = kap * mx / rho + a * my / rho;
    o[4] = (o[1] * mx + o[2] * my) / rho + 8.0 * a * a * a * z * z / (g - 1.0);
  } else if (src == 3) {  // nonlinear_energy_growth
    const real gx = 1.0 - x * x - y * y - z * z;
    const real dg[3] = {-2.0 * x, -2.0 * y, -2.0 * z};
    const real cx = std::cos(b0 * pi * x), cy = std::cos(b1 * pi * y), cz = std::cos(b2 * pi * z);
    const real h = cx * cy * cz;
    const real dh[3] = {-b0 * pi * std::sin(b0 * pi * x) * cy * cz,
                        -b1 * pi * cx * std::sin(b1 * pi * y) * cz,
                        -b2 * pi * cx * cy * std::sin(b2 * pi * z)};
    const real ft = std::exp(-a * t), dfdt = -a * ft;
    const real rho = r0 + ft * gx, drdt = gx * dfdt;
    const real ie = std::pow(-3.0 * (ce + kap * h * h * t), -1.0 / 3.0);
    const real ie4 = std::pow(ie, 4.0);
    o[0] = drdt;
    for (int j = 0; j < 3; ++j) {
      const real dedx = 2.0 * ie4 * kap * h * dh[j] * t, drdx = ft * dg[j];
      o[1 + j] = (g - 1.0) * (rho * dedx + ie * drdx);
    }
    o[4] = rho * (kap * h * h * ie4) + ie * drdt;
  } else if (src == 4) {  // rayleigh_taylor
    const real gx = b0 * x * x + b1 * y * y + b2 * z * z;
    const real ft = std::cos(kap * pi * t), st = std::sin(kap * pi * t);
    const real sx = std::sin(pi * x), cx = std::cos(pi * x);
    const real sy = std::sin(pi * y), cy = std::cos(pi * y);
    // the solution as the problem's initial condition forms it, conserved
    const real r = r0 - gx;
    const real u0 = ft * z * sx, v0 = ft * z * cy, w0 = ft * (-0.5 * pi * z * z * (cx - sy));
    const real rE = (p0 + a * gx) / (g - 1.0) + 0.5 * r * (u0 * u0 + v0 * v0 + w0 * w0);
    const real m[3] = {r * u0, r * v0, r * w0};
    // and back to primitives
    const real rho = r, u = m[0] / rho, v = m[1] / rho, w = m[2] / rho, E = rE / rho;
    const real p = p0 + a * (b0 * x * x + b1 * y * y + b2 * z * z);
    const real drdx[3] = {-2.0 * b0 * x, -2.0 * b1 * y, -2.0 * b2 * z};
    const real dpdx[3] = {2.0 * a * b0 * x, 2.0 * a * b1 * y, 2.0 * a * b2 * z};
    const real dudx[3] = {ft * pi * z * cx, 0.0, ft * sx};
    const real dvdx[3] = {0.0, -ft * pi * z * sy, ft * cy};
    const real dwdx[3] = {ft * pi * 0.5 * pi * z * z * sx, ft * pi * 0.5 * pi * z * z * cy,
                          -ft * pi * z * (cx - sy)};
    real dedx[3];
    for (int j = 0; j < 3; ++j)
      dedx[j] = dpdx[j] / rho / (g - 1.0) - p / (g - 1.0) / rho / rho * drdx[j] + u * dudx[j] +
                v * dvdx[j] + w * dwdx[j];
    const real dudt = -kap * pi * st * z * sx, dvdt = -kap * pi * st * z * cy;
    const real dwdt = kap * pi * st / 2.0 * pi * z * z * (cx - sy);
    const real dedt = u * dudt + v * dvdt + w * dwdt;
    o[0] = u * drdx[0] + v * drdx[1] + w * drdx[2];
    o[1] = rho * dudt + u * o[0] + dpdx[0] + m[0] * dudx[0] + m[1] * dudx[1] + m[2] * dudx[2];
    o[2] = rho * dvdt + v * o[0] + dpdx[1] + m[0] * dvdx[0] + m[1] * dvdx[1] + m[2] * dvdx[2];
    o[3] = rho * dwdt + w * o[0] + dpdx[2] + m[0] * dwdx[0] + m[1] * dwdx[1] + m[2] * dwdx[2];
    o[4] = rho * dedt + E * o[0] + m[0] * dedx[0] + m[1] * dedx[1] + m[2] * dedx[2] +
           u * dpdx[0] + v * dpdx[1] + w * dpdx[2];
  }
}

// The problems' analytic states at (x, y, z, t), conserved variables (the
// problems' ic functions, src/Physics/Problems.cpp: nonlinear_energy_growth
// 117-151, rayleigh_taylor 226-258, taylor_green 409-428, vortical_flow
// 453-478, with eos::totalenergy, src/Physics/EOS.hpp:53-56): what
// physics::dirbc sets where a Dirichlet mask is 1.
void problem_ic(int src, const real* sprm, real gamma, real x, real y, real z, real t,
                real o[5]) {
  const real g = gamma;
  const real a = sprm[0], b0 = sprm[1], b1 = sprm[2], b2 = sprm[3];
  const real kap = sprm[4], r0 = sprm[5], p0 = sprm[6], ce = sprm[7];
  auto energy = [g](real r, real u, real v, real w, real p) {
    return p / (g - 1.0) + 0.5 * r * (u * u + v * v + w * w);
  };
  if (src == 1) {  // taylor_green
    const real r = 1.0;
    const real p = 10.0 + r / 4.0 * (std::cos(2.0 * M_PI * x) + std::cos(2.0 * M_PI * y));
    const real u = std::sin(M_PI * x) * std::cos(M_PI * y);
    const real v = -std::cos(M_PI * x) * std::sin(M_PI * y);
    const real w = 0.0;
    const real rE = energy(r, u, v, w, p);
    o[0] = r, o[1] = r * u, o[2] = r * v, o[3] = r * w, o[4] = rE;
  } else if (src == 2) {  // vortical_flow
    const real ru = a * x - kap * y, rv = kap * x + a * y, rw = -2.0 * a * z;
    const real rE = (ru * ru + rv * rv + rw * rw) / 2.0 + (p0 - 2.0 * a * a * z * z) / (g - 1.0);
    o[0] = 1.0, o[1] = ru, o[2] = rv, o[3] = rw, o[4] = rE;
  } else if (src == 3) {  // nonlinear_energy_growth
    const real h = std::cos(b0 * M_PI * x) * std::cos(b1 * M_PI * y) * std::cos(b2 * M_PI * z);
    const real r = r0 + std::exp(-a * t) * (1.0 - x * x - y * y - z * z);
    const real re = r * std::pow(-3.0 * (ce + kap * h * h * t), -1.0 / 3.0);
    o[0] = r, o[1] = 0.0, o[2] = 0.0, o[3] = 0.0, o[4] = re;
  } else {  // rayleigh_taylor
    const real gx = b0 * x * x + b1 * y * y + b2 * z * z;
    const real r = r0 - gx;
    const real ft = std::cos(kap * M_PI * t);
    const real u = ft * z * std::sin(M_PI * x);
    const real v = ft * z * std::cos(M_PI * y);
    const real w = ft * (-0.5 * M_PI * z * z * (std::cos(M_PI * x) - std::sin(M_PI * y)));
    const real rE = energy(r, u, v, w, p0 + a * gx);
    o[0] = r, o[1] = r * u, o[2] = r * v, o[3] = r * w, o[4] = rE;
  }
}

// Dirichlet values of node p at time t (physics::dirbc, src/Physics/
// BC.cpp:30-71): with a problem set, components of mask 1 take its analytic
// state at t; any other set component its given value.
void dirichlet(int src, const real* sprm, real gamma, real x, real y, real z, real t,
               const int32_t* mask, const real* val, real* u) {
  real ic[5];
  if (src) problem_ic(src, sprm, gamma, x, y, z, t, ic);
  for (int c = 0; c < 5; ++c) {
    if (mask[c] == 1 && src)
      u[c] = ic[c];
    else if (mask[c])
      u[c] = val[c];
  }
}

// riemann::rhs = advdom + advbnd + src (src/Physics/Riemann.cpp:652-946),
// the source at the state's time t (RieCG::rhs passes the time at the start
// of the step to every stage, RieCG.cpp:948-949).
void riecg_rhs(const RieCG& s, const real* G, const real* U, real* R) {
  const int64_t n = s.npoin;
  std::fill(R, R + n * 5, 0.0);
  const int64_t ne = static_cast<int64_t>(s.edge.size() / 2);
  for (int64_t e = 0; e < ne; ++e) {
    int64_t N0 = s.edge[e * 2], N1 = s.edge[e * 2 + 1];
    real u0[5], u1[5], f[5];
    primitive(U, N0, u0);
    primitive(U, N1, u1);
    const real* d = &s.dedge[e * 3];
    if (s.flux == 1)
      hllc(s, G, d, N0, N1, u0, u1, f);
    else
      rusanov(s, G, d, N0, N1, u0, u1, f);
    for (int c = 0; c < 5; ++c) {
      R[N0 * 5 + c] -= f[c];
      R[N1 * 5 + c] += f[c];
    }
  }
  const int64_t nt = static_cast<int64_t>(s.tri.size() / 3);
  for (int64_t e = 0; e < nt; ++e) {
    const int64_t* N = &s.tri[e * 3];
    real ba[3] = {s.x[N[1]] - s.x[N[0]], s.y[N[1]] - s.y[N[0]], s.z[N[1]] - s.z[N[0]]};
    real ca[3] = {s.x[N[2]] - s.x[N[0]], s.y[N[2]] - s.y[N[0]], s.z[N[2]] - s.z[N[0]]};
    real nx, ny, nz;
    cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], nx, ny, nz);
    nx /= 12.0;
    ny /= 12.0;
    nz /= 12.0;
    real f[5][3];
    for (int a = 0; a < 3; ++a) {
      const real* u = &U[N[a] * 5];
      real p = pressure(s, u[4] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
      real vn = s.besym[e * 3 + a] ? 0.0 : (nx * u[1] + ny * u[2] + nz * u[3]) / u[0];
      f[0][a] = u[0] * vn;
      f[1][a] = u[1] * vn + p * nx;
      f[2][a] = u[2] * vn + p * ny;
      f[3][a] = u[3] * vn + p * nz;
      f[4][a] = (u[4] + p) * vn;
    }
    for (int c = 0; c < 5; ++c) {
      real fab = (f[c][0] + f[c][1]) / 4.0;
      real fbc = (f[c][1] + f[c][2]) / 4.0;
      real fca = (f[c][2] + f[c][0]) / 4.0;
      R[N[0] * 5 + c] += fab + fca + f[c][0];
      R[N[1] * 5 + c] += fab + fbc + f[c][1];
      R[N[2] * 5 + c] += fbc + fca + f[c][2];
    }
  }
  if (s.src)
    for (int64_t p = 0; p < n; ++p) {
      real so[5];
      problem_source(s.src, s.sprm, s.gamma, s.x[p], s.y[p], s.z[p], s.t, so);
      for (int c = 0; c < 5; ++c) R[p * 5 + c] -= so[c] * s.vol[p];
    }
}

// RieCG::BC (src/Inciter/RieCG.cpp:764-785) -> physics::dirbc, symbc, farbc,
// prebc (src/Physics/BC.cpp:29-72, 110-136, 152-220, 222-241).  Dirichlet
// values are given per node (time independent).
void riecg_bc(RieCG& s, real* U, real t) {
  for (size_t i = 0; i < s.dirnode.size(); ++i) {
    int64_t p = s.dirnode[i];
    dirichlet(s.src, s.sprm, s.gamma, s.x[p], s.y[p], s.z[p], t, &s.dirmask[i * 5],
              &s.dirval[i * 5], &U[p * 5]);
  }
  for (size_t i = 0; i < s.symnode.size(); ++i) {
    int64_t p = s.symnode[i];
    const real* n = &s.symnorm[i * 3];
    real& u = U[p * 5 + 1];
    real& v = U[p * 5 + 2];
    real& w = U[p * 5 + 3];
    real vn = u * n[0] + v * n[1] + w * n[2];
    u -= vn * n[0];
    v -= vn * n[1];
    w -= vn * n[2];
  }
  for (size_t i = 0; i < s.farnode.size(); ++i) {
    int64_t p = s.farnode[i];
    real nx = s.farnorm[i * 3 + 0], ny = s.farnorm[i * 3 + 1], nz = s.farnorm[i * 3 + 2];
    real& r = U[p * 5 + 0];
    real& ru = U[p * 5 + 1];
    real& rv = U[p * 5 + 2];
    real& rw = U[p * 5 + 3];
    real& re = U[p * 5 + 4];
    real fr = s.far_r, fu = s.far_u[0], fv = s.far_u[1], fw = s.far_u[2], fp = s.far_p;
    real vn = fu * nx + fv * ny + fw * nz;
    real a = soundspeed(s, fr, fp);
    real M = vn / a;
    if (M <= -1.0) {
      r = fr;
      ru = fr * fu;
      rv = fr * fv;
      rw = fr * fw;
      re = totalenergy(s, fr, fu, fv, fw, fp);
    } else if (M > -1.0 && M < 0.0) {
      real pr = pressure(s, re - 0.5 * (ru * ru + rv * rv + rw * rw) / r);
      r = fr;
      ru = fr * fu;
      rv = fr * fv;
      rw = fr * fw;
      re = totalenergy(s, fr, fu, fv, fw, pr);
    } else if (M >= 0.0 && M < 1.0) {
      re = totalenergy(s, r, ru / r, rv / r, rw / r, fp);
    }
  }
  for (size_t i = 0; i < s.prenode.size(); ++i) {
    int64_t p = s.prenode[i];
    U[p * 5 + 0] = s.preval[i * 2 + 0];
    U[p * 5 + 4] = totalenergy(s, U[p * 5 + 0], U[p * 5 + 1] / U[p * 5 + 0],
                               U[p * 5 + 2] / U[p * 5 + 0], U[p * 5 + 3] / U[p * 5 + 0],
                               s.preval[i * 2 + 1]);
  }
}

// RieCG::dt (src/Inciter/RieCG.cpp:787-852), unsteady branch.
real riecg_dt(const RieCG& s, const real* U) {
  if (std::abs(s.const_dt) > std::numeric_limits<real>::epsilon()) return s.const_dt;
  real mindt = std::numeric_limits<real>::max();
  for (int64_t p = 0; p < s.npoin; ++p) {
    real r = U[p * 5 + 0];
    real u = U[p * 5 + 1] / r, v = U[p * 5 + 2] / r, w = U[p * 5 + 3] / r;
    real pr = pressure(s, U[p * 5 + 4] - 0.5 * r * (u * u + v * v + w * w));
    real c = soundspeed(s, r, std::max(pr, 0.0));
    real L = std::cbrt(s.vol[p]);
    real vel = std::sqrt(u * u + v * v + w * w);
    real edt = L / std::max(vel + c, 1.0e-8);
    mindt = std::min(mindt, edt);
  }
  return mindt * s.cfl;
}

// One RK stage: RieCG::grad -> rhs -> solve (src/Inciter/RieCG.cpp:871-893,
// 918-966, 992-1057) with the low-storage coefficients {1/3, 1/2, 1}
// (RieCG.cpp:41).
void riecg_stage(RieCG& s, int stage) {
  static const real rkcoef[3] = {1.0 / 3.0, 1.0 / 2.0, 1.0};
  const int64_t n = s.npoin;
  riecg_grad(s, s.U.data(), s.G.data());
  for (int64_t p = 0; p < n; ++p)
    for (int c = 0; c < 15; ++c) s.G[p * 15 + c] /= s.vol[p];
  riecg_rhs(s, s.G.data(), s.U.data(), s.R.data());
  if (stage == 0) s.Un = s.U;
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 5; ++c)
      s.U[i * 5 + c] = s.Un[i * 5 + c] - rkcoef[stage] * s.dt * s.R[i * 5 + c] / s.vol[i];
  riecg_bc(s, s.U.data(), s.t + rkcoef[stage] * s.dt);  // RieCG.cpp:1028
}

// --------------------------------------------------------------------------
// KozCG state (src/Inciter/KozCG.cpp)
struct KozCG {
  int64_t npoin = 0, nelem = 0;
  std::vector<real> x, y, z, vol;
  std::vector<int64_t> inpoel;
  std::vector<int64_t> symnode;
  std::vector<real> symnorm;
  std::vector<int64_t> dirnode;
  std::vector<int32_t> dirmask;
  std::vector<real> dirval;
  real gamma = 1.4, cfl = 0.5, const_dt = 0.0, ctau = 1.0;
  int fct = 1, fctclip = 0;
  std::vector<int> fctsys;  // zero-based component ids limited together
  std::vector<real> U, R, P, Q, A;
  real t = 0, dt = 0;
  int64_t it = 0;
  int src = 0;  // manufactured source, as RieCG's
  real sprm[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

inline real kpressure(const KozCG& s, real re) { return re * (s.gamma - 1.0); }

// kozak::rhs (src/Physics/Kozak.cpp:29-180) at time t, with the problem's
// source when one is set (Kozak.cpp:125-132, 161-170).
void kozak_rhs(const KozCG& s, const real* U, real t, real dt, real* R) {
  std::fill(R, R + s.npoin * 5, 0.0);
  for (int64_t e = 0; e < s.nelem; ++e) {
    const int64_t* N = &s.inpoel[e * 4];
    Tet g = tetgeo(s.x.data(), s.y.data(), s.z.data(), N);
    real p[4];
    for (int a = 0; a < 4; ++a) {
      const real* u = &U[N[a] * 5];
      p[a] = kpressure(s, u[4] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
    }
    real ue[5];
    for (int c = 0; c < 5; ++c)
      ue[c] = (U[N[0] * 5 + c] + U[N[1] * 5 + c] + U[N[2] * 5 + c] + U[N[3] * 5 + c]) / 4.0;
    real coef = dt / g.J / 2.0;
    for (int j = 0; j < 3; ++j)
      for (int a = 0; a < 4; ++a) {
        const real* u = &U[N[a] * 5];
        real cg = coef * g.grad[a][j];
        real uj = u[j + 1] / u[0];
        ue[0] -= cg * u[j + 1];
        ue[1] -= cg * u[1] * uj;
        ue[2] -= cg * u[2] * uj;
        ue[3] -= cg * u[3] * uj;
        ue[j + 1] -= cg * p[a];
        ue[4] -= cg * (u[4] + p[a]) * uj;
      }
    if (s.src) {  // dt/8 of each node's source at t
      coef = dt / 8.0;
      for (int a = 0; a < 4; ++a) {
        real so[5];
        problem_source(s.src, s.sprm, s.gamma, s.x[N[a]], s.y[N[a]], s.z[N[a]], t, so);
        for (int c = 0; c < 5; ++c) ue[c] += coef * so[c];
      }
    }
    real r = ue[0], ru = ue[1], rv = ue[2], rw = ue[3];
    real pr = kpressure(s, ue[4] - 0.5 * (ru * ru + rv * rv + rw * rw) / r);
    coef = 1.0 / 6.0;
    for (int j = 0; j < 3; ++j) {
      real uj = ue[j + 1] / ue[0];
      for (int a = 0; a < 4; ++a) {
        real cg = coef * g.grad[a][j];
        real* Ra = &R[N[a] * 5];
        Ra[0] += cg * ue[j + 1];
        Ra[1] += cg * ue[1] * uj;
        Ra[2] += cg * ue[2] * uj;
        Ra[3] += cg * ue[3] * uj;
        Ra[j + 1] += cg * pr;
        Ra[4] += cg * (ue[4] + pr) * uj;
      }
    }
    if (s.src) {  // J/24 of the centroid's source at t + dt/2 to each node
      const real xe = (s.x[N[0]] + s.x[N[1]] + s.x[N[2]] + s.x[N[3]]) / 4.0;
      const real ye = (s.y[N[0]] + s.y[N[1]] + s.y[N[2]] + s.y[N[3]]) / 4.0;
      const real ze = (s.z[N[0]] + s.z[N[1]] + s.z[N[2]] + s.z[N[3]]) / 4.0;
      real se[5];
      problem_source(s.src, s.sprm, s.gamma, xe, ye, ze, t + dt / 2.0, se);
      coef = g.J / 24.0;
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 5; ++c) R[N[a] * 5 + c] += coef * se[c];
    }
  }
}

// KozCG::BC for the configured BC kinds (src/Inciter/KozCG.cpp:590-611).
void kozcg_bc(KozCG& s, real* U, real t) {
  for (size_t i = 0; i < s.dirnode.size(); ++i) {
    int64_t p = s.dirnode[i];
    dirichlet(s.src, s.sprm, s.gamma, s.x[p], s.y[p], s.z[p], t, &s.dirmask[i * 5],
              &s.dirval[i * 5], &U[p * 5]);
  }
  for (size_t i = 0; i < s.symnode.size(); ++i) {
    int64_t p = s.symnode[i];
    const real* n = &s.symnorm[i * 3];
    real& u = U[p * 5 + 1];
    real& v = U[p * 5 + 2];
    real& w = U[p * 5 + 3];
    real vn = u * n[0] + v * n[1] + w * n[2];
    u -= vn * n[0];
    v -= vn * n[1];
    w -= vn * n[2];
  }
}

// KozCG::dt (src/Inciter/KozCG.cpp:613-688), unsteady branch, freezeflow 1.
real kozcg_dt(const KozCG& s) {
  if (std::abs(s.const_dt) > std::numeric_limits<real>::epsilon()) return s.const_dt;
  real mindt = std::numeric_limits<real>::max();
  const real* U = s.U.data();
  for (int64_t p = 0; p < s.npoin; ++p) {
    real r = U[p * 5 + 0];
    real u = U[p * 5 + 1] / r, v = U[p * 5 + 2] / r, w = U[p * 5 + 3] / r;
    real pr = kpressure(s, U[p * 5 + 4] - 0.5 * r * (u * u + v * v + w * w));
    real c = std::sqrt(s.gamma * std::max(pr, 0.0) / r);
    real L = std::cbrt(s.vol[p]);
    real vel = std::sqrt(u * u + v * v + w * w);
    mindt = std::min(mindt, L / std::max(vel + c, 1.0e-8));
  }
  return mindt * s.cfl;
}

// One KozCG step: rhs -> aec -> alw -> lim -> solve
// (src/Inciter/KozCG.cpp:708-732, 772-843, 865-948, 978-1097, 1119-1197).
void kozcg_step(KozCG& s) {
  const int64_t n = s.npoin;
  const real* U = s.U.data();
  kozak_rhs(s, U, s.t, s.dt, s.R.data());
  std::vector<real>& R = s.R;
  if (!s.fct) {
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 5; ++c) s.A[i * 5 + c] = U[i * 5 + c] + s.dt * R[i * 5 + c] / s.vol[i];
  } else {
    // aec: antidiffusive element contributions P+/-
    std::fill(s.P.begin(), s.P.end(), 0.0);
    for (int64_t e = 0; e < s.nelem; ++e) {
      const int64_t* N = &s.inpoel[e * 4];
      Tet g = tetgeo(s.x.data(), s.y.data(), s.z.data(), N);
      for (int c = 0; c < 5; ++c) {
        real aec[4] = {0, 0, 0, 0};
        for (int a = 0; a < 4; ++a) {
          for (int b = 0; b < 4; ++b) {
            real m = g.J / 120.0 * ((a == b) ? 3.0 : -1.0);
            aec[a] += m * s.ctau * U[N[b] * 5 + c];
          }
          s.P[N[a] * 10 + c * 2 + 0] += std::max(0.0, aec[a]);
          s.P[N[a] * 10 + c * 2 + 1] += std::min(0.0, aec[a]);
        }
      }
    }
    for (size_t i = 0; i < s.symnode.size(); ++i) {
      int64_t p = s.symnode[i];
      real nx = s.symnorm[i * 3 + 0], ny = s.symnorm[i * 3 + 1], nz = s.symnorm[i * 3 + 2];
      real* P = &s.P[p * 10];
      real rvnp = P[2] * nx + P[4] * ny + P[6] * nz;
      real rvnn = P[3] * nx + P[5] * ny + P[7] * nz;
      P[2] -= rvnp * nx;
      P[3] -= rvnn * nx;
      P[4] -= rvnp * ny;
      P[5] -= rvnn * ny;
      P[6] -= rvnp * nz;
      P[7] -= rvnn * nz;
    }
    // alw: low-order solution and allowed limits Q+/-
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 5; ++c) {
        s.P[i * 10 + c * 2 + 0] /= s.vol[i];
        s.P[i * 10 + c * 2 + 1] /= s.vol[i];
        R[i * 5 + c] = U[i * 5 + c] + s.dt * R[i * 5 + c] / s.vol[i] - s.P[i * 10 + c * 2 + 0] -
                       s.P[i * 10 + c * 2 + 1];
      }
    const real large = std::numeric_limits<real>::max();
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 5; ++c) {
        s.Q[i * 10 + c * 2 + 0] = -large;
        s.Q[i * 10 + c * 2 + 1] = +large;
      }
    for (int64_t e = 0; e < s.nelem; ++e) {
      const int64_t* N = &s.inpoel[e * 4];
      for (int c = 0; c < 5; ++c) {
        real alwp = -large, alwn = +large;
        for (int a = 0; a < 4; ++a) {
          if (s.fctclip) {
            alwp = std::max(alwp, R[N[a] * 5 + c]);
            alwn = std::min(alwn, R[N[a] * 5 + c]);
          } else {
            alwp = std::max(alwp, std::max(R[N[a] * 5 + c], U[N[a] * 5 + c]));
            alwn = std::min(alwn, std::min(R[N[a] * 5 + c], U[N[a] * 5 + c]));
          }
        }
        for (int a = 0; a < 4; ++a) {
          real& qp = s.Q[N[a] * 10 + c * 2 + 0];
          real& qn = s.Q[N[a] * 10 + c * 2 + 1];
          qp = std::max(qp, alwp);
          qn = std::min(qn, alwn);
        }
      }
    }
    // lim: limit coefficients and limited antidiffusive contributions
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 5; ++c) {
        s.Q[i * 10 + c * 2 + 0] -= R[i * 5 + c];
        s.Q[i * 10 + c * 2 + 1] -= R[i * 5 + c];
      }
    const real eps = std::numeric_limits<real>::epsilon();
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 5; ++c) {
        real& qp = s.Q[i * 10 + c * 2 + 0];
        real& qn = s.Q[i * 10 + c * 2 + 1];
        real pp = s.P[i * 10 + c * 2 + 0], pn = s.P[i * 10 + c * 2 + 1];
        qp = pp < eps ? 0.0 : std::min(1.0, qp / pp);
        qn = pn > -eps ? 0.0 : std::min(1.0, qn / pn);
      }
    std::fill(s.A.begin(), s.A.end(), 0.0);
    for (int64_t e = 0; e < s.nelem; ++e) {
      const int64_t* N = &s.inpoel[e * 4];
      Tet g = tetgeo(s.x.data(), s.y.data(), s.z.data(), N);
      real coef[5], aec[5][4];
      for (int c = 0; c < 5; ++c) {
        coef[c] = 1.0;
        for (int a = 0; a < 4; ++a) {
          aec[c][a] = 0.0;
          for (int b = 0; b < 4; ++b) {
            real m = g.J / 120.0 * ((a == b) ? 3.0 : -1.0);
            aec[c][a] += m * s.ctau * U[N[b] * 5 + c];
          }
          coef[c] = std::min(coef[c], aec[c][a] > 0.0 ? s.Q[N[a] * 10 + c * 2 + 0]
                                                      : s.Q[N[a] * 10 + c * 2 + 1]);
        }
      }
      real cs = 1.0;
      for (int c : s.fctsys) cs = std::min(cs, coef[c]);
      for (int c : s.fctsys) coef[c] = cs;
      for (int c = 0; c < 5; ++c)
        for (int a = 0; a < 4; ++a) s.A[N[a] * 5 + c] += coef[c] * aec[c][a];
    }
    // solve: apply limited antidiffusive contributions
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 5; ++c) s.A[i * 5 + c] = R[i * 5 + c] + s.A[i * 5 + c] / s.vol[i];
  }
  kozcg_bc(s, s.A.data(), s.t + s.dt);  // KozCG.cpp:1167
  s.U = s.A;
}

// --------------------------------------------------------------------------
// Sparse matrix and PCG (src/LinearSolver/CSR.cpp, ConjugateGradients.cpp),
// zero-based scalar CSR with full (symmetric) rows sorted by column.
struct CG {
  int64_t n = 0;
  std::vector<int64_t> ia, ja;
  std::vector<real> a;
};

// CSR::mult (src/LinearSolver/CSR.cpp:154-172).
void csr_mult(const CG& A, const real* x, real* r) {
  for (int64_t i = 0; i < A.n; ++i) {
    real s = 0.0;
    for (int64_t j = A.ia[i]; j < A.ia[i + 1]; ++j) s += A.a[j] * x[A.ja[j]];
    r[i] = s;
  }
}


// --------------------------------------------------------------------------
// ChoCG (src/Inciter/ChoCG.cpp, src/Physics/Chorin.cpp) over plain edges:
// each edge (p,q) carries ChoCG's five integrals d[0..2] (dual-face normal),
// d[3] = J/120 and d[4] = grad_p.grad_q/J/6 (ChoCG::domint,
// src/Inciter/ChoCG.cpp:398-445) and contributes -f to p and +f to q, as the
// edge group of the chorin:: loops does (Chorin.cpp:160-170, 264-277, ...).
struct ChoCG {
  int64_t n = 0;
  std::vector<real> xyz, vol;
  std::vector<int64_t> edge;  // 2 per edge
  std::vector<real> dint;     // 5 per edge
  std::vector<int64_t> tri;   // boundary triangles
  real mu = 0, cfl = 0.5, const_dt = 0, stab2coef = 0.2;
  int damp4 = 0, stab = 1, stab2 = 0, rk = 1;
  // velocity BCs (ChoCG::BC, src/Inciter/ChoCG.cpp:1333-1354)
  std::vector<int64_t> dirn;
  std::vector<int32_t> dirmask;  // 3 per node
  std::vector<real> dirval;      // 3 per node
  std::vector<int64_t> symn;
  std::vector<real> symnorm;
  std::vector<int64_t> noslip;
  // pressure Dirichlet nodes and the values of the initial solves
  std::vector<int64_t> pdirn;
  std::vector<real> pdirval;
  // pressure system (ChoCG::prelhs) and its solver settings
  CG A;
  int pc = 1;
  real ptol = 1e-3;
  int64_t pmaxit = 10;
  // state
  std::vector<real> u, un, pr, pgrad, vgrad, flx, div, sgrad, rhs, sol;
  real t = 0, dt = 0;
  int np = 0;
  int64_t last_it = 0;
  real last_normr = 0, last_normb = 0;
  // theta-implicit momentum prediction: tetrahedra, the momentum system's
  // pattern (3 rows per node, row 3i + c), its warm-start solution and the
  // solver settings (mom_pc 0 none, 1 jacobi)
  real theta = 0;
  std::vector<int64_t> inpoel, mia, mja;
  std::vector<real> momx;
  int mom_pc = 0;
  int64_t mom_iter = 10;
  real mom_tol = 1e-3;
  int64_t last_mit = 0;
};

inline real cx(const ChoCG& s, int64_t p) { return s.xyz[p]; }
inline real cy(const ChoCG& s, int64_t p) { return s.xyz[s.n + p]; }
inline real cz(const ChoCG& s, int64_t p) { return s.xyz[2 * s.n + p]; }

// Boundary-face normal / 6 of triangle e (tk::crossdiv(..., 6.0)).
inline void cho_tri_normal(const ChoCG& s, int64_t e, real n[3]) {
  const int64_t* N = &s.tri[e * 3];
  cross(cx(s, N[1]) - cx(s, N[0]), cy(s, N[1]) - cy(s, N[0]), cz(s, N[1]) - cz(s, N[0]),
        cx(s, N[2]) - cx(s, N[0]), cy(s, N[2]) - cy(s, N[0]), cz(s, N[2]) - cz(s, N[0]), n[0],
        n[1], n[2]);
  n[0] /= 6.0;
  n[1] /= 6.0;
  n[2] /= 6.0;
}

// chorin::div (src/Physics/Chorin.cpp:34-83 per edge, 85-209 loops):
// divergence of U (3 components) with 4th-order pressure damping when stab.
void cho_div(const ChoCG& s, const real* U, const real* P, const real* G, real dt, bool stab,
             real* D) {
  for (int64_t e = 0; e < static_cast<int64_t>(s.edge.size() / 2); ++e) {
    const int64_t p = s.edge[2 * e], q = s.edge[2 * e + 1];
    const real* d = &s.dint[5 * e];
    real f = d[0] * (U[p * 3 + 0] + U[q * 3 + 0]) + d[1] * (U[p * 3 + 1] + U[q * 3 + 1]) +
             d[2] * (U[p * 3 + 2] + U[q * 3 + 2]);
    if (stab) {
      real dx = cx(s, p) - cx(s, q), dy = cy(s, p) - cy(s, q), dz = cz(s, p) - cz(s, q);
      real dl = std::sqrt(dx * dx + dy * dy + dz * dz);
      real p2 = P[q] - P[p];
      real Dn = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      real dpx = G[p * 3 + 0] + G[q * 3 + 0];
      real dpy = G[p * 3 + 1] + G[q * 3 + 1];
      real dpz = G[p * 3 + 2] + G[q * 3 + 2];
      real p4 = 0.5 * (dx * dpx + dy * dpy + dz * dpz);
      f += Dn * dt / dl * (p2 + p4);
    }
    D[p] -= f;
    D[q] += f;
  }
  for (int64_t e = 0; e < static_cast<int64_t>(s.tri.size() / 3); ++e) {
    const int64_t* N = &s.tri[e * 3];
    real n[3];
    cho_tri_normal(s, e, n);
    real uA[3], uB[3], uC[3];
    for (int c = 0; c < 3; ++c) {
      uA[c] = U[N[0] * 3 + c];
      uB[c] = U[N[1] * 3 + c];
      uC[c] = U[N[2] * 3 + c];
    }
    real ux = (6.0 * uA[0] + uB[0] + uC[0]) / 8.0;
    real uy = (6.0 * uA[1] + uB[1] + uC[1]) / 8.0;
    real uz = (6.0 * uA[2] + uB[2] + uC[2]) / 8.0;
    D[N[0]] += ux * n[0] + uy * n[1] + uz * n[2];
    ux = (uA[0] + 6.0 * uB[0] + uC[0]) / 8.0;
    uy = (uA[1] + 6.0 * uB[1] + uC[1]) / 8.0;
    uz = (uA[2] + 6.0 * uB[2] + uC[2]) / 8.0;
    D[N[1]] += ux * n[0] + uy * n[1] + uz * n[2];
    ux = (uA[0] + uB[0] + 6.0 * uC[0]) / 8.0;
    uy = (uA[1] + uB[1] + 6.0 * uC[1]) / 8.0;
    uz = (uA[2] + uB[2] + 6.0 * uC[2]) / 8.0;
    D[N[2]] += ux * n[0] + uy * n[1] + uz * n[2];
  }
}

// chorin::vgrad (Chorin.cpp:211-334) for ncomp components into G (ncomp*3);
// chorin::grad (Chorin.cpp:336-449) is the ncomp = 1 case.
void cho_vgrad(const ChoCG& s, const real* U, int ncomp, real* G) {
  const int nc3 = ncomp * 3;
  for (int64_t e = 0; e < static_cast<int64_t>(s.edge.size() / 2); ++e) {
    const int64_t p = s.edge[2 * e], q = s.edge[2 * e + 1];
    const real* d = &s.dint[5 * e];
    for (int i = 0; i < ncomp; ++i) {
      const real u0 = U[p * ncomp + i], u1 = U[q * ncomp + i];
      for (int j = 0; j < 3; ++j) {
        real f = d[j] * (u1 + u0);
        G[p * nc3 + i * 3 + j] -= f;
        G[q * nc3 + i * 3 + j] += f;
      }
    }
  }
  for (int64_t e = 0; e < static_cast<int64_t>(s.tri.size() / 3); ++e) {
    const int64_t* N = &s.tri[e * 3];
    real n[3];
    cho_tri_normal(s, e, n);
    for (int i = 0; i < ncomp; ++i) {
      real u[3] = {U[N[0] * ncomp + i], U[N[1] * ncomp + i], U[N[2] * ncomp + i]};
      real f = (6.0 * u[0] + u[1] + u[2]) / 8.0;
      for (int j = 0; j < 3; ++j) G[N[0] * nc3 + i * 3 + j] += f * n[j];
      f = (u[0] + 6.0 * u[1] + u[2]) / 8.0;
      for (int j = 0; j < 3; ++j) G[N[1] * nc3 + i * 3 + j] += f * n[j];
      f = (u[0] + u[1] + 6.0 * u[2]) / 8.0;
      for (int j = 0; j < 3; ++j) G[N[2] * nc3 + i * 3 + j] += f * n[j];
    }
  }
}

// Momentum flux of one tensor component over edge p-q and in point p
// (chorin flux, Chorin.cpp:451-507).
inline real cho_flux_e(const ChoCG& s, const real* U, const real* G, int i, int j, int64_t p,
                       int64_t q) {
  real inv = U[p * 3 + i] * U[p * 3 + j] + U[q * 3 + i] * U[q * 3 + j];
  const real eps = std::numeric_limits<real>::epsilon();
  if (s.mu < eps) return -inv;
  real vis = G[p * 9 + i * 3 + j] + G[p * 9 + j * 3 + i] + G[q * 9 + i * 3 + j] +
             G[q * 9 + j * 3 + i];
  if (i == j)
    vis -= 2.0 / 3.0 * (G[p * 9 + 0] + G[p * 9 + 4] + G[p * 9 + 8] + G[q * 9 + 0] +
                        G[q * 9 + 4] + G[q * 9 + 8]);
  return s.mu * vis - inv;
}
inline real cho_flux_p(const ChoCG& s, const real* U, const real* G, int i, int j, int64_t p) {
  real inv = U[p * 3 + i] * U[p * 3 + j];
  const real eps = std::numeric_limits<real>::epsilon();
  if (s.mu < eps) return -inv;
  real vis = G[p * 9 + i * 3 + j] + G[p * 9 + j * 3 + i];
  if (i == j) vis -= 2.0 / 3.0 * (G[p * 9 + 0] + G[p * 9 + 4] + G[p * 9 + 8]);
  return s.mu * vis - inv;
}

// chorin::flux (Chorin.cpp:509-638): F_i = d[s_ij - u_i u_j]/dx_j.
void cho_flux(const ChoCG& s, const real* U, const real* G, real* F) {
  for (int64_t e = 0; e < static_cast<int64_t>(s.edge.size() / 2); ++e) {
    const int64_t p = s.edge[2 * e], q = s.edge[2 * e + 1];
    const real* d = &s.dint[5 * e];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        real f = d[j] * cho_flux_e(s, U, G, i, j, q, p);
        F[p * 3 + i] -= f;
        F[q * 3 + i] += f;
      }
  }
  for (int64_t e = 0; e < static_cast<int64_t>(s.tri.size() / 3); ++e) {
    const int64_t* N = &s.tri[e * 3];
    real n[3];
    cho_tri_normal(s, e, n);
    for (int i = 0; i < 3; ++i) {
      real fxA = cho_flux_p(s, U, G, i, 0, N[0]), fyA = cho_flux_p(s, U, G, i, 1, N[0]),
           fzA = cho_flux_p(s, U, G, i, 2, N[0]);
      real fxB = cho_flux_p(s, U, G, i, 0, N[1]), fyB = cho_flux_p(s, U, G, i, 1, N[1]),
           fzB = cho_flux_p(s, U, G, i, 2, N[1]);
      real fxC = cho_flux_p(s, U, G, i, 0, N[2]), fyC = cho_flux_p(s, U, G, i, 1, N[2]),
           fzC = cho_flux_p(s, U, G, i, 2, N[2]);
      real fx = (6.0 * fxA + fxB + fxC) / 8.0;
      real fy = (6.0 * fyA + fyB + fyC) / 8.0;
      real fz = (6.0 * fzA + fzB + fzC) / 8.0;
      F[N[0] * 3 + i] += fx * n[0] + fy * n[1] + fz * n[2];
      fx = (fxA + 6.0 * fxB + fxC) / 8.0;
      fy = (fyA + 6.0 * fyB + fyC) / 8.0;
      fz = (fzA + 6.0 * fzB + fzC) / 8.0;
      F[N[1] * 3 + i] += fx * n[0] + fy * n[1] + fz * n[2];
      fx = (fxA + fxB + 6.0 * fxC) / 8.0;
      fy = (fyA + fyB + 6.0 * fyC) / 8.0;
      fz = (fzA + fzB + 6.0 * fzC) / 8.0;
      F[N[2] * 3 + i] += fx * n[0] + fy * n[1] + fz * n[2];
    }
  }
}

// adv_damp2 / adv_damp4 edge fluxes of the three velocity components
// (Chorin.cpp:640-709, 711-829), no transported scalars.
void cho_adv_edge(const ChoCG& s, const real* d, const real* U, const real* G, const real* P,
                  int64_t p, int64_t q, real f[3]) {
  real uL[3] = {U[p * 3 + 0], U[p * 3 + 1], U[p * 3 + 2]};
  real uR[3] = {U[q * 3 + 0], U[q * 3 + 1], U[q * 3 + 2]};
  if (s.damp4) {
    const real eps = 1.0e-9, k = 1.0 / 3.0;
    real dx = cx(s, q) - cx(s, p), dy = cy(s, q) - cy(s, p), dz = cz(s, q) - cz(s, p);
    for (int c = 0; c < 3; ++c) {
      real g1 = G[p * 9 + c * 3 + 0] * dx + G[p * 9 + c * 3 + 1] * dy + G[p * 9 + c * 3 + 2] * dz;
      real g2 = G[q * 9 + c * 3 + 0] * dx + G[q * 9 + c * 3 + 1] * dy + G[q * 9 + c * 3 + 2] * dz;
      real delta2 = uR[c] - uL[c];
      real delta1 = 2.0 * g1 - delta2;
      real delta3 = 2.0 * g2 - delta2;
      real rL = (delta2 + eps) / (delta1 + eps);
      real rR = (delta2 + eps) / (delta3 + eps);
      real rLinv = (delta1 + eps) / (delta2 + eps);
      real rRinv = (delta3 + eps) / (delta2 + eps);
      real phiL = (std::abs(rL) + rL) / (std::abs(rL) + 1.0);
      real phiR = (std::abs(rR) + rR) / (std::abs(rR) + 1.0);
      real phi_L_inv = (std::abs(rLinv) + rLinv) / (std::abs(rLinv) + 1.0);
      real phi_R_inv = (std::abs(rRinv) + rRinv) / (std::abs(rRinv) + 1.0);
      uL[c] += 0.25 * (delta1 * (1.0 - k) * phiL + delta2 * (1.0 + k) * phi_L_inv);
      uR[c] -= 0.25 * (delta3 * (1.0 - k) * phiR + delta2 * (1.0 + k) * phi_R_inv);
    }
  }
  const real nx = d[0], ny = d[1], nz = d[2];
  real vnL = uL[0] * nx + uL[1] * ny + uL[2] * nz;
  real vnR = uR[0] * nx + uR[1] * ny + uR[2] * nz;
  real aw = 0.0;
  if (s.stab) aw = std::abs(vnL + vnR) / 2.0;
  if (s.stab2) {
    real sl = std::abs(vnL), sr = std::abs(vnR);
    aw += s.stab2coef * std::max(sl, sr);
  }
  real v = d[4] * s.mu;
  real pf = P[p] + P[q];
  if (s.damp4) {
    f[0] = uL[0] * vnL + uR[0] * vnR + pf * nx + aw * (uR[0] - uL[0]) - v * (U[q * 3 + 0] - U[p * 3 + 0]);
    f[1] = uL[1] * vnL + uR[1] * vnR + pf * ny + aw * (uR[1] - uL[1]) - v * (U[q * 3 + 1] - U[p * 3 + 1]);
    f[2] = uL[2] * vnL + uR[2] * vnR + pf * nz + aw * (uR[2] - uL[2]) - v * (U[q * 3 + 2] - U[p * 3 + 2]);
  } else {
    f[0] = uL[0] * vnL + uR[0] * vnR + pf * nx + (aw - v) * (uR[0] - uL[0]);
    f[1] = uL[1] * vnL + uR[1] * vnR + pf * ny + (aw - v) * (uR[1] - uL[1]);
    f[2] = uL[2] * vnL + uR[2] * vnR + pf * nz + (aw - v) * (uR[2] - uL[2]);
  }
}

// chorin::rhs = adv (Chorin.cpp:831-982, 1010-1044); no source term.
void cho_rhs(const ChoCG& s, const real* U, const real* G, const real* P, real* R) {
  std::fill(R, R + s.n * 3, 0.0);
  for (int64_t e = 0; e < static_cast<int64_t>(s.edge.size() / 2); ++e) {
    const int64_t p = s.edge[2 * e], q = s.edge[2 * e + 1];
    real f[3];
    cho_adv_edge(s, &s.dint[5 * e], U, G, P, p, q, f);
    for (int c = 0; c < 3; ++c) {
      R[p * 3 + c] -= f[c];
      R[q * 3 + c] += f[c];
    }
  }
  for (int64_t e = 0; e < static_cast<int64_t>(s.tri.size() / 3); ++e) {
    const int64_t* N = &s.tri[e * 3];
    real n[3];
    cho_tri_normal(s, e, n);
    real f[3][3];
    for (int a = 0; a < 3; ++a) {
      real u = U[N[a] * 3 + 0], v = U[N[a] * 3 + 1], w = U[N[a] * 3 + 2], pp = P[N[a]];
      real vn = n[0] * u + n[1] * v + n[2] * w;
      f[0][a] = u * vn + pp * n[0];
      f[1][a] = v * vn + pp * n[1];
      f[2][a] = w * vn + pp * n[2];
    }
    for (int c = 0; c < 3; ++c) {
      R[N[0] * 3 + c] += (6.0 * f[c][0] + f[c][1] + f[c][2]) / 8.0;
      R[N[1] * 3 + c] += (f[c][0] + 6.0 * f[c][1] + f[c][2]) / 8.0;
      R[N[2] * 3 + c] += (f[c][0] + f[c][1] + 6.0 * f[c][2]) / 8.0;
    }
  }
}

// ChoCG::fingrad (src/Inciter/ChoCG.cpp:841-866): divide by the nodal volume.
void cho_fingrad(const ChoCG& s, real* G, int nprop) {
  for (int64_t p = 0; p < s.n; ++p)
    for (int c = 0; c < nprop; ++c) G[p * nprop + c] /= s.vol[p];
}

// physics::symbc on a 3-component field (src/Physics/BC.cpp:108-132).
void cho_symbc(const ChoCG& s, real* U) {
  for (size_t i = 0; i < s.symn.size(); ++i) {
    const int64_t p = s.symn[i];
    const real* nn = &s.symnorm[i * 3];
    real vn = U[p * 3 + 0] * nn[0] + U[p * 3 + 1] * nn[1] + U[p * 3 + 2] * nn[2];
    U[p * 3 + 0] -= vn * nn[0];
    U[p * 3 + 1] -= vn * nn[1];
    U[p * 3 + 2] -= vn * nn[2];
  }
}

// ChoCG::BC (src/Inciter/ChoCG.cpp:1333-1354): dirbc (time-independent
// values per node, src/Physics/BC.cpp:27-70), symbc, noslipbc (BC.cpp:134-145).
void cho_bc(ChoCG& s, real* U) {
  for (size_t i = 0; i < s.dirn.size(); ++i) {
    const int64_t p = s.dirn[i];
    for (int c = 0; c < 3; ++c)
      if (s.dirmask[i * 3 + c]) U[p * 3 + c] = s.dirval[i * 3 + c];
  }
  cho_symbc(s, U);
  for (int64_t p : s.noslip) U[p * 3 + 0] = U[p * 3 + 1] = U[p * 3 + 2] = 0.0;
}

// ChoCG::dt (src/Inciter/ChoCG.cpp:1356-1412), freezeflow 1, no scalars.
real cho_dt(const ChoCG& s) {
  const real eps = std::numeric_limits<real>::epsilon();
  if (std::abs(s.const_dt) > eps) return s.const_dt;
  real mindt = std::numeric_limits<real>::max();
  const real large = std::numeric_limits<real>::max();
  const real dif = s.mu;  // max(mu, diffusivity 0)
  for (int64_t i = 0; i < s.n; ++i) {
    real u = s.u[i * 3 + 0], v = s.u[i * 3 + 1], w = s.u[i * 3 + 2];
    real vel = std::sqrt(u * u + v * v + w * w);
    real L = std::cbrt(s.vol[i]);
    real euler_dt = L / std::max(vel, 1.0e-8);
    mindt = std::min(mindt, euler_dt);
    real dif_dt = dif > eps ? L * L / dif : large;
    mindt = std::min(mindt, dif_dt);
  }
  return mindt * s.cfl;
}

// Serial PCG of the pressure system (ConjugateGradients::init with apply =
// true, then solve; src/LinearSolver/ConjugateGradients.cpp:335-823): the
// Dirichlet rows and columns of a copy of A are eliminated in decreasing node
// order (CSR::dirichlet, src/LinearSolver/CSR.cpp:106-152), x warm-starts from
// the previous solution.
void cho_psolve(ChoCG& s, const real* b, const std::vector<real>& dval) {
  std::vector<real> a = s.A.a, bb(b, b + s.n);
  std::vector<int64_t> nodes = s.pdirn;
  orc_csr_dirichlet(s.n, s.A.ia.data(), s.A.ja.data(), a.data(), bb.data(),
                    static_cast<int64_t>(nodes.size()), nodes.data(), dval.data());
  int conv = 0;
  s.last_it = orc_pcg(s.n, s.A.ia.data(), s.A.ja.data(), a.data(), bb.data(), s.sol.data(),
                      s.pmaxit, s.ptol, s.pc, &s.last_normr, &s.last_normb, &conv);
  if (!conv) s.last_it = -s.last_it;  // reported, not an error (ConjugateGradients.cpp:792-806)
}

// The initial projection of ChoCG::merge -> div -> pinit -> psolve -> sgrad ->
// psolved (m_np = 0), then velgrad -> flux -> div -> pinit -> psolve ->
// psolved (m_np = 1) and pgrad (src/Inciter/ChoCG.cpp:739-764, 868-1281).
void cho_init(ChoCG& s) {
  const int64_t n = s.n;
  s.np = 0;
  cho_bc(s, s.u.data());
  // m_np = 0: divergence of u without stabilisation, Dirichlet values as set
  std::fill(s.div.begin(), s.div.end(), 0.0);
  cho_div(s, s.u.data(), s.pr.data(), s.pgrad.data(), s.dt, false, s.div.data());
  cho_psolve(s, s.div.data(), s.pdirval);
  std::fill(s.sgrad.begin(), s.sgrad.end(), 0.0);
  cho_vgrad(s, s.sol.data(), 1, s.sgrad.data());
  cho_fingrad(s, s.sgrad.data(), 3);
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) s.u[i * 3 + c] -= 1.0 * s.sgrad[i * 3 + c];
  cho_bc(s, s.u.data());
  // m_np = 1: momentum flux of the projected field as the Poisson rhs
  s.np = 1;
  std::fill(s.vgrad.begin(), s.vgrad.end(), 0.0);
  cho_vgrad(s, s.u.data(), 3, s.vgrad.data());
  cho_fingrad(s, s.vgrad.data(), 9);
  std::fill(s.flx.begin(), s.flx.end(), 0.0);
  cho_flux(s, s.u.data(), s.vgrad.data(), s.flx.data());
  cho_fingrad(s, s.flx.data(), 3);
  cho_symbc(s, s.flx.data());
  std::fill(s.div.begin(), s.div.end(), 0.0);
  cho_div(s, s.flx.data(), s.pr.data(), s.pgrad.data(), s.dt, false, s.div.data());
  cho_psolve(s, s.div.data(), s.pdirval);
  // m_np = 2: initial pressure and its gradient
  s.np = 2;
  s.pr = s.sol;
  std::fill(s.pgrad.begin(), s.pgrad.end(), 0.0);
  cho_vgrad(s, s.pr.data(), 1, s.pgrad.data());
  cho_fingrad(s, s.pgrad.data(), 3);
}

// One time step: dt -> rk stages of rhs/solve/pred(BC, damp4 vgrad) -> div
// (stabilised) / dt -> pressure-increment solve (Dirichlet values 0) ->
// sgrad -> projection and BC -> pressure update and pgrad -> t += dt
// (src/Inciter/ChoCG.cpp:1356-1695, 868-1281).
// The semi-implicit last stage (ChoCG::lhs, src/Inciter/ChoCG.cpp:1433-1477,
// then ChoCG::solve's implicit branch 1576-1606 and msolved 1626-1645): A is
// assembled per element, A(a,b,c) -= J/dt/120 (2 or 1) + theta mu
// grad_a.grad_b/J/6, the velocity Dirichlet components and noslip nodes are
// zero rows (CSR::dirichlet with value 0), the PCG starts from the previous
// increment, and u = un + du.
void cho_momentum(ChoCG& s) {
  const int64_t n = s.n, n3 = 3 * n;
  std::vector<real> a(s.mja.size(), 0.0), b(s.rhs);
  auto pos = [&](int64_t r, int64_t col) {
    return static_cast<int64_t>(
        std::lower_bound(s.mja.begin() + s.mia[r], s.mja.begin() + s.mia[r + 1], col) -
        s.mja.begin());
  };
  for (int64_t e = 0; e < static_cast<int64_t>(s.inpoel.size() / 4); ++e) {
    const int64_t* N = &s.inpoel[e * 4];
    const real ba[3] = {cx(s, N[1]) - cx(s, N[0]), cy(s, N[1]) - cy(s, N[0]),
                        cz(s, N[1]) - cz(s, N[0])};
    const real ca[3] = {cx(s, N[2]) - cx(s, N[0]), cy(s, N[2]) - cy(s, N[0]),
                        cz(s, N[2]) - cz(s, N[0])};
    const real da[3] = {cx(s, N[3]) - cx(s, N[0]), cy(s, N[3]) - cy(s, N[0]),
                        cz(s, N[3]) - cz(s, N[0])};
    real g[4][3];
    cross(ca[0], ca[1], ca[2], da[0], da[1], da[2], g[1][0], g[1][1], g[1][2]);
    cross(da[0], da[1], da[2], ba[0], ba[1], ba[2], g[2][0], g[2][1], g[2][2]);
    cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], g[3][0], g[3][1], g[3][2]);
    for (int k = 0; k < 3; ++k) g[0][k] = -g[1][k] - g[2][k] - g[3][k];
    const real J = ba[0] * g[1][0] + ba[1] * g[1][1] + ba[2] * g[1][2];
    for (int p = 0; p < 4; ++p)
      for (int q = 0; q < 4; ++q) {
        real v = J / s.dt / 120.0 * ((p == q) ? 2.0 : 1.0);
        v += s.theta * s.mu * (g[p][0] * g[q][0] + g[p][1] * g[q][1] + g[p][2] * g[q][2]) / J / 6.0;
        for (int c = 0; c < 3; ++c) a[pos(N[p] * 3 + c, N[q] * 3 + c)] -= v;
      }
  }
  std::vector<uint8_t> mask(n3, 0);
  for (size_t k = 0; k < s.dirn.size(); ++k)
    for (int c = 0; c < 3; ++c)
      if (s.dirmask[k * 3 + c]) mask[s.dirn[k] * 3 + c] = 1;
  for (int64_t p : s.noslip)
    for (int c = 0; c < 3; ++c) mask[p * 3 + c] = 1;
  std::vector<int64_t> rows;
  for (int64_t r = n3 - 1; r >= 0; --r)
    if (mask[r]) rows.push_back(r);
  std::vector<real> zero(rows.size(), 0.0);
  orc_csr_dirichlet(n3, s.mia.data(), s.mja.data(), a.data(), b.data(),
                    static_cast<int64_t>(rows.size()), rows.data(), zero.data());
  real nr = 0, nb = 0;
  int conv = 0;
  s.last_mit = orc_pcg(n3, s.mia.data(), s.mja.data(), a.data(), b.data(), s.momx.data(),
                       s.mom_iter, s.mom_tol, s.mom_pc, &nr, &nb, &conv);
  if (!conv) s.last_mit = -s.last_mit;
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) s.u[i * 3 + c] = s.un[i * 3 + c] + s.momx[i * 3 + c];
}

real cho_step(ChoCG& s) {
  static const real rkc[4][4] = {{1.0, 0, 0, 0},
                                 {1.0 / 2.0, 1.0, 0, 0},
                                 {1.0 / 3.0, 1.0 / 2.0, 1.0, 0},
                                 {1.0 / 4.0, 1.0 / 3.0, 1.0 / 2.0, 1.0}};
  const int64_t n = s.n;
  s.dt = cho_dt(s);
  for (int st = 0; st < s.rk; ++st) {
    cho_rhs(s, s.u.data(), s.vgrad.data(), s.pr.data(), s.rhs.data());
    if (st == 0) s.un = s.u;
    if (s.theta > std::numeric_limits<real>::epsilon() && st + 1 == s.rk) {
      cho_momentum(s);
    } else {
      const real dtk = rkc[s.rk - 1][st] * s.dt;
      for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c)
          s.u[i * 3 + c] = s.un[i * 3 + c] - dtk * s.rhs[i * 3 + c] / s.vol[i];
    }
    cho_bc(s, s.u.data());
    if (s.damp4) {
      std::fill(s.vgrad.begin(), s.vgrad.end(), 0.0);
      cho_vgrad(s, s.u.data(), 3, s.vgrad.data());
      cho_fingrad(s, s.vgrad.data(), 9);
    }
  }
  std::fill(s.div.begin(), s.div.end(), 0.0);
  cho_div(s, s.u.data(), s.pr.data(), s.pgrad.data(), s.dt, true, s.div.data());
  for (auto& d : s.div) d /= s.dt;
  std::vector<real> zero(s.pdirn.size(), 0.0);
  cho_psolve(s, s.div.data(), zero);
  std::fill(s.sgrad.begin(), s.sgrad.end(), 0.0);
  cho_vgrad(s, s.sol.data(), 1, s.sgrad.data());
  cho_fingrad(s, s.sgrad.data(), 3);
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) s.u[i * 3 + c] -= s.dt * s.sgrad[i * 3 + c];
  cho_bc(s, s.u.data());
  for (int64_t i = 0; i < n; ++i) s.pr[i] += s.sol[i];
  std::fill(s.pgrad.begin(), s.pgrad.end(), 0.0);
  cho_vgrad(s, s.pr.data(), 1, s.pgrad.data());
  cho_fingrad(s, s.pgrad.data(), 3);
  s.t += s.dt;
  return s.dt;
}

}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

// ---------------------------------------------------------------- mesh setup

// Nodal volumes, sum of J/24 over tets (src/Inciter/Discretization.cpp:619-660).
// Returns the number of elements with a non-positive Jacobian (the reference
// raises an error for those, Discretization.cpp:636).
int64_t orc_vol(int64_t npoin, const double* xyz, int64_t nelem, const int64_t* inpoel,
                double* vol) {
  const real *x = xyz, *y = xyz + npoin, *z = xyz + 2 * npoin;
  std::fill(vol, vol + npoin, 0.0);
  int64_t bad = 0;
  for (int64_t e = 0; e < nelem; ++e) {
    const int64_t* N = &inpoel[e * 4];
    real ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
    real ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
    real da[3] = {x[N[3]] - x[N[0]], y[N[3]] - y[N[0]], z[N[3]] - z[N[0]]};
    real J = triple(ba, ca, da) / 24.0;
    if (!(J > 0)) ++bad;
    for (int j = 0; j < 4; ++j) vol[N[j]] += J;
  }
  return bad;
}

// Domain edge integrals (src/Inciter/RieCG.cpp:339-382): for each unique
// edge keyed by (smaller, larger) global id, D = sum sig*(grad_p-grad_q)/48.
// With ncoef == 5 the two ChoCG extras are appended per edge
// (src/Inciter/ChoCG.cpp:398-445): J/120 and grad_p.grad_q/J/6 summed over
// the tets sharing the edge.  Returns the number of edges; fills the outputs
// only when cap >= that number.  gid may be null (identity).
int64_t orc_domint(int64_t npoin, const double* xyz, int64_t nelem, const int64_t* inpoel,
                   const int64_t* gid, int ncoef, int64_t cap, int64_t* edge, double* dedge) {
  const real *x = xyz, *y = xyz + npoin, *z = xyz + 2 * npoin;
  std::map<std::pair<int64_t, int64_t>, std::array<real, 5>> m;
  std::vector<int64_t> lid;
  for (int64_t e = 0; e < nelem; ++e) {
    const int64_t* N = &inpoel[e * 4];
    Tet g = tetgeo(x, y, z, N);
    for (int k = 0; k < 6; ++k) {
      int p = lpoed[k][0], q = lpoed[k][1];
      int64_t gp = gid ? gid[N[p]] : N[p];
      int64_t gq = gid ? gid[N[q]] : N[q];
      real sig = 1.0;
      std::pair<int64_t, int64_t> key{gp, gq};
      if (key.first > key.second) {
        std::swap(key.first, key.second);
        sig = -1.0;
      }
      auto& n = m[key];
      n[0] += sig * (g.grad[p][0] - g.grad[q][0]) / 48.0;
      n[1] += sig * (g.grad[p][1] - g.grad[q][1]) / 48.0;
      n[2] += sig * (g.grad[p][2] - g.grad[q][2]) / 48.0;
      if (ncoef == 5) {
        n[3] += g.J / 120.0;
        n[4] += (g.grad[p][0] * g.grad[q][0] + g.grad[p][1] * g.grad[q][1] +
                 g.grad[p][2] * g.grad[q][2]) / g.J / 6.0;
      }
    }
  }
  int64_t ne = static_cast<int64_t>(m.size());
  if (cap < ne) return ne;
  // global -> local ids for the output
  std::map<int64_t, int64_t> g2l;
  if (gid)
    for (int64_t i = 0; i < npoin; ++i) g2l[gid[i]] = i;
  int64_t k = 0;
  for (const auto& [key, d] : m) {
    edge[k * 2 + 0] = gid ? g2l[key.first] : key.first;
    edge[k * 2 + 1] = gid ? g2l[key.second] : key.second;
    for (int c = 0; c < ncoef; ++c) dedge[k * ncoef + c] = d[c];
    ++k;
  }
  return ne;
}

// Boundary point normals for one side set (src/Inciter/RieCG.cpp:281-337,
// 483-525): inverse-distance-squared weighted unit face normals, divided by
// the weight sum.  Writes one normal per node of nodes[] (which must all lie
// on faces of this set) in the same order.
int orc_bnorm(int64_t npoin, const double* xyz, int64_t nface, const int64_t* faces,
              int64_t nnode, const int64_t* nodes, double* norms) {
  const real *x = xyz, *y = xyz + npoin, *z = xyz + 2 * npoin;
  std::map<int64_t, std::array<real, 4>> b;
  for (int64_t f = 0; f < nface; ++f) {
    const int64_t* N = &faces[f * 3];
    real ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
    real ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
    real n[3];
    cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], n[0], n[1], n[2]);
    real A2 = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= A2;
    n[1] /= A2;
    n[2] /= A2;
    real c[3] = {(x[N[0]] + x[N[1]] + x[N[2]]) / 3.0, (y[N[0]] + y[N[1]] + y[N[2]]) / 3.0,
                 (z[N[0]] + z[N[1]] + z[N[2]]) / 3.0};
    for (int i = 0; i < 3; ++i) {
      int64_t p = N[i];
      real r = 1.0 / ((c[0] - x[p]) * (c[0] - x[p]) + (c[1] - y[p]) * (c[1] - y[p]) +
                      (c[2] - z[p]) * (c[2] - z[p]));
      auto& v = b[p];
      v[0] += r * n[0];
      v[1] += r * n[1];
      v[2] += r * n[2];
      v[3] += r;
    }
  }
  for (int64_t i = 0; i < nnode; ++i) {
    auto it = b.find(nodes[i]);
    if (it == b.end()) {
      g_err = "node not on side set";
      return 1;
    }
    for (int j = 0; j < 3; ++j) norms[i * 3 + j] = it->second[j] / it->second[3];
  }
  return 0;
}

// ---------------------------------------------------------------- RieCG

void* orc_riecg_create(int64_t npoin, const double* xyz, const double* vol, int64_t nedge,
                       const int64_t* edge, const double* dedge, int64_t ntri,
                       const int64_t* tri, const uint8_t* besym, double gamma, int flux,
                       int stab2, double stab2coef, double cfl, double const_dt) {
  auto* s = new RieCG;
  s->npoin = npoin;
  s->x.assign(xyz, xyz + npoin);
  s->y.assign(xyz + npoin, xyz + 2 * npoin);
  s->z.assign(xyz + 2 * npoin, xyz + 3 * npoin);
  s->vol.assign(vol, vol + npoin);
  s->edge.assign(edge, edge + nedge * 2);
  s->dedge.assign(dedge, dedge + nedge * 3);
  s->tri.assign(tri, tri + ntri * 3);
  s->besym.assign(besym, besym + ntri * 3);
  s->gamma = gamma;
  s->flux = flux;
  s->stab2 = stab2;
  s->stab2coef = stab2coef;
  s->cfl = cfl;
  s->const_dt = const_dt;
  s->U.assign(npoin * 5, 0.0);
  s->Un = s->U;
  s->R = s->U;
  s->G.assign(npoin * 15, 0.0);
  return s;
}

void orc_riecg_destroy(void* h) { delete static_cast<RieCG*>(h); }

void orc_riecg_set_sym(void* h, int64_t n, const int64_t* nodes, const double* norms) {
  auto* s = static_cast<RieCG*>(h);
  s->symnode.assign(nodes, nodes + n);
  s->symnorm.assign(norms, norms + n * 3);
}

void orc_riecg_set_far(void* h, int64_t n, const int64_t* nodes, const double* norms,
                       double r, double u, double v, double w, double p) {
  auto* s = static_cast<RieCG*>(h);
  s->farnode.assign(nodes, nodes + n);
  s->farnorm.assign(norms, norms + n * 3);
  s->far_r = r;
  s->far_u[0] = u;
  s->far_u[1] = v;
  s->far_u[2] = w;
  s->far_p = p;
}

void orc_riecg_set_dir(void* h, int64_t n, const int64_t* nodes, const int32_t* mask,
                       const double* vals) {
  auto* s = static_cast<RieCG*>(h);
  s->dirnode.assign(nodes, nodes + n);
  s->dirmask.assign(mask, mask + n * 5);
  s->dirval.assign(vals, vals + n * 5);
}

void orc_riecg_set_pre(void* h, int64_t n, const int64_t* nodes, const double* vals) {
  auto* s = static_cast<RieCG*>(h);
  s->prenode.assign(nodes, nodes + n);
  s->preval.assign(vals, vals + n * 2);
}

void orc_riecg_set_state(void* h, const double* U, double t) {
  auto* s = static_cast<RieCG*>(h);
  s->U.assign(U, U + s->npoin * 5);
  s->t = t;
}

void orc_riecg_get_state(void* h, double* U) {
  auto* s = static_cast<RieCG*>(h);
  std::memcpy(U, s->U.data(), sizeof(real) * s->U.size());
}

// Raw weak gradient (not divided by volume), like riemann::grad.
void orc_riecg_grad(void* h, const double* U, double* G) {
  riecg_grad(*static_cast<RieCG*>(h), U, G);
}

// Right-hand side from volume-divided gradients, like riemann::rhs.
void orc_riecg_rhs(void* h, const double* G, const double* U, double* R) {
  riecg_rhs(*static_cast<RieCG*>(h), G, U, R);
}

// The manufactured source of riemann::rhs: problem (0 none, 1 taylor_green,
// 2 vortical_flow, 3 nonlinear_energy_growth, 4 rayleigh_taylor) and its
// parameters alpha, beta[3], kappa, r0, p0, ce (prm may be null).
void orc_riecg_set_source(void* h, int problem, const double* prm) {
  auto* s = static_cast<RieCG*>(h);
  s->src = problem;
  for (int k = 0; k < 8; ++k) s->sprm[k] = prm ? prm[k] : 0.0;
}

void orc_riecg_bc(void* h) {
  auto* s = static_cast<RieCG*>(h);
  riecg_bc(*s, s->U.data(), s->t);
}

double orc_riecg_dt(void* h) {
  auto* s = static_cast<RieCG*>(h);
  return riecg_dt(*s, s->U.data());
}

// Advance nstep full time steps (dt -> 3 stages each); returns the last dt and
// writes the per-step dt history if dts is non-null.
double orc_riecg_run(void* h, int64_t nstep, double* dts) {
  auto* s = static_cast<RieCG*>(h);
  for (int64_t k = 0; k < nstep; ++k) {
    s->dt = riecg_dt(*s, s->U.data());
    if (dts) dts[k] = s->dt;
    for (int st = 0; st < 3; ++st) riecg_stage(*s, st);
    s->t += s->dt;
    ++s->it;
  }
  return s->dt;
}

// Single stage with a given dt (for stage-level parity tests).
// One stage of the given dt; the last stage completes the step and advances
// the time.
void orc_riecg_stage(void* h, int stage, double dt) {
  auto* s = static_cast<RieCG*>(h);
  s->dt = dt;
  riecg_stage(*s, stage);
  if (stage == 2) {
    s->t += dt;
    ++s->it;
  }
}

// ---------------------------------------------------------------- KozCG

void* orc_kozcg_create(int64_t npoin, const double* xyz, const double* vol, int64_t nelem,
                       const int64_t* inpoel, double gamma, double cfl, double const_dt,
                       int fct, double ctau, int fctclip, int nsys, const int32_t* sys) {
  auto* s = new KozCG;
  s->npoin = npoin;
  s->nelem = nelem;
  s->x.assign(xyz, xyz + npoin);
  s->y.assign(xyz + npoin, xyz + 2 * npoin);
  s->z.assign(xyz + 2 * npoin, xyz + 3 * npoin);
  s->vol.assign(vol, vol + npoin);
  s->inpoel.assign(inpoel, inpoel + nelem * 4);
  s->gamma = gamma;
  s->cfl = cfl;
  s->const_dt = const_dt;
  s->fct = fct;
  s->ctau = ctau;
  s->fctclip = fctclip;
  s->fctsys.assign(sys, sys + nsys);
  s->U.assign(npoin * 5, 0.0);
  s->R = s->U;
  s->A = s->U;
  s->P.assign(npoin * 10, 0.0);
  s->Q = s->P;
  return s;
}

void orc_kozcg_destroy(void* h) { delete static_cast<KozCG*>(h); }

void orc_kozcg_set_sym(void* h, int64_t n, const int64_t* nodes, const double* norms) {
  auto* s = static_cast<KozCG*>(h);
  s->symnode.assign(nodes, nodes + n);
  s->symnorm.assign(norms, norms + n * 3);
}

void orc_kozcg_set_dir(void* h, int64_t n, const int64_t* nodes, const int32_t* mask,
                       const double* vals) {
  auto* s = static_cast<KozCG*>(h);
  s->dirnode.assign(nodes, nodes + n);
  s->dirmask.assign(mask, mask + n * 5);
  s->dirval.assign(vals, vals + n * 5);
}

void orc_kozcg_set_state(void* h, const double* U, double t) {
  auto* s = static_cast<KozCG*>(h);
  s->U.assign(U, U + s->npoin * 5);
  s->t = t;
}

void orc_kozcg_set_source(void* h, int problem, const double* prm) {
  auto* s = static_cast<KozCG*>(h);
  s->src = problem;
  for (int k = 0; k < 8; ++k) s->sprm[k] = prm ? prm[k] : 0.0;
}

// One step of the given dt (Discretization::setdt's cut last step).
void orc_kozcg_step(void* h, double dt) {
  auto* s = static_cast<KozCG*>(h);
  s->dt = dt;
  kozcg_step(*s);
  s->t += s->dt;
  ++s->it;
}

double orc_kozcg_dt(void* h) { return kozcg_dt(*static_cast<KozCG*>(h)); }

void orc_kozcg_get_state(void* h, double* U) {
  auto* s = static_cast<KozCG*>(h);
  std::memcpy(U, s->U.data(), sizeof(real) * s->U.size());
}

void orc_kozcg_rhs(void* h, const double* U, double dt, double* R) {
  const auto* s = static_cast<KozCG*>(h);
  kozak_rhs(*s, U, s->t, dt, R);
}

double orc_kozcg_run(void* h, int64_t nstep, double* dts) {
  auto* s = static_cast<KozCG*>(h);
  for (int64_t k = 0; k < nstep; ++k) {
    s->dt = kozcg_dt(*s);
    if (dts) dts[k] = s->dt;
    kozcg_step(*s);
    s->t += s->dt;
    ++s->it;
  }
  return s->dt;
}

// ---------------------------------------------------------------- CSR / PCG

// The pressure Laplacian of ChoCG::prelhs (src/Inciter/ChoCG.cpp:146-188):
// A(a,b) -= grad_a.grad_b / (6J) over tets, on the sparsity of points
// surrounding points plus the diagonal.  Zero-based rows sorted by column.
// Returns nnz; fills only when cap >= nnz.
int64_t orc_pressure_matrix(int64_t npoin, const double* xyz, int64_t nelem,
                            const int64_t* inpoel, int64_t cap, int64_t* ia, int64_t* ja,
                            double* a) {
  const real *x = xyz, *y = xyz + npoin, *z = xyz + 2 * npoin;
  std::vector<std::set<int64_t>> rows(static_cast<size_t>(npoin));
  for (int64_t e = 0; e < nelem; ++e)
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) rows[inpoel[e * 4 + i]].insert(inpoel[e * 4 + j]);
  int64_t nnz = 0;
  for (auto& r : rows) nnz += static_cast<int64_t>(r.size());
  if (cap < nnz) return nnz;
  ia[0] = 0;
  int64_t k = 0;
  for (int64_t i = 0; i < npoin; ++i) {
    for (auto c : rows[i]) {
      ja[k] = c;
      a[k] = 0.0;
      ++k;
    }
    ia[i + 1] = k;
  }
  for (int64_t e = 0; e < nelem; ++e) {
    const int64_t* N = &inpoel[e * 4];
    Tet g = tetgeo(x, y, z, N);
    real J = g.J * 6.0;
    for (int aa = 0; aa < 4; ++aa)
      for (int b = 0; b < 4; ++b) {
        int64_t r = N[aa], c = N[b];
        auto* beg = ja + ia[r];
        auto* pos = std::lower_bound(beg, ja + ia[r + 1], c);
        a[pos - ja] -= (g.grad[aa][0] * g.grad[b][0] + g.grad[aa][1] * g.grad[b][1] +
                        g.grad[aa][2] * g.grad[b][2]) / J;
      }
  }
  return nnz;
}

// Symmetric Dirichlet elimination as ConjugateGradients::apply + r
// (src/LinearSolver/ConjugateGradients.cpp:450-556) with CSR::dirichlet
// (src/LinearSolver/CSR.cpp:106-152), serial (diagonal 1): nodes processed in
// decreasing id order; b becomes b - (column contributions), then BC values.
void orc_csr_dirichlet(int64_t n, const int64_t* ia, const int64_t* ja, double* a, double* b,
                       int64_t ndir, const int64_t* nodes, const double* vals) {
  std::vector<std::pair<int64_t, real>> bc;
  for (int64_t k = 0; k < ndir; ++k) bc.emplace_back(nodes[k], vals[k]);
  std::sort(bc.begin(), bc.end());
  std::vector<real> r(static_cast<size_t>(n), 0.0);
  for (auto it = bc.rbegin(); it != bc.rend(); ++it) {
    int64_t i = it->first;
    real val = it->second;
    for (int64_t row = 0; row < n; ++row)
      for (int64_t j = ia[row]; j < ia[row + 1]; ++j)
        if (ja[j] == i) {
          r[row] += a[j] * val;
          a[j] = 0.0;
          break;
        }
    for (int64_t j = ia[i]; j < ia[i + 1]; ++j) a[j] = (ja[j] == i) ? 1.0 : 0.0;
  }
  for (int64_t i = 0; i < n; ++i) b[i] -= r[i];
  for (auto& [i, val] : bc) b[i] = val;
}

// Serial PCG exactly as ConjugateGradients::setup/initres/next/qAp/q/pq/rz/x
// (src/LinearSolver/ConjugateGradients.cpp:105-823) with an empty node
// communication map: pc 0 = "none" (d = 1), 1 = "jacobi" (d = diag A).
// Returns the iteration count; writes the final residual norm and ||b||.
int64_t orc_pcg(int64_t n, const int64_t* ia, const int64_t* ja, const double* a,
                const double* b, double* x, int64_t maxit, double tol, int pc,
                double* normr_out, double* normb_out, int* converged) {
  CG A;
  A.n = n;
  A.ia.assign(ia, ia + n + 1);
  A.ja.assign(ja, ja + ia[n]);
  A.a.assign(a, a + ia[n]);
  std::vector<real> r(n), p(n), q(n), z(n), d(n);
  csr_mult(A, x, r.data());
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
  p = r;
  for (int64_t i = 0; i < n; ++i) {
    if (pc == 1) {
      real dv = 0;
      for (int64_t j = ia[i]; j < ia[i + 1]; ++j)
        if (ja[j] == i) dv = a[j];
      d[i] = dv;
    } else {
      d[i] = 1.0;
    }
  }
  real normb = 0;
  for (int64_t i = 0; i < n; ++i) normb += b[i] * b[i];
  normb = std::sqrt(normb);
  for (int64_t i = 0; i < n; ++i) z[i] = r[i] / d[i];
  real rho = 0;
  for (int64_t i = 0; i < n; ++i) rho += r[i] * z[i];
  real rho0 = 0, alpha = 0, normr2 = 0;
  int64_t it = 0;
  bool finished = false;
  const real eps = std::numeric_limits<real>::epsilon();
  while (true) {
    // next
    alpha = (it == 0) ? 0.0 : rho / rho0;
    rho0 = rho;
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + alpha * p[i];
    // qAp, q
    csr_mult(A, p.data(), q.data());
    real pq = 0;
    for (int64_t i = 0; i < n; ++i) pq += p[i] * q[i];
    // pq
    if (std::abs(pq) < eps) {
      finished = true;
      alpha = 0.0;
    } else {
      alpha = rho / pq;
    }
    for (int64_t i = 0; i < n; ++i) r[i] -= alpha * q[i];
    for (int64_t i = 0; i < n; ++i) z[i] = r[i] / d[i];
    real rz = 0, rr = 0;
    for (int64_t i = 0; i < n; ++i) rz += r[i] * z[i];
    for (int64_t i = 0; i < n; ++i) rr += r[i] * r[i];
    normr2 = rr;
    // rz
    rho = rz;
    for (int64_t i = 0; i < n; ++i) x[i] += alpha * p[i];
    // x
    ++it;
    real nb = normb > 1.0e-14 ? normb : 1.0;
    real nr = std::sqrt(normr2);
    if (finished || nr < tol * nb || it >= maxit) {
      *converged = nr > tol * nb ? 0 : 1;
      *normr_out = nr;
      *normb_out = normb;
      break;
    }
  }
  return it;
}

void orc_csr_mult(int64_t n, const int64_t* ia, const int64_t* ja, const double* a,
                  const double* x, double* r) {
  CG A;
  A.n = n;
  A.ia.assign(ia, ia + n + 1);
  A.ja.assign(ja, ja + ia[n]);
  A.a.assign(a, a + ia[n]);
  csr_mult(A, x, r);
}

}  // extern "C"

// ---------------------------------------------------------------- ChoCG

extern "C" {

// ChoCG state over plain edges (2 ids + 5 integrals each), boundary triangles
// and the zero-based pressure matrix of ChoCG::prelhs.  flux: 0 damp2,
// 1 damp4; pc: 0 none, 1 jacobi.
void* orc_chocg_create(int64_t npoin, const double* xyz, const double* vol, int64_t nedge,
                       const int64_t* edges, const double* dint, int64_t ntri, const int64_t* tri,
                       const int64_t* ia, const int64_t* ja, const double* a, double mu,
                       double cfl, double const_dt, int damp4, int stab, int stab2,
                       double stab2coef, int rk, int pc, double ptol, int64_t pmaxit) {
  auto* s = new ChoCG;
  s->n = npoin;
  s->xyz.assign(xyz, xyz + 3 * npoin);
  s->vol.assign(vol, vol + npoin);
  s->edge.assign(edges, edges + 2 * nedge);
  s->dint.assign(dint, dint + 5 * nedge);
  s->tri.assign(tri, tri + 3 * ntri);
  s->A.n = npoin;
  s->A.ia.assign(ia, ia + npoin + 1);
  s->A.ja.assign(ja, ja + ia[npoin]);
  s->A.a.assign(a, a + ia[npoin]);
  s->mu = mu;
  s->cfl = cfl;
  s->const_dt = const_dt;
  s->damp4 = damp4;
  s->stab = stab;
  s->stab2 = stab2;
  s->stab2coef = stab2coef;
  s->rk = rk;
  s->pc = pc;
  s->ptol = ptol;
  s->pmaxit = pmaxit;
  const size_t n = static_cast<size_t>(npoin);
  s->u.assign(3 * n, 0.0);
  s->un.assign(3 * n, 0.0);
  s->pr.assign(n, 0.0);
  s->pgrad.assign(3 * n, 0.0);
  s->vgrad.assign(9 * n, 0.0);
  s->flx.assign(3 * n, 0.0);
  s->div.assign(n, 0.0);
  s->sgrad.assign(3 * n, 0.0);
  s->rhs.assign(3 * n, 0.0);
  s->sol.assign(n, 0.0);
  return s;
}

void orc_chocg_destroy(void* h) { delete static_cast<ChoCG*>(h); }

void orc_chocg_set_bc(void* h, int64_t ndir, const int64_t* dirn, const int32_t* dirmask,
                      const double* dirval, int64_t nsym, const int64_t* symn,
                      const double* symnorm, int64_t nnoslip, const int64_t* noslip,
                      int64_t npdir, const int64_t* pdirn, const double* pdirval) {
  auto* s = static_cast<ChoCG*>(h);
  s->dirn.assign(dirn, dirn + ndir);
  s->dirmask.assign(dirmask, dirmask + 3 * ndir);
  s->dirval.assign(dirval, dirval + 3 * ndir);
  s->symn.assign(symn, symn + nsym);
  s->symnorm.assign(symnorm, symnorm + 3 * nsym);
  s->noslip.assign(noslip, noslip + nnoslip);
  s->pdirn.assign(pdirn, pdirn + npdir);
  s->pdirval.assign(pdirval, pdirval + npdir);
}

void orc_chocg_set_state(void* h, const double* u, const double* p, double t) {
  auto* s = static_cast<ChoCG*>(h);
  s->u.assign(u, u + 3 * s->n);
  if (p) s->pr.assign(p, p + s->n);
  s->t = t;
}

// what: 0 u (n x 3), 1 un, 2 pressure, 3 pressure gradient (n x 3),
// 4 velocity gradient (n x 9), 5 divergence (n), 6 last pressure solution (n).
void orc_chocg_get(void* h, int what, double* out) {
  auto* s = static_cast<ChoCG*>(h);
  const std::vector<real>* v = nullptr;
  switch (what) {
    case 0: v = &s->u; break;
    case 1: v = &s->un; break;
    case 2: v = &s->pr; break;
    case 3: v = &s->pgrad; break;
    case 4: v = &s->vgrad; break;
    case 5: v = &s->div; break;
    default: v = &s->sol; break;
  }
  std::memcpy(out, v->data(), v->size() * sizeof(double));
}

// Initial projection and pressure; returns the iterations of the last solve.
int64_t orc_chocg_init(void* h) {
  auto* s = static_cast<ChoCG*>(h);
  cho_init(*s);
  return s->last_it;
}

// One time step; returns dt and writes the pressure-solve iterations.
// theta-implicit momentum prediction: tetrahedra (4 ids each) and the
// momentum solver's settings; the pattern: nodes sharing a tetrahedron and
// the diagonal, 3 rows per node
void orc_chocg_set_theta(void* h, double theta, int64_t ntet, const int64_t* inpoel, int mom_pc,
                         int64_t mom_iter, double mom_tol) {
  auto* s = static_cast<ChoCG*>(h);
  s->theta = theta;
  s->inpoel.assign(inpoel, inpoel + ntet * 4);
  s->mom_pc = mom_pc;
  s->mom_iter = mom_iter;
  s->mom_tol = mom_tol;
  const int64_t n = s->n;
  std::vector<std::vector<int64_t>> nb(n);
  for (int64_t e = 0; e < ntet; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) nb[inpoel[e * 4 + a]].push_back(inpoel[e * 4 + b]);
  s->mia.assign(3 * n + 1, 0);
  s->mja.clear();
  for (int64_t i = 0; i < n; ++i) {
    auto& v = nb[i];
    v.push_back(i);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    for (int c = 0; c < 3; ++c) {
      for (int64_t j : v) s->mja.push_back(j * 3 + c);
      s->mia[i * 3 + c + 1] = static_cast<int64_t>(s->mja.size());
    }
  }
  s->momx.assign(3 * n, 0.0);
}

int64_t orc_chocg_momentum_its(void* h) { return static_cast<ChoCG*>(h)->last_mit; }

double orc_chocg_step(void* h, int64_t* it) {
  auto* s = static_cast<ChoCG*>(h);
  double dt = cho_step(*s);
  if (it) *it = s->last_it;
  return dt;
}

// Single chorin:: passes on caller arrays (for pinning and drop-in parity):
// raw weak results, nothing divided by the volume.
void orc_chocg_div(void* h, const double* U, const double* P, const double* G, double dt,
                   int stab, double* D) {
  auto* s = static_cast<ChoCG*>(h);
  std::fill(D, D + s->n, 0.0);
  cho_div(*s, U, P, G, dt, stab != 0, D);
}
void orc_chocg_vgrad(void* h, const double* U, int ncomp, double* G) {
  auto* s = static_cast<ChoCG*>(h);
  std::fill(G, G + s->n * ncomp * 3, 0.0);
  cho_vgrad(*s, U, ncomp, G);
}
void orc_chocg_flux(void* h, const double* U, const double* G, double* F) {
  auto* s = static_cast<ChoCG*>(h);
  std::fill(F, F + s->n * 3, 0.0);
  cho_flux(*s, U, G, F);
}
void orc_chocg_rhs(void* h, const double* U, const double* G, const double* P, double* R) {
  auto* s = static_cast<ChoCG*>(h);
  cho_rhs(*s, U, G, P, R);
}

}  // extern "C"
