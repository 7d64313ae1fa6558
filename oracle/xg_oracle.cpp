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

// riemann::rhs = advdom + advbnd (src/Physics/Riemann.cpp:652-878, 909-946);
// the manufactured source term is off for the configured problems.
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
}

// RieCG::BC (src/Inciter/RieCG.cpp:764-785) -> physics::dirbc, symbc, farbc,
// prebc (src/Physics/BC.cpp:29-72, 110-136, 152-220, 222-241).  Dirichlet
// values are given per node (time independent).
void riecg_bc(RieCG& s, real* U) {
  for (size_t i = 0; i < s.dirnode.size(); ++i) {
    int64_t p = s.dirnode[i];
    for (int c = 0; c < 5; ++c)
      if (s.dirmask[i * 5 + c]) U[p * 5 + c] = s.dirval[i * 5 + c];
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
  riecg_bc(s, s.U.data());
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
};

inline real kpressure(const KozCG& s, real re) { return re * (s.gamma - 1.0); }

// kozak::rhs (src/Physics/Kozak.cpp:29-180), no source term.
void kozak_rhs(const KozCG& s, const real* U, real dt, real* R) {
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
  }
}

// KozCG::BC for the configured BC kinds (src/Inciter/KozCG.cpp:590-611).
void kozcg_bc(KozCG& s, real* U) {
  for (size_t i = 0; i < s.dirnode.size(); ++i) {
    int64_t p = s.dirnode[i];
    for (int c = 0; c < 5; ++c)
      if (s.dirmask[i * 5 + c]) U[p * 5 + c] = s.dirval[i * 5 + c];
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
  kozak_rhs(s, U, s.dt, s.R.data());
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
  kozcg_bc(s, s.A.data());
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

void orc_riecg_bc(void* h) {
  auto* s = static_cast<RieCG*>(h);
  riecg_bc(*s, s->U.data());
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
void orc_riecg_stage(void* h, int stage, double dt) {
  auto* s = static_cast<RieCG*>(h);
  s->dt = dt;
  riecg_stage(*s, stage);
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

void orc_kozcg_set_state(void* h, const double* U) {
  auto* s = static_cast<KozCG*>(h);
  s->U.assign(U, U + s->npoin * 5);
}

void orc_kozcg_get_state(void* h, double* U) {
  auto* s = static_cast<KozCG*>(h);
  std::memcpy(U, s->U.data(), sizeof(real) * s->U.size());
}

void orc_kozcg_rhs(void* h, const double* U, double dt, double* R) {
  kozak_rhs(*static_cast<KozCG*>(h), U, dt, R);
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
