// ChoCG on one GB300: the chorin:: edge passes as node-gather kernels, the
// explicit RK momentum prediction, nodal BCs, CFL reduction and the
// pressure-increment projection around the context's CG solver.
//
// Reference path (all paths relative to the reference project root):
//   chorin::div/vgrad/grad/flux/rhs  src/Physics/Chorin.cpp:34-1044
//   ChoCG::merge/div/pinit/psolve/sgrad/psolved/pgrad
//                                    src/Inciter/ChoCG.cpp:739-764, 868-1281
//   ChoCG::BC/dt/advance/rhs/solve/pred/corr
//                                    src/Inciter/ChoCG.cpp:1333-1695
//   physics::dirbc/symbc/noslipbc    src/Physics/BC.cpp:27-145
//
// Layout in HBM (n nodes), FP64 throughout (the projection scheme is the
// configuration the reference runs in double precision):
//   u, u2, un     [3][n]  velocity (ping-pong) and the stage-0 copy
//   pr, div       [n]     pressure and the Poisson right-hand side
//   pgrad         [3][n]  pressure gradient
//   vgrad         [9][n]  velocity gradient (damp4 and the start-up flux)
//   flx           [3][n]  momentum flux (start-up only)
//   adjacency     SELL-32 over both ends of every edge, entry (k, lane) of
//                 slice s at off[s] + 32k + lane: the neighbour (~id when the
//                 node is the canonical second end) and (d0, d1, d2, d4), the
//                 dual-face normal and the viscous coefficient of the edge,
//                 plus |d| / |x_a - x_b| for the pressure damping
//   bnode, park   boundary-node list and [nb][9] domain sums between passes
// Every edge term is evaluated in the edge's canonical orientation at both
// ends, so the two ends see bit-identical values and each node owns its
// writes (no atomics except the scalar CFL minimum).  A node's neighbours are
// visited in increasing id, which for an unrenumbered mesh is the order in
// which the reference's edge loop reaches the node.  Each node kernel runs
// as a domain pass over all nodes and a pass over the boundary nodes that
// adds the boundary-triangle terms (see node_of).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "xg_internal.hpp"

namespace xg {

namespace {
constexpr int kSlice = 32;
constexpr int32_t kPad = INT32_MIN;
constexpr int kBlock = 256;
}  // namespace

// The four edge coefficients of an adjacency entry: d0, d1, d2 (dual-face
// normal) and d4 (viscous coefficient).
struct alignas(32) Coef4 {
  double x, y, z, w;
};

struct ChoCGDev {
  Arena arena;    // mesh-sized arrays
  Arena bcarena;  // boundary condition program
  int64_t n = 0, nslice = 0, nent = 0, nbn = 0;
  xg_chocg_params prm{};
  int32_t *soff = nullptr, *swidth = nullptr, *nbr = nullptr;
  Coef4* dd = nullptr;
  double* sdl = nullptr;  // per entry |d| / edge length (the pressure damping of chorin::div)
  int32_t *bidx = nullptr, *bptr = nullptr, *bent = nullptr, *btri = nullptr;
  int32_t* bnode = nullptr;  // boundary index -> node
  double* park = nullptr;    // [nbn][9] domain sums of boundary nodes between passes
  double *xyz = nullptr, *vol = nullptr;
  double *u = nullptr, *u2 = nullptr, *un = nullptr, *pr = nullptr, *pgrad = nullptr,
         *vgrad = nullptr, *div = nullptr, *flx = nullptr, *stage = nullptr;
  unsigned long long* dtmin = nullptr;
  // BC program, one thread per BC node
  int64_t nbc = 0, nsymbc = 0;
  int32_t *bcnode = nullptr, *bcdir = nullptr, *bcsymp = nullptr, *bcnoslip = nullptr,
          *dirmask = nullptr;
  double *dirval = nullptr, *symn = nullptr;
  bool pdir_set = false;
  double t = 0.0;
  bool ready = false;  // start-up done
  int64_t last_it = 0;
  std::vector<double> xyz_host;  // [3][n], for the momentum matrix
  // theta-implicit momentum prediction (ChoCG::lhs/solve/msolve/msolved):
  // its own CG system of 3n rows (row 3i + c), the stiffness and consistent
  // mass values on its pattern (SELL order), the rhs of the last stage
  // ([3][n]) and as the system's right-hand side (row order), and the
  // Dirichlet rows (velocity Dirichlet components and noslip nodes)
  double theta = 0.0;
  int mom_pc = 0;
  int64_t mom_iter = 10;
  double mom_tol = 1.0e-3;
  CGDev* mom = nullptr;
  Arena momarena;
  double *baseK = nullptr, *baseM = nullptr, *R3 = nullptr, *b3 = nullptr;
  std::vector<uint8_t> mommask;
  bool mommask_up = false;
  int64_t last_mit = 0;
};

void destroy_chocg(ChoCGDev* d) {
  if (d && d->mom) destroy_cg(d->mom);
  delete d;
}
size_t bytes_chocg(const ChoCGDev* d) {
  return d ? d->arena.bytes() + d->bcarena.bytes() + d->momarena.bytes() : 0;
}

namespace {

struct ChoAdj {
  const int32_t* soff;
  const int32_t* swidth;
  const int32_t* nbr;
  const Coef4* dd;
  const double* sdl;
};
struct ChoBnd {
  const int32_t* bidx;
  const int32_t* bptr;
  const int32_t* bent;  // (triangle << 2) | position of the node in it
  const int32_t* btri;
  const double* xyz;    // SoA coordinates
  const int32_t* bnode;  // boundary index -> node
  double* park;          // [nb][9]: a boundary node's domain sum between the passes
  int64_t nb;
};

// Every node kernel runs as two passes.  The domain pass (one thread per
// node) sums the edge terms; a boundary node parks that sum and returns.  The
// boundary pass (one thread per boundary node) adds the boundary-triangle
// terms in the reference's order and applies the epilogue.  Folded into the
// domain pass, the few boundary nodes of a warp held all 32 lanes for their
// triangle loops.
__device__ __forceinline__ bool node_of(bool bnd_pass, int64_t n, const ChoBnd& b, int64_t& p,
                                        int32_t& bi) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (bnd_pass) {
    if (t >= b.nb) return false;
    bi = static_cast<int32_t>(t);
    p = __ldg(b.bnode + t);
  } else {
    if (t >= n) return false;
    p = t;
    bi = -1;
  }
  return true;
}

__device__ __forceinline__ Coef4 ldd4(const Coef4* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldg(q), b = __ldg(q + 1);
  return Coef4{a.x, a.y, b.x, b.y};
}

// Boundary-face normal / 6 of triangle t (tk::crossdiv(..., 6.0),
// src/Base/Vector.hpp:68-77), the same expression at every vertex.
__device__ __forceinline__ void tri_normal6(const ChoBnd& b, int64_t n, int32_t t, int32_t N[3],
                                            double nn[3]) {
  N[0] = __ldg(b.btri + 3 * t);
  N[1] = __ldg(b.btri + 3 * t + 1);
  N[2] = __ldg(b.btri + 3 * t + 2);
  const double* x = b.xyz;
  const double* y = b.xyz + n;
  const double* z = b.xyz + 2 * n;
  const double bax = x[N[1]] - x[N[0]], bay = y[N[1]] - y[N[0]], baz = z[N[1]] - z[N[0]];
  const double cax = x[N[2]] - x[N[0]], cay = y[N[2]] - y[N[0]], caz = z[N[2]] - z[N[0]];
  nn[0] = (bay * caz - cay * baz) / 6.0;
  nn[1] = (baz * cax - caz * bax) / 6.0;
  nn[2] = (bax * cay - cax * bay) / 6.0;
}

// (6 f_pos + f_other + f_other)/8 of a triangle's three vertex values, for
// the vertex at pos (Chorin.cpp:183-205 and the same weights elsewhere).
__device__ __forceinline__ double wavg(int pos, double a, double b, double c) {
  return pos == 0 ? (6.0 * a + b + c) / 8.0
                  : (pos == 1 ? (a + 6.0 * b + c) / 8.0 : (a + b + 6.0 * c) / 8.0);
}

__device__ __forceinline__ void block_min(double v, unsigned long long* dst) {
  __shared__ double red[32];
  unsigned long long bits = __double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = other < bits ? other : bits;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = __longlong_as_double(bits);
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    unsigned long long b = __double_as_longlong(lane < nw ? red[lane] : DBL_MAX);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
      b = other < b ? other : b;
    }
    if (lane == 0) atomicMin(dst, b);
  }
}

// Calls f(e, q, first) for the adjacency entries of a node in entry order
// (q the neighbour, first: the node is the edge's canonical first end), in
// rounds fully unrolled to exactly the entries left, at most XM (the slice
// width is uniform across the warp, so the dispatch does not diverge).  A
// round loads its neighbour ids first, so that its gathers are in flight
// together instead of one entry's load chain after another.
template <int R, class F>
__device__ __forceinline__ void adj_round(const int32_t* __restrict__ nbr, int32_t e0, F& f) {
  int32_t qq[R];
#pragma unroll
  for (int u = 0; u < R; ++u) qq[u] = __ldg(nbr + e0 + u * kSlice);
#pragma unroll
  for (int u = 0; u < R; ++u) {
    const int32_t q = qq[u];
    if (q != kPad) f(e0 + u * kSlice, q >= 0 ? q : ~q, q >= 0);
  }
}

template <int R, int XM, class F>
__device__ __forceinline__ void adj_tail(int r, const int32_t* __restrict__ nbr, int32_t e0,
                                         F& f) {
  if constexpr (R <= XM) {
    if (r == R) {
      adj_round<R>(nbr, e0, f);
      return;
    }
    adj_tail<R + 1, XM>(r, nbr, e0, f);
  }
}

template <int XM, class F>
__device__ __forceinline__ void for_adj(const ChoAdj& adj, int32_t off, int w, int lane, F f) {
  const int32_t e0 = off + lane;
  int k = 0;
  for (; w - k > XM; k += XM) adj_round<XM>(adj.nbr, e0 + k * kSlice, f);
  if (w > k) adj_tail<1, XM>(w - k, adj.nbr, e0 + k * kSlice, f);
}

// What the gradient kernel does with a node's gradient g of NC components.
enum GradOut { GRAD_RAW = 0, GRAD_DIVIDE = 1, GRAD_PROJECT = 2 };

// chorin::vgrad / chorin::grad (Chorin.cpp:211-449): G = sum over edges of
// -/+ d (u_p + u_q) plus the boundary-triangle term.  GRAD_RAW stores it,
// GRAD_DIVIDE stores G/vol (ChoCG::fingrad, src/Inciter/ChoCG.cpp:841-866),
// GRAD_PROJECT (NC = 1, the pressure increment) applies the projection of
// ChoCG::psolved (src/Inciter/ChoCG.cpp:1204-1216): u -= dt G/vol, and with
// addp the pressure update pr += increment (src/Inciter/ChoCG.cpp:1246-1250).
template <int NC, int MODE, bool BND>
__global__ void __launch_bounds__(kBlock) k_cgrad(int64_t n, ChoAdj adj, const double* U,
                                                   ChoBnd bnd, const double* __restrict__ vol,
                                                   double* __restrict__ G, double dt, int addp,
                                                   double* u, double* pr) {
  int64_t p;
  int32_t bi;
  if (!node_of(BND, n, bnd, p, bi)) return;
  double up[NC];
#pragma unroll
  for (int i = 0; i < NC; ++i) up[i] = U[i * n + p];
  double g[3 * NC];
  if (!BND) {
#pragma unroll
    for (int i = 0; i < 3 * NC; ++i) g[i] = 0.0;
    const int lane = static_cast<int>(p & (kSlice - 1));
    const int64_t s = p >> 5;
    const int32_t off = __ldg(adj.soff + s), w = __ldg(adj.swidth + s);
    for_adj<NC == 1 ? 16 : 8>(adj, off, w, lane, [&](int32_t e, int32_t q, bool first) {
      const Coef4 d = ldd4(adj.dd + e);
#pragma unroll
      for (int i = 0; i < NC; ++i) {
        const double sum = U[i * n + q] + up[i];
        const double f0 = d.x * sum, f1 = d.y * sum, f2 = d.z * sum;
        if (first) {
          g[i * 3 + 0] -= f0;
          g[i * 3 + 1] -= f1;
          g[i * 3 + 2] -= f2;
        } else {
          g[i * 3 + 0] += f0;
          g[i * 3 + 1] += f1;
          g[i * 3 + 2] += f2;
        }
      }
    });
    const int32_t b = __ldg(bnd.bidx + p);
    if (b >= 0) {
#pragma unroll
      for (int i = 0; i < 3 * NC; ++i) bnd.park[b * 9 + i] = g[i];
      return;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3 * NC; ++i) g[i] = bnd.park[bi * 9 + i];
    for (int32_t j = __ldg(bnd.bptr + bi); j < __ldg(bnd.bptr + bi + 1); ++j) {
      const int32_t ent = __ldg(bnd.bent + j);
      const int pos = ent & 3;
      int32_t N[3];
      double nn[3];
      tri_normal6(bnd, n, ent >> 2, N, nn);
#pragma unroll
      for (int i = 0; i < NC; ++i) {
        const double f = wavg(pos, U[i * n + N[0]], U[i * n + N[1]], U[i * n + N[2]]);
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) g[i * 3 + jj] += f * nn[jj];
      }
    }
  }
  if (MODE == GRAD_RAW) {
#pragma unroll
    for (int i = 0; i < 3 * NC; ++i) G[i * n + p] = g[i];
  } else if (MODE == GRAD_DIVIDE) {
    const double v = vol[p];
#pragma unroll
    for (int i = 0; i < 3 * NC; ++i) G[i * n + p] = g[i] / v;
  } else {
    const double v = vol[p];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) u[jj * n + p] -= dt * (g[jj] / v);
    if (addp) pr[p] += up[0];
  }
}

// chorin::div (Chorin.cpp:34-209): divergence of the 3-component U with the
// 4th-order pressure damping when stab, optionally divided by dt
// (ChoCG::pinit, src/Inciter/ChoCG.cpp:1039).
template <bool BND>
__global__ void __launch_bounds__(kBlock) k_cdiv(int64_t n, ChoAdj adj, const double* U,
                                                  const double* __restrict__ P,
                                                  const double* __restrict__ PG, ChoBnd bnd,
                                                  double dt, int stab, int bydt,
                                                  double* __restrict__ D) {
  int64_t p;
  int32_t bi;
  if (!node_of(BND, n, bnd, p, bi)) return;
  double acc = 0.0;
  if (!BND) {
    const int lane = static_cast<int>(p & (kSlice - 1));
    const int64_t s = p >> 5;
    const int32_t off = __ldg(adj.soff + s), w = __ldg(adj.swidth + s);
    const double* x = bnd.xyz;
    const double* y = bnd.xyz + n;
    const double* z = bnd.xyz + 2 * n;
    for_adj<8>(adj, off, w, lane, [&](int32_t e, int32_t q, bool first) {
      const Coef4 d = ldd4(adj.dd + e);
      const int64_t a = first ? p : q, b = first ? q : p;  // canonical ends
      double f = d.x * (U[a] + U[b]) + d.y * (U[n + a] + U[n + b]) +
                 d.z * (U[2 * n + a] + U[2 * n + b]);
      if (stab) {
        // |d| / |x_a - x_b| is geometric: formed once at setup (two FP64
        // square roots and a division per edge and call are expensive on
        // GB300's FP64 pipe)
        const double dx = x[a] - x[b], dy = y[a] - y[b], dz = z[a] - z[b];
        const double p2 = P[b] - P[a];
        const double dpx = PG[a] + PG[b], dpy = PG[n + a] + PG[n + b],
                     dpz = PG[2 * n + a] + PG[2 * n + b];
        const double p4 = 0.5 * (dx * dpx + dy * dpy + dz * dpz);
        f += __ldg(adj.sdl + e) * dt * (p2 + p4);
      }
      acc = first ? acc - f : acc + f;
    });
    const int32_t b = __ldg(bnd.bidx + p);
    if (b >= 0) {
      bnd.park[b * 9] = acc;
      return;
    }
  } else {
    acc = bnd.park[bi * 9];
    for (int32_t j = __ldg(bnd.bptr + bi); j < __ldg(bnd.bptr + bi + 1); ++j) {
      const int32_t ent = __ldg(bnd.bent + j);
      const int pos = ent & 3;
      int32_t N[3];
      double nn[3];
      tri_normal6(bnd, n, ent >> 2, N, nn);
      const double ux = wavg(pos, U[N[0]], U[N[1]], U[N[2]]);
      const double uy = wavg(pos, U[n + N[0]], U[n + N[1]], U[n + N[2]]);
      const double uz = wavg(pos, U[2 * n + N[0]], U[2 * n + N[1]], U[2 * n + N[2]]);
      acc += ux * nn[0] + uy * nn[1] + uz * nn[2];
    }
  }
  D[p] = bydt ? acc / dt : acc;
}

// Momentum flux of tensor component (i,j) over an edge and in a point
// (Chorin.cpp:451-507).  The edge form is called with the canonical second
// end first, as the reference's loops do.
__device__ __forceinline__ double mflux_e(const double* U, const double* G, int64_t n, int i,
                                          int j, int64_t p, int64_t q, double mu) {
  const double inv = U[i * n + p] * U[j * n + p] + U[i * n + q] * U[j * n + q];
  if (mu < DBL_EPSILON) return -inv;
  double vis = G[(i * 3 + j) * n + p] + G[(j * 3 + i) * n + p] + G[(i * 3 + j) * n + q] +
               G[(j * 3 + i) * n + q];
  if (i == j)
    vis -= 2.0 / 3.0 * (G[0 * n + p] + G[4 * n + p] + G[8 * n + p] + G[0 * n + q] +
                        G[4 * n + q] + G[8 * n + q]);
  return mu * vis - inv;
}
__device__ __forceinline__ double mflux_p(const double* U, const double* G, int64_t n, int i,
                                          int j, int64_t p, double mu) {
  const double inv = U[i * n + p] * U[j * n + p];
  if (mu < DBL_EPSILON) return -inv;
  double vis = G[(i * 3 + j) * n + p] + G[(j * 3 + i) * n + p];
  if (i == j) vis -= 2.0 / 3.0 * (G[0 * n + p] + G[4 * n + p] + G[8 * n + p]);
  return mu * vis - inv;
}

// chorin::flux (Chorin.cpp:509-638): F_i = d[s_ij - u_i u_j]/dx_j, raw or
// divided by the volume (ChoCG::div at start-up, src/Inciter/ChoCG.cpp:877).
template <bool BND>
__global__ void __launch_bounds__(kBlock) k_cflux(int64_t n, ChoAdj adj, const double* U,
                                                   const double* G, ChoBnd bnd,
                                                   const double* __restrict__ vol, double mu,
                                                   int divide, double* __restrict__ F) {
  int64_t p;
  int32_t bi;
  if (!node_of(BND, n, bnd, p, bi)) return;
  double acc[3] = {0.0, 0.0, 0.0};
  if (!BND) {
    const int lane = static_cast<int>(p & (kSlice - 1));
    const int64_t s = p >> 5;
    const int32_t off = __ldg(adj.soff + s), w = __ldg(adj.swidth + s);
    for_adj<4>(adj, off, w, lane, [&](int32_t e, int32_t q, bool first) {
      const Coef4 d = ldd4(adj.dd + e);
      const int64_t a = first ? p : q, b = first ? q : p;
      const double dj[3] = {d.x, d.y, d.z};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const double f = dj[j] * mflux_e(U, G, n, i, j, b, a, mu);
          acc[i] = first ? acc[i] - f : acc[i] + f;
        }
    });
    const int32_t b = __ldg(bnd.bidx + p);
    if (b >= 0) {
#pragma unroll
      for (int i = 0; i < 3; ++i) bnd.park[b * 9 + i] = acc[i];
      return;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) acc[i] = bnd.park[bi * 9 + i];
    for (int32_t jb = __ldg(bnd.bptr + bi); jb < __ldg(bnd.bptr + bi + 1); ++jb) {
      const int32_t ent = __ldg(bnd.bent + jb);
      const int pos = ent & 3;
      int32_t N[3];
      double nn[3];
      tri_normal6(bnd, n, ent >> 2, N, nn);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double fv[3];
#pragma unroll
        for (int j = 0; j < 3; ++j)
          fv[j] = wavg(pos, mflux_p(U, G, n, i, j, N[0], mu), mflux_p(U, G, n, i, j, N[1], mu),
                       mflux_p(U, G, n, i, j, N[2], mu));
        acc[i] += fv[0] * nn[0] + fv[1] * nn[1] + fv[2] * nn[2];
      }
    }
  }
  const double v = divide ? vol[p] : 1.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) F[i * n + p] = divide ? acc[i] / v : acc[i];
}

struct AdvPrm {
  double mu, stab2coef;
  int stab, stab2;
};

// adv_damp2 / adv_damp4 edge flux of the three velocity components on the
// canonical edge a -> b (Chorin.cpp:640-829).
template <bool DAMP4>
__device__ __forceinline__ void adv_edge(const double* U, const double* G, const double* P,
                                         const double* xyz, int64_t n, Coef4 d, int64_t a,
                                         int64_t b, const AdvPrm& ap, double f[3]) {
  double uL[3] = {U[a], U[n + a], U[2 * n + a]};
  double uR[3] = {U[b], U[n + b], U[2 * n + b]};
  if (DAMP4) {
    const double eps = 1.0e-9, k = 1.0 / 3.0;
    const double dx = xyz[b] - xyz[a], dy = xyz[n + b] - xyz[n + a],
                 dz = xyz[2 * n + b] - xyz[2 * n + a];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double g1 = G[(c * 3 + 0) * n + a] * dx + G[(c * 3 + 1) * n + a] * dy +
                        G[(c * 3 + 2) * n + a] * dz;
      const double g2 = G[(c * 3 + 0) * n + b] * dx + G[(c * 3 + 1) * n + b] * dy +
                        G[(c * 3 + 2) * n + b] * dz;
      const double delta2 = uR[c] - uL[c];
      const double delta1 = 2.0 * g1 - delta2;
      const double delta3 = 2.0 * g2 - delta2;
      const double rL = (delta2 + eps) / (delta1 + eps);
      const double rR = (delta2 + eps) / (delta3 + eps);
      const double rLinv = (delta1 + eps) / (delta2 + eps);
      const double rRinv = (delta3 + eps) / (delta2 + eps);
      const double phiL = (fabs(rL) + rL) / (fabs(rL) + 1.0);
      const double phiR = (fabs(rR) + rR) / (fabs(rR) + 1.0);
      const double phiLi = (fabs(rLinv) + rLinv) / (fabs(rLinv) + 1.0);
      const double phiRi = (fabs(rRinv) + rRinv) / (fabs(rRinv) + 1.0);
      uL[c] += 0.25 * (delta1 * (1.0 - k) * phiL + delta2 * (1.0 + k) * phiLi);
      uR[c] -= 0.25 * (delta3 * (1.0 - k) * phiR + delta2 * (1.0 + k) * phiRi);
    }
  }
  const double nx = d.x, ny = d.y, nz = d.z;
  const double vnL = uL[0] * nx + uL[1] * ny + uL[2] * nz;
  const double vnR = uR[0] * nx + uR[1] * ny + uR[2] * nz;
  double aw = 0.0;
  if (ap.stab) aw = fabs(vnL + vnR) / 2.0;
  if (ap.stab2) aw += ap.stab2coef * fmax(fabs(vnL), fabs(vnR));
  const double v = d.w * ap.mu;
  const double pf = P[a] + P[b];
  const double nv[3] = {nx, ny, nz};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (DAMP4)
      f[c] = uL[c] * vnL + uR[c] * vnR + pf * nv[c] + aw * (uR[c] - uL[c]) -
             v * (U[c * n + b] - U[c * n + a]);
    else
      f[c] = uL[c] * vnL + uR[c] * vnR + pf * nv[c] + (aw - v) * (uR[c] - uL[c]);
  }
}

// chorin::rhs (Chorin.cpp:831-1044) at every node, fused with the explicit
// stage update of ChoCG::solve (src/Inciter/ChoCG.cpp:1550-1566):
// u_out = un - dtk R / vol, where un is this stage's input at stage 0.
// With dtk == 0 and a null u_out only R is written (drop-in).
template <bool DAMP4, bool BND>
__global__ void __launch_bounds__(kBlock) k_crhs(int64_t n, ChoAdj adj, const double* U,
                                                  const double* G, const double* P, ChoBnd bnd,
                                                  AdvPrm ap, const double* __restrict__ vol,
                                                  double dtk, int stage0, double* un,
                                                  double* __restrict__ uout,
                                                  double* __restrict__ R) {
  int64_t p;
  int32_t bi;
  if (!node_of(BND, n, bnd, p, bi)) return;
  double acc[3] = {0.0, 0.0, 0.0};
  if (!BND) {
    const int lane = static_cast<int>(p & (kSlice - 1));
    const int64_t s = p >> 5;
    const int32_t off = __ldg(adj.soff + s), w = __ldg(adj.swidth + s);
    for_adj<DAMP4 ? 4 : 8>(adj, off, w, lane, [&](int32_t e, int32_t q, bool first) {
      const Coef4 d = ldd4(adj.dd + e);
      double f[3];
      adv_edge<DAMP4>(U, G, P, bnd.xyz, n, d, first ? p : q, first ? q : p, ap, f);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] = first ? acc[c] - f[c] : acc[c] + f[c];
    });
    const int32_t b = __ldg(bnd.bidx + p);
    if (b >= 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) bnd.park[b * 9 + c] = acc[c];
      return;
    }
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] = bnd.park[bi * 9 + c];
    for (int32_t j = __ldg(bnd.bptr + bi); j < __ldg(bnd.bptr + bi + 1); ++j) {
      const int32_t ent = __ldg(bnd.bent + j);
      const int pos = ent & 3;
      int32_t N[3];
      double nn[3];
      tri_normal6(bnd, n, ent >> 2, N, nn);
      double fl[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double uu = U[N[a]], vv = U[n + N[a]], ww = U[2 * n + N[a]], pp = P[N[a]];
        const double vn = nn[0] * uu + nn[1] * vv + nn[2] * ww;
        fl[0][a] = uu * vn + pp * nn[0];
        fl[1][a] = vv * vn + pp * nn[1];
        fl[2][a] = ww * vn + pp * nn[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] += wavg(pos, fl[c][0], fl[c][1], fl[c][2]);
    }
  }
  if (R) {
#pragma unroll
    for (int c = 0; c < 3; ++c) R[c * n + p] = acc[c];
  }
  if (uout) {
    const double v = vol[p];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double u0;
      if (stage0) {
        u0 = U[c * n + p];
        un[c * n + p] = u0;
      } else {
        u0 = un[c * n + p];
      }
      uout[c * n + p] = u0 - dtk * acc[c] / v;
    }
  }
}

// ChoCG::BC (src/Inciter/ChoCG.cpp:1333-1354) per BC node, in the
// reference's order: Dirichlet components, symmetry projections (one per
// set holding the node), noslip.  sym_only applies just the symmetry
// projections (to the start-up momentum flux, ChoCG.cpp:878).
__global__ void k_cbc(int64_t n, int64_t nbc, const int32_t* __restrict__ node,
                      const int32_t* __restrict__ dir, const int32_t* __restrict__ symp,
                      const int32_t* __restrict__ noslip, const int32_t* __restrict__ dirmask,
                      const double* __restrict__ dirval, const double* __restrict__ symn,
                      int sym_only, double* U) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nbc) return;
  const int64_t p = node[i];
  double u[3] = {U[p], U[n + p], U[2 * n + p]};
  const int32_t dd = dir[i];
  if (!sym_only && dd >= 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (dirmask[dd * 3 + c]) u[c] = dirval[dd * 3 + c];
  }
  for (int32_t k = symp[i]; k < symp[i + 1]; ++k) {
    const double* nn = symn + 3 * k;
    const double vn = u[0] * nn[0] + u[1] * nn[1] + u[2] * nn[2];
    u[0] -= vn * nn[0];
    u[1] -= vn * nn[1];
    u[2] -= vn * nn[2];
  }
  if (!sym_only && noslip[i]) u[0] = u[1] = u[2] = 0.0;
  U[p] = u[0];
  U[n + p] = u[1];
  U[2 * n + p] = u[2];
}

// ChoCG::dt (src/Inciter/ChoCG.cpp:1356-1412): min over nodes of
// cbrt(V)/max(|u|, 1e-8) and, with viscosity, V^(2/3)/mu.
__global__ void __launch_bounds__(kBlock) k_cdt(int64_t n, const double* __restrict__ U,
                                                 const double* __restrict__ vol, double mu,
                                                 unsigned long long* dtmin) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double m = DBL_MAX;
  if (p < n) {
    const double u = U[p], v = U[n + p], w = U[2 * n + p];
    const double vel = sqrt(u * u + v * v + w * w);
    const double L = cbrt(vol[p]);
    m = fmin(m, L / fmax(vel, 1.0e-8));
    if (mu > DBL_EPSILON) m = fmin(m, L * L / mu);
  }
  block_min(m, dtmin);
}

__global__ void k_aos_soa(int64_t n, int nc, const double* __restrict__ a, double* __restrict__ s) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nc) return;
  const int64_t p = i / nc;
  const int c = static_cast<int>(i - p * nc);
  s[c * n + p] = a[i];
}
__global__ void k_soa_aos(int64_t n, int nc, const double* __restrict__ s, double* __restrict__ a) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nc) return;
  const int64_t p = i / nc;
  const int c = static_cast<int>(i - p * nc);
  a[i] = s[c * n + p];
}

// ---------------------------------------------------------------- host side

ChoAdj adj_of(ChoCGDev* d) { return ChoAdj{d->soff, d->swidth, d->nbr, d->dd, d->sdl}; }
ChoBnd bnd_of(ChoCGDev* d) {
  return ChoBnd{d->bidx, d->bptr, d->bent, d->btri, d->xyz, d->bnode, d->park, d->nbn};
}

// Both passes of a node kernel (domain pass over the n nodes, then the
// boundary pass over the boundary nodes), the same arguments to each.
template <auto KD, auto KB, class... A>
void two_pass(cudaStream_t s, int64_t n, int64_t nb, A... args) {
  KD<<<blocks_for(n, kBlock), kBlock, 0, s>>>(args...);
  if (nb > 0) KB<<<blocks_for(nb, kBlock), kBlock, 0, s>>>(args...);
}
AdvPrm adv_of(ChoCGDev* d) {
  return AdvPrm{d->prm.mu, d->prm.stab2coef, d->prm.stab != 0, d->prm.stab2 != 0};
}

int get_ctx(xg_ctx* c, ChoCGDev** out, bool need_cg) {
  int rc = use(c);
  if (rc) return rc;
  ChoCGDev* d = c->chocg;
  if (!d) return fail(c, XG_ERR_STATE, "chocg: no operators (xg_chocg_setup)");
  if (need_cg && cg_rows(c) != d->n)
    return fail(c, XG_ERR_STATE, "chocg: the context's CG system is not the pressure matrix");
  *out = d;
  return XG_OK;
}

template <int NC, int MODE>
int launch_grad(xg_ctx* c, ChoCGDev* d, const double* U, double* G, double dt = 0.0,
                int addp = 0) {
  two_pass<k_cgrad<NC, MODE, false>, k_cgrad<NC, MODE, true>>(
      c->stream, d->n, d->nbn, d->n, adj_of(d), U, bnd_of(d), d->vol, G, dt, addp, d->u, d->pr);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

int launch_bc(xg_ctx* c, ChoCGDev* d, double* U, int sym_only) {
  if (d->nbc == 0) return XG_OK;
  k_cbc<<<blocks_for(d->nbc, kBlock), kBlock, 0, c->stream>>>(
      d->n, d->nbc, d->bcnode, d->bcdir, d->bcsymp, d->bcnoslip, d->dirmask, d->dirval, d->symn,
      sym_only, U);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

int launch_div(xg_ctx* c, ChoCGDev* d, const double* U, double dt, int stab, int bydt) {
  two_pass<k_cdiv<false>, k_cdiv<true>>(c->stream, d->n, d->nbn, d->n, adj_of(d), U, d->pr,
                                        d->pgrad, bnd_of(d), dt, stab, bydt, d->div);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

int launch_rhs(xg_ctx* c, ChoCGDev* d, const double* U, double dtk, int stage0, double* uout,
               double* R) {
  const AdvPrm ap = adv_of(d);
  if (d->prm.flux == XG_DAMP4)
    two_pass<k_crhs<true, false>, k_crhs<true, true>>(c->stream, d->n, d->nbn, d->n, adj_of(d), U,
                                                       d->vgrad, d->pr, bnd_of(d), ap, d->vol,
                                                       dtk, stage0, d->un, uout, R);
  else
    two_pass<k_crhs<false, false>, k_crhs<false, true>>(c->stream, d->n, d->nbn, d->n, adj_of(d),
                                                         U, d->vgrad, d->pr, bnd_of(d), ap, d->vol,
                                                         dtk, stage0, d->un, uout, R);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

// theta-implicit momentum system, per step (ChoCG::lhs, ChoCG.cpp:1433-1477):
// A = -(M / dt + theta mu K) with M the consistent mass sum_e J/120 (1 + d_ab)
// and K the stiffness sum_e grad_a.grad_b / J / 6, both on A's pattern.
__global__ void k_mom_values(int64_t nent, const double* __restrict__ K,
                             const double* __restrict__ M, double thmu, double dt,
                             double* __restrict__ a) {
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= nent) return;
  a[e] = -(M[e] / dt + thmu * K[e]);
}
// [3][n] -> row order 3i + c, and the update u = un + du of ChoCG::msolved
// (ChoCG.cpp:1626-1645).
__global__ void k_to_rows3(int64_t n, const double* __restrict__ R, double* __restrict__ b) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) b[i * 3 + c] = R[c * n + i];
}
__global__ void k_mom_update(int64_t n, const double* __restrict__ un,
                             const double* __restrict__ du, double* __restrict__ u) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c * n + i] = un[c * n + i] + du[i * 3 + c];
}

// The semi-implicit last stage of ChoCG::solve (ChoCG.cpp:1576-1606): the
// momentum system A du = R (R the stage's rhs, [3][n] in d->R3) with the
// Dirichlet rows at zero increment, warm-started from the previous
// increment, mom_iter iterations at most to mom_tol, then u = un + du.  The
// momentum system is the context's CG system while it solves.
int momentum_solve(xg_ctx* c, ChoCGDev* d, double dt) {
  const int64_t n = d->n;
  cudaStream_t s = c->stream;
  CGDev* const saved = c->cg;
  c->cg = d->mom;
  int rc = XG_OK;
  do {
    const int64_t nent = cg_nent(c);
    k_mom_values<<<blocks_for(nent, kBlock), kBlock, 0, s>>>(
        nent, d->baseK, d->baseM, d->theta * d->prm.mu, dt, cg_values_device(c));
    XG_CHECK_LAUNCH(c);
    k_to_rows3<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->R3, d->b3);
    XG_CHECK_LAUNCH(c);
    if (!d->mommask_up) {
      std::vector<uint8_t> mask = d->mommask;
      mask.resize(n * 3, 0);
      std::vector<double> zero(n * 3, 0.0);
      rc = cg_set_dirichlet(c, mask.data(), zero.data());
      if (rc) break;
      d->mommask_up = true;
    }
    rc = cg_init_device(c, d->b3, 1, d->mom_pc);
    if (rc) break;
    int64_t it = 0;
    double normr = 0, normb = 0;
    int conv = 0;
    rc = xg_cg_solve(c, d->mom_iter, d->mom_tol, &it, &normr, &normb, &conv);
    if (rc == XG_ERR_NOTCONV) rc = XG_OK;  // the reference carries on
    if (rc) break;
    d->last_mit = conv ? it : -it;
    k_mom_update<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->un, cg_solution_device(c), d->u);
    XG_CHECK_LAUNCH(c);
  } while (false);
  c->cg = saved;
  return rc;
}

// One pressure solve of ChoCG::pinit/psolve on the context's CG system with
// the device right-hand side d->div: Dirichlet values of the first solves or
// zero, warm start from the previous solution.  As in the reference, a solve
// that stops short of the tolerance (iteration limit or the (p,q) breakdown
// guard) does not stop the scheme: last_it is then the negated count.
int pressure_solve(xg_ctx* c, ChoCGDev* d, int zero_values) {
  int rc = xg_cg_set_guard(c, d->prm.pguard);
  if (rc) return rc;
  rc = cg_init_device(c, d->div, zero_values, d->prm.ppc);
  if (rc) return rc;
  int64_t it = 0, outer = 0;
  double normr = 0, normb = 0;
  int conv = 0;
  if (d->prm.pmixed)
    rc = xg_cg_solve_mixed(c, 1000, d->prm.ptol, d->prm.pinner_tol, d->prm.pmaxit, &outer, &it,
                           &normr, &normb, &conv);
  else
    rc = xg_cg_solve(c, d->prm.pmaxit, d->prm.ptol, &it, &normr, &normb, &conv);
  if (rc && rc != XG_ERR_NOTCONV) return rc;
  d->last_it = conv ? it : -it;
  return XG_OK;
}

// Time step size of the device state (ChoCG::dt): synchronises.
int step_dt(xg_ctx* c, ChoCGDev* d, double* dt) {
  if (std::fabs(d->prm.const_dt) > DBL_EPSILON) {
    *dt = d->prm.const_dt;
    return XG_OK;
  }
  const unsigned long long big = 0x7fefffffffffffffull;  // DBL_MAX bits
  XG_CUDA(c, cudaMemcpyAsync(d->dtmin, &big, sizeof(big), cudaMemcpyHostToDevice, c->stream));
  k_cdt<<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->u, d->vol, d->prm.mu,
                                                             d->dtmin);
  XG_CHECK_LAUNCH(c);
  unsigned long long bits = 0;
  XG_CUDA(c, cudaMemcpyAsync(&bits, d->dtmin, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  double m;
  std::memcpy(&m, &bits, sizeof(m));
  *dt = m * d->prm.cfl;
  return XG_OK;
}

struct EdgeRec {
  int64_t a, b;
  double d[5];
};

}  // namespace

}  // namespace xg

using namespace xg;

extern "C" {

int xg_chocg_setup(xg_ctx* c, const xg_chocg_params* prm, int64_t npoin, const double* coord,
                   const double* vol, int64_t ntet, const uint64_t* dsupedge0,
                   const double* dsupint0, int64_t ntri, const uint64_t* dsupedge1,
                   const double* dsupint1, int64_t nedge, const uint64_t* dsupedge2,
                   const double* dsupint2, int64_t nbtri, const uint64_t* triinpoel) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  if (!prm || npoin <= 0 || !coord || !vol) return fail(c, XG_ERR_ARG, "chocg_setup: bad mesh");
  if (npoin >= (int64_t(1) << 31) - 64) return fail(c, XG_ERR_ARG, "chocg_setup: too many nodes");
  if (prm->flux != XG_DAMP2 && prm->flux != XG_DAMP4)
    return fail(c, XG_ERR_ARG, "Flux not correctly configured");
  if (prm->rk < 1 || prm->rk > 4) return fail(c, XG_ERR_ARG, "chocg_setup: rk must be 1..4");
  if (prm->ppc < 0 || prm->ppc > 2) return fail(c, XG_ERR_ARG, "chocg_setup: unknown pressure pc");
  if (prm->pguard != 0 && prm->pguard != 1)
    return fail(c, XG_ERR_ARG, "chocg_setup: pressure guard is 0 or 1");
  if (prm->pmaxit <= 0 || !(prm->ptol >= 0))
    return fail(c, XG_ERR_ARG, "chocg_setup: bad pressure iteration limit or tolerance");
  if ((ntet && (!dsupedge0 || !dsupint0)) || (ntri && (!dsupedge1 || !dsupint1)) ||
      (nedge && (!dsupedge2 || !dsupint2)) || (nbtri && !triinpoel))
    return fail(c, XG_ERR_ARG, "chocg_setup: null superedge or boundary array");
  const int64_t n = npoin;
  // superedges -> edges in the orientation chorin:: evaluates them
  // (Chorin.cpp:122-170: tet group (0,1),(1,2),(2,0),(0,3),(1,3),(2,3),
  // triangle group (0,1),(1,2),(2,0))
  std::vector<EdgeRec> E;
  E.reserve(static_cast<size_t>(ntet * 6 + ntri * 3 + nedge));
  static const int tp[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  static const int rp[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  auto bad = [&](uint64_t id) { return id >= static_cast<uint64_t>(n); };
  auto push = [&](uint64_t a, uint64_t b, const double* dd) -> bool {
    if (bad(a) || bad(b) || a == b) return false;
    EdgeRec r{int64_t(a), int64_t(b), {dd[0], dd[1], dd[2], dd[3], dd[4]}};
    E.push_back(r);
    return true;
  };
  for (int64_t e = 0; e < ntet; ++e)
    for (int k = 0; k < 6; ++k)
      if (!push(dsupedge0[e * 4 + tp[k][0]], dsupedge0[e * 4 + tp[k][1]],
                dsupint0 + (e * 6 + k) * 5))
        return fail(c, XG_ERR_ARG, "chocg_setup: tet superedge id");
  for (int64_t e = 0; e < ntri; ++e)
    for (int k = 0; k < 3; ++k)
      if (!push(dsupedge1[e * 3 + rp[k][0]], dsupedge1[e * 3 + rp[k][1]],
                dsupint1 + (e * 3 + k) * 5))
        return fail(c, XG_ERR_ARG, "chocg_setup: triangle superedge id");
  for (int64_t e = 0; e < nedge; ++e)
    if (!push(dsupedge2[e * 2], dsupedge2[e * 2 + 1], dsupint2 + e * 5))
      return fail(c, XG_ERR_ARG, "chocg_setup: edge id");
  // per-node entries sorted by neighbour id
  std::vector<int64_t> start(n + 1, 0);
  for (auto& e : E) {
    ++start[e.a + 1];
    ++start[e.b + 1];
  }
  for (int64_t i = 0; i < n; ++i) start[i + 1] += start[i];
  struct Ent {
    int64_t q, eid;
    bool first;
  };
  std::vector<Ent> ent(static_cast<size_t>(start[n]));
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (size_t k = 0; k < E.size(); ++k) {
      ent[fill[E[k].a]++] = {E[k].b, int64_t(k), true};
      ent[fill[E[k].b]++] = {E[k].a, int64_t(k), false};
    }
  }
  for (int64_t p = 0; p < n; ++p)
    std::sort(ent.begin() + start[p], ent.begin() + start[p + 1],
              [](const Ent& x, const Ent& y) { return x.q < y.q || (x.q == y.q && x.eid < y.eid); });
  const int64_t nslice = (n + kSlice - 1) / kSlice;
  std::vector<int32_t> soff(nslice + 1), swidth(nslice);
  int64_t total = 0;
  for (int64_t s = 0; s < nslice; ++s) {
    int64_t w = 0;
    for (int64_t p = s * kSlice; p < std::min(n, (s + 1) * kSlice); ++p)
      w = std::max<int64_t>(w, start[p + 1] - start[p]);
    swidth[s] = static_cast<int32_t>(w);
    soff[s] = static_cast<int32_t>(total);
    total += w * kSlice;
    if (total >= (int64_t(1) << 31)) return fail(c, XG_ERR_ARG, "chocg_setup: adjacency too large");
  }
  soff[nslice] = static_cast<int32_t>(total);
  std::vector<int32_t> nbr(static_cast<size_t>(std::max<int64_t>(1, total)), kPad);
  std::vector<Coef4> dd(nbr.size(), Coef4{0.0, 0.0, 0.0, 0.0});
  std::vector<double> sdl(nbr.size(), 0.0);
  for (int64_t p = 0; p < n; ++p) {
    const int64_t s = p / kSlice, lane = p % kSlice;
    for (int64_t k = 0; k < start[p + 1] - start[p]; ++k) {
      const Ent& en = ent[start[p] + k];
      const int64_t idx = soff[s] + k * kSlice + lane;
      nbr[idx] = en.first ? static_cast<int32_t>(en.q) : ~static_cast<int32_t>(en.q);
      const double* r = E[en.eid].d;
      dd[idx] = Coef4{r[0], r[1], r[2], r[4]};
      const double dx = coord[p] - coord[en.q], dy = coord[n + p] - coord[n + en.q],
                   dz = coord[2 * n + p] - coord[2 * n + en.q];
      sdl[idx] = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) /
                 std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  }
  // boundary triangles, per boundary node the (triangle, position) pairs in
  // triangle order
  std::vector<int32_t> bidx(n, -1), btri(std::max<int64_t>(1, nbtri * 3));
  std::vector<int32_t> bcount;
  int64_t nbn = 0;
  for (int64_t t = 0; t < nbtri; ++t)
    for (int a = 0; a < 3; ++a) {
      const uint64_t p = triinpoel[t * 3 + a];
      if (bad(p)) return fail(c, XG_ERR_ARG, "chocg_setup: triinpoel id");
      btri[t * 3 + a] = static_cast<int32_t>(p);
      if (bidx[p] < 0) {
        bidx[p] = static_cast<int32_t>(nbn++);
        bcount.push_back(0);
      }
      ++bcount[bidx[p]];
    }
  std::vector<int32_t> bptr(nbn + 1, 0), bent(std::max<int64_t>(1, nbtri * 3));
  std::vector<int32_t> bnode(std::max<int64_t>(1, nbn), 0);
  for (int64_t p = 0; p < n; ++p)
    if (bidx[p] >= 0) bnode[bidx[p]] = static_cast<int32_t>(p);
  for (int64_t i = 0; i < nbn; ++i) bptr[i + 1] = bptr[i] + bcount[i];
  {
    std::vector<int32_t> fill(bptr.begin(), bptr.end() - 1);
    for (int64_t t = 0; t < nbtri; ++t)
      for (int a = 0; a < 3; ++a)
        bent[fill[bidx[triinpoel[t * 3 + a]]]++] = static_cast<int32_t>(t * 4 + a);
  }
  if (c->chocg) {
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    destroy_chocg(c->chocg);
    c->chocg = nullptr;
  }
  auto* d = new ChoCGDev;
  c->chocg = d;
  d->n = n;
  d->prm = *prm;
  d->nslice = nslice;
  d->nent = total;
  d->nbn = nbn;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->arena;
    A.plan(d->soff, soff.size());
    A.plan(d->swidth, swidth.size());
    A.plan(d->nbr, nbr.size());
    A.plan(d->dd, dd.size());
    A.plan(d->sdl, sdl.size());
    A.plan(d->bidx, n);
    A.plan(d->bptr, bptr.size());
    A.plan(d->bent, bent.size());
    A.plan(d->btri, btri.size());
    A.plan(d->bnode, bnode.size());
    A.plan(d->park, bnode.size() * 9);
    A.plan(d->xyz, 3 * n);
    A.plan(d->vol, n);
    A.plan(d->u, 3 * n);
    A.plan(d->u2, 3 * n);
    A.plan(d->un, 3 * n);
    A.plan(d->pr, n);
    A.plan(d->pgrad, 3 * n);
    A.plan(d->vgrad, 9 * n);
    A.plan(d->div, n);
    A.plan(d->flx, 3 * n);
    A.plan(d->stage, 9 * n);
    A.plan(d->dtmin, 1);
    if (pass == 0) {
      cudaError_t e = A.reserve();
      if (e != cudaSuccess) {
        destroy_chocg(d);
        c->chocg = nullptr;
        return fail(c, XG_ERR_CUDA, std::string("chocg_setup: ") + cudaGetErrorString(e));
      }
    }
  }
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  };
  XG_CUDA(c, up(d->soff, soff.data(), soff.size() * 4));
  XG_CUDA(c, up(d->swidth, swidth.data(), swidth.size() * 4));
  XG_CUDA(c, up(d->nbr, nbr.data(), nbr.size() * 4));
  XG_CUDA(c, up(d->dd, dd.data(), dd.size() * sizeof(Coef4)));
  XG_CUDA(c, up(d->sdl, sdl.data(), sdl.size() * 8));
  XG_CUDA(c, up(d->bidx, bidx.data(), n * 4));
  XG_CUDA(c, up(d->bptr, bptr.data(), bptr.size() * 4));
  XG_CUDA(c, up(d->bent, bent.data(), bent.size() * 4));
  XG_CUDA(c, up(d->btri, btri.data(), btri.size() * 4));
  XG_CUDA(c, up(d->bnode, bnode.data(), bnode.size() * 4));
  XG_CUDA(c, up(d->xyz, coord, 3 * n * 8));
  d->xyz_host.assign(coord, coord + 3 * n);
  XG_CUDA(c, up(d->vol, vol, n * 8));
  for (double* z : {d->u, d->u2, d->un, d->pr, d->pgrad, d->vgrad, d->div, d->flx})
    XG_CUDA(c, cudaMemset(z, 0, (z == d->vgrad ? 9 : (z == d->pr || z == d->div ? 1 : 3)) * n * 8));
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_chocg_set_theta(xg_ctx* c, double theta, int64_t ntet, const uint64_t* inpoel, int mom_pc,
                       int64_t mom_iter, double mom_tol) {
  XG_HOST_TRY
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!(theta >= 0.0) || mom_iter < 0 || !(mom_tol > 0.0) || (mom_pc != 0 && mom_pc != 1))
    return fail(c, XG_ERR_ARG, "chocg_set_theta: bad theta, iteration limit, tolerance or pc");
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (d->mom) {
    destroy_cg(d->mom);
    d->mom = nullptr;
  }
  d->momarena.release();
  d->theta = 0.0;
  if (theta < std::numeric_limits<double>::epsilon()) return XG_OK;  // explicit prediction
  const int64_t n = d->n;
  if (ntet <= 0 || !inpoel) return fail(c, XG_ERR_ARG, "chocg_set_theta: no tetrahedra");
  for (int64_t k = 0; k < ntet * 4; ++k)
    if (inpoel[k] >= static_cast<uint64_t>(n))
      return fail(c, XG_ERR_ARG, "chocg_set_theta: tetrahedron node out of range");
  // the node pattern (every pair of nodes sharing a tetrahedron, and the
  // diagonal), columns sorted
  std::vector<std::vector<int64_t>> nb(n);
  for (int64_t e = 0; e < ntet; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) nb[inpoel[e * 4 + a]].push_back(int64_t(inpoel[e * 4 + b]));
  std::vector<uint64_t> ia(n + 1, 0);
  std::vector<int64_t> ja;
  for (int64_t i = 0; i < n; ++i) {
    auto& v = nb[i];
    v.push_back(i);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    ia[i + 1] = ia[i] + v.size();
    ja.insert(ja.end(), v.begin(), v.end());
    std::vector<int64_t>().swap(v);
  }
  // stiffness grad_a.grad_b / J / 6 and consistent mass J/120 (1 + d_ab),
  // summed over the elements in element order (ChoCG::lhs)
  std::vector<double> K(ja.size(), 0.0), M(ja.size(), 0.0);
  const double* X = d->xyz_host.data();
  const double* Y = X + n;
  const double* Z = Y + n;
  auto pos = [&](int64_t i, int64_t j) {
    return static_cast<int64_t>(std::lower_bound(ja.begin() + ia[i], ja.begin() + ia[i + 1], j) -
                                ja.begin());
  };
  for (int64_t e = 0; e < ntet; ++e) {
    const uint64_t* N = inpoel + e * 4;
    const double ba[3] = {X[N[1]] - X[N[0]], Y[N[1]] - Y[N[0]], Z[N[1]] - Z[N[0]]};
    const double ca[3] = {X[N[2]] - X[N[0]], Y[N[2]] - Y[N[0]], Z[N[2]] - Z[N[0]]};
    const double da[3] = {X[N[3]] - X[N[0]], Y[N[3]] - Y[N[0]], Z[N[3]] - Z[N[0]]};
    auto cross = [](const double u[3], const double v[3], double w[3]) {
      w[0] = u[1] * v[2] - v[1] * u[2];
      w[1] = u[2] * v[0] - v[2] * u[0];
      w[2] = u[0] * v[1] - v[0] * u[1];
    };
    double g[4][3];
    cross(ca, da, g[1]);
    cross(da, ba, g[2]);
    cross(ba, ca, g[3]);
    for (int k = 0; k < 3; ++k) g[0][k] = -g[1][k] - g[2][k] - g[3][k];
    const double J = ba[0] * g[1][0] + ba[1] * g[1][1] + ba[2] * g[1][2];
    if (!(J > 0.0)) return fail(c, XG_ERR_ARG, "chocg_set_theta: element Jacobian non-positive");
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) {
        const int64_t q = pos(int64_t(N[a]), int64_t(N[b]));
        M[q] += J / 120.0 * ((a == b) ? 2.0 : 1.0);
        K[q] += (g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2]) / J / 6.0;
      }
  }
  // three components per node: row 3i + c, columns 3j + c
  std::vector<uint64_t> ia3(n * 3 + 1, 0), ja3;
  std::vector<double> K3, M3;
  ja3.reserve(ja.size() * 3);
  K3.reserve(ja.size() * 3);
  M3.reserve(ja.size() * 3);
  for (int64_t i = 0; i < n; ++i)
    for (int cc = 0; cc < 3; ++cc) {
      for (uint64_t k = ia[i]; k < ia[i + 1]; ++k) {
        ja3.push_back(uint64_t(ja[k]) * 3 + cc);
        K3.push_back(K[k]);
        M3.push_back(M[k]);
      }
      ia3[i * 3 + cc + 1] = ja3.size();
    }
  // the momentum CG system, set up while it stands in for the context's
  CGDev* const saved = c->cg;
  c->cg = nullptr;
  rc = xg_cg_setup(c, n * 3, ia3.data(), ja3.data(), K3.data(), 0);
  d->mom = c->cg;
  if (rc == XG_OK) {
    const int64_t nent = cg_nent(c);
    for (int pass = 0; pass < 2; ++pass) {
      Arena& A = d->momarena;
      A.plan(d->baseK, nent);
      A.plan(d->baseM, nent);
      A.plan(d->R3, n * 3);
      A.plan(d->b3, n * 3);
      if (pass == 0) {
        const cudaError_t ce = A.reserve();
        if (ce != cudaSuccess) {
          rc = fail(c, XG_ERR_CUDA, std::string("chocg_set_theta: ") + cudaGetErrorString(ce));
          break;
        }
      }
    }
    if (rc == XG_OK) rc = cg_to_sell(c, ia3.data(), K3.data(), d->baseK);
    if (rc == XG_OK) rc = cg_to_sell(c, ia3.data(), M3.data(), d->baseM);
  }
  c->cg = saved;
  if (rc) {
    if (d->mom) destroy_cg(d->mom);
    d->mom = nullptr;
    d->momarena.release();
    return rc;
  }
  d->theta = theta;
  d->mom_pc = mom_pc;
  d->mom_iter = mom_iter;
  d->mom_tol = mom_tol;
  d->mommask_up = false;
  d->last_mit = 0;
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_chocg_momentum_its(xg_ctx* c, int64_t* it) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (it) *it = d->last_mit;
  return XG_OK;
}

int xg_chocg_set_bc(xg_ctx* c, int64_t ndir, const uint64_t* dirnodes, const int32_t* dirmask,
                    const double* dirvals, int64_t nsym, const uint64_t* symnodes,
                    const double* symnorms, int64_t nnoslip, const uint64_t* noslipnodes,
                    int64_t npdir, const uint64_t* pdirnodes, const double* pdirvals) {
  XG_HOST_TRY
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if ((ndir && (!dirnodes || !dirmask || !dirvals)) || (nsym && (!symnodes || !symnorms)) ||
      (nnoslip && !noslipnodes) || (npdir && (!pdirnodes || !pdirvals)) || ndir < 0 ||
      nsym < 0 || nnoslip < 0 || npdir < 0)
    return fail(c, XG_ERR_ARG, "chocg_set_bc: bad BC arrays");
  const int64_t n = d->n;
  auto bad = [&](uint64_t id) { return id >= static_cast<uint64_t>(n); };
  // BC program: one entry per distinct BC node, in node order
  std::vector<int32_t> dirof(n, -1), noslip(n, 0);
  std::vector<std::vector<int32_t>> symof;
  for (int64_t k = 0; k < ndir; ++k) {
    if (bad(dirnodes[k])) return fail(c, XG_ERR_ARG, "chocg_set_bc: Dirichlet node out of range");
    dirof[dirnodes[k]] = static_cast<int32_t>(k);
  }
  for (int64_t k = 0; k < nnoslip; ++k) {
    if (bad(noslipnodes[k])) return fail(c, XG_ERR_ARG, "chocg_set_bc: noslip node out of range");
    noslip[noslipnodes[k]] = 1;
  }
  std::vector<int64_t> symcount(n, 0);
  for (int64_t k = 0; k < nsym; ++k) {
    if (bad(symnodes[k])) return fail(c, XG_ERR_ARG, "chocg_set_bc: symmetry node out of range");
    ++symcount[symnodes[k]];
  }
  std::vector<int32_t> node, dir, nsl, symp(1, 0);
  std::vector<double> symn;
  std::vector<std::vector<int64_t>> symlist(n);
  for (int64_t k = 0; k < nsym; ++k) symlist[symnodes[k]].push_back(k);
  for (int64_t p = 0; p < n; ++p) {
    if (dirof[p] < 0 && !noslip[p] && symcount[p] == 0) continue;
    node.push_back(static_cast<int32_t>(p));
    dir.push_back(dirof[p]);
    nsl.push_back(noslip[p]);
    for (int64_t k : symlist[p])
      for (int a = 0; a < 3; ++a) symn.push_back(symnorms[k * 3 + a]);
    symp.push_back(static_cast<int32_t>(symn.size() / 3));
  }
  d->bcarena.release();
  d->nbc = static_cast<int64_t>(node.size());
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->bcarena;
    A.plan(d->bcnode, std::max<size_t>(1, node.size()));
    A.plan(d->bcdir, std::max<size_t>(1, dir.size()));
    A.plan(d->bcnoslip, std::max<size_t>(1, nsl.size()));
    A.plan(d->bcsymp, symp.size());
    A.plan(d->symn, std::max<size_t>(1, symn.size()));
    A.plan(d->dirmask, std::max<int64_t>(1, ndir * 3));
    A.plan(d->dirval, std::max<int64_t>(1, ndir * 3));
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  XG_CUDA(c, up(d->bcnode, node.data(), node.size() * 4));
  XG_CUDA(c, up(d->bcdir, dir.data(), dir.size() * 4));
  XG_CUDA(c, up(d->bcnoslip, nsl.data(), nsl.size() * 4));
  XG_CUDA(c, up(d->bcsymp, symp.data(), symp.size() * 4));
  XG_CUDA(c, up(d->symn, symn.data(), symn.size() * 8));
  XG_CUDA(c, up(d->dirmask, dirmask, ndir * 3 * 4));
  XG_CUDA(c, up(d->dirval, dirvals, ndir * 3 * 8));
  // Dirichlet rows of the theta-implicit momentum system (ChoCG::solve,
  // ChoCG.cpp:1580-1600): the masked velocity components of the Dirichlet
  // nodes and all three of the noslip nodes, increment 0
  d->mommask.assign(n * 3, 0);
  for (int64_t k = 0; k < ndir; ++k)
    for (int cc = 0; cc < 3; ++cc)
      if (dirmask[k * 3 + cc]) d->mommask[dirnodes[k] * 3 + cc] = 1;
  for (int64_t k = 0; k < nnoslip; ++k)
    for (int cc = 0; cc < 3; ++cc) d->mommask[noslipnodes[k] * 3 + cc] = 1;
  d->mommask_up = false;
  // pressure Dirichlet nodes on the context's CG system
  if (cg_rows(c) != n)
    return fail(c, XG_ERR_STATE, "chocg_set_bc: set up the pressure matrix (xg_cg_setup) first");
  std::vector<uint8_t> mask(n, 0);
  std::vector<double> val(n, 0.0);
  for (int64_t k = 0; k < npdir; ++k) {
    if (bad(pdirnodes[k]))
      return fail(c, XG_ERR_ARG, "chocg_set_bc: pressure Dirichlet node out of range");
    mask[pdirnodes[k]] = 1;
    val[pdirnodes[k]] = pdirvals[k];
  }
  rc = cg_set_dirichlet(c, mask.data(), val.data());
  if (rc) return rc;
  d->pdir_set = true;
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_chocg_set_state(xg_ctx* c, const double* u, const double* p, double t) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!u) return fail(c, XG_ERR_ARG, "chocg_set_state: null velocity");
  const int64_t n = d->n;
  XG_CUDA(c, cudaMemcpyAsync(d->stage, u, n * 3 * 8, cudaMemcpyHostToDevice, c->stream));
  k_aos_soa<<<blocks_for(n * 3, kBlock), kBlock, 0, c->stream>>>(n, 3, d->stage, d->u);
  XG_CHECK_LAUNCH(c);
  if (p)
    XG_CUDA(c, cudaMemcpyAsync(d->pr, p, n * 8, cudaMemcpyHostToDevice, c->stream));
  else
    XG_CUDA(c, cudaMemsetAsync(d->pr, 0, n * 8, c->stream));
  XG_CUDA(c, cudaMemsetAsync(d->pgrad, 0, n * 3 * 8, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  d->t = t;
  d->ready = false;
  return XG_OK;
}

int xg_chocg_get_state(xg_ctx* c, double* u, double* p, double* t) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  const int64_t n = d->n;
  if (u) {
    k_soa_aos<<<blocks_for(n * 3, kBlock), kBlock, 0, c->stream>>>(n, 3, d->u, d->stage);
    XG_CHECK_LAUNCH(c);
    XG_CUDA(c, cudaMemcpyAsync(u, d->stage, n * 3 * 8, cudaMemcpyDeviceToHost, c->stream));
  }
  if (p) XG_CUDA(c, cudaMemcpyAsync(p, d->pr, n * 8, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (t) *t = d->t;
  return XG_OK;
}

int xg_chocg_init(xg_ctx* c, int64_t* it) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, true);
  if (rc) return rc;
  if (!d->pdir_set) return fail(c, XG_ERR_STATE, "chocg_init: no BCs (xg_chocg_set_bc)");
  // m_np = 0 (ChoCG::merge -> div -> pinit -> psolve -> sgrad -> psolved):
  // BCs, divergence without stabilisation, projection with dt = 1
  rc = launch_bc(c, d, d->u, 0);
  if (rc) return rc;
  rc = cg_zero_solution(c);
  if (rc) return rc;
  rc = launch_div(c, d, d->u, 0.0, 0, 0);
  if (rc) return rc;
  rc = pressure_solve(c, d, 0);
  if (rc) return rc;
  rc = launch_grad<1, GRAD_PROJECT>(c, d, cg_solution_device(c), nullptr, 1.0, 0);
  if (rc) return rc;
  rc = launch_bc(c, d, d->u, 0);
  if (rc) return rc;
  // m_np = 1 (velgrad -> flux -> div -> pinit -> psolve -> psolved): the
  // divergence of the volume-divided momentum flux with symmetry applied
  rc = launch_grad<3, GRAD_DIVIDE>(c, d, d->u, d->vgrad);
  if (rc) return rc;
  two_pass<k_cflux<false>, k_cflux<true>>(c->stream, d->n, d->nbn, d->n, adj_of(d), d->u,
                                          d->vgrad, bnd_of(d), d->vol, d->prm.mu, 1, d->flx);
  XG_CHECK_LAUNCH(c);
  rc = launch_bc(c, d, d->flx, 1);
  if (rc) return rc;
  rc = launch_div(c, d, d->flx, 0.0, 0, 0);
  if (rc) return rc;
  rc = pressure_solve(c, d, 0);
  if (rc) return rc;
  // m_np = 2: initial pressure and its gradient
  XG_CUDA(c, cudaMemcpyAsync(d->pr, cg_solution_device(c), d->n * 8, cudaMemcpyDeviceToDevice,
                             c->stream));
  rc = launch_grad<1, GRAD_DIVIDE>(c, d, d->pr, d->pgrad);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  d->ready = true;
  if (it) *it = d->last_it;
  return XG_OK;
}

int xg_chocg_run(xg_ctx* c, int64_t nstep, double* dts, int64_t* its, float* ms) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, true);
  if (rc) return rc;
  if (!d->ready) return fail(c, XG_ERR_STATE, "chocg_run before chocg_init");
  const int64_t n = d->n;
  static const double rkc[4][4] = {{1.0, 0, 0, 0},
                                   {1.0 / 2.0, 1.0, 0, 0},
                                   {1.0 / 3.0, 1.0 / 2.0, 1.0, 0},
                                   {1.0 / 4.0, 1.0 / 3.0, 1.0 / 2.0, 1.0}};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ms) {
    XG_CUDA(c, cudaEventCreate(&e0));
    XG_CUDA(c, cudaEventCreate(&e1));
    XG_CUDA(c, cudaEventRecord(e0, c->stream));
  }
  int status = XG_OK;
  for (int64_t st = 0; st < nstep; ++st) {
    double dt = 0.0;
    rc = step_dt(c, d, &dt);
    if (rc) return rc;
    if (dt < DBL_EPSILON) {
      status = XG_ERR_BLOWUP;
      fail(c, XG_ERR_BLOWUP, "chocg: dt below eps");
      break;
    }
    // momentum prediction (ChoCG::rhs -> solve -> pred -> corr, per stage)
    for (int k = 0; k < d->prm.rk; ++k) {
      if (d->mom && k + 1 == d->prm.rk) {
        // semi-implicit last stage: the stage rhs, then the momentum solve
        rc = launch_rhs(c, d, d->u, 0.0, 0, nullptr, d->R3);
        if (rc) return rc;
        if (k == 0) XG_CUDA(c, cudaMemcpyAsync(d->un, d->u, n * 3 * 8, cudaMemcpyDeviceToDevice,
                                              c->stream));
        rc = momentum_solve(c, d, dt);
        if (rc) return rc;
      } else {
        rc = launch_rhs(c, d, d->u, rkc[d->prm.rk - 1][k] * dt, k == 0, d->u2, nullptr);
        if (rc) return rc;
        std::swap(d->u, d->u2);
      }
      rc = launch_bc(c, d, d->u, 0);
      if (rc) return rc;
      if (d->prm.flux == XG_DAMP4) {
        rc = launch_grad<3, GRAD_DIVIDE>(c, d, d->u, d->vgrad);
        if (rc) return rc;
      }
    }
    // pressure increment (ChoCG::div -> pinit -> psolve) and projection
    // (sgrad -> psolved -> pgrad)
    rc = launch_div(c, d, d->u, dt, 1, 1);
    if (rc) return rc;
    rc = pressure_solve(c, d, 1);
    if (rc) return rc;
    rc = launch_grad<1, GRAD_PROJECT>(c, d, cg_solution_device(c), nullptr, dt, 1);
    if (rc) return rc;
    rc = launch_bc(c, d, d->u, 0);
    if (rc) return rc;
    rc = launch_grad<1, GRAD_DIVIDE>(c, d, d->pr, d->pgrad);
    if (rc) return rc;
    d->t += dt;
    if (dts) dts[st] = dt;
    if (its) its[st] = d->last_it;
  }
  if (ms) {
    XG_CUDA(c, cudaEventRecord(e1, c->stream));
    XG_CUDA(c, cudaEventSynchronize(e1));
    XG_CUDA(c, cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return status;
}

int xg_chocg_fields(xg_ctx* c, int what, double* out) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!out) return fail(c, XG_ERR_ARG, "chocg_fields: null output");
  const int64_t n = d->n;
  const double* src = nullptr;
  int nc = 1;
  switch (what) {
    case 0: src = d->un; nc = 3; break;
    case 1: src = d->pgrad; nc = 3; break;
    case 2: src = d->vgrad; nc = 9; break;
    case 3: src = d->div; break;
    case 4:
      src = cg_solution_device(c);
      if (!src || cg_rows(c) != n) return fail(c, XG_ERR_STATE, "chocg_fields: no pressure solve");
      break;
    default: return fail(c, XG_ERR_ARG, "chocg_fields: unknown field");
  }
  k_soa_aos<<<blocks_for(n * nc, kBlock), kBlock, 0, c->stream>>>(n, nc, src, d->stage);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(out, d->stage, n * nc * 8, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

// ---- drop-ins: host node-major arrays through per-call device buffers (the
// device state of xg_chocg_run is left untouched)

int xg_chorin_div(xg_ctx* c, const double* U, const double* P, const double* G, double dt,
                  int stab, double* D) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!U || !P || !G || !D) return fail(c, XG_ERR_ARG, "chorin_div: null array");
  const int64_t n = d->n;
  double *u, *p, *g, *out;
  Arena A;
  for (int pass = 0; pass < 2; ++pass) {
    A.plan(u, 3 * n);
    A.plan(p, n);
    A.plan(g, 3 * n);
    A.plan(out, 3 * n);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(out, U, n * 24, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, out, u);
  XG_CUDA(c, cudaMemcpyAsync(out, G, n * 24, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, out, g);
  XG_CUDA(c, cudaMemcpyAsync(p, P, n * 8, cudaMemcpyHostToDevice, s));
  two_pass<k_cdiv<false>, k_cdiv<true>>(s, n, d->nbn, n, adj_of(d), u, p, g, bnd_of(d), dt, stab,
                                        0, out);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(D, out, n * 8, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

int xg_chorin_grad(xg_ctx* c, const double* S, double* Gout) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!S || !Gout) return fail(c, XG_ERR_ARG, "chorin_grad: null array");
  const int64_t n = d->n;
  double *sv, *g, *out;
  Arena A;
  for (int pass = 0; pass < 2; ++pass) {
    A.plan(sv, n);
    A.plan(g, 3 * n);
    A.plan(out, 3 * n);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(sv, S, n * 8, cudaMemcpyHostToDevice, s));
  two_pass<k_cgrad<1, GRAD_RAW, false>, k_cgrad<1, GRAD_RAW, true>>(
      s, n, d->nbn, n, adj_of(d), sv, bnd_of(d), d->vol, g, 0.0, 0, nullptr, nullptr);
  XG_CHECK_LAUNCH(c);
  k_soa_aos<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, g, out);
  XG_CUDA(c, cudaMemcpyAsync(Gout, out, n * 24, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

int xg_chorin_vgrad(xg_ctx* c, const double* U, double* Gout) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!U || !Gout) return fail(c, XG_ERR_ARG, "chorin_vgrad: null array");
  const int64_t n = d->n;
  double *u, *g, *out;
  Arena A;
  for (int pass = 0; pass < 2; ++pass) {
    A.plan(u, 3 * n);
    A.plan(g, 9 * n);
    A.plan(out, 9 * n);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(out, U, n * 24, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, out, u);
  two_pass<k_cgrad<3, GRAD_RAW, false>, k_cgrad<3, GRAD_RAW, true>>(
      s, n, d->nbn, n, adj_of(d), u, bnd_of(d), d->vol, g, 0.0, 0, nullptr, nullptr);
  XG_CHECK_LAUNCH(c);
  k_soa_aos<<<blocks_for(n * 9, kBlock), kBlock, 0, s>>>(n, 9, g, out);
  XG_CUDA(c, cudaMemcpyAsync(Gout, out, n * 72, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

int xg_chorin_flux(xg_ctx* c, const double* U, const double* G, double* F) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!U || !G || !F) return fail(c, XG_ERR_ARG, "chorin_flux: null array");
  const int64_t n = d->n;
  double *u, *g, *f, *tmp;
  Arena A;
  for (int pass = 0; pass < 2; ++pass) {
    A.plan(u, 3 * n);
    A.plan(g, 9 * n);
    A.plan(f, 3 * n);
    A.plan(tmp, 9 * n);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(tmp, U, n * 24, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, tmp, u);
  XG_CUDA(c, cudaMemcpyAsync(tmp, G, n * 72, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 9, kBlock), kBlock, 0, s>>>(n, 9, tmp, g);
  two_pass<k_cflux<false>, k_cflux<true>>(s, n, d->nbn, n, adj_of(d), u, g, bnd_of(d), d->vol,
                                          d->prm.mu, 0, f);
  XG_CHECK_LAUNCH(c);
  k_soa_aos<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, f, tmp);
  XG_CUDA(c, cudaMemcpyAsync(F, tmp, n * 24, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

int xg_chorin_rhs(xg_ctx* c, const double* P, const double* U, const double* G, double* R) {
  ChoCGDev* d = nullptr;
  int rc = get_ctx(c, &d, false);
  if (rc) return rc;
  if (!P || !U || !G || !R) return fail(c, XG_ERR_ARG, "chorin_rhs: null array");
  const int64_t n = d->n;
  double *u, *g, *p, *r, *tmp;
  Arena A;
  for (int pass = 0; pass < 2; ++pass) {
    A.plan(u, 3 * n);
    A.plan(g, 9 * n);
    A.plan(p, n);
    A.plan(r, 3 * n);
    A.plan(tmp, 9 * n);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(tmp, U, n * 24, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, tmp, u);
  XG_CUDA(c, cudaMemcpyAsync(tmp, G, n * 72, cudaMemcpyHostToDevice, s));
  k_aos_soa<<<blocks_for(n * 9, kBlock), kBlock, 0, s>>>(n, 9, tmp, g);
  XG_CUDA(c, cudaMemcpyAsync(p, P, n * 8, cudaMemcpyHostToDevice, s));
  const AdvPrm ap = adv_of(d);
  if (d->prm.flux == XG_DAMP4)
    two_pass<k_crhs<true, false>, k_crhs<true, true>>(s, n, d->nbn, n, adj_of(d), u, g, p,
                                                       bnd_of(d), ap, d->vol, 0.0, 0, nullptr,
                                                       nullptr, r);
  else
    two_pass<k_crhs<false, false>, k_crhs<false, true>>(s, n, d->nbn, n, adj_of(d), u, g, p,
                                                         bnd_of(d), ap, d->vol, 0.0, 0, nullptr,
                                                         nullptr, r);
  XG_CHECK_LAUNCH(c);
  k_soa_aos<<<blocks_for(n * 3, kBlock), kBlock, 0, s>>>(n, 3, r, tmp);
  XG_CUDA(c, cudaMemcpyAsync(R, tmp, n * 24, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

}  // extern "C"
