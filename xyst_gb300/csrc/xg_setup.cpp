// Host-side operator setup: the caller side of xg_riecg_setup.  Builds, from
// a tetrahedron mesh, the arrays RieCG computes once per mesh (nodal
// volumes, domain edge integrals, boundary point normals) and a locality
// renumbering.  Plain C++; linear or n log n in the mesh size.  The edge
// integrals run on all host cores, each thread owning whole rows of the edge
// table and summing every edge's element contributions in element order, so
// the result is the serial one bit for bit.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <queue>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/xg.h"

// Every entry point's body runs inside XG_HOST_TRY ... XG_HOST_CATCH, so an
// exception (std::bad_alloc on a large mesh, std::system_error) becomes
// XG_ERR_HOST instead of crossing the C ABI.
#define XG_HOST_TRY try {
#define XG_HOST_CATCH \
  }                   \
  catch (...) {       \
    return XG_ERR_HOST; \
  }

namespace {

// fn(i) for i in [0, n) on the host's cores, in contiguous chunks.
template <class Fn>
void parallel_rows(int64_t n, Fn fn) {
  unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = std::min<int64_t>(hw ? hw : 1, 64);
  if (n < 8192) nt = 1;
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  const int64_t chunk = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  th.reserve(static_cast<size_t>(nt));
  int64_t t = 0;
  try {
    for (; t < nt; ++t) {
      const int64_t b = t * chunk, e = std::min(n, b + chunk);
      if (b >= e) break;
      th.emplace_back([b, e, &fn] {
        for (int64_t i = b; i < e; ++i) fn(i);
      });
    }
  } catch (const std::system_error&) {
    // thread creation refused (rlimits, containers): the chunks not yet
    // handed out run on this thread
    for (; t < nt; ++t) {
      const int64_t b = t * chunk, e = std::min(n, b + chunk);
      for (int64_t i = b; i < e; ++i) fn(i);
    }
  }
  for (auto& x : th) x.join();
}

// Points surrounding points as CSR (sorted, unique, no self) from tets.
void psup(int64_t n, int64_t nelem, const uint64_t* inpoel, std::vector<int64_t>& ptr,
          std::vector<int64_t>& adj) {
  std::vector<int64_t> cnt(n + 1, 0);
  for (int64_t e = 0; e < nelem; ++e)
    for (int a = 0; a < 4; ++a) cnt[inpoel[e * 4 + a] + 1] += 3;
  for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int64_t> tmp(cnt[n]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int64_t e = 0; e < nelem; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        if (a != b) tmp[fill[inpoel[e * 4 + a]]++] = static_cast<int64_t>(inpoel[e * 4 + b]);
  std::vector<int64_t> ucnt(n);
  parallel_rows(n, [&](int64_t i) {
    auto b = tmp.begin() + cnt[i], en = tmp.begin() + cnt[i + 1];
    std::sort(b, en);
    ucnt[i] = std::unique(b, en) - b;
  });
  ptr.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) ptr[i + 1] = ptr[i] + ucnt[i];
  adj.assign(ptr[n], 0);
  parallel_rows(n, [&](int64_t i) {
    std::copy(tmp.begin() + cnt[i], tmp.begin() + cnt[i] + ucnt[i], adj.begin() + ptr[i]);
  });
}

inline void cross(double ax, double ay, double az, double bx, double by, double bz, double& rx,
                  double& ry, double& rz) {
  rx = ay * bz - by * az;
  ry = az * bx - bz * ax;
  rz = ax * by - bx * ay;
}

}  // namespace

extern "C" {

// Reverse Cuthill-McKee: BFS from a minimum-degree node of each connected
// component, visiting neighbours in increasing degree, then reversed.
int xg_mesh_rcm(int64_t npoin, int64_t nelem, const uint64_t* inpoel, uint64_t* new_of_old) {
  XG_HOST_TRY
  if (npoin <= 0 || nelem < 0 || !inpoel || !new_of_old) return XG_ERR_ARG;
  for (int64_t i = 0; i < nelem * 4; ++i)
    if (inpoel[i] >= static_cast<uint64_t>(npoin)) return XG_ERR_ARG;
  std::vector<int64_t> ptr, adj;
  psup(npoin, nelem, inpoel, ptr, adj);
  std::vector<int64_t> deg(npoin);
  for (int64_t i = 0; i < npoin; ++i) deg[i] = ptr[i + 1] - ptr[i];
  std::vector<int64_t> order;
  order.reserve(npoin);
  std::vector<char> seen(npoin, 0);
  std::vector<int64_t> byDeg(npoin);
  std::iota(byDeg.begin(), byDeg.end(), 0);
  std::stable_sort(byDeg.begin(), byDeg.end(),
                   [&](int64_t a, int64_t b) { return deg[a] < deg[b]; });
  std::vector<int64_t> nb;
  for (int64_t root : byDeg) {
    if (seen[root]) continue;
    size_t head = order.size();
    order.push_back(root);
    seen[root] = 1;
    while (head < order.size()) {
      int64_t p = order[head++];
      nb.clear();
      for (int64_t j = ptr[p]; j < ptr[p + 1]; ++j)
        if (!seen[adj[j]]) nb.push_back(adj[j]);
      std::stable_sort(nb.begin(), nb.end(),
                       [&](int64_t a, int64_t b) { return deg[a] < deg[b]; });
      for (int64_t q : nb) {
        seen[q] = 1;
        order.push_back(q);
      }
    }
  }
  for (int64_t k = 0; k < npoin; ++k)
    new_of_old[order[k]] = static_cast<uint64_t>(npoin - 1 - k);
  return XG_OK;
  XG_HOST_CATCH
}

int xg_mesh_vol(int64_t npoin, const double* coord, int64_t nelem, const uint64_t* inpoel,
                double* vol) {
  XG_HOST_TRY
  if (npoin <= 0 || !coord || !inpoel || !vol) return XG_ERR_ARG;
  const double *x = coord, *y = coord + npoin, *z = coord + 2 * npoin;
  std::fill(vol, vol + npoin, 0.0);
  for (int64_t e = 0; e < nelem; ++e) {
    const uint64_t* N = inpoel + e * 4;
    for (int a = 0; a < 4; ++a)
      if (N[a] >= static_cast<uint64_t>(npoin)) return XG_ERR_ARG;
    double ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
    double ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
    double da[3] = {x[N[3]] - x[N[0]], y[N[3]] - y[N[0]], z[N[3]] - z[N[0]]};
    double cx, cy, cz;
    cross(ca[0], ca[1], ca[2], da[0], da[1], da[2], cx, cy, cz);
    double J = (ba[0] * cx + ba[1] * cy + ba[2] * cz) / 24.0;
    if (!(J > 0)) return XG_ERR_ARG;
    for (int a = 0; a < 4; ++a) vol[N[a]] += J;
  }
  return XG_OK;
  XG_HOST_CATCH
}

int xg_mesh_edges(int64_t npoin, const double* coord, int64_t nelem, const uint64_t* inpoel,
                  const uint64_t* gid, int ncoef, int64_t cap, int64_t* nedge, uint64_t* edges,
                  double* dint) {
  XG_HOST_TRY
  if (npoin <= 0 || !coord || !inpoel || !nedge || (ncoef != 3 && ncoef != 5)) return XG_ERR_ARG;
  const double *x = coord, *y = coord + npoin, *z = coord + 2 * npoin;
  auto G = [&](uint64_t p) { return gid ? gid[p] : p; };
  // rows keyed by the smaller-gid end, holding the larger-gid ends
  std::vector<int64_t> cnt(npoin + 1, 0);
  static const int lpoed[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  for (int64_t e = 0; e < nelem; ++e)
    for (int k = 0; k < 6; ++k) {
      uint64_t a = inpoel[e * 4 + lpoed[k][0]], b = inpoel[e * 4 + lpoed[k][1]];
      if (a >= uint64_t(npoin) || b >= uint64_t(npoin)) return XG_ERR_ARG;
      ++cnt[(G(a) < G(b) ? a : b) + 1];
    }
  for (int64_t i = 0; i < npoin; ++i) cnt[i + 1] += cnt[i];
  std::vector<uint64_t> col(cnt[npoin]);
  {
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t e = 0; e < nelem; ++e)
      for (int k = 0; k < 6; ++k) {
        uint64_t a = inpoel[e * 4 + lpoed[k][0]], b = inpoel[e * 4 + lpoed[k][1]];
        if (G(a) < G(b))
          col[fill[a]++] = b;
        else
          col[fill[b]++] = a;
      }
  }
  // each row's distinct neighbours, sorted by gid (rows in parallel)
  std::vector<int64_t> ucnt(npoin);
  parallel_rows(npoin, [&](int64_t i) {
    auto b = col.begin() + cnt[i], en = col.begin() + cnt[i + 1];
    std::sort(b, en, [&](uint64_t p, uint64_t q) { return G(p) < G(q); });
    ucnt[i] = std::unique(b, en) - b;
  });
  std::vector<int64_t> rptr(npoin + 1, 0);
  for (int64_t i = 0; i < npoin; ++i) rptr[i + 1] = rptr[i] + ucnt[i];
  std::vector<uint64_t> rcol(rptr[npoin]);
  parallel_rows(npoin, [&](int64_t i) {
    std::copy(col.begin() + cnt[i], col.begin() + cnt[i] + ucnt[i], rcol.begin() + rptr[i]);
  });
  const int64_t ne = static_cast<int64_t>(rcol.size());
  *nedge = ne;
  if (cap < ne) return XG_OK;
  if (!edges || !dint) return XG_ERR_ARG;
  // the elements of every node in increasing element id
  std::vector<int64_t> eptr(npoin + 1, 0);
  for (int64_t e = 0; e < nelem; ++e)
    for (int a = 0; a < 4; ++a) ++eptr[inpoel[e * 4 + a] + 1];
  for (int64_t i = 0; i < npoin; ++i) eptr[i + 1] += eptr[i];
  std::vector<int64_t> elist(eptr[npoin]);
  {
    std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
    for (int64_t e = 0; e < nelem; ++e)
      for (int a = 0; a < 4; ++a) elist[fill[inpoel[e * 4 + a]]++] = e;
  }
  // row r sums, element by element in increasing id, the contributions of
  // the edges it owns (its smaller-gid end): every edge's sum in the element
  // order of the serial element loop
  std::vector<double> D(static_cast<size_t>(ne) * ncoef, 0.0);
  parallel_rows(npoin, [&](int64_t r) {
    for (int64_t k = eptr[r]; k < eptr[r + 1]; ++k) {
      const uint64_t* N = inpoel + elist[k] * 4;
      double ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
      double ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
      double da[3] = {x[N[3]] - x[N[0]], y[N[3]] - y[N[0]], z[N[3]] - z[N[0]]};
      double g[4][3];
      cross(ca[0], ca[1], ca[2], da[0], da[1], da[2], g[1][0], g[1][1], g[1][2]);
      cross(da[0], da[1], da[2], ba[0], ba[1], ba[2], g[2][0], g[2][1], g[2][2]);
      cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], g[3][0], g[3][1], g[3][2]);
      for (int i = 0; i < 3; ++i) g[0][i] = -g[1][i] - g[2][i] - g[3][i];
      double J = ba[0] * g[1][0] + ba[1] * g[1][1] + ba[2] * g[1][2];
      for (int kk = 0; kk < 6; ++kk) {
        int p = lpoed[kk][0], q = lpoed[kk][1];
        uint64_t a = N[p], b = N[q];
        double sig = 1.0;
        if (G(a) > G(b)) {
          std::swap(a, b);
          sig = -1.0;
        }
        if (a != static_cast<uint64_t>(r)) continue;
        auto beg = rcol.begin() + rptr[a], en = rcol.begin() + rptr[a + 1];
        auto it =
            std::lower_bound(beg, en, b, [&](uint64_t u, uint64_t v) { return G(u) < G(v); });
        double* n = &D[static_cast<size_t>(it - rcol.begin()) * ncoef];
        n[0] += sig * (g[p][0] - g[q][0]) / 48.0;
        n[1] += sig * (g[p][1] - g[q][1]) / 48.0;
        n[2] += sig * (g[p][2] - g[q][2]) / 48.0;
        if (ncoef == 5) {
          n[3] += J / 120.0;
          n[4] += (g[p][0] * g[q][0] + g[p][1] * g[q][1] + g[p][2] * g[q][2]) / J / 6.0;
        }
      }
    }
  });
  // emit in (gid, gid) order
  std::vector<int64_t> rows(npoin);
  std::iota(rows.begin(), rows.end(), 0);
  if (gid) std::sort(rows.begin(), rows.end(), [&](int64_t a, int64_t b) { return gid[a] < gid[b]; });
  std::vector<int64_t> opos(npoin + 1, 0);
  for (int64_t k = 0; k < npoin; ++k) opos[k + 1] = opos[k] + (rptr[rows[k] + 1] - rptr[rows[k]]);
  parallel_rows(npoin, [&](int64_t k) {
    const int64_t a = rows[k];
    int64_t o = opos[k];
    for (int64_t j = rptr[a]; j < rptr[a + 1]; ++j, ++o) {
      edges[o * 2 + 0] = static_cast<uint64_t>(a);
      edges[o * 2 + 1] = rcol[j];
      std::memcpy(dint + o * ncoef, &D[static_cast<size_t>(j) * ncoef], sizeof(double) * ncoef);
    }
  });
  return XG_OK;
  XG_HOST_CATCH
}

int xg_mesh_bnorm(int64_t npoin, const double* coord, int64_t nface, const uint64_t* faces,
                  int64_t nnode, const uint64_t* nodes, double* norms) {
  XG_HOST_TRY
  if (npoin <= 0 || !coord || (nface && !faces) || (nnode && (!nodes || !norms)))
    return XG_ERR_ARG;
  const double *x = coord, *y = coord + npoin, *z = coord + 2 * npoin;
  std::vector<double> acc(static_cast<size_t>(npoin) * 4, 0.0);
  std::vector<char> on(npoin, 0);
  for (int64_t f = 0; f < nface; ++f) {
    const uint64_t* N = faces + f * 3;
    for (int a = 0; a < 3; ++a)
      if (N[a] >= uint64_t(npoin)) return XG_ERR_ARG;
    double ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
    double ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
    double n[3];
    cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], n[0], n[1], n[2]);
    double A2 = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= A2;
    n[1] /= A2;
    n[2] /= A2;
    double c[3] = {(x[N[0]] + x[N[1]] + x[N[2]]) / 3.0, (y[N[0]] + y[N[1]] + y[N[2]]) / 3.0,
                   (z[N[0]] + z[N[1]] + z[N[2]]) / 3.0};
    for (int i = 0; i < 3; ++i) {
      uint64_t p = N[i];
      double r = 1.0 / ((c[0] - x[p]) * (c[0] - x[p]) + (c[1] - y[p]) * (c[1] - y[p]) +
                        (c[2] - z[p]) * (c[2] - z[p]));
      double* v = &acc[p * 4];
      v[0] += r * n[0];
      v[1] += r * n[1];
      v[2] += r * n[2];
      v[3] += r;
      on[p] = 1;
    }
  }
  for (int64_t i = 0; i < nnode; ++i) {
    uint64_t p = nodes[i];
    if (p >= uint64_t(npoin) || !on[p]) return XG_ERR_ARG;
    for (int j = 0; j < 3; ++j) norms[i * 3 + j] = acc[p * 4 + j] / acc[p * 4 + 3];
  }
  return XG_OK;
  XG_HOST_CATCH
}

// Pressure-Poisson matrix of ChoCG::prelhs (src/Inciter/ChoCG.cpp:146-188):
// A(a,b) -= grad_a.grad_b / (6 J) summed over tets on the sparsity of points
// surrounding points plus the diagonal; zero-based rows sorted by column.
// Call with cap = 0 for *nnz, then with arrays of that size.
int xg_mesh_pressure_matrix(int64_t npoin, const double* coord, int64_t nelem,
                            const uint64_t* inpoel, int64_t cap, int64_t* nnz, uint64_t* ia,
                            uint64_t* ja, double* a) {
  XG_HOST_TRY
  if (npoin <= 0 || !coord || !inpoel || !nnz) return XG_ERR_ARG;
  for (int64_t i = 0; i < nelem * 4; ++i)
    if (inpoel[i] >= static_cast<uint64_t>(npoin)) return XG_ERR_ARG;
  std::vector<int64_t> ptr, adj;
  psup(npoin, nelem, inpoel, ptr, adj);
  const int64_t total = static_cast<int64_t>(adj.size()) + npoin;
  *nnz = total;
  if (cap < total) return XG_OK;
  if (!ia || !ja || !a) return XG_ERR_ARG;
  ia[0] = 0;
  int64_t k = 0;
  for (int64_t i = 0; i < npoin; ++i) {
    bool diag = false;
    for (int64_t j = ptr[i]; j < ptr[i + 1]; ++j) {
      if (!diag && adj[j] > i) {
        ja[k++] = static_cast<uint64_t>(i);
        diag = true;
      }
      ja[k++] = static_cast<uint64_t>(adj[j]);
    }
    if (!diag) ja[k++] = static_cast<uint64_t>(i);
    ia[i + 1] = static_cast<uint64_t>(k);
  }
  std::fill(a, a + total, 0.0);
  const double *x = coord, *y = coord + npoin, *z = coord + 2 * npoin;
  // the elements of every node in increasing element id; row r then sums its
  // entries element by element, the serial element loop's order
  std::vector<int64_t> eptr(npoin + 1, 0);
  for (int64_t e = 0; e < nelem; ++e)
    for (int v = 0; v < 4; ++v) ++eptr[inpoel[e * 4 + v] + 1];
  for (int64_t i = 0; i < npoin; ++i) eptr[i + 1] += eptr[i];
  std::vector<int64_t> elist(eptr[npoin]);
  {
    std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
    for (int64_t e = 0; e < nelem; ++e)
      for (int v = 0; v < 4; ++v) elist[fill[inpoel[e * 4 + v]]++] = e;
  }
  parallel_rows(npoin, [&](int64_t r) {
    for (int64_t k = eptr[r]; k < eptr[r + 1]; ++k) {
      const uint64_t* N = inpoel + elist[k] * 4;
      double ba[3] = {x[N[1]] - x[N[0]], y[N[1]] - y[N[0]], z[N[1]] - z[N[0]]};
      double ca[3] = {x[N[2]] - x[N[0]], y[N[2]] - y[N[0]], z[N[2]] - z[N[0]]};
      double da[3] = {x[N[3]] - x[N[0]], y[N[3]] - y[N[0]], z[N[3]] - z[N[0]]};
      double g[4][3];
      cross(ca[0], ca[1], ca[2], da[0], da[1], da[2], g[1][0], g[1][1], g[1][2]);
      cross(da[0], da[1], da[2], ba[0], ba[1], ba[2], g[2][0], g[2][1], g[2][2]);
      cross(ba[0], ba[1], ba[2], ca[0], ca[1], ca[2], g[3][0], g[3][1], g[3][2]);
      for (int i = 0; i < 3; ++i) g[0][i] = -g[1][i] - g[2][i] - g[3][i];
      const double J = (ba[0] * g[1][0] + ba[1] * g[1][1] + ba[2] * g[1][2]) * 6.0;
      for (int p = 0; p < 4; ++p) {
        if (N[p] != static_cast<uint64_t>(r)) continue;
        for (int q = 0; q < 4; ++q) {
          const uint64_t* beg = ja + ia[N[p]];
          const uint64_t* en = ja + ia[N[p] + 1];
          const uint64_t* pos = std::lower_bound(beg, en, N[q]);
          a[pos - ja] -= (g[p][0] * g[q][0] + g[p][1] * g[q][1] + g[p][2] * g[q][2]) / J;
        }
      }
    }
  });
  return XG_OK;
  XG_HOST_CATCH
}

}  // extern "C"
