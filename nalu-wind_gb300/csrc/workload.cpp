// Synthetic mesh inputs (nw_workload.h): seeded hex / tet blocks with STK
// generated-mesh numbering, periodic master ids, edges, and the edge area
// vectors and dual volumes of the CVFEM sub-control surfaces/volumes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "geometry.h"
#include "nw_internal.h"
#include "nw_workload.h"

namespace nw {
void set_last_error(const std::string& s);
}

struct nw_mesh {
  int npe = 8;
  int64_t N = 0, E = 0, M = 0;
  std::vector<double> coords, area, dualvol, bnd;
  std::vector<int64_t> gid, nid, edges, conn;
  // exposed-face integration points on the non-periodic box sides
  std::vector<int32_t> fip_side;   // 0..5 = x-, x+, y-, y+, z-, z+
  std::vector<int64_t> fip_nodes;  // (face node, opposing node) per IP
  std::vector<double> fip_area;    // exposed area vector per IP
};

namespace {

using nw::Error;
using nw::fail;
using nw::hex_geometry;
using nw::quad_area;
using nw::tet_geometry;

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return double(splitmix64(s) >> 11) * 0x1.0p-53; }

const int kHexEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                             {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int kHexLr[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {4, 5}, {5, 6},
                           {6, 7}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int kTetEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
const int kTetLr[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
// Kuhn split of a hex along the c0-c6 diagonal: conforming across blocks.
const int kKuhn[6][4] = {{0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6},
                         {0, 7, 4, 6}, {0, 4, 5, 6}, {0, 5, 1, 6}};

// reverse Cuthill-McKee of the node graph given as CSR adjacency
std::vector<int64_t> rcm_order(int64_t N, const std::vector<int64_t>& ap,
                               const std::vector<int64_t>& aj) {
  std::vector<int64_t> order;
  order.reserve(N);
  std::vector<char> seen(N, 0);
  std::vector<int64_t> deg(N);
  for (int64_t i = 0; i < N; ++i) deg[i] = ap[i + 1] - ap[i];
  std::vector<int64_t> byDeg(N);
  std::iota(byDeg.begin(), byDeg.end(), 0);
  std::stable_sort(byDeg.begin(), byDeg.end(),
                   [&](int64_t a, int64_t b) { return deg[a] < deg[b]; });
  std::vector<int64_t> nb;
  for (int64_t s : byDeg) {
    if (seen[s]) continue;
    size_t head = order.size();
    order.push_back(s);
    seen[s] = 1;
    while (head < order.size()) {
      const int64_t u = order[head++];
      nb.clear();
      for (int64_t p = ap[u]; p < ap[u + 1]; ++p)
        if (!seen[aj[p]]) {
          seen[aj[p]] = 1;
          nb.push_back(aj[p]);
        }
      std::sort(nb.begin(), nb.end(), [&](int64_t a, int64_t b) {
        return deg[a] != deg[b] ? deg[a] < deg[b] : a < b;
      });
      order.insert(order.end(), nb.begin(), nb.end());
    }
  }
  std::reverse(order.begin(), order.end());
  return order;  // order[k] = old node placed at new position k
}

// Exposed faces of the block, as face integration points. A face of nn
// nodes (quad or triangle, ordered counter-clockwise seen from outside) has
// one IP per node; its area vector is that of the sub-face bounded by the
// node, the midpoints of its two face edges and the face centroid
// (Quad3DSCS::determinant_scs, src/master_element/Quad43DCVFEM.C:84-124;
// Tri3DSCS::determinant_scs, src/master_element/Tri33DCVFEM.C:56-129; the
// vector area of a quadrilateral does not depend on its triangulation). The
// opposing node of a face node is the element node joined to it by the one
// element edge that leaves the face (HexSCS::opposingNodes, src/
// master_element/Hex8CVFEM.C:727; TetSCS: the node off the face).
struct FaceIps {
  std::vector<int32_t> side;
  std::vector<int64_t> nodes;
  std::vector<double> area;
  void add(int sd, int nn, const int64_t* fn, const int64_t* opp,
           const std::vector<double>& coords) {
    double p[4][3], c[3] = {0, 0, 0};
    for (int k = 0; k < nn; ++k)
      for (int d = 0; d < 3; ++d) {
        p[k][d] = coords[3 * fn[k] + d];
        c[d] += p[k][d] / nn;
      }
    for (int k = 0; k < nn; ++k) {
      const int kn = (k + 1) % nn, kp = (k + nn - 1) % nn;
      double q[4][3];
      for (int d = 0; d < 3; ++d) {
        q[0][d] = p[k][d];
        q[1][d] = 0.5 * (p[k][d] + p[kn][d]);
        q[2][d] = c[d];
        q[3][d] = 0.5 * (p[kp][d] + p[k][d]);
      }
      double a[3];
      quad_area(q, a);
      side.push_back(sd);
      nodes.push_back(fn[k]);
      nodes.push_back(opp[k]);
      for (int d = 0; d < 3; ++d) area.push_back(a[d]);
    }
  }
};

// Orders a face's nodes so that its normal points away from `inner` (a
// point inside the element).
void orient_outward(int nn, int64_t* fn, int64_t* opp, const double* inner,
                    const std::vector<double>& coords) {
  double c[3] = {0, 0, 0}, nrm[3] = {0, 0, 0};
  for (int k = 0; k < nn; ++k)
    for (int d = 0; d < 3; ++d) c[d] += coords[3 * fn[k] + d] / nn;
  for (int k = 0; k < nn; ++k) {
    const double* a = &coords[3 * fn[k]];
    const double* b = &coords[3 * fn[(k + 1) % nn]];
    nrm[0] += (a[1] - c[1]) * (b[2] - c[2]) - (a[2] - c[2]) * (b[1] - c[1]);
    nrm[1] += (a[2] - c[2]) * (b[0] - c[0]) - (a[0] - c[0]) * (b[2] - c[2]);
    nrm[2] += (a[0] - c[0]) * (b[1] - c[1]) - (a[1] - c[1]) * (b[0] - c[0]);
  }
  double dot = 0;
  for (int d = 0; d < 3; ++d) dot += nrm[d] * (c[d] - inner[d]);
  if (dot < 0) {
    std::reverse(fn + 1, fn + nn);
    std::reverse(opp + 1, opp + nn);
  }
}

// Hex sides in element-local ordinals (the Exodus side numbering of
// HexSCS::sideNodeOrdinals_, include/master_element/Hex8CVFEM.h:395-401),
// indexed by box side x-, x+, y-, y+, z-, z+.
const int kHexBoxSide[6][4] = {{0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4},
                               {2, 3, 7, 6}, {0, 3, 2, 1}, {4, 5, 6, 7}};

void build(nw_mesh& m, int nx, int ny, int nz, const nw_box_opts& o) {
  if (nx < 1 || ny < 1 || nz < 1) fail(NW_INVALID_ARG, "box dimensions < 1");
  if (!(o.lx > 0 && o.ly > 0 && o.lz > 0)) fail(NW_INVALID_ARG, "box lengths <= 0");
  if (o.jitter < 0 || o.jitter >= 0.5) fail(NW_INVALID_ARG, "jitter must be in [0, 0.5)");
  if (o.tets && (o.periodic_x || o.periodic_y))
    fail(NW_INVALID_ARG, "periodic tet blocks are not supported");
  if (o.renumber && (o.periodic_x || o.periodic_y))
    fail(NW_INVALID_ARG, "renumbering of periodic blocks is not supported");
  const int64_t NX = nx + 1, NY = ny + 1, NZ = nz + 1;
  const int64_t N = NX * NY * NZ;
  if (N >= (int64_t(1) << 31)) fail(NW_INVALID_ARG, "too many nodes");
  auto nid = [&](int64_t i, int64_t j, int64_t k) { return i + NX * (j + NY * k); };
  // z coordinates: geometric growth from z = 0
  std::vector<double> zc(NZ);
  const double r = o.stretch_z > 0 ? o.stretch_z : 1.0;
  for (int64_t k = 0; k <= nz; ++k)
    zc[k] = (std::abs(r - 1.0) < 1e-14) ? o.lz * double(k) / nz
                                        : o.lz * (std::pow(r, double(k)) - 1.0) /
                                              (std::pow(r, double(nz)) - 1.0);
  std::vector<double> coords(3 * N);
  uint64_t seed = o.seed;
  for (int64_t k = 0; k < NZ; ++k)
    for (int64_t j = 0; j < NY; ++j)
      for (int64_t i = 0; i < NX; ++i) {
        const int64_t n = nid(i, j, k);
        double x = o.lx * double(i) / nx, y = o.ly * double(j) / ny, z = zc[k];
        if (o.jitter > 0) {
          const double ux = uniform01(seed), uy = uniform01(seed), uz = uniform01(seed);
          if (i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz) {
            const double hz = std::min(zc[k + 1] - zc[k], zc[k] - zc[k - 1]);
            x += o.jitter * (2 * ux - 1) * o.lx / nx;
            y += o.jitter * (2 * uy - 1) * o.ly / ny;
            z += o.jitter * (2 * uz - 1) * hz;
          }
        }
        coords[3 * n] = x;
        coords[3 * n + 1] = y;
        coords[3 * n + 2] = z;
      }
  // periodic masters (low face is the master)
  std::vector<int64_t> master(N);
  for (int64_t k = 0; k < NZ; ++k)
    for (int64_t j = 0; j < NY; ++j)
      for (int64_t i = 0; i < NX; ++i) {
        const int64_t mi = (o.periodic_x && i == nx) ? 0 : i;
        const int64_t mj = (o.periodic_y && j == ny) ? 0 : j;
        master[nid(i, j, k)] = nid(mi, mj, k);
      }
  // elements
  const int npe = o.tets ? 4 : 8;
  const int64_t H = int64_t(nx) * ny * nz;
  const int64_t M = o.tets ? 6 * H : H;
  std::vector<int64_t> conn(M * npe);
  {
    int64_t e = 0;
    for (int64_t k = 0; k < nz; ++k)
      for (int64_t j = 0; j < ny; ++j)
        for (int64_t i = 0; i < nx; ++i) {
          const int64_t c[8] = {nid(i, j, k),         nid(i + 1, j, k),
                                nid(i + 1, j + 1, k), nid(i, j + 1, k),
                                nid(i, j, k + 1),     nid(i + 1, j, k + 1),
                                nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)};
          if (o.tets) {
            for (int t = 0; t < 6; ++t, ++e)
              for (int q = 0; q < 4; ++q) conn[4 * e + q] = c[kKuhn[t][q]];
          } else {
            for (int q = 0; q < 8; ++q) conn[8 * e + q] = c[q];
            ++e;
          }
        }
  }
  // exposed faces (lattice numbering; mapped through any renumbering below)
  FaceIps fips;
  {
    auto lat = [&](int64_t n, int d) {
      return d == 0 ? n % NX : (d == 1 ? (n / NX) % NY : n / (NX * NY));
    };
    const int64_t hi_l[3] = {nx, ny, nz};
    for (int sd = 0; sd < 6; ++sd) {
      const int dir = sd / 2, up = sd % 2;
      if ((dir == 0 && o.periodic_x) || (dir == 1 && o.periodic_y)) continue;
      const int64_t plane = up ? hi_l[dir] : 0;
      const int64_t layer = up ? hi_l[dir] - 1 : 0;
      const int64_t n1 = dir == 0 ? ny : nx, n2 = dir == 2 ? ny : nz;
      for (int64_t b = 0; b < n2; ++b)
        for (int64_t a = 0; a < n1; ++a) {
          int64_t ijk[3];
          ijk[dir] = layer;
          ijk[dir == 0 ? 1 : 0] = a;
          ijk[dir == 2 ? 1 : 2] = b;
          const int64_t h = ijk[0] + int64_t(nx) * (ijk[1] + int64_t(ny) * ijk[2]);
          if (!o.tets) {
            const int64_t* ce = &conn[8 * h];
            double inner[3] = {0, 0, 0};
            for (int q = 0; q < 8; ++q)
              for (int d = 0; d < 3; ++d) inner[d] += coords[3 * ce[q] + d] / 8;
            int64_t fn[4], opp[4];
            for (int k = 0; k < 4; ++k) {
              const int ln = kHexBoxSide[sd][k];
              fn[k] = ce[ln];
              for (int q = 0; q < 12; ++q) {
                const int other = kHexEdge[q][0] == ln ? kHexEdge[q][1]
                                  : kHexEdge[q][1] == ln ? kHexEdge[q][0] : -1;
                if (other < 0) continue;
                bool on_face = false;
                for (int t = 0; t < 4; ++t) on_face |= kHexBoxSide[sd][t] == other;
                if (!on_face) opp[k] = ce[other];
              }
            }
            orient_outward(4, fn, opp, inner, coords);
            fips.add(sd, 4, fn, opp, coords);
          } else {
            for (int t = 0; t < 6; ++t) {
              const int64_t* ce = &conn[4 * (6 * h + t)];
              for (int off = 0; off < 4; ++off) {
                int64_t fn[3], opp[3];
                int k = 0;
                bool on = true;
                for (int q = 0; q < 4; ++q)
                  if (q != off) {
                    fn[k] = ce[q];
                    opp[k++] = ce[off];
                    on = on && lat(ce[q], dir) == plane;
                  }
                if (!on) continue;
                const double* inner = &coords[3 * ce[off]];
                orient_outward(3, fn, opp, inner, coords);
                fips.add(sd, 3, fn, opp, coords);
              }
            }
          }
        }
    }
  }
  // renumbering (relabels ids and reorders node storage by new id)
  if (o.renumber) {
    std::vector<int64_t> perm(N);  // perm[new] = old
    std::iota(perm.begin(), perm.end(), 0);
    uint64_t rs = o.renumber_seed;
    for (int64_t i = N - 1; i > 0; --i) {
      const int64_t j = int64_t(splitmix64(rs) % uint64_t(i + 1));
      std::swap(perm[i], perm[j]);
    }
    std::vector<int64_t> inv(N);
    for (int64_t k = 0; k < N; ++k) inv[perm[k]] = k;
    for (auto& c : conn) c = inv[c];
    for (auto& c : fips.nodes) c = inv[c];
    {
      std::vector<double> nc(3 * N);
      for (int64_t k = 0; k < N; ++k)
        for (int d = 0; d < 3; ++d) nc[3 * k + d] = coords[3 * perm[k] + d];
      coords.swap(nc);
    }
    for (int64_t k = 0; k < N; ++k) master[k] = k;
    if (o.renumber == 2) {
      // node adjacency from element edges
      std::vector<std::vector<int64_t>> adj(N);
      const int ne = o.tets ? 6 : 12;
      for (int64_t e = 0; e < M; ++e)
        for (int q = 0; q < ne; ++q) {
          const int64_t a = conn[npe * e + (o.tets ? kTetEdge[q][0] : kHexEdge[q][0])];
          const int64_t b = conn[npe * e + (o.tets ? kTetEdge[q][1] : kHexEdge[q][1])];
          adj[a].push_back(b);
          adj[b].push_back(a);
        }
      std::vector<int64_t> ap(N + 1, 0), aj;
      for (int64_t i = 0; i < N; ++i) {
        auto& v = adj[i];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        ap[i + 1] = ap[i] + int64_t(v.size());
      }
      aj.reserve(ap[N]);
      for (auto& v : adj) aj.insert(aj.end(), v.begin(), v.end());
      adj.clear();
      adj.shrink_to_fit();
      std::vector<int64_t> ord = rcm_order(N, ap, aj);
      std::vector<int64_t> inv2(N);
      for (int64_t k = 0; k < N; ++k) inv2[ord[k]] = k;
      for (auto& c : conn) c = inv2[c];
      for (auto& c : fips.nodes) c = inv2[c];
      std::vector<double> nc(3 * N);
      for (int64_t k = 0; k < N; ++k)
        for (int d = 0; d < 3; ++d) nc[3 * k + d] = coords[3 * ord[k] + d];
      coords.swap(nc);
    }
  }
  // edges: per-node sorted unique higher neighbours (node[0] = lower id)
  const int ne = o.tets ? 6 : 12;
  std::vector<int64_t> cnt(N + 1, 0);
  for (int64_t e = 0; e < M; ++e)
    for (int q = 0; q < ne; ++q) {
      int64_t a = conn[npe * e + (o.tets ? kTetEdge[q][0] : kHexEdge[q][0])];
      int64_t b = conn[npe * e + (o.tets ? kTetEdge[q][1] : kHexEdge[q][1])];
      cnt[std::min(a, b) + 1]++;
    }
  for (int64_t i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
  std::vector<int64_t> hi(cnt[N]);
  {
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int64_t e = 0; e < M; ++e)
      for (int q = 0; q < ne; ++q) {
        int64_t a = conn[npe * e + (o.tets ? kTetEdge[q][0] : kHexEdge[q][0])];
        int64_t b = conn[npe * e + (o.tets ? kTetEdge[q][1] : kHexEdge[q][1])];
        hi[pos[std::min(a, b)]++] = std::max(a, b);
      }
  }
  std::vector<int64_t> eptr(N + 1, 0), ehi;
  ehi.reserve(hi.size() / 2);
  for (int64_t i = 0; i < N; ++i) {
    auto b = hi.begin() + cnt[i], en = hi.begin() + cnt[i + 1];
    std::sort(b, en);
    auto u = std::unique(b, en);
    ehi.insert(ehi.end(), b, u);
    eptr[i + 1] = int64_t(ehi.size());
  }
  const int64_t E = int64_t(ehi.size());
  std::vector<int64_t> edges(2 * E);
  for (int64_t i = 0; i < N; ++i)
    for (int64_t p = eptr[i]; p < eptr[i + 1]; ++p) {
      edges[2 * p] = i;
      edges[2 * p + 1] = ehi[p];
    }
  auto edge_of = [&](int64_t a, int64_t b) {
    const int64_t lo = std::min(a, b), h = std::max(a, b);
    auto it = std::lower_bound(ehi.begin() + eptr[lo], ehi.begin() + eptr[lo + 1], h);
    return int64_t(it - ehi.begin());
  };
  // geometry: per-element sub-control surfaces and volumes, then gather
  const int nscs = o.tets ? 6 : 12;
  const int nscv = npe;
  std::vector<double> escs(size_t(M) * nscs * 3), escv(size_t(M) * nscv);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < M; ++e) {
    if (o.tets) {
      double c[4][3], s[6][3], v[4];
      for (int q = 0; q < 4; ++q)
        for (int d = 0; d < 3; ++d) c[q][d] = coords[3 * conn[4 * e + q] + d];
      tet_geometry(c, s, v);
      for (int ip = 0; ip < 6; ++ip)
        for (int d = 0; d < 3; ++d) escs[(size_t(e) * 6 + ip) * 3 + d] = s[ip][d];
      for (int ip = 0; ip < 4; ++ip) escv[size_t(e) * 4 + ip] = v[ip];
    } else {
      double c[8][3], s[12][3], v[8];
      for (int q = 0; q < 8; ++q)
        for (int d = 0; d < 3; ++d) c[q][d] = coords[3 * conn[8 * e + q] + d];
      hex_geometry(c, s, v);
      for (int ip = 0; ip < 12; ++ip)
        for (int d = 0; d < 3; ++d) escs[(size_t(e) * 12 + ip) * 3 + d] = s[ip][d];
      for (int ip = 0; ip < 8; ++ip) escv[size_t(e) * 8 + ip] = v[ip];
    }
  }
  std::vector<double> area(3 * E, 0.0), dualvol(N, 0.0);
  for (int64_t e = 0; e < M; ++e) {
    for (int ip = 0; ip < nscs; ++ip) {
      const int la = o.tets ? kTetLr[ip][0] : kHexLr[ip][0];
      const int lb = o.tets ? kTetLr[ip][1] : kHexLr[ip][1];
      const int64_t a = conn[npe * e + la], b = conn[npe * e + lb];
      const int64_t ed = edge_of(a, b);
      // sign rule of GeometryInteriorAlg.C:209-213
      const double sign = (a == edges[2 * ed]) ? 1.0 : -1.0;
      for (int d = 0; d < 3; ++d)
        area[3 * ed + d] += escs[(size_t(e) * nscs + ip) * 3 + d] * sign;
    }
    for (int ip = 0; ip < nscv; ++ip)
      dualvol[conn[npe * e + ip]] += escv[size_t(e) * nscv + ip];
  }
  // lumped exposed area vectors: the sum of the sub-face area vectors of
  // the face IPs at each node (the shifted boundary closure of the nodal
  // gradient, NodalGradBndryElemAlg with useShifted); periodic sides have
  // no face IPs
  std::vector<double> bnd(3 * N, 0.0);
  for (size_t ip = 0; ip < fips.side.size(); ++ip) {
    const int64_t R = fips.nodes[2 * ip];
    for (int d = 0; d < 3; ++d) bnd[3 * R + d] += fips.area[3 * ip + d];
  }
  // periodic sums of nodal quantities: master and slaves hold the total
  for (int64_t n = 0; n < N; ++n)
    if (master[n] != n) {
      dualvol[master[n]] += dualvol[n];
      for (int d = 0; d < 3; ++d) bnd[3 * master[n] + d] += bnd[3 * n + d];
    }
  for (int64_t n = 0; n < N; ++n)
    if (master[n] != n) {
      dualvol[n] = dualvol[master[n]];
      for (int d = 0; d < 3; ++d) bnd[3 * n + d] = bnd[3 * master[n] + d];
    }
  m.npe = npe;
  m.N = N;
  m.E = E;
  m.M = M;
  m.coords.swap(coords);
  m.area.swap(area);
  m.dualvol.swap(dualvol);
  m.bnd.swap(bnd);
  m.fip_side.swap(fips.side);
  m.fip_nodes.swap(fips.nodes);
  m.fip_area.swap(fips.area);
  m.conn.swap(conn);
  m.edges.swap(edges);
  m.gid.resize(N);
  m.nid.resize(N);
  for (int64_t n = 0; n < N; ++n) {
    m.gid[n] = n + 1;
    m.nid[n] = master[n] + 1;
  }
}

template <typename F>
nw_status guard(F&& f) {
  try {
    f();
    return NW_OK;
  } catch (const Error& e) {
    nw::set_last_error(e.msg);
    return e.status;
  } catch (const std::exception& e) {
    nw::set_last_error(e.what());
    return NW_INTERNAL;
  }
}

}  // namespace

extern "C" {

nw_status nw_mesh_box(int nx, int ny, int nz, const nw_box_opts* opts,
                      nw_mesh** out) {
  return guard([&] {
    if (!opts || !out) fail(NW_INVALID_ARG, "null argument");
    *out = nullptr;
    auto m = std::make_unique<nw_mesh>();
    build(*m, nx, ny, nz, *opts);
    *out = m.release();
  });
}

nw_status nw_mesh_destroy(nw_mesh* m) {
  delete m;
  return NW_OK;
}

nw_status nw_mesh_rcm_order(int64_t num_nodes, int64_t num_edges, const int64_t* edges,
                            int64_t* order) {
  return guard([&] {
    if (!order || (num_edges > 0 && !edges)) fail(NW_INVALID_ARG, "null argument");
    if (num_nodes < 1 || num_edges < 0) fail(NW_INVALID_ARG, "size out of range");
    std::vector<int64_t> ap(size_t(num_nodes) + 1, 0);
    for (int64_t e = 0; e < 2 * num_edges; ++e) {
      if (edges[e] < 0 || edges[e] >= num_nodes) fail(NW_INVALID_ARG, "edge node out of range");
      ++ap[edges[e] + 1];
    }
    for (int64_t i = 0; i < num_nodes; ++i) ap[i + 1] += ap[i];
    std::vector<int64_t> aj(size_t(ap[num_nodes])), pos(ap.begin(), ap.end() - 1);
    for (int64_t e = 0; e < num_edges; ++e) {
      const int64_t a = edges[2 * e], b = edges[2 * e + 1];
      aj[pos[a]++] = b;
      aj[pos[b]++] = a;
    }
    // sorted, duplicate-free neighbour lists (the order then depends on the
    // graph only, not on the edge order)
    std::vector<int64_t> ap2(size_t(num_nodes) + 1, 0), aj2;
    aj2.reserve(aj.size());
    for (int64_t i = 0; i < num_nodes; ++i) {
      std::sort(aj.begin() + ap[i], aj.begin() + ap[i + 1]);
      for (int64_t p = ap[i]; p < ap[i + 1]; ++p)
        if (aj[p] != i && (p == ap[i] || aj[p] != aj[p - 1])) aj2.push_back(aj[p]);
      ap2[i + 1] = int64_t(aj2.size());
    }
    const std::vector<int64_t> ord = rcm_order(num_nodes, ap2, aj2);
    std::copy(ord.begin(), ord.end(), order);
  });
}

nw_status nw_mesh_sizes(const nw_mesh* m, int64_t* num_nodes,
                        int64_t* num_edges, int64_t* num_elems,
                        int* nodes_per_elem) {
  return guard([&] {
    if (!m) fail(NW_INVALID_ARG, "null mesh");
    if (num_nodes) *num_nodes = m->N;
    if (num_edges) *num_edges = m->E;
    if (num_elems) *num_elems = m->M;
    if (nodes_per_elem) *nodes_per_elem = m->npe;
  });
}

nw_status nw_mesh_get(const nw_mesh* m, double* coords, int64_t* global_id,
                      int64_t* nalu_id, int64_t* edges, int64_t* conn,
                      double* area, double* dualvol, double* bnd_area) {
  return guard([&] {
    if (!m) fail(NW_INVALID_ARG, "null mesh");
    auto cp = [](auto* dst, const auto& src) {
      if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(src[0]));
    };
    cp(coords, m->coords);
    cp(global_id, m->gid);
    cp(nalu_id, m->nid);
    cp(edges, m->edges);
    cp(conn, m->conn);
    cp(area, m->area);
    cp(dualvol, m->dualvol);
    cp(bnd_area, m->bnd);
  });
}

}  // extern "C"

extern "C" nw_status nw_mesh_face_ips(const nw_mesh* m, int side_mask,
                                      int64_t* count, int64_t* ip_nodes,
                                      double* area, int32_t* side) {
  return guard([&] {
    if (!m || !count) fail(NW_INVALID_ARG, "null argument");
    int64_t n = 0;
    const int64_t total = int64_t(m->fip_side.size());
    for (int64_t i = 0; i < total; ++i) {
      if (!((side_mask >> m->fip_side[i]) & 1)) continue;
      if (ip_nodes) {
        ip_nodes[2 * n] = m->fip_nodes[2 * i];
        ip_nodes[2 * n + 1] = m->fip_nodes[2 * i + 1];
      }
      if (area)
        for (int d = 0; d < 3; ++d) area[3 * n + d] = m->fip_area[3 * i + d];
      if (side) side[n] = m->fip_side[i];
      ++n;
    }
    *count = n;
  });
}
