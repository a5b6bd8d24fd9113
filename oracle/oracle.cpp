// CPU oracle for the nalu-wind edge-assembly + Krylov hot path.
//
// TEST INFRASTRUCTURE ONLY: this is the checker that tests, the smoke check
// and the benchmark's CPU-baseline leg call to compute reference answers on
// the host. Product code never links or calls it.
//
// Every function restates a reference algorithm; the citing comment names
// the reference file:line it follows (paths relative to the nalu-wind tree).
// Built with -O3 -ffp-contract=off so results are identical on x86_64 and
// aarch64 hosts.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <random>
#include <stdexcept>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int32_t kInvalid = std::numeric_limits<int32_t>::max();

// Hex8 edge ordinals of the STK hex topology (node pairs per edge ordinal).
constexpr int kHexEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// HexSCS left/right node of each sub-control surface
// (include/master_element/Hex8CVFEM.h:292).
constexpr int kHexLrscv[24] = {0, 1, 1, 2, 2, 3, 0, 3, 4, 5, 5, 6,
                               6, 7, 4, 7, 0, 4, 1, 5, 2, 6, 3, 7};
// HexSCS scsIpEdgeOrd_ (include/master_element/Hex8CVFEM.h:404): identity.

// subdivide_hex_8 (include/master_element/Hex8GeometryFunctions.h:256-324).
void subdivide_hex8(const double c[8][3], double v[27][3]) {
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) v[n][d] = c[n][d];
  for (int d = 0; d < 3; ++d) {
    v[8][d] = 0.5 * (c[0][d] + c[1][d]);
    v[9][d] = 0.5 * (c[1][d] + c[2][d]);
    v[10][d] = 0.5 * (c[2][d] + c[3][d]);
    v[11][d] = 0.5 * (c[3][d] + c[0][d]);
    v[12][d] = 0.25 * (c[0][d] + c[1][d] + c[2][d] + c[3][d]);
    v[13][d] = 0.5 * (c[4][d] + c[5][d]);
    v[14][d] = 0.5 * (c[5][d] + c[6][d]);
    v[15][d] = 0.5 * (c[6][d] + c[7][d]);
    v[16][d] = 0.5 * (c[7][d] + c[4][d]);
    v[17][d] = 0.25 * (c[4][d] + c[5][d] + c[6][d] + c[7][d]);
    v[18][d] = 0.5 * (c[1][d] + c[5][d]);
    v[19][d] = 0.5 * (c[0][d] + c[4][d]);
    v[20][d] = 0.25 * (c[0][d] + c[1][d] + c[4][d] + c[5][d]);
    v[21][d] = 0.5 * (c[3][d] + c[7][d]);
    v[22][d] = 0.5 * (c[2][d] + c[6][d]);
    v[23][d] = 0.25 * (c[2][d] + c[3][d] + c[6][d] + c[7][d]);
    v[24][d] = 0.25 * (c[1][d] + c[2][d] + c[5][d] + c[6][d]);
    v[25][d] = 0.25 * (c[0][d] + c[3][d] + c[4][d] + c[7][d]);
    v[26][d] = 0.;
    for (int n = 0; n < 8; ++n) v[26][d] += c[n][d];
    v[26][d] *= 0.125;
  }
}

// quad_area_by_triangulation (Hex8GeometryFunctions.h:34-81).
void quad_area(const double q[4][3], double a[3]) {
  a[0] = a[1] = a[2] = 0.0;
  const double xm[3] = {0.25 * (q[0][0] + q[1][0] + q[2][0] + q[3][0]),
                        0.25 * (q[0][1] + q[1][1] + q[2][1] + q[3][1]),
                        0.25 * (q[0][2] + q[1][2] + q[2][2] + q[3][2])};
  double r1[3] = {q[0][0] - xm[0], q[0][1] - xm[1], q[0][2] - xm[2]};
  for (int t = 0; t < 4; ++t) {
    const int ti = (t + 1) % 4;
    const double r2[3] = {q[ti][0] - xm[0], q[ti][1] - xm[1], q[ti][2] - xm[2]};
    a[0] += r1[1] * r2[2] - r2[1] * r1[2];
    a[1] += r1[2] * r2[0] - r2[2] * r1[0];
    a[2] += r1[0] * r2[1] - r2[0] * r1[1];
    r1[0] = r2[0];
    r1[1] = r2[1];
    r1[2] = r2[2];
  }
  a[0] *= 0.5;
  a[1] *= 0.5;
  a[2] *= 0.5;
}

// hex_volume_grandy (Hex8GeometryFunctions.h:83-159).
double hex_volume_grandy(const double s[8][3]) {
  double cv[14][3];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) cv[n][d] = s[n][d];
  constexpr int fn[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                            {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 3, 7}};
  for (int k = 0; k < 6; ++k)
    for (int d = 0; d < 3; ++d)
      cv[k + 8][d] = 0.25 * (cv[fn[k][0]][d] + cv[fn[k][1]][d] +
                             cv[fn[k][2]][d] + cv[fn[k][3]][d]);
  constexpr int tf[24][3] = {
      {0, 8, 1},  {8, 2, 1},  {3, 2, 8},  {3, 8, 0},  {6, 9, 5},  {7, 9, 6},
      {4, 9, 7},  {4, 5, 9},  {10, 0, 1}, {5, 10, 1}, {4, 10, 5}, {4, 0, 10},
      {7, 6, 11}, {6, 2, 11}, {2, 3, 11}, {3, 7, 11}, {6, 12, 2}, {5, 12, 6},
      {5, 1, 12}, {1, 2, 12}, {0, 4, 13}, {4, 7, 13}, {7, 3, 13}, {3, 0, 13}};
  double vol = 0.0;
  for (int k = 0; k < 24; ++k) {
    const int p = tf[k][0], q = tf[k][1], r = tf[k][2];
    const double m[3] = {cv[p][0] + cv[q][0] + cv[r][0],
                         cv[p][1] + cv[q][1] + cv[r][1],
                         cv[p][2] + cv[q][2] + cv[r][2]};
    double dx[3];
    dx[0] = (cv[q][1] - cv[p][1]) * (cv[r][2] - cv[p][2]) -
            (cv[r][1] - cv[p][1]) * (cv[q][2] - cv[p][2]);
    dx[1] = (cv[r][0] - cv[p][0]) * (cv[q][2] - cv[p][2]) -
            (cv[q][0] - cv[p][0]) * (cv[r][2] - cv[p][2]);
    dx[2] = (cv[q][0] - cv[p][0]) * (cv[r][1] - cv[p][1]) -
            (cv[r][0] - cv[p][0]) * (cv[q][1] - cv[p][1]);
    vol += m[0] * dx[0] + m[1] * dx[1] + m[2] * dx[2];
  }
  vol /= 18.0;
  return vol;
}

// van_leer (include/edge_kernels/EdgeKernelUtils.h:18-24).
inline double van_leer(double dqm, double dqp, double eps) {
  return (2.0 * (dqm * dqp + std::abs(dqm * dqp))) /
         ((dqm + dqp) * (dqm + dqp) + eps);
}

// LocalGraphArrays (include/LinearSolver.h:80-151): CSR rows pre-sized by
// row length and filled with INVALID, then sorted insertion with numDof
// block expansion.
struct LocalGraphArrays {
  std::vector<int64_t> rowPointers;
  std::vector<int32_t> colIndices;
  explicit LocalGraphArrays(const std::vector<int64_t>& rowLengths) {
    rowPointers.assign(rowLengths.size() + 1, 0);
    int64_t nnz = 0;
    for (size_t i = 0; i < rowLengths.size(); ++i) {
      rowPointers[i] = nnz;
      nnz += rowLengths[i];
    }
    rowPointers[rowLengths.size()] = nnz;
    colIndices.assign(nnz, kInvalid);
  }
  int64_t row_length(int64_t r) const {
    return rowPointers[r + 1] - rowPointers[r];
  }
  void insertIndices(int64_t r, size_t n, const int32_t* inds, int numDof) {
    int32_t* row = colIndices.data() + rowPointers[r];
    const int64_t len = row_length(r);
    int32_t* rowEnd = std::find(row, row + len, kInvalid);
    for (size_t i = 0; i < n; ++i) {
      int32_t* ip = std::lower_bound(row, rowEnd, inds[i]);
      if (ip <= rowEnd && (ip == row + len || *ip != inds[i])) {
        if (rowEnd + numDof > row + len)
          throw std::runtime_error("LocalGraphArrays: row overflow");
        for (int32_t* p = rowEnd + numDof - 1; p != ip + numDof - 1; --p)
          *p = *(p - numDof);
        for (int d = 0; d < numDof; ++d) ip[d] = inds[i] + d;
        rowEnd += numDof;
      }
    }
  }
};

}  // namespace

extern "C" {

int or_version(void) { return 1; }

// Exposed-face sub-control-surface area vectors, one per face node:
// Quad3DSCS::determinant_scs (src/master_element/Quad43DCVFEM.C:84-124;
// sub-face of node i = (node i, mid edge i->i+1, centroid, mid edge i-1->i)
// by quad_area_by_triangulation) for nn = 4, Tri3DSCS::determinant_scs
// (src/master_element/Tri33DCVFEM.C:56-129; half the cross product of the
// sub-face's diagonals) for nn = 3. faces: nfaces x nn node indices.
void or_face_scs_areas(int64_t nfaces, int nn, const int64_t* faces,
                       const double* coords, double* areav) {
  for (int64_t f = 0; f < nfaces; ++f) {
    double p[4][3], e[4][3], c[3] = {0, 0, 0};
    for (int k = 0; k < nn; ++k)
      for (int d = 0; d < 3; ++d) p[k][d] = coords[3 * faces[nn * f + k] + d];
    for (int k = 0; k < nn; ++k)
      for (int d = 0; d < 3; ++d) {
        e[k][d] = 0.5 * (p[k][d] + p[(k + 1) % nn][d]);
        c[d] += p[k][d];
      }
    for (int d = 0; d < 3; ++d) c[d] /= nn;
    for (int k = 0; k < nn; ++k) {
      double* a = areav + 3 * (nn * f + k);
      const int km = (k + nn - 1) % nn;
      if (nn == 4) {
        double q[4][3];
        for (int d = 0; d < 3; ++d) {
          q[0][d] = p[k][d];
          q[1][d] = e[k][d];
          q[2][d] = c[d];
          q[3][d] = e[km][d];
        }
        quad_area(q, a);
      } else {
        const double d13[3] = {c[0] - p[k][0], c[1] - p[k][1], c[2] - p[k][2]};
        const double d24[3] = {e[km][0] - e[k][0], e[km][1] - e[k][1], e[km][2] - e[k][2]};
        a[0] = 0.5 * (d24[2] * d13[1] - d13[2] * d24[1]);
        a[1] = 0.5 * (d24[0] * d13[2] - d13[0] * d24[2]);
        a[2] = 0.5 * (d24[1] * d13[0] - d13[1] * d24[0]);
      }
    }
  }
}

// Replays insertIndices calls on a LocalGraphArrays of the given row
// lengths (op k inserts op_n[k] columns of op_cols into row op_row[k]);
// writes rowPointers (nrows + 1) and colIndices. Returns 0, or 1 when a
// row overflows.
int or_local_graph_replay(int nrows, const int64_t* row_lengths, int nops,
                          const int32_t* op_row, const int32_t* op_n,
                          const int32_t* op_cols, int num_dof,
                          int64_t* row_ptr, int32_t* col_idx) {
  try {
    LocalGraphArrays g(std::vector<int64_t>(row_lengths, row_lengths + nrows));
    const int32_t* c = op_cols;
    for (int k = 0; k < nops; ++k) {
      g.insertIndices(op_row[k], size_t(op_n[k]), c, num_dof);
      c += op_n[k];
    }
    std::copy(g.rowPointers.begin(), g.rowPointers.end(), row_ptr);
    std::copy(g.colIndices.begin(), g.colIndices.end(), col_idx);
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

// ---------------------------------------------------------------------------
// STK "generated:NXxNYxNZ" numbering: node ids run x fastest, then y, then z,
// from 1; coordinates are the integer lattice (unit spacing).
int64_t or_hex_box_num_nodes(int nx, int ny, int nz) {
  return int64_t(nx + 1) * (ny + 1) * (nz + 1);
}
int64_t or_hex_box_num_elems(int nx, int ny, int nz) {
  return int64_t(nx) * ny * nz;
}
void or_hex_box(int nx, int ny, int nz, double* coords, int64_t* conn) {
  auto nid = [&](int i, int j, int k) {
    return int64_t(i) + int64_t(nx + 1) * (j + int64_t(ny + 1) * k);
  };
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int64_t n = nid(i, j, k);
        coords[3 * n + 0] = i;
        coords[3 * n + 1] = j;
        coords[3 * n + 2] = k;
      }
  int64_t e = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i, ++e) {
        int64_t* c = conn + 8 * e;
        c[0] = nid(i, j, k);
        c[1] = nid(i + 1, j, k);
        c[2] = nid(i + 1, j + 1, k);
        c[3] = nid(i, j + 1, k);
        c[4] = nid(i, j, k + 1);
        c[5] = nid(i + 1, j, k + 1);
        c[6] = nid(i + 1, j + 1, k + 1);
        c[7] = nid(i, j + 1, k + 1);
      }
}

// Seeded synthetic box coordinates (the benchmark workloads' definition,
// not reference code): x = lx i / nx, y = ly j / ny, z geometrically
// stretched from z = 0 with growth ratio `stretch`; every node draws three
// splitmix64 uniforms in node order, and interior nodes move by
// jitter (2u - 1) times the local spacing (z: the smaller neighbouring
// layer). Same numbering as or_hex_box.
static uint64_t or_splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void or_box_coords(int nx, int ny, int nz, double lx, double ly, double lz,
                   double stretch, double jitter, uint64_t seed, double* coords) {
  std::vector<double> zc(nz + 1);
  const double r = stretch > 0 ? stretch : 1.0;
  for (int k = 0; k <= nz; ++k)
    zc[k] = (std::abs(r - 1.0) < 1e-14)
                ? lz * double(k) / nz
                : lz * (std::pow(r, double(k)) - 1.0) / (std::pow(r, double(nz)) - 1.0);
  uint64_t s = seed;
  auto u01 = [&]() { return double(or_splitmix64(s) >> 11) * 0x1.0p-53; };
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int64_t n = int64_t(i) + int64_t(nx + 1) * (j + int64_t(ny + 1) * k);
        double x = lx * double(i) / nx, y = ly * double(j) / ny, z = zc[k];
        if (jitter > 0) {
          const double ux = u01(), uy = u01(), uz = u01();
          if (i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz) {
            const double hz = std::min(zc[k + 1] - zc[k], zc[k] - zc[k - 1]);
            x += jitter * (2 * ux - 1) * lx / nx;
            y += jitter * (2 * uy - 1) * ly / ny;
            z += jitter * (2 * uz - 1) * hz;
          }
        }
        coords[3 * n] = x;
        coords[3 * n + 1] = y;
        coords[3 * n + 2] = z;
      }
}

// STK create_edges: each element's edges by ordinal, created once; node[0]
// is the lower id (lexicographically smallest permutation). The sign rule
// of GeometryInteriorAlg.C:209-213 and the unit-test mdot of +2.5 for a
// uniform +10 velocity (unit_tests/ngp_algorithms/UnitTestMdotAlg.C:56) fix
// this orientation.
int64_t or_hex8_edges(int64_t nelem, const int64_t* conn, int64_t nnodes,
                      int64_t cap, int64_t* edges, int64_t* elem_edges) {
  (void)nnodes;
  std::unordered_map<uint64_t, int64_t> seen;
  seen.reserve(size_t(nelem) * 4);
  int64_t E = 0;
  for (int64_t e = 0; e < nelem; ++e) {
    for (int o = 0; o < 12; ++o) {
      int64_t a = conn[8 * e + kHexEdge[o][0]];
      int64_t b = conn[8 * e + kHexEdge[o][1]];
      if (b < a) std::swap(a, b);
      const uint64_t key = (uint64_t(a) << 32) | uint64_t(b);
      auto it = seen.find(key);
      int64_t idx;
      if (it == seen.end()) {
        idx = E++;
        seen.emplace(key, idx);
        if (idx < cap) {
          edges[2 * idx] = a;
          edges[2 * idx + 1] = b;
        }
      } else {
        idx = it->second;
      }
      if (elem_edges) elem_edges[12 * e + o] = idx;
    }
  }
  return E;
}

// GeometryInteriorAlg::impl_compute_edge_area_vector (:163-225) with
// HexSCS::determinant_scs (src/master_element/Hex8CVFEM.C:565-591), and
// impl_compute_dual_nodal_volume (:70-112) with HexSCV::determinant_scv
// (Hex8CVFEM.C:363-389).
void or_hex8_geometry(int64_t nnodes, const double* coords, int64_t nelem,
                      const int64_t* conn, const int64_t* elem_edges,
                      int64_t nedges, const int64_t* edges, double* area,
                      double* dualvol) {
  constexpr int facet[12][4] = {
      {20, 8, 12, 26},  {24, 9, 12, 26},  {10, 12, 26, 23}, {11, 25, 26, 12},
      {13, 20, 26, 17}, {17, 14, 24, 26}, {17, 15, 23, 26}, {16, 17, 26, 25},
      {19, 20, 26, 25}, {20, 18, 24, 26}, {22, 23, 26, 24}, {21, 25, 26, 23}};
  constexpr int subdiv[8][8] = {
      {0, 8, 12, 11, 19, 20, 26, 25},  {8, 1, 9, 12, 20, 18, 24, 26},
      {12, 9, 2, 10, 26, 24, 22, 23},  {11, 12, 10, 3, 25, 26, 23, 21},
      {19, 20, 26, 25, 4, 13, 17, 16}, {20, 18, 24, 26, 13, 5, 14, 17},
      {26, 24, 22, 23, 17, 14, 6, 15}, {25, 26, 23, 21, 16, 17, 15, 7}};
  std::fill(area, area + 3 * nedges, 0.0);
  std::fill(dualvol, dualvol + nnodes, 0.0);
  for (int64_t e = 0; e < nelem; ++e) {
    double c[8][3], v[27][3];
    for (int n = 0; n < 8; ++n)
      for (int d = 0; d < 3; ++d) c[n][d] = coords[3 * conn[8 * e + n] + d];
    subdivide_hex8(c, v);
    for (int ip = 0; ip < 12; ++ip) {
      double q[4][3], a[3];
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) q[k][d] = v[facet[ip][k]][d];
      quad_area(q, a);
      const int64_t edge = elem_edges[12 * e + ip];
      const int64_t left = conn[8 * e + kHexLrscv[2 * ip]];
      const double sign = (left == edges[2 * edge]) ? 1.0 : -1.0;
      for (int d = 0; d < 3; ++d) area[3 * edge + d] += a[d] * sign;
    }
    for (int ip = 0; ip < 8; ++ip) {
      double s[8][3];
      for (int n = 0; n < 8; ++n)
        for (int d = 0; d < 3; ++d) s[n][d] = v[subdiv[ip][n]][d];
      dualvol[conn[8 * e + ip]] += hex_volume_grandy(s);
    }
  }
}

// ---------------------------------------------------------------------------
// Tpetra graph: beginLinearSystemConstruction (src/TpetraLinearSystem.C:
// 177-387: owned rows sorted by nalu id, LID = numDof*k, periodic slaves are
// skipped and map to their master), addConnections (:420-440: self plus
// (min-id, max-id) pair), compute_graph_row_lengths (:879-959),
// insert_graph_connections (:961-1016), fill_in_extra_dof_rows_per_node and
// remove_invalid_indices (src/TpetraLinearSystemHelpers.C:361-418). Serial:
// the column map equals the row map.
int64_t or_build_graph(int64_t nnodes, const int64_t* nalu_id, int64_t nedges,
                       const int64_t* edges, int num_dof, int64_t* nnz_out,
                       int64_t* row_ptr, int32_t* col_idx, int64_t* node_lid) {
  // owned (non-slave) nodes sorted by id
  std::vector<int64_t> owned;
  for (int64_t n = 0; n < nnodes; ++n)
    if (nalu_id[n] == n + 1) owned.push_back(n);
  std::sort(owned.begin(), owned.end(),
            [&](int64_t a, int64_t b) { return nalu_id[a] < nalu_id[b]; });
  const int64_t nOwned = int64_t(owned.size());
  std::vector<int64_t> lidOfId(nnodes + 1, -1);
  for (int64_t k = 0; k < nOwned; ++k) lidOfId[nalu_id[owned[k]]] = num_dof * k;
  std::vector<int64_t> lid(nnodes);
  for (int64_t n = 0; n < nnodes; ++n) {
    lid[n] = lidOfId[nalu_id[n]];
    if (lid[n] < 0) throw std::runtime_error("slave without master");
  }
  // connections_[row node] = entities (insert_connection, :390-418)
  std::vector<std::vector<int64_t>> conns(nOwned);
  auto insert = [&](int64_t a, int64_t b) {
    auto& v = conns[lid[a] / num_dof];
    if (std::find(v.begin(), v.end(), b) == v.end()) v.push_back(b);
  };
  for (int64_t e = 0; e < nedges; ++e) {
    const int64_t ent[2] = {edges[2 * e], edges[2 * e + 1]};
    for (int a = 0; a < 2; ++a) {
      insert(ent[a], ent[a]);
      for (int b = a + 1; b < 2; ++b) {
        const bool ab = nalu_id[ent[a]] < nalu_id[ent[b]];
        insert(ab ? ent[a] : ent[b], ab ? ent[b] : ent[a]);
      }
    }
  }
  for (auto& v : conns) std::sort(v.begin(), v.end());
  // row lengths (add_to_length, TpetraLinearSystemHelpers.C:170-185)
  const int64_t nrows = nOwned * num_dof;
  std::vector<int64_t> len(nrows, 0);
  for (int64_t k = 0; k < nOwned; ++k) {
    const int64_t a = owned[k];
    const auto& C = conns[k];
    for (int d = 0; d < num_dof; ++d) len[lid[a] + d] += num_dof * C.size();
    for (int64_t b : C) {
      if (b == a) continue;
      for (int d = 0; d < num_dof; ++d) len[lid[b] + d] += num_dof;
    }
  }
  LocalGraphArrays g(len);
  std::vector<int32_t> cols;
  for (int64_t k = 0; k < nOwned; ++k) {
    const int64_t a = owned[k];
    const auto& C = conns[k];
    cols.resize(C.size());
    for (size_t j = 0; j < C.size(); ++j) cols[j] = int32_t(lid[C[j]]);
    g.insertIndices(lid[a], cols.size(), cols.data(), num_dof);
    const int32_t ca = int32_t(lid[a]);
    for (int64_t b : C)
      if (b != a) g.insertIndices(lid[b], 1, &ca, num_dof);
  }
  // fill_in_extra_dof_rows_per_node: copy dof-0 row columns to dof rows 1..
  if (num_dof > 1) {
    for (int64_t i = 0; i < nrows; i += num_dof) {
      const int32_t* row = g.colIndices.data() + g.rowPointers[i];
      const int64_t rl = g.row_length(i);
      for (int d = 1; d < num_dof; ++d) {
        int32_t* rd = g.colIndices.data() + g.rowPointers[i] + rl * d;
        for (int64_t j = 0; j < rl; ++j) rd[j] = row[j];
      }
    }
  }
  // remove_invalid_indices: trim trailing INVALID entries of each row
  std::vector<int64_t> newLen(nrows, 0);
  int64_t nnz = 0;
  for (int64_t i = 0; i < nrows; ++i) {
    const int32_t* row = g.colIndices.data() + g.rowPointers[i];
    for (int64_t j = g.row_length(i) - 1; j >= 0; --j)
      if (row[j] != kInvalid) {
        newLen[i] = j + 1;
        break;
      }
    nnz += newLen[i];
  }
  if (nnz_out) *nnz_out = nnz;
  if (row_ptr) {
    int64_t p = 0;
    for (int64_t i = 0; i < nrows; ++i) {
      row_ptr[i] = p;
      const int32_t* row = g.colIndices.data() + g.rowPointers[i];
      for (int64_t j = 0; j < newLen[i]; ++j) col_idx[p++] = row[j];
    }
    row_ptr[nrows] = p;
  }
  if (node_lid)
    for (int64_t n = 0; n < nnodes; ++n) node_lid[n] = lid[n];
  return nrows;
}

// ---------------------------------------------------------------------------
// Peclet functions (src/PecletFunction.C:39-45, :66-71).
double or_peclet_classic(double pe, double hf) {
  const double m = hf * pe;
  return m * m / (5.0 + m * m);
}
double or_peclet_tanh(double x, double c1, double c2) {
  return 0.50 * (1.0 + std::tanh((x - c1) / c2));
}

}  // extern "C"

namespace {

// Running-magnitude arithmetic for tolerance bounds: every value carries
// m = the same expression evaluated on |inputs| with |a+b| -> m_a + m_b,
// |a*b| -> m_a m_b and |a/b| -> m_a / |b|. The rounding error of any
// evaluation order of the expression is then a small multiple of eps * m,
// which is the scale the parity tests use. With T = double the kernels
// below are the plain FP64 restatement.
struct Mag {
  double v, m;
  Mag() : v(0), m(0) {}
  Mag(double x) : v(x), m(std::abs(x)) {}  // NOLINT: leaves and constants
  Mag(double x, double mm) : v(x), m(mm) {}
};
inline Mag operator+(Mag a, Mag b) { return {a.v + b.v, a.m + b.m}; }
inline Mag operator-(Mag a, Mag b) { return {a.v - b.v, a.m + b.m}; }
inline Mag operator-(Mag a) { return {-a.v, a.m}; }
inline Mag operator+(Mag a) { return a; }
inline Mag operator*(Mag a, Mag b) { return {a.v * b.v, a.m * b.m}; }
inline Mag operator/(Mag a, Mag b) { return {a.v / b.v, a.m / std::abs(b.v)}; }
inline Mag& operator+=(Mag& a, Mag b) { return a = a + b; }
inline Mag& operator-=(Mag& a, Mag b) { return a = a - b; }
inline Mag& operator*=(Mag& a, Mag b) { return a = a * b; }
inline Mag& operator/=(Mag& a, Mag b) { return a = a / b; }
inline bool operator>(Mag a, double b) { return a.v > b; }
inline double val(double x) { return x; }
inline double val(Mag x) { return x.v; }
inline double mag(double x) { return std::abs(x); }
inline double mag(Mag x) { return x.m; }
inline double tabs(double x) { return std::abs(x); }
inline Mag tabs(Mag x) { return {std::abs(x.v), x.m}; }
inline double tmin(double a, double b) { return std::min(a, b); }
inline Mag tmin(Mag a, Mag b) { return a.v <= b.v ? a : b; }
inline double ttanh(double x) { return std::tanh(x); }
inline Mag ttanh(Mag x) { return {std::tanh(x.v), std::abs(std::tanh(x.v))}; }

template <typename T>
T tvan_leer(T dqm, T dqp, double eps) {
  return (2.0 * (dqm * dqp + tabs(dqm * dqp))) /
         ((dqm + dqp) * (dqm + dqp) + T(eps));
}

// ScalarEdgeSolverAlg::execute (src/edge_kernels/ScalarEdgeSolverAlg.C:
// 55-206), one 2x2 local system per edge.
template <typename T>
void scalar_edge(int64_t e, const int64_t* edges, const double* coords,
                 const double* vrtm, const double* q, const double* dqdx,
                 const double* density, const double* dflux,
                 const double* area, const double* mdotA,
                 const or_scalar_opts* o, T* A, T* b) {
  const double eps = 1.0e-16;
  const double alpha = o->alpha, alphaUpw = o->alpha_upw,
               hoUpwind = o->upw_factor, relaxFac = o->relax;
  const double om_alpha = 1.0 - alpha, om_alphaUpw = 1.0 - alphaUpw;
  const int64_t L = edges[2 * e], R = edges[2 * e + 1];
  T av[3];
  for (int d = 0; d < 3; ++d) av[d] = T(area[3 * e + d]);
  const T mdot = T(mdotA[e]);
  const T densityL = T(density[L]), densityR = T(density[R]);
  const T qNp1L = T(q[L]), qNp1R = T(q[R]);
  const T viscosityL = T(dflux[L]), viscosityR = T(dflux[R]);
  const T viscIp = 0.5 * (viscosityL + viscosityR);
  const T diffIp = 0.5 * (viscosityL / densityL + viscosityR / densityR);
  T axdx = T(0.0), asq = T(0.0), udotx = T(0.0);
  for (int d = 0; d < 3; ++d) {
    const T dxj = T(coords[3 * R + d]) - T(coords[3 * L + d]);
    asq += av[d] * av[d];
    axdx += av[d] * dxj;
    udotx += 0.5 * dxj * (T(vrtm[3 * R + d]) + T(vrtm[3 * L + d]));
  }
  const T inv_axdx = T(1.0) / axdx;
  T dqL = T(0.0), dqR = T(0.0), nonOrth = T(0.0);
  for (int d = 0; d < 3; ++d) {
    const T dxj = (T(coords[3 * R + d]) - T(coords[3 * L + d]));
    dqL += 0.5 * dxj * T(dqdx[3 * L + d]);
    dqR += 0.5 * dxj * T(dqdx[3 * R + d]);
    const T kxj = av[d] - asq * inv_axdx * dxj;
    nonOrth += -viscIp * kxj * 0.5 * (T(dqdx[3 * R + d]) + T(dqdx[3 * L + d]));
  }
  const T pecnum = tabs(udotx) / (diffIp + T(eps));
  T pecfac;
  if (o->tanh_form) {
    pecfac = 0.50 * (T(1.0) + ttanh((pecnum - T(o->tanh_trans)) / T(o->tanh_width)));
  } else {
    const T mm = T(o->hybrid_factor) * pecnum;
    pecfac = mm * mm / (T(5.0) + mm * mm);
  }
  const T om_pecfac = T(1.0) - pecfac;
  T limitL = T(1.0), limitR = T(1.0);
  if (o->use_limiter) {
    const T dq = qNp1R - qNp1L;
    const T dqML = 4.0 * dqL - dq;
    const T dqMR = 4.0 * dqR - dq;
    limitL = tvan_leer(dqML, dq, eps);
    limitR = tvan_leer(dqMR, dq, eps);
  }
  const T qIpL = qNp1L + dqL * hoUpwind * limitL;
  const T qIpR = qNp1R - dqR * hoUpwind * limitR;
  const T lhsfac = -viscIp * asq * inv_axdx;
  const T diffFlux = lhsfac * (qNp1R - qNp1L) + nonOrth;
  A[0] = -lhsfac / T(relaxFac);
  A[1] = lhsfac;
  b[0] = -diffFlux;
  A[2] = lhsfac;
  A[3] = -lhsfac / T(relaxFac);
  b[1] = diffFlux;
  const T qIp = 0.5 * (qNp1R + qNp1L);
  const T qUpw = (mdot > 0) ? (alphaUpw * qIpL + om_alphaUpw * qIp)
                            : (alphaUpw * qIpR + om_alphaUpw * qIp);
  const T qHatL = (alpha * qIpL + om_alpha * qIp);
  const T qHatR = (alpha * qIpR + om_alpha * qIp);
  const T qCds = 0.5 * (qHatL + qHatR);
  const T adv_flux = mdot * (pecfac * qUpw + om_pecfac * qCds);
  b[0] -= adv_flux;
  b[1] += adv_flux;
  T alhsfac = 0.5 * (mdot + tabs(mdot)) * pecfac * alphaUpw +
              0.5 * alpha * om_pecfac * mdot;
  A[0] += alhsfac / T(relaxFac);
  A[2] -= alhsfac;
  alhsfac = 0.5 * (mdot - tabs(mdot)) * pecfac * alphaUpw +
            0.5 * alpha * om_pecfac * mdot;
  A[3] -= alhsfac / T(relaxFac);
  A[1] += alhsfac;
  alhsfac = 0.5 * mdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
  A[0] += alhsfac / T(relaxFac);
  A[1] += alhsfac;
  A[2] -= alhsfac;
  A[3] -= alhsfac / T(relaxFac);
}

// ContinuityEdgeSolverAlg::execute (src/edge_kernels/
// ContinuityEdgeSolverAlg.C:37-195) without balanced buoyancy or GCL terms.
template <typename T>
void continuity_edge(int64_t e, const int64_t* edges, const double* coords,
                     const double* velocity, const double* Gpdx,
                     const double* density, const double* pressure,
                     const double* udiag, const double* area,
                     const or_continuity_opts* o, T* A, T* b) {
  const double nocFac = o->noc_fac, tauScale = o->tau_scale;
  const double interpTogether = o->interp_together;
  const double om_interpTogether = 1.0 - interpTogether;
  const double solveIncompressibleEqn = o->solve_incompressible;
  const double om_solveIncompressibleEqn = 1.0 - solveIncompressibleEqn;
  const int64_t L = edges[2 * e], R = edges[2 * e + 1];
  T av[3];
  for (int d = 0; d < 3; ++d) av[d] = T(area[3 * e + d]);
  const T pressureL = T(pressure[L]), pressureR = T(pressure[R]);
  const T densityL = T(density[L]), densityR = T(density[R]);
  const T udiagL = T(udiag[L]), udiagR = T(udiag[R]);
  const T projTimeScale = 0.5 * (T(1.0) / udiagL + T(1.0) / udiagR);
  const T rhoIp = 0.5 * (densityL + densityR);
  const T denScale = (T(1.0) / rhoIp) * solveIncompressibleEqn +
                     T(om_solveIncompressibleEqn);
  T axdx = T(0.0), asq = T(0.0);
  for (int d = 0; d < 3; ++d) {
    const T dxj = T(coords[3 * R + d]) - T(coords[3 * L + d]);
    asq += av[d] * av[d];
    axdx += av[d] * dxj;
  }
  const T inv_axdx = T(1.0) / axdx;
  T tmdot = -projTimeScale * (pressureR - pressureL) * asq * inv_axdx;
  for (int d = 0; d < 3; ++d) {
    const T dxj = T(coords[3 * R + d]) - T(coords[3 * L + d]);
    const T kxj = av[d] - asq * inv_axdx * dxj;
    const T rhoUjIp = 0.5 * (densityR * T(velocity[3 * R + d]) +
                             densityL * T(velocity[3 * L + d]));
    const T ujIp = 0.5 * (T(velocity[3 * R + d]) + T(velocity[3 * L + d]));
    const T GjIp =
        0.5 * (T(Gpdx[3 * R + d]) / (udiagR) + T(Gpdx[3 * L + d]) / (udiagL));
    tmdot += (interpTogether * rhoUjIp + om_interpTogether * rhoIp * ujIp +
              GjIp) * av[d] - kxj * GjIp * nocFac;
  }
  tmdot /= T(tauScale);
  tmdot *= denScale;
  const T lhsfac = -asq * inv_axdx * projTimeScale * denScale / T(tauScale);
  A[0] = -lhsfac;
  A[1] = +lhsfac;
  A[2] = +lhsfac;
  A[3] = -lhsfac;
  b[0] = -tmdot;
  b[1] = tmdot;
}

// MomentumEdgeSolverAlg::execute (src/edge_kernels/MomentumEdgeSolverAlg.C:
// 70-313) with the VOF branch off (realm_has_vof_ = 0).
template <typename T>
void momentum_edge(int64_t e, const int64_t* edges, const double* coords,
                   const double* vel, const double* dudx,
                   const double* viscosity, const double* maskNodeField,
                   const double* area, const double* mdotA, const double* pecA,
                   const or_momentum_opts* o, T* A, T* b) {
  const double eps = 1.0e-16;
  const int ndim = 3;
  const double includeDivU = o->include_div_u, alpha = o->alpha,
               alphaUpw = o->alpha_upw, hoUpwind = o->upw_factor,
               relaxFacU = o->relax;
  const double om_alpha = 1.0 - alpha, om_alphaUpw = 1.0 - alphaUpw;
  const int64_t L = edges[2 * e], R = edges[2 * e + 1];
  for (int k = 0; k < 36; ++k) A[k] = T(0.0);
  for (int k = 0; k < 6; ++k) b[k] = T(0.0);
  auto lhsr = [&](int r, int c) -> T& { return A[6 * r + c]; };
  T av[3];
  for (int d = 0; d < ndim; ++d) av[d] = T(area[3 * e + d]);
  const T mdot = T(mdotA[e]);
  const T viscosityL = T(viscosity[L]), viscosityR = T(viscosity[R]);
  const T viscIp = 0.5 * (viscosityL + viscosityR);
  T axdx = T(0.0), asq = T(0.0);
  for (int d = 0; d < ndim; ++d) {
    const T dxj = T(coords[3 * R + d]) - T(coords[3 * L + d]);
    asq += av[d] * av[d];
    axdx += av[d] * dxj;
  }
  const T inv_axdx = T(1.0) / axdx;
  T duL[3], duR[3];
  for (int i = 0; i < ndim; ++i) {
    const int offset = i * ndim;
    duL[i] = T(0.0);
    duR[i] = T(0.0);
    for (int j = 0; j < ndim; ++j) {
      const T dxj = 0.5 * (T(coords[3 * R + j]) - T(coords[3 * L + j]));
      duL[i] += dxj * T(dudx[9 * L + offset + j]);
      duR[i] += dxj * T(dudx[9 * R + offset + j]);
    }
  }
  T limitL[3] = {T(1.0), T(1.0), T(1.0)}, limitR[3] = {T(1.0), T(1.0), T(1.0)};
  if (o->use_limiter) {
    for (int d = 0; d < ndim; ++d) {
      const T du = T(vel[3 * R + d]) - T(vel[3 * L + d]);
      const T duML = 4.0 * duL[d] - du;
      const T duMR = 4.0 * duR[d] - du;
      limitL[d] = tvan_leer(duML, du, eps);
      limitR[d] = tvan_leer(duMR, du, eps);
    }
  }
  const T pecfac = T(pecA[e]);
  const T om_pecfac = T(1.0) - pecfac;
  const double density_upwinding_factor = 1.0;
  T uIpL[3], uIpR[3];
  for (int d = 0; d < ndim; ++d) {
    uIpL[d] = T(vel[3 * L + d]) +
              duL[d] * hoUpwind * limitL[d] * density_upwinding_factor;
    uIpR[d] = T(vel[3 * R + d]) -
              duR[d] * hoUpwind * limitR[d] * density_upwinding_factor;
  }
  T duidxj[3][3];
  for (int i = 0; i < ndim; ++i) {
    const T dui = T(vel[3 * R + i]) - T(vel[3 * L + i]);
    const int offset = i * ndim;
    T gjuidx = T(0.0);
    for (int j = 0; j < ndim; ++j) {
      const T dxj = T(coords[3 * R + j]) - T(coords[3 * L + j]);
      const T gjui =
          0.5 * (T(dudx[9 * R + offset + j]) + T(dudx[9 * L + offset + j]));
      gjuidx += gjui * dxj;
    }
    for (int j = 0; j < ndim; ++j) {
      const T gjui =
          0.5 * (T(dudx[9 * R + offset + j]) + T(dudx[9 * L + offset + j]));
      duidxj[i][j] = gjui + (dui - gjuidx) * av[j] * inv_axdx;
    }
  }
  const T dlhsfac = -viscIp * asq * inv_axdx;
  for (int i = 0; i < ndim; ++i) {
    const int rowL = i, rowR = i + ndim;
    const T uiIp = 0.5 * (T(vel[3 * R + i]) + T(vel[3 * L + i]));
    const T uiUpw = (mdot > 0.0) ? (alphaUpw * uIpL[i] + om_alphaUpw * uiIp)
                                 : (alphaUpw * uIpR[i] + om_alphaUpw * uiIp);
    const T uiHatL = (alpha * uIpL[i] + om_alpha * uiIp);
    const T uiHatR = (alpha * uIpR[i] + om_alpha * uiIp);
    const T uiCds = 0.5 * (uiHatL + uiHatR);
    const T adv_flux = mdot * (pecfac * uiUpw + om_pecfac * uiCds);
    T diff_flux = T(0.0);
    for (int j = 0; j < ndim; ++j) diff_flux += duidxj[j][j];
    diff_flux *= 2.0 / 3.0 * viscIp * av[i] * includeDivU;
    for (int j = 0; j < ndim; ++j)
      diff_flux += -viscIp * (duidxj[i][j] + duidxj[j][i]) * av[j];
    const T maskNode = tmin(T(maskNodeField[L]), T(maskNodeField[R]));
    const T total_flux = adv_flux + diff_flux * maskNode;
    b[rowL] -= total_flux;
    b[rowR] += total_flux;
    T alhsfac = 0.5 * (mdot + tabs(mdot)) * pecfac * alphaUpw +
                0.5 * alpha * om_pecfac * mdot;
    lhsr(rowL, rowL) += alhsfac / T(relaxFacU);
    lhsr(rowR, rowL) -= alhsfac;
    alhsfac = 0.5 * (mdot - tabs(mdot)) * pecfac * alphaUpw +
              0.5 * alpha * om_pecfac * mdot;
    lhsr(rowR, rowR) -= alhsfac / T(relaxFacU);
    lhsr(rowL, rowR) += alhsfac;
    alhsfac = 0.5 * mdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
    lhsr(rowL, rowL) += alhsfac / T(relaxFacU);
    lhsr(rowL, rowR) += alhsfac;
    lhsr(rowR, rowL) -= alhsfac;
    lhsr(rowR, rowR) -= alhsfac / T(relaxFacU);
    lhsr(rowL, rowL) -= dlhsfac / T(relaxFacU);
    lhsr(rowL, rowR) += dlhsfac;
    lhsr(rowR, rowL) += dlhsfac;
    lhsr(rowR, rowR) -= dlhsfac / T(relaxFacU);
    for (int j = 0; j < ndim; ++j) {
      const T lhsfacNS = -viscIp * av[i] * av[j] * inv_axdx;
      const int colL = j, colR = j + ndim;
      lhsr(rowL, colL) -= lhsfacNS / T(relaxFacU);
      lhsr(rowL, colR) += lhsfacNS;
      lhsr(rowR, colL) += lhsfacNS;
      lhsr(rowR, colR) -= lhsfacNS / T(relaxFacU);
    }
  }
}

// Store value (mode 0) or running magnitude (mode 1) of the local systems.
template <typename T>
inline double pick(const T& x, int mode) {
  return mode ? mag(x) : val(x);
}

template <typename T, typename F>
void run_local(int64_t nedges, int nl, double* lhs, double* rhs, int mode,
               F&& f) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int64_t e = 0; e < nedges; ++e) {
    T A[36], b[6];
    f(e, A, b);
    for (int k = 0; k < nl * nl; ++k) lhs[int64_t(nl) * nl * e + k] = pick(A[k], mode);
    for (int k = 0; k < nl; ++k) rhs[int64_t(nl) * e + k] = pick(b[k], mode);
  }
}

}  // namespace

extern "C" {

void or_scalar_edge_local(int64_t nedges, const int64_t* edges,
                          const double* coords, const double* vrtm,
                          const double* q, const double* dqdx,
                          const double* density, const double* dflux,
                          const double* area, const double* mdotA,
                          const or_scalar_opts* o, double* lhs, double* rhs) {
  run_local<double>(nedges, 2, lhs, rhs, 0, [&](int64_t e, double* A, double* b) {
    scalar_edge<double>(e, edges, coords, vrtm, q, dqdx, density, dflux, area, mdotA, o, A, b);
  });
}

void or_scalar_edge_local_mag(int64_t nedges, const int64_t* edges,
                              const double* coords, const double* vrtm,
                              const double* q, const double* dqdx,
                              const double* density, const double* dflux,
                              const double* area, const double* mdotA,
                              const or_scalar_opts* o, double* lhs, double* rhs) {
  run_local<Mag>(nedges, 2, lhs, rhs, 1, [&](int64_t e, Mag* A, Mag* b) {
    scalar_edge<Mag>(e, edges, coords, vrtm, q, dqdx, density, dflux, area, mdotA, o, A, b);
  });
}

void or_continuity_edge_local(int64_t nedges, const int64_t* edges,
                              const double* coords, const double* velocity,
                              const double* Gpdx, const double* density,
                              const double* pressure, const double* udiag,
                              const double* area, const or_continuity_opts* o,
                              double* lhs, double* rhs) {
  run_local<double>(nedges, 2, lhs, rhs, 0, [&](int64_t e, double* A, double* b) {
    continuity_edge<double>(e, edges, coords, velocity, Gpdx, density, pressure, udiag, area, o, A, b);
  });
}

void or_continuity_edge_local_mag(int64_t nedges, const int64_t* edges,
                                  const double* coords, const double* velocity,
                                  const double* Gpdx, const double* density,
                                  const double* pressure, const double* udiag,
                                  const double* area, const or_continuity_opts* o,
                                  double* lhs, double* rhs) {
  run_local<Mag>(nedges, 2, lhs, rhs, 1, [&](int64_t e, Mag* A, Mag* b) {
    continuity_edge<Mag>(e, edges, coords, velocity, Gpdx, density, pressure, udiag, area, o, A, b);
  });
}

void or_momentum_edge_local(int64_t nedges, const int64_t* edges,
                            const double* coords, const double* vrtm,
                            const double* vel, const double* dudx,
                            const double* viscosity, const double* density,
                            const double* maskNodeField, const double* area,
                            const double* mdotA, const double* pecA,
                            const or_momentum_opts* o, double* lhs,
                            double* rhs) {
  (void)vrtm;
  (void)density;
  run_local<double>(nedges, 6, lhs, rhs, 0, [&](int64_t e, double* A, double* b) {
    momentum_edge<double>(e, edges, coords, vel, dudx, viscosity, maskNodeField, area, mdotA, pecA, o, A, b);
  });
}

void or_momentum_edge_local_mag(int64_t nedges, const int64_t* edges,
                                const double* coords, const double* vrtm,
                                const double* vel, const double* dudx,
                                const double* viscosity, const double* density,
                                const double* maskNodeField, const double* area,
                                const double* mdotA, const double* pecA,
                                const or_momentum_opts* o, double* lhs,
                                double* rhs) {
  (void)vrtm;
  (void)density;
  run_local<Mag>(nedges, 6, lhs, rhs, 1, [&](int64_t e, Mag* A, Mag* b) {
    momentum_edge<Mag>(e, edges, coords, vel, dudx, viscosity, maskNodeField, area, mdotA, pecA, o, A, b);
  });
}

// TpetraLinearSystem::sum_into (src/TpetraLinearSystem.C:1381-1459) with
// sum_into_row (:1337-1379) and sum_into_row_vec_3 (:1293-1335): local ids
// sorted with their permutation, one forward scan per row. Serial adds in
// edge order; threaded adds use atomics (forceAtomic branch).
void or_sum_into_edges(int64_t nedges, const int64_t* edges, int num_dof,
                       const double* lhs, const double* rhs,
                       const int64_t* node_lid, const int64_t* row_ptr,
                       const int32_t* col_idx, double* vals, double* rhs_out,
                       double* vals_abs, double* rhs_abs, int nthreads) {
  const int n_obj = 2;
  const int numRows = n_obj * num_dof;
  const int ldl = numRows;
  const bool atomic = nthreads > 1;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int64_t e = 0; e < nedges; ++e) {
    int32_t localIds[6];
    int sortPermutation[6];
    for (int i = 0; i < n_obj; ++i) {
      const int64_t off = node_lid[edges[2 * e + i]];
      for (int d = 0; d < num_dof; ++d) localIds[i * num_dof + d] = int32_t(off + d);
    }
    for (int i = 0; i < numRows; ++i) sortPermutation[i] = i;
    // shell sort of (keys, values) as Tpetra::Details::shellSortKeysAndValues
    for (int gap = numRows / 2; gap > 0; gap /= 2)
      for (int i = gap; i < numRows; ++i)
        for (int j = i - gap; j >= 0 && localIds[j] > localIds[j + gap];
             j -= gap) {
          std::swap(localIds[j], localIds[j + gap]);
          std::swap(sortPermutation[j], sortPermutation[j + gap]);
        }
    const double* L = lhs + int64_t(numRows) * numRows * e;
    const double* B = rhs + int64_t(numRows) * e;
    for (int r = 0; r < numRows; ++r) {
      const int i = sortPermutation[r] / num_dof;
      const int64_t rowLid = node_lid[edges[2 * e + i]] + sortPermutation[r] % num_dof;
      const int cur = sortPermutation[r];
      const double* cur_lhs = L + ldl * cur;
      const int64_t rs = row_ptr[rowLid], length = row_ptr[rowLid + 1] - rs;
      auto add = [&](int64_t slot, double v) {
        if (atomic) {
#ifdef _OPENMP
#pragma omp atomic
#endif
          vals[slot] += v;
        } else {
          vals[slot] += v;
        }
        if (vals_abs) {
          if (atomic) {
#ifdef _OPENMP
#pragma omp atomic
#endif
            vals_abs[slot] += std::abs(v);
          } else {
            vals_abs[slot] += std::abs(v);
          }
        }
      };
      if (num_dof == 3) {
        int64_t offset = 0;
        for (int j = 0; j < n_obj; ++j) {
          const int id_index = 3 * j;
          const int32_t col = localIds[id_index];
          bool found = true;
          while (col_idx[rs + offset] != col) {
            offset += 3;
            if (offset >= length) {
              found = false;
              break;
            }
          }
          if (!found) break;
          const int eo = sortPermutation[id_index];
          add(rs + offset + 0, cur_lhs[eo + 0]);
          add(rs + offset + 1, cur_lhs[eo + 1]);
          add(rs + offset + 2, cur_lhs[eo + 2]);
          offset += 3;
        }
      } else {
        int64_t offset = 0;
        const int numCols = n_obj * num_dof;
        for (int j = 0; j < numCols; ++j) {
          const int perm_index = sortPermutation[j];
          const int32_t col = localIds[j];
          while (offset < length && col_idx[rs + offset] != col) ++offset;
          if (offset < length) add(rs + offset, cur_lhs[perm_index]);
        }
      }
      const double cr = B[cur];
      if (atomic) {
#ifdef _OPENMP
#pragma omp atomic
#endif
        rhs_out[rowLid] += cr;
      } else {
        rhs_out[rowLid] += cr;
      }
      if (rhs_abs) {
        if (atomic) {
#ifdef _OPENMP
#pragma omp atomic
#endif
          rhs_abs[rowLid] += std::abs(cr);
        } else {
          rhs_abs[rowLid] += std::abs(cr);
        }
      }
    }
  }
}

// applyDirichletBCs (src/TpetraLinearSystem.C:1686-1757) with
// adjust_lhs_row (:1671-1684): owned rows get diag 1 and rhs = bc - q.
void or_apply_dirichlet(int64_t nlist, const int64_t* nodes, int num_dof,
                        int begin, int end, const double* q, const double* bc,
                        const int64_t* node_lid, const int64_t* row_ptr,
                        const int32_t* col_idx, double* vals, double* rhs) {
  for (int64_t k = 0; k < nlist; ++k) {
    const int64_t n = nodes[k];
    const int64_t base = node_lid[n];
    for (int d = begin; d < end; ++d) {
      const int64_t r = base + d;
      for (int64_t p = row_ptr[r]; p < row_ptr[r + 1]; ++p)
        vals[p] = (col_idx[p] == r) ? 1.0 : 0.0;
      rhs[r] = bc[int64_t(num_dof) * n + d] - q[int64_t(num_dof) * n + d];
    }
  }
}

// resetRows / reset_row (src/TpetraLinearSystem.C:1461-1520).
void or_reset_rows(int64_t nlist, const int64_t* nodes, int begin, int end,
                   double diag_value, double rhs_residual,
                   const int64_t* node_lid, const int64_t* row_ptr,
                   const int32_t* col_idx, double* vals, double* rhs) {
  for (int64_t k = 0; k < nlist; ++k) {
    const int64_t base = node_lid[nodes[k]];
    for (int d = begin; d < end; ++d) {
      const int64_t r = base + d;
      for (int64_t p = row_ptr[r]; p < row_ptr[r + 1]; ++p)
        vals[p] = (col_idx[p] == r) ? diag_value : 0.0;
      rhs[r] = rhs_residual;
    }
  }
}

// ---------------------------------------------------------------------------
// Krylov solvers. The reference hands these to Belos/Ifpack2 with the
// parameters set in src/LinearSolverConfig.C:37-140 (Num Blocks = kspace,
// ICGS orthogonalization, implicit residual scaled by the initial
// preconditioned residual, right preconditioning per
// src/LinearSolver.C:110) and solves from x0 = 0 (zeroSystem,
// src/TpetraLinearSystem.C:1290). The algorithms below are the textbook
// forms those parameters select.
void or_spmv(int64_t n, const int64_t* rp, const int32_t* ci, const double* v,
             const double* x, double* y, int nthreads) {
  (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(static)
#endif
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) s += v[p] * x[ci[p]];
    y[i] = s;
  }
}

}  // extern "C"

namespace {

struct Ctx {
  int64_t n;
  const int64_t* rp;
  const int32_t* ci;
  const double* v;
  int nthreads;
  std::vector<double> diag;
  std::vector<int64_t> order;
  int inner = 1;  // two-stage Gauss-Seidel: Jacobi-Richardson corrections
  std::vector<double> lu;  // ILU(0) factors (kind 6), built on first use
  std::vector<int64_t> dpos;
};

// Ifpack2 RILUK at its default level of fill 0 (the reference's "riluk",
// src/LinearSolverConfig.C:109-112, with no further parameters): ILU(0) on
// the matrix pattern in the IKJ form (Saad, Iterative Methods for Sparse
// Linear Systems, 2003, Algorithm 10.4): for each row i and each entry
// k < i in column order, l_ik = a_ik / u_kk, then a_ij -= l_ik u_kj for the
// row's entries j > k present in row k.
void ilu0_factor(Ctx& c) {
  const int64_t n = c.n;
  c.lu.assign(c.v, c.v + c.rp[n]);
  c.dpos.assign(n, -1);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t p = c.rp[i]; p < c.rp[i + 1]; ++p)
      if (c.ci[p] == i) c.dpos[i] = p;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t e = c.rp[i + 1];
    for (int64_t p = c.rp[i]; p < e; ++p) {
      const int64_t k = c.ci[p];
      if (k >= i) break;
      const double l = c.lu[p] / c.lu[c.dpos[k]];
      c.lu[p] = l;
      int64_t qk = c.dpos[k] + 1;
      const int64_t ek = c.rp[k + 1];
      for (int64_t q = p + 1; q < e; ++q) {
        const int64_t j = c.ci[q];
        while (qk < ek && c.ci[qk] < j) ++qk;
        if (qk < ek && c.ci[qk] == j) c.lu[q] = c.lu[q] - l * c.lu[qk];
      }
    }
  }
}

// y = U^-1 L^-1 x (L unit lower, U upper, both in lu)
void ilu0_solve(const Ctx& c, const double* x, double* y) {
  const int64_t n = c.n;
  for (int64_t i = 0; i < n; ++i) {
    double s = x[i];
    for (int64_t p = c.rp[i]; p < c.dpos[i]; ++p) s = s - c.lu[p] * y[c.ci[p]];
    y[i] = s;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int64_t p = c.dpos[i] + 1; p < c.rp[i + 1]; ++p) s = s - c.lu[p] * y[c.ci[p]];
    y[i] = s / c.lu[c.dpos[i]];
  }
}

double dot(const Ctx& c, const double* a, const double* b) {
  double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) reduction(+ : s) schedule(static)
#endif
  for (int64_t i = 0; i < c.n; ++i) s += a[i] * b[i];
  return s;
}

// Two-stage triangular solve: g ~= (D + T)^-1 r with T the strictly lower
// (upper = false) or upper part in row order, by `inner` Jacobi-Richardson
// corrections g <- D^-1 (r - T g) of g = D^-1 r.
void two_stage_tri(const Ctx& c, bool upper, const double* r, double* g) {
  const int64_t n = c.n;
  std::vector<double> prev(n);
  for (int64_t i = 0; i < n; ++i) g[i] = r[i] / c.diag[i];
  for (int k = 0; k < c.inner; ++k) {
    std::copy(g, g + n, prev.begin());
    for (int64_t i = 0; i < n; ++i) {
      double s = r[i];
      for (int64_t p = c.rp[i]; p < c.rp[i + 1]; ++p)
        if (upper ? c.ci[p] > i : c.ci[p] < i) s -= c.v[p] * prev[c.ci[p]];
      g[i] = s / c.diag[i];
    }
  }
}

// Ifpack2 Relaxation, 1 sweep, zero starting solution: Jacobi y = D^-1 x;
// symmetric Gauss-Seidel = forward sweep then backward sweep over `order`;
// kind 4, two-stage symmetric Gauss-Seidel ("sgs2",
// src/LinearSolverConfig.C:97-104): the forward sweep x1 = (D + L)^-1 b
// and the backward correction x = x1 + (D + U)^-1 (b - A x1), each
// triangular solve replaced by the two-stage approximation above
// (Berger-Vergiat et al., "Two-stage Gauss-Seidel preconditioners and
// smoothers for Krylov solvers on a GPU cluster", 2021).
void precond(Ctx& c, int kind, const double* x, double* y) {
  const int64_t n = c.n;
  if (kind == 6) {
    if (c.lu.empty()) ilu0_factor(c);
    ilu0_solve(c, x, y);
    return;
  }
  if (kind == 4) {
    std::vector<double> r(n), h(n);
    two_stage_tri(c, false, x, y);
    or_spmv(n, c.rp, c.ci, c.v, y, r.data(), 1);
    for (int64_t i = 0; i < n; ++i) r[i] = x[i] - r[i];
    two_stage_tri(c, true, r.data(), h.data());
    for (int64_t i = 0; i < n; ++i) y[i] += h[i];
    return;
  }
  if (kind == 0) {
    std::copy(x, x + n, y);
  } else if (kind == 1) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
    for (int64_t i = 0; i < n; ++i) y[i] = x[i] / c.diag[i];
  } else {
    std::fill(y, y + n, 0.0);
    auto relax = [&](int64_t i) {
      double s = x[i];
      for (int64_t p = c.rp[i]; p < c.rp[i + 1]; ++p)
        if (c.ci[p] != i) s -= c.v[p] * y[c.ci[p]];
      y[i] = s / c.diag[i];
    };
    for (int64_t k = 0; k < n; ++k) relax(c.order.empty() ? k : c.order[k]);
    for (int64_t k = n - 1; k >= 0; --k)
      relax(c.order.empty() ? k : c.order[k]);
  }
}

}  // namespace

extern "C" {

void or_precond_apply(int64_t n, const int64_t* rp, const int32_t* ci,
                      const double* v, int kind, const int64_t* order,
                      const double* x, double* y, int inner_sweeps) {
  Ctx c{n, rp, ci, v, 1, {}, {}};
  c.inner = inner_sweeps;
  c.diag.assign(n, 0.0);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p)
      if (ci[p] == i) c.diag[i] = v[p];
  if (order) c.order.assign(order, order + n);
  precond(c, kind, x, y);
}

// Right-preconditioned restarted GMRES(kspace) with two-pass classical
// Gram-Schmidt (ICGS) and Givens rotations; the implicit residual |g_{j+1}|
// relative to ||r0|| = ||b|| (x0 = 0) is tested after every iteration. On
// restart the residual is recomputed explicitly. CG: preconditioned
// conjugate gradients with the same relative test on ||r||.
int or_solve(int64_t n, const int64_t* rp, const int32_t* ci, const double* v,
             const double* b, double* x, int method, int pc,
             const int64_t* order, int m, int maxit, double tol,
             double* history, or_solve_report* rep, int nthreads,
             int inner_sweeps) {
  Ctx c{n, rp, ci, v, nthreads > 0 ? nthreads : 1, {}, {}};
  c.inner = inner_sweeps;
  c.diag.assign(n, 0.0);
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
  for (int64_t i = 0; i < n; ++i)
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p)
      if (ci[p] == i) c.diag[i] = v[p];
  if (order) c.order.assign(order, order + n);
  std::fill(x, x + n, 0.0);
  const double bnorm = std::sqrt(dot(c, b, b));
  or_solve_report r{};
  r.rhs_norm = bnorm;
  int its = 0;
  if (history) history[0] = 1.0;
  if (bnorm == 0.0) {
    r.converged = 1;
    if (rep) *rep = r;
    return 0;
  }
  std::vector<double> res(b, b + n), w(n), z(n);
  double rel = 1.0;
  if (method == 1) {  // CG
    std::vector<double> p(n), q(n);
    precond(c, pc, res.data(), z.data());
    p = z;
    double rz = dot(c, res.data(), z.data());
    while (its < maxit) {
      or_spmv(n, rp, ci, v, p.data(), q.data(), c.nthreads);
      const double alpha = rz / dot(c, p.data(), q.data());
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) {
        x[i] += alpha * p[i];
        res[i] -= alpha * q[i];
      }
      ++its;
      rel = std::sqrt(dot(c, res.data(), res.data())) / bnorm;
      if (history) history[its] = rel;
      if (rel <= tol) break;
      precond(c, pc, res.data(), z.data());
      const double rzn = dot(c, res.data(), z.data());
      const double beta = rzn / rz;
      rz = rzn;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
  } else if (method == 3) {  // BiCGStab
    // van der Vorst (1992), right preconditioned: the iterate x and the
    // recursively updated residual r of A M^-1 y = b, x = M^-1 y.
    std::vector<double> rh(res), p(n, 0.0), vv(n, 0.0), ph(n), sv(n), sh(n), t(n);
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    bool broke = false;
    while (its < maxit) {
      const double rho_n = dot(c, rh.data(), res.data());
      if (rho_n == 0.0 || omega == 0.0) { broke = true; break; }
      const double beta = (rho_n / rho) * (alpha / omega);
      rho = rho_n;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) p[i] = res[i] + beta * (p[i] - omega * vv[i]);
      precond(c, pc, p.data(), ph.data());
      or_spmv(n, rp, ci, v, ph.data(), vv.data(), c.nthreads);
      const double rv = dot(c, rh.data(), vv.data());
      if (rv == 0.0) { broke = true; break; }
      alpha = rho / rv;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) sv[i] = res[i] - alpha * vv[i];
      precond(c, pc, sv.data(), sh.data());
      or_spmv(n, rp, ci, v, sh.data(), t.data(), c.nthreads);
      const double tt = dot(c, t.data(), t.data());
      omega = tt > 0.0 ? dot(c, t.data(), sv.data()) / tt : 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) {
        x[i] += alpha * ph[i] + omega * sh[i];
        res[i] = sv[i] - omega * t[i];
      }
      ++its;
      rel = std::sqrt(dot(c, res.data(), res.data())) / bnorm;
      if (history) history[its] = rel;
      if (rel <= tol) break;
    }
    (void)broke;  // a breakdown ends the iteration unconverged
  } else if (method == 4) {  // TFQMR
    // Freund (1993), as in Saad, Iterative Methods for Sparse Linear
    // Systems (2003), Algorithm 7.8, on A M^-1 with the direction vectors
    // kept in the unpreconditioned space (dh = M^-1 d), so x is updated
    // directly. One iteration = the even and the odd half step (two
    // products with A M^-1); convergence is tested after each iteration on
    // the bound ||r_k|| <= sqrt(k + 1) tau_k (k = half steps).
    std::vector<double> wv(res), u(res), uh(n), Au(n), Au_n(n), vv(n), dh(n, 0.0), rt(res);
    precond(c, pc, u.data(), uh.data());
    or_spmv(n, rp, ci, v, uh.data(), Au.data(), c.nthreads);
    vv = Au;
    double tau = bnorm, theta = 0.0, eta = 0.0, alpha = 0.0;
    double rho = dot(c, rt.data(), res.data());
    for (int64_t mm = 0; its < maxit; ++mm) {
      if (mm % 2 == 0) {
        const double vr = dot(c, vv.data(), rt.data());
        if (vr == 0.0) break;
        alpha = rho / vr;
      }
      const double coef = alpha != 0.0 ? theta * theta / alpha * eta : 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) {
        wv[i] -= alpha * Au[i];
        dh[i] = uh[i] + coef * dh[i];
      }
      theta = std::sqrt(dot(c, wv.data(), wv.data())) / tau;
      const double cc = 1.0 / std::sqrt(1.0 + theta * theta);
      tau = tau * theta * cc;
      eta = cc * cc * alpha;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) x[i] += eta * dh[i];
      if (mm % 2 == 0) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
        for (int64_t i = 0; i < n; ++i) u[i] -= alpha * vv[i];
        precond(c, pc, u.data(), uh.data());
        or_spmv(n, rp, ci, v, uh.data(), Au_n.data(), c.nthreads);
        std::swap(Au, Au_n);  // Au = A M^-1 u_{m+1}
      } else {
        ++its;
        rel = std::sqrt(double(mm + 2)) * tau / bnorm;
        if (history) history[its] = rel;
        if (rel <= tol) break;
        const double rho_n = dot(c, wv.data(), rt.data());
        if (rho == 0.0) break;
        const double beta = rho_n / rho;
        rho = rho_n;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
        for (int64_t i = 0; i < n; ++i) u[i] = wv[i] + beta * u[i];
        precond(c, pc, u.data(), uh.data());
        // Au holds A M^-1 u_m; Au_n gets A M^-1 u_{m+1}
        or_spmv(n, rp, ci, v, uh.data(), Au_n.data(), c.nthreads);
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
        for (int64_t i = 0; i < n; ++i) vv[i] = Au_n[i] + beta * (Au[i] + beta * vv[i]);
        std::swap(Au, Au_n);
      }
    }
  } else {  // GMRES(m)
    std::vector<double> V(size_t(n) * (m + 1));
    std::vector<double> H(size_t(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m);
    std::vector<double> h(m + 1), h2(m + 1);
    double beta = bnorm;
    bool done = false;
    while (!done && its < maxit) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) V[i] = res[i] / beta;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      for (; j < m && its < maxit; ++j) {
        double* vj = V.data() + size_t(n) * j;
        double* vn = V.data() + size_t(n) * (j + 1);
        precond(c, pc, vj, z.data());
        or_spmv(n, rp, ci, v, z.data(), w.data(), c.nthreads);
        for (int k = 0; k <= j; ++k) h[k] = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
          for (int k = 0; k <= j; ++k)
            h2[k] = dot(c, V.data() + size_t(n) * k, w.data());
          for (int k = 0; k <= j; ++k) {
            const double* vk = V.data() + size_t(n) * k;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
            for (int64_t i = 0; i < n; ++i) w[i] -= h2[k] * vk[i];
            h[k] += h2[k];
          }
        }
        const double hn = std::sqrt(dot(c, w.data(), w.data()));
        for (int k = 0; k <= j; ++k) H[size_t(k) * m + j] = h[k];
        H[size_t(j + 1) * m + j] = hn;
        if (hn != 0.0)
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
          for (int64_t i = 0; i < n; ++i) vn[i] = w[i] / hn;
        for (int k = 0; k < j; ++k) {
          const double a = H[size_t(k) * m + j], bb = H[size_t(k + 1) * m + j];
          H[size_t(k) * m + j] = cs[k] * a + sn[k] * bb;
          H[size_t(k + 1) * m + j] = -sn[k] * a + cs[k] * bb;
        }
        const double a = H[size_t(j) * m + j], bb = H[size_t(j + 1) * m + j];
        const double den = std::sqrt(a * a + bb * bb);
        cs[j] = a / den;
        sn[j] = bb / den;
        H[size_t(j) * m + j] = den;
        H[size_t(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        ++its;
        rel = std::abs(g[j + 1]) / bnorm;
        if (history) history[its] = rel;
        if (rel <= tol || hn == 0.0) {
          done = true;
          ++j;
          break;
        }
      }
      // y = H^-1 g, x += M^-1 (V y)
      const int kk = j;
      for (int i = kk - 1; i >= 0; --i) {
        double s = g[i];
        for (int l = i + 1; l < kk; ++l) s -= H[size_t(i) * m + l] * y[l];
        y[i] = s / H[size_t(i) * m + i];
      }
      std::fill(w.begin(), w.end(), 0.0);
      for (int l = 0; l < kk; ++l) {
        const double* vl = V.data() + size_t(n) * l;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
        for (int64_t i = 0; i < n; ++i) w[i] += y[l] * vl[i];
      }
      precond(c, pc, w.data(), z.data());
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) x[i] += z[i];
      if (done || its >= maxit) break;
      or_spmv(n, rp, ci, v, x, w.data(), c.nthreads);
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
      for (int64_t i = 0; i < n; ++i) res[i] = b[i] - w[i];
      beta = std::sqrt(dot(c, res.data(), res.data()));
      if (beta == 0.0) break;
    }
  }
  or_spmv(n, rp, ci, v, x, w.data(), c.nthreads);
#ifdef _OPENMP
#pragma omp parallel for num_threads(c.nthreads) schedule(static)
#endif
  for (int64_t i = 0; i < n; ++i) w[i] = b[i] - w[i];
  r.final_abs_explicit = std::sqrt(dot(c, w.data(), w.data()));
  r.final_rel_implicit = rel;
  r.iterations = its;
  r.converged = rel <= tol ? 1 : 0;
  if (rep) *rep = r;
  return r.converged ? 0 : 1;
}

// ---------------------------------------------------------------------------
// Input producers.
// calc_mass_flow_rate (unit_tests/kernels/UnitTestKernelUtils.C:725-769).
void or_mdot_unit_test(int64_t nedges, const int64_t* edges, const double* vel,
                       const double* rho, const double* area, double* mdot) {
  for (int64_t e = 0; e < nedges; ++e) {
    const int64_t L = edges[2 * e], R = edges[2 * e + 1];
    double t = 0.0;
    for (int d = 0; d < 3; ++d)
      t += 0.5 * (rho[L] * vel[3 * L + d] + rho[R] * vel[3 * R + d]) *
           area[3 * e + d];
    mdot[e] = t;
  }
}

// MdotEdgeAlg::execute (src/ngp_algorithms/MdotEdgeAlg.C:43-194).
void or_mdot_edge(int64_t nedges, const int64_t* edges, const double* coords,
                  const double* velocity, const double* Gpdx,
                  const double* density, const double* pressure,
                  const double* udiag, const double* area, double nocFac,
                  double interpTogether, double* mdot) {
  const double om_interpTogether = 1.0 - interpTogether;
  for (int64_t e = 0; e < nedges; ++e) {
    const int64_t L = edges[2 * e], R = edges[2 * e + 1];
    const double* av = area + 3 * e;
    const double projTimeScale = 0.5 * (1.0 / udiag[L] + 1.0 / udiag[R]);
    const double rhoIp = 0.5 * (density[L] + density[R]);
    double axdx = 0.0, asq = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double dxj = coords[3 * R + d] - coords[3 * L + d];
      asq += av[d] * av[d];
      axdx += av[d] * dxj;
    }
    const double inv_axdx = 1.0 / axdx;
    double tmdot = -projTimeScale * (pressure[R] - pressure[L]) * asq * inv_axdx;
    for (int d = 0; d < 3; ++d) {
      const double dxj = coords[3 * R + d] - coords[3 * L + d];
      const double kxj = av[d] - asq * inv_axdx * dxj;
      const double rhoUjIp = 0.5 * (density[R] * velocity[3 * R + d] +
                                    density[L] * velocity[3 * L + d]);
      const double ujIp = 0.5 * (velocity[3 * R + d] + velocity[3 * L + d]);
      const double GjIp =
          0.5 * (Gpdx[3 * R + d] / udiag[R] + Gpdx[3 * L + d] / udiag[L]);
      tmdot += (interpTogether * rhoUjIp + om_interpTogether * rhoIp * ujIp +
                GjIp) *
                   av[d] -
               kxj * GjIp * nocFac;
    }
    mdot[e] = tmdot;
  }
}

// Lumped-mass BDF node kernels, per node: the diagonal LHS entry and the
// rhs of each dof (added by the node algorithm into the node's own row):
//   kind 0 ScalarMassBDFNodeKernel::execute
//          (src/node_kernels/ScalarMassBDFNodeKernel.C:75-97)
//   kind 1 ContinuityMassBDFNodeKernel::execute
//          (src/node_kernels/ContinuityMassBDFNodeKernel.C:60-82)
//   kind 2 MomentumMassBDFNodeKernel::execute
//          (src/node_kernels/MomentumMassBDFNodeKernel.C:78-107)
// q: scalar (N) or velocity (N x 3); dpdx: momentum only.
void or_mass_bdf(int kind, int64_t n, const double* rhoNm1, const double* rhoN,
                 const double* rhoNp1, const double* dnvNm1, const double* dnvN,
                 const double* dnvNp1, const double* qNm1, const double* qN,
                 const double* qNp1, const double* dpdx, double dt, double g1,
                 double g2, double g3, double* lhs, double* rhs) {
  for (int64_t i = 0; i < n; ++i) {
    if (kind == 0) {
      lhs[i] = g1 * rhoNp1[i] * dnvNp1[i] / dt;
      rhs[i] = -(g1 * rhoNp1[i] * qNp1[i] * dnvNp1[i] + g2 * qN[i] * rhoN[i] * dnvN[i] +
                 g3 * qNm1[i] * rhoNm1[i] * dnvNm1[i]) /
               dt;
    } else if (kind == 1) {
      lhs[i] = 0.0;
      rhs[i] = -(g1 * rhoNp1[i] * dnvNp1[i] + g2 * rhoN[i] * dnvN[i] +
                 g3 * rhoNm1[i] * dnvNm1[i]) /
               dt * (g1 / dt);
    } else {
      const double lhsfac = g1 * rhoNp1[i] * dnvNp1[i] / dt;
      for (int d = 0; d < 3; ++d) {
        lhs[3 * i + d] = lhsfac;
        rhs[3 * i + d] = -(g1 * rhoNp1[i] * qNp1[3 * i + d] * dnvNp1[i] +
                           g2 * rhoN[i] * qN[3 * i + d] * dnvN[i] +
                           g3 * rhoNm1[i] * qNm1[3 * i + d] * dnvNm1[i]) /
                             dt -
                         dpdx[3 * i + d] * dnvNp1[i];
      }
    }
  }
}

// NodalGradEdgeAlg::execute (src/ngp_algorithms/NodalGradEdgeAlg.C:58-111).
void or_nodal_grad_edge(int64_t nedges, const int64_t* edges, int dim1,
                        const double* phi, const double* area,
                        const double* dualvol, double* grad) {
  const int dim2 = 3;
  for (int64_t e = 0; e < nedges; ++e) {
    const int64_t L = edges[2 * e], R = edges[2 * e + 1];
    const double invVolL = 1.0 / dualvol[L], invVolR = 1.0 / dualvol[R];
    int counter = 0;
    for (int i = 0; i < dim1; ++i) {
      const double phiIp = 0.5 * (phi[dim1 * L + i] + phi[dim1 * R + i]);
      for (int j = 0; j < dim2; ++j) {
        const double ajPhiIp = area[3 * e + j] * phiIp;
        grad[int64_t(dim1 * dim2) * L + counter] += ajPhiIp * invVolL;
        grad[int64_t(dim1 * dim2) * R + counter] -= ajPhiIp * invVolR;
        counter++;
      }
    }
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Boundary face-IP kernels. Each face integration point contributes to the
// rows of its face node R, with columns R and L (L the element node opposite
// R across the element edge that leaves the face). The local systems use the
// edge layout with node order (R, L): lhs 2x2 (1 dof) or 6x6 (3 dofs), rhs
// 2 or 6, and the L rows left zero, so or_sum_into_edges assembles them.
namespace {

inline double tsqrt(double x) { return std::sqrt(x); }
inline Mag tsqrt(Mag x) { return {std::sqrt(x.v), std::sqrt(x.m)}; }

// ContinuityOpenEdgeKernel::execute (src/edge_kernels/
// ContinuityOpenEdgeKernel.C:92-160), one face IP.
template <typename T>
void continuity_open_ip(int64_t ip, const int64_t* ipn, const double* coords,
                        const double* velocity, const double* Gpdx,
                        const double* density, const double* pressure,
                        const double* pbcF, const double* udiag,
                        const double* areav, const double* dynp,
                        const or_continuity_open_opts* o, T* A, T* b) {
  const int64_t R = ipn[2 * ip], L = ipn[2 * ip + 1];
  const double tauScale = o->tau_scale, pstabFac = o->pstab_fac,
               nocFac = o->noc_fac, mdotCorr = o->mdot_corr,
               solveInc = o->solve_incompressible;
  T av[3];
  for (int d = 0; d < 3; ++d) av[d] = T(areav[3 * ip + d]);
  const T projTimeScale = T(1.0) / T(udiag[R]);
  const T pressureIp = 0.5 * (T(pressure[R]) + T(pressure[L]));
  T asq = T(0.0), axdx = T(0.0);
  for (int d = 0; d < 3; ++d) {
    const T coordIp = 0.5 * (T(coords[3 * R + d]) + T(coords[3 * L + d]));
    const T dxj = T(coords[3 * R + d]) - coordIp;
    asq += av[d] * av[d];
    axdx += av[d] * dxj;
  }
  const T inv_axdx = T(1.0) / axdx;
  const T pbc = T(pbcF[R]) - T(dynp ? dynp[ip] : 0.0);
  T tmdot = -projTimeScale * (pbc - pressureIp) * asq * inv_axdx * T(pstabFac) -
            T(mdotCorr);
  for (int d = 0; d < 3; ++d) {
    const T coordIp = 0.5 * (T(coords[3 * R + d]) + T(coords[3 * L + d]));
    const T dxj = T(coords[3 * R + d]) - coordIp;
    const T kxj = av[d] - asq * inv_axdx * dxj;
    const T Gjp = T(Gpdx[3 * R + d]);
    tmdot += ((T(solveInc) + T(density[R]) * T(1.0 - solveInc)) *
                  T(velocity[3 * R + d]) +
              projTimeScale * Gjp * T(pstabFac)) *
                 av[d] -
             projTimeScale * kxj * Gjp * T(nocFac) * T(pstabFac);
  }
  const T lhsfac = 0.5 * asq * inv_axdx * T(pstabFac) * projTimeScale / T(tauScale);
  for (int k = 0; k < 4; ++k) A[k] = T(0.0);
  b[0] = -tmdot / T(tauScale);
  b[1] = T(0.0);
  A[0] = lhsfac;  // (R, R)
  A[1] = lhsfac;  // (R, L)
}

// duidxj with the over-relaxed non-orthogonal correction and the viscous
// face flux shared by the open and symmetry momentum kernels
// (MomentumOpenEdgeKernel.C:137-177, MomentumSymmetryEdgeKernel.C:112-152).
template <typename T>
void face_visc_flux(int64_t ip, int64_t R, int64_t L, const double* coords,
                    const double* vel, const double* dudx, const T av[3],
                    T inv_axdx, T visc, const T nx[3], double includeDivU,
                    T fx[3], T& fxnx) {
  T duidxj[3][3];
  for (int i = 0; i < 3; ++i) {
    const T dui = T(vel[3 * R + i]) - T(vel[3 * L + i]);
    T gjuidx = T(0.0);
    for (int j = 0; j < 3; ++j) {
      const T dxj = T(coords[3 * R + j]) - T(coords[3 * L + j]);
      gjuidx += T(dudx[9 * R + 3 * i + j]) * dxj;
    }
    for (int j = 0; j < 3; ++j)
      duidxj[i][j] = T(dudx[9 * R + 3 * i + j]) + (dui - gjuidx) * av[j] * inv_axdx;
  }
  (void)ip;
  T divU = T(0.0);
  for (int d = 0; d < 3; ++d) divU += duidxj[d][d];
  fxnx = T(0.0);
  for (int i = 0; i < 3; ++i) {
    fx[i] = 2.0 / 3.0 * visc * divU * av[i] * T(includeDivU);
    for (int j = 0; j < 3; ++j) fx[i] += -visc * (duidxj[i][j] + duidxj[j][i]) * av[j];
    fxnx += nx[i] * fx[i];
  }
}

// MomentumOpenEdgeKernel::execute (src/edge_kernels/
// MomentumOpenEdgeKernel.C:80-270), one face IP; entrainment 0 = COMPUTED,
// 1 = SPECIFIED.
template <typename T>
void momentum_open_ip(int64_t ip, const int64_t* ipn, const double* coords,
                      const double* vel, const double* dudx,
                      const double* viscosity, const double* ubc,
                      const double* areav, const double* mdot,
                      const or_momentum_open_opts* o, T* A, T* b) {
  const int64_t R = ipn[2 * ip], L = ipn[2 * ip + 1];
  const double nfEntrain = o->nf_entrain, om_nfEntrain = 1.0 - nfEntrain;
  auto lhs = [&](int r, int c) -> T& { return A[6 * r + c]; };
  for (int k = 0; k < 36; ++k) A[k] = T(0.0);
  for (int k = 0; k < 6; ++k) b[k] = T(0.0);
  T av[3], nx[3], fx[3];
  for (int d = 0; d < 3; ++d) av[d] = T(areav[3 * ip + d]);
  const T visc = T(viscosity[R]);
  T axdx = T(0.0), asq = T(0.0);
  for (int d = 0; d < 3; ++d) {
    const T dxj = T(coords[3 * R + d]) - T(coords[3 * L + d]);
    asq += av[d] * av[d];
    axdx += av[d] * dxj;
  }
  const T inv_axdx = T(1.0) / axdx;
  const T amag = tsqrt(asq);
  T uxnx = T(0.0), uxnxip = T(0.0), uspecxnx = T(0.0);
  for (int d = 0; d < 3; ++d) {
    nx[d] = av[d] / amag;
    uxnx += nx[d] * T(vel[3 * R + d]);
    uxnxip += 0.5 * nx[d] * (T(vel[3 * L + d]) + T(vel[3 * R + d]));
    uspecxnx += nx[d] * T(ubc[3 * R + d]);
  }
  T fxnx;
  face_visc_flux(ip, R, L, coords, vel, dudx, av, inv_axdx, visc, nx, o->include_div_u, fx, fxnx);
  // local dofs: R = 0..2, L = 3..5
  for (int i = 0; i < 3; ++i) {
    const int rowR = i, rowL = 3 + i;
    const T axi = av[i];
    b[rowR] -= (fx[i] - nx[i] * fxnx);
    const T om_nxinxi = T(1.0) - nx[i] * nx[i];
    T lhsFac = -visc * asq * inv_axdx * om_nxinxi;
    lhs(rowR, rowL) -= lhsFac;
    lhs(rowR, rowR) += lhsFac;
    for (int j = 0; j < 3; ++j) {
      const int colL = 3 + j, colR = j;
      const T axj = av[j];
      lhsFac = -visc * axi * axj * inv_axdx * om_nxinxi;
      lhs(rowR, colL) -= lhsFac;
      lhs(rowR, colR) += lhsFac;
      if (i == j) continue;
      const T nxinxj = nx[i] * nx[j];
      lhsFac = visc * asq * inv_axdx * nxinxj;
      lhs(rowR, colL) -= lhsFac;
      lhs(rowR, colR) += lhsFac;
      lhsFac = visc * axj * axj * inv_axdx * nxinxj;
      lhs(rowR, colL) -= lhsFac;
      lhs(rowR, colR) += lhsFac;
      lhsFac = visc * axj * axi * inv_axdx * nxinxj;
      lhs(rowR, rowL) -= lhsFac;
      lhs(rowR, rowR) += lhsFac;
    }
  }
  const T tmdot = T(mdot[ip]);
  if (o->entrainment == 1) {  // SPECIFIED
    for (int i = 0; i < 3; ++i) {
      const int rowR = i;
      const T sigma = visc * asq * inv_axdx;
      const T lambda = 0.5 * (tmdot - tsqrt(tmdot * tmdot + 8.0 * sigma * sigma));
      const T uR = T(vel[3 * R + i]);
      if (tmdot > 0.0) {
        b[rowR] -= tmdot * uR;
        lhs(rowR, rowR) += tmdot;
      } else {
        b[rowR] -= tmdot * uR - lambda * (uR - T(ubc[3 * R + i]));
        lhs(rowR, rowR) += tmdot - lambda;
      }
    }
  } else {  // COMPUTED
    for (int i = 0; i < 3; ++i) {
      const int rowR = i;
      if (tmdot > 0.0) {
        b[rowR] -= tmdot * T(vel[3 * R + i]);
        lhs(rowR, rowR) += tmdot;
      } else {
        b[rowR] -= tmdot * ((T(nfEntrain) * uxnx + T(om_nfEntrain) * uxnxip) * nx[i] +
                            (T(ubc[3 * R + i]) - uspecxnx * nx[i]));
        for (int j = 0; j < 3; ++j) {
          lhs(rowR, 3 + j) += tmdot * T(om_nfEntrain) * 0.5 * nx[i] * nx[j];
          lhs(rowR, j) += tmdot * T(nfEntrain + om_nfEntrain * 0.5) * nx[i] * nx[j];
        }
      }
    }
  }
}

// MomentumSymmetryEdgeKernel::execute (src/edge_kernels/
// MomentumSymmetryEdgeKernel.C:64-206), one face IP.
template <typename T>
void momentum_symmetry_ip(int64_t ip, const int64_t* ipn, const double* coords,
                          const double* vel, const double* dudx,
                          const double* viscosity, const double* areav,
                          const or_momentum_symmetry_opts* o, T* A, T* b) {
  const int64_t R = ipn[2 * ip], L = ipn[2 * ip + 1];
  auto lhs = [&](int r, int c) -> T& { return A[6 * r + c]; };
  for (int k = 0; k < 36; ++k) A[k] = T(0.0);
  for (int k = 0; k < 6; ++k) b[k] = T(0.0);
  T av[3], nx[3], fx[3];
  for (int d = 0; d < 3; ++d) av[d] = T(areav[3 * ip + d]);
  const T visc = T(viscosity[R]);
  T axdx = T(0.0), asq = T(0.0);
  for (int d = 0; d < 3; ++d) {
    const T dxj = T(coords[3 * R + d]) - T(coords[3 * L + d]);
    asq += av[d] * av[d];
    axdx += av[d] * dxj;
  }
  const T inv_axdx = T(1.0) / axdx;
  const T amag = tsqrt(asq);
  for (int d = 0; d < 3; ++d) nx[d] = av[d] / amag;
  T fxnx;
  face_visc_flux(ip, R, L, coords, vel, dudx, av, inv_axdx, visc, nx, o->include_div_u, fx, fxnx);
  const T diffusionMassRate = -visc * asq * inv_axdx;
  const T penaltyFac = T(o->penalty_factor) * diffusionMassRate;
  T uN = T(0.0);
  for (int i = 0; i < 3; ++i) uN += T(vel[3 * R + i]) * nx[i];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) lhs(i, j) -= penaltyFac * nx[i] * nx[j];
    b[i] += penaltyFac * uN * nx[i];
  }
  for (int i = 0; i < 3; ++i) {
    const int rowL = 3 + i, rowR = i;
    b[rowR] -= fxnx * nx[i];
    T lhsfac = diffusionMassRate * nx[i] * nx[i];
    lhs(rowR, rowL) -= lhsfac;
    lhs(rowR, rowR) += lhsfac;
    const T axi = av[i];
    const T nxnx = nx[i] * nx[i];
    for (int j = 0; j < 3; ++j) {
      const int colL = 3 + j, colR = j;
      const T axj = av[j];
      lhsfac = -visc * axi * axj * inv_axdx * nxnx;
      lhs(rowR, colL) -= lhsfac;
      lhs(rowR, colR) += lhsfac;
      if (i == j) continue;
      lhsfac = -visc * asq * inv_axdx * nx[i] * nx[j];
      lhs(rowR, colL) -= lhsfac;
      lhs(rowR, colR) += lhsfac;
      // these two terms carry no 1/axdx in the reference
      lhsfac = -visc * axj * axj * nx[i] * nx[j];
      lhs(rowR, colL) -= lhsfac;
      lhs(rowR, colR) += lhsfac;
      lhsfac = -visc * axj * axi * nx[i] * nx[j];
      lhs(rowR, rowL) -= lhsfac;
      lhs(rowR, rowR) += lhsfac;
    }
  }
}

// ScalarOpenEdgeKernel::execute (src/edge_kernels/ScalarOpenEdgeKernel.C:
// 49-72) and ScalarEdgeOpenSolverAlg::execute (src/edge_kernels/
// ScalarEdgeOpenSolverAlg.C:64-104): the same upwind outflow / entrainment
// flux, one face IP.
template <typename T>
void scalar_open_ip(int64_t ip, const int64_t* ipn, const double* q,
                    const double* qbc, const double* mdot, double relax, T* A,
                    T* b) {
  const int64_t R = ipn[2 * ip];
  for (int k = 0; k < 4; ++k) A[k] = T(0.0);
  b[0] = b[1] = T(0.0);
  const T md = T(mdot[ip]);
  const T uUpw = md > 0.0 ? T(q[R]) : T(qbc[R]);
  b[0] -= md * uUpw;
  if (md > 0.0) A[0] += md / T(relax);
}

inline double tlog(double x) { return std::log(x); }
inline Mag tlog(Mag x) { return {std::log(x.v), std::abs(std::log(x.v))}; }

// Monin-Obukhov stability functions (include/wind_energy/MoninObukhov.h:
// 26-55, van der Laan et al. 2017).
inline double psim_stable(double zeta, double beta) { return -beta * zeta; }
inline double psim_unstable(double zeta, double gamma) {
  const double half_pi = 1.5707963267948966;
  const double phim = std::pow(1.0 - gamma * zeta, 0.25);
  const double term1 = 1.0 + phim * phim;
  const double term2 = 1.0 + phim;
  const double term3 = term2 * term2;
  return std::log(0.125 * term1 * term3) - 2.0 * std::atan(phim) + half_pi;
}

// MomentumABLWallFuncEdgeKernel::execute (src/edge_kernels/
// MomentumABLWallFuncEdgeKernel.C:80-158), one face IP: the wall-function
// shear on the tangential velocity of the face node R (no L coupling).
template <typename T>
void abl_wall_ip(int64_t ip, const int64_t* ipn, const double* vel, const double* bcvel,
                 const double* density, const double* heatflux, const double* cp,
                 const double* areav, const double* ustarF, const double* zhF,
                 const or_abl_wall_opts* o, T* A, T* b) {
  const int64_t R = ipn[2 * ip];
  auto lhs = [&](int r, int c) -> T& { return A[6 * r + c]; };
  for (int k = 0; k < 36; ++k) A[k] = T(0.0);
  for (int k = 0; k < 6; ++k) b[k] = T(0.0);
  const double eps = 1.0e-8, Lmax = 1.0e8;
  T av[3], nx[3];
  T amag = T(0.0);
  for (int d = 0; d < 3; ++d) {
    av[d] = T(areav[3 * ip + d]);
    amag += av[d] * av[d];
  }
  amag = tsqrt(amag);
  for (int d = 0; d < 3; ++d) nx[d] = av[d] / amag;
  // the stability correction enters through a logarithm's argument; it is
  // evaluated in FP64 (its rounding is far below the tolerance scale)
  const double zh = zhF[ip], ustar = ustarF[ip];
  const double rho = density[R];
  const double Tflux = heatflux[R] / (rho * cp[R]);
  const double Lfac = std::abs(Tflux) < eps ? Lmax : (-o->Tref / (o->kappa * o->gravity * Tflux));
  double moLen = ustar * ustar * ustar * Lfac;
  const double sign = Tflux < 0.0 ? 1.0 : -1.0;
  moLen = sign * std::max(1.0e-10, std::abs(moLen));
  const double zeta = zh / moLen;
  const double psim = Tflux < -eps ? psim_stable(zeta, o->beta_m)
                      : (Tflux > eps ? psim_unstable(zeta, o->gamma_m) : 0.0);
  const T lambda = (T(rho) * T(o->kappa) * T(ustar) / T(std::log(zh / o->z0) - psim)) * amag;
  for (int i = 0; i < 3; ++i) {
    T uiTan = T(0.0), uiBcTan = T(0.0);
    for (int j = 0; j < 3; ++j) {
      const T ninj = nx[i] * nx[j];
      if (i == j) {
        const T om = T(1.0) - ninj;
        uiTan += om * T(vel[3 * R + j]);
        uiBcTan += om * T(bcvel[3 * R + j]);
        lhs(i, i) += lambda * om;
      } else {
        uiTan -= ninj * T(vel[3 * R + j]);
        uiBcTan -= ninj * T(bcvel[3 * R + j]);
        lhs(i, j) -= lambda * ninj;
      }
    }
    b[i] -= lambda * (uiTan - uiBcTan);
  }
}

// MomentumABLWallShearStressEdgeKernel::execute (src/edge_kernels/
// MomentumABLWallShearStressEdgeKernel.C:49-88), one face IP: the given
// wall shear stress times |A| added to the rhs of the face node (slip) or
// of the opposing node (no slip).
template <typename T>
void abl_shear_ip(int64_t ip, const double* areav, const double* tau, int slip, T* A, T* b) {
  for (int k = 0; k < 36; ++k) A[k] = T(0.0);
  for (int k = 0; k < 6; ++k) b[k] = T(0.0);
  T amag = T(0.0);
  for (int d = 0; d < 3; ++d) amag += T(areav[3 * ip + d]) * T(areav[3 * ip + d]);
  amag = tsqrt(amag);
  const int base = slip ? 0 : 3;  // local node order (R, L)
  for (int i = 0; i < 3; ++i) b[base + i] += T(tau[3 * ip + i]) * amag;
}

}  // namespace

extern "C" {

#define NW_OR_BOTH(name, nl, call)                                          \
  void name(OR_ARGS) { run_local<double>(nip, nl, lhs, rhs, 0, [&](int64_t ip, double* A, double* b) { call; }); } \
  void name##_mag(OR_ARGS) { run_local<Mag>(nip, nl, lhs, rhs, 1, [&](int64_t ip, Mag* A, Mag* b) { call; }); }

#define OR_ARGS                                                                          \
  int64_t nip, const int64_t *ipn, const double *coords, const double *velocity,          \
      const double *Gpdx, const double *density, const double *pressure,                \
      const double *pbc, const double *udiag, const double *areav, const double *dynp,  \
      const or_continuity_open_opts *o, double *lhs, double *rhs
NW_OR_BOTH(or_continuity_open_local, 2,
           continuity_open_ip(ip, ipn, coords, velocity, Gpdx, density, pressure, pbc, udiag,
                              areav, dynp, o, A, b))
#undef OR_ARGS

#define OR_ARGS                                                                          \
  int64_t nip, const int64_t *ipn, const double *coords, const double *vel,               \
      const double *dudx, const double *viscosity, const double *ubc,                    \
      const double *areav, const double *mdot, const or_momentum_open_opts *o,           \
      double *lhs, double *rhs
NW_OR_BOTH(or_momentum_open_local, 6,
           momentum_open_ip(ip, ipn, coords, vel, dudx, viscosity, ubc, areav, mdot, o, A, b))
#undef OR_ARGS

#define OR_ARGS                                                                          \
  int64_t nip, const int64_t *ipn, const double *coords, const double *vel,               \
      const double *dudx, const double *viscosity, const double *areav,                  \
      const or_momentum_symmetry_opts *o, double *lhs, double *rhs
NW_OR_BOTH(or_momentum_symmetry_local, 6,
           momentum_symmetry_ip(ip, ipn, coords, vel, dudx, viscosity, areav, o, A, b))
#undef OR_ARGS

#define OR_ARGS                                                                          \
  int64_t nip, const int64_t *ipn, const double *vel, const double *bcvel,                \
      const double *density, const double *heatflux, const double *cp,                   \
      const double *areav, const double *ustar, const double *zh,                        \
      const or_abl_wall_opts *o, double *lhs, double *rhs
NW_OR_BOTH(or_abl_wall_local, 6,
           abl_wall_ip(ip, ipn, vel, bcvel, density, heatflux, cp, areav, ustar, zh, o, A, b))
#undef OR_ARGS

#define OR_ARGS                                                                          \
  int64_t nip, const int64_t *ipn, const double *areav, const double *tau, int slip,      \
      double *lhs, double *rhs
NW_OR_BOTH(or_abl_shear_local, 6, ((void)ipn, abl_shear_ip(ip, areav, tau, slip, A, b)))
#undef OR_ARGS

#define OR_ARGS                                                                          \
  int64_t nip, const int64_t *ipn, const double *q, const double *qbc,                    \
      const double *mdot, double relax, double *lhs, double *rhs
NW_OR_BOTH(or_scalar_open_local, 2, scalar_open_ip(ip, ipn, q, qbc, mdot, relax, A, b))
#undef OR_ARGS
#undef NW_OR_BOTH

// MdotOpenEdgeAlg::execute (src/ngp_algorithms/MdotOpenEdgeAlg.C:55-150):
// the open mass flow rate of each face IP (ipn as for the face kernels).
void or_mdot_open(int64_t nip, const int64_t* ipn, const double* coords,
                  const double* velocity, const double* Gpdx, const double* density,
                  const double* pressure, const double* pbcF, const double* udiag,
                  const double* areav, const double* dynp, double nocFac,
                  double pstabFac, double* mdot) {
  for (int64_t ip = 0; ip < nip; ++ip) {
    const int64_t R = ipn[2 * ip], L = ipn[2 * ip + 1];
    const double projTimeScale = pstabFac / udiag[R];
    double asq = 0.0, axdx = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double coordIp = 0.5 * (coords[3 * R + d] + coords[3 * L + d]);
      const double dxj = coords[3 * R + d] - coordIp;
      asq += areav[3 * ip + d] * areav[3 * ip + d];
      axdx += areav[3 * ip + d] * dxj;
    }
    const double inv_axdx = 1.0 / axdx;
    const double pbc = pbcF[R] - (dynp ? dynp[ip] : 0.0);
    const double pressureIp = 0.5 * (pressure[L] + pressure[R]);
    double tmdot = -projTimeScale * (pbc - pressureIp) * asq * inv_axdx;
    for (int d = 0; d < 3; ++d) {
      const double coordIp = 0.5 * (coords[3 * R + d] + coords[3 * L + d]);
      const double axj = areav[3 * ip + d];
      const double dxj = coords[3 * R + d] - coordIp;
      const double kxj = axj - asq * inv_axdx * dxj;
      const double Gjp = Gpdx[3 * R + d];
      tmdot += (density[R] * velocity[3 * R + d] + projTimeScale * Gjp) * axj -
               projTimeScale * kxj * Gjp * nocFac;
    }
    mdot[ip] = tmdot;
  }
}

// Threads of the OpenMP loops that take no explicit count (the per-edge
// local systems); 0 leaves the runtime default.
void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// The uniform(lo, hi) draws of one default-seeded std::mt19937 with
// std::uniform_real_distribution<double>, in order (the random inputs of
// unit_tests/edge_kernels/UnitTestScalarOpenEdge.C:216-222).
void or_mt19937_uniform(int n, const double* lo, const double* hi, double* out) {
  std::mt19937 rng;
  rng.seed(std::mt19937::default_seed);
  for (int i = 0; i < n; ++i) {
    std::uniform_real_distribution<double> u(lo[i], hi[i]);
    out[i] = u(rng);
  }
}

}  // extern "C"
