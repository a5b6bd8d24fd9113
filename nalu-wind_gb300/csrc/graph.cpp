// Host-side graph construction for the GB300 linear system.
//
// Produces the CSR graph TpetraLinearSystem builds in serial
// (src/TpetraLinearSystem.C:177-494 and :1137-1272): one node row per
// periodic master, ordered by ascending id; each row holds the master's own
// column and the masters of every node sharing an edge with it or with one
// of its slaves, ascending, each expanded to num_dof consecutive columns and
// repeated for the num_dof rows of the node (fill_in_extra_dof_rows_per_node,
// src/TpetraLinearSystemHelpers.C:361-381). Columns equal rows on one rank.
//
// Instead of the reference's per-row sorted insertion this builds the rows
// with a counting sort over directed edge entries, then derives the
// deterministic assembly plan used by the GPU row kernels.
#include <algorithm>
#include <numeric>
#include <stdexcept>

#include "nw_internal.h"

namespace nw {

void build_graph(HostGraph& g, int num_dof, int64_t num_nodes,
                 const int64_t* global_id, const int64_t* nalu_id,
                 int64_t num_edges, const int64_t* edge_nodes) {
  if (num_dof < 1 || num_dof > 3) fail(NW_INVALID_ARG, "num_dof must be 1..3");
  if (num_nodes <= 0 || num_nodes >= (int64_t(1) << 31))
    fail(NW_INVALID_ARG, "num_nodes out of range");
  if (num_edges < 0 || num_edges >= (int64_t(1) << 30))
    fail(NW_INVALID_ARG, "num_edges out of range (< 2^30 required)");
  g = HostGraph();
  g.num_dof = num_dof;
  g.num_nodes = num_nodes;
  g.num_edges = num_edges;
  auto gid = [&](int64_t n) { return global_id ? global_id[n] : n + 1; };
  auto nid = [&](int64_t n) { return nalu_id ? nalu_id[n] : gid(n); };

  // masters sorted by id (beginLinearSystemConstruction, :255-296)
  std::vector<std::pair<int64_t, int32_t>> masters;
  masters.reserve(num_nodes);
  for (int64_t n = 0; n < num_nodes; ++n)
    if (nid(n) == gid(n)) masters.emplace_back(gid(n), int32_t(n));
  std::sort(masters.begin(), masters.end());
  for (size_t k = 1; k < masters.size(); ++k)
    if (masters[k].first == masters[k - 1].first)
      fail(NW_INVALID_ARG, "duplicate node id among masters");
  const int64_t R = int64_t(masters.size());
  g.node_rows = R;
  g.nrows = R * num_dof;
  g.row_master.resize(R);
  g.row_gid.resize(R);
  for (int64_t k = 0; k < R; ++k) {
    g.row_master[k] = masters[k].second;
    g.row_gid[k] = masters[k].first;
  }
  std::vector<int32_t> node_row(num_nodes);
  g.node_lid.resize(num_nodes);
  for (int64_t n = 0; n < num_nodes; ++n) {
    const int64_t id = nid(n);
    auto it = std::lower_bound(
        masters.begin(), masters.end(), std::make_pair(id, int32_t(-1)));
    if (it == masters.end() || it->first != id)
      fail(NW_INVALID_ARG, "node's nalu_id names no master node");
    node_row[n] = int32_t(it - masters.begin());
    g.node_lid[n] = int64_t(node_row[n]) * num_dof;
  }

  // directed entries (row, col, edge, side), counting sort by row
  g.edges.resize(2 * num_edges);
  std::vector<int64_t> cnt(R + 1, 0);
  std::vector<char> has_conn(R, 0);
  for (int64_t e = 0; e < num_edges; ++e) {
    const int64_t a = edge_nodes[2 * e], b = edge_nodes[2 * e + 1];
    if (a < 0 || a >= num_nodes || b < 0 || b >= num_nodes)
      fail(NW_INVALID_ARG, "edge node index out of range");
    g.edges[2 * e] = int32_t(a);
    g.edges[2 * e + 1] = int32_t(b);
    const int32_t ra = node_row[a], rb = node_row[b];
    if (ra == rb)
      fail(NW_INVALID_ARG, "edge joins two nodes of one periodic master");
    cnt[ra + 1]++;
    cnt[rb + 1]++;
    has_conn[ra] = has_conn[rb] = 1;
  }
  for (int64_t r = 0; r < R; ++r) cnt[r + 1] += cnt[r];
  struct Ent {
    int32_t col;
    uint32_t es;  // edge << 1 | side
  };
  std::vector<Ent> ent(cnt[R]);
  {
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int64_t e = 0; e < num_edges; ++e) {
      const int32_t ra = node_row[edge_nodes[2 * e]];
      const int32_t rb = node_row[edge_nodes[2 * e + 1]];
      ent[pos[ra]++] = Ent{rb, uint32_t(e) << 1};
      ent[pos[rb]++] = Ent{ra, (uint32_t(e) << 1) | 1u};
    }
  }
  g.inc_ptr.resize(R + 1);
  g.inc.resize(ent.size());
  g.nrow_ptr.assign(R + 1, 0);
  g.diag_pos.assign(R, 0);
  std::vector<int32_t> ncol;
  ncol.reserve(ent.size() / 2 + R);
  for (int64_t r = 0; r < R; ++r) {
    auto b = ent.begin() + cnt[r], en = ent.begin() + cnt[r + 1];
    std::sort(b, en, [](const Ent& x, const Ent& y) {
      return x.col != y.col ? x.col < y.col : x.es < y.es;
    });
    g.inc_ptr[r] = int32_t(cnt[r]);
    int32_t prev = -1;
    bool diag_done = !has_conn[r];
    int32_t ndistinct_below = 0;
    for (auto it = b; it != en; ++it) {
      uint32_t packed = it->es;
      if (it->col == prev) {
        packed |= 0x80000000u;
      } else {
        if (!diag_done && it->col > r) {
          ncol.push_back(int32_t(r));
          diag_done = true;
        }
        ncol.push_back(it->col);
        if (it->col < r) ++ndistinct_below;
      }
      prev = it->col;
      g.inc[it - ent.begin()] = packed;
    }
    if (!diag_done) ncol.push_back(int32_t(r));
    g.diag_pos[r] = has_conn[r] ? ndistinct_below : -1;
    g.nrow_ptr[r + 1] = int64_t(ncol.size());
  }
  if (cnt[R] >= (int64_t(1) << 31)) fail(NW_INVALID_ARG, "too many edges");
  g.inc_ptr[R] = int32_t(cnt[R]);
  g.ncol = std::move(ncol);

  // block expansion to num_dof
  const int nd = num_dof;
  g.row_ptr.resize(g.nrows + 1);
  int64_t nnz = 0;
  for (int64_t r = 0; r < R; ++r) {
    const int64_t m = g.nrow_ptr[r + 1] - g.nrow_ptr[r];
    for (int d = 0; d < nd; ++d) {
      g.row_ptr[r * nd + d] = nnz;
      nnz += m * nd;
    }
  }
  g.row_ptr[g.nrows] = nnz;
  if (nnz >= (int64_t(1) << 31)) fail(NW_INVALID_ARG, "nnz >= 2^31");
  g.nnz = nnz;
  g.col_idx.resize(nnz);
  for (int64_t r = 0; r < R; ++r) {
    const int64_t b = g.nrow_ptr[r], m = g.nrow_ptr[r + 1] - b;
    for (int d = 0; d < nd; ++d) {
      int32_t* out = g.col_idx.data() + g.row_ptr[r * nd + d];
      for (int64_t k = 0; k < m; ++k)
        for (int c = 0; c < nd; ++c) out[k * nd + c] = g.ncol[b + k] * nd + c;
    }
  }
}

namespace {

// First-fit colouring of the node rows visited in `order` (every row once).
int greedy_colors(const HostGraph& g, const std::vector<int32_t>& order, std::vector<int32_t>& color) {
  color.assign(g.node_rows, -1);
  int ncolors = 0;
  std::vector<int32_t> extra;
  for (const int32_t r : order) {
    int64_t used = 0;  // bitmask for the first 64 colours
    extra.clear();
    for (int64_t p = g.nrow_ptr[r]; p < g.nrow_ptr[r + 1]; ++p) {
      const int32_t c = g.ncol[p];
      if (c == r || color[c] < 0) continue;
      if (color[c] < 64)
        used |= (int64_t(1) << color[c]);
      else
        extra.push_back(color[c]);
    }
    int k = 0;
    while (k < 64 && (used >> k) & 1) ++k;
    if (k == 64) {
      std::sort(extra.begin(), extra.end());
      while (std::binary_search(extra.begin(), extra.end(), k)) ++k;
    }
    color[r] = k;
    ncolors = std::max(ncolors, k + 1);
  }
  return ncolors;
}

}  // namespace

// First fit in row order, then Culberson's iterated greedy: recolouring the
// rows class by class (highest colour first) with first fit never needs more
// colours than the classes it started from, and repeated passes drain the
// small last classes of a first-fit colouring of an unstructured mesh in
// random order (a 2.1M-node tet block: 12 classes, the last three of 19,215,
// 917 and 3 rows; each class is one launch of every Gauss-Seidel sweep).
// The result replaces the first-fit colouring only when it has fewer
// classes, so one that is already minimal (the two classes of a hex box, or
// an RCM-ordered tet block) stays as it is.
int color_node_graph(const HostGraph& g, std::vector<int32_t>& color) {
  constexpr int kPasses = 8;
  const int64_t R = g.node_rows;
  std::vector<int32_t> order(R);
  for (int64_t r = 0; r < R; ++r) order[r] = int32_t(r);
  const int first = greedy_colors(g, order, color);
  if (first <= 2) return first;
  std::vector<int32_t> cur(color), next;
  int ncolors = first;
  for (int pass = 0; pass < kPasses; ++pass) {
    std::vector<int64_t> start(ncolors + 1, 0);
    for (int64_t r = 0; r < R; ++r) start[ncolors - cur[r]]++;  // class c at position ncolors-1-c
    for (int c = 0; c < ncolors; ++c) start[c + 1] += start[c];
    for (int64_t r = 0; r < R; ++r) order[start[ncolors - 1 - cur[r]]++] = int32_t(r);
    ncolors = greedy_colors(g, order, next);  // never more than before
    cur.swap(next);
  }
  if (ncolors < first) {
    color.swap(cur);
    return ncolors;
  }
  return first;
}

}  // namespace nw
