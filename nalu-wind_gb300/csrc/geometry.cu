// Edge area vectors and dual nodal volumes on the GPU
// (GeometryInteriorAlg::impl_compute_edge_area_vector and
// impl_compute_dual_nodal_volume, src/ngp_algorithms/GeometryInteriorAlg.C:
// 70-225), for meshes whose coordinates change between steps.
//
// Two phases, no atomics:
//  1. element phase: one thread per element evaluates its sub-control-
//     surface area vectors (HexSCS / TetSCS, one per element edge) and
//     sub-control volumes (HexSCV / TetSCV, one per node) into element-major
//     buffers (geometry.h, the same code the host mesh generator runs);
//  2. gather phase: one thread per edge sums the signed area vectors of the
//     element edges that are this edge (+ when the element edge's left node
//     is the edge's node[0], GeometryInteriorAlg.C:209-213), and one thread
//     per node sums its sub-control volumes, each in element order, then
//     periodic masters add their slaves' volumes (in node order) and the
//     slaves take the total.
// This file is compiled with -fmad=false: every multiply and add rounds
// separately, as on the host, so the results equal the host generator's
// bit for bit. FP64 throughout (a geometry update per mesh motion, not per
// solver iteration).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "geometry.h"
#include "nw_internal.h"
#include "nw_workload.h"

namespace nw {
namespace {

constexpr int kGeomThreads = 128;

// element-local node pairs (left, right) of the sub-control surfaces, in
// the order hex_geometry / tet_geometry return them (HexSCS lrscv_,
// include/master_element/Hex8CVFEM.h:292; TetSCS, Tet4CVFEM.h)
const int kHexLrHost[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {4, 5}, {5, 6},
                               {6, 7}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int kTetLrHost[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};

template <int NPE>
__global__ void __launch_bounds__(kGeomThreads)
    geom_elem_k(int64_t M, const int32_t* __restrict__ conn, const double* __restrict__ coords,
                double* __restrict__ escs, double* __restrict__ escv) {
  constexpr int NSCS = NPE == 8 ? 12 : 6;
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= M) return;
  double c[NPE][3], s[NSCS][3], v[NPE];
#pragma unroll
  for (int q = 0; q < NPE; ++q) {
    const int64_t n = conn[NPE * e + q];
#pragma unroll
    for (int d = 0; d < 3; ++d) c[q][d] = coords[3 * n + d];
  }
  if constexpr (NPE == 8)
    hex_geometry(c, s, v);
  else
    tet_geometry(c, s, v);
#pragma unroll
  for (int ip = 0; ip < NSCS; ++ip)
#pragma unroll
    for (int d = 0; d < 3; ++d) escs[(NSCS * e + ip) * 3 + d] = s[ip][d];
#pragma unroll
  for (int q = 0; q < NPE; ++q) escv[NPE * e + q] = v[q];
}

// area[e] = sum over the element edges of edge e of sign * scs
__global__ void __launch_bounds__(kGeomThreads)
    edge_area_k(int64_t E, const int64_t* __restrict__ ptr, const uint32_t* __restrict__ inc,
                const double* __restrict__ escs, double* __restrict__ area) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  double a[3] = {0.0, 0.0, 0.0};
  for (int64_t k = ptr[e]; k < ptr[e + 1]; ++k) {
    const uint32_t w = inc[k];
    const double sign = (w & 1u) ? -1.0 : 1.0;
    const int64_t idx = w >> 1;
#pragma unroll
    for (int d = 0; d < 3; ++d) a[d] = a[d] + escs[3 * idx + d] * sign;
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) area[3 * e + d] = a[d];
}

// dualvol[n] = sum of the node's sub-control volumes, in element order
__global__ void __launch_bounds__(kGeomThreads)
    dual_volume_k(int64_t N, const int64_t* __restrict__ ptr, const uint32_t* __restrict__ inc,
                  const double* __restrict__ escv, double* __restrict__ vol) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double v = 0.0;
  for (int64_t k = ptr[n]; k < ptr[n + 1]; ++k) v = v + escv[inc[k]];
  vol[n] = v;
}

// periodic pairs: masters add their slaves (node order), slaves copy
__global__ void periodic_add_k(int64_t nm, const int32_t* __restrict__ masters,
                               const int64_t* __restrict__ ptr, const int32_t* __restrict__ slaves,
                               double* __restrict__ vol) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= nm) return;
  const int64_t m = masters[k];
  double v = vol[m];
  for (int64_t q = ptr[k]; q < ptr[k + 1]; ++q) v = v + vol[slaves[q]];
  vol[m] = v;
  for (int64_t q = ptr[k]; q < ptr[k + 1]; ++q) vol[slaves[q]] = v;
}

inline unsigned grid_for(int64_t n) { return unsigned((n + kGeomThreads - 1) / kGeomThreads); }

}  // namespace
}  // namespace nw

struct nw_geometry {
  int device = 0;
  int npe = 8;
  int64_t N = 0, M = 0, E = 0;
  nw::DeviceArray<int32_t> conn, masters, slaves;
  nw::DeviceArray<int64_t> eptr, vptr, mptr;
  nw::DeviceArray<uint32_t> einc, vinc;
  nw::DeviceArray<double> escs, escv;
};

namespace {

template <typename F>
nw_status guard_geom(F&& f) {
  try {
    f();
    return NW_OK;
  } catch (const nw::Error& e) {
    nw::set_last_error(e.msg);
    return e.status;
  } catch (const std::exception& e) {
    nw::set_last_error(e.what());
    return NW_INTERNAL;
  }
}

}  // namespace

extern "C" nw_status nw_geometry_create(int64_t num_nodes, int nodes_per_elem, int64_t num_elems,
                                        const int64_t* conn, int64_t num_edges, const int64_t* edge_nodes,
                                        const int64_t* nalu_id, nw_geometry** out) {
  return guard_geom([&] {
    using nw::fail;
    if (!out) fail(NW_INVALID_ARG, "null output");
    *out = nullptr;
    if (nodes_per_elem != 8 && nodes_per_elem != 4) fail(NW_INVALID_ARG, "nodes_per_elem must be 8 or 4");
    if (num_nodes < 1 || num_elems < 1 || num_edges < 1 || !conn || !edge_nodes)
      fail(NW_INVALID_ARG, "empty mesh or null array");
    if (num_nodes >= (int64_t(1) << 31) || num_elems * 12 >= (int64_t(1) << 30))
      fail(NW_INVALID_ARG, "mesh too large for 32-bit element indices");
    const int npe = nodes_per_elem, nscs = npe == 8 ? 12 : 6;
    const int64_t N = num_nodes, M = num_elems, E = num_edges;
    // node pair -> edge index: per lower node, the higher nodes sorted
    std::vector<int64_t> lp(N + 1, 0);
    for (int64_t e = 0; e < E; ++e) {
      const int64_t a = edge_nodes[2 * e], b = edge_nodes[2 * e + 1];
      if (a < 0 || b < 0 || a >= N || b >= N || a == b) fail(NW_INVALID_ARG, "bad edge");
      lp[std::min(a, b) + 1]++;
    }
    for (int64_t i = 0; i < N; ++i) lp[i + 1] += lp[i];
    std::vector<std::pair<int64_t, int64_t>> hi(E);
    {
      std::vector<int64_t> pos(lp.begin(), lp.end() - 1);
      for (int64_t e = 0; e < E; ++e) {
        const int64_t a = edge_nodes[2 * e], b = edge_nodes[2 * e + 1];
        hi[pos[std::min(a, b)]++] = {std::max(a, b), e};
      }
      for (int64_t i = 0; i < N; ++i) std::sort(hi.begin() + lp[i], hi.begin() + lp[i + 1]);
    }
    auto edge_of = [&](int64_t a, int64_t b) -> int64_t {
      const int64_t lo = std::min(a, b), h = std::max(a, b);
      auto it = std::lower_bound(hi.begin() + lp[lo], hi.begin() + lp[lo + 1], std::make_pair(h, int64_t(-1)));
      if (it == hi.begin() + lp[lo + 1] || it->first != h) fail(NW_INVALID_ARG, "element edge missing from the edge list");
      return it->second;
    };
    // incidences, element order then sub-surface / node order
    std::vector<int64_t> ecount(E + 1, 0), vcount(N + 1, 0);
    std::vector<int32_t> c32(size_t(M) * npe);
    for (int64_t e = 0; e < M; ++e)
      for (int q = 0; q < npe; ++q) {
        const int64_t n = conn[npe * e + q];
        if (n < 0 || n >= N) fail(NW_INVALID_ARG, "connectivity out of range");
        c32[npe * e + q] = int32_t(n);
        vcount[n + 1]++;
      }
    std::vector<int64_t> eidx(size_t(M) * nscs);
    for (int64_t e = 0; e < M; ++e)
      for (int ip = 0; ip < nscs; ++ip) {
        const int la = npe == 8 ? nw::kHexLrHost[ip][0] : nw::kTetLrHost[ip][0];
        const int lb = npe == 8 ? nw::kHexLrHost[ip][1] : nw::kTetLrHost[ip][1];
        const int64_t ed = edge_of(conn[npe * e + la], conn[npe * e + lb]);
        eidx[size_t(e) * nscs + ip] = ed;
        ecount[ed + 1]++;
      }
    for (int64_t e = 0; e < E; ++e) ecount[e + 1] += ecount[e];
    for (int64_t n = 0; n < N; ++n) vcount[n + 1] += vcount[n];
    std::vector<uint32_t> einc(ecount[E]), vinc(vcount[N]);
    {
      std::vector<int64_t> pe(ecount.begin(), ecount.end() - 1), pv(vcount.begin(), vcount.end() - 1);
      for (int64_t e = 0; e < M; ++e) {
        for (int ip = 0; ip < nscs; ++ip) {
          const int la = npe == 8 ? nw::kHexLrHost[ip][0] : nw::kTetLrHost[ip][0];
          const int64_t ed = eidx[size_t(e) * nscs + ip];
          const bool neg = conn[npe * e + la] != edge_nodes[2 * ed];
          einc[pe[ed]++] = (uint32_t(e * nscs + ip) << 1) | (neg ? 1u : 0u);
        }
        for (int q = 0; q < npe; ++q) vinc[pv[conn[npe * e + q]]++] = uint32_t(e * npe + q);
      }
    }
    // periodic masters (nalu_id: 1-based master id per node)
    std::vector<int32_t> masters, slaves;
    std::vector<int64_t> mptr(1, 0);
    if (nalu_id) {
      std::vector<std::vector<int32_t>> sl(N);
      for (int64_t n = 0; n < N; ++n) {
        const int64_t m = nalu_id[n] - 1;
        if (m < 0 || m >= N) fail(NW_INVALID_ARG, "nalu_id out of range");
        if (m != n) sl[m].push_back(int32_t(n));
      }
      for (int64_t m = 0; m < N; ++m)
        if (!sl[m].empty()) {
          masters.push_back(int32_t(m));
          slaves.insert(slaves.end(), sl[m].begin(), sl[m].end());
          mptr.push_back(int64_t(slaves.size()));
        }
    }
    auto g = std::make_unique<nw_geometry>();
    NW_CUDA(cudaGetDevice(&g->device));
    g->npe = npe;
    g->N = N;
    g->M = M;
    g->E = E;
    cudaStream_t s = nullptr;
    g->conn.upload(c32, s);
    g->eptr.upload(ecount, s);
    g->einc.upload(einc, s);
    g->vptr.upload(vcount, s);
    g->vinc.upload(vinc, s);
    if (!masters.empty()) {
      g->masters.upload(masters, s);
      g->mptr.upload(mptr, s);
      g->slaves.upload(slaves, s);
    }
    g->escs.resize(size_t(M) * nscs * 3);
    g->escv.resize(size_t(M) * npe);
    NW_CUDA(cudaStreamSynchronize(s));
    *out = g.release();
  });
}

extern "C" nw_status nw_geometry_compute(nw_geometry* g, const double* coords, double* area,
                                         double* dualvol, void* stream) {
  return guard_geom([&] {
    using nw::fail;
    if (!g || !coords || !area || !dualvol) fail(NW_INVALID_ARG, "null argument");
    int cur = -1;
    NW_CUDA(cudaGetDevice(&cur));
    if (cur != g->device) fail(NW_INVALID_ARG, "the geometry handle's device is not the current device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (g->npe == 8)
      nw::geom_elem_k<8><<<nw::grid_for(g->M), nw::kGeomThreads, 0, s>>>(g->M, g->conn.p, coords, g->escs.p,
                                                                         g->escv.p);
    else
      nw::geom_elem_k<4><<<nw::grid_for(g->M), nw::kGeomThreads, 0, s>>>(g->M, g->conn.p, coords, g->escs.p,
                                                                         g->escv.p);
    nw::edge_area_k<<<nw::grid_for(g->E), nw::kGeomThreads, 0, s>>>(g->E, g->eptr.p, g->einc.p, g->escs.p, area);
    nw::dual_volume_k<<<nw::grid_for(g->N), nw::kGeomThreads, 0, s>>>(g->N, g->vptr.p, g->vinc.p, g->escv.p,
                                                                       dualvol);
    const int64_t nm = int64_t(g->masters.n);
    if (nm)
      nw::periodic_add_k<<<nw::grid_for(nm), nw::kGeomThreads, 0, s>>>(nm, g->masters.p, g->mptr.p,
                                                                        g->slaves.p, dualvol);
    NW_CUDA(cudaGetLastError());
  });
}

extern "C" nw_status nw_geometry_destroy(nw_geometry* g) {
  return guard_geom([&] { delete g; });
}
