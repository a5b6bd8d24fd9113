// C ABI implementation: the LinearSystem / LinearSolver surface of
// nalu-wind's Tpetra backend (include/LinearSystem.h:88-256,
// src/TpetraLinearSystem.C, src/LinearSolver.C) on one GB300.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "assemble.h"
#include "boundary.h"
#include "krylov.h"
#include "learned.h"
#include "node_kernels.h"
#include "nw_internal.h"
#include "schedule.h"

namespace nw {

namespace {
thread_local std::string g_last_error;
}

void fail(nw_status s, const std::string& msg) { throw Error{s, msg}; }

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fail(NW_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

void set_last_error(const std::string& s) { g_last_error = s; }
const char* last_error() { return g_last_error.c_str(); }

}  // namespace nw

using namespace nw;

struct nw_linsys {
  int num_dof = 1;
  nw_solver_cfg cfg{};
  cudaStream_t stream = nullptr;
  int device = 0;
  bool built = false;
  bool finalized = false;
  bool pristine = false;  // zeroSystem issued, no values written since
  // with pristine: node rows below this were written by in-order row-range
  // calls (nw_assemble_momentum_rows_range); the rest are still zero
  int64_t pristine_from = 0;
  // continuity assembled in edge ranges (nw_assemble_continuity_edge_range):
  // the end of the ranges evaluated so far, in order from edge 0; -1 none.
  // edge_node_max[e]: the largest node index of edges 0..e (built on first
  // use): a range's node pre-pass covers the nodes that become reachable
  int64_t cont_next = -1;
  std::vector<int32_t> edge_node_max;
  HostGraph g;
  DeviceArray<int64_t> row_ptr, node_lid, row_nodes_ptr;
  DeviceArray<int32_t> row_nodes;
  DeviceArray<int32_t> col_idx, inc_ptr, diag_pos, color_rows;
  DeviceArray<uint32_t> inc;
  DeviceArray<int2> edges;
  DeviceArray<double> values, rhs, buf, nodebuf;
  int stage_bytes[3] = {0, 0, 0};  // row-phase staging per kind
  int max_inc = 0;                 // most incidences of a node row
  // single-kernel momentum assembly (schedule.h), taken when fused_ok and
  // assembly_path is NW_ASSEMBLY_SINGLE_KERNEL
  bool fused_ok = false;
  int assembly_path = NW_ASSEMBLY_TWO_KERNELS;
  FusedSchedule fsched;
  FusedLaunch fl;
  DeviceArray<int32_t> f_items, f_in_ptr, f_in, f_out_ptr, f_out;
  DeviceArray<int> f_eflag, f_rflag, f_ticket, f_err;
  DeviceArray<double> ring;
  DeviceArray<int> err;
  DeviceArray<int64_t> scratch_lid;
  DeviceArray<double> scratch_vals;
  KrylovSolver solver;
  Precond pc;
  std::vector<int64_t> color_ptr;
  std::vector<int32_t> color_rows_host;
  std::vector<double> history;
  nw_solve_report last_report{};  // of the last solve (checkpointed)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // solves of a handle on the legacy default stream run on this stream
  // (non-blocking, joined to the caller's stream by events), because the
  // legacy stream cannot be captured into the solver's CUDA graphs
  cudaStream_t solve_stream = nullptr;
  cudaEvent_t solve_in = nullptr, solve_out = nullptr;
  bool timed = false;
  nw_learned* learned = nullptr;
  std::unique_ptr<CoarseLevel> coarse;
};

struct nw_learned {
  LearnedNet net;
};

namespace {

int g_device = 0;

template <typename F>
nw_status guard(F&& f) {
  try {
    f();
    return NW_OK;
  } catch (const Error& e) {
    set_last_error(e.msg);
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return NW_INTERNAL;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return NW_INTERNAL;
  }
}

nw_solver_cfg default_cfg() {
  nw_solver_cfg c{};
  c.method = NW_GMRES;
  c.preconditioner = NW_PC_JACOBI;
  c.precision = NW_PREC_FP64;
  c.kspace = 50;
  c.max_iterations = 50;
  c.tolerance = 1e-4;
  c.final_tolerance = 1e-4;
  c.inner_kspace = 0;
  c.inner_tolerance = 0;
  c.sgs2_inner_sweeps = 1;
  c.sstep_size = 5;
  return c;
}

void check_cfg(const nw_solver_cfg& c) {
  if (c.kspace < 1 || c.kspace > 1000) fail(NW_INVALID_ARG, "kspace out of range");
  if (c.max_iterations < 0) fail(NW_INVALID_ARG, "max_iterations < 0");
  if (!(c.tolerance >= 0.0)) fail(NW_INVALID_ARG, "tolerance < 0");
  if (c.method < NW_GMRES || c.method > NW_SSTEP_GMRES) fail(NW_INVALID_ARG, "bad method");
  if (c.sstep_size > 64) fail(NW_INVALID_ARG, "sstep_size above 64");
  if (c.preconditioner < NW_PC_NONE || c.preconditioner > NW_PC_RILUK)
    fail(NW_INVALID_ARG, "bad preconditioner");
}

void need_finalized(const nw_linsys* ls) {
  if (!ls) fail(NW_INVALID_ARG, "null handle");
  if (!ls->finalized) fail(NW_NOT_FINALIZED, "linear system not finalized");
}

// materialise a pending zeroSystem before a partial update (the rows that
// in-order row-range calls already wrote are kept)
void materialize_zero(nw_linsys* ls) {
  if (!ls->pristine) return;
  const int64_t r0 = ls->pristine_from * ls->num_dof;
  const int64_t v0 = ls->g.row_ptr.empty() ? 0 : ls->g.row_ptr[r0];
  NW_CUDA(cudaMemsetAsync(ls->values.p + v0, 0, (ls->values.n - v0) * sizeof(double), ls->stream));
  NW_CUDA(cudaMemsetAsync(ls->rhs.p + r0, 0, (ls->rhs.n - r0) * sizeof(double), ls->stream));
  ls->pristine = false;
  ls->pristine_from = 0;
}

// accumulate flag of a kernel that writes every row: 0 (overwrite) on a
// zeroed system, else 1; a partly written zeroed system is materialised
int write_mode(nw_linsys* ls) {
  if (ls->pristine && ls->pristine_from > 0) materialize_zero(ls);
  return ls->pristine ? 0 : 1;
}

void begin_timing(nw_linsys* ls) {
  if (!ls->ev0) {
    NW_CUDA(cudaEventCreate(&ls->ev0));
    NW_CUDA(cudaEventCreate(&ls->ev1));
  }
  NW_CUDA(cudaEventRecord(ls->ev0, ls->stream));
}
void end_timing(nw_linsys* ls) {
  NW_CUDA(cudaEventRecord(ls->ev1, ls->stream));
  ls->timed = true;
}

void check_ptr(const void* p, const char* name) {
  if (!p) fail(NW_INVALID_ARG, std::string("null field pointer: ") + name);
}

}  // namespace

extern "C" {

const char* nw_last_error_string(void) { return last_error(); }
int nw_version(void) { return 1; }

nw_status nw_set_device(int device) {
  return guard([&] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
      fail(NW_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n) fail(NW_INVALID_ARG, "device out of range");
    g_device = device;
    NW_CUDA(cudaSetDevice(device));
  });
}

nw_status nw_linsys_create(int num_dof, const nw_solver_cfg* cfg,
                           nw_linsys** out) {
  return guard([&] {
    if (!out) fail(NW_INVALID_ARG, "null output");
    *out = nullptr;
    if (num_dof < 1 || num_dof > 3) fail(NW_INVALID_ARG, "num_dof must be 1..3");
    // host-only until nw_linsys_finalize: graph construction needs no GPU
    auto ls = std::make_unique<nw_linsys>();
    ls->num_dof = num_dof;
    ls->device = g_device;
    ls->cfg = cfg ? *cfg : default_cfg();
    check_cfg(ls->cfg);
    *out = ls.release();
  });
}

nw_status nw_linsys_destroy(nw_linsys* ls) {
  return guard([&] {
    if (!ls) return;
    if (ls->ev0) cudaEventDestroy(ls->ev0);
    if (ls->ev1) cudaEventDestroy(ls->ev1);
    if (ls->solve_in) cudaEventDestroy(ls->solve_in);
    if (ls->solve_out) cudaEventDestroy(ls->solve_out);
    if (ls->solve_stream) cudaStreamDestroy(ls->solve_stream);
    delete ls;
  });
}

nw_status nw_linsys_set_stream(nw_linsys* ls, void* stream) {
  return guard([&] {
    if (!ls) fail(NW_INVALID_ARG, "null handle");
    ls->stream = static_cast<cudaStream_t>(stream);
  });
}

nw_status nw_linsys_set_solver_cfg(nw_linsys* ls, const nw_solver_cfg* cfg) {
  return guard([&] {
    if (!ls || !cfg) fail(NW_INVALID_ARG, "null argument");
    check_cfg(*cfg);
    const bool grow = ls->finalized && cfg->kspace > ls->cfg.kspace;
    ls->cfg = *cfg;
    if (grow) {
      DevCsr A;
      A.n = ls->g.nrows;
      A.nnz = ls->g.nnz;
      A.row_ptr = ls->row_ptr.p;
      A.col_idx = ls->col_idx.p;
      A.values = ls->values.p;
      A.lanes = ls->num_dof == 1 ? 8 : 32;
      A.row_ptr_host = ls->g.row_ptr.data();
      A.col_idx_host = ls->g.col_idx.data();
      ls->solver.setup(A, std::max(ls->cfg.kspace, ls->cfg.inner_kspace), ls->stream);
    }
  });
}

nw_status nw_linsys_build_edge_graph(nw_linsys* ls, int64_t num_nodes,
                                     const int64_t* global_id,
                                     const int64_t* nalu_id, int64_t num_edges,
                                     const int64_t* edge_nodes) {
  return guard([&] {
    if (!ls) fail(NW_INVALID_ARG, "null handle");
    if (num_edges > 0 && !edge_nodes) fail(NW_INVALID_ARG, "null edge list");
    build_graph(ls->g, ls->num_dof, num_nodes, global_id, nalu_id, num_edges,
                edge_nodes);
    ls->built = true;
    ls->finalized = false;
  });
}

// Work list, ring and flags of the single-kernel momentum assembly. The
// ring holds at most 64 MB of coefficient slots (it is meant to stay in
// L2); a mesh whose rows read edges too far apart for that gets one slot
// per edge chunk, i.e. the whole coefficient buffer.
static void setup_fused(nw_linsys* ls) {
  const HostGraph& g = ls->g;
  cudaStream_t s = ls->stream;
  ls->fused_ok = false;
  if (g.num_edges == 0 || g.node_rows == 0) return;
  const int smem = row_stage_bytes(3, g.row_ptr.data(), g.node_rows);
  const int occ = fused_blocks_per_sm(smem);
  int sms = 0;
  NW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ls->device));
  if (occ < 1 || sms < 1) return;
  const int64_t slot_bytes = int64_t(kFusedChunk) * kMomentumCoefs * int64_t(sizeof(double));
  build_fused_schedule(g.num_edges, g.node_rows, g.inc_ptr.data(), g.inc.data(),
                       int64_t(occ) * sms, (int64_t(64) << 20) / slot_bytes, ls->fsched);
  const FusedSchedule& fs = ls->fsched;
  ls->f_items.upload(fs.items, s);
  ls->f_in_ptr.upload(fs.in_ptr, s);
  ls->f_in.upload(fs.in, s);
  ls->f_out_ptr.upload(fs.out_ptr, s);
  ls->f_out.upload(fs.out, s);
  ls->f_eflag.resize(size_t(fs.chunks));
  ls->f_rflag.resize(size_t(fs.blocks));
  ls->f_ticket.resize(1);
  ls->f_err.resize(1);
  NW_CUDA(cudaMemsetAsync(ls->f_eflag.p, 0, fs.chunks * sizeof(int), s));
  NW_CUDA(cudaMemsetAsync(ls->f_rflag.p, 0, fs.blocks * sizeof(int), s));
  NW_CUDA(cudaMemsetAsync(ls->f_err.p, 0, sizeof(int), s));
  FusedLaunch& L = ls->fl;
  L = FusedLaunch();
  if (fs.ring_chunks < fs.chunks) {
    L.stride = fs.ring_chunks * kFusedChunk;
    L.mask = L.stride - 1;
    ls->ring.resize(size_t(kMomentumCoefs) * size_t(L.stride));
    L.ring = ls->ring.p;
  } else {
    ls->ring.release();
    L.stride = g.num_edges;
    L.mask = -1;
    L.ring = ls->buf.p;
  }
  L.items = ls->f_items.p;
  L.in_ptr = ls->f_in_ptr.p;
  L.in = ls->f_in.p;
  L.out_ptr = ls->f_out_ptr.p;
  L.out = ls->f_out.p;
  L.eflag = ls->f_eflag.p;
  L.rflag = ls->f_rflag.p;
  L.ticket = ls->f_ticket.p;
  L.err = ls->f_err.p;
  L.nitems = int64_t(fs.items.size());
  L.num_edges = g.num_edges;
  L.ring_chunks = fs.ring_chunks;
  L.grid = occ * sms;
  L.smem_bytes = smem;
  L.R = g.node_rows;
  L.inc_ptr = ls->inc_ptr.p;
  L.inc = ls->inc.p;
  L.diag_pos = ls->diag_pos.p;
  L.row_ptr = ls->row_ptr.p;
  L.values = ls->values.p;
  L.rhs = ls->rhs.p;
  ls->fused_ok = true;
}

// Raises if a single-kernel assembly since the last check timed out in a
// dependency wait (the system's values are then not valid).
static void check_fused(nw_linsys* ls) {
  if (!ls->fused_ok || !ls->f_err.p) return;
  int h = 0;
  NW_CUDA(cudaMemcpyAsync(&h, ls->f_err.p, sizeof(int), cudaMemcpyDeviceToHost, ls->stream));
  NW_CUDA(cudaStreamSynchronize(ls->stream));
  if (h) {
    NW_CUDA(cudaMemsetAsync(ls->f_err.p, 0, sizeof(int), ls->stream));
    fail(NW_TIMEOUT, "momentum assembly: a dependency wait of the single-kernel assembly timed out");
  }
}

nw_status nw_linsys_finalize(nw_linsys* ls) {
  return guard([&] {
    if (!ls) fail(NW_INVALID_ARG, "null handle");
    if (!ls->built) fail(NW_NOT_FINALIZED, "no graph built");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      fail(NW_NO_DEVICE, "no CUDA device");
    NW_CUDA(cudaSetDevice(ls->device));
    ls->err.resize(1);
    NW_CUDA(cudaMemset(ls->err.p, 0, sizeof(int)));
    HostGraph& g = ls->g;
    cudaStream_t s = ls->stream;
    ls->row_ptr.upload(g.row_ptr, s);
    ls->col_idx.upload(g.col_idx, s);
    ls->node_lid.upload(g.node_lid, s);
    {
      // node row -> nodes (periodic master first, then its slaves)
      std::vector<int64_t> rp(g.node_rows + 1, 0);
      for (int64_t k = 0; k < g.num_nodes; ++k) rp[g.node_lid[k] / g.num_dof + 1]++;
      for (int64_t r = 0; r < g.node_rows; ++r) rp[r + 1] += rp[r];
      std::vector<int32_t> rn(g.num_nodes);
      std::vector<int64_t> pos(rp.begin(), rp.end() - 1);
      for (int64_t r = 0; r < g.node_rows; ++r) rn[pos[r]++] = g.row_master[r];
      for (int64_t k = 0; k < g.num_nodes; ++k)
        if (g.row_master[g.node_lid[k] / g.num_dof] != k) rn[pos[g.node_lid[k] / g.num_dof]++] = int32_t(k);
      ls->row_nodes_ptr.upload(rp, s);
      ls->row_nodes.upload(rn, s);
    }
    ls->inc_ptr.upload(g.inc_ptr, s);
    ls->inc.upload(g.inc, s);
    ls->diag_pos.upload(g.diag_pos, s);
    ls->edges.resize(g.num_edges);
    if (g.num_edges)
      NW_CUDA(cudaMemcpyAsync(ls->edges.p, g.edges.data(),
                              g.num_edges * sizeof(int2),
                              cudaMemcpyHostToDevice, s));
    ls->values.resize(g.nnz);
    ls->rhs.resize(g.nrows);
    const int coefs = ls->num_dof == 3 ? kMomentumCoefs : kScalarCoefs;
    ls->buf.resize(size_t(coefs) * std::max<int64_t>(g.num_edges, 1));
    if (ls->num_dof == 1) {
      ls->nodebuf.resize(size_t(kContinuityNodeStride) * g.num_nodes);
      ls->stage_bytes[0] = ls->stage_bytes[1] =
          row_stage_bytes(0, g.row_ptr.data(), g.node_rows);
    } else if (ls->num_dof == 3) {
      // the momentum kernels address node fields with 32-bit offsets (up
      // to 9 doubles per node); a system that large would not fit in HBM
      if (9 * g.num_nodes >= (int64_t(1) << 32)) fail(NW_INVALID_ARG, "too many nodes for a 3-dof system");
      ls->stage_bytes[2] = row_stage_bytes(2, g.row_ptr.data(), g.node_rows);
      ls->max_inc = 0;
      for (int64_t r = 0; r < g.node_rows; ++r)
        ls->max_inc = std::max(ls->max_inc, g.inc_ptr[r + 1] - g.inc_ptr[r]);
      setup_fused(ls);
    }
    NW_CUDA(cudaMemsetAsync(ls->values.p, 0, g.nnz * sizeof(double), s));
    NW_CUDA(cudaMemsetAsync(ls->rhs.p, 0, g.nrows * sizeof(double), s));
    ls->pristine = false;
    // multicolour order for Gauss-Seidel: node colours, dof rows interleaved
    std::vector<int32_t> color;
    const int nc = color_node_graph(g, color);
    const int nd = ls->num_dof;
    const int rc = nc * nd;
    std::vector<int64_t> cnt(rc + 1, 0);
    for (int64_t r = 0; r < g.node_rows; ++r)
      for (int d = 0; d < nd; ++d) cnt[color[r] * nd + d + 1]++;
    for (int c = 0; c < rc; ++c) cnt[c + 1] += cnt[c];
    ls->color_ptr = cnt;
    ls->color_rows_host.resize(g.nrows);
    {
      std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
      for (int64_t r = 0; r < g.node_rows; ++r)
        for (int d = 0; d < nd; ++d)
          ls->color_rows_host[pos[color[r] * nd + d]++] = int32_t(r * nd + d);
    }
    ls->color_rows.upload(ls->color_rows_host, s);
    ls->pc.color_rows = ls->color_rows.p;
    ls->pc.color_ptr = ls->color_ptr;
    DevCsr A;
    A.n = g.nrows;
    A.nnz = g.nnz;
    A.row_ptr = ls->row_ptr.p;
    A.col_idx = ls->col_idx.p;
    A.values = ls->values.p;
    A.lanes = nd == 1 ? 8 : 32;
    A.row_ptr_host = g.row_ptr.data();
    A.col_idx_host = g.col_idx.data();
    ls->solver.setup(A, std::max(ls->cfg.kspace, ls->cfg.inner_kspace), s);
    ls->solver.setup_colors(ls->color_rows_host, ls->color_ptr, s);
    NW_CUDA(cudaStreamSynchronize(s));
    ls->finalized = true;
  });
}

nw_status nw_linsys_graph_sizes(const nw_linsys* ls, int64_t* nrows,
                                int64_t* nnz) {
  return guard([&] {
    if (!ls || !ls->built) fail(NW_NOT_FINALIZED, "no graph");
    if (nrows) *nrows = ls->g.nrows;
    if (nnz) *nnz = ls->g.nnz;
  });
}

nw_status nw_linsys_get_graph(const nw_linsys* ls, int64_t* row_ptr,
                              int32_t* col_idx) {
  return guard([&] {
    if (!ls || !ls->built) fail(NW_NOT_FINALIZED, "no graph");
    if (row_ptr)
      std::memcpy(row_ptr, ls->g.row_ptr.data(), ls->g.row_ptr.size() * sizeof(int64_t));
    if (col_idx)
      std::memcpy(col_idx, ls->g.col_idx.data(), ls->g.col_idx.size() * sizeof(int32_t));
  });
}

nw_status nw_linsys_get_node_lid(const nw_linsys* ls, int64_t* node_lid) {
  return guard([&] {
    if (!ls || !ls->built) fail(NW_NOT_FINALIZED, "no graph");
    if (!node_lid) fail(NW_INVALID_ARG, "null output");
    std::memcpy(node_lid, ls->g.node_lid.data(), ls->g.node_lid.size() * sizeof(int64_t));
  });
}

nw_status nw_linsys_zero(nw_linsys* ls) {
  return guard([&] {
    need_finalized(ls);
    // zeroSystem is deferred: the next full assembly overwrites every slot
    ls->pristine = true;
    ls->pristine_from = 0;
  });
}

nw_status nw_assemble_scalar_edges(nw_linsys* ls, const nw_scalar_fields* f,
                                   const nw_scalar_opts* o) {
  return guard([&] {
    need_finalized(ls);
    if (ls->num_dof != 1) fail(NW_INVALID_ARG, "scalar assembly needs num_dof 1");
    if (!f || !o) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->coords, "coords");
    check_ptr(f->velocity_rtm, "velocity_rtm");
    check_ptr(f->q, "q");
    check_ptr(f->dqdx, "dqdx");
    check_ptr(f->density, "density");
    check_ptr(f->diff_coeff, "diff_coeff");
    check_ptr(f->area, "area");
    check_ptr(f->mdot, "mdot");
    if (!(o->relax != 0.0)) fail(NW_INVALID_ARG, "relaxation factor is zero");
    begin_timing(ls);
    const int64_t E = ls->g.num_edges;
    launch_scalar_edges(ls->stream, E, ls->edges.p, *f, *o, ls->buf.p);
    launch_rows(ls->stream, 0, ls->g.node_rows, ls->inc_ptr.p, ls->inc.p,
                ls->diag_pos.p, ls->row_ptr.p, ls->buf.p, E, o->relax,
                ls->values.p, ls->rhs.p, write_mode(ls), ls->stage_bytes[0]);
    NW_CUDA(cudaGetLastError());
    end_timing(ls);
    ls->pristine = false;
  });
}

static void check_continuity_args(const nw_linsys* ls, const nw_continuity_fields* f,
                                  const nw_continuity_opts* o) {
  need_finalized(ls);
  if (ls->num_dof != 1) fail(NW_INVALID_ARG, "continuity assembly needs num_dof 1");
  if (!f || !o) fail(NW_INVALID_ARG, "null argument");
  check_ptr(f->coords, "coords");
  check_ptr(f->velocity, "velocity");
  check_ptr(f->dpdx, "dpdx");
  check_ptr(f->density, "density");
  check_ptr(f->pressure, "pressure");
  check_ptr(f->udiag, "udiag");
  check_ptr(f->area, "area");
  if (!(o->tau_scale != 0.0)) fail(NW_INVALID_ARG, "tau_scale is zero");
}

static void continuity_rows(nw_linsys* ls) {
  launch_rows(ls->stream, 1, ls->g.node_rows, ls->inc_ptr.p, ls->inc.p,
              ls->diag_pos.p, ls->row_ptr.p, ls->buf.p, ls->g.num_edges, 1.0,
              ls->values.p, ls->rhs.p, write_mode(ls), ls->stage_bytes[1]);
  NW_CUDA(cudaGetLastError());
  ls->pristine = false;
}

nw_status nw_assemble_continuity_edges(nw_linsys* ls,
                                       const nw_continuity_fields* f,
                                       const nw_continuity_opts* o) {
  return guard([&] {
    check_continuity_args(ls, f, o);
    begin_timing(ls);
    const int64_t E = ls->g.num_edges;
    ls->cont_next = -1;
    launch_continuity_edges(ls->stream, E, ls->g.num_nodes, ls->edges.p, *f, *o,
                            ls->buf.p, ls->nodebuf.p);
    continuity_rows(ls);
    end_timing(ls);
  });
}

nw_status nw_assemble_continuity_edge_range(nw_linsys* ls, const nw_continuity_fields* f,
                                            const nw_continuity_opts* o, int64_t edge_begin,
                                            int64_t edge_end) {
  return guard([&] {
    check_continuity_args(ls, f, o);
    const int64_t E = ls->g.num_edges;
    if (edge_begin < 0 || edge_end > E || edge_begin > edge_end)
      fail(NW_INVALID_ARG, "edge range out of bounds");
    if (edge_begin != 0 && edge_begin != ls->cont_next)
      fail(NW_INVALID_ARG, "continuity edge ranges must follow each other from edge 0");
    std::vector<int32_t>& pm = ls->edge_node_max;
    if (int64_t(pm.size()) != E) {
      pm.resize(E);
      int32_t m = -1;
      for (int64_t e = 0; e < E; ++e) pm[e] = m = std::max({m, ls->g.edges[2 * e], ls->g.edges[2 * e + 1]});
    }
    // node pre-pass over the nodes the range's edges reach beyond the
    // earlier ranges' (the largest node index so far, plus one)
    const int64_t n0 = edge_begin == 0 ? 0 : int64_t(pm[edge_begin - 1]) + 1;
    const int64_t n1 = edge_end == 0 ? 0 : int64_t(pm[edge_end - 1]) + 1;
    launch_continuity_edge_range(ls->stream, n0, std::max(n0, n1), edge_begin, edge_end, ls->edges.p, *f, *o,
                                 ls->buf.p, ls->nodebuf.p);
    NW_CUDA(cudaGetLastError());
    ls->cont_next = edge_end;
  });
}

nw_status nw_assemble_continuity_rows(nw_linsys* ls) {
  return guard([&] {
    need_finalized(ls);
    if (ls->num_dof != 1) fail(NW_INVALID_ARG, "continuity assembly needs num_dof 1");
    if (ls->cont_next != ls->g.num_edges)
      fail(NW_INVALID_ARG, "continuity edge ranges do not cover every edge");
    continuity_rows(ls);
    ls->cont_next = -1;
  });
}

static void check_momentum_args(const nw_linsys* ls, const nw_momentum_fields* f,
                                const nw_momentum_opts* o) {
  need_finalized(ls);
  if (ls->num_dof != 3) fail(NW_INVALID_ARG, "momentum assembly needs num_dof 3");
  if (!f || !o) fail(NW_INVALID_ARG, "null argument");
  check_ptr(f->coords, "coords");
  check_ptr(f->velocity, "velocity");
  check_ptr(f->dudx, "dudx");
  check_ptr(f->viscosity, "viscosity");
  check_ptr(f->density, "density");
  check_ptr(f->mask, "mask");
  check_ptr(f->area, "area");
  check_ptr(f->mdot, "mdot");
  check_ptr(f->pecfac, "pecfac");
  if (!(o->relax != 0.0)) fail(NW_INVALID_ARG, "relaxation factor is zero");
}

static void momentum_rows(nw_linsys* ls, double relax) {
  launch_rows(ls->stream, 2, ls->g.node_rows, ls->inc_ptr.p, ls->inc.p,
              ls->diag_pos.p, ls->row_ptr.p, ls->buf.p, ls->g.num_edges, relax,
              ls->values.p, ls->rhs.p, write_mode(ls), ls->stage_bytes[2], ls->max_inc);
  NW_CUDA(cudaGetLastError());
  ls->pristine = false;
}

nw_status nw_assemble_momentum_edges(nw_linsys* ls, const nw_momentum_fields* f,
                                     const nw_momentum_opts* o) {
  return guard([&] {
    check_momentum_args(ls, f, o);
    begin_timing(ls);
    const int64_t E = ls->g.num_edges;
    if (ls->fused_ok && ls->assembly_path == NW_ASSEMBLY_SINGLE_KERNEL) {
      FusedLaunch& L = ls->fl;
      if (++L.gen == INT32_MAX) {  // flags hold generations: restart them
        L.gen = 1;
        NW_CUDA(cudaMemsetAsync(L.eflag, 0, ls->fsched.chunks * sizeof(int), ls->stream));
        NW_CUDA(cudaMemsetAsync(L.rflag, 0, ls->fsched.blocks * sizeof(int), ls->stream));
      }
      L.accumulate = write_mode(ls);
      // the system's arrays as they are now
      L.values = ls->values.p;
      L.rhs = ls->rhs.p;
      L.row_ptr = ls->row_ptr.p;
      L.inc_ptr = ls->inc_ptr.p;
      L.inc = ls->inc.p;
      L.diag_pos = ls->diag_pos.p;
      if (!ls->ring.p) L.ring = ls->buf.p;
      launch_momentum_fused(ls->stream, L, ls->edges.p, *f, *o);
      NW_CUDA(cudaGetLastError());
      ls->pristine = false;
    } else {
      launch_momentum_edges(ls->stream, E, 0, E, ls->edges.p, *f, *o, ls->buf.p);
      momentum_rows(ls, o->relax);
    }
    end_timing(ls);
  });
}

nw_status nw_assemble_momentum_edge_range(nw_linsys* ls, const nw_momentum_fields* f,
                                          const nw_momentum_opts* o, int64_t edge_begin,
                                          int64_t edge_end) {
  return guard([&] {
    check_momentum_args(ls, f, o);
    const int64_t E = ls->g.num_edges;
    if (edge_begin < 0 || edge_end > E || edge_begin > edge_end)
      fail(NW_INVALID_ARG, "edge range out of bounds");
    launch_momentum_edges(ls->stream, E, edge_begin, edge_end, ls->edges.p, *f, *o, ls->buf.p);
    NW_CUDA(cudaGetLastError());
  });
}

nw_status nw_assemble_momentum_rows_range(nw_linsys* ls, const nw_momentum_opts* o,
                                          int64_t row_begin, int64_t row_end) {
  return guard([&] {
    need_finalized(ls);
    if (ls->num_dof != 3) fail(NW_INVALID_ARG, "momentum assembly needs num_dof 3");
    if (!o) fail(NW_INVALID_ARG, "null argument");
    if (!(o->relax != 0.0)) fail(NW_INVALID_ARG, "relaxation factor is zero");
    const int64_t R = ls->g.node_rows;
    if (row_begin < 0 || row_end > R || row_begin > row_end) fail(NW_INVALID_ARG, "row range out of bounds");
    if (row_begin == row_end) return;
    int accumulate = 1;
    if (ls->pristine) {
      // on a zeroed system the ranges overwrite, so they must come in order
      if (row_begin != ls->pristine_from)
        fail(NW_INVALID_ARG, "after zeroSystem, row ranges must follow each other from row 0");
      accumulate = 0;
    }
    launch_rows(ls->stream, 2, row_end, ls->inc_ptr.p, ls->inc.p, ls->diag_pos.p, ls->row_ptr.p,
                ls->buf.p, ls->g.num_edges, o->relax, ls->values.p, ls->rhs.p, accumulate,
                ls->stage_bytes[2], ls->max_inc, row_begin);
    NW_CUDA(cudaGetLastError());
    if (ls->pristine) {
      ls->pristine_from = row_end;
      if (row_end == R) {
        ls->pristine = false;
        ls->pristine_from = 0;
      }
    }
  });
}

nw_status nw_assemble_momentum_rows(nw_linsys* ls, const nw_momentum_opts* o) {
  return guard([&] {
    need_finalized(ls);
    if (ls->num_dof != 3) fail(NW_INVALID_ARG, "momentum assembly needs num_dof 3");
    if (!o) fail(NW_INVALID_ARG, "null argument");
    if (!(o->relax != 0.0)) fail(NW_INVALID_ARG, "relaxation factor is zero");
    momentum_rows(ls, o->relax);
  });
}

nw_status nw_linsys_sum_into(nw_linsys* ls, int n_ent, const int64_t* nodes,
                             const double* rhs, const double* lhs) {
  return guard([&] {
    need_finalized(ls);
    if (n_ent < 1 || n_ent * ls->num_dof > 128 || !nodes || !rhs || !lhs)
      fail(NW_INVALID_ARG, "bad sum_into block");
    materialize_zero(ls);
    const int nd = ls->num_dof, nloc = n_ent * nd;
    std::vector<int64_t> lid(n_ent);
    for (int i = 0; i < n_ent; ++i) {
      if (nodes[i] < 0 || nodes[i] >= ls->g.num_nodes)
        fail(NW_INVALID_ARG, "node index out of range");
      lid[i] = ls->g.node_lid[nodes[i]];
    }
    ls->scratch_lid.upload(lid, ls->stream);
    std::vector<double> tmp(size_t(nloc) * nloc + nloc);
    std::memcpy(tmp.data(), lhs, sizeof(double) * nloc * nloc);
    std::memcpy(tmp.data() + size_t(nloc) * nloc, rhs, sizeof(double) * nloc);
    ls->scratch_vals.upload(tmp, ls->stream);
    launch_sum_into_block(ls->stream, n_ent, nd, ls->scratch_lid.p,
                          ls->scratch_vals.p, ls->scratch_vals.p + size_t(nloc) * nloc,
                          ls->row_ptr.p, ls->col_idx.p, ls->values.p, ls->rhs.p);
    NW_CUDA(cudaGetLastError());
    NW_CUDA(cudaStreamSynchronize(ls->stream));
  });
}

nw_status nw_linsys_apply_dirichlet(nw_linsys* ls, int64_t n,
                                    const int64_t* nodes, int begin, int end,
                                    const double* q, const double* bc) {
  return guard([&] {
    need_finalized(ls);
    if (n < 0 || (n > 0 && (!nodes || !q || !bc)) || begin < 0 ||
        end > ls->num_dof || begin > end)
      fail(NW_INVALID_ARG, "bad Dirichlet arguments");
    materialize_zero(ls);
    NW_CUDA(cudaMemsetAsync(ls->err.p, 0, sizeof(int), ls->stream));
    launch_reset_rows(ls->stream, n, nodes, ls->node_lid.p, ls->num_dof, begin,
                      end, ls->row_ptr.p, ls->col_idx.p, ls->values.p,
                      ls->rhs.p, 1.0, 0.0, q, bc, ls->g.num_nodes, ls->err.p);
    NW_CUDA(cudaGetLastError());
    int herr = 0;
    NW_CUDA(cudaMemcpyAsync(&herr, ls->err.p, sizeof(int), cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    if (herr) fail(NW_INVALID_ARG, "Dirichlet node index out of range");
  });
}

nw_status nw_linsys_reset_rows(nw_linsys* ls, int64_t n, const int64_t* nodes,
                               int begin, int end, double diag_value,
                               double rhs_residual) {
  return guard([&] {
    need_finalized(ls);
    if (n < 0 || (n > 0 && !nodes) || begin < 0 || end > ls->num_dof ||
        begin > end)
      fail(NW_INVALID_ARG, "bad resetRows arguments");
    materialize_zero(ls);
    NW_CUDA(cudaMemsetAsync(ls->err.p, 0, sizeof(int), ls->stream));
    launch_reset_rows(ls->stream, n, nodes, ls->node_lid.p, ls->num_dof, begin,
                      end, ls->row_ptr.p, ls->col_idx.p, ls->values.p,
                      ls->rhs.p, diag_value, rhs_residual, nullptr, nullptr,
                      ls->g.num_nodes, ls->err.p);
    NW_CUDA(cudaGetLastError());
    int herr = 0;
    NW_CUDA(cudaMemcpyAsync(&herr, ls->err.p, sizeof(int), cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    if (herr) fail(NW_INVALID_ARG, "resetRows node index out of range");
  });
}

nw_status nw_linsys_load_complete(nw_linsys* ls) {
  return guard([&] {
    need_finalized(ls);
    materialize_zero(ls);
  });
}

nw_status nw_linsys_device_arrays(nw_linsys* ls, double** values, double** rhs,
                                  const int64_t** row_ptr,
                                  const int32_t** col_idx) {
  return guard([&] {
    need_finalized(ls);
    materialize_zero(ls);
    if (values) *values = ls->values.p;
    if (rhs) *rhs = ls->rhs.p;
    if (row_ptr) *row_ptr = ls->row_ptr.p;
    if (col_idx) *col_idx = ls->col_idx.p;
  });
}

nw_status nw_linsys_copy_to_host(nw_linsys* ls, double* values, double* rhs) {
  return guard([&] {
    need_finalized(ls);
    materialize_zero(ls);
    if (values)
      NW_CUDA(cudaMemcpyAsync(values, ls->values.p, ls->values.n * sizeof(double),
                              cudaMemcpyDeviceToHost, ls->stream));
    if (rhs)
      NW_CUDA(cudaMemcpyAsync(rhs, ls->rhs.p, ls->rhs.n * sizeof(double),
                              cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
  });
}

nw_status nw_linsys_copy_from_host(nw_linsys* ls, const double* values,
                                   const double* rhs) {
  return guard([&] {
    need_finalized(ls);
    materialize_zero(ls);
    if (values)
      NW_CUDA(cudaMemcpyAsync(ls->values.p, values, ls->values.n * sizeof(double),
                              cudaMemcpyHostToDevice, ls->stream));
    if (rhs)
      NW_CUDA(cudaMemcpyAsync(ls->rhs.p, rhs, ls->rhs.n * sizeof(double),
                              cudaMemcpyHostToDevice, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    check_fused(ls);
  });
}

nw_status nw_linsys_solve(nw_linsys* ls, double* x, int final_iter,
                          nw_solve_report* rep) {
  return guard([&] {
    need_finalized(ls);
    if (!x) fail(NW_INVALID_ARG, "null solution vector");
    materialize_zero(ls);
    check_fused(ls);
    if (ls->cfg.preconditioner == NW_PC_LEARNED && !ls->coarse)
      fail(NW_INVALID_ARG, "NW_PC_LEARNED needs nw_linsys_attach_learned");
    ls->pc.kind = ls->cfg.preconditioner;
    ls->pc.inner_sweeps = ls->cfg.sgs2_inner_sweeps > 0 ? ls->cfg.sgs2_inner_sweeps : 1;
    const double tol = final_iter ? ls->cfg.final_tolerance : ls->cfg.tolerance;
    cudaEvent_t a, b;
    NW_CUDA(cudaEventCreate(&a));
    NW_CUDA(cudaEventCreate(&b));
    // the timed solve includes the per-solve refresh of the solver's copies
    // of the values (diagonal, sliced layouts, coarse Galerkin operator)
    NW_CUDA(cudaEventRecord(a, ls->stream));
    cudaStream_t s = ls->stream;
    const bool legacy = s == nullptr || s == cudaStreamLegacy;
    if (legacy) {
      if (!ls->solve_stream) {
        NW_CUDA(cudaStreamCreateWithFlags(&ls->solve_stream, cudaStreamNonBlocking));
        NW_CUDA(cudaEventCreateWithFlags(&ls->solve_in, cudaEventDisableTiming));
        NW_CUDA(cudaEventCreateWithFlags(&ls->solve_out, cudaEventDisableTiming));
      }
      NW_CUDA(cudaEventRecord(ls->solve_in, ls->stream));
      NW_CUDA(cudaStreamWaitEvent(ls->solve_stream, ls->solve_in, 0));
      s = ls->solve_stream;
    }
    SolveResult r;
    try {
      ls->solver.refresh(s);
      r = ls->solver.solve(ls->cfg, tol, ls->pc, ls->rhs.p, x, s);
    } catch (...) {
      if (legacy) {  // later work on the caller's stream still follows the solve's
        cudaEventRecord(ls->solve_out, s);
        cudaStreamWaitEvent(ls->stream, ls->solve_out, 0);
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      throw;
    }
    if (legacy) {
      NW_CUDA(cudaEventRecord(ls->solve_out, s));
      NW_CUDA(cudaStreamWaitEvent(ls->stream, ls->solve_out, 0));
    }
    NW_CUDA(cudaEventRecord(b, ls->stream));
    NW_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    NW_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ls->history = r.history;
    nw_solve_report out{};
    out.iterations = r.iterations;
    out.outer_iterations = r.outer;
    out.status = r.status;
    out.converged = r.converged;
    out.final_rel_residual = r.final_rel;
    out.final_abs_residual = r.final_abs;
    out.rhs_norm = r.bnorm;
    out.solve_ms = ms;
    out.fallback = r.fallback;
    ls->last_report = out;
    if (rep) *rep = out;
    if (r.status == NW_NAN_DETECTED) fail(NW_NAN_DETECTED, "non-finite value in the solve");
  });
}

// ---- checkpoint / resume: raw binary file of the system and solver state.
// Layout (little-endian, native sizes): CkptHeader, then row_ptr (int64,
// nrows + 1), col_idx (int32, nnz), values (f64, nnz), rhs (f64, nrows),
// the last residual history (f64, nhist), and x (f64, nrows) when has_x.
// `checksum` is FNV-1a over every byte after the header.
namespace {
struct CkptHeader {
  char magic[8];
  uint32_t version;
  uint32_t num_dof;
  int64_t nrows, nnz, nhist;
  int32_t has_x, pad;
  nw_solver_cfg cfg;
  nw_solve_report report;
  uint64_t checksum;
};
constexpr char kCkptMagic[8] = {'N', 'W', 'C', 'K', 'P', 'T', '0', '1'};

struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void add(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      h ^= c[i];
      h *= 1099511628211ull;
    }
  }
};
}  // namespace

nw_status nw_linsys_checkpoint_save(nw_linsys* ls, const char* path, const double* x) {
  return guard([&] {
    need_finalized(ls);
    if (!path) fail(NW_INVALID_ARG, "null path");
    materialize_zero(ls);
    const HostGraph& g = ls->g;
    std::vector<double> vals(g.nnz), rhs(g.nrows), xh(x ? g.nrows : 0);
    NW_CUDA(cudaMemcpyAsync(vals.data(), ls->values.p, g.nnz * sizeof(double), cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaMemcpyAsync(rhs.data(), ls->rhs.p, g.nrows * sizeof(double), cudaMemcpyDeviceToHost, ls->stream));
    if (x) NW_CUDA(cudaMemcpyAsync(xh.data(), x, g.nrows * sizeof(double), cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    CkptHeader h{};
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = 1;
    h.num_dof = uint32_t(ls->num_dof);
    h.nrows = g.nrows;
    h.nnz = g.nnz;
    h.nhist = int64_t(ls->history.size());
    h.has_x = x ? 1 : 0;
    h.cfg = ls->cfg;
    h.report = ls->last_report;
    Fnv f;
    f.add(g.row_ptr.data(), g.row_ptr.size() * sizeof(int64_t));
    f.add(g.col_idx.data(), g.col_idx.size() * sizeof(int32_t));
    f.add(vals.data(), vals.size() * sizeof(double));
    f.add(rhs.data(), rhs.size() * sizeof(double));
    f.add(ls->history.data(), ls->history.size() * sizeof(double));
    f.add(xh.data(), xh.size() * sizeof(double));
    h.checksum = f.h;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) fail(NW_INVALID_ARG, std::string("cannot open ") + path);
    bool ok = std::fwrite(&h, sizeof(h), 1, fp) == 1;
    auto put = [&](const void* p, size_t n) { ok = ok && (n == 0 || std::fwrite(p, 1, n, fp) == n); };
    put(g.row_ptr.data(), g.row_ptr.size() * sizeof(int64_t));
    put(g.col_idx.data(), g.col_idx.size() * sizeof(int32_t));
    put(vals.data(), vals.size() * sizeof(double));
    put(rhs.data(), rhs.size() * sizeof(double));
    put(ls->history.data(), ls->history.size() * sizeof(double));
    put(xh.data(), xh.size() * sizeof(double));
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) fail(NW_INVALID_ARG, std::string("short write to ") + path);
  });
}

nw_status nw_linsys_checkpoint_load(nw_linsys* ls, const char* path, double* x, nw_solve_report* rep) {
  return guard([&] {
    need_finalized(ls);
    if (!path) fail(NW_INVALID_ARG, "null path");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) fail(NW_INVALID_ARG, std::string("cannot open ") + path);
    std::unique_ptr<FILE, int (*)(FILE*)> closer(fp, std::fclose);
    CkptHeader h{};
    if (std::fread(&h, sizeof(h), 1, fp) != 1 || std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1)
      fail(NW_INVALID_ARG, "not a checkpoint of this library");
    const HostGraph& g = ls->g;
    if (int(h.num_dof) != ls->num_dof || h.nrows != g.nrows || h.nnz != g.nnz || h.nhist < 0 ||
        h.nhist > (int64_t(1) << 32))
      fail(NW_INVALID_ARG, "checkpoint sizes differ from this linear system");
    std::vector<int64_t> rp(g.nrows + 1);
    std::vector<int32_t> ci(g.nnz);
    std::vector<double> vals(g.nnz), rhs(g.nrows), hist(h.nhist), xh(h.has_x ? g.nrows : 0);
    bool ok = true;
    auto get = [&](void* p, size_t n) { ok = ok && (n == 0 || std::fread(p, 1, n, fp) == n); };
    get(rp.data(), rp.size() * sizeof(int64_t));
    get(ci.data(), ci.size() * sizeof(int32_t));
    get(vals.data(), vals.size() * sizeof(double));
    get(rhs.data(), rhs.size() * sizeof(double));
    get(hist.data(), hist.size() * sizeof(double));
    get(xh.data(), xh.size() * sizeof(double));
    if (!ok) fail(NW_INVALID_ARG, "truncated checkpoint");
    Fnv f;
    f.add(rp.data(), rp.size() * sizeof(int64_t));
    f.add(ci.data(), ci.size() * sizeof(int32_t));
    f.add(vals.data(), vals.size() * sizeof(double));
    f.add(rhs.data(), rhs.size() * sizeof(double));
    f.add(hist.data(), hist.size() * sizeof(double));
    f.add(xh.data(), xh.size() * sizeof(double));
    if (f.h != h.checksum) fail(NW_INVALID_ARG, "checkpoint checksum mismatch");
    if (rp != g.row_ptr || ci != g.col_idx) fail(NW_INVALID_ARG, "checkpoint graph differs from this linear system");
    if (x && !h.has_x) fail(NW_INVALID_ARG, "checkpoint holds no solution vector");
    check_cfg(h.cfg);
    NW_CUDA(cudaMemcpyAsync(ls->values.p, vals.data(), g.nnz * sizeof(double), cudaMemcpyHostToDevice, ls->stream));
    NW_CUDA(cudaMemcpyAsync(ls->rhs.p, rhs.data(), g.nrows * sizeof(double), cudaMemcpyHostToDevice, ls->stream));
    if (x) NW_CUDA(cudaMemcpyAsync(x, xh.data(), g.nrows * sizeof(double), cudaMemcpyHostToDevice, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    ls->pristine = false;
    const bool grow = h.cfg.kspace > ls->cfg.kspace || h.cfg.inner_kspace > ls->cfg.inner_kspace;
    ls->cfg = h.cfg;
    if (grow) {
      DevCsr A;
      A.n = g.nrows;
      A.nnz = g.nnz;
      A.row_ptr = ls->row_ptr.p;
      A.col_idx = ls->col_idx.p;
      A.values = ls->values.p;
      A.lanes = ls->num_dof == 1 ? 8 : 32;
      A.row_ptr_host = g.row_ptr.data();
      A.col_idx_host = g.col_idx.data();
      ls->solver.setup(A, std::max(ls->cfg.kspace, ls->cfg.inner_kspace), ls->stream);
      ls->solver.setup_colors(ls->color_rows_host, ls->color_ptr, ls->stream);
    }
    ls->history = hist;
    ls->last_report = h.report;
    if (rep) *rep = h.report;
  });
}

// MatrixMarket files of the system in the layout of
// TpetraLinearSystem::writeToFile (src/TpetraLinearSystem.C:2017-2045):
// <base>-O-<count>.mm.1 (coordinate real general, 1-based global dof ids
// GID = ndof (nalu id - 1) + d + 1, TpetraLinearSystemHelpers.h:33) and
// <base>-O-<count>.rhs.1 (array real general); with x also .sln.1. Sizes
// are the largest global dof id (global ids of periodic slaves are unused).
nw_status nw_linsys_write_matrix_market(nw_linsys* ls, const char* base, int count,
                                        const double* x_host) {
  return guard([&] {
    need_finalized(ls);
    if (!base) fail(NW_INVALID_ARG, "null file name");
    materialize_zero(ls);
    const HostGraph& g = ls->g;
    const int nd = g.num_dof;
    std::vector<double> v(g.nnz), b(g.nrows);
    NW_CUDA(cudaMemcpyAsync(v.data(), ls->values.p, g.nnz * 8, cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaMemcpyAsync(b.data(), ls->rhs.p, g.nrows * 8, cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    auto gid = [&](int64_t row) { return nd * (g.row_gid[row / nd] - 1) + row % nd + 1; };
    int64_t dim = 0;
    for (int64_t r = 0; r < g.node_rows; ++r) dim = std::max<int64_t>(dim, nd * g.row_gid[r]);
    const std::string stem = std::string(base) + "-O-" + std::to_string(count);
    auto open = [&](const std::string& path) {
      FILE* fp = std::fopen(path.c_str(), "w");
      if (!fp) fail(NW_INVALID_ARG, "cannot open " + path + " for writing");
      return fp;
    };
    FILE* fa = open(stem + ".mm.1");
    std::fprintf(fa, "%%%%MatrixMarket matrix coordinate real general\n");
    std::fprintf(fa, "%% nalu-wind linear system (%d dof per node), global dof ids\n", nd);
    std::fprintf(fa, "%lld %lld %lld\n", (long long)dim, (long long)dim, (long long)g.nnz);
    for (int64_t r = 0; r < g.nrows; ++r)
      for (int64_t p = g.row_ptr[r]; p < g.row_ptr[r + 1]; ++p)
        std::fprintf(fa, "%lld %lld %.17e\n", (long long)gid(r), (long long)gid(g.col_idx[p]), v[p]);
    const bool ok_a = std::fclose(fa) == 0;
    auto dense = [&](const std::string& path, const double* a) {
      FILE* fb = open(path);
      std::fprintf(fb, "%%%%MatrixMarket matrix array real general\n");
      std::fprintf(fb, "%lld 1\n", (long long)dim);
      // array format lists every global row; unused ids (periodic slaves) are 0
      std::vector<double> full(dim, 0.0);
      for (int64_t r = 0; r < g.nrows; ++r) full[gid(r) - 1] = a[r];
      for (int64_t k = 0; k < dim; ++k) std::fprintf(fb, "%.17e\n", full[k]);
      return std::fclose(fb) == 0;
    };
    const bool ok_b = dense(stem + ".rhs.1", b.data());
    const bool ok_x = x_host ? dense(stem + ".sln.1", x_host) : true;
    if (!ok_a || !ok_b || !ok_x) fail(NW_INVALID_ARG, "write failed: " + stem);
  });
}

// Reads a coordinate MatrixMarket matrix (and optionally an array rhs)
// written for this graph: every entry must be a column of the graph
// (NW_INVALID_ARG otherwise); entries not in the file become zero.
nw_status nw_linsys_read_matrix_market(nw_linsys* ls, const char* matrix_path,
                                       const char* rhs_path) {
  return guard([&] {
    need_finalized(ls);
    if (!matrix_path) fail(NW_INVALID_ARG, "null file name");
    const HostGraph& g = ls->g;
    const int nd = g.num_dof;
    // global dof id -> local row
    std::vector<int64_t> row_of;
    int64_t dim = 0;
    for (int64_t r = 0; r < g.node_rows; ++r) dim = std::max<int64_t>(dim, nd * g.row_gid[r]);
    row_of.assign(dim + 1, -1);
    for (int64_t r = 0; r < g.nrows; ++r) row_of[nd * (g.row_gid[r / nd] - 1) + r % nd + 1] = r;
    FILE* fa = std::fopen(matrix_path, "r");
    if (!fa) fail(NW_INVALID_ARG, std::string("cannot open ") + matrix_path);
    std::vector<double> v(g.nnz, 0.0), b(g.nrows, 0.0);
    char line[512];
    bool header = false, sized = false;
    long long m = 0, n = 0, cnt = 0, seen = 0;
    std::string err;
    while (std::fgets(line, sizeof line, fa)) {
      if (line[0] == '%') {
        if (!header) header = std::strstr(line, "coordinate") && std::strstr(line, "real");
        continue;
      }
      if (!sized) {
        if (std::sscanf(line, "%lld %lld %lld", &m, &n, &cnt) != 3) { err = "bad size line"; break; }
        if (m != dim || n != dim) { err = "matrix size does not match this system"; break; }
        sized = true;
        continue;
      }
      long long i, j;
      double a;
      if (std::sscanf(line, "%lld %lld %lf", &i, &j, &a) != 3) { err = "bad entry line"; break; }
      const int64_t r = (i >= 1 && i <= dim) ? row_of[i] : -1, c = (j >= 1 && j <= dim) ? row_of[j] : -1;
      if (r < 0 || c < 0) { err = "entry outside the system's rows"; break; }
      const auto b0 = g.col_idx.begin() + g.row_ptr[r], b1 = g.col_idx.begin() + g.row_ptr[r + 1];
      const auto it = std::lower_bound(b0, b1, int32_t(c));
      if (it == b1 || *it != int32_t(c)) { err = "entry not in the graph"; break; }
      v[it - g.col_idx.begin()] += a;
      ++seen;
    }
    std::fclose(fa);
    if (err.empty() && !header) err = "not a coordinate real MatrixMarket file";
    if (err.empty() && seen != cnt) err = "entry count does not match the size line";
    if (!err.empty()) fail(NW_INVALID_ARG, err + ": " + matrix_path);
    if (rhs_path) {
      FILE* fb = std::fopen(rhs_path, "r");
      if (!fb) fail(NW_INVALID_ARG, std::string("cannot open ") + rhs_path);
      bool sz = false;
      int64_t k = 0;
      while (std::fgets(line, sizeof line, fb)) {
        if (line[0] == '%') continue;
        if (!sz) {
          long long mm = 0, nn = 0;
          if (std::sscanf(line, "%lld %lld", &mm, &nn) != 2 || mm != dim || nn != 1) { err = "bad rhs size"; break; }
          sz = true;
          continue;
        }
        double a;
        if (std::sscanf(line, "%lf", &a) != 1 || k >= dim) { err = "bad rhs entry"; break; }
        if (row_of[k + 1] >= 0) b[row_of[k + 1]] = a;
        ++k;
      }
      std::fclose(fb);
      if (err.empty() && k != dim) err = "rhs length does not match";
      if (!err.empty()) fail(NW_INVALID_ARG, err + ": " + rhs_path);
    }
    NW_CUDA(cudaMemcpyAsync(ls->values.p, v.data(), g.nnz * 8, cudaMemcpyHostToDevice, ls->stream));
    if (rhs_path)
      NW_CUDA(cudaMemcpyAsync(ls->rhs.p, b.data(), g.nrows * 8, cudaMemcpyHostToDevice, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    ls->pristine = false;
  });
}

static nw_status mass_bdf(nw_linsys* ls, int kind, const nw_mass_bdf_fields* f,
                          const nw_bdf_opts* o) {
  return guard([&] {
    need_finalized(ls);
    if (!f || !o) fail(NW_INVALID_ARG, "null argument");
    if (ls->num_dof != (kind == 2 ? 3 : 1))
      fail(NW_INVALID_ARG, kind == 2 ? "momentum mass terms need num_dof 3" : "mass terms need num_dof 1");
    if (!f->density_nm1 || !f->density_n || !f->density_np1 || !f->dual_volume_nm1 ||
        !f->dual_volume_n || !f->dual_volume_np1)
      fail(NW_INVALID_ARG, "null density or dual volume");
    if (kind != 1 && (!f->q_nm1 || !f->q_n || !f->q_np1)) fail(NW_INVALID_ARG, "null transported field");
    if (kind == 2 && !f->dpdx) fail(NW_INVALID_ARG, "null dpdx");
    if (!(o->dt != 0.0)) fail(NW_INVALID_ARG, "dt is zero");
    if (kind != 1)
      for (int32_t dp : ls->g.diag_pos)
        if (dp < 0)
          fail(NW_INVALID_ARG,
               "a node in no edge has no diagonal entry in the edge graph; its mass term "
               "cannot be added");
    materialize_zero(ls);
    launch_mass_bdf(ls->stream, kind, plan_view(ls), *f, *o, ls->values.p, ls->rhs.p);
  });
}

}  // extern "C"

// A side set: face IPs grouped by the node row of their face node.
struct nw_sideset {
  const nw_linsys* ls = nullptr;
  int64_t num_ips = 0;
  int64_t nb = 0;
  DeviceArray<int32_t> brow, bptr;
  DeviceArray<int4> ips;
  int64_t nl = 0;  // the IPs grouped by the opposing node's row
  DeviceArray<int32_t> lrow, lptr;
  DeviceArray<int4> lips;
  DeviceArray<double> total;  // device sum of the open mass flow rates
};

namespace {

SideView side_view(const nw_linsys* ls, const nw_sideset* s) {
  need_finalized(ls);
  if (!s) fail(NW_INVALID_ARG, "null side set");
  if (s->ls != ls) fail(NW_INVALID_ARG, "side set was registered on another linear system");
  SideView v;
  v.nip = s->num_ips;
  v.nb = s->nb;
  v.brow = s->brow.p;
  v.bptr = s->bptr.p;
  v.ips = s->ips.p;
  v.row_ptr = ls->row_ptr.p;
  v.diag_pos = ls->diag_pos.p;
  v.nl = s->nl;
  v.lrow = s->lrow.p;
  v.lptr = s->lptr.p;
  v.lips = s->lips.p;
  return v;
}

void need_dof(const nw_linsys* ls, int nd, const char* what) {
  if (ls->num_dof != nd)
    fail(NW_INVALID_ARG, std::string(what) + (nd == 3 ? " needs num_dof 3" : " needs num_dof 1"));
}

}  // namespace

extern "C" {

nw_status nw_sideset_create(nw_linsys* ls, int64_t num_ips, const int64_t* ip_nodes,
                            nw_sideset** out) {
  return guard([&] {
    need_finalized(ls);
    if (!out) fail(NW_INVALID_ARG, "null output");
    *out = nullptr;
    if (num_ips < 0 || num_ips >= (int64_t(1) << 31)) fail(NW_INVALID_ARG, "bad IP count");
    if (num_ips > 0 && !ip_nodes) fail(NW_INVALID_ARG, "null ip_nodes");
    const HostGraph& g = ls->g;
    const int nd = ls->num_dof;
    struct Ip {
      int32_t row, ip, R, L, kL;
    };
    std::vector<Ip> v(static_cast<size_t>(num_ips));
    for (int64_t i = 0; i < num_ips; ++i) {
      const int64_t R = ip_nodes[2 * i], L = ip_nodes[2 * i + 1];
      if (R < 0 || R >= g.num_nodes || L < 0 || L >= g.num_nodes)
        fail(NW_INVALID_ARG, "face IP node index out of range");
      const int64_t rowR = g.node_lid[R] / nd, rowL = g.node_lid[L] / nd;
      const int32_t* b = g.ncol.data() + g.nrow_ptr[rowR];
      const int32_t* e = g.ncol.data() + g.nrow_ptr[rowR + 1];
      const int32_t* it = std::lower_bound(b, e, int32_t(rowL));
      if (it == e || *it != rowL || g.diag_pos[rowR] < 0)
        fail(NW_INVALID_ARG, "face node " + std::to_string(R) + " and opposing node " +
                                 std::to_string(L) + " are not joined by a graph edge");
      v[size_t(i)] = {int32_t(rowR), int32_t(i), int32_t(R), int32_t(L), int32_t(it - b)};
    }
    std::stable_sort(v.begin(), v.end(), [](const Ip& a, const Ip& b) { return a.row < b.row; });
    std::vector<int32_t> brow, bptr{0};
    std::vector<int4> ips(v.size());
    for (size_t k = 0; k < v.size(); ++k) {
      if (k == 0 || v[k].row != v[k - 1].row) {
        if (k) bptr.push_back(int32_t(k));
        brow.push_back(v[k].row);
      }
      ips[k] = make_int4(v[k].ip, v[k].R, v[k].L, v[k].kL);
    }
    if (!v.empty()) bptr.push_back(int32_t(v.size()));
    // the same IPs by the opposing node's row (IP order within a row)
    std::vector<std::pair<int32_t, int32_t>> byl(v.size());  // (row of L, position in v)
    for (size_t k = 0; k < v.size(); ++k) byl[k] = {int32_t(g.node_lid[v[k].L] / nd), int32_t(k)};
    std::stable_sort(byl.begin(), byl.end(), [&](const auto& a, const auto& b) {
      return a.first != b.first ? a.first < b.first : v[a.second].ip < v[b.second].ip;
    });
    std::vector<int32_t> lrow, lptr{0};
    std::vector<int4> lips(v.size());
    for (size_t k = 0; k < byl.size(); ++k) {
      if (k == 0 || byl[k].first != byl[k - 1].first) {
        if (k) lptr.push_back(int32_t(k));
        lrow.push_back(byl[k].first);
      }
      const Ip& q = v[size_t(byl[k].second)];
      lips[k] = make_int4(q.ip, q.R, q.L, 0);
    }
    if (!byl.empty()) lptr.push_back(int32_t(byl.size()));
    auto s = std::make_unique<nw_sideset>();
    s->ls = ls;
    s->num_ips = num_ips;
    s->nb = int64_t(brow.size());
    NW_CUDA(cudaSetDevice(ls->device));
    s->brow.upload(brow, ls->stream);
    s->bptr.upload(bptr, ls->stream);
    s->ips.upload(ips, ls->stream);
    s->nl = int64_t(lrow.size());
    s->lrow.upload(lrow, ls->stream);
    s->lptr.upload(lptr, ls->stream);
    s->lips.upload(lips, ls->stream);
    s->total.resize(1);
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    *out = s.release();
  });
}

nw_status nw_sideset_destroy(nw_sideset* s) {
  delete s;
  return NW_OK;
}

nw_status nw_sideset_sizes(const nw_sideset* s, int64_t* num_ips, int64_t* num_rows) {
  return guard([&] {
    if (!s) fail(NW_INVALID_ARG, "null side set");
    if (num_ips) *num_ips = s->num_ips;
    if (num_rows) *num_rows = s->nb;
  });
}

nw_status nw_assemble_continuity_open(nw_linsys* ls, const nw_sideset* s,
                                      const nw_continuity_open_fields* f,
                                      const nw_continuity_open_opts* o) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    need_dof(ls, 1, "continuity open boundary");
    if (!f || !o) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->coords, "coords");
    check_ptr(f->velocity, "velocity");
    check_ptr(f->dpdx, "dpdx");
    check_ptr(f->density, "density");
    check_ptr(f->pressure, "pressure");
    check_ptr(f->pressure_bc, "pressure_bc");
    check_ptr(f->udiag, "udiag");
    check_ptr(f->exposed_area, "exposed_area");
    if (!(o->tau_scale != 0.0)) fail(NW_INVALID_ARG, "tau_scale is zero");
    materialize_zero(ls);
    launch_continuity_open(ls->stream, v, *f, *o, ls->values.p, ls->rhs.p);
  });
}

nw_status nw_assemble_momentum_open(nw_linsys* ls, const nw_sideset* s,
                                    const nw_momentum_open_fields* f,
                                    const nw_momentum_open_opts* o) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    need_dof(ls, 3, "momentum open boundary");
    if (!f || !o) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->coords, "coords");
    check_ptr(f->velocity, "velocity");
    check_ptr(f->dudx, "dudx");
    check_ptr(f->viscosity, "viscosity");
    check_ptr(f->velocity_bc, "velocity_bc");
    check_ptr(f->exposed_area, "exposed_area");
    check_ptr(f->open_mass_flow_rate, "open_mass_flow_rate");
    if (o->entrainment != NW_ENTRAIN_COMPUTED && o->entrainment != NW_ENTRAIN_SPECIFIED)
      fail(NW_INVALID_ARG, "invalid entrainment method");
    materialize_zero(ls);
    launch_momentum_open(ls->stream, v, *f, *o, ls->values.p, ls->rhs.p);
  });
}

nw_status nw_assemble_momentum_symmetry(nw_linsys* ls, const nw_sideset* s,
                                        const nw_momentum_symmetry_fields* f,
                                        const nw_momentum_symmetry_opts* o) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    need_dof(ls, 3, "momentum symmetry boundary");
    if (!f || !o) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->coords, "coords");
    check_ptr(f->velocity, "velocity");
    check_ptr(f->dudx, "dudx");
    check_ptr(f->viscosity, "viscosity");
    check_ptr(f->exposed_area, "exposed_area");
    materialize_zero(ls);
    launch_momentum_symmetry(ls->stream, v, *f, *o, ls->values.p, ls->rhs.p);
  });
}

nw_status nw_assemble_momentum_abl_wall(nw_linsys* ls, const nw_sideset* s,
                                        const nw_abl_wall_fields* f, const nw_abl_wall_opts* o) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    need_dof(ls, 3, "ABL wall function");
    if (!f || !o) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->velocity, "velocity");
    check_ptr(f->wall_velocity_bc, "wall_velocity_bc");
    check_ptr(f->density, "density");
    check_ptr(f->heat_flux_bc, "heat_flux_bc");
    check_ptr(f->specific_heat, "specific_heat");
    check_ptr(f->exposed_area, "exposed_area");
    check_ptr(f->wall_friction_velocity, "wall_friction_velocity");
    check_ptr(f->wall_normal_distance, "wall_normal_distance");
    if (!(o->z0 > 0.0) || !(o->kappa > 0.0) || !(o->gravity != 0.0))
      fail(NW_INVALID_ARG, "z0 and kappa must be positive, gravity non-zero");
    materialize_zero(ls);
    launch_abl_wall(ls->stream, v, *f, *o, ls->values.p, ls->rhs.p);
  });
}

nw_status nw_assemble_momentum_abl_wall_shear_stress(nw_linsys* ls, const nw_sideset* s,
                                                     const double* exposed_area,
                                                     const double* wall_shear_stress, int slip) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    need_dof(ls, 3, "ABL wall shear stress");
    if (v.nip > 0) {
      check_ptr(exposed_area, "exposed_area");
      check_ptr(wall_shear_stress, "wall_shear_stress");
    }
    materialize_zero(ls);
    launch_abl_shear(ls->stream, v, exposed_area, wall_shear_stress, slip ? 1 : 0, ls->rhs.p);
  });
}

nw_status nw_compute_open_mdot(nw_linsys* ls, const nw_sideset* s,
                               const nw_continuity_open_fields* f, double noc_fac,
                               double pstab_fac, double* mdot, double* total) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    if (!f) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->coords, "coords");
    check_ptr(f->velocity, "velocity");
    check_ptr(f->dpdx, "dpdx");
    check_ptr(f->density, "density");
    check_ptr(f->pressure, "pressure");
    check_ptr(f->pressure_bc, "pressure_bc");
    check_ptr(f->udiag, "udiag");
    check_ptr(f->exposed_area, "exposed_area");
    if (v.nip > 0) check_ptr(mdot, "mdot");
    launch_open_mdot(ls->stream, v, *f, noc_fac, pstab_fac, mdot, s->total.p);
    double t = 0.0;
    NW_CUDA(cudaMemcpyAsync(&t, s->total.p, sizeof(double), cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    if (total) *total = t;
  });
}

nw_status nw_correct_open_mdot(nw_linsys* ls, const nw_sideset* s, double correction,
                               double* mdot, double* total) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    if (v.nip > 0) check_ptr(mdot, "mdot");
    launch_correct_open_mdot(ls->stream, v, correction, mdot, s->total.p);
    double t = 0.0;
    NW_CUDA(cudaMemcpyAsync(&t, s->total.p, sizeof(double), cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    if (total) *total = t;
  });
}

nw_status nw_assemble_scalar_open(nw_linsys* ls, const nw_sideset* s,
                                  const nw_scalar_open_fields* f, double relax) {
  return guard([&] {
    const SideView v = side_view(ls, s);
    need_dof(ls, 1, "scalar open boundary");
    if (!f) fail(NW_INVALID_ARG, "null argument");
    check_ptr(f->q, "q");
    check_ptr(f->q_bc, "q_bc");
    check_ptr(f->open_mass_flow_rate, "open_mass_flow_rate");
    if (!(relax != 0.0)) fail(NW_INVALID_ARG, "relaxation factor is zero");
    materialize_zero(ls);
    launch_scalar_open(ls->stream, v, *f, relax, ls->values.p, ls->rhs.p);
  });
}

nw_status nw_linsys_extract_diagonal(nw_linsys* ls, int dof, double* diag) {
  return guard([&] {
    need_finalized(ls);
    if (dof < 0 || dof >= ls->num_dof) fail(NW_INVALID_ARG, "dof out of range");
    if (ls->g.num_nodes > 0) check_ptr(diag, "diag");
    materialize_zero(ls);
    launch_extract_diagonal(ls->stream, plan_view(ls), dof, ls->values.p, diag);
  });
}

nw_status nw_udiag_postprocess(nw_linsys* ls, const double* density, const double* dual_volume,
                               double dt, double gamma1, double relax, double* udiag) {
  return guard([&] {
    need_finalized(ls);
    if (ls->g.num_nodes > 0) {
      check_ptr(density, "density");
      check_ptr(dual_volume, "dual_volume");
      check_ptr(udiag, "udiag");
    }
    if (!(dt != 0.0)) fail(NW_INVALID_ARG, "dt is zero");
    launch_udiag_postprocess(ls->stream, ls->g.num_nodes, density, dual_volume, gamma1 / dt, relax,
                             udiag);
  });
}

nw_status nw_assemble_scalar_mass_bdf(nw_linsys* ls, const nw_mass_bdf_fields* f,
                                      const nw_bdf_opts* o) {
  return mass_bdf(ls, 0, f, o);
}
nw_status nw_assemble_continuity_mass_bdf(nw_linsys* ls, const nw_mass_bdf_fields* f,
                                          const nw_bdf_opts* o) {
  return mass_bdf(ls, 1, f, o);
}
nw_status nw_assemble_momentum_mass_bdf(nw_linsys* ls, const nw_mass_bdf_fields* f,
                                        const nw_bdf_opts* o) {
  return mass_bdf(ls, 2, f, o);
}

nw_status nw_linsys_residual_history(const nw_linsys* ls, double* hist,
                                     int capacity, int* count) {
  return guard([&] {
    if (!ls) fail(NW_INVALID_ARG, "null handle");
    const int n = int(ls->history.size());
    if (count) *count = n;
    if (hist)
      std::memcpy(hist, ls->history.data(), sizeof(double) * std::min(n, capacity));
  });
}

nw_status nw_linsys_rows_to_nodes(nw_linsys* ls, const double* x_rows,
                                  double* x_nodes) {
  return guard([&] {
    need_finalized(ls);
    if (!x_rows || !x_nodes) fail(NW_INVALID_ARG, "null vector");
    // host-free gather: node_lid maps every node (slaves included) to rows
    const int64_t N = ls->g.num_nodes;
    const int nd = ls->num_dof;
    std::vector<double> hr(ls->g.nrows), hn(size_t(N) * nd);
    NW_CUDA(cudaMemcpyAsync(hr.data(), x_rows, hr.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    for (int64_t n = 0; n < N; ++n)
      for (int d = 0; d < nd; ++d) hn[n * nd + d] = hr[ls->g.node_lid[n] + d];
    NW_CUDA(cudaMemcpyAsync(x_nodes, hn.data(), hn.size() * sizeof(double),
                            cudaMemcpyHostToDevice, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
  });
}

nw_status nw_linsys_spmv(nw_linsys* ls, const double* x, double* y) {
  return guard([&] {
    need_finalized(ls);
    if (!x || !y) fail(NW_INVALID_ARG, "null vector");
    materialize_zero(ls);
    ls->solver.refresh(ls->stream);  // values may have changed since the last solve
    ls->solver.spmv(x, y, ls->stream);
    NW_CUDA(cudaGetLastError());
  });
}

nw_status nw_linsys_precond_apply(nw_linsys* ls, int preconditioner,
                                  const double* x, double* y) {
  return guard([&] {
    need_finalized(ls);
    if (!x || !y) fail(NW_INVALID_ARG, "null vector");
    if (preconditioner < NW_PC_NONE || preconditioner > NW_PC_RILUK ||
        preconditioner == NW_PC_LEARNED)
      fail(NW_INVALID_ARG, "preconditioner must be none, jacobi, mt_sgs, sgs2, sgs or riluk");
    materialize_zero(ls);
    ls->solver.refresh(ls->stream);
    Precond pc = ls->pc;
    pc.kind = preconditioner;
    pc.inner_sweeps = ls->cfg.sgs2_inner_sweeps > 0 ? ls->cfg.sgs2_inner_sweeps : 1;
    ls->solver.apply_precond(pc, x, y, ls->stream);
  });
}

nw_status nw_solver_cfg_from_strings(const char* method, const char* preconditioner,
                                     nw_solver_cfg* cfg) {
  return guard([&] {
    if (!method || !preconditioner || !cfg) fail(NW_INVALID_ARG, "null argument");
    const std::string m(method), p(preconditioner);
    int mi;
    if (m == "gmres") mi = NW_GMRES;
    else if (m == "cg") mi = NW_CG;
    else if (m == "sstep_gmres") mi = NW_SSTEP_GMRES;
    else if (m == "tfqmr") mi = NW_TFQMR;
    else if (m == "bicgstab") mi = NW_BICGSTAB;
    else fail(NW_INVALID_ARG, "unknown linear solver method '" + m + "'");
    int pi;
    if (p == "jacobi" || p == "default") pi = NW_PC_JACOBI;
    else if (p == "sgs") pi = NW_PC_SGS_NATURAL;
    else if (p == "mt_sgs") pi = NW_PC_SGS;
    else if (p == "sgs2") pi = NW_PC_SGS2;
    else if (p == "riluk") pi = NW_PC_RILUK;
    else if (p == "ilut" || p == "muelu")
      fail(NW_INVALID_ARG, "preconditioner '" + p + "' is not built by this library");
    else fail(NW_INVALID_ARG, "invalid linear solver preconditioner specified: '" + p + "'");
    cfg->method = mi;
    cfg->preconditioner = pi;
  });
}

nw_status nw_linsys_sgs_order(nw_linsys* ls, int64_t* order, int* ncolors) {
  return guard([&] {
    need_finalized(ls);
    if (order)
      for (size_t i = 0; i < ls->color_rows_host.size(); ++i)
        order[i] = ls->color_rows_host[i];
    if (ncolors) *ncolors = int(ls->color_ptr.size()) - 1;
  });
}

nw_status nw_linsys_sgs_classes(nw_linsys* ls, int64_t* class_ptr) {
  return guard([&] {
    need_finalized(ls);
    if (!class_ptr) fail(NW_INVALID_ARG, "null class_ptr");
    for (size_t i = 0; i < ls->color_ptr.size(); ++i) class_ptr[i] = ls->color_ptr[i];
  });
}

nw_status nw_linsys_sync(nw_linsys* ls) {
  return guard([&] {
    if (!ls) fail(NW_INVALID_ARG, "null handle");
    NW_CUDA(cudaStreamSynchronize(ls->stream));
    check_fused(ls);
  });
}

nw_status nw_linsys_set_assembly_path(nw_linsys* ls, int path) {
  return guard([&] {
    if (!ls) fail(NW_INVALID_ARG, "null handle");
    if (path != NW_ASSEMBLY_SINGLE_KERNEL && path != NW_ASSEMBLY_TWO_KERNELS)
      fail(NW_INVALID_ARG, "unknown assembly path");
    ls->assembly_path = path;
  });
}

nw_status nw_momentum_schedule(int64_t rows, int64_t num_edges, const int64_t* edge_rows,
                               int64_t concurrency, int64_t max_ring_bytes,
                               nw_assembly_schedule* info, int32_t* items, int32_t* chunk_lo,
                               int32_t* chunk_hi, int32_t* block_lo, int32_t* block_hi) {
  return guard([&] {
    if (!info || (num_edges > 0 && !edge_rows)) fail(NW_INVALID_ARG, "null argument");
    if (rows < 1 || num_edges < 0 || num_edges >= (int64_t(1) << 30) || concurrency < 1)
      fail(NW_INVALID_ARG, "size out of range");
    // incidence lists as the graph builder orders them (by column, then edge)
    std::vector<int32_t> ptr(size_t(rows) + 1, 0);
    for (int64_t e = 0; e < num_edges; ++e)
      for (int sd = 0; sd < 2; ++sd) {
        const int64_t r = edge_rows[2 * e + sd];
        if (r < 0 || r >= rows) fail(NW_INVALID_ARG, "edge row out of range");
        ++ptr[r + 1];
      }
    for (int64_t r = 0; r < rows; ++r) ptr[r + 1] += ptr[r];
    std::vector<uint32_t> inc(size_t(ptr[rows]));
    std::vector<int32_t> pos(ptr.begin(), ptr.end() - 1);
    for (int64_t e = 0; e < num_edges; ++e)
      for (int sd = 0; sd < 2; ++sd) inc[pos[edge_rows[2 * e + sd]]++] = uint32_t(e << 1 | sd);
    FusedSchedule fs;
    const int64_t slot_bytes = int64_t(kFusedChunk) * kMomentumCoefs * int64_t(sizeof(double));
    build_fused_schedule(num_edges, rows, ptr.data(), inc.data(), concurrency,
                         std::max<int64_t>(0, max_ring_bytes) / slot_bytes, fs);
    *info = nw_assembly_schedule{};
    info->single_kernel = 1;
    info->grid = int(std::min<int64_t>(concurrency, INT32_MAX));
    info->chunk_edges = kFusedChunk;
    info->block_rows = kFusedBlock;
    info->edge_chunks = fs.chunks;
    info->row_blocks = fs.blocks;
    info->ring_chunks = fs.ring_chunks;
    info->ring_bytes = fs.ring_chunks < fs.chunks ? fs.ring_chunks * slot_bytes : 0;
    info->lag_chunks = fs.lag;
    auto put = [](int32_t* dst, const std::vector<int32_t>& v) {
      if (dst) std::copy(v.begin(), v.end(), dst);
    };
    put(items, fs.items);
    put(chunk_lo, fs.chunk_lo);
    put(chunk_hi, fs.chunk_hi);
    put(block_lo, fs.block_lo);
    put(block_hi, fs.block_hi);
  });
}

nw_status nw_linsys_assembly_schedule(const nw_linsys* ls, nw_assembly_schedule* info) {
  return guard([&] {
    if (!ls || !info) fail(NW_INVALID_ARG, "null argument");
    need_finalized(ls);
    *info = nw_assembly_schedule{};
    info->single_kernel = ls->fused_ok ? 1 : 0;
    if (!ls->fused_ok) return;
    const FusedSchedule& fs = ls->fsched;
    info->edge_chunks = fs.chunks;
    info->row_blocks = fs.blocks;
    info->ring_chunks = fs.ring_chunks;
    info->ring_bytes = fs.ring_chunks < fs.chunks
                           ? fs.ring_chunks * kFusedChunk * kMomentumCoefs * int64_t(sizeof(double))
                           : 0;
    info->lag_chunks = fs.lag;
    info->grid = ls->fl.grid;
    info->chunk_edges = kFusedChunk;
    info->block_rows = kFusedBlock;
  });
}

nw_status nw_linsys_last_assembly_ms(const nw_linsys* ls, double* ms) {
  return guard([&] {
    if (!ls || !ms) fail(NW_INVALID_ARG, "null argument");
    if (!ls->timed) fail(NW_INVALID_ARG, "no assembly timed yet");
    NW_CUDA(cudaEventSynchronize(ls->ev1));
    float f = 0.f;
    NW_CUDA(cudaEventElapsedTime(&f, ls->ev0, ls->ev1));
    *ms = f;
  });
}

}  // extern "C"

namespace nw {
PlanView plan_view(const nw_linsys* ls) {
  need_finalized(ls);
  PlanView v;
  v.device = ls->device;
  v.num_dof = ls->num_dof;
  v.stream = ls->stream;
  v.num_edges = ls->g.num_edges;
  v.node_rows = ls->g.node_rows;
  v.nrows = ls->g.nrows;
  v.nnz = ls->g.nnz;
  v.edges = ls->edges.p;
  v.inc_ptr = ls->inc_ptr.p;
  v.inc = ls->inc.p;
  v.diag_pos = ls->diag_pos.p;
  v.row_ptr = ls->row_ptr.p;
  v.num_nodes = ls->g.num_nodes;
  v.row_nodes_ptr = ls->row_nodes_ptr.p;
  v.row_nodes = ls->row_nodes.p;
  v.node_lid = ls->node_lid.p;
  return v;
}
}  // namespace nw

// ---------------------------------------------------------------------------
// Learned preconditioner entry points.
namespace {

void need_learned(const nw_linsys* ls) {
  need_finalized(ls);
  if (!ls->coarse || !ls->learned)
    fail(NW_INVALID_ARG, "no learned preconditioner attached to this system");
}

}  // namespace

extern "C" {

int64_t nw_learned_num_params(void) { return kNumParams; }

nw_status nw_learned_create(uint64_t seed, nw_learned** out) {
  return guard([&] {
    if (!out) fail(NW_INVALID_ARG, "null output");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) fail(NW_NO_DEVICE, "no CUDA device");
    NW_CUDA(cudaSetDevice(g_device));
    auto p = std::make_unique<nw_learned>();
    p->net.init(seed, nullptr);
    NW_CUDA(cudaStreamSynchronize(nullptr));
    *out = p.release();
  });
}

nw_status nw_learned_destroy(nw_learned* net) {
  return guard([&] { delete net; });
}

nw_status nw_learned_save(nw_learned* net, const char* path) {
  return guard([&] {
    if (!net || !path) fail(NW_INVALID_ARG, "null argument");
    net->net.download(nullptr);
    save_params(path, net->net.params_h, uint64_t(net->net.adam_step));
  });
}

nw_status nw_learned_load(nw_learned* net, const char* path) {
  return guard([&] {
    if (!net || !path) fail(NW_INVALID_ARG, "null argument");
    std::vector<float> p;
    load_params(path, p);
    net->net.params_h = p;
    net->net.upload(nullptr);
    NW_CUDA(cudaStreamSynchronize(nullptr));
  });
}

nw_status nw_learned_params(nw_learned* net, float* out, const float* in, int64_t n) {
  return guard([&] {
    if (!net || n != kNumParams) fail(NW_INVALID_ARG, "parameter count mismatch");
    if (out) {
      net->net.download(nullptr);
      std::memcpy(out, net->net.params_h.data(), sizeof(float) * n);
    }
    if (in) {
      net->net.params_h.assign(in, in + n);
      net->net.upload(nullptr);
      NW_CUDA(cudaStreamSynchronize(nullptr));
    }
  });
}

nw_status nw_learned_configure(nw_learned* net, int post_smooth, int agg_passes, int smoother) {
  return guard([&] {
    if (!net || (post_smooth != 0 && post_smooth != 1) || agg_passes < 1 || agg_passes > 4 ||
        (smoother != 0 && smoother != 1))
      fail(NW_INVALID_ARG, "bad option");
    net->net.smoother = smoother;
    if (agg_passes != net->net.agg_passes && net->net.npairs > 0)
      fail(NW_INVALID_ARG, "harvested pairs use the current aggregation; clear them first");
    net->net.post_smooth = post_smooth;
    net->net.agg_passes = agg_passes;
  });
}

nw_status nw_learned_set_aggregation(nw_learned* net, double strength) {
  return guard([&] {
    if (!net || !(strength >= 0.0 && strength < 1.0)) fail(NW_INVALID_ARG, "bad aggregation threshold");
    if (strength != net->net.agg_strength && net->net.npairs > 0)
      fail(NW_INVALID_ARG, "harvested pairs use the current aggregation; clear them first");
    net->net.agg_strength = strength;
  });
}

nw_status nw_learned_set_coarse_direction(nw_learned* net, int mode) {
  return guard([&] {
    if (!net || mode < 0 || mode > 2) fail(NW_INVALID_ARG, "bad coarse direction mode");
    net->net.coarse_mode = mode;
  });
}

nw_status nw_linsys_attach_learned(nw_linsys* ls, nw_learned* net) {
  return guard([&] {
    need_finalized(ls);
    if (!net) fail(NW_INVALID_ARG, "null network");
    if (ls->num_dof != 1) fail(NW_INVALID_ARG, "the learned preconditioner needs num_dof 1");
    const double theta = net->net.agg_strength;
    if (!ls->coarse || ls->coarse->passes != net->net.agg_passes || ls->coarse->strength != theta ||
        theta > 0.0) {
      auto cl = std::make_unique<CoarseLevel>();
      if (theta > 0.0) {
        // the aggregation reads the assembled values
        materialize_zero(ls);
        if (int64_t(ls->values.n) != ls->g.nrow_ptr[ls->g.node_rows])
          fail(NW_INTERNAL, "node graph and values differ in size");
        std::vector<double> v(ls->values.n);
        NW_CUDA(cudaMemcpyAsync(v.data(), ls->values.p, v.size() * sizeof(double),
                                cudaMemcpyDeviceToHost, ls->stream));
        NW_CUDA(cudaStreamSynchronize(ls->stream));
        cl->setup(ls->g, net->net.agg_passes, ls->stream, v.data(), theta);
      } else {
        cl->setup(ls->g, net->net.agg_passes, ls->stream);
      }
      ls->coarse = std::move(cl);
    }
    ls->learned = net;
    ls->solver.attach_learned(&net->net, ls->coarse.get());
    NW_CUDA(cudaStreamSynchronize(ls->stream));
  });
}

nw_status nw_linsys_coarse_sizes(nw_linsys* ls, int64_t* nc, int64_t* nnzc) {
  return guard([&] {
    need_learned(ls);
    if (nc) *nc = ls->coarse->nc;
    if (nnzc) *nnzc = ls->coarse->nnzc;
  });
}

nw_status nw_linsys_coarse_graph(nw_linsys* ls, int32_t* agg, int64_t* cptr, int32_t* ccol,
                                 float* wgt, float* dinv) {
  return guard([&] {
    need_learned(ls);
    materialize_zero(ls);
    CoarseLevel& cl = *ls->coarse;
    cl.refresh(ls->values.p, ls->stream);
    if (agg) std::memcpy(agg, cl.agg_h.data(), sizeof(int32_t) * cl.nf);
    if (cptr) std::memcpy(cptr, cl.cptr_h.data(), sizeof(int64_t) * (cl.nc + 1));
    if (ccol) std::memcpy(ccol, cl.ccol_h.data(), sizeof(int32_t) * cl.nnzc);
    if (wgt) NW_CUDA(cudaMemcpyAsync(wgt, cl.wgt.p, sizeof(float) * cl.nnzc, cudaMemcpyDeviceToHost, ls->stream));
    if (dinv) NW_CUDA(cudaMemcpyAsync(dinv, cl.dinv.p, sizeof(float) * cl.nc, cudaMemcpyDeviceToHost, ls->stream));
    NW_CUDA(cudaStreamSynchronize(ls->stream));
  });
}

nw_status nw_learned_clear_data(nw_learned* net) {
  return guard([&] {
    if (!net) fail(NW_INVALID_ARG, "null network");
    net->net.clear_data();
  });
}

nw_status nw_learned_harvest(nw_learned* net, nw_linsys* ls, int restarts, int kspace,
                             int* total_pairs) {
  return guard([&] {
    need_finalized(ls);
    if (!net || restarts < 1 || kspace < 1) fail(NW_INVALID_ARG, "bad harvest arguments");
    if (ls->learned != net) {
      const nw_status st = nw_linsys_attach_learned(ls, net);
      if (st != NW_OK) fail(st, nw_last_error_string());
    }
    materialize_zero(ls);
    LearnedNet& L = net->net;
    CoarseLevel& cl = *ls->coarse;
    cudaStream_t s = ls->stream;
    const int64_t n = ls->g.nrows;
    if (L.npairs > 0 && (L.data_nc != cl.nc || L.data_nnzc != cl.nnzc))
      fail(NW_INVALID_ARG, "harvested pairs come from a different graph; clear them first");
    L.data_nc = cl.nc;
    L.data_nnzc = cl.nnzc;
    KrylovSolver& ks = ls->solver;
    ks.refresh(s);
    ks.ensure_f32(s);
    Precond pc = ls->pc;
    // x*: a tight (1e-11) reference solve. The pressure-Poisson matrix is
    // symmetric, and on strongly stretched meshes (cell growth 1.15 over
    // 127 cells is a 4e7 ratio of the first to the last z spacing)
    // restarted GMRES(50) + SGS stalls near 5e-3 where CG + (symmetric) SGS
    // reaches 2e-10 in ~15k iterations: CG + SGS in FP64 comes first (at
    // most 40,000 iterations); mixed and FP64 SGS-GMRES(50) follow only
    // when CG fails outright (above 1e-3, or non-finite: a matrix that is
    // not symmetric), and the best of the attempts is kept.
    DeviceArray<double> xs, x, d, r;
    xs.resize(n);
    x.resize(n);
    d.resize(n);
    r.resize(n);
    pc.kind = NW_PC_SGS;
    nw_solver_cfg tight = ls->cfg;
    tight.precision = NW_PREC_FP64;
    tight.method = NW_CG;
    tight.max_iterations = 40000;
    SolveResult sr = ks.solve(tight, 1e-11, pc, ls->rhs.p, xs.p, s);
    if (!(sr.final_abs <= 1e-3 * sr.bnorm)) {
      NW_CUDA(cudaMemcpyAsync(x.p, xs.p, n * 8, cudaMemcpyDeviceToDevice, s));  // CG's iterate
      const SolveResult cg_res = sr;
      tight.method = NW_GMRES;
      tight.precision = NW_PREC_MIXED;
      tight.kspace = std::min(50, std::max(ls->cfg.kspace, 30));
      tight.inner_kspace = tight.kspace;
      tight.inner_tolerance = 1e-4;
      tight.max_iterations = 5000;
      sr = ks.solve(tight, 1e-11, pc, ls->rhs.p, xs.p, s);
      if (!sr.converged) {
        // FP32 inner solves cannot refine a system this ill-conditioned
        tight.precision = NW_PREC_FP64;
        sr = ks.solve(tight, 1e-11, pc, ls->rhs.p, xs.p, s);
      }
      if (!(sr.final_abs <= cg_res.final_abs)) {
        sr = cg_res;
        NW_CUDA(cudaMemcpyAsync(xs.p, x.p, n * 8, cudaMemcpyDeviceToDevice, s));
      }
    }
    // The reference x* is kept at the residual r* it reached, and a pair
    // (r, e = x* - x) only while |r| >= 100 |r*|: A e = r - r*, so the
    // target error is then within 1 % of e.
    const double rstar = sr.final_abs;
    if (!(rstar <= 1e-6 * sr.bnorm))
      fail(NW_NOT_CONVERGED, "harvest: reference solve did not converge");
    // system coarse weights
    const int sys = L.nsystems++;
    auto* w = new DeviceArray<float>();
    auto* dv = new DeviceArray<float>();
    w->resize(cl.nnzc);
    dv->resize(cl.nc);
    NW_CUDA(cudaMemcpyAsync(w->p, cl.wgt.p, sizeof(float) * cl.nnzc, cudaMemcpyDeviceToDevice, s));
    NW_CUDA(cudaMemcpyAsync(dv->p, cl.dinv.p, sizeof(float) * cl.nc, cudaMemcpyDeviceToDevice, s));
    L.sys_wgt.push_back(w);
    L.sys_dinv.push_back(dv);
    // restarted Jacobi-GMRES(kspace), one pair per restart
    nw_solver_cfg cyc = ls->cfg;
    cyc.precision = NW_PREC_FP64;
    cyc.method = NW_GMRES;
    cyc.kspace = std::min(kspace, 1000);
    cyc.max_iterations = kspace;
    Precond jac = ls->pc;
    jac.kind = NW_PC_JACOBI;
    NW_CUDA(cudaMemsetAsync(x.p, 0, n * 8, s));
    NW_CUDA(cudaMemcpyAsync(r.p, ls->rhs.p, n * 8, cudaMemcpyDeviceToDevice, s));
    DeviceArray<float> r32, z1, e32;
    r32.resize(n);
    z1.resize(n);
    e32.resize(n);
    std::vector<double> hbuf(n);
    std::vector<float> h32(n), hz(n);
    for (int k = 0; k < restarts; ++k) {
      // pair: r, e = x* - x
      std::vector<double> hr(n), hx(n), hxs(n);
      NW_CUDA(cudaMemcpyAsync(hr.data(), r.p, n * 8, cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaMemcpyAsync(hx.data(), x.p, n * 8, cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaMemcpyAsync(hxs.data(), xs.p, n * 8, cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaStreamSynchronize(s));
      double rn = 0.0;
      for (int64_t i = 0; i < n; ++i) {
        h32[i] = float(hr[i]);
        rn += hr[i] * hr[i];
      }
      if (!(rn > 0.0) || std::sqrt(rn) < 100.0 * rstar) break;
      NW_CUDA(cudaMemcpyAsync(r32.p, h32.data(), n * 4, cudaMemcpyHostToDevice, s));
      // z1 = pre-smoothing sweep of r, r1 = r - A z1, rc = R r1
      ks.learned_presmooth32(r32.p, z1.p, s);
      auto* rc = new DeviceArray<float>();
      rc->resize(cl.nc);
      DeviceArray<float> az;
      az.resize(n);
      ks.spmv32(z1.p, az.p, s);
      NW_CUDA(cudaMemcpyAsync(hz.data(), z1.p, n * 4, cudaMemcpyDeviceToHost, s));
      std::vector<float> haz(n);
      NW_CUDA(cudaMemcpyAsync(haz.data(), az.p, n * 4, cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaStreamSynchronize(s));
      // e = x* - x; eA = e' A e = e' r; cA = (e - z1)' A (e - z1) = (e - z1)' r1
      std::vector<float> rcv(cl.nc, 0.f);
      std::vector<double> racc(cl.nc, 0.0);
      double ea = 0.0, ca = 0.0;
      for (int64_t i = 0; i < n; ++i) {
        const double e = hxs[i] - hx[i];
        const double r1 = double(h32[i]) - double(haz[i]);
        ea += e * hr[i];
        ca += (e - double(hz[i])) * r1;
        racc[cl.agg_h[i]] += r1;
      }
      for (int64_t I = 0; I < cl.nc; ++I) rcv[I] = float(racc[I]);
      NW_CUDA(cudaMemcpyAsync(rc->p, rcv.data(), cl.nc * 4, cudaMemcpyHostToDevice, s));
      NW_CUDA(cudaStreamSynchronize(s));
      if (ea > 0.0 && std::isfinite(ea) && std::isfinite(ca)) {
        L.pair_rc.push_back(rc);
        L.pair_system.push_back(sys);
        L.pair_ea.push_back(ea);
        L.pair_ca.push_back(std::max(ca, 0.0));
        L.npairs++;
      } else {
        delete rc;
      }
      // next restart: d = GMRES(kspace) on A d = r; x += d; r = b - A x
      ks.solve(cyc, 1e-300, jac, r.p, d.p, s);
      std::vector<double> hd(n);
      NW_CUDA(cudaMemcpyAsync(hd.data(), d.p, n * 8, cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaStreamSynchronize(s));
      for (int64_t i = 0; i < n; ++i) hx[i] += hd[i];
      NW_CUDA(cudaMemcpyAsync(x.p, hx.data(), n * 8, cudaMemcpyHostToDevice, s));
      ks.spmv64(x.p, ls->rhs.p, r.p, s);
    }
    NW_CUDA(cudaStreamSynchronize(s));
    if (total_pairs) *total_pairs = L.npairs;
  });
}

nw_status nw_learned_train(nw_learned* net, nw_linsys* ls, int epochs, int batch, double lr,
                           uint64_t shuffle_seed, double* loss) {
  return guard([&] {
    need_learned(ls);
    if (!net || epochs < 1 || batch < 1 || !(lr > 0)) fail(NW_INVALID_ARG, "bad training arguments");
    LearnedNet& L = net->net;
    CoarseLevel& cl = *ls->coarse;
    if (L.npairs == 0) fail(NW_INVALID_ARG, "no harvested pairs");
    if (L.data_nc != cl.nc || L.data_nnzc != cl.nnzc)
      fail(NW_INVALID_ARG, "pairs were harvested on a different graph");
    cudaStream_t s = ls->stream;
    std::vector<int> order(L.npairs);
    std::iota(order.begin(), order.end(), 0);
    uint64_t st = shuffle_seed * 0x9E3779B97F4A7C15ull + 7;
    double last = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
      for (int i = L.npairs - 1; i > 0; --i) {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        std::swap(order[i], order[int(st % uint64_t(i + 1))]);
      }
      double sum = 0.0;
      int inb = 0;
      for (int k = 0; k < L.npairs; ++k) {
        const int p = order[k];
        const int sys = L.pair_system[p];
        sum += L.forward_backward(cl, L.sys_wgt[sys]->p, L.sys_dinv[sys]->p, L.pair_rc[p]->p,
                                  L.pair_ea[p], L.pair_ca[p], s);
        if (++inb == batch || k + 1 == L.npairs) {
          L.adam(lr, 1.0 / inb, s);
          inb = 0;
        }
      }
      last = sum / L.npairs;
    }
    NW_CUDA(cudaStreamSynchronize(s));
    if (tc_status(s)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out during training");
    if (loss) *loss = last;
  });
}

nw_status nw_learned_evaluate(nw_learned* net, nw_linsys* ls, double* loss) {
  return guard([&] {
    need_learned(ls);
    if (!net || !loss) fail(NW_INVALID_ARG, "null argument");
    LearnedNet& L = net->net;
    CoarseLevel& cl = *ls->coarse;
    if (L.npairs == 0) fail(NW_INVALID_ARG, "no harvested pairs");
    if (L.data_nc != cl.nc || L.data_nnzc != cl.nnzc)
      fail(NW_INVALID_ARG, "pairs were harvested on a different graph");
    double sum = 0.0;
    for (int p = 0; p < L.npairs; ++p) {
      const int sys = L.pair_system[p];
      sum += L.forward_backward(cl, L.sys_wgt[sys]->p, L.sys_dinv[sys]->p, L.pair_rc[p]->p,
                                L.pair_ea[p], L.pair_ca[p], ls->stream, false);
    }
    if (tc_status(ls->stream)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out");
    *loss = sum / L.npairs;
  });
}

nw_status nw_learned_loss_grad(nw_learned* net, nw_linsys* ls, const float* rc, double ea,
                               double ca, double* loss, float* grad) {
  return guard([&] {
    need_learned(ls);
    if (!net || !rc || !(ea > 0)) fail(NW_INVALID_ARG, "bad arguments");
    materialize_zero(ls);
    LearnedNet& L = net->net;
    CoarseLevel& cl = *ls->coarse;
    cl.refresh(ls->values.p, ls->stream);
    NW_CUDA(cudaMemsetAsync(L.grads.p, 0, kNumParams * 4, ls->stream));
    const double l = L.forward_backward(cl, cl.wgt.p, cl.dinv.p, rc, ea, ca, ls->stream);
    if (loss) *loss = l;
    if (grad) {
      NW_CUDA(cudaMemcpyAsync(grad, L.grads.p, kNumParams * 4, cudaMemcpyDeviceToHost, ls->stream));
      NW_CUDA(cudaStreamSynchronize(ls->stream));
    }
    NW_CUDA(cudaMemsetAsync(L.grads.p, 0, kNumParams * 4, ls->stream));
    if (tc_status(ls->stream)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out");
  });
}

nw_status nw_learned_forward(nw_learned* net, nw_linsys* ls, const float* rc, float* ec) {
  return guard([&] {
    need_learned(ls);
    if (!net || !rc || !ec) fail(NW_INVALID_ARG, "null vector");
    materialize_zero(ls);
    CoarseLevel& cl = *ls->coarse;
    cl.refresh(ls->values.p, ls->stream);
    net->net.forward(cl, cl.wgt.p, cl.dinv.p, rc, ec, ls->stream);
    if (tc_status(ls->stream)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out");
  });
}

nw_status nw_gemm_bf16(int kind, int64_t m, const void* a, const void* b, void* out) {
  return guard([&] {
    if (!a || !b || !out || m < 0) fail(NW_INVALID_ARG, "bad GEMM arguments");
    const auto* ah = static_cast<const uint16_t*>(a);
    const auto* bh = static_cast<const uint16_t*>(b);
    if (kind == 0) {
      launch_gemm_fwd(ah, bh, static_cast<uint16_t*>(out), m, 64, nullptr);
    } else if (kind == 1) {
      launch_gemm_dx(ah, bh, static_cast<float*>(out), m, nullptr);
    } else if (kind == 3 || kind == 4) {
      if (kind == 3)
        launch_gemm_fwd_tc(ah, bh, static_cast<uint16_t*>(out), m, 64, nullptr);
      else
        launch_gemm_fwd_tma(ah, bh, static_cast<uint16_t*>(out), m, 64, nullptr);
      if (tc_status(nullptr)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out");
    } else if (kind == 2 || kind == 6) {
      DeviceArray<float> part;
      part.resize(size_t(4 * 152) * 128 * 64);
      NW_CUDA(cudaMemsetAsync(out, 0, 128 * 64 * 4, nullptr));
      if (kind == 2)
        launch_gemm_wgrad(ah, bh, part.p, static_cast<float*>(out), m, nullptr);
      else
        launch_gemm_wgrad_tc(ah, bh, part.p, static_cast<float*>(out), m, nullptr);
      NW_CUDA(cudaStreamSynchronize(nullptr));
      if (kind == 6 && tc_status(nullptr)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out");
    } else if (kind == 5) {
      launch_gemm_dx_tma(ah, bh, static_cast<float*>(out), m, nullptr);
      if (tc_status(nullptr)) fail(NW_TIMEOUT, "tensor-core GEMM wait timed out");
    } else {
      fail(NW_INVALID_ARG, "GEMM kind must be 0 to 6");
    }
    NW_CUDA(cudaGetLastError());
    NW_CUDA(cudaStreamSynchronize(nullptr));
  });
}

}  // extern "C"
