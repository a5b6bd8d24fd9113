// Launch wrappers of the edge-assembly kernels (assemble.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "nw_capi.h"

namespace nw {

using ScalarOpts = nw_scalar_opts;
using ContinuityOpts = nw_continuity_opts;
using MomentumOpts = nw_momentum_opts;

// 8-byte coefficient slots per edge written by the edge phase: scalar, six
// FP64 SoA arrays of E; continuity, one 16-byte record (f, tmdot as float
// pairs) per edge; momentum, 11 SoA arrays of E float pairs.
constexpr int kScalarCoefs = 6;
constexpr int kContinuityCoefs = 2;
constexpr int kMomentumCoefs = 11;

void launch_scalar_edges(cudaStream_t s, int64_t E, const int2* edges,
                         const nw_scalar_fields& f, const ScalarOpts& o,
                         double* buf);
void launch_continuity_edges(cudaStream_t s, int64_t E, const int2* edges,
                             const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf);
// With a node buffer (N x 8 doubles) the reference-default options take the
// node-phase + fast edge-phase route.
void launch_continuity_edges(cudaStream_t s, int64_t E, int64_t N,
                             const int2* edges, const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf,
                             double* nodebuf);
// The same over edges [e0, e1) of E (one 16-byte record per edge at its
// index), the node phase of the node-phase route over nodes [n0, n1) first
// (every node an edge of the range reads must have had its node phase).
void launch_continuity_edge_range(cudaStream_t s, int64_t n0, int64_t n1, int64_t e0, int64_t e1,
                                  const int2* edges, const nw_continuity_fields& f,
                                  const ContinuityOpts& o, double* buf, double* nodebuf);
constexpr int kContinuityNodeStride = 8;
// Edge phase of the momentum assembly over edges [e0, e1) of E (the
// coefficient buffer is laid out with stride E).
void launch_momentum_edges(cudaStream_t s, int64_t E, int64_t e0, int64_t e1, const int2* edges,
                           const nw_momentum_fields& f, const MomentumOpts& o,
                           double* buf);
// kind 0 scalar, 1 continuity, 2 momentum (3 dof), over node rows
// [row_begin, R) (row_begin > 0: momentum only). smem_bytes: staging size
// from row_stage_bytes (0 disables staging). max_inc: unused.
void launch_rows(cudaStream_t s, int kind, int64_t R, const int32_t* inc_ptr,
                 const uint32_t* inc, const int32_t* diag_pos,
                 const int64_t* row_ptr, const double* buf, int64_t E,
                 double relax, double* values, double* rhs, int accumulate,
                 int smem_bytes, int max_inc = 0, int64_t row_begin = 0);
// kind 3: the row blocks of the single-kernel momentum assembly.
int row_stage_bytes(int kind, const int64_t* row_ptr_host, int64_t R);

// Single-kernel momentum assembly (momentum_fused_k) over the work list of
// schedule.h. ring: the coefficient slots (stride `stride`, edge e in slot
// e & mask); eflag / rflag: one flag per edge chunk / row block, never
// reset (a launch waits for its own generation `gen`); ticket: the work
// counter (cleared by the launch); err: set to 1 when a wait timed out.
struct FusedLaunch {
  const int32_t* items = nullptr;
  const int32_t* in_ptr = nullptr;   // chunks each row block reads (CSR)
  const int32_t* in = nullptr;
  const int32_t* out_ptr = nullptr;  // row blocks reading each chunk (CSR)
  const int32_t* out = nullptr;
  int* eflag = nullptr;
  int* rflag = nullptr;
  int* ticket = nullptr;
  int* err = nullptr;
  double* ring = nullptr;
  int64_t nitems = 0, num_edges = 0, ring_chunks = 0, stride = 0, mask = -1;
  int gen = 0, grid = 0, smem_bytes = 0;
  int64_t R = 0;
  const int32_t* inc_ptr = nullptr;
  const uint32_t* inc = nullptr;
  const int32_t* diag_pos = nullptr;
  const int64_t* row_ptr = nullptr;
  double* values = nullptr;
  double* rhs = nullptr;
  int accumulate = 0;
};
// resident blocks of the kernel per SM with smem_bytes of row staging
int fused_blocks_per_sm(int smem_bytes);
void launch_momentum_fused(cudaStream_t s, const FusedLaunch& L, const int2* edges,
                           const nw_momentum_fields& f, const MomentumOpts& o);
void launch_reset_rows(cudaStream_t s, int64_t n, const int64_t* nodes,
                       const int64_t* node_lid, int num_dof, int begin,
                       int end, const int64_t* row_ptr, const int32_t* col_idx,
                       double* values, double* rhs, double diag_value,
                       double rhs_value, const double* q, const double* bc,
                       int64_t num_nodes, int* err);
void launch_sum_into_block(cudaStream_t s, int n_ent, int num_dof,
                           const int64_t* ent_lid, const double* lhs,
                           const double* rhs_in, const int64_t* row_ptr,
                           const int32_t* col_idx, double* values,
                           double* rhs);

}  // namespace nw
