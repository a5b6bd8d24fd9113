// Internal types shared by the host C++ and the CUDA translation units of
// libnw_gb300.so. Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "nw_capi.h"

namespace nw {

// Thrown inside the library, converted to nw_status at the C ABI.
struct Error {
  nw_status status;
  std::string msg;
};
[[noreturn]] void fail(nw_status s, const std::string& msg);
void cuda_check(cudaError_t e, const char* what);
#define NW_CUDA(x) ::nw::cuda_check((x), #x)

template <typename T>
struct DeviceArray {
  T* p = nullptr;
  size_t n = 0;
  DeviceArray() = default;
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  ~DeviceArray() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void resize(size_t count) {
    if (count == n && p) return;
    release();
    if (count) NW_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    resize(h.size());
    if (n)
      NW_CUDA(cudaMemcpyAsync(p, h.data(), n * sizeof(T),
                              cudaMemcpyHostToDevice, s));
  }
};

// Host graph of a finalized linear system plus the deterministic assembly
// plan that replaces the reference's atomic CoeffApplier.
//
// Rows: master nodes sorted by id ("node rows"), expanded to num_dof CSR
// rows each. Assembly plan: every node row lists the (edge, side) pairs
// incident to it, sorted by column then by edge; bit 31 marks an entry whose
// column equals the previous entry's (periodic duplicates of one
// master-master pair).
struct HostGraph {
  int num_dof = 1;
  int64_t num_nodes = 0;  // caller's nodes (STK nodes incl. slaves)
  int64_t num_edges = 0;
  int64_t node_rows = 0;  // masters
  int64_t nrows = 0;      // node_rows * num_dof
  int64_t nnz = 0;
  std::vector<int64_t> node_lid;     // per node: first CSR row of its master
  std::vector<int64_t> row_ptr;      // nrows + 1
  std::vector<int32_t> col_idx;      // nnz
  std::vector<int64_t> nrow_ptr;     // node_rows + 1 (node-level graph)
  std::vector<int32_t> ncol;         // node-level columns (node rows)
  std::vector<int32_t> edges;        // E x 2 node indices (int32)
  std::vector<int32_t> inc_ptr;      // node_rows + 1 into inc
  std::vector<uint32_t> inc;         // packed (edge << 1 | side) | dup bit
  std::vector<int32_t> diag_pos;     // per node row: diagonal column slot
  std::vector<int32_t> row_master;   // per node row: caller node index
  std::vector<int64_t> row_gid;      // per node row: the master's (nalu) global id
};

// Build the Tpetra-identical CSR graph and the assembly plan.
void build_graph(HostGraph& g, int num_dof, int64_t num_nodes,
                 const int64_t* global_id, const int64_t* nalu_id,
                 int64_t num_edges, const int64_t* edge_nodes);

// Greedy colouring of the node-level graph (rows adjacent in the graph get
// different colours), used by the multicolour Gauss-Seidel.
int color_node_graph(const HostGraph& g, std::vector<int32_t>& color);

}  // namespace nw

namespace nw {
// Read-only view of a finalized handle's assembly plan (device pointers),
// for entry points that bring their own scratch and outputs.
struct PlanView {
  int device = 0;
  int num_dof = 1;
  cudaStream_t stream = nullptr;
  int64_t num_edges = 0;
  int64_t node_rows = 0;
  int64_t nrows = 0;
  int64_t nnz = 0;
  const int2* edges = nullptr;
  const int32_t* inc_ptr = nullptr;
  const uint32_t* inc = nullptr;
  const int32_t* diag_pos = nullptr;
  const int64_t* row_ptr = nullptr;
  int64_t num_nodes = 0;
  const int64_t* row_nodes_ptr = nullptr;  // node row -> its nodes (master first)
  const int32_t* row_nodes = nullptr;
  const int64_t* node_lid = nullptr;       // per node: first CSR row of its master
};
// Throws Error unless the handle is finalized.
PlanView plan_view(const nw_linsys* ls);
[[noreturn]] void fail(nw_status s, const std::string& msg);
void set_last_error(const std::string& s);
}  // namespace nw
