// Continuity edge assembly that allocates no device memory per call.
//
// Some callers cannot call cudaMalloc at the point where they assemble: a
// host code whose device memory is owned by its own pool allocator (every
// byte accounted for up front), or a coupling layer that is only allowed to
// launch work on memory it was handed. nw_assemble_continuity_edges keeps its per-edge
// coefficients in a buffer the handle owns; this variant keeps them in a
// fixed array that lives in this file instead, and writes the assembled
// matrix into arrays the caller passes. It allocates nothing and calls no
// allocating library routine.
//
// The scratch array is a file-scope __device__ array: every GPU that loads
// the library holds it (8 MiB) until the process exits. The first call on a
// device looks up the array's device address (cudaGetSymbolAddress) with
// that device current and keeps it for the life of the process, so a
// cudaDeviceReset after that first call is not supported. The handle's
// device must be the current device when the entry point is called.
// This path always evaluates the general continuity edge kernel (it has no
// room for the node pre-pass buffer), so its result equals the regular
// entry point's within rounding, not bit for bit.
// All calls share the one array and it keeps the last call's contents;
// nothing in it needs to start at zero, because the edge kernel writes
// every entry the row kernel reads. Calls whose work overlaps on the GPU
// (different streams, or different handles on one device) race on the
// array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "assemble.h"
#include "nw_internal.h"

namespace {

// Two coefficients (lhsfac, tmdot) per edge.
constexpr int64_t kMaxEdges = int64_t(1) << 19;  // 524,288 edges
constexpr int kCoefs = nw::kContinuityCoefs;

static __device__ __align__(256) double g_noalloc_scratch[kCoefs * kMaxEdges];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (looked up once per
// device, with that device current).
double* scratch_on(int device) {
  if (device < 0 || device >= kMaxDevices)
    nw::fail(NW_INVALID_ARG, "device index out of range for the no-alloc path");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[device]) {
    int cur = -1;
    NW_CUDA(cudaGetDevice(&cur));
    if (cur != device) NW_CUDA(cudaSetDevice(device));
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess || !p)
      nw::fail(NW_CUDA_ERROR, std::string("cudaGetSymbolAddress(scratch): ") +
                                  cudaGetErrorString(e));
    g_scratch_ptr[device] = p;
  }
  return static_cast<double*>(g_scratch_ptr[device]);
}

}  // namespace

extern "C" nw_status nw_assemble_continuity_edges_noalloc(
    const nw_linsys* ls, const nw_continuity_fields* f,
    const nw_continuity_opts* o, double* values, double* rhs) {
  try {
    const nw::PlanView v = nw::plan_view(ls);
    if (v.num_dof != 1)
      nw::fail(NW_INVALID_ARG, "continuity assembly needs num_dof 1");
    if (!f || !o || !values || !rhs) nw::fail(NW_INVALID_ARG, "null argument");
    if (!f->coords || !f->velocity || !f->dpdx || !f->density || !f->pressure ||
        !f->udiag || !f->area)
      nw::fail(NW_INVALID_ARG, "null field pointer");
    if (!(o->tau_scale != 0.0)) nw::fail(NW_INVALID_ARG, "tau_scale is zero");
    if (v.num_edges > kMaxEdges)
      nw::fail(NW_INVALID_ARG,
               "mesh has " + std::to_string(v.num_edges) +
                   " edges; the no-allocation path holds at most " +
                   std::to_string(kMaxEdges) +
                   " (use nw_assemble_continuity_edges)");
    int cur = -1;
    NW_CUDA(cudaGetDevice(&cur));
    if (cur != v.device)
      nw::fail(NW_INVALID_ARG, "the handle's device (" + std::to_string(v.device) +
                                   ") is not the current device (" + std::to_string(cur) + ")");
    double* scratch = scratch_on(v.device);
    nw::launch_continuity_edges(v.stream, v.num_edges, v.edges, *f, *o, scratch);
    nw::launch_rows(v.stream, 1, v.node_rows, v.inc_ptr, v.inc, v.diag_pos,
                    v.row_ptr, scratch, v.num_edges, 1.0, values, rhs, 0, 0);
    NW_CUDA(cudaGetLastError());
    return NW_OK;
  } catch (const nw::Error& e) {
    nw::set_last_error(e.msg);
    return e.status;
  } catch (const std::exception& e) {
    nw::set_last_error(e.what());
    return NW_INTERNAL;
  }
}
