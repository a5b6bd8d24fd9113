// Launchers of the boundary face-IP kernels (boundary.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "nw_capi.h"

namespace nw {

// A registered side set on the device: its boundary node rows, each with a
// range of face IPs sorted by IP index. ips[p] = (ip index, face node R,
// opposing node L, column slot of L's row in the node row's column list).
struct SideView {
  int64_t nb = 0;
  const int32_t* brow = nullptr;  // nb node rows
  const int32_t* bptr = nullptr;  // nb + 1
  const int4* ips = nullptr;
  const int64_t* row_ptr = nullptr;
  const int32_t* diag_pos = nullptr;
};

void launch_continuity_open(cudaStream_t s, const SideView& v, const nw_continuity_open_fields& f,
                            const nw_continuity_open_opts& o, double* values, double* rhs);
void launch_momentum_open(cudaStream_t s, const SideView& v, const nw_momentum_open_fields& f,
                          const nw_momentum_open_opts& o, double* values, double* rhs);
void launch_momentum_symmetry(cudaStream_t s, const SideView& v, const nw_momentum_symmetry_fields& f,
                              const nw_momentum_symmetry_opts& o, double* values, double* rhs);
void launch_scalar_open(cudaStream_t s, const SideView& v, const nw_scalar_open_fields& f, double relax,
                        double* values, double* rhs);

}  // namespace nw
