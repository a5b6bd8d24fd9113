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
  int64_t nip = 0;  // face IPs
  int64_t nb = 0;
  const int32_t* brow = nullptr;  // nb node rows
  const int32_t* bptr = nullptr;  // nb + 1
  const int4* ips = nullptr;
  const int64_t* row_ptr = nullptr;
  const int32_t* diag_pos = nullptr;
  // the same IPs grouped by the node row of their opposing node L (for
  // kernels that add to L's rows): lips[p] = (ip index, R, L, unused)
  int64_t nl = 0;
  const int32_t* lrow = nullptr;
  const int32_t* lptr = nullptr;
  const int4* lips = nullptr;
};

void launch_continuity_open(cudaStream_t s, const SideView& v, const nw_continuity_open_fields& f,
                            const nw_continuity_open_opts& o, double* values, double* rhs);
void launch_momentum_open(cudaStream_t s, const SideView& v, const nw_momentum_open_fields& f,
                          const nw_momentum_open_opts& o, double* values, double* rhs);
void launch_momentum_symmetry(cudaStream_t s, const SideView& v, const nw_momentum_symmetry_fields& f,
                              const nw_momentum_symmetry_opts& o, double* values, double* rhs);
void launch_abl_wall(cudaStream_t s, const SideView& v, const nw_abl_wall_fields& f,
                     const nw_abl_wall_opts& o, double* values, double* rhs);
void launch_abl_shear(cudaStream_t s, const SideView& v, const double* area, const double* tau,
                      int slip, double* rhs);
void launch_scalar_open(cudaStream_t s, const SideView& v, const nw_scalar_open_fields& f, double relax,
                        double* values, double* rhs);

// MdotOpenEdgeAlg: per-IP open mass flow rate into mdot (num_ips), and
// its sum (fixed order) into *total_dev.
void launch_open_mdot(cudaStream_t s, const SideView& v, const nw_continuity_open_fields& f,
                      double noc_fac, double pstab_fac, double* mdot, double* total_dev);
// MdotOpenCorrectorAlg: mdot -= correction on every IP, then the sum.
void launch_correct_open_mdot(cudaStream_t s, const SideView& v, double correction, double* mdot,
                              double* total_dev);

}  // namespace nw
