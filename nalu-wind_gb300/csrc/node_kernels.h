// Launchers of the node kernels (node_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "nw_capi.h"
#include "nw_internal.h"

namespace nw {

// kind 0 scalar, 1 continuity, 2 momentum (3 dof): adds the lumped-mass BDF
// terms to each node row's diagonal entry and rhs.
void launch_mass_bdf(cudaStream_t s, int kind, const PlanView& v, const nw_mass_bdf_fields& f,
                     const nw_bdf_opts& o, double* values, double* rhs);

// diag[n] = the assembled diagonal entry of dof `dof` of node n's row (its
// master's), 0 where the row has no diagonal entry.
void launch_extract_diagonal(cudaStream_t s, const PlanView& v, int dof, const double* values,
                             double* diag);
// udiag = (udiag / (rho V) - pts) alpha + pts
void launch_udiag_postprocess(cudaStream_t s, int64_t n, const double* rho, const double* dvol,
                              double pts, double alpha, double* udiag);

}  // namespace nw
