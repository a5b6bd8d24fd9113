// Node kernels of the momentum / continuity / scalar systems: the
// lumped-mass BDF time terms, added to each node row's diagonal and rhs.
// One thread per node row sums the row's nodes (a periodic master and its
// slaves, master first) in FP64 and adds once: no atomics.
#include <cuda_runtime.h>

#include <cstdint>

#include "node_kernels.h"
#include "nw_internal.h"

namespace nw {
namespace {

constexpr int kThreads = 256;

// KIND 0: ScalarMassBDFNodeKernel::execute
//         (src/node_kernels/ScalarMassBDFNodeKernel.C:75-97)
// KIND 1: ContinuityMassBDFNodeKernel::execute
//         (src/node_kernels/ContinuityMassBDFNodeKernel.C:60-82)
// KIND 2: MomentumMassBDFNodeKernel::execute
//         (src/node_kernels/MomentumMassBDFNodeKernel.C:78-107)
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    mass_bdf_k(int64_t R, const int64_t* __restrict__ rn_ptr, const int32_t* __restrict__ rn,
               const int32_t* __restrict__ diag_pos, const int64_t* __restrict__ row_ptr,
               nw_mass_bdf_fields f, nw_bdf_opts o, double* __restrict__ values,
               double* __restrict__ rhs) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= R) return;
  constexpr int ND = KIND == 2 ? 3 : 1;
  const double dt = o.dt, g1 = o.gamma1, g2 = o.gamma2, g3 = o.gamma3;
  double lhs = 0.0, b[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) b[d] = 0.0;
  for (int64_t k = rn_ptr[r]; k < rn_ptr[r + 1]; ++k) {
    const int64_t i = rn[k];
    const double rNm1 = f.density_nm1[i], rN = f.density_n[i], rNp1 = f.density_np1[i];
    const double vNm1 = f.dual_volume_nm1[i], vN = f.dual_volume_n[i], vNp1 = f.dual_volume_np1[i];
    if (KIND == 0) {
      lhs += g1 * rNp1 * vNp1 / dt;
      b[0] += -(g1 * rNp1 * f.q_np1[i] * vNp1 + g2 * f.q_n[i] * rN * vN +
                g3 * f.q_nm1[i] * rNm1 * vNm1) /
              dt;
    } else if (KIND == 1) {
      b[0] += -(g1 * rNp1 * vNp1 + g2 * rN * vN + g3 * rNm1 * vNm1) / dt * (g1 / dt);
    } else {
      lhs += g1 * rNp1 * vNp1 / dt;
#pragma unroll
      for (int d = 0; d < 3; ++d)
        b[d] += -(g1 * rNp1 * f.q_np1[3 * i + d] * vNp1 + g2 * rN * f.q_n[3 * i + d] * vN +
                  g3 * rNm1 * f.q_nm1[3 * i + d] * vNm1) /
                    dt -
                f.dpdx[3 * i + d] * vNp1;
    }
  }
  const int dp = diag_pos[r];
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const int64_t row = ND * r + d;
    if (KIND != 1 && dp >= 0) values[row_ptr[row] + int64_t(ND) * dp + d] += lhs;
    rhs[row] += b[d];
  }
}

// NGPApplyCoeff::extract_diagonal (src/SolverAlgorithm.C:89-104) adds
// lhs(ix, ix), the first dof's diagonal of each entity's block, of every
// local system into momentum_diag as the systems are summed in. The
// assembled CSR diagonal of that dof holds exactly the sum of those terms
// (of every kernel assembled so far), so it is read back once per node:
// call after the assembly and before Dirichlet rows are applied.
__global__ void extract_diag_k(int64_t N, const int64_t* __restrict__ node_lid, int nd, int dof,
                               const int32_t* __restrict__ diag_pos,
                               const int64_t* __restrict__ row_ptr,
                               const double* __restrict__ values, double* __restrict__ out) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t row0 = node_lid[n];
  const int dp = diag_pos[row0 / nd];
  out[n] = dp >= 0 ? values[row_ptr[row0 + dof] + int64_t(nd) * dp + dof] : 0.0;
}

// MomentumEquationSystem::assemble_and_solve post-processing of the
// extracted diagonal (src/LowMachEquationSystem.C:2760-2790): divide by
// rho V, then remove the momentum relaxation factor about gamma1 / dt.
__global__ void udiag_post_k(int64_t n, const double* __restrict__ rho,
                             const double* __restrict__ dvol, double pts, double alpha,
                             double* __restrict__ udiag) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double u = udiag[i] / (rho[i] * dvol[i]);
  udiag[i] = (u - pts) * alpha + pts;
}

inline unsigned grid_for(int64_t n) { return unsigned((n + kThreads - 1) / kThreads); }

}  // namespace

void launch_extract_diagonal(cudaStream_t s, const PlanView& v, int dof, const double* values,
                             double* diag) {
  if (v.num_nodes == 0) return;
  extract_diag_k<<<grid_for(v.num_nodes), kThreads, 0, s>>>(v.num_nodes, v.node_lid, v.num_dof, dof,
                                                             v.diag_pos, v.row_ptr, values, diag);
  NW_CUDA(cudaGetLastError());
}

void launch_udiag_postprocess(cudaStream_t s, int64_t n, const double* rho, const double* dvol,
                              double pts, double alpha, double* udiag) {
  if (n == 0) return;
  udiag_post_k<<<grid_for(n), kThreads, 0, s>>>(n, rho, dvol, pts, alpha, udiag);
  NW_CUDA(cudaGetLastError());
}

void launch_mass_bdf(cudaStream_t s, int kind, const PlanView& v, const nw_mass_bdf_fields& f,
                     const nw_bdf_opts& o, double* values, double* rhs) {
  if (v.node_rows == 0) return;
  if (kind == 0)
    mass_bdf_k<0><<<grid_for(v.node_rows), kThreads, 0, s>>>(
        v.node_rows, v.row_nodes_ptr, v.row_nodes, v.diag_pos, v.row_ptr, f, o, values, rhs);
  else if (kind == 1)
    mass_bdf_k<1><<<grid_for(v.node_rows), kThreads, 0, s>>>(
        v.node_rows, v.row_nodes_ptr, v.row_nodes, v.diag_pos, v.row_ptr, f, o, values, rhs);
  else
    mass_bdf_k<2><<<grid_for(v.node_rows), kThreads, 0, s>>>(
        v.node_rows, v.row_nodes_ptr, v.row_nodes, v.diag_pos, v.row_ptr, f, o, values, rhs);
  NW_CUDA(cudaGetLastError());
}

}  // namespace nw
