// Boundary face-IP kernels of the edge-based open and symmetry conditions.
//
// One thread per boundary node row walks the row's face IPs in IP order and
// adds each IP's contributions (rows of the face node R, columns R and the
// opposing node L) straight into the CSR values and rhs: a row belongs to
// one thread, so there are no atomics and the sums are deterministic. The
// boundary holds O(N^(2/3)) IPs, so these kernels compute in FP64 directly;
// their cost is negligible beside the interior assembly.
#include <cuda_runtime.h>

#include <cstdint>

#include "boundary.h"
#include "nw_internal.h"

namespace nw {
namespace {

constexpr int kThreads = 128;

struct FaceGeom {
  double av[3], asq, axdx, inv_axdx;
};

// duidxj with Jasak's over-relaxed non-orthogonal correction and the viscous
// face flux fx, fx . n (MomentumOpenEdgeKernel.C:137-177,
// MomentumSymmetryEdgeKernel.C:112-152).
__device__ void face_flux(const double* __restrict__ coords, const double* __restrict__ vel,
                          const double* __restrict__ dudx, int R, int L, const FaceGeom& g,
                          double visc, const double nx[3], double include_div_u, double fx[3],
                          double& fxnx) {
  double du[3][3];
  double dx[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) dx[j] = coords[3 * R + j] - coords[3 * L + j];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double dui = vel[3 * R + i] - vel[3 * L + i];
    double gjuidx = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) gjuidx += dudx[9 * R + 3 * i + j] * dx[j];
#pragma unroll
    for (int j = 0; j < 3; ++j)
      du[i][j] = dudx[9 * R + 3 * i + j] + (dui - gjuidx) * g.av[j] * g.inv_axdx;
  }
  const double divU = du[0][0] + du[1][1] + du[2][2];
  fxnx = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double f = 2.0 / 3.0 * visc * divU * g.av[i] * include_div_u;
#pragma unroll
    for (int j = 0; j < 3; ++j) f += -visc * (du[i][j] + du[j][i]) * g.av[j];
    fx[i] = f;
    fxnx += nx[i] * f;
  }
}

// |A|^2 and A . (x_R - x_L)
__device__ FaceGeom geom(const double* __restrict__ coords, const double* __restrict__ area, int ip,
                         int R, int L) {
  FaceGeom g;
  g.asq = 0.0;
  g.axdx = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    g.av[d] = area[3 * ip + d];
    g.asq += g.av[d] * g.av[d];
    g.axdx += g.av[d] * (coords[3 * R + d] - coords[3 * L + d]);
  }
  g.inv_axdx = 1.0 / g.axdx;
  return g;
}

// ContinuityOpenEdgeKernel::execute (src/edge_kernels/
// ContinuityOpenEdgeKernel.C:92-160)
__global__ void __launch_bounds__(kThreads)
    continuity_open_k(SideView v, nw_continuity_open_fields f, nw_continuity_open_opts o,
                      double* __restrict__ values, double* __restrict__ rhs) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= v.nb) return;
  const int row = v.brow[b];
  const int64_t base = v.row_ptr[row];
  const int dp = v.diag_pos[row];
  for (int p = v.bptr[b]; p < v.bptr[b + 1]; ++p) {
    const int4 q = v.ips[p];
    const int ip = q.x, R = q.y, L = q.z;
    const double pts = 1.0 / f.udiag[R];
    const double pIp = 0.5 * (f.pressure[R] + f.pressure[L]);
    // the distance runs from R to the edge midpoint here (coordIp)
    double asq = 0.0, axdx = 0.0, av[3], dxj[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      av[d] = f.exposed_area[3 * ip + d];
      dxj[d] = f.coords[3 * R + d] - 0.5 * (f.coords[3 * R + d] + f.coords[3 * L + d]);
      asq += av[d] * av[d];
      axdx += av[d] * dxj[d];
    }
    const double inv_axdx = 1.0 / axdx;
    const double pbc = f.pressure_bc[R] - (f.dynamic_pressure ? f.dynamic_pressure[ip] : 0.0);
    double tmdot = -pts * (pbc - pIp) * asq * inv_axdx * o.pstab_fac - o.mdot_corr;
    const double rho_w = o.solve_incompressible + f.density[R] * (1.0 - o.solve_incompressible);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double kxj = av[d] - asq * inv_axdx * dxj[d];
      const double G = f.dpdx[3 * R + d];
      tmdot += (rho_w * f.velocity[3 * R + d] + pts * G * o.pstab_fac) * av[d] -
               pts * kxj * G * o.noc_fac * o.pstab_fac;
    }
    const double lhsfac = 0.5 * asq * inv_axdx * o.pstab_fac * pts / o.tau_scale;
    rhs[row] -= tmdot / o.tau_scale;
    values[base + dp] += lhsfac;
    values[base + q.w] += lhsfac;
  }
}

// Adds one IP's 3 x 6 block (rows of R; columns R then L) to the node row.
__device__ void add_block(double* __restrict__ values, double* __restrict__ rhs,
                          const int64_t* __restrict__ row_ptr, int row, int dp, int kL,
                          const double A[3][6], const double bR[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int64_t base = row_ptr[3 * row + i];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      values[base + 3 * dp + j] += A[i][j];
      values[base + 3 * kL + j] += A[i][3 + j];
    }
    rhs[3 * row + i] += bR[i];
  }
}

// MomentumOpenEdgeKernel::execute (src/edge_kernels/
// MomentumOpenEdgeKernel.C:80-270)
__global__ void __launch_bounds__(kThreads)
    momentum_open_k(SideView v, nw_momentum_open_fields f, nw_momentum_open_opts o,
                    double* __restrict__ values, double* __restrict__ rhs) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= v.nb) return;
  const int row = v.brow[b];
  const int dp = v.diag_pos[row];
  const double nf = o.nf_entrain, om_nf = 1.0 - nf;
  for (int p = v.bptr[b]; p < v.bptr[b + 1]; ++p) {
    const int4 q = v.ips[p];
    const int ip = q.x, R = q.y, L = q.z;
    const FaceGeom g = geom(f.coords, f.exposed_area, ip, R, L);
    const double visc = f.viscosity[R];
    const double amag = sqrt(g.asq);
    double nx[3], uxnx = 0.0, uxnxip = 0.0, uspecxnx = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      nx[d] = g.av[d] / amag;
      uxnx += nx[d] * f.velocity[3 * R + d];
      uxnxip += 0.5 * nx[d] * (f.velocity[3 * L + d] + f.velocity[3 * R + d]);
      uspecxnx += nx[d] * f.velocity_bc[3 * R + d];
    }
    double fx[3], fxnx;
    face_flux(f.coords, f.velocity, f.dudx, R, L, g, visc, nx, o.include_div_u, fx, fxnx);
    double A[3][6], bR[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 6; ++j) A[i][j] = 0.0;
      bR[i] = -(fx[i] - nx[i] * fxnx);
    }
    const double vai = visc * g.inv_axdx;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double om = 1.0 - nx[i] * nx[i];
      double fac = -visc * g.asq * g.inv_axdx * om;
      A[i][3 + i] -= fac;
      A[i][i] += fac;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        fac = -visc * g.av[i] * g.av[j] * g.inv_axdx * om;
        A[i][3 + j] -= fac;
        A[i][j] += fac;
        if (i == j) continue;
        const double nn = nx[i] * nx[j];
        fac = vai * g.asq * nn;
        A[i][3 + j] -= fac;
        A[i][j] += fac;
        fac = visc * g.av[j] * g.av[j] * g.inv_axdx * nn;
        A[i][3 + j] -= fac;
        A[i][j] += fac;
        fac = visc * g.av[j] * g.av[i] * g.inv_axdx * nn;
        A[i][3 + i] -= fac;
        A[i][i] += fac;
      }
    }
    const double tmdot = f.open_mass_flow_rate[ip];
    if (o.entrainment == NW_ENTRAIN_SPECIFIED) {
      const double sigma = visc * g.asq * g.inv_axdx;
      const double lambda = 0.5 * (tmdot - sqrt(tmdot * tmdot + 8.0 * sigma * sigma));
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const double uR = f.velocity[3 * R + i];
        if (tmdot > 0.0) {
          bR[i] -= tmdot * uR;
          A[i][i] += tmdot;
        } else {
          bR[i] -= tmdot * uR - lambda * (uR - f.velocity_bc[3 * R + i]);
          A[i][i] += tmdot - lambda;
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if (tmdot > 0.0) {
          bR[i] -= tmdot * f.velocity[3 * R + i];
          A[i][i] += tmdot;
        } else {
          bR[i] -= tmdot * ((nf * uxnx + om_nf * uxnxip) * nx[i] +
                            (f.velocity_bc[3 * R + i] - uspecxnx * nx[i]));
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            A[i][3 + j] += tmdot * om_nf * 0.5 * nx[i] * nx[j];
            A[i][j] += tmdot * (nf + om_nf * 0.5) * nx[i] * nx[j];
          }
        }
      }
    }
    add_block(values, rhs, v.row_ptr, row, dp, q.w, A, bR);
  }
}

// MomentumSymmetryEdgeKernel::execute (src/edge_kernels/
// MomentumSymmetryEdgeKernel.C:64-206)
__global__ void __launch_bounds__(kThreads)
    momentum_symmetry_k(SideView v, nw_momentum_symmetry_fields f, nw_momentum_symmetry_opts o,
                        double* __restrict__ values, double* __restrict__ rhs) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= v.nb) return;
  const int row = v.brow[b];
  const int dp = v.diag_pos[row];
  for (int p = v.bptr[b]; p < v.bptr[b + 1]; ++p) {
    const int4 q = v.ips[p];
    const int ip = q.x, R = q.y, L = q.z;
    const FaceGeom g = geom(f.coords, f.exposed_area, ip, R, L);
    const double visc = f.viscosity[R];
    const double amag = sqrt(g.asq);
    double nx[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) nx[d] = g.av[d] / amag;
    double fx[3], fxnx;
    face_flux(f.coords, f.velocity, f.dudx, R, L, g, visc, nx, o.include_div_u, fx, fxnx);
    const double dmr = -visc * g.asq * g.inv_axdx;
    const double pen = o.penalty_factor * dmr;
    double uN = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) uN += f.velocity[3 * R + i] * nx[i];
    double A[3][6], bR[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        A[i][j] = -pen * nx[i] * nx[j];
        A[i][3 + j] = 0.0;
      }
      bR[i] = pen * uN * nx[i] - fxnx * nx[i];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double fac = dmr * nx[i] * nx[i];
      A[i][3 + i] -= fac;
      A[i][i] += fac;
      const double nxnx = nx[i] * nx[i];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        fac = -visc * g.av[i] * g.av[j] * g.inv_axdx * nxnx;
        A[i][3 + j] -= fac;
        A[i][j] += fac;
        if (i == j) continue;
        fac = -visc * g.asq * g.inv_axdx * nx[i] * nx[j];
        A[i][3 + j] -= fac;
        A[i][j] += fac;
        // the reference carries no 1/axdx in these two terms
        fac = -visc * g.av[j] * g.av[j] * nx[i] * nx[j];
        A[i][3 + j] -= fac;
        A[i][j] += fac;
        fac = -visc * g.av[j] * g.av[i] * nx[i] * nx[j];
        A[i][3 + i] -= fac;
        A[i][i] += fac;
      }
    }
    add_block(values, rhs, v.row_ptr, row, dp, q.w, A, bR);
  }
}

// Monin-Obukhov stability function for momentum (include/wind_energy/
// MoninObukhov.h:26-55, van der Laan et al. 2017), by stratification.
__device__ double abl_psim(double Tflux, double zeta, double beta_m, double gamma_m) {
  const double eps = 1.0e-8;
  if (Tflux < -eps) return -beta_m * zeta;  // stable
  if (Tflux > eps) {                        // unstable
    const double half_pi = 1.5707963267948966;
    const double phim = pow(1.0 - gamma_m * zeta, 0.25);
    const double t2 = 1.0 + phim;
    return log(0.125 * (1.0 + phim * phim) * (t2 * t2)) - 2.0 * atan(phim) + half_pi;
  }
  return 0.0;  // neutral
}

// MomentumABLWallFuncEdgeKernel::execute (src/edge_kernels/
// MomentumABLWallFuncEdgeKernel.C:80-158)
__global__ void __launch_bounds__(kThreads)
    abl_wall_k(SideView v, nw_abl_wall_fields f, nw_abl_wall_opts o, double* __restrict__ values,
               double* __restrict__ rhs) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= v.nb) return;
  const int row = v.brow[b];
  const int dp = v.diag_pos[row];
  const double eps = 1.0e-8, Lmax = 1.0e8;
  for (int p = v.bptr[b]; p < v.bptr[b + 1]; ++p) {
    const int4 q = v.ips[p];
    const int ip = q.x, R = q.y;
    double av[3], nx[3], amag = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      av[d] = f.exposed_area[3 * ip + d];
      amag += av[d] * av[d];
    }
    amag = sqrt(amag);
#pragma unroll
    for (int d = 0; d < 3; ++d) nx[d] = av[d] / amag;
    const double zh = f.wall_normal_distance[ip], ustar = f.wall_friction_velocity[ip];
    const double rho = f.density[R];
    const double Tflux = f.heat_flux_bc[R] / (rho * f.specific_heat[R]);
    const double Lfac = fabs(Tflux) < eps ? Lmax : (-o.Tref / (o.kappa * o.gravity * Tflux));
    double moLen = ustar * ustar * ustar * Lfac;
    moLen = (Tflux < 0.0 ? 1.0 : -1.0) * fmax(1.0e-10, fabs(moLen));
    const double psim = abl_psim(Tflux, zh / moLen, o.beta_m, o.gamma_m);
    const double lambda = (rho * o.kappa * ustar / (log(zh / o.z0) - psim)) * amag;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int64_t base = v.row_ptr[3 * row + i] + 3 * int64_t(dp);
      double uTan = 0.0, uBcTan = 0.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double ninj = nx[i] * nx[j];
        if (i == j) {
          const double om = 1.0 - ninj;
          uTan += om * f.velocity[3 * R + j];
          uBcTan += om * f.wall_velocity_bc[3 * R + j];
          values[base + j] += lambda * om;
        } else {
          uTan -= ninj * f.velocity[3 * R + j];
          uBcTan -= ninj * f.wall_velocity_bc[3 * R + j];
          values[base + j] -= lambda * ninj;
        }
      }
      rhs[3 * row + i] -= lambda * (uTan - uBcTan);
    }
  }
}

// MomentumABLWallShearStressEdgeKernel::execute (src/edge_kernels/
// MomentumABLWallShearStressEdgeKernel.C:49-88): rhs += tau_w |A| on the
// face node's rows (slip) or the opposing node's rows (no slip); one thread
// per receiving node row.
__global__ void __launch_bounds__(kThreads)
    abl_shear_k(int64_t nrows, const int32_t* __restrict__ rows, const int32_t* __restrict__ ptr,
                const int4* __restrict__ ips, const double* __restrict__ area,
                const double* __restrict__ tau, double* __restrict__ rhs) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= nrows) return;
  const int row = rows[b];
  for (int p = ptr[b]; p < ptr[b + 1]; ++p) {
    const int ip = ips[p].x;
    const double a0 = area[3 * ip], a1 = area[3 * ip + 1], a2 = area[3 * ip + 2];
    const double amag = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
#pragma unroll
    for (int i = 0; i < 3; ++i) rhs[3 * row + i] += tau[3 * ip + i] * amag;
  }
}

// ScalarOpenEdgeKernel::execute (src/edge_kernels/ScalarOpenEdgeKernel.C:
// 49-72)
__global__ void __launch_bounds__(kThreads)
    scalar_open_k(SideView v, nw_scalar_open_fields f, double relax, double* __restrict__ values,
                  double* __restrict__ rhs) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= v.nb) return;
  const int row = v.brow[b];
  const int64_t diag = v.row_ptr[row] + v.diag_pos[row];
  for (int p = v.bptr[b]; p < v.bptr[b + 1]; ++p) {
    const int4 q = v.ips[p];
    const double md = f.open_mass_flow_rate[q.x];
    const double up = md > 0.0 ? f.q[q.y] : f.q_bc[q.y];
    rhs[row] -= md * up;
    if (md > 0.0) values[diag] += md / relax;
  }
}

// MdotOpenEdgeAlg::execute (src/ngp_algorithms/MdotOpenEdgeAlg.C:55-150):
// one thread per face IP (in row-sorted position; writes at its IP index).
__global__ void __launch_bounds__(kThreads)
    open_mdot_k(SideView v, nw_continuity_open_fields f, double noc_fac, double pstab_fac,
                double* __restrict__ mdot) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= v.nip) return;
  const int4 q = v.ips[p];
  const int ip = q.x, R = q.y, L = q.z;
  const double pts = pstab_fac / f.udiag[R];
  double asq = 0.0, axdx = 0.0, av[3], dxj[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    av[d] = f.exposed_area[3 * ip + d];
    dxj[d] = f.coords[3 * R + d] - 0.5 * (f.coords[3 * R + d] + f.coords[3 * L + d]);
    asq += av[d] * av[d];
    axdx += av[d] * dxj[d];
  }
  const double inv_axdx = 1.0 / axdx;
  const double pbc = f.pressure_bc[R] - (f.dynamic_pressure ? f.dynamic_pressure[ip] : 0.0);
  const double pIp = 0.5 * (f.pressure[L] + f.pressure[R]);
  double tmdot = -pts * (pbc - pIp) * asq * inv_axdx;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double kxj = av[d] - asq * inv_axdx * dxj[d];
    const double G = f.dpdx[3 * R + d];
    tmdot += (f.density[R] * f.velocity[3 * R + d] + pts * G) * av[d] - pts * kxj * G * noc_fac;
  }
  mdot[ip] = tmdot;
}

// MdotOpenCorrectorAlg::execute (src/ngp_algorithms/MdotOpenCorrectorAlg.C:
// 37-60): the same correction off every open IP.
__global__ void correct_k(int64_t n, double corr, double* __restrict__ mdot) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) mdot[i] -= corr;
}

// Sum of mdot[0..n) by one block in a fixed order (deterministic).
__global__ void __launch_bounds__(256) sum_k(int64_t n, const double* __restrict__ a,
                                             double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += a[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

unsigned blocks(int64_t n) { return unsigned((n + kThreads - 1) / kThreads); }

}  // namespace

void launch_open_mdot(cudaStream_t s, const SideView& v, const nw_continuity_open_fields& f,
                      double noc_fac, double pstab_fac, double* mdot, double* total_dev) {
  if (v.nip > 0) open_mdot_k<<<blocks(v.nip), kThreads, 0, s>>>(v, f, noc_fac, pstab_fac, mdot);
  sum_k<<<1, 256, 0, s>>>(v.nip, mdot, total_dev);
  NW_CUDA(cudaGetLastError());
}
void launch_correct_open_mdot(cudaStream_t s, const SideView& v, double correction, double* mdot,
                              double* total_dev) {
  if (v.nip > 0) correct_k<<<blocks(v.nip), kThreads, 0, s>>>(v.nip, correction, mdot);
  sum_k<<<1, 256, 0, s>>>(v.nip, mdot, total_dev);
  NW_CUDA(cudaGetLastError());
}

void launch_continuity_open(cudaStream_t s, const SideView& v, const nw_continuity_open_fields& f,
                            const nw_continuity_open_opts& o, double* values, double* rhs) {
  if (v.nb == 0) return;
  continuity_open_k<<<blocks(v.nb), kThreads, 0, s>>>(v, f, o, values, rhs);
  NW_CUDA(cudaGetLastError());
}
void launch_momentum_open(cudaStream_t s, const SideView& v, const nw_momentum_open_fields& f,
                          const nw_momentum_open_opts& o, double* values, double* rhs) {
  if (v.nb == 0) return;
  momentum_open_k<<<blocks(v.nb), kThreads, 0, s>>>(v, f, o, values, rhs);
  NW_CUDA(cudaGetLastError());
}
void launch_momentum_symmetry(cudaStream_t s, const SideView& v, const nw_momentum_symmetry_fields& f,
                              const nw_momentum_symmetry_opts& o, double* values, double* rhs) {
  if (v.nb == 0) return;
  momentum_symmetry_k<<<blocks(v.nb), kThreads, 0, s>>>(v, f, o, values, rhs);
  NW_CUDA(cudaGetLastError());
}
void launch_abl_wall(cudaStream_t s, const SideView& v, const nw_abl_wall_fields& f,
                     const nw_abl_wall_opts& o, double* values, double* rhs) {
  if (v.nb == 0) return;
  abl_wall_k<<<blocks(v.nb), kThreads, 0, s>>>(v, f, o, values, rhs);
  NW_CUDA(cudaGetLastError());
}
void launch_abl_shear(cudaStream_t s, const SideView& v, const double* area, const double* tau,
                      int slip, double* rhs) {
  const int64_t n = slip ? v.nb : v.nl;
  if (n == 0) return;
  abl_shear_k<<<blocks(n), kThreads, 0, s>>>(n, slip ? v.brow : v.lrow, slip ? v.bptr : v.lptr,
                                             slip ? v.ips : v.lips, area, tau, rhs);
  NW_CUDA(cudaGetLastError());
}
void launch_scalar_open(cudaStream_t s, const SideView& v, const nw_scalar_open_fields& f, double relax,
                        double* values, double* rhs) {
  if (v.nb == 0) return;
  scalar_open_k<<<blocks(v.nb), kThreads, 0, s>>>(v, f, relax, values, rhs);
  NW_CUDA(cudaGetLastError());
}

}  // namespace nw
