// Edge assembly kernels for sm_103a.
//
// The reference computes each edge's local system in a Kokkos team lambda
// (include/AssembleEdgeSolverAlgorithm.h:47-100) and scatters it with FP64
// atomics (TpetraLinearSystem::sum_into, src/TpetraLinearSystem.C:
// 1381-1459), so its summation order is not reproducible on a GPU. Here
// assembly has deterministic phases and no floating-point atomics:
//
//  0. (continuity) node phase: one thread per node computes the node-only
//     factors every incident edge needs (1/udiag, rho u, grad p / udiag);
//  1. edge phase: one thread per edge evaluates the edge physics once and
//     writes its compact coefficients to an edge-major buffer (SoA);
//  2. row phase: one thread per node row walks the row's incident
//     (edge, side) list, sorted by column then edge, accumulates the
//     diagonal block and rhs in registers, stages the row's CSR values in
//     shared memory and the block writes its contiguous CSR range with
//     coalesced stores (or read-add-writes when the system already holds
//     values).
//
// GB300 issues FP64 at about 1/58 of its FP32 rate, and these kernels are
// bound by FP64 issue, not by HBM. Divisions therefore use a MUFU
// reciprocal seed refined by one cubic and one Newton step (5 FMAs, a few
// ulp), constant divisors become multiplications, node-only factors are
// computed once per node, and option branches are compile-time template
// parameters.
#include <cuda_runtime.h>

#include <cstdint>

#include "assemble.h"
#include "nw_internal.h"

namespace nw {
namespace {

constexpr int kThreads = 256;
constexpr int kRow1Threads = 128;  // node rows per block, 1-dof row phase
constexpr int kRow3Threads = 64;   // node rows per block, 3-dof row phase
constexpr int kMaxRowSmem = 96 * 1024;  // staging capacity limit per block

// 1/x from the MUFU approximation (rcp.approx.ftz.f64) refined by a cubic
// step r(1 + e + e^2) and a Newton step r(1 + e), e = 1 - x r. Zero,
// infinite and denormal inputs return the seed (inf, 0 or inf).
__device__ __forceinline__ double fast_rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  if (r == 0.0 || isinf(r)) return r;
  double e = fma(-x, r, 1.0);
  r = fma(r, fma(e, e, e), r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

__device__ __forceinline__ double van_leer(double dqm, double dqp, double eps) {
  return (2.0 * (dqm * dqp + fabs(dqm * dqp))) *
         fast_rcp((dqm + dqp) * (dqm + dqp) + eps);
}

// ---------------------------------------------------------------------------
// Scalar advection-diffusion: ScalarEdgeSolverAlg::execute
// (src/edge_kernels/ScalarEdgeSolverAlg.C:85-205). Output per edge:
// A00, A01, A10, A11, b0, b1 (six SoA arrays of E doubles).
__global__ void __launch_bounds__(kThreads)
    scalar_edge_k(int64_t E, const int2* __restrict__ edges,
                  const double* __restrict__ coords,
                  const double* __restrict__ vrtm, const double* __restrict__ q,
                  const double* __restrict__ dqdx,
                  const double* __restrict__ density,
                  const double* __restrict__ dflux,
                  const double* __restrict__ area,
                  const double* __restrict__ mdotA, ScalarOpts o,
                  double* __restrict__ buf) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double eps = 1.0e-16;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  double av[3];
  for (int d = 0; d < 3; ++d) av[d] = area[3 * e + d];
  const double mdot = mdotA[e];
  const double densityL = density[L], densityR = density[R];
  const double qNp1L = q[L], qNp1R = q[R];
  const double viscosityL = dflux[L], viscosityR = dflux[R];
  const double viscIp = 0.5 * (viscosityL + viscosityR);
  const double diffIp = 0.5 * (viscosityL * fast_rcp(densityL) +
                               viscosityR * fast_rcp(densityR));
  double dx[3];
  double axdx = 0.0, asq = 0.0, udotx = 0.0;
  for (int d = 0; d < 3; ++d) {
    dx[d] = coords[3 * R + d] - coords[3 * L + d];
    asq += av[d] * av[d];
    axdx += av[d] * dx[d];
    udotx += 0.5 * dx[d] * (vrtm[3 * R + d] + vrtm[3 * L + d]);
  }
  const double inv_axdx = fast_rcp(axdx);
  double dqL = 0.0, dqR = 0.0, nonOrth = 0.0;
  for (int d = 0; d < 3; ++d) {
    const double gL = dqdx[3 * L + d], gR = dqdx[3 * R + d];
    dqL += 0.5 * dx[d] * gL;
    dqR += 0.5 * dx[d] * gR;
    const double kxj = av[d] - asq * inv_axdx * dx[d];
    nonOrth += -viscIp * kxj * 0.5 * (gR + gL);
  }
  const double pecnum = fabs(udotx) * fast_rcp(diffIp + eps);
  double pecfac;
  if (o.tanh_form) {
    pecfac = 0.50 * (1.0 + tanh((pecnum - o.tanh_trans) / o.tanh_width));
  } else {
    const double m = o.hybrid_factor * pecnum;
    pecfac = m * m * fast_rcp(5.0 + m * m);
  }
  const double om_pecfac = 1.0 - pecfac;
  double limitL = 1.0, limitR = 1.0;
  if (o.use_limiter) {
    const double dq = qNp1R - qNp1L;
    limitL = van_leer(4.0 * dqL - dq, dq, eps);
    limitR = van_leer(4.0 * dqR - dq, dq, eps);
  }
  const double qIpL = qNp1L + dqL * o.upw_factor * limitL;
  const double qIpR = qNp1R - dqR * o.upw_factor * limitR;
  const double lhsfac = -viscIp * asq * inv_axdx;
  const double diffFlux = lhsfac * (qNp1R - qNp1L) + nonOrth;
  const double irelax = 1.0 / o.relax;
  double a00 = -lhsfac * irelax, a01 = lhsfac, a10 = lhsfac,
         a11 = -lhsfac * irelax;
  double b0 = -diffFlux, b1 = diffFlux;
  const double alpha = o.alpha, alphaUpw = o.alpha_upw;
  const double om_alpha = 1.0 - alpha, om_alphaUpw = 1.0 - alphaUpw;
  const double qIp = 0.5 * (qNp1R + qNp1L);
  const double qUpw = (mdot > 0) ? (alphaUpw * qIpL + om_alphaUpw * qIp)
                                 : (alphaUpw * qIpR + om_alphaUpw * qIp);
  const double qHatL = (alpha * qIpL + om_alpha * qIp);
  const double qHatR = (alpha * qIpR + om_alpha * qIp);
  const double qCds = 0.5 * (qHatL + qHatR);
  const double adv_flux = mdot * (pecfac * qUpw + om_pecfac * qCds);
  b0 -= adv_flux;
  b1 += adv_flux;
  double alhsfac = 0.5 * (mdot + fabs(mdot)) * pecfac * alphaUpw +
                   0.5 * alpha * om_pecfac * mdot;
  a00 += alhsfac * irelax;
  a10 -= alhsfac;
  alhsfac = 0.5 * (mdot - fabs(mdot)) * pecfac * alphaUpw +
            0.5 * alpha * om_pecfac * mdot;
  a11 -= alhsfac * irelax;
  a01 += alhsfac;
  alhsfac = 0.5 * mdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
  a00 += alhsfac * irelax;
  a01 += alhsfac;
  a10 -= alhsfac;
  a11 -= alhsfac * irelax;
  buf[e] = a00;
  buf[E + e] = a01;
  buf[2 * E + e] = a10;
  buf[3 * E + e] = a11;
  buf[4 * E + e] = b0;
  buf[5 * E + e] = b1;
}

// ---------------------------------------------------------------------------
// Continuity / pressure Poisson: ContinuityEdgeSolverAlg::execute
// (src/edge_kernels/ContinuityEdgeSolverAlg.C:109-194), no balanced buoyancy
// and no GCL term. The 2x2 local matrix is [-f, f; f, -f] with
// f = lhsfac, and the rhs is (-tmdot, tmdot); output per edge: f, tmdot.
//
// Fast form (rho u and rho_Ip u_Ip interpolated together, incompressible
// scaling off: the reference defaults): the node phase stores per node
//   n = (1/udiag, rho u_x, rho u_y, rho u_z, g_x, g_y, g_z, p),
//   g = (grad p) / udiag,
// so that tmdot = -0.5 (n0_L + n0_R) (p_R - p_L) w
//               + sum_d [0.5 (m_R + m_L) + 0.5 (g_R + g_L)]_d A_d
//               - noc sum_d k_d 0.5 (g_R + g_L)_d,
// w = |A|^2 / (A.dx), k = A - w dx, then tmdot /= tau. This is the
// reference expression regrouped; the parity tests bound the difference by
// eps times the running magnitude of each entry.
constexpr int kNodeStride = 8;

__global__ void __launch_bounds__(kThreads)
    continuity_node_k(int64_t N, const double* __restrict__ velocity,
                      const double* __restrict__ Gpdx,
                      const double* __restrict__ density,
                      const double* __restrict__ pressure,
                      const double* __restrict__ udiag,
                      double* __restrict__ nodebuf) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const double iu = fast_rcp(udiag[n]);
  const double rho = density[n];
  double2* out = reinterpret_cast<double2*>(nodebuf + kNodeStride * n);
  out[0] = make_double2(iu, rho * velocity[3 * n]);
  out[1] = make_double2(rho * velocity[3 * n + 1], rho * velocity[3 * n + 2]);
  out[2] = make_double2(Gpdx[3 * n] * iu, Gpdx[3 * n + 1] * iu);
  out[3] = make_double2(Gpdx[3 * n + 2] * iu, pressure[n]);
}

__global__ void __launch_bounds__(kThreads)
    continuity_edge_fast_k(int64_t E, const int2* __restrict__ edges,
                           const double* __restrict__ coords,
                           const double* __restrict__ nodebuf,
                           const double* __restrict__ area, double noc,
                           double inv_tau, double* __restrict__ buf) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  const double2* nl = reinterpret_cast<const double2*>(nodebuf + kNodeStride * L);
  const double2* nr = reinterpret_cast<const double2*>(nodebuf + kNodeStride * R);
  const double2 l0 = nl[0], l1 = nl[1], l2 = nl[2], l3 = nl[3];
  const double2 r0 = nr[0], r1 = nr[1], r2 = nr[2], r3 = nr[3];
  double av[3], dx[3];
  for (int d = 0; d < 3; ++d) {
    av[d] = area[3 * e + d];
    dx[d] = coords[3 * R + d] - coords[3 * L + d];
  }
  const double asq = av[0] * av[0] + av[1] * av[1] + av[2] * av[2];
  const double axdx = av[0] * dx[0] + av[1] * dx[1] + av[2] * dx[2];
  const double w = asq * fast_rcp(axdx);
  const double projTimeScale = 0.5 * (l0.x + r0.x);
  const double m[3] = {l0.y + r0.y, l1.x + r1.x, l1.y + r1.y};
  const double g[3] = {l2.x + r2.x, l2.y + r2.y, l3.x + r3.x};
  double flux = 0.0, corr = 0.0;
  for (int d = 0; d < 3; ++d) {
    const double kxj = av[d] - w * dx[d];
    flux = fma(m[d] + g[d], av[d], flux);
    corr = fma(kxj, g[d], corr);
  }
  double tmdot = -projTimeScale * (r3.y - l3.y) * w;
  tmdot = fma(0.5, fma(-noc, corr, flux), tmdot);
  tmdot *= inv_tau;
  buf[e] = -w * projTimeScale * inv_tau;
  buf[E + e] = tmdot;
}

// General options (interpolation blend, incompressible density scaling).
__global__ void __launch_bounds__(kThreads)
    continuity_edge_k(int64_t E, const int2* __restrict__ edges,
                      const double* __restrict__ coords,
                      const double* __restrict__ velocity,
                      const double* __restrict__ Gpdx,
                      const double* __restrict__ density,
                      const double* __restrict__ pressure,
                      const double* __restrict__ udiag,
                      const double* __restrict__ area, ContinuityOpts o,
                      double* __restrict__ buf) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  double av[3];
  for (int d = 0; d < 3; ++d) av[d] = area[3 * e + d];
  const double iuL = fast_rcp(udiag[L]), iuR = fast_rcp(udiag[R]);
  const double densityL = density[L], densityR = density[R];
  const double projTimeScale = 0.5 * (iuL + iuR);
  const double rhoIp = 0.5 * (densityL + densityR);
  const double denScale =
      fast_rcp(rhoIp) * o.solve_incompressible + (1.0 - o.solve_incompressible);
  double dx[3];
  double axdx = 0.0, asq = 0.0;
  for (int d = 0; d < 3; ++d) {
    dx[d] = coords[3 * R + d] - coords[3 * L + d];
    asq += av[d] * av[d];
    axdx += av[d] * dx[d];
  }
  const double inv_axdx = fast_rcp(axdx);
  double tmdot = -projTimeScale * (pressure[R] - pressure[L]) * asq * inv_axdx;
  const double interp = o.interp_together, om_interp = 1.0 - o.interp_together;
  for (int d = 0; d < 3; ++d) {
    const double kxj = av[d] - asq * inv_axdx * dx[d];
    const double uR = velocity[3 * R + d], uL = velocity[3 * L + d];
    const double rhoUjIp = 0.5 * (densityR * uR + densityL * uL);
    const double ujIp = 0.5 * (uR + uL);
    const double GjIp = 0.5 * (Gpdx[3 * R + d] * iuR + Gpdx[3 * L + d] * iuL);
    tmdot += (interp * rhoUjIp + om_interp * rhoIp * ujIp + GjIp) * av[d] -
             kxj * GjIp * o.noc_fac;
  }
  const double inv_tau = 1.0 / o.tau_scale;
  tmdot *= inv_tau;
  tmdot *= denScale;
  buf[e] = -asq * inv_axdx * projTimeScale * denScale * inv_tau;
  buf[E + e] = tmdot;
}

// ---------------------------------------------------------------------------
// Momentum: MomentumEdgeSolverAlg::execute (src/edge_kernels/
// MomentumEdgeSolverAlg.C:105-312), VOF off. The 6x6 local matrix has the
// block form
//   LL = cLL I - N/relax,  LR = cLR I + N,  RL = cRL I + N,
//   RR = cRR I - N/relax,  N_ij = -viscIp A_i A_j / (A.dx)
// because the advective and diffusive factors do not depend on the
// component; the rhs is (-tf, +tf). Output per edge (13 SoA arrays):
// cLL, cLR, cRL, cRR, N00, N01, N02, N11, N12, N22, tf0, tf1, tf2.
template <bool LIMITER, bool DIVU>
__global__ void __launch_bounds__(kThreads)
    momentum_edge_k(int64_t E, const int2* __restrict__ edges,
                    const double* __restrict__ coords,
                    const double* __restrict__ vel,
                    const double* __restrict__ dudx,
                    const double* __restrict__ viscosity,
                    const double* __restrict__ mask,
                    const double* __restrict__ area,
                    const double* __restrict__ mdotA,
                    const double* __restrict__ pecA, MomentumOpts o,
                    double irelax, double* __restrict__ buf) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double eps = 1.0e-16;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  double av[3], dx[3], uL[3], uR[3];
  for (int d = 0; d < 3; ++d) {
    av[d] = area[3 * e + d];
    dx[d] = coords[3 * R + d] - coords[3 * L + d];
    uL[d] = vel[3 * L + d];
    uR[d] = vel[3 * R + d];
  }
  const double mdot = mdotA[e];
  const double viscIp = 0.5 * (viscosity[L] + viscosity[R]);
  const double asq = av[0] * av[0] + av[1] * av[1] + av[2] * av[2];
  const double axdx = av[0] * dx[0] + av[1] * dx[1] + av[2] * dx[2];
  const double inv_axdx = fast_rcp(axdx);
  double gL[9], gR[9];
  for (int k = 0; k < 9; ++k) {
    gL[k] = dudx[9 * L + k];
    gR[k] = dudx[9 * R + k];
  }
  const double hdx[3] = {0.5 * dx[0], 0.5 * dx[1], 0.5 * dx[2]};
  double duL[3], duR[3];
  for (int i = 0; i < 3; ++i) {
    duL[i] = hdx[0] * gL[3 * i] + hdx[1] * gL[3 * i + 1] + hdx[2] * gL[3 * i + 2];
    duR[i] = hdx[0] * gR[3 * i] + hdx[1] * gR[3 * i + 1] + hdx[2] * gR[3 * i + 2];
  }
  double limitL[3] = {1.0, 1.0, 1.0}, limitR[3] = {1.0, 1.0, 1.0};
  if (LIMITER) {
    for (int d = 0; d < 3; ++d) {
      const double du = uR[d] - uL[d];
      limitL[d] = van_leer(4.0 * duL[d] - du, du, eps);
      limitR[d] = van_leer(4.0 * duR[d] - du, du, eps);
    }
  }
  const double pecfac = pecA[e];
  const double om_pecfac = 1.0 - pecfac;
  const double alpha = o.alpha, alphaUpw = o.alpha_upw;
  const double om_alpha = 1.0 - alpha, om_alphaUpw = 1.0 - alphaUpw;
  // duidxj with the over-relaxed non-orthogonal correction; gj holds the
  // sum (not the mean) of the two nodal gradients
  double duidxj[3][3];
  for (int i = 0; i < 3; ++i) {
    const double dui = uR[i] - uL[i];
    double gj[3];
    for (int j = 0; j < 3; ++j) gj[j] = gR[3 * i + j] + gL[3 * i + j];
    const double gjuidx = hdx[0] * gj[0] + hdx[1] * gj[1] + hdx[2] * gj[2];
    const double corr = (dui - gjuidx) * inv_axdx;
    for (int j = 0; j < 3; ++j) duidxj[i][j] = fma(corr, av[j], 0.5 * gj[j]);
  }
  const double maskNode = fmin(mask[L], mask[R]);
  double tf[3];
  double divU = 0.0;
  if (DIVU) divU = duidxj[0][0] + duidxj[1][1] + duidxj[2][2];
  const bool up = mdot > 0.0;
  for (int i = 0; i < 3; ++i) {
    const double uIpL = uL[i] + duL[i] * o.upw_factor * limitL[i];
    const double uIpR = uR[i] - duR[i] * o.upw_factor * limitR[i];
    const double uiIp = 0.5 * (uR[i] + uL[i]);
    const double uiUpw = alphaUpw * (up ? uIpL : uIpR) + om_alphaUpw * uiIp;
    const double uiCds = 0.5 * (alpha * (uIpL + uIpR)) + om_alpha * uiIp;
    const double adv_flux = mdot * (pecfac * uiUpw + om_pecfac * uiCds);
    double s = (duidxj[i][0] + duidxj[0][i]) * av[0] +
               (duidxj[i][1] + duidxj[1][i]) * av[1] +
               (duidxj[i][2] + duidxj[2][i]) * av[2];
    double diff_flux = -viscIp * s;
    if (DIVU) diff_flux = fma(divU, 2.0 / 3.0 * viscIp * av[i] * o.include_div_u, diff_flux);
    tf[i] = fma(diff_flux, maskNode, adv_flux);
  }
  const double aUL = 0.5 * (mdot + fabs(mdot)) * pecfac * alphaUpw +
                     0.5 * alpha * om_pecfac * mdot;
  const double aUR = 0.5 * (mdot - fabs(mdot)) * pecfac * alphaUpw +
                     0.5 * alpha * om_pecfac * mdot;
  const double aC = 0.5 * mdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
  const double dlhsfac = -viscIp * asq * inv_axdx;
  double* b = buf + e;
  b[0] = ((aUL + aC) - dlhsfac) * irelax;
  b[E] = (aUR + aC) + dlhsfac;
  b[2 * E] = (-aUL - aC) + dlhsfac;
  b[3 * E] = ((-aUR - aC) - dlhsfac) * irelax;
  const double t = -viscIp * inv_axdx;
  const double ta0 = t * av[0], ta1 = t * av[1], ta2 = t * av[2];
  b[4 * E] = ta0 * av[0];
  b[5 * E] = ta0 * av[1];
  b[6 * E] = ta0 * av[2];
  b[7 * E] = ta1 * av[1];
  b[8 * E] = ta1 * av[2];
  b[9 * E] = ta2 * av[2];
  b[10 * E] = tf[0];
  b[11 * E] = tf[1];
  b[12 * E] = tf[2];
}

// ---------------------------------------------------------------------------
// Row phase. Each block owns node rows [r0, r0 + kRowThreads) and therefore
// the contiguous CSR value range [row_ptr[nd r0], row_ptr[nd r1]). Threads
// build their rows in shared memory; the block then writes (or adds) the
// whole range with coalesced accesses. Blocks whose range exceeds the
// staging capacity write straight to global memory.
//
// KIND 0: scalar (six coefficients per edge), KIND 1: continuity (f,
// tmdot). Incident entries come in column order; bit 31 marks a repeat of
// the previous column (periodic duplicates).
template <int KIND>
__global__ void __launch_bounds__(kRow1Threads)
    row1_k(int64_t R, const int32_t* __restrict__ inc_ptr,
           const uint32_t* __restrict__ inc, const int32_t* __restrict__ diag_pos,
           const int64_t* __restrict__ row_ptr, const double* __restrict__ buf,
           int64_t E, double* __restrict__ values, double* __restrict__ rhs,
           int accumulate, int smem_bytes) {
  extern __shared__ double stage[];
  const int64_t r0 = int64_t(blockIdx.x) * kRow1Threads;
  const int64_t r1 = (r0 + kRow1Threads < R) ? r0 + kRow1Threads : R;
  const int64_t base = row_ptr[r0];
  const int64_t cnt = row_ptr[r1] - base;
  const bool staged = cnt * int64_t(sizeof(double)) <= smem_bytes;
  const int64_t r = r0 + threadIdx.x;
  if (r < r1) {
    const int32_t s = inc_ptr[r], t = inc_ptr[r + 1];
    const int64_t rb = row_ptr[r];
    double* out = staged ? stage + (rb - base) : values + rb;
    const bool acc = accumulate && !staged;
    if (s != t) {
      const int dp = diag_pos[r];
      double dg = 0.0, rr = 0.0, off = 0.0;
      int slot = -1;
      for (int32_t qi = s; qi < t; ++qi) {
        const uint32_t w = inc[qi];
        const bool dup = (w >> 31) != 0;
        const int64_t e = (w & 0x7fffffffu) >> 1;
        const int side = w & 1u;
        double co, cd, cr;
        if (KIND == 0) {
          co = buf[(side ? 2 : 1) * E + e];
          cd = buf[(side ? 3 : 0) * E + e];
          cr = buf[(side ? 5 : 4) * E + e];
        } else {
          const double f = buf[e], tm = buf[E + e];
          co = f;
          cd = -f;
          cr = side ? tm : -tm;
        }
        if (!dup) {
          if (slot >= 0) {
            double* p = out + (slot < dp ? slot : slot + 1);
            *p = acc ? *p + off : off;
          }
          ++slot;
          off = co;
        } else {
          off += co;
        }
        dg += cd;
        rr += cr;
      }
      double* p = out + (slot < dp ? slot : slot + 1);
      *p = acc ? *p + off : off;
      out[dp] = acc ? out[dp] + dg : dg;
      rhs[r] = accumulate ? rhs[r] + rr : rr;
    } else if (!acc) {
      // a row without edges: zero it (its entries are not otherwise written)
      for (int64_t k = 0; k < row_ptr[r + 1] - rb; ++k) out[k] = 0.0;
      if (!accumulate) rhs[r] = 0.0;
    }
  }
  if (!staged) return;
  __syncthreads();
  for (int64_t k = threadIdx.x; k < cnt; k += kRow1Threads)
    values[base + k] = accumulate ? values[base + k] + stage[k] : stage[k];
}

// 3-dof momentum: one thread per node row builds the node's three CSR rows
// (block column k at positions 3k..3k+2).
__global__ void __launch_bounds__(kRow3Threads)
    row3_k(int64_t R, const int32_t* __restrict__ inc_ptr,
           const uint32_t* __restrict__ inc, const int32_t* __restrict__ diag_pos,
           const int64_t* __restrict__ row_ptr, const double* __restrict__ buf,
           int64_t E, double irelax, double* __restrict__ values,
           double* __restrict__ rhs, int accumulate, int smem_bytes) {
  extern __shared__ double stage[];
  const int64_t r0 = int64_t(blockIdx.x) * kRow3Threads;
  const int64_t r1 = (r0 + kRow3Threads < R) ? r0 + kRow3Threads : R;
  const int64_t base = row_ptr[3 * r0];
  const int64_t cnt = row_ptr[3 * r1] - base;
  const bool staged = cnt * int64_t(sizeof(double)) <= smem_bytes;
  const int64_t r = r0 + threadIdx.x;
  if (r < r1) {
    const int32_t s = inc_ptr[r], t = inc_ptr[r + 1];
    const int64_t b0 = row_ptr[3 * r], b1 = row_ptr[3 * r + 1],
                  b2 = row_ptr[3 * r + 2];
    double* v0 = staged ? stage + (b0 - base) : values + b0;
    double* v1 = staged ? stage + (b1 - base) : values + b1;
    double* v2 = staged ? stage + (b2 - base) : values + b2;
    const bool acc = accumulate && !staged;
    if (s != t) {
      const int dp = diag_pos[r];
      double dgc = 0.0, dN[6] = {0, 0, 0, 0, 0, 0}, rr[3] = {0, 0, 0};
      double ob[9];
      int slot = -1;
      auto flush = [&](int sl) {
        const int k = 3 * (sl < dp ? sl : sl + 1);
        for (int c = 0; c < 3; ++c) {
          v0[k + c] = acc ? v0[k + c] + ob[c] : ob[c];
          v1[k + c] = acc ? v1[k + c] + ob[3 + c] : ob[3 + c];
          v2[k + c] = acc ? v2[k + c] + ob[6 + c] : ob[6 + c];
        }
      };
      for (int32_t qi = s; qi < t; ++qi) {
        const uint32_t w = inc[qi];
        const bool dup = (w >> 31) != 0;
        const int64_t e = (w & 0x7fffffffu) >> 1;
        const int side = w & 1u;
        const double co = buf[(side ? 2 : 1) * E + e];
        const double cd = buf[(side ? 3 : 0) * E + e];
        double n[6];
        for (int k = 0; k < 6; ++k) n[k] = buf[(4 + k) * E + e];
        const double f0 = buf[10 * E + e], f1 = buf[11 * E + e], f2 = buf[12 * E + e];
        if (side) {
          rr[0] += f0;
          rr[1] += f1;
          rr[2] += f2;
        } else {
          rr[0] -= f0;
          rr[1] -= f1;
          rr[2] -= f2;
        }
        const double blk[9] = {co + n[0], n[1], n[2], n[1], co + n[3], n[4],
                               n[2], n[4], co + n[5]};
        if (!dup) {
          if (slot >= 0) flush(slot);
          ++slot;
          for (int k = 0; k < 9; ++k) ob[k] = blk[k];
        } else {
          for (int k = 0; k < 9; ++k) ob[k] += blk[k];
        }
        dgc += cd;
        for (int k = 0; k < 6; ++k) dN[k] += n[k];
      }
      flush(slot);
      // diagonal block: sum(c) I - sum(N) / relax; cLL and cRR already
      // carry the 1/relax factor, N is scaled here
      if (irelax != 1.0)
        for (int q = 0; q < 6; ++q) dN[q] *= irelax;
      const double db[9] = {dgc - dN[0], -dN[1], -dN[2], -dN[1], dgc - dN[3],
                            -dN[4], -dN[2], -dN[4], dgc - dN[5]};
      const int k = 3 * dp;
      for (int c = 0; c < 3; ++c) {
        v0[k + c] = acc ? v0[k + c] + db[c] : db[c];
        v1[k + c] = acc ? v1[k + c] + db[3 + c] : db[3 + c];
        v2[k + c] = acc ? v2[k + c] + db[6 + c] : db[6 + c];
      }
      for (int q = 0; q < 3; ++q)
        rhs[3 * r + q] = accumulate ? rhs[3 * r + q] + rr[q] : rr[q];
    } else if (!acc) {
      for (int64_t k = 0; k < row_ptr[3 * r + 3] - b0; ++k) v0[k] = 0.0;
      if (!accumulate)
        for (int q = 0; q < 3; ++q) rhs[3 * r + q] = 0.0;
    }
  }
  if (!staged) return;
  __syncthreads();
  for (int64_t k = threadIdx.x; k < cnt; k += kRow3Threads)
    values[base + k] = accumulate ? values[base + k] + stage[k] : stage[k];
}

// applyDirichletBCs / resetRows: identity (or diag_value) rows.
__global__ void reset_rows_k(int64_t n, const int64_t* __restrict__ nodes,
                             const int64_t* __restrict__ node_lid, int num_dof,
                             int begin, int end, const int64_t* __restrict__ row_ptr,
                             const int32_t* __restrict__ col_idx,
                             double* __restrict__ values, double* __restrict__ rhs,
                             double diag_value, double rhs_value,
                             const double* __restrict__ q,
                             const double* __restrict__ bc, int64_t num_nodes,
                             int* __restrict__ err) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t node = nodes[k];
  if (node < 0 || node >= num_nodes) {
    atomicExch(err, 1);
    return;
  }
  const int64_t base = node_lid[node];
  for (int d = begin; d < end; ++d) {
    const int64_t row = base + d;
    for (int64_t p = row_ptr[row]; p < row_ptr[row + 1]; ++p)
      values[p] = (col_idx[p] == row) ? diag_value : 0.0;
    rhs[row] = bc ? (bc[num_dof * node + d] - q[num_dof * node + d]) : rhs_value;
  }
}

// LinearSystem::sumInto for one host-provided entity block: one thread per
// local row scans its CSR row (sum_into_row semantics).
__global__ void sum_into_block_k(int n_ent, int num_dof,
                                 const int64_t* __restrict__ ent_lid,
                                 const double* __restrict__ lhs,
                                 const double* __restrict__ brhs,
                                 const int64_t* __restrict__ row_ptr,
                                 const int32_t* __restrict__ col_idx,
                                 double* __restrict__ values,
                                 double* __restrict__ rhs) {
  const int nloc = n_ent * num_dof;
  const int i = threadIdx.x;
  if (i >= nloc) return;
  const int64_t row = ent_lid[i / num_dof] + i % num_dof;
  for (int j = 0; j < nloc; ++j) {
    const int32_t col = int32_t(ent_lid[j / num_dof] + j % num_dof);
    for (int64_t p = row_ptr[row]; p < row_ptr[row + 1]; ++p)
      if (col_idx[p] == col) {
        values[p] += lhs[i * nloc + j];
        break;
      }
  }
  rhs[row] += brhs[i];
}

inline unsigned grid_for(int64_t n, int t = kThreads) {
  return unsigned((n + t - 1) / t);
}

int g_smem_set_device = -1;
void set_smem_attrs() {
  int dev = 0;
  NW_CUDA(cudaGetDevice(&dev));
  if (g_smem_set_device == dev) return;
  NW_CUDA(cudaFuncSetAttribute(row1_k<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
  NW_CUDA(cudaFuncSetAttribute(row1_k<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
  NW_CUDA(cudaFuncSetAttribute(row3_k, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
  g_smem_set_device = dev;
}

}  // namespace

void launch_scalar_edges(cudaStream_t s, int64_t E, const int2* edges,
                         const nw_scalar_fields& f, const ScalarOpts& o,
                         double* buf) {
  if (E == 0) return;
  scalar_edge_k<<<grid_for(E), kThreads, 0, s>>>(
      E, edges, f.coords, f.velocity_rtm, f.q, f.dqdx, f.density,
      f.diff_coeff, f.area, f.mdot, o, buf);
}

bool continuity_fast_path(const ContinuityOpts& o) {
  return o.interp_together == 1.0 && o.solve_incompressible == 0.0;
}

void launch_continuity_edges(cudaStream_t s, int64_t E, int64_t N,
                             const int2* edges, const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf,
                             double* nodebuf) {
  if (E == 0) return;
  if (nodebuf && continuity_fast_path(o)) {
    continuity_node_k<<<grid_for(N), kThreads, 0, s>>>(
        N, f.velocity, f.dpdx, f.density, f.pressure, f.udiag, nodebuf);
    continuity_edge_fast_k<<<grid_for(E), kThreads, 0, s>>>(
        E, edges, f.coords, nodebuf, f.area, o.noc_fac, 1.0 / o.tau_scale, buf);
  } else {
    continuity_edge_k<<<grid_for(E), kThreads, 0, s>>>(
        E, edges, f.coords, f.velocity, f.dpdx, f.density, f.pressure, f.udiag,
        f.area, o, buf);
  }
}

void launch_continuity_edges(cudaStream_t s, int64_t E, const int2* edges,
                             const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf) {
  launch_continuity_edges(s, E, 0, edges, f, o, buf, nullptr);
}

void launch_momentum_edges(cudaStream_t s, int64_t E, const int2* edges,
                           const nw_momentum_fields& f, const MomentumOpts& o,
                           double* buf) {
  if (E == 0) return;
  const double irelax = 1.0 / o.relax;
  const bool lim = o.use_limiter != 0, divu = o.include_div_u != 0.0;
#define NW_MOM(LIM, DIV)                                                     \
  momentum_edge_k<LIM, DIV><<<grid_for(E), kThreads, 0, s>>>(                \
      E, edges, f.coords, f.velocity, f.dudx, f.viscosity, f.mask, f.area,   \
      f.mdot, f.pecfac, o, irelax, buf)
  if (lim && divu) NW_MOM(true, true);
  else if (lim) NW_MOM(true, false);
  else if (divu) NW_MOM(false, true);
  else NW_MOM(false, false);
#undef NW_MOM
}

int row_block_nodes(int kind) { return kind == 2 ? kRow3Threads : kRow1Threads; }

int row_stage_bytes(int kind, const int64_t* row_ptr_host, int64_t R) {
  const int nb = row_block_nodes(kind);
  const int nd = kind == 2 ? 3 : 1;
  int64_t mx = 0;
  for (int64_t r0 = 0; r0 < R; r0 += nb) {
    const int64_t r1 = r0 + nb < R ? r0 + nb : R;
    const int64_t c = row_ptr_host[nd * r1] - row_ptr_host[nd * r0];
    if (c > mx) mx = c;
  }
  const int64_t bytes = mx * int64_t(sizeof(double));
  return bytes <= kMaxRowSmem ? int(bytes) : kMaxRowSmem;
}

void launch_rows(cudaStream_t s, int kind, int64_t R, const int32_t* inc_ptr,
                 const uint32_t* inc, const int32_t* diag_pos,
                 const int64_t* row_ptr, const double* buf, int64_t E,
                 double relax, double* values, double* rhs, int accumulate,
                 int smem_bytes) {
  if (R == 0) return;
  set_smem_attrs();
  if (kind == 0)
    row1_k<0><<<grid_for(R, kRow1Threads), kRow1Threads, smem_bytes, s>>>(
        R, inc_ptr, inc, diag_pos, row_ptr, buf, E, values, rhs, accumulate, smem_bytes);
  else if (kind == 1)
    row1_k<1><<<grid_for(R, kRow1Threads), kRow1Threads, smem_bytes, s>>>(
        R, inc_ptr, inc, diag_pos, row_ptr, buf, E, values, rhs, accumulate, smem_bytes);
  else
    row3_k<<<grid_for(R, kRow3Threads), kRow3Threads, smem_bytes, s>>>(
        R, inc_ptr, inc, diag_pos, row_ptr, buf, E, 1.0 / relax, values, rhs, accumulate,
        smem_bytes);
}

void launch_reset_rows(cudaStream_t s, int64_t n, const int64_t* nodes,
                       const int64_t* node_lid, int num_dof, int begin,
                       int end, const int64_t* row_ptr, const int32_t* col_idx,
                       double* values, double* rhs, double diag_value,
                       double rhs_value, const double* q, const double* bc,
                       int64_t num_nodes, int* err) {
  if (n == 0) return;
  reset_rows_k<<<grid_for(n), kThreads, 0, s>>>(
      n, nodes, node_lid, num_dof, begin, end, row_ptr, col_idx, values, rhs,
      diag_value, rhs_value, q, bc, num_nodes, err);
}

void launch_sum_into_block(cudaStream_t s, int n_ent, int num_dof,
                           const int64_t* ent_lid, const double* lhs,
                           const double* rhs_in, const int64_t* row_ptr,
                           const int32_t* col_idx, double* values,
                           double* rhs) {
  sum_into_block_k<<<1, 128, 0, s>>>(n_ent, num_dof, ent_lid, lhs, rhs_in,
                                     row_ptr, col_idx, values, rhs);
}

}  // namespace nw
