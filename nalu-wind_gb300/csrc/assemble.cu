// Edge assembly kernels for sm_103a.
//
// The reference computes each edge's local system in a Kokkos team lambda
// (include/AssembleEdgeSolverAlgorithm.h:47-100) and scatters it with FP64
// atomics (TpetraLinearSystem::sum_into, src/TpetraLinearSystem.C:
// 1381-1459), so its summation order is not reproducible on a GPU. Here
// assembly has two deterministic phases:
//
//  1. edge phase: one thread per edge evaluates the edge physics once and
//     writes its compact coefficients to an edge-major buffer (SoA);
//  2. row phase: one thread per node row walks the row's incident
//     (edge, side) list, sorted by column then edge, accumulates the
//     diagonal block and rhs in registers and writes the row's CSR values
//     with plain stores (or adds, when the system already holds values).
//
// No floating-point atomics; the result is bitwise reproducible.
#include <cuda_runtime.h>

#include <cstdint>

#include "assemble.h"

namespace nw {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double van_leer(double dqm, double dqp, double eps) {
  return (2.0 * (dqm * dqp + fabs(dqm * dqp))) /
         ((dqm + dqp) * (dqm + dqp) + eps);
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
  const double diffIp = 0.5 * (viscosityL / densityL + viscosityR / densityR);
  double dx[3];
  double axdx = 0.0, asq = 0.0, udotx = 0.0;
  for (int d = 0; d < 3; ++d) {
    dx[d] = coords[3 * R + d] - coords[3 * L + d];
    asq += av[d] * av[d];
    axdx += av[d] * dx[d];
    udotx += 0.5 * dx[d] * (vrtm[3 * R + d] + vrtm[3 * L + d]);
  }
  const double inv_axdx = 1.0 / axdx;
  double dqL = 0.0, dqR = 0.0, nonOrth = 0.0;
  for (int d = 0; d < 3; ++d) {
    const double gL = dqdx[3 * L + d], gR = dqdx[3 * R + d];
    dqL += 0.5 * dx[d] * gL;
    dqR += 0.5 * dx[d] * gR;
    const double kxj = av[d] - asq * inv_axdx * dx[d];
    nonOrth += -viscIp * kxj * 0.5 * (gR + gL);
  }
  const double pecnum = fabs(udotx) / (diffIp + eps);
  double pecfac;
  if (o.tanh_form) {
    pecfac = 0.50 * (1.0 + tanh((pecnum - o.tanh_trans) / o.tanh_width));
  } else {
    const double m = o.hybrid_factor * pecnum;
    pecfac = m * m / (5.0 + m * m);
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
  const double relax = o.relax;
  double a00 = -lhsfac / relax, a01 = lhsfac, a10 = lhsfac,
         a11 = -lhsfac / relax;
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
  a00 += alhsfac / relax;
  a10 -= alhsfac;
  alhsfac = 0.5 * (mdot - fabs(mdot)) * pecfac * alphaUpw +
            0.5 * alpha * om_pecfac * mdot;
  a11 -= alhsfac / relax;
  a01 += alhsfac;
  alhsfac = 0.5 * mdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
  a00 += alhsfac / relax;
  a01 += alhsfac;
  a10 -= alhsfac;
  a11 -= alhsfac / relax;
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
  const double udiagL = udiag[L], udiagR = udiag[R];
  const double densityL = density[L], densityR = density[R];
  const double projTimeScale = 0.5 * (1.0 / udiagL + 1.0 / udiagR);
  const double rhoIp = 0.5 * (densityL + densityR);
  const double denScale = (1.0 / rhoIp) * o.solve_incompressible +
                          (1.0 - o.solve_incompressible);
  double dx[3];
  double axdx = 0.0, asq = 0.0;
  for (int d = 0; d < 3; ++d) {
    dx[d] = coords[3 * R + d] - coords[3 * L + d];
    asq += av[d] * av[d];
    axdx += av[d] * dx[d];
  }
  const double inv_axdx = 1.0 / axdx;
  double tmdot = -projTimeScale * (pressure[R] - pressure[L]) * asq * inv_axdx;
  const double interp = o.interp_together, om_interp = 1.0 - o.interp_together;
  for (int d = 0; d < 3; ++d) {
    const double kxj = av[d] - asq * inv_axdx * dx[d];
    const double uR = velocity[3 * R + d], uL = velocity[3 * L + d];
    const double rhoUjIp = 0.5 * (densityR * uR + densityL * uL);
    const double ujIp = 0.5 * (uR + uL);
    const double GjIp = 0.5 * (Gpdx[3 * R + d] / udiagR + Gpdx[3 * L + d] / udiagL);
    tmdot += (interp * rhoUjIp + om_interp * rhoIp * ujIp + GjIp) * av[d] -
             kxj * GjIp * o.noc_fac;
  }
  tmdot /= o.tau_scale;
  tmdot *= denScale;
  const double lhsfac = -asq * inv_axdx * projTimeScale * denScale / o.tau_scale;
  buf[e] = lhsfac;
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
                    double* __restrict__ buf) {
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
  double axdx = 0.0, asq = 0.0;
  for (int d = 0; d < 3; ++d) {
    asq += av[d] * av[d];
    axdx += av[d] * dx[d];
  }
  const double inv_axdx = 1.0 / axdx;
  double gL[9], gR[9];
  for (int k = 0; k < 9; ++k) {
    gL[k] = dudx[9 * L + k];
    gR[k] = dudx[9 * R + k];
  }
  double duL[3], duR[3];
  for (int i = 0; i < 3; ++i) {
    duL[i] = 0.0;
    duR[i] = 0.0;
    for (int j = 0; j < 3; ++j) {
      const double hdx = 0.5 * dx[j];
      duL[i] += hdx * gL[3 * i + j];
      duR[i] += hdx * gR[3 * i + j];
    }
  }
  double limitL[3] = {1.0, 1.0, 1.0}, limitR[3] = {1.0, 1.0, 1.0};
  if (o.use_limiter) {
    for (int d = 0; d < 3; ++d) {
      const double du = uR[d] - uL[d];
      limitL[d] = van_leer(4.0 * duL[d] - du, du, eps);
      limitR[d] = van_leer(4.0 * duR[d] - du, du, eps);
    }
  }
  const double pecfac = pecA[e];
  const double om_pecfac = 1.0 - pecfac;
  const double alpha = o.alpha, alphaUpw = o.alpha_upw, relax = o.relax;
  const double om_alpha = 1.0 - alpha, om_alphaUpw = 1.0 - alphaUpw;
  double uIpL[3], uIpR[3];
  for (int d = 0; d < 3; ++d) {
    uIpL[d] = uL[d] + duL[d] * o.upw_factor * limitL[d] * 1.0;
    uIpR[d] = uR[d] - duR[d] * o.upw_factor * limitR[d] * 1.0;
  }
  double duidxj[3][3];
  for (int i = 0; i < 3; ++i) {
    const double dui = uR[i] - uL[i];
    double gjuidx = 0.0;
    double gj[3];
    for (int j = 0; j < 3; ++j) {
      gj[j] = 0.5 * (gR[3 * i + j] + gL[3 * i + j]);
      gjuidx += gj[j] * dx[j];
    }
    for (int j = 0; j < 3; ++j)
      duidxj[i][j] = gj[j] + (dui - gjuidx) * av[j] * inv_axdx;
  }
  const double dlhsfac = -viscIp * asq * inv_axdx;
  const double maskNode = fmin(mask[L], mask[R]);
  double tf[3];
  double divU = 0.0;
  for (int j = 0; j < 3; ++j) divU += duidxj[j][j];
  for (int i = 0; i < 3; ++i) {
    const double uiIp = 0.5 * (uR[i] + uL[i]);
    const double uiUpw = (mdot > 0.0) ? (alphaUpw * uIpL[i] + om_alphaUpw * uiIp)
                                      : (alphaUpw * uIpR[i] + om_alphaUpw * uiIp);
    const double uiHatL = (alpha * uIpL[i] + om_alpha * uiIp);
    const double uiHatR = (alpha * uIpR[i] + om_alpha * uiIp);
    const double uiCds = 0.5 * (uiHatL + uiHatR);
    const double adv_flux = mdot * (pecfac * uiUpw + om_pecfac * uiCds);
    double diff_flux = divU * (2.0 / 3.0 * viscIp * av[i] * o.include_div_u);
    for (int j = 0; j < 3; ++j)
      diff_flux += -viscIp * (duidxj[i][j] + duidxj[j][i]) * av[j];
    tf[i] = adv_flux + diff_flux * maskNode;
  }
  const double aUL = 0.5 * (mdot + fabs(mdot)) * pecfac * alphaUpw +
                     0.5 * alpha * om_pecfac * mdot;
  const double aUR = 0.5 * (mdot - fabs(mdot)) * pecfac * alphaUpw +
                     0.5 * alpha * om_pecfac * mdot;
  const double aC = 0.5 * mdot * (pecfac * om_alphaUpw + om_pecfac * om_alpha);
  // same accumulation order as the reference's per-entry updates
  const double cLL = ((aUL / relax + aC / relax) - dlhsfac / relax);
  const double cLR = ((aUR + aC) + dlhsfac);
  const double cRL = ((-aUL - aC) + dlhsfac);
  const double cRR = ((-aUR / relax - aC / relax) - dlhsfac / relax);
  const double mv = -viscIp;
  double* b = buf + e;
  b[0] = cLL;
  b[E] = cLR;
  b[2 * E] = cRL;
  b[3 * E] = cRR;
  b[4 * E] = mv * av[0] * av[0] * inv_axdx;
  b[5 * E] = mv * av[0] * av[1] * inv_axdx;
  b[6 * E] = mv * av[0] * av[2] * inv_axdx;
  b[7 * E] = mv * av[1] * av[1] * inv_axdx;
  b[8 * E] = mv * av[1] * av[2] * inv_axdx;
  b[9 * E] = mv * av[2] * av[2] * inv_axdx;
  b[10 * E] = tf[0];
  b[11 * E] = tf[1];
  b[12 * E] = tf[2];
}

// ---------------------------------------------------------------------------
// Row phase, one dof per node. KIND 0: scalar (six coefficients per edge),
// KIND 1: continuity (f, tmdot). Incident entries are visited in column
// order; bit 31 marks a repeat of the previous column.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    row1_k(int64_t R, const int32_t* __restrict__ inc_ptr,
           const uint32_t* __restrict__ inc, const int32_t* __restrict__ diag_pos,
           const int64_t* __restrict__ row_ptr, const double* __restrict__ buf,
           int64_t E, double* __restrict__ values, double* __restrict__ rhs,
           int accumulate) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int32_t s = inc_ptr[r], t = inc_ptr[r + 1];
  if (s == t) return;
  const int64_t base = row_ptr[r];
  const int dp = diag_pos[r];
  double dg = 0.0, rr = 0.0, off = 0.0;
  int slot = -1;
  for (int32_t qi = s; qi < t; ++qi) {
    const uint32_t w = inc[qi];
    const bool dup = (w >> 31) != 0;
    const int64_t e = (w & 0x7fffffffu) >> 1;
    const int side = w & 1u;
    if (!dup) {
      if (slot >= 0) {
        const int64_t p = base + (slot < dp ? slot : slot + 1);
        values[p] = accumulate ? values[p] + off : off;
      }
      ++slot;
      off = 0.0;
    }
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
    off += co;
    dg += cd;
    rr += cr;
  }
  {
    const int64_t p = base + (slot < dp ? slot : slot + 1);
    values[p] = accumulate ? values[p] + off : off;
  }
  const int64_t pd = base + dp;
  values[pd] = accumulate ? values[pd] + dg : dg;
  rhs[r] = accumulate ? rhs[r] + rr : rr;
}

// Row phase for the 3-dof momentum system: one thread per node row writes
// the node's three CSR rows (block column k at positions 3k..3k+2).
__global__ void __launch_bounds__(kThreads)
    row3_k(int64_t R, const int32_t* __restrict__ inc_ptr,
           const uint32_t* __restrict__ inc, const int32_t* __restrict__ diag_pos,
           const int64_t* __restrict__ row_ptr, const double* __restrict__ buf,
           int64_t E, double relax, double* __restrict__ values,
           double* __restrict__ rhs, int accumulate) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int32_t s = inc_ptr[r], t = inc_ptr[r + 1];
  if (s == t) return;
  const int64_t b0 = row_ptr[3 * r], b1 = row_ptr[3 * r + 1],
                b2 = row_ptr[3 * r + 2];
  const int dp = diag_pos[r];
  double dgc = 0.0, dN[6] = {0, 0, 0, 0, 0, 0}, rr[3] = {0, 0, 0};
  double ob[9];
  int slot = -1;
  auto flush = [&](int sl) {
    const int k = sl < dp ? sl : sl + 1;
    double* v0 = values + b0 + 3 * k;
    double* v1 = values + b1 + 3 * k;
    double* v2 = values + b2 + 3 * k;
    if (accumulate) {
      for (int c = 0; c < 3; ++c) {
        v0[c] += ob[c];
        v1[c] += ob[3 + c];
        v2[c] += ob[6 + c];
      }
    } else {
      for (int c = 0; c < 3; ++c) {
        v0[c] = ob[c];
        v1[c] = ob[3 + c];
        v2[c] = ob[6 + c];
      }
    }
  };
  for (int32_t qi = s; qi < t; ++qi) {
    const uint32_t w = inc[qi];
    const bool dup = (w >> 31) != 0;
    const int64_t e = (w & 0x7fffffffu) >> 1;
    const int side = w & 1u;
    if (!dup) {
      if (slot >= 0) flush(slot);
      ++slot;
      for (int k = 0; k < 9; ++k) ob[k] = 0.0;
    }
    const double co = buf[(side ? 2 : 1) * E + e];
    const double cd = buf[(side ? 3 : 0) * E + e];
    double n[6];
    for (int k = 0; k < 6; ++k) n[k] = buf[(4 + k) * E + e];
    const double sg = side ? 1.0 : -1.0;
    for (int k = 0; k < 3; ++k) rr[k] += sg * buf[(10 + k) * E + e];
    // off-diagonal block co I + N
    ob[0] += co + n[0];
    ob[1] += n[1];
    ob[2] += n[2];
    ob[3] += n[1];
    ob[4] += co + n[3];
    ob[5] += n[4];
    ob[6] += n[2];
    ob[7] += n[4];
    ob[8] += co + n[5];
    dgc += cd;
    for (int k = 0; k < 6; ++k) dN[k] += n[k];
  }
  flush(slot);
  const double nr[6] = {dN[0] / relax, dN[1] / relax, dN[2] / relax,
                        dN[3] / relax, dN[4] / relax, dN[5] / relax};
  const double db[9] = {dgc - nr[0], -nr[1],      -nr[2],
                        -nr[1],      dgc - nr[3], -nr[4],
                        -nr[2],      -nr[4],      dgc - nr[5]};
  double* v0 = values + b0 + 3 * dp;
  double* v1 = values + b1 + 3 * dp;
  double* v2 = values + b2 + 3 * dp;
  for (int c = 0; c < 3; ++c) {
    v0[c] = accumulate ? v0[c] + db[c] : db[c];
    v1[c] = accumulate ? v1[c] + db[3 + c] : db[3 + c];
    v2[c] = accumulate ? v2[c] + db[6 + c] : db[6 + c];
  }
  for (int k = 0; k < 3; ++k)
    rhs[3 * r + k] = accumulate ? rhs[3 * r + k] + rr[k] : rr[k];
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

inline unsigned grid_for(int64_t n) {
  return unsigned((n + kThreads - 1) / kThreads);
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

void launch_continuity_edges(cudaStream_t s, int64_t E, const int2* edges,
                             const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf) {
  if (E == 0) return;
  continuity_edge_k<<<grid_for(E), kThreads, 0, s>>>(
      E, edges, f.coords, f.velocity, f.dpdx, f.density, f.pressure, f.udiag,
      f.area, o, buf);
}

void launch_momentum_edges(cudaStream_t s, int64_t E, const int2* edges,
                           const nw_momentum_fields& f, const MomentumOpts& o,
                           double* buf) {
  if (E == 0) return;
  momentum_edge_k<<<grid_for(E), kThreads, 0, s>>>(
      E, edges, f.coords, f.velocity, f.dudx, f.viscosity, f.mask, f.area,
      f.mdot, f.pecfac, o, buf);
}

void launch_rows(cudaStream_t s, int kind, int64_t R, const int32_t* inc_ptr,
                 const uint32_t* inc, const int32_t* diag_pos,
                 const int64_t* row_ptr, const double* buf, int64_t E,
                 double relax, double* values, double* rhs, int accumulate) {
  if (R == 0) return;
  if (kind == 0)
    row1_k<0><<<grid_for(R), kThreads, 0, s>>>(R, inc_ptr, inc, diag_pos,
                                               row_ptr, buf, E, values, rhs,
                                               accumulate);
  else if (kind == 1)
    row1_k<1><<<grid_for(R), kThreads, 0, s>>>(R, inc_ptr, inc, diag_pos,
                                               row_ptr, buf, E, values, rhs,
                                               accumulate);
  else
    row3_k<<<grid_for(R), kThreads, 0, s>>>(R, inc_ptr, inc, diag_pos,
                                            row_ptr, buf, E, relax, values,
                                            rhs, accumulate);
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
