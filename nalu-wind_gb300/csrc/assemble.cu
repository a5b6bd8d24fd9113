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
// GB300 issues FP64 at about 1/58 of its FP32 rate, so evaluated in FP64
// these kernels are bound by FP64 issue, not by HBM. The momentum and
// continuity kernels therefore evaluate the FP64 formulas in float-float
// arithmetic (dd.h: about 48 significant bits, error within a few 2^-48 of
// the operand magnitudes) on the FP32 pipes, split the FP64 inputs with
// integer operations, keep their edge coefficients as float pairs (8 bytes,
// the size of a double) and widen each finished CSR entry to FP64 once.
// The scalar kernel stays in FP64 (MUFU-seeded reciprocals). Node-only
// factors are computed once per node, and option branches are compile-time
// template parameters.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "assemble.h"
#include "schedule.h"
#include "dd.h"
#include "nw_internal.h"

namespace nw {
namespace {

constexpr int kThreads = 256;
constexpr int kRow1Threads = 128;  // node rows per block, 1-dof row phase
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
//   g = (grad p) / udiag (the edge phase forms p_R - p_L from the FP64
//   pressures, like the coordinate differences),
// so that tmdot = -0.5 (n0_L + n0_R) (p_R - p_L) w
//               + sum_d [0.5 (m_R + m_L) + 0.5 (g_R + g_L)]_d A_d
//               - noc sum_d k_d 0.5 (g_R + g_L)_d,
// w = |A|^2 / (A.dx), k = A - w dx, then tmdot /= tau. This is the
// reference expression regrouped; the parity tests bound the difference by
// eps times the running magnitude of each entry.
constexpr int kNodeStride = 8;  // dd slots (8 bytes each) per node

__device__ __forceinline__ dd ldd(const double* p) { return dd_from_double(*p); }
__device__ __forceinline__ void st4(dd* p, dd a, dd b, dd c, dd d) {
  float4* q = reinterpret_cast<float4*>(p);
  q[0] = make_float4(a.hi, a.lo, b.hi, b.lo);
  q[1] = make_float4(c.hi, c.lo, d.hi, d.lo);
}

// nodes [n0, n1)
__global__ void __launch_bounds__(kThreads)
    continuity_node_k(int64_t n0, int64_t n1, const double* __restrict__ velocity,
                      const double* __restrict__ Gpdx,
                      const double* __restrict__ density,
                      const double* __restrict__ pressure,
                      const double* __restrict__ udiag,
                      dd* __restrict__ nodebuf) {
  const int64_t n = n0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= n1) return;
  const dd iu = dd_rcp(ldd(udiag + n));
  const dd rho = ldd(density + n);
  dd* out = nodebuf + kNodeStride * n;
  st4(out, iu, rho * ldd(velocity + 3 * n), rho * ldd(velocity + 3 * n + 1),
      rho * ldd(velocity + 3 * n + 2));
  st4(out + 4, ldd(Gpdx + 3 * n) * iu, ldd(Gpdx + 3 * n + 1) * iu,
      ldd(Gpdx + 3 * n + 2) * iu, ldd(pressure + n));
}

__global__ void __launch_bounds__(kThreads)
    continuity_edge_fast_k(int64_t E, const int2* __restrict__ edges,
                           const double* __restrict__ coords,
                           const dd* __restrict__ nodebuf,
                           const double* __restrict__ pressure,
                           const double* __restrict__ area, dd noc,
                           dd inv_tau, dd* __restrict__ buf) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  dd nl[8], nr[8];
  {
    const float4* pl = reinterpret_cast<const float4*>(nodebuf + kNodeStride * L);
    const float4* pr = reinterpret_cast<const float4*>(nodebuf + kNodeStride * R);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 a = pl[k], b = pr[k];
      nl[2 * k] = {a.x, a.y};
      nl[2 * k + 1] = {a.z, a.w};
      nr[2 * k] = {b.x, b.y};
      nr[2 * k + 1] = {b.z, b.w};
    }
  }
  dd av[3], dx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    av[d] = ldd(area + 3 * e + d);
    dx[d] = dd_from_double(coords[3 * R + d] - coords[3 * L + d]);
  }
  const dd asq = dd_dot3(av[0], av[0], av[1], av[1], av[2], av[2]);
  const dd axdx = dd_dot3(av[0], dx[0], av[1], dx[1], av[2], dx[2]);
  const dd w = asq * dd_rcp(axdx);
  const dd projTimeScale = scale2(nl[0] + nr[0], 0.5f);
  dd mg[3], g[3], c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    g[d] = nl[4 + d] + nr[4 + d];
    mg[d] = (nl[1 + d] + nr[1 + d]) + g[d];
    c[d] = av[d] - w * dx[d];
  }
  // sum (rho u + G p / A_p) . A and the non-orthogonal correction
  // sum (A - w dx) . (G p / A_p), as three-term dots
  const dd flux = dd_dot3(mg[0], av[0], mg[1], av[1], mg[2], av[2]);
  const dd corr = dd_dot3(c[0], g[0], c[1], g[1], c[2], g[2]);
  dd tmdot = -(projTimeScale * dd_from_double(pressure[R] - pressure[L]) * w);
  tmdot = (tmdot + scale2(flux - noc * corr, 0.5f)) * inv_tau;
  const dd f = -(w * projTimeScale * inv_tau);
  reinterpret_cast<float4*>(buf)[e] = make_float4(f.hi, f.lo, tmdot.hi, tmdot.lo);
}

// General options (interpolation blend, incompressible density scaling).
struct ContinuityDD {
  dd noc, inv_tau, interp, om_interp, incomp, om_incomp;
};

__global__ void __launch_bounds__(kThreads)
    continuity_edge_k(int64_t E, const int2* __restrict__ edges,
                      const double* __restrict__ coords,
                      const double* __restrict__ velocity,
                      const double* __restrict__ Gpdx,
                      const double* __restrict__ density,
                      const double* __restrict__ pressure,
                      const double* __restrict__ udiag,
                      const double* __restrict__ area, ContinuityDD c,
                      dd* __restrict__ buf) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  const dd iuL = dd_rcp(ldd(udiag + L)), iuR = dd_rcp(ldd(udiag + R));
  const dd densityL = ldd(density + L), densityR = ldd(density + R);
  const dd projTimeScale = scale2(iuL + iuR, 0.5f);
  const dd rhoIp = scale2(densityL + densityR, 0.5f);
  const dd denScale = dd_rcp(rhoIp) * c.incomp + c.om_incomp;
  dd av[3], dx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    av[d] = ldd(area + 3 * e + d);
    dx[d] = dd_from_double(coords[3 * R + d] - coords[3 * L + d]);
  }
  const dd asq = av[0] * av[0] + av[1] * av[1] + av[2] * av[2];
  const dd axdx = av[0] * dx[0] + av[1] * dx[1] + av[2] * dx[2];
  const dd w = asq * dd_rcp(axdx);
  dd tmdot = -(projTimeScale * dd_from_double(pressure[R] - pressure[L]) * w);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const dd kxj = av[d] - w * dx[d];
    const dd uR = ldd(velocity + 3 * R + d), uL = ldd(velocity + 3 * L + d);
    const dd rhoUjIp = scale2(densityR * uR + densityL * uL, 0.5f);
    const dd ujIp = scale2(uR + uL, 0.5f);
    const dd GjIp = scale2(ldd(Gpdx + 3 * R + d) * iuR + ldd(Gpdx + 3 * L + d) * iuL, 0.5f);
    tmdot = tmdot + ((c.interp * rhoUjIp + c.om_interp * rhoIp * ujIp + GjIp) * av[d] -
                     kxj * GjIp * c.noc);
  }
  tmdot = tmdot * c.inv_tau * denScale;
  const dd f = -(w * projTimeScale * denScale * c.inv_tau);
  reinterpret_cast<float4*>(buf)[e] = make_float4(f.hi, f.lo, tmdot.hi, tmdot.lo);
}

__device__ __forceinline__ dd van_leer_dd(dd dqm, dd dqp, dd eps) {
  const dd p = dqm * dqp;
  const dd s = dqm + dqp;
  return scale2(p + dd_abs(p), 2.0f) * dd_rcp(s * s + eps);
}

// ---------------------------------------------------------------------------
// Momentum: MomentumEdgeSolverAlg::execute (src/edge_kernels/
// MomentumEdgeSolverAlg.C:105-312), VOF off. The 6x6 local matrix has the
// block form
//   LL = cLL I - N/relax,  LR = cLR I + N,  RL = cRL I + N,
//   RR = cRR I - N/relax,  N_ij = -viscIp A_i A_j / (A.dx)
// because the advective and diffusive factors do not depend on the
// component; the rhs is (-tf, +tf). In float-float arithmetic negation is
// exact and addition and multiplication are odd, so cLL = -cRL / relax and
// cRR = -cLR / relax hold bit for bit: the row phase derives the diagonal
// constants and the edge phase stores 11 SoA arrays of float pairs per
// edge: cLR, cRL, N00, N01, N02, N11, N12, N22, tf0, tf1, tf2.
struct MomentumDD {
  dd alpha, alpha_upw, om_alpha, om_alpha_upw, upw, divu_fac, irelax, eps;
};

struct MomentumIn {
  const int2* __restrict__ edges;
  const double* __restrict__ coords;
  const double* __restrict__ vel;
  const double* __restrict__ dudx;
  const double* __restrict__ viscosity;
  const double* __restrict__ mask;
  const double* __restrict__ area;
  const double* __restrict__ mdot;
  const double* __restrict__ pec;
};

// DEF: the reference's default advection options alpha = 0, alpha_upw = 1,
// upw_factor = 1 (SolutionOptions, src/SolutionOptions.C:31-80). The general
// formulas then multiply by exactly one and add exact zeros, which in
// float-float arithmetic return their operand unchanged, so the
// specialisation drops those operations and gives the same bits.
template <bool LIMITER, bool DIVU, bool DEF>
__device__ __forceinline__ void momentum_edge(int64_t e, int64_t E, const MomentumIn& in,
                                              const MomentumDD& c, dd* __restrict__ b) {
  const int2* __restrict__ edges = in.edges;
  const double* __restrict__ coords = in.coords;
  const double* __restrict__ vel = in.vel;
  const double* __restrict__ dudx = in.dudx;
  const double* __restrict__ viscosity = in.viscosity;
  const double* __restrict__ mask = in.mask;
  const double* __restrict__ area = in.area;
  const double* __restrict__ mdotA = in.mdot;
  const double* __restrict__ pecA = in.pec;
  const int2 lr = edges[e];
  // 32-bit node offsets (9 N < 2^32 is checked when the system is
  // finalized): fewer registers than 64-bit ones
  const uint32_t L = uint32_t(lr.x), R = uint32_t(lr.y);
  // coordinate and velocity differences are formed in FP64 and split once:
  // splitting each operand to a float pair first would keep only 48 bits of
  // each, and the difference of nearby values would lose the rest
  dd av[3], dx[3], uL[3], uR[3], du[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    av[d] = ldd(area + 3 * e + d);
    dx[d] = dd_from_double(coords[3 * R + d] - coords[3 * L + d]);
    uL[d] = ldd(vel + 3 * L + d);
    uR[d] = ldd(vel + 3 * R + d);
    du[d] = dd_from_double(vel[3 * R + d] - vel[3 * L + d]);
  }
  const dd mdot = ldd(mdotA + e);
  const dd viscIp = scale2(ldd(viscosity + L) + ldd(viscosity + R), 0.5f);
  const dd asq = dd_dot3(av[0], av[0], av[1], av[1], av[2], av[2]);
  const dd axdx = dd_dot3(av[0], dx[0], av[1], dx[1], av[2], dx[2]);
  const dd inv_axdx = dd_rcp(axdx);
  dd hdx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) hdx[d] = scale2(dx[d], 0.5f);
  // duidxj with the over-relaxed non-orthogonal correction (gj holds the
  // sum, not the mean, of the two nodal gradients); duL / duR are the
  // extrapolation increments 0.5 dx . grad u of each side, and their sum is
  // the correction's 0.5 dx . (grad u_L + grad u_R)
  dd duidxj[3][3], duL[3], duR[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dd gl[3], gr[3], gj[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      gl[j] = ldd(dudx + 9 * L + 3 * i + j);
      gr[j] = ldd(dudx + 9 * R + 3 * i + j);
      gj[j] = gr[j] + gl[j];
    }
    duL[i] = dd_dot3(hdx[0], gl[0], hdx[1], gl[1], hdx[2], gl[2]);
    duR[i] = dd_dot3(hdx[0], gr[0], hdx[1], gr[1], hdx[2], gr[2]);
    const dd gjuidx = duL[i] + duR[i];
    const dd corr = (du[i] - gjuidx) * inv_axdx;
#pragma unroll
    for (int j = 0; j < 3; ++j) duidxj[i][j] = corr * av[j] + scale2(gj[j], 0.5f);
  }
  dd limitL[3], limitR[3];
  if (LIMITER) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      limitL[d] = van_leer_dd(scale2(duL[d], 4.0f) - du[d], du[d], c.eps);
      limitR[d] = van_leer_dd(scale2(duR[d], 4.0f) - du[d], du[d], c.eps);
    }
  }
  const dd pecfac = ldd(pecA + e);
  const dd om_pecfac = dd{1.0f, 0.0f} - pecfac;
  const dd maskNode = dd_min(ldd(mask + L), ldd(mask + R));
  dd divU = {0.f, 0.f};
  if (DIVU) divU = duidxj[0][0] + duidxj[1][1] + duidxj[2][2];
  const bool up = dd_gt0(mdot);
  dd tf[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const dd uiIp = scale2(uR[i] + uL[i], 0.5f);
    dd adv_flux;
    if (DEF) {
      const dd uiUpw = up ? uL[i] + (LIMITER ? duL[i] * limitL[i] : duL[i])
                          : uR[i] - (LIMITER ? duR[i] * limitR[i] : duR[i]);
      adv_flux = mdot * (pecfac * uiUpw + om_pecfac * uiIp);
    } else {
      const dd uIpL = uL[i] + (LIMITER ? duL[i] * c.upw * limitL[i] : duL[i] * c.upw);
      const dd uIpR = uR[i] - (LIMITER ? duR[i] * c.upw * limitR[i] : duR[i] * c.upw);
      const dd uiUpw = c.alpha_upw * (up ? uIpL : uIpR) + c.om_alpha_upw * uiIp;
      const dd uiCds = scale2(c.alpha * (uIpL + uIpR), 0.5f) + c.om_alpha * uiIp;
      adv_flux = mdot * (pecfac * uiUpw + om_pecfac * uiCds);
    }
    const dd sd = dd_dot3(duidxj[i][0] + duidxj[0][i], av[0], duidxj[i][1] + duidxj[1][i], av[1],
                          duidxj[i][2] + duidxj[2][i], av[2]);
    dd diff_flux = -(viscIp * sd);
    if (DIVU) diff_flux = divU * (c.divu_fac * viscIp * av[i]) + diff_flux;
    tf[i] = diff_flux * maskNode + adv_flux;
  }
  const dd hm = scale2(mdot, 0.5f);
  const dd habs = scale2(dd_abs(mdot), 0.5f);
  dd aUL, aUR, aC;
  if (DEF) {
    aUL = (hm + habs) * pecfac;
    aUR = (hm - habs) * pecfac;
    aC = hm * om_pecfac;
  } else {
    const dd cen = c.alpha * om_pecfac * hm;
    aUL = (hm + habs) * pecfac * c.alpha_upw + cen;
    aUR = (hm - habs) * pecfac * c.alpha_upw + cen;
    aC = hm * (pecfac * c.om_alpha_upw + om_pecfac * c.om_alpha);
  }
  const dd t = -(viscIp * inv_axdx);
  const dd dlhsfac = t * asq;
  const dd ta0 = t * av[0], ta1 = t * av[1], ta2 = t * av[2];
  b[0] = (aUR + aC) + dlhsfac;
  b[E] = (-aUL - aC) + dlhsfac;
  b[2 * E] = ta0 * av[0];
  b[3 * E] = ta0 * av[1];
  b[4 * E] = ta0 * av[2];
  b[5 * E] = ta1 * av[1];
  b[6 * E] = ta1 * av[2];
  b[7 * E] = ta2 * av[2];
  b[8 * E] = tf[0];
  b[9 * E] = tf[1];
  b[10 * E] = tf[2];
}

template <bool LIMITER, bool DIVU, bool DEF>
__global__ void __launch_bounds__(kThreads, 4)
    momentum_edge_k(int64_t E, int64_t e0, int64_t e1, MomentumIn in, MomentumDD c,
                    dd* __restrict__ buf) {
  const int64_t e = e0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= e1) return;
  momentum_edge<LIMITER, DIVU, DEF>(e, E, in, c, buf + e);
}

// ---------------------------------------------------------------------------
// Row phase. Each block owns node rows [r0, r0 + kRowThreads) and therefore
// the contiguous CSR value range [row_ptr[nd r0], row_ptr[nd r1]). Threads
// build their rows in shared memory; the block then writes (or adds) the
// whole range with coalesced accesses. Blocks whose range exceeds the
// staging capacity write straight to global memory.
//
// KIND 0: scalar (six FP64 coefficients per edge), KIND 1: continuity
// (f, tmdot as float pairs). Incident entries come in column order; bit 31
// marks a repeat of the previous column (periodic duplicates).
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(dd v) { return dd_to_double_int(v); }

template <int KIND>
__global__ void __launch_bounds__(kRow1Threads)
    row1_k(int64_t R, const int32_t* __restrict__ inc_ptr,
           const uint32_t* __restrict__ inc, const int32_t* __restrict__ diag_pos,
           const int64_t* __restrict__ row_ptr, const double* __restrict__ buf,
           int64_t E, double* __restrict__ values, double* __restrict__ rhs,
           int accumulate, int smem_bytes) {
  using C = typename std::conditional<KIND == 0, double, dd>::type;
  const C* cb = reinterpret_cast<const C*>(buf);
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
      C dg{}, rr{}, off{};
      dd_acc dga, rra;  // continuity: the diagonal and rhs sums, deferred renormalisation
      int slot = -1;
      for (int32_t qi = s; qi < t; ++qi) {
        const uint32_t w = inc[qi];
        const bool dup = (w >> 31) != 0;
        const int64_t e = (w & 0x7fffffffu) >> 1;
        const int side = w & 1u;
        C co, cd, cr;
        if constexpr (KIND == 0) {
          co = cb[(side ? 2 : 1) * E + e];
          cd = cb[(side ? 3 : 0) * E + e];
          cr = cb[(side ? 5 : 4) * E + e];
        } else {
          const float4 q = reinterpret_cast<const float4*>(buf)[e];
          const dd f{q.x, q.y}, tm{q.z, q.w};
          co = f;
          cd = -f;
          cr = side ? tm : -tm;
        }
        if (!dup) {
          if (slot >= 0) {
            double* p = out + (slot < dp ? slot : slot + 1);
            const double v = to_f64(off);
            *p = acc ? *p + v : v;
          }
          ++slot;
          off = co;
        } else {
          off = off + co;
        }
        if constexpr (KIND == 0) {
          dg = dg + cd;
          rr = rr + cr;
        } else {
          acc_add(dga, cd);
          acc_add(rra, cr);
        }
      }
      if constexpr (KIND == 1) {
        dg = acc_value(dga);
        rr = acc_value(rra);
      }
      double* p = out + (slot < dp ? slot : slot + 1);
      const double v = to_f64(off), vd = to_f64(dg), vr = to_f64(rr);
      *p = acc ? *p + v : v;
      out[dp] = acc ? out[dp] + vd : vd;
      rhs[r] = accumulate ? rhs[r] + vr : vr;
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

// 3-dof momentum, one thread per CSR row (three per node row, dof q =
// thread % 3): each thread accumulates its row of every 3x3 block from the
// float-pair coefficients and widens it to FP64 with integer operations
// (dd_to_double_int: no FP64 instruction per entry); a block of kRow3Nodes node
// rows stages their CSR range in shared memory and writes it coalesced.
// (One thread per node row, with the symmetric blocks widened once, needs
// a third fewer FP64 adds but ran at a third of the occupancy: the shared
// staging per node is the same, so measured 0.357 against 0.328 ms.)
// Off-diagonal block of an incident edge: c_side I + N; diagonal block:
// -(sum of the other side's constants + sum of N) / relax.
constexpr int kRow3Nodes = 64;
struct Row3Args {
  int64_t R, E;  // end of the node rows; stride of the coefficient arrays
  int64_t r_begin;  // first node row (the row kernel's blocks start here)
  int64_t mask;  // edge -> coefficient slot: e & mask
  const int32_t* __restrict__ inc_ptr;
  const uint32_t* __restrict__ inc;
  const int32_t* __restrict__ diag_pos;
  const int64_t* __restrict__ row_ptr;
  const dd* cb;  // not restrict: the single-kernel assembly writes it in flight
  dd irelax;
  double* __restrict__ values;
  double* __restrict__ rhs;
  int accumulate, smem_bytes;
};

// coefficient loads: through the read-only path when the buffer is not
// written during the kernel (NC), else plain loads
template <bool NC>
__device__ __forceinline__ dd ldc(const dd* p) {
  if constexpr (NC) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return {v.x, v.y};
  } else {
    return *p;
  }
}

// One block of NB node rows starting at r0 (threads 0 .. 3 NB - 1 of the
// block; any others only take part in the staging copy).
// IDX: the type of the coefficient offsets (uint32_t when 11 E < 2^31:
// one register and one wide multiply-add per load instead of a 64-bit
// pointer per coefficient array). ACC: 0 overwrite, 1 add to the values
// present, -1 as a.accumulate says (the write mode as a constant drops the
// read and select of every store).
template <int NB, bool NC, typename IDX = int64_t, int ACC = -1>
__device__ __forceinline__ void row3_block(int64_t r0, const Row3Args& a, double* stage) {
  const dd* cb = a.cb;
  const bool accumulate = ACC < 0 ? a.accumulate != 0 : ACC != 0;
  const IDX E = IDX(a.E);
  const int64_t mask = a.mask;
  const int64_t r1 = (r0 + NB < a.R) ? r0 + NB : a.R;
  const int64_t base = a.row_ptr[3 * r0];
  const int64_t cnt = a.row_ptr[3 * r1] - base;
  const bool staged = cnt * int64_t(sizeof(double)) <= a.smem_bytes;
  const int local = threadIdx.x / 3, q = threadIdx.x - 3 * (threadIdx.x / 3);
  const int64_t r = local < NB ? r0 + local : r1;
  // row q of the symmetric N (N00 N01 N02 N11 N12 N22 at slots 2..7): its
  // diagonal N_qq and the off-diagonals of columns c1 < c2 (the two c != q),
  // so that the block's c_side I term adds to one fixed entry
  const int c1 = q == 0 ? 1 : 0, c2 = q == 2 ? 1 : 2;
  const IDX xd = IDX(q == 0 ? 2 : (q == 1 ? 5 : 7)) * E;
  const IDX x1 = IDX(q == 2 ? 4 : 3) * E;
  const IDX x2 = IDX(q == 0 ? 4 : 6) * E;
  const IDX xf = IDX(8 + q) * E;
  if (r < r1) {
    const int32_t s = a.inc_ptr[r], t = a.inc_ptr[r + 1];
    const int64_t bq = a.row_ptr[3 * r + q];
    double* v = staged ? stage + (bq - base) : a.values + bq;
    const bool acc = accumulate && !staged;
    if (s != t) {
      const int dp = a.diag_pos[r];
      // sums over the incident edges: the diagonal entry's N_qq + c_other,
      // the two off-diagonal N sums and the rhs (deferred renormalisation)
      dd_acc sdg, s1, s2, rr;
      dd od{}, o1{}, o2{};
      int slot = -1;
      auto put3 = [&](int k, dd xd, dd x1, dd x2) {
        const double d0 = dd_to_double_int(xd), d1 = dd_to_double_int(x1),
                     d2 = dd_to_double_int(x2);
        v[k + q] = acc ? v[k + q] + d0 : d0;
        v[k + c1] = acc ? v[k + c1] + d1 : d1;
        v[k + c2] = acc ? v[k + c2] + d2 : d2;
      };
      for (int32_t qi = s; qi < t; ++qi) {
        const uint32_t w = a.inc[qi];
        const bool dup = (w >> 31) != 0;
        const IDX e = IDX(int64_t((w & 0x7fffffffu) >> 1) & mask);
        const int side = w & 1u;
        const dd c0 = ldc<NC>(cb + e), c1v = ldc<NC>(cb + (E + e));
        const dd co = side ? c1v : c0, other = side ? c0 : c1v;
        const dd nd = ldc<NC>(cb + (xd + e)), n1 = ldc<NC>(cb + (x1 + e)), n2 = ldc<NC>(cb + (x2 + e));
        const dd f = ldc<NC>(cb + (xf + e));
        acc_add(rr, side ? f : -f);
        const dd bd = nd + co;
        if (!dup) {
          if (slot >= 0) put3(3 * (slot < dp ? slot : slot + 1), od, o1, o2);
          ++slot;
          od = bd;
          o1 = n1;
          o2 = n2;
        } else {
          od = od + bd;
          o1 = o1 + n1;
          o2 = o2 + n2;
        }
        acc_add(sdg, nd);
        acc_add(sdg, other);
        acc_add(s1, n1);
        acc_add(s2, n2);
      }
      put3(3 * (slot < dp ? slot : slot + 1), od, o1, o2);
      // diagonal block row q: -(sum(other) e_q + sum(N)_q) / relax
      put3(3 * dp, -(acc_value(sdg) * a.irelax), -(acc_value(s1) * a.irelax),
           -(acc_value(s2) * a.irelax));
      const double d = dd_to_double_int(acc_value(rr));
      a.rhs[3 * r + q] = accumulate ? a.rhs[3 * r + q] + d : d;
    } else if (!acc) {
      for (int64_t k = 0; k < a.row_ptr[3 * r + q + 1] - bq; ++k) v[k] = 0.0;
      if (!accumulate) a.rhs[3 * r + q] = 0.0;
    }
  }
  if (!staged) return;
  __syncthreads();
  // a staged range fits the shared array: 32-bit counts
  double* out = a.values + base;
  const int n = int(cnt);
  for (int k = int(threadIdx.x); k < n; k += int(blockDim.x))
    out[k] = accumulate ? out[k] + stage[k] : stage[k];
}

template <typename IDX, int ACC>
__global__ void __launch_bounds__(3 * kRow3Nodes) row3t_k(Row3Args a) {
  extern __shared__ double stage[];
  row3_block<kRow3Nodes, true, IDX, ACC>(a.r_begin + int64_t(blockIdx.x) * kRow3Nodes, a, stage);
}

// ---------------------------------------------------------------------------
// Single-kernel momentum assembly: a persistent kernel whose blocks take
// edge chunks and row blocks from the work list of schedule.h in ticket
// order. Edge chunks write their coefficients into a ring of slots small
// enough to stay in L2, row blocks read them from there, so the coefficient
// round trip of the two-kernel form never reaches DRAM. The arithmetic and
// the summation order are those of momentum_edge_k + row3t_k: the CSR
// values are the same bits.
//
// Dependencies are flags holding the launch's generation number: a chunk's
// flag is set once its coefficients are written, a row block's once its
// reads are done. Waits only point to earlier tickets, held by running
// blocks, so they end; each poll is still bounded (kSpinLimit rounds), after
// which the block records the timeout in *err, skips its work, sets its own
// flag and the remaining blocks stop taking tickets.
struct FusedArgs {
  const int32_t* __restrict__ items;
  const int32_t* __restrict__ in_ptr;   // row block k reads chunks in[in_ptr[k] ..]
  const int32_t* __restrict__ in;
  const int32_t* __restrict__ out_ptr;  // chunk c is read by blocks out[out_ptr[c] ..]
  const int32_t* __restrict__ out;
  int* eflag;
  int* rflag;
  int* ticket;
  int* err;
  int64_t num_edges, ring_chunks;
  int nitems, gen;
};

constexpr int kSpinLimit = 1 << 20;

__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// True once flags[list[0 .. n)] all hold gen. Each thread polls a strided
// share with relaxed loads and, having seen its flags set, issues one
// acquire fence (the flag was set by a release store after the producer's
// writes), then the block agrees at a barrier. False in every thread after a
// timeout, or when another block has reported one.
__device__ bool wait_flags(const int* flags, const int32_t* list, int n, int gen, int* err) {
  bool ok = true, polled = false;
  for (int i = int(threadIdx.x); ok && i < n; i += int(blockDim.x)) {
    const int* fp = flags + list[i];
    polled = true;
    int spins = 0;
    while (ld_relaxed(fp) != gen) {
      if (++spins > kSpinLimit || ((spins & 1023) == 0 && ld_volatile(err) != 0)) {
        ok = false;
        break;
      }
      __nanosleep(64);
    }
  }
  if (polled && ok) fence_acq_rel();
  const bool all = __syncthreads_and(ok) != 0;
  if (!all && threadIdx.x == 0) atomicExch(err, 1);
  return all;
}

template <bool LIMITER, bool DIVU, bool DEF>
__global__ void __launch_bounds__(kFusedChunk, 4)
    momentum_fused_k(FusedArgs f, MomentumIn in, MomentumDD c, Row3Args ra, dd* ring) {
  extern __shared__ double stage[];
  __shared__ int s_item[2];
  int next = 0;
  if (threadIdx.x == 0) next = atomicAdd(f.ticket, 1);
  for (int p = 0;; p ^= 1) {
    // double-buffered item word: the barrier of the next item separates
    // this item's reads from the write two items on
    if (threadIdx.x == 0) s_item[p] = (next < f.nitems && ld_volatile(f.err) == 0) ? f.items[next] : -1;
    __syncthreads();
    const int it = s_item[p];
    if (it < 0) return;
    // the next ticket is taken now; its latency hides behind this item
    if (threadIdx.x == 0) next = atomicAdd(f.ticket, 1);
    const int idx = it >> 1;
    if (it & 1) {
      const int b = f.in_ptr[idx];
      if (wait_flags(f.eflag, f.in + b, f.in_ptr[idx + 1] - b, f.gen, f.err))
        row3_block<kFusedBlock, false>(int64_t(idx) * kFusedBlock, ra, stage);
      __syncthreads();
      if (threadIdx.x == 0) st_release(f.rflag + idx, f.gen);
    } else {
      // the slot's previous chunk must have been read by all its row blocks
      const int64_t prev = int64_t(idx) - f.ring_chunks;
      const bool ok = prev < 0 || wait_flags(f.rflag, f.out + f.out_ptr[prev],
                                             f.out_ptr[prev + 1] - f.out_ptr[prev], f.gen, f.err);
      const int64_t e = int64_t(idx) * kFusedChunk + threadIdx.x;
      if (ok && e < f.num_edges) momentum_edge<LIMITER, DIVU, DEF>(e, ra.E, in, c, ring + (e & ra.mask));
      __syncthreads();
      if (threadIdx.x == 0) st_release(f.eflag + idx, f.gen);
    }
  }
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
  NW_CUDA(cudaFuncSetAttribute(row3t_k<uint32_t, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
  NW_CUDA(cudaFuncSetAttribute(row3t_k<uint32_t, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
  NW_CUDA(cudaFuncSetAttribute(row3t_k<int64_t, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
  NW_CUDA(cudaFuncSetAttribute(row3t_k<int64_t, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem));
#define NW_FUSED_ATTR(LIM, DIV, DEF)                                                      \
  NW_CUDA(cudaFuncSetAttribute(momentum_fused_k<LIM, DIV, DEF>,                           \
                               cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxRowSmem))
  NW_FUSED_ATTR(false, false, false);
  NW_FUSED_ATTR(false, false, true);
  NW_FUSED_ATTR(false, true, false);
  NW_FUSED_ATTR(false, true, true);
  NW_FUSED_ATTR(true, false, false);
  NW_FUSED_ATTR(true, false, true);
  NW_FUSED_ATTR(true, true, false);
  NW_FUSED_ATTR(true, true, true);
#undef NW_FUSED_ATTR
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

dd dd_param(double x) { return dd_from_double(x); }

void launch_continuity_edge_range(cudaStream_t s, int64_t n0, int64_t n1, int64_t e0, int64_t e1,
                                  const int2* edges, const nw_continuity_fields& f,
                                  const ContinuityOpts& o, double* buf, double* nodebuf) {
  // the edge kernels index edges, area vectors and records from 0: shift
  // the per-edge pointers to the range
  const int64_t n = e1 > e0 ? e1 - e0 : 0;
  dd* b = reinterpret_cast<dd*>(buf) + 2 * e0;
  const int2* er = edges + e0;
  const double* ar = f.area + 3 * e0;
  if (nodebuf && continuity_fast_path(o)) {
    dd* nb = reinterpret_cast<dd*>(nodebuf);
    if (n1 > n0)
      continuity_node_k<<<grid_for(n1 - n0), kThreads, 0, s>>>(
          n0, n1, f.velocity, f.dpdx, f.density, f.pressure, f.udiag, nb);
    if (n)
      continuity_edge_fast_k<<<grid_for(n), kThreads, 0, s>>>(
          n, er, f.coords, nb, f.pressure, ar, dd_param(o.noc_fac), dd_param(1.0 / o.tau_scale), b);
  } else if (n) {
    ContinuityDD c;
    c.noc = dd_param(o.noc_fac);
    c.inv_tau = dd_param(1.0 / o.tau_scale);
    c.interp = dd_param(o.interp_together);
    c.om_interp = dd_param(1.0 - o.interp_together);
    c.incomp = dd_param(o.solve_incompressible);
    c.om_incomp = dd_param(1.0 - o.solve_incompressible);
    continuity_edge_k<<<grid_for(n), kThreads, 0, s>>>(
        n, er, f.coords, f.velocity, f.dpdx, f.density, f.pressure, f.udiag,
        ar, c, b);
  }
}

void launch_continuity_edges(cudaStream_t s, int64_t E, int64_t N,
                             const int2* edges, const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf,
                             double* nodebuf) {
  if (E == 0) return;
  launch_continuity_edge_range(s, 0, N, 0, E, edges, f, o, buf, nodebuf);
}

void launch_continuity_edges(cudaStream_t s, int64_t E, const int2* edges,
                             const nw_continuity_fields& f,
                             const ContinuityOpts& o, double* buf) {
  launch_continuity_edges(s, E, 0, edges, f, o, buf, nullptr);
}

namespace {
MomentumDD momentum_dd(const MomentumOpts& o) {
  MomentumDD c;
  c.alpha = dd_param(o.alpha);
  c.alpha_upw = dd_param(o.alpha_upw);
  c.om_alpha = dd_param(1.0 - o.alpha);
  c.om_alpha_upw = dd_param(1.0 - o.alpha_upw);
  c.upw = dd_param(o.upw_factor);
  c.divu_fac = dd_param(2.0 / 3.0 * o.include_div_u);
  c.irelax = dd_param(1.0 / o.relax);
  c.eps = dd_param(1.0e-16);
  return c;
}
MomentumIn momentum_in(const int2* edges, const nw_momentum_fields& f) {
  return MomentumIn{edges, f.coords, f.velocity, f.dudx, f.viscosity, f.mask, f.area, f.mdot, f.pecfac};
}
Row3Args row3_args(int64_t R, const int32_t* inc_ptr, const uint32_t* inc, const int32_t* diag_pos,
                   const int64_t* row_ptr, const double* buf, int64_t E, double relax, double* values,
                   double* rhs, int accumulate, int smem_bytes) {
  return Row3Args{R, E, 0, int64_t(-1), inc_ptr, inc, diag_pos, row_ptr, reinterpret_cast<const dd*>(buf),
                  dd_param(1.0 / relax), values, rhs, accumulate, smem_bytes};
}
}  // namespace

void launch_momentum_edges(cudaStream_t s, int64_t E, int64_t e0, int64_t e1, const int2* edges,
                           const nw_momentum_fields& f, const MomentumOpts& o,
                           double* buf) {
  if (e1 <= e0) return;
  const MomentumDD c = momentum_dd(o);
  const MomentumIn in = momentum_in(edges, f);
  dd* b = reinterpret_cast<dd*>(buf);
  const bool lim = o.use_limiter != 0, divu = o.include_div_u != 0.0;
  const bool def = o.alpha == 0.0 && o.alpha_upw == 1.0 && o.upw_factor == 1.0;
#define NW_MOM(LIM, DIV, DEF) \
  momentum_edge_k<LIM, DIV, DEF><<<grid_for(e1 - e0), kThreads, 0, s>>>(E, e0, e1, in, c, b)
#define NW_MOM2(LIM, DIV) \
  if (def) NW_MOM(LIM, DIV, true); \
  else NW_MOM(LIM, DIV, false)
  if (lim && divu) NW_MOM2(true, true);
  else if (lim) NW_MOM2(true, false);
  else if (divu) NW_MOM2(false, true);
  else NW_MOM2(false, false);
#undef NW_MOM2
#undef NW_MOM
}

int fused_blocks_per_sm(int smem_bytes) {
  set_smem_attrs();
  int occ = 0;
  NW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, momentum_fused_k<false, false, true>,
                                                        kFusedChunk, smem_bytes));
  return occ;
}

void launch_momentum_fused(cudaStream_t s, const FusedLaunch& L, const int2* edges,
                           const nw_momentum_fields& f, const MomentumOpts& o) {
  if (L.nitems == 0) return;
  set_smem_attrs();
  const MomentumDD c = momentum_dd(o);
  const MomentumIn in = momentum_in(edges, f);
  Row3Args ra = row3_args(L.R, L.inc_ptr, L.inc, L.diag_pos, L.row_ptr, L.ring, L.stride, o.relax,
                          L.values, L.rhs, L.accumulate, L.smem_bytes);
  ra.mask = L.mask;
  FusedArgs fa{L.items, L.in_ptr, L.in, L.out_ptr, L.out, L.eflag, L.rflag,
               L.ticket, L.err, L.num_edges, L.ring_chunks, int(L.nitems), L.gen};
  dd* ring = reinterpret_cast<dd*>(L.ring);
  NW_CUDA(cudaMemsetAsync(L.ticket, 0, sizeof(int), s));
  const bool lim = o.use_limiter != 0, divu = o.include_div_u != 0.0;
  const bool def = o.alpha == 0.0 && o.alpha_upw == 1.0 && o.upw_factor == 1.0;
#define NW_FUSED(LIM, DIV, DEF) \
  momentum_fused_k<LIM, DIV, DEF><<<L.grid, kFusedChunk, L.smem_bytes, s>>>(fa, in, c, ra, ring)
#define NW_FUSED2(LIM, DIV) \
  if (def) NW_FUSED(LIM, DIV, true); \
  else NW_FUSED(LIM, DIV, false)
  if (lim && divu) NW_FUSED2(true, true);
  else if (lim) NW_FUSED2(true, false);
  else if (divu) NW_FUSED2(false, true);
  else NW_FUSED2(false, false);
#undef NW_FUSED2
#undef NW_FUSED
}

int row_block_nodes(int kind) { return kind == 3 ? kFusedBlock : (kind == 2 ? kRow3Nodes : kRow1Threads); }

int row_stage_bytes(int kind, const int64_t* row_ptr_host, int64_t R) {
  const int nb = row_block_nodes(kind);
  const int nd = kind >= 2 ? 3 : 1;
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
                 int smem_bytes, int max_inc, int64_t row_begin) {
  if (R <= row_begin) return;
  set_smem_attrs();
  if (kind == 0)
    row1_k<0><<<grid_for(R, kRow1Threads), kRow1Threads, smem_bytes, s>>>(
        R, inc_ptr, inc, diag_pos, row_ptr, buf, E, values, rhs, accumulate, smem_bytes);
  else if (kind == 1)
    row1_k<1><<<grid_for(R, kRow1Threads), kRow1Threads, smem_bytes, s>>>(
        R, inc_ptr, inc, diag_pos, row_ptr, buf, E, values, rhs, accumulate, smem_bytes);
  else {
    Row3Args a = row3_args(R, inc_ptr, inc, diag_pos, row_ptr, buf, E, relax, values, rhs,
                           accumulate, smem_bytes);
    a.r_begin = row_begin;
    const unsigned grid = grid_for(R - row_begin, kRow3Nodes);
    const bool narrow = int64_t(kMomentumCoefs) * E < (int64_t(1) << 31);
    if (narrow && !accumulate)
      row3t_k<uint32_t, 0><<<grid, 3 * kRow3Nodes, smem_bytes, s>>>(a);
    else if (narrow)
      row3t_k<uint32_t, 1><<<grid, 3 * kRow3Nodes, smem_bytes, s>>>(a);
    else if (!accumulate)
      row3t_k<int64_t, 0><<<grid, 3 * kRow3Nodes, smem_bytes, s>>>(a);
    else
      row3t_k<int64_t, 1><<<grid, 3 * kRow3Nodes, smem_bytes, s>>>(a);
  }
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
