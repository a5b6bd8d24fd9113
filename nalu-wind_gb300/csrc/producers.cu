// Input producers of the edge assembly, on the GPU: the per-edge mass flow
// rate (MdotEdgeAlg), the edge-based nodal gradient (NodalGradEdgeAlg with a
// lumped boundary closure) and the per-edge Peclet factor
// (MomentumEdgePecletAlg). They run every nonlinear iteration just before
// the assembly and use the same edge list and incidence lists as the
// handle they are called on; like the assembly kernels they evaluate FP64
// formulas in float-float arithmetic (dd.h) and sum without atomics.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "dd.h"
#include "nw_capi.h"
#include "nw_internal.h"

namespace nw {
namespace {

constexpr int kThreads = 256;
inline unsigned grid_for(int64_t n) { return unsigned((n + kThreads - 1) / kThreads); }

__device__ __forceinline__ dd ldd(const double* p) { return dd_from_double(*p); }

// MdotEdgeAlg::execute (src/ngp_algorithms/MdotEdgeAlg.C:117-190) without
// balanced forcing and GCL terms:
//   tmdot = -projTimeScale (p_R - p_L) |A|^2 / (A.dx)
//         + sum_d (interp rhoU_Ip + (1 - interp) rho_Ip u_Ip + G_Ip)_d A_d
//         - noc sum_d k_d G_Ip,d,   k = A - |A|^2 dx / (A.dx)
__global__ void __launch_bounds__(kThreads)
    mdot_k(int64_t E, const int2* __restrict__ edges, const double* __restrict__ coords,
           const double* __restrict__ velocity, const double* __restrict__ Gpdx,
           const double* __restrict__ density, const double* __restrict__ pressure,
           const double* __restrict__ udiag, const double* __restrict__ area, dd noc,
           dd interp, dd om_interp, double* __restrict__ mdot) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  const dd iuL = dd_rcp(ldd(udiag + L)), iuR = dd_rcp(ldd(udiag + R));
  const dd rhoL = ldd(density + L), rhoR = ldd(density + R);
  const dd projTimeScale = scale2(iuL + iuR, 0.5f);
  const dd rhoIp = scale2(rhoL + rhoR, 0.5f);
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
    const dd uR = ldd(velocity + 3 * R + d), uL = ldd(velocity + 3 * L + d);
    const dd rhoUjIp = scale2(rhoR * uR + rhoL * uL, 0.5f);
    const dd ujIp = scale2(uR + uL, 0.5f);
    const dd GjIp = scale2(ldd(Gpdx + 3 * R + d) * iuR + ldd(Gpdx + 3 * L + d) * iuL, 0.5f);
    tmdot = tmdot + ((interp * rhoUjIp + om_interp * rhoIp * ujIp + GjIp) * av[d] -
                     (av[d] - w * dx[d]) * GjIp * noc);
  }
  mdot[e] = dd_to_double(tmdot);
}

// NodalGradEdgeAlg::execute (src/ngp_algorithms/NodalGradEdgeAlg.C:85-109):
// grad_L += A phi_Ip / V_L, grad_R -= A phi_Ip / V_R, phi_Ip the edge
// midpoint average, plus bnd_area phi on exposed faces; periodic masters
// and slaves hold the sum. Thread per node row: its incident edges in
// order, then the row's nodes' boundary terms; the result goes to every
// node of the row.
template <int DIM1>
__global__ void __launch_bounds__(kThreads)
    nodal_grad_k(int64_t R, const int32_t* __restrict__ inc_ptr, const uint32_t* __restrict__ inc,
                 const int2* __restrict__ edges, const int64_t* __restrict__ rn_ptr,
                 const int32_t* __restrict__ rn, const double* __restrict__ phi,
                 const double* __restrict__ area, const double* __restrict__ dualvol,
                 const double* __restrict__ bnd_area, double* __restrict__ grad) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= R) return;
  dd acc[DIM1][3];
#pragma unroll
  for (int i = 0; i < DIM1; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) acc[i][j] = dd{0.f, 0.f};
  for (int32_t q = inc_ptr[r]; q < inc_ptr[r + 1]; ++q) {
    const uint32_t w = inc[q];
    const int64_t e = (w & 0x7fffffffu) >> 1;
    const bool right = (w & 1u) != 0;
    const int2 lr = edges[e];
    dd a[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      a[j] = ldd(area + 3 * e + j);
      if (right) a[j] = -a[j];
    }
#pragma unroll
    for (int i = 0; i < DIM1; ++i) {
      const dd pip = scale2(ldd(phi + int64_t(DIM1) * lr.x + i) + ldd(phi + int64_t(DIM1) * lr.y + i), 0.5f);
#pragma unroll
      for (int j = 0; j < 3; ++j) acc[i][j] = a[j] * pip + acc[i][j];
    }
  }
  const int64_t n0 = rn_ptr[r], n1 = rn_ptr[r + 1];
  if (bnd_area)
    for (int64_t k = n0; k < n1; ++k) {
      const int64_t nd = rn[k];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const dd b = ldd(bnd_area + 3 * nd + j);
#pragma unroll
        for (int i = 0; i < DIM1; ++i) acc[i][j] = b * ldd(phi + int64_t(DIM1) * nd + i) + acc[i][j];
      }
    }
  const dd iv = dd_rcp(ldd(dualvol + rn[n0]));
  double out[DIM1 * 3];
#pragma unroll
  for (int i = 0; i < DIM1; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) out[3 * i + j] = dd_to_double(acc[i][j] * iv);
  for (int64_t k = n0; k < n1; ++k) {
    double* g = grad + int64_t(DIM1 * 3) * rn[k];
#pragma unroll
    for (int c = 0; c < DIM1 * 3; ++c) g[c] = out[c];
  }
}

// MomentumEdgePecletAlg::execute (src/edge_kernels/MomentumEdgePecletAlg.C:
// 74-101) with ClassicPecletFunction / TanhFunction (src/PecletFunction.C:
// 39-45, 66-71):
//   diff_Ip = 0.5 (mu_L / rho_L + mu_R / rho_R), udotx = 0.5 dx . (u_L + u_R)
//   Pe = |udotx| / (diff_Ip + eps),  f = (hf Pe)^2 / (5 + (hf Pe)^2)
//   or f = 0.5 (1 + tanh((Pe - c1) / c2))
__global__ void __launch_bounds__(kThreads)
    peclet_k(int64_t E, const int2* __restrict__ edges, const double* __restrict__ coords,
             const double* __restrict__ density, const double* __restrict__ viscosity,
             const double* __restrict__ vel, nw_peclet_opts o, dd hf, dd eps,
             double* __restrict__ pecnum, double* __restrict__ pecfac) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int2 lr = edges[e];
  const int64_t L = lr.x, R = lr.y;
  const dd diffIp = scale2(ldd(viscosity + L) * dd_rcp(ldd(density + L)) +
                               ldd(viscosity + R) * dd_rcp(ldd(density + R)),
                           0.5f);
  dd udotx = {0.f, 0.f};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const dd dxj = dd_from_double(coords[3 * R + d] - coords[3 * L + d]);
    udotx = scale2(dxj, 0.5f) * (ldd(vel + 3 * R + d) + ldd(vel + 3 * L + d)) + udotx;
  }
  const dd pe = dd_abs(udotx) * dd_rcp(diffIp + eps);
  if (pecnum) pecnum[e] = dd_to_double(pe);
  double f;
  if (o.tanh_form) {
    f = 0.50 * (1.0 + tanh((dd_to_double(pe) - o.tanh_trans) / o.tanh_width));
  } else {
    const dd m = hf * pe;
    const dd m2 = m * m;
    f = dd_to_double(m2 * dd_rcp(m2 + 5.0f));
  }
  pecfac[e] = f;
}

template <typename F>
nw_status guard_call(F&& f) {
  try {
    f();
    return NW_OK;
  } catch (const Error& e) {
    set_last_error(e.msg);
    return e.status;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return NW_INTERNAL;
  }
}

}  // namespace
}  // namespace nw

using nw::dd;
using nw::dd_from_double;

extern "C" nw_status nw_compute_mdot_edges(nw_linsys* ls, const nw_continuity_fields* f,
                                           double noc_fac, double interp_together,
                                           double* mdot) {
  return nw::guard_call([&] {
    const nw::PlanView v = nw::plan_view(ls);
    if (!f || !mdot) nw::fail(NW_INVALID_ARG, "null argument");
    if (!f->coords || !f->velocity || !f->dpdx || !f->density || !f->pressure || !f->udiag ||
        !f->area)
      nw::fail(NW_INVALID_ARG, "null field pointer");
    if (v.num_edges == 0) return;
    nw::mdot_k<<<nw::grid_for(v.num_edges), nw::kThreads, 0, v.stream>>>(
        v.num_edges, v.edges, f->coords, f->velocity, f->dpdx, f->density, f->pressure,
        f->udiag, f->area, dd_from_double(noc_fac), dd_from_double(interp_together),
        dd_from_double(1.0 - interp_together), mdot);
    NW_CUDA(cudaGetLastError());
  });
}

extern "C" nw_status nw_compute_nodal_gradient(nw_linsys* ls, int dim1, const double* phi,
                                               const double* area, const double* dualvol,
                                               const double* bnd_area, double* grad) {
  return nw::guard_call([&] {
    const nw::PlanView v = nw::plan_view(ls);
    if (!phi || !area || !dualvol || !grad) nw::fail(NW_INVALID_ARG, "null argument");
    if (dim1 != 1 && dim1 != 3) nw::fail(NW_INVALID_ARG, "dim1 must be 1 or 3");
    if (v.node_rows == 0) return;
    if (dim1 == 1)
      nw::nodal_grad_k<1><<<nw::grid_for(v.node_rows), nw::kThreads, 0, v.stream>>>(
          v.node_rows, v.inc_ptr, v.inc, v.edges, v.row_nodes_ptr, v.row_nodes, phi, area,
          dualvol, bnd_area, grad);
    else
      nw::nodal_grad_k<3><<<nw::grid_for(v.node_rows), nw::kThreads, 0, v.stream>>>(
          v.node_rows, v.inc_ptr, v.inc, v.edges, v.row_nodes_ptr, v.row_nodes, phi, area,
          dualvol, bnd_area, grad);
    NW_CUDA(cudaGetLastError());
  });
}

extern "C" nw_status nw_compute_peclet_factor(nw_linsys* ls, const double* coords,
                                              const double* density, const double* viscosity,
                                              const double* velocity, const nw_peclet_opts* o,
                                              double* pecnum, double* pecfac) {
  return nw::guard_call([&] {
    const nw::PlanView v = nw::plan_view(ls);
    if (!coords || !density || !viscosity || !velocity || !o || !pecfac)
      nw::fail(NW_INVALID_ARG, "null argument");
    if (o->tanh_form && !(o->tanh_width != 0.0)) nw::fail(NW_INVALID_ARG, "tanh_width is zero");
    if (v.num_edges == 0) return;
    nw::peclet_k<<<nw::grid_for(v.num_edges), nw::kThreads, 0, v.stream>>>(
        v.num_edges, v.edges, coords, density, viscosity, velocity, *o,
        dd_from_double(o->hybrid_factor), dd_from_double(o->eps), pecnum, pecfac);
    NW_CUDA(cudaGetLastError());
  });
}
