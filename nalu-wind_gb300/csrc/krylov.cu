// Krylov solver kernels and drivers for sm_103a.
//
// Replaces the Belos/Ifpack2 solve behind TpetraLinearSolver::solve
// (src/LinearSolver.C:209-254) with the parameters the reference sets
// (src/LinearSolverConfig.C:37-140): restarted GMRES with "Num Blocks" =
// kspace and iterated classical Gram-Schmidt (two CGS passes), right
// preconditioning (src/LinearSolver.C:110), x0 = 0, and convergence when the
// implicit residual relative to the initial residual norm reaches the
// tolerance. Jacobi and symmetric Gauss-Seidel are one-sweep relaxations
// with zero starting guess; the GPU Gauss-Seidel visits rows colour by
// colour (multicolour ordering), which is sequential Gauss-Seidel in that
// row order.
//
// Sparse kernels use no tensor cores: CSR SpMV assigns a sub-warp to each
// row; reductions are two-stage over a fixed grid, so every dot product is
// bitwise reproducible run to run. Every multiply-add of the FP64 solver
// kernels is an explicit fma and the host-side scalar work is compiled
// without contraction, so the operation order (and rounding) of the FP64
// solvers is fixed by the source and can be restated exactly on a CPU.
//
// The mixed-precision method keeps FP64 for the outer true residual
// (iterative refinement), the Gram-Schmidt dot products and the Hessenberg
// least squares; its inner GMRES stores the basis in FP32 and runs the SpMV
// and the preconditioner in FP32. The inner dot products multiply FP32
// operands exactly (product + FMA error term) and accumulate them with a
// compensated two-float sum (Dekker/Knuth error-free transformations) on
// the FP32 pipes, then combine threads in FP64: FP64-accurate dots without
// spending GB300's scarce FP64 throughput.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "krylov.h"
#include "learned.h"

namespace nw {
namespace {

constexpr int kBlock = 256;
constexpr int kTile = 8;  // vectors per pass of the multi-dot / multi-axpy

// ---------------------------------------------------------------------------
// SpMV: y = A x (or y = b - A x when b != nullptr). LANES threads per row.
template <int LANES, typename VT, typename XT, typename ACC>
__global__ void __launch_bounds__(kBlock)
    spmv_k(int64_t n, const int64_t* __restrict__ rp,
           const int32_t* __restrict__ ci, const VT* __restrict__ v,
           const XT* __restrict__ x, const XT* __restrict__ b,
           XT* __restrict__ y) {
  const int64_t gt = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t row = gt / LANES;
  const int lane = threadIdx.x % LANES;
  if (row >= n) return;
  const int64_t s = rp[row], e = rp[row + 1];
  ACC acc = 0;
  for (int64_t p = s + lane; p < e; p += LANES) acc = fma(ACC(v[p]), ACC(x[ci[p]]), acc);
#pragma unroll
  for (int off = LANES / 2; off > 0; off >>= 1)
    acc += __shfl_down_sync(0xffffffffu, acc, off, LANES);
  if (lane == 0) y[row] = b ? XT(ACC(b[row]) - acc) : XT(acc);
}

// Two-stage Gauss-Seidel step: g_out = D^-1 (r - T g_in), T the strictly
// lower (UPPER false) or upper part of each row in column order. LANES
// threads per row.
template <int LANES, bool UPPER, typename VT, typename T>
__global__ void __launch_bounds__(kBlock)
    ts_tri_k(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
             const VT* __restrict__ v, const T* __restrict__ rd, const T* __restrict__ r,
             const T* __restrict__ gin, T* __restrict__ gout) {
  const int64_t gt = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t row = gt / LANES;
  const int lane = threadIdx.x % LANES;
  if (row >= n) return;
  T acc = 0;
  for (int64_t p = rp[row] + lane; p < rp[row + 1]; p += LANES) {
    const int64_t c = ci[p];
    if (UPPER ? c > row : c < row) acc = fma(T(v[p]), gin[c], acc);
  }
#pragma unroll
  for (int off = LANES / 2; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off, LANES);
  if (lane == 0) gout[row] = rd[row] * (r[row] - acc);
}

template <bool UPPER, typename VT, typename T>
void ts_tri_launch(int lanes, int64_t n, const int64_t* rp, const int32_t* ci, const VT* v,
                   const T* rd, const T* r, const T* gin, T* gout, cudaStream_t s) {
  if (n == 0) return;
  const unsigned grid = unsigned((n * lanes + kBlock - 1) / kBlock);
  switch (lanes) {
    case 4:
      ts_tri_k<4, UPPER, VT, T><<<grid, kBlock, 0, s>>>(n, rp, ci, v, rd, r, gin, gout);
      break;
    case 8:
      ts_tri_k<8, UPPER, VT, T><<<grid, kBlock, 0, s>>>(n, rp, ci, v, rd, r, gin, gout);
      break;
    case 16:
      ts_tri_k<16, UPPER, VT, T><<<grid, kBlock, 0, s>>>(n, rp, ci, v, rd, r, gin, gout);
      break;
    default:
      ts_tri_k<32, UPPER, VT, T><<<grid, kBlock, 0, s>>>(n, rp, ci, v, rd, r, gin, gout);
      break;
  }
}

template <typename VT, typename XT, typename ACC>
void spmv_launch(int lanes, int64_t n, const int64_t* rp, const int32_t* ci,
                 const VT* v, const XT* x, const XT* b, XT* y,
                 cudaStream_t s) {
  if (n == 0) return;
  const int64_t threads = n * lanes;
  const unsigned grid = unsigned((threads + kBlock - 1) / kBlock);
  switch (lanes) {
    case 4:
      spmv_k<4, VT, XT, ACC><<<grid, kBlock, 0, s>>>(n, rp, ci, v, x, b, y);
      break;
    case 8:
      spmv_k<8, VT, XT, ACC><<<grid, kBlock, 0, s>>>(n, rp, ci, v, x, b, y);
      break;
    case 16:
      spmv_k<16, VT, XT, ACC><<<grid, kBlock, 0, s>>>(n, rp, ci, v, x, b, y);
      break;
    default:
      spmv_k<32, VT, XT, ACC><<<grid, kBlock, 0, s>>>(n, rp, ci, v, x, b, y);
      break;
  }
}

// ---------------------------------------------------------------------------
// Sliced-ELL SpMV: one warp per 32-row slice, lane = row; slot k of the
// slice holds row entries k (padding: value 0, column = the row).
template <typename VT, typename XT, typename ACC>
__global__ void __launch_bounds__(kBlock)
    sell_spmv_k(int64_t n, int64_t nslices, const int64_t* __restrict__ off,
                const int32_t* __restrict__ cols, const VT* __restrict__ v,
                const XT* __restrict__ x, const XT* __restrict__ b,
                XT* __restrict__ y) {
  const int64_t sl = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sl >= nslices) return;
  const int64_t o = off[sl];
  const int len = int((off[sl + 1] - o) >> 5);
  const int64_t row = (sl << 5) + lane;
  ACC acc = 0;
  const int32_t* c = cols + o + lane;
  const VT* vv = v + o + lane;
#pragma unroll 4
  for (int k = 0; k < len; ++k) acc = fma(ACC(vv[32 * k]), ACC(x[c[32 * k]]), acc);
  if (row < n) y[row] = b ? XT(ACC(b[row]) - acc) : XT(acc);
}

// values in SELL order (FP64 and optionally FP32) from the CSR values
__global__ void sell_gather_k(int64_t slots, const int32_t* __restrict__ map,
                              const double* __restrict__ csr,
                              double* __restrict__ out64, float* __restrict__ out32) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= slots) return;
  const int32_t p = map[q];
  const double v = p >= 0 ? csr[p] : 0.0;
  out64[q] = v;
  if (out32) out32[q] = float(v);
}

// ---------------------------------------------------------------------------
// Deterministic multi-dot: out[k] = sum_i V[k][i] * w[i] for k < nv.
// Stage 1 writes per-block partials (fixed grid); stage 2 sums them in a
// fixed tree order.
//
// FP32 vectors: every product is formed exactly (p + e with e = fma(a, b,
// -p)) and accumulated as a two-float sum (Knuth two-sum); warp reductions
// combine the pairs on the FP32 pipes and only one value per warp is
// widened to FP64. GB300's FP64 pipe is about 1/58 of its FP32 rate, so
// per-thread FP64 work is kept out of these loops.
struct F2 {
  float s, c;
};
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float x) {
  const float t = s + x;
  const float bp = t - s;
  c += (s - (t - bp)) + (x - bp);
  s = t;
}
__device__ __forceinline__ void acc_prod(double a, double b, double& s,
                                         double& c) {
  s = fma(a, b, s);
  (void)c;
}
__device__ __forceinline__ void acc_prod(float a, float b, float& s,
                                         float& c) {
  const float p = a * b;
  c += fmaf(a, b, -p);
  two_sum_acc(s, c, p);
}
// warp sum of (s, c); result valid in lane 0 as a double
__device__ __forceinline__ double warp_sum(double s, double c) {
  double v = s + c;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}
__device__ __forceinline__ double warp_sum(float s, float c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float os = __shfl_down_sync(0xffffffffu, s, off);
    const float oc = __shfl_down_sync(0xffffffffu, c, off);
    c += oc;
    two_sum_acc(s, c, os);
  }
  return double(s) + double(c);
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
    mdot_k(int64_t n, int nv, const T* __restrict__ V, int64_t ld,
           const T* __restrict__ w, double* __restrict__ partial) {
  __shared__ double red[kTile][kBlock / 32];
  const int G = gridDim.x;
  const int64_t stride = int64_t(G) * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k0 = 0; k0 < nv; k0 += kTile) {
    const int kt = min(kTile, nv - k0);
    T s[kTile], c[kTile];
#pragma unroll
    for (int k = 0; k < kTile; ++k) s[k] = c[k] = T(0);
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    // two elements per step for more loads in flight
    for (; i + stride < n; i += 2 * stride) {
      const T w0 = w[i], w1 = w[i + stride];
      T a0[kTile], a1[kTile];
#pragma unroll
      for (int k = 0; k < kTile; ++k)
        if (k < kt) {
          a0[k] = V[int64_t(k0 + k) * ld + i];
          a1[k] = V[int64_t(k0 + k) * ld + i + stride];
        }
#pragma unroll
      for (int k = 0; k < kTile; ++k)
        if (k < kt) {
          acc_prod(a0[k], w0, s[k], c[k]);
          acc_prod(a1[k], w1, s[k], c[k]);
        }
    }
    if (i < n) {
      const T w0 = w[i];
#pragma unroll
      for (int k = 0; k < kTile; ++k)
        if (k < kt) acc_prod(V[int64_t(k0 + k) * ld + i], w0, s[k], c[k]);
    }
#pragma unroll
    for (int k = 0; k < kTile; ++k) {
      if (k < kt) {
        const double v = warp_sum(s[k], c[k]);
        if (lane == 0) red[k][warp] = v;
      }
    }
    __syncthreads();
    if (threadIdx.x < kt) {
      double v = 0.0;
      for (int q = 0; q < kBlock / 32; ++q) v += red[threadIdx.x][q];
      partial[int64_t(k0 + threadIdx.x) * G + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

// FP32 basis with a padded leading dimension (ld a multiple of 32 floats):
// the multi-dot and multi-axpy below move four consecutive elements per
// thread with 16-byte loads. Elements in [n, ld) are padding and never
// enter a result. The multi-dot forms each group of four products with FP32
// FMAs and adds the group into a compensated (two-float) running sum.
__global__ void __launch_bounds__(kBlock, 6)
    mdot4_k(int64_t n, int nv, const float* __restrict__ V, int64_t ld,
            const float* __restrict__ w, double* __restrict__ partial) {
  __shared__ double red[kTile][kBlock / 32];
  const int G = gridDim.x;
  const int64_t ng = (n + 3) >> 2, full = n >> 2;  // groups of 4; full groups
  const int64_t stride = int64_t(G) * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float4* w4 = reinterpret_cast<const float4*>(w);
  for (int k0 = 0; k0 < nv; k0 += kTile) {
    const int kt = min(kTile, nv - k0);
    float s[kTile], c[kTile];
#pragma unroll
    for (int k = 0; k < kTile; ++k) s[k] = c[k] = 0.f;
    for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < ng; g += stride) {
      float4 wv = w4[g];
      if (g >= full) {  // the last, partial group
        const int64_t i0 = 4 * g;
        if (i0 + 1 >= n) wv.y = 0.f;
        if (i0 + 2 >= n) wv.z = 0.f;
        if (i0 + 3 >= n) wv.w = 0.f;
      }
#pragma unroll
      for (int k = 0; k < kTile; ++k)
        if (k < kt) {
          float4 a = reinterpret_cast<const float4*>(V + int64_t(k0 + k) * ld)[g];
          if (g >= full) {
            const int64_t i0 = 4 * g;
            if (i0 + 1 >= n) a.y = 0.f;
            if (i0 + 2 >= n) a.z = 0.f;
            if (i0 + 3 >= n) a.w = 0.f;
          }
          // the group's four products in FP32 (fused), the running sum
          // compensated: the error is a few ulps of the group's |terms|,
          // not of the whole length-n sum
          const float pg = fmaf(a.x, wv.x, fmaf(a.y, wv.y, fmaf(a.z, wv.z, a.w * wv.w)));
          two_sum_acc(s[k], c[k], pg);
        }
    }
#pragma unroll
    for (int k = 0; k < kTile; ++k) {
      if (k < kt) {
        const double v = warp_sum(s[k], c[k]);
        if (lane == 0) red[k][warp] = v;
      }
    }
    __syncthreads();
    if (threadIdx.x < kt) {
      double v = 0.0;
      for (int q = 0; q < kBlock / 32; ++q) v += red[threadIdx.x][q];
      partial[int64_t(k0 + threadIdx.x) * G + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

// w -= V h for groups of four elements; optional per-block partial sums of
// the updated |w|^2 (elements below n only).
__global__ void __launch_bounds__(kBlock)
    maxpy4_k(int64_t n, int nv, const float* __restrict__ V, int64_t ld,
             const double* __restrict__ h, float* __restrict__ w,
             double* __restrict__ nrm_partial) {
  __shared__ float hs[1024];
  __shared__ double red[kBlock / 32];
  for (int k = threadIdx.x; k < nv; k += blockDim.x) hs[k] = float(h[k]);
  __syncthreads();
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t ng = (n + 3) >> 2;
  float ss = 0.f, cc = 0.f;
  if (g < ng) {
    float4 acc = reinterpret_cast<float4*>(w)[g];
    int k = 0;
    for (; k + 4 <= nv; k += 4) {
      float4 a[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) a[q] = reinterpret_cast<const float4*>(V + int64_t(k + q) * ld)[g];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float hk = hs[k + q];
        acc.x = fmaf(-hk, a[q].x, acc.x);
        acc.y = fmaf(-hk, a[q].y, acc.y);
        acc.z = fmaf(-hk, a[q].z, acc.z);
        acc.w = fmaf(-hk, a[q].w, acc.w);
      }
    }
    for (; k < nv; ++k) {
      const float4 a = reinterpret_cast<const float4*>(V + int64_t(k) * ld)[g];
      const float hk = hs[k];
      acc.x = fmaf(-hk, a.x, acc.x);
      acc.y = fmaf(-hk, a.y, acc.y);
      acc.z = fmaf(-hk, a.z, acc.z);
      acc.w = fmaf(-hk, a.w, acc.w);
    }
    reinterpret_cast<float4*>(w)[g] = acc;
    if (nrm_partial) {
      const int64_t i0 = 4 * g;
      acc_prod(acc.x, acc.x, ss, cc);
      if (i0 + 1 < n) acc_prod(acc.y, acc.y, ss, cc);
      if (i0 + 2 < n) acc_prod(acc.z, acc.z, ss, cc);
      if (i0 + 3 < n) acc_prod(acc.w, acc.w, ss, cc);
    }
  }
  if (!nrm_partial) return;
  const double v = warp_sum(ss, cc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kBlock / 32; ++q) t += red[q];
    nrm_partial[blockIdx.x] = t;
  }
}

// out[k] = sum of partial[k][0..G) (one block per k, fixed tree).
__global__ void reduce_partials_k(int G, const double* __restrict__ partial,
                                  double* __restrict__ out, int mode,
                                  double* __restrict__ aux) {
  __shared__ double sh[kBlock];
  const int k = blockIdx.x;
  double v = 0.0;
  for (int q = threadIdx.x; q < G; q += blockDim.x)
    v += partial[int64_t(k) * G + q];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[k] = sh[0];
    // mode 1: accumulate into aux[k] (second Gram-Schmidt pass)
    if (mode == 1) aux[k] += sh[0];
  }
}

// w -= sum_k h[k] V[k]  (h on the device, FP64), one element per thread.
// The coefficients are converted to the vector precision once per block
// (FP64<->FP32 conversions issue on the narrow FP64 pipe). With
// nrm_partial != nullptr each block also writes the partial ||w||^2 of its
// elements to nrm_partial[blockIdx.x].
constexpr int kMaxVecs = 1024;

template <typename T>
__global__ void __launch_bounds__(kBlock)
    maxpy_k(int64_t n, int nv, const T* __restrict__ V, int64_t ld,
            const double* __restrict__ h, T* __restrict__ w,
            double* __restrict__ nrm_partial) {
  __shared__ T hs[kMaxVecs];
  __shared__ double red[kBlock / 32];
  for (int k = threadIdx.x; k < nv; k += blockDim.x) hs[k] = T(h[k]);
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  T ss = T(0), cc = T(0);
  if (i < n) {
    T acc = w[i];
    int k = 0;
    for (; k + 8 <= nv; k += 8) {
      T a[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) a[q] = V[int64_t(k + q) * ld + i];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc = fma(-hs[k + q], a[q], acc);
    }
    for (; k < nv; ++k) acc = fma(-hs[k], V[int64_t(k) * ld + i], acc);
    w[i] = acc;
    if (nrm_partial) acc_prod(acc, acc, ss, cc);
  }
  if (!nrm_partial) return;
  const double v = warp_sum(ss, cc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kBlock / 32; ++q) t += red[q];
    nrm_partial[blockIdx.x] = t;
  }
}

__global__ void sqrt_scalar_k(double* s) { s[0] = sqrt(s[0]); }

// v32 = float(r / nrm[0]) (start of an inner FP32 cycle).
__global__ void scale_to_f32_k(int64_t n, const double* __restrict__ r,
                               float* __restrict__ v, const double* __restrict__ nrm) {
  __shared__ double inv;
  if (threadIdx.x == 0) inv = nrm[0] != 0.0 ? 1.0 / nrm[0] : 0.0;
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) v[i] = float(r[i] * inv);
}

template <typename T>
__global__ void jacobi_k(int64_t n, const T* __restrict__ rd,
                         const T* __restrict__ x, T* __restrict__ y) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * rd[i];
}

// v = w / nrm[0] and, when rd is given, z = rd * v (the Jacobi application
// of the next Arnoldi step) in the same pass.
template <typename T>
__global__ void scale_jacobi_k(int64_t n, const T* __restrict__ w,
                               T* __restrict__ v, const double* __restrict__ nrm,
                               const T* __restrict__ rd, T* __restrict__ z) {
  __shared__ T inv;
  if (threadIdx.x == 0) {
    const double hn = nrm[0];
    inv = T(hn != 0.0 ? 1.0 / hn : 0.0);
  }
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T vi = w[i] * inv;
  v[i] = vi;
  if (rd) z[i] = vi * rd[i];
}

constexpr int kGsBatch = 8;

// One colour class of the Gauss-Seidel sweep over the class-ordered sliced
// copy (off-diagonal entries only, same column order as the CSR row):
//   y_i = (x_i - sum_{j != i} a_ij y_j) / a_ii
// `first`: every y_j is still zero, so y_i = x_i / a_ii without the sum.
template <typename VT, typename T>
__global__ void __launch_bounds__(kBlock)
    gs_sell_k(int64_t cnt, const int32_t* __restrict__ rows,
              const int64_t* __restrict__ off, const int32_t* __restrict__ len,
              const int32_t* __restrict__ cols, const VT* __restrict__ v,
              const T* __restrict__ rd, const T* __restrict__ x, T* __restrict__ y,
              int first) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t i = rows[k];
  T s = x[i];
  if (!first) {
    const int64_t base = off[k >> 5] + (k & 31);
    const int n = len[k];
    // batches of kGsBatch entries: every column and value load of the batch
    // first, then every y gather, then the multiply-adds in column order
    // (the same sum as one entry at a time, with the loads in flight
    // together instead of one dependent pair per entry)
    for (int q = 0; q < n; q += kGsBatch) {
      int32_t c[kGsBatch];
      T a[kGsBatch], yv[kGsBatch];
#pragma unroll
      for (int j = 0; j < kGsBatch; ++j) {
        const int64_t p = base + 32 * int64_t(q + j);
        c[j] = q + j < n ? cols[p] : i;
        a[j] = q + j < n ? T(v[p]) : T(0);
      }
#pragma unroll
      for (int j = 0; j < kGsBatch; ++j) yv[j] = q + j < n ? y[c[j]] : T(0);
#pragma unroll
      for (int j = 0; j < kGsBatch; ++j)
        if (q + j < n) s = fma(-a[j], yv[j], s);
    }
  }
  y[i] = s * rd[i];
}

// Residual r_i = x_i - a_ii y_i - sum_{j != i} a_ij y_j of the rows of one
// colour class (float, over the class-ordered sliced copy).
__global__ void __launch_bounds__(kBlock)
    gs_resid_k(int64_t cnt, const int32_t* __restrict__ rows, const int64_t* __restrict__ off,
               const int32_t* __restrict__ len, const int32_t* __restrict__ cols,
               const float* __restrict__ v, const float* __restrict__ diag,
               const float* __restrict__ x, const float* __restrict__ y, float* __restrict__ r) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t i = rows[k];
  float s = fmaf(-diag[i], y[i], x[i]);
  const int64_t base = off[k >> 5] + (k & 31);
  const int n = len[k];
  for (int q = 0; q < n; q += kGsBatch) {  // batched loads as in gs_sell_k
    int32_t c[kGsBatch];
    float a[kGsBatch], yv[kGsBatch];
#pragma unroll
    for (int j = 0; j < kGsBatch; ++j) {
      const int64_t p = base + 32 * int64_t(q + j);
      c[j] = q + j < n ? cols[p] : i;
      a[j] = q + j < n ? v[p] : 0.f;
    }
#pragma unroll
    for (int j = 0; j < kGsBatch; ++j) yv[j] = q + j < n ? y[c[j]] : 0.f;
#pragma unroll
    for (int j = 0; j < kGsBatch; ++j)
      if (q + j < n) s = fmaf(-a[j], yv[j], s);
  }
  r[i] = s;
}

__global__ void to_bf16_vals_k(int64_t n, const float* __restrict__ a, __nv_bfloat16* __restrict__ b) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

__global__ void zero_rows_k(int64_t cnt, const int32_t* __restrict__ rows, float* __restrict__ r) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < cnt) r[rows[k]] = 0.f;
}

template <typename T>
__global__ void fill_k(int64_t n, T* y, T val) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = val;
}

__global__ void rdiag_k(int64_t n, const int64_t* __restrict__ rp,
                        const int32_t* __restrict__ ci,
                        const double* __restrict__ v, double* __restrict__ rd,
                        float* __restrict__ d32) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int64_t p = rp[i]; p < rp[i + 1]; ++p)
    if (ci[p] == i) d = v[p];
  rd[i] = 1.0 / d;
  if (d32) d32[i] = float(d);
}

template <typename A, typename B>
__global__ void convert_k(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = B(a[i]);
}

// y = a - y (FP32)
// x += alpha * y (FP64)
__global__ void axpy_k(int64_t n, double alpha, const double* __restrict__ y,
                       double* __restrict__ x) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] = fma(alpha, y[i], x[i]);
}
// x += y (y FP32), mixed correction
__global__ void add_f32_k(int64_t n, const float* __restrict__ y,
                          double* __restrict__ x) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] += double(y[i]);
}
// y += x
template <typename T>
__global__ void axpy_t_k(int64_t n, const T* __restrict__ x, T* __restrict__ y) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}
// out = a x + b y (out may alias x or y)
__global__ void lincomb_k(int64_t n, double a, const double* x, double b, const double* y, double* out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = fma(a, x[i], b * y[i]);
}
// BiCGStab direction: p = r + beta (p - omega v)
__global__ void bicg_dir_k(int64_t n, const double* __restrict__ r, double beta, double omega,
                           const double* __restrict__ v, double* __restrict__ p) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(beta, fma(-omega, v[i], p[i]), r[i]);
}
// BiCGStab update: x += alpha ph + omega sh; r = s - omega t
__global__ void bicg_upd_k(int64_t n, double alpha, const double* __restrict__ ph, double omega,
                           const double* __restrict__ sh, const double* __restrict__ sv,
                           const double* __restrict__ t, double* __restrict__ x,
                           double* __restrict__ r) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) {
    x[i] = fma(omega, sh[i], fma(alpha, ph[i], x[i]));
    r[i] = fma(-omega, t[i], sv[i]);
  }
}
// TFQMR half step: w -= alpha Au; dh = uh + coef dh
__global__ void tfqmr_wd_k(int64_t n, double alpha, const double* __restrict__ Au, double coef,
                           const double* __restrict__ uh, double* __restrict__ w,
                           double* __restrict__ dh) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) {
    w[i] = fma(-alpha, Au[i], w[i]);
    dh[i] = fma(coef, dh[i], uh[i]);
  }
}
// TFQMR: v = Aun + beta (Au + beta v)
__global__ void tfqmr_v_k(int64_t n, const double* __restrict__ Aun, double beta,
                          const double* __restrict__ Au, double* __restrict__ v) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) v[i] = fma(beta, fma(beta, v[i], Au[i]), Aun[i]);
}
// p = z + beta p
__global__ void xpby_k(int64_t n, const double* __restrict__ z, double beta,
                       double* __restrict__ p) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(beta, p[i], z[i]);
}
// y = sum_k c[k] V[k] (c in a device array), in the vector precision.
template <typename T>
__global__ void combine_k(int64_t n, int nv, const T* __restrict__ V,
                          int64_t ld, const double* __restrict__ c,
                          T* __restrict__ y) {
  __shared__ T cs[kMaxVecs];
  for (int k = threadIdx.x; k < nv; k += blockDim.x) cs[k] = T(c[k]);
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T acc = T(0);
  for (int k = 0; k < nv; ++k) acc = fma(cs[k], V[int64_t(k) * ld + i], acc);
  y[i] = acc;
}

inline unsigned grid1(int64_t n) { return unsigned((n + kBlock - 1) / kBlock); }

// Explicitly rounded scalar operations (no contraction into fused
// multiply-adds), so that the level-scheduled sweeps below round exactly as
// a sequential restatement of the same loops does.
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }

// One level of the natural-order Gauss-Seidel sweep (Ifpack2 "Symmetric
// Gauss-Seidel"): y_i = (x_i - sum_{j != i} a_ij y_j) / a_ii over the row's
// entries in column order. The level schedule guarantees that in the
// forward sweep every y_j with j > i in the row is still zero and in the
// backward sweep every y_j with j < i still holds its forward value.
template <typename VT, typename T>
__global__ void __launch_bounds__(kBlock)
    gs_level_k(int64_t cnt, const int32_t* __restrict__ rows, const int64_t* __restrict__ rp,
               const int32_t* __restrict__ ci, const VT* __restrict__ v,
               const int64_t* __restrict__ dpos, const T* __restrict__ x, T* __restrict__ y) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int64_t i = rows[k];
  T s = x[i];
  for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
    const int64_t c = ci[p];
    if (c != i) s = rn_sub(s, rn_mul(T(v[p]), y[c]));
  }
  y[i] = rn_div(s, T(v[dpos[i]]));
}

// ILU(0) factorization of the rows of one forward level (IKJ order, Saad,
// Iterative Methods for Sparse Linear Systems, Algorithm 10.4): for each
// entry k < i of row i in column order, l_ik = a_ik / u_kk, then
// a_ij -= l_ik u_kj for the row's entries j > k present in row k. Rows k < i
// of the pattern lie on earlier levels and are final.
__global__ void __launch_bounds__(kBlock)
    ilu0_level_k(int64_t cnt, const int32_t* __restrict__ rows, const int64_t* __restrict__ rp,
                 const int32_t* __restrict__ ci, const int64_t* __restrict__ dpos,
                 double* __restrict__ lu) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int64_t i = rows[t];
  const int64_t e = rp[i + 1];
  for (int64_t p = rp[i]; p < e; ++p) {
    const int64_t k = ci[p];
    if (k >= i) break;
    const double l = rn_div(lu[p], lu[dpos[k]]);
    lu[p] = l;
    int64_t qk = dpos[k] + 1;
    const int64_t ek = rp[k + 1];
    for (int64_t q = p + 1; q < e; ++q) {
      const int64_t j = ci[q];
      while (qk < ek && ci[qk] < j) ++qk;
      if (qk < ek && ci[qk] == j) lu[q] = rn_sub(lu[q], rn_mul(l, lu[qk]));
    }
  }
}

// One level of the ILU(0) triangular solves: forward (unit L)
// y_i = x_i - sum_{k < i} l_ik y_k; backward (U, in place)
// y_i = (y_i - sum_{j > i} u_ij y_j) / u_ii.
template <bool UPPER, typename T>
__global__ void __launch_bounds__(kBlock)
    ilu0_solve_level_k(int64_t cnt, const int32_t* __restrict__ rows, const int64_t* __restrict__ rp,
                       const int32_t* __restrict__ ci, const int64_t* __restrict__ dpos,
                       const T* __restrict__ lu, const T* __restrict__ x, T* __restrict__ y) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int64_t i = rows[t];
  if (!UPPER) {
    T s = x[i];
    for (int64_t p = rp[i]; p < dpos[i]; ++p) s = rn_sub(s, rn_mul(lu[p], y[ci[p]]));
    y[i] = s;
  } else {
    T s = y[i];
    for (int64_t p = dpos[i] + 1; p < rp[i + 1]; ++p) s = rn_sub(s, rn_mul(lu[p], y[ci[p]]));
    y[i] = rn_div(s, lu[dpos[i]]);
  }
}

// ---------------------------------------------------------------------------
// GMRES least squares on the device. One thread applies the previous
// Givens rotations to the new Hessenberg column, forms the next rotation,
// updates the rotated rhs g and the residual estimate, and records
// convergence; the host reads the control words one chunk of iterations
// behind instead of waiting for every column. Every operation is an
// explicitly rounded FP64 add, multiply, divide or square root (no fused
// multiply-adds), the same arithmetic as the host restatement of the
// solver, so iterates and histories do not depend on where it runs.
struct GivensDev {
  double *H, *cs, *sn, *g, *hist;
  int* ctl;  // done, iterations of the cycle, status, basis vectors
  int m;
};
enum { kCtlDone = 0, kCtlIts = 1, kCtlStatus = 2, kCtlBasis = 3 };

__global__ void givens_init_k(GivensDev G, double g0) {
  if (threadIdx.x != 0) return;
  for (int k = 0; k <= G.m; ++k) G.g[k] = 0.0;
  G.g[0] = g0;
  G.ctl[kCtlDone] = 0;
  G.ctl[kCtlIts] = 0;
  G.ctl[kCtlStatus] = NW_OK;
  G.ctl[kCtlBasis] = 0;
}

// Column j: h = hs[0..j], hn = ||w||. rel = |g[j+1]| / div; the history
// entry is rel * hist_mul / hist_div; the cycle stops when rel <= tol or
// hn == 0 (basis j + 1), on a non-finite estimate (basis j + 1) or when the
// rotation breaks down (basis j).
__global__ void givens_step_k(GivensDev G, int j, const double* __restrict__ hs,
                              const double* __restrict__ hnp, double tol, double div,
                              double hist_mul, double hist_div) {
  if (threadIdx.x != 0 || G.ctl[kCtlDone]) return;
  const int m = G.m;
  double* H = G.H;
  const double hn = hnp[0];
  for (int k = 0; k <= j; ++k) H[size_t(k) * m + j] = hs[k];
  H[size_t(j + 1) * m + j] = hn;
  for (int k = 0; k < j; ++k) {
    const double a = H[size_t(k) * m + j], bb = H[size_t(k + 1) * m + j];
    H[size_t(k) * m + j] = __dadd_rn(__dmul_rn(G.cs[k], a), __dmul_rn(G.sn[k], bb));
    H[size_t(k + 1) * m + j] = __dadd_rn(__dmul_rn(-G.sn[k], a), __dmul_rn(G.cs[k], bb));
  }
  const double a = H[size_t(j) * m + j], bb = H[size_t(j + 1) * m + j];
  const double den = __dsqrt_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(bb, bb)));
  if (!(den > 0.0) || !isfinite(den)) {
    G.ctl[kCtlStatus] = isfinite(den) ? NW_BREAKDOWN : NW_NAN_DETECTED;
    G.ctl[kCtlBasis] = j;
    G.ctl[kCtlDone] = 1;
    return;
  }
  G.cs[j] = __ddiv_rn(a, den);
  G.sn[j] = __ddiv_rn(bb, den);
  H[size_t(j) * m + j] = den;
  H[size_t(j + 1) * m + j] = 0.0;
  G.g[j + 1] = __dmul_rn(-G.sn[j], G.g[j]);
  G.g[j] = __dmul_rn(G.cs[j], G.g[j]);
  G.ctl[kCtlIts] = j + 1;
  const double rel = __ddiv_rn(fabs(G.g[j + 1]), div);
  G.hist[j] = __ddiv_rn(__dmul_rn(rel, hist_mul), hist_div);
  if (!isfinite(rel)) {
    G.ctl[kCtlStatus] = NW_NAN_DETECTED;
    G.ctl[kCtlBasis] = j + 1;
    G.ctl[kCtlDone] = 1;
  } else if (rel <= tol || hn == 0.0) {
    G.ctl[kCtlBasis] = j + 1;
    G.ctl[kCtlDone] = 1;
  }
}

// Back substitution H(0:kk, 0:kk) y = g(0:kk), y scaled by yscale, into y.
__global__ void givens_solve_k(GivensDev G, int kk, double yscale, double* __restrict__ y) {
  if (threadIdx.x != 0) return;
  const int m = G.m;
  for (int i = kk - 1; i >= 0; --i) {
    double sum = G.g[i];
    for (int l = i + 1; l < kk; ++l) sum = __dsub_rn(sum, __dmul_rn(G.H[size_t(i) * m + l], y[l]));
    y[i] = __ddiv_rn(sum, G.H[size_t(i) * m + i]);
  }
  if (yscale != 1.0)
    for (int i = 0; i < kk; ++i) y[i] = __dmul_rn(y[i], yscale);
}

}  // namespace

template <typename StepFn>
KrylovSolver::Cycle KrylovSolver::run_cycle(int m, int max_steps, double g0, double tol, double div,
                                            double hist_mul, double hist_div, StepFn arnoldi,
                                            const double* hs, const double* hn, cudaStream_t s,
                                            bool graph) {
  constexpr int kChunk = 2;  // iterations per poll; the host waits one chunk behind
  GivensDev G{gst_.p,
              gst_.p + size_t(m_ + 1) * m_,
              gst_.p + size_t(m_ + 1) * m_ + m_,
              gst_.p + size_t(m_ + 1) * m_ + 2 * m_,
              gst_.p + size_t(m_ + 1) * m_ + 3 * m_ + 1,
              gctl_.p, m_};
  givens_init_k<<<1, 32, 0, s>>>(G, g0);
  int launched = 0, pending = -1, slot = 0;
  bool stop = false;
  auto step = [&](int j) {
    arnoldi(j);
    givens_step_k<<<1, 32, 0, s>>>(G, j, hs, hn, tol, div, hist_mul, hist_div);
  };
  for (int j = 0; j < m && launched < max_steps && !stop; ++j) {
    // the first step of a cycle runs as plain launches: any one-time set-up
    // (buffer growth) happens there, outside a capture. A stream that cannot
    // be captured (the legacy default stream) keeps plain launches.
    if (graph && j > 0 && cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      graph = false;
    }
    if (graph && j > 0) {
      cudaGraph_t g = nullptr;
      try {
        step(j);
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      NW_CUDA(cudaStreamEndCapture(s, &g));
      if (iter_exec_) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(iter_exec_, g, &info) != cudaSuccess) {
          cudaGetLastError();  // a different node layout: instantiate anew
          cudaGraphExecDestroy(iter_exec_);
          iter_exec_ = nullptr;
        }
      }
      if (!iter_exec_) {
        const cudaError_t e = cudaGraphInstantiate(&iter_exec_, g, 0);
        if (e != cudaSuccess) {
          cudaGraphDestroy(g);
          iter_exec_ = nullptr;
          NW_CUDA(e);
        }
      }
      cudaGraphDestroy(g);
      NW_CUDA(cudaGraphLaunch(iter_exec_, s));
    } else {
      step(j);
    }
    ++launched;
    if (launched % kChunk == 0) {
      NW_CUDA(cudaMemcpyAsync(ctl_pinned_ + 4 * slot, gctl_.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaEventRecord(chunk_ev_[slot], s));
      if (pending >= 0) {
        NW_CUDA(cudaEventSynchronize(chunk_ev_[pending]));
        stop = ctl_pinned_[4 * pending + kCtlDone] != 0;
      }
      pending = slot;
      slot ^= 1;
    }
  }
  NW_CUDA(cudaGetLastError());
  NW_CUDA(cudaMemcpyAsync(ctl_pinned_ + 8, gctl_.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
  NW_CUDA(cudaMemcpyAsync(h_pinned_ + 1024, G.hist, sizeof(double) * std::max(1, launched),
                          cudaMemcpyDeviceToHost, s));
  NW_CUDA(cudaStreamSynchronize(s));
  Cycle c;
  c.done = ctl_pinned_[8 + kCtlDone] != 0;
  c.iterations = ctl_pinned_[8 + kCtlIts];
  c.status = nw_status(ctl_pinned_[8 + kCtlStatus]);
  c.basis = c.done ? ctl_pinned_[8 + kCtlBasis] : launched;
  c.hist.assign(h_pinned_ + 1024, h_pinned_ + 1024 + c.iterations);
  return c;
}

namespace {
// y on the device from the cycle's least squares (launch helper)
void cycle_solution(double* gst, int* gctl, int m, int kk, double yscale, double* y, cudaStream_t s) {
  GivensDev G{gst, gst + size_t(m + 1) * m, gst + size_t(m + 1) * m + m, gst + size_t(m + 1) * m + 2 * m,
              gst + size_t(m + 1) * m + 3 * m + 1, gctl, m};
  givens_solve_k<<<1, 32, 0, s>>>(G, kk, yscale, y);
}
}  // namespace


// ---------------------------------------------------------------------------
KrylovSolver::~KrylovSolver() {
  if (iter_exec_) cudaGraphExecDestroy(iter_exec_);
  if (h_pinned_) cudaFreeHost(h_pinned_);
  if (ctl_pinned_) cudaFreeHost(ctl_pinned_);
  for (cudaEvent_t& e : chunk_ev_)
    if (e) cudaEventDestroy(e);
}

void KrylovSolver::setup(const DevCsr& A, int m, cudaStream_t s) {
  A_ = A;
  m_ = std::max(1, m);
  const int64_t n = A.n;
  int dev = 0;
  NW_CUDA(cudaGetDevice(&dev));
  int sms = 0;
  NW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  red_blocks_ = int(std::max<int64_t>(1, std::min<int64_t>(8 * sms, (n + 2 * kBlock - 1) / (2 * kBlock))));
  // the FP32 multi-dot holds 16 accumulators per thread: size its grid to
  // the blocks that are resident at once (one wave of its grid-stride loop)
  int occ = 0;
  NW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mdot4_k, kBlock, 0));
  mdot4_blocks_ = std::max(1, std::min(red_blocks_, std::max(1, occ) * sms));
  rdiag_.resize(n);
  V_.resize(size_t(m_ + 1) * n);
  Z_.release();
  w_.resize(n);
  z_.resize(n);
  r_.resize(n);
  partial_.resize(std::max<size_t>(size_t(m_ + 2) * red_blocks_, size_t(grid1(n))));
  scal_.resize(4 * (m_ + 4));
  if (!h_pinned_) NW_CUDA(cudaMallocHost(&h_pinned_, sizeof(double) * 4 * 1024));
  if (!ctl_pinned_) NW_CUDA(cudaMallocHost(&ctl_pinned_, sizeof(int) * 12));
  for (cudaEvent_t& e : chunk_ev_)
    if (!e) NW_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  gst_.resize(size_t(m_ + 1) * m_ + 4 * size_t(m_) + 1);
  gctl_.resize(4);
  // sliced-ELL layout from the host CSR
  sell_slices_ = 0;
  if (A.row_ptr_host && A.col_idx_host && n > 0) {
    const int64_t ns = (n + 31) / 32;
    std::vector<int64_t> off(ns + 1, 0);
    for (int64_t sl = 0; sl < ns; ++sl) {
      int64_t len = 0;
      for (int64_t r = sl * 32; r < std::min(n, sl * 32 + 32); ++r)
        len = std::max(len, A.row_ptr_host[r + 1] - A.row_ptr_host[r]);
      off[sl + 1] = off[sl] + 32 * len;
    }
    if (off[ns] < (int64_t(1) << 31)) {
      std::vector<int32_t> cols(off[ns]), map(off[ns]);
      for (int64_t sl = 0; sl < ns; ++sl) {
        const int64_t len = (off[sl + 1] - off[sl]) / 32;
        for (int lane = 0; lane < 32; ++lane) {
          const int64_t r = sl * 32 + lane;
          for (int64_t k = 0; k < len; ++k) {
            const int64_t q = off[sl] + 32 * k + lane;
            const int64_t p = r < n ? A.row_ptr_host[r] + k : -1;
            if (r < n && p < A.row_ptr_host[r + 1]) {
              cols[q] = A.col_idx_host[p];
              map[q] = int32_t(p);
            } else {
              cols[q] = int32_t(r < n ? r : 0);
              map[q] = -1;
            }
          }
        }
      }
      sell_off_.upload(off, s);
      sell_cols_.upload(cols, s);
      sell_map_.upload(map, s);
      sell_vals_.resize(off[ns]);
      sell_slices_ = ns;
    }
  }
  f32_valid_ = false;
  refresh(s);
}

void KrylovSolver::refresh(cudaStream_t s) {
  if (A_.n == 0) return;
  rdiag_k<<<grid1(A_.n), kBlock, 0, s>>>(A_.n, A_.row_ptr, A_.col_idx,
                                          A_.values, rdiag_.p, nullptr);
  if (sell_slices_)
    sell_gather_k<<<grid1(int64_t(sell_vals_.n)), kBlock, 0, s>>>(
        int64_t(sell_vals_.n), sell_map_.p, A_.values, sell_vals_.p, nullptr);
  if (gs_map_.n)
    sell_gather_k<<<grid1(int64_t(gs_map_.n)), kBlock, 0, s>>>(
        int64_t(gs_map_.n), gs_map_.p, A_.values, gs_vals_.p, nullptr);
  if (cl_) cl_->refresh(A_.values, s);
  NW_CUDA(cudaGetLastError());
  f32_valid_ = false;
  ilu_valid_ = false;
  gs_vals16_.release();
}

void KrylovSolver::ensure_f32(cudaStream_t s) {
  if (f32_valid_) return;
  const int64_t n = A_.n;
  vals32_.resize(A_.nnz);
  rdiag32_.resize(n);
  ld32_ = (n + 31) / 32 * 32;
  V32_.resize(size_t(m_ + 1) * ld32_);
  w32_.resize(ld32_);
  z32_.resize(n);
  r32_.resize(n);
  convert_k<double, float><<<grid1(A_.nnz), kBlock, 0, s>>>(A_.nnz, A_.values,
                                                             vals32_.p);
  if (sell_slices_) {
    sell_vals32_.resize(sell_vals_.n);
    sell_gather_k<<<grid1(int64_t(sell_vals_.n)), kBlock, 0, s>>>(
        int64_t(sell_vals_.n), sell_map_.p, A_.values, sell_vals_.p, sell_vals32_.p);
  }
  if (gs_map_.n) {
    gs_vals32_.resize(gs_map_.n);
    convert_k<double, float><<<grid1(int64_t(gs_map_.n)), kBlock, 0, s>>>(
        int64_t(gs_map_.n), gs_vals_.p, gs_vals32_.p);
  }
  convert_k<double, float><<<grid1(n), kBlock, 0, s>>>(n, rdiag_.p, rdiag32_.p);
  diag32_.resize(n);
  {
    DeviceArray<double> tmp;
    tmp.resize(n);
    rdiag_k<<<grid1(n), kBlock, 0, s>>>(n, A_.row_ptr, A_.col_idx, A_.values, tmp.p, diag32_.p);
    NW_CUDA(cudaStreamSynchronize(s));
  }
  NW_CUDA(cudaGetLastError());
  f32_valid_ = true;
}

void KrylovSolver::spmv(const double* x, double* y, cudaStream_t s) const {
  spmv64(x, nullptr, y, s);
}

// y = A x (b == nullptr) or y = b - A x, FP64
void KrylovSolver::spmv64(const double* x, const double* b, double* y,
                          cudaStream_t s) const {
  if (sell_slices_) {
    const int64_t threads = sell_slices_ * 32;
    sell_spmv_k<double, double, double><<<unsigned((threads + kBlock - 1) / kBlock), kBlock, 0, s>>>(
        A_.n, sell_slices_, sell_off_.p, sell_cols_.p, sell_vals_.p, x, b, y);
  } else {
    spmv_launch<double, double, double>(A_.lanes, A_.n, A_.row_ptr, A_.col_idx,
                                        A_.values, x, b, y, s);
  }
}

// FP32 SpMV of the mixed method (FP32 values and accumulation)
void KrylovSolver::spmv32(const float* x, float* y, cudaStream_t s) const {
  if (sell_slices_ && sell_vals32_.n) {
    const int64_t threads = sell_slices_ * 32;
    sell_spmv_k<float, float, float><<<unsigned((threads + kBlock - 1) / kBlock), kBlock, 0, s>>>(
        A_.n, sell_slices_, sell_off_.p, sell_cols_.p, sell_vals32_.p, x, nullptr, y);
  } else {
    spmv_launch<float, float, float>(A_.lanes, A_.n, A_.row_ptr, A_.col_idx,
                                     vals32_.p, x, nullptr, y, s);
  }
}

double KrylovSolver::dot(const double* a, const double* b, cudaStream_t s) {
  mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(A_.n, 1, a, 0, b, partial_.p);
  reduce_partials_k<<<1, kBlock, 0, s>>>(red_blocks_, partial_.p, scal_.p, 0,
                                         nullptr);
  NW_CUDA(cudaMemcpyAsync(h_pinned_, scal_.p, sizeof(double),
                          cudaMemcpyDeviceToHost, s));
  NW_CUDA(cudaStreamSynchronize(s));
  return h_pinned_[0];
}

namespace {

template <typename VT, typename T>
void precond_apply_t(const Precond& pc, int64_t n, const int64_t* rp,
                     const int32_t* ci, const VT* v, const T* rd, const T* x,
                     T* y, cudaStream_t s) {
  if (pc.kind == NW_PC_NONE) {
    NW_CUDA(cudaMemcpyAsync(y, x, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  } else if (pc.kind == NW_PC_JACOBI) {
    jacobi_k<T><<<grid1(n), kBlock, 0, s>>>(n, rd, x, y);
  } else {
    fail(NW_INVALID_ARG, "preconditioner not available for this precision");
  }
  NW_CUDA(cudaGetLastError());
}

// The learned preconditioner is given up (and the solve repeated with
// SGS) when kStallCycles restart cycles in a row each reduce the true
// residual by less than a factor kStallRatio.
constexpr int kStallCycles = 5;
constexpr double kStallRatio = 0.99;
bool stalled(int& stalls, double rnorm, double prev) {
  stalls = rnorm > kStallRatio * prev ? stalls + 1 : 0;
  return stalls >= kStallCycles;
}

}  // namespace

// Symmetric multicolour Gauss-Seidel, y = M^-1 x: forward over the colour
// classes, then backward. The first class of the forward sweep reads only
// zeros (y = x / diag); the last forward class is not repeated at the start
// of the backward sweep (its rows would be recomputed from the same values,
// giving the same bits). With at most two classes nothing reads a y value
// before it is written, so y needs no zero fill.
template <typename VT, typename T>
void KrylovSolver::sgs(const VT* vals, const T* rd, const T* x, T* y, cudaStream_t s,
                       bool from_guess, int sweep) const {
  const int nc = int(gs_cptr_.size()) - 1;
  if (nc < 1) fail(NW_INTERNAL, "Gauss-Seidel colour classes not set up");
  // sweep 0: symmetric (forward then backward); 1: forward only; 2: backward only
  if (nc > 2 && !from_guess) fill_k<T><<<grid1(A_.n), kBlock, 0, s>>>(A_.n, y, T(0));
  auto pass = [&](int c, int first) {
    const int64_t b = gs_cptr_[c], cnt = gs_cptr_[c + 1] - b;
    if (cnt)
      gs_sell_k<VT, T><<<grid1(cnt), kBlock, 0, s>>>(cnt, gs_rows_.p + b, gs_off_.p + gs_slice0_[c],
                                                     gs_len_.p + b, gs_cols_.p, vals, rd, x, y,
                                                     first);
  };
  if (sweep == 2) {
    for (int c = nc - 1; c >= 0; --c) pass(c, c == nc - 1 && !from_guess);
  } else {
    for (int c = 0; c < nc; ++c) pass(c, c == 0 && !from_guess);
    if (sweep == 0)
      for (int c = nc - 2; c >= 0; --c) pass(c, 0);
  }
  NW_CUDA(cudaGetLastError());
}

// r = x - A y after a sweep that produced y: the rows of the class relaxed
// last (`last`) have a zero residual (up to the reciprocal's rounding) and
// get exactly 0; the other classes are evaluated over the sliced copy.
void KrylovSolver::sgs_residual32(const float* x, const float* y, float* r, cudaStream_t s,
                                  int last) const {
  const int nc = int(gs_cptr_.size()) - 1;
  {
    const int64_t b = gs_cptr_[last], cnt = gs_cptr_[last + 1] - b;
    if (cnt) zero_rows_k<<<grid1(cnt), kBlock, 0, s>>>(cnt, gs_rows_.p + b, r);
  }
  for (int c = 0; c < nc; ++c) {
    if (c == last) continue;
    const int64_t b = gs_cptr_[c], cnt = gs_cptr_[c + 1] - b;
    if (cnt)
      gs_resid_k<<<grid1(cnt), kBlock, 0, s>>>(cnt, gs_rows_.p + b, gs_off_.p + gs_slice0_[c],
                                               gs_len_.p + b, gs_cols_.p, gs_vals32_.p, diag32_.p,
                                               x, y, r);
  }
  NW_CUDA(cudaGetLastError());
}

void KrylovSolver::setup_colors(const std::vector<int32_t>& rows,
                                const std::vector<int64_t>& cptr, cudaStream_t s) {
  const int64_t n = A_.n;
  if (!A_.row_ptr_host || (!A_.col_idx_host && A_.nnz > 0)) fail(NW_INTERNAL, "host graph needed");
  if (int64_t(rows.size()) != n || cptr.empty() || cptr.back() != n)
    fail(NW_INTERNAL, "colour classes do not cover the rows");
  const int nc = int(cptr.size()) - 1;
  gs_cptr_ = cptr;
  gs_slice0_.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) gs_slice0_[c + 1] = gs_slice0_[c] + (cptr[c + 1] - cptr[c] + 31) / 32;
  const int64_t ns = gs_slice0_[nc];
  std::vector<int32_t> len(n, 0);
  std::vector<int64_t> off(ns + 1, 0);
  for (int c = 0; c < nc; ++c)
    for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) {
      const int32_t i = rows[k];
      int32_t cnt = 0;
      for (int64_t p = A_.row_ptr_host[i]; p < A_.row_ptr_host[i + 1]; ++p)
        cnt += A_.col_idx_host[p] != i;
      len[k] = cnt;
      const int64_t sl = gs_slice0_[c] + (k - cptr[c]) / 32;
      off[sl + 1] = std::max<int64_t>(off[sl + 1], 32 * int64_t(cnt));
    }
  for (int64_t sl = 0; sl < ns; ++sl) off[sl + 1] += off[sl];
  std::vector<int32_t> cols(off[ns], 0), map(off[ns], -1);
  for (int c = 0; c < nc; ++c)
    for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) {
      const int32_t i = rows[k];
      const int64_t kl = k - cptr[c];
      const int64_t base = off[gs_slice0_[c] + kl / 32] + (kl & 31);
      int64_t q = 0;
      for (int64_t p = A_.row_ptr_host[i]; p < A_.row_ptr_host[i + 1]; ++p) {
        if (A_.col_idx_host[p] == i) continue;
        cols[base + 32 * q] = A_.col_idx_host[p];
        map[base + 32 * q] = int32_t(p);
        ++q;
      }
    }
  gs_rows_.upload(rows, s);
  gs_len_.upload(len, s);
  gs_off_.upload(off, s);
  gs_cols_.upload(cols, s);
  gs_map_.upload(map, s);
  gs_vals_.resize(std::max<int64_t>(off[ns], 1));
  gs_vals32_.release();
  f32_valid_ = false;
}

// Pre-smoothing of the learned cycle (also used when harvesting pairs):
// a symmetric sweep, or a forward sweep with smoother 1.
void KrylovSolver::learned_presmooth32(const float* x, float* y, cudaStream_t s) {
  if (!has_learned()) fail(NW_INVALID_ARG, "no learned preconditioner attached");
  ensure_f32(s);
  const int sweep = net_->smoother == 1 ? 1 : 0;
  if (gs_bf16_)
    sgs<__nv_bfloat16, float>(gs_vals16_.p, rdiag32_.p, x, y, s, false, sweep);
  else
    sgs<float, float>(gs_vals32_.p, rdiag32_.p, x, y, s, false, sweep);
}

// FP32 preconditioner of the mixed method. Learned (two-level, symmetric
// smoothing): z1 = SGS(x), r1 = x - A z1 (evaluated on the classes the
// sweep left a residual on), ec = Net(R r1), z2 = z1 + alpha P ec with the
// energy-optimal alpha, then the post-smoothing z = z2 + SGS(x - A z2),
// evaluated as one symmetric sweep starting from z2.
// Two-stage symmetric Gauss-Seidel ("sgs2", Ifpack2 "Two-stage Symmetric
// Gauss-Seidel", src/LinearSolverConfig.C:97-104), one sweep from zero:
// y1 = (D + L)^-1 x and y = y1 + (D + U)^-1 (x - A y1), each triangular
// solve replaced by g = D^-1 r followed by `inner` Jacobi-Richardson
// corrections g <- D^-1 (r - T g) (Berger-Vergiat et al. 2021). Every pass
// is a row-parallel CSR sweep; no colouring, no row dependences.
template <typename VT, typename T>
void KrylovSolver::sgs2(const VT* vals, const T* rd, const T* x, T* y, int inner, T* scratch,
                        cudaStream_t s) const {
  const int64_t n = A_.n;
  T* g[2] = {scratch, scratch + n};
  T* r1 = scratch + 2 * n;
  auto tri = [&](bool upper, const T* r, T* out) {
    jacobi_k<T><<<grid1(n), kBlock, 0, s>>>(n, rd, r, g[0]);
    int cur = 0;
    for (int k = 0; k < inner; ++k) {
      if (upper)
        ts_tri_launch<true, VT, T>(A_.lanes, n, A_.row_ptr, A_.col_idx, vals, rd, r, g[cur], g[1 - cur], s);
      else
        ts_tri_launch<false, VT, T>(A_.lanes, n, A_.row_ptr, A_.col_idx, vals, rd, r, g[cur], g[1 - cur], s);
      cur = 1 - cur;
    }
    NW_CUDA(cudaMemcpyAsync(out, g[cur], n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  };
  tri(false, x, y);
  spmv_launch<VT, T, T>(A_.lanes, n, A_.row_ptr, A_.col_idx, vals, y, x, r1, s);  // r1 = x - A y
  tri(true, r1, r1);
  axpy_t_k<T><<<grid1(n), kBlock, 0, s>>>(n, r1, y);
  NW_CUDA(cudaGetLastError());
}

void KrylovSolver::setup_levels(cudaStream_t s) {
  if (levels_ready_) return;
  const int64_t n = A_.n;
  if (!A_.row_ptr_host || (!A_.col_idx_host && A_.nnz > 0)) fail(NW_INTERNAL, "host graph needed");
  const int64_t* rp = A_.row_ptr_host;
  const int32_t* ci = A_.col_idx_host;
  std::vector<int32_t> lf(n, 0), lb(n, 0);
  std::vector<int64_t> dp(n, -1);
  for (int64_t i = 0; i < n; ++i) {
    int32_t l = 0;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
      if (ci[p] < i) l = std::max(l, lf[ci[p]] + 1);
      if (ci[p] == i) dp[i] = p;
    }
    if (dp[i] < 0) fail(NW_INVALID_ARG, "a row without a diagonal entry");
    lf[i] = l;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    int32_t l = 0;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p)
      if (ci[p] > i) l = std::max(l, lb[ci[p]] + 1);
    lb[i] = l;
  }
  auto group = [&](const std::vector<int32_t>& lev, std::vector<int64_t>& ptr, DeviceArray<int32_t>& rows) {
    const int32_t nl = n ? *std::max_element(lev.begin(), lev.end()) + 1 : 0;
    ptr.assign(nl + 1, 0);
    for (int64_t i = 0; i < n; ++i) ptr[lev[i] + 1]++;
    for (int32_t l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
    std::vector<int32_t> r(n);
    std::vector<int64_t> pos(ptr.begin(), ptr.end() - 1);
    for (int64_t i = 0; i < n; ++i) r[pos[lev[i]]++] = int32_t(i);
    rows.upload(r, s);
  };
  group(lf, fl_ptr_, fl_rows_);
  group(lb, bl_ptr_, bl_rows_);
  dpos_.upload(dp, s);
  levels_ready_ = true;
}

template <typename VT, typename T>
void KrylovSolver::sgs_natural(const VT* vals, const T* x, T* y, cudaStream_t s) {
  setup_levels(s);
  const int64_t n = A_.n;
  fill_k<T><<<grid1(n), kBlock, 0, s>>>(n, y, T(0));
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<int64_t>& ptr = pass == 0 ? fl_ptr_ : bl_ptr_;
    const int32_t* rows = pass == 0 ? fl_rows_.p : bl_rows_.p;
    for (size_t l = 0; l + 1 < ptr.size(); ++l) {
      const int64_t cnt = ptr[l + 1] - ptr[l];
      if (cnt)
        gs_level_k<VT, T><<<grid1(cnt), kBlock, 0, s>>>(cnt, rows + ptr[l], A_.row_ptr, A_.col_idx, vals,
                                                         dpos_.p, x, y);
    }
  }
  NW_CUDA(cudaGetLastError());
}

void KrylovSolver::ilu0_factor(cudaStream_t s) {
  if (ilu_valid_) return;
  setup_levels(s);
  lu_.resize(A_.nnz);
  NW_CUDA(cudaMemcpyAsync(lu_.p, A_.values, A_.nnz * sizeof(double), cudaMemcpyDeviceToDevice, s));
  for (size_t l = 0; l + 1 < fl_ptr_.size(); ++l) {
    const int64_t cnt = fl_ptr_[l + 1] - fl_ptr_[l];
    if (cnt)
      ilu0_level_k<<<grid1(cnt), kBlock, 0, s>>>(cnt, fl_rows_.p + fl_ptr_[l], A_.row_ptr, A_.col_idx,
                                                 dpos_.p, lu_.p);
  }
  lu32_.resize(A_.nnz);
  convert_k<double, float><<<grid1(A_.nnz), kBlock, 0, s>>>(A_.nnz, lu_.p, lu32_.p);
  NW_CUDA(cudaGetLastError());
  ilu_valid_ = true;
}

template <typename T>
void KrylovSolver::ilu0_solve(const T* lu, const T* x, T* y, cudaStream_t s) {
  for (size_t l = 0; l + 1 < fl_ptr_.size(); ++l) {
    const int64_t cnt = fl_ptr_[l + 1] - fl_ptr_[l];
    if (cnt)
      ilu0_solve_level_k<false, T><<<grid1(cnt), kBlock, 0, s>>>(cnt, fl_rows_.p + fl_ptr_[l], A_.row_ptr,
                                                                  A_.col_idx, dpos_.p, lu, x, y);
  }
  for (size_t l = 0; l + 1 < bl_ptr_.size(); ++l) {
    const int64_t cnt = bl_ptr_[l + 1] - bl_ptr_[l];
    if (cnt)
      ilu0_solve_level_k<true, T><<<grid1(cnt), kBlock, 0, s>>>(cnt, bl_rows_.p + bl_ptr_[l], A_.row_ptr,
                                                                 A_.col_idx, dpos_.p, lu, y, y);
  }
  NW_CUDA(cudaGetLastError());
}

void KrylovSolver::precond32(const Precond& pc, const float* x, float* y,
                             cudaStream_t s) {
  const int64_t n = A_.n;
  if (pc.kind == NW_PC_SGS_NATURAL) {
    sgs_natural<float, float>(vals32_.p, x, y, s);
    return;
  }
  if (pc.kind == NW_PC_RILUK) {
    ilu0_factor(s);
    ilu0_solve<float>(lu32_.p, x, y, s);
    return;
  }
  if (pc.kind == NW_PC_SGS2) {
    sgs2_32_.resize(size_t(3) * n);
    sgs2<float, float>(vals32_.p, rdiag32_.p, x, y, pc.inner_sweeps, sgs2_32_.p, s);
    return;
  }
  if (pc.kind == NW_PC_SGS) {
    if (gs_bf16_)
      sgs<__nv_bfloat16, float>(gs_vals16_.p, rdiag32_.p, x, y, s);
    else
      sgs<float, float>(gs_vals32_.p, rdiag32_.p, x, y, s);
    return;
  }
  if (pc.kind != NW_PC_LEARNED) {
    precond_apply_t<float, float>(pc, n, A_.row_ptr, A_.col_idx, vals32_.p,
                                  rdiag32_.p, x, y, s);
    return;
  }
  if (!has_learned()) fail(NW_INVALID_ARG, "no learned preconditioner attached");
  // smoother 0: symmetric sweeps before and after; 1: forward sweep before,
  // backward sweep after (the cycle stays symmetric)
  const bool half = net_->smoother == 1;
  const int nc = int(gs_cptr_.size()) - 1;
  learned_presmooth32(x, y, s);
  tmp32_.resize(n);
  rc32_.resize(cl_->nc);
  ec32_.resize(cl_->nc);
  sgs_residual32(x, y, tmp32_.p, s, half ? nc - 1 : 0);
  launch_restrict(*cl_, tmp32_.p, rc32_.p, s);
  net_->coarse_correction(*cl_, rc32_.p, ec32_.p, s);
  launch_prolong_add(*cl_, ec32_.p, net_->alpha_dev(), y, s);
  // post-smoothing z2 + S(x - A z2) is one sweep starting from z2
  if (net_->post_smooth) {
    if (gs_bf16_)
      sgs<__nv_bfloat16, float>(gs_vals16_.p, rdiag32_.p, x, y, s, true, half ? 2 : 0);
    else
      sgs<float, float>(gs_vals32_.p, rdiag32_.p, x, y, s, true, half ? 2 : 0);
  }
  NW_CUDA(cudaGetLastError());
}

void KrylovSolver::apply_precond(const Precond& pc, const double* x, double* y,
                                 cudaStream_t s) {
  if (pc.kind == NW_PC_LEARNED) {
    if (pc.apply_fn) {
      pc.apply_fn(x, y, s);
      return;
    }
    // FP64 interface around the FP32 learned preconditioner
    ensure_f32(s);
    const int64_t n = A_.n;
    tmp32b_.resize(n);
    convert_k<double, float><<<grid1(n), kBlock, 0, s>>>(n, x, tmp32b_.p);
    z32_.resize(n);
    precond32(pc, tmp32b_.p, z32_.p, s);
    convert_k<float, double><<<grid1(n), kBlock, 0, s>>>(n, z32_.p, y);
    return;
  }
  if (pc.kind == NW_PC_SGS) {
    sgs<double, double>(gs_vals_.p, rdiag_.p, x, y, s);
    return;
  }
  if (pc.kind == NW_PC_SGS2) {
    sgs2_64_.resize(size_t(3) * A_.n);
    sgs2<double, double>(A_.values, rdiag_.p, x, y, pc.inner_sweeps, sgs2_64_.p, s);
    return;
  }
  if (pc.kind == NW_PC_SGS_NATURAL) {
    sgs_natural<double, double>(A_.values, x, y, s);
    return;
  }
  if (pc.kind == NW_PC_RILUK) {
    ilu0_factor(s);
    ilu0_solve<double>(lu_.p, x, y, s);
    return;
  }
  precond_apply_t<double, double>(pc, A_.n, A_.row_ptr, A_.col_idx, A_.values,
                                  rdiag_.p, x, y, s);
}

SolveResult KrylovSolver::solve(const nw_solver_cfg& cfg, double tol,
                                const Precond& pc, const double* b, double* x,
                                cudaStream_t s) {
  SolveResult r;
  if (cfg.precision == NW_PREC_MIXED || cfg.precision == NW_PREC_MIXED_BF16)
    r = mixed(cfg, tol, pc, b, x, s);
  else if (cfg.method == NW_CG && pc.kind != NW_PC_LEARNED)
    r = cg(cfg, tol, pc, b, x, s);
  else if (cfg.method == NW_BICGSTAB && pc.kind != NW_PC_LEARNED)
    r = bicgstab(cfg, tol, pc, b, x, s);
  else if (cfg.method == NW_TFQMR && pc.kind != NW_PC_LEARNED)
    r = tfqmr(cfg, tol, pc, b, x, s);
  else if (cfg.method == NW_SSTEP_GMRES && pc.kind != NW_PC_LEARNED)
    r = sstep_gmres(cfg, tol, pc, b, x, s);
  else
    r = gmres(cfg, tol, pc, b, x, cfg.method == NW_FGMRES || pc.kind == NW_PC_LEARNED, s);
  // The learned preconditioner is judged by the FP64 residual: if the
  // flexible solve fails (no convergence, breakdown, non-finite values, or
  // a tensor-core wait of the network that gave up) the same solve is
  // repeated with plain symmetric Gauss-Seidel.
  const bool tc_timeout = pc.kind == NW_PC_LEARNED && tc_status(s) != 0;
  if (pc.kind == NW_PC_LEARNED && (!r.converged || tc_timeout) && std::isfinite(r.bnorm)) {
    Precond sgs = pc;
    sgs.kind = NW_PC_SGS;
    const SolveResult first = r;
    r = (cfg.precision == NW_PREC_MIXED || cfg.precision == NW_PREC_MIXED_BF16)
            ? mixed(cfg, tol, sgs, b, x, s)
                                       : gmres(cfg, tol, sgs, b, x, false, s);
    r.fallback = 1;
    r.iterations += first.iterations;
    r.outer += first.outer;
    // history: the failed learned attempt, then the SGS solve
    std::vector<double> h = first.history;
    h.insert(h.end(), r.history.begin(), r.history.end());
    r.history.swap(h);
  }
  return r;
}

// Restarted right-preconditioned GMRES(m) / FGMRES(m), FP64.
SolveResult KrylovSolver::gmres(const nw_solver_cfg& cfg, double tol,
                                const Precond& pc, const double* b, double* x,
                                bool flexible, cudaStream_t s) {
  const int64_t n = A_.n;
  const int m = std::min(m_, std::max(1, cfg.kspace));
  SolveResult res;
  if (flexible && Z_.n < size_t(m) * n) Z_.resize(size_t(m) * n);
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, x, 0.0);
  const double bnorm = std::sqrt(dot(b, b, s));
  res.bnorm = bnorm;
  res.history.push_back(1.0);
  if (!std::isfinite(bnorm)) {
    res.status = NW_NAN_DETECTED;
    return res;
  }
  if (bnorm == 0.0) {
    res.converged = 1;
    return res;
  }
  double* V = V_.p;
  double beta = bnorm;
  NW_CUDA(cudaMemcpyAsync(r_.p, b, n * sizeof(double),
                          cudaMemcpyDeviceToDevice, s));
  double rel = 1.0;
  int its = 0, stalls = 0;
  bool done = false;
  double* hs = scal_.p;             // h (m+1)
  double* h2 = scal_.p + (m_ + 2);  // second-pass h, then norm
  // Jacobi fuses into the normalisation that produces each basis vector
  const bool fuse_jacobi = pc.kind == NW_PC_JACOBI;
  while (!done && its < cfg.max_iterations) {
    // V0 = r / beta (and z0 = D^-1 V0)
    NW_CUDA(cudaMemcpyAsync(h2, &beta, sizeof(double), cudaMemcpyHostToDevice, s));
    scale_jacobi_k<double><<<grid1(n), kBlock, 0, s>>>(
        n, r_.p, V, h2, fuse_jacobi ? rdiag_.p : nullptr, flexible ? Z_.p : z_.p);
    auto arnoldi = [&](int j) {
      double* vj = V + size_t(j) * n;
      double* zj = flexible ? Z_.p + size_t(j) * n : z_.p;
      if (!fuse_jacobi) apply_precond(pc, vj, zj, s);
      spmv(zj, w_.p, s);
      // two classical Gram-Schmidt passes, coefficients kept on the device
      mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, j + 1, V, n, w_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, hs, 0, nullptr);
      maxpy_k<double><<<grid1(n), kBlock, 0, s>>>(n, j + 1, V, n, hs, w_.p, nullptr);
      mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, j + 1, V, n, w_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, h2 + 1, 1, hs);
      maxpy_k<double><<<grid1(n), kBlock, 0, s>>>(n, j + 1, V, n, h2 + 1, w_.p, partial_.p);
      reduce_partials_k<<<1, kBlock, 0, s>>>(int(grid1(n)), partial_.p, h2, 0, nullptr);
      sqrt_scalar_k<<<1, 1, 0, s>>>(h2);
      double* znext = (j + 1 < m) ? (flexible ? Z_.p + size_t(j + 1) * n : z_.p) : nullptr;
      scale_jacobi_k<double><<<grid1(n), kBlock, 0, s>>>(
          n, w_.p, V + size_t(j + 1) * n, h2, (fuse_jacobi && znext) ? rdiag_.p : nullptr, znext);
    };
    const Cycle c = run_cycle(m, cfg.max_iterations - its, beta, tol, bnorm, 1.0, 1.0, arnoldi, hs, h2, s);
    its += c.iterations;
    res.history.insert(res.history.end(), c.hist.begin(), c.hist.end());
    if (!c.hist.empty()) rel = c.hist.back();
    if (c.status != NW_OK) res.status = c.status;
    done = c.done;
    const int kk = c.basis;
    if (kk > 0) {
      cycle_solution(gst_.p, gctl_.p, m_, kk, 1.0, h2, s);
      if (flexible) {
        combine_k<double><<<grid1(n), kBlock, 0, s>>>(n, kk, Z_.p, n, h2, w_.p);
        axpy_k<<<grid1(n), kBlock, 0, s>>>(n, 1.0, w_.p, x);
      } else {
        combine_k<double><<<grid1(n), kBlock, 0, s>>>(n, kk, V, n, h2, w_.p);
        apply_precond(pc, w_.p, z_.p, s);
        axpy_k<<<grid1(n), kBlock, 0, s>>>(n, 1.0, z_.p, x);
      }
      NW_CUDA(cudaGetLastError());
    }
    if (done || its >= cfg.max_iterations) break;
    spmv64(x, b, r_.p, s);
    const double prev = beta;
    beta = std::sqrt(dot(r_.p, r_.p, s));
    if (beta == 0.0) break;
    if (pc.kind == NW_PC_LEARNED && stalled(stalls, beta, prev)) {
      res.status = NW_NOT_CONVERGED;
      break;
    }
  }
  spmv64(x, b, r_.p, s);
  res.final_abs = std::sqrt(dot(r_.p, r_.p, s));
  res.final_rel = rel;
  res.iterations = its;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

// s-step GMRES ("TPETRA GMRES S-STEP", selected by src/LinearSolverConfig.C:
// 57-69 with "Step Size" = krylov_step_size and CholeskyQR2), right
// preconditioned, FP64. Within a restart cycle the basis grows by blocks of
// s vectors: the matrix powers w_k = A M^-1 u_k / sigma (u_0 = the last
// orthonormal vector, u_{k+1} = w_k; sigma, the size of A M^-1 seen on the
// previous block, keeps the scaled monomial basis near unit length) run
// without any reduction, then one block orthogonalisation: two classical
// block Gram-Schmidt passes against the previous basis (C) and CholeskyQR
// twice on the block (R), each pass one batch of dot products. The Arnoldi
// relation of the block follows from the change of basis
//   A M^-1 [u_0 .. u_{s-1}] = sigma [u_1 .. u_s],  U = V T,
// so the Hessenberg columns are H(:, j0:j0+s) = (sigma T(:, 1:s+1) -
// H_old T_old) T_new^-1 with T_new upper triangular; Givens rotations then
// test convergence column by column as in GMRES. In exact arithmetic the
// iterates are GMRES's; the host synchronises once per pass of a block
// instead of once per vector.
SolveResult KrylovSolver::sstep_gmres(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                                      const double* b, double* x, cudaStream_t s) {
  const int64_t n = A_.n;
  const int m = std::min(m_, std::max(1, cfg.kspace));
  const int sstep = cfg.sstep_size > 0 ? cfg.sstep_size : 5;
  SolveResult res;
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, x, 0.0);
  const double bnorm = std::sqrt(dot(b, b, s));
  res.bnorm = bnorm;
  res.history.push_back(1.0);
  if (!std::isfinite(bnorm)) {
    res.status = NW_NAN_DETECTED;
    return res;
  }
  if (bnorm == 0.0) {
    res.converged = 1;
    return res;
  }
  const int ldc = m + 1;
  sst_.resize(size_t(ldc) * sstep + size_t(sstep) * sstep + sstep + 8);
  double* Cd = sst_.p;                        // column k of C at Cd + k ldc
  double* Gd = Cd + size_t(ldc) * sstep;      // column k of the Gram matrix at Gd + k sstep
  double* Rd = Gd + size_t(sstep) * sstep;    // one column of R
  double* Sd = Rd + sstep;                    // one scalar
  // Hr: the Arnoldi Hessenberg as the blocks produce it; H: its columns
  // after the Givens rotations (the triangular factor of the least squares)
  std::vector<double> Hr(size_t(m + 1) * m), H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  std::vector<double> Ch(size_t(ldc) * sstep), Cp(size_t(ldc) * sstep), Gh(size_t(sstep) * sstep);
  double* V = V_.p;
  double* h2 = scal_.p + (m_ + 2);
  NW_CUDA(cudaMemcpyAsync(r_.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  double beta = bnorm, rel = 1.0, sigma = 1.0;
  int its = 0;
  bool done = false;
  auto upload = [&](double* dst, const double* src, size_t cnt) {
    NW_CUDA(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, s));
  };
  auto download = [&](double* dst, const double* src, size_t cnt) {
    NW_CUDA(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
    NW_CUDA(cudaStreamSynchronize(s));
  };
  while (!done && its < cfg.max_iterations) {
    upload(h2, &beta, 1);
    scale_jacobi_k<double><<<grid1(n), kBlock, 0, s>>>(n, r_.p, V, h2, nullptr, nullptr);
    std::fill(H.begin(), H.end(), 0.0);
    std::fill(Hr.begin(), Hr.end(), 0.0);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j0 = 0, kk = 0;
    while (j0 < m && its < cfg.max_iterations && !done) {
      const int sb = std::min(sstep, std::min(m - j0, cfg.max_iterations - its));
      double* W = V + size_t(j0 + 1) * n;
      // matrix powers
      upload(Sd, &sigma, 1);
      for (int k = 0; k < sb; ++k) {
        double* w = W + size_t(k) * n;
        apply_precond(pc, V + size_t(j0 + k) * n, z_.p, s);
        spmv(z_.p, w, s);
        scale_jacobi_k<double><<<grid1(n), kBlock, 0, s>>>(n, w, w, Sd, nullptr, nullptr);
      }
      // two block classical Gram-Schmidt passes against V(:, 0:j0+1)
      std::fill(Ch.begin(), Ch.end(), 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        for (int k = 0; k < sb; ++k) {
          mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, j0 + 1, V, n, W + size_t(k) * n, partial_.p);
          reduce_partials_k<<<j0 + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, Cd + size_t(k) * ldc, 0, nullptr);
        }
        for (int k = 0; k < sb; ++k)
          maxpy_k<double><<<grid1(n), kBlock, 0, s>>>(n, j0 + 1, V, n, Cd + size_t(k) * ldc,
                                                      W + size_t(k) * n, nullptr);
        download(Cp.data(), Cd, size_t(ldc) * sb);
        for (int k = 0; k < sb; ++k)
          for (int i = 0; i <= j0; ++i) Ch[size_t(k) * ldc + i] += Cp[size_t(k) * ldc + i];
      }
      // CholeskyQR twice on the block: W = Q Rt
      std::vector<double> Rt(size_t(sb) * sb, 0.0), Rp(size_t(sb) * sb), tmp(size_t(sb) * sb);
      for (int k = 0; k < sb; ++k) Rt[size_t(k) * sb + k] = 1.0;  // Rt[i][k] at k sb + i
      bool broke = false;
      for (int pass = 0; pass < 2 && !broke; ++pass) {
        for (int k = 0; k < sb; ++k) {
          mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, sb, W, n, W + size_t(k) * n, partial_.p);
          reduce_partials_k<<<sb, kBlock, 0, s>>>(red_blocks_, partial_.p, Gd + size_t(k) * sstep, 0, nullptr);
        }
        download(Gh.data(), Gd, size_t(sstep) * sb);
        std::fill(Rp.begin(), Rp.end(), 0.0);
        for (int k = 0; k < sb && !broke; ++k) {
          for (int i = 0; i < k; ++i) {
            double v = Gh[size_t(k) * sstep + i];
            for (int l = 0; l < i; ++l) v -= Rp[size_t(i) * sb + l] * Rp[size_t(k) * sb + l];
            Rp[size_t(k) * sb + i] = v / Rp[size_t(i) * sb + i];
          }
          double d = Gh[size_t(k) * sstep + k];
          for (int l = 0; l < k; ++l) d -= Rp[size_t(k) * sb + l] * Rp[size_t(k) * sb + l];
          if (!(d > 0.0) || !std::isfinite(d)) {
            broke = true;
            break;
          }
          Rp[size_t(k) * sb + k] = std::sqrt(d);
        }
        if (broke) break;
        for (int k = 0; k < sb; ++k) {
          double* w = W + size_t(k) * n;
          if (k > 0) {
            upload(Rd, &Rp[size_t(k) * sb], size_t(k));
            maxpy_k<double><<<grid1(n), kBlock, 0, s>>>(n, k, W, n, Rd, w, nullptr);
          }
          upload(Sd, &Rp[size_t(k) * sb + k], 1);
          scale_jacobi_k<double><<<grid1(n), kBlock, 0, s>>>(n, w, w, Sd, nullptr, nullptr);
        }
        // Rt = Rp Rt (both upper triangular)
        for (int k = 0; k < sb; ++k)
          for (int i = 0; i <= k; ++i) {
            double v = 0.0;
            for (int l = i; l <= k; ++l) v += Rp[size_t(l) * sb + i] * Rt[size_t(k) * sb + l];
            tmp[size_t(k) * sb + i] = v;
          }
        for (int k = 0; k < sb; ++k)
          for (int i = 0; i <= k; ++i) Rt[size_t(k) * sb + i] = tmp[size_t(k) * sb + i];
      }
      if (broke) {
        res.status = NW_BREAKDOWN;
        done = true;
        break;
      }
      // Hessenberg columns j0 .. j0 + sb - 1: M = sigma T(:, 1:sb+1) - H_old T_old,
      // then H_new = M T_new^-1 (rows 0 .. j0 + sb)
      const int rows = j0 + sb + 1;
      std::vector<double> Mx(size_t(rows) * sb, 0.0), Tn(size_t(sb) * sb, 0.0), Hn(size_t(rows) * sb, 0.0);
      for (int k = 0; k < sb; ++k) {
        for (int i = 0; i <= j0; ++i) Mx[size_t(k) * rows + i] = sigma * Ch[size_t(k) * ldc + i];
        for (int i = 0; i <= k; ++i) Mx[size_t(k) * rows + j0 + 1 + i] = sigma * Rt[size_t(k) * sb + i];
        // - H_old T_old: column k of T_old is column k - 1 of C (rows 0 .. j0 - 1)
        if (k > 0)
          for (int i = 0; i <= j0; ++i) {
            double v = 0.0;
            for (int l = 0; l < j0; ++l) v += Hr[size_t(i) * m + l] * Ch[size_t(k - 1) * ldc + l];
            Mx[size_t(k) * rows + i] -= v;
          }
        // T_new: rows v_j0 .. v_{j0+sb-1}
        if (k == 0) {
          Tn[0] = 1.0;
        } else {
          Tn[size_t(k) * sb + 0] = Ch[size_t(k - 1) * ldc + j0];
          for (int i = 1; i <= k; ++i) Tn[size_t(k) * sb + i] = Rt[size_t(k - 1) * sb + i - 1];
        }
      }
      for (int k = 0; k < sb; ++k)
        for (int i = 0; i < rows; ++i) {
          double v = Mx[size_t(k) * rows + i];
          for (int l = 0; l < k; ++l) v -= Hn[size_t(l) * rows + i] * Tn[size_t(k) * sb + l];
          Hn[size_t(k) * rows + i] = v / Tn[size_t(k) * sb + k];
        }
      for (int k = 0; k < sb; ++k) {
        const int j = j0 + k;
        for (int i = 0; i <= j + 1; ++i) Hr[size_t(i) * m + j] = H[size_t(i) * m + j] = Hn[size_t(k) * rows + i];
      }
      // Givens rotations column by column
      for (int k = 0; k < sb; ++k) {
        const int j = j0 + k;
        for (int q = 0; q < j; ++q) {
          const double a = H[size_t(q) * m + j], bb = H[size_t(q + 1) * m + j];
          H[size_t(q) * m + j] = cs[q] * a + sn[q] * bb;
          H[size_t(q + 1) * m + j] = -sn[q] * a + cs[q] * bb;
        }
        const double a = H[size_t(j) * m + j], bb = H[size_t(j + 1) * m + j];
        const double den = std::sqrt(a * a + bb * bb);
        if (!(den > 0.0) || !std::isfinite(den)) {
          res.status = std::isfinite(den) ? NW_BREAKDOWN : NW_NAN_DETECTED;
          done = true;
          kk = j;
          break;
        }
        cs[j] = a / den;
        sn[j] = bb / den;
        H[size_t(j) * m + j] = den;
        H[size_t(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        ++its;
        rel = std::abs(g[j + 1]) / bnorm;
        res.history.push_back(rel);
        kk = j + 1;
        if (!std::isfinite(rel)) {
          res.status = NW_NAN_DETECTED;
          done = true;
          break;
        }
        if (rel <= tol) {
          done = true;
          break;
        }
      }
      // the next block's scaling: |A M^-1 u_0| of this block
      {
        double w0 = 0.0;
        for (int i = 0; i <= j0; ++i) w0 += Ch[i] * Ch[i];
        w0 += Rt[0] * Rt[0];
        const double next = sigma * std::sqrt(w0);
        if (std::isfinite(next) && next > 0.0) sigma = next;
      }
      j0 += sb;
    }
    for (int i = kk - 1; i >= 0; --i) {
      double sum = g[i];
      for (int l = i + 1; l < kk; ++l) sum -= H[size_t(i) * m + l] * y[l];
      y[i] = sum / H[size_t(i) * m + i];
    }
    if (kk > 0) {
      upload(h2, y.data(), size_t(kk));
      combine_k<double><<<grid1(n), kBlock, 0, s>>>(n, kk, V, n, h2, w_.p);
      apply_precond(pc, w_.p, z_.p, s);
      axpy_k<<<grid1(n), kBlock, 0, s>>>(n, 1.0, z_.p, x);
      NW_CUDA(cudaGetLastError());
    }
    if (done || its >= cfg.max_iterations) break;
    spmv64(x, b, r_.p, s);
    beta = std::sqrt(dot(r_.p, r_.p, s));
    if (beta == 0.0) break;
  }
  spmv64(x, b, r_.p, s);
  res.final_abs = std::sqrt(dot(r_.p, r_.p, s));
  res.final_rel = rel;
  res.iterations = its;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

// Preconditioned conjugate gradients (FP64).
SolveResult KrylovSolver::cg(const nw_solver_cfg& cfg, double tol,
                             const Precond& pc, const double* b, double* x,
                             cudaStream_t s) {
  const int64_t n = A_.n;
  SolveResult res;
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, x, 0.0);
  const double bnorm = std::sqrt(dot(b, b, s));
  res.bnorm = bnorm;
  res.history.push_back(1.0);
  if (!std::isfinite(bnorm)) {
    res.status = NW_NAN_DETECTED;
    return res;
  }
  if (bnorm == 0.0) {
    res.converged = 1;
    return res;
  }
  double* r = r_.p;
  double* p = V_.p;
  double* q = V_.p + n;
  double* z = z_.p;
  NW_CUDA(cudaMemcpyAsync(r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  apply_precond(pc, r, z, s);
  NW_CUDA(cudaMemcpyAsync(p, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  double rz = dot(r, z, s);
  double rel = 1.0;
  int its = 0;
  while (its < cfg.max_iterations) {
    spmv(p, q, s);
    const double pq = dot(p, q, s);
    const double alpha = rz / pq;
    if (!std::isfinite(alpha)) {
      res.status = NW_BREAKDOWN;
      break;
    }
    axpy_k<<<grid1(n), kBlock, 0, s>>>(n, alpha, p, x);
    axpy_k<<<grid1(n), kBlock, 0, s>>>(n, -alpha, q, r);
    ++its;
    rel = std::sqrt(dot(r, r, s)) / bnorm;
    res.history.push_back(rel);
    if (rel <= tol) break;
    apply_precond(pc, r, z, s);
    const double rzn = dot(r, z, s);
    const double beta = rzn / rz;
    rz = rzn;
    xpby_k<<<grid1(n), kBlock, 0, s>>>(n, z, beta, p);
  }
  spmv64(x, b, r, s);
  res.final_abs = std::sqrt(dot(r, r, s));
  res.final_rel = rel;
  res.iterations = its;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

// BiCGStab (van der Vorst 1992), right preconditioned, FP64: Belos
// "bicgstab" as src/LinearSolver.C:114 selects it. Converged when the
// recursively updated residual satisfies ||r|| / ||b|| <= tol.
SolveResult KrylovSolver::bicgstab(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                                   const double* b, double* x, cudaStream_t s) {
  const int64_t n = A_.n;
  SolveResult res;
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, x, 0.0);
  const double bnorm = std::sqrt(dot(b, b, s));
  res.bnorm = bnorm;
  res.history.push_back(1.0);
  if (!std::isfinite(bnorm)) {
    res.status = NW_NAN_DETECTED;
    return res;
  }
  if (bnorm == 0.0) {
    res.converged = 1;
    return res;
  }
  aux_.resize(size_t(7) * n);
  double *rh = aux_.p, *p = rh + n, *v = p + n, *ph = v + n, *sv = ph + n, *sh = sv + n,
         *t = sh + n;
  double* r = r_.p;
  NW_CUDA(cudaMemcpyAsync(r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  NW_CUDA(cudaMemcpyAsync(rh, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, p, 0.0);
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, v, 0.0);
  double rho = 1.0, alpha = 1.0, omega = 1.0, rel = 1.0;
  int its = 0;
  while (its < cfg.max_iterations) {
    const double rho_n = dot(rh, r, s);
    if (rho_n == 0.0 || omega == 0.0 || !std::isfinite(rho_n)) {
      res.status = NW_BREAKDOWN;
      break;
    }
    const double beta = (rho_n / rho) * (alpha / omega);
    rho = rho_n;
    bicg_dir_k<<<grid1(n), kBlock, 0, s>>>(n, r, beta, omega, v, p);
    apply_precond(pc, p, ph, s);
    spmv(ph, v, s);
    const double rv = dot(rh, v, s);
    if (rv == 0.0 || !std::isfinite(rv)) {
      res.status = NW_BREAKDOWN;
      break;
    }
    alpha = rho / rv;
    lincomb_k<<<grid1(n), kBlock, 0, s>>>(n, 1.0, r, -alpha, v, sv);
    apply_precond(pc, sv, sh, s);
    spmv(sh, t, s);
    const double tt = dot(t, t, s);
    omega = tt > 0.0 ? dot(t, sv, s) / tt : 0.0;
    bicg_upd_k<<<grid1(n), kBlock, 0, s>>>(n, alpha, ph, omega, sh, sv, t, x, r);
    ++its;
    rel = std::sqrt(dot(r, r, s)) / bnorm;
    res.history.push_back(rel);
    if (rel <= tol) break;
  }
  spmv64(x, b, r, s);
  res.final_abs = std::sqrt(dot(r, r, s));
  res.final_rel = rel;
  res.iterations = its;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

// TFQMR (Freund 1993; Saad, Iterative Methods for Sparse Linear Systems,
// 2003, Algorithm 7.8) on A M^-1, FP64, with the direction vectors kept as
// dh = M^-1 d so x is updated directly: Belos "tfqmr". One iteration is an
// even and an odd half step (two products with A M^-1); after each the
// residual bound sqrt(k + 1) tau_k (k half steps) is tested against
// tol ||b||.
SolveResult KrylovSolver::tfqmr(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                                const double* b, double* x, cudaStream_t s) {
  const int64_t n = A_.n;
  SolveResult res;
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, x, 0.0);
  const double bnorm = std::sqrt(dot(b, b, s));
  res.bnorm = bnorm;
  res.history.push_back(1.0);
  if (!std::isfinite(bnorm)) {
    res.status = NW_NAN_DETECTED;
    return res;
  }
  if (bnorm == 0.0) {
    res.converged = 1;
    return res;
  }
  aux_.resize(size_t(7) * n);
  double *w = aux_.p, *u = w + n, *uh = u + n, *Au = uh + n, *Aun = Au + n, *v = Aun + n,
         *dh = v + n;
  const double* rt = b;  // shadow residual r0* = r0 = b
  NW_CUDA(cudaMemcpyAsync(w, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  NW_CUDA(cudaMemcpyAsync(u, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, dh, 0.0);
  apply_precond(pc, u, uh, s);
  spmv(uh, Au, s);
  NW_CUDA(cudaMemcpyAsync(v, Au, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  double tau = bnorm, theta = 0.0, eta = 0.0, alpha = 0.0, rel = 1.0;
  double rho = dot(rt, b, s);
  int its = 0;
  for (int64_t mm = 0; its < cfg.max_iterations; ++mm) {
    if (mm % 2 == 0) {
      const double vr = dot(v, rt, s);
      if (vr == 0.0 || !std::isfinite(vr)) {
        res.status = NW_BREAKDOWN;
        break;
      }
      alpha = rho / vr;
    }
    const double coef = alpha != 0.0 ? theta * theta / alpha * eta : 0.0;
    tfqmr_wd_k<<<grid1(n), kBlock, 0, s>>>(n, alpha, Au, coef, uh, w, dh);
    theta = std::sqrt(dot(w, w, s)) / tau;
    const double c = 1.0 / std::sqrt(1.0 + theta * theta);
    tau = tau * theta * c;
    eta = c * c * alpha;
    axpy_k<<<grid1(n), kBlock, 0, s>>>(n, eta, dh, x);
    if (mm % 2 == 0) {
      axpy_k<<<grid1(n), kBlock, 0, s>>>(n, -alpha, v, u);
      apply_precond(pc, u, uh, s);
      spmv(uh, Aun, s);
      std::swap(Au, Aun);
    } else {
      ++its;
      rel = std::sqrt(double(mm + 2)) * tau / bnorm;
      res.history.push_back(rel);
      if (!std::isfinite(rel)) {
        res.status = NW_BREAKDOWN;
        break;
      }
      if (rel <= tol) break;
      if (rho == 0.0) {
        res.status = NW_BREAKDOWN;
        break;
      }
      const double rho_n = dot(w, rt, s);
      const double beta = rho_n / rho;
      rho = rho_n;
      xpby_k<<<grid1(n), kBlock, 0, s>>>(n, w, beta, u);
      apply_precond(pc, u, uh, s);
      spmv(uh, Aun, s);
      tfqmr_v_k<<<grid1(n), kBlock, 0, s>>>(n, Aun, beta, Au, v);
      std::swap(Au, Aun);
    }
  }
  spmv64(x, b, r_.p, s);
  res.final_abs = std::sqrt(dot(r_.p, r_.p, s));
  res.final_rel = rel;
  res.iterations = its;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

// Mixed precision: FP64 iterative refinement around an FP32 inner GMRES.
// Outer: r = b - A x in FP64, stop when ||r||/||b|| <= tol. Inner: GMRES
// restarted once per outer step on A d = r in FP32 storage (FP32 SpMV with
// FP32 accumulation, FP32 Jacobi/SGS), one classical Gram-Schmidt pass
// with FP64-accurate dots, FP64 Hessenberg least squares on the host;
// x += d in FP64.
SolveResult KrylovSolver::mixed(const nw_solver_cfg& cfg, double tol,
                                const Precond& pc, const double* b, double* x,
                                cudaStream_t s) {
  const int64_t n = A_.n;
  ensure_f32(s);
  gs_bf16_ = cfg.precision == NW_PREC_MIXED_BF16;
  if (gs_bf16_ && gs_vals16_.n != gs_vals32_.n) {
    gs_vals16_.resize(gs_vals32_.n);
    if (gs_vals32_.n)
      to_bf16_vals_k<<<grid1(int64_t(gs_vals32_.n)), kBlock, 0, s>>>(int64_t(gs_vals32_.n), gs_vals32_.p,
                                                                    gs_vals16_.p);
  }
  const int m = std::min(m_, std::max(1, cfg.inner_kspace > 0 ? cfg.inner_kspace : cfg.kspace));
  const double itol = cfg.inner_tolerance > 0 ? cfg.inner_tolerance : 1e-4;
  SolveResult res;
  fill_k<double><<<grid1(n), kBlock, 0, s>>>(n, x, 0.0);
  const double bnorm = std::sqrt(dot(b, b, s));
  res.bnorm = bnorm;
  res.history.push_back(1.0);
  if (!std::isfinite(bnorm)) {
    res.status = NW_NAN_DETECTED;
    return res;
  }
  if (bnorm == 0.0) {
    res.converged = 1;
    return res;
  }
  const bool fuse_jacobi = pc.kind == NW_PC_JACOBI;
  const bool flexible = pc.kind == NW_PC_LEARNED;
  const int64_t ld = ld32_;
  if (flexible && Z32_.n < size_t(m) * ld) Z32_.resize(size_t(m) * ld);
  float* V = V32_.p;
  const unsigned g4 = grid1((n + 3) / 4);
  double* hs = scal_.p;
  double* h2 = scal_.p + (m_ + 2);
  double rel = 1.0;
  int its = 0, outer = 0, stalls = 0;
  NW_CUDA(cudaMemcpyAsync(r_.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  double rnorm = bnorm, prev_rnorm = bnorm;
  while (its < cfg.max_iterations) {
    ++outer;
    // inner: solve A d = r (scaled) in FP32
    NW_CUDA(cudaMemcpyAsync(h2, &rnorm, sizeof(double), cudaMemcpyHostToDevice, s));
    scale_to_f32_k<<<grid1(n), kBlock, 0, s>>>(n, r_.p, V, h2);
    if (fuse_jacobi) jacobi_k<float><<<grid1(n), kBlock, 0, s>>>(n, rdiag32_.p, V, z32_.p);
    // inner system solved for r / ||r|| (g0 = 1)
    auto arnoldi = [&](int j) {
      float* vj = V + size_t(j) * ld;
      float* zj = flexible ? Z32_.p + size_t(j) * ld : z32_.p;
      if (!fuse_jacobi) precond32(pc, vj, zj, s);
      spmv32(zj, w32_.p, s);
      // one classical Gram-Schmidt pass (dots accumulated exactly in FP32
      // pairs): the inner solve only reduces the residual by inner_tol per
      // cycle and the FP64 outer loop recomputes the true residual, so the
      // second pass of the FP64 method is not needed here (same iteration
      // counts on the Poisson systems measured)
      mdot4_k<<<mdot4_blocks_, kBlock, 0, s>>>(n, j + 1, V, ld, w32_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(mdot4_blocks_, partial_.p, hs, 0, nullptr);
      maxpy4_k<<<g4, kBlock, 0, s>>>(n, j + 1, V, ld, hs, w32_.p, partial_.p);
      reduce_partials_k<<<1, kBlock, 0, s>>>(int(g4), partial_.p, h2, 0, nullptr);
      sqrt_scalar_k<<<1, 1, 0, s>>>(h2);
      scale_jacobi_k<float><<<grid1(n), kBlock, 0, s>>>(n, w32_.p, V + size_t(j + 1) * ld, h2,
                                                        fuse_jacobi ? rdiag32_.p : nullptr, z32_.p);
    };
    const Cycle c = run_cycle(m, cfg.max_iterations - its, 1.0, itol, 1.0, rnorm, bnorm, arnoldi, hs, h2, s,
                              true);
    its += c.iterations;
    res.history.insert(res.history.end(), c.hist.begin(), c.hist.end());
    if (c.status != NW_OK) res.status = c.status;
    const int kk = c.basis;
    if (kk > 0) {
      cycle_solution(gst_.p, gctl_.p, m_, kk, rnorm, h2, s);
      if (flexible) {
        combine_k<float><<<grid1(n), kBlock, 0, s>>>(n, kk, Z32_.p, ld, h2, z32_.p);
      } else {
        combine_k<float><<<grid1(n), kBlock, 0, s>>>(n, kk, V, ld, h2, w32_.p);
        precond32(pc, w32_.p, z32_.p, s);
      }
      add_f32_k<<<grid1(n), kBlock, 0, s>>>(n, z32_.p, x);
    }
    // outer FP64 true residual
    spmv64(x, b, r_.p, s);
    rnorm = std::sqrt(dot(r_.p, r_.p, s));
    rel = rnorm / bnorm;
    if (!std::isfinite(rel)) {
      res.status = NW_NAN_DETECTED;
      break;
    }
    if (res.history.size() > 1) res.history.back() = rel;
    if (rel <= tol || res.status != NW_OK) break;
    if (flexible && stalled(stalls, rnorm, prev_rnorm)) {
      res.status = NW_NOT_CONVERGED;
      break;
    }
    prev_rnorm = rnorm;
  }
  res.final_abs = rnorm;
  res.final_rel = rel;
  res.iterations = its;
  res.outer = outer;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

}  // namespace nw
