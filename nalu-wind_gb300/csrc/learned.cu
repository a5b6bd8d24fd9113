// Learned two-level preconditioner: aggregation, Galerkin coarse operator,
// and the edge message-passing network's forward, backward and Adam
// kernels. See learned.h for the method.
//
// The dense layers are BF16 GEMMs on the tensor cores through
// mma.sync.m16n8k16 (row.col, FP32 accumulation), staged in shared memory:
//   forward   Z[M x 64]  = X[M x 128] W[128 x 64]   (+ ReLU, BF16 out)
//   input gr. dX[M x 128] = dZ[M x 64] W^T           (FP32 out)
//   weight gr dW[128 x 64] = X^T dZ                  (per-block partials,
//                                                    fixed-order sum)
// At these shapes (K <= 128, N <= 128) the layers move more bytes than
// they compute, so they are HBM-bound rather than tensor-bound on GB300.
// Aggregations over the coarse graph are warp-per-row gathers (lane = two
// channels, FP32 accumulation). All reductions are deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <numeric>

#include "learned.h"

namespace nw {
namespace {

constexpr int kB = 256;
inline unsigned gridn(int64_t n, int t = kB) { return unsigned((n + t - 1) / t); }

__device__ __forceinline__ float bf2f(uint16_t h) {
  return __uint_as_float(uint32_t(h) << 16);
}
__device__ __forceinline__ uint16_t f2bf(float f) {
  const __nv_bfloat16 b = __float2bfloat16_rn(f);
  return *reinterpret_cast<const uint16_t*>(&b);
}
__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) {
  return uint32_t(lo) | (uint32_t(hi) << 16);
}

__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1,
                                         uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------------------
// Forward GEMM: out[r, 0:64] = relu(A[r, 0:128] . W), A row stride 128,
// W given transposed (wt[n][k], 64 x 128), out row stride ldo. 64 rows per
// block of 4 warps; rows padded to 68 words in shared memory (no bank
// conflicts for the fragment loads).
constexpr int kPadF = 68;
__global__ void __launch_bounds__(128)
    gemm_fwd_k(const uint16_t* __restrict__ a, const uint16_t* __restrict__ wt,
               uint16_t* __restrict__ out, int64_t m, int ldo) {
  __shared__ uint32_t ws[64 * kPadF];
  __shared__ uint32_t xs[64 * kPadF];
  const uint32_t* w32 = reinterpret_cast<const uint32_t*>(wt);
  const uint32_t* a32 = reinterpret_cast<const uint32_t*>(a);
  const int64_t r0 = int64_t(blockIdx.x) * 64;
  for (int q = threadIdx.x; q < 64 * 64; q += 128) {
    const int row = q >> 6, col = q & 63;
    ws[row * kPadF + col] = w32[q];
    const int64_t gr = r0 + row;
    xs[row * kPadF + col] = gr < m ? a32[gr * 64 + col] : 0u;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int wr = warp * 16;
  float acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
  for (int ks = 0; ks < 8; ++ks) {
    const int kw = ks * 8 + t;  // word index of k = ks*16 + 2t
    const uint32_t a0 = xs[(wr + g) * kPadF + kw];
    const uint32_t a1 = xs[(wr + g + 8) * kPadF + kw];
    const uint32_t a2 = xs[(wr + g) * kPadF + kw + 4];
    const uint32_t a3 = xs[(wr + g + 8) * kPadF + kw + 4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int n = nt * 8 + g;
      mma16816(acc[nt], a0, a1, a2, a3, ws[n * kPadF + kw], ws[n * kPadF + kw + 4]);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int col = nt * 8 + 2 * t;
    const int64_t ra = r0 + wr + g, rb = ra + 8;
    if (ra < m)
      *reinterpret_cast<uint32_t*>(out + ra * ldo + col) =
          pack2(f2bf(fmaxf(acc[nt][0], 0.f)), f2bf(fmaxf(acc[nt][1], 0.f)));
    if (rb < m)
      *reinterpret_cast<uint32_t*>(out + rb * ldo + col) =
          pack2(f2bf(fmaxf(acc[nt][2], 0.f)), f2bf(fmaxf(acc[nt][3], 0.f)));
  }
}

// Input gradient: dx[r, 0:128] = dz[r, 0:64] . W^T with W row-major
// (128 x 64) serving as the transposed B operand. FP32 output.
constexpr int kPadD = 36;
__global__ void __launch_bounds__(128)
    gemm_dx_k(const uint16_t* __restrict__ dz, const uint16_t* __restrict__ w,
              float* __restrict__ dx, int64_t m) {
  __shared__ uint32_t ws[128 * kPadD];
  __shared__ uint32_t zs[64 * kPadD];
  const uint32_t* w32 = reinterpret_cast<const uint32_t*>(w);
  const uint32_t* z32 = reinterpret_cast<const uint32_t*>(dz);
  const int64_t r0 = int64_t(blockIdx.x) * 64;
  for (int q = threadIdx.x; q < 128 * 32; q += 128) {
    const int row = q >> 5, col = q & 31;
    ws[row * kPadD + col] = w32[q];
  }
  for (int q = threadIdx.x; q < 64 * 32; q += 128) {
    const int row = q >> 5, col = q & 31;
    const int64_t gr = r0 + row;
    zs[row * kPadD + col] = gr < m ? z32[gr * 32 + col] : 0u;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int wr = warp * 16;
  float acc[16][4];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const int kw = ks * 8 + t;
    const uint32_t a0 = zs[(wr + g) * kPadD + kw];
    const uint32_t a1 = zs[(wr + g + 8) * kPadD + kw];
    const uint32_t a2 = zs[(wr + g) * kPadD + kw + 4];
    const uint32_t a3 = zs[(wr + g + 8) * kPadD + kw + 4];
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
      const int n = nt * 8 + g;
      mma16816(acc[nt], a0, a1, a2, a3, ws[n * kPadD + kw], ws[n * kPadD + kw + 4]);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const int col = nt * 8 + 2 * t;
    const int64_t ra = r0 + wr + g, rb = ra + 8;
    if (ra < m) *reinterpret_cast<float2*>(dx + ra * 128 + col) = make_float2(acc[nt][0], acc[nt][1]);
    if (rb < m) *reinterpret_cast<float2*>(dx + rb * 128 + col) = make_float2(acc[nt][2], acc[nt][3]);
  }
}

// Weight gradient partials: partial[block][cin][cout] = sum over this
// block's nodes of x[node][cin] dz[node][cout]. 8 warps cover cin 0..127
// (16 each); nodes are processed in chunks of 64 (grid-stride).
constexpr int kPadXc = 136;  // halfwords per staged row of x (128 + 8)
constexpr int kPadDz = 72;   // halfwords per staged row of dz (64 + 8)
__global__ void __launch_bounds__(256)
    gemm_wgrad_k(const uint16_t* __restrict__ xc, const uint16_t* __restrict__ dz,
                 float* __restrict__ partial, int64_t m) {
  __shared__ uint16_t xs[64 * kPadXc];
  __shared__ uint16_t zs[64 * kPadDz];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int wr = warp * 16;
  float acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
  for (int64_t c0 = int64_t(blockIdx.x) * 64; c0 < m; c0 += int64_t(gridDim.x) * 64) {
    __syncthreads();
    for (int q = threadIdx.x; q < 64 * 128; q += 256) {
      const int row = q >> 7, col = q & 127;
      const int64_t gr = c0 + row;
      xs[row * kPadXc + col] = gr < m ? xc[gr * 128 + col] : uint16_t(0);
    }
    for (int q = threadIdx.x; q < 64 * 64; q += 256) {
      const int row = q >> 6, col = q & 63;
      const int64_t gr = c0 + row;
      zs[row * kPadDz + col] = gr < m ? dz[gr * 64 + col] : uint16_t(0);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int k0 = ks * 16 + 2 * t;  // node index within the chunk
      const int ca = wr + g, cb = wr + g + 8;
      const uint32_t a0 = pack2(xs[k0 * kPadXc + ca], xs[(k0 + 1) * kPadXc + ca]);
      const uint32_t a1 = pack2(xs[k0 * kPadXc + cb], xs[(k0 + 1) * kPadXc + cb]);
      const uint32_t a2 = pack2(xs[(k0 + 8) * kPadXc + ca], xs[(k0 + 9) * kPadXc + ca]);
      const uint32_t a3 = pack2(xs[(k0 + 8) * kPadXc + cb], xs[(k0 + 9) * kPadXc + cb]);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const int n = nt * 8 + g;
        const uint32_t b0 = pack2(zs[k0 * kPadDz + n], zs[(k0 + 1) * kPadDz + n]);
        const uint32_t b1 = pack2(zs[(k0 + 8) * kPadDz + n], zs[(k0 + 9) * kPadDz + n]);
        mma16816(acc[nt], a0, a1, a2, a3, b0, b1);
      }
    }
  }
  float* out = partial + int64_t(blockIdx.x) * (128 * 64);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int col = nt * 8 + 2 * t;
    out[(wr + g) * 64 + col] = acc[nt][0];
    out[(wr + g) * 64 + col + 1] = acc[nt][1];
    out[(wr + g + 8) * 64 + col] = acc[nt][2];
    out[(wr + g + 8) * 64 + col + 1] = acc[nt][3];
  }
}

// dst[j] (+)= sum_b partial[b][j], fixed order over blocks
__global__ void colsum_k(int nblocks, int ncols, const float* __restrict__ partial,
                         float* __restrict__ dst, int accumulate) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncols) return;
  float s = 0.f;
  for (int b = 0; b < nblocks; ++b) s += partial[int64_t(b) * ncols + j];
  dst[j] = accumulate ? dst[j] + s : s;
}

// ---------------------------------------------------------------------------
// Aggregation over the coarse graph (diagonal slot skipped):
// out[I][64 + c] = sum_J w_IJ in[J][c], in/out BF16 with row stride 128.
__global__ void __launch_bounds__(kB)
    agg_fwd_k(int64_t nc, const int64_t* __restrict__ cptr,
              const int32_t* __restrict__ ccol, const int32_t* __restrict__ cdiag,
              const float* __restrict__ wgt, uint16_t* __restrict__ xc) {
  const int64_t I = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (I >= nc) return;
  float a0 = 0.f, a1 = 0.f;
  const int64_t dpos = cdiag[I];
  for (int64_t q = cptr[I]; q < cptr[I + 1]; ++q) {
    if (q == dpos) continue;
    const float w = wgt[q];
    const uint32_t v = *reinterpret_cast<const uint32_t*>(xc + int64_t(ccol[q]) * 128 + 2 * lane);
    a0 = fmaf(w, bf2f(uint16_t(v & 0xffffu)), a0);
    a1 = fmaf(w, bf2f(uint16_t(v >> 16)), a1);
  }
  *reinterpret_cast<uint32_t*>(xc + I * 128 + 64 + 2 * lane) = pack2(f2bf(a0), f2bf(a1));
}

// Transpose aggregation for the backward pass:
// dh[J][c] = dx[J][c] + sum_I w_IJ dx[I][64 + c] (I ranges over the row of J,
// w_IJ read through the transpose slot map).
__global__ void __launch_bounds__(kB)
    agg_bwd_k(int64_t nc, const int64_t* __restrict__ cptr,
              const int32_t* __restrict__ ccol, const int32_t* __restrict__ cdiag,
              const int32_t* __restrict__ rev, const float* __restrict__ wgt,
              const float* __restrict__ dx, float* __restrict__ dh) {
  const int64_t J = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (J >= nc) return;
  float2 acc = *reinterpret_cast<const float2*>(dx + J * 128 + 2 * lane);
  const int64_t dpos = cdiag[J];
  for (int64_t q = cptr[J]; q < cptr[J + 1]; ++q) {
    if (q == dpos) continue;
    const float w = wgt[rev[q]];
    const float2 v = *reinterpret_cast<const float2*>(dx + int64_t(ccol[q]) * 128 + 64 + 2 * lane);
    acc.x = fmaf(w, v.x, acc.x);
    acc.y = fmaf(w, v.y, acc.y);
  }
  *reinterpret_cast<float2*>(dh + J * 64 + 2 * lane) = acc;
}

// dz = bf16(dh * (h > 0)), h BF16 with row stride ldh
__global__ void mask_k(int64_t nc, const float* __restrict__ dh,
                       const uint16_t* __restrict__ h, int ldh,
                       uint16_t* __restrict__ dz) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= nc * 64) return;
  const int64_t I = q >> 6;
  const int c = int(q & 63);
  dz[q] = f2bf(bf2f(h[I * ldh + c]) > 0.f ? dh[q] : 0.f);
}

// u = rc * dinv; partial sums of u^2
__global__ void input_k(int64_t nc, const float* __restrict__ rc,
                        const float* __restrict__ dinv, float* __restrict__ u,
                        float* __restrict__ partial) {
  __shared__ float red[kB / 32];
  const int64_t I = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float v = 0.f;
  if (I < nc) {
    v = rc[I] * dinv[I];
    u[I] = v;
  }
  float s = v * v;
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int q = 0; q < kB / 32; ++q) t += red[q];
    partial[blockIdx.x] = t;
  }
}

// Fixed-order sum of partial[b * stride + which], b < nblocks, by one block
// of kB threads (strided per-thread sums, then a tree).
__device__ double block_sum(int nblocks, const float* __restrict__ partial, int stride, int which,
                            double* red) {
  double t = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kB) t += partial[int64_t(b) * stride + which];
  red[threadIdx.x] = t;
  __syncthreads();
  for (int h = kB / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  const double v = red[0];
  __syncthreads();
  return v;
}

// scal[0] = s = sqrt(sum u^2 / nc), scal[1] = 1 / s (0 when s == 0)
__global__ void __launch_bounds__(kB)
    rms_k(int nblocks, const float* __restrict__ partial, int64_t nc, float* __restrict__ scal) {
  __shared__ double red[kB];
  const double t = block_sum(nblocks, partial, 1, 0, red);
  if (threadIdx.x == 0) {
    const double s = std::sqrt(t / double(nc > 0 ? nc : 1));
    scal[0] = float(s);
    scal[1] = s > 0 ? float(1.0 / s) : 0.f;
  }
}

// x = u / s; ax = sum_J w_IJ x_J; H0 = relu(x W0[0] + ax W0[1]) into
// xc[:, 0:64]. Warp per row (lane = two channels).
__global__ void __launch_bounds__(kB)
    layer0_k(int64_t nc, const int64_t* __restrict__ cptr,
             const int32_t* __restrict__ ccol, const int32_t* __restrict__ cdiag,
             const float* __restrict__ wgt, const float* __restrict__ u,
             const float* __restrict__ scal, const float* __restrict__ w0,
             float* __restrict__ x, float* __restrict__ ax, uint16_t* __restrict__ xc) {
  const int64_t I = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (I >= nc) return;
  const float inv = scal[1];
  const float xi = u[I] * inv;
  float a = 0.f;
  const int64_t dpos = cdiag[I];
  for (int64_t q = cptr[I] + lane; q < cptr[I + 1]; q += 32)
    if (q != dpos) a = fmaf(wgt[q], u[ccol[q]] * inv, a);
  for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
  if (lane == 0) {
    x[I] = xi;
    ax[I] = a;
  }
  const int c = 2 * lane;
  const float h0 = fmaxf(fmaf(xi, w0[c], a * w0[64 + c]), 0.f);
  const float h1 = fmaxf(fmaf(xi, w0[c + 1], a * w0[64 + c + 1]), 0.f);
  *reinterpret_cast<uint32_t*>(xc + I * 128 + c) = pack2(f2bf(h0), f2bf(h1));
}

// ec = s * (h3 . wout); warp per row
__global__ void __launch_bounds__(kB)
    output_k(int64_t nc, const uint16_t* __restrict__ h3, const float* __restrict__ wout,
             const float* __restrict__ scal, float* __restrict__ y, float* __restrict__ ec) {
  const int64_t I = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (I >= nc) return;
  const uint32_t v = *reinterpret_cast<const uint32_t*>(h3 + I * 64 + 2 * lane);
  float s = bf2f(uint16_t(v & 0xffffu)) * wout[2 * lane] + bf2f(uint16_t(v >> 16)) * wout[2 * lane + 1];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) {
    y[I] = s;
    ec[I] = scal[0] * s;
  }
}

// Coarse operator applied to the network output, thread per coarse row:
//   (Ac ec)_I = (ec_I - sum_J w_IJ ec_J) / dinv_I     (Ac = D (I - W))
// with per-block partial sums of ec' rc and ec' Ac ec (two per block).
// Jacobi step on the coarse operator, written with w_IJ = -Ac_IJ / Ac_II
// and dinv = 1 / Ac_II: e_out = dinv r + sum_J w_IJ e_in,J (e_in == nullptr:
// e_out = dinv r, the step from zero).
__global__ void coarse_jacobi_k(int64_t nc, const int64_t* __restrict__ cptr,
                                const int32_t* __restrict__ ccol, const int32_t* __restrict__ cdiag,
                                const float* __restrict__ wgt, const float* __restrict__ dinv,
                                const float* __restrict__ rc, const float* __restrict__ ein,
                                float* __restrict__ eout) {
  const int64_t I = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (I >= nc) return;
  float v = dinv[I] * rc[I];
  if (ein) {
    const int64_t dpos = cdiag[I];
    for (int64_t q = cptr[I]; q < cptr[I + 1]; ++q)
      if (q != dpos) v = fmaf(wgt[q], ein[ccol[q]], v);
  }
  eout[I] = v;
}

__global__ void coarse_apply_k(int64_t nc, const int64_t* __restrict__ cptr,
                               const int32_t* __restrict__ ccol,
                               const int32_t* __restrict__ cdiag,
                               const float* __restrict__ wgt, const float* __restrict__ dinv,
                               const float* __restrict__ ec, const float* __restrict__ rc,
                               float* __restrict__ aec, float* __restrict__ partial) {
  __shared__ float red[2][kB / 32];
  const int64_t I = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float num = 0.f, den = 0.f;
  if (I < nc) {
    const float e = ec[I];
    float a = e;
    const int64_t dpos = cdiag[I];
    for (int64_t q = cptr[I]; q < cptr[I + 1]; ++q)
      if (q != dpos) a = fmaf(-wgt[q], ec[ccol[q]], a);
    const float d = dinv[I];
    const float v = d != 0.f ? a / d : 0.f;
    aec[I] = v;
    num = e * rc[I];
    den = e * v;
  }
  for (int off = 16; off > 0; off >>= 1) {
    num += __shfl_down_sync(0xffffffffu, num, off);
    den += __shfl_down_sync(0xffffffffu, den, off);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = num;
    red[1][threadIdx.x >> 5] = den;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int q = 0; q < kB / 32; ++q) {
      a += red[0][q];
      b += red[1][q];
    }
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

// Energy-optimal scaling of the coarse correction, fixed-order sums:
//   scal[2] = alpha = ec' rc / ec' Ac ec   (0 unless the denominator is > 0)
//   scal[3] = (ec' rc)^2 / ec' Ac ec       (A-norm error energy removed)
__global__ void __launch_bounds__(kB)
    alpha_k(int nblocks, const float* __restrict__ partial, float* __restrict__ scal) {
  __shared__ double red[kB];
  const double num = block_sum(nblocks, partial, 2, 0, red);
  const double den = block_sum(nblocks, partial, 2, 1, red);
  if (threadIdx.x == 0) {
    const bool ok = den > 0.0 && isfinite(num) && isfinite(den);
    scal[2] = ok ? float(num / den) : 0.f;
    scal[3] = ok ? float(num * num / den) : 0.f;
  }
}

// dL/dy for the scaled loss L = (cA - (ec' rc)^2 / ec' Ac ec) / eA:
//   dL/dy_I = s * (2 / eA) (alpha^2 (Ac ec)_I - alpha rc_I)   (Ac symmetric)
__global__ void loss_grad_k(int64_t nc, const float* __restrict__ aec,
                            const float* __restrict__ rc, const float* __restrict__ scal,
                            float inv_ea, float* __restrict__ dy) {
  const int64_t I = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (I >= nc) return;
  const float al = scal[2];
  dy[I] = scal[0] * 2.f * inv_ea * al * (al * aec[I] - rc[I]);
}

// dz3 = bf16(dy * wout * (h3 > 0)); per-block partial of dwout = h3^T dy.
__global__ void __launch_bounds__(kB)
    out_bwd_k(int64_t nc, const uint16_t* __restrict__ h3, const float* __restrict__ dy,
              const float* __restrict__ wout, uint16_t* __restrict__ dz,
              float* __restrict__ partial) {
  __shared__ float red[kB / 64][64];
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;  // (row, channel)
  const int c = threadIdx.x & 63;
  float g = 0.f;
  if (q < nc * 64) {
    const int64_t I = q >> 6;
    const float h = bf2f(h3[q]);
    const float d = dy[I];
    dz[q] = f2bf(h > 0.f ? d * wout[c] : 0.f);
    g = h * d;
  }
  red[threadIdx.x >> 6][c] = g;
  __syncthreads();
  if (threadIdx.x < 64) {
    float s = 0.f;
    for (int k = 0; k < kB / 64; ++k) s += red[k][threadIdx.x];
    partial[int64_t(blockIdx.x) * 64 + threadIdx.x] = s;
  }
}

// layer-0 weight-gradient partials: [x, ax]^T dz0 with dz0 = dh0 * (h0 > 0)
__global__ void __launch_bounds__(kB)
    layer0_bwd_k(int64_t nc, const float* __restrict__ dh, const uint16_t* __restrict__ xc,
                 const float* __restrict__ x, const float* __restrict__ ax,
                 float* __restrict__ partial) {
  __shared__ float r0[kB / 64][64], r1[kB / 64][64];
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int c = threadIdx.x & 63;
  float g0 = 0.f, g1 = 0.f;
  if (q < nc * 64) {
    const int64_t I = q >> 6;
    const float h = bf2f(xc[I * 128 + c]);
    const float d = h > 0.f ? dh[q] : 0.f;
    g0 = x[I] * d;
    g1 = ax[I] * d;
  }
  r0[threadIdx.x >> 6][c] = g0;
  r1[threadIdx.x >> 6][c] = g1;
  __syncthreads();
  if (threadIdx.x < 64) {
    float s0 = 0.f, s1 = 0.f;
    for (int k = 0; k < kB / 64; ++k) {
      s0 += r0[k][threadIdx.x];
      s1 += r1[k][threadIdx.x];
    }
    partial[int64_t(blockIdx.x) * 128 + threadIdx.x] = s0;
    partial[int64_t(blockIdx.x) * 128 + 64 + threadIdx.x] = s1;
  }
}

__global__ void adam_k(int n, float* __restrict__ p, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr,
                       float scale, float b1, float b2, float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] * scale;
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 copies of W1..W3: row-major (128 x 64) and transposed (64 x 128)
__global__ void to_bf16_k(const float* __restrict__ p, uint16_t* __restrict__ w,
                          uint16_t* __restrict__ wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * kIn2 * kHid) return;
  const int l = i / (kIn2 * kHid), r = i % (kIn2 * kHid);
  const int k = r / kHid, n = r % kHid;
  const uint16_t b = f2bf(p[kOffW1 + i]);
  w[i] = b;
  wt[l * kIn2 * kHid + n * kIn2 + k] = b;
}

// Galerkin sums Ac[q] = sum of the fine values mapped to coarse slot q:
// warp per slot, lanes stride the contribution list, fixed-order butterfly
// sum. (A diagonal slot collects every entry inside its aggregate, ~10^3
// after two aggregation passes, so a thread per slot serialised the kernel
// on those few slots.)
__global__ void __launch_bounds__(kB)
    galerkin_k(int64_t nnzc, const int64_t* __restrict__ gptr,
               const int32_t* __restrict__ gfine, const double* __restrict__ v,
               double* __restrict__ ac) {
  const int64_t q = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= nnzc) return;
  double s = 0.0;
  for (int64_t k = gptr[q] + lane; k < gptr[q + 1]; k += 32) s += v[gfine[k]];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) ac[q] = s;
}

__global__ void coarse_weights_k(int64_t nc, const int64_t* __restrict__ cptr,
                                 const int32_t* __restrict__ cdiag,
                                 const double* __restrict__ ac, float* __restrict__ wgt,
                                 float* __restrict__ dinv) {
  const int64_t I = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (I >= nc) return;
  const double d = ac[cdiag[I]];
  const double id = d != 0.0 ? 1.0 / d : 0.0;
  dinv[I] = float(id);
  for (int64_t q = cptr[I]; q < cptr[I + 1]; ++q)
    wgt[q] = q == cdiag[I] ? 0.f : float(-ac[q] * id);
}

// rc_I = sum of r over aggregate I: warp per aggregate, lanes stride the
// member list, fixed-order butterfly sum
__global__ void __launch_bounds__(kB)
    restrict_k(int64_t nc, const int64_t* __restrict__ mptr, const int32_t* __restrict__ mrows,
               const float* __restrict__ r, float* __restrict__ rc) {
  const int64_t I = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (I >= nc) return;
  float s = 0.f;
  for (int64_t k = mptr[I] + lane; k < mptr[I + 1]; k += 32) s += r[mrows[k]];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) rc[I] = s;
}

// z_i += alpha ec_agg(i), alpha read from the device
__global__ void prolong_add_k(int64_t nf, const int32_t* __restrict__ agg,
                              const float* __restrict__ ec, const float* __restrict__ alpha,
                              float* __restrict__ z) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < nf) z[i] += *alpha * ec[agg[i]];
}

uint64_t fnv1a(const void* data, size_t n) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

}  // namespace

// ---------------------------------------------------------------------------
void launch_gemm_fwd(const uint16_t* a, const uint16_t* wt, uint16_t* out,
                     int64_t m, int ldo, cudaStream_t s) {
  if (m > 0) gemm_fwd_k<<<gridn(m, 64), 128, 0, s>>>(a, wt, out, m, ldo);
}
void launch_gemm_dx(const uint16_t* dz, const uint16_t* w, float* dx, int64_t m,
                    cudaStream_t s) {
  if (m > 0) gemm_dx_k<<<gridn(m, 64), 128, 0, s>>>(dz, w, dx, m);
}
static int wgrad_blocks(int64_t m) {
  return int(std::max<int64_t>(1, std::min<int64_t>(4 * 152, (m + 63) / 64)));
}
void launch_gemm_wgrad(const uint16_t* xc, const uint16_t* dz, float* partial,
                       float* dw, int64_t m, cudaStream_t s) {
  const int nb = wgrad_blocks(m);
  gemm_wgrad_k<<<nb, 256, 0, s>>>(xc, dz, partial, m);
  colsum_k<<<gridn(128 * 64), kB, 0, s>>>(nb, 128 * 64, partial, dw, 1);
}
void launch_gemm_wgrad_tc(const uint16_t* xc, const uint16_t* dz, float* partial,
                          float* dw, int64_t m, cudaStream_t s) {
  const int nb = wgrad_blocks(m);
  launch_wgrad_partials_tc(xc, dz, partial, m, nb, s);
  colsum_k<<<gridn(128 * 64), kB, 0, s>>>(nb, 128 * 64, partial, dw, 1);
}

void launch_restrict(const CoarseLevel& cl, const float* r, float* rc, cudaStream_t s) {
  restrict_k<<<gridn(cl.nc * 32), kB, 0, s>>>(cl.nc, cl.mptr.p, cl.mrows.p, r, rc);
}
void launch_prolong_add(const CoarseLevel& cl, const float* ec, const float* alpha, float* z,
                        cudaStream_t s) {
  prolong_add_k<<<gridn(cl.nf), kB, 0, s>>>(cl.nf, cl.agg.p, ec, alpha, z);
}

// ---------------------------------------------------------------------------
// Plain aggregation of a graph (rows 0..R-1, CSR ptr/col including the
// diagonal): visiting rows in a fixed pseudo-random order, a row whose
// neighbours are all free starts an aggregate with them; leftover rows join
// the aggregate of their first aggregated neighbour (column order), or start
// their own. The seeded visiting order keeps the aggregates' shape
// independent of the node numbering (in bandwidth-reducing orders such as
// RCM, visiting rows in index order grows ragged aggregates: 240 instead of
// 87 FGMRES iterations on a 2.1M-node tet mesh). Deterministic.
static int32_t plain_aggregate(int64_t R, const int64_t* ptr, const int32_t* col,
                               std::vector<int32_t>& agg) {
  agg.assign(R, -1);
  int32_t na = 0;
  std::vector<int64_t> visit(R);
  std::iota(visit.begin(), visit.end(), 0);
  uint64_t st = 0x2545F4914F6CDD1Dull;  // xorshift64, fixed seed
  for (int64_t i = R - 1; i > 0; --i) {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    std::swap(visit[i], visit[int64_t(st % uint64_t(i + 1))]);
  }
  for (const int64_t r : visit) {
    if (agg[r] >= 0) continue;
    bool free_nbrs = true;
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p)
      if (agg[col[p]] >= 0) {
        free_nbrs = false;
        break;
      }
    if (!free_nbrs) continue;
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p) agg[col[p]] = na;
    agg[r] = na++;
  }
  for (int64_t r = 0; r < R; ++r) {
    if (agg[r] >= 0) continue;
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p)
      if (agg[col[p]] >= 0) {
        agg[r] = agg[col[p]];
        break;
      }
    if (agg[r] < 0) agg[r] = na++;
  }
  return na;
}

// The same aggregation over strong connections only: c is a strong
// neighbour of r when |a_rc| >= theta sqrt(|a_rr| |a_cc|) (the strength
// measure of smoothed aggregation). On stretched meshes the thin cells'
// couplings dominate, so the aggregates follow them (semi-coarsening). A
// row with no strong neighbour does not seed an aggregate; leftover rows
// join the aggregated neighbour they are most strongly coupled to, or
// start their own.
static int32_t strength_aggregate(int64_t R, const int64_t* ptr, const int32_t* col,
                                  const double* val, double theta, std::vector<int32_t>& agg) {
  std::vector<double> d(R, 0.0);
  for (int64_t r = 0; r < R; ++r)
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p)
      if (col[p] == r) d[r] = std::fabs(val[p]);
  std::vector<char> strong(size_t(ptr[R]), 0);
  for (int64_t r = 0; r < R; ++r)
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p)
      strong[p] = col[p] != r && std::fabs(val[p]) >= theta * std::sqrt(d[r] * d[col[p]]);
  agg.assign(R, -1);
  int32_t na = 0;
  std::vector<int64_t> visit(R);
  std::iota(visit.begin(), visit.end(), 0);
  uint64_t st = 0x2545F4914F6CDD1Dull;  // xorshift64, fixed seed (as plain_aggregate)
  for (int64_t i = R - 1; i > 0; --i) {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    std::swap(visit[i], visit[int64_t(st % uint64_t(i + 1))]);
  }
  for (const int64_t r : visit) {
    if (agg[r] >= 0) continue;
    int nstrong = 0;
    bool free_nbrs = true;
    for (int64_t p = ptr[r]; p < ptr[r + 1] && free_nbrs; ++p)
      if (strong[p]) {
        ++nstrong;
        if (agg[col[p]] >= 0) free_nbrs = false;
      }
    if (!free_nbrs || nstrong == 0) continue;
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p)
      if (strong[p]) agg[col[p]] = na;
    agg[r] = na++;
  }
  for (int64_t r = 0; r < R; ++r) {
    if (agg[r] >= 0) continue;
    int64_t best = -1;
    double bw = -1.0;
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p)
      if (col[p] != r && agg[col[p]] >= 0 && std::fabs(val[p]) > bw) {
        bw = std::fabs(val[p]);
        best = p;
      }
    agg[r] = best >= 0 ? agg[col[best]] : na++;
  }
  return na;
}

// Graph of the aggregates (sorted, unique columns) from a fine graph.
static void aggregate_graph(int64_t R, const int64_t* ptr, const int32_t* col,
                            const std::vector<int32_t>& agg, int64_t nagg,
                            std::vector<int64_t>& cptr, std::vector<int32_t>& ccol) {
  std::vector<std::vector<int32_t>> cols(nagg);
  for (int64_t r = 0; r < R; ++r)
    for (int64_t p = ptr[r]; p < ptr[r + 1]; ++p) cols[agg[r]].push_back(agg[col[p]]);
  cptr.assign(nagg + 1, 0);
  for (int64_t I = 0; I < nagg; ++I) {
    auto& v = cols[I];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    cptr[I + 1] = cptr[I] + int64_t(v.size());
  }
  ccol.resize(cptr[nagg]);
  for (int64_t I = 0; I < nagg; ++I)
    std::copy(cols[I].begin(), cols[I].end(), ccol.begin() + cptr[I]);
}

// Aggregation applied `passes` times (aggregates of aggregates), composed
// into one fine-row -> aggregate map.
void CoarseLevel::setup(const HostGraph& g, int npasses, cudaStream_t s, const double* values,
                        double theta) {
  if (g.num_dof != 1) fail(NW_INVALID_ARG, "the learned preconditioner needs num_dof 1");
  if (npasses < 1 || npasses > 4) fail(NW_INVALID_ARG, "aggregation passes must be 1..4");
  passes = npasses;
  strength = values ? theta : 0.0;
  const int64_t R = g.node_rows;
  nf = R;
  int32_t na = 0;
  if (strength > 0.0) {
    // every pass on the Galerkin values of the previous level
    std::vector<int64_t> lp(g.nrow_ptr);
    std::vector<int32_t> lc(g.ncol);
    std::vector<double> lv(values, values + g.nrow_ptr[R]);
    std::vector<int32_t> a;
    int64_t lr = R;
    for (int pass = 0; pass < npasses; ++pass) {
      const int32_t n2 = strength_aggregate(lr, lp.data(), lc.data(), lv.data(), strength, a);
      if (pass == 0) {
        agg_h = a;
      } else {
        for (int64_t r = 0; r < R; ++r) agg_h[r] = a[agg_h[r]];
      }
      if (pass + 1 < npasses) {
        std::vector<int64_t> p1;
        std::vector<int32_t> c1;
        aggregate_graph(lr, lp.data(), lc.data(), a, n2, p1, c1);
        std::vector<double> v1(size_t(p1[n2]), 0.0);
        for (int64_t r = 0; r < lr; ++r)
          for (int64_t p = lp[r]; p < lp[r + 1]; ++p) {
            const int32_t I = a[r], J = a[lc[p]];
            const auto b = c1.begin() + p1[I], e = c1.begin() + p1[I + 1];
            v1[size_t(std::lower_bound(b, e, J) - c1.begin())] += lv[p];
          }
        lp.swap(p1);
        lc.swap(c1);
        lv.swap(v1);
        lr = n2;
      }
      na = n2;
    }
  } else {
    na = plain_aggregate(R, g.nrow_ptr.data(), g.ncol.data(), agg_h);
    for (int pass = 1; pass < npasses; ++pass) {
      std::vector<int64_t> p1;
      std::vector<int32_t> c1, agg2;
      aggregate_graph(R, g.nrow_ptr.data(), g.ncol.data(), agg_h, na, p1, c1);
      na = plain_aggregate(na, p1.data(), c1.data(), agg2);
      for (int64_t r = 0; r < R; ++r) agg_h[r] = agg2[agg_h[r]];
    }
  }
  nc = na;
  // members
  std::vector<int64_t> mp(nc + 1, 0);
  for (int64_t r = 0; r < R; ++r) mp[agg_h[r] + 1]++;
  for (int64_t I = 0; I < nc; ++I) mp[I + 1] += mp[I];
  std::vector<int32_t> mr(R);
  {
    std::vector<int64_t> pos(mp.begin(), mp.end() - 1);
    for (int64_t r = 0; r < R; ++r) mr[pos[agg_h[r]]++] = int32_t(r);
  }
  // coarse graph and Galerkin contribution lists over the fine CSR
  aggregate_graph(R, g.nrow_ptr.data(), g.ncol.data(), agg_h, nc, cptr_h, ccol_h);
  nnzc = cptr_h[nc];
  cdiag_h.assign(nc, -1);
  for (int64_t I = 0; I < nc; ++I)
    for (int64_t q = cptr_h[I]; q < cptr_h[I + 1]; ++q)
      if (ccol_h[q] == I) cdiag_h[I] = int32_t(q);
  auto slot = [&](int64_t I, int32_t J) {
    auto b = ccol_h.begin() + cptr_h[I], e = ccol_h.begin() + cptr_h[I + 1];
    return int64_t(std::lower_bound(b, e, J) - ccol_h.begin());
  };
  rev_h.resize(nnzc);
  for (int64_t I = 0; I < nc; ++I)
    for (int64_t q = cptr_h[I]; q < cptr_h[I + 1]; ++q) rev_h[q] = int32_t(slot(ccol_h[q], int32_t(I)));
  // fine nnz p (row r, col c) -> coarse slot
  const int64_t nnz = g.nrow_ptr[R];
  std::vector<int64_t> gcount(nnzc + 1, 0);
  std::vector<int32_t> pslot(nnz);
  for (int64_t r = 0; r < R; ++r)
    for (int64_t p = g.nrow_ptr[r]; p < g.nrow_ptr[r + 1]; ++p) {
      pslot[p] = int32_t(slot(agg_h[r], agg_h[g.ncol[p]]));
      gcount[pslot[p] + 1]++;
    }
  for (int64_t q = 0; q < nnzc; ++q) gcount[q + 1] += gcount[q];
  std::vector<int32_t> gf(nnz);
  {
    std::vector<int64_t> pos(gcount.begin(), gcount.end() - 1);
    for (int64_t p = 0; p < nnz; ++p) gf[pos[pslot[p]]++] = int32_t(p);
  }
  agg.upload(agg_h, s);
  mptr.upload(mp, s);
  mrows.upload(mr, s);
  cptr.upload(cptr_h, s);
  ccol.upload(ccol_h, s);
  cdiag.upload(cdiag_h, s);
  rev.upload(rev_h, s);
  gptr.upload(gcount, s);
  gfine.upload(gf, s);
  ac.resize(nnzc);
  wgt.resize(nnzc);
  dinv.resize(nc);
}

void CoarseLevel::refresh(const double* fine_values, cudaStream_t s) {
  galerkin_k<<<gridn(nnzc * 32), kB, 0, s>>>(nnzc, gptr.p, gfine.p, fine_values, ac.p);
  coarse_weights_k<<<gridn(nc), kB, 0, s>>>(nc, cptr.p, cdiag.p, ac.p, wgt.p, dinv.p);
  NW_CUDA(cudaGetLastError());
}

void NetWork::resize(int64_t n) {
  if (n == nc && u.p) return;
  nc = n;
  u.resize(n);
  x.resize(n);
  ax.resize(n);
  y.resize(n);
  dy.resize(n);
  scal.resize(4);
  partial.resize(2 * gridn(n) + 2);
  aec.resize(n);
  ec.resize(n);
  part2.resize(size_t(gridn(n * 64)) * 128);
  xc1.resize(n * 128);
  xc2.resize(n * 128);
  xc3.resize(n * 128);
  h3.resize(n * 64);
  dz.resize(n * 64);
  dxc.resize(n * 128);
  dh.resize(n * 64);
}

LearnedNet::~LearnedNet() { clear_data(); }

void LearnedNet::init(uint64_t sd, cudaStream_t s) {
  seed = sd;
  params_h.assign(kNumParams, 0.f);
  uint64_t st = sd * 0x9E3779B97F4A7C15ull + 12345;
  auto uni = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return float((st >> 11) * 0x1.0p-53) * 2.f - 1.f;
  };
  const float a0 = std::sqrt(6.f / 2.f), a1 = std::sqrt(6.f / float(kIn2)),
              ao = std::sqrt(3.f / float(kHid));
  for (int i = 0; i < 2 * kHid; ++i) params_h[kOffW0 + i] = a0 * uni();
  for (int i = 0; i < 3 * kIn2 * kHid; ++i) params_h[kOffW1 + i] = a1 * uni();
  for (int i = 0; i < kHid; ++i) params_h[kOffWout + i] = ao * uni();
  upload(s);
  grads.resize(kNumParams);
  adam_m.resize(kNumParams);
  adam_v.resize(kNumParams);
  NW_CUDA(cudaMemsetAsync(grads.p, 0, kNumParams * 4, s));
  NW_CUDA(cudaMemsetAsync(adam_m.p, 0, kNumParams * 4, s));
  NW_CUDA(cudaMemsetAsync(adam_v.p, 0, kNumParams * 4, s));
  adam_step = 0;
}

void LearnedNet::upload(cudaStream_t s) {
  params.upload(params_h, s);
  wbf.resize(3 * kIn2 * kHid);
  wtbf.resize(3 * kIn2 * kHid);
  sync_bf16(s);
}

void LearnedNet::download(cudaStream_t s) {
  params_h.resize(kNumParams);
  NW_CUDA(cudaMemcpyAsync(params_h.data(), params.p, kNumParams * 4, cudaMemcpyDeviceToHost, s));
  NW_CUDA(cudaStreamSynchronize(s));
}

void LearnedNet::sync_bf16(cudaStream_t s) {
  to_bf16_k<<<gridn(3 * kIn2 * kHid), kB, 0, s>>>(params.p, wbf.p, wtbf.p);
  NW_CUDA(cudaGetLastError());
}

void LearnedNet::clear_data() {
  for (auto* p : sys_wgt) delete p;
  for (auto* p : sys_dinv) delete p;
  for (auto* p : pair_rc) delete p;
  sys_wgt.clear();
  sys_dinv.clear();
  pair_rc.clear();
  pair_system.clear();
  pair_ea.clear();
  pair_ca.clear();
  npairs = nsystems = 0;
}

void LearnedNet::forward(const CoarseLevel& cl, const float* wgt, const float* dinv,
                         const float* rc, float* ec, cudaStream_t s) {
  const int64_t nc = cl.nc;
  work.resize(nc);
  const unsigned gw = gridn(nc * 32);  // warp per row
  input_k<<<gridn(nc), kB, 0, s>>>(nc, rc, dinv, work.u.p, work.partial.p);
  rms_k<<<1, kB, 0, s>>>(int(gridn(nc)), work.partial.p, nc, work.scal.p);
  layer0_k<<<gw, kB, 0, s>>>(nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, wgt, work.u.p, work.scal.p,
                             params.p + kOffW0, work.x.p, work.ax.p, work.xc1.p);
  uint16_t* xcs[4] = {work.xc1.p, work.xc2.p, work.xc3.p, nullptr};
  for (int l = 0; l < 3; ++l) {
    agg_fwd_k<<<gw, kB, 0, s>>>(nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, wgt, xcs[l]);
    uint16_t* out = l < 2 ? xcs[l + 1] : work.h3.p;
    launch_gemm_fwd_tma(xcs[l], wtbf.p + size_t(l) * kIn2 * kHid, out, nc, l < 2 ? 128 : 64, s);
  }
  output_k<<<gw, kB, 0, s>>>(nc, work.h3.p, params.p + kOffWout, work.scal.p, work.y.p, ec);
  NW_CUDA(cudaGetLastError());
}

void LearnedNet::coarse_correction(const CoarseLevel& cl, const float* rc, float* ec,
                                   cudaStream_t s) {
  const int nb = int(gridn(cl.nc));
  if (coarse_mode == 0) {
    forward(cl, cl.wgt.p, cl.dinv.p, rc, ec, s);
  } else {
    work.resize(cl.nc);
    coarse_jacobi_k<<<nb, kB, 0, s>>>(cl.nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, cl.wgt.p, cl.dinv.p, rc,
                                      nullptr, coarse_mode == 1 ? ec : work.u.p);
    if (coarse_mode == 2)
      coarse_jacobi_k<<<nb, kB, 0, s>>>(cl.nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, cl.wgt.p, cl.dinv.p, rc,
                                        work.u.p, ec);
  }
  coarse_apply_k<<<nb, kB, 0, s>>>(cl.nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, cl.wgt.p, cl.dinv.p,
                                   ec, rc, work.aec.p, work.partial.p);
  alpha_k<<<1, kB, 0, s>>>(nb, work.partial.p, work.scal.p);
  NW_CUDA(cudaGetLastError());
}

double LearnedNet::forward_backward(const CoarseLevel& cl, const float* wgt,
                                    const float* dinv, const float* rc, double ea,
                                    double ca, cudaStream_t s, bool with_grad) {
  const int64_t nc = cl.nc;
  work.resize(nc);
  float* ec = work.ec.p;
  forward(cl, wgt, dinv, rc, ec, s);
  const unsigned gw = gridn(nc * 32);
  const int nb = int(gridn(nc));
  coarse_apply_k<<<nb, kB, 0, s>>>(nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, wgt, dinv, ec, rc,
                                   work.aec.p, work.partial.p);
  alpha_k<<<1, kB, 0, s>>>(nb, work.partial.p, work.scal.p);
  float sc[4];
  NW_CUDA(cudaMemcpyAsync(sc, work.scal.p, sizeof(sc), cudaMemcpyDeviceToHost, s));
  NW_CUDA(cudaStreamSynchronize(s));
  const double loss = (ca - double(sc[3])) / ea;
  if (!with_grad) return loss;
  loss_grad_k<<<nb, kB, 0, s>>>(nc, work.aec.p, rc, work.scal.p, float(1.0 / ea), work.dy.p);
  // output layer
  const int nb64 = int(gridn(nc * 64));
  float* part2 = work.part2.p;
  wpartial.resize(size_t(wgrad_blocks(nc)) * 128 * 64);
  out_bwd_k<<<nb64, kB, 0, s>>>(nc, work.h3.p, work.dy.p, params.p + kOffWout, work.dz.p, part2);
  colsum_k<<<1, 64, 0, s>>>(nb64, 64, part2, grads.p + kOffWout, 1);
  uint16_t* xcs[3] = {work.xc1.p, work.xc2.p, work.xc3.p};
  for (int l = 2; l >= 0; --l) {
    // dW_l += X_l^T dZ_l ; dX_l = dZ_l W_l^T
    launch_gemm_wgrad_tc(xcs[l], work.dz.p, wpartial.p, grads.p + kOffW1 + size_t(l) * kIn2 * kHid,
                         nc, s);
    launch_gemm_dx_tma(work.dz.p, wbf.p + size_t(l) * kIn2 * kHid, work.dxc.p, nc, s);
    agg_bwd_k<<<gw, kB, 0, s>>>(nc, cl.cptr.p, cl.ccol.p, cl.cdiag.p, cl.rev.p, wgt, work.dxc.p,
                                work.dh.p);
    if (l > 0) mask_k<<<nb64, kB, 0, s>>>(nc, work.dh.p, xcs[l], 128, work.dz.p);
  }
  layer0_bwd_k<<<nb64, kB, 0, s>>>(nc, work.dh.p, work.xc1.p, work.x.p, work.ax.p, part2);
  colsum_k<<<1, 128, 0, s>>>(nb64, 128, part2, grads.p + kOffW0, 1);
  NW_CUDA(cudaGetLastError());
  NW_CUDA(cudaStreamSynchronize(s));
  return loss;
}

void LearnedNet::adam(double lr, double scale, cudaStream_t s) {
  ++adam_step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, float(adam_step)), c2 = 1.f - std::pow(b2, float(adam_step));
  adam_k<<<gridn(kNumParams), kB, 0, s>>>(kNumParams, params.p, grads.p, adam_m.p, adam_v.p,
                                          float(lr), float(scale), b1, b2, c1, c2, 1e-8f);
  NW_CUDA(cudaMemsetAsync(grads.p, 0, kNumParams * 4, s));
  sync_bf16(s);
}

void save_params(const std::string& path, const std::vector<float>& p, uint64_t step) {
  std::ofstream f(path, std::ios::binary);
  if (!f) fail(NW_INVALID_ARG, "cannot open " + path + " for writing");
  const char magic[8] = {'N', 'W', 'G', 'N', 'N', '0', '0', '1'};
  const uint32_t hdr[4] = {uint32_t(kHid), uint32_t(kIn2), 4u, uint32_t(p.size())};
  const uint64_t sum = fnv1a(p.data(), p.size() * sizeof(float));
  f.write(magic, 8);
  f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
  f.write(reinterpret_cast<const char*>(&step), 8);
  f.write(reinterpret_cast<const char*>(p.data()), p.size() * sizeof(float));
  f.write(reinterpret_cast<const char*>(&sum), 8);
  if (!f) fail(NW_INVALID_ARG, "write failed: " + path);
}

void load_params(const std::string& path, std::vector<float>& p) {
  std::ifstream f(path, std::ios::binary);
  if (!f) fail(NW_INVALID_ARG, "cannot open " + path);
  char magic[8];
  uint32_t hdr[4];
  uint64_t step = 0, sum = 0;
  f.read(magic, 8);
  f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
  f.read(reinterpret_cast<char*>(&step), 8);
  if (!f || std::memcmp(magic, "NWGNN001", 8) != 0) fail(NW_INVALID_ARG, "not a network weight file: " + path);
  if (hdr[0] != uint32_t(kHid) || hdr[1] != uint32_t(kIn2) || hdr[2] != 4u || hdr[3] != uint32_t(kNumParams))
    fail(NW_INVALID_ARG, "weight file shape does not match this network: " + path);
  std::vector<float> q(kNumParams);
  f.read(reinterpret_cast<char*>(q.data()), q.size() * sizeof(float));
  f.read(reinterpret_cast<char*>(&sum), 8);
  if (!f) fail(NW_INVALID_ARG, "truncated weight file: " + path);
  if (sum != fnv1a(q.data(), q.size() * sizeof(float)))
    fail(NW_INVALID_ARG, "weight file checksum mismatch: " + path);
  p.swap(q);
}

}  // namespace nw
