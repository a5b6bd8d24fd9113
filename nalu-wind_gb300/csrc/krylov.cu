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
// bitwise reproducible run to run.
//
// The mixed-precision method keeps FP64 for the outer true residual
// (iterative refinement), the Gram-Schmidt dot products and the Hessenberg
// least squares; its inner GMRES stores the basis in FP32 and runs the SpMV
// and the preconditioner in FP32. The inner dot products multiply FP32
// operands exactly (product + FMA error term) and accumulate them with a
// compensated two-float sum (Dekker/Knuth error-free transformations) on
// the FP32 pipes, then combine threads in FP64: FP64-accurate dots without
// spending GB300's scarce FP64 throughput.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "krylov.h"

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
  for (int64_t p = s + lane; p < e; p += LANES)
    acc += ACC(v[p]) * ACC(x[ci[p]]);
#pragma unroll
  for (int off = LANES / 2; off > 0; off >>= 1)
    acc += __shfl_down_sync(0xffffffffu, acc, off, LANES);
  if (lane == 0) y[row] = b ? XT(ACC(b[row]) - acc) : XT(acc);
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
// Deterministic multi-dot: out[k] = sum_i V[k][i] * w[i] for k < nv.
// Stage 1 writes per-block partials (fixed grid); stage 2 sums them in a
// fixed tree order.
__device__ __forceinline__ void acc_prod(double a, double b, double& s,
                                         double& c) {
  s = fma(a, b, s);
  (void)c;
}
// Exact FP32 product p + e, added to (s, c) with a two-sum; c collects the
// rounding errors.
__device__ __forceinline__ void acc_prod(float a, float b, float& s,
                                         float& c) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float t = s + p;
  const float bp = t - s;
  const float err = (s - (t - bp)) + (p - bp);
  s = t;
  c += err + e;
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
    mdot_k(int64_t n, int nv, const T* __restrict__ V, int64_t ld,
           const T* __restrict__ w, double* __restrict__ partial) {
  __shared__ double red[kTile][kBlock / 32];
  const int G = gridDim.x;
  for (int k0 = 0; k0 < nv; k0 += kTile) {
    const int kt = min(kTile, nv - k0);
    T s[kTile], c[kTile];
#pragma unroll
    for (int k = 0; k < kTile; ++k) s[k] = c[k] = T(0);
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += int64_t(G) * blockDim.x) {
      const T wi = w[i];
#pragma unroll
      for (int k = 0; k < kTile; ++k)
        if (k < kt) acc_prod(V[int64_t(k0 + k) * ld + i], wi, s[k], c[k]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kTile; ++k) {
      double v = double(s[k]) + double(c[k]);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, off);
      if (lane == 0) red[k][warp] = v;
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

// w -= sum_k h[k] V[k]  (h on the device, FP64)
template <typename T>
__global__ void __launch_bounds__(kBlock)
    maxpy_k(int64_t n, int nv, const T* __restrict__ V, int64_t ld,
            const double* __restrict__ h, T* __restrict__ w) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T acc = w[i];
  for (int k = 0; k < nv; ++k) acc -= T(h[k]) * V[int64_t(k) * ld + i];
  w[i] = acc;
}

// y = x / nrm[0] (y = 0 when the norm is zero). One FP64 reciprocal per
// block, then a multiply per element in the vector's own precision.
template <typename T>
__global__ void scale_by_norm_k(int64_t n, const T* __restrict__ x,
                                T* __restrict__ y,
                                const double* __restrict__ nrm) {
  __shared__ double inv;
  if (threadIdx.x == 0) {
    const double hn = nrm[0];
    inv = hn != 0.0 ? 1.0 / hn : 0.0;
  }
  __syncthreads();
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] = x[i] * T(inv);
}

__global__ void sqrt_scalar_k(double* s) { s[0] = sqrt(s[0]); }

template <typename T>
__global__ void jacobi_k(int64_t n, const T* __restrict__ rd,
                         const T* __restrict__ x, T* __restrict__ y) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * rd[i];
}

// one colour of a Gauss-Seidel sweep: rows of this colour are mutually
// independent, so they relax in parallel using the current y.
template <typename VT, typename T>
__global__ void __launch_bounds__(kBlock)
    gs_color_k(int64_t cnt, const int32_t* __restrict__ rows,
               const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
               const VT* __restrict__ v, const T* __restrict__ rd,
               const T* __restrict__ x, T* __restrict__ y) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t i = rows[k];
  T s = x[i];
  for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
    const int32_t j = ci[p];
    if (j != i) s -= T(v[p]) * y[j];
  }
  y[i] = s * rd[i];
}

template <typename T>
__global__ void fill_k(int64_t n, T* y, T val) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = val;
}

__global__ void rdiag_k(int64_t n, const int64_t* __restrict__ rp,
                        const int32_t* __restrict__ ci,
                        const double* __restrict__ v, double* __restrict__ rd,
                        float* __restrict__ rd32) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int64_t p = rp[i]; p < rp[i + 1]; ++p)
    if (ci[p] == i) d = v[p];
  const double r = 1.0 / d;
  rd[i] = r;
  if (rd32) rd32[i] = float(r);
}

template <typename A, typename B>
__global__ void convert_k(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = B(a[i]);
}

// x += alpha * y (FP64)
__global__ void axpy_k(int64_t n, double alpha, const double* __restrict__ y,
                       double* __restrict__ x) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] += alpha * y[i];
}
// x += y (y FP32), mixed correction
__global__ void add_f32_k(int64_t n, const float* __restrict__ y,
                          double* __restrict__ x) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] += double(y[i]);
}
// p = z + beta p
__global__ void xpby_k(int64_t n, const double* __restrict__ z, double beta,
                       double* __restrict__ p) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] = z[i] + beta * p[i];
}
// y = sum_k c[k] V[k] (c on host -> passed in device scalar array)
template <typename T>
__global__ void combine_k(int64_t n, int nv, const T* __restrict__ V,
                          int64_t ld, const double* __restrict__ c,
                          T* __restrict__ y) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  for (int k = 0; k < nv; ++k) acc += c[k] * double(V[int64_t(k) * ld + i]);
  y[i] = T(acc);
}

inline unsigned grid1(int64_t n) { return unsigned((n + kBlock - 1) / kBlock); }

}  // namespace

// ---------------------------------------------------------------------------
KrylovSolver::~KrylovSolver() {
  if (h_pinned_) cudaFreeHost(h_pinned_);
}

void KrylovSolver::setup(const DevCsr& A, int m, cudaStream_t s) {
  A_ = A;
  m_ = std::max(1, m);
  const int64_t n = A.n;
  int dev = 0;
  NW_CUDA(cudaGetDevice(&dev));
  int sms = 0;
  NW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  red_blocks_ = int(std::max<int64_t>(1, std::min<int64_t>(4 * sms, (n + kBlock - 1) / kBlock)));
  rdiag_.resize(n);
  V_.resize(size_t(m_ + 1) * n);
  Z_.release();
  w_.resize(n);
  z_.resize(n);
  r_.resize(n);
  partial_.resize(size_t(m_ + 2) * red_blocks_);
  scal_.resize(4 * (m_ + 4));
  if (!h_pinned_) NW_CUDA(cudaMallocHost(&h_pinned_, sizeof(double) * 4 * 1024));
  f32_valid_ = false;
  refresh(s);
}

void KrylovSolver::refresh(cudaStream_t s) {
  if (A_.n == 0) return;
  rdiag_k<<<grid1(A_.n), kBlock, 0, s>>>(A_.n, A_.row_ptr, A_.col_idx,
                                          A_.values, rdiag_.p, nullptr);
  NW_CUDA(cudaGetLastError());
  f32_valid_ = false;
}

void KrylovSolver::ensure_f32(cudaStream_t s) {
  if (f32_valid_) return;
  const int64_t n = A_.n;
  vals32_.resize(A_.nnz);
  rdiag32_.resize(n);
  V32_.resize(size_t(m_ + 1) * n);
  w32_.resize(n);
  z32_.resize(n);
  r32_.resize(n);
  convert_k<double, float><<<grid1(A_.nnz), kBlock, 0, s>>>(A_.nnz, A_.values,
                                                             vals32_.p);
  convert_k<double, float><<<grid1(n), kBlock, 0, s>>>(n, rdiag_.p, rdiag32_.p);
  NW_CUDA(cudaGetLastError());
  f32_valid_ = true;
}

void KrylovSolver::spmv(const double* x, double* y, cudaStream_t s) const {
  spmv_launch<double, double, double>(A_.lanes, A_.n, A_.row_ptr, A_.col_idx,
                                      A_.values, x, nullptr, y, s);
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
  } else if (pc.kind == NW_PC_SGS) {
    fill_k<T><<<grid1(n), kBlock, 0, s>>>(n, y, T(0));
    const int nc = int(pc.color_ptr.size()) - 1;
    for (int c = 0; c < nc; ++c) {
      const int64_t b = pc.color_ptr[c], cnt = pc.color_ptr[c + 1] - b;
      if (cnt) gs_color_k<VT, T><<<grid1(cnt), kBlock, 0, s>>>(
          cnt, pc.color_rows + b, rp, ci, v, rd, x, y);
    }
    for (int c = nc - 1; c >= 0; --c) {
      const int64_t b = pc.color_ptr[c], cnt = pc.color_ptr[c + 1] - b;
      if (cnt) gs_color_k<VT, T><<<grid1(cnt), kBlock, 0, s>>>(
          cnt, pc.color_rows + b, rp, ci, v, rd, x, y);
    }
  } else {
    fail(NW_INVALID_ARG, "preconditioner not available for this precision");
  }
  NW_CUDA(cudaGetLastError());
}

}  // namespace

void KrylovSolver::apply_precond(const Precond& pc, const double* x, double* y,
                                 cudaStream_t s) {
  if (pc.kind == NW_PC_LEARNED) {
    if (!pc.apply_fn) fail(NW_INVALID_ARG, "learned preconditioner not set");
    pc.apply_fn(x, y, s);
    return;
  }
  precond_apply_t<double, double>(pc, A_.n, A_.row_ptr, A_.col_idx, A_.values,
                                  rdiag_.p, x, y, s);
}

SolveResult KrylovSolver::solve(const nw_solver_cfg& cfg, double tol,
                                const Precond& pc, const double* b, double* x,
                                cudaStream_t s) {
  if (cfg.precision == NW_PREC_MIXED) return mixed(cfg, tol, pc, b, x, s);
  if (cfg.method == NW_CG) return cg(cfg, tol, pc, b, x, s);
  return gmres(cfg, tol, pc, b, x,
               cfg.method == NW_FGMRES || pc.kind == NW_PC_LEARNED, s);
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
  std::vector<double> H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  double* V = V_.p;
  double beta = bnorm;
  NW_CUDA(cudaMemcpyAsync(r_.p, b, n * sizeof(double),
                          cudaMemcpyDeviceToDevice, s));
  double rel = 1.0;
  int its = 0;
  bool done = false;
  double* hs = scal_.p;             // h (m+1)
  double* h2 = scal_.p + (m_ + 2);  // second-pass h, then norm
  while (!done && its < cfg.max_iterations) {
    // V0 = r / beta
    NW_CUDA(cudaMemcpyAsync(h2, &beta, sizeof(double), cudaMemcpyHostToDevice, s));
    scale_by_norm_k<double><<<grid1(n), kBlock, 0, s>>>(n, r_.p, V, h2);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && its < cfg.max_iterations; ++j) {
      double* vj = V + size_t(j) * n;
      double* zj = flexible ? Z_.p + size_t(j) * n : z_.p;
      apply_precond(pc, vj, zj, s);
      spmv(zj, w_.p, s);
      // two classical Gram-Schmidt passes, coefficients kept on the device
      mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, j + 1, V, n, w_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, hs, 0, nullptr);
      maxpy_k<double><<<grid1(n), kBlock, 0, s>>>(n, j + 1, V, n, hs, w_.p);
      mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, j + 1, V, n, w_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, h2 + 1, 1, hs);
      maxpy_k<double><<<grid1(n), kBlock, 0, s>>>(n, j + 1, V, n, h2 + 1, w_.p);
      mdot_k<double><<<red_blocks_, kBlock, 0, s>>>(n, 1, w_.p, 0, w_.p, partial_.p);
      reduce_partials_k<<<1, kBlock, 0, s>>>(red_blocks_, partial_.p, h2, 0, nullptr);
      sqrt_scalar_k<<<1, 1, 0, s>>>(h2);
      scale_by_norm_k<double><<<grid1(n), kBlock, 0, s>>>(n, w_.p, V + size_t(j + 1) * n, h2);
      NW_CUDA(cudaGetLastError());
      NW_CUDA(cudaMemcpyAsync(h_pinned_, hs, sizeof(double) * (j + 1),
                              cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaMemcpyAsync(h_pinned_ + (j + 1), h2, sizeof(double),
                              cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaStreamSynchronize(s));
      const double hn = h_pinned_[j + 1];
      for (int k = 0; k <= j; ++k) H[size_t(k) * m + j] = h_pinned_[k];
      H[size_t(j + 1) * m + j] = hn;
      for (int k = 0; k < j; ++k) {
        const double a = H[size_t(k) * m + j], bb = H[size_t(k + 1) * m + j];
        H[size_t(k) * m + j] = cs[k] * a + sn[k] * bb;
        H[size_t(k + 1) * m + j] = -sn[k] * a + cs[k] * bb;
      }
      const double a = H[size_t(j) * m + j], bb = H[size_t(j + 1) * m + j];
      const double den = std::sqrt(a * a + bb * bb);
      if (!(den > 0.0) || !std::isfinite(den)) {
        res.status = std::isfinite(den) ? NW_BREAKDOWN : NW_NAN_DETECTED;
        done = true;
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
      if (!std::isfinite(rel)) {
        res.status = NW_NAN_DETECTED;
        done = true;
        ++j;
        break;
      }
      if (rel <= tol || hn == 0.0) {
        done = true;
        ++j;
        break;
      }
    }
    const int kk = j;
    for (int i = kk - 1; i >= 0; --i) {
      double sum = g[i];
      for (int l = i + 1; l < kk; ++l) sum -= H[size_t(i) * m + l] * y[l];
      y[i] = sum / H[size_t(i) * m + i];
    }
    if (kk > 0) {
      NW_CUDA(cudaMemcpyAsync(h2, y.data(), sizeof(double) * kk,
                              cudaMemcpyHostToDevice, s));
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
    spmv_launch<double, double, double>(A_.lanes, n, A_.row_ptr, A_.col_idx,
                                        A_.values, x, b, r_.p, s);
    beta = std::sqrt(dot(r_.p, r_.p, s));
    if (beta == 0.0) break;
  }
  spmv_launch<double, double, double>(A_.lanes, n, A_.row_ptr, A_.col_idx,
                                      A_.values, x, b, r_.p, s);
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
  spmv_launch<double, double, double>(A_.lanes, n, A_.row_ptr, A_.col_idx,
                                      A_.values, x, b, r, s);
  res.final_abs = std::sqrt(dot(r, r, s));
  res.final_rel = rel;
  res.iterations = its;
  res.converged = rel <= tol ? 1 : 0;
  if (res.status == NW_OK && !res.converged) res.status = NW_NOT_CONVERGED;
  return res;
}

// Mixed precision: FP64 iterative refinement around an FP32 inner GMRES.
// Outer: r = b - A x in FP64, stop when ||r||/||b|| <= tol. Inner: GMRES
// restarted once per outer step on A d = r in FP32 storage (FP32 SpMV with
// FP32 accumulation, FP32 Jacobi/SGS), FP64-accurate Gram-Schmidt dots,
// FP64 Hessenberg least squares on the host; x += d in FP64.
SolveResult KrylovSolver::mixed(const nw_solver_cfg& cfg, double tol,
                                const Precond& pc, const double* b, double* x,
                                cudaStream_t s) {
  const int64_t n = A_.n;
  ensure_f32(s);
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
  std::vector<double> H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  float* V = V32_.p;
  double* hs = scal_.p;
  double* h2 = scal_.p + (m_ + 2);
  double rel = 1.0;
  int its = 0, outer = 0;
  NW_CUDA(cudaMemcpyAsync(r_.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  double rnorm = bnorm;
  while (its < cfg.max_iterations) {
    ++outer;
    // inner: solve A d = r (scaled) in FP32
    convert_k<double, float><<<grid1(n), kBlock, 0, s>>>(n, r_.p, r32_.p);
    NW_CUDA(cudaMemcpyAsync(h2, &rnorm, sizeof(double), cudaMemcpyHostToDevice, s));
    scale_by_norm_k<float><<<grid1(n), kBlock, 0, s>>>(n, r32_.p, V, h2);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = 1.0;  // inner system solved for r / ||r||
    int j = 0;
    for (; j < m && its < cfg.max_iterations; ++j) {
      float* vj = V + size_t(j) * n;
      precond_apply_t<float, float>(pc, n, A_.row_ptr, A_.col_idx, vals32_.p,
                                    rdiag32_.p, vj, z32_.p, s);
      spmv_launch<float, float, float>(A_.lanes, n, A_.row_ptr, A_.col_idx,
                                       vals32_.p, z32_.p, nullptr, w32_.p, s);
      mdot_k<float><<<red_blocks_, kBlock, 0, s>>>(n, j + 1, V, n, w32_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, hs, 0, nullptr);
      maxpy_k<float><<<grid1(n), kBlock, 0, s>>>(n, j + 1, V, n, hs, w32_.p);
      mdot_k<float><<<red_blocks_, kBlock, 0, s>>>(n, j + 1, V, n, w32_.p, partial_.p);
      reduce_partials_k<<<j + 1, kBlock, 0, s>>>(red_blocks_, partial_.p, h2 + 1, 1, hs);
      maxpy_k<float><<<grid1(n), kBlock, 0, s>>>(n, j + 1, V, n, h2 + 1, w32_.p);
      mdot_k<float><<<red_blocks_, kBlock, 0, s>>>(n, 1, w32_.p, 0, w32_.p, partial_.p);
      reduce_partials_k<<<1, kBlock, 0, s>>>(red_blocks_, partial_.p, h2, 0, nullptr);
      sqrt_scalar_k<<<1, 1, 0, s>>>(h2);
      scale_by_norm_k<float><<<grid1(n), kBlock, 0, s>>>(n, w32_.p, V + size_t(j + 1) * n, h2);
      NW_CUDA(cudaGetLastError());
      NW_CUDA(cudaMemcpyAsync(h_pinned_, hs, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaMemcpyAsync(h_pinned_ + (j + 1), h2, sizeof(double), cudaMemcpyDeviceToHost, s));
      NW_CUDA(cudaStreamSynchronize(s));
      const double hn = h_pinned_[j + 1];
      for (int k = 0; k <= j; ++k) H[size_t(k) * m + j] = h_pinned_[k];
      H[size_t(j + 1) * m + j] = hn;
      for (int k = 0; k < j; ++k) {
        const double a = H[size_t(k) * m + j], bb = H[size_t(k + 1) * m + j];
        H[size_t(k) * m + j] = cs[k] * a + sn[k] * bb;
        H[size_t(k + 1) * m + j] = -sn[k] * a + cs[k] * bb;
      }
      const double a = H[size_t(j) * m + j], bb = H[size_t(j + 1) * m + j];
      const double den = std::sqrt(a * a + bb * bb);
      if (!(den > 0.0) || !std::isfinite(den)) {
        res.status = std::isfinite(den) ? NW_BREAKDOWN : NW_NAN_DETECTED;
        break;
      }
      cs[j] = a / den;
      sn[j] = bb / den;
      H[size_t(j) * m + j] = den;
      H[size_t(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      ++its;
      const double inner_rel = std::abs(g[j + 1]);
      res.history.push_back(inner_rel * rnorm / bnorm);
      if (inner_rel <= itol || hn == 0.0) {
        ++j;
        break;
      }
    }
    const int kk = j;
    for (int i = kk - 1; i >= 0; --i) {
      double sum = g[i];
      for (int l = i + 1; l < kk; ++l) sum -= H[size_t(i) * m + l] * y[l];
      y[i] = sum / H[size_t(i) * m + i] * 1.0;
    }
    if (kk > 0) {
      for (int i = 0; i < kk; ++i) y[i] *= rnorm;
      NW_CUDA(cudaMemcpyAsync(h2, y.data(), sizeof(double) * kk, cudaMemcpyHostToDevice, s));
      combine_k<float><<<grid1(n), kBlock, 0, s>>>(n, kk, V, n, h2, w32_.p);
      precond_apply_t<float, float>(pc, n, A_.row_ptr, A_.col_idx, vals32_.p,
                                    rdiag32_.p, w32_.p, z32_.p, s);
      add_f32_k<<<grid1(n), kBlock, 0, s>>>(n, z32_.p, x);
    }
    // outer FP64 true residual
    spmv_launch<double, double, double>(A_.lanes, n, A_.row_ptr, A_.col_idx,
                                        A_.values, x, b, r_.p, s);
    rnorm = std::sqrt(dot(r_.p, r_.p, s));
    rel = rnorm / bnorm;
    if (!std::isfinite(rel)) {
      res.status = NW_NAN_DETECTED;
      break;
    }
    res.history.back() = rel;
    if (rel <= tol || res.status != NW_OK) break;
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
