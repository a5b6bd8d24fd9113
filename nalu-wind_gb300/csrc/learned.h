// Learned two-level preconditioner (learned.cu).
//
// M(v) = z2 + S(v - A z2),  z2 = z1 + alpha P Net(R (v - A z1)),
// z1 = S(v), S = one multicolour symmetric Gauss-Seidel sweep (FP32),
// R / P = restriction (sum) / prolongation (copy) over aggregates of the
// matrix graph (plain aggregation, applied twice by default: aggregates of
// aggregates), and Net = a 4-layer edge message-passing network with
// 64 channels acting as the coarse solver on the aggregate graph. The coarse
// operator Ac = R A P (Galerkin, summed in a fixed order) supplies the edge
// weights w_IJ = -Ac_IJ / Ac_II and the Jacobi scaling 1 / Ac_II.
//
// Network (BF16 weights and activations, FP32 accumulation):
//   u = D^-1 r_c, s = rms(u), x = u / s
//   H0 = relu([x, W x] W0)                 W0: 2 x 64
//   Hl = relu([H(l-1), W H(l-1)] Wl)       Wl: 128 x 64, l = 1..3
//   e_c = s * (H3 wout)                    wout: 64
// and the preconditioner adds alpha P e_c (alpha below).
// where (W h)_I = sum_J w_IJ h_J. Trained on the GPU (forward, backward
// and Adam kernels in learned.cu; the dense layers use mma.sync BF16 tensor
// core instructions) over (residual, error) pairs harvested at the restarts
// of plain Jacobi-GMRES, minimising the energy norm of the error left after
// the smoothing and the coarse correction,
// with the coarse correction scaled by its energy-optimal factor
//   alpha = e_c' r_c / e_c' Ac e_c:
//   L = min_alpha ||z1 + alpha P e_c - e||_A^2 / ||e||_A^2
//     = (cA - (e_c' r_c)^2 / e_c' Ac e_c) / eA,
// with r_c = R (r - A z1) = P' A (e - z1), cA = ||e - z1||_A^2 and
// eA = ||e||_A^2 = e' r. Its minimisers are the multiples of the exact
// Galerkin coarse solve Ac^-1 r_c, so the network learns the direction
// of that solve. The same alpha is applied at every use, so the coarse
// correction never increases the A-norm error of the smoothed iterate
// (whatever the network outputs). The form assumes a symmetric operator
// (the pressure Poisson system is).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "nw_internal.h"

namespace nw {

constexpr int kHid = 64;
constexpr int kIn2 = 2 * kHid;  // concatenated [h, W h]
// flat parameter layout: W0 (2 x 64) | W1 | W2 | W3 (128 x 64 each) | wout
constexpr int kOffW0 = 0;
constexpr int kOffW1 = kOffW0 + 2 * kHid;
constexpr int kOffW2 = kOffW1 + kIn2 * kHid;
constexpr int kOffW3 = kOffW2 + kIn2 * kHid;
constexpr int kOffWout = kOffW3 + kIn2 * kHid;
constexpr int kNumParams = kOffWout + kHid;

// Aggregation and Galerkin structures for one fine graph (1 dof).
struct CoarseLevel {
  int64_t nf = 0, nc = 0, nnzc = 0;
  int passes = 1;                          // aggregation passes
  double strength = 0.0;                   // strong-connection threshold (0: plain)
  std::vector<int32_t> agg_h;              // fine row -> aggregate
  std::vector<int64_t> cptr_h;             // coarse CSR
  std::vector<int32_t> ccol_h, cdiag_h, rev_h;
  DeviceArray<int32_t> agg, mrows, ccol, cdiag, rev, gfine;
  DeviceArray<int64_t> mptr, cptr, gptr;
  DeviceArray<double> ac;                  // Galerkin values
  DeviceArray<float> wgt, dinv;            // edge weights, 1 / Ac_II
  // values (host, aligned with the node graph) and theta > 0: aggregation
  // over strong connections; otherwise plain aggregation of the graph
  void setup(const HostGraph& g, int passes, cudaStream_t s, const double* values = nullptr,
             double theta = 0.0);
  void refresh(const double* fine_values, cudaStream_t s);
};

// Activations of one forward pass on a coarse graph (sized to nc).
struct NetWork {
  int64_t nc = 0;
  DeviceArray<float> u, x, ax, y, dy, ec, aec, scal, partial, part2;
  DeviceArray<uint16_t> xc1, xc2, xc3, h3, dz;  // BF16
  DeviceArray<float> dxc, dh;
  void resize(int64_t n);
};

struct LearnedNet {
  std::vector<float> params_h;           // host master copy (save/load)
  DeviceArray<float> params, grads, adam_m, adam_v;
  DeviceArray<uint16_t> wbf, wtbf;       // BF16 W1..W3 (row-major) and transposes
  DeviceArray<float> wpartial;           // weight-gradient partials
  int64_t adam_step = 0;
  uint64_t seed = 0;
  int post_smooth = 1;  // SGS sweep after the coarse correction
  int agg_passes = 2;   // aggregation passes of the coarse level
  double agg_strength = 0.0;  // strong-connection threshold of the aggregation (0: plain)
  int smoother = 0;     // 0: symmetric GS sweeps around the coarse step; 1: forward / backward
  // coarse direction: 0 the network; 1 D_c^-1 r_c and 2 two Jacobi sweeps on
  // Ac (the same cycle and alpha rule without the network, as controls)
  int coarse_mode = 0;
  // training data (coarse vectors of one aggregation)
  int64_t data_nc = 0, data_nnzc = 0;
  int npairs = 0, nsystems = 0;
  std::vector<int> pair_system;
  std::vector<double> pair_ea, pair_ca;   // ||e||_A^2, ||e - z1||_A^2
  std::vector<DeviceArray<float>*> sys_wgt, sys_dinv, pair_rc;
  NetWork work;
  ~LearnedNet();
  void init(uint64_t seed, cudaStream_t s);
  void sync_bf16(cudaStream_t s);  // BF16 copies from the FP32 masters
  void upload(cudaStream_t s);
  void download(cudaStream_t s);
  void clear_data();
  // forward: coarse residual -> coarse correction (FP32, device)
  void forward(const CoarseLevel& cl, const float* wgt, const float* dinv,
               const float* rc, float* ec, cudaStream_t s);
  // network output ec plus its scaling alpha (device, alpha_dev()); ec
  // must not alias the work buffers
  void coarse_correction(const CoarseLevel& cl, const float* rc, float* ec, cudaStream_t s);
  const float* alpha_dev() const { return work.scal.p + 2; }
  // loss and parameter gradients (accumulated into grads) for one pair;
  // returns the loss (host sync). with_grad = false: loss only.
  double forward_backward(const CoarseLevel& cl, const float* wgt,
                          const float* dinv, const float* rc, double ea,
                          double ca, cudaStream_t s, bool with_grad = true);
  void adam(double lr, double scale, cudaStream_t s);
};

// Weight file with a header and an FNV-1a checksum.
void save_params(const std::string& path, const std::vector<float>& p, uint64_t step);
void load_params(const std::string& path, std::vector<float>& p);

// Kernel launchers used by the tests through the C ABI.
// The same forward GEMM on the tcgen05 tensor cores (tc_gemm.cu); tc_status
// reads and clears its timeout flag (non-zero: a wait gave up).
void launch_gemm_fwd_tc(const uint16_t* a, const uint16_t* wt, uint16_t* out, int64_t m,
                        int ldo, cudaStream_t s);
int tc_status(cudaStream_t s);
// The same GEMM with the tiles loaded by TMA (cp.async.bulk.tensor,
// 128-byte swizzle).
void launch_gemm_fwd_tma(const uint16_t* a, const uint16_t* wt, uint16_t* out, int64_t m,
                         int ldo, cudaStream_t s);
void launch_gemm_fwd(const uint16_t* a, const uint16_t* wt, uint16_t* out,
                     int64_t m, int ldo, cudaStream_t s);
void launch_gemm_dx(const uint16_t* dz, const uint16_t* w, float* dx, int64_t m,
                    cudaStream_t s);
void launch_gemm_wgrad(const uint16_t* xc, const uint16_t* dz, float* partial,
                       float* dw, int64_t m, cudaStream_t s);
// The backward GEMMs on the tcgen05 tensor cores (tc_gemm.cu): dX = dZ W^T
// with TMA-loaded tiles, and the dW partials (one 128 x 64 block per CTA,
// `blocks` CTAs over 64-node chunks); launch_gemm_wgrad_tc adds the fixed-
// order column sum into dw. Timeouts go to tc_status.
void launch_gemm_dx_tma(const uint16_t* dz, const uint16_t* w, float* dx, int64_t m,
                        cudaStream_t s);
void launch_wgrad_partials_tc(const uint16_t* xc, const uint16_t* dz, float* partial, int64_t m,
                              int blocks, cudaStream_t s);
void launch_gemm_wgrad_tc(const uint16_t* xc, const uint16_t* dz, float* partial,
                          float* dw, int64_t m, cudaStream_t s);

// Two-level application helpers (FP32).
void launch_restrict(const CoarseLevel& cl, const float* r, float* rc, cudaStream_t s);
void launch_prolong_add(const CoarseLevel& cl, const float* ec, const float* alpha, float* z,
                        cudaStream_t s);

}  // namespace nw
