// Krylov solver on the GPU: SpMV, deterministic reductions, Jacobi and
// multicolour Gauss-Seidel relaxation, GMRES / FGMRES / CG, and the
// mixed-precision iterative-refinement driver (krylov.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <vector>

#include "nw_internal.h"

namespace nw {

struct LearnedNet;
struct CoarseLevel;

// A CSR matrix resident on the device (FP64 values; optional FP32 copy).
struct DevCsr {
  int64_t n = 0;
  int64_t nnz = 0;
  const int64_t* row_ptr = nullptr;
  const int32_t* col_idx = nullptr;
  const double* values = nullptr;
  int lanes = 8;  // sub-warp width per row for the CSR kernels
  // host copies of the graph (setup only: builds the sliced-ELL layout)
  const int64_t* row_ptr_host = nullptr;
  const int32_t* col_idx_host = nullptr;
};

// Preconditioner applied inside the solver (right preconditioning).
struct Precond {
  int kind = NW_PC_JACOBI;
  int inner_sweeps = 1;  // NW_PC_SGS2: Jacobi-Richardson corrections per triangular solve
  // multicolour SGS: rows grouped by colour
  const int32_t* color_rows = nullptr;   // nrows, rows of colour 0, 1, ...
  std::vector<int64_t> color_ptr;        // host, ncolors + 1
  // user-supplied preconditioner (learned): y = M(x), FP64 device vectors
  std::function<void(const double*, double*, cudaStream_t)> apply_fn;
};

struct SolveResult {
  int fallback = 0;  // learned preconditioner replaced by SGS after failing
  int iterations = 0;
  int outer = 0;
  int converged = 0;
  nw_status status = NW_OK;
  double final_rel = 0.0;
  double final_abs = 0.0;
  double bnorm = 0.0;
  std::vector<double> history;
};

class KrylovSolver {
 public:
  KrylovSolver() = default;
  ~KrylovSolver();
  KrylovSolver(const KrylovSolver&) = delete;
  KrylovSolver& operator=(const KrylovSolver&) = delete;

  // Bind to a matrix; allocates work space for restart length m.
  void setup(const DevCsr& A, int m, cudaStream_t s);
  // Colour classes of the multicolour Gauss-Seidel sweep (rows of class 0,
  // then class 1, ...; cptr on the host): builds the class-ordered sliced
  // copy of the off-diagonal entries the sweep reads.
  void setup_colors(const std::vector<int32_t>& rows, const std::vector<int64_t>& cptr,
                    cudaStream_t s);
  // Recompute diagonal-dependent data after the values changed.
  void refresh(cudaStream_t s);

  SolveResult solve(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                    const double* b, double* x, cudaStream_t s);

  // Building blocks (device vectors of length n).
  void spmv(const double* x, double* y, cudaStream_t s) const;
  void spmv64(const double* x, const double* b, double* y, cudaStream_t s) const;
  void spmv32(const float* x, float* y, cudaStream_t s) const;
  void apply_precond(const Precond& pc, const double* x, double* y,
                     cudaStream_t s);
  double dot(const double* a, const double* b, cudaStream_t s);
  // Learned two-level preconditioner (NW_PC_LEARNED); the coarse level is
  // refreshed from the matrix values on every refresh().
  void attach_learned(LearnedNet* net, CoarseLevel* cl) {
    net_ = net;
    cl_ = cl;
  }
  bool has_learned() const { return net_ && cl_; }
  void ensure_f32(cudaStream_t s);
  // FP32 preconditioner application (Jacobi, SGS or learned) of the mixed
  // method; y and x must not alias.
  void precond32(const Precond& pc, const float* x, float* y, cudaStream_t s);
  // the learned cycle's pre-smoothing sweep alone (pair harvesting)
  void learned_presmooth32(const float* x, float* y, cudaStream_t s);
  const float* vals32() const { return vals32_.p; }

 private:
  SolveResult gmres(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                    const double* b, double* x, bool flexible,
                    cudaStream_t s);
  SolveResult cg(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                 const double* b, double* x, cudaStream_t s);
  SolveResult mixed(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                    const double* b, double* x, cudaStream_t s);
  SolveResult bicgstab(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                       const double* b, double* x, cudaStream_t s);
  SolveResult tfqmr(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                    const double* b, double* x, cudaStream_t s);
  SolveResult sstep_gmres(const nw_solver_cfg& cfg, double tol, const Precond& pc,
                          const double* b, double* x, cudaStream_t s);
  DeviceArray<double> sst_;     // s-step GMRES block coefficients
  DeviceArray<double> aux_;     // work vectors of BiCGStab / TFQMR
  LearnedNet* net_ = nullptr;
  CoarseLevel* cl_ = nullptr;
  DeviceArray<float> Z32_, rc32_, ec32_, tmp32_, tmp32b_;

  DevCsr A_;
  int m_ = 0;
  DeviceArray<double> rdiag_;   // 1 / a_ii
  DeviceArray<double> V_;       // (m+1) x n basis
  DeviceArray<double> Z_;       // m x n (flexible)
  DeviceArray<double> w_, z_, r_;
  DeviceArray<double> partial_; // deterministic reduction partials
  DeviceArray<double> scal_;    // small device scalars
  double* h_pinned_ = nullptr;  // host mirror of scal_
  // GMRES least squares on the device (Givens rotations of the Hessenberg
  // columns, the rotated rhs g, the per-iteration residual estimates, the
  // back substitution): H (m+1) x m | cs m | sn m | g m+1 | hist m, and the
  // control words done, iterations of the cycle, status, basis size.
  DeviceArray<double> gst_;
  DeviceArray<int> gctl_;
  int* ctl_pinned_ = nullptr;   // host mirrors of gctl_ (3 slots)
  cudaEvent_t chunk_ev_[2] = {nullptr, nullptr};
  struct Cycle {
    int iterations = 0;  // rotations applied (iterations counted)
    int basis = 0;       // vectors in the update
    bool done = false;   // converged, broke down or non-finite
    nw_status status = NW_OK;
    std::vector<double> hist;
  };
  // One restart cycle's Arnoldi steps (arnoldi(j) launches iteration j's
  // kernels, ending with the new column in hs[0..j] and its norm at h2[0])
  // with the Givens update on the device and the host one chunk behind.
  // With `graph`, the steps after the first of the cycle are captured from
  // the same launches into a CUDA graph each, which updates iter_exec_ in
  // place and is launched as one unit (the kernels then follow each other
  // without the per-launch gaps of a stream).
  template <typename StepFn>
  Cycle run_cycle(int m, int max_steps, double g0, double tol, double div, double hist_mul, double hist_div,
                  StepFn arnoldi, const double* hs, const double* hn, cudaStream_t s, bool graph = false);
  cudaGraphExec_t iter_exec_ = nullptr;
  // Sliced ELLPACK copy (slices of 32 rows, column-major within a slice)
  // used by the solver's SpMV: coalesced value/column loads for short rows.
  // sell_map_ holds the CSR index of every slot (-1 for padding).
  DeviceArray<int64_t> sell_off_;
  DeviceArray<int32_t> sell_cols_, sell_map_;
  DeviceArray<double> sell_vals_;
  DeviceArray<float> sell_vals32_;
  int64_t sell_slices_ = 0;
  // Gauss-Seidel copy: per colour class, slices of 32 class rows holding
  // their off-diagonal entries column-major; slice offsets, row lengths,
  // columns, CSR positions (for the value gathers) and values.
  std::vector<int64_t> gs_cptr_, gs_slice0_;  // host: class row / slice starts
  DeviceArray<int32_t> gs_rows_, gs_len_, gs_cols_, gs_map_;
  DeviceArray<int64_t> gs_off_;
  DeviceArray<double> gs_vals_;
  DeviceArray<float> gs_vals32_;
  DeviceArray<__nv_bfloat16> gs_vals16_;  // BF16 copy (NW_PREC_MIXED_BF16)
  bool gs_bf16_ = false;
  template <typename VT, typename T>
  void sgs(const VT* vals, const T* rd, const T* x, T* y, cudaStream_t s,
           bool from_guess = false, int sweep = 0) const;
  // two-stage symmetric Gauss-Seidel (CSR, row order), scratch 3 n
  template <typename VT, typename T>
  void sgs2(const VT* vals, const T* rd, const T* x, T* y, int inner, T* scratch,
            cudaStream_t s) const;
  DeviceArray<double> sgs2_64_;
  DeviceArray<float> sgs2_32_;
  // Level schedules of the natural row order (NW_PC_SGS_NATURAL,
  // NW_PC_RILUK): forward level of row i = 1 + the largest level of the
  // rows j < i in its pattern, backward the same over j > i; rows of one
  // level are independent. Built on first use from the host graph.
  void setup_levels(cudaStream_t s);
  bool levels_ready_ = false;
  std::vector<int64_t> fl_ptr_, bl_ptr_;
  DeviceArray<int32_t> fl_rows_, bl_rows_;
  DeviceArray<int64_t> dpos_;   // CSR position of each row's diagonal
  template <typename VT, typename T>
  void sgs_natural(const VT* vals, const T* x, T* y, cudaStream_t s);
  // ILU(0) factors on the matrix pattern (L unit lower, U upper), FP64 and
  // an FP32 copy for the mixed method; refactored after refresh()
  void ilu0_factor(cudaStream_t s);
  bool ilu_valid_ = false;
  DeviceArray<double> lu_;
  DeviceArray<float> lu32_;
  template <typename T>
  void ilu0_solve(const T* lu, const T* x, T* y, cudaStream_t s);
  void sgs_residual32(const float* x, const float* y, float* r, cudaStream_t s, int last) const;
  DeviceArray<float> diag32_;   // FP32 diagonal
  // FP32 copies for the inner solve of the mixed method
  DeviceArray<float> vals32_, rdiag32_, V32_, w32_, z32_, r32_;
  int64_t ld32_ = 0;  // leading dimension of the FP32 basis (n rounded up to 32)
  bool f32_valid_ = false;
  int red_blocks_ = 0;
  int mdot4_blocks_ = 0;  // grid of the FP32 multi-dot (one resident wave)
};

}  // namespace nw
