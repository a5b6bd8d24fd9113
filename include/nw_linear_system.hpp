/*
 * nw_linear_system.hpp - the reference's LinearSystem / LinearSolverConfig
 * surface in C++ over the C ABI (header only; link libnw_gb300.so).
 *
 * nalu-wind's equation systems talk to their linear system through
 * sierra::nalu::LinearSystem (include/LinearSystem.h:70-260), created by the
 * backend factory LinearSystem::create (src/LinearSystem.C:117-159) from the
 * solver's PetraType (include/LinearSolver.h:54-60), and configured by
 * TpetraLinearSolverConfig::load (src/LinearSolverConfig.C:37-140). This
 * header restates that surface without STK or Trilinos types: nodes are
 * indices into the caller's node arrays, fields are device pointers, and
 * the solver options are the reference's strings. A nalu-wind build adds a
 * thin sierra::nalu::LinearSystem subclass that forwards each virtual to
 * the member of the same name here, translating stk::mesh::Entity to node
 * indices (the integration notes show it). Errors of the C ABI become
 * std::runtime_error, as the reference throws (src/TpetraLinearSystem.C:
 * 1900-1913).
 */
#ifndef NW_LINEAR_SYSTEM_HPP
#define NW_LINEAR_SYSTEM_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nw_capi.h"

namespace nw {

/* include/LinearSolver.h:54-60 plus this library's backend. */
enum PetraType {
  PT_TPETRA,
  PT_TPETRA_SEGREGATED,
  PT_HYPRE,
  PT_HYPRE_SEGREGATED,
  PT_GB300,  /* this library: one GPU, the C ABI of nw_capi.h */
  PT_END
};

inline void check_status(nw_status s, const char* what) {
  if (s != NW_OK)
    throw std::runtime_error(std::string(what) + ": " + nw_last_error_string());
}

/* TpetraLinearSolverConfig (src/LinearSolverConfig.C:37-140): the YAML
 * keys with the reference's defaults. */
struct LinearSolverConfig {
  std::string method = "gmres";
  std::string preconditioner = "default";
  double tolerance = 1.e-4;
  double final_tolerance = -1.0;  // < 0: equal to tolerance
  int max_iterations = 50;
  int kspace = 50;
  int inner_iterations = 1;  // "inner_iterations" of sgs2
  int krylov_step_size = 5;  // "krylov_step_size" of sstep_gmres

  nw_solver_cfg to_c() const {
    nw_solver_cfg c{};
    c.precision = NW_PREC_FP64;
    c.kspace = kspace;
    c.max_iterations = max_iterations;
    c.tolerance = tolerance;
    c.final_tolerance = final_tolerance < 0.0 ? tolerance : final_tolerance;
    c.sgs2_inner_sweeps = inner_iterations;
    c.sstep_size = krylov_step_size;
    check_status(nw_solver_cfg_from_strings(method.c_str(), preconditioner.c_str(), &c), "solver options");
    return c;
  }
};

/* sierra::nalu::LinearSystem, restated (the members an edge-assembled
 * equation system calls). */
class LinearSystem {
 public:
  virtual ~LinearSystem() = default;

  /* LinearSystem::create (src/LinearSystem.C:117-159): the backend of the
   * solver's type. This library provides PT_GB300; the Trilinos and hypre
   * backends belong to the reference build and are refused here, as the
   * reference refuses a type it was built without ("create lin sys"). */
  static std::unique_ptr<LinearSystem> create(PetraType type, unsigned numDof,
                                              const LinearSolverConfig& config);

  unsigned numDof() const { return numDof_; }
  const int& linearSolveIterations() const { return linearSolveIterations_; }
  const double& linearResidual() const { return linearResidual_; }
  const double& nonLinearResidual() const { return nonLinearResidual_; }

  /* graph: the node and Dirichlet graphs add no entries the edge graph
   * lacks (a node's own column is always present; the Tpetra Dirichlet
   * graph is a no-op, include/LinearSystem.h:137-147) */
  virtual void buildEdgeToNodeGraph(int64_t numNodes, const std::vector<int64_t>& edgeNodes,
                                    const std::vector<int64_t>& globalIds = {},
                                    const std::vector<int64_t>& naluIds = {}) = 0;
  virtual void buildNodeGraph() {}
  virtual void buildDirichletNodeGraph() {}
  virtual void finalizeLinearSystem() = 0;

  virtual void zeroSystem() = 0;
  /* host-vector sumInto (include/LinearSystem.h:167-173): nodes, rhs
   * (n numDof) and row-major lhs ((n numDof)^2) */
  virtual void sumInto(const std::vector<int64_t>& nodes, const std::vector<double>& rhs,
                       const std::vector<double>& lhs) = 0;
  /* applyDirichletBCs over device node lists and fields */
  virtual void applyDirichletBCs(const int64_t* nodesDev, int64_t n, const double* solutionDev,
                                 const double* bcValuesDev, unsigned beginPos, unsigned endPos) = 0;
  virtual void resetRows(const int64_t* nodesDev, int64_t n, unsigned beginPos, unsigned endPos,
                         double diag_value = 0.0, double rhs_residual = 0.0) = 0;
  virtual void loadComplete() = 0;
  /* solve into the device correction vector (nrows); returns the status */
  virtual int solve(double* deltaDev, bool finalIteration = false) = 0;
  virtual void writeToFile(const char* filename, int count = 0) = 0;

  /* the C handle, for the edge-assembly entry points of nw_capi.h */
  virtual nw_linsys* handle() = 0;

 protected:
  explicit LinearSystem(unsigned numDof) : numDof_(numDof) {}
  unsigned numDof_;
  int linearSolveIterations_ = 0;
  double linearResidual_ = 0.0;
  double nonLinearResidual_ = 0.0;
};

/* The GB300 backend. */
class Gb300LinearSystem final : public LinearSystem {
 public:
  Gb300LinearSystem(unsigned numDof, const LinearSolverConfig& config) : LinearSystem(numDof) {
    const nw_solver_cfg c = config.to_c();
    check_status(nw_linsys_create(int(numDof), &c, &ls_), "nw_linsys_create");
  }
  ~Gb300LinearSystem() override {
    if (ls_) nw_linsys_destroy(ls_);
  }
  Gb300LinearSystem(const Gb300LinearSystem&) = delete;
  Gb300LinearSystem& operator=(const Gb300LinearSystem&) = delete;

  void buildEdgeToNodeGraph(int64_t numNodes, const std::vector<int64_t>& edgeNodes,
                            const std::vector<int64_t>& globalIds,
                            const std::vector<int64_t>& naluIds) override {
    check_status(nw_linsys_build_edge_graph(ls_, numNodes, globalIds.empty() ? nullptr : globalIds.data(),
                                            naluIds.empty() ? nullptr : naluIds.data(),
                                            int64_t(edgeNodes.size() / 2), edgeNodes.data()),
                 "buildEdgeToNodeGraph");
  }
  void finalizeLinearSystem() override { check_status(nw_linsys_finalize(ls_), "finalizeLinearSystem"); }
  void zeroSystem() override { check_status(nw_linsys_zero(ls_), "zeroSystem"); }
  void sumInto(const std::vector<int64_t>& nodes, const std::vector<double>& rhs,
               const std::vector<double>& lhs) override {
    const size_t m = nodes.size() * numDof_;
    if (rhs.size() != m || lhs.size() != m * m) throw std::runtime_error("sumInto: block sizes");
    check_status(nw_linsys_sum_into(ls_, int(nodes.size()), nodes.data(), rhs.data(), lhs.data()), "sumInto");
  }
  void applyDirichletBCs(const int64_t* nodesDev, int64_t n, const double* solutionDev,
                         const double* bcValuesDev, unsigned beginPos, unsigned endPos) override {
    check_status(nw_linsys_apply_dirichlet(ls_, n, nodesDev, int(beginPos), int(endPos), solutionDev,
                                           bcValuesDev),
                 "applyDirichletBCs");
  }
  void resetRows(const int64_t* nodesDev, int64_t n, unsigned beginPos, unsigned endPos, double diag_value,
                 double rhs_residual) override {
    check_status(nw_linsys_reset_rows(ls_, n, nodesDev, int(beginPos), int(endPos), diag_value, rhs_residual),
                 "resetRows");
  }
  void loadComplete() override { check_status(nw_linsys_load_complete(ls_), "loadComplete"); }
  int solve(double* deltaDev, bool finalIteration) override {
    nw_solve_report r{};
    const nw_status s = nw_linsys_solve(ls_, deltaDev, finalIteration ? 1 : 0, &r);
    if (s != NW_OK && s != NW_NOT_CONVERGED) check_status(s, "solve");
    linearSolveIterations_ = r.iterations;
    linearResidual_ = r.final_abs_residual;
    nonLinearResidual_ = r.rhs_norm;
    return r.status;
  }
  void writeToFile(const char* filename, int count) override {
    check_status(nw_linsys_write_matrix_market(ls_, filename, count, nullptr), "writeToFile");
  }
  nw_linsys* handle() override { return ls_; }

 private:
  nw_linsys* ls_ = nullptr;
};

inline std::unique_ptr<LinearSystem> LinearSystem::create(PetraType type, unsigned numDof,
                                                          const LinearSolverConfig& config) {
  switch (type) {
    case PT_GB300:
      return std::unique_ptr<LinearSystem>(new Gb300LinearSystem(numDof, config));
    case PT_TPETRA:
    case PT_TPETRA_SEGREGATED:
    case PT_HYPRE:
    case PT_HYPRE_SEGREGATED:
      throw std::logic_error("create lin sys: backend not built into this library (Trilinos / hypre)");
    default:
      throw std::logic_error("create lin sys");
  }
}

}  // namespace nw

#endif /* NW_LINEAR_SYSTEM_HPP */
