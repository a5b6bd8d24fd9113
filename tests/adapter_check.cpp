// Exercises include/nw_linear_system.hpp (the reference's LinearSystem /
// LinearSolverConfig surface over the C ABI) from C++, as a nalu-wind
// build would: backend factory, string options, graph, sumInto, resetRows,
// solve. Mode "host" runs what needs no GPU; mode "device" assembles a
// 1-D Laplacian chain by sumInto blocks, fixes node 0, solves with each
// preconditioner string and checks the solution against a dense solve.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "nw_linear_system.hpp"

static int fails = 0;
#define EXPECT(c)                                                  \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAILED %s:%d %s\n", __FILE__, __LINE__, #c);    \
      ++fails;                                                     \
    }                                                              \
  } while (0)

template <typename E, typename F>
bool throws(F&& f) {
  try {
    f();
  } catch (const E&) {
    return true;
  }
  return false;
}

int main(int argc, char** argv) {
  const bool device = argc > 1 && std::strcmp(argv[1], "device") == 0;
  nw::LinearSolverConfig cfg;
  cfg.method = "gmres";
  cfg.preconditioner = "sgs";
  cfg.tolerance = 1e-12;
  cfg.max_iterations = 200;
  cfg.kspace = 50;
  EXPECT(cfg.to_c().preconditioner == NW_PC_SGS_NATURAL);
  EXPECT(throws<std::logic_error>([&] { nw::LinearSystem::create(nw::PT_TPETRA, 1, cfg); }));
  EXPECT(throws<std::logic_error>([&] { nw::LinearSystem::create(nw::PT_HYPRE_SEGREGATED, 3, cfg); }));
  nw::LinearSolverConfig bad = cfg;
  bad.preconditioner = "ilut";
  EXPECT(throws<std::runtime_error>([&] { bad.to_c(); }));
  const int64_t N = 24;
  std::vector<int64_t> edges;
  for (int64_t i = 0; i + 1 < N; ++i) {
    edges.push_back(i);
    edges.push_back(i + 1);
  }
  if (!device) {
    auto ls = nw::LinearSystem::create(nw::PT_GB300, 1, cfg);
    EXPECT(ls->numDof() == 1);
    ls->buildEdgeToNodeGraph(N, edges);
    int64_t nrows = 0, nnz = 0;
    nw_linsys_graph_sizes(ls->handle(), &nrows, &nnz);
    EXPECT(nrows == N && nnz == N + 2 * (N - 1));
    std::printf("%s\n", fails ? "host checks failed" : "host checks passed");
    return fails ? 1 : 0;
  }
  for (const char* pc : {"jacobi", "sgs", "mt_sgs", "sgs2", "riluk"}) {
    cfg.preconditioner = pc;
    auto ls = nw::LinearSystem::create(nw::PT_GB300, 1, cfg);
    ls->buildEdgeToNodeGraph(N, edges);
    ls->buildNodeGraph();
    ls->buildDirichletNodeGraph();
    ls->finalizeLinearSystem();
    ls->zeroSystem();
    // -u'' = 1 on a chain of unit edges, u(0) = 0
    std::vector<double> A(size_t(N) * N, 0.0), b(N, 0.0);
    for (int64_t i = 0; i + 1 < N; ++i) {
      const double k = 1.0 + 0.1 * double(i % 3);
      ls->sumInto({i, i + 1}, {0.5, 0.5}, {k, -k, -k, k});
      A[i * N + i] += k;
      A[i * N + i + 1] -= k;
      A[(i + 1) * N + i] -= k;
      A[(i + 1) * N + i + 1] += k;
      b[i] += 0.5;
      b[i + 1] += 0.5;
    }
    int64_t* nodes = nullptr;
    cudaMalloc(&nodes, sizeof(int64_t));
    const int64_t zero = 0;
    cudaMemcpy(nodes, &zero, sizeof(int64_t), cudaMemcpyHostToDevice);
    ls->resetRows(nodes, 1, 0, 1, 1.0, 0.0);
    for (int64_t j = 0; j < N; ++j) A[j] = 0.0;
    A[0] = 1.0;
    b[0] = 0.0;
    ls->loadComplete();
    double* x = nullptr;
    cudaMalloc(&x, sizeof(double) * N);
    const int st = ls->solve(x, false);
    std::vector<double> xh(N);
    cudaMemcpy(xh.data(), x, sizeof(double) * N, cudaMemcpyDeviceToHost);
    cudaFree(x);
    cudaFree(nodes);
    // dense Gaussian elimination
    for (int64_t k = 0; k < N; ++k)
      for (int64_t i = k + 1; i < N; ++i) {
        const double f = A[i * N + k] / A[k * N + k];
        if (f == 0.0) continue;
        for (int64_t j = k; j < N; ++j) A[i * N + j] -= f * A[k * N + j];
        b[i] -= f * b[k];
      }
    std::vector<double> u(N);
    for (int64_t i = N - 1; i >= 0; --i) {
      double s = b[i];
      for (int64_t j = i + 1; j < N; ++j) s -= A[i * N + j] * u[j];
      u[i] = s / A[i * N + i];
    }
    double err = 0.0, mx = 0.0;
    for (int64_t i = 0; i < N; ++i) {
      err = std::fmax(err, std::fabs(xh[i] - u[i]));
      mx = std::fmax(mx, std::fabs(u[i]));
    }
    std::printf("%-7s status %d iterations %d residual %.3e error %.3e\n", pc, st, ls->linearSolveIterations(),
                ls->linearResidual(), err / mx);
    EXPECT(st == NW_OK);
    EXPECT(ls->linearSolveIterations() > 0);
    EXPECT(err <= 1e-9 * mx);
  }
  std::printf("%s\n", fails ? "device checks failed" : "device checks passed");
  return fails ? 1 : 0;
}
