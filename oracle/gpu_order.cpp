/*
 * The FP64 Krylov solvers restated in the GPU library's operation order.
 *
 * TEST INFRASTRUCTURE ONLY (part of liboracle.so, the checker).
 *
 * oracle.cpp's or_solve restates the reference's solvers (Belos GMRES with
 * ICGS, CG, BiCGStab, TFQMR; Ifpack2 relaxations) in the natural serial
 * order. The GPU computes the same algorithms, but its sums run in a fixed
 * two-stage order (per-thread partial sums over a fixed grid, warp and block
 * trees, then a tree over the per-block partials), its sparse rows are
 * summed with fused multiply-adds, and its Gauss-Seidel sweeps visit the rows
 * colour class by colour class. Rounding in a different order changes the
 * iterates at the level of the unit roundoff, and a Krylov method carries
 * such changes forward, so histories in the two orders agree to about
 * 1e-10. This file restates the same solvers in the GPU's order, operation
 * for operation (every fma where the GPU kernels call fma; the same grid of
 * `red_blocks` blocks of 256 threads; the same sliced-ELL padding), so that
 * the parity tests can compare residual histories at 1e-12 and tighter.
 * The algorithms are those or_solve restates (src/LinearSolver.C:209-254,
 * src/LinearSolverConfig.C:37-140); only the order of the arithmetic is the
 * GPU's.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

struct Csr {
  int64_t n;
  const int64_t* rp;
  const int32_t* ci;
  const double* v;
};

// lane 0 of a __shfl_down tree over 32 lanes
double warp_tree(double* a) {
  for (int off = 16; off > 0; off >>= 1)
    for (int l = 0; l < off; ++l) a[l] = a[l] + a[l + off];
  return a[0];
}

// reduce_partials_k: thread t sums partials t, t + 256, ...; then a shared
// memory tree
double reduce_partials(const double* p, int64_t G) {
  double sh[kBlock];
  for (int t = 0; t < kBlock; ++t) {
    double v = 0.0;
    for (int64_t q = t; q < G; q += kBlock) v += p[q];
    sh[t] = v;
  }
  for (int off = kBlock / 2; off > 0; off >>= 1)
    for (int t = 0; t < off; ++t) sh[t] += sh[t + off];
  return sh[0];
}

// warp sums of per-thread values, then thread-serial sum over the block's
// warps (the block stage of mdot_k / maxpy_k)
double block_sum(const double* thread_vals) {
  double red[kWarps];
  for (int w = 0; w < kWarps; ++w) {
    double a[32];
    for (int l = 0; l < 32; ++l) a[l] = thread_vals[32 * w + l] + 0.0;
    red[w] = warp_tree(a);
  }
  double v = 0.0;
  for (int q = 0; q < kWarps; ++q) v += red[q];
  return v;
}

// mdot_k<double> + reduce_partials_k: sum_i a[i] b[i]
double gdot(int64_t n, const double* a, const double* b, int G) {
  std::vector<double> partial(G);
  const int64_t stride = int64_t(G) * kBlock;
#pragma omp parallel for schedule(static)
  for (int blk = 0; blk < G; ++blk) {
    double tv[kBlock];
    for (int t = 0; t < kBlock; ++t) {
      double s = 0.0;
      int64_t i = int64_t(blk) * kBlock + t;
      for (; i + stride < n; i += 2 * stride) {
        s = std::fma(a[i], b[i], s);
        s = std::fma(a[i + stride], b[i + stride], s);
      }
      if (i < n) s = std::fma(a[i], b[i], s);
      tv[t] = s;
    }
    partial[blk] = block_sum(tv);
  }
  return reduce_partials(partial.data(), G);
}

// sliced-ELL SpMV (sell_spmv_k): rows in slices of 32; each row's entries
// in CSR order, then padding slots (value 0, column = the row) up to the
// slice's longest row. y = A x, or y = b - A x.
void gspmv(const Csr& A, const double* x, const double* b, double* y) {
  const int64_t ns = (A.n + 31) / 32;
#pragma omp parallel for schedule(static)
  for (int64_t sl = 0; sl < ns; ++sl) {
    const int64_t r0 = 32 * sl, r1 = std::min(A.n, r0 + 32);
    int64_t len = 0;
    for (int64_t r = r0; r < r1; ++r) len = std::max(len, A.rp[r + 1] - A.rp[r]);
    for (int64_t r = r0; r < r1; ++r) {
      double acc = 0.0;
      for (int64_t k = 0; k < len; ++k) {
        const int64_t p = A.rp[r] + k;
        acc = p < A.rp[r + 1] ? std::fma(A.v[p], x[A.ci[p]], acc) : std::fma(0.0, x[r], acc);
      }
      y[r] = b ? b[r] - acc : acc;
    }
  }
}

// CSR SpMV with LANES threads per row (spmv_k): lane l sums entries
// l, l + LANES, ...; then a shuffle tree over the lanes
void gspmv_lanes(const Csr& A, int lanes, const double* x, const double* b, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < A.n; ++r) {
    double a[32];
    for (int l = 0; l < lanes; ++l) {
      double acc = 0.0;
      for (int64_t p = A.rp[r] + l; p < A.rp[r + 1]; p += lanes) acc = std::fma(A.v[p], x[A.ci[p]], acc);
      a[l] = acc;
    }
    for (int off = lanes / 2; off > 0; off >>= 1)
      for (int l = 0; l < off; ++l) a[l] = a[l] + a[l + off];
    y[r] = b ? b[r] - a[0] : a[0];
  }
}

// ts_tri_k: gout = rd (r - T gin), T the strict lower / upper part
void gtri(const Csr& A, int lanes, bool upper, const double* rd, const double* r, const double* gin,
          double* gout) {
#pragma omp parallel for schedule(static)
  for (int64_t row = 0; row < A.n; ++row) {
    double a[32];
    for (int l = 0; l < lanes; ++l) {
      double acc = 0.0;
      for (int64_t p = A.rp[row] + l; p < A.rp[row + 1]; p += lanes) {
        const int64_t c = A.ci[p];
        if (upper ? c > row : c < row) acc = std::fma(A.v[p], gin[c], acc);
      }
      a[l] = acc;
    }
    for (int off = lanes / 2; off > 0; off >>= 1)
      for (int l = 0; l < off; ++l) a[l] = a[l] + a[l + off];
    gout[row] = rd[row] * (r[row] - a[0]);
  }
}

struct Solver {
  Csr A;
  int G;       // blocks of the reductions
  int lanes;   // CSR sub-warp width
  int precond; // 0 none, 1 Jacobi, 2 multicolour SGS, 4 two-stage SGS
  const int64_t* order;  // colour-class row order
  const int64_t* cptr;   // class boundaries (ncol + 1)
  int ncol;
  int inner;
  std::vector<double> rd;
  std::vector<double> sc;  // scratch for sgs2
  std::vector<double> lu;  // ILU(0) factors (precond 6)
  std::vector<int64_t> dpos;

  double dot(const double* a, const double* b) const { return gdot(A.n, a, b, G); }

  // one colour class of gs_sell_k
  void gs_class(int c, bool first, const double* x, double* y) const {
#pragma omp parallel for schedule(static)
    for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) {
      const int64_t i = order[k];
      double s = x[i];
      if (!first)
        for (int64_t p = A.rp[i]; p < A.rp[i + 1]; ++p)
          if (A.ci[p] != i) s = std::fma(-A.v[p], y[A.ci[p]], s);
      y[i] = s * rd[i];
    }
  }

  // natural-order symmetric Gauss-Seidel (precond 5) and ILU(0) (precond
  // 6): the GPU runs them as level-scheduled sweeps whose rows compute
  // exactly these sequential loops (explicitly rounded, no fused
  // multiply-adds), so they are restated in row order
  void natural_sgs(const double* x, double* y) const {
    const int64_t n = A.n;
    std::fill(y, y + n, 0.0);
    auto relax = [&](int64_t i) {
      double s = x[i];
      for (int64_t p = A.rp[i]; p < A.rp[i + 1]; ++p)
        if (A.ci[p] != i) s = s - A.v[p] * y[A.ci[p]];
      y[i] = s / A.v[dpos[i]];
    };
    for (int64_t i = 0; i < n; ++i) relax(i);
    for (int64_t i = n - 1; i >= 0; --i) relax(i);
  }
  void ilu0(const double* x, double* y) {
    const int64_t n = A.n;
    if (lu.empty()) {
      lu.assign(A.v, A.v + A.rp[n]);
      for (int64_t i = 0; i < n; ++i) {
        const int64_t e = A.rp[i + 1];
        for (int64_t p = A.rp[i]; p < e; ++p) {
          const int64_t k = A.ci[p];
          if (k >= i) break;
          const double l = lu[p] / lu[dpos[k]];
          lu[p] = l;
          int64_t qk = dpos[k] + 1;
          const int64_t ek = A.rp[k + 1];
          for (int64_t q = p + 1; q < e; ++q) {
            const int64_t j = A.ci[q];
            while (qk < ek && A.ci[qk] < j) ++qk;
            if (qk < ek && A.ci[qk] == j) lu[q] = lu[q] - l * lu[qk];
          }
        }
      }
    }
    for (int64_t i = 0; i < n; ++i) {
      double s = x[i];
      for (int64_t p = A.rp[i]; p < dpos[i]; ++p) s = s - lu[p] * y[A.ci[p]];
      y[i] = s;
    }
    for (int64_t i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (int64_t p = dpos[i] + 1; p < A.rp[i + 1]; ++p) s = s - lu[p] * y[A.ci[p]];
      y[i] = s / lu[dpos[i]];
    }
  }

  void apply(const double* x, double* y) {
    const int64_t n = A.n;
    if (precond == 5) {
      natural_sgs(x, y);
    } else if (precond == 6) {
      ilu0(x, y);
    } else if (precond == 0) {
      std::memcpy(y, x, sizeof(double) * n);
    } else if (precond == 1) {
      for (int64_t i = 0; i < n; ++i) y[i] = x[i] * rd[i];
    } else if (precond == 2) {
      std::fill(y, y + n, 0.0);
      for (int c = 0; c < ncol; ++c) gs_class(c, c == 0, x, y);
      for (int c = ncol - 2; c >= 0; --c) gs_class(c, false, x, y);
    } else {
      sc.resize(3 * n);
      double* g[2] = {sc.data(), sc.data() + n};
      double* r1 = sc.data() + 2 * n;
      auto tri = [&](bool upper, const double* r, double* out) {
        for (int64_t i = 0; i < n; ++i) g[0][i] = r[i] * rd[i];
        int cur = 0;
        for (int k = 0; k < inner; ++k) {
          gtri(A, lanes, upper, rd.data(), r, g[cur], g[1 - cur]);
          cur = 1 - cur;
        }
        std::memcpy(out, g[cur], sizeof(double) * n);
      };
      tri(false, x, y);
      gspmv_lanes(A, lanes, y, x, r1);
      tri(true, r1, r1);
      for (int64_t i = 0; i < n; ++i) y[i] += r1[i];
    }
  }

  // maxpy_k: w -= sum_k h[k] V[k]; optionally ||w||^2 in the kernel's order
  double maxpy(int nv, const double* V, const double* h, double* w, bool norm) const {
    const int64_t n = A.n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      double acc = w[i];
      for (int k = 0; k < nv; ++k) acc = std::fma(-h[k], V[int64_t(k) * n + i], acc);
      w[i] = acc;
    }
    if (!norm) return 0.0;
    const int64_t G1 = (n + kBlock - 1) / kBlock;
    std::vector<double> partial(G1);
#pragma omp parallel for schedule(static)
    for (int64_t blk = 0; blk < G1; ++blk) {
      double tv[kBlock];
      for (int t = 0; t < kBlock; ++t) {
        const int64_t i = blk * kBlock + t;
        tv[t] = i < n ? std::fma(w[i], w[i], 0.0) : 0.0;
      }
      partial[blk] = block_sum(tv);
    }
    return reduce_partials(partial.data(), G1);
  }
};

void fill_report(or_solve_report* rep, int its, int conv, double rel, double fabs, double bn) {
  if (!rep) return;
  rep->iterations = its;
  rep->converged = conv;
  rep->final_rel_implicit = rel;
  rep->final_abs_explicit = fabs;
  rep->rhs_norm = bn;
}

// KrylovSolver::gmres (restarted, right preconditioned, ICGS: two classical
// Gram-Schmidt passes; the Jacobi scaling fused into the normalisation)
int gmres(Solver& S, const double* b, double* x, int m, int max_iters, double tol, bool flexible,
          std::vector<double>& hist, or_solve_report* rep) {
  const int64_t n = S.A.n;
  std::fill(x, x + n, 0.0);
  const double bnorm = std::sqrt(S.dot(b, b));
  hist.assign(1, 1.0);
  if (!std::isfinite(bnorm)) return 6;
  if (bnorm == 0.0) {
    fill_report(rep, 0, 1, 0.0, 0.0, 0.0);
    return 0;
  }
  std::vector<double> V(size_t(m + 1) * n), Z(flexible ? size_t(m) * n : n), w(n), r(b, b + n), zt(n);
  std::vector<double> H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), hs(m + 1), h2(m + 1);
  const bool fuse = S.precond == 1;
  double beta = bnorm, rel = 1.0;
  int its = 0, status = 0;
  bool done = false;
  auto zvec = [&](int j) { return flexible ? Z.data() + size_t(j) * n : Z.data(); };
  auto scale = [&](const double* src, double* dst, double nrm, double* z) {
    const double inv = nrm != 0.0 ? 1.0 / nrm : 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const double vi = src[i] * inv;
      dst[i] = vi;
      if (z) z[i] = vi * S.rd[i];
    }
  };
  while (!done && its < max_iters) {
    scale(r.data(), V.data(), beta, fuse ? zvec(0) : nullptr);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && its < max_iters; ++j) {
      double* vj = V.data() + size_t(j) * n;
      double* zj = zvec(j);
      if (!fuse) S.apply(vj, zj);
      gspmv(S.A, zj, nullptr, w.data());
      for (int k = 0; k <= j; ++k) hs[k] = S.dot(V.data() + size_t(k) * n, w.data());
      S.maxpy(j + 1, V.data(), hs.data(), w.data(), false);
      for (int k = 0; k <= j; ++k) {
        h2[k] = S.dot(V.data() + size_t(k) * n, w.data());
        hs[k] += h2[k];
      }
      const double hn = std::sqrt(S.maxpy(j + 1, V.data(), h2.data(), w.data(), true));
      double* znext = (j + 1 < m) ? zvec(j + 1) : nullptr;
      scale(w.data(), V.data() + size_t(j + 1) * n, hn, (fuse && znext) ? znext : nullptr);
      for (int k = 0; k <= j; ++k) H[size_t(k) * m + j] = hs[k];
      H[size_t(j + 1) * m + j] = hn;
      for (int k = 0; k < j; ++k) {
        const double a = H[size_t(k) * m + j], bb = H[size_t(k + 1) * m + j];
        H[size_t(k) * m + j] = cs[k] * a + sn[k] * bb;
        H[size_t(k + 1) * m + j] = -sn[k] * a + cs[k] * bb;
      }
      const double a = H[size_t(j) * m + j], bb = H[size_t(j + 1) * m + j];
      const double den = std::sqrt(a * a + bb * bb);
      if (!(den > 0.0) || !std::isfinite(den)) {
        status = std::isfinite(den) ? 7 : 6;
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
      hist.push_back(rel);
      if (!std::isfinite(rel)) {
        status = 6;
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
      const double* basis = flexible ? Z.data() : V.data();
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int k = 0; k < kk; ++k) acc = std::fma(y[k], basis[size_t(k) * n + i], acc);
        w[i] = acc;
      }
      if (flexible) {
        for (int64_t i = 0; i < n; ++i) x[i] = std::fma(1.0, w[i], x[i]);
      } else {
        S.apply(w.data(), zt.data());
        for (int64_t i = 0; i < n; ++i) x[i] = std::fma(1.0, zt[i], x[i]);
      }
    }
    if (done || its >= max_iters) break;
    gspmv(S.A, x, b, r.data());
    beta = std::sqrt(S.dot(r.data(), r.data()));
    if (beta == 0.0) break;
  }
  gspmv(S.A, x, b, r.data());
  const double fabs_ = std::sqrt(S.dot(r.data(), r.data()));
  fill_report(rep, its, rel <= tol ? 1 : 0, rel, fabs_, bnorm);
  return status;
}

// KrylovSolver::cg
int cg(Solver& S, const double* b, double* x, int max_iters, double tol, std::vector<double>& hist,
       or_solve_report* rep) {
  const int64_t n = S.A.n;
  std::fill(x, x + n, 0.0);
  const double bnorm = std::sqrt(S.dot(b, b));
  hist.assign(1, 1.0);
  if (!std::isfinite(bnorm)) return 6;
  if (bnorm == 0.0) {
    fill_report(rep, 0, 1, 0.0, 0.0, 0.0);
    return 0;
  }
  std::vector<double> r(b, b + n), z(n), p(n), q(n);
  S.apply(r.data(), z.data());
  p = z;
  double rz = S.dot(r.data(), z.data()), rel = 1.0;
  int its = 0, status = 0;
  while (its < max_iters) {
    gspmv(S.A, p.data(), nullptr, q.data());
    const double pq = S.dot(p.data(), q.data());
    const double alpha = rz / pq;
    if (!std::isfinite(alpha)) {
      status = 7;
      break;
    }
    for (int64_t i = 0; i < n; ++i) x[i] = std::fma(alpha, p[i], x[i]);
    for (int64_t i = 0; i < n; ++i) r[i] = std::fma(-alpha, q[i], r[i]);
    ++its;
    rel = std::sqrt(S.dot(r.data(), r.data())) / bnorm;
    hist.push_back(rel);
    if (rel <= tol) break;
    S.apply(r.data(), z.data());
    const double rzn = S.dot(r.data(), z.data());
    const double beta = rzn / rz;
    rz = rzn;
    for (int64_t i = 0; i < n; ++i) p[i] = std::fma(beta, p[i], z[i]);
  }
  gspmv(S.A, x, b, r.data());
  fill_report(rep, its, rel <= tol ? 1 : 0, rel, std::sqrt(S.dot(r.data(), r.data())), bnorm);
  return status;
}

// KrylovSolver::bicgstab
int bicgstab(Solver& S, const double* b, double* x, int max_iters, double tol, std::vector<double>& hist,
             or_solve_report* rep) {
  const int64_t n = S.A.n;
  std::fill(x, x + n, 0.0);
  const double bnorm = std::sqrt(S.dot(b, b));
  hist.assign(1, 1.0);
  if (!std::isfinite(bnorm)) return 6;
  if (bnorm == 0.0) {
    fill_report(rep, 0, 1, 0.0, 0.0, 0.0);
    return 0;
  }
  std::vector<double> r(b, b + n), rh(b, b + n), p(n, 0.0), v(n, 0.0), ph(n), sv(n), sh(n), t(n);
  double rho = 1.0, alpha = 1.0, omega = 1.0, rel = 1.0;
  int its = 0, status = 0;
  while (its < max_iters) {
    const double rho_n = S.dot(rh.data(), r.data());
    if (rho_n == 0.0 || omega == 0.0 || !std::isfinite(rho_n)) {
      status = 7;
      break;
    }
    const double beta = (rho_n / rho) * (alpha / omega);
    rho = rho_n;
    for (int64_t i = 0; i < n; ++i) p[i] = std::fma(beta, std::fma(-omega, v[i], p[i]), r[i]);
    S.apply(p.data(), ph.data());
    gspmv(S.A, ph.data(), nullptr, v.data());
    const double rv = S.dot(rh.data(), v.data());
    if (rv == 0.0 || !std::isfinite(rv)) {
      status = 7;
      break;
    }
    alpha = rho / rv;
    for (int64_t i = 0; i < n; ++i) sv[i] = std::fma(1.0, r[i], -alpha * v[i]);
    S.apply(sv.data(), sh.data());
    gspmv(S.A, sh.data(), nullptr, t.data());
    const double tt = S.dot(t.data(), t.data());
    omega = tt > 0.0 ? S.dot(t.data(), sv.data()) / tt : 0.0;
    for (int64_t i = 0; i < n; ++i) {
      x[i] = std::fma(omega, sh[i], std::fma(alpha, ph[i], x[i]));
      r[i] = std::fma(-omega, t[i], sv[i]);
    }
    ++its;
    rel = std::sqrt(S.dot(r.data(), r.data())) / bnorm;
    hist.push_back(rel);
    if (rel <= tol) break;
  }
  gspmv(S.A, x, b, r.data());
  fill_report(rep, its, rel <= tol ? 1 : 0, rel, std::sqrt(S.dot(r.data(), r.data())), bnorm);
  return status;
}

// KrylovSolver::tfqmr
int tfqmr(Solver& S, const double* b, double* x, int max_iters, double tol, std::vector<double>& hist,
          or_solve_report* rep) {
  const int64_t n = S.A.n;
  std::fill(x, x + n, 0.0);
  const double bnorm = std::sqrt(S.dot(b, b));
  hist.assign(1, 1.0);
  if (!std::isfinite(bnorm)) return 6;
  if (bnorm == 0.0) {
    fill_report(rep, 0, 1, 0.0, 0.0, 0.0);
    return 0;
  }
  std::vector<double> w(b, b + n), u(b, b + n), uh(n), Aub(n), Aunb(n), v(n), dh(n, 0.0), r(n);
  double* Au = Aub.data();
  double* Aun = Aunb.data();
  S.apply(u.data(), uh.data());
  gspmv(S.A, uh.data(), nullptr, Au);
  std::memcpy(v.data(), Au, sizeof(double) * n);
  double tau = bnorm, theta = 0.0, eta = 0.0, alpha = 0.0, rel = 1.0;
  double rho = S.dot(b, b);
  int its = 0, status = 0;
  for (int64_t mm = 0; its < max_iters; ++mm) {
    if (mm % 2 == 0) {
      const double vr = S.dot(v.data(), b);
      if (vr == 0.0 || !std::isfinite(vr)) {
        status = 7;
        break;
      }
      alpha = rho / vr;
    }
    const double coef = alpha != 0.0 ? theta * theta / alpha * eta : 0.0;
    for (int64_t i = 0; i < n; ++i) {
      w[i] = std::fma(-alpha, Au[i], w[i]);
      dh[i] = std::fma(coef, dh[i], uh[i]);
    }
    theta = std::sqrt(S.dot(w.data(), w.data())) / tau;
    const double c = 1.0 / std::sqrt(1.0 + theta * theta);
    tau = tau * theta * c;
    eta = c * c * alpha;
    for (int64_t i = 0; i < n; ++i) x[i] = std::fma(eta, dh[i], x[i]);
    if (mm % 2 == 0) {
      for (int64_t i = 0; i < n; ++i) u[i] = std::fma(-alpha, v[i], u[i]);
      S.apply(u.data(), uh.data());
      gspmv(S.A, uh.data(), nullptr, Aun);
      std::swap(Au, Aun);
    } else {
      ++its;
      rel = std::sqrt(double(mm + 2)) * tau / bnorm;
      hist.push_back(rel);
      if (!std::isfinite(rel)) {
        status = 7;
        break;
      }
      if (rel <= tol) break;
      if (rho == 0.0) {
        status = 7;
        break;
      }
      const double rho_n = S.dot(w.data(), b);
      const double beta = rho_n / rho;
      rho = rho_n;
      for (int64_t i = 0; i < n; ++i) u[i] = std::fma(beta, u[i], w[i]);
      S.apply(u.data(), uh.data());
      gspmv(S.A, uh.data(), nullptr, Aun);
      for (int64_t i = 0; i < n; ++i) v[i] = std::fma(beta, std::fma(beta, v[i], Au[i]), Aun[i]);
      std::swap(Au, Aun);
    }
  }
  gspmv(S.A, x, b, r.data());
  fill_report(rep, its, rel <= tol ? 1 : 0, rel, std::sqrt(S.dot(r.data(), r.data())), bnorm);
  return status;
}

// s-step GMRES (method 5): KrylovSolver::sstep_gmres in the GPU's order.
// Blocks of s vectors by the scaled matrix powers, two block classical
// Gram-Schmidt passes, CholeskyQR twice, the block's Hessenberg columns
// from the change of basis, Givens rotations column by column.
int sstep_gmres(Solver& S, const double* b, double* x, int m, int sstep, int max_iters, double tol,
                std::vector<double>& hist, or_solve_report* rep) {
  const int64_t n = S.A.n;
  std::fill(x, x + n, 0.0);
  const double bnorm = std::sqrt(S.dot(b, b));
  hist.assign(1, 1.0);
  if (!std::isfinite(bnorm)) return 6;
  if (bnorm == 0.0) {
    fill_report(rep, 0, 1, 0.0, 0.0, 0.0);
    return 0;
  }
  const int ldc = m + 1;
  std::vector<double> V(size_t(m + 1) * n), r(b, b + n), z(n), w(n);
  std::vector<double> Hr(size_t(m + 1) * m), H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  std::vector<double> Ch(size_t(ldc) * sstep), Cp(size_t(ldc) * sstep), Gh(size_t(sstep) * sstep);
  auto scale = [&](const double* src, double* dst, double nrm) {
    const double inv = nrm != 0.0 ? 1.0 / nrm : 0.0;
    for (int64_t i = 0; i < n; ++i) dst[i] = src[i] * inv;
  };
  double beta = bnorm, rel = 1.0, sigma = 1.0;
  int its = 0, status = 0;
  bool done = false;
  while (!done && its < max_iters) {
    scale(r.data(), V.data(), beta);
    std::fill(H.begin(), H.end(), 0.0);
    std::fill(Hr.begin(), Hr.end(), 0.0);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j0 = 0, kk = 0;
    while (j0 < m && its < max_iters && !done) {
      const int sb = std::min(sstep, std::min(m - j0, max_iters - its));
      double* W = V.data() + size_t(j0 + 1) * n;
      for (int k = 0; k < sb; ++k) {
        double* wk = W + size_t(k) * n;
        S.apply(V.data() + size_t(j0 + k) * n, z.data());
        gspmv(S.A, z.data(), nullptr, wk);
        scale(wk, wk, sigma);
      }
      std::fill(Ch.begin(), Ch.end(), 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        for (int k = 0; k < sb; ++k)
          for (int i = 0; i <= j0; ++i) Cp[size_t(k) * ldc + i] = S.dot(V.data() + size_t(i) * n, W + size_t(k) * n);
        for (int k = 0; k < sb; ++k) S.maxpy(j0 + 1, V.data(), &Cp[size_t(k) * ldc], W + size_t(k) * n, false);
        for (int k = 0; k < sb; ++k)
          for (int i = 0; i <= j0; ++i) Ch[size_t(k) * ldc + i] += Cp[size_t(k) * ldc + i];
      }
      std::vector<double> Rt(size_t(sb) * sb, 0.0), Rp(size_t(sb) * sb), tmp(size_t(sb) * sb);
      for (int k = 0; k < sb; ++k) Rt[size_t(k) * sb + k] = 1.0;
      bool broke = false;
      for (int pass = 0; pass < 2 && !broke; ++pass) {
        for (int k = 0; k < sb; ++k)
          for (int i = 0; i < sb; ++i) Gh[size_t(k) * sstep + i] = S.dot(W + size_t(i) * n, W + size_t(k) * n);
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
          double* wk = W + size_t(k) * n;
          if (k > 0) S.maxpy(k, W, &Rp[size_t(k) * sb], wk, false);
          scale(wk, wk, Rp[size_t(k) * sb + k]);
        }
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
        status = 7;
        done = true;
        break;
      }
      const int rows = j0 + sb + 1;
      std::vector<double> Mx(size_t(rows) * sb, 0.0), Tn(size_t(sb) * sb, 0.0), Hn(size_t(rows) * sb, 0.0);
      for (int k = 0; k < sb; ++k) {
        for (int i = 0; i <= j0; ++i) Mx[size_t(k) * rows + i] = sigma * Ch[size_t(k) * ldc + i];
        for (int i = 0; i <= k; ++i) Mx[size_t(k) * rows + j0 + 1 + i] = sigma * Rt[size_t(k) * sb + i];
        if (k > 0)
          for (int i = 0; i <= j0; ++i) {
            double v = 0.0;
            for (int l = 0; l < j0; ++l) v += Hr[size_t(i) * m + l] * Ch[size_t(k - 1) * ldc + l];
            Mx[size_t(k) * rows + i] -= v;
          }
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
          status = std::isfinite(den) ? 7 : 6;
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
        hist.push_back(rel);
        kk = j + 1;
        if (!std::isfinite(rel)) {
          status = 6;
          done = true;
          break;
        }
        if (rel <= tol) {
          done = true;
          break;
        }
      }
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
      for (int64_t i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int k = 0; k < kk; ++k) acc = std::fma(y[k], V[size_t(k) * n + i], acc);
        w[i] = acc;
      }
      S.apply(w.data(), z.data());
      for (int64_t i = 0; i < n; ++i) x[i] = std::fma(1.0, z[i], x[i]);
    }
    if (done || its >= max_iters) break;
    gspmv(S.A, x, b, r.data());
    beta = std::sqrt(S.dot(r.data(), r.data()));
    if (beta == 0.0) break;
  }
  gspmv(S.A, x, b, r.data());
  fill_report(rep, its, rel <= tol ? 1 : 0, rel, std::sqrt(S.dot(r.data(), r.data())), bnorm);
  return status;
}

}  // namespace

extern "C" int or_solve_gpu_order(int64_t nrows, const int64_t* row_ptr, const int32_t* col_idx,
                                  const double* vals, const double* b, double* x, int method,
                                  int precond, const int64_t* order, const int64_t* class_ptr,
                                  int nclasses, int kspace, int max_iters, double tol,
                                  double* history, or_solve_report* rep, int inner_sweeps,
                                  int red_blocks, int lanes, int sstep_size) {
  Solver S;
  S.A = {nrows, row_ptr, col_idx, vals};
  S.G = std::max(1, red_blocks);
  S.lanes = lanes;
  S.precond = precond;
  S.order = order;
  S.cptr = class_ptr;
  S.ncol = nclasses;
  S.inner = inner_sweeps;
  if (precond == 2 && (!order || !class_ptr || nclasses < 1)) return 1;
  S.rd.resize(nrows);
  S.dpos.assign(nrows, 0);
  for (int64_t i = 0; i < nrows; ++i) {
    double d = 0.0;
    for (int64_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p)
      if (col_idx[p] == i) {
        d = vals[p];
        S.dpos[i] = p;
      }
    S.rd[i] = 1.0 / d;
  }
  std::vector<double> hist;
  int st;
  if (method == 1)
    st = cg(S, b, x, max_iters, tol, hist, rep);
  else if (method == 3)
    st = bicgstab(S, b, x, max_iters, tol, hist, rep);
  else if (method == 4)
    st = tfqmr(S, b, x, max_iters, tol, hist, rep);
  else if (method == 5)
    st = sstep_gmres(S, b, x, std::max(1, kspace), sstep_size > 0 ? sstep_size : 5, max_iters, tol, hist, rep);
  else
    st = gmres(S, b, x, std::max(1, kspace), max_iters, tol, method == 2, hist, rep);
  if (history)
    for (size_t k = 0; k < hist.size() && k <= size_t(max_iters); ++k) history[k] = hist[k];
  return st;
}
