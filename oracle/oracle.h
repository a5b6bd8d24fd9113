/*
 * CPU oracle for the nalu-wind edge-assembly + Krylov hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it to compute the
 * reference answer on the host. No product code path links or calls it.
 *
 * It restates, in FP64 C++, the reference algorithms cited at each function:
 *   - STK "generated:NXxNYxNZ" hex mesh numbering and STK edge creation
 *   - Hex8 sub-control-surface area vectors and dual nodal volumes
 *   - the Tpetra CSR graph of TpetraLinearSystem (row/column LID rules)
 *   - ScalarEdgeSolverAlg / ContinuityEdgeSolverAlg / MomentumEdgeSolverAlg
 *   - TpetraLinearSystem::sum_into (serial semantics, or OpenMP atomics)
 *   - applyDirichletBCs / resetRows
 *   - Ifpack2-style Jacobi and symmetric Gauss-Seidel relaxation (1 sweep)
 *   - right-preconditioned restarted GMRES with iterated classical
 *     Gram-Schmidt, and preconditioned CG.
 *
 * Parity of the edge kernels, graph and geometry is pinned by the
 * reference's unit-test golds (tests/golden). The Krylov residual history is
 * not pinned by any reference test (Belos is a third-party, unversioned
 * dependency); the GMRES restated here defines it.
 *
 * All node arrays are indexed by 0-based node index; node "ids" are the
 * 1-based STK identifiers. Edge arrays are E x 2 node indices.
 */
#ifndef NW_ORACLE_H
#define NW_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int or_version(void);

/* ---- mesh restatement (STK generated mesh, create_edges) ---- */
/* Node/element counts of a generated:NXxNYxNZ block. */
int64_t or_hex_box_num_nodes(int nx, int ny, int nz);
int64_t or_hex_box_num_elems(int nx, int ny, int nz);
/* Unit-cube coordinates (N x 3) and exodus-ordered Hex8 connectivity
 * (nelem x 8, 0-based node indices). */
void or_hex_box(int nx, int ny, int nz, double* coords, int64_t* conn);
/* Seeded synthetic box coordinates (N x 3, or_hex_box numbering): z
 * stretched from z = 0 by `stretch`, interior nodes jittered by
 * jitter x local spacing from splitmix64(seed) draws, three per node in node
 * order. The benchmark workloads' definition, not reference code. */
void or_box_coords(int nx, int ny, int nz, double lx, double ly, double lz,
                   double stretch, double jitter, uint64_t seed, double* coords);
/* STK create_edges restatement for Hex8: edges in order of first creation
 * (elements in order, hex edge ordinals 0..11), node[0] = lower id.
 * Returns E; writes up to cap edges (E x 2). elem_edges (nelem x 12) gets the
 * edge index of each element edge ordinal. */
int64_t or_hex8_edges(int64_t nelem, const int64_t* conn, int64_t nnodes,
                      int64_t cap, int64_t* edges, int64_t* elem_edges);

/* ---- geometry restatement ---- */
/* Edge area vectors (E x 3) and dual nodal volumes (N) from Hex8 SCS/SCV. */
void or_hex8_geometry(int64_t nnodes, const double* coords, int64_t nelem,
                      const int64_t* conn, const int64_t* elem_edges,
                      int64_t nedges, const int64_t* edges, double* area,
                      double* dualvol);

/* ---- Tpetra graph restatement ---- */
/* nalu_id[n] = 1-based id of the master of node n (own id if not a slave).
 * Rows are the non-slave nodes sorted by id, numDof rows each.
 * Pass 1 (row_ptr==NULL): returns nrows and *nnz_out. Pass 2 fills
 * row_ptr (nrows+1), col_idx (nnz), node_lid (nnodes, first row of the node's
 * master). */
/* LocalGraphArrays (include/LinearSolver.h:80-151) replay: row lengths,
 * then insertIndices(op_row[k], op_n[k], next op_n[k] of op_cols, num_dof)
 * in order; returns 1 on row overflow. */
int or_local_graph_replay(int nrows, const int64_t* row_lengths, int nops,
                          const int32_t* op_row, const int32_t* op_n,
                          const int32_t* op_cols, int num_dof,
                          int64_t* row_ptr, int32_t* col_idx);
/* Face-IP area vectors of quad (nn 4, Quad3DSCS) or triangle (nn 3,
 * Tri3DSCS) faces; faces: nfaces x nn node ids; areav: nfaces x nn x 3. */
void or_face_scs_areas(int64_t nfaces, int nn, const int64_t* faces,
                       const double* coords, double* areav);
int64_t or_build_graph(int64_t nnodes, const int64_t* nalu_id, int64_t nedges,
                       const int64_t* edges, int num_dof, int64_t* nnz_out,
                       int64_t* row_ptr, int32_t* col_idx, int64_t* node_lid);

/* ---- edge kernels ---- */
typedef struct or_scalar_opts {
  double alpha, alpha_upw, upw_factor, relax, hybrid_factor;
  int use_limiter;
  int tanh_form; /* 0 = classic Peclet function, 1 = tanh */
  double tanh_trans, tanh_width;
} or_scalar_opts;

typedef struct or_momentum_opts {
  double alpha, alpha_upw, upw_factor, relax, include_div_u;
  int use_limiter;
} or_momentum_opts;

typedef struct or_continuity_opts {
  double noc_fac, tau_scale, interp_together, solve_incompressible;
} or_continuity_opts;

/* ---- boundary face-IP kernels ----
 * ipn: nip x 2 (face node R, opposing element node L). Local systems in the
 * edge layout with node order (R, L), L rows zero: lhs nip x 4 / rhs nip x 2
 * (1 dof) or lhs nip x 36 / rhs nip x 6 (3 dofs). areav: exposed area
 * vector per face IP (nip x 3); dynp, mdot: per face IP. The *_mag variants
 * return running magnitudes instead of values. */
typedef struct or_continuity_open_opts {
  double tau_scale, noc_fac, pstab_fac, mdot_corr, solve_incompressible;
} or_continuity_open_opts;
typedef struct or_momentum_open_opts {
  double include_div_u, nf_entrain;
  int entrainment; /* 0 = COMPUTED, 1 = SPECIFIED */
} or_momentum_open_opts;
typedef struct or_momentum_symmetry_opts {
  double include_div_u, penalty_factor;
} or_momentum_symmetry_opts;
/* ContinuityOpenEdgeKernel.C:92-160 (dynp may be NULL: zero) */
void or_continuity_open_local(int64_t nip, const int64_t* ipn, const double* coords,
                              const double* velocity, const double* dpdx,
                              const double* density, const double* pressure,
                              const double* pressure_bc, const double* udiag,
                              const double* areav, const double* dynp,
                              const or_continuity_open_opts* o, double* lhs, double* rhs);
/* MomentumOpenEdgeKernel.C:80-270 */
void or_momentum_open_local(int64_t nip, const int64_t* ipn, const double* coords,
                            const double* velocity, const double* dudx,
                            const double* viscosity, const double* velocity_bc,
                            const double* areav, const double* mdot,
                            const or_momentum_open_opts* o, double* lhs, double* rhs);
/* MomentumSymmetryEdgeKernel.C:64-206 */
void or_momentum_symmetry_local(int64_t nip, const int64_t* ipn, const double* coords,
                                const double* velocity, const double* dudx,
                                const double* viscosity, const double* areav,
                                const or_momentum_symmetry_opts* o, double* lhs, double* rhs);
typedef struct or_abl_wall_opts {
  double gravity, z0, Tref, kappa, beta_m, gamma_m;
} or_abl_wall_opts;
/* MomentumABLWallFuncEdgeKernel.C:80-158 (ustar, zh: per face IP) */
void or_abl_wall_local(int64_t nip, const int64_t* ipn, const double* velocity,
                       const double* wall_velocity_bc, const double* density,
                       const double* heat_flux_bc, const double* specific_heat,
                       const double* areav, const double* ustar, const double* zh,
                       const or_abl_wall_opts* o, double* lhs, double* rhs);
/* MomentumABLWallShearStressEdgeKernel.C:49-88 (tau: per face IP x 3) */
void or_abl_shear_local(int64_t nip, const int64_t* ipn, const double* areav,
                        const double* tau, int slip, double* lhs, double* rhs);
/* ScalarOpenEdgeKernel.C:49-72 / ScalarEdgeOpenSolverAlg.C:64-104 */
void or_scalar_open_local(int64_t nip, const int64_t* ipn, const double* q,
                          const double* q_bc, const double* mdot, double relax,
                          double* lhs, double* rhs);
/* MdotOpenEdgeAlg.C:55-150: open mass flow rate per face IP */
void or_mdot_open(int64_t nip, const int64_t* ipn, const double* coords,
                  const double* velocity, const double* dpdx, const double* density,
                  const double* pressure, const double* pressure_bc, const double* udiag,
                  const double* areav, const double* dynp, double noc_fac,
                  double pstab_fac, double* mdot);
/* threads of the OpenMP loops without an explicit count (0: default) */
void or_set_threads(int n);
/* default-seeded std::mt19937 uniform(lo[i], hi[i]) draws, in order */
void or_mt19937_uniform(int n, const double* lo, const double* hi, double* out);

/* Per-edge local systems: lhs (E x 4) row-major 2x2 and rhs (E x 2). */
void or_scalar_edge_local(int64_t nedges, const int64_t* edges,
                          const double* coords, const double* vrtm,
                          const double* q, const double* dqdx,
                          const double* density, const double* diff_coeff,
                          const double* area, const double* mdot,
                          const or_scalar_opts* o, double* lhs, double* rhs);
void or_continuity_edge_local(int64_t nedges, const int64_t* edges,
                              const double* coords, const double* velocity,
                              const double* dpdx, const double* density,
                              const double* pressure, const double* udiag,
                              const double* area, const or_continuity_opts* o,
                              double* lhs, double* rhs);
/* lhs (E x 36) row-major 6x6 with local dof = node*3 + component. */
void or_momentum_edge_local(int64_t nedges, const int64_t* edges,
                            const double* coords, const double* vrtm,
                            const double* velocity, const double* dudx,
                            const double* viscosity, const double* density,
                            const double* mask, const double* area,
                            const double* mdot, const double* pecfac,
                            const or_momentum_opts* o, double* lhs,
                            double* rhs);

/* Running-magnitude versions of the three kernels: each output entry is
 * the same expression evaluated on |inputs| (|a+b| -> |a|+|b|,
 * |ab| -> |a||b|, |a/b| -> |a|/|b|). Any evaluation order of an entry
 * differs from the value above by a small multiple of eps times this
 * magnitude; the GPU parity tests use it as their tolerance scale. */
void or_scalar_edge_local_mag(int64_t nedges, const int64_t* edges,
                              const double* coords, const double* vrtm,
                              const double* q, const double* dqdx,
                              const double* density, const double* diff_coeff,
                              const double* area, const double* mdot,
                              const or_scalar_opts* o, double* lhs, double* rhs);
void or_continuity_edge_local_mag(int64_t nedges, const int64_t* edges,
                                  const double* coords, const double* velocity,
                                  const double* dpdx, const double* density,
                                  const double* pressure, const double* udiag,
                                  const double* area,
                                  const or_continuity_opts* o, double* lhs,
                                  double* rhs);
void or_momentum_edge_local_mag(int64_t nedges, const int64_t* edges,
                                const double* coords, const double* vrtm,
                                const double* velocity, const double* dudx,
                                const double* viscosity, const double* density,
                                const double* mask, const double* area,
                                const double* mdot, const double* pecfac,
                                const or_momentum_opts* o, double* lhs,
                                double* rhs);

/* TpetraLinearSystem::sum_into over all edges in order. nthreads <= 1 is
 * the serial (Kokkos Serial) semantics; > 1 adds with OpenMP atomics as
 * the reference's threaded build does. vals_abs / rhs_abs (optional)
 * accumulate |contribution| for tolerance scaling. */
void or_sum_into_edges(int64_t nedges, const int64_t* edges, int num_dof,
                       const double* lhs, const double* rhs,
                       const int64_t* node_lid, const int64_t* row_ptr,
                       const int32_t* col_idx, double* vals, double* rhs_out,
                       double* vals_abs, double* rhs_abs, int nthreads);

/* applyDirichletBCs restatement: for each listed node, dof rows
 * [begin,end): zero row, diag 1, rhs = bc - q (per-node arrays of
 * num_dof components). */
void or_apply_dirichlet(int64_t nlist, const int64_t* nodes, int num_dof,
                        int begin, int end, const double* q, const double* bc,
                        const int64_t* node_lid, const int64_t* row_ptr,
                        const int32_t* col_idx, double* vals, double* rhs);
/* resetRows restatement. */
void or_reset_rows(int64_t nlist, const int64_t* nodes, int begin, int end,
                   double diag_value, double rhs_residual,
                   const int64_t* node_lid, const int64_t* row_ptr,
                   const int32_t* col_idx, double* vals, double* rhs);

/* ---- Krylov ---- */
void or_spmv(int64_t nrows, const int64_t* row_ptr, const int32_t* col_idx,
             const double* vals, const double* x, double* y, int nthreads);

typedef struct or_solve_report {
  int iterations;
  int converged;
  double final_rel_implicit;
  double final_abs_explicit; /* ||b - A x||_2 */
  double rhs_norm;
} or_solve_report;

/* precond: 0 none, 1 Jacobi, 2 symmetric Gauss-Seidel in the row order
 * given by `order` (NULL = natural order; 5 is the same), 6 ILU(0) (Ifpack2
 * RILUK at level of fill 0), 4 two-stage symmetric
 * Gauss-Seidel with inner_sweeps Jacobi-Richardson corrections per
 * triangular solve (row order). method: 0 GMRES(kspace), 1 CG,
 * 3 BiCGStab, 4 TFQMR (Belos "bicgstab" / "tfqmr", the strings
 * src/LinearSolver.C:114 passes to the Belos factory; right preconditioned).
 * history (optional, capacity max_iters+1) gets ||r_k||/||r_0|| (TFQMR:
 * its residual bound sqrt(k+1) tau_k / ||r_0||). */
int or_solve(int64_t nrows, const int64_t* row_ptr, const int32_t* col_idx,
             const double* vals, const double* b, double* x, int method,
             int precond, const int64_t* order, int kspace, int max_iters,
             double tol, double* history, or_solve_report* rep,
             int nthreads, int inner_sweeps);

/* The same solvers (method 0 GMRES, 1 CG, 2 FGMRES, 3 BiCGStab, 4 TFQMR,
 * 5 s-step GMRES with step sstep_size;
 * precond 0 none, 1 Jacobi, 2 multicolour symmetric Gauss-Seidel over the
 * colour classes order[class_ptr[c] .. class_ptr[c + 1]), 4 two-stage SGS,
 * 5 natural-order symmetric Gauss-Seidel, 6 ILU(0))
 * with every sum in the GPU library's fixed order: reductions over
 * red_blocks blocks of 256 threads, sliced-ELL SpMV rows, CSR rows over
 * `lanes` lanes, fused multiply-adds where the GPU kernels use them
 * (gpu_order.cpp). For parity tests only. Returns 0 or a status. */
int or_solve_gpu_order(int64_t nrows, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* b, double* x, int method,
                       int precond, const int64_t* order, const int64_t* class_ptr,
                       int nclasses, int kspace, int max_iters, double tol,
                       double* history, or_solve_report* rep, int inner_sweeps,
                       int red_blocks, int lanes, int sstep_size);

/* Preconditioner application alone (for unit tests). */
void or_precond_apply(int64_t nrows, const int64_t* row_ptr,
                      const int32_t* col_idx, const double* vals, int precond,
                      const int64_t* order, const double* x, double* y,
                      int inner_sweeps);

/* ---- input producers ---- */
/* Unit-test mass flow rate 0.5 (rhoL uL + rhoR uR) . A. */
void or_mdot_unit_test(int64_t nedges, const int64_t* edges,
                       const double* velocity, const double* density,
                       const double* area, double* mdot);
/* MdotEdgeAlg restatement (no balanced forcing, no GCL). */
void or_mdot_edge(int64_t nedges, const int64_t* edges, const double* coords,
                  const double* velocity, const double* dpdx,
                  const double* density, const double* pressure,
                  const double* udiag, const double* area, double noc_fac,
                  double interp_together, double* mdot);
/* NodalGradEdgeAlg interior restatement: grad (N x dim1*3) += edge terms. */
void or_nodal_grad_edge(int64_t nedges, const int64_t* edges, int dim1,
                        const double* phi, const double* area,
                        const double* dualvol, double* grad);
/* Peclet functions (PecletFunction.C). */
double or_peclet_classic(double pe, double hybrid_factor);
double or_peclet_tanh(double x, double c1, double c2);

#ifdef __cplusplus
}
#endif
#endif
