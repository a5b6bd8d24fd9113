/*
 * nw_capi.h - C ABI of the GB300 edge-assembly + Krylov library
 * (libnw_gb300.so).
 *
 * This is the drop-in boundary for nalu-wind's implicit hot path. Each entry
 * point names the reference interface it replaces (paths are relative to
 * the nalu-wind source tree). Plain pointers and sizes only; no C++ or torch
 * types cross this boundary and no exception escapes it.
 *
 * Conventions
 *  - Every function returns nw_status. On error, nw_last_error_string()
 *    describes the failure (thread-local).
 *  - A handle is used from one host thread. Device work is stream-ordered on
 *    the handle's CUDA stream (nw_linsys_set_stream); pointers marked
 *    "device" must be valid device memory for the duration of the call.
 *  - Node indices are 0-based indices into the caller's node arrays. Node
 *    ids (nalu_id) are the 1-based global ids that order the matrix rows.
 *  - Node fields are interleaved per node (N x ncomp), as STK stores them.
 */
#ifndef NW_CAPI_H
#define NW_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nw_status {
  NW_OK = 0,
  NW_INVALID_ARG = 1,
  NW_CUDA_ERROR = 2,
  NW_NOT_FINALIZED = 3,
  NW_NAN_DETECTED = 4,
  NW_NOT_CONVERGED = 5,
  NW_BREAKDOWN = 6,
  NW_TIMEOUT = 7,
  NW_NO_DEVICE = 8,
  NW_INTERNAL = 9
} nw_status;

/* Krylov methods (the `method` strings passed to the Belos factory,
 * src/LinearSolver.C:114) and preconditioners (src/LinearSolverConfig.C:
 * 89-121). CG, BiCGStab and TFQMR run in FP64; with a NW_PREC_MIXED*
 * precision or NW_PC_LEARNED the solve is (F)GMRES whatever the method. */
enum { NW_GMRES = 0, NW_CG = 1, NW_FGMRES = 2, NW_BICGSTAB = 3, NW_TFQMR = 4,
       NW_SSTEP_GMRES = 5 /* "sstep_gmres": s-step GMRES with CholeskyQR2 */ };
enum {
  NW_PC_NONE = 0,
  NW_PC_JACOBI = 1, /* "jacobi" / "default": Ifpack2 Jacobi, 1 sweep */
  NW_PC_SGS = 2,    /* "mt_sgs": symmetric Gauss-Seidel, 1 sweep, multicolour
                       order (rows colour class by colour class) */
  NW_PC_LEARNED = 3, /* learned edge message-passing preconditioner (FGMRES) */
  NW_PC_SGS2 = 4,    /* "sgs2": two-stage symmetric Gauss-Seidel, 1 sweep, row
                        order, sgs2_inner_sweeps Jacobi-Richardson corrections
                        per triangular solve */
  NW_PC_SGS_NATURAL = 5, /* "sgs": Ifpack2 symmetric Gauss-Seidel, 1 sweep,
                            natural row order (forward then backward), run
                            as level-scheduled sweeps */
  NW_PC_RILUK = 6    /* "riluk": Ifpack2 RILUK at its default level of fill 0,
                        i.e. ILU(0) on the matrix's own pattern; level-scheduled
                        factorization and triangular solves */
};
/* Arithmetic of the solve. */
enum {
  NW_PREC_FP64 = 0,       /* FP64 Krylov, FP64 SpMV and preconditioner */
  NW_PREC_MIXED = 1,      /* FP32 inner Krylov inside FP64 iterative refinement */
  NW_PREC_MIXED_BF16 = 2  /* as NW_PREC_MIXED, with the Gauss-Seidel sweeps
                             reading BF16 matrix values (FP32 accumulation) */
};

/* The reference's string options as TpetraLinearSolverConfig::load reads
 * them (src/LinearSolverConfig.C:37-140): method "gmres", "cg",
 * "sstep_gmres", "tfqmr", "bicgstab" and preconditioner "jacobi" /
 * "default", "sgs", "mt_sgs", "sgs2", "riluk". Sets cfg->method and
 * cfg->preconditioner and leaves the other fields as they are.
 * "ilut" and "muelu" are rejected with NW_INVALID_ARG (not built: see the
 * library's design notes). */
nw_status nw_solver_cfg_from_strings(const char* method, const char* preconditioner,
                                     struct nw_solver_cfg* cfg);

/* TpetraLinearSolverConfig::load keys (src/LinearSolverConfig.C:37-140). */
typedef struct nw_solver_cfg {
  int method;             /* NW_GMRES, NW_CG, NW_FGMRES, NW_BICGSTAB, NW_TFQMR */
  int preconditioner;     /* NW_PC_* */
  int precision;          /* NW_PREC_* */
  int kspace;             /* "kspace", default 50 */
  int max_iterations;     /* "max_iterations", default 50 */
  double tolerance;       /* "tolerance", default 1e-4 */
  double final_tolerance; /* "final_tolerance", default = tolerance */
  int inner_kspace;       /* mixed: inner restart length */
  double inner_tolerance; /* mixed: relative reduction per inner solve */
  int sgs2_inner_sweeps;  /* "inner_iterations" of sgs2, default 1 (values < 1 mean 1) */
  int sstep_size;         /* "krylov_step_size" of sstep_gmres, default 5 (values < 1 mean 5) */
} nw_solver_cfg;

/* Per-solve report: LinearSystem::linearSolveIterations / linearResidual /
 * nonLinearResidual (include/LinearSystem.h:212-218). */
typedef struct nw_solve_report {
  int iterations;             /* total Krylov iterations */
  int outer_iterations;       /* iterative-refinement steps (mixed) */
  int status;                 /* nw_status of the solve */
  int converged;
  double final_rel_residual;  /* last tested relative residual */
  double final_abs_residual;  /* explicit ||b - A x||_2 in FP64 */
  double rhs_norm;            /* ||b||_2 (nonLinearResidual / l2Scaling) */
  double solve_ms;            /* device time of the solve, with the per-solve refresh
                                 of the solver's value copies (diagonal, sliced
                                 layouts, coarse operator) */
  int fallback;               /* learned preconditioner failed; SGS result */
} nw_solve_report;

/* SolutionOptions numerics of ScalarEdgeSolverAlg::execute
 * (src/edge_kernels/ScalarEdgeSolverAlg.C:61-69) and the Peclet function
 * factory (include/EquationSystem.h:399-413). */
typedef struct nw_scalar_opts {
  double alpha, alpha_upw, upw_factor, relax, hybrid_factor;
  int use_limiter;
  int tanh_form; /* 0 classic Peclet function, 1 tanh */
  double tanh_trans, tanh_width;
} nw_scalar_opts;

/* MomentumEdgeSolverAlg::execute options
 * (src/edge_kernels/MomentumEdgeSolverAlg.C:76-88); VOF off. */
typedef struct nw_momentum_opts {
  double alpha, alpha_upw, upw_factor, relax, include_div_u;
  int use_limiter;
} nw_momentum_opts;

/* ContinuityEdgeSolverAlg::execute options
 * (src/edge_kernels/ContinuityEdgeSolverAlg.C:42-56); tau_scale = dt/gamma1. */
typedef struct nw_continuity_opts {
  double noc_fac, tau_scale, interp_together, solve_incompressible;
} nw_continuity_opts;

/* Device field pointers. Node fields are indexed by node index, edge fields
 * by edge index in the order given to nw_linsys_build_edge_graph. */
typedef struct nw_scalar_fields {
  const double* coords;       /* N x 3 */
  const double* velocity_rtm; /* N x 3 */
  const double* q;            /* N */
  const double* dqdx;         /* N x 3 */
  const double* density;      /* N */
  const double* diff_coeff;   /* N (diffFluxCoeff) */
  const double* area;         /* E x 3 (edge_area_vector) */
  const double* mdot;         /* E (mass_flow_rate) */
} nw_scalar_fields;

typedef struct nw_continuity_fields {
  const double* coords;   /* N x 3 */
  const double* velocity; /* N x 3 */
  const double* dpdx;     /* N x 3 */
  const double* density;  /* N */
  const double* pressure; /* N */
  const double* udiag;    /* N (momentum_diag) */
  const double* area;     /* E x 3 */
} nw_continuity_fields;

typedef struct nw_momentum_fields {
  const double* coords;    /* N x 3 */
  const double* velocity;  /* N x 3 */
  const double* dudx;      /* N x 9 */
  const double* viscosity; /* N */
  const double* density;   /* N */
  const double* mask;      /* N (abl_wall_no_slip_wall_func_node_mask) */
  const double* area;      /* E x 3 */
  const double* mdot;      /* E */
  const double* pecfac;    /* E (peclet_factor) */
} nw_momentum_fields;

typedef struct nw_linsys nw_linsys;

/* ---- library ---- */
const char* nw_last_error_string(void);
int nw_version(void);
/* Select the CUDA device used by handles created afterwards. */
nw_status nw_set_device(int device);

/* ---- construction: LinearSystem::create (src/LinearSystem.C:117-159) and
 * the TpetraLinearSystem constructor; num_dof = LinearSystem::numDof. ---- */
nw_status nw_linsys_create(int num_dof, const nw_solver_cfg* cfg,
                           nw_linsys** out);
nw_status nw_linsys_destroy(nw_linsys* ls);
/* Stream for all device work of this handle (cudaStream_t; NULL = the
 * legacy default stream). */
nw_status nw_linsys_set_stream(nw_linsys* ls, void* stream);
nw_status nw_linsys_set_solver_cfg(nw_linsys* ls, const nw_solver_cfg* cfg);

/* ---- graph: LinearSystem::buildEdgeToNodeGraph
 * (include/LinearSystem.h:114-117; src/TpetraLinearSystem.C:489-494) over a
 * host edge list, then finalizeLinearSystem (src/TpetraLinearSystem.C:
 * 1137-1272). Host arrays: global_id (N) is the STK identifier of each node
 * (NULL: index + 1); nalu_id (N) is the naluGlobalId field, the id of each
 * node's periodic master (NULL: no periodic slaves). Rows are the master
 * nodes in ascending id, num_dof rows each. edge_nodes is E x 2 node
 * indices. ---- */
nw_status nw_linsys_build_edge_graph(nw_linsys* ls, int64_t num_nodes,
                                     const int64_t* global_id,
                                     const int64_t* nalu_id,
                                     int64_t num_edges,
                                     const int64_t* edge_nodes);
nw_status nw_linsys_finalize(nw_linsys* ls);
/* Graph export for parity checks (host arrays; pass NULL to query sizes). */
nw_status nw_linsys_graph_sizes(const nw_linsys* ls, int64_t* nrows,
                                int64_t* nnz);
nw_status nw_linsys_get_graph(const nw_linsys* ls, int64_t* row_ptr,
                              int32_t* col_idx);
/* Row LID (first dof row) of every node: entityToLID. Host, N entries. */
nw_status nw_linsys_get_node_lid(const nw_linsys* ls, int64_t* node_lid);

/* ---- assembly: zeroSystem (src/TpetraLinearSystem.C:1274-1291) ---- */
nw_status nw_linsys_zero(nw_linsys* ls);

/* AssembleEdgeSolverAlgorithm::run_algorithm
 * (include/AssembleEdgeSolverAlgorithm.h:47-100) with the per-edge physics
 * of ScalarEdgeSolverAlg::execute (src/edge_kernels/
 * ScalarEdgeSolverAlg.C:55-206) and the CoeffApplier sum into CSR
 * (TpetraLinearSystem::sum_into, src/TpetraLinearSystem.C:1381-1459).
 * Deterministic: no floating-point atomics. num_dof must be 1. */
nw_status nw_assemble_scalar_edges(nw_linsys* ls, const nw_scalar_fields* f,
                                   const nw_scalar_opts* o);
/* ContinuityEdgeSolverAlg::execute (src/edge_kernels/
 * ContinuityEdgeSolverAlg.C:37-195) + sum_into. num_dof must be 1. */
nw_status nw_assemble_continuity_edges(nw_linsys* ls,
                                       const nw_continuity_fields* f,
                                       const nw_continuity_opts* o);
/* The same assembly in parts, for a caller that streams its inputs to the
 * device (ContinuityEdgeSolverAlg::execute split at its edge loop):
 * nw_assemble_continuity_edge_range evaluates the coefficients of edges
 * [edge_begin, edge_end) into the handle's edge buffer. The ranges of one
 * assembly come in order from edge 0 (a later range must start where the
 * previous one ended, else NW_INVALID_ARG). Each range reads the node
 * fields of nodes 0 .. m only, m the largest node index of edges
 * 0 .. edge_end - 1 (it also evaluates the per-node quantities of the node
 * pre-pass form for the nodes that m newly covers), so a caller can copy
 * the node fields in index order, a slice ahead of each edge range.
 * nw_assemble_continuity_rows then sums the coefficients into the CSR values
 * and rhs (NW_INVALID_ARG unless the ranges covered every edge). Together
 * they equal nw_assemble_continuity_edges bit for bit. */
nw_status nw_assemble_continuity_edge_range(nw_linsys* ls, const nw_continuity_fields* f,
                                            const nw_continuity_opts* o, int64_t edge_begin,
                                            int64_t edge_end);
nw_status nw_assemble_continuity_rows(nw_linsys* ls);
/* No counterpart in the reference. The continuity assembly above for
 * callers that cannot allocate device memory when they assemble (a host
 * code whose device memory all comes from its own pool allocator, sized up
 * front): per-edge scratch lives in a fixed 8 MiB device array inside the
 * library, and the assembled values (nnz) and rhs (nrows) go to the
 * caller's device arrays, overwritten. The result equals
 * nw_linsys_zero + nw_assemble_continuity_edges within rounding: this path
 * always evaluates the general continuity edge kernel, which rounds
 * differently from the node pre-pass form the regular entry point takes
 * with the reference's default options. Allocates nothing. Meshes above
 * 524,288 edges are rejected with NW_INVALID_ARG. The handle's device must
 * be the current device (else NW_INVALID_ARG). The first call on a device
 * looks up the array's address with that device current and keeps it for
 * the life of the process: a cudaDeviceReset afterwards is not supported.
 * All calls share the array, so calls that overlap on the GPU race. The
 * handle's own values and rhs are not touched. */
nw_status nw_assemble_continuity_edges_noalloc(const nw_linsys* ls,
                                               const nw_continuity_fields* f,
                                               const nw_continuity_opts* o,
                                               double* values, double* rhs);
/* MomentumEdgeSolverAlg::execute (src/edge_kernels/
 * MomentumEdgeSolverAlg.C:70-313) + sum_into_row_vec_3
 * (src/TpetraLinearSystem.C:1293-1335). num_dof must be 3. */
nw_status nw_assemble_momentum_edges(nw_linsys* ls,
                                     const nw_momentum_fields* f,
                                     const nw_momentum_opts* o);
/* The same assembly in two parts, for callers that stream the edge inputs
 * in while earlier edges assemble (the reference walks its edge buckets one
 * by one, AssembleEdgeSolverAlgorithm::execute): the edge phase over edges
 * [edge_begin, edge_end) of the graph's edge list (it reads area, mdot and
 * pecfac of those edges only, and every node field), then, once every edge
 * has been covered exactly once, the row phase, which adds the result into
 * the CSR values and rhs. Both are ordered on the handle's stream; the sum
 * equals nw_assemble_momentum_edges bit for bit. */
nw_status nw_assemble_momentum_edge_range(nw_linsys* ls, const nw_momentum_fields* f,
                                          const nw_momentum_opts* o, int64_t edge_begin,
                                          int64_t edge_end);
nw_status nw_assemble_momentum_rows(nw_linsys* ls, const nw_momentum_opts* o);
/* The row phase over node rows [row_begin, row_end) only, so that it can
 * run as soon as every edge incident to those rows has been through the
 * edge phase (with edges ordered by their first node, the rows below a
 * chunk's last first node are then complete). On a system zeroed by
 * nw_linsys_zero the ranges must follow each other from row 0 (each
 * overwrites its rows; the system counts as assembled once the last row is
 * covered, and an operation in between zeroes the rows not yet covered);
 * otherwise each range adds into its rows. The rows of all ranges together
 * equal nw_assemble_momentum_rows bit for bit. */
nw_status nw_assemble_momentum_rows_range(nw_linsys* ls, const nw_momentum_opts* o,
                                          int64_t row_begin, int64_t row_end);

/* How nw_assemble_momentum_edges runs on the GPU. TWO_KERNELS (default):
 * the edge kernel writes every edge's coefficients to a buffer in HBM, then
 * the row kernel reads them back. SINGLE_KERNEL: one persistent kernel takes
 * edge chunks and node-row blocks from a fixed work list; the coefficients
 * pass through a ring of slots sized to stay in L2 (at most 64 MB), so they
 * never travel to DRAM (about 1.1x the compulsory bytes instead of 1.6x),
 * but on GB300 it runs slower than the two kernels (both phases are bound by
 * instruction issue, not by HBM). Both give the same CSR values and rhs, bit
 * for bit. A wait of the single kernel that times out (it cannot, by the
 * construction of the work list, but every wait is bounded) is reported as
 * NW_TIMEOUT by the next nw_linsys_sync, nw_linsys_copy_to_host or
 * nw_linsys_solve. */
enum { NW_ASSEMBLY_SINGLE_KERNEL = 0, NW_ASSEMBLY_TWO_KERNELS = 1 };
nw_status nw_linsys_set_assembly_path(nw_linsys* ls, int path);
typedef struct {
  int single_kernel;     /* 1: the single-kernel path is set up */
  int grid;              /* resident blocks it launches */
  int chunk_edges;       /* edges per edge chunk */
  int block_rows;        /* node rows per row block */
  int64_t edge_chunks, row_blocks;
  int64_t ring_chunks;   /* ring slots; >= edge_chunks: no reuse */
  int64_t ring_bytes;    /* 0 when the ring is the whole coefficient buffer */
  int64_t lag_chunks;    /* chunks between a row block's last input and it */
} nw_assembly_schedule;
nw_status nw_linsys_assembly_schedule(const nw_linsys* ls, nw_assembly_schedule* info);
/* The work list of the single-kernel assembly for a graph given by its edge
 * list (host only, no GPU: for inspection and tests). edge_rows: E pairs of
 * node rows (0 .. rows-1); concurrency: resident blocks; max_ring_bytes:
 * the ring's limit. Sizes go to info (grid = concurrency); with non-null
 * arrays also: items (edge_chunks + row_blocks entries, 2 c for edge chunk
 * c, 2 k + 1 for row block k, in ticket order), chunk_lo / chunk_hi
 * (row_blocks entries: the chunks a block reads) and block_lo / block_hi
 * (edge_chunks entries: the blocks reading a chunk). */
nw_status nw_momentum_schedule(int64_t rows, int64_t num_edges, const int64_t* edge_rows,
                               int64_t concurrency, int64_t max_ring_bytes,
                               nw_assembly_schedule* info, int32_t* items,
                               int32_t* chunk_lo, int32_t* chunk_hi, int32_t* block_lo,
                               int32_t* block_hi);

/* LinearSystem::sumInto, host-vector overload (include/LinearSystem.h:
 * 167-173): one entity block. nodes (host, n_ent) are node indices; rhs
 * (host, n_ent*num_dof) and lhs (host, row-major square of that size). */
nw_status nw_linsys_sum_into(nw_linsys* ls, int n_ent, const int64_t* nodes,
                             const double* rhs, const double* lhs);

/* applyDirichletBCs (src/TpetraLinearSystem.C:1686-1757): for each node in
 * nodes (device, n), dof rows [begin, end) become identity rows and the rhs
 * becomes bc - q. q and bc are device node fields (N x num_dof). */
nw_status nw_linsys_apply_dirichlet(nw_linsys* ls, int64_t n,
                                    const int64_t* nodes, int begin, int end,
                                    const double* q, const double* bc);
/* resetRows (src/TpetraLinearSystem.C:1759-1786). nodes: device. */
nw_status nw_linsys_reset_rows(nw_linsys* ls, int64_t n, const int64_t* nodes,
                               int begin, int end, double diag_value,
                               double rhs_residual);
/* loadComplete (src/TpetraLinearSystem.C:1788-1809): on one GPU there are
 * no shared-not-owned rows; this only orders the stream. */
nw_status nw_linsys_load_complete(nw_linsys* ls);

/* Device views of the assembled system (owned by the handle). */
nw_status nw_linsys_device_arrays(nw_linsys* ls, double** values,
                                  double** rhs, const int64_t** row_ptr,
                                  const int32_t** col_idx);
/* Copy values (nnz) and rhs (nrows) to host arrays (either may be NULL). */
nw_status nw_linsys_copy_to_host(nw_linsys* ls, double* values, double* rhs);
/* Overwrite values / rhs from host arrays (either may be NULL). */
nw_status nw_linsys_copy_from_host(nw_linsys* ls, const double* values,
                                   const double* rhs);

/* ---- solve: LinearSystem::solve (src/TpetraLinearSystem.C:1811-1881) ->
 * TpetraLinearSolver::solve (src/LinearSolver.C:209-254). x (device, nrows)
 * receives the solution from x0 = 0; final_iter selects final_tolerance.
 * Returns when the solve is done (the report needs its results). The mixed
 * methods launch their inner iterations as CUDA graphs captured on the
 * handle's stream; on the legacy default stream, which cannot be captured,
 * the solve runs on a stream of the handle's own, ordered after earlier
 * work on the caller's stream and before later work by events. */
nw_status nw_linsys_solve(nw_linsys* ls, double* x, int final_iter,
                          nw_solve_report* rep);
/* Residual history of the last solve (relative, first entry 1). */
nw_status nw_linsys_residual_history(const nw_linsys* ls, double* hist,
                                     int capacity, int* count);
/* copy_tpetra_to_stk (src/TpetraLinearSystem.C:2183-2227): scatter a row
 * vector (device, nrows) to a node field (device, N x num_dof); periodic
 * slaves receive their master's value. */
nw_status nw_linsys_rows_to_nodes(nw_linsys* ls, const double* x_rows,
                                  double* x_nodes);

/* ---- plain kernels on the assembled system (device vectors) ---- */
nw_status nw_linsys_spmv(nw_linsys* ls, const double* x, double* y);
nw_status nw_linsys_precond_apply(nw_linsys* ls, int preconditioner,
                                  const double* x, double* y);
/* Row order used by the multicolour SGS (host, nrows): rows of colour 0 in
 * ascending order, then colour 1, ... */
nw_status nw_linsys_sgs_order(nw_linsys* ls, int64_t* order, int* ncolors);
/* Boundaries of the colour classes in that order (host, ncolors + 1): class
 * c is order[class_ptr[c] .. class_ptr[c + 1]). Ifpack2's MT-SGS has the
 * same notion (a colour set per sweep); there is no single reference call
 * to cite. */
nw_status nw_linsys_sgs_classes(nw_linsys* ls, int64_t* class_ptr);

/* ---- learned preconditioner (NW_PC_LEARNED). No counterpart in the
 * reference: nalu-wind's preconditioners are Ifpack2 relaxations and MueLu
 * (src/LinearSolverConfig.C:89-121). M(v) = z2 + SGS(v - A z2),
 * z2 = z1 + alpha P Net(R (v - A z1)), z1 = SGS(v): one multicolour SGS
 * sweep, a coarse correction over plain aggregates (R sums, P copies) by a
 * 4-layer, 64-channel edge message-passing network (BF16, FP32
 * accumulation) scaled by its energy-optimal factor alpha, and a second
 * SGS sweep. Applied inside FGMRES; the solve is repeated with SGS when the
 * flexible solve fails or stalls. ---- */
typedef struct nw_learned nw_learned;
/* Network with seeded random weights (device resident). */
nw_status nw_learned_create(uint64_t seed, nw_learned** out);
nw_status nw_learned_destroy(nw_learned* net);
/* Weight file: magic, shapes, Adam step, FP32 weights, FNV-1a checksum. */
nw_status nw_learned_save(nw_learned* net, const char* path);
nw_status nw_learned_load(nw_learned* net, const char* path);
/* Host copy of the flat FP32 parameters (get when out != NULL, then set
 * when in != NULL). n must equal nw_learned_num_params(). */
int64_t nw_learned_num_params(void);
nw_status nw_learned_params(nw_learned* net, float* out, const float* in,
                            int64_t n);
/* post_smooth 1 (default): M(v) ends with a second SGS sweep on
 * v - A z (symmetric two-level cycle); 0: no post-smoothing.
 * agg_passes (1..4, default 2): plain aggregation applied that many times
 * (aggregates of aggregates) to build the coarse level; takes effect at
 * the next nw_linsys_attach_learned. smoother 0 (default): symmetric GS
 * sweeps before and after the coarse step; 1: a forward sweep before and
 * a backward sweep after (half the smoothing work, still symmetric). */
nw_status nw_learned_configure(nw_learned* net, int post_smooth, int agg_passes, int smoother);
/* Build the aggregation / coarse level of this system's graph (num_dof 1)
 * and use `net` for NW_PC_LEARNED solves of this handle. */
/* Coarse direction of the two-level cycle: 0 (default) the network; 1 the
 * Jacobi direction D_c^-1 r_c and 2 two Jacobi sweeps on the Galerkin coarse
 * operator, each with the same energy-optimal scaling. Modes 1 and 2 are
 * the cycle without the network, kept to measure what the network adds. */
nw_status nw_learned_set_coarse_direction(nw_learned* net, int mode);
/* Aggregation of the coarse level: 0 (default) plain aggregation of the
 * matrix graph; strength in (0, 1): aggregation over strong connections
 * (|a_ij| >= strength sqrt(|a_ii a_jj|)), each pass on the Galerkin values
 * of the previous one, so that aggregates follow the dominant couplings
 * of stretched cells. Takes effect at nw_linsys_attach_learned, which then
 * reads the assembled values. */
nw_status nw_learned_set_aggregation(nw_learned* net, double strength);
nw_status nw_linsys_attach_learned(nw_linsys* ls, nw_learned* net);
/* Coarse level of an attached handle, refreshed from the current values
 * (host arrays; NULL entries skipped). */
nw_status nw_linsys_coarse_sizes(nw_linsys* ls, int64_t* nc, int64_t* nnzc);
nw_status nw_linsys_coarse_graph(nw_linsys* ls, int32_t* agg, int64_t* cptr,
                                 int32_t* ccol, float* wgt, float* dinv);
/* Harvest (residual, error) pairs from the handle's assembled system:
 * x* from a tight (1e-11) FP64 CG + SGS solve (at most 40,000 iterations),
 * or, when that fails outright (above 1e-3 or non-finite), the better of it
 * and SGS-GMRES(50) (mixed precision, then FP64; at most 5,000 iterations
 * each), then
 * `restarts` cycles of plain FP64 Jacobi-GMRES(kspace) from x0 = 0, one
 * pair per restart while the restart's residual is at least 100 times
 * that of x* (the error target is then accurate to 1 %); NW_NOT_CONVERGED
 * when x* itself is not below 1e-6 relative. Stored on the device as the
 * coarse residual R (r - A z1) with the energy norms ||e||_A^2 and
 * ||e - z1||_A^2 of the error e = x* - x. */
nw_status nw_learned_harvest(nw_learned* net, nw_linsys* ls, int restarts,
                             int kspace, int* total_pairs);
nw_status nw_learned_clear_data(nw_learned* net);
/* Adam training over the harvested pairs (`epochs` passes), on the graph
 * of `ls`; loss = ||z1 + P e_c - e||_A^2 / ||e||_A^2 (the A-norm error
 * left after the smoothing sweep and the coarse correction), mean over
 * the last epoch in *loss. */
nw_status nw_learned_train(nw_learned* net, nw_linsys* ls, int epochs,
                           int batch, double lr, uint64_t shuffle_seed,
                           double* loss);
/* Mean loss over the harvested pairs, parameters unchanged. */
nw_status nw_learned_evaluate(nw_learned* net, nw_linsys* ls, double* loss);
/* One pair through forward and backward on the coarse level of `ls`
 * (device rc of length nc, ea = ||e||_A^2, ca = ||e - z1||_A^2): the loss
 * (e_c' Ac e_c - 2 e_c' rc + ca) / ea and its parameter gradient (host). */
nw_status nw_learned_loss_grad(nw_learned* net, nw_linsys* ls, const float* rc,
                               double ea, double ca, double* loss, float* grad);
/* Coarse correction ec = Net(rc) (device vectors of length nc). */
nw_status nw_learned_forward(nw_learned* net, nw_linsys* ls, const float* rc,
                             float* ec);
/* The network's BF16 tensor-core GEMMs on device buffers (testing):
 * kind 0: out_bf16[m x 64] = relu(a_bf16[m x 128] b), b given transposed
 *         (64 x 128); kind 1: out_f32[m x 128] = a_bf16[m x 64] b^T, b
 *         row-major 128 x 64; kind 2: out_f32[128 x 64] = a_bf16[m x 128]^T
 *         b_bf16[m x 64]; kind 3: kind 0 on the tcgen05 tensor cores (TMEM
 *         accumulator), NW_TIMEOUT if one of its bounded waits gave up;
 *         kind 4: kind 3 with the tiles loaded by TMA (cp.async.bulk.tensor,
 *         128-byte swizzle); kind 5: kind 1 on the tcgen05 tensor cores
 *         (TMA tiles); kind 6: kind 2 on the tcgen05 tensor cores (node
 *         chunks transposed while staged). The training step uses kinds 4,
 *         5 and 6. */
nw_status nw_gemm_bf16(int kind, int64_t m, const void* a, const void* b,
                       void* out);

/* ---- input producers of the assembly (run before it every nonlinear
 * iteration). Edge outputs are in the order given to
 * nw_linsys_build_edge_graph; node inputs/outputs are indexed by the
 * caller's nodes. All pointers are device pointers. ---- */

/* MdotEdgeAlg::execute (src/ngp_algorithms/MdotEdgeAlg.C:117-190): mass
 * flow rate per edge (E) from the continuity fields; no balanced-buoyancy
 * forcing and no GCL term (as in nw_assemble_continuity_edges). */
nw_status nw_compute_mdot_edges(nw_linsys* ls, const nw_continuity_fields* f,
                                double noc_fac, double interp_together,
                                double* mdot);
/* NodalGradEdgeAlg::execute (src/ngp_algorithms/NodalGradEdgeAlg.C:85-109):
 * edge-based Green-Gauss gradient of phi (N x dim1, dim1 = 1 or 3) into
 * grad (N x dim1*3, component i, direction j at 3i + j). bnd_area (N x 3,
 * or NULL) adds the lumped exposed-face closure bnd_area * phi (the role of
 * NodalGradBndryElemAlg); periodic masters and slaves receive the summed
 * value, divided by dualvol (already summed over periodic pairs). */
nw_status nw_compute_nodal_gradient(nw_linsys* ls, int dim1, const double* phi,
                                    const double* area, const double* dualvol,
                                    const double* bnd_area, double* grad);
/* Peclet blending function (EquationSystem::ngp_create_peclet_function,
 * include/EquationSystem.h:399-413; src/PecletFunction.C:39-71). */
typedef struct nw_peclet_opts {
  int tanh_form;        /* 0 classic (hf Pe)^2 / (5 + (hf Pe)^2), 1 tanh */
  double hybrid_factor; /* hf of the classic form */
  double tanh_trans;    /* c1 of the tanh form */
  double tanh_width;    /* c2 of the tanh form */
  double eps;           /* 1e-16 in MomentumEdgePecletAlg */
} nw_peclet_opts;
/* MomentumEdgePecletAlg::execute (src/edge_kernels/MomentumEdgePecletAlg.C:
 * 74-101): Peclet number (pecnum, optional) and factor per edge. */
nw_status nw_compute_peclet_factor(nw_linsys* ls, const double* coords,
                                   const double* density, const double* viscosity,
                                   const double* velocity, const nw_peclet_opts* o,
                                   double* pecnum, double* pecfac);

/* Edge area vectors and dual nodal volumes on the device
 * (GeometryInteriorAlg::impl_compute_edge_area_vector and
 * impl_compute_dual_nodal_volume, src/ngp_algorithms/GeometryInteriorAlg.C:
 * 70-225, with the Hex8 / Tet4 sub-control surfaces and volumes of
 * src/master_element/Hex8CVFEM.C:361-405,565-591 and Tet4CVFEM.C), for
 * meshes whose coordinates change. nw_geometry_create takes the host
 * element connectivity (num_elems x nodes_per_elem, 8 = Hex8 in Exodus
 * order, 4 = Tet4), the edge list (num_edges x 2, the order of the area
 * output; every element edge must be in it) and optionally nalu_id
 * (1-based periodic master id per node: masters and slaves receive the
 * summed volume); it builds the element -> edge and element -> node
 * incidences once. nw_geometry_compute then evaluates, from device
 * coordinates (N x 3), area (E x 3) and dualvol (N) on the given stream
 * (NULL: the default stream), with no atomics: the area vectors of an edge
 * and the volumes of a node are summed in element order, so the results
 * equal nw_mesh_get's host values bit for bit. */
typedef struct nw_geometry nw_geometry;
nw_status nw_geometry_create(int64_t num_nodes, int nodes_per_elem, int64_t num_elems,
                             const int64_t* conn, int64_t num_edges, const int64_t* edge_nodes,
                             const int64_t* nalu_id, nw_geometry** out);
nw_status nw_geometry_compute(nw_geometry* g, const double* coords, double* area,
                              double* dualvol, void* stream);
nw_status nw_geometry_destroy(nw_geometry* g);

/* ---- node kernels: lumped-mass BDF time terms, added into the system
 * (like sumInto) after the edge assembly. States Nm1, N, Np1; device
 * pointers of the caller's nodes. The edge graph has no entry at all in
 * the row of a node that is in no edge; the scalar and momentum kernels
 * then return NW_INVALID_ARG (their diagonal term has nowhere to go). ---- */
typedef struct nw_mass_bdf_fields {
  const double* density_nm1;     /* N */
  const double* density_n;       /* N */
  const double* density_np1;     /* N */
  const double* dual_volume_nm1; /* N (dual_nodal_volume states) */
  const double* dual_volume_n;   /* N */
  const double* dual_volume_np1; /* N */
  const double* q_nm1;           /* scalar: N; momentum: velocity N x 3 */
  const double* q_n;
  const double* q_np1;
  const double* dpdx;            /* momentum: N x 3 */
} nw_mass_bdf_fields;
typedef struct nw_bdf_opts {
  double dt;     /* Realm::get_time_step */
  double gamma1; /* BDF coefficients (Realm::get_gamma1..3) */
  double gamma2;
  double gamma3;
} nw_bdf_opts;
/* ScalarMassBDFNodeKernel::execute (src/node_kernels/ScalarMassBDFNodeKernel.C:
 * 75-97): diag += g1 rho dnv / dt; rhs -= (g1 rho q dnv |Np1 + g2 .. |N +
 * g3 .. |Nm1) / dt. num_dof 1. */
nw_status nw_assemble_scalar_mass_bdf(nw_linsys* ls, const nw_mass_bdf_fields* f,
                                      const nw_bdf_opts* o);
/* ContinuityMassBDFNodeKernel::execute (src/node_kernels/
 * ContinuityMassBDFNodeKernel.C:60-82): rhs only. num_dof 1. */
nw_status nw_assemble_continuity_mass_bdf(nw_linsys* ls, const nw_mass_bdf_fields* f,
                                          const nw_bdf_opts* o);
/* MomentumMassBDFNodeKernel::execute (src/node_kernels/
 * MomentumMassBDFNodeKernel.C:78-107): per component, plus -dpdx dnv on the
 * rhs. num_dof 3. */
nw_status nw_assemble_momentum_mass_bdf(nw_linsys* ls, const nw_mass_bdf_fields* f,
                                        const nw_bdf_opts* o);

/* ---- boundary face kernels (edge-based open / symmetry conditions) ----
 * The reference assembles these through AssembleFaceElemSolverAlgorithm
 * (src/AssembleFaceElemSolverAlgorithm.C) with the face-element kernels of
 * src/edge_kernels/ (ContinuityOpenEdgeKernel, MomentumOpenEdgeKernel,
 * MomentumSymmetryEdgeKernel, ScalarOpenEdgeKernel), each adding through
 * sumInto. Here a side set is registered once as its face integration
 * points: per IP the face node R (ipNodeMap[ip] / side_node_ordinals) and
 * the element node L opposite it (MasterElement::opposingNodes). Every IP
 * adds to the rows of R only, at columns R and L. The kernels run one thread
 * per boundary node row over that row's IPs in IP order (no atomics) and
 * ADD to the values and rhs already in the handle: call them after the
 * interior edge assembly. Face-IP fields (exposed_area_vector, open mass
 * flow rate, dynamic pressure) are indexed by IP in registration order;
 * node fields by the caller's node index. */
typedef struct nw_sideset nw_sideset;
/* ip_nodes: host, num_ips x 2 (face node, opposing node). The handle must be
 * finalized and outlive the side set. NW_INVALID_ARG when a node index is
 * out of range or a pair is not joined by a graph edge. */
nw_status nw_sideset_create(nw_linsys* ls, int64_t num_ips, const int64_t* ip_nodes,
                            nw_sideset** out);
nw_status nw_sideset_destroy(nw_sideset* s);
/* number of IPs and of distinct boundary node rows */
nw_status nw_sideset_sizes(const nw_sideset* s, int64_t* num_ips, int64_t* num_rows);

typedef struct nw_continuity_open_fields {
  const double* coords;           /* N x 3 */
  const double* velocity;         /* N x 3 (velocity_rtm on moving meshes) */
  const double* dpdx;             /* N x 3 */
  const double* density;          /* N */
  const double* pressure;         /* N */
  const double* pressure_bc;      /* N; the pressure itself with the open mdot correction */
  const double* udiag;            /* N (momentum_diag) */
  const double* exposed_area;     /* num_ips x 3 */
  const double* dynamic_pressure; /* num_ips, or NULL for zero */
} nw_continuity_open_fields;
typedef struct nw_continuity_open_opts {
  double tau_scale;            /* dt / gamma1 */
  double noc_fac;              /* get_noc_usage("pressure") */
  double pstab_fac;            /* 1; 0 with activateOpenMdotCorrection_ */
  double mdot_corr;            /* mdotAlgOpenCorrection_ with the correction, else 0 */
  double solve_incompressible; /* solveIncompressibleContinuity_ ? 1 : 0 */
} nw_continuity_open_opts;
/* ContinuityOpenEdgeKernel::execute (src/edge_kernels/
 * ContinuityOpenEdgeKernel.C:92-160). num_dof 1. */
nw_status nw_assemble_continuity_open(nw_linsys* ls, const nw_sideset* s,
                                      const nw_continuity_open_fields* f,
                                      const nw_continuity_open_opts* o);

#define NW_ENTRAIN_COMPUTED 0
#define NW_ENTRAIN_SPECIFIED 1
typedef struct nw_momentum_open_fields {
  const double* coords;              /* N x 3 */
  const double* velocity;            /* N x 3 (state np1) */
  const double* dudx;                /* N x 9 */
  const double* viscosity;           /* N */
  const double* velocity_bc;         /* N x 3 (open_velocity_bc) */
  const double* exposed_area;        /* num_ips x 3 */
  const double* open_mass_flow_rate; /* num_ips */
} nw_momentum_open_fields;
typedef struct nw_momentum_open_opts {
  double include_div_u; /* includeDivU_ */
  double nf_entrain;    /* nearestFaceEntrain_ */
  int entrainment;      /* NW_ENTRAIN_COMPUTED or NW_ENTRAIN_SPECIFIED */
} nw_momentum_open_opts;
/* MomentumOpenEdgeKernel::execute (src/edge_kernels/
 * MomentumOpenEdgeKernel.C:80-270). num_dof 3. */
nw_status nw_assemble_momentum_open(nw_linsys* ls, const nw_sideset* s,
                                    const nw_momentum_open_fields* f,
                                    const nw_momentum_open_opts* o);

typedef struct nw_momentum_symmetry_fields {
  const double* coords;       /* N x 3 */
  const double* velocity;     /* N x 3 (state np1) */
  const double* dudx;         /* N x 9 */
  const double* viscosity;    /* N */
  const double* exposed_area; /* num_ips x 3 */
} nw_momentum_symmetry_fields;
typedef struct nw_momentum_symmetry_opts {
  double include_div_u;  /* includeDivU_ */
  double penalty_factor; /* symmetryBcPenaltyFactor_ */
} nw_momentum_symmetry_opts;
/* MomentumSymmetryEdgeKernel::execute (src/edge_kernels/
 * MomentumSymmetryEdgeKernel.C:64-206). num_dof 3. */
nw_status nw_assemble_momentum_symmetry(nw_linsys* ls, const nw_sideset* s,
                                        const nw_momentum_symmetry_fields* f,
                                        const nw_momentum_symmetry_opts* o);

typedef struct nw_abl_wall_fields {
  const double* velocity;               /* N x 3 (state np1) */
  const double* wall_velocity_bc;       /* N x 3 */
  const double* density;                /* N */
  const double* heat_flux_bc;           /* N */
  const double* specific_heat;          /* N */
  const double* exposed_area;           /* num_ips x 3 */
  const double* wall_friction_velocity; /* num_ips (wall_friction_velocity_bip) */
  const double* wall_normal_distance;   /* num_ips (wall_normal_distance_bip) */
} nw_abl_wall_fields;
typedef struct nw_abl_wall_opts {
  double gravity; /* m/s^2 */
  double z0;      /* roughness height */
  double Tref;    /* reference temperature */
  double kappa;   /* von Karman constant (0.41) */
  double beta_m;  /* stable Monin-Obukhov coefficient (5) */
  double gamma_m; /* unstable Monin-Obukhov coefficient (16) */
} nw_abl_wall_opts;
/* MomentumABLWallFuncEdgeKernel::execute (src/edge_kernels/
 * MomentumABLWallFuncEdgeKernel.C:80-158) with the Monin-Obukhov functions
 * of include/wind_energy/MoninObukhov.h: the wall shear on the tangential
 * velocity of each face node (its rows and columns only). num_dof 3. */
nw_status nw_assemble_momentum_abl_wall(nw_linsys* ls, const nw_sideset* s,
                                        const nw_abl_wall_fields* f, const nw_abl_wall_opts* o);

/* MomentumABLWallShearStressEdgeKernel::execute (src/edge_kernels/
 * MomentumABLWallShearStressEdgeKernel.C:49-88): rhs += wall_shear_stress
 * (num_ips x 3) times |exposed_area| on the rows of the face node (slip != 0)
 * or of the opposing node (slip == 0). num_dof 3. */
nw_status nw_assemble_momentum_abl_wall_shear_stress(nw_linsys* ls, const nw_sideset* s,
                                                     const double* exposed_area,
                                                     const double* wall_shear_stress, int slip);

typedef struct nw_scalar_open_fields {
  const double* q;                   /* N (state np1) */
  const double* q_bc;                /* N (entrained value) */
  const double* open_mass_flow_rate; /* num_ips */
} nw_scalar_open_fields;
/* ScalarOpenEdgeKernel::execute (src/edge_kernels/ScalarOpenEdgeKernel.C:
 * 49-72) = ScalarEdgeOpenSolverAlg::execute (ScalarEdgeOpenSolverAlg.C:
 * 64-104): upwind outflow, entrainment at q_bc; relax = the equation's
 * relaxation factor. num_dof 1. */
nw_status nw_assemble_scalar_open(nw_linsys* ls, const nw_sideset* s,
                                  const nw_scalar_open_fields* f, double relax);

/* MdotOpenEdgeAlg::execute (src/ngp_algorithms/MdotOpenEdgeAlg.C:55-150):
 * the open_mass_flow_rate of every face IP into mdot (device, num_ips, IP
 * order) from the same fields as the continuity open kernel
 * (dynamic_pressure may be NULL), with noc_fac = get_noc_usage("pressure")
 * and pstab_fac = 0 with activateOpenMdotCorrection_ else 1; *total (host,
 * may be NULL) gets the sum over the IPs in a fixed order (the value
 * MdotAlgDriver::add_open_mdot receives). */
nw_status nw_compute_open_mdot(nw_linsys* ls, const nw_sideset* s,
                               const nw_continuity_open_fields* f, double noc_fac,
                               double pstab_fac, double* mdot, double* total);
/* MdotOpenCorrectorAlg::execute (src/ngp_algorithms/MdotOpenCorrectorAlg.C:
 * 37-60): mdot -= correction on every IP of the side set; *total gets the
 * corrected sum (MdotAlgDriver's mdot_open_post). The correction itself is
 * (density accumulation + inflow + open) / (open IP count)
 * (src/ngp_algorithms/MdotAlgDriver.C:145-146), computed by the caller. */
nw_status nw_correct_open_mdot(nw_linsys* ls, const nw_sideset* s, double correction,
                               double* mdot, double* total);

/* ---- momentum_diag (the Udiag time scale of the pressure projection) ---- */
/* NGPApplyCoeff::extract_diagonal (src/SolverAlgorithm.C:89-104), enabled
 * by MomentumEquationSystem::assemble_and_solve when tscaleType is
 * TSCALE_UDIAGINV (src/LowMachEquationSystem.C:2729-2760): every local
 * system's lhs(ix, ix) (first dof of each node) summed per node. Here it is
 * read from the assembled matrix: diag (device, one value per caller node;
 * periodic slaves get their master's) = the diagonal entry of dof `dof` of
 * the node's row, which holds the sum of every kernel assembled so far.
 * Call after the assembly and before nw_linsys_apply_dirichlet. */
nw_status nw_linsys_extract_diagonal(nw_linsys* ls, int dof, double* diag);
/* The post-processing that follows the momentum solve (src/
 * LowMachEquationSystem.C:2760-2790): udiag = (udiag / (rho V) - gamma1/dt)
 * relax + gamma1/dt, per node (device arrays of the handle's node count,
 * relax = the velocity relaxation factor). */
nw_status nw_udiag_postprocess(nw_linsys* ls, const double* density, const double* dual_volume,
                               double dt, double gamma1, double relax, double* udiag);

/* ---- checkpoint / resume (raw binary; the reference restarts through
 * Exodus/STK I/O, src/OutputInfo.C:163-181, and dumps matrices with
 * writeToFile, src/TpetraLinearSystem.C:2017-2102). save writes the graph
 * (row_ptr, col_idx), values, rhs, the solver configuration, the last
 * solve's report and residual history and, when x (device, nrows) is not
 * NULL, that vector; the file carries an FNV-1a checksum. load restores
 * values, rhs, configuration, report and history into a finalized handle
 * with the same graph (NW_INVALID_ARG on a different graph, a truncated or
 * corrupted file), and x when not NULL; rep (optional) receives the saved
 * report. ---- */
nw_status nw_linsys_checkpoint_save(nw_linsys* ls, const char* path, const double* x);
nw_status nw_linsys_checkpoint_load(nw_linsys* ls, const char* path, double* x,
                                    nw_solve_report* rep);

/* ---- MatrixMarket export / import ---- */
/* TpetraLinearSystem::writeToFile (src/TpetraLinearSystem.C:2017-2045):
 * writes <base>-O-<count>.mm.1 (coordinate real general, 1-based global dof
 * ids ndof (nalu id - 1) + d + 1) and <base>-O-<count>.rhs.1 (array real
 * general); with x_host (nrows, row order) also <base>-O-<count>.sln.1.
 * Values are written with 17 significant digits (round trip exact). */
nw_status nw_linsys_write_matrix_market(nw_linsys* ls, const char* base, int count,
                                        const double* x_host);
/* Reads such files back into this handle's graph (values and, when
 * rhs_path is not NULL, the rhs). No reference counterpart: it lets a
 * system exported elsewhere be solved here. */
nw_status nw_linsys_read_matrix_market(nw_linsys* ls, const char* matrix_path,
                                       const char* rhs_path);

/* ---- timing helpers (CUDA events on the handle's stream) ---- */
nw_status nw_linsys_sync(nw_linsys* ls);
/* Milliseconds of the last assembly call (edge + row phases). */
nw_status nw_linsys_last_assembly_ms(const nw_linsys* ls, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* NW_CAPI_H */
