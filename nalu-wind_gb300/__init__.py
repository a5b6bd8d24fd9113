"""Python bindings (ctypes) for libnw_gb300.so.

The library is the product: a C ABI (include/nw_capi.h, include/nw_workload.h)
over hand-written sm_103a kernels. This module only loads it and mirrors the
reference's LinearSystem / LinearSolver surface (include/LinearSystem.h,
src/LinearSolver.C) for tests and benchmarks. Device buffers are passed as
integer device pointers (e.g. torch.Tensor.data_ptr()). There is no CPU
fallback: every call fails loudly when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libnw_gb300.so"

# status codes (nw_status)
NW_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "CUDA_ERROR", 3: "NOT_FINALIZED", 4: "NAN_DETECTED",
                5: "NOT_CONVERGED", 6: "BREAKDOWN", 7: "TIMEOUT", 8: "NO_DEVICE", 9: "INTERNAL"}
GMRES, CG, FGMRES, BICGSTAB, TFQMR, SSTEP_GMRES = 0, 1, 2, 3, 4, 5
PC_NONE, PC_JACOBI, PC_SGS, PC_LEARNED, PC_SGS2, PC_SGS_NATURAL, PC_RILUK = 0, 1, 2, 3, 4, 5, 6
PC_MT_SGS = PC_SGS  # "mt_sgs": multicolour order
PREC_FP64, PREC_MIXED, PREC_MIXED_BF16 = 0, 1, 2
ASSEMBLY_SINGLE_KERNEL, ASSEMBLY_TWO_KERNELS = 0, 1


class NwError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class SolverCfg(C.Structure):
    _fields_ = [("method", C.c_int), ("preconditioner", C.c_int), ("precision", C.c_int),
                ("kspace", C.c_int), ("max_iterations", C.c_int), ("tolerance", C.c_double),
                ("final_tolerance", C.c_double), ("inner_kspace", C.c_int),
                ("inner_tolerance", C.c_double), ("sgs2_inner_sweeps", C.c_int), ("sstep_size", C.c_int)]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer_iterations", C.c_int), ("status", C.c_int),
                ("converged", C.c_int), ("final_rel_residual", C.c_double),
                ("final_abs_residual", C.c_double), ("rhs_norm", C.c_double),
                ("solve_ms", C.c_double), ("fallback", C.c_int)]


class ScalarOpts(C.Structure):
    _fields_ = [("alpha", C.c_double), ("alpha_upw", C.c_double), ("upw_factor", C.c_double),
                ("relax", C.c_double), ("hybrid_factor", C.c_double), ("use_limiter", C.c_int),
                ("tanh_form", C.c_int), ("tanh_trans", C.c_double), ("tanh_width", C.c_double)]


class MomentumOpts(C.Structure):
    _fields_ = [("alpha", C.c_double), ("alpha_upw", C.c_double), ("upw_factor", C.c_double),
                ("relax", C.c_double), ("include_div_u", C.c_double), ("use_limiter", C.c_int)]


class ContinuityOpts(C.Structure):
    _fields_ = [("noc_fac", C.c_double), ("tau_scale", C.c_double),
                ("interp_together", C.c_double), ("solve_incompressible", C.c_double)]


class MassBdfFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("density_nm1", "density_n", "density_np1", "dual_volume_nm1",
                                           "dual_volume_n", "dual_volume_np1", "q_nm1", "q_n", "q_np1", "dpdx")]


class BdfOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("gamma1", C.c_double), ("gamma2", C.c_double), ("gamma3", C.c_double)]


class PecletOpts(C.Structure):
    _fields_ = [("tanh_form", C.c_int), ("hybrid_factor", C.c_double), ("tanh_trans", C.c_double),
                ("tanh_width", C.c_double), ("eps", C.c_double)]


class ContinuityOpenFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("coords", "velocity", "dpdx", "density", "pressure", "pressure_bc",
                                           "udiag", "exposed_area", "dynamic_pressure")]


class ContinuityOpenOpts(C.Structure):
    _fields_ = [("tau_scale", C.c_double), ("noc_fac", C.c_double), ("pstab_fac", C.c_double),
                ("mdot_corr", C.c_double), ("solve_incompressible", C.c_double)]


class MomentumOpenFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("coords", "velocity", "dudx", "viscosity", "velocity_bc",
                                           "exposed_area", "open_mass_flow_rate")]


ENTRAIN_COMPUTED, ENTRAIN_SPECIFIED = 0, 1


class MomentumOpenOpts(C.Structure):
    _fields_ = [("include_div_u", C.c_double), ("nf_entrain", C.c_double), ("entrainment", C.c_int)]


class MomentumSymmetryFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("coords", "velocity", "dudx", "viscosity", "exposed_area")]


class MomentumSymmetryOpts(C.Structure):
    _fields_ = [("include_div_u", C.c_double), ("penalty_factor", C.c_double)]


class AblWallFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("velocity", "wall_velocity_bc", "density", "heat_flux_bc",
                                           "specific_heat", "exposed_area", "wall_friction_velocity",
                                           "wall_normal_distance")]


class AblWallOpts(C.Structure):
    _fields_ = [("gravity", C.c_double), ("z0", C.c_double), ("Tref", C.c_double), ("kappa", C.c_double),
                ("beta_m", C.c_double), ("gamma_m", C.c_double)]


class ScalarOpenFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("q", "q_bc", "open_mass_flow_rate")]


_P = C.c_void_p


class ScalarFields(C.Structure):
    _fields_ = [(n, _P) for n in ("coords", "velocity_rtm", "q", "dqdx", "density", "diff_coeff",
                                  "area", "mdot")]


class ContinuityFields(C.Structure):
    _fields_ = [(n, _P) for n in ("coords", "velocity", "dpdx", "density", "pressure", "udiag", "area")]


class MomentumFields(C.Structure):
    _fields_ = [(n, _P) for n in ("coords", "velocity", "dudx", "viscosity", "density", "mask",
                                  "area", "mdot", "pecfac")]


class AssemblySchedule(C.Structure):
    _fields_ = [("single_kernel", C.c_int), ("grid", C.c_int), ("chunk_edges", C.c_int),
                ("block_rows", C.c_int), ("edge_chunks", C.c_int64), ("row_blocks", C.c_int64),
                ("ring_chunks", C.c_int64), ("ring_bytes", C.c_int64), ("lag_chunks", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BoxOpts(C.Structure):
    _fields_ = [("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("stretch_z", C.c_double), ("jitter", C.c_double), ("seed", C.c_uint64),
                ("periodic_x", C.c_int), ("periodic_y", C.c_int), ("tets", C.c_int),
                ("renumber", C.c_int), ("renumber_seed", C.c_uint64)]


# every exported symbol with its argument types (checked by the CPU tests)
_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "nw_last_error_string": (C.c_char_p, []),
    "nw_version": (C.c_int, []),
    "nw_set_device": (C.c_int, [C.c_int]),
    "nw_linsys_create": (C.c_int, [C.c_int, C.POINTER(SolverCfg), C.POINTER(C.c_void_p)]),
    "nw_linsys_destroy": (C.c_int, [C.c_void_p]),
    "nw_linsys_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "nw_linsys_extract_diagonal": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "nw_udiag_postprocess": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                       C.c_void_p]),
    "nw_linsys_set_solver_cfg": (C.c_int, [C.c_void_p, C.POINTER(SolverCfg)]),
    "nw_linsys_build_edge_graph": (C.c_int, [C.c_void_p, C.c_int64, _I64P, _I64P, C.c_int64, _I64P]),
    "nw_linsys_finalize": (C.c_int, [C.c_void_p]),
    "nw_linsys_graph_sizes": (C.c_int, [C.c_void_p, _I64P, _I64P]),
    "nw_linsys_get_graph": (C.c_int, [C.c_void_p, _I64P, _I32P]),
    "nw_linsys_get_node_lid": (C.c_int, [C.c_void_p, _I64P]),
    "nw_linsys_zero": (C.c_int, [C.c_void_p]),
    "nw_assemble_scalar_edges": (C.c_int, [C.c_void_p, C.POINTER(ScalarFields), C.POINTER(ScalarOpts)]),
    "nw_assemble_continuity_edges": (C.c_int, [C.c_void_p, C.POINTER(ContinuityFields),
                                               C.POINTER(ContinuityOpts)]),
    "nw_assemble_continuity_edge_range": (C.c_int, [C.c_void_p, C.POINTER(ContinuityFields),
                                                    C.POINTER(ContinuityOpts), C.c_int64, C.c_int64]),
    "nw_assemble_continuity_rows": (C.c_int, [C.c_void_p]),
    "nw_assemble_momentum_edges": (C.c_int, [C.c_void_p, C.POINTER(MomentumFields), C.POINTER(MomentumOpts)]),
    "nw_assemble_momentum_edge_range": (C.c_int, [C.c_void_p, C.POINTER(MomentumFields), C.POINTER(MomentumOpts),
                                                  C.c_int64, C.c_int64]),
    "nw_assemble_momentum_rows": (C.c_int, [C.c_void_p, C.POINTER(MomentumOpts)]),
    "nw_assemble_momentum_rows_range": (C.c_int, [C.c_void_p, C.POINTER(MomentumOpts), C.c_int64, C.c_int64]),
    "nw_linsys_sgs_classes": (C.c_int, [C.c_void_p, _I64P]),
    "nw_linsys_set_assembly_path": (C.c_int, [C.c_void_p, C.c_int]),
    "nw_linsys_assembly_schedule": (C.c_int, [C.c_void_p, C.POINTER(AssemblySchedule)]),
    "nw_momentum_schedule": (C.c_int, [C.c_int64, C.c_int64, _I64P, C.c_int64, C.c_int64,
                                       C.POINTER(AssemblySchedule), _I32P, _I32P, _I32P, _I32P, _I32P]),
    "nw_linsys_checkpoint_save": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    "nw_linsys_checkpoint_load": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.POINTER(SolveReport)]),
    "nw_solver_cfg_from_strings": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(SolverCfg)]),
    "nw_learned_set_coarse_direction": (C.c_int, [C.c_void_p, C.c_int]),
    "nw_learned_set_aggregation": (C.c_int, [C.c_void_p, C.c_double]),
    "nw_assemble_continuity_edges_noalloc": (C.c_int, [C.c_void_p, C.POINTER(ContinuityFields),
                                                       C.POINTER(ContinuityOpts), C.c_void_p, C.c_void_p]),
    "nw_linsys_sum_into": (C.c_int, [C.c_void_p, C.c_int, _I64P, _DP, _DP]),
    "nw_linsys_apply_dirichlet": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p]),
    "nw_linsys_reset_rows": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_int,
                                       C.c_double, C.c_double]),
    "nw_linsys_load_complete": (C.c_int, [C.c_void_p]),
    "nw_linsys_device_arrays": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                          C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "nw_linsys_copy_to_host": (C.c_int, [C.c_void_p, _DP, _DP]),
    "nw_linsys_copy_from_host": (C.c_int, [C.c_void_p, _DP, _DP]),
    "nw_linsys_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(SolveReport)]),
    "nw_linsys_residual_history": (C.c_int, [C.c_void_p, _DP, C.c_int, C.POINTER(C.c_int)]),
    "nw_linsys_rows_to_nodes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "nw_linsys_spmv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "nw_linsys_precond_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "nw_linsys_sgs_order": (C.c_int, [C.c_void_p, _I64P, C.POINTER(C.c_int)]),
    "nw_linsys_sync": (C.c_int, [C.c_void_p]),
    "nw_linsys_last_assembly_ms": (C.c_int, [C.c_void_p, _DP]),
    "nw_learned_create": (C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    "nw_learned_destroy": (C.c_int, [C.c_void_p]),
    "nw_learned_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "nw_learned_load": (C.c_int, [C.c_void_p, C.c_char_p]),
    "nw_learned_num_params": (C.c_int64, []),
    "nw_learned_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64]),
    "nw_learned_configure": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "nw_linsys_attach_learned": (C.c_int, [C.c_void_p, C.c_void_p]),
    "nw_linsys_coarse_sizes": (C.c_int, [C.c_void_p, _I64P, _I64P]),
    "nw_linsys_coarse_graph": (C.c_int, [C.c_void_p, _I32P, _I64P, _I32P, C.POINTER(C.c_float),
                                         C.POINTER(C.c_float)]),
    "nw_learned_harvest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "nw_learned_clear_data": (C.c_int, [C.c_void_p]),
    "nw_learned_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_uint64,
                                   C.POINTER(C.c_double)]),
    "nw_learned_evaluate": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "nw_learned_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                       C.POINTER(C.c_double), C.POINTER(C.c_float)]),
    "nw_learned_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "nw_gemm_bf16": (C.c_int, [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "nw_compute_mdot_edges": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p]),
    "nw_compute_nodal_gradient": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p]),
    "nw_compute_peclet_factor": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.POINTER(PecletOpts), C.c_void_p, C.c_void_p]),
    "nw_assemble_scalar_mass_bdf": (C.c_int, [C.c_void_p, C.POINTER(MassBdfFields), C.POINTER(BdfOpts)]),
    "nw_sideset_create": (C.c_int, [C.c_void_p, C.c_int64, _I64P, C.POINTER(C.c_void_p)]),
    "nw_sideset_destroy": (C.c_int, [C.c_void_p]),
    "nw_sideset_sizes": (C.c_int, [C.c_void_p, _I64P, _I64P]),
    "nw_assemble_continuity_open": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(ContinuityOpenFields),
                                              C.POINTER(ContinuityOpenOpts)]),
    "nw_assemble_momentum_open": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(MomentumOpenFields),
                                            C.POINTER(MomentumOpenOpts)]),
    "nw_assemble_momentum_symmetry": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(MomentumSymmetryFields),
                                                C.POINTER(MomentumSymmetryOpts)]),
    "nw_assemble_scalar_open": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(ScalarOpenFields), C.c_double]),
    "nw_assemble_momentum_abl_wall": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(AblWallFields),
                                                C.POINTER(AblWallOpts)]),
    "nw_assemble_momentum_abl_wall_shear_stress": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                             C.c_int]),
    "nw_compute_open_mdot": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(ContinuityOpenFields), C.c_double,
                                       C.c_double, C.c_void_p, C.POINTER(C.c_double)]),
    "nw_correct_open_mdot": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                       C.POINTER(C.c_double)]),
    "nw_assemble_continuity_mass_bdf": (C.c_int, [C.c_void_p, C.POINTER(MassBdfFields), C.POINTER(BdfOpts)]),
    "nw_assemble_momentum_mass_bdf": (C.c_int, [C.c_void_p, C.POINTER(MassBdfFields), C.POINTER(BdfOpts)]),
    "nw_linsys_write_matrix_market": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_void_p]),
    "nw_linsys_read_matrix_market": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    "nw_mesh_box": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(BoxOpts), C.POINTER(C.c_void_p)]),
    "nw_geometry_create": (C.c_int, [C.c_int64, C.c_int, C.c_int64, _I64P, C.c_int64, _I64P, _I64P,
                                     C.POINTER(C.c_void_p)]),
    "nw_geometry_compute": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "nw_geometry_destroy": (C.c_int, [C.c_void_p]),
    "nw_mesh_destroy": (C.c_int, [C.c_void_p]),
    "nw_mesh_rcm_order": (C.c_int, [C.c_int64, C.c_int64, _I64P, _I64P]),
    "nw_mesh_sizes": (C.c_int, [C.c_void_p, _I64P, _I64P, _I64P, C.POINTER(C.c_int)]),
    "nw_mesh_get": (C.c_int, [C.c_void_p, _DP, _I64P, _I64P, _I64P, _I64P, _DP, _DP, _DP]),
    "nw_mesh_face_ips": (C.c_int, [C.c_void_p, C.c_int, _I64P, _I64P, _DP, C.POINTER(C.c_int32)]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libnw_gb300.so (in-tree). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise NwError(9, f"{p} is not built; run nalu-wind_gb300/build.py")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != NW_OK:
        msg = load().nw_last_error_string().decode()
        raise NwError(status, msg)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def dptr(x) -> int:
    """Device pointer of a torch tensor (or an int already)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def solver_cfg(method=GMRES, preconditioner=PC_JACOBI, precision=PREC_FP64, kspace=50,
               max_iterations=50, tolerance=1e-4, final_tolerance=None, inner_kspace=0,
               inner_tolerance=0.0, sgs2_inner_sweeps=1, sstep_size=5) -> SolverCfg:
    """TpetraLinearSolverConfig::load defaults (src/LinearSolverConfig.C:37-52)."""
    return SolverCfg(method, preconditioner, precision, kspace, max_iterations, tolerance,
                     tolerance if final_tolerance is None else final_tolerance, inner_kspace,
                     inner_tolerance, sgs2_inner_sweeps, sstep_size)


def rcm_order(num_nodes: int, edges: np.ndarray) -> np.ndarray:
    """Reverse Cuthill-McKee order of the node graph (nw_mesh_rcm_order):
    order[k] is the node to place at position k."""
    e = np.ascontiguousarray(edges, np.int64).reshape(-1, 2)
    out = np.zeros(int(num_nodes), np.int64)
    check(load().nw_mesh_rcm_order(int(num_nodes), e.shape[0], _ptr(e, C.c_int64), _ptr(out, C.c_int64)))
    return out


def momentum_schedule(rows: int, edge_rows: np.ndarray, concurrency: int,
                      max_ring_bytes: int = 64 << 20) -> dict:
    """Work list of the single-kernel momentum assembly for a graph given by
    its edge list (E x 2 node rows); host only. Returns the sizes plus the
    arrays items, chunk_lo, chunk_hi, block_lo, block_hi."""
    lib = load()
    er = np.ascontiguousarray(edge_rows, np.int64).reshape(-1, 2)
    info = AssemblySchedule()
    args = (int(rows), er.shape[0], _ptr(er, C.c_int64), int(concurrency), int(max_ring_bytes),
            C.byref(info))
    check(lib.nw_momentum_schedule(*args, None, None, None, None, None))
    out = info.as_dict()
    arrs = {k: np.zeros(n, np.int32) for k, n in (
        ("items", info.edge_chunks + info.row_blocks), ("chunk_lo", info.row_blocks),
        ("chunk_hi", info.row_blocks), ("block_lo", info.edge_chunks), ("block_hi", info.edge_chunks))}
    check(lib.nw_momentum_schedule(*args, *(_ptr(arrs[k], C.c_int32) for k in
                                            ("items", "chunk_lo", "chunk_hi", "block_lo", "block_hi"))))
    out.update(arrs)
    return out


def solver_cfg_from_strings(method: str, preconditioner: str, **kw) -> SolverCfg:
    """The reference's YAML strings ("gmres", "cg", "tfqmr", "bicgstab";
    "jacobi" / "default", "sgs", "mt_sgs", "sgs2", "riluk") mapped by the
    library (nw_solver_cfg_from_strings), other fields as solver_cfg."""
    cfg = solver_cfg(**kw)
    check(load().nw_solver_cfg_from_strings(method.encode(), preconditioner.encode(), C.byref(cfg)))
    return cfg


class LinearSystem:
    """One GPU linear system: graph, assembly, Dirichlet rows and solve."""

    def __init__(self, num_dof: int = 1, cfg: SolverCfg | None = None, stream: int | None = None):
        self.lib = load()
        self.num_dof = num_dof
        h = C.c_void_p()
        check(self.lib.nw_linsys_create(num_dof, C.byref(cfg) if cfg else None, C.byref(h)))
        self.h = h
        if stream is not None:
            check(self.lib.nw_linsys_set_stream(self.h, C.c_void_p(stream)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.nw_linsys_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream: int) -> None:
        check(self.lib.nw_linsys_set_stream(self.h, C.c_void_p(stream)))

    def set_solver_cfg(self, cfg: SolverCfg) -> None:
        check(self.lib.nw_linsys_set_solver_cfg(self.h, C.byref(cfg)))

    # -- graph (buildEdgeToNodeGraph + finalizeLinearSystem)
    def build_edge_graph(self, num_nodes: int, edges: np.ndarray, global_id=None, nalu_id=None) -> None:
        e = np.ascontiguousarray(edges, dtype=np.int64)
        g = None if global_id is None else np.ascontiguousarray(global_id, dtype=np.int64)
        n = None if nalu_id is None else np.ascontiguousarray(nalu_id, dtype=np.int64)
        check(self.lib.nw_linsys_build_edge_graph(
            self.h, num_nodes, None if g is None else _ptr(g, C.c_int64),
            None if n is None else _ptr(n, C.c_int64), e.shape[0], _ptr(e, C.c_int64)))

    def finalize(self) -> None:
        check(self.lib.nw_linsys_finalize(self.h))

    def sizes(self) -> tuple[int, int]:
        nr, nz = C.c_int64(), C.c_int64()
        check(self.lib.nw_linsys_graph_sizes(self.h, C.byref(nr), C.byref(nz)))
        return nr.value, nz.value

    def graph(self) -> tuple[np.ndarray, np.ndarray]:
        nr, nz = self.sizes()
        rp = np.zeros(nr + 1, np.int64)
        ci = np.zeros(nz, np.int32)
        check(self.lib.nw_linsys_get_graph(self.h, _ptr(rp, C.c_int64), _ptr(ci, C.c_int32)))
        return rp, ci

    def node_lid(self, num_nodes: int) -> np.ndarray:
        out = np.zeros(num_nodes, np.int64)
        check(self.lib.nw_linsys_get_node_lid(self.h, _ptr(out, C.c_int64)))
        return out

    # -- assembly
    def zero_system(self) -> None:
        check(self.lib.nw_linsys_zero(self.h))

    def assemble_scalar(self, f: ScalarFields, o: ScalarOpts) -> None:
        check(self.lib.nw_assemble_scalar_edges(self.h, C.byref(f), C.byref(o)))

    def assemble_continuity(self, f: ContinuityFields, o: ContinuityOpts) -> None:
        check(self.lib.nw_assemble_continuity_edges(self.h, C.byref(f), C.byref(o)))

    def assemble_continuity_range(self, f: ContinuityFields, o: ContinuityOpts, edge_begin: int,
                                  edge_end: int) -> None:
        """Edge phase over edges [edge_begin, edge_end), ranges in order from
        edge 0; finish with assemble_continuity_rows."""
        check(self.lib.nw_assemble_continuity_edge_range(self.h, C.byref(f), C.byref(o), edge_begin, edge_end))

    def assemble_continuity_rows(self) -> None:
        check(self.lib.nw_assemble_continuity_rows(self.h))

    def assemble_continuity_noalloc(self, f: ContinuityFields, o: ContinuityOpts, values_dev, rhs_dev) -> None:
        """Continuity assembly into caller-owned device arrays with no device
        allocation (fixed in-library scratch; at most 524,288 edges)."""
        check(self.lib.nw_assemble_continuity_edges_noalloc(self.h, C.byref(f), C.byref(o), dptr(values_dev),
                                                            dptr(rhs_dev)))

    def assemble_momentum(self, f: MomentumFields, o: MomentumOpts) -> None:
        check(self.lib.nw_assemble_momentum_edges(self.h, C.byref(f), C.byref(o)))

    def assemble_momentum_range(self, fields: "MomentumFields", opts: "MomentumOpts", edge_begin: int,
                                edge_end: int) -> None:
        """Edge phase over edges [edge_begin, edge_end); finish with assemble_momentum_rows."""
        check(self.lib.nw_assemble_momentum_edge_range(self.h, C.byref(fields), C.byref(opts), edge_begin,
                                                       edge_end))

    def assemble_momentum_rows(self, opts: "MomentumOpts") -> None:
        check(self.lib.nw_assemble_momentum_rows(self.h, C.byref(opts)))

    def assemble_momentum_rows_range(self, opts: "MomentumOpts", row_begin: int, row_end: int) -> None:
        """Row phase over node rows [row_begin, row_end)."""
        check(self.lib.nw_assemble_momentum_rows_range(self.h, C.byref(opts), int(row_begin), int(row_end)))

    def sum_into(self, nodes, rhs, lhs) -> None:
        nodes = np.ascontiguousarray(nodes, np.int64)
        rhs = np.ascontiguousarray(rhs, np.float64)
        lhs = np.ascontiguousarray(lhs, np.float64)
        check(self.lib.nw_linsys_sum_into(self.h, len(nodes), _ptr(nodes, C.c_int64),
                                          _ptr(rhs, C.c_double), _ptr(lhs, C.c_double)))

    def apply_dirichlet(self, n: int, nodes_dev, begin: int, end: int, q_dev, bc_dev) -> None:
        check(self.lib.nw_linsys_apply_dirichlet(self.h, n, dptr(nodes_dev), begin, end,
                                                 dptr(q_dev), dptr(bc_dev)))

    def reset_rows(self, n: int, nodes_dev, begin: int, end: int, diag: float, rhs: float) -> None:
        check(self.lib.nw_linsys_reset_rows(self.h, n, dptr(nodes_dev), begin, end, diag, rhs))

    def load_complete(self) -> None:
        check(self.lib.nw_linsys_load_complete(self.h))

    def to_host(self) -> tuple[np.ndarray, np.ndarray]:
        nr, nz = self.sizes()
        v = np.zeros(nz)
        r = np.zeros(nr)
        check(self.lib.nw_linsys_copy_to_host(self.h, _ptr(v, C.c_double), _ptr(r, C.c_double)))
        return v, r

    def from_host(self, values=None, rhs=None) -> None:
        v = None if values is None else np.ascontiguousarray(values, np.float64)
        r = None if rhs is None else np.ascontiguousarray(rhs, np.float64)
        check(self.lib.nw_linsys_copy_from_host(self.h, None if v is None else _ptr(v, C.c_double),
                                                None if r is None else _ptr(r, C.c_double)))

    def device_arrays(self):
        v, r, rp, ci = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(self.lib.nw_linsys_device_arrays(self.h, C.byref(v), C.byref(r), C.byref(rp), C.byref(ci)))
        return v.value, r.value, rp.value, ci.value

    # -- solve
    def solve(self, x_dev, final_iter: bool = False) -> SolveReport:
        rep = SolveReport()
        check(self.lib.nw_linsys_solve(self.h, dptr(x_dev), int(final_iter), C.byref(rep)))
        return rep

    def residual_history(self) -> np.ndarray:
        cnt = C.c_int()
        check(self.lib.nw_linsys_residual_history(self.h, None, 0, C.byref(cnt)))
        out = np.zeros(cnt.value)
        check(self.lib.nw_linsys_residual_history(self.h, _ptr(out, C.c_double), cnt.value, C.byref(cnt)))
        return out

    def spmv(self, x_dev, y_dev) -> None:
        check(self.lib.nw_linsys_spmv(self.h, dptr(x_dev), dptr(y_dev)))

    def precond_apply(self, kind: int, x_dev, y_dev) -> None:
        check(self.lib.nw_linsys_precond_apply(self.h, kind, dptr(x_dev), dptr(y_dev)))

    def sgs_order(self) -> tuple[np.ndarray, int]:
        nr, _ = self.sizes()
        order = np.zeros(nr, np.int64)
        nc = C.c_int()
        check(self.lib.nw_linsys_sgs_order(self.h, _ptr(order, C.c_int64), C.byref(nc)))
        return order, nc.value

    def sgs_classes(self) -> np.ndarray:
        """Colour-class boundaries of sgs_order() (ncolors + 1)."""
        _, nc = self.sgs_order()
        cp = np.zeros(nc + 1, np.int64)
        check(self.lib.nw_linsys_sgs_classes(self.h, _ptr(cp, C.c_int64)))
        return cp

    def checkpoint_save(self, path, x_dev=None) -> None:
        """Raw binary checkpoint of the system and solver state (and x)."""
        check(self.lib.nw_linsys_checkpoint_save(self.h, str(path).encode(),
                                                 None if x_dev is None else C.c_void_p(dptr(x_dev))))

    def checkpoint_load(self, path, x_dev=None) -> "SolveReport":
        rep = SolveReport()
        check(self.lib.nw_linsys_checkpoint_load(self.h, str(path).encode(),
                                                 None if x_dev is None else C.c_void_p(dptr(x_dev)),
                                                 C.byref(rep)))
        return rep

    def sync(self) -> None:
        check(self.lib.nw_linsys_sync(self.h))

    def set_assembly_path(self, path: int) -> None:
        """ASSEMBLY_TWO_KERNELS (default) or ASSEMBLY_SINGLE_KERNEL for
        the momentum assembly; both give the same bits."""
        check(self.lib.nw_linsys_set_assembly_path(self.h, int(path)))

    def assembly_schedule(self) -> dict:
        info = AssemblySchedule()
        check(self.lib.nw_linsys_assembly_schedule(self.h, C.byref(info)))
        return info.as_dict()

    # -- MatrixMarket
    def write_matrix_market(self, base, count: int = 0, x=None) -> None:
        xx = None if x is None else np.ascontiguousarray(x, np.float64)
        check(self.lib.nw_linsys_write_matrix_market(self.h, str(base).encode(), count,
                                                     None if xx is None else xx.ctypes.data))

    def read_matrix_market(self, matrix_path, rhs_path=None) -> None:
        check(self.lib.nw_linsys_read_matrix_market(self.h, str(matrix_path).encode(),
                                                    None if rhs_path is None else str(rhs_path).encode()))

    # -- node kernels (lumped-mass BDF time terms)
    def assemble_mass_bdf(self, kind: str, density, dual_volume, q=None, dpdx=None, dt=0.1,
                          gamma=(1.0, -1.0, 0.0)) -> None:
        """kind "scalar", "continuity" or "momentum"; density, dual_volume and
        q are (Nm1, N, Np1) triples of device tensors."""
        qq = q if q is not None else (None, None, None)
        f = MassBdfFields(*(dptr(a) for a in (*density, *dual_volume, *qq, dpdx)))
        o = BdfOpts(dt, *gamma)
        fn = {"scalar": self.lib.nw_assemble_scalar_mass_bdf,
              "continuity": self.lib.nw_assemble_continuity_mass_bdf,
              "momentum": self.lib.nw_assemble_momentum_mass_bdf}[kind]
        check(fn(self.h, C.byref(f), C.byref(o)))

    # -- momentum_diag (Udiag) of the pressure projection
    def extract_diagonal(self, diag_dev, dof=0) -> None:
        check(self.lib.nw_linsys_extract_diagonal(self.h, dof, dptr(diag_dev)))

    def udiag_postprocess(self, density_dev, dual_volume_dev, udiag_dev, dt, gamma1=1.0, relax=1.0) -> None:
        check(self.lib.nw_udiag_postprocess(self.h, dptr(density_dev), dptr(dual_volume_dev), dt, gamma1, relax,
                                            dptr(udiag_dev)))

    # -- boundary face kernels (add to the assembled system)
    def sideset(self, ip_nodes) -> "SideSet":
        return SideSet(self, ip_nodes)

    def assemble_continuity_open(self, ss: "SideSet", fields: ContinuityOpenFields,
                                 opts: ContinuityOpenOpts) -> None:
        check(self.lib.nw_assemble_continuity_open(self.h, ss.h, C.byref(fields), C.byref(opts)))

    def assemble_momentum_open(self, ss: "SideSet", fields: MomentumOpenFields, opts: MomentumOpenOpts) -> None:
        check(self.lib.nw_assemble_momentum_open(self.h, ss.h, C.byref(fields), C.byref(opts)))

    def assemble_momentum_symmetry(self, ss: "SideSet", fields: MomentumSymmetryFields,
                                   opts: MomentumSymmetryOpts) -> None:
        check(self.lib.nw_assemble_momentum_symmetry(self.h, ss.h, C.byref(fields), C.byref(opts)))

    def assemble_momentum_abl_wall(self, ss: "SideSet", fields: AblWallFields, opts: AblWallOpts) -> None:
        check(self.lib.nw_assemble_momentum_abl_wall(self.h, ss.h, C.byref(fields), C.byref(opts)))

    def assemble_momentum_abl_wall_shear_stress(self, ss: "SideSet", area_dev, tau_dev, slip=False) -> None:
        check(self.lib.nw_assemble_momentum_abl_wall_shear_stress(self.h, ss.h, dptr(area_dev), dptr(tau_dev),
                                                                  int(bool(slip))))

    def assemble_scalar_open(self, ss: "SideSet", fields: ScalarOpenFields, relax=1.0) -> None:
        check(self.lib.nw_assemble_scalar_open(self.h, ss.h, C.byref(fields), relax))

    def open_mdot(self, ss: "SideSet", fields: ContinuityOpenFields, mdot_dev, noc_fac=1.0, pstab_fac=1.0) -> float:
        """Open mass flow rate per face IP into mdot_dev; returns the sum."""
        t = C.c_double()
        check(self.lib.nw_compute_open_mdot(self.h, ss.h, C.byref(fields), noc_fac, pstab_fac, dptr(mdot_dev),
                                            C.byref(t)))
        return t.value

    def correct_open_mdot(self, ss: "SideSet", correction: float, mdot_dev) -> float:
        t = C.c_double()
        check(self.lib.nw_correct_open_mdot(self.h, ss.h, correction, dptr(mdot_dev), C.byref(t)))
        return t.value

    # -- input producers (device tensors in and out)
    def compute_mdot(self, fields: "ContinuityFields", mdot_dev, noc_fac=1.0, interp_together=1.0) -> None:
        check(self.lib.nw_compute_mdot_edges(self.h, C.byref(fields), noc_fac, interp_together, dptr(mdot_dev)))

    def nodal_gradient(self, phi_dev, area_dev, dualvol_dev, grad_dev, bnd_area_dev=None, dim1=1) -> None:
        check(self.lib.nw_compute_nodal_gradient(self.h, dim1, dptr(phi_dev), dptr(area_dev), dptr(dualvol_dev),
                                                 dptr(bnd_area_dev), dptr(grad_dev)))

    def peclet_factor(self, coords_dev, density_dev, viscosity_dev, velocity_dev, pecfac_dev,
                      opts: "PecletOpts | None" = None, pecnum_dev=None) -> None:
        o = opts if opts is not None else PecletOpts(0, 1.0, 2.0, 4.0, 1e-16)
        check(self.lib.nw_compute_peclet_factor(self.h, dptr(coords_dev), dptr(density_dev), dptr(viscosity_dev),
                                                dptr(velocity_dev), C.byref(o), dptr(pecnum_dev),
                                                dptr(pecfac_dev)))

    # -- learned preconditioner
    def attach_learned(self, net: "Learned") -> None:
        check(self.lib.nw_linsys_attach_learned(self.h, net.h))
        self._learned = net  # keep alive

    def coarse_graph(self) -> dict:
        nc, nnzc = C.c_int64(), C.c_int64()
        check(self.lib.nw_linsys_coarse_sizes(self.h, C.byref(nc), C.byref(nnzc)))
        nr, _ = self.sizes()
        agg = np.zeros(nr, np.int32)
        cptr = np.zeros(nc.value + 1, np.int64)
        ccol = np.zeros(nnzc.value, np.int32)
        wgt = np.zeros(nnzc.value, np.float32)
        dinv = np.zeros(nc.value, np.float32)
        check(self.lib.nw_linsys_coarse_graph(self.h, _ptr(agg, C.c_int32), _ptr(cptr, C.c_int64),
                                              _ptr(ccol, C.c_int32), _ptr(wgt, C.c_float),
                                              _ptr(dinv, C.c_float)))
        return dict(nc=nc.value, agg=agg, cptr=cptr, ccol=ccol, wgt=wgt, dinv=dinv)

    def last_assembly_ms(self) -> float:
        ms = C.c_double()
        check(self.lib.nw_linsys_last_assembly_ms(self.h, C.byref(ms)))
        return ms.value


class Learned:
    """Learned two-level preconditioner network (NW_PC_LEARNED)."""

    def __init__(self, seed: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.nw_learned_create(seed, C.byref(h)))
        self.h = h
        self.num_params = int(self.lib.nw_learned_num_params())

    def close(self):
        if getattr(self, "h", None):
            self.lib.nw_learned_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(self.lib.nw_learned_params(self.h, _ptr(out, C.c_float), None, self.num_params))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(self.lib.nw_learned_params(self.h, None, _ptr(p, C.c_float), self.num_params))

    def configure(self, post_smooth: bool = True, agg_passes: int = 2, smoother: int = 0) -> None:
        check(self.lib.nw_learned_configure(self.h, int(post_smooth), int(agg_passes), int(smoother)))

    def set_aggregation(self, strength: float) -> None:
        """0: plain aggregation; in (0, 1): aggregation over strong
        connections (nw_learned_set_aggregation)."""
        check(self.lib.nw_learned_set_aggregation(self.h, float(strength)))

    def set_coarse_direction(self, mode: int) -> None:
        """0: the network; 1: D_c^-1 r_c; 2: two Jacobi sweeps on Ac (controls
        without the network, same cycle and scaling)."""
        check(self.lib.nw_learned_set_coarse_direction(self.h, int(mode)))

    def save(self, path) -> None:
        check(self.lib.nw_learned_save(self.h, str(path).encode()))

    def load(self, path) -> None:
        check(self.lib.nw_learned_load(self.h, str(path).encode()))

    def harvest(self, ls: "LinearSystem", restarts: int, kspace: int = 30) -> int:
        n = C.c_int()
        check(self.lib.nw_learned_harvest(self.h, ls.h, restarts, kspace, C.byref(n)))
        return n.value

    def clear_data(self) -> None:
        check(self.lib.nw_learned_clear_data(self.h))

    def train(self, ls: "LinearSystem", epochs: int, batch: int = 8, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_double()
        check(self.lib.nw_learned_train(self.h, ls.h, epochs, batch, lr, seed, C.byref(loss)))
        return loss.value

    def evaluate(self, ls: "LinearSystem") -> float:
        loss = C.c_double()
        check(self.lib.nw_learned_evaluate(self.h, ls.h, C.byref(loss)))
        return loss.value

    def loss_grad(self, ls: "LinearSystem", rc_dev, ea: float, ca: float):
        loss = C.c_double()
        g = np.zeros(self.num_params, np.float32)
        check(self.lib.nw_learned_loss_grad(self.h, ls.h, dptr(rc_dev), ea, ca, C.byref(loss),
                                            _ptr(g, C.c_float)))
        return loss.value, g

    def forward(self, ls: "LinearSystem", rc_dev, ec_dev) -> None:
        check(self.lib.nw_learned_forward(self.h, ls.h, dptr(rc_dev), dptr(ec_dev)))


def gemm_bf16(kind: int, m: int, a_dev, b_dev, out_dev) -> None:
    check(load().nw_gemm_bf16(kind, m, dptr(a_dev), dptr(b_dev), dptr(out_dev)))


class Geometry:
    """Edge area vectors and dual volumes of a mesh on the device
    (nw_geometry_*): built once from the connectivity and edge list, then
    compute(coords_dev, area_dev, dualvol_dev) after every mesh motion."""

    def __init__(self, num_nodes: int, conn: np.ndarray, edges: np.ndarray, nalu_id=None):
        self.lib = load()
        conn = np.ascontiguousarray(conn, np.int64)
        edges = np.ascontiguousarray(edges, np.int64)
        nid = None if nalu_id is None else np.ascontiguousarray(nalu_id, np.int64)
        h = C.c_void_p()
        check(self.lib.nw_geometry_create(num_nodes, conn.shape[1], conn.shape[0], _ptr(conn, C.c_int64),
                                          edges.shape[0], _ptr(edges, C.c_int64),
                                          None if nid is None else _ptr(nid, C.c_int64), C.byref(h)))
        self.h = h

    def compute(self, coords_dev, area_dev, dualvol_dev, stream=None) -> None:
        check(self.lib.nw_geometry_compute(self.h, dptr(coords_dev), dptr(area_dev), dptr(dualvol_dev),
                                           C.c_void_p(stream) if stream else None))

    def close(self):
        if getattr(self, "h", None):
            self.lib.nw_geometry_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SideSet:
    """Face integration points of one boundary registered on a finalized
    LinearSystem: ip_nodes (n, 2) = (face node, opposing element node)."""

    def __init__(self, ls: "LinearSystem", ip_nodes):
        self.lib = ls.lib
        self._ls = ls  # the handle must outlive the side set
        ipn = np.ascontiguousarray(np.asarray(ip_nodes, np.int64).reshape(-1, 2))
        h = C.c_void_p()
        check(self.lib.nw_sideset_create(ls.h, ipn.shape[0], _ptr(ipn, C.c_int64), C.byref(h)))
        self.h = h

    def sizes(self):
        n, r = C.c_int64(), C.c_int64()
        check(self.lib.nw_sideset_sizes(self.h, C.byref(n), C.byref(r)))
        return n.value, r.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.nw_sideset_destroy(self.h)
            self.h = None


class Mesh:
    """Synthetic block mesh (nw_workload.h): coordinates, ids, edges, geometry."""

    def __init__(self, nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, stretch_z=1.0, jitter=0.0, seed=0,
                 periodic_x=False, periodic_y=False, tets=False, renumber=0, renumber_seed=0):
        lib = load()
        o = BoxOpts(lx, ly, lz, stretch_z, jitter, seed, int(periodic_x), int(periodic_y), int(tets),
                    renumber, renumber_seed)
        h = C.c_void_p()
        check(lib.nw_mesh_box(nx, ny, nz, C.byref(o), C.byref(h)))
        try:
            N, E, M, npe = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int()
            check(lib.nw_mesh_sizes(h, C.byref(N), C.byref(E), C.byref(M), C.byref(npe)))
            self.num_nodes, self.num_edges, self.num_elems, self.npe = N.value, E.value, M.value, npe.value
            self.coords = np.zeros((self.num_nodes, 3))
            self.global_id = np.zeros(self.num_nodes, np.int64)
            self.nalu_id = np.zeros(self.num_nodes, np.int64)
            self.edges = np.zeros((self.num_edges, 2), np.int64)
            self.conn = np.zeros((self.num_elems, self.npe), np.int64)
            self.area = np.zeros((self.num_edges, 3))
            self.dualvol = np.zeros(self.num_nodes)
            self.bnd_area = np.zeros((self.num_nodes, 3))
            check(lib.nw_mesh_get(h, _ptr(self.coords, C.c_double), _ptr(self.global_id, C.c_int64),
                                  _ptr(self.nalu_id, C.c_int64), _ptr(self.edges, C.c_int64),
                                  _ptr(self.conn, C.c_int64), _ptr(self.area, C.c_double),
                                  _ptr(self.dualvol, C.c_double), _ptr(self.bnd_area, C.c_double)))
            cnt = C.c_int64()
            check(lib.nw_mesh_face_ips(h, 63, C.byref(cnt), None, None, None))
            self._fip_nodes = np.zeros((cnt.value, 2), np.int64)
            self._fip_area = np.zeros((cnt.value, 3))
            self._fip_side = np.zeros(cnt.value, np.int32)
            check(lib.nw_mesh_face_ips(h, 63, C.byref(cnt), _ptr(self._fip_nodes, C.c_int64),
                                       _ptr(self._fip_area, C.c_double), _ptr(self._fip_side, C.c_int32)))
        finally:
            lib.nw_mesh_destroy(h)
        self.shape = (nx, ny, nz)
        self.periodic = (bool(periodic_x), bool(periodic_y))

    SIDES = {"x-": 0, "x+": 1, "y-": 2, "y+": 3, "z-": 4, "z+": 5}

    def face_ips(self, sides=("x-", "x+", "y-", "y+", "z-", "z+")):
        """Exposed-face integration points of the given box sides:
        (ip_nodes (n, 2) = face node, opposing element node; area (n, 3))."""
        want = np.isin(self._fip_side, [self.SIDES[s] for s in sides])
        return self._fip_nodes[want].copy(), self._fip_area[want].copy()


from . import workload  # noqa: E402  (seeded synthetic inputs)
from . import training  # noqa: E402  (learned preconditioner recipe)
