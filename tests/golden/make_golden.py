"""Extract the reference's known-answer golds for the edge-assembly path.

Reads nalu-wind unit-test sources as text (no code from them is run) and
writes tests/golden/reference_golds.json. Run in a checkout that has the
reference tree:  python tests/golden/make_golden.py /path/to/nalu-wind
The JSON is committed; tests never read the reference tree.

Sources (paths within the nalu-wind tree):
  unit_tests/edge_kernels/UnitTestScalarAdvDiffEdge.C   serial Tpetra CSR
      graph, values and rhs (plain, FixPressureAtNode and Dirichlet)
  unit_tests/edge_kernels/UnitTestContinuityAdvEdge.C   dense 8x8 LHS, rhs
  unit_tests/edge_kernels/UnitTestMomentumAdvDiffEdge.C dense 24x24 LHS, rhs
  unit_tests/UnitTestPecletFunction.C                   Peclet factors
  unit_tests/ngp_algorithms/UnitTestGeometryAlg.C       dual volume, |A|^2
  unit_tests/ngp_algorithms/UnitTestMdotAlg.C           mdot
  unit_tests/node_kernels/UnitTest{Momentum,Continuity,Scalar}MassBDFNodeKernel.C
      lumped-mass BDF node kernels: diagonal LHS and rhs
  unit_tests/edge_kernels/UnitTestContinuityOpenEdge.C  open boundary (x+ side),
      dense 8x8 in node-id order
  unit_tests/edge_kernels/UnitTestMomentumOpenEdge.C    open boundary, COMPUTED
      entrainment, dense 24x24 in node-id order
  unit_tests/edge_kernels/UnitTestMomentumSymmetryEdge.C symmetry boundary, plain
      and penalty factor 2, dense 24x24 in element-node order
  unit_tests/edge_kernels/UnitTestScalarOpenEdge.C      scalar open flux with
      relaxation 0.5 and mt19937-drawn inputs (closed-form expectation)
  unit_tests/ngp_algorithms/UnitTestMdotAlg.C           open mass flow rate on the
      z+ side and the open mass-flow correction
  unit_tests/ngp_algorithms/UnitTestNodalGradAlg.C      interior edge nodal
      gradients of linear fields (scalar and vector)
  unit_tests/UnitTestLocalGraphArrays.C                 sorted, deduplicated
      insertion with numDof expansion (numDof 1 and 3)
  unit_tests/edge_kernels/UnitTestMomentumABLWallFuncEdge.C ABL wall function on
      the z- side (fixture constants of MomentumABLKernelHex8Mesh,
      unit_tests/kernels/UnitTestKernelUtils.h), closed-form expectation
"""
from __future__ import annotations

import json
import math
import re
import sys
from pathlib import Path

NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def _block(text: str, name: str) -> str:
    """Body between the braces that follow `name` (first match)."""
    i = text.index(name)
    j = text.index("=", i)
    k = text.index("{", j)
    depth = 0
    for p in range(k, len(text)):
        if text[p] == "{":
            depth += 1
        elif text[p] == "}":
            depth -= 1
            if depth == 0:
                return text[k + 1:p]
    raise ValueError(name)


def _nums(body: str) -> list[float]:
    body = re.sub(r"//[^\n]*", "", body)
    return [float(x) for x in re.findall(NUM, body)]


def main(ref: Path, out: Path) -> None:
    g: dict = {}
    s = (ref / "unit_tests/edge_kernels/UnitTestScalarAdvDiffEdge.C").read_text()
    sc = {}
    for name in ["rowOffsets_serial", "cols_serial", "vals_serial", "fixed_vals_serial",
                 "dirichlet_vals_serial", "rhs_serial", "fixed_rhs_serial", "dirichlet_rhs_serial"]:
        vals = _nums(_block(s, f" {name} "))
        sc[name] = [int(v) for v in vals] if name in ("rowOffsets_serial", "cols_serial") else vals
    g["scalar_adv_diff_hex8"] = sc

    c = (ref / "unit_tests/edge_kernels/UnitTestContinuityAdvEdge.C").read_text()
    g["continuity_hex8"] = {"rhs": _nums(_block(c, "rhs[8]")), "lhs": _nums(_block(c, "lhs[8][8]"))}

    m = (ref / "unit_tests/edge_kernels/UnitTestMomentumAdvDiffEdge.C").read_text()
    g["momentum_hex8"] = {"rhs": _nums(_block(m, "rhs[24]")), "lhs": _nums(_block(m, "lhs[24][24]"))}

    p = (ref / "unit_tests/UnitTestPecletFunction.C").read_text()
    assert "std::sqrt(5.0)" in p and "1.0 / 6.0" in p
    g["peclet_classic"] = {"A": 5.0, "hybrid_factor": 1.0,
                           "peclet": [0.0, 1.0, math.sqrt(5.0), 1e5],
                           "factor": [0.0, 1.0 / 6.0, 0.5, 1.0]}
    assert "c1 = 5000.0" in p and "c2 = 200.0" in p
    g["peclet_tanh"] = {"c1": 5000.0, "c2": 200.0,
                        "x": [-5000.0 - 2000.0, 5000.0, 5000.0 + 2000.0], "factor": [0.0, 0.5, 1.0]}

    geo = (ref / "unit_tests/ngp_algorithms/UnitTestGeometryAlg.C").read_text()
    assert "EXPECT_NEAR(0.125, dVol[0], tol)" in geo and "0.25 * 0.25" in geo
    g["geometry_hex8_unit_cube"] = {"dual_volume": 0.125, "area_mag_sq": 0.0625, "num_edges": 12}

    md = (ref / "unit_tests/ngp_algorithms/UnitTestMdotAlg.C").read_text()
    assert "EXPECT_NEAR(mdot[0], 2.5, tol)" in md and "field_fill(10.0, *velocity_)" in md
    g["mdot_hex8_unit_cube"] = {"density": 1.0, "velocity": 10.0, "mdot": 2.5}

    nk = ref / "unit_tests/node_kernels"
    mm = (nk / "UnitTestMomentumMassBDFNodeKernel.C").read_text()
    assert "timeStepN_ = 0.1" in mm and "gamma2_ = -1.0" in mm and "lhsExact[i * 24 + i] = 1.25" in mm
    g["momentum_mass_bdf_hex8"] = {"dt": 0.1, "gamma": [1.0, -1.0, 0.0], "lhs_diag": 1.25,
                                   "rhs": _nums(_block(mm, "rhs[24]"))}
    cm = (nk / "UnitTestContinuityMassBDFNodeKernel.C").read_text()
    assert "expect_all_near(helperObjs.linsys->rhs_, -12.5)" in cm and "lhs_, 0.0)" in cm
    g["continuity_mass_bdf_hex8"] = {"dt": 0.1, "gamma": [1.0, -1.0, 0.0], "lhs_diag": 0.0, "rhs": -12.5}
    sm = (nk / "UnitTestScalarMassBDFNodeKernel.C").read_text()
    lhs = _nums(_block(sm, "lhs[8][8]"))
    assert len(lhs) == 64
    g["scalar_mass_bdf_hex8"] = {"dt": 0.1, "gamma": [1.0, -1.0, 0.0],
                                 "lhs_diag": [lhs[9 * i] for i in range(8)], "rhs": _nums(_block(sm, "rhs[8]"))}

    ek = ref / "unit_tests/edge_kernels"
    co = (ek / "UnitTestContinuityOpenEdge.C").read_text()
    assert 'get_part("surface_2")' in co and "gamma1_ = 1.0" in co and "timeStepN_ = 1.0" in co
    g["continuity_open_hex8_xplus"] = {"rhs": _nums(_block(co, "rhs[8]")), "lhs": _nums(_block(co, "lhs[8][8]"))}
    mo = (ek / "UnitTestMomentumOpenEdge.C").read_text()
    assert 'get_part("surface_2")' in mo and "EntrainmentMethod::COMPUTED" in mo
    g["momentum_open_hex8_xplus"] = {"rhs": _nums(_block(mo, "rhs[24]")), "lhs": _nums(_block(mo, "lhs[24][24]"))}
    sy = (ek / "UnitTestMomentumSymmetryEdge.C").read_text()
    assert 'get_part("surface_2")' in sy and "symmetryBcPenaltyFactor_ = 2.0" in sy
    assert "check_against_gold_values" in sy  # element-node ordering
    pen = sy.index("namespace hex8_golds_penalty")
    g["momentum_symmetry_hex8_xplus"] = {
        "element_node_order": True, "penalty_factor": [0.0, 2.0],
        "rhs": [_nums(_block(sy, "rhs[24]")), _nums(_block(sy[pen:], "rhs[24]"))],
        "lhs": [_nums(_block(sy, "lhs[24][24]")), _nums(_block(sy[pen:], "lhs[24][24]"))]}
    so = (ek / "UnitTestScalarOpenEdge.C").read_text()
    for frag in ("rand_num(1.0, 2.0)", "rand_mdot(-1.0, 1.0)", "const double tkeVal = rand_num(rng);",
                 "const double bcTkeVal = rand_num(rng);", "const double mdotVal = rand_mdot(rng);",
                 'relaxFactorMap_["turbulent_ke"] = 0.5', "(-mdotVal * tkeVal) : (-mdotVal * bcTkeVal)",
                 "(mdotVal * 2.0) : 0.0"):
        assert frag in so, frag
    md = (ref / "unit_tests/ngp_algorithms/UnitTestMdotAlg.C").read_text()
    i0 = md.index("NGP_mdot_open_edge")
    blk = md[i0:]
    for frag in ('field_fill(1.0, *density_)', 'field_fill(1.0, *velocity_)', 'field_fill(0.0, *pressure_)',
                 'field_fill(0.0, *dpdx_)', 'get_part("surface_6")', "activateOpenMdotCorrection_ = true",
                 "EXPECT_NEAR(mdotDriver.mdot_open(), 1.0, 1.0e-15)"):
        assert frag in blk, frag
    g["mdot_open_hex8_zplus"] = {"density": 1.0, "velocity": 1.0, "pstab_fac": 0.0, "mdot_open": 1.0}
    blk = md[md.index("NGP_mdot_open_correction"):]
    for frag in ("mdotInflow = -124.0", "mdotOpen = 100.0", "(mdotInflow + mdotOpen) / 24.0",
                 "-mdotCorrection * 4.0", 'get_part("surface_5")', "field_fill(0.0, *openMassFlowRate_)"):
        assert frag in blk, frag
    g["mdot_open_correction_hex8"] = {"inflow": -124.0, "open": 100.0, "ip_count": 24, "side_ips": 4,
                                      "correction": -1.0, "post": 4.0}
    aw = (ek / "UnitTestMomentumABLWallFuncEdge.C").read_text()
    kf = (ref / "unit_tests/kernels/UnitTestKernelUtils.h").read_text()
    for frag in ('get_part("surface_5")', "ustar_ * kappa_ / std::log(zh_ / z0_) * 0.25",
                 "{-ustar_ * ustar_ * 0.25, 0.0, 0.0}"):
        assert frag in aw, frag
    for frag in ("z0_{0.1}", "zh_{0.25}", "uh_{0.15}", "kappa_{0.41}", "gravity_{9.81}", "Tref_{300.0}",
                 "const double vel[3] = {uh_, 0.0, 0.0};", "field_fill(0.0, *bcHeatFlux_)",
                 "field_fill(1000.0, *specificHeat_)", "ustar_(kappa_ * uh_ / std::log(zh_ / z0_))"):
        assert frag in kf, frag
    g["abl_wall_function_quad4_zminus"] = {"z0": 0.1, "zh": 0.25, "uh": 0.15, "kappa": 0.41, "gravity": 9.81,
                                          "Tref": 300.0, "heat_flux": 0.0, "specific_heat": 1000.0,
                                          "density": 1.0, "ip_area": 0.25}
    lg = (ref / "unit_tests/UnitTestLocalGraphArrays.C").read_text()
    for frag in ("create_graph({2, 3, 4})", "cols = {7, 8, 6, 5};", "create_graph({6, 9, 12})",
                 "cols = {21, 18, 24, 15};", "EXPECT_EQ(27u, csg->colIndices.size());",
                 "EXPECT_EQ((int)i, csg->colIndices[i]);"):
        assert frag in lg, frag
    g["local_graph_arrays"] = {
        "num_dof_1": {"row_lengths": [2, 3, 4], "ops": [[0, [0, 1]], [1, [2, 3, 4]], [2, [7, 8, 6, 5]],
                                                        [0, [0, 1]], [1, [2, 3, 4]]]},
        "num_dof_3": {"row_lengths": [6, 9, 12], "ops": [[0, [0, 3]], [1, [6, 9, 12]], [2, [21, 18, 24, 15]],
                                                         [0, [0, 3]], [1, [6, 9, 12]]]},
        "expect": "colIndices[i] == i for every i"}
    ng = (ref / "unit_tests/ngp_algorithms/UnitTestNodalGradAlg.C").read_text()
    ua = (ref / "unit_tests/ngp_algorithms/UnitTestNgpAlgUtils.C").read_text()
    assert "coordsData[0] * xCoeff + coordsData[1] * yCoeff" in ua and "fieldData[0] = coordsData[0] * xCoeff;" in ua
    s0 = ng[ng.index("NGP_nodal_grad_edge)"):]
    s1 = ng[ng.index("NGP_nodal_grad_edge_vec)"):]
    for s_ in (s0, s1):
        assert "const double xCoeff = 2.0;" in s_[:600] and "zCoeff = 2.0;" in s_[:700]
    sb = ng[ng.index("NGP_nodal_grad_bndry)"):]
    ss = ng[ng.index("NGP_nodal_grad_bndry_shifted)"):]
    assert 'get_part("surface_5")' in sb[:1500] and "const bool useShifted = false;" in sb[:1500]
    assert "const bool useShifted = true;" in ss[:1500]
    g["nodal_grad_bndry_hex8_zminus"] = {"coeff": [2.0, 2.0, 2.0],
                                         "unshifted": _nums(_block(sb, "expectedValues")),
                                         "shifted": _nums(_block(ss, "expectedValues"))}
    g["nodal_grad_edge_hex8"] = {"coeff": [2.0, 2.0, 2.0],
                                 "scalar": _nums(_block(s0, "expectedValues")),
                                 "vector_diagonal": _nums(_block(s1, "expectedValues"))}
    g["scalar_open_quad4"] = {"draws": [[1.0, 2.0], [1.0, 2.0], [-1.0, 1.0]], "relax": 0.5, "nodes": 4}

    assert len(g["continuity_hex8"]["lhs"]) == 64 and len(g["momentum_hex8"]["lhs"]) == 576
    assert len(g["momentum_hex8"]["rhs"]) == 24
    out.write_text(json.dumps(g, indent=1))
    print(f"wrote {out}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/nalu-wind")
    main(Path(sys.argv[1]), Path(__file__).resolve().parent / "reference_golds.json")
