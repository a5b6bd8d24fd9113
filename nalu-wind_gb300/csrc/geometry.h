// Hex8 / Tet4 sub-control-surface area vectors and sub-control volumes of
// one element, shared by the host mesh generator (workload.cpp) and the
// device geometry kernels (geometry.cu). Both are compiled without fused
// multiply-adds (host -ffp-contract=off, device -fmad=false), so the same
// coordinates give the same bits on either side.
#pragma once

#include "dd.h"  // NW_HD

namespace nw {

// Hex8 sub-control geometry, same construction as HexSCS::determinant_scs
// and HexSCV::determinant_scv (src/master_element/Hex8CVFEM.C:363-389,
// 565-591; include/master_element/Hex8GeometryFunctions.h).
NW_HD void hex_points(const double c[8][3], double v[27][3]) {
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) v[n][d] = c[n][d];
  for (int d = 0; d < 3; ++d) {
    v[8][d] = 0.5 * (c[0][d] + c[1][d]);
    v[9][d] = 0.5 * (c[1][d] + c[2][d]);
    v[10][d] = 0.5 * (c[2][d] + c[3][d]);
    v[11][d] = 0.5 * (c[3][d] + c[0][d]);
    v[12][d] = 0.25 * (c[0][d] + c[1][d] + c[2][d] + c[3][d]);
    v[13][d] = 0.5 * (c[4][d] + c[5][d]);
    v[14][d] = 0.5 * (c[5][d] + c[6][d]);
    v[15][d] = 0.5 * (c[6][d] + c[7][d]);
    v[16][d] = 0.5 * (c[7][d] + c[4][d]);
    v[17][d] = 0.25 * (c[4][d] + c[5][d] + c[6][d] + c[7][d]);
    v[18][d] = 0.5 * (c[1][d] + c[5][d]);
    v[19][d] = 0.5 * (c[0][d] + c[4][d]);
    v[20][d] = 0.25 * (c[0][d] + c[1][d] + c[4][d] + c[5][d]);
    v[21][d] = 0.5 * (c[3][d] + c[7][d]);
    v[22][d] = 0.5 * (c[2][d] + c[6][d]);
    v[23][d] = 0.25 * (c[2][d] + c[3][d] + c[6][d] + c[7][d]);
    v[24][d] = 0.25 * (c[1][d] + c[2][d] + c[5][d] + c[6][d]);
    v[25][d] = 0.25 * (c[0][d] + c[3][d] + c[4][d] + c[7][d]);
    double s = 0.0;
    for (int n = 0; n < 8; ++n) s += c[n][d];
    v[26][d] = s * 0.125;
  }
}

// Vector area of a quadrilateral sub-control surface q0 q1 q2 q3: half the
// cross product of its diagonals. The vector area of a closed polygon
// depends only on its boundary, so this equals, in exact arithmetic, the
// sum over the four triangles fanned around the face centre that
// Quad3DSCS / HexSCS::determinant_scs evaluate (planar or not), with one
// cross product instead of four.
NW_HD void quad_area(const double q[4][3], double a[3]) {
  const double d1[3] = {q[2][0] - q[0][0], q[2][1] - q[0][1], q[2][2] - q[0][2]};
  const double d2[3] = {q[3][0] - q[1][0], q[3][1] - q[1][1], q[3][2] - q[1][2]};
  a[0] = 0.5 * (d1[1] * d2[2] - d1[2] * d2[1]);
  a[1] = 0.5 * (d1[2] * d2[0] - d1[0] * d2[2]);
  a[2] = 0.5 * (d1[0] * d2[1] - d1[1] * d2[0]);
}

NW_HD double grandy(const double s[8][3]) {
  double cv[14][3];
  for (int n = 0; n < 8; ++n)
    for (int d = 0; d < 3; ++d) cv[n][d] = s[n][d];
  const int fn[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                               {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 3, 7}};
  for (int k = 0; k < 6; ++k)
    for (int d = 0; d < 3; ++d)
      cv[8 + k][d] = 0.25 * (cv[fn[k][0]][d] + cv[fn[k][1]][d] +
                             cv[fn[k][2]][d] + cv[fn[k][3]][d]);
  const int tf[24][3] = {
      {0, 8, 1},  {8, 2, 1},  {3, 2, 8},  {3, 8, 0},  {6, 9, 5},  {7, 9, 6},
      {4, 9, 7},  {4, 5, 9},  {10, 0, 1}, {5, 10, 1}, {4, 10, 5}, {4, 0, 10},
      {7, 6, 11}, {6, 2, 11}, {2, 3, 11}, {3, 7, 11}, {6, 12, 2}, {5, 12, 6},
      {5, 1, 12}, {1, 2, 12}, {0, 4, 13}, {4, 7, 13}, {7, 3, 13}, {3, 0, 13}};
  double vol = 0.0;
  for (int k = 0; k < 24; ++k) {
    const int p = tf[k][0], q = tf[k][1], r = tf[k][2];
    double m[3], dx[3];
    for (int d = 0; d < 3; ++d) m[d] = cv[p][d] + cv[q][d] + cv[r][d];
    dx[0] = (cv[q][1] - cv[p][1]) * (cv[r][2] - cv[p][2]) -
            (cv[r][1] - cv[p][1]) * (cv[q][2] - cv[p][2]);
    dx[1] = (cv[r][0] - cv[p][0]) * (cv[q][2] - cv[p][2]) -
            (cv[q][0] - cv[p][0]) * (cv[r][2] - cv[p][2]);
    dx[2] = (cv[q][0] - cv[p][0]) * (cv[r][1] - cv[p][1]) -
            (cv[r][0] - cv[p][0]) * (cv[q][1] - cv[p][1]);
    vol += m[0] * dx[0] + m[1] * dx[1] + m[2] * dx[2];
  }
  return vol / 18.0;
}

NW_HD void hex_geometry(const double c[8][3], double scs[12][3], double scv[8]) {
  const int facet[12][4] = {
      {20, 8, 12, 26},  {24, 9, 12, 26},  {10, 12, 26, 23}, {11, 25, 26, 12},
      {13, 20, 26, 17}, {17, 14, 24, 26}, {17, 15, 23, 26}, {16, 17, 26, 25},
      {19, 20, 26, 25}, {20, 18, 24, 26}, {22, 23, 26, 24}, {21, 25, 26, 23}};
  const int sub[8][8] = {
      {0, 8, 12, 11, 19, 20, 26, 25},  {8, 1, 9, 12, 20, 18, 24, 26},
      {12, 9, 2, 10, 26, 24, 22, 23},  {11, 12, 10, 3, 25, 26, 23, 21},
      {19, 20, 26, 25, 4, 13, 17, 16}, {20, 18, 24, 26, 13, 5, 14, 17},
      {26, 24, 22, 23, 17, 14, 6, 15}, {25, 26, 23, 21, 16, 17, 15, 7}};
  double v[27][3];
  hex_points(c, v);
  for (int ip = 0; ip < 12; ++ip) {
    double q[4][3];
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) q[k][d] = v[facet[ip][k]][d];
    quad_area(q, scs[ip]);
  }
  for (int ip = 0; ip < 8; ++ip) {
    double s[8][3];
    for (int n = 0; n < 8; ++n)
      for (int d = 0; d < 3; ++d) s[n][d] = v[sub[ip][n]][d];
    scv[ip] = grandy(s);
  }
}

// Tet4 sub-control geometry (TetSCS::determinant_scs / TetSCV::
// determinant_scv, src/master_element/Tet4CVFEM.C:243-360, 522-620).
//
// Sub-control surfaces: each is the quadrilateral (edge midpoint, face
// centroid, element centroid, face centroid) of one edge, and its vector
// area is half the cross product of its diagonals (quad_area). Both
// diagonals are fixed combinations of the edge vectors e_k = c_k - c_0 (one
// runs from a midpoint or face centroid to the centroid or a face centroid:
// (e_a + e_b - e_c) / 4 or e_k / 3 and the like), so every area is a
// small-integer combination of the three cross products X = e1 x e2,
// Y = e2 x e3, Z = e3 x e1, divided by 24. For the facets of edges
// 0-1, 1-2, 2-0, 0-3, 1-3, 2-3 (the reference's ordering of TetSCS's
// integration points): X + 2Y + Z, Z - Y, X + Y + 2Z, 2X + Y + Z, X - Y,
// X - Z. Equal to the reference's four-triangle fans in exact arithmetic,
// with three cross products instead of twenty-four.
NW_HD void tet_geometry(const double c[4][3], double scs[6][3], double scv[4]) {
  double e1[3], e2[3], e3[3];
  for (int d = 0; d < 3; ++d) {
    e1[d] = c[1][d] - c[0][d];
    e2[d] = c[2][d] - c[0][d];
    e3[d] = c[3][d] - c[0][d];
  }
  const double X[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                       e1[0] * e2[1] - e1[1] * e2[0]};
  const double Y[3] = {e2[1] * e3[2] - e2[2] * e3[1], e2[2] * e3[0] - e2[0] * e3[2],
                       e2[0] * e3[1] - e2[1] * e3[0]};
  const double Z[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2],
                       e3[0] * e1[1] - e3[1] * e1[0]};
  const double k = 1.0 / 24.0;
  for (int d = 0; d < 3; ++d) {
    scs[0][d] = k * (X[d] + 2.0 * Y[d] + Z[d]);
    scs[1][d] = k * (Z[d] - Y[d]);
    scs[2][d] = k * (X[d] + Y[d] + 2.0 * Z[d]);
    scs[3][d] = k * (2.0 * X[d] + Y[d] + Z[d]);
    scs[4][d] = k * (X[d] - Y[d]);
    scs[5][d] = k * (X[d] - Z[d]);
  }
  // The four sub-control volumes of a linear tet (node, three edge
  // midpoints, three face centroids, centroid) are its barycentric
  // subdivision: equal quarters of the tet's volume (true for a regular
  // tet by symmetry, and volume ratios are affine invariants). TetSCV
  // evaluates each with Grandy's hexahedron formula, equal in exact
  // arithmetic; the signed volume here, (e1 x e2) . e3 / 6, is taken from
  // the edge vectors, which also avoids that formula's cancellation far
  // from the origin.
  const double det = X[0] * e3[0] + X[1] * e3[1] + X[2] * e3[2];
  const double quarter = det / 24.0;
  for (int ip = 0; ip < 4; ++ip) scv[ip] = quarter;
}


}  // namespace nw
