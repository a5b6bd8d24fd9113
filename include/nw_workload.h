/*
 * nw_workload.h - synthetic mesh inputs for the edge-assembly path
 * (part of libnw_gb300.so).
 *
 * nalu-wind reads Exodus meshes through STK and computes edge geometry in
 * GeometryInteriorAlg. The benchmarks here run on seeded synthetic blocks
 * with the numbering of STK's "generated:NXxNYxNZ" meshes, so this API
 * produces what that pipeline hands the hot path:
 *   - node coordinates, global ids and periodic master ids (naluGlobalId,
 *     PeriodicManager::update_global_id_field, src/PeriodicManager.C:
 *     899-924),
 *   - the edge list with node[0] the lower id (STK create_edges),
 *   - edge_area_vector and dual_nodal_volume
 *     (GeometryInteriorAlg::impl_compute_edge_area_vector and
 *     impl_compute_dual_nodal_volume, src/ngp_algorithms/
 *     GeometryInteriorAlg.C:70-225, with the Hex8/Tet4 sub-control-surface
 *     geometry of src/master_element/Hex8CVFEM.C:565-591 and
 *     Tet4CVFEM.C),
 *   - lumped exposed-face area vectors per node for the Green-Gauss
 *     boundary closure (the sum of the node's face-IP sub-face area vectors:
 *     NodalGradBndryElemAlg with the shifted operator, src/ngp_algorithms/
 *     NodalGradBndryElemAlg.C:130-152), and the face IPs themselves.
 * All arrays are host arrays.
 */
#ifndef NW_WORKLOAD_H
#define NW_WORKLOAD_H

#include <stdint.h>

#include "nw_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nw_mesh nw_mesh;

typedef struct nw_box_opts {
  double lx, ly, lz;    /* box lengths */
  double stretch_z;     /* geometric growth ratio of z spacing from z = 0 (1 = uniform) */
  double jitter;        /* interior-node jitter, fraction of the local spacing */
  uint64_t seed;        /* jitter seed */
  int periodic_x;       /* x = lx face slaved to x = 0 */
  int periodic_y;       /* y = ly face slaved to y = 0 */
  int tets;             /* split each hex into 6 tetrahedra */
  int renumber;         /* 0 lexicographic, 1 random permutation, 2 random then RCM */
  uint64_t renumber_seed;
} nw_box_opts;

nw_status nw_mesh_box(int nx, int ny, int nz, const nw_box_opts* opts,
                      nw_mesh** out);
nw_status nw_mesh_destroy(nw_mesh* m);
/* Reverse Cuthill-McKee order of a mesh's node graph, for callers whose node
 * numbering scatters neighbours (the assembly gathers node data per edge and
 * the row phase reads every incident edge, so locality in the numbering is
 * locality in memory: on 2.1M-node tets the assembly runs 2.3x faster in
 * RCM order than in random order). edges: E pairs of node indices;
 * order[k] = the node to place at position k (breadth-first from a
 * minimum-degree node of each component, neighbours by ascending degree,
 * then reversed). Host only. */
nw_status nw_mesh_rcm_order(int64_t num_nodes, int64_t num_edges, const int64_t* edges,
                            int64_t* order);
/* nodes_per_elem: 8 (hex) or 4 (tet). */
nw_status nw_mesh_sizes(const nw_mesh* m, int64_t* num_nodes,
                        int64_t* num_edges, int64_t* num_elems,
                        int* nodes_per_elem);
/* Any output pointer may be NULL. coords N x 3, global_id N, nalu_id N,
 * edges E x 2, conn nelem x npe (node indices), area E x 3, dualvol N,
 * bnd_area N x 3 (lumped exposed area vectors; zero inside and on periodic
 * faces). Dual volumes and boundary areas are summed over periodic pairs
 * (master and slave hold the same total). */
nw_status nw_mesh_get(const nw_mesh* m, double* coords, int64_t* global_id,
                      int64_t* nalu_id, int64_t* edges, int64_t* conn,
                      double* area, double* dualvol, double* bnd_area);

/* Exposed-face integration points on the box sides selected by side_mask
 * (bit s: s = 0..5 for x-, x+, y-, y+, z-, z+; the sidesets surface_1 ..
 * surface_6 of a "generated:...|sideset:xXyYzZ" mesh; periodic sides have
 * none). One IP per face node, in side order, then element order, then
 * face-node order; faces are oriented outward. Outputs (any may be NULL):
 * ip_nodes count x 2 (face node, opposing element node), area count x 3
 * (exposed area vector of the IP's sub-face), side count. Call with NULL
 * outputs to get count. */
nw_status nw_mesh_face_ips(const nw_mesh* m, int side_mask, int64_t* count,
                           int64_t* ip_nodes, double* area, int32_t* side);

#ifdef __cplusplus
}
#endif
#endif /* NW_WORKLOAD_H */
