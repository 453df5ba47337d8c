/*
 * Seeded synthetic PEEC meshes for tests and benchmarks (host code).
 *
 * Builds a Mesh directly (no Gmsh file) and derives its topology and dual
 * mesh with the same numbering rules as the reference:
 *   - unique edges numbered in first-seen order over cells and local sides
 *     (q0q1, q1q2, q2q3, q3q0), oriented as first seen
 *     (reference src/mesh/topology.c:111-304);
 *   - node regions from quarter-quads, edge regions from half-quads, appended
 *     cell by cell (reference src/mesh/dual_mesh.c:356-692).
 * The results are layout-compatible Mesh / DualMesh structs that the GPU
 * entry points (and the reference's own code) accept.  Names are prefixed so
 * the library can sit beside the reference's mesh_* / dual_mesh_* symbols.
 */
#ifndef PEEC_SYNTH_MESH_H
#define PEEC_SYNTH_MESH_H

#include "dual_mesh.h"
#include "mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Flat plate [0,lx] x [0,ly] in z = 0 with nx x ny cells; vertex (i,j) has id
 * j*(nx+1)+i; cells row-major, counter-clockwise seen from +z.  Fills xyz and
 * quads only; call peec_synth_topology() next.  0 ok, -1 bad arguments. */
int peec_synth_plate(double lx, double ly, int nx, int ny, Mesh *mesh);

/* Closed axis-aligned box [0,lx]x[0,ly]x[0,lz] with nx, ny, nz cells along
 * the axes, every face wound counter-clockwise seen from outside.  Vertices
 * are numbered in first-seen order over the faces -z, +z, -y, +y, -x, +x. */
int peec_synth_box(double lx, double ly, double lz, int nx, int ny, int nz, Mesh *mesh);

/* Copies caller arrays into a fresh Mesh (xyz[3*n_nodes], quads[4*n_quads]). */
int peec_synth_from_arrays(const double *xyz, size_t n_nodes, const int *quads,
                           size_t n_quads, Mesh *mesh);

/* Edges, cell-edge maps and signs, edge and cell geometry. */
int peec_synth_topology(Mesh *mesh);

/* Quarter-quad node regions and half-quad edge regions with their areas and
 * area-weighted centres. */
int peec_synth_dual(const Mesh *mesh, DualMesh *dual);

void peec_synth_mesh_free(Mesh *mesh);
void peec_synth_dual_free(DualMesh *dual);

#ifdef __cplusplus
}
#endif

#endif
