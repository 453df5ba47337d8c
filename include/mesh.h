/*
 * Surface quad mesh as the PEEC hot path consumes it.
 *
 * Layout-compatible with the reference's `Mesh` (include/mesh.h:12-150 of the
 * reference project): the same members in the same order, so a Mesh built by
 * the reference's Gmsh reader and topology code can be passed straight to the
 * GPU assembly entry points.  Only the type lives here; the reference's own
 * mesh_* functions are not part of the GPU library.
 */
#ifndef PEEC_MESH_H
#define PEEC_MESH_H

#include <stddef.h>

typedef struct
{
    size_t n_nodes;          /* vertices                                   */
    size_t n_quads;          /* quad cells                                 */
    size_t n_edges;          /* unique edges, first-seen order             */

    double *xyz;             /* [3*n_nodes]  vertex coordinates, metres    */
    int *quads;              /* [4*n_quads]  vertex ids per cell           */
    int *edges;              /* [2*n_edges]  (a,b), current flows a -> b   */
    int *cell_edges;         /* [4*n_quads]  global edge id per cell side  */
    int *cell_edge_signs;    /* [4*n_quads]  +1/-1 local vs global sense   */

    double *edge_vectors;    /* [3*n_edges]  r_b - r_a                     */
    double *edge_lengths;    /* [n_edges]                                  */
    double *edge_directions; /* [3*n_edges]  unit vectors                  */
    double *edge_centers;    /* [3*n_edges]                                */

    double *cell_centers;    /* [3*n_quads]                                */
    double *cell_areas;      /* [n_quads]                                  */
    double *cell_normals;    /* [3*n_quads]                                */
} Mesh;

#endif
