/*
 * Dual-mesh geometry: the quadrilateral patches whose pairwise 1/R integrals
 * fill Lp and P.
 *
 * Layout-compatible with the reference's QuadPatch / PatchList / DualMesh
 * (include/dual_mesh.h:25-89 of the reference project).  Node regions are
 * unions of quarter-quads around a vertex, edge regions unions of half-quads
 * beside an edge.  Only the types live here.
 */
#ifndef PEEC_DUAL_MESH_H
#define PEEC_DUAL_MESH_H

#include "mesh.h"

#include <stddef.h>

typedef struct
{
    double points[12];   /* 4 corners, x0 y0 z0 x1 y1 z1 ... (metres)  */
    int owner_id;        /* node or edge the patch belongs to          */
    int cell_id;         /* source quad cell                           */
} QuadPatch;             /* 104 bytes                                  */

typedef struct
{
    QuadPatch *patches;
    size_t count;
    size_t capacity;
} PatchList;

typedef struct
{
    size_t n_nodes;
    size_t n_edges;

    PatchList *node_patches;      /* [n_nodes] */
    PatchList *edge_patches;      /* [n_edges] */

    double *node_region_areas;    /* [n_nodes]   */
    double *edge_region_areas;    /* [n_edges]   */

    double *node_region_centers;  /* [3*n_nodes] */
    double *edge_region_centers;  /* [3*n_edges] */
} DualMesh;

#endif
