/*
 * Prints sizeof / offsetof of every struct the drop-in ABI shares with the
 * reference.  tests/test_relink.py compiles it once against the reference's
 * own headers and once against this repository's include/, and requires the
 * two outputs (and the ctypes declarations) to agree.
 */
#include <stddef.h>
#include <stdio.h>

#include "complex_lu.h"
#include "dual_mesh.h"
#include "incidence.h"
#include "inductance.h"
#include "lu.h"
#include "matrix.h"
#include "mesh.h"
#include "potential.h"
#include "resistance.h"

#define S(T) printf("%s %zu\n", #T, sizeof(T))
#define F(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))

int main(void)
{
    S(Mesh);
    F(Mesh, n_nodes); F(Mesh, n_quads); F(Mesh, n_edges); F(Mesh, xyz); F(Mesh, quads); F(Mesh, edges);
    F(Mesh, cell_edges); F(Mesh, cell_edge_signs); F(Mesh, edge_vectors); F(Mesh, edge_lengths);
    F(Mesh, edge_directions); F(Mesh, edge_centers); F(Mesh, cell_centers); F(Mesh, cell_areas);
    F(Mesh, cell_normals);
    S(QuadPatch); F(QuadPatch, points); F(QuadPatch, owner_id); F(QuadPatch, cell_id);
    S(PatchList); F(PatchList, patches); F(PatchList, count); F(PatchList, capacity);
    S(DualMesh);
    F(DualMesh, n_nodes); F(DualMesh, n_edges); F(DualMesh, node_patches); F(DualMesh, edge_patches);
    F(DualMesh, node_region_areas); F(DualMesh, edge_region_areas); F(DualMesh, node_region_centers);
    F(DualMesh, edge_region_centers);
    S(InductanceOptions);
    F(InductanceOptions, far_order); F(InductanceOptions, near_order); F(InductanceOptions, touching_order);
    F(InductanceOptions, self_order); F(InductanceOptions, near_factor); F(InductanceOptions, parallel_threads);
    F(InductanceOptions, direction_tolerance);
    S(InductanceMatrix); F(InductanceMatrix, n); F(InductanceMatrix, data);
    S(PotentialOptions);
    F(PotentialOptions, far_order); F(PotentialOptions, near_order); F(PotentialOptions, touching_order);
    F(PotentialOptions, self_order); F(PotentialOptions, near_factor); F(PotentialOptions, parallel_threads);
    S(PotentialMatrix); F(PotentialMatrix, n); F(PotentialMatrix, data);
    S(LUOptions); F(LUOptions, parallel_threads); F(LUOptions, pivot_tolerance); F(LUOptions, parallel_threshold);
    S(LUFactorization);
    F(LUFactorization, n); F(LUFactorization, data); F(LUFactorization, pivots); F(LUFactorization, swap_count);
    F(LUFactorization, matrix_scale); F(LUFactorization, factorized);
    S(Complex); F(Complex, re); F(Complex, im);
    S(ComplexLUOptions);
    F(ComplexLUOptions, parallel_threads); F(ComplexLUOptions, pivot_tolerance);
    F(ComplexLUOptions, parallel_threshold);
    S(ComplexLUFactorization);
    F(ComplexLUFactorization, n); F(ComplexLUFactorization, data); F(ComplexLUFactorization, pivots);
    F(ComplexLUFactorization, swap_count); F(ComplexLUFactorization, matrix_scale);
    F(ComplexLUFactorization, row_scale); F(ComplexLUFactorization, column_scale);
    F(ComplexLUFactorization, factorized);
    S(IncidenceMatrix); F(IncidenceMatrix, rows); F(IncidenceMatrix, cols); F(IncidenceMatrix, data);
    S(Matrix); F(Matrix, rows); F(Matrix, cols); F(Matrix, data);
    S(ResistanceMatrix); F(ResistanceMatrix, n); F(ResistanceMatrix, diagonal);
    return 0;
}
