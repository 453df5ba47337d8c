/*
 * 1/R panel quadrature: the kernel underneath every Lp and P entry.
 *
 *     K(a,b) = \int_{Pi_a} \int_{Pi_b} 1/|r - r'| dS dS'
 *
 * Drop-in for the reference's include/quadrature.h (declarations at
 * quadrature.h:55-218 of the reference project).  In this library the
 * pair kernel quad_patch_kernel_1_over_r() runs on the GPU (sm_103a); the
 * small geometric helpers are host functions shared with the device code.
 */
#ifndef PEEC_QUADRATURE_H
#define PEEC_QUADRATURE_H

#include "dual_mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Patch-pair class; decides which integration scheme is used.
 * Replaces the reference's QuadPairType (quadrature.h:19-55). */
typedef enum
{
    QUAD_PAIR_SELF = 0,   /* same patch, or the same four vertices          */
    QUAD_PAIR_TOUCHING,   /* at least one shared vertex (within 1e-12 m)     */
    QUAD_PAIR_NEAR,       /* bounding-box gap < near_factor * max side       */
    QUAD_PAIR_FAR         /* everything else: plain Gauss-Legendre product   */
} QuadPairType;

/* Orders with a tabulated Gauss-Legendre rule (reference quadrature.h:85-89). */
static inline int gauss_legendre_order_supported(int order)
{
    return order == 2 || order == 3 || order == 4 || order == 5 || order == 6
        || order == 8 || order == 10 || order == 12 || order == 16;
}

/* Nodes x[] and weights w[] on [-1,1]; 0 on success, -1 for an unsupported
 * order or NULL output (reference quadrature.c:94-313). */
int gauss_legendre_rule(int order, double *x, double *w);

/* 0.5*|(p1-p0) x (p2-p0)| (reference quadrature.c:321-345). */
double triangle_area(const double p0[3], const double p1[3], const double p2[3]);

/* Area of the split (0,1,2)+(0,2,3); 0 for NULL (reference quadrature.c:352-376). */
double quad_patch_area(const QuadPatch *patch);

/* Longest of the four sides; 0 for NULL (reference quadrature.c:384-416). */
double quad_patch_size(const QuadPatch *patch);

/* Smallest vertex-to-vertex distance; 0 for NULL (reference quadrature.c:424-458). */
double quad_patch_min_vertex_distance(const QuadPatch *a, const QuadPatch *b);

/* SELF / TOUCHING / NEAR / FAR; FAR for NULL (reference quadrature.c:550-607). */
QuadPairType quad_patch_classify_pair(const QuadPatch *a, const QuadPatch *b,
                                      double near_factor);

/* K(a,b) for one patch pair, evaluated on the GPU.  Returns NaN for NULL
 * patches, unsupported orders, a negative or non-finite near_factor, or an
 * adaptive refinement that failed to converge within depth 24
 * (reference quadrature.c:975-1079). */
double quad_patch_kernel_1_over_r(const QuadPatch *a, const QuadPatch *b,
                                  int far_order, int near_order,
                                  int touching_order, int self_order,
                                  double near_factor);

#ifdef __cplusplus
}
#endif

#endif
