// Patch geometry shared by host and device.
//
// Every expression is written in the reference's evaluation order
// (src/peec/quadrature.c of the reference project) and the library is built
// with --fmad=false, so host and device produce the same bits for the
// classification and the triangle maps.
#pragma once

#include <math.h>

#include "gauss_legendre_table.h"

#define PEEC_HD __host__ __device__ __forceinline__

namespace peec {

enum PairClass { CLS_SELF = 0, CLS_TOUCHING = 1, CLS_NEAR = 2, CLS_FAR = 3 };

PEEC_HD double dist3(const double *a, const double *b) {
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

PEEC_HD void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

PEEC_HD double norm3(const double *a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

PEEC_HD double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// vertices coincide within 1e-12 m (reference quadrature.c:80-86)
PEEC_HD bool same_point(const double *a, const double *b) { return dist3(a, b) <= 1.0e-12; }

// longest side of a 4-corner patch (reference quadrature.c:384-416)
PEEC_HD double patch_size(const double *c) {
    double longest = 0.0;
    for (int i = 0; i < 4; ++i) {
        double s = dist3(c + 3 * i, c + 3 * ((i + 1) % 4));
        if (s > longest) longest = s;
    }
    return longest;
}

// number of a's corners that coincide with some corner of b (quadrature.c:466-496)
PEEC_HD int shared_corners(const double *a, const double *b) {
    int shared = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            if (same_point(a + 3 * i, b + 3 * j)) {
                ++shared;
                break;
            }
    return shared;
}

// one-to-one corner matching (quadrature.c:503-542)
PEEC_HD bool same_corner_set(const double *a, const double *b) {
    bool used[4] = {false, false, false, false};
    for (int i = 0; i < 4; ++i) {
        bool hit = false;
        for (int j = 0; j < 4 && !hit; ++j) {
            if (used[j]) continue;
            if (same_point(a + 3 * i, b + 3 * j)) {
                used[j] = true;
                hit = true;
            }
        }
        if (!hit) return false;
    }
    return true;
}

// bounding box [min xyz, max xyz] with the reference's fmin/fmax sweep
PEEC_HD void patch_aabb(const double *c, double *box) {
    for (int k = 0; k < 3; ++k) {
        double lo = c[k], hi = lo;
        for (int i = 1; i < 4; ++i) {
            lo = fmin(lo, c[3 * i + k]);
            hi = fmax(hi, c[3 * i + k]);
        }
        box[k] = lo;
        box[3 + k] = hi;
    }
}

// Pair class (reference quadrature.c:550-607).  `same_object` stands for the
// reference's pointer test a == b.  When the bounding boxes are more than
// 2e-12 m apart no pair of corners can lie within 1e-12 m, so the corner
// tests are skipped; the outcome is identical.
PEEC_HD int classify_pair(const double *ca, const double *boxa, double ha, const double *cb,
                          const double *boxb, double hb, double near_factor, bool same_object) {
    if (same_object) return CLS_SELF;
    double gap2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        double g = fmax(0.0, fmax(boxa[k] - boxb[3 + k], boxb[k] - boxa[3 + k]));
        gap2 += g * g;
    }
    double gap = sqrt(gap2);
    if (!(gap > 2.0e-12)) {
        if (same_corner_set(ca, cb)) return CLS_SELF;
        if (shared_corners(ca, cb) > 0) return CLS_TOUCHING;
    }
    double h = (ha > hb) ? ha : hb;
    if (h > 0.0 && gap < near_factor * h) return CLS_NEAR;
    return CLS_FAR;
}

// Collapsed-square map of the unit square onto triangle (p0,p1,p2):
// xi = u, eta = (1-u) v, r = p0 + xi e1 + eta e2, J = |e1 x e2| (1-u)
// (reference quadrature.c:632-666).
PEEC_HD void tri_map(const double *p0, const double *p1, const double *p2, double u, double v,
                     double *r, double *jac) {
    double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double xi = u, eta = (1.0 - u) * v;
    for (int k = 0; k < 3; ++k) r[k] = p0[k] + xi * e1[k] + eta * e2[k];
    double n[3];
    cross3(e1, e2, n);
    *jac = norm3(n) * (1.0 - u);
}

PEEC_HD int gl_row(int order) {
    switch (order) {
        case 2: return 0;
        case 3: return 1;
        case 4: return 2;
        case 5: return 3;
        case 6: return 4;
        case 8: return 5;
        case 10: return 6;
        case 12: return 7;
        case 16: return 8;
        default: return -1;
    }
}

}  // namespace peec
