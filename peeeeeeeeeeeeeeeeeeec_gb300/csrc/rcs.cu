// RCS radiation vectors of solved edge currents, on the device.
//
// Reference (paths inside the reference project):
//   src/physics/rcs.c:238-362   integral over a triangle of exp(j k r_hat.r) dS
//                               (collapsed-square Gauss rule, cos / sin per point)
//   src/physics/rcs.c:364-533   the same over the edge's dual patches
//   src/physics/rcs.c:701-1000  F(r_hat) = sum_e (I_e / w_e) G_e(r_hat) e_hat,
//                               w_e = S_e / l_e, edges with l_e <= 0 or
//                               S_e <= 0 skipped (dual-patch quadrature mode)
//
// Many directions and many right-hand sides at once: G[d][e] (one warp per
// direction and edge, the points of all the edge's patches over the lanes)
// depends on the geometry only, and F[d][s] is then a sum over edges of
// G[d][e] times each solution's current (one warp per direction and
// solution) -- the config-3 form (720 plane waves) of the reference's
// per-direction, per-solution loop.  Everything is FP64, as the reference.
#include <math.h>

#include <vector>

#include "../../include/complex_matrix.h"
#include "../../include/dual_mesh.h"
#include "../../include/mesh.h"
#include "../../include/peec_gb300.h"
#include "common.cuh"
#include "gauss_legendre_table.h"
#include "geometry.cuh"

namespace peec {

__constant__ double c_rcs_x[GL_NUM_ORDERS][16];
__constant__ double c_rcs_w[GL_NUM_ORDERS][16];

struct RcsEdges {
    int ne;
    const int *off;          // [ne + 1] patch offsets
    const double *corner;    // [patches][12]
    const double *dir;       // [ne][3] unit edge direction
    const double *width;     // [ne] S_e / l_e, <= 0: edge skipped
};

// G[d][e] = sum over the edge's patches, triangles (0,1,2) and (0,2,3), of
// the order x order collapsed-square rule of exp(j k r_hat.r)
__global__ void k_rcs_g(RcsEdges E, const double *dirs, int n_dir, double k, int order, int row, double2 *G) {
    const int lane = threadIdx.x & 31;
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    if (w >= (long long)n_dir * E.ne) return;
    const int d = (int)(w / E.ne), e = (int)(w % E.ne);
    double re = 0.0, im = 0.0;
    if (E.width[e] > 0.0) {
        const double *rh = dirs + 3 * (size_t)d;
        const int oo = order * order, per = 2 * oo;
        const int p0 = E.off[e], np = E.off[e + 1] - p0;
        for (int t = lane; t < np * per; t += 32) {
            const int p = t / per, tri = (t / oo) & 1, iu = (t % oo) / order, iv = t % order;
            const double *c = E.corner + 12 * (size_t)(p0 + p);
            const double *a = c, *b = c + (tri == 0 ? 3 : 6), *q = c + (tri == 0 ? 6 : 9);
            const double u = 0.5 * (c_rcs_x[row][iu] + 1.0), wu = 0.5 * c_rcs_w[row][iu];
            const double v = 0.5 * (c_rcs_x[row][iv] + 1.0), wv = 0.5 * c_rcs_w[row][iv];
            double r[3], jac;
            tri_map(a, b, q, u, v, r, &jac);
            const double phase = k * dot3(rh, r);
            const double weight = wu * wv * jac;
            double s, co;
            sincos(phase, &s, &co);
            re += weight * co;
            im += weight * s;
        }
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if (lane == 0) G[(size_t)d * E.ne + e] = make_double2(re, im);
}

// F[d][s][c] = sum_e ((I_e / w_e) G[d][e]) e_hat_c
__global__ void k_rcs_f(RcsEdges E, const double2 *G, const double2 *cur, size_t stride, int n_dir, int n_rhs,
                        double2 *F) {
    const int lane = threadIdx.x & 31;
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    if (w >= (long long)n_dir * n_rhs) return;
    const int d = (int)(w / n_rhs), s = (int)(w % n_rhs);
    double f[6] = {0, 0, 0, 0, 0, 0};
    for (int e = lane; e < E.ne; e += 32) {
        const double wd = E.width[e];
        if (!(wd > 0.0)) continue;
        const double2 I = cur[(size_t)s * stride + e], g = G[(size_t)d * E.ne + e];
        const double cr = I.x / wd, ci = I.y / wd;
        const double sr = cr * g.x - ci * g.y, si = cr * g.y + ci * g.x;
        for (int c = 0; c < 3; ++c) {
            f[2 * c] += sr * E.dir[3 * e + c];
            f[2 * c + 1] += si * E.dir[3 * e + c];
        }
    }
    for (int c = 0; c < 6; ++c) f[c] = warp_sum(f[c]);
    if (lane == 0)
        for (int c = 0; c < 3; ++c) F[((size_t)d * n_rhs + s) * 3 + c] = make_double2(f[2 * c], f[2 * c + 1]);
}

}  // namespace peec

using namespace peec;

extern "C" int peec_gb300_rcs_radiation_device(const Mesh *mesh, const DualMesh *dual, const Complex *d_current,
                                               size_t n_rhs, size_t current_stride, double wave_number,
                                               const double *directions, size_t n_dir, int order,
                                               Complex *radiation) {
    if (!mesh || !dual || !d_current || !directions || !radiation || n_rhs == 0 || n_dir == 0) return -1;
    if (!mesh->edge_vectors || !dual->edge_patches || !dual->edge_region_areas || dual->n_edges != mesh->n_edges ||
        mesh->n_edges == 0 || mesh->n_edges > 0x7fffffff || current_stride < mesh->n_edges)
        return -1;
    if (!isfinite(wave_number) || wave_number <= 0.0) return -1;
    const int row = gl_row(order);
    if (row < 0 || n_dir > 0x7fffffff || n_rhs > 0x7fffffff) return -1;
    static const bool tables = cuda_ok(cudaMemcpyToSymbol(c_rcs_x, GL_NODES, sizeof(GL_NODES)), "GL table") &&
                               cuda_ok(cudaMemcpyToSymbol(c_rcs_w, GL_WEIGHTS, sizeof(GL_WEIGHTS)), "GL table");
    if (!tables) return -1;
    const int ne = (int)mesh->n_edges;
    // edge directions and widths as rcs.c:795-880 computes them
    std::vector<int> off(ne + 1, 0);
    std::vector<double> corner, dir(3 * (size_t)ne, 0.0), width(ne, 0.0);
    for (int e = 0; e < ne; ++e) {
        const double *ev = mesh->edge_vectors + 3 * (size_t)e;
        const double len = sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
        const PatchList &list = dual->edge_patches[e];
        off[e + 1] = off[e];
        if (!(len > 0.0)) continue;
        const double area = dual->edge_region_areas[e];
        if (!(area > 0.0)) continue;
        for (int c = 0; c < 3; ++c) dir[3 * (size_t)e + c] = ev[c] / len;
        width[e] = area / len;
        for (size_t q = 0; q < list.count; ++q)
            for (int k = 0; k < 12; ++k) corner.push_back(list.patches[q].points[k]);
        off[e + 1] = off[e] + (int)list.count;
    }
    for (size_t d = 0; d < 3 * n_dir; ++d)
        if (!isfinite(directions[d])) return -1;
    DBuf<int> d_off(ne + 1);
    DBuf<double> d_corner(corner.size()), d_dir(dir.size()), d_width(width.size()), d_dirs(3 * n_dir);
    DBuf<double2> d_G(n_dir * (size_t)ne), d_F(n_dir * n_rhs * 3);
    if (!d_off.p || (!corner.empty() && !d_corner.p) || !d_dir.p || !d_width.p || !d_dirs.p || !d_G.p || !d_F.p)
        return -1;
    if (!d_off.upload(off.data(), off.size()) || (!corner.empty() && !d_corner.upload(corner.data(), corner.size())) ||
        !d_dir.upload(dir.data(), dir.size()) || !d_width.upload(width.data(), width.size()) ||
        !d_dirs.upload(directions, 3 * n_dir))
        return -1;
    RcsEdges E{ne, d_off.p, d_corner.p, d_dir.p, d_width.p};
    const long long warps_g = (long long)n_dir * ne, warps_f = (long long)n_dir * (long long)n_rhs;
    PEEC_LAUNCH(k_rcs_g, (unsigned)((warps_g * 32 + 255) / 256), 256, 0, E, d_dirs.p, (int)n_dir, wave_number, order,
                row, d_G.p);
    PEEC_LAUNCH(k_rcs_f, (unsigned)((warps_f * 32 + 255) / 256), 256, 0, E, d_G.p,
                reinterpret_cast<const double2 *>(d_current), current_stride, (int)n_dir, (int)n_rhs, d_F.p);
    if (!d_F.download(reinterpret_cast<double2 *>(radiation), n_dir * n_rhs * 3)) return -1;
    return sync("RCS radiation vectors") ? 0 : -1;
}
