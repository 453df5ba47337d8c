/*
 * Synthetic meshes, topology and dual mesh (host code, libpeec_mesh.so).
 *
 * Input preparation for tests and benchmarks: the GPU entry points take a
 * Mesh + DualMesh exactly as the reference's own mesh code produces them, and
 * this file reproduces that numbering and geometry so the index maps are
 * bit-identical:
 *   peec_synth_topology  follows reference src/mesh/topology.c:111-529
 *                        (first-seen edge numbering and orientation; the
 *                        lookup structure is free, only the order matters);
 *   peec_synth_dual      follows reference src/mesh/dual_mesh.c:356-692.
 * Floating-point expressions are written in the reference's evaluation order
 * and this file is compiled without FP contraction.
 */
#include "../../include/peec_synth_mesh.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* mesh construction                                                   */
/* ------------------------------------------------------------------ */

static void mesh_zero(Mesh *m) { memset(m, 0, sizeof(*m)); }

void peec_synth_mesh_free(Mesh *m)
{
    if (!m) return;
    free(m->xyz);
    free(m->quads);
    free(m->edges);
    free(m->cell_edges);
    free(m->cell_edge_signs);
    free(m->edge_vectors);
    free(m->edge_lengths);
    free(m->edge_directions);
    free(m->edge_centers);
    free(m->cell_centers);
    free(m->cell_areas);
    free(m->cell_normals);
    mesh_zero(m);
}

int peec_synth_from_arrays(const double *xyz, size_t n_nodes, const int *quads,
                           size_t n_quads, Mesh *m)
{
    if (!xyz || !quads || !m || n_nodes == 0 || n_quads == 0) return -1;
    mesh_zero(m);
    m->xyz = malloc(3 * n_nodes * sizeof(double));
    m->quads = malloc(4 * n_quads * sizeof(int));
    if (!m->xyz || !m->quads) {
        peec_synth_mesh_free(m);
        return -1;
    }
    memcpy(m->xyz, xyz, 3 * n_nodes * sizeof(double));
    memcpy(m->quads, quads, 4 * n_quads * sizeof(int));
    for (size_t t = 0; t < 4 * n_quads; ++t)
        if (quads[t] < 0 || (size_t)quads[t] >= n_nodes) {
            peec_synth_mesh_free(m);
            return -1;
        }
    m->n_nodes = n_nodes;
    m->n_quads = n_quads;
    return 0;
}

int peec_synth_plate(double lx, double ly, int nx, int ny, Mesh *m)
{
    if (!m || nx < 1 || ny < 1 || !(lx > 0.0) || !(ly > 0.0)) return -1;
    mesh_zero(m);
    size_t nn = (size_t)(nx + 1) * (size_t)(ny + 1), nq = (size_t)nx * (size_t)ny;
    m->xyz = malloc(3 * nn * sizeof(double));
    m->quads = malloc(4 * nq * sizeof(int));
    if (!m->xyz || !m->quads) {
        peec_synth_mesh_free(m);
        return -1;
    }
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            size_t v = (size_t)j * (size_t)(nx + 1) + (size_t)i;
            m->xyz[3 * v + 0] = lx * (double)i / (double)nx;
            m->xyz[3 * v + 1] = ly * (double)j / (double)ny;
            m->xyz[3 * v + 2] = 0.0;
        }
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            size_t c = (size_t)j * (size_t)nx + (size_t)i;
            int v00 = j * (nx + 1) + i;
            m->quads[4 * c + 0] = v00;
            m->quads[4 * c + 1] = v00 + 1;
            m->quads[4 * c + 2] = v00 + 1 + (nx + 1);
            m->quads[4 * c + 3] = v00 + (nx + 1);
        }
    m->n_nodes = nn;
    m->n_quads = nq;
    return 0;
}

/* Lattice-vertex id, created on first use. */
typedef struct {
    int nx, ny, nz;
    double lx, ly, lz;
    int *id;
    size_t count;
    double *xyz;
} Lattice;

static int lattice_vertex(Lattice *L, int i, int j, int k)
{
    size_t key = ((size_t)k * (size_t)(L->ny + 1) + (size_t)j) * (size_t)(L->nx + 1) + (size_t)i;
    if (L->id[key] < 0) {
        size_t v = L->count++;
        L->id[key] = (int)v;
        L->xyz[3 * v + 0] = L->lx * (double)i / (double)L->nx;
        L->xyz[3 * v + 1] = L->ly * (double)j / (double)L->ny;
        L->xyz[3 * v + 2] = L->lz * (double)k / (double)L->nz;
    }
    return L->id[key];
}

int peec_synth_box(double lx, double ly, double lz, int nx, int ny, int nz, Mesh *m)
{
    if (!m || nx < 1 || ny < 1 || nz < 1 || !(lx > 0.0) || !(ly > 0.0) || !(lz > 0.0))
        return -1;
    mesh_zero(m);
    size_t lattice = (size_t)(nx + 1) * (size_t)(ny + 1) * (size_t)(nz + 1);
    size_t nq = 2 * ((size_t)nx * ny + (size_t)nx * nz + (size_t)ny * nz);
    size_t nn = nq + 2; /* closed genus-0 quad surface: V = F + 2 */
    Lattice L = {nx, ny, nz, lx, ly, lz, malloc(lattice * sizeof(int)), 0,
                 malloc(3 * nn * sizeof(double))};
    m->quads = malloc(4 * nq * sizeof(int));
    if (!L.id || !L.xyz || !m->quads) {
        free(L.id);
        free(L.xyz);
        peec_synth_mesh_free(m);
        return -1;
    }
    for (size_t t = 0; t < lattice; ++t) L.id[t] = -1;
    size_t c = 0;
#define QUAD(a0, a1, a2, a3)                      \
    do {                                          \
        m->quads[4 * c + 0] = (a0);               \
        m->quads[4 * c + 1] = (a1);               \
        m->quads[4 * c + 2] = (a2);               \
        m->quads[4 * c + 3] = (a3);               \
        ++c;                                      \
    } while (0)
    /* -z: normal -z */
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            int a = lattice_vertex(&L, i, j, 0), b = lattice_vertex(&L, i, j + 1, 0);
            int d = lattice_vertex(&L, i + 1, j + 1, 0), e = lattice_vertex(&L, i + 1, j, 0);
            QUAD(a, b, d, e);
        }
    /* +z */
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            int a = lattice_vertex(&L, i, j, nz), b = lattice_vertex(&L, i + 1, j, nz);
            int d = lattice_vertex(&L, i + 1, j + 1, nz), e = lattice_vertex(&L, i, j + 1, nz);
            QUAD(a, b, d, e);
        }
    /* -y */
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
            int a = lattice_vertex(&L, i, 0, k), b = lattice_vertex(&L, i + 1, 0, k);
            int d = lattice_vertex(&L, i + 1, 0, k + 1), e = lattice_vertex(&L, i, 0, k + 1);
            QUAD(a, b, d, e);
        }
    /* +y */
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
            int a = lattice_vertex(&L, i, ny, k), b = lattice_vertex(&L, i, ny, k + 1);
            int d = lattice_vertex(&L, i + 1, ny, k + 1), e = lattice_vertex(&L, i + 1, ny, k);
            QUAD(a, b, d, e);
        }
    /* -x */
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            int a = lattice_vertex(&L, 0, j, k), b = lattice_vertex(&L, 0, j, k + 1);
            int d = lattice_vertex(&L, 0, j + 1, k + 1), e = lattice_vertex(&L, 0, j + 1, k);
            QUAD(a, b, d, e);
        }
    /* +x */
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            int a = lattice_vertex(&L, nx, j, k), b = lattice_vertex(&L, nx, j + 1, k);
            int d = lattice_vertex(&L, nx, j + 1, k + 1), e = lattice_vertex(&L, nx, j, k + 1);
            QUAD(a, b, d, e);
        }
#undef QUAD
    free(L.id);
    if (L.count != nn || c != nq) {
        free(L.xyz);
        peec_synth_mesh_free(m);
        return -1;
    }
    m->xyz = L.xyz;
    m->n_nodes = nn;
    m->n_quads = nq;
    return 0;
}

/* ------------------------------------------------------------------ */
/* topology (reference topology.c:111-529)                             */
/* ------------------------------------------------------------------ */

typedef struct {
    uint64_t key; /* (lo << 32) | hi, 0 = empty slot (lo < hi so never 0 for a real edge) */
    int id;
} EdgeSlot;

static size_t slot_of(uint64_t key, size_t mask)
{
    /* Fibonacci hashing of the packed vertex pair */
    return (size_t)((key * UINT64_C(0x9E3779B97F4A7C15)) >> 20) & mask;
}

int peec_synth_topology(Mesh *m)
{
    if (!m || !m->xyz || !m->quads) return -1;
    size_t nq = m->n_quads;
    m->edges = malloc(8 * nq * sizeof(int));
    m->cell_edges = malloc(4 * nq * sizeof(int));
    m->cell_edge_signs = malloc(4 * nq * sizeof(int));
    size_t cap = 16;
    while (cap < 8 * nq) cap <<= 1;
    EdgeSlot *table = calloc(cap, sizeof(EdgeSlot));
    if (!m->edges || !m->cell_edges || !m->cell_edge_signs || !table) {
        free(table);
        fprintf(stderr, "ERROR: cannot allocate topology arrays.\n");
        return -1;
    }
    size_t ne = 0;
    for (size_t c = 0; c < nq; ++c) {
        const int *q = &m->quads[4 * c];
        for (int s = 0; s < 4; ++s) {
            int a = q[s], b = q[(s + 1) % 4];
            if (a == b) {
                free(table);
                fprintf(stderr, "ERROR: degenerate cell side in cell %zu.\n", c);
                return -1;
            }
            uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
            uint64_t key = ((uint64_t)lo << 32) | (uint64_t)hi;
            size_t slot = slot_of(key, cap - 1);
            while (table[slot].key != 0 && table[slot].key != key) slot = (slot + 1) & (cap - 1);
            if (table[slot].key == 0) {
                table[slot].key = key;
                table[slot].id = (int)ne;
                m->edges[2 * ne + 0] = a;
                m->edges[2 * ne + 1] = b;
                m->cell_edges[4 * c + s] = (int)ne;
                m->cell_edge_signs[4 * c + s] = +1;
                ++ne;
            } else {
                int e = table[slot].id;
                int sign = (m->edges[2 * e] == a && m->edges[2 * e + 1] == b) ? +1 : -1;
                m->cell_edges[4 * c + s] = e;
                m->cell_edge_signs[4 * c + s] = sign;
            }
        }
    }
    free(table);
    m->n_edges = ne;
    int *shrunk = realloc(m->edges, 2 * ne * sizeof(int));
    if (shrunk) m->edges = shrunk;
    m->edge_vectors = malloc(3 * ne * sizeof(double));
    m->edge_lengths = malloc(ne * sizeof(double));
    m->edge_directions = malloc(3 * ne * sizeof(double));
    m->edge_centers = malloc(3 * ne * sizeof(double));
    m->cell_centers = malloc(3 * nq * sizeof(double));
    m->cell_areas = malloc(nq * sizeof(double));
    m->cell_normals = malloc(3 * nq * sizeof(double));
    if (!m->edge_vectors || !m->edge_lengths || !m->edge_directions || !m->edge_centers
        || !m->cell_centers || !m->cell_areas || !m->cell_normals) {
        fprintf(stderr, "ERROR: cannot allocate mesh geometry arrays.\n");
        return -1;
    }
    for (size_t e = 0; e < ne; ++e) {
        const double *pa = &m->xyz[3 * m->edges[2 * e]];
        const double *pb = &m->xyz[3 * m->edges[2 * e + 1]];
        double dx = pb[0] - pa[0], dy = pb[1] - pa[1], dz = pb[2] - pa[2];
        double len = sqrt(dx * dx + dy * dy + dz * dz);
        if (len <= 0.0) {
            fprintf(stderr, "ERROR: zero-length edge %zu.\n", e);
            return -1;
        }
        m->edge_vectors[3 * e + 0] = dx;
        m->edge_vectors[3 * e + 1] = dy;
        m->edge_vectors[3 * e + 2] = dz;
        m->edge_lengths[e] = len;
        m->edge_directions[3 * e + 0] = dx / len;
        m->edge_directions[3 * e + 1] = dy / len;
        m->edge_directions[3 * e + 2] = dz / len;
        m->edge_centers[3 * e + 0] = 0.5 * (pa[0] + pb[0]);
        m->edge_centers[3 * e + 1] = 0.5 * (pa[1] + pb[1]);
        m->edge_centers[3 * e + 2] = 0.5 * (pa[2] + pb[2]);
    }
    for (size_t c = 0; c < nq; ++c) {
        const int *q = &m->quads[4 * c];
        double p[4][3];
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) p[k][d] = m->xyz[3 * q[k] + d];
        for (int d = 0; d < 3; ++d)
            m->cell_centers[3 * c + d] = 0.25 * (p[0][d] + p[1][d] + p[2][d] + p[3][d]);
        double u[3], v[3], w[3], c1[3], c2[3];
        for (int d = 0; d < 3; ++d) {
            u[d] = p[1][d] - p[0][d];
            v[d] = p[2][d] - p[0][d];
            w[d] = p[3][d] - p[0][d];
        }
        c1[0] = u[1] * v[2] - u[2] * v[1];
        c1[1] = u[2] * v[0] - u[0] * v[2];
        c1[2] = u[0] * v[1] - u[1] * v[0];
        c2[0] = v[1] * w[2] - v[2] * w[1];
        c2[1] = v[2] * w[0] - v[0] * w[2];
        c2[2] = v[0] * w[1] - v[1] * w[0];
        double n1 = sqrt(c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2]);
        double n2 = sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2]);
        m->cell_areas[c] = 0.5 * (n1 + n2);
        double nx = c1[0] + c2[0], ny = c1[1] + c2[1], nz = c1[2] + c2[2];
        double nl = sqrt(nx * nx + ny * ny + nz * nz);
        if (nl > 0.0) {
            nx /= nl;
            ny /= nl;
            nz /= nl;
        }
        m->cell_normals[3 * c + 0] = nx;
        m->cell_normals[3 * c + 1] = ny;
        m->cell_normals[3 * c + 2] = nz;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* dual mesh (reference dual_mesh.c:356-692)                           */
/* ------------------------------------------------------------------ */

void peec_synth_dual_free(DualMesh *d)
{
    if (!d) return;
    if (d->node_patches)
        for (size_t i = 0; i < d->n_nodes; ++i) free(d->node_patches[i].patches);
    if (d->edge_patches)
        for (size_t i = 0; i < d->n_edges; ++i) free(d->edge_patches[i].patches);
    free(d->node_patches);
    free(d->edge_patches);
    free(d->node_region_areas);
    free(d->edge_region_areas);
    free(d->node_region_centers);
    free(d->edge_region_centers);
    memset(d, 0, sizeof(*d));
}

static int append_patch(PatchList *list, const double *c0, const double *c1,
                        const double *c2, const double *c3, int owner, int cell)
{
    if (list->count >= list->capacity) {
        size_t cap = list->capacity == 0 ? 4 : 2 * list->capacity;
        QuadPatch *grown = realloc(list->patches, cap * sizeof(QuadPatch));
        if (!grown) return -1;
        list->patches = grown;
        list->capacity = cap;
    }
    QuadPatch *p = &list->patches[list->count++];
    const double *c[4] = {c0, c1, c2, c3};
    for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) p->points[3 * k + d] = c[k][d];
    p->owner_id = owner;
    p->cell_id = cell;
    return 0;
}

static double patch_area(const QuadPatch *p)
{
    const double *q = p->points;
    double u[3], v[3], w[3], c1[3], c2[3];
    for (int d = 0; d < 3; ++d) {
        u[d] = q[3 + d] - q[d];
        v[d] = q[6 + d] - q[d];
        w[d] = q[9 + d] - q[d];
    }
    c1[0] = u[1] * v[2] - u[2] * v[1];
    c1[1] = u[2] * v[0] - u[0] * v[2];
    c1[2] = u[0] * v[1] - u[1] * v[0];
    c2[0] = v[1] * w[2] - v[2] * w[1];
    c2[1] = v[2] * w[0] - v[0] * w[2];
    c2[2] = v[0] * w[1] - v[1] * w[0];
    double a1 = 0.5 * sqrt(c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2]);
    double a2 = 0.5 * sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2]);
    return a1 + a2;
}

static void region_totals(const PatchList *list, double *area, double centre[3])
{
    double total = 0.0, wc[3] = {0.0, 0.0, 0.0};
    for (size_t k = 0; k < list->count; ++k) {
        const double *q = list->patches[k].points;
        double a = patch_area(&list->patches[k]);
        total += a;
        for (int d = 0; d < 3; ++d) wc[d] += a * (0.25 * (q[d] + q[3 + d] + q[6 + d] + q[9 + d]));
    }
    *area = total;
    if (total > 0.0)
        for (int d = 0; d < 3; ++d) centre[d] = wc[d] / total;
}

int peec_synth_dual(const Mesh *m, DualMesh *d)
{
    if (!m || !d || !m->xyz || !m->quads || !m->cell_edges) {
        fprintf(stderr, "ERROR: topology must be built before dual mesh.\n");
        return -1;
    }
    memset(d, 0, sizeof(*d));
    d->n_nodes = m->n_nodes;
    d->n_edges = m->n_edges;
    d->node_patches = calloc(m->n_nodes, sizeof(PatchList));
    d->edge_patches = calloc(m->n_edges, sizeof(PatchList));
    d->node_region_areas = calloc(m->n_nodes, sizeof(double));
    d->edge_region_areas = calloc(m->n_edges, sizeof(double));
    d->node_region_centers = calloc(3 * m->n_nodes, sizeof(double));
    d->edge_region_centers = calloc(3 * m->n_edges, sizeof(double));
    if (!d->node_patches || !d->edge_patches || !d->node_region_areas
        || !d->edge_region_areas || !d->node_region_centers || !d->edge_region_centers) {
        peec_synth_dual_free(d);
        return -1;
    }
    for (size_t c = 0; c < m->n_quads; ++c) {
        const int *q = &m->quads[4 * c];
        double p[4][3], mid[4][3], ctr[3];
        for (int k = 0; k < 4; ++k)
            for (int x = 0; x < 3; ++x) p[k][x] = m->xyz[3 * q[k] + x];
        /* mid[k] = midpoint of side k -> k+1 */
        for (int k = 0; k < 4; ++k)
            for (int x = 0; x < 3; ++x) mid[k][x] = 0.5 * (p[k][x] + p[(k + 1) % 4][x]);
        for (int x = 0; x < 3; ++x) ctr[x] = 0.25 * (p[0][x] + p[1][x] + p[2][x] + p[3][x]);
        int ci = (int)c, fail = 0;
        /* vertex k: [p_k, mid_k, centre, mid_{k-1}] */
        for (int k = 0; k < 4; ++k)
            fail |= append_patch(&d->node_patches[q[k]], p[k], mid[k], ctr, mid[(k + 3) % 4],
                                 q[k], ci);
        /* side k (p_k -> p_{k+1}): [p_k, p_{k+1}, mid_{k+1}, mid_{k+3}] */
        for (int k = 0; k < 4; ++k) {
            int e = m->cell_edges[4 * c + k];
            fail |= append_patch(&d->edge_patches[e], p[k], p[(k + 1) % 4], mid[(k + 1) % 4],
                                 mid[(k + 3) % 4], e, ci);
        }
        if (fail) {
            fprintf(stderr, "ERROR: cannot allocate dual mesh patch.\n");
            peec_synth_dual_free(d);
            return -1;
        }
    }
    for (size_t v = 0; v < d->n_nodes; ++v)
        region_totals(&d->node_patches[v], &d->node_region_areas[v], &d->node_region_centers[3 * v]);
    for (size_t e = 0; e < d->n_edges; ++e)
        region_totals(&d->edge_patches[e], &d->edge_region_areas[e], &d->edge_region_centers[3 * e]);
    return 0;
}
