// The small potential.h helpers on the GPU and the *_print_info diagnostics.
//
// Reference (paths inside the reference project):
//   src/peec/potential.c:483-520  potential_build_self_capacitance   F_j = 1/P_jj
//   src/peec/potential.c:528-559  potential_self_voltage_to_charge   q_j = V_j/P_jj
//   src/peec/potential.c:567-612  potential_self_voltage_to_full_potential
//                                  phi_j = sum_a P_ja V_a / P_aa
//   src/peec/inductance.c:568-646, potential.c:403-475  print_info
#include <math.h>
#include <stdio.h>

#include "../../include/inductance.h"
#include "../../include/potential.h"
#include "common.cuh"

namespace peec {

// diag[j] must be finite and > 0, else flag = 1 (first offender in *bad)
__global__ void k_diag_ratio(const double *diag, const double *num, double *out, int n, int *bad) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double d = diag[j];
    if (!isfinite(d) || d <= 0.0) {
        atomicMin(bad, j);
        return;
    }
    out[j] = num ? num[j] / d : 1.0 / d;
}

// phi_j = sum_a P_ja (V_a / P_aa), one warp per row, accumulated in index
// order per lane and reduced by shuffles
__global__ void k_full_potential(const double *P, const double *v, int n, double *phi, int *bad) {
    int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    double acc = 0.0;
    for (int a = lane; a < n; a += 32) {
        double d = P[(size_t)a * n + a];
        if (!isfinite(d) || d <= 0.0) {
            atomicMin(bad, a);
            continue;
        }
        acc += P[(size_t)row * n + a] * v[a] / d;
    }
    acc = warp_sum(acc);
    if (lane == 0) phi[row] = acc;
}

static int diag_op(const PotentialMatrix *P, const double *num, double *out) {
    if (!P || !P->data || P->n == 0 || !out) return -1;
    int n = (int)P->n;
    DBuf<double> dd(n), dn(num ? n : 0), dout(n);
    DBuf<int> bad(1);
    if (!dd.p || !dout.p || !bad.p || (num && !dn.p)) return -1;
    // strided copy of the diagonal
    if (!cuda_ok(cudaMemcpy2DAsync(dd.p, sizeof(double), P->data, (P->n + 1) * sizeof(double), sizeof(double), n,
                                   cudaMemcpyHostToDevice, stream()),
                 "diagonal upload"))
        return -1;
    if (num && !dn.upload(num, n)) return -1;
    int init = n;
    cudaMemcpyAsync(bad.p, &init, sizeof(int), cudaMemcpyHostToDevice, stream());
    PEEC_LAUNCH(k_diag_ratio, (n + 255) / 256, 256, 0, dd.p, num ? dn.p : nullptr, dout.p, n, bad.p);
    int hb = n;
    cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!sync("potential helper")) return -1;
    if (hb < n) return -2 - hb;  // encoded offender
    if (!dout.download(out, n) || !sync("potential helper")) return -1;
    return 0;
}

}  // namespace peec

using namespace peec;

extern "C" {

int potential_build_self_capacitance(const PotentialMatrix *P, double *F) {
    int s = diag_op(P, nullptr, F);
    if (s <= -2) {
        size_t j = (size_t)(-2 - s);
        fprintf(stderr, "ERROR: invalid diagonal P[%zu,%zu] in potential_build_self_capacitance().\n", j, j);
        return -1;
    }
    return s;
}

int potential_self_voltage_to_charge(const PotentialMatrix *P, const double *V_c, double *charge) {
    if (!V_c) return -1;
    int s = diag_op(P, V_c, charge);
    return s == 0 ? 0 : -1;
}

int potential_self_voltage_to_full_potential(const PotentialMatrix *P, const double *V_c, double *phi) {
    if (!P || !P->data || P->n == 0 || !V_c || !phi) return -1;
    int n = (int)P->n;
    size_t nn = (size_t)n * n;
    DBuf<double> dP(nn), dv(n), dphi(n);
    DBuf<int> bad(1);
    if (!dP.p || !dv.p || !dphi.p || !bad.p) return -1;
    if (!dP.upload(P->data, nn) || !dv.upload(V_c, n)) return -1;
    int init = n;
    cudaMemcpyAsync(bad.p, &init, sizeof(int), cudaMemcpyHostToDevice, stream());
    PEEC_LAUNCH(k_full_potential, (unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, dP.p, dv.p, n, dphi.p, bad.p);
    int hb = n;
    cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!sync("full potential")) return -1;
    if (hb < n) return -1;
    if (!dphi.download(phi, n) || !sync("full potential")) return -1;
    return 0;
}

// Diagnostics: summary statistics of a host matrix, printed to stdout.
static void print_matrix_info(const char *title, const char *unit, size_t n, const double *data) {
    double mn = data[0], mx = data[0], dmn = HUGE_VAL, dmx = -HUGE_VAL, sym = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double d = data[i * n + i];
        if (d < dmn) dmn = d;
        if (d > dmx) dmx = d;
        for (size_t j = 0; j < n; ++j) {
            double v = data[i * n + j];
            if (v < mn) mn = v;
            if (v > mx) mx = v;
            double e = fabs(v - data[j * n + i]);
            if (e > sym) sym = e;
        }
    }
    printf("\n========================================\n%s\n========================================\n", title);
    printf("Size               : %zu x %zu\n", n, n);
    printf("Memory             : %.3f MiB\n", (double)n * (double)n * sizeof(double) / (1024.0 * 1024.0));
    printf("Minimum            : %.9e %s\n", mn, unit);
    printf("Maximum            : %.9e %s\n", mx, unit);
    printf("Minimum diagonal   : %.9e %s\n", dmn, unit);
    printf("Maximum diagonal   : %.9e %s\n", dmx, unit);
    printf("Max symmetry error : %.3e %s\n", sym, unit);
    printf("========================================\n");
}

void inductance_print_info(const InductanceMatrix *L) {
    if (!L || !L->data || L->n == 0) return;
    print_matrix_info("INDUCTANCE MATRIX (GPU)", "H", L->n, L->data);
}

void potential_print_info(const PotentialMatrix *P) {
    if (!P || !P->data || P->n == 0) return;
    print_matrix_info("POTENTIAL MATRIX (GPU)", "1/F", P->n, P->data);
}

}  // extern "C"
