// Batched frequency sweep: the harmonic systems of one mesh at many
// frequencies, each solved by the mixed-precision solve in its graph form.
//
// The whole per-frequency sequence -- MNA fill Z = [R + j w L, A; -P A^T,
// j w I] (harmonic.c:175-372), the nrhs plane-wave right-hand sides
// (scattering.c:263-336), power-of-two equilibration, FP32 LU with
// split-BF16 tcgen05 trailing updates, a fixed number of FP64 refinement
// sweeps -- is recorded once into a CUDA graph (its scratch as graph
// allocations) and replayed for every frequency; omega and k0 live in
// device memory and are copied in before each replay, so one graph serves
// the whole sweep.  Different meshes run their plans from different host
// threads (each thread has its own stream), so their graphs overlap on the
// device.  Systems that the fast graph leaves above the tolerance are
// replayed with the robust graph; those still above it are solved again
// outside the graphs: by the mixed solve from its BF16x6 rung (then
// FGMRES-IR), then, if that does not reach the gate, by the FP64 LU with
// FP64 refinement.
//
// A plan holds two graphs: a fast one (split-BF16x3 products, up to 10
// refinement sweeps) and a robust one (BF16x6, up to 16) for the
// low-frequency end of the band, where the systems are worst conditioned;
// in both, the sweeps after the one that reaches 1e-10 are no-ops (a device
// flag), so the bound costs little.  The autotuner replays the fast graph
// at the probe frequencies and finds the lowest frequency from which every
// probe reaches the gate (the split frequency: below it the robust graph
// runs), and times the wide tensor-core update tiles (64 or 128 columns) on
// the fast graph at the top probe, keeping the faster.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/peec_gb300.h"
#include "common.cuh"
#include "mixed_capture.cuh"

namespace peec {

bool launch_harmonic_fill_dev(const double *L, const double *P, const int *edges, const double *R, int ne, int nv,
                              const double *omega_dev, void *Z);
bool launch_plane_waves_dev(const double *centers, const double *vectors, int ne, int nv, int nrhs,
                            const double *d_k_hat, const double *d_e_hat, const double *k0_dev, void *rhs);
int set_tc_wide_tile(int bn);
int set_mixed_start_terms(int t);

static const double kC0 = 299792458.0;

struct SweepPlan {
    const double *L, *P, *R, *centers, *vectors;
    const int *edges;
    int ne, nv, n, nrhs;
    PeecSweepTuning tuning;         // the fast graph's
    PeecSweepTuning robust = {6, 16, 0};
    double f_split = 0.0;           // frequencies below use the robust graph
    cudaGraphExec_t exec_robust = nullptr;
    unsigned long long robust_launches = 0;
    double *d_params = nullptr;     // omega, k0
    double *h_params = nullptr;     // pinned: one (omega, k0) pair per frequency of a run
    size_t h_params_cap = 0;
    double *d_dirs = nullptr;       // k_hat [nrhs][3], e_hat [nrhs][3]
    Complex *d_Z = nullptr, *d_b = nullptr, *d_x = nullptr;
    unsigned long long *d_eta = nullptr;  // per graph replay
    int *d_status = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long graph_launches = 0;  // kernels per replay
};

static void drop(cudaGraphExec_t &e) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
}

// Record the per-frequency sequence with tuning t into exec.
static bool record(SweepPlan &p, const PeecSweepTuning &t, cudaGraphExec_t &exec, unsigned long long &launches) {
    drop(exec);
    if (!sync("sweep: before recording")) return false;
    const int prev_bn = set_tc_wide_tile(t.tile_bn);
    cudaGraph_t g = nullptr;
    bool ok = cuda_ok(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal), "sweep: begin capture");
    if (ok) {
        const unsigned long long l0 = launch_count();
        MixedCapture cap{t.split_terms, t.sweeps, 1e-10, p.d_eta, p.d_status};
        bool body = launch_harmonic_fill_dev(p.L, p.P, p.edges, p.R, p.ne, p.nv, p.d_params, p.d_Z) &&
                    launch_plane_waves_dev(p.centers, p.vectors, p.ne, p.nv, p.nrhs, p.d_dirs, p.d_dirs + 3 * p.nrhs,
                                           p.d_params + 1, p.d_b) &&
                    mixed_solve_impl(p.d_Z, (size_t)p.n, p.d_b, p.d_x, (size_t)p.nrhs, 0.0, 1, nullptr, nullptr,
                                     &cap) == 0;
        launches = launch_count() - l0;
        const bool ended = cuda_ok(cudaStreamEndCapture(stream(), &g), "sweep: end capture");
        ok = body && ended && g && cuda_ok(cudaGraphInstantiate(&exec, g, 0), "sweep: graph instantiation");
    }
    if (g) cudaGraphDestroy(g);
    set_tc_wide_tile(prev_bn);
    if (!ok) {
        cudaGetLastError();
        drop(exec);
    }
    return ok;
}

static bool record(SweepPlan &p) { return record(p, p.tuning, p.exec, p.graph_launches); }

static bool ensure_params(SweepPlan &p, size_t n_freq) {
    if (p.h_params_cap >= n_freq) return true;
    if (p.h_params) cudaFreeHost(p.h_params);
    p.h_params = nullptr;
    p.h_params_cap = 0;
    if (!cuda_ok(cudaMallocHost((void **)&p.h_params, 2 * n_freq * sizeof(double)), "sweep: pinned parameters"))
        return false;
    p.h_params_cap = n_freq;
    return true;
}

// Replays of the graph for freqs[0..n_freq): X, eta bits and status per
// frequency into device arrays (copied after each replay).  The robust graph
// runs below the split frequency, or for every frequency with all_robust.
static bool replay(SweepPlan &p, const double *freqs, size_t n_freq, Complex *d_X, unsigned long long *d_eta_all,
                   int *d_status_all, bool all_robust = false) {
    if (!ensure_params(p, n_freq)) return false;
    for (size_t f = 0; f < n_freq; ++f) {
        const double w = 2.0 * M_PI * freqs[f];
        p.h_params[2 * f] = w;
        p.h_params[2 * f + 1] = w / kC0;
    }
    const size_t xs = (size_t)p.n * p.nrhs;
    for (size_t f = 0; f < n_freq; ++f) {
        const bool robust = p.exec_robust && (all_robust || freqs[f] < p.f_split);
        if (!cuda_ok(cudaMemcpyAsync(p.d_params, p.h_params + 2 * f, 2 * sizeof(double), cudaMemcpyHostToDevice,
                                     stream()),
                     "sweep: parameters") ||
            !cuda_ok(cudaGraphLaunch(robust ? p.exec_robust : p.exec, stream()), "sweep: graph launch"))
            return false;
        note_launch((int)(robust ? p.robust_launches : p.graph_launches));
        if (!cuda_ok(cudaMemcpyAsync(d_X + f * xs, p.d_x, xs * sizeof(Complex), cudaMemcpyDeviceToDevice, stream()),
                     "sweep: solution copy") ||
            !cuda_ok(cudaMemcpyAsync(d_eta_all + f, p.d_eta, sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                                     stream()),
                     "sweep: backward error copy") ||
            !cuda_ok(cudaMemcpyAsync(d_status_all + f, p.d_status, sizeof(int), cudaMemcpyDeviceToDevice, stream()),
                     "sweep: status copy"))
            return false;
    }
    return true;
}

// One system outside the graph: the mixed solve with its precision ladder,
// then the FP64 LU with FP64 refinement.  0 at the gate (fallback 1 or 2),
// 1 when neither reached it, -1 on errors.
static int solve_fallback(SweepPlan &p, double freq, double tol, Complex *d_X, double *eta, int *fallback) {
    const double w = 2.0 * M_PI * freq, params[2] = {w, w / kC0};
    if (!cuda_ok(cudaMemcpyAsync(p.d_params, params, sizeof(params), cudaMemcpyHostToDevice, stream()),
                 "sweep: parameters") ||
        !launch_harmonic_fill_dev(p.L, p.P, p.edges, p.R, p.ne, p.nv, p.d_params, p.d_Z) ||
        !launch_plane_waves_dev(p.centers, p.vectors, p.ne, p.nv, p.nrhs, p.d_dirs, p.d_dirs + 3 * p.nrhs,
                                p.d_params + 1, p.d_b) ||
        !sync("sweep: fallback set-up"))
        return -1;
    int it = 0;
    // straight to BF16x6 (then FGMRES-IR if that stalls): the graph's own
    // attempt already showed BF16x3 (or BF16x6 refinement alone) short
    const int prev_terms = set_mixed_start_terms(6);
    int s = mixed_solve_impl(p.d_Z, (size_t)p.n, p.d_b, d_X, (size_t)p.nrhs, tol, 30, eta, &it, nullptr);
    set_mixed_start_terms(prev_terms);
    if (s == 0) {
        *fallback = 1;
        return 0;
    }
    if (s == -1) return -1;
    // FP64 LU of Z with FP64 refinement of the mixed solution (or from zero)
    const size_t nn = (size_t)p.n * p.n;
    DBuf<Complex> lu(nn);
    DBuf<long long> piv(p.n);
    DBuf<int> perm(p.n);
    DBuf<double> rs(p.n), cs(p.n);
    if (!lu.p || !piv.p || !perm.p || !rs.p || !cs.p) return -1;
    if (!cuda_ok(cudaMemcpyAsync(lu.p, p.d_Z, nn * sizeof(Complex), cudaMemcpyDeviceToDevice, stream()), "sweep: Z"))
        return -1;
    double scale = 0.0;
    int col = -1;
    if (peec_gb300_complex_lu_factor_device(lu.p, (size_t)p.n, 1e-14, piv.p, perm.p, rs.p, cs.p, &scale, &col) != 0)
        return -1;
    if (s != 1 &&
        peec_gb300_complex_lu_solve_device(lu.p, perm.p, rs.p, cs.p, (size_t)p.n, p.d_b, d_X, (size_t)p.nrhs) != 0)
        return -1;
    int r = peec_gb300_complex_refine_device(p.d_Z, lu.p, perm.p, rs.p, cs.p, (size_t)p.n, p.d_b, d_X,
                                             (size_t)p.nrhs, tol, 10, eta, &it);
    if (r < 0) return -1;
    *fallback = 2;
    return r;
}

}  // namespace peec

using namespace peec;

extern "C" {

void *peec_gb300_sweep_create(const double *d_L, const double *d_P, const int *d_edges, const double *d_R,
                              const double *d_edge_centers, const double *d_edge_vectors, size_t n_edges,
                              size_t n_nodes, size_t nrhs, const double *k_hat, const double *e_hat,
                              const PeecSweepTuning *tuning) {
    if (!d_L || !d_P || !d_edges || !d_edge_centers || !d_edge_vectors || !k_hat || !e_hat || n_edges == 0 ||
        n_nodes == 0 || nrhs == 0 || n_edges + n_nodes > 0x7fffffff || nrhs > 4096)
        return nullptr;
    SweepPlan *p = new SweepPlan();
    p->L = d_L;
    p->P = d_P;
    p->R = d_R;
    p->edges = d_edges;
    p->centers = d_edge_centers;
    p->vectors = d_edge_vectors;
    p->ne = (int)n_edges;
    p->nv = (int)n_nodes;
    p->n = p->ne + p->nv;
    p->nrhs = (int)nrhs;
    p->tuning = tuning ? *tuning : PeecSweepTuning{3, 10, 0};
    const size_t n = (size_t)p->n;
    bool ok = cuda_ok(cudaMalloc((void **)&p->d_params, 2 * sizeof(double)), "sweep plan") &&
              cuda_ok(cudaMalloc((void **)&p->d_dirs, 6 * nrhs * sizeof(double)), "sweep plan") &&
              cuda_ok(cudaMalloc((void **)&p->d_Z, n * n * sizeof(Complex)), "sweep plan") &&
              cuda_ok(cudaMalloc((void **)&p->d_b, n * nrhs * sizeof(Complex)), "sweep plan") &&
              cuda_ok(cudaMalloc((void **)&p->d_x, n * nrhs * sizeof(Complex)), "sweep plan") &&
              cuda_ok(cudaMalloc((void **)&p->d_eta, sizeof(unsigned long long)), "sweep plan") &&
              cuda_ok(cudaMalloc((void **)&p->d_status, sizeof(int)), "sweep plan");
    if (ok) {
        std::vector<double> dirs(6 * nrhs);
        memcpy(dirs.data(), k_hat, 3 * nrhs * sizeof(double));
        memcpy(dirs.data() + 3 * nrhs, e_hat, 3 * nrhs * sizeof(double));
        ok = cuda_ok(cudaMemcpyAsync(p->d_dirs, dirs.data(), dirs.size() * sizeof(double), cudaMemcpyHostToDevice,
                                     stream()),
                     "sweep plan") &&
             sync("sweep plan");
    }
    if (!ok) {
        peec_gb300_sweep_destroy(p);
        return nullptr;
    }
    return p;
}

int peec_gb300_sweep_tune(void *plan, const double *probe_frequencies, size_t n_probe, PeecSweepTuning *chosen,
                          double *ms_per_system) {
    if (!plan || !probe_frequencies || n_probe == 0 || n_probe > 64) return -1;
    SweepPlan &p = *static_cast<SweepPlan *>(plan);
    std::vector<double> probes(probe_frequencies, probe_frequencies + n_probe);
    std::sort(probes.begin(), probes.end());
    const size_t xs = (size_t)p.n * p.nrhs;
    DBuf<unsigned long long> eta_all(n_probe);
    DBuf<int> st_all(n_probe);
    DBuf<Complex> X(n_probe * xs);
    if (!eta_all.p || !st_all.p || !X.p) return -1;
    // the fast graph's backward errors at the probes; false on errors
    auto try_probes = [&](std::vector<double> &eta) -> bool {
        std::vector<unsigned long long> eb(n_probe);
        std::vector<int> sb(n_probe);
        if (!replay(p, probes.data(), n_probe, X.p, eta_all.p, st_all.p)) return false;
        cudaMemcpyAsync(eb.data(), eta_all.p, n_probe * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        stream());
        cudaMemcpyAsync(sb.data(), st_all.p, n_probe * sizeof(int), cudaMemcpyDeviceToHost, stream());
        if (!sync("sweep: tuning probes")) return false;
        eta.resize(n_probe);
        for (size_t f = 0; f < n_probe; ++f) {
            memcpy(&eta[f], &eb[f], sizeof(double));
            if (sb[f] != 0) eta[f] = INFINITY;
        }
        return true;
    };
    const double tol = 1e-10;
    drop(p.exec_robust);
    p.f_split = 0.0;
    // 1. fast graph: BF16x3, up to 10 sweeps; the split frequency
    p.tuning = PeecSweepTuning{3, 10, 128};
    std::vector<double> eta;
    if (!record(p) || !try_probes(eta)) return -1;
    size_t first_ok = n_probe;  // every probe from here on passes
    for (size_t f = n_probe; f-- > 0;) {
        if (!(eta[f] <= tol)) break;
        first_ok = f;
    }
    if (first_ok > 0) {  // the low end needs the robust graph
        p.f_split = first_ok < n_probe ? probes[first_ok] : INFINITY;
        p.robust.tile_bn = p.tuning.tile_bn;
        if (!record(p, p.robust, p.exec_robust, p.robust_launches)) return -1;
    }
    // 2. tile width of the wide updates, timed on the fast graph at the top
    // probe: the 128-column graph is the one just replayed at the probes
    // (recorded and warm), the 64-column one is recorded and warmed once;
    // two timed replays each
    const double ftop = probes.back(), fr[2] = {ftop, ftop};
    double best_ms = INFINITY;
    int best_bn = 128;
    for (int bn : {128, 64}) {
        if (bn != p.tuning.tile_bn) {
            p.tuning.tile_bn = bn;
            if (!record(p)) continue;
        }
        const double f_split = p.f_split;
        p.f_split = 0.0;  // time the fast graph
        bool ok = bn == 128 || (replay(p, fr, 1, X.p, eta_all.p, st_all.p) && sync("sweep: tuning warm-up"));
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, stream());
        ok = ok && replay(p, fr, 2, X.p, eta_all.p, st_all.p);
        cudaEventRecord(e1, stream());
        float ms = 0.0f;
        ok = sync("sweep: tuning") && ok;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        p.f_split = f_split;
        if (!ok) return -1;
        if (ms / 2.0 < best_ms) {
            best_ms = ms / 2.0;
            best_bn = bn;
        }
    }
    if (!isfinite(best_ms)) return -1;
    if (p.tuning.tile_bn != best_bn) {  // the 64-column graph was the last recorded
        p.tuning.tile_bn = best_bn;
        if (!record(p)) return -1;
    }
    if (p.exec_robust && p.robust.tile_bn != best_bn) {
        p.robust.tile_bn = best_bn;
        if (!record(p, p.robust, p.exec_robust, p.robust_launches)) return -1;
    }
    if (chosen) *chosen = p.tuning;
    if (ms_per_system) *ms_per_system = best_ms;
    return 0;
}

int peec_gb300_sweep_split(void *plan, double *split_frequency, PeecSweepTuning *robust) {
    if (!plan) return -1;
    SweepPlan &p = *static_cast<SweepPlan *>(plan);
    if (split_frequency) *split_frequency = p.exec_robust ? p.f_split : 0.0;
    if (robust) *robust = p.robust;
    return 0;
}

int peec_gb300_sweep_run(void *plan, const double *frequencies, size_t n_freq, double tol, Complex *d_X,
                         double *backward_error, int *fallback) {
    if (!plan || !frequencies || n_freq == 0 || !d_X) return -1;
    SweepPlan &p = *static_cast<SweepPlan *>(plan);
    if (!p.exec && !record(p)) return -1;
    DBuf<unsigned long long> eta_all(n_freq);
    DBuf<int> st_all(n_freq);
    if (!eta_all.p || !st_all.p) return -1;
    if (!replay(p, frequencies, n_freq, d_X, eta_all.p, st_all.p)) return -1;
    std::vector<unsigned long long> eb(n_freq);
    std::vector<int> sb(n_freq);
    cudaMemcpyAsync(eb.data(), eta_all.p, n_freq * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream());
    cudaMemcpyAsync(sb.data(), st_all.p, n_freq * sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!sync("sweep: results")) return -1;
    const size_t xs = (size_t)p.n * p.nrhs;
    auto missed = [&](size_t f) {
        double eta;
        memcpy(&eta, &eb[f], sizeof(eta));
        return sb[f] != 0 || !(eta <= tol);
    };
    for (size_t f = 0; f < n_freq; ++f)
        if (sb[f] == 6) {
            set_error("sweep: a triangular-solve wait timed out in the graph");
            return -1;
        }
    // systems the fast graph left above tol: the robust graph first (recorded
    // here if the tuner did not need it), replayed for all of them
    std::vector<double> rf;
    std::vector<size_t> ri;
    for (size_t f = 0; f < n_freq; ++f)
        if (missed(f) && !(p.exec_robust && frequencies[f] < p.f_split)) {
            rf.push_back(frequencies[f]);
            ri.push_back(f);
        }
    std::vector<int> rescued(n_freq, 0);
    if (!ri.empty()) {
        if (!p.exec_robust) {
            p.robust.tile_bn = p.tuning.tile_bn;
            if (!record(p, p.robust, p.exec_robust, p.robust_launches)) return -1;
        }
        const size_t m = ri.size();
        DBuf<Complex> X2(m * xs);
        DBuf<unsigned long long> eta2(m);
        DBuf<int> st2(m);
        if (!X2.p || !eta2.p || !st2.p || !replay(p, rf.data(), m, X2.p, eta2.p, st2.p, true)) return -1;
        std::vector<unsigned long long> e2(m);
        std::vector<int> s2(m);
        cudaMemcpyAsync(e2.data(), eta2.p, m * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream());
        cudaMemcpyAsync(s2.data(), st2.p, m * sizeof(int), cudaMemcpyDeviceToHost, stream());
        if (!sync("sweep: robust replays")) return -1;
        for (size_t j = 0; j < m; ++j) {
            double eta;
            memcpy(&eta, &e2[j], sizeof(eta));
            if (s2[j] == 6) {
                set_error("sweep: a triangular-solve wait timed out in the graph");
                return -1;
            }
            if (s2[j] != 0 || !(eta <= tol)) continue;
            const size_t f = ri[j];
            if (!cuda_ok(cudaMemcpyAsync(d_X + f * xs, X2.p + j * xs, xs * sizeof(Complex), cudaMemcpyDeviceToDevice,
                                         stream()),
                         "sweep: solution copy"))
                return -1;
            eb[f] = e2[j];
            sb[f] = 0;
            rescued[f] = 1;
        }
    }
    int worst = 0;
    for (size_t f = 0; f < n_freq; ++f) {
        double eta;
        memcpy(&eta, &eb[f], sizeof(eta));
        int fb = rescued[f] ? 3 : 0;
        if (missed(f)) {
            const int s = solve_fallback(p, frequencies[f], tol, d_X + f * xs, &eta, &fb);
            if (s < 0) return -1;
            worst = std::max(worst, s);
        }
        if (backward_error) backward_error[f] = eta;
        if (fallback) fallback[f] = fb;
    }
    return worst;
}

int peec_gb300_sweep_tuning(void *plan, PeecSweepTuning *tuning) {
    if (!plan || !tuning) return -1;
    *tuning = static_cast<SweepPlan *>(plan)->tuning;
    return 0;
}

void peec_gb300_sweep_destroy(void *plan) {
    if (!plan) return;
    SweepPlan *p = static_cast<SweepPlan *>(plan);
    sync("sweep: destroy");
    drop(p->exec);
    drop(p->exec_robust);
    for (void *d : {(void *)p->d_params, (void *)p->d_dirs, (void *)p->d_Z, (void *)p->d_b, (void *)p->d_x,
                    (void *)p->d_eta, (void *)p->d_status})
        if (d) cudaFree(d);
    if (p->h_params) cudaFreeHost(p->h_params);
    delete p;
}

}  // extern "C"
