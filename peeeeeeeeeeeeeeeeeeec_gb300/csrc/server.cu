// Serving loop: continuous admission of harmonic and transient requests on
// one GPU.
//
// Requests enter a FIFO.  Worker threads -- each with its own CUDA stream,
// so admitted requests overlap on the device -- admit the head request as
// soon as a worker is free and its HBM estimate fits the remaining budget.
// Assembled Lp / P stay device-resident per mesh key and are reused by every
// later request on that mesh (any frequency); a transient system (its
// factorised MNA matrix) stays resident per mesh, scheme and time step and
// is reused by every later lightning run on it.  Cached meshes are evicted,
// least recently used first, when a new request needs the memory.  Each
// request records submit / start / end times for latency percentiles.
#include <math.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/peec_gb300.h"
#include "common.cuh"

namespace peec {

int transient_lightning_runs(void *system, int nrun, const double *K, const double *alpha, const double *beta,
                             const double *delay, const size_t *strike_node, const size_t *return_node,
                             const long long *start, size_t step0, size_t n_steps, double *d_X,
                             const int *d_probe_nodes, size_t n_probe_nodes, const int *d_probe_edges,
                             size_t n_probe_edges, double *d_probes);

struct TransientEntry {
    void *sys = nullptr;
    size_t bytes = 0;
    bool ready = false;
    int status = 0;
    int session_room = 0;  // free run slots of the stepping sessions on this system
};

struct MeshEntry {
    unsigned long long key = 0;
    double *L = nullptr, *P = nullptr, *ctr = nullptr, *vec = nullptr;
    int *edges = nullptr;
    size_t ne = 0, nv = 0, bytes = 0;  // bytes: Lp / P / geometry plus every transient system
    int users = 0;
    bool ready = false;
    int status = 0;
    unsigned long long last_use = 0;
    std::map<std::pair<int, double>, TransientEntry> transient;  // (scheme, dt)
};

struct Job {
    long long ticket = 0;
    int kind = 0;  // 0 harmonic, 1 transient lightning
    PeecHarmonicRequest req{};
    PeecTransientRequest treq{};
    std::vector<double> k_hat, e_hat;           // harmonic: copies
    std::vector<int> probe_nodes, probe_edges;  // transient: copies
    const Mesh *mesh = nullptr;
    const DualMesh *dual = nullptr;
    unsigned long long mesh_key = 0;
    size_t bytes = 0;       // per-request device estimate (caches excluded)
    size_t mesh_bytes = 0;  // Lp / P / geometry of the mesh
    size_t sys_bytes = 0;   // transient system of (scheme, dt)
    PeecRequestResult res{};
    bool done = false;
};

// a transient system at its peak (the factor and the inverse formed from
// it, before the factor is freed) + Lp and A S as float pairs (+ the FP64
// A S while they are formed) + vectors
static size_t transient_system_bytes(size_t ne, size_t nv) {
    size_t nt = ne + nv;
    return 16 * nt * nt + 8 * ne * ne + 16 * ne * nv + 64 * nt + 16 * ne;
}

class Server {
  public:
    Server(size_t budget, int workers) : budget_(budget), t0_(std::chrono::steady_clock::now()) {
        if (workers < 1) workers = 1;
        cudaGetDevice(&device_);
        for (int w = 0; w < workers; ++w) threads_.emplace_back([this] { worker(); });
    }
    ~Server() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : threads_) t.join();
        for (auto &m : meshes_) free_mesh(m.second);
        sync("server shutdown");
    }

    double clock() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    }

    long long submit(const PeecHarmonicRequest *r) {
        if (!r || !r->mesh || !r->dual || !r->x || r->nrhs == 0 || !r->k_hat || !r->e_hat ||
            !(r->frequency > 0.0) || r->mesh->n_edges == 0 || r->mesh->n_nodes == 0) {
            set_error("server: invalid request");
            return -1;
        }
        auto j = std::make_shared<Job>();
        j->kind = 0;
        j->req = *r;
        j->mesh = r->mesh;
        j->dual = r->dual;
        j->mesh_key = r->mesh_key;
        j->k_hat.assign(r->k_hat, r->k_hat + 3 * r->nrhs);
        j->e_hat.assign(r->e_hat, r->e_hat + 3 * r->nrhs);
        size_t ne = r->mesh->n_edges, nv = r->mesh->n_nodes, n = ne + nv;
        j->mesh_bytes = mesh_bytes(ne, nv);
        // Z + working copy (mixed: FP32 LU + FP32 |Z| + BF16 splits, or the
        // FP64 LU of a fallback, whichever is larger; plain: FP64 LU) +
        // vectors + scratch; a mixed solve of 32 or more right-hand sides
        // also keeps Z as float pairs for its residual
        j->bytes = 32 * n * n + (r->mixed ? 9216 * n : 0) + (r->mixed && r->nrhs >= 32 ? 16 * n * n : 0) +
                   112 * n * r->nrhs + (64 << 20);
        return enqueue(j);
    }

    long long submit(const PeecTransientRequest *r) {
        if (!r || !r->mesh || !r->dual || r->n_steps == 0 || r->mesh->n_edges == 0 || r->mesh->n_nodes == 0 ||
            (r->scheme != 1 && r->scheme != 2) || !(r->dt > 0.0) || !isfinite(r->dt) ||
            (r->n_probe_nodes && !r->probe_nodes) || (r->n_probe_edges && !r->probe_edges) ||
            ((r->n_probe_nodes || r->n_probe_edges) && !r->probes)) {
            set_error("server: invalid request");
            return -1;
        }
        auto j = std::make_shared<Job>();
        j->kind = 1;
        j->treq = *r;
        j->mesh = r->mesh;
        j->dual = r->dual;
        j->mesh_key = r->mesh_key;
        j->probe_nodes.assign(r->probe_nodes, r->probe_nodes + r->n_probe_nodes);
        j->probe_edges.assign(r->probe_edges, r->probe_edges + r->n_probe_edges);
        size_t ne = r->mesh->n_edges, nv = r->mesh->n_nodes, nt = ne + nv;
        size_t np = r->n_probe_nodes + r->n_probe_edges;
        j->mesh_bytes = mesh_bytes(ne, nv);
        j->sys_bytes = transient_system_bytes(ne, nv);
        j->bytes = 8 * r->n_steps * np + 64 * nt + 4 * np + (64 << 20);
        return enqueue(j);
    }

    int wait(long long ticket, PeecRequestResult *out) {
        std::unique_lock<std::mutex> g(mu_);
        auto it = jobs_.find(ticket);
        if (it == jobs_.end()) return -1;
        auto j = it->second;
        done_cv_.wait(g, [&] { return j->done; });
        if (out) *out = j->res;
        jobs_.erase(ticket);
        return 0;
    }

  private:
    size_t budget_, used_ = 0;
    int device_ = 0;
    std::chrono::steady_clock::time_point t0_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<std::shared_ptr<Job>> queue_;
    std::map<long long, std::shared_ptr<Job>> jobs_;
    std::map<unsigned long long, MeshEntry> meshes_;
    std::vector<std::thread> threads_;
    long long next_ticket_ = 0;
    unsigned long long tick_ = 0;
    bool stop_ = false;

    static size_t mesh_bytes(size_t ne, size_t nv) { return 8 * (ne * ne + nv * nv) + 56 * ne; }

    long long enqueue(const std::shared_ptr<Job> &j) {
        if (j->bytes + j->mesh_bytes + j->sys_bytes > budget_) {
            set_error("server: request needs more device memory than the server's budget");
            return -1;
        }
        std::lock_guard<std::mutex> g(mu_);
        j->ticket = next_ticket_++;
        j->res.t_submit = clock();
        jobs_[j->ticket] = j;
        queue_.push_back(j);
        cv_.notify_all();
        return j->ticket;
    }

    // stream-ordered free on the calling thread's stream: an entry is freed
    // only when no request uses it and every user has synchronised
    static void free_mesh(MeshEntry &m) {
        for (auto &t : m.transient)
            if (t.second.sys) peec_gb300_transient_destroy(t.second.sys);
        m.transient.clear();
        for (void *p : {(void *)m.L, (void *)m.P, (void *)m.ctr, (void *)m.vec, (void *)m.edges}) dfree(p);
        m.L = m.P = m.ctr = m.vec = nullptr;
        m.edges = nullptr;
    }

    // a lightning run that a stepping session of its system has room for
    // (it joins that session at its next chunk boundary)
    bool steered(const Job &j) {
        if (j.kind != 1) return false;
        auto it = meshes_.find(j.mesh_key);
        if (it == meshes_.end()) return false;
        auto ti = it->second.transient.find({j.treq.scheme, j.treq.dt});
        return ti != it->second.transient.end() && ti->second.session_room > 0;
    }

    // bytes the job needs now: its own, plus the mesh and the transient
    // system when they are not cached
    size_t need(const Job &j) {
        auto it = meshes_.find(j.mesh_key);
        if (it == meshes_.end()) return j.bytes + j.mesh_bytes + j.sys_bytes;
        if (j.kind == 1 && !it->second.transient.count({j.treq.scheme, j.treq.dt})) return j.bytes + j.sys_bytes;
        return j.bytes;
    }

    // evict unused cached meshes (least recently used first, never `keep`)
    // until `bytes` fit
    void make_room(size_t bytes, unsigned long long keep) {
        while (used_ + bytes > budget_) {
            auto victim = meshes_.end();
            for (auto it = meshes_.begin(); it != meshes_.end(); ++it)
                if (it->second.users == 0 && it->second.ready && it->first != keep &&
                    (victim == meshes_.end() || it->second.last_use < victim->second.last_use))
                    victim = it;
            if (victim == meshes_.end()) return;
            used_ -= victim->second.bytes;
            free_mesh(victim->second);
            meshes_.erase(victim);
        }
    }

    void worker() {
        cudaSetDevice(device_);
        for (;;) {
            std::shared_ptr<Job> j;
            std::vector<std::shared_ptr<Job>> batch;  // transient runs stepped with j
            MeshEntry *me = nullptr;
            TransientEntry *te = nullptr;
            bool build_mesh = false, build_sys = false;
            {
                std::unique_lock<std::mutex> g(mu_);
                auto pick = queue_.end();
                for (;;) {
                    if (stop_ && queue_.empty()) return;
                    // the first request in arrival order, passing over lightning
                    // runs that a stepping session of their system will admit
                    pick = queue_.begin();
                    while (pick != queue_.end() && steered(**pick)) ++pick;
                    if (pick != queue_.end()) {
                        size_t nb = need(**pick);
                        make_room(nb, (*pick)->mesh_key);
                        if (used_ + nb <= budget_) break;
                    }
                    cv_.wait(g);
                }
                j = *pick;
                queue_.erase(pick);
                auto it = meshes_.find(j->mesh_key);
                if (it == meshes_.end()) {
                    MeshEntry e;
                    e.key = j->mesh_key;
                    e.bytes = j->mesh_bytes;
                    it = meshes_.emplace(e.key, e).first;
                    used_ += j->mesh_bytes;
                    build_mesh = true;
                }
                me = &it->second;
                if (j->kind == 1) {
                    auto key = std::make_pair(j->treq.scheme, j->treq.dt);
                    auto ti = me->transient.find(key);
                    if (ti == me->transient.end()) {
                        ti = me->transient.emplace(key, TransientEntry()).first;
                        ti->second.bytes = j->sys_bytes;
                        me->bytes += j->sys_bytes;
                        used_ += j->sys_bytes;
                        build_sys = true;
                    }
                    te = &ti->second;
                }
                me->users++;
                me->last_use = ++tick_;
                used_ += j->bytes;
                j->res.t_start = clock();
                if (j->kind == 1) admit_runs(*j, me, batch, kMaxSlots - 1, j->res.t_start);  // start with j
            }
            cv_.notify_all();
            if (build_mesh) {
                int s = assemble_mesh(*me, j->mesh, j->dual);
                std::lock_guard<std::mutex> g(mu_);
                me->status = s;
                me->ready = true;
                cv_.notify_all();
            } else {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return me->ready; });
            }
            int status = me->status == 0 ? 0 : -1;
            if (status == 0 && j->kind == 1) {
                if (build_sys) {
                    void *sys = nullptr;
                    int s = peec_gb300_transient_create(me->L, me->P, me->edges, nullptr, me->ne, me->nv,
                                                        j->treq.scheme, j->treq.dt, &sys);
                    std::lock_guard<std::mutex> g(mu_);
                    te->sys = sys;
                    te->status = s;
                    te->ready = true;
                    cv_.notify_all();
                } else {
                    std::unique_lock<std::mutex> g(mu_);
                    cv_.wait(g, [&] { return te->ready; });
                }
                status = te->status;
            }
            batch.insert(batch.begin(), j);
            if (j->kind == 1) {
                // the stepping session finishes every run it steps: those of
                // batch and those it admits on the way
                run_session(me, *te, batch, status);
            } else {
                if (status == 0) status = solve(*me, *j);
                std::lock_guard<std::mutex> g(mu_);
                finish(me, j, status);
            }
            {
                std::lock_guard<std::mutex> g(mu_);
                if ((me->status != 0 || (te && te->status != 0)) && me->users == 0) {
                    // a failed assembly or factorisation is not kept
                    used_ -= me->bytes;
                    free_mesh(*me);
                    meshes_.erase(me->key);
                }
            }
            cv_.notify_all();
            done_cv_.notify_all();
        }
    }

    int assemble_mesh(MeshEntry &e, const Mesh *m, const DualMesh *dual) {
        e.ne = m->n_edges;
        e.nv = m->n_nodes;
        e.L = static_cast<double *>(dalloc(8 * e.ne * e.ne));
        e.P = static_cast<double *>(dalloc(8 * e.nv * e.nv));
        e.ctr = static_cast<double *>(dalloc(24 * e.ne));
        e.vec = static_cast<double *>(dalloc(24 * e.ne));
        e.edges = static_cast<int *>(dalloc(8 * e.ne));
        if (!e.L || !e.P || !e.ctr || !e.vec || !e.edges) return -1;
        InductanceOptions lo;
        inductance_options_default(&lo, 1);
        PotentialOptions po;
        potential_options_default(&po, 1);
        if (peec_gb300_inductance_device(m, dual, &lo, e.L, nullptr) != 0) return -1;
        if (peec_gb300_potential_device(m, dual, &po, e.P, nullptr) != 0) return -1;
        if (peec_gb300_copy_to_device(e.ctr, m->edge_centers, 24 * e.ne) != 0 ||
            peec_gb300_copy_to_device(e.vec, m->edge_vectors, 24 * e.ne) != 0 ||
            peec_gb300_copy_to_device(e.edges, m->edges, 8 * e.ne) != 0)
            return -1;
        return peec_gb300_synchronize() == 0 ? 0 : -1;
    }

    int solve(const MeshEntry &e, Job &j) {
        const PeecHarmonicRequest &r = j.req;
        size_t n = e.ne + e.nv, nrhs = r.nrhs;
        DBuf<Complex> Z(n * n), B(n * nrhs), X(n * nrhs), W;
        if (!Z.p || !B.p || !X.p) return -1;
        if (peec_gb300_harmonic_build_device(e.L, e.P, e.edges, nullptr, e.ne, e.nv, r.frequency, Z.p) != 0)
            return -1;
        double k0 = 2.0 * M_PI * r.frequency / 299792458.0;
        for (size_t q = 0; q < nrhs; ++q)
            if (peec_gb300_plane_wave_rhs_device(e.ctr, e.vec, e.ne, e.nv, &j.k_hat[3 * q], &j.e_hat[3 * q], k0,
                                                 B.p + q * n) != 0)
                return -1;
        int status;
        double be = 0.0;
        int iters = 0;
        if (r.mixed) {
            double tol = r.tolerance > 0.0 ? r.tolerance : 1e-10;
            status = peec_gb300_complex_solve_mixed_device(Z.p, n, B.p, X.p, nrhs, tol, 30, &be, &iters);
            // refinement that stalls (ill-conditioned systems, e.g. very low
            // frequencies) or an FP32 pivot breakdown: solve again in FP64
            if (status == 1 || status == -2) j.res.fallback = 1;
        }
        if (!r.mixed || j.res.fallback) {
            DBuf<long long> piv(n);
            DBuf<int> perm(n);
            DBuf<double> rs(n), cs(n);
            if (!W.alloc(n * n) || !piv.p || !perm.p || !rs.p || !cs.p) return -1;
            if (peec_gb300_copy_device(W.p, Z.p, n * n * sizeof(Complex)) != 0) return -1;
            double scale;
            int col;
            status = peec_gb300_complex_lu_factor_device(W.p, n, 1e-14, piv.p, perm.p, rs.p, cs.p, &scale, &col);
            if (status == 0)
                status = peec_gb300_complex_lu_solve_device(W.p, perm.p, rs.p, cs.p, n, B.p, X.p, nrhs);
            if (status == 0) {
                // FP64 iterative refinement with the FP64 factor up to the
                // gate: the mixed path's fallback, and the plain path's
                // answer when the LU solution itself misses the gate (very
                // low frequencies), so that both paths deliver the same
                // accuracy
                double tol = r.tolerance > 0.0 ? r.tolerance : 1e-10;
                status = peec_gb300_complex_refine_device(Z.p, W.p, perm.p, rs.p, cs.p, n, B.p, X.p, nrhs, tol, 5,
                                                          &be, &iters);
            }
        }
        j.res.backward_error = be;
        j.res.iterations = iters;
        if (status < 0) return status;
        if (!X.download(r.x, n * nrhs) || !sync("serving result")) return -1;
        return status;
    }

    // a finished request (the caller holds mu_)
    void finish(MeshEntry *me, const std::shared_ptr<Job> &b, int status) {
        b->res.status = status;
        b->res.t_end = clock();
        if (b->kind == 1) b->res.iterations = (int)b->treq.n_steps;
        used_ -= b->bytes;
        me->users--;
        b->done = true;
    }

    // queued lightning runs that can join a stepping batch of j's system
    // (same mesh, scheme and time step), up to `room` of them and as far as
    // the budget allows; the caller holds mu_
    void admit_runs(const Job &j, MeshEntry *me, std::vector<std::shared_ptr<Job>> &out, size_t room,
                    double t_start) {
        for (auto q = queue_.begin(); q != queue_.end() && out.size() < room;) {
            const Job &o = **q;
            if (o.kind == 1 && o.mesh_key == j.mesh_key && o.treq.scheme == j.treq.scheme &&
                o.treq.dt == j.treq.dt && used_ + o.bytes <= budget_) {
                used_ += o.bytes;
                me->users++;
                me->last_use = ++tick_;
                (*q)->res.t_start = t_start;
                out.push_back(*q);
                q = queue_.erase(q);
            } else {
                ++q;
            }
        }
    }

    // Continuous batching of lightning runs on one transient system: up to
    // kMaxSlots runs step together, in chunks of at most kChunk steps; between chunks
    // the runs that reached their length leave (waveforms and final state
    // copied out, the request finished) and queued runs of the same system
    // join with their state at rest and their own step 0 at the current
    // step.  While the session has free slots, workers leave that system's
    // queued runs to it (steered()).  Each run keeps its own probe lists:
    // a chunk records the concatenation of all runs' lists for every run,
    // and each request takes its own columns.  A run's arithmetic does not
    // depend on its slot or on the other runs, so its results equal a run
    // alone bit for bit.
    static constexpr size_t kChunk = 256;
    static constexpr int kMaxSlots = 8;
    struct Slot {
        std::shared_ptr<Job> job;
        long long start = 0;  // the session step of its own step 0
        size_t done = 0;      // its steps so far
    };
    void run_session(MeshEntry *me, TransientEntry &t, const std::vector<std::shared_ptr<Job>> &first, int status) {
        const size_t nt = me->ne + me->nv;
        const Job &j0 = *first[0];
        std::vector<Slot> slots;
        for (auto &b : first) slots.push_back(Slot{b, 0, 0});
        int room = 0;  // this session's share of t.session_room
        auto set_room = [&](int r) {  // the caller holds mu_
            t.session_room += r - room;
            room = r;
        };
        DBuf<double> X(nt * kMaxSlots), probes;
        DBuf<int> pn, pe;
        if (status == 0 && !X.p) status = -1;
        if (status == 0) {
            cudaMemsetAsync(X.p, 0, 8 * nt * slots.size(), stream());
            std::lock_guard<std::mutex> g(mu_);
            set_room(kMaxSlots - (int)slots.size());
        }
        std::vector<double> hp, hx(nt);
        std::vector<int> cn, ce;  // the chunk's concatenated probe lists
        std::vector<size_t> on, oe;  // each slot's offsets in them
        long long step = 0;
        while (status == 0 && !slots.empty()) {
            const int nrun = (int)slots.size();
            size_t chunk = kChunk;
            for (auto &sl : slots) chunk = std::min(chunk, (size_t)sl.job->treq.n_steps - sl.done);
            std::vector<double> K(nrun), al(nrun), be(nrun), de(nrun);
            std::vector<size_t> sk(nrun), rt(nrun);
            std::vector<long long> st(nrun);
            cn.clear();
            ce.clear();
            on.assign(nrun, 0);
            oe.assign(nrun, 0);
            for (int r = 0; r < nrun; ++r) {
                const Job &jr = *slots[r].job;
                const PeecTransientRequest &q = jr.treq;
                K[r] = q.K;
                al[r] = q.alpha;
                be[r] = q.beta;
                de[r] = q.delay;
                sk[r] = q.strike_node;
                rt[r] = q.return_node;
                st[r] = slots[r].start;
                on[r] = cn.size();
                oe[r] = ce.size();
                cn.insert(cn.end(), jr.probe_nodes.begin(), jr.probe_nodes.end());
                ce.insert(ce.end(), jr.probe_edges.begin(), jr.probe_edges.end());
            }
            const size_t npn = cn.size(), npe = ce.size(), np = npn + npe;
            if ((npn > pn.n && !pn.alloc(npn)) || (npe > pe.n && !pe.alloc(npe)) ||
                (np * chunk * nrun > probes.n && !probes.alloc(np * kChunk * kMaxSlots)) ||
                (npn && !pn.upload(cn.data(), npn)) || (npe && !pe.upload(ce.data(), npe))) {
                status = -1;
                break;
            }
            status = transient_lightning_runs(t.sys, nrun, K.data(), al.data(), be.data(), de.data(), sk.data(),
                                              rt.data(), st.data(), (size_t)step, chunk, X.p, pn.p, npn, pe.p, npe,
                                              probes.p);
            if (status != 0) break;
            hp.resize(chunk * nrun * np);
            if (np && (!probes.download(hp.data(), hp.size()) || !sync("transient probes"))) {
                status = -1;
                break;
            }
            for (int r = 0; r < nrun; ++r) {  // rows [k][run][np] -> each request's own columns
                const Job &jr = *slots[r].job;
                const size_t rn = jr.probe_nodes.size(), re = jr.probe_edges.size();
                if ((rn + re) && jr.treq.probes)
                    for (size_t k = 0; k < chunk; ++k) {
                        const double *row = hp.data() + (k * nrun + r) * np;
                        double *dst = jr.treq.probes + (slots[r].done + k) * (rn + re);
                        memcpy(dst, row + on[r], rn * sizeof(double));
                        memcpy(dst + rn, row + npn + oe[r], re * sizeof(double));
                    }
                slots[r].done += chunk;
            }
            step += (long long)chunk;
            // runs that reached their length leave, the last slot moving into
            // each freed one
            std::vector<std::shared_ptr<Job>> finished;
            for (int r = nrun - 1; r >= 0; --r) {
                if (slots[r].done < slots[r].job->treq.n_steps) continue;
                const PeecTransientRequest &q = slots[r].job->treq;
                if (cudaMemcpyAsync(hx.data(), X.p + (size_t)r * nt, 8 * nt, cudaMemcpyDeviceToHost, stream()) !=
                        cudaSuccess ||
                    !sync("transient result")) {
                    status = -1;
                    break;
                }
                if (q.I) memcpy(q.I, hx.data(), me->ne * sizeof(double));
                if (q.V) memcpy(q.V, hx.data() + me->ne, me->nv * sizeof(double));
                finished.push_back(slots[r].job);
                const int last = (int)slots.size() - 1;
                if (r != last) {
                    cudaMemcpyAsync(X.p + (size_t)r * nt, X.p + (size_t)last * nt, 8 * nt, cudaMemcpyDeviceToDevice,
                                    stream());
                    slots[r] = slots[last];
                }
                slots.pop_back();
            }
            std::vector<std::shared_ptr<Job>> joined;
            {
                std::lock_guard<std::mutex> g(mu_);
                for (auto &b : finished) finish(me, b, 0);
                if (status == 0) admit_runs(j0, me, joined, kMaxSlots - slots.size(), clock());
                set_room(status == 0 && slots.size() + joined.size() > 0
                             ? kMaxSlots - (int)(slots.size() + joined.size())
                             : 0);
            }
            if (!finished.empty()) done_cv_.notify_all();
            for (auto &b : joined) {  // at rest, own step 0 at the current step
                cudaMemsetAsync(X.p + slots.size() * nt, 0, 8 * nt, stream());
                slots.push_back(Slot{b, step, 0});
            }
        }
        {
            std::lock_guard<std::mutex> g(mu_);
            set_room(0);
            for (auto &sl : slots) finish(me, sl.job, status == 0 ? -1 : status);
        }
        cv_.notify_all();  // runs passed over for this session are open to every worker again
    }
};

}  // namespace peec

extern "C" {

void *peec_gb300_server_create(size_t hbm_budget_bytes, int workers) {
    try {
        return new peec::Server(hbm_budget_bytes, workers);
    } catch (...) {
        return nullptr;
    }
}

long long peec_gb300_server_submit(void *server, const PeecHarmonicRequest *request) {
    return server ? static_cast<peec::Server *>(server)->submit(request) : -1;
}

long long peec_gb300_server_submit_transient(void *server, const PeecTransientRequest *request) {
    return server ? static_cast<peec::Server *>(server)->submit(request) : -1;
}

int peec_gb300_server_wait(void *server, long long ticket, PeecRequestResult *result) {
    return server ? static_cast<peec::Server *>(server)->wait(ticket, result) : -1;
}

double peec_gb300_server_clock(void *server) { return server ? static_cast<peec::Server *>(server)->clock() : -1.0; }

void peec_gb300_server_destroy(void *server) { delete static_cast<peec::Server *>(server); }

}  // extern "C"
