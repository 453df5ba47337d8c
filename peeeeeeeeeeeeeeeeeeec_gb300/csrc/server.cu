// Serving loop: continuous batching of harmonic solves on one GPU.
//
// Requests (mesh, frequency, plane-wave right-hand sides, plain or mixed
// precision) enter a FIFO.  Worker threads -- each with its own CUDA stream,
// so admitted requests overlap on the device -- admit the head request as
// soon as a worker is free and its HBM estimate fits the remaining budget.
// Assembled Lp / P stay device-resident per mesh key and are reused by every
// later request on that mesh (any frequency); the cache is evicted least-
// recently-used when a new request needs the memory.  Each request records
// submit / start / end times for latency percentiles.
#include <math.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/peec_gb300.h"
#include "common.cuh"

namespace peec {

struct MeshEntry {
    unsigned long long key = 0;
    double *L = nullptr, *P = nullptr, *ctr = nullptr, *vec = nullptr;
    int *edges = nullptr;
    size_t ne = 0, nv = 0, bytes = 0;
    int users = 0;
    bool ready = false;
    int status = 0;
    unsigned long long last_use = 0;
};

struct Job {
    long long ticket;
    PeecHarmonicRequest req;
    std::vector<double> k_hat, e_hat;  // copies
    size_t bytes = 0;                  // per-request device estimate (mesh cache excluded)
    size_t mesh_bytes = 0;
    PeecRequestResult res{};
    bool done = false;
};

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
        j->req = *r;
        j->k_hat.assign(r->k_hat, r->k_hat + 3 * r->nrhs);
        j->e_hat.assign(r->e_hat, r->e_hat + 3 * r->nrhs);
        size_t ne = r->mesh->n_edges, nv = r->mesh->n_nodes, n = ne + nv;
        j->mesh_bytes = 8 * (ne * ne + nv * nv) + 56 * ne;
        // Z + working copy (FP32 LU for mixed, FP64 LU for plain) + vectors
        j->bytes = 16 * n * n + (r->mixed ? 8 * n * n + 6 * n * 192 : 16 * n * n) + 64 * n * r->nrhs + (64 << 20);
        if (j->bytes + j->mesh_bytes > budget_) {
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

    // stream-ordered free on the calling thread's stream: an entry is freed
    // only when no request uses it and every user has synchronised
    static void free_mesh(MeshEntry &m) {
        for (void *p : {(void *)m.L, (void *)m.P, (void *)m.ctr, (void *)m.vec, (void *)m.edges}) dfree(p);
        m.L = m.P = m.ctr = m.vec = nullptr;
        m.edges = nullptr;
    }

    // bytes the head job needs now (its own + the mesh entry if not cached)
    size_t need(const Job &j) {
        auto it = meshes_.find(j.req.mesh_key);
        return j.bytes + (it == meshes_.end() ? j.mesh_bytes : 0);
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
            MeshEntry *me = nullptr;
            bool build_mesh = false;
            {
                std::unique_lock<std::mutex> g(mu_);
                for (;;) {
                    if (stop_ && queue_.empty()) return;
                    if (!queue_.empty()) {
                        size_t nb = need(*queue_.front());
                        make_room(nb, queue_.front()->req.mesh_key);
                        if (used_ + nb <= budget_) break;
                    }
                    cv_.wait(g);
                }
                j = queue_.front();
                queue_.pop_front();
                auto it = meshes_.find(j->req.mesh_key);
                if (it == meshes_.end()) {
                    MeshEntry e;
                    e.key = j->req.mesh_key;
                    e.bytes = j->mesh_bytes;
                    it = meshes_.emplace(e.key, e).first;
                    used_ += j->mesh_bytes;
                    build_mesh = true;
                }
                me = &it->second;
                me->users++;
                me->last_use = ++tick_;
                used_ += j->bytes;
                j->res.t_start = clock();
            }
            cv_.notify_all();
            if (build_mesh) {
                int s = assemble_mesh(*me, j->req);
                std::lock_guard<std::mutex> g(mu_);
                me->status = s;
                me->ready = true;
                cv_.notify_all();
            } else {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return me->ready; });
            }
            int status = me->status == 0 ? solve(*me, *j) : -1;
            {
                std::lock_guard<std::mutex> g(mu_);
                j->res.status = status;
                j->res.t_end = clock();
                used_ -= j->bytes;
                me->users--;
                if (me->status != 0 && me->users == 0) {  // a failed assembly is not kept
                    used_ -= me->bytes;
                    free_mesh(*me);
                    meshes_.erase(me->key);
                }
                j->done = true;
            }
            cv_.notify_all();
            done_cv_.notify_all();
        }
    }

    int assemble_mesh(MeshEntry &e, const PeecHarmonicRequest &r) {
        const Mesh *m = r.mesh;
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
        if (peec_gb300_inductance_device(m, r.dual, &lo, e.L, nullptr) != 0) return -1;
        if (peec_gb300_potential_device(m, r.dual, &po, e.P, nullptr) != 0) return -1;
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
        } else {
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
            double out[3];
            if (status == 0 && peec_gb300_backward_error_device(Z.p, n, X.p, B.p, nrhs, out) == 0) be = out[0];
            iters = 0;
        }
        j.res.backward_error = be;
        j.res.iterations = iters;
        if (status < 0) return status;
        if (!X.download(r.x, n * nrhs) || !sync("serving result")) return -1;
        return status;
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

int peec_gb300_server_wait(void *server, long long ticket, PeecRequestResult *result) {
    return server ? static_cast<peec::Server *>(server)->wait(ticket, result) : -1;
}

double peec_gb300_server_clock(void *server) { return server ? static_cast<peec::Server *>(server)->clock() : -1.0; }

void peec_gb300_server_destroy(void *server) { delete static_cast<peec::Server *>(server); }

}  // extern "C"
