// Continuous-batching request server.
//
// Single-point energy/force/stress requests (one periodic configuration each)
// are submitted from any thread and queue in arrival order.  Each worker
// thread owns one Engine -- its own CUDA stream, device-resident parameter
// sets and grow-only workspace -- and loops: take the oldest waiting requests
// while the batch stays under the atom limit and the device-memory estimate of
// everything in flight stays under the HBM budget, evaluate them as one batch
// (one set of launches, see ck_engine.h), publish the results, repeat.  With
// several workers, a batch forms and starts while earlier ones still run, so
// requests that arrive during a batch are admitted as soon as a worker and
// memory free up, and their work overlaps on the device.  Latency is measured
// per request from submit to published result.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ck_engine.h"
#include "ck_geom.h"

namespace ck {

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    long long id = 0;
    int slot = 0;
    int n = 0;
    std::vector<double> pos;
    std::vector<int> types;
    double cell[9] = {0};
    bool small = false;
    double est_bytes = 0.0;
    // results
    bool done = false;
    int status = 0;
    std::string err;
    double energy = 0.0, stress[9] = {0};
    std::vector<double> force;
    double t_submit = 0.0, t_done = 0.0;
};

}  // namespace

class Server {
public:
    Server(int n_workers, double budget_bytes, long long max_batch_atoms, int precision)
        : budget_(budget_bytes), max_atoms_(max_batch_atoms) {
        if (n_workers < 1) n_workers = 1;
        for (int w = 0; w < n_workers; w++) {
            engines_.emplace_back(new Engine());
            engines_.back()->precision = precision;
            engine_mu_.emplace_back(new std::mutex());
        }
    }

    ~Server() { stop(); }

    Status start(std::string& err) {
        for (auto& e : engines_) {
            Status st = e->init_device(err);
            if (st != kOk) return st;
        }
        for (size_t w = 0; w < engines_.size(); w++) threads_.emplace_back([this, w] { worker((int)w); });
        return kOk;
    }

    void stop() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stopping_ = true;
        }
        cv_work_.notify_all();
        for (auto& t : threads_)
            if (t.joinable()) t.join();
        threads_.clear();
    }

    // Loads a parameter file into every worker's engine (same slot everywhere).
    int load_params(const std::string& path, std::string& err) {
        std::lock_guard<std::mutex> g(load_mu_);
        int slot = -1;
        for (size_t w = 0; w < engines_.size(); w++) {
            std::lock_guard<std::mutex> ge(*engine_mu_[w]);
            int s = engines_[w]->load_params(path, err);
            if (s < 0) return s;
            if (slot >= 0 && s != slot) {
                err = "parameter slots diverged between workers";
                return kErrState;
            }
            slot = s;
        }
        nslots_ = slot + 1;
        return slot;
    }

    long long submit(int slot, int n, const double* pos, const int* types, const double* cell, bool small,
                     std::string& err) {
        if (slot < 0 || slot >= nslots_) {
            err = "parameter set not loaded";
            return kErrState;
        }
        if (n <= 0) {
            err = "natom must be positive";
            return kErrInput;
        }
        std::unique_ptr<Request> r(new Request());
        r->slot = slot;
        r->n = n;
        r->pos.assign(pos, pos + 3 * (size_t)n);
        r->types.assign(types, types + n);
        std::memcpy(r->cell, cell, sizeof(r->cell));
        r->small = small;
        r->est_bytes = estimate_bytes(*r);
        r->t_submit = now_s();
        std::lock_guard<std::mutex> g(mu_);
        r->id = next_id_++;
        const long long id = r->id;
        queue_.push_back(r.get());
        all_[id] = std::move(r);
        submitted_++;
        cv_work_.notify_one();
        return id;
    }

    // 1 done (results copied, request released), 0 pending, < 0 failed (released)
    int take(long long id, bool wait, double timeout_s, double* energy, double* force, double* stress,
             double* latency, std::string& err) {
        std::unique_lock<std::mutex> g(mu_);
        auto it = all_.find(id);
        if (it == all_.end()) {
            err = "unknown request id";
            return kErrInput;
        }
        Request* r = it->second.get();
        if (!r->done && wait) {
            const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
            cv_done_.wait_until(g, deadline, [r] { return r->done; });
        }
        if (!r->done) return 0;
        int st = r->status;
        if (st == kOk) {
            if (energy) *energy = r->energy;
            if (force) std::memcpy(force, r->force.data(), sizeof(double) * r->force.size());
            if (stress) std::memcpy(stress, r->stress, sizeof(r->stress));
            if (latency) *latency = r->t_done - r->t_submit;
        } else {
            err = r->err;
        }
        all_.erase(it);
        return st == kOk ? 1 : st;
    }

    // Tunes worker 0's engine on a representative batch (Engine::autotune:
    // contraction form, lanes per cluster, resident blocks) and gives every
    // worker the same choices.  Meant for start-up, before requests arrive:
    // batches running meanwhile on other workers disturb the timings.
    Status autotune(const std::vector<SystemSpec>& specs, int* chosen, std::string& err) {
        std::lock_guard<std::mutex> g(load_mu_);
        ForceLaunch t;
        {
            std::lock_guard<std::mutex> ge(*engine_mu_[0]);
            Engine& e = *engines_[0];
            Status st = e.stage(specs, err);
            if (st != kOk) return st;
            st = e.autotune(chosen, err);
            if (st != kOk) return st;
            t = e.tuning;
        }
        for (size_t w = 1; w < engines_.size(); w++) {
            std::lock_guard<std::mutex> ge(*engine_mu_[w]);
            ForceLaunch& d = engines_[w]->tuning;
            d.tpc3 = t.tpc3, d.tpc4 = t.tpc4, d.blocks_per_sm = t.blocks_per_sm;
            d.ftpc3 = t.ftpc3, d.ftpc4 = t.ftpc4, d.fbps3 = t.fbps3, d.fbps4 = t.fbps4;
            d.want_fact3 = t.want_fact3, d.want_fact4 = t.want_fact4, d.noy3 = t.noy3;
            d.want_tc3 = t.want_tc3;
            d.want_tc4 = t.want_tc4;
        }
        return kOk;
    }

    // Offers a trace of requests at given arrival times (seconds from the
    // start) from one native thread and takes their results in order from
    // another, so that a client's own overhead does not cap what the server
    // shows; writes each request's latency (submit to result) and energy.
    // Returns the wall time from the first submission to the last result.
    Status replay(int nreq, const int* slots, const int* natoms, const double* pos, const int* types,
                  const double* cells, const int* small, const double* arrival, double* latency, double* energy,
                  double& wall, std::string& err) {
        std::vector<long long> off(nreq + 1, 0);
        for (int q = 0; q < nreq; q++) off[q + 1] = off[q] + natoms[q];
        std::vector<long long> ids(nreq, 0);
        std::vector<char> ready(nreq, 0);
        std::mutex mu;
        std::condition_variable cv;
        Status sub_status = kOk;
        std::string sub_err;
        const double t0 = now_s();
        std::thread submitter([&] {
            for (int q = 0; q < nreq; q++) {
                for (;;) {
                    const double dt = t0 + arrival[q] - now_s();
                    if (dt <= 0) break;
                    if (dt > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(dt - 1e-4));
                }
                std::string e;
                long long id = submit(slots[q], natoms[q], pos + 3 * off[q], types + off[q], cells + 9LL * q,
                                      small ? small[q] != 0 : false, e);
                std::lock_guard<std::mutex> g(mu);
                if (id < 0) {
                    sub_status = (Status)id;
                    sub_err = e;
                    for (int r = q; r < nreq; r++) ready[r] = 2;
                    cv.notify_all();
                    return;
                }
                ids[q] = id;
                ready[q] = 1;
                cv.notify_all();
            }
        });
        Status st = kOk;
        std::vector<double> force;
        for (int q = 0; q < nreq; q++) {
            {
                std::unique_lock<std::mutex> g(mu);
                cv.wait(g, [&] { return ready[q] != 0; });
                if (ready[q] == 2) {
                    st = sub_status;
                    err = sub_err;
                    break;
                }
            }
            force.resize(3 * (size_t)natoms[q]);
            double stress[9], e = 0.0, lat = 0.0;
            std::string terr;
            const int r = take(ids[q], true, 600.0, &e, force.data(), stress, &lat, terr);
            if (r != 1) {
                st = r < 0 ? (Status)r : kErrTimeout;
                err = r < 0 ? terr : "request not finished within 600 s";
                break;
            }
            if (latency) latency[q] = lat;
            if (energy) energy[q] = e;
        }
        wall = now_s() - t0;
        submitter.join();
        return st;
    }

    // worker w's launch preferences (the values ck_get_tuning reports, with
    // the contraction-form entries as preferences)
    Status worker_tuning(int w, int* out, std::string& err) {
        if (w < 0 || w >= (int)engines_.size()) {
            err = "no such worker";
            return kErrInput;
        }
        std::lock_guard<std::mutex> ge(*engine_mu_[w]);
        const ForceLaunch& L = engines_[w]->tuning;
        const int v[11] = {L.tpc3, L.tpc4, L.blocks_per_sm, L.want_fact3, L.want_fact4, L.ftpc3,
                           L.ftpc4, L.fbps3, L.fbps4, L.noy3, L.want_tc3 | (L.want_tc4 << 1)};
        for (int k = 0; k < 11; k++) out[k] = v[k];
        return kOk;
    }

    void stats(long long* out) {
        std::lock_guard<std::mutex> g(mu_);
        out[0] = submitted_;
        out[1] = completed_;
        out[2] = batches_;
        out[3] = max_batch_;
        out[4] = (long long)inflight_bytes_;
        out[5] = (long long)peak_inflight_bytes_;
    }

private:
    // Device bytes a request needs while in flight: ghost-image slots, bins,
    // lists and clusters, from the same host geometry the engine uses.
    double estimate_bytes(const Request& r) {
        std::lock_guard<std::mutex> g(load_mu_);
        const HostParams& P = engines_[0]->params(r.slot);
        SysDesc d;
        std::memset(&d, 0, sizeof(d));
        double vol = 0.0;
        std::string e;
        if (system_geometry(&r.cell[0], &r.cell[3], &r.cell[6], r.n, r.small, P.max_cut2(), P.max_cut3(),
                            P.max_cut4(), P.o3 > 0, P.o4 > 0, d, vol, e) != kOk)
            return 0.0;   // rejected later by the engine with its message
        const double rho = d.n_atoms / (vol > 0 ? vol : 1.0);
        const double m = rho * 4.18879 * d.search * d.search * d.search;
        const double n2 = d.n_atoms * (0.55 * m + 4);
        const double n3 = d.has3 ? d.n_atoms * (0.3 * m * m * std::pow(d.c3 / d.search, 6.0) + 4) : 0.0;
        const double n4 = d.has4 ? d.n_atoms * (0.1 * m * m * m * std::pow(d.c4 / d.search, 9.0) + 4) : 0.0;
        // pair lists ~70 B per pair plus the factored kernels' per-entry table cache
        // (~350 B per pair in FP64 for the 3- and 4-body orders), cluster lists
        // with their entry indices
        return (double)d.n_atoms * d.gstride * 110.0 + (double)d.bin_cap * 20.0 + n2 * 420.0 + n3 * 20.0 +
               n4 * 28.0 + d.n_atoms * 120.0;
    }

    void worker(int w) {
        for (;;) {
            std::vector<Request*> batch;
            double bytes = 0.0;
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_work_.wait(g, [this] { return stopping_ || admissible(); });
                if (stopping_ && queue_.empty()) return;
                long long atoms = 0;
                while (!queue_.empty()) {
                    Request* r = queue_.front();
                    const bool first = batch.empty();
                    if (!first && atoms + r->n > max_atoms_) break;
                    if (inflight_bytes_ + bytes + r->est_bytes > budget_ && !(first && inflight_bytes_ == 0.0)) break;
                    queue_.pop_front();
                    batch.push_back(r);
                    atoms += r->n;
                    bytes += r->est_bytes;
                }
                if (batch.empty()) continue;
                inflight_bytes_ += bytes;
                peak_inflight_bytes_ = std::max(peak_inflight_bytes_, inflight_bytes_);
            }
            run_batch(w, batch);
            {
                std::lock_guard<std::mutex> g(mu_);
                inflight_bytes_ -= bytes;
                if (inflight_bytes_ < 1e-6) inflight_bytes_ = 0.0;
                batches_++;
                max_batch_ = std::max(max_batch_, (long long)batch.size());
                completed_ += (long long)batch.size();
            }
            cv_done_.notify_all();
            cv_work_.notify_all();
        }
    }

    // the oldest waiting request fits the budget (always true when nothing is in flight)
    bool admissible() const {
        if (queue_.empty()) return false;
        return inflight_bytes_ == 0.0 || inflight_bytes_ + queue_.front()->est_bytes <= budget_;
    }

    void run_batch(int w, const std::vector<Request*>& batch) {
        Engine& eng = *engines_[w];
        std::vector<SystemSpec> specs(batch.size());
        long long total = 0;
        for (size_t i = 0; i < batch.size(); i++) {
            SystemSpec& s = specs[i];
            s.n = batch[i]->n;
            s.pos = batch[i]->pos.data();
            s.types = batch[i]->types.data();
            std::memcpy(s.cell, batch[i]->cell, sizeof(s.cell));
            s.small = batch[i]->small;
            s.pset = batch[i]->slot;
            total += s.n;
        }
        std::vector<double> force(3 * (size_t)total);
        std::vector<SystemResult> res;
        std::string err;
        Status st;
        {
            std::lock_guard<std::mutex> ge(*engine_mu_[w]);
            st = eng.run(specs, force.data(), res, err);
        }
        if (st != kOk && batch.size() > 1) {
            // isolate the failing request(s): evaluate each one alone
            for (Request* r : batch) run_batch(w, {r});
            return;
        }
        std::lock_guard<std::mutex> g(mu_);
        long long off = 0;
        const double t = now_s();
        for (size_t i = 0; i < batch.size(); i++) {
            Request* r = batch[i];
            r->status = st;
            if (st == kOk) {
                const SystemResult& q = res[i];
                r->energy = q.energy;
                const double* v = q.virial;
                const double full[9] = {v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]};
                for (int k = 0; k < 9; k++) r->stress[k] = full[k] / q.vol;
                r->force.assign(force.begin() + 3 * off, force.begin() + 3 * (off + r->n));
            } else {
                r->err = err;
            }
            r->t_done = t;
            r->done = true;
            off += r->n;
        }
    }

    std::vector<std::unique_ptr<Engine>> engines_;
    std::vector<std::unique_ptr<std::mutex>> engine_mu_;
    std::vector<std::thread> threads_;
    std::mutex mu_, load_mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<Request*> queue_;
    std::map<long long, std::unique_ptr<Request>> all_;
    long long next_id_ = 1;
    int nslots_ = 0;
    bool stopping_ = false;
    double budget_;
    long long max_atoms_;
    double inflight_bytes_ = 0.0, peak_inflight_bytes_ = 0.0;
    long long submitted_ = 0, completed_ = 0, batches_ = 0, max_batch_ = 0;
};

}  // namespace ck

extern "C" {

void* ck_server_open(int n_workers, double hbm_budget_gb, long long max_batch_atoms, int precision) {
    if (max_batch_atoms <= 0) max_batch_atoms = 1 << 20;
    if (!(hbm_budget_gb > 0)) hbm_budget_gb = 150.0;
    ck::Server* s = new ck::Server(n_workers, hbm_budget_gb * 1e9, max_batch_atoms, precision ? 1 : 0);
    std::string err;
    if (s->start(err) != ck::kOk) {
        delete s;
        ck::report_error(ck::kErrCuda, err);
        return nullptr;
    }
    return s;
}

void ck_server_close(void* s) { delete static_cast<ck::Server*>(s); }

int ck_server_load_params(void* s, const char* path) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    std::string err;
    int slot = static_cast<ck::Server*>(s)->load_params(path ? path : "", err);
    if (slot < 0) return ck::report_error(slot, err);
    return slot;
}

long long ck_server_submit(void* s, int slot, int natom, const double* pos, const int* types, const double* cell,
                           int small) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    std::string err;
    long long id = static_cast<ck::Server*>(s)->submit(slot, natom, pos, types, cell, small != 0, err);
    if (id < 0) return ck::report_error((int)id, err);
    return id;
}

int ck_server_take(void* s, long long id, int wait, double timeout_s, double* energy, double* force, double* stress,
                   double* latency_s) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    std::string err;
    int st = static_cast<ck::Server*>(s)->take(id, wait != 0, timeout_s, energy, force, stress, latency_s, err);
    if (st < 0) return ck::report_error(st, err);
    return st;
}

int ck_server_autotune(void* s, int nsys, const int* natoms, const double* pos, const int* types, const double* cells,
                       const int* small, const int* pset, int* chosen) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    if (nsys <= 0 || !natoms || !pos || !types || !cells) return ck::report_error(ck::kErrInput, "empty batch");
    std::vector<ck::SystemSpec> specs(nsys);
    long long off = 0;
    for (int i = 0; i < nsys; i++) {
        ck::SystemSpec& q = specs[i];
        q.n = natoms[i];
        if (q.n <= 0) return ck::report_error(ck::kErrInput, "natom must be positive");
        q.pos = pos + 3 * off;
        q.types = types + off;
        std::memcpy(q.cell, cells + 9 * (size_t)i, sizeof(q.cell));
        q.small = small ? small[i] != 0 : false;
        q.pset = pset ? pset[i] : 0;
        off += q.n;
    }
    std::string err;
    ck::Status st = static_cast<ck::Server*>(s)->autotune(specs, chosen, err);
    if (st != ck::kOk) return ck::report_error(st, err);
    return ck::kOk;
}

int ck_server_replay(void* s, int nreq, const int* slots, const int* natoms, const double* pos, const int* types,
                     const double* cells, const int* small, const double* arrival_s, double* latency_s,
                     double* energy, double* wall_s) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    if (nreq <= 0 || !slots || !natoms || !pos || !types || !cells || !arrival_s)
        return ck::report_error(ck::kErrInput, "empty request trace");
    std::string err;
    double wall = 0.0;
    ck::Status st = static_cast<ck::Server*>(s)->replay(nreq, slots, natoms, pos, types, cells, small, arrival_s,
                                                        latency_s, energy, wall, err);
    if (wall_s) *wall_s = wall;
    if (st != ck::kOk) return ck::report_error(st, err);
    return ck::kOk;
}

int ck_server_worker_tuning(void* s, int worker, int* out) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    std::string err;
    const ck::Status st = static_cast<ck::Server*>(s)->worker_tuning(worker, out, err);
    if (st != ck::kOk) return ck::report_error(st, err);
    return ck::kOk;
}

int ck_server_stats(void* s, long long* out) {
    if (!s) return ck::report_error(ck::kErrState, "no server");
    static_cast<ck::Server*>(s)->stats(out);
    return ck::kOk;
}

}  // extern "C"
