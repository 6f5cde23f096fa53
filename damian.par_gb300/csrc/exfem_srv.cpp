// exfem_srv.cpp — continuous-batching server over the exfem_gpu C ABI
// (include/exfem_srv.h).  Host code only: every device action goes through
// exfem_gpu_* on the request's own context and stream.
#include "exfem_host.h"
#include "exfem_srv.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

enum State { MESHING, WAITING, PREPARING, ACTIVE, DONE };

struct Req {
    long long id = 0;
    int nsteps = 0;
    State state = WAITING;
    int status = EXFEM_OK;
    std::string err;
    // deep copies of the caller's arrays and the views over them
    std::vector<int> eptr, eind, ematprop, absorbing, hanging, seismic, recv_elem, point_nodes;
    std::vector<unsigned char> ediv;
    std::vector<double> nodes, matconst, recv_xy;
    std::vector<exfem_wave> waves;
    exfem_mesh mesh{};
    exfem_problem prob{};
    std::string deck;                  // deck requests: the text, then the model built from it
    exfem_model *model = nullptr;
    size_t est = 0, held = 0, actual = 0;
    exfem_ctx *ctx = nullptr;
    int bypassed = 0;
    double t_submit = 0, t_meshed = 0, t_admit = 0, t_ready = 0, t_done = 0;
    std::vector<double> seis;
    bool reported = false;
    ~Req() {
        if (model) exfem_model_free(model);
    }
};

template <typename T>
void copy_arr(std::vector<T> &dst, const T *src, size_t n) {
    dst.assign(src, src + n);
}

}  // namespace

struct exfem_srv {
    exfem_srv_opts opts{};
    std::mutex mu;
    std::condition_variable cv_sched, cv_prep, cv_done;
    std::map<long long, Req *> reqs;
    std::deque<Req *> waiting;
    std::deque<Req *> prep_queue;
    std::deque<Req *> mesh_queue;   // deck requests to mesh
    int meshing = 0;
    std::vector<Req *> active;
    std::deque<Req *> finished;
    size_t budget = 0, held = 0;
    int preparing = 0, peak_active = 0;
    long long next_id = 1, n_finished = 0;
    bool stop = false;
    std::thread sched;
    std::vector<std::thread> preps;
    std::chrono::steady_clock::time_point t0;
    std::string err;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // Admission by HBM footprint, first fit in arrival order with a bounded
    // number of passes over the head request.  Called with mu held.
    void admit() {
        const int slots = opts.max_active;
        for (auto it = waiting.begin(); it != waiting.end();) {
            int running = (int)active.size() + preparing;
            if (running >= slots) break;
            Req *r = *it;
            bool head = (it == waiting.begin());
            if (held + r->est <= budget) {
                if (!head) waiting.front()->bypassed++;
                r->state = PREPARING;
                r->t_admit = now();
                r->held = r->est;
                held += r->est;
                preparing++;
                prep_queue.push_back(r);
                cv_prep.notify_one();
                it = waiting.erase(it);
                continue;
            }
            if (head && r->bypassed >= opts.max_bypass) break;   // the head waits for memory
            if (head && r->est > budget) {                          // can never fit
                r->status = EXFEM_E_NOMEM;
                r->err = "request needs more device memory than the server's budget";
                r->state = DONE;
                r->t_admit = r->t_ready = r->t_done = now();
                finished.push_back(r);
                n_finished++;
                cv_done.notify_all();
                it = waiting.erase(it);
                continue;
            }
            ++it;
        }
    }

    void finish(Req *r, int status) {   // mu held
        r->status = status;
        r->state = DONE;
        r->t_done = now();
        held -= std::min(held, r->held);
        r->held = 0;
        finished.push_back(r);
        n_finished++;
        cv_done.notify_all();
    }

    // Builds a deck request's model (no lock held), then queues it for
    // admission or finishes it with the deck's error.
    void mesh_one(Req *r) {
        exfem_model *m = nullptr;
        int rc = exfem_model_build(r->deck.c_str(), &m);
        if (!rc && r->nsteps > 0) rc = exfem_model_set_nsteps(m, r->nsteps);
        std::string msg = rc ? exfem_model_error() : std::string();
        size_t est = 0;
        if (!rc) {
            exfem_model_views(m, &r->mesh, &r->prob);
            r->nsteps = r->prob.nsteps;
            est = exfem_gpu_estimate_bytes(&r->mesh, &r->prob, &opts.solver);
        } else if (m) {
            exfem_model_free(m);
            m = nullptr;
        }
        std::lock_guard<std::mutex> lk(mu);
        meshing--;
        r->model = m;
        r->deck.clear();
        r->deck.shrink_to_fit();
        r->t_meshed = now();
        if (rc) {
            r->err = msg;
            r->t_admit = r->t_ready = r->t_meshed;
            finish(r, rc);
        } else {
            r->est = est;
            r->state = WAITING;
            waiting.push_back(r);
        }
        cv_sched.notify_one();
    }

    void prep_loop() {
        for (;;) {
            Req *r = nullptr;
            bool mesh_job = false;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_prep.wait(lk, [&] { return stop || !prep_queue.empty() || !mesh_queue.empty(); });
                if (stop && prep_queue.empty()) return;   // queued decks are dropped on close
                if (!prep_queue.empty()) {   // admitted requests first: they feed the GPU
                    r = prep_queue.front();
                    prep_queue.pop_front();
                } else {
                    r = mesh_queue.front();
                    mesh_queue.pop_front();
                    mesh_job = true;
                }
            }
            if (mesh_job) {
                mesh_one(r);
                continue;
            }
            exfem_ctx *ctx = nullptr;
            int rc = exfem_gpu_create(&r->mesh, &r->prob, &opts.solver, &ctx);
            std::string msg;
            if (rc) msg = exfem_gpu_last_error(nullptr);
            if (!rc) {
                rc = exfem_gpu_init_explicit(ctx, nullptr);
                if (rc) msg = exfem_gpu_last_error(ctx);
            }
            std::lock_guard<std::mutex> lk(mu);
            preparing--;
            if (rc) {
                if (ctx) exfem_gpu_destroy(ctx);
                r->err = msg;
                finish(r, rc);
            } else {
                r->ctx = ctx;
                r->actual = exfem_gpu_device_bytes(ctx);   // the reservation stays at the estimate
                r->t_ready = now();
                r->state = ACTIVE;
                active.push_back(r);
                peak_active = std::max(peak_active, (int)active.size());
            }
            cv_sched.notify_one();
        }
    }

    void sched_loop() {
        for (;;) {
            std::vector<Req *> act;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (stop) return;
                admit();
                act = active;
            }
            bool progressed = false;
            std::vector<std::pair<Req *, int>> done_now;
            for (Req *r : act) {
                int q = exfem_gpu_query(r->ctx);
                if (q == 1) continue;   // still running its queued chunks
                if (q < 0) { done_now.push_back({r, q}); continue; }
                int left = r->nsteps - exfem_gpu_steps_done(r->ctx);
                if (left > 0) {
                    int chunk = std::min(left, 2 * opts.chunk_steps);   // two chunks queued per round
                    int rc = exfem_gpu_run(r->ctx, chunk);
                    if (rc) done_now.push_back({r, rc});
                    progressed = true;
                } else {
                    int nsave = 0;
                    exfem_gpu_get_seismograms(r->ctx, nullptr, 0, &nsave);
                    size_t n = (size_t)r->prob.nrhs * (size_t)(r->nsteps / r->prob.io_interval + 1) * r->prob.nrecv * 2;
                    r->seis.assign(n, 0.0);
                    int rc = n ? exfem_gpu_get_seismograms(r->ctx, r->seis.data(), n, &nsave) : EXFEM_OK;
                    done_now.push_back({r, rc});
                    progressed = true;
                }
            }
            if (!done_now.empty()) {
                for (auto &pr : done_now) {
                    Req *r = pr.first;
                    if (pr.second) r->err = exfem_gpu_last_error(r->ctx);
                    exfem_gpu_destroy(r->ctx);
                    r->ctx = nullptr;
                }
                std::lock_guard<std::mutex> lk(mu);
                for (auto &pr : done_now) {
                    active.erase(std::remove(active.begin(), active.end(), pr.first), active.end());
                    finish(pr.first, pr.second);
                }
            }
            if (!progressed) {
                std::unique_lock<std::mutex> lk(mu);
                cv_sched.wait_for(lk, std::chrono::microseconds(200));
            }
        }
    }
};

extern "C" {

void exfem_srv_default_opts(exfem_srv_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_active = 16;
    o->chunk_steps = 256;
    o->preparers = 4;
    o->max_bypass = 8;
    exfem_gpu_default_opts(&o->solver);
    o->solver.precision = EXFEM_FP32_KAHAN;
    // requests stepping at once hide each other's DRM pass: no second stream
    o->solver.drm_inline = 1;
}

int exfem_srv_open(const exfem_srv_opts *opts, exfem_srv **out) {
    if (!out) return EXFEM_E_ARG;
    *out = nullptr;
    exfem_srv *s = new (std::nothrow) exfem_srv();
    if (!s) return EXFEM_E_NOMEM;
    if (opts) s->opts = *opts;
    else exfem_srv_default_opts(&s->opts);
    exfem_srv_opts &o = s->opts;
    if (o.max_active <= 0) o.max_active = 16;
    if (o.chunk_steps <= 0) o.chunk_steps = 256;
    if (o.preparers <= 0) o.preparers = 4;
    if (o.max_bypass <= 0) o.max_bypass = 8;
    o.solver.use_graph = o.solver.use_graph ? 1 : 0;
    s->budget = o.hbm_budget;
    if (s->budget == 0) {
        size_t fr = 0, tot = 0;
        if (cudaSetDevice(o.solver.device) != cudaSuccess || cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            delete s;
            return EXFEM_E_CUDA;
        }
        s->budget = (size_t)(0.9 * (double)fr);
    }
    s->t0 = std::chrono::steady_clock::now();
    try {
        s->sched = std::thread([s] { s->sched_loop(); });
        for (int i = 0; i < o.preparers; ++i) s->preps.emplace_back([s] { s->prep_loop(); });
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_prep.notify_all();
        if (s->sched.joinable()) s->sched.join();
        for (auto &t : s->preps) if (t.joinable()) t.join();
        delete s;
        return EXFEM_E_NOMEM;
    }
    *out = s;
    return EXFEM_OK;
}

int exfem_srv_submit(exfem_srv *s, const exfem_mesh *mesh, const exfem_problem *prob, int nsteps, long long *id) {
    if (!s || !mesh || !prob || nsteps < 0 || nsteps > prob->nsteps) return EXFEM_E_ARG;
    Req *r = new (std::nothrow) Req();
    if (!r) return EXFEM_E_NOMEM;
    try {
        size_t L = (size_t)(mesh->eptr[mesh->nelems] - 1);
        copy_arr(r->eptr, mesh->eptr, (size_t)mesh->nelems + 1);
        copy_arr(r->eind, mesh->eind, L);
        copy_arr(r->ediv, mesh->ediv, L);
        copy_arr(r->nodes, mesh->nodes, 2 * (size_t)mesh->nnodes);
        copy_arr(r->ematprop, mesh->ematprop, (size_t)mesh->nelems);
        copy_arr(r->matconst, prob->matconst, 5 * (size_t)prob->nmat);
        copy_arr(r->absorbing, prob->absorbing, (size_t)mesh->nnodes);
        if (prob->nhanging) copy_arr(r->hanging, prob->hanging, 3 * (size_t)prob->nhanging);
        if (prob->nseismic) copy_arr(r->seismic, prob->seismic, 2 * (size_t)prob->nseismic);
        if (prob->waves) copy_arr(r->waves, prob->waves, (size_t)prob->nrhs);
        if (prob->npoint > 0 && prob->point_nodes) copy_arr(r->point_nodes, prob->point_nodes, (size_t)prob->npoint);
        if (prob->nrecv) {
            copy_arr(r->recv_xy, prob->recv_xy, 2 * (size_t)prob->nrecv);
            copy_arr(r->recv_elem, prob->recv_elem, (size_t)prob->nrecv);
        }
    } catch (...) {
        delete r;
        return EXFEM_E_NOMEM;
    }
    r->mesh = *mesh;
    r->mesh.eptr = r->eptr.data(); r->mesh.eind = r->eind.data(); r->mesh.ediv = r->ediv.data();
    r->mesh.nodes = r->nodes.data(); r->mesh.ematprop = r->ematprop.data();
    r->prob = *prob;
    r->prob.matconst = r->matconst.data(); r->prob.absorbing = r->absorbing.data();
    r->prob.hanging = r->hanging.empty() ? nullptr : r->hanging.data();
    r->prob.seismic = r->seismic.empty() ? nullptr : r->seismic.data();
    r->prob.waves = r->waves.empty() ? nullptr : r->waves.data();
    r->prob.point_nodes = r->point_nodes.empty() ? nullptr : r->point_nodes.data();
    r->prob.recv_xy = r->recv_xy.empty() ? nullptr : r->recv_xy.data();
    r->prob.recv_elem = r->recv_elem.empty() ? nullptr : r->recv_elem.data();
    r->prob.nsteps = nsteps;
    r->nsteps = nsteps;
    r->est = exfem_gpu_estimate_bytes(&r->mesh, &r->prob, &s->opts.solver);
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    r->t_submit = r->t_meshed = s->now();
    s->reqs[r->id] = r;
    s->waiting.push_back(r);
    if (id) *id = r->id;
    s->cv_sched.notify_one();
    return EXFEM_OK;
}

int exfem_srv_submit_deck(exfem_srv *s, const char *deck, int nsteps, long long *id) {
    if (!s || !deck) return EXFEM_E_ARG;
    Req *r = new (std::nothrow) Req();
    if (!r) return EXFEM_E_NOMEM;
    try {
        r->deck = deck;
    } catch (...) {
        delete r;
        return EXFEM_E_NOMEM;
    }
    r->nsteps = nsteps > 0 ? nsteps : 0;
    r->state = MESHING;
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    r->t_submit = s->now();
    s->reqs[r->id] = r;
    s->mesh_queue.push_back(r);
    s->meshing++;
    if (id) *id = r->id;
    s->cv_prep.notify_one();
    return EXFEM_OK;
}

int exfem_srv_poll(exfem_srv *s, exfem_srv_result *out, int cap, int wait_ms) {
    if (!s || (!out && cap > 0)) return EXFEM_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->finished.empty() && wait_ms > 0)
        s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->finished.empty(); });
    int n = 0;
    while (n < cap && !s->finished.empty()) {
        Req *r = s->finished.front();
        s->finished.pop_front();
        r->reported = true;
        exfem_srv_result &o = out[n++];
        o.id = r->id;
        o.status = r->status;
        o.nsteps = r->nsteps;
        o.nelems = r->mesh.nelems;
        o.nrhs = r->prob.nrhs;
        o.nrecv = r->prob.nrecv;
        o.nsave = r->prob.io_interval > 0 ? r->nsteps / r->prob.io_interval + 1 : 0;
        o.device_bytes = r->actual;
        o.reserved_bytes = r->est;
        o.t_submit = r->t_submit;
        o.t_meshed = r->t_meshed;
        o.t_admit = r->t_admit;
        o.t_ready = r->t_ready;
        o.t_done = r->t_done;
    }
    return n;
}

int exfem_srv_fetch(exfem_srv *s, long long id, double *out, size_t cap) {
    if (!s) return EXFEM_E_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { s->err = "unknown request id"; return EXFEM_E_ARG; }
    Req *r = it->second;
    if (r->state != DONE) { s->err = "request not finished"; return EXFEM_E_STATE; }
    if (r->status != EXFEM_OK) { s->err = r->err; int st = r->status; s->reqs.erase(it); delete r; return st; }
    if (out) {
        if (cap < r->seis.size()) { s->err = "buffer too small"; return EXFEM_E_ARG; }
        std::memcpy(out, r->seis.data(), r->seis.size() * sizeof(double));
    }
    s->reqs.erase(it);
    delete r;
    return EXFEM_OK;
}

int exfem_srv_stats(exfem_srv *s, int *waiting, int *preparing, int *active, long long *finished, size_t *bytes,
                    int *peak_active) {
    if (!s) return EXFEM_E_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (waiting) *waiting = (int)s->waiting.size() + s->meshing;   // deck requests still meshing count as waiting
    if (preparing) *preparing = s->preparing;
    if (active) *active = (int)s->active.size();
    if (finished) *finished = s->n_finished;
    if (bytes) *bytes = s->held;
    if (peak_active) *peak_active = s->peak_active;
    return EXFEM_OK;
}

const char *exfem_srv_last_error(const exfem_srv *s) { return s ? s->err.c_str() : ""; }

void exfem_srv_close(exfem_srv *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_prep.notify_all();
    s->cv_sched.notify_all();
    if (s->sched.joinable()) s->sched.join();
    for (auto &t : s->preps) if (t.joinable()) t.join();
    for (auto &kv : s->reqs) {
        if (kv.second->ctx) exfem_gpu_destroy(kv.second->ctx);
        delete kv.second;
    }
    delete s;
}

}  // extern "C"
