// Serving loop: LES cases arrive at any time, are admitted while their
// device footprint fits an HBM budget, stay resident on the GPU for their
// whole run, and advance together.  Resident cases are grouped in size
// buckets (same grid shape and options); a bucket advances all its cases one
// step at a time through one captured CUDA graph -- every case's kernels on
// its own stream branch, and for the multigrid Poisson solvers the mode
// solves of all the bucket's cases as one batched launch per substep -- and
// the worker keeps a chunk of bucket steps in flight on every bucket, so the
// work of different buckets overlaps on the device as well.  A case that
// finishes is read back and freed at once (its bucket's graph is captured
// again without it), and the freed memory admits the next waiting case
// (continuous batching, not a queue in front of a single solver).
//
// The API (include/lesgpu.h, lesgpu_server_*) copies every input at
// submission, so the caller's buffers are free on return; results are
// copied out on request.  All CUDA work happens on the worker thread.
#include <cstdlib>

#include "lesgpu_internal.cuh"
#include <stdlib.h>
#include <string.h>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// deep copy of a lesgpu_grid
struct GridCopy {
    lesgpu_grid g;
    std::vector<double> d[18];
    std::vector<int64_t> iv[12];
    void set(const lesgpu_grid *src) {
        g = *src;
        const double *dsrc[18] = {src->x, src->y, src->z, src->c2cx, src->c2cy, src->c2cz, src->c2cxi, src->c2cyi,
                                  src->c2czi, src->f2fx, src->f2fy, src->f2fz, src->f2fxi, src->f2fyi, src->f2fzi,
                                  src->xmp, src->ymp, src->zmp};
        const size_t dn[18] = {(size_t)src->n1, (size_t)src->n2, (size_t)src->n3,
                               (size_t)src->n1 + 1, (size_t)src->n2 + 1, (size_t)src->n3 + 1,
                               (size_t)src->n1 + 1, (size_t)src->n2 + 1, (size_t)src->n3 + 1,
                               (size_t)src->n1 + 1, (size_t)src->n2 + 1, (size_t)src->n3 + 1,
                               (size_t)src->n1 + 1, (size_t)src->n2 + 1, (size_t)src->n3 + 1,
                               (size_t)src->n1 + 1, (size_t)src->n2 + 1, (size_t)src->n3 + 1};
        const double **ddst[18] = {&g.x, &g.y, &g.z, &g.c2cx, &g.c2cy, &g.c2cz, &g.c2cxi, &g.c2cyi, &g.c2czi,
                             &g.f2fx, &g.f2fy, &g.f2fz, &g.f2fxi, &g.f2fyi, &g.f2fzi, &g.xmp, &g.ymp, &g.zmp};
        for (int q = 0; q < 18; q++) {
            d[q].assign(dsrc[q], dsrc[q] + dn[q]);
            *ddst[q] = d[q].data();
        }
        const int64_t *isrc[12] = {src->ipv, src->jpv, src->kpv, src->imv, src->jmv, src->kmv,
                                   src->fixil, src->fixjl, src->fixkl, src->fixiu, src->fixju, src->fixku};
        const size_t in[12] = {(size_t)src->n1m, (size_t)src->n2m, (size_t)src->n3m, (size_t)src->n1m, (size_t)src->n2m,
                               (size_t)src->n3m, (size_t)src->n1m, (size_t)src->n2m, (size_t)src->n3m,
                               (size_t)src->n1m, (size_t)src->n2m, (size_t)src->n3m};
        const int64_t **idst[12] = {&g.ipv, &g.jpv, &g.kpv, &g.imv, &g.jmv, &g.kmv,
                              &g.fixil, &g.fixjl, &g.fixkl, &g.fixiu, &g.fixju, &g.fixku};
        for (int q = 0; q < 12; q++) {
            iv[q].assign(isrc[q], isrc[q] + in[q]);
            *idst[q] = iv[q].data();
        }
    }
};

// deep copy of a lesgpu_ibm
struct IbmCopy {
    lesgpu_ibm b;
    std::vector<int64_t> fc[4], ix[4], nz[3], nwall, omega;
    std::vector<double> gf[4], cstar, kstar;
    void set(const lesgpu_ibm *src, size_t ncell) {
        b = *src;
        for (int l = 0; l < 4; l++) {
            size_t nb = src->nbody[l] > 0 ? (size_t)src->nbody[l] : 0, ni = src->nintp[l] > 0 ? (size_t)src->nintp[l] : 0;
            fc[l].assign(src->fc[l] ? src->fc[l] : nullptr, src->fc[l] ? src->fc[l] + 3 * nb : nullptr);
            ix[l].assign(src->intpindx[l] ? src->intpindx[l] : nullptr, src->intpindx[l] ? src->intpindx[l] + 3 * ni : nullptr);
            gf[l].assign(src->geomfac[l] ? src->geomfac[l] : nullptr, src->geomfac[l] ? src->geomfac[l] + 27 * ni : nullptr);
            b.fc[l] = fc[l].empty() ? nullptr : fc[l].data();
            b.intpindx[l] = ix[l].empty() ? nullptr : ix[l].data();
            b.geomfac[l] = gf[l].empty() ? nullptr : gf[l].data();
        }
        size_t nz0 = src->nzero > 0 ? (size_t)src->nzero : 0;
        const int64_t *zs[3] = {src->inz, src->jnz, src->knz};
        const int64_t **zd[3] = {&b.inz, &b.jnz, &b.knz};
        for (int q = 0; q < 3; q++) {
            nz[q].assign(zs[q] ? zs[q] : nullptr, zs[q] ? zs[q] + nz0 : nullptr);
            *zd[q] = nz[q].empty() ? nullptr : nz[q].data();
        }
        auto cp_i = [&](const int64_t *s, std::vector<int64_t> &v, const int64_t *&dst) {
            if (s) { v.assign(s, s + ncell); dst = v.data(); } else dst = nullptr;
        };
        auto cp_d = [&](const double *s, std::vector<double> &v, const double *&dst, size_t n) {
            if (s) { v.assign(s, s + n); dst = v.data(); } else dst = nullptr;
        };
        cp_i(src->nwall_dvm, nwall, b.nwall_dvm);
        cp_i(src->omega, omega, b.omega);
        cp_d(src->cstar, cstar, b.cstar, ncell);
        cp_d(src->kstar, kstar, b.kstar, 6 * ncell);
    }
};

enum { S_PENDING = 0, S_ACTIVE = 1, S_DONE = 2, S_FAILED = 3, S_CANCELLED = 4 };

struct Request {
    int64_t ticket = 0;
    lesgpu_config cfg;
    GridCopy grid;
    IbmCopy ibm;
    bool has_ibm = false;
    std::vector<double> f[5];
    double time0 = 0, dt0 = 0;
    int64_t ihist0 = 0, m0 = 0, nsteps = 0;
    // progress
    int state = S_PENDING;
    int rc = 0;
    lesgpu_case *c = nullptr;
    int64_t done = 0, inflight = 0;   // steps completed; steps of its bucket's work in flight
    size_t footprint = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    lesgpu_step_report rep;
};

}  // namespace

struct lesgpu_server {
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request *> pending;
    std::vector<Request *> active;
    std::map<int64_t, Request *> all;
    std::map<long long, size_t> bucket_bytes;     // measured footprint per size bucket
    size_t budget = 0, used = 0;
    int max_active = 64;
    int64_t chunk = 4;          // steps in flight per bucket
    int device = 0;
    int64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    // statistics
    double busy_cell_steps = 0;
};

namespace {

long long bucket_key(const Request *r) {
    const lesgpu_config &c = r->cfg;
    const lesgpu_grid &g = r->grid.g;
    return ((((((long long)g.n1m * 4099 + g.n2m) * 4099 + g.n3m) * 4 + c.poisson) * 2 + c.iles) * 2 + c.ihtrans) * 2 +
           c.precision;
}

// first-case estimate of a bucket: ~130 FP64 words per cell of the padded grid
size_t estimate_bytes(const Request *r) {
    const lesgpu_grid &g = r->grid.g;
    size_t nt = (size_t)(g.n1 + 1) * (g.n2 + 1) * (g.n3 + 1);
    return nt * 8 * 130 + (64u << 20);
}

void finish(lesgpu_server *S, Request *r, int state) {
    if (r->c) {
        if (state == S_DONE) {
            for (int q = 0; q < 5; q++) r->f[q].resize((size_t)(r->grid.g.n1 + 1) * (r->grid.g.n2 + 1) * (r->grid.g.n3 + 1));
            int rc = lesgpu_get_fields(r->c, r->f[0].data(), r->f[1].data(), r->f[2].data(), r->f[3].data(), r->f[4].data());
            if (!rc) rc = lesgpu_get_report(r->c, &r->rep);
            if (rc) { r->rc = rc; state = S_FAILED; }
        }
        lesgpu_destroy(r->c);
        r->c = nullptr;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->used -= r->footprint;
    r->footprint = 0;
    r->state = state;
    r->t_done = now_s();
}

int admit(lesgpu_server *S, Request *r) {
    size_t free0 = 0, total = 0;
    cudaMemGetInfo(&free0, &total);
    int rc = lesgpu_create(&r->cfg, &r->grid.g, &r->c);
    if (!rc && r->has_ibm) rc = lesgpu_load_ibm(r->c, &r->ibm.b);
    if (!rc) rc = lesgpu_set_fields(r->c, r->f[0].data(), r->f[1].data(), r->f[2].data(), r->f[3].data(),
                                    r->f[4].empty() ? nullptr : r->f[4].data(), r->time0, r->dt0, r->ihist0, r->m0);
    if (!rc) rc = lesgpu_start(r->c);
    size_t free1 = 0;
    cudaMemGetInfo(&free1, &total);
    size_t fp = free0 > free1 ? free0 - free1 : 0;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        long long key = bucket_key(r);
        if (!rc && fp > 0) S->bucket_bytes[key] = fp;
        // the admission reserved an estimate; book the measured size instead
        S->used -= r->footprint;
        r->footprint = fp;
        S->used += fp;
        r->t_admit = now_s();
        if (!rc) r->state = S_ACTIVE;
    }
    // the host copies of the inputs are on the device now
    if (!rc)
        for (int q = 0; q < 5; q++) std::vector<double>().swap(r->f[q]);
    return rc;
}

struct Bucket {
    std::vector<Request *> members;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    lg::BucketGraph bg;
    bool valid = false;            // bg holds a step of exactly these members
    int64_t inflight = 0;          // bucket steps enqueued since the last completed event
};

void destroy_bucket(Bucket &B) {
    lg::free_bucket_graph(&B.bg);
    if (B.ev) cudaEventDestroy(B.ev);
    if (B.st) cudaStreamDestroy(B.st);
    B.ev = nullptr;
    B.st = nullptr;
}

void remove_active(lesgpu_server *S, Request *r) {
    std::lock_guard<std::mutex> lk(S->mu);
    for (size_t q = 0; q < S->active.size(); q++)
        if (S->active[q] == r) { S->active.erase(S->active.begin() + q); break; }
}

void worker_main(lesgpu_server *S) {
    cudaSetDevice(S->device);
    std::map<std::pair<std::pair<long long, long long>, int>, Bucket> buckets;
    // LESGPU_SERVER_BUCKET_MAX: cases per bucket at most (a full bucket's
    // shape opens another one); 0: no limit.  Default 1: on the benchmark
    // stream (16 cases arriving at once) one case per graph served 128
    // Mcell-steps/s against 117 with whole buckets in one graph -- the
    // batched solve joins every case of its bucket before each Poisson
    // solve, while separate graphs let the cases' phases overlap freely
    const char *bm = getenv("LESGPU_SERVER_BUCKET_MAX");
    const size_t bucket_max = bm ? (atoi(bm) >= 1 ? (size_t)atoi(bm) : (size_t)-1) : 1;
    // resident cases share the GPU: their multigrid solves are latency-bound,
    // so each gets small clusters and the solves of different cases run side
    // by side (4 blocks per cluster served the benchmark stream fastest, 128
    // Mcell-steps/s against 122 with 2 and 101 with 8)
    const char *cap = getenv("LESGPU_SERVER_MG_CLUSTER");
    lg::set_mg_cluster_cap(cap && atoi(cap) >= 1 ? atoi(cap) : 4);
    for (;;) {
        // ---- admission
        for (;;) {
            Request *r = nullptr;
            {
                std::unique_lock<std::mutex> lk(S->mu);
                if (S->stop) break;
                if (S->pending.empty() || (int)S->active.size() >= S->max_active) break;
                Request *cand = S->pending.front();
                auto it = S->bucket_bytes.find(bucket_key(cand));
                size_t need = it != S->bucket_bytes.end() ? it->second : estimate_bytes(cand);
                if (S->used + need > S->budget && !S->active.empty()) break;   // wait for memory
                S->pending.pop_front();
                cand->footprint = need;
                S->used += need;
                r = cand;
            }
            int rc = admit(S, r);
            if (!rc && r->cfg.iread == 0 && r->nsteps > 0) {
                // the first step of a fresh start differs from the others
                // (the SGS model starts from zero): it runs on the case's own
                // path, the bucket graphs hold steady-state steps only
                rc = lesgpu_step_async(r->c, 1);
                if (!rc && cudaStreamSynchronize(r->c->stream) != cudaSuccess) rc = LESGPU_ERR_CUDA;
                if (!rc) {
                    r->done = 1;
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->busy_cell_steps += (double)r->grid.g.n1m * r->grid.g.n2m * r->grid.g.n3m;
                }
            }
            if (rc) {
                r->rc = rc;
                finish(S, r, S_FAILED);
                continue;
            }
            {
                std::lock_guard<std::mutex> lk(S->mu);
                S->active.push_back(r);
            }
            // a bucket is the cases of one shape and options that can share
            // a batched solve (the same multigrid cluster size and levels)
            const std::pair<long long, long long> shape(bucket_key(r), lg::mg2d_batch_key(r->c));
            int slot = 0;
            for (;; slot++) {
                auto f = buckets.find(std::make_pair(shape, slot));
                if (f == buckets.end() || f->second.members.size() < bucket_max) break;
            }
            Bucket &B = buckets[std::make_pair(shape, slot)];
            if (!B.st) {
                if (cudaStreamCreateWithFlags(&B.st, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaEventCreateWithFlags(&B.ev, cudaEventDisableTiming) != cudaSuccess)
                    r->rc = LESGPU_ERR_CUDA;
            }
            B.members.push_back(r);
            B.valid = false;
        }
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->stop) break;
            if (S->active.empty()) {
                S->cv.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
        }
        // ---- keep a chunk of bucket steps in flight on every bucket
        bool progressed = false;
        for (auto it = buckets.begin(); it != buckets.end();) {
            Bucket &B = it->second;
            if (B.inflight > 0) {
                cudaError_t e = cudaEventQuery(B.ev);
                if (e == cudaErrorNotReady) { ++it; continue; }
                for (Request *r : B.members) {     // a case admitted meanwhile has nothing in flight
                    if (r->inflight == 0) continue;
                    if (e != cudaSuccess) r->rc = LESGPU_ERR_CUDA;
                    r->done += r->inflight;
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->busy_cell_steps += (double)r->inflight * r->grid.g.n1m * r->grid.g.n2m * r->grid.g.n3m;
                    r->inflight = 0;
                }
                B.inflight = 0;
                progressed = true;
            }
            // finished, failed and cancelled cases leave the bucket (nothing
            // of the bucket is in flight here)
            for (size_t q = 0; q < B.members.size();) {
                Request *r = B.members[q];
                bool cancelled;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    cancelled = r->state == S_CANCELLED;
                }
                if (r->rc || cancelled || r->done >= r->nsteps) {
                    finish(S, r, r->rc ? S_FAILED : cancelled ? S_CANCELLED : S_DONE);
                    remove_active(S, r);
                    B.members.erase(B.members.begin() + q);
                    B.valid = false;
                    progressed = true;
                } else {
                    q++;
                }
            }
            if (B.members.empty()) {
                destroy_bucket(B);
                it = buckets.erase(it);
                continue;
            }
            std::vector<lesgpu_case *> cs;
            int64_t n = S->chunk;
            for (Request *r : B.members) {
                cs.push_back(r->c);
                n = std::min<int64_t>(n, r->nsteps - r->done);
            }
            int rc = 0;
            if (!B.valid) {
                rc = lg::capture_bucket_step(cs.data(), (int)cs.size(), B.st, &B.bg);
                B.valid = rc == 0;
            }
            if (!rc) rc = lg::bucket_prologue(cs.data(), (int)cs.size());
            int64_t launched = 0;
            for (int64_t k = 0; k < n && !rc; k++) {
                if (cudaGraphLaunch(B.bg.exec, B.st) != cudaSuccess) rc = LESGPU_ERR_CUDA;
                else launched++;
            }
            if (!rc && cudaEventRecord(B.ev, B.st) != cudaSuccess) rc = LESGPU_ERR_CUDA;
            if (rc) {
                // nothing of theirs may be in flight when the members are freed
                if (launched > 0) cudaStreamSynchronize(B.st);
                for (Request *r : B.members) r->rc = rc;     // they leave at the next pass
                ++it;
                continue;
            }
            lg::bucket_replayed(cs.data(), (int)cs.size(), (int)n);
            for (Request *r : B.members) r->inflight = n;
            B.inflight = n;
            ++it;
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    // shutdown: wait for the work in flight, drop whatever is still resident
    for (auto &kv : buckets) {
        if (kv.second.inflight > 0) cudaEventSynchronize(kv.second.ev);
        destroy_bucket(kv.second);
    }
    buckets.clear();
    for (Request *r : S->active) finish(S, r, S_CANCELLED);
    S->active.clear();
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" int lesgpu_server_create(int64_t device, int64_t hbm_budget_bytes, int64_t max_active,
                                    int64_t steps_in_flight, lesgpu_server **out) {
    if (!out || hbm_budget_bytes <= 0 || max_active < 1 || steps_in_flight < 1 || device < 0) return LESGPU_ERR_ARG;
    lesgpu_server *S = new lesgpu_server();
    S->device = (int)device;
    S->budget = (size_t)hbm_budget_bytes;
    S->max_active = (int)max_active;
    S->chunk = steps_in_flight;
    S->worker = std::thread(worker_main, S);
    *out = S;
    return 0;
}

extern "C" int lesgpu_server_submit(lesgpu_server *S, const lesgpu_config *cfg, const lesgpu_grid *grid,
                                    const lesgpu_ibm *ibm, const double *u, const double *v, const double *w,
                                    const double *p, const double *t, double time, double dt, int64_t ihist,
                                    int64_t m, int64_t nsteps, int64_t *ticket) {
    if (!S || !cfg || !grid || !u || !v || !w || !p || !ticket || nsteps < 1) return LESGPU_ERR_ARG;
    if (grid->n1 != grid->n1m + 1 || grid->n2 != grid->n2m + 1 || grid->n3 != grid->n3m + 1 || grid->n1m < 2 ||
        grid->n2m < 2 || grid->n3m < 1)
        return LESGPU_ERR_ARG;
    Request *r = new Request();
    r->cfg = *cfg;
    r->grid.set(grid);
    size_t nt = (size_t)(grid->n1 + 1) * (grid->n2 + 1) * (grid->n3 + 1);
    if (ibm) {
        r->ibm.set(ibm, (size_t)grid->n1m * grid->n2m * grid->n3m);
        r->has_ibm = true;
    }
    const double *src[5] = {u, v, w, p, t};
    for (int q = 0; q < 5; q++)
        if (src[q]) r->f[q].assign(src[q], src[q] + nt);
    r->time0 = time; r->dt0 = dt; r->ihist0 = ihist; r->m0 = m; r->nsteps = nsteps;
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->ticket = S->next_ticket++;
        S->all[r->ticket] = r;
        S->pending.push_back(r);
    }
    S->cv.notify_one();
    *ticket = r->ticket;
    return 0;
}

extern "C" int lesgpu_server_poll(lesgpu_server *S, int64_t ticket, int64_t *state, int64_t *steps_done) {
    if (!S || !state) return LESGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return LESGPU_ERR_ARG;
    *state = it->second->state;
    if (steps_done) *steps_done = it->second->done;
    return 0;
}

extern "C" int lesgpu_server_result(lesgpu_server *S, int64_t ticket, double *u, double *v, double *w, double *p,
                                    double *t, lesgpu_step_report *rep, double *seconds_to_solution) {
    if (!S) return LESGPU_ERR_ARG;
    Request *r;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->all.find(ticket);
        if (it == S->all.end()) return LESGPU_ERR_ARG;
        r = it->second;
        if (r->state == S_FAILED) return r->rc ? r->rc : LESGPU_ERR_CUDA;
        if (r->state != S_DONE) return LESGPU_ERR_STATE;
    }
    size_t nt = r->f[0].size();
    double *dst[5] = {u, v, w, p, t};
    for (int q = 0; q < 5; q++)
        if (dst[q]) memcpy(dst[q], r->f[q].data(), nt * sizeof(double));
    if (rep) *rep = r->rep;
    if (seconds_to_solution) *seconds_to_solution = r->t_done - r->t_submit;
    return 0;
}

// Drop a finished request's stored results (or cancel a waiting / running one).
extern "C" int lesgpu_server_release(lesgpu_server *S, int64_t ticket) {
    if (!S) return LESGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return LESGPU_ERR_ARG;
    Request *r = it->second;
    if (r->state == S_PENDING) {
        for (auto q = S->pending.begin(); q != S->pending.end(); ++q)
            if (*q == r) { S->pending.erase(q); break; }
        r->state = S_CANCELLED;
    } else if (r->state == S_ACTIVE) {
        r->state = S_CANCELLED;        // the worker frees it at its next pass
        return 0;
    }
    S->all.erase(it);
    delete r;
    return 0;
}

extern "C" int lesgpu_server_stats(lesgpu_server *S, int64_t *pending, int64_t *active, int64_t *bytes_used,
                                   double *cell_steps) {
    if (!S) return LESGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    if (pending) *pending = (int64_t)S->pending.size();
    if (active) *active = (int64_t)S->active.size();
    if (bytes_used) *bytes_used = (int64_t)S->used;
    if (cell_steps) *cell_steps = S->busy_cell_steps;
    return 0;
}

extern "C" int lesgpu_server_destroy(lesgpu_server *S) {
    if (!S) return 0;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (auto &kv : S->all) delete kv.second;
    delete S;
    return 0;
}
