// server.cpp -- continuous-batching request loop over the GPU engine.
//
// Requests (a case, its initial state and a number of steps) are submitted by
// any thread into a lock-protected queue. Each storage type (FP64, FP32-, FP16-
// shifted) has its own lane: a thread that repeats rounds of
//   1. taking queued requests of its storage type in arrival order while the
//      device's free memory (read live each round, less a reserve) and the
//      slot limit (over all lanes) allow, and the optional budget;
//   2. launching one chunk for its active requests: they form one Batch (one
//      persistent kernel per step over all their tiles, graph-captured),
//      reused from the previous round while the set of requests is the same;
//      a chunk is the smallest remaining step count of the set, capped at the
//      chunk size, so requests join and leave between chunks;
//   3. while that chunk runs on the device, admitting the requests taken in 1
//      (device setup and state upload on their own streams);
//   4. waiting for the chunk and retiring finished requests: their fields (and,
//      on request, populations and impedance spectra) are copied to host memory
//      and their device memory is returned to the pool (stream-ordered, so no
//      device-wide synchronization).
// The lanes' batches run concurrently on their own streams. Because
// Solver::run(a) followed by run(b) equals run(a + b) and every case's
// arithmetic is independent of the others in a batch, a request's result is
// the same alone and in any mix.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <atomic>
#include <vector>

#include "../../include/lbm_gpu.h"
#include "engine.h"

using namespace lbm;

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct ImpSpec {
    int entry = -1;
    std::vector<double> R, m, K, omegas;
    double rho_ref = 1.0, alpha = 0.0;
    int window = 0;
};

struct Request {
    int id = 0;
    int state = 0;  // 0 prepared, 1 queued, 2 active, 3 done, 4 failed
    // owned copies of the case description
    int Nx = 0, Ny = 0, storage = 0;
    double w[9];
    std::vector<int> mask;
    std::vector<double> omega, phi, wall_u, wall_v;
    int use_ibb = 0, px = 0, py = 0;
    double Fx = 0, Fy = 0;
    std::vector<BCEntry> bcs;
    std::vector<std::vector<double>> bc_vals;  // 2 per entry
    std::vector<double> f, f_new, rho, u, v;    // inputs, then results
    bool from_equilibrium = false;              // f = f_new = f_eq(rho, u, v) at admission
    int nsteps = 0, remaining = 0;
    bool keep_populations = false;
    ImpSpec imp;
    std::vector<double> spectra;
    std::unique_ptr<Solver> solver;
    size_t est_bytes = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::string error;
};

size_t estimate_bytes(const Request &r) {
    const size_t N = (size_t)r.Nx * r.Ny;
    const size_t pitchN = (size_t)((r.Nx + 63) / 64 * 64) * r.Ny;
    const size_t es = (r.storage == LBM_GPU_F64 || r.storage == LBM_GPU_F64_FMA)
                          ? 8 : (r.storage == LBM_GPU_F32_SHIFTED ? 4 : 2);
    return 2 * 9 * es * pitchN + (size_t)staging_rows(r.Nx, r.Ny) * r.Nx * 72 + 24 * N + 2 * pitchN +
           (r.use_ibb ? 4 * pitchN : 0) + 8 * N + (1u << 20);
}

}  // namespace

// One storage type's share of the server: its active requests and the batch
// that advances them (rebuilt only when the set of request ids changes).
struct Lane {
    int storage = 0;
    double busy_s = 0;  // wall time of this lane's rounds that ran a chunk
    std::vector<Request *> active;
    std::unique_ptr<Batch> batch;
    std::vector<int> batch_ids;
    std::thread worker;
};

struct lbm_gpu_server {
    std::mutex mu;
    std::map<int, std::unique_ptr<Request>> reqs;
    std::deque<Request *> queue;
    Lane lanes[4];
    int n_active = 0;  // over all lanes
    size_t budget = 0;    // optional cap on the requests' estimated bytes (0: none)
    size_t in_use = 0;    // estimated bytes of the active requests
    size_t reserve = 0;   // device memory admissions leave free
    size_t pending = 0;   // estimated bytes of requests taken but not set up yet
    int max_active = 64;
    int chunk = 1000;
    int next_id = 1;
    long long lups_done = 0;
    double busy_s = 0;
    // time spent per phase of the rounds (host wall clock)
    long long rounds = 0;
    double t_admit = 0, t_build = 0, t_run = 0, t_retire = 0;
    std::thread worker;
    std::atomic<bool> running{false};
    std::string err;
};

static bool admit(Request *r) {
    CaseDesc d;
    d.Nx = r->Nx;
    d.Ny = r->Ny;
    for (int k = 0; k < 9; k++) d.w[k] = r->w[k];
    d.mask = r->mask.data();
    d.omega = r->omega.data();
    d.phi = r->phi.empty() ? nullptr : r->phi.data();
    d.use_ibb = r->use_ibb;
    d.wall_u = r->wall_u.empty() ? nullptr : r->wall_u.data();
    d.wall_v = r->wall_v.empty() ? nullptr : r->wall_v.data();
    d.px = r->px;
    d.py = r->py;
    d.Fx = r->Fx;
    d.Fy = r->Fy;
    d.bcs = r->bcs;
    for (size_t e = 0; e < d.bcs.size(); e++) {
        d.bcs[e].val1 = r->bc_vals[2 * e].empty() ? nullptr : r->bc_vals[2 * e].data();
        d.bcs[e].val2 = r->bc_vals[2 * e + 1].empty() ? nullptr : r->bc_vals[2 * e + 1].data();
    }
    storage_to_desc(r->storage, d);
    std::unique_ptr<Solver> s(new Solver(d));
    if (!s->ok()) {
        r->error = last_error();
        return false;
    }
    if (r->imp.entry >= 0 &&
        !s->set_impedance(r->imp.entry, r->imp.R.data(), r->imp.m.data(), r->imp.K.data(),
                          (int)r->imp.omegas.size(), r->imp.omegas.data(), r->imp.rho_ref,
                          r->imp.alpha, r->imp.window)) {
        r->error = last_error();
        return false;
    }
    if (r->from_equilibrium) {
        // f_eq in lbc's operation order (as its case mains initialise f);
        // host memory for it only while the request is admitted.
        static const int kCX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
        static const int kCY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
        const size_t N = (size_t)r->Nx * r->Ny;
        r->f.resize(N * 9);
        for (size_t n = 0; n < N; n++) {
            const double ux = r->u[n], uy = r->v[n], rho = r->rho[n];
            const double v_sq = ux * ux + uy * uy;
            for (int k = 0; k < 9; k++) {
                const double cu = (double)kCX[k] * ux + (double)kCY[k] * uy;
                r->f[n * 9 + k] = r->w[k] * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * v_sq);
            }
        }
    }
    const double *fn = r->from_equilibrium ? r->f.data() : r->f_new.data();
    if (!s->set_state(r->f.data(), fn, r->rho.data(), r->u.data(), r->v.data()) ||
        !check_cuda(cudaStreamSynchronize(s->stream()), "admit")) {
        r->error = last_error();
        return false;
    }
    // Inputs are on the device now.
    std::vector<double>().swap(r->f);
    std::vector<double>().swap(r->f_new);
    r->solver = std::move(s);
    return true;
}

static bool retire(Request *r) {
    Solver *s = r->solver.get();
    const size_t N = (size_t)r->Nx * r->Ny;
    r->rho.assign(N, 0.0);
    r->u.assign(N, 0.0);
    r->v.assign(N, 0.0);
    bool okk;
    if (r->keep_populations) {
        r->f.assign(N * 9, 0.0);
        r->f_new.assign(N * 9, 0.0);
        okk = s->get_state(r->f.data(), r->f_new.data(), r->rho.data(), r->u.data(), r->v.data());
    } else {
        okk = s->get_fields(r->rho.data(), r->u.data(), r->v.data());
    }
    if (okk && r->imp.entry >= 0) {
        r->spectra.assign((size_t)r->Nx * r->imp.omegas.size() * 4, 0.0);
        okk = s->impedance_readback(r->imp.entry, r->spectra.data(), nullptr);
    }
    if (!okk) r->error = last_error();
    r->solver.reset();
    return okk;
}

// Device memory a new request may take now: the device's free memory plus
// what the stream-ordered pool holds unused (freed by retired requests and
// kept for reuse), less the reserve. Read live, so memory taken by anything
// else in or outside this process after the server started holds admissions
// back.
static size_t device_available(const lbm_gpu_server *S) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    size_t slack = 0;
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long reserved = 0, used = 0;  // cuuint64_t
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
            slack = (size_t)(reserved - used);
    }
    cudaGetLastError();
    const size_t have = fr + slack;
    return have > S->reserve ? have - S->reserve : 0;
}

// Queued requests of this lane's storage type, in arrival order, while the
// slot limit, the device memory available now (less what requests taken by
// any lane but not set up yet will take) and the optional budget allow. One
// request is always let in when nothing at all is active, so a request larger
// than the memory left still runs alone (or fails cleanly when it cannot
// allocate). The FP64 lanes hold at most a quarter of the slots while
// requests of another type are queued or running: FP64 requests step at
// GB300's FP64 rate, 7-12x slower per node than FP32, and without the cap
// they accumulate in the active set and leave the shorter requests queued
// behind them.
static std::vector<Request *> take_admissions(lbm_gpu_server *S, Lane &L) {
    std::vector<Request *> out;
    const size_t avail = device_available(S);
    std::lock_guard<std::mutex> lk(S->mu);
    int cap = S->max_active;
    if (L.storage == LBM_GPU_F64 || L.storage == LBM_GPU_F64_FMA) {
        bool others = S->n_active > (int)L.active.size();
        for (const Request *r : S->queue)
            if (r->storage != L.storage) { others = true; break; }
        if (others) cap = std::max(1, S->max_active / 4);
    }
    for (auto it = S->queue.begin(); it != S->queue.end();) {
        Request *r = *it;
        if (r->storage != L.storage) {
            ++it;
            continue;
        }
        if (S->n_active >= S->max_active || (int)(L.active.size() + out.size()) >= cap) break;
        const bool fits_live = S->pending + r->est_bytes <= avail;
        const bool fits_cap = S->budget == 0 || S->in_use + r->est_bytes <= S->budget;
        if (!(fits_live && fits_cap) && S->n_active > 0) break;
        it = S->queue.erase(it);
        out.push_back(r);
        S->in_use += r->est_bytes;
        S->pending += r->est_bytes;
        S->n_active++;
    }
    return out;
}

static void finish_request(lbm_gpu_server *S, Request *r, int st) {
    std::lock_guard<std::mutex> lk(S->mu);
    r->t_done = now_s();
    r->state = st;
    S->in_use -= r->est_bytes;
    S->n_active--;
}

// One round of one lane; returns the number of this lane's requests still
// active plus the requests queued for any lane.
static int lane_round(lbm_gpu_server *S, Lane &L) {
    const std::vector<Request *> taken = take_admissions(S, L);
    double t_b = 0, t_run0 = now_s();
    bool launched = false, okk = true;
    int n = 0;
    if (!L.active.empty()) {
        n = S->chunk;
        std::vector<int> ids;
        for (Request *r : L.active) {
            n = std::min(n, r->remaining);
            ids.push_back(r->id);
        }
        if (!L.batch || ids != L.batch_ids) {
            const double tb = now_s();
            std::vector<Solver *> sv;
            for (Request *r : L.active) sv.push_back(r->solver.get());
            L.batch.reset(new Batch(sv));
            L.batch_ids = ids;
            t_b = now_s() - tb;
        }
        okk = L.batch->ok() && L.batch->run(n);
        launched = true;
    }
    // Admissions overlap the chunk on the device.
    const double t_adm0 = now_s();
    std::vector<Request *> joined;
    for (Request *r : taken) {
        const double ta = now_s();
        const bool good = admit(r);
        {
            std::lock_guard<std::mutex> lk(S->mu);
            r->t_admit = ta;
            S->pending -= r->est_bytes;   // allocated now (or failed): the live figure has it
            if (good) r->state = 2;
        }
        if (good) joined.push_back(r);
        else finish_request(S, r, 4);
    }
    const double t_adm = now_s() - t_adm0;
    double t_wait = 0, t_ret = 0;
    if (launched) {
        const double tw = now_s();
        okk = okk && check_cuda(cudaStreamSynchronize(L.batch->stream()), "server");
        t_wait = now_s() - tw;
        const double tr = now_s();
        std::vector<Request *> keep;
        for (Request *r : L.active) {
            r->remaining -= n;
            int st;
            if (!okk) {
                r->error = last_error();
                r->solver.reset();
                st = 4;
            } else if (r->remaining <= 0) {
                st = retire(r) ? 3 : 4;
            } else {
                keep.push_back(r);
                continue;
            }
            finish_request(S, r, st);
        }
        if (okk) {
            std::lock_guard<std::mutex> lk(S->mu);
            for (Request *r : L.active) S->lups_done += (long long)r->Nx * r->Ny * n;
        }
        if (keep.size() != L.active.size() || !okk) {
            L.batch.reset();
            L.batch_ids.clear();
        }
        L.active.swap(keep);
        t_ret = now_s() - tr;
    }
    L.active.insert(L.active.end(), joined.begin(), joined.end());
    std::lock_guard<std::mutex> lk(S->mu);
    if (launched || !taken.empty()) {
        S->rounds++;
        S->t_admit += t_adm;
        S->t_build += t_b;
        S->t_run += (launched ? (t_adm0 - t_run0 - t_b) : 0.0) + t_wait;
        S->t_retire += t_ret;
        S->busy_s += now_s() - t_run0;
        if (launched) L.busy_s += now_s() - t_run0;
    }
    return (int)(S->queue.size() + L.active.size());
}

// One round of every lane (the caller's thread).
static int server_round(lbm_gpu_server *S) {
    int left = 0;
    for (Lane &L : S->lanes) left = std::max(left, lane_round(S, L));
    std::lock_guard<std::mutex> lk(S->mu);
    return (int)S->queue.size() + S->n_active;
}

extern "C" {

int lbm_gpu_server_create(size_t budget_bytes, int max_active, int chunk_steps, lbm_gpu_server **out) {
    if (!out || max_active < 1 || chunk_steps < 1) {
        set_error("bad arguments");
        return LBM_GPU_ERR_ARG;
    }
    size_t fr = 0, tot = 0;
    if (!check_cuda(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo")) return LBM_GPU_ERR_CUDA;
    lbm_gpu_server *S = new lbm_gpu_server();
    S->budget = budget_bytes;
    S->reserve = tot / 20;
    S->max_active = max_active;
    S->chunk = chunk_steps;
    S->lanes[0].storage = LBM_GPU_F64;
    S->lanes[1].storage = LBM_GPU_F32_SHIFTED;
    S->lanes[2].storage = LBM_GPU_F16_SHIFTED;
    S->lanes[3].storage = LBM_GPU_F64_FMA;
    *out = S;
    return LBM_GPU_OK;
}

int lbm_gpu_server_prepare(lbm_gpu_server *S, const lbm_gpu_case *c, const double *f,
                           const double *f_new, const double *rho, const double *u, const double *v,
                           int nsteps, int keep_populations) {
    if (!S || !c || !rho || !u || !v || nsteps < 1 || (!f) != (!f_new)) {
        set_error("bad arguments");
        return LBM_GPU_ERR_ARG;
    }
    CaseDesc probe;
    if (!storage_to_desc(c->storage, probe)) {
        set_error("bad storage");
        return LBM_GPU_ERR_ARG;
    }
    std::unique_ptr<Request> r(new Request());
    r->Nx = c->Nx;
    r->Ny = c->Ny;
    r->storage = c->storage;
    const size_t N = (size_t)c->Nx * c->Ny;
    for (int k = 0; k < 9; k++) r->w[k] = c->w[k];
    r->mask.assign(c->solid_mask, c->solid_mask + N);
    r->omega.assign(c->omega_eff, c->omega_eff + N);
    if (c->phi) r->phi.assign(c->phi, c->phi + N);
    if (c->wall_u) r->wall_u.assign(c->wall_u, c->wall_u + N);
    if (c->wall_v) r->wall_v.assign(c->wall_v, c->wall_v + N);
    r->use_ibb = c->use_IBB;
    r->px = c->isperiodic_x;
    r->py = c->isperiodic_y;
    r->Fx = c->Fx;
    r->Fy = c->Fy;
    for (int b = 0; b < c->num_boundaries; b++) {
        const int kind = bc_kind_of((const void *)c->boundaries[b].apply);
        if (kind < 0) {
            set_error("boundary entry " + std::to_string(b) + ": not one of lbc's BC functions");
            return LBM_GPU_ERR_ARG;
        }
        const bool col = bc_is_column(kind);
        const size_t along = col ? c->Ny : c->Nx;
        r->bcs.push_back(BCEntry{kind, c->boundaries[b].index, nullptr, nullptr});
        const double *v1 = c->boundaries[b].val1, *v2 = c->boundaries[b].val2;
        r->bc_vals.push_back(v1 ? std::vector<double>(v1, v1 + along) : std::vector<double>());
        r->bc_vals.push_back(v2 ? std::vector<double>(v2, v2 + along) : std::vector<double>());
    }
    if (f) {
        r->f.assign(f, f + 9 * N);
        r->f_new.assign(f_new, f_new + 9 * N);
    } else {
        r->from_equilibrium = true;
    }
    r->rho.assign(rho, rho + N);
    r->u.assign(u, u + N);
    r->v.assign(v, v + N);
    r->nsteps = r->remaining = nsteps;
    r->keep_populations = keep_populations != 0;
    r->est_bytes = estimate_bytes(*r);
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    const int id = r->id;
    S->reqs[id] = std::move(r);
    return id;
}

int lbm_gpu_server_set_impedance(lbm_gpu_server *S, int id, int entry, const double *R,
                                 const double *m, const double *K, int nf, const double *omegas,
                                 double rho_ref, double alpha, int window_steps) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second->state != 0) {
        set_error("request not found or already queued");
        return LBM_GPU_ERR_ARG;
    }
    Request *r = it->second.get();
    r->imp.entry = entry;
    r->imp.R.assign(R, R + r->Nx);
    r->imp.m.assign(m, m + r->Nx);
    r->imp.K.assign(K, K + r->Nx);
    r->imp.omegas.assign(omegas, omegas + nf);
    r->imp.rho_ref = rho_ref;
    r->imp.alpha = alpha;
    r->imp.window = window_steps;
    return LBM_GPU_OK;
}

int lbm_gpu_server_enqueue(lbm_gpu_server *S, int id) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second->state != 0) {
        set_error("request not found or already queued");
        return LBM_GPU_ERR_ARG;
    }
    it->second->state = 1;
    it->second->t_submit = now_s();
    S->queue.push_back(it->second.get());
    return LBM_GPU_OK;
}

int lbm_gpu_server_poll(lbm_gpu_server *S) {
    if (!S) return LBM_GPU_ERR_ARG;
    return server_round(S);
}

int lbm_gpu_server_start(lbm_gpu_server *S) {
    if (!S || S->running) return LBM_GPU_ERR_ARG;
    S->running = true;
    int dev = 0;
    cudaGetDevice(&dev);
    for (Lane &L : S->lanes) {
        Lane *pl = &L;
        L.worker = std::thread([S, pl, dev] {
            cudaSetDevice(dev);
            while (S->running) {
                const bool busy = !pl->active.empty();
                lane_round(S, *pl);
                if (!busy && pl->active.empty()) std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
        });
    }
    return LBM_GPU_OK;
}

int lbm_gpu_server_stop(lbm_gpu_server *S) {
    if (!S) return LBM_GPU_ERR_ARG;
    S->running = false;
    for (Lane &L : S->lanes)
        if (L.worker.joinable()) L.worker.join();
    return LBM_GPU_OK;
}

int lbm_gpu_server_status(lbm_gpu_server *S, int id, double *t_submit, double *t_admit,
                          double *t_done) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) {
        set_error("request not found");
        return LBM_GPU_ERR_ARG;
    }
    Request *r = it->second.get();
    if (t_submit) *t_submit = r->t_submit;
    if (t_admit) *t_admit = r->t_admit;
    if (t_done) *t_done = r->t_done;
    if (r->state == 4) set_error(r->error);
    return r->state;
}

int lbm_gpu_server_fetch(lbm_gpu_server *S, int id, double *f, double *f_new, double *rho,
                         double *u, double *v, double *spectra) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second->state != 3) {
        set_error("request not finished");
        return LBM_GPU_ERR_ARG;
    }
    Request *r = it->second.get();
    const size_t N = (size_t)r->Nx * r->Ny;
    if ((f || f_new) && !r->keep_populations) {
        set_error("populations were not kept (keep_populations = 0)");
        return LBM_GPU_ERR_ARG;
    }
    if (f) std::memcpy(f, r->f.data(), N * 9 * sizeof(double));
    if (f_new) std::memcpy(f_new, r->f_new.data(), N * 9 * sizeof(double));
    if (rho) std::memcpy(rho, r->rho.data(), N * sizeof(double));
    if (u) std::memcpy(u, r->u.data(), N * sizeof(double));
    if (v) std::memcpy(v, r->v.data(), N * sizeof(double));
    if (spectra && !r->spectra.empty()) std::memcpy(spectra, r->spectra.data(), r->spectra.size() * sizeof(double));
    return LBM_GPU_OK;
}

int lbm_gpu_server_release(lbm_gpu_server *S, int id) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second->state == 1 || it->second->state == 2) {
        set_error("request not found or still running");
        return LBM_GPU_ERR_ARG;
    }
    S->reqs.erase(it);
    return LBM_GPU_OK;
}

int lbm_gpu_server_stats(lbm_gpu_server *S, long long *lups_done, double *busy_s, int *queued,
                         int *active, size_t *bytes_in_use) {
    std::lock_guard<std::mutex> lk(S->mu);
    if (lups_done) *lups_done = S->lups_done;
    if (busy_s) *busy_s = S->busy_s;
    if (queued) *queued = (int)S->queue.size();
    if (active) *active = S->n_active;
    if (bytes_in_use) *bytes_in_use = S->in_use;
    return LBM_GPU_OK;
}

int lbm_gpu_server_set_reserve(lbm_gpu_server *S, size_t reserve_bytes) {
    if (!S) {
        set_error("bad arguments");
        return LBM_GPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->reserve = reserve_bytes;
    return LBM_GPU_OK;
}

int lbm_gpu_server_available(lbm_gpu_server *S, size_t *bytes) {
    if (!S || !bytes) {
        set_error("bad arguments");
        return LBM_GPU_ERR_ARG;
    }
    const size_t a = device_available(S);
    std::lock_guard<std::mutex> lk(S->mu);
    *bytes = a > S->pending ? a - S->pending : 0;
    return LBM_GPU_OK;
}

int lbm_gpu_server_profile(lbm_gpu_server *S, double *out, int n) {
    if (!S || !out || n < 1) {
        set_error("bad arguments");
        return LBM_GPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    const double v[9] = {(double)S->rounds, S->t_admit, S->t_build, S->t_run, S->t_retire,
                         S->lanes[0].busy_s, S->lanes[1].busy_s, S->lanes[2].busy_s, S->lanes[3].busy_s};
    for (int q = 0; q < n && q < 9; q++) out[q] = v[q];
    return LBM_GPU_OK;
}

int lbm_gpu_server_destroy(lbm_gpu_server *S) {
    if (!S) return LBM_GPU_OK;
    lbm_gpu_server_stop(S);
    for (Lane &L : S->lanes) {
        L.batch.reset();
        for (Request *r : L.active) r->solver.reset();
    }
    delete S;
    return LBM_GPU_OK;
}

}  // extern "C"
