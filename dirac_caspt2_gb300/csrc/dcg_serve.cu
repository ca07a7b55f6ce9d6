// Serving runtime: continuous batching of independent CASPT2 solves on one GPU.
//
// A server owns `slots` contexts, one worker thread and one CUDA stream each, so the kernels
// of different requests overlap on the device.  Requests (each a complete system: the
// dcg_system of dcg_set_system) wait in a queue; whenever a slot is free, the worker takes the
// first queued request whose device footprint fits the HBM budget together with what the
// other slots hold.  A context keeps its integrals, CI vectors and workspace resident after a
// request, so that memory stays counted for its slot.  Finished requests are collected with
// dcg_server_poll, with submit / start / end stamps on the server's steady clock.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "dcg_common.cuh"

namespace {

struct Request {
    uint64_t id = 0;
    dcg_system sys{};
    int64_t bytes = 0;
    double t_submit = 0.0;
    int attempts = 0;
};

// Device footprint of one solve (bytes), from its dimensions, for either precision.  Terms:
// the record stream (indices, values, packed values), the active/inactive two-electron block,
// the fourteen integral classes with their transformed copies, the CASCI matrix and CI
// rotation (ndet^2), the densities of the full determinant space (E_pq psi and E_pq E_rs psi
// for the state and its orbital-energy-weighted copy), the subspace matrices (up to
// na^3 x na^3 for A and C), the Gram factors (C(na, ne+-1) rows) and the eigensolver slots; on
// the split path also the BF16 slices of the largest class and of the density operand.  The
// 1.25 margin keeps it above dcg_device_bytes of a fresh context on every size measured (4 to
// 40 inactive, 4 to 14 active, 60 to 800 secondary spinors: 1.15 to 1.7 times the use).
double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    double r = 1.0;
    for (int q = 1; q <= k; q++) r = r * (n - k + q) / q;
    return r;
}

int64_t footprint(const dcg_system &s) {
    const double ni = s.ninact, na = s.nact, ns = s.nsec, nmoc = ni + na;
    const double z = 16.0;   // complex128
    const double sizes[] = {ns * na * na * na, ns * na * ni * ni, ns * ni * ni * na, ns * ni * na * na,
                            ns * na * na * ni, ns * ni * ni * ni, ns * ni * na * ni, ns * na * ns * na,
                            ns * ni * ns * na, ns * ni * ns * ni, ns * ns * na * na, ns * na * na * ns,
                            ns * ns * ni, ns * ns * ni};
    double cls = 0.0, largest = 0.0;
    for (double x : sizes) {
        cls += x;
        largest = std::max(largest, x);
    }
    const double ndet = binom(s.nact, s.nelec);
    const double mp = std::max(binom(s.nact, s.nelec + 1), binom(s.nact, s.nelec - 1));
    const double n3 = na * na * na, na2 = na * na;
    const double dens = z * ndet * 2.0 * (na2 * na2 + na2);   // E_pq psi and E_pq E_rs psi, two vectors
    double b = 48.0 * (double)s.nrec + z * nmoc * nmoc * nmoc * nmoc + 2.0 * z * cls;
    b += 3.0 * z * ndet * ndet;         // CASCI matrix, vectors, CI rotation
    b += dens;
    b += 10.0 * z * n3 * n3;            // S, B, X, BX, B', W of the largest block
    b += 6.0 * z * mp * (mp + n3);      // Gram factor, metric, P, PD
    b += 64.0 * 1024.0 * 1024.0;        // eigensolver slots, reductions
    b += 1.3 * z * largest + 0.7 * dens;   // split-precision slices
    return (int64_t)(1.25 * b);
}

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct dcg_server {
    int device = 0, precision = DCG_PREC_FP64, nslots = 0;
    int64_t budget = 0;
    std::vector<dcg_ctx *> ctx;
    std::vector<int64_t> held;   // bytes a slot holds: its resident workspace, or the running request's estimate
    std::vector<std::thread> workers;
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> queue;
    std::deque<dcg_request_result> done;
    int running = 0;
    bool stop = false;
};

namespace {

// One request on one context: the reference's per-entry sequence (dcaspt2_run_subprograms.F90:
// r4dcasci then r4dcaspt2_tra) through the public entry points.
int run_request(dcg_ctx *c, const Request &rq, dcg_request_result &res) {
    int st = dcg_set_system(c, &rq.sys);
    if (st != DCG_OK) return st;
    const int nroot = std::max(1, rq.sys.selectroot);
    std::vector<double> eig(nroot, 0.0);
    int32_t ndet = 0;
    st = dcg_casci(c, nroot, eig.data(), nullptr, nullptr, &ndet);
    res.ndet = ndet;
    if (st != DCG_OK) return st;
    res.casci_energy = eig[std::min(nroot, std::max(ndet, 1)) - 1];
    return dcg_caspt2(c, 0u, res.e2, res.sumc2, &res.e0, &res.etotal);
}

void worker_loop(dcg_server *sv, int w) {
    dcg_ctx *c = sv->ctx[w];
    for (;;) {
        Request rq;
        {
            std::unique_lock<std::mutex> lk(sv->m);
            for (;;) {
                if (sv->stop) return;
                int64_t others = 0;
                for (int v = 0; v < sv->nslots; v++)
                    if (v != w) others += sv->held[v];
                auto it = std::find_if(sv->queue.begin(), sv->queue.end(), [&](const Request &r) {
                    return others + std::max(sv->held[w], r.bytes) <= sv->budget;
                });
                if (it != sv->queue.end()) {
                    rq = *it;
                    sv->queue.erase(it);
                    sv->held[w] = std::max(sv->held[w], rq.bytes);
                    sv->running++;
                    break;
                }
                if (!sv->queue.empty() && sv->held[w] > 0) {
                    // nothing fits: give this idle slot's resident workspace back
                    lk.unlock();
                    dcg_trim(c);
                    lk.lock();
                    sv->held[w] = 0;
                    sv->cv_work.notify_all();   // the freed bytes may let another slot start
                    continue;
                }
                sv->cv_work.wait(lk);
            }
        }
        dcg_request_result res;
        std::memset(&res, 0, sizeof(res));
        res.request_id = rq.id;
        res.t_submit = rq.t_submit;
        res.slot = w;
        res.attempts = rq.attempts + 1;
        res.t_start = now_s();
        int st = run_request(c, rq, res);
        res.status = st;
        if (st != DCG_OK) {
            const char *msg = dcg_last_error(c);
            std::strncpy(res.error, msg ? msg : "", sizeof(res.error) - 1);
        }
        res.t_end = now_s();
        if (st == DCG_E_NOMEM) dcg_trim(c);   // the estimate was short or another slot grew: retry once
        {
            std::lock_guard<std::mutex> lk(sv->m);
            sv->held[w] = dcg_device_bytes(c);
            sv->running--;
            if (st == DCG_E_NOMEM && rq.attempts == 0) {
                rq.attempts = 1;
                rq.bytes = std::max(rq.bytes, sv->budget / std::max(1, sv->nslots));
                sv->queue.push_front(rq);
            } else {
                sv->done.push_back(res);
            }
        }
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int64_t dcg_footprint_estimate(const dcg_system *sys) {
    if (!sys || sys->nact < 0 || sys->ninact < 0 || sys->nsec < 0) return -1;
    return footprint(*sys);
}

int dcg_server_create(int device, int precision, int32_t slots, int64_t hbm_budget_bytes, dcg_server **out) {
    if (!out || slots < 1 || slots > 64) return DCG_E_ARG;
    *out = nullptr;
    if (precision != DCG_PREC_FP64 && precision != DCG_PREC_SPLIT) return DCG_E_ARG;
    dcg_server *sv = new (std::nothrow) dcg_server;
    if (!sv) return DCG_E_NOMEM;
    sv->device = device;
    sv->precision = precision;
    sv->nslots = slots;
    size_t fr = 0, tot = 0;
    if (cudaSetDevice(device) != cudaSuccess || cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        delete sv;
        return DCG_E_CUDA;
    }
    sv->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (int64_t)(0.9 * (double)fr);
    for (int w = 0; w < slots; w++) {
        dcg_ctx *c = nullptr;
        const int st = dcg_create(device, precision, &c);
        if (st != DCG_OK) {
            for (dcg_ctx *x : sv->ctx) dcg_destroy(x);
            delete sv;
            return st;
        }
        // a served stream meets most shapes once: its slots use tuned entries and heuristics
        // and run no tuning trials of their own (they would sit in the requests' latency)
        dcg_set_autotune_trials(c, 0);
        // the slots' Householder reductions run merged: requests solving at the same time share
        // one cooperative launch (dcg_set_merge_reductions)
        dcg_set_merge_reductions(c, 1);
        sv->ctx.push_back(c);
        sv->held.push_back(dcg_device_bytes(c));
    }
    for (int w = 0; w < slots; w++) sv->workers.emplace_back(worker_loop, sv, w);
    *out = sv;
    return DCG_OK;
}

int dcg_server_submit(dcg_server *sv, const dcg_system *sys, uint64_t request_id) {
    if (!sv || !sys) return DCG_E_ARG;
    Request r;
    r.id = request_id;
    r.sys = *sys;
    r.bytes = footprint(*sys);
    r.t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(sv->m);
        if (r.bytes > sv->budget) return DCG_E_NOMEM;   // could never be admitted
        sv->queue.push_back(r);
    }
    sv->cv_work.notify_all();
    return DCG_OK;
}

int dcg_server_poll(dcg_server *sv, int32_t timeout_ms, dcg_request_result *out) {
    if (!sv || !out) return DCG_E_ARG;
    std::unique_lock<std::mutex> lk(sv->m);
    if (sv->done.empty() && timeout_ms > 0)
        sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !sv->done.empty(); });
    if (sv->done.empty()) return 1;
    *out = sv->done.front();
    sv->done.pop_front();
    return DCG_OK;
}

int dcg_server_pending(dcg_server *sv, int32_t *queued, int32_t *running) {
    if (!sv) return DCG_E_ARG;
    std::lock_guard<std::mutex> lk(sv->m);
    if (queued) *queued = (int32_t)sv->queue.size();
    if (running) *running = sv->running;
    return DCG_OK;
}

double dcg_server_clock(const dcg_server *sv) {
    (void)sv;
    return now_s();
}

int64_t dcg_server_device_bytes(dcg_server *sv) {
    if (!sv) return -1;
    int64_t b = 0;
    for (dcg_ctx *c : sv->ctx) b += dcg_device_bytes(c);
    return b;
}

int dcg_server_destroy(dcg_server *sv) {
    if (!sv) return DCG_E_ARG;
    {
        std::lock_guard<std::mutex> lk(sv->m);
        sv->stop = true;
        sv->queue.clear();
    }
    sv->cv_work.notify_all();
    for (std::thread &t : sv->workers) t.join();
    for (dcg_ctx *c : sv->ctx) dcg_destroy(c);
    delete sv;
    return DCG_OK;
}

}  // extern "C"
