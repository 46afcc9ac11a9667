// Serving loop: RREF and load+RREF requests admitted by device memory, run
// concurrently on a set of CUDA streams, completed through host callbacks.
//
// linac has no serving layer: each caller makes one synchronous
// cuda_row_reduce / load_matrices call per system
// (linac/pycuda_row_reduce.py:18-151, linac/pycuda_matrix_loader.py:127-230),
// so the GPU idles during every host step and runs one matrix at a time.
//
// Here a scheduler thread owns `max_inflight` streams ("slots").  A queued
// request is admitted when a slot is free and its footprint (input + output
// matrix, pivots, the solve's scratch, loader inputs) fits the budget next to
// the requests in flight.  Admission enqueues the whole request on the slot's
// stream without waiting: stream-ordered allocation, host->device copy (or
// the monomial loader writing straight into the matrix the solve reduces),
// the solve, device->host copies of the result, pivots and rank, the frees,
// and a host callback that hands the slot back to the scheduler.  Solves of
// different requests overlap on the device (one request's single-CTA
// candidate panel runs beside another's contractions).  F_p solves use
// LNC_FLAG_DEFER_FALLBACK so no request launches a grid-wide panel kernel in
// the common case; a request whose candidate panels missed a pivot (rank -1)
// is re-run on its slot with the exhaustive panel before it completes.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "rref_internal.cuh"

namespace lnc {

int load_matrix_dispatch(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         uint64_t p, const void* bases, const uint32_t* lind, void* out, int64_t ldo,
                         cudaStream_t s);

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxBypass = 8;  // times a queued request may be passed by later ones

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct Layout {  // one device block per request
    size_t work = 0, out = 0, piv = 0, rank = 0, bases = 0, lind = 0, total = 0, scratch = 0;
};

Layout request_layout(const lnc_serve_request& r) {
    Layout L;
    const size_t elt = dtype_size(r.dtype);
    const size_t mn = elt * (size_t)r.m * (size_t)r.n;
    const int64_t kmax = std::min(r.m, r.n);
    size_t off = 0;
    L.work = off; off += al256(mn);
    L.out = off; off += al256(mn);
    L.piv = off; off += al256(sizeof(int64_t) * (size_t)std::max<int64_t>(kmax, 1));
    L.rank = off; off += 256;
    if (r.kind == LNC_SERVE_LOAD_RREF) {
        L.bases = off; off += al256(elt * (size_t)r.m * (size_t)std::max<int64_t>(r.basis_len, 1));
        L.lind = off; off += al256(sizeof(uint32_t) * (size_t)r.n * (size_t)std::max<int64_t>(r.degree, 1));
    }
    L.total = off;
    L.scratch = rref_device_scratch(r.dtype, r.m, r.n);
    return L;
}

int validate_request(const lnc_serve_request& r) {
    if (r.kind != LNC_SERVE_RREF && r.kind != LNC_SERVE_LOAD_RREF) {
        set_error("serve: unknown request kind %d", r.kind);
        return LNC_ERR_INVALID;
    }
    int rc = validate_rref_args(r.dtype, r.m, r.n, r.p, r.kind == LNC_SERVE_RREF ? r.ld_in : r.n);
    if (rc) return rc;
    if (r.m == 0 || r.n == 0) { set_error("serve: empty matrix"); return LNC_ERR_INVALID; }
    if (!r.host_out || r.ld_out < r.n) { set_error("serve: missing output or ld_out < n"); return LNC_ERR_INVALID; }
    if (r.kind == LNC_SERVE_RREF && !r.host_in) { set_error("serve: missing input matrix"); return LNC_ERR_INVALID; }
    if (r.kind == LNC_SERVE_LOAD_RREF) {
        if (!r.host_bases || !r.host_lindices || r.basis_len <= 0 || r.degree <= 0) {
            set_error("serve: load request needs bases and lindices");
            return LNC_ERR_INVALID;
        }
    }
    return LNC_OK;
}

enum class State { Queued, Running, Done };

struct Ticket {
    lnc_serve_request req;
    Layout lay;
    int64_t bytes = 0;
    State state = State::Queued;
    int status = LNC_OK;
    int bypassed = 0;
    int attempts = 0;
    int slot = -1;
    Clock::time_point t_submit, t_admit, t_done;
};

struct Server;

struct Slot {
    Server* srv = nullptr;
    int idx = 0;
    cudaStream_t stream = nullptr;
    int64_t* h_rank = nullptr;  // page-locked: the solve's rank (or -1 / -2)
    int64_t ticket = -1;
    Clock::time_point t_fired;
};

struct Server {
    int device = 0;
    int64_t budget = 0, in_use = 0, peak = 0;
    int max_inflight = 16;
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, Ticket> tickets;
    std::vector<Slot> slots;
    std::vector<int> free_slots;
    std::vector<int> fired;  // slots whose callback ran
    std::vector<double> latencies;
    int64_t next_id = 1;
    int64_t submitted = 0, completed = 0, failed = 0, redone = 0, inflight = 0;
    bool stop = false;
    std::thread thread;
};

void CUDART_CB slot_fired(void* arg) {
    Slot* sl = (Slot*)arg;
    Server* S = sl->srv;
    sl->t_fired = Clock::now();
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->fired.push_back(sl->idx);
    }
    S->cv_sched.notify_one();
}

// enqueue one attempt of a request on its slot's stream (no host waits)
int launch(Server* S, Ticket& t, Slot& sl, int flags) {
    const lnc_serve_request& r = t.req;
    const Layout& L = t.lay;
    cudaStream_t s = sl.stream;
    const size_t elt = dtype_size(r.dtype);
    unsigned char* blk = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&blk, L.total, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("serve: device allocation of %zu bytes: %s", L.total, cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    void* work = blk + L.work;
    void* out = blk + L.out;
    int64_t* piv = (int64_t*)(blk + L.piv);
    int64_t* rank = (int64_t*)(blk + L.rank);
    int rc = LNC_OK;
    if (r.kind == LNC_SERVE_RREF) {
        e = cudaMemcpy2DAsync(work, elt * r.n, r.host_in, elt * r.ld_in, elt * r.n, r.m, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) rc = cuda_status(e, "serve: input copy");
    } else {
        e = cudaMemcpyAsync(blk + L.bases, r.host_bases, elt * (size_t)r.m * r.basis_len, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(blk + L.lind, r.host_lindices, sizeof(uint32_t) * (size_t)r.n * r.degree,
                                cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) rc = cuda_status(e, "serve: loader input copy");
        if (!rc)
            rc = load_matrix_dispatch(r.dtype, r.m, r.n, r.basis_len, r.degree, r.p, blk + L.bases,
                                      (const uint32_t*)(blk + L.lind), work, r.n, s);
    }
    if (!rc) {
        const double tol = r.tol > 0 ? r.tol : 1e-9;
        rc = rref_device_dispatch(r.dtype, r.m, r.n, r.p, tol, work, r.n, out, r.n, piv, rank, s, flags);
    }
    if (!rc) {
        e = cudaMemcpyAsync(sl.h_rank, rank, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(r.host_out, elt * r.ld_out, out, elt * r.n, elt * r.n, r.m, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && r.host_pivot_cols)
            e = cudaMemcpyAsync(r.host_pivot_cols, piv, sizeof(int64_t) * (size_t)std::min(r.m, r.n),
                                cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_status(e, "serve: result copy");
    }
    cudaFreeAsync(blk, s);
    if (rc) {
        cudaStreamSynchronize(s);  // the caller's host buffers may be reused once the request fails
        return rc;
    }
    e = cudaLaunchHostFunc(s, slot_fired, &sl);
    if (e != cudaSuccess) return cuda_status(e, "serve: completion callback");
    return LNC_OK;
}

int solve_flags(const Ticket& t) {
    int f = t.req.flags & ~LNC_FLAG_DEFER_FALLBACK;
    if (t.attempts == 0) f |= LNC_FLAG_DEFER_FALLBACK;
    else f |= LNC_FLAG_ROBUST_PANEL;
    return f;
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

// called with the lock held
void finish_locked(Server* S, int64_t id, Ticket& t, int status) {
    t.state = State::Done;
    t.status = status;
    t.t_done = Clock::now();
    Slot& sl = S->slots[t.slot];
    if (status == LNC_OK && sl.t_fired > t.t_admit) t.t_done = sl.t_fired;
    sl.ticket = -1;
    S->free_slots.push_back(t.slot);
    S->in_use -= t.bytes;
    --S->inflight;
    if (status == LNC_OK) {
        ++S->completed;
        S->latencies.push_back(std::chrono::duration<double, std::milli>(t.t_done - t.t_submit).count());
    } else {
        ++S->failed;
    }
    (void)id;
}

// a queued request can be admitted now (same scan as the admission loop; lock held)
bool admissible(Server* S) {
    if (S->free_slots.empty()) return false;
    for (int64_t id : S->queue) {
        const Ticket& q = S->tickets[id];
        if (q.bytes <= S->budget - S->in_use) return true;
        if (q.bypassed >= kMaxBypass) return false;
    }
    return false;
}

void scheduler(Server* S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        // ---- completions
        while (!S->fired.empty()) {
            std::vector<int> done;
            done.swap(S->fired);
            for (int idx : done) {
                Slot& sl = S->slots[idx];
                auto it = S->tickets.find(sl.ticket);
                if (it == S->tickets.end()) continue;
                Ticket& t = it->second;
                const int64_t rank = *sl.h_rank;
                int status = LNC_OK;
                if (rank == -2) status = LNC_ERR_TIMEOUT;
                if (rank == -1 && t.attempts == 0) {  // candidate panels missed a pivot: exhaustive redo
                    t.attempts = 1;
                    ++S->redone;
                    const int flags = solve_flags(t);
                    lk.unlock();
                    const int rc = launch(S, t, sl, flags);
                    lk.lock();
                    if (rc) finish_locked(S, it->first, t, rc);
                    continue;
                }
                if (rank < 0 && status == LNC_OK) status = LNC_ERR_CUDA;
                if (t.req.host_rank) *t.req.host_rank = rank < 0 ? 0 : rank;
                finish_locked(S, it->first, t, status);
            }
            S->cv_done.notify_all();
        }
        // ---- admission
        while (!S->free_slots.empty() && !S->queue.empty()) {
            int64_t pick = -1;
            size_t pos = 0;
            for (size_t i = 0; i < S->queue.size(); ++i) {
                Ticket& q = S->tickets[S->queue[i]];
                if (q.bytes <= S->budget - S->in_use) {
                    pick = S->queue[i];
                    pos = i;
                    break;
                }
                if (q.bypassed >= kMaxBypass) break;  // it has waited long enough: nothing passes it
            }
            if (pick < 0) break;
            for (size_t i = 0; i < pos; ++i) ++S->tickets[S->queue[i]].bypassed;
            S->queue.erase(S->queue.begin() + (ptrdiff_t)pos);
            Ticket& t = S->tickets[pick];
            const int idx = S->free_slots.back();
            S->free_slots.pop_back();
            Slot& sl = S->slots[idx];
            sl.ticket = pick;
            t.slot = idx;
            t.state = State::Running;
            t.t_admit = Clock::now();
            S->in_use += t.bytes;
            S->peak = std::max(S->peak, S->in_use);
            ++S->inflight;
            const int flags = solve_flags(t);
            lk.unlock();
            const int rc = launch(S, t, sl, flags);
            lk.lock();
            if (rc) {
                finish_locked(S, pick, t, rc);
                S->cv_done.notify_all();
            }
        }
        if (S->stop && S->inflight == 0 && S->queue.empty()) break;
        S->cv_sched.wait(lk, [&] {
            return !S->fired.empty() || (S->stop && S->inflight == 0 && S->queue.empty()) || admissible(S);
        });
    }
}

}  // namespace
}  // namespace lnc

using namespace lnc;

extern "C" {

int64_t lnc_serve_request_bytes(const lnc_serve_request* req) {
    if (!req || validate_request(*req)) return -1;
    const Layout L = request_layout(*req);
    return (int64_t)(L.total + L.scratch);
}

int lnc_server_create(int64_t budget_bytes, int max_inflight, void** server) {
    if (!server) { set_error("server: null handle"); return LNC_ERR_INVALID; }
    *server = nullptr;
    Server* S = new Server();
    cudaError_t e = cudaGetDevice(&S->device);
    if (e != cudaSuccess) { delete S; return cuda_status(e, "cudaGetDevice"); }
    if (budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) { delete S; return cuda_status(e, "cudaMemGetInfo"); }
        budget_bytes = (int64_t)(0.9 * (double)fr);
    }
    S->budget = budget_bytes;
    S->max_inflight = max_inflight > 0 ? max_inflight : 16;
    S->slots.resize(S->max_inflight);
    for (int i = 0; i < S->max_inflight; ++i) {
        Slot& sl = S->slots[i];
        sl.srv = S;
        sl.idx = i;
        e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&sl.h_rank, sizeof(int64_t));
        if (e != cudaSuccess) {
            for (auto& x : S->slots) {
                if (x.stream) cudaStreamDestroy(x.stream);
                if (x.h_rank) cudaFreeHost(x.h_rank);
            }
            delete S;
            return cuda_status(e, "server slots");
        }
        S->free_slots.push_back(S->max_inflight - 1 - i);
    }
    S->thread = std::thread(scheduler, S);
    *server = S;
    return LNC_OK;
}

int lnc_server_destroy(void* server) {
    Server* S = (Server*)server;
    if (!S) return LNC_OK;
    {
        std::lock_guard<std::mutex> g(S->mu);
        for (int64_t id : S->queue) {
            Ticket& t = S->tickets[id];
            t.state = State::Done;
            t.status = LNC_ERR_INVALID;
            t.t_done = Clock::now();
        }
        S->queue.clear();
        S->stop = true;
    }
    S->cv_sched.notify_one();
    S->cv_done.notify_all();
    if (S->thread.joinable()) S->thread.join();
    for (auto& sl : S->slots) {
        cudaStreamSynchronize(sl.stream);
        cudaStreamDestroy(sl.stream);
        cudaFreeHost(sl.h_rank);
    }
    delete S;
    return LNC_OK;
}

int lnc_serve_submit(void* server, const lnc_serve_request* req, int64_t* ticket) {
    Server* S = (Server*)server;
    if (!S || !req || !ticket) { set_error("serve: null argument"); return LNC_ERR_INVALID; }
    int rc = validate_request(*req);
    if (!rc && req->kind == LNC_SERVE_LOAD_RREF)  // the host index list must be readable at submission
        rc = check_loader_indices(req->host_lindices, req->n, req->degree, req->basis_len);
    if (rc) return rc;
    const int prev = [&] { int d = 0; cudaGetDevice(&d); return d; }();
    if (prev != S->device) cudaSetDevice(S->device);
    const Layout L = request_layout(*req);
    if (prev != S->device) cudaSetDevice(prev);
    const int64_t bytes = (int64_t)(L.total + L.scratch);
    if (bytes > S->budget) {
        set_error("serve: request needs %lld device bytes, budget is %lld", (long long)bytes, (long long)S->budget);
        return LNC_ERR_ADMISSION;
    }
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (S->stop) { set_error("serve: server is shutting down"); return LNC_ERR_INVALID; }
        const int64_t id = S->next_id++;
        Ticket& t = S->tickets[id];
        t.req = *req;
        t.lay = L;
        t.bytes = bytes;
        t.t_submit = Clock::now();
        S->queue.push_back(id);
        ++S->submitted;
        *ticket = id;
    }
    S->cv_sched.notify_one();
    return LNC_OK;
}

int lnc_serve_poll(void* server, int64_t ticket, int* done, int* status) {
    Server* S = (Server*)server;
    if (!S) { set_error("serve: null server"); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end()) { set_error("serve: unknown ticket %lld", (long long)ticket); return LNC_ERR_INVALID; }
    if (done) *done = it->second.state == State::Done;
    if (status) *status = it->second.state == State::Done ? it->second.status : LNC_OK;
    return LNC_OK;
}

int lnc_serve_wait(void* server, int64_t ticket, double timeout_s, int* status) {
    Server* S = (Server*)server;
    if (!S) { set_error("serve: null server"); return LNC_ERR_INVALID; }
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end()) { set_error("serve: unknown ticket %lld", (long long)ticket); return LNC_ERR_INVALID; }
    auto is_done = [&] { return S->tickets[ticket].state == State::Done; };
    if (timeout_s < 0) S->cv_done.wait(lk, is_done);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), is_done)) {
        set_error("serve: ticket %lld not done after %.3f s", (long long)ticket, timeout_s);
        return LNC_ERR_TIMEOUT;
    }
    if (status) *status = S->tickets[ticket].status;
    return LNC_OK;
}

int lnc_serve_latency(void* server, int64_t ticket, double* queue_ms, double* total_ms) {
    Server* S = (Server*)server;
    if (!S) { set_error("serve: null server"); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end() || it->second.state != State::Done) {
        set_error("serve: ticket %lld unknown or not done", (long long)ticket);
        return LNC_ERR_INVALID;
    }
    const Ticket& t = it->second;
    using ms = std::chrono::duration<double, std::milli>;
    if (queue_ms) *queue_ms = t.slot >= 0 ? ms(t.t_admit - t.t_submit).count() : ms(t.t_done - t.t_submit).count();
    if (total_ms) *total_ms = ms(t.t_done - t.t_submit).count();
    return LNC_OK;
}

int lnc_serve_release(void* server, int64_t ticket) {
    Server* S = (Server*)server;
    if (!S) { set_error("serve: null server"); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end()) { set_error("serve: unknown ticket %lld", (long long)ticket); return LNC_ERR_INVALID; }
    if (it->second.state != State::Done) { set_error("serve: ticket %lld still running", (long long)ticket); return LNC_ERR_INVALID; }
    S->tickets.erase(it);
    return LNC_OK;
}

int lnc_serve_stats_read(void* server, lnc_serve_stats* out) {
    Server* S = (Server*)server;
    if (!S || !out) { set_error("serve: null argument"); return LNC_ERR_INVALID; }
    std::vector<double> lat;
    {
        std::lock_guard<std::mutex> g(S->mu);
        out->submitted = S->submitted;
        out->completed = S->completed;
        out->failed = S->failed;
        out->redone = S->redone;
        out->queued = (int64_t)S->queue.size();
        out->inflight = S->inflight;
        out->bytes_in_use = S->in_use;
        out->peak_bytes = S->peak;
        out->budget_bytes = S->budget;
        lat = S->latencies;
    }
    out->p50_ms = percentile(lat, 0.50);
    out->p99_ms = percentile(lat, 0.99);
    double sum = 0.0, mx = 0.0;
    for (double v : lat) { sum += v; mx = std::max(mx, v); }
    out->mean_ms = lat.empty() ? 0.0 : sum / (double)lat.size();
    out->max_ms = mx;
    return LNC_OK;
}

int lnc_serve_stats_reset(void* server) {
    Server* S = (Server*)server;
    if (!S) { set_error("serve: null server"); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(S->mu);
    S->latencies.clear();
    S->submitted = S->completed = S->failed = S->redone = 0;
    S->peak = S->in_use;
    return LNC_OK;
}

}  // extern "C"
