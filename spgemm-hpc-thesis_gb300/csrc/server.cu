// Serving loop of the GB300 SpGEMM engine (spg_server_* / spg_submit / spg_poll).
//
// Requests (one product each) wait in a FIFO queue.  `lanes` worker threads,
// each owning an engine handle and therefore its own CUDA stream, take the
// longest prefix of the queue that fits the free part of the HBM budget (at
// most max_batch requests, and no more than max_batch_products scalar products
// unless the prefix is a single request) and run it as one batched call:
// every phase is one launch per row bin over the concatenated rows of all
// admitted products.
// While one lane's batch is on the device, another lane admits what arrived in
// the meantime, so successive batches overlap on the GPU (continuous
// batching); a lane whose head request does not fit waits until a finishing
// batch gives its reservation back.
//
// Admission charges a request its upper-bound device footprint, computed from
// its scalar-product count P (the binning pass's row upper bounds summed):
//   36 B x P   (12 B upper-bound C slots + 12 B compacted C + 12 B per-request
//               copy of the result or heavy-row scratch)
// + 40 B x rows(A) (row work, offsets, bin lists)
// + the staged operands when they come from host memory.
// A device result stays charged (its own size) until spg_poll hands it over,
// so results that nobody has collected yet cannot push HBM over the budget.
// Host-resident operands are counted on the host at submit time; device ones
// by a counting pass (the engine's K1) on the lane before admission.
//
// Every row is computed by the same kernel and in the same order whatever
// else shares its batch, so a result is bit-identical alone and in a mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/spgemm_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

enum class State { Pending, Counting, Running, Done, Failed, Cancelled };

struct Request {
    uint64_t ticket = 0;
    spg_csr_view A{}, B{};
    int64_t products = -1;   // -1: not counted yet
    int64_t footprint = 0;   // admission charge in bytes
    State state = State::Pending;
    spg_status status = SPG_OK;
    std::string message;
    spg_csr_result result{};
    Clock::time_point t_submit, t_admit, t_done;
    int32_t batch_requests = 0;
    int32_t lane = -1;
    uint64_t batch_id = 0;
    int64_t batch_launches = 0;
    int64_t held = 0;  // bytes still charged after completion: an unpolled device result
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

int64_t staged_bytes(const spg_csr_view& m) {
    return m.location == SPG_HOST ? 8 * (static_cast<int64_t>(m.rows) + 1) + 12 * m.nnz : 0;
}

int64_t footprint_of(const Request& r) {
    int64_t f = 36 * r.products + 40 * (static_cast<int64_t>(r.A.rows) + 1) + staged_bytes(r.A);
    const bool same = r.A.row_ptr == r.B.row_ptr && r.A.col == r.B.col && r.A.val == r.B.val;
    if (!same) f += staged_bytes(r.B);
    return f + (4 << 20);
}

// P of host-resident operands (the sum over A's entries of B's row lengths).
// Malformed inputs give -1: the engine reports their error when they run.
int64_t host_products(const spg_csr_view& A, const spg_csr_view& B) {
    if (A.rows < 0 || B.rows < 0 || !A.row_ptr || !B.row_ptr || A.cols != B.rows) return -1;
    if (A.nnz > 0 && !A.col) return -1;
    int64_t p = 0;
    for (int64_t i = 0; i < A.nnz; ++i) {
        const int32_t k = A.col[i];
        if (k < 0 || k >= B.rows) return -1;
        const int64_t len = B.row_ptr[k + 1] - B.row_ptr[k];
        if (len < 0) return -1;
        p += len;
    }
    return p;
}

}  // namespace

struct spg_server {
    spg_server_config cfg{};
    std::vector<spg_handle*> handles;  // one per lane, used only by its worker thread
    spg_handle* svc = nullptr;          // frees results on behalf of callers
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, Request*> live;
    uint64_t next_ticket = 1;
    uint64_t next_batch = 1;
    int64_t in_use = 0;
    bool stop = false;

    void lane_main(int lane);
    void run_batch(int lane, std::vector<Request*>& batch);
    void count_products(int lane, std::vector<Request*>& reqs);
};

namespace {

void finish_request(Request* r, spg_status s, const std::string& msg) {
    r->status = s;
    r->message = msg;
    r->state = s == SPG_OK ? State::Done : State::Failed;
    r->t_done = Clock::now();
}

}  // namespace

// Counts P of device-resident requests with one batched K1 pass on the lane.
void spg_server::count_products(int lane, std::vector<Request*>& reqs) {
    spg_handle* h = handles[lane];
    const int n = static_cast<int>(reqs.size());
    std::vector<spg_csr_view> A(n), B(n);
    for (int i = 0; i < n; ++i) {
        A[i] = reqs[i]->A;
        B[i] = reqs[i]->B;
    }
    std::vector<int64_t> p(n, 0);
    spg_status s = spg_scalar_multiplication_count_batch(h, n, A.data(), B.data(), p.data());
    std::vector<spg_status> each(n, s);
    std::vector<std::string> msg(n, s == SPG_OK ? "" : spg_last_error(h));
    if (s != SPG_OK && n > 1) {  // attribute the failure request by request
        for (int i = 0; i < n; ++i) {
            each[i] = spg_scalar_multiplication_count(h, &A[i], &B[i], &p[i]);
            msg[i] = each[i] == SPG_OK ? "" : spg_last_error(h);
        }
    }
    std::lock_guard<std::mutex> lk(mu);
    for (int i = 0; i < n; ++i) {
        Request* r = reqs[i];
        if (each[i] != SPG_OK) {
            pending.erase(std::find(pending.begin(), pending.end(), r));
            finish_request(r, each[i], msg[i]);
            continue;
        }
        r->products = p[i];
        r->footprint = footprint_of(*r);
        r->state = State::Pending;
    }
    cv.notify_all();
}

void spg_server::run_batch(int lane, std::vector<Request*>& batch) {
    spg_handle* h = handles[lane];
    const int n = static_cast<int>(batch.size());
    std::vector<spg_csr_view> A(n), B(n);
    std::vector<spg_csr_result> C(n);
    for (int i = 0; i < n; ++i) {
        A[i] = batch[i]->A;
        B[i] = batch[i]->B;
    }
    std::vector<spg_status> each(n);
    std::vector<std::string> msg(n);
    const spg_status s = spg_multiply_batch(h, n, A.data(), B.data(), cfg.out_location, C.data());
    spg_timings t{};
    spg_last_timings(h, &t);
    int64_t launches = t.launches;
    if (s == SPG_OK) {
        std::fill(each.begin(), each.end(), SPG_OK);
    } else if (n > 1 && (s == SPG_INVALID_ARGUMENT || s == SPG_OUT_OF_RANGE_COLUMN || s == SPG_OVERFLOW)) {
        // an input error of some request: run them one by one so that only it fails
        for (int i = 0; i < n; ++i) {
            each[i] = spg_multiply(h, &A[i], &B[i], cfg.out_location, &C[i]);
            if (each[i] != SPG_OK) msg[i] = spg_last_error(h);
            spg_last_timings(h, &t);
            launches += t.launches;
        }
    } else {
        std::fill(each.begin(), each.end(), s);
        std::fill(msg.begin(), msg.end(), std::string(spg_last_error(h)));
    }
    std::lock_guard<std::mutex> lk(mu);
    int64_t fp = 0;
    for (int i = 0; i < n; ++i) {
        Request* r = batch[i];
        r->batch_launches = launches;
        if (each[i] == SPG_OK) {
            r->result = C[i];
            if (C[i].location == SPG_DEVICE)
                r->held = std::min<int64_t>(r->footprint, 8 * (static_cast<int64_t>(C[i].rows) + 1) + 12 * C[i].nnz);
        }
        fp += r->footprint - r->held;
        finish_request(r, each[i], msg[i]);
    }
    in_use -= fp;
    cv.notify_all();
}

void spg_server::lane_main(int lane) {
    const int64_t budget = static_cast<int64_t>(cfg.hbm_budget_bytes);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        if (stop) return;
        // 1. requests whose footprint is unknown (device operands): count them first
        std::vector<Request*> to_count;
        for (Request* r : pending) {
            if (static_cast<int>(to_count.size()) >= cfg.max_batch) break;
            if (r->products < 0 && r->state == State::Pending) to_count.push_back(r);
        }
        if (!to_count.empty()) {
            for (Request* r : to_count) r->state = State::Counting;
            lk.unlock();
            count_products(lane, to_count);
            lk.lock();
            continue;
        }
        // 2. admission: the longest FIFO prefix that fits the free budget
        std::vector<Request*> batch;
        int64_t fp = 0, batch_products = 0;
        for (auto it = pending.begin(); it != pending.end();) {
            Request* r = *it;
            if (r->products < 0) break;  // still being counted by another lane: keep the order
            if (r->footprint > budget) {  // can never fit
                it = pending.erase(it);
                finish_request(r, SPG_BUDGET_EXCEEDED,
                               "request footprint (" + std::to_string(r->footprint) + " B) exceeds the HBM budget");
                cv.notify_all();
                continue;
            }
            if (in_use + fp + r->footprint > budget) break;  // wait for memory: FIFO order
            if (!batch.empty() && batch_products + r->products > cfg.max_batch_products) break;
            batch.push_back(r);
            fp += r->footprint;
            batch_products += r->products;
            ++it;
            if (static_cast<int>(batch.size()) >= cfg.max_batch) break;
        }
        if (batch.empty()) {
            cv.wait(lk);  // new arrivals, a finished batch, a finished count or shutdown
            continue;
        }
        pending.erase(pending.begin(), pending.begin() + static_cast<long>(batch.size()));
        in_use += fp;
        const auto now = Clock::now();
        const uint64_t id = next_batch++;
        for (Request* r : batch) {
            r->batch_id = id;
            r->state = State::Running;
            r->t_admit = now;
            r->batch_requests = static_cast<int32_t>(batch.size());
            r->lane = lane;
        }
        lk.unlock();
        run_batch(lane, batch);
        lk.lock();
    }
}

extern "C" {

spg_status spg_server_config_default(spg_server_config* c) {
    if (!c) return SPG_INVALID_ARGUMENT;
    std::memset(c, 0, sizeof(*c));
    c->lanes = 2;
    c->max_batch = 256;
    c->out_location = SPG_DEVICE;
    c->mode = SPG_MODE_AUTO;
    c->hbm_budget_bytes = 150ull * 1000 * 1000 * 1000;
    c->max_batch_products = int64_t{1} << 28;
    return SPG_OK;
}

spg_status spg_server_create(const spg_server_config* config, spg_server** out) {
    if (!out) return SPG_INVALID_ARGUMENT;
    *out = nullptr;
    spg_server_config cfg;
    spg_server_config_default(&cfg);
    if (config) cfg = *config;
    if (cfg.lanes < 1 || cfg.lanes > 16 || cfg.max_batch < 1 || cfg.hbm_budget_bytes == 0 ||
        cfg.max_batch_products < 1 ||
        (cfg.out_location != SPG_HOST && cfg.out_location != SPG_DEVICE))
        return SPG_INVALID_ARGUMENT;
    auto* s = new spg_server;
    s->cfg = cfg;
    for (int i = 0; i <= cfg.lanes; ++i) {
        spg_config hc;
        spg_config_default(&hc);
        hc.device = cfg.device;
        hc.mode = cfg.mode;
        hc.bin_streams = cfg.lanes > 1 ? 1 : 0;  // the lanes already overlap batches on the device
        spg_handle* h = nullptr;
        const spg_status st = spg_create(&hc, &h);
        if (st != SPG_OK) {
            for (spg_handle* q : s->handles) spg_destroy(q);
            if (s->svc) spg_destroy(s->svc);
            delete s;
            return st;
        }
        if (i < cfg.lanes) s->handles.push_back(h);
        else s->svc = h;
    }
    for (int i = 0; i < cfg.lanes; ++i) s->workers.emplace_back([s, i] { s->lane_main(i); });
    *out = s;
    return SPG_OK;
}

void spg_server_destroy(spg_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Request* r : s->pending) finish_request(r, SPG_CANCELLED, "server destroyed");
        s->pending.clear();
        s->cv.notify_all();
    }
    for (auto& t : s->workers) t.join();
    for (auto& kv : s->live) {
        Request* r = kv.second;
        if (r->state == State::Done) spg_result_free(s->svc, &r->result);
        delete r;
    }
    for (spg_handle* h : s->handles) spg_destroy(h);
    spg_destroy(s->svc);
    delete s;
}

spg_status spg_submit(spg_server* s, const spg_csr_view* A, const spg_csr_view* B, uint64_t* ticket) {
    if (!s || !A || !B || !ticket) return SPG_INVALID_ARGUMENT;
    auto* r = new Request;
    r->A = *A;
    r->B = *B;
    r->t_submit = Clock::now();
    if (A->location == SPG_HOST && B->location == SPG_HOST) {
        r->products = host_products(*A, *B);
        if (r->products < 0) r->products = 0;  // malformed: the engine reports it when the request runs
        r->footprint = footprint_of(*r);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        delete r;
        return SPG_CANCELLED;
    }
    r->ticket = s->next_ticket++;
    s->live[r->ticket] = r;
    s->pending.push_back(r);
    *ticket = r->ticket;
    s->cv.notify_all();
    return SPG_OK;
}

spg_status spg_poll(spg_server* s, uint64_t ticket, int32_t wait_ms, spg_csr_result* C, spg_request_info* info) {
    if (!s || !C) return SPG_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return SPG_INVALID_ARGUMENT;
    Request* r = it->second;
    auto terminal = [r] { return r->state == State::Done || r->state == State::Failed || r->state == State::Cancelled; };
    if (wait_ms < 0) s->cv.wait(lk, terminal);
    else if (wait_ms > 0) s->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), terminal);
    if (!terminal()) return SPG_NOT_READY;
    if (info) {
        std::memset(info, 0, sizeof(*info));
        const bool ran = r->lane >= 0;
        info->queue_ms = ran ? ms_between(r->t_submit, r->t_admit) : ms_between(r->t_submit, r->t_done);
        info->service_ms = ran ? ms_between(r->t_admit, r->t_done) : 0.0;
        info->latency_ms = ms_between(r->t_submit, r->t_done);
        info->products = r->products;
        info->footprint_bytes = r->footprint;
        info->batch_requests = r->batch_requests;
        info->lane = r->lane;
        info->batch_id = r->batch_id;
        info->batch_launches = r->batch_launches;
        std::snprintf(info->message, sizeof info->message, "%s", r->message.c_str());
    }
    const spg_status st = r->state == State::Cancelled ? SPG_CANCELLED : r->status;
    std::memset(C, 0, sizeof(*C));
    if (r->state == State::Done) *C = r->result;
    if (r->held) {  // the result is the caller's from now on
        s->in_use -= r->held;
        s->cv.notify_all();
    }
    s->live.erase(it);
    delete r;
    return st;
}

spg_status spg_cancel(spg_server* s, uint64_t ticket) {
    if (!s) return SPG_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return SPG_INVALID_ARGUMENT;
    Request* r = it->second;
    if (r->state != State::Pending) return r->state == State::Cancelled ? SPG_OK : SPG_NOT_READY;
    s->pending.erase(std::find(s->pending.begin(), s->pending.end(), r));
    r->state = State::Cancelled;
    r->t_done = Clock::now();
    s->cv.notify_all();
    return SPG_OK;
}

spg_status spg_server_result_free(spg_server* s, spg_csr_result* C) {
    if (!s || !C) return SPG_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);  // serialises callers on the service handle
    return spg_result_free(s->svc, C);
}

}  // extern "C"
