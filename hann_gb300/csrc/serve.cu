// serve.cu -- continuous-batching search server on one GPU.
//
// Requests (a block of queries with its own k and nprobe) arrive from any
// number of host threads. A scheduler thread packs waiting requests into
// device batches and runs each batch on one of `slots` CUDA streams, each
// with its own scratch (SearchScratch) and pinned staging buffers, so up to
// `slots` batches are in flight and overlap on the device. Requests that
// arrive while batches run are admitted into the next free slot; a batch
// takes requests in arrival order while its queries fit max_batch_queries,
// its summed nprobe fits max_batch_probes (when set) and its device scratch
// fits the slot's share of the memory budget
// (admission by device memory). Add/Delete requests go, in order, to a
// mutation thread that applies them beside the running batches: an append
// into spare capacity and a tombstone delete move no row, so batches in
// flight see each mutation either not at all or whole. Only a mutation that
// must move rows (a relayout) stops the scheduler from starting batches;
// the mutation thread then waits for the running ones and applies it under
// the index's exclusive lock. A search sees every mutation whose ticket was
// waited for before the search was submitted.
//
// Every request is an ordinary Search of its queries (pqivf/index.go:850-949)
// with per-query k and nprobe, so its result does not depend on what it was
// batched with.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <vector>

#include "index_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    int kind = 0;  // 0 search, 1 add, 2 delete
    int32_t nq = 0, k = 0, nprobe = 0;
    std::vector<float> queries;
    std::vector<int64_t> ids;  // add/delete
    std::vector<float> vectors;
    std::vector<int64_t> out_ids;
    std::vector<double> out_dist;
    std::vector<int32_t> out_n;
    int priority = 0;  // 1: taken before every normal request still queued
    int status = 1;  // 1 pending, 0 done, <0 error
    std::string error;
    Clock::time_point t_submit, t_done;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    SearchScratch sc;
    float* h_q = nullptr;  // pinned staging
    int32_t* h_k = nullptr;
    int32_t* h_np = nullptr;
    int64_t* h_ids = nullptr;
    double* h_dist = nullptr;
    int32_t* h_n = nullptr;
    DBuf<float> d_q;
    DBuf<int32_t> d_k, d_np, d_n;
    DBuf<int64_t> d_ids;
    DBuf<double> d_dist;
    bool busy = false;
    int kmax = 0;
    std::vector<std::shared_ptr<Request>> reqs;
    std::vector<int32_t> offsets;
};

}  // namespace

// Message of the calling thread's last failed hann_serve_* call.
static thread_local std::string t_serve_error;

static int serve_fail(int rc, const char* msg) {
    t_serve_error = msg;
    return rc;
}

struct hann_server {
    hann_pqivf* h = nullptr;
    hann_serve_options o{};
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::deque<std::shared_ptr<Request>> queue_hi;  // high-priority searches, taken first
    std::unordered_map<uint64_t, std::shared_ptr<Request>> tickets;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread thr;
    // statistics
    std::vector<double> lat_ms;
    int64_t queries_done = 0, requests_done = 0, batches = 0, mutations = 0;
    int64_t peak_admitted = 0, cur_admitted = 0, relayouts = 0;
    double mutation_ms = 0.0, drain_ms = 0.0, relayout_ms = 0.0, relayout_max_ms = 0.0;
    // mutation thread: its FIFO, and the drain handshake for relayouts
    std::deque<std::shared_ptr<Request>> mqueue;
    std::condition_variable cv_mut;
    std::thread mthr;
    bool drain_wanted = false;  // set by the mutation thread; the scheduler stops launching
    bool drained = false;       // set by the scheduler once nothing is in flight
    bool mstop = false;
    bool sched_done = false;    // the scheduler has exited: nothing runs any more
    Clock::time_point t_first{}, t_last{};
    bool any = false;
    std::shared_lock<std::shared_mutex> read_lock;  // held while batches run
    int64_t slot_budget = 0;
};

namespace {

int64_t batch_bytes(const hann_pqivf* h, int64_t nq, int kmax, int np_max, int mode) {
    const int R = rerank_depth(h, kmax, mode);
    const int64_t dim = h->o.dimension;
    const int64_t dump = scan_adc_supported(h->o.num_subquantizers) ? (int64_t)scan_dump_bytes(R) : 0;
    return nq * (h->nlist * 4 + np_max * 8 + R * 12 + dim * 4 + h->kp * 2 + 4 * 6 + kmax * 16 + dump) + 4096;
}

void complete(hann_server* s, Slot& sl) {
    // results are in the slot's pinned buffers
    for (size_t i = 0; i < sl.reqs.size(); i++) {
        auto& r = sl.reqs[i];
        const int off = sl.offsets[i];
        r->out_ids.resize((size_t)r->nq * r->k);
        r->out_dist.resize((size_t)r->nq * r->k);
        r->out_n.resize((size_t)r->nq);
        for (int q = 0; q < r->nq; q++) {
            std::memcpy(&r->out_ids[(size_t)q * r->k], &sl.h_ids[(size_t)(off + q) * sl.kmax], sizeof(int64_t) * r->k);
            std::memcpy(&r->out_dist[(size_t)q * r->k], &sl.h_dist[(size_t)(off + q) * sl.kmax],
                        sizeof(double) * r->k);
            r->out_n[q] = sl.h_n[off + q];
        }
        r->t_done = Clock::now();
        r->status = 0;
        s->lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
        s->queries_done += r->nq;
        s->requests_done++;
        s->t_last = r->t_done;
    }
    sl.reqs.clear();
    sl.offsets.clear();
    sl.busy = false;
}

// Launches a batch on a free slot. Called with s->mu held and the index's
// shared lock taken.
int launch_batch(hann_server* s, Slot& sl, std::vector<std::shared_ptr<Request>>& take) {
    hann_pqivf* h = s->h;
    int64_t nq = 0;
    int kmax = 1, np_max = 1;
    for (auto& r : take) {
        nq += r->nq;
        kmax = std::max(kmax, r->k);
        np_max = std::max(np_max, std::min(r->nprobe, h->nlist));
    }
    const int dim = h->o.dimension;
    int64_t off = 0;
    sl.reqs = take;
    sl.offsets.clear();
    for (auto& r : take) {
        sl.offsets.push_back((int32_t)off);
        std::memcpy(sl.h_q + off * dim, r->queries.data(), sizeof(float) * r->nq * dim);
        for (int q = 0; q < r->nq; q++) {
            sl.h_k[off + q] = r->k;
            sl.h_np[off + q] = std::min(r->nprobe, h->nlist);
        }
        off += r->nq;
    }
    sl.kmax = kmax;
    cudaStream_t st = sl.stream;
    CK(cudaMemcpyAsync(sl.d_q.p, sl.h_q, sizeof(float) * nq * dim, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(sl.d_k.p, sl.h_k, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(sl.d_np.p, sl.h_np, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, st));
    CK(sl.sc.fbcount.reserve(1));
    CK(cudaMemsetAsync(sl.sc.fbcount.p, 0, sizeof(unsigned long long), st));
    int rc = run_search(h, sl.sc, sl.d_q.p, nq, sl.d_k.p, sl.d_np.p, np_max, kmax, s->o.mode, sl.d_ids.p,
                        sl.d_dist.p, sl.d_n.p, st);
    if (rc) return rc;
    CK(cudaMemcpyAsync(sl.h_ids, sl.d_ids.p, sizeof(int64_t) * nq * kmax, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(sl.h_dist, sl.d_dist.p, sizeof(double) * nq * kmax, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(sl.h_n, sl.d_n.p, sizeof(int32_t) * nq, cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(sl.done, st));
    sl.busy = true;
    s->batches++;
    const int64_t b = batch_bytes(h, nq, kmax, np_max, s->o.mode);
    s->cur_admitted += b;
    s->peak_admitted = std::max(s->peak_admitted, s->cur_admitted);
    return HANN_OK;
}

void fail_requests(hann_server* s, std::vector<std::shared_ptr<Request>>& rs, int code, const std::string& msg) {
    for (auto& r : rs) {
        r->status = code < 0 ? code : HANN_E_CUDA;
        r->error = msg;
    }
}

// Applies Add/Delete requests in submission order. An append or tombstone
// delete runs under the writer lock beside the scheduler's batches; one that
// needs a relayout asks the scheduler to drain, then runs under the index's
// exclusive lock.
void mutator(hann_server* s) {
    hann_pqivf* h = s->h;
    cudaSetDevice(h->o.device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_mut.wait(lk, [&] { return s->mstop || !s->mqueue.empty(); });
        if (s->mqueue.empty()) break;
        auto r = s->mqueue.front();
        lk.unlock();
        auto apply = [&](bool allow, bool* needs) {
            return r->kind == 1 ? bulk_add_locked(h, r->ids.data(), r->vectors.data(), (int64_t)r->ids.size(), allow,
                                                  needs)
                                : bulk_delete_locked(h, r->ids.data(), (int64_t)r->ids.size(), allow, needs);
        };
        const auto t0 = Clock::now();
        bool needs = false, relaid = false;
        Clock::time_point t1, t2, t3;
        int rc;
        {
            std::lock_guard<std::mutex> wl(h->wmu);
            rc = apply(false, &needs);
        }
        if (needs) {
            lk.lock();
            s->drain_wanted = true;
            s->drained = s->sched_done;
            s->cv_work.notify_one();
            t1 = Clock::now();
            s->cv_mut.wait(lk, [&] { return s->drained; });
            lk.unlock();
            t2 = Clock::now();
            {
                std::lock_guard<std::mutex> wl(h->wmu);
                std::unique_lock<std::shared_mutex> xl(h->mu);
                const cudaError_t we = wait_device_searches(h);
                rc = we == cudaSuccess ? apply(true, nullptr) : h->cuda_fail(we, "waiting for device searches");
            }
            t3 = Clock::now();
            relaid = true;
        }
        lk.lock();
        if (relaid) {
            s->drain_wanted = false;
            s->drained = false;
            s->relayouts++;
            s->drain_ms += std::chrono::duration<double, std::milli>(t2 - t1).count();
            s->relayout_ms += std::chrono::duration<double, std::milli>(t3 - t2).count();
            s->relayout_max_ms =
                std::max(s->relayout_max_ms, std::chrono::duration<double, std::milli>(t3 - t1).count());
            s->cv_work.notify_one();
        }
        s->mqueue.pop_front();
        if (rc) r->error = hann_thread_error();
        r->status = rc;
        r->t_done = Clock::now();
        s->mutations++;
        s->mutation_ms += std::chrono::duration<double, std::milli>(r->t_done - t0).count();
        s->cv_done.notify_all();
    }
}

void scheduler(hann_server* s) {
    hann_pqivf* h = s->h;
    cudaSetDevice(h->o.device);
    std::unique_lock<std::mutex> lk(s->mu);
    std::vector<int64_t> slot_bytes(s->slots.size(), 0);
    for (;;) {
        // 1. completions
        bool any_busy = false;
        for (size_t i = 0; i < s->slots.size(); i++) {
            Slot& sl = *s->slots[i];
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaSuccess) {
                complete(s, sl);
                s->cur_admitted -= slot_bytes[i];
                slot_bytes[i] = 0;
                s->cv_done.notify_all();
            } else if (q != cudaErrorNotReady) {
                fail_requests(s, sl.reqs, HANN_E_CUDA, cudaGetErrorString(q));
                sl.reqs.clear();
                sl.busy = false;
                s->cv_done.notify_all();
            } else {
                any_busy = true;
            }
        }
        if (!any_busy && s->read_lock.owns_lock()) s->read_lock.unlock();
        if (s->stop && s->queue.empty() && s->queue_hi.empty() && !any_busy) break;
        // 2. mutations at the head of the queue go to the mutation thread
        while (!s->queue.empty() && s->queue.front()->kind != 0) {
            s->mqueue.push_back(s->queue.front());
            s->queue.pop_front();
            s->cv_mut.notify_one();
        }
        // a relayout waits for the batches in flight; none start meanwhile
        if (s->drain_wanted) {
            if (!any_busy && !s->drained) {
                if (s->read_lock.owns_lock()) s->read_lock.unlock();
                s->drained = true;
                s->cv_mut.notify_one();
            }
        } else if (!s->queue.empty() || !s->queue_hi.empty()) {
            // 3. pack waiting searches into every free slot, high priority first
            auto next = [&]() -> std::deque<std::shared_ptr<Request>>* {
                if (!s->queue_hi.empty()) return &s->queue_hi;
                if (!s->queue.empty() && s->queue.front()->kind == 0) return &s->queue;
                return nullptr;
            };
            for (size_t i = 0; i < s->slots.size() && next(); i++) {
                Slot& sl = *s->slots[i];
                if (sl.busy) continue;
                std::vector<std::shared_ptr<Request>> take;
                int64_t nq = 0, probes = 0;
                int kmax = 1, npm = 1;
                while (auto* qq = next()) {
                    auto& r = qq->front();
                    const int64_t nq2 = nq + r->nq;
                    const int k2 = std::max(kmax, r->k), np2 = std::max(npm, std::min(r->nprobe, h->nlist));
                    const int64_t pr2 = probes + (int64_t)r->nq * std::min(r->nprobe, h->nlist);
                    if (!take.empty() && s->o.max_batch_probes > 0 && pr2 > s->o.max_batch_probes) break;
                    if (nq2 > s->o.max_batch_queries || batch_bytes(h, nq2, k2, np2, s->o.mode) > s->slot_budget) {
                        if (take.empty()) {
                            // a request that can never fit
                            r->status = HANN_E_UNSUPPORTED;
                            r->error = "request exceeds the server's per-batch query or memory limit";
                            qq->pop_front();
                            s->cv_done.notify_all();
                            continue;
                        }
                        break;
                    }
                    nq = nq2;
                    kmax = k2;
                    npm = np2;
                    probes = pr2;
                    take.push_back(r);
                    qq->pop_front();
                }
                if (take.empty()) continue;
                if (!s->read_lock.owns_lock()) s->read_lock = std::shared_lock<std::shared_mutex>(h->mu);
                const int rc = launch_batch(s, sl, take);
                if (rc) {
                    fail_requests(s, take, rc, hann_thread_error());
                    sl.reqs.clear();
                    sl.busy = false;
                    s->cv_done.notify_all();
                } else {
                    slot_bytes[i] = batch_bytes(h, nq, kmax, npm, s->o.mode);
                    any_busy = true;
                }
            }
        }
        // 4. wait for new work or a completion (poll completions every 50 us)
        if (s->drain_wanted && s->drained) {
            s->cv_work.wait_for(lk, std::chrono::milliseconds(1));
        } else if (any_busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(50));
            lk.lock();
        } else if (s->queue.empty() && s->queue_hi.empty() && !s->stop) {
            s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        }
    }
    if (s->read_lock.owns_lock()) s->read_lock.unlock();
    // nothing runs any more: a pending relayout may go ahead
    s->sched_done = true;
    s->drained = true;
    s->cv_mut.notify_one();
}

void free_slot(Slot& sl) {
    if (sl.stream) {
        cudaStreamSynchronize(sl.stream);
        cudaStreamDestroy(sl.stream);
    }
    if (sl.done) cudaEventDestroy(sl.done);
    cudaFreeHost(sl.h_q);
    cudaFreeHost(sl.h_k);
    cudaFreeHost(sl.h_np);
    cudaFreeHost(sl.h_ids);
    cudaFreeHost(sl.h_dist);
    cudaFreeHost(sl.h_n);
}

}  // namespace

extern "C" {

void hann_serve_options_init(hann_serve_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->slots = 4;
    o->max_batch_queries = 4096;
    o->max_k = 100;
    o->max_nprobe = 256;
    o->mode = 1;
    o->memory_budget = (int64_t)120 << 30;
}

int hann_serve_start(hann_pqivf* h, const hann_serve_options* opts, hann_server** out) {
    if (!h || !opts || !out) return HANN_E_INVALID;
    hann_serve_options o = *opts;
    if (o.slots < 1 || o.slots > 64 || o.max_batch_queries < 1 || o.max_k < 1 || o.max_nprobe < 1 ||
        (o.mode != 0 && o.mode != 1) || o.memory_budget <= 0)
        return h->fail(HANN_E_INVALID, "invalid server options");
    {
        std::shared_lock<std::shared_mutex> lk(h->mu);
        int rc = check_searchable(h);
        if (rc) return rc;
    }
    cudaSetDevice(h->o.device);
    auto s = std::make_unique<hann_server>();
    s->h = h;
    s->o = o;
    const int np_max = std::min(o.max_nprobe, h->nlist);
    s->slot_budget = o.memory_budget / o.slots;
    const int64_t need = batch_bytes(h, o.max_batch_queries, o.max_k, np_max, o.mode);
    if (need > s->slot_budget)
        return h->fail(HANN_E_NOMEM, "memory budget %lld below %d slots x %lld bytes for %d-query batches",
                       (long long)o.memory_budget, o.slots, (long long)need, o.max_batch_queries);
    const int dim = h->o.dimension;
    const int64_t Q = o.max_batch_queries, K = o.max_k;
    for (int i = 0; i < o.slots; i++) {
        auto sl = std::make_unique<Slot>();
        cudaError_t e = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->h_q, sizeof(float) * Q * dim);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->h_k, sizeof(int32_t) * Q);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->h_np, sizeof(int32_t) * Q);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->h_ids, sizeof(int64_t) * Q * K);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->h_dist, sizeof(double) * Q * K);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->h_n, sizeof(int32_t) * Q);
        if (e == cudaSuccess) e = sl->d_q.reserve((size_t)Q * dim);
        if (e == cudaSuccess) e = sl->d_k.reserve((size_t)Q);
        if (e == cudaSuccess) e = sl->d_np.reserve((size_t)Q);
        if (e == cudaSuccess) e = sl->d_n.reserve((size_t)Q);
        if (e == cudaSuccess) e = sl->d_ids.reserve((size_t)Q * K);
        if (e == cudaSuccess) e = sl->d_dist.reserve((size_t)Q * K);
        // Size the slot's search scratch for its largest batch now, so the
        // scheduler never calls the allocator while batches are in flight.
        if (e == cudaSuccess && reserve_search_scratch(h, sl->sc, Q, np_max, o.max_k, o.mode) != HANN_OK)
            e = cudaErrorMemoryAllocation;
        sl->sc.dump_off = sl->sc.dump.p == nullptr;
        if (e != cudaSuccess) {
            free_slot(*sl);
            for (auto& x : s->slots) free_slot(*x);
            return h->cuda_fail(e, "server slot allocation");
        }
        s->slots.push_back(std::move(sl));
    }
    hann_server* raw = s.release();
    raw->thr = std::thread(scheduler, raw);
    raw->mthr = std::thread(mutator, raw);
    *out = raw;
    return HANN_OK;
}

static int submit(hann_server* s, std::shared_ptr<Request> r, uint64_t* ticket) {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return serve_fail(HANN_E_STATE, "the server is stopping");
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    if (!s->any) {
        s->t_first = r->t_submit;
        s->any = true;
    }
    s->tickets[r->ticket] = r;
    if (r->kind == 0 && r->priority > 0) s->queue_hi.push_back(r);
    else s->queue.push_back(r);
    s->cv_work.notify_one();
    if (ticket) *ticket = r->ticket;
    return HANN_OK;
}

int hann_serve_submit(hann_server* s, const float* queries, int32_t nq, int32_t k, int32_t nprobe, uint64_t* ticket) {
    if (!s || !queries || nq <= 0) return serve_fail(HANN_E_INVALID, "invalid arguments: no queries");
    if (k <= 0 || k > s->o.max_k) return serve_fail(HANN_E_INVALID, "k must be in [1, the server's max_k]");
    if (nprobe <= 0) nprobe = s->h->o.candidate_clusters;
    if (nprobe > s->o.max_nprobe) nprobe = s->o.max_nprobe;
    auto r = std::make_shared<Request>();
    r->kind = 0;
    r->nq = nq;
    r->k = k;
    r->nprobe = nprobe;
    r->queries.assign(queries, queries + (size_t)nq * s->h->o.dimension);
    return submit(s, r, ticket);
}

int hann_serve_submit_priority(hann_server* s, const float* queries, int32_t nq, int32_t k, int32_t nprobe,
                               int32_t priority, uint64_t* ticket) {
    if (!s || !queries || nq <= 0) return serve_fail(HANN_E_INVALID, "invalid arguments: no queries");
    if (k <= 0 || k > s->o.max_k) return serve_fail(HANN_E_INVALID, "k must be in [1, the server's max_k]");
    if (nprobe <= 0) nprobe = s->h->o.candidate_clusters;
    if (nprobe > s->o.max_nprobe) nprobe = s->o.max_nprobe;
    auto r = std::make_shared<Request>();
    r->kind = 0;
    r->nq = nq;
    r->k = k;
    r->nprobe = nprobe;
    r->priority = priority > 0 ? 1 : 0;
    r->queries.assign(queries, queries + (size_t)nq * s->h->o.dimension);
    return submit(s, r, ticket);
}

int hann_serve_cancel(hann_server* s, uint64_t ticket) {
    if (!s) return HANN_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return serve_fail(HANN_E_NOT_FOUND, "unknown ticket");
    auto r = it->second;
    for (auto* qq : {&s->queue_hi, &s->queue}) {
        for (auto q = qq->begin(); q != qq->end(); ++q) {
            if (q->get() != r.get()) continue;
            if (r->kind != 0) break;  // mutations are not cancelled
            qq->erase(q);
            r->status = HANN_E_STATE;
            r->error = "request cancelled";
            r->t_done = Clock::now();
            s->cv_done.notify_all();
            return HANN_OK;
        }
    }
    return serve_fail(HANN_E_STATE, "request already started or finished");
}

int hann_serve_submit_add(hann_server* s, const int64_t* ids, const float* vectors, int64_t n, uint64_t* ticket) {
    if (!s || n < 0 || (n > 0 && (!ids || !vectors))) return serve_fail(HANN_E_INVALID, "invalid arguments");
    auto r = std::make_shared<Request>();
    r->kind = 1;
    r->ids.assign(ids, ids + n);
    r->vectors.assign(vectors, vectors + n * s->h->o.dimension);
    return submit(s, r, ticket);
}

int hann_serve_submit_delete(hann_server* s, const int64_t* ids, int64_t n, uint64_t* ticket) {
    if (!s || n < 0 || (n > 0 && !ids)) return serve_fail(HANN_E_INVALID, "invalid arguments");
    auto r = std::make_shared<Request>();
    r->kind = 2;
    r->ids.assign(ids, ids + n);
    return submit(s, r, ticket);
}

int hann_serve_wait(hann_server* s, uint64_t ticket, int64_t* ids, double* distances, int32_t* n_out,
                    int32_t timeout_ms, double* latency_ms) {
    if (!s) return HANN_E_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return serve_fail(HANN_E_NOT_FOUND, "unknown ticket");
    auto r = it->second;
    const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 1000000000 : timeout_ms);
    while (r->status == 1) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && r->status == 1) {
            return serve_fail(HANN_E_STATE, "timed out waiting for the request");
        }
    }
    s->tickets.erase(it);
    if (r->status < 0) {
        t_serve_error = r->error;
        return r->status;
    }
    if (r->kind == 0) {
        if (ids) std::memcpy(ids, r->out_ids.data(), sizeof(int64_t) * r->out_ids.size());
        if (distances) std::memcpy(distances, r->out_dist.data(), sizeof(double) * r->out_dist.size());
        if (n_out) std::memcpy(n_out, r->out_n.data(), sizeof(int32_t) * r->out_n.size());
    }
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    return HANN_OK;
}

int hann_serve_stats(hann_server* s, hann_serve_statistics* out) {
    if (!s || !out) return HANN_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->requests = s->requests_done;
    out->queries = s->queries_done;
    out->batches = s->batches;
    out->mutations = s->mutations;
    out->peak_admitted_bytes = s->peak_admitted;
    out->relayouts = s->relayouts;
    out->mutation_ms = s->mutation_ms;
    out->drain_ms = s->drain_ms;
    out->relayout_ms = s->relayout_ms;
    out->relayout_max_ms = s->relayout_max_ms;
    std::vector<double> l = s->lat_ms;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
        out->queries_per_s = span > 0 ? s->queries_done / span : 0.0;
    }
    return HANN_OK;
}

const char* hann_serve_last_error(const hann_server*) { return t_serve_error.c_str(); }

int hann_serve_stop(hann_server* s) {
    if (!s) return HANN_E_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->thr.joinable()) s->thr.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->mstop = true;
        s->cv_mut.notify_all();
    }
    if (s->mthr.joinable()) s->mthr.join();
    for (auto& sl : s->slots) free_slot(*sl);
    delete s;
    return HANN_OK;
}

int hann_serve_replay(hann_server* s, const hann_serve_request* reqs, int64_t n, const float* queries,
                      int64_t n_queries, const int64_t* query_rows, int64_t n_query_rows, const int64_t* add_ids,
                      const float* add_vectors, int64_t n_add, const int64_t* del_ids, int64_t n_del,
                      int64_t* out_ids, int64_t n_out_ids, double* latency_ms, double* late_ms) {
    if (!s || (n > 0 && (!reqs || !latency_ms || !late_ms))) return serve_fail(HANN_E_INVALID, "null buffer");
    const int dim = s->h->o.dimension;
    // every range a request names must lie inside the array it indexes
    for (int64_t i = 0; i < n; i++) {
        const hann_serve_request& r = reqs[i];
        bool ok = r.count >= 0 && r.first >= 0 && r.at_ms >= 0.0;
        if (ok && r.kind == 0) {
            ok = queries && query_rows && r.count > 0 && r.count <= INT32_MAX && r.first + r.count <= n_query_rows &&
                 (r.out_offset < 0 || (out_ids && r.k > 0 && r.out_offset + r.count * r.k <= n_out_ids));
            for (int64_t j = 0; ok && j < r.count; j++)
                ok = query_rows[r.first + j] >= 0 && query_rows[r.first + j] < n_queries;
        } else if (ok && r.kind == 1) {
            ok = add_ids && add_vectors && r.first + r.count <= n_add;
        } else if (ok) {
            ok = r.kind == 2 && del_ids && r.first + r.count <= n_del;
        }
        if (!ok) return serve_fail(HANN_E_INVALID, "invalid request in the schedule");
    }
    // The waiter takes the tickets in submission order and records each
    // request's latency (the server's clock); results are copied out only
    // for the searches that keep them.
    struct Pending {
        int64_t i;
        uint64_t ticket;
    };
    std::mutex qm;
    std::condition_variable qcv;
    std::deque<Pending> pending;
    bool submitted_all = false;
    int wait_rc = HANN_OK;
    std::string wait_msg;
    std::thread waiter([&]() {
        std::vector<int64_t> ids;
        while (true) {
            Pending p;
            {
                std::unique_lock<std::mutex> lk(qm);
                qcv.wait(lk, [&] { return !pending.empty() || submitted_all; });
                if (pending.empty()) return;
                p = pending.front();
                pending.pop_front();
            }
            const hann_serve_request& r = reqs[p.i];
            const bool keep = r.kind == 0 && r.out_offset >= 0;
            if (keep) ids.resize((size_t)r.count * r.k);
            double lat = 0.0;
            const int rc = hann_serve_wait(s, p.ticket, keep ? ids.data() : nullptr, nullptr, nullptr, -1, &lat);
            latency_ms[p.i] = lat;
            if (rc != HANN_OK && wait_rc == HANN_OK) {
                wait_rc = rc;
                wait_msg = t_serve_error;
            }
            if (keep && rc == HANN_OK) std::memcpy(out_ids + r.out_offset, ids.data(), sizeof(int64_t) * ids.size());
        }
    });
    int rc = HANN_OK;
    std::vector<float> qbuf;
    const auto t0 = Clock::now();
    for (int64_t i = 0; i < n && rc == HANN_OK; i++) {
        const hann_serve_request& r = reqs[i];
        const auto target = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double, std::milli>(r.at_ms));
        // sleep to within 0.2 ms of the arrival, then spin
        while (true) {
            const auto now = Clock::now();
            if (now >= target) break;
            if (target - now > std::chrono::microseconds(300)) std::this_thread::sleep_for(target - now - std::chrono::microseconds(200));
        }
        late_ms[i] = std::chrono::duration<double, std::milli>(Clock::now() - target).count();
        uint64_t ticket = 0;
        if (r.kind == 0) {
            qbuf.resize((size_t)r.count * dim);
            for (int64_t j = 0; j < r.count; j++)
                std::memcpy(qbuf.data() + (size_t)j * dim, queries + (size_t)query_rows[r.first + j] * dim,
                            sizeof(float) * dim);
            rc = hann_serve_submit(s, qbuf.data(), (int32_t)r.count, r.k, r.nprobe, &ticket);
        } else if (r.kind == 1) {
            rc = hann_serve_submit_add(s, add_ids + r.first, add_vectors + (size_t)r.first * dim, r.count, &ticket);
        } else {
            rc = hann_serve_submit_delete(s, del_ids + r.first, r.count, &ticket);
        }
        if (rc == HANN_OK) {
            std::lock_guard<std::mutex> lk(qm);
            pending.push_back({i, ticket});
            qcv.notify_one();
        }
    }
    const std::string submit_msg = rc == HANN_OK ? std::string() : t_serve_error;
    {
        std::lock_guard<std::mutex> lk(qm);
        submitted_all = true;
        qcv.notify_one();
    }
    waiter.join();
    if (rc != HANN_OK) return serve_fail(rc, submit_msg.c_str());
    if (wait_rc != HANN_OK) return serve_fail(wait_rc, wait_msg.c_str());
    return HANN_OK;
}

}  // extern "C"
