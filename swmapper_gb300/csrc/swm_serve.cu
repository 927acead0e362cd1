// swm_serve.cu -- request loop over resident index: continuous batching of
// mapping requests into block slots.
//
// The reference maps one fixed block of reads at a time and double-buffers
// two of them (mapper_mpe.c:945-1106: read block i + 1 while block i runs on
// the CPEs, athread_spawn / athread_join). A server instead takes requests of
// any size as they arrive: an engine thread coalesces the requests waiting in
// the queue into the next block (up to block_reads reads) as soon as a block
// slot is free, so requests that arrive while other blocks are on the GPU are
// admitted as slots free up and their blocks overlap on the device. A slot is
// one mapper (its own stream and work buffers). Slots are created on demand,
// each only when the device has the memory for it at that moment (and the
// caller's limit allows it); a request that could never be admitted, or that
// would overfill the waiting queue, is refused at submission with a status
// instead of waiting forever. Each block's packed records are split back per
// request; read ids in a request's records are relative to the request.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "swm_common.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id;
    uint32_t n;
    std::vector<char> reads;     // n * server stride
    std::vector<uint32_t> lens;  // n
    std::vector<uint8_t> e;      // n thresholds
    Clock::time_point t_submit, t_done;
    uint32_t block_reads, slot;
    int status;
    std::vector<uint32_t> words, rlen, unmapped;
    std::vector<uint8_t> cigar;
};

struct Slot {
    swm_mapper *m = nullptr;
    bool busy = false;
    std::vector<Request *> reqs;
    std::vector<uint32_t> offs;  // first read of each request in the block
    uint32_t nreads = 0;
    // page-locked block inputs and packed outputs (the mapper copies them directly)
    char *h_reads = nullptr;
    uint32_t *h_lens = nullptr;
    uint8_t *h_e = nullptr;
    uint32_t *h_words = nullptr, *h_rlen = nullptr, *h_unm = nullptr;
    uint8_t *h_cigar = nullptr;
    uint64_t cap_words = 0, cap_cigar = 0, cap_recs = 0;
};

} // namespace

struct swm_server {
    swm_index *ix = nullptr;
    swm_serve_config cfg{};
    std::thread engine;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending, done;
    uint64_t pending_reads = 0;
    std::vector<Slot *> slots;
    uint64_t slot_bytes = 0;  // device memory of one slot, measured when the first was made
    uint64_t held_bytes = 0;
    bool no_slot_fits = false;
    bool stopping = false;
    uint64_t next_id = 1;
    swm_serve_counters st{};
    int engine_error = SWM_OK;
};

static void free_slot(Slot *s) {
    if (!s) return;
    if (s->m) swm_mapper_free(s->m);
    cudaFreeHost(s->h_reads);
    cudaFreeHost(s->h_lens);
    cudaFreeHost(s->h_e);
    cudaFreeHost(s->h_words);
    cudaFreeHost(s->h_rlen);
    cudaFreeHost(s->h_unm);
    cudaFreeHost(s->h_cigar);
    delete s;
}

static bool host_grow(void **p, uint64_t *cap, uint64_t need, size_t elt) {
    if (need <= *cap && *p) return true;
    uint64_t n = need + need / 2 + 4096;
    cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaHostAlloc(p, n * elt, 0) != cudaSuccess) {
        *p = nullptr;
        return false;
    }
    *cap = n;
    return true;
}

// A new slot: one mapper for blocks of cfg.block_reads reads and its
// page-locked staging. Returns nullptr when the device has no room for it.
static Slot *make_slot(swm_server *s) {
    const uint64_t B = s->cfg.block_reads;
    Slot *sl = new Slot();
    size_t free0 = 0, free1 = 0, total = 0;
    cudaMemGetInfo(&free0, &total);
    bool ok = swm_mapper_create(s->ix, B, &sl->m) == SWM_OK &&
              cudaHostAlloc((void **)&sl->h_reads, B * s->cfg.stride, 0) == cudaSuccess &&
              cudaHostAlloc((void **)&sl->h_lens, B * 4, 0) == cudaSuccess &&
              cudaHostAlloc((void **)&sl->h_e, B, 0) == cudaSuccess &&
              cudaHostAlloc((void **)&sl->h_unm, B * 4, 0) == cudaSuccess &&
              host_grow((void **)&sl->h_words, &sl->cap_words, B * 16, 4) &&
              host_grow((void **)&sl->h_cigar, &sl->cap_cigar, B * 64, 1) &&
              host_grow((void **)&sl->h_rlen, &sl->cap_recs, B * 4, 4);
    if (!ok) {
        free_slot(sl);
        cudaGetLastError();
        return nullptr;
    }
    cudaMemGetInfo(&free1, &total);
    if (!s->slot_bytes) {
        // the mapper allocates its read buffer at its first block: count it
        const uint64_t reads_buf = B * (s->cfg.stride > 256 ? s->cfg.stride : 256);
        s->slot_bytes = (free0 > free1 ? free0 - free1 : 0) + reads_buf;
    }
    return sl;
}

// Whether one more slot may be made now: below max_slots, within the
// caller's device-memory limit, and the device reports that much free memory
// beyond the reserve. Called with the lock held.
static bool slot_admissible(swm_server *s) {
    if (s->slots.size() >= s->cfg.max_slots || s->no_slot_fits) return false;
    if (s->cfg.device_mem_limit && s->held_bytes + s->slot_bytes > s->cfg.device_mem_limit) return false;
    size_t fr = 0, total = 0;
    if (cudaMemGetInfo(&fr, &total) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return fr >= s->slot_bytes + s->cfg.device_mem_reserve;
}

// Split the block's packed records back per request (records are in read
// order, so each request's records are contiguous).
static void deliver(swm_server *s, Slot *sl, int status, const swm_packed_result &r) {
    const auto now = Clock::now();
    uint64_t wq = 0, cq = 0, q = 0, uq = 0;
    for (size_t i = 0; i < sl->reqs.size(); i++) {
        Request *rq = sl->reqs[i];
        const uint32_t lo = sl->offs[i], hi = lo + rq->n;
        rq->status = status;
        rq->t_done = now;
        rq->block_reads = sl->nreads;
        if (status == SWM_OK) {
            while (q < r.n_records) {
                const uint32_t cur = sl->h_words[wq];
                if ((cur >> 1) >= hi) break;
                const uint32_t nloc = sl->h_words[wq + 1] & 0x7fffffffu;
                rq->words.push_back(cur - 2 * lo);
                rq->words.insert(rq->words.end(), sl->h_words + wq + 1, sl->h_words + wq + 2 + nloc);
                const uint32_t cl = sl->h_rlen[q];
                rq->cigar.insert(rq->cigar.end(), sl->h_cigar + cq, sl->h_cigar + cq + cl);
                rq->rlen.push_back(cl);
                wq += 2 + nloc;
                cq += cl;
                q++;
            }
            while (uq < r.n_unmapped && (sl->h_unm[uq] >> 1) < hi) rq->unmapped.push_back(sl->h_unm[uq++] - 2 * lo);
        }
    }
    std::lock_guard<std::mutex> lk(s->mu);
    for (Request *rq : sl->reqs) {
        s->done.push_back(rq);
        s->st.requests_done++;
        s->st.reads_done += rq->n;
    }
    sl->reqs.clear();
    sl->offs.clear();
    sl->busy = false;
    s->cv_done.notify_all();
}

// Wait for a slot's block (its stream has drained) and hand out the results.
static void finish_slot(swm_server *s, Slot *sl) {
    swm_packed_result r;
    for (int attempt = 0; attempt < 4; attempt++) {
        memset(&r, 0, sizeof r);
        r.words = sl->h_words;
        r.cigar = sl->h_cigar;
        r.record_cigar_len = sl->h_rlen;
        r.unmapped = sl->h_unm;
        r.words_cap = sl->cap_words;
        r.cigar_cap = sl->cap_cigar;
        r.records_cap = sl->cap_recs;
        r.unmapped_cap = s->cfg.block_reads;
        int rc = attempt == 0 ? swm_map_wait_packed(sl->m, &r) : swm_map_fetch_packed(sl->m, &r);
        if (rc == SWM_ERR_OVERFLOW && r.n_unmapped <= r.unmapped_cap) {
            // more records than the staging holds: grow it and fetch again
            if (host_grow((void **)&sl->h_words, &sl->cap_words, r.n_words, 4) &&
                host_grow((void **)&sl->h_cigar, &sl->cap_cigar, r.n_cigar, 1) &&
                host_grow((void **)&sl->h_rlen, &sl->cap_recs, r.n_records, 4))
                continue;
            rc = SWM_ERR_OOM;
        }
        deliver(s, sl, rc, r);
        return;
    }
    deliver(s, sl, SWM_ERR_OOM, r);
}

// Coalesce waiting requests into slot sl's next block and queue it.
static void launch(swm_server *s, Slot *sl, std::vector<Request *> &take) {
    const uint64_t stride = s->cfg.stride;
    uint32_t n = 0, emax = 0;
    sl->offs.clear();
    for (Request *rq : take) {
        sl->offs.push_back(n);
        memcpy(sl->h_reads + (uint64_t)n * stride, rq->reads.data(), (uint64_t)rq->n * stride);
        memcpy(sl->h_lens + n, rq->lens.data(), rq->n * 4ull);
        memcpy(sl->h_e + n, rq->e.data(), rq->n);
        for (uint8_t v : rq->e) emax = v > emax ? v : emax;
        n += rq->n;
    }
    sl->reqs = take;
    sl->nreads = n;
    swm_batch b;
    b.reads = sl->h_reads;
    b.reads_len = sl->h_lens;
    b.stride = stride;
    b.reads_num = n;
    b.errors = emax;
    b.errors_per_read = sl->h_e;
    const int rc = swm_map_submit(sl->m, &b);
    if (rc != SWM_OK) {
        swm_packed_result r;
        memset(&r, 0, sizeof r);
        deliver(s, sl, rc, r);
        return;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.blocks++;
    uint32_t busy = 0;
    for (Slot *x : s->slots) busy += x->busy ? 1u : 0u;
    if (busy > s->st.max_blocks_in_flight) s->st.max_blocks_in_flight = busy;
}

static void engine_main(swm_server *s) {
    cudaSetDevice(s->ix->device);
    for (;;) {
        bool progressed = false;
        // 1. blocks whose streams have drained
        std::vector<Slot *> slots;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            slots = s->slots;
        }
        for (Slot *sl : slots) {
            if (!sl->busy) continue;
            const cudaError_t q = cudaStreamQuery((cudaStream_t)swm_mapper_stream(sl->m));
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) cudaGetLastError(); // the wait below reports the block's error
            finish_slot(s, sl);
            progressed = true;
        }
        // 2. waiting requests into free (or newly admitted) slots
        for (;;) {
            std::vector<Request *> take;
            Slot *sl = nullptr;
            {
                std::unique_lock<std::mutex> lk(s->mu);
                if (s->pending.empty()) break;
                for (Slot *x : s->slots)
                    if (!x->busy) {
                        sl = x;
                        break;
                    }
                if (!sl && slot_admissible(s)) {
                    lk.unlock();
                    Slot *ns = make_slot(s);
                    lk.lock();
                    if (ns) {
                        s->slots.push_back(ns);
                        s->held_bytes += s->slot_bytes;
                        s->st.slots = s->slots.size();
                        sl = ns;
                    } else if (s->slots.empty()) {
                        s->no_slot_fits = true;
                    }
                }
                if (!sl) break;
                uint64_t n = 0;
                while (!s->pending.empty() && n + s->pending.front()->n <= s->cfg.block_reads) {
                    Request *rq = s->pending.front();
                    s->pending.pop_front();
                    n += rq->n;
                    take.push_back(rq);
                }
                s->pending_reads -= n;
                sl->busy = true;
            }
            launch(s, sl, take);
            progressed = true;
        }
        {
            std::unique_lock<std::mutex> lk(s->mu);
            bool any_busy = false;
            for (Slot *x : s->slots) any_busy |= x->busy;
            if (s->stopping && s->pending.empty() && !any_busy) break;
            if (s->no_slot_fits && !s->pending.empty() && s->slots.empty()) {
                // nothing can ever run: refuse what is waiting
                while (!s->pending.empty()) {
                    Request *rq = s->pending.front();
                    s->pending.pop_front();
                    s->pending_reads -= rq->n;
                    rq->status = SWM_ERR_OOM;
                    rq->t_done = Clock::now();
                    s->done.push_back(rq);
                }
                s->cv_done.notify_all();
            }
            if (!progressed) {
                if (any_busy) { // poll the busy streams again shortly
                    lk.unlock();
                    std::this_thread::sleep_for(std::chrono::microseconds(20));
                } else {
                    s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
                }
            }
        }
    }
}

extern "C" int swm_serve_open(swm_index *ix, const swm_serve_config *cfg, swm_server **out) {
    if (!ix || !cfg || !out || cfg->block_reads == 0 || cfg->block_reads > (1u << 24) || cfg->max_slots == 0 ||
        cfg->stride == 0 || cfg->stride > 4096 || cfg->max_queued_reads < cfg->block_reads) {
        swm_set_error("swm_serve_open: block_reads in [1, 2^24], max_slots >= 1, stride in [1, 4096] and "
                      "max_queued_reads >= block_reads required");
        return SWM_ERR_ARG;
    }
    SWM_CUDA(cudaSetDevice(ix->device));
    swm_server *s = new swm_server();
    s->ix = ix;
    s->cfg = *cfg;
    // the first slot is made now, which also measures a slot's device memory;
    // it is released again when the caller's limit does not allow one
    Slot *first = make_slot(s);
    if (!first) {
        delete s;
        swm_set_error("swm_serve_open: not enough device memory for one block slot of %llu reads",
                      (unsigned long long)cfg->block_reads);
        return SWM_ERR_OOM;
    }
    if (cfg->device_mem_limit && s->slot_bytes > cfg->device_mem_limit) {
        free_slot(first);
        s->no_slot_fits = true;
    } else {
        s->slots.push_back(first);
        s->held_bytes = s->slot_bytes;
        s->st.slots = 1;
    }
    s->st.slot_bytes = s->slot_bytes;
    s->engine = std::thread(engine_main, s);
    *out = s;
    return SWM_OK;
}

extern "C" int swm_serve_submit(swm_server *s, const swm_batch *b, uint64_t *id) {
    if (!s || !b || !id || (!b->reads && b->reads_num) || (!b->reads_len && b->reads_num)) return SWM_ERR_ARG;
    if (b->reads_num == 0 || b->reads_num > s->cfg.block_reads) {
        swm_set_error("swm_serve_submit: a request holds 1 to block_reads (%llu) reads",
                      (unsigned long long)s->cfg.block_reads);
        return SWM_ERR_ARG;
    }
    if (b->errors > SWM_MAX_ERRORS) {
        swm_set_error("swm_serve_submit: errors must be <= %d", SWM_MAX_ERRORS);
        return SWM_ERR_ARG;
    }
    const uint64_t n = b->reads_num, sstride = s->cfg.stride;
    const uint32_t klong = s->ix->k + SWM_SEED_STEP - 1;
    for (uint64_t r = 0; r < n; r++) {
        const uint32_t L = b->reads_len[r];
        if (L > SWM_MAX_READ_LEN || L > b->stride || L > sstride || L / klong > 16 ||
            (b->errors_per_read && b->errors_per_read[r] > SWM_MAX_ERRORS)) {
            swm_set_error("swm_serve_submit: read %llu: length %u or threshold outside the envelope "
                          "(L <= %d, L <= the request and server strides, e <= %d)",
                          (unsigned long long)r, L, SWM_MAX_READ_LEN, SWM_MAX_ERRORS);
            return SWM_ERR_ARG;
        }
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) {
            swm_set_error("swm_serve_submit: the server is closing");
            return SWM_ERR_STATE;
        }
        if (s->no_slot_fits && s->slots.empty()) {
            s->st.refused_memory++;
            swm_set_error("swm_serve_submit: no block slot fits the device memory allowed (%llu bytes a slot, "
                          "limit %llu)", (unsigned long long)s->slot_bytes,
                          (unsigned long long)s->cfg.device_mem_limit);
            return SWM_ERR_OOM;
        }
        if (s->pending_reads + n > s->cfg.max_queued_reads) {
            s->st.refused_queue++;
            swm_set_error("swm_serve_submit: %llu reads already wait for a block slot (limit %llu)",
                          (unsigned long long)s->pending_reads, (unsigned long long)s->cfg.max_queued_reads);
            return SWM_ERR_STATE;
        }
    }
    Request *rq = new Request();
    rq->n = (uint32_t)n;
    rq->reads.assign(n * sstride, 0);
    for (uint64_t r = 0; r < n; r++)
        memcpy(rq->reads.data() + r * sstride, b->reads + r * b->stride, b->reads_len[r]);
    rq->lens.assign(b->reads_len, b->reads_len + n);
    if (b->errors_per_read) rq->e.assign(b->errors_per_read, b->errors_per_read + n);
    else rq->e.assign(n, (uint8_t)b->errors);
    rq->status = SWM_OK;
    rq->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        rq->id = s->next_id++;
        s->pending.push_back(rq);
        s->pending_reads += n;
        s->st.requests_admitted++;
    }
    s->cv_work.notify_one();
    *id = rq->id;
    return SWM_OK;
}

extern "C" int swm_serve_poll(swm_server *s, int timeout_ms, uint64_t *id, swm_packed_result *r,
                              swm_request_info *info) {
    if (!s || !id) return SWM_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto ready = [&] { return !s->done.empty(); };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return SWM_ERR_TIMEOUT;
    Request *rq = s->done.front();
    *id = rq->id;
    if (info) {
        info->id = rq->id;
        info->reads = rq->n;
        info->block_reads = rq->block_reads;
        info->latency_ms = std::chrono::duration<double, std::milli>(rq->t_done - rq->t_submit).count();
    }
    if (rq->status != SWM_OK) {
        const int st = rq->status;
        s->done.pop_front();
        delete rq;
        swm_set_error("request %llu failed (%d)", (unsigned long long)*id, st);
        return st;
    }
    if (r) {
        r->n_words = rq->words.size();
        r->n_cigar = rq->cigar.size();
        r->n_records = rq->rlen.size();
        r->n_unmapped = rq->unmapped.size();
        if (r->n_words > r->words_cap || r->n_cigar > r->cigar_cap || r->n_records > r->records_cap ||
            r->n_unmapped > r->unmapped_cap || (r->n_words && !r->words) || (r->n_cigar && !r->cigar) ||
            (r->n_unmapped && !r->unmapped)) {
            swm_set_error("request %llu: result buffers too small (words %llu, bytes %llu, records %llu, "
                          "unmapped %llu); the result stays first in line",
                          (unsigned long long)*id, (unsigned long long)r->n_words, (unsigned long long)r->n_cigar,
                          (unsigned long long)r->n_records, (unsigned long long)r->n_unmapped);
            return SWM_ERR_OVERFLOW;
        }
        if (r->n_words) memcpy(r->words, rq->words.data(), r->n_words * 4);
        if (r->n_cigar) memcpy(r->cigar, rq->cigar.data(), r->n_cigar);
        if (r->n_records && r->record_cigar_len) memcpy(r->record_cigar_len, rq->rlen.data(), r->n_records * 4);
        if (r->n_unmapped) memcpy(r->unmapped, rq->unmapped.data(), r->n_unmapped * 4);
    }
    s->done.pop_front();
    delete rq;
    return SWM_OK;
}

extern "C" int swm_serve_stats(swm_server *s, swm_serve_counters *out) {
    if (!s || !out) return SWM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->queued_reads = s->pending_reads;
    return SWM_OK;
}

extern "C" int swm_serve_close(swm_server *s) {
    if (!s) return SWM_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    if (s->engine.joinable()) s->engine.join();
    for (Slot *sl : s->slots) free_slot(sl);
    for (Request *rq : s->pending) delete rq;
    for (Request *rq : s->done) delete rq;
    delete s;
    return SWM_OK;
}
