// Request server: compress (forward BWT) and decompress (inverse BWT) requests on host buffers, batched as they arrive
// and run by `slots` workers, each with its own engines and stream, so that batches of different workers overlap on
// the device. Continuous batching: a worker that finishes takes the next batch at once from whatever is pending (the
// oldest request's kind, then every later pending request of that kind in arrival order while the batch fits). A
// batch is admitted only while the device bytes of all workers stay within the HBM budget; workers keep their
// buffers resident between batches and give them back when another batch could not be admitted otherwise.
//
// The reference has no server: its block workers call the sorter directly (src/core/blocks.c:181, pool.c:74). The
// requests run through the same worker code as the drop-in calls (run_fwd_jobs / run_inv_jobs), so a request's
// result does not depend on what else is in its batch.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "worker.cuh"

namespace kgb {

static double now_us() {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device bytes one worker holds after running a batch of `count` requests of `kind` with lengths n[] (and sampling
// intervals r[], forward only), given the workspaces it already holds (engines only grow).
static u64 batch_bytes(int kind, const int32_t *n, const int32_t *r, int count, u64 have_fwd, u64 have_inv) {
    if (count <= 0) return have_fwd + have_inv;
    std::vector<u32> nn;
    u64 total = 0, samples = 0;
    for (int i = 0; i < count; i++) {
        if (n[i] < 2) continue;  // handled on the host
        nn.push_back((u32)n[i]);
        total += ((u64)n[i] + 15) / 16 * 16;
        samples += kind == KGBWT_REQ_FWD && r && r[i] > 0 ? (u64)(n[i] - 1) / (u64)r[i] + 1 : 1;
    }
    if (nn.empty()) return have_fwd + have_inv;
    if (kind == KGBWT_REQ_FWD) {
        FwdEngine e;
        return std::max(have_fwd, e.estimate_bytes(total, (u32)nn.size(), (u32)std::min<u64>(samples, 0xFFFFFFFFu))) +
               have_inv;
    }
    InvEngine e;
    return have_fwd + std::max(have_inv, e.estimate_bytes(nn.data(), (int)nn.size()));
}

// The batching policy (pure host logic, shared with kgbwt_server_plan): from the pending requests in arrival order,
// the oldest one's kind and then every later request of that kind, in order, while the worker's bytes after the batch
// stay within `avail` and the batch's input bytes within max_batch_bytes (the first request is exempt from the
// latter). Stops at the first request of the kind that does not fit, so requests of one kind keep their order.
// Returns the number taken (their indexes in take[]); 0 when the oldest request does not fit in `avail`.
static int plan_batch(const int32_t *kinds, const int32_t *n, const int32_t *r, int count, u64 have_fwd,
                      u64 have_inv, u64 avail, u64 max_batch_bytes, int32_t *take) {
    if (count <= 0) return 0;
    const int kind = kinds[0];
    std::vector<int32_t> bn, br;
    u64 bytes = 0;
    int k = 0;
    for (int i = 0; i < count; i++) {
        if (kinds[i] != kind) continue;
        const u64 nb = n[i] > 0 ? (u64)n[i] : 0;
        if (k > 0 && bytes + nb > max_batch_bytes) break;
        bn.push_back(n[i]);
        br.push_back(r ? r[i] : 0);
        if (batch_bytes(kind, bn.data(), br.data(), (int)bn.size(), have_fwd, have_inv) > avail) break;
        take[k++] = i;
        bytes += nb;
    }
    return k;
}

struct ServReq {
    int64_t id;
    int kind;
    const u8 *in;
    u8 *out;
    int32_t *idx;
    int32_t n, r;
    int rc = 0;
    int state = 0;  // 0 pending, 1 running, 2 done
    double t_submit = 0, t_done = 0;
};

struct Slot {
    Worker w;
    std::thread th;
    bool busy = false;
    u64 resident = 0;  // device bytes held (admission counts max(resident, reservation) while busy)
    u64 reserved = 0;
};

}  // namespace kgb

struct kgbwt_server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<kgb::ServReq *> pending;
    std::unordered_map<int64_t, kgb::ServReq *> reqs;
    std::vector<kgb::Slot *> slots;
    int64_t next_id = 0;
    bool stop = false;
    int device = -1;
    uint64_t budget = 0, max_batch = 0;
    int inject_oom = 0;
    kgbwt_server_stats st{};
};

namespace kgb {

static u64 held_by_others(kgbwt_server *S, const Slot *self) {
    u64 t = 0;
    for (const Slot *o : S->slots)
        if (o != self) t += o->busy ? std::max(o->resident, o->reserved) : o->resident;
    return t;
}

static void note_memory(kgbwt_server *S) {
    u64 t = 0;
    for (const Slot *o : S->slots) t += o->busy ? std::max(o->resident, o->reserved) : o->resident;
    S->st.hbm_in_use = t;
    S->st.hbm_peak = std::max<uint64_t>(S->st.hbm_peak, t);
}

static void finish(kgbwt_server *S, ServReq *q, int rc) {
    q->rc = rc;
    q->state = 2;
    q->t_done = now_us();
    if (rc == 0) { S->st.completed++; S->st.bytes += (u64)(q->n > 0 ? q->n : 0); }
    else if (rc == -3) S->st.cancelled++;
    else S->st.failed++;
}

static void slot_main(kgbwt_server *S, Slot *sl) {
    if (S->device >= 0) cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
        if (S->stop) break;
        // plan a batch from the pending requests
        const int np = (int)S->pending.size();
        std::vector<int32_t> kinds(np), ns(np), rs(np), take(np);
        for (int i = 0; i < np; i++) { kinds[i] = S->pending[i]->kind; ns[i] = S->pending[i]->n; rs[i] = S->pending[i]->r; }
        const u64 have_f = sl->w.eng.fwd.workspace_bytes(), have_i = sl->w.eng.inv.workspace_bytes();
        const u64 others = held_by_others(S, sl);
        const u64 avail = S->budget ? (S->budget > others ? S->budget - others : 0) : ~0ull;
        int k = plan_batch(kinds.data(), ns.data(), rs.data(), np, have_f, have_i, avail, S->max_batch, take.data());
        if (k == 0) {
            ServReq *first = S->pending.front();
            // could it run on an empty device at all?
            const u64 alone = batch_bytes(first->kind, &first->n, &first->r, 1, 0, 0);
            if (S->budget && alone > S->budget) {
                S->pending.pop_front();
                kgb::record_error("server: request needs more device memory than the HBM budget");
                finish(S, first, -2);
                S->cv_done.notify_all();
                continue;
            }
            bool others_busy = false;
            for (Slot *o : S->slots) others_busy |= (o != sl && o->busy);
            if (others_busy) {  // memory comes back when they finish
                S->cv_work.wait(lk);
                continue;
            }
            // everyone else is idle: take back idle workers' resident buffers, then this worker's own
            bool freed = false;
            for (Slot *o : S->slots)
                if (o != sl && !o->busy && o->resident) { o->w.release(); o->resident = 0; freed = true; }
            if (!freed && (have_f || have_i)) { sl->w.release(); sl->resident = 0; freed = true; }
            note_memory(S);
            if (!freed) {  // nothing left to free and it still does not fit: give up on this request
                S->pending.pop_front();
                kgb::record_error("server: request does not fit the HBM budget");
                finish(S, first, -2);
                S->cv_done.notify_all();
            }
            continue;
        }
        std::vector<ServReq *> batch(k);
        for (int i = 0; i < k; i++) batch[i] = S->pending[take[i]];
        {
            std::vector<bool> gone(np, false);
            for (int i = 0; i < k; i++) gone[take[i]] = true;
            std::deque<ServReq *> rest;
            for (int i = 0; i < np; i++) if (!gone[i]) rest.push_back(S->pending[i]);
            S->pending.swap(rest);
        }
        for (ServReq *q : batch) q->state = 1;
        std::vector<int32_t> bn(k), br(k);
        for (int i = 0; i < k; i++) { bn[i] = batch[i]->n; br[i] = batch[i]->r; }
        sl->reserved = batch_bytes(batch[0]->kind, bn.data(), br.data(), k, have_f, have_i);
        sl->busy = true;
        note_memory(S);
        const bool inject = S->inject_oom > 0;
        if (inject) S->inject_oom--;
        S->st.batches++;
        lk.unlock();
        // ---- run the batch on this worker (no lock held)
        std::vector<int> rcs(k, 0);
        if (inject) {  // test hook: this batch's device allocation fails
            kgb::record_error("server: injected device allocation failure");
            std::fill(rcs.begin(), rcs.end(), -2);
        } else if (batch[0]->kind == KGBWT_REQ_FWD) {
            std::vector<kgbwt_fwd_job> jobs(k);
            for (int i = 0; i < k; i++) jobs[i] = {batch[i]->in, batch[i]->out, batch[i]->n, batch[i]->r, batch[i]->idx, 0};
            int rc = run_fwd_jobs(sl->w, jobs.data(), k, 0);
            for (int i = 0; i < k; i++) rcs[i] = jobs[i].rc ? jobs[i].rc : rc;
        } else {
            std::vector<kgbwt_inv_job> jobs(k);
            for (int i = 0; i < k; i++) jobs[i] = {batch[i]->in, batch[i]->out, batch[i]->n, batch[i]->r, batch[i]->idx, 0};
            int rc = run_inv_jobs(sl->w, jobs.data(), k, 0);
            for (int i = 0; i < k; i++) rcs[i] = jobs[i].rc ? jobs[i].rc : (rc == -2 ? rc : 0);
        }
        lk.lock();
        sl->busy = false;
        sl->reserved = 0;
        sl->resident = sl->w.device_bytes();
        note_memory(S);
        for (int i = 0; i < k; i++) finish(S, batch[i], rcs[i]);
        S->cv_done.notify_all();
        S->cv_work.notify_all();  // memory came back: workers waiting for room may plan again
    }
}

}  // namespace kgb

using namespace kgb;

extern "C" {

kgbwt_server *kgbwt_server_create(int32_t slots, uint64_t hbm_budget, uint64_t max_batch_bytes) {
    if (slots < 1 || slots > 16) return nullptr;
    kgbwt_server *S = new (std::nothrow) kgbwt_server();
    if (!S) return nullptr;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); dev = -1; }
    S->device = dev;
    S->budget = hbm_budget;
    S->max_batch = max_batch_bytes ? max_batch_bytes : (1ull << 30);
    for (int i = 0; i < slots; i++) S->slots.push_back(new Slot());
    for (Slot *sl : S->slots) sl->th = std::thread(slot_main, S, sl);
    return S;
}

void kgbwt_server_destroy(kgbwt_server *S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        for (ServReq *q : S->pending) finish(S, q, -3);
        S->pending.clear();
    }
    S->cv_work.notify_all();
    for (Slot *sl : S->slots) if (sl->th.joinable()) sl->th.join();
    for (Slot *sl : S->slots) delete sl;
    for (auto &kv : S->reqs) delete kv.second;
    S->cv_done.notify_all();
    delete S;
}

int64_t kgbwt_server_submit(kgbwt_server *S, int32_t kind, const uint8_t *in, uint8_t *out, int32_t *idx, int32_t n,
                            int32_t r) {
    if (!S || !in || !out || !idx || n < 0 || (kind != KGBWT_REQ_FWD && kind != KGBWT_REQ_INV)) return -1;
    if (kind == KGBWT_REQ_FWD && bad_r(r)) return -1;
    if (kind == KGBWT_REQ_INV && r != n && bad_r(r)) return -1;
    ServReq *q = new (std::nothrow) ServReq();
    if (!q) return -1;
    q->kind = kind; q->in = in; q->out = out; q->idx = idx; q->n = n; q->r = r;
    q->t_submit = now_us();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) { delete q; return -1; }
        q->id = S->next_id++;
        S->reqs[q->id] = q;
        S->pending.push_back(q);
        S->st.submitted++;
    }
    S->cv_work.notify_one();
    return q->id;
}

int32_t kgbwt_server_wait(kgbwt_server *S, int64_t id, int32_t timeout_ms, int32_t *rc, double *latency_us) {
    if (!S) return -1;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return -1;
    ServReq *q = it->second;
    auto done = [&] { return q->state == 2; };
    if (timeout_ms < 0) S->cv_done.wait(lk, done);
    else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return 0;
    if (rc) *rc = q->rc;
    if (latency_us) *latency_us = q->t_done - q->t_submit;
    S->reqs.erase(it);
    delete q;
    return 1;
}

int32_t kgbwt_server_cancel(kgbwt_server *S, int64_t id) {
    if (!S) return -1;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = std::find_if(S->pending.begin(), S->pending.end(), [&](const ServReq *q) { return q->id == id; });
    if (it == S->pending.end()) return -1;
    ServReq *q = *it;
    S->pending.erase(it);
    finish(S, q, -3);
    S->cv_done.notify_all();
    return 0;
}

int32_t kgbwt_server_stats_read(kgbwt_server *S, kgbwt_server_stats *out) {
    if (!S || !out) return -1;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->st;
    return 0;
}

int32_t kgbwt_server_inject_oom(kgbwt_server *S, int32_t batches) {
    if (!S || batches < 0) return -1;
    std::lock_guard<std::mutex> lk(S->mu);
    S->inject_oom = batches;
    return 0;
}

int32_t kgbwt_server_plan(const int32_t *kinds, const int32_t *n, const int32_t *r, int32_t count, uint64_t have_fwd,
                          uint64_t have_inv, uint64_t avail, uint64_t max_batch_bytes, int32_t *take) {
    if (!kinds || !n || !take || count < 0) return -1;
    return plan_batch(kinds, n, r, count, have_fwd, have_inv, avail, max_batch_bytes ? max_batch_bytes : (1ull << 30),
                      take);
}

uint64_t kgbwt_estimate_bytes(int32_t kind, const int32_t *n, const int32_t *r, int32_t count) {
    if (!n || count < 0 || (kind != KGBWT_REQ_FWD && kind != KGBWT_REQ_INV)) return 0;
    return batch_bytes(kind, n, r, count, 0, 0);
}

}  // extern "C"

// ---- libcubwt's entry points (include/kgbwt_cubwt.h): a storage is one worker
#include "kgbwt_cubwt.h"

namespace kgb {
struct CubwtStorage {
    unsigned magic = 0x6B637762u;
    std::mutex mu;
    Worker w;
};
static CubwtStorage *cubwt_of(void *p) {
    CubwtStorage *s = static_cast<CubwtStorage *>(p);
    return s && s->magic == 0x6B637762u ? s : nullptr;
}
static int64_t cubwt_code(int rc) {
    return rc == 0 ? KGBWT_CUBWT_NO_ERROR
           : rc == -1 ? KGBWT_CUBWT_BAD_PARAMETER
           : rc == -2 ? KGBWT_CUBWT_NOT_ENOUGH_MEMORY
                      : KGBWT_CUBWT_GPU_ERROR;
}
}  // namespace kgb

extern "C" {

int64_t libcubwt_allocate_device_storage(void **device_storage, int64_t max_length) {
    if (!device_storage || max_length < 0 || max_length > ((int64_t)1 << 30)) return KGBWT_CUBWT_BAD_PARAMETER;
    CubwtStorage *s = new (std::nothrow) CubwtStorage();
    if (!s) return KGBWT_CUBWT_NOT_ENOUGH_MEMORY;
    *device_storage = s;  // the device workspace grows on the first call that needs it
    return KGBWT_CUBWT_NO_ERROR;
}

int64_t libcubwt_free_device_storage(void *device_storage) {
    CubwtStorage *s = cubwt_of(device_storage);
    if (!s) return KGBWT_CUBWT_BAD_PARAMETER;
    s->magic = 0;
    delete s;
    return KGBWT_CUBWT_NO_ERROR;
}

int64_t libcubwt_bwt_aux(void *device_storage, const uint8_t *T, uint8_t *L, int64_t n, int64_t r, uint32_t *I) {
    CubwtStorage *s = cubwt_of(device_storage);
    if (!s || !T || !L || !I || n < 2 || n > ((int64_t)1 << 30) || r < 2 || r > n || bad_r((int32_t)r))
        return KGBWT_CUBWT_BAD_PARAMETER;
    std::lock_guard<std::mutex> lock(s->mu);
    kgbwt_fwd_job j = {T, L, (int32_t)n, (int32_t)r, reinterpret_cast<int32_t *>(I), 0};
    const int rc = run_fwd_jobs(s->w, &j, 1, 0);
    return cubwt_code(rc ? rc : j.rc);
}

int64_t libcubwt_bwt(void *device_storage, const uint8_t *T, uint8_t *L, int64_t n) {
    CubwtStorage *s = cubwt_of(device_storage);
    if (!s || !T || !L || n < 2 || n > ((int64_t)1 << 30)) return KGBWT_CUBWT_BAD_PARAMETER;
    std::lock_guard<std::mutex> lock(s->mu);
    // the smallest power of two >= n as the sampling interval: only the primary index is sampled
    int32_t r = 2;
    while ((int64_t)r < n) r <<= 1;
    int32_t idx = 0;
    kgbwt_fwd_job j = {T, L, (int32_t)n, r, &idx, 0};
    const int rc = run_fwd_jobs(s->w, &j, 1, 0);
    const int code = rc ? rc : j.rc;
    return code ? cubwt_code(code) : (int64_t)idx;
}

int64_t libcubwt_unbwt(void *device_storage, const uint8_t *T, uint8_t *U, int64_t n, const int32_t *freq, int32_t i) {
    (void)freq;
    CubwtStorage *s = cubwt_of(device_storage);
    if (!s || !T || !U || n < 2 || n > ((int64_t)1 << 30) || i < 1 || i > n) return KGBWT_CUBWT_BAD_PARAMETER;
    std::lock_guard<std::mutex> lock(s->mu);
    kgbwt_inv_job j = {T, U, (int32_t)n, (int32_t)n, &i, 0};
    const int rc = run_inv_jobs(s->w, &j, 1, 0);
    const int code = j.rc ? j.rc : rc;
    return code == -1 ? KGBWT_CUBWT_GPU_ERROR : cubwt_code(code);  // -1 here: not a valid BWT
}

}  // extern "C"
