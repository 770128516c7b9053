// C ABI of the GB300 block-sorting engine: the reference's suffix-sorter entry points (drop-in), batch calls and
// device-buffer engines. See include/kgbwt.h for the contract of every function.
#include "kgbwt.h"

#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "worker.cuh"

namespace kgb {

static thread_local char g_err[512];

const char *kernel_name(int k) {
    static const char *names[K_NKERNELS] = {
        "init", "fixup", "keygen", "msd_hist", "msd_scan", "msd_scatter", "tile_sort_prefix", "tile_sort_prefix_keyed",
        "tile_sort_rank", "tile_sort_rank_keyed", "control", "samples",
        "tile_warp_prefix", "tile_warp_prefix_keyed", "tile_warp_rank", "tile_warp_rank_keyed",
        "lsd_begin", "lsd_key0", "lsd_hist", "lsd_pass", "seg_count", "seg_scan", "seg_emit1", "seg_emit2",
        "group_thread", "group_warp", "mkeys", "lsd_ident", "seg_rank",
        "inv_chunkhist", "inv_chunkscan", "inv_scatter", "inv_walk", "inv_rank_init", "inv_jump", "inv_emit", "chain"};
    return k >= 0 && k < K_NKERNELS ? names[k] : "?";
}

void record_error(const char *msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

int record_cuda_error(cudaError_t e, const char *what, const char *file, int line) {
    const char *f = strrchr(file, '/');
    snprintf(g_err, sizeof g_err, "%s: %s (%s:%d)", what, cudaGetErrorString(e), f ? f + 1 : file, line);
    return -2;
}

int Pinned::need(size_t bytes) {
    if (bytes <= cap) return 0;
    release();
    size_t want = bytes + bytes / 4 + 4096;
    KGB_CHECK(cudaMallocHost(&p, want));
    cap = want;
    return 0;
}
void Pinned::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
}

int Worker::init() {
    if (stream) return 0;
    KGB_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    return 0;
}
void Worker::release() {
    eng.fwd.~FwdEngine();
    new (&eng.fwd) FwdEngine();
    eng.inv.~InvEngine();
    new (&eng.inv) InvEngine();
    stage_L.release();
    stage_I.release();
}
Worker::~Worker() {
    if (stream) cudaStreamDestroy(stream);
}

// One drop-in or batch call waiting for the default worker.
struct Pending {
    int kind;           // 0 forward, 1 inverse
    void *jobs;         // kgbwt_fwd_job[count] or kgbwt_inv_job[count]
    int32_t count;
    uint32_t flags;
    u64 bytes;          // input bytes of the call's jobs
    int rc = 0;         // the device-level return code of the batch that carried the call
    bool done = false;
    char err[256] = {0};
};

// The default worker of the drop-in and batch calls. Concurrent callers (the reference's block workers call the
// sorter from one thread per block, src/core/blocks.c:181, src/core/compress.c:221) are coalesced: the first caller
// to find the worker idle runs the oldest pending call together with every later pending call of the same kind, in
// arrival order, while their input stays within the batch cap; the others wait for their results.
struct Context {
    std::mutex mu;  // guards the queue, `busy` and the counters; the worker itself belongs to the running leader
    std::condition_variable cv;
    std::deque<Pending *> q;
    bool busy = false;
    Worker w;
    int64_t calls[2] = {0, 0}, batches[2] = {0, 0}, largest[2] = {0, 0}, retried = 0;
};
static Context &ctx() {
    static Context *c = new Context();  // never destroyed: callers may run at process exit
    return *c;
}

// Input bytes per coalesced batch: KGBWT_BATCH_MIB (default 256 MiB, about 32 GB of forward workspace).
static u64 batch_cap() {
    static u64 cap = 0;
    if (!cap) {
        const char *e = getenv("KGBWT_BATCH_MIB");
        const long v = e ? atol(e) : 0;
        cap = (u64)(v > 0 ? v : 256) << 20;
    }
    return cap;
}

bool bad_r(int32_t r) { return r < 2 || (r & (r - 1)) != 0; }

// Host memory the device can copy into directly (cudaMallocHost / cudaHostRegister): true when the runtime reports a
// host (page-locked) or managed allocation at p.
static bool page_locked(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged;
}

// KGBWT_PLAIN=1 in the environment makes the drop-in and batch calls use the plain path (debugging aid).
static uint32_t env_flags() {
    static int plain = -1;
    if (plain < 0) { const char *e = getenv("KGBWT_PLAIN"); plain = e && e[0] == '1'; }
    return plain ? KGBWT_PLAIN : 0u;
}

int run_fwd_jobs(Worker &C, kgbwt_fwd_job *jobs, int32_t count, uint32_t flags) {
    std::vector<int> dev;
    std::vector<u32> n, r;
    for (int i = 0; i < count; i++) {
        kgbwt_fwd_job &j = jobs[i];
        if (!j.T || !j.U || !j.I || j.n < 0 || bad_r(j.r)) { j.rc = -1; continue; }
        if (j.n <= 1) {
            if (j.n == 1) j.U[0] = j.T[0];
            j.I[0] = j.n;
            j.rc = 0;
            continue;
        }
        j.rc = 0;
        dev.push_back(i);
        n.push_back((u32)j.n);
        r.push_back((u32)j.r);
    }
    if (dev.empty()) return 0;  // argument errors and n <= 1 never touch the device
    if (int rc = C.init()) { for (int i : dev) jobs[i].rc = rc; return rc; }
    FwdEngine &E = C.eng.fwd;
    int rc = E.plan(n.data(), r.data(), (int)dev.size(), false);
    if (rc) { for (int i : dev) jobs[i].rc = rc; return rc; }
    cudaStream_t s = C.stream;
    auto fail = [&](int code) { for (int i : dev) jobs[i].rc = code; return code; };
    for (size_t k = 0; k < dev.size(); k++) {
        if (cudaMemcpyAsync(E.text() + E.offsets()[k], jobs[dev[k]].T, n[k], cudaMemcpyHostToDevice, s) != cudaSuccess)
            return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(text)", __FILE__, __LINE__));
    }
    if (cudaMemsetAsync(E.text() + E.total(), 0, 64, s) != cudaSuccess)
        return fail(record_cuda_error(cudaGetLastError(), "cudaMemsetAsync", __FILE__, __LINE__));
    if ((rc = E.run(s, !(flags & KGBWT_PLAIN)))) return fail(rc);
    // sampled indexes first (small); then each block's L column without its sentinel row: straight into the
    // caller's U when every U is page-locked (two device-to-host copies per block), else through one copy into pinned
    // staging and host copies (device-to-host copies into pageable memory are staged by the CUDA driver, block by block)
    bool direct = true;
    for (size_t k = 0; k < dev.size() && direct; k++) direct = page_locked(jobs[dev[k]].U);
    if (!direct) {
        const size_t lbytes = E.total() + dev.size();
        if ((rc = C.stage_L.need(lbytes))) return fail(rc);
        if (cudaMemcpyAsync(C.stage_L.p, E.lcol(), lbytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(L)", __FILE__, __LINE__));
    }
    if ((rc = C.stage_I.need((size_t)E.samples() * 4))) return fail(rc);
    if (cudaMemcpyAsync(C.stage_I.p, E.samples_dev(), (size_t)E.samples() * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(samples)", __FILE__, __LINE__));
    u32 err = 0;
    if ((rc = E.error_flag(s, &err))) return fail(rc);
    if (err) {
        char m[96];
        snprintf(m, sizeof m, "forward sort: device error bits 0x%x (internal error)", err);
        record_error(m);
        return fail(-2);
    }
    const u32 *I = reinterpret_cast<const u32 *>(C.stage_I.p);
    for (size_t k = 0; k < dev.size() && !direct; k++) {
        kgbwt_fwd_job &j = jobs[dev[k]];
        const u8 *L = C.stage_L.p + E.offsets()[k] + k;
        const u32 p0 = I[E.iouts()[k]];
        if (p0 < 1 || p0 > (u32)j.n) return fail(-2);
        memcpy(j.U, L, p0);
        memcpy(j.U + p0, L + p0 + 1, (size_t)j.n - p0);
    }
    for (size_t k = 0; k < dev.size() && direct; k++) {
        kgbwt_fwd_job &j = jobs[dev[k]];
        const u8 *L = E.lcol() + E.offsets()[k] + k;
        const u32 p0 = I[E.iouts()[k]];
        if (p0 < 1 || p0 > (u32)j.n) return fail(-2);
        if ((p0 && cudaMemcpyAsync(j.U, L, p0, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
            ((u32)j.n > p0 && cudaMemcpyAsync(j.U + p0, L + p0 + 1, (size_t)j.n - p0, cudaMemcpyDeviceToHost, s) !=
                                 cudaSuccess))
            return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(result)", __FILE__, __LINE__));
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
        return fail(record_cuda_error(cudaGetLastError(), "cudaStreamSynchronize", __FILE__, __LINE__));
    for (size_t k = 0; k < dev.size(); k++) {
        kgbwt_fwd_job &j = jobs[dev[k]];
        const u32 *Ib = I + E.iouts()[k];
        const u32 ns = (u32)((j.n - 1) / j.r + 1);
        for (u32 t = 0; t < ns; t++) j.I[t] = (int32_t)Ib[t];
    }
    return 0;
}

int run_inv_jobs(Worker &C, kgbwt_inv_job *jobs, int32_t count, uint32_t flags) {
    std::vector<int> dev;
    std::vector<u32> n, p0;
    for (int i = 0; i < count; i++) {
        kgbwt_inv_job &j = jobs[i];
        if (!j.T || !j.U || !j.I || j.n < 0 || ((j.r != j.n) && bad_r(j.r))) { j.rc = -1; continue; }
        if (j.n <= 1) {
            if (j.I[0] != j.n) { j.rc = -1; continue; }
            if (j.n == 1) j.U[0] = j.T[0];
            j.rc = 0;
            continue;
        }
        bool ok = true;
        for (int32_t t = 0; t <= (j.n - 1) / j.r; t++)
            if (j.I[t] <= 0 || j.I[t] > j.n) { ok = false; break; }
        if (!ok) { j.rc = -1; continue; }
        j.rc = 0;
        dev.push_back(i);
        n.push_back((u32)j.n);
        p0.push_back((u32)j.I[0]);
    }
    if (dev.empty()) return 0;
    if (int rc = C.init()) { for (int i : dev) jobs[i].rc = rc; return rc; }
    InvEngine &E = C.eng.inv;
    int rc = E.plan(n.data(), p0.data(), (int)dev.size());
    auto fail = [&](int code) { for (int i : dev) jobs[i].rc = code; return code; };
    if (rc) return fail(rc);
    cudaStream_t s = C.stream;
    for (size_t k = 0; k < dev.size(); k++)
        if (cudaMemcpyAsync(E.input() + E.offsets()[k], jobs[dev[k]].T, n[k], cudaMemcpyHostToDevice, s) != cudaSuccess)
            return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(bwt)", __FILE__, __LINE__));
    if ((rc = E.run(s, !(flags & KGBWT_PLAIN)))) return fail(rc);
    // the decoded texts: straight into the callers' buffers when all are page-locked, else through pinned staging
    bool direct = true;
    for (size_t k = 0; k < dev.size() && direct; k++) direct = page_locked(jobs[dev[k]].U);
    if (!direct) {
        if ((rc = C.stage_L.need(E.total()))) return fail(rc);
        if (cudaMemcpyAsync(C.stage_L.p, E.output(), E.total(), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(text)", __FILE__, __LINE__));
    }
    std::vector<int> st;
    if ((rc = E.fetch_status(s, st))) return fail(rc);
    int first = 0;
    for (size_t k = 0; k < dev.size(); k++) {
        kgbwt_inv_job &j = jobs[dev[k]];
        if (st[k]) {
            j.rc = -1;
            if (!first) { first = -1; record_error("inverse BWT: not a valid BWT string for its primary index"); }
            continue;
        }
        if (!direct) {
            memcpy(j.U, C.stage_L.p + E.offsets()[k], (size_t)j.n);
            continue;
        }
        if (cudaMemcpyAsync(j.U, E.output() + E.offsets()[k], (size_t)j.n, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return fail(record_cuda_error(cudaGetLastError(), "cudaMemcpyAsync(text)", __FILE__, __LINE__));
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
        return fail(record_cuda_error(cudaGetLastError(), "cudaStreamSynchronize", __FILE__, __LINE__));
    return first;
}

// ---- tuning table: configurations by batch size, written by kolmo_gb300/autotune.py as JSON
// {"buckets": [{"max_bytes": B, "tile_ctas": ..., "msd_ctas": ..., "small_group": ..., "warp_path": ...,
// "lsd_round0": ..., "lsd_bytes": ...}, ...]}; a batch of n bytes takes the first bucket with n <= max_bytes (else the last).
struct TuneBucket {
    u64 max_bytes;
    FwdConfig c;
};
static std::mutex g_tune_mu;
static std::vector<TuneBucket> g_tune;
static bool g_tune_tried = false;

static const char *skip_ws(const char *p) {
    while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') p++;
    return p;
}

// Parses the bucket objects of a tuning file. Returns the number of buckets, or -1 when the text is not a tuning
// table (no "buckets" array, a bucket without max_bytes, or a value out of range).
static int parse_tuning(const char *text, std::vector<TuneBucket> &out) {
    out.clear();
    const char *p = strstr(text, "\"buckets\"");
    if (!p) return -1;
    p = strchr(p, '[');
    if (!p) return -1;
    p++;
    for (;;) {
        p = skip_ws(p);
        if (*p == ',') { p++; continue; }
        if (*p == ']') break;
        if (*p != '{') return -1;
        p++;
        TuneBucket b{0, FwdConfig()};
        bool have_max = false;
        for (;;) {
            p = skip_ws(p);
            if (*p == ',') { p++; continue; }
            if (*p == '}') { p++; break; }
            if (*p != '"') return -1;
            const char *k0 = ++p;
            while (*p && *p != '"') p++;
            if (!*p) return -1;
            std::string key(k0, p - k0);
            p = skip_ws(p + 1);
            if (*p != ':') return -1;
            p = skip_ws(p + 1);
            if (*p == '"') {  // string value (a note): skip
                p++;
                while (*p && *p != '"') p++;
                if (!*p) return -1;
                p++;
                continue;
            }
            char *e = nullptr;
            const double v = strtod(p, &e);
            if (e == p) return -1;
            p = e;
            if (key == "max_bytes") { if (v < 0) return -1; b.max_bytes = (u64)v; have_max = true; }
            else if (key == "tile_ctas") { if (v < 1 || v > 8) return -1; b.c.tile_ctas = (int)v; }
            else if (key == "msd_ctas") { if (v < 1 || v > 16) return -1; b.c.msd_ctas = (int)v; }
            else if (key == "small_group") { if (v < 0 || v > 1024) return -1; b.c.small_group = (int)v; }
            else if (key == "warp_path") { if (v != 0 && v != 1) return -1; b.c.warp_path = (int)v; }
            else if (key == "lsd_round0") { if (v != 0 && v != 1) return -1; b.c.lsd_round0 = (int)v; }
            else if (key == "lsd_bytes") { if (v != 8 && v != 12 && v != 16) return -1; b.c.lsd_bytes = (int)v; }
            else if (key == "chain_from") { if (v < 0 || v > 64) return -1; b.c.chain_from = (int)v; }
        }
        if (!have_max) return -1;
        out.push_back(b);
    }
    std::sort(out.begin(), out.end(), [](const TuneBucket &a, const TuneBucket &b) { return a.max_bytes < b.max_bytes; });
    return (int)out.size();
}

static int load_tuning_file(const char *path, std::vector<TuneBucket> &out) {
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    std::string text;
    char buf[4096];
    size_t k;
    while ((k = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
    fclose(f);
    return parse_tuning(text.c_str(), out);
}

// First use: KGBWT_TUNING=<path> (or "off"), else the table shipped beside the package (../tuning_gb300.json
// relative to this library's directory), else none.
static void tune_autoload() {
    if (g_tune_tried) return;
    g_tune_tried = true;
    const char *env = getenv("KGBWT_TUNING");
    if (env && !strcmp(env, "off")) return;
    if (env && *env) { if (load_tuning_file(env, g_tune) < 0) g_tune.clear(); return; }
    Dl_info info;
    if (dladdr((void *)&kgbwt_version, &info) && info.dli_fname) {
        std::string p(info.dli_fname);
        const size_t slash = p.rfind('/');
        p = (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/../tuning_gb300.json";
        if (load_tuning_file(p.c_str(), g_tune) < 0) g_tune.clear();
    }
}

bool tuned_config(u64 n, FwdConfig *out) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_autoload();
    if (g_tune.empty()) return false;
    const TuneBucket *b = &g_tune.back();
    for (const TuneBucket &t : g_tune)
        if (n <= t.max_bytes) { b = &t; break; }
    *out = b->c;
    return true;
}

// KGBWT_STATS=<path>: every coalesced batch appends one line (kind, calls, jobs, input bytes, return code, and the
// first 32 job lengths).
static void log_batch(int kind, size_t calls, size_t jobs, u64 bytes, int rc, const std::vector<Pending *> &take) {
    static const char *path = getenv("KGBWT_STATS");
    if (!path || !*path) return;
    std::string sizes;
    size_t listed = 0;
    for (const Pending *p : take) {
        for (int32_t i = 0; i < p->count && listed < 32; i++, listed++) {
            const int32_t n = kind ? ((const kgbwt_inv_job *)p->jobs)[i].n : ((const kgbwt_fwd_job *)p->jobs)[i].n;
            sizes += (listed ? "," : "") + std::to_string(n);
        }
    }
    if (FILE *f = fopen(path, "a")) {
        fprintf(f, "%s calls=%zu jobs=%zu bytes=%llu rc=%d sizes=%s\n", kind ? "inv" : "fwd", calls, jobs,
                (unsigned long long)bytes, rc, sizes.c_str());
        fclose(f);
    }
}

// Runs the calls `take` as one batch on the default worker (the caller is the leader and owns the worker).
static void run_coalesced(Context &C, std::vector<Pending *> &take) {
    const int kind = take[0]->kind;
    const uint32_t flags = take[0]->flags;
    size_t total = 0;
    u64 bytes = 0;
    for (Pending *p : take) { total += (size_t)p->count; bytes += p->bytes; }
    int rc;
    if (take.size() == 1) {
        Pending *p = take[0];
        rc = kind ? run_inv_jobs(C.w, (kgbwt_inv_job *)p->jobs, p->count, flags)
                  : run_fwd_jobs(C.w, (kgbwt_fwd_job *)p->jobs, p->count, flags);
        p->rc = rc;
        if (rc) snprintf(p->err, sizeof p->err, "%s", g_err);
    } else {
        std::vector<kgbwt_fwd_job> fj;
        std::vector<kgbwt_inv_job> ij;
        for (Pending *p : take) {
            if (kind) ij.insert(ij.end(), (kgbwt_inv_job *)p->jobs, (kgbwt_inv_job *)p->jobs + p->count);
            else fj.insert(fj.end(), (kgbwt_fwd_job *)p->jobs, (kgbwt_fwd_job *)p->jobs + p->count);
        }
        rc = kind ? run_inv_jobs(C.w, ij.data(), (int32_t)ij.size(), flags)
                  : run_fwd_jobs(C.w, fj.data(), (int32_t)fj.size(), flags);
        // Per-job outcomes (bad arguments, a string that is no BWT) are in the jobs' rc and stay with their jobs. A
        // failure of the combined batch as a whole (device memory, a batch too large to lay out) fails every job:
        // then each call runs again alone, so that a call's result never depends on what it was batched with.
        bool whole = rc == -2;
        if (rc && !whole) {
            whole = true;
            for (size_t i = 0; i < total && whole; i++) whole = (kind ? ij[i].rc : fj[i].rc) != 0;
        }
        if (whole) {
            std::lock_guard<std::mutex> lock(C.mu);
            C.retried++;
        }
        size_t k = 0;
        for (Pending *p : take) {
            bool failed = false;
            if (whole) {
                p->rc = kind ? run_inv_jobs(C.w, (kgbwt_inv_job *)p->jobs, p->count, flags)
                             : run_fwd_jobs(C.w, (kgbwt_fwd_job *)p->jobs, p->count, flags);
                failed = p->rc != 0;
            } else {
                for (int32_t i = 0; i < p->count; i++, k++) {
                    const int32_t jr = kind ? ij[k].rc : fj[k].rc;
                    if (kind) ((kgbwt_inv_job *)p->jobs)[i].rc = jr;
                    else ((kgbwt_fwd_job *)p->jobs)[i].rc = jr;
                    failed = failed || jr != 0;
                }
                p->rc = 0;
            }
            if (failed) snprintf(p->err, sizeof p->err, "%s", g_err);
        }
    }
    log_batch(kind, take.size(), total, bytes, rc, take);
}

// Queues one call and returns its device-level return code once a leader (possibly this thread) has run it.
static int submit(Pending &p) {
    Context &C = ctx();
    std::unique_lock<std::mutex> lk(C.mu);
    C.q.push_back(&p);
    C.calls[p.kind]++;
    while (!p.done) {
        if (C.busy) { C.cv.wait(lk); continue; }
        C.busy = true;
        std::vector<Pending *> take;
        const Pending *first = C.q.front();
        u64 bytes = 0;
        for (auto it = C.q.begin(); it != C.q.end();) {
            Pending *x = *it;
            if (x->kind != first->kind || x->flags != first->flags) { ++it; continue; }
            if (!take.empty() && bytes + x->bytes > batch_cap()) break;
            take.push_back(x);
            bytes += x->bytes;
            it = C.q.erase(it);
        }
        lk.unlock();
        run_coalesced(C, take);
        lk.lock();
        C.batches[take[0]->kind]++;
        C.largest[take[0]->kind] = std::max<int64_t>(C.largest[take[0]->kind], (int64_t)take.size());
        for (Pending *x : take) x->done = true;
        C.busy = false;
        C.cv.notify_all();
    }
    if (p.err[0]) record_error(p.err);
    return p.rc;
}

static int fwd_batch_impl(kgbwt_fwd_job *jobs, int32_t count, uint32_t flags) {
    Pending p{0, jobs, count, flags, 0};
    for (int32_t i = 0; i < count; i++) p.bytes += jobs[i].n > 0 ? (u64)jobs[i].n : 0;
    return submit(p);
}
static int inv_batch_impl(kgbwt_inv_job *jobs, int32_t count, uint32_t flags) {
    Pending p{1, jobs, count, flags, 0};
    for (int32_t i = 0; i < count; i++) p.bytes += jobs[i].n > 0 ? (u64)jobs[i].n : 0;
    return submit(p);
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int32_t kolmo_sais_bwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, int32_t *I,
                           int32_t threads) {
    (void)threads;
    if (!T || !U || !A || n < 0 || bad_r(r) || !I) return -1;
    kgbwt_fwd_job j = {T, U, n, r, I, 0};
    int rc = fwd_batch_impl(&j, 1, env_flags());
    return rc ? rc : j.rc;
}

int32_t kolmo_sais_unbwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, const int32_t *I,
                             int32_t threads) {
    (void)threads;
    if (!T || !U || !A || n < 0 || ((r != n) && bad_r(r)) || !I) return -1;
    kgbwt_inv_job j = {T, U, n, r, I, 0};
    int rc = inv_batch_impl(&j, 1, env_flags());
    return rc ? rc : j.rc;
}

int32_t kolmo_sais_unbwt(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t i, int32_t threads) {
    return kolmo_sais_unbwt_aux(T, U, A, n, n, &i, threads);
}

int32_t kgbwt_fwd_batch(kgbwt_fwd_job *jobs, int32_t count, uint32_t flags) {
    if (!jobs || count < 0) return -1;
    int rc = fwd_batch_impl(jobs, count, flags | env_flags());
    if (rc) return rc;
    for (int i = 0; i < count; i++) if (jobs[i].rc) return jobs[i].rc;
    return 0;
}

int32_t kgbwt_inv_batch(kgbwt_inv_job *jobs, int32_t count, uint32_t flags) {
    if (!jobs || count < 0) return -1;
    int rc = inv_batch_impl(jobs, count, flags | env_flags());
    if (rc) return rc;
    for (int i = 0; i < count; i++) if (jobs[i].rc) return jobs[i].rc;
    return 0;
}

kgbwt_engine *kgbwt_engine_create(void) { return new (std::nothrow) kgbwt_engine(); }
void kgbwt_engine_destroy(kgbwt_engine *e) { delete e; }

int32_t kgbwt_engine_config(kgbwt_engine *e, int32_t tile_cap, int32_t tile_ctas, int32_t msd_ctas) {
    if (!e) return -1;
    if (tile_cap && tile_cap != 4096 && tile_cap != 8192) return -1;
    if (tile_ctas < 0 || tile_ctas > 8 || msd_ctas < 0 || msd_ctas > 16) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    if (tile_cap && tile_cap != e->fwd.ucfg.tile_cap) {
        // a different tile capacity changes list capacities: drop the workspace (it is rebuilt on the next call)
        const FwdConfig keep = e->fwd.ucfg;
        const u32 mask = e->fwd.cfg_explicit;
        e->fwd.~FwdEngine();
        new (&e->fwd) FwdEngine();
        e->fwd.ucfg = keep;
        e->fwd.cfg_explicit = mask;
        e->fwd.ucfg.tile_cap = tile_cap;
    }
    if (tile_ctas) { e->fwd.ucfg.tile_ctas = tile_ctas; e->fwd.cfg_explicit |= CFG_TILE_CTAS; }
    if (msd_ctas) { e->fwd.ucfg.msd_ctas = msd_ctas; e->fwd.cfg_explicit |= CFG_MSD_CTAS; }
    return 0;
}

int32_t kgbwt_engine_option(kgbwt_engine *e, int32_t option, int32_t value) {
    if (!e) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    switch (option) {
        case KGBWT_OPT_SMALL_GROUP:
            if (value < 0 || value > 1024) return -1;
            e->fwd.ucfg.small_group = value;
            e->fwd.cfg_explicit |= CFG_SMALL_GROUP;
            return 0;
        case KGBWT_OPT_WARP_PATH:
            if (value != 0 && value != 1) return -1;
            e->fwd.ucfg.warp_path = value;
            e->fwd.cfg_explicit |= CFG_WARP_PATH;
            return 0;
        case KGBWT_OPT_LSD_ROUND0:
            if (value != 0 && value != 1) return -1;
            e->fwd.ucfg.lsd_round0 = value;
            e->fwd.cfg_explicit |= CFG_LSD_ROUND0;
            return 0;
        case KGBWT_OPT_LSD_BYTES:
            if (value != 8 && value != 12 && value != 16) return -1;
            e->fwd.ucfg.lsd_bytes = value;
            e->fwd.cfg_explicit |= CFG_LSD_BYTES;
            return 0;
        case KGBWT_OPT_CHAIN_FROM:
            if (value < 0 || value > 64) return -1;
            e->fwd.ucfg.chain_from = value;
            e->fwd.cfg_explicit |= CFG_CHAIN_FROM;
            return 0;
        default:
            return -1;
    }
}

int32_t kgbwt_engine_fwd(kgbwt_engine *e, const uint8_t *dT, uint8_t *dL, int32_t *dI, int32_t *dSA,
                         const kgbwt_block *blocks, int32_t count, void *stream, uint32_t flags) {
    if (!e || !dT || !dL || !dI || !blocks || count <= 0) return -1;
    if (((uintptr_t)dT & 7) != 0) { record_error("text buffer must be 8-byte aligned"); return -1; }
    std::lock_guard<std::mutex> lock(e->mu);
    std::vector<u32> off(count), n(count), r(count), io(count);
    for (int b = 0; b < count; b++) {
        if (blocks[b].n < 2 || bad_r((int32_t)blocks[b].r) || blocks[b].n > 0x7FFFFFFFu) return -1;
        off[b] = blocks[b].off; n[b] = blocks[b].n; r[b] = blocks[b].r; io[b] = blocks[b].iout;
    }
    int rc = e->fwd.plan_external(off.data(), n.data(), r.data(), io.data(), count, const_cast<uint8_t *>(dT), dL,
                                  reinterpret_cast<u32 *>(dI), reinterpret_cast<u32 *>(dSA));
    if (rc) return rc;
    e->last = (cudaStream_t)stream;
    e->last_kind = 1;
    return e->fwd.run((cudaStream_t)stream, !(flags & KGBWT_PLAIN));
}

int32_t kgbwt_engine_inv(kgbwt_engine *e, const uint8_t *dU, uint8_t *dOut, const kgbwt_iblock *blocks,
                         int32_t count, void *stream, uint32_t flags) {
    if (!e || !dU || !dOut || !blocks || count <= 0) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    std::vector<u32> off(count), n(count), p0(count);
    for (int b = 0; b < count; b++) {
        if (blocks[b].n < 2 || blocks[b].p0 < 1 || blocks[b].p0 > blocks[b].n || blocks[b].n > 0x7FFFFFFFu) return -1;
        off[b] = blocks[b].off; n[b] = blocks[b].n; p0[b] = blocks[b].p0;
    }
    int rc = e->inv.plan_external(off.data(), n.data(), p0.data(), count, const_cast<uint8_t *>(dU), dOut);
    if (rc) return rc;
    e->last = (cudaStream_t)stream;
    e->last_kind = 2;
    return e->inv.run((cudaStream_t)stream, !(flags & KGBWT_PLAIN));
}

int32_t kgbwt_engine_wait(kgbwt_engine *e, int32_t *status) {
    if (!e) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    if (e->last_kind == 1) {
        u32 err = 0;
        if (int rc = e->fwd.error_flag(e->last, &err)) return rc;
        if (err) { record_error("forward sort: round limit exceeded (internal error)"); return -2; }
        return 0;
    }
    if (e->last_kind == 2) {
        std::vector<int> st;
        if (int rc = e->inv.fetch_status(e->last, st)) return rc;
        int first = 0;
        for (size_t b = 0; b < st.size(); b++) {
            int v = st[b] ? -1 : 0;
            if (status) status[b] = v;
            if (v && !first) first = v;
        }
        return first;
    }
    return 0;
}

int32_t kgbwt_engine_stats(kgbwt_engine *e, int32_t *rounds, int32_t *passes, int64_t *launches) {
    if (!e) return -1;
    if (e->last_kind == 2) {
        if (rounds) *rounds = 0;
        if (passes) *passes = e->inv.stats.jumps;
        if (launches) *launches = e->inv.stats.launches;
        return 0;
    }
    if (rounds) *rounds = e->fwd.stats.rounds;
    if (passes) *passes = e->fwd.stats.passes;
    if (launches) *launches = e->fwd.stats.launches;
    return 0;
}

uint64_t kgbwt_engine_workspace_bytes(kgbwt_engine *e) { return e ? e->fwd.workspace_bytes() + e->inv.workspace_bytes() : 0; }

int32_t kgbwt_engine_profile(kgbwt_engine *e, int32_t enable) {
    if (!e) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    e->fwd.prof.on = enable != 0;
    e->inv.prof.on = enable != 0;
    return 0;
}

int32_t kgbwt_engine_profile_read(kgbwt_engine *e, kgbwt_prof *out, int32_t cap) {
    if (!e || (!out && cap)) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    Profiler &P = e->last_kind == 2 ? e->inv.prof : e->fwd.prof;
    P.finish();
    int32_t k = 0;
    for (const ProfRec &r : P.recs) {
        if (k >= cap) break;
        out[k++] = kgbwt_prof{r.kernel, r.round, r.pass, r.elems, r.segs, r.ms};
    }
    return (int32_t)P.recs.size();
}

const char *kgbwt_kernel_name(int32_t kernel) { return kernel_name(kernel); }

int32_t kgbwt_tuning_load(const char *path) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_tried = true;  // an explicit load (or clear) replaces the automatic one
    if (!path) { g_tune.clear(); return 0; }
    std::vector<TuneBucket> t;
    const int k = load_tuning_file(path, t);
    if (k < 0) { record_error("kgbwt_tuning_load: not a readable tuning table"); return -1; }
    g_tune.swap(t);
    return k;
}

int32_t kgbwt_tuning_lookup(uint64_t n, int32_t *cfg) {
    if (!cfg) return -1;
    FwdConfig c;
    const bool t = tuned_config(n, &c);
    cfg[0] = c.tile_cap; cfg[1] = c.tile_ctas; cfg[2] = c.msd_ctas; cfg[3] = c.small_group; cfg[4] = c.warp_path;
    cfg[5] = c.lsd_round0; cfg[6] = c.lsd_bytes;
    return t ? 1 : 0;
}

int32_t kgbwt_engine_last_config(kgbwt_engine *e, int32_t *cfg) {
    if (!e || !cfg) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    const FwdConfig &c = e->fwd.cfg;
    cfg[0] = c.tile_cap; cfg[1] = c.tile_ctas; cfg[2] = c.msd_ctas; cfg[3] = c.small_group; cfg[4] = c.warp_path;
    cfg[5] = c.lsd_round0; cfg[6] = c.lsd_bytes;
    return 0;
}

// The configuration fields in their reporting order, the first ncfg of them (at most KGBWT_CONFIG_FIELDS).
static void config_fields(const FwdConfig &c, int32_t *cfg, int32_t ncfg) {
    const int32_t f[KGBWT_CONFIG_FIELDS] = {c.tile_cap,   c.tile_ctas,  c.msd_ctas,  c.small_group,
                                            c.warp_path,  c.lsd_round0, c.lsd_bytes, c.chain_from};
    for (int32_t i = 0; i < ncfg && i < KGBWT_CONFIG_FIELDS; i++) cfg[i] = f[i];
}

int32_t kgbwt_tuning_lookup_n(uint64_t n, int32_t *cfg, int32_t ncfg) {
    if (!cfg || ncfg < 1) return -1;
    FwdConfig c;
    const bool t = tuned_config(n, &c);
    config_fields(c, cfg, ncfg);
    return t ? 1 : 0;
}

int32_t kgbwt_engine_last_config_n(kgbwt_engine *e, int32_t *cfg, int32_t ncfg) {
    if (!e || !cfg || ncfg < 1) return -1;
    std::lock_guard<std::mutex> lock(e->mu);
    config_fields(e->fwd.cfg, cfg, ncfg);
    return 0;
}

int32_t kgbwt_dropin_stats(int64_t *out, int32_t cap) {
    if (!out || cap < 0) return -1;
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    const int64_t v[7] = {C.calls[0], C.batches[0], C.largest[0], C.calls[1], C.batches[1], C.largest[1], C.retried};
    for (int32_t i = 0; i < cap && i < 7; i++) out[i] = v[i];
    return 7;
}

const char *kgbwt_last_error(void) { return g_err; }
int32_t kgbwt_version(void) { return 100; }

}  // extern "C"
