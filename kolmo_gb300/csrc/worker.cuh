// A sorting worker: one forward engine, one inverse engine, one stream and pinned staging. The drop-in calls run on
// the library's default worker; the request server runs one worker per slot. Both use run_fwd_jobs / run_inv_jobs,
// so a request gives the same bytes whichever path carries it.
#pragma once
#include <mutex>
#include <vector>

#include "fwd.cuh"
#include "inv.cuh"
#include "kgbwt.h"

struct kgbwt_engine {
    kgb::FwdEngine fwd;
    kgb::InvEngine inv;
    cudaStream_t last = nullptr;
    int last_kind = 0;
    std::vector<int> inv_status;
    std::mutex mu;
};

namespace kgb {

// Pinned host staging, grown on demand.
struct Pinned {
    u8 *p = nullptr;
    size_t cap = 0;
    int need(size_t bytes);
    void release();
    ~Pinned() { release(); }
};

struct Worker {
    kgbwt_engine eng;
    cudaStream_t stream = nullptr;
    Pinned stage_L, stage_I;  // results for pageable destinations; sampled indexes
    int init();                   // creates the stream on first use
    u64 device_bytes() const { return eng.fwd.workspace_bytes() + eng.inv.workspace_bytes(); }
    void release();               // frees both workspaces and the staging (the stream stays)
    ~Worker();
};

bool bad_r(int32_t r);
// Forward / inverse BWT of host jobs on worker W (argument checks, n <= 1 cases, copies, device run, results).
// Per-job codes land in jobs[i].rc; the return value is 0 or the first device-level failure.
int run_fwd_jobs(Worker &W, kgbwt_fwd_job *jobs, int32_t count, uint32_t flags);
int run_inv_jobs(Worker &W, kgbwt_inv_job *jobs, int32_t count, uint32_t flags);

}  // namespace kgb
