// Inverse BWT engine: parallel psi-walk decode of a batch of blocks on one GPU.
#pragma once
#include "common.cuh"

#include <vector>

namespace kgb {

struct InvBlock {
    u32 off;         // first byte of the block's BWT string (and of its decoded text)
    u32 n;           // block length
    u32 p0;          // primary index (row of the sentinel in the L column), 1..n
    u32 chunk_base;  // first 64 KiB chunk of the block (psi build)
    u32 nchunk;
    u32 chain_base;  // first chain record of the block
    u32 nreg;        // regular marks: chain m in 1..nreg starts at row (m * hmul) & hmask when that row is <= n
    u32 chain_cap;   // chain records reserved for the block
    u32 hmask;       // 2^k - 1 with 2^k >= n
    u32 hmul;        // odd multiplier: the top k bits of 2^64 / golden ratio (rows of the marks are a Weyl sequence)
    u32 hinv;        // hmul^-1 mod 2^32: row q is mark (q * hinv) & hmask
    u32 qbase;       // the block's chains in the walk's sequence over all blocks: qbase .. qbase + nreg
};

struct InvStats {
    long long launches;
    int jumps;
};

class InvEngine {
   public:
    InvEngine();
    ~InvEngine();
    // blocks of lengths n[] (>= 2) with primary indexes p0[] in 1..n. Returns 0, -1 or -2.
    int plan(const u32 *n, const u32 *p0, int count);
    int plan_external(const u32 *off, const u32 *n, const u32 *p0, int count, u8 *dU, u8 *dOut);
    u8 *input() const { return d_U; }
    const u8 *output() const { return d_out; }
    const std::vector<u32> &offsets() const { return h_off; }
    u64 total() const { return N; }
    // decode on stream s; per-block status (0 ok, -1 not a valid BWT) lands in status() after sync
    int run(cudaStream_t s, bool graph);
    int fetch_status(cudaStream_t s, std::vector<int> &status);
    InvStats stats{};
    Profiler prof;  // plain path only
    bool prof_run = false;
    u64 workspace_bytes() const { return pool_bytes; }
    // device bytes the workspace would hold after a call on blocks of these lengths (no allocation; host only)
    u64 estimate_bytes(const u32 *n, int count);

   private:
    int grow(u64 ncap, u32 bcap, u64 tcap, u64 ccap);
    template <typename Add>
    void layout(u64 ncap, u32 bcap, u64 tcap, u64 ccap, Add add);
    int build_graph(cudaStream_t s);
    int enqueue(cudaStream_t s, long long *launches);
    void free_all();
    u64 Ncap = 0, Tcap = 0, Ccap = 0;
    u32 Bcap = 0;
    u64 N = 0, nchunk_all = 0, nchains = 0;
    u32 B = 0, maxchains = 0, njump = 0, nchunks = 0, nwalk = 0;
    int walk_grid = 0;   // resident CTAs of the persistent walk kernel
    bool small = false;  // a small batch: denser marks and the persistent walk
    std::vector<u32> h_off;
    std::vector<InvBlock> h_blk;
    std::vector<u32> h_chunks;  // (block, first chain, end chain) triples for the walk
    bool ext = false;
    u8 *d_U = nullptr, *d_out = nullptr, *own_U = nullptr, *own_out = nullptr;
    u32 *d_psi = nullptr, *d_csum = nullptr, *d_C = nullptr, *d_cblk = nullptr;
    u32 *d_len = nullptr, *d_succ = nullptr, *d_nx[2] = {nullptr, nullptr}, *d_dist[2] = {nullptr, nullptr};
    u32 *d_dyn = nullptr, *d_status = nullptr, *d_chunks = nullptr;
    u8 *d_buf = nullptr;
    InvBlock *d_blk = nullptr;
    void *pool = nullptr;
    size_t pool_bytes = 0;
    int *h_status = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t cap_stream = nullptr;
    // everything a captured graph depends on; a shape runs as plain launches the first time it is seen and is
    // captured when it comes back
    struct GraphKey {
        u64 N, Ncap, nchunk_all, nchains;
        u32 B, njump, nchunks;
        const void *U, *out;
        bool small;
        bool operator==(const GraphKey &o) const {
            return N == o.N && Ncap == o.Ncap && nchunk_all == o.nchunk_all && nchains == o.nchains && B == o.B &&
                   njump == o.njump && nchunks == o.nchunks && U == o.U && out == o.out && small == o.small;
        }
    };
    GraphKey graph_key{}, seen_key{};
    bool seen_valid = false;
    int sm_count = 0;
};

}  // namespace kgb
