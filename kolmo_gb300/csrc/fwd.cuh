// Forward BWT engine: prefix-doubling suffix sorting of a batch of independent blocks on one GPU.
#pragma once
#include "common.cuh"

#include <vector>

namespace kgb {

struct FwdArgs;

// One block of a batch. `off` is the block's first byte in the concatenated text; the block's L column (n + 1
// bytes, sentinel row included) starts at off + index of the block; its sampled indexes start at `iout`.
struct BlockInfo {
    u32 off, n, r, iout;
    u32 soff;  // first position of the block in the dense order of all suffixes of the batch (prefix sum of n)
    u32 lt0;   // first round-0 sort tile of the block (tiles never straddle blocks)
};

// A segment of an element list: `len` consecutive elements starting at `start` that form one group (equal sort
// keys so far) whose first member sits at suffix-array position `head` of block `bd & 0xFFFFFF`. The top byte of
// `bd` holds the next radix digit for segments still being split by the bucket passes.
struct Seg {
    u32 start, len, head, bd;
};

enum : u32 {
    L_S0, L_S1,  // small groups (<= SMAX elements), one list per round parity
    L_L0, L_L1,  // large groups, one list per round parity
    L_K0, L_K1,  // bucket-pass work lists (ping-pong across passes)
    L_KS,        // small buckets produced by the bucket passes, keys attached
    L_R0, L_R1,  // suffixes resolved in a round (their ranks are copied to the other rank buffer next round)
    L_P0, L_P1,  // tiny groups (2..GTINY elements) of the rank rounds: descriptors per round parity, ids in one array
    L_M0, L_M1,  // medium groups (GTINY+1..GMED elements) of the rank rounds, one list per round parity
    NLISTS
};

struct ListView {
    u32 *eid;   // element: global suffix index
    u32 *ekey;  // element: current sort key (rank rounds), may be null
    Seg *seg;   // segment descriptors
    u32 *tmap;  // tile map (see fwd.cu)
    u32 *tbig;  // small lists: per tile window, the round stamp of a group longer than WARP_GROUP starting there
};

// Device-resident control block of one forward sort (read by every kernel, written by the 1-thread control
// kernels), so that the whole sort can run inside a CUDA graph without host round trips.
struct Ctl {
    u64 cnt[NLISTS];  // per list: (segments << 32) | elements
    u32 rpar;         // round parity
    u32 pass;         // bucket pass within the round
    u32 round;        // doubling round (0: 8-byte prefixes)
    u32 h;            // characters already sorted (rank rounds)
    u32 done;
    u32 err;
    u32 maxrounds;
    u32 lsd_tiles;    // round-0 sort tiles of the batch
    u64 tile_elems[2];  // elements sorted so far by the block-level and the warp-level tile kernels (statistics)
    // round 0 as an LSD radix sort
    u32 lsd_act;        // bit s: digit slot s varies (a pass runs for it)
    u32 h0;             // characters round 0 sorts (the first rank round's h)
    u32 m;              // suffixes sorted
    u32 seq;            // call sequence number (tags the look-back words of the radix passes)
    u32 p_alloc;        // slots taken so far in the tiny-group id array (shared by both parities, never reused)
    u32 idn;            // suffix ids of the batch lie in [0, idn) (the rank buffers' used extent)
    u32 prev_active;    // active suffixes of the round that just ended (the round-end kernel's last count)
    u32 chain_go;       // this round follows repeat chains (doubling split less than a fifth of the actives)
};

struct FwdConfig {
    int tile_cap = 4096;  // small-group tile capacity: 4096 or 8192 (groups up to tile_cap / 2 go to the tiles)
    int tile_ctas = 2;    // persistent CTAs per SM for the tile sorter
    int msd_ctas = 8;     // persistent CTAs per SM for the bucket passes
    int small_group = 64; // tiles whose groups are all at most this long skip the radix passes (counting sort)
    int warp_path = 1;    // tiles whose groups are all <= 32 long go to the warp-level kernel
    int lsd_round0 = 1;   // round 0 as one LSD radix sort of all suffixes; 0: bucket passes + tiles over 8-byte prefixes
    int lsd_bytes = 16;   // prefix bytes the LSD round 0 sorts (8, 12 or 16)
    int chain_from = 1;   // first rank round whose tiny groups may be ordered along their repeat chains (0: never)
};
// Fields of FwdConfig a caller set explicitly (they override the tuning table).
enum : u32 {
    CFG_TILE_CTAS = 1, CFG_MSD_CTAS = 2, CFG_SMALL_GROUP = 4, CFG_WARP_PATH = 8, CFG_LSD_ROUND0 = 16, CFG_LSD_BYTES = 32,
    CFG_CHAIN_FROM = 64
};
// The tuning table's configuration for a batch of n text bytes: fills the fields the table sets (tile_ctas,
// msd_ctas, small_group, warp_path, lsd_round0) and returns true, or returns false when no table is loaded.
bool tuned_config(u64 n, FwdConfig *out);

struct FwdStats {
    int rounds;
    int passes;
    long long launches;
    double ms;
};

// Device buffers for batches up to (ncap bytes, bcap blocks). Reused across calls; grown on demand.
class FwdEngine {
   public:
    FwdConfig ucfg;         // the caller's configuration (api: kgbwt_engine_config / _option)
    u32 cfg_explicit = 0;   // CFG_* bits of the fields the caller set
    void resolve_config();  // cfg = ucfg, with the tuning table's values for the fields the caller left alone
    FwdEngine();
    ~FwdEngine();
    // Prepares a batch of `count` blocks with lengths n[] (each >= 2) and sampling intervals r[]: lays the blocks
    // out, grows the buffers and fills the block table. Returns 0, -1 (too large) or -2 (out of device memory).
    int plan(const u32 *n, const u32 *r, int count, bool want_sa);
    // Device text buffer of the planned batch (block b at offsets()[b]); 16 zero bytes follow the last block.
    u8 *text() const { return d_T; }
    const std::vector<u32> &offsets() const { return h_off; }
    const std::vector<u32> &iouts() const { return h_iout; }
    u64 total() const { return N; }
    u32 samples() const { return nI; }
    // Runs the sort on `s`: graph = one CUDA-graph launch with device-side loops, else one launch per kernel with a
    // host read of the control block after each round and bucket pass. Results stay on the device.
    int run(cudaStream_t s, bool graph);
    // Result buffers (device): L columns (block b at off + b, n + 1 bytes), sampled indexes, suffix arrays.
    const u8 *lcol() const { return d_L; }
    const u32 *samples_dev() const { return d_I; }
    const u32 *sa_dev() const { return d_SA; }
    int error_flag(cudaStream_t s, u32 *err);  // reads the device error word (after run)
    u64 workspace_bytes() const { return pool_bytes; }
    // device bytes the workspace would hold after a call with these totals (no allocation; host only)
    u64 estimate_bytes(u64 n, u32 blocks, u32 samples);
    FwdConfig cfg;          // the configuration of the current call
    FwdStats stats{};
    Profiler prof;  // plain path only: events around every launch when prof.on

    // External-buffer mode: sort texts already on the device (dT: concatenated texts, 16 readable bytes past the
    // last; dL / dI / dSA receive the results). Lays the batch out from caller offsets.
    int plan_external(const u32 *off, const u32 *n, const u32 *r, const u32 *iout, int count, u8 *dT, u8 *dL,
                      u32 *dI, u32 *dSA);

   private:
    int grow(u64 ncap, u32 bcap, u32 icap, bool want_sa);
    template <typename Add>
    void layout(u64 ncap, u32 bcap, u32 icap, bool want_sa, Add add);
    int run_plain(cudaStream_t s);
    int run_graph(cudaStream_t s);
    int build_graph(cudaStream_t s);
    void free_all();
    int setup_round0(cudaStream_t s);
    void set_caps(FwdArgs &a) const;
    bool lsd_enabled() const;
    u32 call_seq = 0;
    u64 cap_segs = 0, cap_segk = 0, cap_segl = 0, cap_segt = 0, cap_segm = 0, cap_tms = 0, cap_tml = 0;

    // capacities
    u64 Ncap = 0;
    u32 Bcap = 0, Icap = 0;
    bool sa_cap = false;
    // planned batch
    u64 N = 0;
    u32 B = 0, nI = 0;
    u32 maxn = 0;
    std::vector<u32> h_off, h_n, h_r, h_iout;
    bool ext = false;
    bool want_sa_run = false;

    // device buffers
    u8 *d_T = nullptr, *d_L = nullptr;
    u8 *own_T = nullptr, *own_L = nullptr;
    u32 *d_I = nullptr, *own_I = nullptr;
    u32 *d_SA = nullptr, *own_SA = nullptr;
    u32 *d_isa[2] = {nullptr, nullptr};
    BlockInfo *d_blk = nullptr;
    ListView lists[NLISTS];
    u32 *d_hist = nullptr, *d_cursor = nullptr, *d_bhead = nullptr, *d_orand = nullptr;
    u64 *d_orand64 = nullptr;
    // LSD path
    u32 *d_lval[2] = {nullptr, nullptr}, *d_lhi[2] = {nullptr, nullptr};
    u64 *d_lstat = nullptr;
    u32 *d_lbase = nullptr;
    u32 *d_lhist = nullptr, *d_ltile = nullptr, *d_segagg = nullptr, *d_segbits = nullptr;
    u32 *d_cbits = nullptr, *d_cnz = nullptr, *d_ctn = nullptr;  // repeat chains
    u64 lsd_tiles_cap = 0, seg_tiles_cap = 0;
    u8 *d_dest = nullptr;
    Ctl *d_ctl = nullptr;
    Ctl *h_ctl = nullptr;  // pinned mirror
    void *pool = nullptr;
    size_t pool_bytes = 0;

    // graph cache
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t cap_stream = nullptr;
    int graph_cap_key = 0;
    // everything a captured graph depends on: pointers, sizes and the configuration it was captured with
    struct GraphKey {
        u64 N, Ncap;
        u32 B;
        const void *T, *L, *I, *SA;
        FwdConfig cfg;
        bool lsd;
        bool operator==(const GraphKey &o) const {
            return N == o.N && Ncap == o.Ncap && B == o.B && T == o.T && L == o.L && I == o.I && SA == o.SA &&
                   cfg.tile_cap == o.cfg.tile_cap && cfg.tile_ctas == o.cfg.tile_ctas &&
                   cfg.msd_ctas == o.cfg.msd_ctas && cfg.small_group == o.cfg.small_group &&
                   cfg.warp_path == o.cfg.warp_path && cfg.lsd_round0 == o.cfg.lsd_round0 &&
                   cfg.lsd_bytes == o.cfg.lsd_bytes && cfg.chain_from == o.cfg.chain_from && lsd == o.lsd;
        }
    };
    GraphKey graph_key{};
    // the shape of the last call that ran without a graph: a shape runs as plain launches the first time it is seen
    // and is captured when it comes back (a capture costs more than the plain path saves on one call)
    GraphKey seen_key{};
    bool seen_valid = false;
    int sm_count = 0;
    int grid_tile = 0, grid_msd = 0, grid_scan = 0, grid_tile_prefix = 0, grid_warp = 0, grid_lsd = 0;
};

}  // namespace kgb
