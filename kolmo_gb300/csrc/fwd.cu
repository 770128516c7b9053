// Forward BWT on the GPU: prefix-doubling suffix sorting over a batch of independent blocks (sm_103a).
//
// Algorithm (Manber-Myers prefix doubling, as restated for GPUs by the reference's Metal sorter,
// src/arch/metal/sa_metal.m:1-13 and src/arch/metal/sa.metal:178-256 of adnaneben/kolmo):
//   round 0   group all suffixes by their first 8 bytes (zero padded past the block end);
//   round j   h = 8 * 2^(j-1) characters are sorted; every suffix i still in a group of two or more ("active") is
//             re-sorted inside its group by rank(i + h), where past the end of the block the key is below every
//             rank and decreases with i (a shorter suffix sorts first: the reference's implicit sentinel);
//   a suffix alone in its group is final: its rank is its suffix-array position.
// The rank of a group is the suffix-array position of its first member (sa.metal:209-217).
//
// GB300 formulation. There is no global sort per round. Groups are segments of an element list and are refined
// in place of a sort:
//   * groups of up to SMAX elements are packed into tiles of TILE elements and sorted inside shared memory (one
//     CTA per tile, block-wide LSD radix over only the key bytes that vary in the tile); the same kernel gathers
//     the keys, splits the groups, writes ranks and the L column of finished suffixes, and appends the surviving
//     groups to the next round's list. One kernel, one read of each active suffix per round.
//   * larger groups go through most-significant-digit bucket passes (histogram, per-group scan, scatter) until
//     their buckets fit a tile or hold one key value.
// Ranks are double-buffered: a round gathers from isa[rpar] and writes isa[rpar ^ 1], so no round reads a rank
// that the same round refined. Suffixes finished in a round are copied into the other buffer during the next.
// The L column is written as suffixes finish (row p + 1 = T[SA[p] - 1], the reference's BWT convention
// sais.c:12043-12049), so no suffix array pass is needed. A device control block drives every loop, so the whole
// sort is one CUDA graph with conditional while-nodes (no host synchronisation), or, for the plain path, one
// kernel launch per step with a host read of the control block after every pass.
#include "fwd.cuh"

#include <algorithm>
#include <type_traits>
#include <cstdio>
#include <cstring>
#include <functional>

namespace kgb {

constexpr int TPB = 256;
constexpr int TSM = 2048;  // elements per tile of the bucket passes
constexpr int IPM = TSM / TPB;
constexpr u32 DEPTH_PREFIX = 8, DEPTH_RANK = 4;
constexpr u32 WARP_GROUP = 32;  // groups up to this long are handled by one warp (k_tile_warp)
constexpr u32 GTINY = 8;        // groups up to this long leave the rank rounds' tile lists for one thread each
constexpr u32 GMED = 256;       // groups up to this long (and longer than GTINY) are sorted by one warp each
// Seg.bd flag of small groups: the group came from the previous round's small-group list and passed that round
// unsplit, so both rank buffers already hold its head (set only on groups whose input was a small-group list: a group
// cut out of a larger one by the bucket passes has its parent's head in the other buffer).
constexpr u32 STABLE = 0x80000000u;

enum : u8 { C_NONE = 0, C_KS = 1, C_KO = 2, C_LN = 3, C_ONE = 4 };

struct FwdArgs {
    Ctl *ctl;
    const u8 *T;
    const BlockInfo *blk;
    u32 *isa[2];
    u8 *L;
    u32 *SA;
    u32 *I;
    ListView lists[NLISTS];
    u32 *hist, *cursor, *bhead, *orand;
    u64 *orand64;  // prefix rounds: OR and AND of each bucket-pass group's 8-byte prefixes
    u8 *dest;
    u32 B;
    u32 smax;
    u32 small_group;  // tiles whose groups are all at most this long are sorted by counting, not radix passes
    u32 lsd_bytes;    // prefix bytes of the LSD round 0 (8, 12 or 16)
    u32 idn;          // suffix ids of the batch lie in [0, idn)
    u32 rank_passes;  // round 0's ranks: passes of k_seg_rank over id ranges, or 0: written by the emit kernels
    u32 warp_path;    // 1: tiles without a group longer than WARP_GROUP belong to the warp-level kernel
    unsigned long long hcond;  // cudaGraphConditionalHandle of the loop this kernel closes (0: none)
    // round 0 as an LSD radix sort
    u32 *lval[2], *lhi[2], *segbits;
    unsigned long long *lit[2];  // round 0: (key group << 32 | id) items, aliasing lval[q] and lhi[q]
    u64 *lstat;
    u32 *lhist, *ltile, *segagg;
    u32 *lbase;  // round 0: per block and digit slot, the pass's first position of every digit
    u32 spin_limit;
    // repeat chains (rank rounds >= chain_from): bit x of cbits = the group of suffix x continues at x + 1;
    // cnz / ctn: the next-zero tables over cbits' words (see k_chain_nz)
    u32 *cbits, *cnz, *ctn;
    u32 cwords, ctiles, chain_from;
    // capacities (checked build): elements / text bytes, small and large segment records, tile-map entries
    u64 cap_n, cap_segs, cap_segk, cap_segl, cap_segt, cap_segm, cap_tms, cap_tml;
    u32 cap_res;  // entries of each resolved list
};

// device error bits
enum : u32 { E_ROUNDS = 1, E_PASSES = 2, E_TILE = 4, E_LIST = 8, E_SEG = 16, E_TMAP = 32, E_RANK = 64, E_HIST = 128 };

__device__ __forceinline__ u32 seg_blk(u32 bd) { return bd & 0xFFFFFFu; }
// End (exclusive text offset) of block b.
__device__ __forceinline__ u64 blk_end(const FwdArgs &a, u32 b) {
    const BlockInfo B = a.blk[b];
    return (u64)B.off + B.n;
}
__device__ __forceinline__ u32 seg_depth(u32 bd) { return bd >> 24; }

// Depth of the first bucket pass of a rank-round group from the OR/AND of its keys: the byte of the highest
// varying bit (3 when all keys are equal, which then finishes the group in one pass).
__device__ __forceinline__ u32 depth_from_vary(u32 orv, u32 andv) {
    u32 vary = orv ^ andv;
    if (!vary) return DEPTH_RANK - 1;
    u32 msb = 31 - __clz(vary);
    return (31 - msb) >> 3;
}

// Byte d of the zero-padded 8-byte prefix of suffix i of a block ending at `end`.
__device__ __forceinline__ u32 prefix_byte(const u8 *__restrict__ T, u32 i, u32 d, u64 end) {
    return (u64)i + d < end ? (u32)__ldg(T + i + d) : 0u;
}

// Rank-round key of suffix i (block ending at `end`), h characters sorted: rank(i + h) + h, or, past the end,
// end - 1 - i (below every shifted rank, decreasing with i).
__device__ __forceinline__ u32 rank_key(const u32 *__restrict__ isa, u32 i, u32 h, u64 end) {
    u32 d = (u32)(end - i);
    return h < d ? __ldg(isa + i + h) + h : d - 1;
}

// The final state of a suffix: rank = suffix-array position p (block-local), L column row p + 1 = T[i - 1]
// (the sentinel row's byte value is never read), optional suffix array, and its index in the resolved list. The
// resolved list holds cap_res entries, a sixteenth of the ids: the next round's fixup scatters the list only when a
// round finished at most that many suffixes and copies the whole rank buffer otherwise, so entries past the
// capacity are counted but never needed.
// As resolve, with the block's descriptor and the L-column byte (T[id - 1], 0 for the block's first suffix) already
// loaded: callers load the bytes of several finished suffixes at once.
__device__ __forceinline__ void resolve_byte(const FwdArgs &a, u32 *isa_nxt, u32 id, u32 p, u32 b, const BlockInfo &B,
                                             ListView res, u32 ridx, u8 byte) {
    if (!KGB_OK(id < a.cap_n && p < B.n && id >= B.off && id - B.off < B.n, &a.ctl->err, E_RANK)) return;
    isa_nxt[id] = p;
    a.L[(u64)B.off + b + p + 1] = byte;
    if (a.SA) a.SA[(u64)B.off + p] = id - B.off;
    if (ridx < a.cap_res) { res.eid[ridx] = id; res.ekey[ridx] = p; }
}
// As resolve, for round 0: no resolved-list entry (round 1's fixup copies the whole rank buffer) and the rank only
// when the caller writes it.
__device__ __forceinline__ void resolve_round0(const FwdArgs &a, u32 *isa_nxt, u32 id, u32 p, u32 b) {
    BlockInfo B = a.blk[b];
    if (!KGB_OK(id < a.cap_n && p < B.n && id >= B.off && id - B.off < B.n, &a.ctl->err, E_RANK)) return;
    if (isa_nxt) isa_nxt[id] = p;
    a.L[(u64)B.off + b + p + 1] = id == B.off ? 0 : __ldg(a.T + id - 1);
    if (a.SA) a.SA[(u64)B.off + p] = id - B.off;
}
__device__ __forceinline__ void resolve(const FwdArgs &a, u32 *isa_nxt, u32 id, u32 p, u32 b, ListView res,
                                        u32 ridx) {
    BlockInfo B = a.blk[b];
    if (!KGB_OK(id < a.cap_n && p < B.n && id >= B.off && id - B.off < B.n, &a.ctl->err, E_RANK)) return;
    isa_nxt[id] = p;
    a.L[(u64)B.off + b + p + 1] = id == B.off ? 0 : __ldg(a.T + id - 1);
    if (a.SA) a.SA[(u64)B.off + p] = id - B.off;
    if (ridx < a.cap_res) { res.eid[ridx] = id; res.ekey[ridx] = p; }
}

// Tiny groups keep their ids in one array for the whole sort (a tiny group only shrinks, so its members never move to
// another list): a producer takes `elems` fresh slots there and `groups` descriptors in the next round's tiny list.
// Returns (first slot, first descriptor).
__device__ __forceinline__ uint2 alloc_tiny(Ctl *c, u32 rpar, u32 groups, u32 elems) {
    const u32 e = atomicAdd(&c->p_alloc, elems);
    const u64 o = atomicAdd(&c->cnt[L_P0 + (rpar ^ 1)], ((u64)groups << 32) | elems);
    return make_uint2(e, (u32)(o >> 32));
}

// ------------------------------------------------------------------------------------------------ tile sorter
// Tile t of a small-group list covers every segment whose start lies in [t * TS, (t + 1) * TS) (TS = TILE / 2 =
// SMAX, so a tile holds at most TILE elements). tmap[t] = index of the first such segment; the producers of a
// list write it (a segment covering position t * TS writes tmap[t]: its own index if it starts there, else the next).

template <int TILE, typename KeyT>
struct TileSmem {
    static constexpr int TS = TILE / 2;
    KeyT klo[TILE];
    u32 val[TILE];
    u16 khi[TILE];
    u16 wcnt[TPB / 32][256];
    u32 lstart[TS + 1];
    u32 lhead[TS];
    u32 lblk[TS];
    u32 ws[TPB / 32 + 1];
    u32 ws2[TPB / 32 + 1];
    u64 red[4][TPB / 32];
    u32 bases[4];
    u32 pbases[4];
};

__device__ __forceinline__ void write_tmap_small(const FwdArgs &a, u32 *tmap, u32 ts, u32 start, u32 len, u32 sidx) {
    u32 t = (start + ts - 1) / ts;
    if ((u64)t * ts < (u64)start + len) {
        KGB_GUARD(t < a.cap_tms, &a.ctl->err, E_TMAP) tmap[t] = (u64)t * ts == start ? sidx : sidx + 1;
    }
}

template <bool PREFIX, int TILE>
struct TileTraits {
    typedef typename std::conditional<PREFIX, u64, u32>::type KeyT;  // rank keys fit 32 bits
    static constexpr int MINB = TILE == 4096 ? 2 : 1;   // CTAs per SM the registers must allow
};

template <bool PREFIX, bool KEYED, int TILE>
__global__ void __launch_bounds__(TPB, TileTraits<PREFIX, TILE>::MINB) k_tile_sort(FwdArgs a) {
    typedef typename TileTraits<PREFIX, TILE>::KeyT KeyT;
    constexpr int TS = TILE / 2, IPT = TILE / TPB, WS = 32 * IPT, NW = TPB / 32, KB = (int)sizeof(KeyT);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem<TILE, KeyT> &S = *reinterpret_cast<TileSmem<TILE, KeyT> *>(smem_raw);
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, h = ctl->h;
    const u32 lin = KEYED ? L_KS : L_S0 + rpar;
    const ListView in = a.lists[lin];
    const ListView out = a.lists[L_S0 + (rpar ^ 1)];
    const ListView res = a.lists[L_R0 + rpar];
    const u64 c = ctl->cnt[lin];
    const u32 nelem = (u32)c, nseg = (u32)(c >> 32);
    if (nelem > a.cap_n || nseg > (KEYED ? a.cap_segk : a.cap_segs)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 ntiles = (u32)(((u64)nelem + TS - 1) / TS);
    const u32 *isa_cur = a.isa[rpar];
    u32 *isa_nxt = a.isa[rpar ^ 1];
    const u32 lane = lane_id(), warp = warp_id(), tid = threadIdx.x;

    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const u32 sa_ = in.tmap[t];
        const u32 sb_ = t + 1 < ntiles ? in.tmap[t + 1] : nseg;
        if (sa_ > nseg || sb_ > nseg) {
            if (threadIdx.x == 0) atomicOr(&a.ctl->err, E_TMAP);
            continue;
        }
        if (sa_ >= sb_) continue;
        if (a.warp_path && in.tbig[t] != ctl->round) continue;  // all groups short: the warp kernel's tile
        const u32 nsegs = sb_ - sa_;
        const u32 E0 = in.seg[sa_].start;
        const u32 E1 = sb_ < nseg ? in.seg[sb_].start : nelem;
        const u32 cnt = E1 - E0;
        if (nsegs > TS || E1 < E0 || cnt > TILE || E1 > nelem) {  // broken list invariant: report, never overrun
            if (tid == 0) atomicOr(&a.ctl->err, E_TILE);
            continue;
        }
        for (u32 j = tid; j < nsegs; j += TPB) {
            Seg g = in.seg[sa_ + j];
            S.lstart[j] = g.start - E0;
            S.lhead[j] = g.head;  // bit 31 is set below when the group splits
            S.lblk[j] = g.bd;     // block | STABLE
        }
        if (tid == 0) S.lstart[nsegs] = cnt;
        __syncthreads();

        // ---- load: warp-striped arrangement, x = warp * WS + j * 32 + lane
        KeyT k[IPT];
        u32 hi[IPT], v[IPT];
        KeyT orl = 0, andl = (KeyT)~(KeyT)0;
        u32 orh = 0, andh = ~0u;
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const u32 x = warp * WS + j * 32 + lane;
            if (x < cnt) {
                const u32 id = in.eid[E0 + x];
                u32 lo = 0, hh = nsegs - 1;
                while (lo < hh) {
                    u32 mid = (lo + hh + 1) >> 1;
                    if (S.lstart[mid] <= x) lo = mid; else hh = mid - 1;
                }
                KeyT key;
                if (PREFIX) {
                    const BlockInfo B = a.blk[seg_blk(S.lblk[lo])];
                    const u64 end = (u64)B.off + B.n;
                    u64 kk = load_be64(a.T, id);
                    const u64 rem = end - id;
                    if (rem < 8) kk &= ~0ull << (8 * (8 - rem));
                    key = (KeyT)kk;
                } else if (KEYED) {
                    key = in.ekey[E0 + x];
                } else {
                    const BlockInfo B = a.blk[seg_blk(S.lblk[lo])];
                    key = rank_key(isa_cur, id, h, (u64)B.off + B.n);
                }
                k[j] = key;
                hi[j] = lo;
                v[j] = id;
                orl |= key; andl &= key; orh |= lo; andh &= lo;
            } else {
                k[j] = (KeyT)~(KeyT)0;
                hi[j] = 0xFFFFu;
                v[j] = 0;
            }
        }
        // ---- which key bytes vary inside the tile
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            orl |= __shfl_xor_sync(0xffffffffu, orl, o);
            andl &= __shfl_xor_sync(0xffffffffu, andl, o);
            orh |= __shfl_xor_sync(0xffffffffu, orh, o);
            andh &= __shfl_xor_sync(0xffffffffu, andh, o);
        }
        if (lane == 0) { S.red[0][warp] = orl; S.red[1][warp] = andl; S.red[2][warp] = orh; S.red[3][warp] = andh; }
        __syncthreads();
        orl = 0; andl = (KeyT)~(KeyT)0; orh = 0; andh = ~0u;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            orl |= (KeyT)S.red[0][w]; andl &= (KeyT)S.red[1][w]; orh |= (u32)S.red[2][w]; andh &= (u32)S.red[3][w];
        }
        const KeyT vary_lo = orl ^ andl;
        const u32 vary_hi = (orh ^ andh) & 0xFFFFu;
        // longest group of the tile
        u32 ml = 0;
        for (u32 j = tid; j < nsegs; j += TPB) ml = max(ml, S.lstart[j + 1] - S.lstart[j]);
        ml = block_incl_max<TPB>(ml, S.ws);
        if (tid == TPB - 1) S.bases[3] = ml;
        __syncthreads();
        const u32 maxlen = S.bases[3];

        bool in_smem = false;
        if (maxlen <= a.small_group && vary_lo) {
            // ---- small groups: counting sort inside each group (position = keys below + equal keys before)
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = warp * WS + j * 32 + lane;
                S.klo[x] = k[j];
            }
            __syncthreads();
            u32 dst[IPT];
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = warp * WS + j * 32 + lane;
                dst[j] = x;
                if (x < cnt) {
                    const u32 g0 = S.lstart[hi[j]], g1 = S.lstart[hi[j] + 1];
                    u32 below = 0;
                    for (u32 y = g0; y < g1; y++) {
                        const KeyT ky = S.klo[y];
                        below += ky < k[j] || (ky == k[j] && y < x);
                    }
                    dst[j] = g0 + below;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < IPT; j++) { S.klo[dst[j]] = k[j]; S.khi[dst[j]] = (u16)hi[j]; S.val[dst[j]] = v[j]; }
            __syncthreads();
            in_smem = true;
        }

        // ---- LSD radix over the varying bytes: 8 bytes of the key, then 2 bytes of the segment index
        const bool radix = !in_smem;
        for (int digit = 0; digit < KB + 2 && radix; digit++) {
            const bool lo_part = digit < KB;
            const u32 sh = lo_part ? 8 * digit : 8 * (digit - KB);
            if (lo_part ? !((vary_lo >> sh) & 0xFF) : !((vary_hi >> sh) & 0xFF)) continue;
            for (int i = tid; i < NW * 256; i += TPB) (&S.wcnt[0][0])[i] = 0;
            __syncthreads();
            u32 dg[IPT], rk[IPT];
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 d = lo_part ? (u32)(k[j] >> sh) & 0xFF : (hi[j] >> sh) & 0xFF;
                dg[j] = d;
                const u32 peers = __match_any_sync(0xffffffffu, d);
                const u32 before = S.wcnt[warp][d];
                rk[j] = before + __popc(peers & lanemask_lt());
                __syncwarp();
                if ((__ffs(peers) - 1) == (int)lane) S.wcnt[warp][d] = (u16)(before + __popc(peers));
                __syncwarp();
            }
            __syncthreads();
            {   // digit-major exclusive scan: thread tid owns digit tid
                u32 tot = 0;
#pragma unroll
                for (int w = 0; w < NW; w++) tot += S.wcnt[w][tid];
                u32 run = block_excl_sum<TPB>(tot, S.ws, nullptr);
#pragma unroll
                for (int w = 0; w < NW; w++) { u32 cc = S.wcnt[w][tid]; S.wcnt[w][tid] = (u16)run; run += cc; }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 dst = S.wcnt[warp][dg[j]] + rk[j];
                S.klo[dst] = k[j];
                S.khi[dst] = (u16)hi[j];
                S.val[dst] = v[j];
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = warp * WS + j * 32 + lane;
                k[j] = S.klo[x]; hi[j] = S.khi[x]; v[j] = S.val[x];
            }
            in_smem = true;
            __syncthreads();
        }
        if (!in_smem) {
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = warp * WS + j * 32 + lane;
                S.klo[x] = k[j]; S.khi[x] = (u16)hi[j]; S.val[x] = v[j];
            }
            __syncthreads();
        }

        // ---- split groups: blocked arrangement x = tid * IPT + j
        u32 st[IPT], en[IPT];
        u32 gl = 0;
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const u32 x = tid * IPT + j;
            st[j] = en[j] = 0;
            if (x < cnt) {
                const u32 sj = S.khi[x];
                const KeyT kx = S.klo[x];
                st[j] = x == S.lstart[sj] || kx != S.klo[x - 1];
                en[j] = x + 1 == S.lstart[sj + 1] || kx != S.klo[x + 1];
                if (st[j]) gl = x;
                if (st[j] && x != S.lstart[sj]) atomicOr(&S.lhead[sj], 0x80000000u);  // the group splits
            }
        }
        // group first member: inclusive max-scan of group starts (gl = last start in this thread, or 0)
        const u32 incl = block_incl_max<TPB>(gl, S.ws);
        __syncthreads();
        u32 carry;
        {
            // exclusive max = inclusive max of the previous thread
            __shared__ u32 prevmax[TPB];
            prevmax[tid] = incl;
            __syncthreads();
            carry = tid ? prevmax[tid - 1] : 0u;
            __syncthreads();
        }
        // run lengths at the runs' first positions (the keys are no longer needed)
        {
            u32 gf = carry;
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = tid * IPT + j;
                if (x >= cnt) break;
                if (st[j]) gf = x;
                if (en[j]) S.klo[gf] = (KeyT)(x - gf + 1);
            }
        }
        __syncthreads();
        // survivors and runs per destination: tiny runs (<= GTINY) to the tiny list, medium runs (<= GMED) to the
        // medium list, longer ones to the small list
        u32 ns = 0, ng = 0, np = 0, ngp = 0, nm = 0, ngm = 0;
        {
            u32 gf = carry;
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = tid * IPT + j;
                if (x >= cnt) break;
                if (st[j]) gf = x;
                if (st[j] && en[j]) continue;
                const u32 rl = (u32)S.klo[gf];
                if (rl <= GTINY) { np++; ngp += st[j]; }
                else if (rl <= GMED) { nm++; ngm += st[j]; }
                else { ns++; ng += st[j]; }
            }
        }
        u32 tot_pack = 0, tot_packp = 0, tot_packm = 0;
        const u32 pre = block_excl_sum<TPB>(ns | (ng << 16), S.ws, &tot_pack);
        const u32 prep = block_excl_sum<TPB>(np | (ngp << 16), S.ws, &tot_packp);
        const u32 prem = block_excl_sum<TPB>(nm | (ngm << 16), S.ws, &tot_packm);
        const u32 tot_s = tot_pack & 0xFFFFu, tot_g = tot_pack >> 16;
        const u32 tot_p = tot_packp & 0xFFFFu, tot_gp = tot_packp >> 16;
        const u32 tot_m = tot_packm & 0xFFFFu, tot_gm = tot_packm >> 16;
        if (tid == 0) {
            atomicAdd(&a.ctl->tile_elems[0], (u64)cnt);
            if (tot_s) {
                const u64 o = atomicAdd(&a.ctl->cnt[L_S0 + (rpar ^ 1)], ((u64)tot_g << 32) | tot_s);
                S.bases[0] = (u32)o;
                S.bases[1] = (u32)(o >> 32);
            }
            if (tot_p) {
                const uint2 o = alloc_tiny(a.ctl, rpar, tot_gp, tot_p);
                S.pbases[0] = o.x;
                S.pbases[1] = o.y;
            }
            if (tot_m) {
                const u64 o = atomicAdd(&a.ctl->cnt[L_M0 + (rpar ^ 1)], ((u64)tot_gm << 32) | tot_m);
                S.pbases[2] = (u32)o;
                S.pbases[3] = (u32)(o >> 32);
            }
            S.bases[2] = (u32)atomicAdd(&a.ctl->cnt[L_R0 + rpar], (u64)(cnt - tot_s - tot_p - tot_m));
        }
        __syncthreads();
        const ListView outp = a.lists[L_P0 + (rpar ^ 1)], outm = a.lists[L_M0 + (rpar ^ 1)];
        const u32 ebase = S.bases[0], sbase = S.bases[1], rbase = S.bases[2];
        const u32 pebase = S.pbases[0], psbase = S.pbases[1], mebase = S.pbases[2], msbase = S.pbases[3];
        u32 es = pre & 0xFFFFu, gs = pre >> 16, ep = prep & 0xFFFFu, gp = prep >> 16;
        u32 em = prem & 0xFFFFu, gm = prem >> 16;
        u32 gfirst = carry;
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const u32 x = tid * IPT + j;
            if (x >= cnt) break;
            if (st[j]) gfirst = x;
            const u32 sj = S.khi[x], id = S.val[x];
            const u32 s0 = S.lstart[sj];
            const u32 lh = S.lhead[sj], bd = S.lblk[sj];
            const bool unsplit = !(lh >> 31);
            if (st[j] && en[j]) {
                // finished suffixes take the resolved slots in position order after the survivors before them
                resolve(a, isa_nxt, id, (lh & 0x7FFFFFFFu) + (x - s0), seg_blk(bd), res, rbase + (x - es - ep - em));
                continue;
            }
            const u32 head = (lh & 0x7FFFFFFFu) + (gfirst - s0);
            // a group that passed the previous round unsplit and passes this one unsplit already has this head
            // in the write buffer (written two rounds ago)
            if (!((bd & STABLE) && unsplit)) {
                KGB_GUARD(id < a.cap_n, &a.ctl->err, E_RANK) isa_nxt[id] = head;
            }
            const u32 len = (u32)S.klo[gfirst];
            const u32 sbd = seg_blk(bd) | (!PREFIX && !KEYED && unsplit ? STABLE : 0u);
            if (len <= GTINY) {
                KGB_GUARD(pebase + ep < a.cap_n, &a.ctl->err, E_LIST) outp.eid[pebase + ep] = id;
                if (st[j]) gp++;
                if (en[j]) {
                    Seg g;
                    g.start = pebase + ep + 1 - len; g.len = len; g.head = head; g.bd = sbd;
                    KGB_GUARD(psbase + gp - 1 < a.cap_segt, &a.ctl->err, E_SEG) outp.seg[psbase + gp - 1] = g;
                }
                ep++;
            } else if (len <= GMED) {
                KGB_GUARD(mebase + em < a.cap_n, &a.ctl->err, E_LIST) outm.eid[mebase + em] = id;
                if (st[j]) gm++;
                if (en[j]) {
                    Seg g;
                    g.start = mebase + em + 1 - len; g.len = len; g.head = head; g.bd = sbd;
                    KGB_GUARD(msbase + gm - 1 < a.cap_segm, &a.ctl->err, E_SEG) outm.seg[msbase + gm - 1] = g;
                }
                em++;
            } else {
                KGB_GUARD(ebase + es < a.cap_n, &a.ctl->err, E_LIST) out.eid[ebase + es] = id;
                if (st[j]) gs++;
                if (en[j]) {
                    const u32 sidx = sbase + gs - 1, start = ebase + es + 1 - len;
                    Seg g;
                    g.start = start; g.len = len; g.head = head; g.bd = sbd;
                    KGB_GUARD(sidx < a.cap_segs, &a.ctl->err, E_SEG) out.seg[sidx] = g;
                    write_tmap_small(a, out.tmap, TS, start, len, sidx);
                    if (len > WARP_GROUP) out.tbig[start / TS] = ctl->round + 1;
                }
                es++;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------ warp tiles
// Tiles whose groups are all at most WARP_GROUP long (no stamp in tbig for this round). The CTA loads the tile's
// segment descriptors once; then each warp independently takes the groups starting in one eighth of the tile window:
// it gathers their keys into shared memory, sorts every group by counting (a group fits in one warp), and emits
// ranks, finished suffixes and surviving groups with warp scans and one allocation atomic per warp. No block-wide
// barrier after the descriptor load.

template <int TILE, typename KeyT>
struct WarpSmem {
    static constexpr int TS = TILE / 2;
    static constexpr int CAPE = TS + WARP_GROUP;  // at most TS + WARP_GROUP - 1 elements in a window
    u32 lstart[TS + 1];
    u32 lhead[TS];
    u32 lbd[TS];
    KeyT key[2][CAPE];  // gathered order, then sorted order
    u32 val[2][CAPE];
    u16 sg[2][CAPE];
};

template <bool PREFIX, bool KEYED, int TILE>
__global__ void __launch_bounds__(TPB, 3) k_tile_warp(FwdArgs a) {
    typedef typename TileTraits<PREFIX, TILE>::KeyT KeyT;
    constexpr int TS = TILE / 2, NW = TPB / 32, SW = TS / NW, PER = (SW + WARP_GROUP + 31) / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpSmem<TILE, KeyT> &S = *reinterpret_cast<WarpSmem<TILE, KeyT> *>(smem_raw);
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, h = ctl->h, round = ctl->round;
    const u32 lin = KEYED ? L_KS : L_S0 + rpar;
    const ListView in = a.lists[lin];
    const ListView res = a.lists[L_R0 + rpar];
    const u64 c = ctl->cnt[lin];
    const u32 nelem = (u32)c, nseg = (u32)(c >> 32);
    if (nelem > a.cap_n || nseg > (KEYED ? a.cap_segk : a.cap_segs)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 ntiles = (u32)(((u64)nelem + TS - 1) / TS);
    const u32 *isa_cur = a.isa[rpar];
    u32 *isa_nxt = a.isa[rpar ^ 1];
    const u32 lane = lane_id(), warp = warp_id(), tid = threadIdx.x;
    const u32 lt_mask = lanemask_lt();

    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const u32 sa_ = in.tmap[t];
        const u32 sb_ = t + 1 < ntiles ? in.tmap[t + 1] : nseg;
        if (sa_ > nseg || sb_ > nseg) {
            if (tid == 0) atomicOr(&a.ctl->err, E_TMAP);
            continue;
        }
        if (sa_ >= sb_ || in.tbig[t] == round) continue;  // empty, or a block-kernel tile
        const u32 nsegs = sb_ - sa_;
        const u32 E0 = in.seg[sa_].start;
        const u32 E1 = sb_ < nseg ? in.seg[sb_].start : nelem;
        const u32 cnt = E1 - E0;
        if (nsegs > (u32)TS || E1 < E0 || cnt > (u32)(TS + WARP_GROUP) || E1 > nelem) {
            if (tid == 0) atomicOr(&a.ctl->err, E_TILE);
            continue;
        }
        __syncthreads();  // the previous tile's warps are done with the descriptors
        for (u32 j = tid; j < nsegs; j += TPB) {
            const Seg g = in.seg[sa_ + j];
            S.lstart[j] = g.start - E0;
            S.lhead[j] = g.head;
            S.lbd[j] = g.bd;
        }
        if (tid == 0) S.lstart[nsegs] = cnt;
        __syncthreads();

        // this warp's groups: those starting in [t*TS + warp*SW, t*TS + (warp+1)*SW) of the list
        auto first_at = [&](u64 pos) -> u32 {  // first segment with list start >= pos
            if (pos <= E0) return 0;
            const u32 lp = (u32)(pos - E0);
            u32 lo = 0, hi = nsegs;
            while (lo < hi) {
                const u32 mid = (lo + hi) >> 1;
                if (S.lstart[mid] < lp) lo = mid + 1; else hi = mid;
            }
            return lo;
        };
        const u64 w0 = (u64)t * TS + (u64)warp * SW;
        const u32 j0 = first_at(w0);
        const u32 j1 = warp + 1 == NW ? nsegs : first_at(w0 + SW);
        if (j0 >= j1) continue;
        const u32 X0 = S.lstart[j0], X1 = S.lstart[j1];
        if (X1 - X0 > (u32)PER * 32) {  // a long group reached a warp tile: report, never overrun
            if (lane == 0) atomicOr(&a.ctl->err, E_TILE);
            continue;
        }

        // ---- gather keys (4 loads in flight per lane) into buffer 0
        for (u32 xb = X0; xb < X1; xb += 128) {
            u32 ids[4], sgs[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const u32 x = xb + q * 32 + lane;
                ids[q] = x < X1 ? in.eid[E0 + x] : 0u;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const u32 x = xb + q * 32 + lane;
                u32 lo = j0, hi = j1 - 1;  // last segment with lstart <= x
                while (lo < hi) {
                    const u32 mid = (lo + hi + 1) >> 1;
                    if (S.lstart[mid] <= x) lo = mid; else hi = mid - 1;
                }
                sgs[q] = lo;
            }
            KeyT keys[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const u32 x = xb + q * 32 + lane;
                keys[q] = 0;
                if (x < X1) {
                    if (KEYED && !PREFIX) {
                        keys[q] = in.ekey[E0 + x];
                    } else {
                        const BlockInfo B = a.blk[seg_blk(S.lbd[sgs[q]])];
                        const u64 end = (u64)B.off + B.n;
                        if (PREFIX) {
                            u64 kk = load_be64(a.T, ids[q]);
                            const u64 rem = end - ids[q];
                            if (rem < 8) kk &= ~0ull << (8 * (8 - rem));
                            keys[q] = (KeyT)kk;
                        } else {
                            keys[q] = (KeyT)rank_key(isa_cur, ids[q], h, end);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const u32 x = xb + q * 32 + lane;
                if (x < X1) { S.key[0][x] = keys[q]; S.val[0][x] = ids[q]; S.sg[0][x] = (u16)sgs[q]; }
            }
        }
        __syncwarp();
        // ---- sort each group by counting into buffer 1 (position = keys below + equal keys before); lanes of a
        // long group read the same key at each step (shared-memory broadcast)
        for (u32 x = X0 + lane; x < X1; x += 32) {
            const u32 sj = S.sg[0][x];
            const u32 g0 = S.lstart[sj], g1 = S.lstart[sj + 1];
            const KeyT kx = S.key[0][x];
            u32 below = 0;
            for (u32 y = g0; y < g1; y++) {
                const KeyT ky = S.key[0][y];
                below += ky < kx || (ky == kx && y < x);
            }
            const u32 d = g0 + below;
            S.key[1][d] = kx; S.val[1][d] = S.val[0][x]; S.sg[1][d] = (u16)sj;
        }
        __syncwarp();
        // ---- mark segments that split; run lengths at the runs' first positions (buffer 0 is free)
        {
            u32 carry = X0;
            for (u32 xb = X0; xb < X1; xb += 32) {
                const u32 x = xb + lane;
                bool st = false, en = false;
                if (x < X1) {
                    const u32 sj = S.sg[1][x];
                    const KeyT kx = S.key[1][x];
                    st = x == S.lstart[sj] || kx != S.key[1][x - 1];
                    en = x + 1 == S.lstart[sj + 1] || kx != S.key[1][x + 1];
                    if (st && x != S.lstart[sj]) atomicOr(&S.lhead[sj], 0x80000000u);
                }
                const u32 gfirst = max(carry, warp_incl_max(x < X1 && st ? x : 0u));
                if (x < X1 && en) S.key[0][gfirst] = (KeyT)(x - gfirst + 1);
                carry = __shfl_sync(0xffffffffu, gfirst, 31);
            }
        }
        __syncwarp();
        // ---- count survivors and runs per destination (tiny runs to the tiny list), finished suffixes
        u32 ns = 0, ng = 0, np = 0, ngp = 0;
        {
            u32 carry = X0;
            for (u32 xb = X0; xb < X1; xb += 32) {
                const u32 x = xb + lane;
                bool st = false, en = false;
                if (x < X1) {
                    const u32 sj = S.sg[1][x];
                    const KeyT kx = S.key[1][x];
                    st = x == S.lstart[sj] || kx != S.key[1][x - 1];
                    en = x + 1 == S.lstart[sj + 1] || kx != S.key[1][x + 1];
                }
                const u32 gfirst = max(carry, warp_incl_max(x < X1 && st ? x : 0u));
                carry = __shfl_sync(0xffffffffu, gfirst, 31);
                const bool surv = x < X1 && !(st && en);
                const bool tiny = surv && (u32)S.key[0][gfirst] <= GTINY;
                ns += __popc(__ballot_sync(0xffffffffu, surv && !tiny));
                ng += __popc(__ballot_sync(0xffffffffu, surv && !tiny && st));
                np += __popc(__ballot_sync(0xffffffffu, tiny));
                ngp += __popc(__ballot_sync(0xffffffffu, tiny && st));
            }
        }
        const u32 nres = (X1 - X0) - ns - np;
        u32 ebase = 0, sbase = 0, rbase = 0, pebase = 0, psbase = 0;
        if (lane == 0) {
            atomicAdd(&a.ctl->tile_elems[1], (u64)(X1 - X0));
            if (ns) {  // runs of 9..WARP_GROUP go to the medium list
                const u64 o = atomicAdd(&a.ctl->cnt[L_M0 + (rpar ^ 1)], ((u64)ng << 32) | ns);
                ebase = (u32)o; sbase = (u32)(o >> 32);
            }
            if (np) {
                const uint2 o = alloc_tiny(a.ctl, rpar, ngp, np);
                pebase = o.x; psbase = o.y;
            }
            if (nres) rbase = (u32)atomicAdd(&a.ctl->cnt[L_R0 + rpar], (u64)nres);
        }
        ebase = __shfl_sync(0xffffffffu, ebase, 0);
        sbase = __shfl_sync(0xffffffffu, sbase, 0);
        rbase = __shfl_sync(0xffffffffu, rbase, 0);
        pebase = __shfl_sync(0xffffffffu, pebase, 0);
        psbase = __shfl_sync(0xffffffffu, psbase, 0);
        const ListView outp = a.lists[L_P0 + (rpar ^ 1)], outm = a.lists[L_M0 + (rpar ^ 1)];
        // ---- emit
        u32 es = 0, gs = 0, ep = 0, gp = 0, rs = 0, carry = X0;  // running counts; carry: start of the open run
        for (u32 xb = X0; xb < X1; xb += 32) {
            const u32 x = xb + lane;
            const bool valid = x < X1;
            bool st = false, en = false;
            u32 sj = 0;
            if (valid) {
                sj = S.sg[1][x];
                const KeyT kx = S.key[1][x];
                st = x == S.lstart[sj] || kx != S.key[1][x - 1];
                en = x + 1 == S.lstart[sj + 1] || kx != S.key[1][x + 1];
            }
            const u32 gf = warp_incl_max(valid && st ? x : 0u);
            const u32 gfirst = max(gf, carry);
            const bool single = valid && st && en, surv = valid && !(st && en);
            const u32 len = surv ? (u32)S.key[0][gfirst] : 0u;
            const bool tiny = surv && len <= GTINY, smallg = surv && len > GTINY;
            const u32 b_s = __ballot_sync(0xffffffffu, smallg), b_gs = __ballot_sync(0xffffffffu, smallg && st);
            const u32 b_p = __ballot_sync(0xffffffffu, tiny), b_gp = __ballot_sync(0xffffffffu, tiny && st);
            const u32 b_one = __ballot_sync(0xffffffffu, single);
            const u32 my_es = es + __popc(b_s & lt_mask), my_gs = gs + __popc(b_gs & lt_mask);
            const u32 my_ep = ep + __popc(b_p & lt_mask), my_gp = gp + __popc(b_gp & lt_mask);
            const u32 my_rs = rs + __popc(b_one & lt_mask);
            if (valid) {
                const u32 id = S.val[1][x], s0 = S.lstart[sj], lh = S.lhead[sj], bd = S.lbd[sj];
                const bool unsplit = !(lh >> 31);
                if (single) {
                    resolve(a, isa_nxt, id, (lh & 0x7FFFFFFFu) + (x - s0), seg_blk(bd), res, rbase + my_rs);
                } else {
                    const u32 head = (lh & 0x7FFFFFFFu) + (gfirst - s0);
                    if (!((bd & STABLE) && unsplit)) {
                        KGB_GUARD(id < a.cap_n, &a.ctl->err, E_RANK) isa_nxt[id] = head;
                    }
                    const u32 sbd = seg_blk(bd) | (!PREFIX && !KEYED && unsplit ? STABLE : 0u);
                    if (tiny) {
                        KGB_GUARD(pebase + my_ep < a.cap_n, &a.ctl->err, E_LIST) outp.eid[pebase + my_ep] = id;
                        if (en) {
                            const u32 sidx = psbase + my_gp + (st ? 1u : 0u) - 1u;
                            Seg g;
                            g.start = pebase + my_ep + 1 - len; g.len = len; g.head = head; g.bd = sbd;
                            KGB_GUARD(sidx < a.cap_segt, &a.ctl->err, E_SEG) outp.seg[sidx] = g;
                        }
                    } else {
                        KGB_GUARD(ebase + my_es < a.cap_n, &a.ctl->err, E_LIST) outm.eid[ebase + my_es] = id;
                        if (en) {
                            const u32 sidx = sbase + my_gs + (st ? 1u : 0u) - 1u;
                            Seg g;
                            g.start = ebase + my_es + 1 - len; g.len = len; g.head = head; g.bd = sbd;
                            KGB_GUARD(sidx < a.cap_segm, &a.ctl->err, E_SEG) outm.seg[sidx] = g;
                        }
                    }
                }
            }
            es += __popc(b_s);
            gs += __popc(b_gs);
            ep += __popc(b_p);
            gp += __popc(b_gp);
            rs += __popc(b_one);
            carry = __shfl_sync(0xffffffffu, gfirst, 31);
        }
    }
}

// ------------------------------------------------------------------------------------------------ repeat chains
// Suffixes in one group have equal first characters, so they sort among themselves as their successors (each
// position + 1) do. Inside a repeat (equal stretches of text) the members of a group G move along together: their
// successors fill one group G', whose successors fill one group G'', and so on, round after round, until the
// doubling step reaches the end of the repeat, about log2(length / h) rounds later. The chain kernels order such
// groups in one step. For every tiny group of this round whose members' successors all lie in one group, each
// member's bit in cbits is set (x's chain continues at x + 1). The first clear bit e >= x1 (x1: any member) ends the
// chain: the members x_i sort as the suffixes x_i + (e - x1) + 1 do, by their current ranks, a suffix past the block
// end first (at most one member's can be: they are distinct positions inside the block). The successor sets along
// the chain are contained in single groups, so every member's chain has the same length. The step runs only where
// doubling has stalled (the round follows one that finished less than a fifth of its actives): earlier, common short
// phrases put most chains through groups whose other members leave the repeat, and the chains end undecided.
// Exclusive suffix minimum over the threads of a CTA of NT threads: thread i gets min(v_j, j > i) (0xFFFFFFFF for the
// last). sm holds NT / 32 words; the call synchronises the CTA and leaves sm free for reuse.
template <int NT>
__device__ __forceinline__ u32 block_suffix_min_excl(u32 v, u32 *sm) {
    const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32 incl = v;  // inclusive suffix minimum within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 t = __shfl_down_sync(0xffffffffu, incl, o);
        if (lane + o < 32) incl = min(incl, t);
    }
    if (lane == 0) sm[warp] = incl;  // the warp's minimum
    __syncthreads();
    u32 later = 0xFFFFFFFFu;  // minimum of the later warps
    for (u32 w = warp + 1; w < (u32)(NT / 32); w++) later = min(later, sm[w]);
    u32 excl = __shfl_down_sync(0xffffffffu, incl, 1);
    if (lane == 31) excl = 0xFFFFFFFFu;
    __syncthreads();
    return min(excl, later);
}

constexpr u32 NZ_TILE = 4096;  // words per tile of the next-zero table
constexpr u32 NZ_NONE = 0xFFFFFFFFu;

__device__ __forceinline__ bool chain_on(const FwdArgs &a) {
    const Ctl *c = a.ctl;
    return a.chain_from && c->round >= a.chain_from && c->chain_go && (u32)c->cnt[L_P0 + c->rpar] != 0;
}

__global__ void __launch_bounds__(TPB) k_chain_clear(FwdArgs a) {
    if (!chain_on(a)) return;
    for (u32 w = blockIdx.x * TPB + threadIdx.x; w < a.cwords; w += gridDim.x * TPB) a.cbits[w] = 0;
}

// Bits of the tiny groups whose members' successors all share one group.
__global__ void __launch_bounds__(TPB) k_chain_link(FwdArgs a) {
    if (!chain_on(a)) return;
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar;
    const ListView in = a.lists[L_P0 + rpar];
    const u32 nseg = min((u32)(ctl->cnt[L_P0 + rpar] >> 32), (u32)a.cap_segt), nslots = min(ctl->p_alloc, (u32)a.cap_n);
    const u32 *isa = a.isa[rpar];
    for (u32 s = blockIdx.x * TPB + threadIdx.x; s < nseg; s += gridDim.x * TPB) {
        const Seg g = in.seg[s];
        const u32 len = g.len;
        if (len < 2 || len > GTINY || (u64)g.start + len > nslots) continue;
        const u64 end = blk_end(a, seg_blk(g.bd));
        u32 v[GTINY];
        bool ok = true;
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) {
            v[q] = q < len ? in.eid[g.start + q] : 0u;
            if (q < len && (u64)v[q] + 1 >= end) ok = false;
        }
        if (!ok) continue;
        u32 r0 = 0;
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) {
            if (q >= len) break;
            const u32 r = __ldg(isa + v[q] + 1);
            if (q == 0) r0 = r; else ok = ok && r == r0;
        }
        if (!ok) continue;
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) {
            if (q >= len) break;
            if (KGB_OK((v[q] >> 5) < a.cwords, &a.ctl->err, E_RANK)) atomicOr(a.cbits + (v[q] >> 5), 1u << (v[q] & 31));
        }
    }
}

// Next-zero table, part 1: for every word w, the first word at or after w within w's tile of NZ_TILE words that has a
// clear bit (NZ_NONE if none), and per tile the first such word (ctn, NZ_NONE if none). One CTA per tile.
__global__ void __launch_bounds__(TPB) k_chain_nz(FwdArgs a) {
    if (!chain_on(a)) return;
    __shared__ u32 sm[TPB / 32];
    constexpr u32 PER = NZ_TILE / TPB;
    for (u32 t = blockIdx.x; t < a.ctiles; t += gridDim.x) {
        const u32 w0 = t * NZ_TILE + threadIdx.x * PER;
        u32 loc[PER];
        u32 nxt = NZ_NONE;  // first word with a clear bit at or after the current one, within this thread's run
#pragma unroll
        for (int q = PER - 1; q >= 0; q--) {
            const u32 w = w0 + q;
            if (w < a.cwords && a.cbits[w] != 0xFFFFFFFFu) nxt = w;
            loc[q] = nxt;
        }
        // the first such word after this thread's run: the minimum over the later threads' runs (words grow with the
        // thread index and NZ_NONE is the largest value)
        const u32 after = block_suffix_min_excl<TPB>(nxt, sm);
#pragma unroll
        for (int q = 0; q < (int)PER; q++) {
            const u32 w = w0 + q;
            if (w < a.cwords) a.cnz[w] = loc[q] != NZ_NONE ? loc[q] : after;
        }
        if (threadIdx.x == 0) a.ctn[t] = nxt != NZ_NONE ? nxt : after;
        __syncthreads();
    }
}

// Next-zero table, part 2 (one CTA): ctn[t] = the first word with a clear bit in tiles t, t + 1, ... (a suffix
// minimum over the tiles); ctn[ctiles] is the last word, which is never set.
__global__ void __launch_bounds__(1024) k_chain_tiles(FwdArgs a) {
    if (!chain_on(a)) return;
    __shared__ u32 sm[1024 / 32];
    const u32 nt = a.ctiles;
    const u32 per = (nt + 1023) / 1024;
    const u32 t0 = threadIdx.x * per;
    u32 nxt = NZ_NONE;
    for (int q = (int)per - 1; q >= 0; q--) {
        const u32 t = t0 + q;
        if (t < nt && a.ctn[t] != NZ_NONE) nxt = a.ctn[t];
    }
    u32 after = block_suffix_min_excl<1024>(nxt, sm);
    if (after == NZ_NONE) after = a.cwords - 1;
    for (int q = (int)per - 1; q >= 0; q--) {
        const u32 t = t0 + q;
        if (t < nt) {
            if (a.ctn[t] != NZ_NONE) after = a.ctn[t];
            a.ctn[t] = after;
        }
    }
    if (threadIdx.x == 0) a.ctn[nt] = a.cwords - 1;
}

// The end of x's chain: the first id e >= x whose bit is clear.
__device__ __forceinline__ u32 chain_end(const FwdArgs &a, u32 x) {
    const u32 w = x >> 5;
    const u32 z = ~a.cbits[w] & (~0u << (x & 31));
    if (z) return (w << 5) + __ffs(z) - 1;
    u32 w2 = w + 1 < a.cwords ? a.cnz[w + 1] : a.cwords - 1;
    if (w2 == NZ_NONE) w2 = a.ctn[(w + 1) / NZ_TILE + 1];
    if (!KGB_OK(w2 < a.cwords, &a.ctl->err, E_RANK)) return x;
    return (w2 << 5) + __ffs(~a.cbits[w2]) - 1;
}

// The chain key of member x of a group whose chain has length d (this round's ranks isa): 0 for a suffix whose
// position x + d + 1 lies past the block end (the shorter suffix sorts first), else 1 + the rank there.
__device__ __forceinline__ u32 chain_key(const u32 *__restrict__ isa, u32 x, u32 d, u64 end) {
    const u64 f = (u64)x + d + 1;
    return f >= end ? 0u : __ldg(isa + f) + 1u;
}

// ------------------------------------------------------------------------------------------------ tiny groups
// Rank rounds: one thread per group of at most GTINY suffixes. The thread gathers the group's keys into registers,
// sorts them with a sorting network (2, 4 or 8 inputs, the widest group of the warp decides), and emits ranks,
// finished suffixes and the surviving runs, which are tiny again; allocations are aggregated per warp.

__device__ __forceinline__ void cswap(u32 &ka, u32 &va, u32 &kb, u32 &vb) {
    const bool sw = kb < ka;
    const u32 tk = sw ? kb : ka, tv = sw ? vb : va;
    kb = sw ? ka : kb;
    vb = sw ? va : vb;
    ka = tk;
    va = tv;
}
#define KGB_CS(i, j) cswap(k[i], v[i], k[j], v[j])

__global__ void __launch_bounds__(TPB, 4) k_group_thread(FwdArgs a) {
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, h = ctl->h;
    // in and out share the id array: a group's ids stay in its slots; only descriptors move to the next list
    const ListView in = a.lists[L_P0 + rpar], out = a.lists[L_P0 + (rpar ^ 1)], res = a.lists[L_R0 + rpar];
    const u64 c = ctl->cnt[L_P0 + rpar];
    const u32 nseg = (u32)(c >> 32), nslots = ctl->p_alloc;
    if ((u32)c > a.cap_n || nseg > a.cap_segt || nslots > a.cap_n) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 *isa_cur = a.isa[rpar];
    u32 *isa_nxt = a.isa[rpar ^ 1];
    u32 *ids = in.eid;
    const u32 lane = lane_id();
    const u32 stride = gridDim.x * TPB;
    // software pipeline over the thread's groups: the next group's descriptor is loaded when this one starts, and
    // its ids once this group's keys are in flight
    Seg gq = {0, 0, 0, 0};
    u32 vq[GTINY];
    if (blockIdx.x * TPB + threadIdx.x < nseg) gq = in.seg[blockIdx.x * TPB + threadIdx.x];
    for (u32 base = blockIdx.x * TPB; base < nseg; base += stride) {
        const u32 s = base + threadIdx.x;
        const bool ok = s < nseg;
        Seg g = {0, 0, 0, 0};
        if (ok) g = gq;
        if (s + stride < nseg) gq = in.seg[s + stride];
        u32 len = g.len;
        if (len > GTINY || (u64)g.start + len > nslots) {  // broken list invariant: report, never overrun
            atomicOr(&a.ctl->err, E_SEG);
            len = 0;
        }
        const u32 b = seg_blk(g.bd);
        const u64 end = len ? blk_end(a, b) : 0;
        u32 k[GTINY], v[GTINY];
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) v[q] = q < len ? (base == blockIdx.x * TPB ? ids[g.start + q] : vq[q]) : 0u;
        // In a round that follows repeat chains, a group whose chain is at least h long would come out of doubling
        // whole (its members' positions + h share one group); its chain key, the rank d + 1 positions on, orders it
        // at least as far, so it takes that key instead (one gather per member either way). Shorter chains, and
        // rounds without chains, take the doubling key.
        u32 d = 0;
        if (len >= 2 && chain_on(a)) d = chain_end(a, v[0]) - v[0];
        const bool by_chain = d >= h;
#pragma unroll
        for (u32 q = 0; q < GTINY; q++)
            k[q] = q >= len ? 0xFFFFFFFFu : by_chain ? chain_key(isa_cur, v[q], d, end) : rank_key(isa_cur, v[q], h, end);
        {
            const u32 lq = gq.len <= GTINY && (u64)gq.start + gq.len <= nslots && s + stride < nseg ? gq.len : 0u;
#pragma unroll
            for (u32 q = 0; q < GTINY; q++) vq[q] = q < lq ? ids[gq.start + q] : 0u;
        }
        const u32 mlen = __reduce_max_sync(0xffffffffu, len);
        if (mlen <= 2) {
            KGB_CS(0, 1);
        } else if (mlen <= 4) {
            KGB_CS(0, 1); KGB_CS(2, 3); KGB_CS(0, 2); KGB_CS(1, 3); KGB_CS(1, 2);
        } else {
            KGB_CS(0, 1); KGB_CS(2, 3); KGB_CS(4, 5); KGB_CS(6, 7);
            KGB_CS(0, 2); KGB_CS(1, 3); KGB_CS(4, 6); KGB_CS(5, 7);
            KGB_CS(1, 2); KGB_CS(5, 6);
            KGB_CS(0, 4); KGB_CS(1, 5); KGB_CS(2, 6); KGB_CS(3, 7);
            KGB_CS(2, 4); KGB_CS(3, 5);
            KGB_CS(1, 2); KGB_CS(3, 4); KGB_CS(5, 6);
        }
        // runs of equal keys: survivors (runs of two or more), their runs, finished suffixes
        u32 ns = 0, ng = 0, n1 = 0;
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) {
            if (q >= len) break;
            const bool st = q == 0 || k[q] != k[q - 1];
            const bool en = q + 1 == len || k[q] != k[q + 1];
            if (st && en) n1++;
            else { ns++; ng += st; }
        }
        const bool unsplit = ng == 1 && ns == len;  // one run covers the group
        const u32 pk = ng | (n1 << 16);  // each at most GTINY per thread: warp totals <= 256
        const u32 incl = warp_incl_sum(pk), tot = __shfl_sync(0xffffffffu, incl, 31), excl = incl - pk;
        const u32 ts = warp_sum(ns);
        u32 sbase = 0, rbase = 0;
        if (lane == 0) {
            const u32 tg = tot & 0xFFFF, t1 = tot >> 16;
            if (tg) sbase = (u32)(atomicAdd(&a.ctl->cnt[L_P0 + (rpar ^ 1)], ((u64)tg << 32) | ts) >> 32);
            if (t1) rbase = (u32)atomicAdd(&a.ctl->cnt[L_R0 + rpar], (u64)t1);
        }
        u32 gi = __shfl_sync(0xffffffffu, sbase, 0) + (excl & 0xFFFF);
        u32 r = __shfl_sync(0xffffffffu, rbase, 0) + (excl >> 16);
        const bool skip_rank = (g.bd & STABLE) && unsplit;
        // the L-column bytes of the finished suffixes, all loads in flight before any write
        BlockInfo bi{};
        u8 tv[GTINY];
        if (n1) bi = a.blk[b];
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) {
            tv[q] = 0;
            if (q >= len) continue;
            const bool st = q == 0 || k[q] != k[q - 1];
            const bool en = q + 1 == len || k[q] != k[q + 1];
            if (st && en && v[q] != bi.off) tv[q] = __ldg(a.T + v[q] - 1);
        }
        // a group that split is rewritten in sorted order, so that each surviving run is contiguous in its slots
        if (!unsplit && len) {
#pragma unroll
            for (u32 q = 0; q < GTINY; q++)
                if (q < len) ids[g.start + q] = v[q];
        }
        u32 rs = 0;  // first position of the current run
#pragma unroll
        for (u32 q = 0; q < GTINY; q++) {
            if (q >= len) break;
            const bool st = q == 0 || k[q] != k[q - 1];
            const bool en = q + 1 == len || k[q] != k[q + 1];
            if (st) rs = q;
            if (st && en) {
                resolve_byte(a, isa_nxt, v[q], g.head + q, b, bi, res, r++, tv[q]);
                continue;
            }
            const u32 head = g.head + rs;
            if (!skip_rank) {
                KGB_GUARD(v[q] < a.cap_n, &a.ctl->err, E_RANK) isa_nxt[v[q]] = head;
            }
            if (en) {
                Seg ng_;
                ng_.len = q - rs + 1; ng_.start = g.start + rs; ng_.head = head;
                ng_.bd = b | (unsplit ? STABLE : 0u);
                KGB_GUARD(gi < a.cap_segt, &a.ctl->err, E_SEG) out.seg[gi] = ng_;
                gi++;
            }
        }
    }
}
#undef KGB_CS

// ------------------------------------------------------------------------------------------------ medium groups
// Rank rounds: one warp per group of GTINY+1..GMED suffixes. A flat pass first gathers every member's raw key
// rank(i + h) into a scratch array in list order (all loads independent); the group's warp then loads ids and raw keys
// with coalesced reads, corrects the keys of suffixes whose i + h lies past their block, sorts in its shared-memory
// slice (counting for groups of up to 32, bitonic network otherwise), and walks the sorted runs twice: once for their
// lengths and offsets in the next lists, once to emit ranks, finished suffixes and runs (tiny ones to the tiny list,
// the others to the medium list).

// Raw keys of the medium list: mkey[x] = ISA[eid[x] + h] (clamped into the rank buffer; corrected per block later).
__global__ void __launch_bounds__(TPB) k_mkeys(FwdArgs a) {
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, h = ctl->h;
    const ListView in = a.lists[L_M0 + rpar];
    const u32 nelem = min((u32)ctl->cnt[L_M0 + rpar], (u32)a.cap_n);
    const u32 *isa_cur = a.isa[rpar];
    u32 *mk = a.lval[0];
    for (u32 x = blockIdx.x * TPB + threadIdx.x; x < nelem; x += gridDim.x * TPB) {
        const u64 j = (u64)in.eid[x] + h;
        mk[x] = j < a.cap_n ? __ldg(isa_cur + j) : 0u;
    }
}

struct GWarpSmem {
    u32 key[2][GMED];  // [1]: keys being sorted / sorted; [0]: run lengths and offsets after the sort
    u32 val[2][GMED];
};

__global__ void __launch_bounds__(TPB) k_group_warp(FwdArgs a) {
    __shared__ GWarpSmem SM[TPB / 32];
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, h = ctl->h;
    const ListView in = a.lists[L_M0 + rpar], outm = a.lists[L_M0 + (rpar ^ 1)], outp = a.lists[L_P0 + (rpar ^ 1)];
    const ListView res = a.lists[L_R0 + rpar];
    const u64 c = ctl->cnt[L_M0 + rpar];
    const u32 nelem = (u32)c, nseg = (u32)(c >> 32);
    if (nelem > a.cap_n || nseg > a.cap_segm) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 *mk = a.lval[0];
    u32 *isa_nxt = a.isa[rpar ^ 1];
    const u32 lane = lane_id(), lt = lanemask_lt();
    GWarpSmem &W = SM[warp_id()];
    u32 *K = W.key[1], *V = W.val[1];
    u16 *RL = reinterpret_cast<u16 *>(W.key[0]);  // run length at the run's first sorted position
    u16 *RO = RL + GMED;                           // run's element offset within its destination
    u16 *RG = reinterpret_cast<u16 *>(W.val[0]);   // run's segment offset within its destination
    const u32 gw = blockIdx.x * (TPB / 32) + warp_id(), nw = gridDim.x * (TPB / 32);
    for (u32 s = gw; s < nseg; s += nw) {
        const Seg g = in.seg[s];
        const u32 len = g.len;
        if (len > GMED || len < 2 || (u64)g.start + len > nelem) {  // broken list invariant: report, skip
            if (lane == 0) atomicOr(&a.ctl->err, E_SEG);
            continue;
        }
        const u32 b = seg_blk(g.bd);
        const u64 end = blk_end(a, b);
        if (len <= 32) {
            // ---- counting sort, one member per lane (position = keys below + equal keys before)
            u32 id = 0, kx = 0xFFFFFFFFu;
            if (lane < len) {
                id = in.eid[g.start + lane];
                const u32 d = (u32)(end - id);
                kx = h < d ? mk[g.start + lane] + h : d - 1;
            }
            u32 below = 0;
            for (u32 y = 0; y < len; y++) {
                const u32 ky = __shfl_sync(0xffffffffu, kx, y);
                below += ky < kx || (ky == kx && y < lane);
            }
            if (lane < len) { K[below] = kx; V[below] = id; }
        } else {
            // ---- bitonic sort of the group padded to a power of two (padding keys sort last)
            const u32 p2 = 1u << (32 - __clz(len - 1));
            for (u32 q = lane; q < p2; q += 32) {
                u32 id = 0, kx = 0xFFFFFFFFu;
                if (q < len) {
                    id = in.eid[g.start + q];
                    const u32 d = (u32)(end - id);
                    kx = h < d ? mk[g.start + q] + h : d - 1;
                }
                K[q] = kx;
                V[q] = id;
            }
            __syncwarp();
            for (u32 k = 2; k <= p2; k <<= 1) {
                for (u32 j = k >> 1; j > 0; j >>= 1) {
                    for (u32 t = lane; t < p2 / 2; t += 32) {
                        const u32 i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i + j;
                        const u32 ki = K[i], kl = K[l];
                        if ((ki > kl) == ((i & k) == 0) && ki != kl) {
                            const u32 vi = V[i];
                            K[i] = kl; K[l] = ki;
                            V[i] = V[l]; V[l] = vi;
                        }
                    }
                    __syncwarp();
                }
            }
        }
        __syncwarp();
        const bool unsplit = K[0] == K[len - 1];
        // ---- runs: lengths and offsets (per destination) at each run's first position
        u32 carry = 0, off_p = 0, off_m = 0, g_p = 0, g_m = 0, n1 = 0;
        for (u32 c0 = 0; c0 < len; c0 += 32) {
            const u32 q = c0 + lane;
            const bool valid = q < len;
            bool st = false, en = false;
            if (valid) {
                const u32 kq = K[q];
                st = q == 0 || kq != K[q - 1];
                en = q + 1 == len || kq != K[q + 1];
            }
            const u32 gf = max(carry, warp_incl_max(valid && st ? q : 0u));
            const u32 rl = valid && en ? q - gf + 1 : 0u;
            const u32 pe = rl >= 2 && rl <= GTINY ? rl : 0u, me = rl > GTINY ? rl : 0u;
            const u32 pei = warp_incl_sum(pe), mei = warp_incl_sum(me);
            const u32 bp = __ballot_sync(0xffffffffu, pe != 0), bm = __ballot_sync(0xffffffffu, me != 0);
            const u32 b1 = __ballot_sync(0xffffffffu, rl == 1);
            if (rl >= 2) {
                RL[gf] = (u16)rl;
                RO[gf] = (u16)(pe ? off_p + pei - pe : off_m + mei - me);
                RG[gf] = (u16)(pe ? g_p + __popc(bp & lt) : g_m + __popc(bm & lt));
            }
            off_p += __shfl_sync(0xffffffffu, pei, 31);
            off_m += __shfl_sync(0xffffffffu, mei, 31);
            g_p += __popc(bp);
            g_m += __popc(bm);
            n1 += __popc(b1);
            carry = __shfl_sync(0xffffffffu, gf, 31);
        }
        u32 pb = 0, psb = 0, mb = 0, msb = 0, rb = 0;
        if (lane == 0) {
            if (off_p) { const uint2 o = alloc_tiny(a.ctl, rpar, g_p, off_p); pb = o.x; psb = o.y; }
            if (off_m) { const u64 o = atomicAdd(&a.ctl->cnt[L_M0 + (rpar ^ 1)], ((u64)g_m << 32) | off_m); mb = (u32)o; msb = (u32)(o >> 32); }
            if (n1) rb = (u32)atomicAdd(&a.ctl->cnt[L_R0 + rpar], (u64)n1);
        }
        pb = __shfl_sync(0xffffffffu, pb, 0); psb = __shfl_sync(0xffffffffu, psb, 0);
        mb = __shfl_sync(0xffffffffu, mb, 0); msb = __shfl_sync(0xffffffffu, msb, 0);
        rb = __shfl_sync(0xffffffffu, rb, 0);
        __syncwarp();
        // ---- emit
        const bool skip_rank = (g.bd & STABLE) && unsplit;
        const u32 sbd = b | (unsplit ? STABLE : 0u);
        carry = 0;
        u32 r1 = 0;
        for (u32 c0 = 0; c0 < len; c0 += 32) {
            const u32 q = c0 + lane;
            const bool valid = q < len;
            bool st = false, en = false;
            if (valid) {
                const u32 kq = K[q];
                st = q == 0 || kq != K[q - 1];
                en = q + 1 == len || kq != K[q + 1];
            }
            const u32 gf = max(carry, warp_incl_max(valid && st ? q : 0u));
            carry = __shfl_sync(0xffffffffu, gf, 31);
            const bool single = valid && st && en;
            const u32 b1 = __ballot_sync(0xffffffffu, single);
            const u32 my1 = r1 + __popc(b1 & lt);
            r1 += __popc(b1);
            if (!valid) continue;
            const u32 id = V[q];
            if (single) {
                resolve(a, isa_nxt, id, g.head + q, b, res, rb + my1);
                continue;
            }
            const u32 head = g.head + gf;
            if (!skip_rank) {
                KGB_GUARD(id < a.cap_n, &a.ctl->err, E_RANK) isa_nxt[id] = head;
            }
            const u32 rl = RL[gf], ro = RO[gf], rg = RG[gf];
            const bool tiny = rl <= GTINY;
            const ListView &o = tiny ? outp : outm;
            const u32 eb = (tiny ? pb : mb) + ro;
            KGB_GUARD(eb + (q - gf) < a.cap_n, &a.ctl->err, E_LIST) o.eid[eb + (q - gf)] = id;
            if (en) {
                Seg ng_;
                ng_.start = eb; ng_.len = rl; ng_.head = head; ng_.bd = sbd;
                const u32 si = (tiny ? psb : msb) + rg;
                KGB_GUARD(si < (tiny ? a.cap_segt : a.cap_segm), &a.ctl->err, E_SEG) o.seg[si] = ng_;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------------------ bucket passes
// Work lists of large groups are tiled by TSM elements; every group is longer than TSM, so a tile meets at most
// two. tmap[t] = the group containing element t * TSM.

struct MsdTile {
    u32 s0, s1, bound, d0, d1;
    Seg g0, g1;
};

template <bool PREFIX>
__device__ __forceinline__ void msd_tile_info(const FwdArgs &a, const ListView &in, u32 nseg, u32 t, bool first,
                                              MsdTile &m) {
    m.s0 = in.tmap[t];
    if (m.s0 >= nseg) {  // broken tile map: report and use a valid index (the round result is discarded)
        atomicOr(&a.ctl->err, E_TMAP);
        m.s0 = 0;
    }
    m.g0 = in.seg[m.s0];
    m.bound = m.g0.start + m.g0.len;
    m.s1 = m.s0 + 1 < nseg ? m.s0 + 1 : m.s0;
    m.g1 = in.seg[m.s1];
    if (!PREFIX && first) {
        m.d0 = depth_from_vary(a.orand[2 * m.s0], a.orand[2 * m.s0 + 1]);
        m.d1 = depth_from_vary(a.orand[2 * m.s1], a.orand[2 * m.s1 + 1]);
    } else {
        m.d0 = seg_depth(m.g0.bd);
        m.d1 = seg_depth(m.g1.bd);
    }
}

template <bool PREFIX>
__device__ __forceinline__ u32 msd_digit(const FwdArgs &a, const ListView &in, u32 x, u32 id, const Seg &g, u32 d,
                                         u32 *key) {
    if (PREFIX) {
        const BlockInfo B = a.blk[seg_blk(g.bd)];
        return prefix_byte(a.T, id, d, (u64)B.off + B.n);
    }
    *key = in.ekey[x];
    return (*key >> (24 - 8 * d)) & 0xFF;
}

// Rank rounds, first pass: gather the keys of the large groups and the OR/AND of each group's keys.
__global__ void __launch_bounds__(TPB) k_keygen(FwdArgs a) {
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, h = ctl->h;
    const ListView in = a.lists[L_L0 + rpar];
    const u64 c = ctl->cnt[L_L0 + rpar];
    const u32 nelem = (u32)c, nseg = (u32)(c >> 32);
    if (nelem > a.cap_n || nseg > a.cap_segl) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 ntiles = (nelem + TSM - 1) / TSM;
    const u32 *isa = a.isa[rpar];
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const u32 s0 = in.tmap[t];
        if (s0 >= nseg) { if (threadIdx.x == 0) atomicOr(&a.ctl->err, E_TMAP); continue; }
        const Seg g0 = in.seg[s0];
        const u32 bound = g0.start + g0.len, s1 = s0 + 1 < nseg ? s0 + 1 : s0;
        const Seg g1 = in.seg[s1];
        const BlockInfo B0 = a.blk[seg_blk(g0.bd)], B1 = a.blk[seg_blk(g1.bd)];
        u32 or0 = 0, and0 = ~0u, or1 = 0, and1 = ~0u;
#pragma unroll
        for (int j = 0; j < IPM; j++) {
            const u32 x = t * TSM + j * TPB + threadIdx.x;
            if (x < nelem) {
                const bool sel = x >= bound;
                const BlockInfo &B = sel ? B1 : B0;
                const u32 id = in.eid[x];
                const u32 key = rank_key(isa, id, h, (u64)B.off + B.n);
                in.ekey[x] = key;
                if (sel) { or1 |= key; and1 &= key; } else { or0 |= key; and0 &= key; }
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            or0 |= __shfl_xor_sync(0xffffffffu, or0, o);
            and0 &= __shfl_xor_sync(0xffffffffu, and0, o);
            or1 |= __shfl_xor_sync(0xffffffffu, or1, o);
            and1 &= __shfl_xor_sync(0xffffffffu, and1, o);
        }
        if (lane_id() == 0) {
            if (or0 || and0 != ~0u) { atomicOr(&a.orand[2 * s0], or0); atomicAnd(&a.orand[2 * s0 + 1], and0); }
            if (s1 != s0 && (or1 || and1 != ~0u)) { atomicOr(&a.orand[2 * s1], or1); atomicAnd(&a.orand[2 * s1 + 1], and1); }
        }
    }
}

__device__ __forceinline__ const ListView &msd_in(const FwdArgs &a, u32 rpar, u32 pass, u32 *lid) {
    *lid = pass == 0 ? L_L0 + rpar : L_K0 + ((pass - 1) & 1);
    return a.lists[*lid];
}

template <bool PREFIX>
__global__ void __launch_bounds__(TPB) k_msd_hist(FwdArgs a) {
    __shared__ u32 hs[2][256];
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, pass = ctl->pass;
    u32 lid;
    const ListView in = msd_in(a, rpar, pass, &lid);
    const u64 c = ctl->cnt[lid];
    const u32 nelem = (u32)c, nseg = (u32)(c >> 32);
    if (nelem > a.cap_n || nseg > a.cap_segl) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 ntiles = (nelem + TSM - 1) / TSM;
    const u32 lane = lane_id();
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        for (int i = threadIdx.x; i < 512; i += TPB) (&hs[0][0])[i] = 0;
        MsdTile m;
        msd_tile_info<PREFIX>(a, in, nseg, t, pass == 0, m);
        __syncthreads();
        u64 or0 = 0, and0 = ~0ull, or1 = 0, and1 = ~0ull;  // prefix rounds: which prefix bytes vary per group
#pragma unroll
        for (int j = 0; j < IPM; j++) {
            const u32 x = t * TSM + j * TPB + threadIdx.x;
            const bool valid = x < nelem;
            u32 kk = 0xFFFFFFFFu;
            if (valid) {
                const bool sel = x >= m.bound;
                const u32 id = in.eid[x];
                u32 d;
                if (PREFIX) {
                    const BlockInfo B = a.blk[seg_blk((sel ? m.g1 : m.g0).bd)];
                    u64 pk = load_be64(a.T, id);
                    const u64 rem = (u64)B.off + B.n - id;
                    if (rem < 8) pk &= ~0ull << (8 * (8 - rem));
                    d = (u32)(pk >> (56 - 8 * (sel ? m.d1 : m.d0))) & 0xFF;
                    if (sel) { or1 |= pk; and1 &= pk; } else { or0 |= pk; and0 &= pk; }
                } else {
                    u32 key;
                    d = msd_digit<PREFIX>(a, in, x, id, sel ? m.g1 : m.g0, sel ? m.d1 : m.d0, &key);
                }
                kk = ((u32)sel << 8) | d;
            }
            const u32 peers = __match_any_sync(0xffffffffu, kk);
            if (valid && (__ffs(peers) - 1) == (int)lane) atomicAdd(&(&hs[0][0])[kk], __popc(peers));
        }
        if (PREFIX) {
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                or0 |= __shfl_xor_sync(0xffffffffu, or0, o);
                and0 &= __shfl_xor_sync(0xffffffffu, and0, o);
                or1 |= __shfl_xor_sync(0xffffffffu, or1, o);
                and1 &= __shfl_xor_sync(0xffffffffu, and1, o);
            }
            if (lane == 0) {
                if (or0 || and0 != ~0ull) { atomicOr(&a.orand64[2 * m.s0], or0); atomicAnd(&a.orand64[2 * m.s0 + 1], and0); }
                if (m.s1 != m.s0 && (or1 || and1 != ~0ull)) {
                    atomicOr(&a.orand64[2 * m.s1], or1);
                    atomicAnd(&a.orand64[2 * m.s1 + 1], and1);
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 512; i += TPB) {
            const u32 cc = (&hs[0][0])[i];
            if (cc) {
                const u32 sx = i < 256 ? m.s0 : m.s1;
                KGB_GUARD(sx < a.cap_segl, &a.ctl->err, E_HIST) atomicAdd(&a.hist[(u64)sx * 256 + (i & 255)], cc);
            }
        }
        __syncthreads();
    }
}

struct ScanSmem {
    u32 ws[TPB / 32 + 1];
    u32 base_e[5], base_s[5];
    u32 nb_off[TPB];
    u32 t0[TPB];
    u32 sidx[TPB];
    u8 cls[TPB];
};

// One CTA per group of the pass: bucket sizes -> class, destination and descriptors of every bucket.
template <bool PREFIX>
__global__ void __launch_bounds__(TPB) k_msd_scan(FwdArgs a) {
    __shared__ ScanSmem S;
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, pass = ctl->pass;
    u32 lid;
    const ListView in = msd_in(a, rpar, pass, &lid);
    const u32 nseg = min((u32)(ctl->cnt[lid] >> 32), (u32)a.cap_segl);
    const u32 lko = L_K0 + (pass & 1), lln = L_L0 + (rpar ^ 1);
    const u32 tid = threadIdx.x;
    for (u32 s = blockIdx.x; s < nseg; s += gridDim.x) {
        if (s >= a.cap_segl) { if (tid == 0) atomicOr(&a.ctl->err, E_HIST); break; }
        const Seg g = in.seg[s];
        u32 d;
        if (!PREFIX && pass == 0) {
            d = depth_from_vary(a.orand[2 * s], a.orand[2 * s + 1]);
        } else {
            d = seg_depth(g.bd);
        }
        const u64 hrow = (u64)s * 256;
        const u32 cc = a.hist[hrow + tid];
        a.hist[hrow + tid] = 0;
        const u32 excl = block_excl_sum<TPB>(cc, S.ws, nullptr);
        u32 nd = d + 1;
        const u32 maxd = PREFIX ? DEPTH_PREFIX : DEPTH_RANK;
        if (PREFIX) {
            // the next depth skips prefix bytes that are the same in the whole group (all of them: the group is final)
            const u64 vary = a.orand64[2 * s] ^ a.orand64[2 * s + 1];
            while (nd < DEPTH_PREFIX && !((vary >> (56 - 8 * nd)) & 0xFF)) nd++;
        }
        u8 cls = cc == 0 ? C_NONE : cc == 1 ? C_ONE : cc <= a.smax ? C_KS : nd >= maxd ? C_LN : C_KO;
        // element and segment counts per class (singletons need only a resolved-list slot)
        u32 e_ks = cls == C_KS ? cc : 0, e_ko = cls == C_KO ? cc : 0, e_ln = cls == C_LN ? cc : 0;
        u32 tks, tko, tln, tone;
        const u32 x_ks = block_excl_sum<TPB>(e_ks, S.ws, &tks);
        const u32 x_ko = block_excl_sum<TPB>(e_ko, S.ws, &tko);
        const u32 x_ln = block_excl_sum<TPB>(e_ln, S.ws, &tln);
        const u32 spack = (cls == C_KS) | ((u32)(cls == C_KO) << 10) | ((u32)(cls == C_LN) << 20);
        u32 tsp;
        const u32 x_sp = block_excl_sum<TPB>(spack, S.ws, &tsp);
        const u32 x_one = block_excl_sum<TPB>(cls == C_ONE, S.ws, &tone);
        if (tid == 0) {
            if (tks) { u64 o = atomicAdd(&a.ctl->cnt[L_KS], ((u64)(tsp & 1023) << 32) | tks); S.base_e[C_KS] = (u32)o; S.base_s[C_KS] = (u32)(o >> 32); }
            if (tko) { u64 o = atomicAdd(&a.ctl->cnt[lko], ((u64)((tsp >> 10) & 1023) << 32) | tko); S.base_e[C_KO] = (u32)o; S.base_s[C_KO] = (u32)(o >> 32); }
            if (tln) { u64 o = atomicAdd(&a.ctl->cnt[lln], ((u64)((tsp >> 20) & 1023) << 32) | tln); S.base_e[C_LN] = (u32)o; S.base_s[C_LN] = (u32)(o >> 32); }
            if (tone) { S.base_e[C_ONE] = (u32)atomicAdd(&a.ctl->cnt[L_R0 + rpar], (u64)tone); }
        }
        __syncthreads();
        const u32 head = g.head + excl, blk = seg_blk(g.bd);
        u32 nb = 0, t0 = 0, sidx = 0;
        if (cls == C_ONE) {
            a.cursor[hrow + tid] = S.base_e[C_ONE] + x_one;  // slot in the resolved list
        } else if (cls != C_NONE) {
            u32 start;
            ListView o;
            u32 bd = blk;
            if (cls == C_KS) { start = S.base_e[C_KS] + x_ks; sidx = S.base_s[C_KS] + (x_sp & 1023); o = a.lists[L_KS]; }
            else if (cls == C_KO) { start = S.base_e[C_KO] + x_ko; sidx = S.base_s[C_KO] + ((x_sp >> 10) & 1023); o = a.lists[lko]; bd |= nd << 24; }
            else { start = S.base_e[C_LN] + x_ln; sidx = S.base_s[C_LN] + ((x_sp >> 20) & 1023); o = a.lists[lln]; }
            Seg ng;
            ng.start = start; ng.len = cc; ng.head = head; ng.bd = bd;
            KGB_GUARD(sidx < (cls == C_KS ? a.cap_segk : a.cap_segl) && (u64)start + cc <= a.cap_n, &a.ctl->err, E_SEG)
            o.seg[sidx] = ng;
            a.cursor[hrow + tid] = start;
            if (cls == C_KS) {
                write_tmap_small(a, o.tmap, a.smax, start, cc, sidx);
                if (cc > WARP_GROUP) o.tbig[start / a.smax] = ctl->round;
            } else {
                t0 = (start + TSM - 1) / TSM;
                const u32 t1 = (u32)(((u64)start + cc - 1) / TSM);
                nb = t1 >= t0 ? t1 - t0 + 1 : 0;
            }
        }
        a.bhead[hrow + tid] = head;
        a.dest[hrow + tid] = cls;
        __syncthreads();  // every thread has read orand64[s]
        if (PREFIX && tid == 0) { a.orand64[2 * s] = 0; a.orand64[2 * s + 1] = ~0ull; }
        if (!PREFIX && pass == 0 && tid == 0) {  // the scatter reads the digit from the descriptor
            a.orand[2 * s] = 0;
            a.orand[2 * s + 1] = ~0u;
            in.seg[s].bd = blk | (d << 24);
        }
        // tile-map entries of the large buckets, spread over the CTA
        u32 nbt;
        const u32 nbx = block_excl_sum<TPB>(nb, S.ws, &nbt);
        S.nb_off[tid] = nbx; S.t0[tid] = t0; S.sidx[tid] = sidx; S.cls[tid] = cls;
        __syncthreads();
        for (u32 q = tid; q < nbt; q += TPB) {
            u32 lo = 0, hh = TPB - 1;  // last bucket with nb_off <= q and a nonzero count
            while (lo < hh) {
                u32 mid = (lo + hh + 1) >> 1;
                if (S.nb_off[mid] <= q) lo = mid; else hh = mid - 1;
            }
            // the last bucket whose range starts at or before q owns q (later buckets start past it)
            ListView o = a.lists[S.cls[lo] == C_KO ? lko : lln];
            const u32 ti = S.t0[lo] + (q - S.nb_off[lo]);
            KGB_GUARD(ti < a.cap_tml, &a.ctl->err, E_TMAP) o.tmap[ti] = S.sidx[lo];
        }
        __syncthreads();
    }
}

template <bool PREFIX>
__global__ void __launch_bounds__(TPB) k_msd_scatter(FwdArgs a) {
    __shared__ u32 cnt[2][256];
    __shared__ u32 base[2][256];
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar, pass = ctl->pass;
    u32 lid;
    const ListView in = msd_in(a, rpar, pass, &lid);
    const u64 c = ctl->cnt[lid];
    const u32 nelem = (u32)c, nseg = (u32)(c >> 32);
    if (nelem > a.cap_n || nseg > a.cap_segl) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctl->err, E_LIST);
        return;
    }
    const u32 ntiles = (nelem + TSM - 1) / TSM;
    const ListView ks = a.lists[L_KS], ko = a.lists[L_K0 + (pass & 1)], ln = a.lists[L_L0 + (rpar ^ 1)];
    const ListView res = a.lists[L_R0 + rpar];
    u32 *isa_nxt = a.isa[rpar ^ 1];
    const u32 lane = lane_id();
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        for (int i = threadIdx.x; i < 512; i += TPB) (&cnt[0][0])[i] = 0;
        MsdTile m;
        msd_tile_info<PREFIX>(a, in, nseg, t, false, m);  // digits come from the descriptors the scan updated
        __syncthreads();
        u32 kk[IPM], slot[IPM], ids[IPM], keys[IPM];
#pragma unroll
        for (int j = 0; j < IPM; j++) {
            const u32 x = t * TSM + j * TPB + threadIdx.x;
            const bool valid = x < nelem;
            kk[j] = 0xFFFFFFFFu;
            if (valid) {
                const bool sel = x >= m.bound;
                ids[j] = in.eid[x];
                const u32 d = msd_digit<PREFIX>(a, in, x, ids[j], sel ? m.g1 : m.g0, sel ? m.d1 : m.d0, &keys[j]);
                kk[j] = ((u32)sel << 8) | d;
            }
            const u32 peers = __match_any_sync(0xffffffffu, kk[j]);
            const int leader = __ffs(peers) - 1;
            u32 old = 0;
            if (valid && leader == (int)lane) old = atomicAdd(&(&cnt[0][0])[kk[j]], __popc(peers));
            old = __shfl_sync(0xffffffffu, old, leader);
            slot[j] = old + __popc(peers & lanemask_lt());
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 512; i += TPB) {
            const u32 cc = (&cnt[0][0])[i];
            if (cc) {
                const u64 row = (u64)(i < 256 ? m.s0 : m.s1) * 256 + (i & 255);
                (&base[0][0])[i] = a.dest[row] == C_ONE ? a.cursor[row] : atomicAdd(&a.cursor[row], cc);
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < IPM; j++) {
            if (kk[j] == 0xFFFFFFFFu) continue;
            const u32 sel = kk[j] >> 8, d = kk[j] & 255;
            const u64 row = (u64)(sel ? m.s1 : m.s0) * 256 + d;
            const u8 cls = a.dest[row];
            const u32 pos = (&base[0][0])[kk[j]] + slot[j];
            const u32 id = ids[j];
            if (!KGB_OK(pos < a.cap_n && id < a.cap_n, &a.ctl->err, E_LIST)) continue;
            if (cls == C_KS) {
                ks.eid[pos] = id;
                if (!PREFIX) ks.ekey[pos] = keys[j];
            } else if (cls == C_KO) {
                ko.eid[pos] = id;
                if (!PREFIX) ko.ekey[pos] = keys[j];
            } else if (cls == C_LN) {
                ln.eid[pos] = id;
                isa_nxt[id] = a.bhead[row];
            } else {  // C_ONE
                resolve(a, isa_nxt, id, a.bhead[row], seg_blk((sel ? m.g1 : m.g0).bd), res, pos);
            }
        }
        __syncthreads();
    }
}

// The suffixes resolved in the previous round: copy their final rank into this round's write buffer (one by one from
// the resolved list, or, when they are many, by copying the whole current buffer).
__global__ void __launch_bounds__(TPB) k_fixup(FwdArgs a) {
    const Ctl *ctl = a.ctl;
    const u32 rpar = ctl->rpar;
    const ListView r = a.lists[L_R0 + (rpar ^ 1)];
    const u32 n = min((u32)ctl->cnt[L_R0 + (rpar ^ 1)], (u32)a.cap_n);
    u32 *nxt = a.isa[rpar ^ 1];
    const u32 idn = min(ctl->idn, (u32)a.cap_n);
    const u32 stride = gridDim.x * TPB;
    if ((u64)n * 16 > idn) {
        // many suffixes finished last round: copy the whole current rank buffer instead of scattering them (every
        // suffix's current rank, which this round's kernels then overwrite for the active ones); a streaming copy
        // costs far less than millions of random 4-byte writes
        const uint4 *src = reinterpret_cast<const uint4 *>(a.isa[rpar]);
        uint4 *dst = reinterpret_cast<uint4 *>(nxt);
        const u32 n4 = idn / 4;
        for (u32 i = blockIdx.x * TPB + threadIdx.x; i < n4; i += stride) __stcs(dst + i, __ldcs(src + i));
        for (u32 i = n4 * 4 + blockIdx.x * TPB + threadIdx.x; i < idn; i += stride) nxt[i] = a.isa[rpar][i];
        return;
    }
    const u32 nl = min(n, a.cap_res);  // n <= idn / 16 < cap_res here: the list holds every entry
    for (u32 i = blockIdx.x * TPB + threadIdx.x; i < nl; i += stride) nxt[r.eid[i]] = r.ekey[i];
}

// ------------------------------------------------------------------------------------------------ control
__device__ __forceinline__ void set_cond(unsigned long long h, u32 v) {
    if (h) cudaGraphSetConditional((cudaGraphConditionalHandle)h, v);
}
__device__ __forceinline__ u32 elems(const Ctl *c, u32 l) { return (u32)c->cnt[l]; }

__global__ void k_ctl_msd_begin(FwdArgs a) {
    Ctl *c = a.ctl;
    c->pass = 0;
    c->cnt[L_K0] = 0;
    set_cond(a.hcond, elems(c, L_L0 + c->rpar) > 0);
}
__global__ void k_ctl_msd_next(FwdArgs a) {
    Ctl *c = a.ctl;
    const u32 p = c->pass;
    const u32 produced = L_K0 + (p & 1);
    if (p == 0) c->cnt[L_L0 + c->rpar] = 0; else c->cnt[L_K0 + ((p - 1) & 1)] = 0;
    c->pass = p + 1;
    const u32 more = elems(c, produced) > 0;
    if (p + 1 > 2 * DEPTH_PREFIX + 2) { c->err |= 2; set_cond(a.hcond, 0); return; }
    set_cond(a.hcond, more);
}
__global__ void k_ctl_round_end(FwdArgs a) {
    Ctl *c = a.ctl;
    const u32 rp = c->rpar;
    const u32 active = elems(c, L_S0 + (rp ^ 1)) + elems(c, L_L0 + (rp ^ 1)) + elems(c, L_P0 + (rp ^ 1)) +
                       elems(c, L_M0 + (rp ^ 1));
    c->cnt[L_S0 + rp] = 0;
    c->cnt[L_L0 + rp] = 0;
    c->cnt[L_P0 + rp] = 0;
    c->cnt[L_M0 + rp] = 0;
    c->cnt[L_KS] = 0;
    c->cnt[L_K0] = 0;
    c->cnt[L_K1] = 0;
    c->cnt[L_R0 + (rp ^ 1)] = 0;
    c->rpar = rp ^ 1;
    c->round += 1;
    c->h = c->round == 1 ? c->h0 : c->h * 2;
    // repeat chains pay off once doubling stalls: the next round follows them when this one left at least four
    // fifths of its actives unfinished (round 0 counts every suffix as active)
    const u32 prev = c->round == 1 ? c->m : c->prev_active;
    c->chain_go = (u64)active * 5 >= (u64)prev * 4;
    c->prev_active = active;
    c->pass = 0;
    u32 cont = active > 0;
    if (cont && c->round > c->maxrounds) { c->err |= 1; cont = 0; }
    c->done = !cont;
    set_cond(a.hcond, cont);
}

// Sampled indexes: I[k] = 1 + rank of suffix k * r (I[0] is the primary index).
__global__ void k_samples(FwdArgs a) {
    const u32 *isa = a.isa[a.ctl->rpar];
    for (u32 b = blockIdx.x; b < a.B; b += gridDim.x) {
        const BlockInfo B = a.blk[b];
        const u32 ns = (B.n - 1) / B.r + 1;
        for (u32 k = threadIdx.x; k < ns; k += blockDim.x) a.I[B.iout + k] = isa[B.off + k * B.r] + 1;
    }
}

// Element lists of round 0: blocks up to SMAX bytes are single small groups, longer blocks single large ones.
// The L column's row 0 (the sentinel rotation) holds the block's last byte.
__global__ void k_init(FwdArgs a, const u32 *__restrict__ blk_list_start, const u8 *__restrict__ blk_is_large) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u32 b = 0; b < a.B; b++) {
        const BlockInfo bi = a.blk[b];
        u32 *eid = a.lists[blk_is_large[b] ? L_L0 : L_S0].eid + blk_list_start[b];
        for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < bi.n; j += stride) eid[j] = bi.off + (u32)j;
        if (blockIdx.x == 0 && threadIdx.x == 0) a.L[(u64)bi.off + b] = a.T[(u64)bi.off + bi.n - 1];
    }
}

#include "fwd_lsd.cuh"

// ------------------------------------------------------------------------------------------------ host engine
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

FwdEngine::FwdEngine() {
    for (auto &l : lists) l = ListView{nullptr, nullptr, nullptr, nullptr};
}
FwdEngine::~FwdEngine() { free_all(); }

void FwdEngine::free_all() {
    if (cap_stream) cudaStreamDestroy(cap_stream);
    cap_stream = nullptr;
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr;
    graph = nullptr;
    if (pool) cudaFree(pool);
    if (h_ctl) cudaFreeHost(h_ctl);
    pool = nullptr;
    h_ctl = nullptr;
    pool_bytes = 0;
    Ncap = 0;
    Bcap = Icap = 0;
}

// The workspace of n text bytes, bcap blocks and icap sampled indexes: every device array in pool order. `add`
// receives each array's address field and size (the estimate below only sums the sizes).
template <typename Add>
void FwdEngine::layout(u64 ncap, u32 bcap, u32 icap, bool want_sa, Add add) {
    const u64 n = ncap;
    const u32 smax = (u32)cfg.tile_cap / 2;
    const u64 nseg_small = n / 2 + bcap + 8;
    const u64 nseg_large = n / smax + bcap + 8;
    const u64 nseg_med = n / (GTINY + 1) + bcap + 8;
    // small-group lists hold groups longer than GMED (every producer sends shorter ones to the tiny and medium
    // lists), besides one group per block in the tile path's round 0; the keyed list takes any bucket size
    const u64 nseg_s = n / (GMED + 1) + bcap + 8;
    const u64 ntm_small = n / smax + 8, ntm_large = n / TSM + 8;
    add((void **)&own_T, n + 64);
    add((void **)&own_L, n + bcap + 64);
    add((void **)&own_I, (size_t)icap * 4 + 16);
    if (want_sa) add((void **)&own_SA, n * 4);
    add((void **)&d_isa[0], n * 4);
    add((void **)&d_isa[1], n * 4);
    add((void **)&d_blk, (size_t)bcap * sizeof(BlockInfo));
    const u64 nres = n / 16 + 64;  // resolved-list entries (see resolve)
    for (int l = 0; l < NLISTS; l++) {
        const bool small = l == L_S0 || l == L_S1 || l == L_KS;
        const bool res = l == L_R0 || l == L_R1;
        const bool tiny = l == L_P0 || l == L_P1, med = l == L_M0 || l == L_M1;
        if (l != L_P1) add((void **)&lists[l].eid, (res ? nres : n) * 4);  // the two tiny lists share one id array
        if (tiny || med) {  // ids and segment descriptors only
            add((void **)&lists[l].seg, (tiny ? nseg_small : nseg_med) * sizeof(Seg));
            continue;
        }
        // keys: the large lists share one array (only the round's input list carries keys, from its key generation
        // on); the small lists have none
        if (l != L_S0 && l != L_S1 && l != L_L1) add((void **)&lists[l].ekey, (res ? nres : n) * 4);
        if (!res) {
            add((void **)&lists[l].seg, (l == L_KS ? nseg_small : small ? nseg_s : nseg_large) * sizeof(Seg));
            add((void **)&lists[l].tmap, (small ? ntm_small : ntm_large) * 4);
            if (small) add((void **)&lists[l].tbig, ntm_small * 4);
        }
    }
    add((void **)&d_hist, nseg_large * 256 * 4);
    add((void **)&d_cursor, nseg_large * 256 * 4);
    add((void **)&d_bhead, nseg_large * 256 * 4);
    add((void **)&d_dest, nseg_large * 256);
    add((void **)&d_orand, nseg_large * 8);
    add((void **)&d_orand64, nseg_large * 16);
    const u64 ltiles = n / LSD_TILE + bcap + 2, stiles = n / SEG_TILE + 2;
    // the round-0 radix items (8 bytes each, ping-pong) alias the bucket-pass work lists: item buffer q spans K_q's
    // id array and the key array laid out right after it (checked in grow()). Round 0 on the LSD path uses neither
    // list, and in the rank rounds the medium-key scratch (lval[0]) is written after the round's bucket passes and
    // read before the next round's
    add((void **)&d_lstat, ltiles * 256 * 8);
    add((void **)&d_segbits, n / 8 + 64);
    add((void **)&d_lhist, (size_t)bcap * 256 * 4);  // byte histogram of every block
    add((void **)&d_lbase, (size_t)bcap * NSLOT * 256 * 4);
    add((void **)&d_ltile, NSLOT * 4);
    add((void **)&d_segagg, stiles * 8 * 4);
    // repeat chains: a bit per id, its next-zero table per word and per tile of words
    const u64 cwords = n / 32 + 2, ctiles = cwords / NZ_TILE + 1;
    add((void **)&d_cbits, cwords * 4);
    add((void **)&d_cnz, cwords * 4);
    add((void **)&d_ctn, (ctiles + 1) * 4);
    add((void **)&d_ctl, sizeof(Ctl));
}

u64 FwdEngine::estimate_bytes(u64 n, u32 bcap, u32 icap) {
    u64 total = 0;
    layout(std::max<u64>(n, Ncap), std::max<u32>(bcap, Bcap), std::max<u32>(icap, Icap), sa_cap,
           [&](void **, size_t bytes) { total += align_up(std::max<size_t>(bytes, 16), 256); });
    return total;
}

int FwdEngine::grow(u64 ncap, u32 bcap, u32 icap, bool want_sa) {
    if (ncap <= Ncap && bcap <= Bcap && icap <= Icap && (!want_sa || sa_cap)) return 0;
    ncap = std::max<u64>(ncap, Ncap);
    bcap = std::max<u32>(bcap, Bcap);
    icap = std::max<u32>(icap, Icap);
    want_sa = want_sa || sa_cap;
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    if (pool) { cudaFree(pool); pool = nullptr; }
    own_SA = nullptr;
    for (auto &l : lists) l = ListView{nullptr, nullptr, nullptr, nullptr};
    struct Item { void **p; size_t bytes; };
    std::vector<Item> items;
    layout(ncap, bcap, icap, want_sa,
           [&](void **p, size_t bytes) { items.push_back({p, align_up(std::max<size_t>(bytes, 16), 256)}); });
    const u64 n = ncap;
    const u32 smax = (u32)cfg.tile_cap / 2;
    const u64 nseg_small = n / 2 + bcap + 8;
    const u64 nseg_large = n / smax + bcap + 8;
    const u64 nseg_med = n / (GTINY + 1) + bcap + 8;
    const u64 nseg_s = n / (GMED + 1) + bcap + 8;
    const u64 ntm_small = n / smax + 8, ntm_large = n / TSM + 8;
    const u64 ltiles = n / LSD_TILE + bcap + 2, stiles = n / SEG_TILE + 2;
    size_t total = 0;
    for (auto &it : items) total += it.bytes;
    cudaError_t e = cudaMalloc(&pool, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        pool = nullptr;
        Ncap = 0;
        return record_cuda_error(e, "cudaMalloc(forward workspace)", __FILE__, __LINE__);
    }
    pool_bytes = total;
    size_t off = 0;
    for (auto &it : items) { *it.p = (char *)pool + off; off += it.bytes; }
    lists[L_P1].eid = lists[L_P0].eid;
    lists[L_L1].ekey = lists[L_L0].ekey;
    d_lval[0] = lists[L_K0].eid; d_lval[1] = lists[L_K1].eid;
    d_lhi[0] = lists[L_K0].ekey; d_lhi[1] = lists[L_K1].ekey;
    for (int q = 0; q < 2; q++)  // round 0's 8-byte items need each id array and its key array to be adjacent
        if ((char *)d_lhi[q] != (char *)d_lval[q] + align_up(std::max<size_t>(n * 4, 16), 256)) {
            cudaFree(pool);  // leave no half-made workspace behind: the next call lays it out again
            pool = nullptr;
            pool_bytes = 0;
            Ncap = 0;
            return record_cuda_error(cudaErrorInvalidValue, "forward workspace layout", __FILE__, __LINE__);
        }
    KGB_CHECK(cudaMemset(d_hist, 0, nseg_large * 256 * 4));
    for (int l : {(int)L_S0, (int)L_S1, (int)L_KS}) KGB_CHECK(cudaMemset(lists[l].tbig, 0xFF, ntm_small * 4));
    // orand rows start as (or = 0, and = ~0)
    {
        std::vector<u32> init(2 * nseg_large);
        for (size_t i = 0; i < nseg_large; i++) { init[2 * i] = 0; init[2 * i + 1] = ~0u; }
        KGB_CHECK(cudaMemcpy(d_orand, init.data(), init.size() * 4, cudaMemcpyHostToDevice));
        std::vector<u64> init64(2 * nseg_large);
        for (size_t i = 0; i < nseg_large; i++) { init64[2 * i] = 0; init64[2 * i + 1] = ~0ull; }
        KGB_CHECK(cudaMemcpy(d_orand64, init64.data(), init64.size() * 8, cudaMemcpyHostToDevice));
    }
    if (!h_ctl) KGB_CHECK(cudaMallocHost(&h_ctl, sizeof(Ctl)));
    Ncap = ncap;
    Bcap = bcap;
    Icap = icap;
    sa_cap = want_sa;
    cap_segs = nseg_s; cap_segk = nseg_small; cap_segl = nseg_large; cap_segt = nseg_small; cap_segm = nseg_med;
    cap_tms = ntm_small;
    cap_tml = ntm_large;
    lsd_tiles_cap = ltiles; seg_tiles_cap = stiles;
    KGB_CHECK(cudaMemset(d_lstat, 0, ltiles * 256 * 8));
    return 0;
}

void FwdEngine::set_caps(FwdArgs &a) const {
    a.orand64 = d_orand64;
    for (int q = 0; q < 2; q++) { a.lval[q] = d_lval[q]; a.lhi[q] = d_lhi[q]; }
    for (int q = 0; q < 2; q++) a.lit[q] = reinterpret_cast<unsigned long long *>(d_lval[q]);
    a.segbits = d_segbits;
    a.lstat = d_lstat; a.lhist = d_lhist; a.ltile = d_ltile; a.segagg = d_segagg; a.lbase = d_lbase;
    a.cbits = d_cbits; a.cnz = d_cnz; a.ctn = d_ctn;
    a.cwords = (u32)(N / 32 + 2);
    a.ctiles = (a.cwords + NZ_TILE - 1) / NZ_TILE;
    a.chain_from = (u32)cfg.chain_from;
    a.spin_limit = 1u << 22;
    a.small_group = (u32)cfg.small_group;
    a.lsd_bytes = (u32)cfg.lsd_bytes;
    a.idn = (u32)N;
    {
        // the emit kernels' rank writes stay within one block's ids at a time (the sorted order is block-major), so
        // they only miss L2 when a block is larger than a pass's span
        const u64 p = (N + RANK_SPAN - 1) / RANK_SPAN;
        a.rank_passes = maxn > RANK_SPAN && p <= RANK_PASSES_MAX ? (u32)p : 0u;
    }
    a.warp_path = (u32)cfg.warp_path;
    a.cap_n = Ncap; a.cap_segs = cap_segs; a.cap_segk = cap_segk; a.cap_segl = cap_segl; a.cap_segt = cap_segt;
    a.cap_segm = cap_segm;
    a.cap_tms = cap_tms;
    a.cap_tml = cap_tml;
    a.cap_res = (u32)(Ncap / 16 + 64);
}

int FwdEngine::plan(const u32 *n, const u32 *r, int count, bool want_sa) {
    if (count <= 0) return -1;
    h_off.resize(count); h_n.resize(count); h_r.resize(count); h_iout.resize(count);
    u64 off = 0, io = 0;
    maxn = 0;
    for (int b = 0; b < count; b++) {
        if (n[b] < 2 || r[b] < 2) return -1;
        h_off[b] = (u32)off; h_n[b] = n[b]; h_r[b] = r[b]; h_iout[b] = (u32)io;
        off += n[b];
        io += (n[b] - 1) / r[b] + 1;
        maxn = std::max(maxn, n[b]);
        if (off > 0xFFFF0000ull || io > 0xFFFF0000ull) return -1;
    }
    N = off; B = (u32)count; nI = (u32)io;
    ext = false;
    want_sa_run = want_sa;
    resolve_config();
    int rc = grow(N, B, nI, want_sa);
    if (rc) return rc;
    d_T = own_T; d_L = own_L; d_I = own_I; d_SA = want_sa ? own_SA : nullptr;
    return 0;
}

int FwdEngine::plan_external(const u32 *off, const u32 *n, const u32 *r, const u32 *iout, int count, u8 *dT, u8 *dL,
                             u32 *dI, u32 *dSA) {
    if (count <= 0) return -1;
    h_off.assign(off, off + count); h_n.assign(n, n + count); h_r.assign(r, r + count); h_iout.assign(iout, iout + count);
    u64 end = 0, io = 0;
    maxn = 0;
    for (int b = 0; b < count; b++) {
        if (n[b] < 2 || r[b] < 2) return -1;
        end = std::max<u64>(end, (u64)off[b] + n[b]);
        io = std::max<u64>(io, (u64)iout[b] + (n[b] - 1) / r[b] + 1);
        maxn = std::max(maxn, n[b]);
    }
    if (end > 0xFFFF0000ull) return -1;
    N = end; B = (u32)count; nI = (u32)io;
    ext = true;
    want_sa_run = dSA != nullptr;
    resolve_config();
    int rc = grow(N, B, 0, false);
    if (rc) return rc;
    d_T = dT; d_L = dL; d_I = dI; d_SA = dSA;
    return 0;
}

void FwdEngine::resolve_config() {
    cfg = ucfg;
    FwdConfig t;
    if (!tuned_config(N, &t)) return;
    if (!(cfg_explicit & CFG_TILE_CTAS)) cfg.tile_ctas = t.tile_ctas;
    if (!(cfg_explicit & CFG_MSD_CTAS)) cfg.msd_ctas = t.msd_ctas;
    if (!(cfg_explicit & CFG_SMALL_GROUP)) cfg.small_group = t.small_group;
    if (!(cfg_explicit & CFG_WARP_PATH)) cfg.warp_path = t.warp_path;
    if (!(cfg_explicit & CFG_LSD_ROUND0)) cfg.lsd_round0 = t.lsd_round0;
    if (!(cfg_explicit & CFG_LSD_BYTES)) cfg.lsd_bytes = t.lsd_bytes;
    if (!(cfg_explicit & CFG_CHAIN_FROM)) cfg.chain_from = t.chain_from;
}

static int ceil_log2(u64 x) { int k = 0; while ((1ull << k) < x) k++; return k; }

bool FwdEngine::lsd_enabled() const { return cfg.lsd_round0 && N < (1ull << 30); }

int FwdEngine::setup_round0(cudaStream_t s) {
    // block table, round-0 lists and their tile maps are laid out on the host (B entries, small)
    const u32 smax = (u32)cfg.tile_cap / 2;
    std::vector<BlockInfo> bi(B);
    u32 soff_b = 0, lt_b = 0;
    std::vector<u32> lstart(B);
    std::vector<u8> large(B);
    std::vector<Seg> seg_s, seg_l;
    std::vector<u32> tm_s, tm_l, big_s;
    u64 es = 0, el = 0;
    for (u32 b = 0; b < B; b++) {
        bi[b] = BlockInfo{h_off[b], h_n[b], h_r[b], h_iout[b], soff_b, lt_b};
        soff_b += h_n[b];
        lt_b += (h_n[b] + LSD_TILE - 1) / LSD_TILE;
        large[b] = h_n[b] > smax;
        Seg g;
        g.len = h_n[b]; g.head = 0; g.bd = b;
        if (large[b]) {
            g.start = (u32)el; lstart[b] = (u32)el;
            for (u64 t = (el + TSM - 1) / TSM; t * TSM < el + h_n[b]; t++) { if (tm_l.size() <= t) tm_l.resize(t + 1); tm_l[t] = (u32)seg_l.size(); }
            seg_l.push_back(g);
            el += h_n[b];
        } else {
            g.start = (u32)es; lstart[b] = (u32)es;
            u64 t = (es + smax - 1) / smax;
            if (t * smax < es + h_n[b]) { if (tm_s.size() <= t) tm_s.resize(t + 1); tm_s[t] = (u32)seg_s.size() + (t * smax == es ? 0 : 1); }
            if (h_n[b] > WARP_GROUP) big_s.push_back((u32)(es / smax));
            seg_s.push_back(g);
            es += h_n[b];
        }
    }
    // staging: the small vectors go through one pinned buffer
    Ctl c;
    memset(&c, 0, sizeof(c));
    c.cnt[L_S0] = ((u64)seg_s.size() << 32) | es;
    c.cnt[L_L0] = ((u64)seg_l.size() << 32) | el;
    c.maxrounds = (u32)ceil_log2(maxn) + 3;
    c.seq = ++call_seq;
    c.h0 = lsd_enabled() ? (u32)cfg.lsd_bytes : 8u;
    c.lsd_tiles = lt_b;
    c.idn = (u32)N;  // N is the batch's extent: max over blocks of off + n
    KGB_CHECK(cudaMemcpyAsync(d_blk, bi.data(), B * sizeof(BlockInfo), cudaMemcpyHostToDevice, s));
    const size_t ntm = cap_tms;
    for (int l : {(int)L_S0, (int)L_S1, (int)L_KS}) KGB_CHECK(cudaMemsetAsync(lists[l].tbig, 0xFF, ntm * 4, s));
    if (!seg_s.empty()) {
        KGB_CHECK(cudaMemcpyAsync(lists[L_S0].seg, seg_s.data(), seg_s.size() * sizeof(Seg), cudaMemcpyHostToDevice, s));
        if (!tm_s.empty()) KGB_CHECK(cudaMemcpyAsync(lists[L_S0].tmap, tm_s.data(), tm_s.size() * 4, cudaMemcpyHostToDevice, s));
        // round-0 stamps (value 0) of windows where a block longer than WARP_GROUP starts
        std::vector<u32> stamp(tm_s.size() + 1, 0xFFFFFFFFu);
        for (u32 t : big_s) if (t < stamp.size()) stamp[t] = 0;
        KGB_CHECK(cudaMemcpyAsync(lists[L_S0].tbig, stamp.data(), stamp.size() * 4, cudaMemcpyHostToDevice, s));
        KGB_CHECK(cudaStreamSynchronize(s));  // `stamp` is a local
    }
    if (!seg_l.empty()) {
        KGB_CHECK(cudaMemcpyAsync(lists[L_L0].seg, seg_l.data(), seg_l.size() * sizeof(Seg), cudaMemcpyHostToDevice, s));
        KGB_CHECK(cudaMemcpyAsync(lists[L_L0].tmap, tm_l.data(), tm_l.size() * 4, cudaMemcpyHostToDevice, s));
    }
    *h_ctl = c;
    KGB_CHECK(cudaMemcpyAsync(d_ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    // per-block list starts and classes: stored behind the block table in the histogram rows, which are zero
    // outside a bucket pass and are restored to zero by k_init's caller below
    u32 *d_lstart = d_cursor;
    u8 *d_large = d_dest;
    KGB_CHECK(cudaMemcpyAsync(d_lstart, lstart.data(), B * 4, cudaMemcpyHostToDevice, s));
    KGB_CHECK(cudaMemcpyAsync(d_large, large.data(), B, cudaMemcpyHostToDevice, s));
    // these host vectors must outlive the async copies
    KGB_CHECK(cudaStreamSynchronize(s));
    return 0;
}

static FwdArgs make_args(Ctl *ctl, const u8 *T, const BlockInfo *blk, u32 *const isa[2], u8 *L, u32 *SA, u32 *I,
                         const ListView *lists, u32 *hist, u32 *cursor, u32 *bhead, u32 *orand, u8 *dest, u32 B,
                         u32 smax) {
    FwdArgs a;
    memset(&a, 0, sizeof(a));
    a.ctl = ctl; a.T = T; a.blk = blk; a.isa[0] = isa[0]; a.isa[1] = isa[1]; a.L = L; a.SA = SA; a.I = I;
    for (int l = 0; l < NLISTS; l++) a.lists[l] = lists[l];
    a.hist = hist; a.cursor = cursor; a.bhead = bhead; a.orand = orand; a.dest = dest; a.B = B; a.smax = smax;
    a.orand64 = nullptr;
    a.hcond = 0;
    return a;
}

static size_t lsd_smem() { return sizeof(LsdSmem); }
template <bool PREFIX, int TILE>
static int tile_smem() { return (int)sizeof(TileSmem<TILE, typename TileTraits<PREFIX, TILE>::KeyT>); }
template <bool PREFIX, int TILE>
static int warp_smem() { return (int)sizeof(WarpSmem<TILE, typename TileTraits<PREFIX, TILE>::KeyT>); }

struct Launcher {
    cudaStream_t s;
    int grid_tile, grid_msd, grid_scan, tile_cap, grid_tile_prefix, grid_warp, grid_lsd;
    long long *launches;
    Profiler *prof;
    template <typename K, typename... Args>
    cudaError_t go(K kern, int grid, int block, size_t smem, Args... args) {
        (*launches)++;
        auto fn = [&]() -> cudaError_t {
            kern<<<grid, block, smem, s>>>(args...);
            return cudaGetLastError();
        };
        return prof ? prof->launch(s, fn) : fn();
    }
    void tag(int k, u32 e, u32 sg = 0) { if (prof) prof->tag(k, e, sg); }
};

static bool g_attr_done[4] = {false, false, false, false};
static int set_tile_attrs(int tile) {
    int idx = tile == 8192 ? 1 : 0;
    if (g_attr_done[idx]) return 0;
    if (tile == 4096) {
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<true, false, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<true, 4096>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<true, true, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<true, 4096>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<false, false, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<false, 4096>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<false, true, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<false, 4096>()));
    } else {
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<true, false, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<true, 8192>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<true, true, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<true, 8192>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<false, false, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<false, 8192>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_sort<false, true, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem<false, 8192>()));
    }
    if (tile == 4096) {
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<true, false, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<true, 4096>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<true, true, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<true, 4096>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<false, false, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<false, 4096>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<false, true, 4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<false, 4096>()));
    } else {
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<true, false, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<true, 8192>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<true, true, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<true, 8192>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<false, false, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<false, 8192>()));
        KGB_CHECK(cudaFuncSetAttribute(k_tile_warp<false, true, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize, warp_smem<false, 8192>()));
    }
    KGB_CHECK(cudaFuncSetAttribute(k_lsd_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsd_smem()));
    g_attr_done[idx] = true;
    return 0;
}

// Kernel sequences shared by the plain and graph paths.
static cudaError_t enq_tile_warp(Launcher &L, const FwdArgs &a, bool prefix, bool keyed) {
    if (L.prof) L.prof->kernel = prefix ? (keyed ? K_WARP_PREFIX_KEYED : K_WARP_PREFIX) : (keyed ? K_WARP_RANK_KEYED : K_WARP_RANK);
    const int g = L.grid_warp;
    if (L.tile_cap == 4096) {
        if (prefix) {
            const size_t sm = warp_smem<true, 4096>();
            return keyed ? L.go(k_tile_warp<true, true, 4096>, g, TPB, sm, a) : L.go(k_tile_warp<true, false, 4096>, g, TPB, sm, a);
        }
        const size_t sm = warp_smem<false, 4096>();
        return keyed ? L.go(k_tile_warp<false, true, 4096>, g, TPB, sm, a) : L.go(k_tile_warp<false, false, 4096>, g, TPB, sm, a);
    }
    if (prefix) {
        const size_t sm = warp_smem<true, 8192>();
        return keyed ? L.go(k_tile_warp<true, true, 8192>, g, TPB, sm, a) : L.go(k_tile_warp<true, false, 8192>, g, TPB, sm, a);
    }
    const size_t sm = warp_smem<false, 8192>();
    return keyed ? L.go(k_tile_warp<false, true, 8192>, g, TPB, sm, a) : L.go(k_tile_warp<false, false, 8192>, g, TPB, sm, a);
}

static cudaError_t enq_tile_block(Launcher &L, const FwdArgs &a, bool prefix, bool keyed);

// one small-group list: the block kernel for tiles holding a longer group, then the warp kernel for the others
static cudaError_t enq_tile(Launcher &L, const FwdArgs &a, bool prefix, bool keyed) {
    const u32 el = L.prof ? L.prof->elems : 0, sg = L.prof ? L.prof->segs : 0;
    cudaError_t e = enq_tile_block(L, a, prefix, keyed);
    if (e || !a.warp_path) return e;
    if (L.prof) L.prof->tag(0, el, sg);
    return enq_tile_warp(L, a, prefix, keyed);
}

static cudaError_t enq_tile_block(Launcher &L, const FwdArgs &a, bool prefix, bool keyed) {
    if (L.prof) L.prof->kernel = prefix ? (keyed ? K_TILE_PREFIX_KEYED : K_TILE_PREFIX) : (keyed ? K_TILE_RANK_KEYED : K_TILE_RANK);
    if (L.tile_cap == 4096) {
        if (prefix) {
            const size_t sm = tile_smem<true, 4096>();
            const int g = L.grid_tile_prefix;
            return keyed ? L.go(k_tile_sort<true, true, 4096>, g, TPB, sm, a) : L.go(k_tile_sort<true, false, 4096>, g, TPB, sm, a);
        }
        const size_t sm = tile_smem<false, 4096>();
        return keyed ? L.go(k_tile_sort<false, true, 4096>, L.grid_tile, TPB, sm, a) : L.go(k_tile_sort<false, false, 4096>, L.grid_tile, TPB, sm, a);
    }
    if (prefix) {
        const size_t sm = tile_smem<true, 8192>();
        const int g = L.grid_tile_prefix;
        return keyed ? L.go(k_tile_sort<true, true, 8192>, g, TPB, sm, a) : L.go(k_tile_sort<true, false, 8192>, g, TPB, sm, a);
    }
    const size_t sm = tile_smem<false, 8192>();
    return keyed ? L.go(k_tile_sort<false, true, 8192>, L.grid_tile, TPB, sm, a) : L.go(k_tile_sort<false, false, 8192>, L.grid_tile, TPB, sm, a);
}
static cudaError_t enq_msd_pass(Launcher &L, const FwdArgs &a, bool prefix) {
    cudaError_t e;
    auto k = [&](int id) { if (L.prof) L.prof->kernel = id; };
    if (prefix) {
        k(K_MSD_HIST);
        if ((e = L.go(k_msd_hist<true>, L.grid_msd, TPB, 0, a))) return e;
        k(K_MSD_SCAN);
        if ((e = L.go(k_msd_scan<true>, L.grid_scan, TPB, 0, a))) return e;
        k(K_MSD_SCATTER);
        return L.go(k_msd_scatter<true>, L.grid_msd, TPB, 0, a);
    }
    k(K_MSD_HIST);
    if ((e = L.go(k_msd_hist<false>, L.grid_msd, TPB, 0, a))) return e;
    k(K_MSD_SCAN);
    if ((e = L.go(k_msd_scan<false>, L.grid_scan, TPB, 0, a))) return e;
    k(K_MSD_SCATTER);
    return L.go(k_msd_scatter<false>, L.grid_msd, TPB, 0, a);
}

static int report_err(u32 bits) {
    char m[96];
    snprintf(m, sizeof m, "forward sort: device error bits 0x%x (internal error)", bits);
    record_error(m);
    return -2;
}


// Round 0 as an LSD radix sort, in two parts: begin, keys and the first histogram; then the radix passes (one per
// slot in `slots`; each returns at once when its key byte does not vary) and the segmentation.
static cudaError_t enq_lsd_keys(Launcher &L, const FwdArgs &a) {
    cudaError_t e;
    L.tag(K_LSD_BEGIN, 0);
    if ((e = L.go(k_lsd_begin, L.grid_msd, 256, 0, a))) return e;
    L.tag(K_LSD_KEY0, 0);
    if ((e = L.go(k_lsd_key0, L.grid_msd, TPB, 0, a))) return e;
    L.tag(K_LSD_HIST, 0);
    return L.go(k_lsd_hist0, std::min<int>((int)a.B, L.grid_msd), TPB, 0, a);
}
static cudaError_t enq_lsd_sort_seg(Launcher &L, const FwdArgs &a, u32 slots, u32 m_tag) {
    cudaError_t e;
    if (L.prof) L.prof->pass = -1;
    L.tag(K_LSD_IDENT, m_tag);
    if ((e = L.go(k_lsd_ident, L.grid_msd, TPB, 0, a))) return e;
    for (int slot = 0; slot < NSLOT; slot++) {
        if (!((slots >> slot) & 1)) continue;
        L.tag(K_LSD_PASS, m_tag);
        if (L.prof) L.prof->pass = slot;
        if ((e = L.go(k_lsd_pass, L.grid_lsd, TPB, lsd_smem(), a, slot)))
            return e;
    }
    if (L.prof) L.prof->pass = -1;
    L.tag(K_SEG_COUNT, m_tag);
    if ((e = L.go(k_seg_count, L.grid_msd, TPB, 0, a))) return e;
    L.tag(K_SEG_SCAN, m_tag);
    if ((e = L.go(k_seg_scan, 1, 1024, 0, a))) return e;
    L.tag(K_SEG_EMIT1, m_tag);
    if ((e = L.go(k_seg_emit1, L.grid_msd, TPB, 0, a))) return e;
    L.tag(K_SEG_EMIT2, m_tag);
    if ((e = L.go(k_seg_emit2, L.grid_msd, TPB, 0, a))) return e;
    for (u64 lo = 0; a.rank_passes && lo < a.idn; lo += RANK_SPAN) {
        L.tag(K_SEG_RANK, m_tag);
        if ((e = L.go(k_seg_rank, L.grid_msd, TPB, 0, a, (u32)lo, (u32)std::min<u64>(lo + RANK_SPAN, a.idn)))) return e;
    }
    return cudaSuccess;
}

static u32 host_active_slots(const Ctl &c) { return c.lsd_act; }

// The repeat-chain tables of a rank round (each kernel returns at once before round chain_from or on an empty tiny
// list, and in rounds where doubling has not stalled): clear the bits, set them for the linked tiny groups, build the
// next-zero tables.
static cudaError_t enq_chain(Launcher &L, const FwdArgs &a, u32 elems, u32 segs) {
    cudaError_t e;
    L.tag(K_CHAIN, elems, segs);
    if ((e = L.go(k_chain_clear, L.grid_msd, TPB, 0, a))) return e;
    L.tag(K_CHAIN, elems, segs);
    if ((e = L.go(k_chain_link, L.grid_msd, TPB, 0, a))) return e;
    L.tag(K_CHAIN, elems, segs);
    if ((e = L.go(k_chain_nz, L.grid_msd, TPB, 0, a))) return e;
    L.tag(K_CHAIN, elems, segs);
    return L.go(k_chain_tiles, 1, 1024, 0, a);
}

int FwdEngine::run_plain(cudaStream_t s) {
    const u32 smax = (u32)cfg.tile_cap / 2;
    FwdArgs a = make_args(d_ctl, d_T, d_blk, d_isa, d_L, d_SA, d_I, lists, d_hist, d_cursor, d_bhead, d_orand, d_dest,
                          B, smax);
    set_caps(a);
    prof.reset();
    Launcher L{s, grid_tile, grid_msd, grid_scan, cfg.tile_cap, grid_tile_prefix, grid_warp, grid_lsd, &stats.launches, prof.on ? &prof : nullptr};
    auto cnt_e = [&](u32 l) { return (u32)h_ctl->cnt[l]; };
    auto cnt_s = [&](u32 l) { return (u32)(h_ctl->cnt[l] >> 32); };
    auto read_ctl = [&]() -> int {
        KGB_CHECK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        KGB_CHECK(cudaStreamSynchronize(s));
        return 0;
    };
    prof.round = 0; prof.pass = 0;
    const bool lsd0 = lsd_enabled();
    if (!lsd0) {
        L.tag(K_INIT, (u32)N, B);
        KGB_CHECK(L.go(k_init, grid_msd, TPB, 0, a, (const u32 *)d_cursor, (const u8 *)d_dest));
    }
    if (int rc = read_ctl()) return rc;
    for (int round = 0;; round++) {
        const bool prefix = round == 0;
        const u32 rp = h_ctl->rpar;
        prof.round = round; prof.pass = -1;
        if (prefix && lsd0) {
            // LSD round 0: launch only the passes whose key byte varies (the host reads them after the keys)
            KGB_CHECK(enq_lsd_keys(L, a));
            if (int rc = read_ctl()) return rc;
            const u32 slots = host_active_slots(*h_ctl);
            KGB_CHECK(enq_lsd_sort_seg(L, a, slots, (u32)N));
            stats.passes += __builtin_popcount(slots);
        } else {
            if (!prefix) {
                L.tag(K_FIXUP, cnt_e(L_R0 + (rp ^ 1)));
                KGB_CHECK(L.go(k_fixup, grid_msd, TPB, 0, a));
                L.tag(K_KEYGEN, cnt_e(L_L0 + rp), cnt_s(L_L0 + rp));
                KGB_CHECK(L.go(k_keygen, grid_msd, TPB, 0, a));
            }
            L.tag(K_CTL, 0);
            KGB_CHECK(L.go(k_ctl_msd_begin, 1, 1, 0, a));
            if (int rc = read_ctl()) return rc;
            u32 lin = L_L0 + h_ctl->rpar;
            u32 more = cnt_e(lin) > 0;
            int pass = 0;
            while (more) {
                prof.pass = pass++;
                L.tag(K_MSD_HIST, cnt_e(lin), cnt_s(lin));
                KGB_CHECK(enq_msd_pass(L, a, prefix));
                L.tag(K_CTL, 0);
                KGB_CHECK(L.go(k_ctl_msd_next, 1, 1, 0, a));
                stats.passes++;
                if (int rc = read_ctl()) return rc;
                if (h_ctl->err) return report_err(h_ctl->err);
                lin = L_K0 + ((h_ctl->pass - 1) & 1);
                more = cnt_e(lin) > 0;
            }
            prof.pass = -1;
            if (prof.on) {
                // one kernel at a time, with the control block read after each, so every record carries the elements
                // that kernel itself sorted (tiles split between the block and the warp kernel)
                for (int keyed = 0; keyed < 2; keyed++) {
                    const u32 lid = keyed ? L_KS : L_S0 + h_ctl->rpar;
                    const u32 segs = cnt_s(lid);
                    for (int wk = 0; wk < 2; wk++) {
                        if (wk && !cfg.warp_path) break;
                        const u64 before = h_ctl->tile_elems[wk];
                        prof.tag(0, 0, segs);
                        KGB_CHECK(wk ? enq_tile_warp(L, a, prefix, keyed) : enq_tile_block(L, a, prefix, keyed));
                        if (int rc = read_ctl()) return rc;
                        prof.recs.back().elems = (u32)(h_ctl->tile_elems[wk] - before);
                    }
                }
            } else {
                KGB_CHECK(enq_tile(L, a, prefix, false));
                KGB_CHECK(enq_tile(L, a, prefix, true));
            }
            if (!prefix && cnt_e(L_M0 + rp)) {
                L.tag(K_MKEYS, cnt_e(L_M0 + rp), cnt_s(L_M0 + rp));
                KGB_CHECK(L.go(k_mkeys, grid_msd, TPB, 0, a));
                L.tag(K_GROUP_WARP, cnt_e(L_M0 + rp), cnt_s(L_M0 + rp));
                KGB_CHECK(L.go(k_group_warp, grid_scan, TPB, 0, a));
            }
            if (!prefix && cnt_e(L_P0 + rp)) {
                if (a.chain_from && (u32)round >= a.chain_from && h_ctl->chain_go)
                    KGB_CHECK(enq_chain(L, a, cnt_e(L_P0 + rp), cnt_s(L_P0 + rp)));
                L.tag(K_GROUP, cnt_e(L_P0 + rp), cnt_s(L_P0 + rp));
                KGB_CHECK(L.go(k_group_thread, grid_msd, TPB, 0, a));
            }
        }
        L.tag(K_CTL, 0);
        KGB_CHECK(L.go(k_ctl_round_end, 1, 1, 0, a));
        stats.rounds++;
        if (int rc = read_ctl()) return rc;
        if (h_ctl->err) return report_err(h_ctl->err);
        if (h_ctl->done) break;
    }
    L.tag(K_SAMPLES, nI, B);
    KGB_CHECK(L.go(k_samples, std::min<u32>(B, 1024u), 128, 0, a));
    return 0;
}

// Graph: init -> round 0 -> while (active) { rank round } -> samples, where a round is
//   fixup, keygen, msd_begin -> while (pass input non-empty) { hist, scan, scatter, msd_next } -> tiles, round_end.
// Round 0 (prefix keys) is laid out once before the loop, the rank round is the loop body; the loops close with
// conditional while-nodes whose handles the 1-thread control kernels set.
typedef std::vector<cudaGraphNode_t> Deps;

// Captures the kernels enqueued by fn into graph g after the nodes in deps; returns the new leaves in deps.
template <typename F>
static int capture_into(cudaStream_t s, cudaGraph_t g, Deps &deps, F fn) {
    KGB_CHECK(cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                            cudaStreamCaptureModeThreadLocal));
    cudaError_t e = fn();
    const cudaGraphNode_t *d = nullptr;
    size_t nd = 0;
    cudaStreamCaptureStatus st;
    cudaError_t e2 = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &d, nullptr, &nd);
    Deps leaves(d, d + (e2 == cudaSuccess ? nd : 0));
    cudaGraph_t out = g;
    cudaError_t e3 = cudaStreamEndCapture(s, &out);
    KGB_CHECK(e);
    KGB_CHECK(e2);
    KGB_CHECK(e3);
    deps = leaves;
    return 0;
}

static int add_while(cudaGraph_t g, Deps &deps, cudaGraphConditionalHandle h, cudaGraph_t *body) {
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    KGB_CHECK(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &cp));
    *body = cp.conditional.phGraph_out[0];
    deps.assign(1, node);
    return 0;
}

// A tile-path round (prefix or rank) into graph g after deps; hmsd closes its bucket-pass loop.
static int add_tile_round(cudaStream_t s, cudaGraph_t g, Deps &deps, Launcher &L, const FwdArgs &a, bool prefix,
                          cudaGraphConditionalHandle hmsd) {
    FwdArgs am = a;
    am.hcond = (unsigned long long)hmsd;
    if (int rc = capture_into(s, g, deps, [&]() -> cudaError_t {
            cudaError_t e;
            if (!prefix) {
                if ((e = L.go(k_fixup, L.grid_msd, TPB, 0, a))) return e;
                if ((e = L.go(k_keygen, L.grid_msd, TPB, 0, a))) return e;
            }
            return L.go(k_ctl_msd_begin, 1, 1, 0, am);
        }))
        return rc;
    cudaGraph_t mbody;
    if (int rc = add_while(g, deps, hmsd, &mbody)) return rc;
    Deps md;
    if (int rc = capture_into(s, mbody, md, [&]() -> cudaError_t {
            cudaError_t e = enq_msd_pass(L, a, prefix);
            if (e) return e;
            return L.go(k_ctl_msd_next, 1, 1, 0, am);
        }))
        return rc;
    return capture_into(s, g, deps, [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = enq_tile(L, a, prefix, false))) return e;
        if ((e = enq_tile(L, a, prefix, true))) return e;
        if (prefix) return cudaSuccess;
        if ((e = L.go(k_mkeys, L.grid_msd, TPB, 0, a))) return e;
        if ((e = L.go(k_group_warp, L.grid_scan, TPB, 0, a))) return e;
        if (a.chain_from && (e = enq_chain(L, a, 0, 0))) return e;
        return L.go(k_group_thread, L.grid_msd, TPB, 0, a);
    });
}

// Graph: round 0 (the LSD sort and segmentation, or the tile path's init + prefix round), round end, then
// while (active) { rank round ; round end }, then the sampled indexes. The 1-thread round-end kernel sets the loop
// handle; the bucket-pass loops have their own handles.
int FwdEngine::build_graph(cudaStream_t s) {
    const u32 smax = (u32)cfg.tile_cap / 2;
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    KGB_CHECK(cudaGraphCreate(&graph, 0));
    // every handle created here belongs to exactly one conditional node below
    const bool lsd = lsd_enabled();
    cudaGraphConditionalHandle hround = 0, hmsd0 = 0, hmsd = 0;
    KGB_CHECK(cudaGraphConditionalHandleCreate(&hround, graph, 0, cudaGraphCondAssignDefault));
    if (!lsd) KGB_CHECK(cudaGraphConditionalHandleCreate(&hmsd0, graph, 0, cudaGraphCondAssignDefault));
    KGB_CHECK(cudaGraphConditionalHandleCreate(&hmsd, graph, 0, cudaGraphCondAssignDefault));
    FwdArgs a = make_args(d_ctl, d_T, d_blk, d_isa, d_L, d_SA, d_I, lists, d_hist, d_cursor, d_bhead, d_orand, d_dest,
                          B, smax);
    set_caps(a);
    FwdArgs ar = a;
    ar.hcond = (unsigned long long)hround;
    long long dummy = 0;
    Launcher L{s, grid_tile, grid_msd, grid_scan, cfg.tile_cap, grid_tile_prefix, grid_warp, grid_lsd, &dummy, nullptr};
    Deps deps;
    if (lsd) {
        if (int rc = capture_into(s, graph, deps, [&]() -> cudaError_t {
                cudaError_t e = enq_lsd_keys(L, a);
                if (e) return e;
                return enq_lsd_sort_seg(L, a, 0xFFFFFFFFu, 0);
            }))
            return rc;
    } else {
        if (int rc = capture_into(s, graph, deps, [&]() -> cudaError_t {
                return L.go(k_init, L.grid_msd, TPB, 0, a, (const u32 *)d_cursor, (const u8 *)d_dest);
            }))
            return rc;
        if (int rc = add_tile_round(s, graph, deps, L, a, true, hmsd0)) return rc;
    }
    if (int rc = capture_into(s, graph, deps, [&]() -> cudaError_t { return L.go(k_ctl_round_end, 1, 1, 0, ar); }))
        return rc;
    cudaGraph_t rbody;
    if (int rc = add_while(graph, deps, hround, &rbody)) return rc;
    Deps rd;
    if (int rc = add_tile_round(s, rbody, rd, L, a, false, hmsd)) return rc;
    if (int rc = capture_into(s, rbody, rd, [&]() -> cudaError_t { return L.go(k_ctl_round_end, 1, 1, 0, ar); }))
        return rc;
    if (int rc = capture_into(s, graph, deps, [&]() -> cudaError_t {
            return L.go(k_samples, (int)std::min<u32>(B, 1024u), 128, 0, a);
        }))
        return rc;
    KGB_CHECK(cudaGraphInstantiate(&gexec, graph, 0));
    return 0;
}

int FwdEngine::run(cudaStream_t s, bool use_graph) {
    stats = FwdStats{};
    if (!sm_count) {
        int dev;
        KGB_CHECK(cudaGetDevice(&dev));
        KGB_CHECK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
    }
    if (int rc = set_tile_attrs(cfg.tile_cap)) return rc;
    // persistent grids: as many CTAs as are resident at once (rank tiles: 3 per SM at 4096, prefix tiles: 2)
    grid_tile = sm_count * (cfg.tile_cap == 4096 ? std::min(std::max(cfg.tile_ctas, 1), 2) : 1);
    grid_tile_prefix = sm_count * (cfg.tile_cap == 4096 ? 2 : 1);
    grid_warp = sm_count * (cfg.tile_cap == 4096 ? 4 : 2);
    grid_lsd = (int)((N + LSD_TILE - 1) / LSD_TILE + B);  // at least the batch's sort tiles (one partial per block)
    grid_msd = sm_count * cfg.msd_ctas;
    grid_scan = sm_count * 4;
    // the host-side round-0 layout borrows the cursor/dest rows; they are rewritten by every bucket scan
    if (int rc = setup_round0(s)) return rc;
    if (!use_graph) return run_plain(s);
    const GraphKey key{N, Ncap, B, d_T, d_L, d_I, d_SA, cfg, lsd_enabled()};
    if (!gexec || !(key == graph_key)) {
        if (!(seen_valid && key == seen_key)) {  // first sight of this shape: plain launches, no capture
            seen_key = key;
            seen_valid = true;
            return run_plain(s);
        }
        // capture on the engine's own stream: the caller's may be the legacy default stream, which cannot capture
        if (!cap_stream) KGB_CHECK(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
        if (int rc = build_graph(cap_stream)) return rc;
        graph_key = key;
    }
    KGB_CHECK(cudaGraphLaunch(gexec, s));
    stats.launches = -1;
    return 0;
}

int FwdEngine::error_flag(cudaStream_t s, u32 *err) {
    KGB_CHECK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    KGB_CHECK(cudaStreamSynchronize(s));
    *err = h_ctl->err;
    stats.rounds = (int)h_ctl->round;
    return 0;
}

}  // namespace kgb
