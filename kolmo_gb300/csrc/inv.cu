// Inverse BWT on the GPU (sm_103a): psi table by a stable counting sort, then a parallel walk of many short chains.
//
// Conventions are the reference's (src/algo/sais/sais.c:12055-12082, the LF walk of tests/bwt_reference.py:270-290
// in adnaneben/kolmo): the L column is U with the sentinel re-inserted at row p0 = I[0]; row 0 of the sorted matrix
// is the sentinel rotation. Instead of LF (backwards) this decodes forwards with psi = LF^-1:
//   F row x holds the first byte of the suffix at row x, psi[x] is the row of the next suffix,
//   T[0] = F(p0), T[j + 1] = F(psi^(j+1)(p0)), and the walk ends at row 0 (the suffix of length 0).
// psi is built by a stable counting sort of the L column by byte (psi[C[c] + k] = row of the k-th c in L).
//
// Parallel decode (the chain idea of libsais's split decoder, sais.c:11573-11703, re-designed for a GPU):
//   * row p0 and about one row in MARK are marks; bit 31 of psi[x] flags "psi[x] is a mark" so a walk learns it
//     reached the next mark from the load it needs anyway. The regular marks are the rows (m * hmul) mod 2^k for
//     m = 1..n/MARK (2^k >= n, hmul odd near 2^k / golden ratio): a Weyl sequence, so the marks spread evenly over
//     every arithmetic progression of rows. Rows every MARK apart would leave whole stretches of a periodic text
//     unmarked (its rows interleave the periods), and one thread would walk each such stretch alone;
//   * one chain per mark walks psi until the next mark (or row 0), writing its bytes into its own CAPC-byte
//     buffer; a walk that reaches CAPC bytes closes its chain and continues as a new chain, so buffers never overflow
//     and no row is walked twice;
//   * chains are ranked by pointer jumping over (successor, length); a chain's text position is n minus its
//     distance to the end of the text;
//   * chains are copied to their positions.
// A string that is not a valid BWT has more than one psi cycle: the walk from p0 then reaches row 0 before n bytes.
// That block is reported (-1) instead of decoded. Every loop is bounded by the number of rows.
#include "inv.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>

#include "kgbwt.h"

namespace kgb {

constexpr int ITPB = 256;
constexpr u32 ITILE = 4096;
constexpr u32 MARK = 64;
// Small batches (at most SMALL_BATCH bytes, the drop-in call on a block of a few MiB) mark one row in MARK_SMALL and
// walk on the persistent grid (k_inv_walk_flat): they have too few chains to fill the GPU otherwise. Larger batches
// fill it with MARK and one CTA per work item (k_inv_walk), which is faster there (on a 64 MiB block: 3.38 ms for
// the whole inverse against 3.66 with the persistent walk, 3.99 with one mark in 32 and 4.93 with one in 16; on a
// 1 MiB block: 0.78 ms against 0.60, 0.50 and 0.46).
constexpr u32 MARK_SMALL = 16;
constexpr u64 SMALL_BATCH = 4u << 20;
constexpr u32 CAPC = 256;
constexpr u32 ENDC = 0xFFFFFFFFu;
constexpr u32 CHUNK = 1024;  // start chains per walk work item
constexpr int KSLOT = 4;     // chains walked at once by one thread
constexpr u32 CHUNKT = 16;   // tiles per chunk of the psi build

struct InvArgs {
    const u8 *U;
    u8 *out;
    u32 *psi;
    u32 *csum;
    const u32 *cblk;
    u32 *C;
    const InvBlock *blk;
    u32 B;
    u64 nchunk_all;
    u64 nchains;
    u32 *len, *succ, *dyn, *status;
    u32 *nx[2], *dist[2];
    u8 *buf;
    const u32 *chunks;
    u32 nchunks;
    u32 nwalk;  // chains in the walk's sequence over all blocks (sum of nreg + 1)
    u32 jpar;
    u64 cap_n;  // bytes of the text buffers (checked build)
};

// Chain id of a regular mark at row q (in 1..nreg when q is one).
__device__ __forceinline__ u32 mark_id(u32 q, const InvBlock &B) { return (q * B.hinv) & B.hmask; }
__device__ __forceinline__ u32 is_mark(u32 q, const InvBlock &B) {
    if (q == 0) return 0;
    const u32 m = mark_id(q, B);
    return q == B.p0 || (m >= 1 && m <= B.nreg);
}
// Start row of chain id (0: p0; m >= 1: the m-th regular mark, or none (0) when that row is past n or is p0).
__device__ __forceinline__ u32 chain_start(u32 id, const InvBlock &B) {
    if (id == 0) return B.p0;
    const u32 q = (id * B.hmul) & B.hmask;
    return q > B.n || q == B.p0 ? 0u : q;
}

// Per-chunk byte histograms (a chunk is CHUNKT consecutive tiles of one block).
__global__ void __launch_bounds__(ITPB) k_inv_chunkhist(InvArgs a) {
    __shared__ u32 h[256];
    const u32 lane = lane_id();
    for (u64 q = blockIdx.x; q < a.nchunk_all; q += gridDim.x) {
        const InvBlock B = a.blk[a.cblk[q]];
        const u32 start = (u32)(q - B.chunk_base) * (ITILE * CHUNKT);
        const u32 cnt = min(ITILE * CHUNKT, B.n - start);
        const u8 *src = a.U + (u64)B.off + start;
        h[threadIdx.x] = 0;
        __syncthreads();
        for (u32 i0 = 0; i0 < cnt; i0 += ITPB) {
            const u32 i = i0 + threadIdx.x;
            const u32 c = i < cnt ? (u32)src[i] : 0x100u;
            const u32 peers = __match_any_sync(0xffffffffu, c);
            if (c < 256 && (__ffs(peers) - 1) == (int)lane) atomicAdd(&h[c], __popc(peers));
        }
        __syncthreads();
        a.csum[q * 256 + threadIdx.x] = h[threadIdx.x];
        __syncthreads();
    }
}

// Per block: C array (C[c] = 1 + number of bytes below c: F row 0 is the sentinel) and the exclusive scan of the
// chunk histograms, so csum[q][c] becomes the first psi slot of chunk q's c bytes.
__global__ void __launch_bounds__(ITPB) k_inv_chunkscan(InvArgs a) {
    __shared__ u32 ws[ITPB / 32 + 1];
    const u32 c = threadIdx.x;
    for (u32 b = blockIdx.x; b < a.B; b += gridDim.x) {
        const InvBlock B = a.blk[b];
        u32 *col = a.csum + (u64)B.chunk_base * 256 + c;
        u32 tot = 0;
        u32 q = 0;
        for (; q + 8 <= B.nchunk; q += 8) {
            u32 v[8];
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = col[(u64)(q + k) * 256];
#pragma unroll
            for (int k = 0; k < 8; k++) tot += v[k];
        }
        for (; q < B.nchunk; q++) tot += col[(u64)q * 256];
        u32 all;
        const u32 cc = 1 + block_excl_sum<ITPB>(tot, ws, &all);
        a.C[(u64)b * 257 + c] = cc;
        if (c == 255) a.C[(u64)b * 257 + 256] = 1 + all;
        u32 run = cc;
        q = 0;
        for (; q + 8 <= B.nchunk; q += 8) {
            u32 v[8];
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = col[(u64)(q + k) * 256];
#pragma unroll
            for (int k = 0; k < 8; k++) { col[(u64)(q + k) * 256] = run; run += v[k]; }
        }
        for (; q < B.nchunk; q++) {
            const u32 v = col[(u64)q * 256];
            col[(u64)q * 256] = run;
            run += v;
        }
        if (c == 0) a.psi[(u64)B.off + b] = B.p0 | 0x80000000u;  // psi[0]: the sentinel row leads to row p0
    }
}

// Stable scatter, one CTA per chunk walking its tiles in order: psi[C[c] + occurrences of c before row q] = q,
// with the mark flag of q.
__global__ void __launch_bounds__(ITPB) k_inv_scatter(InvArgs a) {
    constexpr int NW = ITPB / 32, IPT = ITILE / ITPB, WS = 32 * IPT;
    __shared__ u16 wc[NW][256];
    __shared__ u32 woff[NW][256];
    __shared__ u32 run_s[256];
    const u32 lane = lane_id(), warp = warp_id();
    for (u64 q = blockIdx.x; q < a.nchunk_all; q += gridDim.x) {
        const u32 b = a.cblk[q];
        const InvBlock B = a.blk[b];
        const u32 cstart = (u32)(q - B.chunk_base) * (ITILE * CHUNKT);
        const u32 ccnt = min(ITILE * CHUNKT, B.n - cstart);
        run_s[threadIdx.x] = a.csum[q * 256 + threadIdx.x];
        u32 *psi = a.psi + (u64)B.off + b;
        for (u32 t0 = 0; t0 < ccnt; t0 += ITILE) {
            const u32 start = cstart + t0;
            const u32 cnt = min(ITILE, ccnt - t0);
            for (int i = threadIdx.x; i < NW * 256; i += ITPB) (&wc[0][0])[i] = 0;
            __syncthreads();
            u32 cs[IPT], rk[IPT];
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = warp * WS + j * 32 + lane;
                const u32 c = x < cnt ? (u32)a.U[(u64)B.off + start + x] : 0x100u;
                cs[j] = c;
                const u32 peers = __match_any_sync(0xffffffffu, c);
                const u32 before = c < 256 ? wc[warp][c] : 0u;
                rk[j] = before + __popc(peers & lanemask_lt());
                __syncwarp();
                if (c < 256 && (__ffs(peers) - 1) == (int)lane) wc[warp][c] = (u16)(before + __popc(peers));
                __syncwarp();
            }
            __syncthreads();
            {
                u32 run = run_s[threadIdx.x];
#pragma unroll
                for (int w = 0; w < NW; w++) { woff[w][threadIdx.x] = run; run += wc[w][threadIdx.x]; }
                run_s[threadIdx.x] = run;
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const u32 x = warp * WS + j * 32 + lane;
                if (x < cnt) {
                    const u32 u = start + x;
                    const u32 qr = u + (u >= B.p0);
                    const u32 dst = woff[warp][cs[j]] + rk[j];
                    KGB_GUARD(dst >= 1 && dst <= B.n, &a.status[b], 0x100) psi[dst] = qr | (is_mark(qr, B) << 31);
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ u32 f_of(const u32 *Cs, u32 row) {  // largest c with C[c] <= row
    u32 lo = 0;
#pragma unroll
    for (u32 step = 128; step; step >>= 1)
        if (Cs[lo + step] <= row) lo += step;
    return lo;
}

// Walk every chain of a work item (block, [c0, c1) start chains). Chain 0 starts at p0; chain m >= 1 at its mark
// (none when that row is past n or is p0). Chains that reach CAPC bytes continue under a new id taken from the block's counter.
__global__ void __launch_bounds__(ITPB) k_inv_walk(InvArgs a) {
    __shared__ u32 Cs[257];
    for (u32 w = blockIdx.x; w < a.nchunks; w += gridDim.x) {
        const u32 b = a.chunks[3 * w], c0 = a.chunks[3 * w + 1], c1 = a.chunks[3 * w + 2];
        const InvBlock B = a.blk[b];
        __syncthreads();
        for (u32 i = threadIdx.x; i < 257; i += ITPB) Cs[i] = a.C[(u64)b * 257 + i];
        __syncthreads();
        const u32 *psi = a.psi + (u64)B.off + b;
        u32 next = c0 + threadIdx.x;
        u32 row[KSLOT], steps[KSLOT], acc[KSLOT], cid[KSLOT];
        bool act[KSLOT];
#pragma unroll
        for (int k = 0; k < KSLOT; k++) {
            act[k] = false;
            while (next < c1) {
                const u32 id = next;
                next += ITPB;
                const u32 start = chain_start(id, B);
                if (start == 0) continue;  // no such row, or chain 0 covers the mark at p0
                row[k] = start; steps[k] = 0; acc[k] = 0; cid[k] = id; act[k] = true;
                break;
            }
        }
        for (;;) {
            bool any = false;
            u32 v[KSLOT];
#pragma unroll
            for (int k = 0; k < KSLOT; k++)
                if (act[k]) { v[k] = __ldg(psi + row[k]); any = true; }
            if (!any) break;
#pragma unroll
            for (int k = 0; k < KSLOT; k++) {
                if (!act[k]) continue;
                const u64 g = (u64)B.chain_base + cid[k];
                const u32 c = f_of(Cs, row[k]);
                acc[k] |= c << (8 * (steps[k] & 3));
                if ((steps[k] & 3) == 3) {
                    reinterpret_cast<u32 *>(a.buf + g * CAPC)[steps[k] >> 2] = acc[k];
                    acc[k] = 0;
                }
                steps[k]++;
                u32 nxt = v[k] & 0x7FFFFFFFu;
                if (nxt > B.n) {  // psi entries are rows 0..n: anything else is an internal error
                    a.status[b] = 3;
                    nxt = 0;
                }
                const bool stop = (v[k] >> 31) || nxt == 0;
                if (stop || steps[k] == CAPC) {
                    if (steps[k] & 3) reinterpret_cast<u32 *>(a.buf + g * CAPC)[steps[k] >> 2] = acc[k];
                    a.len[g] = steps[k];
                    if (stop) {
                        a.succ[g] = nxt == 0 ? ENDC : B.chain_base + (nxt == B.p0 ? 0u : mark_id(nxt, B));
                        act[k] = false;
                        while (next < c1) {
                            const u32 id = next;
                            next += ITPB;
                            const u32 start = chain_start(id, B);
                            if (start == 0) continue;
                            row[k] = start; steps[k] = 0; acc[k] = 0; cid[k] = id; act[k] = true;
                            break;
                        }
                    } else {
                        const u32 nid = B.nreg + 1 + atomicAdd(&a.dyn[b], 1u);
                        if (nid >= B.chain_cap) {  // cannot happen for any input: each record covers CAPC rows
                            a.status[b] = 2;
                            a.succ[g] = ENDC;
                            act[k] = false;
                        } else {
                            a.succ[g] = B.chain_base + nid;
                            cid[k] = nid; row[k] = nxt; steps[k] = 0; acc[k] = 0;
                        }
                    }
                } else {
                    row[k] = nxt;
                }
            }
        }
    }
}

// The block whose walk range holds chain q of the sequence over all blocks (blocks in order of qbase).
__device__ __forceinline__ u32 walk_block(const InvArgs &a, u32 q) {
    u32 lo = 0, hi = a.B - 1;
    while (lo < hi) {
        const u32 mid = (lo + hi + 1) >> 1;
        if (__ldg(&a.blk[mid].qbase) <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The walk as one sequence of chains over all blocks, on a persistent grid: thread t walks chains t, t + T,
// t + 2T, ... (T threads in all), KSLOT at a time, and a slot takes the thread's next chain as soon as its chain
// ends. Small batches use it: the work-item kernel above runs one CTA per 1024 chains, a few CTAs for a block of
// a few MiB, while this one spreads the chains over every SM. Each step is the same as there.
__global__ void __launch_bounds__(ITPB) k_inv_walk_flat(InvArgs a) {
    __shared__ u32 Cs0[257];
    const bool one = a.B == 1;  // a single block keeps its C array in shared memory
    if (one) {
        for (u32 i = threadIdx.x; i < 257; i += ITPB) Cs0[i] = a.C[i];
        __syncthreads();
    }
    const u32 T = gridDim.x * ITPB;
    u32 q = blockIdx.x * ITPB + threadIdx.x;
    // per slot: current row, bytes so far, the word being filled, chain record, block, psi offset, block length
    u32 row[KSLOT], steps[KSLOT], acc[KSLOT], grec[KSLOT], bk[KSLOT], pb[KSLOT], bn[KSLOT];
    bool act[KSLOT];
    // the thread's next chain into slot k (none left: the slot stays idle)
#define KGB_TAKE(k)                                                                                              \
    do {                                                                                                         \
        act[k] = false;                                                                                          \
        while (q < a.nwalk) {                                                                                    \
            const u32 b_ = one ? 0u : walk_block(a, q);                                                          \
            const InvBlock B_ = a.blk[b_];                                                                       \
            const u32 id_ = q - B_.qbase;                                                                        \
            q += T;                                                                                              \
            const u32 st_ = chain_start(id_, B_);                                                                \
            if (st_ == 0) continue; /* no such row, or chain 0 covers the mark at p0 */                        \
            row[k] = st_; steps[k] = 0; acc[k] = 0; grec[k] = B_.chain_base + id_; bk[k] = b_;                 \
            pb[k] = B_.off + b_; bn[k] = B_.n; act[k] = true;                                                   \
            break;                                                                                               \
        }                                                                                                        \
    } while (0)
#pragma unroll
    for (int k = 0; k < KSLOT; k++) KGB_TAKE(k);
    for (;;) {
        bool any = false;
        u32 v[KSLOT];
#pragma unroll
        for (int k = 0; k < KSLOT; k++)
            if (act[k]) { v[k] = __ldg(a.psi + pb[k] + row[k]); any = true; }
        if (!any) break;
#pragma unroll
        for (int k = 0; k < KSLOT; k++) {
            if (!act[k]) continue;
            const u32 *Cs = one ? Cs0 : a.C + (u64)bk[k] * 257;
            acc[k] |= f_of(Cs, row[k]) << (8 * (steps[k] & 3));
            steps[k]++;
            u32 nxt = v[k] & 0x7FFFFFFFu;
            if (nxt > bn[k]) {  // psi entries are rows 0..n: anything else is an internal error
                a.status[bk[k]] = 3;
                nxt = 0;
            }
            const bool stop = (v[k] >> 31) || nxt == 0;
            if ((steps[k] & 3) == 0 || stop || steps[k] == CAPC) {
                const u64 g = grec[k];
                reinterpret_cast<u32 *>(a.buf + g * CAPC)[(steps[k] - 1) >> 2] = acc[k];
                acc[k] = 0;
                if (stop || steps[k] == CAPC) {
                    const InvBlock B = a.blk[bk[k]];
                    a.len[g] = steps[k];
                    if (stop) {
                        a.succ[g] = nxt == 0 ? ENDC : B.chain_base + (nxt == B.p0 ? 0u : mark_id(nxt, B));
                        KGB_TAKE(k);
                    } else {
                        const u32 nid = B.nreg + 1 + atomicAdd(&a.dyn[bk[k]], 1u);
                        if (nid >= B.chain_cap) {  // cannot happen for any input: each record covers CAPC rows
                            a.status[bk[k]] = 2;
                            a.succ[g] = ENDC;
                            act[k] = false;
                        } else {
                            a.succ[g] = B.chain_base + nid;
                            grec[k] = B.chain_base + nid; row[k] = nxt; steps[k] = 0;
                        }
                    }
                    continue;
                }
            }
            row[k] = nxt;
        }
    }
#undef KGB_TAKE
}

__global__ void k_inv_rank_init(InvArgs a) {
    for (u64 g = (u64)blockIdx.x * blockDim.x + threadIdx.x; g < a.nchains; g += (u64)gridDim.x * blockDim.x) {
        a.nx[0][g] = a.succ[g];
        a.dist[0][g] = a.len[g];
    }
}

// One pointer-jumping step: dist[g] += dist[nx[g]], nx[g] = nx[nx[g]] (saturating; chains off the main path may
// form cycles and are discarded later).
__global__ void k_inv_jump(InvArgs a) {
    const u32 *nxi = a.nx[a.jpar], *di = a.dist[a.jpar];
    u32 *nxo = a.nx[a.jpar ^ 1], *dout = a.dist[a.jpar ^ 1];
    for (u64 g = (u64)blockIdx.x * blockDim.x + threadIdx.x; g < a.nchains; g += (u64)gridDim.x * blockDim.x) {
        const u32 x = nxi[g];
        const u32 d = di[g];
        if (x == ENDC) { nxo[g] = ENDC; dout[g] = d; continue; }
        const u64 s = (u64)d + di[x];
        nxo[g] = nxi[x];
        dout[g] = s > 0xFFFFFFFFull ? 0xFFFFFFFFu : (u32)s;
    }
}

// Copy every chain on the main path to its text position (one warp per chain) and set the block status.
__global__ void k_inv_emit(InvArgs a) {
    const u32 lane = lane_id();
    const u32 *nx = a.nx[a.jpar], *dist = a.dist[a.jpar];
    const u64 wid = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 g = wid; g < a.nchains; g += nw) {
        u32 lo = 0, hi = a.B - 1;  // block of chain g: last block with chain_base <= g
        while (lo < hi) {
            u32 mid = (lo + hi + 1) >> 1;
            if (a.blk[mid].chain_base <= g) lo = mid; else hi = mid - 1;
        }
        const InvBlock B = a.blk[lo];
        if (g >= (u64)B.chain_base + B.chain_cap) continue;
        const u32 x = nx[g], d = dist[g], L = a.len[g];
        if (g == B.chain_base && lane == 0 && a.status[lo] != 2) a.status[lo] = (x == ENDC && d == B.n) ? 0 : 1;
        if (x != ENDC || L == 0 || d > B.n || L > d) continue;
        const u64 dst = (u64)B.off + (B.n - d);
        const u8 *src = a.buf + g * CAPC;
        if (!KGB_OK(L <= CAPC && dst + L <= a.cap_n, &a.status[lo], 0x100)) continue;
        for (u32 i = lane; i < L; i += 32) a.out[dst + i] = src[i];
    }
}

// ------------------------------------------------------------------------------------------------ host engine
static size_t ialign(size_t x, size_t al) { return (x + al - 1) / al * al; }

InvEngine::InvEngine() {}
InvEngine::~InvEngine() { free_all(); }

void InvEngine::free_all() {
    if (cap_stream) cudaStreamDestroy(cap_stream);
    cap_stream = nullptr;
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr; graph = nullptr;
    if (pool) cudaFree(pool);
    pool = nullptr;
    if (h_status) cudaFreeHost(h_status);
    h_status = nullptr;
    Ncap = Tcap = Ccap = 0; Bcap = 0;
}

// The workspace for ncap text bytes, bcap blocks, tcap psi-build chunks and ccap chain records, in pool order.
template <typename Add>
void InvEngine::layout(u64 ncap, u32 bcap, u64 tcap, u64 ccap, Add add) {
    add((void **)&own_U, ncap + 64);
    add((void **)&own_out, ncap + 64);
    add((void **)&d_psi, (ncap + bcap + 16) * 4);
    add((void **)&d_csum, tcap * 256 * 4);
    add((void **)&d_cblk, tcap * 4);
    add((void **)&d_C, (size_t)bcap * 257 * 4);
    add((void **)&d_blk, (size_t)bcap * sizeof(InvBlock));
    add((void **)&d_len, ccap * 4);
    add((void **)&d_succ, ccap * 4);
    add((void **)&d_nx[0], ccap * 4);
    add((void **)&d_nx[1], ccap * 4);
    add((void **)&d_dist[0], ccap * 4);
    add((void **)&d_dist[1], ccap * 4);
    add((void **)&d_buf, ccap * CAPC);
    add((void **)&d_dyn, (size_t)bcap * 4);
    add((void **)&d_status, (size_t)bcap * 4);
    add((void **)&d_chunks, (ccap / CHUNK + bcap + 8) * 12);
}

int InvEngine::grow(u64 ncap, u32 bcap, u64 tcap, u64 ccap) {
    if (ncap <= Ncap && bcap <= Bcap && tcap <= Tcap && ccap <= Ccap) return 0;
    ncap = std::max(ncap, Ncap); bcap = std::max(bcap, Bcap); tcap = std::max(tcap, Tcap); ccap = std::max(ccap, Ccap);
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    if (pool) { cudaFree(pool); pool = nullptr; }
    struct Item { void **p; size_t bytes; };
    std::vector<Item> items;
    layout(ncap, bcap, tcap, ccap,
           [&](void **p, size_t bytes) { items.push_back({p, ialign(std::max<size_t>(bytes, 16), 256)}); });
    size_t total = 0;
    for (auto &it : items) total += it.bytes;
    cudaError_t e = cudaMalloc(&pool, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        pool = nullptr;
        Ncap = 0;
        return record_cuda_error(e, "cudaMalloc(inverse workspace)", __FILE__, __LINE__);
    }
    pool_bytes = total;
    size_t off = 0;
    for (auto &it : items) { *it.p = (char *)pool + off; off += it.bytes; }
    if (h_status) cudaFreeHost(h_status);
    KGB_CHECK(cudaMallocHost(&h_status, (size_t)bcap * sizeof(int)));
    Ncap = ncap; Bcap = bcap; Tcap = tcap; Ccap = ccap;
    return 0;
}

// Mark parameters of a block of B.n bytes: the smallest 2^k >= n, the Weyl multiplier and its inverse. Rows run
// 0..n; when n = 2^k, row n maps to id 0 and is never a regular mark.
static void mark_params(InvBlock &B) {
    int k = 1;
    while (k < 32 && (1ull << k) < B.n) k++;
    B.hmask = (u32)((1ull << k) - 1);
    B.hmul = (u32)(0x9E3779B97F4A7C15ull >> (64 - k)) | 1u;
    u32 inv = B.hmul;  // Newton iteration for the inverse mod 2^32 (each step doubles the correct low bits)
    for (int it = 0; it < 5; it++) inv *= 2u - B.hmul * inv;
    B.hinv = inv;
}

// A batch of at most SMALL_BATCH bytes (the persistent walk and denser marks).
static bool small_batch(const u32 *n, int count) {
    u64 t = 0;
    for (int b = 0; b < count; b++) t += n[b];
    return t <= SMALL_BATCH;
}

static int plan_layout(const u32 *off, const u32 *n, const u32 *p0, int count, std::vector<InvBlock> &blk,
                       std::vector<u32> &cblk, std::vector<u32> &chunks, u64 &nchunk_all, u64 &nchains, u32 &maxchains,
                       u32 &nwalk) {
    blk.resize(count);
    nwalk = 0;
    const u32 mark = small_batch(n, count) ? MARK_SMALL : MARK;
    cblk.clear();
    chunks.clear();
    nchunk_all = 0; nchains = 0; maxchains = 0;
    for (int b = 0; b < count; b++) {
        if (n[b] < 2 || p0[b] < 1 || p0[b] > n[b]) return -1;
        InvBlock B;
        B.off = off[b]; B.n = n[b]; B.p0 = p0[b];
        B.chunk_base = (u32)nchunk_all;
        B.nchunk = (n[b] + ITILE * CHUNKT - 1) / (ITILE * CHUNKT);
        B.nreg = n[b] / mark;
        mark_params(B);
        B.chain_base = (u32)nchains;
        B.chain_cap = B.nreg + 1 + n[b] / CAPC + 4;
        B.qbase = nwalk;
        nwalk += B.nreg + 1;
        for (u32 t = 0; t < B.nchunk; t++) cblk.push_back((u32)b);
        for (u32 c = 0; c < B.nreg + 1; c += CHUNK) {
            chunks.push_back((u32)b); chunks.push_back(c); chunks.push_back(std::min(B.nreg + 1, c + CHUNK));
        }
        nchunk_all += B.nchunk;
        nchains += B.chain_cap;
        maxchains = std::max(maxchains, B.chain_cap);
        blk[b] = B;
        if (nchunk_all > 0xFFFF0000ull || nchains > 0xFFFF0000ull || nwalk > 0xFFFF0000u) return -1;
    }
    return 0;
}

u64 InvEngine::estimate_bytes(const u32 *n, int count) {
    std::vector<u32> off(count), p0(count, 1);
    u64 o = 0;
    for (int b = 0; b < count; b++) { off[b] = (u32)o; o += ((u64)n[b] + 15) / 16 * 16; }
    std::vector<InvBlock> blk;
    std::vector<u32> cblk, chunks;
    u64 nch = 0, nchains_ = 0;
    u32 maxc = 0, nw = 0;
    if (plan_layout(off.data(), n, p0.data(), count, blk, cblk, chunks, nch, nchains_, maxc, nw)) return ~0ull;
    u64 total = 0;
    layout(std::max<u64>(o, Ncap), std::max<u32>((u32)count, Bcap), std::max<u64>(nch, Tcap),
           std::max<u64>(nchains_, Ccap),
           [&](void **, size_t bytes) { total += ialign(std::max<size_t>(bytes, 16), 256); });
    return total;
}

int InvEngine::plan(const u32 *n, const u32 *p0, int count) {
    if (count <= 0) return -1;
    h_off.resize(count);
    u64 off = 0;
    for (int b = 0; b < count; b++) {
        h_off[b] = (u32)off;
        off += ((u64)n[b] + 15) / 16 * 16;
        if (off > 0xFFFF0000ull) return -1;
    }
    std::vector<u32> cblk;
    if (plan_layout(h_off.data(), n, p0, count, h_blk, cblk, h_chunks, nchunk_all, nchains, maxchains, nwalk)) return -1;
    small = small_batch(n, count);
    N = off; B = (u32)count;
    int rc = grow(N, B, nchunk_all, nchains);
    if (rc) return rc;
    ext = false;
    d_U = own_U; d_out = own_out;
    KGB_CHECK(cudaMemcpy(d_cblk, cblk.data(), cblk.size() * 4, cudaMemcpyHostToDevice));
    return 0;
}

int InvEngine::plan_external(const u32 *off, const u32 *n, const u32 *p0, int count, u8 *dU, u8 *dOut) {
    if (count <= 0) return -1;
    h_off.assign(off, off + count);
    std::vector<u32> cblk;
    if (plan_layout(off, n, p0, count, h_blk, cblk, h_chunks, nchunk_all, nchains, maxchains, nwalk)) return -1;
    small = small_batch(n, count);
    u64 end = 0;
    for (int b = 0; b < count; b++) end = std::max<u64>(end, (u64)off[b] + n[b]);
    N = end; B = (u32)count;
    int rc = grow(N, B, nchunk_all, nchains);
    if (rc) return rc;
    ext = true;
    d_U = dU; d_out = dOut;
    KGB_CHECK(cudaMemcpy(d_cblk, cblk.data(), cblk.size() * 4, cudaMemcpyHostToDevice));
    return 0;
}

int InvEngine::enqueue(cudaStream_t s, long long *launches) {
    InvArgs a;
    memset(&a, 0, sizeof(a));
    a.U = d_U; a.out = d_out; a.psi = d_psi; a.csum = d_csum; a.cblk = d_cblk; a.C = d_C; a.blk = d_blk; a.B = B;
    a.nchunk_all = nchunk_all; a.nchains = nchains; a.len = d_len; a.succ = d_succ; a.dyn = d_dyn; a.status = d_status;
    a.nx[0] = d_nx[0]; a.nx[1] = d_nx[1]; a.dist[0] = d_dist[0]; a.dist[1] = d_dist[1]; a.buf = d_buf;
    a.chunks = d_chunks; a.nchunks = nchunks; a.nwalk = nwalk; a.jpar = 0; a.cap_n = Ncap;
    const int g4 = sm_count * 4;
    KGB_CHECK(cudaMemsetAsync(d_len, 0, nchains * 4, s));
    KGB_CHECK(cudaMemsetAsync(d_succ, 0xFF, nchains * 4, s));
    KGB_CHECK(cudaMemsetAsync(d_dyn, 0, (size_t)B * 4, s));
    KGB_CHECK(cudaMemsetAsync(d_status, 0, (size_t)B * 4, s));
    Profiler *P = prof_run ? &prof : nullptr;
    auto go = [&](int kid, u32 elems, auto fn) -> cudaError_t {
        (*launches)++;
        if (!P) { fn(); return cudaGetLastError(); }
        P->tag(kid, elems);
        return P->launch(s, [&]() -> cudaError_t { fn(); return cudaGetLastError(); });
    };
    const u32 nbytes = (u32)std::min<u64>(N, 0xFFFFFFFFull);
    const int gch = (int)std::min<u64>(nchunk_all, (u64)sm_count * 8);
    KGB_CHECK(go(K_INV_TILEHIST, nbytes, [&] { k_inv_chunkhist<<<gch, ITPB, 0, s>>>(a); }));
    KGB_CHECK(go(K_INV_COLSCAN, (u32)nchunk_all, [&] { k_inv_chunkscan<<<(int)std::min<u32>(B, 4096u), ITPB, 0, s>>>(a); }));
    KGB_CHECK(go(K_INV_SCATTER, nbytes, [&] { k_inv_scatter<<<gch, ITPB, 0, s>>>(a); }));
    if (small) {
        // the persistent grid: the CTAs the GPU holds at once, or fewer when there are fewer chains than threads
        const int gw = (int)std::max<u64>(1, std::min<u64>((u64)walk_grid, ((u64)nwalk + ITPB - 1) / ITPB));
        KGB_CHECK(go(K_INV_WALK, nbytes, [&] { k_inv_walk_flat<<<gw, ITPB, 0, s>>>(a); }));
    } else {
        KGB_CHECK(go(K_INV_WALK, nbytes, [&] { k_inv_walk<<<(int)std::min<u32>(nchunks, (u32)sm_count * 8), ITPB, 0, s>>>(a); }));
    }
    KGB_CHECK(go(K_INV_RANKINIT, (u32)nchains, [&] { k_inv_rank_init<<<g4, 256, 0, s>>>(a); }));
    for (u32 j = 0; j < njump; j++) {
        a.jpar = j & 1;
        KGB_CHECK(go(K_INV_JUMP, (u32)nchains, [&] { k_inv_jump<<<g4, 256, 0, s>>>(a); }));
    }
    a.jpar = njump & 1;
    KGB_CHECK(go(K_INV_EMIT, nbytes, [&] { k_inv_emit<<<g4, 256, 0, s>>>(a); }));
    return 0;
}

int InvEngine::run(cudaStream_t s, bool use_graph) {
    stats = InvStats{};
    if (!sm_count) {
        int dev;
        KGB_CHECK(cudaGetDevice(&dev));
        KGB_CHECK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
        int per_sm = 0;
        KGB_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_inv_walk_flat, ITPB, 0));
        walk_grid = std::max(per_sm, 1) * sm_count;
    }
    nchunks = (u32)(h_chunks.size() / 3);
    njump = 1;
    while ((1ull << njump) < (u64)maxchains + 1) njump++;
    njump += 1;
    stats.jumps = (int)njump;
    KGB_CHECK(cudaMemcpyAsync(d_blk, h_blk.data(), h_blk.size() * sizeof(InvBlock), cudaMemcpyHostToDevice, s));
    KGB_CHECK(cudaMemcpyAsync(d_chunks, h_chunks.data(), h_chunks.size() * 4, cudaMemcpyHostToDevice, s));
    KGB_CHECK(cudaStreamSynchronize(s));  // host vectors are pageable: finish before they can change
    prof.reset();
    prof_run = !use_graph && prof.on;
    if (!use_graph) return enqueue(s, &stats.launches);
    prof_run = false;
    const GraphKey key{N, Ncap, (u64)nchunk_all, (u64)nchains, (u32)B, njump, nchunks, d_U, d_out, small};
    if (!gexec || !(key == graph_key)) {
        if (!(seen_valid && key == seen_key)) {  // first sight of this shape: plain launches, no capture
            seen_key = key;
            seen_valid = true;
            return enqueue(s, &stats.launches);
        }
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        if (!cap_stream) KGB_CHECK(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
        KGB_CHECK(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
        long long dummy = 0;
        int rc = enqueue(cap_stream, &dummy);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(cap_stream, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        KGB_CHECK(e);
        graph = g;
        KGB_CHECK(cudaGraphInstantiate(&gexec, graph, 0));
        graph_key = key;
    }
    KGB_CHECK(cudaGraphLaunch(gexec, s));
    stats.launches = -1;
    return 0;
}

int InvEngine::fetch_status(cudaStream_t s, std::vector<int> &status) {
    KGB_CHECK(cudaMemcpyAsync(h_status, d_status, (size_t)B * sizeof(int), cudaMemcpyDeviceToHost, s));
    KGB_CHECK(cudaStreamSynchronize(s));
    status.assign(h_status, h_status + B);
    return 0;
}

}  // namespace kgb

// ------------------------------------------------------------------------------------------------ allocation-free
// Inverse BWT for callers that cannot allocate device memory: code that runs where cudaMalloc is not allowed or not
// wanted (a host that owns every device allocation through its own pool, a plugin loaded into such a host, a
// process that must not grow its device footprint after start-up). Its scratch is one file-scope device array
// sized for one block of at most NOALLOC_MAX_N bytes; every GPU that loads this library holds that array
// (about 2.5 MB) until the process exits. The caller passes device input and output buffers.
namespace kgb {

constexpr u32 NOALLOC_MAX_N = 1u << 18;  // 256 KiB
constexpr u32 NA_CHUNKS = (NOALLOC_MAX_N + ITILE * CHUNKT - 1) / (ITILE * CHUNKT);
constexpr u32 NA_NREG = NOALLOC_MAX_N / MARK;
constexpr u32 NA_CHAINS = NA_NREG + 1 + NOALLOC_MAX_N / CAPC + 4;
constexpr u32 NA_WALK = (NA_NREG + 1 + CHUNK - 1) / CHUNK;

struct NoAllocScratch {
    u32 psi[NOALLOC_MAX_N + 16];
    u32 csum[NA_CHUNKS * 256];
    u32 C[264];
    u32 cblk[NA_CHUNKS];
    u32 chunks[3 * NA_WALK];
    InvBlock blk[1];
    u32 len[NA_CHAINS], succ[NA_CHAINS], nx[2][NA_CHAINS], dist[2][NA_CHAINS];
    u32 dyn[4], status[4];
    u8 buf[(size_t)NA_CHAINS * CAPC];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// Device address of the scratch array, looked up once per device (with that device current).
static NoAllocScratch *noalloc_scratch(int *rc) {
    static std::mutex mu;
    static NoAllocScratch *addr[128] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { *rc = record_cuda_error(e, "cudaGetDevice", __FILE__, __LINE__); return nullptr; }
    if (dev < 0 || dev >= 128) { record_error("device index out of range"); *rc = -2; return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) { *rc = record_cuda_error(e, "cudaGetSymbolAddress", __FILE__, __LINE__); return nullptr; }
        addr[dev] = reinterpret_cast<NoAllocScratch *>(p);
    }
    *rc = 0;
    return addr[dev];
}

static int unbwt_noalloc(const u8 *dU, u8 *dT, u32 n, u32 p0, cudaStream_t s) {
    int rc = 0;
    NoAllocScratch *S = noalloc_scratch(&rc);
    if (!S) return rc;
    // host-side tables on the stack: one block, its chunk map and its walk work items
    InvBlock B;
    B.off = 0; B.n = n; B.p0 = p0;
    B.chunk_base = 0; B.nchunk = (n + ITILE * CHUNKT - 1) / (ITILE * CHUNKT);
    B.nreg = n / MARK; B.chain_base = 0; B.chain_cap = B.nreg + 1 + n / CAPC + 4; B.qbase = 0;
    mark_params(B);
    u32 cblk[NA_CHUNKS] = {0};
    u32 chunks[3 * NA_WALK];
    u32 nwalk = 0;
    for (u32 c = 0; c < B.nreg + 1; c += CHUNK, nwalk++) {
        chunks[3 * nwalk] = 0; chunks[3 * nwalk + 1] = c; chunks[3 * nwalk + 2] = std::min(B.nreg + 1, c + CHUNK);
    }
    u32 njump = 1;
    while ((1ull << njump) < (u64)B.chain_cap + 1) njump++;
    njump += 1;
    KGB_CHECK(cudaMemcpyAsync(S->blk, &B, sizeof(B), cudaMemcpyHostToDevice, s));
    KGB_CHECK(cudaMemcpyAsync(S->cblk, cblk, sizeof(u32) * B.nchunk, cudaMemcpyHostToDevice, s));
    KGB_CHECK(cudaMemcpyAsync(S->chunks, chunks, sizeof(u32) * 3 * nwalk, cudaMemcpyHostToDevice, s));
    // the array keeps the previous call's contents: reset what must start at zero (or at "no successor")
    KGB_CHECK(cudaMemsetAsync(S->len, 0, sizeof(u32) * B.chain_cap, s));
    KGB_CHECK(cudaMemsetAsync(S->succ, 0xFF, sizeof(u32) * B.chain_cap, s));
    KGB_CHECK(cudaMemsetAsync(S->dyn, 0, sizeof(S->dyn), s));
    KGB_CHECK(cudaMemsetAsync(S->status, 0, sizeof(S->status), s));
    InvArgs a;
    memset(&a, 0, sizeof(a));
    a.U = dU; a.out = dT; a.psi = S->psi; a.csum = S->csum; a.cblk = S->cblk; a.C = S->C; a.blk = S->blk; a.B = 1;
    a.nchunk_all = B.nchunk; a.nchains = B.chain_cap; a.len = S->len; a.succ = S->succ; a.dyn = S->dyn;
    a.status = S->status; a.nx[0] = S->nx[0]; a.nx[1] = S->nx[1]; a.dist[0] = S->dist[0]; a.dist[1] = S->dist[1];
    a.buf = S->buf; a.chunks = S->chunks; a.nchunks = nwalk; a.jpar = 0; a.cap_n = n;
    k_inv_chunkhist<<<B.nchunk, ITPB, 0, s>>>(a);
    k_inv_chunkscan<<<1, ITPB, 0, s>>>(a);
    k_inv_scatter<<<B.nchunk, ITPB, 0, s>>>(a);
    k_inv_walk<<<nwalk, ITPB, 0, s>>>(a);
    const int g = (int)((B.chain_cap + 255) / 256);
    k_inv_rank_init<<<g, 256, 0, s>>>(a);
    for (u32 j = 0; j < njump; j++) {
        a.jpar = j & 1;
        k_inv_jump<<<g, 256, 0, s>>>(a);
    }
    a.jpar = njump & 1;
    k_inv_emit<<<(int)std::min<u32>(1024u, (B.chain_cap + 7) / 8), 256, 0, s>>>(a);
    KGB_CHECK(cudaGetLastError());
    u32 status = 0;
    KGB_CHECK(cudaMemcpyAsync(&status, S->status, sizeof(u32), cudaMemcpyDeviceToHost, s));
    KGB_CHECK(cudaStreamSynchronize(s));
    if (status) { record_error("inverse BWT: not a valid BWT string for its primary index"); return -1; }
    return 0;
}

}  // namespace kgb

extern "C" int32_t kgbwt_unbwt_noalloc(const uint8_t *dU, uint8_t *dT, int32_t n, int32_t p0, void *stream) {
    if (!dU || !dT || n < 2 || p0 < 1 || p0 > n) {
        kgb::record_error("kgbwt_unbwt_noalloc: bad arguments (device buffers, n >= 2, 1 <= p0 <= n)");
        return -1;
    }
    if ((uint32_t)n > kgb::NOALLOC_MAX_N) {
        kgb::record_error("kgbwt_unbwt_noalloc: n exceeds the maximum of 262144 bytes of the static scratch");
        return -1;
    }
    // both buffers must be memory the device can address (device or managed allocations): a host pointer would
    // send the kernels to an address they cannot use
    for (const void *p : {(const void *)dU, (const void *)dT}) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
            (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            kgb::record_error("kgbwt_unbwt_noalloc: dU and dT must be device (or managed) memory");
            return -1;
        }
    }
    // every call reads its status back and waits for the stream, which a stream under capture does not allow
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        kgb::record_error("kgbwt_unbwt_noalloc: the stream is being captured; this call synchronises with it");
        return -1;
    }
    return kgb::unbwt_noalloc(dU, dT, (kgb::u32)n, (kgb::u32)p0, (cudaStream_t)stream);
}
