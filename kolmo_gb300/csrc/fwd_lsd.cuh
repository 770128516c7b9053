// Round 0 of the forward sort as one LSD radix sort: the suffixes of each block of the batch are sorted by their
// zero-padded W-byte prefix, W = 16 (or 12 or 8), with one pass per varying key byte (single-pass scatter with decoupled
// look-back), then a segmentation turns the sorted order into ranks, finished suffixes and the rank rounds' groups
// (tiny, medium, small and large lists). The sort tiles never straddle two blocks: every block's suffixes keep their
// own range of the dense order (the block's soff onward), a pass takes each tile's digit bases from its own block's
// counts and looks back only over the block's earlier tiles, so the block index is neither carried nor sorted. The
// passes move 8-byte (id, key) items whose key is the 4-byte group of prefix bytes the passes of that group sort:
// the first pass builds its items from the text (ids still in text order, so the loads coalesce), and the last pass
// of a group writes the next group's key, gathered from the text (which stays in L2 at these sizes), so each pass
// reads and writes 16 B per suffix. The segmentation compares the whole W-byte prefixes, read from the text. Sorting
// 16 bytes here replaces the first rank round (which would take the groups from 8 to 16 bytes) with eight passes over
// all suffixes. Included by fwd.cu inside namespace kgb, after the kernels it shares (FwdArgs, resolve, tile-map
// writers).
#pragma once
// (included inside namespace kgb)

constexpr int LSD_IPT = 16, LSD_TILE = TPB * LSD_IPT;  // elements per sort tile
// digit slots: slot s sorts prefix byte 15 - s, carried in key group (15 - s) / 4 (bytes 4g..4g+3, big-endian)
constexpr int NSLOT = 16;
static_assert(NSLOT <= 32, "the look-back epoch holds the slot in 5 bits");
constexpr int SEG_IPT = 16, SEG_TILE = TPB * SEG_IPT;  // positions per segmentation tile (SEG_IPT <= 32)
// look-back words: epoch (32 bits: call sequence << 5 | digit slot) | flag (2 bits) | value (30 bits); a word of another
// epoch (an earlier slot or call) counts as not yet published
constexpr u64 ST_AGG = 1ull << 30, ST_PRE = 2ull << 30, ST_VAL = (1ull << 30) - 1;
constexpr u64 ST_EPOCH = 0xFFFFFFFF00000000ull;
constexpr int LB_WIN = 8;  // look-back window (predecessor words read per step)

__device__ __forceinline__ u32 active_slots(const Ctl *c) { return c->lsd_act; }  // bit s: slot s varies

// The zero-padded 8-byte text word at position q of a block ending at end, as a big-endian word (0 past the end).
__device__ __forceinline__ u64 lsd_key(const u8 *__restrict__ T, u64 q, u64 end) {
    if (q >= end) return 0;
    u64 k = load_be64(T, q);
    const u64 rem = end - q;
    if (rem < 8) k &= ~0ull << (8 * (8 - rem));
    return k;
}
// The zero-padded 16-byte prefix at position q as two big-endian words (k: bytes 0-7, k2: bytes 8-15, 0 past the
// block end), from three aligned 8-byte loads; `two` false: k2 = 0 and only two loads. The third load is made only
// when byte q + 8 lies in the block, so no load reaches more than 15 bytes past the block's end (the padding that
// callers of the engine guarantee).
__device__ __forceinline__ void lsd_key16(const u8 *__restrict__ T, u64 q, u64 end, bool two, u64 &k, u64 &k2) {
    k = k2 = 0;
    if (q >= end) return;
    const u64 *p = reinterpret_cast<const u64 *>(T + (q & ~7ull));
    const u64 a = __ldg(p), b = __ldg(p + 1), c = two && end - q > 8 ? __ldg(p + 2) : 0ull;
    const u32 s = (u32)(q & 7) * 8;
    const u64 w0 = s ? (a >> s) | (b << (64 - s)) : a, w1 = s ? (b >> s) | (c << (64 - s)) : b;
    auto be = [](u64 w) {
        return ((u64)__byte_perm((u32)w, 0, 0x0123) << 32) | (u64)__byte_perm((u32)(w >> 32), 0, 0x0123);
    };
    const u64 rem = end - q;
    k = be(w0);
    if (rem < 8) k &= ~0ull << (8 * (8 - rem));
    if (two && rem > 8) {
        k2 = be(w1);
        if (rem < 16) k2 &= ~0ull << (8 * (16 - rem));
    }
}
// Key group g (prefix bytes 4g..4g+3) of the suffix at id, big-endian, zero past the block end.
__device__ __forceinline__ u32 lsd_group(const u8 *__restrict__ T, u32 id, u32 g, u64 end) {
    return (u32)(lsd_key(T, (u64)id + 4 * g, end) >> 32);
}
// Key group of slot s.
__device__ __forceinline__ u32 lsd_slot_group(int slot) { return (15u - (u32)slot) >> 2; }

// The block of sort tile t: the last block whose first tile (lt0) is <= t (blocks in batch order, lt0 ascending).
__device__ __forceinline__ u32 blk_of_tile(const FwdArgs &a, u32 t) {
    u32 lo = 0, hi = a.B - 1;
    while (lo < hi) {
        const u32 mid = (lo + hi + 1) >> 1;
        if (__ldg(&a.blk[mid].lt0) <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}
// The block holding dense position p, searched within blocks [lo, hi]: the last block whose soff is <= p.
__device__ __forceinline__ u32 blk_of_pos(const FwdArgs &a, u32 p, u32 lo, u32 hi) {
    while (lo < hi) {
        const u32 mid = (lo + hi + 1) >> 1;
        if (__ldg(&a.blk[mid].soff) <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}
// A sort tile: its block, first dense position and element count.
struct LsdTile {
    u32 b, base, cnt;
};
__device__ __forceinline__ LsdTile lsd_tile(const FwdArgs &a, u32 t) {
    LsdTile r;
    r.b = blk_of_tile(a, t);
    const BlockInfo bi = a.blk[r.b];
    const u32 k = (t - bi.lt0) * (u32)LSD_TILE;
    r.base = bi.soff + k;
    r.cnt = min((u32)LSD_TILE, bi.n - k);
    return r;
}

// Start: clear the blocks' byte histograms, the tile counters, the active mask and the resolved count.
__global__ void k_lsd_begin(FwdArgs a) {
    Ctl *c = a.ctl;
    const u64 nh = (u64)a.B * 256;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += (u64)gridDim.x * blockDim.x) a.lhist[i] = 0;
    if (blockIdx.x == 0) {
        if (threadIdx.x < NSLOT) a.ltile[threadIdx.x] = 0;
        if (threadIdx.x == 0) {
            // round 0 lists no finished suffixes: with every id counted as finished, round 1's fixup copies the
            // whole rank buffer
            c->cnt[L_R0 + c->rpar] = a.idn;
            c->lsd_act = 0;
            c->m = a.blk[a.B - 1].soff + a.blk[a.B - 1].n;
        }
    }
}

// Each block's byte histogram, from which every pass's digit counts follow, and row 0 of its L column. CTA c takes a
// contiguous run of sort tiles and adds its shared histogram into a block's row when the run leaves it.
__global__ void __launch_bounds__(TPB) k_lsd_key0(FwdArgs a) {
    __shared__ u32 hs[256];
    const u32 nt = a.ctl->lsd_tiles;
    const u32 per = (nt + gridDim.x - 1) / gridDim.x;
    const u32 t0 = blockIdx.x * per, t1 = min(nt, t0 + per);
    hs[threadIdx.x] = 0;
    __syncthreads();
    u32 cur = ~0u;  // block whose counts hs holds
    for (u32 t = t0; t < t1; t++) {
        const LsdTile tl = lsd_tile(a, t);
        if (tl.b != cur) {
            if (cur != ~0u) {
                __syncthreads();
                const u32 v = hs[threadIdx.x];
                if (v) atomicAdd(&a.lhist[(u64)cur * 256 + threadIdx.x], v);
                hs[threadIdx.x] = 0;
                __syncthreads();
            }
            cur = tl.b;
        }
        const BlockInfo bi = a.blk[tl.b];
        const u64 end = (u64)bi.off + bi.n;
        // row 0 of the L column (the sentinel rotation) holds the block's last byte
        if (t == bi.lt0 && threadIdx.x == 0) a.L[(u64)bi.off + tl.b] = a.T[end - 1];
        const u32 id0 = bi.off + (tl.base - bi.soff);
        for (u32 j = threadIdx.x; j < tl.cnt; j += TPB) atomicAdd(&hs[__ldg(a.T + id0 + j)], 1u);
    }
    __syncthreads();
    if (cur != ~0u && hs[threadIdx.x]) atomicAdd(&a.lhist[(u64)cur * 256 + threadIdx.x], hs[threadIdx.x]);
}

// Digit bases of every pass and the active slots (256 threads per CTA, thread = digit value, CTAs over blocks).
// Suffix i of a block of n bytes has key byte d = T[i + d] when i + d < n, else 0, so the counts of key byte d are
// the block's byte counts minus those of its first min(d, n) bytes, plus min(d, n) zeros; their exclusive scan plus
// the block's soff gives the pass's first position of every digit (lbase row (block, slot), slot = 15 - d). A slot
// runs when its key byte takes two or more values within some block (slots 16 - W..15 only).
__global__ void __launch_bounds__(TPB) k_lsd_hist0(FwdArgs a) {
    __shared__ u32 wm[8];
    __shared__ u32 ws[TPB / 32 + 1];
    const u32 x = threadIdx.x;
    const int first = 16 - (int)a.lsd_bytes;
    for (u32 b = blockIdx.x; b < a.B; b += gridDim.x) {
        const BlockInfo bi = a.blk[b];
        const u32 h = a.lhist[(u64)b * 256 + x];
        u32 pre = 0, mask = 0;  // pre: bytes x among the block's first d bytes
        for (int slot = 15; slot >= first; slot--) {
            const u32 d = 15 - slot;
            if (d >= 1 && d <= bi.n) pre += __ldg(a.T + (u64)bi.off + d - 1) == x;
            const u32 v = h - pre + (x == 0 ? min(d, bi.n) : 0u);
            if (v != 0 && v != bi.n) mask |= 1u << slot;
            a.lbase[((u64)b * NSLOT + slot) * 256 + x] = bi.soff + block_excl_sum<TPB>(v, ws, nullptr);
        }
        for (int o = 16; o; o >>= 1) mask |= __shfl_xor_sync(0xffffffffu, mask, o);
        if ((x & 31) == 0) wm[x >> 5] = mask;
        __syncthreads();
        if (x == 0) {
            u32 m = 0;
            for (int w = 0; w < 8; w++) m |= wm[w];
            if (m & ~a.ctl->lsd_act) atomicOr(&a.ctl->lsd_act, m);
        }
        __syncthreads();
    }
}

// When no key byte varies within any block, no pass runs: the sorted order is the text order (ids written here for
// the segmentation). Otherwise returns at once.
__global__ void __launch_bounds__(TPB) k_lsd_ident(FwdArgs a) {
    const Ctl *c = a.ctl;
    if (active_slots(c)) return;
    const u32 nt = c->lsd_tiles;
    for (u32 t = blockIdx.x; t < nt; t += gridDim.x) {
        const LsdTile tl = lsd_tile(a, t);
        const u32 id0 = a.blk[tl.b].off + (tl.base - a.blk[tl.b].soff);
        for (u32 j = threadIdx.x; j < tl.cnt; j += TPB) __stcs(a.lval[0] + tl.base + j, id0 + j);
    }
}

struct LsdSmem {
    unsigned long long item[LSD_TILE];
    u16 wcnt[TPB / 32][256];
    u32 gbase[256];
    u32 ws[TPB / 32 + 1];
    u32 tile;
};

// One sort tile of an LSD pass over digit `slot`: rank the tile's suffixes by digit, publish the tile's digit counts,
// look back over the block's earlier tiles for the offsets (bounded spin), stage the tile in shared memory in digit
// order and write it out in runs. FULL: the tile holds LSD_TILE suffixes (every tile but a block's last), so no
// element needs a bounds check.
template <bool FULL>
__device__ __forceinline__ void lsd_pass_tile(const FwdArgs &a, LsdSmem &S, int slot, u32 act, u64 epoch, u32 tile,
                                              const LsdTile &tl) {
    const u32 lower = act & ((1u << slot) - 1), higher = act & ~((2u << slot) - 1);
    const u32 par = __popc(lower) & 1;
    const u32 tid = threadIdx.x, lane = lane_id(), warp = warp_id();
    const u32 base = tl.base, cnt = FULL ? (u32)LSD_TILE : tl.cnt;
    const bool head = tile == __ldg(&a.blk[tl.b].lt0);  // the block's first tile: its counts are the inclusive prefix
    // this pass's first position of digit tid in the block
    const u32 dbase = __ldg(a.lbase + ((u64)tl.b * NSLOT + slot) * 256 + tid);
    const unsigned long long *iin = a.lit[par];
    // rr: each item's rank in its warp's digit bucket (< 512), two 16-bit ranks per register; the digit itself is
    // recomputed from the key where it is needed
    u32 v[LSD_IPT], rr[LSD_IPT / 2], k[LSD_IPT];
    const u32 dsh = 8 * (slot & 3);  // byte 15 - slot of the prefix within the key group
    if (!lower) {
        // the first pass: the tile's suffixes are still in text order, ids and keys come from the text
        const BlockInfo bi = a.blk[tl.b];
        const u32 id0 = bi.off + (base - bi.soff);
        const u64 end = (u64)bi.off + bi.n;
        const u32 g = lsd_slot_group(slot);
#pragma unroll
        for (int j = 0; j < LSD_IPT; j++) {
            const u32 x = warp * (32 * LSD_IPT) + j * 32 + lane;
            v[j] = id0 + x;
            k[j] = (FULL || x < cnt) ? lsd_group(a.T, id0 + x, g, end) : 0u;
        }
    } else {
#pragma unroll
        for (int j = 0; j < LSD_IPT; j++) {
            const u32 x = warp * (32 * LSD_IPT) + j * 32 + lane;
            const bool ok = FULL || x < cnt;
            const unsigned long long it = ok ? __ldcs(iin + base + x) : 0ull;
            v[j] = (u32)it;
            k[j] = (u32)(it >> 32);
        }
    }
#pragma unroll
    for (int j = 0; j < LSD_IPT; j++) {
        const u32 x = warp * (32 * LSD_IPT) + j * 32 + lane;
        const u32 d = (FULL || x < cnt) ? (k[j] >> dsh) & 0xFFu : 0x100u;  // 0x100: past the tile's end
        const u32 peers = __match_any_sync(0xffffffffu, d);
        const u32 before = (FULL || d < 256) ? S.wcnt[warp][d] : 0u;
        const u32 r = before + __popc(peers & lanemask_lt());
        if (j & 1) rr[j >> 1] |= r << 16; else rr[j >> 1] = r;
        __syncwarp();
        if ((FULL || d < 256) && (__ffs(peers) - 1) == (int)lane) S.wcnt[warp][d] = (u16)(before + __popc(peers));
        __syncwarp();
    }
    __syncthreads();
    // thread tid owns digit tid: tile count, publish, local start, look back
    u32 tot = 0;
#pragma unroll
    for (int w = 0; w < TPB / 32; w++) tot += S.wcnt[w][tid];
    u64 *st = a.lstat + (u64)tile * 256 + tid;
    if (head) atomicExch((unsigned long long *)st, epoch | ST_PRE | tot);
    else atomicExch((unsigned long long *)st, epoch | ST_AGG | tot);
    const u32 dstart = block_excl_sum<TPB>(tot, S.ws, nullptr);
    {
        u32 run = dstart;
#pragma unroll
        for (int w = 0; w < TPB / 32; w++) { const u32 cc = S.wcnt[w][tid]; S.wcnt[w][tid] = (u16)run; run += cc; }
    }
    __syncthreads();
    // stage in digit order (tile-local offsets only: the items leave registers before the look-back)
#pragma unroll
    for (int j = 0; j < LSD_IPT; j++) {
        const u32 x = warp * (32 * LSD_IPT) + j * 32 + lane;
        if (FULL || x < cnt) {
            const u32 d = (k[j] >> dsh) & 0xFFu;
            const u32 p = S.wcnt[warp][d] + ((rr[j >> 1] >> (16 * (j & 1))) & 0xFFFFu);
            S.item[p] = (unsigned long long)k[j] << 32 | v[j];
        }
    }
    u32 excl = 0;
    if (!head) {
        // windowed look-back: read LB_WIN predecessors' words at once, add aggregates in order up to the first
        // inclusive prefix (at the latest the block's first tile); a word not yet published ends the window and the
        // walk resumes there
        long j = (long)tile - 1;
        u32 spins = 0;
        while (true) {
            u64 w[LB_WIN];
#pragma unroll
            for (int q = 0; q < LB_WIN; q++)
                w[q] = j - q >= 0 ? *(volatile u64 *)(a.lstat + (u64)(j - q) * 256 + tid) : 0ull;
            int used = 0;
            bool done = false;
#pragma unroll
            for (int q = 0; q < LB_WIN; q++) {
                if (done || used < q) continue;  // stopped earlier in the window
                const u64 x = w[q];
                if ((x & ST_EPOCH) != epoch || !(x & (ST_AGG | ST_PRE))) continue;
                excl += (u32)(x & ST_VAL);
                used = q + 1;
                if (x & ST_PRE) done = true;
            }
            if (done) break;
            j -= used;
            if (used == 0) {
                if (++spins > a.spin_limit) {  // a predecessor never published: report and stop waiting
                    atomicOr(&a.ctl->err, 256u);
                    break;
                }
                __nanosleep(32);
            }
        }
        atomicExch((unsigned long long *)st, epoch | ST_PRE | (u64)(excl + tot));
    }
    S.gbase[tid] = dbase + excl - dstart;
    __syncthreads();
    unsigned long long *iout = a.lit[par ^ 1];
    const BlockInfo bi = a.blk[tl.b];
    const u32 bend = bi.soff + bi.n;  // bound of the checked build's write checks
    (void)bend;
    // the key the next pass reads: this group's (carried), the next group's (gathered from the text) or none
    const u32 g = lsd_slot_group(slot);
    const int gn = higher ? (int)lsd_slot_group(__ffs(higher) - 1) : -1;
    if (gn == (int)g) {
        for (u32 i = tid; i < cnt; i += TPB) {
            const unsigned long long it = S.item[i];
            const u32 dst = S.gbase[((u32)(it >> 32) >> dsh) & 0xFFu] + i;
            if (KGB_OK(dst < bend, &a.ctl->err, E_LIST)) __stcs(iout + dst, it);
        }
    } else if (gn >= 0) {
        const u64 end = (u64)bi.off + bi.n;
        constexpr int WB = 4;  // gathers in flight per thread
        for (u32 i0 = tid; i0 < cnt; i0 += WB * TPB) {
            u32 id[WB], kk[WB], dst[WB];
#pragma unroll
            for (int q = 0; q < WB; q++) {
                const u32 i = i0 + q * TPB;
                const bool ok = i < cnt;
                const unsigned long long it = ok ? S.item[i] : 0ull;
                id[q] = (u32)it;
                dst[q] = ok ? S.gbase[((u32)(it >> 32) >> dsh) & 0xFFu] + i : 0u;
                kk[q] = ok ? lsd_group(a.T, id[q], (u32)gn, end) : 0u;
            }
#pragma unroll
            for (int q = 0; q < WB; q++) {
                if (i0 + q * TPB < cnt && KGB_OK(dst[q] < bend, &a.ctl->err, E_LIST)) {
                    __stcs(iout + dst[q], (unsigned long long)kk[q] << 32 | id[q]);
                }
            }
        }
    } else {  // the last pass: the segmentation reads ids only
        u32 *vout = a.lval[par ^ 1];
        for (u32 i = tid; i < cnt; i += TPB) {
            const unsigned long long it = S.item[i];
            const u32 dst = S.gbase[((u32)(it >> 32) >> dsh) & 0xFFu] + i;
            if (KGB_OK(dst < bend, &a.ctl->err, E_LIST)) __stcs(vout + dst, (u32)it);
        }
    }
}

// One LSD pass over digit `slot` (skipped when that key byte is constant within every block): each CTA takes the
// next sort tile in order.
__global__ void __launch_bounds__(TPB, 3) k_lsd_pass(FwdArgs a, int slot) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LsdSmem &S = *reinterpret_cast<LsdSmem *>(smem_raw);
    const Ctl *c = a.ctl;
    const u32 act = active_slots(c);
    if (!((act >> slot) & 1)) return;
    const u32 ntiles = c->lsd_tiles;
    const u64 epoch = (u64)((c->seq << 5) | (u32)slot) << 32;
    const u32 tid = threadIdx.x;
    if (tid == 0) S.tile = atomicAdd(&a.ltile[slot], 1u);
    for (int i = tid; i < (TPB / 32) * 256; i += TPB) (&S.wcnt[0][0])[i] = 0;
    __syncthreads();
    const u32 tile = S.tile;
    if (tile >= ntiles) return;
    const LsdTile tl = lsd_tile(a, tile);
    if (tl.cnt == (u32)LSD_TILE) lsd_pass_tile<true>(a, S, slot, act, epoch, tile, tl);
    else lsd_pass_tile<false>(a, S, slot, act, epoch, tile, tl);
}

// ---- segmentation of the sorted keys
// Positions are handled in tiles of SEG_TILE; warp w of a tile owns the SEG_IPT * 32 consecutive positions starting at
// tile base + w * 32 * SEG_IPT and visits them lane-striped (position = chunk base + j * 32 + lane), so every load is
// coalesced. Group starts are kept as a bitmask (bit p of the mask: a group starts at position p), written by the
// count kernel (which compares neighbouring sorted keys); the emit kernels read only the bits.
__device__ __forceinline__ u32 lsd_final_par(const Ctl *c) { return __popc(active_slots(c)) & 1; }

struct SegBufs {
    const u32 *val;
    u32 *bits;          // start bitmask
    u32 *gbase, *gidx;  // per group start: list slot base, list index | GRP_LARGE (free value buffers)
    u32 *rk;            // per position: the round-0 rank, for the rank passes (the free half of the ids' item buffer)
    u32 m;
};
__device__ __forceinline__ SegBufs seg_bufs(const FwdArgs &a) {
    const Ctl *c = a.ctl;
    const u32 par = lsd_final_par(c);
    SegBufs v;
    v.val = a.lval[par];
    v.bits = a.segbits;
    v.gbase = a.lval[par ^ 1];
    v.gidx = a.lhi[par ^ 1];  // lval[q] and lhi[q] are the two halves of item buffer q
    v.rk = a.lhi[par];
    v.m = c->m;
    return v;
}
constexpr u32 GRP_LARGE = 0x80000000u, GRP_TINY = 0x40000000u, GRP_MED = 0x20000000u;
constexpr u32 SEG_WORDS = SEG_IPT;  // mask words per warp chunk

// The blocks a warp's chunk of SEG_IPT * 32 positions from cb spans: [lo, hi] (the same for every lane).
__device__ __forceinline__ uint2 seg_chunk_blocks(const FwdArgs &a, u32 cb, u32 m) {
    const u32 lo = blk_of_pos(a, cb, 0, a.B - 1);
    const u32 hi = blk_of_pos(a, min(cb + SEG_IPT * 32, m) - 1, lo, a.B - 1);
    return make_uint2(lo, hi);
}

// Per tile: start bits and the tile's last group start (position 0 always starts a group, and so does every block's
// first position).
__global__ void __launch_bounds__(TPB) k_seg_count(FwdArgs a) {
    __shared__ u32 ws[TPB / 32];
    const SegBufs v = seg_bufs(a);
    const u32 ntiles = (v.m + SEG_TILE - 1) / SEG_TILE;
    const u32 lane = lane_id(), warp = warp_id();
    // the prefix's second 8-byte word: its first W - 8 bytes (none for W = 8)
    const u64 m2 = a.lsd_bytes >= 16 ? ~0ull : a.lsd_bytes == 12 ? 0xFFFFFFFF00000000ull : 0ull;
    const bool two = m2 != 0;
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const u32 cb = t * SEG_TILE + warp * 32 * SEG_IPT;
        const uint2 br = cb < v.m ? seg_chunk_blocks(a, cb, v.m) : make_uint2(0u, 0u);
        u32 last = 0;
#pragma unroll 4
        for (int j = 0; j < SEG_IPT; j++) {
            const u32 p = cb + j * 32 + lane;
            const bool ok = p < v.m;
            const u32 b = ok ? (br.x == br.y ? br.x : blk_of_pos(a, p, br.x, br.y)) : 0u;
            const BlockInfo bi = a.blk[b];
            const u64 end = (u64)bi.off + bi.n;
            // the prefix's two 8-byte words (the second cut to its first W - 8 bytes), from the text
            const u32 id = ok ? v.val[p] : 0u;
            u64 k = 0, k2 = 0;
            if (ok) lsd_key16(a.T, id, end, two, k, k2);
            k2 &= m2;
            u64 kp = __shfl_up_sync(0xffffffffu, k, 1), k2p = __shfl_up_sync(0xffffffffu, k2, 1);
            if (lane == 0 && ok && p > bi.soff) {  // the neighbour is in the same block
                lsd_key16(a.T, v.val[p - 1], end, two, kp, k2p);
                k2p &= m2;
            }
            const bool st = ok && (p == bi.soff || k != kp || k2 != k2p);
            const u32 sb = __ballot_sync(0xffffffffu, st);
            if (lane == 0 && cb + j * 32 < v.m) v.bits[(cb >> 5) + j] = sb;
            if (st) last = p;
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
        if (lane == 0) ws[warp] = last;
        __syncthreads();
        if (threadIdx.x == 0) {
            u32 tl = 0;
            for (int w = 0; w < TPB / 32; w++) tl = max(tl, ws[w]);
            a.segagg[(u64)t * 2] = tl;
        }
        __syncthreads();
    }
}

// Exclusive max-scan of the tiles' last starts (one CTA): the start of the group open at each tile's first position.
__global__ void __launch_bounds__(1024) k_seg_scan(FwdArgs a) {
    __shared__ u32 ws[33];
    __shared__ u32 prev[1024];
    const u32 m = a.ctl->m;
    const u32 ntiles = (m + SEG_TILE - 1) / SEG_TILE;
    u32 carry = 0;
    for (u32 t0 = 0; t0 < ntiles; t0 += 1024) {
        const u32 t = t0 + threadIdx.x;
        const u32 l = t < ntiles ? a.segagg[(u64)t * 2] : 0u;
        const u32 il = block_incl_max<1024>(l, ws);
        prev[threadIdx.x] = il;
        __syncthreads();
        if (t < ntiles) a.segagg[(u64)t * 2 + 1] = max(carry, threadIdx.x ? prev[threadIdx.x - 1] : 0u);
        carry = max(carry, prev[1023]);
        __syncthreads();
    }
}

// The warp's view of its chunk: the mask words (lane j holds word j), and the start of the group open at the chunk's
// first position.
struct SegChunk {
    u32 cb, word, nextw, carry0;
    u32 blo, bhi;  // the blocks the chunk spans
};
__device__ __forceinline__ SegChunk seg_chunk(const FwdArgs &a, const SegBufs &v, u32 t, u32 *wl) {
    const u32 lane = lane_id(), warp = warp_id();
    SegChunk c;
    c.cb = t * SEG_TILE + warp * 32 * SEG_IPT;
    const u32 w0 = c.cb >> 5;
    const u32 nw = (v.m + 31) >> 5;
    c.word = lane < SEG_WORDS && w0 + lane < nw ? v.bits[w0 + lane] : 0u;
    // bit 0 of the word after the chunk: the start flag of the first position past it
    c.nextw = w0 + SEG_WORDS < nw ? v.bits[w0 + SEG_WORDS] : 1u;
    u32 last = 0;
    if (lane < SEG_WORDS && c.word) last = c.cb + lane * 32 + 31 - __clz(c.word);
#pragma unroll
    for (int o = 16; o; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
    if (lane == 0) wl[warp] = last;
    __syncthreads();
    u32 cr = a.segagg[(u64)t * 2 + 1];
    for (u32 w = 0; w < warp; w++) cr = max(cr, wl[w]);
    c.carry0 = cr;
    const uint2 br = c.cb < v.m ? seg_chunk_blocks(a, c.cb, v.m) : make_uint2(0u, 0u);
    c.blo = br.x; c.bhi = br.y;
    return c;
}
// Position j * 32 + lane of the chunk: start / end flags and the group's first position (carry: running start).
__device__ __forceinline__ void seg_step(const SegBufs &v, const SegChunk &c, int j, u32 &carry, u32 &p, bool &valid,
                                         bool &st, bool &en, u32 &gfirst) {
    const u32 lane = lane_id();
    const u32 w = __shfl_sync(0xffffffffu, c.word, j);
    const u32 wn = j + 1 < SEG_IPT ? __shfl_sync(0xffffffffu, c.word, (j + 1) & 31) : c.nextw;
    p = c.cb + j * 32 + lane;
    valid = p < v.m;
    st = (w >> lane) & 1;
    en = p + 1 >= v.m || (lane < 31 ? (w >> (lane + 1)) & 1 : wn & 1);
    const u32 x = warp_incl_max(valid && st ? p : 0u);
    gfirst = max(carry, x);
    carry = __shfl_sync(0xffffffffu, gfirst, 31);
}

// Block-wide exclusive sum of a 64-bit value (TPB threads); contains __syncthreads().
__device__ __forceinline__ u64 block_excl_sum64(u64 v, u64 *ws, u64 *total) {
    u64 inc = v;
    const u32 lane = lane_id(), warp = warp_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u64 t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (u32)o) inc += t;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    u64 before = 0, tot = 0;
    for (u32 w = 0; w < TPB / 32; w++) {
        const u64 x = ws[w];
        if (w < warp) before += x;
        tot += x;
    }
    __syncthreads();
    *total = tot;
    return before + inc - v;
}

// Emit, part 1 (group ends): groups of one resolve (rank unless k_seg_rank writes the ranks, L column); every other
// group takes its slots in the next tiny-group list
// (<= GTINY), medium-group list (<= GMED), small-group list (<= SMAX) or large-group list, writes its descriptor (and
// tile-map entries), and records its slot base and index at its first position for part 2. Slots are allocated once
// per tile (a count pass, a block scan, one atomic per list).
__global__ void __launch_bounds__(TPB) k_seg_emit1(FwdArgs a) {
    __shared__ u32 wl[TPB / 32];
    __shared__ u64 ws[4][TPB / 32];
    __shared__ u64 base[5];
    Ctl *c = a.ctl;
    const SegBufs v = seg_bufs(a);
    const u32 rpar = c->rpar, round = c->round;
    const ListView sl = a.lists[L_S0 + (rpar ^ 1)], ll = a.lists[L_L0 + (rpar ^ 1)], tl_ = a.lists[L_P0 + (rpar ^ 1)];
    const ListView ml_ = a.lists[L_M0 + (rpar ^ 1)];
    const u32 ntiles = (v.m + SEG_TILE - 1) / SEG_TILE;
    const u32 TS = a.smax;
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const SegChunk ch = seg_chunk(a, v, t, wl);
        // count: singles | small groups << 16 | small elements << 32 ; large groups | large elements << 32 ;
        // tiny groups | tiny elements << 32 ; medium groups | medium elements << 32
        u64 cs = 0, cl = 0, ct = 0, cm = 0;
        {
            u32 carry = ch.carry0;
            for (int j = 0; j < SEG_IPT; j++) {
                u32 p, gf; bool ok, st, en;
                seg_step(v, ch, j, carry, p, ok, st, en, gf);
                if (!ok || !en) continue;
                const u32 len = p - gf + 1;
                if (len == 1) cs += 1;
                else if (len <= GTINY) ct += 1ull | ((u64)len << 32);
                else if (len <= GMED) cm += 1ull | ((u64)len << 32);
                else if (len <= TS) cs += (1ull << 16) | ((u64)len << 32);
                else cl += 1ull | ((u64)len << 32);
            }
        }
        u64 ts, tl, tt;
        u64 xs = block_excl_sum64(cs, ws[0], &ts);
        u64 xl = block_excl_sum64(cl, ws[1], &tl);
        u64 xt = block_excl_sum64(ct, ws[2], &tt);
        u64 tm;
        u64 xm = block_excl_sum64(cm, ws[3], &tm);
        if (threadIdx.x == 0) {
            base[4] = (u32)tm ? atomicAdd(&c->cnt[L_M0 + (rpar ^ 1)], (tm << 32) | (tm >> 32)) : 0ull;
            if ((u32)tt) {
                const uint2 o = alloc_tiny(c, rpar, (u32)tt, (u32)(tt >> 32));
                base[3] = ((u64)o.y << 32) | o.x;
            } else {
                base[3] = 0;
            }
            base[1] = (ts >> 16) & 0xFFFF ? atomicAdd(&c->cnt[L_S0 + (rpar ^ 1)], (((ts >> 16) & 0xFFFF) << 32) | (ts >> 32)) : 0ull;
            base[2] = (u32)tl ? atomicAdd(&c->cnt[L_L0 + (rpar ^ 1)], (tl << 32) | (tl >> 32)) : 0ull;
        }
        __syncthreads();
        u32 sidx = (u32)(base[1] >> 32) + (u32)((xs >> 16) & 0xFFFF), se = (u32)base[1] + (u32)(xs >> 32);
        u32 lidx = (u32)(base[2] >> 32) + (u32)xl, le = (u32)base[2] + (u32)(xl >> 32);
        u32 tidx = (u32)(base[3] >> 32) + (u32)xt, te = (u32)base[3] + (u32)(xt >> 32);
        u32 midx = (u32)(base[4] >> 32) + (u32)xm, me = (u32)base[4] + (u32)(xm >> 32);
        u32 carry = ch.carry0;
        constexpr int QB = 8;  // positions per phase: group ends first, then their loads, then the writes
        for (int j0 = 0; j0 < SEG_IPT; j0 += QB) {
            u32 pv[QB], gfv[QB], live = 0;
#pragma unroll
            for (int q = 0; q < QB; q++) {
                u32 p, gf; bool ok, st, en;
                seg_step(v, ch, j0 + q, carry, p, ok, st, en, gf);
                pv[q] = p; gfv[q] = gf;
                if (ok && en) live |= 1u << q;
            }
            u32 bv[QB], idv[QB];
#pragma unroll
            for (int q = 0; q < QB; q++) {
                if (!((live >> q) & 1)) continue;
                bv[q] = ch.blo == ch.bhi ? ch.blo : blk_of_pos(a, pv[q], ch.blo, ch.bhi);
                idv[q] = pv[q] == gfv[q] ? __ldg(v.val + pv[q]) : 0u;  // ids of finished suffixes (groups of one)
            }
#pragma unroll
            for (int q = 0; q < QB; q++) {
                if (!((live >> q) & 1)) continue;
                const u32 p = pv[q], gf = gfv[q];
                const u32 len = p - gf + 1;
                const u32 b = bv[q];
                const u32 head = gf - a.blk[b].soff;
                if (len == 1) {
                    resolve_round0(a, a.rank_passes ? nullptr : a.isa[rpar ^ 1], idv[q], head, b);
                    continue;
                }
                Seg g;
                g.len = len; g.head = head; g.bd = b;
                if (len <= GTINY) {
                    g.start = te;
                    KGB_GUARD(tidx < a.cap_segt && (u64)te + len <= a.cap_n, &c->err, E_SEG) {
                        tl_.seg[tidx] = g;
                        v.gbase[gf] = te;
                        v.gidx[gf] = tidx | GRP_TINY;
                    }
                    tidx++; te += len;
                } else if (len <= GMED) {
                    g.start = me;
                    KGB_GUARD(midx < a.cap_segm && (u64)me + len <= a.cap_n, &c->err, E_SEG) {
                        ml_.seg[midx] = g;
                        v.gbase[gf] = me;
                        v.gidx[gf] = midx | GRP_MED;
                    }
                    midx++; me += len;
                } else if (len <= TS) {
                    g.start = se;
                    KGB_GUARD(sidx < a.cap_segs && (u64)se + len <= a.cap_n, &c->err, E_SEG) {
                        sl.seg[sidx] = g;
                        write_tmap_small(a, sl.tmap, TS, se, len, sidx);
                        if (len > WARP_GROUP) sl.tbig[se / TS] = round + 1;
                        v.gbase[gf] = se;
                        v.gidx[gf] = sidx;
                    }
                    sidx++; se += len;
                } else {
                    g.start = le;
                    KGB_GUARD(lidx < a.cap_segl && (u64)le + len <= a.cap_n, &c->err, E_SEG) {
                        ll.seg[lidx] = g;
                        v.gbase[gf] = le;
                        v.gidx[gf] = lidx | GRP_LARGE;
                    }
                    lidx++; le += len;
                }
            }
        }
        __syncthreads();
    }
}

// Emit, part 2 (every suffix of a group of two or more): its rank (the group's first position) unless k_seg_rank
// writes the ranks, its slot in its group's list, and for large groups the bucket-pass tile map (the suffix at a
// multiple of TSM names its group).
__global__ void __launch_bounds__(TPB) k_seg_emit2(FwdArgs a) {
    __shared__ u32 wl[TPB / 32];
    Ctl *c = a.ctl;
    const SegBufs v = seg_bufs(a);
    const u32 rpar = c->rpar;
    const ListView sl = a.lists[L_S0 + (rpar ^ 1)], ll = a.lists[L_L0 + (rpar ^ 1)], tl_ = a.lists[L_P0 + (rpar ^ 1)];
    const ListView ml_ = a.lists[L_M0 + (rpar ^ 1)];
    const u32 ntiles = (v.m + SEG_TILE - 1) / SEG_TILE;
    constexpr int QB = 8;  // positions per phase: group starts first, then every load, then every store
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const SegChunk ch = seg_chunk(a, v, t, wl);
        u32 carry = ch.carry0;
        for (int j0 = 0; j0 < SEG_IPT; j0 += QB) {
            u32 pv[QB], gfv[QB], live = 0;
#pragma unroll
            for (int q = 0; q < QB; q++) {
                u32 p, gf; bool ok, st, en;
                seg_step(v, ch, j0 + q, carry, p, ok, st, en, gf);
                pv[q] = p; gfv[q] = gf;
                if (ok && !(st && en)) live |= 1u << q;  // groups of one were resolved by part 1
                if (ok && a.rank_passes) {  // every position's rank, streamed by the rank passes
                    const u32 b = ch.blo == ch.bhi ? ch.blo : blk_of_pos(a, p, ch.blo, ch.bhi);
                    __stcg(v.rk + p, gf - a.blk[b].soff);
                }
            }
            u32 idv[QB], giv[QB], gbv[QB];
#pragma unroll
            for (int q = 0; q < QB; q++) {
                if (!((live >> q) & 1)) continue;
                idv[q] = __ldg(v.val + pv[q]);
                giv[q] = __ldg(v.gidx + gfv[q]);
                gbv[q] = __ldg(v.gbase + gfv[q]);
            }
#pragma unroll
            for (int q = 0; q < QB; q++) {
                if (!((live >> q) & 1)) continue;
                const u32 id = idv[q], gi = giv[q], p = pv[q], gf = gfv[q];
                const u32 slot = gbv[q] + (p - gf);
                KGB_GUARD(id < a.cap_n && slot < a.cap_n, &c->err, E_LIST) {
                    if (!a.rank_passes) {
                        const u32 b = ch.blo == ch.bhi ? ch.blo : blk_of_pos(a, p, ch.blo, ch.bhi);
                        a.isa[rpar ^ 1][id] = gf - a.blk[b].soff;
                    }
                    if (gi & GRP_LARGE) {
                        ll.eid[slot] = id;
                        if (slot % TSM == 0) {
                            KGB_GUARD(slot / TSM < a.cap_tml, &c->err, E_TMAP) ll.tmap[slot / TSM] = gi & ~GRP_LARGE;
                        }
                    } else if (gi & GRP_TINY) {
                        tl_.eid[slot] = id;
                    } else if (gi & GRP_MED) {
                        ml_.eid[slot] = id;
                    } else {
                        sl.eid[slot] = id;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// Ranks after round 0 (every suffix: its group's first position in its block), for the suffixes whose id lies in
// [lo, hi). The host runs one pass per id range of RANK_SPAN ids, so that the rank writes of a pass (a scatter over
// 4 * RANK_SPAN bytes) stay in L2 and reach DRAM as whole sectors, instead of one read-modify-write per suffix;
// every pass streams the sorted ids again and reads the ranks that the second emit kernel wrote per position.
constexpr u32 RANK_SPAN = 16u << 20;
// More passes than this cost more streaming than the random writes they replace (about 4 ps per suffix and pass
// against about 29 ps per random rank write, measured on a 64 MiB block): the emit kernels write the ranks instead,
// as they do when no block exceeds RANK_SPAN suffixes (their writes then stay within one block's ids at a time).
constexpr u32 RANK_PASSES_MAX = 4;
__global__ void __launch_bounds__(TPB) k_seg_rank(FwdArgs a, u32 lo, u32 hi) {
    Ctl *c = a.ctl;
    const SegBufs v = seg_bufs(a);
    u32 *isa_nxt = a.isa[c->rpar ^ 1];
    const u32 span = hi - lo;
    // four positions per thread and step: one 16-byte load of their ids, the ranks loaded only where an id is in range
    const u32 m4 = v.m / 4;
    const uint4 *ids4 = reinterpret_cast<const uint4 *>(v.val);
    for (u32 i = blockIdx.x * TPB + threadIdx.x; i < m4; i += gridDim.x * TPB) {
        const uint4 q = __ldcs(ids4 + i);
        const u32 id[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (id[k] - lo >= span) continue;
            KGB_GUARD(id[k] < a.cap_n, &c->err, E_RANK) isa_nxt[id[k]] = __ldg(v.rk + 4 * i + k);
        }
    }
    for (u32 p = m4 * 4 + blockIdx.x * TPB + threadIdx.x; p < v.m; p += gridDim.x * TPB) {
        const u32 id = v.val[p];
        if (id - lo >= span) continue;
        KGB_GUARD(id < a.cap_n, &c->err, E_RANK) isa_nxt[id] = v.rk[p];
    }
}
