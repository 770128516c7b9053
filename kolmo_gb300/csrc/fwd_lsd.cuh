// Round 0 of the forward sort as one LSD radix sort: every suffix of the batch is sorted by (block, zero-padded
// 8-byte prefix) with one pass per varying key byte (single-pass scatter with decoupled look-back), then a
// segmentation turns the sorted order into ranks, finished suffixes and the rank rounds' groups (the small-group list
// for the tile kernels, the large-group list for the bucket passes). The passes move (key, id) items, the 8-byte key
// as two 32-bit halves (and the block index when the batch has several blocks): a pass takes its digit from the key
// it carries, and the segmentation compares neighbouring keys without touching the text. Included by fwd.cu inside
// namespace kgb, after the kernels it shares (FwdArgs, resolve, tile-map writers).
#pragma once
// (included inside namespace kgb)

constexpr int LSD_IPT = 16, LSD_TILE = TPB * LSD_IPT;  // elements per sort tile
constexpr int NSLOT = 12;                              // digit slots: key bytes 0..7, then block-index bytes 0..3
constexpr int SEG_IPT = 16, SEG_TILE = TPB * SEG_IPT;  // positions per segmentation tile (SEG_IPT <= 32)
// look-back words: epoch (32 bits: call sequence, digit slot) | flag (2 bits) | value (30 bits); a word of another
// epoch (an earlier slot or call) counts as not yet published
constexpr u64 ST_AGG = 1ull << 30, ST_PRE = 2ull << 30, ST_VAL = (1ull << 30) - 1;
constexpr u64 ST_EPOCH = 0xFFFFFFFF00000000ull;
constexpr int LB_WIN = 8;  // look-back window (predecessor words read per step)

__device__ __forceinline__ u32 active_slots(const Ctl *c) {  // bit s: key byte s varies
    const u64 vl = c->vary_lo ^ c->and_lo;
    const u32 vh = c->vary_hi ^ c->and_hi;
    u32 m = 0;
#pragma unroll
    for (int s = 0; s < 8; s++) m |= ((vl >> (8 * s)) & 0xFF) ? 1u << s : 0u;
#pragma unroll
    for (int s = 0; s < 4; s++) m |= ((vh >> (8 * s)) & 0xFF) ? 1u << (8 + s) : 0u;
    return m;
}
__device__ __forceinline__ bool lsd_has_hi(const FwdArgs &a) { return a.B > 1; }

// The zero-padded 8-byte prefix of suffix id (block ending at end) as a big-endian word.
__device__ __forceinline__ u64 lsd_key(const u8 *__restrict__ T, u32 id, u64 end) {
    u64 k = load_be64(T, id);
    const u64 rem = end - id;
    if (rem < 8) k &= ~0ull << (8 * (8 - rem));
    return k;
}

// Start (256 threads): clear the text byte histogram, the tile counters and the resolved count.
__global__ void k_lsd_begin(FwdArgs a) {
    Ctl *c = a.ctl;
    for (int i = threadIdx.x; i < NSLOT * 256; i += blockDim.x) a.lhist[i] = 0;
    if (threadIdx.x < NSLOT) a.ltile[threadIdx.x] = 0;
    if (threadIdx.x == 0) c->cnt[L_R0 + c->rpar] = 0;
}

// Suffix ids and their 8-byte keys in the dense order of the batch (block index beside them when the batch has
// several blocks), and the byte histogram of the whole text (row 0 of the histogram table), from which every pass's
// digit counts follow.
__global__ void __launch_bounds__(TPB) k_lsd_key0(FwdArgs a) {
    __shared__ u32 hs[256];
    const bool hi = lsd_has_hi(a);
    const u64 stride = (u64)gridDim.x * blockDim.x;
    hs[threadIdx.x] = 0;
    __syncthreads();
    for (u32 b = 0; b < a.B; b++) {
        const BlockInfo bi = a.blk[b];
        // row 0 of the L column (the sentinel rotation) holds the block's last byte
        if (blockIdx.x == 0 && threadIdx.x == 0) a.L[(u64)bi.off + b] = a.T[(u64)bi.off + bi.n - 1];
        for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < bi.n; j += stride) {
            const u32 id = bi.off + (u32)j;
            const u64 x = (u64)bi.soff + j;
            __stcs(a.lval[0] + x, id);
            if (hi) __stcs(a.lhi[0] + x, b);
            const u64 k = lsd_key(a.T, id, (u64)bi.off + bi.n);
            __stcs(a.lkh[0] + x, (u32)(k >> 32));
            __stcs(a.lkl[0] + x, (u32)k);
            atomicAdd(&hs[(u32)(k >> 56)], 1u);
        }
    }
    __syncthreads();
    if (hs[threadIdx.x]) atomicAdd(&a.lhist[threadIdx.x], hs[threadIdx.x]);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->m = a.B ? a.blk[a.B - 1].soff + a.blk[a.B - 1].n : 0;
}

// Digit counts of every pass (one CTA of 256 threads, thread = digit value). Suffix i of a block of n bytes has key
// byte d = T[i + d] when i + d < n, else 0, so the counts of key byte d are the block's byte counts minus those of
// its first min(d, n) bytes, plus min(d, n) zeros; block-index digits count each block's n. A slot whose counts sit
// in one digit is constant: the vary words mark the others, which the passes run.
__global__ void k_lsd_hist0(FwdArgs a) {
    __shared__ u32 pre[8][256];  // pre[d][x]: bytes x among the first d bytes of every block (d = 1..7)
    __shared__ u32 zeros[8];
    __shared__ u32 hib[4][256];
    __shared__ u32 flag[NSLOT];
    const u32 x = threadIdx.x;
    for (int d = 0; d < 8; d++) pre[d][x] = 0;
    for (int q = 0; q < 4; q++) hib[q][x] = 0;
    if (x < 8) zeros[x] = 0;
    if (x < NSLOT) flag[x] = 0;
    __syncthreads();
    for (u32 b = x; b < a.B; b += blockDim.x) {
        const BlockInfo bi = a.blk[b];
        for (u32 d = 1; d < 8; d++) {
            if (d <= bi.n) atomicAdd(&pre[d][a.T[(u64)bi.off + d - 1]], 1u);
            atomicAdd(&zeros[d], d < bi.n ? d : bi.n);  // min(d, n) zero digits per block
        }
        if (a.B > 1)
            for (int q = 0; q < 4; q++) atomicAdd(&hib[q][(b >> (8 * q)) & 0xFF], bi.n);
    }
    __syncthreads();
    // pre[d] holds the bytes at offset d - 1 only: accumulate to the first d bytes
    for (int d = 2; d < 8; d++) pre[d][x] += pre[d - 1][x];
    const u32 m = a.ctl->m;
    const u32 h0 = a.lhist[x];  // byte counts of the whole text
    for (int slot = 0; slot < 8; slot++) {
        const u32 d = 7 - slot;
        const u32 v = d ? h0 - pre[d][x] + (x == 0 ? zeros[d] : 0u) : h0;
        a.lhist[slot * 256 + x] = v;
        if (v != 0 && v != m) flag[slot] = 1;  // at least two digits occur
    }
    if (a.B > 1)
        for (int q = 0; q < 4; q++) {
            const u32 v = hib[q][x];
            a.lhist[(8 + q) * 256 + x] = v;
            if (v != 0 && v != m) flag[8 + q] = 1;
        }
    __syncthreads();
    if (x == 0) {
        Ctl *c = a.ctl;
        u64 vl = 0;
        u32 vh = 0;
        for (int q = 0; q < 8; q++) if (flag[q]) vl |= 0xFFull << (8 * q);
        for (int q = 0; q < 4; q++) if (flag[8 + q]) vh |= 0xFFu << (8 * q);
        c->vary_lo = vl; c->and_lo = 0; c->vary_hi = vh; c->and_hi = 0;
    }
}

template <bool HI>
struct LsdSmem {
    u32 val[LSD_TILE];
    u32 kh[LSD_TILE], kl[LSD_TILE];
    u32 hi[HI ? LSD_TILE : 1];
    u8 dg[LSD_TILE];
    u16 wcnt[TPB / 32][256];
    u32 gbase[256];
    u32 dbase[256];
    u32 ws[TPB / 32 + 1];
    u32 tile;
};

// One LSD pass over digit `slot` (skipped when that key byte is the same in every key): rank the tile's suffixes by
// digit, publish the tile's digit counts, look back over earlier tiles for the global offsets (bounded spin), stage
// the tile in shared memory in digit order and write it out in runs.
template <bool HI>
__global__ void __launch_bounds__(TPB, 3) k_lsd_pass(FwdArgs a, int slot) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LsdSmem<HI> &S = *reinterpret_cast<LsdSmem<HI> *>(smem_raw);
    const Ctl *c = a.ctl;
    const u32 act = active_slots(c);
    if (!((act >> slot) & 1)) return;
    const u32 par = __popc(act & ((1u << slot) - 1)) & 1;
    const u32 m = c->m;
    const u32 ntiles = (m + LSD_TILE - 1) / LSD_TILE;
    const u64 epoch = (u64)((c->seq << 4) | (u32)slot) << 32;
    const u32 tid = threadIdx.x, lane = lane_id(), warp = warp_id();
    if (tid == 0) S.tile = atomicAdd(&a.ltile[slot], 1u);
    // digit bases of the pass: exclusive scan of the slot's counts
    {
        const u32 hcount = a.lhist[slot * 256 + tid];
        S.dbase[tid] = block_excl_sum<TPB>(hcount, S.ws, nullptr);
    }
    for (int i = tid; i < (TPB / 32) * 256; i += TPB) (&S.wcnt[0][0])[i] = 0;
    __syncthreads();
    const u32 tile = S.tile;
    if (tile >= ntiles) return;
    const u32 base = tile * LSD_TILE;
    const u32 cnt = min((u32)LSD_TILE, m - base);
    const u32 *vin = a.lval[par], *hin = a.lhi[par], *khin = a.lkh[par], *klin = a.lkl[par];
    // rk[j]: rank in the warp's digit bucket (bits 0..15) | digit, 0x100 past the end (bits 16..24)
    u32 v[LSD_IPT], hh[LSD_IPT], rk[LSD_IPT], kh[LSD_IPT], kl[LSD_IPT];
#pragma unroll
    for (int j = 0; j < LSD_IPT; j++) {
        const u32 x = warp * (32 * LSD_IPT) + j * 32 + lane;
        const bool ok = x < cnt;
        v[j] = ok ? __ldcs(vin + base + x) : 0u;
        kh[j] = ok ? __ldcs(khin + base + x) : 0u;
        kl[j] = ok ? __ldcs(klin + base + x) : 0u;
        hh[j] = ok && HI ? __ldcs(hin + base + x) : 0u;
    }
#pragma unroll
    for (int j = 0; j < LSD_IPT; j++) {
        const u32 x = warp * (32 * LSD_IPT) + j * 32 + lane;
        u32 d;
        if (slot >= 8) d = (hh[j] >> (8 * (slot - 8))) & 0xFFu;
        else d = ((slot < 4 ? kl[j] : kh[j]) >> (8 * (slot & 3))) & 0xFFu;
        rk[j] = (x < cnt ? d : 0x100u) << 16;
    }
#pragma unroll
    for (int j = 0; j < LSD_IPT; j++) {
        const u32 d = rk[j] >> 16;
        const u32 peers = __match_any_sync(0xffffffffu, d);
        const u32 before = d < 256 ? S.wcnt[warp][d] : 0u;
        rk[j] |= before + __popc(peers & lanemask_lt());
        __syncwarp();
        if (d < 256 && (__ffs(peers) - 1) == (int)lane) S.wcnt[warp][d] = (u16)(before + __popc(peers));
        __syncwarp();
    }
    __syncthreads();
    // thread tid owns digit tid: tile count, publish, local start, look back
    u32 tot = 0;
#pragma unroll
    for (int w = 0; w < TPB / 32; w++) tot += S.wcnt[w][tid];
    u64 *st = a.lstat + (u64)tile * 256 + tid;
    if (tile == 0) atomicExch((unsigned long long *)st, epoch | ST_PRE | tot);
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
        const u32 d = rk[j] >> 16;
        if (d < 256) {
            const u32 p = S.wcnt[warp][d] + (rk[j] & 0xFFFFu);
            S.val[p] = v[j];
            S.kh[p] = kh[j];
            S.kl[p] = kl[j];
            if (HI) S.hi[p] = hh[j];
            S.dg[p] = (u8)d;
        }
    }
    u32 excl = 0;
    if (tile > 0) {
        // windowed look-back: read LB_WIN predecessors' words at once, add aggregates in order up to the first
        // inclusive prefix; a word not yet published ends the window and the walk resumes there
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
    S.gbase[tid] = S.dbase[tid] + excl - dstart;
    __syncthreads();
    u32 *vout = a.lval[par ^ 1], *hout = a.lhi[par ^ 1], *khout = a.lkh[par ^ 1], *klout = a.lkl[par ^ 1];
    for (u32 i = tid; i < cnt; i += TPB) {
        const u32 dst = S.gbase[S.dg[i]] + i;
        if (KGB_OK(dst < m, &a.ctl->err, E_LIST)) {
            __stcs(vout + dst, S.val[i]);
            __stcs(khout + dst, S.kh[i]);
            __stcs(klout + dst, S.kl[i]);
            if (HI) __stcs(hout + dst, S.hi[i]);
        }
    }
}

// ---- segmentation of the sorted keys
// Positions are handled in tiles of SEG_TILE; warp w of a tile owns the SEG_IPT * 32 consecutive positions starting at
// tile base + w * 32 * SEG_IPT and visits them lane-striped (position = chunk base + j * 32 + lane), so every load is
// coalesced. Group starts are kept as a bitmask (bit p of the mask: a group starts at position p), written by the
// count kernel (which compares neighbouring sorted keys); the emit kernels read only the bits.
__device__ __forceinline__ u32 lsd_final_par(const Ctl *c) { return __popc(active_slots(c)) & 1; }

struct SegBufs {
    const u32 *val, *hi;
    u32 *bits;          // start bitmask
    u32 *gbase, *gidx;  // per group start: list slot base, list index | GRP_LARGE (free value / block buffers)
    bool has_hi;
    u32 m;
};
__device__ __forceinline__ SegBufs seg_bufs(const FwdArgs &a) {
    const Ctl *c = a.ctl;
    const u32 par = lsd_final_par(c);
    SegBufs v;
    v.val = a.lval[par]; v.hi = a.lhi[par];
    v.bits = a.segbits;
    v.gbase = a.lval[par ^ 1];
    v.gidx = a.lhi[par ^ 1];
    v.has_hi = lsd_has_hi(a);
    v.m = c->m;
    return v;
}
constexpr u32 GRP_LARGE = 0x80000000u, GRP_TINY = 0x40000000u, GRP_MED = 0x20000000u;
constexpr u32 SEG_WORDS = SEG_IPT;  // mask words per warp chunk

// Per tile: start bits and the tile's last group start (position 0 always starts a group).
__global__ void __launch_bounds__(TPB) k_seg_count(FwdArgs a) {
    __shared__ u32 ws[TPB / 32];
    const SegBufs v = seg_bufs(a);
    const u32 ntiles = (v.m + SEG_TILE - 1) / SEG_TILE;
    const u32 lane = lane_id(), warp = warp_id();
    for (u32 t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const u32 cb = t * SEG_TILE + warp * 32 * SEG_IPT;
        u32 last = 0;
#pragma unroll 4
        for (int j = 0; j < SEG_IPT; j++) {
            const u32 p = cb + j * 32 + lane;
            const bool ok = p < v.m;
            const u32 fp = lsd_final_par(a.ctl);
            const u32 *KH = a.lkh[fp], *KL = a.lkl[fp];
            u32 h = ok && v.has_hi ? v.hi[p] : 0u;
            u64 k = ok ? ((u64)KH[p] << 32) | KL[p] : 0ull;
            u64 kp = __shfl_up_sync(0xffffffffu, k, 1);
            u32 hp = __shfl_up_sync(0xffffffffu, h, 1);
            if (lane == 0 && ok && p > 0) {
                hp = v.has_hi ? v.hi[p - 1] : 0u;
                kp = ((u64)KH[p - 1] << 32) | KL[p - 1];
            }
            const bool st = ok && (p == 0 || k != kp || h != hp);
            const u32 b = __ballot_sync(0xffffffffu, st);
            if (lane == 0 && cb + j * 32 < v.m) v.bits[(cb >> 5) + j] = b;
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

// Emit, part 1 (group ends): groups of one resolve; every other group takes its slots in the next tiny-group list
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
    const ListView res = a.lists[L_R0 + rpar];
    u32 *isa_nxt = a.isa[rpar ^ 1];
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
            base[0] = (ts & 0xFFFF) ? atomicAdd(&c->cnt[L_R0 + rpar], ts & 0xFFFF) : 0ull;
            base[1] = (ts >> 16) & 0xFFFF ? atomicAdd(&c->cnt[L_S0 + (rpar ^ 1)], (((ts >> 16) & 0xFFFF) << 32) | (ts >> 32)) : 0ull;
            base[2] = (u32)tl ? atomicAdd(&c->cnt[L_L0 + (rpar ^ 1)], (tl << 32) | (tl >> 32)) : 0ull;
        }
        __syncthreads();
        u32 r1 = (u32)base[0] + (u32)(xs & 0xFFFF);
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
                bv[q] = v.has_hi ? __ldg(v.hi + pv[q]) : 0u;
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
                    resolve(a, isa_nxt, idv[q], head, b, res, r1++);
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

// Emit, part 2 (every suffix of a group of two or more): its rank (the group's first position), its slot in its
// group's list, and for large groups the bucket-pass tile map (the suffix at a multiple of TSM names its group).
__global__ void __launch_bounds__(TPB) k_seg_emit2(FwdArgs a) {
    __shared__ u32 wl[TPB / 32];
    Ctl *c = a.ctl;
    const SegBufs v = seg_bufs(a);
    const u32 rpar = c->rpar;
    const ListView sl = a.lists[L_S0 + (rpar ^ 1)], ll = a.lists[L_L0 + (rpar ^ 1)], tl_ = a.lists[L_P0 + (rpar ^ 1)];
    const ListView ml_ = a.lists[L_M0 + (rpar ^ 1)];
    u32 *isa_nxt = a.isa[rpar ^ 1];
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
            }
            u32 idv[QB], giv[QB], gbv[QB], bv[QB];
#pragma unroll
            for (int q = 0; q < QB; q++) {
                if (!((live >> q) & 1)) continue;
                idv[q] = __ldg(v.val + pv[q]);
                bv[q] = v.has_hi ? __ldg(v.hi + pv[q]) : 0u;
                giv[q] = __ldg(v.gidx + gfv[q]);
                gbv[q] = __ldg(v.gbase + gfv[q]);
            }
#pragma unroll
            for (int q = 0; q < QB; q++) {
                if (!((live >> q) & 1)) continue;
                const u32 id = idv[q], gi = giv[q], p = pv[q], gf = gfv[q];
                const u32 head = gf - a.blk[bv[q]].soff;
                const u32 slot = gbv[q] + (p - gf);
                KGB_GUARD(id < a.cap_n && slot < a.cap_n, &c->err, E_LIST) {
                    isa_nxt[id] = head;
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
