// Shared device helpers for the block-sorting kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace kgb {

typedef uint8_t u8;
typedef uint16_t u16;
typedef uint32_t u32;
typedef unsigned long long u64;

// Error plumbing: every CUDA call on the host goes through KGB_CHECK, which records the failure and makes the
// enclosing function return the C-ABI code (-2 for resources and device errors).
int record_cuda_error(cudaError_t e, const char *what, const char *file, int line);
void record_error(const char *msg);
#define KGB_CHECK(x)                                                                         \
    do {                                                                                     \
        cudaError_t e__ = (x);                                                               \
        if (e__ != cudaSuccess) return ::kgb::record_cuda_error(e__, #x, __FILE__, __LINE__); \
    } while (0)

// Bounds guards of the checked build (-DKGB_CHECKED): `KGB_GUARD(cond, err, bit) stmt;` runs stmt only when cond
// holds and otherwise sets `bit` in the device error word *err. In the normal build it is just `stmt;`.
#ifdef KGB_CHECKED
#define KGB_GUARD(cond, errp, bit) \
    if (!(cond)) {                 \
        atomicOr((errp), (bit));   \
    } else
#define KGB_OK(cond, errp, bit) ((cond) ? true : (atomicOr((errp), (bit)), false))
#else
#define KGB_GUARD(cond, errp, bit)
#define KGB_OK(cond, errp, bit) true
#endif

__device__ __forceinline__ u32 lanemask_lt() {
    u32 m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ u32 lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ u32 warp_id() { return threadIdx.x >> 5; }

__device__ __forceinline__ u32 warp_incl_sum(u32 v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        u32 t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= (u32)o) v += t;
    }
    return v;
}
__device__ __forceinline__ u32 warp_incl_max(u32 v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        u32 t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= (u32)o) v = max(v, t);
    }
    return v;
}
__device__ __forceinline__ u32 warp_sum(u32 v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide exclusive sum over NT threads (NT multiple of 32, <= 1024). `ws` needs NT/32 + 1 words of shared
// memory. Returns the thread's exclusive prefix; *total receives the block sum. Contains __syncthreads().
template <int NT>
__device__ __forceinline__ u32 block_excl_sum(u32 v, u32 *ws, u32 *total) {
    constexpr int W = NT / 32;
    u32 inc = warp_incl_sum(v);
    if (lane_id() == 31) ws[warp_id()] = inc;
    __syncthreads();
    if (warp_id() == 0) {
        u32 x = lane_id() < (u32)W ? ws[lane_id()] : 0u;
        u32 xi = warp_incl_sum(x);
        if (lane_id() < (u32)W) ws[lane_id()] = xi - x;
        if (lane_id() == (u32)W - 1) ws[W] = xi;
    }
    __syncthreads();
    u32 r = ws[warp_id()] + inc - v;
    if (total) *total = ws[W];
    __syncthreads();
    return r;
}

// Block-wide inclusive max-scan over NT threads; `ws` needs NT/32 words. Contains __syncthreads().
template <int NT>
__device__ __forceinline__ u32 block_incl_max(u32 v, u32 *ws) {
    constexpr int W = NT / 32;
    u32 inc = warp_incl_max(v);
    if (lane_id() == 31) ws[warp_id()] = inc;
    __syncthreads();
    if (warp_id() == 0) {
        u32 x = lane_id() < (u32)W ? ws[lane_id()] : 0u;
        u32 xi = warp_incl_max(x);
        if (lane_id() < (u32)W) ws[lane_id()] = xi;
    }
    __syncthreads();
    u32 before = warp_id() ? ws[warp_id() - 1] : 0u;
    __syncthreads();
    return max(before, inc);
}

// 8 bytes of T starting at i as a big-endian word (T[i] most significant). T must have 16 readable bytes past
// every position read and an 8-byte aligned base.
__device__ __forceinline__ u64 load_be64(const u8 *__restrict__ T, u64 i) {
    const u64 *p = reinterpret_cast<const u64 *>(T + (i & ~7ull));
    u64 a = __ldg(p), b = __ldg(p + 1);
    u32 s = (u32)(i & 7) * 8;
    u64 w = s ? (a >> s) | (b << (64 - s)) : a;
    u32 lo = (u32)w, hi = (u32)(w >> 32);
    return ((u64)__byte_perm(lo, 0, 0x0123) << 32) | (u64)__byte_perm(hi, 0, 0x0123);
}

// ---- host-side kernel profiler: CUDA events around every launch of the plain path, tagged with the kernel, the
// round and the size of the kernel's input (elements and segments of its work list).
enum KernelId : int {
    K_INIT, K_FIXUP, K_KEYGEN, K_MSD_HIST, K_MSD_SCAN, K_MSD_SCATTER, K_TILE_PREFIX, K_TILE_PREFIX_KEYED,
    K_TILE_RANK, K_TILE_RANK_KEYED, K_CTL, K_SAMPLES,
    K_WARP_PREFIX, K_WARP_PREFIX_KEYED, K_WARP_RANK, K_WARP_RANK_KEYED,
    K_LSD_BEGIN, K_LSD_KEY0, K_LSD_HIST, K_LSD_PASS, K_SEG_COUNT, K_SEG_SCAN, K_SEG_EMIT1, K_SEG_EMIT2, K_GROUP, K_GROUP_WARP, K_MKEYS, K_LSD_IDENT, K_SEG_RANK,
    K_INV_TILEHIST, K_INV_COLSCAN, K_INV_SCATTER, K_INV_WALK, K_INV_RANKINIT, K_INV_JUMP, K_INV_EMIT, K_CHAIN, K_NKERNELS
};
const char *kernel_name(int k);

struct ProfRec {
    int kernel, round, pass;
    u32 elems, segs;
    cudaEvent_t e0, e1;
    float ms;
};

struct Profiler {
    bool on = false;
    std::vector<ProfRec> recs;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    int kernel = 0, round = 0, pass = 0;
    u32 elems = 0, segs = 0;
    void tag(int k, u32 e, u32 sg = 0) { kernel = k; elems = e; segs = sg; }
    void reset() { recs.clear(); used = 0; }
    cudaEvent_t ev() {
        if (used == pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            pool.push_back(e);
        }
        return pool[used++];
    }
    // wraps one launch
    template <typename F>
    cudaError_t launch(cudaStream_t s, F fn) {
        if (!on) return fn();
        ProfRec r{kernel, round, pass, elems, segs, ev(), ev(), 0.f};
        if (r.e0) cudaEventRecord(r.e0, s);
        cudaError_t e = fn();
        if (r.e1) cudaEventRecord(r.e1, s);
        recs.push_back(r);
        return e;
    }
    // after the stream has synchronised
    void finish() {
        for (auto &r : recs)
            if (r.e0 && r.e1 && cudaEventElapsedTime(&r.ms, r.e0, r.e1) != cudaSuccess) r.ms = -1.f;
    }
    ~Profiler() {
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace kgb
