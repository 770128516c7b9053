/* kgbwt: the GB300 block-sorting engine behind kolmo's BWT path (sm_103a CUDA).
 *
 * 1. Drop-in entry points. Same names, arguments, conventions and return codes as the reference's suffix-sorter
 *    interface (adnaneben/kolmo src/algo/sais/sais.h:10-20, implemented at src/algo/sais/sais.c:12027-12082), so
 *    this library links in place of the reference's sais.o and every caller (the codec-18 and codec-5 stream glue,
 *    src/codecs/bwt_stream.c:52, 73-74, 233, 294) stays unchanged. A is the caller's scratch; the device sorter
 *    checks it like the reference does and does not touch it. `threads` is accepted and ignored (the output never
 *    depends on it, as in the reference). Returns 0, -1 for bad arguments or indexes out of range (for the inverse
 *    also: a string that is not a valid BWT), -2 when device memory or the device is unavailable. There is no CPU
 *    fallback. Calls from several threads are serialised on one device context.
 * 2. Batch entry points: many blocks in one device pass (one CUDA-graph launch).
 * 3. Engine entry points: device-resident buffers on a caller stream, for servers that keep data on the GPU.
 */
#ifndef KGBWT_H
#define KGBWT_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1. drop-in (reference: src/algo/sais/sais.h:13) -------------------------------------------------------------
 * BWT of T[0..n) into U (T == U allowed). r, a power of two >= 2, is the sampling interval of the auxiliary indexes:
 * I[i] = 1 + rank of the suffix starting at i * r for i <= (n - 1) / r; I[0] is the primary index. */
int32_t kolmo_sais_bwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, int32_t *I, int32_t threads);

/* reference: src/algo/sais/sais.h:17. Inverse of the above (T == U allowed). r == n or a power of two >= 2; every
 * I[t], t <= (n - 1) / r, must lie in 1..n. The decode starts from the primary index I[0]. */
int32_t kolmo_sais_unbwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, const int32_t *I,
                             int32_t threads);

/* reference: src/algo/sais/sais.h:20. kolmo_sais_unbwt_aux with r = n and primary index i. */
int32_t kolmo_sais_unbwt(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t i, int32_t threads);

/* ---- 2. batches of host buffers ----------------------------------------------------------------------------------
 * No reference counterpart as one call: the reference runs one kolmo_sais_bwt_aux per block on its block workers
 * (src/core/blocks.c:181, src/core/compress.c:221). Each job has the meaning of one drop-in call; rc receives that
 * call's return code. The return value is 0 when every job succeeded, else the first nonzero rc. */
typedef struct {
    const uint8_t *T;
    uint8_t *U;
    int32_t n;
    int32_t r;
    int32_t *I;
    int32_t rc;
} kgbwt_fwd_job;

typedef struct {
    const uint8_t *T; /* BWT string */
    uint8_t *U;       /* decoded text */
    int32_t n;
    int32_t r;
    const int32_t *I;
    int32_t rc;
} kgbwt_inv_job;

#define KGBWT_PLAIN 1u /* one kernel launch per step with host synchronisation per round (no CUDA graph) */

int32_t kgbwt_fwd_batch(kgbwt_fwd_job *jobs, int32_t count, uint32_t flags);
int32_t kgbwt_inv_batch(kgbwt_inv_job *jobs, int32_t count, uint32_t flags);

/* ---- 3. engines on device buffers ---------------------------------------------------------------------------------
 * An engine owns the device workspace of one batch in flight; use one engine per concurrent stream. All pointers
 * below are device pointers except `blocks`. Enqueue calls return once the work is queued on `stream` (a
 * cudaStream_t, NULL = the legacy default stream); kgbwt_engine_wait synchronises with it and reports errors. */
typedef struct kgbwt_engine kgbwt_engine;

typedef struct {
    uint32_t off;  /* first byte of the block in the text buffer */
    uint32_t n;    /* length, >= 2 */
    uint32_t r;    /* sampling interval, power of two >= 2 */
    uint32_t iout; /* first sampled-index slot of the block */
} kgbwt_block;

typedef struct {
    uint32_t off; /* first byte of the block's BWT string and of its decoded text */
    uint32_t n;   /* length, >= 2 */
    uint32_t p0;  /* primary index I[0], 1..n */
    uint32_t pad;
} kgbwt_iblock;

kgbwt_engine *kgbwt_engine_create(void);
void kgbwt_engine_destroy(kgbwt_engine *e);
/* tile_cap 4096 or 8192 (largest group sorted in one tile = tile_cap / 2); tile_ctas, msd_ctas: persistent CTAs
 * per SM of the tile sorter and of the bucket passes. 0 keeps the current value. Returns 0 or -1. */
int32_t kgbwt_engine_config(kgbwt_engine *e, int32_t tile_cap, int32_t tile_ctas, int32_t msd_ctas);
/* Tuning options (results never depend on them). Returns 0 or -1 for an unknown option or value.
 * KGBWT_OPT_SMALL_GROUP (0..1024, default 64): tiles whose groups are all at most this long are sorted by counting
 *   inside each group instead of radix passes (0: always radix).
 * KGBWT_OPT_WARP_PATH (0/1, default 1): tiles whose groups are all at most 32 long go to the warp-level kernel.
 * KGBWT_OPT_LSD_ROUND0 (0/1, default 1): the first round (all suffixes by their 8-byte prefix) is one LSD radix
 *   sort of the whole batch; 0: bucket passes and tile kernels as in the later rounds. */
#define KGBWT_OPT_SMALL_GROUP 1
#define KGBWT_OPT_WARP_PATH 2
#define KGBWT_OPT_LSD_ROUND0 3
int32_t kgbwt_engine_option(kgbwt_engine *e, int32_t option, int32_t value);
/* Forward: text blocks in dT (16 readable bytes past the last block). Results: dL receives each block's L column
 * with its sentinel row (n + 1 bytes at off + block index; row p0 holds no text byte), dI the sampled indexes at
 * iout (dI[iout] = primary index), dSA (may be NULL) the suffix array at off. */
int32_t kgbwt_engine_fwd(kgbwt_engine *e, const uint8_t *dT, uint8_t *dL, int32_t *dI, int32_t *dSA,
                         const kgbwt_block *blocks, int32_t count, void *stream, uint32_t flags);
/* Inverse: BWT strings (sentinel removed, as the drop-in U) in dU; decoded texts into dOut at the same offsets. */
int32_t kgbwt_engine_inv(kgbwt_engine *e, const uint8_t *dU, uint8_t *dOut, const kgbwt_iblock *blocks,
                         int32_t count, void *stream, uint32_t flags);
/* Waits for the engine's last enqueued call. status (may be NULL) receives one code per block of an inverse call
 * (0, or -1 for a string that is not a valid BWT). Returns 0 or the first error. */
int32_t kgbwt_engine_wait(kgbwt_engine *e, int32_t *status);
/* Statistics of the engine's last call: doubling rounds, bucket passes, kernels launched (-1: one graph launch). */
int32_t kgbwt_engine_stats(kgbwt_engine *e, int32_t *rounds, int32_t *passes, int64_t *launches);
/* Device bytes held by the engine's workspaces. */
uint64_t kgbwt_engine_workspace_bytes(kgbwt_engine *e);

/* Kernel profile of the engine's plain-path calls (flag KGBWT_PLAIN): with profiling enabled every kernel launch is
 * bracketed by CUDA events on the call's stream. After kgbwt_engine_wait, kgbwt_engine_profile_read copies up to
 * cap records of the last call and returns their number. kernel is an id named by kgbwt_kernel_name; elems / segs
 * are the size of the launch's input (elements and groups of its work list; bytes or chain records for the inverse). */
typedef struct {
    int32_t kernel;
    int32_t round;
    int32_t pass;
    uint32_t elems;
    uint32_t segs;
    float ms;
} kgbwt_prof;
int32_t kgbwt_engine_profile(kgbwt_engine *e, int32_t enable);
int32_t kgbwt_engine_profile_read(kgbwt_engine *e, kgbwt_prof *out, int32_t cap);
const char *kgbwt_kernel_name(int32_t kernel);

/* ---- allocation-free inverse --------------------------------------------------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device memory (an embedding host that owns
 * every device allocation through its own pool, a plugin inside such a host, a process whose device footprint must
 * not grow after start-up): the inverse BWT of one block with all scratch in a static device array inside this
 * library, sized for n <= 262144 bytes (about 2.5 MB, held on every GPU that loads the library until exit).
 * dU: the block's BWT string (sentinel removed, as the drop-in U), dT: the decoded text, both device buffers of n
 * bytes; p0 = I[0]. Returns 0, -1 for bad arguments, n above the maximum, or a string that is not a valid BWT,
 * -2 for a CUDA error. The call waits for its work on `stream` (a cudaStream_t, NULL = the legacy default stream).
 * It calls no device allocator. Every call uses the same static array: calls that overlap on the GPU (from two
 * host threads, or on two streams) race and corrupt each other. The first call on each device looks up the array's
 * device address; make that first call before any stream capture. */
int32_t kgbwt_unbwt_noalloc(const uint8_t *dU, uint8_t *dT, int32_t n, int32_t p0, void *stream);

/* ---- misc --------------------------------------------------------------------------------------------------------- */
const char *kgbwt_last_error(void); /* text of the last error on this thread ("" if none) */
int32_t kgbwt_version(void);

#ifdef __cplusplus
}
#endif
#endif
