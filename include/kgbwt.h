/* kgbwt: the GB300 block-sorting engine behind kolmo's BWT path (sm_103a CUDA).
 *
 * 1. Drop-in entry points. Same names, arguments, conventions and return codes as the reference's suffix-sorter
 *    interface (adnaneben/kolmo src/algo/sais/sais.h:10-20, implemented at src/algo/sais/sais.c:12027-12082), so
 *    this library links in place of the reference's sais.o and every caller (the codec-18 and codec-5 stream glue,
 *    src/codecs/bwt_stream.c:52, 73-74, 233, 294) stays unchanged. A is the caller's scratch; the device sorter
 *    checks it like the reference does and does not touch it. `threads` is accepted and ignored (the output never
 *    depends on it, as in the reference). Returns 0, -1 for bad arguments or indexes out of range (for the inverse
 *    also: a string that is not a valid BWT), -2 when device memory or the device is unavailable. There is no CPU
 *    fallback. Calls from several threads share one device worker: concurrent calls are coalesced into batches
 *    (kgbwt_dropin_stats), and each call's result is the one it would get alone.
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
 * KGBWT_OPT_LSD_ROUND0 (0/1, default 1): the first round (all suffixes by their prefix) is one LSD radix sort of the
 *   whole batch; 0: bucket passes and tile kernels over 8-byte prefixes as in the later rounds.
 * KGBWT_OPT_LSD_BYTES (8, 12 or 16, default 16): prefix bytes that LSD round sorts (16 replaces the first rank round;
 *   the rank rounds then double from there).
 * KGBWT_OPT_CHAIN_FROM (0..64, default 1): from this rank round on, in rounds where doubling has stalled, a group of
 *   up to eight suffixes that doubling leaves whole is ordered along its repeat chain (the copies of a repeated
 *   stretch move through the rounds together and are ordered where the repeat ends) instead of waiting for the
 *   doubling to reach the repeat's end; 0: never. */
#define KGBWT_OPT_SMALL_GROUP 1
#define KGBWT_OPT_WARP_PATH 2
#define KGBWT_OPT_LSD_ROUND0 3
#define KGBWT_OPT_LSD_BYTES 4
#define KGBWT_OPT_CHAIN_FROM 5
int32_t kgbwt_engine_option(kgbwt_engine *e, int32_t option, int32_t value);
/* The configuration the engine's last forward call ran with: tile_cap, tile_ctas, msd_ctas, small_group, warp_path,
 * lsd_round0, lsd_bytes (cfg[0..6]). Fields the caller set with kgbwt_engine_config / kgbwt_engine_option are used as set; the
 * others come from the tuning table for the call's batch size when one is loaded, else the defaults. */
int32_t kgbwt_engine_last_config(kgbwt_engine *e, int32_t *cfg);
/* Tuning table (no counterpart in the reference): configurations by batch size, a JSON file written by
 * kolmo_gb300/autotune.py ({"buckets": [{"max_bytes": ..., "tile_ctas": ..., "msd_ctas": ..., "small_group": ...,
 * "warp_path": ..., "lsd_round0": ..., "lsd_bytes": ...}, ...]}; a batch of n bytes takes the first bucket with n <= max_bytes, else the
 * last). Loaded on first use from $KGBWT_TUNING ("off": none), else from tuning_gb300.json in the package directory.
 * kgbwt_tuning_load replaces it (NULL: no table) and returns the number of buckets or -1; kgbwt_tuning_lookup writes
 * the configuration a batch of n bytes would get (as kgbwt_engine_last_config) and returns 1 when it came from the
 * table, 0 for the defaults. */
int32_t kgbwt_tuning_load(const char *path);
int32_t kgbwt_tuning_lookup(uint64_t n, int32_t *cfg);
/* The same two reports with every configuration field: the first ncfg (1..KGBWT_CONFIG_FIELDS) of tile_cap,
 * tile_ctas, msd_ctas, small_group, warp_path, lsd_round0, lsd_bytes, chain_from (cfg[7]: the first rank round whose
 * tiny groups may follow repeat chains, 0 for none). Return values as kgbwt_tuning_lookup and
 * kgbwt_engine_last_config; -1 for ncfg < 1. */
#define KGBWT_CONFIG_FIELDS 8
int32_t kgbwt_tuning_lookup_n(uint64_t n, int32_t *cfg, int32_t ncfg);
int32_t kgbwt_engine_last_config_n(kgbwt_engine *e, int32_t *cfg, int32_t ncfg);
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
 * bytes; p0 = I[0]. Returns 0, -1 for bad arguments (a buffer that is not device or managed memory included), n
 * above the maximum, a string that is not a valid BWT, or a stream that is being captured, -2 for a CUDA error. The
 * call waits for its work on `stream` (a cudaStream_t, NULL = the legacy default stream) and reads its status back,
 * so it cannot be called while that stream is capturing. It calls no device allocator. Every call uses the same
 * static array: calls that overlap on the GPU (from two host threads, or on two streams) race and corrupt each
 * other. The first call on each device looks up the array's device address (with that device current). */
int32_t kgbwt_unbwt_noalloc(const uint8_t *dU, uint8_t *dT, int32_t n, int32_t p0, void *stream);

/* ---- request server -----------------------------------------------------------------------------------------------
 * No counterpart in the reference (its block workers call the sorter directly, src/core/blocks.c:181 and
 * src/core/pool.c:74). Compress (forward) and decompress (inverse) requests on host buffers are queued and run by
 * `slots` workers (1..16), each with its own engines and stream, so batches of different workers overlap on the GPU.
 * Continuous batching: a worker that is free takes the oldest pending request's kind and every later pending request
 * of that kind, in arrival order, while the batch's input stays within max_batch_bytes (0: 1 GiB) and the device
 * bytes held by all workers stay within hbm_budget (0: no limit). Workers keep their buffers resident between
 * batches and give them back when a pending batch could not be admitted otherwise; a request that cannot fit the
 * budget even alone fails with -2. A request's result equals that of kolmo_sais_bwt_aux / kolmo_sais_unbwt_aux on
 * the same arguments, whatever else shares its batch. Calls are thread-safe. */
typedef struct kgbwt_server kgbwt_server;
#define KGBWT_REQ_FWD 1 /* in = T (n bytes), out = U (n bytes), idx = I ((n-1)/r+1 entries, written), r = 2^k >= 2 */
#define KGBWT_REQ_INV 2 /* in = U (n bytes), out = T (n bytes), idx = I (read), r = 2^k >= 2 or r = n */
typedef struct {
    int64_t submitted, completed, failed, cancelled, batches;
    uint64_t bytes;      /* input bytes of the completed requests */
    uint64_t hbm_in_use; /* device bytes held by the workers now (reservations of running batches included) */
    uint64_t hbm_peak;
} kgbwt_server_stats;
kgbwt_server *kgbwt_server_create(int32_t slots, uint64_t hbm_budget, uint64_t max_batch_bytes);
/* Stops the workers after their running batches; pending requests end with -3 (cancelled). */
void kgbwt_server_destroy(kgbwt_server *s);
/* Queues one request; the host buffers must stay valid until it completes. Returns its id (>= 0) or -1. */
int64_t kgbwt_server_submit(kgbwt_server *s, int32_t kind, const uint8_t *in, uint8_t *out, int32_t *idx, int32_t n,
                            int32_t r);
/* Waits for request `id` (timeout_ms < 0: no limit). Returns 1 when it completed (*rc: 0, -1, -2 or -3 cancelled;
 * *latency_us: submission to completion; the id is then forgotten), 0 on timeout, -1 for an unknown id. */
int32_t kgbwt_server_wait(kgbwt_server *s, int64_t id, int32_t timeout_ms, int32_t *rc, double *latency_us);
/* Cancels a request that has not started: 0, or -1 when it is running, done or unknown. */
int32_t kgbwt_server_cancel(kgbwt_server *s, int64_t id);
int32_t kgbwt_server_stats_read(kgbwt_server *s, kgbwt_server_stats *st);
/* Test hook: the next `batches` batches fail as if their device allocation had failed (-2), without running. */
int32_t kgbwt_server_inject_oom(kgbwt_server *s, int32_t batches);
/* The batching policy on its own (host only): kinds[], n[], r[] of the pending requests in arrival order, the
 * worker's current forward / inverse workspace bytes and the device bytes it may hold after the batch. Writes the
 * indexes of the requests it would batch to take[] and returns their number (0: the oldest does not fit). */
int32_t kgbwt_server_plan(const int32_t *kinds, const int32_t *n, const int32_t *r, int32_t count, uint64_t have_fwd,
                          uint64_t have_inv, uint64_t avail, uint64_t max_batch_bytes, int32_t *take);
/* Device bytes a worker with no workspace needs for one batch of these requests (host only). */
uint64_t kgbwt_estimate_bytes(int32_t kind, const int32_t *n, const int32_t *r, int32_t count);

/* ---- coalescing of concurrent drop-in and batch calls -------------------------------------------------------------
 * No counterpart in the reference, whose block workers each run their own CPU sort (src/core/blocks.c:181,
 * src/core/compress.c:221, src/core/decode.c:405). Every call of sections 1 and 2 queues on the library's default
 * worker; the first caller to find it idle runs the oldest pending call together with every later pending call of
 * the same direction, in arrival order, while their input stays within KGBWT_BATCH_MIB (environment, default 256)
 * MiB, and the other callers wait. A job's own failure (bad arguments, a string that is no BWT) stays with that job;
 * if the combined batch fails as a whole (device memory, a layout too large), each of its calls is run again alone.
 * With KGBWT_STATS=<path> in the environment every batch appends one line to that file.
 * kgbwt_dropin_stats writes up to cap of: forward calls, forward batches, largest forward batch (calls), inverse
 * calls, inverse batches, largest inverse batch, combined batches retried call by call; returns 7. */
int32_t kgbwt_dropin_stats(int64_t *out, int32_t cap);

/* ---- misc --------------------------------------------------------------------------------------------------------- */
const char *kgbwt_last_error(void); /* text of the last error on this thread ("" if none) */
int32_t kgbwt_version(void);

#ifdef __cplusplus
}
#endif
#endif
