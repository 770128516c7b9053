/* libcubwt's C entry points on the GB300 sorter. libbsc calls these from its GPU hook (bwt.cpp built with
 * LIBBSC_CUDA_SUPPORT): allocate, then bwt_aux (or unbwt), then free, for a BWT block. The reference routes the same
 * five functions to its Metal sorter (adnaneben/kolmo src/arch/metal/cubwt_metal.c:14-37); linking this library
 * instead sends them to the GPU here, with the drop-in calls' exact bytes.
 *
 * Return codes: 0 on success; every failure is negative (the caller tests for success only): KGBWT_CUBWT_BAD_PARAMETER
 * for arguments outside the contract, KGBWT_CUBWT_NOT_ENOUGH_MEMORY when the device workspace cannot be allocated,
 * KGBWT_CUBWT_GPU_ERROR for any other device failure (and a string that is not a valid BWT in unbwt).
 *
 * Storage: one sorting worker (its own engines, stream and pinned staging); calls on one storage are serialised,
 * different storages run concurrently. bwt_aux: T, L host buffers of n bytes (2 <= n <= 2^30), r a power of two
 * with 2 <= r <= n; L receives the BWT without its sentinel row and I ((n - 1) / r + 1 entries) the 1-based rows of
 * the suffixes at multiples of r (I[0] the primary index), exactly as kolmo_sais_bwt_aux. bwt: the same with only the
 * primary index, which it returns (> 0) instead of 0. unbwt: the inverse from the primary index i (freq, a symbol
 * count table some callers pass, is not needed and may be NULL). */
#ifndef KGBWT_CUBWT_H
#define KGBWT_CUBWT_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGBWT_CUBWT_NO_ERROR 0
#define KGBWT_CUBWT_BAD_PARAMETER (-1)
#define KGBWT_CUBWT_NOT_ENOUGH_MEMORY (-2)
#define KGBWT_CUBWT_GPU_ERROR (-3)

int64_t libcubwt_allocate_device_storage(void **device_storage, int64_t max_length);
int64_t libcubwt_free_device_storage(void *device_storage);
int64_t libcubwt_bwt_aux(void *device_storage, const uint8_t *T, uint8_t *L, int64_t n, int64_t r, uint32_t *I);
int64_t libcubwt_bwt(void *device_storage, const uint8_t *T, uint8_t *L, int64_t n);
int64_t libcubwt_unbwt(void *device_storage, const uint8_t *T, uint8_t *U, int64_t n, const int32_t *freq, int32_t i);

#ifdef __cplusplus
}
#endif
#endif
