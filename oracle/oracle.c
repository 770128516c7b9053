/* ORACLE -- test infrastructure only. This file is the CPU oracle of the GPU BWT path; it is never part of the
 * product. Only the tests, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 * A plain-C restatement of the reference's block-sorting entry points (src/algo/sais/sais.c:12027-12082 of
 * adnaneben/kolmo, declared in src/algo/sais/sais.h:10-20):
 *   orc_bwt_aux    = kolmo_sais_bwt_aux   (forward BWT with sampled indexes)
 *   orc_unbwt_aux  = kolmo_sais_unbwt_aux (inverse BWT)
 *   orc_unbwt      = kolmo_sais_unbwt     (inverse with the primary index only)
 * The reference computes the BWT by SA-IS induced sorting (libsais 2.12.1, sais.c:8747-8789). The suffix array of a
 * string is unique, so this file sorts with its own SA-IS (Nong, Zhang & Chan, "Two efficient algorithms for linear
 * time suffix array construction", 2009) and then applies the reference's output conventions:
 *   - the end of the text is an implicit sentinel smaller than every byte (a suffix sorts before its extensions);
 *   - U[0] = T[n-1]; row p+1 of the (n+1)-row matrix holds T[SA[p]-1]; the sentinel row is dropped
 *     (sais.c:12043-12049, the Metal restatement src/arch/metal/sa.metal:249-256);
 *   - I[0] = 1 + ISA[0] is the primary index, I[k] = 1 + ISA[k*r] for k <= (n-1)/r (sais.h:10-12, sais.c:6971-7041
 *     where the final induction scans record the 1-based row whenever a suffix index is a multiple of r).
 * The inverse is the LF walk of the reference's independent Python decoder (tests/bwt_reference.py:270-290).
 * Argument checks and return codes follow sais.c:12029-12038 and 12057-12068. */
#include <stdint.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- SA-IS over an int alphabet */
/* s[0..m) with s[m-1] == 0 the unique smallest symbol, symbols in [0, K). SA receives the suffix array. */
static void buckets_of(const int32_t *s, int32_t m, int32_t K, int32_t *bkt, int end) {
    memset(bkt, 0, (size_t)K * sizeof(int32_t));
    for (int32_t i = 0; i < m; i++) bkt[s[i]]++;
    int32_t sum = 0;
    for (int32_t c = 0; c < K; c++) { sum += bkt[c]; bkt[c] = end ? sum : sum - bkt[c]; }
}
static void induce(const int32_t *s, int32_t *SA, const uint8_t *t, int32_t m, int32_t K, int32_t *bkt) {
    buckets_of(s, m, K, bkt, 0);                                      /* L-type suffixes, left to right */
    for (int32_t i = 0; i < m; i++) {
        int32_t j = SA[i] - 1;
        if (SA[i] > 0 && !t[j]) SA[bkt[s[j]]++] = j;
    }
    buckets_of(s, m, K, bkt, 1);                                      /* S-type suffixes, right to left */
    for (int32_t i = m - 1; i >= 0; i--) {
        int32_t j = SA[i] - 1;
        if (SA[i] > 0 && t[j]) SA[--bkt[s[j]]] = j;
    }
}
#define IS_LMS(t, i) ((i) > 0 && (t)[i] && !(t)[(i) - 1])
static int sais_int(const int32_t *s, int32_t *SA, int32_t m, int32_t K) {
    uint8_t *t = (uint8_t *)malloc((size_t)m);
    int32_t *bkt = (int32_t *)malloc((size_t)K * sizeof(int32_t));
    if (!t || !bkt) { free(t); free(bkt); return -2; }
    t[m - 1] = 1;                                                     /* 1 = S-type, 0 = L-type */
    for (int32_t i = m - 2; i >= 0; i--) t[i] = s[i] < s[i + 1] || (s[i] == s[i + 1] && t[i + 1]);
    /* 1. sort the LMS substrings: LMS positions at their bucket ends, then two induction scans */
    buckets_of(s, m, K, bkt, 1);
    for (int32_t i = 0; i < m; i++) SA[i] = -1;
    for (int32_t i = 1; i < m; i++) if (IS_LMS(t, i)) SA[--bkt[s[i]]] = i;
    induce(s, SA, t, m, K, bkt);
    /* 2. compact the sorted LMS substrings and name them */
    int32_t n1 = 0;
    for (int32_t i = 0; i < m; i++) if (IS_LMS(t, SA[i])) SA[n1++] = SA[i];
    for (int32_t i = n1; i < m; i++) SA[i] = -1;
    int32_t name = 0, prev = -1;
    for (int32_t i = 0; i < n1; i++) {
        int32_t pos = SA[i], diff = 0;
        for (int32_t d = 0; d < m; d++) {
            if (prev == -1 || s[pos + d] != s[prev + d] || t[pos + d] != t[prev + d]) { diff = 1; break; }
            if (d > 0 && (IS_LMS(t, pos + d) || IS_LMS(t, prev + d))) break;
        }
        if (diff) { name++; prev = pos; }
        SA[n1 + pos / 2] = name - 1;
    }
    for (int32_t i = m - 1, j = m - 1; i >= n1; i--) if (SA[i] >= 0) SA[j--] = SA[i];
    /* 3. sort the reduced string (recursively when names repeat) */
    int32_t *s1 = SA + m - n1, *SA1 = SA;
    int rc = 0;
    if (name < n1) rc = sais_int(s1, SA1, n1, name);
    else for (int32_t i = 0; i < n1; i++) SA1[s1[i]] = i;
    if (rc) { free(t); free(bkt); return rc; }
    /* 4. place the sorted LMS suffixes at their bucket ends and induce the full order */
    for (int32_t i = 1, j = 0; i < m; i++) if (IS_LMS(t, i)) s1[j++] = i;
    for (int32_t i = 0; i < n1; i++) SA1[i] = s1[SA1[i]];
    for (int32_t i = n1; i < m; i++) SA[i] = -1;
    buckets_of(s, m, K, bkt, 1);
    for (int32_t i = n1 - 1; i >= 0; i--) { int32_t j = SA[i]; SA[i] = -1; SA[--bkt[s[j]]] = j; }
    induce(s, SA, t, m, K, bkt);
    free(t); free(bkt);
    return 0;
}

/* Suffix array of T[0..n) with the implicit smallest sentinel (a suffix sorts before every extension of it). */
int32_t orc_sa(const uint8_t *T, int32_t *SA, int32_t n) {
    if (!T || !SA || n < 0) return -1;
    if (n == 0) return 0;
    int32_t m = n + 1;
    int32_t *s = (int32_t *)malloc((size_t)m * sizeof(int32_t)), *sa = (int32_t *)malloc((size_t)m * sizeof(int32_t));
    if (!s || !sa) { free(s); free(sa); return -2; }
    for (int32_t i = 0; i < n; i++) s[i] = (int32_t)T[i] + 1;
    s[n] = 0;
    int rc = sais_int(s, sa, m, 257);
    if (!rc) memcpy(SA, sa + 1, (size_t)n * sizeof(int32_t));          /* sa[0] is the sentinel suffix n */
    free(s); free(sa);
    return rc;
}

/* kolmo_sais_bwt_aux semantics (sais.c:12027-12053). A is the caller's scratch, unused here but checked like the
 * reference checks it. Optionally returns the suffix array (SA may be NULL). */
int32_t orc_bwt_aux_sa(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, int32_t *I, int32_t *SAout) {
    if (!T || !U || !A || n < 0 || r < 2 || (r & (r - 1)) != 0 || !I) return -1;
    if (n <= 1) { if (n == 1) { U[0] = T[0]; if (SAout) SAout[0] = 0; } I[0] = n; return 0; }
    int32_t *SA = SAout ? SAout : (int32_t *)malloc((size_t)n * sizeof(int32_t));
    uint8_t *L = (uint8_t *)malloc((size_t)n + 1);
    if (!SA || !L) { if (!SAout) free(SA); free(L); return -2; }
    int rc = orc_sa(T, SA, n);
    if (!rc) {
        int32_t p0 = 0;
        L[0] = T[n - 1];                                              /* row 0: the sentinel rotation */
        for (int32_t p = 0; p < n; p++) {
            int32_t j = SA[p];
            if (j == 0) { p0 = p + 1; L[p + 1] = 0; } else L[p + 1] = T[j - 1];
            if (j % r == 0) I[j / r] = p + 1;
        }
        memcpy(U, L, (size_t)p0);                                     /* T == U allowed: T is read no more */
        memcpy(U + p0, L + p0 + 1, (size_t)(n - p0));
        I[0] = p0;
    }
    if (!SAout) free(SA);
    free(L);
    return rc;
}
int32_t orc_bwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, int32_t *I) {
    return orc_bwt_aux_sa(T, U, A, n, r, I, NULL);
}

/* The LF walk (tests/bwt_reference.py:270-290): L is U with the sentinel re-inserted at row idx; the C array counts
 * the sentinel as row 0; walking LF from row 0 emits the text backwards. rows (may be NULL) receives the row of
 * every suffix, i.e. 1 + ISA. Returns 0, or -2 when out of memory. */
static int32_t lf_walk(const uint8_t *U, uint8_t *out, int32_t n, int32_t idx, int32_t *rows) {
    uint32_t *lf = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    uint8_t *tmp = (uint8_t *)malloc((size_t)n);
    if (!lf || !tmp) { free(lf); free(tmp); return -2; }
    uint32_t cnt[256] = {0}, base[256];
    for (int32_t i = 0; i < n; i++) cnt[U[i]]++;
    uint32_t s = 1;
    for (int c = 0; c < 256; c++) { base[c] = s; s += cnt[c]; }
    lf[idx] = 0;
    for (int32_t q = 0; q <= n; q++) {
        if (q == idx) continue;
        uint8_t c = U[q - (q > idx)];
        lf[q] = base[c]++;
    }
    uint32_t row = 0;
    for (int32_t k = n - 1; k >= 0; k--) {
        tmp[k] = row == (uint32_t)idx ? 0 : U[row - (row > (uint32_t)idx)];
        row = lf[row];
        if (rows) rows[k] = (int32_t)row;
    }
    memcpy(out, tmp, (size_t)n);                                      /* T == U allowed */
    free(lf); free(tmp);
    return 0;
}

/* kolmo_sais_unbwt_aux semantics (sais.c:12055-12077): same argument checks and range checks of every sampled
 * index; the decode itself uses the primary index I[0]. */
int32_t orc_unbwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, const int32_t *I) {
    if (!T || !U || !A || n < 0 || ((r != n) && ((r < 2) || ((r & (r - 1)) != 0))) || !I) return -1;
    if (n <= 1) { if (I[0] != n) return -1; if (n == 1) U[0] = T[0]; return 0; }
    for (int32_t t = 0; t <= (n - 1) / r; t++) if (I[t] <= 0 || I[t] > n) return -1;
    return lf_walk(T, U, n, I[0], NULL);
}
/* Multi-threaded decode from the sampled indexes, as the reference's per-sample decoder does
 * (libsais_unbwt_decode_omp, sais.c:10842-): I[t] (t >= 1) is the row of the suffix starting at t * r, so segment t
 * [t*r, (t+1)*r) is produced by walking LF backwards from the row of suffix (t+1)*r (from row 0, the sentinel, for
 * the last segment). Every segment is independent; `threads` workers take them in turn. The LF table is built once.
 * Returns 0, -1 (arguments, as orc_unbwt_aux) or -2 (memory). */
struct seg_job {
    const uint8_t *U;
    uint8_t *out;
    const uint32_t *lf;
    const int32_t *I;
    int32_t n, r, idx, k, next, stride;
};
static void *seg_worker(void *arg) {
    struct seg_job *J = (struct seg_job *)arg;
    for (int32_t t = J->next; t <= J->k; t += J->stride) {
        const int32_t lo = t * J->r, hi = t == J->k ? J->n : (t + 1) * J->r;
        uint32_t row = t == J->k ? 0u : (uint32_t)J->I[t + 1];
        for (int32_t j = hi - 1; j >= lo; j--) {
            J->out[j] = row == (uint32_t)J->idx ? 0 : J->U[row - (row > (uint32_t)J->idx)];
            row = J->lf[row];
        }
    }
    return NULL;
}
int32_t orc_unbwt_aux_mt(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t r, const int32_t *I,
                         int32_t threads) {
    if (!T || !U || !A || n < 0 || ((r != n) && ((r < 2) || ((r & (r - 1)) != 0))) || !I) return -1;
    if (n <= 1) { if (I[0] != n) return -1; if (n == 1) U[0] = T[0]; return 0; }
    for (int32_t t = 0; t <= (n - 1) / r; t++) if (I[t] <= 0 || I[t] > n) return -1;
    const int32_t k = (n - 1) / r, idx = I[0];
    if (threads < 2 || k < 1) return lf_walk(T, U, n, idx, NULL);
    uint32_t *lf = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    uint8_t *tmp = (uint8_t *)malloc((size_t)n);
    if (!lf || !tmp) { free(lf); free(tmp); return -2; }
    uint32_t cnt[256] = {0}, base[256];
    for (int32_t i = 0; i < n; i++) cnt[T[i]]++;
    uint32_t s = 1;
    for (int c = 0; c < 256; c++) { base[c] = s; s += cnt[c]; }
    lf[idx] = 0;
    for (int32_t q = 0; q <= n; q++) {
        if (q == idx) continue;
        lf[q] = base[T[q - (q > idx)]]++;
    }
    if (threads > k + 1) threads = k + 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    struct seg_job *jobs = (struct seg_job *)malloc(sizeof(struct seg_job) * (size_t)threads);
    if (!th || !jobs) { free(lf); free(tmp); free(th); free(jobs); return -2; }
    char *live = (char *)calloc((size_t)threads, 1);
    if (!live) { free(lf); free(tmp); free(th); free(jobs); return -2; }
    for (int32_t w = 0; w < threads; w++) {
        jobs[w] = (struct seg_job){T, tmp, lf, I, n, r, idx, k, w, threads};
        if (pthread_create(&th[w], NULL, seg_worker, &jobs[w]) == 0) live[w] = 1;
        else seg_worker(&jobs[w]);  /* no thread: decode its segments here */
    }
    for (int32_t w = 0; w < threads; w++) if (live[w]) pthread_join(th[w], NULL);
    free(live);
    memcpy(U, tmp, (size_t)n); /* T == U allowed */
    free(lf); free(tmp); free(th); free(jobs);
    return 0;
}

/* kolmo_sais_unbwt (sais.c:12079-12082) */
int32_t orc_unbwt(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t i) {
    return orc_unbwt_aux(T, U, A, n, n, &i);
}

/* The suffix array implied by a BWT and its primary index, from the rows of the LF walk: SA[rows[k] - 1] = k. The
 * suffix array is a permutation, so this is the unique suffix array of the decoded text. */
int32_t orc_sa_from_bwt(const uint8_t *U, int32_t n, int32_t idx, int32_t *SA) {
    if (!U || !SA || n < 1 || idx < 1 || idx > n) return -1;
    int32_t *rows = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    uint8_t *tmp = (uint8_t *)malloc((size_t)n);
    if (!rows || !tmp) { free(rows); free(tmp); return -2; }
    int32_t rc = lf_walk(U, tmp, n, idx, rows);
    if (!rc) for (int32_t k = 0; k < n; k++) SA[rows[k] - 1] = k;
    free(rows); free(tmp);
    return rc;
}

uint64_t orc_fnv1a(const uint8_t *p, uint64_t n) {
    uint64_t h = 1469598103934665603ull;
    while (n--) { h ^= *p++; h *= 1099511628211ull; }
    return h;
}
