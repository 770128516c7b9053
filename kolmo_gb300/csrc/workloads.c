/* Seeded synthetic inputs for the BWT path, used by the benchmark and the autotuner: the benchmark sources (order-2
 * Markov bytes, Zipf word prose with verbatim repeats, ACGT, templated log lines, periodic text with flips, the
 * Fibonacci word) plus the size distributions of the batched and serving runs.
 *
 * Every generator is a pure function of its seed and produces the same bytes on x86-64 and aarch64: the only
 * floating point is IEEE double +, -, *, / and sqrt (correctly rounded on both), this file is compiled with
 * -ffp-contract=off, and log/exp are series evaluations written here instead of libm calls (whose last-ulp
 * results may differ between C libraries and architectures). Public domain methods used: splitmix64 and
 * xoshiro256** (Blackman & Vigna), Marsaglia-Tsang gamma sampling, Marsaglia's polar normal method. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- PRNG */
typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix64(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static void rng_seed(rng_t *r, uint64_t seed) { for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&seed); }
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t rng_next(rng_t *r) {
    uint64_t *s = r->s, res = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return res;
}
/* uniform in [0, k) (k > 0), multiply-shift (Lemire) without the rejection step: bias < k / 2^64 */
static inline uint64_t rng_below(rng_t *r, uint64_t k) { return (uint64_t)(((unsigned __int128)rng_next(r) * k) >> 64); }
/* uniform double in (0, 1): 53 random bits, never 0 */
static inline double rng_unit(rng_t *r) { return ((double)(rng_next(r) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

/* ---------------------------------------------------------------- portable log / exp */
static const double LN2 = 0.69314718055994530942;
/* natural log for x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), log(m) = 2 atanh((m - 1) / (m + 1)) */
static double k_log(double x) {
    if (!(x > 0)) return -1e300;
    int e = 0;
    while (x >= 1.4142135623730951) { x *= 0.5; e++; }
    while (x < 0.7071067811865476) { x *= 2.0; e--; }
    double z = (x - 1.0) / (x + 1.0), z2 = z * z, term = z, sum = 0.0;
    for (int k = 1; k < 60; k += 2) { sum += term / k; term *= z2; }
    return 2.0 * sum + e * LN2;
}
/* e^x: x = k ln2 + f, |f| <= ln2 / 2, Taylor series of e^f, then scaling by 2^k */
static double k_exp(double x) {
    if (x > 700) x = 700;
    if (x < -700) return 0.0;
    double kf = x / LN2;
    long k = (long)(kf < 0 ? kf - 0.5 : kf + 0.5);
    double f = x - (double)k * LN2, term = 1.0, sum = 1.0;
    for (int i = 1; i < 30; i++) { term *= f / i; sum += term; }
    while (k > 0) { sum *= 2.0; k--; }
    while (k < 0) { sum *= 0.5; k++; }
    return sum;
}
static double k_pow(double b, double e) { return k_exp(e * k_log(b)); }

/* standard normal (Marsaglia polar method) */
static double rng_normal(rng_t *r) {
    for (;;) {
        double u = 2.0 * rng_unit(r) - 1.0, v = 2.0 * rng_unit(r) - 1.0, s = u * u + v * v;
        if (s > 0.0 && s < 1.0) return u * __builtin_sqrt(-2.0 * k_log(s) / s);
    }
}
/* Gamma(a, 1) for a > 0 (Marsaglia & Tsang 2000; a < 1 through Gamma(a + 1) * U^(1/a)) */
static double rng_gamma(rng_t *r, double a) {
    double boost = 1.0;
    if (a < 1.0) { boost = k_pow(rng_unit(r), 1.0 / a); a += 1.0; }
    double d = a - 1.0 / 3.0, c = 1.0 / __builtin_sqrt(9.0 * d);
    for (;;) {
        double x = rng_normal(r), v = 1.0 + c * x;
        if (v <= 0) continue;
        v = v * v * v;
        double u = rng_unit(r);
        if (k_log(u) < 0.5 * x * x + d - d * v + d * k_log(v)) return d * v * boost;
    }
}

uint64_t kgw_fnv1a(const uint8_t *p, uint64_t n) {
    uint64_t h = 1469598103934665603ull;
    while (n--) { h ^= *p++; h *= 1099511628211ull; }
    return h;
}

/* ---------------------------------------------------------------- order-2 Markov bytes */
/* nsym distinct byte values (a seeded choice), 2-symbol contexts, each context's next-symbol distribution drawn
 * from Dirichlet(alpha). Rows are stored as cumulative 32-bit thresholds and sampled by binary search. */
int kgw_markov2(uint8_t *out, uint64_t n, uint64_t seed, int nsym, double alpha) {
    if (nsym < 2 || nsym > 256) return -1;
    rng_t r; rng_seed(&r, seed);
    uint8_t sym[256]; int perm[256];
    for (int i = 0; i < 256; i++) perm[i] = i;
    for (int i = 255; i > 0; i--) { int j = (int)rng_below(&r, (uint64_t)i + 1); int t = perm[i]; perm[i] = perm[j]; perm[j] = t; }
    for (int i = 0; i < nsym; i++) sym[i] = (uint8_t)perm[i];
    size_t rows = (size_t)nsym * nsym;
    uint32_t *cum = (uint32_t *)malloc(rows * nsym * sizeof(uint32_t));
    double *g = (double *)malloc(nsym * sizeof(double));
    if (!cum || !g) { free(cum); free(g); return -2; }
    for (size_t c = 0; c < rows; c++) {
        double tot = 0;
        for (int k = 0; k < nsym; k++) { g[k] = rng_gamma(&r, alpha); tot += g[k]; }
        double acc = 0;
        for (int k = 0; k < nsym; k++) {
            acc += g[k] / tot;
            double t = acc * 4294967296.0;
            cum[c * nsym + k] = k == nsym - 1 || t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
        }
    }
    int a = (int)rng_below(&r, (uint64_t)nsym), b = (int)rng_below(&r, (uint64_t)nsym);
    for (uint64_t i = 0; i < n; i++) {
        const uint32_t *row = cum + ((size_t)a * nsym + b) * nsym;
        uint32_t u = (uint32_t)(rng_next(&r) >> 32);
        int lo = 0, hi = nsym - 1;                                   /* first k with u < row[k] (u <= 2^32 - 2 ok) */
        while (lo < hi) { int mid = (lo + hi) >> 1; if (u < row[mid]) hi = mid; else lo = mid + 1; }
        out[i] = sym[lo]; a = b; b = lo;
    }
    free(cum); free(g);
    return 0;
}

/* ---------------------------------------------------------------- Zipf word prose with verbatim repeats */
/* vocab words of 2-12 lowercase letters, drawn with Zipf(s) over their rank, separated by a space (a newline with
 * probability 1/16); noise_ppm bytes per million of the generated words replaced by a uniform random byte; ncopies
 * verbatim copies of earlier [copy_min, copy_max] byte segments inserted at uniformly spread output offsets. */
int kgw_zipf_prose(uint8_t *out, uint64_t n, uint64_t seed, int vocab, double s, uint32_t noise_ppm,
                   int ncopies, uint32_t copy_min, uint32_t copy_max) {
    rng_t r; rng_seed(&r, seed);
    if (vocab < 1) return -1;
    char *words = (char *)malloc((size_t)vocab * 13);
    uint64_t *cdf = (uint64_t *)malloc((size_t)vocab * sizeof(uint64_t));
    uint64_t *ins = (uint64_t *)malloc((size_t)(ncopies > 0 ? ncopies : 1) * sizeof(uint64_t));
    if (!words || !cdf || !ins) { free(words); free(cdf); free(ins); return -2; }
    for (int w = 0; w < vocab; w++) {
        int L = 2 + (int)rng_below(&r, 11);
        for (int k = 0; k < L; k++) words[w * 13 + k] = (char)('a' + rng_below(&r, 26));
        words[w * 13 + L] = 0;
    }
    double tot = 0;
    for (int k = 1; k <= vocab; k++) tot += k_pow((double)k, -s);
    double acc = 0;
    for (int k = 1; k <= vocab; k++) {
        acc += k_pow((double)k, -s) / tot;
        double t = acc * 18446744073709551616.0;
        cdf[k - 1] = k == vocab || t >= 18446744073709549568.0 ? ~0ull : (uint64_t)t;
    }
    for (int c = 0; c < ncopies; c++) ins[c] = rng_below(&r, n);
    for (int i = 1; i < ncopies; i++) {                               /* insertion sort of the insertion offsets */
        uint64_t v = ins[i]; int j = i - 1;
        while (j >= 0 && ins[j] > v) { ins[j + 1] = ins[j]; j--; }
        ins[j + 1] = v;
    }
    uint64_t i = 0; int c = 0;
    while (i < n) {
        if (c < ncopies && i >= ins[c]) {
            uint64_t L = copy_min + rng_below(&r, (uint64_t)copy_max - copy_min + 1);
            c++;
            if (L < i) {
                uint64_t src = rng_below(&r, i - L + 1);
                for (uint64_t k = 0; k < L && i < n; k++) out[i++] = out[src + k];
            }
            continue;
        }
        uint64_t u = rng_next(&r);
        int lo = 0, hi = vocab - 1;
        while (lo < hi) { int mid = (lo + hi) >> 1; if (u < cdf[mid]) hi = mid; else lo = mid + 1; }
        const char *wd = words + lo * 13;
        for (int k = 0; wd[k] && i < n; k++) {
            uint8_t ch = (uint8_t)wd[k];
            if ((uint32_t)rng_below(&r, 1000000) < noise_ppm) ch = (uint8_t)rng_next(&r);
            out[i++] = ch;
        }
        if (i < n) out[i++] = rng_below(&r, 16) == 0 ? '\n' : ' ';
    }
    free(words); free(cdf); free(ins);
    return 0;
}

/* ---------------------------------------------------------------- ACGT with rare N */
int kgw_acgt(uint8_t *out, uint64_t n, uint64_t seed, uint32_t n_ppm) {
    rng_t r; rng_seed(&r, seed);
    static const uint8_t base[4] = {'A', 'C', 'G', 'T'};
    for (uint64_t i = 0; i < n; i++) {
        uint64_t x = rng_next(&r);
        out[i] = (uint32_t)((x >> 40) % 1000000) < n_ppm ? 'N' : base[x & 3];
    }
    return 0;
}

/* ---------------------------------------------------------------- templated log lines */
/* 40 templates, each a fixed run of words with slots: an increasing decimal timestamp, a dotted IPv4 from a pool of
 * 500 hosts, a 6-hex request id, a small decimal number. Lines end with '\n'. */
static const char *LOGW[] = {"GET", "POST", "PUT", "DELETE", "user", "login", "failed", "ok", "session", "opened",
    "closed", "request", "served", "bytes", "cache", "miss", "hit", "worker", "started", "stopped", "timeout", "retry",
    "db", "query", "slow", "index", "rebuild", "disk", "full", "warn", "error", "info", "debug", "auth", "token",
    "expired", "upstream", "reset", "connection", "from"};
enum { SLOT_TS = -1, SLOT_IP = -2, SLOT_HEX = -3, SLOT_NUM = -4 };
int kgw_logs(uint8_t *out, uint64_t n, uint64_t seed) {
    rng_t r; rng_seed(&r, seed);
    int tmpl[40][12], tlen[40];
    const int nw = (int)(sizeof(LOGW) / sizeof(LOGW[0]));
    for (int t = 0; t < 40; t++) {
        int L = 4 + (int)rng_below(&r, 8), k = 0;
        tmpl[t][k++] = SLOT_TS;
        tmpl[t][k++] = (int)rng_below(&r, 4) + 29;                     /* level word: warn/error/info/debug */
        for (; k < L; k++) {
            uint64_t x = rng_below(&r, 10);
            tmpl[t][k] = x == 0 ? SLOT_IP : x == 1 ? SLOT_HEX : x == 2 ? SLOT_NUM : (int)rng_below(&r, (uint64_t)nw);
        }
        tlen[t] = L;
    }
    uint32_t ips[500];
    for (int k = 0; k < 500; k++) ips[k] = (uint32_t)rng_next(&r);
    uint64_t ts = 1700000000000ull + rng_below(&r, 1000000000ull);
    uint64_t i = 0;
    char buf[64];
    while (i < n) {
        int t = (int)rng_below(&r, 40);
        ts += rng_below(&r, 2000);
        for (int k = 0; k < tlen[t] && i < n; k++) {
            int v = tmpl[t][k], L = 0;
            if (v == SLOT_TS) {                                         /* seconds.milliseconds */
                uint64_t x = ts / 1000; char tmp[24]; int m = 0;
                do { tmp[m++] = (char)('0' + x % 10); x /= 10; } while (x);
                while (m) buf[L++] = tmp[--m];
                unsigned ms = (unsigned)(ts % 1000);
                buf[L++] = '.'; buf[L++] = (char)('0' + ms / 100); buf[L++] = (char)('0' + ms / 10 % 10); buf[L++] = (char)('0' + ms % 10);
            } else if (v == SLOT_IP) {
                uint32_t ip = ips[rng_below(&r, 500)];
                for (int q = 3; q >= 0; q--) {
                    unsigned o = (ip >> (8 * q)) & 255; char tmp[4]; int m = 0;
                    do { tmp[m++] = (char)('0' + o % 10); o /= 10; } while (o);
                    while (m) buf[L++] = tmp[--m];
                    if (q) buf[L++] = '.';
                }
            } else if (v == SLOT_HEX) {
                uint32_t x = (uint32_t)rng_next(&r);
                buf[L++] = 'i'; buf[L++] = 'd'; buf[L++] = '=';
                for (int q = 5; q >= 0; q--) buf[L++] = "0123456789abcdef"[(x >> (4 * q)) & 15];
            } else if (v == SLOT_NUM) {
                unsigned x = (unsigned)rng_below(&r, 100000); char tmp[8]; int m = 0;
                do { tmp[m++] = (char)('0' + x % 10); x /= 10; } while (x);
                while (m) buf[L++] = tmp[--m];
            } else {
                const char *wd = LOGW[v];
                while (*wd) buf[L++] = *wd++;
            }
            buf[L++] = k + 1 == tlen[t] ? '\n' : ' ';
            for (int q = 0; q < L && i < n; q++) out[i++] = (uint8_t)buf[q];
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- degenerate inputs */
/* A seeded pattern of `period` bytes repeated to n bytes, then one random byte flipped (XOR with a nonzero byte)
 * at a random offset inside every flip_every bytes (0: no flips). */
int kgw_periodic(uint8_t *out, uint64_t n, uint64_t seed, uint64_t period, uint64_t flip_every) {
    rng_t r; rng_seed(&r, seed);
    if (period < 1) return -1;
    for (uint64_t i = 0; i < period && i < n; i++) out[i] = (uint8_t)('a' + rng_below(&r, 26));
    for (uint64_t i = period; i < n; i++) out[i] = out[i - period];
    if (flip_every)
        for (uint64_t b = 0; b < n; b += flip_every) {
            uint64_t span = n - b < flip_every ? n - b : flip_every;
            out[b + rng_below(&r, span)] ^= (uint8_t)(1 + rng_below(&r, 255));
        }
    return 0;
}
/* The Fibonacci word over {a, b}: S0 = a, S1 = ab, S(k) = S(k-1) S(k-2), truncated to n bytes. Since S(k-1) is a
 * prefix of S(k) the word is built in place by appending its own prefix of length |S(k-2)|. */
int kgw_fibonacci(uint8_t *out, uint64_t n) {
    if (n == 0) return 0;
    out[0] = 'a';
    if (n == 1) return 0;
    out[1] = 'b';
    uint64_t la = 1, lb = 2;
    while (lb < n) {
        for (uint64_t k = 0; k < la && lb + k < n; k++) out[lb + k] = out[k];
        uint64_t t = lb + la; la = lb; lb = t;
    }
    return 0;
}

/* ---------------------------------------------------------------- size and arrival distributions */
/* count sizes log-uniform in [lo, hi] */
void kgw_loguniform_sizes(uint64_t seed, int count, uint64_t lo, uint64_t hi, uint64_t *sizes) {
    rng_t r; rng_seed(&r, seed);
    double span = k_log((double)hi / (double)lo);
    for (int i = 0; i < count; i++) {
        uint64_t v = (uint64_t)((double)lo * k_exp(rng_unit(&r) * span));
        sizes[i] = v < lo ? lo : v > hi ? hi : v;
    }
}
/* count draws: a lognormal size (median, sigma, capped; at least 64 bytes), an exponential inter-arrival gap in
 * seconds with rate lambda, a uniform choice in [0, 1000) (the request mix) and a source id in [0, 3) */
void kgw_requests(uint64_t seed, int count, double median, double sigma, uint64_t cap, double lambda,
                  uint64_t *sizes, double *gaps, uint32_t *mix, uint32_t *source) {
    rng_t r; rng_seed(&r, seed);
    for (int i = 0; i < count; i++) {
        double v = median * k_exp(sigma * rng_normal(&r));
        uint64_t s = v >= (double)cap ? cap : (uint64_t)v;
        sizes[i] = s < 64 ? 64 : s;
        gaps[i] = -k_log(rng_unit(&r)) / lambda;
        mix[i] = (uint32_t)rng_below(&r, 1000);
        source[i] = (uint32_t)rng_below(&r, 3);
    }
}
/* a block from source kind 0 Markov, 1 ACGT, 2 log lines (the three sources of the mixed batch) */
int kgw_source_block(int source, uint8_t *out, uint64_t n, uint64_t seed) {
    switch (source) {
        case 0: return kgw_markov2(out, n, seed, 64, 0.3);
        case 1: return kgw_acgt(out, n, seed, 1000);
        case 2: return kgw_logs(out, n, seed);
        default: return -1;
    }
}
