/* Test infrastructure: the block generator of the reference's suffix-sorter tests, so that the GPU path is tested on
 * the reference's own inputs. Same kinds and xorshift stream as tests/test_bwt.c:24-45 of adnaneben/kolmo (alike by
 * necessity: the inputs must be the same bytes); built and loaded by tests/refgen.py. */
#include <stdint.h>

/* Same kinds and xorshift stream as the generator of the reference's suffix-sorter tests (tests/test_bwt.c:24-45):
 * 0 zeros, 1 random, 2 0xF2-heavy, 3 periodic "abcabcabd", 4 ternary, 5 slow ramp, 6 second half repeats the first,
 * 7 periodic text with flags, 8 words with long repeats. */
void kgw_test_block(int kind, int n, uint8_t *in) {
    uint64_t x = 88172645463325252ull + (uint64_t)kind;
    static const char *words[] = {"the ", "block ", "sorting ", "kolmo ", "data ", "\n", "run ", "of ", "a ", "1234 "};
    int w = 0, wp = 0;
    for (int i = 0; i < n; i++) {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        switch (kind) {
            case 0: in[i] = 0; break;
            case 1: in[i] = (uint8_t)x; break;
            case 2: in[i] = (x & 3) ? 0xf2 : (uint8_t)(x >> 8); break;
            case 3: in[i] = (uint8_t)("abcabcabd"[i % 9]); break;
            case 4: in[i] = (uint8_t)(x % 3); break;
            case 5: in[i] = (uint8_t)((i / 1000) & 0xff); break;
            case 6: in[i] = i < n / 2 ? (uint8_t)x : in[i - n / 2]; break;
            case 7: in[i] = (i % 97 == 0) ? 0xf2 : (uint8_t)("the quick brown fox "[i % 20]); break;
            default:
                if (!words[w][wp]) {
                    w = (int)(x % 10); wp = 0;
                    if ((x >> 20) % 50 == 0 && i > 5000) {          /* a repeat of 200..499 bytes from 4000 back */
                        int L = 200 + (int)(x >> 40) % 300, s = i - 4000;
                        for (int k = 0; k < L && i < n; k++) in[i++] = in[s + k];
                        i--; continue;
                    }
                }
                in[i] = (uint8_t)words[w][wp++]; break;
        }
    }
}
