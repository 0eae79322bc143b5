/* kat_oracle.c -- TEST INFRASTRUCTURE: the reference's planted-pattern
 * known-answer data set, restated in C.
 *
 * code/engine_tensorfim/code/batch_proto/batch_proto.cu:
 *   xs64      :193     xorshift64 (<<13, >>7, <<17), 64-bit wrap-around
 *   gen_data  :195-231 from seed 0xC0FFEE123456789: n_pat patterns of
 *                      2..maxpat distinct items (sorted), frequency
 *                      (0.2 + 1.3 * (r % 1000) / 1000) / 100; then per
 *                      transaction every pattern fires when the low 32 bits
 *                      of the next draw fall below freq * 2^32; then
 *                      (int)(n_tx * 0.0002) noise bits per item
 *   constants :45-51   d = 512, n_tx = 2^23, 80 patterns of at most 6 items,
 *                      minsup 0.15% of n_tx
 * The bitmaps are uint32 words, bit t & 31 of word t >> 5 of row item.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t xs64(uint64_t *s) {
    *s ^= *s << 13;
    *s ^= *s >> 7;
    *s ^= *s << 17;
    return *s;
}

/* bits: d * (n_tx / 32) words, zeroed by the caller; pat_ptr: n_pat + 1;
 * pat_items: n_pat * maxpat; pat_freq: n_pat.  n_tx must be a multiple of 32. */
int orc_planted_kat(uint64_t n_tx, uint32_t d, uint32_t n_pat, uint32_t maxpat, uint32_t *bits, uint32_t *pat_ptr,
                    uint32_t *pat_items, double *pat_freq) {
    if (n_tx % 32 || d == 0 || maxpat < 2 || n_pat == 0) return -1;
    const uint64_t W32 = n_tx / 32;
    uint64_t seed = 0xC0FFEE123456789ULL;
    uint32_t *thr = (uint32_t *)malloc(sizeof(uint32_t) * n_pat);
    if (!thr) return -1;
    pat_ptr[0] = 0;
    for (uint32_t p = 0; p < n_pat; ++p) {
        const uint32_t sz = 2 + (uint32_t)(xs64(&seed) % (maxpat - 1));
        const double freq = (0.2 + 1.3 * (double)(xs64(&seed) % 1000) / 1000.0) / 100.0;
        uint32_t *it = pat_items + pat_ptr[p];
        uint32_t n = 0;
        while (n < sz) {
            const uint32_t x = (uint32_t)(xs64(&seed) % d);
            int seen = 0;
            for (uint32_t i = 0; i < n; ++i) seen |= it[i] == x;
            if (!seen) it[n++] = x;
        }
        for (uint32_t i = 1; i < n; ++i)   /* std::sort of distinct ints */
            for (uint32_t j = i; j > 0 && it[j - 1] > it[j]; --j) {
                const uint32_t t = it[j - 1];
                it[j - 1] = it[j];
                it[j] = t;
            }
        pat_ptr[p + 1] = pat_ptr[p] + n;
        pat_freq[p] = freq;
        thr[p] = (uint32_t)(freq * 4294967296.0);
    }
    for (uint64_t t = 0; t < n_tx; ++t) {
        const uint64_t wd = t >> 5;
        const uint32_t bit = 1u << (t & 31);
        for (uint32_t p = 0; p < n_pat; ++p)
            if ((uint32_t)xs64(&seed) < thr[p])
                for (uint32_t i = pat_ptr[p]; i < pat_ptr[p + 1]; ++i) bits[(uint64_t)pat_items[i] * W32 + wd] |= bit;
    }
    const uint64_t n_noise = (uint64_t)(int)((double)n_tx * 0.0002);
    for (uint32_t j = 0; j < d; ++j)
        for (uint64_t q = 0; q < n_noise; ++q) {
            const uint64_t t = xs64(&seed) % n_tx;
            bits[(uint64_t)j * W32 + (t >> 5)] |= 1u << (t & 31);
        }
    free(thr);
    return 0;
}
