/*
 * pa_oracle.c -- CPU restatement of the privacy-amplification hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU engine: only
 * tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline leg and its
 * "--impl reference" arm) may load it.  The product library never links it and
 * never falls back to it.
 *
 * What it restates (paths relative to the nicoboss/PrivacyAmplification tree):
 *   - key split                  PrivacyAmplification/PrivacyAmplification.cu:861-892 (key2StartRest)
 *   - input bit order            PrivacyAmplification.cu:223-257, 584-593 (intTobinMask_dev, binInt2float):
 *                                bit i of a block = (word[i/32] >> (31 - i%32)) & 1
 *   - the product                cuFFT R2C/C2R convolution, PrivacyAmplification.cu:1898-1979:
 *                                out[i] = sum_{j=0..h} key_start[j] * seed[(i-j) mod n]   (mod 2)
 *                                The DC-zeroing + correction of PrivacyAmplification.cu:364-372,
 *                                408-418, 751 only changes the value by an even integer, so the
 *                                parity is that of the exact cyclic convolution.
 *   - rounding mod 2 + XOR       PrivacyAmplification.cu:740-813 (ToBinaryArray / ToBinaryArrayNoXOR),
 *                                output bit i -> byte i/8, bit 7-i%8 (AMPOUT_REVERSE_ENDIAN,
 *                                PrivacyAmplification.h:38, PrivacyAmplification.cu:260-267),
 *                                key_rest bit i = (key_rest[i/32] >> (31-i%32)) & 1 (the byte swap of
 *                                PrivacyAmplification.cu:756-762 makes both orders agree)
 *   - output length              do_compress ? v bits : n/2 bits (PrivacyAmplification.cu:1197, 2034-2040)
 *
 * Two independent ways of computing the convolution parity are given:
 *   (a) pa_oracle_direct: bit-packed rows, 64-bit AND + XOR-accumulate + parity.  O(out_bits * h / 64).
 *   (b) pa_oracle_ntt:    exact integer cyclic convolution by a number-theoretic transform modulo the
 *                         prime p = 2^64 - 2^32 + 1 (all values are <= h+1 < p, so it is exact).
 * Parity is pinned by the SHA3 known-answer vectors of examples/LargeBlocksizeExample/Matrix.h
 * (tests/golden/), which both (a) and (b) reproduce.
 *
 * Build: oracle/Makefile (gcc -O3 -fopenmp -shared).  Portable C99 + unsigned __int128 (x86_64, aarch64).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PA_FLAG_XOR_KEY_REST 1u
#define PA_FLAG_COMPRESS 2u

static inline uint32_t bit_msb(const uint32_t *w, uint64_t i) {
    return (w[i >> 5] >> (31u - (uint32_t)(i & 31u))) & 1u;
}

static inline uint32_t brev32(uint32_t x) {
    x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
    x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
    x = ((x >> 4) & 0x0F0F0F0Fu) | ((x & 0x0F0F0F0Fu) << 4);
    x = ((x >> 8) & 0x00FF00FFu) | ((x & 0x00FF00FFu) << 8);
    return (x >> 16) | (x << 16);
}

static inline uint64_t brev64(uint64_t x) { return ((uint64_t)brev32((uint32_t)x) << 32) | brev32((uint32_t)(x >> 32)); }

/* key2StartRest (PrivacyAmplification.cu:861-892): key_start = key words 0..h/32-1 plus the top bit of
 * word h/32 (h+1 bits); key_rest = key bits h+1 .. h+v realigned by a 1-bit left shift.
 * recv_key holds n/32+1 words.  key_start receives n/32 words (zero past h/32), key_rest v/32 words. */
void pa_oracle_key_split(const uint32_t *recv_key, uint32_t n, uint32_t v,
                         uint32_t *key_start, uint32_t *key_rest) {
    uint32_t hb = (n - v) / 32u, vb = v / 32u, nb = n / 32u;
    memset(key_start, 0, (size_t)nb * 4u);
    memcpy(key_start, recv_key, (size_t)hb * 4u);
    key_start[hb] = recv_key[hb] & 0x80000000u;
    for (uint32_t i = 0; i < vb; ++i)
        key_rest[i] = (recv_key[hb + i] << 1) | (recv_key[hb + i + 1] >> 31);
}

/* Number of output bits and bytes (PrivacyAmplification.cu:1197). */
uint32_t pa_oracle_out_bits(uint32_t n, uint32_t v, uint32_t flags) {
    return (flags & PA_FLAG_COMPRESS) ? v : n / 2u;
}

/* Writes out bits [i0, i1) of a parity vector into the reference byte stream. par[k] is the parity
 * of output bit i0+k.  XOR with key_rest applies to bits < v when PA_FLAG_XOR_KEY_REST is set. */
static void emit_bits(const uint8_t *par, uint64_t i0, uint64_t i1, const uint32_t *key_rest, uint32_t v,
                      uint32_t flags, uint8_t *out) {
    for (uint64_t i = i0; i < i1; ++i) {
        uint32_t b = par[i - i0] & 1u;
        if ((flags & PA_FLAG_XOR_KEY_REST) && key_rest && i < v) b ^= bit_msb(key_rest, i);
        uint8_t m = (uint8_t)(1u << (7u - (uint32_t)(i & 7u)));
        if (b) out[i >> 3] |= m; else out[i >> 3] &= (uint8_t)~m;
    }
}

/* ---------------------------------------------------------------- (a) direct bit-packed rows ---- */

/* Per-block state of the direct method: the key packed LSB-first (h+1 bits) and the seed stored
 * reversed and periodically extended, so that row i reads the window R[o .. o+h] with
 * o = (-i) mod n, R[m] = seed[(-m) mod n]. */
typedef struct {
    uint32_t n, h;
    uint64_t kw;
    uint64_t *K, *R;
} direct_ctx;

void *pa_oracle_direct_prepare(const uint32_t *seed, const uint32_t *key_start, uint32_t n, uint32_t v) {
    if (n == 0 || v >= n) return NULL;
    direct_ctx *c = (direct_ctx *)calloc(1, sizeof(direct_ctx));
    c->n = n;
    c->h = n - v;
    c->kw = ((uint64_t)c->h + 1u + 63u) / 64u;
    uint64_t rbits = (uint64_t)n + c->kw * 64u + 64u;
    uint64_t rw = (rbits + 63u) / 64u + 1u;
    c->K = (uint64_t *)calloc(c->kw, 8);
    c->R = (uint64_t *)calloc(rw, 8);
    /* K: key bits 0..h, LSB-first 64-bit words (bit-reversal of the MSB-first 32-bit words) */
    for (uint64_t w = 0; w <= c->h / 32; ++w) {
        uint64_t b = brev32(key_start[w]);
        c->K[w >> 1] |= b << (32 * (w & 1));
    }
    if ((c->h + 1) % 64) c->K[c->kw - 1] &= ~0ull >> (64 - (c->h + 1) % 64);
    /* S: seed, LSB-first; R[m] = S[(n - m) mod n], periodically extended: 64 bits of R at m0 are the
     * bit-reversed window S[a .. a+63] with a = n - m0 - 63 (taken mod n, bit by bit only on a wrap) */
    uint64_t sw = ((uint64_t)n + 63) / 64 + 1;
    uint64_t *S = (uint64_t *)calloc(sw, 8);
    for (uint64_t w = 0; w < n / 32; ++w) S[w >> 1] |= (uint64_t)brev32(seed[w]) << (32 * (w & 1));
    for (uint64_t k = 0; k * 64 < rbits; ++k) {
        uint64_t m0 = 64 * k, win = 0;
        int64_t a = ((int64_t)n - (int64_t)(m0 % n) - 63) % (int64_t)n;
        if (a < 0) a += n;
        if ((uint64_t)a + 63 < n) {
            uint64_t wi = (uint64_t)a >> 6, sh = (uint64_t)a & 63;
            win = sh ? (S[wi] >> sh) | (S[wi + 1] << (64 - sh)) : S[wi];
        } else {
            for (int b = 0; b < 64; ++b) {
                uint64_t idx = ((uint64_t)a + b) % n;
                win |= ((S[idx >> 6] >> (idx & 63)) & 1ull) << b;
            }
        }
        c->R[k] = brev64(win);
    }
    free(S);
    return c;
}

void pa_oracle_direct_free(void *ctx) {
    direct_ctx *c = (direct_ctx *)ctx;
    if (!c) return;
    free(c->K);
    free(c->R);
    free(c);
}

/* Parity of sum_{j=0..h} ks[j] * seed[(i-j) mod n] for i in [i0, i1); one byte per row. */
void pa_oracle_direct_rows(void *ctx, uint64_t i0, uint64_t i1, uint8_t *par, int nthreads) {
    direct_ctx *c = (direct_ctx *)ctx;
    const uint64_t kw = c->kw, n = c->n;
    const uint64_t *K = c->K, *R = c->R;
    (void)nthreads;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t ii = (int64_t)i0; ii < (int64_t)i1; ++ii) {
        uint64_t o = (n - ((uint64_t)ii % n)) % n;
        uint64_t ow = o >> 6, sh = o & 63;
        uint64_t acc = 0;
        if (sh == 0) {
            for (uint64_t w = 0; w < kw; ++w) acc ^= K[w] & R[ow + w];
        } else {
            for (uint64_t w = 0; w < kw; ++w)
                acc ^= K[w] & ((R[ow + w] >> sh) | (R[ow + w + 1] << (64 - sh)));
        }
        par[ii - (int64_t)i0] = (uint8_t)(__builtin_popcountll(acc) & 1);
    }
}

static void direct_rows(const uint32_t *seed, const uint32_t *key_start, uint32_t n, uint32_t h,
                        uint64_t i0, uint64_t i1, uint8_t *par, int nthreads) {
    void *c = pa_oracle_direct_prepare(seed, key_start, n, n - h);
    pa_oracle_direct_rows(c, i0, i1, par, nthreads);
    pa_oracle_direct_free(c);
}

/* Full or partial block by the direct method.  Computes output bits [i0, i1) (clipped to the output
 * length) and writes them into out (a buffer of the full output length; other bytes untouched apart
 * from the partial bytes at the range edges).  Returns 0, or -1 on bad sizes. */
int pa_oracle_direct(const uint32_t *seed, const uint32_t *key_start, const uint32_t *key_rest,
                     uint32_t n, uint32_t v, uint32_t flags, uint64_t i0, uint64_t i1, uint8_t *out,
                     int nthreads) {
    if (n == 0 || (n & 31u) || (v & 31u) || v == 0 || v >= n) return -1;
    uint64_t ob = pa_oracle_out_bits(n, v, flags);
    if (i1 > ob) i1 = ob;
    if (i0 >= i1) return 0;
    uint8_t *par = (uint8_t *)malloc(i1 - i0);
    direct_rows(seed, key_start, n, n - v, i0, i1, par, nthreads);
    emit_bits(par, i0, i1, key_rest, v, flags, out);
    free(par);
    return 0;
}

/* ---------------------------------------------------------------- (b) exact NTT ---------------- */

#define GP 0xFFFFFFFF00000001ull /* 2^64 - 2^32 + 1 */

static inline uint64_t gadd(uint64_t a, uint64_t b) {
    uint64_t s = a + b;
    if (s < a || s >= GP) s -= GP;
    return s;
}
static inline uint64_t gsub(uint64_t a, uint64_t b) { return a >= b ? a - b : a + (GP - b); }
static inline uint64_t gred(unsigned __int128 x) {
    /* 2^64 = 2^32 - 1 and 2^96 = -1 (mod p) */
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    uint64_t hh = hi >> 32, hl = hi & 0xFFFFFFFFull;
    uint64_t t = gsub(lo % GP, hh % GP);
    uint64_t u = hl * 0xFFFFFFFFull; /* < 2^64, may exceed p */
    return gadd(t, u % GP);
}
static inline uint64_t gmul(uint64_t a, uint64_t b) { return gred((unsigned __int128)a * b); }
static uint64_t gpow(uint64_t a, uint64_t e) {
    uint64_t r = 1;
    while (e) {
        if (e & 1) r = gmul(r, a);
        a = gmul(a, a);
        e >>= 1;
    }
    return r;
}

/* In-place iterative radix-2 NTT of length L (power of two <= 2^32), natural order in and out. */
static void ntt(uint64_t *a, uint64_t L, int inverse) {
    for (uint64_t i = 1, j = 0; i < L; ++i) {
        uint64_t bit = L >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { uint64_t t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (uint64_t len = 2; len <= L; len <<= 1) {
        /* 7 generates the multiplicative group of GP */
        uint64_t w = gpow(7, (GP - 1) / len);
        if (inverse) w = gpow(w, GP - 2);
        uint64_t half = len >> 1;
        uint64_t *tw = (uint64_t *)malloc(half * 8);
        tw[0] = 1;
        for (uint64_t k = 1; k < half; ++k) tw[k] = gmul(tw[k - 1], w);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (L >= (1u << 16))
#endif
        for (int64_t s = 0; s < (int64_t)L; s += (int64_t)len) {
            for (uint64_t k = 0; k < half; ++k) {
                uint64_t x = a[s + k], y = gmul(a[s + k + half], tw[k]);
                a[s + k] = gadd(x, y);
                a[s + k + half] = gsub(x, y);
            }
        }
        free(tw);
    }
    if (inverse) {
        uint64_t inv = gpow(L % GP, GP - 2);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (L >= (1u << 16))
#endif
        for (int64_t i = 0; i < (int64_t)L; ++i) a[i] = gmul(a[i], inv);
    }
}

/* Exact cyclic convolution c[i] = sum_{j=0..h} key_start[j] * seed[(i-j) mod n] for i < count.
 * Uses a length-n transform when n is a power of two, else a linear convolution of length
 * >= n+h+1 folded mod n.  conv receives count int64 values.  Returns 0 or -1. */
int pa_oracle_conv_exact(const uint32_t *seed, const uint32_t *key_start, uint32_t n, uint32_t v,
                         uint64_t count, int64_t *conv, int nthreads) {
    if (n == 0 || (n & 31u) || v >= n || count > n) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    uint32_t h = n - v;
    int pow2 = (n & (n - 1u)) == 0;
    uint64_t L = 1;
    uint64_t need = pow2 ? n : (uint64_t)n + h + 1u;
    while (L < need) L <<= 1;
    uint64_t *A = (uint64_t *)calloc(L, 8), *B = (uint64_t *)calloc(L, 8);
    if (!A || !B) { free(A); free(B); return -1; }
    for (uint64_t j = 0; j <= h; ++j) A[j] = bit_msb(key_start, j);
    for (uint64_t m = 0; m < n; ++m) B[m] = bit_msb(seed, m);
    ntt(A, L, 0);
    ntt(B, L, 0);
    for (uint64_t i = 0; i < L; ++i) A[i] = gmul(A[i], B[i]);
    ntt(A, L, 1);
    for (uint64_t i = 0; i < count; ++i) {
        uint64_t c = A[i];
        if (!pow2 && i + n < L) c += A[i + n];
        conv[i] = (int64_t)c;
    }
    free(A);
    free(B);
    return 0;
}

/* Full block by the exact NTT method; same output convention as pa_oracle_direct (all bits). */
int pa_oracle_ntt(const uint32_t *seed, const uint32_t *key_start, const uint32_t *key_rest, uint32_t n,
                  uint32_t v, uint32_t flags, uint8_t *out, int nthreads) {
    if (n == 0 || (n & 31u) || (v & 31u) || v == 0 || v >= n) return -1;
    uint64_t ob = pa_oracle_out_bits(n, v, flags);
    int64_t *c = (int64_t *)malloc(ob * 8);
    if (!c) return -1;
    if (pa_oracle_conv_exact(seed, key_start, n, v, ob, c, nthreads)) { free(c); return -1; }
    uint8_t *par = (uint8_t *)malloc(ob);
    for (uint64_t i = 0; i < ob; ++i) par[i] = (uint8_t)(c[i] & 1);
    free(c);
    emit_bits(par, 0, ob, key_rest, v, flags, out);
    free(par);
    return 0;
}

/* Popcount of the first `bits` bits of an MSB-first word array (the Hamming weights that
 * binInt2float accumulates, PrivacyAmplification.cu:594-599). */
uint64_t pa_oracle_popcount(const uint32_t *w, uint64_t bits) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < bits / 32; ++i) c += (uint64_t)__builtin_popcount(w[i]);
    if (bits & 31u) c += (uint64_t)__builtin_popcount(w[bits / 32] & ~(0xFFFFFFFFu >> (bits & 31u)));
    return c;
}
