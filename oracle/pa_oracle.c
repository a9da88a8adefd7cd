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

/* Arithmetic modulo p = 2^64 - 2^32 + 1, values kept canonical in [0, p).  2^64 = 2^32 - 1 and
 * 2^96 = -1 (mod p), so a 128-bit product reduces with shifts, one multiply by 2^32 - 1 and carries
 * (no division). */
#define GP 0xFFFFFFFF00000001ull
#define GEPS 0xFFFFFFFFull /* 2^64 mod p */

/* Branch-free (masks instead of branches): transformed data is random, so branches would mispredict. */
static inline uint64_t gadd(uint64_t a, uint64_t b) {
    uint64_t s = a + b;
    s += (0 - (uint64_t)(s < a)) & GEPS;     /* wrapped past 2^64: add 2^64 mod p back; stays below 2^64 */
    return s - ((0 - (uint64_t)(s >= GP)) & GP);
}
static inline uint64_t gsub(uint64_t a, uint64_t b) { return a - b + ((0 - (uint64_t)(a < b)) & GP); }
static inline uint64_t gred(unsigned __int128 x) {
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    uint64_t hh = hi >> 32, hl = hi & GEPS;
    uint64_t t = lo - hh;                       /* lo + hl 2^64 + hh 2^96 = lo - hh + hl (2^32 - 1) */
    t -= (0 - (uint64_t)(lo < hh)) & GEPS;      /* borrow: the wrapped value holds an extra 2^64 = 2^32 - 1 */
    uint64_t u = hl * GEPS;                     /* < 2^64 */
    uint64_t r = t + u;
    r += (0 - (uint64_t)(r < u)) & GEPS;        /* carry: 2^64 = 2^32 - 1 again; cannot wrap twice */
    return r - ((0 - (uint64_t)(r >= GP)) & GP);
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
/* Primitive len-th root of unity (len a power of two <= 2^32); 7 generates the multiplicative group. */
static uint64_t groot(uint64_t len, int inverse) {
    uint64_t w = gpow(7, (GP - 1) / len);
    return inverse ? gpow(w, GP - 2) : w;
}

/* Transforms are cache-blocked: layers whose butterfly span fits a block of NTT_BLOCK values run block
 * by block (one pass over memory for all of them), the wider layers one pass each.  Twiddles of the
 * narrow layers come from per-length tables (tab[len/2 + k] = w_len^k), those of the wide layers are
 * formed by repeated multiplication, which is exact in the field. */
#define NTT_LOG_BLOCK 14
#define NTT_BLOCK (1ull << NTT_LOG_BLOCK)

typedef struct {
    uint64_t fwd[NTT_BLOCK], inv[NTT_BLOCK];
} root_tables;

static root_tables *g_roots;

static const root_tables *roots(void) {
    root_tables *r = __atomic_load_n(&g_roots, __ATOMIC_ACQUIRE);
    if (r) return r;
    r = (root_tables *)malloc(sizeof(root_tables));
    r->fwd[0] = r->inv[0] = 0;
    for (uint64_t len = 2; len <= NTT_BLOCK; len <<= 1) {
        uint64_t w = groot(len, 0), wi = groot(len, 1), a = 1, b = 1;
        for (uint64_t k = 0; k < len / 2; ++k) {
            r->fwd[len / 2 + k] = a;
            r->inv[len / 2 + k] = b;
            a = gmul(a, w);
            b = gmul(b, wi);
        }
    }
    root_tables *expected = NULL;
    if (!__atomic_compare_exchange_n(&g_roots, &expected, r, 0, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE)) {
        free(r);
        return expected;
    }
    return r;
}

/* All wide layers (len > NTT_BLOCK) of one direction.  A wide butterfly pairs indices that differ by a
 * multiple of NTT_BLOCK, so the wide layers act on each column of the L/NTT_BLOCK x NTT_BLOCK matrix
 * view separately: a thread copies WIDE_COLS neighbouring columns (one cache line per row) into a buffer,
 * runs every wide layer there and writes them back -- one pass over memory instead of one per layer.
 * Butterfly k = q NTT_BLOCK + c (row q of its block, column c) has twiddle w_len^k = w_lr^q w_len^c with
 * lr = len / NTT_BLOCK; the factors are formed once per layer, group and row q (not per block). */
#define WIDE_COLS 8

static void wide_layers(uint64_t *a, uint64_t L, int inverse) {
    const uint64_t M = L / NTT_BLOCK; /* rows */
    if (M < 2) return;
    int nl = 0;
    uint64_t wl[40], wr[40]; /* per layer: w_len, w_lr (inverse roots for the inverse transform) */
    for (uint64_t len = 2 * NTT_BLOCK; len <= L; len <<= 1, ++nl) {
        wl[nl] = groot(len, inverse);
        wr[nl] = groot(len / NTT_BLOCK, inverse);
    }
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        uint64_t *buf = (uint64_t *)malloc(M * WIDE_COLS * 8);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t g = 0; g < (int64_t)(NTT_BLOCK / WIDE_COLS); ++g) {
            const uint64_t c0 = (uint64_t)g * WIDE_COLS;
            for (uint64_t r = 0; r < M; ++r)
                for (int c = 0; c < WIDE_COLS; ++c) buf[r * WIDE_COLS + c] = a[r * NTT_BLOCK + c0 + c];
            for (int li = 0; li < nl; ++li) {
                /* DIF runs the layers from the widest down, DIT from the narrowest up */
                const int l = inverse ? li : nl - 1 - li;
                const uint64_t lr = 2ull << l, hr = lr >> 1; /* rows per block of this layer, half */
                uint64_t tc[WIDE_COLS];
                tc[0] = gpow(wl[l], c0);
                for (int c = 1; c < WIDE_COLS; ++c) tc[c] = gmul(tc[c - 1], wl[l]);
                /* row q of every block shares its twiddles: q outermost, so each is formed once */
                for (uint64_t q = 0; q < hr; ++q) {
                    for (uint64_t r0 = 0; r0 < M; r0 += lr) {
                        uint64_t *x = buf + (r0 + q) * WIDE_COLS, *y = x + hr * WIDE_COLS;
                        for (int c = 0; c < WIDE_COLS; ++c) {
                            if (!inverse) {
                                uint64_t u = x[c], v = y[c];
                                x[c] = gadd(u, v);
                                y[c] = gmul(gsub(u, v), tc[c]);
                            } else {
                                uint64_t u = x[c], v = gmul(y[c], tc[c]);
                                x[c] = gadd(u, v);
                                y[c] = gsub(u, v);
                            }
                        }
                    }
                    for (int c = 0; c < WIDE_COLS; ++c) tc[c] = gmul(tc[c], wr[l]);
                }
            }
            for (uint64_t r = 0; r < M; ++r)
                for (int c = 0; c < WIDE_COLS; ++c) a[r * NTT_BLOCK + c0 + c] = buf[r * WIDE_COLS + c];
        }
        free(buf);
    }
}

/* All layers with len <= min(L, NTT_BLOCK) on each block of that size. */
static void narrow_layers(uint64_t *a, uint64_t L, int inverse) {
    const root_tables *rt = roots();
    const uint64_t B = L < NTT_BLOCK ? L : NTT_BLOCK;
    const uint64_t *tab = inverse ? rt->inv : rt->fwd;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (L > B)
#endif
    for (int64_t b = 0; b < (int64_t)(L / B); ++b) {
        uint64_t *x = a + (uint64_t)b * B;
        if (!inverse) {
            for (uint64_t len = B; len >= 2; len >>= 1) {
                const uint64_t half = len >> 1, *w = tab + half;
                for (uint64_t s = 0; s < B; s += len)
                    for (uint64_t k = 0; k < half; ++k) {
                        uint64_t u = x[s + k], v = x[s + k + half];
                        x[s + k] = gadd(u, v);
                        x[s + k + half] = gmul(gsub(u, v), w[k]);
                    }
            }
        } else {
            for (uint64_t len = 2; len <= B; len <<= 1) {
                const uint64_t half = len >> 1, *w = tab + half;
                for (uint64_t s = 0; s < B; s += len)
                    for (uint64_t k = 0; k < half; ++k) {
                        uint64_t u = x[s + k], v = gmul(x[s + k + half], w[k]);
                        x[s + k] = gadd(u, v);
                        x[s + k + half] = gsub(u, v);
                    }
            }
        }
    }
}

/* Forward transform, natural order in, bit-reversed order out (decimation in frequency). */
static void ntt_dif(uint64_t *a, uint64_t L) {
    wide_layers(a, L, 0);
    narrow_layers(a, L, 0);
}

/* Inverse transform without the 1/L factor, bit-reversed order in, natural order out (decimation in
 * time): ntt_dit(ntt_dif(x)) = L x. */
static void ntt_dit(uint64_t *a, uint64_t L) {
    narrow_layers(a, L, 1);
    wide_layers(a, L, 1);
}

/* Transform length: n for power-of-two n (cyclic), else the next power of two >= n + h + 1 (a linear
 * convolution, folded mod n afterwards). */
static uint64_t conv_length(uint32_t n, uint32_t h) {
    int pow2 = (n & (n - 1u)) == 0;
    uint64_t L = 1, need = pow2 ? n : (uint64_t)n + h + 1u;
    while (L < need) L <<= 1;
    return L;
}

/* A seed's transform for blocks of size (n, v), scaled by 1/L so that one product and the inverse
 * transform give the convolution. */
typedef struct {
    uint32_t n, v, h;
    uint64_t L;
    uint64_t *S;
} ntt_seed;

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

void *pa_oracle_ntt_seed_prepare(const uint32_t *seed, uint32_t n, uint32_t v, int nthreads) {
    if (n == 0 || (n & 31u) || v >= n) return NULL;
    set_threads(nthreads);
    ntt_seed *c = (ntt_seed *)calloc(1, sizeof(ntt_seed));
    c->n = n;
    c->v = v;
    c->h = n - v;
    c->L = conv_length(n, c->h);
    c->S = (uint64_t *)malloc(c->L * 8);
    if (!c->S) { free(c); return NULL; }
    const uint64_t L = c->L;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t m = 0; m < (int64_t)L; ++m) c->S[m] = (uint64_t)m < n ? bit_msb(seed, (uint64_t)m) : 0u;
    ntt_dif(c->S, L);
    const uint64_t linv = gpow(L % GP, GP - 2);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < (int64_t)L; ++i) c->S[i] = gmul(c->S[i], linv);
    return c;
}

void pa_oracle_ntt_seed_free(void *ctx) {
    ntt_seed *c = (ntt_seed *)ctx;
    if (!c) return;
    free(c->S);
    free(c);
}

/* The exact linear (or, for power-of-two n, cyclic) convolution of key_start bits 0..h with the seed, in
 * natural order: L values, freed by the caller.  Value i + n folds onto i for non-power-of-two n. */
static uint64_t *conv_values(const ntt_seed *c, const uint32_t *key_start) {
    const uint64_t L = c->L, h = c->h;
    uint64_t *A = (uint64_t *)malloc(L * 8);
    if (!A) return NULL;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t j = 0; j < (int64_t)L; ++j) A[j] = (uint64_t)j <= h ? bit_msb(key_start, (uint64_t)j) : 0u;
    ntt_dif(A, L);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < (int64_t)L; ++i) A[i] = gmul(A[i], c->S[i]);
    ntt_dit(A, L);
    return A;
}

/* c[i] = sum_{j=0..h} key_start[j] * seed[(i-j) mod n] for i < count, exact, into conv (count values). */
static int conv_with_seed(const ntt_seed *c, const uint32_t *key_start, uint64_t count, int64_t *conv) {
    const uint64_t L = c->L, n = c->n;
    const int pow2 = (c->n & (c->n - 1u)) == 0;
    if (count > n) return -1;
    uint64_t *A = conv_values(c, key_start);
    if (!A) return -1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < (int64_t)count; ++i) {
        uint64_t v = A[i];
        if (!pow2 && (uint64_t)i + n < L) v += A[(uint64_t)i + n];
        conv[i] = (int64_t)v;
    }
    free(A);
    return 0;
}

/* Exact cyclic convolution c[i] = sum_{j=0..h} key_start[j] * seed[(i-j) mod n] for i < count.
 * Uses a length-n transform when n is a power of two, else a linear convolution of length
 * >= n+h+1 folded mod n.  conv receives count int64 values.  Returns 0 or -1. */
int pa_oracle_conv_exact(const uint32_t *seed, const uint32_t *key_start, uint32_t n, uint32_t v,
                         uint64_t count, int64_t *conv, int nthreads) {
    if (n == 0 || (n & 31u) || v >= n || count > n) return -1;
    ntt_seed *c = (ntt_seed *)pa_oracle_ntt_seed_prepare(seed, n, v, nthreads);
    if (!c) return -1;
    int rc = conv_with_seed(c, key_start, count, conv);
    pa_oracle_ntt_seed_free(c);
    return rc;
}

/* Full block with a prepared seed transform (pa_oracle_ntt_seed_prepare for the same n, v).  Output bit
 * i = c[i] mod 2 (XOR key_rest bit i for i < v when PA_FLAG_XOR_KEY_REST) goes to byte i/8, bit
 * 7 - i%8; the output length is a multiple of 8 bits. */
int pa_oracle_ntt_with_seed(void *ctx, const uint32_t *key_start, const uint32_t *key_rest, uint32_t flags,
                            uint8_t *out, int nthreads) {
    ntt_seed *c = (ntt_seed *)ctx;
    if (!c) return -1;
    set_threads(nthreads);
    const uint64_t ob = pa_oracle_out_bits(c->n, c->v, flags), L = c->L, n = c->n;
    const int pow2 = (c->n & (c->n - 1u)) == 0, x = (flags & PA_FLAG_XOR_KEY_REST) && key_rest;
    const uint32_t v = c->v;
    uint64_t *A = conv_values(c, key_start);
    if (!A) return -1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t b = 0; b < (int64_t)(ob / 8); ++b) {
        uint32_t byte = 0;
        for (uint32_t t = 0; t < 8; ++t) {
            uint64_t i = 8u * (uint64_t)b + t;
            uint32_t bit = (uint32_t)(A[i] & 1u);
            if (!pow2 && i + n < L) bit ^= (uint32_t)(A[i + n] & 1u);
            if (x && i < v) bit ^= bit_msb(key_rest, i);
            byte |= bit << (7u - t);
        }
        out[b] = (uint8_t)byte;
    }
    free(A);
    return 0;
}

/* Full block by the exact NTT method; same output convention as pa_oracle_direct (all bits). */
int pa_oracle_ntt(const uint32_t *seed, const uint32_t *key_start, const uint32_t *key_rest, uint32_t n,
                  uint32_t v, uint32_t flags, uint8_t *out, int nthreads) {
    if (n == 0 || (n & 31u) || (v & 31u) || v == 0 || v >= n) return -1;
    void *c = pa_oracle_ntt_seed_prepare(seed, n, v, nthreads);
    if (!c) return -1;
    int rc = pa_oracle_ntt_with_seed(c, key_start, key_rest, flags, out, nthreads);
    pa_oracle_ntt_seed_free(c);
    return rc;
}

/* Popcount of the first `bits` bits of an MSB-first word array (the Hamming weights that
 * binInt2float accumulates, PrivacyAmplification.cu:594-599). */
uint64_t pa_oracle_popcount(const uint32_t *w, uint64_t bits) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < bits / 32; ++i) c += (uint64_t)__builtin_popcount(w[i]);
    if (bits & 31u) c += (uint64_t)__builtin_popcount(w[bits / 32] & ~(0xFFFFFFFFu >> (bits & 31u)));
    return c;
}
