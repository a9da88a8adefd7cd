// pa_ntt.cu -- exact path: integer cyclic convolution by NTT modulo p = 3*2^30 + 1.
//
// The FP32 path is exact only while every output value stays within its rounding budget; the engine
// measures that budget per block (max |x - rint(x)|).  Blocks that exceed it, blocks larger than the
// FP32 path supports (n > 2^27), and calls that ask for it (PA_FLAG_EXACT) run here instead:
// c = key_start (*) seed computed modulo p, which equals the integer convolution because
// 0 <= c[i] <= h+1 < 2^30 < p.  Parity, key_rest XOR and packing follow the reference
// (PrivacyAmplification.cu:740-813).
//
// Arithmetic: Montgomery multiplication with R = 2^32 (p > 2^31, so the reduction sum is formed in
// 64 bits); data in normal form, twiddles in Montgomery form.  Transforms: Stockham passes over HBM,
// each pass a radix-2^k stage (k <= 10) whose length-2^k sub-transforms run in shared memory as
// radix-2 DIF networks, 16 butterflies per CTA so that loads and stores move 64-byte row segments.
#include "pa_kernels.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace pa {
namespace ntt {

constexpr uint32_t P = 3221225473u;  // 3 * 2^30 + 1, primitive root 5
constexpr uint32_t G = 5u;

__host__ __device__ constexpr uint32_t neg_inv_p() {
    // -p^{-1} mod 2^32 by Newton iteration
    uint32_t x = P;  // p * p = 1 mod 8
    for (int i = 0; i < 5; ++i) x *= 2u - P * x;
    return 0u - x;
}
constexpr uint32_t PN = neg_inv_p();

__device__ __forceinline__ uint32_t mmul(uint32_t a, uint32_t b) {  // a * b * 2^-32 mod p
    const uint32_t lo = a * b, hi = __umulhi(a, b);
    const uint32_t m = lo * PN;
    const uint64_t u = (uint64_t)hi + __umulhi(m, P) + (lo != 0u);
    return (uint32_t)(u >= P ? u - P : u);
}
__device__ __forceinline__ uint32_t madd(uint32_t a, uint32_t b) {
    uint32_t s = a + b;
    return (s < a || s >= P) ? s - P : s;
}
__device__ __forceinline__ uint32_t msub(uint32_t a, uint32_t b) { return a >= b ? a - b : a - b + P; }

// host modular arithmetic for the tables
static uint64_t hmul(uint64_t a, uint64_t b) { return (uint64_t)((unsigned __int128)a * b % P); }
static uint64_t hpow(uint64_t a, uint64_t e) {
    uint64_t r = 1;
    for (a %= P; e; e >>= 1, a = hmul(a, a))
        if (e & 1) r = hmul(r, a);
    return r;
}
static uint32_t to_mont(uint64_t a) { return (uint32_t)((unsigned __int128)a * (1ull << 32) % P); }

}  // namespace ntt

using namespace ntt;

// Twiddle of exponent e (< L) in Montgomery form: thi[e >> 15] * tlo[e & 32767].
__device__ __forceinline__ uint32_t twiddle(const uint32_t* __restrict__ thi, const uint32_t* __restrict__ tlo,
                                            uint32_t e) {
    return mmul(__ldg(thi + (e >> 15)), __ldg(tlo + (e & 32767u)));
}

// One Stockham stage of radix R = 2^LOGR on L = 2^logL elements: butterfly j (< L/R) reads
// in[j + r L/R], multiplies by w_{Ns R}^{r (j mod Ns)}, transforms, writes out[(j/Ns) Ns R + j%Ns + r Ns].
template <int LOGR>
__global__ void __launch_bounds__(256) k_ntt_pass(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                  int logL, int logNs, const uint32_t* __restrict__ thi,
                                                  const uint32_t* __restrict__ tlo) {
    constexpr int R = 1 << LOGR, B = 16, RS = R + 1;  // 16 butterflies per CTA, padded rows
    __shared__ uint32_t s[B * RS];
    __shared__ uint32_t w[R / 2 > 0 ? R / 2 : 1];
    const uint32_t L = 1u << logL, LR = L >> LOGR, Ns = 1u << logNs;
    const uint32_t j0 = blockIdx.x * B;
    const int t = threadIdx.x;
    for (int k = t; k < R / 2; k += 256) w[k] = twiddle(thi, tlo, (uint32_t)k << (logL - LOGR));  // w_R^k
    for (int idx = t; idx < B * R; idx += 256) {
        const int r = idx / B, jj = idx % B;
        const uint32_t j = j0 + jj;
        uint32_t v = __ldcs(in + j + (size_t)r * LR);
        if (Ns > 1 && r) {
            const uint32_t e = (uint32_t)(((uint64_t)(L >> (logNs + LOGR)) * r * (j & (Ns - 1))) & (L - 1));
            v = mmul(v, twiddle(thi, tlo, e));
        }
        s[jj * RS + r] = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int hs = R / 2; hs >= 1; hs >>= 1) {  // radix-2 DIF, half size hs
        for (int i = t; i < B * R / 2; i += 256) {
            const int jj = i / (R / 2), ii = i % (R / 2);
            const int g = ii / hs, pos = ii % hs;
            uint32_t* row = s + jj * RS;
            const int ia = g * 2 * hs + pos, ib = ia + hs;
            const uint32_t a = row[ia], b = row[ib];
            row[ia] = madd(a, b);
            row[ib] = mmul(msub(a, b), w[pos * (R / (2 * hs))]);
        }
        __syncthreads();
    }
    if (Ns == 1) {  // outputs j R + r: contiguous per butterfly
        for (int idx = t; idx < B * R; idx += 256) {
            const int jj = idx / R, r = idx % R;
            const uint32_t j = j0 + jj;
            __stcs(out + (size_t)j * R + r, s[jj * RS + (int)(__brev((uint32_t)r) >> (32 - LOGR))]);
        }
    } else {  // outputs (j/Ns) Ns R + j%Ns + r Ns: 16 consecutive j share the block
        for (int idx = t; idx < B * R; idx += 256) {
            const int r = idx / B, jj = idx % B;
            const uint32_t j = j0 + jj;
            const size_t o = (size_t)(j & ~(Ns - 1)) * R + (j & (Ns - 1)) + (size_t)r * Ns;
            __stcs(out + o, s[jj * RS + (int)(__brev((uint32_t)r) >> (32 - LOGR))]);
        }
    }
}

// Placed key / seed bits -> 0/1 residues over the cyclic length Np.
__global__ void k_exact_bits(const uint32_t* __restrict__ src, BlockGeom g, int seed, uint32_t* __restrict__ a) {
    const uint64_t np = 1ull << g.log_np;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < np; x += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t s = x;
        bool on;
        if (seed) on = seed_source(g, x, &s);
        else on = x <= g.h;
        a[x] = on ? (__ldg(src + (s >> 5)) >> (31u - (uint32_t)(s & 31u))) & 1u : 0u;
    }
}

__global__ void k_exact_mul(uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint64_t np) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = mmul(a[i], __ldg(b + i));
}

// c[i] (scaled by `scale` = R^2 / Np, Montgomery) -> parity -> output word i/32, reference byte order.
__global__ void k_exact_out(const uint32_t* __restrict__ c, BlockGeom g, uint32_t scale,
                            const uint32_t* __restrict__ key_rest, uint32_t flags, uint32_t* __restrict__ out,
                            uint32_t nwords) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    uint32_t word = 0;
#pragma unroll 4
    for (int b = 0; b < 32; ++b) {
        const uint64_t i = 32ull * w + b;
        if (i < g.out_bits) word |= (mmul(__ldg(c + i), scale) & 1u) << (31 - b);
    }
    if ((flags & 1u) && 32ull * w < g.v) word ^= __ldg(key_rest + w);
    out[w] = __byte_perm(word, 0, 0x0123);
}

// ------------------------------------------------------------------------------------ host side
struct NttTables {
    int log_len = -1;
    uint32_t* d = nullptr;  // [fwd hi | fwd lo | inv hi | inv lo]
    size_t hi_n = 0;
};

static int make_tables(NttTables& tb, int logL, cudaStream_t s) {
    if (tb.log_len == logL) return 0;
    const size_t lo_n = 32768, hi_n = std::max<size_t>(1, (size_t(1) << logL) / 32768);
    std::vector<uint32_t> h(2 * (hi_n + lo_n));
    for (int dir = 0; dir < 2; ++dir) {
        uint64_t wL = hpow(G, (P - 1) >> logL);
        if (dir) wL = hpow(wL, P - 2);
        uint32_t* hi = h.data() + dir * (hi_n + lo_n);
        uint32_t* lo = hi + hi_n;
        uint64_t acc = 1;
        for (size_t k = 0; k < lo_n; ++k, acc = hmul(acc, wL)) lo[k] = to_mont(acc);
        const uint64_t step = hpow(wL, 32768);
        acc = 1;
        for (size_t k = 0; k < hi_n; ++k, acc = hmul(acc, step)) hi[k] = to_mont(acc);
    }
    if (tb.d) cudaFree(tb.d);
    tb.d = nullptr;
    cudaError_t e = cudaMalloc(&tb.d, h.size() * sizeof(uint32_t));
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyAsync(tb.d, h.data(), h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return (int)e;
    e = cudaStreamSynchronize(s);  // h is a host temporary
    if (e != cudaSuccess) return (int)e;
    tb.log_len = logL;
    tb.hi_n = hi_n;
    return 0;
}

template <int LOGR>
static void pass_l(const uint32_t* in, uint32_t* out, int logL, int logNs, const uint32_t* thi, const uint32_t* tlo,
                   cudaStream_t s) {
    const uint32_t blocks = (uint32_t)((1ull << logL) >> LOGR) / 16u;
    k_ntt_pass<LOGR><<<blocks, 256, 0, s>>>(in, out, logL, logNs, thi, tlo);
}

// Transform of length 2^logL in place in `a` (tmp: scratch of the same size).  Stage radices: passes of
// at most min(10, logL - 4) bits, so every pass has at least 16 butterflies per sub-transform column.
static int transform(uint32_t* a, uint32_t* tmp, int logL, bool inverse, const NttTables& tb, cudaStream_t s) {
    const uint32_t* thi = tb.d + (inverse ? tb.hi_n + 32768 : 0);
    const uint32_t* tlo = thi + tb.hi_n;
    const int maxr = std::min(10, logL - 4);
    std::vector<int> radices;
    for (int rem = logL; rem > 0;) {
        int r = std::min(maxr, rem);
        radices.push_back(r);
        rem -= r;
    }
    uint32_t* src = a;
    uint32_t* dst = tmp;
    int logNs = 0;
    for (int r : radices) {
        switch (r) {
            case 1: pass_l<1>(src, dst, logL, logNs, thi, tlo, s); break;
            case 2: pass_l<2>(src, dst, logL, logNs, thi, tlo, s); break;
            case 3: pass_l<3>(src, dst, logL, logNs, thi, tlo, s); break;
            case 4: pass_l<4>(src, dst, logL, logNs, thi, tlo, s); break;
            case 5: pass_l<5>(src, dst, logL, logNs, thi, tlo, s); break;
            case 6: pass_l<6>(src, dst, logL, logNs, thi, tlo, s); break;
            case 7: pass_l<7>(src, dst, logL, logNs, thi, tlo, s); break;
            case 8: pass_l<8>(src, dst, logL, logNs, thi, tlo, s); break;
            case 9: pass_l<9>(src, dst, logL, logNs, thi, tlo, s); break;
            default: pass_l<10>(src, dst, logL, logNs, thi, tlo, s); break;
        }
        logNs += r;
        std::swap(src, dst);
    }
    if (src != a) cudaMemcpyAsync(a, src, sizeof(uint32_t) << logL, cudaMemcpyDeviceToDevice, s);
    return (int)cudaGetLastError();
}

void free_ntt_tables(NttTables* t) {
    if (!t) return;
    cudaFree(t->d);
    delete t;
}

int exact_kernel_count(const BlockGeom& g) {
    const int logL = g.log_np, maxr = std::min(10, logL - 4);
    const int passes = (logL + maxr - 1) / maxr;
    return 1 + passes + 1 + passes + 1;
}

static int tables_for(NttTables** tb, int logL, cudaStream_t s) {
    if (!*tb) *tb = new NttTables();
    return make_tables(**tb, logL, s);
}

int launch_exact_seed(const BlockGeom& g, const uint32_t* seed, uint32_t* seed_hat, uint32_t* tmp, NttTables** tables,
                      cudaStream_t s) {
    if (g.log_np < 9 || g.log_np > 30) return (int)cudaErrorInvalidValue;
    int rc = tables_for(tables, g.log_np, s);
    if (rc) return rc;
    k_exact_bits<<<1184, 256, 0, s>>>(seed, g, 1, seed_hat);
    return transform(seed_hat, tmp, g.log_np, false, **tables, s);
}

int launch_exact_block(const BlockGeom& g, const uint32_t* key_start, const uint32_t* key_rest, uint32_t flags,
                       const uint32_t* seed_hat, uint32_t* a, uint32_t* tmp, uint32_t* out_words, NttTables** tables,
                       cudaStream_t s) {
    if (g.log_np < 9 || g.log_np > 30) return (int)cudaErrorInvalidValue;
    int rc = tables_for(tables, g.log_np, s);
    if (rc) return rc;
    const NttTables& tb = **tables;
    const uint64_t np = 1ull << g.log_np;
    k_exact_bits<<<1184, 256, 0, s>>>(key_start, g, 0, a);
    rc = transform(a, tmp, g.log_np, false, tb, s);
    if (rc) return rc;
    k_exact_mul<<<1184, 256, 0, s>>>(a, seed_hat, np);
    rc = transform(a, tmp, g.log_np, true, tb, s);
    if (rc) return rc;
    // a now holds Np * c * R^-1; scale = R^2 / Np in Montgomery form undoes both factors
    const uint64_t inv_np = hpow(np % P, P - 2);
    const uint32_t scale = to_mont(hmul(to_mont(inv_np), 1));  // (R / Np) * R mod p
    const uint32_t nwords = (g.out_bits + 31u) / 32u;
    k_exact_out<<<(nwords + 255) / 256, 256, 0, s>>>(a, g, scale, key_rest, flags, out_words, nwords);
    return (int)cudaGetLastError();
}

}  // namespace pa
