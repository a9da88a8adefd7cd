// pa_kernels.cu -- sm_103a kernels of the privacy-amplification hot path.
//
// Replaces, for one block, the reference's launch sequence (PrivacyAmplification.cu:1797-2042):
// binInt2float x2, calculateCorrectionFloat, cufftExecR2C x2, setFirstElementToZero,
// ElementWiseProduct, cufftExecC2R, ToBinaryArray[NoXOR] -- with no cuFFT and no float staging arrays.
//
// Two shapes:
//   * single-CTA ("mono") path, N = Np/2 <= 2^14 complex samples: the whole convolution of one block
//     in shared memory, bits in, packed bytes out;
//   * three-pass four-step path, N = N1 * N2 (N2 <= 2^14, N1 <= 2^12):
//       pass A  row FFTs over m2 (length N2) straight from the key bits, twiddle, write Y[m1][.]
//       pass B  column FFTs over m1 (length N1), real split, spectral product with the cached seed
//               spectrum (DC removed), real merge, inverse column FFTs, inverse twiddle, write Y
//       pass C  inverse row FFTs, + correction, round, parity -> bit planes
//       finish  bit planes -> reference byte order, XOR key_rest
//     Rows of Y are stored "pair-adjacent": column p and its mirror N2-p side by side, so that pass B
//     reads each mirror pair of columns as one 16-byte vector.
#include "pa_device.cuh"
#include "pa_kernels.cuh"

#include <algorithm>

namespace pa {

#define PA_FLAG_XOR_KEY_REST 1u
#define PA_FLAG_COMPRESS 2u

__device__ __forceinline__ uint32_t bit_of(const uint32_t* __restrict__ w, uint64_t x) {
    return (__ldg(w + (x >> 5)) >> (31u - (uint32_t)(x & 31u))) & 1u;
}

// Bits (x, x+1) of the key_start sequence (zero past bit h).  x is even.
__device__ __forceinline__ void key_pair(const uint32_t* __restrict__ ks, const BlockGeom& g, uint64_t x,
                                         uint32_t& b0, uint32_t& b1) {
    if (x + 1 <= g.h) {
        uint32_t w = __ldg(ks + (x >> 5));
        uint32_t o = (uint32_t)(x & 31u);
        b0 = (w >> (31u - o)) & 1u;
        b1 = (w >> (30u - o)) & 1u;
    } else {
        b0 = x <= g.h ? bit_of(ks, x) : 0u;
        b1 = 0u;
    }
}

// Bits (x, x+1) of the placed seed sequence.
__device__ __forceinline__ void seed_pair(const uint32_t* __restrict__ sd, const BlockGeom& g, uint64_t x,
                                          uint32_t& b0, uint32_t& b1) {
    if ((1u << g.log_np) == g.n) {
        uint32_t w = __ldg(sd + (x >> 5));
        uint32_t o = (uint32_t)(x & 31u);
        b0 = (w >> (31u - o)) & 1u;
        b1 = (w >> (30u - o)) & 1u;
        return;
    }
    uint64_t src;
    b0 = seed_source(g, x, &src) ? bit_of(sd, src) : 0u;
    b1 = seed_source(g, x + 1, &src) ? bit_of(sd, src) : 0u;
}

// W_N^e from the two-level table (e < N).
__device__ __forceinline__ float2 tw_n(const DeviceTables& t, uint32_t e) {
    return cmul(__ldg(t.glo + (e & 8191u)), __ldg(t.ghi + (e >> 13)));
}

__device__ __forceinline__ unsigned long long block_sum(unsigned long long v, unsigned long long* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    return t;  // valid in thread 0
}

__device__ __forceinline__ float block_max(float v, float* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = 0.f;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t = fmaxf(t, red[i]);
    return t;
}

// correction = (Ck * Cs / Np) mod 2: restores the parity removed with the DC bins
// (PrivacyAmplification.cu:364-372, 408-418).
__device__ __forceinline__ float correction(const unsigned long long* cnt, int log_np) {
    unsigned long long ck = cnt[0], cs = cnt[1];
    unsigned long long prod_mod = (ck * cs) & ((2ull << log_np) - 1ull);  // mod 2*Np (exact, Np <= 2^31)
    return (float)((double)prod_mod / (double)(1ull << log_np));
}

// Morton interleave of two 16-bit values: a -> even bits, b -> odd bits.
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
    x &= 0xFFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

// Output word from parities: bit t of sample u (u < 16) is output bit 2u+t of the word.  The result
// is the little-endian word of the reference byte stream (bit i -> byte i/8, bit 7-i%8), XORed with
// the MSB-first key_rest word when requested (PrivacyAmplification.cu:740-783).
__device__ __forceinline__ uint32_t out_word(uint32_t even16, uint32_t odd16, uint32_t key_rest_word) {
    uint32_t seq = spread16(even16) | (spread16(odd16) << 1);  // bit i%32 at position i%32
    uint32_t msb = __brev(seq) ^ key_rest_word;                // bit i%32 at position 31 - i%32
    return __byte_perm(msb, 0, 0x0123);                         // byte swap
}

// ============================================================================ setup kernels
__global__ void k_twiddle_tables(int log_n, float2* glo, float2* ghi, uint32_t nhi) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 8192u) glo[i] = expmi_pi(2u * i, log_n);             // W_N^i
    if (i < nhi) ghi[i] = expmi_pi((uint32_t)(2ull * 8192ull * i), log_n);  // W_N^(8192 i)
}

// ============================================================================ single-CTA path
// Loads the 2N placed bits into the tile; returns the number of ones seen by this thread.
template <int N, int NT, bool SEED>
__device__ __forceinline__ uint32_t mono_load(const uint32_t* __restrict__ bits, const BlockGeom& g, float2* sm) {
    uint32_t ones = 0;
    for (int m = threadIdx.x; m < N; m += NT) {
        uint32_t b0, b1;
        if (SEED) seed_pair(bits, g, 2ull * m, b0, b1);
        else key_pair(bits, g, 2ull * m, b0, b1);
        ones += b0 + b1;
        sm[pad16(m)] = make_float2((float)b0, (float)b1);
    }
    return ones;
}

template <int N, int NT>
__global__ void __launch_bounds__(NT) k_mono_seed(const uint32_t* __restrict__ seed, BlockGeom g,
                                                  float2* __restrict__ spec, unsigned long long* cnt_seed) {
    extern __shared__ float2 sm[];
    __shared__ unsigned long long red[32];
    uint32_t ones = mono_load<N, NT, true>(seed, g, sm);
    unsigned long long tot = block_sum(ones, red);
    if (threadIdx.x == 0) *cnt_seed = tot;
    __syncthreads();
    fft_tile<N, 1, NT, -1>(sm);
    const float sc = 1.0f / (float)(4ull << g.log_np);  // S' = 2X/(4Np) = X/(2Np)
    for (int k = threadIdx.x; k <= N / 2; k += NT) {
        if (k == 0) {
            float2 z = sm[0];
            spec[0] = make_float2(2.0f * (z.x - z.y) * sc, 0.0f);  // Nyquist bin X[N]; DC is dropped
            continue;
        }
        float2 za = sm[pad16(k)], zb = sm[pad16(N - k)];
        float2 xa, xb;
        real_split(za, zb, expmi_pi((uint32_t)k, g.log_n), xa, xb);
        spec[k] = cscale(xa, sc);
        if (k != N - k) spec[N - k] = cscale(xb, sc);
    }
}

template <int N, int NT>
__global__ void __launch_bounds__(NT) k_mono_key(const uint32_t* __restrict__ key_start,
                                                 const uint32_t* __restrict__ key_rest, BlockGeom g, uint32_t flags,
                                                 const float2* __restrict__ spec, unsigned long long* cnt,
                                                 unsigned int* resid_bits, uint32_t* __restrict__ out_words) {
    extern __shared__ float2 sm[];
    __shared__ unsigned long long red[32];
    __shared__ float redf[32];
    __shared__ float s_corr;
    uint32_t ones = mono_load<N, NT, false>(key_start, g, sm);
    unsigned long long tot = block_sum(ones, red);
    if (threadIdx.x == 0) {
        cnt[0] = tot;
        unsigned long long c2[2] = {tot, cnt[1]};
        s_corr = correction(c2, g.log_np);
    }
    __syncthreads();
    fft_tile<N, 1, NT, -1>(sm);
    for (int k = threadIdx.x; k <= N / 2; k += NT) {
        if (k == 0) {
            float2 z = sm[0];
            float pn = 2.0f * (z.x - z.y) * __ldg(&spec[0].x);
            sm[0] = make_float2(pn, -pn);
            continue;
        }
        float2 w = expmi_pi((uint32_t)k, g.log_n);
        float2 za = sm[pad16(k)], zb = sm[pad16(N - k)];
        float2 xa, xb, qa, qb;
        real_split(za, zb, w, xa, xb);
        float2 pa_ = cmul(xa, __ldg(spec + k)), pb_ = cmul(xb, __ldg(spec + (N - k)));
        real_merge(pa_, pb_, w, qa, qb);
        sm[pad16(k)] = qa;
        if (k != N - k) sm[pad16(N - k)] = qb;
    }
    __syncthreads();
    fft_tile<N, 1, NT, +1>(sm);
    const float corr = s_corr;
    const bool do_xor = flags & PA_FLAG_XOR_KEY_REST;
    float res = 0.f;
    const int lane = threadIdx.x & 31;
    for (int m = threadIdx.x; m < N; m += NT) {  // a warp covers 32 consecutive samples
        float2 q = sm[pad16(m)];
        uint32_t x0 = 2u * (uint32_t)m;
        float v0 = q.x + corr, v1 = q.y + corr;
        float r0 = rintf(v0), r1 = rintf(v1);
        bool ok0 = x0 < g.out_bits, ok1 = x0 + 1 < g.out_bits;
        uint32_t b0 = ok0 ? ((uint32_t)(int)r0 & 1u) : 0u;
        uint32_t b1 = ok1 ? ((uint32_t)(int)r1 & 1u) : 0u;
        if (ok0) res = fmaxf(res, fabsf(v0 - r0));
        if (ok1) res = fmaxf(res, fabsf(v1 - r1));
        uint32_t be = __ballot_sync(0xffffffffu, b0), bo = __ballot_sync(0xffffffffu, b1);
        if (lane < 2) {
            uint32_t w = (uint32_t)(m - lane) / 16u + lane;  // two words per 32 samples
            if (32u * w < g.out_bits) {
                uint32_t kr = (do_xor && 32u * w < g.v) ? __ldg(key_rest + w) : 0u;
                out_words[w] = out_word(lane ? be >> 16 : be, lane ? bo >> 16 : bo, kr);
            }
        }
    }
    float bm = block_max(res, redf);
    if (threadIdx.x == 0) atomicMax(resid_bits, __float_as_uint(bm));
}

// ============================================================================ three-pass path
// Pass A: row m1 of the N1 x N2 view (element m2 <-> complex sample m1 + N1*m2), FFT over m2,
// twiddle W_N^{m1 k2}, store pair-adjacent.
template <int N2, int NT, bool SEED>
__global__ void __launch_bounds__(NT) k_pass_a(const uint32_t* __restrict__ bits, BlockGeom g, DeviceTables tw,
                                               float2* __restrict__ Y, unsigned long long* cnt) {
    extern __shared__ float2 sm[];
    __shared__ unsigned long long red[32];
    const uint32_t n1 = 1u << g.log_n1;
    uint32_t ones = 0;
    for (uint32_t m1 = blockIdx.x; m1 < n1; m1 += gridDim.x) {
        for (int m2 = threadIdx.x; m2 < N2; m2 += NT) {
            uint64_t x = 2ull * ((uint64_t)m1 + ((uint64_t)m2 << g.log_n1));
            uint32_t b0, b1;
            if (SEED) seed_pair(bits, g, x, b0, b1);
            else key_pair(bits, g, x, b0, b1);
            ones += b0 + b1;
            sm[pad16(m2)] = make_float2((float)b0, (float)b1);
        }
        __syncthreads();
        fft_tile<N2, 1, NT, -1>(sm);
        float4* row = reinterpret_cast<float4*>(Y + ((size_t)m1 << g.log_n2));
        for (int p = threadIdx.x; p < N2 / 2; p += NT) {
            uint32_t k0 = (uint32_t)p, k1 = p ? (uint32_t)(N2 - p) : (uint32_t)(N2 / 2);
            float2 z0 = cmul(sm[pad16(k0)], tw_n(tw, m1 * k0));
            float2 z1 = cmul(sm[pad16(k1)], tw_n(tw, m1 * k1));
            row[p] = make_float4(z0.x, z0.y, z1.x, z1.y);
        }
        __syncthreads();
    }
    unsigned long long tot = block_sum(ones, red);
    if (threadIdx.x == 0 && tot) atomicAdd(cnt, tot);
}

// Pass B.  A tile is CPT columns (CPT/2 mirror pairs) x N1 rows.  Column c of tile t is pair
// p = t*CPT/2 + c/2, slot c&1: k2 = p (slot 0) or N2-p (slot 1); pair 0 holds k2 = 0 and N2/2.
template <int N1, int CPT>
__device__ __forceinline__ uint32_t tile_k2(int t, int c, uint32_t n2) {
    uint32_t p = (uint32_t)t * (CPT / 2) + (uint32_t)(c >> 1);
    if ((c & 1) == 0) return p;
    return p ? n2 - p : n2 / 2;
}

template <int N1, int CPT, int NT>
__device__ __forceinline__ void pass_b_load(const float2* __restrict__ Y, int t, uint32_t n2, float2* sm) {
    constexpr int SP = Padded<N1>::value;
    const float4* Y4 = reinterpret_cast<const float4*>(Y);
    for (int idx = threadIdx.x; idx < N1 * CPT / 2; idx += NT) {
        int m1 = idx / (CPT / 2), cp = idx % (CPT / 2);
        float4 v = __ldcs(Y4 + (((size_t)m1 * n2 + (size_t)t * CPT) >> 1) + cp);
        sm[(2 * cp) * SP + pad16(m1)] = make_float2(v.x, v.y);
        sm[(2 * cp + 1) * SP + pad16(m1)] = make_float2(v.z, v.w);
    }
}

// Visits every bin of the tile once as a mirror pair (k, N-k).  f(a_idx, b_idx, k) receives the
// smem indices of both bins (equal for self-mirrored bins, b_idx < 0 for the DC/Nyquist slot).
template <int N1, int CPT, int NT, class F>
__device__ __forceinline__ void pass_b_pairs(int t, uint32_t n2, F&& f) {
    constexpr int SP = Padded<N1>::value;
    for (int u = threadIdx.x; u < (CPT / 2) * N1; u += NT) {
        int pp = u / N1, k1 = u % N1;
        uint32_t p = (uint32_t)t * (CPT / 2) + (uint32_t)pp;
        int c0 = 2 * pp, c1 = 2 * pp + 1;
        if (p != 0) {
            f(c0 * SP + pad16(k1), c1 * SP + pad16(N1 - 1 - k1), p + n2 * (uint32_t)k1, (uint32_t)c0 * N1 + k1,
              (uint32_t)c1 * N1 + (N1 - 1 - k1));
        } else if (k1 < N1 / 2) {  // column k2 = 0: rows k1 <-> N1-k1
            if (k1 == 0) {
                f(c0 * SP, -1, 0u, (uint32_t)c0 * N1, 0u);
                f(c0 * SP + pad16(N1 / 2), c0 * SP + pad16(N1 / 2), n2 * (uint32_t)(N1 / 2),
                  (uint32_t)c0 * N1 + N1 / 2, (uint32_t)c0 * N1 + N1 / 2);
            } else {
                f(c0 * SP + pad16(k1), c0 * SP + pad16(N1 - k1), n2 * (uint32_t)k1, (uint32_t)c0 * N1 + k1,
                  (uint32_t)c0 * N1 + (N1 - k1));
            }
        } else {  // column k2 = N2/2: rows j <-> N1-1-j
            int j = k1 - N1 / 2;
            f(c1 * SP + pad16(j), c1 * SP + pad16(N1 - 1 - j), n2 / 2 + n2 * (uint32_t)j, (uint32_t)c1 * N1 + j,
              (uint32_t)c1 * N1 + (N1 - 1 - j));
        }
    }
}

template <int N1, int CPT, int NT>
__global__ void __launch_bounds__(NT) k_pass_b_seed(float2* __restrict__ Y, BlockGeom g, float2* __restrict__ spec) {
    extern __shared__ float2 sm[];
    const uint32_t n2 = 1u << g.log_n2;
    const int ntiles = (int)(n2 / CPT);
    const float sc = 1.0f / (float)(4ull << g.log_np);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        pass_b_load<N1, CPT, NT>(Y, t, n2, sm);
        __syncthreads();
        fft_tile<N1, CPT, NT, -1>(sm);
        float2* tspec = spec + (size_t)t * (CPT * N1);
        pass_b_pairs<N1, CPT, NT>(t, n2, [&](int ia, int ib, uint32_t k, uint32_t oa, uint32_t ob) {
            if (ib < 0) {
                float2 z = sm[ia];
                tspec[oa] = make_float2(2.0f * (z.x - z.y) * sc, 0.0f);
                return;
            }
            float2 xa, xb;
            real_split(sm[ia], sm[ib], expmi_pi(k, g.log_n), xa, xb);
            tspec[oa] = cscale(xa, sc);
            if (ib != ia) tspec[ob] = cscale(xb, sc);
        });
        __syncthreads();
    }
}

template <int N1, int CPT, int NT>
__global__ void __launch_bounds__(NT) k_pass_b_key(float2* __restrict__ Y, BlockGeom g,
                                                   const float2* __restrict__ spec, DeviceTables tw) {
    extern __shared__ float2 sm[];
    constexpr int SP = Padded<N1>::value;
    const uint32_t n2 = 1u << g.log_n2;
    const int ntiles = (int)(n2 / CPT);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        pass_b_load<N1, CPT, NT>(Y, t, n2, sm);
        __syncthreads();
        fft_tile<N1, CPT, NT, -1>(sm);
        const float2* tspec = spec + (size_t)t * (CPT * N1);
        pass_b_pairs<N1, CPT, NT>(t, n2, [&](int ia, int ib, uint32_t k, uint32_t oa, uint32_t ob) {
            if (ib < 0) {
                float2 z = sm[ia];
                float pn = 2.0f * (z.x - z.y) * __ldg(&tspec[oa].x);
                sm[ia] = make_float2(pn, -pn);
                return;
            }
            float2 w = expmi_pi(k, g.log_n);
            float2 xa, xb, qa, qb;
            real_split(sm[ia], sm[ib], w, xa, xb);
            float2 pa_ = cmul(xa, __ldg(tspec + oa)), pb_ = cmul(xb, __ldg(tspec + ob));
            real_merge(pa_, pb_, w, qa, qb);
            sm[ia] = qa;
            if (ib != ia) sm[ib] = qb;
        });
        __syncthreads();
        fft_tile<N1, CPT, NT, +1>(sm);
        float4* Y4 = reinterpret_cast<float4*>(Y);
        for (int idx = threadIdx.x; idx < N1 * CPT / 2; idx += NT) {
            int m1 = idx / (CPT / 2), cp = idx % (CPT / 2);
            uint32_t ka = tile_k2<N1, CPT>(t, 2 * cp, n2), kb = tile_k2<N1, CPT>(t, 2 * cp + 1, n2);
            float2 a = cmulconj(sm[(2 * cp) * SP + pad16(m1)], tw_n(tw, (uint32_t)m1 * ka));
            float2 b = cmulconj(sm[(2 * cp + 1) * SP + pad16(m1)], tw_n(tw, (uint32_t)m1 * kb));
            __stcs(Y4 + (((size_t)m1 * n2 + (size_t)t * CPT) >> 1) + cp, make_float4(a.x, a.y, b.x, b.y));
        }
        __syncthreads();
    }
}

// Pass C: inverse row FFT over k2 -> m2, then value + correction, rounding, parity.  Parities of
// row m1 go to two bit planes (even / odd real sample), bit m2 of plane row m1.
template <int N2, int NT>
__global__ void __launch_bounds__(NT) k_pass_c(const float2* __restrict__ Y, BlockGeom g,
                                               const unsigned long long* cnt, uint32_t* __restrict__ planes,
                                               unsigned int* resid_bits) {
    extern __shared__ float2 sm[];
    __shared__ float redf[32];
    const uint32_t n1 = 1u << g.log_n1;
    const float corr = correction(cnt, g.log_np);
    const size_t plane_words = (size_t)n1 * (N2 / 32);
    float res = 0.f;
    const int lane = threadIdx.x & 31;
    for (uint32_t m1 = blockIdx.x; m1 < n1; m1 += gridDim.x) {
        // rows whose first sample is past the output need no work
        if (2ull * m1 >= g.out_bits) {
            for (int w = threadIdx.x; w < N2 / 32; w += NT) {
                planes[(size_t)m1 * (N2 / 32) + w] = 0u;
                planes[plane_words + (size_t)m1 * (N2 / 32) + w] = 0u;
            }
            continue;
        }
        const float4* row = reinterpret_cast<const float4*>(Y + ((size_t)m1 << g.log_n2));
        for (int p = threadIdx.x; p < N2 / 2; p += NT) {
            float4 v = __ldcs(row + p);
            int k0 = p, k1 = p ? N2 - p : N2 / 2;
            sm[pad16(k0)] = make_float2(v.x, v.y);
            sm[pad16(k1)] = make_float2(v.z, v.w);
        }
        __syncthreads();
        fft_tile<N2, 1, NT, +1>(sm);
        for (int m2 = threadIdx.x; m2 < N2; m2 += NT) {
            float2 q = sm[pad16(m2)];
            uint64_t x0 = 2ull * ((uint64_t)m1 + ((uint64_t)m2 << g.log_n1));
            float v0 = q.x + corr, v1 = q.y + corr;
            float r0 = rintf(v0), r1 = rintf(v1);
            bool ok0 = x0 < g.out_bits, ok1 = x0 + 1 < g.out_bits;
            uint32_t b0 = ok0 ? ((uint32_t)(int)r0 & 1u) : 0u;
            uint32_t b1 = ok1 ? ((uint32_t)(int)r1 & 1u) : 0u;
            if (ok0) res = fmaxf(res, fabsf(v0 - r0));
            if (ok1) res = fmaxf(res, fabsf(v1 - r1));
            uint32_t be = __ballot_sync(0xffffffffu, b0), bo = __ballot_sync(0xffffffffu, b1);
            if (lane == 0) {
                planes[(size_t)m1 * (N2 / 32) + (m2 >> 5)] = be;
                planes[plane_words + (size_t)m1 * (N2 / 32) + (m2 >> 5)] = bo;
            }
        }
        __syncthreads();
    }
    float bm = block_max(res, redf);
    if (threadIdx.x == 0) atomicMax(resid_bits, __float_as_uint(bm));
}

// Bit planes -> output words.  Output word w covers samples m = 16w .. 16w+15, which share m2 and
// have consecutive m1.
__global__ void k_finish(const uint32_t* __restrict__ planes, BlockGeom g, const uint32_t* __restrict__ key_rest,
                         uint32_t flags, uint32_t* __restrict__ out_words, uint32_t nwords) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const size_t plane_words = (size_t)n1 * wpr;
    uint32_t m0 = 16u * w;
    uint32_t m1 = m0 & (n1 - 1u), m2 = m0 >> g.log_n1;
    uint32_t col = m2 >> 5, sh = m2 & 31u;
    uint32_t ev = 0, od = 0;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        size_t off = (size_t)(m1 + u) * wpr + col;
        ev |= ((__ldg(planes + off) >> sh) & 1u) << u;
        od |= ((__ldg(planes + plane_words + off) >> sh) & 1u) << u;
    }
    uint32_t kr = ((flags & PA_FLAG_XOR_KEY_REST) && 32u * w < g.v) ? __ldg(key_rest + w) : 0u;
    out_words[w] = out_word(ev, od, kr);
}

// ============================================================================ host launchers
template <class K>
static void set_smem(K kernel, size_t bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int launch_twiddle_tables(const BlockGeom& g, float2* glo, float2* ghi, cudaStream_t s) {
    uint32_t nhi = std::max<uint32_t>(1u, (1u << g.log_n) / 8192u);
    uint32_t tot = std::max<uint32_t>(8192u, nhi);
    k_twiddle_tables<<<(tot + 255) / 256, 256, 0, s>>>(g.log_n, glo, ghi, nhi);
    return (int)cudaGetLastError();
}

template <int N>
static constexpr int mono_threads() { return N >= 16384 ? 512 : (N / 16 < 32 ? 32 : N / 16); }

template <int N>
static int mono_seed(const BlockGeom& g, const uint32_t* seed, float2* spec, unsigned long long* cnt_seed,
                     cudaStream_t s) {
    constexpr int NT = mono_threads<N>();
    size_t smem = (size_t)Padded<N>::value * sizeof(float2);
    set_smem(k_mono_seed<N, NT>, smem);
    k_mono_seed<N, NT><<<1, NT, smem, s>>>(seed, g, spec, cnt_seed);
    return (int)cudaGetLastError();
}

template <int N>
static int mono_key(const BlockGeom& g, const uint32_t* ks, const uint32_t* kr, uint32_t flags, const float2* spec,
                    unsigned long long* cnt, unsigned int* resid, uint32_t* out, cudaStream_t s) {
    constexpr int NT = mono_threads<N>();
    size_t smem = (size_t)Padded<N>::value * sizeof(float2);
    set_smem(k_mono_key<N, NT>, smem);
    k_mono_key<N, NT><<<1, NT, smem, s>>>(ks, kr, g, flags, spec, cnt, resid, out);
    return (int)cudaGetLastError();
}

template <int N2>
static constexpr int row_threads() { return N2 / 32 < 32 ? 32 : (N2 / 32 > 512 ? 512 : N2 / 32); }

static int grid_for(uint32_t units, int num_sms) {
    return (int)std::max<uint32_t>(1u, std::min<uint32_t>(units, (uint32_t)num_sms));
}

template <int N2>
static int pass_a(const BlockGeom& g, const uint32_t* bits, bool seed, DeviceTables tw, float2* Y,
                  unsigned long long* cnt, int num_sms, cudaStream_t s) {
    constexpr int NT = row_threads<N2>();
    size_t smem = (size_t)Padded<N2>::value * sizeof(float2);
    int grid = grid_for(1u << g.log_n1, num_sms);
    if (seed) {
        set_smem(k_pass_a<N2, NT, true>, smem);
        k_pass_a<N2, NT, true><<<grid, NT, smem, s>>>(bits, g, tw, Y, cnt);
    } else {
        set_smem(k_pass_a<N2, NT, false>, smem);
        k_pass_a<N2, NT, false><<<grid, NT, smem, s>>>(bits, g, tw, Y, cnt);
    }
    return (int)cudaGetLastError();
}

template <int N2>
static int pass_c(const BlockGeom& g, const float2* Y, const unsigned long long* cnt, uint32_t* planes,
                  unsigned int* resid, int num_sms, cudaStream_t s) {
    constexpr int NT = row_threads<N2>();
    size_t smem = (size_t)Padded<N2>::value * sizeof(float2);
    set_smem(k_pass_c<N2, NT>, smem);
    k_pass_c<N2, NT><<<grid_for(1u << g.log_n1, num_sms), NT, smem, s>>>(Y, g, cnt, planes, resid);
    return (int)cudaGetLastError();
}

template <int N1>
static int pass_b(const BlockGeom& g, bool seed, float2* Y, float2* spec, DeviceTables tw, int num_sms,
                  cudaStream_t s) {
    constexpr int CPT = 16384 / N1;
    constexpr int NT = 512;
    size_t smem = (size_t)CPT * Padded<N1>::value * sizeof(float2);
    int grid = grid_for((1u << g.log_n2) / CPT, num_sms);
    if (seed) {
        set_smem(k_pass_b_seed<N1, CPT, NT>, smem);
        k_pass_b_seed<N1, CPT, NT><<<grid, NT, smem, s>>>(Y, g, spec);
    } else {
        set_smem(k_pass_b_key<N1, CPT, NT>, smem);
        k_pass_b_key<N1, CPT, NT><<<grid, NT, smem, s>>>(Y, g, spec, tw);
    }
    return (int)cudaGetLastError();
}

#define PA_DISPATCH_MONO(L, CALL)          \
    switch (L) {                           \
        case 9: return CALL(512);          \
        case 10: return CALL(1024);        \
        case 11: return CALL(2048);        \
        case 12: return CALL(4096);        \
        case 13: return CALL(8192);        \
        case 14: return CALL(16384);       \
        default: return (int)cudaErrorInvalidValue; \
    }

#define PA_DISPATCH_N1(L, CALL)            \
    switch (L) {                           \
        case 6: return CALL(64);           \
        case 7: return CALL(128);          \
        case 8: return CALL(256);          \
        case 9: return CALL(512);          \
        case 10: return CALL(1024);        \
        case 11: return CALL(2048);        \
        case 12: return CALL(4096);        \
        default: return (int)cudaErrorInvalidValue; \
    }

int launch_seed_spectrum(const BlockGeom& g, const uint32_t* seed, float2* spec, float2* work,
                         unsigned long long* cnt_seed, DeviceTables tw, cudaStream_t s) {
    if (g.log_n1 == 0) {
#define C(NN) mono_seed<NN>(g, seed, spec, cnt_seed, s)
        PA_DISPATCH_MONO(g.log_n, C)
#undef C
    }
    int num_sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaMemsetAsync(cnt_seed, 0, sizeof(unsigned long long), s);
    int rc;
#define C(NN) pass_a<NN>(g, seed, true, tw, work, cnt_seed, num_sms, s)
    rc = [&]() -> int { PA_DISPATCH_MONO(g.log_n2, C) }();
#undef C
    if (rc) return rc;
#define C(NN) pass_b<NN>(g, true, work, spec, tw, num_sms, s)
    PA_DISPATCH_N1(g.log_n1, C)
#undef C
}

int launch_key_block(const BlockGeom& g, const uint32_t* key_start, const uint32_t* key_rest, uint32_t flags,
                     const float2* spec, float2* work, uint32_t* planes, unsigned long long* cnt,
                     unsigned int* resid_bits, uint32_t* out_words, DeviceTables tw, int num_sms, cudaStream_t s,
                     cudaEvent_t* ev) {
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], s);
    };
    cudaMemsetAsync(resid_bits, 0, sizeof(unsigned int), s);
    if (g.log_n1 == 0) {
        mark(0);
        int rc;
#define C(NN) mono_key<NN>(g, key_start, key_rest, flags, spec, cnt, resid_bits, out_words, s)
        rc = [&]() -> int { PA_DISPATCH_MONO(g.log_n, C) }();
#undef C
        mark(1);
        return rc;
    }
    cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s);  // key popcount; cnt[1] is the seed's
    int rc;
    mark(0);
#define C(NN) pass_a<NN>(g, key_start, false, tw, work, cnt, num_sms, s)
    rc = [&]() -> int { PA_DISPATCH_MONO(g.log_n2, C) }();
#undef C
    if (rc) return rc;
    mark(1);
#define C(NN) pass_b<NN>(g, false, work, const_cast<float2*>(spec), tw, num_sms, s)
    rc = [&]() -> int { PA_DISPATCH_N1(g.log_n1, C) }();
#undef C
    if (rc) return rc;
    mark(2);
#define C(NN) pass_c<NN>(g, work, cnt, planes, resid_bits, num_sms, s)
    rc = [&]() -> int { PA_DISPATCH_MONO(g.log_n2, C) }();
#undef C
    if (rc) return rc;
    mark(3);
    uint32_t nwords = (g.out_bits + 31u) / 32u;
    k_finish<<<(nwords + 255) / 256, 256, 0, s>>>(planes, g, key_rest, flags, out_words, nwords);
    mark(4);
    return (int)cudaGetLastError();
}

int kernel_count_key_block(const BlockGeom& g) { return g.log_n1 == 0 ? 1 : 4; }

}  // namespace pa
