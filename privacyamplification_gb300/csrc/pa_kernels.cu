// pa_kernels.cu -- sm_103a kernels of the privacy-amplification hot path.
//
// Replaces, for one block, the reference's launch sequence (PrivacyAmplification.cu:1797-2042):
// binInt2float x2, calculateCorrectionFloat, cufftExecR2C x2, setFirstElementToZero,
// ElementWiseProduct, cufftExecC2R, ToBinaryArray[NoXOR] -- with no cuFFT and no float staging arrays.
//
// Two shapes:
//   * single-CTA ("mono") path, N = Np/2 <= 2^14 complex samples: the whole convolution of one block
//     in shared memory, bits in, packed bytes out;
//   * three-pass four-step path, N = N1 * N2 (N2 <= 2^14, N1 <= 2^12), kernels in pa_passes.cu:
//       bit rows  key bits -> per-row bit planes
//       pass A    row FFTs over m2 (length N2), 4-step twiddle, write Y
//       pass B    column FFTs over m1 (length N1), real split, spectral product with the cached seed
//                 spectrum (DC removed), real merge, inverse column FFTs, inverse twiddle, write Y
//       pass C    inverse row FFTs, + correction, round, parity -> bit planes
//       finish    bit planes -> reference byte order, XOR key_rest
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

// A group (gp.e set): block blockIdx.x of the group, its seed and popcount from its entry, its spectrum at
// spec + blockIdx.x * gp.work.
template <int N, int NT>
__global__ void __launch_bounds__(NT) k_mono_seed(const uint32_t* __restrict__ seed, BlockGeom g,
                                                  float2* __restrict__ spec, unsigned long long* cnt_seed, Group gp) {
    extern __shared__ float2 sm[];
    __shared__ unsigned long long red[32];
    if (gp.e) {
        seed = gp.e[blockIdx.x].seed;
        spec += (size_t)blockIdx.x * gp.work;
        cnt_seed = gp.e[blockIdx.x].cnt + 1;
    }
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

// A group (gp.e set): block blockIdx.x of the group, everything it reads and writes from its entry.
template <int N, int NT>
__global__ void __launch_bounds__(NT) k_mono_key(const uint32_t* __restrict__ key_start,
                                                 const uint32_t* __restrict__ key_rest, BlockGeom g, uint32_t flags,
                                                 const float2* __restrict__ spec, unsigned long long* cnt,
                                                 unsigned int* resid_bits, uint32_t* __restrict__ out_words, Group gp) {
    extern __shared__ float2 sm[];
    __shared__ unsigned long long red[32];
    __shared__ float redf[32];
    __shared__ float s_corr;
    if (gp.e) {
        const GroupEntry& en = gp.e[blockIdx.x];
        key_start = en.key_start;
        key_rest = en.key_rest;
        spec = en.spec;
        cnt = en.cnt;
        resid_bits = en.resid;
        out_words = en.out;
    }
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

// ============================================================================ host launchers
template <class K>
static void set_smem(K kernel, size_t bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int N>
static constexpr int mono_threads() { return N >= 16384 ? 512 : (N / 16 < 32 ? 32 : N / 16); }

template <int N>
static int mono_seed(const BlockGeom& g, const uint32_t* seed, float2* spec, unsigned long long* cnt_seed,
                     cudaStream_t s, const Group& gp = kOneBlock) {
    constexpr int NT = mono_threads<N>();
    size_t smem = (size_t)Padded<N>::value * sizeof(float2);
    set_smem(k_mono_seed<N, NT>, smem);
    k_mono_seed<N, NT><<<gp.count, NT, smem, s>>>(seed, g, spec, cnt_seed, gp);
    return (int)cudaGetLastError();
}

template <int N>
static int mono_key(const BlockGeom& g, const uint32_t* ks, const uint32_t* kr, uint32_t flags, const float2* spec,
                    unsigned long long* cnt, unsigned int* resid, uint32_t* out, cudaStream_t s,
                    const Group& gp = kOneBlock) {
    constexpr int NT = mono_threads<N>();
    size_t smem = (size_t)Padded<N>::value * sizeof(float2);
    set_smem(k_mono_key<N, NT>, smem);
    k_mono_key<N, NT><<<gp.count, NT, smem, s>>>(ks, kr, g, flags, spec, cnt, resid, out, gp);
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

int launch_seed_spectrum(const BlockGeom& g, const uint32_t* seed, float2* spec, const Scratch& sc,
                         unsigned long long* cnt_seed, int num_sms, cudaStream_t s) {
    if (g.log_n1 == 0) {
#define C(NN) mono_seed<NN>(g, seed, spec, cnt_seed, s)
        PA_DISPATCH_MONO(g.log_n, C)
#undef C
    }
    cudaMemsetAsync(cnt_seed, 0, sizeof(unsigned long long), s);
    int rc = launch_bit_rows(g, seed, true, sc.planes, s);
    if (!rc) rc = launch_pass_a(g, sc.planes, true, sc.work, cnt_seed, num_sms, s);
    if (!rc) rc = launch_pass_b(g, true, *sc.maps, sc.work, sc.work2, spec, sc.err, num_sms, s);
    return rc;
}

int launch_key_block(const BlockGeom& g, const uint32_t* key_start, const uint32_t* key_rest, uint32_t flags,
                     const float2* spec, const Scratch& sc, unsigned long long* cnt, unsigned int* resid_bits,
                     uint32_t* out_words, int num_sms, cudaStream_t s, cudaEvent_t* ev, cudaEvent_t key_rest_ready) {
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], s);
    };
    cudaMemsetAsync(resid_bits, 0, sizeof(unsigned int), s);
    if (g.log_n1 == 0) {
        if (key_rest_ready) cudaStreamWaitEvent(s, key_rest_ready, 0);
        mark(0);
        int rc;
#define C(NN) mono_key<NN>(g, key_start, key_rest, flags, spec, cnt, resid_bits, out_words, s)
        rc = [&]() -> int { PA_DISPATCH_MONO(g.log_n, C) }();
#undef C
        mark(1);
        return rc;
    }
    cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s);  // key popcount; cnt[1] is the seed's
    mark(0);
    int rc = launch_bit_rows(g, key_start, false, sc.planes, s);
    if (!rc) rc = launch_pass_a(g, sc.planes, false, sc.work, cnt, num_sms, s);
    mark(1);
    if (!rc) rc = launch_pass_b(g, false, *sc.maps, sc.work, sc.work2, const_cast<float2*>(spec), sc.err, num_sms, s);
    mark(2);
    if (!rc) rc = launch_pass_c(g, *sc.maps, sc.work2, cnt, sc.planes, resid_bits, sc.err, num_sms, s);
    mark(3);
    if (!rc && key_rest_ready) rc = (int)cudaStreamWaitEvent(s, key_rest_ready, 0);  // key_rest copied meanwhile
    if (!rc) rc = launch_finish(g, sc.planes, key_rest, flags, out_words, s);
    mark(4);
    return rc;
}

int launch_fused_block(const BlockGeom& g, const uint32_t* seed, const uint32_t* key_start, const uint32_t* key_rest,
                       uint32_t flags, float2* seed_y, const PassMaps& seed_maps, float2* park, uint32_t park_ctas,
                       const Scratch& sc, unsigned long long* cnt, unsigned int* resid_bits, uint32_t* out_words,
                       int num_sms, cudaStream_t s, cudaEvent_t* ev, cudaEvent_t key_rest_ready) {
    if (!fused_geom(g)) return (int)cudaErrorInvalidValue;
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], s);
    };
    cudaMemsetAsync(resid_bits, 0, sizeof(unsigned int), s);
    cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), s);  // key and seed popcounts
    mark(0);
    int rc = launch_bit_rows(g, seed, true, sc.planes, s);
    if (!rc) rc = launch_pass_a(g, sc.planes, true, seed_y, cnt + 1, num_sms, s);
    if (!rc) rc = launch_bit_rows(g, key_start, false, sc.planes, s);
    if (!rc) rc = launch_pass_a(g, sc.planes, false, sc.work, cnt, num_sms, s);
    mark(1);
    if (!rc) rc = launch_pass_b_fused(g, seed_maps, *sc.maps, sc.work2, park, park_ctas, sc.err, num_sms, s);
    mark(2);
    if (!rc) rc = launch_pass_c(g, *sc.maps, sc.work2, cnt, sc.planes, resid_bits, sc.err, num_sms, s);
    mark(3);
    if (!rc && key_rest_ready) rc = (int)cudaStreamWaitEvent(s, key_rest_ready, 0);  // key_rest copied meanwhile
    if (!rc) rc = launch_finish(g, sc.planes, key_rest, flags, out_words, s);
    mark(4);
    return rc;
}

// A group of single-CTA blocks: one CTA per block, one launch for the group.
int launch_group_mono_seed(const BlockGeom& g, const Group& gp, float2* spec, cudaStream_t s) {
    if (!gp.e) return (int)cudaErrorInvalidValue;
#define C(NN) mono_seed<NN>(g, nullptr, spec, nullptr, s, gp)
    PA_DISPATCH_MONO(g.log_n, C)
#undef C
}

int launch_group_mono_key(const BlockGeom& g, const Group& gp, uint32_t flags, cudaStream_t s) {
    if (!gp.e) return (int)cudaErrorInvalidValue;
#define C(NN) mono_key<NN>(g, nullptr, nullptr, flags, nullptr, nullptr, nullptr, nullptr, s, gp)
    PA_DISPATCH_MONO(g.log_n, C)
#undef C
}

int kernel_count_key_block(const BlockGeom& g) { return g.log_n1 == 0 ? 1 : 5; }
int stage_count_key_block(const BlockGeom& g) { return g.log_n1 == 0 ? 1 : 4; }

}  // namespace pa
