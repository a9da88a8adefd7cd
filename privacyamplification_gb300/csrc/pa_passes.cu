// pa_passes.cu -- the three-pass four-step FP32 convolution for N = N1 * N2 complex samples.
//
// Data layout in HBM for one block (n = 2^27: N1 = 2^12, N2 = 2^14):
//   rows     bit planes, row m1 holds the 2*N2 sample bits x = 2(m1 + N1*m2) + t, 16 m2 per word,
//            MSB first (n/8 bytes)                                  -- k_bit_rows
//   Y        N complex64, row m1 = N2 values in "pair" order: float4 p holds columns p and N2-p
//            (p = 0 holds 0 and N2/2)                               -- pass A writes, pass B rewrites
//   spec     N complex64, the seed's real spectrum / (2 Np) in the thread order of pass B
//   planes   parity bits, [t][m1][N2/32 words], bit m2 of row m1 -- pass C writes
//   out      v/8 bytes in the reference byte order                  -- k_finish
// Each pass is one persistent CTA per SM walking rows (A, C) or column tiles (B); the FFT data stay
// in registers (32 complex per thread) and meet in shared memory only between radix stages.
#include "pa_device.cuh"
#include "pa_fft.cuh"
#include "pa_kernels.cuh"

#include <algorithm>

namespace pa {

namespace {

constexpr uint32_t kXor = 1u;  // PA_FLAG_XOR_KEY_REST

__device__ __forceinline__ uint32_t spread16p(uint32_t x) {
    x &= 0xFFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

// MSB-first word from 16 (even, odd) bit pairs: pair u at bits 31-2u (even) and 30-2u (odd).
__device__ __forceinline__ uint32_t msb_pairs(uint32_t even16, uint32_t odd16) {
    return __brev(spread16p(even16) | (spread16p(odd16) << 1));
}

__device__ __forceinline__ unsigned long long block_sum_ull(unsigned long long v, unsigned long long* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    return t;
}

__device__ __forceinline__ float block_max_f(float v, float* red) {
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

__device__ __forceinline__ uint32_t load_bit(const uint32_t* __restrict__ w, uint64_t x) {
    return (__ldg(w + (x >> 5)) >> (31u - (uint32_t)(x & 31u))) & 1u;
}

}  // namespace

// ============================================================================ input bit planes
// Warp (a, c): rows m1 = 16a .. 16a+15, columns m2 = 32c .. 32c+31 (lane = m2 - 32c).  The lane's
// input word holds the 32 bits x = 2 N1 m2 + 32a + [0, 32) = bit pairs of rows 16a..16a+15.
template <bool SEED>
__global__ void __launch_bounds__(256) k_bit_rows(const uint32_t* __restrict__ src, BlockGeom g,
                                                  uint32_t* __restrict__ rows) {
    const int lane = threadIdx.x & 31;
    const uint32_t n1 = 1u << g.log_n1, n2 = 1u << g.log_n2;
    const uint32_t a = blockIdx.x * 8u + (threadIdx.x >> 5);  // 16-row group
    const uint32_t c = blockIdx.y;                             // 32-column group
    if (a >= n1 / 16u) return;
    const uint32_t m2 = 32u * c + (uint32_t)lane;
    const uint64_t x0 = 2ull * n1 * m2 + 32ull * a;
    uint32_t v;
    if (!SEED) {
        if (x0 + 31 <= g.h) v = __ldg(src + (x0 >> 5));
        else if (x0 > g.h) v = 0u;
        else v = __ldg(src + (x0 >> 5)) & ~(0xFFFFFFFFu >> (uint32_t)(g.h - x0 + 1));
    } else if ((1u << g.log_np) == g.n) {
        v = __ldg(src + (x0 >> 5));
    } else {
        v = 0u;
        for (int b = 0; b < 32; ++b) {
            uint64_t s;
            if (seed_source(g, x0 + b, &s)) v |= load_bit(src, s) << (31 - b);
        }
    }
    uint32_t mine = 0;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        uint32_t e = __ballot_sync(0xffffffffu, (v >> (31 - 2 * u)) & 1u);
        uint32_t o = __ballot_sync(0xffffffffu, (v >> (30 - 2 * u)) & 1u);
        if ((lane >> 1) == u) mine = (lane & 1) ? msb_pairs(e >> 16, o >> 16) : msb_pairs(e, o);
    }
    const uint32_t row = 16u * a + (uint32_t)(lane >> 1);
    rows[(size_t)row * (n2 / 16u) + 2u * c + (uint32_t)(lane & 1)] = mine;
}

// ============================================================================ pass A
// Row m1: FFT over m2 of the 2N2 bits of the row, 4-step twiddle W_N^{m1 k2}, pair-order store.
template <int LOGL, bool SEED>
__global__ void __launch_bounds__((1 << LOGL) / 32, 1)
    k_pass_a(const uint32_t* __restrict__ rows, BlockGeom g, float2* __restrict__ Y, unsigned long long* cnt) {
    constexpr int L = 1 << LOGL, NT = L / 32, E = 32, LR = L / 16;
    using P = Plan<LOGL>;
    using Lin = MapLinear<NT>;
    extern __shared__ float2 sm[];
    __shared__ float2 rho[16];
    __shared__ uint32_t bits[L / 16];
    __shared__ unsigned long long red[32];
    const uint32_t n1 = 1u << g.log_n1;
    const int t = threadIdx.x;
    uint32_t ones = 0;
    for (uint32_t m1 = blockIdx.x; m1 < n1; m1 += gridDim.x) {
        __syncthreads();  // previous row done with bits / rho / sm
        const uint32_t* rw = rows + (size_t)m1 * (L / 16);
        for (int i = t; i < L / 16; i += NT) {
            uint32_t w = __ldg(rw + i);
            bits[i] = w;
            ones += __popc(w);
        }
        if (t < 16) rho[t] = expmi_pi((uint32_t)((2ull * m1 * LR * (uint64_t)t) & ((2ull << g.log_n) - 1)), g.log_n);
        __syncthreads();
        float2 x[E];
        // first stage inputs: butterfly u = t + q*NT, element m2 = u + r*(L/RA)
#pragma unroll
        for (int q = 0; q < E / P::RA; ++q) {
            const int j = t + q * NT;
#pragma unroll
            for (int r = 0; r < P::RA; ++r) {
                const int m2 = j + r * (L / P::RA);
                const uint32_t w = bits[m2 >> 4];
                const int sh = 30 - 2 * (m2 & 15);
                x[q * P::RA + r] = make_float2((float)((w >> (sh + 1)) & 1u), (float)((w >> sh) & 1u));
            }
        }
        stage<L, P::RA, 1, -1, E, Lin>(x);
        if (P::NSTAGE == 2) {
            exchange<L, E, P::RA, 1, Lin, P::RB, Lin>(x, sm);
            stage<L, P::RB, P::RA, -1, E, Lin>(x);
            exchange<L, E, P::RB, P::RA, Lin, 16, MapMirrorRow>(x, sm);
        } else {
            exchange<L, E, P::RA, 1, Lin, 16, MapMirrorRow>(x, sm);
        }
        // mirror stage (NS = L/16) with the 4-step twiddle W_N^{m1 (j + LR r)} folded in:
        // W_N^{m1 j} on the inputs, rho[r] = W_N^{m1 LR r} on the outputs.
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int seq, j;
            MapMirrorRow::at<L, 16>(q, seq, j);
            float2 c = expmi_pi(2u * m1 * (uint32_t)j, g.log_n);
            twiddle_powers<16, true>(&x[16 * q], unit_root<-1>(j, L), c);
            dft<16, -1>(reinterpret_cast<float2(&)[16]>(x[16 * q]));
#pragma unroll
            for (int r = 0; r < 16; ++r) x[16 * q + r] = cmul(x[16 * q + r], rho[r]);
        }
        float4* row4 = reinterpret_cast<float4*>(Y + ((size_t)m1 << LOGL));
        if (t != 0) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float2 a0 = x[r], a1 = x[16 + 15 - r], b0 = x[16 + r], b1 = x[15 - r];
                __stcg(row4 + t + LR * r, make_float4(a0.x, a0.y, a1.x, a1.y));
                __stcg(row4 + (LR - t) + LR * r, make_float4(b0.x, b0.y, b1.x, b1.y));
            }
        } else {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float2 a0 = x[r], a1 = r == 0 ? x[8] : x[16 - r], b0 = x[16 + r], b1 = x[16 + 15 - r];
                __stcg(row4 + LR * r, make_float4(a0.x, a0.y, a1.x, a1.y));
                __stcg(row4 + LR / 2 + LR * r, make_float4(b0.x, b0.y, b1.x, b1.y));
            }
        }
    }
    unsigned long long tot = block_sum_ull(ones, red);
    if (threadIdx.x == 0 && tot) atomicAdd(cnt, tot);
}

// ============================================================================ pass B
// Tile t: CPT columns (CPT/2 mirror pairs) x N1 rows.  Column c of tile t: pair p = t*CPT/2 + c/2,
// k2 = p (c even) or N2 - p (c odd); pair 0 holds k2 = 0 and N2/2.
__device__ __forceinline__ uint32_t col_k2(uint32_t p, int slot, uint32_t n2) {
    if (slot == 0) return p;
    return p ? n2 - p : n2 / 2;
}

// Index of bin (column c, row k1) in the thread-order spectrum of one tile (layout [c][r][jj]):
// the mirror-pair stage gives column 2pp+q, butterfly j, output r the bin k1 = j + LR r, with
// j = jj (q = 0) or LR-1-jj (q = 1).
template <int LR>
__device__ __forceinline__ int spec_index(int c, int k1) {
    int r = k1 / LR, j = k1 % LR;
    int jj = (c & 1) ? LR - 1 - j : j;
    return (c * 16 + r) * LR + jj;
}

template <int LOGL, bool SEED>
__global__ void __launch_bounds__(512, 1)
    k_pass_b(float2* __restrict__ Y, BlockGeom g, float2* __restrict__ spec) {
    constexpr int L = 1 << LOGL, NT = 512, E = 32, CPT = 16384 / L, LR = L / 16, SP = Padded<L>::value;
    constexpr int RL = Plan<LOGL>::RA;  // radix of the last inverse stage
    using P = Plan<LOGL>;
    using Lin = MapLinear<NT>;
    extern __shared__ float2 sm[];
    float2* sigma = sm + CPT * SP;  // [CPT][RL] output twists of the last inverse stage
    const uint32_t n2 = 1u << g.log_n2;
    const int ntiles = (int)(n2 / CPT);
    const int t = threadIdx.x;
    const int pp = t / LR, jj = t % LR;
    const float sc = 1.0f / (float)(4ull << g.log_np);  // seed spectrum scale 2X/(4Np)
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        __syncthreads();  // previous tile done with sm
        {   // coalesced load of the tile: row m1, pair cp -> columns 2cp, 2cp+1
            const float4* Y4 = reinterpret_cast<const float4*>(Y);
            for (int idx = t; idx < L * CPT / 2; idx += NT) {
                int m1 = idx / (CPT / 2), cp = idx % (CPT / 2);
                float4 v = __ldcs(Y4 + (((size_t)m1 * n2 + (size_t)tile * CPT) >> 1) + cp);
                sm[(2 * cp) * SP + pad16(m1)] = make_float2(v.x, v.y);
                sm[(2 * cp + 1) * SP + pad16(m1)] = make_float2(v.z, v.w);
            }
        }
        if (!SEED) {
            for (int i = t; i < CPT * RL; i += NT) {
                int c = i / RL, r = i % RL;
                uint32_t k2 = col_k2((uint32_t)tile * (CPT / 2) + (uint32_t)(c >> 1), c & 1, n2);
                uint64_t e = ((uint64_t)(L / RL) * (uint64_t)r * k2) & ((1ull << g.log_n) - 1);
                sigma[i] = cconj(expmi_pi((uint32_t)(2 * e), g.log_n));
            }
        }
        __syncthreads();
        float2 x[E];
        gather_inputs<L, E, P::RA, Lin>(x, sm);
        stage<L, P::RA, 1, -1, E, Lin>(x);
        if (P::NSTAGE == 2) {
            exchange<L, E, P::RA, 1, Lin, P::RB, Lin>(x, sm);
            stage<L, P::RB, P::RA, -1, E, Lin>(x);
            exchange<L, E, P::RB, P::RA, Lin, 16, MapMirrorPair>(x, sm);
        } else {
            exchange<L, E, P::RA, 1, Lin, 16, MapMirrorPair>(x, sm);
        }
        stage<L, 16, LR, -1, E, MapMirrorPair>(x);

        // ---- spectral step: real split, product with the seed spectrum, real merge
        float2* tspec = spec + (size_t)tile * (CPT * L);
        const bool special = tile == 0;  // pair 0 holds the self-mirrored columns 0 and N2/2
        if (special) {
            __syncthreads();
            if (pp == 0) {
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    int seq, j;
                    MapMirrorPair::at<L, 16>(q, seq, j);
#pragma unroll
                    for (int r = 0; r < 16; ++r) sm[seq * SP + pad16(j + LR * r)] = x[16 * q + r];
                }
            }
            __syncthreads();
            if (pp == 0) {
                for (int u = jj; u < L; u += LR) {
                    int ca, ka, cb, kb;
                    uint32_t k;
                    if (u < L / 2) {  // column k2 = 0, rows u <-> L-u
                        ca = cb = 0;
                        ka = u;
                        kb = u ? L - u : L / 2;
                        k = n2 * (uint32_t)ka;
                    } else {  // column k2 = N2/2, rows j <-> L-1-j
                        ca = cb = 1;
                        ka = u - L / 2;
                        kb = L - 1 - ka;
                        k = n2 / 2 + n2 * (uint32_t)ka;
                    }
                    if (u == 0) {  // DC (dropped) and Nyquist in slot (0, 0); then the self pair N/2
                        float2 z = sm[pad16(0)];
                        float nyq = 2.0f * (z.x - z.y);
                        if (SEED) {
                            tspec[spec_index<LR>(0, 0)] = make_float2(nyq * sc, 0.f);
                        } else {
                            float pn = nyq * tspec[spec_index<LR>(0, 0)].x;
                            sm[pad16(0)] = make_float2(pn, -pn);
                        }
                        ka = kb = L / 2;
                        k = n2 * (uint32_t)(L / 2);
                    }
                    float2 w = expmi_pi(k, g.log_n);
                    float2 za = sm[ca * SP + pad16(ka)], zb = sm[cb * SP + pad16(kb)];
                    float2 xa, xb;
                    real_split(za, zb, w, xa, xb);
                    int ia = spec_index<LR>(ca, ka), ib = spec_index<LR>(cb, kb);
                    if (SEED) {
                        tspec[ia] = cscale(xa, sc);
                        tspec[ib] = cscale(xb, sc);
                    } else {
                        float2 qa, qb;
                        real_merge(cmul(xa, tspec[ia]), cmul(xb, tspec[ib]), w, qa, qb);
                        sm[ca * SP + pad16(ka)] = qa;
                        sm[cb * SP + pad16(kb)] = qb;
                    }
                }
            }
            __syncthreads();
            if (pp == 0 && !SEED) {
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    int seq, j;
                    MapMirrorPair::at<L, 16>(q, seq, j);
#pragma unroll
                    for (int r = 0; r < 16; ++r) x[16 * q + r] = sm[seq * SP + pad16(j + LR * r)];
                }
            }
        }
        if (!special || pp != 0) {
            // bins (k1 = jj + LR r, k2 = p) and (L-1-k1, N2-p): x[r] and x[16 + 15 - r];
            // W_2N^{p + N2 (jj + LR r)} = W_2N^{p + N2 jj} * W_32^r
            const uint32_t p = (uint32_t)tile * (CPT / 2) + (uint32_t)pp;
            const float2 base = expmi_pi(p + n2 * (uint32_t)jj, g.log_n);
            const int ia0 = (2 * pp) * 16 * LR + jj, ib0 = (2 * pp + 1) * 16 * LR + jj;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                // W_32^r = e^{-i pi r/16} = (cos, -sin)(2 pi r/32), r < 16
                const float2 w = r ? cmul(base, make_float2(w32(r).x, -w32(r).y)) : base;
                float2 xa, xb;
                real_split(x[r], x[16 + 15 - r], w, xa, xb);
                const int ia = ia0 + r * LR, ib = ib0 + (15 - r) * LR;
                if (SEED) {
                    __stcs(tspec + ia, cscale(xa, sc));
                    __stcs(tspec + ib, cscale(xb, sc));
                } else {
                    float2 qa, qb;
                    real_merge(cmul(xa, __ldcs(tspec + ia)), cmul(xb, __ldcs(tspec + ib)), w, qa, qb);
                    x[r] = qa;
                    x[16 + 15 - r] = qb;
                }
            }
        }
        if (SEED) continue;

        // ---- inverse column FFTs (radices 16, RB, RA) with the inverse 4-step twiddle folded into
        // the last stage: conj(W_N^{m1 k2}), m1 = j + (L/RL) r
        stage<L, 16, 1, +1, E, MapMirrorPair>(x);
        if (P::NSTAGE == 2) {
            exchange<L, E, 16, 1, MapMirrorPair, P::RB, Lin>(x, sm);
            stage<L, P::RB, 16, +1, E, Lin>(x);
            exchange<L, E, P::RB, 16, Lin, P::RA, Lin>(x, sm);
        } else {
            exchange<L, E, 16, 1, MapMirrorPair, P::RA, Lin>(x, sm);
        }
        constexpr int NSL = L / RL;
#pragma unroll
        for (int q = 0; q < E / RL; ++q) {
            int seq, j;
            Lin::at<L, RL>(q, seq, j);
            uint32_t k2 = col_k2((uint32_t)tile * (CPT / 2) + (uint32_t)(seq >> 1), seq & 1, n2);
            uint64_t e = ((uint64_t)j * k2) & ((1ull << g.log_n) - 1);
            float2 c = cconj(expmi_pi((uint32_t)(2 * e), g.log_n));
            if (NSL > 1) twiddle_powers<RL, true>(&x[q * RL], unit_root<+1>(j % NSL, NSL * RL), c);
            else {
#pragma unroll
                for (int r = 0; r < RL; ++r) x[q * RL + r] = cmul(x[q * RL + r], c);
            }
            dft<RL, +1>(reinterpret_cast<float2(&)[RL]>(x[q * RL]));
#pragma unroll
            for (int r = 0; r < RL; ++r) x[q * RL + r] = cmul(x[q * RL + r], sigma[seq * RL + r]);
        }
        __syncthreads();
        scatter_outputs<L, E, RL, Lin>(x, sm);
        __syncthreads();
        {
            float4* Y4 = reinterpret_cast<float4*>(Y);
            for (int idx = t; idx < L * CPT / 2; idx += NT) {
                int m1 = idx / (CPT / 2), cp = idx % (CPT / 2);
                float2 a = sm[(2 * cp) * SP + pad16(m1)], b = sm[(2 * cp + 1) * SP + pad16(m1)];
                __stcg(Y4 + (((size_t)m1 * n2 + (size_t)tile * CPT) >> 1) + cp, make_float4(a.x, a.y, b.x, b.y));
            }
        }
    }
}

// ============================================================================ pass C
// Row m1: inverse FFT over k2 (radices 16, RB, RA), + correction, round, parity bit planes.
template <int LOGL>
__global__ void __launch_bounds__((1 << LOGL) / 32, 1)
    k_pass_c(const float2* __restrict__ Y, BlockGeom g, const unsigned long long* cnt,
             uint32_t* __restrict__ planes, unsigned int* resid_bits) {
    constexpr int L = 1 << LOGL, NT = L / 32, E = 32, LR = L / 16;
    using P = Plan<LOGL>;
    using Lin = MapLinear<NT>;
    constexpr int RL = P::RA, NSL = L / RL;
    extern __shared__ float2 sm[];
    __shared__ float redf[32];
    const uint32_t n1 = 1u << g.log_n1;
    const int t = threadIdx.x, lane = t & 31;
    float corr;
    {
        unsigned long long ck = cnt[0], cs = cnt[1];
        unsigned long long pm = (ck * cs) & ((2ull << g.log_np) - 1ull);
        corr = (float)((double)pm / (double)(1ull << g.log_np));
    }
    const size_t plane_words = (size_t)n1 * (L / 32);
    float res = 0.f;
    for (uint32_t m1 = blockIdx.x; m1 < n1; m1 += gridDim.x) {
        uint32_t* pe = planes + (size_t)m1 * (L / 32);
        uint32_t* po = pe + plane_words;
        if (2ull * m1 >= g.out_bits) {  // no output sample in this row
            for (int w = t; w < L / 32; w += NT) pe[w] = po[w] = 0u;
            continue;
        }
        float2 x[E];
        const float4* row4 = reinterpret_cast<const float4*>(Y + ((size_t)m1 << LOGL));
        if (t != 0) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float4 a = __ldcs(row4 + t + LR * r), b = __ldcs(row4 + (LR - t) + LR * r);
                x[r] = make_float2(a.x, a.y);
                x[16 + 15 - r] = make_float2(a.z, a.w);
                x[16 + r] = make_float2(b.x, b.y);
                x[15 - r] = make_float2(b.z, b.w);
            }
        } else {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float4 a = __ldcs(row4 + LR * r), b = __ldcs(row4 + LR / 2 + LR * r);
                x[r] = make_float2(a.x, a.y);
                x[r == 0 ? 8 : 16 - r] = make_float2(a.z, a.w);
                x[16 + r] = make_float2(b.x, b.y);
                x[16 + 15 - r] = make_float2(b.z, b.w);
            }
        }
        stage<L, 16, 1, +1, E, MapMirrorRow>(x);
        if (P::NSTAGE == 2) {
            exchange<L, E, 16, 1, MapMirrorRow, P::RB, Lin>(x, sm);
            stage<L, P::RB, 16, +1, E, Lin>(x);
            exchange<L, E, P::RB, 16, Lin, RL, Lin>(x, sm);
            stage<L, RL, 16 * P::RB, +1, E, Lin>(x);
        } else {
            exchange<L, E, 16, 1, MapMirrorRow, RL, Lin>(x, sm);
            stage<L, RL, 16, +1, E, Lin>(x);
        }
        // outputs: butterfly u = t + q*NT (j = u), sample m2 = j + NSL*r; lanes hold consecutive m2
#pragma unroll
        for (int q = 0; q < E / RL; ++q) {
            const int j = t + q * NT;
#pragma unroll
            for (int r = 0; r < RL; ++r) {
                const uint32_t m2 = (uint32_t)(j + NSL * r);
                const uint64_t x0 = 2ull * ((uint64_t)m1 + ((uint64_t)m2 << g.log_n1));
                const float2 v = x[q * RL + r];
                const float v0 = v.x + corr, v1 = v.y + corr;
                const float r0 = rintf(v0), r1 = rintf(v1);
                const bool ok0 = x0 < g.out_bits, ok1 = x0 + 1 < g.out_bits;
                if (ok0) res = fmaxf(res, fabsf(v0 - r0));
                if (ok1) res = fmaxf(res, fabsf(v1 - r1));
                const uint32_t be = __ballot_sync(0xffffffffu, ok0 && ((int)r0 & 1));
                const uint32_t bo = __ballot_sync(0xffffffffu, ok1 && ((int)r1 & 1));
                if (lane == 0) {
                    pe[m2 >> 5] = be;
                    po[m2 >> 5] = bo;
                }
            }
        }
        __syncthreads();  // exchanges of the next row reuse sm
    }
    float bm = block_max_f(res, redf);
    if (threadIdx.x == 0) atomicMax(resid_bits, __float_as_uint(bm));
}

// ============================================================================ finish
// Warp (a, c): plane rows m1 = 32a .. 32a+31 (lane), plane word column c (m2 = 32c .. 32c+31).
// Output word ow = (m2 N1 + m1_0)/16 holds samples m1_0 .. m1_0+15 of column m2, bits (even, odd)
// interleaved in the reference byte order; XOR with key_rest word ow.
__global__ void __launch_bounds__(1024) k_finish(const uint32_t* __restrict__ planes, BlockGeom g,
                                                 const uint32_t* __restrict__ key_rest, uint32_t flags,
                                                 uint32_t* __restrict__ out, uint32_t nwords) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const size_t plane_words = (size_t)n1 * wpr;
    const uint32_t a = blockIdx.x * 4u + (uint32_t)(warp & 3);
    const uint32_t c = blockIdx.y * 8u + (uint32_t)(warp >> 2);
    if (a >= n1 / 32u || c >= wpr) return;
    const size_t off = (size_t)(32u * a + (uint32_t)lane) * wpr + c;
    const uint32_t ve = __ldg(planes + off), vo = __ldg(planes + plane_words + off);
    uint32_t e_lo = 0, o_lo = 0;
#pragma unroll
    for (int b = 0; b < 32; ++b) {
        uint32_t e = __ballot_sync(0xffffffffu, (ve >> b) & 1u);
        uint32_t o = __ballot_sync(0xffffffffu, (vo >> b) & 1u);
        if (lane == b) {
            e_lo = e;
            o_lo = o;
        }
    }
    const uint32_t m2 = 32u * c + (uint32_t)lane;
    const uint64_t ow0 = ((uint64_t)m2 * n1 + 32ull * a) / 16ull;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint64_t ow = ow0 + (uint64_t)h;
        if (ow >= nwords) continue;
        uint32_t w = msb_pairs(h ? e_lo >> 16 : e_lo, h ? o_lo >> 16 : o_lo);
        if ((flags & kXor) && 32ull * ow < g.v) w ^= __ldg(key_rest + ow);
        out[ow] = __byte_perm(w, 0, 0x0123);
    }
}

// ============================================================================ launchers
template <class K>
static void smem_attr(K k, size_t bytes) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

static int grid_units(uint32_t units, int num_sms) {
    return (int)std::max<uint32_t>(1u, std::min<uint32_t>(units, (uint32_t)num_sms));
}

int launch_bit_rows(const BlockGeom& g, const uint32_t* bits, bool seed, uint32_t* rows, cudaStream_t s) {
    const uint32_t n1 = 1u << g.log_n1, n2 = 1u << g.log_n2;
    dim3 grid((n1 / 16u + 7u) / 8u, n2 / 32u);
    if (seed) k_bit_rows<true><<<grid, 256, 0, s>>>(bits, g, rows);
    else k_bit_rows<false><<<grid, 256, 0, s>>>(bits, g, rows);
    return (int)cudaGetLastError();
}

template <int LOGL>
static int pass_a_l(const BlockGeom& g, const uint32_t* rows, bool seed, float2* Y, unsigned long long* cnt,
                    int num_sms, cudaStream_t s) {
    constexpr int NT = (1 << LOGL) / 32;
    size_t smem = (size_t)Padded<(1 << LOGL)>::value * sizeof(float2);
    int grid = grid_units(1u << g.log_n1, num_sms);
    if (seed) {
        smem_attr(k_pass_a<LOGL, true>, smem);
        k_pass_a<LOGL, true><<<grid, NT, smem, s>>>(rows, g, Y, cnt);
    } else {
        smem_attr(k_pass_a<LOGL, false>, smem);
        k_pass_a<LOGL, false><<<grid, NT, smem, s>>>(rows, g, Y, cnt);
    }
    return (int)cudaGetLastError();
}

template <int LOGL>
static int pass_b_l(const BlockGeom& g, bool seed, float2* Y, float2* spec, int num_sms, cudaStream_t s) {
    constexpr int L = 1 << LOGL, CPT = 16384 / L;
    size_t smem = ((size_t)CPT * Padded<L>::value + (size_t)CPT * Plan<LOGL>::RA) * sizeof(float2);
    int grid = grid_units((1u << g.log_n2) / CPT, num_sms);
    if (seed) {
        smem_attr(k_pass_b<LOGL, true>, smem);
        k_pass_b<LOGL, true><<<grid, 512, smem, s>>>(Y, g, spec);
    } else {
        smem_attr(k_pass_b<LOGL, false>, smem);
        k_pass_b<LOGL, false><<<grid, 512, smem, s>>>(Y, g, spec);
    }
    return (int)cudaGetLastError();
}

template <int LOGL>
static int pass_c_l(const BlockGeom& g, const float2* Y, const unsigned long long* cnt, uint32_t* planes,
                    unsigned int* resid, int num_sms, cudaStream_t s) {
    constexpr int NT = (1 << LOGL) / 32;
    size_t smem = (size_t)Padded<(1 << LOGL)>::value * sizeof(float2);
    smem_attr(k_pass_c<LOGL>, smem);
    k_pass_c<LOGL><<<grid_units(1u << g.log_n1, num_sms), NT, smem, s>>>(Y, g, cnt, planes, resid);
    return (int)cudaGetLastError();
}

#define PA_ROWS_DISPATCH(LG, CALL)                   \
    switch (LG) {                                    \
        case 10: return CALL(10);                    \
        case 11: return CALL(11);                    \
        case 12: return CALL(12);                    \
        case 13: return CALL(13);                    \
        case 14: return CALL(14);                    \
        default: return (int)cudaErrorInvalidValue; \
    }
#define PA_COLS_DISPATCH(LG, CALL)                   \
    switch (LG) {                                    \
        case 5: return CALL(5);                      \
        case 6: return CALL(6);                      \
        case 7: return CALL(7);                      \
        case 8: return CALL(8);                      \
        case 9: return CALL(9);                      \
        case 10: return CALL(10);                    \
        case 11: return CALL(11);                    \
        case 12: return CALL(12);                    \
        default: return (int)cudaErrorInvalidValue; \
    }

int launch_pass_a(const BlockGeom& g, const uint32_t* rows, bool seed, float2* Y, unsigned long long* cnt,
                  int num_sms, cudaStream_t s) {
#define C(LG) pass_a_l<LG>(g, rows, seed, Y, cnt, num_sms, s)
    PA_ROWS_DISPATCH(g.log_n2, C)
#undef C
}

int launch_pass_b(const BlockGeom& g, bool seed, float2* Y, float2* spec, int num_sms, cudaStream_t s) {
#define C(LG) pass_b_l<LG>(g, seed, Y, spec, num_sms, s)
    PA_COLS_DISPATCH(g.log_n1, C)
#undef C
}

int launch_pass_c(const BlockGeom& g, const float2* Y, const unsigned long long* cnt, uint32_t* planes,
                  unsigned int* resid, int num_sms, cudaStream_t s) {
#define C(LG) pass_c_l<LG>(g, Y, cnt, planes, resid, num_sms, s)
    PA_ROWS_DISPATCH(g.log_n2, C)
#undef C
}

int launch_finish(const BlockGeom& g, const uint32_t* planes, const uint32_t* key_rest, uint32_t flags,
                  uint32_t* out, cudaStream_t s) {
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const uint32_t nwords = (g.out_bits + 31u) / 32u;
    // only plane columns that hold output samples: m2 < ceil(out_bits / (2 N1))
    const uint32_t m2max = (uint32_t)(((uint64_t)g.out_bits + 2ull * n1 - 1ull) / (2ull * n1));
    const uint32_t cols = std::min<uint32_t>(wpr, (m2max + 31u) / 32u);
    dim3 grid((n1 / 32u + 3u) / 4u, (cols + 7u) / 8u);
    k_finish<<<grid, 1024, 0, s>>>(planes, g, key_rest, flags, out, nwords);
    return (int)cudaGetLastError();
}

}  // namespace pa
