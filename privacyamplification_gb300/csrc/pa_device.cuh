// pa_device.cuh -- device building blocks of the GB300 privacy-amplification engine.
//
// The engine computes, for one block of n key/seed bits,
//     out[i] = ( sum_{j=0..h} key_start[j] * seed[(i-j) mod n] ) mod 2  XOR  key_rest[i],   i < v,
// the modified Toeplitz hash of nicoboss/PrivacyAmplification (PrivacyAmplification.cu:1686-2118),
// by an FP32 FFT convolution.  n real samples are folded into N = n/2 complex samples
// z[m] = x[2m] + i*x[2m+1]; the real spectrum is recovered by the usual split
// X[k] = ((Z[k] + conj Z[N-k]) - i W_2N^k (Z[k] - conj Z[N-k])) / 2.
//
// Everything here is plain SIMT FP32: the path is HBM/FP32 bound, not a contraction.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pa {

// ------------------------------------------------------------------------------ complex helpers
// Complex add / subtract as one packed two-lane FP32 instruction each (add.rn.f32x2 / sub.rn.f32x2,
// IEEE round-to-nearest per lane, so the same values as two scalar operations): the butterflies issue
// about half as many add instructions, which matters for these issue-bound passes.
__device__ __forceinline__ unsigned long long pk2(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 upk2(unsigned long long r) {
    float2 d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(r));
    return d;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cmulconj(float2 a, float2 b) {  // a * conj(b)
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 mul_i(float2 a) { return make_float2(-a.y, a.x); }
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }

// Shared-memory padding: one spare element after every 16 keeps strided butterfly accesses on
// distinct banks.
__device__ __forceinline__ constexpr int pad16(int k) { return k + (k >> 4); }
template <int L> struct Padded { static constexpr int value = L + L / 16; };

// e^{-i*pi*k/D} for D = 2^logD, k < 2^32, computed from exactly representable sincospif arguments
// (k is split so that both parts have at most 15 significant bits).  ~1 ulp per factor.
__device__ __forceinline__ float2 expmi_pi(uint32_t k, int logD) {
    k &= (2u << logD) - 1u;  // reduce mod 2D
    float s, c;
    if (logD <= 15) {
        sincospif(-(float)k * __int_as_float((127 - logD) << 23), &s, &c);
        return make_float2(c, s);
    }
    uint32_t kh = k >> 15, kl = k & 0x7FFFu;
    float s2, c2;
    sincospif(-(float)kh * __int_as_float((127 - (logD - 15)) << 23), &s, &c);
    sincospif(-(float)kl * __int_as_float((127 - logD) << 23), &s2, &c2);
    return cmul(make_float2(c, s), make_float2(c2, s2));
}

// ------------------------------------------------------------------------------ radix-R DFT
// cos/sin(2*pi*k/32), k < 16
__device__ __forceinline__ float2 w32(int k) {
    float c, s;
    switch (k) {
        case 0: c = 1.0f; s = 0.0f; break;
        case 1: c = 9.807852804e-01f; s = 1.950903220e-01f; break;
        case 2: c = 9.238795325e-01f; s = 3.826834324e-01f; break;
        case 3: c = 8.314696123e-01f; s = 5.555702330e-01f; break;
        case 4: c = 7.071067812e-01f; s = 7.071067812e-01f; break;
        case 5: c = 5.555702330e-01f; s = 8.314696123e-01f; break;
        case 6: c = 3.826834324e-01f; s = 9.238795325e-01f; break;
        case 7: c = 1.950903220e-01f; s = 9.807852804e-01f; break;
        case 8: c = 0.0f; s = 1.0f; break;
        case 9: c = -1.950903220e-01f; s = 9.807852804e-01f; break;
        case 10: c = -3.826834324e-01f; s = 9.238795325e-01f; break;
        case 11: c = -5.555702330e-01f; s = 8.314696123e-01f; break;
        case 12: c = -7.071067812e-01f; s = 7.071067812e-01f; break;
        case 13: c = -8.314696123e-01f; s = 5.555702330e-01f; break;
        case 14: c = -9.238795325e-01f; s = 3.826834324e-01f; break;
        default: c = -9.807852804e-01f; s = 1.950903220e-01f; break;
    }
    return make_float2(c, s);
}

// x * e^{DIR * 2*pi*i * k / 32}, k < 16; trivial angles become swaps/negations after inlining.
template <int DIR>
__device__ __forceinline__ float2 mul_w32(float2 x, int k) {
    if (k == 0) return x;
    if (k == 8) return DIR < 0 ? mul_mi(x) : mul_i(x);
    float2 w = w32(k);
    if (DIR < 0) w.y = -w.y;
    return cmul(x, w);
}

__device__ __forceinline__ constexpr int bitrev(int x, int bits) {
    int r = 0;
    for (int i = 0; i < bits; ++i) r |= ((x >> i) & 1) << (bits - 1 - i);
    return r;
}
__device__ __forceinline__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

// In-register DFT of size R (power of two <= 32), natural order in and out.
// DIR = -1: forward (e^{-2 pi i rk/R}), DIR = +1: inverse (unnormalised).
template <int R, int DIR>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
#pragma unroll
    for (int s = R / 2; s >= 1; s >>= 1) {
#pragma unroll
        for (int b = 0; b < R; b += 2 * s) {
#pragma unroll
            for (int i = 0; i < s; ++i) {
                float2 x = a[b + i], y = a[b + i + s];
                a[b + i] = cadd(x, y);
                a[b + i + s] = mul_w32<DIR>(csub(x, y), i * (32 / (2 * s)));
            }
        }
    }
    float2 t[R];
#pragma unroll
    for (int k = 0; k < R; ++k) t[k] = a[bitrev(k, ilog2(R))];
#pragma unroll
    for (int k = 0; k < R; ++k) a[k] = t[k];
}

// ------------------------------------------------------------------------------ CTA tile FFT
// In-place Stockham FFT of NSEQ sequences of length L (power of two) stored in shared memory,
// sequence s at sm + s * Padded<L>, element k at pad16(k).  NT threads; every thread owns
// E = NSEQ*L/NT elements per stage (E >= 16).  Radix-16 stages, then one radix-2/4/8 stage.
template <int L, int R, int NS, int NSEQ, int NT, int DIR>
__device__ __forceinline__ void fft_stage(float2* sm) {
    constexpr int E = NSEQ * L / NT;
    constexpr int Q = E / R;
    constexpr int LR = L / R;
    constexpr int SP = Padded<L>::value;
    static_assert(E % R == 0, "radix must divide the per-thread element count");
    float2 a[Q][R];
    int seq[Q], jj[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int u = threadIdx.x + q * NT;
        seq[q] = u / LR;
        jj[q] = u % LR;
#pragma unroll
        for (int r = 0; r < R; ++r) a[q][r] = sm[seq[q] * SP + pad16(jj[q] + r * LR)];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = jj[q];
        if (NS > 1) {
            const int t = j % NS;
            float s, c;
            sincospif((float)(DIR * 2 * t) / (float)(NS * R), &s, &c);
            const float2 w1 = make_float2(c, s);
            float2 w = w1;
#pragma unroll
            for (int r = 1; r < R; ++r) {
                a[q][r] = cmul(a[q][r], w);
                if (r + 1 < R) w = cmul(w, w1);
            }
        }
        dft<R, DIR>(a[q]);
        const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
        for (int r = 0; r < R; ++r) sm[seq[q] * SP + pad16(base + r * NS)] = a[q][r];
    }
    __syncthreads();
}

template <int L, int NS, int NSEQ, int NT, int DIR>
struct FftStages {
    static __device__ __forceinline__ void run(float2* sm) {
        constexpr int REM = L / NS;
        constexpr int R = REM >= 16 ? 16 : REM;
        fft_stage<L, R, NS, NSEQ, NT, DIR>(sm);
        FftStages<L, NS * R, NSEQ, NT, DIR>::run(sm);
    }
};
template <int NSEQ, int NT, int DIR>
struct FftStagesEnd {
    static __device__ __forceinline__ void run(float2*) {}
};
// Termination when NS == L.
#define PA_FFT_END(LL)                                                          \
    template <int NSEQ, int NT, int DIR>                                        \
    struct FftStages<LL, LL, NSEQ, NT, DIR> {                                   \
        static __device__ __forceinline__ void run(float2*) {}                 \
    };
PA_FFT_END(2) PA_FFT_END(4) PA_FFT_END(8) PA_FFT_END(16) PA_FFT_END(32) PA_FFT_END(64)
PA_FFT_END(128) PA_FFT_END(256) PA_FFT_END(512) PA_FFT_END(1024) PA_FFT_END(2048) PA_FFT_END(4096)
PA_FFT_END(8192) PA_FFT_END(16384)
#undef PA_FFT_END

// Unnormalised in-place FFT of the tile.  Caller must __syncthreads() after filling the tile.
template <int L, int NSEQ, int NT, int DIR>
__device__ __forceinline__ void fft_tile(float2* sm) {
    FftStages<L, 1, NSEQ, NT, DIR>::run(sm);
}

// ------------------------------------------------------------------------------ spectral step
// For a bin pair (k, N-k) of the half-length spectrum Z of a real sequence of length 2N:
//   A_k = 2 X[k] = (Z_a + conj Z_b) - i W_2N^k (Z_a - conj Z_b),   Z_a = Z[k], Z_b = Z[N-k]
// w = W_2N^k = e^{-i pi k/N}.  W_2N^{N-k} = -conj(w).
__device__ __forceinline__ void real_split(float2 za, float2 zb, float2 w, float2& xa2, float2& xb2) {
    float2 zbc = cconj(zb), zac = cconj(za);
    xa2 = csub(cadd(za, zbc), mul_i(cmul(w, csub(za, zbc))));
    float2 wb = make_float2(-w.x, w.y);  // -conj(w)
    xb2 = csub(cadd(zb, zac), mul_i(cmul(wb, csub(zb, zac))));
}

// Inverse of the split for a product pair P_a = P[k], P_b = P[N-k]:
//   Q[k] = (P_a + conj P_b) + i conj(w) (P_a - conj P_b)
//   Q[N-k] = (P_b + conj P_a) + i (-w) (P_b - conj P_a)
// IDFT_N(Q)[m] = y[2m] + i y[2m+1], y = unnormalised length-2N real IDFT of P.
__device__ __forceinline__ void real_merge(float2 pa, float2 pb, float2 w, float2& qa, float2& qb) {
    float2 pbc = cconj(pb), pac = cconj(pa);
    qa = cadd(cadd(pa, pbc), mul_i(cmul(cconj(w), csub(pa, pbc))));
    qb = cadd(cadd(pb, pac), mul_i(cmul(make_float2(-w.x, -w.y), csub(pb, pac))));
}

}  // namespace pa
