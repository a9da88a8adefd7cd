// pa_fft.cuh -- register-resident Stockham FFT stages for the three-pass kernels.
//
// A CTA owns a tile of NSEQ sequences of length L (NSEQ * L = 32 * NT): every thread keeps
// E = 32 complex values in registers.  A stage of radix R gives each thread E/R butterflies; the data
// only touches shared memory in the exchange between two stages (one write, one read, per element).
//
// Butterfly maps decide which butterflies (sequence, j) a thread owns in a stage:
//   MapLinear      u = tid + q*NT, seq = u / (L/R), j = u % (L/R)
//   MapMirrorRow   NSEQ == 1, R == 16: q = 0 -> j = tid, q = 1 -> j = L/16 - tid (tid 0: L/32)
//   MapMirrorPair  NSEQ even, R == 16: tid -> pair pp = tid / (L/16), jj = tid % (L/16);
//                  q = 0 -> (2pp, jj), q = 1 -> (2pp+1, L/16-1-jj)
// The mirror maps put bin k and its real-FFT partner in the same thread (see pa_passes.cu).
//
// Shared-memory positions are padded, k -> k + (k >> S) with S = 4 or 5 per exchange: S = 5 for the
// exchange after a radix-32 stage with NS = 1 (stride-32 writes), S = 4 otherwise.  For every
// stage shape used here pad(o + r*D) = pad(o) + r*D + (r*D >> S), so each thread computes one base
// address per butterfly and all R accesses use constant offsets.
#pragma once
#include "pa_device.cuh"

namespace pa {

template <int S>
__device__ __forceinline__ constexpr int padk(int k) { return k + (k >> S); }
template <int S>
__device__ __forceinline__ constexpr int padoff(int d) { return d + (d >> S); }

// Sequence stride of a tile in shared memory (elements): room for pad16, rounded to 4 mod 16 so that
// neighbouring columns written by one half-warp fall on different banks.
template <int L>
struct TileStride {
    static constexpr int value = (L + L / 16 + 11) / 16 * 16 + 4;  // smallest s >= L + L/16, s = 4 mod 16
};

template <int NT>
struct MapLinear {
    template <int L, int R>
    static __device__ __forceinline__ void at(int q, int& seq, int& j) {
        int u = (int)threadIdx.x + q * NT;
        seq = u / (L / R);
        j = u % (L / R);
    }
};

struct MapMirrorRow {
    template <int L, int R>
    static __device__ __forceinline__ void at(int q, int& seq, int& j) {
        static_assert(R == 16, "mirror stages are radix 16");
        int t = (int)threadIdx.x;
        seq = 0;
        j = q == 0 ? t : (t == 0 ? L / 32 : L / 16 - t);
    }
};

struct MapMirrorPair {
    template <int L, int R>
    static __device__ __forceinline__ void at(int q, int& seq, int& j) {
        static_assert(R == 16, "mirror stages are radix 16");
        int t = (int)threadIdx.x;
        int pp = t / (L / 16), jj = t % (L / 16);
        seq = 2 * pp + q;
        j = q == 0 ? jj : L / 16 - 1 - jj;
    }
};

// a[r] *= c * w^r for r = 0..R-1 (c = 1 when APPLY_C is false).  Powers are built as
// w^(4a+b) = (w^4)^a * w^b with w^2, w^3, w^4 from w: error ~(R/4 + 2) ulp instead of R ulp.
template <int R, bool APPLY_C>
__device__ __forceinline__ void twiddle_powers(float2* a, float2 w, float2 c) {
    float2 w2 = cmul(w, w), w3 = cmul(w2, w), w4 = cmul(w2, w2);
    float2 base = c;
#pragma unroll
    for (int blk = 0; blk < R; blk += 4) {
#pragma unroll
        for (int b = 0; b < 4 && blk + b < R; ++b) {
            int r = blk + b;
            if (r == 0) {
                if (APPLY_C) a[0] = cmul(a[0], c);
                continue;
            }
            float2 t;
            if (b == 0) t = base;
            else if (blk == 0 && !APPLY_C) t = b == 1 ? w : (b == 2 ? w2 : w3);
            else t = cmul(base, b == 1 ? w : (b == 2 ? w2 : w3));
            a[r] = cmul(a[r], t);
        }
        if (blk + 4 < R) base = (blk == 0 && !APPLY_C) ? w4 : cmul(base, w4);
    }
}

// e^{DIR * 2 pi i * t / M} for M a power of two <= 2^15 (exact sincospif argument).
template <int DIR>
__device__ __forceinline__ float2 unit_root(int t, int M) {
    float s, c;
    sincospif((float)(2 * DIR * t) / (float)M, &s, &c);
    return make_float2(c, s);
}

// Stage compute: twiddles (NS > 1, bases w[q] = W_{NS R}^{DIR (j mod NS)} precomputed by the caller)
// then radix-R DFTs of the thread's Q = E/R butterflies.
template <int R, int NS, int DIR, int E>
__device__ __forceinline__ void stage(float2 (&x)[E], const float2* w) {
    constexpr int Q = E / R;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (NS > 1) twiddle_powers<R, false>(&x[q * R], w[q], make_float2(1.f, 0.f));
        dft<R, DIR>(reinterpret_cast<float2(&)[R]>(x[q * R]));
    }
}

// Twiddle table of a stage (radix R, NS): tab[r * NS + m] = W_{NS R}^{DIR m r}, m < NS, r < R, filled
// by all threads of the block.  Laid out by r so that a warp's lanes (consecutive j, so consecutive
// m = j mod NS) read consecutive entries.
template <int R, int NS, int DIR>
__device__ __forceinline__ void fill_stage_table(float2* tab) {
    for (int i = threadIdx.x; i < R * NS; i += blockDim.x) tab[i] = unit_root<DIR>((i % NS) * (i / NS), NS * R);
}

// Stage compute with the twiddles read from a table made by fill_stage_table (instead of the power
// ladder of `stage`), then radix-R DFTs of the thread's butterflies (map Map over sequences of L).
template <int R, int NS, int DIR, int E, int L, class Map>
__device__ __forceinline__ void stage_tab(float2 (&x)[E], const float2* tab) {
#pragma unroll
    for (int q = 0; q < E / R; ++q) {
        int seq, j;
        Map::template at<L, R>(q, seq, j);
        const float2* tq = tab + (j % NS);
#pragma unroll
        for (int r = 1; r < R; ++r) x[q * R + r] = cmul(x[q * R + r], tq[r * NS]);
        dft<R, DIR>(reinterpret_cast<float2(&)[R]>(x[q * R]));
    }
}

// Twiddle bases of a stage for the thread's butterflies: w[q] = W_{NS R}^{DIR (j_q mod NS)}.
template <int L, int R, int NS, int DIR, int E, class Map>
__device__ __forceinline__ void stage_bases(float2* w) {
#pragma unroll
    for (int q = 0; q < E / R; ++q) {
        int seq, j;
        Map::template at<L, R>(q, seq, j);
        w[q] = unit_root<DIR>(j % NS, NS * R);
    }
}

struct NoHook {
    __device__ __forceinline__ void operator()() const {}
};

// Exchange between stage A (radix RA, NSA, map MA: its outputs) and stage B (radix RB, map MB: its
// inputs) through the shared tile sm (sequence stride SP, padding shift S).  Starts with a barrier
// so that earlier reads of sm are complete (LEAD = false: the caller's last barrier already follows
// them); `after_barrier` runs right after it (a copy into memory that every thread has finished
// reading can start there without a barrier of its own).
template <int L, int SP, int S, int E, int RA, int NSA, class MA, int RB, class MB, class Hook = NoHook,
          bool LEAD = true>
__device__ __forceinline__ void exchange(float2 (&x)[E], float2* sm, Hook after_barrier = Hook()) {
    if (LEAD) __syncthreads();
    after_barrier();
#pragma unroll
    for (int q = 0; q < E / RA; ++q) {
        int seq, j;
        MA::template at<L, RA>(q, seq, j);
        float2* b = sm + seq * SP + padk<S>((j / NSA) * NSA * RA + (j % NSA));
#pragma unroll
        for (int r = 0; r < RA; ++r) b[padoff<S>(r * NSA)] = x[q * RA + r];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E / RB; ++q) {
        int seq, j;
        MB::template at<L, RB>(q, seq, j);
        const float2* b = sm + seq * SP + padk<S>(j);
#pragma unroll
        for (int r = 0; r < RB; ++r) x[q * RB + r] = b[padoff<S>(r * (L / RB))];
    }
}

// Reads the inputs of a first stage (radix R, map M) from a tile stored with pad16.
template <int L, int SP, int E, int R, class M>
__device__ __forceinline__ void gather_inputs(float2 (&x)[E], const float2* sm) {
#pragma unroll
    for (int q = 0; q < E / R; ++q) {
        int seq, j;
        M::template at<L, R>(q, seq, j);
        const float2* b = sm + seq * SP + padk<4>(j);
#pragma unroll
        for (int r = 0; r < R; ++r) x[q * R + r] = b[padoff<4>(r * (L / R))];
    }
}

// Writes the outputs of a last stage (radix R, NS = L/R, map M) to the tile in natural order, pad16.
template <int L, int SP, int E, int R, class M>
__device__ __forceinline__ void scatter_outputs(const float2 (&x)[E], float2* sm) {
#pragma unroll
    for (int q = 0; q < E / R; ++q) {
        int seq, j;
        M::template at<L, R>(q, seq, j);
        float2* b = sm + seq * SP + padk<4>(j);
#pragma unroll
        for (int r = 0; r < R; ++r) b[padoff<4>(r * (L / R))] = x[q * R + r];
    }
}

// Radix plan of a length-2^LOGL transform with a radix-16 mirror stage: the other LOGL-4 bits are
// split into at most two stages of radix <= 32.
template <int LOGL>
struct Plan {
    static constexpr int REST = LOGL - 4;
    static constexpr int NSTAGE = REST <= 5 ? 1 : 2;               // stages besides the mirror one
    static constexpr int RA = 1 << (NSTAGE == 1 ? REST : (REST + 1) / 2);
    static constexpr int RB = NSTAGE == 1 ? 1 : 1 << (REST / 2);
    static_assert(REST >= 1 && REST <= 10, "transform length out of range");
};

// Padding shift of an exchange that follows a stage of radix R with NS = 1.
template <int R>
struct PadAfterFirst {
    static constexpr int value = R == 32 ? 5 : 4;
};

}  // namespace pa
