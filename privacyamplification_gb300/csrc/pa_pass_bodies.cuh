// pa_pass_bodies.cuh -- the three passes of the four-step FP32 convolution as device functions, shared by
// the per-pass kernels (pa_passes.cu: one launch per pass, the grid walks rows or tiles) and the persistent
// lane kernel (pa_lanes.cu: a few CTAs of one lane walk a block's rows and tiles between lane barriers).
//
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
#pragma once
#include "pa_device.cuh"
#include "pa_fft.cuh"
#include "pa_kernels.cuh"
#include "pa_tma.cuh"

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

// Asynchronous prefetch of [p, p + bytes) into L2 (bytes a multiple of 16, p 16-byte aligned).
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// 8-byte asynchronous global -> shared copy (L2 only), and the wait for all of a thread's copies.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Waits until at most N of this thread's committed copy groups are still in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

}  // namespace

// ============================================================================ bit-plane transposes
// 16 x 16 transpose of 2-bit elements inside each half-warp (Eklundh's recursive block swap):
// element e of lane L (bits 31-2e and 30-2e) becomes element L of lane e.
__device__ __forceinline__ uint32_t transpose16x2(uint32_t w, int lane) {
    const uint32_t masks[4] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u};  // elements with e & s
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int s = 8 >> i;
        const uint32_t m = masks[i];
        const uint32_t p = __shfl_xor_sync(0xffffffffu, w, s);
        w = (lane & s) ? ((w & m) | ((p & m) << (2 * s))) : ((w & ~m) | ((p & ~m) >> (2 * s)));
    }
    return w;
}

// ============================================================================ pass A
// Row m1: FFT over m2 of the 2N2 bits of the row, 4-step twiddle W_N^{m1 k2}, pair-order store.
// Radices RA, RB (linear) then 16 (mirror, NS = L/16).  The CTA (L/32 threads) takes rows first,
// first + stride, ... (the kernel: blockIdx.x, gridDim.x).
template <int LOGL>
__device__ __forceinline__ void pass_a_rows(const uint32_t* __restrict__ rows, const BlockGeom& g,
                                            float2* __restrict__ Y, unsigned long long* cnt, uint32_t first,
                                            uint32_t stride) {
    constexpr int L = 1 << LOGL, NT = L / 32, E = 32, LR = L / 16, SP = TileStride<L>::value;
    using P = Plan<LOGL>;
    using Lin = MapLinear<NT>;
    constexpr int QB = P::NSTAGE == 2 ? E / P::RB : 0;   // butterflies per thread in stage B
    constexpr int T1N = LR < 32 ? LR : 32, T2N = LR / T1N;  // W_N^{m1 j} = T1[j % 32] T2[j / 32]
    extern __shared__ float2 sm[];
    __shared__ float2 rho[2][16], t1[2][T1N], t2[2][T2N];  // per-row tables, double-buffered like bits
    __shared__ float2 tws[(QB > 0 ? QB : 1) + 2][NT];
    __shared__ __align__(16) uint32_t bits[2][L / 16];  // double buffer: this row, next row
    __shared__ unsigned long long red[32];
    const uint32_t n1 = 1u << g.log_n1;
    const int t = threadIdx.x;
    // per-thread stage twiddle bases (the same for every row)
    float2 wb[QB > 0 ? QB : 1], wm[2];
    if (P::NSTAGE == 2) stage_bases<L, P::RB, P::RA, -1, E, Lin>(wb);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        int seq, j;
        MapMirrorRow::at<L, 16>(q, seq, j);
        wm[q] = unit_root<-1>(j, L);
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) tws[q][t] = wb[q];
    tws[QB][t] = wm[0];
    tws[QB + 1][t] = wm[1];
    uint32_t ones = 0;
    // A row's bits (L/16 words, two per thread) are copied asynchronously one row ahead.
    static_assert(L / 16 == 2 * NT, "two bit words per thread");
    auto fetch_row = [&](uint32_t r, int buf) {
        if (r < n1) cp_async8(&bits[buf][2 * t], rows + (size_t)r * (L / 16) + 2 * t);
        cp_async_commit();
    };
    // Row tables W_N^{m1 LR r}, W_N^{m1 i}, W_N^{m1 T1N i} of row m1 into buffer b.  Row m1 + G's are
    // computed while row m1's first stage runs (independent work the compiler interleaves), so the few
    // threads doing it do not hold the block at a barrier.
    auto row_tables = [&](uint32_t m1, int b) {
        if (m1 >= n1) return;
        for (int i = t; i < 16 + T1N + T2N; i += NT) {
            uint64_t e = i < 16 ? (uint64_t)LR * (uint64_t)i : (i < 16 + T1N ? (uint64_t)(i - 16)
                                                                                : (uint64_t)T1N * (uint64_t)(i - 16 - T1N));
            float2 w = expmi_pi((uint32_t)((2ull * m1 * e) & ((2ull << g.log_n) - 1)), g.log_n);
            if (i < 16) rho[b][i] = w;
            else if (i < 16 + T1N) t1[b][i - 16] = w;
            else t2[b][i - 16 - T1N] = w;
        }
    };
    fetch_row(first, 0);
    row_tables(first, 0);
    int buf = 0;
    for (uint32_t m1 = first; m1 < n1; m1 += stride, buf ^= 1) {
        cp_async_wait_group<0>();  // this thread's copy of row m1 (the only one in flight) has landed
        // One barrier: row m1's bits and tables visible; the previous row is past its mirror stage, the
        // last reader of tables[buf ^ 1] (bits[buf ^ 1] were read at its start).
        __syncthreads();
        fetch_row(m1 + stride, buf ^ 1);
        row_tables(m1 + stride, buf ^ 1);
        ones += __popc(bits[buf][2 * t]) + __popc(bits[buf][2 * t + 1]);
        float2 x[E];
#pragma unroll
        for (int q = 0; q < E / P::RA; ++q) {
            const int j = t + q * NT;
#pragma unroll
            for (int r = 0; r < P::RA; ++r) {
                const int m2 = j + r * (L / P::RA);
                const uint32_t w = bits[buf][m2 >> 4];
                const int sh = 30 - 2 * (m2 & 15);
                x[q * P::RA + r] = make_float2((float)((w >> (sh + 1)) & 1u), (float)((w >> sh) & 1u));
            }
        }
        stage<P::RA, 1, -1, E>(x, nullptr);
        // the first exchange needs no leading barrier: the row's barrier above follows the previous
        // row's last reads of sm, and nothing reads sm since
        if (P::NSTAGE == 2) {
            exchange<L, SP, PadAfterFirst<P::RA>::value, E, P::RA, 1, Lin, P::RB, Lin, NoHook, false>(x, sm);
            float2 w[QB > 0 ? QB : 1];
#pragma unroll
            for (int q = 0; q < QB; ++q) w[q] = tws[q][t];
            stage<P::RB, P::RA, -1, E>(x, w);
            exchange<L, SP, 4, E, P::RB, P::RA, Lin, 16, MapMirrorRow>(x, sm);
        } else {
            exchange<L, SP, PadAfterFirst<P::RA>::value, E, P::RA, 1, Lin, 16, MapMirrorRow, NoHook, false>(x, sm);
        }
        // mirror stage (NS = L/16) with the 4-step twiddle W_N^{m1 (j + LR r)} folded in:
        // W_N^{m1 j} on the inputs, rho[r] = W_N^{m1 LR r} on the outputs.
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int seq, j;
            MapMirrorRow::at<L, 16>(q, seq, j);
            const float2 c = cmul(t1[buf][j % T1N], t2[buf][j / T1N]);
            twiddle_powers<16, true>(&x[16 * q], tws[QB + q][t], c);
            dft<16, -1>(reinterpret_cast<float2(&)[16]>(x[16 * q]));
#pragma unroll
            for (int r = 0; r < 16; ++r) x[16 * q + r] = cmul(x[16 * q + r], rho[buf][r]);
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

// Slots of pass B's per-thread stage-base table (NT = 256 entries each): forward second stage, mirror
// stage (2), inverse second stage, last inverse stage.  When the linear map gives a thread the same
// butterfly index j in both of its butterflies (NT a multiple of L/R) one slot serves both, and with
// first-stage radix 16 the inverse second stage's bases are the conjugates of the forward ones.
template <int LOGL, int NT_ = 256>
struct PassBBases {
    static constexpr int L = 1 << LOGL, NT = NT_, E = 32;
    using P = Plan<LOGL>;
    static constexpr int RL = P::RA, NSL = L / RL, QB = P::NSTAGE == 2 ? E / P::RB : 0, QL = E / RL;
    static constexpr bool LEAN = LOGL <= 6;
    static constexpr bool SHARE2 = P::NSTAGE == 2 && P::RA == 16 && NT % (L / P::RB) == 0;
    static constexpr bool SHAREL = !LEAN && NT % NSL == 0;
    static constexpr int F2 = 0, NF2 = SHARE2 ? 1 : QB;
    static constexpr int M = F2 + NF2;
    static constexpr int I2 = M + 2, NI2 = SHARE2 ? 0 : QB;
    static constexpr int LS = I2 + NI2, NLS = LEAN ? 0 : (SHAREL ? 1 : QL);
    static constexpr int SLOTS = LS + NLS;
    static constexpr int f2(int q) { return F2 + (SHARE2 ? 0 : q); }
    static constexpr int i2(int q) { return I2 + q; }
    static constexpr int ls(int q) { return LS + (SHAREL ? 0 : q); }
};

// NT threads x 32 values: the kernel's tile is 8192 complex values with NT = 256 (one mirror pair of
// 4096-point columns at n = 2^27), so that two CTAs share an SM and hide each other's HBM latency.
// Input: Y (row-major pairs, as pass A wrote it) through 2D TMA boxes of 256 rows x CPT columns (the
// next tile's first `early` boxes copied into a buffer of their own as soon as the current tile is in
// registers; every warp issues its share), or per-thread asynchronous copies when the tile is too wide
// for a box.  Output (key pass): Z, tile-major (Z[tile][m1][CPT columns]), stored coalesced from
// registers; (seed pass): spec.
// The CTA takes tiles first, first + stride, ... (the kernel: blockIdx.x, gridDim.x).  GRP: the tiles of
// `nblocks` blocks of a group, one after another (unit u = block * ntiles + tile), so that a CTA's next
// tile may be another block's and its copy still overlaps the current one; Y, Z, mapY and a seed pass's
// spec hold the blocks one after another (N complex values, N1 rows of mapY each), and a key pass reads
// block b's spectrum from ge[b].spec.
// FUSED: a seed used by this block only.  Every tile is taken twice, first from the seed's row pass output
// (mapYs) as a seed pass, its spectrum tile parked in this CTA's CPT * L values of `spec` (written and read
// back by the same CTA a tile later, so it stays in L2), then from the key's (mapY) as a key pass against it.
template <int LOGL, bool SEED, int NT, bool GRP = false, bool FUSED = false>
__device__ __forceinline__ void pass_b_tiles(const CUtensorMap* mapY, const float2* __restrict__ Y,
                                             float2* __restrict__ Z, const BlockGeom& g, float2* __restrict__ spec,
                                             int* err, int early, uint32_t first, uint32_t stride,
                                             const GroupEntry* ge = nullptr, uint32_t nblocks = 1,
                                             const CUtensorMap* mapYs = nullptr) {
    constexpr int L = 1 << LOGL, E = 32, CPT = 32 * NT / L, LR = L / 16, SP = TileStride<L>::value;
    constexpr bool TMA = CPT <= 128;              // box inner extent 2*CPT floats <= 256
    static_assert(!FUSED || (TMA && !GRP && !SEED), "the fused pass is a one-block key pass with TMA tiles");
    constexpr int BOXR = L < 256 ? L : 256;       // rows per box
    using P = Plan<LOGL>;
    using Lin = MapLinear<NT>;
    constexpr int RL = P::RA;                      // radix of the last inverse stage
    constexpr int NSL = L / RL;                    // its NS
    constexpr int QB = P::NSTAGE == 2 ? E / P::RB : 0;
    constexpr int QL = E / RL;
    // Short columns (many per tile): the last inverse stage computes its twiddles directly instead of
    // keeping per-column tables, which would not fit in shared memory.
    constexpr bool LEAN = LOGL <= 6;
    constexpr int U1N = LEAN ? 0 : (NSL < 16 ? NSL : 16), U2N = LEAN ? 0 : NSL / U1N;  // W_N^{j k2}
    // The last inverse stage writes straight from registers when the linear map gives each thread both
    // columns of a pair for the same rows; the tile buffer is then free during that stage and the next
    // tile's copies overlap with it.
    constexpr bool DIRECT = CPT == 2 && NSL == NT && QL == 2;
    constexpr int NBOX = L / BOXR;               // TMA boxes per tile
    // Shared memory: [tile boxes 0 .. early-1][tile / exchange buffer][tables].  A tile occupies the
    // first `early` boxes' own space and the start of the exchange buffer, so the next tile's first
    // boxes are copied as soon as the current tile is in registers, the rest once the exchange buffer
    // is free (after the last exchange in the DIRECT key pass, else at the next tile's start).
    if (!TMA) early = 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* srow = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float2* sm = srow + early * BOXR * CPT;
    float2* sigma = sm + CPT * SP;       // [CPT][RL]   conj(W_N^{NSL r k2})
    float2* u1 = sigma + CPT * RL;       // [CPT][U1N]  W_N^{k2 (j % 16)}
    float2* u2 = u1 + CPT * U1N;         // [CPT][U2N]  W_N^{k2 16 (j / 16)}
    float2* tws = u2 + CPT * U2N;        // [PassBBases slots][NT] per-thread stage bases
    using TB = PassBBases<LOGL, NT>;
    constexpr int U1D = U1N > 0 ? U1N : 1, U2D = U2N > 0 ? U2N : 1;  // divisors (unused when LEAN)
    __shared__ __align__(8) uint64_t bar;       // TMA completion of the current tile (boxes early ..)
    __shared__ __align__(8) uint64_t bar_early; // TMA completion of boxes 0 .. early-1
    __shared__ __align__(8) uint64_t bar_spec;  // bulk copy of the tile's seed spectrum (key pass)
    __shared__ int s_fail;                      // a bounded wait expired: stop waiting
    const uint32_t n2 = 1u << g.log_n2;
    const int ntiles = (int)(n2 / CPT);
    const int nunits = GRP ? ntiles * (int)nblocks : ntiles;
    const int tshift = __ffs(ntiles) - 1;  // ntiles is a power of two
    auto unit_tile = [&](int u) { return GRP ? (u & (ntiles - 1)) : u; };
    auto unit_block = [&](int u) { return GRP ? (uint32_t)(u >> tshift) : 0u; };
    const int t = threadIdx.x;
    const int pp = t / LR, jj = t % LR;
    const float sc = 1.0f / (float)(4ull << g.log_np);  // seed spectrum scale 2X/(4Np)
    {
        float2 w[4];
        if (P::NSTAGE == 2) {
            stage_bases<L, P::RB, P::RA, -1, E, Lin>(w);
#pragma unroll
            for (int q = 0; q < TB::NF2; ++q) tws[TB::f2(q) * NT + t] = w[q];
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int seq, j;
            MapMirrorPair::at<L, 16>(q, seq, j);
            tws[(TB::M + q) * NT + t] = unit_root<-1>(j, L);
        }
        if (P::NSTAGE == 2 && !TB::SHARE2) {
            stage_bases<L, P::RB, 16, +1, E, Lin>(w);
#pragma unroll
            for (int q = 0; q < TB::NI2; ++q) tws[TB::i2(q) * NT + t] = w[q];
        }
        if (!LEAN) {
#pragma unroll
            for (int q = 0; q < TB::NLS; ++q) {
                int seq, j;
                Lin::template at<L, RL>(q, seq, j);
                tws[TB::ls(q) * NT + t] = unit_root<+1>(j % NSL, NSL * RL);
            }
        }
    }
    // Tile tl -> sm.  TMA: L/BOXR boxes land row-major, sm[m1 * CPT + c], and complete on `bar`
    // (caller: all threads past their last generic access to sm and a proxy fence).  Otherwise 8-byte
    // asynchronous copies into the padded column layout sm[c * SP + pad(m1)].  The row segments of
    // neighbouring tiles share sectors, so both forms read through L2 normally.
    // TMA boxes [b0, b1) of tile tl, called by every thread: thread 0 announces the bytes, lane 0 of
    // each warp issues every (NT/32)-th box (a copy landing first cannot complete the phase: its
    // arrival is pending).
    auto load_boxes = [&](int u, int b0, int b1, uint64_t* bb, const CUtensorMap* map) {
        if (u >= nunits || b0 >= b1) return;
        const int tl = unit_tile(u), y0 = (int)(unit_block(u) << g.log_n1);
        if (t == 0) mbar_expect_tx(bb, (uint32_t)((b1 - b0) * BOXR * CPT * sizeof(float2)));
        if ((t & 31) == 0) {
#pragma unroll 1
            for (int b = b0 + (t >> 5); b < b1; b += NT / 32)
                tma_load_2d(srow + b * BOXR * CPT, map, 2 * CPT * tl, y0 + BOXR * b, bb);
        }
    };
    auto load_tile = [&](int u, const CUtensorMap* map) {
        if (u >= nunits) return;
        if (TMA) {
            load_boxes(u, 0, early, &bar_early, map);
            load_boxes(u, early, NBOX, &bar, map);
        } else {
            const int tl = unit_tile(u);
            const float2* Yb = Y + ((size_t)unit_block(u) << g.log_n);
#pragma unroll 4
            for (int i = 0; i < L * CPT / 2 / NT; ++i) {
                const int idx = t + i * NT, m1 = idx / (CPT / 2), cp = idx % (CPT / 2);
                const float2* src = Yb + (size_t)m1 * n2 + (size_t)tl * CPT + 2 * cp;
                cp_async8(sm + (2 * cp) * SP + padk<4>(m1), src);
                cp_async8(sm + (2 * cp + 1) * SP + padk<4>(m1), src + 1);
            }
        }
    };
    uint32_t parity = 0, parity_early = 0;
    auto wait_bar = [&](uint64_t* bb, uint32_t& par) {
        if (!s_fail && !mbar_wait(bb, par)) {
            s_fail = 1;
            atomicExch(err, kErrTmaTimeout);
        }
        par ^= 1u;
    };
    auto wait_tile = [&]() {
        if (TMA) {
            if (early > 0) wait_bar(&bar_early, parity_early);
            if (early < NBOX) wait_bar(&bar, parity);
        } else {
            cp_async_wait_all();
        }
    };
    if (t == 0) {
        s_fail = 0;
        mbar_init(&bar, 1);
        mbar_init(&bar_early, 1);
        mbar_init(&bar_spec, 1);
    }
    __syncthreads();
    uint32_t parity_spec = 0;
    fence_proxy_async();
    load_tile((int)first, FUSED ? mapYs : mapY);
    for (int unit = (int)first; unit < nunits; unit += (int)stride) {
#pragma unroll
        for (int part = 0; part < (FUSED ? 2 : 1); ++part) {
            // sd: this part is a seed pass (FUSED: part 0 the seed's tile, part 1 the key's)
            const bool sd = FUSED ? part == 0 : SEED;
            const CUtensorMap* const map_self = FUSED && sd ? mapYs : mapY;
            // the part after this one: FUSED alternates seed and key tiles, otherwise the next tile (formed
            // where it is used, so that nothing extra stays live across the transform)
            auto next_u = [&]() { return FUSED && sd ? unit : unit + (int)stride; };
            auto map_next = [&]() { return FUSED ? (sd ? mapY : mapYs) : mapY; };
            const int tile = unit_tile(unit);
            const uint32_t blk = unit_block(unit);
            // this block's spectrum: the seed pass writes it, the key pass reads it
            float2* const bspec = !GRP ? spec : (SEED ? spec + ((size_t)blk << g.log_n) : const_cast<float2*>(ge[blk].spec));
            // the tile's seed spectrum (contiguous) is read after the forward FFT: start it into L2 now
            if (!FUSED && !SEED && t == 0)
                prefetch_l2(bspec + (size_t)tile * (CPT * L), CPT * L * sizeof(float2));
            // The rest of a part's boxes were issued by the part before it when that was a DIRECT key pass
            // (after its last exchange); otherwise here, once every thread is done with sm.
            const bool preloaded = DIRECT && (FUSED ? sd : !SEED);
            const bool first_part = unit == (int)first && (!FUSED || sd);
            if (!preloaded && !first_part) {
                __syncthreads();  // previous tile done with sm
                fence_proxy_async();
                if (TMA) load_boxes(unit, early, NBOX, &bar, map_self);  // its first boxes came early
                else load_tile(unit, map_self);
            }
            wait_tile();
            __syncthreads();  // tile copies visible; previous tile done with the tables
            // The tile's column tables are first read by the last inverse stage, several block barriers
            // later: no barrier of their own, so the few threads computing them overlap the first stages.
            if (!sd) {
                for (int i = t; i < CPT * (RL + U1N + U2N); i += NT) {
                    int c, kind, r;
                    if (i < CPT * RL) { c = i / RL; r = i % RL; kind = 0; }
                    else if (i < CPT * (RL + U1N)) { c = (i - CPT * RL) / U1D; r = (i - CPT * RL) % U1D; kind = 1; }
                    else { c = (i - CPT * (RL + U1N)) / U2D; r = (i - CPT * (RL + U1N)) % U2D; kind = 2; }
                    uint64_t k2 = col_k2((uint32_t)tile * (CPT / 2) + (uint32_t)(c >> 1), c & 1, n2);
                    uint64_t mult = kind == 0 ? (uint64_t)NSL * r : (kind == 1 ? (uint64_t)r : (uint64_t)U1N * r);
                    uint64_t e = (mult * k2) & ((1ull << g.log_n) - 1);
                    float2 w = expmi_pi((uint32_t)(2 * e), g.log_n);
                    if (kind == 0) sigma[c * RL + r] = cconj(w);
                    else if (kind == 1) u1[c * U1N + r] = w;
                    else u2[c * U2N + r] = w;
                }
            }
            float2 x[E];
            if (TMA) {  // row-major tile: element m1 of column c at sm[m1 * CPT + c]
#pragma unroll
                for (int q = 0; q < E / P::RA; ++q) {
                    int seq, j;
                    Lin::template at<L, P::RA>(q, seq, j);
#pragma unroll
                    for (int r = 0; r < P::RA; ++r) x[q * P::RA + r] = srow[(j + r * (L / P::RA)) * CPT + seq];
                }
            } else {
                gather_inputs<L, SP, E, P::RA, Lin>(x, sm);
            }
            stage<P::RA, 1, -1, E>(x, nullptr);
            // after the first exchange's barrier every thread has read the tile: the next tile's own boxes
            // are copied under the rest of this tile's work
            auto copy_early = [&]() {
                if (early > 0) {
                    fence_proxy_async();
                    load_boxes(next_u(), 0, early, &bar_early, map_next());
                }
            };
            if (P::NSTAGE == 2) {
                exchange<L, SP, PadAfterFirst<P::RA>::value, E, P::RA, 1, Lin, P::RB, Lin>(x, sm, copy_early);
                float2 w[QB > 0 ? QB : 1];
#pragma unroll
                for (int q = 0; q < QB; ++q) w[q] = tws[TB::f2(q) * NT + t];
                stage<P::RB, P::RA, -1, E>(x, w);
                exchange<L, SP, 4, E, P::RB, P::RA, Lin, 16, MapMirrorPair>(x, sm);
            } else {
                exchange<L, SP, PadAfterFirst<P::RA>::value, E, P::RA, 1, Lin, 16, MapMirrorPair>(x, sm, copy_early);
            }
            float2* tspec = FUSED ? spec + (size_t)first * (CPT * L) : bspec + (size_t)tile * (CPT * L);
            const bool special = tile == 0;  // pair 0 holds the self-mirrored columns 0 and N2/2
            // Key pass: the tile buffer is free until the inverse exchange, so the tile's seed spectrum
            // (CPT * L values, contiguous) is copied into it while the mirror stage computes, and the
            // spectral step reads shared memory instead of waiting on L2.
            const bool spec_smem = !sd && !special;
            if (spec_smem) {
                __syncthreads();  // every thread done reading sm
                fence_proxy_async();
                constexpr uint32_t kBytes = CPT * L * sizeof(float2), kChunk = 16384;
                if (t == 0) mbar_expect_tx(&bar_spec, kBytes);
                if ((t & 31) == 0) {  // one chunk per warp
#pragma unroll 1
                    for (uint32_t off = (uint32_t)(t >> 5) * kChunk; off < kBytes; off += (NT / 32) * kChunk)
                        bulk_load(reinterpret_cast<char*>(sm) + off, reinterpret_cast<const char*>(tspec) + off, kChunk,
                                  &bar_spec);
                }
            }
            {
                float2 w[2] = {tws[TB::M * NT + t], tws[(TB::M + 1) * NT + t]};
                stage<16, LR, -1, E>(x, w);
            }
            if (spec_smem) {
                if (!s_fail && !mbar_wait(&bar_spec, parity_spec)) {
                    s_fail = 1;
                    atomicExch(err, kErrTmaTimeout);
                }
                parity_spec ^= 1u;
            }

            // ---- spectral step: real split, product with the seed spectrum, real merge
            if (special) {
                __syncthreads();
                if (pp == 0) {
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        int seq, j;
                        MapMirrorPair::at<L, 16>(q, seq, j);
                        float2* b = sm + seq * SP + padk<4>(j);
#pragma unroll
                        for (int r = 0; r < 16; ++r) b[padoff<4>(LR * r)] = x[16 * q + r];
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
                            float2 z = sm[padk<4>(0)];
                            float nyq = 2.0f * (z.x - z.y);
                            if (sd) {
                                tspec[spec_index<LR>(0, 0)] = make_float2(nyq * sc, 0.f);
                            } else {
                                float pn = nyq * tspec[spec_index<LR>(0, 0)].x;
                                sm[padk<4>(0)] = make_float2(pn, -pn);
                            }
                            ka = kb = L / 2;
                            k = n2 * (uint32_t)(L / 2);
                        }
                        float2 w = expmi_pi(k, g.log_n);
                        float2 za = sm[ca * SP + padk<4>(ka)], zb = sm[cb * SP + padk<4>(kb)];
                        float2 xa, xb;
                        real_split(za, zb, w, xa, xb);
                        int ia = spec_index<LR>(ca, ka), ib = spec_index<LR>(cb, kb);
                        if (sd) {
                            tspec[ia] = cscale(xa, sc);
                            tspec[ib] = cscale(xb, sc);
                        } else {
                            float2 qa, qb;
                            real_merge(cmul(xa, tspec[ia]), cmul(xb, tspec[ib]), w, qa, qb);
                            sm[ca * SP + padk<4>(ka)] = qa;
                            sm[cb * SP + padk<4>(kb)] = qb;
                        }
                    }
                }
                __syncthreads();
                if (pp == 0 && !sd) {
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        int seq, j;
                        MapMirrorPair::at<L, 16>(q, seq, j);
                        const float2* b = sm + seq * SP + padk<4>(j);
#pragma unroll
                        for (int r = 0; r < 16; ++r) x[16 * q + r] = b[padoff<4>(LR * r)];
                    }
                }
            }
            if (!special || pp != 0) {
                // bins (k1 = jj + LR r, k2 = p) and (L-1-k1, N2-p): x[r] and x[16 + 15 - r];
                // W_2N^{p + N2 (jj + LR r)} = W_2N^{p + N2 jj} * W_32^r
                const uint32_t p = (uint32_t)tile * (CPT / 2) + (uint32_t)pp;
                const float2 base = expmi_pi(p + n2 * (uint32_t)jj, g.log_n);
                const float2* sbase = spec_smem ? sm : tspec;  // key pass: the copy in shared memory
                const float2* sa = sbase + (2 * pp) * 16 * LR + jj;
                const float2* sb = sbase + (2 * pp + 1) * 16 * LR + jj;
                float2* da = tspec + (2 * pp) * 16 * LR + jj;
                float2* db = tspec + (2 * pp + 1) * 16 * LR + jj;
                if (sd) {
#pragma unroll
                    for (int r = 0; r < 16; ++r) {
                        // W_32^r = e^{-i pi r/16} = (cos, -sin)(2 pi r/32), r < 16
                        const float2 w = r ? cmul(base, make_float2(w32(r).x, -w32(r).y)) : base;
                        float2 xa, xb;
                        real_split(x[r], x[16 + 15 - r], w, xa, xb);
                        if (FUSED) {  // parked for this CTA's key pass: keep it in L2
                            da[r * LR] = cscale(xa, sc);
                            db[(15 - r) * LR] = cscale(xb, sc);
                        } else {
                            __stcs(da + r * LR, cscale(xa, sc));
                            __stcs(db + (15 - r) * LR, cscale(xb, sc));
                        }
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < 16; ++r) {
                        const float2 w = r ? cmul(base, make_float2(w32(r).x, -w32(r).y)) : base;
                        float2 xa, xb;
                        real_split(x[r], x[16 + 15 - r], w, xa, xb);
                        float2 qa, qb;
                        float2 fa, fb;
                        if (spec_smem) {
                            fa = sa[r * LR];
                            fb = sb[(15 - r) * LR];
                        } else {
                            fa = __ldcs(sa + r * LR);
                            fb = __ldcs(sb + (15 - r) * LR);
                        }
                        real_merge(cmul(xa, fa), cmul(xb, fb), w, qa, qb);
                        x[r] = qa;
                        x[16 + 15 - r] = qb;
                    }
                }
            }
            if (sd) {
                // the key pass copies the parked spectrum with the bulk-copy (async) proxy: order this
                // thread's generic writes before it (the block barriers in between order the threads)
                if (FUSED) fence_proxy_async_global();
                continue;
            }

            // ---- inverse column FFTs (radices 16, RB, RA) with the inverse 4-step twiddle folded into
            // the last stage: conj(W_N^{m1 k2}), m1 = j + NSL r
            stage<16, 1, +1, E>(x, nullptr);
            if (P::NSTAGE == 2) {
                exchange<L, SP, 4, E, 16, 1, MapMirrorPair, P::RB, Lin>(x, sm);
                float2 w[QB > 0 ? QB : 1];
#pragma unroll
                for (int q = 0; q < QB; ++q)
                    w[q] = TB::SHARE2 ? cconj(tws[TB::f2(q) * NT + t]) : tws[TB::i2(q) * NT + t];
                stage<P::RB, 16, +1, E>(x, w);
                exchange<L, SP, 4, E, P::RB, 16, Lin, RL, Lin>(x, sm);
            } else {
                exchange<L, SP, 4, E, 16, 1, MapMirrorPair, RL, Lin>(x, sm);
            }
            if (DIRECT) {  // after the last exchange sm is free until the next tile: the rest of its boxes
                __syncthreads();
                fence_proxy_async();
                if (TMA) load_boxes(next_u(), early, NBOX, &bar, map_next());
                else load_tile(next_u(), map_next());
            }
#pragma unroll
            for (int q = 0; q < QL; ++q) {
                int seq, j;
                Lin::template at<L, RL>(q, seq, j);
                float2 c, wbase;
                if (LEAN) {
                    uint32_t k2 = col_k2((uint32_t)tile * (CPT / 2) + (uint32_t)(seq >> 1), seq & 1, n2);
                    c = cconj(expmi_pi((uint32_t)((2ull * j * k2) & ((2ull << g.log_n) - 1)), g.log_n));
                    wbase = unit_root<+1>(j % NSL, NSL * RL);
                } else {
                    c = cconj(cmul(u1[seq * U1N + j % U1D], u2[seq * U2N + j / U1D]));
                    wbase = tws[TB::ls(q) * NT + t];
                }
                twiddle_powers<RL, true>(&x[q * RL], wbase, c);
                dft<RL, +1>(reinterpret_cast<float2(&)[RL]>(x[q * RL]));
#pragma unroll
                for (int r = 0; r < RL; ++r) x[q * RL + r] = cmul(x[q * RL + r], sigma[seq * RL + r]);
            }
            float4* Z4 = reinterpret_cast<float4*>(Z + ((size_t)blk << g.log_n)) + (size_t)tile * L * (CPT / 2);  // [m1][CPT/2]
            if (DIRECT) {  // thread holds column 0 (x[0..RL)) and column 1 (x[RL..2RL)) of rows j + NSL r
#pragma unroll
                for (int r = 0; r < RL; ++r)
                    __stcg(Z4 + t + NSL * r, make_float4(x[r].x, x[r].y, x[RL + r].x, x[RL + r].y));
                continue;
            }
            __syncthreads();
            scatter_outputs<L, SP, E, RL, Lin>(x, sm);
            __syncthreads();
#pragma unroll 4
            for (int i = 0; i < L * CPT / 2 / NT; ++i) {
                int idx = t + i * NT, m1 = idx / (CPT / 2), cp = idx % (CPT / 2);
                float2 a = sm[(2 * cp) * SP + padk<4>(m1)], b = sm[(2 * cp + 1) * SP + padk<4>(m1)];
                __stcg(Z4 + idx, make_float4(a.x, a.y, b.x, b.y));
            }
        }  // part
    }  // unit
    // every wait is behind: the barriers may be initialised again by a later call in the same CTA
    __syncthreads();
    if (t == 0) {
        mbar_inval(&bar);
        mbar_inval(&bar_early);
        mbar_inval(&bar_spec);
    }
}

// ============================================================================ pass C
// Row m1: inverse FFT over k2 (radices 16, RB, RA), + correction, round, parity bit planes.
// Input: Z, tile-major from pass B.  Row m1 is the CPT/2 pairs of row m1 of every tile; 3D TMA boxes
// (256 tiles x 1 row x CPT/2 pairs) gather it into shared memory in pair order (float4 p = pair p),
// or cooperative loads when a tile row is too wide for a box.  Shared memory holds [row boxes 0 ..
// early-1][exchange buffer], so a row occupies the first `early` boxes' own space and the start of the
// exchange buffer.  The next row's first `early` boxes are gathered as soon as the current row has been
// read into registers (issued after the first exchange's barrier, so they land under the rest of the
// row's transform); the rest as soon as the last exchange has finished with the buffer.  `early` is as
// many boxes as shared memory holds (all of them for rows up to 2^13; 19 of 32 for rows of 2^14 with
// v = 3n/8).  Every warp issues its share of the boxes.  The parity words of a row are staged in
// shared memory and written out with coalesced stores at the next row's start.
// KEEP8: the last stage's outputs r < KEEP8 * RL / 8 (samples m2 = j + NSL r) are the only ones that can
// fall below out_bits; the others are neither rounded nor stored, and the compiler drops their share of
// the last radix stage.  Their plane words keep whatever the buffer held: k_finish never reads a word
// past out_bits.
// BNT: threads of the pass B that wrote Z (its tile width is 32 BNT / N1 columns).  The CTA takes rows
// first, first + stride, ... (the kernel: blockIdx.x, gridDim.x).  blockIdx.y is the block of a group (0
// otherwise): mapZ holds the group's blocks one after another, ntiles tiles each.
template <int LOGL, int KEEP8, int BNT>
__device__ __forceinline__ void pass_c_rows(const CUtensorMap* mapZ, const float2* __restrict__ Z, const BlockGeom& g,
                                            const unsigned long long* cnt, uint32_t* __restrict__ planes,
                                            unsigned int* resid_bits, int* err, int early, uint32_t first,
                                            uint32_t stride) {
    constexpr int L = 1 << LOGL, NT = L / 32, E = 32, LR = L / 16, SP = TileStride<L>::value;
    using P = Plan<LOGL>;
    using Lin = MapLinear<NT>;
    constexpr int RL = P::RA, NSL = L / RL;
    constexpr int KR = KEEP8 * RL / 8;
    static_assert(KEEP8 >= 1 && KEEP8 <= 8 && KR * 8 == KEEP8 * RL, "KEEP8 must split the last radix evenly");
    constexpr int QL = E / RL;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ float2 tws[QL][NT];  // last-stage per-thread twiddle bases (the second stage reads tab2)
    __shared__ float2 tab2[P::NSTAGE == 2 ? P::RB * 16 : 1];  // second-stage twiddles
    __shared__ float redf[32];
    __shared__ __align__(8) uint64_t bar, bar_late;  // TMA completion: boxes [0, early), [early, nb)
    // Parity words of a row (the KR * NSL / 32 live words of each plane), double-buffered by row: lane 0
    // of each warp writes its ballots here, and every thread copies the previous row's words out with
    // coalesced stores after the next row's first barrier.
    constexpr int PW = KR * NSL / 32;
    __shared__ uint32_t pstage[2][2][PW];
    __shared__ int s_fail;
    const uint32_t n1 = 1u << g.log_n1;
    const int cpt = (32 * BNT) >> g.log_n1;         // pass B tile width (columns)
    const int pairs_per_tile = cpt / 2;
    const int ntiles = (int)(L / cpt);
    const bool tma = cpt <= 128;
    const int boxt = ntiles < 256 ? ntiles : 256;   // tiles per box
    const int nb = ntiles / boxt;                   // boxes per row
    if (!tma) early = 0;
    float2* srow = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float2* sm = srow + (size_t)early * boxt * cpt;  // exchange buffer
    const int t = threadIdx.x, lane = t & 31;
    {
        float2 w[4];
        if (P::NSTAGE == 2) stage_bases<L, RL, 16 * P::RB, +1, E, Lin>(w);
        else stage_bases<L, RL, 16, +1, E, Lin>(w);
#pragma unroll
        for (int q = 0; q < QL; ++q) tws[q][t] = w[q];
        if (P::NSTAGE == 2) fill_stage_table<P::RB, 16, +1>(tab2);
    }
    float corr;
    {
        unsigned long long ck = cnt[0], cs = cnt[1];
        unsigned long long pm = (ck * cs) & ((2ull << g.log_np) - 1ull);
        corr = (float)((double)pm / (double)(1ull << g.log_np));
    }
    // rows holding at least one output sample: m1 < min(N1, ceil(out_bits / 2))
    const uint32_t rows_out = (uint32_t)(((uint64_t)g.out_bits + 1ull) / 2ull < n1 ? (g.out_bits + 1u) / 2u : n1);
    const uint32_t box_bytes = (uint32_t)(boxt * cpt * sizeof(float2));
    // Boxes [b0, b1) of row r, called by every thread: thread 0 announces the bytes, and lane 0 of
    // each warp issues every (NT/32)-th box, so no single warp is held up issuing a row's copies.
    // A copy that lands before the announcement cannot complete the phase: its arrival is pending.
    auto issue_boxes = [&](uint32_t r, int b0, int b1, uint64_t* bb) {
        if (r >= rows_out || b0 >= b1) return;
        if (t == 0) mbar_expect_tx(bb, (uint32_t)(b1 - b0) * box_bytes);
        if (lane == 0) {
#pragma unroll 1
            for (int b = b0 + (t >> 5); b < b1; b += NT / 32)
                tma_load_3d(srow + (size_t)b * boxt * cpt, mapZ, 0, (int)r, (int)blockIdx.y * ntiles + boxt * b, bb);
        }
    };
    auto load_early = [&](uint32_t r) {  // boxes [0, early) of row r (TMA only)
        if (early > 0) issue_boxes(r, 0, early, &bar);
    };
    auto load_late = [&](uint32_t r) {  // boxes [early, nb) of row r, or the whole row by cooperative loads
        if (r >= rows_out) return;
        if (tma) {
            issue_boxes(r, early, nb, &bar_late);
        } else {
            const float4* z4 = reinterpret_cast<const float4*>(Z);
            float4* s4 = reinterpret_cast<float4*>(srow);
            for (int p = t; p < L / 2; p += NT) {
                int tl = p / pairs_per_tile, cp = p % pairs_per_tile;
                s4[p] = __ldcs(z4 + ((size_t)tl * n1 + r) * pairs_per_tile + cp);
            }
        }
    };
    auto wait_bar = [&](uint64_t* b, uint32_t& parity) {
        if (!s_fail && !mbar_wait(b, parity)) {
            s_fail = 1;
            atomicExch(err, kErrTmaTimeout);
        }
        parity ^= 1u;
    };
    uint32_t parity = 0, parity_late = 0;
    if (t == 0) {
        s_fail = 0;
        mbar_init(&bar, 1);
        mbar_init(&bar_late, 1);
    }
    __syncthreads();
    const size_t plane_words = (size_t)n1 * (L / 32);
    // rows without output samples: zero planes
    for (uint32_t m1 = rows_out + first; m1 < n1; m1 += stride)
        for (int w = t; w < L / 32; w += NT) planes[(size_t)m1 * (L / 32) + w] = planes[plane_words + (size_t)m1 * (L / 32) + w] = 0u;
    fence_proxy_async();
    load_early(first);
    load_late(first);
    float res = 0.f;
    auto flush = [&](uint32_t row, int b) {  // staged parity words of `row` (buffer b) to the planes
        uint32_t* dst = planes + (size_t)row * (L / 32);
        for (int i = t; i < 2 * PW; i += NT)
            dst[(i >= PW ? plane_words : 0) + (size_t)(i % PW)] = pstage[b][i / PW][i % PW];
    };
    int pb = 0;
    for (uint32_t m1 = first; m1 < rows_out; m1 += stride, pb ^= 1) {
        if (tma) {
            if (early > 0) wait_bar(&bar, parity);
            if (early < nb) wait_bar(&bar_late, parity_late);
        }
        __syncthreads();  // row in shared memory; the previous row's parity words staged
        if (m1 != first) flush(m1 - stride, pb ^ 1);
        float2 x[E];
        const float4* row4 = reinterpret_cast<const float4*>(srow);
        if (t != 0) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float4 a = row4[t + LR * r], b = row4[(LR - t) + LR * r];
                x[r] = make_float2(a.x, a.y);
                x[16 + 15 - r] = make_float2(a.z, a.w);
                x[16 + r] = make_float2(b.x, b.y);
                x[15 - r] = make_float2(b.z, b.w);
            }
        } else {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float4 a = row4[LR * r], b = row4[LR / 2 + LR * r];
                x[r] = make_float2(a.x, a.y);
                x[r == 0 ? 8 : 16 - r] = make_float2(a.z, a.w);
                x[16 + r] = make_float2(b.x, b.y);
                x[16 + 15 - r] = make_float2(b.z, b.w);
            }
        }
        stage<16, 1, +1, E>(x, nullptr);
        // after the first exchange's barrier every thread has read the row: the next row's own boxes
        // are gathered under the rest of this row's transform
        auto gather_early = [&]() {
            if (early > 0) {
                fence_proxy_async();
                load_early(m1 + stride);
            }
        };
        {
            float2 w[4];
            if (P::NSTAGE == 2) {
                exchange<L, SP, 4, E, 16, 1, MapMirrorRow, P::RB, Lin>(x, sm, gather_early);
                stage_tab<P::RB, 16, +1, E, L, Lin>(x, tab2);
                exchange<L, SP, 4, E, P::RB, 16, Lin, RL, Lin>(x, sm);
            } else {
                exchange<L, SP, 4, E, 16, 1, MapMirrorRow, RL, Lin>(x, sm, gather_early);
            }
            // the exchange buffer is free: the rest of the next row's copy runs under the last stage
            __syncthreads();
            fence_proxy_async();
            load_late(m1 + stride);
#pragma unroll
            for (int q = 0; q < QL; ++q) w[q] = tws[q][t];
            stage<RL, (P::NSTAGE == 2 ? 16 * P::RB : 16), +1, E>(x, w);
        }
        // outputs: butterfly u = t + q*NT (j = u), sample m2 = j + NSL*r; lanes hold consecutive m2.
        // Sample x = 2 (m1 + N1 m2) + tt is below out_bits iff m2 < lim[tt] = ceil((out_bits - 2 m1 - tt) / 2N1).
        const uint32_t two_m1 = 2u * m1, span = 2u << g.log_n1;
        const uint32_t lim0 = g.out_bits > two_m1 ? (g.out_bits - two_m1 + span - 1u) >> (g.log_n1 + 1) : 0u;
        const uint32_t lim1 = g.out_bits > two_m1 + 1u ? (g.out_bits - two_m1 - 1u + span - 1u) >> (g.log_n1 + 1) : 0u;
#pragma unroll
        for (int q = 0; q < QL; ++q) {
            const int j = t + q * NT;
#pragma unroll
            for (int r = 0; r < KR; ++r) {
                const uint32_t m2 = (uint32_t)(j + NSL * r);
                const float2 v = x[q * RL + r];
                const float v0 = v.x + corr, v1 = v.y + corr;
                const float r0 = rintf(v0), r1 = rintf(v1);
                const bool ok0 = m2 < lim0, ok1 = m2 < lim1;
                if (ok0) res = fmaxf(res, fabsf(v0 - r0));
                if (ok1) res = fmaxf(res, fabsf(v1 - r1));
                const uint32_t be = __ballot_sync(0xffffffffu, ok0 && ((int)r0 & 1));
                const uint32_t bo = __ballot_sync(0xffffffffu, ok1 && ((int)r1 & 1));
                if (lane == 0) {
                    pstage[pb][0][m2 >> 5] = be;
                    pstage[pb][1][m2 >> 5] = bo;
                }
            }
        }
        if (!tma) __syncthreads();  // cooperative loads of the next row happen at the top
    }
    // the last row's parity words (the barrier orders them after every warp's ballots)
    __syncthreads();
    {
        const uint32_t nrows = rows_out > first ? (rows_out - first + stride - 1) / stride : 0;
        if (nrows > 0) flush(first + (nrows - 1) * stride, (int)((nrows - 1) & 1));
    }
    float bm = block_max_f(res, redf);  // its barriers follow every thread's last wait
    if (threadIdx.x == 0) {
        atomicMax(resid_bits, __float_as_uint(bm));
        mbar_inval(&bar);
        mbar_inval(&bar_late);
    }
}

}  // namespace pa
