// pa_passes.cu -- the three-pass four-step FP32 convolution for N = N1 * N2 complex samples: one kernel
// launch per pass (bodies in pa_pass_bodies.cuh), the bit-row and finish transposes, and the launchers.
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
#include "pa_pass_bodies.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

namespace pa {

// ============================================================================ bit-plane transposes
// Input bit planes.  Warp (a, c): rows m1 = 16a .. 16a+15, columns m2 = 32c .. 32c+31 (lane = m2 - 32c).
// The lane's input word holds x = 2 N1 m2 + 32a + [0, 32), i.e. 16 (even, odd) pairs of rows
// 16a..16a+15; after the half-warp transpose, lane L of half h holds row 16a + L, columns
// 32c + 16h .. 32c + 16h + 15 -- one word of the row plane.
template <bool SEED>
__global__ void __launch_bounds__(256) k_bit_rows(const uint32_t* __restrict__ src, BlockGeom g,
                                                  uint32_t* __restrict__ rows, Group gp) {
    if (gp.e) {  // block blockIdx.z of a group
        src = SEED ? gp.e[blockIdx.z].seed : gp.e[blockIdx.z].key_start;
        rows += (size_t)blockIdx.z * gp.planes;
    }
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
    } else {  // padded placement: whole words
        v = __ldg(src + seed_word(g, x0));
    }
    const uint32_t w = transpose16x2(v, lane);
    rows[(size_t)(16u * a + (uint32_t)(lane & 15)) * (n2 / 16u) + 2u * c + (uint32_t)(lane >> 4)] = w;
}

// Tiled form for N1, N2 >= 256 (the large blocks): a CTA moves a 256 x 256 block of 2-bit elements,
// input rows m2 (16 words of 16 m1 each, 64-byte segments) into shared memory, half-warp 16 x 16
// transposes from there, and output rows m1 (16 words of 16 m2 each) back out -- every global access
// is a 64-byte run instead of one word per row.  Rows padded to 17 words keep the column reads of the
// transpose on distinct banks.  SEED with a padded Np: each word comes from its placed source word.
template <bool SEED>
__global__ void __launch_bounds__(256) k_bit_rows_tiled(const uint32_t* __restrict__ src, BlockGeom g,
                                                        uint32_t* __restrict__ rows, Group gp) {
    __shared__ uint32_t tile[256][17];  // [m2 - m20][a - a0], then [m1 - 16 a0][(m2 - m20) / 16]
    if (gp.e) {
        src = SEED ? gp.e[blockIdx.z].seed : gp.e[blockIdx.z].key_start;
        rows += (size_t)blockIdx.z * gp.planes;
    }
    const int t = threadIdx.x, lane = t & 31;
    const uint32_t win = (1u << g.log_n1) / 16u, wout = (1u << g.log_n2) / 16u;  // words per input / output row
    const uint32_t a0 = blockIdx.x * 16u, m20 = blockIdx.y * 256u;
    // all 16 loads of the thread are issued before the first is used: one memory round trip
    uint32_t v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int r = (t >> 4) + 16 * i, w = t & 15;
        const uint64_t word = (uint64_t)(m20 + (uint32_t)r) * win + a0 + (uint32_t)w;
        const uint64_t x0 = 32ull * word;  // first sample of the word
        if (SEED) v[i] = __ldg(src + ((1u << g.log_np) == g.n ? word : seed_word(g, x0)));
        else v[i] = x0 <= g.h ? __ldg(src + word) : 0u;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int r = (t >> 4) + 16 * i, w = t & 15;
        const uint64_t x0 = 32ull * ((uint64_t)(m20 + (uint32_t)r) * win + a0 + (uint32_t)w);
        if (!SEED && x0 <= g.h && x0 + 31 > g.h) v[i] &= ~(0xFFFFFFFFu >> (uint32_t)(g.h - x0 + 1));
        tile[r][w] = v[i];
    }
    __syncthreads();
    // half-warp hw takes 16 x 16 blocks (cb, w): input words of m2 = m20 + 16 cb + L, column a0 + w;
    // the results wait in registers until every input word is read, then reuse the tile (one tile per
    // CTA keeps the whole grid resident in one wave)
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int b = (t >> 4) + 16 * i, cb = b >> 4, w = b & 15, L = lane & 15;
        v[i] = transpose16x2(tile[16 * cb + L][w], lane);  // row m1 = 16 (a0 + w) + L
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int b = (t >> 4) + 16 * i, cb = b >> 4, w = b & 15, L = lane & 15;
        tile[16 * w + L][cb] = v[i];
    }
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
        const int r = (t >> 4) + 16 * i, w = t & 15;
        rows[(size_t)(16u * a0 + (uint32_t)r) * wout + m20 / 16u + (uint32_t)w] = tile[r][w];
    }
}

// The pass kernels take block blockIdx.y of a group: its slices of the working set and its entry.
template <int LOGL, bool SEED>
__global__ void __launch_bounds__((1 << LOGL) / 32, 1)
    k_pass_a(const uint32_t* __restrict__ rows, BlockGeom g, float2* __restrict__ Y, unsigned long long* cnt,
             Group gp) {
    if (gp.e) {
        rows += (size_t)blockIdx.y * gp.planes;
        Y += (size_t)blockIdx.y * gp.work;
        cnt = gp.e[blockIdx.y].cnt + (SEED ? 1 : 0);
    }
    pass_a_rows<LOGL>(rows, g, Y, cnt, blockIdx.x, gridDim.x);
}

// One block (a group's pass B is k_pass_b_group in pa_group.cu: pass B runs at the 128-register limit
// of two CTAs per SM, and this kernel keeps its pointers in the constant bank instead of registers).
template <int LOGL, bool SEED>
__global__ void __launch_bounds__(256, 2)
    k_pass_b(const __grid_constant__ CUtensorMap mapY, const float2* __restrict__ Y, float2* __restrict__ Z,
             BlockGeom g, float2* __restrict__ spec, int* err, int early) {
    pass_b_tiles<LOGL, SEED, 256>(&mapY, Y, Z, g, spec, err, early, blockIdx.x, gridDim.x);
}

template <int LOGL, int KEEP8>
__global__ void __launch_bounds__((1 << LOGL) / 32, 1)
    k_pass_c(const __grid_constant__ CUtensorMap mapZ, const float2* __restrict__ Z, BlockGeom g,
             const unsigned long long* cnt, uint32_t* __restrict__ planes, unsigned int* resid_bits, int* err,
             int early, Group gp) {
    if (gp.e) {  // (the body finds the block's tiles of mapZ from blockIdx.y)
        Z += (size_t)blockIdx.y * gp.work;
        cnt = gp.e[blockIdx.y].cnt;
        planes += (size_t)blockIdx.y * gp.planes;
        resid_bits = gp.e[blockIdx.y].resid;
    }
    pass_c_rows<LOGL, KEEP8, 256>(&mapZ, Z, g, cnt, planes, resid_bits, err, early, blockIdx.x, gridDim.x);
}

// ============================================================================ finish
// Warp (a, c): plane rows m1 = 32a + lane, plane word column c (m2 = 32c .. 32c+31).  Each lane packs
// its (even, odd) parities of 16 columns into 2-bit elements and a half-warp transpose turns them into
// output words: lane L of half h holds column 32c + L (+16 for the second word), samples
// m1 = 32a + 16h .. +15 -- output word ow = (m2 N1 + 32a + 16h)/16, bits in the reference byte order,
// XORed with key_rest word ow.
__global__ void __launch_bounds__(1024) k_finish(const uint32_t* __restrict__ planes, BlockGeom g,
                                                 const uint32_t* __restrict__ key_rest, uint32_t flags,
                                                 uint32_t* __restrict__ out, uint32_t nwords, Group gp) {
    if (gp.e) {  // block blockIdx.z of a group
        planes += (size_t)blockIdx.z * gp.planes;
        key_rest = gp.e[blockIdx.z].key_rest;
        out = gp.e[blockIdx.z].out;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const size_t plane_words = (size_t)n1 * wpr;
    const uint32_t a = blockIdx.x * 4u + (uint32_t)(warp & 3);
    const uint32_t c = blockIdx.y * 8u + (uint32_t)(warp >> 2);
    if (a >= n1 / 32u || c >= wpr) return;
    const size_t off = (size_t)(32u * a + (uint32_t)lane) * wpr + c;
    const uint32_t ve = __ldg(planes + off), vo = __ldg(planes + plane_words + off);
    const uint32_t lo = transpose16x2(msb_pairs(ve, vo), lane);
    const uint32_t hi = transpose16x2(msb_pairs(ve >> 16, vo >> 16), lane);
    const uint32_t L = (uint32_t)(lane & 15), h = (uint32_t)(lane >> 4);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint64_t m2 = 32ull * c + L + 16u * k;
        const uint64_t ow = (m2 * n1 + 32ull * a + 16ull * h) / 16ull;
        if (ow >= nwords) continue;
        uint32_t w = k ? hi : lo;
        if ((flags & kXor) && 32ull * ow < g.v) w ^= __ldg(key_rest + ow);
        out[ow] = __byte_perm(w, 0, 0x0123);
    }
}

// Tiled form for N1 >= 256: a CTA takes plane rows m1 = m10 .. m10+255 and plane word columns
// c0 .. c0+7 (m2 = 32 c0 .. 32 c0 + 255).  Plane words arrive as 32-byte row segments, the half-warp
// transposes of k_finish run on shared memory, and each m2 leaves as 16 consecutive output words
// (64 bytes), with key_rest read the same way.
__global__ void __launch_bounds__(256) k_finish_tiled(const uint32_t* __restrict__ planes, BlockGeom g,
                                                      const uint32_t* __restrict__ key_rest, uint32_t flags,
                                                      uint32_t* __restrict__ out, uint32_t nwords, Group gp) {
    __shared__ uint32_t se[256][9], so[256][9];  // [m1 - m10][c - c0], even / odd samples
    __shared__ uint32_t sw[256][17];             // [m2 - 32 c0][(m1 - m10) / 16]
    if (gp.e) {
        planes += (size_t)blockIdx.z * gp.planes;
        key_rest = gp.e[blockIdx.z].key_rest;
        out = gp.e[blockIdx.z].out;
    }
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const size_t plane_words = (size_t)n1 * wpr;
    const uint32_t m10 = blockIdx.x * 256u, c0 = blockIdx.y * 8u;
    // Every load of the thread (16 plane words, and the 16 key_rest words its output words XOR with) is
    // issued before the first is used: one memory round trip per CTA.
    uint32_t pv[16], kr[16];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = (t >> 3) + 32 * i, w = t & 7;
        const uint32_t c = c0 + (uint32_t)w;
        const size_t off = (size_t)(m10 + (uint32_t)r) * wpr + c;
        pv[2 * i] = c < wpr ? __ldg(planes + off) : 0u;
        pv[2 * i + 1] = c < wpr ? __ldg(planes + plane_words + off) : 0u;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int ml = (t >> 4) + 16 * i, j = t & 15;
        const uint64_t ow = ((32ull * c0 + (uint64_t)ml) * n1 + m10) / 16ull + (uint64_t)j;
        kr[i] = ((flags & kXor) && ow < nwords && 32ull * ow < g.v) ? __ldg(key_rest + ow) : 0u;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = (t >> 3) + 32 * i, w = t & 7;
        se[r][w] = pv[2 * i];
        so[r][w] = pv[2 * i + 1];
    }
    __syncthreads();
#pragma unroll 2
    for (int i = 0; i < 8; ++i) {
        const int u = warp + 8 * i, al = u >> 3, cl = u & 7;  // rows 32 al + lane, word column cl
        const uint32_t ve = se[32 * al + lane][cl], vo = so[32 * al + lane][cl];
        const uint32_t lo = transpose16x2(msb_pairs(ve, vo), lane);
        const uint32_t hi = transpose16x2(msb_pairs(ve >> 16, vo >> 16), lane);
        const int L = lane & 15, h = lane >> 4;
        sw[32 * cl + L][2 * al + h] = lo;        // m2 = 32 (c0 + cl) + L, rows m10 + 32 al + 16 h ...
        sw[32 * cl + 16 + L][2 * al + h] = hi;   // m2 + 16
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int ml = (t >> 4) + 16 * i, j = t & 15;
        const uint64_t ow = ((32ull * c0 + (uint64_t)ml) * n1 + m10) / 16ull + (uint64_t)j;
        if (ow < nwords) out[ow] = __byte_perm(sw[ml][j] ^ kr[i], 0, 0x0123);
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

// CTAs of `kernel` resident on one SM with `threads` threads and `smem` bytes of dynamic shared memory
// (its dynamic shared-memory attribute already set); 1 if the query fails.
template <class K>
static int resident_ctas(K kernel, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) {
        cudaGetLastError();
        return 1;
    }
    return n;
}

// CTAs per block of a (grouped) persistent pass: one wave of `per_wave` CTAs shared by the group's
// blocks, at least one and at most `units` (rows or tiles) per block.  One block: min(units, per_wave).
static int group_ctas(uint32_t units, int per_wave, const Group& gp) {
    const uint32_t share = ((uint32_t)per_wave + gp.count - 1u) / gp.count;
    return grid_units(units, (int)std::max<uint32_t>(1u, share));
}

int launch_bit_rows(const BlockGeom& g, const uint32_t* bits, bool seed, uint32_t* rows, cudaStream_t s,
                    const Group& gp) {
    const uint32_t n1 = 1u << g.log_n1, n2 = 1u << g.log_n2;
    if (n1 >= 256u && n2 >= 256u) {
        dim3 grid(n1 / 256u, n2 / 256u, gp.count);
        if (seed) k_bit_rows_tiled<true><<<grid, 256, 0, s>>>(bits, g, rows, gp);
        else k_bit_rows_tiled<false><<<grid, 256, 0, s>>>(bits, g, rows, gp);
        return (int)cudaGetLastError();
    }
    dim3 grid((n1 / 16u + 7u) / 8u, n2 / 32u, gp.count);
    if (seed) k_bit_rows<true><<<grid, 256, 0, s>>>(bits, g, rows, gp);
    else k_bit_rows<false><<<grid, 256, 0, s>>>(bits, g, rows, gp);
    return (int)cudaGetLastError();
}

template <int LOGL>
static int pass_a_l(const BlockGeom& g, const uint32_t* rows, bool seed, float2* Y, unsigned long long* cnt,
                    int num_sms, cudaStream_t s, const Group& gp) {
    constexpr int NT = (1 << LOGL) / 32;
    size_t smem = (size_t)TileStride<(1 << LOGL)>::value * sizeof(float2);
    // a wave is every SM times the CTAs one SM holds: one for rows of 2^14, several for shorter rows
    // (a row of 2^10 is one warp), so that short rows still fill the SMs
    auto go = [&](auto kernel) {
        smem_attr(kernel, smem);
        static const int per_sm = resident_ctas(kernel, NT, smem);
        const dim3 grid(group_ctas(1u << g.log_n1, num_sms * per_sm, gp), gp.count);
        kernel<<<grid, NT, smem, s>>>(rows, g, Y, cnt, gp);
    };
    if (seed) go(k_pass_a<LOGL, true>);
    else go(k_pass_a<LOGL, false>);
    return (int)cudaGetLastError();
}

// Pass B's shared memory without the early boxes: tile / exchange buffer, column tables, stage bases, and
// the alignment of the TMA destination.
template <int LOGL>
static constexpr size_t pass_b_smem() {
    constexpr int L = 1 << LOGL, CPT = 8192 / L, RL = Plan<LOGL>::RA, NSL = L / RL;
    constexpr bool LEAN = LOGL <= 6;
    constexpr int U1N = LEAN ? 0 : (NSL < 16 ? NSL : 16), U2N = LEAN ? 0 : NSL / U1N;
    constexpr size_t words = (size_t)CPT * TileStride<L>::value + (size_t)CPT * (RL + U1N + U2N) +
                             (size_t)PassBBases<LOGL, 256>::SLOTS * 256;
    static_assert(words * sizeof(float2) + 128 <= 112 * 1024, "pass B tile too large for two CTAs per SM");
    return words * sizeof(float2) + 128;
}

template <int LOGL>
static int pass_b_l(const BlockGeom& g, bool seed, const PassMaps& maps, float2* Y, float2* Z, float2* spec,
                    int* err, int num_sms, cudaStream_t s, const Group& gp) {
    constexpr int L = 1 << LOGL, CPT = 8192 / L;
    const size_t smem = pass_b_smem<LOGL>();
    // a group's CTAs walk all its blocks' tiles (one dimension); one block's walk its own
    const dim3 grid(grid_units(((1u << g.log_n2) / CPT) * gp.count, 2 * num_sms));
    // As many of the next tile's boxes as fit beside the tile while two CTAs stay resident per SM.
    constexpr int BOXR = L < 256 ? L : 256;
    const size_t box = (size_t)BOXR * CPT * sizeof(float2);
    auto early_boxes = [&](auto kernel) {
        int e = CPT <= 128 ? L / BOXR : 0;
        for (; e > 0; --e) {
            int per_sm = 0;
            const size_t bytes = smem + (size_t)e * box;
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
                    cudaSuccess &&
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, bytes) == cudaSuccess &&
                per_sm >= 2)
                break;
        }
        cudaGetLastError();  // a refused attribute above is not an error of this launch
        return e;
    };
    static const int early_seed = early_boxes(k_pass_b<LOGL, true>);
    static const int early_key = early_boxes(k_pass_b<LOGL, false>);
    const int early = seed ? early_seed : early_key;
    const size_t bytes = smem + (size_t)early * box;
    if (gp.e) return launch_pass_b_group<LOGL>(seed, grid, bytes, maps.y, Y, Z, spec, g, err, early, gp, s);
    if (seed) {
        smem_attr(k_pass_b<LOGL, true>, bytes);
        k_pass_b<LOGL, true><<<grid, 256, bytes, s>>>(maps.y, Y, Z, g, spec, err, early);
    } else {
        smem_attr(k_pass_b<LOGL, false>, bytes);
        k_pass_b<LOGL, false><<<grid, 256, bytes, s>>>(maps.y, Y, Z, g, spec, err, early);
    }
    return (int)cudaGetLastError();
}

// Per-block shared memory limit of the current device (opt-in maximum).
static size_t smem_optin_limit() {
    static const size_t limit = [] {
        int dev = 0, optin = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            return (size_t)0;
        return (size_t)optin;
    }();
    return limit;
}

// Boxes of a pass C row that fit in shared memory beside the exchange buffer and the kernel's static
// arrays (see k_pass_c); 0 for cooperative row loads or when the kernel's attributes are unknown.
static int pass_c_early(const BlockGeom& g, int logl, size_t exch_bytes, size_t static_bytes) {
    const uint32_t cpt = 8192u >> g.log_n1;
    if (cpt > 128u || static_bytes == 0) return 0;
    const uint32_t ntiles = (1u << logl) / cpt, boxt = ntiles < 256u ? ntiles : 256u;
    const size_t box_bytes = (size_t)boxt * cpt * sizeof(float2), nb = ntiles / boxt;
    const size_t limit = smem_optin_limit(), used = exch_bytes + static_bytes + 1024;  // 1 KB margin
    if (limit <= used) return 0;
    return (int)std::min<size_t>(nb, (limit - used) / box_bytes);
}

template <int LOGL, int KEEP8>
static int pass_c_k(const BlockGeom& g, const PassMaps& maps, const float2* Z, const unsigned long long* cnt,
                    uint32_t* planes, unsigned int* resid, int* err, int num_sms, cudaStream_t s, const Group& gp) {
    constexpr int NT = (1 << LOGL) / 32;
    const size_t exch = (size_t)TileStride<(1 << LOGL)>::value * sizeof(float2) + 128;  // + TMA alignment
    static const size_t static_bytes = [] {  // the kernel's own __shared__ arrays
        cudaFuncAttributes fa{};
        return cudaFuncGetAttributes(&fa, k_pass_c<LOGL, KEEP8>) == cudaSuccess ? (size_t)fa.sharedSizeBytes
                                                                                 : (size_t)0;
    }();
    const int early = pass_c_early(g, LOGL, exch, static_bytes);
    const uint32_t cpt = 8192u >> g.log_n1, ntiles = (1u << LOGL) / cpt;
    const size_t box_bytes = (size_t)(ntiles < 256u ? ntiles : 256u) * cpt * sizeof(float2);
    const size_t smem = exch + (size_t)early * box_bytes;
    smem_attr(k_pass_c<LOGL, KEEP8>, smem);
    const int per_sm = resident_ctas(k_pass_c<LOGL, KEEP8>, NT, smem);  // smem depends on the geometry
    const dim3 grid(group_ctas(1u << g.log_n1, num_sms * per_sm, gp), gp.count);
    k_pass_c<LOGL, KEEP8><<<grid, NT, smem, s>>>(maps.z, Z, g, cnt, planes, resid, err, early, gp);
    return (int)cudaGetLastError();
}

// Eighths of the last stage's outputs that hold samples below out_bits: samples m2 < ceil(out_bits / 2N1)
// of every row, in last-stage output groups of NSL.
static int pass_c_keep8(const BlockGeom& g, int rl) {
    const uint64_t lim = ((uint64_t)g.out_bits + (2ull << g.log_n1) - 1ull) >> (g.log_n1 + 1);
    const uint64_t nsl = (1ull << g.log_n2) / (uint64_t)rl;
    const uint64_t live = (lim + nsl - 1ull) / nsl;  // last-stage outputs r < live
    return (int)((live * 8ull + (uint64_t)rl - 1ull) / (uint64_t)rl);
}

// Long rows (the large blocks) have variants for 2/8, 3/8 (v = 3n/8) and 4/8 (n/2 outputs); short rows
// and every other ratio run the full last stage.
template <int LOGL>
static int pass_c_l(const BlockGeom& g, const PassMaps& maps, const float2* Z, const unsigned long long* cnt,
                    uint32_t* planes, unsigned int* resid, int* err, int num_sms, cudaStream_t s, const Group& gp) {
    const int k8 = pass_c_keep8(g, Plan<LOGL>::RA);
    if constexpr (LOGL >= 12) {
        if (k8 <= 2) return pass_c_k<LOGL, 2>(g, maps, Z, cnt, planes, resid, err, num_sms, s, gp);
        if (k8 == 3) return pass_c_k<LOGL, 3>(g, maps, Z, cnt, planes, resid, err, num_sms, s, gp);
        if (k8 == 4) return pass_c_k<LOGL, 4>(g, maps, Z, cnt, planes, resid, err, num_sms, s, gp);
    }
    return pass_c_k<LOGL, 8>(g, maps, Z, cnt, planes, resid, err, num_sms, s, gp);
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
                  int num_sms, cudaStream_t s, const Group& gp) {
#define C(LG) pass_a_l<LG>(g, rows, seed, Y, cnt, num_sms, s, gp)
    PA_ROWS_DISPATCH(g.log_n2, C)
#undef C
}

int launch_pass_b(const BlockGeom& g, bool seed, const PassMaps& maps, float2* Y, float2* Z, float2* spec, int* err,
                  int num_sms, cudaStream_t s, const Group& gp) {
#define C(LG) pass_b_l<LG>(g, seed, maps, Y, Z, spec, err, num_sms, s, gp)
    PA_COLS_DISPATCH(g.log_n1, C)
#undef C
}

template <int LOGL>
static int pass_b_fused_l(const BlockGeom& g, const PassMaps& seed_maps, const PassMaps& maps, float2* Z,
                          float2* park, uint32_t park_ctas, int* err, int num_sms, cudaStream_t s) {
    constexpr int L = 1 << LOGL, CPT = 8192 / L, BOXR = L < 256 ? L : 256;
    static_assert(CPT * L * sizeof(float2) == kParkBytes, "a parked spectrum tile is one pass B tile");
    const int grid = std::min(grid_units((1u << g.log_n2) / CPT, 2 * num_sms), (int)park_ctas);
    if (grid < 1) return (int)cudaErrorInvalidValue;
    return launch_pass_b_fused_k<LOGL>(dim3(grid), pass_b_smem<LOGL>(), (size_t)BOXR * CPT * sizeof(float2),
                                       L / BOXR, seed_maps.y, maps.y, Z, g, park, err, s);
}

int launch_pass_b_fused(const BlockGeom& g, const PassMaps& seed_maps, const PassMaps& maps, float2* Z, float2* park,
                        uint32_t park_ctas, int* err, int num_sms, cudaStream_t s) {
    switch (g.log_n1) {
        case 10: return pass_b_fused_l<10>(g, seed_maps, maps, Z, park, park_ctas, err, num_sms, s);
        case 11: return pass_b_fused_l<11>(g, seed_maps, maps, Z, park, park_ctas, err, num_sms, s);
        case 12: return pass_b_fused_l<12>(g, seed_maps, maps, Z, park, park_ctas, err, num_sms, s);
        default: return (int)cudaErrorInvalidValue;
    }
}

int launch_pass_c(const BlockGeom& g, const PassMaps& maps, const float2* Z, const unsigned long long* cnt,
                  uint32_t* planes, unsigned int* resid, int* err, int num_sms, cudaStream_t s, const Group& gp) {
#define C(LG) pass_c_l<LG>(g, maps, Z, cnt, planes, resid, err, num_sms, s, gp)
    PA_ROWS_DISPATCH(g.log_n2, C)
#undef C
}

// Tensor maps of the two strided transfers of a three-pass block with columns of 2^log_n1, rows of
// 2^log_n2 and pass B tiles of cpt columns (see pass_b_tiles / pass_c_rows).  cuTensorMapEncodeTiled is
// taken from the driver through the runtime, so the library does not link libcuda.
int encode_pass_maps(int log_n1, int log_n2, uint32_t cpt, const float2* Y, const float2* Z, CUtensorMap* out,
                     uint32_t blocks) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return (int)cudaErrorNotSupported;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const uint64_t n1 = 1ull << log_n1, n2 = 1ull << log_n2;
    const cuuint32_t estr[3] = {1, 1, 1};
    {   // Y: rows of 2 N2 floats (N1 per block); box = 2 cpt floats x min(N1, 256) rows
        const cuuint64_t dims[2] = {2 * n2, n1 * blocks};
        const cuuint64_t strides[1] = {2 * n2 * sizeof(float)};
        const cuuint32_t box[2] = {(cuuint32_t)(2 * cpt), (cuuint32_t)(n1 < 256 ? n1 : 256)};
        CUresult r = encode(&out[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(Y), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return (int)cudaErrorInvalidValue;
    }
    {   // Z: [tile][m1][2 cpt floats] (ntiles per block); box = 2 cpt floats x 1 row x min(ntiles, 256) tiles
        const uint64_t ntiles = n2 / cpt;
        const cuuint64_t dims[3] = {2 * cpt, n1, ntiles * blocks};
        const cuuint64_t strides[2] = {2 * cpt * sizeof(float), n1 * 2 * cpt * sizeof(float)};
        const cuuint32_t box[3] = {(cuuint32_t)(2 * cpt), 1, (cuuint32_t)(ntiles < 256 ? ntiles : 256)};
        CUresult r = encode(&out[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(Z), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return (int)cudaErrorInvalidValue;
    }
    return 0;
}

// The per-pass kernels' maps (pass B with 256 threads: tiles of 8192 / N1 columns).
int make_pass_maps(const BlockGeom& g, const float2* Y, const float2* Z, PassMaps* out) {
    return make_group_maps(g, Y, Z, 1, out);
}

int make_group_maps(const BlockGeom& g, const float2* Y, const float2* Z, uint32_t blocks, PassMaps* out) {
    std::memset(out, 0, sizeof(*out));
    if (g.log_n1 == 0) return 0;
    const uint64_t cpt = 8192ull >> g.log_n1;
    if (cpt > 128) return 0;  // transfers use per-thread copies instead
    CUtensorMap m[2];
    int rc = encode_pass_maps(g.log_n1, g.log_n2, (uint32_t)cpt, Y, Z, m, blocks);
    if (rc) return rc;
    out->y = m[0];
    out->z = m[1];
    return 0;
}

int launch_finish(const BlockGeom& g, const uint32_t* planes, const uint32_t* key_rest, uint32_t flags,
                  uint32_t* out, cudaStream_t s, const Group& gp) {
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const uint32_t nwords = (g.out_bits + 31u) / 32u;
    // only plane columns that hold output samples: m2 < ceil(out_bits / (2 N1))
    const uint32_t m2max = (uint32_t)(((uint64_t)g.out_bits + 2ull * n1 - 1ull) / (2ull * n1));
    const uint32_t cols = std::min<uint32_t>(wpr, (m2max + 31u) / 32u);
    if (n1 >= 256u) {
        dim3 grid(n1 / 256u, (cols + 7u) / 8u, gp.count);
        k_finish_tiled<<<grid, 256, 0, s>>>(planes, g, key_rest, flags, out, nwords, gp);
        return (int)cudaGetLastError();
    }
    dim3 grid((n1 / 32u + 3u) / 4u, (cols + 7u) / 8u, gp.count);
    k_finish<<<grid, 1024, 0, s>>>(planes, g, key_rest, flags, out, nwords, gp);
    return (int)cudaGetLastError();
}

}  // namespace pa
