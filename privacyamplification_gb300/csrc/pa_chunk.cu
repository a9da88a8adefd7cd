// pa_chunk.cu -- blocks beyond the single-pass FP32 size (n > 2^27) as 2^27-bit FP32 chunk blocks.
//
// The block's result bit i (i < out_bits) is XOR_{j <= h} key_start[j] AND T[i - j] with
// T[m] = seed[m mod n], a linear Toeplitz product.  Rows i and key positions j are cut into chunks of
// side s = 2^26; chunk (a, b) is one key block of n' = 2s, v' = h' = s (no XOR, no compression) with
// key_start' = key_start[b s .. b s + s) followed by a zero bit and seed' = T[d s, d s + s) followed by
// T[d s - s, d s) for d = a - b -- the technique of the reference's examples/LargeBlocksizeExample
// (GetLocalSeed / GetLocalKey / XorWithRow, main.cpp:104-124), run on the device.  Chunks on one
// diagonal d share seed' and so one seed spectrum.  The kernels here move the chunk inputs and
// combine the chunk outputs; the chunk blocks themselves are the ordinary three-pass kernels.
#include "pa_kernels.cuh"

namespace pa {

namespace {

constexpr uint32_t kXorFlag = 1u;  // PA_FLAG_XOR_KEY_REST

// dst[i] = seed[(start + i) mod nw], i < count (whole 32-bit words; start may be negative).
__global__ void k_seed_window(uint32_t* __restrict__ dst, const uint32_t* __restrict__ seed, uint32_t nw,
                              long long start, uint32_t count) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        long long src = (start + (long long)i) % (long long)nw;
        if (src < 0) src += nw;
        dst[i] = __ldg(seed + src);
    }
}

// Key chunk: sw words of key_start from bit `first` (a multiple of 32), bits past h cleared, then one
// word whose first bit is the chunk's bit h' = s: zero, or with `extra` key bit first + s (= h, the one
// tap past the last full column).
__global__ void k_key_chunk(uint32_t* __restrict__ dst, const uint32_t* __restrict__ ks, unsigned long long first,
                            uint32_t sw, uint32_t h, uint32_t extra) {
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w <= sw; w += gridDim.x * blockDim.x) {
        const unsigned long long bit = first + 32ull * w;
        uint32_t v = 0u;
        if ((w < sw || extra) && bit <= h) {
            v = __ldg(ks + (bit >> 5));
            if (bit + 31 > h) v &= ~(0xFFFFFFFFu >> (uint32_t)(h - bit + 1));
        }
        dst[w] = v;
    }
}

__global__ void k_xor_rows(uint32_t* __restrict__ acc, const uint32_t* __restrict__ add, uint32_t words) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < words; i += gridDim.x * blockDim.x) acc[i] ^= add[i];
}

// Output words (reference byte-stream order) = accumulated rows (of both lanes, acc2 may be null) XOR
// key_rest (byte-swapped words).
__global__ void k_chunk_final(uint32_t* __restrict__ out, const uint32_t* __restrict__ acc,
                              const uint32_t* __restrict__ acc2, const uint32_t* __restrict__ key_rest, uint32_t words,
                              uint32_t v, uint32_t flags) {
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x) {
        uint32_t x = acc[w];
        if (acc2) x ^= acc2[w];
        if ((flags & kXorFlag) && 32ull * w < v) x ^= __byte_perm(__ldg(key_rest + w), 0, 0x0123);
        out[w] = x;
    }
}

__global__ void k_max_words(unsigned int* __restrict__ dst, const unsigned int* __restrict__ src, int count) {
    unsigned int m = 0u;
    for (int i = threadIdx.x; i < count; i += blockDim.x) m = max(m, src[i]);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(dst, m);
}

int grid_for(uint32_t items, int num_sms) {
    uint32_t b = (items + 255u) / 256u;
    const uint32_t cap = 4u * (uint32_t)num_sms;
    return (int)(b < 1u ? 1u : (b > cap ? cap : b));
}

}  // namespace

ChunkPlan chunk_plan(const BlockGeom& g) {
    ChunkPlan p;
    p.side = 1u << kChunkLog;
    p.rows = (g.out_bits + p.side - 1u) / p.side;
    p.cols = (uint32_t)(((uint64_t)g.h + 1u + p.side - 1u) / p.side);
    // A chunk block's key has h' + 1 = side + 1 positions, the last one zero: when the taps past the last
    // full column are exactly one (h = cols * side, e.g. v = 3n/8), that tap takes the last column's
    // spare position instead of a column of its own.  Its seed index (i - h) lies in the column's seed
    // window like every other tap's.
    p.absorb = 0;
    if (p.cols > 1 && ((uint64_t)g.h + 1u) % p.side == 1u) {
        p.cols -= 1;
        p.absorb = 1;
    }
    p.chunks = p.rows * p.cols;
    p.diagonals = p.rows + p.cols - 1u;
    return p;
}

size_t chunk_staging_words(const BlockGeom& g) {
    const ChunkPlan p = chunk_plan(g);
    const size_t sw = p.side / 32u;
    return 5 * sw + (size_t)p.rows * sw + p.chunks + 64;
}

// Second lane: seed window (2 sw), key chunk (2 sw), chunk output (sw), row accumulators (rows sw), its
// popcounts (4 words).
size_t chunk_lane_words(const BlockGeom& g) {
    const ChunkPlan p = chunk_plan(g);
    const size_t sw = p.side / 32u;
    return 5 * sw + (size_t)p.rows * sw + 64;
}

int chunk_kernel_count(const BlockGeom& g, const BlockGeom& gc) {
    const ChunkPlan p = chunk_plan(g);
    // per diagonal: 2 window copies + seed spectrum (3); per chunk: key chunk, key block, xor; then 2
    return (int)(p.diagonals * 5u + p.chunks * (2u + (uint32_t)kernel_count_key_block(gc)) + 2u);
}

int launch_chunked_block(const BlockGeom& g, const BlockGeom& gc, const uint32_t* seed, const uint32_t* key_start,
                         const uint32_t* key_rest, uint32_t flags, uint32_t* out_words, uint32_t* staging,
                         float2* spec, const Scratch& sc, unsigned long long* cnt, unsigned int* resid_bits,
                         int num_sms, cudaStream_t s, const ChunkLane* lane2) {
    const ChunkPlan p = chunk_plan(g);
    const uint32_t sw = p.side / 32u, nw = g.n / 32u;
    // Per lane: seed window (2 sw words), key chunk (sw + 1 words, 2 sw reserved), chunk output (sw),
    // row accumulators (rows * sw; each lane its own, combined at the end), popcounts.  The chunks'
    // residual words (one per chunk) are lane 0's.
    struct Lane {
        uint32_t *seedwin, *keyc, *cout, *acc;
        unsigned long long* cnt;
        float2* spec;
        const Scratch* sc;
        cudaStream_t s;
    } lanes[2];
    lanes[0] = {staging, staging + 2 * sw, staging + 4 * sw, staging + 5 * sw, cnt, spec, &sc, s};
    unsigned int* res = reinterpret_cast<unsigned int*>(staging + 5 * sw + (size_t)p.rows * sw);  // one per chunk
    const int nlanes = lane2 ? 2 : 1;
    if (lane2) {
        uint32_t* st = lane2->staging;
        lanes[1] = {st, st + 2 * sw, st + 4 * sw, st + 5 * sw,
                    reinterpret_cast<unsigned long long*>(st + 5 * sw + (size_t)p.rows * sw), lane2->spec, &lane2->sc,
                    lane2->s};
    }
    for (int l = 0; l < nlanes; ++l) {
        cudaError_t err = cudaMemsetAsync(lanes[l].acc, 0, (size_t)p.rows * sw * sizeof(uint32_t), s);
        if (err != cudaSuccess) return (int)err;
    }
    if (lane2) {  // the second lane starts once the inputs and both accumulators are ready
        cudaError_t err = cudaEventRecord(lane2->fork, s);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(lane2->s, lane2->fork, 0);
        if (err != cudaSuccess) return (int)err;
    }
    const int gw = grid_for(sw, num_sms);
    uint32_t idx = 0;
    int diag = 0;  // diagonals alternate between the lanes
    for (int d = -(int)(p.cols - 1); d < (int)p.rows; ++d) {
        const int a0 = d > 0 ? d : 0;
        const int a1 = (int)p.rows < (int)p.cols + d ? (int)p.rows : (int)p.cols + d;
        if (a0 >= a1) continue;
        const Lane& L = lanes[diag++ % nlanes];
        k_seed_window<<<gw, 256, 0, L.s>>>(L.seedwin, seed, nw, (long long)d * sw, sw);
        k_seed_window<<<gw, 256, 0, L.s>>>(L.seedwin + sw, seed, nw, (long long)(d - 1) * sw, sw);
        int rc = launch_seed_spectrum(gc, L.seedwin, L.spec, *L.sc, L.cnt + 1, num_sms, L.s);
        if (rc) return rc;
        for (int a = a0; a < a1; ++a) {
            const int b = a - d;
            const uint32_t extra = p.absorb && b == (int)p.cols - 1 ? 1u : 0u;
            k_key_chunk<<<gw, 256, 0, L.s>>>(L.keyc, key_start, (unsigned long long)b * p.side, sw, g.h, extra);
            rc = launch_key_block(gc, L.keyc, nullptr, 0u, L.spec, *L.sc, L.cnt, res + idx, L.cout, num_sms, L.s,
                                  nullptr);
            if (rc) return rc;
            k_xor_rows<<<gw, 256, 0, L.s>>>(L.acc + (size_t)a * sw, L.cout, sw);
            ++idx;
        }
    }
    if (lane2) {
        cudaError_t err = cudaEventRecord(lane2->join, lane2->s);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(s, lane2->join, 0);
        if (err != cudaSuccess) return (int)err;
    }
    cudaError_t err = cudaMemsetAsync(resid_bits, 0, sizeof(unsigned int), s);
    if (err != cudaSuccess) return (int)err;
    k_max_words<<<1, 256, 0, s>>>(resid_bits, res, (int)idx);
    const uint32_t owords = (g.out_bits + 31u) / 32u;
    k_chunk_final<<<grid_for(owords, num_sms), 256, 0, s>>>(out_words, lanes[0].acc, lane2 ? lanes[1].acc : nullptr,
                                                            key_rest, owords, g.v, flags);
    return (int)cudaGetLastError();
}

}  // namespace pa
