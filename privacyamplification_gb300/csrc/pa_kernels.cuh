// pa_kernels.cuh -- block geometry shared by the host engine and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pa {

// One privacy-amplification block, sizes in bits (nicoboss/PrivacyAmplification naming:
// sample_size n, vertical_len v, horizontal_len h; PrivacyAmplification.cu:1423-1430).
struct BlockGeom {
    uint32_t n, v, h;      // h = n - v
    uint32_t out_bits;     // v (do_compress) or n/2 (PrivacyAmplification.cu:1197)
    int log_np;            // cyclic length Np = 2^log_np >= n (== n when n is a power of two)
    int log_n;             // complex length N = Np/2
    int log_n1, log_n2;    // three-pass split N = N1 * N2 (0, 0 for the single-CTA path)
    uint32_t seed_direct;  // seed positions < seed_direct map to themselves (see seed_source)
    int exact_only;        // 1: beyond the FP32 path (n > 2^27), only the exact NTT path applies
};

// Seed placement in the cyclic length Np.  For Np == n this is the identity.  For a padded Np the
// outputs i < out_bits see exactly the reference's seed[(i-j) mod n] when
//   s'[x] = s[x]               for x < seed_direct = min(Np - h, n),
//   s'[x] = s[x - (Np - n)]    for x >= Np - h.
// Positions in between (present when n + h < Np) are read by no output i < out_bits; they are filled
// with seed bits s[(x - seed_direct) mod n] rather than zeros: a long run of zeros would give the placed
// seed large near-DC spectral coefficients and cost the FP32 path most of its rounding budget.  With the
// smallest Np (below 2n) the index x - seed_direct is already below n; a larger Np (the persistent lanes
// place every block in at least 2^20) needs the reduction, or the filler would read past the seed.
// A power-of-two n in a larger Np (the persistent lanes' smallest cyclic length) is placed periodically,
// s'[x] = s[x mod n]: Np is then a multiple of n, so every output sees s[(i-j) mod n] for any h, and one
// spectrum serves every v.
__host__ __device__ inline int seed_source(const BlockGeom& g, uint64_t x, uint64_t* src) {
    uint64_t np = 1ull << g.log_np;
    if ((g.n & (g.n - 1u)) == 0) { *src = x & (g.n - 1u); return 1; }
    if (x < g.seed_direct) { *src = x; return 1; }
    if (x >= np - g.h) { *src = x - (np - g.n); return 1; }
    uint64_t f = x - g.seed_direct;
    if (f >= g.n) f %= g.n;
    *src = f;
    return 1;
}

// Source word of the placed seed's word x0 / 32 (x0 a multiple of 32).  n, v and so h, Np - h, Np - n and
// seed_direct are multiples of 32 (the engine accepts no other sizes), so every boundary of the placement,
// and every wrap of the filler and of the periodic form, falls between words: a placed word is one whole
// source word, in the same MSB-first bit order.
__host__ __device__ inline uint64_t seed_word(const BlockGeom& g, uint64_t x0) {
    uint64_t s = 0;
    seed_source(g, x0, &s);
    return s >> 5;
}

}  // namespace pa

// Host launch API (pa_kernels.cu).  All launches are asynchronous on `stream`.
namespace pa {
// Seed spectrum (FP32, scaled by 1/(2Np)) in the layout the key path consumes.  work (N complex) and
// rows (Np/8 bytes) are scratch of the three-pass path.  cnt_seed receives the popcount of the
// placed seed.
struct PassMaps;
struct Scratch {
    float2* work;       // N complex: pass A output (row-major)
    float2* work2;      // N complex: pass B output (tile-major)
    uint32_t* planes;   // Np/8 bytes: input bit rows, then parity planes
    int* err;           // device error word (bounded waits)
    const PassMaps* maps;
};
int launch_seed_spectrum(const BlockGeom& g, const uint32_t* seed, float2* spec, const Scratch& sc,
                         unsigned long long* cnt_seed, int num_sms, cudaStream_t s);
// Key block: out_words receives ceil(out_bits/32) little-endian words of the reference byte stream.
// stage_ev (optional, kernel_count_key_block()+1 events) is recorded before the first kernel and
// after each stage.  key_rest_ready (optional): the stream waits on it before the first kernel that
// reads key_rest (k_finish, or the single-CTA kernel), so key_rest may still be arriving meanwhile.
int launch_key_block(const BlockGeom& g, const uint32_t* key_start, const uint32_t* key_rest, uint32_t flags,
                     const float2* spec, const Scratch& sc, unsigned long long* cnt, unsigned int* resid_bits,
                     uint32_t* out_words, int num_sms, cudaStream_t s, cudaEvent_t* stage_ev,
                     cudaEvent_t key_rest_ready = nullptr);
// A key block whose seed serves it alone, the seed's column transform fused into the key's column pass
// (fused_geom(g) only): seed_y (N complex values, where the spectrum would go) receives the seed's row
// pass, seed_maps are over seed_y, park holds park_ctas * kParkBytes; cnt[0] / cnt[1] receive the key and
// seed popcounts.  Otherwise as launch_key_block (the seed's bit rows and row pass time as stage 0).
int launch_fused_block(const BlockGeom& g, const uint32_t* seed, const uint32_t* key_start, const uint32_t* key_rest,
                       uint32_t flags, float2* seed_y, const PassMaps& seed_maps, float2* park, uint32_t park_ctas,
                       const Scratch& sc, unsigned long long* cnt, unsigned int* resid_bits, uint32_t* out_words,
                       int num_sms, cudaStream_t s, cudaEvent_t* stage_ev, cudaEvent_t key_rest_ready = nullptr);
int kernel_count_key_block(const BlockGeom& g);   // kernels one key block launches
int stage_count_key_block(const BlockGeom& g);    // timed stages (events - 1) of a key block

// Grouped launches: G blocks of one geometry run as one launch per pass (grid dimension y, or z for the
// two-dimensional transposes, is the block).  The group's working set is contiguous, block b's rows /
// planes, Y, Z and own spectrum at base + b * stride; what the caller owns comes from a table of
// entries in device memory.
struct GroupEntry {
    const uint32_t* key_start;
    const uint32_t* key_rest;
    const uint32_t* seed;                // the block's own seed words (a dynamic group), else null
    const float2* spec;                  // the spectrum the key pass multiplies by
    uint32_t* out;
    unsigned long long* cnt;             // [0] key, [1] seed popcount
    unsigned int* resid;                 // largest FP32 residual
    const unsigned long long* seed_cnt;  // popcount of a cached seed (a static group), else null
};
struct Group {
    const GroupEntry* e;  // null: one block, nothing offset
    uint32_t count;       // blocks
    size_t work;          // complex values per block in Y, Z and the group's own spectra
    size_t planes;        // words per block of bit rows / parity planes
};
constexpr Group kOneBlock{nullptr, 1, 0, 0};
// Zeroes each block's key popcount and residual word and copies a cached seed's popcount (or zero).
int launch_group_prep(const Group& gp, cudaStream_t s);
// The seed spectra of a dynamic group: block b's spectrum at spec + b * gp.work.
int launch_group_seed(const BlockGeom& g, const Group& gp, float2* spec, const Scratch& sc, int num_sms,
                      cudaStream_t s);
// The key blocks of a group (after launch_group_prep and, for a dynamic group, launch_group_seed).
int launch_group_key(const BlockGeom& g, const Group& gp, uint32_t flags, const Scratch& sc, int num_sms,
                     cudaStream_t s);
// The same for single-CTA geometries (n <= 2^15: one CTA per block; pa_kernels.cu).
int launch_group_mono_seed(const BlockGeom& g, const Group& gp, float2* spec, cudaStream_t s);
int launch_group_mono_key(const BlockGeom& g, const Group& gp, uint32_t flags, cudaStream_t s);

// Three-pass kernels (pa_passes.cu).  `rows` and the parity planes share one buffer of Np/8 bytes.
// With a group, the pointer arguments are the group's bases (rows, Y, Z, the own spectra) or are
// replaced by the entries (bits, key_rest, out, cnt, resid, the key pass's spectrum).
int launch_bit_rows(const BlockGeom& g, const uint32_t* bits, bool seed, uint32_t* rows, cudaStream_t s,
                    const Group& gp = kOneBlock);
int launch_pass_a(const BlockGeom& g, const uint32_t* rows, bool seed, float2* Y, unsigned long long* cnt,
                  int num_sms, cudaStream_t s, const Group& gp = kOneBlock);
struct PassMaps {
    CUtensorMap y;  // Y (pass A output, row-major) as read by pass B
    CUtensorMap z;  // Z (pass B output, tile-major) as read by pass C
};
int make_pass_maps(const BlockGeom& g, const float2* Y, const float2* Z, PassMaps* out);
// The maps of `blocks` consecutive blocks' Y and Z (a group's working set).
int make_group_maps(const BlockGeom& g, const float2* Y, const float2* Z, uint32_t blocks, PassMaps* out);
// The Y and Z maps (out[0], out[1]) for columns of 2^log_n1, rows of 2^log_n2, pass B tiles of cpt
// columns, over `blocks` consecutive blocks.
int encode_pass_maps(int log_n1, int log_n2, uint32_t cpt, const float2* Y, const float2* Z, CUtensorMap* out,
                     uint32_t blocks = 1);
int launch_pass_b(const BlockGeom& g, bool seed, const PassMaps& maps, float2* Y, float2* Z, float2* spec, int* err,
                  int num_sms, cudaStream_t s, const Group& gp = kOneBlock);
// A group's pass B with columns of 2^LOGL (pa_group.cu), grid and shared memory as launch_pass_b chose.
template <int LOGL>
int launch_pass_b_group(bool seed, dim3 grid, size_t smem, const CUtensorMap& mapY, float2* Y, float2* Z,
                        float2* spec, const BlockGeom& g, int* err, int early, const Group& gp, cudaStream_t s);
// The fused column pass of a block whose seed serves it alone (pa_fused.cu): seed_maps.y over the seed's
// row-pass output, maps.y over the key's; park: park_ctas * kParkBytes, one spectrum tile per CTA.
constexpr size_t kParkBytes = 8192 * sizeof(float2);
inline bool fused_geom(const BlockGeom& g) { return g.log_n1 >= 10 && g.log_n1 <= 12; }
int launch_pass_b_fused(const BlockGeom& g, const PassMaps& seed_maps, const PassMaps& maps, float2* Z, float2* park,
                        uint32_t park_ctas, int* err, int num_sms, cudaStream_t s);
template <int LOGL>
int launch_pass_b_fused_k(dim3 grid, size_t smem_base, size_t box, int max_early, const CUtensorMap& mapYs,
                          const CUtensorMap& mapY, float2* Z, const BlockGeom& g, float2* park, int* err,
                          cudaStream_t s);
int launch_pass_c(const BlockGeom& g, const PassMaps& maps, const float2* Z, const unsigned long long* cnt,
                  uint32_t* planes, unsigned int* resid, int* err, int num_sms, cudaStream_t s,
                  const Group& gp = kOneBlock);
int launch_finish(const BlockGeom& g, const uint32_t* planes, const uint32_t* key_rest, uint32_t flags,
                  uint32_t* out, cudaStream_t s, const Group& gp = kOneBlock);

// Exact path (pa_ntt.cu): integer convolution modulo 3*2^30+1.  seed_hat, a, tmp: Np words each.
struct NttTables;
void free_ntt_tables(NttTables* t);
int launch_exact_seed(const BlockGeom& g, const uint32_t* seed, uint32_t* seed_hat, uint32_t* tmp,
                      NttTables** tables, cudaStream_t s);
int launch_exact_block(const BlockGeom& g, const uint32_t* key_start, const uint32_t* key_rest, uint32_t flags,
                       const uint32_t* seed_hat, uint32_t* a, uint32_t* tmp, uint32_t* out_words, NttTables** tables,
                       cudaStream_t s);
int exact_kernel_count(const BlockGeom& g);

// Blocks beyond the single-pass FP32 size (pa_chunk.cu): side x side chunk blocks (n' = 2 side) on the
// FP32 path.  gc: geometry of a chunk block (n' = 2 side, v' = side, no flags).  staging:
// chunk_staging_words(g) words; spec / sc / cnt: the FP32 path's buffers for gc.  resid_bits receives
// the largest chunk residual.
constexpr int kChunkLog = 26;
struct ChunkPlan {
    uint32_t side, rows, cols, chunks, diagonals;
    uint32_t absorb;  // 1: key bit h = cols * side (alone past the last full column) rides in that column
};
ChunkPlan chunk_plan(const BlockGeom& g);
size_t chunk_staging_words(const BlockGeom& g);
int chunk_kernel_count(const BlockGeom& g, const BlockGeom& gc);
// A second lane for the chunk blocks: its own staging (chunk_lane_words(g) words), seed spectrum and
// three-pass buffers, and a stream; the diagonals alternate between the lanes, so one lane's short kernels
// and kernel tails overlap the other's work.  fork / join: events the lanes synchronise with.
struct ChunkLane {
    uint32_t* staging;
    float2* spec;
    Scratch sc;
    cudaStream_t s;
    cudaEvent_t fork, join;
};
size_t chunk_lane_words(const BlockGeom& g);
int launch_chunked_block(const BlockGeom& g, const BlockGeom& gc, const uint32_t* seed, const uint32_t* key_start,
                         const uint32_t* key_rest, uint32_t flags, uint32_t* out_words, uint32_t* staging,
                         float2* spec, const Scratch& sc, unsigned long long* cnt, unsigned int* resid_bits,
                         int num_sms, cudaStream_t s, const ChunkLane* lane2 = nullptr);
}  // namespace pa
