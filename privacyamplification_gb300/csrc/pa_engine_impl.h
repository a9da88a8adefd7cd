// pa_engine_impl.h -- the engine object behind the C ABI, shared by pa_engine.cu (single blocks) and
// pa_batch.cu (slot pool: batched and served blocks, seed-spectrum cache, split autotuner).
#pragma once
#include "../../include/pa_gb300.h"
#include "pa_kernels.cuh"

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <vector>

namespace pa_host {
struct Pool;  // pa_batch.cu
}

struct pa_engine {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // pa_process copies key_rest on `side` while the block's passes run; the finish waits on kr_ready
    cudaStream_t side = nullptr;
    cudaEvent_t kr_ready = nullptr, main_ready = nullptr;
    uint32_t max_n = 0;
    int cap_log_np = 0;  // largest cyclic length the buffers hold
    float residual_limit = 0.25f;
    // three-pass split: log2 of the row length N2 for each log2 N (0 = default rule)
    int8_t split[32] = {};
    // HBM working set
    uint32_t* d_key_start = nullptr;
    uint32_t* d_key_rest = nullptr;
    uint32_t* d_seed = nullptr;
    uint32_t* d_out = nullptr;
    float2* d_work = nullptr;   // pass A output (row-major)
    float2* d_work2 = nullptr;  // pass B output (tile-major)
    float2* d_spec = nullptr;
    int* d_err = nullptr;       // device error word of the bounded TMA waits
    uint32_t* d_exact_seed = nullptr;  // NTT of the placed seed (exact path), Np words
    pa::NttTables* ntt = nullptr;      // exact-path twiddle tables
    bool exact_valid = false;          // d_exact_seed matches the current seed for exact_geom
    bool last_exact = false;           // the last block ran on the exact path
    bool last_chunked = false;         // the last block ran as FP32 chunk blocks (n > 2^27)
    pa::BlockGeom exact_geom{};
    pa::PassMaps maps{};        // tensor maps for the geometry maps_key
    int maps_key = -1;
    // second lane of the chunk blocks (n > 2^27): tensor maps over the upper halves of d_work / d_work2,
    // its stream is `side`, and the events it forks and joins on
    pa::PassMaps lane_maps{};
    int lane_maps_key = -1;
    cudaEvent_t lane_fork = nullptr, lane_join = nullptr;
    // a seed that serves one block is transformed inside that block's column pass: its row pass output
    // goes to d_spec (tensor maps seed_maps), its spectrum tiles to park (park_ctas * kParkBytes)
    pa::PassMaps seed_maps{};
    int seed_maps_key = -1;
    float2* d_park = nullptr;
    uint32_t park_ctas = 0;
    uint32_t* d_planes = nullptr;
    unsigned long long* d_cnt = nullptr;  // [0] key popcount, [1] seed popcount
    unsigned int* d_resid = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // seed state
    bool seed_valid = false;
    uint32_t seed_n = 0;
    int64_t seed_left = 0;  // -1 = unlimited
    bool spec_valid = false;
    pa::BlockGeom spec_geom{};
    int last_cuda = 0;
    bool pending = false;  // device-form work queued and not yet synchronised
    // per-kernel timing ring (pa_set_timing / pa_stage_times)
    bool timing = false;
    std::vector<std::array<cudaEvent_t, 5>> tev;
    std::vector<int> tev_stages;
    size_t tev_next = 0, tev_count = 0;
    // slot pool (pa_batch.cu), created on first use
    pa_host::Pool* pool = nullptr;
};

namespace pa_host {

inline int ceil_log2(uint64_t x) {
    int l = 0;
    while ((1ull << l) < x) ++l;
    return l;
}

inline bool is_pow2(uint32_t x) { return x && !(x & (x - 1u)); }

inline int cuda_fail(pa_engine* e, cudaError_t err) {
    e->last_cuda = (int)err;
    return PA_ERR_CUDA;
}

#define PA_CUDA(e, call)                                      \
    do {                                                      \
        cudaError_t err__ = (call);                           \
        if (err__ != cudaSuccess) return pa_host::cuda_fail(e, err__); \
    } while (0)

// Row-length exponents the three-pass kernels are built for, for complex length 2^log_n:
// rows 2^10..2^14 (passes A, C) and columns 2^5..2^12 (pass B).
inline int split_min(int log_n) { return log_n - 12 > 10 ? log_n - 12 : 10; }
inline int split_max(int log_n) { return log_n - 5 < 14 ? log_n - 5 : 14; }
// Row length (log2) by default, from the autotuner's choices on GB300 one block after another: from
// N = 2^20 complex on, the shortest rows allowed (columns of 2^12, the longest pass B takes; rows of 2^14
// at N = 2^26); below that, rows of N / 64 (2^10 .. 2^13).
inline int split_default(int log_n) {
    if (log_n >= 20) return split_min(log_n);
    const int l = log_n - 6;
    return l < split_min(log_n) ? split_min(log_n) : (l > split_max(log_n) ? split_max(log_n) : l);
}

// Block geometry (sizes, padded cyclic length, three-pass split) for (n, v, flags); `split` is a
// per-log_n table of row exponents (0 entries and a null table mean the default).
int make_geom(uint32_t n, uint32_t v, uint32_t flags, const int8_t* split, pa::BlockGeom* g);
// Two geometries whose seed spectra are interchangeable (placement and layout).
bool same_seed_geom(const pa::BlockGeom& a, const pa::BlockGeom& b);
// Key used to cache tensor maps: (log_n, log_n2).
inline int maps_key(const pa::BlockGeom& g) { return g.log_n * 32 + g.log_n2; }

void pool_destroy(pa_engine* e);  // pa_batch.cu

}  // namespace pa_host
