// pa_lanes.cuh -- the persistent lane kernel: many blocks of different sizes in one launch.
//
// The grid (one 512-thread CTA per SM, launched cooperatively so that every CTA is resident) is cut
// into lanes of T CTAs.  A lane takes one block at a time and its T CTAs run the block's stages -- bit
// rows, pass A, pass B, pass C, finish (preceded by bit rows, pass A and pass B of the seed for a block
// that brings its own seed) -- each CTA taking every T-th row or tile, with a lane barrier between
// stages.  Blocks are taken longest first from one list by an atomic counter, so lanes stay balanced
// without a host-side schedule, and no lane waits on another.
//
// Geometry: rows (passes A and C) of N2 = 2^14 complex values, columns (pass B) of N1 = 2^5 .. 2^12, so
// the cyclic length Np = 4 N1 N2 runs from 2^20 to 2^27; smaller blocks are placed in Np = 2^20 (the
// seed placement of pa_kernels.cuh holds for any Np >= max(n, out_bits + h)).  Pass B runs 512 threads
// per tile (tile width 2^14 / N1 columns), so its spectra and Z layout differ from the per-pass kernels'.
//
// Every wait is bounded: a lane barrier that does not complete within its limit records
// kErrLaneTimeout in the lane's error word, and once a lane's error word is set its CTAs stop taking
// blocks; TMA waits inside the passes record kErrTmaTimeout as in the per-pass kernels.
#pragma once
#include "pa_kernels.cuh"

#include <cuda.h>
#include <stdint.h>

namespace pa {

constexpr int kLaneThreads = 512;
constexpr int kLaneLogRow = 14;                    // log2 N2
constexpr int kLaneMinLogN1 = 5, kLaneMaxLogN1 = 12;
constexpr int kLaneMinLogNp = kLaneLogRow + kLaneMinLogN1 + 1;  // 2^20
constexpr int kLaneMaxLogNp = kLaneLogRow + kLaneMaxLogN1 + 1;  // 2^27
constexpr int kLaneMaps = kLaneMaxLogN1 - kLaneMinLogN1 + 1;    // tensor-map pairs per lane
constexpr int kErrLaneTimeout = 2;

// One block of a lane launch (device memory).  key_start / seed / key_rest and out are device pointers
// or, for blocks served from host memory, host pointers the device can reach (HOSTIN below).
struct LaneJob {
    const uint32_t* key_start;           // n/32 words (null: spectrum build only)
    const uint32_t* key_rest;            // v/32 words, or null without PA_FLAG_XOR_KEY_REST
    const uint32_t* seed;                // own seed (n/32 words), or null with a cached spectrum
    const float2* spec;                  // cached spectrum in the lane layout (static seed)
    float2* spec_out;                    // spectrum build: pass B of the seed writes here, no key stages
    uint32_t* out;                       // ceil(out_bits / 32) words
    unsigned long long* cnt;             // [2] key, seed popcount (zeroed by the lane before the block)
    const unsigned long long* seed_cnt;  // popcount of a cached seed, copied into cnt[1]
    unsigned int* resid;                 // largest FP32 residual (zeroed by the lane before the block)
    BlockGeom g;
    uint32_t flags;
    uint32_t pad_;
};

// One request of the serving loop, in pinned host memory: the host fills `job` (its pointers are host
// pointers the device can reach, or device pointers) and publishes the request by raising the ring's
// tail; the lane that served it writes the statistics and then done = ticket + 1.
struct ServeSlot {
    LaneJob job;
    unsigned long long cnt[2];
    unsigned int resid;
    int err;
    unsigned long long done;
};

// Host-memory words of the serving loop.
struct ServeCtl {
    unsigned long long tail;  // requests published (tickets 0 .. tail-1)
    int stop;                 // the host asks the loop to end once every published request is taken
    int pad_;
};

struct LaneArgs {
    const LaneJob* jobs;
    uint32_t njobs;
    unsigned int* next;      // claim counter (zero before the launch)
    unsigned int* bar;       // per lane: arrivals at lane barriers (zero before the launch)
    int* slot;               // per lane: index of the lane's current block
    int* err;                // per lane: error word
    float2* work;            // lane l: work + l * work_stride (pass A output Y)
    float2* work2;           //         work2 + l * work_stride (pass B output Z)
    float2* spec;            //         spec + l * work_stride (a block's own seed spectrum)
    uint32_t* planes;        //         planes + l * planes_stride (bit rows, then parity planes)
    size_t work_stride, planes_stride;
    const CUtensorMap* maps; // [lane][log_n1 - kLaneMinLogN1][Y, Z]
    int T;                   // CTAs per lane
    int lanes;
    int early_b[kLaneMaps];  // pass B boxes copied ahead, per log_n1
    int early_c[kLaneMaps];  // pass C boxes copied ahead, per log_n1
    uint32_t wait_limit;     // lane-barrier poll rounds before giving up
    // serving loop (serve != 0): requests come from a ring of host slots instead of `jobs`
    int serve;
    ServeSlot* ring;                 // host memory, ring_size slots; ticket t uses slot t % ring_size
    uint32_t ring_size;
    ServeCtl* host;                  // host memory
    unsigned long long* claimed;     // device: tickets taken so far
    LaneJob* lane_job;               // device, two per lane (used in turn): requests being served
    unsigned long long* lane_stats;  // device, two per lane: cnt[2], resid word, ticket
    unsigned long long idle_ns;      // time without a request after which the loop ends by itself
    uint32_t* stage;                 // device, per lane: a served request's key_start, seed, key_rest
    size_t stage_stride;             // words per lane (3 * (Np / 32) for the largest Np)
};

// Host side (pa_lanes.cu).
size_t lane_smem_bytes();                                    // dynamic shared memory of the lane kernel
int lane_early_boxes(int log_n1, int pass, size_t dyn_bytes);  // pass 'b' or 'c'
int launch_lanes(const LaneArgs& a, int grid, size_t smem, cudaStream_t s);
constexpr int kLaneIdle = -2, kLaneExit = -1;  // slot values besides a job index
int make_lane_maps(const float2* Y, const float2* Z, CUtensorMap* out /* kLaneMaps * 2 */);
int lane_max_ctas(int* ctas);  // resident CTAs of the lane kernel on the current device

}  // namespace pa
