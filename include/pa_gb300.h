/*
 * pa_gb300.h -- C ABI of the GB300 privacy-amplification engine (libpa_gb300.so).
 *
 * Drop-in for the per-block GPU body of nicoboss/PrivacyAmplification's host loop
 * (PrivacyAmplification/PrivacyAmplification.cu:1686-2118, `mainloop`): the launch sequence
 * binInt2float -> calculateCorrectionFloat -> cufftExecR2C -> setFirstElementToZero ->
 * ElementWiseProduct -> cufftExecC2R -> ToBinaryArray[NoXOR] becomes one call.  The reference has no
 * FFI of its own; every entry point below names the reference code it replaces.
 *
 * Conventions (identical to the reference):
 *   - n ("sample_size", PrivacyAmplification.cu:1248) is the block size in bits; v ("vertical_len")
 *     the output length; h = n - v.  n and v are multiples of 32, 0 < v < n.
 *   - Bit i of an input word array is (word[i/32] >> (31 - i%32)) & 1 (PrivacyAmplification.cu:223-257).
 *   - key_start holds key bits 0..h (h+1 bits; bits past h are ignored), key_rest v bits: the split of
 *     PrivacyAmplification.cu:861-892 (pa_key_split below).
 *   - Output bit i goes to byte i/8, bit 7 - i%8 (AMPOUT_REVERSE_ENDIAN, PrivacyAmplification.h:38);
 *     length pa_output_bytes(): v/8 bytes, or n/16 bytes when PA_FLAG_COMPRESS is clear
 *     (PrivacyAmplification.cu:1197).
 *   - Result: out[i] = (sum_{j=0..h} key_start[j] * seed[(i-j) mod n] mod 2) XOR key_rest[i].
 *   - Precision: the FP32 FFT path measures every block's largest distance of an output value to the
 *     nearest integer; above residual_limit pa_process recomputes the block on the exact integer
 *     (NTT mod 3*2^30+1) path.  Blocks with n > 2^27 (up to 2^30) run as 2^27-bit FP32 chunk blocks
 *     (large-block decomposition) under the same guard.
 *
 * All functions return 0 (PA_OK) or a negative PA_ERR_* code; nothing exits the process.
 * An engine is bound to one CUDA device and must be used from one host thread at a time.
 */
#ifndef PA_GB300_H
#define PA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PA_API __attribute__((visibility("default")))
#else
#define PA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PA_OK 0
#define PA_ERR_INVALID_ARG (-1)   /* sizes / pointers rejected before any GPU work */
#define PA_ERR_CUDA (-2)          /* a CUDA call failed; see pa_last_cuda_error() */
#define PA_ERR_NO_SEED (-3)       /* no seed set, or its reuse_seed_amount is used up */
#define PA_ERR_TOO_LARGE (-4)     /* n above the engine's max_sample_size */
#define PA_ERR_PRECISION (-5)     /* FP32 residual above the limit (result withheld) */

#define PA_FLAG_XOR_KEY_REST 1u   /* do_xor_key_rest (config.yaml, key-server message) */
#define PA_FLAG_COMPRESS 2u       /* do_compress */
#define PA_FLAG_EXACT 4u          /* force the exact integer (NTT) path for this block */

typedef struct pa_engine pa_engine;

/* Engine configuration; mirrors the config.yaml keys the hot path reads
 * (PrivacyAmplification.cu:1244-1271). */
typedef struct pa_config {
    int32_t device_id;              /* gpu_device_id_to_use */
    uint32_t max_sample_size;       /* largest n the engine will see (2^factor_exp); sizes HBM buffers */
    uint32_t reduction_exp;         /* accepted for compatibility: power-of-two scalings cancel exactly */
    uint32_t pre_mul_reduction_exp; /* accepted for compatibility */
    float residual_limit;           /* precision guard: max |x - rint(x)| allowed (0 -> 0.25) */
} pa_config;

typedef struct pa_stats {
    float max_residual;       /* largest distance of an output value to the nearest integer */
    uint64_t popcount_key;    /* Hamming weight of key_start (count_one_of_global_key) */
    uint64_t popcount_seed;   /* Hamming weight of the seed (count_one_of_global_seed) */
    float gpu_ms;             /* device time of the block (CUDA events) */
    int32_t seed_uses_left;   /* remaining blocks for the cached seed, -1 = unlimited */
    int32_t exact;            /* 0: FP32 path, one pass; 2: FP32 path as 2^27-bit chunk blocks (n > 2^27);
                                 1: exact path (guard fallback or PA_FLAG_EXACT).  Popcounts are 0 for 1, 2 */
} pa_stats;

/* Creates an engine on cfg->device_id and allocates its HBM working set for n <= max_sample_size.
 * Replaces the allocation part of main() (PrivacyAmplification.cu:1536-1606). */
PA_API int pa_create(const pa_config* cfg, pa_engine** out);
PA_API void pa_destroy(pa_engine* e);

/* Sets the Toeplitz seed (n/32 words) and computes its cached FP32 spectrum.  reuse_seed_amount
 * follows the reference: 0 = this block only, k > 0 = the next k blocks, -1 = forever
 * (PrivacyAmplification.cu:1786, 2099-2101).  A seed for one block only (0 or 1) of 2^21 bits and more
 * is transformed inside that block's column pass instead (no spectrum is stored).  Replaces
 * binInt2float(seed) + cufftExecR2C(seed) (PrivacyAmplification.cu:1831, 1903). */
PA_API int pa_set_seed(pa_engine* e, const uint32_t* seed_words, uint32_t n, int32_t reuse_seed_amount);

/* Processes one block synchronously (host buffers, pageable or pinned).  key_rest may be NULL when
 * PA_FLAG_XOR_KEY_REST is clear.  out receives pa_output_bytes(n, v, flags) bytes.  stats may be NULL.
 * Replaces the mainloop body PrivacyAmplification.cu:1797-2042. */
PA_API int pa_process(pa_engine* e, const uint32_t* key_start, const uint32_t* key_rest, uint32_t n, uint32_t v,
               uint32_t flags, uint8_t* out, pa_stats* stats);

/* Device-resident forms: pointers are device memory, work is queued on `stream` (a cudaStream_t;
 * NULL = the engine's stream) and the call returns without synchronising.  d_out receives
 * pa_output_bytes() bytes rounded up to a multiple of 4.  pa_sync() waits and fills stats. */
PA_API int pa_set_seed_device(pa_engine* e, const uint32_t* d_seed_words, uint32_t n, int32_t reuse_seed_amount,
                       void* stream);
PA_API int pa_process_device(pa_engine* e, const uint32_t* d_key_start, const uint32_t* d_key_rest, uint32_t n,
                      uint32_t v, uint32_t flags, uint8_t* d_out, void* stream);
PA_API int pa_sync(pa_engine* e, pa_stats* stats);

/* key2StartRest (PrivacyAmplification.cu:861-892), host only: recv_key has n/32+1 words; key_start
 * receives n/32 words (zero past word h/32), key_rest v/32 words. */
PA_API int pa_key_split(const uint32_t* recv_key, uint32_t n, uint32_t v, uint32_t* key_start, uint32_t* key_rest);

/* Output length in bytes (PrivacyAmplification.cu:1197). */
PA_API size_t pa_output_bytes(uint32_t n, uint32_t v, uint32_t flags);

/* Number of kernels one pa_process_device launches for (n, v) with a cached seed spectrum (a one-use
 * seed of 2^21 bits and more adds its two row-pass kernels: bit rows and row FFTs). */
PA_API int pa_kernels_per_block(uint32_t n, uint32_t v, uint32_t flags);

/* Per-kernel timing, the counterpart of the reference's STOPWATCH stage deltas
 * (PrivacyAmplification.cu:146-166, 2053-2074).  When enabled, every block records CUDA events on its
 * stream before the first and after each kernel (no host synchronisation).  pa_stage_times() waits
 * for the recorded blocks and writes the mean device time per kernel in ms (up to max_stages values,
 * order: pass A, pass B, pass C, finish; one value for single-CTA blocks), the stage count and the
 * number of blocks averaged, then clears the record. */
PA_API int pa_set_timing(pa_engine* e, int enable);
PA_API int pa_stage_times(pa_engine* e, float* ms, int max_stages, int* nstages, int* nblocks);

PA_API const char* pa_error_string(int code);
PA_API int pa_last_cuda_error(pa_engine* e);

/* Self-test of the failure path (no counterpart in the reference, whose kernels have no bounded
 * waits): runs one CTA whose mbarrier wait is never satisfied, with a limit of `rounds` try_wait rounds
 * (1..2^20), and stores the device error word in *status: 1 = the wait expired and was reported, as a
 * TMA wait of the three-pass kernels does (pa_process then returns PA_ERR_CUDA with
 * cudaErrorLaunchTimeout in pa_last_cuda_error).  The context stays usable afterwards. */
PA_API int pa_selftest_wait_timeout(int32_t device_id, uint32_t rounds, int32_t* status);

/* Measurement of one radix-16 DFT stage on the tensor cores against the FP32 butterflies (no counterpart
 * in the reference, whose transforms are cuFFT calls, PrivacyAmplification.cu:1736,1745).  d_in / d_out
 * hold `butterflies` (a multiple of 128) groups of 16 complex FP32 values, re/im interleaved, 16-byte
 * aligned; each group gets `reps` forward 16-point DFTs, scaled by 1/256 after every fourth (so that
 * reps % 4 == 0 returns the input).  method 0: FP32 butterflies in registers (the passes' stage);
 * 1: tcgen05.mma kind::tf32 with operands split into TF32 high and low parts, three products (FP32-level
 * accuracy); 2: one TF32 product.  ctas_per_sm: 1..16 for method 0, 1..4 for the tensor methods.  A
 * bounded wait that expires stores 1 in *d_err (device int).  Queued on `stream`, not synchronised. */
PA_API int pa_dft16_stages(const float* d_in, float* d_out, uint32_t butterflies, uint32_t reps, int32_t method,
                           int32_t ctas_per_sm, int32_t* d_err, void* stream);

/* ---- Batched and served blocks -------------------------------------------------------------------
 * No counterpart in the reference: its mainloop (PrivacyAmplification.cu:1686-2118) runs one block at
 * a time with a host sync after every step.  Here blocks of different sizes run concurrently on a pool
 * of slots; a slot is a CUDA stream with its own working set (about 12.6 * Np bytes for cyclic length
 * Np), created on demand within the pool's HBM budget.  Sizes: the FP32 path (n <= 2^27); a block
 * whose residual exceeds residual_limit is recomputed on the exact path when its result is collected
 * (pa_batch_sync, pa_poll), as in pa_process. */
#define PA_ERR_BUSY (-6) /* pa_submit: no slot or HBM free now; collect a block with pa_poll and retry */
#define PA_PENDING 1     /* pa_poll: the block is still running */

typedef struct pa_job {
    const uint32_t* seed_words; /* n/32 words: the block's own (dynamic) seed; NULL when seed_id >= 0 */
    int32_t seed_id;            /* static seed: a spectrum from pa_seed_cache_add, or -1 */
    const uint32_t* key_start;  /* n/32 words as from pa_key_split (words past h/32 are not read) */
    const uint32_t* key_rest;   /* v/32 words; may be NULL when PA_FLAG_XOR_KEY_REST is clear */
    uint32_t n, v, flags;       /* PA_FLAG_EXACT is not accepted here */
    uint8_t* out;               /* pa_output_bytes() bytes (device pointers: 4-byte aligned, rounded up to 4) */
} pa_job;

/* Pool limits: HBM bytes all slots may hold (0 = 60 % of the free memory at first use), the number
 * of slots (0 = 16) and the slots one batch spreads over (0 = 8).  Idle slots are freed first. */
PA_API int pa_set_pool(pa_engine* e, uint64_t hbm_budget_bytes, int32_t max_slots, int32_t batch_slots);

/* Creates idle slots up front so that later admissions (pa_submit) and batches find their working set
 * ready instead of allocating it: up to `count` slots (within max_slots and the HBM budget) that hold
 * blocks with cyclic length up to max_np (a power of two; n itself for power-of-two n).  Returns the
 * number of slots that now hold such blocks, or a negative PA_ERR_* code. */
PA_API int pa_pool_reserve(pa_engine* e, uint32_t max_np, int32_t count);

/* Static seeds: computes and keeps the FP32 spectrum of a seed (host words, n/32) for blocks of
 * geometry (n, v, flags) -- for a power-of-two n any v and flags share it.  Synchronous.  The id is
 * valid until pa_seed_cache_clear.  Replaces the reference's reuse of do2 across blocks
 * (PrivacyAmplification.cu:1903, reuse_seed_amount) for many seeds at once. */
PA_API int pa_seed_cache_add(pa_engine* e, const uint32_t* seed_words, uint32_t n, uint32_t v, uint32_t flags,
                             int32_t* seed_id);
PA_API int pa_seed_cache_clear(pa_engine* e);

/* Batch of blocks with DEVICE pointers, queued on `stream` (NULL = the engine's stream); returns
 * without synchronising.  Jobs are spread over the pool's batch slots, longest first.
 * PA_BATCH_GRAPH: capture the whole batch as one CUDA graph the first time these exact jobs are seen
 * and replay it afterwards.  PA_BATCH_SERIAL: one slot, jobs in order (the per-block launch
 * sequence, for comparison).  pa_batch_sync waits, recomputes blocks over the residual limit
 * exactly, and fills stats[i] for job i (gpu_ms: the whole batch's device time).
 * Jobs of one geometry (same n, v, flags, and all static or all with their own seed), four or more of
 * them, run as groups: one launch per pass for up to 2^24 bits of cyclic length, instead of one per pass
 * and block (the reference's sub-block variant batches equal sub-blocks on cuFFT the same way,
 * PrivacyAmplification_subblocks.cu:1058-1081); groups spread over the slots like single blocks.
 * PA_BATCH_NO_GROUP launches every block on its own. */
#define PA_BATCH_GRAPH 1u
#define PA_BATCH_SERIAL 2u
#define PA_BATCH_PERSISTENT 4u
#define PA_BATCH_NO_GROUP 8u
PA_API int pa_batch_run(pa_engine* e, const pa_job* jobs, uint32_t count, uint32_t batch_flags, void* stream);
/* Group sizing: at least min_blocks (>= 2; 0 = 4) equal jobs form groups of up to 2^log_bits bits of
 * cyclic length each (17..30; 0 = 24).  No batch may be pending. */
PA_API int pa_set_groups(pa_engine* e, int32_t min_blocks, int32_t log_bits);
PA_API int pa_batch_sync(pa_engine* e, pa_stats* stats, uint32_t count);

/* PA_BATCH_PERSISTENT: the whole batch runs as ONE persistent kernel launch (with PA_BATCH_GRAPH, that
 * launch captured in a CUDA graph and replayed).  The launch holds one 512-thread CTA per SM, cut into
 * lanes of ctas_per_lane CTAs; a lane takes one block at a time, longest first from a device-side list,
 * and its CTAs run the block's passes between lane barriers (bounded waits: an expired one makes
 * pa_batch_sync return PA_ERR_CUDA with cudaErrorLaunchTimeout).  Every block's arrays live in its
 * lane's working set (about 12 * Np bytes, Np the largest cyclic length the lanes hold), so the number of
 * lanes is what the pool's HBM budget admits.  Blocks run with rows of 2^14 and a cyclic length of at
 * least 2^20 (a smaller block is placed in 2^20), up to n = 2^27.  Static seeds get a spectrum in the
 * lanes' layout the first time a batch uses them.  pa_set_lanes sets the CTAs per lane (0 = 4) and
 * sizes the lanes for cyclic lengths up to max_np (a power of two; 0 = the largest block of each batch);
 * returns the number of lanes allocated (0 if none yet) or a negative PA_ERR_* code.  No counterpart
 * in the reference (one block per mainloop pass, PrivacyAmplification.cu:1686-2118). */
PA_API int pa_set_lanes(pa_engine* e, int32_t ctas_per_lane, uint32_t max_np);

/* Device-resident serving loop.  pa_serve_start launches the lane kernel in serving mode: its lanes
 * (ctas_per_lane CTAs each, 0 = 38, i.e. four lanes on 152 SMs; as many as the HBM budget admits for
 * cyclic lengths up to max_np, a power of two) poll a ring of ring_slots request slots (0 = 64) in pinned
 * host memory.  A lane takes the next published request, runs it -- reading the request's inputs from
 * host memory and writing its output there directly -- and publishes its completion; requests that
 * arrive while others run are taken by the next free lane, so they overlap on the device.  The host only
 * writes descriptors and reads completions: no launch or copy per request.  pa_serve_submit publishes a
 * request (job pointers: pinned host or device memory -- pageable memory is refused with
 * PA_ERR_INVALID_ARG; out holds pa_output_bytes() rounded up to a multiple of 4; a static seed_id needs its
 * spectrum cached with pa_seed_cache_add before pa_serve_start) and returns its ticket, PA_ERR_BUSY when
 * every ring slot holds a request not yet collected, PA_ERR_TOO_LARGE beyond max_np.  pa_serve_poll
 * returns PA_PENDING, or PA_OK once job->out holds the result (a block over the residual limit is first
 * recomputed exactly); the ring slot is then free.  The loop ends by itself after about two idle seconds
 * and is started again by the next submit; pa_serve_stop ends it (after the requests it has taken) and
 * frees the ring.  While serving, persistent batches return PA_ERR_BUSY.  The reference's counterpart is
 * its host loop over ring slots with spin-waits (PrivacyAmplification.cu:1781-1797, 1990-1992). */
PA_API int pa_serve_start(pa_engine* e, int32_t ctas_per_lane, uint32_t max_np, int32_t ring_slots);
PA_API int pa_serve_submit(pa_engine* e, const pa_job* job, uint64_t* ticket);
PA_API int pa_serve_poll(pa_engine* e, uint64_t ticket, pa_stats* stats);
PA_API int pa_serve_stop(pa_engine* e);

/* Served blocks with HOST pointers (pinned memory lets the copies overlap): pa_submit admits the
 * block to a free slot (creating one if the HBM budget allows), queues copy-in, kernels and copy-out,
 * and returns a ticket; PA_ERR_BUSY when nothing is free.  pa_poll returns PA_PENDING while the block
 * runs, then PA_OK once job->out holds the result (stats filled, slot released).  The job's host
 * buffers must stay valid until then. */
PA_API int pa_submit(pa_engine* e, const pa_job* job, uint64_t* ticket);
PA_API int pa_poll(pa_engine* e, uint64_t ticket, pa_stats* stats);

/* Three-pass split (N = N1 * N2, N = Np/2): pa_set_split fixes log2 N2 for log2 N = log_n (row FFT
 * length; allowed max(10, log_n-12) .. min(14, log_n-5)); pa_get_split returns the one in use.
 * pa_autotune times every allowed split of each log_n in [log2(min_n)-1, log2(max_n)-1] on a synthetic
 * block and keeps the fastest; ms_out (optional, 32 floats) receives the best key-block time per
 * log_n.  Cached spectra keep the split they were built with. */
PA_API int pa_set_split(pa_engine* e, uint32_t log_n, uint32_t log_n2);
PA_API int pa_get_split(pa_engine* e, uint32_t log_n);
PA_API int pa_autotune(pa_engine* e, uint32_t min_n, uint32_t max_n, float* ms_out);

/* No counterpart in the reference.  One block hashed with its own seed, without any engine and without
 * allocating device memory: for callers that may not call cudaMalloc (device memory owned by another
 * allocator, or a memory map fixed at start-up).  All pointers are device memory the caller owns:
 * d_seed_words n/32 words, d_key_start and d_key_rest as for pa_process_device (d_key_rest may be NULL
 * when PA_FLAG_XOR_KEY_REST is clear), d_out (4-byte aligned) pa_output_bytes() bytes rounded up to a
 * multiple of 4.  Work is queued on `stream` (a cudaStream_t; NULL = the legacy default stream) and the
 * call returns without synchronising; no statistics are produced and the precision guard does not run.
 * Limit: n <= 32768 (padded cyclic length <= 32768); larger n returns PA_ERR_TOO_LARGE, and
 * PA_FLAG_EXACT returns PA_ERR_INVALID_ARG.  The scratch (128 KiB + 256 B = 131,328 bytes) is a static
 * device array of the library, one per GPU: every call looks up its address in the current context (the
 * first call in a context also loads the library's device code, so make it before any stream capture),
 * and calls that overlap on one GPU race on it. */
PA_API int pa_process_noalloc(const uint32_t* d_seed_words, const uint32_t* d_key_start, const uint32_t* d_key_rest,
                              uint32_t n, uint32_t v, uint32_t flags, uint8_t* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PA_GB300_H */
