// pa_engine.cu -- host side of the C ABI declared in include/pa_gb300.h.
//
// Owns the HBM working set of one GPU (the reference's device buffers di1/di2/do1/do2 and its cuFFT
// plans, PrivacyAmplification.cu:1567-1593, 1714-1751), the cached seed spectrum and the
// reuse_seed_amount bookkeeping of the host loop (PrivacyAmplification.cu:1762-1797, 2099-2101).
#include "pa_engine_impl.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

using pa::BlockGeom;
using pa_host::ceil_log2;
using pa_host::cuda_fail;
using pa_host::is_pow2;

namespace pa_host {

// Block geometry (sizes, padded cyclic length, three-pass split) for (n, v, flags).
int make_geom(uint32_t n, uint32_t v, uint32_t flags, const int8_t* split, BlockGeom* g) {
    if (n < 1024u || (n & 31u) || (v & 31u) || v == 0 || v >= n) return PA_ERR_INVALID_ARG;
    g->n = n;
    g->v = v;
    g->h = n - v;
    g->out_bits = (flags & PA_FLAG_COMPRESS) ? v : n / 2u;
    if (is_pow2(n)) {
        g->log_np = ceil_log2(n);
        g->seed_direct = n;
    } else {
        uint64_t need = std::max<uint64_t>(n, (uint64_t)g->out_bits + g->h);
        g->log_np = ceil_log2(need);
        uint64_t np = 1ull << g->log_np;
        g->seed_direct = (uint32_t)std::min<uint64_t>(np - g->h, n);
    }
    g->log_n = g->log_np - 1;
    g->exact_only = 0;
    if (g->log_n <= 14) {
        g->log_n1 = g->log_n2 = 0;
    } else if (g->log_n <= 26) {
        int l2 = split ? split[g->log_n] : 0;
        if (l2 < split_min(g->log_n) || l2 > split_max(g->log_n)) l2 = split_default(g->log_n);
        g->log_n2 = l2;  // rows 2^10..2^14, columns 2^5..2^12
        g->log_n1 = g->log_n - g->log_n2;
    } else {  // beyond the FP32 path: exact NTT only
        g->log_n1 = g->log_n2 = 0;
        g->exact_only = 1;
        if (g->log_np > 30) return PA_ERR_TOO_LARGE;
    }
    return PA_OK;
}

bool same_seed_geom(const BlockGeom& a, const BlockGeom& b) {
    if (a.log_np != b.log_np || a.n != b.n || a.log_n2 != b.log_n2) return false;
    if (is_pow2(a.n)) return true;  // placement is the identity
    return a.seed_direct == b.seed_direct && a.h == b.h;
}

}  // namespace pa_host

namespace {

using pa_host::make_geom;
using pa_host::same_seed_geom;

int ensure_maps(pa_engine* e, const BlockGeom& g) {
    if (g.log_n1 == 0 || e->maps_key == pa_host::maps_key(g)) return PA_OK;
    int rc = pa::make_pass_maps(g, e->d_work, e->d_work2, &e->maps);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    e->maps_key = pa_host::maps_key(g);
    return PA_OK;
}

pa::Scratch scratch(pa_engine* e) { return {e->d_work, e->d_work2, e->d_planes, e->d_err, &e->maps}; }

int build_exact_seed(pa_engine* e, const BlockGeom& g, cudaStream_t s) {
    int rc = pa::launch_exact_seed(g, e->d_seed, e->d_exact_seed, reinterpret_cast<uint32_t*>(e->d_work2), &e->ntt, s);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    e->exact_geom = g;
    e->exact_valid = true;
    return PA_OK;
}

int build_spectrum(pa_engine* e, const BlockGeom& g, cudaStream_t s) {
    if (g.exact_only) return build_exact_seed(e, g, s);
    int rc = ensure_maps(e, g);
    if (rc) return rc;
    rc = pa::launch_seed_spectrum(g, e->d_seed, e->d_spec, scratch(e), e->d_cnt + 1, e->num_sms, s);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    e->spec_geom = g;
    e->spec_valid = true;
    return PA_OK;
}

// The seed serves the next block only and that block's column pass can transform it (the fused pass).
bool fuse_seed(const pa_engine* e, const BlockGeom& g) {
    return e->seed_left == 1 && e->d_park && pa::fused_geom(g);
}

int seed_common(pa_engine* e, uint32_t n, int32_t reuse, cudaStream_t s) {
    e->seed_valid = true;
    e->seed_n = n;
    e->seed_left = reuse < 0 ? -1 : std::max<int64_t>(reuse, 1);
    e->spec_valid = false;
    e->exact_valid = false;
    if (is_pow2(n)) {  // placement does not depend on v: build the spectrum now
        BlockGeom g;
        int rc = make_geom(n, n / 2u, PA_FLAG_COMPRESS, e->split, &g);
        if (rc) return rc;
        if (g.exact_only) return PA_OK;  // chunk spectra are built per block, the exact transform on demand
        if (fuse_seed(e, g)) return PA_OK;  // transformed inside the block's column pass
        return build_spectrum(e, g, s);
    }
    return PA_OK;
}

// A block whose seed serves it alone: the seed's row pass into d_spec, then the fused column pass.
// d_spec then holds no spectrum.
int fused_block(pa_engine* e, const uint32_t* d_ks, const uint32_t* d_kr, const BlockGeom& g, uint32_t flags,
                uint32_t* d_out, cudaStream_t s, cudaEvent_t* sev, cudaEvent_t kr_ready) {
    int rc = ensure_maps(e, g);
    if (rc) return rc;
    if (e->seed_maps_key != pa_host::maps_key(g)) {
        rc = pa::make_pass_maps(g, e->d_spec, e->d_work2, &e->seed_maps);
        if (rc) return cuda_fail(e, (cudaError_t)rc);
        e->seed_maps_key = pa_host::maps_key(g);
    }
    e->spec_valid = false;
    rc = pa::launch_fused_block(g, e->d_seed, d_ks, d_kr, flags, e->d_spec, e->seed_maps, e->d_park, e->park_ctas,
                                scratch(e), e->d_cnt, e->d_resid, d_out, e->num_sms, s, sev, kr_ready);
    return rc ? cuda_fail(e, (cudaError_t)rc) : PA_OK;
}

// n > 2^27: the block as 2^27-bit FP32 chunk blocks (pa_chunk.cu).  The exact seed transform's buffer
// is the chunks' staging area and the chunk spectra go through d_spec, so both caches are invalidated.
// Block popcounts are not formed on this path (read_stats reports 0).
//
// Two lanes take the diagonals in turn.  The second lane's three-pass buffers are the upper halves of
// d_work / d_work2 (each holds Np / 2 >= 2^27 complex here, a chunk block needs 2^26); its staging, bit
// planes and seed spectrum follow the first lane's staging in d_exact_seed (Np >= 2^28 words, the four
// need under 2^28); its stream is `side`, free here because the block waited for key_rest's copy.
int chunked_block(pa_engine* e, const uint32_t* d_ks, const uint32_t* d_kr, const BlockGeom& g, uint32_t flags,
                  uint32_t* d_out, cudaStream_t s) {
    BlockGeom gc;
    const uint32_t side = 1u << pa::kChunkLog;
    int rc = make_geom(2u * side, side, 0u, e->split, &gc);
    if (rc) return rc;
    const size_t np = size_t(1) << e->cap_log_np;
    if (pa::chunk_staging_words(g) > np) return PA_ERR_TOO_LARGE;
    rc = ensure_maps(e, gc);
    if (rc) return rc;
    e->exact_valid = false;
    e->spec_valid = false;
    auto align64 = [](size_t w) { return (w + 63u) & ~size_t(63); };
    const size_t nc = size_t(1) << gc.log_n;                               // complex per three-pass buffer
    const size_t w0 = align64(pa::chunk_staging_words(g));                 // first lane's staging
    const size_t w1 = align64(pa::chunk_lane_words(g));                    // second lane's staging
    const size_t wp = align64((size_t(1) << gc.log_np) / 32u + 64u);       // bit planes: Np / 8 + 256 bytes
    pa::ChunkLane lane{};
    const pa::ChunkLane* lp = nullptr;
    if (2 * nc <= np / 2 && w0 + w1 + wp + 2 * nc <= np) {
        if (e->lane_maps_key != pa_host::maps_key(gc)) {
            rc = pa::make_pass_maps(gc, e->d_work + nc, e->d_work2 + nc, &e->lane_maps);
            if (rc) return cuda_fail(e, (cudaError_t)rc);
            e->lane_maps_key = pa_host::maps_key(gc);
        }
        uint32_t* base = e->d_exact_seed;
        lane.staging = base + w0;
        lane.sc = {e->d_work + nc, e->d_work2 + nc, base + w0 + w1, e->d_err, &e->lane_maps};
        lane.spec = reinterpret_cast<float2*>(base + w0 + w1 + wp);
        lane.s = e->side;
        lane.fork = e->lane_fork;
        lane.join = e->lane_join;
        lp = &lane;
    }
    rc = pa::launch_chunked_block(g, gc, e->d_seed, d_ks, d_kr, flags, d_out, e->d_exact_seed, e->d_spec, scratch(e),
                                  e->d_cnt, e->d_resid, e->num_sms, s, lp);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    return PA_OK;
}

// Exact path for one block (the seed's NTT is built on first use and cached with the seed).
int exact_block(pa_engine* e, const uint32_t* d_ks, const uint32_t* d_kr, const BlockGeom& g, uint32_t flags,
                uint32_t* d_out, cudaStream_t s) {
    if (!e->exact_valid || !same_seed_geom(e->exact_geom, g)) {
        int rc = build_exact_seed(e, g, s);
        if (rc) return rc;
    }
    int rc = pa::launch_exact_block(g, d_ks, d_kr, flags, e->d_exact_seed, reinterpret_cast<uint32_t*>(e->d_work),
                                    reinterpret_cast<uint32_t*>(e->d_work2), d_out, &e->ntt, s);
    if (rc) return cuda_fail(e, (cudaError_t)rc);
    // the exact path leaves no residual: report 0 and the reference popcounts are not needed
    PA_CUDA(e, cudaMemsetAsync(e->d_resid, 0, sizeof(unsigned int), s));
    return PA_OK;
}

int block_common(pa_engine* e, const uint32_t* d_ks, const uint32_t* d_kr, const BlockGeom& g, uint32_t flags,
                 uint32_t* d_out, cudaStream_t s, cudaEvent_t kr_ready = nullptr) {
    if (!e->seed_valid || e->seed_left == 0) return PA_ERR_NO_SEED;
    if (g.n != e->seed_n) return PA_ERR_INVALID_ARG;
    e->last_chunked = false;
    if (kr_ready && ((flags & PA_FLAG_EXACT) || g.exact_only))  // these paths read key_rest early
        PA_CUDA(e, cudaStreamWaitEvent(s, kr_ready, 0));
    if (flags & PA_FLAG_EXACT) {
        PA_CUDA(e, cudaEventRecord(e->ev0, s));
        int rc = exact_block(e, d_ks, d_kr, g, flags, d_out, s);
        if (rc) return rc;
        PA_CUDA(e, cudaEventRecord(e->ev1, s));
        e->last_exact = true;
        if (e->seed_left > 0) --e->seed_left;
        return PA_OK;
    }
    e->last_exact = false;
    if (g.exact_only) {
        PA_CUDA(e, cudaEventRecord(e->ev0, s));
        int rc = chunked_block(e, d_ks, d_kr, g, flags, d_out, s);
        if (rc) return rc;
        PA_CUDA(e, cudaEventRecord(e->ev1, s));
        e->last_chunked = true;
        if (e->seed_left > 0) --e->seed_left;
        return PA_OK;
    }
    const bool fused = (!e->spec_valid || !same_seed_geom(e->spec_geom, g)) && fuse_seed(e, g);
    if (!fused && (!e->spec_valid || !same_seed_geom(e->spec_geom, g))) {
        int rc = build_spectrum(e, g, s);
        if (rc) return rc;
    }
    int mrc = ensure_maps(e, g);
    if (mrc) return mrc;
    PA_CUDA(e, cudaEventRecord(e->ev0, s));
    cudaEvent_t* sev = nullptr;
    if (e->timing && !e->tev.empty()) {
        size_t slot = e->tev_next;
        sev = e->tev[slot].data();
        e->tev_stages[slot] = pa::stage_count_key_block(g);
        e->tev_next = (slot + 1) % e->tev.size();
        e->tev_count = std::min(e->tev_count + 1, e->tev.size());
    }
    if (fused) {
        int rc = fused_block(e, d_ks, d_kr, g, flags, d_out, s, sev, kr_ready);
        if (rc) return rc;
    } else {
        int rc = pa::launch_key_block(g, d_ks, d_kr, flags, e->d_spec, scratch(e), e->d_cnt, e->d_resid, d_out,
                                      e->num_sms, s, sev, kr_ready);
        if (rc) return cuda_fail(e, (cudaError_t)rc);
    }
    PA_CUDA(e, cudaEventRecord(e->ev1, s));
    if (e->seed_left > 0) --e->seed_left;
    return PA_OK;
}

int read_stats(pa_engine* e, pa_stats* st, float* resid_out) {
    unsigned long long cnt[2] = {0, 0};
    unsigned int rb = 0;
    PA_CUDA(e, cudaMemcpy(cnt, e->d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
    PA_CUDA(e, cudaMemcpy(&rb, e->d_resid, sizeof(rb), cudaMemcpyDeviceToHost));
    int derr = 0;
    PA_CUDA(e, cudaMemcpy(&derr, e->d_err, sizeof(derr), cudaMemcpyDeviceToHost));
    if (derr) {  // a bounded device wait expired: the block's result is not valid
        cudaMemset(e->d_err, 0, sizeof(int));
        e->last_cuda = (int)cudaErrorLaunchTimeout;
        return PA_ERR_CUDA;
    }
    float resid;
    std::memcpy(&resid, &rb, sizeof(resid));
    *resid_out = resid;
    if (st) {
        st->max_residual = resid;
        const bool counted = !e->last_exact && !e->last_chunked;  // popcounts exist on the one-pass FP32 path
        st->popcount_key = counted ? cnt[0] : 0;
        st->popcount_seed = counted ? cnt[1] : 0;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e->ev0, e->ev1);
        st->gpu_ms = ms;
        st->seed_uses_left = e->seed_left < 0 ? -1 : (int32_t)e->seed_left;
        st->exact = e->last_exact ? 1 : (e->last_chunked ? 2 : 0);
    }
    return PA_OK;
}

}  // namespace

extern "C" {

size_t pa_output_bytes(uint32_t n, uint32_t v, uint32_t flags) {
    return (flags & PA_FLAG_COMPRESS) ? v / 8u : n / 16u;
}

int pa_kernels_per_block(uint32_t n, uint32_t v, uint32_t flags) {
    BlockGeom g;
    if (make_geom(n, v, flags, nullptr, &g)) return 0;
    if (flags & PA_FLAG_EXACT) return pa::exact_kernel_count(g);
    if (g.exact_only) {
        BlockGeom gc;
        if (make_geom(2u << pa::kChunkLog, 1u << pa::kChunkLog, 0u, nullptr, &gc)) return 0;
        return pa::chunk_kernel_count(g, gc);
    }
    return pa::kernel_count_key_block(g);
}

const char* pa_error_string(int code) {
    switch (code) {
        case PA_OK: return "ok";
        case PA_ERR_INVALID_ARG: return "invalid argument";
        case PA_ERR_CUDA: return "CUDA error";
        case PA_ERR_NO_SEED: return "no seed set or reuse_seed_amount used up";
        case PA_ERR_TOO_LARGE: return "block larger than the engine or the pool can hold";
        case PA_ERR_PRECISION: return "FP32 residual above the precision limit";
        case PA_ERR_BUSY: return "no slot or HBM free for the block now";
        case PA_PENDING: return "block still running";
        default: return "unknown error";
    }
}

int pa_last_cuda_error(pa_engine* e) { return e ? e->last_cuda : 0; }

int pa_create(const pa_config* cfg, pa_engine** out) {
    if (!cfg || !out || cfg->max_sample_size < 1024u || (cfg->max_sample_size & 31u)) return PA_ERR_INVALID_ARG;
    *out = nullptr;
    pa_engine* e = new (std::nothrow) pa_engine();
    if (!e) return PA_ERR_INVALID_ARG;
    e->device = cfg->device_id;
    e->max_n = cfg->max_sample_size;
    e->residual_limit = cfg->residual_limit > 0.f ? cfg->residual_limit : 0.25f;
    e->cap_log_np = ceil_log2(cfg->max_sample_size);
    if (e->cap_log_np > 30) {
        delete e;
        return PA_ERR_TOO_LARGE;
    }
    auto fail = [&](cudaError_t) {
        pa_destroy(e);
        return PA_ERR_CUDA;
    };
    cudaError_t err = cudaSetDevice(e->device);
    if (err != cudaSuccess) return fail(err);
    cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device);
    if ((err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(err);
    if ((err = cudaEventCreate(&e->ev0)) != cudaSuccess) return fail(err);
    if ((err = cudaEventCreate(&e->ev1)) != cudaSuccess) return fail(err);
    if ((err = cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking)) != cudaSuccess) return fail(err);
    if ((err = cudaEventCreateWithFlags(&e->kr_ready, cudaEventDisableTiming)) != cudaSuccess) return fail(err);
    if ((err = cudaEventCreateWithFlags(&e->main_ready, cudaEventDisableTiming)) != cudaSuccess) return fail(err);
    if ((err = cudaEventCreateWithFlags(&e->lane_fork, cudaEventDisableTiming)) != cudaSuccess) return fail(err);
    if ((err = cudaEventCreateWithFlags(&e->lane_join, cudaEventDisableTiming)) != cudaSuccess) return fail(err);
    size_t np = 1ull << e->cap_log_np;
    size_t words = np / 32 + 64;
    if ((err = cudaMalloc(&e->d_key_start, words * 4)) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_key_rest, words * 4)) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_seed, words * 4)) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_out, words * 4)) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_work, (np / 2) * sizeof(float2))) != cudaSuccess) return fail(err);
    const size_t np_fp32 = std::min<size_t>(np, size_t(1) << 27);  // the FP32 path stops at n = 2^27
    if ((err = cudaMalloc(&e->d_spec, (np_fp32 / 2) * sizeof(float2))) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_exact_seed, np * sizeof(uint32_t))) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_work2, (np / 2) * sizeof(float2))) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_err, sizeof(int))) != cudaSuccess) return fail(err);
    cudaMemset(e->d_err, 0, sizeof(int));
    if ((err = cudaMalloc(&e->d_planes, np_fp32 / 8 + 256)) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_cnt, 2 * sizeof(unsigned long long))) != cudaSuccess) return fail(err);
    if ((err = cudaMalloc(&e->d_resid, sizeof(unsigned int))) != cudaSuccess) return fail(err);
    if (e->cap_log_np >= 21) {  // blocks with columns of 2^10 and more: the fused column pass's park
        // one spectrum tile per CTA: two CTAs per SM, at most one per tile of the largest block
        e->park_ctas = std::min<uint32_t>(2u * (uint32_t)e->num_sms, (uint32_t)((np / 2) / 8192u));
        if ((err = cudaMalloc(&e->d_park, e->park_ctas * pa::kParkBytes)) != cudaSuccess) return fail(err);
    }
    cudaMemset(e->d_cnt, 0, 2 * sizeof(unsigned long long));
    cudaMemset(e->d_resid, 0, sizeof(unsigned int));
    *out = e;
    return PA_OK;
}

void pa_destroy(pa_engine* e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    pa_host::pool_destroy(e);
    cudaFree(e->d_key_start);
    cudaFree(e->d_key_rest);
    cudaFree(e->d_seed);
    cudaFree(e->d_out);
    cudaFree(e->d_work);
    cudaFree(e->d_spec);
    cudaFree(e->d_exact_seed);
    pa::free_ntt_tables(e->ntt);
    cudaFree(e->d_work2);
    cudaFree(e->d_err);
    cudaFree(e->d_planes);
    cudaFree(e->d_cnt);
    cudaFree(e->d_resid);
    cudaFree(e->d_park);
    for (auto& a : e->tev)
        for (auto ev : a) cudaEventDestroy(ev);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->kr_ready) cudaEventDestroy(e->kr_ready);
    if (e->main_ready) cudaEventDestroy(e->main_ready);
    if (e->lane_fork) cudaEventDestroy(e->lane_fork);
    if (e->lane_join) cudaEventDestroy(e->lane_join);
    if (e->side) cudaStreamDestroy(e->side);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

static int check_n(pa_engine* e, uint32_t n, uint32_t v, uint32_t flags, BlockGeom* g) {
    int rc = make_geom(n, v, flags, e->split, g);
    if (rc) return rc;
    if (n > e->max_n || g->log_np > e->cap_log_np) return PA_ERR_TOO_LARGE;
    return PA_OK;
}

// Seed sizes: any block size the engine accepts (the output length is only known per key block).
static int check_seed_n(pa_engine* e, uint32_t n) {
    BlockGeom g;
    return check_n(e, n, 32u, PA_FLAG_COMPRESS, &g);
}

int pa_set_seed(pa_engine* e, const uint32_t* seed_words, uint32_t n, int32_t reuse_seed_amount) {
    if (!e || !seed_words) return PA_ERR_INVALID_ARG;
    int rc = check_seed_n(e, n);
    if (rc) return rc;
    PA_CUDA(e, cudaSetDevice(e->device));
    PA_CUDA(e, cudaMemcpyAsync(e->d_seed, seed_words, (size_t)(n / 32u) * 4u, cudaMemcpyHostToDevice, e->stream));
    rc = seed_common(e, n, reuse_seed_amount, e->stream);
    if (rc) return rc;
    PA_CUDA(e, cudaStreamSynchronize(e->stream));
    return PA_OK;
}

int pa_set_seed_device(pa_engine* e, const uint32_t* d_seed_words, uint32_t n, int32_t reuse_seed_amount,
                       void* stream) {
    if (!e || !d_seed_words) return PA_ERR_INVALID_ARG;
    int rc = check_seed_n(e, n);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    PA_CUDA(e, cudaSetDevice(e->device));
    PA_CUDA(e, cudaMemcpyAsync(e->d_seed, d_seed_words, (size_t)(n / 32u) * 4u, cudaMemcpyDeviceToDevice, s));
    e->pending = true;
    return seed_common(e, n, reuse_seed_amount, s);
}

int pa_process(pa_engine* e, const uint32_t* key_start, const uint32_t* key_rest, uint32_t n, uint32_t v,
               uint32_t flags, uint8_t* out, pa_stats* stats) {
    if (!e || !key_start || !out) return PA_ERR_INVALID_ARG;
    if ((flags & PA_FLAG_XOR_KEY_REST) && !key_rest) return PA_ERR_INVALID_ARG;
    BlockGeom g;
    int rc = check_n(e, n, v, flags, &g);
    if (rc) return rc;
    if (!e->seed_valid || e->seed_left == 0) return PA_ERR_NO_SEED;
    if (n != e->seed_n) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    cudaStream_t s = e->stream;
    PA_CUDA(e, cudaMemcpyAsync(e->d_key_start, key_start, (size_t)(g.h / 32u + 1u) * 4u, cudaMemcpyHostToDevice, s));
    // key_rest is first read by the block's last kernel: it is copied on the side stream (after
    // whatever the engine stream had queued) while the passes run
    cudaEvent_t kr_ready = nullptr;
    if (flags & PA_FLAG_XOR_KEY_REST) {
        PA_CUDA(e, cudaEventRecord(e->main_ready, s));
        PA_CUDA(e, cudaStreamWaitEvent(e->side, e->main_ready, 0));
        PA_CUDA(e, cudaMemcpyAsync(e->d_key_rest, key_rest, (size_t)(v / 32u) * 4u, cudaMemcpyHostToDevice, e->side));
        PA_CUDA(e, cudaEventRecord(e->kr_ready, e->side));
        kr_ready = e->kr_ready;
    }
    rc = block_common(e, e->d_key_start, e->d_key_rest, g, flags, e->d_out, s, kr_ready);
    if (rc) {
        if (kr_ready) cudaStreamSynchronize(e->side);  // the caller's key_rest is not read after we return
        return rc;
    }
    size_t ob = pa_output_bytes(n, v, flags);
    PA_CUDA(e, cudaStreamSynchronize(s));
    float resid = 0.f;
    rc = read_stats(e, stats, &resid);
    if (rc) return rc;
    if (!(resid <= e->residual_limit)) {
        // FP32 rounding budget exceeded: recompute this block exactly (same inputs, same seed use)
        if (e->seed_left >= 0) ++e->seed_left;
        rc = block_common(e, e->d_key_start, e->d_key_rest, g, flags | PA_FLAG_EXACT, e->d_out, s);
        if (rc) return rc;
        PA_CUDA(e, cudaStreamSynchronize(s));
        float r2 = 0.f;
        rc = read_stats(e, stats, &r2);
        if (rc) return rc;
        if (stats) stats->max_residual = resid;  // report what the FP32 path measured
    }
    PA_CUDA(e, cudaMemcpy(out, e->d_out, ob, cudaMemcpyDeviceToHost));
    return PA_OK;
}

int pa_process_device(pa_engine* e, const uint32_t* d_key_start, const uint32_t* d_key_rest, uint32_t n, uint32_t v,
                      uint32_t flags, uint8_t* d_out, void* stream) {
    if (!e || !d_key_start || !d_out) return PA_ERR_INVALID_ARG;
    if ((flags & PA_FLAG_XOR_KEY_REST) && !d_key_rest) return PA_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(d_out) & 3u) return PA_ERR_INVALID_ARG;
    BlockGeom g;
    int rc = check_n(e, n, v, flags, &g);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
    PA_CUDA(e, cudaSetDevice(e->device));
    e->pending = true;
    return block_common(e, d_key_start, d_key_rest, g, flags, reinterpret_cast<uint32_t*>(d_out), s);
}

int pa_sync(pa_engine* e, pa_stats* stats) {
    if (!e) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    PA_CUDA(e, cudaDeviceSynchronize());
    e->pending = false;
    float resid = 0.f;
    int rc = read_stats(e, stats, &resid);
    if (rc) return rc;
    return resid <= e->residual_limit ? PA_OK : PA_ERR_PRECISION;
}

int pa_set_timing(pa_engine* e, int enable) {
    if (!e) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    if (enable && e->tev.empty()) {
        const size_t slots = 1024;
        e->tev.resize(slots);
        e->tev_stages.assign(slots, 0);
        for (auto& a : e->tev)
            for (auto& ev : a) PA_CUDA(e, cudaEventCreate(&ev));
    }
    e->timing = enable != 0;
    e->tev_next = e->tev_count = 0;
    return PA_OK;
}

int pa_stage_times(pa_engine* e, float* ms, int max_stages, int* nstages, int* nblocks) {
    if (!e || !ms || max_stages <= 0) return PA_ERR_INVALID_ARG;
    PA_CUDA(e, cudaSetDevice(e->device));
    double acc[4] = {0, 0, 0, 0};
    int stages = 0, blocks = 0;
    size_t n = e->tev_count, first = (e->tev_next + e->tev.size() - n) % std::max<size_t>(1, e->tev.size());
    for (size_t k = 0; k < n; ++k) {
        size_t slot = (first + k) % e->tev.size();
        int st = e->tev_stages[slot];
        if (blocks && st != stages) continue;  // average blocks of one shape only
        stages = st;
        PA_CUDA(e, cudaEventSynchronize(e->tev[slot][st]));
        for (int i = 0; i < st; ++i) {
            float t = 0.f;
            PA_CUDA(e, cudaEventElapsedTime(&t, e->tev[slot][i], e->tev[slot][i + 1]));
            acc[i] += t;
        }
        ++blocks;
    }
    for (int i = 0; i < std::min(stages, max_stages); ++i) ms[i] = blocks ? (float)(acc[i] / blocks) : 0.f;
    if (nstages) *nstages = stages;
    if (nblocks) *nblocks = blocks;
    e->tev_next = e->tev_count = 0;
    return PA_OK;
}

int pa_key_split(const uint32_t* recv_key, uint32_t n, uint32_t v, uint32_t* key_start, uint32_t* key_rest) {
    if (!recv_key || !key_start || !key_rest || (n & 31u) || (v & 31u) || v == 0 || v >= n)
        return PA_ERR_INVALID_ARG;
    uint32_t hb = (n - v) / 32u, vb = v / 32u, nb = n / 32u;
    std::memset(key_start, 0, (size_t)nb * 4u);
    std::memcpy(key_start, recv_key, (size_t)hb * 4u);
    key_start[hb] = recv_key[hb] & 0x80000000u;
    for (uint32_t i = 0; i < vb; ++i) key_rest[i] = (recv_key[hb + i] << 1) | (recv_key[hb + i + 1] >> 31);
    return PA_OK;
}

}  // extern "C"
