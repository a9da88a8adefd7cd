// pa_lanes.cu -- the persistent lane kernel (see pa_lanes.cuh) and its launch helpers.
//
// No counterpart in the reference, which runs one block at a time with a host sync after every step
// (PrivacyAmplification/PrivacyAmplification.cu:1686-2118).  The per-block arithmetic is the same pass
// bodies the per-pass kernels run (pa_pass_bodies.cuh).
#include "pa_lanes.cuh"
#include "pa_pass_bodies.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

namespace pa {

namespace {

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
__device__ __forceinline__ unsigned long long ld_acquire_sys_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void st_release_sys_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Inputs: device memory written before the launch (L2 loads), or host memory the host may have
// rewritten since the last block (loads that bypass the caches).
__device__ __forceinline__ uint32_t ld_in(const uint32_t* p, bool hostin) { return hostin ? __ldcv(p) : __ldcg(p); }

// Lane barrier: every CTA of the lane has finished the stage before any of them starts the next one.
// Thread 0 arrives (release) and polls the lane's counter (acquire) with a bounded number of rounds; the
// proxy fence orders the next stage's TMA and bulk reads after the generic writes of this one.  Returns
// false once the lane's error word is set (a wait expired here or in another CTA of the lane).
__device__ __forceinline__ bool lane_sync(const LaneArgs& a, int lane, unsigned int& target) {
    __shared__ int s_ok;
    target += (unsigned int)a.T;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        if (a.serve) __threadfence_system();  // served outputs go to host memory: visible to the host too
        else __threadfence();
        atomicAdd(a.bar + lane, 1u);
        for (uint32_t i = 0; (int)(ld_acquire_gpu(a.bar + lane) - target) < 0; ++i) {
            if (ld_volatile(a.err + lane)) {
                ok = 0;
                break;
            }
            if (i >= a.wait_limit) {
                atomicExch(a.err + lane, kErrLaneTimeout);
                ok = 0;
                break;
            }
            __nanosleep(128);
        }
        if (ok && ld_volatile(a.err + lane)) ok = 0;
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    fence_proxy_async_global();
    return s_ok != 0;
}

// ---------------------------------------------------------------------------------------- bit rows
// Key or seed bits -> bit rows (the transposes of k_bit_rows / k_bit_rows_tiled).  Tiled form (N1 >=
// 256, seed only when it is placed word by word): the two 256-thread halves of the CTA take one 256 x 256
// tile of 2-bit elements each, per round; otherwise every warp takes 16 rows x 32 columns, one word per
// lane.  The CTA takes rounds first, first + stride, ...
__device__ __noinline__ void lane_bit_rows(const uint32_t* __restrict__ src, bool seed, bool hostin,
                                              const BlockGeom& g, uint32_t* __restrict__ rows, uint32_t first,
                                              uint32_t stride) {
    const uint32_t n1 = 1u << g.log_n1, n2 = 1u << g.log_n2;
    // a power-of-two seed repeats with period n (word index mod n/32); any other n in a larger Np is placed
    // word by word (seed_word: the placement's boundaries fall between words)
    const bool periodic = seed && (g.n & (g.n - 1u)) == 0;
    const bool placed = seed && !periodic && (1u << g.log_np) != g.n;
    const uint64_t wmask = periodic ? (uint64_t)(g.n / 32u) - 1u : ~0ull;
    const int lane = threadIdx.x & 31;
    if (n1 >= 256u) {
        extern __shared__ __align__(16) uint32_t lane_smem[];
        uint32_t(*tile)[17] = reinterpret_cast<uint32_t(*)[17]>(lane_smem + (threadIdx.x >> 8) * (256 * 17));
        const int t = threadIdx.x & 255;
        const uint32_t tx = n1 / 256u, total = tx * (n2 / 256u);
        const uint32_t win = n1 / 16u, wout = n2 / 16u;
        for (uint32_t base = 2u * first; base < total; base += 2u * stride) {
            const uint32_t u = base + (threadIdx.x >> 8);
            const bool act = u < total;
            const uint32_t a0 = (u % tx) * 16u, m20 = (u / tx) * 256u;
            uint32_t v[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int r = (t >> 4) + 16 * i, w = t & 15;
                const uint64_t word = (uint64_t)(m20 + (uint32_t)r) * win + a0 + (uint32_t)w;
                const uint64_t x0 = 32ull * word;
                v[i] = (act && (seed || x0 <= g.h)) ? ld_in(src + (placed ? seed_word(g, x0) : (word & wmask)), hostin)
                                                    : 0u;
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int r = (t >> 4) + 16 * i, w = t & 15;
                const uint64_t x0 = 32ull * ((uint64_t)(m20 + (uint32_t)r) * win + a0 + (uint32_t)w);
                if (!seed && x0 <= g.h && x0 + 31 > g.h) v[i] &= ~(0xFFFFFFFFu >> (uint32_t)(g.h - x0 + 1));
                tile[r][w] = v[i];
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int b = (t >> 4) + 16 * i, cb = b >> 4, w = b & 15, L = lane & 15;
                v[i] = transpose16x2(tile[16 * cb + L][w], lane);
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int b = (t >> 4) + 16 * i, cb = b >> 4, w = b & 15, L = lane & 15;
                tile[16 * w + L][cb] = v[i];
            }
            __syncthreads();
            if (act) {
#pragma unroll 4
                for (int i = 0; i < 16; ++i) {
                    const int r = (t >> 4) + 16 * i, w = t & 15;
                    rows[(size_t)(16u * a0 + (uint32_t)r) * wout + m20 / 16u + (uint32_t)w] = tile[r][w];
                }
            }
            __syncthreads();  // the next round writes the tile again
        }
        return;
    }
    const uint32_t warp = threadIdx.x >> 5, ga = n1 / 16u, total = ga * (n2 / 32u);
    for (uint32_t task = first * 16u + warp; task < total; task += stride * 16u) {
        const uint32_t a = task % ga, c = task / ga;
        const uint32_t m2 = 32u * c + (uint32_t)lane;
        const uint64_t x0 = 2ull * n1 * m2 + 32ull * a;
        uint32_t v;
        if (!seed) {
            if (x0 + 31 <= g.h) v = ld_in(src + (x0 >> 5), hostin);
            else if (x0 > g.h) v = 0u;
            else v = ld_in(src + (x0 >> 5), hostin) & ~(0xFFFFFFFFu >> (uint32_t)(g.h - x0 + 1));
        } else if (!placed) {
            v = ld_in(src + ((x0 >> 5) & wmask), hostin);
        } else {
            v = ld_in(src + seed_word(g, x0), hostin);
        }
        const uint32_t w = transpose16x2(v, lane);
        rows[(size_t)(16u * a + (uint32_t)(lane & 15)) * (n2 / 16u) + 2u * c + (uint32_t)(lane >> 4)] = w;
    }
}

// ------------------------------------------------------------------------------------------ finish
// Parity planes -> output words with the key_rest XOR (the transposes of k_finish / k_finish_tiled).
// Tiled form (N1 >= 256): the two halves of the CTA take one 256-row x 8-word-column tile each, per
// round; otherwise every warp takes 32 plane rows x one word column.
__device__ __noinline__ void lane_finish(const uint32_t* __restrict__ planes, const BlockGeom& g,
                                            const uint32_t* __restrict__ key_rest, uint32_t flags, bool hostin,
                                            uint32_t* __restrict__ out, uint32_t first, uint32_t stride) {
    const uint32_t n1 = 1u << g.log_n1, wpr = (1u << g.log_n2) / 32u;
    const size_t plane_words = (size_t)n1 * wpr;
    const uint32_t nwords = (g.out_bits + 31u) / 32u;
    const uint32_t m2max = (uint32_t)(((uint64_t)g.out_bits + 2ull * n1 - 1ull) / (2ull * n1));
    const uint32_t cols = min(wpr, (m2max + 31u) / 32u);
    const bool xr = (flags & kXor) != 0;
    const int lane = threadIdx.x & 31;
    if (n1 >= 256u) {
        extern __shared__ __align__(16) uint32_t lane_smem[];
        uint32_t* base_smem = lane_smem + (threadIdx.x >> 8) * (2 * 256 * 9 + 256 * 17);
        uint32_t(*se)[9] = reinterpret_cast<uint32_t(*)[9]>(base_smem);
        uint32_t(*so)[9] = reinterpret_cast<uint32_t(*)[9]>(base_smem + 256 * 9);
        uint32_t(*sw)[17] = reinterpret_cast<uint32_t(*)[17]>(base_smem + 2 * 256 * 9);
        const int t = threadIdx.x & 255, warp = t >> 5;
        const uint32_t tx = n1 / 256u, total = tx * ((cols + 7u) / 8u);
        for (uint32_t base = 2u * first; base < total; base += 2u * stride) {
            const uint32_t u = base + (threadIdx.x >> 8);
            const bool act = u < total;
            const uint32_t m10 = (u % tx) * 256u, c0 = (u / tx) * 8u;
            uint32_t pv[16], kr[16];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int r = (t >> 3) + 32 * i, w = t & 7;
                const uint32_t c = c0 + (uint32_t)w;
                const size_t off = (size_t)(m10 + (uint32_t)r) * wpr + c;
                pv[2 * i] = (act && c < wpr) ? __ldcg(planes + off) : 0u;
                pv[2 * i + 1] = (act && c < wpr) ? __ldcg(planes + plane_words + off) : 0u;
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int ml = (t >> 4) + 16 * i, j = t & 15;
                const uint64_t ow = ((32ull * c0 + (uint64_t)ml) * n1 + m10) / 16ull + (uint64_t)j;
                kr[i] = (act && xr && ow < nwords && 32ull * ow < g.v) ? ld_in(key_rest + ow, hostin) : 0u;
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
                const int uu = warp + 8 * i, al = uu >> 3, cl = uu & 7;
                const uint32_t ve = se[32 * al + lane][cl], vo = so[32 * al + lane][cl];
                const uint32_t lo = transpose16x2(msb_pairs(ve, vo), lane);
                const uint32_t hi = transpose16x2(msb_pairs(ve >> 16, vo >> 16), lane);
                const int L = lane & 15, h = lane >> 4;
                sw[32 * cl + L][2 * al + h] = lo;
                sw[32 * cl + 16 + L][2 * al + h] = hi;
            }
            __syncthreads();
            if (act) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int ml = (t >> 4) + 16 * i, j = t & 15;
                    const uint64_t ow = ((32ull * c0 + (uint64_t)ml) * n1 + m10) / 16ull + (uint64_t)j;
                    if (ow < nwords) out[ow] = __byte_perm(sw[ml][j] ^ kr[i], 0, 0x0123);
                }
            }
            __syncthreads();  // the next round writes the tiles again
        }
        return;
    }
    const uint32_t warp = threadIdx.x >> 5, ga = n1 / 32u, total = ga * cols;
    for (uint32_t task = first * 16u + warp; task < total; task += stride * 16u) {
        const uint32_t a = task % ga, c = task / ga;
        const size_t off = (size_t)(32u * a + (uint32_t)lane) * wpr + c;
        const uint32_t ve = __ldcg(planes + off), vo = __ldcg(planes + plane_words + off);
        const uint32_t lo = transpose16x2(msb_pairs(ve, vo), lane);
        const uint32_t hi = transpose16x2(msb_pairs(ve >> 16, vo >> 16), lane);
        const uint32_t L = (uint32_t)(lane & 15), h = (uint32_t)(lane >> 4);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint64_t m2 = 32ull * c + L + 16u * k;
            const uint64_t ow = (m2 * n1 + 32ull * a + 16ull * h) / 16ull;
            if (ow >= nwords) continue;
            uint32_t w = k ? hi : lo;
            if (xr && 32ull * ow < g.v) w ^= ld_in(key_rest + ow, hostin);
            out[ow] = __byte_perm(w, 0, 0x0123);
        }
    }
}

// The stages below are separate functions (not inlined into the lane loop), so that each is register-
// allocated on its own as in the per-pass kernels; only the loop's few live values cross a call.
__device__ __noinline__ void lane_pass_a(const uint32_t* planes, const BlockGeom& g, float2* Y, unsigned long long* cnt,
                                         uint32_t first, uint32_t stride) {
    pass_a_rows<kLaneLogRow>(planes, g, Y, cnt, first, stride);
}

__device__ __noinline__ void lane_pass_c(const CUtensorMap* mapZ, const float2* Z, const BlockGeom& g,
                                         const unsigned long long* cnt, uint32_t* planes, unsigned int* resid, int* err,
                                         int early, uint32_t first, uint32_t stride) {
    pass_c_rows<kLaneLogRow, 8, kLaneThreads>(mapZ, Z, g, cnt, planes, resid, err, early, first, stride);
}

// Pass B of the block's column length (seed: the spectrum into spec; key: Z from Y and spec), one
// function per column length and direction.
template <int LG, bool SEED>
__device__ __noinline__ void lane_pass_b_t(const CUtensorMap* mapY, float2* Y, float2* Z, const BlockGeom& g,
                                           float2* spec, int* err, int early, uint32_t first, uint32_t stride) {
    pass_b_tiles<LG, SEED, kLaneThreads>(mapY, Y, Z, g, spec, err, early, first, stride);
}

__device__ __forceinline__ void lane_pass_b(bool seed, const CUtensorMap* mapY, float2* Y, float2* Z,
                                            const BlockGeom& g, float2* spec, int* err, int early, uint32_t first,
                                            uint32_t stride) {
#define PA_LANE_B(LG)                                                                     \
    case LG:                                                                              \
        if (seed) lane_pass_b_t<LG, true>(mapY, Y, Z, g, spec, err, early, first, stride); \
        else lane_pass_b_t<LG, false>(mapY, Y, Z, g, spec, err, early, first, stride);     \
        break;
    switch (g.log_n1) {
        PA_LANE_B(5) PA_LANE_B(6) PA_LANE_B(7) PA_LANE_B(8) PA_LANE_B(9) PA_LANE_B(10) PA_LANE_B(11) PA_LANE_B(12)
        default: break;
    }
#undef PA_LANE_B
}

// One block on one lane.  Returns false when a lane barrier failed (the lane's error word is set).
// Copies `words` words from host memory into the lane's device staging, the lane's CTAs taking
// interleaved runs of 512 consecutive words (coalesced loads that bypass the caches; the host may have
// rewritten the buffer since an earlier request).
__device__ __noinline__ void lane_stage_in(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, size_t words,
                                           uint32_t first, uint32_t stride) {
    const size_t step = (size_t)stride * kLaneThreads * 4;
    for (size_t base = (size_t)first * kLaneThreads * 4 + threadIdx.x; base < words; base += step) {
        uint32_t v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = base + (size_t)u * kLaneThreads;
            v[u] = i < words ? __ldcv(src + i) : 0u;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = base + (size_t)u * kLaneThreads;
            if (i < words) dst[i] = v[u];
        }
    }
}

__device__ __forceinline__ bool lane_block(const LaneArgs& a, const LaneJob& jin, bool hostin, int lane, int rank,
                                           unsigned int& target) {
    LaneJob j = jin;
    const BlockGeom g = j.g;
    float2* Y = a.work + (size_t)lane * a.work_stride;
    float2* Z = a.work2 + (size_t)lane * a.work_stride;
    uint32_t* planes = a.planes + (size_t)lane * a.planes_stride;
    const int mi = g.log_n1 - kLaneMinLogN1;
    const CUtensorMap* maps = a.maps + ((size_t)lane * kLaneMaps + (size_t)mi) * 2;
    int* err = a.err + lane;
    const uint32_t first = (uint32_t)rank, stride = (uint32_t)a.T;
    if (hostin) {  // a served request: its inputs move to the lane's device staging first, in one pass
        uint32_t* st = a.stage + (size_t)lane * a.stage_stride;
        const size_t wn = g.n / 32u, wh = g.h / 32u + 1u, wv = g.v / 32u;
        lane_stage_in(j.key_start, st, wh, first, stride);
        if (j.seed) lane_stage_in(j.seed, st + wn, wn, first, stride);
        if (j.key_rest) lane_stage_in(j.key_rest, st + 2 * wn, wv, first, stride);
        j.key_start = st;
        if (j.seed) j.seed = st + wn;
        if (j.key_rest) j.key_rest = st + 2 * wn;
        hostin = false;  // the output is still written to host memory directly
        if (!lane_sync(a, lane, target)) return false;
    }
    float2* spec = const_cast<float2*>(j.spec);
    // phase 0: the block's own seed (bit rows, pass A, pass B into its spectrum); phase 1: the key
    for (int phase = j.seed ? 0 : 1; phase < 2; ++phase) {
        const bool sp = phase == 0;
        lane_bit_rows(sp ? j.seed : j.key_start, sp, hostin, g, planes, first, stride);
        if (!lane_sync(a, lane, target)) return false;
        lane_pass_a(planes, g, Y, j.cnt + (sp ? 1 : 0), first, stride);
        if (!lane_sync(a, lane, target)) return false;
        if (sp) {
            spec = j.spec_out ? j.spec_out : a.spec + (size_t)lane * a.work_stride;
            lane_pass_b(true, maps, Y, Z, g, spec, err, a.early_b[mi], first, stride);
            if (!j.key_start) return true;  // a spectrum build: no key stages
            if (!lane_sync(a, lane, target)) return false;
            continue;
        }
        lane_pass_b(false, maps, Y, Z, g, spec, err, a.early_b[mi], first, stride);
        if (!lane_sync(a, lane, target)) return false;
        lane_pass_c(maps + 1, Z, g, j.cnt, planes, j.resid, err, a.early_c[mi], first, stride);
        if (!lane_sync(a, lane, target)) return false;
        lane_finish(planes, g, j.key_rest, j.flags, hostin, j.out, first, stride);
    }
    return true;
}

}  // namespace

// Batch: the next block of the list (atomic counter, longest first), its counters cleared.
__device__ __forceinline__ int batch_claim(const LaneArgs& a, int lane) {
    if (ld_volatile(a.err + lane)) return kLaneExit;
    const unsigned int k = atomicAdd(a.next, 1u);
    if (k >= a.njobs) return kLaneExit;
    const LaneJob& jb = a.jobs[k];
    jb.cnt[0] = 0ull;
    jb.cnt[1] = jb.seed_cnt ? *jb.seed_cnt : 0ull;
    *jb.resid = 0u;
    return (int)k;
}

// Serving loop: the next published request (ticket) not yet taken by any lane; its descriptor is copied
// from the host ring into the lane's device slot `buf` (two per lane, used in turn) with its counters,
// and `buf` is returned.  Two slots, because rank 0 takes the next request before the lane barrier, while
// the lane's other CTAs may still be finishing the previous request from the other slot and before that
// request's completion is published from it.  With nothing published the lane idles (a short sleep),
// and it ends when the host asks it to or after idle_ns without a request.
__device__ __forceinline__ int serve_claim(const LaneArgs& a, int lane, int buf, unsigned long long& idle_since) {
    if (ld_volatile(a.err + lane)) return kLaneExit;
    const unsigned long long tail = ld_acquire_sys_u64(&a.host->tail);
    for (;;) {
        const unsigned long long c = *reinterpret_cast<volatile unsigned long long*>(a.claimed);
        if (c >= tail) break;
        if (atomicCAS(a.claimed, c, c + 1ull) != c) continue;
        const volatile LaneJob* src = &a.ring[c % a.ring_size].job;
        LaneJob j;
        j.key_start = src->key_start;
        j.key_rest = src->key_rest;
        j.seed = src->seed;
        j.spec = src->spec;
        j.spec_out = nullptr;
        j.out = src->out;
        j.seed_cnt = src->seed_cnt;
        j.g.n = src->g.n;
        j.g.v = src->g.v;
        j.g.h = src->g.h;
        j.g.out_bits = src->g.out_bits;
        j.g.log_np = src->g.log_np;
        j.g.log_n = src->g.log_n;
        j.g.log_n1 = src->g.log_n1;
        j.g.log_n2 = src->g.log_n2;
        j.g.seed_direct = src->g.seed_direct;
        j.g.exact_only = src->g.exact_only;
        j.flags = src->flags;
        unsigned long long* st = a.lane_stats + 4 * (2 * lane + buf);
        j.cnt = st;
        j.resid = reinterpret_cast<unsigned int*>(st + 2);
        j.pad_ = 0;
        st[0] = 0ull;
        st[1] = j.seed_cnt ? *j.seed_cnt : 0ull;
        st[2] = 0ull;
        st[3] = c;  // the ticket, for the completion
        a.lane_job[2 * lane + buf] = j;
        idle_since = 0;
        return buf;
    }
    if (*reinterpret_cast<volatile int*>(&a.host->stop)) return kLaneExit;
    const unsigned long long now = global_ns();
    if (!idle_since) idle_since = now;
    else if (now - idle_since > a.idle_ns) return kLaneExit;
    __nanosleep(2000);
    return kLaneIdle;
}

// Completion of the lane's last request (device slot buf), once every CTA of the lane has passed the
// barrier after its finish stage: statistics into the host slot, then done = ticket + 1 (release at system
// scope).
__device__ __forceinline__ void serve_publish(const LaneArgs& a, int lane, int buf) {
    const unsigned long long* st = a.lane_stats + 4 * (2 * lane + buf);
    const unsigned long long tk = st[3];
    ServeSlot* s = a.ring + (tk % a.ring_size);
    volatile ServeSlot* vs = s;
    vs->cnt[0] = st[0];
    vs->cnt[1] = st[1];
    vs->resid = *reinterpret_cast<const unsigned int*>(st + 2);
    vs->err = ld_volatile(a.err + lane);
    __threadfence_system();
    st_release_sys_u64(&s->done, tk + 1ull);
}

// The lane loop: rank 0 of a lane takes the next block and writes its index to the lane's slot; a lane
// barrier hands it to the lane's other CTAs, which also separates the previous block's last stage from
// this block's first.
__global__ void __launch_bounds__(kLaneThreads, 1) k_lanes(const __grid_constant__ LaneArgs a) {
    const int lane = (int)blockIdx.x / a.T, rank = (int)blockIdx.x % a.T;
    if (lane >= a.lanes) return;
    __shared__ int s_job;
    unsigned int target = 0;
    unsigned long long idle_since = 0;
    int served = -1;  // serving: the device slot of this lane's request whose completion is not yet published
    int next_buf = 0;
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) {
            const int j = a.serve ? serve_claim(a, lane, next_buf, idle_since) : batch_claim(a, lane);
            *reinterpret_cast<volatile int*>(a.slot + lane) = j;
        }
        const bool ok = lane_sync(a, lane, target);
        if (served >= 0 && rank == 0 && threadIdx.x == 0) serve_publish(a, lane, served);
        served = -1;
        if (!ok) break;
        if (threadIdx.x == 0) s_job = ld_volatile(a.slot + lane);
        __syncthreads();
        const int j = s_job;
        if (j == kLaneIdle) continue;
        if (j < 0) break;
        if (!lane_block(a, a.serve ? a.lane_job[2 * lane + j] : a.jobs[j], a.serve != 0, lane, rank, target)) break;
        if (a.serve) {
            served = j;
            next_buf = j ^ 1;
        }
    }
}

// ------------------------------------------------------------------------------------- host helpers
static size_t lane_static_smem() {
    static const size_t bytes = [] {
        cudaFuncAttributes fa{};
        return cudaFuncGetAttributes(&fa, k_lanes) == cudaSuccess ? (size_t)fa.sharedSizeBytes : (size_t)0;
    }();
    return bytes;
}

size_t lane_smem_bytes() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return 0;
    const size_t st = lane_static_smem();
    if (st == 0 || (size_t)optin <= st + 1024) return 0;
    return (size_t)optin - st - 1024;
}

// Shared memory pass B needs besides its early boxes, with 512 threads and columns of 2^log_n1.
template <int LOGL>
static size_t pass_b_lane_bytes() {
    constexpr int L = 1 << LOGL, CPT = 32 * kLaneThreads / L, RL = Plan<LOGL>::RA, NSL = L / RL;
    constexpr bool LEAN = LOGL <= 6;
    constexpr int U1N = LEAN ? 0 : (NSL < 16 ? NSL : 16), U2N = LEAN ? 0 : NSL / U1N;
    constexpr size_t words = (size_t)CPT * TileStride<L>::value + (size_t)CPT * (RL + U1N + U2N) +
                             (size_t)PassBBases<LOGL, kLaneThreads>::SLOTS * kLaneThreads;
    return words * sizeof(float2) + 128;
}

static size_t pass_b_lane_bytes_rt(int log_n1) {
    switch (log_n1) {
        case 5: return pass_b_lane_bytes<5>();
        case 6: return pass_b_lane_bytes<6>();
        case 7: return pass_b_lane_bytes<7>();
        case 8: return pass_b_lane_bytes<8>();
        case 9: return pass_b_lane_bytes<9>();
        case 10: return pass_b_lane_bytes<10>();
        case 11: return pass_b_lane_bytes<11>();
        case 12: return pass_b_lane_bytes<12>();
        default: return 0;
    }
}

int lane_early_boxes(int log_n1, int pass, size_t dyn) {
    const uint32_t n1 = 1u << log_n1;
    const uint32_t cpt = (32u * kLaneThreads) >> log_n1;  // pass B tile width (columns)
    if (cpt > 128u) return 0;                              // per-thread copies instead of TMA boxes
    if (pass == 'b') {
        const size_t need = pass_b_lane_bytes_rt(log_n1);
        const uint32_t boxr = n1 < 256u ? n1 : 256u, nbox = n1 / boxr;
        const size_t box = (size_t)boxr * cpt * sizeof(float2);
        if (dyn <= need) return 0;
        return (int)std::min<size_t>(nbox, (dyn - need) / box);
    }
    const uint32_t ntiles = (1u << kLaneLogRow) / cpt, boxt = ntiles < 256u ? ntiles : 256u, nb = ntiles / boxt;
    const size_t box = (size_t)boxt * cpt * sizeof(float2);
    const size_t exch = (size_t)TileStride<(1 << kLaneLogRow)>::value * sizeof(float2) + 128;
    if (dyn <= exch) return 0;
    return (int)std::min<size_t>(nb, (dyn - exch) / box);
}

int lane_max_ctas(int* ctas) {
    int dev = 0, sms = 0, per = 0;
    const size_t smem = lane_smem_bytes();
    if (!smem) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lanes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lanes, kLaneThreads, smem);
    if (e != cudaSuccess) return (int)e;
    *ctas = per * sms;
    return 0;
}

int launch_lanes(const LaneArgs& a, int grid, size_t smem, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(k_lanes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kLaneThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident at once: lane barriers never wait on
    attr[0].val.cooperative = 1;                   // a CTA that has not started
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return (int)cudaLaunchKernelEx(&cfg, k_lanes, a);
}

int make_lane_maps(const float2* Y, const float2* Z, CUtensorMap* out) {
    std::memset(out, 0, sizeof(CUtensorMap) * kLaneMaps * 2);
    for (int ln1 = kLaneMinLogN1; ln1 <= kLaneMaxLogN1; ++ln1) {
        const uint32_t cpt = (32u * kLaneThreads) >> ln1;
        if (cpt > 128u) continue;  // per-thread copies instead of TMA boxes
        int rc = encode_pass_maps(ln1, kLaneLogRow, cpt, Y, Z, out + 2 * (ln1 - kLaneMinLogN1));
        if (rc) return rc;
    }
    return 0;
}

}  // namespace pa
