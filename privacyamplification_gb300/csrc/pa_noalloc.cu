// pa_noalloc.cu -- pa_process_noalloc: one small block without any device allocation.
//
// Some callers cannot call cudaMalloc at all: a host whose device memory is owned by another
// allocator (a framework's caching pool that must see every byte), a latency-critical loop that may
// not take the implicit synchronisation of an allocation, or a deployment that fixes its memory map
// at start-up.  For them this entry point runs the single-CTA path of one block (n <= 2^15) on
// buffers the caller already owns; the only other device memory it touches is the scratch below,
// which lives in the library image itself.
//
// The scratch is a file-scope __device__ array: every GPU that loads the library holds it until the
// process exits, every call on that GPU shares it, and it keeps the previous call's contents.  Calls
// that overlap on the GPU (different streams, or different host threads on one device) race on it.
#include "../../include/pa_gb300.h"
#include "pa_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>

namespace {

// Largest block: n = 2^15 bits -> N = 2^14 complex seed-spectrum values.
constexpr uint32_t kMaxN = 1u << 15;
constexpr size_t kSpecBytes = (size_t)(kMaxN / 2) * sizeof(float2);   // 128 KiB
constexpr size_t kScratchBytes = kSpecBytes + 256;                       // + popcounts, residual word

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch in the current context.  In host code the symbol is only a
// host-side stand-in, so the address comes from cudaGetSymbolAddress with the caller's device current.
// It is looked up on every call rather than cached: after a cudaDeviceReset, or under a context the
// caller made current itself, the library's device code is loaded again and the array moves.  The
// lookup costs about a microsecond; the first one in a context also loads the library's device code.
int scratch_address(void** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PA_ERR_CUDA;
    *out = p;
    return PA_OK;
}

int ceil_log2u(uint64_t x) {
    int l = 0;
    while ((1ull << l) < x) ++l;
    return l;
}

// Geometry of a block for the single-CTA path (same placement rules as the engine).
int small_geom(uint32_t n, uint32_t v, uint32_t flags, pa::BlockGeom* g) {
    if (n < 1024u || (n & 31u) || (v & 31u) || v == 0 || v >= n) return PA_ERR_INVALID_ARG;
    if (n > kMaxN) return PA_ERR_TOO_LARGE;
    g->n = n;
    g->v = v;
    g->h = n - v;
    g->out_bits = (flags & PA_FLAG_COMPRESS) ? v : n / 2u;
    const bool pow2 = (n & (n - 1u)) == 0;
    if (pow2) {
        g->log_np = ceil_log2u(n);
        g->seed_direct = n;
    } else {
        g->log_np = ceil_log2u(std::max<uint64_t>(n, (uint64_t)g->out_bits + g->h));
        g->seed_direct = (uint32_t)std::min<uint64_t>((1ull << g->log_np) - g->h, n);
    }
    g->log_n = g->log_np - 1;
    g->log_n1 = g->log_n2 = 0;
    g->exact_only = 0;
    if (g->log_n > 14) return PA_ERR_TOO_LARGE;  // padded length beyond one CTA
    return PA_OK;
}

}  // namespace

extern "C" int pa_process_noalloc(const uint32_t* d_seed_words, const uint32_t* d_key_start,
                                  const uint32_t* d_key_rest, uint32_t n, uint32_t v, uint32_t flags,
                                  uint8_t* d_out, void* stream) {
    if (!d_seed_words || !d_key_start || !d_out) return PA_ERR_INVALID_ARG;
    if ((flags & PA_FLAG_XOR_KEY_REST) && !d_key_rest) return PA_ERR_INVALID_ARG;
    if (flags & PA_FLAG_EXACT) return PA_ERR_INVALID_ARG;  // the exact path needs allocated buffers
    if (reinterpret_cast<uintptr_t>(d_out) & 3u) return PA_ERR_INVALID_ARG;
    pa::BlockGeom g;
    int rc = small_geom(n, v, flags, &g);
    if (rc) return rc;
    void* base = nullptr;
    rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    float2* spec = reinterpret_cast<float2*>(base);
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(static_cast<unsigned char*>(base) + kSpecBytes);
    unsigned int* resid = reinterpret_cast<unsigned int*>(cnt + 2);
    // the scratch keeps the last call's contents: clear the counters and the residual word
    if (cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long) + sizeof(unsigned int), s) != cudaSuccess)
        return PA_ERR_CUDA;
    const pa::Scratch none{nullptr, nullptr, nullptr, nullptr, nullptr};  // unused by the single-CTA path
    if (pa::launch_seed_spectrum(g, d_seed_words, spec, none, cnt + 1, 1, s) != 0) return PA_ERR_CUDA;
    if (pa::launch_key_block(g, d_key_start, d_key_rest, flags, spec, none, cnt, resid,
                             reinterpret_cast<uint32_t*>(d_out), 1, s, nullptr) != 0)
        return PA_ERR_CUDA;
    return PA_OK;
}
