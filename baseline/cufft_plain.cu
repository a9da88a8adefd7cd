// cufft_plain.cu -- GPU baseline: the reference's plain single-block pipeline on cuFFT.
//
// This is NOT part of the engine.  It restates, in code written for this project, the sequence the
// reference's CUDA build runs per block (PrivacyAmplification/PrivacyAmplification.cu, mainloop
// :1797-2042) so that the engine can be timed against it on the same GPU and the same inputs:
//
//   binInt2float(seed) :1831 (only when the seed is recalculated)   -> sync
//   binInt2float(key)  :1867                                         -> sync
//   calculateCorrectionFloat :1885 (one thread)                      -> sync
//   cufftExecR2C(key) :1898, cufftExecR2C(seed) :1903 (if recalc)    -> cudaDeviceSynchronize after each
//   setFirstElementToZero :1941                                      -> sync
//   ElementWiseProduct :1966                                         -> sync
//   cufftExecC2R :1979                                               -> cudaDeviceSynchronize
//   ToBinaryArray / ToBinaryArrayNoXOR :2029-2036                    -> sync
//
// As in the reference, the seed/key/key_rest ring slots and the output slot are pinned host memory
// (cudaMallocHost, :1537-1552) that the kernels read and write directly, the launch shapes are the
// reference's (1024-bit unpack blocks, 992-bit pack blocks), the unpack counts ones with one atomic
// per set bit, the FP32 constants are h1 = 2^-11, r = 2^5, normalisation n / 2^32 (:1597, :1729), and
// the cuFFT plans are single 1-D R2C / C2R plans of length n (:1736, :1745).  The host syncs between
// steps are kept because they are part of what the reference's per-block time measures.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>

#define CP_API extern "C" __attribute__((visibility("default")))

namespace {

// The reference's own kernels (binInt2float, calculateCorrectionFloat, setFirstElementToZero,
// ElementWiseProduct, ToBinaryArray[NoXOR]), compiled for sm_103a from PrivacyAmplification.cu by
// baseline/ref_cuda.py into a fatbin and loaded at run time (cp_load_reference).  When they are loaded,
// cp_process launches them, with the reference's launch shapes and its __constant__ values, in place of
// the restated kernels below; cuFFT, the pinned slots and the host syncs are the same either way.
struct RefKernels {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t unpack = nullptr, corr = nullptr, zero = nullptr, product = nullptr, pack = nullptr,
                 pack_noxor = nullptr;
};
RefKernels g_ref;

constexpr float kH1 = 1.0f / 2048.0f;  // 1 / 2^reduction_exp
constexpr float kR = 32.0f;            // 2^pre_mul_reduction_exp

struct Plain {
    uint32_t n = 0, v = 0;
    cufftHandle fwd = 0, inv = 0;
    float* di1 = nullptr;   // key as floats (n)
    float* di2 = nullptr;   // seed as floats, later the C2R output (n + 992)
    float2* do1 = nullptr;  // key spectrum, product in place
    float2* do2 = nullptr;  // seed spectrum (kept for a static seed)
    uint32_t* cnt = nullptr;  // [0] seed ones, [1] key ones
    float* corr = nullptr;
    float* resid = nullptr;
    uint32_t *h_seed = nullptr, *h_ks = nullptr, *h_kr = nullptr;
    uint8_t* h_out = nullptr;
    cudaStream_t s = nullptr;
    bool seed_ready = false;
    double step_ms[8] = {};  // host wall time of each step of the last block (see cp_step_ms)
};

// One thread per bit, 1024 bits per block; a set bit stores h1 and adds 1 to the counter.
__global__ void k_unpack(const uint32_t* __restrict__ words, float* __restrict__ out, uint32_t* ones) {
    __shared__ uint32_t w[32];
    const uint32_t t = threadIdx.x;
    if (t < 32) w[t] = words[32u * blockIdx.x + t];
    __syncthreads();
    const uint32_t bit = (w[t >> 5] >> (31u - (t & 31u))) & 1u;
    if (bit) atomicAdd(ones, 1u);
    out[1024u * blockIdx.x + t] = bit ? kH1 : 0.0f;
}

// corr = fmod(((Cs * Ck) mod 2^32) / n, 2): the product is taken in 32-bit arithmetic.
__global__ void k_correction(const uint32_t* cnt, float* corr, uint32_t n) {
    const uint32_t prod = cnt[0] * cnt[1];
    *corr = (float)fmod((double)prod / (double)n, 2.0);
}

__global__ void k_zero_dc(float2* a, float2* b) {
    if (threadIdx.x == 0) a[0] = make_float2(0.f, 0.f);
    else b[0] = make_float2(0.f, 0.f);
}

// key spectrum <- (key / r) * (seed / r), complex, in place.
__global__ void k_product(float2* __restrict__ key, const float2* __restrict__ seed, uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float2 a = key[i], b = seed[i];
    const float ax = a.x / kR, ay = a.y / kR, bx = b.x / kR, by = b.y / kR;
    key[i] = make_float2(ax * bx - ay * by, ax * by + ay * bx);
}

// 992 output bits (31 words) per block: rint(x / norm + corr) & 1, bit i of a word at byte i/8,
// bit 7 - i%8; with XOR, key_rest words are byte-swapped into the same layout.
template <bool XOR>
__global__ void k_pack(const float* __restrict__ inv, uint32_t* __restrict__ out, const uint32_t* __restrict__ key_rest,
                       const float* corr_p, float norm) {
    __shared__ uint32_t bits[992];
    __shared__ uint32_t kr[31];
    const uint32_t t = threadIdx.x, b = blockIdx.x;
    const float corr = *corr_p;
    if (t < 992) {
        const uint32_t k = t & 31u;
        const uint32_t shift = 8u * (k >> 3) + 7u - (k & 7u);
        bits[t] = ((uint32_t)__float2int_rn(inv[b * 992u + t] / norm + corr) & 1u) << shift;
    } else if (XOR && t < 1023) {
        const uint32_t x = key_rest[b * 31u + t - 992u];
        kr[t - 992] = __byte_perm(x, 0, 0x0123);
    }
    __syncthreads();
    if (t < 31) {
        uint32_t w = 0;
        for (int k = 0; k < 32; ++k) w |= bits[t * 32u + k];
        if (XOR) w ^= kr[t];
        out[b * 31u + t] = w;
    }
}

// Untimed diagnostics: largest distance of an output value from the nearest integer.
__global__ void k_residual(const float* __restrict__ inv, uint32_t count, const float* corr_p, float norm, float* res) {
    float m = 0.f;
    const float corr = *corr_p;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float x = inv[i] / norm + corr;
        m = fmaxf(m, fabsf(x - rintf(x)));
    }
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned int*>(res), __float_as_uint(m));
}

void destroy(Plain* p) {
    if (!p) return;
    if (p->fwd) cufftDestroy(p->fwd);
    if (p->inv) cufftDestroy(p->inv);
    cudaFree(p->di1);
    cudaFree(p->di2);
    cudaFree(p->do1);
    cudaFree(p->do2);
    cudaFree(p->cnt);
    cudaFree(p->corr);
    cudaFree(p->resid);
    cudaFreeHost(p->h_seed);
    cudaFreeHost(p->h_ks);
    cudaFreeHost(p->h_kr);
    cudaFreeHost(p->h_out);
    if (p->s) cudaStreamDestroy(p->s);
    delete p;
}

#define CP_TRY(x)                                     \
    do {                                              \
        if ((x) != cudaSuccess) return -2;            \
    } while (0)
#define CP_FFT(x)                                     \
    do {                                              \
        if ((x) != CUFFT_SUCCESS) return -3;          \
    } while (0)

}  // namespace

// n: power of two in [2^10, 2^30]; v: multiple of 32 below n.  Returns 0 or a negative code.
CP_API int cp_create(uint32_t n, uint32_t v, void** out) {
    if (!out || n < 1024u || (n & (n - 1u)) || (v & 31u) || v == 0 || v >= n) return -1;
    Plain* p = new (std::nothrow) Plain;
    if (!p) return -2;
    p->n = n;
    p->v = v;
    const size_t words = n / 32u;
    auto fail = [&](int rc) {
        destroy(p);
        return rc;
    };
    // the reference's buffer sizes (PrivacyAmplification.cu:1572-1592): its kernels write past the n/2 + 1
    // spectrum bins (ElementWiseProduct has no bounds check; its grid is rounded up to 1024 threads)
    const size_t di1_floats = 2 * (((size_t)n + 992) / 2 + 1);
    if (cudaMalloc(&p->di1, di1_floats * sizeof(float)) != cudaSuccess) return fail(-2);
    if (cudaMalloc(&p->di2, ((size_t)n + 992) * sizeof(float)) != cudaSuccess) return fail(-2);
    if (cudaMalloc(&p->do1, (size_t)n * sizeof(float2)) != cudaSuccess) return fail(-2);
    if (cudaMalloc(&p->do2, std::max((size_t)n * sizeof(float2), ((size_t)n + 992) * sizeof(float))) != cudaSuccess)
        return fail(-2);
    if (cudaMalloc(&p->cnt, 2 * sizeof(uint32_t)) != cudaSuccess) return fail(-2);
    if (cudaMalloc(&p->corr, sizeof(float)) != cudaSuccess) return fail(-2);
    if (cudaMalloc(&p->resid, sizeof(float)) != cudaSuccess) return fail(-2);
    if (cudaMallocHost(&p->h_seed, words * 4) != cudaSuccess) return fail(-2);
    if (cudaMallocHost(&p->h_ks, words * 4) != cudaSuccess) return fail(-2);
    if (cudaMallocHost(&p->h_kr, (words + 31) * 4) != cudaSuccess) return fail(-2);
    if (cudaMallocHost(&p->h_out, (words + 31) * 4) != cudaSuccess) return fail(-2);
    if (cudaStreamCreateWithFlags(&p->s, cudaStreamNonBlocking) != cudaSuccess) return fail(-2);
    std::memset(p->h_seed, 0, words * 4);
    std::memset(p->h_ks, 0, words * 4);
    std::memset(p->h_kr, 0, (words + 31) * 4);
    if (cudaMemset(p->di1, 0, di1_floats * sizeof(float)) != cudaSuccess) return fail(-2);
    if (cudaMemset(p->di2, 0, ((size_t)n + 992) * sizeof(float)) != cudaSuccess) return fail(-2);
    if (cufftPlan1d(&p->fwd, (int)n, CUFFT_R2C, 1) != CUFFT_SUCCESS) return fail(-3);
    if (cufftPlan1d(&p->inv, (int)n, CUFFT_C2R, 1) != CUFFT_SUCCESS) return fail(-3);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(-2);
    *out = p;
    return 0;
}

CP_API void cp_destroy(void* h) { destroy(static_cast<Plain*>(h)); }

// Pinned host slots: seed n/32 words, key_start n/32 words (zero past word h/32), key_rest v/32 + 31
// words, output (n/32 + 31) words.
CP_API uint32_t* cp_seed_slot(void* h) { return static_cast<Plain*>(h)->h_seed; }
CP_API uint32_t* cp_key_start_slot(void* h) { return static_cast<Plain*>(h)->h_ks; }
CP_API uint32_t* cp_key_rest_slot(void* h) { return static_cast<Plain*>(h)->h_kr; }
CP_API uint8_t* cp_output_slot(void* h) { return static_cast<Plain*>(h)->h_out; }

// One block from the slots, synchronous.  recalc_seed = 0 reuses the last seed spectrum (the first
// call always computes it).  wall_ms receives the host wall time of the whole sequence.
CP_API int cp_process(void* h, int recalc_seed, int do_xor, int do_compress, double* wall_ms) {
    Plain* p = static_cast<Plain*>(h);
    const uint32_t n = p->n, hl = n - p->v;
    const bool seed = recalc_seed || !p->seed_ready;
    const auto t0 = std::chrono::steady_clock::now();
    auto tprev = t0;
    auto mark = [&](int i) {  // each step ends in a host sync, so wall time per step is its cost
        const auto now = std::chrono::steady_clock::now();
        p->step_ms[i] = std::chrono::duration<double, std::milli>(now - tprev).count();
        tprev = now;
    };
    for (double& x : p->step_ms) x = 0.0;
    cudaStream_t s = p->s;
    const bool ref = g_ref.lib != nullptr;
    auto launch = [&](cudaKernel_t k, uint32_t grid, uint32_t block, void** args) {
        return cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(grid), dim3(block), args, 0, s);
    };
    uint32_t* cnt_seed = p->cnt;
    uint32_t* cnt_key = p->cnt + 1;
    if (seed) {
        CP_TRY(cudaMemsetAsync(p->cnt, 0, 2 * sizeof(uint32_t), s));
        if (ref) {
            void* a[] = {&p->h_seed, &p->di2, &cnt_seed};
            CP_TRY(launch(g_ref.unpack, (n + 1023u) / 1024u, n < 1024u ? n : 1024u, a));
        } else {
            k_unpack<<<(n + 1023u) / 1024u, 1024, 0, s>>>(p->h_seed, p->di2, p->cnt);
        }
        CP_TRY(cudaStreamSynchronize(s));
    } else {
        CP_TRY(cudaMemsetAsync(p->cnt + 1, 0, sizeof(uint32_t), s));
    }
    mark(0);
    const uint32_t key_words = hl / 32u + 1u;
    if (ref) {
        void* a[] = {&p->h_ks, &p->di1, &cnt_key};
        CP_TRY(launch(g_ref.unpack, (key_words * 32u + 1023u) / 1024u, key_words * 32u < 1024u ? key_words * 32u : 1024u,
                      a));
    } else {
        k_unpack<<<(key_words * 32u + 1023u) / 1024u, 1024, 0, s>>>(p->h_ks, p->di1, p->cnt + 1);
    }
    CP_TRY(cudaStreamSynchronize(s));
    mark(1);
    if (ref) {
        void* a[] = {&cnt_seed, &cnt_key, &p->corr};
        CP_TRY(launch(g_ref.corr, 1, 1, a));
    } else {
        k_correction<<<1, 1, 0, s>>>(p->cnt, p->corr, n);
    }
    CP_TRY(cudaStreamSynchronize(s));
    mark(2);
    CP_FFT(cufftSetStream(p->fwd, s));
    CP_FFT(cufftExecR2C(p->fwd, p->di1, reinterpret_cast<cufftComplex*>(p->do1)));
    CP_TRY(cudaDeviceSynchronize());
    mark(3);
    if (seed) {
        CP_FFT(cufftExecR2C(p->fwd, p->di2, reinterpret_cast<cufftComplex*>(p->do2)));
        CP_TRY(cudaDeviceSynchronize());
        p->seed_ready = true;
    }
    mark(4);
    const uint32_t bins = n / 2u + 1u;
    if (ref) {
        void* a[] = {&p->do1, &p->do2};
        CP_TRY(launch(g_ref.zero, 1, 2, a));
        CP_TRY(cudaStreamSynchronize(s));
        CP_TRY(launch(g_ref.product, (bins + 1023u) / 1024u, bins < 1024u ? bins : 1024u, a));
    } else {
        k_zero_dc<<<1, 2, 0, s>>>(p->do1, p->do2);
        CP_TRY(cudaStreamSynchronize(s));
        k_product<<<(bins + 1023u) / 1024u, bins < 1024u ? bins : 1024u, 0, s>>>(p->do1, p->do2, bins);
    }
    CP_TRY(cudaStreamSynchronize(s));
    mark(5);
    CP_FFT(cufftSetStream(p->inv, s));
    CP_FFT(cufftExecC2R(p->inv, reinterpret_cast<cufftComplex*>(p->do1), p->di2));
    CP_TRY(cudaDeviceSynchronize());
    mark(6);
    const float norm = (float)n / (2048.0f * kR) / (2048.0f * kR);
    uint32_t* out = reinterpret_cast<uint32_t*>(p->h_out);
    if (ref) {
        if (do_xor) {
            void* a[] = {&p->di2, &out, &p->h_kr, &p->corr};
            CP_TRY(launch(g_ref.pack, p->v / 32u / 31u + 1u, 1023, a));
        } else {
            const uint32_t words = do_compress ? p->v / 32u : n / 64u;
            void* a[] = {&p->di2, &out, &p->corr};
            CP_TRY(launch(g_ref.pack_noxor, words / 31u + 1u, 1023, a));
        }
    } else if (do_xor) {
        k_pack<true><<<p->v / 32u / 31u + 1u, 1023, 0, s>>>(p->di2, out, p->h_kr, p->corr, norm);
    } else {
        const uint32_t words = do_compress ? p->v / 32u : n / 64u;
        k_pack<false><<<words / 31u + 1u, 1023, 0, s>>>(p->di2, out, nullptr, p->corr, norm);
    }
    CP_TRY(cudaStreamSynchronize(s));
    mark(7);
    CP_TRY(cudaGetLastError());
    if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

// Host wall time (ms) of each step of the last cp_process, 8 values: seed unpack, key unpack,
// correction, R2C key, R2C seed, zero DC + product, C2R, pack to the pinned output.
CP_API void cp_step_ms(void* h, double* ms) {
    for (int i = 0; i < 8; ++i) ms[i] = static_cast<Plain*>(h)->step_ms[i];
}

// After cp_process: largest distance from the nearest integer over the first out_bits outputs.
CP_API int cp_residual(void* h, uint32_t out_bits, float* max_resid) {
    Plain* p = static_cast<Plain*>(h);
    if (out_bits > p->n) return -1;
    const float norm = (float)p->n / (2048.0f * kR) / (2048.0f * kR);
    CP_TRY(cudaMemsetAsync(p->resid, 0, sizeof(float), p->s));
    k_residual<<<1216, 256, 0, p->s>>>(p->di2, out_bits, p->corr, norm, p->resid);
    CP_TRY(cudaMemcpyAsync(max_resid, p->resid, sizeof(float), cudaMemcpyDeviceToHost, p->s));
    CP_TRY(cudaStreamSynchronize(p->s));
    return 0;
}

// Loads the reference's kernels from a fatbin built from PrivacyAmplification.cu (baseline/ref_cuda.py)
// and sets their __constant__ values for blocks of n bits (PrivacyAmplification.cu:1597-1606, 1729-1732):
// c0 = 0, h0 = 0, h1_reduced = 2^-11, sample_size = n, pre_mul_reduction = 2^5,
// normalisation_float = n / (2^11 2^5)^2.  Returns 0, or a negative code when the file or a kernel is
// missing.  From then on cp_process launches the reference's kernels (cp_unload_reference undoes it).
CP_API int cp_load_reference(const char* path, uint32_t n) {
    cudaLibrary_t lib = g_ref.lib;
    RefKernels r = g_ref;
    if (lib) goto constants;  // loaded: only the constants for n
    if (cudaLibraryLoadFromFile(&lib, path, nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
        cudaGetLastError();
        return -4;
    }
    {
    cudaKernel_t ks[64];
    unsigned int count = 0;
    if (cudaLibraryGetKernelCount(&count, lib) != cudaSuccess || count == 0 || count > 64 ||
        cudaLibraryEnumerateKernels(ks, count, lib) != cudaSuccess) {
        cudaLibraryUnload(lib);
        return -5;
    }
    r.lib = lib;
    for (unsigned int i = 0; i < count; ++i) {
        const char* name = nullptr;
        if (cudaFuncGetName(&name, reinterpret_cast<const void*>(ks[i])) != cudaSuccess || !name) continue;
        if (std::strstr(name, "binInt2float")) r.unpack = ks[i];
        else if (std::strstr(name, "calculateCorrectionFloat")) r.corr = ks[i];
        else if (std::strstr(name, "setFirstElementToZero")) r.zero = ks[i];
        else if (std::strstr(name, "ElementWiseProduct")) r.product = ks[i];
        else if (std::strstr(name, "ToBinaryArrayNoXOR")) r.pack_noxor = ks[i];
        else if (std::strstr(name, "ToBinaryArray")) r.pack = ks[i];
    }
    if (!r.unpack || !r.corr || !r.zero || !r.product || !r.pack || !r.pack_noxor) {
        cudaLibraryUnload(lib);
        return -6;
    }
    }
constants:
    const float zero = 0.0f, h1 = kH1, normf = (float)n / (2048.0f * kR) / (2048.0f * kR);
    const float2 c0 = make_float2(0.f, 0.f);
    const uint32_t pre = (uint32_t)kR;
    struct Sym {
        const char* name;
        const void* val;
        size_t bytes;
    } syms[] = {{"c0_dev", &c0, sizeof(c0)},
                {"h0_dev", &zero, sizeof(zero)},
                {"h1_reduced_dev", &h1, sizeof(h1)},
                {"normalisation_float_dev", &normf, sizeof(normf)},
                {"sample_size_dev", &n, sizeof(n)},
                {"pre_mul_reduction_dev", &pre, sizeof(pre)}};
    for (const Sym& sy : syms) {
        void* dptr = nullptr;
        size_t bytes = 0;
        if (cudaLibraryGetGlobal(&dptr, &bytes, lib, sy.name) != cudaSuccess || bytes != sy.bytes ||
            cudaMemcpy(dptr, sy.val, sy.bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            if (!g_ref.lib) cudaLibraryUnload(lib);
            return -7;
        }
    }
    g_ref = r;
    return 0;
}

CP_API void cp_unload_reference() {
    if (g_ref.lib) cudaLibraryUnload(g_ref.lib);
    g_ref = RefKernels{};
}
