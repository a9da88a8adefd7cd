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

// ============================================================================ sub-block bank
// The reference's sub-block variant (PrivacyAmplification/PrivacyAmplification_subblocks.cu): a bank of
// 2^27 bits cut into B = 2^27 / s sub-blocks of s bits (:1006-1031; its speedtest sweeps s = 2^10..2^27
// with v = s/4 + s/8, :1210-1236), every step one launch over the whole bank and the transforms one
// batched cuFFT plan per direction (cufftPlan1d(s, R2C / C2R, B), :1058-1081).  Each sub-block is an
// ordinary block with its own seed, key and counts, so the restatement here keeps the per-sub-block
// counts, corrections and DC bins (the reference file's own kernels do not: it is not built by any of
// its Makefiles).  Unlike cp_process, the bank runs from device memory with no host sync between steps,
// and is timed with CUDA events: the strongest form of the batched-cuFFT design, to hold the engine's
// batch of equal blocks against.
namespace {

struct Bank {
    uint32_t s = 0, v = 0, B = 0, log_s = 0;
    cufftHandle fwd = 0, inv = 0;
    uint32_t *seed = nullptr, *ks = nullptr, *kr = nullptr, *out = nullptr;  // device words
    float *di1 = nullptr, *di2 = nullptr;
    float2 *do1 = nullptr, *do2 = nullptr;
    uint32_t* cnt = nullptr;  // [0, B) seed ones, [B, 2B) key ones
    float* corr = nullptr;    // B
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool seed_ready = false;
};

// One thread per bit of the bank, 1024 bits per CUDA block (s >= 1024: a CUDA block never straddles
// two sub-blocks); a set bit stores h1 and adds 1 to its sub-block's counter.
__global__ void k_unpack_bank(const uint32_t* __restrict__ words, float* __restrict__ out, uint32_t* ones,
                              uint32_t log_s) {
    __shared__ uint32_t w[32];
    const uint32_t t = threadIdx.x;
    const size_t base = (size_t)blockIdx.x * 1024u;
    if (t < 32) w[t] = words[base / 32u + t];
    __syncthreads();
    const uint32_t bit = (w[t >> 5] >> (31u - (t & 31u))) & 1u;
    if (bit) atomicAdd(ones + (base >> log_s), 1u);
    out[base + t] = bit ? kH1 : 0.0f;
}

__global__ void k_correction_bank(const uint32_t* cnt, float* corr, uint32_t B, uint32_t s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    const uint32_t prod = cnt[i] * cnt[B + i];
    corr[i] = (float)fmod((double)prod / (double)s, 2.0);
}

__global__ void k_zero_dc_bank(float2* a, float2* b, uint32_t B, uint32_t dist) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    a[(size_t)i * dist] = make_float2(0.f, 0.f);
    b[(size_t)i * dist] = make_float2(0.f, 0.f);
}

__global__ void k_product_bank(float2* __restrict__ key, const float2* __restrict__ seed, size_t count) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float2 a = key[i], b = seed[i];
    const float ax = a.x / kR, ay = a.y / kR, bx = b.x / kR, by = b.y / kR;
    key[i] = make_float2(ax * bx - ay * by, ax * by + ay * bx);
}

// One thread per output bit: rint(x / norm + corr) & 1, a warp's 32 bits gathered by ballot into one
// word in the reference's byte order (bit k at byte k/8, bit 7 - k%8), XORed with key_rest in the same
// layout.  Grid: (v/32 words per sub-block / 8 warps, B).
template <bool XOR>
__global__ void k_pack_bank(const float* __restrict__ inv, uint32_t* __restrict__ out,
                            const uint32_t* __restrict__ key_rest, const float* corr, uint32_t s, uint32_t v,
                            float norm) {
    const uint32_t i = blockIdx.y, words = v / 32u;
    const uint32_t word = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
    if (word >= words) return;  // whole warps
    const uint32_t lane = threadIdx.x & 31u;
    const float x = inv[(size_t)i * s + word * 32u + lane] / norm + corr[i];
    const uint32_t bits = __ballot_sync(0xffffffffu, ((uint32_t)__float2int_rn(x) & 1u) != 0u);
    if (lane == 0) {
        uint32_t w = __byte_perm(__brev(bits), 0, 0x0123);
        if (XOR) w ^= __byte_perm(key_rest[(size_t)i * words + word], 0, 0x0123);
        out[(size_t)i * words + word] = w;
    }
}

void destroy_bank(Bank* b) {
    if (!b) return;
    if (b->fwd) cufftDestroy(b->fwd);
    if (b->inv) cufftDestroy(b->inv);
    cudaFree(b->seed);
    cudaFree(b->ks);
    cudaFree(b->kr);
    cudaFree(b->out);
    cudaFree(b->di1);
    cudaFree(b->di2);
    cudaFree(b->do1);
    cudaFree(b->do2);
    cudaFree(b->cnt);
    cudaFree(b->corr);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

}  // namespace

// s: power of two in [2^10, 2^27]; v: multiple of 32 below s; B sub-blocks (B * s <= 2^28).
CP_API int cb_create(uint32_t s, uint32_t v, uint32_t B, void** out) {
    if (!out || s < 1024u || s > (1u << 27) || (s & (s - 1u)) || (v & 31u) || v == 0 || v >= s || B == 0 ||
        (uint64_t)B * s > (1ull << 28))
        return -1;
    Bank* b = new (std::nothrow) Bank;
    if (!b) return -2;
    b->s = s, b->v = v, b->B = B;
    while ((1u << b->log_s) < s) ++b->log_s;
    const size_t bits = (size_t)B * s, dist = s / 2u + 1u;
    auto fail = [&](int rc) {
        destroy_bank(b);
        return rc;
    };
    if (cudaMalloc(&b->seed, bits / 8) != cudaSuccess || cudaMalloc(&b->ks, bits / 8) != cudaSuccess ||
        cudaMalloc(&b->kr, (size_t)B * v / 8) != cudaSuccess || cudaMalloc(&b->out, (size_t)B * v / 8) != cudaSuccess ||
        cudaMalloc(&b->di1, bits * sizeof(float)) != cudaSuccess || cudaMalloc(&b->di2, bits * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&b->do1, B * dist * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&b->do2, B * dist * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&b->cnt, 2 * (size_t)B * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&b->corr, (size_t)B * sizeof(float)) != cudaSuccess)
        return fail(-2);
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess)
        return fail(-2);
    if (cudaMemset(b->seed, 0, bits / 8) != cudaSuccess || cudaMemset(b->ks, 0, bits / 8) != cudaSuccess ||
        cudaMemset(b->kr, 0, (size_t)B * v / 8) != cudaSuccess)
        return fail(-2);
    if (cufftPlan1d(&b->fwd, (int)s, CUFFT_R2C, (int)B) != CUFFT_SUCCESS) return fail(-3);
    if (cufftPlan1d(&b->inv, (int)s, CUFFT_C2R, (int)B) != CUFFT_SUCCESS) return fail(-3);
    if (cufftSetStream(b->fwd, b->st) != CUFFT_SUCCESS || cufftSetStream(b->inv, b->st) != CUFFT_SUCCESS) return fail(-3);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(-2);
    *out = b;
    return 0;
}

CP_API void cb_destroy(void* h) { destroy_bank(static_cast<Bank*>(h)); }

// Host -> device copies of the bank's inputs: seed and key_start B * s/32 words (sub-block i at i * s/32,
// key_start zero past bit h of each sub-block), key_rest B * v/32 words (null: keep).  Not timed.
CP_API int cb_load(void* h, const uint32_t* seed, const uint32_t* key_start, const uint32_t* key_rest) {
    Bank* b = static_cast<Bank*>(h);
    const size_t bytes = (size_t)b->B * b->s / 8;
    if (seed) {
        CP_TRY(cudaMemcpy(b->seed, seed, bytes, cudaMemcpyHostToDevice));
        b->seed_ready = false;
    }
    if (key_start) CP_TRY(cudaMemcpy(b->ks, key_start, bytes, cudaMemcpyHostToDevice));
    if (key_rest) CP_TRY(cudaMemcpy(b->kr, key_rest, (size_t)b->B * b->v / 8, cudaMemcpyHostToDevice));
    return 0;
}

// Queues one bank on the bank's stream between two events and waits for it; *ms = device time.
// recalc_seed = 0 reuses the seed spectra (the first call always computes them).
CP_API int cb_run(void* h, int recalc_seed, int do_xor, float* ms) {
    Bank* b = static_cast<Bank*>(h);
    const uint32_t s = b->s, B = b->B, dist = s / 2u + 1u;
    const size_t bits = (size_t)B * s;
    const bool seed = recalc_seed || !b->seed_ready;
    cudaStream_t st = b->st;
    CP_TRY(cudaEventRecord(b->ev[0], st));
    if (seed) {
        CP_TRY(cudaMemsetAsync(b->cnt, 0, (size_t)B * sizeof(uint32_t), st));
        k_unpack_bank<<<(unsigned)(bits / 1024u), 1024, 0, st>>>(b->seed, b->di2, b->cnt, b->log_s);
        CP_FFT(cufftExecR2C(b->fwd, b->di2, reinterpret_cast<cufftComplex*>(b->do2)));
    }
    CP_TRY(cudaMemsetAsync(b->cnt + B, 0, (size_t)B * sizeof(uint32_t), st));
    k_unpack_bank<<<(unsigned)(bits / 1024u), 1024, 0, st>>>(b->ks, b->di1, b->cnt + B, b->log_s);
    k_correction_bank<<<(B + 255u) / 256u, 256, 0, st>>>(b->cnt, b->corr, B, s);
    CP_FFT(cufftExecR2C(b->fwd, b->di1, reinterpret_cast<cufftComplex*>(b->do1)));
    k_zero_dc_bank<<<(B + 255u) / 256u, 256, 0, st>>>(b->do1, b->do2, B, dist);
    const size_t count = (size_t)B * dist;
    k_product_bank<<<(unsigned)((count + 255u) / 256u), 256, 0, st>>>(b->do1, b->do2, count);
    CP_FFT(cufftExecC2R(b->inv, reinterpret_cast<cufftComplex*>(b->do1), b->di2));
    const float norm = (float)s / (2048.0f * kR) / (2048.0f * kR);
    const dim3 grid((b->v / 32u + 7u) / 8u, B);
    if (do_xor) k_pack_bank<true><<<grid, 256, 0, st>>>(b->di2, b->out, b->kr, b->corr, s, b->v, norm);
    else k_pack_bank<false><<<grid, 256, 0, st>>>(b->di2, b->out, nullptr, b->corr, s, b->v, norm);
    CP_TRY(cudaGetLastError());
    CP_TRY(cudaEventRecord(b->ev[1], st));
    CP_TRY(cudaEventSynchronize(b->ev[1]));
    if (seed) b->seed_ready = !recalc_seed;  // a static seed's spectra are kept; C2R overwrote its floats only
    if (ms) CP_TRY(cudaEventElapsedTime(ms, b->ev[0], b->ev[1]));
    return 0;
}

// Device -> host copy of the B * v/32 output words (sub-block i at i * v/32).
CP_API int cb_output(void* h, uint32_t* out) {
    Bank* b = static_cast<Bank*>(h);
    CP_TRY(cudaMemcpy(out, b->out, (size_t)b->B * b->v / 8, cudaMemcpyDeviceToHost));
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
