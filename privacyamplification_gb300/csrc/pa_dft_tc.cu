// pa_dft_tc.cu -- a radix-16 DFT stage as a tcgen05 tensor-core product, measured against the FP32
// butterflies the three passes use.
//
// Every pass of the convolution is a chain of radix-16 stages on 16 complex values per butterfly.
// A stage is a matrix product: with the 16 inputs of a butterfly as 32 reals (re, im interleaved),
// the 16 outputs are y = B x for the 32 x 32 real matrix B of the 16-point DFT.  For a tile of 128
// butterflies (one per thread of a 128-thread CTA) that is D[128 x 32] = A[128 x 32] B^T, one
// tcgen05.mma chain with M = 128, N = 32, K = 32: A (the data) and B (the DFT matrix) in shared memory,
// D in tensor memory, read back to registers with tcgen05.ld (thread t owns row t, its butterfly).
//
// The tensor cores take FP32 operands only as TF32 (10 explicit mantissa bits), so the product keeps
// FP32-level accuracy only by splitting both operands, x = x_hi + x_lo and B = B_hi + B_lo, and
// accumulating three products A_hi B_hi + A_hi B_lo + A_lo B_hi in FP32 (about 2^-22 relative).
// Methods, all on the same data and the same thread-per-butterfly mapping:
//   0  FP32 butterflies in registers (pa::dft<16, -1>, the passes' own stage)
//   1  tcgen05 kind::tf32, three split products (FP32-level accuracy)
//   2  tcgen05 kind::tf32, one product A_hi B_hi (TF32 accuracy, the tensor path's ceiling)
// Each thread loads its butterfly once, applies `reps` forward stages (after every fourth stage it
// multiplies by 1/256, since F^4 = 256 I, so that values stay in range and reps % 4 == 0 returns the
// input), and stores the result.
//
// Tensor-memory and barrier discipline: warp 0 allocates 32 columns and frees them before the CTA
// exits; the MMA completion is an mbarrier arrival (tcgen05.commit), and every wait on it is bounded:
// a wait that gives up records kErrTmaTimeout, waits once more (bounded) for the MMAs in flight, frees
// the tensor memory and ends the CTA's work.  Shared-memory descriptors only address the CTA's own
// 40 KB of operands, whichever way the hardware reads their two stride fields.
#include "../../include/pa_gb300.h"
#include "pa_device.cuh"
#include "pa_tma.cuh"

#include <cuda_runtime.h>

#include <algorithm>

namespace {

constexpr int kRows = 128;                      // butterflies per tile (MMA M)
constexpr int kVals = 32;                       // reals per butterfly (MMA K and N)
constexpr uint32_t kTileBytes = kRows * kVals * 4;  // one A operand: 16 KB
constexpr uint32_t kMatBytes = kVals * kVals * 4;   // one B operand: 4 KB
constexpr uint32_t kTmemCols = 32;
constexpr uint32_t kLbo = 128;                  // bytes between core matrices adjacent in K
constexpr uint32_t kSbo = 1024;                 // bytes between core matrices adjacent in M / N

// Byte offset of element (row, k) of a K-major operand without swizzle: core matrices of 8 rows x 16
// bytes (4 TF32), K-adjacent ones kLbo apart, row-group-adjacent ones kSbo apart.
__device__ __forceinline__ uint32_t op_offset(int row, int k) {
    return (uint32_t)(row >> 3) * kSbo + (uint32_t)(k >> 2) * kLbo + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

// Shared-memory matrix descriptor: start address, leading and stride byte offsets (all >> 4), the fixed
// value 1 at bits 46-48, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((kLbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((kSbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both
// K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kVals >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(pa::smem_addr(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's tensor-memory lane, then the wait for them.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[kVals]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]),
          "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]), "=f"(v[16]),
          "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]), "=f"(v[24]),
          "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31])
        : "r"(taddr)
        : "memory");
}

// x rounded to TF32 (nearest, ties away), as an FP32 bit pattern whose low 13 mantissa bits are zero.
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void load_row(const float* in, size_t row, float (&v)[kVals]) {
    const float4* p = reinterpret_cast<const float4*>(in + row * kVals);
#pragma unroll
    for (int i = 0; i < kVals / 4; ++i) {
        float4 t = __ldcs(p + i);
        v[4 * i] = t.x, v[4 * i + 1] = t.y, v[4 * i + 2] = t.z, v[4 * i + 3] = t.w;
    }
}

__device__ __forceinline__ void store_row(float* out, size_t row, const float (&v)[kVals]) {
    float4* p = reinterpret_cast<float4*>(out + row * kVals);
#pragma unroll
    for (int i = 0; i < kVals / 4; ++i) __stcs(p + i, make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]));
}

__device__ __forceinline__ void scale_after(int s, float (&v)[kVals]) {
    if ((s & 3) == 3) {
#pragma unroll
        for (int i = 0; i < kVals; ++i) v[i] *= 0.00390625f;  // 1/256, exact
    }
}

__global__ void __launch_bounds__(kRows) k_dft16_fp32(const float* in, float* out, uint32_t tiles, uint32_t reps) {
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const size_t row = (size_t)tile * kRows + threadIdx.x;
        const float4* p = reinterpret_cast<const float4*>(in + row * kVals);
        float2 z[16];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float4 q = __ldcs(p + i);
            z[2 * i] = make_float2(q.x, q.y), z[2 * i + 1] = make_float2(q.z, q.w);
        }
        for (uint32_t s = 0; s < reps; ++s) {
            pa::dft<16, -1>(z);
            if ((s & 3) == 3) {
#pragma unroll
                for (int i = 0; i < 16; ++i) z[i] = pa::cscale(z[i], 0.00390625f);  // 1/256, exact
            }
        }
        float4* o = reinterpret_cast<float4*>(out + row * kVals);
#pragma unroll
        for (int i = 0; i < 8; ++i) __stcs(o + i, make_float4(z[2 * i].x, z[2 * i].y, z[2 * i + 1].x, z[2 * i + 1].y));
    }
}

// B[n][k] of the real 32 x 32 DFT matrix: output n = 2p (+1 for the imaginary part), input k = 2j (+1).
__device__ __forceinline__ double dft_entry(int n, int k) {
    const int p = n >> 1, j = k >> 1;
    double s, c;
    sincospi(-2.0 * (double)((p * j) & 15) / 16.0, &s, &c);  // F_pj = c + i s
    if ((n & 1) == 0) return (k & 1) == 0 ? c : -s;             // Re y = c Re x - s Im x
    return (k & 1) == 0 ? s : c;                                  // Im y = s Re x + c Im x
}

template <int SPLIT>
__global__ void __launch_bounds__(kRows) k_dft16_tc(const float* in, float* out, uint32_t tiles, uint32_t reps, int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* a_hi = smem;
    unsigned char* a_lo = smem + kTileBytes;
    unsigned char* b_hi = smem + 2 * kTileBytes;
    unsigned char* b_lo = b_hi + kMatBytes;
    uint64_t* bar = reinterpret_cast<uint64_t*>(b_lo + kMatBytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
    const int t = threadIdx.x, warp = t >> 5;

    // the DFT matrix, split into TF32 high and low parts
    for (int i = t; i < kVals * kVals; i += kRows) {
        const int n = i / kVals, k = i % kVals;
        const double e = dft_entry(n, k);
        const float hi = tf32_round((float)e);
        const float lo = tf32_round((float)(e - (double)hi));
        *reinterpret_cast<float*>(b_hi + op_offset(n, k)) = hi;
        *reinterpret_cast<float*>(b_lo + op_offset(n, k)) = lo;
    }
    if (t == 0) pa::mbar_init(bar, 1);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(pa::smem_addr(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    pa::fence_proxy_async();  // the B operands, written by these threads, are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t my_lane = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t sa_hi = pa::smem_addr(a_hi), sa_lo = pa::smem_addr(a_lo);
    const uint32_t sb_hi = pa::smem_addr(b_hi), sb_lo = pa::smem_addr(b_lo);

    uint32_t phase = 0;
    bool failed = false;
    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const size_t row = (size_t)tile * kRows + t;
        float v[kVals];
        load_row(in, row, v);
        for (uint32_t s = 0; s < reps; ++s) {
            // split this butterfly into TF32 parts and write row t of both A operands
#pragma unroll
            for (int c = 0; c < kVals / 4; ++c) {
                float4 h, l;
                h.x = tf32_round(v[4 * c]), l.x = v[4 * c] - h.x;
                h.y = tf32_round(v[4 * c + 1]), l.y = v[4 * c + 1] - h.y;
                h.z = tf32_round(v[4 * c + 2]), l.z = v[4 * c + 2] - h.z;
                h.w = tf32_round(v[4 * c + 3]), l.w = v[4 * c + 3] - h.w;
                *reinterpret_cast<float4*>(a_hi + op_offset(t, 4 * c)) = h;
                if (SPLIT) *reinterpret_cast<float4*>(a_lo + op_offset(t, 4 * c)) = l;
            }
            pa::fence_proxy_async();
            tc_fence_before();
            __syncthreads();
            if (t == 0) {
                tc_fence_after();
                // K = 32 as four steps of 8 TF32 (32 bytes = two core matrices along K)
#pragma unroll
                for (int kk = 0; kk < kVals / 8; ++kk) {
                    const uint32_t off = (uint32_t)kk * 2u * kLbo;
                    tc_mma(tmem, smem_desc(sa_hi + off), smem_desc(sb_hi + off), kk > 0);
                    if (SPLIT) {
                        tc_mma(tmem, smem_desc(sa_hi + off), smem_desc(sb_lo + off), 1);
                        tc_mma(tmem, smem_desc(sa_lo + off), smem_desc(sb_hi + off), 1);
                    }
                }
                tc_commit(bar);
            }
            const bool ok = pa::mbar_wait(bar, phase);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                if (t == 0) atomicExch(err, pa::kErrTmaTimeout);
                pa::mbar_wait(bar, phase ^ 1u);  // the MMAs in flight, once more, bounded
                failed = true;
                break;
            }
            tc_fence_after();
            tc_ld32(my_lane, v);
            scale_after((int)s, v);
        }
        if (!failed) store_row(out, row, v);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

constexpr size_t kTcSmem = 2 * kTileBytes + 2 * kMatBytes + 16;

}  // namespace

extern "C" int pa_dft16_stages(const float* d_in, float* d_out, uint32_t butterflies, uint32_t reps, int32_t method,
                               int32_t ctas_per_sm, int32_t* d_err, void* stream) {
    if (!d_in || !d_out || !d_err || butterflies == 0 || butterflies % kRows || reps == 0 || reps > (1u << 16))
        return PA_ERR_INVALID_ARG;
    if ((reinterpret_cast<uintptr_t>(d_in) | reinterpret_cast<uintptr_t>(d_out)) & 15u) return PA_ERR_INVALID_ARG;
    if (method < 0 || method > 2 || ctas_per_sm < 1 || ctas_per_sm > (method == 0 ? 16 : 4)) return PA_ERR_INVALID_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return PA_ERR_CUDA;
    const uint32_t tiles = butterflies / kRows;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(tiles, (uint64_t)sms * (uint64_t)ctas_per_sm);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (method == 0) {
        k_dft16_fp32<<<grid, kRows, 0, s>>>(d_in, d_out, tiles, reps);
    } else {
        // at most 5 CTAs of 40 KB fit an SM, 32 tensor-memory columns each: an allocation never waits
        auto k = method == 1 ? k_dft16_tc<1> : k_dft16_tc<0>;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem) != cudaSuccess)
            return PA_ERR_CUDA;
        k<<<grid, kRows, kTcSmem, s>>>(d_in, d_out, tiles, reps, d_err);
    }
    return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}
