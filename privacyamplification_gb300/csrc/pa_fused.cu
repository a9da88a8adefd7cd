// pa_fused.cu -- a block whose seed serves that block only: one column pass for the seed and the key.
//
// A fresh seed's spectrum is otherwise written to HBM by a column pass of its own and read back by the
// key's (N complex values each way: 1 GiB of traffic at n = 2^27).  Here both row passes run first, the
// seed's into the buffer its spectrum would take, and one column pass takes every tile twice: the seed's
// tile, transformed and split into its spectrum tile, which is parked in the CTA's own 64 KiB of a small
// buffer (2 CTAs per SM: about 20 MB, rewritten by the same CTA a tile later, so it stays in L2), then
// the key's tile against it (pass_b_tiles, FUSED).
#include "pa_pass_bodies.cuh"

namespace pa {

template <int LOGL>
__global__ void __launch_bounds__(256, 2)
    k_pass_b_fused(const __grid_constant__ CUtensorMap mapYs, const __grid_constant__ CUtensorMap mapY,
                   float2* __restrict__ Z, BlockGeom g, float2* __restrict__ park, int* err, int early) {
    pass_b_tiles<LOGL, false, 256, false, true>(&mapY, nullptr, Z, g, park, err, early, blockIdx.x, gridDim.x,
                                                nullptr, 1u, &mapYs);
}

template <int LOGL>
int launch_pass_b_fused_k(dim3 grid, size_t smem_base, size_t box, int max_early, const CUtensorMap& mapYs,
                          const CUtensorMap& mapY, float2* Z, const BlockGeom& g, float2* park, int* err,
                          cudaStream_t s) {
    auto kernel = k_pass_b_fused<LOGL>;
    // as many of the next tile's boxes beside the tile as keep two CTAs per SM (the sizes depend on LOGL only)
    static const int early = [&] {
        int e = max_early;
        for (; e > 0; --e) {
            int per_sm = 0;
            const size_t bytes = smem_base + (size_t)e * box;
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
                    cudaSuccess &&
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, bytes) == cudaSuccess &&
                per_sm >= 2)
                break;
        }
        cudaGetLastError();  // a refused attribute above is not an error of this launch
        return e;
    }();
    const size_t bytes = smem_base + (size_t)early * box;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    kernel<<<grid, 256, bytes, s>>>(mapYs, mapY, Z, g, park, err, early);
    return (int)cudaGetLastError();
}

#define PA_FUSED_B(LG)                                                                                           \
    template int launch_pass_b_fused_k<LG>(dim3, size_t, size_t, int, const CUtensorMap&, const CUtensorMap&,   \
                                           float2*, const BlockGeom&, float2*, int*, cudaStream_t);
PA_FUSED_B(10)
PA_FUSED_B(11)
PA_FUSED_B(12)
#undef PA_FUSED_B

}  // namespace pa
