// pa_group.cu -- grouped launches: G blocks of one geometry as one launch per pass.
//
// Many small blocks launched one by one are bound by the launches themselves: a 2^18-bit block's five
// kernels each run for a few microseconds, and a CUDA graph of 512 such blocks spends about a
// microsecond per kernel node.  A group runs its blocks' bit rows, pass A, pass B, pass C and finish as
// five launches whose second grid dimension (third for the two-dimensional transposes) is the block:
// each block's CTAs walk its own rows and tiles exactly as a single block's do.  The working set is
// contiguous (block b's bit rows / planes, Y, Z and own seed spectrum at base + b * stride, and the
// tensor maps span all blocks); the caller's buffers (key_start, key_rest, seed words, out), the
// spectrum of a cached seed and the per-block statistics come from a table of GroupEntry in device
// memory.
#include "pa_pass_bodies.cuh"

namespace pa {

// A group's pass B: the CTAs walk the tiles of all the group's blocks one after another (a seed pass
// writes the group's own spectra, a key pass reads each entry's), so that a CTA's next tile -- often
// another block's, short columns have few tiles -- is still copied under the current one.
template <int LOGL, bool SEED>
__global__ void __launch_bounds__(256, 2)
    k_pass_b_group(const __grid_constant__ CUtensorMap mapY, const float2* __restrict__ Y, float2* __restrict__ Z,
                   BlockGeom g, float2* __restrict__ spec, int* err, int early, Group gp) {
    pass_b_tiles<LOGL, SEED, 256, true>(&mapY, Y, Z, g, spec, err, early, blockIdx.x, gridDim.x, gp.e, gp.count);
}

template <int LOGL>
int launch_pass_b_group(bool seed, dim3 grid, size_t smem, const CUtensorMap& mapY, float2* Y, float2* Z,
                        float2* spec, const BlockGeom& g, int* err, int early, const Group& gp, cudaStream_t s) {
    if (!gp.e) return (int)cudaErrorInvalidValue;
    if (seed) {
        cudaFuncSetAttribute(k_pass_b_group<LOGL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pass_b_group<LOGL, true><<<grid, 256, smem, s>>>(mapY, Y, Z, g, spec, err, early, gp);
    } else {
        cudaFuncSetAttribute(k_pass_b_group<LOGL, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pass_b_group<LOGL, false><<<grid, 256, smem, s>>>(mapY, Y, Z, g, spec, err, early, gp);
    }
    return (int)cudaGetLastError();
}

#define PA_GROUP_B(LG)                                                                                            \
    template int launch_pass_b_group<LG>(bool, dim3, size_t, const CUtensorMap&, float2*, float2*, float2*,      \
                                         const BlockGeom&, int*, int, const Group&, cudaStream_t);
PA_GROUP_B(5)
PA_GROUP_B(6)
PA_GROUP_B(7)
PA_GROUP_B(8)
PA_GROUP_B(9)
PA_GROUP_B(10)
PA_GROUP_B(11)
PA_GROUP_B(12)
#undef PA_GROUP_B

__global__ void k_group_prep(const GroupEntry* __restrict__ e, uint32_t count) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    e[b].cnt[0] = 0ull;
    e[b].cnt[1] = e[b].seed_cnt ? *e[b].seed_cnt : 0ull;
    *e[b].resid = 0u;
}

int launch_group_prep(const Group& gp, cudaStream_t s) {
    if (!gp.e || gp.count == 0) return (int)cudaErrorInvalidValue;
    k_group_prep<<<(gp.count + 127u) / 128u, 128, 0, s>>>(gp.e, gp.count);
    return (int)cudaGetLastError();
}

int launch_group_seed(const BlockGeom& g, const Group& gp, float2* spec, const Scratch& sc, int num_sms,
                      cudaStream_t s) {
    if (!gp.e) return (int)cudaErrorInvalidValue;
    if (g.log_n1 == 0) return launch_group_mono_seed(g, gp, spec, s);
    int rc = launch_bit_rows(g, nullptr, true, sc.planes, s, gp);
    if (!rc) rc = launch_pass_a(g, sc.planes, true, sc.work, nullptr, num_sms, s, gp);
    if (!rc) rc = launch_pass_b(g, true, *sc.maps, sc.work, sc.work2, spec, sc.err, num_sms, s, gp);
    return rc;
}

int launch_group_key(const BlockGeom& g, const Group& gp, uint32_t flags, const Scratch& sc, int num_sms,
                     cudaStream_t s) {
    if (!gp.e) return (int)cudaErrorInvalidValue;
    if (g.log_n1 == 0) return launch_group_mono_key(g, gp, flags, s);
    int rc = launch_bit_rows(g, nullptr, false, sc.planes, s, gp);
    if (!rc) rc = launch_pass_a(g, sc.planes, false, sc.work, nullptr, num_sms, s, gp);
    if (!rc) rc = launch_pass_b(g, false, *sc.maps, sc.work, sc.work2, nullptr, sc.err, num_sms, s, gp);
    if (!rc) rc = launch_pass_c(g, *sc.maps, sc.work2, nullptr, sc.planes, nullptr, sc.err, num_sms, s, gp);
    if (!rc) rc = launch_finish(g, sc.planes, nullptr, flags, nullptr, s, gp);
    return rc;
}

}  // namespace pa
