// pa_selftest.cu -- checks that a bounded device wait which is never satisfied ends with an error
// status on the host and leaves the CUDA context usable (the failure path every TMA wait of the
// three-pass kernels relies on).  Nothing here faults or hangs: the wait gives up after `rounds`.
#include "../../include/pa_gb300.h"
#include "pa_tma.cuh"

#include <cuda_runtime.h>

namespace {

// One CTA: an mbarrier that expects one arrival which never comes; every thread waits with the limit,
// and a thread that gives up records kErrTmaTimeout.
__global__ void k_wait_expires(uint32_t rounds, int* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) pa::mbar_init(&bar, 1);
    __syncthreads();
    if (!pa::mbar_wait(&bar, 0u, rounds)) atomicExch(err, pa::kErrTmaTimeout);
}

}  // namespace

extern "C" int pa_selftest_wait_timeout(int32_t device_id, uint32_t rounds, int32_t* status) {
    if (!status || rounds == 0 || rounds > (1u << 20)) return PA_ERR_INVALID_ARG;
    if (cudaSetDevice(device_id) != cudaSuccess) return PA_ERR_CUDA;
    int* d_err = nullptr;
    if (cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) return PA_ERR_CUDA;
    int rc = PA_OK;
    int h = 0;
    if (cudaMemset(d_err, 0, sizeof(int)) != cudaSuccess) rc = PA_ERR_CUDA;
    if (!rc) {
        k_wait_expires<<<1, 128>>>(rounds, d_err);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = PA_ERR_CUDA;
    }
    if (!rc && cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = PA_ERR_CUDA;
    cudaFree(d_err);
    *status = h;
    return rc;
}
