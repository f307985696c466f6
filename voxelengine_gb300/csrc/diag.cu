// diag.cu — measurement helper: the L2 read bandwidth this GPU delivers to a
// streaming kernel, the denominator of the L2 side of the occlusion kernel's
// roofline (its grid stays resident in L2 while a frame is traced).
#include "vxl_device.cuh"

namespace vxl {

// every thread reads 16-byte vectors in a grid-stride loop; one xor per block
// is stored so that the loads are not removed
__global__ void __launch_bounds__(256) k_l2_read(const uint4* __restrict__ p, size_t n, uint32_t* out) {
    uint32_t acc = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint4 v = __ldcg(p + i);  // cached in L2 only: the L2 is what is measured
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    acc = __reduce_xor_sync(0xffffffffu, acc);
    if ((threadIdx.x & 31) == 0) atomicXor(out + blockIdx.x, acc);
}

}  // namespace vxl

using namespace vxl;

extern "C" vxl_status vxl_diag_l2_read_gbs(vxl_ctx* ctx, size_t bytes, int reps, double* best_gbs, double* best_ms) {
    if (!ctx || !best_gbs || reps < 1 || bytes < (1u << 20) || (bytes & 15))
        return fail(VXL_ERR_INVALID_ARG, "diag_l2_read_gbs: bad argument");
    VXL_TRY_CUDA(cudaSetDevice(ctx->device));
    const size_t n = bytes / 16;
    const unsigned blocks = (unsigned)ctx->sm_count * 8;
    uint4* buf = nullptr;
    uint32_t* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&buf, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&out, blocks * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(buf, 0x5a, bytes);
    if (e == cudaSuccess) e = cudaMemset(out, 0, blocks * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    double best = 1e30;
    // the first launches bring the buffer into L2; the best of the rest is reported
    for (int r = 0; r < reps + 3 && e == cudaSuccess; r++) {
        e = cudaEventRecord(e0, 0);
        if (e == cudaSuccess) {
            k_l2_read<<<blocks, 256>>>(buf, n, out);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && r >= 3 && ms < best) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (buf) cudaFree(buf);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return cuda_fail(e, "diag_l2_read_gbs");
    ctx->launches += (uint64_t)reps + 3;
    *best_gbs = (double)bytes / (best * 1e-3) / 1e9;
    if (best_ms) *best_ms = best;
    return VXL_OK;
}
