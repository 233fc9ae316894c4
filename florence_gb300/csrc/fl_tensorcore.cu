// fl_tensorcore.cu -- self-test of the tcgen05 path (fl_tc.cuh): one CTA multiplies a 128 x 48
// BF16 matrix by the transpose of a 32 x 48 one on the fifth-generation tensor cores (operands in
// shared memory in the K-major core-matrix layout, FP32 accumulator in tensor memory) and
// returns the product, so a test can check the descriptors, the instruction descriptor and the
// tensor-memory read-back against an exact host product.
#include <cuda_bf16.h>

#include "fl_common.cuh"
#include "fl_tc.cuh"

namespace fl {

constexpr int TC_M = 128, TC_N = 32, TC_K = 48;
constexpr long long TC_WAIT_LIMIT = 1ll << 22;

__global__ void __launch_bounds__(128) tc_selftest_kernel(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D,
                                                          int *status) {
    __shared__ __align__(1024) __nv_bfloat16 As[TC_M * TC_K];
    __shared__ __align__(1024) __nv_bfloat16 Bs[TC_N * TC_K];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t taddr_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // operands: row-major in global -> K-major core-matrix layout in shared memory
    for (int i = tid; i < TC_M * TC_K; i += 128) {
        const int r = i / TC_K, k = i % TC_K;
        As[tc::kmajor_offset(r, k, TC_K) / 2] = A[i];
    }
    for (int i = tid; i < TC_N * TC_K; i += 128) {
        const int r = i / TC_K, k = i % TC_K;
        Bs[tc::kmajor_offset(r, k, TC_K) / 2] = B[i];
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&taddr_s, 32);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = taddr_s;

    if (tid == 0) {
        constexpr uint32_t idesc = tc::idesc_bf16_f32(TC_M, TC_N);
        const uint32_t sbo = (TC_K / 8) * 128;
#pragma unroll
        for (int ks = 0; ks < TC_K / 16; ++ks) {
            const uint64_t da = tc::smem_desc(As + ks * 16 * 8, 128, sbo);  // core matrices (i, 2ks), (i, 2ks+1)
            const uint64_t db = tc::smem_desc(Bs + ks * 16 * 8, 128, sbo);
            tc::mma_bf16(taddr, da, db, idesc, ks > 0);
        }
        tc::mma_commit(&mbar);
    }
    const bool ok = tc::mbar_wait(&mbar, 0, TC_WAIT_LIMIT);
    tc::fence_after_sync();
    if (ok) {
        float v[32];
        tc::tmem_ld32(taddr + ((uint32_t)(32 * warp) << 16), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) D[(size_t)(32 * warp + lane) * TC_N + j] = v[j];
    } else {
        if (lane == 0) atomicOr(status, 1);
        // the MMAs may still be writing the accumulator: wait once more (bounded) before the
        // tensor memory is released
        tc::mbar_wait(&mbar, 0, TC_WAIT_LIMIT);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 32);
}

}  // namespace fl

extern "C" int fl_TensorCoreSelfTest(const void *A_bf16, const void *B_bf16, float *D, int *status,
                                     fl_stream_t stream) {
    if (!A_bf16 || !B_bf16 || !D || !status) return FL_ERR_ARG;
    fl::tc_selftest_kernel<<<1, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A_bf16,
                                                                (const __nv_bfloat16 *)B_bf16, D, status);
    return fl::launch_status();
}
