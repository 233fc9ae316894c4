// fl_measure.cu -- FP64 roof measurement: many independent FMA chains per thread over the whole
// GPU, timed with CUDA events. MEASURED_PEAKS-style copy/GEMM figures do not cover FP64, and the
// assembly kernels are bound by the FP64 pipe, so the benchmark measures this roof in the same run.
#include "fl_common.cuh"

namespace fl {

constexpr int PK_CHAINS = 16, PK_ITERS = 2048, PK_NT = 256;

__global__ void __launch_bounds__(PK_NT) fp64_fma_kernel(double *out, double seed) {
    double a[PK_CHAINS];
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) a[c] = seed + threadIdx.x * 1e-9 + c * 1e-7;
    const double m = 0.999999, k = 1e-9;
#pragma unroll 4
    for (int it = 0; it < PK_ITERS; ++it) {
#pragma unroll
        for (int c = 0; c < PK_CHAINS; ++c) a[c] = fma(a[c], m, k);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) s += a[c];
    if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains alive without a store per thread
}

}  // namespace fl

extern "C" int fl_measure_fp64_peak(double *gflops, fl_stream_t stream) {
    if (!gflops) return FL_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    FL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = sms * 8;
    double *out = nullptr;
    FL_CUDA_TRY(cudaMallocAsync(&out, sizeof(double) * grid, s));
    cudaEvent_t e0, e1;
    FL_CUDA_TRY(cudaEventCreate(&e0));
    FL_CUDA_TRY(cudaEventCreate(&e1));
    fl::fp64_fma_kernel<<<grid, fl::PK_NT, 0, s>>>(out, 1.0);  // warm-up
    FL_CUDA_TRY(cudaEventRecord(e0, s));
    const int reps = 5;
    for (int r = 0; r < reps; ++r) fl::fp64_fma_kernel<<<grid, fl::PK_NT, 0, s>>>(out, 1.0 + r);
    FL_CUDA_TRY(cudaEventRecord(e1, s));
    FL_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FL_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    FL_CUDA_TRY(cudaFreeAsync(out, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * fl::PK_CHAINS * fl::PK_ITERS * (double)fl::PK_NT * grid * reps;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return FL_OK;
}
