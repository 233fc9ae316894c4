// fl_measure.cu -- FP64 and FP32 FMA roof measurement: many independent FMA chains per thread
// over the whole GPU, timed with CUDA events. Copy and GEMM peak figures do not cover the FP64 or
// FP32 SIMT pipes that bound the assembly kernels, so the benchmark measures these roofs in the
// same run.
#include "fl_common.cuh"

namespace fl {

constexpr int PK_CHAINS = 16, PK_ITERS = 2048, PK_NT = 256;

template <class T>
__global__ void __launch_bounds__(PK_NT) fma_roof_kernel(T *out, T seed, int iters) {
    T a[PK_CHAINS];
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) a[c] = seed + (T)(threadIdx.x * 1e-9 + c * 1e-7);
    const T m = (T)0.999999, k = (T)1e-9;
#pragma unroll 4
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < PK_CHAINS; ++c) a[c] = fma(a[c], m, k);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) s += a[c];
    if (s == (T)12345.678) out[blockIdx.x] = s;  // keeps the chains alive without a store per thread
}

template <class T>
static int measure_peak(double *gflops, int iters, cudaStream_t s) {
    if (!gflops) return FL_ERR_ARG;
    int dev = 0, sms = 0;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    FL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = sms * 8;
    T *out = nullptr;
    FL_CUDA_TRY(cudaMallocAsync((void **)&out, sizeof(T) * grid, s));
    cudaEvent_t e0, e1;
    FL_CUDA_TRY(cudaEventCreate(&e0));
    FL_CUDA_TRY(cudaEventCreate(&e1));
    fma_roof_kernel<T><<<grid, PK_NT, 0, s>>>(out, (T)1, iters);  // warm-up
    FL_CUDA_TRY(cudaEventRecord(e0, s));
    const int reps = 5;
    for (int r = 0; r < reps; ++r) fma_roof_kernel<T><<<grid, PK_NT, 0, s>>>(out, (T)(1 + r), iters);
    FL_CUDA_TRY(cudaEventRecord(e1, s));
    FL_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FL_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    FL_CUDA_TRY(cudaFreeAsync(out, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * PK_CHAINS * (double)iters * (double)PK_NT * grid * reps;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return FL_OK;
}

}  // namespace fl

extern "C" int fl_measure_fp64_peak(double *gflops, fl_stream_t stream) {
    return fl::measure_peak<double>(gflops, fl::PK_ITERS, (cudaStream_t)stream);
}

extern "C" int fl_measure_fp32_peak(double *gflops, fl_stream_t stream) {
    return fl::measure_peak<float>(gflops, 32 * fl::PK_ITERS, (cudaStream_t)stream);
}
