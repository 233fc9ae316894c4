// fl_mlp.cu -- training and inference kernels of the warm-start network: an MLP 3 -> 256 -> 256 -> 64
// with GELU activations, BF16 arithmetic (every GEMM operand rounded to BF16, products exact and
// accumulated in FP32) and FP32 master weights updated by Adam. It maps (load, material)
// parameters to the coefficients of the next increment's displacement in a POD basis; Newton
// starts from the prediction when its residual beats the previous-increment guess.
//
// Parameter vector (FP32, row-major weights, x W convention):
//   W1 [3][256], b1 [256], W2 [256][256], b2 [256], W3 [256][64], b3 [64]   (83 264 floats)
// Forward:  z1 = x W1 + b1, h1 = gelu(z1), z2 = h1 W2 + b2, h2 = gelu(z2), y = h2 W3 + b3
// Loss:     L = sum (y - t)^2 / (2 B 64)
// Backward: dy = (y - t) / (B 64); dW3 = h2^T dy; db3 = sum dy; dz2 = (dy W3^T) .* gelu'(z2);
//           dW2 = h1^T dz2; db2 = sum dz2; dz1 = (dz2 W2^T) .* gelu'(z1); dW1 = x^T dz1; db1 = sum dz1
// gelu(z) = z/2 (1 + erf(z / sqrt 2)).
#include <cuda_bf16.h>

#include "fl_common.cuh"

namespace fl {

constexpr int MLP_IN = 3, MLP_H = 256, MLP_OUT = 64;
constexpr int64_t OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_IN * MLP_H, OFF_W2 = OFF_B1 + MLP_H, OFF_B2 = OFF_W2 + MLP_H * MLP_H,
                  OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_H * MLP_OUT, MLP_NPARAM = OFF_B3 + MLP_OUT;

struct MlpWs {
    __nv_bfloat16 *wb;                 // BF16 copy of the parameters [MLP_NPARAM]
    __nv_bfloat16 *xb, *h1b, *h2b;     // BF16 operands [B][3], [B][256], [B][256]
    float *z1, *z2, *y;                // pre-activations and output (FP32)
    __nv_bfloat16 *dyb, *dz2b, *dz1b;  // BF16 gradient operands
    float *dh;                         // [B][256] scratch
};

static size_t mlp_layout(int64_t B, MlpWs *w, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    MlpWs t;
    t.wb = (__nv_bfloat16 *)take(2 * MLP_NPARAM);
    t.xb = (__nv_bfloat16 *)take(2 * B * MLP_IN);
    t.h1b = (__nv_bfloat16 *)take(2 * B * MLP_H);
    t.h2b = (__nv_bfloat16 *)take(2 * B * MLP_H);
    t.z1 = (float *)take(4 * B * MLP_H);
    t.z2 = (float *)take(4 * B * MLP_H);
    t.y = (float *)take(4 * B * MLP_OUT);
    t.dyb = (__nv_bfloat16 *)take(2 * B * MLP_OUT);
    t.dz2b = (__nv_bfloat16 *)take(2 * B * MLP_H);
    t.dz1b = (__nv_bfloat16 *)take(2 * B * MLP_H);
    t.dh = (float *)take(4 * B * MLP_H);
    if (w) *w = t;
    return off;
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__global__ void to_bf16(const float *a, __nv_bfloat16 *b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

// C[M][N] = op(A) op(B) (+ bias[N]); op(A)[m][k] = TA ? A[k][m] : A[m][k] (A has row stride lda),
// op(B)[k][n] = TB ? B[n][k] : B[k][n]. BF16 operands, FP32 accumulation, 64x64 tile per block.
// EPI 0: C = acc + bias (FP32 out); EPI 1: z = acc + bias, h = bf16(gelu(z)); EPI 2: C = acc
// (gradient of a weight).
constexpr int GT = 64, GK = 16;

template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) mlp_gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *Bm, int ldb,
                                                const float *bias, float *C, __nv_bfloat16 *H, int ldc, int M, int N,
                                                int K) {
    __shared__ float As[GK][GT + 1], Bs[GK][GT + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int i = threadIdx.x; i < GK * GT; i += 256) {
            const int kk = i / GT, mm = i % GT;
            const int m = m0 + mm, k = k0 + kk, n = n0 + mm;
            float av = 0.f, bv = 0.f;
            if (m < M && k < K) av = __bfloat162float(TA ? A[(int64_t)k * lda + m] : A[(int64_t)m * lda + k]);
            if (n < N && k < K) bv = __bfloat162float(TB ? Bm[(int64_t)n * ldb + k] : Bm[(int64_t)k * ldb + n]);
            As[kk][mm] = av;
            Bs[kk][mm] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j];
            if (EPI != 2 && bias) v += bias[n];
            C[(int64_t)m * ldc + n] = v;
            if (EPI == 1) H[(int64_t)m * ldc + n] = __float2bfloat16_rn(gelu(v));
        }
}

// dy = (y - t) / (B*64) -> bf16; loss partial sums
__global__ void mlp_loss(const float *y, const float *t, int64_t n, float scale, __nv_bfloat16 *dyb, float *loss) {
    float l = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        l += d * d;
        dyb[i] = __float2bfloat16_rn(d * scale);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, 0.5f * scale * l);
}

// dz = dh .* gelu'(z) -> bf16
__global__ void mlp_gelu_back(const float *dh, const float *z, int64_t n, __nv_bfloat16 *dzb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dzb[i] = __float2bfloat16_rn(dh[i] * gelu_d(z[i]));
}

// column sums of a [B][N] bf16 gradient into grad[N]
__global__ void mlp_colsum(const __nv_bfloat16 *g, int64_t B, int N, float *out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int64_t b = 0; b < B; ++b) s += __bfloat162float(g[b * N + n]);
    out[n] = s;
}

__global__ void mlp_adam(float *w, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
                         float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

static dim3 ggrid(int M, int N) { return dim3((N + GT - 1) / GT, (M + GT - 1) / GT); }

static int mlp_forward(const float *params, const float *x, int64_t B, MlpWs &w, cudaStream_t s) {
    to_bf16<<<256, 256, 0, s>>>(params, w.wb, MLP_NPARAM);
    to_bf16<<<64, 256, 0, s>>>(x, w.xb, B * MLP_IN);
    mlp_gemm<false, false, 1><<<ggrid((int)B, MLP_H), 256, 0, s>>>(w.xb, MLP_IN, w.wb + OFF_W1, MLP_H, params + OFF_B1,
                                                                   w.z1, w.h1b, MLP_H, (int)B, MLP_H, MLP_IN);
    mlp_gemm<false, false, 1><<<ggrid((int)B, MLP_H), 256, 0, s>>>(w.h1b, MLP_H, w.wb + OFF_W2, MLP_H, params + OFF_B2,
                                                                   w.z2, w.h2b, MLP_H, (int)B, MLP_H, MLP_H);
    mlp_gemm<false, false, 0><<<ggrid((int)B, MLP_OUT), 256, 0, s>>>(w.h2b, MLP_H, w.wb + OFF_W3, MLP_OUT,
                                                                     params + OFF_B3, w.y, nullptr, MLP_OUT, (int)B,
                                                                     MLP_OUT, MLP_H);
    return launch_status();
}

}  // namespace fl

extern "C" {

int64_t fl_MLP_num_params(void) { return fl::MLP_NPARAM; }

size_t fl_MLP_workspace_size(int64_t batch) { return fl::mlp_layout(batch, nullptr, nullptr); }

int fl_MLPForward(const float *params, const float *x, int64_t batch, float *y, void *workspace, size_t ws_bytes,
                  fl_stream_t stream) {
    if (!params || !x || !y || !workspace || batch <= 0) return FL_ERR_ARG;
    if (fl::mlp_layout(batch, nullptr, nullptr) > ws_bytes) return FL_ERR_CAPACITY;
    fl::MlpWs w;
    fl::mlp_layout(batch, &w, (char *)workspace);
    cudaStream_t s = (cudaStream_t)stream;
    const int st = fl::mlp_forward(params, x, batch, w, s);
    if (st != FL_OK) return st;
    FL_CUDA_TRY(cudaMemcpyAsync(y, w.y, sizeof(float) * batch * fl::MLP_OUT, cudaMemcpyDeviceToDevice, s));
    return FL_OK;
}

int fl_MLPGradients(const float *params, const float *x, const float *target, int64_t batch, float *grads,
                    float *loss, void *workspace, size_t ws_bytes, fl_stream_t stream) {
    using namespace fl;
    if (!params || !x || !target || !grads || !workspace || batch <= 0) return FL_ERR_ARG;
    if (mlp_layout(batch, nullptr, nullptr) > ws_bytes) return FL_ERR_CAPACITY;
    MlpWs w;
    mlp_layout(batch, &w, (char *)workspace);
    cudaStream_t s = (cudaStream_t)stream;
    const int B = (int)batch;
    int st = mlp_forward(params, x, batch, w, s);
    if (st != FL_OK) return st;
    if (loss) FL_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
    mlp_loss<<<64, 256, 0, s>>>(w.y, target, batch * MLP_OUT, 1.f / (float)(batch * MLP_OUT), w.dyb, loss);
    // layer 3
    mlp_gemm<true, false, 2><<<ggrid(MLP_H, MLP_OUT), 256, 0, s>>>(w.h2b, MLP_H, w.dyb, MLP_OUT, nullptr,
                                                                   grads + OFF_W3, nullptr, MLP_OUT, MLP_H, MLP_OUT, B);
    mlp_colsum<<<1, MLP_OUT, 0, s>>>(w.dyb, batch, MLP_OUT, grads + OFF_B3);
    mlp_gemm<false, true, 2><<<ggrid(B, MLP_H), 256, 0, s>>>(w.dyb, MLP_OUT, w.wb + OFF_W3, MLP_OUT, nullptr, w.dh,
                                                             nullptr, MLP_H, B, MLP_H, MLP_OUT);
    mlp_gelu_back<<<64, 256, 0, s>>>(w.dh, w.z2, batch * MLP_H, w.dz2b);
    // layer 2
    mlp_gemm<true, false, 2><<<ggrid(MLP_H, MLP_H), 256, 0, s>>>(w.h1b, MLP_H, w.dz2b, MLP_H, nullptr, grads + OFF_W2,
                                                                 nullptr, MLP_H, MLP_H, MLP_H, B);
    mlp_colsum<<<1, MLP_H, 0, s>>>(w.dz2b, batch, MLP_H, grads + OFF_B2);
    mlp_gemm<false, true, 2><<<ggrid(B, MLP_H), 256, 0, s>>>(w.dz2b, MLP_H, w.wb + OFF_W2, MLP_H, nullptr, w.dh,
                                                             nullptr, MLP_H, B, MLP_H, MLP_H);
    mlp_gelu_back<<<64, 256, 0, s>>>(w.dh, w.z1, batch * MLP_H, w.dz1b);
    // layer 1
    mlp_gemm<true, false, 2><<<ggrid(MLP_IN, MLP_H), 256, 0, s>>>(w.xb, MLP_IN, w.dz1b, MLP_H, nullptr, grads + OFF_W1,
                                                                  nullptr, MLP_H, MLP_IN, MLP_H, B);
    mlp_colsum<<<1, MLP_H, 0, s>>>(w.dz1b, batch, MLP_H, grads + OFF_B1);
    return launch_status();
}

int fl_MLPAdamStep(float *params, const float *grads, float *m, float *v, int64_t step, float lr, float beta1,
                   float beta2, float eps, fl_stream_t stream) {
    if (!params || !grads || !m || !v || step < 1) return FL_ERR_ARG;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    fl::mlp_adam<<<256, 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, fl::MLP_NPARAM, lr, beta1, beta2, eps, c1,
                                                        c2);
    return fl::launch_status();
}

}  // extern "C"
