// Host build of the reference-tensor contraction's arithmetic (florence_gb300/csrc/
// fl_reftensor_math.cuh), test infrastructure: digit planes, the exact recombination of the level
// sums, and an emulation of one GEMM entry as the tensor cores form it (exact level sums for the
// levels 0-3, FP32 accumulation per 16-wide K step for the shared levels 4 to 6).
#include <cmath>

#include "../florence_gb300/csrc/fl_reftensor_math.cuh"

extern "C" {

void rt_digits_c(float h, float l, float sc, float *out) {
    float p[fl::RT_DIG];
    fl::rt_digits(h, l, sc, p);
    for (int s = 0; s < fl::RT_DIG; ++s) out[s] = p[s];
}

void rt_digits_f64_c(double y, float *out) {
    float q[fl::RT_DIG];
    fl::rt_digits_f64(y, q);
    for (int t = 0; t < fl::RT_DIG; ++t) out[t] = q[t];
}

double rt_i64_to_f64_c(long long z, int e2) { return fl::rt_i64_to_f64(z, e2); }

double rt_combine_c(const float *acc, int e2) { return fl::rt_combine(acc[0], acc[1], acc[2], acc[3], acc[4], e2); }

void rt_pair_c(int n, int *a, int *b) { fl::rt_pair(n, *a, *b); }

void rt_row_scale_c(float amax, int *E, float *sc) { fl::rt_row_scale(amax, *E, *sc); }

int rt_sym9_c(int I, int K) { return fl::rt_sym9(I, K); }

// One entry sum_k (ah[k] + al[k]) b[k] as the contraction forms it, K <= 256.
double rt_dot_c(int K, const float *ah, const float *al, const double *b) {
    float amax = 0.f;
    double bmax = 0.0;
    for (int k = 0; k < K; ++k) {
        amax = std::fmax(amax, std::fabs(ah[k]));
        bmax = std::fmax(bmax, std::fabs(b[k]));
    }
    int E, F = 0;
    float sc;
    fl::rt_row_scale(amax, E, sc);
    if (bmax > 0.0) std::frexp(bmax, &F);
    double lev[4] = {0, 0, 0, 0};
    float acc4 = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        double l45 = 0.0;  // levels 4 to 6 of this K step, exact
        for (int k = k0; k < k0 + 16 && k < K; ++k) {
            float p[fl::RT_DIG], q[fl::RT_DIG];
            fl::rt_digits(ah[k], al[k], sc, p);
            fl::rt_digits_f64(std::ldexp(b[k], 7 - F), q);
            for (int s = 0; s < fl::RT_DIG; ++s)
                for (int t = 0; t + s < fl::RT_DIG; ++t) {
                    const double pr = (double)p[s] * (double)q[t];  // exact: 8-bit significands
                    if (s + t < 4) lev[s + t] += pr;
                    else l45 += pr;
                }
        }
        acc4 = acc4 + (float)l45;  // FP32 accumulation across K steps
    }
    return fl::rt_combine((float)lev[0], (float)lev[1], (float)lev[2], (float)lev[3], acc4, E + F - 14);
}

}  // extern "C"
