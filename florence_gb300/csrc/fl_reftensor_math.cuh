// fl_reftensor_math.cuh -- integer and float arithmetic of the reference-tensor contraction
// (fl_reftensor.cu) that does not depend on the GPU: digit planes of a float pair, the exact
// recombination of the level sums into an FP64 value, index maps. Plain C++ so that the kernel
// and a host build of the same source (the CPU tests) use identical arithmetic.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define FL_RT_HD __host__ __device__ __forceinline__
#else
#define FL_RT_HD inline
#endif

namespace fl {

constexpr int RT_DIG = 7;   // digit planes per operand
constexpr int RT_NB = 80;   // node-pair columns per chunk

FL_RT_HD constexpr int rt_pairs(int npe) { return npe * (npe + 1) / 2; }
FL_RT_HD constexpr int rt_chunks(int npe) { return (rt_pairs(npe) + RT_NB - 1) / RT_NB; }
FL_RT_HD constexpr int rt_ksteps(int nq) { return (9 * nq + 15) / 16; }

// byte offset of (row r, column k) in a K-major, unswizzled BF16 operand 16 columns wide: 8 x 8
// core matrices of 128 bytes, K-adjacent ones 128 bytes apart, row-adjacent ones 256
FL_RT_HD uint32_t kmaj16(int r, int k) {
    return (uint32_t)((r >> 3) * 256 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// index of (I,K), I,K in 0..8, in the packed upper triangle of a symmetric 9x9 (the Gauss-point
// kernel's layout of the pulled-back tangent)
FL_RT_HD int rt_sym9(int I, int K) {
    const int a = I < K ? I : K, b = I < K ? K : I;
    return a * 9 - (a * (a - 1)) / 2 + (b - a);
}

// node pair (a <= b) of pair column n: n = b (b + 1) / 2 + a
FL_RT_HD void rt_pair(int n, int &a, int &b) {
    int bb = (int)((std::sqrt(8.0f * (float)n + 1.0f) - 1.0f) * 0.5f);
    while (bb * (bb + 1) / 2 > n) --bb;
    while ((bb + 1) * (bb + 2) / 2 <= n) ++bb;
    b = bb;
    a = n - bb * (bb + 1) / 2;
}

#ifdef __CUDA_ARCH__
#define FL_RT_ADD(x, y) __fadd_rn((x), (y))
#define FL_RT_SUB(x, y) __fsub_rn((x), (y))
#else
#define FL_RT_ADD(x, y) ((x) + (y))
#define FL_RT_SUB(x, y) ((x) - (y))
#endif

// Seven digit planes of the float pair (h + l) * sc, |h sc| < 128 (sc a power of two): p_s is a
// multiple of 2^-8s with |p_s| <= 128 * 2^-8s (eight significant bits, exact in BF16) and
// p_0 + ... + p_6 = (h + l) sc to within 2^-48. Each rounding is the add-and-subtract of
// 1.5 * 2^m, which rounds to the nearest multiple of 2^(m-23); every remainder is exact (Sterbenz);
// the low word joins through an error-free two-sum, its rounding error after the fourth digit.
FL_RT_HD void rt_digits(float h, float l, float sc, float (&p)[RT_DIG]) {
    const float yh = h * sc, yl = l * sc;
    p[0] = FL_RT_SUB(FL_RT_ADD(yh, 12582912.0f), 12582912.0f);  // 1.5 * 2^23: integers
    float r = FL_RT_SUB(yh, p[0]);
    p[1] = FL_RT_SUB(FL_RT_ADD(r, 49152.0f), 49152.0f);         // 1.5 * 2^15: multiples of 2^-8
    r = FL_RT_SUB(r, p[1]);
    const float s0 = FL_RT_ADD(r, yl);                          // two-sum: s0 + e = r + yl
    const float bv = FL_RT_SUB(s0, r);
    const float e = FL_RT_ADD(FL_RT_SUB(r, FL_RT_SUB(s0, bv)), FL_RT_SUB(yl, bv));
    p[2] = FL_RT_SUB(FL_RT_ADD(s0, 192.0f), 192.0f);            // 1.5 * 2^7: multiples of 2^-16
    float s = FL_RT_SUB(s0, p[2]);
    p[3] = FL_RT_SUB(FL_RT_ADD(s, 0.75f), 0.75f);               // 1.5 * 2^-1: multiples of 2^-24
    s = FL_RT_ADD(FL_RT_SUB(s, p[3]), e);
    p[4] = FL_RT_SUB(FL_RT_ADD(s, 0.0029296875f), 0.0029296875f);             // 1.5 * 2^-9: 2^-32
    s = FL_RT_SUB(s, p[4]);
    p[5] = FL_RT_SUB(FL_RT_ADD(s, 1.1444091796875e-05f), 1.1444091796875e-05f);  // 1.5 * 2^-17: 2^-40
    s = FL_RT_SUB(s, p[5]);
    p[6] = FL_RT_SUB(FL_RT_ADD(s, 4.470348358154297e-08f), 4.470348358154297e-08f);  // 1.5 * 2^-25: 2^-48
}

#undef FL_RT_ADD
#undef FL_RT_SUB

// Seven digit planes of an FP64 value y, |y| < 128 (the reference tensor, split once per call):
// q_t = rint of the remainder in units of 2^-8t, times 2^-8t; |q_t| <= 128 * 2^-8t, exact in BF16
FL_RT_HD void rt_digits_f64(double y, float (&q)[RT_DIG]) {
    double scale = 1.0;
    for (int t = 0; t < RT_DIG; ++t) {
        const double d = std::rint(y);
        q[t] = (float)(d * scale);
        y = (y - d) * 256.0;
        scale *= 1.0 / 256.0;
    }
}

// z * 2^e2 rounded to the nearest FP64 value (ties to even) with integer instructions; results
// outside the normal range take the slow path
FL_RT_HD double rt_i64_to_f64(long long z, int e2) {
    if (z == 0) return 0.0;
    const unsigned long long sgn = z < 0 ? 0x8000000000000000ull : 0ull;
    unsigned long long m = z < 0 ? 0ull - (unsigned long long)z : (unsigned long long)z;
#ifdef __CUDA_ARCH__
    int lz = __clzll((long long)m);
#else
    int lz = __builtin_clzll(m);
#endif
    m <<= lz;                                   // leading one at bit 63
    unsigned long long mant = m >> 11;          // 53 significant bits
    const unsigned rem = (unsigned)(m & 0x7ffull);
    if (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) {
        ++mant;
        if (mant >> 53) {
            mant >>= 1;
            --lz;
        }
    }
    const int ex = 63 - lz + e2 + 1023;
    if (ex <= 0 || ex >= 2047) return std::ldexp((double)z, e2);
    const unsigned long long bits = sgn | ((unsigned long long)ex << 52) | (mant & 0xfffffffffffffull);
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)bits);
#else
    double d;
    std::memcpy(&d, &bits, sizeof d);
    return d;
#endif
}

FL_RT_HD int rt_rint(float x) {
#ifdef __CUDA_ARCH__
    return __float2int_rn(x);
#else
    return (int)std::nearbyint(x);
#endif
}
FL_RT_HD long long rt_llrint(float x) {
#ifdef __CUDA_ARCH__
    return __float2ll_rn(x);
#else
    return (long long)std::nearbyint((double)x);
#endif
}

// The FP64 entry from the five level accumulators: a_L (L <= 3) holds the exact integer sum of
// level L times 2^-8L, a4 the levels 4 to 6 (rounded). Their sum, as a fixed-point integer in units
// of 2^-40, times 2^(e2 - 40) where e2 = row exponent + column exponent - 14.
FL_RT_HD double rt_combine(float a0, float a1, float a2, float a3, float a4, int e2) {
    const long long z = ((long long)rt_rint(a0) << 40) + ((long long)rt_rint(a1 * 256.0f) << 32) +
                        ((long long)rt_rint(a2 * 65536.0f) << 24) + ((long long)rt_rint(a3 * 16777216.0f) << 16) +
                        rt_llrint(a4 * 1099511627776.0f);
    return rt_i64_to_f64(z, e2 - 40);
}

// Row scale of the digit split: E with max |x| < 2^E and sc = 2^(7 - E), so |x sc| < 128. A row
// whose largest magnitude is zero or below 2^-100 gets sc = 0 (all digits zero) and E = 0.
FL_RT_HD void rt_row_scale(float amax, int &E, float &sc) {
    unsigned bits;
#ifdef __CUDA_ARCH__
    bits = __float_as_uint(amax);
#else
    std::memcpy(&bits, &amax, sizeof bits);
#endif
    const int ef = (int)((bits >> 23) & 0xffu);  // amax >= 0
    if (ef < 27) {
        E = 0;
        sc = 0.0f;
        return;
    }
    E = ef - 126;                                 // amax < 2^(ef - 126)
    const unsigned sb = (unsigned)(127 + 7 - E) << 23;
#ifdef __CUDA_ARCH__
    sc = __uint_as_float(sb);
#else
    std::memcpy(&sc, &sb, sizeof sc);
#endif
}

}  // namespace fl
