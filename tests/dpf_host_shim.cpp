// Host build of the device DPF arithmetic (florence_gb300/csrc/fl_dpf.cuh), test infrastructure:
// the element tangent and residual of one element, summed over its Gauss points exactly as the
// kernel sums them, for comparison with the reference's golden element matrices.
#include <vector>

#include "../florence_gb300/csrc/fl_dpf.cuh"

template <class MAT>
static double element(const MAT &m, int npe, int nq, const double *Jm, const double *w, const double *X,
                      const double *x, const double *phi, int update, const double *N, double *K, double *t) {
    using namespace fl::dpf;
    const int ndof = NV * npe;
    std::vector<double> SG(3 * npe * nq), H(HV * HV * nq), sig(9 * nq), D(3 * nq), dv(nq);
    double minJ = 1e300;
    for (int g = 0; g < nq; ++g) {
        const double J = gauss_point(npe, nq, g, Jm, w[g], X, x, phi, update, m, N, &SG[3 * npe * g], &dv[g],
                                     &D[3 * g], &sig[9 * g], &H[HV * HV * g]);
        minJ = J < minJ ? J : minJ;
    }
    for (int r = 0; r < ndof; ++r) {
        for (int c = 0; c < ndof; ++c) {
            double s = 0.0;
            for (int g = 0; g < nq; ++g)
                s += dv[g] * entry(r / NV, r % NV, c / NV, c % NV, npe, &SG[3 * npe * g], &H[HV * HV * g], &sig[9 * g]);
            K[r * ndof + c] = s;
        }
        double s = 0.0;
        if (update)
            for (int g = 0; g < nq; ++g) s += dv[g] * residual(r / NV, r % NV, npe, &SG[3 * npe * g], &D[3 * g], &sig[9 * g]);
        t[r] = s;
    }
    return minJ;
}

// the same element through pair_block (the kernel's node-pair blocks, upper node pairs mirrored)
template <class MAT>
static double element_blocks(const MAT &m, int npe, int nq, const double *Jm, const double *w, const double *X,
                             const double *x, const double *phi, int update, const double *N, double *K, double *t) {
    using namespace fl::dpf;
    const int ndof = NV * npe;
    std::vector<double> SG(3 * npe * nq), H(HV * HV * nq), sig(9 * nq), D(3 * nq), dv(nq);
    double minJ = 1e300;
    for (int g = 0; g < nq; ++g) {
        const double J = gauss_point(npe, nq, g, Jm, w[g], X, x, phi, update, m, N, &SG[3 * npe * g], &dv[g],
                                     &D[3 * g], &sig[9 * g], &H[HV * HV * g]);
        minJ = J < minJ ? J : minJ;
    }
    for (int a = 0; a < npe; ++a)
        for (int b = a; b < npe; ++b) {
            double B[NV][NV] = {};
            for (int g = 0; g < nq; ++g) pair_block(a, b, npe, &SG[3 * npe * g], &H[HV * HV * g], &sig[9 * g], dv[g], B);
            for (int v = 0; v < NV; ++v)
                for (int u = 0; u < NV; ++u) {
                    K[(a * NV + v) * ndof + b * NV + u] = B[v][u];
                    K[(b * NV + u) * ndof + a * NV + v] = B[v][u];
                }
        }
    for (int r = 0; r < ndof; ++r) {
        double s = 0.0;
        if (update)
            for (int g = 0; g < nq; ++g) s += dv[g] * residual(r / NV, r % NV, npe, &SG[3 * npe * g], &D[3 * g], &sig[9 * g]);
        t[r] = s;
    }
    return minJ;
}

// material: 108 (params mu1, mu2, lamb, eps_2), 105 or 106 (mu1, mu2, lamb, eps_1, eps_2), 101 or 0
// (mu, lamb, eps_1), 1 the Steinmann model (mu, lamb, c1, c2, eps_1), 100 Piezoelectric_100
// (mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3, with the element's fibre direction N)
extern "C" double dpf_element(int material, int npe, int nq, const double *Jm, const double *w, const double *X,
                              const double *x, const double *phi, int update, const double *p, const double *N,
                              double *K, double *t, int blocks) {
    using namespace fl::dpf;
    if (blocks) {
        if (material == 108) return element_blocks(Em108{p[0], p[1], p[2], p[3]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
        if (material == 101) return element_blocks(Em101{p[0], p[1], p[2]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
        if (material == 0) return element_blocks(Em0{p[0], p[1], p[2]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
        if (material == 1)
            return element_blocks(EmSteinmann{p[0], p[1], p[2], p[3], p[4]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
        if (material == 105)
            return element_blocks(Em105{p[0], p[1], p[2], p[3], p[4]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
        if (material == 106)
            return element_blocks(Em106{p[0], p[1], p[2], p[3], p[4]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
        if (material == 100)
            return element_blocks(EmPiezo100{p[0], p[1], p[2], p[3], p[4], p[5], p[6]}, npe, nq, Jm, w, X, x, phi,
                                  update, N, K, t);
        return -1.0;
    }
    if (material == 108) return element(Em108{p[0], p[1], p[2], p[3]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
    if (material == 101) return element(Em101{p[0], p[1], p[2]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
    if (material == 0) return element(Em0{p[0], p[1], p[2]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
    if (material == 1)
        return element(EmSteinmann{p[0], p[1], p[2], p[3], p[4]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
    if (material == 105) return element(Em105{p[0], p[1], p[2], p[3], p[4]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
    if (material == 106) return element(Em106{p[0], p[1], p[2], p[3], p[4]}, npe, nq, Jm, w, X, x, phi, update, N, K, t);
    if (material == 100)
        return element(EmPiezo100{p[0], p[1], p[2], p[3], p[4], p[5], p[6]}, npe, nq, Jm, w, X, x, phi, update, N, K,
                       t);
    return -1.0;
}
