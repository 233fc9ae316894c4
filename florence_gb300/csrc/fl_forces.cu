// fl_forces.cu -- external forces on the device: surface traction on the boundary faces
// (replaces AssembleExternalTractionForces, Florence/FiniteElements/Assembly/Assembly.py:451-514)
// and the body force (AssembleBodyForces, Assembly.py:516-560).
//
// The reference integrates both with the parent-element quadrature weights alone (no face or
// volume Jacobian): F[(a, i)] += t_i sum_g N_a(g) w_g for every face a traction is applied on
// (Assembly.py:476-481), and F[(a, z)] += -rho sum_g N_a(g) w_g for every element (:534-538).
// With face gradients Jm_face [2][npf][nq] and the points, the traction is integrated over the
// physical face instead: w_g |dX/dxi x dX/deta| at every Gauss point. One thread per (face or
// element, node); the node's sum of the basis values is formed once per thread.
#include <cstdint>

#include "fl_common.cuh"

namespace fl {

__global__ void traction_kernel(const uint64_t *faces, int64_t nface, int npf, const uint8_t *flags,
                                const double *traction, const double *Bases, const double *w, int nq,
                                const double *points, const double *Jm_face, int64_t nnode, double *F, int *err) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nface * npf) return;
    const int64_t f = t / npf;
    const int a = (int)(t % npf);
    if (flags && !flags[f]) return;
    const uint64_t nd = faces[f * npf + a];
    if (nd >= (uint64_t)nnode) {
        atomicOr(err, FL_FLAG_BAD_INDEX);
        return;
    }
    double s = 0.0;
    for (int g = 0; g < nq; ++g) {
        double wg = w[g];
        if (Jm_face) {  // |dX/dxi x dX/deta| of the physical face at Gauss point g
            double d0[3] = {0, 0, 0}, d1[3] = {0, 0, 0};
            for (int b = 0; b < npf; ++b) {
                const uint64_t nb = faces[f * npf + b];
                const double j0 = Jm_face[((size_t)0 * npf + b) * nq + g], j1 = Jm_face[((size_t)1 * npf + b) * nq + g];
                if (nb >= (uint64_t)nnode) continue;
                for (int k = 0; k < 3; ++k) {
                    d0[k] = fma(j0, points[nb * 3 + k], d0[k]);
                    d1[k] = fma(j1, points[nb * 3 + k], d1[k]);
                }
            }
            const double c0 = d0[1] * d1[2] - d0[2] * d1[1], c1 = d0[2] * d1[0] - d0[0] * d1[2],
                         c2 = d0[0] * d1[1] - d0[1] * d1[0];
            wg *= sqrt(c0 * c0 + c1 * c1 + c2 * c2);
        }
        s = fma(Bases[(size_t)a * nq + g], wg, s);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) atomicAdd(F + nd * 3 + i, traction[f * 3 + i] * s);
}

__global__ void body_force_kernel(const uint64_t *elements, int64_t nelem, int npe, const double *Bases,
                                  const double *w, int nq, double rho, int64_t nnode, double *F, int *err) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nelem * npe) return;
    const int64_t e = t / npe;
    const int a = (int)(t % npe);
    const uint64_t nd = elements[e * npe + a];
    if (nd >= (uint64_t)nnode) {
        atomicOr(err, FL_FLAG_BAD_INDEX);
        return;
    }
    double s = 0.0;
    for (int g = 0; g < nq; ++g) s = fma(Bases[(size_t)a * nq + g], w[g], s);
    atomicAdd(F + nd * 3 + 2, -rho * s);  // applied in the z direction (Assembly.py:534-535)
}

}  // namespace fl

extern "C" {

int fl_AssembleExternalTractionForces(const uint64_t *faces, int64_t nface, int64_t nodeperface,
                                      const uint8_t *neumann_flags, const double *applied_neumann,
                                      const double *Bases, const double *AllGauss, int64_t ngauss,
                                      const double *points, const double *Jm_face, int64_t nnode, double *F,
                                      int *flags, fl_stream_t stream) {
    if (nface < 0 || nodeperface <= 0 || ngauss <= 0 || nnode <= 0) return FL_ERR_ARG;
    if (nface == 0) return FL_OK;
    if (!faces || !applied_neumann || !Bases || !AllGauss || !F || !flags) return FL_ERR_ARG;
    if (Jm_face && !points) return FL_ERR_ARG;
    const int64_t n = nface * nodeperface;
    fl::traction_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        faces, nface, (int)nodeperface, neumann_flags, applied_neumann, Bases, AllGauss, (int)ngauss, points, Jm_face,
        nnode, F, flags);
    return fl::launch_status();
}

int fl_AssembleBodyForces(const uint64_t *elements, int64_t nelem, int64_t nodeperelem, const double *Bases,
                          const double *AllGauss, int64_t ngauss, double rho, int64_t nnode, double *F, int *flags,
                          fl_stream_t stream) {
    if (nelem < 0 || nodeperelem <= 0 || ngauss <= 0 || nnode <= 0) return FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!elements || !Bases || !AllGauss || !F || !flags) return FL_ERR_ARG;
    const int64_t n = nelem * nodeperelem;
    fl::body_force_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        elements, nelem, (int)nodeperelem, Bases, AllGauss, (int)ngauss, rho, nnode, F, flags);
    return fl::launch_status();
}

}  // extern "C"
