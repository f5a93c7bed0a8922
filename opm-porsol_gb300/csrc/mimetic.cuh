// mimetic.cuh -- per-cell pieces of the mimetic inner product shared by the static
// inner-product kernel and the adjoint (derivative) kernel.
//
// MimeticIPEvaluator::buildStaticContrib (MimeticIPEvaluator.hpp:201-270):
//   W = (N K N^T + t A (I - Q Q^T) A) / |c|,  t = 6 tr(K) / 3,
//   N = A n (area-weighted normals), Q = orth(A (x_f - x_c)).
// W is linear in K, which the adjoint uses: dW/d ln k_a of a diagonal tensor is W evaluated
// at k_a e_a e_a^T, and dW/d ln s of K -> s K is W itself.
#pragma once

#include "porsol_internal.h"

namespace porsol {

// Packed index of the symmetric entry (r, s): upper triangle, column by column.
__device__ __forceinline__ int pk(int r, int s)
{
    return r <= s ? s * (s + 1) / 2 + r : r * (r + 1) / 2 + s;
}

// Face areas a, area-weighted normals N and the orthonormalised area-weighted centroid
// offsets Q of cell c (faces f0 .. f0+nf-1; rows >= nf are zero).  Q is formed by
// Gram-Schmidt with one re-orthogonalisation pass; Q Q^T does not depend on the orthonormal
// basis chosen, so this matches the reference's Householder QR.  Returns false for a
// degenerate cell (the reference asserts there).
template <int MAXNF>
__device__ __forceinline__ bool cell_frame(int c, int f0, int nf, const double* __restrict__ area,
                                           const double* __restrict__ fcent, const double* __restrict__ fnormal,
                                           const double* __restrict__ ccent, double (&a)[MAXNF],
                                           double (&N)[MAXNF][3], double (&Q)[MAXNF][3])
{
    const double cc0 = ccent[3 * (size_t)c], cc1 = ccent[3 * (size_t)c + 1], cc2 = ccent[3 * (size_t)c + 2];
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        a[i] = 0.0;
        N[i][0] = N[i][1] = N[i][2] = 0.0;
        Q[i][0] = Q[i][1] = Q[i][2] = 0.0;
        if (i < nf) {
            const size_t hf = f0 + i;
            a[i] = area[hf];
            Q[i][0] = (fcent[3 * hf] - cc0) * a[i];
            Q[i][1] = (fcent[3 * hf + 1] - cc1) * a[i];
            Q[i][2] = (fcent[3 * hf + 2] - cc2) * a[i];
            N[i][0] = fnormal[3 * hf] * a[i];
            N[i][1] = fnormal[3 * hf + 1] * a[i];
            N[i][2] = fnormal[3 * hf + 2] * a[i];
        }
    }
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
            for (int k = 0; k < j; ++k) {
                double d = 0.0;
#pragma unroll
                for (int i = 0; i < MAXNF; ++i) d += Q[i][k] * Q[i][j];
#pragma unroll
                for (int i = 0; i < MAXNF; ++i) Q[i][j] -= d * Q[i][k];
            }
        }
        double nrm = 0.0;
#pragma unroll
        for (int i = 0; i < MAXNF; ++i) nrm += Q[i][j] * Q[i][j];
        nrm = sqrt(nrm);
        if (!(nrm > 0.0)) {
            ok = false;
            nrm = 1.0;
        }
        const double inv = 1.0 / nrm;
#pragma unroll
        for (int i = 0; i < MAXNF; ++i) Q[i][j] *= inv;
    }
    return ok;
}

// (A (I - Q Q^T) A)_{ij}
template <int MAXNF>
__device__ __forceinline__ double projected(int i, int j, const double (&a)[MAXNF], const double (&Q)[MAXNF][3])
{
    const double P = (i == j ? 1.0 : 0.0) - (Q[i][0] * Q[j][0] + Q[i][1] * Q[j][1] + Q[i][2] * Q[j][2]);
    return a[i] * P * a[j];
}

}  // namespace porsol
