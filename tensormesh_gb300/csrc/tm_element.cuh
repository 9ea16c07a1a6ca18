// Element geometry shared by the assembly, geometry and adjoint kernels.
//
// Convention of the reference (element/element.py:962-966): the Jacobian is
// J[i][j] = sum_b dphi[i][b] X[b][j] = d x_j / d xi_i (the transpose of
// dx/dxi), and the physical gradient of phi_b is
// g_b[j] = sum_i dphi[i][b] Jinv[j][i].  With the cofactor rows cof[i] of J
// (Jinv[j][i] = cof[i][j] / det J) this is g_b = (sum_i dphi[i][b] cof[i]) / det.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/tensormesh_gb300.h"

namespace tmk {

template <int ET> struct Traits;
template <> struct Traits<TM_TRI3>  { static constexpr int D = 2, B = 3,  P1 = 1; };
template <> struct Traits<TM_TET4>  { static constexpr int D = 3, B = 4,  P1 = 1; };
template <> struct Traits<TM_TRI6>  { static constexpr int D = 2, B = 6,  P1 = 0; };
template <> struct Traits<TM_TET10> { static constexpr int D = 3, B = 10, P1 = 0; };
template <> struct Traits<TM_QUAD4> { static constexpr int D = 2, B = 4,  P1 = 0; };
template <> struct Traits<TM_QUAD9> { static constexpr int D = 2, B = 9,  P1 = 0; };

// offsets (in doubles) of the packed reference tables
struct TableLayout {
    int w, phi, dphi, mhat, lhat, wsum, total;
};
__host__ __device__ inline TableLayout table_layout(int Q, int B, int D) {
    TableLayout t;
    t.w = 0;
    t.phi = Q;
    t.dphi = t.phi + Q * B;
    t.mhat = t.dphi + Q * D * B;
    t.lhat = t.mhat + B * B;
    t.wsum = t.lhat + B;
    t.total = t.wsum + 1;
    return t;
}

// (a, b) of the l-th entry of the upper triangle, row-major
template <int B>
__device__ __forceinline__ void upper_pair(int l, int& a, int& b) {
    a = 0;
    while (l >= B - a) {
        l -= B - a;
        ++a;
    }
    b = a + l;
}

template <typename R>
__device__ __forceinline__ R ldg(const R* p) { return __ldg(p); }

// cofactor rows of a DxD matrix given by rows J[i][:]; returns det
template <typename R>
__device__ __forceinline__ R cofactors(const R (&J)[2][2], R (&cof)[2][2]) {
    cof[0][0] = J[1][1];
    cof[0][1] = -J[1][0];
    cof[1][0] = -J[0][1];
    cof[1][1] = J[0][0];
    return J[0][0] * J[1][1] - J[0][1] * J[1][0];
}
template <typename R>
__device__ __forceinline__ R cofactors(const R (&J)[3][3], R (&cof)[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        cof[i][0] = J[i1][1] * J[i2][2] - J[i1][2] * J[i2][1];
        cof[i][1] = J[i1][2] * J[i2][0] - J[i1][0] * J[i2][2];
        cof[i][2] = J[i1][0] * J[i2][1] - J[i1][1] * J[i2][0];
    }
    return J[0][0] * cof[0][0] + J[0][1] * cof[0][1] + J[0][2] * cof[0][2];
}

// P1 simplex: "unscaled gradients" C[b] with g_b = C[b] / det
template <typename R, int D>
__device__ __forceinline__ R p1_gradients(const R (&X)[D + 1][D], R (&C)[D + 1][D]) {
    R J[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) J[i][j] = X[i + 1][j] - X[0][j];
    R cof[D][D];
    const R det = cofactors<R>(J, cof);
#pragma unroll
    for (int j = 0; j < D; ++j) {
        R s = 0;
#pragma unroll
        for (int i = 0; i < D; ++i) {
            C[i + 1][j] = cof[i][j];
            s += cof[i][j];
        }
        C[0][j] = -s;
    }
    return det;
}

template <typename R, int D>
__device__ __forceinline__ R dot(const R* a, const R* b) {
    R s = a[0] * b[0];
#pragma unroll
    for (int d = 1; d < D; ++d) s += a[d] * b[d];
    return s;
}

// isotropic elasticity block (B_a^T C B_b) for gradients ga, gb, scaled by f:
// f * (lam ga[r] gb[s] + mu (ga[s] gb[r] + delta_rs ga.gb))
template <typename R, int D>
__device__ __forceinline__ void elastic_block(const R* ga, const R* gb, R lam, R mu, R f, R* blk,
                                              bool accumulate) {
    const R gg = dot<R, D>(ga, gb);
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int s = 0; s < D; ++s) {
            R v = lam * ga[r] * gb[s] + mu * (ga[s] * gb[r] + (r == s ? gg : R(0)));
            v *= f;
            blk[r * D + s] = accumulate ? blk[r * D + s] + v : v;
        }
}

// the same block from the outer-product sum A = sum_q f_q ga_q gb_q^T:
// lam A[r][s] + mu (A[s][r] + delta_rs tr A).  Accumulating A over the
// quadrature points (D multiplies and D^2 FMAs per point) and forming the
// block once takes about a quarter of the float64 instructions of
// elastic_block per point
template <typename R, int D>
__device__ __forceinline__ void elastic_block_outer(const R (&A)[D][D], R lam, R mu, R* blk) {
    R tr = A[0][0];
#pragma unroll
    for (int d = 1; d < D; ++d) tr += A[d][d];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int s = 0; s < D; ++s) blk[r * D + s] = lam * A[r][s] + mu * (A[s][r] + (r == s ? tr : R(0)));
}

}  // namespace tmk
