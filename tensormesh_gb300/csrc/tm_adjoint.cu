// Hand-written adjoint of the P1 diffusion and mass assembly (and of the load
// vector) with respect to the per-element coefficient and the node
// coordinates.
//
// The reference obtains these gradients by letting torch autograd run
// backwards through its assembly graph (index_add_, the integrand, the
// gradient einsums, torch.inverse, det and the coordinate gather,
// element/element.py:960-966, element/transformation.py:1267-1273,
// assemble/element_assembler.py:390-445), storing every intermediate.  Here
// one thread per element recomputes the geometry and applies the closed-form
// derivative; nothing per element is stored between forward and backward.
//
// For a P1 simplex with edge matrix J (rows x_{i+1} - x_0), M = J^-1,
// reference gradients G^ (columns -1, e_1 .. e_D) and element matrix
// K = kappa w |det J| G^T (J J^T)^-1 G^, a weight W_ab = dL/dK_ab gives, with
// S = G^ sym(W) G^T and P = M S M^T:
//     dL/dkappa = w |det J| tr(P)
//     dL/dJ     = kappa w |det J| M^T (tr(P) I - 2 P)
// The load vector b_a = |det J| beta_a (beta from the mass / load template)
// weighted by lambda_a adds (sum_a lambda_a b_a) M^T to dL/dJ; a mass matrix
// s |det J| Mhat weighted by W adds s |det J| (W : Mhat) M^T.  dL/dJ is
// spread to the nodes (row i to node i+1, minus the row sum to node 0) and
// reduced per node with the node chunk plan (fixed order, no atomics on
// values).  The weights come either from a CSR array dL/dvalues through the
// element->CSR slot map, or, for a loss through a linear solve K u = b with
// adjoint K lambda = dL/du, as W_ab = -lambda_a u_b without forming dL/dK.
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/tensormesh_gb300.h"
#include "tm_element.cuh"
#include "tm_reduce.cuh"
#include "tm_status.h"

namespace tmk {

constexpr int kAdjThreads = 256;

template <int ET, int KMODE, int LOAD>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint(const tm_adjoint_args a) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const TableLayout TL = table_layout(Q, B, D);
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm);
    double* LV = reinterpret_cast<double*>(sm + align16(sizeof(double) * TL.total));
    for (int k = threadIdx.x; k < TL.total; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();
    const double wsum = tab[TL.wsum];
    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const double* pts = static_cast<const double*>(a.points);
    const double* kap = static_cast<const double*>(a.kappa);
    const double* u = static_cast<const double*>(a.u);
    const double* lam = static_cast<const double*>(a.lam);
    const double* wcsr = static_cast<const double*>(a.weights);
    const double* fval = static_cast<const double*>(a.load_values);
    double* gkap = static_cast<double*>(a.grad_kappa);
    for (int el = threadIdx.x; el < ne; el += blockDim.x) {
        const int64_t i = i0 + el;
        const int64_t e = P.elem_perm[i];
        int32_t c[B];
        double X[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            c[b] = P.conn[i * B + b];
#pragma unroll
            for (int d = 0; d < D; ++d) X[b][d] = ldg(pts + (int64_t)c[b] * D + d);
        }
        double J[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int k = 0; k < D; ++k) J[r][k] = X[r + 1][k] - X[0][k];
        double cof[D][D];
        const double det = cofactors<double>(J, cof);
        const double inv = 1.0 / det;
        const double adet = fabs(det);
        double M[D][D];                       // M = J^-1, M[j][i] = cof[i][j] / det
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int k = 0; k < D; ++k) M[k][r] = cof[r][k] * inv;
        double GJ[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int k = 0; k < D; ++k) GJ[r][k] = 0.0;
        if constexpr (KMODE == TM_ADJ_M_CSR) {
            // M = s |det J| Mhat: dL/ds-part sum_ab W_ab Mhat_ab, and
            // d|det J| / dJ = |det J| J^-T
            double wm = 0.0;
#pragma unroll
            for (int p = 0; p < B; ++p)
#pragma unroll
                for (int q = 0; q < B; ++q) wm += ldg(wcsr + a.slot_map[(e * B + p) * B + q]) * tab[TL.mhat + p * B + q];
            if (gkap) gkap[e] = adet * wm;
            const double f = a.kappa_scale * adet * wm;
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) GJ[r][k] += f * M[k][r];
        }
        if constexpr (KMODE == TM_ADJ_K_CSR || KMODE == TM_ADJ_K_OUTER) {
            double W[B][B];
#pragma unroll
            for (int p = 0; p < B; ++p)
#pragma unroll
                for (int q = 0; q < B; ++q) {
                    if constexpr (KMODE == TM_ADJ_K_CSR)
                        W[p][q] = ldg(wcsr + a.slot_map[(e * B + p) * B + q]);
                    else
                        W[p][q] = -ldg(lam + c[p]) * ldg(u + c[q]);
                }
            double S[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) S[r][k] = W[r + 1][k + 1] - W[r + 1][0] - W[0][k + 1] + W[0][0];
            double Ps[D][D], MS[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    double s = 0.0;
#pragma unroll
                    for (int m = 0; m < D; ++m) s += M[r][m] * 0.5 * (S[m][k] + S[k][m]);
                    MS[r][k] = s;
                }
            double tr = 0.0;
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    double s = 0.0;
#pragma unroll
                    for (int m = 0; m < D; ++m) s += MS[r][m] * M[k][m];
                    Ps[r][k] = s;
                    if (r == k) tr += s;
                }
            const double kv = (kap ? ldg(kap + e) : 1.0) * a.kappa_scale;
            const double base = wsum * adet;
            if (gkap) gkap[e] = base * tr * a.kappa_scale;
            const double f = kv * base;
            // GJ += f M^T (tr I - 2 P)
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    double s = 0.0;
#pragma unroll
                    for (int m = 0; m < D; ++m) s += M[m][r] * ((m == k ? tr : 0.0) - 2.0 * Ps[m][k]);
                    GJ[r][k] += f * s;
                }
        }
        if constexpr (LOAD != TM_ADJ_LOAD_NONE) {
            double lb = 0.0;
#pragma unroll
            for (int p = 0; p < B; ++p) {
                double beta;
                if constexpr (LOAD == TM_ADJ_LOAD_CONST) {
                    beta = a.load_const * tab[TL.lhat + p];
                } else {
                    beta = 0.0;
#pragma unroll
                    for (int q = 0; q < B; ++q) beta += tab[TL.mhat + p * B + q] * ldg(fval + c[q]);
                }
                lb += ldg(lam + c[p]) * adet * beta;
            }
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) GJ[r][k] += lb * M[k][r];
        }
        double* lv = LV + (size_t)el * B * D;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            double s = 0.0;
#pragma unroll
            for (int r = 0; r < D; ++r) {
                lv[(r + 1) * D + k] = GJ[r][k];
                s += GJ[r][k];
            }
            lv[k] = -s;
        }
    }
    __syncthreads();
    if (a.grad_points) node_reduce<double, D>(P, LV, static_cast<double*>(a.grad_points), a.workspace);
}

inline int adj_status(const char* what);

// The same derivatives on elements whose Jacobian varies (P2 triangles and
// tetrahedra, quadrilaterals), per quadrature point: with M = J_q^-1 and the
// reference gradients dphi(q) [D x B], a diffusion weight W gives S =
// dphi sym(W) dphi^T, P = M S M^T and dL/dJ_q = kappa w_q |det J_q| M^T
// (tr(P) I - 2 P), dL/dkappa = sum_q w_q |det J_q| tr(P); a mass weight gives
// dL/dJ_q = s w_q |det J_q| (sum_ab W_ab phi_a(q) phi_b(q)) M^T; a load term
// L = lam . b, b_a = sum_q w_q |det J_q| phi_a(q) f(q) (f constant or the
// nodal source interpolated) adds w_q |det J_q| (sum_a lam_a phi_a(q)) f(q)
// M^T.  Node c of the element receives sum_q sum_r dL/dJ_q[r][d]
// dphi(q)[r][c].  KIND: the weights' form (kGenDiff, kGenMass or kGenNone).
enum { kGenDiff = 0, kGenMass = 1, kGenNone = 2 };
template <int ET, int KIND>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint_gen(const tm_adjoint_args a) {
    constexpr bool MASS = KIND == kGenMass;
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const TableLayout TL = table_layout(Q, B, D);
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm);
    double* LV = reinterpret_cast<double*>(sm + align16(sizeof(double) * TL.total));
    for (int k = threadIdx.x; k < TL.total; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();
    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const double* pts = static_cast<const double*>(a.points);
    const double* kap = static_cast<const double*>(a.kappa);
    const double* wcsr = static_cast<const double*>(a.weights);
    double* gkap = static_cast<double*>(a.grad_kappa);
    const double* lam = static_cast<const double*>(a.lam);
    const double* fnod = static_cast<const double*>(a.load_values);
    const int lsrc = a.load_source;
    for (int el = threadIdx.x; el < ne; el += blockDim.x) {
        const int64_t i = i0 + el;
        const int64_t e = P.elem_perm[i];
        double X[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int64_t node = P.conn[i * B + b];
#pragma unroll
            for (int d = 0; d < D; ++d) X[b][d] = ldg(pts + node * D + d);
        }
        const int64_t* slot = KIND == kGenNone ? nullptr : a.slot_map + e * B * B;
        const double kv = (!MASS && kap ? ldg(kap + e) : 1.0) * a.kappa_scale;
        double lv[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int d = 0; d < D; ++d) lv[b][d] = 0.0;
        double gk = 0.0;
        for (int q = 0; q < Q; ++q) {
            const double* dp = tab + TL.dphi + q * D * B;
            double J[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double t = 0.0;
#pragma unroll
                    for (int b = 0; b < B; ++b) t += dp[r * B + b] * X[b][d];
                    J[r][d] = t;
                }
            double cof[D][D];
            const double det = cofactors<double>(J, cof);
            const double inv = 1.0 / det, adet = fabs(det);
            double M[D][D];                   // M = J^-1, M[k][r] = cof[r][k] / det
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) M[k][r] = cof[r][k] * inv;
            const double wq = tab[TL.w + q];
            double GJ[D][D];
            if constexpr (KIND == kGenNone) {
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) GJ[r][k] = 0.0;
            } else if constexpr (MASS) {
                const double* ph = tab + TL.phi + q * B;
                double wm = 0.0;
                for (int pa = 0; pa < B; ++pa)
#pragma unroll
                    for (int pb = 0; pb < B; ++pb) wm += ldg(wcsr + slot[pa * B + pb]) * ph[pa] * ph[pb];
                const double f = kv * wq * adet * wm;
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) GJ[r][k] = f * M[k][r];
            } else {
                double S[D][D];
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) S[r][k] = 0.0;
                for (int pa = 0; pa < B; ++pa)
#pragma unroll
                    for (int pb = 0; pb < B; ++pb) {
                        const double w = 0.5 * (ldg(wcsr + slot[pa * B + pb]) + ldg(wcsr + slot[pb * B + pa]));
#pragma unroll
                        for (int r = 0; r < D; ++r)
#pragma unroll
                            for (int k = 0; k < D; ++k) S[r][k] += w * dp[r * B + pa] * dp[k * B + pb];
                    }
                double MS[D][D], Pm[D][D];
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        double t = 0.0;
#pragma unroll
                        for (int m = 0; m < D; ++m) t += M[r][m] * S[m][k];
                        MS[r][k] = t;
                    }
                double tr = 0.0;
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        double t = 0.0;
#pragma unroll
                        for (int m = 0; m < D; ++m) t += MS[r][m] * M[k][m];
                        Pm[r][k] = t;
                        if (r == k) tr += t;
                    }
                gk += wq * adet * tr;
                const double f = kv * wq * adet;
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        double t = 0.0;
#pragma unroll
                        for (int m = 0; m < D; ++m) t += M[m][r] * ((m == k ? tr : 0.0) - 2.0 * Pm[m][k]);
                        GJ[r][k] = f * t;
                    }
            }
            if (lsrc != TM_ADJ_LOAD_NONE) {
                const double* ph = tab + TL.phi + q * B;
                double lq = 0.0, fq = lsrc == TM_ADJ_LOAD_CONST ? a.load_const
                                    : lsrc == TM_ADJ_LOAD_QUAD ? ldg(fnod + e * Q + q) : 0.0;
#pragma unroll
                for (int b = 0; b < B; ++b) {
                    const int64_t node = P.conn[i * B + b];
                    lq += ph[b] * ldg(lam + node);
                    if (lsrc == TM_ADJ_LOAD_NODAL) fq += ph[b] * ldg(fnod + node);
                }
                const double f = wq * adet * lq * fq;
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int k = 0; k < D; ++k) GJ[r][k] += f * M[k][r];
            }
#pragma unroll
            for (int c = 0; c < B; ++c)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double t = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r) t += GJ[r][d] * dp[r * B + c];
                    lv[c][d] += t;
                }
        }
        if (gkap) gkap[e] = KIND == kGenDiff ? gk * a.kappa_scale : 0.0;
        double* out = LV + (size_t)el * B * D;
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int d = 0; d < D; ++d) out[b * D + d] = lv[b][d];
    }
    __syncthreads();
    if (a.grad_points) node_reduce<double, D>(P, LV, static_cast<double*>(a.grad_points), a.workspace);
}

// Elasticity (weights W = dL/dvalues as [nnz, D, D] blocks, E per element
// in kappa, the Poisson ratio in a.poisson): per quadrature point, with g =
// M dphi, L_q = w_q |det J| F(M), F = E sum_ab (lam' g_a^T W_ab g_b + mu'
// (g_b^T W_ab g_a + tr(W_ab) g_a . g_b)); dL/dJ_q = w_q |det J| (F M^T -
// M^T G M^T) with G = dF/dM = E sum_ab (lam' ((W_ab g_b) d_a^T + (W_ab^T
// g_a) d_b^T) + mu' ((W_ab g_a) d_b^T + (W_ab^T g_b) d_a^T + tr(W_ab)
// (g_b d_a^T + g_a d_b^T))), d_a = dphi(q)[:, a].
template <int ET>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint_elast(const tm_adjoint_args a) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const TableLayout TL = table_layout(Q, B, D);
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm);
    double* LV = reinterpret_cast<double*>(sm + align16(sizeof(double) * TL.total));
    for (int k = threadIdx.x; k < TL.total; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();
    const double nu = a.poisson;
    const double clam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), cmu = 1.0 / (2.0 * (1.0 + nu));
    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const double* pts = static_cast<const double*>(a.points);
    const double* Ey = static_cast<const double*>(a.kappa);
    const double* wb = static_cast<const double*>(a.weights);
    for (int el = threadIdx.x; el < ne; el += blockDim.x) {
        const int64_t i = i0 + el;
        const int64_t e = P.elem_perm[i];
        const int64_t* slot = a.slot_map + e * B * B;
        const double E = (Ey ? ldg(Ey + e) : 1.0) * a.kappa_scale;
        double* lv = LV + (size_t)el * B * D;
        for (int k = 0; k < B * D; ++k) lv[k] = 0.0;
        for (int q = 0; q < Q; ++q) {
            const double* dp = tab + TL.dphi + q * D * B;
            double J[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double t = 0.0;
                    for (int b = 0; b < B; ++b) t += dp[r * B + b] * ldg(pts + (int64_t)P.conn[i * B + b] * D + d);
                    J[r][d] = t;
                }
            double cof[D][D];
            const double det = cofactors<double>(J, cof);
            const double inv = 1.0 / det, adet = fabs(det);
            double M[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) M[k][r] = cof[r][k] * inv;
            double F = 0.0, G[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k < D; ++k) G[r][k] = 0.0;
            for (int pa = 0; pa < B; ++pa) {
                double da[D], ga[D];
#pragma unroll
                for (int r = 0; r < D; ++r) da[r] = dp[r * B + pa];
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    double t = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r) t += M[c][r] * da[r];
                    ga[c] = t;
                }
                for (int pb = 0; pb < B; ++pb) {
                    double db[D], gb[D];
#pragma unroll
                    for (int r = 0; r < D; ++r) db[r] = dp[r * B + pb];
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        double t = 0.0;
#pragma unroll
                        for (int r = 0; r < D; ++r) t += M[c][r] * db[r];
                        gb[c] = t;
                    }
                    const double* w = wb + slot[pa * B + pb] * (D * D);
                    double W[D][D], tw = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = 0; c < D; ++c) {
                            W[r][c] = ldg(w + r * D + c);
                            if (r == c) tw += W[r][c];
                        }
                    double h1[D], h2[D], h3[D], h4[D], gg = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r) {
                        h1[r] = h2[r] = h3[r] = h4[r] = 0.0;
                        gg += ga[r] * gb[r];
#pragma unroll
                        for (int c = 0; c < D; ++c) {
                            h1[r] += W[r][c] * gb[c];      // W g_b
                            h2[r] += W[c][r] * ga[c];      // W^T g_a
                            h3[r] += W[r][c] * ga[c];      // W g_a
                            h4[r] += W[c][r] * gb[c];      // W^T g_b
                        }
                    }
                    double f1 = 0.0, f2 = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r) {
                        f1 += ga[r] * h1[r];
                        f2 += gb[r] * h3[r];
                    }
                    F += clam * f1 + cmu * (f2 + tw * gg);
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = 0; c < D; ++c)
                            G[r][c] += clam * (h1[r] * da[c] + h2[r] * db[c]) +
                                       cmu * (h3[r] * db[c] + h4[r] * da[c] + tw * (gb[r] * da[c] + ga[r] * db[c]));
                }
            }
            // dL/dJ = w |det| E (F M^T - M^T G M^T)
            const double f = tab[TL.w + q] * adet * E;
            double GM[D][D];                  // G M^T
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    double t = 0.0;
#pragma unroll
                    for (int m = 0; m < D; ++m) t += G[r][m] * M[c][m];
                    GM[r][c] = t;
                }
            double GJ[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    double t = 0.0;
#pragma unroll
                    for (int m = 0; m < D; ++m) t += M[m][r] * GM[m][c];
                    GJ[r][c] = f * (F * M[c][r] - t);
                }
            for (int b = 0; b < B; ++b)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double t = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r) t += GJ[r][d] * dp[r * B + b];
                    lv[b * D + d] += t;
                }
        }
    }
    __syncthreads();
    if (a.grad_points) node_reduce<double, D>(P, LV, static_cast<double*>(a.grad_points), a.workspace);
}

template <int ET>
int run_adjoint_elast(const tm_adjoint_args& a, cudaStream_t st) {
    using T = Traits<ET>;
    const TableLayout TL = table_layout(a.tables.n_quad, T::B, T::D);
    const size_t smem = align16(sizeof(double) * TL.total) + sizeof(double) * (size_t)a.plan.chunk_elems * T::B * T::D;
    if (smem > 227 * 1024) return tm_set_error(TM_ERR_TOO_LARGE, "tm_adjoint_general: chunk too large for shared memory");
    if (!a.grad_points) return TM_OK;
    if (cudaMemsetAsync(a.grad_points, 0, sizeof(double) * (size_t)a.n_points * T::D, st) != cudaSuccess)
        return adj_status("cudaMemsetAsync");
    if (a.plan.n_shared > 0) {
        void* counters = static_cast<unsigned char*>(a.workspace) + node_counters_offset<double>(a.plan, T::D);
        if (cudaMemsetAsync(counters, 0, sizeof(int32_t) * (size_t)a.plan.n_shared, st) != cudaSuccess)
            return adj_status("cudaMemsetAsync");
    }
    if (a.plan.n_chunks == 0) return TM_OK;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_adjoint_elast<ET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return adj_status("cudaFuncSetAttribute");
    k_adjoint_elast<ET><<<a.plan.n_chunks, kAdjThreads, smem, st>>>(a);
    return adj_status("k_adjoint_elast");
}

template <int ET, int KIND>
int run_adjoint_gen(const tm_adjoint_args& a, cudaStream_t st) {
    using T = Traits<ET>;
    const TableLayout TL = table_layout(a.tables.n_quad, T::B, T::D);
    const size_t smem = align16(sizeof(double) * TL.total) + sizeof(double) * (size_t)a.plan.chunk_elems * T::B * T::D;
    if (smem > 227 * 1024) return tm_set_error(TM_ERR_TOO_LARGE, "tm_adjoint_general: chunk too large for shared memory");
    if (a.grad_points) {
        if (cudaMemsetAsync(a.grad_points, 0, sizeof(double) * (size_t)a.n_points * T::D, st) != cudaSuccess)
            return adj_status("cudaMemsetAsync");
        if (a.plan.n_shared > 0) {
            void* counters = static_cast<unsigned char*>(a.workspace) + node_counters_offset<double>(a.plan, T::D);
            if (cudaMemsetAsync(counters, 0, sizeof(int32_t) * (size_t)a.plan.n_shared, st) != cudaSuccess)
                return adj_status("cudaMemsetAsync");
        }
    }
    if (a.plan.n_chunks == 0) return TM_OK;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_adjoint_gen<ET, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return adj_status("cudaFuncSetAttribute");
    k_adjoint_gen<ET, KIND><<<a.plan.n_chunks, kAdjThreads, smem, st>>>(a);
    return adj_status("k_adjoint_gen");
}

template <int ET>
int dispatch_gen(const tm_adjoint_args& a, cudaStream_t st) {
    if (a.plan.n_basis != Traits<ET>::B)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: node plan of another element type");
    if (a.k_mode == TM_ADJ_E_CSR) return run_adjoint_elast<ET>(a, st);
    if (a.k_mode == TM_ADJ_K_NONE) return run_adjoint_gen<ET, kGenNone>(a, st);
    return a.k_mode == TM_ADJ_M_CSR ? run_adjoint_gen<ET, kGenMass>(a, st) : run_adjoint_gen<ET, kGenDiff>(a, st);
}

inline int adj_status(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

template <int ET, int KMODE, int LOAD>
int run_adjoint(const tm_adjoint_args& a, cudaStream_t st) {
    using T = Traits<ET>;
    const TableLayout TL = table_layout(a.tables.n_quad, T::B, T::D);
    const size_t smem = align16(sizeof(double) * TL.total) + sizeof(double) * (size_t)a.plan.chunk_elems * T::B * T::D;
    if (smem > 227 * 1024) return tm_set_error(TM_ERR_TOO_LARGE, "tm_adjoint_p1: chunk too large for shared memory");
    if (a.grad_points) {
        if (cudaMemsetAsync(a.grad_points, 0, sizeof(double) * (size_t)a.n_points * T::D, st) != cudaSuccess)
            return adj_status("cudaMemsetAsync");
        if (a.plan.n_shared > 0) {
            void* counters = static_cast<unsigned char*>(a.workspace) + node_counters_offset<double>(a.plan, T::D);
            if (cudaMemsetAsync(counters, 0, sizeof(int32_t) * (size_t)a.plan.n_shared, st) != cudaSuccess)
                return adj_status("cudaMemsetAsync");
        }
    }
    if (a.plan.n_chunks == 0) return TM_OK;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_adjoint<ET, KMODE, LOAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return adj_status("cudaFuncSetAttribute");
    k_adjoint<ET, KMODE, LOAD><<<a.plan.n_chunks, kAdjThreads, smem, st>>>(a);
    return adj_status("k_adjoint");
}

template <int ET, int KMODE>
int dispatch_load(const tm_adjoint_args& a, cudaStream_t st) {
    switch (a.load_source) {
        case TM_ADJ_LOAD_NONE: return run_adjoint<ET, KMODE, TM_ADJ_LOAD_NONE>(a, st);
        case TM_ADJ_LOAD_CONST: return run_adjoint<ET, KMODE, TM_ADJ_LOAD_CONST>(a, st);
        case TM_ADJ_LOAD_NODAL: return run_adjoint<ET, KMODE, TM_ADJ_LOAD_NODAL>(a, st);
        default: return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: unknown load source");
    }
}

template <int ET>
int dispatch_kmode(const tm_adjoint_args& a, cudaStream_t st) {
    switch (a.k_mode) {
        case TM_ADJ_K_NONE: return dispatch_load<ET, TM_ADJ_K_NONE>(a, st);
        case TM_ADJ_K_CSR: return dispatch_load<ET, TM_ADJ_K_CSR>(a, st);
        case TM_ADJ_K_OUTER: return dispatch_load<ET, TM_ADJ_K_OUTER>(a, st);
        case TM_ADJ_M_CSR: return dispatch_load<ET, TM_ADJ_M_CSR>(a, st);
        default: return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: unknown k_mode");
    }
}

}  // namespace tmk

using namespace tmk;

extern "C" size_t tm_adjoint_workspace_bytes(const tm_adjoint_args* a) {
    if (!a) return 0;
    const int et = a->tables.element_type;
    const int D = (et == TM_TET4 || et == TM_TET10) ? 3 : 2;
    return node_counters_offset<double>(a->plan, D) + sizeof(int32_t) * (size_t)a->plan.n_shared;
}

extern "C" int tm_adjoint_p1(const tm_adjoint_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: null args");
    if (a->dtype != TM_F64) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_adjoint_p1: float64 only");
    const int et = a->tables.element_type;
    if (et != TM_TRI3 && et != TM_TET4)
        return tm_set_error(TM_ERR_UNSUPPORTED, "tm_adjoint_p1: P1 triangles and tetrahedra only");
    const int B = et == TM_TRI3 ? 3 : 4;
    if (a->plan.n_basis != B || a->plan.n_local != B)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: expects a node plan of the mesh");
    if (!a->tables.packed || (a->plan.n_elements > 0 && !a->points))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: null tables or points");
    if ((a->k_mode == TM_ADJ_K_CSR || a->k_mode == TM_ADJ_M_CSR) && (!a->weights || !a->slot_map))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: CSR weights need weights and slot_map");
    if (a->k_mode == TM_ADJ_K_OUTER && (!a->u || !a->lam))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: outer-product weights need u and lam");
    if (a->load_source != TM_ADJ_LOAD_NONE && !a->lam)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: the load term needs lam");
    if (a->load_source == TM_ADJ_LOAD_NODAL && !a->load_values)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: nodal load needs load_values");
    if (a->load_source == TM_ADJ_LOAD_QUAD)
        return tm_set_error(TM_ERR_UNSUPPORTED, "tm_adjoint_p1: quadrature-point loads go to tm_adjoint_general");
    if (a->grad_points && a->plan.n_shared > 0 && !a->workspace)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_p1: workspace is null");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return et == TM_TRI3 ? dispatch_kmode<TM_TRI3>(*a, st) : dispatch_kmode<TM_TET4>(*a, st);
}

extern "C" int tm_adjoint_general(const tm_adjoint_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: null args");
    if (a->dtype != TM_F64) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_adjoint_general: float64 only");
    if (a->k_mode != TM_ADJ_K_NONE && a->k_mode != TM_ADJ_K_CSR && a->k_mode != TM_ADJ_M_CSR &&
        a->k_mode != TM_ADJ_E_CSR)
        return tm_set_error(TM_ERR_UNSUPPORTED,
                            "tm_adjoint_general: k_mode TM_ADJ_K_NONE, TM_ADJ_K_CSR, TM_ADJ_M_CSR or TM_ADJ_E_CSR");
    if (a->k_mode == TM_ADJ_E_CSR && !(a->poisson > -1.0 && a->poisson < 0.5))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: Poisson ratio outside (-1, 0.5)");
    if (a->load_source != TM_ADJ_LOAD_NONE && a->load_source != TM_ADJ_LOAD_CONST &&
        a->load_source != TM_ADJ_LOAD_NODAL && a->load_source != TM_ADJ_LOAD_QUAD)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: unknown load source");
    if (a->load_source != TM_ADJ_LOAD_NONE && a->k_mode == TM_ADJ_E_CSR)
        return tm_set_error(TM_ERR_UNSUPPORTED, "tm_adjoint_general: no load term with elasticity weights");
    if (a->load_source != TM_ADJ_LOAD_NONE && a->plan.n_elements > 0 &&
        (!a->lam || ((a->load_source == TM_ADJ_LOAD_NODAL || a->load_source == TM_ADJ_LOAD_QUAD) &&
                     !a->load_values)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: a load term needs lam (and load_values)");
    if (a->k_mode != TM_ADJ_K_NONE && (!a->weights || !a->slot_map))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: null weights or slot map");
    if (!a->tables.packed || (a->plan.n_elements > 0 && !a->points))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: null tables or points");
    if (a->grad_points && a->plan.n_shared > 0 && !a->workspace)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_adjoint_general: workspace is null");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    switch (a->tables.element_type) {
        case TM_TRI3: return dispatch_gen<TM_TRI3>(*a, st);
        case TM_TET4: return dispatch_gen<TM_TET4>(*a, st);
        case TM_TRI6: return dispatch_gen<TM_TRI6>(*a, st);
        case TM_TET10: return dispatch_gen<TM_TET10>(*a, st);
        case TM_QUAD4: return dispatch_gen<TM_QUAD4>(*a, st);
        case TM_QUAD9: return dispatch_gen<TM_QUAD9>(*a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_adjoint_general: unknown element type");
    }
}
