// Gradient of a diffusion or isotropic linear-elasticity matrix with respect
// to its per-element coefficient (float64, any element type).
//
// Diffusion: K_e = kappa_e sum_q jw_q g_a . g_b, so for weights W =
// dL/dvalues ([nnz]) dL/dkappa_e = s sum_{a,b} W[slot(e,a,b)] sum_q jw_q
// g_a . g_b.
//
// The reference differentiates its elasticity assembly with autograd through
// the vmap'd integrand B_a^T C B_b (functional/elasticity.py:132-284,
// assemble/element_assembler.py:390-445); C is linear in E, so for weights
// W = dL/dvalues ([nnz, D, D] blocks) the derivative with respect to the
// modulus of element e is the contraction of W with the element's blocks at
// unit modulus:
//     dL/dE_e = s sum_{a,b} W[slot(e,a,b)] : K_e[a][b](E = 1),
//     K_e[a][b](1) = sum_q jw_q (lam' g_a g_b^T + mu' (g_b g_a^T + (g_a . g_b) I)),
// with lam' = nu / ((1 + nu)(1 - 2 nu)), mu' = 1 / (2 (1 + nu)) and s the
// modulus scale of the call, that is, per quadrature point
//     jw_q (lam' g_a^T W g_b + mu' (g_b^T W g_a + tr(W) g_a . g_b)).
// With flags TM_COEF_GRAD_LAME_PARTS the two parts come back apart, grad[e] =
// s sum jw_q g_a^T W g_b (unit lam) and grad[E + e] = s sum jw_q (g_b^T W
// g_a + tr(W) g_a . g_b) (unit mu), for the derivative with respect to the
// Poisson ratio through lam'(nu) and mu'(nu).
// One CTA per chunk of the plan, in sub-batches of 32 elements: one thread
// per (element, quadrature point) computes the Jacobian, its cofactors and
// the gradients into shared memory; four threads per element then take its
// B x B (a, b) pairs in a fixed interleave, and the element's four partial
// sums are added in a fixed order (deterministic).
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/tensormesh_gb300.h"
#include "tm_element.cuh"
#include "tm_reduce.cuh"
#include "tm_status.h"

namespace tmk {

constexpr int kEgThreads = 128;
constexpr int kEgSub = 32;                      // elements per sub-batch
constexpr int kEgPer = kEgThreads / kEgSub;     // threads per element in the pair phase

template <int ET>
__host__ __device__ inline size_t eg_smem(int Q) {
    using T = Traits<ET>;
    const TableLayout TL = table_layout(Q, T::B, T::D);
    return align16(sizeof(double) * TL.total) + sizeof(double) * (size_t)kEgSub * Q * (T::B * T::D + 1) +
           2 * sizeof(double) * kEgSub * kEgPer;
}

template <int ET, bool ELAST>
__global__ void __launch_bounds__(kEgThreads) k_coef_grad(const tm_coef_grad_args a) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const TableLayout TL = table_layout(Q, B, D);
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm);
    double* G = reinterpret_cast<double*>(sm + align16(sizeof(double) * TL.total));   // [sub][Q][B][D]
    double* JW = G + (size_t)kEgSub * Q * B * D;                                        // [sub][Q]
    double* part = JW + kEgSub * Q;                                                     // [sub][kEgPer]
    for (int k = threadIdx.x; k < TL.total; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();
    const double nu = a.poisson;
    const double clam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), cmu = 1.0 / (2.0 * (1.0 + nu));
    const bool split = ELAST && (a.flags & TM_COEF_GRAD_LAME_PARTS) != 0;
    const double* pts = static_cast<const double*>(a.points);
    const double* W = static_cast<const double*>(a.weights);
    double* gE = static_cast<double*>(a.grad);
    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    for (int s0 = 0; s0 < ne; s0 += kEgSub) {
        const int ns = min(kEgSub, ne - s0);
        // geometry: one thread per (element, quadrature point)
        for (int k = threadIdx.x; k < ns * Q; k += blockDim.x) {
            const int el = k / Q, q = k - el * Q;
            const int64_t i = i0 + s0 + el;
            double X[B][D];
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int64_t node = P.conn[i * B + b];
#pragma unroll
                for (int d = 0; d < D; ++d) X[b][d] = pts[node * D + d];
            }
            const double* dp = tab + TL.dphi + q * D * B;
            double J[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    double s = 0.0;
#pragma unroll
                    for (int b = 0; b < B; ++b) s += dp[r * B + b] * X[b][c];
                    J[r][c] = s;
                }
            double cof[D][D];
            const double det = cofactors<double>(J, cof);
            const double inv = 1.0 / det;
            double* g = G + ((size_t)el * Q + q) * B * D;
#pragma unroll
            for (int b = 0; b < B; ++b)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    double s = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r) s += dp[r * B + b] * cof[r][c];
                    g[b * D + c] = s * inv;
                }
            JW[el * Q + q] = tab[TL.w + q] * fabs(det);
        }
        __syncthreads();
        // pairs: kEgPer threads per element, pair p = t, t + kEgPer, ...
        {
            const int el = threadIdx.x / kEgPer, t = threadIdx.x - el * kEgPer;
            double acc = 0.0, acc_mu = 0.0;     // (acc_mu: the unit-mu part when split)
            if (el < ns) {
                const int64_t e = P.elem_perm[i0 + s0 + el];
                const double* ge = G + (size_t)el * Q * B * D;
                for (int p = t; p < B * B; p += kEgPer) {
                    const int pa = p / B, pb = p - pa * B;
                    if constexpr (!ELAST) {
                        const double w = W[a.slot_map[(e * B + pa) * B + pb]];
                        double s = 0.0;
                        for (int q = 0; q < Q; ++q) {
                            const double* gq = ge + (size_t)q * B * D;
                            double dd = 0.0;
#pragma unroll
                            for (int r = 0; r < D; ++r) dd += gq[pa * D + r] * gq[pb * D + r];
                            s += JW[el * Q + q] * dd;
                        }
                        acc += w * s;
                        continue;
                    }
                    const double* w = W + a.slot_map[(e * B + pa) * B + pb] * (D * D);
                    double Wm[D][D];
                    double trw = 0.0;
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = 0; c < D; ++c) {
                            Wm[r][c] = w[r * D + c];
                            if (r == c) trw += Wm[r][c];
                        }
                    for (int q = 0; q < Q; ++q) {
                        const double* gq = ge + (size_t)q * B * D;
                        const double* ga = gq + pa * D;
                        const double* gb = gq + pb * D;
                        double s1 = 0.0, s2 = 0.0, dd = 0.0;
#pragma unroll
                        for (int r = 0; r < D; ++r) {
                            dd += ga[r] * gb[r];
#pragma unroll
                            for (int c = 0; c < D; ++c) {
                                s1 += ga[r] * Wm[r][c] * gb[c];
                                s2 += gb[r] * Wm[r][c] * ga[c];
                            }
                        }
                        if (split) {
                            acc += JW[el * Q + q] * s1;
                            acc_mu += JW[el * Q + q] * (s2 + trw * dd);
                        } else {
                            acc += JW[el * Q + q] * (clam * s1 + cmu * (s2 + trw * dd));
                        }
                    }
                }
            }
            part[el * kEgPer + t] = acc;
            part[kEgSub * kEgPer + el * kEgPer + t] = acc_mu;
        }
        __syncthreads();
        if (threadIdx.x < ns) {
            const int el = threadIdx.x;
            double s = 0.0, sm = 0.0;
#pragma unroll
            for (int t = 0; t < kEgPer; ++t) {
                s += part[el * kEgPer + t];
                sm += part[kEgSub * kEgPer + el * kEgPer + t];
            }
            const int64_t e = P.elem_perm[i0 + s0 + el];
            gE[e] = a.scale * s;
            if (split) gE[P.n_elements + e] = a.scale * sm;
        }
        __syncthreads();
    }
}

inline int eg_status(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

template <int ET, bool ELAST>
int run_coef_grad_form(const tm_coef_grad_args& a, cudaStream_t st) {
    const size_t smem = eg_smem<ET>(a.tables.n_quad);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_coef_grad<ET, ELAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return eg_status("cudaFuncSetAttribute");
    k_coef_grad<ET, ELAST><<<a.plan.n_chunks, kEgThreads, smem, st>>>(a);
    return eg_status("k_coef_grad");
}

template <int ET>
int run_coef_grad(const tm_coef_grad_args& a, cudaStream_t st) {
    using T = Traits<ET>;
    if (a.plan.n_basis != T::B) return tm_set_error(TM_ERR_INVALID_ARG, "tm_coef_grad: plan of another element type");
    if (eg_smem<ET>(a.tables.n_quad) > 227 * 1024)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_coef_grad: too many quadrature points");
    if (a.plan.n_chunks == 0) return TM_OK;
    return a.form == TM_FORM_ELASTICITY ? run_coef_grad_form<ET, true>(a, st) : run_coef_grad_form<ET, false>(a, st);
}

}  // namespace tmk

using namespace tmk;

extern "C" int tm_coef_grad(const tm_coef_grad_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_coef_grad: null args");
    if (a->form != TM_FORM_ELASTICITY && a->form != TM_FORM_DIFFUSION)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_coef_grad: form must be TM_FORM_DIFFUSION or TM_FORM_ELASTICITY");
    if (a->plan.n_elements > 0 && (!a->points || !a->weights || !a->slot_map || !a->grad ||
                                   !a->tables.packed || !a->plan.conn || !a->plan.elem_perm))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_coef_grad: null pointer");
    if (a->form == TM_FORM_ELASTICITY && !(a->poisson > -1.0 && a->poisson < 0.5))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_coef_grad: Poisson ratio outside (-1, 0.5)");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    switch (a->tables.element_type) {
        case TM_TRI3: return run_coef_grad<TM_TRI3>(*a, st);
        case TM_TET4: return run_coef_grad<TM_TET4>(*a, st);
        case TM_TRI6: return run_coef_grad<TM_TRI6>(*a, st);
        case TM_TET10: return run_coef_grad<TM_TET10>(*a, st);
        case TM_QUAD4: return run_coef_grad<TM_QUAD4>(*a, st);
        case TM_QUAD9: return run_coef_grad<TM_QUAD9>(*a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_coef_grad: unknown element type");
    }
}
