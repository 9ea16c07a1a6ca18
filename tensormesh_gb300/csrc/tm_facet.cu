// Boundary-facet load vectors (FacetAssembler.__call__ for its load forms,
// assemble/facet_assembler.py:123-277).
//
// One CTA per chunk of facet items (selected (element, facet) pairs, given by
// the facet's own nodes).  Phase 1, one thread per item: for every facet
// quadrature point the map's Jacobian F = sum_b X_b (x) dpsi_b (D x (D-1)),
// the measure |F| = sqrt(det(F^T F)) (a length for lines, |c0 x c1| for
// triangles), the source value g at the point (constant, nodal values
// interpolated with psi, or given per point) and the item's local values
// w_q |F| g psi_a into shared memory.  Phase 2 is the deterministic node-plan
// reduction shared with the volume load vectors (tm_reduce.cuh).
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/tensormesh_gb300.h"
#include "tm_reduce.cuh"
#include "tm_status.h"

namespace tmk {
namespace {

constexpr int kFacetThreads = 256;

template <int FT>
struct FacetTraits;
template <>
struct FacetTraits<TM_FACET_LINE2> {
    static constexpr int FD = 1, B = 2;
};
template <>
struct FacetTraits<TM_FACET_LINE3> {
    static constexpr int FD = 1, B = 3;
};
template <>
struct FacetTraits<TM_FACET_TRI3> {
    static constexpr int FD = 2, B = 3;
};
template <>
struct FacetTraits<TM_FACET_TRI6> {
    static constexpr int FD = 2, B = 6;
};

struct FacetLayout {
    size_t tab, lv, total;
};
template <typename R, int FT, int W>
__host__ __device__ inline FacetLayout facet_layout(int CH, int Q) {
    using T = FacetTraits<FT>;
    FacetLayout L;
    L.tab = 0;
    L.lv = align16(sizeof(double) * (size_t)Q * (1 + T::B + T::FD * T::B));
    L.total = align16(L.lv + sizeof(R) * (size_t)CH * T::B * W);
    return L;
}

template <typename R, int FT, int SRC, int W>
__global__ void __launch_bounds__(kFacetThreads) k_facet_vector(const tm_facet_vector_args a) {
    using T = FacetTraits<FT>;
    constexpr int FD = T::FD, B = T::B, D = FD + 1;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const FacetLayout L = facet_layout<R, FT, W>(CH, Q);
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm + L.tab);
    R* LV = reinterpret_cast<R*>(sm + L.lv);
    const double* tw = tab;                   // [Q]
    const double* tpsi = tab + Q;             // [Q][B]
    const double* tdpsi = tab + Q + Q * B;    // [Q][FD][B]
    const int n_tab = Q * (1 + B + FD * B);
    for (int k = threadIdx.x; k < n_tab; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();

    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const R* pts = static_cast<const R*>(a.points);
    const R* val = static_cast<const R*>(a.values);
    for (int el = threadIdx.x; el < ne; el += blockDim.x) {
        const int64_t i = i0 + el;
        int64_t node[B];
        R X[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            node[b] = P.conn[i * B + b];
#pragma unroll
            for (int d = 0; d < D; ++d) X[b][d] = pts[node[b] * D + d];
        }
        R acc[B][W];
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int w = 0; w < W; ++w) acc[b][w] = 0;
        for (int q = 0; q < Q; ++q) {
            // F[:, c] = sum_b X_b dpsi_b / dt_c
            R F[FD][D];
#pragma unroll
            for (int c = 0; c < FD; ++c)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    R s = 0;
#pragma unroll
                    for (int b = 0; b < B; ++b) s += (R)tdpsi[(q * FD + c) * B + b] * X[b][d];
                    F[c][d] = s;
                }
            R m;
            if constexpr (FD == 1) {
                m = sqrt(F[0][0] * F[0][0] + F[0][1] * F[0][1]);
            } else {
                const R cx = F[0][1] * F[1][2] - F[0][2] * F[1][1];
                const R cy = F[0][2] * F[1][0] - F[0][0] * F[1][2];
                const R cz = F[0][0] * F[1][1] - F[0][1] * F[1][0];
                m = sqrt(cx * cx + cy * cy + cz * cz);
            }
            const R wm = (R)tw[q] * m;
            R g[W];
#pragma unroll
            for (int w = 0; w < W; ++w) {
                if constexpr (SRC == TM_SOURCE_CONST) {
                    g[w] = (R)a.const_value[w];
                } else if constexpr (SRC == TM_SOURCE_NODAL) {
                    R s = 0;
#pragma unroll
                    for (int b = 0; b < B; ++b) s += (R)tpsi[q * B + b] * val[node[b] * W + w];
                    g[w] = s;
                } else {
                    g[w] = val[((int64_t)P.elem_perm[i] * Q + q) * W + w];
                }
            }
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const R c = wm * (R)tpsi[q * B + b];
#pragma unroll
                for (int w = 0; w < W; ++w) acc[b][w] += c * g[w];
            }
        }
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int w = 0; w < W; ++w) LV[(el * B + b) * W + w] = acc[b][w];
    }
    __syncthreads();
    node_reduce<R, W>(P, LV, static_cast<R*>(a.out), a.workspace);
}

inline int status(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

template <typename R, int FT, int SRC, int W>
int run_facet(const tm_facet_vector_args& a, cudaStream_t st) {
    const FacetLayout L = facet_layout<R, FT, W>(a.plan.chunk_elems, a.tables.n_quad);
    if (L.total > 227 * 1024)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_assemble_facet_vector: chunk needs more than 227 KB of shared memory");
    if (cudaMemsetAsync(a.out, 0, sizeof(R) * a.n_points * W, st) != cudaSuccess) return status("cudaMemsetAsync");
    if (a.plan.n_chunks == 0) return TM_OK;
    if (a.plan.n_shared > 0) {
        void* counters = static_cast<unsigned char*>(a.workspace) + node_counters_offset<R>(a.plan, W);
        if (cudaMemsetAsync(counters, 0, sizeof(int32_t) * (size_t)a.plan.n_shared, st) != cudaSuccess)
            return status("cudaMemsetAsync");
    }
    if (L.total > 48 * 1024 &&
        cudaFuncSetAttribute(k_facet_vector<R, FT, SRC, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)L.total) != cudaSuccess)
        return status("cudaFuncSetAttribute");
    k_facet_vector<R, FT, SRC, W><<<a.plan.n_chunks, kFacetThreads, L.total, st>>>(a);
    return status("k_facet_vector");
}

template <typename R, int FT, int SRC>
int facet_width(const tm_facet_vector_args& a, cudaStream_t st) {
    switch (a.width) {
        case 1: return run_facet<R, FT, SRC, 1>(a, st);
        case 2: return run_facet<R, FT, SRC, 2>(a, st);
        case 3: return run_facet<R, FT, SRC, 3>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_facet_vector: width must be 1..3");
    }
}

template <typename R, int FT>
int facet_source(const tm_facet_vector_args& a, cudaStream_t st) {
    switch (a.source) {
        case TM_SOURCE_CONST: return facet_width<R, FT, TM_SOURCE_CONST>(a, st);
        case TM_SOURCE_NODAL: return facet_width<R, FT, TM_SOURCE_NODAL>(a, st);
        case TM_SOURCE_QUAD: return facet_width<R, FT, TM_SOURCE_QUAD>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_facet_vector: unknown source kind");
    }
}

template <typename R>
int facet_type(const tm_facet_vector_args& a, cudaStream_t st) {
    switch (a.tables.facet_type) {
        case TM_FACET_LINE2: return facet_source<R, TM_FACET_LINE2>(a, st);
        case TM_FACET_LINE3: return facet_source<R, TM_FACET_LINE3>(a, st);
        case TM_FACET_TRI3: return facet_source<R, TM_FACET_TRI3>(a, st);
        case TM_FACET_TRI6: return facet_source<R, TM_FACET_TRI6>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_facet_vector: unknown facet type");
    }
}

// The adjoint of the facet loads for L = sum_i lam_i . b_i (float64): per
// item and facet quadrature point, with s = sum_w lam_w(t_q) g_w(t_q) (lam
// interpolated with psi), L_q = w_q |F| s; d|F|/dF_0 = F_0 / |F| for lines,
// d|F|/dF_0 = (F_1 x c) / |F| and d|F|/dF_1 = (c x F_0) / |F| with c = F_0 x
// F_1 for triangles; node b of the item receives sum_c w_q s d|F|/dF_c
// dpsi_b/dt_c (node-plan reduction).  grad_values (a source given per
// point): w_q |F| lam_w(t_q) per (item, point, component), item order.
template <int FT, int SRC, int W>
__global__ void __launch_bounds__(kFacetThreads) k_facet_adjoint(const tm_facet_adjoint_args a) {
    using T = FacetTraits<FT>;
    constexpr int FD = T::FD, B = T::B, D = FD + 1;
    const tm_facet_vector_args& v = a.base;
    const tm_chunk_plan& P = v.plan;
    const int CH = P.chunk_elems, Q = v.tables.n_quad;
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm);
    double* LV = reinterpret_cast<double*>(sm + align16(sizeof(double) * (size_t)Q * (1 + B + FD * B)));
    const double* tw = tab;
    const double* tpsi = tab + Q;
    const double* tdpsi = tab + Q + Q * B;
    const int n_tab = Q * (1 + B + FD * B);
    for (int k = threadIdx.x; k < n_tab; k += blockDim.x) tab[k] = v.tables.packed[k];
    __syncthreads();
    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const double* pts = static_cast<const double*>(v.points);
    const double* val = static_cast<const double*>(v.values);
    const double* lam = static_cast<const double*>(a.lam);
    double* gq = static_cast<double*>(a.grad_values);
    for (int el = threadIdx.x; el < ne; el += blockDim.x) {
        const int64_t i = i0 + el;
        const int64_t item = P.elem_perm[i];
        int64_t node[B];
        double X[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            node[b] = P.conn[i * B + b];
#pragma unroll
            for (int d = 0; d < D; ++d) X[b][d] = pts[node[b] * D + d];
        }
        double lv[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int d = 0; d < D; ++d) lv[b][d] = 0.0;
        for (int q = 0; q < Q; ++q) {
            double F[FD][D];
#pragma unroll
            for (int c = 0; c < FD; ++c)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double t = 0.0;
#pragma unroll
                    for (int b = 0; b < B; ++b) t += tdpsi[(q * FD + c) * B + b] * X[b][d];
                    F[c][d] = t;
                }
            double m, dm[FD][D];
            if constexpr (FD == 1) {
                m = sqrt(F[0][0] * F[0][0] + F[0][1] * F[0][1]);
                dm[0][0] = F[0][0] / m;
                dm[0][1] = F[0][1] / m;
            } else {
                const double c[3] = {F[0][1] * F[1][2] - F[0][2] * F[1][1], F[0][2] * F[1][0] - F[0][0] * F[1][2],
                                     F[0][0] * F[1][1] - F[0][1] * F[1][0]};
                m = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
                const double im = 1.0 / m;
                // F_1 x c and c x F_0
                dm[0][0] = (F[1][1] * c[2] - F[1][2] * c[1]) * im;
                dm[0][1] = (F[1][2] * c[0] - F[1][0] * c[2]) * im;
                dm[0][2] = (F[1][0] * c[1] - F[1][1] * c[0]) * im;
                dm[1][0] = (c[1] * F[0][2] - c[2] * F[0][1]) * im;
                dm[1][1] = (c[2] * F[0][0] - c[0] * F[0][2]) * im;
                dm[1][2] = (c[0] * F[0][1] - c[1] * F[0][0]) * im;
            }
            double s = 0.0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double lw = 0.0, g = 0.0;
#pragma unroll
                for (int b = 0; b < B; ++b) lw += tpsi[q * B + b] * lam[node[b] * W + w];
                if constexpr (SRC == TM_SOURCE_CONST) {
                    g = v.const_value[w];
                } else if constexpr (SRC == TM_SOURCE_NODAL) {
#pragma unroll
                    for (int b = 0; b < B; ++b) g += tpsi[q * B + b] * val[node[b] * W + w];
                } else {
                    g = val[(item * Q + q) * W + w];
                }
                s += lw * g;
                if (gq) gq[(item * Q + q) * W + w] = tw[q] * m * lw;
            }
            const double f = tw[q] * s;
#pragma unroll
            for (int b = 0; b < B; ++b)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double t = 0.0;
#pragma unroll
                    for (int c = 0; c < FD; ++c) t += dm[c][d] * tdpsi[(q * FD + c) * B + b];
                    lv[b][d] += f * t;
                }
        }
        double* out = LV + (size_t)el * B * D;
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int d = 0; d < D; ++d) out[b * D + d] = lv[b][d];
    }
    __syncthreads();
    if (a.grad_points) node_reduce<double, D>(P, LV, static_cast<double*>(a.grad_points), v.workspace);
}

template <int FT, int SRC, int W>
int run_facet_adjoint(const tm_facet_adjoint_args& a, cudaStream_t st) {
    using T = FacetTraits<FT>;
    constexpr int D = T::FD + 1;
    const tm_facet_vector_args& v = a.base;
    const size_t smem = align16(sizeof(double) * (size_t)v.tables.n_quad * (1 + T::B + T::FD * T::B)) +
                        sizeof(double) * (size_t)v.plan.chunk_elems * T::B * D;
    if (smem > 227 * 1024) return tm_set_error(TM_ERR_TOO_LARGE, "tm_facet_adjoint: chunk too large");
    if (a.grad_points) {
        if (cudaMemsetAsync(a.grad_points, 0, sizeof(double) * (size_t)v.n_points * D, st) != cudaSuccess)
            return status("cudaMemsetAsync");
        if (v.plan.n_shared > 0) {
            void* counters = static_cast<unsigned char*>(v.workspace) + node_counters_offset<double>(v.plan, D);
            if (cudaMemsetAsync(counters, 0, sizeof(int32_t) * (size_t)v.plan.n_shared, st) != cudaSuccess)
                return status("cudaMemsetAsync");
        }
    }
    if (v.plan.n_chunks == 0) return TM_OK;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_facet_adjoint<FT, SRC, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return status("cudaFuncSetAttribute");
    k_facet_adjoint<FT, SRC, W><<<v.plan.n_chunks, kFacetThreads, smem, st>>>(a);
    return status("k_facet_adjoint");
}

template <int FT, int SRC>
int adjoint_width(const tm_facet_adjoint_args& a, cudaStream_t st) {
    switch (a.base.width) {
        case 1: return run_facet_adjoint<FT, SRC, 1>(a, st);
        case 2: return run_facet_adjoint<FT, SRC, 2>(a, st);
        case 3: return run_facet_adjoint<FT, SRC, 3>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_facet_adjoint: width must be 1..3");
    }
}

template <int FT>
int adjoint_source(const tm_facet_adjoint_args& a, cudaStream_t st) {
    switch (a.base.source) {
        case TM_SOURCE_CONST: return adjoint_width<FT, TM_SOURCE_CONST>(a, st);
        case TM_SOURCE_NODAL: return adjoint_width<FT, TM_SOURCE_NODAL>(a, st);
        case TM_SOURCE_QUAD: return adjoint_width<FT, TM_SOURCE_QUAD>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_facet_adjoint: unknown source kind");
    }
}

int facet_basis(int ft) {
    switch (ft) {
        case TM_FACET_LINE2: return 2;
        case TM_FACET_LINE3: return 3;
        case TM_FACET_TRI3: return 3;
        case TM_FACET_TRI6: return 6;
        default: return -1;
    }
}

}  // namespace
}  // namespace tmk

using namespace tmk;

extern "C" size_t tm_facet_vector_workspace_bytes(const tm_facet_vector_args* a) {
    if (!a) return 0;
    return align16((a->dtype == TM_F32 ? 4 : 8) * (size_t)a->plan.n_partials * (size_t)a->width) +
           sizeof(int32_t) * (size_t)a->plan.n_shared;
}

extern "C" int tm_assemble_facet_vector(const tm_facet_vector_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: null args");
    const int B = facet_basis(a->tables.facet_type);
    if (B < 0) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_facet_vector: unknown facet type");
    const tm_chunk_plan& P = a->plan;
    if (P.n_basis != B || P.n_local != B)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: plan is not a node plan over this facet type");
    if (P.chunk_elems < 1 || P.chunk_elems > 4096 || a->width < 1 || a->width > 3 || a->n_points < 0)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: bad chunk size, width or n_points");
    if (!a->out || (a->n_points > 0 && P.n_elements > 0 && !a->points) || !a->tables.packed || a->tables.n_quad < 1)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: null pointer");
    if (P.n_elements > 0 && (!P.elem_perm || !P.conn || !P.chunk_begin || !P.slot_ptr || !P.contrib ||
                             !P.slot_target || !P.slot_mirror))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: plan arrays must not be null");
    if (P.n_shared > 0 && (!P.shared_ptr || !P.shared_target || !a->workspace))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: shared arrays or workspace is null");
    if ((a->source == TM_SOURCE_NODAL || a->source == TM_SOURCE_QUAD) && P.n_elements > 0 && !a->values)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: values is null");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (a->dtype == TM_F64) return facet_type<double>(*a, st);
    if (a->dtype == TM_F32) return facet_type<float>(*a, st);
    return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_facet_vector: dtype must be TM_F64 or TM_F32");
}

extern "C" size_t tm_facet_adjoint_workspace_bytes(const tm_facet_adjoint_args* a) {
    if (!a) return 0;
    const int D = (a->base.tables.facet_type == TM_FACET_TRI3 || a->base.tables.facet_type == TM_FACET_TRI6) ? 3 : 2;
    return node_counters_offset<double>(a->base.plan, D) + sizeof(int32_t) * (size_t)a->base.plan.n_shared;
}

extern "C" int tm_facet_adjoint(const tm_facet_adjoint_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_facet_adjoint: null args");
    const tm_facet_vector_args& v = a->base;
    if (v.dtype != TM_F64) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_facet_adjoint: float64 only");
    const int B = facet_basis(v.tables.facet_type);
    if (B < 0) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_facet_adjoint: unknown facet type");
    const tm_chunk_plan& P = v.plan;
    if (P.n_basis != B || P.n_local != B)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_facet_adjoint: plan is not a node plan over this facet type");
    if (P.chunk_elems < 1 || P.chunk_elems > 4096 || v.width < 1 || v.width > 3 || v.n_points < 0)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_facet_adjoint: bad chunk size, width or n_points");
    if (P.n_elements > 0 && (!v.points || !a->lam || !v.tables.packed || !P.elem_perm || !P.conn))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_facet_adjoint: null points, lam, tables or plan");
    if ((v.source == TM_SOURCE_NODAL || v.source == TM_SOURCE_QUAD) && P.n_elements > 0 && !v.values)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_facet_adjoint: values is null");
    if (a->grad_points && P.n_shared > 0 && (!P.shared_ptr || !P.shared_target || !v.workspace))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_facet_adjoint: shared arrays or workspace is null");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    switch (v.tables.facet_type) {
        case TM_FACET_LINE2: return adjoint_source<TM_FACET_LINE2>(*a, st);
        case TM_FACET_LINE3: return adjoint_source<TM_FACET_LINE3>(*a, st);
        case TM_FACET_TRI3: return adjoint_source<TM_FACET_TRI3>(*a, st);
        case TM_FACET_TRI6: return adjoint_source<TM_FACET_TRI6>(*a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_facet_adjoint: unknown facet type");
    }
}
