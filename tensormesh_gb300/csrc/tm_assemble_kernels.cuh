// Kernel templates of the fused assembly (k_matrix, k_matrix_finalize,
// k_vector, the geometry kernels) and their per-form / per-source launchers,
// shared by the translation units that instantiate them for their element
// types: tm_assemble.cu (triangles and tetrahedra, and the C entry points)
// and tm_assemble_quad.cu (quadrilaterals).  The algorithm is described at
// the top of tm_assemble.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>
#include <type_traits>

#include "../../include/tensormesh_gb300.h"
#include "tm_df64.cuh"
#include "tm_df2.cuh"
#include "tm_element.cuh"
#include "tm_reduce.cuh"
#include "tm_status.h"
#include "tm_tma.cuh"

namespace tmk {

constexpr int kThreads = 256;

// set by a kernel whose bounded wait on a staged copy ran out; one word per
// translation unit that includes this header (file scope), read and cleared
// through take_unit_fault by tm_device_fault
static __device__ int g_device_fault = 0;

// this translation unit's fault word, read and cleared; -1 on a CUDA error
static inline int take_unit_fault() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_device_fault, sizeof(int)) != cudaSuccess) return -1;
    if (v) {
        const int zero = 0;
        if (cudaMemcpyToSymbol(g_device_fault, &zero, sizeof(int)) != cudaSuccess) return -1;
    }
    return v;
}

// the float64 P1 diffusion / mass kernels run in double-float arithmetic
template <typename R, int ET, int FORMS>
__host__ __device__ constexpr bool use_df64() {
    return std::is_same<R, double>::value && Traits<ET>::P1 != 0 && (FORMS & TM_FORM_ELASTICITY) == 0;
}

// threads of a k_matrix CTA: one per element of a 384-tet chunk (a 4x4x4
// octant of cubes in Morton order) for the double-float tet kernel
template <typename R, int ET, int FORMS>
constexpr int matrix_threads() {
    return use_df64<R, ET, FORMS>() && ET == TM_TET4 ? 384 : kThreads;
}

// resident CTAs per SM the compiler must allow: four 384-thread CTAs of the
// double-float tet kernel (40 registers), five 256-thread CTAs of the
// double-float triangle kernel (48 registers), three of the double-float
// kernels on non-affine elements (at most 85 registers)
template <typename R, int ET, int FORMS>
constexpr int matrix_min_blocks() {
    if (use_df64<R, ET, FORMS>()) return ET == TM_TET4 ? 4 : 5;
    if (std::is_same<R, double>::value && !Traits<ET>::P1) return 3;
    return 1;
}

struct MatLayout {
    size_t tab, mhl, x, g, jw, ph, ld, ls, lm, le, bar, sp, ct, total;
};

// MS / MC: the plan's largest chunk in slots / contributions (staged copies)
template <typename R, int ET, int FORMS>
__host__ __device__ inline MatLayout mat_layout(int CH, int Q, int MS, int MC) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B, NL = B * (B + 1) / 2;
    constexpr bool DIFF = (FORMS & TM_FORM_DIFFUSION) != 0;
    constexpr bool MASS = (FORMS & TM_FORM_MASS) != 0;
    constexpr bool ELAST = (FORMS & TM_FORM_ELASTICITY) != 0;
    constexpr bool DF64 = use_df64<R, ET, FORMS>();
    constexpr bool DFG = std::is_same<R, double>::value && !T::P1;
    MatLayout L;
    size_t o = 0;
    L.tab = o;
    o = align16(o + sizeof(double) * table_layout(Q, B, D).total);
    L.mhl = o;
    o = align16(o + sizeof(double) * NL * 2);   // mass template: doubles, then double-float pairs
    L.x = L.g = L.jw = o;
    if (!T::P1) {
        L.x = o;
        o = align16(o + sizeof(R) * CH * B * D);
        L.g = o;
        o = align16(o + sizeof(R) * CH * Q * B * D);
        L.jw = o;
        o = align16(o + sizeof(R) * CH * Q);
    }
    L.ph = o;   // double-float path: dphi and w, then (mass) phi, at the quadrature points as pairs
    if (DFG) o = align16(o + 8 * (size_t)Q * (D * B + 1 + (MASS ? B : 0)));
    L.ld = o;
    if (DIFF) o = align16(o + sizeof(R) * CH * NL);
    L.ls = o;   // double-float paths: per element {scale, |det| rho} as four floats
                // (affine) or four exponents (the scalar forms on other elements)
    if (DF64 || DFG) o = align16(o + 16 * (size_t)CH);
    L.lm = o;   // the double-float path's FP64 fallback keeps its masses in the records' space
    if (DF64)
        L.lm = L.ls;
    else if (MASS)
        o = align16(o + sizeof(R) * CH * (T::P1 ? 1 : NL));
    L.le = o;
    // affine elements: the element blocks; the others: {E lam, E mu} per
    // element, the blocks being formed from the gradients during the
    // reduction
    if (ELAST) o = align16(o + sizeof(R) * CH * (T::P1 ? NL * D * D : 2));
    // the chunk's plan: an mbarrier, then 16-byte windows of slot_ptr and
    // contrib
    L.bar = o;
    o += 16;
    L.sp = o;
    o += stage_capacity((int64_t)MS + 1, 4);
    L.ct = o;
    o += stage_capacity(MC, 2);
    L.total = o;
    return L;
}

// tries of the bounded wait for a chunk's staged plan (seconds at most)
constexpr uint32_t kStageTries = 1u << 22;

template <typename R>
__device__ __forceinline__ R rabs(R x) { return x < R(0) ? -x : x; }

template <typename R>
__device__ __forceinline__ R ld_cg(const R* p) { return __ldcg(p); }

template <typename R, int ET, int FORMS>
__global__ void __launch_bounds__((matrix_threads<R, ET, FORMS>()), (matrix_min_blocks<R, ET, FORMS>()))
    k_matrix(const tm_matrix_args a) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B, NL = B * (B + 1) / 2;
    constexpr bool DIFF = (FORMS & TM_FORM_DIFFUSION) != 0;
    constexpr bool MASS = (FORMS & TM_FORM_MASS) != 0;
    constexpr bool ELAST = (FORMS & TM_FORM_ELASTICITY) != 0;
    constexpr bool DF64 = use_df64<R, ET, FORMS>();
    // float64 elasticity on non-affine elements: geometry in FP64, blocks
    // and their sums in double-float arithmetic on the FP32 pipes
    constexpr bool DFE = std::is_same<R, double>::value && !T::P1 && ELAST;
    // float64 diffusion / mass on non-affine elements: the pair integrals
    // and the target sums in double-float
    constexpr bool DFS = std::is_same<R, double>::value && !T::P1 && (DIFF || MASS);
    // any float64 form on non-affine elements: geometry in double-float too
    constexpr bool DFG = DFE || DFS;
    constexpr int HH = ELAST ? D * D : 1;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const MatLayout L = mat_layout<R, ET, FORMS>(CH, Q, P.max_chunk_slots, P.max_chunk_contrib);
    const TableLayout TL = table_layout(Q, B, D);
    extern __shared__ __align__(16) unsigned char sm[];

    // the finalising grid may be scheduled once every chunk has started
    asm volatile("griddepcontrol.launch_dependents;");

    // stage this chunk's slots and contributions (bulk copies that land
    // while phase 1 runs)
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L.bar);
    const int32_t s0 = P.chunk_begin[blockIdx.x], s1 = P.chunk_begin[blockIdx.x + 1];
    const int32_t c0 = P.chunk_contrib[blockIdx.x], c1 = P.chunk_contrib[blockIdx.x + 1];
    const StageRange w_sp = stage_range(s0, (int64_t)s1 + 1, 4);
    const StageRange w_ct = stage_range(c0, c1, 2);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_arrive_expect_tx(bar, w_sp.bytes + w_ct.bytes);
        const unsigned char* g_sp = reinterpret_cast<const unsigned char*>(P.slot_ptr);
        const unsigned char* g_ct = reinterpret_cast<const unsigned char*>(P.contrib);
        bulk_copy_g2s(sm + L.sp, g_sp + w_sp.begin, w_sp.bytes, bar);
        if (w_ct.bytes) bulk_copy_g2s(sm + L.ct, g_ct + w_ct.begin, w_ct.bytes, bar);
    }
    const int32_t* SP = reinterpret_cast<const int32_t*>(sm + L.sp) + w_sp.skip;   // slot_ptr[s0 + j]
    const uint16_t* CT = reinterpret_cast<const uint16_t*>(sm + L.ct) + w_ct.skip;  // contrib[c0 + q]
    double* tab = reinterpret_cast<double*>(sm + L.tab);
    double* mhl = reinterpret_cast<double*>(sm + L.mhl);
    f2* mh2 = reinterpret_cast<f2*>(mhl + NL);
    R* LD = reinterpret_cast<R*>(sm + L.ld);
    R* LS = reinterpret_cast<R*>(sm + L.ls);
    R* LM = reinterpret_cast<R*>(sm + L.lm);
    R* LE = reinterpret_cast<R*>(sm + L.le);
    // per (element, quadrature point) gradients and weights (non-affine elements)
    [[maybe_unused]] R* G = reinterpret_cast<R*>(sm + L.g);
    [[maybe_unused]] R* JW = reinterpret_cast<R*>(sm + L.jw);

    // per-CTA constants of the double-float path, computed once by thread 0:
    // the range check of the scales and of the mass template, and the
    // template's class structure (bit l of diag_mask set when local entry l
    // is a diagonal (a, a); mass_sym when the template has one diagonal and
    // one off-diagonal value, as every symmetric quadrature rule gives, so
    // that the mass of a target is its class value times the sum of |det| rho
    // of its contributions)
    __shared__ struct {
        unsigned diag_mask;
        int mass_sym, bad;
    } cta;
    if constexpr (DF64) {
        if (threadIdx.x == 0) {
            const double* pk = a.tables.packed;
            int bad = !exponent_in_band(a.kappa_scale, 30) || !exponent_in_band(a.mass_scale, 30) ||
                      !exponent_in_band(pk[TL.wsum], 30);
            unsigned dm = 0;
            int msym = 0;
            if constexpr (MASS) {
                for (int k = 0; k < B * B; ++k) bad |= !exponent_in_band(pk[TL.mhat + k], 30);
                for (int pa = 0; pa < B; ++pa) dm |= 1u << (pa * B - pa * (pa - 1) / 2);
                const double m_diag = pk[TL.mhat], m_off = pk[TL.mhat + 1];
                msym = 1;
                for (int pa = 0; pa < B; ++pa)
                    for (int pb = pa; pb < B; ++pb) msym &= pk[TL.mhat + pa * B + pb] == (pa == pb ? m_diag : m_off);
            }
            cta.diag_mask = dm;
            cta.mass_sym = msym;
            cta.bad = bad;
        }
    }
    for (int k = threadIdx.x; k < TL.total; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();
    if (MASS && T::P1)
        for (int l = threadIdx.x; l < NL; l += blockDim.x) {
            int pa, pb;
            upper_pair<B>(l, pa, pb);
            mhl[l] = tab[TL.mhat + pa * B + pb];
            if (DF64) mh2[l] = split_double(mhl[l]);
        }

    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const R* pts = static_cast<const R*>(a.points);
    const R* kap = static_cast<const R*>(a.kappa);
    const R* yng = static_cast<const R*>(a.young);
    const R kscale = (R)a.kappa_scale, mscale = (R)a.mass_scale, yscale = (R)a.young_scale;
    const R nu = (R)a.poisson;
    const R clam = nu / ((R(1) + nu) * (R(1) - R(2) * nu));
    const R cmu = R(1) / (R(2) * (R(1) + nu));

    bool use_df = false;
    [[maybe_unused]] bool use_dfg = false;
    // per element (double-float, non-affine): the exponents {sg, sw, sk, sm}
    // of its gradient, weight, kappa and mass scalings (elasticity: {sg, sw,
    // se, S})
    [[maybe_unused]] int* SI = reinterpret_cast<int*>(sm + L.ls);
    // dphi [Q][D][B], w [Q] and (mass) phi [Q][B] as double-float pairs
    [[maybe_unused]] f2* DP2 = reinterpret_cast<f2*>(sm + L.ph);
    [[maybe_unused]] f2* W2 = DP2 + Q * D * B;
    [[maybe_unused]] f2* PH2 = W2 + Q;
    if constexpr (T::P1 != 0) {
        const R wsum = (R)tab[TL.wsum];
        // P1 simplices in the arithmetic of R: unscaled gradients C_b (g_b = C_b / det)
        auto native_p1 = [&]() {
            for (int el = threadIdx.x; el < ne; el += blockDim.x) {
                const int64_t i = i0 + el;
                const int e = P.elem_perm[i];
                R X[B][D];
#pragma unroll
                for (int b = 0; b < B; ++b) {
                    const int64_t node = P.conn[i * B + b];
#pragma unroll
                    for (int d = 0; d < D; ++d) X[b][d] = ldg(pts + node * D + d);
                }
                R C[B][D];
                const R det = p1_gradients<R, D>(X, C);
                const R adet = rabs(det);
                if constexpr (DIFF) {
                    const R kv = (kap ? ldg(kap + e) : R(1)) * kscale;
                    const R s = kv * wsum / adet;
                    int l = 0;
#pragma unroll
                    for (int p = 0; p < B; ++p)
#pragma unroll
                        for (int q = p; q < B; ++q, ++l) LD[el * NL + l] = s * dot<R, D>(C[p], C[q]);
                }
                if constexpr (MASS) LM[el] = adet * mscale;
                if constexpr (ELAST) {
                    const R Ey = (yng ? ldg(yng + e) : R(1)) * yscale;
                    const R s = wsum / adet;
                    int l = 0;
#pragma unroll
                    for (int p = 0; p < B; ++p)
#pragma unroll
                        for (int q = p; q < B; ++q, ++l)
                            elastic_block<R, D>(C[p], C[q], Ey * clam, Ey * cmu, s, LE + (el * NL + l) * HH, false);
                }
            }
        };
        if constexpr (DF64) {
            // Double-float locals: for diffusion the unscaled Gram entries
            // G_ab = C_a . C_b (LD) and the per-element scale kappa W / |det|
            // (LS), multiplied during the reduction; for mass |det| rho (LM).
            f2* LG2 = reinterpret_cast<f2*>(LD);
            float4* LR = reinterpret_cast<float4*>(LS);
            bool bad = cta.bad != 0;
            const f2 ks = split_double(a.kappa_scale), ms = split_double(a.mass_scale);
            const f2 ws = split_double(tab[TL.wsum]);
            for (int el = threadIdx.x; el < ne; el += blockDim.x) {
                const int64_t i = i0 + el;
                const int e = P.elem_perm[i];
                double X[B][D];
#pragma unroll
                for (int b = 0; b < B; ++b) {
                    const int64_t node = P.conn[i * B + b];
#pragma unroll
                    for (int d = 0; d < D; ++d) X[b][d] = ldg(static_cast<const double*>(a.points) + node * D + d);
                }
                // J[i][j] = x_{i+1,j} - x_{0,j}: the one FP64 step, then split.
                // The element's scale (its largest edge component) must lie in
                // [2^-20, 2^20]; smaller components are fine at that scale.
                f2 J[D][D];
                int emax = 0;
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        const double dd = X[r + 1][c] - X[0][c];
                        emax = max(emax, biased_exponent(dd));
                        J[r][c] = split_double(dd);
                    }
                bad |= emax < 1023 - 20 || emax >= 1023 + 20;
                f2 cof[D][D];
                f2 det;
                if constexpr (D == 3) {
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        const int r1 = (r + 1) % 3, r2 = (r + 2) % 3;
                        cof[r][0] = f2_diff_of_products(J[r1][1], J[r2][2], J[r1][2], J[r2][1]);
                        cof[r][1] = f2_diff_of_products(J[r1][2], J[r2][0], J[r1][0], J[r2][2]);
                        cof[r][2] = f2_diff_of_products(J[r1][0], J[r2][1], J[r1][1], J[r2][0]);
                    }
                    det = f2_dot3(J[0], cof[0]);
                } else {
                    cof[0][0] = J[1][1];
                    cof[0][1] = f2_neg(J[1][0]);
                    cof[1][0] = f2_neg(J[0][1]);
                    cof[1][1] = J[0][0];
                    det = f2_diff_of_products(J[0][0], J[1][1], J[0][1], J[1][0]);
                }
                const f2 adet = f2_abs(det);
                bad |= !(adet.hi > 0.0f) || !f2_in_band(adet, -100, 100);
                float4 rec = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if constexpr (DIFF) {
                    // Gram matrix of the cofactor rows; vertex 0 has C_0 = -sum_i cof_i,
                    // so C_0.C_0 = sum_ij G_ij and C_0.C_{j+1} = -sum_i G_ij
                    f2 G[D][D];
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = r; c < D; ++c) {
                            G[r][c] = D == 3 ? f2_dot3(cof[r], cof[c]) : f2_dot2(cof[r], cof[c]);
                            G[c][r] = G[r][c];
                        }
                    f2 rs[D];
                    int gmax = 0;
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        f2 acc = G[0][c];
#pragma unroll
                        for (int r = 1; r < D; ++r) acc = f2_add(acc, G[r][c]);
                        rs[c] = acc;
                        gmax = max(gmax, (int)((__float_as_uint(G[c][c].hi) >> 23) & 0xFF));
                    }
                    f2 tot = rs[0];
#pragma unroll
                    for (int c = 1; c < D; ++c) tot = f2_add(tot, rs[c]);
                    gmax = max(gmax, (int)((__float_as_uint(tot.hi) >> 23) & 0xFF));
                    const double kd = kap ? ldg(static_cast<const double*>(a.kappa) + e) : 1.0;
                    bad |= !exponent_in_band(kd, 30);
                    const f2 sc = f2_mul(f2_mul(split_double(kd), ks), f2_mul(ws, f2_recip(adet)));
                    const int sexp = (int)((__float_as_uint(sc.hi) >> 23) & 0xFF);
                    bad |= !f2_finite(sc) || (gmax - 127) + (sexp - 127) >= 100;
                    rec.x = sc.hi;
                    rec.y = sc.lo;
                    f2* g = LG2 + el * NL;
                    int l = 0;
                    g[l++] = tot;
#pragma unroll
                    for (int q = 0; q < D; ++q) g[l++] = f2_neg(rs[q]);
#pragma unroll
                    for (int p = 0; p < D; ++p)
#pragma unroll
                        for (int q = p; q < D; ++q) g[l++] = G[p][q];
                }
                if constexpr (MASS) {
                    const f2 v = f2_mul(adet, ms);
                    bad |= !f2_in_band(v, -127, 100);
                    rec.z = v.hi;
                    rec.w = v.lo;
                }
                LR[el] = rec;
            }
            use_df = !__syncthreads_or(bad);
            if (!use_df) {
                if (threadIdx.x == 0 && a.stats) atomicAdd(a.stats, 1);
                native_p1();
            }
        } else {
            native_p1();
        }
    } else {
        R* X = reinterpret_cast<R*>(sm + L.x);
        auto stage_x = [&]() {
            for (int k = threadIdx.x; k < ne * B; k += blockDim.x) {
                const int64_t node = P.conn[i0 * B + k];
#pragma unroll
                for (int d = 0; d < D; ++d) X[k * D + d] = ldg(pts + node * D + d);
            }
            __syncthreads();
        };
        // geometry per (element, quadrature point) in the arithmetic of R
        auto geometry_native = [&]() {
            for (int k = threadIdx.x; k < ne * Q; k += blockDim.x) {
                const int el = k / Q, q = k - el * Q;
                const double* dphi = tab + TL.dphi + q * D * B;
                R J[D][D];
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        R s = 0;
#pragma unroll
                        for (int b = 0; b < B; ++b) s += (R)dphi[r * B + b] * X[(el * B + b) * D + c];
                        J[r][c] = s;
                    }
                R cof[D][D];
                const R det = cofactors<R>(J, cof);
                const R inv = R(1) / det;
                R* g = G + (size_t)k * B * D;
#pragma unroll
                for (int b = 0; b < B; ++b)
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        R s = 0;
#pragma unroll
                        for (int r = 0; r < D; ++r) s += (R)dphi[r * B + b] * cof[r][c];
                        g[b * D + c] = s * inv;
                    }
                JW[k] = (R)tab[TL.w + q] * rabs(det);
            }
            if constexpr (ELAST) {
                // the element's scaled Lame constants; its blocks are formed
                // from G and JW during the reduction (elasticity is never fused)
                for (int el = threadIdx.x; el < ne; el += blockDim.x) {
                    const R Ey = (yng ? ldg(yng + P.elem_perm[i0 + el]) : R(1)) * yscale;
                    LE[2 * el] = Ey * clam;
                    LE[2 * el + 1] = Ey * cmu;
                }
            }
            __syncthreads();
        };
        stage_x();
        if constexpr (DFG) {
            // Float64 on non-affine elements, in double-float on the FP32
            // pipes.  (1) Per element, the coordinate differences to its
            // first node (FP64 subtractions) scaled by the power of two of
            // the largest one and split.  (2) Per (element, quadrature
            // point): Jacobian, cofactors, determinant, its reciprocal, the
            // gradients and the weight |det| w, on those scaled coordinates.
            // (3) Per element, powers of two that bring its largest gradient
            // entry and weight to [1/2, 1), and the form's scales: kappa and
            // the mass scale (pair integrals scaled back by 2^(2 sg + sw +
            // sk), 2^(sw + sm)) or the moduli (blocks by 2^S, S = 2 sg + sw +
            // se).  A chunk with a degenerate element, a value that is not
            // finite or a shift outside (-70, 100) runs in FP64 instead.
            for (int t = threadIdx.x; t < Q * D * B; t += blockDim.x) DP2[t] = split_double(tab[TL.dphi + t]);
            for (int t = threadIdx.x; t < Q; t += blockDim.x) W2[t] = split_double(tab[TL.w + t]);
            if constexpr (MASS)
                for (int t = threadIdx.x; t < Q * B; t += blockDim.x) PH2[t] = split_double(tab[TL.phi + t]);
            f2* X2 = reinterpret_cast<f2*>(X);
            f2* G2 = reinterpret_cast<f2*>(G);
            f2* JW2 = reinterpret_cast<f2*>(JW);
            bool ok = true;
            for (int el = threadIdx.x; el < ne; el += blockDim.x) {
                const R* xe = X + el * B * D;
                int ex = 0;
#pragma unroll
                for (int b = 1; b < B; ++b)
#pragma unroll
                    for (int c = 0; c < D; ++c) ex = max(ex, biased_exponent(xe[b * D + c] - xe[c]));
                ok = ok && ex > 0 && ex < 2047;
                const int sx = ex - 1022;
                // in place, node 0 last (the others are taken relative to it)
                for (int b = B - 1; b >= 0; --b)
#pragma unroll
                    for (int c = 0; c < D; ++c) X2[(el * B + b) * D + c] = split_scaled(xe[b * D + c] - xe[c], sx);
                SI[4 * el] = sx;
            }
            __syncthreads();
            // two threads per (element, point): both form J, its cofactors
            // and determinant, each half of the gradients
            for (int k2 = threadIdx.x; k2 < 2 * ne * Q; k2 += blockDim.x) {
                const int k = k2 >> 1, half = k2 & 1;
                const int el = k / Q, q = k - el * Q;
                const f2* dp = DP2 + q * D * B;
                const f2* xe = X2 + el * B * D;
                f2 J[D][D];
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        acc2 t = {0.0f, 0.0f};
#pragma unroll
                        for (int b = 1; b < B; ++b) acc_fma(t, dp[r * B + b], xe[b * D + c]);
                        J[r][c] = acc_value(t);
                    }
                f2 cof[D][D];
                f2 det;
                if constexpr (D == 3) {
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        const int r1 = (r + 1) % 3, r2 = (r + 2) % 3;
                        cof[r][0] = f2_diff_of_products(J[r1][1], J[r2][2], J[r1][2], J[r2][1]);
                        cof[r][1] = f2_diff_of_products(J[r1][2], J[r2][0], J[r1][0], J[r2][2]);
                        cof[r][2] = f2_diff_of_products(J[r1][0], J[r2][1], J[r1][1], J[r2][0]);
                    }
                    det = f2_dot3(J[0], cof[0]);
                } else {
                    cof[0][0] = J[1][1];
                    cof[0][1] = f2_neg(J[1][0]);
                    cof[1][0] = f2_neg(J[0][1]);
                    cof[1][1] = J[0][0];
                    det = f2_diff_of_products(J[0][0], J[1][1], J[0][1], J[1][0]);
                }
                const f2 adet = f2_abs(det);
                const f2 inv = f2_recip(det);
                ok = ok && adet.hi > 0.0f && f2_in_band(adet, -60, 60) && f2_finite(inv);
                if constexpr (DIFF || ELAST) {    // (mass needs only the weights)
                    f2* g = G2 + (size_t)k * B * D;
#pragma unroll
                    for (int bb = 0; bb < (B + 1) / 2; ++bb) {
                        const int b = 2 * bb + half;
                        if (b < B)
#pragma unroll
                            for (int c = 0; c < D; ++c) {
                                acc2 t = {0.0f, 0.0f};
#pragma unroll
                                for (int r = 0; r < D; ++r) acc_fma(t, dp[r * B + b], cof[r][c]);
                                g[b * D + c] = f2_mul(acc_value(t), inv);
                            }
                    }
                }
                if (half == 0) JW2[k] = f2_mul(W2[q], adet);
            }
            __syncthreads();
            auto fexp = [](f2 v) { return (int)((__float_as_uint(v.hi) >> 23) & 0xFF); };
            auto shift = [](double v) {
                const int e = biased_exponent(v);
                return e == 0 ? 0 : e - 1022;
            };
            // eight threads per element (a group of lanes of one warp) find
            // and apply its scales; the group's first thread the rest
            constexpr int GS = 8;
            const int gi = threadIdx.x & (GS - 1);
            const unsigned gmask = 0xFFu << ((threadIdx.x & 31) & ~(GS - 1));
            for (int el = threadIdx.x / GS; el < ne; el += blockDim.x / GS) {
                const int sx = SI[4 * el];
                f2* g = G2 + (size_t)el * Q * B * D;
                f2* w = JW2 + el * Q;
                int fg = 126, fw = 0;    // (126: a mass-only kernel has no gradients to scale)
                if constexpr (DIFF || ELAST) {
                    fg = 0;
                    for (int t = gi; t < Q * B * D; t += GS) fg = max(fg, fexp(g[t]));
                }
                for (int q = gi; q < Q; q += GS) fw = max(fw, fexp(w[q]));
#pragma unroll
                for (int o = GS / 2; o > 0; o >>= 1) {
                    fg = max(fg, __shfl_xor_sync(gmask, fg, o));
                    fw = max(fw, __shfl_xor_sync(gmask, fw, o));
                }
                // (float exponents in [2^-125, 2^124): the scale factors
                // below stay normal floats)
                ok = ok && fg >= 2 && fg <= 251 && fw >= 2 && fw <= 251;
                const float cg = pow2f(126 - fg), cw = pow2f(126 - fw);    // max to [1/2, 1)
                if constexpr (DIFF || ELAST)
                    for (int t = gi; t < Q * B * D; t += GS) g[t] = {__fmul_rn(g[t].hi, cg), __fmul_rn(g[t].lo, cg)};
                for (int q = gi; q < Q; q += GS) w[q] = {__fmul_rn(w[q].hi, cw), __fmul_rn(w[q].lo, cw)};
                if (gi != 0) continue;
                const int sg = fg - 126 - sx, sw = fw - 126 + D * sx;
                const int e = P.elem_perm[i0 + el];
                int s2 = 0, s3 = 0;
                if constexpr (ELAST) {
                    // the element's weight E 2^S (S = 2 sg + sw + se): its
                    // A, on scaled gradients and weights, times the weight
                    // is A at true scale times E; lam and mu are E times the
                    // call's two constants, applied once per target
                    const double Ey = (yng ? ldg(yng + e) : 1.0) * yscale;
                    const int ee = biased_exponent(Ey);
                    const int se = ee == 0 ? 0 : ee - 1022;
                    s2 = se;
                    s3 = 2 * sg + sw + se;
                    ok = ok && ee > 0 && ee < 2047 && s3 > -70 && s3 < 100;
                    const f2 wy = split_scaled(Ey, se);
                    const float sc = pow2f(s3);
                    reinterpret_cast<f2*>(LE + 2 * el)[0] = {__fmul_rn(wy.hi, sc), __fmul_rn(wy.lo, sc)};
                }
                if constexpr (DIFF) {
                    const double kv = (kap ? ldg(kap + e) : 1.0) * kscale;
                    s2 = shift(kv);
                    const int S = 2 * sg + sw + s2;
                    ok = ok && biased_exponent(kv) < 2047 && S > -70 && S < 100;
                }
                if constexpr (MASS) {
                    s3 = shift(mscale);
                    const int S = sw + s3;
                    ok = ok && biased_exponent(mscale) < 2047 && S > -70 && S < 100;
                }
                SI[4 * el] = sg;
                SI[4 * el + 1] = sw;
                SI[4 * el + 2] = s2;
                SI[4 * el + 3] = s3;
            }
            use_dfg = !__syncthreads_or(!ok);
            if (!use_dfg) {
                if (threadIdx.x == 0 && a.stats) atomicAdd(a.stats, 1);
                stage_x();
                geometry_native();
            }
        } else {
            geometry_native();
        }
        for (int k = threadIdx.x; k < (DIFF || MASS ? ne * NL : 0); k += blockDim.x) {
            const int el = k / NL, l = k - el * NL;
            int pa, pb;
            upper_pair<B>(l, pa, pb);
            const int e = P.elem_perm[i0 + el];
            if (DFS && use_dfg) {
                // the scaled pair integrals in double-float
                const f2* G2 = reinterpret_cast<const f2*>(G);
                const f2* JW2 = reinterpret_cast<const f2*>(JW);
                if constexpr (DIFF) {
                    acc2 sd = {0.0f, 0.0f};
                    for (int q = 0; q < Q; ++q) {
                        const f2* g = G2 + (size_t)(el * Q + q) * B * D;
                        const f2 d = D == 3 ? f2_dot3(g + pa * D, g + pb * D) : f2_dot2(g + pa * D, g + pb * D);
                        acc_fma(sd, JW2[el * Q + q], d);
                    }
                    const double kv = (kap ? ldg(kap + e) : 1.0) * kscale;
                    reinterpret_cast<f2*>(LD)[k] = f2_mul(split_scaled(kv, SI[4 * el + 2]), acc_value(sd));
                }
                if constexpr (MASS) {
                    acc2 sv = {0.0f, 0.0f};
                    for (int q = 0; q < Q; ++q) acc_fma(sv, JW2[el * Q + q], f2_mul(PH2[q * B + pa], PH2[q * B + pb]));
                    reinterpret_cast<f2*>(LM)[k] = f2_mul(split_scaled(mscale, SI[4 * el + 3]), acc_value(sv));
                }
                continue;
            }
            if constexpr (DIFF) {
                R s = 0;
                for (int q = 0; q < Q; ++q) {
                    const R* g = G + (size_t)(el * Q + q) * B * D;
                    s += JW[el * Q + q] * dot<R, D>(g + pa * D, g + pb * D);
                }
                LD[k] = s * ((kap ? ldg(kap + e) : R(1)) * kscale);
            }
            if constexpr (MASS) {
                R s = 0;
                for (int q = 0; q < Q; ++q)
                    s += JW[el * Q + q] * (R)tab[TL.phi + q * B + pa] * (R)tab[TL.phi + q * B + pb];
                LM[k] = s * mscale;
            }
        }
    }
    // the staged plan must have landed; a wait that runs out flags the
    // device and leaves the chunk unwritten
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0, kStageTries))) {
        if (threadIdx.x == 0) atomicExch(&g_device_fault, 1);
        mbar_wait_bounded(bar, 0, kStageTries);      // copies in flight end before the CTA does
        return;
    }

    // phase 2: fixed-order reduction of the chunk's targets
    uint32_t diag_mask = 0;
    bool mass_sym = false;
    if constexpr (DF64 && MASS) {
        diag_mask = cta.diag_mask;
        mass_sym = cta.mass_sym != 0;
    }
    R* oD = static_cast<R*>(a.out_diffusion);
    R* oM = static_cast<R*>(a.out_mass);
    R* oE = static_cast<R*>(a.out_elasticity);
    R* part = static_cast<R*>(a.workspace);
    // a target's value at its CSR position and, for symmetric forms, the
    // transpose at the mirrored position
    auto write_out = [&](int64_t tgt, int64_t mir, R ad, R am, const R* ae) {
        if constexpr (DIFF) {
            oD[tgt] = ad;
            if (mir != tgt) oD[mir] = ad;
        }
        if constexpr (MASS) {
            oM[tgt] = am;
            if (mir != tgt) oM[mir] = am;
        }
        if constexpr (ELAST) {
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    oE[tgt * HH + r * D + c] = ae[r * D + c];
                    if (mir != tgt) oE[mir * HH + c * D + r] = ae[r * D + c];
                }
        }
    };
    // a slot's result: its CSR position(s), or this chunk's partial of a
    // shared target (summed in chunk order by k_matrix_finalize; partials
    // interleaved per target)
    auto emit = [&](int64_t tgt, int64_t mir, R ad, R am, const R* ae) {
        if (tgt < 0) {
            const int64_t pi = -tgt - 1;
            if constexpr (ELAST) {
#pragma unroll
                for (int k = 0; k < HH; ++k) part[pi * HH + k] = ae[k];
            } else if constexpr (DIFF && MASS) {
                part[2 * pi] = ad;
                part[2 * pi + 1] = am;
            } else {
                part[pi] = DIFF ? ad : am;
            }
            return;
        }
        write_out(tgt, mir, ad, am, ae);
    };
    const int ns = s1 - s0;

    if constexpr (DF64) {
        if (use_df) {
            // compensated sums: TwoSum on the high parts, the error terms and
            // the low parts summed in plain float (|error| ~ 2^-48 of the
            // terms).  A CSR position receives only diagonal local entries
            // (a, a) or only off-diagonal ones, so with mass_sym one sum of
            // |det| per target is scaled by the template value of its class.
            const f2* LG2 = reinterpret_cast<const f2*>(LD);
            const float4* LR = reinterpret_cast<const float4*>(LS);
            auto reduce = [&](auto msym_tag) {
                [[maybe_unused]] constexpr bool MSYM = decltype(msym_tag)::value;
                for (int j = threadIdx.x; j < ns; j += blockDim.x) {
                    const int p0 = SP[j] - c0, p1 = SP[j + 1] - c0;
                    const int32_t tgt = __ldcs(P.slot_target + s0 + j), mir = __ldcs(P.slot_mirror + s0 + j);
                    [[maybe_unused]] float kh = 0.0f, ke = 0.0f;   // diffusion
                    [[maybe_unused]] float vh = 0.0f, ve = 0.0f;   // mass: sum of |det| (mass_sym)
                    [[maybe_unused]] f2 sm2 = {0.0f, 0.0f};        // mass, general template
                    for (int p = p0; p < p1; ++p) {
                        const unsigned idx = (unsigned)CT[p] >> 1;
                        const unsigned el = idx / (unsigned)NL;
                        float4 r;
                        if constexpr (MASS) {
                            r = LR[el];
                        } else {
                            const float2 h = reinterpret_cast<const float2*>(LR)[2 * el];
                            r = make_float4(h.x, h.y, 0.0f, 0.0f);
                        }
                        if constexpr (DIFF) {
                            const f2 g = LG2[idx];
                            const float pr = __fmul_rn(r.x, g.hi);
                            float er = __fmaf_rn(r.x, g.hi, -pr);
                            er = __fmaf_rn(r.x, g.lo, er);
                            er = __fmaf_rn(r.y, g.hi, er);
                            const f2 t = two_sum(kh, pr);
                            kh = t.hi;
                            ke = __fadd_rn(ke, __fadd_rn(t.lo, er));
                        }
                        if constexpr (MASS) {
                            if constexpr (MSYM) {
                                const f2 t = two_sum(vh, r.z);
                                vh = t.hi;
                                ve = __fadd_rn(ve, __fadd_rn(t.lo, r.w));
                            } else {
                                sm2 = f2_add(sm2, f2_mul(f2_make(r.z, r.w), mh2[idx - el * (unsigned)NL]));
                            }
                        }
                    }
                    R ad = 0, am = 0;
                    if constexpr (DIFF) ad = (R)f2_to_double(two_sum(kh, ke));
                    if constexpr (MASS) {
                        if constexpr (MSYM) {
                            const unsigned idx = (unsigned)CT[p0] >> 1;
                            const unsigned l = idx - (idx / (unsigned)NL) * (unsigned)NL;
                            sm2 = f2_mul(two_sum(vh, ve), mh2[((diag_mask >> l) & 1u) ? 0 : 1]);
                        }
                        am = (R)f2_to_double(sm2);
                    }
                    emit(tgt, mir, ad, am, nullptr);
                }
            };
            if (mass_sym)
                reduce(std::true_type{});
            else
                reduce(std::false_type{});
            return;
        }
    }

    if constexpr (DFS) {
        if (use_dfg) {
            // compensated sums of the scaled pair integrals, scaled back by
            // their element's power of two, in element order; one FP64 add
            // rounds each target
            const f2* LD2 = reinterpret_cast<const f2*>(LD);
            const f2* LM2 = reinterpret_cast<const f2*>(LM);
            for (int j = threadIdx.x; j < ns; j += blockDim.x) {
                const int p0 = SP[j] - c0, p1 = SP[j + 1] - c0;
                const int32_t tgt = __ldcs(P.slot_target + s0 + j), mir = __ldcs(P.slot_mirror + s0 + j);
                acc2 sd = {0.0f, 0.0f}, sv = {0.0f, 0.0f};
                for (int p = p0; p < p1; ++p) {
                    const int idx = CT[p] >> 1;
                    const int el = idx / NL;
                    const int4 sh = reinterpret_cast<const int4*>(SI)[el];
                    if constexpr (DIFF) {
                        f2 v = LD2[idx];
                        const float sc = pow2f(2 * sh.x + sh.y + sh.z);
                        v.hi = __fmul_rn(v.hi, sc);
                        v.lo = __fmul_rn(v.lo, sc);
                        acc_add(sd, v);
                    }
                    if constexpr (MASS) {
                        f2 v = LM2[idx];
                        const float sc = pow2f(sh.y + sh.w);
                        v.hi = __fmul_rn(v.hi, sc);
                        v.lo = __fmul_rn(v.lo, sc);
                        acc_add(sv, v);
                    }
                }
                const R ad = DIFF ? (R)f2_to_double(acc_value(sd)) : R(0);
                const R am = MASS ? (R)f2_to_double(acc_value(sv)) : R(0);
                emit(tgt, mir, ad, am, nullptr);
            }
            return;
        }
    }

    if constexpr (DFE) {
        if (use_dfg) {
            // Per target, S = sum over its contributions of E_e X_e, X_e =
            // A_e = sum_q jw g_a g_b^T of the contribution's (element, pair)
            // (A_e^T for a transposed one), in double-float on the element's
            // scaled values and weight E 2^S, as a compensated sum in
            // element order; the target's block is then lam' S + mu' (S^T +
            // tr S I) (lam = E lam', mu = E mu' for the call's Poisson
            // ratio: the sum of the contributions' blocks), rounded once.
            // The entries go two by two through the paired FP32
            // instructions: rows (r, 0), (r, 1) and, in 3-D, the column
            // (0, 2), (1, 2) as pairs, (2, 2) alone.
            const f2* G2 = reinterpret_cast<const f2*>(G);
            const f2* JW2 = reinterpret_cast<const f2*>(JW);
            using L2 = float2;
            using P2 = ddv<L2>;
            constexpr int NP = D == 3 ? 4 : 2;                 // entry pairs (and, in 3-D, (2, 2))
            auto pair = [](f2 x, f2 y) { return P2{make_float2(x.hi, y.hi), make_float2(x.lo, y.lo)}; };
            auto bcast = [](f2 x) { return P2{make_float2(x.hi, x.hi), make_float2(x.lo, x.lo)}; };
            auto lane = [](P2 v, int k) { return k ? f2_make(v.hi.y, v.lo.y) : f2_make(v.hi.x, v.lo.x); };
            // the transpose in the same pairs
            auto transp = [&](const P2* V, P2* T) {
                T[0] = pair(lane(V[0], 0), lane(V[1], 0));
                T[1] = pair(lane(V[0], 1), lane(V[1], 1));
                if constexpr (D == 3) {
                    T[2] = V[3];
                    T[3] = V[2];
                }
            };
            const f2 cl = split_double((double)clam), cm = split_double((double)cmu);
            for (int j = threadIdx.x; j < ns; j += blockDim.x) {
                const int p0 = SP[j] - c0, p1 = SP[j + 1] - c0;
                const int32_t tgt = __ldcs(P.slot_target + s0 + j), mir = __ldcs(P.slot_mirror + s0 + j);
                dacc<L2> sum[NP];
                acc2 sum22 = {0.0f, 0.0f};
#pragma unroll
                for (int k = 0; k < NP; ++k) sum[k] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
                for (int p = p0; p < p1; ++p) {
                    const int code = CT[p];
                    const int idx = code >> 1;
                    const int el = idx / NL;
                    int pa, pb;
                    upper_pair<B>(idx - el * NL, pa, pb);
                    // A in pairs: {(r,0),(r,1)} for each row r, then (3-D) {(0,2),(1,2)}
                    dacc<L2> A[NP];
                    acc2 a22 = {0.0f, 0.0f};
#pragma unroll
                    for (int k = 0; k < NP; ++k) A[k] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
                    for (int q = 0; q < Q; ++q) {
                        const f2* g = G2 + (size_t)(el * Q + q) * B * D;
                        const f2 w = JW2[el * Q + q];
                        // t = w g_b: (t0, t1) paired, t2 alone
                        const P2 t01 = p_mul(bcast(w), pair(g[pb * D], g[pb * D + 1]));
#pragma unroll
                        for (int r = 0; r < D; ++r) d_fma(A[r], bcast(g[pa * D + r]), t01);
                        if constexpr (D == 3) {
                            const f2 t2 = f2_mul(w, g[pb * D + 2]);
                            d_fma(A[3], pair(g[pa * D], g[pa * D + 1]), bcast(t2));
                            acc_fma(a22, g[pa * D + 2], t2);
                        }
                    }
                    P2 V[NP], T[NP];
#pragma unroll
                    for (int k = 0; k < NP; ++k) V[k] = d_value(A[k]);
                    transp(V, T);
                    const bool tp = code & 1;
                    const P2 wy = bcast(reinterpret_cast<const f2*>(LE + 2 * el)[0]);
#pragma unroll
                    for (int k = 0; k < NP; ++k) d_fma(sum[k], wy, tp ? T[k] : V[k]);
                    if constexpr (D == 3) acc_fma(sum22, lane(wy, 0), acc_value(a22));
                }
                // the block: lam' S + mu' (S^T + tr S I)
                P2 S[NP], ST[NP];
#pragma unroll
                for (int k = 0; k < NP; ++k) S[k] = d_value(sum[k]);
                transp(S, ST);
                const f2 s22 = acc_value(sum22);
                f2 tr = f2_add(lane(S[0], 0), lane(S[1], 1));
                if constexpr (D == 3) tr = f2_add(tr, s22);
                const P2 CL = bcast(cl), CM = bcast(cm);
                P2 K[NP];
#pragma unroll
                for (int k = 0; k < NP; ++k) {
                    P2 Y = ST[k];
                    if (k < 2) {
                        // the diagonal lane: (0,0) in pair 0, (1,1) in pair 1
                        const P2 trk = k == 0 ? P2{make_float2(tr.hi, 0.0f), make_float2(tr.lo, 0.0f)}
                                              : P2{make_float2(0.0f, tr.hi), make_float2(0.0f, tr.lo)};
                        Y = p_add(Y, trk);
                    }
                    K[k] = p_add(p_mul(CL, S[k]), p_mul(CM, Y));
                }
                // back to row-major entries
                R ae[HH];
                if constexpr (D == 3) {
                    const f2 k22 = f2_add(f2_mul(cl, s22), f2_mul(cm, f2_add(s22, tr)));
                    const int src[9][2] = {{0, 0}, {0, 1}, {3, 0}, {1, 0}, {1, 1}, {3, 1}, {2, 0}, {2, 1}, {-1, 0}};
#pragma unroll
                    for (int k = 0; k < 9; ++k)
                        ae[k] = (R)f2_to_double(src[k][0] < 0 ? k22 : lane(K[src[k][0]], src[k][1]));
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) ae[k] = (R)f2_to_double(lane(K[k >> 1], k & 1));
                }
                emit(tgt, mir, R(0), R(0), ae);
            }
            return;
        }
    }

    for (int j = threadIdx.x; j < ns; j += blockDim.x) {
        const int p0 = SP[j] - c0, p1 = SP[j + 1] - c0;
        const int32_t tgt = __ldcs(P.slot_target + s0 + j), mir = __ldcs(P.slot_mirror + s0 + j);
        R ad = 0, am = 0;
        R ae[HH];
#pragma unroll
        for (int k = 0; k < HH; ++k) ae[k] = 0;
        for (int p = p0; p < p1; ++p) {
            const int code = CT[p];
            const int idx = code >> 1;
            if constexpr (DIFF) ad += LD[idx];
            if constexpr (MASS) {
                if constexpr (T::P1 != 0) {
                    const int el = idx / NL;
                    am += LM[el] * (R)mhl[idx - el * NL];
                } else {
                    am += LM[idx];
                }
            }
            if constexpr (ELAST) {
                [[maybe_unused]] R tmp[HH];
                const R* blk;
                if constexpr (T::P1 != 0) {
                    blk = LE + (size_t)idx * HH;
                } else {
                    // A = sum_q jw_q g_a g_b^T of (element, pair), then its block
                    const int el = idx / NL;
                    int pa, pb;
                    upper_pair<B>(idx - el * NL, pa, pb);
                    R A[D][D];
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = 0; c < D; ++c) A[r][c] = 0;
                    for (int q = 0; q < Q; ++q) {
                        const R* g = G + (size_t)(el * Q + q) * B * D;
                        const R jw = JW[el * Q + q];
                        R t[D];
#pragma unroll
                        for (int c = 0; c < D; ++c) t[c] = jw * g[pb * D + c];
#pragma unroll
                        for (int r = 0; r < D; ++r) {
                            const R ar = g[pa * D + r];
#pragma unroll
                            for (int c = 0; c < D; ++c) A[r][c] += ar * t[c];
                        }
                    }
                    elastic_block_outer<R, D>(A, LE[2 * el], LE[2 * el + 1], tmp);
                    blk = tmp;
                }
                if (code & 1) {
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = 0; c < D; ++c) ae[r * D + c] += blk[c * D + r];
                } else {
#pragma unroll
                    for (int k = 0; k < HH; ++k) ae[k] += blk[k];
                }
            }
        }
        emit(tgt, mir, ad, am, ae);
    }
}

// sum the partials of the targets shared by several chunks, in chunk order
template <typename R, int ET, int FORMS>
__global__ void __launch_bounds__(kThreads) k_matrix_finalize(const tm_matrix_args a) {
    constexpr int D = Traits<ET>::D;
    constexpr bool DIFF = (FORMS & TM_FORM_DIFFUSION) != 0;
    constexpr bool MASS = (FORMS & TM_FORM_MASS) != 0;
    constexpr bool ELAST = (FORMS & TM_FORM_ELASTICITY) != 0;
    constexpr int W = ELAST ? D * D : ((DIFF ? 1 : 0) + (MASS ? 1 : 0));
    // float64 scalar partials are summed in double-float arithmetic (FP32
    // pipes) and rounded once; a target with a partial outside the range in
    // which the split keeps 48 bits is summed in FP64
    constexpr bool DFSUM = std::is_same<R, double>::value && !ELAST;
    const tm_chunk_plan& P = a.plan;
    const R* part = static_cast<const R*>(a.workspace);
    R* oD = static_cast<R*>(a.out_diffusion);
    R* oM = static_cast<R*>(a.out_mass);
    R* oE = static_cast<R*>(a.out_elasticity);
    // launched as a programmatic dependent of k_matrix: wait for its results
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if constexpr (ELAST) {
        // a team of W lanes per shared target, lane k summing component k
        // over the target's partials (in chunk order, as one thread per
        // target would): a team's loads and stores cover W consecutive
        // values, 32 / W teams per warp
        constexpr int TPW = 32 / W;
        const int lane = threadIdx.x & 31, team = lane / W, k = lane - team * W;
        const int r = k / D, c = k - r * D;
        const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
        if (team >= TPW) return;
        for (int64_t sh = warp * TPW + team; sh < P.n_shared; sh += nwarp * TPW) {
            const int q0 = P.shared_ptr[sh], q1 = P.shared_ptr[sh + 1];
            const int64_t tgt = P.shared_target[sh], mir = P.shared_mirror[sh];
            R acc = 0;
            for (int q = q0; q < q1; ++q) acc += __ldcs(part + (int64_t)q * W + k);
            oE[tgt * W + k] = acc;
            if (mir != tgt) oE[mir * W + c * D + r] = acc;
        }
        return;
    }
    for (int64_t sh = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sh < P.n_shared;
         sh += (int64_t)gridDim.x * blockDim.x) {
        const int q0 = P.shared_ptr[sh], q1 = P.shared_ptr[sh + 1];
        const int64_t tgt = P.shared_target[sh], mir = P.shared_mirror[sh];
        R acc[W];
        bool done = false;
        if constexpr (DFSUM) {
            f2 acc2[W];
            bool ok = true;
#pragma unroll
            for (int k = 0; k < W; ++k) acc2[k] = f2_make(0.0f, 0.0f);
            for (int q = q0; q < q1; ++q)
#pragma unroll
                for (int k = 0; k < W; ++k) {
                    const double x = __ldcg(reinterpret_cast<const double*>(part) + (int64_t)q * W + k);
                    const int e = biased_exponent(x);
                    ok &= x == 0.0 || (e >= 1023 - 78 && e < 1023 + 120);
                    acc2[k] = f2_add(acc2[k], split_double(x));
                }
            if (ok) {
#pragma unroll
                for (int k = 0; k < W; ++k) acc[k] = (R)f2_to_double(acc2[k]);
                done = true;
            }
        }
        if (!done) {
#pragma unroll
            for (int k = 0; k < W; ++k) acc[k] = 0;
            for (int q = q0; q < q1; ++q)
#pragma unroll
                for (int k = 0; k < W; ++k) acc[k] += part[(int64_t)q * W + k];
        }
        if constexpr (ELAST) {
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    oE[tgt * W + r * D + c] = acc[r * D + c];
                    if (mir != tgt) oE[mir * W + c * D + r] = acc[r * D + c];
                }
        } else {
            if constexpr (DIFF) {
                oD[tgt] = acc[0];
                if (mir != tgt) oD[mir] = acc[0];
            }
            if constexpr (MASS) {
                oM[tgt] = acc[W - 1];
                if (mir != tgt) oM[mir] = acc[W - 1];
            }
        }
    }
}

// ---------------------------------------------------------------- vectors
struct VecLayout {
    size_t tab, lv, total;
};
template <typename R, int ET, int W>
__host__ __device__ inline VecLayout vec_layout(int CH, int Q) {
    using T = Traits<ET>;
    VecLayout L;
    L.tab = 0;
    L.lv = align16(sizeof(double) * table_layout(Q, T::B, T::D).total);
    L.total = align16(L.lv + sizeof(R) * CH * T::B * W);
    return L;
}

template <typename R, int ET, int SRC, int W>
__global__ void __launch_bounds__(kThreads) k_vector(const tm_vector_args a) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems, Q = a.tables.n_quad;
    const VecLayout L = vec_layout<R, ET, W>(CH, Q);
    const TableLayout TL = table_layout(Q, B, D);
    extern __shared__ __align__(16) unsigned char sm[];
    double* tab = reinterpret_cast<double*>(sm + L.tab);
    R* LV = reinterpret_cast<R*>(sm + L.lv);
    for (int k = threadIdx.x; k < TL.total; k += blockDim.x) tab[k] = a.tables.packed[k];
    __syncthreads();

    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const R* pts = static_cast<const R*>(a.points);
    const R* val = static_cast<const R*>(a.values);
    for (int el = threadIdx.x; el < ne; el += blockDim.x) {
        const int64_t i = i0 + el;
        const int64_t e = P.elem_perm[i];
        int32_t c[B];
        R X[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            c[b] = P.conn[i * B + b];
#pragma unroll
            for (int d = 0; d < D; ++d) X[b][d] = ldg(pts + (int64_t)c[b] * D + d);
        }
        R acc[B][W];
#pragma unroll
        for (int p = 0; p < B; ++p)
#pragma unroll
            for (int w = 0; w < W; ++w) acc[p][w] = 0;
        if constexpr (T::P1 != 0) {
            R Xs[D + 1][D], C[D + 1][D];
#pragma unroll
            for (int b = 0; b <= D; ++b)
#pragma unroll
                for (int d = 0; d < D; ++d) Xs[b][d] = X[b][d];
            const R adet = rabs(p1_gradients<R, D>(Xs, C));
#pragma unroll
            for (int p = 0; p < B; ++p)
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    R s = 0;
                    if constexpr (SRC == TM_SOURCE_NODAL) {
#pragma unroll
                        for (int b = 0; b < B; ++b) s += (R)tab[TL.mhat + p * B + b] * ldg(val + (int64_t)c[b] * W + w);
                    } else if constexpr (SRC == TM_SOURCE_CONST) {
                        s = (R)tab[TL.lhat + p] * (R)a.constant[w];
                    } else {
                        for (int q = 0; q < Q; ++q)
                            s += (R)tab[TL.w + q] * (R)tab[TL.phi + q * B + p] * ldg(val + (e * Q + q) * W + w);
                    }
                    acc[p][w] = adet * s;
                }
        } else {
            for (int q = 0; q < Q; ++q) {
                const double* dphi = tab + TL.dphi + q * D * B;
                const double* phi = tab + TL.phi + q * B;
                R J[D][D];
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int cc = 0; cc < D; ++cc) {
                        R s = 0;
#pragma unroll
                        for (int b = 0; b < B; ++b) s += (R)dphi[r * B + b] * X[b][cc];
                        J[r][cc] = s;
                    }
                R cof[D][D];
                const R jxw = (R)tab[TL.w + q] * rabs(cofactors<R>(J, cof));
                R fq[W];
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    if constexpr (SRC == TM_SOURCE_NODAL) {
                        R s = 0;
#pragma unroll
                        for (int b = 0; b < B; ++b) s += ldg(val + (int64_t)c[b] * W + w) * (R)phi[b];
                        fq[w] = s;
                    } else if constexpr (SRC == TM_SOURCE_CONST) {
                        fq[w] = (R)a.constant[w];
                    } else {
                        fq[w] = ldg(val + (e * Q + q) * W + w);
                    }
                }
#pragma unroll
                for (int p = 0; p < B; ++p)
#pragma unroll
                    for (int w = 0; w < W; ++w) acc[p][w] += jxw * (R)phi[p] * fq[w];
            }
        }
#pragma unroll
        for (int p = 0; p < B; ++p)
#pragma unroll
            for (int w = 0; w < W; ++w) LV[(el * B + p) * W + w] = acc[p][w];
    }
    __syncthreads();
    node_reduce<R, W>(P, LV, static_cast<R*>(a.out), a.workspace);
}

// ----------------------------------------------------- geometry, x at q
template <int ET>
__global__ void __launch_bounds__(kThreads) k_shape_grad_jxw(int64_t E, const int32_t* conn, const double* pts,
                                                            tm_element_tables tb, double* grad, double* jxw) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const int Q = tb.n_quad;
    const TableLayout TL = table_layout(Q, B, D);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < E * Q;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = k / Q;
        const int q = (int)(k - e * Q);
        const double* dphi = tb.packed + TL.dphi + q * D * B;
        double X[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int64_t node = conn[e * B + b];
#pragma unroll
            for (int d = 0; d < D; ++d) X[b][d] = ldg(pts + node * D + d);
        }
        double J[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int c = 0; c < D; ++c) {
                double s = 0;
#pragma unroll
                for (int b = 0; b < B; ++b) s += ldg(dphi + r * B + b) * X[b][c];
                J[r][c] = s;
            }
        double cof[D][D];
        const double det = cofactors<double>(J, cof);
        const double inv = 1.0 / det;
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
            for (int c = 0; c < D; ++c) {
                double s = 0;
#pragma unroll
                for (int r = 0; r < D; ++r) s += ldg(dphi + r * B + b) * cof[r][c];
                grad[(k * B + b) * D + c] = s * inv;
            }
        jxw[k] = ldg(tb.packed + TL.w + q) * fabs(det);
    }
}

template <typename R, int ET>
__global__ void __launch_bounds__(kThreads) k_quadrature_points(int64_t E, const int32_t* conn, const R* pts,
                                                               tm_element_tables tb, R* xq) {
    using T = Traits<ET>;
    constexpr int D = T::D, B = T::B;
    const int Q = tb.n_quad;
    const TableLayout TL = table_layout(Q, B, D);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < E * Q;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = k / Q;
        const int q = (int)(k - e * Q);
        R x[D];
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = 0;
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int64_t node = conn[e * B + b];
            const R ph = (R)ldg(tb.packed + TL.phi + q * B + b);
#pragma unroll
            for (int d = 0; d < D; ++d) x[d] += ph * ldg(pts + node * D + d);
        }
#pragma unroll
        for (int d = 0; d < D; ++d) xq[k * D + d] = x[d];
    }
}

// ------------------------------------------------------------- projector
template <typename R>
__global__ void __launch_bounds__(kThreads) k_project(int64_t n_to, int64_t width, const int64_t* seg,
                                                     const int64_t* src, const R* x, R* out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_to * width;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = k / width, w = k - t * width;
        R s = 0;
        for (int64_t p = seg[t]; p < seg[t + 1]; ++p) s += x[src[p] * width + w];
        out[k] = s;
    }
}

inline int grid_for(int64_t work, int per_block = kThreads) {
    int64_t g = (work + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > 152 * 64) g = 152 * 64;
    return (int)g;
}

inline int launch_status(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

template <typename K>
inline int set_smem(K kernel, size_t bytes) {
    if (bytes > 48 * 1024) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
            return launch_status("cudaFuncSetAttribute");
    }
    return TM_OK;
}

// float64 diffusion / mass on P1 simplices: tm_p1df.cuh (included at the
// end of this header)
template <int ET, int FORMS>
int run_p1df(const tm_matrix_args& a, cudaStream_t st);
template <typename R, int ET, int FORMS>
int run_matrix_general(const tm_matrix_args& a, cudaStream_t st);

template <typename R, int ET, int FORMS>
int run_matrix(const tm_matrix_args& a, cudaStream_t st) {
    if constexpr (use_df64<R, ET, FORMS>()) {
        return run_p1df<ET, FORMS>(a, st);
    } else {
        return run_matrix_general<R, ET, FORMS>(a, st);
    }
}

template <typename R, int ET, int FORMS>
int run_matrix_general(const tm_matrix_args& a, cudaStream_t st) {
    const MatLayout L = mat_layout<R, ET, FORMS>(a.plan.chunk_elems, a.tables.n_quad, a.plan.max_chunk_slots,
                                                 a.plan.max_chunk_contrib);
    if (L.total > 227 * 1024) return tm_set_error(TM_ERR_TOO_LARGE, "tm_assemble_matrix: chunk needs more than 227 KB of shared memory");
    if (a.plan.n_chunks == 0) return TM_OK;
    int s = set_smem(k_matrix<R, ET, FORMS>, L.total);
    if (s) return s;
    if (a.event_begin && cudaEventRecord(static_cast<cudaEvent_t>(a.event_begin), st) != cudaSuccess)
        return launch_status("cudaEventRecord");
    k_matrix<R, ET, FORMS><<<a.plan.n_chunks, matrix_threads<R, ET, FORMS>(), L.total, st>>>(a);
    if ((s = launch_status("k_matrix"))) return s;
    if (a.event_end && cudaEventRecord(static_cast<cudaEvent_t>(a.event_end), st) != cudaSuccess)
        return launch_status("cudaEventRecord");
    if (a.plan.n_shared > 0) {
        // programmatic dependent launch: the finalising grid is scheduled
        // while k_matrix drains and waits (griddepcontrol.wait) for its
        // results; not when an event separates the two launches
        cudaLaunchConfig_t cfg = {};
        // (block forms: a team of D x D lanes per shared target, 32 / (D x D)
        // teams per warp)
        constexpr int DD = Traits<ET>::D * Traits<ET>::D;
        const int64_t fin_threads = (FORMS & TM_FORM_ELASTICITY)
                                        ? (a.plan.n_shared + 32 / DD - 1) / (32 / DD) * 32
                                        : a.plan.n_shared;
        cfg.gridDim = dim3(grid_for(fin_threads));
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = a.event_end ? 0 : 1;
        if (cudaLaunchKernelEx(&cfg, k_matrix_finalize<R, ET, FORMS>, a) != cudaSuccess)
            return launch_status("k_matrix_finalize");
        if ((s = launch_status("k_matrix_finalize"))) return s;
    }
    if (a.event_done && cudaEventRecord(static_cast<cudaEvent_t>(a.event_done), st) != cudaSuccess)
        return launch_status("cudaEventRecord");
    return TM_OK;
}

template <typename R, int ET>
int dispatch_forms(const tm_matrix_args& a, cudaStream_t st) {
    switch (a.forms) {
        case TM_FORM_DIFFUSION: return run_matrix<R, ET, TM_FORM_DIFFUSION>(a, st);
        case TM_FORM_MASS: return run_matrix<R, ET, TM_FORM_MASS>(a, st);
        case TM_FORM_DIFFUSION | TM_FORM_MASS: return run_matrix<R, ET, TM_FORM_DIFFUSION | TM_FORM_MASS>(a, st);
        case TM_FORM_ELASTICITY: return run_matrix<R, ET, TM_FORM_ELASTICITY>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix: unsupported form combination");
    }
}

template <typename R, int ET, int SRC, int W>
int run_vector(const tm_vector_args& a, cudaStream_t st) {
    const VecLayout L = vec_layout<R, ET, W>(a.plan.chunk_elems, a.tables.n_quad);
    if (L.total > 227 * 1024) return tm_set_error(TM_ERR_TOO_LARGE, "tm_assemble_vector: chunk needs more than 227 KB of shared memory");
    if (cudaMemsetAsync(a.out, 0, sizeof(R) * a.n_points * W, st) != cudaSuccess)
        return launch_status("cudaMemsetAsync");
    if (a.plan.n_chunks == 0) return TM_OK;
    if (a.plan.n_shared > 0) {
        void* counters = static_cast<unsigned char*>(a.workspace) + align16(sizeof(R) * W * (size_t)a.plan.n_partials);
        if (cudaMemsetAsync(counters, 0, sizeof(int32_t) * (size_t)a.plan.n_shared, st) != cudaSuccess)
            return launch_status("cudaMemsetAsync");
    }
    int s = set_smem(k_vector<R, ET, SRC, W>, L.total);
    if (s) return s;
    k_vector<R, ET, SRC, W><<<a.plan.n_chunks, kThreads, L.total, st>>>(a);
    return launch_status("k_vector");
}

template <typename R, int ET, int SRC>
int dispatch_width(const tm_vector_args& a, cudaStream_t st) {
    switch (a.width) {
        case 1: return run_vector<R, ET, SRC, 1>(a, st);
        case 2: return run_vector<R, ET, SRC, 2>(a, st);
        case 3: return run_vector<R, ET, SRC, 3>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_vector: width must be 1..3");
    }
}

template <typename R, int ET>
int dispatch_source(const tm_vector_args& a, cudaStream_t st) {
    switch (a.source) {
        case TM_SOURCE_NODAL: return dispatch_width<R, ET, TM_SOURCE_NODAL>(a, st);
        case TM_SOURCE_CONST: return dispatch_width<R, ET, TM_SOURCE_CONST>(a, st);
        case TM_SOURCE_QUAD: return dispatch_width<R, ET, TM_SOURCE_QUAD>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_vector: unknown source kind");
    }
}

}  // namespace tmk

#include "tm_p1df.cuh"
