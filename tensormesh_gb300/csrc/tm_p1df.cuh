// Float64 diffusion and mass assembly on P1 simplices (3-node triangles,
// 4-node tetrahedra) in paired double-float arithmetic: the path of the
// P1-tet benchmark (K(kappa) and M of a jittered Kuhn-split cube).
//
// The reference computes per element J, J^-1, det J, the integrand
// kappa gradu.gradv |det J| w at each quadrature point and the quadrature
// sum (element/element.py:875-968, element/transformation.py:1219-1276,
// assemble/element_assembler.py:190-209, 390-445), then index_add_'s the
// locals into the CSR values (assemble/projector.py:95-123).  On a P1
// simplex the gradients are constant, so the stiffness local is
//     K_e[a][b] = kappa_e W / |det| * C_a . C_b,
// C_a the cofactor rows of J (C_0 = -sum of the others) and W the sum of the
// quadrature weights, and the mass local is |det| rho M^[a][b] with M^ the
// reference template.  This kernel evaluates exactly that, to about 2^-46
// relative, in double-float arithmetic on the FP32 pipes (FP64 runs at 1/62
// of the FP32 rate on GB300).
//
// One CTA per chunk of the plan (Morton-ordered elements):
//  * phase 0: one thread issues the bulk copies of the chunk's slot_ptr and
//    contrib windows into shared memory (they land during phase 1);
//  * phase 1: each thread takes NE elements (NE = 2: elements e and e + NT
//    through paired double-float instructions, one lane per element, at most
//    384 threads; NE = 1: one element per thread, at most 768 threads and
//    about half the registers, so twice the resident warps): the coordinate
//    differences (one FP64 subtraction each, then split on the integer
//    pipe), cofactors, determinant, the Gram entries C_a . C_b, the scale
//    kappa W / |det| and the scaled locals K_e[a][b] (upper triangle), and
//    |det| rho; both go to shared memory as hi/lo float pairs, one record of
//    NL + 1 pairs per element;
//  * phase 2: one thread per target (CSR position) of the chunk, targets
//    ordered by contribution count so that a warp's loops are equally long,
//    sums its contributions in element order: the stiffness sum in lane x and
//    the sum of |det| rho in lane y of one paired TwoSum (a CSR position
//    receives only diagonal or only off-diagonal local entries, so its mass
//    is the template value of its class times that sum).  Targets of one
//    chunk are written to their CSR position and its mirror; a target
//    shared with other chunks writes a float64 partial that
//    k_p1df_finalize sums in chunk order.
// The plan alone fixes every summation order: results are bitwise
// reproducible.  A chunk whose data leave the double-float range (an edge
// component scale outside [2^-20, 2^20], kappa outside [2^-30, 2^30],
// |det| rho or a local's scale outside [2^-80, 2^100], a mass template that
// is not two-valued to 1e-14) runs the whole chunk in FP64 arithmetic instead
// (tm_matrix_args.stats counts those chunks).
#pragma once
#include <algorithm>

#include "tm_df2.cuh"

namespace tmk {

// most threads of a k_p1df CTA for NE elements per thread
template <int NE>
__host__ __device__ constexpr int p1_threads() { return NE == 2 ? 384 : 768; }

struct P1Layout {
    size_t bar, sp, ct, rec, total;
};

// REC: per element a record of NL + 1 values of 8 bytes (a hi/lo float
// pair, or a double on the FP64 path): the scaled locals (upper triangle)
// and |det| rho.  The odd record stride (88 bytes for a tetrahedron) spreads
// a warp's stores over the banks.
template <int ET>
__host__ __device__ inline P1Layout p1_layout(int CH, int MS, int MC) {
    constexpr int B = Traits<ET>::B, NL = B * (B + 1) / 2;
    P1Layout L;
    size_t o = 0;
    L.bar = o;
    o += 16;
    L.sp = o;
    o += stage_capacity((int64_t)MS + 1, 4);
    L.ct = o;
    o += stage_capacity(MC, 2);
    o = align16(o);
    L.rec = o;
    o = align16(o + 8 * (size_t)CH * (NL + 1));
    L.total = o;
    return L;
}

// L2 policy that keeps lines (evict_last) and stores under it
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void st_keep(double* p, double v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_keep2(double* p, double x, double y, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(x), "d"(y), "l"(pol) : "memory");
}

// largest biased double exponent among the components (their scale)
__device__ __forceinline__ uint32_t exp_field(double x) {
    return ((uint32_t)__double2hiint(x) >> 20) & 0x7FFu;
}

template <int ET, int FORMS, int NE>
__global__ void __launch_bounds__(p1_threads<NE>(), 2) k_p1df(const tm_matrix_args a) {
    using T = Traits<ET>;
    using Ln = typename std::conditional<NE == 2, float2, float>::type;   // lane type
    using V = ddv<Ln>;
    constexpr int D = T::D, B = T::B, NL = B * (B + 1) / 2, NR = NL + 1;
    const int NT = blockDim.x;
    constexpr bool DIFF = (FORMS & TM_FORM_DIFFUSION) != 0;
    constexpr bool MASS = (FORMS & TM_FORM_MASS) != 0;
    const tm_chunk_plan& P = a.plan;
    const int CH = P.chunk_elems;
    const P1Layout L = p1_layout<ET>(CH, P.max_chunk_slots, P.max_chunk_contrib);
    extern __shared__ __align__(16) unsigned char sm[];

    // the finalising grid may be scheduled once every chunk has started
    asm volatile("griddepcontrol.launch_dependents;");

    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L.bar);
    const int32_t s0 = P.chunk_begin[blockIdx.x], s1 = P.chunk_begin[blockIdx.x + 1];
    const int32_t c0 = P.chunk_contrib[blockIdx.x], c1 = P.chunk_contrib[blockIdx.x + 1];
    const StageRange w_sp = stage_range(s0, (int64_t)s1 + 1, 4);
    const StageRange w_ct = stage_range(c0, c1, 2);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_arrive_expect_tx(bar, w_sp.bytes + w_ct.bytes);
        bulk_copy_g2s(sm + L.sp, reinterpret_cast<const unsigned char*>(P.slot_ptr) + w_sp.begin, w_sp.bytes, bar);
        if (w_ct.bytes)
            bulk_copy_g2s(sm + L.ct, reinterpret_cast<const unsigned char*>(P.contrib) + w_ct.begin, w_ct.bytes, bar);
    }
    const int32_t* SP = reinterpret_cast<const int32_t*>(sm + L.sp) + w_sp.skip;   // slot_ptr[s0 + j]
    const uint16_t* CT = reinterpret_cast<const uint16_t*>(sm + L.ct) + w_ct.skip;  // contrib[c0 + q]
    float2* REC = reinterpret_cast<float2*>(sm + L.rec);
    double* RECd = reinterpret_cast<double*>(sm + L.rec);

    // per-CTA constants: the mass template's two class values (diagonal and
    // off-diagonal entries) and whether the template has that structure
    __shared__ struct {
        double m_diag, m_off;
    } cta;
    const TableLayout TL = table_layout(a.tables.n_quad, B, D);
    const double* pk = a.tables.packed;
    // thread 0 checks the tables; the other threads start their element
    // loads at once (the constants are read after the barrier that ends
    // phase 1, and thread 0's verdict joins that barrier's vote)
    bool bad = false;
    if (threadIdx.x == 0) {
        int tbad = !exponent_in_band(a.kappa_scale, 30) || !exponent_in_band(a.mass_scale, 30) ||
                   !exponent_in_band(pk[TL.wsum], 30);
        const double md = MASS ? pk[TL.mhat] : 0.0, mo = MASS && B > 1 ? pk[TL.mhat + 1] : 0.0;
        if (MASS) {
            // a symmetric quadrature rule gives one diagonal and one
            // off-diagonal value, up to the rounding of the sums that
            // tabulated them (entries of one class differ in the last bits)
            tbad |= !exponent_in_band(md, 30) || !exponent_in_band(mo, 30);
            for (int pa = 0; pa < B; ++pa)
                for (int pb = 0; pb < B; ++pb) {
                    const double m = pk[TL.mhat + pa * B + pb], c = pa == pb ? md : mo;
                    tbad |= !(fabs(m - c) <= 1e-14 * fabs(c));
                }
        }
        cta.m_diag = md;
        cta.m_off = mo;
        bad = tbad != 0;
    }

    const int64_t i0 = (int64_t)blockIdx.x * CH;
    const int ne = (int)min((int64_t)CH, P.n_elements - i0);
    const double* pts = static_cast<const double*>(a.points);
    const double* kap = static_cast<const double*>(a.kappa);
    float ks_h, ks_l, ms_h, ms_l, ws_h, ws_l;
    split_to_pair(a.kappa_scale, ks_h, ks_l);
    split_to_pair(a.mass_scale, ms_h, ms_l);
    split_to_pair(pk[TL.wsum], ws_h, ws_l);

    // ---------------------------------------------------------------- phase 1
    for (int base = 0; base < ne; base += NE * NT) {
        int el[NE];
        bool has[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            el[k] = base + threadIdx.x + k * NT;
            has[k] = el[k] < ne;
        }
        if (!has[0]) break;
#pragma unroll
        for (int k = 1; k < NE; ++k)
            if (!has[k]) el[k] = el[0];              // a copy of element 0 fills the lane, unstored
        int nd[NE][B];
        if constexpr (B == 4) {
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                const int4 c = __ldcs(reinterpret_cast<const int4*>(P.conn) + i0 + el[k]);
                nd[k][0] = c.x, nd[k][1] = c.y, nd[k][2] = c.z, nd[k][3] = c.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < NE; ++k)
#pragma unroll
                for (int b = 0; b < B; ++b) nd[k][b] = __ldcs(P.conn + (i0 + el[k]) * B + b);
        }
        double kv[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) kv[k] = (DIFF && kap) ? __ldg(kap + __ldcs(P.elem_perm + i0 + el[k])) : 1.0;
        double X[NE][B][D];
#pragma unroll
        for (int k = 0; k < NE; ++k)
#pragma unroll
            for (int b = 0; b < B; ++b)
#pragma unroll
                for (int d = 0; d < D; ++d) X[k][b][d] = __ldg(pts + (int64_t)nd[k][b] * D + d);
        // J[r][c] = x_{r+1,c} - x_{0,c}: the one FP64 step, then split
        V J[D][D];
        uint32_t emax[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) emax[k] = 0;
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int c = 0; c < D; ++c)
#pragma unroll
                for (int k = 0; k < NE; ++k) {
                    const double dd = X[k][r + 1][c] - X[k][0][c];
                    emax[k] = max(emax[k], exp_field(dd));
                    float h, l;
                    split_to_pair(dd, h, l);
                    l_put(J[r][c].hi, k, h);
                    l_put(J[r][c].lo, k, l);
                }
#pragma unroll
        for (int k = 0; k < NE; ++k) bad |= emax[k] < 1023 - 20 || emax[k] >= 1023 + 20;
        V cof[D][D];
        V det;
        if constexpr (D == 3) {
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const int r1 = (r + 1) % 3, r2 = (r + 2) % 3;
                cof[r][0] = p_diff_of_products(J[r1][1], J[r2][2], J[r1][2], J[r2][1]);
                cof[r][1] = p_diff_of_products(J[r1][2], J[r2][0], J[r1][0], J[r2][2]);
                cof[r][2] = p_diff_of_products(J[r1][0], J[r2][1], J[r1][1], J[r2][0]);
            }
            det = p_dot3(J[0], cof[0]);
        } else {
            cof[0][0] = J[1][1];
            cof[0][1] = p_neg(J[1][0]);
            cof[1][0] = p_neg(J[0][1]);
            cof[1][1] = J[0][0];
            det = p_diff_of_products(J[0][0], J[1][1], J[0][1], J[1][0]);
        }
        const V adet = p_abs(det);
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const float ad = l_get(adet.hi, k);
            bad |= !f2_in_band({ad, 0.0f}, -100, 100) || !(ad > 0.0f);
        }
        if constexpr (DIFF) {
#pragma unroll
            for (int k = 0; k < NE; ++k) bad |= !exponent_in_band(kv[k], 30);
            // Gram entries of the cofactor rows; C_0 = -sum_r cof_r gives
            // C_0.C_0 = sum_rc G_rc and C_0.C_{c+1} = -sum_r G_rc
            V G[D][D];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = r; c < D; ++c) {
                    G[r][c] = D == 3 ? p_dot3(cof[r], cof[c]) : p_dot2(cof[r], cof[c]);
                    G[c][r] = G[r][c];
                }
            V rs[D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                V acc = G[0][c];
#pragma unroll
                for (int r = 1; r < D; ++r) acc = p_add(acc, G[r][c]);
                rs[c] = acc;
            }
            V tot = rs[0];
#pragma unroll
            for (int c = 1; c < D; ++c) tot = p_add(tot, rs[c]);
            // scale kappa * kappa_scale * W / |det|
            V kd;
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                float h, l;
                split_to_pair(kv[k], h, l);
                l_put(kd.hi, k, h);
                l_put(kd.lo, k, l);
            }
            const V sc = p_mul(p_mul(kd, p_const<Ln>(ks_h, ks_l)), p_mul(p_const<Ln>(ws_h, ws_l), p_recip(adet)));
            // largest local: the diagonal entries; its exponent with the
            // scale's must keep every product a normal float
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                float g = fabsf(l_get(tot.hi, k));
#pragma unroll
                for (int c = 0; c < D; ++c) g = fmaxf(g, fabsf(l_get(G[c][c].hi, k)));
                const float sh = l_get(sc.hi, k);
                const int le = (int)((__float_as_uint(g) >> 23) & 0xFF) + (int)((__float_as_uint(sh) >> 23) & 0xFF) - 254;
                bad |= le < -80 || le >= 100 || !isfinite(sh);
            }
            V kl[NL];
            int l = 0;
            kl[l++] = p_mul(sc, tot);
#pragma unroll
            for (int q = 0; q < D; ++q) kl[l++] = p_neg(p_mul(sc, rs[q]));
#pragma unroll
            for (int p = 0; p < D; ++p)
#pragma unroll
                for (int q = p; q < D; ++q) kl[l++] = p_mul(sc, G[p][q]);
#pragma unroll
            for (int k = 0; k < NE; ++k)
                if (has[k])
#pragma unroll
                    for (int m = 0; m < NL; ++m)
                        REC[el[k] * NR + m] = make_float2(l_get(kl[m].hi, k), l_get(kl[m].lo, k));
        }
        if constexpr (MASS) {
            const V v = p_mul(adet, p_const<Ln>(ms_h, ms_l));
#pragma unroll
            for (int k = 0; k < NE; ++k) {
                bad |= !f2_in_band({l_get(v.hi, k), 0.0f}, -80, 100);
                if (has[k]) REC[el[k] * NR + NL] = make_float2(l_get(v.hi, k), l_get(v.lo, k));
            }
        }
    }
    const bool use_df = !__syncthreads_or(bad);
    if (!use_df) {
        // FP64 arithmetic for the whole chunk: the locals as doubles in the
        // same shared-memory slots
        if (threadIdx.x == 0 && a.stats) atomicAdd(a.stats, 1);
        const double wsum = pk[TL.wsum];
        for (int el = threadIdx.x; el < ne; el += NT) {
            const int64_t i = i0 + el;
            double X[B][D];
#pragma unroll
            for (int k = 0; k < B; ++k) {
                const int64_t node = P.conn[i * B + k];
#pragma unroll
                for (int d = 0; d < D; ++d) X[k][d] = pts[node * D + d];
            }
            double C[B][D];
            const double det = p1_gradients<double, D>(X, C);
            const double adet = det < 0.0 ? -det : det;
            if constexpr (DIFF) {
                const double kv = (kap ? kap[P.elem_perm[i]] : 1.0) * a.kappa_scale;
                const double s = kv * wsum / adet;
                int l = 0;
#pragma unroll
                for (int p = 0; p < B; ++p)
#pragma unroll
                    for (int q = p; q < B; ++q, ++l) RECd[el * NR + l] = s * dot<double, D>(C[p], C[q]);
            }
            if constexpr (MASS) RECd[el * NR + NL] = adet * a.mass_scale;
        }
        __syncthreads();
    }

    // the staged plan must have landed; a wait that runs out flags the
    // device and leaves the chunk unwritten
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0, kStageTries))) {
        if (threadIdx.x == 0) atomicExch(&g_device_fault, 1);
        mbar_wait_bounded(bar, 0, kStageTries);      // copies in flight end before the CTA does
        return;
    }

    // ---------------------------------------------------------------- phase 2
    constexpr int WP = (DIFF ? 1 : 0) + (MASS ? 1 : 0);   // float64 values per partial
    // upper-triangle entries l that are diagonal (a, a)
    constexpr unsigned kDiag = B == 4 ? (1u | 1u << 4 | 1u << 7 | 1u << 9) : (1u | 1u << 3 | 1u << 5);
    const int ns = s1 - s0;
    double* oD = static_cast<double*>(a.out_diffusion);
    double* oM = static_cast<double*>(a.out_mass);
    double* part = static_cast<double*>(a.workspace);
    auto emit = [&](int32_t tgt, int32_t mir, double kd, double md) {
        if (tgt >= 0) {
            if constexpr (DIFF) {
                oD[tgt] = kd;
                if (mir != tgt) oD[mir] = kd;
            }
            if constexpr (MASS) {
                oM[tgt] = md;
                if (mir != tgt) oM[mir] = md;
            }
        } else {
            // partials stay in L2 for the finalising grid
            const int64_t pi = -(int64_t)tgt - 1;
            const uint64_t pol = l2_keep_policy();
            if constexpr (WP == 2)
                st_keep2(part + 2 * pi, kd, md, pol);
            else
                st_keep(part + pi, DIFF ? kd : md, pol);
        }
    };

    if (use_df) {
        float mdh = 0.0f, mdl = 0.0f, moh = 0.0f, mol = 0.0f;
        if constexpr (MASS) {
            split_to_pair(cta.m_diag, mdh, mdl);
            split_to_pair(cta.m_off, moh, mol);
        }
        for (int j = threadIdx.x; j < ns; j += NT) {
            const int p0 = SP[j] - c0, p1 = SP[j + 1] - c0;
            const int32_t tgt = __ldcs(P.slot_target + s0 + j), mir = __ldcs(P.slot_mirror + s0 + j);
            // lane x: the stiffness sum, lane y: the sum of |det| rho; TwoSum
            // on the leading parts, the error terms and low parts summed
            float2 acc = make_float2(0.0f, 0.0f), err = make_float2(0.0f, 0.0f);
            // unrolled so that the next contributions' loads issue early
#pragma unroll 4
            for (int p = p0; p < p1; ++p) {
                const unsigned idx = (unsigned)CT[p] >> 1;
                const unsigned e = idx / (unsigned)NL;       // record e, entry idx - e NL
                const float2 kv = DIFF ? REC[idx + e] : make_float2(0.0f, 0.0f);
                const float2 mv = MASS ? REC[e * NR + NL] : make_float2(0.0f, 0.0f);
                const pf2 t = p_two_sum(acc, make_float2(kv.x, mv.x));
                acc = t.hi;
                err = l_add(err, l_add(t.lo, make_float2(kv.y, mv.y)));
            }
            const pf2 r = p_fast_two_sum(acc, err);
            double kd = 0.0, md = 0.0;
            if constexpr (DIFF) kd = pair_to_double(r.hi.x, r.lo.x);
            if constexpr (MASS) {
                // the class of the target's first contribution (all share it)
                const unsigned idx = (unsigned)CT[p0] >> 1;
                const unsigned l = idx - (idx / (unsigned)NL) * (unsigned)NL;
                const bool dg = (kDiag >> l) & 1u;
                const f2 m = f2_mul(f2_make(r.hi.y, r.lo.y), f2_make(dg ? mdh : moh, dg ? mdl : mol));
                md = pair_to_double(m.hi, m.lo);
            }
            emit(tgt, mir, kd, md);
        }
        return;
    }

    // FP64 path: the template per local entry
    __shared__ double mhl[NL];
    if (MASS && threadIdx.x < NL) {
        int pa, pb;
        upper_pair<B>(threadIdx.x, pa, pb);
        mhl[threadIdx.x] = pk[TL.mhat + pa * B + pb];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < ns; j += NT) {
        const int p0 = SP[j] - c0, p1 = SP[j + 1] - c0;
        const int32_t tgt = P.slot_target[s0 + j], mir = P.slot_mirror[s0 + j];
        double kd = 0.0, md = 0.0;
        for (int p = p0; p < p1; ++p) {
            const unsigned idx = (unsigned)CT[p] >> 1;
            const unsigned el = idx / (unsigned)NL;
            if constexpr (DIFF) kd += RECd[idx + el];
            if constexpr (MASS) md += RECd[el * NR + NL] * mhl[idx - el * (unsigned)NL];
        }
        emit(tgt, mir, kd, md);
    }
}

// sum the float64 partials of the targets shared by several chunks, in
// chunk order (FP64 adds: about two per target and form)
template <int FORMS>
__global__ void __launch_bounds__(kThreads) k_p1df_finalize(const tm_matrix_args a) {
    constexpr bool DIFF = (FORMS & TM_FORM_DIFFUSION) != 0;
    constexpr bool MASS = (FORMS & TM_FORM_MASS) != 0;
    constexpr int WP = (DIFF ? 1 : 0) + (MASS ? 1 : 0);
    const tm_chunk_plan& P = a.plan;
    const double* part = static_cast<const double*>(a.workspace);
    double* oD = static_cast<double*>(a.out_diffusion);
    double* oM = static_cast<double*>(a.out_mass);
    // launched as a programmatic dependent of k_p1df: wait for its results
    asm volatile("griddepcontrol.wait;" ::: "memory");
    for (int64_t sh = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sh < P.n_shared;
         sh += (int64_t)gridDim.x * blockDim.x) {
        const int q0 = __ldcs(P.shared_ptr + sh), q1 = __ldcs(P.shared_ptr + sh + 1);
        const int32_t tgt = __ldcs(P.shared_target + sh), mir = __ldcs(P.shared_mirror + sh);
        double kd = 0.0, md = 0.0;
        for (int q = q0; q < q1; ++q) {
            if constexpr (WP == 2) {
                const double2 v = __ldcs(reinterpret_cast<const double2*>(part) + q);
                kd += v.x;
                md += v.y;
            } else if constexpr (DIFF) {
                kd += __ldcs(part + q);
            } else {
                md += __ldcs(part + q);
            }
        }
        if constexpr (DIFF) {
            oD[tgt] = kd;
            if (mir != tgt) oD[mir] = kd;
        }
        if constexpr (MASS) {
            oM[tgt] = md;
            if (mir != tgt) oM[mir] = md;
        }
    }
}

}  // namespace tmk

namespace tmk {

// k_p1df, then (when the plan has shared targets) k_p1df_finalize as its
// programmatic dependent
template <int ET, int FORMS, int NE>
int run_p1df_ne(const tm_matrix_args& a, cudaStream_t st) {
    const P1Layout L = p1_layout<ET>(a.plan.chunk_elems, a.plan.max_chunk_slots, a.plan.max_chunk_contrib);
    if (L.total > 227 * 1024)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_assemble_matrix: chunk needs more than 227 KB of shared memory");
    if (Traits<ET>::B == 4 && (reinterpret_cast<uintptr_t>(a.plan.conn) & 15) != 0)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: plan.conn must start on a 16-byte boundary");
    if (a.plan.n_chunks == 0) return TM_OK;
    int s = set_smem(k_p1df<ET, FORMS, NE>, L.total);
    if (s) return s;
    if (a.event_begin && cudaEventRecord(static_cast<cudaEvent_t>(a.event_begin), st) != cudaSuccess)
        return launch_status("cudaEventRecord");
    // threads: enough for the chunk's elements (NE each), at most the bound
    const int want = (a.plan.chunk_elems + NE - 1) / NE;
    const int threads = std::min(p1_threads<NE>(), std::max(32, (want + 31) / 32 * 32));
    k_p1df<ET, FORMS, NE><<<a.plan.n_chunks, threads, L.total, st>>>(a);
    if ((s = launch_status("k_p1df"))) return s;
    if (a.event_end && cudaEventRecord(static_cast<cudaEvent_t>(a.event_end), st) != cudaSuccess)
        return launch_status("cudaEventRecord");
    if (a.plan.n_shared > 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid_for(a.plan.n_shared));
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = a.event_end ? 0 : 1;
        if (cudaLaunchKernelEx(&cfg, k_p1df_finalize<FORMS>, a) != cudaSuccess)
            return launch_status("k_p1df_finalize");
        if ((s = launch_status("k_p1df_finalize"))) return s;
    }
    if (a.event_done && cudaEventRecord(static_cast<cudaEvent_t>(a.event_done), st) != cudaSuccess)
        return launch_status("cudaEventRecord");
    return TM_OK;
}

// two elements per thread on the paired FP32 instructions: 28 % fewer
// issued instructions per element than one element per thread (whose twice
// as many resident warps do not make up for them: pass 0.136 against
// 0.144 ms on 1.57 M tets)
template <int ET, int FORMS>
int run_p1df(const tm_matrix_args& a, cudaStream_t st) {
    return run_p1df_ne<ET, FORMS, 2>(a, st);
}

}  // namespace tmk
