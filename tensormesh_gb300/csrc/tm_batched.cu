// Batched Jacobi-PCG over the diagonal blocks of one block-diagonal CSR
// matrix: many independent SPD systems of uneven sizes (offset-concatenated
// meshes) solved in one launch.
//
// The reference has no batched varying-mesh solve: it builds, assembles,
// condenses and solves one mesh after another
// (docs/source/user_guide/batched_workflows.rst:247-249), with Jacobi-
// preconditioned Krylov loops of torch SpMVs as its in-tree templates
// (sparse/solve/torch_solve.py:70-248).
//
// Persistent CTAs take systems from a queue (one integer counter, over an
// optional largest-first order) and run the whole PCG of a system with
// __syncthreads only: no grid-wide barrier, no waiting on other CTAs.  The
// batch time is set by its largest systems on one CTA each, so the loops
// keep several rows per thread in flight: the SpMV interleaves the loads of
// four rows, the vector updates load four elements before using them
// (measured on 512 uneven meshes: 79 ms per batch against 122 ms one row at
// a time).  Every loop is bounded by max_iter.  Reductions are per thread
// in row order, then summed in a fixed order by one warp, so the result of
// a system does not depend on which CTA solved it.  (Keeping the search
// direction in shared memory instead measured slower, 93 ms against 79: it
// takes L1 capacity that the matrix and vector streams hit in.)  Dirichlet rows
// (dirichlet[i] != 0) keep x_i as given on input and are excluded from the
// iteration (p_i = r_i = 0), which solves the condensed system
// K_ii x_i = b_i - K_io x_o without extracting K_ii.
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>
#include <type_traits>

#include "../../include/tensormesh_gb300.h"
#include "tm_status.h"

namespace tmk {

constexpr int kBatchThreads = 512;

// butterfly sum over the 32 lanes of a warp (both lanes of a pair add the
// same two operands, so every lane ends with the same value)
__device__ __forceinline__ double warp_sum(double s) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    return s;
}

// Fixed-order block sums of N values per thread: staged in shared memory
// (red: [N][kBatchThreads]) and summed by warp 0 alone, each lane a pairwise
// tree over its 16 entries, then a butterfly (float64 adds are scarce on this
// GPU: the other warps issue none); every thread returns the same sums
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double* red) {
    static_assert(kBatchThreads == 512, "block_sum sums 16 entries per lane of warp 0");
    __shared__ double res[N];
#pragma unroll
    for (int k = 0; k < N; ++k) red[k * kBatchThreads + threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const double* e = red + k * kBatchThreads + threadIdx.x;
            double t8[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) t8[j] = e[64 * j] + e[64 * j + 32];
            const double t = ((t8[0] + t8[1]) + (t8[2] + t8[3])) + ((t8[4] + t8[5]) + (t8[6] + t8[7]));
            const double w = warp_sum(t);
            if (threadIdx.x == 0) res[k] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = res[k];
}

template <typename R>
__global__ void __launch_bounds__(kBatchThreads) k_batched_pcg(const tm_batched_pcg_args a) {
    __shared__ double red[3 * kBatchThreads];
    __shared__ int sys_s;
    const int64_t* rp = a.A.row_ptr;
    const int32_t* col = a.A.col;
    const R* val = static_cast<const R*>(a.A.values);
    const R* b = static_cast<const R*>(a.b);
    R* x = static_cast<R*>(a.x);
    const int64_t n_all = a.A.n_rows;
    R* r = static_cast<R*>(a.work);
    R* z = r + n_all;
    R* p = z + n_all;
    R* q = p + n_all;
    R* dinv = q + n_all;
    const uint8_t* fixed = a.dirichlet;
    const double tol2 = a.rtol * a.rtol;
    for (;;) {
        if (threadIdx.x == 0) {
            const int k = atomicAdd(a.queue, 1);
            sys_s = k < a.n_systems ? (a.order ? a.order[k] : k) : a.n_systems;
        }
        __syncthreads();
        const int sys = sys_s;
        __syncthreads();
        if (sys >= a.n_systems) return;
        const int64_t r0 = a.system_offset[sys], r1 = a.system_offset[sys + 1];
        // start: r = b - A x on free rows, z = r / diag, p = z
        double v3[3] = {0.0, 0.0, 0.0};   // rz, rr, bb
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kBatchThreads) {
            if (fixed && fixed[i]) {
                r[i] = z[i] = p[i] = q[i] = dinv[i] = R(0);
                continue;
            }
            double ax = 0.0, d = 0.0;
            for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
                const int64_t c = col[k];
                const double v = (double)val[k];
                ax += v * (double)x[c];
                if (c == i) d += v;
            }
            const double ri = (double)b[i] - ax;
            const double di = d != 0.0 ? 1.0 / d : 0.0;
            const double zi = ri * di;
            dinv[i] = (R)di;
            r[i] = (R)ri;
            z[i] = (R)zi;
            p[i] = (R)zi;
            v3[0] += ri * zi;
            v3[1] += ri * ri;
            v3[2] += (double)b[i] * (double)b[i];
        }
        block_sum<3>(v3, red);
        double rz = v3[0], rr = v3[1];
        const double bb = v3[2];
        int it = 0, flag = 0;
        while (true) {
            if (rr <= tol2 * bb || bb == 0.0) {
                flag = TM_PCG_CONVERGED;
                break;
            }
            if (it >= a.max_iter) {
                flag = TM_PCG_MAX_ITER;
                break;
            }
            // q = A p, pq: four rows per thread at a time, their loads
            // interleaved (rows r, r + T, r + 2T, r + 3T), each row summed in
            // its entry order
            double v1[1] = {0.0};
            constexpr int RU = 4;
            for (int64_t i0 = r0 + threadIdx.x; i0 < r1; i0 += RU * kBatchThreads) {
                int64_t beg[RU], len[RU];
                int64_t maxlen = 0;
#pragma unroll
                for (int u = 0; u < RU; ++u) {
                    const int64_t i = i0 + (int64_t)u * kBatchThreads;
                    const bool on = i < r1 && !(fixed && fixed[i]);
                    beg[u] = on ? rp[i] : 0;
                    len[u] = on ? rp[i + 1] - beg[u] : 0;
                    maxlen = len[u] > maxlen ? len[u] : maxlen;
                }
                double s[RU] = {};
                for (int64_t k = 0; k < maxlen; ++k)
#pragma unroll
                    for (int u = 0; u < RU; ++u)
                        if (k < len[u]) s[u] += (double)val[beg[u] + k] * (double)p[col[beg[u] + k]];
#pragma unroll
                for (int u = 0; u < RU; ++u) {
                    const int64_t i = i0 + (int64_t)u * kBatchThreads;
                    if (i < r1 && !(fixed && fixed[i])) {
                        q[i] = (R)s[u];
                        v1[0] += (double)p[i] * s[u];
                    }
                }
            }
            block_sum<1>(v1, red);
            const double pq = v1[0];
            if (!(pq > 0.0)) {
                flag = TM_PCG_BREAKDOWN;
                break;
            }
            const double alpha = rz / pq;
            double v2[2] = {0.0, 0.0};
            for (int64_t i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * kBatchThreads) {
                double xv[4], pv[4], rv[4], qv[4], dv[4];
                bool on[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t i = i0 + (int64_t)u * kBatchThreads;
                    on[u] = i < r1 && !(fixed && fixed[i]);
                    if (on[u]) { xv[u] = (double)x[i]; pv[u] = (double)p[i]; rv[u] = (double)r[i]; qv[u] = (double)q[i]; dv[u] = (double)dinv[i]; }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (!on[u]) continue;
                    const int64_t i = i0 + (int64_t)u * kBatchThreads;
                    x[i] = (R)(xv[u] + alpha * pv[u]);
                    const double ri = rv[u] - alpha * qv[u];
                    r[i] = (R)ri;
                    const double zi = ri * dv[u];
                    z[i] = (R)zi;
                    v2[0] += ri * zi;
                    v2[1] += ri * ri;
                }
            }
            block_sum<2>(v2, red);
            const double beta = rz != 0.0 ? v2[0] / rz : 0.0;
            rz = v2[0];
            rr = v2[1];
            for (int64_t i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * kBatchThreads) {
                double zv[4], pv[4];
                bool on[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t i = i0 + (int64_t)u * kBatchThreads;
                    on[u] = i < r1 && !(fixed && fixed[i]);
                    if (on[u]) { zv[u] = (double)z[i]; pv[u] = (double)p[i]; }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (on[u]) p[i0 + (int64_t)u * kBatchThreads] = (R)(zv[u] + beta * pv[u]);
            }
            __syncthreads();
            ++it;
        }
        if (threadIdx.x == 0 && a.status) {
            a.status[sys].iterations = it;
            a.status[sys].flag = flag;
            a.status[sys].relative_residual = bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
        }
        __syncthreads();
    }
}

// Fixed-order block sums in float32 (the inner solves of the refinement:
// their scalars need a few digits, not float64 adds)
template <int N>
__device__ __forceinline__ void block_sumf(float (&v)[N], float* red) {
    __shared__ float resf[N];
#pragma unroll
    for (int k = 0; k < N; ++k) red[k * kBatchThreads + threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float* e = red + k * kBatchThreads + threadIdx.x;
            float t8[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) t8[j] = e[64 * j] + e[64 * j + 32];
            float t = ((t8[0] + t8[1]) + (t8[2] + t8[3])) + ((t8[4] + t8[5]) + (t8[6] + t8[7]));
#pragma unroll
            for (int msk = 16; msk > 0; msk >>= 1) t += __shfl_xor_sync(0xffffffffu, t, msk);
            if (threadIdx.x == 0) resf[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = resf[k];
}

// Mixed-precision iterative refinement, one system per CTA as above: the
// float64 residual r = b - A x (true, not recursive), then a float32
// Jacobi-PCG solve of A d = r / ||r|| (float32 values, vectors, arithmetic
// and block sums) until its residual falls by inner_rtol, then x += ||r|| d
// in float64; until ||b - A x|| <= rtol ||b|| or max_outer corrections or
// max_iter inner iterations in all.  On GB300 float64 runs at 1/64 of the
// float32 rate, and the float64 PCG's FMAs bound a system's iteration.
// Float workspace: r, z, p, q, d, dinv as float [n_rows] each after the
// float64 residual in work (4 n_rows doubles of the 5).
__global__ void __launch_bounds__(kBatchThreads) k_batched_ir(const tm_batched_mixed_args m) {
    const tm_batched_pcg_args& a = m.base;
    __shared__ double red[kBatchThreads];
    __shared__ float redf[2 * kBatchThreads];
    __shared__ int sys_s;
    const int64_t* rp = a.A.row_ptr;
    const int32_t* col = a.A.col;
    const double* val = static_cast<const double*>(a.A.values);
    float* v32 = static_cast<float*>(m.values32);
    const double* b = static_cast<const double*>(a.b);
    double* x = static_cast<double*>(a.x);
    const int64_t n_all = a.A.n_rows;
    double* r64 = static_cast<double*>(a.work);
    float* r = reinterpret_cast<float*>(r64 + n_all);
    float* z = r + n_all;
    float* p = z + n_all;
    float* q = p + n_all;
    float* d = q + n_all;
    float* dinv = d + n_all;
    const uint8_t* fixed = a.dirichlet;
    const double tol2 = a.rtol * a.rtol;
    const float eta2 = (float)(m.inner_rtol * m.inner_rtol);
    for (;;) {
        if (threadIdx.x == 0) {
            const int k = atomicAdd(a.queue, 1);
            sys_s = k < a.n_systems ? (a.order ? a.order[k] : k) : a.n_systems;
        }
        __syncthreads();
        const int sys = sys_s;
        __syncthreads();
        if (sys >= a.n_systems) return;
        const int64_t r0 = a.system_offset[sys], r1 = a.system_offset[sys + 1];
        // float32 copies of the system's values, the inverse diagonal, ||b||^2
        double vb[1] = {0.0};
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kBatchThreads) {
            double dg = 0.0;
            for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
                const double v = val[k];
                v32[k] = (float)v;
                if (col[k] == i) dg += v;
            }
            const bool fx = fixed && fixed[i];
            dinv[i] = (!fx && dg != 0.0) ? (float)(1.0 / dg) : 0.0f;
            if (!fx) vb[0] += b[i] * b[i];
        }
        block_sum<1>(vb, red);
        const double bb = vb[0];
        int total = 0, flag = 0;
        double rr = 0.0;
        for (int outer = 0;; ++outer) {
            double vr[1] = {0.0};
            for (int64_t i = r0 + threadIdx.x; i < r1; i += kBatchThreads) {
                if (fixed && fixed[i]) continue;
                double ax = 0.0;
                for (int64_t k = rp[i]; k < rp[i + 1]; ++k) ax += val[k] * x[col[k]];
                const double ri = b[i] - ax;
                r64[i] = ri;
                vr[0] += ri * ri;
            }
            block_sum<1>(vr, red);
            rr = vr[0];
            if (rr <= tol2 * bb || bb == 0.0) {
                flag = TM_PCG_CONVERGED;
                break;
            }
            if (outer >= m.max_outer || total >= a.max_iter) {
                flag = TM_PCG_MAX_ITER;
                break;
            }
            // the correction: float32 Jacobi-PCG on A d = r / ||r||, d0 = 0
            const double nr = sqrt(rr);
            const double sc = 1.0 / nr;
            float v2[2] = {0.0f, 0.0f};
            for (int64_t i = r0 + threadIdx.x; i < r1; i += kBatchThreads) {
                if (fixed && fixed[i]) {
                    r[i] = z[i] = p[i] = q[i] = d[i] = 0.0f;
                    continue;
                }
                const float ri = (float)(r64[i] * sc);
                const float zi = ri * dinv[i];
                r[i] = ri;
                z[i] = zi;
                p[i] = zi;
                d[i] = 0.0f;
                v2[0] += ri * zi;
                v2[1] += ri * ri;
            }
            block_sumf<2>(v2, redf);
            float rz = v2[0];
            const float rr0 = v2[1];
            float rri = rr0;
            int it = 0;
            while (rri > eta2 * rr0 && total + it < a.max_iter) {
                float v1[1] = {0.0f};
                constexpr int RU = 4;
                for (int64_t i0 = r0 + threadIdx.x; i0 < r1; i0 += RU * kBatchThreads) {
                    int64_t beg[RU], len[RU];
                    int64_t maxlen = 0;
#pragma unroll
                    for (int u = 0; u < RU; ++u) {
                        const int64_t i = i0 + (int64_t)u * kBatchThreads;
                        const bool on = i < r1 && !(fixed && fixed[i]);
                        beg[u] = on ? rp[i] : 0;
                        len[u] = on ? rp[i + 1] - beg[u] : 0;
                        maxlen = len[u] > maxlen ? len[u] : maxlen;
                    }
                    float sv[RU] = {};
                    for (int64_t k = 0; k < maxlen; ++k)
#pragma unroll
                        for (int u = 0; u < RU; ++u)
                            if (k < len[u]) sv[u] += v32[beg[u] + k] * p[col[beg[u] + k]];
#pragma unroll
                    for (int u = 0; u < RU; ++u) {
                        const int64_t i = i0 + (int64_t)u * kBatchThreads;
                        if (i < r1 && !(fixed && fixed[i])) {
                            q[i] = sv[u];
                            v1[0] += p[i] * sv[u];
                        }
                    }
                }
                block_sumf<1>(v1, redf);
                const float pq = v1[0];
                if (!(pq > 0.0f)) break;             // breakdown: d as it stands
                const float alpha = rz / pq;
                float w2[2] = {0.0f, 0.0f};
                for (int64_t i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * kBatchThreads) {
                    float dv[4], pv[4], rv[4], qv[4], iv[4];
                    bool on[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int64_t i = i0 + (int64_t)u * kBatchThreads;
                        on[u] = i < r1 && !(fixed && fixed[i]);
                        if (on[u]) { dv[u] = d[i]; pv[u] = p[i]; rv[u] = r[i]; qv[u] = q[i]; iv[u] = dinv[i]; }
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (!on[u]) continue;
                        const int64_t i = i0 + (int64_t)u * kBatchThreads;
                        d[i] = dv[u] + alpha * pv[u];
                        const float ri = rv[u] - alpha * qv[u];
                        r[i] = ri;
                        const float zi = ri * iv[u];
                        z[i] = zi;
                        w2[0] += ri * zi;
                        w2[1] += ri * ri;
                    }
                }
                block_sumf<2>(w2, redf);
                const float beta = rz != 0.0f ? w2[0] / rz : 0.0f;
                rz = w2[0];
                rri = w2[1];
                for (int64_t i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * kBatchThreads) {
                    float zv[4], pv[4];
                    bool on[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int64_t i = i0 + (int64_t)u * kBatchThreads;
                        on[u] = i < r1 && !(fixed && fixed[i]);
                        if (on[u]) { zv[u] = z[i]; pv[u] = p[i]; }
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (on[u]) p[i0 + (int64_t)u * kBatchThreads] = zv[u] + beta * pv[u];
                }
                __syncthreads();
                ++it;
            }
            total += it;
            for (int64_t i = r0 + threadIdx.x; i < r1; i += kBatchThreads)
                if (!(fixed && fixed[i])) x[i] += nr * (double)d[i];
            __syncthreads();
            if (it == 0) {                                // no correction made
                flag = total >= a.max_iter ? TM_PCG_MAX_ITER : TM_PCG_BREAKDOWN;
                break;
            }
        }
        if (threadIdx.x == 0 && a.status) {
            a.status[sys].iterations = total;
            a.status[sys].flag = flag;
            a.status[sys].relative_residual = bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
        }
        __syncthreads();
    }
}

inline int bstatus(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

}  // namespace tmk

using namespace tmk;

extern "C" int tm_batched_pcg(const tm_batched_pcg_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg: null args");
    if (a->n_systems < 0 || a->max_iter < 0 || a->A.block != 1 || a->A.n_rows < 0)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg: bad sizes (scalar CSR only)");
    if (a->n_systems == 0) return TM_OK;
    if (!a->system_offset || !a->A.row_ptr || !a->A.col || !a->A.values || !a->b || !a->x || !a->work ||
        !a->queue)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg: null pointer");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(a->queue, 0, sizeof(int32_t), st) != cudaSuccess) return bstatus("cudaMemsetAsync");
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (a->A.dtype == TM_F64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batched_pcg<double>, kBatchThreads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batched_pcg<float>, kBatchThreads, 0);
    // resident CTAs only: each one loops over the queue
    int grid = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 152);
    if (grid > a->n_systems) grid = a->n_systems;
    if (a->A.dtype == TM_F64)
        k_batched_pcg<double><<<grid, kBatchThreads, 0, st>>>(*a);
    else if (a->A.dtype == TM_F32)
        k_batched_pcg<float><<<grid, kBatchThreads, 0, st>>>(*a);
    else
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg: dtype must be TM_F64 or TM_F32");
    return bstatus("k_batched_pcg");
}

extern "C" int tm_batched_pcg_mixed(const tm_batched_mixed_args* m, tm_stream_t stream) {
    if (!m) return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg_mixed: null args");
    const tm_batched_pcg_args* a = &m->base;
    if (a->n_systems < 0 || a->max_iter < 0 || a->A.block != 1 || a->A.n_rows < 0 || m->max_outer < 0)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg_mixed: bad sizes (scalar CSR only)");
    if (a->A.dtype != TM_F64) return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg_mixed: float64 matrix only");
    if (!(m->inner_rtol > 0.0 && m->inner_rtol < 1.0))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg_mixed: inner_rtol outside (0, 1)");
    if (a->n_systems == 0) return TM_OK;
    if (!a->system_offset || !a->A.row_ptr || !a->A.col || !a->A.values || !a->b || !a->x || !a->work ||
        !a->queue || !m->values32)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_batched_pcg_mixed: null pointer");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(a->queue, 0, sizeof(int32_t), st) != cudaSuccess) return bstatus("cudaMemsetAsync");
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batched_ir, kBatchThreads, 0);
    int grid = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 152);
    if (grid > a->n_systems) grid = a->n_systems;
    k_batched_ir<<<grid, kBatchThreads, 0, st>>>(*m);
    return bstatus("k_batched_ir");
}
