// Jacobi-preconditioned conjugate gradients on the GPU.
//
// Replaces the solve behind SparseMatrix.solve for SPD systems (the
// reference's in-tree Krylov solvers are sparse/solve/torch_solve.py:70-248:
// CG without preconditioner and Jacobi-BiCGSTAB, both a Python loop of torch
// SpMVs).  Every scalar of the iteration (rz, pq, alpha, beta, residual
// norms) stays on the device; one tm_pcg_iterate call runs n_iter
// iterations as 6 kernel launches each with no host synchronisation, so the
// host only reads the residual between batches of iterations;
// tm_pcg_iterate_until runs them in one cooperative persistent launch that
// stops on the device at convergence.  Dot products
// are reduced in a fixed order (per-block partials, then one block), so the
// iteration is bitwise reproducible.  Dots are accumulated in float64 for
// both float64 and float32 vectors.
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>
#include <algorithm>
#include <type_traits>

#include "../../include/tensormesh_gb300.h"
#include "tm_status.h"

namespace tmk {

constexpr int kSolveThreads = 256;
constexpr int kDotBlocks = 608;   // 4 x 152 SMs
constexpr int kBlockLanes = 4;    // lanes per block row of a block (H > 1) operator
constexpr int kVecUnroll = 2;     // vector elements per thread and pass in the persistent PCG

// scalar slots
enum { S_RZ = 0, S_PQ = 1, S_RZ_NEW = 2, S_RR = 3, S_BB = 4, S_ITER = 5, S_FLAG = 6 };

template <typename R>
__device__ __forceinline__ R ld(const R* p) { return __ldg(p); }

// the (block) row taken at position i of the operator's row order; -1 for
// an entry outside [0, n_rows)
__device__ __forceinline__ int64_t row_at(const tm_linear_operator& A, int64_t i) {
    if (!A.row_order) return i;
    const int64_t r = __ldg(A.row_order + i);
    return (r >= 0 && r < A.n_rows) ? r : -1;
}

// lane-partial of row `row` of A x for scalar CSR (H == 1) or block CSR rows:
// lane l of the 8-lane group sums entries l, l+8, ... of the (block) row
template <typename R, int H>
__device__ __forceinline__ double row_partial(const tm_linear_operator& A, const R* x, int64_t row, int lane) {
    const int64_t br = row / H;
    const int a = (int)(row - br * H);
    const R* val = static_cast<const R*>(A.values);
    double s = 0;
    for (int64_t p = A.row_ptr[br] + lane; p < A.row_ptr[br + 1]; p += 8) {
        const int64_t c = A.col[p];
        if (H == 1) {
            s += (double)ld(val + p) * (double)ld(x + c);
        } else {
#pragma unroll
            for (int b = 0; b < H; ++b) s += (double)ld(val + p * H * H + a * H + b) * (double)ld(x + c * H + b);
        }
    }
    return s;
}

// butterfly sum over the 8 lanes of a group; every lane of the warp must call it
__device__ __forceinline__ double group_sum(double s) {
    s += __shfl_xor_sync(0xffffffffu, s, 4, 8);
    s += __shfl_xor_sync(0xffffffffu, s, 2, 8);
    s += __shfl_xor_sync(0xffffffffu, s, 1, 8);
    return s;
}

// first row position of this block's chunk of `per` rows in pass `pass`:
// odd passes hand the chunks out in reverse block order, so that with rows
// sorted longest first no block takes the longest chunk of every pass; a
// block whose chunk starts past the end has none in later passes either
__device__ __forceinline__ int64_t serpentine_base(int64_t pass, int per) {
    const int64_t b = (pass & 1) ? (int64_t)(gridDim.x - 1 - blockIdx.x) : (int64_t)blockIdx.x;
    return (pass * gridDim.x + b) * per;
}

// the H partial sums of block row `br` of A x: lane l of the L-lane group
// takes blocks row_ptr[br] + l, + 2L, ...; each block is read once (its H*H
// values, one column index, H entries of x), and every scalar row sums its
// terms in the same order as row_partial_cg
template <typename R, int H, int L, bool kL2 = true>
__device__ __forceinline__ void block_row_cg(const tm_linear_operator& A, const R* x, int64_t br, int lane,
                                             double (&s)[H]) {
    const R* val = static_cast<const R*>(A.values);
#pragma unroll
    for (int a = 0; a < H; ++a) s[a] = 0;
    const int64_t end = A.row_ptr[br + 1];
#pragma unroll 2
    for (int64_t p = A.row_ptr[br] + lane; p < end; p += L) {
        const int64_t c = A.col[p];
        R v[H * H];
#pragma unroll
        for (int k = 0; k < H * H; ++k) v[k] = ld(val + p * H * H + k);
        double xb[H];
#pragma unroll
        for (int b = 0; b < H; ++b) xb[b] = (double)(kL2 ? __ldcg(x + c * H + b) : ld(x + c * H + b));
#pragma unroll
        for (int a = 0; a < H; ++a)
#pragma unroll
            for (int b = 0; b < H; ++b) s[a] += (double)v[a * H + b] * xb[b];
    }
}

// butterfly sum over the L lanes of a group; every lane of the warp calls it
template <int L>
__device__ __forceinline__ double lane_sum(double s) {
#pragma unroll
    for (int m = L / 2; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m, L);
    return s;
}

// reduce-scatter of the H (<= 4) sums s[] over the 4 lanes of a group: lane
// k < H returns the group's sum of s[k], grouped (s_k[0] + s_k[2]) +
// (s_k[1] + s_k[3]) exactly as lane_sum<4> groups it, with 3 adds per lane
// instead of 2H (float64 adds are the scarce resource of this kernel)
template <int H>
__device__ __forceinline__ double group4_scatter(const double (&s)[H], int lane) {
    static_assert(H >= 1 && H <= 4, "group4_scatter takes 1..4 sums");
    double t[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int c = 0; c < H; ++c) t[c] = s[c];
    const bool hi = (lane & 2) != 0, odd = (lane & 1) != 0;
    // lanes l and l^2: the low lane keeps sums 0 and 1, the high lane 2 and 3
    const double ta = (hi ? t[2] : t[0]) + __shfl_xor_sync(0xffffffffu, hi ? t[0] : t[2], 2, 4);
    const double tb = (hi ? t[3] : t[1]) + __shfl_xor_sync(0xffffffffu, hi ? t[1] : t[3], 2, 4);
    // lanes l and l^1: the even lane keeps the first, the odd lane the second
    return (odd ? tb : ta) + __shfl_xor_sync(0xffffffffu, odd ? ta : tb, 1, 4);
}

// q = A p ; partial[blk] = sum p.q over this block's rows (in row order)
template <typename R, int H>
__global__ void __launch_bounds__(kSolveThreads) k_spmv_dot(tm_linear_operator A, const R* p, R* q,
                                                            double* partial, const double* scal) {
    __shared__ double red[kSolveThreads / 8];
    const int64_t n = A.n_rows * H;
    const int lane = threadIdx.x & 7, grp = threadIdx.x >> 3;
    const bool stop = scal && scal[S_FLAG] != 0.0;
    double acc = 0;
    if (!stop && H == 1) {
        for (int64_t pass = 0;; ++pass) {
            const int64_t base = serpentine_base(pass, kSolveThreads / 8);
            if (base >= n) break;
            const int64_t r = base + grp < n ? row_at(A, base + grp) : -1;
            // all 8 lanes of a group share r; the loop bound is uniform per block
            const double s = group_sum(r >= 0 ? row_partial<R, H>(A, p, r, lane) : 0.0);
            if (r >= 0 && lane == 0) {
                q[r] = (R)s;
                acc += s * (double)p[r];
            }
        }
    } else if (!stop) {
        // 4-lane groups, one block row each; the 8-lane slots of red hold
        // the sums of pairs of groups
        constexpr int L = kBlockLanes;
        static_assert(L == 4, "block rows are summed by group4_scatter");
        const int bl = threadIdx.x & (L - 1), bg = threadIdx.x / L;
        const int64_t nb = A.n_rows;
        for (int64_t pass = 0;; ++pass) {
            const int64_t base = serpentine_base(pass, kSolveThreads / L);
            if (base >= nb) break;
            const int64_t bi = base + bg < nb ? row_at(A, base + bg) : -1;
            double s[H];
            if (bi >= 0) {
                block_row_cg<R, H, L, false>(A, p, bi, bl, s);
            } else {
#pragma unroll
                for (int c = 0; c < H; ++c) s[c] = 0;
            }
            const double u = group4_scatter<H>(s, bl);     // row bi * H + bl on lanes bl < H
            if (bi >= 0 && bl < H) {
                q[bi * H + bl] = (R)u;
                acc += u * (double)p[bi * H + bl];
            }
        }
        acc = lane_sum<8>(acc);   // lane 0 of each 8-lane slot: both groups' sums
    }
    if (lane == 0) red[grp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int g = 0; g < kSolveThreads / 8; ++g) t += red[g];
        if (partial) partial[blockIdx.x] = t;
    }
}

// fixed-order sum of per-block partials into scal[slot] (one block)
__global__ void k_reduce_partials(const double* partial, int n, double* scal, int slot, int n_vec, int slot2) {
    __shared__ double red[kSolveThreads];
    for (int v = 0; v < n_vec; ++v) {
        double s = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[v * n + i];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) scal[v == 0 ? slot : slot2] = red[0];
        __syncthreads();
    }
}

// x += alpha p ; r -= alpha q ; z = dinv r ; partials: r.z and r.r
template <typename R>
__global__ void __launch_bounds__(kSolveThreads) k_update_xr(int64_t n, R* x, R* r, const R* p, const R* q, R* z,
                                                             const R* dinv, double* partial, double* scal) {
    __shared__ double red[2][kSolveThreads];
    const double pq = scal[S_PQ];
    bool stop = scal[S_FLAG] != 0.0;
    if (!(pq > 0.0)) stop = true;   // breakdown (p^T A p <= 0 or NaN): freeze
    const double alpha = stop ? 0.0 : scal[S_RZ] / pq;
    double rz = 0, rr = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double ri = (double)r[i];
        if (!stop) {
            x[i] = (R)((double)x[i] + alpha * (double)p[i]);
            ri = ri - alpha * (double)q[i];
            r[i] = (R)ri;
        }
        const double zi = ri * (double)dinv[i];
        z[i] = (R)zi;
        rz += ri * zi;
        rr += ri * ri;
    }
    red[0][threadIdx.x] = rz;
    red[1][threadIdx.x] = rr;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = red[0][0];
        partial[gridDim.x + blockIdx.x] = red[1][0];
        if (blockIdx.x == 0 && !(pq > 0.0) && scal[S_FLAG] == 0.0) scal[S_FLAG] = 2.0;
    }
}

// p = z + beta p ; rz <- rz_new ; iteration counter
template <typename R>
__global__ void __launch_bounds__(kSolveThreads) k_update_p(int64_t n, const R* z, R* p, double* scal) {
    const bool stop = scal[S_FLAG] != 0.0;
    const double rz_old = scal[S_RZ], rz_new = scal[S_RZ_NEW];
    const double beta = rz_old != 0.0 ? rz_new / rz_old : 0.0;
    if (!stop)
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            p[i] = (R)((double)z[i] + beta * (double)p[i]);
    // rz is replaced by rz_new in k_commit_rz, after every block has read it
}

__global__ void k_commit_rz(double* scal) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (scal[S_FLAG] == 0.0) {
            scal[S_RZ] = scal[S_RZ_NEW];
            scal[S_ITER] += 1.0;
        }
    }
}

// dinv = 1 / diag(A); r = b - A x ; z = dinv r ; p = z ; partials r.z, r.r, b.b
template <typename R, int H>
__global__ void __launch_bounds__(kSolveThreads) k_pcg_start(tm_linear_operator A, const R* b, const R* x,
                                                             R* dinv, R* r, R* z, R* p, double* partial) {
    __shared__ double red[3][kSolveThreads / 8];
    const int64_t n = A.n_rows * H;
    const R* val = static_cast<const R*>(A.values);
    const int lane = threadIdx.x & 7, grp = threadIdx.x >> 3;
    double rz = 0, rr = 0, bb = 0;
    const int64_t groups_total = (int64_t)gridDim.x * (kSolveThreads / 8);
    for (int64_t base = (int64_t)blockIdx.x * (kSolveThreads / 8); base < n; base += groups_total) {
        const int64_t i = base + grp;
        const double ax = group_sum(i < n ? row_partial<R, H>(A, x, i, lane) : 0.0);
        if (i < n && lane == 0) {
            // diagonal entry of row i
            const int64_t br = i / H;
            const int a = (int)(i - br * H);
            double d = 0;
            for (int64_t q = A.row_ptr[br]; q < A.row_ptr[br + 1]; ++q)
                if (A.col[q] == br) d += (double)val[q * H * H + a * H + a];
            const double di = d != 0.0 ? 1.0 / d : 0.0;
            dinv[i] = (R)di;
            const double ri = (double)b[i] - ax;
            r[i] = (R)ri;
            const double zi = ri * di;
            z[i] = (R)zi;
            p[i] = (R)zi;
            rz += ri * zi;
            rr += ri * ri;
            bb += (double)b[i] * (double)b[i];
        }
    }
    if (lane == 0) {
        red[0][grp] = rz;
        red[1][grp] = rr;
        red[2][grp] = bb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0, t1 = 0, t2 = 0;
        for (int g = 0; g < kSolveThreads / 8; ++g) {
            t0 += red[0][g];
            t1 += red[1][g];
            t2 += red[2][g];
        }
        partial[blockIdx.x] = t0;
        partial[gridDim.x + blockIdx.x] = t1;
        partial[2 * gridDim.x + blockIdx.x] = t2;
    }
}

__global__ void k_reduce_start(const double* partial, int n, double* scal) {
    __shared__ double red[kSolveThreads];
    const int slots[3] = {S_RZ, S_RR, S_BB};
    for (int v = 0; v < 3; ++v) {
        double s = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[v * n + i];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) scal[slots[v]] = red[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scal[S_ITER] = 0.0;
        scal[S_FLAG] = 0.0;
        scal[S_PQ] = 0.0;
        scal[S_RZ_NEW] = scal[S_RZ];
    }
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

inline int grid_rows(int64_t n) {
    int64_t g = (n + kSolveThreads / 8 - 1) / (kSolveThreads / 8);
    return (int)(g < 1 ? 1 : (g > kDotBlocks ? kDotBlocks : g));
}
inline int grid_vec(int64_t n) {
    int64_t g = (n + kSolveThreads - 1) / kSolveThreads;
    return (int)(g < 1 ? 1 : (g > kDotBlocks ? kDotBlocks : g));
}

template <typename R, int H>
int pcg_start(const tm_pcg_args& a, cudaStream_t st) {
    const int64_t n = a.A.n_rows * H;
    const int g = grid_rows(n);
    k_pcg_start<R, H><<<g, kSolveThreads, 0, st>>>(a.A, static_cast<const R*>(a.b), static_cast<const R*>(a.x),
                                                     static_cast<R*>(a.dinv), static_cast<R*>(a.r),
                                                     static_cast<R*>(a.z), static_cast<R*>(a.p), a.partials);
    k_reduce_start<<<1, kSolveThreads, 0, st>>>(a.partials, g, a.scalars);
    return status("tm_pcg_start");
}

template <typename R, int H>
int pcg_iterate(const tm_pcg_args& a, int n_iter, cudaStream_t st) {
    const int64_t n = a.A.n_rows * H;
    const int gr = grid_rows(n), gv = grid_vec(n);
    for (int it = 0; it < n_iter; ++it) {
        k_spmv_dot<R, H><<<gr, kSolveThreads, 0, st>>>(a.A, static_cast<const R*>(a.p), static_cast<R*>(a.q),
                                                         a.partials, a.scalars);
        k_reduce_partials<<<1, kSolveThreads, 0, st>>>(a.partials, gr, a.scalars, S_PQ, 1, 0);
        k_update_xr<R><<<gv, kSolveThreads, 0, st>>>(n, static_cast<R*>(a.x), static_cast<R*>(a.r),
                                                     static_cast<const R*>(a.p), static_cast<const R*>(a.q),
                                                     static_cast<R*>(a.z), static_cast<const R*>(a.dinv),
                                                     a.partials, a.scalars);
        k_reduce_partials<<<1, kSolveThreads, 0, st>>>(a.partials, gv, a.scalars, S_RZ_NEW, 2, S_RR);
        k_update_p<R><<<gv, kSolveThreads, 0, st>>>(n, static_cast<const R*>(a.z), static_cast<R*>(a.p), a.scalars);
        k_commit_rz<<<1, 32, 0, st>>>(a.scalars);
    }
    return status("tm_pcg_iterate");
}

template <typename R, int H>
__global__ void __launch_bounds__(kSolveThreads) k_spmv_op(tm_linear_operator A, const R* x, R* y, double alpha,
                                                           double beta) {
    const int64_t n = A.n_rows * H;
    if constexpr (H == 1) {
        const int lane = threadIdx.x & 7, grp = threadIdx.x >> 3;
        const int64_t groups_total = (int64_t)gridDim.x * (kSolveThreads / 8);
        for (int64_t base = (int64_t)blockIdx.x * (kSolveThreads / 8); base < n; base += groups_total) {
            const int64_t r = base + grp < n ? row_at(A, base + grp) : -1;
            const double s = group_sum(r >= 0 ? row_partial<R, H>(A, x, r, lane) : 0.0);
            if (r >= 0 && lane == 0) y[r] = (R)(beta == 0.0 ? alpha * s : alpha * s + beta * (double)y[r]);
        }
    } else {
        constexpr int L = kBlockLanes;
        static_assert(L == 4, "block rows are summed by group4_scatter");
        const int lane = threadIdx.x & (L - 1), grp = threadIdx.x / L;
        const int64_t nb = A.n_rows, groups_total = (int64_t)gridDim.x * (kSolveThreads / L);
        for (int64_t base = (int64_t)blockIdx.x * (kSolveThreads / L); base < nb; base += groups_total) {
            const int64_t bi = base + grp < nb ? row_at(A, base + grp) : -1;
            double s[H];
            if (bi >= 0) {
                block_row_cg<R, H, L, false>(A, x, bi, lane, s);
            } else {
#pragma unroll
                for (int c = 0; c < H; ++c) s[c] = 0;
            }
            const double u = group4_scatter<H>(s, lane);   // row bi * H + lane on lanes < H
            if (bi >= 0 && lane < H) {
                const int64_t r = bi * H + lane;
                y[r] = (R)(beta == 0.0 ? alpha * u : alpha * u + beta * (double)y[r]);
            }
        }
    }
}

template <typename R, int H>
int spmv_op(const tm_linear_operator& A, const void* x, void* y, double alpha, double beta, cudaStream_t st) {
    const int64_t n = A.n_rows * H;
    int64_t g = (n + kSolveThreads / 8 - 1) / (kSolveThreads / 8);
    if (g > 152 * 64) g = 152 * 64;
    if (g < 1) g = 1;
    k_spmv_op<R, H><<<(int)g, kSolveThreads, 0, st>>>(A, static_cast<const R*>(x), static_cast<R*>(y), alpha, beta);
    return status("tm_spmv");
}

template <typename F>
int dispatch_op(const tm_linear_operator& A, F&& f) {
    if (A.dtype == TM_F64) {
        switch (A.block) {
            case 1: return f(double(), std::integral_constant<int, 1>());
            case 2: return f(double(), std::integral_constant<int, 2>());
            case 3: return f(double(), std::integral_constant<int, 3>());
        }
    } else if (A.dtype == TM_F32) {
        switch (A.block) {
            case 1: return f(float(), std::integral_constant<int, 1>());
            case 2: return f(float(), std::integral_constant<int, 2>());
            case 3: return f(float(), std::integral_constant<int, 3>());
        }
    }
    return tm_set_error(TM_ERR_UNSUPPORTED, "linear operator: dtype must be F64/F32 and block 1..3");
}

// ---------------------------------------------------------------------------
// Persistent PCG: up to max_iter iterations in one cooperative launch (all
// blocks co-resident), three grid barriers per iteration, convergence or
// breakdown decided identically by every block from the same fixed-order sums
// of the per-block partials.  Vectors written by other blocks of the launch
// are read through L2 (__ldcg), never through the non-coherent L1.

// set when a grid barrier's bounded wait ran out (read by tm_device_fault)
__device__ int g_solve_fault = 0;

constexpr unsigned kBarrierTries = 1u << 22;   // L2 round trips: about a second

// Grid barrier on one arrival counter (bar[0], zero before the launch, never
// reset within it): the barrier of epoch e completes when the counter
// reaches (e + 1) * nblocks (modulo 2^32).  Thread 0 of each block releases
// the block's writes (fence, then the arrival add) and polls with acquire
// loads; no reset or generation word sits on the critical path.  False when
// the wait ran out, in which case the caller returns.
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned& epoch) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = (epoch + 1u) * nblocks;
        __threadfence();
        unsigned v;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(v) : "l"(bar) : "memory");
        v += 1u;
        unsigned it = 0;
        while ((int)(v - target) < 0 && ++it < kBarrierTries)
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
        ok = (int)(v - target) >= 0;
        if (!ok) atomicExch(&g_solve_fault, 1);
    }
    __syncthreads();
    ++epoch;
    return ok != 0;
}

// butterfly sum over the 32 lanes of a warp; every lane ends with the same
// value (both lanes of a pair add the same two operands)
__device__ __forceinline__ double warp_sum(double s) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    return s;
}

// Fixed-order block sums of K values per thread (blockDim.x ==
// kSolveThreads): staged in shared memory and summed by warp 0 alone (a
// pairwise tree over each lane's 8 entries, then a butterfly), so that few
// FP64 instructions and a short chain of dependent adds are spent; every
// thread returns the same sums
template <int K>
__device__ __forceinline__ void block_sums(const double (&v)[K], double (&out)[K], double (*red)[kSolveThreads],
                                           double* res) {
    static_assert(kSolveThreads == 256, "block_sums sums 8 entries per lane of warp 0");
#pragma unroll
    for (int k = 0; k < K; ++k) red[k][threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const double* e = red[k] + threadIdx.x;
            const double t = ((e[0] + e[32]) + (e[64] + e[96])) + ((e[128] + e[160]) + (e[192] + e[224]));
            const double w = warp_sum(t);
            if (threadIdx.x == 0) res[k] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = res[k];
}

// sums of the K arrays part[k * stride + 0..n) in a fixed order (strided per
// thread, then block_sums): the same values in every block of the launch
template <int K>
__device__ __forceinline__ void ordered_sums(const double* part, int stride, int n, double (&out)[K],
                                             double (*red)[kSolveThreads], double* res) {
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double t = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) t += __ldcg(part + k * stride + i);
        v[k] = t;
    }
    block_sums<K>(v, out, red, res);
}

template <typename R, int H, int L>
__device__ __forceinline__ double row_partial_cg(const tm_linear_operator& A, const R* x, int64_t row, int lane) {
    const int64_t br = row / H;
    const int a = (int)(row - br * H);
    const R* val = static_cast<const R*>(A.values);
    double s = 0;
    for (int64_t p = A.row_ptr[br] + lane; p < A.row_ptr[br + 1]; p += L) {
        const int64_t c = A.col[p];
#pragma unroll
        for (int b = 0; b < H; ++b) s += (double)ld(val + p * H * H + a * H + b) * (double)__ldcg(x + c * H + b);
    }
    return s;
}

template <typename R, int H, int L>
__global__ void __launch_bounds__(kSolveThreads, 2) k_pcg_persistent(const tm_pcg_args a, int max_iter, double tol2) {
    __shared__ double red[2][kSolveThreads];
    __shared__ double res[2];
    const int64_t n = a.A.n_rows * H;
    const unsigned G = gridDim.x;
    unsigned epoch = 0;
    unsigned* bar = reinterpret_cast<unsigned*>(a.partials + 3 * kDotBlocks);
    double* part_pq = a.partials;
    double* part_rz = a.partials + kDotBlocks;
    double* part_rr = a.partials + 2 * kDotBlocks;
    R* x = static_cast<R*>(a.x);
    R* r = static_cast<R*>(a.r);
    R* z = static_cast<R*>(a.z);
    R* p = static_cast<R*>(a.p);
    R* q = static_cast<R*>(a.q);
    const R* dinv = static_cast<const R*>(a.dinv);
    double* scal = a.scalars;
    double rz = scal[S_RZ], rr = scal[S_RR], pq = scal[S_PQ];
    const double bb = scal[S_BB];
    double iters = scal[S_ITER];
    int flag = (int)scal[S_FLAG];
    if (flag == 0 && rr <= tol2 * bb) flag = 1;
    const int lane = threadIdx.x & (L - 1), grp = threadIdx.x / L;
    const int64_t stride = (int64_t)G * blockDim.x;
    for (int it = 0; it < max_iter && flag == 0; ++it) {
        // q = A p and this block's part of p.q
        double acc = 0;
        if constexpr (H == 1) {
            for (int64_t pass = 0;; ++pass) {
                const int64_t base = serpentine_base(pass, kSolveThreads / L);
                if (base >= n) break;
                const int64_t i = base + grp < n ? row_at(a.A, base + grp) : -1;
                const double s = lane_sum<L>(i >= 0 ? row_partial_cg<R, H, L>(a.A, p, i, lane) : 0.0);
                if (i >= 0 && lane == 0) {
                    __stcg(q + i, (R)s);
                    acc += s * (double)__ldcg(p + i);
                }
            }
        } else {
            // one group per block row: H rows of q from one pass over the blocks
            const int64_t nb = a.A.n_rows;
            for (int64_t pass = 0;; ++pass) {
                const int64_t base = serpentine_base(pass, kSolveThreads / L);
                if (base >= nb) break;
                const int64_t bi = base + grp < nb ? row_at(a.A, base + grp) : -1;
                double s[H];
                if (bi >= 0) {
                    block_row_cg<R, H, L>(a.A, p, bi, lane, s);
                } else {
#pragma unroll
                    for (int c = 0; c < H; ++c) s[c] = 0;
                }
                double u;
                if constexpr (L == 4) {
                    u = group4_scatter<H>(s, lane);          // row bi * H + lane on lanes < H
                } else {
                    u = 0;
#pragma unroll
                    for (int c = 0; c < H; ++c) {
                        const double t = lane_sum<L>(s[c]);
                        if (lane == c) u = t;
                    }
                }
                if (bi >= 0 && lane < H) {
                    __stcg(q + bi * H + lane, (R)u);
                    acc += u * (double)__ldcg(p + bi * H + lane);
                }
            }
        }
        {
            const double v[1] = {acc};
            double o[1];
            block_sums<1>(v, o, red, res);
            if (threadIdx.x == 0) __stcg(part_pq + blockIdx.x, o[0]);
        }
        if (!grid_barrier(bar, G, epoch)) return;
        {
            double o[1];
            ordered_sums<1>(part_pq, 0, (int)G, o, red, res);
            pq = o[0];
        }
        if (!(pq > 0.0)) {   // breakdown (p^T A p <= 0 or NaN): x stays as it is
            flag = 2;
            break;
        }
        const double alpha = rz / pq;
        // x += alpha p ; r -= alpha q ; z = dinv r ; partials r.z and r.r
        // (kVecUnroll elements per thread and pass, all loads issued first)
        double lrz = 0, lrr = 0;
        for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kVecUnroll * stride) {
            double xv[kVecUnroll], pv[kVecUnroll], rv[kVecUnroll], qv[kVecUnroll], dv[kVecUnroll];
#pragma unroll
            for (int u = 0; u < kVecUnroll; ++u) {
                const int64_t i = i0 + u * stride;
                if (i < n) {
                    xv[u] = (double)__ldcg(x + i);
                    pv[u] = (double)__ldcg(p + i);
                    rv[u] = (double)__ldcg(r + i);
                    qv[u] = (double)__ldcg(q + i);
                    dv[u] = (double)ld(dinv + i);
                }
            }
#pragma unroll
            for (int u = 0; u < kVecUnroll; ++u) {
                const int64_t i = i0 + u * stride;
                if (i < n) {
                    __stcg(x + i, (R)(xv[u] + alpha * pv[u]));
                    const double ri = rv[u] - alpha * qv[u];
                    __stcg(r + i, (R)ri);
                    const double zi = ri * dv[u];
                    __stcg(z + i, (R)zi);
                    lrz += ri * zi;
                    lrr += ri * ri;
                }
            }
        }
        {
            const double v[2] = {lrz, lrr};
            double o[2];
            block_sums<2>(v, o, red, res);
            if (threadIdx.x == 0) {
                __stcg(part_rz + blockIdx.x, o[0]);
                __stcg(part_rr + blockIdx.x, o[1]);
            }
        }
        if (!grid_barrier(bar, G, epoch)) return;
        double rz_new;
        {
            double o[2];
            ordered_sums<2>(part_rz, kDotBlocks, (int)G, o, red, res);
            rz_new = o[0];
            rr = o[1];
        }
        const double beta = rz != 0.0 ? rz_new / rz : 0.0;
        rz = rz_new;
        iters += 1.0;
        if (rr <= tol2 * bb) flag = 1;
        if (flag == 0) {
            for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kVecUnroll * stride) {
                double zv[kVecUnroll], pv[kVecUnroll];
#pragma unroll
                for (int u = 0; u < kVecUnroll; ++u) {
                    const int64_t i = i0 + u * stride;
                    if (i < n) {
                        zv[u] = (double)__ldcg(z + i);
                        pv[u] = (double)__ldcg(p + i);
                    }
                }
#pragma unroll
                for (int u = 0; u < kVecUnroll; ++u) {
                    const int64_t i = i0 + u * stride;
                    if (i < n) __stcg(p + i, (R)(zv[u] + beta * pv[u]));
                }
            }
            if (!grid_barrier(bar, G, epoch)) return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        scal[S_RZ] = rz;
        scal[S_RZ_NEW] = rz;
        scal[S_PQ] = pq;
        scal[S_RR] = rr;
        scal[S_ITER] = iters;
        scal[S_FLAG] = (double)flag;
    }
}

template <typename R, int H, int L>
int pcg_iterate_until_l(const tm_pcg_args& a, int max_iter, double rtol, cudaStream_t st) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_persistent<R, H, L>, kSolveThreads, 0) != cudaSuccess)
        return status("tm_pcg_iterate_until: device query");
    const int64_t n = a.A.n_rows * H;
    int64_t g = std::min<int64_t>((int64_t)sms * std::max(1, std::min(per_sm, 2)), kDotBlocks);
    g = std::min<int64_t>(g, std::max<int64_t>(1, (n + kSolveThreads / L - 1) / (kSolveThreads / L)));
    // barrier words after the three partial arrays start at zero
    if (cudaMemsetAsync(a.partials + 3 * kDotBlocks, 0, sizeof(unsigned), st) != cudaSuccess)
        return status("tm_pcg_iterate_until: memset");
    const double tol2 = rtol * rtol;
    void* params[] = {const_cast<tm_pcg_args*>(&a), &max_iter, const_cast<double*>(&tol2)};
    if (cudaLaunchCooperativeKernel((const void*)k_pcg_persistent<R, H, L>, dim3((unsigned)g), dim3(kSolveThreads),
                                    params, 0, st) != cudaSuccess)
        return status("tm_pcg_iterate_until: cooperative launch");
    return status("tm_pcg_iterate_until");
}

// 4 lanes per row and two blocks per SM measured fastest (C4 system: 37 us
// per iteration against 44 us for the six launches of tm_pcg_iterate); the
// iteration is bound by the latency of the grid barriers and fixed-order
// block reductions, not by the SpMV
template <typename R, int H>
int pcg_iterate_until(const tm_pcg_args& a, int max_iter, double rtol, cudaStream_t st) {
    return pcg_iterate_until_l<R, H, 4>(a, max_iter, rtol, st);
}

// ---------------------------------------------------------------------------
// Jacobi-preconditioned BiCGSTAB (right preconditioning, M^-1 = 1 / diag A)
// for general square systems: the algorithm of the reference's bicgstab_py
// (sparse/solve/torch_solve.py:130-248), with its safeguards: a missing or
// |d| < 1e-12 diagonal counts as 1, |r0^ . v| < 1e-12 is a breakdown, omega
// is 0 when t . t < 1e-12 (and the iteration stops after that update), and
// the iteration stops when ||s|| or ||r|| reaches the threshold.  Scalars
// stay on the device; every block takes the same decisions from the same
// fixed-order sums, and one thread commits them at the end of an iteration.

enum {
    B_RHO = 0, B_DEN = 1, B_SS = 2, B_TT = 3, B_TS = 4, B_RR = 5, B_RHO_NEW = 6, B_BB = 7,
    B_ITER = 8, B_FLAG = 9, B_THR2 = 10, B_ALPHA = 11, B_OMEGA = 12
};

// the decisions of the current iteration, identical in every block
struct BicgState {
    bool stop;      // the solve had ended before this iteration
    bool brk;       // |r0^ . v| < 1e-12
    bool sconv;     // ||s|| at the threshold: x += alpha p^ ends the solve
    double alpha, omega;
};
__device__ __forceinline__ BicgState bicg_state(const double* sc) {
    BicgState s;
    s.stop = sc[B_FLAG] != 0.0;
    const double den = sc[B_DEN];
    s.brk = !(fabs(den) >= 1e-12);
    s.alpha = s.brk ? 0.0 : sc[B_RHO] / den;
    s.sconv = sc[B_SS] <= sc[B_THR2];
    const double tt = sc[B_TT];
    s.omega = !(fabs(tt) >= 1e-12) ? 0.0 : sc[B_TS] / tt;
    return s;
}

// fixed-order block reduction of ND per-thread sums into partial[k * gridDim.x + blockIdx.x]
template <int ND>
__device__ __forceinline__ void block_partials(double (&v)[ND], double* partial) {
    __shared__ double red[ND][kSolveThreads];
#pragma unroll
    for (int k = 0; k < ND; ++k) red[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
#pragma unroll
            for (int k = 0; k < ND; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < ND; ++k) partial[k * gridDim.x + blockIdx.x] = red[k][0];
}

// y = A x and the partials of w_k . y (w_k null: y . y); mode 0: skipped
// once the solve has stopped, mode 1: also on breakdown or ||s|| converged
template <typename R, int H, int ND>
__global__ void __launch_bounds__(kSolveThreads) k_bicg_spmv(tm_linear_operator A, const R* x, R* y, const R* w0,
                                                             const R* w1, double* partial, const double* sc,
                                                             int mode) {
    const int64_t n = A.n_rows * H;
    const BicgState st = bicg_state(sc);
    const bool skip = st.stop || (mode == 1 && (st.brk || st.sconv));
    const R* w[2] = {w0, w1};
    double acc[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) acc[k] = 0.0;
    auto take = [&](int64_t r, double s) {
        y[r] = (R)s;
#pragma unroll
        for (int k = 0; k < ND; ++k) acc[k] += (w[k] ? (double)w[k][r] : s) * s;
    };
    if (!skip) {
        if constexpr (H == 1) {
            const int lane = threadIdx.x & 7, grp = threadIdx.x >> 3;
            const int64_t groups_total = (int64_t)gridDim.x * (kSolveThreads / 8);
            for (int64_t base = (int64_t)blockIdx.x * (kSolveThreads / 8); base < n; base += groups_total) {
                const int64_t r = base + grp < n ? base + grp : -1;
                const double s = group_sum(r >= 0 ? row_partial<R, H>(A, x, r, lane) : 0.0);
                if (r >= 0 && lane == 0) take(r, s);
            }
        } else {
            constexpr int L = kBlockLanes;
            const int lane = threadIdx.x & (L - 1), grp = threadIdx.x / L;
            const int64_t nb = A.n_rows, groups_total = (int64_t)gridDim.x * (kSolveThreads / L);
            for (int64_t base = (int64_t)blockIdx.x * (kSolveThreads / L); base < nb; base += groups_total) {
                const int64_t bi = base + grp < nb ? base + grp : -1;
                double s[H];
                if (bi >= 0) {
                    block_row_cg<R, H, L, false>(A, x, bi, lane, s);
                } else {
#pragma unroll
                    for (int c = 0; c < H; ++c) s[c] = 0;
                }
                const double u = group4_scatter<H>(s, lane);
                if (bi >= 0 && lane < H) take(bi * H + lane, u);
            }
        }
    }
    block_partials<ND>(acc, partial);
}

// x0 given: minv, r = b - A x, r0^ = r, p = r; partials r.r (= rho) and b.b
template <typename R, int H>
__global__ void __launch_bounds__(kSolveThreads) k_bicg_start(tm_linear_operator A, const R* b, const R* x, R* r,
                                                              R* r0h, R* p, R* minv, double* partial) {
    const int64_t n = A.n_rows * H;
    const R* val = static_cast<const R*>(A.values);
    const int lane = threadIdx.x & 7, grp = threadIdx.x >> 3;
    double acc[2] = {0.0, 0.0};
    const int64_t groups_total = (int64_t)gridDim.x * (kSolveThreads / 8);
    for (int64_t base = (int64_t)blockIdx.x * (kSolveThreads / 8); base < n; base += groups_total) {
        const int64_t i = base + grp;
        const double ax = group_sum(i < n ? row_partial<R, H>(A, x, i, lane) : 0.0);
        if (i < n && lane == 0) {
            const int64_t br = i / H;
            const int a = (int)(i - br * H);
            double d = 1.0;                              // a missing diagonal counts as 1
            bool found = false;
            for (int64_t q = A.row_ptr[br]; q < A.row_ptr[br + 1]; ++q)
                if (A.col[q] == br) {
                    d = found ? d + (double)val[q * H * H + a * H + a] : (double)val[q * H * H + a * H + a];
                    found = true;
                }
            if (!(fabs(d) >= 1e-12)) d = 1.0;
            minv[i] = (R)(1.0 / d);
            const double ri = (double)b[i] - ax;
            r[i] = (R)ri;
            r0h[i] = (R)ri;
            p[i] = (R)ri;
            acc[0] += ri * ri;
            acc[1] += (double)b[i] * (double)b[i];
        }
    }
    block_partials<2>(acc, partial);
}

// fixed-order sum of the per-block partials of ND dots into sc[slot_k]; with
// start set, also the initial scalars (threshold from atol, rtol and ||b||)
template <int ND>
__global__ void k_bicg_reduce(const double* partial, int n, double* sc, int s0, int s1, int start, double atol,
                              double rtol) {
    __shared__ double red[kSolveThreads];
    const int slots[2] = {s0, s1};
    for (int v = 0; v < ND; ++v) {
        double s = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[v * n + i];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) sc[slots[v]] = red[0];
        __syncthreads();
    }
    if (start && threadIdx.x == 0) {
        // rho = r0^ . r = r . r at the start; rr = r . r
        sc[B_RR] = sc[B_RHO];
        const double thr = fmax(atol, rtol * sqrt(sc[B_BB]));
        sc[B_THR2] = thr * thr;
        sc[B_ITER] = 0.0;
        sc[B_DEN] = sc[B_SS] = sc[B_TT] = sc[B_TS] = 0.0;
        sc[B_ALPHA] = sc[B_OMEGA] = 0.0;
        sc[B_FLAG] = sc[B_RR] <= sc[B_THR2] ? 1.0 : 0.0;
    }
}

// p^ = minv p
template <typename R>
__global__ void __launch_bounds__(kSolveThreads) k_bicg_phat(int64_t n, const R* p, const R* minv, R* ph,
                                                             const double* sc) {
    if (sc[B_FLAG] != 0.0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        ph[i] = (R)((double)minv[i] * (double)p[i]);
}

// s = r - alpha v (into r), s^ = minv s; partial s . s
template <typename R>
__global__ void __launch_bounds__(kSolveThreads) k_bicg_s(int64_t n, R* r, const R* v, const R* minv, R* sh,
                                                          double* partial, const double* sc) {
    const BicgState st = bicg_state(sc);
    double acc[1] = {0.0};
    if (!st.stop && !st.brk)
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const double si = (double)r[i] - st.alpha * (double)v[i];
            r[i] = (R)si;
            sh[i] = (R)((double)minv[i] * si);
            acc[0] += si * si;
        }
    block_partials<1>(acc, partial);
}

// x += alpha p^ (+ omega s^), r = s - omega t; partials r . r and r0^ . r
template <typename R>
__global__ void __launch_bounds__(kSolveThreads) k_bicg_x(int64_t n, R* x, R* r, const R* r0h, const R* ph,
                                                          const R* sh, const R* t, double* partial, const double* sc) {
    const BicgState st = bicg_state(sc);
    const bool upd = !st.stop && !st.brk;
    double acc[2] = {0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double ri = (double)r[i];
        if (upd) {
            double xi = (double)x[i] + st.alpha * (double)ph[i];
            if (!st.sconv) {
                xi += st.omega * (double)sh[i];
                ri -= st.omega * (double)t[i];
                r[i] = (R)ri;
            }
            x[i] = (R)xi;
        }
        acc[0] += ri * ri;
        acc[1] += (double)r0h[i] * ri;
    }
    block_partials<2>(acc, partial);
}

// p = r + beta (p - omega v)
template <typename R>
__global__ void __launch_bounds__(kSolveThreads) k_bicg_p(int64_t n, const R* r, R* p, const R* v, const double* sc) {
    const BicgState st = bicg_state(sc);
    if (st.stop || st.brk || st.sconv || sc[B_RR] <= sc[B_THR2] || st.omega == 0.0) return;
    const double beta = (sc[B_RHO_NEW] / sc[B_RHO]) * (st.alpha / st.omega);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (R)((double)r[i] + beta * ((double)p[i] - st.omega * (double)v[i]));
}

// the end of an iteration: flag (1 converged, 2 breakdown), rho, counter
__global__ void k_bicg_commit(double* sc) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const BicgState st = bicg_state(sc);
    if (st.stop) return;
    sc[B_ITER] += 1.0;
    sc[B_ALPHA] = st.alpha;
    sc[B_OMEGA] = st.omega;
    if (st.brk)
        sc[B_FLAG] = 2.0;
    else if (st.sconv || sc[B_RR] <= sc[B_THR2])
        sc[B_FLAG] = 1.0;
    else if (st.omega == 0.0)
        sc[B_FLAG] = 2.0;
    else
        sc[B_RHO] = sc[B_RHO_NEW];
}

template <typename R, int H>
int bicg_start(const tm_bicgstab_args& a, cudaStream_t st) {
    const int64_t n = a.A.n_rows * H;
    R* w = static_cast<R*>(a.work);
    const int g = grid_rows(n);
    k_bicg_start<R, H><<<g, kSolveThreads, 0, st>>>(a.A, static_cast<const R*>(a.b), static_cast<const R*>(a.x),
                                                      w, w + n, w + 2 * n, w + 7 * n, a.partials);
    k_bicg_reduce<2><<<1, kSolveThreads, 0, st>>>(a.partials, g, a.scalars, B_RHO, B_BB, 1, a.atol, a.rtol);
    return status("tm_bicgstab_start");
}

template <typename R, int H>
int bicg_iterate(const tm_bicgstab_args& a, int n_iter, cudaStream_t st) {
    const int64_t n = a.A.n_rows * H;
    R* w = static_cast<R*>(a.work);
    R *r = w, *r0h = w + n, *p = w + 2 * n, *v = w + 3 * n, *ph = w + 4 * n, *sh = w + 5 * n, *t = w + 6 * n,
      *minv = w + 7 * n;
    R* x = static_cast<R*>(a.x);
    const int gr = grid_rows(n), gv = grid_vec(n);
    double* sc = a.scalars;
    for (int it = 0; it < n_iter; ++it) {
        k_bicg_phat<R><<<gv, kSolveThreads, 0, st>>>(n, p, minv, ph, sc);
        k_bicg_spmv<R, H, 1><<<gr, kSolveThreads, 0, st>>>(a.A, ph, v, r0h, nullptr, a.partials, sc, 0);
        k_bicg_reduce<1><<<1, kSolveThreads, 0, st>>>(a.partials, gr, sc, B_DEN, 0, 0, 0.0, 0.0);
        k_bicg_s<R><<<gv, kSolveThreads, 0, st>>>(n, r, v, minv, sh, a.partials, sc);
        k_bicg_reduce<1><<<1, kSolveThreads, 0, st>>>(a.partials, gv, sc, B_SS, 0, 0, 0.0, 0.0);
        k_bicg_spmv<R, H, 2><<<gr, kSolveThreads, 0, st>>>(a.A, sh, t, nullptr, r, a.partials, sc, 1);
        k_bicg_reduce<2><<<1, kSolveThreads, 0, st>>>(a.partials, gr, sc, B_TT, B_TS, 0, 0.0, 0.0);
        k_bicg_x<R><<<gv, kSolveThreads, 0, st>>>(n, x, r, r0h, ph, sh, t, a.partials, sc);
        k_bicg_reduce<2><<<1, kSolveThreads, 0, st>>>(a.partials, gv, sc, B_RR, B_RHO_NEW, 0, 0.0, 0.0);
        k_bicg_p<R><<<gv, kSolveThreads, 0, st>>>(n, r, p, v, sc);
        k_bicg_commit<<<1, 32, 0, st>>>(sc);
    }
    return status("tm_bicgstab_iterate");
}

int check_op(const tm_linear_operator& A) {
    if (A.n_rows < 0 || (A.n_rows > 0 && (!A.row_ptr || !A.values || !A.col)))
        return tm_set_error(TM_ERR_INVALID_ARG, "linear operator: null arrays");
    return TM_OK;
}

}  // namespace tmk

using namespace tmk;

extern "C" int tm_spmv(const tm_linear_operator* A, const void* x, void* y, double alpha, double beta,
                       tm_stream_t stream) {
    if (!A || !x || !y) return tm_set_error(TM_ERR_INVALID_ARG, "tm_spmv: null argument");
    int s = check_op(*A);
    if (s) return s;
    if (A->n_rows == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return dispatch_op(*A, [&](auto r, auto h) {
        return spmv_op<decltype(r), decltype(h)::value>(*A, x, y, alpha, beta, st);
    });
}

extern "C" size_t tm_pcg_partials_bytes(void) { return sizeof(double) * 3 * kDotBlocks + 256; }

extern "C" int tm_pcg_iterate_until(const tm_pcg_args* a, int32_t max_iter, double rtol, tm_stream_t stream) {
    if (!a || max_iter < 0 || !(rtol >= 0.0)) return tm_set_error(TM_ERR_INVALID_ARG, "tm_pcg_iterate_until: bad argument");
    int s = check_op(a->A);
    if (s) return s;
    if (!a->x || !a->r || !a->z || !a->p || !a->q || !a->dinv || !a->scalars || !a->partials)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_pcg_iterate_until: null argument");
    if (a->A.n_rows == 0 || max_iter == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return dispatch_op(a->A, [&](auto r, auto h) {
        return pcg_iterate_until<decltype(r), decltype(h)::value>(*a, max_iter, rtol, st);
    });
}

// the solver's device fault word, read and cleared by tm_device_fault
int tmk_take_solve_fault() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, tmk::g_solve_fault, sizeof(int)) != cudaSuccess) return -1;
    if (v) {
        const int zero = 0;
        if (cudaMemcpyToSymbol(tmk::g_solve_fault, &zero, sizeof(int)) != cudaSuccess) return -1;
    }
    return v;
}

extern "C" int tm_pcg_start(const tm_pcg_args* a, tm_stream_t stream) {
    if (!a || !a->b || !a->x || !a->r || !a->z || !a->p || !a->q || !a->dinv || !a->scalars || !a->partials)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_pcg_start: null argument");
    int s = check_op(a->A);
    if (s) return s;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return dispatch_op(a->A, [&](auto r, auto h) { return pcg_start<decltype(r), decltype(h)::value>(*a, st); });
}

extern "C" int tm_pcg_iterate(const tm_pcg_args* a, int32_t n_iter, tm_stream_t stream) {
    if (!a || n_iter < 0) return tm_set_error(TM_ERR_INVALID_ARG, "tm_pcg_iterate: bad argument");
    int s = check_op(a->A);
    if (s) return s;
    if (a->A.n_rows == 0 || n_iter == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return dispatch_op(a->A, [&](auto r, auto h) {
        return pcg_iterate<decltype(r), decltype(h)::value>(*a, n_iter, st);
    });
}

extern "C" int tm_bicgstab_start(const tm_bicgstab_args* a, tm_stream_t stream) {
    if (!a || !a->b || !a->x || !a->work || !a->scalars || !a->partials || !(a->atol >= 0.0) || !(a->rtol >= 0.0))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_bicgstab_start: bad argument");
    int s = check_op(a->A);
    if (s) return s;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return dispatch_op(a->A, [&](auto r, auto h) { return bicg_start<decltype(r), decltype(h)::value>(*a, st); });
}

extern "C" int tm_bicgstab_iterate(const tm_bicgstab_args* a, int32_t n_iter, tm_stream_t stream) {
    if (!a || n_iter < 0 || !a->x || !a->work || !a->scalars || !a->partials)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_bicgstab_iterate: bad argument");
    int s = check_op(a->A);
    if (s) return s;
    if (a->A.n_rows == 0 || n_iter == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    return dispatch_op(a->A, [&](auto r, auto h) {
        return bicg_iterate<decltype(r), decltype(h)::value>(*a, n_iter, st);
    });
}
