// Device-side construction of the processing order and of the element-chunk
// reduction plans: the GPU counterpart of tm_morton_order and
// tm_plan_build (tm_plan.cpp), producing the same arrays, so that a mesh
// whose connectivity is on the GPU is planned without a host pass.
//
// * Processing order (tm_morton_order_device): the centroid of every
//   element's vertices and its group's bounding box (atomic min / max on an
//   order-preserving integer image of the doubles), the same quantisation to
//   31 (2-D) or 21 (3-D) bits per axis with the same double operations as
//   the host, the bits interleaved, then a stable LSD radix sort of the
//   codes (8-bit digits) with the element indices as values and, for
//   several groups, a second stable sort by group: the host's order of
//   (group, code, element).
// * Chunk plans (tm_chunk_plan_device): one CTA per chunk forms the chunk's
//   contributions in (element, entry) order, sorts them by (target, order)
//   and the resulting slots by (decreasing count, target) with bitonic
//   sorts in shared memory, and writes slots, mirrors and contribution codes
//   at the chunk's offsets (a first pass counts, a scan places the chunks).
//   Shared targets (touched by more than one chunk) are numbered by
//   decreasing count, then target, through one scan per count class; each
//   shared target's slots, gathered by atomic cursors and sorted, give every
//   slot its partial in chunk order.
// Every step is deterministic; integer atomics only count or reserve
// places whose order is fixed afterwards.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <vector>

#include "../../include/tensormesh_gb300.h"
#include "tm_status.h"

namespace {

int dp_status(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

int dp_grid(int64_t n, int per) {
    int64_t g = (n + per - 1) / per;
    if (g < 1) g = 1;
    if (g > 152 * 32) g = 152 * 32;
    return (int)g;
}

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// bump allocator over a caller's workspace (base == nullptr: sizes only)
struct Bump {
    unsigned char* base;
    size_t off = 0;
    template <class T>
    T* take(size_t n) {
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += al256(sizeof(T) * (n ? n : 1));
        return p;
    }
};

// ------------------------------------------------------------------ scan
__global__ void k_dscan_block(const int32_t* in32, const int64_t* in64, int64_t n_in, int64_t n_out, int64_t* out,
                              int64_t* sums) {
    __shared__ int64_t ws[32];
    const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
    int64_t v = 0;
    if (i < n_in) v = in32 ? (int64_t)in32[i] : in64[i];
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        int64_t t = ws[threadIdx.x];
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (threadIdx.x >= o) t += y;
        }
        ws[threadIdx.x] = t;
    }
    __syncthreads();
    const int64_t before = (threadIdx.x >= 32) ? ws[(threadIdx.x >> 5) - 1] : 0;
    if (i < n_out) out[i] = before + x - v;
    if (threadIdx.x == 1023 && sums) sums[blockIdx.x] = before + x;
}

__global__ void k_dscan_add(int64_t* out, int64_t n, const int64_t* offs) {
    const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += offs[blockIdx.x];
}

int64_t dscan_tmp(int64_t n) {
    const int64_t nb = (n + 1 + 1023) / 1024;
    if (nb <= 1) return 0;
    return nb + (nb + 1) + dscan_tmp(nb);
}

// out[0..n] = exclusive scan of n values (out[n] = their sum)
int dscan(const int32_t* in32, const int64_t* in64, int64_t n, int64_t* out, int64_t* tmp, cudaStream_t st) {
    const int64_t m = n + 1;
    const int64_t nb = (m + 1023) / 1024;
    int64_t* sums = nb > 1 ? tmp : nullptr;
    k_dscan_block<<<(unsigned)nb, 1024, 0, st>>>(in32, in64, n, m, out, sums);
    int s = dp_status("device plan scan");
    if (s) return s;
    if (nb > 1) {
        int64_t* offs = tmp + nb;
        if ((s = dscan(nullptr, sums, nb, offs, offs + nb + 1, st))) return s;
        k_dscan_add<<<(unsigned)nb, 1024, 0, st>>>(out, m, offs);
        if ((s = dp_status("device plan scan"))) return s;
    }
    return TM_OK;
}

// ------------------------------------------------------------------ radix sort
// stable LSD sort of (uint64 key, uint32 value) pairs by 8-bit digits
constexpr int kRsThreads = 256, kRsRounds = 16, kRsTile = kRsThreads * kRsRounds;

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint64_t* keys, int64_t n, int shift, int64_t n_tiles,
                                                       int32_t* hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = blockIdx.x * (int64_t)kRsTile;
    for (int k = threadIdx.x; k < kRsTile; k += kRsThreads) {
        const int64_t i = base + k;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * n_tiles + blockIdx.x] = h[threadIdx.x];
}

// items of a tile in rounds of 256, in index order; within a round a warp
// ranks its lanes by digit (match), warps in order through shared counts
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint64_t* kin, const uint32_t* vin, uint64_t* kout,
                                                          uint32_t* vout, int64_t n, int shift, int64_t n_tiles,
                                                          const int64_t* offs) {
    __shared__ int64_t base[256];
    __shared__ int wcnt[kRsThreads / 32][256];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    base[tid] = offs[(int64_t)tid * n_tiles + blockIdx.x];
    for (int r = 0; r < kRsRounds; ++r) {
        const int64_t i = blockIdx.x * (int64_t)kRsTile + r * kRsThreads + tid;
        const bool valid = i < n;
        uint64_t key = 0;
        uint32_t val = 0;
        int digit = 256;                                   // no valid item matches it
        if (valid) {
            key = kin[i];
            val = vin[i];
            digit = (int)((key >> shift) & 255u);
        }
#pragma unroll
        for (int w = 0; w < kRsThreads / 32; ++w) wcnt[w][tid] = 0;
        __syncthreads();
        const unsigned mask = __match_any_sync(0xffffffffu, digit);
        const int rank = __popc(mask & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][digit] = __popc(mask);
        __syncthreads();
        if (valid) {
            int64_t pos = base[digit] + rank;
            for (int w = 0; w < warp; ++w) pos += wcnt[w][digit];
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        int add = 0;
#pragma unroll
        for (int w = 0; w < kRsThreads / 32; ++w) add += wcnt[w][tid];
        base[tid] += add;
        __syncthreads();
    }
}

struct RsBuffers {
    uint64_t *k0, *k1;
    uint32_t *v0, *v1;
    int32_t* hist;
    int64_t *offs, *tmp;
};

size_t rs_plan(Bump& b, int64_t n, RsBuffers& r) {
    const int64_t tiles = (n + kRsTile - 1) / kRsTile;
    r.k0 = b.take<uint64_t>(n);
    r.k1 = b.take<uint64_t>(n);
    r.v0 = b.take<uint32_t>(n);
    r.v1 = b.take<uint32_t>(n);
    r.hist = b.take<int32_t>(256 * tiles);
    r.offs = b.take<int64_t>(256 * tiles + 1);
    r.tmp = b.take<int64_t>(dscan_tmp(256 * tiles));
    return b.off;
}

// sorts (k0, v0) by the low `bits` bits of the keys; the result is in
// (k0, v0) when the number of passes is even, else in (k1, v1): returned
int radix_sort(RsBuffers& r, int64_t n, int bits, bool& in_second, cudaStream_t st) {
    const int64_t tiles = (n + kRsTile - 1) / kRsTile;
    uint64_t *ki = r.k0, *ko = r.k1;
    uint32_t *vi = r.v0, *vo = r.v1;
    int s = TM_OK;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_hist<<<(unsigned)tiles, kRsThreads, 0, st>>>(ki, n, shift, tiles, r.hist);
        if ((s = dp_status("radix sort"))) return s;
        if ((s = dscan(r.hist, nullptr, 256 * tiles, r.offs, r.tmp, st))) return s;
        k_rs_scatter<<<(unsigned)tiles, kRsThreads, 0, st>>>(ki, vi, ko, vo, n, shift, tiles, r.offs);
        if ((s = dp_status("radix sort"))) return s;
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    in_second = ki == r.k1;
    return TM_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------------ Morton order
// order-preserving int64 image of a double (and back)
__device__ __forceinline__ long long ord_of(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : b ^ 0x7FFFFFFFFFFFFFFFLL;
}
__device__ __forceinline__ double of_ord(long long b) {
    return __longlong_as_double(b >= 0 ? b : b ^ 0x7FFFFFFFFFFFFFFFLL);
}

__device__ __forceinline__ int group_of(const int64_t* groups, int32_t G, int64_t e) {
    int lo = 0, hi = G;                                // groups[lo] <= e < groups[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (groups[mid] <= e)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// centroid of each element's vertices, ((x0 + x1) + x2 ...) / V in the
// host's order, and its group's box.  Each thread keeps a running box of
// its elements (flushed when the group changes); at the end a warp whose
// lanes share one group reduces by shuffles, and a block whose warps share
// one reduces in shared memory, so the box words see a few thousand
// atomics rather than one per element and coordinate.  256 threads.
template <int D>
__global__ void __launch_bounds__(256) k_centroids(const double* pts, const int32_t* conn, int64_t E, int32_t B,
                                                   const int64_t* groups, int32_t G, double* cent, long long* box) {
    constexpr long long kHi = 0x7FFFFFFFFFFFFFFFLL, kLo = -kHi - 1;
    int gc = -1;
    long long mn[D], mx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) mn[d] = kHi, mx[d] = kLo;
    auto flush = [&](int g) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            atomicMin(box + (int64_t)g * 2 * D + d, mn[d]);
            atomicMax(box + (int64_t)g * 2 * D + D + d, mx[d]);
            mn[d] = kHi, mx[d] = kLo;
        }
    };
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int g = groups ? group_of(groups, G, e) : 0;
        if (g != gc) {
            if (gc >= 0) flush(gc);
            gc = g;
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
            double s = pts[(int64_t)conn[e * B] * D + d];
            for (int v = 1; v <= D; ++v) s = __dadd_rn(s, pts[(int64_t)conn[e * B + v] * D + d]);
            s = __ddiv_rn(s, (double)(D + 1));
            cent[e * D + d] = s;
            mn[d] = min(mn[d], ord_of(s));
            mx[d] = max(mx[d], ord_of(s));
        }
    }
    // warp: one group among the lanes that hold a box (-1: none)
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int gw = gc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gw = max(gw, __shfl_xor_sync(full, gw, o));
    const bool wuni = __all_sync(full, gc < 0 || gc == gw);
    if (wuni) {
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                mn[d] = min(mn[d], __shfl_xor_sync(full, mn[d], o));
                mx[d] = max(mx[d], __shfl_xor_sync(full, mx[d], o));
            }
    } else if (gc >= 0) {
        flush(gc);
    }
    // block: one group among the warps that still hold a box
    __shared__ int wg[8];
    __shared__ long long wmn[8][D], wmx[8][D];
    if (lane == 0) {
        wg[warp] = wuni ? gw : -1;
#pragma unroll
        for (int d = 0; d < D; ++d) wmn[warp][d] = mn[d], wmx[warp][d] = mx[d];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        int gb = -1;
        bool buni = true;
        for (int w = 0; w < nw; ++w)
            if (wg[w] >= 0) {
                if (gb < 0) gb = wg[w];
                buni &= wg[w] == gb;
            }
        if (gb >= 0) {
            if (buni) {
#pragma unroll
                for (int d = 0; d < D; ++d) mn[d] = kHi, mx[d] = kLo;
                for (int w = 0; w < nw; ++w)
                    if (wg[w] >= 0)
#pragma unroll
                        for (int d = 0; d < D; ++d) mn[d] = min(mn[d], wmn[w][d]), mx[d] = max(mx[d], wmx[w][d]);
                flush(gb);
            } else {
                for (int w = 0; w < nw; ++w)
                    if (wg[w] >= 0) {
#pragma unroll
                        for (int d = 0; d < D; ++d) mn[d] = wmn[w][d], mx[d] = wmx[w][d];
                        flush(wg[w]);
                    }
            }
        }
    }
}

__device__ __forceinline__ uint64_t spread(uint64_t x, int D) {
    if (D == 2) {
        x &= 0xFFFFFFFFull;
        x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
        x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
        x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
        x = (x | (x << 2)) & 0x3333333333333333ull;
        x = (x | (x << 1)) & 0x5555555555555555ull;
    } else {
        x &= 0x1FFFFFull;
        x = (x | (x << 32)) & 0x1F00000000FFFFull;
        x = (x | (x << 16)) & 0x1F0000FF0000FFull;
        x = (x | (x << 8)) & 0x100F00F00F00F00Full;
        x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
        x = (x | (x << 2)) & 0x1249249249249249ull;
    }
    return x;
}

// Morton code of each element over its group's box (the host's
// floor((c - lo) / span * scale)), and the element index as value
template <int D>
__global__ void k_codes(const double* cent, int64_t E, const int64_t* groups, int32_t G, const long long* box,
                        uint64_t* key, uint32_t* val) {
    const int bits = D == 2 ? 31 : 21;
    const double scale = (double)((1ll << bits) - 1);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int g = groups ? group_of(groups, G, e) : 0;
        uint64_t k = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double lo = of_ord(box[(int64_t)g * 2 * D + d]), hi = of_ord(box[(int64_t)g * 2 * D + D + d]);
            const double span = hi > lo ? __dsub_rn(hi, lo) : 1.0;
            const double q = floor(__dmul_rn(__ddiv_rn(__dsub_rn(cent[e * D + d], lo), span), scale));
            k |= spread((uint64_t)q, D) << d;
        }
        key[e] = k;
        val[e] = (uint32_t)e;
    }
}

__global__ void k_group_keys(const uint32_t* val, int64_t E, const int64_t* groups, int32_t G, uint64_t* key) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x)
        key[i] = (uint64_t)group_of(groups, G, (int64_t)val[i]);
}

__global__ void k_box_fill(long long* box, int64_t G, int D) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G * 2 * D; i += (int64_t)gridDim.x * blockDim.x)
        box[i] = ((i % (2 * D)) < D) ? LLONG_MAX : LLONG_MIN;
}

__global__ void k_copy_perm(const uint32_t* val, int64_t E, int32_t* perm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x)
        perm[i] = (int32_t)val[i];
}

// 1 in *bad when an index lies outside [0, limit)
__global__ void k_check_range32(const int32_t* a, int64_t n, int64_t limit, int32_t* bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (a[i] < 0 || a[i] >= limit) atomicExch(bad, 1);
}
__global__ void k_check_range64(const int64_t* a, int64_t n, int64_t limit, int32_t* bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (a[i] < 0 || a[i] >= limit) atomicExch(bad, 1);
}

// the index arrays a call reads through, checked before any kernel uses
// them as addresses (one small flag copied back; the call synchronises)
int check_indices(const int32_t* conn, int64_t n_conn, int64_t n_points, const int32_t* perm, int64_t n_perm,
                  const int64_t* slot, int64_t n_slot, int64_t nnz, int32_t* flag, cudaStream_t st, const char* who) {
    if (cudaMemsetAsync(flag, 0, 4, st) != cudaSuccess) return dp_status(who);
    if (n_conn > 0) k_check_range32<<<dp_grid(n_conn, 256), 256, 0, st>>>(conn, n_conn, n_points, flag);
    if (perm && n_perm > 0) k_check_range32<<<dp_grid(n_perm, 256), 256, 0, st>>>(perm, n_perm, n_perm, flag);
    if (slot && n_slot > 0) k_check_range64<<<dp_grid(n_slot, 256), 256, 0, st>>>(slot, n_slot, nnz, flag);
    int32_t bad = 0;
    if (cudaMemcpyAsync(&bad, flag, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
        return dp_status(who);
    if (bad) {
        char buf[200];
        snprintf(buf, sizeof(buf), "%s: a node, element or slot index is out of range", who);
        return tm_set_error(TM_ERR_INVALID_ARG, buf);
    }
    return TM_OK;
}

struct MortonWs {
    double* cent;
    long long* box;
    int32_t* flag;
    RsBuffers rs;
    size_t bytes;
};

MortonWs morton_layout(void* ws, int64_t E, int32_t dim, int32_t G) {
    MortonWs m;
    Bump b{static_cast<unsigned char*>(ws)};
    m.flag = b.take<int32_t>(4);
    m.cent = b.take<double>((size_t)E * dim);
    m.box = b.take<long long>((size_t)G * 2 * dim);
    rs_plan(b, E, m.rs);
    m.bytes = b.off;
    return m;
}

}  // namespace

extern "C" size_t tm_morton_workspace_bytes(int64_t n_elements, int32_t dim, int32_t n_groups) {
    if (n_elements < 0 || (dim != 2 && dim != 3) || n_groups < 0) return 0;
    return morton_layout(nullptr, n_elements, dim, n_groups < 1 ? 1 : n_groups).bytes;
}

extern "C" int tm_morton_order_device(const double* points, int64_t n_points, int32_t dim, const int32_t* conn,
                                      int64_t n_elements, int32_t n_basis, const int64_t* groups, int32_t n_groups,
                                      void* workspace, int32_t* perm, tm_stream_t stream) {
    if (n_elements < 0 || n_points < 0 || (dim != 2 && dim != 3) || n_basis < dim + 1 ||
        (n_elements > 0 && (!points || !conn || !perm || !workspace)) || (groups && n_groups < 1))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_morton_order_device: bad arguments");
    if (n_elements > INT32_MAX) return tm_set_error(TM_ERR_TOO_LARGE, "tm_morton_order_device: more than 2^31 elements");
    if (n_elements == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int32_t G = groups ? n_groups : 1;
    MortonWs m = morton_layout(workspace, n_elements, dim, G);
    int s = check_indices(conn, n_elements * n_basis, n_points, nullptr, 0, nullptr, 0, 0, m.flag, st,
                          "tm_morton_order_device");
    if (s) return s;
    k_box_fill<<<dp_grid(G * 2 * dim, 256), 256, 0, st>>>(m.box, G, dim);
    if ((s = dp_status("tm_morton_order_device"))) return s;
    const int g = dp_grid(n_elements, 256);
    const int gc = std::min(g, 152 * 4);                  // a few elements per thread: fewer box atomics
    if (dim == 2) {
        k_centroids<2><<<gc, 256, 0, st>>>(points, conn, n_elements, n_basis, groups, G, m.cent, m.box);
        if ((s = dp_status("tm_morton_order_device"))) return s;
        k_codes<2><<<g, 256, 0, st>>>(m.cent, n_elements, groups, G, m.box, m.rs.k0, m.rs.v0);
    } else {
        k_centroids<3><<<gc, 256, 0, st>>>(points, conn, n_elements, n_basis, groups, G, m.cent, m.box);
        if ((s = dp_status("tm_morton_order_device"))) return s;
        k_codes<3><<<g, 256, 0, st>>>(m.cent, n_elements, groups, G, m.box, m.rs.k0, m.rs.v0);
    }
    if ((s = dp_status("tm_morton_order_device"))) return s;
    bool second = false;
    if ((s = radix_sort(m.rs, n_elements, 64, second, st))) return s;
    const uint32_t* v = second ? m.rs.v1 : m.rs.v0;
    if (groups && G > 1) {
        // stable by group: keys from the sorted values, into (k0, v0)
        if (second) {
            k_group_keys<<<g, 256, 0, st>>>(m.rs.v1, n_elements, groups, G, m.rs.k0);
            if ((s = dp_status("tm_morton_order_device"))) return s;
            cudaMemcpyAsync(m.rs.v0, m.rs.v1, 4 * (size_t)n_elements, cudaMemcpyDeviceToDevice, st);
        } else {
            k_group_keys<<<g, 256, 0, st>>>(m.rs.v0, n_elements, groups, G, m.rs.k0);
        }
        if ((s = dp_status("tm_morton_order_device"))) return s;
        int gbits = 8;
        while ((1ll << gbits) < G) gbits += 8;
        if ((s = radix_sort(m.rs, n_elements, gbits, second, st))) return s;
        v = second ? m.rs.v1 : m.rs.v0;
    }
    k_copy_perm<<<g, 256, 0, st>>>(v, n_elements, perm);
    return dp_status("tm_morton_order_device");
}

namespace {

// ------------------------------------------------------------------ chunk plans
constexpr int kCpThreads = 1024;
constexpr int kCpCap = 8192;          // contributions of one chunk (codes carry 13 bits of order)
constexpr int kCpMaxChunk = 1024;     // elements of one chunk (one thread each)

struct CpSmem {
    uint64_t key1[kCpCap];   // (target << 13 | order), sorted
    uint64_t key2[kCpCap];   // ((65535 - count) << 44 | target << 13 | group), sorted
    int32_t mirror[kCpCap];  // by order; then, by group, the group's mirror
    int32_t gstart[kCpCap];  // by group: first position in key1
    uint16_t code[kCpCap];   // by order
    int32_t scan[kCpThreads];
    int32_t misc[4];
};

__device__ __forceinline__ int cta_exclusive_scan(int v, int32_t* buf, int& total) {
    // inclusive scan of one value per thread (blockDim.x == kCpThreads)
    int x = v;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) buf[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = buf[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        buf[lane] = t;
    }
    __syncthreads();
    const int before = w > 0 ? buf[w - 1] : 0;
    total = buf[31];
    __syncthreads();
    return before + x - v;
}

__device__ __forceinline__ void bitonic_sort(uint64_t* a, int P) {
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & k) == 0;
                    const uint64_t x = a[i], y = a[ixj];
                    if ((x > y) == up) {
                        a[i] = y;
                        a[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
}

// one chunk: its contributions grouped into slots ordered by (decreasing
// count, target).  WRITE = false: the chunk's slot and contribution counts;
// WRITE = true: slots, mirrors, slot pointers and codes at the chunk's offsets
template <bool WRITE>
__global__ void __launch_bounds__(kCpThreads) k_chunk_slots(
    const int32_t* conn_p, const int32_t* perm, const int64_t* slot, int64_t E, int32_t B, int32_t NL, int32_t CH,
    int32_t matrix, int32_t* n_slots, int32_t* n_contrib, int32_t* overflow, const int64_t* slot_off,
    const int64_t* contrib_off, int32_t* slot_target, int32_t* slot_mirror, int32_t* slot_ptr, uint16_t* contrib) {
    extern __shared__ __align__(16) unsigned char smraw[];
    CpSmem& S = *reinterpret_cast<CpSmem*>(smraw);
    const int k = blockIdx.x;
    const int64_t i0 = (int64_t)k * CH;
    const int ne = (int)min((int64_t)CH, E - i0);
    const int t = threadIdx.x;
    // contributions of this thread's element
    int cnt = 0;
    int c[10];
    int64_t e = 0;
    if (t < ne) {
        e = perm[i0 + t];
        for (int a = 0; a < B; ++a) c[a] = conn_p[(i0 + t) * B + a];
        if (matrix) {
            for (int a = 0; a < B; ++a)
                for (int b = a; b < B; ++b) cnt += 1 + (c[a] == c[b] && a != b);
        } else {
            cnt = B;
        }
    }
    int Q;
    const int q0 = cta_exclusive_scan(cnt, S.scan, Q);
    if (Q > kCpCap) {
        if (t == 0) atomicExch(overflow, 1);
        return;
    }
    if (t < ne) {
        int q = q0;
        if (matrix) {
            int l = 0;
            for (int a = 0; a < B; ++a)
                for (int b = a; b < B; ++b, ++l) {
                    const int32_t pab = (int32_t)slot[(e * B + a) * B + b];
                    const int32_t pba = (int32_t)slot[(e * B + b) * B + a];
                    const uint16_t code = (uint16_t)((t * NL + l) << 1);
                    if (c[a] < c[b]) {
                        S.key1[q] = (uint64_t)pab << 13 | q, S.mirror[q] = pba, S.code[q] = code, ++q;
                    } else if (c[a] > c[b]) {
                        S.key1[q] = (uint64_t)pba << 13 | q, S.mirror[q] = pab, S.code[q] = (uint16_t)(code | 1), ++q;
                    } else {
                        S.key1[q] = (uint64_t)pab << 13 | q, S.mirror[q] = pab, S.code[q] = code, ++q;
                        if (a != b) S.key1[q] = (uint64_t)pab << 13 | q, S.mirror[q] = pab, S.code[q] = (uint16_t)(code | 1), ++q;
                    }
                }
        } else {
            for (int a = 0; a < B; ++a, ++q) {
                S.key1[q] = (uint64_t)c[a] << 13 | q;
                S.mirror[q] = -1;
                S.code[q] = (uint16_t)((t * NL + a) << 1);
            }
        }
    }
    int P = 2;
    while (P < Q) P <<= 1;
    for (int j = Q + t; j < P; j += kCpThreads) S.key1[j] = ~0ull;
    __syncthreads();
    bitonic_sort(S.key1, P);
    // groups (runs of one target): per thread a block of consecutive positions
    const int per = (Q + kCpThreads - 1) / kCpThreads;
    const int j0 = min(Q, t * per), j1 = min(Q, j0 + per);
    int nf = 0;
    for (int j = j0; j < j1; ++j) nf += (j == 0 || (S.key1[j] >> 13) != (S.key1[j - 1] >> 13));
    int G;
    int g = cta_exclusive_scan(nf, S.scan, G);
    for (int j = j0; j < j1; ++j)
        if (j == 0 || (S.key1[j] >> 13) != (S.key1[j - 1] >> 13)) S.gstart[g++] = j;
    __syncthreads();
    // slots: by decreasing count, then target (the group's first position
    // keeps its order-sorted contributions together); a group's mirror is
    // its first contribution's
    for (int h = t; h < G; h += kCpThreads) {
        const int s0 = S.gstart[h], s1 = h + 1 < G ? S.gstart[h + 1] : Q;
        const uint64_t tg = S.key1[s0] >> 13;
        S.key2[h] = (uint64_t)(65535 - (s1 - s0)) << 44 | tg << 13 | (uint64_t)h;
    }
    int P2 = 2;
    while (P2 < G) P2 <<= 1;
    for (int h = G + t; h < P2; h += kCpThreads) S.key2[h] = ~0ull;
    __syncthreads();
    if (!WRITE) {
        if (t == 0) {
            n_slots[k] = G;
            n_contrib[k] = Q;
        }
        return;
    }
    bitonic_sort(S.key2, P2);
    // slot lengths in slot order, scanned for the contribution offsets
    const int perG = (G + kCpThreads - 1) / kCpThreads;
    const int h0 = min(G, t * perG), h1 = min(G, h0 + perG);
    int len = 0;
    for (int h = h0; h < h1; ++h) len += 65535 - (int)(S.key2[h] >> 44);
    int tot;
    int off = cta_exclusive_scan(len, S.scan, tot);
    const int64_t so = slot_off[k], co = contrib_off[k];
    for (int h = h0; h < h1; ++h) {
        const int grp = (int)(S.key2[h] & 8191u);
        const int n = 65535 - (int)(S.key2[h] >> 44);
        const int st = S.gstart[grp];
        const int q_first = (int)(S.key1[st] & 8191u);
        slot_target[so + h] = (int32_t)(S.key1[st] >> 13);
        slot_mirror[so + h] = matrix ? S.mirror[q_first] : -1;
        for (int r = 0; r < n; ++r) contrib[co + off + r] = S.code[S.key1[st + r] & 8191u];
        off += n;
        slot_ptr[so + h + 1] = (int32_t)(co + off);
    }
    if (k == 0 && t == 0) slot_ptr[0] = 0;
}

__global__ void k_conn_perm(const int32_t* conn, const int32_t* perm, int64_t E, int32_t B, int32_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E * B; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = conn[(int64_t)perm[i / B] * B + i % B];
}

__global__ void k_offsets32(const int64_t* in, int64_t n, int32_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)in[i];
}

__global__ void k_max2(const int32_t* a, const int32_t* b, int64_t n, int32_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        atomicMax(out, a[i]);
        atomicMax(out + 1, b[i]);
    }
}

__global__ void k_target_counts(const int32_t* slot_target, const int32_t* slot_mirror, int64_t n_slots,
                                int32_t* cpt, int32_t* mirror_of, int32_t matrix) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_slots; s += (int64_t)gridDim.x * blockDim.x) {
        const int32_t tg = slot_target[s];
        atomicAdd(cpt + tg, 1);
        if (matrix) mirror_of[tg] = slot_mirror[s];        // all slots of a target carry the same mirror
    }
}

__global__ void k_count_hist(const int32_t* cpt, int64_t n, int32_t* hist, int32_t max_c) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = cpt[i];
        if (c > 1) atomicAdd(hist + min(c, max_c), 1);
    }
}

__global__ void k_class_flags(const int32_t* cpt, int64_t n, int32_t c, int32_t* flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = cpt[i] == c;
}

__global__ void k_class_assign(const int32_t* cpt, const int64_t* idx, int64_t n, int32_t c, int64_t first,
                               int64_t partial, const int32_t* mirror_of, int32_t matrix, int32_t* shared_index,
                               int32_t* sh_target, int32_t* sh_mirror, int32_t* sh_ptr) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        if (cpt[t] != c) continue;
        const int64_t i = first + idx[t];
        shared_index[t] = (int32_t)i;
        sh_target[i] = (int32_t)t;
        sh_mirror[i] = matrix ? mirror_of[t] : -1;
        sh_ptr[i] = (int32_t)(partial + (i - first) * c);
    }
}

__global__ void k_shared_lists(const int32_t* slot_target, int64_t n_slots, const int32_t* shared_index,
                               const int32_t* sh_ptr, int32_t* cursor, int32_t* list) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_slots; s += (int64_t)gridDim.x * blockDim.x) {
        const int32_t sh = shared_index[slot_target[s]];
        if (sh < 0) continue;
        const int32_t k = atomicAdd(cursor + sh, 1);
        list[sh_ptr[sh] + k] = (int32_t)s;
    }
}

// each shared target's slots in slot (= chunk) order: slot s gets the
// target's next partial
__global__ void k_shared_relabel(const int32_t* sh_ptr, int64_t n_shared, int32_t* list, int32_t* slot_target,
                                 int32_t* slot_mirror) {
    for (int64_t sh = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sh < n_shared;
         sh += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = sh_ptr[sh], b = sh_ptr[sh + 1];
        for (int32_t i = a + 1; i < b; ++i) {
            const int32_t x = list[i];
            int32_t j = i - 1;
            while (j >= a && list[j] > x) {
                list[j + 1] = list[j];
                --j;
            }
            list[j + 1] = x;
        }
        for (int32_t p = a; p < b; ++p) {
            slot_target[list[p]] = -(p + 1);
            slot_mirror[list[p]] = (int32_t)sh;
        }
    }
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void k_chunk_contrib(const int32_t* chunk_begin, const int32_t* slot_ptr, int64_t n, int32_t* out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = slot_ptr[chunk_begin[k]];
}

}  // namespace

namespace {

constexpr int kCpMaxClass = 1023;     // most chunks touching one target

struct CpWs {
    int32_t *cnt_s, *cnt_q, *flags, *cpt, *mirror_of, *shared_index, *classflag, *hist, *cursor, *list;
    int64_t *off_s, *off_q, *tmp, *classidx;
    size_t bytes;
};

CpWs cp_layout(void* ws, int64_t E, int32_t B, int64_t n_targets, int32_t kind, int32_t CH) {
    CpWs w;
    Bump b{static_cast<unsigned char*>(ws)};
    const int64_t n_chunks = CH > 0 ? (E + CH - 1) / CH : 0;
    const int64_t NL = kind == TM_PLAN_KIND_MATRIX ? (int64_t)B * (B + 1) / 2 : B;
    w.cnt_s = b.take<int32_t>(n_chunks);
    w.cnt_q = b.take<int32_t>(n_chunks);
    w.off_s = b.take<int64_t>(n_chunks + 1);
    w.off_q = b.take<int64_t>(n_chunks + 1);
    w.tmp = b.take<int64_t>(dscan_tmp(std::max<int64_t>(n_chunks, n_targets)));
    w.flags = b.take<int32_t>(8);
    w.cpt = b.take<int32_t>(n_targets);
    w.mirror_of = b.take<int32_t>(n_targets);
    w.shared_index = b.take<int32_t>(n_targets);
    w.classflag = b.take<int32_t>(n_targets);
    w.classidx = b.take<int64_t>(n_targets + 1);
    w.hist = b.take<int32_t>(kCpMaxClass + 1);
    w.cursor = b.take<int32_t>(n_targets);
    w.list = b.take<int32_t>(E * NL);
    w.bytes = b.off;
    return w;
}

}  // namespace

extern "C" size_t tm_chunk_plan_device_workspace_bytes(int64_t n_elements, int32_t n_basis, int64_t n_targets,
                                                      int32_t kind, int32_t chunk_elems) {
    if (n_elements < 0 || n_basis < 1 || n_targets < 0 || chunk_elems < 1) return 0;
    return cp_layout(nullptr, n_elements, n_basis, n_targets, kind, chunk_elems).bytes;
}

extern "C" int tm_chunk_plan_device(const int32_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                                    int32_t kind, int32_t chunk_elems, const int32_t* perm, const int64_t* slot,
                                    int64_t nnz, void* workspace, tm_device_chunk_plan* out, tm_stream_t stream) {
    const bool matrix = kind == TM_PLAN_KIND_MATRIX;
    if (!out || n_elements < 0 || n_basis < 1 || n_basis > 10 || n_points < 0 || chunk_elems < 1 ||
        (kind != TM_PLAN_KIND_MATRIX && kind != TM_PLAN_KIND_NODE) ||
        (n_elements > 0 && (!conn || !perm || !workspace || (matrix && !slot))))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_chunk_plan_device: bad arguments");
    const int32_t NL = matrix ? n_basis * (n_basis + 1) / 2 : n_basis;
    if (chunk_elems > kCpMaxChunk || (int64_t)chunk_elems * NL * 2 > 65536)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: chunk_elems above 1024 or its 16-bit codes");
    if (n_points > INT32_MAX || n_elements > INT32_MAX || nnz > INT32_MAX)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: more than 2^31 nodes, elements or CSR entries");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t n_targets = matrix ? nnz : n_points;
    const int64_t n_chunks = (n_elements + chunk_elems - 1) / chunk_elems;
    out->n_chunks = n_chunks;
    out->n_slots = out->n_contrib = out->n_shared = out->n_partials = 0;
    out->max_chunk_slots = out->max_chunk_contrib = 0;
    if (n_elements == 0) return TM_OK;
    CpWs w = cp_layout(workspace, n_elements, n_basis, n_targets, kind, chunk_elems);
    const size_t smem = sizeof(CpSmem);
    int s = check_indices(conn, n_elements * n_basis, n_points, perm, n_elements, matrix ? slot : nullptr,
                          n_elements * n_basis * n_basis, nnz, w.flags + 4, st, "tm_chunk_plan_device");
    if (s) return s;
    if (cudaFuncSetAttribute(k_chunk_slots<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_chunk_slots<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return dp_status("tm_chunk_plan_device");
    k_fill_i32<<<1, 32, 0, st>>>(w.flags, 8, 0);
    k_conn_perm<<<dp_grid(n_elements * n_basis, 256), 256, 0, st>>>(conn, perm, n_elements, n_basis, out->conn);
    if ((s = dp_status("tm_chunk_plan_device"))) return s;
    // pass A: slots and contributions per chunk
    k_chunk_slots<false><<<(unsigned)n_chunks, kCpThreads, smem, st>>>(
        out->conn, perm, slot, n_elements, n_basis, NL, chunk_elems, matrix, w.cnt_s, w.cnt_q, w.flags, nullptr,
        nullptr, nullptr, nullptr, nullptr, nullptr);
    if ((s = dp_status("tm_chunk_plan_device"))) return s;
    if ((s = dscan(w.cnt_s, nullptr, n_chunks, w.off_s, w.tmp, st))) return s;
    if ((s = dscan(w.cnt_q, nullptr, n_chunks, w.off_q, w.tmp, st))) return s;
    k_max2<<<dp_grid(n_chunks, 256), 256, 0, st>>>(w.cnt_s, w.cnt_q, n_chunks, w.flags + 1);
    if ((s = dp_status("tm_chunk_plan_device"))) return s;
    int32_t flags[3] = {0, 0, 0};
    int64_t tot[2] = {0, 0};
    if (cudaMemcpyAsync(flags, w.flags, 12, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&tot[0], w.off_s + n_chunks, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&tot[1], w.off_q + n_chunks, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return dp_status("tm_chunk_plan_device");
    if (flags[0]) return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: a chunk has more than 8192 contributions");
    if (tot[0] > out->cap_slots || tot[1] > out->cap_contrib || tot[0] > INT32_MAX || tot[1] > INT32_MAX)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: slots or contributions above the capacity given");
    const int64_t n_slots = tot[0], n_contrib = tot[1];
    out->n_slots = n_slots;
    out->n_contrib = n_contrib;
    out->max_chunk_slots = flags[1];
    out->max_chunk_contrib = flags[2];
    k_offsets32<<<dp_grid(n_chunks + 1, 256), 256, 0, st>>>(w.off_s, n_chunks + 1, out->chunk_begin);
    if ((s = dp_status("tm_chunk_plan_device"))) return s;
    // pass B: the slots, in chunk order
    k_chunk_slots<true><<<(unsigned)n_chunks, kCpThreads, smem, st>>>(
        out->conn, perm, slot, n_elements, n_basis, NL, chunk_elems, matrix, nullptr, nullptr, w.flags, w.off_s,
        w.off_q, out->slot_target, out->slot_mirror, out->slot_ptr, out->contrib);
    if ((s = dp_status("tm_chunk_plan_device"))) return s;
    k_chunk_contrib<<<dp_grid(n_chunks + 1, 256), 256, 0, st>>>(out->chunk_begin, out->slot_ptr, n_chunks + 1,
                                                                 out->chunk_contrib);
    // chunks touching each target, and the mirror of each
    k_fill_i32<<<dp_grid(n_targets, 256), 256, 0, st>>>(w.cpt, n_targets, 0);
    k_fill_i32<<<dp_grid(n_targets, 256), 256, 0, st>>>(w.shared_index, n_targets, -1);
    k_fill_i32<<<dp_grid(kCpMaxClass + 1, 256), 256, 0, st>>>(w.hist, kCpMaxClass + 1, 0);
    k_target_counts<<<dp_grid(n_slots, 256), 256, 0, st>>>(out->slot_target, out->slot_mirror, n_slots, w.cpt,
                                                            w.mirror_of, matrix);
    k_count_hist<<<dp_grid(n_targets, 256), 256, 0, st>>>(w.cpt, n_targets, w.hist, kCpMaxClass);
    if ((s = dp_status("tm_chunk_plan_device"))) return s;
    std::vector<int32_t> hist(kCpMaxClass + 1);
    if (cudaMemcpyAsync(hist.data(), w.hist, 4 * (kCpMaxClass + 1), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return dp_status("tm_chunk_plan_device");
    if (hist[kCpMaxClass] > 0)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: a target touched by more than 1022 chunks");
    // shared targets: by decreasing count, then target; partials contiguous
    int64_t n_shared = 0, n_partials = 0;
    for (int c = kCpMaxClass - 1; c >= 2; --c) {
        if (hist[c] == 0) continue;
        k_class_flags<<<dp_grid(n_targets, 256), 256, 0, st>>>(w.cpt, n_targets, c, w.classflag);
        if ((s = dp_status("tm_chunk_plan_device"))) return s;
        if ((s = dscan(w.classflag, nullptr, n_targets, w.classidx, w.tmp, st))) return s;
        if (n_shared + hist[c] > out->cap_shared)
            return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: shared targets above the capacity given");
        k_class_assign<<<dp_grid(n_targets, 256), 256, 0, st>>>(w.cpt, w.classidx, n_targets, c, n_shared, n_partials,
                                                                 w.mirror_of, matrix, w.shared_index,
                                                                 out->shared_target, out->shared_mirror,
                                                                 out->shared_ptr);
        if ((s = dp_status("tm_chunk_plan_device"))) return s;
        n_shared += hist[c];
        n_partials += (int64_t)hist[c] * c;
    }
    if (n_partials > INT32_MAX) return tm_set_error(TM_ERR_TOO_LARGE, "tm_chunk_plan_device: more than 2^31 partials");
    const int32_t np32 = (int32_t)n_partials;
    if (cudaMemcpyAsync(out->shared_ptr + n_shared, &np32, 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return dp_status("tm_chunk_plan_device");
    if (n_shared > 0) {
        k_fill_i32<<<dp_grid(n_shared, 256), 256, 0, st>>>(w.cursor, n_shared, 0);
        k_shared_lists<<<dp_grid(n_slots, 256), 256, 0, st>>>(out->slot_target, n_slots, w.shared_index,
                                                               out->shared_ptr, w.cursor, w.list);
        if ((s = dp_status("tm_chunk_plan_device"))) return s;
        k_shared_relabel<<<dp_grid(n_shared, 256), 256, 0, st>>>(out->shared_ptr, n_shared, w.list, out->slot_target,
                                                                 out->slot_mirror);
        if ((s = dp_status("tm_chunk_plan_device"))) return s;
    }
    out->n_shared = n_shared;
    out->n_partials = n_partials;
    if (cudaStreamSynchronize(st) != cudaSuccess) return dp_status("tm_chunk_plan_device");
    return TM_OK;
}
