// Device-side construction of the CSR pattern and the element->CSR slot map
// (ElementAssembler.from_mesh, assemble/element_assembler.py:811-851).
//
// The reference forms every local pair (conn[e,i], conn[e,j]) of every
// element, lets SciPy's COO->CSR conversion remove duplicates and sort them
// row-major, and looks every pair up again in an id matrix to get the slot
// map.  Here the same two arrays are built on the GPU without a global sort:
//
//  1. node incidence (the (element, local node) entries of every node) by a
//     counting sort: histogram, exclusive scan, scatter, then each node's
//     short list sorted so that its order does not depend on the scatter's
//     atomic order;
//  2. one warp per row node r gathers the columns of every element incident
//     to r (the candidates); a candidate is the first copy of its value when
//     no earlier candidate equals it, and its rank among the distinct values
//     is the number of first copies of smaller values.  Pass A counts the
//     distinct values (row lengths), an exclusive scan gives the row
//     pointer, pass B writes each distinct value at row_ptr[r] + rank: the
//     row's columns, sorted;
//  3. one thread per (element, local row) finds every column of its row
//     segment by binary search: slot[(e*B + i)*B + j].
//
// Every step is deterministic and the output is, by construction, the
// reference's: unique pairs sorted row-major and the element-major,
// i-major, j-minor slot map.  A row's candidates are held in shared memory,
// kPatWarpCand per warp; a row with more (a node in more than
// kPatWarpCand / B elements) is handled by a whole CTA with kPatBlockCand,
// and beyond that the call returns TM_ERR_TOO_LARGE.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

#include "../../include/tensormesh_gb300.h"
#include "tm_status.h"

namespace {

constexpr int kPatThreads = 256;
constexpr int kPatWarps = kPatThreads / 32;
constexpr int kPatWarpCand = 512;        // candidates per warp (shared memory)
constexpr int kPatBlockCand = 8192;      // candidates of a row done by a whole CTA

int pat_status(const char* what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}

int grid_of(int64_t n, int per) {
    int64_t g = (n + per - 1) / per;
    if (g < 1) g = 1;
    if (g > 152 * 32) g = 152 * 32;
    return (int)g;
}

__global__ void k_incidence_count(const int32_t* conn, int64_t n, int64_t n_points, int32_t* cnt, int32_t* bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = conn[i];
        if (v < 0 || v >= n_points) {
            atomicExch(bad, 1);
            continue;
        }
        atomicAdd(cnt + v, 1);
    }
}

// exclusive scan, in blocks of 1024: out[i] = sum of in[0..i) for i <
// n_out, the input read as zero from n_in on; each block's total goes to
// sums (the block sums are scanned the same way, recursively)
__global__ void k_scan_block(const int32_t* in32, const int64_t* in64, int64_t n_in, int64_t n_out, int64_t* out,
                             int64_t* sums) {
    __shared__ int64_t ws[32];
    const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
    int64_t v = 0;
    if (i < n_in) v = in32 ? (int64_t)in32[i] : in64[i];
    int64_t x = v;                                  // inclusive warp scan
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

__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* offs) {
    const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += offs[blockIdx.x];
}

// int64 temporaries of exclusive_scan over n values
int64_t scan_tmp_elems(int64_t n) {
    const int64_t nb = (n + 1 + 1023) / 1024;
    if (nb <= 1) return 0;
    return nb + (nb + 1) + scan_tmp_elems(nb);
}

// out[0..n] = exclusive scan of the n values (out[n] = their sum)
int exclusive_scan(const int32_t* in32, const int64_t* in64, int64_t n, int64_t* out, int64_t* tmp,
                   cudaStream_t st) {
    const int64_t m = n + 1;
    const int64_t nb = (m + 1023) / 1024;
    int64_t* sums = nb > 1 ? tmp : nullptr;
    k_scan_block<<<(unsigned)nb, 1024, 0, st>>>(in32, in64, n, m, out, sums);
    int s = pat_status("tm_pattern scan");
    if (s) return s;
    if (nb > 1) {
        int64_t* offs = tmp + nb;
        if ((s = exclusive_scan(nullptr, sums, nb, offs, offs + nb + 1, st))) return s;
        k_scan_add<<<(unsigned)nb, 1024, 0, st>>>(out, m, offs);
        if ((s = pat_status("tm_pattern scan"))) return s;
    }
    return TM_OK;
}

__global__ void k_incidence_fill(const int32_t* conn, int64_t n, const int64_t* ptr, int32_t* cursor,
                                 int32_t* inc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = conn[i];
        const int32_t k = atomicAdd(cursor + v, 1);
        inc[ptr[v] + k] = (int32_t)i;                       // element * B + local node
    }
}

// each node's incidence list in increasing order (insertion sort: lists are short)
__global__ void k_incidence_sort(const int64_t* ptr, int64_t n_points, int32_t* inc) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_points;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = ptr[r], b = ptr[r + 1];
        for (int64_t i = a + 1; i < b; ++i) {
            const int32_t x = inc[i];
            int64_t j = i - 1;
            while (j >= a && inc[j] > x) {
                inc[j + 1] = inc[j];
                --j;
            }
            inc[j + 1] = x;
        }
    }
}

// the candidates of a row into buf (their count; -1 when above cap)
template <int B>
__device__ __forceinline__ int gather_row(const int32_t* conn, const int32_t* inc, int64_t a, int64_t b, int32_t* buf,
                                          int cap, int lane, int width) {
    const int n = (int)(b - a) * B;
    if (n > cap) return -1;
    for (int k = lane; k < n; k += width) {
        const int32_t ie = inc[a + k / B];
        const int64_t e = ie / B;
        buf[k] = conn[e * B + (k % B)];
    }
    return n;
}

// first[k] = 1 when candidate k is the first copy of its value
__device__ __forceinline__ void mark_first(const int32_t* buf, int n, uint8_t* first, int lane, int width) {
    for (int k = lane; k < n; k += width) {
        const int32_t c = buf[k];
        bool f = true;
        for (int j = 0; j < k && f; ++j) f = buf[j] != c;
        first[k] = f;
    }
}

// distinct values (their first copies) counted, or (WRITE) written at their
// rank: the number of distinct values below them
template <bool WRITE>
__device__ __forceinline__ int rank_distinct(const int32_t* buf, const uint8_t* first, int n, int lane, int width,
                                             int32_t* out_col, int32_t* out_row, int32_t row) {
    int cnt = 0;
    for (int k = lane; k < n; k += width) {
        if (!first[k]) continue;
        ++cnt;
        if (WRITE) {
            const int32_t c = buf[k];
            int less = 0;
            for (int j = 0; j < n; ++j) less += first[j] && buf[j] < c;
            out_col[less] = c;
            out_row[less] = row;
        }
    }
    return cnt;
}

// pass A (row lengths) or pass B (columns and rows of the pattern), one warp
// per row; rows with more candidates than a warp's buffer are left to the
// CTA-wide kernel (pass A marks them with length -1)
template <int B, bool WRITE>
__global__ void __launch_bounds__(kPatThreads) k_rows_warp(const int32_t* conn, const int64_t* iptr, const int32_t* inc,
                                                           int64_t n_points, int32_t* row_len, const int64_t* row_ptr,
                                                           int32_t* ecol, int32_t* erow) {
    __shared__ int32_t sbuf[kPatWarps][kPatWarpCand];
    __shared__ uint8_t sfirst[kPatWarps][kPatWarpCand];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t r = blockIdx.x * (int64_t)kPatWarps + w; r < n_points; r += (int64_t)gridDim.x * kPatWarps) {
        const int n = gather_row<B>(conn, inc, iptr[r], iptr[r + 1], sbuf[w], kPatWarpCand, lane, 32);
        if (n < 0) {
            if (!WRITE && lane == 0) row_len[r] = -1;
            continue;
        }
        __syncwarp();
        mark_first(sbuf[w], n, sfirst[w], lane, 32);
        __syncwarp();
        if (WRITE) {
            const int64_t o = row_ptr[r];
            rank_distinct<true>(sbuf[w], sfirst[w], n, lane, 32, ecol + o, erow + o, (int32_t)r);
        } else {
            int c = rank_distinct<false>(sbuf[w], sfirst[w], n, lane, 32, nullptr, nullptr, 0);
            for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if (lane == 0) row_len[r] = c;
        }
        __syncwarp();
    }
}

// the rows a warp's buffer could not hold, one CTA each; a row above the
// CTA's buffer sets too_big (the call then fails)
template <int B, bool WRITE>
__global__ void __launch_bounds__(kPatThreads) k_rows_block(const int32_t* conn, const int64_t* iptr, const int32_t* inc,
                                                            int64_t n_points, int32_t* row_len, const int64_t* row_ptr,
                                                            int32_t* ecol, int32_t* erow, int32_t* too_big) {
    __shared__ int32_t sbuf[kPatBlockCand];
    __shared__ uint8_t sfirst[kPatBlockCand];
    __shared__ int red[kPatWarps];
    for (int64_t r = blockIdx.x; r < n_points; r += gridDim.x) {
        const int64_t a = iptr[r], b = iptr[r + 1];
        if ((b - a) * B <= kPatWarpCand) continue;      // done by the warp kernel
        const int n = gather_row<B>(conn, inc, a, b, sbuf, kPatBlockCand, threadIdx.x, kPatThreads);
        if (n < 0) {
            if (threadIdx.x == 0) {
                atomicExch(too_big, 1);
                if (!WRITE) row_len[r] = 0;
            }
            continue;
        }
        __syncthreads();
        mark_first(sbuf, n, sfirst, threadIdx.x, kPatThreads);
        __syncthreads();
        if (WRITE) {
            const int64_t o = row_ptr[r];
            rank_distinct<true>(sbuf, sfirst, n, threadIdx.x, kPatThreads, ecol + o, erow + o, (int32_t)r);
        } else {
            int c = rank_distinct<false>(sbuf, sfirst, n, threadIdx.x, kPatThreads, nullptr, nullptr, 0);
            for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
            __syncthreads();
            if (threadIdx.x == 0) {
                int t = 0;
                for (int k = 0; k < kPatWarps; ++k) t += red[k];
                row_len[r] = t;
            }
        }
        __syncthreads();
    }
}

template <int B>
__global__ void k_slot_map(const int32_t* conn, int64_t n_elements, const int64_t* row_ptr, const int32_t* ecol,
                           int64_t* slot) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_elements * B;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / B;
        const int32_t row = conn[i];
        const int64_t lo0 = row_ptr[row], hi0 = row_ptr[row + 1];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const int32_t c = conn[e * B + j];
            int64_t lo = lo0, hi = hi0;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (ecol[mid] < c)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            slot[i * B + j] = lo;
        }
    }
}

struct PatWorkspace {
    int32_t *cnt, *cursor, *inc, *row_len, *flags;
    int64_t *iptr, *tmp;
    size_t bytes;
};

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

PatWorkspace pat_layout(void* base, int64_t E, int32_t B, int64_t N) {
    PatWorkspace w{};
    unsigned char* p = static_cast<unsigned char*>(base);
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char* q = p ? p + o : nullptr;
        o += al(bytes);
        return q;
    };
    w.cnt = reinterpret_cast<int32_t*>(take(4 * (size_t)N));
    w.cursor = reinterpret_cast<int32_t*>(take(4 * (size_t)N));
    w.row_len = reinterpret_cast<int32_t*>(take(4 * (size_t)N));
    w.flags = reinterpret_cast<int32_t*>(take(16));
    w.inc = reinterpret_cast<int32_t*>(take(4 * (size_t)E * B));
    w.iptr = reinterpret_cast<int64_t*>(take(8 * (size_t)(N + 1)));
    w.tmp = reinterpret_cast<int64_t*>(take(8 * (size_t)scan_tmp_elems(N)));
    w.bytes = o;
    return w;
}

int pat_args(const int32_t* conn, int64_t E, int32_t B, int64_t N, const void* ws, const char* who) {
    char buf[200];
    if (E < 0 || N < 0 || (E > 0 && (!conn || !ws))) {
        snprintf(buf, sizeof(buf), "%s: null pointer or negative size", who);
        return tm_set_error(TM_ERR_INVALID_ARG, buf);
    }
    if (B != 3 && B != 4 && B != 6 && B != 9 && B != 10) {
        snprintf(buf, sizeof(buf), "%s: n_basis must be 3, 4, 6, 9 or 10", who);
        return tm_set_error(TM_ERR_UNSUPPORTED, buf);
    }
    if (E * (int64_t)B >= (int64_t(1) << 31) || N >= (int64_t(1) << 31)) {
        snprintf(buf, sizeof(buf), "%s: n_elements * n_basis and n_points must stay below 2^31", who);
        return tm_set_error(TM_ERR_TOO_LARGE, buf);
    }
    return TM_OK;
}

template <int B>
int count_rows(const int32_t* conn, int64_t N, const PatWorkspace& w, cudaStream_t st) {
    k_rows_warp<B, false><<<grid_of(N, kPatWarps), kPatThreads, 0, st>>>(conn, w.iptr, w.inc, N, w.row_len, nullptr,
                                                                         nullptr, nullptr);
    int s = pat_status("tm_pattern_count");
    if (s) return s;
    k_rows_block<B, false><<<grid_of(N, 1), kPatThreads, 0, st>>>(conn, w.iptr, w.inc, N, w.row_len, nullptr,
                                                                  nullptr, nullptr, w.flags + 1);
    return pat_status("tm_pattern_count");
}

template <int B>
int fill_rows(const int32_t* conn, int64_t E, int64_t N, const PatWorkspace& w, const int64_t* row_ptr, int32_t* erow,
              int32_t* ecol, int64_t* slot, cudaStream_t st) {
    k_rows_warp<B, true><<<grid_of(N, kPatWarps), kPatThreads, 0, st>>>(conn, w.iptr, w.inc, N, w.row_len, row_ptr,
                                                                        ecol, erow);
    int s = pat_status("tm_pattern_fill");
    if (s) return s;
    k_rows_block<B, true><<<grid_of(N, 1), kPatThreads, 0, st>>>(conn, w.iptr, w.inc, N, w.row_len, row_ptr, ecol,
                                                                 erow, w.flags + 1);
    if ((s = pat_status("tm_pattern_fill"))) return s;
    if (E > 0) {
        k_slot_map<B><<<grid_of(E * B, 256), 256, 0, st>>>(conn, E, row_ptr, ecol, slot);
        if ((s = pat_status("tm_pattern_fill"))) return s;
    }
    return TM_OK;
}

}  // namespace

extern "C" size_t tm_pattern_workspace_bytes(int64_t n_elements, int32_t n_basis, int64_t n_points) {
    if (n_elements < 0 || n_points < 0 || n_basis < 1) return 0;
    return pat_layout(nullptr, n_elements, n_basis, n_points).bytes;
}

extern "C" int tm_pattern_count(const int32_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                                void* workspace, int64_t* row_ptr, int64_t* nnz, tm_stream_t stream) {
    int s = pat_args(conn, n_elements, n_basis, n_points, workspace, "tm_pattern_count");
    if (s) return s;
    if (!row_ptr || !nnz) return tm_set_error(TM_ERR_INVALID_ARG, "tm_pattern_count: row_ptr and nnz are required");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const PatWorkspace w = pat_layout(workspace, n_elements, n_basis, n_points);
    const int64_t EB = n_elements * n_basis;
    if (cudaMemsetAsync(w.cnt, 0, 4 * (size_t)n_points, st) != cudaSuccess ||
        cudaMemsetAsync(w.cursor, 0, 4 * (size_t)n_points, st) != cudaSuccess ||
        cudaMemsetAsync(w.flags, 0, 16, st) != cudaSuccess)
        return pat_status("tm_pattern_count");
    if (EB > 0) {
        k_incidence_count<<<grid_of(EB, 256), 256, 0, st>>>(conn, EB, n_points, w.cnt, w.flags);
        if ((s = pat_status("tm_pattern_count"))) return s;
    }
    if ((s = exclusive_scan(w.cnt, nullptr, n_points, w.iptr, w.tmp, st))) return s;
    // a node index out of range stops here, before anything is scattered by it
    int32_t bad_index = 0;
    if (cudaMemcpyAsync(&bad_index, w.flags, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return pat_status("tm_pattern_count");
    if (bad_index) return tm_set_error(TM_ERR_INVALID_ARG, "tm_pattern_count: a node index is outside [0, n_points)");
    if (EB > 0) {
        k_incidence_fill<<<grid_of(EB, 256), 256, 0, st>>>(conn, EB, w.iptr, w.cursor, w.inc);
        if ((s = pat_status("tm_pattern_count"))) return s;
        k_incidence_sort<<<grid_of(n_points, 256), 256, 0, st>>>(w.iptr, n_points, w.inc);
        if ((s = pat_status("tm_pattern_count"))) return s;
    }
    switch (n_basis) {
        case 3: s = count_rows<3>(conn, n_points, w, st); break;
        case 4: s = count_rows<4>(conn, n_points, w, st); break;
        case 6: s = count_rows<6>(conn, n_points, w, st); break;
        case 9: s = count_rows<9>(conn, n_points, w, st); break;
        default: s = count_rows<10>(conn, n_points, w, st); break;
    }
    if (s) return s;
    if ((s = exclusive_scan(w.row_len, nullptr, n_points, row_ptr, w.tmp, st))) return s;
    int32_t too_big = 0;
    if (cudaMemcpyAsync(nnz, row_ptr + n_points, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&too_big, w.flags + 1, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return pat_status("tm_pattern_count");
    if (too_big) {
        char buf[200];
        snprintf(buf, sizeof(buf), "tm_pattern_count: a node lies in more than %d elements", kPatBlockCand / n_basis);
        return tm_set_error(TM_ERR_TOO_LARGE, buf);
    }
    return TM_OK;
}

extern "C" int tm_pattern_fill(const int32_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                               const void* workspace, const int64_t* row_ptr, int32_t* edge_row, int32_t* edge_col,
                               int64_t* slot, tm_stream_t stream) {
    int s = pat_args(conn, n_elements, n_basis, n_points, workspace, "tm_pattern_fill");
    if (s) return s;
    if (n_elements > 0 && (!row_ptr || !edge_row || !edge_col || !slot))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_pattern_fill: null output");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const PatWorkspace w = pat_layout(const_cast<void*>(workspace), n_elements, n_basis, n_points);
    switch (n_basis) {
        case 3: return fill_rows<3>(conn, n_elements, n_points, w, row_ptr, edge_row, edge_col, slot, st);
        case 4: return fill_rows<4>(conn, n_elements, n_points, w, row_ptr, edge_row, edge_col, slot, st);
        case 6: return fill_rows<6>(conn, n_elements, n_points, w, row_ptr, edge_row, edge_col, slot, st);
        case 9: return fill_rows<9>(conn, n_elements, n_points, w, row_ptr, edge_row, edge_col, slot, st);
        default: return fill_rows<10>(conn, n_elements, n_points, w, row_ptr, edge_row, edge_col, slot, st);
    }
}
