// Phase 2 of the node-plan kernels (load vectors, adjoint point gradients):
// the fixed-order reduction of a chunk's per-element, per-node values into
// nodal outputs, with the last-arrival summation of shared nodes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/tensormesh_gb300.h"

namespace tmk {

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// workspace of a node plan with W values per node: partials, then one int32
// counter per shared node
template <typename R>
__host__ __device__ inline size_t node_counters_offset(const tm_chunk_plan& P, int W) {
    return align16(sizeof(R) * (size_t)W * (size_t)P.n_partials);
}

// LV[(el*B + a)*W + w]: value of local node a of chunk element el.  Targets
// touched only by this chunk are written to out[node*W + w]; for the others
// this chunk's partial is published and the last chunk to publish one (a
// counter per shared node, cleared before the launch) sums the node's
// partials in chunk order.  No thread waits on another.
template <typename R, int W>
__device__ __forceinline__ void node_reduce(const tm_chunk_plan& P, const R* LV, R* out, void* workspace) {
    const int32_t s0 = P.chunk_begin[blockIdx.x], s1 = P.chunk_begin[blockIdx.x + 1];
    R* part = static_cast<R*>(workspace);
    int32_t* counters = reinterpret_cast<int32_t*>(static_cast<unsigned char*>(workspace) +
                                                   node_counters_offset<R>(P, W));
    for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        const int p0 = P.slot_ptr[s], p1 = P.slot_ptr[s + 1];
        R acc[W];
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] = 0;
        for (int p = p0; p < p1; ++p) {
            const int idx = P.contrib[p] >> 1;
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] += LV[idx * W + w];
        }
        const int64_t tgt = P.slot_target[s];
        if (tgt < 0) {
            const int64_t pi = -tgt - 1;
#pragma unroll
            for (int w = 0; w < W; ++w) part[pi * W + w] = acc[w];
            continue;
        }
#pragma unroll
        for (int w = 0; w < W; ++w) out[tgt * W + w] = acc[w];
    }
    if (P.n_partials > 0) {
        __threadfence();
        for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            const int32_t tgt = P.slot_target[s];
            if (tgt >= 0) continue;
            const int32_t sh = P.slot_mirror[s];
            const int32_t q0 = P.shared_ptr[sh], q1 = P.shared_ptr[sh + 1];
            if (atomicAdd(counters + sh, 1) != q1 - q0 - 1) continue;
            __threadfence();
            R acc[W];
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] = 0;
            for (int q = q0; q < q1; ++q)
#pragma unroll
                for (int w = 0; w < W; ++w) acc[w] += __ldcg(part + (int64_t)q * W + w);
#pragma unroll
            for (int w = 0; w < W; ++w) out[(int64_t)P.shared_target[sh] * W + w] = acc[w];
        }
    }
}

}  // namespace tmk
