// Dirichlet static condensation in one launch (operator/condense.py:238-296):
// the values of K_ii and K_io gathered from the full matrix's values at
// positions cached by the caller, and f_i = rhs[inner] - K_io u_o with each
// inner row's K_io entries summed in a fixed order.  The reference computes
// the same with boolean-mask indexing (a host synchronisation per call) and a
// SparseMatrix product.
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/tensormesh_gb300.h"
#include "tm_status.h"

namespace tmk {
namespace {

constexpr int kCondThreads = 256;

template <typename R>
__global__ void __launch_bounds__(kCondThreads) k_condense(const tm_condense_args a) {
    const R* v = static_cast<const R*>(a.values);
    const R* uo = static_cast<const R*>(a.outer_value);
    const R* rhs = static_cast<const R*>(a.rhs);
    R* okept = static_cast<R*>(a.out_kept);
    R* oio = static_cast<R*>(a.out_io);
    R* orhs = static_cast<R*>(a.out_rhs);
    const int64_t n1 = a.n_kept, n2 = n1 + a.n_io, n3 = n2 + a.n_inner;
    const int W = a.width;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n3; k += (int64_t)gridDim.x * blockDim.x) {
        if (k < n1) {
            okept[k] = v[a.kept_src[k]];
        } else if (k < n2) {
            const int64_t j = k - n1;
            oio[j] = v[a.io_src[j]];
        } else {
            const int64_t r = k - n2;
            R t = 0;
            for (int64_t q = a.row_ptr[r]; q < a.row_ptr[r + 1]; ++q) t += v[a.row_src[q]] * uo[a.row_col[q]];
            const int64_t src = a.inner_dof[r] * W, dst = r * W;
            for (int w = 0; w < W; ++w) orhs[dst + w] = rhs[src + w] - t;
        }
    }
}

}  // namespace
}  // namespace tmk

using namespace tmk;

extern "C" int tm_condense(const tm_condense_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_condense: null args");
    if (a->dtype != TM_F64 && a->dtype != TM_F32)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_condense: dtype must be TM_F64 or TM_F32");
    if (a->n_kept < 0 || a->n_io < 0 || a->n_inner < 0 || a->n_row_entries < 0 || a->width < 1)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_condense: negative size or width < 1");
    if ((a->n_kept > 0 && (!a->kept_src || !a->out_kept)) || (a->n_io > 0 && (!a->io_src || !a->out_io)) ||
        (a->n_inner > 0 && (!a->inner_dof || !a->row_ptr || !a->rhs || !a->out_rhs)) ||
        (a->n_row_entries > 0 && (!a->row_src || !a->row_col || !a->outer_value)) ||
        ((a->n_kept > 0 || a->n_io > 0 || a->n_inner > 0) && !a->values))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_condense: null array for a non-empty part");
    const int64_t total = a->n_kept + a->n_io + a->n_inner;
    if (total == 0) return TM_OK;
    int64_t blocks = (total + kCondThreads - 1) / kCondThreads;
    if (blocks > 152 * 32) blocks = 152 * 32;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (a->dtype == TM_F64)
        k_condense<double><<<(unsigned)blocks, kCondThreads, 0, st>>>(*a);
    else
        k_condense<float><<<(unsigned)blocks, kCondThreads, 0, st>>>(*a);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "tm_condense: %s", cudaGetErrorString(err));
        return tm_set_error(TM_ERR_CUDA, buf);
    }
    return TM_OK;
}
