// Fused FEM assembly kernels for sm_103a.
//
// One CTA per element chunk (tm_chunk_plan).  Phase 1 computes the element
// locals of the chunk into shared memory: the geometry of
// element/element.py:875-968 and element/transformation.py:1219-1276 (for P1
// simplices once per element, the Jacobian being constant; for P2 and
// quadrilaterals per quadrature point), then the integrand of the form
// summed over quadrature points (assemble/element_assembler.py:190-209,
// builtin.py:61-178).  Phase 2 walks the chunk's targets (CSR positions or
// nodes) in increasing order and adds their contributions from shared
// memory in a fixed order (element, then local entry), replacing
// ReduceProjector's index_add_ (assemble/projector.py:95-123).  Targets
// touched by one chunk only are written directly -- for symmetric forms the
// value is also written to the transposed CSR position.  For the others
// each chunk writes a partial, and k_matrix_finalize sums each shared
// target's partials in chunk order (the node-plan kernels instead let the
// last chunk to deliver a partial do that sum, see tm_reduce.cuh).  No
// floating-point value is accumulated atomically: results are bitwise
// reproducible run to run.
//
// Float64 forms do their arithmetic in double-float on the FP32 pipes
// (tm_df64.cuh; the FP64 rate of this GPU is 1/62 of its FP32 rate): the P1
// diffusion / mass kernels from the FP64 coordinate differences on, and on
// every other element type all forms, on per-element power-of-two scaled
// values, scaled back exactly before the compensated target sums.  A chunk
// whose data leave the double-float range runs the same computation in
// FP64 (counted in tm_matrix_args.stats).  Elasticity on P1 simplices and
// all float32 forms use the arithmetic of their type.
#include "tm_assemble_kernels.cuh"
#include "tm_assemble_quad.h"

namespace tmk {

template <typename R>
int dispatch_matrix(const tm_matrix_args& a, cudaStream_t st) {
    switch (a.tables.element_type) {
        case TM_TRI3: return dispatch_forms<R, TM_TRI3>(a, st);
        case TM_TET4: return dispatch_forms<R, TM_TET4>(a, st);
        case TM_TRI6: return dispatch_forms<R, TM_TRI6>(a, st);
        case TM_TET10: return dispatch_forms<R, TM_TET10>(a, st);
        case TM_QUAD4:
        case TM_QUAD9: return quad_matrix(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix: unknown element type");
    }
}

template <typename R>
int dispatch_vector(const tm_vector_args& a, cudaStream_t st) {
    switch (a.tables.element_type) {
        case TM_TRI3: return dispatch_source<R, TM_TRI3>(a, st);
        case TM_TET4: return dispatch_source<R, TM_TET4>(a, st);
        case TM_TRI6: return dispatch_source<R, TM_TRI6>(a, st);
        case TM_TET10: return dispatch_source<R, TM_TET10>(a, st);
        case TM_QUAD4:
        case TM_QUAD9: return quad_vector(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_vector: unknown element type");
    }
}

inline int basis_of(int et) {
    switch (et) {
        case TM_TRI3: return 3;
        case TM_TET4: return 4;
        case TM_TRI6: return 6;
        case TM_TET10: return 10;
        case TM_QUAD4: return 4;
        case TM_QUAD9: return 9;
        default: return -1;
    }
}

int check_plan(const tm_chunk_plan& P, int B, int n_local, const char* who) {
    char buf[256];
    if (P.n_basis != B || P.n_local != n_local) {
        snprintf(buf, sizeof(buf), "%s: plan has %d basis / %d local entries, expected %d / %d", who,
                 P.n_basis, P.n_local, B, n_local);
        return tm_set_error(TM_ERR_INVALID_ARG, buf);
    }
    if (P.n_elements > 0 && (!P.elem_perm || !P.conn || !P.chunk_begin || !P.slot_ptr || !P.contrib ||
                             !P.slot_target || !P.slot_mirror))
        return tm_set_error(TM_ERR_INVALID_ARG, "plan arrays must not be null");
    if (P.n_shared > 0 && (!P.shared_ptr || !P.shared_target || !P.shared_mirror))
        return tm_set_error(TM_ERR_INVALID_ARG, "plan shared arrays must not be null");
    if (P.n_elements > 0 && !P.chunk_contrib)
        return tm_set_error(TM_ERR_INVALID_ARG, "plan chunk_contrib must not be null");
    if (P.chunk_elems < 1 || (int64_t)P.chunk_elems * P.n_local * 2 > 65536)
        return tm_set_error(TM_ERR_INVALID_ARG, "plan chunk size out of range");
    return TM_OK;
}

// the arrays k_matrix stages with bulk copies start on 16-byte boundaries,
// and the plan's chunk sizes are consistent with its arrays' lengths
int check_staged(const tm_chunk_plan& P, const char* who) {
    char buf[256];
    const uintptr_t mis = reinterpret_cast<uintptr_t>(P.slot_ptr) | reinterpret_cast<uintptr_t>(P.contrib);
    if (P.n_elements > 0 && (mis & 15u)) {
        snprintf(buf, sizeof(buf), "%s: slot_ptr and contrib must be 16-byte aligned", who);
        return tm_set_error(TM_ERR_INVALID_ARG, buf);
    }
    if (P.n_elements > 0 && (P.max_chunk_slots < 1 || P.max_chunk_contrib < 1)) {
        snprintf(buf, sizeof(buf), "%s: plan max_chunk_slots / max_chunk_contrib not set", who);
        return tm_set_error(TM_ERR_INVALID_ARG, buf);
    }
    return TM_OK;
}

}  // namespace tmk

using namespace tmk;

extern "C" int tm_device_fault(void) {
    if (cudaDeviceSynchronize() != cudaSuccess) return launch_status("tm_device_fault");
    const int own = take_unit_fault(), quad = quad_take_fault(), solver = tmk_take_solve_fault();
    if (own < 0 || quad < 0 || solver < 0) return launch_status("tm_device_fault");
    if (!(own | quad | solver)) return TM_OK;
    return tm_set_error(TM_ERR_DEVICE_WAIT, "a kernel's bounded wait (staged copy or grid barrier) ran out");
}

extern "C" size_t tm_matrix_workspace_bytes(const tm_matrix_args* a) {
    if (!a) return 0;
    const size_t rs = a->dtype == TM_F32 ? 4 : 8;
    int per = 0;
    if (a->forms & TM_FORM_ELASTICITY) {
        const int et = a->tables.element_type;
        const int D = (et == TM_TRI3 || et == TM_TRI6 || et == TM_QUAD4 || et == TM_QUAD9) ? 2 : 3;
        per = D * D;
    } else {
        per = ((a->forms & TM_FORM_DIFFUSION) ? 1 : 0) + ((a->forms & TM_FORM_MASS) ? 1 : 0);
    }
    return rs * (size_t)a->plan.n_partials * per;
}

extern "C" int tm_assemble_matrix(const tm_matrix_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: null args");
    const int B = basis_of(a->tables.element_type);
    if (B < 0) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix: unknown element type");
    int s = check_plan(a->plan, B, B * (B + 1) / 2, "tm_assemble_matrix");
    if (s) return s;
    if ((a->forms & TM_FORM_ELASTICITY) && (a->forms & ~TM_FORM_ELASTICITY))
        return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix: elasticity cannot be fused with other forms");
    if (!a->tables.packed || a->tables.n_quad < 1)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: missing element tables");
    if (a->plan.n_elements > 0 && !a->points)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: points is null");
    if (a->plan.n_elements > 0 &&
        (((a->forms & TM_FORM_DIFFUSION) && !a->out_diffusion) || ((a->forms & TM_FORM_MASS) && !a->out_mass) ||
         ((a->forms & TM_FORM_ELASTICITY) && !a->out_elasticity)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: output pointer is null");
    if (a->plan.n_partials > 0 && !a->workspace)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: workspace is null");
    if ((s = check_staged(a->plan, "tm_assemble_matrix"))) return s;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (a->dtype == TM_F64) return dispatch_matrix<double>(*a, st);
    if (a->dtype == TM_F32) return dispatch_matrix<float>(*a, st);
    return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix: dtype must be TM_F64 or TM_F32");
}

extern "C" size_t tm_vector_workspace_bytes(const tm_vector_args* a) {
    if (!a) return 0;
    return align16((a->dtype == TM_F32 ? 4 : 8) * (size_t)a->plan.n_partials * (size_t)a->width) +
           sizeof(int32_t) * (size_t)a->plan.n_shared;
}

extern "C" int tm_assemble_vector(const tm_vector_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_vector: null args");
    const int B = basis_of(a->tables.element_type);
    if (B < 0) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_vector: unknown element type");
    int s = check_plan(a->plan, B, B, "tm_assemble_vector");
    if (s) return s;
    if (!a->tables.packed || a->tables.n_quad < 1)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_vector: missing element tables");
    if (!a->out || (a->plan.n_elements > 0 && !a->points) ||
        (a->source != TM_SOURCE_CONST && a->plan.n_elements > 0 && !a->values))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_vector: null pointer");
    if (a->plan.n_partials > 0 && !a->workspace)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_vector: workspace is null");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (a->dtype == TM_F64) return dispatch_vector<double>(*a, st);
    if (a->dtype == TM_F32) return dispatch_vector<float>(*a, st);
    return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_vector: dtype must be TM_F64 or TM_F32");
}

extern "C" int tm_shape_grad_jxw(int64_t E, const int32_t* conn, const double* points, tm_element_tables tb,
                                 double* grad, double* jxw, tm_stream_t stream) {
    if (E < 0 || (E > 0 && (!conn || !points || !grad || !jxw || !tb.packed)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_shape_grad_jxw: bad arguments");
    if (E == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int g = grid_for(E * tb.n_quad);
    switch (tb.element_type) {
        case TM_TRI3: k_shape_grad_jxw<TM_TRI3><<<g, kThreads, 0, st>>>(E, conn, points, tb, grad, jxw); break;
        case TM_TET4: k_shape_grad_jxw<TM_TET4><<<g, kThreads, 0, st>>>(E, conn, points, tb, grad, jxw); break;
        case TM_TRI6: k_shape_grad_jxw<TM_TRI6><<<g, kThreads, 0, st>>>(E, conn, points, tb, grad, jxw); break;
        case TM_TET10: k_shape_grad_jxw<TM_TET10><<<g, kThreads, 0, st>>>(E, conn, points, tb, grad, jxw); break;
        case TM_QUAD4:
        case TM_QUAD9: return quad_shape_grad_jxw(E, conn, points, tb, grad, jxw, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_shape_grad_jxw: unknown element type");
    }
    return launch_status("k_shape_grad_jxw");
}

template <typename R>
static int run_xq(int64_t E, const int32_t* conn, const void* pts, tm_element_tables tb, void* xq, cudaStream_t st) {
    const int g = grid_for(E * tb.n_quad);
    const R* p = static_cast<const R*>(pts);
    R* o = static_cast<R*>(xq);
    switch (tb.element_type) {
        case TM_TRI3: k_quadrature_points<R, TM_TRI3><<<g, kThreads, 0, st>>>(E, conn, p, tb, o); break;
        case TM_TET4: k_quadrature_points<R, TM_TET4><<<g, kThreads, 0, st>>>(E, conn, p, tb, o); break;
        case TM_TRI6: k_quadrature_points<R, TM_TRI6><<<g, kThreads, 0, st>>>(E, conn, p, tb, o); break;
        case TM_TET10: k_quadrature_points<R, TM_TET10><<<g, kThreads, 0, st>>>(E, conn, p, tb, o); break;
        case TM_QUAD4:
        case TM_QUAD9: return quad_quadrature_points(std::is_same<R, float>::value, E, conn, pts, tb, xq, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_quadrature_points: unknown element type");
    }
    return launch_status("k_quadrature_points");
}

extern "C" int tm_quadrature_points(int32_t dtype, int64_t E, const int32_t* conn, const void* points,
                                    tm_element_tables tb, void* xq, tm_stream_t stream) {
    if (E < 0 || (E > 0 && (!conn || !points || !xq || !tb.packed)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_quadrature_points: bad arguments");
    if (E == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (dtype == TM_F64) return run_xq<double>(E, conn, points, tb, xq, st);
    if (dtype == TM_F32) return run_xq<float>(E, conn, points, tb, xq, st);
    return tm_set_error(TM_ERR_INVALID_ARG, "tm_quadrature_points: bad dtype");
}

extern "C" int tm_project_reduce(int32_t dtype, int64_t n_to, int64_t width, const int64_t* seg_ptr,
                                 const int64_t* src, const void* x, void* out, tm_stream_t stream) {
    if (n_to < 0 || width < 1 || (n_to > 0 && (!seg_ptr || !out)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_project_reduce: bad arguments");
    if (n_to == 0) return TM_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int g = grid_for(n_to * width);
    if (dtype == TM_F64)
        k_project<double><<<g, kThreads, 0, st>>>(n_to, width, seg_ptr, src, static_cast<const double*>(x),
                                                  static_cast<double*>(out));
    else if (dtype == TM_F32)
        k_project<float><<<g, kThreads, 0, st>>>(n_to, width, seg_ptr, src, static_cast<const float*>(x),
                                                 static_cast<float*>(out));
    else
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_project_reduce: bad dtype");
    return launch_status("k_project");
}

// ---------------------------------------------------------------------------
// Allocation-free variant of tm_assemble_matrix.
//
// Some callers cannot allocate GPU memory: a host runtime that binds this
// library through a foreign-function interface and only holds device
// pointers handed to it by another framework, or a process whose device
// memory is owned by a fixed pool it may not grow.  They still pass the
// points, coefficients and output arrays, but cannot provide the partial-sum
// workspace.  This entry point runs the same kernels with that workspace
// taken from a file-scope device array of TM_NOALLOC_SCRATCH_BYTES, which
// every GPU that loads the library holds until the process exits.
//
// The array's address is looked up once per device, with that device
// current, by the first call on that device (cudaGetSymbolAddress), and
// again on the first call after the device's context changed (after a
// cudaDeviceReset the module is loaded anew); make that first call before
// any stream capture.  Nothing in the array has to start at zero: each call
// writes every partial it later reads.  If a chunk's bounded wait for its
// staged plan runs out, that chunk writes no partials and the finalising
// kernel sums whatever the previous call left there: as with
// tm_assemble_matrix, check tm_device_fault() before using the results.
// All calls share the one array, so calls whose kernels overlap on the GPU
// (on different streams, or from different host threads) race on it; order
// them on one stream or serialise them.
// ---------------------------------------------------------------------------
#include <cuda.h>
#include <mutex>

namespace tmk {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static void* g_noalloc_ptr[kMaxDevices] = {};
// the context each cached address belongs to: after cudaDeviceReset the
// device gets a new context (new id), the module is loaded again and the
// array may sit elsewhere, so the address is looked up again
static unsigned long long g_noalloc_ctx[kMaxDevices] = {};
static std::mutex g_noalloc_mutex;

// unique id of the calling thread's current context (0 if there is none);
// called with g_noalloc_mutex held.
// The driver functions are fetched through the runtime, so that the library
// does not link the driver library (it also loads on machines without one).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
static unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
        looked_up = true;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

static int noalloc_scratch(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return launch_status("cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix_noalloc: device index above 63");
    // 0 when this host thread has no current context yet: the lookup below
    // binds the device's primary context, and its id is read after it
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    const unsigned long long ctx = current_context_id();
    if (!g_noalloc_ptr[dev] || ctx == 0 || g_noalloc_ctx[dev] != ctx) {
        g_noalloc_ptr[dev] = nullptr;
        void* p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess || !p) {
            char buf[256];
            snprintf(buf, sizeof(buf), "tm_assemble_matrix_noalloc: cudaGetSymbolAddress failed: %s",
                     cudaGetErrorString(err));
            cudaGetLastError();
            return tm_set_error(TM_ERR_CUDA, buf);
        }
        g_noalloc_ptr[dev] = p;
        g_noalloc_ctx[dev] = current_context_id();
    }
    *out = g_noalloc_ptr[dev];
    return TM_OK;
}

}  // namespace tmk

extern "C" int tm_assemble_matrix_noalloc(const tm_matrix_args* a, tm_stream_t stream) {
    if (!a) return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix_noalloc: null args");
    const int B = basis_of(a->tables.element_type);
    if (B < 0) return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix_noalloc: unknown element type");
    int s = check_plan(a->plan, B, B * (B + 1) / 2, "tm_assemble_matrix_noalloc");
    if (s) return s;
    if ((a->forms & TM_FORM_ELASTICITY) && (a->forms & ~TM_FORM_ELASTICITY))
        return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix_noalloc: elasticity cannot be fused with other forms");
    if (!a->tables.packed || a->tables.n_quad < 1)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix_noalloc: missing element tables");
    if (a->plan.n_elements > 0 && !a->points)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix_noalloc: points is null");
    if (a->plan.n_elements > 0 &&
        (((a->forms & TM_FORM_DIFFUSION) && !a->out_diffusion) || ((a->forms & TM_FORM_MASS) && !a->out_mass) ||
         ((a->forms & TM_FORM_ELASTICITY) && !a->out_elasticity)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix_noalloc: output pointer is null");
    if (a->dtype != TM_F64 && a->dtype != TM_F32)
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_assemble_matrix_noalloc: dtype must be TM_F64 or TM_F32");
    if ((s = check_staged(a->plan, "tm_assemble_matrix_noalloc"))) return s;
    const size_t need = tm_matrix_workspace_bytes(a);
    if (need > (size_t)TM_NOALLOC_SCRATCH_BYTES) {
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "tm_assemble_matrix_noalloc: this plan needs %zu bytes of partial sums, above the %zu-byte "
                 "static scratch; use tm_assemble_matrix with a caller-provided workspace",
                 need, (size_t)TM_NOALLOC_SCRATCH_BYTES);
        return tm_set_error(TM_ERR_TOO_LARGE, buf);
    }
    void* scratch = nullptr;
    if ((s = noalloc_scratch(&scratch))) return s;
    tm_matrix_args b = *a;
    b.workspace = scratch;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (b.dtype == TM_F64) return dispatch_matrix<double>(b, st);
    return dispatch_matrix<float>(b, st);
}
