// Assembly kernels instantiated for quadrilaterals ("quad", 4 nodes, and
// "quad9", 9 nodes; element/element.py:1801-1935 of the reference).  Their
// Jacobian varies over the element, so they take the general path of
// k_matrix: geometry per (element, quadrature point) into shared memory,
// then one thread per (element, local pair).  Kept in a translation unit of
// their own so that the library's translation units compile in parallel.
#include "tm_assemble_kernels.cuh"
#include "tm_assemble_quad.h"

namespace tmk {

template <typename R>
static int quad_matrix_r(const tm_matrix_args& a, cudaStream_t st) {
    switch (a.tables.element_type) {
        case TM_QUAD4: return dispatch_forms<R, TM_QUAD4>(a, st);
        case TM_QUAD9: return dispatch_forms<R, TM_QUAD9>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_matrix: unknown element type");
    }
}

int quad_matrix(const tm_matrix_args& a, cudaStream_t st) {
    return a.dtype == TM_F32 ? quad_matrix_r<float>(a, st) : quad_matrix_r<double>(a, st);
}

template <typename R>
static int quad_vector_r(const tm_vector_args& a, cudaStream_t st) {
    switch (a.tables.element_type) {
        case TM_QUAD4: return dispatch_source<R, TM_QUAD4>(a, st);
        case TM_QUAD9: return dispatch_source<R, TM_QUAD9>(a, st);
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_assemble_vector: unknown element type");
    }
}

int quad_vector(const tm_vector_args& a, cudaStream_t st) {
    return a.dtype == TM_F32 ? quad_vector_r<float>(a, st) : quad_vector_r<double>(a, st);
}

int quad_shape_grad_jxw(int64_t E, const int32_t* conn, const double* points, tm_element_tables tb, double* grad,
                        double* jxw, cudaStream_t st) {
    const int g = grid_for(E * tb.n_quad);
    switch (tb.element_type) {
        case TM_QUAD4: k_shape_grad_jxw<TM_QUAD4><<<g, kThreads, 0, st>>>(E, conn, points, tb, grad, jxw); break;
        case TM_QUAD9: k_shape_grad_jxw<TM_QUAD9><<<g, kThreads, 0, st>>>(E, conn, points, tb, grad, jxw); break;
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_shape_grad_jxw: unknown element type");
    }
    return launch_status("k_shape_grad_jxw");
}

template <typename R>
static int quad_xq(int64_t E, const int32_t* conn, const void* pts, tm_element_tables tb, void* xq, cudaStream_t st) {
    const int g = grid_for(E * tb.n_quad);
    const R* p = static_cast<const R*>(pts);
    R* o = static_cast<R*>(xq);
    switch (tb.element_type) {
        case TM_QUAD4: k_quadrature_points<R, TM_QUAD4><<<g, kThreads, 0, st>>>(E, conn, p, tb, o); break;
        case TM_QUAD9: k_quadrature_points<R, TM_QUAD9><<<g, kThreads, 0, st>>>(E, conn, p, tb, o); break;
        default: return tm_set_error(TM_ERR_UNSUPPORTED, "tm_quadrature_points: unknown element type");
    }
    return launch_status("k_quadrature_points");
}

int quad_quadrature_points(bool f32, int64_t E, const int32_t* conn, const void* points, tm_element_tables tb,
                           void* xq, cudaStream_t st) {
    return f32 ? quad_xq<float>(E, conn, points, tb, xq, st) : quad_xq<double>(E, conn, points, tb, xq, st);
}

int quad_take_fault() { return take_unit_fault(); }

}  // namespace tmk
