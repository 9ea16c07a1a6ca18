// Quadrilateral instantiations of the assembly kernels (tm_assemble_quad.cu),
// called by the element-type dispatch of tm_assemble.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tensormesh_gb300.h"

namespace tmk {

// a.tables.element_type is TM_QUAD4 or TM_QUAD9; arguments already checked
int quad_matrix(const tm_matrix_args& a, cudaStream_t st);
int quad_vector(const tm_vector_args& a, cudaStream_t st);
int quad_shape_grad_jxw(int64_t E, const int32_t* conn, const double* points, tm_element_tables tb, double* grad,
                        double* jxw, cudaStream_t st);
int quad_quadrature_points(bool f32, int64_t E, const int32_t* conn, const void* points, tm_element_tables tb,
                           void* xq, cudaStream_t st);
// the quadrilateral unit's device fault word, read and cleared (-1 on a CUDA error)
int quad_take_fault();

}  // namespace tmk
