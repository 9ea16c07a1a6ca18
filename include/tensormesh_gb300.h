/*
 * tensormesh_gb300 -- C ABI of the GB300 (sm_103a) tensorized FEM assembly path.
 *
 * Plain pointers and sizes only.  Every array argument named "device" lives
 * in GPU memory owned by the caller; the library allocates nothing on the
 * GPU inside these calls and keeps no state between them.  Calls are
 * stream-ordered on the stream passed in (0 = legacy default stream) and
 * return a status code (TM_OK = 0).  A launch error is reported as
 * TM_ERR_CUDA; tm_last_error_message() gives the text.
 *
 * The reference (TensorMesh) is pure Python on PyTorch and has no native
 * interface; each entry point below cites the reference function whose work
 * it replaces.  The Python package tensormesh_gb300 binds these with ctypes
 * (tensormesh_gb300/_lib.py).
 */
#ifndef TENSORMESH_GB300_H
#define TENSORMESH_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* tm_stream_t;   /* == cudaStream_t */

/* ---- status codes ------------------------------------------------------ */
#define TM_OK                 0
#define TM_ERR_INVALID_ARG    1   /* bad size, null pointer, unsupported combination */
#define TM_ERR_UNSUPPORTED    2   /* element type / form not built */
#define TM_ERR_CUDA           3   /* kernel launch or runtime error */
#define TM_ERR_PLAN           4   /* plan construction failed (host) */
#define TM_ERR_TOO_LARGE      5   /* size above a documented limit */
#define TM_ERR_DEVICE_WAIT    6   /* a kernel's bounded wait on an asynchronous copy ran out */

/* ---- element types (element/element_type.py:57-87) --------------------- */
#define TM_TRI3   0   /* "triangle"  */
#define TM_TET4   1   /* "tetra"     */
#define TM_TRI6   2   /* "triangle6" */
#define TM_TET10  3   /* "tetra10"   */
#define TM_QUAD4  4   /* "quad": bilinear on [0,1]^2, nodes (0,0) (1,0) (0,1) (1,1) (element/element.py:1801-1816) */
#define TM_QUAD9  5   /* "quad9": biquadratic; vertices, mid-points of edges [[0,1],[0,2],[1,3],[2,3]], centre */

/* ---- floating types ---------------------------------------------------- */
#define TM_F64 0
#define TM_F32 1

/* ---- bilinear forms (bit mask) ----------------------------------------- */
#define TM_FORM_DIFFUSION   1   /* kappa_e grad u . grad v  (assemble/builtin.py:61-62) */
#define TM_FORM_MASS        2   /* rho u v                  (assemble/builtin.py:99-100) */
#define TM_FORM_ELASTICITY  4   /* B^T C(E_e, nu) B         (assemble/builtin.py:172-178) */

/* ---- linear-form sources ------------------------------------------------ */
#define TM_SOURCE_NODAL  0   /* f given at nodes, interpolated with phi (node_assembler.py:389) */
#define TM_SOURCE_CONST  1   /* constant c                  (builtin.py:730-771) */
#define TM_SOURCE_QUAD   2   /* f given per quadrature point (builtin.py:773-813) */

const char* tm_error_string(int status);
const char* tm_last_error_message(void);
int tm_version(void);
/* Device-side fault word of the current device: kernels whose bounded wait
 * on an asynchronous copy ran out set it and skip their remaining work
 * instead of hanging.  Synchronises the device, returns TM_ERR_DEVICE_WAIT
 * when the word was set (and clears it), TM_OK otherwise.  No counterpart
 * in the reference. */
int tm_device_fault(void);

/*
 * Reference-element tables of one (element type, quadrature order): a flat
 * float64 device array [w(Q) | phi(Q*B) | dphi(Q*D*B) | mass_hat(B*B) |
 * load_hat(B) | wsum], see tensormesh_gb300/element.py packed_tables().
 * Replaces the quadrature / shape-function caches of
 * element/transformation.py:266-367 and element/element.py:557-872.
 */
typedef struct tm_element_tables {
    int32_t element_type;      /* TM_TRI3 ... */
    int32_t n_quad;            /* Q */
    const double* packed;      /* device */
} tm_element_tables;

/*
 * Element-chunk reduction plan (built once per mesh by tm_plan_build and
 * copied to the device).  Elements are processed in chunks of chunk_elems
 * consecutive entries of the processing order; each chunk reduces the
 * contributions its elements make to a target (a CSR position for matrix
 * plans, a node for node plans) in shared memory, in a fixed order, and
 * writes either the final value (the target is touched by this chunk only)
 * or a partial.  Matrix plans sum the partials of each shared target in
 * chunk order in a second kernel; node plans let the last chunk to deliver a
 * partial of a shared node (one counter per shared node) do that sum.  No
 * floating-point atomics and no waiting: the result is bitwise reproducible.
 */
typedef struct tm_chunk_plan {
    int64_t n_elements;
    int32_t n_basis;
    int32_t n_local;           /* entries per element: B(B+1)/2 (matrix) or B (node) */
    int32_t chunk_elems;
    int32_t n_chunks;
    int64_t n_targets;         /* nnz (matrix) or n_points (node) */
    int32_t n_shared;          /* targets with contributions from >1 chunk */
    int32_t n_partials;
    const int32_t* elem_perm;      /* [E] processing position -> element id */
    const int32_t* conn;           /* [E*B] connectivity in processing order */
    const int32_t* chunk_begin;    /* [n_chunks+1] */
    const int32_t* slot_ptr;       /* [n_chunk_slots+1]; a chunk's slots by decreasing count */
    const uint16_t* contrib;       /* [n_contrib] ((e_local*n_local + l) << 1) | transpose */
    const int32_t* slot_target;    /* [n_chunk_slots] >= 0 target; < 0: -(partial+1) */
    const int32_t* slot_mirror;    /* [n_chunk_slots] target < 0: its shared index; else the
                                      transposed CSR position (matrix plans) or -1 */
    const int32_t* shared_ptr;     /* [n_shared+1] partial ranges, chunk order; shared
                                      targets by decreasing partial count, then target */
    const int32_t* shared_target;  /* [n_shared] */
    const int32_t* shared_mirror;  /* [n_shared] */
    const int32_t* chunk_contrib;  /* [n_chunks+1] slot_ptr[chunk_begin[k]] */
    int32_t max_chunk_slots;       /* largest chunk_begin[k+1] - chunk_begin[k] */
    int32_t max_chunk_contrib;     /* largest chunk_contrib[k+1] - chunk_contrib[k] */
} tm_chunk_plan;
/* tm_assemble_matrix copies each chunk's part of slot_ptr and contrib into
 * shared memory with bulk asynchronous copies (TMA): these two arrays must
 * start on a 16-byte boundary and stay readable up to the next multiple of 16
 * bytes past their last element (allocate 16 bytes more); the call checks the
 * alignment. */

/*
 * Host-side plan construction (replaces ElementAssembler.from_mesh,
 * assemble/element_assembler.py:811-851, and NodeAssembler.from_elements,
 * assemble/node_assembler.py:665-670).  conn is a host int64 [E*B] array,
 * perm an optional host int32 [E] processing order (NULL = identity).
 * kind: 0 = matrix (CSR pattern + element->CSR slot map + chunk plan),
 *       1 = node   (chunk plan onto nodes).
 * slot_map: optional host int64 [E*B*B] slot map of an earlier matrix plan of
 * the same mesh (NULL = build the pattern); lets one mesh carry chunk plans
 * of several chunk sizes.  A negative entry is rejected (TM_ERR_INVALID_ARG),
 * as are connectivity outside [0, n_points) and a perm that is not a
 * permutation; chunk_elems * n_local * 2 above 65536 gives TM_ERR_TOO_LARGE
 * (contribution codes are 16-bit; n_local = B(B+1)/2 for matrix plans, B for
 * node plans).
 * The CSR pattern is the reference's: unique (row, col) pairs sorted
 * row-major, and the slot map is the element-major, i-major, j-minor
 * position of every local pair in that pattern.
 */
typedef struct tm_host_plan tm_host_plan;
/*
 * Processing order of the elements (host): increasing Morton code of the
 * centroid of each element's first dim+1 nodes (its vertices), quantised to
 * 31 (2-D) or 21 (3-D) bits per axis over the centroids' bounding box; ties
 * keep element order.  points: host float64 [n_points*dim]; conn: host int64
 * [n_elements*n_basis]; perm: host int32 [n_elements] out.  Chunks of
 * consecutive elements in this order are compact regions of the mesh (a
 * locality renumbering; no counterpart in the reference).
 */
int tm_morton_order(const double* points, int64_t n_points, int32_t dim, const int64_t* conn,
                    int64_t n_elements, int32_t n_basis, int32_t* perm);
/* Plan construction and tm_morton_order run on TM_HOST_THREADS host threads
 * (default: all hardware threads); their results do not depend on it. */
#define TM_PLAN_KIND_MATRIX 0
#define TM_PLAN_KIND_NODE   1
int tm_plan_build(const int64_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                  int32_t kind, int32_t chunk_elems, const int32_t* perm, const int64_t* slot_map,
                  tm_host_plan** out);
/* array ids for tm_plan_array_size / tm_plan_copy_array */
#define TM_PLAN_EDGE_ROW      0   /* int32  [nnz]       */
#define TM_PLAN_EDGE_COL      1   /* int32  [nnz]       */
#define TM_PLAN_SLOT          2   /* int64  [E*B*B]     */
#define TM_PLAN_CHUNK_BEGIN   3   /* int32               */
#define TM_PLAN_SLOT_PTR      4   /* int32               */
#define TM_PLAN_CONTRIB       5   /* uint16              */
#define TM_PLAN_SLOT_TARGET   6   /* int32               */
#define TM_PLAN_SLOT_MIRROR   7   /* int32               */
#define TM_PLAN_SHARED_PTR    8   /* int32               */
#define TM_PLAN_SHARED_TARGET 9   /* int32               */
#define TM_PLAN_SHARED_MIRROR 10  /* int32               */
#define TM_PLAN_CONN          11  /* int32  [E*B]        */
#define TM_PLAN_PERM          12  /* int32  [E]          */
#define TM_PLAN_CHUNK_CONTRIB 13  /* int32  [n_chunks+1] */
int64_t tm_plan_array_size(const tm_host_plan* plan, int32_t array_id);   /* elements */
int tm_plan_copy_array(const tm_host_plan* plan, int32_t array_id, void* host_dst);
/* scalars: 0 nnz, 1 n_chunks, 2 n_chunk_slots, 3 n_contrib, 4 n_shared, 5 n_partials, 6 n_local,
 *          7 max_chunk_slots, 8 max_chunk_contrib */
int64_t tm_plan_scalar(const tm_host_plan* plan, int32_t which);
void tm_plan_free(tm_host_plan* plan);

/*
 * Device-side construction of the CSR pattern and the slot map (replaces
 * ElementAssembler.from_mesh's SciPy COO->CSR conversion and id lookup,
 * assemble/element_assembler.py:811-851): the same int32 edges (unique
 * (row, col) pairs sorted row-major) and int64 slot map (element-major,
 * i-major, j-minor), built on the GPU by a node-incidence counting sort and
 * per-row ranking of the candidate columns; deterministic.
 *   conn: device int32 [n_elements*n_basis] (element order), n_basis one of
 *         3, 4, 6, 9, 10; n_elements*n_basis and n_points below 2^31.
 *   workspace: device, tm_pattern_workspace_bytes(...) bytes, shared by the
 *         two calls (tm_pattern_fill reads what tm_pattern_count left there).
 * tm_pattern_count writes row_ptr (device int64 [n_points+1]), synchronises
 * the stream and returns nnz in *nnz (host); a node index outside
 * [0, n_points) gives TM_ERR_INVALID_ARG, a node lying in more than
 * 8192 / n_basis elements TM_ERR_TOO_LARGE.  tm_pattern_fill then writes
 * edge_row, edge_col (device int32 [nnz]) and slot (device int64
 * [n_elements*n_basis*n_basis]), stream-ordered.
 */
size_t tm_pattern_workspace_bytes(int64_t n_elements, int32_t n_basis, int64_t n_points);
int tm_pattern_count(const int32_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                     void* workspace, int64_t* row_ptr, int64_t* nnz, tm_stream_t stream);
int tm_pattern_fill(const int32_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                    const void* workspace, const int64_t* row_ptr, int32_t* edge_row, int32_t* edge_col,
                    int64_t* slot, tm_stream_t stream);

/*
 * Device-side processing order and chunk plans: the GPU counterparts of
 * tm_morton_order and tm_plan_build, producing the same arrays from a
 * connectivity already on the device (no counterpart in the reference, whose
 * from_mesh builds no such plan; they complete the device-side from_mesh).
 *
 * tm_morton_order_device: perm (device int32 [n_elements]) = the elements by
 * increasing Morton code of their vertices' centroid over the bounding box of
 * their group, ties by element index, groups in sequence (groups: device int64
 * [n_groups+1] element offsets, or NULL for one group).  points: device
 * float64 [n_points*dim]; conn: device int32 [n_elements*n_basis]; workspace:
 * tm_morton_workspace_bytes(n_elements, dim, n_groups) bytes.  The order is
 * the host function's.
 *
 * tm_chunk_plan_device: the plan of tm_plan_build (kind TM_PLAN_KIND_MATRIX
 * with the device slot map of tm_pattern_fill and its nnz, or
 * TM_PLAN_KIND_NODE), from device conn (int32, element order) and perm.
 * Outputs go to the caller's device arrays of tm_device_chunk_plan, sized at
 * least: conn [n_elements*n_basis], chunk_begin and chunk_contrib
 * [n_chunks+1], slot_ptr [cap_slots+1], contrib [cap_contrib],
 * slot_target and slot_mirror [cap_slots], shared_ptr [cap_shared+1],
 * shared_target and shared_mirror [cap_shared] (enough: cap_slots =
 * n_elements*n_local, cap_contrib = twice that for matrix plans (n_local for
 * node plans), cap_shared = the number of targets).  The call synchronises
 * its stream and writes the sizes into the struct.  chunk_elems at most
 * 1024; a chunk with more than 8192 contributions or a capacity exceeded
 * gives TM_ERR_TOO_LARGE (tm_plan_build on the host has no such limits).
 */
typedef struct tm_device_chunk_plan {
    int32_t* conn;
    int32_t* chunk_begin;
    int32_t* chunk_contrib;
    int32_t* slot_ptr;
    uint16_t* contrib;
    int32_t* slot_target;
    int32_t* slot_mirror;
    int32_t* shared_ptr;
    int32_t* shared_target;
    int32_t* shared_mirror;
    int64_t cap_slots, cap_contrib, cap_shared;
    /* written by the call */
    int64_t n_chunks, n_slots, n_contrib, n_shared, n_partials;
    int32_t max_chunk_slots, max_chunk_contrib;
} tm_device_chunk_plan;
size_t tm_morton_workspace_bytes(int64_t n_elements, int32_t dim, int32_t n_groups);
int tm_morton_order_device(const double* points, int64_t n_points, int32_t dim, const int32_t* conn,
                           int64_t n_elements, int32_t n_basis, const int64_t* groups, int32_t n_groups,
                           void* workspace, int32_t* perm, tm_stream_t stream);
size_t tm_chunk_plan_device_workspace_bytes(int64_t n_elements, int32_t n_basis, int64_t n_targets,
                                            int32_t kind, int32_t chunk_elems);
int tm_chunk_plan_device(const int32_t* conn, int64_t n_elements, int32_t n_basis, int64_t n_points,
                         int32_t kind, int32_t chunk_elems, const int32_t* perm, const int64_t* slot,
                         int64_t nnz, void* workspace, tm_device_chunk_plan* out, tm_stream_t stream);

/*
 * Float64 P1 diffusion / mass locals and their reduction are computed in
 * double-float arithmetic (hi + lo pairs of floats, ~48 bits, relative
 * error ~1e-14) on the FP32 pipes; chunks whose data fall outside the
 * range where that is exact enough (an element whose largest edge component
 * is outside [2^-20, 2^20], a coefficient outside [2^-30, 2^30], |det J|
 * below 2^-100, a local above 2^100) are recomputed in FP64 arithmetic.
 *
 * Bilinear-form assembly into CSR values (ElementAssembler.__call__,
 * assemble/element_assembler.py:231-445, with Transformation.batch_shape_grad_jxw,
 * element/transformation.py:1219-1276, Element.eval_shape_grad,
 * element/element.py:875-968, and ReduceProjector.__call__,
 * assemble/projector.py:95-123, fused in one pass).
 * Outputs: out_* [nnz] (diffusion, mass) and [nnz*D*D] (elasticity, blocks
 * in [edge, a, b] order as SparseMatrix.from_block_coo expects,
 * sparse/matrix.py:332-381).  workspace: device, >= tm_matrix_workspace_bytes()
 * (the partial sums of shared targets).
 */
typedef struct tm_matrix_args {
    int32_t dtype;             /* TM_F64 / TM_F32: points, coefficients and outputs */
    int32_t forms;             /* TM_FORM_* mask; ELASTICITY cannot be combined */
    int64_t n_points;
    const void* points;        /* device [N*D] */
    const void* kappa;         /* device [E] per-element diffusion coefficient, or NULL */
    double kappa_scale;        /* multiplies kappa (or is kappa when NULL) */
    double mass_scale;         /* rho */
    const void* young;         /* device [E] per-element Young's modulus, or NULL */
    double young_scale;        /* multiplies young (or is E when NULL) */
    double poisson;            /* nu */
    void* out_diffusion;       /* outputs of the forms asked for: [nnz] values, [nnz, D, D] for */
    void* out_mass;            /* elasticity; may be NULL when the plan has no elements */
    void* out_elasticity;
    void* workspace;
    tm_element_tables tables;
    tm_chunk_plan plan;
    void* event_begin;         /* optional cudaEvent_t recorded before the element-chunk kernel */
    void* event_end;           /* optional cudaEvent_t recorded after it (before finalisation) */
    int32_t* stats;            /* optional device int32 [1]: += chunks whose float64 data left the
                                  double-float range (P1 diffusion / mass, and every form on
                                  P2 and quadrilateral elements) and ran in FP64 arithmetic */
    void* event_done;          /* optional cudaEvent_t recorded after the call's last launch */
} tm_matrix_args;
size_t tm_matrix_workspace_bytes(const tm_matrix_args* args);
int tm_assemble_matrix(const tm_matrix_args* args, tm_stream_t stream);

/*
 * Allocation-free variant of tm_assemble_matrix.  It has no counterpart in
 * the reference.  For callers that cannot allocate GPU memory (an FFI host
 * that only holds device pointers given to it by another framework, a
 * process confined to a fixed device pool): same arguments and results, but
 * args->workspace is ignored and the partial sums live in a static device
 * array of TM_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps
 * until exit.  Plans needing more (tm_matrix_workspace_bytes) are rejected
 * with TM_ERR_TOO_LARGE.  The first call on a device (and the first after
 * its context changed, e.g. after cudaDeviceReset) looks the array up with
 * that device current: make it before any stream capture.  Calls share the
 * array and it keeps the last call's partials: calls whose kernels overlap
 * on the GPU race, and a result may be used only after tm_device_fault()
 * reports 0 (a chunk whose bounded wait ran out leaves the previous call's
 * partials in its place).
 */
#define TM_NOALLOC_SCRATCH_BYTES (64u << 20)
int tm_assemble_matrix_noalloc(const tm_matrix_args* args, tm_stream_t stream);

/*
 * Linear-form assembly into a nodal vector (NodeAssembler.__call__,
 * assemble/node_assembler.py:242-409, with const_node_assembler /
 * func_node_assembler, assemble/builtin.py:730-813).
 * values: TM_SOURCE_NODAL [N*width], TM_SOURCE_QUAD [E*Q*width] in element
 * order, ignored for TM_SOURCE_CONST (constant[width]).  out [N*width].
 */
typedef struct tm_vector_args {
    int32_t dtype;
    int32_t source;
    int32_t width;             /* components per node, 1..3 */
    int64_t n_points;
    const void* points;
    const void* values;
    double constant[3];
    void* out;
    void* workspace;
    tm_element_tables tables;
    tm_chunk_plan plan;        /* node plan */
} tm_vector_args;
size_t tm_vector_workspace_bytes(const tm_vector_args* args);
int tm_assemble_vector(const tm_vector_args* args, tm_stream_t stream);

/*
 * Boundary-facet load vectors (FacetAssembler.__call__ for the forms
 * c v, f v with nodal f, and g(x) v, assemble/facet_assembler.py:123-277):
 *   out[i, w] = sum over facet items of sum_q w_q |F_q| g_w(x_q) psi_i(t_q)
 * where an item is one selected (element, facet) pair given by its facet's
 * nodes (plan.conn, facet-local order: vertices, then P2 edge nodes for
 * facet edges [[1,2],[0,2],[0,1]]), psi its own Lagrange basis at the facet
 * quadrature points t_q, and |F| = sqrt(det(F^T F)) the measure of its map
 * from the reference facet (Gauss-Legendre on [0, 1] for lines, the triangle
 * rule for triangles).  The plan is a node plan (tm_plan_build kind 1) over
 * the items' connectivity; the reduction is the deterministic node-plan
 * reduction of tm_assemble_vector.  out [n_points*width] is overwritten.
 */
#define TM_FACET_LINE2  0   /* P1 edge of a triangle, in 2-D */
#define TM_FACET_LINE3  1   /* P2 edge of a triangle6, in 2-D */
#define TM_FACET_TRI3   2   /* P1 face of a tetra, in 3-D */
#define TM_FACET_TRI6   3   /* P2 face of a tetra10, in 3-D */
typedef struct tm_facet_tables {
    int32_t facet_type;        /* TM_FACET_* */
    int32_t n_quad;            /* Q */
    const double* packed;      /* device [w(Q) | psi(Q*Bf) | dpsi(Q*(D-1)*Bf)] */
} tm_facet_tables;
typedef struct tm_facet_vector_args {
    int32_t dtype;
    int32_t source;            /* TM_SOURCE_CONST, TM_SOURCE_NODAL or TM_SOURCE_QUAD */
    int32_t width;             /* 1..3 */
    int32_t pad0;
    int64_t n_points;
    const void* points;        /* [n_points, D] */
    const void* values;        /* NODAL: [n_points, width]; QUAD: [n_items, Q, width], item order */
    double const_value[3];     /* CONST: one value per component */
    void* out;                 /* [n_points, width] */
    void* workspace;           /* tm_facet_vector_workspace_bytes */
    tm_facet_tables tables;
    tm_chunk_plan plan;
} tm_facet_vector_args;
size_t tm_facet_vector_workspace_bytes(const tm_facet_vector_args* args);
int tm_assemble_facet_vector(const tm_facet_vector_args* args, tm_stream_t stream);

/*
 * Gradients of a facet load (float64) for L = sum_i lam_i . out_i: the
 * node coordinates through the facet measure (grad_points [n_points*D],
 * overwritten) and, for a source given per point, dL/dvalues = w_q |F_q|
 * lam(t_q) (grad_values [n_items*Q*width], item order); base as for
 * tm_assemble_facet_vector (its out is not used; its workspace sized by
 * tm_facet_adjoint_workspace_bytes).  Replaces autograd through
 * assemble/facet_assembler.py:123-277.
 */
typedef struct tm_facet_adjoint_args {
    tm_facet_vector_args base;
    const void* lam;           /* [n_points, width] */
    void* grad_points;         /* [n_points, D] or NULL */
    void* grad_values;         /* TM_SOURCE_QUAD: [n_items, Q, width] or NULL */
} tm_facet_adjoint_args;
size_t tm_facet_adjoint_workspace_bytes(const tm_facet_adjoint_args* args);
int tm_facet_adjoint(const tm_facet_adjoint_args* args, tm_stream_t stream);

/*
 * Physical shape gradients and |det J| w per element and quadrature point
 * (Transformation.batch_shape_grad_jxw, element/transformation.py:1219-1276).
 * grad [E*Q*B*D], jxw [E*Q], element order, float64.
 */
int tm_shape_grad_jxw(int64_t n_elements, const int32_t* conn, const double* points,
                      tm_element_tables tables, double* grad, double* jxw, tm_stream_t stream);

/*
 * Deterministic scatter-add (ReduceProjector.__call__, assemble/projector.py:95-123,
 * and SparseProjector.__call__, :217-242): out[t, :] = sum over k in
 * [seg_ptr[t], seg_ptr[t+1]) of x[src[k], :], in src order.
 * src/seg_ptr are the inverse of the projector's index map (tm_project_plan).
 */
int tm_project_reduce(int32_t dtype, int64_t n_to, int64_t width, const int64_t* seg_ptr,
                      const int64_t* src, const void* x, void* out, tm_stream_t stream);

/*
 * Dirichlet static condensation in one launch (Condenser.__call__ and
 * condense_rhs, operator/condense.py:238-337): from the values of the full
 * matrix,
 *   out_kept[k] = values[kept_src[k]]               (the values of K_ii)
 *   out_io[j]   = values[io_src[j]]                 (the values of K_io)
 *   out_rhs[r, w] = rhs[inner_dof[r], w] - sum over q in [row_ptr[r], row_ptr[r+1])
 *                   of values[row_src[q]] * outer_value[row_col[q]]
 * (the same K_io u_o for every trailing column w, as the reference
 * broadcasts it), each row's sum in q order.  The index arrays are the
 * caller's cached layout; no host synchronisation.  Any part may be empty.
 */
typedef struct tm_condense_args {
    int32_t dtype;
    int32_t width;                 /* columns of rhs / out_rhs (trailing dims flattened) */
    const void* values;            /* [nnz] scalar entries of the full matrix */
    int64_t n_kept;
    const int64_t* kept_src;       /* [n_kept] */
    void* out_kept;                /* [n_kept] */
    int64_t n_io;
    const int64_t* io_src;         /* [n_io] */
    void* out_io;                  /* [n_io] */
    int64_t n_inner;
    const int64_t* inner_dof;      /* [n_inner] full index of each inner dof */
    const int64_t* row_ptr;        /* [n_inner+1] K_io entries of each inner row */
    int64_t n_row_entries;         /* row_ptr[n_inner] */
    const int64_t* row_src;        /* [n_row_entries] positions in values */
    const int64_t* row_col;        /* [n_row_entries] outer dof (local index) */
    const void* outer_value;       /* [n_outer] prescribed values u_o */
    const void* rhs;               /* [n_dof, width] */
    void* out_rhs;                 /* [n_inner, width] */
} tm_condense_args;
int tm_condense(const tm_condense_args* args, tm_stream_t stream);

/*
 * Physical coordinates of the quadrature points, x_q = sum_b phi_b(q) X_b
 * (the "x" argument of NodeAssembler forms, node_assembler.py:302-303),
 * xq [E*Q*D], element order.  Used to evaluate func_node_assembler sources.
 */
int tm_quadrature_points(int32_t dtype, int64_t n_elements, const int32_t* conn, const void* points,
                         tm_element_tables tables, void* xq, tm_stream_t stream);

/*
 * Adjoint of P1 diffusion / load assembly (float64): gradients with respect
 * to the per-element coefficient and the node coordinates, recomputing the
 * geometry per element.  Replaces autograd through the reference's assembly
 * graph (assemble/element_assembler.py:390-445 -> element/element.py:960-966
 * -> element/transformation.py:1267-1273) and, for a loss through a linear
 * solve, the adjoint of sparse/solve/torch_sla_solve.py:90-137 combined with
 * it: with k_mode TM_ADJ_K_OUTER the weights dL/dK_ab = -lambda_a u_b are
 * formed per element from the solution u and the adjoint lambda.
 *   k_mode TM_ADJ_K_CSR:   weights[nnz] = dL/dvalues, slot_map [E*B*B] int64
 *   k_mode TM_ADJ_M_CSR:   the same weights on a mass matrix M_e =
 *                          kappa_scale |det J| Mhat (grad_kappa: dL/dM_e
 *                          contracted with |det J| Mhat, per element)
 *   load_source:           adds the term of b = |det J| beta weighted by lam
 * Outputs (either may be NULL): grad_kappa [E] (dL/dkappa, element order),
 * grad_points [N*D] (dL/dx, reduced with the node plan).
 */
#define TM_ADJ_K_NONE   0
#define TM_ADJ_K_CSR    1
#define TM_ADJ_K_OUTER  2
#define TM_ADJ_M_CSR    3
#define TM_ADJ_E_CSR    4
#define TM_ADJ_LOAD_NONE  0
#define TM_ADJ_LOAD_CONST 1
#define TM_ADJ_LOAD_NODAL 2
#define TM_ADJ_LOAD_QUAD  3   /* tm_adjoint_general only: f given per quadrature point */
typedef struct tm_adjoint_args {
    int32_t dtype;             /* TM_F64 */
    int32_t k_mode;
    int32_t load_source;
    int32_t reserved;
    int64_t n_points;
    const void* points;        /* [N*D] */
    const void* kappa;         /* [E] or NULL */
    double kappa_scale;
    const void* weights;       /* TM_ADJ_K_CSR: [nnz] */
    const int64_t* slot_map;   /* TM_ADJ_K_CSR: [E*B*B] */
    const void* u;             /* TM_ADJ_K_OUTER: [N] */
    const void* lam;           /* TM_ADJ_K_OUTER and load term: [N] */
    double load_const;         /* TM_ADJ_LOAD_CONST */
    const void* load_values;   /* TM_ADJ_LOAD_NODAL: [N]; TM_ADJ_LOAD_QUAD: [E*Q], element order */
    void* grad_kappa;          /* [E] or NULL */
    void* grad_points;         /* [N*D] or NULL */
    void* workspace;           /* >= tm_adjoint_workspace_bytes() */
    tm_element_tables tables;
    tm_chunk_plan plan;        /* node plan of the mesh */
    double poisson;            /* TM_ADJ_E_CSR: the Poisson ratio */
} tm_adjoint_args;
size_t tm_adjoint_workspace_bytes(const tm_adjoint_args* args);
int tm_adjoint_p1(const tm_adjoint_args* args, tm_stream_t stream);
/*
 * The same gradients on any element type (P2 triangles and tetrahedra,
 * quadrilaterals, and P1), per quadrature point, for k_mode TM_ADJ_K_CSR
 * (diffusion: grad_kappa and grad_points), TM_ADJ_M_CSR (mass:
 * grad_points), TM_ADJ_E_CSR (isotropic elasticity, weights [nnz, D, D]
 * blocks, kappa the per-element modulus, poisson the ratio: grad_points) or
 * TM_ADJ_K_NONE; a load term (constant or nodal source, weighted by lam)
 * with any k_mode but TM_ADJ_E_CSR; no outer-product weights.
 */
int tm_adjoint_general(const tm_adjoint_args* args, tm_stream_t stream);

/*
 * dL/dc per element of a diffusion matrix (c = kappa) or an isotropic
 * linear-elasticity matrix (c = E), float64, any element type: replaces
 * autograd through the reference's integrand with respect to a per-element
 * coefficient (assemble/element_assembler.py:390-445; for elasticity
 * functional/elasticity.py:132-284).  form: TM_FORM_DIFFUSION (weights =
 * dL/dvalues [nnz]) or TM_FORM_ELASTICITY (weights [nnz, D, D] blocks,
 * poisson the call's Poisson ratio); slot_map [E*B*B] int64 (element
 * order); grad[e] = scale * sum_ab W[slot(e,a,b)] : K_e[a][b](c = 1)
 * (element order), K_e(1) the element's matrix at unit coefficient.
 * plan: a plan of the mesh (its conn and elem_perm).  flags
 * TM_COEF_GRAD_LAME_PARTS (elasticity): grad [2E], grad[e] the contraction
 * with the unit-lam part of K_e (sum_q jw g_a g_b^T) and grad[E + e] with
 * the unit-mu part (sum_q jw (g_b g_a^T + g_a . g_b I)), each times scale;
 * for dL/dnu through lam' = nu / ((1 + nu)(1 - 2 nu)), mu' = 1 / (2 (1 + nu)).
 */
#define TM_COEF_GRAD_LAME_PARTS 1
typedef struct tm_coef_grad_args {
    int32_t form;                  /* TM_FORM_DIFFUSION or TM_FORM_ELASTICITY */
    int32_t flags;                 /* 0 or TM_COEF_GRAD_LAME_PARTS */
    int64_t n_points;
    const void* points;            /* device [N*D] float64 */
    const void* weights;           /* device [nnz] or [nnz*D*D] float64 */
    const int64_t* slot_map;       /* device [E*B*B] */
    double scale;
    double poisson;
    void* grad;                    /* device [E] (or [2E], TM_COEF_GRAD_LAME_PARTS) float64 */
    tm_element_tables tables;
    tm_chunk_plan plan;
} tm_coef_grad_args;
int tm_coef_grad(const tm_coef_grad_args* args, tm_stream_t stream);

/* ---- sparse linear algebra (SparseMatrix @ and solve) ------------------- */
/*
 * CSR (block == 1) or block-CSR (block == H, HxH row-major blocks) operator.
 * Rows sorted by column are not required.  row_order (optional) is the
 * order in which the SpMV and PCG kernels take the (block) rows, a
 * permutation of [0, n_rows): longest rows first keeps the lanes of a warp
 * on rows of equal length.  It changes which lanes compute a row, not the
 * order of the terms of its sum; the dot products of tm_pcg_* follow it.
 * NULL: natural order.  Entries outside [0, n_rows) are skipped.
 */
typedef struct tm_linear_operator {
    int32_t dtype;             /* TM_F64 / TM_F32 */
    int32_t block;             /* 1, 2 or 3 */
    int64_t n_rows;            /* block rows */
    const int64_t* row_ptr;    /* device [n_rows+1] */
    const int32_t* col;        /* device [nnz_blocks] block columns */
    const void* values;        /* device [nnz_blocks*block*block] */
    const int32_t* row_order;  /* device [n_rows] or NULL */
} tm_linear_operator;

/* y = alpha A x + beta y  (SparseMatrix.__matmul__, inherited from torch-sla) */
int tm_spmv(const tm_linear_operator* A, const void* x, void* y, double alpha, double beta,
            tm_stream_t stream);

/*
 * Jacobi-preconditioned CG for SPD A (replaces SparseMatrix.solve for SPD
 * systems; in-tree templates: sparse/solve/torch_solve.py:70-248).
 * tm_pcg_start computes diag(A)^-1, r = b - A x, z, p and the scalars;
 * tm_pcg_iterate runs n_iter iterations without host synchronisation.
 * scalars (device float64 [8]): 0 rz, 1 pAp, 2 rz_new, 3 r.r, 4 b.b,
 * 5 iterations done, 6 flag (0 running, 1 converged (tm_pcg_iterate_until),
 * 2 breakdown: pAp <= 0 or NaN).
 * A breakdown freezes x; convergence is decided by the caller from r.r/b.b.
 */
typedef struct tm_pcg_args {
    tm_linear_operator A;
    const void* b;
    void* x;                   /* initial guess on entry, solution on exit */
    void* r;
    void* z;
    void* p;
    void* q;
    void* dinv;
    double* scalars;
    double* partials;          /* device, tm_pcg_partials_bytes() */
} tm_pcg_args;
size_t tm_pcg_partials_bytes(void);
int tm_pcg_start(const tm_pcg_args* args, tm_stream_t stream);
int tm_pcg_iterate(const tm_pcg_args* args, int32_t n_iter, tm_stream_t stream);
/*
 * Up to max_iter iterations in one cooperative launch (every block resident,
 * grid barriers between the SpMV, the x/r/z update and the p update of each
 * iteration), stopping on the device once r.r <= rtol^2 b.b (flag 1) or on a
 * breakdown (flag 2).  Same scalars as tm_pcg_iterate; dot products in a
 * fixed order, so the result is bitwise reproducible for a given GPU.  A
 * barrier wait that runs out (it cannot while all blocks are resident) ends
 * the launch and sets the word read by tm_device_fault.
 */
int tm_pcg_iterate_until(const tm_pcg_args* args, int32_t max_iter, double rtol, tm_stream_t stream);

/*
 * Jacobi-preconditioned BiCGSTAB for general square systems, replacing the
 * reference's bicgstab_py (sparse/solve/torch_solve.py:130-248; the CUDA
 * fallback of spsolve, sparse/solve/__init__.py:195-246): right
 * preconditioning by 1 / diag(A), a missing or |d| < 1e-12 diagonal taken
 * as 1; breakdown when |r0^ . v| < 1e-12; omega = 0 when t . t < 1e-12 (the
 * iteration then stops); stop when ||s|| or ||r|| <= max(atol, rtol ||b||).
 * tm_bicgstab_start sets r = b - A x, r0^ = r, p = r and the scalars;
 * tm_bicgstab_iterate runs n_iter iterations (11 launches each) without host
 * synchronisation.  work: device [8 * n] of the value type (n = n_rows x
 * block).  scalars: device double [16]: TM_BICG_RR (||r||^2), TM_BICG_BB
 * (||b||^2), TM_BICG_ITER (iterations), TM_BICG_FLAG (0 running, 1
 * converged, 2 breakdown).  Dot products in a fixed order: bitwise
 * reproducible.
 */
#define TM_BICG_RR   5
#define TM_BICG_BB   7
#define TM_BICG_ITER 8
#define TM_BICG_FLAG 9
typedef struct tm_bicgstab_args {
    tm_linear_operator A;
    const void* b;
    void* x;                   /* initial guess on entry, solution on exit */
    void* work;
    double* scalars;
    double* partials;          /* device, tm_pcg_partials_bytes() */
    double atol;
    double rtol;
} tm_bicgstab_args;
int tm_bicgstab_start(const tm_bicgstab_args* args, tm_stream_t stream);
int tm_bicgstab_iterate(const tm_bicgstab_args* args, int32_t n_iter, tm_stream_t stream);

/*
 * Batched Jacobi-PCG over the diagonal blocks [system_offset[s],
 * system_offset[s+1]) of one block-diagonal CSR matrix (offset-concatenated
 * meshes), all systems in one launch; no counterpart in the reference, which
 * solves varying meshes one at a time (batched_workflows.rst:247-249).
 * Rows with dirichlet[i] != 0 keep x[i] as given and are excluded from the
 * iteration (solving K_ii x_i = b_i - K_io x_o).  x holds the initial guess
 * on entry.  work: device [5 * n_rows] of the matrix type.  queue: device
 * int32 [1] (cleared by the call).  status: device [n_systems] or NULL.
 * Convergence: ||r|| <= rtol ||b|| over the free rows of the system.
 */
#define TM_PCG_CONVERGED 1
#define TM_PCG_MAX_ITER  2
#define TM_PCG_BREAKDOWN 3
typedef struct tm_pcg_status {
    int32_t iterations;
    int32_t flag;              /* TM_PCG_* */
    double relative_residual;
} tm_pcg_status;
typedef struct tm_batched_pcg_args {
    int32_t n_systems;
    int32_t max_iter;
    double rtol;
    const int64_t* system_offset;   /* device [n_systems+1] */
    tm_linear_operator A;           /* block == 1 */
    const uint8_t* dirichlet;       /* device [n_rows] or NULL */
    const void* b;
    void* x;
    void* work;
    int32_t* queue;
    tm_pcg_status* status;
    const int32_t* order;           /* device [n_systems]: the queue's order of the systems
                                       (largest first keeps the longest solves off the end);
                                       NULL = 0, 1, ... */
} tm_batched_pcg_args;
int tm_batched_pcg(const tm_batched_pcg_args* args, tm_stream_t stream);

/*
 * The same batch (float64 matrix) by mixed-precision iterative refinement
 * (no counterpart in the reference, whose per-mesh solves run the Jacobi
 * CG of sparse/solve/torch_solve.py:70-127 in the matrix's precision):
 * per system, the float64 residual r = b - A x, a float32 Jacobi-PCG solve
 * of A d = r / ||r|| until its residual falls by inner_rtol, x += ||r|| d in
 * float64, until the true residual meets ||b - A x|| <= rtol ||b|| (the
 * convergence test of tm_batched_pcg) or max_outer corrections or
 * base.max_iter inner iterations in all.  base.work: device [5 * n_rows]
 * float64 (the float64 residual and six float32 vectors); values32: device
 * float [nnz], written by the call.  status.iterations counts the inner
 * iterations; status.relative_residual is the true float64 residual.
 */
typedef struct tm_batched_mixed_args {
    tm_batched_pcg_args base;
    void* values32;
    double inner_rtol;         /* e.g. 1e-4 */
    int32_t max_outer;
    int32_t reserved;
} tm_batched_mixed_args;
int tm_batched_pcg_mixed(const tm_batched_mixed_args* args, tm_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* TENSORMESH_GB300_H */
