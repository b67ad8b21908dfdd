/*
 * tensormesh_gb300 -- C ABI of the GB300 (sm_103a) finite-element hot path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*, the caller's cudaStream_t), never allocates, never
 * synchronises the stream (except where stated), and returns an int status:
 *
 *   TM_OK            0  success
 *   TM_ERR_INVALID   1  bad argument (null pointer, unsupported combination)
 *   TM_ERR_INDEX     2  an index or size out of range
 *   TM_ERR_MAXITER   3  iterative solver hit its iteration cap
 *   TM_ERR_BREAKDOWN 4  iterative solver breakdown (p^T A p <= 0, NaN)
 *   TM_ERR_CUDA      5  a CUDA launch failed
 *   TM_ERR_UNSUPPORTED 6 element/form/dtype combination not built
 *   TM_ERR_TIMEOUT   7  a bounded device-side wait gave up
 *
 * Citations name the reference (TensorMesh) interface each entry replaces.
 */
#ifndef TENSORMESH_GB300_H
#define TENSORMESH_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TM_OK 0
#define TM_ERR_INVALID 1
#define TM_ERR_INDEX 2
#define TM_ERR_MAXITER 3
#define TM_ERR_BREAKDOWN 4
#define TM_ERR_CUDA 5
#define TM_ERR_UNSUPPORTED 6
#define TM_ERR_TIMEOUT 7

/* element types: "triangle", "triangle6", "tetra", "tetra10" */
#define TM_TRI3 0
#define TM_TRI6 1
#define TM_TET4 2
#define TM_TET10 3

/* integrands (assemble/builtin.py): Laplace gradu@gradv (62-63), mass u*v
 * (100-101), isotropic linear elasticity Ba^T C Bb (173-179), load c*v /
 * f(x)*v / f*v (886-969) */
#define TM_FORM_LAPLACE 0
#define TM_FORM_MASS 1
#define TM_FORM_ELASTICITY 2
#define TM_FORM_LOAD 3

#define TM_F32 0
#define TM_F64 1

/* FP64 arithmetic: emulated double-float on the FP32 pipe (default) or
 * native FP64 instructions (slow on GB300; kept as a cross-check). */
#define TM_PREC_EMULATED 0
#define TM_PREC_NATIVE 1

/* where the coefficient of the integrand comes from */
#define TM_COEF_SCALAR 0   /* scal[0..H-1]                          */
#define TM_COEF_ELEMENT 1  /* coef[E]          (element_data)        */
#define TM_COEF_POINT 2    /* coef[N*H]        (point_data, interpolated
                              at quadrature points, node_assembler.py:389) */
#define TM_COEF_QUAD 3     /* coef[E*Q*H]      (f(x_q) evaluated by caller) */

/*
 * Patch plan: the precomputed, mesh-only structure that replaces the
 * reference's per-entry slot map ``elem_eids`` / ReduceProjector indices
 * (assemble/element_assembler.py:838-875, assemble/projector.py:24-136,
 * assemble/node_assembler.py:665-670).  Nodes are partitioned into patches;
 * a patch owns a set of CSR rows and lists every element touching them.
 * All arrays are device arrays.
 *
 *   vptr[P+1], vtx[]       local vertex table of each patch (global node ids)
 *   eptr[P+1], elem[]      elements touching each patch (global ids)
 *   econn[eptr[P]*B]       element connectivity in patch-local vertex ids
 *   rptr[P+1], rows[]      owned rows of each patch (global node ids)
 *   racc[]                 accumulator offset (in node slots) of each owned row
 *   iptr[n_rows+1]         incidence range of each owned row (rows[] order)
 *   inc_elem[], inc_a[]    incidence: patch-local element index, local vertex
 *   inc_pos[n_inc*B]       position of column conn[e,b] inside row conn[e,a]
 *   indptr[N+1]            node-level CSR row pointer (int64)
 *   inc_pack[n_inc]        P1 tetrahedra: the incidence in one 64-bit record
 *   inc_pack32[n_inc]      the same in 32 bits, when it fits
 *   rdiag[n_rows]          position of each owned row's own column (rows[] order)
 *
 * Records (o_j = (a + 1 + j) mod 4, pos o_j = position of column conn[e, o_j]
 * inside row conn[e, a]):
 *   inc_pack:   local element (bits 0-15) | a (16-17) | pos o_0, o_1, o_2
 *               (8 bits each, from bit 18)
 *   inc_pack32: local element (bits 0-14) | a (15-16) | pos o_0, o_1, o_2
 *               (5 bits each, from bit 17); built when every row has at most
 *               32 entries and every patch at most 32767 elements
 * Elements inside a patch are in processing order (not sorted by id).
 */
typedef struct tm_patch_plan {
  int32_t n_patches;
  int32_t n_elements;
  int32_t n_points;
  int32_t n_basis;
  const int32_t* vptr;
  const int32_t* vtx;
  const int32_t* eptr;
  const int32_t* elem;
  const uint16_t* econn;
  const int32_t* rptr;
  const int32_t* rows;
  const int32_t* racc;
  const int32_t* iptr;
  const uint16_t* inc_elem;
  const uint8_t* inc_a;
  const uint8_t* inc_pos;
  const int64_t* indptr;
  int32_t max_vtx;    /* max local vertices of a patch */
  int32_t max_slots;  /* max node slots owned by a patch */
  int32_t max_rows;   /* max owned rows of a patch */
  int32_t max_elems;  /* max elements touching a patch */
  const uint64_t* inc_pack;   /* P1 tetrahedra (NULL otherwise) */
  const uint32_t* inc_pack32; /* NULL when it does not fit */
  const uint8_t* rdiag;       /* with inc_pack */
  int32_t max_deg;            /* max entries of one CSR row */
  int32_t pad1;
} tm_patch_plan;

typedef struct tm_assemble_args {
  int32_t element;    /* TM_TRI3 ... */
  int32_t form;       /* TM_FORM_* */
  int32_t dtype;      /* TM_F32 / TM_F64: points, coef and output */
  int32_t precision;  /* TM_PREC_* (TM_F64 only) */
  int32_t coef_kind;  /* TM_COEF_* */
  int32_t n_comp;     /* components of a load (H); 1 for bilinear forms */
  int32_t n_quad;     /* quadrature points */
  int32_t pad0;
  const double* tables; /* w[Q], N[Q][B], dN[Q][B][D] (float64, device) */
  const void* points;   /* [N][D] in dtype */
  const void* coef;     /* see coef_kind, dtype */
  double scal[3];       /* scalar coefficient(s) */
  double lam;           /* elasticity: Lame lambda per unit coefficient */
  double mu;            /* elasticity: Lame mu per unit coefficient */
  void* out;            /* CSR values (dof level) or load vector [N*H] */
} tm_assemble_args;

/*
 * Assemble a bilinear form straight into CSR values (canonical row/column
 * order) or a linear form into a node vector.  Deterministic: the same
 * inputs give bitwise-identical outputs on every run.
 * Replaces ElementAssembler.__call__ (assemble/element_assembler.py:243-466)
 * and NodeAssembler.__call__ (assemble/node_assembler.py:242-409) for the
 * built-in forms, including the ReduceProjector scatter
 * (assemble/projector.py:95-130).
 */
int tm_assemble(const tm_patch_plan* plan, const tm_assemble_args* args, void* stream);

/*
 * Backward (adjoint) assembly.  Given dL/d(values) of a tm_assemble call
 * with the same plan and args, writes per-(patch, element) partial gradients:
 *   pair_dX[n_pairs][B][D]          dL/dX of the element's nodes;
 *   pair_dcoef: TM_COEF_ELEMENT [n_pairs], TM_COEF_POINT [n_pairs][B][C],
 *               TM_COEF_QUAD [n_pairs][Q][C] (C = load components or 1).
 * Either output may be NULL.  The partials of one element (or node) are
 * summed in a fixed order with tm_segment_sum.  Replaces the reference's
 * autograd through vmap/einsum/torch.inverse/index_add_
 * (element/element.py:962-966, element/transformation.py:1289,
 * assemble/projector.py:125).  FP64 runs native FP64 arithmetic.
 */
typedef struct tm_backward_args {
  const void* grad_out; /* dL/d(values) [dof nnz] or dL/d(load) [N*H], dtype */
  void* pair_dX;
  void* pair_dcoef;
} tm_backward_args;

int tm_assemble_backward(const tm_patch_plan* plan, const tm_assemble_args* args, const tm_backward_args* bw,
                         void* stream);

/* dst[s][w] = sum_{k = ptr[s]}^{ptr[s+1]-1} src[perm[k]][w], in k order
 * (deterministic segmented reduction). */
int tm_segment_sum(int32_t dtype, int64_t n_segments, const int64_t* ptr, const int64_t* perm, int32_t width,
                   const void* src, void* dst, void* stream);

/*
 * Batched assemble + Jacobi-PCG of many independent meshes in ONE persistent
 * launch (capturable in a CUDA graph).  The union mesh's patch plan must keep
 * each instance's patches contiguous (inst_pbeg) and its rows contiguous
 * (inst_rbeg).  Clusters of `cluster` CTAs pop instances in `order` and, per
 * instance, assemble K (mat, float32) and b (load, float32) into mat->out /
 * load->out, then run Jacobi-PCG on the non-Dirichlet dofs to
 * ||r|| <= rtol ||b||, writing x and per-instance status / iterations /
 * residual.  work: 6 * n_rows floats.  queue: one device uint.
 * Replaces the reference's per-mesh Python loop of assembler calls and
 * solves (no batched path exists in the reference).
 */
typedef struct tm_batched_args {
  int32_t element;     /* TM_TRI3 or TM_TET4 */
  int32_t cluster;     /* CTAs per cluster (1..16) */
  int32_t n_clusters;  /* persistent clusters launched */
  int32_t n_inst;
  int32_t maxiter;
  int32_t chunk;       /* staging chunk of the patch assembly */
  float rtol;
  int32_t pad0;
  int64_t n_rows;      /* rows of the union */
  int64_t smem_bytes;  /* dynamic shared memory per CTA */
  const tm_patch_plan* plan;
  const tm_assemble_args* mat;
  const tm_assemble_args* load;
  const int32_t* order;
  const int32_t* inst_pbeg;
  const int64_t* inst_rbeg;
  const int32_t* indices;   /* node-level CSR column indices of the union */
  const uint8_t* dirichlet; /* [n_rows] */
  float* x;
  void* work;
  int32_t* status;
  int32_t* iters;
  float* resid;
  unsigned int* queue;
  void* stream;
} tm_batched_args;

int tm_batched_assemble_pcg(const tm_batched_args* args, void* stream);
/* clusters of the given size that fit on the device at once (occupancy) */
int tm_batched_max_clusters(int32_t element, int32_t cluster, int64_t smem_bytes);
/* dynamic shared memory of one patch-assembly CTA */
int64_t tm_patch_smem_bytes(int32_t element, int32_t form, int32_t n_comp, int32_t dtype,
                            const tm_patch_plan* plan, int32_t coef_kind, int32_t chunk);

/*
 * Physical coordinates of every quadrature point, out[E][Q][D] =
 * sum_b N_b(xi_q) X[conn[e,b]] -- what the reference feeds to a ``func`` /
 * ``x`` argument (assemble/node_assembler.py:389, element_assembler.py:440).
 */
int tm_quadrature_points(int32_t element, int32_t dtype, int32_t n_quad, const double* tables,
                         const void* points, const int32_t* elements, int64_t n_elements,
                         void* out, void* stream);

/*
 * Two-level preconditioner of the learned solver (no counterpart in the
 * reference, whose K.solve has only Jacobi): z = C r + (I - C K) S (I - K C) r
 * with C = P K_c^-1 P^T (P piecewise constant over nc aggregates) and
 * S = diag(sw).  float32 inside; r and z are FP64 device vectors of length n.
 * work: float32 scratch of 2 n + 4 nc values (16-byte aligned for the fastest
 * coarse matvecs).  Graph-capturable (no host
 * synchronisation, no allocation).
 */
typedef struct tm_twolevel {
  int64_t n;                  /* fine dofs */
  int32_t nc;                 /* aggregates */
  int32_t pad0;
  const int32_t* agg;         /* [n] aggregate of each dof */
  const int64_t* agg_ptr;     /* [nc+1] dof range of each aggregate in agg_perm */
  const int32_t* agg_perm;    /* [n] dofs grouped by aggregate */
  const float* kc_inv;        /* [nc*nc] K_c^-1, row-major */
  const int64_t* kp_indptr;   /* [n+1] K P as CSR with nc columns */
  const int32_t* kp_indices;
  const float* kp_values;
  int64_t k_nnz;              /* K (float32 values) */
  const int64_t* k_indptr;
  const int32_t* k_indices;
  const float* k_values;
  const float* sw;            /* [n] smoother weights w_i / K_ii */
  float* work;
  /* optional SELL-32 copy of K in float32 (tm_sell_fill); NULL k_slice_ptr
   * = the products use the CSR arrays above */
  const int64_t* k_slice_ptr;
  const void* k_scol;
  const float* k_sval;
  int32_t k_narrow;
  int32_t pad1;
  /* optional half-precision copy of K_c^-1 for the coarse matvecs: kc_half
   * [nc*nc] IEEE binary16 H_ij = K_c^-1_ij / (kc_scale_i kc_scale_j) with
   * kc_scale_i = sqrt(K_c^-1_ii) (|H_ij| <= 1, symmetric), kc_scale [nc]
   * float32; NULL kc_half = the float32 kc_inv above */
  const void* kc_half;
  const float* kc_scale;
} tm_twolevel;

int tm_twolevel_apply(const tm_twolevel* t, const double* r, double* z, void* stream);

/*
 * `iters` iterations of flexible CG (Polak-Ribiere beta, clamped at 0) with
 * the two-level preconditioner, on FP64 vectors, with every scalar on the
 * device (graph-capturable, no host synchronisation):
 *   q = A p; alpha = rz / (p, q); x += alpha p; r -= alpha q; z = M r;
 *   beta = max(0, -alpha (z, q) / rz); rz = (r, z); p = z + beta p.
 * A is the FP64 CSR matrix (a_indptr, a_indices, a_values), or, when
 * a_slice_ptr is non-NULL, its tm_sell_fill copy (a_slice_ptr, a_narrow,
 * a_scol, a_sval), M the two-level operator t.  x, r, p are
 * updated in place; q and z are scratch of n doubles; sc[0] holds rz on
 * entry and on exit (sc: 8 doubles: rz, alpha, beta, (p, q), the rz of odd
 * iterations, scratch); part is
 * scratch of tm_fcg_workspace_doubles() doubles.  Dot products reduce in a
 * fixed order (bitwise repeatable).  A non-positive (p, q) sets alpha = 0.
 */
int64_t tm_fcg_workspace_doubles(void);
/* K P of the two-level coarse space (P piecewise constant over aggregates
 * agg[n]): tm_kp_count writes count[i], the aggregates among the columns of
 * row i; kp_indptr is its exclusive scan; tm_kp_fill writes row i as
 * (aggregate, sum of K_ij over its columns j in CSR order) in ascending
 * aggregate order.  FP64 values. */
int tm_kp_count(int64_t n, const int64_t* indptr, const int32_t* indices, const int32_t* agg, int64_t* count,
                void* stream);
int tm_kp_fill(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values, const int32_t* agg,
               const int64_t* kp_indptr, int32_t* kp_indices, double* kp_values, void* stream);
int tm_fcg_twolevel_iterations(const tm_twolevel* t, int64_t a_nnz, const int64_t* a_indptr, const int32_t* a_indices,
                               const double* a_values, const int64_t* a_slice_ptr, int32_t a_narrow,
                               const void* a_scol, const double* a_sval, double* x, double* r, double* p, double* q,
                               double* z, double* sc, double* part, int32_t iters, void* stream);

/*
 * Neo-Hookean energy per element and its displacement gradient per (element,
 * local node) (replaces NeoHookeanModel.energy, assemble/builtin.py:220-334,
 * the quadrature loop of ElementAssembler.energy, element_assembler.py:
 * 468-680, and the autograd of both).  tables: the flat [w(Q), N(Q*B),
 * dN(Q*B*D)] float64 table; points and u are [N][D] in dtype; energy_el
 * [n_elements] float64; grad_el [n_elements][B][D] in dtype, or NULL for the
 * energy alone.  mu, lam: Lame constants.  FP64 arithmetic in the kernel.
 */
int tm_neohookean(int32_t element, int32_t dtype, int32_t n_quad, const double* tables, const void* points,
                  const int32_t* elements, int64_t n_elements, const void* u, double mu, double lam,
                  double* energy_el, void* grad_el, void* stream);

/*
 * Facet (boundary) load contributions (replaces FacetAssembler.__call__,
 * assemble/facet_assembler.py:130-235, for integrands g * v).  Per selected
 * facet s (sel[s] = element * F + local facet f; F = 3 for triangles, 4 for
 * tetrahedra; facet f is the one opposite vertex f) and cell node b:
 *   out[s][b][h] = sum_q w[f][q] |F_q| g_h(q) N[f][q][b],
 * |F_q| = |t_0| (edges) or |t_0 x t_1| (faces), t_k = sum_b Tc[f][q][k][b] X_b.
 * tables (float64): w [F][Qf], N [F][Qf][B], Tc [F][Qf][D-1][B].
 * coef_kind: TM_COEF_SCALAR (scal: HOST array of n_comp values),
 * TM_COEF_POINT (coef [N][n_comp] in dtype, interpolated with N),
 * TM_COEF_QUAD (coef [n_sel][Qf][n_comp] in dtype).  n_comp <= 3.
 * With x_out non-NULL the call writes only the physical facet quadrature
 * points x_out [n_sel][Qf][D] (dtype), for callers that evaluate g(x).
 * out [n_sel][B][n_comp] in dtype; FP64 arithmetic.  The caller reduces out
 * to the nodes (tm_segment_sum in a fixed order).
 */
int tm_facet_load(int32_t element, int32_t dtype, int32_t n_quad, const double* tables, const void* points,
                  const int32_t* elements, const int64_t* sel, int64_t n_sel, int32_t coef_kind, const void* coef,
                  const double* scal, int32_t n_comp, void* out, void* x_out, void* stream);

/* y = A x for CSR A (replaces SparseMatrix @ / spmv, sparse/mm/__init__.py:
 * 22-72).  dtype applies to values, x and y; nnz = indptr[n_rows] (it sets
 * the lanes per row; the row extents come from indptr). */
int tm_spmv_csr(int32_t dtype, int64_t n_rows, int64_t nnz, const int64_t* indptr, const int32_t* indices,
                const void* values, const void* x, void* y, void* stream);

/*
 * Jacobi-preconditioned CG, whole iteration in one cooperative launch.
 * Replaces K.solve for SPD systems (torch_sla SparseTensor.solve; in-repo
 * equivalents sparse/solve/torch_solve.py:24-59 Jacobi, 70-128 cg_py,
 * 130-248 bicgstab_py).  Stops when ||r|| <= max(rtol*||b||, atol) on the
 * recurrence residual or after maxiter iterations.  x holds the initial guess
 * on entry.  work: caller-owned device scratch of at least
 * tm_pcg_workspace_bytes(dtype, n, nnz, tm_pcg_max_blocks(dtype)) bytes
 * (-TM_ERR_INVALID for a negative size or an unknown dtype).
 * FP64 systems are iterated in double-float arithmetic on the FP32 pipe
 * (values and vectors held as float pairs in the workspace).
 * Statuses of the solve itself are read back with tm_pcg_result.
 */
int64_t tm_pcg_workspace_bytes(int32_t dtype, int64_t n, int64_t nnz, int32_t max_blocks);
int tm_pcg_max_blocks(int32_t dtype);
int tm_pcg_jacobi(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                  const void* values, const void* b, void* x, double rtol, double atol, int32_t maxiter,
                  void* work, int64_t work_bytes, void* stream);
/* Synchronises the stream; returns the solve status (TM_OK, TM_ERR_MAXITER,
 * TM_ERR_BREAKDOWN, TM_ERR_TIMEOUT) and its iteration count / residuals. */
int tm_pcg_result(const void* work, int32_t* iters, double* res, double* bnorm, void* stream);

/*
 * The same Jacobi-PCG over a SELL-32 copy of the matrix (coalesced row
 * slices, the preconditioner folded into the stored values).  method
 * TM_PCG_STANDARD: the recurrence of tm_pcg_jacobi, two grid barriers per
 * iteration; TM_PCG_PIPELINED: pipelined CG (Ghysels & Vanroose 2014), one
 * barrier per iteration, whose recurrences lose accuracy faster (it can stop
 * with TM_ERR_BREAKDOWN where the standard form converges).  Same stopping
 * rule, statuses and meaning of x as tm_pcg_jacobi; the result is read back
 * with tm_pcg_result on `work`.
 *
 * tm_sell_plan: slice pointers of the SELL-32 layout of an n-row CSR pattern,
 * slice_ptr [ceil(n / 32) + 1] (device, int64): slice s holds rows
 * 32 s .. 32 s + 31, padded to its longest row, entry j of row 32 s + l at
 * slice_ptr[s] + 32 j + l.  Returns the padded entry count
 * slice_ptr[ceil(n / 32)] (synchronises the stream), or -TM_ERR_* on error.
 * out_narrow (host, may be NULL) is set to 1 when every |column - row| <= 32767:
 * the solve may then pass TM_PCG_NARROW and store 16-bit column offsets.
 * The plan depends on the pattern only: compute it once per pattern.
 *
 * tm_pcg_jacobi_sell: work is caller-owned device scratch of at least
 * tm_pcg_sell_workspace_bytes(dtype, n, n_pad) bytes (the SELL copy of the
 * values, the preconditioned vectors, per-CTA partial sums).  A slice_ptr
 * that does not cover every row, or a column index outside [0, n), returns
 * TM_ERR_INDEX through tm_pcg_result (nothing is iterated).  Asynchronous
 * on `stream`.
 */
int64_t tm_sell_plan(int64_t n, const int64_t* indptr, const int32_t* indices, int64_t* slice_ptr,
                     int32_t* out_narrow, void* stream);
int64_t tm_pcg_sell_workspace_bytes(int32_t dtype, int64_t n, int64_t n_pad);
#define TM_PCG_STANDARD 0   /* Hestenes-Stiefel PCG, two grid barriers per iteration */
#define TM_PCG_PIPELINED 1  /* Ghysels-Vanroose pipelined PCG, one barrier; less stable */
#define TM_PCG_NARROW 2     /* or-ed in: 16-bit column offsets (the plan's out_narrow must be 1;
                               an offset that does not fit returns TM_ERR_INDEX) */
/* A plain SELL-32 copy of a CSR matrix on a tm_sell_plan slice plan (values
 * as given: FP64 in double, FP32 in float; scol int16 offsets from the row
 * when narrow, else int32 columns), and y = A x on it.  *bad_flag (device
 * int32) is set to 1 when the plan does not cover a row, a column lies
 * outside [0, n) or an offset does not fit 16 bits. */
int tm_sell_fill(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices, const void* values,
                 const int64_t* slice_ptr, int64_t n_pad, int32_t narrow, void* scol, void* sval, int32_t* bad_flag,
                 void* stream);
int tm_spmv_sell(int32_t dtype, int64_t n, const int64_t* slice_ptr, int32_t narrow, const void* scol,
                 const void* sval, const void* x, void* y, void* stream);
int tm_pcg_jacobi_sell(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices, const void* values,
                       const int64_t* slice_ptr, int64_t n_pad, const void* b, void* x, double rtol, double atol,
                       int32_t maxiter, int32_t method, void* work, int64_t work_bytes, void* stream);

/*
 * Allocation-free float32 Jacobi-PCG.  This entry point has no counterpart in
 * the reference.  It exists for callers that cannot allocate device memory
 * when they solve -- hosts that plan all device buffers up front, plugins
 * whose host framework owns the only allocator, solves issued while a memory
 * pool is exhausted.  It runs the same solver as tm_pcg_jacobi but keeps its
 * scratch in a 32 MiB array inside this library (reserved on every GPU that
 * loads it, until exit), so the caller passes only A, b and x.
 * Limits and rules: n <= 1,000,000 rows, else TM_ERR_INDEX; calls share the
 * array, so calls that overlap on the GPU race and must be serialised; every
 * call looks up the array's address on the current device (no allocation);
 * the call synchronises `stream` to read the result, so it cannot run on a
 * stream that is being captured (TM_ERR_INVALID, nothing launched); it
 * returns the solve status (as tm_pcg_result) with the iteration count and
 * recurrence residual, which are set to 0 before any early return.
 */
int tm_pcg_jacobi_noalloc(int64_t n, const int64_t* indptr, const int32_t* indices, const float* values,
                          const float* b, float* x, double rtol, double atol, int32_t maxiter, int32_t* out_iters,
                          double* out_res, void* stream);

/*
 * CSR pattern of a mesh on the GPU (replaces the reference's from_mesh pattern
 * build, assemble/element_assembler.py:838-866, and its per-entry slot map
 * `elem_eids`).  elements: [n_elements][n_basis] int32 node ids in
 * [0, n_points) (device).  Two calls:
 *   tm_pattern_count writes indptr [n_points + 1] (int64): the row offsets of
 *     the unique (row, col) pairs of every element's node pairs;
 *   tm_pattern_fill (after the caller has read nnz = indptr[n_points] and
 *     allocated) writes indices [nnz] (int32, ascending inside each row) and,
 *     when out_slots is not NULL, slots [n_elements][n_basis][n_basis]
 *     (int64): the CSR position of entry (row = el[e][a], col = el[e][b]).
 * `work` (device, tm_pattern_workspace_bytes) carries the node -> element
 * incidence from the first call to the second.  Deterministic; no host
 * synchronisation inside.
 */
int64_t tm_pattern_workspace_bytes(int64_t n_elements, int32_t n_basis, int64_t n_points);
int tm_pattern_count(const int32_t* elements, int64_t n_elements, int32_t n_basis, int64_t n_points, void* work,
                     int64_t* out_indptr, void* stream);
int tm_pattern_fill(const int32_t* elements, int64_t n_elements, int32_t n_basis, int64_t n_points, const void* work,
                    const int64_t* indptr, int32_t* out_indices, int64_t* out_slots, void* stream);

/*
 * Morton (Z-order) keys of n points in dim <= 3 dimensions (coords [n][dim]
 * float64, lo / hi [dim] the bounding box, on the device): coordinate d is
 * quantised to q = rint((x - lo_d) / max(hi_d - lo_d, 1e-300) * (2^bits - 1))
 * and bit b of q is bit b * dim + d of keys[i] (bits * dim <= 63).  Used by
 * the octree partition of the two-level coarse space (no counterpart in the
 * reference).
 */
int tm_morton_keys(int64_t n, int32_t dim, const double* coords, const double* lo, const double* hi, int32_t bits,
                   int64_t* keys, void* stream);

/*
 * Self-test of the bounded grid barrier the PCG kernels use (no counterpart
 * in the reference: the reference has no device-side waits).  Launches
 * n_blocks cooperative CTAs of which one never arrives at the barrier; the
 * others give up after `spins` polls 32 ns apart (at most the PCG kernels'
 * ~1 s limit) and record TM_ERR_TIMEOUT, which is returned in *out_status.
 * `work` is device memory of at least 64 bytes.  Synchronises `stream`.
 * Returns TM_OK when the test ran.
 */
int tm_selftest_barrier_timeout(int32_t n_blocks, int64_t spins, int32_t* out_status, void* work, void* stream);

/* 1/diag(A) with missing diagonals taken as 1 (torch_solve.py:24-59). */
int tm_csr_diagonal_inverse(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                            const void* values, void* out, void* stream);

/* dst[i] = src[map[i]] and dst[map[i]] = src[i]: the value compaction and
 * recovery of static condensation (operator/condense.py:294-299, 429-458). */
int tm_gather(int32_t dtype, int64_t n, const int64_t* map, const void* src, void* dst, void* stream);
int tm_scatter(int32_t dtype, int64_t n, const int64_t* map, const void* src, void* dst, void* stream);

/* f_i = rhs[inner_dof] - K_io u_o (operator/condense.py:300-309, 388-427). */
int tm_condense_rhs(int32_t dtype, int64_t n_inner, const int64_t* inner_dof, const void* rhs,
                    const int64_t* io_indptr, const int32_t* io_indices, const void* io_values,
                    const void* u_outer, void* out, void* stream);

/*
 * Message-passing network of the learned preconditioner (hidden width 64,
 * BF16 features/weights on the tensor cores via mma.sync, FP32 accumulate).
 * Graph = CSR pattern of the condensed matrix with normalised off-diagonal
 * weights aoff (float32, 0 on the diagonal).  Features are row-major [n][64]
 * bf16.  No reference counterpart exists: the reference has no learned
 * preconditioner; these kernels serve the flexible-PCG path that replaces
 * K.solve (torch_sla) for the 128^3 configuration.
 *   input_fwd : H0 = relu(x w[0] + (A x) w[1] + w[2]), y = A x
 *   layer_fwd : Hout = act([Hin | A Hin] Wt^T + b), Wt = [64 out][128 in]
 *   readout   : out = scale * (H wr[0:64] + A (H wr[64:128]))
 * Backward kernels return dH and fixed-order reduced weight gradients.
 */
int tm_mpnn_input_fwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                      const float* x, const float* w, void* H0, float* y, void* stream);
int tm_mpnn_layer_fwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                      const void* Hin, const void* Wt, const float* bias, void* Hout, int32_t relu, void* stream);
int tm_mpnn_readout_fwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff, const void* H,
                        const float* wr, const float* scale, float* u, float* t, float* out, void* stream);
int tm_mpnn_readout_bwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff, const void* H,
                        const float* g, const float* wr, float* dH, float* part, float* dwr, void* stream);
int tm_mpnn_layer_bwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                      const void* Hin, const void* Hout, const float* dHout, const void* W, int32_t relu,
                      float* part_dW, float* part_db, float* U, float* T, float* dHin, float* dW, float* db,
                      void* stream);
int tm_mpnn_input_bwd(int64_t n, const float* x, const float* y, const void* H0, const float* dH0, float* part,
                      float* dw, void* stream);
/* out = scale * (u + A t) over a float32 CSR (u, scale may be NULL) */
int tm_gather_axpy_f32(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                       const float* u, const float* t, const float* scale, float* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
