/*
 * gbfem.h — C ABI of libgbfem, the GB300 (sm_103a) implementation of femx's
 * data-parallel assembly path.
 *
 * Conventions (femx v0.4.0 semantics, femx/common/Types.hpp:17-19):
 *   - Real = double, Index = int32. Array arguments are DEVICE pointers unless
 *     stated otherwise; sizes are element counts.
 *   - Every call returns GBFEM_OK (0) or an error code; the message of the
 *     last failure on the calling thread is gbfem_last_error(). The messages
 *     are the ones femx's require() throws (femx/common/Checks.hpp:11-17).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream). Hot-path calls
 *     (assemble, boundary operations, SpMV, VJP) only enqueue work: they do not
 *     synchronize, allocate or read back, so they can be captured in CUDA
 *     graphs. Map creation is setup: it allocates and synchronizes `stream`.
 *   - Handles own their device buffers; the caller owns the stream and every
 *     array it passes in.
 */
#ifndef GBFEM_H
#define GBFEM_H

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBFEM_API __attribute__((visibility("default")))
#else
#define GBFEM_API
#endif

#define GBFEM_OK 0
#define GBFEM_EINVAL 1 /* invalid argument: sizes, aliasing, layout (require) */
#define GBFEM_ECUDA 2  /* CUDA runtime failure */
#define GBFEM_EDATA 3  /* invalid mesh / DOF data found on the device */
#define GBFEM_ENOMEM 4 /* device allocation failed */

/* Arithmetic of the element kernels. FP64: plain double everywhere (the
 * drop-in). FP32_QUAD: element quadrature in float (Jacobian and residual
 * contributions); accumulation, scatter and all global vectors in double.
 * MIXED: the Newton scheme — Jacobian from FP32 quadrature, residual to
 * FP64 accuracy (Taylor-Hood: double-float arithmetic on the FP32 pipe,
 * about 1e-14 from the FP64 residual; P1: FP64); accumulation in double.
 * Residual-only calls in MIXED use the FP64 kernels. */
#define GBFEM_PREC_FP64 0
#define GBFEM_PREC_FP32_QUAD 1
#define GBFEM_PREC_MIXED 2
/* DOUBLE_FLOAT (Taylor-Hood and P1 assembly, Taylor-Hood state VJP): the
 * element arithmetic of the Jacobian and residual in double-float (each
 * value a pair of floats, about 48 significant bits) on the FP32 pipe, which
 * GB300 issues about 64x faster than FP64; accumulation, scatter and vectors
 * in FP64. Results within about 1e-14 (relative to the largest entry) of
 * the FP64 path: the FP64-accurate fast path. Deterministic Taylor-Hood
 * calls use FP64 records; the P1 VJP runs FP64. */
#define GBFEM_PREC_DOUBLE_FLOAT 3
/* OR-ed into a Taylor-Hood precision argument: deterministic assembly —
 * element rows are written as records and each CSR row sums its records in
 * element order (no atomics, no zero-fill), so repeated calls agree bit for
 * bit, like femx's serial CPU loop. Needs gbfem_assembly_map_enable_gather
 * on the map first. */
#define GBFEM_DETERMINISTIC 0x100
/* OR-ed into a precision argument (P1, Taylor-Hood, their VJPs, the batch):
 * coloured assembly — elements run colour by colour with plain
 * read-add-writes, no atomics (gbfem_assembly_map_enable_colouring first);
 * bitwise reproducible like GBFEM_DETERMINISTIC, for any layout. */
#define GBFEM_COLOURED 0x200
/* OR-ed into a P1 assembly precision argument (FP64, FP32_QUAD or
 * DOUBLE_FLOAT): owner-computes tiled assembly (gbfem_assembly_map_enable_tiles
 * first). Every residual row belongs to one tile of nearby rows; a block per
 * tile evaluates the tile's elements into shared memory, then writes each of
 * its rows once: no atomics, no zero fill, bitwise reproducible. With
 * DOUBLE_FLOAT it is the FP64-accurate fast assembly: the element
 * arithmetic and every conversion run on the FP32 and integer pipes, FP64
 * instructions only form the coordinate differences. */
#define GBFEM_TILED 0x400 /* also for gbfem_vjp_p1_kappa (FP64 or DOUBLE_FLOAT): g_u
                           * summed row by row, g_m written by each element's
                           * owner tile, no atomics, no zero fill */

GBFEM_API const char* gbfem_last_error(void);
GBFEM_API int         gbfem_version(void);

/* ---------------------------------------------------------------------------
 * AssemblyMap — replaces femx::assembly::makeAssemblyMap(num_res, num_states,
 * res_dofs, state_dofs) (femx/assembly/AssemblyMap.hpp:230-234,
 * AssemblyMap.cpp:54-176) and copy(Host -> Device) (AssemblyMap.cpp:201-235).
 * The CSR pattern (union of every element block, rows sorted by column,
 * duplicates merged) and jac_map (row-major local entry -> CSR slot) are built
 * on the GPU and are bit-identical to the reference's. Inputs are the element
 * DOF tables in femx's flattened form (AssemblyMapView, AssemblyMap.hpp:21-68).
 * ------------------------------------------------------------------------ */
typedef struct gbfem_assembly_map gbfem_assembly_map;

typedef struct
{
  int                num_elems, num_res, num_states;
  int                nnz, jac_nnz, max_res, max_state, max_jac;
  unsigned long long layout_id; /* femx CsrPattern::layoutId analogue */
  const int *        res_offsets, *res_dofs, *state_offsets, *state_dofs;
  const int *        jac_offsets, *jac_map, *row_ptr, *col_ind;
} gbfem_assembly_map_view;

GBFEM_API int  gbfem_assembly_map_create(int num_res, int num_states, int num_elems,
                               const int* res_offsets, const int* res_dofs,
                               const int* state_offsets, const int* state_dofs,
                               void* stream, gbfem_assembly_map** out);
GBFEM_API int  gbfem_assembly_map_get_view(const gbfem_assembly_map* map,
                                 gbfem_assembly_map_view* view);
GBFEM_API void gbfem_assembly_map_destroy(gbfem_assembly_map* map);
/* Reads and clears the map's device status word, set by a hot-path kernel
 * that met invalid data (a degenerate element: femx throws "Singular 2D
 * Jacobian." from ElementValues::invJacobian, ElementValues.cpp:210-229).
 * Synchronizes `stream`; returns GBFEM_EDATA with the message if set. */
GBFEM_API int  gbfem_assembly_map_check(const gbfem_assembly_map* map, void* stream);
/* Builds the row-gather tables behind GBFEM_DETERMINISTIC assembly (setup:
 * allocates and synchronizes `stream`; later calls return at once). A record
 * per element row, numbered row by row in ascending element order; about
 * 150 bytes of device memory per element row. Needs a uniform layout with
 * 6..16 DOFs per element and rows up to 256 entries (Taylor-Hood: yes);
 * otherwise GBFEM_EINVAL. Not to be called concurrently with other work on
 * the same map. No counterpart in the reference, whose CPU loop is serial
 * and deterministic by construction (Assembly.hpp:186-223). */
GBFEM_API int  gbfem_assembly_map_enable_gather(gbfem_assembly_map* map, void* stream);
/* Colours the map's elements so that no two elements of one colour share a
 * residual or state DOF (greedy, elements in ascending order, at most 64
 * colours; setup: reads the DOF tables back, allocates, synchronizes
 * `stream`; later calls return at once). With GBFEM_COLOURED the element
 * kernels then run colour by colour and add with plain read-add-writes
 * instead of FP64 atomics: a fixed summation order, bitwise reproducible
 * results, for any element layout. No counterpart in the reference, whose
 * OpenMP NS assembly uses atomics (NavierStokesModel.cpp:227-318) and whose
 * CUDA assembly FP64 atomics (CudaAssembly.hpp:160-168).
 * gbfem_assembly_map_num_colours: 0 before colouring. */
GBFEM_API int  gbfem_assembly_map_enable_colouring(gbfem_assembly_map* map, void* stream);
GBFEM_API int  gbfem_assembly_map_num_colours(const gbfem_assembly_map* map);
/* Builds the owner-computes tiles behind GBFEM_TILED for a P1 layout (three
 * identical residual and state DOFs per element; setup: reads the DOF table,
 * `conn`, `coords` and the pattern back, builds on the host, allocates and
 * synchronizes `stream`; later calls return at once). Rows are ordered along
 * a Morton curve of their vertex coordinates (coords: num_nodes x 2,
 * node-major; conn: the geometry connectivity, num_elems x 3, or null when
 * geometry nodes are the DOFs, and then null in every tiled assembly call
 * too); tiles are runs of at most 256 rows, 1024 elements and 1024
 * vertices. About 4 bytes per CSR slot plus 20 bytes per element of device
 * memory. GBFEM_EINVAL for other layouts, for an element with a repeated
 * DOF, a DOF on two geometry nodes, or an edge shared by more than two
 * elements (a non-conforming mesh). No counterpart in the reference, whose
 * assembly scatter-adds (Assembly.hpp:186-223, CudaAssembly.hpp:160-168).
 * gbfem_assembly_map_num_tiles: 0 before tiling. */
GBFEM_API int  gbfem_assembly_map_enable_tiles(gbfem_assembly_map* map, int num_nodes,
                                               const double* coords, const int* conn,
                                               void* stream);
GBFEM_API int  gbfem_assembly_map_num_tiles(const gbfem_assembly_map* map);

/* ---------------------------------------------------------------------------
 * BoundaryMap — replaces femx::assembly::makeBoundaryMap(dofs, pattern)
 * (femx/assembly/BoundaryMap.hpp:183-184, BoundaryMap.cpp:59-139) plus
 * copy(Host -> Device) (:141-170). Built on the GPU; bc_rows, diag,
 * col_offsets, col_entries, col_rows and bc_mask are bit-identical to the
 * reference's. `dofs` keeps its input order (it defines bc_vals order).
 * ------------------------------------------------------------------------ */
typedef struct gbfem_boundary_map gbfem_boundary_map;

typedef struct
{
  int                num_rows, num_cols, nnz, num_bcs, num_col_entries;
  unsigned long long layout_id;
  const int *        bc_rows, *diag, *col_offsets, *col_entries, *col_rows;
  const int*         bc_mask;
} gbfem_boundary_map_view;

GBFEM_API int  gbfem_boundary_map_create(int num_bcs, const int* dofs, int rows, int cols,
                               const int* row_ptr, const int* col_ind,
                               unsigned long long layout_id, void* stream,
                               gbfem_boundary_map** out);
GBFEM_API int  gbfem_boundary_map_get_view(const gbfem_boundary_map* bc,
                                 gbfem_boundary_map_view* view);
GBFEM_API void gbfem_boundary_map_destroy(gbfem_boundary_map* bc);

/* replaceRows(map, jac, diag, ctx): BoundaryMap.hpp:215-226,
 * BoundaryMap.cu:122-141 (replaceRowsKernel). Zero constrained rows, set the
 * diagonal to `diag`; columns untouched. */
GBFEM_API int gbfem_replace_rows(const gbfem_boundary_map* bc, double* vals, double diag,
                       void* stream);
/* replaceRes(map, state, bc_vals, res, ctx): BoundaryMap.hpp:246-250,
 * BoundaryMap.cu:69-80,155-173. res[bc_row] = state[bc_row] - bc_vals[ib]. */
GBFEM_API int gbfem_replace_res(const gbfem_boundary_map* bc, const double* state,
                      const double* bc_vals, double* res, void* stream);
/* zeroBoundary(map, vals, ctx): BoundaryMap.hpp:255-258, BoundaryMap.cu:82-94. */
GBFEM_API int gbfem_zero_boundary(const gbfem_boundary_map* bc, double* v, void* stream);
/* prepareForwardSolve(map, solve_mat, rhs, bc_vals, ctx): BoundaryMap.hpp:
 * 287-291, BoundaryMap.cpp:218-247, BoundaryMap.cu:192-211. Lifting
 * rhs[r] -= A[r][c] g_c on unconstrained rows, constrained columns zeroed,
 * constrained rows -> identity, rhs[bc] = g. Subtractions are applied in
 * constraint order, so rhs matches the CPU reference bit for bit. */
GBFEM_API int gbfem_prepare_forward_solve(const gbfem_boundary_map* bc, double* vals,
                                double* rhs, const double* bc_vals,
                                void* stream);

/* Same result as gbfem_boundary_map_create + gbfem_prepare_forward_solve,
 * for callers that cannot call cudaMalloc (e.g. code running while another
 * allocator owns the device memory, such as a PyTorch process whose caching
 * allocator has reserved it, or a real-time solver loop that must not pay for
 * allocation). It has no counterpart in the reference. It allocates nothing:
 * its scratch is a fixed library-owned device array of 8 MiB + 256 B, held by
 * every GPU that loads the library until the process exits, so `rows` may be
 * at most GBFEM_NOALLOC_MAX_ROWS; larger calls are rejected with
 * GBFEM_EINVAL. The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress), which also makes CUDA load the part of
 * the library that holds the array if it is not loaded yet (with CUDA's lazy
 * module loading, the array's device memory is committed at that moment),
 * so make the first call before any stream capture and before any section
 * that must not see device memory change. It
 * synchronizes `stream` to report invalid input (out-of-range or repeated
 * DOFs, a missing diagonal, a malformed pattern) before touching vals/rhs.
 * The pattern is square (rows x rows), as femx's makeBoundaryMap requires
 * (BoundaryMap.cpp:62); a row that repeats a constrained column has every
 * such entry lifted and zeroed, as in femx. All calls share the array and
 * leave it cleared (a call that fails midway has the next call clear it
 * whole); calls whose GPU work overlaps (unordered streams) race on it. The
 * looked-up address does not survive cudaDeviceReset: do not call this entry
 * point after a device reset in the same process. */
#define GBFEM_NOALLOC_MAX_ROWS 2097152
GBFEM_API int gbfem_prepare_forward_solve_noalloc(int num_bcs, const int* dofs,
                                                  int rows, const int* row_ptr,
                                                  const int* col_ind, double* vals,
                                                  double* rhs, const double* bc_vals,
                                                  void* stream);

/* ---------------------------------------------------------------------------
 * CSR SpMV — replaces MatrixHandler<CudaCsrBackend>::matvec / matvecT
 * (femx/linalg/handler/MatrixHandler.hpp:270-317, MatrixHandler.cu:335-398,
 * 514-542; host semantics MatrixHandler.cpp:157-198):
 *   y = alpha A x + beta y,   y = alpha A^T x + beta y.
 * ------------------------------------------------------------------------ */
GBFEM_API int gbfem_spmv(int rows, int cols, const int* row_ptr, const int* col_ind,
               const double* vals, const double* x, double* y, double alpha,
               double beta, void* stream);
GBFEM_API int gbfem_spmv_t(int rows, int cols, const int* row_ptr, const int* col_ind,
                 const double* vals, const double* x, double* y, double alpha,
                 double beta, void* stream);

/* ---------------------------------------------------------------------------
 * Mesh ingestion — replaces femx::fem::GmshReader::read (GmshReader.cpp:
 * 446-548; ASCII Gmsh 2.x/4.x) with flat arrays for the device path:
 * coordinates [num_nodes][3] (nodes in file order), connectivity of the
 * elements of the mesh dimension [num_elems][nodes_per_elem] and of the
 * boundary facets one dimension lower, each with its entity tag and its
 * physical tag (from the element, else the first of its entity's). femx's
 * errors and messages; a mesh mixing element shapes is rejected (the
 * kernels take one node count per element). Host memory owned by the
 * handle.
 * ------------------------------------------------------------------------ */
typedef struct gbfem_mesh gbfem_mesh;

typedef struct
{
  int           dim, num_nodes, num_elems, nodes_per_elem, num_facets, nodes_per_facet;
  const double* coords;
  const int *   conn, *elem_etag, *elem_ptag;
  const int *   facet_conn, *facet_etag, *facet_ptag;
} gbfem_mesh_view;

GBFEM_API int  gbfem_mesh_read_gmsh(const char* path, gbfem_mesh** out);
GBFEM_API int  gbfem_mesh_get_view(const gbfem_mesh* mesh, gbfem_mesh_view* view);
/* The physical name of (dim, tag), "" when the file names none. */
GBFEM_API int  gbfem_mesh_physical_name(const gbfem_mesh* mesh, int dim, int tag, char* buf,
                                        int buf_len);
GBFEM_API void gbfem_mesh_destroy(gbfem_mesh* mesh);

/* ---------------------------------------------------------------------------
 * Explicit CSR transpose — replaces MatrixHandler::transpose(src, dst)
 * (femx/linalg/handler/MatrixHandler.cpp:140-155, MatrixHandler.cu:401-512).
 * _create builds, once per source layout, the transposed pattern (rows =
 * source cols; column indices ascending, as femx's transposeCsr) and the
 * value permutation (setup: allocates, synchronizes `stream`). _apply moves
 * the values only: t_vals[p] = vals[src_slot[p]] (in-place is rejected, as
 * in femx). The handle owns the transposed pattern.
 * ------------------------------------------------------------------------ */
typedef struct gbfem_csr_transpose gbfem_csr_transpose;

typedef struct
{
  int        rows, cols, nnz;   /* of the transpose */
  const int *row_ptr, *col_ind; /* transposed pattern */
  const int* src_slot;          /* source slot of every transposed slot */
} gbfem_csr_transpose_view;

GBFEM_API int  gbfem_csr_transpose_create(int rows, int cols, const int* row_ptr,
                                          const int* col_ind, void* stream,
                                          gbfem_csr_transpose** out);
GBFEM_API int  gbfem_csr_transpose_get_view(const gbfem_csr_transpose* t,
                                            gbfem_csr_transpose_view* view);
GBFEM_API int  gbfem_csr_transpose_apply(const gbfem_csr_transpose* t, const double* vals,
                                         double* t_vals, void* stream);
GBFEM_API void gbfem_csr_transpose_destroy(gbfem_csr_transpose* t);

/* y = a x + b y — VectorHandler<Cuda>::axpby (femx/linalg/handler/
 * VectorHandler.cu:124-136), used by the state solvers for rhs = -res
 * (femx/state/StateSolver.hpp:90-108). y is not read when b == 0. */
GBFEM_API int gbfem_axpby(int n, double a, const double* x, double b, double* y,
                void* stream);
/* y = exp(x) elementwise: the control map kappa = exp(m) of the per-element
 * control of the kappa-Poisson residual (femx's Residual::res and
 * applyParamJacT take the parameter vector m itself, Residual.hpp:42-59).
 * x and y may alias. */
GBFEM_API int gbfem_exp(int n, const double* x, double* y, void* stream);

/* ---------------------------------------------------------------------------
 * kappa-weighted P1 Poisson assembly — replaces assembly::assemble(op, geom,
 * map, state, res, jac, ctx) (femx/assembly/CudaAssembly.hpp:319-364, CPU
 * contract Assembly.hpp:153-226) for the element operator
 *   K_e = kappa_e int grad N_i . grad N_j,  res_e = K_e u_e - int f_h N_i,
 * f_h the P1 interpolant of nodal values f_nodal (NULL = no load).
 * coords: node-major [num_nodes][2]; conn: [num_elems][3] geometry
 * connectivity, or NULL when it equals the map's DOF table (scalar P1 space,
 * FESpace.cpp:27-54). res [num_res] and vals [nnz] are overwritten; vals may
 * be NULL (residual only, like assembleResidual, CudaAssembly.hpp:420-472).
 * ------------------------------------------------------------------------ */
GBFEM_API int gbfem_assemble_p1_kappa(const gbfem_assembly_map* map, int num_nodes,
                            const double* coords, const int* conn,
                            const double* kappa, const double* f_nodal,
                            const double* u, double* res, double* vals,
                            int precision, void* stream);

/* Residual VJPs of the same operator, the transpose actions behind
 * Residual::applyParamJacT and the state adjoint (femx/state/Residual.hpp:
 * 55-59, femx/inverse/ReducedFunctional.hpp:94-117), without forming the
 * Jacobian: g_u = sum_e K_e^T lam_e, g_m[e] = kappa_e lam_e^T Khat_e u_e
 * (kappa = exp(m)). Element quadrature is recomputed. g_u [num_states] and
 * g_m [num_elems] are overwritten; either may be NULL. */
GBFEM_API int gbfem_vjp_p1_kappa(const gbfem_assembly_map* map, int num_nodes,
                       const double* coords, const int* conn,
                       const double* kappa, const double* u, const double* lam,
                       double* g_u, double* g_m, int precision, void* stream);

/* ---------------------------------------------------------------------------
 * Taylor-Hood P2/P1 steady Navier-Stokes Newton residual + Jacobian through
 * the same assemble contract (CudaAssembly.hpp:319-364). The map's element
 * DOF tables follow MixedFESpace (velocity 2*node+comp, then pressure), 15 per
 * element; conn6 [num_elems][6] = [v0 v1 v2 m01 m12 m20] in P2-node ids;
 * coords [num_p2_nodes][2]. vals may be NULL (residual only).
 * ------------------------------------------------------------------------ */
GBFEM_API int gbfem_assemble_th_ns(const gbfem_assembly_map* map, int num_p2_nodes,
                         const double* coords, const int* conn6, double nu,
                         const double* state, double* res, double* vals,
                         int precision, void* stream);
/* One Newton system per call for a host-resident state (femx's Newton
 * iteration, femx/solver/Newton.hpp, with host vectors): uploads state_host
 * into `state` (device, num_states), assembles res and vals as
 * gbfem_assemble_th_ns does, applies replaceRes (bc_vals) and, when vals is
 * not NULL, replaceRows (diag), and downloads the final residual into
 * res_host (num_res). The upload overlaps the zero fill and the download
 * overlaps replaceRows, on a side stream owned by the calling host thread
 * (created on its first call); all of it is ordered on `stream`. Host
 * buffers should be page-locked for the copies to be asynchronous. */
GBFEM_API int gbfem_newton_system_th_ns_host(
    const gbfem_assembly_map* map, const gbfem_boundary_map* bc, int num_p2_nodes,
    const double* coords, const int* conn6, double nu, const double* state_host, double* state,
    const double* bc_vals, double* res, double* vals, double diag, double* res_host,
    int precision, void* stream);
/* State VJP of the Taylor-Hood residual: g_state = J(state)^T lam, computed
 * element by element without forming J (the transpose action behind
 * Residual::applyJacT / adjoint solves, femx/state/Residual.hpp:42-59,
 * TimeResidual.hpp:223-227). g_state is overwritten. FP64, or FP32
 * quadrature (FP32_QUAD and MIXED) with FP64 accumulation. */
GBFEM_API int gbfem_vjp_th_ns(const gbfem_assembly_map* map, int num_p2_nodes,
                              const double* coords, const int* conn6, double nu,
                              const double* state, const double* lam, double* g_state,
                              int precision, void* stream);

/* ---------------------------------------------------------------------------
 * femx's NS time operator — the equal-order GLS Navier-Stokes step of
 * NavierOperator (femx/model/ns/Components.hpp:330-577) on P1 triangles,
 * assembled like femx's time assemble with wrt = NextState
 * (Assembly.hpp:235-303, CudaAssembly.hpp:367-413, the kernel
 * assembleTimeKernel): res = K(hist) nxt - F(hist), vals = K (the
 * next-state Jacobian; null for the residual alone, assembleResidual
 * CudaAssembly.hpp:420-472). Crank-Nicolson with AB2 advection at step > 0
 * when num_hist > 1; GLS tau with femx's streamline element length.
 * Local DOFs in femx's mixed layout: velocity (node, comp) then pressure
 * (9 per element); conn = the 3 vertices; hist lag-major (num_hist x
 * num_states, lag 0 = current state). FP64. wrt_hist_lag selects the
 * Jacobian block as femx's VariableBlock: -1 = NextState (K); a history lag
 * gives the zero matrix, as femx's operator does (its history derivatives
 * are VJPs only, Components.hpp:412-435).
 * gbfem_vjp_navier_hist: out[lag][dof] = d(adj . R)/d hist[lag][dof] — the
 * history VJP femx obtains from Enzyme (histVjp / histVjpKernel,
 * Components.cpp:67-125, Components.cu:25-98), here reverse mode written
 * out by hand; out (num_hist x num_states) is overwritten.
 * ------------------------------------------------------------------------ */
GBFEM_API int gbfem_assemble_navier(const gbfem_assembly_map* map, int num_nodes,
                                    const double* coords, const int* conn, double rho,
                                    double mu, double dt, int step, int num_hist,
                                    int wrt_hist_lag, const double* hist, const double* nxt,
                                    double* res, double* vals, void* stream);
GBFEM_API int gbfem_vjp_navier_hist(const gbfem_assembly_map* map, int num_nodes,
                                    const double* coords, const int* conn, double rho,
                                    double mu, double dt, int step, int num_hist,
                                    const double* hist, const double* nxt, const double* adj,
                                    double* out, void* stream);

/* ---------------------------------------------------------------------------
 * Batched assembly: many independent instances (meshes of uneven size, P1
 * Poisson and Taylor-Hood NS mixed) assembled by one persistent launch.
 * Each instance is the work of one gbfem_assemble_p1_kappa /
 * gbfem_assemble_th_ns call (femx's assembly::assemble per instance,
 * CudaAssembly.hpp:319-364) plus, when `lam` is given, the residual VJPs:
 * P1: g_state = K^T lam, g_control[e] = lam_e^T K_e u_e (gbfem_vjp_p1_kappa);
 * Taylor-Hood: g_state = J^T lam of the assembled Jacobian. femx has no
 * batched entry; this replaces a loop of per-instance calls.
 * gbfem_batch_run enqueues two kernels (zero outputs, persistent assembly;
 * MIXED adds a flat launch for the Taylor-Hood residuals), allocates nothing
 * and does not synchronize.
 * ------------------------------------------------------------------------ */
#define GBFEM_BATCH_P1_KAPPA 1
#define GBFEM_BATCH_TH_NS 2

typedef struct
{
  int                       kind; /* GBFEM_BATCH_P1_KAPPA or GBFEM_BATCH_TH_NS */
  const gbfem_assembly_map* map;
  int                       num_nodes;
  const double*             coords;  /* [num_nodes][2], 16-byte aligned */
  const int*                conn;    /* P1: [E][3] or NULL; Taylor-Hood: conn6 */
  const double*             kappa;   /* P1 */
  const double*             f_nodal; /* P1, may be NULL */
  double                    nu;      /* Taylor-Hood */
  const double*             state;
  const double*             lam;       /* adjoint; NULL skips the VJP */
  double*                   res;       /* [num_res] */
  double*                   vals;      /* [nnz] */
  double*                   g_state;   /* [num_states] */
  double*                   g_control; /* P1: [num_elems] */
} gbfem_batch_instance;

typedef struct gbfem_batch gbfem_batch;

GBFEM_API int       gbfem_batch_create(int num_instances,
                                       const gbfem_batch_instance* instances,
                                       void* stream, gbfem_batch** out);
/* precision: GBFEM_PREC_FP64, GBFEM_PREC_FP32_QUAD or GBFEM_PREC_MIXED
 * (Jacobian from FP32 quadrature; residual and P1 gradients in FP64; the
 * Taylor-Hood J^T lam uses the FP32 Jacobian), optionally OR-ed with
 * GBFEM_COLOURED (FP64 and FP32_QUAD): every instance's map coloured before
 * gbfem_batch_create, the persistent kernel then runs once per colour round
 * (colour r of every instance) with plain adds, bitwise reproducible. Work
 * items are p1_chunk P1 elements (multiple of 128) or th_chunk Taylor-Hood
 * elements (multiple of 8); the grid is blocks_per_sm x SM count.
 * stage_depth 1: a block claims its next work item while running the current
 * one and prefetches that item's DOF table, connectivity and coefficients
 * into L2 (0: claims one at a time). */
GBFEM_API int       gbfem_batch_run(gbfem_batch* batch, int precision, int p1_chunk,
                                    int th_chunk, int blocks_per_sm, int stage_depth,
                                    void* stream);
GBFEM_API int       gbfem_batch_check(const gbfem_batch* batch, void* stream);
GBFEM_API long long gbfem_batch_num_elems(const gbfem_batch* batch);
GBFEM_API void      gbfem_batch_destroy(gbfem_batch* batch);

#ifdef __cplusplus
}
#endif

#endif /* GBFEM_H */
