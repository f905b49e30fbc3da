/*
 * femx_oracle.h — CPU oracle for the femx assembly hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library restates, in plain C++, the
 * reference algorithms of femx (v0.4.0) that the GB300 kernels replace, to
 * check them against: only the test-suite, the smoke check and the CPU legs
 * of the benchmark (its CPU baseline and its reference arm) may load it. The
 * product library (libgbfem) never links or calls it, and has no CPU
 * fallback.
 *
 * Parity is pinned in two ways (tests/test_oracle_golden.py):
 *   - against the known-answer vectors held by the reference's own unit tests
 *     (tests/unit/backend/runBackendAssemblyTests.cpp, runBackendStateTests.cpp,
 *     runCudaAssemblyTests.cu, tests/unit/linalg/runLinalgTests.cpp), and
 *   - against golden dumps produced by the real reference library compiled
 *     from its sources (oracle/ref/Makefile, oracle/ref/ref_driver.cpp;
 *     fixtures under tests/golden/).
 *
 * All functions return 0 on success and a nonzero code on failure; the
 * message of the last failure on the calling thread is orc_last_error(),
 * mirroring femx's require() -> std::runtime_error contract
 * (femx/common/Checks.hpp:11-17).
 */
#ifndef FEMX_ORACLE_H
#define FEMX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

const char* orc_last_error(void);

/* ---- AssemblyMap: femx/assembly/AssemblyMap.cpp:54-176 ------------------ */
/* sizes[0]=nnz, [1]=jac_nnz, [2]=max_res, [3]=max_state, [4]=max_jac */
void* orc_map_create(int num_res, int num_states, int num_elems,
                     const int* res_offsets, const int* res_dofs,
                     const int* state_offsets, const int* state_dofs);
void  orc_map_sizes(const void* map, long long* sizes);
void  orc_map_copy(const void* map, int* row_ptr, int* col_ind,
                   int* jac_offsets, int* jac_map);
void  orc_map_free(void* map);

/* ---- BoundaryMap: femx/assembly/BoundaryMap.cpp:59-139 ------------------ */
/* sizes[0]=num_bcs, [1]=number of constrained-column entries */
void* orc_bc_create(int num_bcs, const int* dofs, int rows, int cols,
                    const int* row_ptr, const int* col_ind);
void  orc_bc_sizes(const void* bc, long long* sizes);
void  orc_bc_copy(const void* bc, int* bc_rows, int* diag, int* col_offsets,
                  int* col_entries, int* col_rows, int* bc_mask);
void  orc_bc_free(void* bc);
/* BoundaryMap.cpp:38-55,208-216 */
int orc_replace_rows(const void* bc, const int* row_ptr, double* vals,
                     double diag);
/* BoundaryMap.cpp:172-189 */
int orc_replace_res(const void* bc, const double* state,
                    const double* bc_vals, double* res);
/* BoundaryMap.cpp:199-207 */
int orc_zero_boundary(const void* bc, double* v);
/* BoundaryMap.cpp:218-247 */
int orc_prepare_forward_solve(const void* bc, const int* row_ptr,
                              double* vals, double* rhs,
                              const double* bc_vals);

/* ---- CSR SpMV: femx/linalg/handler/MatrixHandler.cpp:157-198 ------------ */
void orc_matvec(int rows, const int* row_ptr, const int* col_ind,
                const double* vals, const double* x, double* y,
                double alpha, double beta);
void orc_matvec_t(int rows, int cols, const int* row_ptr, const int* col_ind,
                  const double* vals, const double* x, double* y,
                  double alpha, double beta);

/* ---- P1 triangle quadrature tables: ElementQuadratureData.cpp:14-59 ----- */
void* orc_p1_quad_create(int num_nodes, const double* coords, int num_elems,
                         const int* conn, int order);
void  orc_p1_quad_free(void* quad);
/* The tables themselves, in femx's ElementQuadratureData layout (N [nq][3],
 * dNdx [E][nq][3][2], JxW [E][nq]); valid while the quad lives. */
int   orc_p1_quad_tables(const void* quad, int* nq, const double** N, const double** dNdx,
                         const double** JxW);

/* ---- kappa-weighted P1 Poisson through the generic element loop --------
 * femx/assembly/Assembly.hpp:153-226 with a KappaPoissonP1 element operator
 * written after examples/poisson/PoissonComponents.hpp:35-64:
 *   K_e[i][j] = kappa_e * sum_q dN_i . dN_j JxW_q
 *   res_e[i]  = sum_j K_e[i][j] u_j - sum_q f_h(x_q) N_i(x_q) JxW_q
 * with f_h the P1 interpolant of nodal source values f_nodal (may be NULL).
 * res and vals are overwritten (zeroed, then accumulated). */
int orc_assemble_p1_kappa(const void* map, const void* quad,
                          const int* conn, const double* kappa,
                          const double* f_nodal, const double* u,
                          double* res, double* vals);

/* Residual VJPs of the same operator, the transpose action the adjoint
 * drivers use (femx/state/Residual.hpp:55-59, ReducedFunctional.hpp:94-117):
 *   g_u = (dR/du)^T lam = sum_e K_e^T lam_e          (scattered to nodes)
 *   g_m[e] = lam_e^T dR_e/dm_e = kappa_e lam_e^T Khat_e u_e,  kappa = exp(m)
 * Either output may be NULL. Outputs are overwritten. */
int orc_vjp_p1_kappa(const void* map, const void* quad, const int* conn,
                     const double* kappa, const double* u, const double* lam,
                     double* g_u, double* g_m);

/* ---- Taylor-Hood P2/P1 steady Navier-Stokes (Newton) -------------------
 * Element DOFs (15): velocity 2*a+c for P2 shape a in 0..5 and component c,
 * then pressure 12+b for P1 shape b in 0..2 (femx MixedFESpace layout,
 * MixedFESpace.cpp:57-84, FESpace.cpp:96-106). conn6 holds
 * [v0 v1 v2 m01 m12 m20] per element in P2-node numbering; coords are the
 * P2 nodes. The residual of the Galerkin weak form
 *   R_u(a,c) = int nu grad u_c . grad phi_a + (u . grad u_c) phi_a - p d_c phi_a
 *   R_p(b)   = -int psi_b div u
 * and its exact Jacobian are accumulated through the generic element loop
 * with one evalRow per local row (femx/assembly/Assembly.hpp:153-226), using
 * the 6-point degree-4 triangle rule. state/res/vals in global DOF order.
 * orc_th_quad_create builds the per-element tables once (the analogue of
 * ElementQuadratureData, ElementQuadratureData.cpp:14-59). */
void* orc_th_quad_create(int num_p2_nodes, const double* coords,
                         int num_elems, const int* conn6);
void  orc_th_quad_free(void* th);
/* Assembles elements [elem_begin, elem_end) (the whole mesh when
 * elem_end < 0); outputs are zeroed first. */
int orc_assemble_th_range(const void* map, const void* th, double nu,
                          const double* state, double* res, double* vals,
                          int elem_begin, int elem_end);
/* The same assembly on `nthreads` host threads with atomic adds, the scheme
 * of femx's OpenMP NS assembly (NavierStokesModel.cpp:227-318). */
int orc_assemble_th_threads(const void* map, const void* th, double nu,
                            const double* state, double* res, double* vals,
                            int nthreads);
/* Whole-mesh convenience: builds the tables and assembles every element. */
int orc_assemble_th_ns(const void* map, int num_p2_nodes,
                       const double* coords, const int* conn6, double nu,
                       const double* state, double* res, double* vals);

/* Elements [elem_begin, elem_end) of the P1 assembly (bounded CPU samples). */
int orc_assemble_p1_range(const void* map, const void* quad, const int* conn,
                          const double* kappa, const double* f_nodal,
                          const double* u, double* res, double* vals,
                          int elem_begin, int elem_end);

/* femx's equal-order GLS Navier-Stokes time operator on P1 triangles
 * (NavierOperator, femx/model/ns/Components.hpp:397-577) through the
 * generic time loop with wrt = NextState (Assembly.hpp:235-303): res =
 * K(hist) nxt - F(hist), vals = K. `quad` is an order-2 orc_p1_quad (femx's
 * makeNavierData); hist is lag-major with num_states values per lag, lag 0
 * the current state; vals may be null. */
int orc_assemble_navier(const void* map, const void* quad, double rho, double mu,
                        double dt, int step, int num_hist, const double* hist,
                        const double* nxt, double* res, double* vals);
/* out[lag][dof] = d/d hist[lag][dof] of sum_rows adj . R (femx's history
 * VJP, Components.cpp:67-125, there by Enzyme), here by forward-mode dual
 * numbers per history entry: exact to rounding, for testing. */
int orc_vjp_navier_hist(const void* map, const void* quad, double rho, double mu,
                        double dt, int step, int num_hist, const double* hist,
                        const double* nxt, const double* adj, double* out);

/* The same on `nthreads` host threads with atomic adds (femx's OpenMP NS
 * assembly scheme, NavierStokesModel.cpp:227-318); vals must not be null. */
int orc_assemble_navier_threads(const void* map, const void* quad, double rho, double mu,
                                double dt, int step, int num_hist, const double* hist,
                                const double* nxt, double* res, double* vals, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
