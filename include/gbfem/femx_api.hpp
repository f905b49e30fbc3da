// femx_api.hpp — C++ layer over the libgbfem C ABI with femx's call shapes.
//
// A femx user switches the assembly path by including this header and
// calling the same function names with the same argument order:
//   femx::assembly::makeAssemblyMap(...)          -> gbfem::makeAssemblyMap
//   femx::assembly::assemble(op, geom, map, state, res, jac, ctx)
//                                                 -> gbfem::assemble(...)
//   femx::assembly::makeBoundaryMap / replaceRows / replaceRes /
//     zeroBoundary / prepareForwardSolve          -> same names in gbfem::
//   MatrixHandler<CudaCsrBackend>::matvec/matvecT -> gbfem::matvec/matvecT
// The reference's ElementOperator is a compile-time functor
// (femx/assembly/Assembly.hpp:138-152); a C ABI cannot take one, so this
// layer dispatches on operator tag types (KappaPoissonP1, TaylorHoodNS) to
// the per-physics entry points; any other operator goes through the
// header-only templated kernels of generic_assembly.cuh. Failures throw
// std::runtime_error with femx's messages, like femx::require
// (femx/common/Checks.hpp:11-17).
// Every array is a device pointer; the stream comes from the CudaContext.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>

#include "../gbfem.h"

#if defined(__CUDACC__)
#define GBFEM_HD __host__ __device__
#else
#define GBFEM_HD
#endif

namespace gbfem
{

using Real  = double;       // femx/common/Types.hpp:17
using Index = std::int32_t; // femx/common/Types.hpp:19

/** Jacobian block of a time residual (femx/state/TimeResidual.hpp:94-166). */
class VariableBlock
{
public:
  enum class Kind : int
  {
    HistoryState,
    NextState,
    Param
  };
  GBFEM_HD constexpr VariableBlock(Kind kind = Kind::HistoryState, Index lag = 0)
    : kind_(kind), lag_(lag)
  {
  }
  GBFEM_HD static constexpr VariableBlock hist(Index lag) { return {Kind::HistoryState, lag}; }
  GBFEM_HD static constexpr VariableBlock next() { return {Kind::NextState, 0}; }
  GBFEM_HD static constexpr VariableBlock param() { return {Kind::Param, 0}; }
  GBFEM_HD constexpr bool  isHistoryState() const { return kind_ == Kind::HistoryState; }
  GBFEM_HD constexpr bool  isNextState() const { return kind_ == Kind::NextState; }
  GBFEM_HD constexpr bool  isParam() const { return kind_ == Kind::Param; }
  GBFEM_HD constexpr Index historyLag() const { return lag_; }

private:
  Kind  kind_;
  Index lag_;
};

inline void check(int rc)
{
  if (rc != GBFEM_OK)
  {
    throw std::runtime_error(gbfem_last_error());
  }
}

inline void require(bool cond, const char* msg)
{
  if (!cond)
  {
    throw std::runtime_error(msg);
  }
}

/** One stream, like femx::CudaContext (femx/common/Context.hpp:26-90). */
struct CudaContext
{
  void* stream{nullptr}; // cudaStream_t
};

/** Non-owning device vector view (femx/linalg/View.hpp). */
template <class T>
struct DeviceView
{
  T*    ptr{nullptr};
  Index n{0};
  T*    data() const { return ptr; }
  Index size() const { return n; }
};
using DeviceVectorView      = DeviceView<Real>;
using DeviceConstVectorView = DeviceView<const Real>;

/** Non-owning device geometry (femx/fem/Geometry.hpp:33-196) with a fixed
 * node count per element: node-major coords [num_nodes][dim], element-major
 * connectivity [num_elems][nodes_per_elem]. The tagged fast paths are 2-D;
 * user operators (generic_assembly.cuh) take any dim. */
struct DeviceGeometry
{
  Index        num_nodes{0};
  Index        num_elems{0};
  Index        nodes_per_elem{0};
  const Real*  coords{nullptr};
  const Index* conn{nullptr};
  Index        dim{2};
};

/** Shared immutable CSR pattern with a layout identity
 * (femx/linalg/CsrPattern.hpp:42-217). */
struct DeviceCsrPattern
{
  Index              rows{0}, cols{0}, nnz{0};
  const Index*       row_ptr{nullptr};
  const Index*       col_ind{nullptr};
  unsigned long long layout_id{0};
};

/** CSR values over a pattern (femx/linalg/CsrMatrix.hpp:17-105). */
struct DeviceCsrMatrix
{
  DeviceCsrPattern pattern;
  Real*            vals{nullptr};
};

/** Owning device AssemblyMap (femx/assembly/AssemblyMap.hpp:78-206). */
class DeviceAssemblyMap
{
public:
  explicit DeviceAssemblyMap(gbfem_assembly_map* h) : h_(h, &gbfem_assembly_map_destroy)
  {
    check(gbfem_assembly_map_get_view(h, &v_));
  }
  Index numElems() const { return v_.num_elems; }
  Index numRes() const { return v_.num_res; }
  Index numStates() const { return v_.num_states; }
  Index maxRes() const { return v_.max_res; }
  Index maxState() const { return v_.max_state; }
  Index maxJac() const { return v_.max_jac; }
  DeviceCsrPattern pattern() const
  {
    return {v_.num_res, v_.num_states, v_.nnz, v_.row_ptr, v_.col_ind, v_.layout_id};
  }
  const gbfem_assembly_map_view& view() const { return v_; }
  gbfem_assembly_map*            handle() const { return h_.get(); }
  /** Builds the row-gather tables deterministic assembly needs (setup). */
  void enableDeterministic(CudaContext& ctx) const
  {
    check(gbfem_assembly_map_enable_gather(h_.get(), ctx.stream));
  }

private:
  std::shared_ptr<gbfem_assembly_map> h_;
  gbfem_assembly_map_view             v_{};
};

/** Owning device BoundaryMap (femx/assembly/BoundaryMap.hpp:69-175). */
class DeviceBoundaryMap
{
public:
  explicit DeviceBoundaryMap(gbfem_boundary_map* h) : h_(h, &gbfem_boundary_map_destroy)
  {
    check(gbfem_boundary_map_get_view(h, &v_));
  }
  Index                          rows() const { return v_.num_rows; }
  Index                          numBcs() const { return v_.num_bcs; }
  unsigned long long             layoutId() const { return v_.layout_id; }
  const gbfem_boundary_map_view& view() const { return v_; }
  gbfem_boundary_map*            handle() const { return h_.get(); }

private:
  std::shared_ptr<gbfem_boundary_map> h_;
  gbfem_boundary_map_view             v_{};
};

/** makeAssemblyMap(num_res, num_states, res_dofs, state_dofs) over
 * flattened device tables (AssemblyMap.hpp:230-234). */
inline DeviceAssemblyMap makeAssemblyMap(Index num_res, Index num_states, Index num_elems,
                                         const Index* res_offsets, const Index* res_dofs,
                                         const Index* state_offsets,
                                         const Index* state_dofs, CudaContext& ctx)
{
  gbfem_assembly_map* h = nullptr;
  check(gbfem_assembly_map_create(num_res, num_states, num_elems, res_offsets, res_dofs,
                                  state_offsets, state_dofs, ctx.stream, &h));
  return DeviceAssemblyMap(h);
}

/** makeBoundaryMap(dofs, pattern) (BoundaryMap.hpp:183-184). */
inline DeviceBoundaryMap makeBoundaryMap(DeviceView<const Index> dofs,
                                         const DeviceCsrPattern& pattern, CudaContext& ctx)
{
  gbfem_boundary_map* h = nullptr;
  check(gbfem_boundary_map_create(dofs.size(), dofs.data(), pattern.rows, pattern.cols,
                                  pattern.row_ptr, pattern.col_ind, pattern.layout_id,
                                  ctx.stream, &h));
  return DeviceBoundaryMap(h);
}

namespace detail
{
inline void checkLayout(const DeviceBoundaryMap& map, const DeviceCsrMatrix& mat)
{
  require(mat.pattern.layout_id == map.layoutId(),
          "BoundaryMap matrix does not match the mapped CSR layout");
}
inline void checkLayout(const DeviceAssemblyMap& map, const DeviceCsrMatrix& mat)
{
  require(mat.pattern.layout_id == map.pattern().layout_id,
          "Assembly matrix must use the AssemblyMap CSR layout");
}
} // namespace detail

/** replaceRows(map, jac, diag, ctx) (BoundaryMap.hpp:215-226). */
inline void replaceRows(const DeviceBoundaryMap& map, DeviceCsrMatrix& jac, Real diag,
                        CudaContext& ctx)
{
  detail::checkLayout(map, jac);
  check(gbfem_replace_rows(map.handle(), jac.vals, diag, ctx.stream));
}

/** replaceRes(map, state, bc_vals, res, ctx) (BoundaryMap.hpp:246-250). */
inline void replaceRes(const DeviceBoundaryMap& map, DeviceConstVectorView state,
                       DeviceConstVectorView bc_vals, DeviceVectorView res, CudaContext& ctx)
{
  require(state.size() == map.rows() && res.size() == map.rows()
              && bc_vals.size() == map.numBcs(),
          "BoundaryMap residual vectors have incompatible sizes");
  check(gbfem_replace_res(map.handle(), state.data(), bc_vals.data(), res.data(), ctx.stream));
}

/** zeroBoundary(map, vals, ctx) (BoundaryMap.hpp:255-258). */
inline void zeroBoundary(const DeviceBoundaryMap& map, DeviceVectorView vals, CudaContext& ctx)
{
  require(vals.size() == map.rows(), "BoundaryMap vector has incompatible size");
  check(gbfem_zero_boundary(map.handle(), vals.data(), ctx.stream));
}

/** prepareForwardSolve(map, solve_mat, rhs, bc_vals, ctx)
 * (BoundaryMap.hpp:287-291). */
inline void prepareForwardSolve(const DeviceBoundaryMap& map, DeviceCsrMatrix& solve_mat,
                                DeviceVectorView rhs, DeviceConstVectorView bc_vals,
                                CudaContext& ctx)
{
  detail::checkLayout(map, solve_mat);
  require(rhs.size() == map.rows() && bc_vals.size() == map.numBcs(),
          "BoundaryMap forward vectors have incompatible sizes");
  check(gbfem_prepare_forward_solve(map.handle(), solve_mat.vals, rhs.data(), bc_vals.data(),
                                    ctx.stream));
}

/** MatrixHandler<CudaCsrBackend>::matvec: y = alpha A x + beta y. */
inline void matvec(const DeviceCsrMatrix& mat, DeviceConstVectorView x, DeviceVectorView y,
                   Real alpha, Real beta, CudaContext& ctx)
{
  require(x.size() == mat.pattern.cols && y.size() == mat.pattern.rows,
          "CSR matvec vectors have incompatible sizes");
  check(gbfem_spmv(mat.pattern.rows, mat.pattern.cols, mat.pattern.row_ptr,
                   mat.pattern.col_ind, mat.vals, x.data(), y.data(), alpha, beta, ctx.stream));
}

/** MatrixHandler<CudaCsrBackend>::matvecT: y = alpha A^T x + beta y. */
inline void matvecT(const DeviceCsrMatrix& mat, DeviceConstVectorView x, DeviceVectorView y,
                    Real alpha, Real beta, CudaContext& ctx)
{
  require(x.size() == mat.pattern.rows && y.size() == mat.pattern.cols,
          "CSR matvecT vectors have incompatible sizes");
  check(gbfem_spmv_t(mat.pattern.rows, mat.pattern.cols, mat.pattern.row_ptr,
                     mat.pattern.col_ind, mat.vals, x.data(), y.data(), alpha, beta,
                     ctx.stream));
}

enum class Precision : int
{
  FP64     = GBFEM_PREC_FP64,
  FP32Quad = GBFEM_PREC_FP32_QUAD,
  Mixed    = GBFEM_PREC_MIXED,
  DoubleFloat = GBFEM_PREC_DOUBLE_FLOAT,
};

/** Element operator tag: kappa-weighted P1 Poisson with nodal load. */
struct KappaPoissonP1
{
  const Real* kappa{nullptr};   // [num_elems]
  const Real* f_nodal{nullptr}; // [num_nodes] or nullptr
  Precision   precision{Precision::FP64};
};

/** Element operator tag: Taylor-Hood P2/P1 steady Navier-Stokes (Newton). */
struct TaylorHoodNS
{
  Real      nu{1.0};
  Precision precision{Precision::FP64};
  bool      deterministic{false}; // needs map.enableDeterministic(ctx) first
};

/** assemble(op, geom, map, state, res, jac, ctx) for KappaPoissonP1
 * (femx/assembly/CudaAssembly.hpp:319-364). jac.vals may be null. */
inline void assemble(const KappaPoissonP1& op, const DeviceGeometry& geom,
                     const DeviceAssemblyMap& map, DeviceConstVectorView state,
                     DeviceVectorView res, DeviceCsrMatrix& jac, CudaContext& ctx)
{
  require(geom.num_elems == map.numElems(),
          "Geometry and AssemblyMap have different element counts");
  require(state.size() == map.numStates(), "Assembly state size does not match AssemblyMap");
  require(res.size() == map.numRes(), "Assembly residual size does not match AssemblyMap");
  if (jac.vals != nullptr)
  {
    detail::checkLayout(map, jac);
  }
  require(geom.nodes_per_elem == 3 && geom.dim == 2,
          "KappaPoissonP1 expects three-node triangles in 2-D");
  check(gbfem_assemble_p1_kappa(map.handle(), geom.num_nodes, geom.coords, geom.conn, op.kappa,
                                op.f_nodal, state.data(), res.data(), jac.vals,
                                static_cast<int>(op.precision), ctx.stream));
}

/** assemble(op, geom, map, state, res, jac, ctx) for TaylorHoodNS. */
inline void assemble(const TaylorHoodNS& op, const DeviceGeometry& geom,
                     const DeviceAssemblyMap& map, DeviceConstVectorView state,
                     DeviceVectorView res, DeviceCsrMatrix& jac, CudaContext& ctx)
{
  require(geom.num_elems == map.numElems(),
          "Geometry and AssemblyMap have different element counts");
  require(state.size() == map.numStates(), "Assembly state size does not match AssemblyMap");
  require(res.size() == map.numRes(), "Assembly residual size does not match AssemblyMap");
  if (jac.vals != nullptr)
  {
    detail::checkLayout(map, jac);
  }
  require(geom.nodes_per_elem == 6 && geom.dim == 2,
          "Taylor-Hood geometry expects six-node triangles in 2-D");
  const int mode = static_cast<int>(op.precision) | (op.deterministic ? GBFEM_DETERMINISTIC : 0);
  check(gbfem_assemble_th_ns(map.handle(), geom.num_nodes, geom.coords, geom.conn, op.nu,
                             state.data(), res.data(), jac.vals, mode, ctx.stream));
}

/** Residual VJPs of KappaPoissonP1: g_u = (dR/du)^T lam, g_m = (dR/dm)^T lam
 * with kappa = exp(m) — the transpose actions behind Residual::applyParamJacT
 * (femx/state/Residual.hpp:55-59). Either output may have a null pointer. */
inline void applyJacT(const KappaPoissonP1& op, const DeviceGeometry& geom,
                      const DeviceAssemblyMap& map, DeviceConstVectorView state,
                      DeviceConstVectorView lam, DeviceVectorView g_u, DeviceVectorView g_m,
                      CudaContext& ctx)
{
  require(lam.size() == map.numRes() && state.size() == map.numStates(),
          "VJP vectors have incompatible sizes");
  check(gbfem_vjp_p1_kappa(map.handle(), geom.num_nodes, geom.coords, geom.conn, op.kappa,
                           state.data(), lam.data(), g_u.data(), g_m.data(),
                           static_cast<int>(op.precision), ctx.stream));
}

/** Element operator tag: femx's equal-order GLS Navier-Stokes time step
 * (NavierOperator, femx/model/ns/Components.hpp:397-577) on P1 triangles;
 * femx carries the element data in the operator (NavierDataView), this tag
 * carries the geometry it is computed from. */
struct NavierGLS
{
  DeviceGeometry geom;
  Real           rho{1.0}, mu{1.0}, dt{1.0};
};

/** Time assemble (femx/assembly/CudaAssembly.hpp:367-413) for NavierGLS:
 * res = K(hist) nxt - F(hist) and the Jacobian block `wrt` (K for the next
 * state; zero for a history lag, as femx's operator). jac.vals may be null. */
inline void assemble(const NavierGLS& op, Index step, Index num_hist, VariableBlock wrt,
                     const DeviceAssemblyMap& map, DeviceConstVectorView hist,
                     DeviceConstVectorView nxt, DeviceVectorView res, DeviceCsrMatrix& jac,
                     CudaContext& ctx)
{
  require(num_hist > 0 && hist.size() == num_hist * map.numStates()
              && nxt.size() == map.numStates(),
          "Time assembly state dimensions do not match AssemblyMap");
  require(!wrt.isParam()
              && (!wrt.isHistoryState()
                  || (wrt.historyLag() >= 0 && wrt.historyLag() < num_hist)),
          "Time assembly variable block is invalid");
  require(res.size() == map.numRes(), "Time assembly residual size does not match AssemblyMap");
  if (jac.vals != nullptr)
  {
    require(jac.pattern.layout_id == map.pattern().layout_id,
            "Time assembly matrix must use the AssemblyMap CSR layout");
  }
  require(op.geom.nodes_per_elem == 3 && op.geom.dim == 2,
          "Navier operator expects three-node triangles in 2-D");
  check(gbfem_assemble_navier(map.handle(), op.geom.num_nodes, op.geom.coords, op.geom.conn,
                              op.rho, op.mu, op.dt, step, num_hist,
                              wrt.isNextState() ? -1 : wrt.historyLag(), hist.data(),
                              nxt.data(), res.data(), jac.vals, ctx.stream));
}

/** History VJP of NavierGLS: out = (dR/d hist)^T adj for every lag
 * (num_hist x numStates, lag-major) — femx's histVjp (Components.cpp:67-125)
 * behind ConstrainedTimeResidual::applyJacT (:379-405), which zeroes the
 * constrained adjoint entries first (zeroBoundary). */
inline void applyHistJacT(const NavierGLS& op, Index step, Index num_hist,
                          const DeviceAssemblyMap& map, DeviceConstVectorView hist,
                          DeviceConstVectorView nxt, DeviceConstVectorView adj,
                          DeviceVectorView out, CudaContext& ctx)
{
  require(num_hist > 0 && hist.size() == num_hist * map.numStates()
              && nxt.size() == map.numStates() && adj.size() == map.numRes()
              && out.size() == num_hist * map.numStates(),
          "Navier history VJP element dimensions do not match");
  check(gbfem_vjp_navier_hist(map.handle(), op.geom.num_nodes, op.geom.coords, op.geom.conn,
                              op.rho, op.mu, op.dt, step, num_hist, hist.data(), nxt.data(),
                              adj.data(), out.data(), ctx.stream));
}

/** State VJP of TaylorHoodNS: g_state = J(state)^T lam without forming J
 * (Residual::applyJacT, femx/state/Residual.hpp:42-59). */
inline void applyJacT(const TaylorHoodNS& op, const DeviceGeometry& geom,
                      const DeviceAssemblyMap& map, DeviceConstVectorView state,
                      DeviceConstVectorView lam, DeviceVectorView g_state, CudaContext& ctx)
{
  require(lam.size() == map.numRes() && state.size() == map.numStates()
              && g_state.size() == map.numStates(),
          "VJP vectors have incompatible sizes");
  require(geom.nodes_per_elem == 6 && geom.dim == 2,
          "Taylor-Hood geometry expects six-node triangles in 2-D");
  check(gbfem_vjp_th_ns(map.handle(), geom.num_nodes, geom.coords, geom.conn, op.nu,
                        state.data(), lam.data(), g_state.data(),
                        static_cast<int>(op.precision), ctx.stream));
}

} // namespace gbfem
