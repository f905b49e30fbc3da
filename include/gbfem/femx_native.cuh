// femx_native.cuh — libgbfem behind femx's own C++ types: the drop-in for
// femx's CUDA assembly path at femx's C++ boundary.
//
// Include it from a CUDA translation unit (nvcc) that has femx's headers on
// its include path, and link libgbfem. It provides, in gbfem::native:
//
//  * assemble(op, geom, map, state, res, jac, ctx) with the signature of
//    femx::assembly::assemble (femx/assembly/CudaAssembly.hpp:319-326) for
//    the KappaPoissonP1 and TaylorHoodNS operator tags, over femx's
//    fem::DeviceGeometry, assembly::DeviceAssemblyMap, DeviceVector,
//    DeviceCsrMatrix and CudaContext, with femx's checks and messages
//    (sizes, aliasing, CsrPattern::layoutId; Assembly.hpp:61-90);
//  * KappaPoissonResidual and TaylorHoodResidual, subclasses of
//    femx::state::Residual<linalg::CudaCsrBackend> (Residual.hpp:42-59),
//    and NavierTimeResidual, a subclass of
//    femx::state::TimeResidual<linalg::CudaCsrBackend> (TimeResidual.hpp:
//    172-239) computing femx's GLS Navier-Stokes operator as femx's own
//    NavierResidual does (femx/model/ns/NavierStokesModel.cpp:374-543).
//    femx's drivers take them unchanged: LinearStateSolver /
//    NewtonStateSolver (femx/state/StateSolver.hpp:90-108,206-249),
//    ReducedFunctional::gradAt (femx/inverse/ReducedFunctional.hpp:94-117),
//    ConstrainedTimeResidual (femx/assembly/ConstrainedTimeResidual.hpp) and
//    TimeIntegrator / TimeReducedFunctional through it.
//
// gbfem builds its own AssemblyMap on the GPU from the femx map's element DOF
// tables; the pattern it builds is femx's, bit for bit (checked once per
// layout here, and by the library's parity tests), so the values of a femx
// DeviceCsrMatrix on the map's pattern are addressed directly. The femx
// layoutId is carried into every gbfem handle, and each call checks that a
// matrix uses the map's layout, as femx does.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include <femx/assembly/AssemblyMap.hpp>
#include <femx/common/Checks.hpp>
#include <femx/common/Context.hpp>
#include <femx/common/Types.hpp>
#include <femx/fem/Geometry.hpp>
#include <femx/linalg/Backend.hpp>
#include <femx/linalg/CsrMatrix.hpp>
#include <femx/linalg/CsrPattern.hpp>
#include <femx/linalg/Vector.hpp>
#include <femx/state/Residual.hpp>
#include <femx/state/TimeResidual.hpp>

#include "femx_api.hpp"

namespace gbfem::native
{

using femx::Index;
using femx::Real;
using Backend = femx::linalg::CudaCsrBackend;

namespace detail
{

inline void cuda(cudaError_t err, const char* what)
{
  if (err != cudaSuccess)
  {
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(err));
  }
}

/** Device buffer owned by an adapter object (setup-time allocation). */
template <class T>
class Buffer
{
public:
  Buffer() = default;
  explicit Buffer(std::size_t n) { resize(n); }
  Buffer(const Buffer&)            = delete;
  Buffer& operator=(const Buffer&) = delete;
  ~Buffer() { cudaFree(p_); }
  void resize(std::size_t n)
  {
    if (n <= n_)
    {
      return;
    }
    T* q = nullptr;
    cuda(cudaMalloc(&q, n * sizeof(T)), "cudaMalloc failed");
    cudaFree(p_);
    p_ = q;
    n_ = n;
  }
  void upload(const T* host, std::size_t n, void* stream)
  {
    resize(n);
    if (n > 0)
    {
      cuda(cudaMemcpyAsync(p_, host, n * sizeof(T), cudaMemcpyHostToDevice,
                           static_cast<cudaStream_t>(stream)),
           "cudaMemcpyAsync failed");
    }
  }
  T*          data() const { return p_; }
  std::size_t size() const { return n_; }

private:
  T*          p_{nullptr};
  std::size_t n_{0};
};

/** Resize a femx device vector only when its size differs (femx's resize
 * always reallocates). */
inline void fit(femx::DeviceVector& v, Index n)
{
  if (v.size() != n)
  {
    v.resize(n);
  }
}

using MapHandle = std::shared_ptr<gbfem_assembly_map>;

inline MapHandle makeMap(Index num_res, Index num_states, Index num_elems,
                         const Index* res_offsets, const Index* res_dofs,
                         const Index* state_offsets, const Index* state_dofs, void* stream)
{
  gbfem_assembly_map* h = nullptr;
  check(gbfem_assembly_map_create(num_res, num_states, num_elems, res_offsets, res_dofs,
                                  state_offsets, state_dofs, stream, &h));
  return MapHandle(h, &gbfem_assembly_map_destroy);
}

/** The gbfem pattern must be the femx pattern: row_ptr and col_ind are
 * compared once per layout (setup). */
inline void requireSamePattern(const gbfem_assembly_map* map, Index rows, Index nnz,
                               const Index* femx_row_ptr, const Index* femx_col_ind,
                               bool femx_on_device, void* stream)
{
  gbfem_assembly_map_view v{};
  check(gbfem_assembly_map_get_view(map, &v));
  femx::require(v.num_res == rows && v.nnz == nnz,
                "AssemblyMap pattern does not match the gbfem pattern");
  std::vector<Index> a(rows + 1), b(rows + 1), ca(nnz), cb(nnz);
  auto s = static_cast<cudaStream_t>(stream);
  cuda(cudaMemcpyAsync(a.data(), v.row_ptr, sizeof(Index) * (rows + 1), cudaMemcpyDeviceToHost,
                       s),
       "cudaMemcpyAsync failed");
  if (nnz > 0)
  {
    cuda(cudaMemcpyAsync(ca.data(), v.col_ind, sizeof(Index) * nnz, cudaMemcpyDeviceToHost, s),
         "cudaMemcpyAsync failed");
  }
  const cudaMemcpyKind k = femx_on_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
  cuda(cudaMemcpyAsync(b.data(), femx_row_ptr, sizeof(Index) * (rows + 1), k, s),
       "cudaMemcpyAsync failed");
  if (nnz > 0)
  {
    cuda(cudaMemcpyAsync(cb.data(), femx_col_ind, sizeof(Index) * nnz, k, s),
         "cudaMemcpyAsync failed");
  }
  cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize failed");
  femx::require(a == b && ca == cb, "AssemblyMap pattern does not match the gbfem pattern");
}

/** gbfem maps bound to femx layouts, one per CsrPattern::layoutId: femx
 * creates a new layoutId for every pattern makeAssemblyMap builds, and its
 * device copies keep it, so the id names one set of DOF tables. Built on the
 * first assemble call with a map (setup: allocates and synchronizes); released
 * by release(map). */
class MapRegistry
{
public:
  static MapRegistry& instance()
  {
    static MapRegistry r;
    return r;
  }

  MapHandle get(const femx::assembly::DeviceAssemblyMap& map, void* stream)
  {
    const std::uint64_t id = map.pattern().layoutId();
    {
      std::lock_guard<std::mutex> lock(m_);
      auto it = maps_.find(id);
      if (it != maps_.end())
      {
        return it->second;
      }
    }
    const auto v = map.view();
    MapHandle  h = makeMap(v.num_res, v.num_states, v.num_elems, v.res_offsets, v.res_dofs,
                           v.state_offsets, v.state_dofs, stream);
    const auto& p = map.pattern();
    requireSamePattern(h.get(), p.rows(), p.nnz(), p.rowPtrData(), p.colIndData(), true,
                       stream);
    std::lock_guard<std::mutex> lock(m_);
    return maps_.emplace(id, std::move(h)).first->second;
  }

  void release(std::uint64_t id)
  {
    std::lock_guard<std::mutex> lock(m_);
    maps_.erase(id);
  }

private:
  std::mutex                                   m_;
  std::unordered_map<std::uint64_t, MapHandle> maps_;
};

/** Flat node-major coordinates (dim 2) and element-major connectivity with a
 * uniform node count, gathered from a femx geometry view on the device. */
__global__ void gatherGeometry(femx::fem::GeometryView<femx::MemorySpace::Device> g,
                               Index npe, double* xy, Index* conn)
{
  const long long i  = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  const long long nn = g.numNodes(), ne = g.numElems();
  if (i < 2 * nn)
  {
    xy[i] = g.coord(static_cast<Index>(i / 2), static_cast<Index>(i % 2));
  }
  if (i < npe * ne)
  {
    conn[i] = g.elemNode(static_cast<Index>(i / npe), static_cast<Index>(i % npe));
  }
}

/** Geometry flattened for the gbfem kernels. */
struct FlatGeometry
{
  Buffer<double> xy;
  Buffer<Index>  conn;
  Index          num_nodes{0}, num_elems{0}, npe{0};

  void fromDevice(const femx::fem::DeviceGeometry& geom, Index expect_npe, void* stream)
  {
    femx::require(geom.dim() == 2, "gbfem's tagged operators expect 2-D geometry");
    femx::require(geom.maxElemNodes() == expect_npe,
                  "Geometry element node count does not match the operator");
    num_nodes = geom.numNodes();
    num_elems = geom.numElems();
    npe       = expect_npe;
    xy.resize(2 * static_cast<std::size_t>(num_nodes));
    conn.resize(static_cast<std::size_t>(npe) * num_elems);
    const long long n = std::max<long long>(2LL * num_nodes, 1LL * npe * num_elems);
    if (n > 0)
    {
      gatherGeometry<<<static_cast<unsigned>((n + 255) / 256), 256, 0,
                       static_cast<cudaStream_t>(stream)>>>(geom.view(), npe, xy.data(),
                                                            conn.data());
      cuda(cudaGetLastError(), "geometry gather launch");
    }
  }

  void fromHost(const femx::fem::HostGeometry& geom, Index expect_npe, void* stream)
  {
    femx::require(geom.dim() == 2, "gbfem's tagged operators expect 2-D geometry");
    const auto g = geom.view();
    num_nodes    = g.numNodes();
    num_elems    = g.numElems();
    npe          = expect_npe;
    std::vector<double> x(2 * static_cast<std::size_t>(num_nodes));
    std::vector<Index>  c(static_cast<std::size_t>(npe) * num_elems);
    for (Index i = 0; i < num_nodes; ++i)
    {
      x[2 * i]     = g.coord(i, 0);
      x[2 * i + 1] = g.coord(i, 1);
    }
    for (Index e = 0; e < num_elems; ++e)
    {
      femx::require(g.elemNumNodes(e) == npe,
                    "Geometry element node count does not match the operator");
      for (Index k = 0; k < npe; ++k)
      {
        c[static_cast<std::size_t>(npe) * e + k] = g.elemNode(e, k);
      }
    }
    xy.upload(x.data(), x.size(), stream);
    conn.upload(c.data(), c.size(), stream);
    cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)),
         "cudaStreamSynchronize failed");
  }
};

inline void checkAssembly(const femx::fem::DeviceGeometry& geom,
                          const femx::assembly::DeviceAssemblyMap& map,
                          const femx::DeviceVector& state, femx::DeviceVector& res,
                          femx::DeviceCsrMatrix& jac)
{
  // femx/assembly/Assembly.hpp:61-90 (checkAssemblyInputs)
  femx::require(geom.numElems() == map.numElems(),
                "Geometry and AssemblyMap have different element counts");
  femx::require(state.size() == map.numStates(),
                "Assembly state size does not match AssemblyMap");
  femx::require(res.size() == map.numRes(), "Assembly residual size does not match AssemblyMap");
  femx::require(jac.pattern().layoutId() == map.pattern().layoutId(),
                "Assembly matrix must use the AssemblyMap CSR layout");
  femx::require(static_cast<const void*>(state.data()) != res.data()
                    && static_cast<const void*>(state.data()) != jac.valsData()
                    && static_cast<const void*>(res.data()) != jac.valsData(),
                "Assembly state, residual, and matrix values must not alias");
}

/** Per-thread scratch geometry of the free assemble() calls. */
inline FlatGeometry& scratchGeometry()
{
  thread_local FlatGeometry g;
  return g;
}

} // namespace detail

/** Drop the gbfem map built for a femx AssemblyMap (its first assemble call
 * built it). */
inline void release(const femx::assembly::DeviceAssemblyMap& map)
{
  detail::MapRegistry::instance().release(map.pattern().layoutId());
}

/** femx::assembly::assemble(op, geom, map, state, res, jac, ctx) for the
 * kappa-weighted P1 Poisson tag (femx/assembly/CudaAssembly.hpp:319-364).
 * The geometry is flattened on the device on every call (2 x 8 bytes per
 * node, 12 per element); the map's gbfem twin is built on its first call. */
inline void assemble(const KappaPoissonP1& op, const femx::fem::DeviceGeometry& geom,
                     const femx::assembly::DeviceAssemblyMap& map,
                     const femx::DeviceVector& state, femx::DeviceVector& res,
                     femx::DeviceCsrMatrix& jac, femx::CudaContext& ctx)
{
  detail::checkAssembly(geom, map, state, res, jac);
  auto  h = detail::MapRegistry::instance().get(map, ctx.stream());
  auto& g = detail::scratchGeometry();
  g.fromDevice(geom, 3, ctx.stream());
  check(gbfem_assemble_p1_kappa(h.get(), g.num_nodes, g.xy.data(), g.conn.data(), op.kappa,
                                op.f_nodal, state.data(), res.data(), jac.valsData(),
                                static_cast<int>(op.precision), ctx.stream()));
}

/** femx::assembly::assemble(op, geom, map, state, res, jac, ctx) for the
 * Taylor-Hood P2/P1 steady Navier-Stokes Newton tag: six-node triangles
 * (vertices, then the midpoints of edges 01, 12, 20), MixedFESpace DOFs. */
inline void assemble(const TaylorHoodNS& op, const femx::fem::DeviceGeometry& geom,
                     const femx::assembly::DeviceAssemblyMap& map,
                     const femx::DeviceVector& state, femx::DeviceVector& res,
                     femx::DeviceCsrMatrix& jac, femx::CudaContext& ctx)
{
  detail::checkAssembly(geom, map, state, res, jac);
  femx::require(!op.deterministic,
                "deterministic Taylor-Hood assembly goes through TaylorHoodResidual");
  auto  h = detail::MapRegistry::instance().get(map, ctx.stream());
  auto& g = detail::scratchGeometry();
  g.fromDevice(geom, 6, ctx.stream());
  check(gbfem_assemble_th_ns(h.get(), g.num_nodes, g.xy.data(), g.conn.data(), op.nu,
                             state.data(), res.data(), jac.valsData(),
                             static_cast<int>(op.precision), ctx.stream()));
}

namespace detail
{

/** What the three residuals share: the gbfem map built from femx's host
 * AssemblyMap, femx's pattern on the device (same layoutId), the geometry,
 * and optionally the Dirichlet rows. */
class ResidualCore
{
public:
  ResidualCore(const femx::fem::HostGeometry& geom, Index npe,
               const femx::assembly::HostAssemblyMap& map, const femx::Array<Index>* bc_dofs,
               const femx::HostVector* bc_vals, femx::CudaContext& ctx)
    : host_pattern_(map.pattern())
  {
    void*      s = ctx.stream();
    const auto v = map.view();
    femx::require(geom.numElems() == v.num_elems,
                  "Geometry and AssemblyMap have different element counts");
    num_elems_  = v.num_elems;
    num_res_    = v.num_res;
    num_states_ = v.num_states;
    const std::size_t nres = v.num_elems > 0 ? v.res_offsets[v.num_elems] : 0;
    const std::size_t nst  = v.num_elems > 0 ? v.state_offsets[v.num_elems] : 0;
    Buffer<Index>     ro, rd, so, sd;
    ro.upload(v.res_offsets, v.num_elems + 1, s);
    rd.upload(v.res_dofs, nres, s);
    so.upload(v.state_offsets, v.num_elems + 1, s);
    sd.upload(v.state_dofs, nst, s);
    map_ = makeMap(v.num_res, v.num_states, v.num_elems, ro.data(), rd.data(), so.data(),
                   sd.data(), s);
    const auto& p = map.pattern();
    requireSamePattern(map_.get(), p.rows(), p.nnz(), p.rowPtrData(), p.colIndData(), false, s);
    femx::copy(host_pattern_, pattern_, ctx); // keeps femx's layoutId
    geom_.fromHost(geom, npe, s);
    if (bc_dofs != nullptr)
    {
      femx::require(bc_vals != nullptr && bc_vals->size() == bc_dofs->size(),
                    "BoundaryMap values do not match the constrained DOFs");
      Buffer<Index> d;
      d.upload(bc_dofs->data(), bc_dofs->size(), s);
      gbfem_assembly_map_view mv{};
      check(gbfem_assembly_map_get_view(map_.get(), &mv));
      gbfem_boundary_map* b = nullptr;
      check(gbfem_boundary_map_create(bc_dofs->size(), d.data(), mv.num_res, mv.num_states,
                                      mv.row_ptr, mv.col_ind, p.layoutId(), s, &b));
      bc_.reset(b, &gbfem_boundary_map_destroy);
      bc_vals_.upload(bc_vals->data(), bc_vals->size(), s);
      num_bcs_ = bc_dofs->size();
    }
    cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(s)), "cudaStreamSynchronize failed");
  }

  gbfem_assembly_map*           map() const { return map_.get(); }
  gbfem_boundary_map*           bc() const { return bc_.get(); }
  const double*                 bcVals() const { return bc_vals_.data(); }
  const FlatGeometry&           geom() const { return geom_; }
  const femx::HostCsrPattern&   hostPattern() const { return host_pattern_; }
  const femx::DeviceCsrPattern& pattern() const { return pattern_; }
  Index                         numElems() const { return num_elems_; }
  Index                         numRes() const { return num_res_; }
  Index                         numStates() const { return num_states_; }

  void requireLayout(const femx::DeviceCsrMatrix& jac) const
  {
    femx::require(jac.pattern().layoutId() == pattern_.layoutId(),
                  "Assembly matrix must use the AssemblyMap CSR layout");
  }

private:
  MapHandle                           map_;
  std::shared_ptr<gbfem_boundary_map> bc_;
  Buffer<double>                      bc_vals_;
  Index                               num_bcs_{0};
  FlatGeometry                        geom_;
  femx::HostCsrPattern                host_pattern_;
  femx::DeviceCsrPattern              pattern_;
  Index                               num_elems_{0}, num_res_{0}, num_states_{0};
};

} // namespace detail

/**
 * Stationary residual R(u, m) = K(kappa) u - F of the kappa-weighted P1
 * Poisson operator, kappa = exp(m) per element (m = the parameter vector),
 * F the load of a nodal source; constrained rows replaced by u - g
 * (replaceRes, BoundaryMap.cpp:172-189) and the Jacobian's by identity rows
 * (replaceRows), the system femx's state solvers and ReducedFunctional use.
 * applyParamJacT: (dR/dm)^T adj with the adjoint's constrained entries
 * zeroed (zeroBoundary), element by element, without forming dR/dm.
 */
class KappaPoissonResidual final : public femx::state::Residual<Backend>
{
public:
  KappaPoissonResidual(const femx::fem::HostGeometry& geom,
                       const femx::assembly::HostAssemblyMap& map,
                       const femx::HostVector& f_nodal, const femx::Array<Index>& bc_dofs,
                       const femx::HostVector& bc_vals, femx::CudaContext& ctx,
                       Precision precision = Precision::FP64)
    : core_(geom, 3, map, &bc_dofs, &bc_vals, ctx), precision_(precision)
  {
    kappa_.resize(core_.numElems());
    scratch_.resize(core_.numRes());
    if (f_nodal.size() > 0)
    {
      femx::require(f_nodal.size() == core_.geom().num_nodes,
                    "Poisson source size does not match the geometry");
      f_.upload(f_nodal.data(), f_nodal.size(), ctx.stream());
      detail::cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(ctx.stream())),
                   "cudaStreamSynchronize failed");
    }
  }

  femx::state::Dimensions dims() const override
  {
    return {core_.numStates(), core_.numElems(), core_.numRes()};
  }
  const femx::HostCsrPattern& hostPattern() const override { return core_.hostPattern(); }
  const Pattern&              pattern() const override { return core_.pattern(); }

  void res(const Vec& state, const Vec& prm, Vec& out, Ctx& ctx) const override
  {
    checkInputs(state, prm);
    detail::fit(out, core_.numRes());
    setKappa(prm, ctx);
    const auto& g = core_.geom();
    check(gbfem_assemble_p1_kappa(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(),
                                  kappa_.data(), f_.data(), state.data(), out.data(), nullptr,
                                  static_cast<int>(precision_), ctx.stream()));
    check(gbfem_replace_res(core_.bc(), state.data(), core_.bcVals(), out.data(),
                            ctx.stream()));
  }

  void assembleStateJac(const Vec& state, const Vec& prm, Mat& out, Ctx& ctx) const override
  {
    checkInputs(state, prm);
    core_.requireLayout(out);
    setKappa(prm, ctx);
    const auto& g = core_.geom();
    check(gbfem_assemble_p1_kappa(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(),
                                  kappa_.data(), f_.data(), state.data(), scratch_.data(),
                                  out.valsData(), static_cast<int>(precision_), ctx.stream()));
    check(gbfem_replace_rows(core_.bc(), out.valsData(), 1.0, ctx.stream()));
  }

  void applyParamJacT(const Vec& state, const Vec& prm, const Vec& adj, Vec& out,
                      Ctx& ctx) const override
  {
    checkInputs(state, prm);
    femx::require(adj.size() == core_.numRes(), "Residual adjoint size mismatch");
    detail::fit(out, core_.numElems());
    setKappa(prm, ctx);
    auto s = static_cast<cudaStream_t>(ctx.stream());
    detail::cuda(cudaMemcpyAsync(scratch_.data(), adj.data(), sizeof(Real) * adj.size(),
                                 cudaMemcpyDeviceToDevice, s),
                 "cudaMemcpyAsync failed");
    check(gbfem_zero_boundary(core_.bc(), scratch_.data(), ctx.stream()));
    const auto& g = core_.geom();
    check(gbfem_vjp_p1_kappa(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(),
                             kappa_.data(), state.data(), scratch_.data(), nullptr, out.data(),
                             static_cast<int>(precision_), ctx.stream()));
  }

private:
  void checkInputs(const Vec& state, const Vec& prm) const
  {
    femx::require(state.size() == core_.numStates(), "Residual state size mismatch");
    femx::require(prm.size() == core_.numElems(), "Residual parameter size mismatch");
  }
  void setKappa(const Vec& prm, Ctx& ctx) const
  {
    check(gbfem_exp(prm.size(), prm.data(), kappa_.data(), ctx.stream()));
  }

  detail::ResidualCore           core_;
  Precision                      precision_;
  mutable detail::Buffer<double> kappa_, scratch_;
  detail::Buffer<double>         f_;
};

/**
 * Stationary Taylor-Hood P2/P1 Navier-Stokes residual (Galerkin, Newton
 * Jacobian) with constrained rows replaced (replaceRes / replaceRows): the
 * system femx's NewtonStateSolver iterates on. The viscosity is fixed at
 * construction; the residual has no parameters (num_param = 0).
 * applyStateJacT: J(state)^T adj with the adjoint's constrained entries
 * zeroed and adj added back on the constrained rows, element by element.
 * deterministic = true assembles bitwise reproducibly (row-gather tables
 * built at construction).
 */
class TaylorHoodResidual final : public femx::state::Residual<Backend>
{
public:
  TaylorHoodResidual(const femx::fem::HostGeometry& geom,
                     const femx::assembly::HostAssemblyMap& map, Real nu,
                     const femx::Array<Index>& bc_dofs, const femx::HostVector& bc_vals,
                     femx::CudaContext& ctx, Precision precision = Precision::FP64,
                     bool deterministic = false)
    : core_(geom, 6, map, &bc_dofs, &bc_vals, ctx), nu_(nu),
      mode_(static_cast<int>(precision) | (deterministic ? GBFEM_DETERMINISTIC : 0)),
      precision_(precision)
  {
    scratch_.resize(core_.numRes());
    if (deterministic)
    {
      check(gbfem_assembly_map_enable_gather(core_.map(), ctx.stream()));
    }
  }

  femx::state::Dimensions dims() const override
  {
    return {core_.numStates(), 0, core_.numRes()};
  }
  const femx::HostCsrPattern& hostPattern() const override { return core_.hostPattern(); }
  const Pattern&              pattern() const override { return core_.pattern(); }

  void res(const Vec& state, const Vec& prm, Vec& out, Ctx& ctx) const override
  {
    checkInputs(state, prm);
    detail::fit(out, core_.numRes());
    const auto& g = core_.geom();
    check(gbfem_assemble_th_ns(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(), nu_,
                               state.data(), out.data(), nullptr, mode_, ctx.stream()));
    check(gbfem_replace_res(core_.bc(), state.data(), core_.bcVals(), out.data(),
                            ctx.stream()));
  }

  void assembleStateJac(const Vec& state, const Vec& prm, Mat& out, Ctx& ctx) const override
  {
    checkInputs(state, prm);
    core_.requireLayout(out);
    const auto& g = core_.geom();
    check(gbfem_assemble_th_ns(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(), nu_,
                               state.data(), scratch_.data(), out.valsData(), mode_,
                               ctx.stream()));
    check(gbfem_replace_rows(core_.bc(), out.valsData(), 1.0, ctx.stream()));
  }

  void applyParamJacT(const Vec& state, const Vec& prm, const Vec& adj, Vec& out,
                      Ctx&) const override
  {
    checkInputs(state, prm);
    femx::require(adj.size() == core_.numRes(), "Residual adjoint size mismatch");
    detail::fit(out, 0); // parameter-free
  }

  /** (dR/dstate)^T adj of the constrained residual, without forming J. */
  void applyStateJacT(const Vec& state, const Vec& adj, Vec& out, Ctx& ctx) const
  {
    femx::require(state.size() == core_.numStates() && adj.size() == core_.numRes(),
                  "Residual adjoint size mismatch");
    detail::fit(out, core_.numStates());
    auto s = static_cast<cudaStream_t>(ctx.stream());
    detail::cuda(cudaMemcpyAsync(scratch_.data(), adj.data(), sizeof(Real) * adj.size(),
                                 cudaMemcpyDeviceToDevice, s),
                 "cudaMemcpyAsync failed");
    check(gbfem_zero_boundary(core_.bc(), scratch_.data(), ctx.stream()));
    const auto& g = core_.geom();
    check(gbfem_vjp_th_ns(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(), nu_,
                          state.data(), scratch_.data(), out.data(),
                          static_cast<int>(precision_), ctx.stream()));
    // constrained rows R_bc = u_bc - g contribute adj_bc to their own DOF:
    // out += adj - zeroBoundary(adj) (the difference is adj on those rows)
    check(gbfem_axpby(adj.size(), 1.0, adj.data(), 1.0, out.data(), ctx.stream()));
    check(gbfem_axpby(adj.size(), -1.0, scratch_.data(), 1.0, out.data(), ctx.stream()));
  }

private:
  void checkInputs(const Vec& state, const Vec& prm) const
  {
    femx::require(state.size() == core_.numStates(), "Residual state size mismatch");
    femx::require(prm.size() == 0, "Taylor-Hood residual is parameter-free");
  }

  detail::ResidualCore           core_;
  Real                           nu_;
  int                            mode_;
  Precision                      precision_;
  mutable detail::Buffer<double> scratch_;
};

/**
 * femx's GLS Navier-Stokes time residual (NavierOperator, equal-order P1/P1,
 * Crank-Nicolson with AB2 advection; femx/model/ns/Components.hpp:330-577)
 * as a TimeResidual<CudaCsrBackend> with the behaviour of femx's own
 * NavierResidual (femx/model/ns/NavierStokesModel.cpp:374-543): two history
 * lags, no parameters, res / assembleNext on the next state, applyJacT for
 * the history lags (femx: Enzyme's reverse mode, here written out by hand)
 * and an empty parameter block; the next-state block has no transpose apply,
 * as in femx (its adjoint solves with the assembled Jacobian). Decorate it
 * with femx's ConstrainedTimeResidual for the Dirichlet constraints.
 */
class NavierTimeResidual final : public femx::state::TimeResidual<Backend>
{
public:
  static constexpr Index kNumHist = 2;

  NavierTimeResidual(Index nstep, const femx::fem::HostGeometry& geom,
                     const femx::assembly::HostAssemblyMap& map, Real rho, Real mu, Real dt,
                     femx::CudaContext& ctx)
    : core_(geom, 3, map, nullptr, nullptr, ctx), nstep_(nstep), rho_(rho), mu_(mu), dt_(dt)
  {
    hist_grad_.resize(static_cast<std::size_t>(kNumHist) * core_.numStates());
  }

  femx::state::TimeDims dims() const override
  {
    return {nstep_, core_.numStates(), 0, core_.numRes(), kNumHist};
  }
  const femx::HostCsrPattern& hostPattern() const override { return core_.hostPattern(); }
  const Pattern&              pattern() const override { return core_.pattern(); }

  void initialState(ConstView prm, Vec& out, Ctx& ctx) const override
  {
    femx::require(prm.size() == 0, "Navier physics residual is parameter-free");
    detail::fit(out, core_.numStates());
    detail::cuda(cudaMemsetAsync(out.data(), 0, sizeof(Real) * out.size(),
                                 static_cast<cudaStream_t>(ctx.stream())),
                 "cudaMemsetAsync failed");
  }

  void res(const StepCtx& time, Vec& out, Ctx& ctx) const override
  {
    checkCtx(time);
    detail::fit(out, core_.numRes());
    const auto& g = core_.geom();
    check(gbfem_assemble_navier(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(), rho_, mu_,
                                dt_, time.step, kNumHist, -1, time.hist.data(),
                                time.nxt.data(), out.data(), nullptr, ctx.stream()));
  }

  void assembleNext(const StepCtx& time, Vec& res, Mat& jac, Ctx& ctx) const override
  {
    checkCtx(time);
    core_.requireLayout(jac);
    detail::fit(res, core_.numRes());
    const auto& g = core_.geom();
    check(gbfem_assemble_navier(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(), rho_, mu_,
                                dt_, time.step, kNumHist, -1, time.hist.data(),
                                time.nxt.data(), res.data(), jac.valsData(), ctx.stream()));
  }

  void applyJacT(const StepCtx& time, femx::state::VariableBlock wrt, ConstView adj, Vec& out,
                 Ctx& ctx) const override
  {
    checkCtx(time);
    femx::require(!wrt.isNextState(),
                  "Navier transpose apply supports only history and parameter blocks");
    femx::require(adj.size() == core_.numRes(), "Navier residual adjoint size mismatch");
    if (wrt.isParam())
    {
      detail::fit(out, 0);
      return;
    }
    femx::require(wrt.historyLag() >= 0 && wrt.historyLag() < kNumHist,
                  "Navier residual history lag is out of range");
    // one pass gives every lag's VJP; the requested lag is copied out
    const auto& g = core_.geom();
    check(gbfem_vjp_navier_hist(core_.map(), g.num_nodes, g.xy.data(), g.conn.data(), rho_,
                                mu_, dt_, time.step, kNumHist, time.hist.data(),
                                time.nxt.data(), adj.data(), hist_grad_.data(), ctx.stream()));
    detail::fit(out, core_.numStates());
    detail::cuda(
        cudaMemcpyAsync(out.data(),
                        hist_grad_.data()
                            + static_cast<std::size_t>(wrt.historyLag()) * core_.numStates(),
                        sizeof(Real) * core_.numStates(), cudaMemcpyDeviceToDevice,
                        static_cast<cudaStream_t>(ctx.stream())),
        "cudaMemcpyAsync failed");
  }

private:
  // femx's NavierResidual::checkCtx (NavierStokesModel.cpp:550-558)
  void checkCtx(const StepCtx& time) const
  {
    femx::require(time.step >= 0 && time.step < nstep_, "Navier residual step is out of range");
    femx::require(time.hist.count() >= kNumHist && time.hist.stateSize() == core_.numStates()
                      && time.nxt.size() == core_.numStates() && time.prm.size() == 0,
                  "Navier residual vector size mismatch");
  }

  detail::ResidualCore           core_;
  Index                          nstep_;
  Real                           rho_, mu_, dt_;
  mutable detail::Buffer<double> hist_grad_;
};

} // namespace gbfem::native
