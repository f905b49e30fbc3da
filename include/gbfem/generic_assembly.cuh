// generic_assembly.cuh — assembly of user element operators on the GPU.
//
// femx's plug-in point is a compile-time ElementOperator functor with
//   evalRow(ElementView, row, res, jac_row)                (steady)
//   evalRow(TimeElementView, wrt, row, res, jac_row)       (time step)
// (femx/assembly/Assembly.hpp:138-152 and :228-234,
//  femx/assembly/CudaAssembly.hpp:302-318). A C ABI cannot carry a functor,
// so the library's fast paths dispatch on operator tags (femx_api.hpp); any
// other operator compiles here, in the user's translation unit, into a
// templated kernel. Header-only, nvcc only; no CPU fallback.
//
// Kernel shape: a group of G lanes per element, G the smallest power of two
// not below the largest element row count (P1: 4 lanes, eight elements per
// warp; Taylor-Hood and femx's NS element: 16 lanes, two per warp; 32 at
// most); the reference runs one 128-thread block per element,
// CudaAssembly.hpp:100-214. A group stages its element's inputs in shared
// memory, its lanes evaluate rows sub, sub + G, ..., and the group adds the
// element block into res and the CSR values with FP64 atomics through the
// AssemblyMap (jac_map, femx AssemblyMap.hpp:173-188). Results equal femx's
// to rounding; FP64 atomics make the order of the additions into one slot
// run-dependent.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "femx_api.hpp"

namespace gbfem
{

/** Device vector view (femx VectorView<Device, T>, femx/linalg/View.hpp). */
template <class T>
struct Span
{
  T*    ptr{nullptr};
  Index n{0};
  __host__ __device__ T&    operator[](Index i) const { return ptr[i]; }
  __host__ __device__ Index size() const { return n; }
  __host__ __device__ T*    data() const { return ptr; }
  __host__ __device__ Span  subview(Index off, Index count) const { return {ptr + off, count}; }
};

/** Element inputs (femx/assembly/Assembly.hpp:21-28): element index, spatial
 * dimension, node count, element state in local DOF order and node-major
 * element coordinates. */
struct ElementView
{
  Index            ie{0};
  Index            dim{0};
  Index            num_nodes{0};
  Span<const Real> state;
  Span<const Real> coords;
};

/** Time-step element inputs (femx/assembly/Assembly.hpp:31-45): history
 * states lag-major, next state, both in local DOF order. */
struct TimeElementView
{
  Index            ie{0};
  Index            step{0};
  Index            num_hist{0};
  Span<const Real> hist;
  Span<const Real> nxt;
  __host__ __device__ Span<const Real> histState(Index lag) const
  {
    return hist.subview(lag * nxt.size(), nxt.size());
  }
};

namespace detail
{
constexpr int kGenericWarps = 4;

/** Per-element shared-memory staging, in doubles, and the lane group. */
struct GenericLayout
{
  int in{0};    // element inputs (state + coordinates, or history + next)
  int res{0};   // max_res
  int jac{0};   // max_jac
  int group{32}; // lanes per element (a power of two, at most 32)
  __host__ __device__ int per_elem() const { return in + res + jac; }
  __host__ __device__ int per_warp() const { return per_elem() * (32 / group); }
};

/** Lanes per element: the smallest power of two not below max_res. */
inline int genericGroup(int max_res)
{
  int g = 1;
  while (g < max_res && g < 32)
  {
    g *= 2;
  }
  return g;
}

template <class T>
__device__ __forceinline__ void atomicAddF64(T* addr, T v)
{
  atomicAdd(addr, v);
}

template <class Op>
__global__ void __launch_bounds__(32 * kGenericWarps)
    genericAssembleKernel(Op op, int dim, int npe, const Real* __restrict__ coords,
                          const Index* __restrict__ conn, gbfem_assembly_map_view map,
                          const Real* __restrict__ state, Real* __restrict__ res,
                          Real* __restrict__ vals, GenericLayout lay, int max_state)
{
  extern __shared__ Real gbfem_generic_work[];
  const int G    = lay.group;
  const int lane = threadIdx.x & 31;
  const int sub  = lane & (G - 1);
  const int warp = threadIdx.x >> 5;
  const int slot = warp * (32 / G) + lane / G;
  const int ie   = blockIdx.x * kGenericWarps * (32 / G) + slot;
  if (ie >= map.num_elems)
  {
    return; // no barrier follows: groups synchronise on their own lanes
  }
  const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (lane & ~(G - 1));
  Real*       st = gbfem_generic_work + slot * lay.per_elem();
  Real*       xc = st + max_state;
  Real*       re = st + lay.in;
  Real*       jc = re + lay.res;
  const Index r0 = map.res_offsets[ie], nr = map.res_offsets[ie + 1] - r0;
  const Index s0 = map.state_offsets[ie], nc = map.state_offsets[ie + 1] - s0;
  for (Index c = sub; c < nc; c += G)
  {
    st[c] = state[map.state_dofs[s0 + c]];
  }
  for (Index i = sub; i < npe * dim; i += G)
  {
    const Index node = conn[static_cast<long long>(ie) * npe + i / dim];
    xc[i]            = coords[static_cast<long long>(node) * dim + i % dim];
  }
  __syncwarp(gmask);
  const ElementView ev{ie, dim, npe, {st, nc}, {xc, npe * dim}};
  for (Index row = sub; row < nr; row += G)
  {
    Real r = 0.0;
    op.evalRow(ev, row, r, Span<Real>{jc + row * nc, nc});
    re[row] = r;
  }
  __syncwarp(gmask);
  for (Index row = sub; row < nr; row += G)
  {
    atomicAddF64(res + map.res_dofs[r0 + row], re[row]);
  }
  if (vals != nullptr)
  {
    const Index j0 = map.jac_offsets[ie];
    for (Index i = sub; i < nr * nc; i += G)
    {
      atomicAddF64(vals + map.jac_map[j0 + i], jc[i]);
    }
  }
}

template <class Op>
__global__ void __launch_bounds__(32 * kGenericWarps)
    genericTimeKernel(Op op, Index step, Index num_hist, VariableBlock wrt,
                      gbfem_assembly_map_view map, const Real* __restrict__ hist,
                      const Real* __restrict__ nxt, Real* __restrict__ res,
                      Real* __restrict__ vals, GenericLayout lay, int max_state)
{
  extern __shared__ Real gbfem_generic_work[];
  const int G    = lay.group;
  const int lane = threadIdx.x & 31;
  const int sub  = lane & (G - 1);
  const int warp = threadIdx.x >> 5;
  const int slot = warp * (32 / G) + lane / G;
  const int ie   = blockIdx.x * kGenericWarps * (32 / G) + slot;
  if (ie >= map.num_elems)
  {
    return;
  }
  const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (lane & ~(G - 1));
  Real*       hs = gbfem_generic_work + slot * lay.per_elem();
  Real*       nx = hs + num_hist * max_state;
  Real*       re = hs + lay.in;
  Real*       jc = re + lay.res;
  const Index r0 = map.res_offsets[ie], nr = map.res_offsets[ie + 1] - r0;
  const Index s0 = map.state_offsets[ie], nc = map.state_offsets[ie + 1] - s0;
  // history lag-major with numStates() values per lag (Assembly.hpp:274-282)
  for (Index i = sub; i < num_hist * nc; i += G)
  {
    const Index lag = i / nc, col = i - lag * nc;
    hs[i] = hist[static_cast<long long>(lag) * map.num_states + map.state_dofs[s0 + col]];
  }
  for (Index c = sub; c < nc; c += G)
  {
    nx[c] = nxt[map.state_dofs[s0 + c]];
  }
  __syncwarp(gmask);
  const TimeElementView ev{ie, step, num_hist, {hs, num_hist * nc}, {nx, nc}};
  for (Index row = sub; row < nr; row += G)
  {
    Real r = 0.0;
    op.evalRow(ev, wrt, row, r, Span<Real>{jc + row * nc, nc});
    re[row] = r;
  }
  __syncwarp(gmask);
  for (Index row = sub; row < nr; row += G)
  {
    atomicAddF64(res + map.res_dofs[r0 + row], re[row]);
  }
  if (vals != nullptr)
  {
    const Index j0 = map.jac_offsets[ie];
    for (Index i = sub; i < nr * nc; i += G)
    {
      atomicAddF64(vals + map.jac_map[j0 + i], jc[i]);
    }
  }
}

inline void cudaCheckApi(cudaError_t e, const char* what)
{
  if (e != cudaSuccess)
  {
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
  }
}

template <class Kernel>
inline unsigned prepareLaunch(Kernel kernel, const GenericLayout& lay, size_t* smem)
{
  *smem = sizeof(Real) * static_cast<size_t>(lay.per_warp()) * kGenericWarps;
  if (*smem > 48 * 1024)
  {
    cudaCheckApi(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(*smem)),
                 "generic assembly shared memory");
  }
  return 32 * kGenericWarps;
}
} // namespace detail

/** assemble(op, geom, map, state, res, jac, ctx) for a user operator
 * (femx/assembly/CudaAssembly.hpp:319-364): zeroes res and the CSR values,
 * then adds every element's rows. geom.dim gives the coordinate layout
 * [num_nodes][dim]. jac.vals may be null (residual only; evalRow still gets
 * a Jacobian row to write). */
template <class Op>
void assemble(const Op& op, const DeviceGeometry& geom, const DeviceAssemblyMap& map,
              DeviceConstVectorView state, DeviceVectorView res, DeviceCsrMatrix& jac,
              CudaContext& ctx)
{
  static_assert(std::is_trivially_copyable<Op>::value,
                "CUDA ElementOperator must be trivially copyable");
  require(geom.num_elems == map.numElems(),
          "Geometry and AssemblyMap have different element counts");
  require(state.size() == map.numStates(), "Assembly state size does not match AssemblyMap");
  require(res.size() == map.numRes(), "Assembly residual size does not match AssemblyMap");
  require(state.data() != res.data() && state.data() != jac.vals && res.data() != jac.vals,
          "Assembly state, residual, and matrix values must not alias");
  if (jac.vals != nullptr)
  {
    detail::checkLayout(map, jac);
  }
  const auto s = static_cast<cudaStream_t>(ctx.stream);
  detail::cudaCheckApi(cudaMemsetAsync(res.data(), 0, sizeof(Real) * res.size(), s), "zero");
  if (jac.vals != nullptr)
  {
    detail::cudaCheckApi(
        cudaMemsetAsync(jac.vals, 0, sizeof(Real) * jac.pattern.nnz, s), "zero");
  }
  if (map.numElems() == 0)
  {
    return;
  }
  const auto&           v = map.view();
  detail::GenericLayout lay;
  lay.in    = v.max_state + geom.nodes_per_elem * geom.dim;
  lay.res   = v.max_res;
  lay.jac   = v.max_jac;
  lay.group = detail::genericGroup(v.max_res);
  size_t         smem    = 0;
  const auto     kernel  = detail::genericAssembleKernel<Op>;
  const unsigned threads = detail::prepareLaunch(kernel, lay, &smem);
  const unsigned per_blk = detail::kGenericWarps * (32 / lay.group);
  const unsigned blocks  = (static_cast<unsigned>(map.numElems()) + per_blk - 1) / per_blk;
  kernel<<<blocks, threads, smem, s>>>(op, geom.dim, geom.nodes_per_elem, geom.coords, geom.conn,
                                       v, state.data(), res.data(), jac.vals, lay, v.max_state);
  detail::cudaCheckApi(cudaGetLastError(), "generic assembly launch");
}

/** assemble(op, step, num_hist, wrt, map, hist, nxt, res, jac, ctx): one time
 * residual and the Jacobian block `wrt` (next state or a history lag)
 * (femx/assembly/CudaAssembly.hpp:367-413, CPU Assembly.hpp:235-303). hist
 * is lag-major, num_hist * numStates() values. jac.vals may be null (the
 * residual alone, assembleResidual, CudaAssembly.hpp:420-472). */
template <class Op>
void assemble(const Op& op, Index step, Index num_hist, VariableBlock wrt,
              const DeviceAssemblyMap& map, DeviceConstVectorView hist,
              DeviceConstVectorView nxt, DeviceVectorView res, DeviceCsrMatrix& jac,
              CudaContext& ctx)
{
  static_assert(std::is_trivially_copyable<Op>::value,
                "CUDA time ElementOperator must be trivially copyable");
  require(num_hist > 0 && hist.size() == num_hist * map.numStates()
              && nxt.size() == map.numStates(),
          "Time assembly state dimensions do not match AssemblyMap");
  require(!wrt.isParam()
              && (!wrt.isHistoryState()
                  || (wrt.historyLag() >= 0 && wrt.historyLag() < num_hist)),
          "Time assembly variable block is invalid");
  require(res.size() == map.numRes(), "Time assembly residual size does not match AssemblyMap");
  require(hist.data() != res.data() && hist.data() != jac.vals && nxt.data() != res.data()
              && nxt.data() != jac.vals && res.data() != jac.vals,
          "Time assembly outputs must not alias inputs or each other");
  if (jac.vals != nullptr)
  {
    require(jac.pattern.layout_id == map.pattern().layout_id,
            "Time assembly matrix must use the AssemblyMap CSR layout");
  }
  const auto s = static_cast<cudaStream_t>(ctx.stream);
  detail::cudaCheckApi(cudaMemsetAsync(res.data(), 0, sizeof(Real) * res.size(), s), "zero");
  if (jac.vals != nullptr)
  {
    detail::cudaCheckApi(
        cudaMemsetAsync(jac.vals, 0, sizeof(Real) * jac.pattern.nnz, s), "zero");
  }
  if (map.numElems() == 0)
  {
    return;
  }
  const auto&           v = map.view();
  detail::GenericLayout lay;
  lay.in    = (num_hist + 1) * v.max_state;
  lay.res   = v.max_res;
  lay.jac   = v.max_jac;
  lay.group = detail::genericGroup(v.max_res);
  size_t         smem    = 0;
  const auto     kernel  = detail::genericTimeKernel<Op>;
  const unsigned threads = detail::prepareLaunch(kernel, lay, &smem);
  const unsigned per_blk = detail::kGenericWarps * (32 / lay.group);
  const unsigned blocks  = (static_cast<unsigned>(map.numElems()) + per_blk - 1) / per_blk;
  kernel<<<blocks, threads, smem, s>>>(op, step, num_hist, wrt, v, hist.data(), nxt.data(),
                                       res.data(), jac.vals, lay, v.max_state);
  detail::cudaCheckApi(cudaGetLastError(), "generic time assembly launch");
}

/** assembleResidual(op, step, num_hist, map, hist, nxt, res, ctx)
 * (femx/assembly/CudaAssembly.hpp:420-472). */
template <class Op>
void assembleResidual(const Op& op, Index step, Index num_hist, const DeviceAssemblyMap& map,
                      DeviceConstVectorView hist, DeviceConstVectorView nxt,
                      DeviceVectorView res, CudaContext& ctx)
{
  DeviceCsrMatrix none{map.pattern(), nullptr};
  assemble(op, step, num_hist, VariableBlock::next(), map, hist, nxt, res, none, ctx);
}

} // namespace gbfem
