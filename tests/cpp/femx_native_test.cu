// femx_native_test.cu — builds gbfem's femx-native adapter (femx_native.cuh)
// against femx's own headers and library, the way a femx user would: femx's
// Mesh, makeGeometry and makeAssemblyMap produce the inputs, the adapter's
// Residual / TimeResidual subclasses are handed to code written against
// femx's interfaces only (femx::state::Residual<CudaCsrBackend>,
// TimeResidual<CudaCsrBackend>), and femx's assemble signature is called
// with femx's device types.
//
// Build (tests/test_femx_native.py): nvcc ... -I<femx tree> -Iinclude
// femx_native_test.cu <femx host library> -lgbfem. Without a CUDA device
// femx's CudaContext cannot be created; the program then prints "SKIP" after
// the host-side steps and exits 0.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <utility>

#include <femx/fem/Mesh.hpp>

#include "gbfem/femx_native.cuh"

using femx::Array;
using femx::Index;
using femx::Real;

namespace
{

// structured n x n triangles on the unit square (each square split in two)
femx::fem::Mesh squareMesh(Index n, Array<Array<Index>>& elems)
{
  femx::fem::Mesh mesh(2);
  for (Index j = 0; j <= n; ++j)
  {
    for (Index i = 0; i <= n; ++i)
    {
      mesh.addNode({Real(i) / n, Real(j) / n, 0.0});
    }
  }
  for (Index j = 0; j < n; ++j)
  {
    for (Index i = 0; i < n; ++i)
    {
      const Index a = j * (n + 1) + i, b = a + 1, c = a + n + 1, d = c + 1;
      for (const Array<Index>& t : {Array<Index>{a, b, d}, Array<Index>{a, d, c}})
      {
        mesh.addElem(t);
        elems.push_back(t);
      }
    }
  }
  return mesh;
}

// Taylor-Hood: the same triangles with edge-midpoint nodes (six-node
// elements: vertices, then midpoints of edges 01, 12, 20) and MixedFESpace
// DOFs (velocity 2 node + comp, then pressure on the vertices).
femx::fem::Mesh p2Mesh(const femx::fem::Mesh& p1mesh, const Array<Array<Index>>& tris,
                       Array<Array<Index>>& dofs, Index& num_dofs)
{
  femx::fem::Mesh mesh(2);
  const Index     nv = p1mesh.numNodes();
  for (Index i = 0; i < nv; ++i)
  {
    mesh.addNode(p1mesh.node(i));
  }
  std::map<std::pair<Index, Index>, Index> mid;
  Array<Array<Index>>                      six;
  for (const auto& t : tris)
  {
    Array<Index> e{t[0], t[1], t[2]};
    for (Index k = 0; k < 3; ++k)
    {
      const Index a = t[k], b = t[(k + 1) % 3];
      const auto  key = std::make_pair(std::min(a, b), std::max(a, b));
      auto        it  = mid.find(key);
      if (it == mid.end())
      {
        const auto& pa = p1mesh.node(a);
        const auto& pb = p1mesh.node(b);
        mesh.addNode({0.5 * (pa[0] + pb[0]), 0.5 * (pa[1] + pb[1]), 0.0});
        it = mid.emplace(key, mesh.numNodes() - 1).first;
      }
      e.push_back(it->second);
    }
    mesh.addElem(e);
    six.push_back(e);
  }
  const Index np2 = mesh.numNodes();
  for (const auto& e : six)
  {
    Array<Index> d;
    for (Index k = 0; k < 6; ++k)
    {
      d.push_back(2 * e[k]);
      d.push_back(2 * e[k] + 1);
    }
    for (Index k = 0; k < 3; ++k)
    {
      d.push_back(2 * np2 + e[k]);
    }
    dofs.push_back(d);
  }
  num_dofs = 2 * np2 + nv;
  return mesh;
}

// Code written against femx's interfaces only: one Newton-style evaluation
// of a stationary residual (LinearStateSolver's sequence,
// femx/state/StateSolver.hpp:90-108) and its parameter VJP.
template <class Backend>
void stationaryPass(const femx::state::Residual<Backend>& r, femx::CudaContext& ctx)
{
  const auto            d = r.dims();
  femx::DeviceVector    u(d.num_states), m(d.num_param), res(d.num_res), g(0);
  femx::DeviceCsrMatrix jac(r.pattern());
  r.res(u, m, res, ctx);
  r.assembleStateJac(u, m, jac, ctx);
  r.applyParamJacT(u, m, res, g, ctx);
  ctx.sync();
  if (g.size() != d.num_param)
  {
    throw std::runtime_error("applyParamJacT output size");
  }
}

// One time step through femx's TimeResidual interface (TimeIntegrator's
// sequence, femx/state/TimeIntegrator.hpp:271-298) and the history VJPs
// TimeReducedFunctional::solveAdj asks for.
template <class Backend>
void timePass(const femx::state::TimeResidual<Backend>& r, femx::CudaContext& ctx)
{
  const auto            d = r.dims();
  femx::DeviceVector    hist(d.num_hist * d.num_states), nxt(d.num_states), res(d.num_res),
      out(0);
  femx::DeviceCsrMatrix jac(r.pattern());
  femx::state::TimeContext<femx::MemorySpace::Device> t;
  t.step = 1;
  t.nxt  = {nxt.data(), nxt.size()};
  t.hist = {hist.data(), d.num_hist, d.num_states};
  r.assembleNext(t, res, jac, ctx);
  r.res(t, res, ctx);
  for (Index lag = 0; lag < d.num_hist; ++lag)
  {
    r.applyJacT(t, femx::state::VariableBlock::hist(lag), {res.data(), res.size()}, out, ctx);
  }
  r.applyJacT(t, femx::state::VariableBlock::Param, {res.data(), res.size()}, out, ctx);
  ctx.sync();
}

// femx's assemble signature (CudaAssembly.hpp:319-326) over femx's device
// types, for both operator tags: the overloads must resolve and link.
using P1Assemble = void (*)(const gbfem::KappaPoissonP1&, const femx::fem::DeviceGeometry&,
                            const femx::assembly::DeviceAssemblyMap&, const femx::DeviceVector&,
                            femx::DeviceVector&, femx::DeviceCsrMatrix&, femx::CudaContext&);
using ThAssemble = void (*)(const gbfem::TaylorHoodNS&, const femx::fem::DeviceGeometry&,
                            const femx::assembly::DeviceAssemblyMap&, const femx::DeviceVector&,
                            femx::DeviceVector&, femx::DeviceCsrMatrix&, femx::CudaContext&);
volatile P1Assemble p1_assemble = &gbfem::native::assemble;
volatile ThAssemble th_assemble = &gbfem::native::assemble;

} // namespace

int main()
{
  // host side: femx builds the mesh, geometry and maps
  Array<Array<Index>> p1;
  const auto          mesh = squareMesh(4, p1);
  const auto          geom = femx::fem::makeGeometry(mesh);
  const Index         n    = mesh.numNodes();
  const auto          map  = femx::assembly::makeAssemblyMap(n, n, p1, p1);
  Array<Index>        bc;
  femx::HostVector    g;
  for (Index i = 0; i < n; ++i)
  {
    const Real x = mesh.node(i)[0], y = mesh.node(i)[1];
    if (x == 0.0 || y == 0.0 || x == 1.0 || y == 1.0)
    {
      bc.push_back(i);
      g.push_back(x - y);
    }
  }
  // GLS Navier-Stokes on the same triangles: femx's mixed layout, velocity
  // (node, comp) then pressure, 9 DOFs per element
  Array<Array<Index>> ns;
  for (const auto& t : p1)
  {
    Array<Index> e;
    for (Index k = 0; k < 3; ++k)
    {
      e.push_back(2 * t[k]);
      e.push_back(2 * t[k] + 1);
    }
    for (Index k = 0; k < 3; ++k)
    {
      e.push_back(2 * n + t[k]);
    }
    ns.push_back(e);
  }
  const auto ns_map = femx::assembly::makeAssemblyMap(3 * n, 3 * n, ns, ns);
  Array<Array<Index>> th;
  Index               nth  = 0;
  const auto          m2   = p2Mesh(mesh, p1, th, nth);
  const auto          geo2 = femx::fem::makeGeometry(m2);
  const auto          th_map = femx::assembly::makeAssemblyMap(nth, nth, th, th);
  Array<Index>        th_bc{0, 1, 2 * m2.numNodes()}; // two velocity DOFs and a pressure pin
  femx::HostVector    th_g(3, 0.0);
  std::printf("host: %d nodes, %d elements, P1 nnz %d, NS nnz %d, Taylor-Hood nnz %d\n", n,
              geom.numElems(), map.pattern().nnz(), ns_map.pattern().nnz(),
              th_map.pattern().nnz());

  try
  {
    femx::CudaContext ctx;
    femx::HostVector  f(n, 1.0);
    gbfem::native::KappaPoissonResidual poisson(geom, map, f, bc, g, ctx);
    stationaryPass(poisson, ctx);
    gbfem::native::TaylorHoodResidual taylor_hood(geo2, th_map, 1e-3, th_bc, th_g, ctx);
    stationaryPass(taylor_hood, ctx);
    gbfem::native::NavierTimeResidual navier(4, geom, ns_map, 1.0, 0.01, 0.1, ctx);
    timePass(navier, ctx);
    std::printf("device passes done\n");
  }
  catch (const std::exception& e)
  {
    std::printf("SKIP: %s\n", e.what());
    return 0;
  }
  return 0;
}
