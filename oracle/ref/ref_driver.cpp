// ref_driver.cpp — runs the femx reference library (built from its own
// sources by oracle/ref/Makefile) on input files and writes its outputs, to
// produce the golden vectors under tests/golden/ (tests/golden/make_golden.py
// drives it). Test infrastructure only; it never ships with the product.
//
// The element operators below are this project's (the reference has no
// kappa-weighted Poisson operator and no Taylor-Hood element). They plug into
// the reference's ElementOperator concept (femx/assembly/Assembly.hpp:138-152)
// so that the reference's own assemble, AssemblyMap, DirichletBC, BoundaryMap,
// MatrixHandler and ReducedFunctional produce the numbers.
//
// kind "navier" runs femx's own equal-order GLS Navier-Stokes time operator
// (femx/model/ns/Components.hpp:397-577) unchanged, with femx's
// makeNavierData on a P1 triangle mesh and femx's mixed-space DOF layout.
//
// kind "gmsh" runs femx's GmshReader on case_dir/mesh.msh.
//
// Usage: ref_driver <kind> <case_dir>, kind in {kat, p1, th, inverse, navier, gmsh}.
// Inputs and outputs are raw little-endian arrays named <name>.bin in
// case_dir; scalar parameters are read from params.txt ("key value" lines).

#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include <femx/assembly/Assembly.hpp>
#include <femx/assembly/AssemblyMap.hpp>
#include <femx/assembly/BoundaryMap.hpp>
#include <femx/fem/DirichletBC.hpp>
#include <femx/fem/DofLayout.hpp>
#include <femx/fem/ElementQuadratureData.hpp>
#include <femx/fem/FESpace.hpp>
#include <femx/fem/GaussQuadrature.hpp>
#include <femx/fem/GmshReader.hpp>
#include <femx/fem/Geometry.hpp>
#include <femx/fem/Mesh.hpp>
#include <femx/fem/elements/LagrangeTriangleP1.hpp>
#include <femx/inverse/Objective.hpp>
#include <femx/inverse/ReducedFunctional.hpp>
#include <femx/linalg/handler/MatrixHandler.hpp>
#include <femx/linalg/native/DenseLinearSolver.hpp>
#include <femx/fem/MixedFESpace.hpp>
#include <femx/model/ns/Components.hpp>
#include <femx/state/Residual.hpp>
#include <femx/state/StateSolver.hpp>

using namespace femx;

namespace
{

std::string g_dir;

template <class T>
std::vector<T> readBin(const std::string& name)
{
  std::ifstream in(g_dir + "/" + name + ".bin", std::ios::binary);
  if (!in)
  {
    throw std::runtime_error("missing input " + name);
  }
  in.seekg(0, std::ios::end);
  const auto bytes = static_cast<std::size_t>(in.tellg());
  in.seekg(0);
  std::vector<T> out(bytes / sizeof(T));
  in.read(reinterpret_cast<char*>(out.data()), std::streamsize(bytes));
  return out;
}

template <class T>
void writeBin(const std::string& name, const T* data, std::size_t n)
{
  std::ofstream out(g_dir + "/" + name + ".bin", std::ios::binary);
  out.write(reinterpret_cast<const char*>(data), std::streamsize(n * sizeof(T)));
}

template <class V>
void writeVec(const std::string& name, const V& v)
{
  writeBin(name, v.data(), static_cast<std::size_t>(v.size()));
}

std::map<std::string, double> readParams()
{
  std::map<std::string, double> p;
  std::ifstream                 in(g_dir + "/params.txt");
  std::string                   key;
  double                        val;
  while (in >> key >> val)
  {
    p[key] = val;
  }
  return p;
}

// kappa-weighted P1 Poisson with a P1-interpolated load, after
// examples/poisson/PoissonComponents.hpp:35-64.
struct KappaPoissonP1
{
  fem::ElementQuadratureDataView<MemorySpace::Host> data;
  fem::GeometryView<MemorySpace::Host>              geom;
  const Real*                                       kappa{nullptr};
  const Real*                                       f{nullptr};

  void evalRow(const assembly::ElementView<MemorySpace::Host>& e,
               Index                                           row,
               Real&                                           res,
               HostVectorView                                  jac) const
  {
    res = 0.0;
    for (Index c = 0; c < jac.size(); ++c)
    {
      jac[c] = 0.0;
    }
    for (Index iq = 0; iq < data.numQuadraturePoints(); ++iq)
    {
      for (Index c = 0; c < jac.size(); ++c)
      {
        Real dot = 0.0;
        for (Index d = 0; d < data.dim(); ++d)
        {
          dot += data.dNdx(e.ie, iq, row, d) * data.dNdx(e.ie, iq, c, d);
        }
        jac[c] += dot * data.JxW(e.ie, iq);
      }
    }
    for (Index c = 0; c < jac.size(); ++c)
    {
      jac[c] *= kappa[e.ie];
      res += jac[c] * e.state[c];
    }
    if (f != nullptr)
    {
      for (Index iq = 0; iq < data.numQuadraturePoints(); ++iq)
      {
        Real fq = 0.0;
        for (Index n = 0; n < data.numShapes(); ++n)
        {
          fq += f[geom.elemNode(e.ie, n)] * data.N(iq, n);
        }
        res -= fq * data.N(iq, row) * data.JxW(e.ie, iq);
      }
    }
  }
};

// Taylor-Hood P2/P1 steady Navier-Stokes row operator (Galerkin, Newton).
struct TaylorHoodNS
{
  Real nu{1.0};

  static void p2(Real r, Real s, Real* N, Real* dN)
  {
    const Real l0 = 1.0 - r - s, l1 = r, l2 = s;
    const Real g0[2] = {-1.0, -1.0}, g1[2] = {1.0, 0.0}, g2[2] = {0.0, 1.0};
    N[0] = l0 * (2.0 * l0 - 1.0);
    N[1] = l1 * (2.0 * l1 - 1.0);
    N[2] = l2 * (2.0 * l2 - 1.0);
    N[3] = 4.0 * l0 * l1;
    N[4] = 4.0 * l1 * l2;
    N[5] = 4.0 * l2 * l0;
    for (int d = 0; d < 2; ++d)
    {
      dN[0 * 2 + d] = (4.0 * l0 - 1.0) * g0[d];
      dN[1 * 2 + d] = (4.0 * l1 - 1.0) * g1[d];
      dN[2 * 2 + d] = (4.0 * l2 - 1.0) * g2[d];
      dN[3 * 2 + d] = 4.0 * (l1 * g0[d] + l0 * g1[d]);
      dN[4 * 2 + d] = 4.0 * (l2 * g1[d] + l1 * g2[d]);
      dN[5 * 2 + d] = 4.0 * (l0 * g2[d] + l2 * g0[d]);
    }
  }

  void evalRow(const assembly::ElementView<MemorySpace::Host>& e,
               Index                                           row,
               Real&                                           res,
               HostVectorView                                  jac) const
  {
    const Real a1 = 0.445948490915964886, w1 = 0.223381589678011466 * 0.5;
    const Real a2 = 0.091576213509770743, w2 = 0.109951743655321868 * 0.5;
    const Real qr[6][3] = {{a1, a1, w1},
                           {1.0 - 2.0 * a1, a1, w1},
                           {a1, 1.0 - 2.0 * a1, w1},
                           {a2, a2, w2},
                           {1.0 - 2.0 * a2, a2, w2},
                           {a2, 1.0 - 2.0 * a2, w2}};
    const Real dP1[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
    Real       J[4]      = {0.0, 0.0, 0.0, 0.0};
    for (int in = 0; in < 3; ++in)
    {
      for (int a = 0; a < 2; ++a)
      {
        for (int b = 0; b < 2; ++b)
        {
          J[a * 2 + b] += e.coords[in * 2 + a] * dP1[in][b];
        }
      }
    }
    const Real det = J[0] * J[3] - J[1] * J[2];
    if (std::abs(det) < 1.0e-30)
    {
      throw std::runtime_error("Singular 2D Jacobian.");
    }
    const Real inv     = 1.0 / det;
    const Real invJ[4] = {J[3] * inv, -J[1] * inv, -J[2] * inv, J[0] * inv};
    const Real adet    = std::abs(det);
    const auto& st     = e.state;

    res = 0.0;
    for (Index c = 0; c < jac.size(); ++c)
    {
      jac[c] = 0.0;
    }
    for (int iq = 0; iq < 6; ++iq)
    {
      Real N[6], dNr[12], dN[12], P[3], dP[6];
      p2(qr[iq][0], qr[iq][1], N, dNr);
      P[0] = 1.0 - qr[iq][0] - qr[iq][1];
      P[1] = qr[iq][0];
      P[2] = qr[iq][1];
      for (int i = 0; i < 6; ++i)
      {
        for (int a = 0; a < 2; ++a)
        {
          Real v = 0.0;
          for (int b = 0; b < 2; ++b)
          {
            v += dNr[i * 2 + b] * invJ[b * 2 + a];
          }
          dN[i * 2 + a] = v;
        }
      }
      for (int i = 0; i < 3; ++i)
      {
        for (int a = 0; a < 2; ++a)
        {
          Real v = 0.0;
          for (int b = 0; b < 2; ++b)
          {
            v += dP1[i][b] * invJ[b * 2 + a];
          }
          dP[i * 2 + a] = v;
        }
      }
      (void)dP;
      const Real jxw  = adet * qr[iq][2];
      Real       u[2] = {0.0, 0.0}, G[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
      Real       p    = 0.0;
      for (int a = 0; a < 6; ++a)
      {
        for (int c = 0; c < 2; ++c)
        {
          u[c] += N[a] * st[2 * a + c];
          for (int d = 0; d < 2; ++d)
          {
            G[c][d] += st[2 * a + c] * dN[a * 2 + d];
          }
        }
      }
      for (int b = 0; b < 3; ++b)
      {
        p += P[b] * st[12 + b];
      }
      if (row < 12)
      {
        const int a = row / 2, c = row % 2;
        Real      r = 0.0;
        for (int d = 0; d < 2; ++d)
        {
          r += nu * G[c][d] * dN[a * 2 + d] + u[d] * G[c][d] * N[a];
        }
        r -= p * dN[a * 2 + c];
        res += r * jxw;
        for (int b = 0; b < 6; ++b)
        {
          Real adv = 0.0, diff = 0.0;
          for (int d = 0; d < 2; ++d)
          {
            adv += u[d] * dN[b * 2 + d];
            diff += dN[b * 2 + d] * dN[a * 2 + d];
          }
          for (int ec = 0; ec < 2; ++ec)
          {
            Real v = N[b] * G[c][ec] * N[a];
            if (ec == c)
            {
              v += nu * diff + adv * N[a];
            }
            jac[2 * b + ec] += v * jxw;
          }
        }
        for (int b = 0; b < 3; ++b)
        {
          jac[12 + b] -= P[b] * dN[a * 2 + c] * jxw;
        }
      }
      else
      {
        const int b = row - 12;
        res -= P[b] * (G[0][0] + G[1][1]) * jxw;
        for (int a = 0; a < 6; ++a)
        {
          for (int ec = 0; ec < 2; ++ec)
          {
            jac[2 * a + ec] -= P[b] * dN[a * 2 + ec] * jxw;
          }
        }
      }
    }
  }
};

fem::Mesh triMesh(const std::vector<double>& coords,
                  const std::vector<int>&    conn,
                  int                        nodes_per_elem)
{
  fem::Mesh  mesh(2);
  const auto n = coords.size() / 2;
  for (std::size_t i = 0; i < n; ++i)
  {
    mesh.addNode({coords[2 * i], coords[2 * i + 1], 0.0});
  }
  for (std::size_t e = 0; e < conn.size() / nodes_per_elem; ++e)
  {
    Array<Index> nids(nodes_per_elem);
    for (int k = 0; k < nodes_per_elem; ++k)
    {
      nids[k] = conn[e * nodes_per_elem + k];
    }
    mesh.addElem(nids);
  }
  return mesh;
}

bool onUnitSquareBoundary(const fem::Mesh::Node& x, Real)
{
  const Real tol = 1.0e-12;
  return std::abs(x[0]) < tol || std::abs(x[0] - 1.0) < tol
         || std::abs(x[1]) < tol || std::abs(x[1] - 1.0) < tol;
}

void writeMap(const assembly::HostAssemblyMap& map)
{
  const auto v = map.view();
  writeVec("row_ptr", map.pattern().rowPtr());
  writeVec("col_ind", map.pattern().colInd());
  writeBin("jac_offsets", v.jac_offsets, std::size_t(map.numElems() + 1));
  writeBin("jac_map", v.jac_map, std::size_t(v.jac_offsets[map.numElems()]));
}

void writeBcMap(const assembly::HostBoundaryMap& bc)
{
  const auto v = bc.view();
  writeBin("bc_rows", v.bc_rows, std::size_t(v.num_bcs));
  writeBin("bc_diag", v.diag_entries, std::size_t(v.num_bcs));
  writeBin("bc_col_offsets", v.col_offsets, std::size_t(v.num_bcs + 1));
  writeBin("bc_col_entries", v.col_entries, std::size_t(v.col_offsets[v.num_bcs]));
  writeBin("bc_col_rows", v.col_rows, std::size_t(v.col_offsets[v.num_bcs]));
  writeBin("bc_mask", v.bc_mask, std::size_t(v.num_rows));
}

// Known-answer cases of the reference's unit tests, run through the library.
void runKat()
{
  {
    const Array<Array<Index>> dofs{{0, 1}, {1, 2}};
    const auto map = assembly::makeAssemblyMap(3, 3, dofs, dofs);
    const auto v   = map.view();
    writeVec("shared_row_ptr", map.pattern().rowPtr());
    writeVec("shared_col_ind", map.pattern().colInd());
    writeBin("shared_jac_map", v.jac_map, 8);
  }
  {
    const Array<Array<Index>> res{{0, 1}, {1}};
    const Array<Array<Index>> st{{0}, {0, 1}};
    const auto map = assembly::makeAssemblyMap(2, 2, res, st);
    const auto v   = map.view();
    writeVec("rect_row_ptr", map.pattern().rowPtr());
    writeVec("rect_col_ind", map.pattern().colInd());
    writeBin("rect_jac_map", v.jac_map, 4);
  }
  const HostCsrPattern dense{3, 3, HostIndexVector{0, 3, 6, 9},
                             HostIndexVector{0, 1, 2, 0, 1, 2, 0, 1, 2}};
  auto setVals = [](HostCsrMatrix& m) {
    m.vals() = {4.0, 1.0, 2.0, 3.0, 5.0, 6.0, 7.0, 8.0, 9.0};
  };
  for (int which = 0; which < 2; ++which)
  {
    const Array<Index> bcs = which == 0 ? Array<Index>{1} : Array<Index>{0, 2};
    const HostVector   g   = which == 0 ? HostVector{2.0} : HostVector{2.0, -1.0};
    const std::string  tag = which == 0 ? "bc1_" : "bc02_";
    const auto         map = assembly::makeBoundaryMap(bcs, dense);
    HostCsrMatrix      a(dense), h(dense), s(dense);
    setVals(a);
    setVals(h);
    setVals(s);
    assembly::replaceRows(map, a, 1.0);
    assembly::replaceRows(map, h, 0.0);
    HostVector res{10.0, 20.0, 30.0};
    assembly::replaceRes(map, HostVector{4.0, 7.0, 9.0}, g, res);
    HostVector rhs{10.0, 20.0, 30.0};
    assembly::prepareForwardSolve(map, s, rhs, g);
    writeVec(tag + "rows1", a.vals());
    writeVec(tag + "rows0", h.vals());
    writeVec(tag + "res", res);
    writeVec(tag + "fwd_vals", s.vals());
    writeVec(tag + "fwd_rhs", rhs);
  }
}

void runP1()
{
  auto       p      = readParams();
  const auto coords = readBin<double>("coords");
  const auto conn   = readBin<int>("conn");
  const auto kappa  = readBin<double>("kappa");
  const auto f      = readBin<double>("f");
  const auto u      = readBin<double>("u");
  const auto x      = readBin<double>("x");
  const auto lam    = readBin<double>("lam");

  fem::Mesh               mesh = triMesh(coords, conn, 3);
  fem::LagrangeTriangleP1 fe;
  fem::FESpace            space(&mesh, &fe);
  space.setup();
  const auto geom = fem::makeGeometry(mesh);
  const auto quad = fem::makeElementQuadratureData(
      space, fem::GaussQuadrature::make(fe.referenceElement(), 2));
  const auto map = assembly::makeAssemblyMap(fem::DofLayout(space));

  fem::DirichletBC bc;
  const Real       gx = p["gx"], gy = p["gy"], g0 = p["g0"];
  bc.addBoundary(space, onUnitSquareBoundary,
                 [=](const fem::Mesh::Node& n, Real) {
                   return g0 + gx * n[0] + gy * n[1];
                 });
  const auto bcmap = assembly::makeBoundaryMap(bc.dofs(), map.pattern());

  const KappaPoissonP1 op{quad.view(), geom.view(), kappa.data(), f.data()};
  HostCsrMatrix        jac(map.pattern());
  HostVector           res;
  HostVector           state(static_cast<Index>(u.size()));
  for (std::size_t i = 0; i < u.size(); ++i)
  {
    state[Index(i)] = u[i];
  }
  CpuContext ctx;
  const auto t0 = std::chrono::steady_clock::now();
  assembly::assemble(op, geom, map, state, res, jac, ctx);
  const auto t1 = std::chrono::steady_clock::now();
  std::printf("assemble_seconds %.6f\n",
              std::chrono::duration<double>(t1 - t0).count());

  writeMap(map);
  writeVec("res", res);
  writeVec("vals", jac.vals());
  writeVec("bc_dofs", bc.dofs());
  writeVec("bc_vals", bc.vals());
  writeBcMap(bcmap);

  // y = J x and y = J^T x through MatrixHandler<Host>.
  linalg::HostMatrixHandler mh(ctx);
  HostVector xv(static_cast<Index>(x.size()));
  for (std::size_t i = 0; i < x.size(); ++i)
  {
    xv[Index(i)] = x[i];
  }
  HostVector y(map.numRes(), 0.0), yt(map.numStates(), 0.0);
  mh.matvec(jac, xv.view(), y.view());
  mh.matvecT(jac, xv.view(), yt.view());
  writeVec("y_matvec", y);
  writeVec("y_matvec_t", yt);

  // replaceRows / replaceRes / prepareForwardSolve on copies.
  HostCsrMatrix rows1(map.pattern());
  rows1.vals() = jac.vals();
  assembly::replaceRows(bcmap, rows1, 1.0);
  writeVec("vals_rows1", rows1.vals());
  HostVector rres = res;
  assembly::replaceRes(bcmap, state, bc.vals(), rres);
  writeVec("res_replaced", rres);
  HostCsrMatrix fwd(map.pattern());
  fwd.vals() = jac.vals();
  HostVector rhs(res.size());
  for (Index i = 0; i < res.size(); ++i)
  {
    rhs[i] = -res[i];
  }
  assembly::prepareForwardSolve(bcmap, fwd, rhs, bc.vals());
  writeVec("vals_fwd", fwd.vals());
  writeVec("rhs_fwd", rhs);

  // Element-wise VJP through the operator's rows (transpose action).
  HostVector g_u(map.numStates(), 0.0), g_m(map.numElems(), 0.0);
  const auto mv = map.view();
  for (Index e = 0; e < map.numElems(); ++e)
  {
    Real st[3], le[3], jr[9], dummy;
    for (int i = 0; i < 3; ++i)
    {
      st[i] = state[mv.stateDof(e, i)];
      le[i] = lam[static_cast<std::size_t>(mv.resDof(e, i))];
    }
    Real crd[6];
    for (int in = 0; in < 3; ++in)
    {
      for (int d = 0; d < 2; ++d)
      {
        crd[in * 2 + d] = geom.view().coord(geom.view().elemNode(e, in), d);
      }
    }
    const assembly::ElementView<MemorySpace::Host> ev{
        e, 2, 3, HostConstVectorView(st, 3), HostConstVectorView(crd, 6)};
    const KappaPoissonP1 op0{quad.view(), geom.view(), kappa.data(), nullptr};
    for (int r = 0; r < 3; ++r)
    {
      op0.evalRow(ev, r, dummy, HostVectorView(jr + 3 * r, 3));
    }
    Real gm = 0.0;
    for (int r = 0; r < 3; ++r)
    {
      Real ku = 0.0;
      for (int c = 0; c < 3; ++c)
      {
        ku += jr[3 * r + c] * st[c];
        g_u[mv.stateDof(e, c)] += jr[3 * r + c] * le[r];
      }
      gm += le[r] * ku;
    }
    g_m[e] = gm;
  }
  writeVec("g_u", g_u);
  writeVec("g_m", g_m);
}

void runTh()
{
  auto       p      = readParams();
  const auto coords = readBin<double>("coords");
  const auto conn6  = readBin<int>("conn6");
  const auto dofs   = readBin<int>("elem_dofs");
  const auto state0 = readBin<double>("state");
  const int  ndofs  = int(p["num_dofs"]);
  const int  ne     = int(conn6.size() / 6);

  fem::Mesh  mesh = triMesh(coords, conn6, 6);
  const auto geom = fem::makeGeometry(mesh);
  Array<Array<Index>> ed(ne);
  for (int e = 0; e < ne; ++e)
  {
    ed[e].resize(15);
    for (int k = 0; k < 15; ++k)
    {
      ed[e][k] = dofs[std::size_t(e) * 15 + k];
    }
  }
  const auto   map = assembly::makeAssemblyMap(ndofs, ndofs, ed, ed);
  TaylorHoodNS op{p["nu"]};
  HostVector   state(ndofs);
  for (int i = 0; i < ndofs; ++i)
  {
    state[i] = state0[std::size_t(i)];
  }
  HostCsrMatrix jac(map.pattern());
  HostVector    res;
  CpuContext    ctx;
  const auto    t0 = std::chrono::steady_clock::now();
  assembly::assemble(op, geom, map, state, res, jac, ctx);
  const auto t1 = std::chrono::steady_clock::now();
  std::printf("assemble_seconds %.6f\n",
              std::chrono::duration<double>(t1 - t0).count());
  writeMap(map);
  writeVec("res", res);
  writeVec("vals", jac.vals());
}

// Poisson inverse problem for femx's own adjoint gradient
// (femx/inverse/ReducedFunctional.hpp:94-117): R(u, m) with kappa = exp(m)
// and Dirichlet rows replaced, misfit J = 0.5 |u - d|^2.
class KappaResidual final : public state::Residual<linalg::HostCsrBackend>
{
public:
  KappaResidual(const fem::HostGeometry&              geom,
                const fem::HostElementQuadratureData& quad,
                const assembly::HostAssemblyMap&      map,
                const assembly::HostBoundaryMap&      bc,
                const HostVector&                     g,
                const std::vector<double>&            f)
    : geom_(geom), quad_(quad), map_(map), bc_(bc), g_(g), f_(f)
  {
  }

  state::Dimensions dims() const override
  {
    return {map_.numStates(), map_.numElems(), map_.numRes()};
  }
  const HostCsrPattern& hostPattern() const override
  {
    return map_.pattern();
  }
  const HostCsrPattern& pattern() const override
  {
    return map_.pattern();
  }

  void res(const HostVector& state, const HostVector& prm, HostVector& out,
           CpuContext& ctx) const override
  {
    HostCsrMatrix jac(map_.pattern());
    assembleAt(state, prm, out, jac, ctx);
    assembly::replaceRes(bc_, state, g_, out);
  }

  void assembleStateJac(const HostVector& state, const HostVector& prm,
                        HostCsrMatrix& out, CpuContext& ctx) const override
  {
    HostVector r;
    assembleAt(state, prm, r, out, ctx);
    assembly::replaceRows(bc_, out, 1.0);
  }

  void applyParamJacT(const HostVector& state, const HostVector& prm,
                      const HostVector& adj, HostVector& out,
                      CpuContext&) const override
  {
    HostVector lam = adj;
    assembly::zeroBoundary(bc_, lam.view());
    std::vector<double> kappa = kappaOf(prm);
    const KappaPoissonP1 op{quad_.view(), geom_.view(), kappa.data(), nullptr};
    const auto           mv = map_.view();
    out.assign(map_.numElems(), 0.0);
    for (Index e = 0; e < map_.numElems(); ++e)
    {
      Real st[3], crd[6], jr[9], dummy;
      for (int i = 0; i < 3; ++i)
      {
        st[i] = state[mv.stateDof(e, i)];
      }
      const assembly::ElementView<MemorySpace::Host> ev{
          e, 2, 3, HostConstVectorView(st, 3), HostConstVectorView(crd, 6)};
      for (int r = 0; r < 3; ++r)
      {
        op.evalRow(ev, r, dummy, HostVectorView(jr + 3 * r, 3));
      }
      Real gm = 0.0;
      for (int r = 0; r < 3; ++r)
      {
        Real ku = 0.0;
        for (int c = 0; c < 3; ++c)
        {
          ku += jr[3 * r + c] * st[c];
        }
        gm += lam[mv.resDof(e, r)] * ku;
      }
      out[e] = gm;
    }
  }

private:
  std::vector<double> kappaOf(const HostVector& prm) const
  {
    std::vector<double> k(static_cast<std::size_t>(prm.size()));
    for (Index e = 0; e < prm.size(); ++e)
    {
      k[std::size_t(e)] = std::exp(prm[e]);
    }
    return k;
  }

  void assembleAt(const HostVector& state, const HostVector& prm,
                  HostVector& r, HostCsrMatrix& jac, CpuContext& ctx) const
  {
    std::vector<double> kappa = kappaOf(prm);
    const KappaPoissonP1 op{quad_.view(), geom_.view(), kappa.data(), f_.data()};
    assembly::assemble(op, geom_, map_, state, r, jac, ctx);
  }

  const fem::HostGeometry&              geom_;
  const fem::HostElementQuadratureData& quad_;
  const assembly::HostAssemblyMap&      map_;
  const assembly::HostBoundaryMap&      bc_;
  const HostVector&                     g_;
  const std::vector<double>&            f_;
};

class Misfit final : public inverse::Objective
{
public:
  Misfit(const std::vector<double>& d, Index np) : d_(d), np_(np) {}
  Index numStates() const override { return Index(d_.size()); }
  Index numParams() const override { return np_; }
  Real  value(const HostVector& u, const HostVector&) const override
  {
    Real v = 0.0;
    for (Index i = 0; i < u.size(); ++i)
    {
      const Real r = u[i] - d_[std::size_t(i)];
      v += 0.5 * r * r;
    }
    return v;
  }
  void stateGrad(const HostVector& u, const HostVector&,
                 HostVector& out) const override
  {
    out.resize(u.size());
    for (Index i = 0; i < u.size(); ++i)
    {
      out[i] = u[i] - d_[std::size_t(i)];
    }
  }
  void paramGrad(const HostVector&, const HostVector&,
                 HostVector& out) const override
  {
    out.assign(np_, 0.0);
  }

private:
  const std::vector<double>& d_;
  Index                      np_;
};

void runInverse()
{
  const auto coords = readBin<double>("coords");
  const auto conn   = readBin<int>("conn");
  const auto m      = readBin<double>("m");
  const auto d      = readBin<double>("d");
  const auto f      = readBin<double>("f");

  fem::Mesh               mesh = triMesh(coords, conn, 3);
  fem::LagrangeTriangleP1 fe;
  fem::FESpace            space(&mesh, &fe);
  space.setup();
  const auto geom = fem::makeGeometry(mesh);
  const auto quad = fem::makeElementQuadratureData(
      space, fem::GaussQuadrature::make(fe.referenceElement(), 2));
  const auto       map = assembly::makeAssemblyMap(fem::DofLayout(space));
  fem::DirichletBC bc;
  bc.addBoundary(space, onUnitSquareBoundary, 0.0);
  const auto bcmap = assembly::makeBoundaryMap(bc.dofs(), map.pattern());

  KappaResidual                                      res(geom, quad, map, bcmap, bc.vals(), f);
  Misfit                                             obj(d, map.numElems());
  HostCsrMatrix                                      fwd_jac(map.pattern());
  HostCsrMatrix                                      adj_jac(map.pattern());
  linalg::DenseLinearSolver                          fwd_solver;
  linalg::DenseLinearSolver                          adj_solver;
  CpuContext                                         ctx;
  state::LinearStateSolver<linalg::HostCsrBackend>   state_solver(res, fwd_jac, fwd_solver, ctx);
  inverse::ReducedFunctional<linalg::HostCsrBackend> reduced(state_solver, adj_jac, adj_solver, obj);

  HostVector prm(map.numElems());
  for (Index e = 0; e < map.numElems(); ++e)
  {
    prm[e] = m[std::size_t(e)];
  }
  HostVector grad;
  const Real val = reduced.valueGrad(prm, grad);
  HostVector u;
  state_solver.solve(prm, u);
  writeBin("value", &val, 1);
  writeVec("grad", grad);
  writeVec("u", u);
}

} // namespace

// femx's NS time step operator on P1 triangles (velocity + pressure, equal
// order; order-2 quadrature as NavierStokesModel.cpp:34). Inputs: coords,
// conn, hist (2 lags x num_dofs, lag-major), nxt; params rho, mu, dt, step.
// Outputs: the mixed-space element DOF tables, the CSR map, res and the
// next-state Jacobian from the reference's time assemble
// (Assembly.hpp:235-303).
void runNavier()
{
  auto       p      = readParams();
  const auto coords = readBin<double>("coords");
  const auto conn   = readBin<int>("conn");
  const auto hist   = readBin<double>("hist");
  const auto nxt    = readBin<double>("nxt");

  fem::Mesh               mesh = triMesh(coords, conn, 3);
  fem::LagrangeTriangleP1 fe;
  fem::FESpace            u_space(&mesh, &fe, 2);
  fem::FESpace            p_space(&mesh, &fe);
  fem::MixedFESpace       space;
  space.addField(u_space);
  space.addField(p_space);
  space.setup();
  u_space.setup();
  const auto map  = assembly::makeAssemblyMap(fem::DofLayout(space));
  const auto data = model::ns::makeNavierData(
      u_space, fem::GaussQuadrature::make(fe.referenceElement(), 2));
  const model::ns::NavierOperator<MemorySpace::Host> op(
      data.view(), model::ns::KernelFluid{p["rho"], p["mu"]}, p["dt"]);

  HostVector hv(static_cast<Index>(hist.size())), nv(static_cast<Index>(nxt.size()));
  for (std::size_t i = 0; i < hist.size(); ++i)
  {
    hv[Index(i)] = hist[i];
  }
  for (std::size_t i = 0; i < nxt.size(); ++i)
  {
    nv[Index(i)] = nxt[i];
  }
  HostCsrMatrix jac(map.pattern());
  HostVector    res;
  CpuContext    ctx;
  const Index   step = static_cast<Index>(p["step"]);
  const auto    t0   = std::chrono::steady_clock::now();
  assembly::assemble(op, step, 2, state::VariableBlock::NextState, map, hv, nv, res, jac, ctx);
  const auto t1 = std::chrono::steady_clock::now();
  std::printf("assemble_seconds %.6f\n", std::chrono::duration<double>(t1 - t0).count());

  const auto v = map.view();
  writeBin("res_offsets", v.res_offsets, std::size_t(map.numElems() + 1));
  writeBin("res_dofs", v.res_dofs, std::size_t(v.res_offsets[map.numElems()]));
  writeBin("state_offsets", v.state_offsets, std::size_t(map.numElems() + 1));
  writeBin("state_dofs", v.state_dofs, std::size_t(v.state_offsets[map.numElems()]));
  writeMap(map);
  writeVec("res", res);
  writeVec("vals", jac.vals());
  const Index nd = space.numDofs();
  writeBin("num_dofs", &nd, 1);
}

// femx's GmshReader on case_dir/mesh.msh: nodes, elements and boundary
// facets with their entity and physical tags, and the physical names.
void runGmsh()
{
  const fem::Mesh     mesh = fem::GmshReader::read(g_dir + "/mesh.msh");
  std::vector<double> xyz;
  for (Index i = 0; i < mesh.numNodes(); ++i)
  {
    for (int d = 0; d < 3; ++d)
    {
      xyz.push_back(mesh.node(i)[d]);
    }
  }
  std::vector<int> conn, etag, ptag, fconn, fetag, fptag;
  for (Index ie = 0; ie < mesh.numElems(); ++ie)
  {
    const auto& el = mesh.elem(ie);
    for (Index k = 0; k < el.numNodes(); ++k)
    {
      conn.push_back(el.nodeIds()[k]);
    }
    etag.push_back(el.entityTag());
    ptag.push_back(el.physicalTag());
  }
  for (const auto& f : mesh.boundaryFacets())
  {
    for (Index k = 0; k < f.nids.size(); ++k)
    {
      fconn.push_back(f.nids[k]);
    }
    fetag.push_back(f.etag);
    fptag.push_back(f.ptag);
  }
  const int dim = static_cast<int>(mesh.dim());
  writeBin("dim", &dim, 1);
  writeBin("coords", xyz.data(), xyz.size());
  writeBin("conn", conn.data(), conn.size());
  writeBin("etag", etag.data(), etag.size());
  writeBin("ptag", ptag.data(), ptag.size());
  writeBin("fconn", fconn.data(), fconn.size());
  writeBin("fetag", fetag.data(), fetag.size());
  writeBin("fptag", fptag.data(), fptag.size());
  std::ofstream names(g_dir + "/names.txt");
  for (const auto& pn : mesh.physicalNames())
  {
    names << pn.first.first << " " << pn.first.second << " " << pn.second << "\n";
  }
}

int main(int argc, char** argv)
{
  if (argc != 3)
  {
    std::cerr << "usage: ref_driver <kat|p1|th|inverse|navier|gmsh> <case_dir>\n";
    return 2;
  }
  const std::string kind = argv[1];
  g_dir                  = argv[2];
  try
  {
    if (kind == "kat")
    {
      runKat();
    }
    else if (kind == "p1")
    {
      runP1();
    }
    else if (kind == "th")
    {
      runTh();
    }
    else if (kind == "inverse")
    {
      runInverse();
    }
    else if (kind == "navier")
    {
      runNavier();
    }
    else if (kind == "gmsh")
    {
      runGmsh();
    }
    else
    {
      std::cerr << "unknown kind " << kind << "\n";
      return 2;
    }
  }
  catch (const std::exception& e)
  {
    std::cerr << "ref_driver failed: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
