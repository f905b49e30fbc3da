// GPU test program for the C++ layer (include/gbfem/femx_api.hpp) and the
// header-only user-operator assembly (include/gbfem/generic_assembly.cuh).
//
// Part 1 reproduces femx's own known-answer tests of the generic assembly
// loop with row operators of the same definition
// (tests/unit/backend/runBackendAssemblyTests.cpp):
//   cpuAssemblyUsesRuntimeMapAndSharedGraph      (:190-226)
//   cpuAssemblySupportsRectangularLocalLayouts   (:228-256)
//   cpuTimeAssemblyHandlesHistoryBlocks          (:259-304)
// and prints "KAT <name> PASS|FAIL".
//
// Part 2 (when a data directory is given) assembles the P1 stiffness of a
// mesh written by the Python test through (a) a user operator restating
// femx's PoissonComponents::evalRow (examples/poisson/PoissonComponents.hpp:
// 35-64) and (b) the KappaPoissonP1 tag with kappa = 1, then applies the
// C++ BoundaryMap calls and a matvec; raw outputs go back to the directory
// for comparison with the CPU oracle.
//
// Part 3 ("navier" mode) runs femx's NS time operator through the NavierGLS
// tag (next-state block, a history block, the history VJP) on a golden case.
//
// Usage: generic_assembly_test [dir num_nodes num_elems num_bcs]
//        generic_assembly_test navier dir num_nodes num_elems
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gbfem/generic_assembly.cuh"

using gbfem::Index;
using gbfem::Real;

namespace
{
int g_fail = 0;

void cuda(cudaError_t e, const char* what)
{
  if (e != cudaSuccess)
  {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
}

template <class T>
struct Dev
{
  T*    p{nullptr};
  Index n{0};
  explicit Dev(const std::vector<T>& h) : n(static_cast<Index>(h.size()))
  {
    cuda(cudaMalloc(&p, sizeof(T) * (h.empty() ? 1 : h.size())), "malloc");
    if (!h.empty())
    {
      cuda(cudaMemcpy(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice), "h2d");
    }
  }
  explicit Dev(Index count) : n(count)
  {
    cuda(cudaMalloc(&p, sizeof(T) * (count > 0 ? count : 1)), "malloc");
    cuda(cudaMemset(p, 0, sizeof(T) * (count > 0 ? count : 1)), "memset");
  }
  ~Dev() { cudaFree(p); }
  Dev(const Dev&)            = delete;
  Dev& operator=(const Dev&) = delete;
  std::vector<T> host() const
  {
    std::vector<T> h(n);
    cuda(cudaMemcpy(h.data(), p, sizeof(T) * n, cudaMemcpyDeviceToHost), "d2h");
    return h;
  }
  gbfem::DeviceView<T>       view() { return {p, n}; }
  gbfem::DeviceView<const T> cview() const { return {p, n}; }
};

gbfem::DeviceAssemblyMap mapFrom(Index num_res, Index num_states,
                                 const std::vector<std::vector<Index>>& res,
                                 const std::vector<std::vector<Index>>& st,
                                 gbfem::CudaContext& ctx)
{
  std::vector<Index> ro{0}, rd, so{0}, sd;
  for (const auto& r : res)
  {
    rd.insert(rd.end(), r.begin(), r.end());
    ro.push_back(static_cast<Index>(rd.size()));
  }
  for (const auto& s : st)
  {
    sd.insert(sd.end(), s.begin(), s.end());
    so.push_back(static_cast<Index>(sd.size()));
  }
  Dev<Index> dro(ro), drd(rd), dso(so), dsd(sd);
  auto       m = gbfem::makeAssemblyMap(num_res, num_states, static_cast<Index>(res.size()),
                                        dro.p, drd.p, dso.p, dsd.p, ctx);
  cuda(cudaDeviceSynchronize(), "map");
  return m;
}

Real csrVal(const std::vector<Index>& rp, const std::vector<Index>& ci,
            const std::vector<Real>& v, Index row, Index col)
{
  for (Index k = rp[row]; k < rp[row + 1]; ++k)
  {
    if (ci[k] == col)
    {
      return v[k];
    }
  }
  return 0.0;
}

template <class T>
std::vector<T> hostOf(const T* d, Index n)
{
  std::vector<T> h(n);
  cuda(cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost), "d2h");
  return h;
}

void report(const char* name, bool ok)
{
  std::printf("KAT %s %s\n", name, ok ? "PASS" : "FAIL");
  g_fail += ok ? 0 : 1;
}

bool near(Real a, Real b) { return std::fabs(a - b) <= 1e-12 * (1.0 + std::fabs(b)); }

// res = state[row] + (ie + 1) + coords[0]; jac = 2 on the diagonal, 1 off it
struct AffineRows
{
  __device__ void evalRow(const gbfem::ElementView& in, Index row, Real& res,
                          gbfem::Span<Real> jac) const
  {
    res = in.state[row] + static_cast<Real>(in.ie + 1) + in.coords[0];
    for (Index col = 0; col < jac.size(); ++col)
    {
      jac[col] = row == col ? 2.0 : 1.0;
    }
  }
};

// res = (row + 1) + sum(state); jac[col] = 10 (row + 1) + (col + 1)
struct RectangularRows
{
  __device__ void evalRow(const gbfem::ElementView& in, Index row, Real& res,
                          gbfem::Span<Real> jac) const
  {
    res = static_cast<Real>(row + 1);
    for (Index col = 0; col < in.state.size(); ++col)
    {
      res += in.state[col];
      jac[col] = 10.0 * static_cast<Real>(row + 1) + static_cast<Real>(col + 1);
    }
  }
};

// res = nxt - 2 h0 + 0.5 h1 + (ie + step); jac = diag of the chosen block
struct TimeRows
{
  __device__ void evalRow(const gbfem::TimeElementView& e, gbfem::VariableBlock wrt, Index row,
                          Real& res, gbfem::Span<Real> jac) const
  {
    res = e.nxt[row] - 2.0 * e.histState(0)[row] + 0.5 * e.histState(1)[row]
          + static_cast<Real>(e.ie + e.step);
    const Real d = wrt.isNextState() ? 1.0 : (wrt.historyLag() == 0 ? -2.0 : 0.5);
    for (Index col = 0; col < jac.size(); ++col)
    {
      jac[col] = row == col ? d : 0.0;
    }
  }
};

// P1 Laplacian row: K_ij = |T| grad N_i . grad N_j, res_i = sum_j K_ij u_j.
struct PoissonRows
{
  __device__ void evalRow(const gbfem::ElementView& in, Index row, Real& res,
                          gbfem::Span<Real> jac) const
  {
    const Real x0 = in.coords[0], y0 = in.coords[1];
    const Real x1 = in.coords[2], y1 = in.coords[3];
    const Real x2 = in.coords[4], y2 = in.coords[5];
    const Real det = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
    // grad N_k = (y_{k+1} - y_{k+2}, x_{k+2} - x_{k+1}) / det
    const Real gx[3] = {(y1 - y2) / det, (y2 - y0) / det, (y0 - y1) / det};
    const Real gy[3] = {(x2 - x1) / det, (x0 - x2) / det, (x1 - x0) / det};
    const Real area  = 0.5 * std::fabs(det);
    res              = 0.0;
    for (Index j = 0; j < 3; ++j)
    {
      jac[j] = area * (gx[row] * gx[j] + gy[row] * gy[j]);
      res += jac[j] * in.state[j];
    }
  }
};

void knownAnswers(gbfem::CudaContext& ctx)
{
  // 2 x 1 structured quad mesh on the unit square, element nodes
  // (n0, n1, n2, n3) counter-clockwise, scalar DOF = node.
  const std::vector<Real>  xy{0.0, 0.0, 0.5, 0.0, 1.0, 0.0, 0.0, 1.0, 0.5, 1.0, 1.0, 1.0};
  const std::vector<Index> conn{0, 1, 4, 3, 1, 2, 5, 4};
  Dev<Real>                dxy(xy);
  Dev<Index>               dconn(conn);
  {
    auto map = mapFrom(6, 6, {{0, 1, 4, 3}, {1, 2, 5, 4}}, {{0, 1, 4, 3}, {1, 2, 5, 4}}, ctx);
    const gbfem::DeviceGeometry geom{6, 2, 4, dxy.p, dconn.p, 2};
    Dev<Real>                   st(std::vector<Real>{1, 2, 3, 4, 5, 6});
    Dev<Real>                   res(6);
    Dev<Real>                   vals(map.pattern().nnz);
    gbfem::DeviceCsrMatrix      jac{map.pattern(), vals.p};
    gbfem::assemble(AffineRows{}, geom, map, st.cview(), res.view(), jac, ctx);
    cuda(cudaDeviceSynchronize(), "affine");
    const auto r  = res.host();
    const auto v  = vals.host();
    const auto rp = hostOf(map.pattern().row_ptr, 7);
    const auto ci = hostOf(map.pattern().col_ind, map.pattern().nnz);
    const Real want[6] = {2.0, 7.5, 5.5, 5.0, 13.5, 8.5};
    bool       ok      = map.pattern().nnz == 28;
    for (int i = 0; i < 6; ++i)
    {
      ok = ok && near(r[i], want[i]);
    }
    ok = ok && near(csrVal(rp, ci, v, 0, 0), 2.0) && near(csrVal(rp, ci, v, 1, 1), 4.0)
         && near(csrVal(rp, ci, v, 4, 4), 4.0) && near(csrVal(rp, ci, v, 1, 4), 2.0)
         && near(csrVal(rp, ci, v, 0, 2), 0.0);
    report("cpuAssemblyUsesRuntimeMapAndSharedGraph", ok);
  }
  {
    auto map = mapFrom(2, 2, {{0, 1}, {1}}, {{0}, {0, 1}}, ctx);
    const gbfem::DeviceGeometry geom{6, 2, 4, dxy.p, dconn.p, 2};
    Dev<Real>                   st(std::vector<Real>{2.0, 3.0});
    Dev<Real>                   res(2);
    Dev<Real>                   vals(map.pattern().nnz);
    gbfem::DeviceCsrMatrix      jac{map.pattern(), vals.p};
    gbfem::assemble(RectangularRows{}, geom, map, st.cview(), res.view(), jac, ctx);
    cuda(cudaDeviceSynchronize(), "rectangular");
    const auto r  = res.host();
    const auto v  = vals.host();
    const auto rp = hostOf(map.pattern().row_ptr, 3);
    const auto ci = hostOf(map.pattern().col_ind, map.pattern().nnz);
    const bool ok = near(r[0], 3.0) && near(r[1], 10.0) && near(csrVal(rp, ci, v, 0, 0), 11.0)
                    && near(csrVal(rp, ci, v, 1, 0), 32.0) && near(csrVal(rp, ci, v, 1, 1), 12.0);
    report("cpuAssemblySupportsRectangularLocalLayouts", ok);
  }
  {
    auto map = mapFrom(3, 3, {{0, 1}, {1, 2}}, {{0, 1}, {1, 2}}, ctx);
    Dev<Real>              hist(std::vector<Real>{1, 2, 3, 4, 5, 6});
    Dev<Real>              nxt(std::vector<Real>{7, 8, 9});
    Dev<Real>              res(3);
    Dev<Real>              vals(map.pattern().nnz);
    gbfem::DeviceCsrMatrix jac{map.pattern(), vals.p};
    const auto rp = hostOf(map.pattern().row_ptr, 4);
    const auto ci = hostOf(map.pattern().col_ind, map.pattern().nnz);
    gbfem::assemble(TimeRows{}, 3, 2, gbfem::VariableBlock::next(), map, hist.cview(),
                    nxt.cview(), res.view(), jac, ctx);
    cuda(cudaDeviceSynchronize(), "time next");
    auto r  = res.host();
    auto v  = vals.host();
    bool ok = near(r[0], 10.0) && near(r[1], 20.0) && near(r[2], 10.0)
              && near(csrVal(rp, ci, v, 0, 0), 1.0) && near(csrVal(rp, ci, v, 1, 1), 2.0)
              && near(csrVal(rp, ci, v, 2, 2), 1.0);
    gbfem::assemble(TimeRows{}, 3, 2, gbfem::VariableBlock::hist(0), map, hist.cview(),
                    nxt.cview(), res.view(), jac, ctx);
    cuda(cudaDeviceSynchronize(), "time hist");
    v  = vals.host();
    ok = ok && near(csrVal(rp, ci, v, 0, 0), -2.0) && near(csrVal(rp, ci, v, 1, 1), -4.0)
         && near(csrVal(rp, ci, v, 2, 2), -2.0);
    // the residual-only entry point gives the same residual
    gbfem::assembleResidual(TimeRows{}, 3, 2, map, hist.cview(), nxt.cview(), res.view(), ctx);
    cuda(cudaDeviceSynchronize(), "time residual");
    r  = res.host();
    ok = ok && near(r[0], 10.0) && near(r[1], 20.0) && near(r[2], 10.0);
    report("cpuTimeAssemblyHandlesHistoryBlocks", ok);
  }
  {
    // femx's input checks: a history lag outside [0, num_hist) is rejected
    auto map = mapFrom(3, 3, {{0, 1}, {1, 2}}, {{0, 1}, {1, 2}}, ctx);
    Dev<Real>              hist(6), nxt(3), res(3), vals(map.pattern().nnz);
    gbfem::DeviceCsrMatrix jac{map.pattern(), vals.p};
    bool                   threw = false;
    try
    {
      gbfem::assemble(TimeRows{}, 0, 2, gbfem::VariableBlock::hist(2), map, hist.cview(),
                      nxt.cview(), res.view(), jac, ctx);
    }
    catch (const std::runtime_error& e)
    {
      threw = std::string(e.what()) == "Time assembly variable block is invalid";
    }
    report("timeAssemblyRejectsInvalidBlock", threw);
  }
}

template <class T>
std::vector<T> readFile(const std::string& path, size_t n)
{
  std::vector<T> v(n);
  FILE*          f = std::fopen(path.c_str(), "rb");
  if (f == nullptr || std::fread(v.data(), sizeof(T), n, f) != n)
  {
    std::fprintf(stderr, "cannot read %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <class T>
void writeFile(const std::string& path, const std::vector<T>& v)
{
  FILE* f = std::fopen(path.c_str(), "wb");
  if (f == nullptr || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size())
  {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

void poissonThroughTheCppLayer(const std::string& dir, Index nn, Index ne, Index nb,
                               gbfem::CudaContext& ctx)
{
  const auto         xy    = readFile<Real>(dir + "/coords.f64", 2 * static_cast<size_t>(nn));
  const auto         conn  = readFile<Index>(dir + "/conn.i32", 3 * static_cast<size_t>(ne));
  const auto         u     = readFile<Real>(dir + "/state.f64", nn);
  const auto         bdofs = readFile<Index>(dir + "/bdofs.i32", nb);
  const auto         g     = readFile<Real>(dir + "/g.f64", nb);
  std::vector<Index> offs(ne + 1);
  for (Index e = 0; e <= ne; ++e)
  {
    offs[e] = 3 * e;
  }
  Dev<Real>  dxy(xy), du(u), dg(g), ones(std::vector<Real>(ne, 1.0));
  Dev<Index> dconn(conn), doffs(offs), dbd(bdofs);
  auto map = gbfem::makeAssemblyMap(nn, nn, ne, doffs.p, dconn.p, doffs.p, dconn.p, ctx);
  const gbfem::DeviceGeometry geom{nn, ne, 3, dxy.p, dconn.p, 2};
  const Index                 nnz = map.pattern().nnz;

  Dev<Real>              res_g(nn), vals_g(nnz), res_t(nn), vals_t(nnz);
  gbfem::DeviceCsrMatrix jac_g{map.pattern(), vals_g.p}, jac_t{map.pattern(), vals_t.p};
  gbfem::assemble(PoissonRows{}, geom, map, du.cview(), res_g.view(), jac_g, ctx);
  gbfem::assemble(gbfem::KappaPoissonP1{ones.p, nullptr, gbfem::Precision::FP64}, geom, map,
                  du.cview(), res_t.view(), jac_t, ctx);

  // BoundaryMap calls on the tag path's matrix
  auto      bc = gbfem::makeBoundaryMap(dbd.cview(), map.pattern(), ctx);
  Dev<Real> rows_vals(nnz), res_bc(nn), rhs(nn), y(nn);
  cuda(cudaMemcpy(rows_vals.p, vals_t.p, sizeof(Real) * nnz, cudaMemcpyDeviceToDevice), "copy");
  cuda(cudaMemcpy(res_bc.p, res_t.p, sizeof(Real) * nn, cudaMemcpyDeviceToDevice), "copy");
  gbfem::DeviceCsrMatrix rows_mat{map.pattern(), rows_vals.p};
  gbfem::replaceRows(bc, rows_mat, 1.0, ctx);
  gbfem::replaceRes(bc, du.cview(), dg.cview(), res_bc.view(), ctx);
  // forward solve on the tag matrix itself: rhs = -res(u), lifting with g
  {
    const auto r = res_t.host();
    std::vector<Real> mr(nn);
    for (Index i = 0; i < nn; ++i)
    {
      mr[i] = -r[i];
    }
    cuda(cudaMemcpy(rhs.p, mr.data(), sizeof(Real) * nn, cudaMemcpyHostToDevice), "h2d");
  }
  Dev<Real> solve_vals(nnz);
  cuda(cudaMemcpy(solve_vals.p, vals_t.p, sizeof(Real) * nnz, cudaMemcpyDeviceToDevice), "copy");
  gbfem::DeviceCsrMatrix solve_mat{map.pattern(), solve_vals.p};
  gbfem::prepareForwardSolve(bc, solve_mat, rhs.view(), dg.cview(), ctx);
  gbfem::matvec(jac_t, du.cview(), y.view(), 1.0, 0.0, ctx);
  cuda(cudaDeviceSynchronize(), "poisson");

  writeFile(dir + "/res_generic.f64", res_g.host());
  writeFile(dir + "/vals_generic.f64", vals_g.host());
  writeFile(dir + "/res_tag.f64", res_t.host());
  writeFile(dir + "/vals_tag.f64", vals_t.host());
  writeFile(dir + "/rows_vals.f64", rows_vals.host());
  writeFile(dir + "/res_bc.f64", res_bc.host());
  writeFile(dir + "/solve_vals.f64", solve_vals.host());
  writeFile(dir + "/rhs.f64", rhs.host());
  writeFile(dir + "/y.f64", y.host());
  writeFile(dir + "/row_ptr.i32", hostOf(map.pattern().row_ptr, nn + 1));
  writeFile(dir + "/col_ind.i32", hostOf(map.pattern().col_ind, nnz));
  std::printf("POISSON written nnz=%d\n", nnz);
}
// femx's NS time operator through the C++ tag: next-state block, a history
// block (zero) and the history VJP, for one golden case written by the test.
void navierThroughTheCppLayer(const std::string& dir, Index nn, Index ne, gbfem::CudaContext& ctx)
{
  const Index nd     = 3 * nn;
  const auto  xy     = readFile<Real>(dir + "/coords.f64", 2 * static_cast<size_t>(nn));
  const auto  conn   = readFile<Index>(dir + "/conn.i32", 3 * static_cast<size_t>(ne));
  const auto  dofs   = readFile<Index>(dir + "/dofs.i32", 9 * static_cast<size_t>(ne));
  const auto  hist   = readFile<Real>(dir + "/hist.f64", 2 * static_cast<size_t>(nd));
  const auto  nxt    = readFile<Real>(dir + "/nxt.f64", nd);
  const auto  adj    = readFile<Real>(dir + "/adj.f64", nd);
  const auto  prm    = readFile<Real>(dir + "/prm.f64", 4);
  std::vector<Index> offs(ne + 1);
  for (Index e = 0; e <= ne; ++e)
  {
    offs[e] = 9 * e;
  }
  Dev<Real>  dxy(xy), dh(hist), dx(nxt), da(adj);
  Dev<Index> dconn(conn), doffs(offs), ddofs(dofs);
  auto map = gbfem::makeAssemblyMap(nd, nd, ne, doffs.p, ddofs.p, doffs.p, ddofs.p, ctx);
  const gbfem::NavierGLS op{{nn, ne, 3, dxy.p, dconn.p, 2}, prm[0], prm[1], prm[2]};
  const Index            step = static_cast<Index>(prm[3]);
  Dev<Real>              res(nd), vals(map.pattern().nnz), res_h(nd), vals_h(map.pattern().nnz);
  Dev<Real>              out(2 * nd);
  gbfem::DeviceCsrMatrix jac{map.pattern(), vals.p}, jac_h{map.pattern(), vals_h.p};
  gbfem::assemble(op, step, 2, gbfem::VariableBlock::next(), map, dh.cview(), dx.cview(),
                  res.view(), jac, ctx);
  gbfem::assemble(op, step, 2, gbfem::VariableBlock::hist(0), map, dh.cview(), dx.cview(),
                  res_h.view(), jac_h, ctx);
  gbfem::applyHistJacT(op, step, 2, map, dh.cview(), dx.cview(), da.cview(), out.view(), ctx);
  cuda(cudaDeviceSynchronize(), "navier");
  writeFile(dir + "/ns_res.f64", res.host());
  writeFile(dir + "/ns_vals.f64", vals.host());
  writeFile(dir + "/ns_res_hist.f64", res_h.host());
  writeFile(dir + "/ns_vals_hist.f64", vals_h.host());
  writeFile(dir + "/ns_vjp.f64", out.host());
  std::printf("NAVIER written\n");
}
// Times the user-operator path (PoissonRows through generic_assembly.cuh)
// against the KappaPoissonP1 tag (FP64) on a structured nx x nx mesh, both
// with their zero fill, CUDA events on the stream after three warm-ups:
// prints "TIME generic <ms> tag <ms> elements <E>".
void timeGenericAgainstTag(int nx, int reps, gbfem::CudaContext& ctx)
{
  const Index        nn = (nx + 1) * (nx + 1), ne = 2 * nx * nx;
  std::vector<Real>  xy(2 * static_cast<size_t>(nn));
  std::vector<Index> conn(3 * static_cast<size_t>(ne)), offs(ne + 1);
  for (Index j = 0; j <= nx; ++j)
  {
    for (Index i = 0; i <= nx; ++i)
    {
      xy[2 * (j * (nx + 1) + i)]     = static_cast<Real>(i) / nx;
      xy[2 * (j * (nx + 1) + i) + 1] = static_cast<Real>(j) / nx;
    }
  }
  for (Index j = 0; j < nx; ++j)
  {
    for (Index i = 0; i < nx; ++i)
    {
      const Index a = j * (nx + 1) + i, b = a + 1, c = a + nx + 1, d = c + 1;
      const Index e = 2 * (j * nx + i);
      const Index t[6] = {a, b, d, a, d, c};
      for (int k = 0; k < 6; ++k)
      {
        conn[3 * static_cast<size_t>(e) + k] = t[k];
      }
    }
  }
  for (Index e = 0; e <= ne; ++e)
  {
    offs[e] = 3 * e;
  }
  Dev<Real>  dxy(xy), du(std::vector<Real>(nn, 1.0)), ones(std::vector<Real>(ne, 1.0));
  Dev<Index> dconn(conn), doffs(offs);
  auto map = gbfem::makeAssemblyMap(nn, nn, ne, doffs.p, dconn.p, doffs.p, dconn.p, ctx);
  const gbfem::DeviceGeometry geom{nn, ne, 3, dxy.p, dconn.p, 2};
  Dev<Real>              res(nn), vals(map.pattern().nnz);
  gbfem::DeviceCsrMatrix jac{map.pattern(), vals.p};
  const auto             s = static_cast<cudaStream_t>(ctx.stream);
  cudaEvent_t            e0, e1;
  cuda(cudaEventCreate(&e0), "event");
  cuda(cudaEventCreate(&e1), "event");
  float ms[2];
  for (int which = 0; which < 2; ++which)
  {
    auto run = [&] {
      if (which == 0)
      {
        gbfem::assemble(PoissonRows{}, geom, map, du.cview(), res.view(), jac, ctx);
      }
      else
      {
        gbfem::assemble(gbfem::KappaPoissonP1{ones.p, nullptr, gbfem::Precision::FP64}, geom,
                        map, du.cview(), res.view(), jac, ctx);
      }
    };
    for (int w = 0; w < 3; ++w)
    {
      run();
    }
    cuda(cudaEventRecord(e0, s), "event");
    for (int r = 0; r < reps; ++r)
    {
      run();
    }
    cuda(cudaEventRecord(e1, s), "event");
    cuda(cudaEventSynchronize(e1), "event");
    cuda(cudaEventElapsedTime(&ms[which], e0, e1), "event");
    ms[which] /= static_cast<float>(reps);
  }
  std::printf("TIME generic %.6f tag %.6f elements %d\n", ms[0], ms[1], ne);
}
} // namespace

int main(int argc, char** argv)
{
  cudaStream_t s = nullptr;
  cuda(cudaStreamCreate(&s), "stream");
  gbfem::CudaContext ctx{s};
  try
  {
    if (argc == 4 && std::string(argv[1]) == "time")
    {
      timeGenericAgainstTag(std::atoi(argv[2]), std::atoi(argv[3]), ctx);
      cuda(cudaStreamDestroy(s), "stream");
      return 0;
    }
    knownAnswers(ctx);
    if (argc == 5 && std::string(argv[1]) == "navier")
    {
      navierThroughTheCppLayer(argv[2], std::atoi(argv[3]), std::atoi(argv[4]), ctx);
    }
    else if (argc == 5)
    {
      poissonThroughTheCppLayer(argv[1], std::atoi(argv[2]), std::atoi(argv[3]),
                                std::atoi(argv[4]), ctx);
    }
  }
  catch (const std::exception& e)
  {
    std::fprintf(stderr, "exception: %s\n", e.what());
    return 3;
  }
  cuda(cudaStreamDestroy(s), "stream");
  return g_fail == 0 ? 0 : 1;
}
