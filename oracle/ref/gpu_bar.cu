// gpu_bar.cu — the reference's own CUDA assembly kernel as a measurement bar.
//
// Test and measurement infrastructure, not product code. Compiled by
// oracle/ref/Makefile from the femx sources where they lie (REF), never
// copied:
//   * device pass (-cubin, sm_103a): femx's assembleKernel
//     (femx/assembly/CudaAssembly.hpp:100-169) instantiated for the
//     kappa-weighted P1 Poisson operator below, into oracle/_ref/
//     gpu_bar.cubin. A cubin is GPU code only: it runs on the GPU machine, where
//     femx's sources are absent, through oracle/gpu_bar_launch.cpp.
//   * host pass (-DREFBAR_LAYOUT, run here): prints the byte layout of the
//     kernel's arguments (femx's GeometryView, AssemblyMapView and the
//     operator with its ElementQuadratureDataView), found by filling every
//     field with a distinct sentinel through femx's own constructors and
//     locating the sentinels in the object bytes; the launcher fills the
//     same offsets with real device addresses and sizes.
//
// A second instantiation is femx's own NS time assembly: assembleTimeKernel
// (CudaAssembly.hpp:171-236) with femx's NavierOperator<Device>
// (femx/model/ns/Components.hpp:400-577), the operator of femx's NS model.
//
// The operator follows femx's Poisson example (examples/poisson/
// PoissonComponents.hpp:35-64, quadrature over ElementQuadratureData) with
// the per-element coefficient and the load of the oracle's KappaPoissonP1:
//   jac_rc = kappa_e sum_q dN_r . dN_c JxW_q,  res_r = sum_c jac_rc u_c
//            - sum_q f_h(x_q) N_r(x_q) JxW_q.
#include <femx/assembly/CudaAssembly.hpp>
#include <femx/fem/ElementQuadratureData.hpp>
#include <femx/fem/Geometry.hpp>
#include <femx/model/ns/Components.hpp>

#ifdef REFBAR_LAYOUT
#include <cstdint>
#include <cstdio>
#include <cstring>
#endif

namespace refbar
{
using femx::Index;
using femx::MemorySpace;
using femx::Real;

struct KappaPoissonP1Dev
{
  femx::fem::ElementQuadratureDataView<MemorySpace::Device> data;
  femx::fem::GeometryView<MemorySpace::Device>              geom;
  const Real*                                               kappa;
  const Real*                                               f;

  FEMX_HOST_DEVICE void evalRow(const femx::assembly::ElementView<MemorySpace::Device>& e,
                                Index row, Real& res,
                                femx::VectorView<MemorySpace::Device, Real> jac) const
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

} // namespace refbar

#ifndef REFBAR_LAYOUT
template __global__ void femx::assembly::detail::assembleKernel<refbar::KappaPoissonP1Dev>(
    refbar::KappaPoissonP1Dev, femx::fem::GeometryView<femx::MemorySpace::Device>,
    femx::assembly::AssemblyMapView<femx::MemorySpace::Device>, const femx::Real*,
    femx::Real*, femx::Real*);
template __global__ void femx::assembly::detail::assembleTimeKernel<
    femx::model::ns::NavierOperator<femx::MemorySpace::Device>>(
    femx::model::ns::NavierOperator<femx::MemorySpace::Device>, femx::Index, femx::Index,
    femx::state::VariableBlock, femx::assembly::AssemblyMapView<femx::MemorySpace::Device>,
    const femx::Real*, const femx::Real*, femx::Real*, femx::Real*);
#else
namespace
{
// sentinel for field k: recognisable 8-byte (pointer) and 4-byte (index) values
std::uint64_t sentP(int k)
{
  return 0x5a5a000000000000ull | (std::uint64_t(k) << 8) | 0x11u;
}
int sentI(int k)
{
  return 0x3c3c0000 | (k << 4) | 0x7;
}

// an 8-byte sentinel for a double field: the bit pattern of a finite double
double sentD(int k)
{
  const std::uint64_t u = 0x4b4b000000000000ull | (std::uint64_t(k) << 8) | 0x33u;
  double              d;
  std::memcpy(&d, &u, 8);
  return d;
}

template <class T>
void dump(const char* param, const T& obj, int nfields, const char* const* names,
          const bool* is_ptr, bool last, const bool* is_dbl = nullptr)
{
  unsigned char b[sizeof(T)];
  std::memcpy(b, &obj, sizeof(T));
  std::printf("  \"%s\": {\"size\": %zu, \"fields\": {", param, sizeof(T));
  for (int k = 0; k < nfields; ++k)
  {
    long       off  = -1;
    const bool dbl  = is_dbl != nullptr && is_dbl[k];
    const bool wide = is_ptr[k] || dbl;
    for (size_t o = 0; o + (wide ? 8 : 4) <= sizeof(T); o += 4)
    {
      if (wide)
      {
        std::uint64_t v, want;
        std::memcpy(&v, b + o, 8);
        if (dbl)
        {
          const double d = sentD(k);
          std::memcpy(&want, &d, 8);
        }
        else
        {
          want = sentP(k);
        }
        if (v == want)
        {
          off = long(o);
          break;
        }
      }
      else
      {
        int v;
        std::memcpy(&v, b + o, 4);
        if (v == sentI(k))
        {
          off = long(o);
          break;
        }
      }
    }
    if (off < 0)
    {
      std::fprintf(stderr, "field %s of %s not found\n", names[k], param);
      std::exit(1);
    }
    std::printf("%s\"%s\": [%ld, %d%s]", k ? ", " : "", names[k], off, wide ? 8 : 4,
                dbl ? ", \"f64\"" : "");
  }
  std::printf("}}%s\n", last ? "" : ",");
}

template <class V>
V vview(int kp, int ks)
{
  using T = typename std::remove_pointer<decltype(V().data())>::type;
  return V(reinterpret_cast<T*>(sentP(kp)), sentI(ks));
}
} // namespace

int main()
{
  using namespace femx;
  using DevGeom = fem::GeometryView<MemorySpace::Device>;
  using DevQuad = fem::ElementQuadratureDataView<MemorySpace::Device>;
  using CR      = VectorView<MemorySpace::Device, const Real>;
  using CI      = VectorView<MemorySpace::Device, const Index>;
  std::printf("{\n");
  {
    // GeometryView(dim, num_nodes, num_elems, max_elem_nodes, coords, offsets, conn)
    const DevGeom g(sentI(0), sentI(1), sentI(2), sentI(3), vview<CR>(4, 5), vview<CI>(6, 7),
                    vview<CI>(8, 9));
    const char* n[] = {"dim",          "num_nodes",       "num_elems",  "max_elem_nodes",
                       "coords",       "coords_size",     "elem_offsets", "elem_offsets_size",
                       "conn",         "conn_size"};
    const bool  p[] = {0, 0, 0, 0, 1, 0, 1, 0, 1, 0};
    dump("geom", g, 10, n, p, false);
  }
  {
    assembly::AssemblyMapView<MemorySpace::Device> m;
    m.num_elems     = sentI(0);
    m.num_res       = sentI(1);
    m.num_states    = sentI(2);
    m.res_offsets   = reinterpret_cast<const Index*>(sentP(3));
    m.res_dofs      = reinterpret_cast<const Index*>(sentP(4));
    m.state_offsets = reinterpret_cast<const Index*>(sentP(5));
    m.state_dofs    = reinterpret_cast<const Index*>(sentP(6));
    m.jac_offsets   = reinterpret_cast<const Index*>(sentP(7));
    m.jac_map       = reinterpret_cast<const Index*>(sentP(8));
    m.max_res       = sentI(9);
    m.max_state     = sentI(10);
    m.max_jac       = sentI(11);
    const char* n[] = {"num_elems", "num_res",     "num_states", "res_offsets",
                       "res_dofs",  "state_offsets", "state_dofs", "jac_offsets",
                       "jac_map",   "max_res",     "max_state",  "max_jac"};
    const bool  p[] = {0, 0, 0, 1, 1, 1, 1, 1, 1, 0, 0, 0};
    dump("map", m, 12, n, p, false);
  }
  {
    refbar::KappaPoissonP1Dev op{
        DevQuad(sentI(0), sentI(1), sentI(2), sentI(3), vview<CR>(4, 5), vview<CR>(6, 7),
                vview<CR>(8, 9)),
        DevGeom(sentI(10), sentI(11), sentI(12), sentI(13), vview<CR>(14, 15),
                vview<CI>(16, 17), vview<CI>(18, 19)),
        reinterpret_cast<const Real*>(sentP(20)), reinterpret_cast<const Real*>(sentP(21))};
    const char* n[] = {"q_num_elems", "q_num_qpts", "q_num_shapes", "q_dim",
                       "q_N",         "q_N_size",   "q_dNdx",       "q_dNdx_size",
                       "q_JxW",       "q_JxW_size", "g_dim",        "g_num_nodes",
                       "g_num_elems", "g_max_elem_nodes", "g_coords", "g_coords_size",
                       "g_elem_offsets", "g_elem_offsets_size", "g_conn", "g_conn_size",
                       "kappa",       "f"};
    const bool  p[] = {0, 0, 0, 0, 1, 0, 1, 0, 1, 0, 0, 0, 0, 0, 1, 0, 1, 0, 1, 0, 1, 1};
    dump("op", op, 22, n, p, false);
  }
  {
    using Nav = model::ns::NavierOperator<MemorySpace::Device>;
    const Nav op(model::ns::NavierDataView<MemorySpace::Device>(
                     sentI(0), sentI(1), sentI(2), sentI(3), vview<CR>(4, 5), vview<CR>(6, 7),
                     vview<CR>(8, 9)),
                 model::ns::KernelFluid{sentD(10), sentD(11)}, sentD(12));
    const char* n[] = {"num_elems", "num_qpts", "num_nodes", "dim",  "N",   "N_size", "dNdx",
                       "dNdx_size", "JxW",      "JxW_size",  "rho",  "mu",  "dt"};
    const bool  p[] = {0, 0, 0, 0, 1, 0, 1, 0, 1, 0, 0, 0, 0};
    const bool  d[] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1};
    dump("navier_op", op, 13, n, p, false, d);
  }
  {
    // the Jacobian block of femx's next-state assembly, as bytes
    const state::VariableBlock w = state::VariableBlock::NextState;
    unsigned char              b[sizeof(w)];
    std::memcpy(b, &w, sizeof(w));
    std::printf("  \"wrt_next\": [");
    for (size_t i = 0; i < sizeof(w); ++i)
    {
      std::printf("%s%d", i ? ", " : "", b[i]);
    }
    std::printf("]\n");
  }
  std::printf("}\n");
  return 0;
}
#endif
