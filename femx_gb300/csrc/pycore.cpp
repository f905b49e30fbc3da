// pycore.cpp — the pybind11 module femx_gb300._core: femx's Python surface
// (femx._core, python/bindings/Module.cpp:7-30) for the assembly path, over
// libgbfem's C ABI.
//
// What it keeps from femx's module: the module attributes (__version__,
// _cuda_available), the time-residual protocol types TimeDims, VariableBlock
// and TimeResidual with femx's Python names (python/bindings/State.cpp:
// 649-667) and a trampoline so that Python subclasses override the
// protocol's methods (PyTimeResidual, State.cpp:259-460). What it adds: the
// assembly path itself under femx's C++ names in snake case —
// make_assembly_map, make_boundary_map, assemble_* per operator, replace_rows,
// replace_res, zero_boundary, prepare_forward_solve, matvec, matvec_t, the
// residual VJPs — and NavierTimeResidual, femx's GLS Navier-Stokes time
// residual implemented natively (femx's own is NavierResidual,
// NavierStokesModel.cpp:374-543).
//
// Arrays are CUDA tensors (any object with data_ptr(), or exposing
// __cuda_array_interface__); outputs are passed in, as femx's C++ assemble
// takes them (CudaAssembly.hpp:319-326), except for the time-residual
// protocol, whose methods return new tensors (allocated through torch, so
// that they come from the caller's caching allocator). Work is ordered on
// torch's current CUDA stream. The GIL is released around every library
// call; failures raise RuntimeError with femx's require() messages.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>

#include "gbfem.h"

namespace py = pybind11;
using namespace py::literals;

namespace
{

void check(int rc)
{
  if (rc != GBFEM_OK)
  {
    throw std::runtime_error(gbfem_last_error());
  }
}

// runs a library call without the GIL and raises on failure
template <class F>
void call(F&& f)
{
  int rc;
  {
    py::gil_scoped_release nogil;
    rc = f();
  }
  check(rc);
}

py::module_& torchMod()
{
  static py::module_ t = py::module_::import("torch");
  return t;
}

void* currentStream()
{
  return reinterpret_cast<void*>(
      torchMod().attr("cuda").attr("current_stream")().attr("cuda_stream").cast<uintptr_t>());
}

// A device array argument: its address after checking device, dtype,
// contiguity and (n >= 0) the element count. dtype: "float64" or "int32".
struct Arr
{
  void*     p = nullptr;
  long long n = 0;
};

Arr arr(const py::object& o, const char* dtype, long long n, const char* what,
        bool allow_none = false)
{
  Arr a;
  if (o.is_none())
  {
    if (!allow_none)
    {
      throw std::runtime_error(std::string(what) + " must not be None");
    }
    return a;
  }
  if (py::hasattr(o, "data_ptr"))
  {
    if (!o.attr("is_cuda").cast<bool>())
    {
      throw std::runtime_error(std::string(what) + " must be a CUDA tensor");
    }
    const std::string dt = py::str(o.attr("dtype")).cast<std::string>();
    if (dt != std::string("torch.") + dtype)
    {
      throw std::runtime_error(std::string(what) + " must be " + dtype + ", got " + dt);
    }
    if (!o.attr("is_contiguous")().cast<bool>())
    {
      throw std::runtime_error(std::string(what) + " must be contiguous");
    }
    a.p = reinterpret_cast<void*>(o.attr("data_ptr")().cast<uintptr_t>());
    a.n = o.attr("numel")().cast<long long>();
  }
  else if (py::hasattr(o, "__cuda_array_interface__"))
  {
    const py::dict ai = o.attr("__cuda_array_interface__");
    const std::string ts = ai["typestr"].cast<std::string>();
    if (ts != (std::string(dtype) == "float64" ? "<f8" : "<i4"))
    {
      throw std::runtime_error(std::string(what) + " must be " + dtype);
    }
    a.p = reinterpret_cast<void*>(ai["data"].cast<py::tuple>()[0].cast<uintptr_t>());
    a.n = 1;
    for (auto d : ai["shape"].cast<py::tuple>())
    {
      a.n *= d.cast<long long>();
    }
  }
  else
  {
    throw std::runtime_error(std::string(what) + " must be a CUDA array");
  }
  if (n >= 0 && a.n != n)
  {
    throw std::runtime_error(std::string(what) + " size mismatch: expected " + std::to_string(n)
                             + ", got " + std::to_string(a.n));
  }
  return a;
}

double* f64(const py::object& o, long long n, const char* what, bool allow_none = false)
{
  return static_cast<double*>(arr(o, "float64", n, what, allow_none).p);
}

int* i32(const py::object& o, long long n, const char* what, bool allow_none = false)
{
  return static_cast<int*>(arr(o, "int32", n, what, allow_none).p);
}

long long numNodes(const py::object& coords)
{
  const Arr a = arr(coords, "float64", -1, "coords");
  if (a.n % 2 != 0)
  {
    throw std::runtime_error("coords must hold two coordinates per node");
  }
  return a.n / 2;
}

// A float64 vector argument of the time-residual protocol: femx passes host
// arrays in ctx (numpy); anything that is not a CUDA float64 tensor is copied
// to the device first (the copy is kept alive in `keep` for the call).
const double* vecF64(const py::object& o, long long n, const char* what, py::list& keep)
{
  py::module_& t = torchMod();
  py::object   d = t.attr("as_tensor")(o, "dtype"_a = t.attr("float64"), "device"_a = "cuda")
                     .attr("reshape")(-1)
                     .attr("contiguous")();
  keep.append(d);
  return f64(d, n, what);
}

py::object emptyF64(long long n)
{
  py::module_& t = torchMod();
  return t.attr("empty")(n, "dtype"_a = t.attr("float64"), "device"_a = "cuda");
}

int precisionMode(const std::string& p)
{
  if (p == "fp64")
  {
    return GBFEM_PREC_FP64;
  }
  if (p == "fp32_quad")
  {
    return GBFEM_PREC_FP32_QUAD;
  }
  if (p == "mixed")
  {
    return GBFEM_PREC_MIXED;
  }
  if (p == "double_float")
  {
    return GBFEM_PREC_DOUBLE_FLOAT;
  }
  throw std::runtime_error("unknown precision mode: " + p);
}

// A view of a device array owned by a handle (not to be written), exposing
// __cuda_array_interface__ (torch.as_tensor(view, device="cuda") shares it).
struct DeviceView
{
  uintptr_t   ptr = 0;
  long long   n   = 0;
  std::string typestr;
  py::dict    interface() const
  {
    py::dict d;
    d["shape"]   = py::make_tuple(n);
    d["typestr"] = typestr;
    d["data"]    = py::make_tuple(ptr, false);
    d["version"] = 3;
    d["strides"] = py::none();
    return d;
  }
};

// femx AssemblyMap<Device> with its CSR pattern (AssemblyMap.hpp:78-206)
struct AssemblyMap
{
  gbfem_assembly_map*     h = nullptr;
  gbfem_assembly_map_view v{};
  explicit AssemblyMap(gbfem_assembly_map* m) : h(m)
  {
    check(gbfem_assembly_map_get_view(h, &v));
  }
  ~AssemblyMap()
  {
    gbfem_assembly_map_destroy(h);
  }
  AssemblyMap(const AssemblyMap&)            = delete;
  AssemblyMap& operator=(const AssemblyMap&) = delete;
};

// femx BoundaryMap<Device> (BoundaryMap.hpp:69-175)
struct BoundaryMap
{
  gbfem_boundary_map*     h = nullptr;
  gbfem_boundary_map_view v{};
  explicit BoundaryMap(gbfem_boundary_map* b) : h(b)
  {
    check(gbfem_boundary_map_get_view(h, &v));
  }
  ~BoundaryMap()
  {
    gbfem_boundary_map_destroy(h);
  }
  BoundaryMap(const BoundaryMap&)            = delete;
  BoundaryMap& operator=(const BoundaryMap&) = delete;
};

// femx::state::TimeDims (TimeResidual.hpp:13-21)
struct TimeDims
{
  int num_steps = 0, num_states = 0, num_param = 0, num_res = 0, num_hist = 1;
};

// femx::state::VariableBlock (TimeResidual.hpp:93-166)
struct VariableBlock
{
  enum Kind
  {
    History,
    NextState,
    Parameter
  };
  Kind kind = History;
  int  lag  = 0;
};

// femx's Python time residual (the PyTimeResidual contract): ctx is the
// dict femx builds (step, next_state, parameters, history lag-major).
struct TimeResidual
{
  virtual ~TimeResidual() = default;
  virtual TimeDims   dims() const = 0;
  virtual py::object initial_state(const py::object& prm) const
  {
    (void)prm;
    py::module_& t = torchMod();
    return t.attr("zeros")(dims().num_states, "dtype"_a = t.attr("float64"), "device"_a = "cuda");
  }
  virtual py::object residual(const py::dict& ctx) const      = 0;
  virtual py::object assemble_next(const py::dict& ctx) const = 0;
  virtual py::object apply_jacobian_transpose(const py::dict& ctx, const VariableBlock& wrt,
                                              const py::object& adj) const = 0;
  virtual py::object prepare_linear_solve(const py::dict& ctx, const py::object& jac,
                                          const py::object& rhs) const
  {
    (void)ctx;
    (void)jac;
    (void)rhs;
    return py::none();
  }
};

// lets Python subclasses implement the protocol
struct PyTimeResidual : TimeResidual
{
  TimeDims dims() const override
  {
    PYBIND11_OVERRIDE_PURE(TimeDims, TimeResidual, dims, );
  }
  py::object initial_state(const py::object& prm) const override
  {
    PYBIND11_OVERRIDE(py::object, TimeResidual, initial_state, prm);
  }
  py::object residual(const py::dict& ctx) const override
  {
    PYBIND11_OVERRIDE_PURE(py::object, TimeResidual, residual, ctx);
  }
  py::object assemble_next(const py::dict& ctx) const override
  {
    PYBIND11_OVERRIDE_PURE(py::object, TimeResidual, assemble_next, ctx);
  }
  py::object apply_jacobian_transpose(const py::dict& ctx, const VariableBlock& wrt,
                                      const py::object& adj) const override
  {
    PYBIND11_OVERRIDE_PURE(py::object, TimeResidual, apply_jacobian_transpose, ctx, wrt, adj);
  }
  py::object prepare_linear_solve(const py::dict& ctx, const py::object& jac,
                                  const py::object& rhs) const override
  {
    PYBIND11_OVERRIDE(py::object, TimeResidual, prepare_linear_solve, ctx, jac, rhs);
  }
};

// femx's GLS Navier-Stokes time residual (NavierResidual's behaviour: two
// history lags, no parameters, its checks and messages) on the GPU. The
// caller builds the map in femx's mixed layout (velocity 2 node + comp,
// then pressure) and keeps coords (N x 2 float64) and conn (E x 3 int32).
struct NavierTimeResidual : TimeResidual
{
  static constexpr int          kHist = 2;
  std::shared_ptr<AssemblyMap>  map;
  py::object                    coords, conn;
  double                        rho, mu, dt;
  int                           num_steps;

  NavierTimeResidual(std::shared_ptr<AssemblyMap> m, py::object xy, py::object c, double r,
                     double m_u, double d, int steps)
    : map(std::move(m)), coords(std::move(xy)), conn(std::move(c)), rho(r), mu(m_u), dt(d),
      num_steps(steps)
  {
    (void)f64(coords, -1, "coords");
    (void)i32(conn, 3LL * map->v.num_elems, "conn");
  }

  TimeDims dims() const override
  {
    return TimeDims{num_steps, map->v.num_states, 0, map->v.num_res, kHist};
  }

  py::object initial_state(const py::object& prm) const override
  {
    if (!prm.is_none() && py::len(prm) != 0)
    {
      throw std::runtime_error("Navier physics residual is parameter-free");
    }
    return TimeResidual::initial_state(prm);
  }

  // femx's NavierResidual::checkCtx (NavierStokesModel.cpp:550-558)
  struct Ctx
  {
    int           step;
    const double* hist;
    const double* nxt;
    py::list      keep; // device copies of host inputs
  };
  Ctx ctxOf(const py::dict& ctx) const
  {
    const int n    = map->v.num_states;
    const int step = ctx["step"].cast<int>();
    if (step < 0 || step >= num_steps)
    {
      throw std::runtime_error("Navier residual step is out of range");
    }
    if (ctx.contains("parameters") && !ctx["parameters"].is_none()
        && py::len(ctx["parameters"]) != 0)
    {
      throw std::runtime_error("Navier residual vector size mismatch");
    }
    Ctx             c;
    const double*   h  = vecF64(ctx["history"], -1, "history", c.keep);
    const long long hn = c.keep[0].attr("numel")().cast<long long>();
    if (hn < static_cast<long long>(kHist) * n || (n > 0 && hn % n != 0))
    {
      throw std::runtime_error("Navier residual vector size mismatch");
    }
    c.step = step;
    c.hist = h;
    c.nxt  = vecF64(ctx["next_state"], n, "next state", c.keep);
    return c;
  }

  py::object residual(const py::dict& ctx) const override
  {
    const Ctx    c   = ctxOf(ctx);
    py::object   res = emptyF64(map->v.num_res);
    double*      r   = f64(res, -1, "residual");
    const double* xy = f64(coords, -1, "coords");
    const int*    k  = i32(conn, -1, "conn");
    const long long nn = numNodes(coords);
    void* s = currentStream();
    call([&] {
      return gbfem_assemble_navier(map->h, static_cast<int>(nn), xy, k, rho, mu, dt, c.step,
                                   kHist, -1, c.hist, c.nxt, r, nullptr, s);
    });
    return res;
  }

  // (Jacobian values on the map's pattern, residual)
  py::object assemble_next(const py::dict& ctx) const override
  {
    const Ctx     c    = ctxOf(ctx);
    py::object    res  = emptyF64(map->v.num_res);
    py::object    vals = emptyF64(map->v.nnz);
    double*       r    = f64(res, -1, "residual");
    double*       v    = f64(vals, -1, "values");
    const double* xy   = f64(coords, -1, "coords");
    const int*    k    = i32(conn, -1, "conn");
    const long long nn = numNodes(coords);
    void* s = currentStream();
    call([&] {
      return gbfem_assemble_navier(map->h, static_cast<int>(nn), xy, k, rho, mu, dt, c.step,
                                   kHist, -1, c.hist, c.nxt, r, v, s);
    });
    return py::make_tuple(vals, res);
  }

  py::object apply_jacobian_transpose(const py::dict& ctx, const VariableBlock& wrt,
                                      const py::object& adj) const override
  {
    Ctx c = ctxOf(ctx);
    if (wrt.kind == VariableBlock::NextState)
    {
      throw std::runtime_error(
          "Navier transpose apply supports only history and parameter blocks");
    }
    const double* a = vecF64(adj, map->v.num_res, "adjoint", c.keep);
    if (wrt.kind == VariableBlock::Parameter)
    {
      return emptyF64(0);
    }
    if (wrt.lag < 0 || wrt.lag >= kHist)
    {
      throw std::runtime_error("Navier residual history lag is out of range");
    }
    const int     n   = map->v.num_states;
    py::object    out = emptyF64(static_cast<long long>(kHist) * n);
    double*       o   = f64(out, -1, "out");
    const double* xy  = f64(coords, -1, "coords");
    const int*    k   = i32(conn, -1, "conn");
    const long long nn = numNodes(coords);
    void* s = currentStream();
    call([&] {
      return gbfem_vjp_navier_hist(map->h, static_cast<int>(nn), xy, k, rho, mu, dt, c.step,
                                   kHist, c.hist, c.nxt, a, o, s);
    });
    return out.attr("narrow")(0, static_cast<long long>(wrt.lag) * n, n).attr("clone")();
  }
};

} // namespace

PYBIND11_MODULE(_core, m)
{
  m.doc()               = "femx-style native Python bindings of the GB300 assembly path (libgbfem).";
  m.attr("__version__") = "0.4.0";
  m.attr("_gbfem_version") = gbfem_version();
  m.attr("_cuda_available") = torchMod().attr("cuda").attr("is_available")();
  m.attr("_has_enzyme")     = false;

  py::class_<DeviceView>(m, "_DeviceView")
      .def_property_readonly("__cuda_array_interface__", &DeviceView::interface);

  py::class_<AssemblyMap, std::shared_ptr<AssemblyMap>>(m, "AssemblyMap")
      .def_property_readonly("num_elems", [](const AssemblyMap& a) { return a.v.num_elems; })
      .def_property_readonly("num_res", [](const AssemblyMap& a) { return a.v.num_res; })
      .def_property_readonly("num_states", [](const AssemblyMap& a) { return a.v.num_states; })
      .def_property_readonly("nnz", [](const AssemblyMap& a) { return a.v.nnz; })
      .def_property_readonly("max_res", [](const AssemblyMap& a) { return a.v.max_res; })
      .def_property_readonly("max_state", [](const AssemblyMap& a) { return a.v.max_state; })
      .def_property_readonly("max_jac", [](const AssemblyMap& a) { return a.v.max_jac; })
      .def_property_readonly("layout_id", [](const AssemblyMap& a) { return a.v.layout_id; })
      .def(
          "row_ptr",
          [](const AssemblyMap& a) {
            return DeviceView{reinterpret_cast<uintptr_t>(a.v.row_ptr), a.v.num_res + 1LL,
                              "<i4"};
          },
          py::keep_alive<0, 1>())
      .def(
          "col_ind",
          [](const AssemblyMap& a) {
            return DeviceView{reinterpret_cast<uintptr_t>(a.v.col_ind), a.v.nnz, "<i4"};
          },
          py::keep_alive<0, 1>())
      .def(
          "jac_map",
          [](const AssemblyMap& a) {
            return DeviceView{reinterpret_cast<uintptr_t>(a.v.jac_map), a.v.jac_nnz, "<i4"};
          },
          py::keep_alive<0, 1>())
      .def(
          "enable_tiles",
          [](AssemblyMap& a, const py::object& coords, const py::object& conn) {
            const long long nn = numNodes(coords);
            const double*   xy = f64(coords, -1, "coords");
            const int*      k  = i32(conn, 3LL * a.v.num_elems, "conn", true);
            void*           s  = currentStream();
            call([&] {
              return gbfem_assembly_map_enable_tiles(a.h, static_cast<int>(nn), xy, k, s);
            });
            return gbfem_assembly_map_num_tiles(a.h);
          },
          "coords"_a, "conn"_a = py::none())
      .def("enable_colouring",
           [](AssemblyMap& a) {
             void* s = currentStream();
             call([&] { return gbfem_assembly_map_enable_colouring(a.h, s); });
             return gbfem_assembly_map_num_colours(a.h);
           })
      .def("enable_deterministic",
           [](AssemblyMap& a) {
             void* s = currentStream();
             call([&] { return gbfem_assembly_map_enable_gather(a.h, s); });
           })
      .def("check", [](const AssemblyMap& a) {
        void* s = currentStream();
        call([&] { return gbfem_assembly_map_check(a.h, s); });
      });

  // makeAssemblyMap(num_res, num_states, res_dofs, state_dofs) + copy to the
  // device (AssemblyMap.hpp:220-246): offsets and DOF tables as int32 tensors
  m.def(
      "make_assembly_map",
      [](int num_res, int num_states, const py::object& res_offsets, const py::object& res_dofs,
         const py::object& state_offsets, const py::object& state_dofs) {
        const Arr ro = arr(res_offsets, "int32", -1, "res_offsets");
        const Arr so = arr(state_offsets, "int32", ro.n, "state_offsets");
        const int ne = static_cast<int>(ro.n > 0 ? ro.n - 1 : 0);
        const int* rd = i32(res_dofs, -1, "res_dofs");
        const int* sd = i32(state_dofs, -1, "state_dofs");
        void*      s  = currentStream();
        gbfem_assembly_map* h = nullptr;
        call([&] {
          return gbfem_assembly_map_create(num_res, num_states, ne,
                                           static_cast<const int*>(ro.p), rd,
                                           static_cast<const int*>(so.p), sd, s, &h);
        });
        return std::make_shared<AssemblyMap>(h);
      },
      "num_res"_a, "num_states"_a, "res_offsets"_a, "res_dofs"_a, "state_offsets"_a,
      "state_dofs"_a);

  py::class_<BoundaryMap, std::shared_ptr<BoundaryMap>>(m, "BoundaryMap")
      .def_property_readonly("num_bcs", [](const BoundaryMap& b) { return b.v.num_bcs; })
      .def_property_readonly("layout_id", [](const BoundaryMap& b) { return b.v.layout_id; });

  // makeBoundaryMap(dofs, pattern) (BoundaryMap.hpp:183-184) on the map's pattern
  m.def(
      "make_boundary_map",
      [](const py::object& dofs, const AssemblyMap& a) {
        const Arr d = arr(dofs, "int32", -1, "dofs");
        void*     s = currentStream();
        gbfem_boundary_map* h = nullptr;
        call([&] {
          return gbfem_boundary_map_create(static_cast<int>(d.n), static_cast<const int*>(d.p),
                                           a.v.num_res, a.v.num_states, a.v.row_ptr,
                                           a.v.col_ind, a.v.layout_id, s, &h);
        });
        return std::make_shared<BoundaryMap>(h);
      },
      "dofs"_a, "assembly_map"_a);

  m.def(
      "replace_rows",
      [](const BoundaryMap& b, const py::object& vals, double diag) {
        double* v = f64(vals, b.v.nnz, "values");
        void*   s = currentStream();
        call([&] { return gbfem_replace_rows(b.h, v, diag, s); });
      },
      "bc"_a, "vals"_a, "diag"_a);
  m.def(
      "replace_res",
      [](const BoundaryMap& b, const py::object& state, const py::object& bc_vals,
         const py::object& res) {
        const double* x = f64(state, b.v.num_cols, "state");
        const double* g = f64(bc_vals, b.v.num_bcs, "bc_vals");
        double*       r = f64(res, b.v.num_rows, "residual");
        void*         s = currentStream();
        call([&] { return gbfem_replace_res(b.h, x, g, r, s); });
      },
      "bc"_a, "state"_a, "bc_vals"_a, "res"_a);
  m.def(
      "zero_boundary",
      [](const BoundaryMap& b, const py::object& v) {
        double* p = f64(v, b.v.num_rows, "vector");
        void*   s = currentStream();
        call([&] { return gbfem_zero_boundary(b.h, p, s); });
      },
      "bc"_a, "v"_a);
  m.def(
      "prepare_forward_solve",
      [](const BoundaryMap& b, const py::object& vals, const py::object& rhs,
         const py::object& bc_vals) {
        double*       v = f64(vals, b.v.nnz, "values");
        double*       r = f64(rhs, b.v.num_rows, "rhs");
        const double* g = f64(bc_vals, b.v.num_bcs, "bc_vals");
        void*         s = currentStream();
        call([&] { return gbfem_prepare_forward_solve(b.h, v, r, g, s); });
      },
      "bc"_a, "vals"_a, "rhs"_a, "bc_vals"_a);

  // MatrixHandler<CudaCsrBackend>::matvec / matvecT on the map's pattern
  for (const bool tr : {false, true})
  {
    m.def(
        tr ? "matvec_t" : "matvec",
        [tr](const AssemblyMap& a, const py::object& vals, const py::object& x,
             const py::object& y, double alpha, double beta) {
          const double* v  = f64(vals, a.v.nnz, "values");
          const double* xp = f64(x, tr ? a.v.num_res : a.v.num_states, "x");
          double*       yp = f64(y, tr ? a.v.num_states : a.v.num_res, "y");
          void*         s  = currentStream();
          call([&] {
            return tr ? gbfem_spmv_t(a.v.num_res, a.v.num_states, a.v.row_ptr, a.v.col_ind, v,
                                     xp, yp, alpha, beta, s)
                      : gbfem_spmv(a.v.num_res, a.v.num_states, a.v.row_ptr, a.v.col_ind, v,
                                   xp, yp, alpha, beta, s);
          });
        },
        "assembly_map"_a, "vals"_a, "x"_a, "y"_a, "alpha"_a = 1.0, "beta"_a = 0.0);
  }

  // assemble(KappaPoissonP1{...}, geometry, map, state, res, jac, ctx)
  m.def(
      "assemble_p1_kappa",
      [](const AssemblyMap& a, const py::object& coords, const py::object& kappa,
         const py::object& f_nodal, const py::object& u, const py::object& res,
         const py::object& jac, const py::object& conn, const std::string& precision,
         bool tiled, bool coloured) {
        const long long nn = numNodes(coords);
        const double*   xy = f64(coords, -1, "coords");
        const double*   kp = f64(kappa, a.v.num_elems, "kappa");
        const double*   f  = f64(f_nodal, nn, "source", true);
        const double*   x  = f64(u, a.v.num_states, "state");
        double*         r  = f64(res, a.v.num_res, "residual");
        double*         v  = f64(jac, a.v.nnz, "values", true);
        const int*      k  = i32(conn, 3LL * a.v.num_elems, "conn", true);
        const int mode = precisionMode(precision) | (tiled ? GBFEM_TILED : 0)
                         | (coloured ? GBFEM_COLOURED : 0);
        void* s = currentStream();
        call([&] {
          return gbfem_assemble_p1_kappa(a.h, static_cast<int>(nn), xy, k, kp, f, x, r, v,
                                         mode, s);
        });
      },
      "assembly_map"_a, "coords"_a, "kappa"_a, "f_nodal"_a, "u"_a, "res"_a,
      "jac"_a = py::none(), "conn"_a = py::none(), "precision"_a = "fp64", "tiled"_a = false,
      "coloured"_a = false);

  // Residual::applyParamJacT / state adjoint of the same operator
  m.def(
      "vjp_p1_kappa",
      [](const AssemblyMap& a, const py::object& coords, const py::object& kappa,
         const py::object& u, const py::object& lam, const py::object& g_u,
         const py::object& g_m, const py::object& conn, const std::string& precision,
         bool tiled) {
        const long long nn = numNodes(coords);
        const double*   xy = f64(coords, -1, "coords");
        const double*   kp = f64(kappa, a.v.num_elems, "kappa");
        const double*   x  = f64(u, a.v.num_states, "state");
        const double*   l  = f64(lam, a.v.num_res, "adjoint");
        double*         gu = f64(g_u, a.v.num_states, "g_u", true);
        double*         gm = f64(g_m, a.v.num_elems, "g_m", true);
        const int*      k  = i32(conn, 3LL * a.v.num_elems, "conn", true);
        const int       mode = precisionMode(precision) | (tiled ? GBFEM_TILED : 0);
        void*           s    = currentStream();
        call([&] {
          return gbfem_vjp_p1_kappa(a.h, static_cast<int>(nn), xy, k, kp, x, l, gu, gm, mode, s);
        });
      },
      "assembly_map"_a, "coords"_a, "kappa"_a, "u"_a, "lam"_a, "g_u"_a = py::none(),
      "g_m"_a = py::none(), "conn"_a = py::none(), "precision"_a = "fp64", "tiled"_a = false);

  // the Taylor-Hood P2/P1 Newton residual and Jacobian
  m.def(
      "assemble_taylor_hood",
      [](const AssemblyMap& a, const py::object& coords, const py::object& conn6, double nu,
         const py::object& state, const py::object& res, const py::object& jac,
         const std::string& precision, bool deterministic) {
        const long long nn = numNodes(coords);
        const double*   xy = f64(coords, -1, "coords");
        const int*      k  = i32(conn6, 6LL * a.v.num_elems, "conn6");
        const double*   x  = f64(state, a.v.num_states, "state");
        double*         r  = f64(res, a.v.num_res, "residual");
        double*         v  = f64(jac, a.v.nnz, "values", true);
        const int mode = precisionMode(precision) | (deterministic ? GBFEM_DETERMINISTIC : 0);
        void*     s    = currentStream();
        call([&] {
          return gbfem_assemble_th_ns(a.h, static_cast<int>(nn), xy, k, nu, x, r, v, mode, s);
        });
      },
      "assembly_map"_a, "coords"_a, "conn6"_a, "nu"_a, "state"_a, "res"_a,
      "jac"_a = py::none(), "precision"_a = "fp64", "deterministic"_a = false);

  // its state VJP, J^T lam without forming J (Residual::applyJacT)
  m.def(
      "vjp_taylor_hood",
      [](const AssemblyMap& a, const py::object& coords, const py::object& conn6, double nu,
         const py::object& state, const py::object& lam, const py::object& g_state,
         const std::string& precision) {
        const long long nn = numNodes(coords);
        const double*   xy = f64(coords, -1, "coords");
        const int*      k  = i32(conn6, 6LL * a.v.num_elems, "conn6");
        const double*   x  = f64(state, a.v.num_states, "state");
        const double*   l  = f64(lam, a.v.num_res, "adjoint");
        double*         g  = f64(g_state, a.v.num_states, "g_state");
        const int       mode = precisionMode(precision);
        void*           s    = currentStream();
        call([&] {
          return gbfem_vjp_th_ns(a.h, static_cast<int>(nn), xy, k, nu, x, l, g, mode, s);
        });
      },
      "assembly_map"_a, "coords"_a, "conn6"_a, "nu"_a, "state"_a, "lam"_a, "g_state"_a,
      "precision"_a = "fp64");

  py::class_<TimeDims>(m, "TimeDims")
      .def(py::init<>())
      .def_readwrite("num_steps", &TimeDims::num_steps)
      .def_readwrite("num_states", &TimeDims::num_states)
      .def_readwrite("num_param", &TimeDims::num_param)
      .def_readwrite("num_res", &TimeDims::num_res)
      .def_readwrite("num_hist", &TimeDims::num_hist);

  py::class_<VariableBlock>(m, "VariableBlock")
      .def_static("history",
                  [](int lag) { return VariableBlock{VariableBlock::History, lag}; }, "lag"_a)
      .def_static("next_state", [] { return VariableBlock{VariableBlock::NextState, 0}; })
      .def_static("parameter", [] { return VariableBlock{VariableBlock::Parameter, 0}; })
      .def_property_readonly("is_history_state",
                             [](const VariableBlock& b) { return b.kind == VariableBlock::History; })
      .def_property_readonly("is_next_state", [](const VariableBlock& b) {
        return b.kind == VariableBlock::NextState;
      })
      .def_property_readonly("is_parameter", [](const VariableBlock& b) {
        return b.kind == VariableBlock::Parameter;
      })
      .def_property_readonly("history_lag", [](const VariableBlock& b) { return b.lag; });

  py::class_<TimeResidual, PyTimeResidual, std::shared_ptr<TimeResidual>>(m, "TimeResidual")
      .def(py::init<>())
      .def("dims", &TimeResidual::dims)
      .def("initial_state", &TimeResidual::initial_state, "prm"_a)
      .def("residual", &TimeResidual::residual, "ctx"_a)
      .def("assemble_next", &TimeResidual::assemble_next, "ctx"_a)
      .def("apply_jacobian_transpose", &TimeResidual::apply_jacobian_transpose, "ctx"_a,
           "wrt"_a, "adj"_a)
      .def("prepare_linear_solve", &TimeResidual::prepare_linear_solve, "ctx"_a, "jac"_a,
           "rhs"_a);

  py::class_<NavierTimeResidual, TimeResidual, std::shared_ptr<NavierTimeResidual>>(
      m, "NavierTimeResidual")
      .def(py::init<std::shared_ptr<AssemblyMap>, py::object, py::object, double, double, double,
                    int>(),
           "assembly_map"_a, "coords"_a, "conn"_a, "rho"_a, "mu"_a, "dt"_a, "num_steps"_a)
      .def_property_readonly("assembly_map",
                             [](const NavierTimeResidual& r) { return r.map; });
}
