// p1.cu — kappa-weighted P1 Poisson residual + Jacobian assembly and its
// residual VJPs (the operator of femx's Poisson example,
// examples/poisson/PoissonComponents.hpp:35-64, with a per-element
// coefficient and a load), replacing the generic assembleKernel
// (femx/assembly/CudaAssembly.hpp:100-169) for this operator.
//
// One thread owns one element. P1 gradients are constant, so the element
// needs one 2x2 inverse: with edge vectors a = x1-x0, b = x2-x0, the scaled
// gradients are h1 = (b.y, -b.x), h2 = (-a.y, a.x), h0 = -(h1+h2), and
//   K_ij = kappa / (2|det|) h_i . h_j,   det = a.x b.y - b.x a.y,
// which is the reference's sum over the order-2 rule (weights 1/6) of
// dN_i . dN_j JxW, rows summing to zero. The load of the P1-interpolated
// source is exact for that rule: F_i = |det|/24 (f_i + f_0 + f_1 + f_2).
// Results are scatter-added with FP64 reductions at L2 (red.global.add.f64).
#include "p1_elem.cuh"
#include "p1_tiled.cuh"

namespace
{

template <int kF32, bool kSepConn, bool kLoad, bool kJac, bool kRes = true>
__global__ void __launch_bounds__(256) p1AssembleKernel(P1Args a)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < a.ne)
  {
    p1Element<kF32, kSepConn, kLoad, kJac, kRes, false>(a, e);
  }
}

template <int kF32, bool kSepConn>
__global__ void __launch_bounds__(256) p1VjpKernel(P1Args a)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < a.ne)
  {
    p1Element<kF32, kSepConn, false, false, false, true>(a, e);
  }
}

// Coloured element pass: thread i takes element elems[i] of one colour and
// adds with plain read-add-writes (no element of the colour shares a DOF).
template <int kF32, bool kSep, bool kLoad, bool kJac, bool kRes, bool kVjp>
__global__ void __launch_bounds__(256)
    p1ColourKernel(P1Args a, const int* __restrict__ elems, int n)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    p1Element<kF32, kSep, kLoad, kJac, kRes, kVjp, true>(a, elems[i]);
  }
}

// One element pass: every element at once with FP64 reductions, or, when
// coloured, one launch per colour in colour order. dep: the (first) launch
// is a dependent of the zero fill before it and overlaps it up to its first
// addition; later colours wait for the whole colour before them.
template <int kF32, bool kSep, bool kLoad, bool kJac, bool kRes, bool kVjp>
void p1Pass(const P1Args& a, const gbfem_assembly_map* map, bool coloured, bool dep,
            cudaStream_t s)
{
  if (!coloured)
  {
    if constexpr (kVjp)
    {
      gbfem::launchMaybeDependent(dep, p1VjpKernel<kF32, kSep>, gbfem::blocksFor(a.ne, 256),
                                  256, s, a);
    }
    else
    {
      gbfem::launchMaybeDependent(dep, p1AssembleKernel<kF32, kSep, kLoad, kJac, kRes>,
                                  gbfem::blocksFor(a.ne, 256), 256, s, a);
    }
    return;
  }
  for (int c = 0; c < map->num_colours; ++c)
  {
    const int b = map->colour_off_host[c], n = map->colour_off_host[c + 1] - b;
    if (n > 0)
    {
      gbfem::launchMaybeDependent(dep && c == 0,
                                  p1ColourKernel<kF32, kSep, kLoad, kJac, kRes, kVjp>,
                                  gbfem::blocksFor(n, 256), 256, s, a,
                                  static_cast<const int*>(map->colour_elems + b), n);
    }
  }
}

template <int kF32, bool kSep>
void launchAssemble(const P1Args& a, const gbfem_assembly_map* map, bool coloured, bool load,
                    bool jac, bool dep, cudaStream_t s)
{
  if (load && jac)
  {
    p1Pass<kF32, kSep, true, true, true, false>(a, map, coloured, dep, s);
  }
  else if (load)
  {
    p1Pass<kF32, kSep, true, false, true, false>(a, map, coloured, dep, s);
  }
  else if (jac)
  {
    p1Pass<kF32, kSep, false, true, true, false>(a, map, coloured, dep, s);
  }
  else
  {
    p1Pass<kF32, kSep, false, false, true, false>(a, map, coloured, dep, s);
  }
}

P1Args makeArgs(const gbfem_assembly_map* map, int num_nodes,
                const double* coords, const int* conn, const double* kappa,
                const double* u)
{
  using gbfem::require;
  require(map != nullptr, "AssemblyMap handle is null");
  require(map->num_elems == 0
              || (map->uniform_res == 3 && map->uniform_state == 3),
          "KappaPoissonP1 expects three DOFs per element");
  require(map->num_res == map->num_states && map->same_dofs,
          "KappaPoissonP1 expects identical residual and state DOF tables");
  require(num_nodes >= 0, "Geometry node count must be non-negative");
  require(map->num_elems == 0 || (coords && kappa && u),
          "Assembly inputs must not be null");
  require(conn != nullptr || num_nodes == map->num_states,
          "Geometry and AssemblyMap have different node counts");
  P1Args a{};
  a.ne        = map->num_elems;
  a.num_nodes = num_nodes;
  a.dofs    = map->state_dofs;
  a.conn    = conn;
  a.coords  = reinterpret_cast<const double2*>(coords);
  a.kappa   = kappa;
  a.u       = u;
  a.jac_map = map->jac_map;
  a.row_ptr = map->row_ptr;
  a.jac_pos = map->pos_stride == 4 ? reinterpret_cast<const unsigned*>(map->jac_pos)
                                   : nullptr;
  a.status  = map->status;
  return a;
}

} // namespace

extern "C" int gbfem_assemble_p1_kappa(const gbfem_assembly_map* map,
                                       int num_nodes, const double* coords,
                                       const int* conn, const double* kappa,
                                       const double* f_nodal, const double* u,
                                       double* res, double* vals,
                                       int precision, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    P1Args a = makeArgs(map, num_nodes, coords, conn, kappa, u);
    require(res != nullptr, "Assembly residual output is null");
    require(res != u && vals != u && (vals == nullptr || res != vals),
            "Assembly state, residual, and matrix values must not alias");
    const bool col   = (precision & GBFEM_COLOURED) != 0;
    const bool tiled = (precision & GBFEM_TILED) != 0;
    precision &= ~(GBFEM_COLOURED | GBFEM_TILED);
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_DOUBLE_FLOAT,
            "unknown precision mode");
    require(!col || map->num_elems == 0 || map->colour_elems != nullptr,
            "coloured assembly needs gbfem_assembly_map_enable_colouring on the map");
    require((reinterpret_cast<uintptr_t>(coords) & 15) == 0,
            "Geometry coordinates must be 16-byte aligned");
    cudaStream_t s = asStream(stream);
    a.f            = f_nodal;
    a.res          = res;
    a.vals         = vals;
    if (tiled)
    {
      require(!col, "tiled and coloured assembly are exclusive");
      require(precision != GBFEM_PREC_MIXED,
              "tiled assembly runs in FP64, FP32_QUAD or DOUBLE_FLOAT");
      require(map->tile_row_off != nullptr,
              "tiled assembly needs gbfem_assembly_map_enable_tiles on the map");
      require((conn != nullptr) == map->tile_sep_conn,
              "tiled assembly: pass the geometry connectivity exactly when the tiles were "
              "built with it");
      P1TileArgs t{};
      t.row_off   = map->tile_row_off;
      t.row_info  = map->tile_row_info;
      t.run_off   = map->tile_run_off;
      t.runs      = map->tile_runs;
      t.elem_off  = map->tile_elem_off;
      t.elems     = map->tile_elems;
      t.tconn     = map->tile_conn;
      t.vert_off  = map->tile_vert_off;
      t.vert_dof  = map->tile_vert_dof;
      t.vert_node = map->tile_vert_node;
      t.slot_ref  = map->slot_ref;
      t.coords    = a.coords;
      t.kappa     = kappa;
      t.f         = f_nodal;
      t.u         = u;
      t.res       = res;
      t.vals      = vals;
      t.status    = map->status;
      const bool load = f_nodal != nullptr, jac = vals != nullptr;
      if (precision == GBFEM_PREC_DOUBLE_FLOAT)
      {
        load ? (jac ? launchP1Tiled<Dd, true, true>(t, map, s)
                    : launchP1Tiled<Dd, true, false>(t, map, s))
             : (jac ? launchP1Tiled<Dd, false, true>(t, map, s)
                    : launchP1Tiled<Dd, false, false>(t, map, s));
      }
      else if (precision == GBFEM_PREC_FP64)
      {
        load ? (jac ? launchP1Tiled<double, true, true>(t, map, s)
                    : launchP1Tiled<double, true, false>(t, map, s))
             : (jac ? launchP1Tiled<double, false, true>(t, map, s)
                    : launchP1Tiled<double, false, false>(t, map, s));
      }
      else
      {
        load ? (jac ? launchP1Tiled<float, true, true>(t, map, s)
                    : launchP1Tiled<float, true, false>(t, map, s))
             : (jac ? launchP1Tiled<float, false, true>(t, map, s)
                    : launchP1Tiled<float, false, false>(t, map, s));
      }
      cudaCheck(cudaGetLastError(), "tiled P1 assembly launch");
      return;
    }
    zeroForNext(vals, vals != nullptr ? map->nnz : 0, res, map->num_res, s);
    if (a.ne == 0)
    {
      return;
    }
    const bool load = f_nodal != nullptr, jac = vals != nullptr;
    const bool sep  = conn != nullptr;
    if (precision == GBFEM_PREC_FP64 || (precision == GBFEM_PREC_MIXED && !jac))
    {
      sep ? launchAssemble<0, true>(a, map, col, load, jac, true, s)
          : launchAssemble<0, false>(a, map, col, load, jac, true, s);
    }
    else if (precision == GBFEM_PREC_DOUBLE_FLOAT)
    {
      sep ? launchAssemble<2, true>(a, map, col, load, jac, true, s)
          : launchAssemble<2, false>(a, map, col, load, jac, true, s);
    }
    else if (precision == GBFEM_PREC_FP32_QUAD)
    {
      sep ? launchAssemble<true, true>(a, map, col, load, jac, true, s)
          : launchAssemble<true, false>(a, map, col, load, jac, true, s);
    }
    else
    {
      // Jacobian from FP32 quadrature, residual from FP64 element math
      sep ? p1Pass<true, true, false, true, false, false>(a, map, col, true, s)
          : p1Pass<true, false, false, true, false, false>(a, map, col, true, s);
      sep ? launchAssemble<false, true>(a, map, col, load, false, false, s)
          : launchAssemble<false, false>(a, map, col, load, false, false, s);
    }
    cudaCheck(cudaGetLastError(), "P1 assembly launch");
  });
}

extern "C" int gbfem_vjp_p1_kappa(const gbfem_assembly_map* map, int num_nodes,
                                  const double* coords, const int* conn,
                                  const double* kappa, const double* u,
                                  const double* lam, double* g_u, double* g_m,
                                  int precision, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    P1Args a = makeArgs(map, num_nodes, coords, conn, kappa, u);
    require(lam != nullptr, "VJP adjoint input is null");
    require(g_u != lam && g_u != u && g_m != lam && g_m != u,
            "VJP outputs must not alias inputs");
    const bool col   = (precision & GBFEM_COLOURED) != 0;
    const bool tiled = (precision & GBFEM_TILED) != 0;
    precision &= ~(GBFEM_COLOURED | GBFEM_TILED);
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_DOUBLE_FLOAT,
            "unknown precision mode");
    if (tiled)
    {
      require(!col, "tiled and coloured assembly are exclusive");
      require(precision != GBFEM_PREC_MIXED,
              "tiled assembly runs in FP64, FP32_QUAD or DOUBLE_FLOAT");
      require(map->tile_row_off != nullptr,
              "tiled assembly needs gbfem_assembly_map_enable_tiles on the map");
      require((conn != nullptr) == map->tile_sep_conn,
              "tiled assembly: pass the geometry connectivity exactly when the tiles were "
              "built with it");
      P1TileArgs t{};
      t.row_off   = map->tile_row_off;
      t.row_info  = map->tile_row_info;
      t.run_off   = map->tile_run_off;
      t.runs      = map->tile_runs;
      t.elem_off  = map->tile_elem_off;
      t.elems     = map->tile_elems;
      t.tconn     = map->tile_conn;
      t.vert_off  = map->tile_vert_off;
      t.vert_dof  = map->tile_vert_dof;
      t.vert_node = map->tile_vert_node;
      t.slot_ref  = map->slot_ref;
      t.coords    = a.coords;
      t.kappa     = kappa;
      t.u         = lam;
      t.u_state   = u;
      t.res       = g_u;
      t.g_m       = g_m;
      t.status    = map->status;
      // FP32 element gradients would put ~1e-7 relative noise on every g_m[e],
      // which directional derivatives over many elements amplify: the tiled
      // VJP runs FP64-accurate only
      require(precision == GBFEM_PREC_DOUBLE_FLOAT || precision == GBFEM_PREC_FP64,
              "the tiled P1 VJP runs in FP64 or DOUBLE_FLOAT");
      cudaStream_t s = asStream(stream);
      if (precision == GBFEM_PREC_DOUBLE_FLOAT)
      {
        launchP1Tiled<Dd, false, false, true>(t, map, s);
      }
      else
      {
        launchP1Tiled<double, false, false, true>(t, map, s);
      }
      cudaCheck(cudaGetLastError(), "tiled P1 VJP launch");
      return;
    }
    require(!col || map->num_elems == 0 || map->colour_elems != nullptr,
            "coloured assembly needs gbfem_assembly_map_enable_colouring on the map");
    cudaStream_t s = asStream(stream);
    a.lam          = lam;
    a.g_u          = g_u;
    a.g_m          = g_m;
    if (g_u != nullptr)
    {
      // the VJP kernel is launched as a dependent of this zero fill
      zeroForNext(g_u, map->num_states, nullptr, 0, s);
    }
    if (a.ne == 0 || (g_u == nullptr && g_m == nullptr))
    {
      return;
    }
    const bool sep = conn != nullptr;
    const bool dep = g_u != nullptr;
    if (precision != GBFEM_PREC_FP32_QUAD)
    {
      sep ? p1Pass<false, true, false, false, false, true>(a, map, col, dep, s)
          : p1Pass<false, false, false, false, false, true>(a, map, col, dep, s);
    }
    else
    {
      sep ? p1Pass<true, true, false, false, false, true>(a, map, col, dep, s)
          : p1Pass<true, false, false, false, false, true>(a, map, col, dep, s);
    }
    cudaCheck(cudaGetLastError(), "P1 VJP launch");
  });
}

// Reads and clears the map's device status word (e.g. a degenerate element
// met by an assembly or VJP kernel). Synchronizes `stream`; not a hot call.
extern "C" int gbfem_assembly_map_check(const gbfem_assembly_map* map,
                                        void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(map != nullptr, "AssemblyMap handle is null");
    cudaStream_t s = asStream(stream);
    try
    {
      checkDeviceStatus(map->status, s);
    }
    catch (...)
    {
      cudaMemsetAsync(map->status, 0, sizeof(DeviceStatus), s);
      cudaStreamSynchronize(s);
      throw;
    }
  });
}
