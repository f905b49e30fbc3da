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
#include <type_traits>

#include "maps.cuh"

namespace
{
using gbfem::DeviceStatus;

struct P1Args
{
  int                  ne;
  int                  num_nodes;
  const int*           dofs;   // res/state DOF table [ne][3]
  const int*           conn;   // geometry connectivity, or == dofs
  const double2*       coords; // [num_nodes]
  const double*        kappa;  // [ne]
  const double*        f;      // nodal source or nullptr
  const double*        u;      // state
  const int*           jac_map;
  const int*           row_ptr;
  const unsigned*      jac_pos; // [ne][3] words: in-row positions, or null
  double*              res;
  double*              vals;
  DeviceStatus*        status;
};

template <class T>
struct ElemK
{
  T k01, k02, k12, k00, k11, k22;
  T adet;
};

// Element stiffness from the three vertices; coordinates differences are
// always formed in FP64 (they carry the mesh scale), the rest in T.
template <class T>
__device__ __forceinline__ bool elementK(double2 x0, double2 x1, double2 x2,
                                         double kappa, ElemK<T>& K)
{
  const T ax = gbfem::fromF64<T>(x1.x - x0.x), ay = gbfem::fromF64<T>(x1.y - x0.y);
  const T bx = gbfem::fromF64<T>(x2.x - x0.x), by = gbfem::fromF64<T>(x2.y - x0.y);
  const T det  = ax * by - bx * ay;
  const T adet = det < T(0) ? -det : det;
  if (!(adet >= T(1.0e-30)))
  {
    return false;
  }
  // h1 = (by, -bx), h2 = (-ay, ax), h0 = -(h1 + h2) = (ay - by, bx - ax)
  const T h0x = ay - by, h0y = bx - ax;
  const T s   = gbfem::fromF64<T>(kappa) * T(0.5) / adet;
  K.k01       = s * (h0x * by - h0y * bx);
  K.k02       = s * (-h0x * ay + h0y * ax);
  K.k12       = s * (-by * ay - bx * ax);
  K.k00       = -(K.k01 + K.k02);
  K.k11       = -(K.k01 + K.k12);
  K.k22       = -(K.k02 + K.k12);
  K.adet      = adet;
  return true;
}

template <bool kF32, bool kSepConn, bool kLoad, bool kJac, bool kRes = true>
__global__ void __launch_bounds__(256) p1AssembleKernel(P1Args a)
{
  using T     = typename std::conditional<kF32, float, double>::type;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne)
  {
    return;
  }
  const int d0 = a.dofs[3 * e + 0], d1 = a.dofs[3 * e + 1], d2 = a.dofs[3 * e + 2];
  int       n0 = d0, n1 = d1, n2 = d2;
  if (kSepConn)
  {
    n0 = a.conn[3 * e + 0];
    n1 = a.conn[3 * e + 1];
    n2 = a.conn[3 * e + 2];
    if (static_cast<unsigned>(n0) >= static_cast<unsigned>(a.num_nodes)
        || static_cast<unsigned>(n1) >= static_cast<unsigned>(a.num_nodes)
        || static_cast<unsigned>(n2) >= static_cast<unsigned>(a.num_nodes))
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
      return;
    }
  }
  ElemK<T> K;
  if (!elementK<T>(a.coords[n0], a.coords[n1], a.coords[n2], a.kappa[e], K))
  {
    gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    return;
  }
  // Element residual in T (FP64 on the plain path); accumulation in FP64.
  const T u0 = gbfem::fromF64<T>(a.u[d0]), u1 = gbfem::fromF64<T>(a.u[d1]);
  const T u2 = gbfem::fromF64<T>(a.u[d2]);
  T r0 = K.k00 * u0 + K.k01 * u1 + K.k02 * u2;
  T r1 = K.k01 * u0 + K.k11 * u1 + K.k12 * u2;
  T r2 = K.k02 * u0 + K.k12 * u1 + K.k22 * u2;
  if (kLoad)
  {
    const T f0 = gbfem::fromF64<T>(a.f[n0]), f1 = gbfem::fromF64<T>(a.f[n1]);
    const T f2 = gbfem::fromF64<T>(a.f[n2]);
    const T fs = f0 + f1 + f2;
    const T c  = K.adet * T(1.0 / 24.0);
    r0 -= c * (f0 + fs);
    r1 -= c * (f1 + fs);
    r2 -= c * (f2 + fs);
  }
  if (kRes)
  {
    gbfem::redAdd(a.res + d0, gbfem::toF64(r0));
    gbfem::redAdd(a.res + d1, gbfem::toF64(r1));
    gbfem::redAdd(a.res + d2, gbfem::toF64(r2));
  }
  if (kJac)
  {
    const double k00 = gbfem::toF64(K.k00), k01 = gbfem::toF64(K.k01);
    const double k02 = gbfem::toF64(K.k02), k11 = gbfem::toF64(K.k11);
    const double k12 = gbfem::toF64(K.k12), k22 = gbfem::toF64(K.k22);
    const double v[9] = {k00, k01, k02, k01, k11, k12, k02, k12, k22};
    if (a.jac_pos != nullptr)
    {
      const int d[3] = {d0, d1, d2};
#pragma unroll
      for (int i = 0; i < 3; ++i)
      {
        const int      rs = a.row_ptr[d[i]];
        const unsigned w  = a.jac_pos[3 * e + i];
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
          gbfem::redAdd(a.vals + rs + int((w >> (8 * j)) & 0xffu), v[3 * i + j]);
        }
      }
    }
    else
    {
      const int* jm = a.jac_map + 9 * e;
#pragma unroll
      for (int i = 0; i < 9; ++i)
      {
        gbfem::redAdd(a.vals + jm[i], v[i]);
      }
    }
  }
}

template <bool kF32, bool kSepConn>
__global__ void __launch_bounds__(256)
    p1VjpKernel(P1Args a, const double* __restrict__ lam, double* g_u,
                double* g_m)
{
  using T     = typename std::conditional<kF32, float, double>::type;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne)
  {
    return;
  }
  const int d0 = a.dofs[3 * e + 0], d1 = a.dofs[3 * e + 1], d2 = a.dofs[3 * e + 2];
  int       n0 = d0, n1 = d1, n2 = d2;
  if (kSepConn)
  {
    n0 = a.conn[3 * e + 0];
    n1 = a.conn[3 * e + 1];
    n2 = a.conn[3 * e + 2];
    if (static_cast<unsigned>(n0) >= static_cast<unsigned>(a.num_nodes)
        || static_cast<unsigned>(n1) >= static_cast<unsigned>(a.num_nodes)
        || static_cast<unsigned>(n2) >= static_cast<unsigned>(a.num_nodes))
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
      return;
    }
  }
  ElemK<T> K;
  if (!elementK<T>(a.coords[n0], a.coords[n1], a.coords[n2], a.kappa[e], K))
  {
    gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    return;
  }
  const T l0 = gbfem::fromF64<T>(lam[d0]), l1 = gbfem::fromF64<T>(lam[d1]);
  const T l2 = gbfem::fromF64<T>(lam[d2]);
  // K is symmetric: K^T lam = K lam.
  const T v0 = K.k00 * l0 + K.k01 * l1 + K.k02 * l2;
  const T v1 = K.k01 * l0 + K.k11 * l1 + K.k12 * l2;
  const T v2 = K.k02 * l0 + K.k12 * l1 + K.k22 * l2;
  if (g_u != nullptr)
  {
    gbfem::redAdd(g_u + d0, gbfem::toF64(v0));
    gbfem::redAdd(g_u + d1, gbfem::toF64(v1));
    gbfem::redAdd(g_u + d2, gbfem::toF64(v2));
  }
  if (g_m != nullptr)
  {
    // lam^T K u = (K lam) . u
    const T u0 = gbfem::fromF64<T>(a.u[d0]), u1 = gbfem::fromF64<T>(a.u[d1]);
    const T u2 = gbfem::fromF64<T>(a.u[d2]);
    g_m[e]     = gbfem::toF64(v0 * u0 + v1 * u1 + v2 * u2);
  }
}

template <bool kF32, bool kSep>
void launchAssemble(const P1Args& a, bool load, bool jac, cudaStream_t s)
{
  const unsigned blocks = gbfem::blocksFor(a.ne, 256);
  if (load && jac)
  {
    p1AssembleKernel<kF32, kSep, true, true><<<blocks, 256, 0, s>>>(a);
  }
  else if (load)
  {
    p1AssembleKernel<kF32, kSep, true, false><<<blocks, 256, 0, s>>>(a);
  }
  else if (jac)
  {
    p1AssembleKernel<kF32, kSep, false, true><<<blocks, 256, 0, s>>>(a);
  }
  else
  {
    p1AssembleKernel<kF32, kSep, false, false><<<blocks, 256, 0, s>>>(a);
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
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_MIXED,
            "unknown precision mode");
    require((reinterpret_cast<uintptr_t>(coords) & 15) == 0,
            "Geometry coordinates must be 16-byte aligned");
    cudaStream_t s = asStream(stream);
    a.f            = f_nodal;
    a.res          = res;
    a.vals         = vals;
    cudaCheck(cudaMemsetAsync(res, 0, sizeof(double) * map->num_res, s),
              "residual zero");
    if (vals != nullptr && map->nnz > 0)
    {
      cudaCheck(cudaMemsetAsync(vals, 0, sizeof(double) * map->nnz, s),
                "matrix zero");
    }
    if (a.ne == 0)
    {
      return;
    }
    const bool load = f_nodal != nullptr, jac = vals != nullptr;
    const bool sep  = conn != nullptr;
    if (precision == GBFEM_PREC_FP64 || (precision == GBFEM_PREC_MIXED && !jac))
    {
      sep ? launchAssemble<false, true>(a, load, jac, s)
          : launchAssemble<false, false>(a, load, jac, s);
    }
    else if (precision == GBFEM_PREC_FP32_QUAD)
    {
      sep ? launchAssemble<true, true>(a, load, jac, s)
          : launchAssemble<true, false>(a, load, jac, s);
    }
    else
    {
      // Jacobian from FP32 quadrature, residual from FP64 element math
      const unsigned blocks = blocksFor(a.ne, 256);
      if (sep)
      {
        p1AssembleKernel<true, true, false, true, false><<<blocks, 256, 0, s>>>(a);
      }
      else
      {
        p1AssembleKernel<true, false, false, true, false><<<blocks, 256, 0, s>>>(a);
      }
      sep ? launchAssemble<false, true>(a, load, false, s)
          : launchAssemble<false, false>(a, load, false, s);
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
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_MIXED,
            "unknown precision mode");
    cudaStream_t s = asStream(stream);
    if (g_u != nullptr)
    {
      cudaCheck(cudaMemsetAsync(g_u, 0, sizeof(double) * map->num_states, s),
                "VJP state zero");
    }
    if (a.ne == 0 || (g_u == nullptr && g_m == nullptr))
    {
      return;
    }
    const unsigned blocks = blocksFor(a.ne, 256);
    const bool     sep    = conn != nullptr;
    if (precision != GBFEM_PREC_FP32_QUAD)
    {
      sep ? p1VjpKernel<false, true><<<blocks, 256, 0, s>>>(a, lam, g_u, g_m)
          : p1VjpKernel<false, false><<<blocks, 256, 0, s>>>(a, lam, g_u, g_m);
    }
    else
    {
      sep ? p1VjpKernel<true, true><<<blocks, 256, 0, s>>>(a, lam, g_u, g_m)
          : p1VjpKernel<true, false><<<blocks, 256, 0, s>>>(a, lam, g_u, g_m);
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
