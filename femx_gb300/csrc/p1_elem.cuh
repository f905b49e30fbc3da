// p1_elem.cuh — device code of the kappa-weighted P1 Poisson element, shared
// by the standalone kernels (p1.cu) and the batched persistent kernel
// (batch.cu). See p1.cu for the formulation.
#pragma once

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
  const double*        lam; // adjoint for the fused VJP, or null
  double*              g_u; // K^T lam accumulated here (null: skipped)
  double*              g_m; // lam_e^T K_e u_e per element (null: skipped)
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
  T s;
  if constexpr (std::is_same<T, double>::value)
  {
    s = kappa * 0.5 * gbfem::rcpF64(adet);
  }
  else
  {
    s = gbfem::fromF64<T>(kappa) * T(0.5) / adet;
  }
  K.k01       = s * (h0x * by - h0y * bx);
  K.k02       = s * (-h0x * ay + h0y * ax);
  K.k12       = s * (-by * ay - bx * ax);
  K.k00       = -(K.k01 + K.k02);
  K.k11       = -(K.k01 + K.k12);
  K.k22       = -(K.k02 + K.k12);
  K.adet      = adet;
  return true;
}

// One element: residual (kRes), Jacobian scatter (kJac) and the fused
// residual VJPs (kVjp: K^T lam into g_u, lam^T K u into g_m), all from one
// evaluation of the element stiffness.
template <bool kF32, bool kSepConn, bool kLoad, bool kJac, bool kRes, bool kVjp>
__device__ __forceinline__ void p1Element(const P1Args& a, int e)
{
  using T = typename std::conditional<kF32, float, double>::type;
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
  // the outputs are zero-filled by the kernel this one may overlap
  gbfem::awaitPrerequisites();
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
  if (kVjp)
  {
    gbfem::awaitPrerequisites(); // g_u's zero fill may still be running
    const T l0 = gbfem::fromF64<T>(a.lam[d0]), l1 = gbfem::fromF64<T>(a.lam[d1]);
    const T l2 = gbfem::fromF64<T>(a.lam[d2]);
    // K is symmetric: K^T lam = K lam.
    const T v0 = K.k00 * l0 + K.k01 * l1 + K.k02 * l2;
    const T v1 = K.k01 * l0 + K.k11 * l1 + K.k12 * l2;
    const T v2 = K.k02 * l0 + K.k12 * l1 + K.k22 * l2;
    if (a.g_u != nullptr)
    {
      gbfem::redAdd(a.g_u + d0, gbfem::toF64(v0));
      gbfem::redAdd(a.g_u + d1, gbfem::toF64(v1));
      gbfem::redAdd(a.g_u + d2, gbfem::toF64(v2));
    }
    if (a.g_m != nullptr)
    {
      // lam^T K u = (K lam) . u
      const T w0 = gbfem::fromF64<T>(a.u[d0]), w1 = gbfem::fromF64<T>(a.u[d1]);
      const T w2 = gbfem::fromF64<T>(a.u[d2]);
      a.g_m[e]   = gbfem::toF64(v0 * w0 + v1 * w1 + v2 * w2);
    }
  }
}


} // namespace
