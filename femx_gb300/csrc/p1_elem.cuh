// p1_elem.cuh — device code of the kappa-weighted P1 Poisson element, shared
// by the standalone kernels (p1.cu) and the batched persistent kernel
// (batch.cu). See p1.cu for the formulation.
#pragma once

#include <type_traits>

#include "dfloat.cuh"
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
// evaluation of the element stiffness. kPlain: coloured assembly, plain
// read-add-writes instead of FP64 reductions.
// kArith: the element arithmetic, 0 = FP64, 1 = FP32 (quadrature),
// 2 = double-float (FP64-accurate, on the FP32 pipe; residual and Jacobian
// only).
template <int kArith, bool kSepConn, bool kLoad, bool kJac, bool kRes, bool kVjp,
          bool kPlain = false>
__device__ __forceinline__ void p1Element(const P1Args& a, int e)
{
  static_assert(kArith != 2 || !kVjp, "the double-float P1 element has no VJP");
  constexpr bool kF32 = kArith == 1;
  using T = typename std::conditional<
      kArith == 2, gbfem::Dd, typename std::conditional<kF32, float, double>::type>::type;
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
  // FP32: the element is formed for kappa = 1 (geometry only; exact on a
  // uniform mesh, whose edge vectors, determinant and h_i . h_j are exact in
  // FP32), kappa is applied afterwards: in FP32 for the residual and the
  // Jacobian, in FP64 for the gradients.
  const double kap = a.kappa[e];
  ElemK<T>     K;
  if (!elementK<T>(a.coords[n0], a.coords[n1], a.coords[n2], kF32 ? 1.0 : kap, K))
  {
    gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    return;
  }
  ElemK<T> Kh = K;
  if constexpr (kF32)
  {
    const T kf = gbfem::fromF64<T>(kap);
    K.k00 *= kf;
    K.k01 *= kf;
    K.k02 *= kf;
    K.k11 *= kf;
    K.k12 *= kf;
    K.k22 *= kf;
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
    gbfem::addTo<kPlain>(a.res + d0, gbfem::toF64(r0));
    gbfem::addTo<kPlain>(a.res + d1, gbfem::toF64(r1));
    gbfem::addTo<kPlain>(a.res + d2, gbfem::toF64(r2));
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
          gbfem::addTo<kPlain>(a.vals + rs + int((w >> (8 * j)) & 0xffu), v[3 * i + j]);
        }
      }
    }
    else
    {
      const int* jm = a.jac_map + 9 * e;
#pragma unroll
      for (int i = 0; i < 9; ++i)
      {
        gbfem::addTo<kPlain>(a.vals + jm[i], v[i]);
      }
    }
  }
  if constexpr (kVjp)
  {
    gbfem::awaitPrerequisites(); // g_u's zero fill may still be running
    if constexpr (kF32)
    {
      // The gradient reduction in FP64 (the FP32 element's geometry widened
      // exactly, kappa, adjoint and state in FP64): FP32 rounding here would
      // put ~1e-7 relative noise on every element's gradient, which
      // directional derivatives over many elements amplify by cancellation.
      const double h00 = gbfem::f32ToF64(Kh.k00), h01 = gbfem::f32ToF64(Kh.k01);
      const double h02 = gbfem::f32ToF64(Kh.k02), h11 = gbfem::f32ToF64(Kh.k11);
      const double h12 = gbfem::f32ToF64(Kh.k12), h22 = gbfem::f32ToF64(Kh.k22);
      const double l0 = a.lam[d0], l1 = a.lam[d1], l2 = a.lam[d2];
      const double v0 = h00 * l0 + h01 * l1 + h02 * l2;
      const double v1 = h01 * l0 + h11 * l1 + h12 * l2;
      const double v2 = h02 * l0 + h12 * l1 + h22 * l2;
      if (a.g_u != nullptr)
      {
        gbfem::addTo<kPlain>(a.g_u + d0, kap * v0);
        gbfem::addTo<kPlain>(a.g_u + d1, kap * v1);
        gbfem::addTo<kPlain>(a.g_u + d2, kap * v2);
      }
      if (a.g_m != nullptr)
      {
        a.g_m[e] = kap * (v0 * a.u[d0] + v1 * a.u[d1] + v2 * a.u[d2]);
      }
    }
    else
    {
      const T l0 = a.lam[d0], l1 = a.lam[d1], l2 = a.lam[d2];
      // K is symmetric: K^T lam = K lam.
      const T v0 = K.k00 * l0 + K.k01 * l1 + K.k02 * l2;
      const T v1 = K.k01 * l0 + K.k11 * l1 + K.k12 * l2;
      const T v2 = K.k02 * l0 + K.k12 * l1 + K.k22 * l2;
      if (a.g_u != nullptr)
      {
        gbfem::addTo<kPlain>(a.g_u + d0, v0);
        gbfem::addTo<kPlain>(a.g_u + d1, v1);
        gbfem::addTo<kPlain>(a.g_u + d2, v2);
      }
      if (a.g_m != nullptr)
      {
        // lam^T K u = (K lam) . u
        a.g_m[e] = v0 * a.u[d0] + v1 * a.u[d1] + v2 * a.u[d2];
      }
    }
  }
}

} // namespace
