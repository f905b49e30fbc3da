// navier.cu — femx's equal-order GLS Navier-Stokes time operator on P1
// triangles (NavierOperator, femx/model/ns/Components.hpp:330-577), the
// operator femx's NS time path assembles with its CUDA time kernel
// (CudaAssembly.hpp:215-300, :367-413) and differentiates with Enzyme for
// the history VJP (Components.cpp:67-125, Components.cu:25-98).
//
// One step: R(hist, nxt) = K(hist) nxt - F(hist), K the next-state Jacobian;
// Crank-Nicolson in time with AB2-extrapolated advection velocity
// adv = 1.5 u^n - 0.5 u^(n-1) (u^n at step 0 or with one history state);
// GLS stabilisation tau = (4/dt^2 + (2|u|/h)^2 + (4 nu/h^2)^2)^(-1/2) with
// femx's streamline element length h. Local DOFs: velocity (node, comp) at
// 2 node + comp, then pressure at 6 + node; order-2 rule (3 points).
//
// GB300 formulation (FP64 throughout: this is the drop-in). The FP64 pipe is
// the bound, so the element is factorised instead of evaluated row by row
// (femx re-evaluates every quadrature point for every row): on the affine
// triangle the shape gradients g_i and grad u^n are constant, and with
//   s_i = N_i + tau dv_i,  phi_j = (2/dt) N_j + dv_j,  dv_i = adv . g_i,
//   w_c = u_c/dt - ag_c/2  (ag = (adv . grad) u^n)
// every block of the element matrix is a short sum over the 3 points:
//   K(ic,jc)  = sum_q Jw [rho/2 s_i phi_j + mu/2 g_i.g_j]
//   K(ic,pj)  = sum_q Jw [-g_i[c] N_j + tau dv_i g_j[c]]
//   K(pi,jd)  = sum_q Jw [N_i g_j[d] + tau/2 g_i[d] phi_j]
//   K(pi,pj)  = sum_q Jw tau/rho g_i.g_j
//   F(ic)     = sum_q Jw [rho s_i w_c - mu/2 g_i . grad_c],  F(pi) = sum_q Jw tau g_i . w
// — algebraically the terms of evalPhysicsRow, at about 450 FP64
// operations per element. One thread owns one element (all 32 lanes busy);
// it scatter-adds the 81 entries and 9 residual terms with FP64 reductions.
// The history VJP is reverse mode written out by hand (no Enzyme): per point
// the adjoint contractions give dL/d(u, grad u, adv, tau), tau's dependence
// on u (through |u| and the streamline length) is chained in, and the 12
// velocity history entries of both lags are reduced per element.
#include "maps.cuh"

namespace
{

using gbfem::DeviceStatus;

constexpr int kThreads = 128;
constexpr int kQ       = 3;
constexpr int kDofs    = 9;

// order-2 rule points (GaussQuadrature.hpp:189-198) and P1 basis values there,
// formed as femx forms them (N = 1 - r - s, r, s)
__device__ __forceinline__ double basisN(int q, int in)
{
  const double r = q == 1 ? 2.0 / 3.0 : 1.0 / 6.0;
  const double s = q == 2 ? 2.0 / 3.0 : 1.0 / 6.0;
  return in == 0 ? 1.0 - r - s : (in == 1 ? r : s);
}
constexpr double kW = 1.0 / 6.0;

struct NsArgs
{
  int                  ne, num_nodes, num_states;
  const int*           dofs;  // [ne][9]
  const int*           conn;  // [ne][3]
  const double2*       coords;
  double               rho, mu, dt;
  // host-side constants, so that no kernel divides by them: 1/dt, 2/dt,
  // (2/dt)^2, rho/dt, 1/rho, nu = mu/rho
  double               inv_dt, two_dt, time2, rho_dt, inv_rho, nu;
  int                  step, num_hist;
  const double*        hist;  // [num_hist][num_states]
  const double*        nxt;
  const double*        adj;   // VJP only
  double*              res;
  double*              vals;
  double*              out;   // VJP only: [num_hist][num_states]
  const int*           row_ptr;
  const unsigned char* jac_pos; // column-major, stride 16, or null
  const int*           jac_map;
  DeviceStatus*        status;
};

// One element's inputs, geometry and the history-only per-element fields.
struct NsElem
{
  int    dofs[kDofs];
  double h0[6], an[6];   // lag-0 velocity, AB2 advection velocity at the nodes
  double g[3][2];        // dN_i/dx_d, constant on the affine triangle
  double jxw;            // |det| w, equal at the three points
  double grad[2][2];     // grad u^n (constant)
  bool   ab2;
};

// Geometry as ElementValues forms it (J = sum x dN^/dr, invJ, dN/dx).
__device__ bool loadElement(const NsArgs& a, int e, NsElem& E)
{
  int n[3];
  for (int k = 0; k < 3; ++k)
  {
    n[k] = a.conn[3 * e + k];
    if (static_cast<unsigned>(n[k]) >= static_cast<unsigned>(a.num_nodes))
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
      return false;
    }
  }
  const double2 x0 = a.coords[n[0]], x1 = a.coords[n[1]], x2 = a.coords[n[2]];
  const double  J0 = x0.x * -1.0 + x1.x * 1.0 + x2.x * 0.0;
  const double  J1 = x0.x * -1.0 + x1.x * 0.0 + x2.x * 1.0;
  const double  J2 = x0.y * -1.0 + x1.y * 1.0 + x2.y * 0.0;
  const double  J3 = x0.y * -1.0 + x1.y * 0.0 + x2.y * 1.0;
  const double  det = J0 * J3 - J1 * J2;
  if (!(fabs(det) >= 1.0e-30))
  {
    gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    return false;
  }
  const double inv = gbfem::rcpF64(det);
  const double i0 = J3 * inv, i1 = -J1 * inv, i2 = -J2 * inv, i3 = J0 * inv;
  // dN/dx_d = sum_b dN^/dr_b invJ[b][d], dN^/dr = (-1,-1), (1,0), (0,1)
  E.g[0][0] = -i0 - i2;
  E.g[0][1] = -i1 - i3;
  E.g[1][0] = i0;
  E.g[1][1] = i1;
  E.g[2][0] = i2;
  E.g[2][1] = i3;
  E.jxw     = fabs(det) * kW;
  for (int k = 0; k < kDofs; ++k)
  {
    E.dofs[k] = a.dofs[kDofs * e + k];
  }
  E.ab2 = a.step > 0 && a.num_hist > 1;
  for (int k = 0; k < 6; ++k)
  {
    const double v = a.hist[E.dofs[k]];
    E.h0[k]        = v;
    E.an[k] = E.ab2 ? 1.5 * v - 0.5 * a.hist[static_cast<long long>(a.num_states) + E.dofs[k]]
                    : v;
  }
  for (int c = 0; c < 2; ++c)
  {
    for (int d = 0; d < 2; ++d)
    {
      E.grad[c][d] = E.g[0][d] * E.h0[c] + E.g[1][d] * E.h0[2 + c] + E.g[2][d] * E.h0[4 + c];
    }
  }
  return true;
}

// Point state: u, adv, ag = (adv . grad) u, tau and femx's streamline length
// pieces (elemLength, Components.hpp:273-327; evalQp :330-395).
struct NsQp
{
  double N[3], u[2], adv[2], ag[2], tau, speed, h, sum, dir[2];
  double inv_speed, inv_h; // 1/|u| (when not fallback), 1/h = sum/2 (when h > 0)
  bool   fallback;
};

__device__ __forceinline__ void pointState(const NsArgs& a, const NsElem& E, int q, NsQp& P)
{
  for (int i = 0; i < 3; ++i)
  {
    P.N[i] = basisN(q, i);
  }
  for (int c = 0; c < 2; ++c)
  {
    P.u[c]   = P.N[0] * E.h0[c] + P.N[1] * E.h0[2 + c] + P.N[2] * E.h0[4 + c];
    P.adv[c] = P.N[0] * E.an[c] + P.N[1] * E.an[2 + c] + P.N[2] * E.an[4 + c];
  }
  for (int c = 0; c < 2; ++c)
  {
    P.ag[c] = E.grad[c][0] * P.adv[0] + E.grad[c][1] * P.adv[1];
  }
  // The same quantities as femx's evalQp/elemLength with the divisions and
  // square roots recast: |u| = s2 / sqrt(s2) from one reciprocal square root,
  // u/|u| as a product, h = 2/sum enters only as (2|u|/h) = |u| sum and
  // (4 nu/h^2) = nu sum^2; tau = 1/sqrt(...) from rsqrtF64 (the FP64 pipe
  // is GB300's scarce resource; results agree with the divided forms to a
  // few ulps).
  const double s2  = P.u[0] * P.u[0] + P.u[1] * P.u[1];
  const double is  = s2 > 0.0 ? gbfem::rsqrtF64(s2) : 0.0;
  const double speed = s2 * is;
  P.fallback         = !(speed > 1.0e-10);
  P.inv_speed        = is;
  if (!P.fallback)
  {
    P.dir[0] = P.u[0] * is;
    P.dir[1] = P.u[1] * is;
  }
  else
  {
    P.dir[0] = P.dir[1] = 0.70710678118654752440; // 1/sqrt(2)
  }
  double sum = 0.0;
  for (int i = 0; i < 3; ++i)
  {
    sum += fabs(P.dir[0] * E.g[i][0] + P.dir[1] * E.g[i][1]);
  }
  double h = 0.0, flow = 0.0, diff = 0.0;
  P.inv_h  = 0.0;
  if (sum > 1.0e-14)
  {
    h          = 2.0 * gbfem::rcpF64(sum);
    P.inv_h    = 0.5 * sum;
    const double fs = speed * sum, ds = a.nu * sum * sum;
    flow       = fs * fs;
    diff       = ds * ds;
  }
  P.tau   = gbfem::rsqrtF64(a.time2 + flow + diff);
  P.speed = speed;
  P.h     = h;
  P.sum   = sum;
}

__device__ __forceinline__ int csrSlot(const NsArgs& a, int e, const int* rs, int i, int j,
                                       const uint4* pw)
{
  if (a.jac_pos != nullptr)
  {
    const unsigned w = (&pw[j].x)[i >> 2];
    return rs[i] + static_cast<int>((w >> (8 * (i & 3))) & 0xffu);
  }
  return a.jac_map[81LL * e + kDofs * i + j];
}

template <bool kJac>
__global__ void __launch_bounds__(kThreads) nsAssembleKernel(NsArgs a)
{
  const int e = blockIdx.x * kThreads + threadIdx.x;
  if (e >= a.ne)
  {
    return;
  }
  NsElem E;
  if (!loadElement(a, e, E))
  {
    return; // reported through the status word; the element adds nothing
  }
  const double rho = a.rho, mu = a.mu;
  double       Ss[3][3] = {}, T[3] = {}, Pj[3] = {}, Fv[3][2] = {}, V[2] = {}, Tt = 0.0;
  double       Nsum[3] = {};
  for (int q = 0; q < kQ; ++q)
  {
    NsQp P;
    pointState(a, E, q, P);
    double dv[3], s[3], phi[3];
    for (int i = 0; i < 3; ++i)
    {
      dv[i]  = E.g[i][0] * P.adv[0] + E.g[i][1] * P.adv[1];
      s[i]   = P.N[i] + P.tau * dv[i];
      phi[i] = a.two_dt * P.N[i] + dv[i];
      Nsum[i] += P.N[i];
    }
    const double w[2] = {P.u[0] * a.inv_dt - 0.5 * P.ag[0], P.u[1] * a.inv_dt - 0.5 * P.ag[1]};
    for (int i = 0; i < 3; ++i)
    {
      for (int j = 0; j < 3; ++j)
      {
        Ss[i][j] += s[i] * phi[j];
      }
      T[i] += P.tau * dv[i];
      Pj[i] += P.tau * phi[i];
      Fv[i][0] += s[i] * w[0];
      Fv[i][1] += s[i] * w[1];
    }
    V[0] += P.tau * w[0];
    V[1] += P.tau * w[1];
    Tt += P.tau;
  }
  const double Jw = E.jxw, J3 = 3.0 * E.jxw;
  double       x[kDofs];
  for (int k = 0; k < kDofs; ++k)
  {
    x[k] = a.nxt[E.dofs[k]];
  }
  int   rs[kDofs];
  uint4 pw[kDofs];
  if (kJac)
  {
    for (int k = 0; k < kDofs; ++k)
    {
      rs[k] = a.row_ptr[E.dofs[k]];
      if (a.jac_pos != nullptr)
      {
        pw[k] = *reinterpret_cast<const uint4*>(a.jac_pos + (9LL * e + k) * 16);
      }
    }
  }
  // velocity rows (i, c)
  // the outputs are zero-filled by the kernel this one may overlap
  gbfem::awaitPrerequisites();
  for (int i = 0; i < 3; ++i)
  {
    double kvv[3], kvp[2][3];
    for (int j = 0; j < 3; ++j)
    {
      const double gd = E.g[i][0] * E.g[j][0] + E.g[i][1] * E.g[j][1];
      kvv[j]          = 0.5 * rho * Jw * Ss[i][j] + 0.5 * mu * J3 * gd;
      for (int c = 0; c < 2; ++c)
      {
        kvp[c][j] = -E.g[i][c] * Jw * Nsum[j] + E.g[j][c] * Jw * T[i];
      }
    }
    for (int c = 0; c < 2; ++c)
    {
      const double gradc = E.g[i][0] * E.grad[c][0] + E.g[i][1] * E.grad[c][1];
      double       r     = -(rho * Jw * Fv[i][c] - 0.5 * mu * J3 * gradc);
      for (int j = 0; j < 3; ++j)
      {
        r += kvv[j] * x[2 * j + c] + kvp[c][j] * x[6 + j];
      }
      const int row = 2 * i + c;
      gbfem::redAdd(a.res + E.dofs[row], r);
      if (kJac)
      {
        for (int j = 0; j < 3; ++j)
        {
          gbfem::redAdd(a.vals + csrSlot(a, e, rs, row, 2 * j + c, pw), kvv[j]);
          gbfem::redAdd(a.vals + csrSlot(a, e, rs, row, 6 + j, pw), kvp[c][j]);
        }
        // the cross-component entries (j, 1 - c) are structurally zero
      }
    }
  }
  // pressure rows i
  for (int i = 0; i < 3; ++i)
  {
    const int row = 6 + i;
    double    r   = -(Jw * (E.g[i][0] * V[0] + E.g[i][1] * V[1]));
    for (int j = 0; j < 3; ++j)
    {
      const double gd  = E.g[i][0] * E.g[j][0] + E.g[i][1] * E.g[j][1];
      const double kpp = gd * Jw * Tt * a.inv_rho;
      r += kpp * x[6 + j];
      for (int dd = 0; dd < 2; ++dd)
      {
        const double kpv = E.g[j][dd] * Jw * Nsum[i] + 0.5 * E.g[i][dd] * Jw * Pj[j];
        r += kpv * x[2 * j + dd];
        if (kJac)
        {
          gbfem::redAdd(a.vals + csrSlot(a, e, rs, row, 2 * j + dd, pw), kpv);
        }
      }
      if (kJac)
      {
        gbfem::redAdd(a.vals + csrSlot(a, e, rs, row, 6 + j, pw), kpp);
      }
    }
    gbfem::redAdd(a.res + E.dofs[row], r);
  }
}

// History VJP: out[lag][dof] += d/d hist[lag][dof] of sum_rows adj . R.
// With the adjoint and next-state fields at a point (X, A, Xp, AP; their
// constant gradients Gx, GA, Gp, GAP), the adjoint-weighted integrand is
//   E = sum_c [rho/dt A_c (X_c - u_c) + rho/2 A_c (Dv_c + ag_c)
//              + mu/2 GA_c.(Gx_c + grad_c) + tau rho/dt Av_c (X_c - u_c)
//              + tau rho/2 Av_c (Dv_c + ag_c) - GA_c[c] Xp + tau Av_c Gp_c]
//     + AP div(X) + tau GAP.(X/dt + Dv/2 + Gp/rho - u/dt + ag/2),
// Dv_c = adv.Gx_c, Av_c = adv.GA_c; its partials in (u, grad, adv, tau) are
// chained back to the nodal history values.
// An explicit minimum of one resident block lets the compiler use up to 255
// registers (201 without it): the reverse sweep then keeps its tape in
// registers, 287 against 342 us at 256x256.
__global__ void __launch_bounds__(kThreads, 1) nsHistVjpKernel(NsArgs a)
{
  const int e = blockIdx.x * kThreads + threadIdx.x;
  if (e >= a.ne)
  {
    return;
  }
  NsElem E;
  if (!loadElement(a, e, E))
  {
    return;
  }
  const double rho = a.rho, mu = a.mu, nu = a.nu;
  const double idt = a.inv_dt, rdt = a.rho_dt, irho = a.inv_rho;
  double       x[kDofs], ad[kDofs];
  for (int k = 0; k < kDofs; ++k)
  {
    x[k]  = a.nxt[E.dofs[k]];
    ad[k] = a.adj[E.dofs[k]];
  }
  double Gx[2][2], GA[2][2], Gp[2], GAP[2];
  for (int d = 0; d < 2; ++d)
  {
    for (int c = 0; c < 2; ++c)
    {
      Gx[c][d] = E.g[0][d] * x[c] + E.g[1][d] * x[2 + c] + E.g[2][d] * x[4 + c];
      GA[c][d] = E.g[0][d] * ad[c] + E.g[1][d] * ad[2 + c] + E.g[2][d] * ad[4 + c];
    }
    Gp[d]  = E.g[0][d] * x[6] + E.g[1][d] * x[7] + E.g[2][d] * x[8];
    GAP[d] = E.g[0][d] * ad[6] + E.g[1][d] * ad[7] + E.g[2][d] * ad[8];
  }
  double SU[3][2] = {}, SA[3][2] = {}, SG[2][2] = {};
  for (int q = 0; q < kQ; ++q)
  {
    NsQp P;
    pointState(a, E, q, P);
    const double tau = P.tau;
    double       X[2], A[2], Xp = 0.0, AP = 0.0;
    for (int c = 0; c < 2; ++c)
    {
      X[c] = P.N[0] * x[c] + P.N[1] * x[2 + c] + P.N[2] * x[4 + c];
      A[c] = P.N[0] * ad[c] + P.N[1] * ad[2 + c] + P.N[2] * ad[4 + c];
    }
    for (int j = 0; j < 3; ++j)
    {
      Xp += P.N[j] * x[6 + j];
      AP += P.N[j] * ad[6 + j];
    }
    double Dv[2], Av[2];
    for (int c = 0; c < 2; ++c)
    {
      Dv[c] = P.adv[0] * Gx[c][0] + P.adv[1] * Gx[c][1];
      Av[c] = P.adv[0] * GA[c][0] + P.adv[1] * GA[c][1];
    }
    double Ptau = 0.0, W[2], PAv[2], du[2];
    for (int c = 0; c < 2; ++c)
    {
      const double xm = X[c] - P.u[c], dg = Dv[c] + P.ag[c];
      Ptau += rdt * Av[c] * xm + 0.5 * rho * Av[c] * dg + Av[c] * Gp[c];
      Ptau += GAP[c] * (X[c] * idt + 0.5 * Dv[c] + Gp[c] * irho - P.u[c] * idt + 0.5 * P.ag[c]);
      W[c]   = 0.5 * rho * A[c] + 0.5 * tau * rho * Av[c] + 0.5 * tau * GAP[c];
      PAv[c] = tau * rdt * xm + 0.5 * tau * rho * dg + tau * Gp[c];
      du[c]  = -rdt * A[c] - tau * rdt * Av[c] - tau * idt * GAP[c];
    }
    // tau(u) through |u| and h(u/|u|): dtau = -tau^3/2 d(flow + diff)
    if (P.h > 0.0)
    {
      double dh[2] = {0.0, 0.0};
      if (!P.fallback)
      {
        for (int i = 0; i < 3; ++i)
        {
          const double gr = P.dir[0] * E.g[i][0] + P.dir[1] * E.g[i][1];
          const double sg = gr >= 0.0 ? 1.0 : -1.0;
          dh[0] += sg * (E.g[i][0] - gr * P.dir[0]);
          dh[1] += sg * (E.g[i][1] - gr * P.dir[1]);
        }
        const double f = -0.5 * (P.h * P.h) * P.inv_speed; // -2/(sum^2 |u|), 1/sum = h/2
        dh[0] *= f;
        dh[1] *= f;
      }
      const double h = P.h, t3 = tau * tau * tau;
      const double ih = P.inv_h, ih3 = ih * ih * ih, ih5 = ih3 * ih * ih;
      for (int c = 0; c < 2; ++c)
      {
        const double dflow = 8.0 * (P.u[c] * h - P.speed * P.speed * dh[c]) * ih3;
        const double ddiff = -64.0 * nu * nu * dh[c] * ih5;
        du[c] += Ptau * (-0.5 * t3 * (dflow + ddiff));
      }
    }
    for (int c = 0; c < 2; ++c)
    {
      double da = 0.0;
      for (int cc = 0; cc < 2; ++cc)
      {
        da += W[cc] * (E.grad[cc][c] + Gx[cc][c]) + PAv[cc] * GA[cc][c];
      }
      for (int i = 0; i < 3; ++i)
      {
        SU[i][c] += P.N[i] * du[c];
        SA[i][c] += P.N[i] * da;
      }
      for (int d = 0; d < 2; ++d)
      {
        SG[c][d] += 0.5 * mu * GA[c][d] + W[c] * P.adv[d];
      }
    }
  }
  const double Jw  = E.jxw;
  const double al0 = E.ab2 ? 1.5 : 1.0;
  gbfem::awaitPrerequisites(); // the output's zero fill may still be running
  for (int i = 0; i < 3; ++i)
  {
    for (int c = 0; c < 2; ++c)
    {
      const int    dof = E.dofs[2 * i + c];
      const double v0 =
          Jw * (SU[i][c] + E.g[i][0] * SG[c][0] + E.g[i][1] * SG[c][1] + al0 * SA[i][c]);
      gbfem::redAdd(a.out + dof, v0);
      if (E.ab2)
      {
        gbfem::redAdd(a.out + static_cast<long long>(a.num_states) + dof, Jw * -0.5 * SA[i][c]);
      }
    }
  }
}

NsArgs makeArgs(const gbfem_assembly_map* map, int num_nodes, const double* coords,
                const int* conn, double rho, double mu, double dt, int step, int num_hist,
                const double* hist, const double* nxt)
{
  NsArgs a{};
  a.ne         = map->num_elems;
  a.num_nodes  = num_nodes;
  a.num_states = map->num_states;
  a.dofs       = map->state_dofs;
  a.conn       = conn;
  a.coords     = reinterpret_cast<const double2*>(coords);
  a.rho        = rho;
  a.mu         = mu;
  a.dt         = dt;
  a.inv_dt     = 1.0 / dt;
  a.two_dt     = 2.0 / dt;
  a.time2      = (2.0 / dt) * (2.0 / dt);
  a.rho_dt     = rho / dt;
  a.inv_rho    = 1.0 / rho;
  a.nu         = mu / rho;
  a.step       = step;
  a.num_hist   = num_hist;
  a.hist       = hist;
  a.nxt        = nxt;
  a.row_ptr    = map->row_ptr;
  a.jac_pos    = map->pos_stride == 16 ? map->jac_pos : nullptr;
  a.jac_map    = map->jac_map;
  a.status     = map->status;
  return a;
}

void checkCommon(const gbfem_assembly_map* map, int num_nodes, const double* coords,
                 const int* conn, double rho, double mu, double dt, int num_hist,
                 const double* hist, const double* nxt)
{
  using gbfem::require;
  require(map != nullptr, "AssemblyMap handle is null");
  require(map->num_elems == 0 || (map->uniform_res == 9 && map->uniform_state == 9),
          "Navier operator expects nine DOFs per P1 triangle");
  require(map->num_res == map->num_states && map->same_dofs,
          "Navier assembly expects identical residual and state DOF tables");
  require(num_hist > 0, "Time assembly state dimensions do not match AssemblyMap");
  require(num_nodes >= 0, "Geometry node count must be non-negative");
  require(map->num_elems == 0 || (coords && conn && hist && nxt),
          "Assembly inputs must not be null");
  require(rho > 0.0 && mu > 0.0 && dt > 0.0,
          "NavierStokesModel requires positive density, viscosity and time step");
  require((reinterpret_cast<uintptr_t>(coords) & 15) == 0,
          "Geometry coordinates must be 16-byte aligned");
}

} // namespace

extern "C" int gbfem_assemble_navier(const gbfem_assembly_map* map, int num_nodes,
                                     const double* coords, const int* conn, double rho,
                                     double mu, double dt, int step, int num_hist,
                                     int wrt_hist_lag, const double* hist, const double* nxt,
                                     double* res, double* vals, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    checkCommon(map, num_nodes, coords, conn, rho, mu, dt, num_hist, hist, nxt);
    require(wrt_hist_lag >= -1 && wrt_hist_lag < num_hist,
            "Time assembly variable block is invalid");
    require(res != nullptr, "Assembly residual output is null");
    require(res != hist && res != nxt && vals != hist && vals != nxt
                && (vals == nullptr || res != vals),
            "Time assembly outputs must not alias inputs or each other");
    cudaStream_t s = asStream(stream);
    zeroForNext(vals, vals != nullptr ? map->nnz : 0, res, map->num_res, s);
    if (map->num_elems == 0)
    {
      return;
    }
    NsArgs a = makeArgs(map, num_nodes, coords, conn, rho, mu, dt, step, num_hist, hist, nxt);
    a.res    = res;
    // femx's operator has no history Jacobian rows (history derivatives are
    // VJPs, Components.hpp:412-435): a history block is the zero matrix
    a.vals   = wrt_hist_lag < 0 ? vals : nullptr;
    const unsigned blocks = blocksFor(a.ne, kThreads);
    a.vals != nullptr ? launchDependent(nsAssembleKernel<true>, blocks, kThreads, s, a)
                      : launchDependent(nsAssembleKernel<false>, blocks, kThreads, s, a);
    cudaCheck(cudaGetLastError(), "Navier assembly launch");
  });
}

extern "C" int gbfem_vjp_navier_hist(const gbfem_assembly_map* map, int num_nodes,
                                     const double* coords, const int* conn, double rho,
                                     double mu, double dt, int step, int num_hist,
                                     const double* hist, const double* nxt, const double* adj,
                                     double* out, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    checkCommon(map, num_nodes, coords, conn, rho, mu, dt, num_hist, hist, nxt);
    require(map->num_elems == 0 || adj != nullptr, "VJP adjoint must not be null");
    require(out != nullptr, "VJP output is null");
    require(out != hist && out != nxt && out != adj, "VJP output must not alias its inputs");
    cudaStream_t s = asStream(stream);
    // the VJP kernel is launched as a dependent of this zero fill
    zeroForNext(out, num_hist * static_cast<long long>(map->num_states), nullptr, 0, s);
    if (map->num_elems == 0)
    {
      return;
    }
    NsArgs a = makeArgs(map, num_nodes, coords, conn, rho, mu, dt, step, num_hist, hist, nxt);
    a.adj    = adj;
    a.out    = out;
    launchDependent(nsHistVjpKernel, blocksFor(a.ne, kThreads), kThreads, s, a);
    cudaCheck(cudaGetLastError(), "Navier history VJP launch");
  });
}
