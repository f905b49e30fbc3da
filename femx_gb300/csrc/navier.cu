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
// Layout (FP64 throughout: this is the drop-in): a 16-lane group owns one
// element, 8 elements per 128-thread block. Lane 15 forms the geometry
// (constant gradients of the affine P1 map, as ElementValues does), lanes
// 0..2 evaluate the quadrature-point state once per element (femx repeats
// it for every row), lanes 0..8 produce the nine rows, and the block is
// added into CSR row-coalesced through the column-major in-row position map
// (one FP64 reduction instruction per row). The history VJP is reverse mode
// written out by hand (no Enzyme): per quadrature point the adjoint
// contractions give dL/d(u, grad u, adv, tau), tau's dependence on u
// (through |u| and the streamline length) is chained in, and lanes 0..11
// scatter the velocity history entries of both lags.
#include "maps.cuh"

namespace
{

using gbfem::DeviceStatus;

constexpr int kLanes    = 16;
constexpr int kElems    = 8;
constexpr int kThreads  = kLanes * kElems;
constexpr int kQ        = 3;
constexpr int kDofs     = 9;

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

struct NsQp
{
  double u[2], adv[2], grad[2][2], ag[2], tau;
  // for the VJP: streamline length pieces
  double speed, h, sum, dir[2];
  bool   fallback;
};

struct NsElem
{
  double h0[16], h1[16], x[16], a[16];
  double g[3][2]; // dN_in/dx_d (constant on the affine triangle)
  double jxw;     // |det| * w, equal at the three points
  int    ok;
  NsQp   qp[kQ];
};

struct NsSmem
{
  NsElem el[kElems];
  double kv[kElems][kDofs][kDofs + 1]; // staged rows (odd stride: no conflicts)
  int    rs[kElems][16];
};

__device__ __forceinline__ double advDeriv(const NsElem& E, const NsQp& qp, int in)
{
  double v = 0.0;
  for (int d = 0; d < 2; ++d)
  {
    v += E.g[in][d] * qp.adv[d];
  }
  return v;
}

// Gather + geometry (lane 15). Returns whether the element is live.
__device__ bool stageElement(const NsArgs& a, NsElem& E, int e, int l, bool has, bool vjp)
{
  if (has && l < kDofs)
  {
    const int dof = a.dofs[kDofs * e + l];
    E.h0[l]       = a.hist[dof];
    E.h1[l]       = a.num_hist > 1 ? a.hist[static_cast<long long>(a.num_states) + dof] : 0.0;
    E.x[l]        = a.nxt[dof];
    if (vjp)
    {
      E.a[l] = a.adj[dof];
    }
  }
  if (has && l == 15)
  {
    E.ok          = 0;
    bool nodes_ok = true;
    for (int k = 0; k < 3; ++k)
    {
      nodes_ok = nodes_ok
                 && static_cast<unsigned>(a.conn[3 * e + k]) < static_cast<unsigned>(a.num_nodes);
    }
    if (!nodes_ok)
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
    }
    else
    {
      // ElementValues: J[a][b] = sum_in x_a(in) dN^_in/dr_b, invJ, dN/dx
      const double2 x0 = a.coords[a.conn[3 * e + 0]];
      const double2 x1 = a.coords[a.conn[3 * e + 1]];
      const double2 x2 = a.coords[a.conn[3 * e + 2]];
      double        J[4];
      J[0] = x0.x * -1.0 + x1.x * 1.0 + x2.x * 0.0;
      J[1] = x0.x * -1.0 + x1.x * 0.0 + x2.x * 1.0;
      J[2] = x0.y * -1.0 + x1.y * 1.0 + x2.y * 0.0;
      J[3] = x0.y * -1.0 + x1.y * 0.0 + x2.y * 1.0;
      const double det = J[0] * J[3] - J[1] * J[2];
      if (fabs(det) >= 1.0e-30)
      {
        const double inv     = 1.0 / det;
        const double invJ[4] = {J[3] * inv, -J[1] * inv, -J[2] * inv, J[0] * inv};
        const double dr[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
        for (int i = 0; i < 3; ++i)
        {
          for (int d = 0; d < 2; ++d)
          {
            double v = 0.0;
            for (int b = 0; b < 2; ++b)
            {
              v += dr[i][b] * invJ[b * 2 + d];
            }
            E.g[i][d] = v;
          }
        }
        E.jxw = fabs(det) * kW;
        E.ok  = 1;
      }
      else
      {
        gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
      }
    }
  }
  __syncthreads();
  return has && E.ok;
}

// evalQp + elemLength (Components.hpp:273-395) at point q.
__device__ void evalQp(const NsArgs& a, NsElem& E, int q)
{
  NsQp& qp = E.qp[q];
  for (int c = 0; c < 2; ++c)
  {
    qp.u[c] = qp.adv[c] = qp.ag[c] = 0.0;
    qp.grad[c][0] = qp.grad[c][1] = 0.0;
  }
  const bool ab2 = a.step > 0 && a.num_hist > 1;
  for (int in = 0; in < 3; ++in)
  {
    const double N = basisN(q, in);
    for (int c = 0; c < 2; ++c)
    {
      const int    id = 2 * in + c;
      const double v  = E.h0[id];
      qp.u[c] += N * v;
      for (int d = 0; d < 2; ++d)
      {
        qp.grad[c][d] += E.g[in][d] * v;
      }
      const double adv = ab2 ? 1.5 * v - 0.5 * E.h1[id] : v;
      qp.adv[c] += N * adv;
    }
  }
  double speed2 = 0.0;
  for (int c = 0; c < 2; ++c)
  {
    speed2 += qp.u[c] * qp.u[c];
    for (int d = 0; d < 2; ++d)
    {
      qp.ag[c] += qp.grad[c][d] * qp.adv[d];
    }
  }
  const double speed = sqrt(speed2);
  // elemLength: streamline direction (or the diagonal at rest)
  double     dir[2];
  const bool fallback = !(speed > 1.0e-10);
  if (!fallback)
  {
    dir[0] = qp.u[0] / speed;
    dir[1] = qp.u[1] / speed;
  }
  else
  {
    dir[0] = dir[1] = 1.0 / sqrt(2.0);
  }
  double sum = 0.0;
  for (int in = 0; in < 3; ++in)
  {
    double gr = 0.0;
    for (int d = 0; d < 2; ++d)
    {
      gr += dir[d] * E.g[in][d];
    }
    sum += gr >= 0.0 ? gr : -gr;
  }
  const double h    = sum > 1.0e-14 ? 2.0 / sum : 0.0;
  const double nu   = a.mu / a.rho;
  const double time = (2.0 / a.dt) * (2.0 / a.dt);
  double       flow = 0.0, diff = 0.0;
  if (h > 0.0)
  {
    flow = (2.0 * speed / h) * (2.0 * speed / h);
    diff = (4.0 * nu / (h * h)) * (4.0 * nu / (h * h));
  }
  qp.tau      = 1.0 / sqrt(time + flow + diff);
  qp.speed    = speed;
  qp.h        = h;
  qp.sum      = sum;
  qp.dir[0]   = dir[0];
  qp.dir[1]   = dir[1];
  qp.fallback = fallback;
}

// Row `row` of K into K[9] and the residual K x - F
// (NavierOperator::evalPhysicsRow, Components.hpp:473-575).
__device__ double evalRow(const NsArgs& a, const NsElem& E, int row, double* K)
{
  for (int col = 0; col < kDofs; ++col)
  {
    K[col] = 0.0;
  }
  const bool   vel = row < 6;
  const int    i   = vel ? row / 2 : row - 6;
  const int    c   = vel ? row - 2 * i : 0;
  const double rho = a.rho, mu = a.mu, dt = a.dt;
  double       F   = 0.0;
  for (int q = 0; q < kQ; ++q)
  {
    const NsQp&  qp  = E.qp[q];
    const double Jw  = E.jxw;
    const double Ni  = basisN(q, i);
    const double dvi = advDeriv(E, qp, i);
    if (vel)
    {
      double grad_u = 0.0;
      for (int d = 0; d < 2; ++d)
      {
        grad_u += E.g[i][d] * qp.grad[c][d];
      }
      F += (rho / dt * Ni * qp.u[c] - 0.5 * rho * Ni * qp.ag[c] - 0.5 * mu * grad_u
            + qp.tau * rho / dt * dvi * qp.u[c] - 0.5 * qp.tau * rho * dvi * qp.ag[c])
           * Jw;
      for (int j = 0; j < 3; ++j)
      {
        const double Nj  = basisN(q, j);
        const double dvj = advDeriv(E, qp, j);
        const double gd  = E.g[i][0] * E.g[j][0] + E.g[i][1] * E.g[j][1];
        K[2 * j + c] += (rho / dt * Ni * Nj + 0.5 * rho * Ni * dvj + 0.5 * mu * gd
                         + qp.tau * rho / dt * dvi * Nj + 0.5 * qp.tau * rho * dvi * dvj)
                        * Jw;
        K[6 + j] += (-E.g[i][c] * Nj + qp.tau * dvi * E.g[j][c]) * Jw;
      }
    }
    else
    {
      double div_u = 0.0, div_adv = 0.0;
      for (int d = 0; d < 2; ++d)
      {
        div_u += E.g[i][d] * qp.u[d];
        div_adv += E.g[i][d] * qp.ag[d];
      }
      F += (qp.tau / dt * div_u - 0.5 * qp.tau * div_adv) * Jw;
      for (int j = 0; j < 3; ++j)
      {
        const double Nj  = basisN(q, j);
        const double dvj = advDeriv(E, qp, j);
        for (int d = 0; d < 2; ++d)
        {
          const double gi = E.g[i][d];
          K[2 * j + d] += (Ni * E.g[j][d] + qp.tau / dt * gi * Nj + 0.5 * qp.tau * gi * dvj) * Jw;
        }
        const double gd = E.g[i][0] * E.g[j][0] + E.g[i][1] * E.g[j][1];
        K[6 + j] += qp.tau / rho * gd * Jw;
      }
    }
  }
  double out = -F;
  for (int col = 0; col < kDofs; ++col)
  {
    out += K[col] * E.x[col];
  }
  return out;
}

template <bool kJac>
__global__ void __launch_bounds__(kThreads) nsAssembleKernel(NsArgs a)
{
  __shared__ NsSmem sm;
  const int  l   = threadIdx.x & (kLanes - 1);
  const int  le  = threadIdx.x / kLanes;
  const int  e   = blockIdx.x * kElems + le;
  const bool has = e < a.ne;
  NsElem&    E   = sm.el[le];
  const bool live = stageElement(a, E, e, l, has, false);
  if (live && l < kQ)
  {
    evalQp(a, E, l);
  }
  __syncthreads();
  if (live && l < kDofs)
  {
    double    K[kDofs];
    const double r   = evalRow(a, E, l, K);
    const int    dof = a.dofs[kDofs * e + l];
    gbfem::redAdd(a.res + dof, r);
    if (kJac)
    {
      for (int col = 0; col < kDofs; ++col)
      {
        sm.kv[le][l][col] = K[col];
      }
      sm.rs[le][l] = a.row_ptr[dof];
    }
  }
  if (kJac)
  {
    __syncwarp();
    if (live && l < kDofs)
    {
      // lane l owns local column l: one reduction instruction per row
      unsigned char pos[16];
      if (a.jac_pos != nullptr)
      {
        const uint4    w4    = *reinterpret_cast<const uint4*>(a.jac_pos + (9LL * e + l) * 16);
        const unsigned wd[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int i = 0; i < 16; ++i)
        {
          pos[i] = static_cast<unsigned char>(wd[i >> 2] >> (8 * (i & 3)));
        }
      }
#pragma unroll
      for (int row = 0; row < kDofs; ++row)
      {
        const int slot = a.jac_pos != nullptr ? sm.rs[le][row] + pos[row]
                                              : a.jac_map[81LL * e + kDofs * row + l];
        gbfem::redAdd(a.vals + slot, sm.kv[le][row][l]);
      }
    }
  }
}

// History VJP: out[lag][dof] += d/d hist[lag][dof] of sum_rows adj . R.
__global__ void __launch_bounds__(kThreads) nsHistVjpKernel(NsArgs a)
{
  __shared__ NsSmem sm;
  __shared__ double dEu[kElems][kQ][2], dEg[kElems][kQ][2][2], dEa[kElems][kQ][2];
  const int  l    = threadIdx.x & (kLanes - 1);
  const int  le   = threadIdx.x / kLanes;
  const int  e    = blockIdx.x * kElems + le;
  const bool has  = e < a.ne;
  NsElem&    E    = sm.el[le];
  const bool live = stageElement(a, E, e, l, has, true);
  if (live && l < kQ)
  {
    const int q = l;
    evalQp(a, E, q);
    const NsQp&  qp  = E.qp[q];
    const double rho = a.rho, mu = a.mu, dt = a.dt, tau = qp.tau;
    // next-state and adjoint fields at the point
    double X[2] = {0, 0}, Gx[2][2] = {{0, 0}, {0, 0}}, Xp = 0, Gp[2] = {0, 0};
    double A[2] = {0, 0}, GA[2][2] = {{0, 0}, {0, 0}}, AP = 0, GAP[2] = {0, 0};
    for (int j = 0; j < 3; ++j)
    {
      const double N = basisN(q, j);
      for (int c = 0; c < 2; ++c)
      {
        X[c] += N * E.x[2 * j + c];
        A[c] += N * E.a[2 * j + c];
        for (int d = 0; d < 2; ++d)
        {
          Gx[c][d] += E.g[j][d] * E.x[2 * j + c];
          GA[c][d] += E.g[j][d] * E.a[2 * j + c];
        }
      }
      Xp += N * E.x[6 + j];
      AP += N * E.a[6 + j];
      for (int d = 0; d < 2; ++d)
      {
        Gp[d] += E.g[j][d] * E.x[6 + j];
        GAP[d] += E.g[j][d] * E.a[6 + j];
      }
    }
    double Dv[2], Av[2];
    for (int c = 0; c < 2; ++c)
    {
      Dv[c] = qp.adv[0] * Gx[c][0] + qp.adv[1] * Gx[c][1];
      Av[c] = qp.adv[0] * GA[c][0] + qp.adv[1] * GA[c][1];
    }
    // partial derivatives of the adjoint-weighted integrand
    double Ptau = 0.0, W[2], PAv[2], du[2];
    for (int c = 0; c < 2; ++c)
    {
      const double xm = X[c] - qp.u[c], dg = Dv[c] + qp.ag[c];
      Ptau += rho / dt * Av[c] * xm + 0.5 * rho * Av[c] * dg + Av[c] * Gp[c];
      Ptau += GAP[c] * (X[c] / dt + 0.5 * Dv[c] + Gp[c] / rho - qp.u[c] / dt + 0.5 * qp.ag[c]);
      W[c]   = 0.5 * rho * A[c] + 0.5 * tau * rho * Av[c] + 0.5 * tau * GAP[c];
      PAv[c] = tau * rho / dt * xm + 0.5 * tau * rho * dg + tau * Gp[c];
      du[c]  = -rho / dt * A[c] - tau * rho / dt * Av[c] - tau / dt * GAP[c];
    }
    // tau(u): through |u| and the streamline length h(u/|u|)
    if (qp.h > 0.0)
    {
      double dh[2] = {0.0, 0.0};
      if (!qp.fallback)
      {
        // dh/du_c = -2/sum^2 sum_in sgn(g_in) sum_d dN_in/dx_d (delta_dc - dir_d dir_c)/|u|
        for (int in = 0; in < 3; ++in)
        {
          const double gr = qp.dir[0] * E.g[in][0] + qp.dir[1] * E.g[in][1];
          const double sg = gr >= 0.0 ? 1.0 : -1.0;
          for (int c = 0; c < 2; ++c)
          {
            dh[c] += sg * (E.g[in][c] - gr * qp.dir[c]);
          }
        }
        for (int c = 0; c < 2; ++c)
        {
          dh[c] *= -2.0 / (qp.sum * qp.sum * qp.speed);
        }
      }
      const double nu  = mu / rho;
      const double h   = qp.h;
      const double t3  = tau * tau * tau;
      for (int c = 0; c < 2; ++c)
      {
        const double dflow = 8.0 * (qp.u[c] * h - qp.speed * qp.speed * dh[c]) / (h * h * h);
        const double ddiff = -64.0 * nu * nu * dh[c] / (h * h * h * h * h);
        du[c] += Ptau * (-0.5 * t3 * (dflow + ddiff));
      }
    }
    const double Jw = E.jxw;
    for (int c = 0; c < 2; ++c)
    {
      dEu[le][q][c] = Jw * du[c];
      double da     = 0.0;
      for (int cc = 0; cc < 2; ++cc)
      {
        da += W[cc] * (qp.grad[cc][c] + Gx[cc][c]) + PAv[cc] * GA[cc][c];
      }
      dEa[le][q][c] = Jw * da;
      for (int d = 0; d < 2; ++d)
      {
        dEg[le][q][c][d] = Jw * (0.5 * mu * GA[c][d] + W[c] * qp.adv[d]);
      }
    }
  }
  __syncthreads();
  if (live && l < 12)
  {
    // velocity history entry: lag l / 6, local velocity DOF l % 6
    const int  lag = l / 6, vd = l % 6, in = vd / 2, c = vd % 2;
    const bool ab2 = a.step > 0 && a.num_hist > 1;
    if (lag == 0 || ab2)
    {
      const double al0 = ab2 ? 1.5 : 1.0, al1 = -0.5;
      double       v   = 0.0;
      for (int q = 0; q < kQ; ++q)
      {
        const double N = basisN(q, in);
        if (lag == 0)
        {
          v += N * dEu[le][q][c] + E.g[in][0] * dEg[le][q][c][0] + E.g[in][1] * dEg[le][q][c][1]
               + al0 * N * dEa[le][q][c];
        }
        else
        {
          v += al1 * N * dEa[le][q][c];
        }
      }
      const int dof = a.dofs[kDofs * e + vd];
      gbfem::redAdd(a.out + static_cast<long long>(lag) * a.num_states + dof, v);
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
                                     const double* hist, const double* nxt, double* res,
                                     double* vals, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    checkCommon(map, num_nodes, coords, conn, rho, mu, dt, num_hist, hist, nxt);
    require(res != nullptr, "Assembly residual output is null");
    require(res != hist && res != nxt && vals != hist && vals != nxt
                && (vals == nullptr || res != vals),
            "Time assembly outputs must not alias inputs or each other");
    cudaStream_t s = asStream(stream);
    cudaCheck(cudaMemsetAsync(res, 0, sizeof(double) * map->num_res, s), "residual zero");
    if (vals != nullptr && map->nnz > 0)
    {
      cudaCheck(cudaMemsetAsync(vals, 0, sizeof(double) * map->nnz, s), "matrix zero");
    }
    if (map->num_elems == 0)
    {
      return;
    }
    NsArgs a = makeArgs(map, num_nodes, coords, conn, rho, mu, dt, step, num_hist, hist, nxt);
    a.res    = res;
    a.vals   = vals;
    const unsigned blocks = blocksFor(a.ne, kElems);
    vals != nullptr ? nsAssembleKernel<true><<<blocks, kThreads, 0, s>>>(a)
                    : nsAssembleKernel<false><<<blocks, kThreads, 0, s>>>(a);
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
    cudaCheck(cudaMemsetAsync(out, 0, sizeof(double) * num_hist * static_cast<size_t>(map->num_states), s),
              "VJP zero");
    if (map->num_elems == 0)
    {
      return;
    }
    NsArgs a = makeArgs(map, num_nodes, coords, conn, rho, mu, dt, step, num_hist, hist, nxt);
    a.adj    = adj;
    a.out    = out;
    nsHistVjpKernel<<<blocksFor(a.ne, kElems), kThreads, 0, s>>>(a);
    cudaCheck(cudaGetLastError(), "Navier history VJP launch");
  });
}
