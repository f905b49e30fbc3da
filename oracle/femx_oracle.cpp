// femx_oracle.cpp — serial CPU restatement of femx's assembly hot path.
//
// TEST INFRASTRUCTURE ONLY (see femx_oracle.h). Every function names the
// reference file:line whose algorithm it restates. The element operators
// (kappa-weighted P1 Poisson, its VJPs, Taylor-Hood P2/P1 Navier-Stokes) are
// not in the reference; they are written against the reference's
// ElementOperator plug-in contract (femx/assembly/Assembly.hpp:138-152) and
// run through a restatement of the reference's generic element loop.

#include "femx_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace
{

thread_local std::string g_err;

struct Failure : std::runtime_error
{
  using std::runtime_error::runtime_error;
};

void require(bool cond, const char* msg)
{
  if (!cond)
  {
    throw Failure(msg);
  }
}

template <class F>
int guarded(F&& fn)
{
  try
  {
    fn();
    return 0;
  }
  catch (const std::exception& e)
  {
    g_err = e.what();
    return 1;
  }
}

// ---------------------------------------------------------------------------
// AssemblyMap — femx/assembly/AssemblyMap.cpp:54-176
// ---------------------------------------------------------------------------
struct Map
{
  int num_elems = 0, num_res = 0, num_states = 0;
  std::vector<int> res_offsets, res_dofs, state_offsets, state_dofs;
  std::vector<int> jac_offsets, jac_map, row_ptr, col_ind;
  int max_res = 0, max_state = 0, max_jac = 0;

  int nrow(int e) const { return res_offsets[e + 1] - res_offsets[e]; }
  int ncol(int e) const { return state_offsets[e + 1] - state_offsets[e]; }
};

Map* buildMap(int num_res, int num_states, int num_elems,
              const int* res_offsets, const int* res_dofs,
              const int* state_offsets, const int* state_dofs)
{
  require(num_res >= 0 && num_states >= 0,
          "AssemblyMap global dimensions must be non-negative");
  require(num_elems >= 0, "AssemblyMap residual/state element counts differ");
  auto* m       = new Map;
  m->num_elems  = num_elems;
  m->num_res    = num_res;
  m->num_states = num_states;
  m->res_offsets.assign(num_elems + 1, 0);
  m->state_offsets.assign(num_elems + 1, 0);
  m->jac_offsets.assign(num_elems + 1, 0);
  try
  {
    // Flattened element tables and local Jacobian offsets (:71-104).
    for (int e = 0; e < num_elems; ++e)
    {
      const int r0 = res_offsets[e], r1 = res_offsets[e + 1];
      const int s0 = state_offsets[e], s1 = state_offsets[e + 1];
      require(r1 >= r0 && s1 >= s0,
              "AssemblyMap local dimensions must be non-negative");
      for (int i = r0; i < r1; ++i)
      {
        require(res_dofs[i] >= 0 && res_dofs[i] < num_res,
                "AssemblyMap residual DOF is out of range");
        m->res_dofs.push_back(res_dofs[i]);
      }
      for (int i = s0; i < s1; ++i)
      {
        require(state_dofs[i] >= 0 && state_dofs[i] < num_states,
                "AssemblyMap state DOF is out of range");
        m->state_dofs.push_back(state_dofs[i]);
      }
      const std::int64_t ennz = std::int64_t(r1 - r0) * (s1 - s0);
      require(ennz <= std::numeric_limits<int>::max(),
              "AssemblyMap local Jacobian is too large");
      const std::int64_t next = std::int64_t(m->jac_offsets[e]) + ennz;
      require(next <= std::numeric_limits<int>::max(),
              "AssemblyMap flattened data exceeds the Index range");
      m->res_offsets[e + 1]   = int(m->res_dofs.size());
      m->state_offsets[e + 1] = int(m->state_dofs.size());
      m->jac_offsets[e + 1]   = int(next);
      m->max_res              = std::max(m->max_res, r1 - r0);
      m->max_state            = std::max(m->max_state, s1 - s0);
      m->max_jac              = std::max(m->max_jac, int(ennz));
    }

    // COO of every (row, col) pair of every element block (:106-120).
    const int        nnz = m->jac_offsets[num_elems];
    std::vector<int> coo_r(nnz), coo_c(nnz), order(nnz);
    int              k = 0;
    for (int e = 0; e < num_elems; ++e)
    {
      for (int i = m->res_offsets[e]; i < m->res_offsets[e + 1]; ++i)
      {
        for (int j = m->state_offsets[e]; j < m->state_offsets[e + 1]; ++j)
        {
          coo_r[k] = m->res_dofs[i];
          coo_c[k] = m->state_dofs[j];
          order[k] = k;
          ++k;
        }
      }
    }
    // Global sort by (row, col) (:122-132).
    std::sort(order.begin(), order.end(), [&](int a, int b) {
      if (coo_r[a] != coo_r[b])
      {
        return coo_r[a] < coo_r[b];
      }
      return coo_c[a] < coo_c[b];
    });
    // Dedupe, count rows, and record every entry's CSR slot (:134-156).
    m->row_ptr.assign(num_res + 1, 0);
    m->jac_map.assign(nnz, 0);
    m->col_ind.reserve(nnz);
    int csr = -1;
    for (int i = 0; i < nnz; ++i)
    {
      const int  cur    = order[i];
      const bool is_new = i == 0 || coo_r[cur] != coo_r[order[i - 1]]
                          || coo_c[cur] != coo_c[order[i - 1]];
      if (is_new)
      {
        ++csr;
        m->col_ind.push_back(coo_c[cur]);
        ++m->row_ptr[coo_r[cur] + 1];
      }
      m->jac_map[cur] = csr;
    }
    for (int r = 0; r < num_res; ++r)
    {
      m->row_ptr[r + 1] += m->row_ptr[r];
    }
  }
  catch (...)
  {
    delete m;
    throw;
  }
  return m;
}

// ---------------------------------------------------------------------------
// BoundaryMap — femx/assembly/BoundaryMap.cpp:59-139
// ---------------------------------------------------------------------------
struct Bc
{
  int rows = 0, cols = 0, nnz = 0;
  std::vector<int> bc_rows, diag, col_offsets, col_entries, col_rows, bc_mask;
  int num() const { return int(bc_rows.size()); }
};

Bc* buildBc(int num_bcs, const int* dofs, int rows, int cols,
            const int* row_ptr, const int* col_ind)
{
  require(rows == cols, "BoundaryMap requires a square CSR pattern");
  auto* b = new Bc;
  try
  {
    b->rows = rows;
    b->cols = cols;
    b->nnz  = row_ptr[rows];
    b->bc_rows.assign(num_bcs, 0);
    b->diag.assign(num_bcs, -1);
    b->col_offsets.assign(num_bcs + 1, 0);
    b->bc_mask.assign(rows, 0);
    std::vector<int> bc_by_col(cols, -1);
    for (int ib = 0; ib < num_bcs; ++ib)
    {
      const int dof = dofs[ib];
      require(dof >= 0 && dof < rows,
              "BoundaryMap constrained DOF is out of range");
      require(b->bc_mask[dof] == 0,
              "BoundaryMap constrained DOFs must be unique");
      b->bc_rows[ib]  = dof;
      b->bc_mask[dof] = 1;
      bc_by_col[dof]  = ib;
    }
    // Count constrained-column entries and find diagonals (:83-103).
    for (int r = 0; r < rows; ++r)
    {
      for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
      {
        const int ib = bc_by_col[col_ind[k]];
        if (ib >= 0)
        {
          ++b->col_offsets[ib + 1];
          if (r == col_ind[k])
          {
            require(b->diag[ib] < 0,
                    "BoundaryMap constrained row has duplicate diagonal "
                    "entries");
            b->diag[ib] = k;
          }
        }
      }
    }
    for (int ib = 0; ib < num_bcs; ++ib)
    {
      require(b->diag[ib] >= 0,
              "BoundaryMap constrained row has no diagonal entry");
      b->col_offsets[ib + 1] += b->col_offsets[ib];
    }
    // Fill grouped by constraint, rows ascending (:112-126).
    b->col_entries.assign(b->col_offsets[num_bcs], 0);
    b->col_rows.assign(b->col_offsets[num_bcs], 0);
    std::vector<int> next(b->col_offsets.begin(), b->col_offsets.end());
    for (int r = 0; r < rows; ++r)
    {
      for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
      {
        const int ib = bc_by_col[col_ind[k]];
        if (ib >= 0)
        {
          const int dst      = next[ib]++;
          b->col_entries[dst] = k;
          b->col_rows[dst]    = r;
        }
      }
    }
  }
  catch (...)
  {
    delete b;
    throw;
  }
  return b;
}

// BoundaryMap.cpp:38-55
void replaceRowsRaw(const Bc& b, const int* row_ptr, double* vals, double d)
{
  for (int ib = 0; ib < b.num(); ++ib)
  {
    const int r = b.bc_rows[ib];
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
    {
      vals[k] = 0.0;
    }
    vals[b.diag[ib]] = d;
  }
}

// ---------------------------------------------------------------------------
// Reference-element tables — GaussQuadrature.hpp:175-204,
// elements/LagrangeTriangleP1.hpp:48-70, ElementValues.cpp:138-252
// ---------------------------------------------------------------------------
struct QuadPt
{
  double r, s, w;
};

std::vector<QuadPt> triangleRule(int order)
{
  if (order == 1)
  {
    return {{1.0 / 3.0, 1.0 / 3.0, 0.5}};
  }
  if (order == 2)
  {
    return {{1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0},
            {2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0},
            {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0}};
  }
  throw Failure("Unsupported triangle quad order");
}

// Published 6-point degree-4 triangle rule (Dunavant 1985), weights scaled to
// the reference-triangle area 1/2. The reference ships orders 1-2 only.
std::vector<QuadPt> triangleRuleDeg4()
{
  const double a1 = 0.445948490915964886, w1 = 0.223381589678011466 * 0.5;
  const double a2 = 0.091576213509770743, w2 = 0.109951743655321868 * 0.5;
  return {{a1, a1, w1},
          {1.0 - 2.0 * a1, a1, w1},
          {a1, 1.0 - 2.0 * a1, w1},
          {a2, a2, w2},
          {1.0 - 2.0 * a2, a2, w2},
          {a2, 1.0 - 2.0 * a2, w2}};
}

// ElementValues::invJacobian, dim 2 (ElementValues.cpp:210-229).
double invJacobian2(const double J[4], double invJ[4])
{
  const double det = J[0] * J[3] - J[1] * J[2];
  require(std::abs(det) >= 1.0e-30, "Singular 2D Jacobian.");
  const double inv = 1.0 / det;
  invJ[0]          = J[3] * inv;
  invJ[1]          = -J[1] * inv;
  invJ[2]          = -J[2] * inv;
  invJ[3]          = J[0] * inv;
  return det;
}

// makeElementQuadratureData for P1 triangles (ElementQuadratureData.cpp:14-59
// over ElementValues::calcPhysicalValues, ElementValues.cpp:138-181).
struct P1Quad
{
  int nq = 0, ne = 0;
  std::vector<double> N;    // [nq][3]
  std::vector<double> dNdx; // [E][nq][3][2]
  std::vector<double> JxW;  // [E][nq]
};

const double kP1dNdr[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};

P1Quad* buildP1Quad(int num_nodes, const double* coords, int num_elems,
                    const int* conn, int order)
{
  const auto rule = triangleRule(order);
  auto*      q    = new P1Quad;
  q->nq           = int(rule.size());
  q->ne           = num_elems;
  q->N.resize(q->nq * 3);
  q->dNdx.resize(std::size_t(num_elems) * q->nq * 6);
  q->JxW.resize(std::size_t(num_elems) * q->nq);
  for (int iq = 0; iq < q->nq; ++iq)
  {
    q->N[iq * 3 + 0] = 1.0 - rule[iq].r - rule[iq].s;
    q->N[iq * 3 + 1] = rule[iq].r;
    q->N[iq * 3 + 2] = rule[iq].s;
  }
  try
  {
    for (int e = 0; e < num_elems; ++e)
    {
      for (int iq = 0; iq < q->nq; ++iq)
      {
        double J[4] = {0.0, 0.0, 0.0, 0.0};
        for (int in = 0; in < 3; ++in)
        {
          const int node = conn[3 * e + in];
          require(node >= 0 && node < num_nodes,
                  "Geometry element connectivity is out of range");
          for (int a = 0; a < 2; ++a)
          {
            const double xa = coords[2 * node + a];
            for (int b = 0; b < 2; ++b)
            {
              J[a * 2 + b] += xa * kP1dNdr[in][b];
            }
          }
        }
        double       invJ[4];
        const double det = std::abs(invJacobian2(J, invJ));
        q->JxW[std::size_t(e) * q->nq + iq] = det * rule[iq].w;
        double* g = &q->dNdx[(std::size_t(e) * q->nq + iq) * 6];
        for (int i = 0; i < 3; ++i)
        {
          for (int a = 0; a < 2; ++a)
          {
            double v = 0.0;
            for (int b = 0; b < 2; ++b)
            {
              v += kP1dNdr[i][b] * invJ[b * 2 + a];
            }
            g[i * 2 + a] = v;
          }
        }
      }
    }
  }
  catch (...)
  {
    delete q;
    throw;
  }
  return q;
}

// KappaPoissonP1 element operator: one evalRow per local row, after
// examples/poisson/PoissonComponents.hpp:35-64 with kappa and a load term.
struct KappaPoissonP1
{
  const P1Quad* q;
  const int*    conn;
  const double* kappa;
  const double* f;

  void evalRow(int e, int row, const double* state, double& res,
               double* jac) const
  {
    res = 0.0;
    for (int c = 0; c < 3; ++c)
    {
      jac[c] = 0.0;
    }
    for (int iq = 0; iq < q->nq; ++iq)
    {
      const double* g   = &q->dNdx[(std::size_t(e) * q->nq + iq) * 6];
      const double  jxw = q->JxW[std::size_t(e) * q->nq + iq];
      for (int c = 0; c < 3; ++c)
      {
        double dot = 0.0;
        for (int d = 0; d < 2; ++d)
        {
          dot += g[row * 2 + d] * g[c * 2 + d];
        }
        jac[c] += dot * jxw;
      }
    }
    for (int c = 0; c < 3; ++c)
    {
      jac[c] *= kappa[e];
      res += jac[c] * state[c];
    }
    if (f != nullptr)
    {
      for (int iq = 0; iq < q->nq; ++iq)
      {
        double fq = 0.0;
        for (int n = 0; n < 3; ++n)
        {
          fq += f[conn[3 * e + n]] * q->N[iq * 3 + n];
        }
        res -= fq * q->N[iq * 3 + row] * q->JxW[std::size_t(e) * q->nq + iq];
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Taylor-Hood P2/P1 element operator (new physics; no reference file).
// ---------------------------------------------------------------------------
struct P2Basis
{
  // values [6], reference gradients [6][2] at (r, s)
  static void eval(double r, double s, double* N, double* dN)
  {
    const double l0 = 1.0 - r - s, l1 = r, l2 = s;
    const double g0[2] = {-1.0, -1.0}, g1[2] = {1.0, 0.0}, g2[2] = {0.0, 1.0};
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
};

struct TaylorHoodNS
{
  double nu;
  // Per-element physical tables, built like ElementQuadratureData.
  int                 nq;
  std::vector<QuadPt> rule;
  std::vector<double> Nv;   // [nq][6]
  std::vector<double> Np;   // [nq][3]
  std::vector<double> dNv;  // [E][nq][6][2]
  std::vector<double> dNp;  // [E][nq][3][2]
  std::vector<double> JxW;  // [E][nq]

  void build(int num_nodes, const double* coords, int ne, const int* conn6)
  {
    rule = triangleRuleDeg4();
    nq   = int(rule.size());
    Nv.resize(nq * 6);
    Np.resize(nq * 3);
    dNv.resize(std::size_t(ne) * nq * 12);
    dNp.resize(std::size_t(ne) * nq * 6);
    JxW.resize(std::size_t(ne) * nq);
    std::vector<double> dNr(nq * 12);
    for (int iq = 0; iq < nq; ++iq)
    {
      P2Basis::eval(rule[iq].r, rule[iq].s, &Nv[iq * 6], &dNr[iq * 12]);
      Np[iq * 3 + 0] = 1.0 - rule[iq].r - rule[iq].s;
      Np[iq * 3 + 1] = rule[iq].r;
      Np[iq * 3 + 2] = rule[iq].s;
    }
    for (int e = 0; e < ne; ++e)
    {
      double J[4] = {0.0, 0.0, 0.0, 0.0};
      for (int in = 0; in < 3; ++in)
      {
        const int node = conn6[6 * e + in];
        require(node >= 0 && node < num_nodes,
                "Geometry element connectivity is out of range");
        for (int a = 0; a < 2; ++a)
        {
          for (int b = 0; b < 2; ++b)
          {
            J[a * 2 + b] += coords[2 * node + a] * kP1dNdr[in][b];
          }
        }
      }
      double       invJ[4];
      const double det = std::abs(invJacobian2(J, invJ));
      for (int iq = 0; iq < nq; ++iq)
      {
        JxW[std::size_t(e) * nq + iq] = det * rule[iq].w;
        for (int i = 0; i < 6; ++i)
        {
          for (int a = 0; a < 2; ++a)
          {
            double v = 0.0;
            for (int b = 0; b < 2; ++b)
            {
              v += dNr[iq * 12 + i * 2 + b] * invJ[b * 2 + a];
            }
            dNv[((std::size_t(e) * nq + iq) * 6 + i) * 2 + a] = v;
          }
        }
        for (int i = 0; i < 3; ++i)
        {
          for (int a = 0; a < 2; ++a)
          {
            double v = 0.0;
            for (int b = 0; b < 2; ++b)
            {
              v += kP1dNdr[i][b] * invJ[b * 2 + a];
            }
            dNp[((std::size_t(e) * nq + iq) * 3 + i) * 2 + a] = v;
          }
        }
      }
    }
  }

  // One local row (0..11 velocity, 12..14 pressure) of residual and Jacobian.
  // Like NavierOperator::evalRow (femx/model/ns/Components.hpp:412-435), the
  // quadrature-point state is recomputed for every row.
  void evalRow(int e, int row, const double* st, double& res,
               double* jac) const
  {
    evalRowNu(nu, e, row, st, res, jac);
  }

  void evalRowNu(double nu, int e, int row, const double* st, double& res,
                 double* jac) const
  {
    res = 0.0;
    for (int c = 0; c < 15; ++c)
    {
      jac[c] = 0.0;
    }
    for (int iq = 0; iq < nq; ++iq)
    {
      const double* N   = &Nv[iq * 6];
      const double* P   = &Np[iq * 3];
      const double* dN  = &dNv[(std::size_t(e) * nq + iq) * 12];
      const double* dP  = &dNp[(std::size_t(e) * nq + iq) * 6];
      const double  jxw = JxW[std::size_t(e) * nq + iq];
      double        u[2] = {0.0, 0.0}, G[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
      double        p    = 0.0;
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
        double    r = 0.0;
        for (int d = 0; d < 2; ++d)
        {
          r += nu * G[c][d] * dN[a * 2 + d] + u[d] * G[c][d] * N[a];
        }
        r -= p * dN[a * 2 + c];
        res += r * jxw;
        for (int b = 0; b < 6; ++b)
        {
          double adv = 0.0, diff = 0.0;
          for (int d = 0; d < 2; ++d)
          {
            adv += u[d] * dN[b * 2 + d];
            diff += dN[b * 2 + d] * dN[a * 2 + d];
          }
          for (int ec = 0; ec < 2; ++ec)
          {
            double v = N[b] * G[c][ec] * N[a];
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

// Generic element loop — femx/assembly/Assembly.hpp:153-226: zero the
// outputs, gather element state, evaluate every local row, scatter-add
// residual rows through res_dofs and Jacobian entries through jac_map.
template <class Op>
void assembleLoop(const Map& m, const Op& op, const double* state,
                  double* res, double* vals, int e0 = 0, int e1 = -1)
{
  if (e1 < 0 || e1 > m.num_elems)
  {
    e1 = m.num_elems;
  }
  require(e0 >= 0 && e0 <= e1, "element range is invalid");
  std::fill(res, res + m.num_res, 0.0);
  std::fill(vals, vals + m.row_ptr[m.num_res], 0.0);
  std::vector<double> st(m.max_state), re(m.max_res), jac(m.max_jac);
  for (int e = e0; e < e1; ++e)
  {
    const int nr = m.nrow(e), nc = m.ncol(e);
    for (int c = 0; c < nc; ++c)
    {
      st[c] = state[m.state_dofs[m.state_offsets[e] + c]];
    }
    for (int r = 0; r < nr; ++r)
    {
      op.evalRow(e, r, st.data(), re[r], jac.data() + r * nc);
    }
    for (int r = 0; r < nr; ++r)
    {
      res[m.res_dofs[m.res_offsets[e] + r]] += re[r];
    }
    for (int i = 0; i < nr * nc; ++i)
    {
      vals[m.jac_map[m.jac_offsets[e] + i]] += jac[i];
    }
  }
}

// Atomic FP64 add on the value's bit pattern (compare-exchange loop), the
// effect of `#pragma omp atomic` on `vals[k] += v`.
inline void atomicAddDouble(double* addr, double v)
{
  auto*         bits = reinterpret_cast<std::uint64_t*>(addr);
  std::uint64_t old  = __atomic_load_n(bits, __ATOMIC_RELAXED);
  for (;;)
  {
    double cur;
    std::memcpy(&cur, &old, sizeof(double));
    const double  nxt = cur + v;
    std::uint64_t nb;
    std::memcpy(&nb, &nxt, sizeof(double));
    if (__atomic_compare_exchange_n(bits, &old, nb, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
    {
      return;
    }
  }
}

// Multi-threaded element loop: the scheme of femx's OpenMP NS assembly
// (femx/model/ns/NavierStokesModel.cpp:227-318): element chunks shared by
// the threads, residual and CSR adds atomic (addElem(atomic),
// femx/assembly/Assembly.cpp:8-41). Same operator as assembleLoop; the
// order of the additions into one slot depends on thread timing.
template <class Op>
void assembleLoopThreads(const Map& m, const Op& op, const double* state, double* res,
                         double* vals, int nthreads)
{
  nthreads          = std::max(1, nthreads);
  const long long n = m.row_ptr[m.num_res];
  {
    std::vector<std::thread> zero;
    for (int t = 0; t < nthreads; ++t)
    {
      zero.emplace_back([&, t] {
        const long long a = n * t / nthreads, b = n * (t + 1) / nthreads;
        std::fill(vals + a, vals + b, 0.0);
        const long long ra = static_cast<long long>(m.num_res) * t / nthreads;
        const long long rb = static_cast<long long>(m.num_res) * (t + 1) / nthreads;
        std::fill(res + ra, res + rb, 0.0);
      });
    }
    for (auto& th : zero)
    {
      th.join();
    }
  }
  constexpr int            kChunk = 256;
  int                      next   = 0;
  std::vector<std::thread> work;
  for (int t = 0; t < nthreads; ++t)
  {
    work.emplace_back([&] {
      std::vector<double> st(m.max_state), re(m.max_res), jac(m.max_jac);
      for (;;)
      {
        const int e0 = __atomic_fetch_add(&next, kChunk, __ATOMIC_RELAXED);
        if (e0 >= m.num_elems)
        {
          return;
        }
        const int e1 = std::min(m.num_elems, e0 + kChunk);
        for (int e = e0; e < e1; ++e)
        {
          const int nr = m.nrow(e), nc = m.ncol(e);
          for (int c = 0; c < nc; ++c)
          {
            st[c] = state[m.state_dofs[m.state_offsets[e] + c]];
          }
          for (int r = 0; r < nr; ++r)
          {
            op.evalRow(e, r, st.data(), re[r], jac.data() + r * nc);
          }
          for (int r = 0; r < nr; ++r)
          {
            atomicAddDouble(res + m.res_dofs[m.res_offsets[e] + r], re[r]);
          }
          for (int i = 0; i < nr * nc; ++i)
          {
            atomicAddDouble(vals + m.jac_map[m.jac_offsets[e] + i], jac[i]);
          }
        }
      }
    });
  }
  for (auto& th : work)
  {
    th.join();
  }
}

// ---------------------------------------------------------------------------
// femx's equal-order GLS Navier-Stokes time operator, restated
// (femx/model/ns/Components.hpp:330-577: evalQp, elemLength, advDeriv,
// gradDot, NavierOperator::evalPhysicsRow). P1 triangles in 2-D: 3 nodes,
// local DOFs vdof(in, c) = 2 in + c then pdof(in) = 6 + in; element data
// from P1Quad (makeNavierData = ElementValues over the order-2 rule).
// Templated on the scalar so that the forward-mode Dual below gives exact
// history derivatives (the role Enzyme plays in femx, Components.cpp:67-125).

struct Dual
{
  double v = 0.0, d = 0.0;
  Dual() = default;
  Dual(double x) : v(x) {}
  Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b)
{
  return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)};
}
inline Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
inline Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
inline double val(double x) { return x; }
inline double val(Dual x) { return x.v; }
inline double sqrtS(double x) { return std::sqrt(x); }
// sqrt at 0 gets the derivative 0 (its one-sided limit of the squared
// quantities it feeds is 0: flow = (2|u|/h)^2 is smooth in u).
inline Dual sqrtS(Dual x)
{
  const double r = std::sqrt(x.v);
  return {r, r > 0.0 ? 0.5 * x.d / r : 0.0};
}
inline double absS(double x) { return x >= 0.0 ? x : -x; }
inline Dual absS(Dual x) { return x.v >= 0.0 ? x : -x; }

template <class S>
struct NsQp
{
  S u[2], adv[2], grad[2][2], adv_grad[2], tau;
};

struct NavierGLS
{
  const P1Quad* q;
  double        rho, mu, dt;
  int           step, num_hist;

  double N(int iq, int in) const { return q->N[iq * 3 + in]; }
  double dNdx(int e, int iq, int in, int d) const
  {
    return q->dNdx[((std::size_t(e) * q->nq + iq) * 3 + in) * 2 + d];
  }
  double JxW(int e, int iq) const { return q->JxW[std::size_t(e) * q->nq + iq]; }

  template <class S>
  S elemLength(const NsQp<S>& qp, int e, int iq) const
  {
    S speed2 = 0.0;
    for (int d = 0; d < 2; ++d)
    {
      speed2 += qp.u[d] * qp.u[d];
    }
    const S speed = sqrtS(speed2);
    S       dir[2];
    if (val(speed) > 1.0e-10)
    {
      for (int d = 0; d < 2; ++d)
      {
        dir[d] = qp.u[d] / speed;
      }
    }
    else
    {
      const double c = 1.0 / std::sqrt(2.0);
      dir[0]         = c;
      dir[1]         = c;
    }
    S sum = 0.0;
    for (int in = 0; in < 3; ++in)
    {
      S g = 0.0;
      for (int d = 0; d < 2; ++d)
      {
        g += dir[d] * dNdx(e, iq, in, d);
      }
      sum += absS(g);
    }
    return val(sum) > 1.0e-14 ? S(2.0) / sum : S(0.0);
  }

  template <class S>
  void evalQp(int e, int iq, const S* h0, const S* h1, NsQp<S>& qp) const
  {
    for (int c = 0; c < 2; ++c)
    {
      qp.u[c] = qp.adv[c] = qp.adv_grad[c] = 0.0;
      qp.grad[c][0] = qp.grad[c][1] = 0.0;
    }
    for (int in = 0; in < 3; ++in)
    {
      const double Nv = N(iq, in);
      for (int c = 0; c < 2; ++c)
      {
        const int id = 2 * in + c;
        const S   v  = h0[id];
        qp.u[c] += Nv * v;
        for (int d = 0; d < 2; ++d)
        {
          qp.grad[c][d] += dNdx(e, iq, in, d) * v;
        }
        S adv = v;
        if (step > 0 && num_hist > 1)
        {
          adv = 1.5 * v - 0.5 * h1[id];
        }
        qp.adv[c] += Nv * adv;
      }
    }
    S speed2 = 0.0;
    for (int c = 0; c < 2; ++c)
    {
      speed2 += qp.u[c] * qp.u[c];
      for (int d = 0; d < 2; ++d)
      {
        qp.adv_grad[c] += qp.grad[c][d] * qp.adv[d];
      }
    }
    const S      speed = sqrtS(speed2);
    const S      h     = elemLength(qp, e, iq);
    const double nu    = mu / rho;
    const double time  = (2.0 / dt) * (2.0 / dt);
    S            flow  = 0.0, diff = 0.0;
    if (val(h) > 0.0)
    {
      flow = (2.0 * speed / h) * (2.0 * speed / h);
      diff = (4.0 * nu / (h * h)) * (4.0 * nu / (h * h));
    }
    qp.tau = S(1.0) / sqrtS(time + flow + diff);
  }

  template <class S>
  S advDeriv(const NsQp<S>& qp, int e, int iq, int in) const
  {
    S v = 0.0;
    for (int d = 0; d < 2; ++d)
    {
      v += dNdx(e, iq, in, d) * qp.adv[d];
    }
    return v;
  }

  double gradDot(int e, int iq, int i, int j) const
  {
    double v = 0.0;
    for (int d = 0; d < 2; ++d)
    {
      v += dNdx(e, iq, i, d) * dNdx(e, iq, j, d);
    }
    return v;
  }

  // Row `row` of K (next-state Jacobian) into K[9]; returns K nxt - F.
  template <class S>
  S evalRowT(int e, int row, const S* h0, const S* h1, const double* nxt, S* K) const
  {
    for (int col = 0; col < 9; ++col)
    {
      K[col] = 0.0;
    }
    const bool vel_row = row < 6;
    const int  i       = vel_row ? row / 2 : row - 6;
    const int  c       = vel_row ? row - 2 * i : 0;
    S          F       = 0.0;
    for (int iq = 0; iq < q->nq; ++iq)
    {
      NsQp<S> qp;
      evalQp(e, iq, h0, h1, qp);
      const double Jw  = JxW(e, iq);
      const double Ni  = N(iq, i);
      const S      dvi = advDeriv(qp, e, iq, i);
      if (vel_row)
      {
        S grad_u = 0.0;
        for (int d = 0; d < 2; ++d)
        {
          grad_u += dNdx(e, iq, i, d) * qp.grad[c][d];
        }
        F += (rho / dt * Ni * qp.u[c] - 0.5 * rho * Ni * qp.adv_grad[c] - 0.5 * mu * grad_u
              + qp.tau * rho / dt * dvi * qp.u[c] - 0.5 * qp.tau * rho * dvi * qp.adv_grad[c])
             * Jw;
        for (int j = 0; j < 3; ++j)
        {
          const double Nj  = N(iq, j);
          const S      dvj = advDeriv(qp, e, iq, j);
          K[2 * j + c] += (rho / dt * Ni * Nj + 0.5 * rho * Ni * dvj
                           + 0.5 * mu * gradDot(e, iq, i, j) + qp.tau * rho / dt * dvi * Nj
                           + 0.5 * qp.tau * rho * dvi * dvj)
                          * Jw;
          K[6 + j] += (-dNdx(e, iq, i, c) * Nj + qp.tau * dvi * dNdx(e, iq, j, c)) * Jw;
        }
      }
      else
      {
        S div_u = 0.0, div_adv = 0.0;
        for (int d = 0; d < 2; ++d)
        {
          const double g = dNdx(e, iq, i, d);
          div_u += g * qp.u[d];
          div_adv += g * qp.adv_grad[d];
        }
        F += (qp.tau / dt * div_u - 0.5 * qp.tau * div_adv) * Jw;
        for (int j = 0; j < 3; ++j)
        {
          const double Nj  = N(iq, j);
          const S      dvj = advDeriv(qp, e, iq, j);
          for (int d = 0; d < 2; ++d)
          {
            const double gi = dNdx(e, iq, i, d);
            K[2 * j + d] += (Ni * dNdx(e, iq, j, d) + qp.tau / dt * gi * Nj
                             + 0.5 * qp.tau * gi * dvj)
                            * Jw;
          }
          K[6 + j] += qp.tau / rho * gradDot(e, iq, i, j) * Jw;
        }
      }
    }
    S out = -F;
    for (int col = 0; col < 9; ++col)
    {
      out += K[col] * nxt[col];
    }
    return out;
  }
};

} // namespace

extern "C" {

const char* orc_last_error(void)
{
  return g_err.c_str();
}

void* orc_map_create(int num_res, int num_states, int num_elems,
                     const int* res_offsets, const int* res_dofs,
                     const int* state_offsets, const int* state_dofs)
{
  Map* out = nullptr;
  guarded([&] {
    out = buildMap(num_res, num_states, num_elems, res_offsets, res_dofs,
                   state_offsets, state_dofs);
  });
  return out;
}

void orc_map_sizes(const void* h, long long* s)
{
  const Map& m = *static_cast<const Map*>(h);
  s[0]         = m.row_ptr[m.num_res];
  s[1]         = m.jac_offsets[m.num_elems];
  s[2]         = m.max_res;
  s[3]         = m.max_state;
  s[4]         = m.max_jac;
}

void orc_map_copy(const void* h, int* row_ptr, int* col_ind, int* jac_offsets,
                  int* jac_map)
{
  const Map& m = *static_cast<const Map*>(h);
  std::copy(m.row_ptr.begin(), m.row_ptr.end(), row_ptr);
  std::copy(m.col_ind.begin(), m.col_ind.end(), col_ind);
  std::copy(m.jac_offsets.begin(), m.jac_offsets.end(), jac_offsets);
  std::copy(m.jac_map.begin(), m.jac_map.end(), jac_map);
}

void orc_map_free(void* h)
{
  delete static_cast<Map*>(h);
}

void* orc_bc_create(int num_bcs, const int* dofs, int rows, int cols,
                    const int* row_ptr, const int* col_ind)
{
  Bc* out = nullptr;
  guarded([&] { out = buildBc(num_bcs, dofs, rows, cols, row_ptr, col_ind); });
  return out;
}

void orc_bc_sizes(const void* h, long long* s)
{
  const Bc& b = *static_cast<const Bc*>(h);
  s[0]        = b.num();
  s[1]        = b.col_offsets[b.num()];
}

void orc_bc_copy(const void* h, int* bc_rows, int* diag, int* col_offsets,
                 int* col_entries, int* col_rows, int* bc_mask)
{
  const Bc& b = *static_cast<const Bc*>(h);
  std::copy(b.bc_rows.begin(), b.bc_rows.end(), bc_rows);
  std::copy(b.diag.begin(), b.diag.end(), diag);
  std::copy(b.col_offsets.begin(), b.col_offsets.end(), col_offsets);
  std::copy(b.col_entries.begin(), b.col_entries.end(), col_entries);
  std::copy(b.col_rows.begin(), b.col_rows.end(), col_rows);
  std::copy(b.bc_mask.begin(), b.bc_mask.end(), bc_mask);
}

void orc_bc_free(void* h)
{
  delete static_cast<Bc*>(h);
}

int orc_replace_rows(const void* h, const int* row_ptr, double* vals,
                     double diag)
{
  return guarded(
      [&] { replaceRowsRaw(*static_cast<const Bc*>(h), row_ptr, vals, diag); });
}

int orc_replace_res(const void* h, const double* state, const double* bc_vals,
                    double* res)
{
  return guarded([&] {
    const Bc& b = *static_cast<const Bc*>(h);
    require(state != res && bc_vals != res,
            "BoundaryMap residual output must not alias its inputs");
    for (int ib = 0; ib < b.num(); ++ib)
    {
      const int r = b.bc_rows[ib];
      res[r]      = state[r] - bc_vals[ib];
    }
  });
}

int orc_zero_boundary(const void* h, double* v)
{
  return guarded([&] {
    const Bc& b = *static_cast<const Bc*>(h);
    for (int ib = 0; ib < b.num(); ++ib)
    {
      v[b.bc_rows[ib]] = 0.0;
    }
  });
}

int orc_prepare_forward_solve(const void* h, const int* row_ptr, double* vals,
                              double* rhs, const double* bc_vals)
{
  return guarded([&] {
    const Bc& b = *static_cast<const Bc*>(h);
    require(rhs != bc_vals,
            "BoundaryMap RHS and prescribed values must not alias");
    for (int ib = 0; ib < b.num(); ++ib)
    {
      const double g = bc_vals[ib];
      for (int i = b.col_offsets[ib]; i < b.col_offsets[ib + 1]; ++i)
      {
        const int r = b.col_rows[i];
        const int k = b.col_entries[i];
        if (b.bc_mask[r] == 0)
        {
          rhs[r] -= vals[k] * g;
        }
        vals[k] = 0.0;
      }
    }
    replaceRowsRaw(b, row_ptr, vals, 1.0);
    for (int ib = 0; ib < b.num(); ++ib)
    {
      rhs[b.bc_rows[ib]] = bc_vals[ib];
    }
  });
}

void orc_matvec(int rows, const int* row_ptr, const int* col_ind,
                const double* vals, const double* x, double* y, double alpha,
                double beta)
{
  for (int r = 0; r < rows; ++r)
  {
    double v = 0.0;
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
    {
      v += vals[k] * x[col_ind[k]];
    }
    y[r] = alpha * v + beta * y[r];
  }
}

void orc_matvec_t(int rows, int cols, const int* row_ptr, const int* col_ind,
                  const double* vals, const double* x, double* y, double alpha,
                  double beta)
{
  for (int c = 0; c < cols; ++c)
  {
    y[c] *= beta;
  }
  for (int r = 0; r < rows; ++r)
  {
    const double v = alpha * x[r];
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
    {
      y[col_ind[k]] += vals[k] * v;
    }
  }
}

void* orc_p1_quad_create(int num_nodes, const double* coords, int num_elems,
                         const int* conn, int order)
{
  P1Quad* out = nullptr;
  guarded([&] {
    out = buildP1Quad(num_nodes, coords, num_elems, conn, order);
  });
  return out;
}

void orc_p1_quad_free(void* h)
{
  delete static_cast<P1Quad*>(h);
}

int orc_p1_quad_tables(const void* h, int* nq, const double** N, const double** dNdx,
                       const double** JxW)
{
  return guarded([&] {
    const P1Quad& q = *static_cast<const P1Quad*>(h);
    *nq             = q.nq;
    *N              = q.N.data();
    *dNdx           = q.dNdx.data();
    *JxW            = q.JxW.data();
  });
}

int orc_assemble_p1_kappa(const void* mh, const void* qh, const int* conn,
                          const double* kappa, const double* f_nodal,
                          const double* u, double* res, double* vals)
{
  return guarded([&] {
    const Map&    m = *static_cast<const Map*>(mh);
    const P1Quad& q = *static_cast<const P1Quad*>(qh);
    require(q.ne == m.num_elems,
            "Geometry and AssemblyMap have different element counts");
    require(m.max_res <= 3 && m.max_state <= 3,
            "KappaPoissonP1 expects three DOFs per element");
    const KappaPoissonP1 op{&q, conn, kappa, f_nodal};
    assembleLoop(m, op, u, res, vals);
  });
}

int orc_vjp_p1_kappa(const void* mh, const void* qh, const int* conn,
                     const double* kappa, const double* u, const double* lam,
                     double* g_u, double* g_m)
{
  return guarded([&] {
    const Map&    m = *static_cast<const Map*>(mh);
    const P1Quad& q = *static_cast<const P1Quad*>(qh);
    require(q.ne == m.num_elems,
            "Geometry and AssemblyMap have different element counts");
    const KappaPoissonP1 op{&q, conn, kappa, nullptr};
    if (g_u != nullptr)
    {
      std::fill(g_u, g_u + m.num_states, 0.0);
    }
    double st[3], jac[9], dummy;
    for (int e = 0; e < m.num_elems; ++e)
    {
      double le[3], ue[3];
      for (int i = 0; i < 3; ++i)
      {
        const int dof = m.state_dofs[m.state_offsets[e] + i];
        ue[i]         = u[dof];
        st[i]         = ue[i];
        le[i]         = lam[m.res_dofs[m.res_offsets[e] + i]];
      }
      for (int r = 0; r < 3; ++r)
      {
        op.evalRow(e, r, st, dummy, jac + 3 * r);
      }
      if (g_u != nullptr)
      {
        for (int c = 0; c < 3; ++c)
        {
          double v = 0.0;
          for (int r = 0; r < 3; ++r)
          {
            v += jac[3 * r + c] * le[r];
          }
          g_u[m.state_dofs[m.state_offsets[e] + c]] += v;
        }
      }
      if (g_m != nullptr)
      {
        // d(kappa_e Khat_e u_e)/dm_e = kappa_e Khat_e u_e = K_e u_e.
        double v = 0.0;
        for (int r = 0; r < 3; ++r)
        {
          double ku = 0.0;
          for (int c = 0; c < 3; ++c)
          {
            ku += jac[3 * r + c] * ue[c];
          }
          v += le[r] * ku;
        }
        g_m[e] = v;
      }
    }
  });
}

void* orc_th_quad_create(int num_p2_nodes, const double* coords,
                         int num_elems, const int* conn6)
{
  TaylorHoodNS* out = nullptr;
  guarded([&] {
    auto* t = new TaylorHoodNS;
    try
    {
      t->build(num_p2_nodes, coords, num_elems, conn6);
    }
    catch (...)
    {
      delete t;
      throw;
    }
    out = t;
  });
  return out;
}

void orc_th_quad_free(void* h)
{
  delete static_cast<TaylorHoodNS*>(h);
}

int orc_assemble_th_range(const void* mh, const void* th, double nu,
                          const double* state, double* res, double* vals,
                          int e0, int e1)
{
  return guarded([&] {
    const Map& m = *static_cast<const Map*>(mh);
    require(m.max_res <= 15 && m.max_state <= 15,
            "Taylor-Hood element expects 15 DOFs per element");
    // Borrow the prebuilt tables; only the viscosity is per call.
    struct Op
    {
      const TaylorHoodNS* t;
      double              nu;
      void evalRow(int e, int row, const double* st, double& res, double* jac) const
      {
        t->evalRowNu(nu, e, row, st, res, jac);
      }
    } op{static_cast<const TaylorHoodNS*>(th), nu};
    assembleLoop(m, op, state, res, vals, e0, e1);
  });
}

int orc_assemble_th_threads(const void* mh, const void* th, double nu,
                            const double* state, double* res, double* vals,
                            int nthreads)
{
  return guarded([&] {
    const Map& m = *static_cast<const Map*>(mh);
    require(m.max_res <= 15 && m.max_state <= 15,
            "Taylor-Hood element expects 15 DOFs per element");
    struct Op
    {
      const TaylorHoodNS* t;
      double              nu;
      void evalRow(int e, int row, const double* st, double& res, double* jac) const
      {
        t->evalRowNu(nu, e, row, st, res, jac);
      }
    } op{static_cast<const TaylorHoodNS*>(th), nu};
    assembleLoopThreads(m, op, state, res, vals, nthreads);
  });
}

int orc_assemble_th_ns(const void* mh, int num_p2_nodes, const double* coords,
                       const int* conn6, double nu, const double* state,
                       double* res, double* vals)
{
  return guarded([&] {
    const Map& m = *static_cast<const Map*>(mh);
    require(m.max_res <= 15 && m.max_state <= 15,
            "Taylor-Hood element expects 15 DOFs per element");
    TaylorHoodNS op;
    op.nu = nu;
    op.build(num_p2_nodes, coords, m.num_elems, conn6);
    assembleLoop(m, op, state, res, vals);
  });
}

int orc_assemble_p1_range(const void* mh, const void* qh, const int* conn,
                          const double* kappa, const double* f_nodal,
                          const double* u, double* res, double* vals, int e0,
                          int e1)
{
  return guarded([&] {
    const Map&    m = *static_cast<const Map*>(mh);
    const P1Quad& q = *static_cast<const P1Quad*>(qh);
    require(q.ne == m.num_elems,
            "Geometry and AssemblyMap have different element counts");
    const KappaPoissonP1 op{&q, conn, kappa, f_nodal};
    assembleLoop(m, op, u, res, vals, e0, e1);
  });
}


int orc_assemble_navier(const void* mh, const void* qh, double rho, double mu, double dt,
                        int step, int num_hist, const double* hist, const double* nxt,
                        double* res, double* vals)
{
  return guarded([&] {
    const Map&    m = *static_cast<const Map*>(mh);
    const P1Quad& q = *static_cast<const P1Quad*>(qh);
    require(q.ne == m.num_elems, "Geometry and AssemblyMap have different element counts");
    require(m.max_res <= 9 && m.max_state <= 9,
            "Navier operator expects nine DOFs per P1 triangle");
    require(num_hist > 0, "Time assembly state dimensions do not match AssemblyMap");
    const NavierGLS op{&q, rho, mu, dt, step, num_hist};
    std::fill(res, res + m.num_res, 0.0);
    if (vals != nullptr)
    {
      std::fill(vals, vals + m.row_ptr[m.num_res], 0.0);
    }
    double h0[9], h1[9], xn[9], K[9];
    for (int e = 0; e < m.num_elems; ++e)
    {
      for (int c = 0; c < 9; ++c)
      {
        const int dof = m.state_dofs[m.state_offsets[e] + c];
        h0[c]         = hist[dof];
        h1[c]         = num_hist > 1 ? hist[std::size_t(m.num_states) + dof] : 0.0;
        xn[c]         = nxt[dof];
      }
      for (int r = 0; r < 9; ++r)
      {
        const double rr = op.evalRowT<double>(e, r, h0, h1, xn, K);
        res[m.res_dofs[m.res_offsets[e] + r]] += rr;
        if (vals != nullptr)
        {
          for (int c = 0; c < 9; ++c)
          {
            vals[m.jac_map[m.jac_offsets[e] + 9 * r + c]] += K[c];
          }
        }
      }
    }
  });
}

int orc_vjp_navier_hist(const void* mh, const void* qh, double rho, double mu, double dt,
                        int step, int num_hist, const double* hist, const double* nxt,
                        const double* adj, double* out)
{
  return guarded([&] {
    const Map&    m = *static_cast<const Map*>(mh);
    const P1Quad& q = *static_cast<const P1Quad*>(qh);
    require(q.ne == m.num_elems, "Geometry and AssemblyMap have different element counts");
    require(num_hist > 0, "Time assembly state dimensions do not match AssemblyMap");
    const NavierGLS op{&q, rho, mu, dt, step, num_hist};
    std::fill(out, out + std::size_t(num_hist) * m.num_states, 0.0);
    double xn[9], a[9];
    Dual   h0[9], h1[9], K[9];
    for (int e = 0; e < m.num_elems; ++e)
    {
      int dofs[9];
      for (int c = 0; c < 9; ++c)
      {
        dofs[c] = m.state_dofs[m.state_offsets[e] + c];
        xn[c]   = nxt[dofs[c]];
        a[c]    = adj[m.res_dofs[m.res_offsets[e] + c]];
      }
      for (int lag = 0; lag < std::min(num_hist, 2); ++lag)
      {
        for (int k = 0; k < 9; ++k)
        {
          for (int c = 0; c < 9; ++c)
          {
            h0[c] = Dual(hist[dofs[c]], lag == 0 && c == k ? 1.0 : 0.0);
            h1[c] = Dual(num_hist > 1 ? hist[std::size_t(m.num_states) + dofs[c]] : 0.0,
                         lag == 1 && c == k ? 1.0 : 0.0);
          }
          double g = 0.0;
          for (int r = 0; r < 9; ++r)
          {
            g += a[r] * op.evalRowT<Dual>(e, r, h0, h1, xn, K).d;
          }
          out[std::size_t(lag) * m.num_states + dofs[k]] += g;
        }
      }
    }
  });
}


int orc_assemble_navier_threads(const void* mh, const void* qh, double rho, double mu,
                                double dt, int step, int num_hist, const double* hist,
                                const double* nxt, double* res, double* vals, int nthreads)
{
  return guarded([&] {
    const Map&    m = *static_cast<const Map*>(mh);
    const P1Quad& q = *static_cast<const P1Quad*>(qh);
    require(q.ne == m.num_elems, "Geometry and AssemblyMap have different element counts");
    require(m.max_res <= 9 && m.max_state <= 9,
            "Navier operator expects nine DOFs per P1 triangle");
    const NavierGLS op{&q, rho, mu, dt, step, num_hist};
    struct Row
    {
      const NavierGLS* op;
      const double*    hist;
      const double*    nxt;
      std::size_t      ns;
      const Map*       m;
      void evalRow(int e, int r, const double* st, double& res, double* jac) const
      {
        (void) st;
        double h0[9], h1[9], xn[9];
        for (int c = 0; c < 9; ++c)
        {
          const int dof = m->state_dofs[m->state_offsets[e] + c];
          h0[c]         = hist[dof];
          h1[c]         = op->num_hist > 1 ? hist[ns + dof] : 0.0;
          xn[c]         = nxt[dof];
        }
        res = op->evalRowT<double>(e, r, h0, h1, xn, jac);
      }
    } row{&op, hist, nxt, std::size_t(m.num_states), &m};
    // the generic threaded loop gathers `state` per element; the operator
    // reads the history and next state itself, so pass nxt as the state
    assembleLoopThreads(m, row, nxt, res, vals, nthreads);
  });
}

} // extern "C"
