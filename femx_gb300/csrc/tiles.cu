// tiles.cu — owner-computes tiles for the atomic-free P1 assembly (setup).
//
// femx's assembly adds every element block into the CSR values with
// scattered additions: serially on the CPU (Assembly.hpp:186-223), with
// FP64 atomics on the GPU (CudaAssembly.hpp:160-168). On GB300 the FP64
// reductions at L2 bound a P1 element pass well below the HBM roofline (12
// reductions per element), and they need a zero-filled output first. The
// tiled assembly instead gives every residual row one owner: a tile of
// rows that are close in space, whose block evaluates all elements touching
// those rows into shared memory and then writes each of its rows once. This
// file builds the tiles from the map's DOF table and the mesh coordinates:
//   1. rows are ordered along a Morton (Z-order) curve of their vertex
//      coordinates, so consecutive rows are close in space;
//   2. tiles are greedy runs of that order, closed when a tile would exceed
//      256 rows, 512 elements (two per thread of the 256-thread block that
//      evaluates them) or 1024 vertices (the field width of the tile-local
//      vertex indices);
//   3. for every CSR slot (r, c), c != r, of a row the slot records which
//      one or two element edges join r and c (a P1 edge belongs to at most
//      two triangles of a conforming mesh; more is refused), and which
//      element residual terms the slot carries.
// The tiles depend on the mesh topology only; the coordinates steer the
// locality. Setup on the host (like the colouring): reads the DOF table,
// the connectivity, the coordinates and the pattern back, allocates and
// synchronizes.
#include <algorithm>
#include <numeric>
#include <vector>

#include "maps.cuh"

namespace
{
using gbfem::cudaCheck;
using gbfem::require;

constexpr int kTileRows  = 256;
constexpr int kTileElems = 512;
constexpr int kTileVerts = 1024;

template <class T>
std::vector<T> readBack(const T* d, long long n, cudaStream_t s)
{
  std::vector<T> h(static_cast<size_t>(n > 0 ? n : 0));
  if (n > 0)
  {
    cudaCheck(cudaMemcpyAsync(h.data(), d, sizeof(T) * static_cast<size_t>(n),
                              cudaMemcpyDeviceToHost, s),
              "tile setup readback");
  }
  return h;
}

template <class T>
T* upload(const std::vector<T>& h, cudaStream_t s)
{
  T* d = gbfem::deviceAlloc<T>(static_cast<long long>(h.size()));
  if (!h.empty())
  {
    cudaCheck(cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s),
              "tile setup upload");
  }
  return d;
}

// interleaves the low 16 bits of x with zeros (bit i -> bit 2i)
unsigned spread16(unsigned x)
{
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

struct Tiles
{
  int                   max_rows = 0, max_elems = 0, max_verts = 0, max_slots = 0, max_runs = 0;
  std::vector<int>      row_off{0}, rows, run_off{0}, elem_off{0}, elems, vert_off{0},
      vert_dof, vert_node;
  std::vector<int4>     row_info, runs;
  std::vector<unsigned> conn, slot_ref;
};

Tiles buildTiles(int ne, int nrows, const std::vector<int>& dofs,
                 const std::vector<int>& nodes, const std::vector<double>& xy,
                 const std::vector<int>& row_ptr, const std::vector<int>& col_ind)
{
  const int nn = static_cast<int>(xy.size() / 2);
  // one geometry node per DOF, three distinct DOFs per element
  std::vector<int> dof_node(nrows, -1);
  for (int e = 0; e < ne; ++e)
  {
    const int* d = &dofs[3 * static_cast<size_t>(e)];
    require(d[0] != d[1] && d[0] != d[2] && d[1] != d[2],
            "tiled assembly needs three distinct DOFs per element");
    for (int v = 0; v < 3; ++v)
    {
      const int n = nodes[3 * static_cast<size_t>(e) + v];
      require(n >= 0 && n < nn, "Geometry node index out of range");
      require(dof_node[d[v]] < 0 || dof_node[d[v]] == n,
              "tiled assembly needs one geometry node per DOF");
      dof_node[d[v]] = n;
    }
  }
  // 1. Morton order of the rows (rows without elements last)
  double xmin = 0, xmax = 0, ymin = 0, ymax = 0;
  bool   first = true;
  for (int r = 0; r < nrows; ++r)
  {
    if (dof_node[r] < 0)
    {
      continue;
    }
    const double x = xy[2 * static_cast<size_t>(dof_node[r])];
    const double y = xy[2 * static_cast<size_t>(dof_node[r]) + 1];
    xmin  = first ? x : std::min(xmin, x);
    xmax  = first ? x : std::max(xmax, x);
    ymin  = first ? y : std::min(ymin, y);
    ymax  = first ? y : std::max(ymax, y);
    first = false;
  }
  const double sx = xmax > xmin ? 65535.0 / (xmax - xmin) : 0.0;
  const double sy = ymax > ymin ? 65535.0 / (ymax - ymin) : 0.0;
  std::vector<unsigned long long> key(nrows);
  for (int r = 0; r < nrows; ++r)
  {
    unsigned m = 0xffffffffu;
    if (dof_node[r] >= 0)
    {
      const double x  = xy[2 * static_cast<size_t>(dof_node[r])];
      const double y  = xy[2 * static_cast<size_t>(dof_node[r]) + 1];
      const auto   qx = static_cast<unsigned>(std::min(65535.0, std::max(0.0, (x - xmin) * sx)));
      const auto   qy = static_cast<unsigned>(std::min(65535.0, std::max(0.0, (y - ymin) * sy)));
      m               = spread16(qx) | (spread16(qy) << 1);
    }
    key[r] = (static_cast<unsigned long long>(m) << 32) | static_cast<unsigned>(r);
  }
  std::sort(key.begin(), key.end());
  // row -> element adjacency
  std::vector<int> adj_off(nrows + 1, 0), adj(3 * static_cast<size_t>(ne));
  for (int i = 0; i < 3 * ne; ++i)
  {
    ++adj_off[dofs[i] + 1];
  }
  std::partial_sum(adj_off.begin(), adj_off.end(), adj_off.begin());
  {
    std::vector<int> next(adj_off.begin(), adj_off.end() - 1);
    for (int i = 0; i < 3 * ne; ++i)
    {
      adj[next[dofs[i]]++] = i / 3;
    }
  }
  // 2. greedy tiles along the Morton order
  Tiles            T;
  std::vector<int> owner(nrows, -1), stamp_e(ne, -1), stamp_v(nrows, -1), trial_v(nrows, -1);
  std::vector<int> cur_elems, cur_verts, cur_rows;
  std::vector<int> vloc(nrows, -1);
  int              t = 0, trial = 0;
  auto             close = [&] {
    std::sort(cur_rows.begin(), cur_rows.end());
    std::sort(cur_elems.begin(), cur_elems.end());
    std::sort(cur_verts.begin(), cur_verts.end());
    T.rows.insert(T.rows.end(), cur_rows.begin(), cur_rows.end());
    int nslots = 0;
    for (size_t i = 0; i < cur_rows.size(); ++i)
    {
      const int r = cur_rows[i];
      if (i == 0 || r != cur_rows[i - 1] + 1)
      {
        T.runs.push_back(int4{r, static_cast<int>(i), row_ptr[r], nslots});
      }
      T.row_info.push_back(int4{r, row_ptr[r], row_ptr[r + 1], nslots});
      nslots += row_ptr[r + 1] - row_ptr[r];
    }
    T.runs.push_back(int4{0, static_cast<int>(cur_rows.size()), 0, nslots});
    T.max_slots = std::max(T.max_slots, nslots);
    T.max_runs  = std::max(T.max_runs, static_cast<int>(T.runs.size()) - T.run_off.back());
    T.run_off.push_back(static_cast<int>(T.runs.size()));
    for (size_t i = 0; i < cur_verts.size(); ++i)
    {
      vloc[cur_verts[i]] = static_cast<int>(i);
      T.vert_dof.push_back(cur_verts[i]);
      T.vert_node.push_back(dof_node[cur_verts[i]]);
    }
    for (int e : cur_elems)
    {
      const int* d = &dofs[3 * static_cast<size_t>(e)];
      T.elems.push_back(e);
      // bit 30: this tile owns the element (the row of its first vertex),
      // the one tile that writes per-element outputs
      T.conn.push_back(static_cast<unsigned>(vloc[d[0]])
                       | (static_cast<unsigned>(vloc[d[1]]) << 10)
                       | (static_cast<unsigned>(vloc[d[2]]) << 20)
                       | (owner[d[0]] == t ? 0x40000000u : 0u));
    }
    T.max_rows  = std::max(T.max_rows, static_cast<int>(cur_rows.size()));
    T.max_elems = std::max(T.max_elems, static_cast<int>(cur_elems.size()));
    T.max_verts = std::max(T.max_verts, static_cast<int>(cur_verts.size()));
    T.row_off.push_back(static_cast<int>(T.rows.size()));
    T.elem_off.push_back(static_cast<int>(T.elems.size()));
    T.vert_off.push_back(static_cast<int>(T.vert_dof.size()));
    cur_rows.clear();
    cur_elems.clear();
    cur_verts.clear();
    ++t;
  };
  // elements and vertices that row r would add to the open tile
  auto count_new = [&](int r, int& ne_new, int& nv_new) {
    ne_new = nv_new = 0;
    ++trial;
    for (int k = adj_off[r]; k < adj_off[r + 1]; ++k)
    {
      const int e = adj[k];
      if (stamp_e[e] == t)
      {
        continue;
      }
      ++ne_new;
      for (int v = 0; v < 3; ++v)
      {
        const int d = dofs[3 * static_cast<size_t>(e) + v];
        if (stamp_v[d] != t && trial_v[d] != trial)
        {
          trial_v[d] = trial;
          ++nv_new;
        }
      }
    }
  };
  for (int i = 0; i < nrows; ++i)
  {
    const int r     = static_cast<int>(key[i] & 0xffffffffull);
    int       add_e = 0, add_v = 0;
    count_new(r, add_e, add_v);
    if (!cur_rows.empty()
        && (static_cast<int>(cur_rows.size()) + 1 > kTileRows
            || static_cast<int>(cur_elems.size()) + add_e > kTileElems
            || static_cast<int>(cur_verts.size()) + add_v > kTileVerts))
    {
      close();
      count_new(r, add_e, add_v);
    }
    require(add_e <= kTileElems && add_v <= kTileVerts,
            "tiled assembly: one row touches more elements than a tile holds");
    owner[r] = t;
    cur_rows.push_back(r);
    for (int k = adj_off[r]; k < adj_off[r + 1]; ++k)
    {
      const int e = adj[k];
      if (stamp_e[e] == t)
      {
        continue;
      }
      stamp_e[e] = t;
      cur_elems.push_back(e);
      for (int v = 0; v < 3; ++v)
      {
        const int d = dofs[3 * static_cast<size_t>(e) + v];
        if (stamp_v[d] != t)
        {
          stamp_v[d] = t;
          cur_verts.push_back(d);
        }
      }
    }
  }
  if (!cur_rows.empty())
  {
    close();
  }
  // 3. slot records
  T.slot_ref.assign(col_ind.size(), 0xffffffffu);
  const int ntiles = static_cast<int>(T.row_off.size()) - 1;
  for (int tt = 0; tt < ntiles; ++tt)
  {
    for (int l = 0; l < T.elem_off[tt + 1] - T.elem_off[tt]; ++l)
    {
      const int  e = T.elems[T.elem_off[tt] + l];
      const int* d = &dofs[3 * static_cast<size_t>(e)];
      for (int k = 0; k < 3; ++k)
      {
        const int ends[2] = {(k + 1) % 3, (k + 2) % 3};
        for (int w = 0; w < 2; ++w)
        {
          const int vr = ends[w], vc = ends[1 - w];
          const int r = d[vr], c = d[vc];
          if (owner[r] != tt)
          {
            continue;
          }
          const int* b  = col_ind.data() + row_ptr[r];
          const int* en = col_ind.data() + row_ptr[r + 1];
          const int* it = std::lower_bound(b, en, c);
          require(it != en && *it == c, "tiled assembly: the CSR pattern lacks an element entry");
          // edge record 3 l + k; the direction from vertex k+1 to vertex
          // k+2 carries the residual term of vertex k+1
          const unsigned ref = static_cast<unsigned>(3 * l + k) | (w == 0 ? 0x1000u : 0u);
          unsigned& slot = T.slot_ref[static_cast<size_t>(it - col_ind.data())];
          if (slot == 0xffffffffu)
          {
            slot = ref | (0xfffu << 13);
          }
          else
          {
            require((slot >> 13) == 0xfffu,
                    "tiled assembly: more than two elements share an edge");
            slot = (slot & 0x1fffu) | (ref << 13);
          }
        }
      }
    }
  }
  return T;
}

} // namespace

extern "C" int gbfem_assembly_map_enable_tiles(gbfem_assembly_map* m, int num_nodes,
                                               const double* coords, const int* conn,
                                               void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(m != nullptr, "AssemblyMap handle is null");
    if (m->tile_row_off != nullptr)
    {
      return;
    }
    require(m->num_elems == 0
                || (m->uniform_res == 3 && m->uniform_state == 3 && m->same_dofs
                    && m->num_res == m->num_states),
            "tiled assembly needs a P1 layout: three identical residual and state DOFs "
            "per element");
    require(num_nodes >= 0 && (m->num_elems == 0 || coords != nullptr),
            "Geometry coordinates must not be null");
    cudaStream_t           s  = asStream(stream);
    const int              ne = m->num_elems;
    const std::vector<int> dofs = readBack(m->state_dofs, 3LL * ne, s);
    std::vector<int> nodes = conn != nullptr ? readBack(conn, 3LL * ne, s) : std::vector<int>();
    const std::vector<double> xy = readBack(coords, 2LL * num_nodes, s);
    const std::vector<int>    rp = readBack(m->row_ptr, m->num_res + 1LL, s);
    const std::vector<int>    ci = readBack(m->col_ind, static_cast<long long>(m->nnz), s);
    cudaCheck(cudaStreamSynchronize(s), "tile setup readback");
    if (conn == nullptr)
    {
      nodes = dofs;
    }
    const Tiles T          = buildTiles(ne, m->num_res, dofs, nodes, xy, rp, ci);
    int*        d_row_off  = nullptr;
    int4*       d_rinfo    = nullptr;
    int*        d_run_off  = nullptr;
    int4*       d_runs     = nullptr;
    int*        d_elem_off = nullptr;
    int*        d_elems    = nullptr;
    unsigned*   d_conn     = nullptr;
    int*        d_vert_off = nullptr;
    int*        d_vdof     = nullptr;
    int*        d_vnode    = nullptr;
    unsigned*   d_ref      = nullptr;
    try
    {
      d_row_off  = upload(T.row_off, s);
      d_rinfo    = upload(T.row_info, s);
      d_run_off  = upload(T.run_off, s);
      d_runs     = upload(T.runs, s);
      d_elem_off = upload(T.elem_off, s);
      d_elems    = upload(T.elems, s);
      d_conn     = upload(T.conn, s);
      d_vert_off = upload(T.vert_off, s);
      d_vdof     = upload(T.vert_dof, s);
      d_vnode    = upload(T.vert_node, s);
      d_ref      = upload(T.slot_ref, s);
      cudaCheck(cudaStreamSynchronize(s), "tile setup upload");
    }
    catch (...)
    {
      for (int* p : {d_row_off, d_run_off, d_elem_off, d_elems, d_vert_off, d_vdof, d_vnode})
      {
        deviceFree(p);
      }
      deviceFree(d_rinfo);
      deviceFree(d_runs);
      deviceFree(d_conn);
      deviceFree(d_ref);
      throw;
    }
    m->num_tiles      = static_cast<int>(T.row_off.size()) - 1;
    m->tile_max_rows  = T.max_rows;
    m->tile_max_elems = T.max_elems;
    m->tile_max_verts = T.max_verts;
    m->tile_sep_conn  = conn != nullptr;
    m->tile_max_slots = T.max_slots;
    m->tile_max_runs  = T.max_runs;
    m->tile_row_off   = d_row_off;
    m->tile_row_info  = d_rinfo;
    m->tile_run_off   = d_run_off;
    m->tile_runs      = d_runs;
    m->tile_elem_off  = d_elem_off;
    m->tile_elems     = d_elems;
    m->tile_conn      = d_conn;
    m->tile_vert_off  = d_vert_off;
    m->tile_vert_dof  = d_vdof;
    m->tile_vert_node = d_vnode;
    m->slot_ref       = d_ref;
  });
}

extern "C" int gbfem_assembly_map_num_tiles(const gbfem_assembly_map* m)
{
  return m != nullptr ? m->num_tiles : 0;
}
