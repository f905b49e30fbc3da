// maps.cuh — the device-resident AssemblyMap and BoundaryMap handles.
#pragma once

#include <vector>

#include "common.cuh"

// femx AssemblyMap<Device> (femx/assembly/AssemblyMap.hpp:78-206) plus the
// CSR pattern it owns (CsrPattern.hpp:42-217). All arrays are device memory
// owned by the handle.
struct gbfem_assembly_map
{
  int                num_elems  = 0;
  int                num_res    = 0;
  int                num_states = 0;
  int                nnz        = 0;
  int                jac_nnz    = 0;
  int                max_res = 0, max_state = 0, max_jac = 0;
  int                uniform_res   = -1; // rows per element when uniform
  int                uniform_state = -1; // cols per element when uniform
  bool               same_dofs     = false; // res tables == state tables
  unsigned long long layout_id     = 0;

  int* res_offsets   = nullptr;
  int* res_dofs      = nullptr;
  int* state_offsets = nullptr;
  int* state_dofs    = nullptr;
  int* jac_offsets   = nullptr;
  int* jac_map       = nullptr;
  int* row_ptr       = nullptr;
  int* col_ind       = nullptr;

  // Compact Jacobian scatter map for uniform layouts: one byte per local
  // entry (i, j) giving its in-row position, CSR slot = row_ptr[res_dof(e,
  // i)] + position. Blocks up to 4 columns (P1) are row-major,
  //   jac_pos[(e * uniform_res + i) * 4 + j],
  // wider blocks (up to 16 rows, e.g. Taylor-Hood's 15) column-major,
  //   jac_pos[(e * uniform_state + j) * pos_stride + i],
  // records padded to pos_stride bytes so a kernel loads one record with one
  // vector load. Null when the layout is not uniform or a row has more than
  // 256 entries; kernels then fall back to jac_map.
  unsigned char* jac_pos    = nullptr;
  int            pos_stride = 0;
  // Row-major twin of a column-major jac_pos (blocks of 5..16 columns):
  // jac_pos_rows[(e * uniform_res + i) * 16 + j].
  unsigned char* jac_pos_rows = nullptr;

  // Row-gather tables, built on request by gbfem_assembly_map_enable_gather
  // (uniform maps with 6..16 residual and state DOFs per element and rows up
  // to 256 entries, e.g. Taylor-Hood). A record is one
  // element row (e, i); records are numbered row by row, and within a
  // residual row in ascending (e, i) order:
  //   gather_off[r] .. gather_off[r + 1]   records adding into row r
  //   gather_slot[e * nr + i]              record index of element row (e, i)
  //   gather_pos[k * 16 + j]               in-row CSR position of entry j
  // Element kernels write record k (16 values: the row's entries, padded)
  // to gather_eb and the row's residual term to gather_res; a row kernel
  // then sums each row's records in record order. No atomics: results are
  // bitwise reproducible run to run. gather_eb holds 16 doubles per record
  // (the FP32 path uses the first half of each as 16 floats).
  int            max_in_row_pos = -1; // largest in-row position (uniform maps)
  int            gather_records = 0;
  int*           gather_off     = nullptr;
  int*           gather_slot    = nullptr;
  unsigned char* gather_pos     = nullptr;
  double*        gather_eb      = nullptr;
  double*        gather_res     = nullptr;

  // Element colouring, built on request by
  // gbfem_assembly_map_enable_colouring: no two elements of one colour share
  // a residual or state DOF, so the elements of a colour add into the
  // residual, the matrix and the gradients with plain read-add-writes, no
  // atomics, and colours run one after another: a fixed summation order,
  // bitwise reproducible results. colour_elems lists the elements colour by
  // colour (ascending within a colour); colour c is colour_elems[
  // colour_off[c] .. colour_off[c + 1]) (host copy and device copy).
  int               num_colours = 0;
  std::vector<int>  colour_off_host;
  int*              colour_off   = nullptr;
  int*              colour_elems = nullptr;

  // Owner-computes tiles of a P1 layout, built on request by
  // gbfem_assembly_map_enable_tiles. Every residual row is owned by one
  // tile; a tile's elements are all elements with a vertex among its rows
  // (elements on a tile border belong to two or three tiles and are
  // evaluated once in each). A tiled assembly runs one block per tile: the
  // block evaluates its elements into shared memory, then each owned row
  // sums its entries from there and writes every CSR value and residual
  // entry of the row once (no atomics, no zero fill, bitwise reproducible).
  //   tile_row_off[t] .. [t + 1]    owned rows, ascending: {row, first CSR
  //                                 slot, end slot, first slot in the tile's
  //                                 staged row values} (tile_row_info)
  //   tile_run_off[t] .. [t + 1]    runs of consecutive owned rows, for the
  //                                 coalesced write-out: {first row, its
  //                                 index in the tile, first CSR slot, its
  //                                 index in the staged values}, closed by a
  //                                 sentinel {0, rows, 0, slots} (tile_runs)
  //   tile_elem_off[t] .. [t + 1]   elements (tile_elems, ascending) and
  //                                 their vertices as tile-local indices,
  //                                 three 10-bit fields (tile_conn; bit 30:
  //                                 the tile owns the element, i.e. the row
  //                                 of its first vertex)
  //   tile_vert_off[t] .. [t + 1]   tile vertices: DOF and geometry node
  //   slot_ref[s]                   CSR slot s of an owned row (r, c), c != r:
  //                                 the one or two element edges joining r
  //                                 and c, 13 bits each (bits 0-12, 13-25):
  //                                 edge record 3 l + k (0xfff: none) |
  //                                 carries-residual << 12; the diagonal
  //                                 slot holds 0xffffffff.
  // Edge k of tile element l is the edge opposite its vertex k; its record
  // holds the stiffness entry of the edge and the residual term of vertex
  // k + 1 (mod 3), which the slot of the direction k + 1 -> k + 2 carries:
  // every (element, vertex) residual term is carried by exactly one slot.
  int       num_tiles      = 0;
  int       tile_max_rows  = 0;
  int       tile_max_elems = 0;
  int       tile_max_verts = 0;
  int       tile_max_slots = 0;
  int       tile_max_runs  = 0;     // runs of one tile, sentinel included
  bool      tile_sep_conn  = false; // geometry nodes differ from DOFs
  int*      tile_row_off   = nullptr;
  int4*     tile_row_info  = nullptr;
  int*      tile_run_off   = nullptr;
  int4*     tile_runs      = nullptr;
  int*      tile_elem_off  = nullptr;
  int*      tile_elems     = nullptr;
  unsigned* tile_conn      = nullptr;
  int*      tile_vert_off  = nullptr;
  int*      tile_vert_dof  = nullptr;
  int*      tile_vert_node = nullptr;
  unsigned* slot_ref       = nullptr;

  // Status word written by hot-path kernels that meet invalid data
  // (degenerate elements); read by gbfem_assembly_map_check().
  gbfem::DeviceStatus* status = nullptr;

  ~gbfem_assembly_map();
};

// femx BoundaryMap<Device> (femx/assembly/BoundaryMap.hpp:69-175) plus a
// row-grouped view of the constrained-column entries that lets the lifting
// run one thread per affected row, without atomics, applying subtractions
// in constraint order (identical to BoundaryMap.cpp:224-238).
struct gbfem_boundary_map
{
  int                num_rows = 0, num_cols = 0, nnz = 0, num_bcs = 0;
  int                num_col_entries = 0;
  unsigned long long layout_id       = 0;

  int* bc_rows     = nullptr;
  int* diag        = nullptr;
  int* col_offsets = nullptr;
  int* col_entries = nullptr;
  int* col_rows    = nullptr;
  int* bc_mask     = nullptr;
  int* row_begin   = nullptr; // CSR extent of each constrained row
  int* row_end     = nullptr;

  // Lifting list: unconstrained rows touching constrained columns.
  int  num_lift_rows = 0;
  int* lift_rows     = nullptr; // [num_lift_rows]
  int* lift_offsets  = nullptr; // [num_lift_rows + 1]
  int* lift_k        = nullptr; // CSR slot, sorted by constraint index
  int* lift_ib       = nullptr; // constraint index of that column

  ~gbfem_boundary_map();
};

namespace gbfem
{
unsigned long long nextLayoutId();
}
