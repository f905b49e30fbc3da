"""Seeded synthetic meshes and fields for the assembly workloads.

Everything here is host-side input generation (numpy); none of it is on the
timed path. Layouts follow femx's flattened geometry
(femx/fem/Geometry.hpp:33-196): node-major coordinates ``coords[N, 2]``
(float64) and element-major connectivity ``conn[E, k]`` (int32).

Meshes
  * ``structured_tri(nx)``: the unit square cut into nx*nx cells, each split
    into two counter-clockwise triangles along the (i,j)-(i+1,j+1) diagonal.
    Nodes are numbered row-major, ``id = j*(nx+1) + i``, like
    ``Mesh::makeStructuredQuad`` (femx/fem/Mesh.cpp:10-51).
  * ``jittered_tri(nx, seed)``: the same topology with interior nodes moved
    by up to ``amp*h`` and, optionally, node and element ids permuted.
  * ``p2_mesh(coords, conn)``: Taylor-Hood geometry — P2 nodes are the
    vertices (ids unchanged) followed by edge midpoints numbered in order of
    first appearance; element nodes are ``[v0 v1 v2 m01 m12 m20]``.

Fields
  * ``fourier_source``: f(x,y) = sum_k a_k sin(pi p_k x) sin(pi q_k y),
    a_k ~ N(0,1), (p_k, q_k) uniform in 1..8.
  * ``grf_centroids``: a Gaussian random field with squared-exponential
    covariance (correlation length ell, variance var) built by a seeded
    spectral method on a periodic grid and sampled at element centroids.
  * ``stream_velocity``: u = (d psi/dy, -d psi/dx) for
    psi = sum_k c_k sin(pi k1 x) sin(pi k2 y), c_k ~ N(0,1)/|k|^2.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "structured_tri",
    "jittered_tri",
    "p2_mesh",
    "th_elem_dofs",
    "scalar_elem_dofs",
    "fourier_source",
    "grf_centroids",
    "stream_velocity",
    "boundary_nodes",
    "dirichlet_dofs",
    "structured_counts",
]


def structured_counts(nx: int) -> dict:
    """Element, node, edge and P1-nonzero counts of ``structured_tri(nx)``."""
    n = (nx + 1) ** 2
    e = 2 * nx * nx
    edges = 2 * nx * (nx + 1) + nx * nx
    return {"elems": e, "nodes": n, "edges": edges, "nnz_p1": n + 2 * edges}


def structured_tri(nx: int, ny: int | None = None):
    ny = nx if ny is None else ny
    xs = np.arange(nx + 1, dtype=np.float64) / nx
    ys = np.arange(ny + 1, dtype=np.float64) / ny
    X, Y = np.meshgrid(xs, ys)  # row j = y index
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    n0 = (j * (nx + 1) + i).ravel()
    n1 = n0 + 1
    n3 = n0 + (nx + 1)
    n2 = n3 + 1
    conn = np.empty((2 * nx * ny, 3), dtype=np.int32)
    conn[0::2] = np.stack([n0, n1, n2], axis=1)
    conn[1::2] = np.stack([n0, n2, n3], axis=1)
    return np.ascontiguousarray(coords), conn


def jittered_tri(nx: int, seed: int, amp: float = 0.2, permute: bool = True):
    """Structured topology, interior nodes perturbed by U(-amp*h, amp*h)."""
    rng = np.random.default_rng(seed)
    coords, conn = structured_tri(nx)
    h = 1.0 / nx
    on_bnd = boundary_nodes(coords)
    jitter = rng.uniform(-amp * h, amp * h, size=coords.shape)
    jitter[on_bnd] = 0.0
    coords = coords + jitter
    if permute:
        n = coords.shape[0]
        perm = rng.permutation(n)  # new id of old node i is inv[i]
        inv = np.empty(n, dtype=np.int64)
        inv[perm] = np.arange(n)
        coords = coords[perm]
        conn = inv[conn].astype(np.int32)
        conn = conn[rng.permutation(conn.shape[0])]
    return np.ascontiguousarray(coords), np.ascontiguousarray(conn, dtype=np.int32)


def p2_mesh(coords: np.ndarray, conn: np.ndarray):
    """Add edge-midpoint nodes; return (coords_p2, conn6, num_vertices)."""
    nv = coords.shape[0]
    e = conn.shape[0]
    local_edges = ((0, 1), (1, 2), (2, 0))
    a = np.concatenate([conn[:, i] for i, _ in local_edges]).astype(np.int64)
    b = np.concatenate([conn[:, j] for _, j in local_edges]).astype(np.int64)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = lo * nv + hi
    # occurrence index in element-major, edge-minor order
    occ = np.concatenate([np.arange(e) * 3 + k for k in range(3)])
    order = np.argsort(occ, kind="stable")
    key_ordered = key[order]
    uniq, first_idx, inverse_ordered = np.unique(
        key_ordered, return_index=True, return_inverse=True
    )
    # number edges by first appearance
    rank_of_uniq = np.empty(len(uniq), dtype=np.int64)
    rank_of_uniq[np.argsort(first_idx, kind="stable")] = np.arange(len(uniq))
    edge_id_ordered = rank_of_uniq[inverse_ordered]
    edge_id = np.empty_like(edge_id_ordered)
    edge_id[order] = edge_id_ordered
    mids = np.empty((len(uniq), 2), dtype=np.float64)
    ulo = uniq // nv
    uhi = uniq % nv
    mids[rank_of_uniq] = 0.5 * (coords[ulo] + coords[uhi])
    coords_p2 = np.concatenate([coords, mids], axis=0)
    conn6 = np.empty((e, 6), dtype=np.int32)
    conn6[:, :3] = conn
    for k in range(3):
        conn6[:, 3 + k] = nv + edge_id[k * e:(k + 1) * e]
    return np.ascontiguousarray(coords_p2), conn6, nv


def scalar_elem_dofs(conn: np.ndarray):
    """(offsets, dofs) of a scalar one-component space (FESpace.cpp:27-54)."""
    e, k = conn.shape
    offsets = (np.arange(e + 1, dtype=np.int64) * k).astype(np.int32)
    return offsets, np.ascontiguousarray(conn.reshape(-1), dtype=np.int32)


def th_elem_dofs(conn6: np.ndarray, num_p2_nodes: int):
    """Taylor-Hood element DOFs following MixedFESpace (MixedFESpace.cpp:57-84).

    Velocity (2 components) first: dof = 2*node + comp, local = 2*a + comp;
    then pressure on the vertices: dof = 2*num_p2_nodes + vertex.
    Returns (offsets, dofs, num_dofs).
    """
    e = conn6.shape[0]
    d = np.empty((e, 15), dtype=np.int64)
    d[:, 0:12:2] = 2 * conn6
    d[:, 1:12:2] = 2 * conn6 + 1
    d[:, 12:15] = 2 * num_p2_nodes + conn6[:, :3]
    offsets = (np.arange(e + 1, dtype=np.int64) * 15).astype(np.int32)
    nd = 2 * num_p2_nodes + int(conn6[:, :3].max()) + 1
    return offsets, np.ascontiguousarray(d.reshape(-1), dtype=np.int32), nd


def navier_elem_dofs(conn: np.ndarray, num_nodes: int):
    """Equal-order P1/P1 element DOFs of femx's NS model (MixedFESpace of a
    2-component velocity field and a pressure field, Helper.cpp:40-50):
    velocity dof = 2*node + comp at local 2*a + comp, pressure dof =
    2*num_nodes + node at local 6 + a. Returns (offsets, dofs, num_dofs)."""
    e = conn.shape[0]
    d = np.empty((e, 9), dtype=np.int64)
    d[:, 0:6:2] = 2 * conn
    d[:, 1:6:2] = 2 * conn + 1
    d[:, 6:9] = 2 * num_nodes + conn
    offsets = (np.arange(e + 1, dtype=np.int64) * 9).astype(np.int32)
    return offsets, np.ascontiguousarray(d.reshape(-1), dtype=np.int32), 3 * num_nodes


def boundary_nodes(coords: np.ndarray, tol: float = 1e-12) -> np.ndarray:
    x, y = coords[:, 0], coords[:, 1]
    return (np.abs(x) < tol) | (np.abs(x - 1) < tol) | (np.abs(y) < tol) | (np.abs(y - 1) < tol)


def dirichlet_dofs(coords: np.ndarray, mask: np.ndarray, comps: int = 1,
                   comp: int = 0, offset: int = 0) -> np.ndarray:
    """Constrained DOFs of a marker, in ascending node order.

    Follows DirichletBC::addBoundary(space, marker, ...) which visits nodes
    in ascending id order (femx/fem/DirichletBC.cpp:127-146); the DOF of node
    n is offset + comps*n + comp (FESpace.cpp:96-106).
    """
    nodes = np.nonzero(mask)[0]
    return (offset + comps * nodes + comp).astype(np.int32)


def fourier_source(coords: np.ndarray, seed: int, nmodes: int = 8) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(nmodes)
    p = rng.integers(1, 9, size=nmodes)
    q = rng.integers(1, 9, size=nmodes)
    x, y = coords[:, 0], coords[:, 1]
    f = np.zeros(coords.shape[0])
    for k in range(nmodes):
        f += a[k] * np.sin(np.pi * p[k] * x) * np.sin(np.pi * q[k] * y)
    return f


def grf_centroids(coords: np.ndarray, conn: np.ndarray, seed: int,
                  ell: float = 0.05, var: float = 1.0, grid: int = 512) -> np.ndarray:
    """Gaussian random field g at element centroids (spectral method)."""
    rng = np.random.default_rng(seed)
    m = grid
    L = 2.0  # periodic box twice the domain to limit wrap-around correlation
    k = np.fft.fftfreq(m, d=L / m)
    KX, KY = np.meshgrid(k, k, indexing="ij")
    # 2-D spectral density of var*exp(-r^2/(2 ell^2))
    S = var * 2.0 * np.pi * ell ** 2 * np.exp(-2.0 * np.pi ** 2 * ell ** 2 * (KX ** 2 + KY ** 2))
    noise = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    field = np.fft.ifft2(noise * np.sqrt(S)).real
    field = (field - field.mean()) / field.std() * np.sqrt(var)
    c = coords[conn].mean(axis=1)  # centroids in [0,1]^2
    gx = c[:, 0] / L * m
    gy = c[:, 1] / L * m
    i0 = np.floor(gx).astype(np.int64)
    j0 = np.floor(gy).astype(np.int64)
    tx = gx - i0
    ty = gy - j0
    i0 %= m
    j0 %= m
    i1 = (i0 + 1) % m
    j1 = (j0 + 1) % m
    return ((1 - tx) * (1 - ty) * field[i0, j0] + tx * (1 - ty) * field[i1, j0]
            + (1 - tx) * ty * field[i0, j1] + tx * ty * field[i1, j1])


def stream_velocity(coords: np.ndarray, seed: int, nmodes: int = 16) -> np.ndarray:
    rng = np.random.default_rng(seed)
    k1 = rng.integers(1, 9, size=nmodes)
    k2 = rng.integers(1, 9, size=nmodes)
    c = rng.standard_normal(nmodes) / (k1 ** 2 + k2 ** 2)
    x, y = coords[:, 0], coords[:, 1]
    u = np.zeros((coords.shape[0], 2))
    for k in range(nmodes):
        a, b = np.pi * k1[k], np.pi * k2[k]
        u[:, 0] += c[k] * np.sin(a * x) * b * np.cos(b * y)
        u[:, 1] -= c[k] * a * np.cos(a * x) * np.sin(b * y)
    return u


def cavity_dirichlet(coords_p2: np.ndarray, num_p2_nodes: int, tol: float = 1e-12):
    """Lid-driven cavity constraints on the Taylor-Hood layout.

    Issued the way a femx user would with DirichletBC (DirichletBC.cpp:127-146,
    ascending nodes per call): lid u_x = 1, lid u_y = 0, walls u_x = 0,
    walls u_y = 0 (lid = nodes with y = 1, corners included), then the
    pressure pin at vertex 0 (gaugeDofs, femx/model/ns/Helper.cpp:61-82).
    Returns (dofs int32, values float64).
    """
    bnd = boundary_nodes(coords_p2, tol)
    lid = np.abs(coords_p2[:, 1] - 1.0) < tol
    wall = bnd & ~lid
    parts = [
        (dirichlet_dofs(coords_p2, lid, comps=2, comp=0), 1.0),
        (dirichlet_dofs(coords_p2, lid, comps=2, comp=1), 0.0),
        (dirichlet_dofs(coords_p2, wall, comps=2, comp=0), 0.0),
        (dirichlet_dofs(coords_p2, wall, comps=2, comp=1), 0.0),
        (np.array([2 * num_p2_nodes], dtype=np.int32), 0.0),
    ]
    dofs = np.concatenate([p[0] for p in parts]).astype(np.int32)
    vals = np.concatenate([np.full(len(p[0]), p[1]) for p in parts])
    return dofs, vals


def cavity_state(coords_p2: np.ndarray, num_vertices: int, seed: int):
    """Seeded Newton iterate: stream-function velocity at the P2 nodes, N(0,1)
    pressure at the vertices; flattened in the Taylor-Hood DOF order."""
    vel = stream_velocity(coords_p2, seed)
    p = np.random.default_rng(seed).standard_normal(num_vertices)
    return np.concatenate([vel.reshape(-1), p])


def boundary_edges(coords: np.ndarray, conn: np.ndarray, tol: float = 1e-12):
    """Edges of a unit-square triangulation that lie on its boundary, with the
    side they lie on (1 bottom, 2 right, 3 top, 4 left)."""
    out = []
    x, y = coords[:, 0], coords[:, 1]
    for e in range(conn.shape[0]):
        for a, b in ((0, 1), (1, 2), (2, 0)):
            i, j = int(conn[e, a]), int(conn[e, b])
            for side, on in ((1, lambda k: abs(y[k]) < tol), (2, lambda k: abs(x[k] - 1) < tol),
                             (3, lambda k: abs(y[k] - 1) < tol), (4, lambda k: abs(x[k]) < tol)):
                if on(i) and on(j):
                    out.append((side, i, j))
    return out


def write_gmsh(path: str, coords: np.ndarray, conn: np.ndarray, version: int = 4,
               tag_offset: int = 100, seed: int = 0):
    """Write a unit-square triangle mesh as an ASCII Gmsh file (2.2 or 4.1)
    with physical groups wall_bottom/right/top/left (1-4, the boundary
    segments) and fluid (5, the triangles). Node tags are a seeded
    permutation shifted by tag_offset, so readers must map tags; a point
    element and a $Comments section are included to be skipped."""
    rng = np.random.default_rng(seed)
    n = coords.shape[0]
    tags = rng.permutation(n) + tag_offset
    edges = boundary_edges(coords, conn)
    names = {1: "wall_bottom", 2: "wall_right", 3: "wall_top", 4: "wall_left"}
    lines = ["$MeshFormat", "2.2 0 8" if version == 2 else "4.1 0 8", "$EndMeshFormat",
             "$Comments", "written by femx_gb300.meshes.write_gmsh $EndComments-not-a-marker",
             "$EndComments", "$PhysicalNames", "5"]
    lines += [f'1 {k} "{v}"' for k, v in names.items()] + ['2 5 "fluid"', "$EndPhysicalNames"]
    if version == 2:
        lines += ["$Nodes", str(n)]
        lines += [f"{tags[i]} {float(coords[i, 0])!r} {float(coords[i, 1])!r} 0" for i in range(n)]
        lines += ["$EndNodes", "$Elements", str(1 + len(edges) + conn.shape[0])]
        k = 1
        lines.append(f"{k} 15 2 0 1 {tags[0]}")
        for side, i, j in edges:
            k += 1
            lines.append(f"{k} 1 2 {side} {side} {tags[i]} {tags[j]}")
        for e in range(conn.shape[0]):
            k += 1
            a, b, c = (int(v) for v in conn[e])
            lines.append(f"{k} 2 2 5 1 {tags[a]} {tags[b]} {tags[c]}")
        lines.append("$EndElements")
    else:
        lines += ["$Entities", "0 4 1 0"]
        for side in range(1, 5):
            lines.append(f"{side} 0 0 0 1 1 0 1 {side} 0")
        lines.append("1 0 0 0 1 1 0 1 5 4 1 2 3 4")
        lines.append("$EndEntities")
        lines += ["$Nodes", f"1 {n} {tags.min()} {tags.max()}", f"2 1 0 {n}"]
        lines += [str(tags[i]) for i in range(n)]
        lines += [f"{float(coords[i, 0])!r} {float(coords[i, 1])!r} 0" for i in range(n)]
        lines.append("$EndNodes")
        by_side = {s: [(i, j) for (s2, i, j) in edges if s2 == s] for s in range(1, 5)}
        nelem = len(edges) + conn.shape[0]
        lines += ["$Elements", f"5 {nelem} 1 {nelem}"]
        k = 0
        for side in range(1, 5):
            lines.append(f"1 {side} 1 {len(by_side[side])}")
            for i, j in by_side[side]:
                k += 1
                lines.append(f"{k} {tags[i]} {tags[j]}")
        lines.append(f"2 1 2 {conn.shape[0]}")
        for e in range(conn.shape[0]):
            k += 1
            a, b, c = (int(v) for v in conn[e])
            lines.append(f"{k} {tags[a]} {tags[b]} {tags[c]}")
        lines.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
