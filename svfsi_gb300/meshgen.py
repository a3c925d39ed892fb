"""Synthetic tet4 meshes and their CSR sparsity.

* ``kuhn_box``: a structured hex grid with every hex split into 6 tets
  around its main diagonal (Kuhn/Freudenthal split), positively oriented as
  the reference's CHECKIEN leaves tet4 elements
  (Code/Source/svFSI/READMSH.f:1010-1185: node 1/2 swapped when the
  orientation test is positive, so that det(x1-x4, x2-x4, x3-x4) > 0).
* ``cylinder``: a seeded Delaunay cross-section extruded into a tet4
  cylinder (inlet, outlet and wall node sets included).
* ``csr_from_ien``: sorted unique column lists per row, the result of LHSA
  (Code/Source/svFSI/LHSA.f:38-262) for a single tet4 mesh.
"""
from __future__ import annotations

import itertools

import numpy as np


def kuhn_box(nx: int, ny: int, nz: int, Lx: float = 1.0, Ly: float = 1.0, Lz: float = 1.0,
             origin=(0.0, 0.0, 0.0)):
    """Return (x[nNo,3] float64, ien[nEl,4] int32 0-based)."""
    xs = np.linspace(0.0, Lx, nx + 1) + origin[0]
    ys = np.linspace(0.0, Ly, ny + 1) + origin[1]
    zs = np.linspace(0.0, Lz, nz + 1) + origin[2]
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    # node id = i + (nx+1)*(j + (ny+1)*k)
    x = np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(),
                  Z.transpose(2, 1, 0).ravel()], axis=1).astype(np.float64)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()

    def nid(di, dj, dk):
        return (i + di) + (nx + 1) * ((j + dj) + (ny + 1) * (k + dk))

    e = np.eye(3, dtype=int)
    tets = []
    for perm in itertools.permutations(range(3)):
        p0 = np.zeros(3, dtype=int)
        p1 = p0 + e[perm[0]]
        p2 = p1 + e[perm[1]]
        p3 = np.ones(3, dtype=int)
        verts = [p0, p1, p2, p3]
        # orientation of this tet type on a unit cube
        v = np.array(verts, dtype=float)
        jac = np.linalg.det(np.stack([v[0] - v[3], v[1] - v[3], v[2] - v[3]], axis=1))
        if jac < 0:
            verts = [verts[1], verts[0], verts[2], verts[3]]
        tets.append(np.stack([nid(*vv) for vv in verts], axis=1))
    # element order: hex-major, the 6 tets of a hex consecutive
    ien = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return x, ien


def cylinder(R: float = 0.5, L: float = 5.0, h: float = 0.027, seed: int = 20261203):
    """Seeded tet4 mesh of the cylinder r <= R, 0 <= z <= L.

    The cross-section is the 2-D Delaunay triangulation (scipy) of points on
    concentric rings (spacing ~h; interior rings jittered with the seed, the
    boundary ring exactly on the circle), extruded into round(L/h) layers of
    prisms.  Each prism is split into three tets with the diagonal of every
    side quad running from its lower-numbered bottom node to its
    higher-numbered top node, which keeps neighbouring prisms conforming.
    Elements are oriented like ``kuhn_box`` (positive Jacobian).
    Returns (x[nNo,3], ien[nEl,4] int32, info) with info holding the node
    sets ``inlet`` (z = 0), ``outlet`` (z = L), ``wall`` (r = R) and the
    inlet faces.
    """
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    nr = max(1, int(round(R / h)))
    pts = [np.zeros((1, 2))]
    for k in range(1, nr + 1):
        r = R * k / nr
        n = max(6, int(round(2.0 * np.pi * r / h)))
        th = 2.0 * np.pi * (np.arange(n) + (0.5 if k % 2 else 0.0)) / n
        if k < nr:
            th = th + rng.uniform(-0.15, 0.15, n) * (2.0 * np.pi / n)
            rr = r + rng.uniform(-0.1, 0.1, n) * (R / nr)
        else:
            th = 2.0 * np.pi * np.arange(n) / n
            rr = np.full(n, r)
        pts.append(np.stack([rr * np.cos(th), rr * np.sin(th)], axis=1))
    p2 = np.concatenate(pts, axis=0)
    n2 = p2.shape[0]
    tri = np.sort(Delaunay(p2).simplices.astype(np.int64), axis=1)
    nz = max(1, int(round(L / h)))
    zs = np.linspace(0.0, L, nz + 1)
    x = np.concatenate([np.concatenate([p2, np.full((n2, 1), z)], axis=1) for z in zs])
    a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
    tets = []
    for k in range(nz):
        o0, o1 = k * n2, (k + 1) * n2
        tets.append(np.stack([a + o0, b + o0, c + o0, c + o1], axis=1))
        tets.append(np.stack([a + o0, b + o0, b + o1, c + o1], axis=1))
        tets.append(np.stack([a + o0, a + o1, b + o1, c + o1], axis=1))
    ien = np.concatenate(tets, axis=0)
    jac = tet_jacobians(x, ien)
    neg = jac < 0
    ien[neg, 0], ien[neg, 1] = ien[neg, 1].copy(), ien[neg, 0].copy()
    ien = ien.astype(np.int32)
    ring = np.arange(n2 - int(round(2.0 * np.pi * R / h)) if nr else 0, n2)
    ring = ring[np.abs(np.hypot(p2[ring, 0], p2[ring, 1]) - R) <= 1e-12 * max(R, 1.0)]
    wall = (ring[None, :] + (np.arange(nz + 1) * n2)[:, None]).ravel().astype(np.int32)
    info = dict(inlet=np.arange(n2, dtype=np.int32),
                outlet=(np.arange(n2) + nz * n2).astype(np.int32), wall=np.sort(wall),
                inlet_faces=faces_on_plane(x, ien, 2, 0.0), n2=n2, nz=nz)
    return x, ien, info


def parabolic_profile(x: np.ndarray, faces: np.ndarray, face_nodes: np.ndarray,
                      perimeter: np.ndarray) -> np.ndarray:
    """Spatial profile gx of a parabolic Dirichlet face (BCINI,
    Code/Source/svFSI/BAFINI.f:362-403): centre = area-weighted centroid of
    the face; for each face node the perimeter node whose unit direction from
    the centre has the largest projection on the node's offset, and
    gx = 1 - |x - c|^2 / |x_perimeter - c|^2."""
    p0, p1, p2 = x[faces[:, 0]], x[faces[:, 1]], x[faces[:, 2]]
    area = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0), axis=1)
    center = (area[:, None] * (p0 + p1 + p2) / 3.0).sum(axis=0) / area.sum()
    sV = x[perimeter] - center
    sVl = sV / np.sqrt((sV * sV).sum(axis=1))[:, None]
    nV = x[face_nodes] - center
    proj = nV @ sVl.T
    i = np.argmax(proj, axis=1)  # first maximum, as the strict '>' scan
    return 1.0 - (nV * nV).sum(axis=1) / (sV[i] * sV[i]).sum(axis=1)


def tet_jacobians(x: np.ndarray, ien: np.ndarray) -> np.ndarray:
    """det(x1-x4, x2-x4, x3-x4) per element (GNN's Jac for tet4)."""
    a = x[ien[:, 0]] - x[ien[:, 3]]
    b = x[ien[:, 1]] - x[ien[:, 3]]
    c = x[ien[:, 2]] - x[ien[:, 3]]
    return np.einsum("ij,ij->i", a, np.cross(b, c))


def nodes_on_plane(x: np.ndarray, axis: int, value: float, tol: float = 1e-12) -> np.ndarray:
    return np.nonzero(np.abs(x[:, axis] - value) <= tol)[0].astype(np.int32)


def faces_on_plane(x: np.ndarray, ien: np.ndarray, axis: int, value: float,
                   tol: float = 1e-12) -> np.ndarray:
    """tri3 boundary faces (0-based node triples) of tets lying on a plane."""
    on = np.abs(x[:, axis] - value) <= tol
    faces = []
    for drop in range(4):
        f = np.delete(ien, drop, axis=1)
        m = on[f].all(axis=1)
        faces.append(f[m])
    return np.concatenate(faces, axis=0).astype(np.int32)


def csr_from_ien(nNo: int, ien: np.ndarray):
    """0-based rowPtr[nNo+1], colPtr[nnz] with sorted unique columns per row."""
    eNoN = ien.shape[1]
    rows = np.repeat(ien, eNoN, axis=1).ravel().astype(np.int64)
    cols = np.tile(ien, (1, eNoN)).ravel().astype(np.int64)
    key = np.unique(rows * nNo + cols)
    r = (key // nNo).astype(np.int32)
    c = (key % nNo).astype(np.int32)
    rowPtr = np.zeros(nNo + 1, dtype=np.int32)
    np.add.at(rowPtr, r + 1, 1)
    rowPtr = np.cumsum(rowPtr).astype(np.int32)
    if np.any(np.diff(rowPtr) == 0):
        raise ValueError("isolated node in mesh")
    return rowPtr, c
