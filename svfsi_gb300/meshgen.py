"""Synthetic tet4 meshes and their CSR sparsity.

* ``kuhn_box``: a structured hex grid with every hex split into 6 tets
  around its main diagonal (Kuhn/Freudenthal split), positively oriented as
  the reference's CHECKIEN leaves tet4 elements
  (Code/Source/svFSI/READMSH.f:1010-1185: node 1/2 swapped when the
  orientation test is positive, so that det(x1-x4, x2-x4, x3-x4) > 0).
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
