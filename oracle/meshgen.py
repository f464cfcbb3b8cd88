"""Structured box meshes for the oracle -- TEST INFRASTRUCTURE ONLY.

numpy restatement of the library's structured hexahedral box (the transfinite periodic box of
examples/periodic_3d_ceuler.cpp:60-130), so that the timed CPU baseline and the reference arm of bench.py
build their mesh without loading the GPU library.  Node numbering, hexahedron vertex order, boundary quads
and periodic master nodes equal the library's sdg_mesh_generate_3d bit for bit (tests/test_oracle.py).
The arrays feed the plain mesh holder subrosadg_gb300.Mesh, whose construction loads nothing.
"""
from __future__ import annotations

import numpy as np


def box_3d(x0, y0, z0, lx, ly, lz, nx, ny, nz, periodic=True, boundary_conditions=None):
    """nx x ny x nz hexahedra of [x0, x0+lx] x [y0, y0+ly] x [z0, z0+lz]; periodic = one group with every
    opposite side paired, else six groups x-, x+, y-, y+, z-, z+ with boundary_conditions[0..5]."""
    from subrosadg_gb300.solver import Mesh
    from subrosadg_gb300._abi import PERIODIC

    px, py, pz = nx + 1, ny + 1, nz + 1
    k, j, i = np.meshgrid(np.arange(pz), np.arange(py), np.arange(px), indexing="ij")
    nodes = np.stack([x0 + lx * i.astype(np.float64) / nx, y0 + ly * j.astype(np.float64) / ny,
                      z0 + lz * k.astype(np.float64) / nz], -1).reshape(-1, 3)

    def nid(i, j, k):
        return ((k * py + j) * px + i).astype(np.int32)

    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    hexes = np.stack([nid(I, J, K), nid(I + 1, J, K), nid(I + 1, J + 1, K), nid(I, J + 1, K),
                      nid(I, J, K + 1), nid(I + 1, J, K + 1), nid(I + 1, J + 1, K + 1), nid(I, J + 1, K + 1)], 1)
    quads, groups = [], []
    # x- / x+ interleaved per (k, j), as the library emits them
    K2, J2 = [a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij")]
    z0i, nxi = np.zeros_like(J2), np.full_like(J2, nx)
    xm = [nid(z0i, J2, K2), nid(z0i, J2, K2 + 1), nid(z0i, J2 + 1, K2 + 1), nid(z0i, J2 + 1, K2)]
    xp = [nid(nxi, J2, K2), nid(nxi, J2 + 1, K2), nid(nxi, J2 + 1, K2 + 1), nid(nxi, J2, K2 + 1)]
    K3, I3 = [a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")]
    z0j, nyj = np.zeros_like(I3), np.full_like(I3, ny)
    ym = [nid(I3, z0j, K3), nid(I3 + 1, z0j, K3), nid(I3 + 1, z0j, K3 + 1), nid(I3, z0j, K3 + 1)]
    yp = [nid(I3, nyj, K3), nid(I3, nyj, K3 + 1), nid(I3 + 1, nyj, K3 + 1), nid(I3 + 1, nyj, K3)]
    J4, I4 = [a.ravel() for a in np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")]
    z0k, nzk = np.zeros_like(I4), np.full_like(I4, nz)
    zm = [nid(I4, J4, z0k), nid(I4, J4 + 1, z0k), nid(I4 + 1, J4 + 1, z0k), nid(I4 + 1, J4, z0k)]
    zp = [nid(I4, J4, nzk), nid(I4 + 1, J4, nzk), nid(I4 + 1, J4 + 1, nzk), nid(I4, J4 + 1, nzk)]
    for a, b, ga, gb in ((xm, xp, 1, 2), (ym, yp, 3, 4), (zm, zp, 5, 6)):
        qa, qb = np.stack(a, 1), np.stack(b, 1)
        inter = np.empty((2 * len(qa), 4), np.int32)
        inter[0::2], inter[1::2] = qa, qb
        quads.append(inter)
        g = np.empty(2 * len(qa), np.int32)
        g[0::2], g[1::2] = (1, 1) if periodic else (ga, gb)
        groups.append(g)
    boundary = np.concatenate(quads)
    physical = np.concatenate(groups)
    master = None
    if periodic:
        kk, jj, ii = np.meshgrid(np.arange(pz), np.arange(py), np.arange(px), indexing="ij")
        master = nid(np.where(ii == nx, 0, ii), np.where(jj == ny, 0, jj), np.where(kk == nz, 0, kk)).ravel()
        conditions = np.array([PERIODIC], np.int32)
    else:
        if boundary_conditions is None or len(boundary_conditions) != 6:
            raise ValueError("a non-periodic box needs six boundary conditions")
        conditions = np.asarray(boundary_conditions, np.int32)
    return Mesh(3, nodes, hexahedra=hexes, boundary=boundary, boundary_physical=physical,
                physical_conditions=conditions, periodic_master=master)
