"""Meshes for the monodomain step, in OpenFOAM's lduMesh form.

``box_mesh`` builds what blockMesh makes of one hex block with uniform
spacing: cells numbered x fastest, internal faces in upper-triangular order
(per owner: +x, +y, +z neighbour), face area vectors pointing from owner to
neighbour, and deltaCoeffs = 1/|d_PN|.  The arithmetic (point coordinates
l*i/n, centres as the mean of the two bounding points) is the same sequence
of IEEE operations the CPU oracle uses, so both see identical geometry.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np


@dataclass
class LduMesh:
    n_cells: int
    owner: np.ndarray            # int32 [nf]
    neighbour: np.ndarray        # int32 [nf]
    volumes: np.ndarray          # [n]
    centres: np.ndarray          # [n, 3]
    face_sf: np.ndarray          # [nf, 3]
    face_delta_coeffs: np.ndarray  # [nf]
    structured: Tuple[int, int, int] = (0, 0, 0)

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    def face_coeff(self, sigma) -> np.ndarray:
        """deltaCoeffs * (Sf . sigma . Sf)/|Sf| for a uniform symmTensor sigma
        (xx xy xz yy yz zz), evaluated in the same order as the library."""
        s = sigma
        S = self.face_sf
        mag = np.sqrt(S[:, 0] * S[:, 0] + S[:, 1] * S[:, 1] + S[:, 2] * S[:, 2])
        g0 = S[:, 0] * s[0] + S[:, 1] * s[1] + S[:, 2] * s[2]
        g1 = S[:, 0] * s[1] + S[:, 1] * s[3] + S[:, 2] * s[4]
        g2 = S[:, 0] * s[2] + S[:, 1] * s[4] + S[:, 2] * s[5]
        sfgsn = (g0 * S[:, 0] + g1 * S[:, 1] + g2 * S[:, 2]) / mag
        return self.face_delta_coeffs * sfgsn


def box_mesh(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float) -> LduMesh:
    i = np.arange(nx, dtype=np.float64)
    j = np.arange(ny, dtype=np.float64)
    k = np.arange(nz, dtype=np.float64)
    x0, x1 = lx * i / nx, lx * (i + 1) / nx
    y0, y1 = ly * j / ny, ly * (j + 1) / ny
    z0, z1 = lz * k / nz, lz * (k + 1) / nz
    cx, cy, cz = 0.5 * (x0 + x1), 0.5 * (y0 + y1), 0.5 * (z0 + z1)
    n = nx * ny * nz
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    centres = np.stack([cx[I], cy[J], cz[K]], axis=-1).reshape(n, 3)
    vol = ((x1 - x0)[I] * (y1 - y0)[J] * (z1 - z0)[K]).reshape(n)
    cid = np.arange(n, dtype=np.int64).reshape(nz, ny, nx)
    ax, ay, az = (ly / ny) * (lz / nz), (lx / nx) * (lz / nz), (lx / nx) * (ly / ny)
    # faces per owner cell in the order +x, +y, +z: build (owner, dir) pairs
    owners, nbrs, dirs = [], [], []
    for d, ok in enumerate(((I + 1 < nx), (J + 1 < ny), (K + 1 < nz))):
        o = cid[ok]
        owners.append(o)
        nbrs.append(o + (1, nx, nx * ny)[d])
        dirs.append(np.full(o.shape, d))
    owner = np.concatenate(owners)
    neigh = np.concatenate(nbrs)
    dirv = np.concatenate(dirs)
    order = np.lexsort((dirv, owner))        # by owner, then +x,+y,+z
    owner, neigh, dirv = owner[order], neigh[order], dirv[order]
    sf = np.zeros((owner.size, 3))
    area = np.array([ax, ay, az])
    sf[np.arange(owner.size), dirv] = area[dirv]
    delta = centres[neigh, dirv] - centres[owner, dirv]
    return LduMesh(n_cells=n, owner=owner.astype(np.int32), neighbour=neigh.astype(np.int32),
                   volumes=vol, centres=np.ascontiguousarray(centres), face_sf=sf,
                   face_delta_coeffs=1.0 / delta, structured=(nx, ny, nz))


def slab(h_mm: float, lx_mm: float = 20.0, ly_mm: float = 7.0, lz_mm: float = 3.0) -> LduMesh:
    """The cuboid of the benchmark configurations (20 x 7 x 3 mm) at spacing h."""
    nx, ny, nz = (int(round(l / h_mm)) for l in (lx_mm, ly_mm, lz_mm))
    return box_mesh(nx, ny, nz, lx_mm * 1e-3, ly_mm * 1e-3, lz_mm * 1e-3)
