"""Meshes for the monodomain step, in OpenFOAM's lduMesh form.

``box_mesh`` builds what blockMesh makes of one hex block with uniform
spacing: cells numbered x fastest, internal faces in upper-triangular order
(per owner: +x, +y, +z neighbour), face area vectors pointing from owner to
neighbour, and deltaCoeffs = 1/|d_PN|.  The arithmetic (point coordinates
l*i/n, centres as the mean of the two bounding points) is the same sequence
of IEEE operations the CPU oracle uses, so both see identical geometry.

``tet_mesh`` turns points and tetrahedra into the same form with the full
geometry the corrected Laplacian needs on a non-orthogonal mesh: face
centres, and the boundary faces (owner cell, outward area vector, centre).
Face and cell geometry follow OpenFOAM's primitiveMesh
(primitiveMeshFaceCentresAndAreas: triangle centre = vertex mean, area =
half the cross product; primitiveMeshCellCentresAndVols: face pyramids about
the mean of the face centres).
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
    # full geometry (general meshes): face centres and boundary faces
    face_centres: Optional[np.ndarray] = None     # [nf, 3]
    boundary_cell: Optional[np.ndarray] = None    # int32 [nb]
    boundary_sf: Optional[np.ndarray] = None      # [nb, 3] outward
    boundary_centres: Optional[np.ndarray] = None  # [nb, 3]

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def has_geometry(self) -> bool:
        return self.face_centres is not None

    @property
    def n_boundary_faces(self) -> int:
        return 0 if self.boundary_cell is None else int(self.boundary_cell.shape[0])

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


def with_box_geometry(m: LduMesh, lx: float, ly: float, lz: float) -> LduMesh:
    """The box mesh with its full geometry (face centres, boundary faces), so
    that it can run through the general-mesh path of the Laplacian."""
    nx, ny, nz = m.structured
    c = m.centres
    d = np.argmax(np.abs(m.face_sf), axis=1)
    fc = 0.5 * (c[m.owner] + c[m.neighbour])
    # the face lies on the grid plane between the two centres
    for k, (l, nk) in enumerate(((lx, nx), (ly, ny), (lz, nz))):
        sel = d == k
        i_hi = np.rint((c[m.neighbour[sel], k] / l) * nk - 0.5).astype(np.int64)
        fc[sel, k] = l * i_hi / nk
    cid = np.arange(m.n_cells).reshape(nz, ny, nx)
    ax, ay, az = (ly / ny) * (lz / nz), (lx / nx) * (lz / nz), (lx / nx) * (ly / ny)
    cells, sfs, cfs = [], [], []
    for k, (sl_lo, sl_hi, area, l, nk) in enumerate((
            ((slice(None), slice(None), 0), (slice(None), slice(None), -1), ax, lx, nx),
            ((slice(None), 0, slice(None)), (slice(None), -1, slice(None)), ay, ly, ny),
            ((0, slice(None), slice(None)), (-1, slice(None), slice(None)), az, lz, nz))):
        for sl, sign, pos in ((sl_lo, -1.0, 0.0), (sl_hi, 1.0, l)):
            cc = cid[sl].ravel()
            sf = np.zeros((cc.size, 3))
            sf[:, k] = sign * area
            cf = c[cc].copy()
            cf[:, k] = pos
            cells.append(cc)
            sfs.append(sf)
            cfs.append(cf)
    bc = np.concatenate(cells)
    order = np.argsort(bc, kind="stable")
    return LduMesh(n_cells=m.n_cells, owner=m.owner, neighbour=m.neighbour, volumes=m.volumes,
                   centres=m.centres, face_sf=m.face_sf, face_delta_coeffs=m.face_delta_coeffs,
                   structured=(0, 0, 0), face_centres=np.ascontiguousarray(fc),
                   boundary_cell=bc[order].astype(np.int32),
                   boundary_sf=np.ascontiguousarray(np.concatenate(sfs)[order]),
                   boundary_centres=np.ascontiguousarray(np.concatenate(cfs)[order]))


# outward faces of a positively oriented tetrahedron (v0 v1 v2 v3), each
# opposite one vertex, ordered so the right-hand normal points out
_TET_FACES = np.array([[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]])


def tet_volumes6(points: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Six times the signed volume of each tetrahedron."""
    p = points[tets]
    return np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))


def tet_mesh(points: np.ndarray, tets: np.ndarray) -> LduMesh:
    """lduMesh of a tetrahedral mesh: cells in the given order, internal faces
    owner < neighbour in upper-triangular order with the area vector from
    owner to neighbour, boundary faces sorted by cell with outward areas."""
    points = np.ascontiguousarray(points, dtype=np.float64)
    tets = np.array(tets, dtype=np.int64)
    neg = tet_volumes6(points, tets) < 0
    tets[neg] = tets[neg][:, [0, 2, 1, 3]]
    n = tets.shape[0]
    tri = tets[:, _TET_FACES].reshape(-1, 3)          # outward, per cell
    cell = np.repeat(np.arange(n, dtype=np.int64), 4)
    key = np.sort(tri, axis=1)
    order = np.lexsort((cell, key[:, 2], key[:, 1], key[:, 0]))
    ks = key[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    if np.any(same[1:] & same[:-1]):
        raise ValueError("a face is shared by more than two cells")
    first = np.flatnonzero(same)                      # pair (first, first+1)
    paired = np.zeros(order.size, bool)
    paired[first] = paired[first + 1] = True
    a, b = order[first], order[first + 1]             # a: lower cell (lexsort by cell)
    own, nei = cell[a], cell[b]
    if np.any(own == nei):
        raise ValueError("a cell meets itself")
    fpts = tri[a]                                     # outward of the owner
    srt = np.lexsort((nei, own))
    own, nei, fpts = own[srt], nei[srt], fpts[srt]
    bidx = order[~paired]
    bidx = bidx[np.argsort(cell[bidx], kind="stable")]
    bcell, bpts = cell[bidx], tri[bidx]

    def tri_geom(f):
        p0, p1, p2 = points[f[:, 0]], points[f[:, 1]], points[f[:, 2]]
        return (1.0 / 3.0) * (p0 + p1 + p2), 0.5 * np.cross(p1 - p0, p2 - p0)

    fc, sf = tri_geom(fpts)
    bfc, bsf = tri_geom(bpts)
    # primitiveMeshCellCentresAndVols over the four faces of each cell
    cfc, csf = tri_geom(tri)
    cfc = cfc.reshape(n, 4, 3)
    csf = csf.reshape(n, 4, 3)
    c_est = cfc.sum(axis=1) / 4.0
    pyr3 = np.einsum("ijk,ijk->ij", csf, cfc - c_est[:, None, :])
    pc = 0.75 * cfc + 0.25 * c_est[:, None, :]
    vol3 = pyr3.sum(axis=1)
    centres = (pyr3[:, :, None] * pc).sum(axis=1) / vol3[:, None]
    d = centres[nei] - centres[own]
    return LduMesh(n_cells=n, owner=own.astype(np.int32), neighbour=nei.astype(np.int32),
                   volumes=vol3 * (1.0 / 3.0), centres=np.ascontiguousarray(centres),
                   face_sf=np.ascontiguousarray(sf),
                   face_delta_coeffs=1.0 / np.sqrt(np.einsum("ij,ij->i", d, d)),
                   face_centres=np.ascontiguousarray(fc), boundary_cell=bcell.astype(np.int32),
                   boundary_sf=np.ascontiguousarray(bsf), boundary_centres=np.ascontiguousarray(bfc))
