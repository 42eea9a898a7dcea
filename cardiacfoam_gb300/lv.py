"""Synthetic left ventricle: a truncated prolate-ellipsoid shell meshed with
tetrahedra, with a rule-based fibre field, per-cell conductivity tensors and
TNNP cell types by transmural depth.

Geometry.  Endocardium x^2/a0^2 + y^2/a0^2 + z^2/c0^2 = 1 (a0 = 25 mm,
c0 = 60 mm), epicardium with both semi-axes 10 mm larger, cut at the base
z = 0 (apex at negative z).  A point is (s, S, phi): transmural fraction s
(0 endo, 1 epi) with semi-axes a(s) = a0 + s*w, c(s) = c0 + s*w; arc length S
from the apex along the mid-wall meridian, which fixes the polar angle theta;
and azimuth phi.  x = a(s) sin(theta) cos(phi), y = a(s) sin(theta) sin(phi),
z = -c(s) cos(theta).

Grid.  Around the apex a square m x m patch mapped onto a disk of arc radius
S_cap (an O-grid cap, so no cell degenerates at the pole); from S_cap to the
base, rings of 4m circumferential nodes that continue the patch's perimeter;
nt layers through the wall.  Each hexahedron is split into six tetrahedra by
the pulling rule (cone from its lowest-numbered vertex over the faces that do
not contain it, each quad split through its own lowest-numbered vertex), so
the splits of neighbouring hexahedra meet face to face.

Fibres.  As setFibreField (applications/utilities/setFibreField/
setFibreField.C:60-130): e_t is the transmural direction, e_n the base
direction k = (0,0,1) with its e_t part removed, e_l = e_n x e_t, and the
fibre is e_l rotated about e_t by alpha = alpha_endo (1-s) + alpha_epi s with
alpha_endo = +60 deg and alpha_epi = -60 deg: f = cos(alpha) e_l +
sin(alpha) e_n.  Here e_t is the normal of the ellipsoid s = const through
the cell (the gradient of the transmural coordinate) instead of the gradient
of a Laplace solution.  The conductivity is sigma_t I + (sigma_l - sigma_t) f f.

Cell types.  TNNP flags by the cell's transmural fraction: endocardial
(3) below 0.3, M cells (2) below 0.6, epicardial (1) above.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Tuple

import numpy as np

from .mesh import LduMesh, tet_mesh, tet_volumes6

ENDO_A, ENDO_C, WALL = 25e-3, 60e-3, 10e-3      # m
ALPHA_ENDO, ALPHA_EPI = np.deg2rad(60.0), np.deg2rad(-60.0)
SIGMA_L, SIGMA_T = 0.1334, 0.0176                # S/m


@dataclass
class LeftVentricle:
    mesh: LduMesh
    points: np.ndarray          # [np, 3]
    tets: np.ndarray            # [n, 4]
    transmural: np.ndarray      # [n] s of each cell (mean of its vertices)
    fibre: np.ndarray           # [n, 3] unit fibre direction
    conductivity: np.ndarray    # [n, 6] xx xy xz yy yz zz
    tissue: np.ndarray          # uint8 [n] TNNP tissue flags
    dims: Tuple[int, int, int]  # (nt, m, nr)

    def apex_box(self, size: float = 2e-3):
        """Axis-aligned cube of side `size` at the epicardial apex (its
        lower face on the apex point)."""
        z0 = -(ENDO_C + WALL)
        h = 0.5 * size
        return (-h, -h, z0), (h, h, z0 + size)

    def ecg_electrodes(self) -> np.ndarray:
        """Five pseudo-ECG electrodes around the shell [m]: below the apex,
        above the base, and three to the sides at 1.5 to 2 outer radii."""
        a, c = ENDO_A + WALL, ENDO_C + WALL
        return np.array([[0.0, 0.0, -1.5 * c], [0.0, 0.0, 0.6 * c], [2.0 * a, 0.0, -0.4 * c],
                         [0.0, -1.8 * a, -0.5 * c], [1.2 * a, 1.2 * a, -0.2 * c]])


def _meridian(n: int = 200001):
    """Polar angle as a function of arc length on the mid-wall meridian."""
    a, c = ENDO_A + 0.5 * WALL, ENDO_C + 0.5 * WALL
    th = np.linspace(0.0, 0.5 * np.pi, n)
    ds = np.sqrt((a * np.cos(th)) ** 2 + (c * np.sin(th)) ** 2)
    S = np.concatenate([[0.0], np.cumsum(0.5 * (ds[1:] + ds[:-1]) * np.diff(th))])
    return th, S


def _point(s, theta, phi):
    s, theta, phi = np.broadcast_arrays(s, theta, phi)
    a = ENDO_A + s * WALL
    c = ENDO_C + s * WALL
    st = np.sin(theta)
    return np.stack([a * st * np.cos(phi), a * st * np.sin(phi), -c * np.cos(theta)], axis=-1)


# quad faces of a hexahedron whose corner (d0, d1, d2) has local index
# d0 + 2 d1 + 4 d2: _HEX_FACES[axis][side] in cyclic order
_HEX_FACES = np.array([
    [[0, 2, 6, 4], [1, 3, 7, 5]],
    [[0, 1, 5, 4], [2, 3, 7, 6]],
    [[0, 1, 3, 2], [4, 5, 7, 6]],
])


def split_hexes(g: np.ndarray) -> np.ndarray:
    """Pulling triangulation of hexahedra given by global vertex ids [nh, 8]
    (local corner d0 + 2 d1 + 4 d2): six tetrahedra per hexahedron."""
    nh = g.shape[0]
    rows = np.arange(nh)
    lo = np.argmin(g, axis=1)
    v0 = g[rows, lo]
    out = np.empty((nh, 6, 4), dtype=np.int64)
    for axis in range(3):
        side = 1 - ((lo >> axis) & 1)
        q = g[rows[:, None], _HEX_FACES[axis][side]]            # [nh, 4]
        m = np.argmin(q, axis=1)
        qr = q[rows[:, None], (m[:, None] + np.arange(4)) % 4]
        out[:, 2 * axis, :] = np.stack([v0, qr[:, 0], qr[:, 1], qr[:, 2]], axis=1)
        out[:, 2 * axis + 1, :] = np.stack([v0, qr[:, 0], qr[:, 2], qr[:, 3]], axis=1)
    return out.reshape(-1, 4)


def left_ventricle(nt: int, m: int, nr: int, cap_fraction: float = 0.3,
                   roundness: float = 0.5, sigma_l: float = SIGMA_L,
                   sigma_t: float = SIGMA_T) -> LeftVentricle:
    """LV shell with nt transmural layers, an m x m apical cap and nr rings
    of 4m cells from the cap to the base: 6 nt (m^2 + 4 m nr) tetrahedra.
    `cap_fraction` is the arc length from the apex to the middle of the
    cap's sides as a share of the apex-to-base arc; `roundness` blends the
    cap's outline from a square (0) to a circle (1)."""
    th_tab, S_tab = _meridian()
    S_tot = S_tab[-1]
    S_cap = cap_fraction * S_tot
    n_i = nt + 1
    s_lvl = np.arange(n_i) / nt
    # cap nodes: the square (p, q) mapped onto a rounded square of the
    # apex's geodesic polar plane (arc length S, azimuth phi): a blend of
    # the identity and the square-to-disk map, so the cap's corners keep
    # angles well below 180 degrees
    u = -1.0 + 2.0 * np.arange(m + 1) / m
    U, V = np.meshgrid(u, u, indexing="xy")                    # [q, p]
    X = (1.0 - roundness) * U + roundness * U * np.sqrt(1.0 - 0.5 * V * V)
    Y = (1.0 - roundness) * V + roundness * V * np.sqrt(1.0 - 0.5 * U * U)
    S_node = S_cap * np.sqrt(X * X + Y * Y)
    psi = np.arctan2(Y, X)
    th_cap = np.interp(S_node, S_tab, th_tab)
    cap_pts = _point(s_lvl[None, None, :], th_cap[:, :, None], psi[:, :, None])  # [q, p, i, 3]
    n_cap = (m + 1) * (m + 1) * n_i

    def cap_id(p, q, i):
        return (q * (m + 1) + p) * n_i + i

    # perimeter of the square, counter-clockwise from (p, q) = (m, 0); each
    # perimeter node starts a meridian line of ring nodes whose arc length
    # grows linearly to the base
    per_p = np.concatenate([np.full(m, m), np.arange(m, 0, -1), np.zeros(m, int), np.arange(0, m)])
    per_q = np.concatenate([np.arange(0, m), np.full(m, m), np.arange(m, 0, -1), np.zeros(m, int)])
    nc = 4 * m
    phi = psi[per_q, per_p]
    S0 = S_node[per_q, per_p]
    frac = np.arange(1, nr + 1) / nr
    S_ring = S0[None, :] + (S_tot - S0[None, :]) * frac[:, None]          # [k, j]
    th_ring = np.interp(S_ring, S_tab, th_tab)
    th_ring[-1, :] = 0.5 * np.pi                               # the base plane z = 0
    ring_pts = _point(s_lvl[None, None, :], th_ring[:, :, None], phi[None, :, None])  # [k, j, i, 3]
    points = np.concatenate([cap_pts.reshape(-1, 3), ring_pts.reshape(-1, 3)])

    def node(j, k, i):
        """Ring node j at ring level k (0 = the cap's perimeter)."""
        j = j % nc
        return np.where(k == 0, cap_id(per_p[j], per_q[j], i),
                        n_cap + ((np.maximum(k, 1) - 1) * nc + j) * n_i + i)

    d0 = np.array([0, 1, 0, 1, 0, 1, 0, 1])
    d1 = np.array([0, 0, 1, 1, 0, 0, 1, 1])
    d2 = np.array([0, 0, 0, 0, 1, 1, 1, 1])
    Q, P, I = np.meshgrid(np.arange(m), np.arange(m), np.arange(nt), indexing="ij")
    Q, P, I = Q.ravel(), P.ravel(), I.ravel()
    g_cap = cap_id(P[:, None] + d1, Q[:, None] + d2, I[:, None] + d0)
    K, J, I = np.meshgrid(np.arange(nr), np.arange(nc), np.arange(nt), indexing="ij")
    K, J, I = K.ravel(), J.ravel(), I.ravel()
    g_ring = node(J[:, None] + d1, K[:, None] + d2, I[:, None] + d0)
    tets = split_hexes(np.concatenate([g_cap, g_ring]))
    neg = tet_volumes6(points, tets) < 0
    tets[neg] = tets[neg][:, [0, 2, 1, 3]]
    mesh = tet_mesh(points, tets)
    # cell fields
    s_node = (np.arange(points.shape[0]) % n_i) / nt
    s = s_node[tets].mean(axis=1)
    x = mesh.centres
    a = ENDO_A + s * WALL
    c = ENDO_C + s * WALL
    et = np.stack([x[:, 0] / a ** 2, x[:, 1] / a ** 2, x[:, 2] / c ** 2], axis=1)
    et /= np.linalg.norm(et, axis=1)[:, None]
    k = np.array([0.0, 0.0, 1.0])
    en = k[None, :] - et[:, 2:3] * et
    nn = np.linalg.norm(en, axis=1)
    pole = nn < 1e-12
    if np.any(pole):                                           # e_t along the axis
        alt = np.array([1.0, 0.0, 0.0])
        en[pole] = alt - (et[pole] @ alt)[:, None] * et[pole]
        nn[pole] = np.linalg.norm(en[pole], axis=1)
    en /= nn[:, None]
    el = np.cross(en, et)
    el /= np.linalg.norm(el, axis=1)[:, None]
    alpha = ALPHA_ENDO * (1.0 - s) + ALPHA_EPI * s
    f = np.cos(alpha)[:, None] * el + np.sin(alpha)[:, None] * en
    dsig = sigma_l - sigma_t
    sig = np.stack([sigma_t + dsig * f[:, 0] * f[:, 0], dsig * f[:, 0] * f[:, 1],
                    dsig * f[:, 0] * f[:, 2], sigma_t + dsig * f[:, 1] * f[:, 1],
                    dsig * f[:, 1] * f[:, 2], sigma_t + dsig * f[:, 2] * f[:, 2]], axis=1)
    tissue = np.where(s < 0.3, 3, np.where(s < 0.6, 2, 1)).astype(np.uint8)
    return LeftVentricle(mesh=mesh, points=points, tets=tets, transmural=s, fibre=f,
                         conductivity=np.ascontiguousarray(sig), tissue=tissue, dims=(nt, m, nr))


def config_sizes(target_cells: float = 4.0e6, nt: int = 16):
    """(nt, m, nr) of an LV of about `target_cells` tetrahedra with cells of
    similar size around the wall and along the meridian."""
    th, S = _meridian(20001)
    S_tot = S[-1]
    best = None
    for m in range(8, 400, 2):
        h = 2.0 * np.pi * (ENDO_A + 0.5 * WALL) / (4 * m)      # equatorial spacing
        nr = max(1, int(round(0.7 * S_tot / h)))
        n = 6 * nt * (m * m + 4 * m * nr)
        if best is None or abs(n - target_cells) < abs(best[3] - target_cells):
            best = (nt, m, nr, n)
    return best[:3]
