"""Manufactured-solution verification of the monodomain step (the GPU
counterpart of the reference's ``manufacturedFDAMonodomainVerifier``).

The monodomainFDAManufactured ionic model and the exact solution

    V  = sqrt(1 + t) F(x),   F = cos(pi x) [cos(2 pi y) [cos(3 pi z)]]
    u1 = (1 + t) G(x) + sqrt(1 + t) F(x),  G = 1 + x [y^2 [z^3]]
    u2 = G(x)^(-1/2) / (1 + t),  u3 = 0

(src/verificationModels/monodomainVerification/manufacturedFDAReference.H:33-167)
solve chi Cm dV/dt = div(sigma grad V) - chi Cm Im with zero-gradient walls
on the unit cube (1D: 1 x 0.1 x 0.1, 2D: 1 x 1 x 0.1), chi = 3, Cm = 2 and
the tutorial's anisotropic conductivity
(tutorials/manufacturedSolutions/monodomainPseudoECG/constant/electroProperties).
Errors are the verifier's L1 (mean), L2 (RMS) and L-infinity norms over the
cells (manufacturedFDAMonodomainVerifier.C:139-169); the convergence rate
between two meshes is log(e1/e2)/log(h1/h2) with h = 1/N
(setupManufacturedFDA/post_processing_manufactured.py:119-124), the time step
shrinking with h^2 as in the tutorial's sweep (10/20/40/80 cells at
dt = 8.92857e-3 / 2.24215e-3 / 5.60538e-4 / 1.40174e-4 s, to t = 0.2 s).
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np

from . import api
from . import lib as _L
from .mesh import box_mesh, with_box_geometry

SIGMA = (0.111453302, 0.0, 0.0, 0.121585420, 0.0, 0.030396355)
CHI, CM = 3.0, 2.0
END_TIME = 0.2
SWEEP = {10: 0.00892857, 20: 0.00224215, 40: 0.000560538, 80: 0.000140174}


def manufactured_fields(centres: np.ndarray, t: float, dim: int):
    """Exact V, u1, u2, u3 at the cell centres (computeF/G/V/U,
    manufacturedFDAReference.H:33-135)."""
    x, y, z = centres[:, 0], centres[:, 1], centres[:, 2]
    pi = math.pi
    if dim == 1:
        F, G = np.cos(pi * x), 1.0 + x
    elif dim == 2:
        F, G = np.cos(pi * x) * np.cos(2.0 * pi * y), 1.0 + x * y ** 2
    else:
        F = np.cos(pi * x) * np.cos(2.0 * pi * y) * np.cos(3.0 * pi * z)
        G = 1.0 + x * y ** 2 * z ** 3
    s = math.sqrt(1.0 + t)
    V = s * F
    u1 = (1.0 + t) * G + s * F
    u2 = (1.0 / (1.0 + t)) * G ** -0.5
    return V, u1, u2, np.zeros_like(V)


def norms(num: np.ndarray, exact: np.ndarray) -> Tuple[float, float, float]:
    """(L1 mean, L2 RMS, L-infinity) of num - exact."""
    d = np.abs(num - exact)
    return float(d.sum() / d.size), float(math.sqrt((d * d).sum() / d.size)), float(d.max())


def rate(e1: float, e2: float, n1: int, n2: int) -> float:
    """Observed order between meshes of n1 and n2 cells per direction."""
    return math.log(e1 / e2) / math.log((1.0 / n1) / (1.0 / n2))


def mesh_for(dim: int, n: int):
    """The tutorial's blockMesh: n cells per resolved direction, 0.1 thick
    (one cell) in the others."""
    nx, ny, nz = n, (n if dim >= 2 else 1), (n if dim == 3 else 1)
    return box_mesh(nx, ny, nz, 1.0, 1.0 if dim >= 2 else 0.1, 1.0 if dim == 3 else 0.1)


# the tutorial's electrodes (monodomainPseudoECG/constant/electroProperties)
ECG_ELECTRODES = (("E1", (-0.5, 0.5, 0.5)), ("E2", (1.5, 0.5, 0.5)), ("E3", (1.2, 0.23, 0.61)),
                  ("E4", (1.35, 0.74, 0.28)), ("E5", (1.55, 0.41, 0.83)))


def gauss_legendre(order: int):
    """Nodes and weights of the order-point Gauss-Legendre rule on [-1, 1]
    (pseudoECGManufacturedQuadratureRule, manufacturedFDAReference.H:220-292,
    finds the same roots of P_order by Newton's method)."""
    if order <= 0:
        raise ValueError("quadrature order must be positive")
    return np.polynomial.legendre.leggauss(order)


def pseudo_ecg_spatial_reference(electrodes, dim: int, order: int = 96,
                                 sigma=SIGMA) -> np.ndarray:
    """Integral over the unit line/square/cube of (sigma grad F) . r / |r|^3,
    r = x - P (the in-plane distance in 1D/2D), by the tensor Gauss-Legendre
    rule mapped to [0, 1] (computeManufacturedPseudoECGSpatialReference,
    manufacturedFDAReference.H:393-472); points with |r|^2 <= VSMALL add 0."""
    nodes, weights = gauss_legendre(order)
    x = 0.5 * (nodes + 1.0)
    pi = math.pi
    s = np.array([[sigma[0], sigma[1], sigma[2]], [sigma[1], sigma[3], sigma[4]],
                  [sigma[2], sigma[4], sigma[5]]])
    out = []
    for P in np.asarray(electrodes, dtype=np.float64).reshape(-1, 3):
        if dim == 1:
            X = x
            g = np.stack([-pi * np.sin(pi * X), 0 * X, 0 * X])
            W = weights
            r = np.stack([X - P[0], 0 * X, 0 * X])
        elif dim == 2:
            X, Y = np.meshgrid(x, x, indexing="ij")
            g = np.stack([-pi * np.sin(pi * X) * np.cos(2 * pi * Y),
                          -2 * pi * np.cos(pi * X) * np.sin(2 * pi * Y), 0 * X])
            W = np.multiply.outer(weights, weights)
            r = np.stack([X - P[0], Y - P[1], 0 * X])
        else:
            X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
            cx, cy, cz = np.cos(pi * X), np.cos(2 * pi * Y), np.cos(3 * pi * Z)
            g = np.stack([-pi * np.sin(pi * X) * cy * cz,
                          -2 * pi * cx * np.sin(2 * pi * Y) * cz,
                          -3 * pi * cx * cy * np.sin(3 * pi * Z)])
            W = np.multiply.outer(np.multiply.outer(weights, weights), weights)
            r = np.stack([X - P[0], Y - P[1], Z - P[2]])
        sg = np.einsum("ij,j...->i...", s, g)
        r2 = (r * r).sum(axis=0)
        f = np.where(r2 > 1e-300, (sg * r).sum(axis=0) / np.where(r2 > 1e-300, r2, 1.0) ** 1.5,
                     0.0)
        out.append(0.5 ** dim * float((W * f).sum()))
    return np.array(out)


def pseudo_ecg_reference(t: float, electrodes, dim: int, order: int = 96) -> np.ndarray:
    """sqrt(1 + t) times the spatial reference (computeManufacturedPseudoECGReference,
    manufacturedFDAReference.H:495-512)."""
    return math.sqrt(1.0 + t) * pseudo_ecg_spatial_reference(electrodes, dim, order)


def geometry_mesh_for(dim: int, n: int):
    """mesh_for with the face centres and walls the pseudo-ECG gradient needs."""
    return with_box_geometry(mesh_for(dim, n), 1.0, 1.0 if dim >= 2 else 0.1,
                             1.0 if dim == 3 else 0.1)


def run(dim: int, n: int, dt: float | None = None, end_time: float = END_TIME,
        precision: int = _L.PRECISION_FP64, pcg_tol: float = 1e-12, ecg: bool = False,
        ecg_order: int = 96) -> Dict:
    """One manufactured case on the GPU: implicit backward ddt, two PIMPLE
    correctors (the tutorial's fvSolution), PCG to `pcg_tol`.  Returns the
    error norms of V, u1 and u2 at the end time; with ``ecg`` also the
    pseudo-ECG at the tutorial's electrodes after every step (Gauss linear
    gradient, the tutorial's gradSchemes) against the quadrature reference,
    as pseudoECGManufacturedVerifier::updateStatistics accumulates them
    (pseudoECGManufacturedVerifier.C:257-300): per electrode the L1 (mean),
    L2 (RMS) and L-infinity of the error over the samples."""
    dt = SWEEP[n] if dt is None else dt
    mesh = mesh_for(dim, n)
    md = api.Monodomain(mesh, model="monodomainFDAManufactured", tissue=f"{dim}D", sigma=SIGMA,
                        chi=CHI, cm=CM, dt=dt, precision=precision, implicit=True,
                        ddt_backward=True, pcg_tol=pcg_tol, pcg_rel_tol=0.0,
                        pcg_max_iter=2000, n_outer=2, outer_tol=0.0)
    V, u1, u2, u3 = manufactured_fields(mesh.centres, 0.0, dim)
    md.set_field(_L.FIELD_VM, V)
    md.set_states(np.stack([V, u1, u2, u3]))
    steps = int(round(end_time / dt))
    pe = None
    if ecg:
        pe = api.PseudoECG(geometry_mesh_for(dim, n), [p for _, p in ECG_ELECTRODES],
                           names=[k for k, _ in ECG_ELECTRODES], sigma=SIGMA,
                           grad_scheme=_L.GRAD_GAUSS_LINEAR, max_rows=steps)
        for _ in range(steps):
            md.step(dt)
            pe.record(md)
    else:
        md.run(dt, steps)
    t = md.time()
    Ve, u1e, u2e, _ = manufactured_fields(mesh.centres, t, dim)
    st = md.states()
    out = {"dim": dim, "n": n, "dt": dt, "steps": steps, "t": t,
           "V": norms(md.vm(), Ve), "u1": norms(st[1], u1e), "u2": norms(st[2], u2e)}
    if pe is not None:
        times, values = pe.series()
        spatial = pseudo_ecg_spatial_reference([p for _, p in ECG_ELECTRODES], dim, ecg_order)
        ref = np.sqrt(1.0 + times)[:, None] * spatial[None, :]
        err = np.abs(values - ref)
        out["ecg"] = {"times": times, "values": values, "reference": ref,
                      "L1": err.mean(axis=0), "L2": np.sqrt((err * err).mean(axis=0)),
                      "Linf": err.max(axis=0)}
        pe.close()
    md.close()
    return out


# --------------------------------------------------------------------- bidomain
# tutorials/manufacturedSolutions/bidomain/constant/electroProperties
BIDOMAIN_SIGMA_I = SIGMA
BIDOMAIN_SIGMA_E = (0.046165469, 0.0, 0.0, 0.050362330, 0.0, 0.012590582)
BIDOMAIN_K = 0.7071067811865476
BIDOMAIN_REF_POINT = (0.125, 0.05, 0.05)


def bidomain_shift(t: float, dim: int, k: float = BIDOMAIN_K, ref_point=BIDOMAIN_REF_POINT,
                   ref_value: float = 0.0) -> float:
    """manufacturedFDABidomainShift (manufacturedFDABidomainReference.H:28-45):
    phiE's constant, so that the exact phiE equals ref_value at ref_point."""
    F = manufactured_fields(np.array([ref_point], dtype=np.float64), 0.0, dim)[0][0]
    return ref_value + k * math.sqrt(1.0 + t) * F


def bidomain_fields(centres: np.ndarray, t: float, dim: int, k: float = BIDOMAIN_K,
                    ref_point=BIDOMAIN_REF_POINT, ref_value: float = 0.0):
    """Exact V, phiE = -k sqrt(1 + t) F + shift, phiI = V + phiE, u1, u2, u3
    (computeManufacturedBidomainPhiE/PhiI, manufacturedFDABidomainReference.H:
    47-100; V and u as the monodomain case)."""
    V, u1, u2, u3 = manufactured_fields(centres, t, dim)
    F = manufactured_fields(centres, 0.0, dim)[0]
    phie = (-k * math.sqrt(1.0 + t)) * F + bidomain_shift(t, dim, k, ref_point, ref_value)
    return V, phie, V + phie, u1, u2, u3


def run_bidomain(dim: int, n: int, dt: float | None = None, end_time: float = END_TIME,
                 precision: int = _L.PRECISION_FP64, pcg_tol: float = 1e-12,
                 phie_tol: float = 1e-12, steps: int | None = None) -> Dict:
    """The bidomain tutorial's manufactured case on the GPU (bidomainSolver,
    bidomainFDAManufactured, Gi and Ge of the tutorial, phiERefPoint
    (0.125 0.05 0.05), backward ddt, two PIMPLE correctors, Gauss linear
    gradients): norms of V, phiE, phiI, u1 and u2 at the end, as
    manufacturedFDABidomainVerifier computes them.  The tutorial's PCG
    tolerance is 1e-15 for both fields; at 1e-12 the solves converge instead
    of running to maxIter, and the discretisation error is orders of
    magnitude larger."""
    dt = SWEEP[n] if dt is None else dt
    mesh = geometry_mesh_for(dim, n)
    bd = api.Bidomain(mesh, model="bidomainFDAManufactured", tissue=f"{dim}D",
                      sigma_i=BIDOMAIN_SIGMA_I, sigma_e=BIDOMAIN_SIGMA_E, chi=CHI, cm=CM, dt=dt,
                      precision=precision, ddt_backward=True, pcg_tol=pcg_tol, pcg_rel_tol=0.0,
                      pcg_max_iter=2000, phie_tol=phie_tol, phie_rel_tol=0.0,
                      phie_max_iter=4000, n_outer=2, outer_tol=0.0,
                      ref_point=BIDOMAIN_REF_POINT, grad_scheme=_L.GRAD_GAUSS_LINEAR)
    V, phie, _, u1, u2, u3 = bidomain_fields(mesh.centres, 0.0, dim)
    bd.set_field(_L.FIELD_VM, V)
    bd.set_field(_L.FIELD_PHIE, phie)
    bd.set_states(np.stack([V, u1, u2, u3]))
    steps = int(round(end_time / dt)) if steps is None else steps
    bd.run(dt, steps)
    t = bd.time()
    Ve, pe, pie, u1e, u2e, _ = bidomain_fields(mesh.centres, t, dim)
    st = bd.states()
    out = {"dim": dim, "n": n, "dt": dt, "steps": steps, "t": t,
           "V": norms(bd.vm(), Ve), "phiE": norms(bd.phie(), pe), "phiI": norms(bd.phii(), pie),
           "u1": norms(st[1], u1e), "u2": norms(st[2], u2e)}
    bd.close()
    return out
