"""ctypes view of the C oracle (test infrastructure only).

Mirrors oracle.h.  Models are addressed by the reference's class names
(``TNNP``, ``ORd``, ``ToRORd_dynCl``, ``AlievPanfilov``, ``BuenoOrovio``) and
tissues by the flags of ``ionicSelector::tissueFlag``
(src/ionicModels/ionicModel/ionicSelector.C:56-63).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import build as _build

MODELS = {"TNNP": 0, "ORd": 1, "ToRORd_dynCl": 2, "AlievPanfilov": 3, "BuenoOrovio": 4,
          "monodomainFDAManufactured": 5, "bidomainFDAManufactured": 6}
TISSUES = {"epicardialCells": 1, "mCells": 2, "endocardialCells": 3, "myocyte": 4,
           "1D": 11, "2D": 12, "3D": 13}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Stimulus(C.Structure):
    _fields_ = [("start", C.c_double), ("period_s1", C.c_double), ("duration", C.c_double),
                ("amplitude", C.c_double), ("n1", C.c_int), ("period_s2", C.c_double),
                ("n2", C.c_int)]


class OdeSettings(C.Structure):
    _fields_ = [("abs_tol", C.c_double), ("rel_tol", C.c_double), ("max_steps", C.c_long),
                ("safe_scale", C.c_double), ("min_scale", C.c_double),
                ("max_scale", C.c_double), ("alpha_inc", C.c_double),
                ("alpha_dec", C.c_double)]


class TissueDesc(C.Structure):
    _fields_ = [("model", C.c_int), ("tissue", C.c_int), ("sigma", C.c_double * 6),
                ("chi", C.c_double), ("cm", C.c_double), ("implicit", C.c_int),
                ("ddt_backward", C.c_int), ("precond_dic", C.c_int),
                ("pcg_tol", C.c_double), ("pcg_rel_tol", C.c_double),
                ("pcg_max_iter", C.c_int), ("n_outer", C.c_int), ("outer_tol", C.c_double),
                ("vm0", C.c_double), ("n_boxes", C.c_int),
                ("box_min", (C.c_double * 3) * 8), ("box_max", (C.c_double * 3) * 8),
                ("box_start", C.c_double * 8), ("box_duration", C.c_double * 8),
                ("box_intensity", C.c_double * 8), ("ode", OdeSettings),
                ("grad_gauss", C.c_int), ("uncorrected", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.oracle_model_sizes.argtypes = [C.c_int, _ip, _ip, _ip]
        L.oracle_model_init.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.oracle_model_supplement.argtypes = [C.c_int, _dp]
        L.oracle_model_rates.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp, _dp, C.c_int,
                                         C.c_int, C.POINTER(Stimulus)]
        L.oracle_model_variables.argtypes = L.oracle_model_rates.argtypes
        L.oracle_model_iion_index.argtypes = [C.c_int]
        L.oracle_ode_default.argtypes = [C.POINTER(OdeSettings)]
        L.oracle_ionic_new.argtypes = [C.c_int, C.c_long, C.c_int, C.c_double, C.c_int,
                                       C.POINTER(OdeSettings), C.POINTER(Stimulus), _dp]
        L.oracle_ionic_new.restype = C.c_void_p
        L.oracle_ionic_free.argtypes = [C.c_void_p]
        L.oracle_ionic_solve.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, _dp, C.c_int]
        L.oracle_ionic_solve.restype = C.c_long
        L.oracle_ionic_states.argtypes = [C.c_void_p]
        L.oracle_ionic_states.restype = _dp
        L.oracle_ionic_steps.argtypes = [C.c_void_p]
        L.oracle_ionic_steps.restype = _dp
        L.oracle_ionic_rhs_evals.argtypes = [C.c_void_p]
        L.oracle_ionic_rhs_evals.restype = C.c_long
        L.oracle_mesh_box.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                      C.c_double]
        L.oracle_mesh_box.restype = C.c_void_p
        L.oracle_mesh_free.argtypes = [C.c_void_p]
        L.oracle_mesh_ncells.argtypes = [C.c_void_p]
        L.oracle_mesh_ncells.restype = C.c_long
        L.oracle_mesh_nfaces.argtypes = [C.c_void_p]
        L.oracle_mesh_nfaces.restype = C.c_long
        L.oracle_mesh_addressing.argtypes = [C.c_void_p, _ip, _ip]
        L.oracle_mesh_centres.argtypes = [C.c_void_p, _dp]
        L.oracle_mesh_general.argtypes = [C.c_long, C.c_long, _ip, _ip, _dp, _dp, _dp, _dp,
                                          C.c_long, _ip, _dp, _dp]
        L.oracle_mesh_general.restype = C.c_void_p
        L.oracle_blockmesh_centres.argtypes = [C.c_int, C.c_int, C.c_int, _dp, C.c_double, _ip,
                                               C.c_int, _dp]
        L.oracle_tissue_set_conductivity.argtypes = [C.c_void_p, _dp]
        L.oracle_tissue_set_cell_tissue.argtypes = [C.c_void_p, C.POINTER(C.c_ubyte)]
        L.oracle_tissue_laplacian.argtypes = [C.c_void_p, _dp, _dp]
        L.oracle_tissue_gradient.argtypes = [C.c_void_p, _dp, _dp]
        L.oracle_tissue_pseudo_ecg.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp]
        L.oracle_bidomain_new.argtypes = [C.POINTER(TissueDesc), _dp, C.c_void_p, _dp,
                                          C.c_double, C.c_double, C.c_double, C.c_int]
        L.oracle_bidomain_new.restype = C.c_void_p
        L.oracle_bidomain_free.argtypes = [C.c_void_p]
        L.oracle_bidomain_step.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.oracle_bidomain_tissue.argtypes = [C.c_void_p]
        L.oracle_bidomain_tissue.restype = C.c_void_p
        for f in ("phie", "phii"):
            getattr(L, f"oracle_bidomain_{f}").argtypes = [C.c_void_p]
            getattr(L, f"oracle_bidomain_{f}").restype = _dp
        L.oracle_bidomain_ref_cell.argtypes = [C.c_void_p]
        L.oracle_bidomain_ref_cell.restype = C.c_long
        L.oracle_bidomain_last_solves.argtypes = [C.c_void_p, _dp, _dp, _ip, C.c_int]
        L.oracle_tissue_new.argtypes = [C.POINTER(TissueDesc), C.c_void_p]
        L.oracle_tissue_new.restype = C.c_void_p
        L.oracle_tissue_free.argtypes = [C.c_void_p]
        L.oracle_tissue_step.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.oracle_tissue_time.argtypes = [C.c_void_p]
        L.oracle_tissue_time.restype = C.c_double
        for f in ("vm", "iion", "activation", "source"):
            getattr(L, f"oracle_tissue_{f}").argtypes = [C.c_void_p]
            getattr(L, f"oracle_tissue_{f}").restype = _dp
        L.oracle_tissue_init_ionic.argtypes = [C.c_void_p, C.c_double]
        L.oracle_tissue_ionic.argtypes = [C.c_void_p]
        L.oracle_tissue_ionic.restype = C.c_void_p
        L.oracle_tissue_last_solves.argtypes = [C.c_void_p, _dp, _dp, _ip, C.c_int]
        L.oracle_single_cell.argtypes = [C.c_int, C.c_int, C.c_double, C.c_long,
                                         C.POINTER(OdeSettings), C.POINTER(Stimulus), _dp,
                                         _dp, _dp]
        L.oracle_single_cell.restype = C.c_long
        L.oracle_single_cell_traces.argtypes = [C.c_int, C.c_int, C.c_double, C.c_long,
                                                C.POINTER(OdeSettings), C.POINTER(Stimulus),
                                                _dp, _dp, C.c_int, _dp, _dp]
        L.oracle_single_cell_traces.restype = C.c_long
        L.oracle_purkinje_new.argtypes = [C.c_long, _ip, _ip, _dp, _dp, C.c_int, C.c_int,
                                          C.POINTER(OdeSettings), C.c_double, C.c_double,
                                          C.c_double, C.c_int, C.c_double, C.c_double,
                                          C.c_double, C.c_long, _ip, _dp]
        L.oracle_purkinje_new.restype = C.c_void_p
        L.oracle_purkinje_free.argtypes = [C.c_void_p]
        L.oracle_purkinje_advance.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
        L.oracle_purkinje_couple.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                             C.c_int]
        L.oracle_purkinje_coupled_step.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int]
        for f in ("vm", "iion", "terminal_current"):
            getattr(L, f"oracle_purkinje_{f}").argtypes = [C.c_void_p]
            getattr(L, f"oracle_purkinje_{f}").restype = _dp
        L.oracle_purkinje_nodes.argtypes = [C.c_void_p]
        L.oracle_purkinje_nodes.restype = C.c_long
        _lib = L
    return _lib


def ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def sizes(model: str):
    ns, na, nc = C.c_int(), C.c_int(), C.c_int()
    lib().oracle_model_sizes(MODELS[model], C.byref(ns), C.byref(na), C.byref(nc))
    return ns.value, na.value, nc.value


def model_init(model: str, tissue: int, scale: Optional[np.ndarray] = None,
               supplement: bool = False):
    """initConsts as the reference runs it; with supplement=True also the
    constants the reference leaves unset (as the ionic/tissue paths use)."""
    ns, na, nc = sizes(model)
    Cc = np.zeros(nc)
    y = np.zeros(ns)
    lib().oracle_model_init(MODELS[model], tissue, ptr(Cc), ptr(y),
                            ptr(scale) if scale is not None else None)
    if supplement:
        lib().oracle_model_supplement(MODELS[model], ptr(Cc))
    return Cc, y


def make_stimulus(start=0.0, period_s1=0.0, duration=0.0, amplitude=0.0, n1=0,
                  period_s2=0.0, n2=0) -> Stimulus:
    return Stimulus(start, period_s1, duration, amplitude, n1, period_s2, n2)


def ode_settings(**kw) -> OdeSettings:
    s = OdeSettings()
    lib().oracle_ode_default(C.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def model_rates(model, t, consts, y, tissue, solve_vm, stim: Optional[Stimulus] = None):
    ns, na, nc = sizes(model)
    dydt = np.zeros(ns)
    alg = np.zeros(na)
    lib().oracle_model_rates(MODELS[model], t, ptr(consts), ptr(y), ptr(dydt), ptr(alg),
                             tissue, int(solve_vm), C.byref(stim) if stim else None)
    return dydt, alg


def model_variables(model, t, consts, y, tissue, solve_vm, stim=None, alg=None, rates=None):
    ns, na, nc = sizes(model)
    rates = np.zeros(ns) if rates is None else rates
    alg = np.zeros(na) if alg is None else alg
    lib().oracle_model_variables(MODELS[model], t, ptr(consts), ptr(y), ptr(rates), ptr(alg),
                                 tissue, int(solve_vm), C.byref(stim) if stim else None)
    return rates, alg


class Ionic:
    """One ionicModel instance over n cells (tissue or single-cell mode)."""

    def __init__(self, model: str, n: int, tissue: int, initial_dt: float, solve_vm=False,
                 ode: Optional[OdeSettings] = None, stim: Optional[Stimulus] = None,
                 scales: Optional[np.ndarray] = None):
        self.model = model
        self.n = n
        self.ns, self.na, self.nc = sizes(model)
        self._scales = None if scales is None else np.ascontiguousarray(scales, dtype=np.float64)
        self.h = lib().oracle_ionic_new(MODELS[model], n, tissue, initial_dt, int(solve_vm),
                                        C.byref(ode) if ode else None,
                                        C.byref(stim) if stim else None,
                                        ptr(self._scales) if self._scales is not None else None)
        if not self.h:
            raise ValueError("oracle_ionic_new failed")

    def solve(self, t0, dt, vm: np.ndarray, im: np.ndarray, nthreads=1) -> int:
        k = lib().oracle_ionic_solve(self.h, t0, dt, ptr(vm), ptr(im), nthreads)
        if k < 0:
            raise RuntimeError("oracle RKF45 exceeded maxSteps")
        return k

    def states(self) -> np.ndarray:
        p = lib().oracle_ionic_states(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n, self.ns)).copy()

    def steps(self) -> np.ndarray:
        p = lib().oracle_ionic_steps(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n,)).copy()

    def rhs_evals(self) -> int:
        return lib().oracle_ionic_rhs_evals(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_ionic_free(self.h)
            self.h = None


BLOCK_FACES = ("x-min", "x-max", "y-min", "y-max", "z-min", "z-max")


def blockmesh_centres(ni, nj, nk, extent, scale, patch_order, contract=0) -> np.ndarray:
    """Cell centres [ni*nj*nk, 3] (x fastest) of one uniformly graded
    blockMesh block, rounded as OpenFOAM's geometry code rounds them.
    extent: the far block vertex before `scale` (the near one is the origin);
    patch_order: the block faces (names of BLOCK_FACES) in the order the
    boundary patch lists them; contract: which expressions are fused into fma
    (bits 1 blockMesh weights, 2 cross products, 4 dot products, 8 squared
    magnitudes), as a compiler that contracts within expressions builds it."""
    out = np.zeros((ni * nj * nk, 3))
    ext = np.ascontiguousarray(extent, dtype=np.float64)
    order = np.array([BLOCK_FACES.index(f) for f in patch_order], dtype=np.int32)
    if sorted(order.tolist()) != list(range(6)):
        raise ValueError("patch_order must name each block face once")
    if lib().oracle_blockmesh_centres(ni, nj, nk, ptr(ext), scale, iptr(order), contract,
                                      ptr(out)) != 0:
        raise ValueError("invalid block")
    return out


class Mesh:
    """blockMesh-style single block of nx*ny*nz hexes over [0,lx]x[0,ly]x[0,lz],
    or (``Mesh.general``) any mesh given by its lduAddressing and geometry."""

    def __init__(self, nx, ny, nz, lx, ly, lz):
        self.h = lib().oracle_mesh_box(nx, ny, nz, lx, ly, lz)
        self.n = lib().oracle_mesh_ncells(self.h)
        self.nf = lib().oracle_mesh_nfaces(self.h)

    @classmethod
    def general(cls, m):
        """From an object with n_cells, owner, neighbour, centres, volumes,
        face_centres, face_sf, boundary_cell, boundary_sf, boundary_centres."""
        self = cls.__new__(cls)
        keep = [np.ascontiguousarray(a, dtype=t) for a, t in (
            (m.owner, np.int32), (m.neighbour, np.int32), (m.centres, np.float64),
            (m.volumes, np.float64), (m.face_centres, np.float64), (m.face_sf, np.float64),
            (m.boundary_cell, np.int32), (m.boundary_sf, np.float64),
            (m.boundary_centres, np.float64))]
        o, nb, c, v, fc, sf, bc, bsf, bcf = keep
        self.h = lib().oracle_mesh_general(m.n_cells, o.size, iptr(o), iptr(nb), ptr(c), ptr(v),
                                           ptr(fc), ptr(sf), bc.size, iptr(bc), ptr(bsf),
                                           ptr(bcf))
        self.n = m.n_cells
        self.nf = o.size
        return self

    def addressing(self):
        o = np.zeros(self.nf, np.int32)
        nb = np.zeros(self.nf, np.int32)
        lib().oracle_mesh_addressing(self.h, iptr(o), iptr(nb))
        return o, nb

    def centres(self):
        c = np.zeros((self.n, 3))
        lib().oracle_mesh_centres(self.h, ptr(c))
        return c

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_mesh_free(self.h)
            self.h = None


def tissue_desc(model="TNNP", tissue=1, sigma=(0.1334177215, 0, 0, 0.01760617761, 0,
                                                0.01760617761),
                chi=140000.0, cm=0.01, implicit=True, ddt_backward=True, precond_dic=True,
                pcg_tol=1e-8, pcg_rel_tol=0.0, pcg_max_iter=1000, n_outer=1000,
                outer_tol=1e-6, vm0=-0.084, boxes: Sequence = (), ode=None,
                grad_gauss=False, uncorrected=False) -> TissueDesc:
    d = TissueDesc()
    d.model = MODELS[model] if isinstance(model, str) else model
    d.tissue = tissue
    for i, s in enumerate(sigma):
        d.sigma[i] = s
    d.chi, d.cm = chi, cm
    d.implicit, d.ddt_backward, d.precond_dic = int(implicit), int(ddt_backward), int(precond_dic)
    d.pcg_tol, d.pcg_rel_tol, d.pcg_max_iter = pcg_tol, pcg_rel_tol, pcg_max_iter
    d.n_outer, d.outer_tol, d.vm0 = n_outer, outer_tol, vm0
    d.n_boxes = len(boxes)
    for b, (lo, hi, t0, dur, inten) in enumerate(boxes):
        for k in range(3):
            d.box_min[b][k] = lo[k]
            d.box_max[b][k] = hi[k]
        d.box_start[b], d.box_duration[b], d.box_intensity[b] = t0, dur, inten
    d.ode = ode if ode is not None else ode_settings(max_steps=1000000000)
    d.grad_gauss, d.uncorrected = int(grad_gauss), int(uncorrected)
    return d


class Tissue:
    def __init__(self, desc: TissueDesc, mesh: Mesh):
        self.mesh = mesh
        self.desc = desc
        self.h = lib().oracle_tissue_new(C.byref(desc), mesh.h)
        self.n = mesh.n

    def step(self, dt, nthreads=1) -> int:
        it = lib().oracle_tissue_step(self.h, dt, nthreads)
        if it < 0:
            raise RuntimeError("oracle tissue step failed")
        return it

    def _arr(self, name):
        p = getattr(lib(), f"oracle_tissue_{name}")(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n,)).copy()

    def vm(self):
        return self._arr("vm")

    def set_vm(self, a):
        p = lib().oracle_tissue_vm(self.h)
        np.ctypeslib.as_array(p, shape=(self.n,))[:] = a

    def set_states(self, a, dt):
        """Ionic states as [n_states][n_cells]; constructs the ionic model
        with initialDeltaT = dt if no step has run yet."""
        if lib().oracle_tissue_init_ionic(self.h, dt):
            raise RuntimeError("oracle ionic model construction failed")
        p = lib().oracle_tissue_ionic(self.h)
        ns = sizes(list(MODELS)[self.desc.model])[0]
        sp = lib().oracle_ionic_states(p)
        np.ctypeslib.as_array(sp, shape=(self.n, ns))[:] = np.asarray(a).T

    def iion(self):
        return self._arr("iion")

    def activation(self):
        return self._arr("activation")

    def source(self):
        return self._arr("source")

    def time(self):
        return lib().oracle_tissue_time(self.h)

    def solves(self):
        ir = np.zeros(64)
        fr = np.zeros(64)
        it = np.zeros(64, np.int32)
        k = lib().oracle_tissue_last_solves(self.h, ptr(ir), ptr(fr), iptr(it), 64)
        return ir[:k], fr[:k], it[:k]

    def states(self):
        p = lib().oracle_tissue_ionic(self.h)
        if not p:
            return None
        ns = sizes(list(MODELS)[self.desc.model])[0]
        sp = lib().oracle_ionic_states(p)
        return np.ctypeslib.as_array(sp, shape=(self.n, ns)).copy()

    def set_conductivity(self, sigma6: np.ndarray):
        """Per-cell conductivity [n][6] (xx xy xz yy yz zz)."""
        a = np.ascontiguousarray(sigma6, dtype=np.float64).reshape(self.n, 6)
        lib().oracle_tissue_set_conductivity(self.h, ptr(a))

    def set_cell_tissue(self, flags: np.ndarray):
        a = np.ascontiguousarray(flags, dtype=np.uint8)
        if lib().oracle_tissue_set_cell_tissue(self.h, a.ctypes.data_as(C.POINTER(C.c_ubyte))):
            raise RuntimeError("cell tissue flags must be set before the first step")

    def laplacian(self, phi: np.ndarray) -> np.ndarray:
        """fvc::laplacian(sigma, phi) per cell."""
        p = np.ascontiguousarray(phi, dtype=np.float64)
        out = np.zeros(self.n)
        lib().oracle_tissue_laplacian(self.h, ptr(p), ptr(out))
        return out

    def pseudo_ecg(self, vm: np.ndarray, electrodes) -> np.ndarray:
        """PseudoECGSolver::compute of the field vm at the electrodes [n][3]."""
        v = np.ascontiguousarray(vm, dtype=np.float64)
        el = np.ascontiguousarray(electrodes, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(el.shape[0])
        if lib().oracle_tissue_pseudo_ecg(self.h, ptr(v), el.shape[0], ptr(el), ptr(out)):
            raise RuntimeError("the pseudo-ECG needs a general mesh")
        return out

    def gradient(self, phi: np.ndarray) -> np.ndarray:
        p = np.ascontiguousarray(phi, dtype=np.float64)
        g = np.zeros((self.n, 3))
        if lib().oracle_tissue_gradient(self.h, ptr(p), ptr(g)):
            raise RuntimeError("the cell gradient needs a general mesh")
        return g

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_tissue_free(self.h)
            self.h = None


def single_cell(model: str, tissue: int, dt: float, n_steps: int, ode=None, stim=None,
                scales=None):
    ns = sizes(model)[0]
    trace = np.zeros(n_steps)
    final = np.zeros(ns)
    sc = None if scales is None else np.ascontiguousarray(scales, dtype=np.float64)
    k = lib().oracle_single_cell(MODELS[model], tissue, dt, n_steps,
                                 C.byref(ode) if ode else None, C.byref(stim) if stim else None,
                                 ptr(sc) if sc is not None else None, ptr(trace), ptr(final))
    if k < 0:
        raise RuntimeError("oracle single cell failed")
    return trace, final, k


def single_cell_traces(model: str, tissue: int, dt: float, n_steps: int, state_b: int,
                       ode=None, stim=None, scales=None):
    """single_cell plus the trace of state `state_b` after each step."""
    ns = sizes(model)[0]
    trace = np.zeros(n_steps)
    btrace = np.zeros(n_steps)
    final = np.zeros(ns)
    sc = None if scales is None else np.ascontiguousarray(scales, dtype=np.float64)
    k = lib().oracle_single_cell_traces(MODELS[model], tissue, dt, n_steps,
                                        C.byref(ode) if ode else None,
                                        C.byref(stim) if stim else None,
                                        ptr(sc) if sc is not None else None, ptr(trace),
                                        state_b, ptr(btrace), ptr(final))
    if k < 0:
        raise RuntimeError("oracle single cell failed")
    return trace, btrace, final, k


# --- the reference's own model code, compiled verbatim (pinning only) -----

_ref = None


def ref_lib():
    """ctypes handle of oracle/_ref/libref_models.so, or None when absent."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not path.exists():
            if _build.build_ref() is None:
                return None
        L = C.CDLL(str(path))
        for m in ("tnnp", "ord", "torord_dyncl", "alievpanfilov", "buenoorovio"):
            getattr(L, f"ref_{m}_sizes").argtypes = [_ip, _ip, _ip]
            getattr(L, f"ref_{m}_init").argtypes = [_dp, _dp, _dp, C.c_int]
            for fn in ("rates", "variables"):
                getattr(L, f"ref_{m}_{fn}").argtypes = [C.c_double, _dp, _dp, _dp, _dp, C.c_int,
                                                       C.c_int, _dp]
        _ref = L
    return _ref


class _BorrowedTissue(Tissue):
    """The Vm side of a Bidomain (owned by it)."""

    def __init__(self, h, desc, mesh):
        self.h, self.desc, self.mesh, self.n = h, desc, mesh, mesh.n

    def __del__(self):
        pass


class Bidomain:
    """BidomainSolver restated (oracle_bidomain_*): desc carries Gi and the
    Vm solver settings; sigma_e is Ge; phiE's PCG has its own tolerances."""

    def __init__(self, desc: TissueDesc, sigma_e, mesh: Mesh, ref_point, ref_value=0.0,
                 phie_tol=1e-15, phie_rel_tol=0.0, phie_max_iter=1000):
        self.mesh = mesh
        self.n = mesh.n
        se = np.ascontiguousarray(sigma_e, dtype=np.float64)
        rp = np.ascontiguousarray(ref_point, dtype=np.float64)
        self.h = lib().oracle_bidomain_new(C.byref(desc), ptr(se), mesh.h, ptr(rp), ref_value,
                                           phie_tol, phie_rel_tol, phie_max_iter)
        if not self.h:
            raise RuntimeError("the oracle bidomain needs a general mesh")
        self.tissue = _BorrowedTissue(lib().oracle_bidomain_tissue(self.h), desc, mesh)

    def step(self, dt, nthreads=1) -> int:
        it = lib().oracle_bidomain_step(self.h, dt, nthreads)
        if it < 0:
            raise RuntimeError("oracle bidomain step failed")
        return it

    def phie(self):
        return np.ctypeslib.as_array(lib().oracle_bidomain_phie(self.h), shape=(self.n,)).copy()

    def phii(self):
        return np.ctypeslib.as_array(lib().oracle_bidomain_phii(self.h), shape=(self.n,)).copy()

    def set_phie(self, a):
        np.ctypeslib.as_array(lib().oracle_bidomain_phie(self.h), shape=(self.n,))[:] = a

    def ref_cell(self) -> int:
        return int(lib().oracle_bidomain_ref_cell(self.h))

    def phie_solves(self):
        ir, fr, it = np.zeros(64), np.zeros(64), np.zeros(64, np.int32)
        k = lib().oracle_bidomain_last_solves(self.h, ptr(ir), ptr(fr), iptr(it), 64)
        return ir[:k], fr[:k], it[:k]

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_bidomain_free(self.h)
            self.h = None


class Purkinje:
    """A conduction network (ConductionSystemDomain with Monodomain1DSolver)
    and, after ``couple``, its reaction-diffusion PVJ coupling to a Tissue."""

    def __init__(self, edges, model: str, tissue: int, initial_dt: float, chi=140000.0,
                 cm=0.01, root=0, root_stimulus=(1e300, 0.0, 0.0), pvj_nodes=(),
                 pvj_locations=(), ode: Optional[OdeSettings] = None):
        e = np.asarray(edges, dtype=np.float64).reshape(-1, 4)
        self._a = np.ascontiguousarray(e[:, 0], dtype=np.int32)
        self._b = np.ascontiguousarray(e[:, 1], dtype=np.int32)
        self._len = np.ascontiguousarray(e[:, 2])
        self._cond = np.ascontiguousarray(e[:, 3])
        self._tn = np.ascontiguousarray(pvj_nodes, dtype=np.int32).reshape(-1)
        self._tl = np.ascontiguousarray(pvj_locations, dtype=np.float64).reshape(-1, 3)
        start, dur, inten = root_stimulus
        self.h = lib().oracle_purkinje_new(
            len(e), iptr(self._a), iptr(self._b), ptr(self._len), ptr(self._cond), MODELS[model],
            tissue, C.byref(ode if ode is not None else ode_settings(max_steps=10 ** 6)),
            initial_dt, chi, cm, root, start, dur, inten, self._tn.size,
            iptr(self._tn) if self._tn.size else None,
            ptr(np.ascontiguousarray(self._tl)) if self._tn.size else None)
        if not self.h:
            raise ValueError("oracle_purkinje_new failed (not a connected tree?)")
        self.n = lib().oracle_purkinje_nodes(self.h)
        self.t = 0.0

    def _arr(self, name, n):
        p = getattr(lib(), f"oracle_purkinje_{name}")(self.h)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def vm(self):
        return self._arr("vm", self.n)

    def iion(self):
        return self._arr("iion", self.n)

    def terminal_current(self):
        return self._arr("terminal_current", max(self._tn.size, 1))[:self._tn.size]

    def advance(self, dt, nthreads=1):
        """The network alone: Monodomain1DSolver::advance(t, dt), then t += dt."""
        if lib().oracle_purkinje_advance(self.h, self.t, dt, nthreads) < 0:
            raise RuntimeError("oracle Purkinje advance failed")
        self.t = self.t + dt

    def couple(self, mesh: "Mesh", r_pvj: float, radius: float, bidirectional=False):
        if lib().oracle_purkinje_couple(self.h, mesh.h, r_pvj, radius, int(bidirectional)) < 0:
            raise ValueError("PVJ mapping failed (pvjRadius below the cell size?)")
        self._mesh = mesh

    def coupled_step(self, tissue: "Tissue", dt, nthreads=1):
        """One staggered step of the network coupled to the tissue."""
        if lib().oracle_purkinje_coupled_step(self.h, tissue.h, dt, nthreads) < 0:
            raise RuntimeError("oracle coupled step failed")
        self.t = tissue.time()

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_purkinje_free(self.h)
            self.h = None
