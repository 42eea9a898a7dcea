"""Python view of the C ABI, shaped like the reference's plugin interfaces.

``IonicModel`` mirrors ``ionicModel::New(dict, nIntegrationPoints,
initialDeltaT, solveVmWithinODESolver)`` and ``solveODE(t0, dt, Vm, Im)``
(src/ionicModels/ionicModel/ionicModel.H:184-256); ``Monodomain`` mirrors a
MyocardiumDomain driven by MonodomainSolver (myocardiumDomain.C:180-529).
Both hold GPU-resident state; host arrays cross the boundary only in the
calls that take or return them.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import lib as _L
from .mesh import LduMesh

TISSUE_FLAGS = {"epicardialCells": 1, "mCells": 2, "endocardialCells": 3, "myocyte": 4,
                "1D": 11, "2D": 12, "3D": 13}


def ode_desc(solver="RKF45", abs_tol=-1.0, rel_tol=-1.0, max_steps=-1) -> _L.OdeDesc:
    d = _L.OdeDesc()
    d.solver = solver.encode() if solver else None
    d.abs_tol, d.rel_tol, d.max_steps = abs_tol, rel_tol, max_steps
    d.safe_scale = d.min_scale = d.max_scale = d.alpha_increase = d.alpha_decrease = -1.0
    return d


def stimulus_desc(stim_start=0.0, stim_period_s1=0.0, stim_duration=0.0, stim_amplitude=0.0,
                  nstim1=0, stim_period_s2=0.0, nstim2=0) -> _L.StimulusDesc:
    return _L.StimulusDesc(stim_start, stim_period_s1, stim_duration, stim_amplitude, nstim1,
                           stim_period_s2, nstim2)


def ionic_desc(model: str, tissue: str, n_cells: int, initial_delta_t: float,
               solve_vm_within_ode: bool = False, precision: int = _L.PRECISION_FP64,
               ode: Optional[_L.OdeDesc] = None, stimulus: Optional[_L.StimulusDesc] = None,
               tissue_per_cell: Optional[np.ndarray] = None,
               scales: Optional[np.ndarray] = None, _keep: Optional[list] = None) -> _L.IonicDesc:
    d = _L.IonicDesc()
    d.ionic_model = model.encode()
    d.tissue = tissue.encode() if tissue else None
    d.n_cells = n_cells
    d.initial_delta_t = initial_delta_t
    d.solve_vm_within_ode = int(solve_vm_within_ode)
    d.precision = precision
    d.ode = ode if ode is not None else ode_desc()
    d.stimulus = stimulus if stimulus is not None else stimulus_desc()
    if tissue_per_cell is not None:
        t = np.ascontiguousarray(tissue_per_cell, dtype=np.uint8)
        d.tissue_per_cell = _L.uptr(t)
        if _keep is not None:
            _keep.append(t)
    if scales is not None:
        s = np.ascontiguousarray(scales, dtype=np.float64)
        d.scales = _L.dptr(s)
        if _keep is not None:
            _keep.append(s)
    return d


class IonicModel:
    """ionicModel::New + solveODE on the GPU."""

    def __init__(self, model: str, tissue: str, n_cells: int, initial_delta_t: float,
                 solve_vm_within_ode: bool = False, precision: int = _L.PRECISION_FP64,
                 ode: Optional[_L.OdeDesc] = None, stimulus: Optional[_L.StimulusDesc] = None,
                 tissue_per_cell=None, scales=None):
        self._lib = _L.load()
        keep: list = []
        d = ionic_desc(model, tissue, n_cells, initial_delta_t, solve_vm_within_ode, precision,
                       ode, stimulus, tissue_per_cell, scales, keep)
        h = C.c_void_p()
        _L.check(self._lib.cfg_ionic_create(C.byref(d), C.byref(h)))
        self.h = h
        self.n = n_cells
        ns = C.c_int()
        _L.check(self._lib.cfg_ionic_num_states(self.h, C.byref(ns)))
        self.n_states = ns.value

    def solveODE(self, t0: float, dt: float, vm: Optional[np.ndarray], im: np.ndarray):
        vm_p = _L.dptr(vm) if vm is not None else None
        _L.check(self._lib.cfg_ionic_solve(self.h, t0, dt, vm_p, _L.dptr(im)))

    def state_names(self):
        out = []
        buf = C.create_string_buffer(128)
        for i in range(self.n_states):
            _L.check(self._lib.cfg_ionic_state_name(self.h, i, buf, 128))
            out.append(buf.value.decode())
        return out

    def sweep_currents(self) -> list:
        """availableSweepCurrents."""
        buf = C.create_string_buffer(8192)
        _L.check(self._lib.cfg_ionic_sweep_currents(self.h, buf, len(buf)))
        return buf.value.decode().split()

    def sweep_current(self, current: str, v_min: float, v_max: float, n_points: int):
        """sweepCurrent: (header column names, [n_points, columns] table)."""
        nc = C.c_int()
        hdr = C.create_string_buffer(8192)
        _L.check(self._lib.cfg_ionic_sweep_current(self.h, current.encode(), v_min, v_max,
                                                   n_points, None, C.byref(nc), hdr, len(hdr)))
        out = np.zeros((n_points, nc.value))
        _L.check(self._lib.cfg_ionic_sweep_current(self.h, current.encode(), v_min, v_max,
                                                   n_points, out.ctypes.data, C.byref(nc),
                                                   None, 0))
        return hdr.value.decode().split(","), out

    def states(self) -> np.ndarray:
        a = np.zeros((self.n_states, self.n))
        _L.check(self._lib.cfg_ionic_get_states(self.h, _L.dptr(a)))
        return a

    def set_states(self, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _L.check(self._lib.cfg_ionic_set_states(self.h, _L.dptr(a)))

    def steps(self) -> np.ndarray:
        a = np.zeros(self.n)
        _L.check(self._lib.cfg_ionic_get_steps(self.h, _L.dptr(a)))
        return a

    def rhs_evaluations(self) -> int:
        v = C.c_ulonglong()
        _L.check(self._lib.cfg_ionic_rhs_evaluations(self.h, C.byref(v)))
        return v.value

    def trace_header(self, columns: Optional[str] = None) -> str:
        buf = C.create_string_buffer(1 << 16)
        _L.check(self._lib.cfg_ionic_trace_header(self.h, columns.encode() if columns else None,
                                                  buf, len(buf)))
        return buf.value.decode()

    def trace_row(self, cell: int, t: float, columns: Optional[str] = None) -> str:
        buf = C.create_string_buffer(1 << 16)
        _L.check(self._lib.cfg_ionic_trace_row(self.h, cell, t,
                                               columns.encode() if columns else None, buf,
                                               len(buf)))
        return buf.value.decode()

    def set_launch(self, block: int, cells_per_thread: int):
        _L.check(self._lib.cfg_ionic_set_launch(self.h, block, cells_per_thread))

    def autotune(self, t0: float, dt: float):
        """(block, cells per thread, ms per step) chosen by timing."""
        b, c, ms = C.c_int(), C.c_int(), C.c_float()
        _L.check(self._lib.cfg_ionic_autotune(self.h, t0, dt, None, C.byref(b), C.byref(c),
                                              C.byref(ms)))
        return b.value, c.value, ms.value

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_ionic_destroy(self.h)
            self.h = None

    __del__ = close


def mesh_desc(mesh: LduMesh, face_coeff: Optional[np.ndarray] = None,
              structured: bool = True) -> tuple:
    keep = [mesh.owner, mesh.neighbour, mesh.volumes, mesh.centres, mesh.face_sf,
            mesh.face_delta_coeffs]
    d = _L.MeshDesc()
    d.n_cells = mesh.n_cells
    d.n_faces = mesh.n_faces
    d.owner = _L.iptr(mesh.owner)
    d.neighbour = _L.iptr(mesh.neighbour)
    d.volumes = _L.dptr(mesh.volumes)
    d.centres = _L.dptr(mesh.centres)
    d.face_sf = _L.dptr(np.ascontiguousarray(mesh.face_sf))
    d.face_delta_coeffs = _L.dptr(mesh.face_delta_coeffs)
    if face_coeff is not None:
        fc = np.ascontiguousarray(face_coeff, dtype=np.float64)
        keep.append(fc)
        d.face_coeff = _L.dptr(fc)
    if structured:
        for i in range(3):
            d.structured[i] = mesh.structured[i]
    if mesh.has_geometry:
        geo = [np.ascontiguousarray(mesh.face_centres, dtype=np.float64),
               np.ascontiguousarray(mesh.boundary_cell, dtype=np.int32),
               np.ascontiguousarray(mesh.boundary_sf, dtype=np.float64),
               np.ascontiguousarray(mesh.boundary_centres, dtype=np.float64)]
        keep.extend(geo)
        d.face_centres = _L.dptr(geo[0])
        d.n_boundary_faces = mesh.n_boundary_faces
        d.boundary_cell = _L.iptr(geo[1])
        d.boundary_sf = _L.dptr(geo[2])
        d.boundary_centres = _L.dptr(geo[3])
    return d, keep


class Monodomain:
    """MyocardiumDomain + MonodomainSolver on the GPU."""

    def __init__(self, mesh: LduMesh, model="TNNP", tissue="epicardialCells",
                 sigma=(0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176), chi=140000.0, cm=0.01,
                 dt=1e-5, precision=_L.PRECISION_FP64, implicit=True, ddt_backward=True,
                 pcg_tol=1e-8, pcg_rel_tol=0.0, pcg_max_iter=1000, n_outer=1000,
                 outer_tol=1e-6, vm0=-0.084, boxes: Sequence = (), ode=None,
                 tissue_per_cell=None, scales=None, stencil=True, max_steps=10 ** 6,
                 conductivity_per_cell=None, grad_scheme=_L.GRAD_LEAST_SQUARES,
                 laplacian_uncorrected=False):
        self._lib = _L.load()
        self.mesh = mesh
        keep: list = []
        d = _L.MonodomainDesc()
        d.ionic = ionic_desc(model, tissue, mesh.n_cells, dt, False, precision,
                             ode if ode is not None else ode_desc(max_steps=max_steps),
                             None, tissue_per_cell, scales, keep)
        for i, s in enumerate(sigma):
            d.conductivity[i] = s
        d.chi, d.cm = chi, cm
        d.implicit, d.ddt_backward = int(implicit), int(ddt_backward)
        d.pcg_tol, d.pcg_rel_tol, d.pcg_max_iter = pcg_tol, pcg_rel_tol, pcg_max_iter
        d.n_outer, d.outer_tol, d.vm0 = n_outer, outer_tol, vm0
        d.n_boxes = len(boxes)
        for b, (lo, hi, t0, dur, inten) in enumerate(boxes):
            for k in range(3):
                d.box_min[b][k] = lo[k]
                d.box_max[b][k] = hi[k]
            d.box_start[b], d.box_duration[b], d.box_intensity[b] = t0, dur, inten
        if conductivity_per_cell is not None:
            sig = np.ascontiguousarray(conductivity_per_cell, dtype=np.float64).reshape(-1, 6)
            if sig.shape[0] != mesh.n_cells:
                raise ValueError("conductivity_per_cell needs one row of 6 per cell")
            keep.append(sig)
            d.conductivity_per_cell = _L.dptr(sig)
        d.grad_scheme = int(grad_scheme)
        d.laplacian_uncorrected = int(laplacian_uncorrected)
        md, keep2 = mesh_desc(mesh, structured=stencil)
        h = C.c_void_p()
        _L.check(self._lib.cfg_monodomain_create(C.byref(d), C.byref(md), C.byref(h)))
        self.h = h
        self.n = mesh.n_cells

    @classmethod
    def from_dict(cls, text: str, mesh: LduMesh, dt: float, precision=_L.PRECISION_FP64,
                  stencil=True):
        self = cls.__new__(cls)
        self._lib = _L.load()
        self.mesh = mesh
        md, keep = mesh_desc(mesh, structured=stencil)
        h = C.c_void_p()
        _L.check(self._lib.cfg_monodomain_create_from_dict(text.encode(), C.byref(md), dt,
                                                           precision, C.byref(h)))
        self.h = h
        self.n = mesh.n_cells
        return self

    def step(self, dt: float):
        _L.check(self._lib.cfg_monodomain_step(self.h, dt))

    def run(self, dt: float, n_steps: int):
        _L.check(self._lib.cfg_monodomain_run(self.h, dt, n_steps))

    def field(self, which: int) -> np.ndarray:
        a = np.zeros(self.n)
        _L.check(self._lib.cfg_monodomain_get_field(self.h, which, _L.dptr(a)))
        return a

    def set_field(self, which: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _L.check(self._lib.cfg_monodomain_set_field(self.h, which, _L.dptr(a)))

    def vm(self):
        return self.field(_L.FIELD_VM)

    def iion(self):
        return self.field(_L.FIELD_IION)

    def activation(self):
        return self.field(_L.FIELD_ACTIVATION)

    def source(self):
        return self.field(_L.FIELD_SOURCE)

    def time(self) -> float:
        return self._lib.cfg_monodomain_time(self.h)

    def delta_t(self) -> float:
        """The context's time step (the explicit algorithm's Courant limit
        when created from an explicit electroProperties)."""
        v = C.c_double()
        _L.check(self._lib.cfg_monodomain_delta_t(self.h, C.byref(v)))
        return v.value

    def suggest_explicit_delta_t(self, max_co: float = 0.1) -> float:
        """MyocardiumDomain::suggestExplicitDeltaT(maxCo)."""
        v = C.c_double()
        _L.check(self._lib.cfg_monodomain_suggest_explicit_delta_t(self.h, max_co, C.byref(v)))
        return v.value

    def stats(self):
        s = _L.StepStats()
        _L.check(self._lib.cfg_monodomain_last_stats(self.h, C.byref(s)))
        k = min(s.n_solves, 16)
        return (np.array(s.initial_residual[:k]), np.array(s.final_residual[:k]),
                np.array(s.iterations[:k]))

    def states(self) -> np.ndarray:
        ion = self._lib.cfg_monodomain_ionic(self.h)
        ns = C.c_int()
        _L.check(self._lib.cfg_ionic_num_states(ion, C.byref(ns)))
        a = np.zeros((ns.value, self.n))
        _L.check(self._lib.cfg_ionic_get_states(ion, _L.dptr(a)))
        return a

    def set_states(self, a: np.ndarray):
        """Ionic states as [n_states][n_cells] (importFields)."""
        ion = self._lib.cfg_monodomain_ionic(self.h)
        a = np.ascontiguousarray(a, dtype=np.float64)
        _L.check(self._lib.cfg_ionic_set_states(ion, _L.dptr(a)))

    def rhs_evaluations(self) -> int:
        ion = self._lib.cfg_monodomain_ionic(self.h)
        v = C.c_ulonglong()
        _L.check(self._lib.cfg_ionic_rhs_evaluations(ion, C.byref(v)))
        return v.value

    def set_graph(self, enable: bool = True):
        _L.check(self._lib.cfg_monodomain_set_graph(self.h, int(enable)))

    def set_persistent(self, enable: bool = True):
        """One persistent diffusion kernel per step (default) or the kernel
        sequence per PCG iteration."""
        _L.check(self._lib.cfg_monodomain_set_persistent(self.h, int(enable)))

    def set_pcg_arithmetic(self, arithmetic: int):
        """PCG of the persistent solve in FP64 (lib.PCG_FP64) or float pairs
        (lib.PCG_FLOAT_PAIRS, the mixed form's default)."""
        _L.check(self._lib.cfg_monodomain_set_pcg_arithmetic(self.h, int(arithmetic)))

    def set_timing(self, enable: bool = True):
        _L.check(self._lib.cfg_monodomain_set_timing(self.h, int(enable)))

    def track_apd(self, every_steps: int):
        """Per-cell beat detection on Vm after every `every_steps`-th step
        (0 stops it)."""
        _L.check(self._lib.cfg_monodomain_track_apd(self.h, int(every_steps)))

    def apd_results(self):
        """(beats, last-beat APD90 [ms], its upstroke time [s]) per cell."""
        nb = np.zeros(self.n, dtype=np.int32)
        apd, tup = np.zeros(self.n), np.zeros(self.n)
        _L.check(self._lib.cfg_monodomain_apd_results(self.h, nb.ctypes.data, _L.dptr(apd),
                                                      _L.dptr(tup)))
        return nb, apd, tup

    def set_wait_limit(self, spins: int = -1):
        """Bound on each grid-barrier wait of the persistent diffusion
        kernel (spins; negative = the default, about a second)."""
        _L.check(self._lib.cfg_monodomain_set_wait_limit(self.h, int(spins)))

    def write(self, case_dir, patches=(("walls", "zeroGradient"),), precision=6):
        """Vm and activationTime as OpenFOAM ASCII volScalarFields in
        <case_dir>/<timeName>/."""
        from .io import write_monodomain_fields
        return write_monodomain_fields(self, case_dir, patches, precision)

    def autotune(self):
        """Pick the ionic kernel's launch shape by timing; (block, cells per
        thread, ms per ionic step)."""
        b, c, ms = C.c_int(), C.c_int(), C.c_float()
        _L.check(self._lib.cfg_monodomain_autotune(self.h, C.byref(b), C.byref(c), C.byref(ms)))
        return b.value, c.value, ms.value

    def timings(self):
        """(ionic ms, diffusion ms, steps, kernel launches) since set_timing."""
        a, b, n, k = C.c_double(), C.c_double(), C.c_longlong(), C.c_longlong()
        _L.check(self._lib.cfg_monodomain_timings(self.h, C.byref(a), C.byref(b), C.byref(n),
                                                  C.byref(k)))
        return a.value, b.value, n.value, k.value

    def stream(self) -> int:
        return self._lib.cfg_monodomain_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_monodomain_destroy(self.h)
            self.h = None

    __del__ = close


# NUM_STATES of the compiled models
STATE_COUNTS = {"TNNP": 17, "ORd": 41, "ToRORd_dynCl": 45, "AlievPanfilov": 2, "BuenoOrovio": 4,
                "monodomainFDAManufactured": 4, "bidomainFDAManufactured": 4}


class BatchCells:
    """SingleCellSolver for many independent cells (per-cell conductance
    scales, S1/S2 protocol and end time) in one persistent, work-stealing
    launch, with APD90 and peak Ca of each cell's last beat computed on the
    device.  ``stimuli`` is a sequence of ``stimulus_desc`` (model time
    units), ``end_time`` an array [s]."""

    def __init__(self, model: str, tissue: str, dt: float, stimuli: Sequence,
                 end_time: np.ndarray, precision: int = _L.PRECISION_FP64,
                 scales: Optional[np.ndarray] = None, ode=None, trace_cells: int = 0,
                 trace_samples: int = 0, chunk: int = 0):
        self._lib = _L.load()
        n = len(end_time)
        self.n = n
        self.model = model
        self._stim = (_L.StimulusDesc * n)(*stimuli)
        self._end = np.ascontiguousarray(end_time, dtype=np.float64)
        self._scales = None if scales is None else np.ascontiguousarray(scales, dtype=np.float64)
        d = _L.BatchDesc()
        d.ionic_model = model.encode()
        d.tissue = tissue.encode()
        d.n_cells = n
        d.delta_t = dt
        d.precision = precision
        d.ode = ode if ode is not None else ode_desc()
        d.stimulus = C.cast(self._stim, C.c_void_p)
        d.end_time = self._end.ctypes.data
        d.scales = None if self._scales is None else self._scales.ctypes.data
        d.trace_cells, d.trace_samples, d.chunk = trace_cells, trace_samples, chunk
        self.trace_cells, self.trace_samples = trace_cells, trace_samples
        h = C.c_void_p()
        _L.check(self._lib.cfg_batch_create(C.byref(d), C.byref(h)))
        self.h = h

    def run(self):
        _L.check(self._lib.cfg_batch_run(self.h))

    def results(self):
        """(beats detected, last-beat APD90 [ms], its upstroke time [s], its peak Ca)."""
        nb = np.zeros(self.n, dtype=np.int32)
        apd, tup, ca = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        _L.check(self._lib.cfg_batch_results(self.h, nb.ctypes.data, apd.ctypes.data,
                                             tup.ctypes.data, ca.ctypes.data))
        return nb, apd, tup, ca

    def trace(self) -> np.ndarray:
        """[trace_cells, 2, trace_samples]: Vm [mV] and Ca from t = 0."""
        a = np.zeros((self.trace_cells, 2, self.trace_samples))
        _L.check(self._lib.cfg_batch_trace(self.h, _L.dptr(a)))
        return a

    def states(self) -> np.ndarray:
        a = np.zeros((STATE_COUNTS[self.model], self.n))
        _L.check(self._lib.cfg_batch_get_states(self.h, _L.dptr(a)))
        return a

    def stats(self):
        """(RHS evaluations, solver steps, launches)."""
        e, s, l = C.c_ulonglong(), C.c_longlong(), C.c_longlong()
        _L.check(self._lib.cfg_batch_stats(self.h, C.byref(e), C.byref(s), C.byref(l)))
        return e.value, s.value, l.value

    def stream(self) -> int:
        return self._lib.cfg_batch_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_batch_destroy(self.h)
            self.h = None

    __del__ = close


class Bidomain:
    """MyocardiumDomain with the bidomainSolver on the GPU (cfg_bidomain_*,
    bidomainSolver.C:36-263): Vm, phiE and phiI, FP64 diffusion.  The mesh
    needs its full geometry; sigma_i / sigma_e are the uniform intra- and
    extracellular conductivity tensors (xx xy xz yy yz zz)."""

    def __init__(self, mesh: LduMesh, model="TNNP", tissue="epicardialCells",
                 sigma_i=(0.17, 0.0, 0.0, 0.019, 0.0, 0.019),
                 sigma_e=(0.62, 0.0, 0.0, 0.24, 0.0, 0.24), chi=140000.0, cm=0.01, dt=1e-5,
                 precision=_L.PRECISION_FP64, ddt_backward=True, pcg_tol=1e-8, pcg_rel_tol=0.0,
                 pcg_max_iter=1000, phie_tol=1e-8, phie_rel_tol=0.0, phie_max_iter=1000,
                 n_outer=1, outer_tol=0.0, vm0=-0.084, ref_point=(0.0, 0.0, 0.0),
                 ref_value=0.0, boxes: Sequence = (), ode=None, max_steps=10 ** 6,
                 grad_scheme=_L.GRAD_LEAST_SQUARES, implicit=True):
        self._lib = _L.load()
        if not mesh.has_geometry:
            raise ValueError("the bidomain step needs a mesh with its full geometry")
        self.mesh = mesh
        self.n = mesh.n_cells
        keep: list = []
        d = _L.BidomainDesc()
        d.ionic = ionic_desc(model, tissue, mesh.n_cells, dt, False, precision,
                             ode if ode is not None else ode_desc(max_steps=max_steps),
                             None, None, None, keep)
        for i in range(6):
            d.conductivity_i[i] = sigma_i[i]
            d.conductivity_e[i] = sigma_e[i]
        # ECGDomain::conductivity() of a bidomain source is Gi (bidomainSolver.H:76-78)
        self.sigma_i = tuple(float(v) for v in sigma_i)
        d.chi, d.cm = chi, cm
        d.ddt_backward = int(ddt_backward)
        d.explicit_algorithm = int(not implicit)
        d.pcg_tol, d.pcg_rel_tol, d.pcg_max_iter = pcg_tol, pcg_rel_tol, pcg_max_iter
        d.phie_tol, d.phie_rel_tol, d.phie_max_iter = phie_tol, phie_rel_tol, phie_max_iter
        d.n_outer, d.outer_tol, d.vm0 = n_outer, outer_tol, vm0
        for k in range(3):
            d.ref_point[k] = ref_point[k]
        d.ref_value = ref_value
        d.n_boxes = len(boxes)
        for b, (lo, hi, t0, dur, inten) in enumerate(boxes):
            for k in range(3):
                d.box_min[b][k] = lo[k]
                d.box_max[b][k] = hi[k]
            d.box_start[b], d.box_duration[b], d.box_intensity[b] = t0, dur, inten
        d.grad_scheme = int(grad_scheme)
        md, keep2 = mesh_desc(mesh, structured=False)
        h = C.c_void_p()
        _L.check(self._lib.cfg_bidomain_create(C.byref(d), C.byref(md), C.byref(h)))
        self.h = h

    @classmethod
    def from_dict(cls, text: str, mesh: LduMesh, dt: float, precision=_L.PRECISION_FP64):
        """From the text of a constant/electroProperties file with
        myocardiumSolver bidomainSolver (cfg_bidomain_create_from_dict)."""
        if not mesh.has_geometry:
            raise ValueError("the bidomain step needs a mesh with its full geometry")
        self = cls.__new__(cls)
        self._lib = _L.load()
        self.mesh = mesh
        self.n = mesh.n_cells
        md, keep = mesh_desc(mesh, structured=False)
        h = C.c_void_p()
        _L.check(self._lib.cfg_bidomain_create_from_dict(text.encode(), C.byref(md), dt,
                                                         precision, C.byref(h)))
        self.h = h
        return self

    def step(self, dt: float):
        _L.check(self._lib.cfg_bidomain_step(self.h, dt))

    def set_pcg_arithmetic(self, arithmetic: int):
        """PCG of both systems in FP64 (lib.PCG_FP64) or float pairs
        (lib.PCG_FLOAT_PAIRS, the mixed form's default)."""
        _L.check(self._lib.cfg_bidomain_set_pcg_arithmetic(self.h, int(arithmetic)))

    def run(self, dt: float, n_steps: int):
        _L.check(self._lib.cfg_bidomain_run(self.h, dt, n_steps))

    def field(self, which: int) -> np.ndarray:
        a = np.zeros(self.n)
        _L.check(self._lib.cfg_bidomain_get_field(self.h, which, _L.dptr(a)))
        return a

    def set_field(self, which: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _L.check(self._lib.cfg_bidomain_set_field(self.h, which, _L.dptr(a)))

    def vm(self):
        return self.field(_L.FIELD_VM)

    def phie(self):
        return self.field(_L.FIELD_PHIE)

    def phii(self):
        return self.field(_L.FIELD_PHII)

    def iion(self):
        return self.field(_L.FIELD_IION)

    def activation(self):
        return self.field(_L.FIELD_ACTIVATION)

    def time(self) -> float:
        return self._lib.cfg_bidomain_time(self.h)

    def reference_cell(self) -> int:
        return int(self._lib.cfg_bidomain_reference_cell(self.h))

    def stats(self):
        """((init, final, iterations) of the Vm solves, the same of the phiE
        solves) of the last step."""
        a, b = _L.StepStats(), _L.StepStats()
        _L.check(self._lib.cfg_bidomain_last_stats(self.h, C.byref(a), C.byref(b)))
        out = []
        for s in (a, b):
            k = min(s.n_solves, 16)
            out.append((np.array(s.initial_residual[:k]), np.array(s.final_residual[:k]),
                        np.array(s.iterations[:k])))
        return tuple(out)

    def states(self) -> np.ndarray:
        ion = self._lib.cfg_bidomain_ionic(self.h)
        ns = C.c_int()
        _L.check(self._lib.cfg_ionic_num_states(ion, C.byref(ns)))
        a = np.zeros((ns.value, self.n))
        _L.check(self._lib.cfg_ionic_get_states(ion, _L.dptr(a)))
        return a

    def set_states(self, a: np.ndarray):
        ion = self._lib.cfg_bidomain_ionic(self.h)
        a = np.ascontiguousarray(a, dtype=np.float64)
        _L.check(self._lib.cfg_ionic_set_states(ion, _L.dptr(a)))

    def stream(self) -> int:
        return self._lib.cfg_bidomain_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_bidomain_destroy(self.h)
            self.h = None

    __del__ = close


def ecg_electrodes(text: str, domain: Optional[str] = None):
    """(names, positions [n][3]) of an ecgDomains entry of an electroProperties
    text (ECGDomain::readElectrodes, ecgDomain.C:53-82), in the dictionary's
    order; the first ecgDomains entry when domain is None."""
    lib = _L.load()
    n = C.c_int()
    dom = domain.encode() if domain else None
    rc = lib.cfg_pseudo_ecg_electrodes_from_dict(text.encode(), dom, None, 0, None, 0,
                                                 C.byref(n))
    k = n.value
    if rc != _L.CFG_OK and k == 0:   # with k > 0 the first call only found no room
        _L.check(rc)
    pos = np.zeros((max(k, 1), 3))
    buf = C.create_string_buffer(len(text) + 1)
    _L.check(lib.cfg_pseudo_ecg_electrodes_from_dict(text.encode(), dom, buf, len(buf),
                                                     _L.dptr(pos), k, C.byref(n)))
    names = buf.value.decode().split()
    return names, pos[:k].copy()


class PseudoECG:
    """ECGDomain with the pseudoECG solver on the GPU (cfg_pseudo_ecg_*,
    pseudoECGSolver.C:34-87): phi at each electrode of the domain's Vm.

    The mesh needs its full geometry (LduMesh.has_geometry); conductivity is
    the monodomain's (uniform or per cell) and grad_scheme its gradSchemes
    default.  ``record`` after each step keeps the time series on the device
    (up to ``max_rows`` rows) without waiting for the GPU.  ``arithmetic``:
    ECG_FLOAT_PAIRS (default; 48-bit significands on the FP32 pipe, within
    1e-12 of the FP64 sum relative to the largest electrode value on the
    tests' fields) or ECG_FP64 (bound by GB300's FP64 pipe)."""

    def __init__(self, mesh: LduMesh, electrodes, names: Optional[Sequence[str]] = None,
                 sigma=(0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176), conductivity_per_cell=None,
                 grad_scheme=_L.GRAD_LEAST_SQUARES, max_rows: int = 0,
                 arithmetic=_L.ECG_FLOAT_PAIRS):
        self._lib = _L.load()
        if not mesh.has_geometry:
            raise ValueError("the pseudo-ECG needs a mesh with its full geometry")
        self.electrodes = np.ascontiguousarray(electrodes, dtype=np.float64).reshape(-1, 3)
        self.n_electrodes = self.electrodes.shape[0]
        self.names = list(names) if names is not None else [f"E{i + 1}" for i in
                                                            range(self.n_electrodes)]
        if len(self.names) != self.n_electrodes:
            raise ValueError("one name per electrode")
        self.n = mesh.n_cells
        self.max_rows = int(max_rows)
        self.sigma = tuple(float(v) for v in sigma)
        self.per_cell = conductivity_per_cell is not None
        d = _L.PseudoEcgDesc()
        for i, v in enumerate(sigma):
            d.conductivity[i] = v
        keep = [self.electrodes]
        if conductivity_per_cell is not None:
            sig = np.ascontiguousarray(conductivity_per_cell, dtype=np.float64).reshape(-1, 6)
            if sig.shape[0] != mesh.n_cells:
                raise ValueError("conductivity_per_cell needs one row of 6 per cell")
            keep.append(sig)
            d.conductivity_per_cell = _L.dptr(sig)
        d.grad_scheme = int(grad_scheme)
        d.n_electrodes = self.n_electrodes
        d.electrodes = _L.dptr(self.electrodes)
        d.max_rows = self.max_rows
        d.arithmetic = int(arithmetic)
        md, keep2 = mesh_desc(mesh, structured=False)
        h = C.c_void_p()
        _L.check(self._lib.cfg_pseudo_ecg_create(C.byref(d), C.byref(md), C.byref(h)))
        self.h = h

    @classmethod
    def from_dict(cls, text: str, mesh: LduMesh, domain: Optional[str] = None, **kw):
        """Electrodes of the electroProperties' ecgDomains entry."""
        names, pos = ecg_electrodes(text, domain)
        return cls(mesh, pos, names=names, **kw)

    def _device_field(self, x):
        import torch
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float64
                and x.is_contiguous() and x.numel() == self.n):
            raise ValueError("a contiguous CUDA float64 tensor of n_cells values")
        return (C.c_void_p(x.data_ptr()),
                C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream))

    def _bidomain_vm(self, bd: "Bidomain"):
        if bd.n != self.n:
            raise ValueError("the bidomain context has another cell count")
        # the lead rows fold in the conductivity: for a bidomain source it must
        # be the intracellular Gi, as ECGDomain::conductivity() gives it
        if self.per_cell or self.sigma != bd.sigma_i:
            raise ValueError("a pseudo-ECG of a bidomain context needs that context's "
                             "intracellular conductivity sigma_i")
        return (C.c_void_p(self._lib.cfg_bidomain_device_field(bd.h, _L.FIELD_VM)),
                C.c_void_p(bd.stream()))

    def compute(self, source) -> np.ndarray:
        """phi [n_electrodes] of a Monodomain's or a Bidomain's Vm, or of a CUDA
        tensor of n_cells doubles (on torch's current stream)."""
        out = np.zeros(self.n_electrodes)
        if isinstance(source, Monodomain):
            _L.check(self._lib.cfg_pseudo_ecg_compute_monodomain(self.h, source.h,
                                                                 _L.dptr(out)))
            return out
        if isinstance(source, Bidomain):
            vm, stream = self._bidomain_vm(source)
            _L.check(self._lib.cfg_pseudo_ecg_compute(self.h, vm, stream, _L.dptr(out)))
            return out
        vm, stream = self._device_field(source)
        _L.check(self._lib.cfg_pseudo_ecg_compute(self.h, vm, stream, _L.dptr(out)))
        return out

    def record(self, source, t: Optional[float] = None):
        """Append phi of a Monodomain's or a Bidomain's Vm (at its time), or of
        a CUDA tensor at time t, to the device series without waiting."""
        if isinstance(source, Monodomain):
            _L.check(self._lib.cfg_pseudo_ecg_record(self.h, source.h))
            return
        if isinstance(source, Bidomain):
            vm, stream = self._bidomain_vm(source)
            _L.check(self._lib.cfg_pseudo_ecg_record_field(self.h, vm, stream, source.time()))
            return
        vm, stream = self._device_field(source)
        _L.check(self._lib.cfg_pseudo_ecg_record_field(self.h, vm, stream,
                                                       float(0.0 if t is None else t)))

    def series(self):
        """(times [rows], values [rows][n_electrodes]) recorded so far."""
        n = C.c_longlong()
        _L.check(self._lib.cfg_pseudo_ecg_series(self.h, None, None, 0, C.byref(n)))
        t = np.zeros(max(n.value, 1))
        v = np.zeros((max(n.value, 1), self.n_electrodes))
        _L.check(self._lib.cfg_pseudo_ecg_series(self.h, _L.dptr(t), _L.dptr(v), n.value,
                                                 C.byref(n)))
        return t[:n.value].copy(), v[:n.value].copy()

    def reset(self):
        _L.check(self._lib.cfg_pseudo_ecg_reset(self.h))

    def set_wait_limit(self, cycles: int = -1):
        """Bound on each tile-copy wait of the staged kernel (clock cycles;
        negative = the default, about a second)."""
        _L.check(self._lib.cfg_pseudo_ecg_set_wait_limit(self.h, int(cycles)))

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_pseudo_ecg_destroy(self.h)
            self.h = None

    __del__ = close


class Purkinje:
    """ConductionSystemDomain with Monodomain1DSolver on the GPU
    (cfg_purkinje_*, monodomain1DSolver.C:36-190): a tree of conduction
    edges (nodeA, nodeB, length [m], conductance [S/m]) rooted at node 0, an
    ionic model on its nodes, a root stimulus (node, start [s], duration [s],
    intensity) and PVJ terminals (nodes and locations)."""

    def __init__(self, edges, model="BuenoOrovio", tissue="epicardialCells", dt=1e-5,
                 precision=_L.PRECISION_FP64, chi=140000.0, cm=0.01, root_stimulus=None,
                 pvj_nodes=(), pvj_locations=(), ode=None, max_steps=10 ** 6):
        self._lib = _L.load()
        e = np.asarray(edges, dtype=np.float64).reshape(-1, 4)
        self._a = np.ascontiguousarray(e[:, 0], dtype=np.int32)
        self._b = np.ascontiguousarray(e[:, 1], dtype=np.int32)
        self._len = np.ascontiguousarray(e[:, 2])
        self._cond = np.ascontiguousarray(e[:, 3])
        self.n = int(max(self._a.max(), self._b.max())) + 1
        self._tn = np.ascontiguousarray(pvj_nodes, dtype=np.int32).reshape(-1)
        self._tl = np.ascontiguousarray(pvj_locations, dtype=np.float64).reshape(-1, 3)
        self.n_pvj = int(self._tn.size)
        keep: list = []
        d = _L.PurkinjeDesc()
        d.ionic = ionic_desc(model, tissue, self.n, dt, False, precision,
                             ode if ode is not None else ode_desc(max_steps=max_steps),
                             None, None, None, keep)
        d.n_edges = len(e)
        d.edge_a, d.edge_b = _L.iptr(self._a), _L.iptr(self._b)
        d.edge_length, d.edge_conductance = _L.dptr(self._len), _L.dptr(self._cond)
        d.chi, d.cm = chi, cm
        node, start, dur, inten = root_stimulus if root_stimulus else (0, 1e300, 0.0, 0.0)
        d.root_node, d.root_start, d.root_duration, d.root_intensity = node, start, dur, inten
        d.n_pvj = self.n_pvj
        if self.n_pvj:
            d.pvj_nodes = _L.iptr(self._tn)
            d.pvj_locations = _L.dptr(self._tl)
        h = C.c_void_p()
        _L.check(self._lib.cfg_purkinje_create(C.byref(d), C.byref(h)))
        self.h = h

    def step(self, dt: float):
        _L.check(self._lib.cfg_purkinje_step(self.h, dt))

    def couple(self, tissue: "Monodomain", r_pvj: float, pvj_radius: float,
               bidirectional=False):
        """reactionDiffusionPvjCoupler with a monodomain context: from now on
        the context's steps advance the network too."""
        md, self._mesh_keep = mesh_desc(tissue.mesh, structured=False)
        _L.check(self._lib.cfg_purkinje_couple(self.h, tissue.h, C.byref(md), r_pvj, pvj_radius,
                                               int(bidirectional)))
        self._tissue = tissue

    def vm(self) -> np.ndarray:
        a = np.zeros(self.n)
        _L.check(self._lib.cfg_purkinje_get_field(self.h, _L.FIELD_VM, _L.dptr(a)))
        return a

    def iion(self) -> np.ndarray:
        a = np.zeros(self.n)
        _L.check(self._lib.cfg_purkinje_get_field(self.h, _L.FIELD_IION, _L.dptr(a)))
        return a

    def terminal_current(self) -> np.ndarray:
        a = np.zeros(max(self.n_pvj, 1))
        _L.check(self._lib.cfg_purkinje_terminal_current(self.h, _L.dptr(a)))
        return a[:self.n_pvj]

    def time(self) -> float:
        return self._lib.cfg_purkinje_time(self.h)

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_purkinje_destroy(self.h)
            self.h = None

    __del__ = close


class AdjointProblem:
    """Probe-voltage misfit of the differentiable monodomain step and its
    gradient (cfg_adjoint_*): per-cell log-scales of TNNP g_Na and g_K1 and
    the conductivities sigma_l, sigma_t along/across the fibre direction."""

    def __init__(self, mesh: LduMesh, n_steps: int, dt: float, probes: Sequence[int],
                 sample_every: int, checkpoint_every: int = 200, substeps: int = 5,
                 tissue="epicardialCells", chi=140000.0, cm=0.01, vm0=-0.084,
                 fibre=(1.0, 0.0, 0.0), boxes: Sequence = (), pcg_tol=1e-13,
                 pcg_max_iter=10000, precision=_L.PRECISION_FP64):
        self._lib = _L.load()
        self.mesh = mesh
        self.n = mesh.n_cells
        self.n_steps = n_steps
        self.dt = dt
        self.probes = np.ascontiguousarray(probes, dtype=np.int32)
        self.n_samples = n_steps // sample_every
        d = _L.AdjointDesc()
        d.ionic_model = b"TNNP"
        d.tissue = tissue.encode()
        d.delta_t = dt
        d.n_steps = n_steps
        d.substeps = substeps
        d.checkpoint_every = checkpoint_every
        d.sample_every = sample_every
        d.n_probes = self.probes.size
        d.probes = _L.iptr(self.probes)
        d.chi, d.cm, d.vm0 = chi, cm, vm0
        for k in range(3):
            d.fibre[k] = fibre[k]
        d.n_boxes = len(boxes)
        for b, (lo, hi, t0, dur, inten) in enumerate(boxes):
            for k in range(3):
                d.box_min[b][k] = lo[k]
                d.box_max[b][k] = hi[k]
            d.box_start[b], d.box_duration[b], d.box_intensity[b] = t0, dur, inten
        d.pcg_tol, d.pcg_max_iter = pcg_tol, pcg_max_iter
        d.precision = precision
        md, self._keep = mesh_desc(mesh, structured=False)
        h = C.c_void_p()
        _L.check(self._lib.cfg_adjoint_create(C.byref(d), C.byref(md), C.byref(h)))
        self.h = h

    def set_target(self, target: np.ndarray):
        t = np.ascontiguousarray(target, dtype=np.float64).reshape(self.n_samples,
                                                                   self.probes.size)
        _L.check(self._lib.cfg_adjoint_set_target(self.h, _L.dptr(t)))

    def forward(self, log_gna: np.ndarray, log_gk1: np.ndarray, sigma_l: float,
                sigma_t: float):
        """(J, probe trace [n_samples][n_probes])."""
        a = np.ascontiguousarray(log_gna, dtype=np.float64)
        b = np.ascontiguousarray(log_gk1, dtype=np.float64)
        loss = np.zeros(1)
        trace = np.zeros((self.n_samples, self.probes.size))
        _L.check(self._lib.cfg_adjoint_forward(self.h, _L.dptr(a), _L.dptr(b), float(sigma_l),
                                               float(sigma_t), _L.dptr(loss), _L.dptr(trace)))
        return float(loss[0]), trace

    def backward(self):
        """(dJ/dlog_gna [n], dJ/dlog_gk1 [n], dJ/d(sigma_l, sigma_t) [2])."""
        ga, gb, gs = np.zeros(self.n), np.zeros(self.n), np.zeros(2)
        _L.check(self._lib.cfg_adjoint_backward(self.h, _L.dptr(ga), _L.dptr(gb), _L.dptr(gs)))
        return ga, gb, gs

    def close(self):
        if getattr(self, "h", None):
            self._lib.cfg_adjoint_destroy(self.h)
            self.h = None

    __del__ = close
