"""ctypes bindings of the C ABI in include/cardiac_gpu.h.

The shared library is built in-tree by :func:`cardiacfoam_gb300.build.build`.
There is no CPU fallback: every entry point runs on the GPU, and loading
fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Optional

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libcardiac_gpu.so"

CFG_OK = 0
CFG_ERR_INVALID = 1
CFG_ERR_CUDA = 2
CFG_ERR_ODE_STEPS = 4
CFG_ERR_NONFINITE = 8
CFG_ERR_PCG = 16
CFG_ERR_UNSUPPORTED = 32
PRECISION_FP64 = 0
PRECISION_MIXED = 1
FIELD_VM, FIELD_IION, FIELD_ACTIVATION, FIELD_SOURCE, FIELD_VM_OLD, FIELD_PHIE, FIELD_PHII = range(7)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)


class CfgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class OdeDesc(C.Structure):
    _fields_ = [("solver", C.c_char_p), ("abs_tol", C.c_double), ("rel_tol", C.c_double),
                ("max_steps", C.c_longlong), ("safe_scale", C.c_double),
                ("min_scale", C.c_double), ("max_scale", C.c_double),
                ("alpha_increase", C.c_double), ("alpha_decrease", C.c_double)]


class StimulusDesc(C.Structure):
    _fields_ = [("stim_start", C.c_double), ("stim_period_s1", C.c_double),
                ("stim_duration", C.c_double), ("stim_amplitude", C.c_double),
                ("nstim1", C.c_int), ("stim_period_s2", C.c_double), ("nstim2", C.c_int)]


class IonicDesc(C.Structure):
    _fields_ = [("ionic_model", C.c_char_p), ("tissue", C.c_char_p), ("n_cells", C.c_longlong),
                ("initial_delta_t", C.c_double), ("solve_vm_within_ode", C.c_int),
                ("precision", C.c_int), ("ode", OdeDesc), ("stimulus", StimulusDesc),
                ("tissue_per_cell", _up), ("scales", _dp)]


GRAD_LEAST_SQUARES, GRAD_GAUSS_LINEAR = 0, 1
ECG_FP64, ECG_FLOAT_PAIRS = 0, 1
PCG_FP64, PCG_FLOAT_PAIRS = 0, 1


class MeshDesc(C.Structure):
    _fields_ = [("n_cells", C.c_longlong), ("n_faces", C.c_longlong), ("owner", _ip),
                ("neighbour", _ip), ("volumes", _dp), ("centres", _dp), ("face_coeff", _dp),
                ("face_sf", _dp), ("face_delta_coeffs", _dp), ("structured", C.c_int * 3),
                ("face_centres", _dp), ("n_boundary_faces", C.c_longlong),
                ("boundary_cell", _ip), ("boundary_sf", _dp), ("boundary_centres", _dp)]


class MonodomainDesc(C.Structure):
    _fields_ = [("ionic", IonicDesc), ("conductivity", C.c_double * 6), ("chi", C.c_double),
                ("cm", C.c_double),
                ("implicit", C.c_int), ("ddt_backward", C.c_int), ("pcg_tol", C.c_double),
                ("pcg_rel_tol", C.c_double), ("pcg_max_iter", C.c_int), ("n_outer", C.c_int),
                ("outer_tol", C.c_double), ("vm0", C.c_double), ("n_boxes", C.c_int),
                ("box_min", (C.c_double * 3) * 8), ("box_max", (C.c_double * 3) * 8),
                ("box_start", C.c_double * 8), ("box_duration", C.c_double * 8),
                ("box_intensity", C.c_double * 8), ("conductivity_per_cell", _dp),
                ("grad_scheme", C.c_int), ("laplacian_uncorrected", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("n_solves", C.c_int), ("iterations", C.c_int * 16),
                ("initial_residual", C.c_double * 16), ("final_residual", C.c_double * 16)]


class BoxDiffusionDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("cell_volume", C.c_double), ("face_coeff", C.c_double * 3),
                ("chi", C.c_double), ("cm", C.c_double), ("ddt_backward", C.c_int),
                ("pcg_tol", C.c_double), ("pcg_rel_tol", C.c_double),
                ("pcg_max_iter", C.c_int)]


class SolveResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int),
                ("initial_residual", C.c_double), ("final_residual", C.c_double)]


NOALLOC_MAX_CELLS = 65536


class BatchDesc(C.Structure):
    _fields_ = [("ionic_model", C.c_char_p), ("tissue", C.c_char_p), ("n_cells", C.c_longlong),
                ("delta_t", C.c_double), ("precision", C.c_int), ("ode", OdeDesc),
                ("stimulus", C.c_void_p), ("end_time", C.c_void_p), ("scales", C.c_void_p),
                ("trace_cells", C.c_longlong), ("trace_samples", C.c_longlong),
                ("chunk", C.c_longlong)]

class AdjointDesc(C.Structure):
    _fields_ = [("ionic_model", C.c_char_p), ("tissue", C.c_char_p), ("delta_t", C.c_double),
                ("n_steps", C.c_longlong), ("substeps", C.c_int), ("checkpoint_every", C.c_int),
                ("sample_every", C.c_int), ("n_probes", C.c_int), ("probes", _ip),
                ("chi", C.c_double), ("cm", C.c_double), ("vm0", C.c_double),
                ("fibre", C.c_double * 3), ("n_boxes", C.c_int),
                ("box_min", (C.c_double * 3) * 8), ("box_max", (C.c_double * 3) * 8),
                ("box_start", C.c_double * 8), ("box_duration", C.c_double * 8),
                ("box_intensity", C.c_double * 8), ("pcg_tol", C.c_double),
                ("pcg_max_iter", C.c_int), ("precision", C.c_int)]


# every symbol declared in include/cardiac_gpu.h
class BidomainDesc(C.Structure):
    _fields_ = [("ionic", IonicDesc), ("conductivity_i", C.c_double * 6),
                ("conductivity_e", C.c_double * 6), ("chi", C.c_double), ("cm", C.c_double),
                ("ddt_backward", C.c_int), ("pcg_tol", C.c_double), ("pcg_rel_tol", C.c_double),
                ("pcg_max_iter", C.c_int), ("phie_tol", C.c_double),
                ("phie_rel_tol", C.c_double), ("phie_max_iter", C.c_int), ("n_outer", C.c_int),
                ("outer_tol", C.c_double), ("vm0", C.c_double), ("ref_point", C.c_double * 3),
                ("ref_value", C.c_double), ("n_boxes", C.c_int),
                ("box_min", (C.c_double * 3) * 8), ("box_max", (C.c_double * 3) * 8),
                ("box_start", C.c_double * 8), ("box_duration", C.c_double * 8),
                ("box_intensity", C.c_double * 8), ("grad_scheme", C.c_int),
                ("explicit_algorithm", C.c_int)]


class PurkinjeDesc(C.Structure):
    _fields_ = [("ionic", IonicDesc), ("n_edges", C.c_longlong), ("edge_a", _ip), ("edge_b", _ip),
                ("edge_length", _dp), ("edge_conductance", _dp), ("chi", C.c_double),
                ("cm", C.c_double), ("root_node", C.c_int), ("root_start", C.c_double),
                ("root_duration", C.c_double), ("root_intensity", C.c_double),
                ("n_pvj", C.c_int), ("pvj_nodes", _ip), ("pvj_locations", _dp)]


class PseudoEcgDesc(C.Structure):
    _fields_ = [("conductivity", C.c_double * 6), ("conductivity_per_cell", _dp),
                ("grad_scheme", C.c_int), ("n_electrodes", C.c_int), ("electrodes", _dp),
                ("max_rows", C.c_longlong), ("arithmetic", C.c_int)]


EXPORTS = [
    "cfg_last_error", "cfg_ionic_create", "cfg_ionic_solve", "cfg_ionic_solve_device",
    "cfg_ionic_num_states", "cfg_ionic_state_name", "cfg_ionic_get_states",
    "cfg_ionic_set_states", "cfg_ionic_get_steps", "cfg_ionic_rhs_evaluations",
    "cfg_ionic_destroy", "cfg_ionic_sweep_currents", "cfg_ionic_sweep_current", "cfg_monodomain_create", "cfg_monodomain_create_from_dict",
    "cfg_monodomain_step", "cfg_monodomain_run", "cfg_monodomain_set_graph", "cfg_monodomain_get_field",
    "cfg_monodomain_set_field", "cfg_monodomain_time", "cfg_monodomain_ionic",
    "cfg_monodomain_last_stats", "cfg_monodomain_set_timing", "cfg_monodomain_timings",
    "cfg_monodomain_stream", "cfg_monodomain_destroy", "cfg_box_diffusion_solve_noalloc",
    "cfg_monodomain_set_persistent", "cfg_monodomain_suggest_explicit_delta_t",
    "cfg_monodomain_set_pcg_arithmetic", "cfg_bidomain_set_pcg_arithmetic",
    "cfg_monodomain_delta_t", "cfg_monodomain_set_delta_t", "cfg_monodomain_set_wait_limit",
    "cfg_pseudo_ecg_set_wait_limit", "cfg_monodomain_track_apd", "cfg_monodomain_apd_results",
    "cfg_purkinje_create", "cfg_purkinje_step", "cfg_purkinje_couple", "cfg_purkinje_get_field",
    "cfg_purkinje_terminal_current", "cfg_purkinje_nodes", "cfg_purkinje_time",
    "cfg_purkinje_destroy",
    "cfg_batch_create", "cfg_batch_run", "cfg_batch_results",
    "cfg_batch_trace", "cfg_batch_get_states", "cfg_batch_stats", "cfg_batch_stream",
    "cfg_batch_destroy", "cfg_adjoint_create", "cfg_adjoint_set_target", "cfg_adjoint_forward",
    "cfg_adjoint_backward", "cfg_adjoint_destroy", "cfg_ionic_autotune", "cfg_monodomain_autotune",
    "cfg_ionic_set_launch", "cfg_ionic_trace_header", "cfg_ionic_trace_row",
    "cfg_pseudo_ecg_create", "cfg_pseudo_ecg_compute", "cfg_pseudo_ecg_compute_monodomain",
    "cfg_pseudo_ecg_record", "cfg_pseudo_ecg_record_field", "cfg_pseudo_ecg_series", "cfg_pseudo_ecg_reset",
    "cfg_pseudo_ecg_destroy", "cfg_pseudo_ecg_electrodes_from_dict",
    "cfg_bidomain_create", "cfg_bidomain_create_from_dict", "cfg_bidomain_step", "cfg_bidomain_run", "cfg_bidomain_get_field",
    "cfg_bidomain_set_field", "cfg_bidomain_device_field", "cfg_bidomain_last_stats",
    "cfg_bidomain_time",
    "cfg_bidomain_reference_cell", "cfg_bidomain_ionic", "cfg_bidomain_stream",
    "cfg_bidomain_destroy",
]

_lib = None


def load(path: Optional[os.PathLike] = None):
    """Load libcardiac_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with cardiacfoam_gb300.build.build() "
                           "(the GPU path has no CPU fallback)")
    L = C.CDLL(str(p))
    L.cfg_last_error.restype = C.c_char_p
    L.cfg_ionic_create.argtypes = [C.POINTER(IonicDesc), C.POINTER(C.c_void_p)]
    L.cfg_ionic_solve.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, _dp]
    L.cfg_ionic_solve_device.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p,
                                         C.c_void_p]
    L.cfg_ionic_num_states.argtypes = [C.c_void_p, _ip]
    L.cfg_ionic_state_name.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]
    L.cfg_ionic_get_states.argtypes = [C.c_void_p, _dp]
    L.cfg_ionic_set_states.argtypes = [C.c_void_p, _dp]
    L.cfg_ionic_get_steps.argtypes = [C.c_void_p, _dp]
    L.cfg_ionic_rhs_evaluations.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong)]
    L.cfg_ionic_destroy.argtypes = [C.c_void_p]
    L.cfg_ionic_sweep_currents.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.cfg_ionic_sweep_current.argtypes = [C.c_void_p, C.c_char_p, C.c_double, C.c_double, C.c_int,
                                          C.c_void_p, _ip, C.c_char_p, C.c_size_t]
    L.cfg_monodomain_create.argtypes = [C.POINTER(MonodomainDesc), C.POINTER(MeshDesc),
                                        C.POINTER(C.c_void_p)]
    L.cfg_monodomain_create_from_dict.argtypes = [C.c_char_p, C.POINTER(MeshDesc), C.c_double,
                                                  C.c_int, C.POINTER(C.c_void_p)]
    L.cfg_monodomain_step.argtypes = [C.c_void_p, C.c_double]
    L.cfg_monodomain_run.argtypes = [C.c_void_p, C.c_double, C.c_longlong]
    L.cfg_monodomain_set_graph.argtypes = [C.c_void_p, C.c_int]
    L.cfg_monodomain_get_field.argtypes = [C.c_void_p, C.c_int, _dp]
    L.cfg_monodomain_set_field.argtypes = [C.c_void_p, C.c_int, _dp]
    L.cfg_monodomain_time.argtypes = [C.c_void_p]
    L.cfg_monodomain_time.restype = C.c_double
    L.cfg_monodomain_ionic.argtypes = [C.c_void_p]
    L.cfg_monodomain_ionic.restype = C.c_void_p
    L.cfg_monodomain_last_stats.argtypes = [C.c_void_p, C.POINTER(StepStats)]
    L.cfg_monodomain_set_timing.argtypes = [C.c_void_p, C.c_int]
    L.cfg_monodomain_timings.argtypes = [C.c_void_p, _dp, _dp, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_longlong)]
    L.cfg_monodomain_stream.argtypes = [C.c_void_p]
    L.cfg_monodomain_stream.restype = C.c_void_p
    L.cfg_monodomain_destroy.argtypes = [C.c_void_p]
    L.cfg_monodomain_set_persistent.argtypes = [C.c_void_p, C.c_int]
    L.cfg_monodomain_set_pcg_arithmetic.argtypes = [C.c_void_p, C.c_int]
    L.cfg_bidomain_set_pcg_arithmetic.argtypes = [C.c_void_p, C.c_int]
    L.cfg_monodomain_suggest_explicit_delta_t.argtypes = [C.c_void_p, C.c_double, _dp]
    L.cfg_monodomain_delta_t.argtypes = [C.c_void_p, _dp]
    L.cfg_monodomain_set_delta_t.argtypes = [C.c_void_p, C.c_double]
    L.cfg_monodomain_set_wait_limit.argtypes = [C.c_void_p, C.c_longlong]
    L.cfg_monodomain_track_apd.argtypes = [C.c_void_p, C.c_int]
    L.cfg_purkinje_create.argtypes = [C.POINTER(PurkinjeDesc), C.POINTER(C.c_void_p)]
    L.cfg_purkinje_step.argtypes = [C.c_void_p, C.c_double]
    L.cfg_purkinje_couple.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(MeshDesc), C.c_double,
                                      C.c_double, C.c_int]
    L.cfg_purkinje_get_field.argtypes = [C.c_void_p, C.c_int, _dp]
    L.cfg_purkinje_terminal_current.argtypes = [C.c_void_p, _dp]
    L.cfg_purkinje_nodes.argtypes = [C.c_void_p]
    L.cfg_purkinje_nodes.restype = C.c_longlong
    L.cfg_purkinje_time.argtypes = [C.c_void_p]
    L.cfg_purkinje_time.restype = C.c_double
    L.cfg_purkinje_destroy.argtypes = [C.c_void_p]
    L.cfg_monodomain_apd_results.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp]
    L.cfg_pseudo_ecg_set_wait_limit.argtypes = [C.c_void_p, C.c_longlong]
    L.cfg_batch_create.argtypes = [C.POINTER(BatchDesc), C.POINTER(C.c_void_p)]
    L.cfg_batch_run.argtypes = [C.c_void_p]
    L.cfg_batch_results.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.cfg_batch_trace.argtypes = [C.c_void_p, _dp]
    L.cfg_batch_get_states.argtypes = [C.c_void_p, _dp]
    L.cfg_batch_stats.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_longlong)]
    L.cfg_batch_stream.argtypes = [C.c_void_p]
    L.cfg_batch_stream.restype = C.c_void_p
    L.cfg_batch_destroy.argtypes = [C.c_void_p]
    L.cfg_adjoint_create.argtypes = [C.POINTER(AdjointDesc), C.POINTER(MeshDesc),
                                     C.POINTER(C.c_void_p)]
    L.cfg_adjoint_set_target.argtypes = [C.c_void_p, _dp]
    L.cfg_adjoint_forward.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_double, _dp, _dp]
    L.cfg_adjoint_backward.argtypes = [C.c_void_p, _dp, _dp, _dp]
    L.cfg_adjoint_destroy.argtypes = [C.c_void_p]
    L.cfg_ionic_autotune.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p, _ip, _ip,
                                     C.POINTER(C.c_float)]
    L.cfg_monodomain_autotune.argtypes = [C.c_void_p, _ip, _ip, C.POINTER(C.c_float)]
    L.cfg_ionic_set_launch.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.cfg_ionic_trace_header.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_size_t]
    L.cfg_ionic_trace_row.argtypes = [C.c_void_p, C.c_longlong, C.c_double, C.c_char_p,
                                      C.c_char_p, C.c_size_t]
    L.cfg_pseudo_ecg_create.argtypes = [C.POINTER(PseudoEcgDesc), C.POINTER(MeshDesc),
                                        C.POINTER(C.c_void_p)]
    L.cfg_pseudo_ecg_compute.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, _dp]
    L.cfg_pseudo_ecg_compute_monodomain.argtypes = [C.c_void_p, C.c_void_p, _dp]
    L.cfg_pseudo_ecg_record.argtypes = [C.c_void_p, C.c_void_p]
    L.cfg_pseudo_ecg_record_field.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
    L.cfg_pseudo_ecg_series.argtypes = [C.c_void_p, _dp, _dp, C.c_longlong,
                                        C.POINTER(C.c_longlong)]
    L.cfg_pseudo_ecg_reset.argtypes = [C.c_void_p]
    L.cfg_pseudo_ecg_destroy.argtypes = [C.c_void_p]
    L.cfg_pseudo_ecg_electrodes_from_dict.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p,
                                                      C.c_size_t, _dp, C.c_int, _ip]
    L.cfg_bidomain_create.argtypes = [C.POINTER(BidomainDesc), C.POINTER(MeshDesc),
                                      C.POINTER(C.c_void_p)]
    L.cfg_bidomain_create_from_dict.argtypes = [C.c_char_p, C.POINTER(MeshDesc), C.c_double,
                                                C.c_int, C.POINTER(C.c_void_p)]
    L.cfg_bidomain_step.argtypes = [C.c_void_p, C.c_double]
    L.cfg_bidomain_run.argtypes = [C.c_void_p, C.c_double, C.c_longlong]
    L.cfg_bidomain_get_field.argtypes = [C.c_void_p, C.c_int, _dp]
    L.cfg_bidomain_set_field.argtypes = [C.c_void_p, C.c_int, _dp]
    L.cfg_bidomain_device_field.argtypes = [C.c_void_p, C.c_int]
    L.cfg_bidomain_device_field.restype = C.c_void_p
    L.cfg_bidomain_last_stats.argtypes = [C.c_void_p, C.POINTER(StepStats), C.POINTER(StepStats)]
    L.cfg_bidomain_time.argtypes = [C.c_void_p]
    L.cfg_bidomain_time.restype = C.c_double
    L.cfg_bidomain_reference_cell.argtypes = [C.c_void_p]
    L.cfg_bidomain_reference_cell.restype = C.c_longlong
    L.cfg_bidomain_ionic.argtypes = [C.c_void_p]
    L.cfg_bidomain_ionic.restype = C.c_void_p
    L.cfg_bidomain_stream.argtypes = [C.c_void_p]
    L.cfg_bidomain_stream.restype = C.c_void_p
    L.cfg_bidomain_destroy.argtypes = [C.c_void_p]
    L.cfg_box_diffusion_solve_noalloc.argtypes = [C.POINTER(BoxDiffusionDesc), C.c_double,
                                                  C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_void_p,
                                                  C.POINTER(SolveResult)]
    if path is None:
        _lib = L
    return L


def check(rc: int):
    if rc != CFG_OK:
        raise CfgError(rc, load().cfg_last_error().decode())


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def uptr(a: np.ndarray):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(_up)
