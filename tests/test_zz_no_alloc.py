"""The diffusion solve that allocates no device memory
(cfg_box_diffusion_solve_noalloc) against the existing entry point,
cfg_monodomain_step, on the same inputs.

The entry point keeps its temporaries in one static device array shared by
every call; the file is named to be collected last so that it also runs
after everything else has used the device in the same process, and it
passes alone in a fresh process as well.  Two calls in a row check that
what the first call leaves in the array does not leak into the second.
"""
import ctypes as C

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from cardiacfoam_gb300.mesh import box_mesh

H = 2.0 ** -13          # cell size [m]: exact geometry, one coefficient per direction
DIMS = (24, 16, 10)
SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
CHI, CM = 140000.0, 0.01
DT = 1e-5
RTOL = 1e-9             # the FP64 tolerance of the GPU parity tests


def _box():
    nx, ny, nz = DIMS
    return box_mesh(nx, ny, nz, nx * H, ny * H, nz * H)


def _desc(mesh, backward, max_iter=1000):
    nx, ny, nz = mesh.structured
    fc = mesh.face_coeff(SIGMA)
    step = mesh.neighbour.astype(np.int64) - mesh.owner
    d = lib.BoxDiffusionDesc()
    d.nx, d.ny, d.nz = nx, ny, nz
    assert np.all(mesh.volumes == mesh.volumes[0])
    d.cell_volume = float(mesh.volumes[0])
    for k, s in enumerate((1, nx, nx * ny)):
        v = fc[step == s]
        assert v.size and np.all(v == v[0])
        d.face_coeff[k] = float(v[0])
    d.chi, d.cm = CHI, CM
    d.ddt_backward = int(backward)
    d.pcg_tol, d.pcg_rel_tol, d.pcg_max_iter = 1e-8, 0.0, max_iter
    return d


def test_rejects_box_above_maximum(gpu_lib):
    """Size check before any device work (runs without a GPU)."""
    d = lib.BoxDiffusionDesc()
    d.nx, d.ny, d.nz = lib.NOALLOC_MAX_CELLS + 1, 1, 1
    d.cell_volume, d.chi, d.cm = 1e-12, CHI, CM
    d.face_coeff[0] = d.face_coeff[1] = d.face_coeff[2] = 1e-6
    d.pcg_tol, d.pcg_max_iter = 1e-8, 1000
    fake = C.c_void_p(256)      # never dereferenced: the size check fails first
    rc = gpu_lib.cfg_box_diffusion_solve_noalloc(C.byref(d), DT, fake, fake, fake, fake, None,
                                                 None)
    assert rc == lib.CFG_ERR_INVALID
    msg = gpu_lib.cfg_last_error().decode()
    assert "exceeds" in msg and str(lib.NOALLOC_MAX_CELLS) in msg


@pytest.mark.gpu
@pytest.mark.parametrize("backward", [False, True], ids=["euler", "backward"])
def test_noalloc_matches_monodomain_step(gpu_lib, backward):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh = _box()
    md = api.Monodomain(mesh, model="TNNP", tissue="epicardialCells", sigma=SIGMA, chi=CHI,
                        cm=CM, dt=DT, ddt_backward=backward, n_outer=1, pcg_tol=1e-8,
                        pcg_rel_tol=0.0, pcg_max_iter=1000)
    # a depolarised spot so that the solve has real work
    c = mesh.centres
    r2 = ((c - c.mean(axis=0)) ** 2).sum(axis=1)
    vm0 = -0.084 + 0.06 * np.exp(-r2 / (2 * (4 * H) ** 2))
    md.set_field(lib.FIELD_VM, vm0)          # before the first step: also the old levels
    md.run(DT, 2)
    d = _desc(mesh, backward)
    dev = torch.device("cuda", 0)
    for call in range(2):
        vm_before = md.vm()
        vm_old_before = md.field(lib.FIELD_VM_OLD)
        md.step(DT)                          # existing entry point
        expected = md.vm()
        iion = md.iion()
        iters = md.stats()[2]
        vo = torch.from_numpy(vm_before).to(dev)
        voo = torch.from_numpy(vm_old_before).to(dev)
        ii = torch.from_numpy(iion).to(dev)
        vm = vo.clone()                      # initial guess, as in the step
        torch.cuda.synchronize()
        res = lib.SolveResult()
        rc = gpu_lib.cfg_box_diffusion_solve_noalloc(
            C.byref(d), DT, C.c_void_p(vo.data_ptr()),
            C.c_void_p(voo.data_ptr()) if backward else None, C.c_void_p(ii.data_ptr()),
            C.c_void_p(vm.data_ptr()), None, C.byref(res))
        assert rc == lib.CFG_OK, gpu_lib.cfg_last_error().decode()
        got = vm.cpu().numpy()
        err = np.max(np.abs(got - expected)) / np.max(np.abs(expected))
        assert err <= RTOL, (call, err)
        assert np.max(np.abs(got - vm_before)) > 1e-6   # the solve changed Vm
        assert res.converged == 1
        assert abs(res.iterations - int(iters[0])) <= 1, (res.iterations, iters)
    md.close()


@pytest.mark.gpu
def test_noalloc_leaves_device_memory_unchanged(gpu_lib):
    """After a first call (which sets up the array's address), further calls
    change neither the free device memory (cudaMemGetInfo) nor the memory
    torch has reserved: the entry point allocates nothing."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh = _box()
    d = _desc(mesh, True)
    dev = torch.device("cuda", 0)
    n = mesh.n_cells
    c = mesh.centres
    r2 = ((c - c.mean(axis=0)) ** 2).sum(axis=1)
    v0 = torch.from_numpy(-0.084 + 0.06 * np.exp(-r2 / (2 * (4 * H) ** 2))).to(dev)
    vo, voo = v0.clone(), v0.clone()
    ii = torch.zeros(n, dtype=torch.float64, device=dev)
    vm = v0.clone()

    def call():
        res = lib.SolveResult()
        rc = gpu_lib.cfg_box_diffusion_solve_noalloc(
            C.byref(d), DT, C.c_void_p(vo.data_ptr()), C.c_void_p(voo.data_ptr()),
            C.c_void_p(ii.data_ptr()), C.c_void_p(vm.data_ptr()), None, C.byref(res))
        assert rc == lib.CFG_OK, gpu_lib.cfg_last_error().decode()
        assert res.converged == 1

    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    reserved0 = torch.cuda.memory_reserved(dev)
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
    assert torch.cuda.memory_reserved(dev) == reserved0
