"""Oracle runs of the manufactured monodomain case (shared by the CPU and
GPU manufactured-solution tests)."""
import numpy as np

from cardiacfoam_gb300 import verification as vf


def oracle_run(po, dim, n, dt=None, end=vf.END_TIME, precond_dic=False, tol=1e-12,
               nthreads=4):
    dt = vf.SWEEP[n] if dt is None else dt
    mesh = vf.mesh_for(dim, n)
    om = po.Mesh(*mesh.structured, 1.0, 1.0 if dim >= 2 else 0.1, 1.0 if dim == 3 else 0.1)
    d = po.tissue_desc("monodomainFDAManufactured", 10 + dim, vf.SIGMA, chi=vf.CHI, cm=vf.CM,
                       implicit=True, ddt_backward=True, precond_dic=precond_dic, pcg_tol=tol,
                       pcg_max_iter=2000, n_outer=2, outer_tol=0.0, vm0=0.0)
    T = po.Tissue(d, om)
    V, u1, u2, u3 = vf.manufactured_fields(mesh.centres, 0.0, dim)
    T.set_vm(V)
    T.set_states(np.stack([V, u1, u2, u3]), dt)
    for _ in range(int(round(end / dt))):
        T.step(dt, nthreads)
    Ve, u1e, u2e, _ = vf.manufactured_fields(mesh.centres, T.time(), dim)
    st = T.states().T
    return {"vm": T.vm(), "V": vf.norms(T.vm(), Ve), "u1": vf.norms(st[1], u1e),
            "u2": vf.norms(st[2], u2e), "t": T.time()}
