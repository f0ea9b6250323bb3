"""The allocation-free CVWM deposition (pic_deposit_cvwm_noalloc) against pic_deposit.

The entry point serves callers that cannot call cudaMalloc during their time loop: they pass
their own device arrays, and the node-sum scratch is a fixed device array inside the library.
This test plays such a caller (its device arrays are made with torch beforehand), calls the
entry point twice in a row through the C-ABI and compares each result with the context's own
deposition at the tolerance the other parity tests use (1e-12 of the maximum: atomic order).
"""
import ctypes as C

import numpy as np
import pytest

from piclas_gb300 import ParticleLoop, capi, workloads
from piclas_gb300.mesh import build_box_mesh

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_noalloc_deposit_matches_pic_deposit(gpu_lib):
    import torch
    w = workloads.plasma_wave(n_cells=8, N=3, n_particles=30000, seed=21, T_eV=50.0)
    loop = ParticleLoop(w.config(), w.mesh)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    ref = loop.deposition()
    ps = torch.from_numpy(np.ascontiguousarray(w.part_state)).cuda()
    el = torch.from_numpy(np.ascontiguousarray(w.elem, dtype=np.int32)).cuda()
    sp = torch.from_numpy(np.ascontiguousarray(w.part_species, dtype=np.int32)).cuda()
    out = torch.empty(w.mesh.n_elems * w.mesh.n_dof * 4, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        out.fill_(float("nan"))            # the result must be fully written by the call
        torch.cuda.synchronize()
        rc = gpu_lib.pic_deposit_cvwm_noalloc(loop.handle, C.c_void_p(ps.data_ptr()), C.c_void_p(el.data_ptr()),
                                              C.c_void_p(sp.data_ptr()), w.n, C.c_void_p(out.data_ptr()), None)
        assert rc == 0, gpu_lib.pic_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(ref.shape)
        assert np.all(np.isfinite(got)), call
        assert _rel(got, ref) <= 1e-12, (call, _rel(got, ref))
    assert loop.status()["error_word"] == 0
    loop.close()


def test_noalloc_rejects_meshes_beyond_its_scratch(gpu_lib):
    mesh = build_box_mesh(52, 52, 52, 1)           # 140608 periodic-unique nodes > 131072
    cfg = capi.make_config(1, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64,
                           [(workloads.Q_ELECTRON, workloads.M_ELECTRON, 1.0)], 16)
    loop = ParticleLoop(cfg, mesh)
    import torch
    out = torch.empty(mesh.n_elems * 8 * 4, dtype=torch.float64, device="cuda")
    rc = gpu_lib.pic_deposit_cvwm_noalloc(loop.handle, None, None, None, 0, C.c_void_p(out.data_ptr()), None)
    assert rc == 6                                 # PIC_ERR_CAPACITY
    assert b"131072" in gpu_lib.pic_last_error()
    loop.close()
