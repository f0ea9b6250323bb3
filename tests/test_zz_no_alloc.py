"""The allocation-free CVWM deposition (pic_deposit_cvwm_noalloc) against pic_deposit.

The entry point serves callers that cannot call cudaMalloc during their time loop: they pass
their own device arrays, and the node-sum scratch is a fixed device array inside the library.
These tests play such a caller (its device arrays are made with torch beforehand), call the
entry point through the C-ABI and compare each result with the context's own deposition at the
tolerance the other parity tests use (1e-12 of the maximum: atomic order): twice in a row with
every particle inside; with removed particles (ParticleInside = 0) whose element ids are stale or
out of range; and with out-of-range element and species ids, which are skipped and reported.
"""
import ctypes as C

import numpy as np
import pytest

from piclas_gb300 import ParticleLoop, capi, workloads
from piclas_gb300.mesh import build_box_mesh

pytestmark = pytest.mark.gpu

PIC_STATUS_BAD_ELEMENT = 0x10


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _reference(w, keep):
    """pic_deposit of a context holding only the particles in `keep`."""
    loop = ParticleLoop(w.config(), w.mesh)
    loop.upload_particles(w.part_state[keep], w.elem[keep], w.part_species[keep])
    ref = loop.deposition()
    loop.close()
    return ref


def test_noalloc_deposit_matches_pic_deposit(gpu_lib):
    import torch
    w = workloads.plasma_wave(n_cells=8, N=3, n_particles=30000, seed=21, T_eV=50.0)
    loop = ParticleLoop(w.config(), w.mesh)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    ref = loop.deposition()
    ps = _dev(torch, w.part_state, np.float64)
    el = _dev(torch, w.elem, np.int32)
    sp = _dev(torch, w.part_species, np.int32)
    out = torch.empty(w.mesh.n_elems * w.mesh.n_dof * 4, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        out.fill_(float("nan"))            # the result must be fully written by the call
        torch.cuda.synchronize()
        rc = gpu_lib.pic_deposit_cvwm_noalloc(loop.handle, _ptr(ps), _ptr(el), _ptr(sp), None, w.n, _ptr(out), None)
        assert rc == 0, gpu_lib.pic_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(ref.shape)
        assert np.all(np.isfinite(got)), call
        assert _rel(got, ref) <= 1e-12, (call, _rel(got, ref))
    assert loop.status()["error_word"] == 0
    loop.close()


def test_noalloc_skips_removed_particles(gpu_lib):
    """PDM%ParticleInside = .FALSE. particles are skipped before their element is read: a removed
    particle's GlobalElemID may be stale (a valid but wrong element) or out of range, and neither may
    deposit charge or raise a status bit."""
    import torch
    w = workloads.plasma_wave(n_cells=6, N=2, n_particles=20000, seed=23, T_eV=50.0)
    rng = np.random.default_rng(5)
    inside = (rng.random(w.n) > 0.2).astype(np.uint8)
    elem = w.elem.copy()
    gone = np.nonzero(inside == 0)[0]
    elem[gone[::3]] = 0                                          # out of range
    elem[gone[1::3]] = w.mesh.n_elems + 7                        # out of range
    elem[gone[2::3]] = (elem[gone[2::3]] % w.mesh.n_elems) + 1   # stale: a neighbouring element
    ref = _reference(w, inside == 1)
    loop = ParticleLoop(w.config(), w.mesh)
    ps = _dev(torch, w.part_state, np.float64)
    el = _dev(torch, elem, np.int32)
    sp = _dev(torch, w.part_species, np.int32)
    ins = _dev(torch, inside, np.uint8)
    out = torch.full((w.mesh.n_elems * w.mesh.n_dof * 4,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = gpu_lib.pic_deposit_cvwm_noalloc(loop.handle, _ptr(ps), _ptr(el), _ptr(sp), _ptr(ins), w.n, _ptr(out), None)
    assert rc == 0, gpu_lib.pic_last_error()
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(ref.shape)
    assert _rel(got, ref) <= 1e-12
    assert loop.status()["error_word"] == 0
    loop.close()


def test_noalloc_bad_ids_skipped_and_reported(gpu_lib):
    """Element ids outside 1..nElems and species ids outside 1..nSpecies: the particle is skipped (nothing
    is read out of range) and PIC_STATUS_BAD_ELEMENT is set.  The call runs on a stream of the caller's
    own; pic_get_status is called without synchronising that stream and still sees the bit, because the
    context's stream waits for the call.  The valid particles' charge matches pic_deposit."""
    import torch
    w = workloads.plasma_wave(n_cells=6, N=3, n_particles=20000, seed=29, T_eV=50.0)
    elem = w.elem.copy()
    spec = w.part_species.copy()
    bad = np.zeros(w.n, bool)
    elem[10:20] = 0
    elem[20:30] = w.mesh.n_elems + 1
    spec[30:40] = 0
    spec[40:50] = 2                                              # one species configured
    bad[10:50] = True
    ref = _reference(w, ~bad)
    loop = ParticleLoop(w.config(), w.mesh)
    ps = _dev(torch, w.part_state, np.float64)
    el = _dev(torch, elem, np.int32)
    sp = _dev(torch, spec, np.int32)
    out = torch.empty(w.mesh.n_elems * w.mesh.n_dof * 4, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc = gpu_lib.pic_deposit_cvwm_noalloc(loop.handle, _ptr(ps), _ptr(el), _ptr(sp), None, w.n, _ptr(out),
                                          C.c_void_p(s.cuda_stream))
    assert rc == 0, gpu_lib.pic_last_error()
    st = loop.status()
    assert st["error_word"] & PIC_STATUS_BAD_ELEMENT
    s.synchronize()
    got = out.cpu().numpy().reshape(ref.shape)
    assert _rel(got, ref) <= 1e-12
    loop.reset_status()
    assert loop.status()["error_word"] == 0
    loop.close()


def test_noalloc_rejects_meshes_beyond_its_scratch(gpu_lib):
    mesh = build_box_mesh(52, 52, 52, 1)           # 140608 periodic-unique nodes > 131072
    cfg = capi.make_config(1, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64,
                           [(workloads.Q_ELECTRON, workloads.M_ELECTRON, 1.0)], 16)
    loop = ParticleLoop(cfg, mesh)
    import torch
    out = torch.empty(mesh.n_elems * 8 * 4, dtype=torch.float64, device="cuda")
    rc = gpu_lib.pic_deposit_cvwm_noalloc(loop.handle, None, None, None, None, 0, C.c_void_p(out.data_ptr()), None)
    assert rc == 6                                 # PIC_ERR_CAPACITY
    assert b"131072" in gpu_lib.pic_last_error()
    loop.close()
