"""piclas_gb300 -- GB300-native (sm_103a) PIC particle loop of PICLas behind a C-ABI.

Host-side mirror of the reference's Boris-Leapfrog particle loop
(src/timedisc/timedisc_TimeStepPoissonByBorisLeapfrog.f90).  The method names follow the
reference routines the C-ABI replaces:

    ParticleLoop.interpolate_field_to_particle()   InterpolateFieldToParticle
    ParticleLoop.push(dt)                          Boris push loop (+ LastPartPos save)
    ParticleLoop.perform_tracking()                PerformTracking
    ParticleLoop.deposition()                      Deposition
    ParticleLoop.time_step(dt, n)                  TimeStepPoissonByBorisLeapfrog, field frozen

Every call goes through ``libpiclas_gpu.so``; there is no CPU fallback.  A non-zero return
code raises :class:`PicError` carrying the library's message (where the reference would
``abort``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import capi
from .capi import (PIC_DEPO_CVWM, PIC_DEPO_SHAPE_FUNCTION, PIC_DEPO_SHAPE_FUNCTION_CC, PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE, PIC_PREC_FP64, PIC_PREC_MIXED, PIC_TRACK_REFMAPPING,
                   PIC_TRACK_TRIA, MeshStruct, PicConfig, PicMesh, PicStatus, make_config)

__all__ = ["ParticleLoop", "PicError", "load_library", "library_path", "MeshStruct", "make_config",
           "PIC_TRACK_TRIA", "PIC_TRACK_REFMAPPING", "PIC_DEPO_CVWM", "PIC_DEPO_SHAPE_FUNCTION", "PIC_DEPO_SHAPE_FUNCTION_CC", "PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE",
           "PIC_PREC_FP64", "PIC_PREC_MIXED", "EXPORTED_SYMBOLS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

EXPORTED_SYMBOLS = ["pic_version", "pic_last_error", "pic_create", "pic_destroy", "pic_set_field",
                    "pic_upload_particles", "pic_download_particles", "pic_interpolate", "pic_push", "pic_track",
                    "pic_deposit", "pic_get_field_at_particles", "pic_step", "pic_get_status", "pic_reset_status",
                    "pic_synchronize", "pic_launch_count", "pic_stream", "pic_profile", "pic_profile_read",
                    "pic_deposit_cvwm_noalloc", "pic_adjoint_run", "pic_get_part_data", "pic_set_part_data", "pic_fp64_fma_rate",
                    "pic_hdg_init", "pic_hdg_set_dirichlet", "pic_hdg_solve", "pic_hdg_get_lambda",
                    "pic_hdg_get_elem_mat", "pic_hdg_set_lambda", "pic_verify_deposited_charge",
                    "pic_fp32_fma_rate"]


class PicError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where}: {capi.ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


def library_path() -> str:
    return os.path.join(_HERE, "_lib", "libpiclas_gpu.so")


def load_library(build_if_missing: bool = False):
    """Load libpiclas_gpu.so (built by ``piclas_gb300.build``)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            from .build import build
            build()
        else:
            raise RuntimeError(f"{path} missing: run `python -m piclas_gb300.build` (no CPU fallback exists)")
    L = C.CDLL(path)
    P = C.POINTER
    dp, ip, u8p = P(C.c_double), P(C.c_int32), P(C.c_uint8)
    L.pic_version.restype = C.c_char_p
    L.pic_last_error.restype = C.c_char_p
    L.pic_create.argtypes = [P(PicConfig), P(PicMesh), P(C.c_void_p)]
    L.pic_destroy.argtypes = [C.c_void_p]
    L.pic_destroy.restype = None
    L.pic_set_field.argtypes = [C.c_void_p, dp, C.c_int32]
    L.pic_upload_particles.argtypes = [C.c_void_p, dp, ip, ip, u8p, u8p, C.c_int32]
    L.pic_download_particles.argtypes = [C.c_void_p, dp, ip, u8p, u8p, dp, C.c_int32]
    L.pic_interpolate.argtypes = [C.c_void_p]
    L.pic_push.argtypes = [C.c_void_p, C.c_double]
    L.pic_track.argtypes = [C.c_void_p]
    L.pic_deposit.argtypes = [C.c_void_p, dp]
    L.pic_get_field_at_particles.argtypes = [C.c_void_p, dp, C.c_int32]
    i64p = P(C.c_int64)
    L.pic_get_part_data.argtypes = [C.c_void_p, dp, i64p, C.c_int64, C.c_int32, P(C.c_int32)]
    L.pic_set_part_data.argtypes = [C.c_void_p, dp, i64p, C.c_int64, C.c_int32]
    L.pic_fp64_fma_rate.argtypes = [C.c_void_p, dp]
    L.pic_fp32_fma_rate.argtypes = [C.c_void_p, dp]
    L.pic_step.argtypes = [C.c_void_p, C.c_double, C.c_int32, dp]
    L.pic_get_status.argtypes = [C.c_void_p, P(PicStatus)]
    L.pic_reset_status.argtypes = [C.c_void_p]
    L.pic_synchronize.argtypes = [C.c_void_p]
    L.pic_launch_count.argtypes = [C.c_void_p]
    L.pic_launch_count.restype = C.c_int64
    L.pic_profile.argtypes = [C.c_void_p, C.c_int32]
    L.pic_profile_read.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int64), C.c_int32]
    L.pic_deposit_cvwm_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                           C.c_void_p, C.c_void_p]
    L.pic_adjoint_run.argtypes = [C.c_void_p, P(capi.PicAdjointConfig), dp, dp, dp, dp]
    L.pic_verify_deposited_charge.argtypes = [C.c_void_p, dp, dp]
    L.pic_stream.argtypes = [C.c_void_p]
    L.pic_stream.restype = C.c_void_p
    L.pic_hdg_init.argtypes = [C.c_void_p, P(capi.PicHdg)]
    L.pic_hdg_set_dirichlet.argtypes = [C.c_void_p, dp]
    L.pic_hdg_solve.argtypes = [C.c_void_p, dp, dp, dp, P(capi.PicHdgStatus)]
    L.pic_hdg_get_lambda.argtypes = [C.c_void_p, dp]
    L.pic_hdg_set_lambda.argtypes = [C.c_void_p, dp]
    L.pic_hdg_get_elem_mat.argtypes = [C.c_void_p, C.c_int32, dp, dp, dp]
    _LIB = L
    return L


def _null(t):
    return C.POINTER(t)()


class ParticleLoop:
    """One GPU context of the particle loop (one mesh, one particle population)."""

    def __init__(self, cfg: PicConfig, mesh, lib=None):
        self.lib = lib or load_library()
        self.cfg = cfg
        self.mesh_struct = mesh if isinstance(mesh, MeshStruct) else MeshStruct(mesh)
        self.mesh = self.mesh_struct.mesh
        self.N = cfg.n_dg
        self.nd = (self.N + 1) ** 3
        self.n = 0
        h = C.c_void_p()
        self._check(self.lib.pic_create(C.byref(cfg), self.mesh_struct.ptr, C.byref(h)), "pic_create")
        self.handle = h

    def _check(self, rc: int, where: str):
        if rc != 0:
            msg = self.lib.pic_last_error().decode(errors="replace")
            raise PicError(rc, where, msg)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pic_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state hand-over -------------------------------------------------------------------
    def set_field(self, e_dof: np.ndarray):
        """U_N(e)%E(1:3,0:Nloc,0:Nloc,0:Nloc) for all elements: array (nElems, (N+1)^3, 3), or on a p-adapted
        mesh packed (nDofs, 3) (mesh.dof_shape(3))."""
        e = np.ascontiguousarray(e_dof, dtype=np.float64)
        if e.size != self.mesh.n_dofs * 3:
            raise ValueError("field has the wrong size")
        self._check(self.lib.pic_set_field(self.handle, capi.dptr(e), self.mesh.n_elems), "pic_set_field")

    def upload_particles(self, part_state, elem, species, inside=None, is_new=None):
        ps = np.ascontiguousarray(part_state, dtype=np.float64)
        n = ps.shape[0]
        el = np.ascontiguousarray(elem, dtype=np.int32)
        sp = np.ascontiguousarray(species, dtype=np.int32)
        ins = np.ones(n, np.uint8) if inside is None else np.ascontiguousarray(inside, np.uint8)
        new = np.ones(n, np.uint8) if is_new is None else np.ascontiguousarray(is_new, np.uint8)
        self._check(self.lib.pic_upload_particles(self.handle, capi.dptr(ps), capi.iptr(el), capi.iptr(sp),
                                                  capi.u8ptr(ins), capi.u8ptr(new), n), "pic_upload_particles")
        self.n = n

    def download_particles(self, with_ref: bool = False):
        n = self.n
        ps = np.zeros((n, 6))
        el = np.zeros(n, np.int32)
        ins = np.zeros(n, np.uint8)
        new = np.zeros(n, np.uint8)
        ref = np.zeros((n, 3)) if with_ref else None
        self._check(self.lib.pic_download_particles(self.handle, capi.dptr(ps), capi.iptr(el), capi.u8ptr(ins),
                                                    capi.u8ptr(new), capi.dptr(ref) if with_ref else _null(C.c_double),
                                                    n), "pic_download_particles")
        out = dict(part_state=ps, elem=el, inside=ins, is_new=new)
        if with_ref:
            out["part_pos_ref"] = ref
        return out

    # -- loop pieces ------------------------------------------------------------------------
    def interpolate_field_to_particle(self):
        self._check(self.lib.pic_interpolate(self.handle), "pic_interpolate")

    def push(self, dt: float):
        self._check(self.lib.pic_push(self.handle, dt), "pic_push")

    def perform_tracking(self):
        self._check(self.lib.pic_track(self.handle), "pic_track")

    def deposition(self, out: np.ndarray | None = None, copy: bool = True):
        """PS_N(e)%PartSource(1:4,...) for all elements as (nElems, (N+1)^3, 4), or on a p-adapted mesh packed
        (nDofs, 4) (mesh.dof_shape(4))."""
        if not copy:
            self._check(self.lib.pic_deposit(self.handle, _null(C.c_double)), "pic_deposit")
            return None
        ps = out if out is not None else np.zeros(self.mesh.dof_shape(4))
        self._check(self.lib.pic_deposit(self.handle, capi.dptr(ps)), "pic_deposit")
        return ps

    def fp64_fma_rate(self) -> float:
        """Sustained FP64 FMA rate of the GPU (GFLOP/s), measured by the library."""
        r = C.c_double(0.0)
        self._check(self.lib.pic_fp64_fma_rate(self.handle, C.byref(r)), "pic_fp64_fma_rate")
        return r.value

    def fp32_fma_rate(self) -> float:
        """Sustained FP32 FMA rate of the GPU (GFLOP/s), measured by the library."""
        r = C.c_double(0.0)
        self._check(self.lib.pic_fp32_fma_rate(self.handle, C.byref(r)), "pic_fp32_fma_rate")
        return r.value

    def get_part_data(self, offset_npart: int = 0):
        """Checkpoint layout of the reference (FillParticleData): PartData (n, 7) = x, y, z, vx, vy, vz, species
        of the particles inside, grouped by element; PartInt (nElems, 2) = (FirstPartID, LastPartID)."""
        ne = self.mesh.n_elems
        part_int = np.zeros((ne, 2), np.int64)
        n = C.c_int32(0)
        i64 = part_int.ctypes.data_as(C.POINTER(C.c_int64))
        self._check(self.lib.pic_get_part_data(self.handle, _null(C.c_double), i64, offset_npart, 0, C.byref(n)),
                    "pic_get_part_data")
        part_data = np.zeros((n.value, 7))
        self._check(self.lib.pic_get_part_data(self.handle, capi.dptr(part_data), i64, offset_npart, n.value,
                                               C.byref(n)), "pic_get_part_data")
        return part_data, part_int

    def set_part_data(self, part_data: np.ndarray, part_int: np.ndarray, offset_npart: int = 0):
        """Restart from the checkpoint layout: IsNewPart = F; the caller order becomes the PartData order."""
        pd = np.ascontiguousarray(part_data, dtype=np.float64)
        pi = np.ascontiguousarray(part_int, dtype=np.int64)
        self._check(self.lib.pic_set_part_data(self.handle, capi.dptr(pd), pi.ctypes.data_as(C.POINTER(C.c_int64)),
                                               offset_npart, pd.shape[0]), "pic_set_part_data")
        self.n = pd.shape[0]

    def field_at_particles(self) -> np.ndarray:
        f = np.zeros((self.n, 6))
        self._check(self.lib.pic_get_field_at_particles(self.handle, capi.dptr(f), self.n), "pic_get_field_at_particles")
        return f

    def time_step(self, dt: float, nsteps: int = 1, part_source: np.ndarray | None = None):
        ptr = capi.dptr(part_source) if part_source is not None else _null(C.c_double)
        self._check(self.lib.pic_step(self.handle, dt, nsteps, ptr), "pic_step")
        return part_source

    def status(self) -> dict:
        s = PicStatus()
        self._check(self.lib.pic_get_status(self.handle, C.byref(s)), "pic_get_status")
        return dict(error_word=int(s.error_word), n_lost=int(s.n_lost), n_inside=int(s.n_inside),
                    n_newton_failed=int(s.n_newton_failed), n_steps=int(s.n_steps))

    def verify_deposited_charge(self) -> tuple[float, float]:
        """VerifyDepositedCharge of the last deposition: (ChargeNumerical, ChargeAnalytical) in C."""
        num, ana = C.c_double(0.0), C.c_double(0.0)
        self._check(self.lib.pic_verify_deposited_charge(self.handle, C.byref(num), C.byref(ana)),
                    "pic_verify_deposited_charge")
        return num.value, ana.value

    def reset_status(self):
        self._check(self.lib.pic_reset_status(self.handle), "pic_reset_status")

    def synchronize(self):
        self._check(self.lib.pic_synchronize(self.handle), "pic_synchronize")

    def adjoint(self, nsteps: int, dt: float, rho_target: np.ndarray, rho_scale: float, b_scale: float = 1.0,
                checkpoint_every: int = 10, precision: int = PIC_PREC_FP64, gradients: bool = True):
        """Loss of the differentiable loop and (optionally) dL/dv0 (n,3) and dL/d|B|."""
        a = capi.PicAdjointConfig(nsteps, checkpoint_every, precision, dt, rho_scale, b_scale)
        tgt = np.ascontiguousarray(rho_target, dtype=np.float64)
        if tgt.size != self.mesh.n_elems * self.nd:
            raise ValueError("rho_target has the wrong size")
        loss = C.c_double(0.0)
        gv = np.zeros((self.n, 3)) if gradients else None
        gb = C.c_double(0.0)
        self._check(self.lib.pic_adjoint_run(self.handle, C.byref(a), capi.dptr(tgt), C.byref(loss),
                                             capi.dptr(gv) if gradients else _null(C.c_double),
                                             C.byref(gb) if gradients else _null(C.c_double)), "pic_adjoint_run")
        return (loss.value, gv, gb.value) if gradients else loss.value

    PHASES = ("deposit_main", "sort_pack", "particle_update", "node_to_dof", "reorder", "cvwm_deposit", "hdg")

    def profile(self, enable: bool):
        self._check(self.lib.pic_profile(self.handle, 1 if enable else 0), "pic_profile")

    def profile_read(self) -> dict:
        n = len(self.PHASES)
        ms = (C.c_double * n)()
        ln = (C.c_int64 * n)()
        self._check(self.lib.pic_profile_read(self.handle, ms, ln, n), "pic_profile_read")
        return {name: dict(ms=float(ms[i]), launches=int(ln[i])) for i, name in enumerate(self.PHASES)}

    # -- HDG Poisson solve --------------------------------------------------------------------
    def hdg_init(self, hmesh, precond_type: int = 2, eps_cg: float = 1e-6, max_iter_cg: int = 500,
                 relative: bool = False, solve_in_step: bool = False, cg_kernel: int = 0):
        """InitHDG/Elem_Mat/BuildPrecond from a :class:`piclas_gb300.hdg_mesh.HdgMesh`."""
        self._hdg_keep = [np.ascontiguousarray(hmesh.elem_to_side, dtype=np.int32),
                          np.ascontiguousarray(hmesh.side_to_elem, dtype=np.int32),
                          np.ascontiguousarray(hmesh.metrics_f, dtype=np.float64),
                          np.ascontiguousarray(hmesh.metrics_g, dtype=np.float64),
                          np.ascontiguousarray(hmesh.metrics_h, dtype=np.float64),
                          np.ascontiguousarray(hmesh.sj, dtype=np.float64),
                          np.ascontiguousarray(hmesh.dirichlet_sides, dtype=np.int32)]
        e2s, s2e, mf, mg, mh, sj, ds = self._hdg_keep
        h = capi.PicHdg(hmesh.n_sides, capi.iptr(e2s), capi.iptr(s2e), capi.dptr(mf), capi.dptr(mg), capi.dptr(mh),
                        capi.dptr(sj), len(ds), capi.iptr(ds) if len(ds) else _null(C.c_int32), int(precond_type),
                        int(max_iter_cg), float(eps_cg), int(bool(relative)), int(bool(solve_in_step)),
                        int(cg_kernel))
        self._check(self.lib.pic_hdg_init(self.handle, C.byref(h)), "pic_hdg_init")
        self.hdg_n_sides = hmesh.n_sides
        self.hdg_n_dirichlet = len(ds)

    def hdg_set_dirichlet(self, lambda_bc: np.ndarray):
        lb = np.ascontiguousarray(lambda_bc, dtype=np.float64)
        self._check(self.lib.pic_hdg_set_dirichlet(self.handle, capi.dptr(lb)), "pic_hdg_set_dirichlet")

    def hdg_solve(self, source: np.ndarray | None = None, want_phi: bool = True, want_e: bool = True):
        """One HDGLinear solve; source = CalcSourceHDG values (nElems, (N+1)^3) or None for the deposited
        charge.  Returns (phi (nElems,(N+1)^3) | None, E (nElems,(N+1)^3,3) | None, status dict)."""
        src = None if source is None else np.ascontiguousarray(source, dtype=np.float64)
        phi = np.zeros((self.mesh.n_elems, self.nd)) if want_phi else None
        E = np.zeros((self.mesh.n_elems, self.nd, 3)) if want_e else None
        st = capi.PicHdgStatus()
        self._check(self.lib.pic_hdg_solve(self.handle, capi.dptr(src) if src is not None else _null(C.c_double),
                                           capi.dptr(phi) if phi is not None else _null(C.c_double),
                                           capi.dptr(E) if E is not None else _null(C.c_double), C.byref(st)),
                    "pic_hdg_solve")
        return phi, E, dict(iterations=st.iterations, converged=st.converged, norm_r=st.norm_r, n_solves=st.n_solves)

    def hdg_lambda(self) -> np.ndarray:
        nf = (self.N + 1) ** 2
        lam = np.zeros((self.hdg_n_sides, nf))
        self._check(self.lib.pic_hdg_get_lambda(self.handle, capi.dptr(lam)), "pic_hdg_get_lambda")
        return lam

    def hdg_set_lambda(self, lam: np.ndarray):
        lm = np.ascontiguousarray(lam, dtype=np.float64)
        if lm.size != self.hdg_n_sides * (self.N + 1) ** 2:
            raise ValueError("lambda has the wrong size")
        self._check(self.lib.pic_hdg_set_lambda(self.handle, capi.dptr(lm)), "pic_hdg_set_lambda")

    def hdg_elem_mat(self, elem: int):
        """(Ehat (6,nv,nf), InvDhat (nv,nv), Smat (6,6,nf,nf)) of 1-based element ``elem`` (C views of the
        reference's Fortran arrays)."""
        nv, nf = self.nd, (self.N + 1) ** 2
        eh = np.zeros((6, nv, nf))
        di = np.zeros((nv, nv))
        sm = np.zeros((6, 6, nf, nf))
        self._check(self.lib.pic_hdg_get_elem_mat(self.handle, int(elem), capi.dptr(eh), capi.dptr(di), capi.dptr(sm)),
                    "pic_hdg_get_elem_mat")
        return eh, di, sm

    def set_field_ptr(self, ptr: int):
        """Field from a host pointer (e.g. pinned memory)."""
        self._check(self.lib.pic_set_field(self.handle, C.cast(ptr, C.POINTER(C.c_double)), self.mesh.n_elems),
                    "pic_set_field")

    def time_step_ptr(self, dt: float, nsteps: int, part_source_ptr: int):
        self._check(self.lib.pic_step(self.handle, dt, nsteps, C.cast(part_source_ptr, C.POINTER(C.c_double))),
                    "pic_step")

    @property
    def launch_count(self) -> int:
        return int(self.lib.pic_launch_count(self.handle))

    @property
    def stream_ptr(self) -> int:
        return int(self.lib.pic_stream(self.handle) or 0)
