"""ctypes wrapper of the CPU oracle (oracle/pic_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py as the checker.  The piclas_gb300 package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from piclas_gb300.capi import PicConfig, PicMesh, dptr, iptr, u8ptr

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpic_oracle.so")
_TIMING_PATH = os.path.join(_HERE, "_build", "libpic_oracle_timing.so")
_libs = {}
_timing = False


def set_timing_build(flag: bool) -> None:
    """Route the wrappers below to the timing build (-O3, FMA contraction: the reference's release flags)
    instead of the checker build.  Only the CPU-baseline leg of the benchmark uses it."""
    global _timing
    _timing = bool(flag)


class OrcParticles(C.Structure):
    _fields_ = [("n", C.c_int32), ("part_state", C.POINTER(C.c_double)), ("last_part_pos", C.POINTER(C.c_double)),
                ("part_pos_ref", C.POINTER(C.c_double)), ("field", C.POINTER(C.c_double)),
                ("elem", C.POINTER(C.c_int32)), ("last_elem", C.POINTER(C.c_int32)),
                ("species", C.POINTER(C.c_int32)), ("inside", C.POINTER(C.c_uint8)),
                ("is_new", C.POINTER(C.c_uint8))]


class OrcCounters(C.Structure):
    _fields_ = [("n_lost", C.c_int64), ("n_newton_failed", C.c_int64), ("n_ref_tolerance", C.c_int64),
                ("n_hop_limit", C.c_int64)]


class OrcHdgMesh(C.Structure):
    _fields_ = [("N", C.c_int), ("ne", C.c_int), ("n_sides", C.c_int), ("e2s", C.POINTER(C.c_int32)),
                ("s2e", C.POINTER(C.c_int32)), ("mf", C.POINTER(C.c_double)), ("mg", C.POINTER(C.c_double)),
                ("mh", C.POINTER(C.c_double)), ("sj", C.POINTER(C.c_double)), ("xgp", C.POINTER(C.c_double)),
                ("wgp", C.POINTER(C.c_double)), ("n_dir", C.c_int), ("dir_sides", C.POINTER(C.c_int32))]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc): the checker (-ffp-contract=off) and the timing build."""
    srcs = [os.path.join(_HERE, f) for f in ("pic_oracle.c", "pic_oracle_hdg.c", "pic_oracle.h", "Makefile")]
    newest = max(map(os.path.getmtime, srcs))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < newest for p in (_LIB_PATH, _TIMING_PATH)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    path = _TIMING_PATH if _timing else _LIB_PATH
    if path not in _libs:
        build()
        L = C.CDLL(path)
        P = C.POINTER
        L.orc_step.argtypes = [P(PicConfig), P(PicMesh), P(C.c_double), P(OrcParticles), C.c_double, C.c_int,
                               P(C.c_double), P(OrcCounters), C.c_int]
        L.orc_deposit.argtypes = [P(PicConfig), P(PicMesh), P(OrcParticles), P(C.c_double), P(OrcCounters), C.c_int]
        L.orc_interpolate.argtypes = [P(PicConfig), P(PicMesh), P(C.c_double), P(OrcParticles), P(OrcCounters),
                                      C.c_int]
        L.orc_push.argtypes = [P(PicConfig), P(OrcParticles), C.c_double, C.c_int]
        L.orc_track.argtypes = [P(PicConfig), P(PicMesh), P(OrcParticles), P(OrcCounters), C.c_int]
        L.orc_map_particles.argtypes = [P(PicConfig), P(PicMesh), P(OrcParticles), C.c_int]
        L.orc_integrate_charge.argtypes = [P(PicMesh), C.c_int, P(C.c_double)]
        L.orc_integrate_charge.restype = C.c_double
        L.orc_lagrange_polys.argtypes = [C.c_double, C.c_int, P(C.c_double), P(C.c_double), P(C.c_double)]
        L.orc_get_position_in_ref_elem.argtypes = [P(PicConfig), P(PicMesh), P(C.c_double), P(C.c_double), C.c_int,
                                                   C.c_int]
        L.orc_max_threads.restype = C.c_int
        L.orc_hdg_elem_mat.argtypes = [P(OrcHdgMesh), P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double)]
        L.orc_hdg_solve.argtypes = [P(OrcHdgMesh), P(C.c_double), P(C.c_double), P(C.c_double), C.c_int, C.c_double,
                                    C.c_int, C.c_int, P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                                    P(C.c_double), P(C.c_int), P(C.c_double)]
        _libs[path] = L
    return _libs[path]


class OracleState:
    """Particle arrays in the reference layout plus the oracle's counters."""

    def __init__(self, part_state, elem, species, inside=None, is_new=None, part_pos_ref=None):
        n = part_state.shape[0]
        self.n = n
        self.part_state = np.ascontiguousarray(part_state, dtype=np.float64).copy()     # (n,6) = PartState(1:6,n)
        self.last_part_pos = np.zeros((n, 3))
        self.part_pos_ref = (np.zeros((n, 3)) if part_pos_ref is None
                             else np.ascontiguousarray(part_pos_ref, dtype=np.float64).copy())
        self.field = np.zeros((n, 6))
        self.elem = np.ascontiguousarray(elem, dtype=np.int32).copy()
        self.last_elem = self.elem.copy()
        self.species = np.ascontiguousarray(species, dtype=np.int32).copy()
        self.inside = (np.ones(n, np.uint8) if inside is None else np.ascontiguousarray(inside, np.uint8).copy())
        self.is_new = (np.ones(n, np.uint8) if is_new is None else np.ascontiguousarray(is_new, np.uint8).copy())
        self.counters = OrcCounters()
        self._s = OrcParticles(n, dptr(self.part_state), dptr(self.last_part_pos), dptr(self.part_pos_ref),
                               dptr(self.field), iptr(self.elem), iptr(self.last_elem), iptr(self.species),
                               u8ptr(self.inside), u8ptr(self.is_new))

    @property
    def ptr(self):
        return C.byref(self._s)


def map_particles(cfg, mesh_struct, st: OracleState, nthreads: int = 1):
    lib().orc_map_particles(C.byref(cfg), mesh_struct.ptr, st.ptr, nthreads)


def step(cfg, mesh_struct, e_dof, st: OracleState, dt, nsteps, part_source=None, nthreads: int = 1):
    e_dof = np.ascontiguousarray(e_dof, dtype=np.float64)
    ps = dptr(part_source) if part_source is not None else C.POINTER(C.c_double)()
    rc = lib().orc_step(C.byref(cfg), mesh_struct.ptr, dptr(e_dof), st.ptr, dt, nsteps, ps,
                        C.byref(st.counters), nthreads)
    if rc:
        raise RuntimeError(f"orc_step failed: {rc}")


def deposit(cfg, mesh_struct, st: OracleState, part_source, nthreads: int = 1):
    rc = lib().orc_deposit(C.byref(cfg), mesh_struct.ptr, st.ptr, dptr(part_source), C.byref(st.counters), nthreads)
    if rc:
        raise RuntimeError(f"orc_deposit failed: {rc}")


def interpolate(cfg, mesh_struct, e_dof, st: OracleState, nthreads: int = 1):
    lib().orc_interpolate(C.byref(cfg), mesh_struct.ptr, dptr(np.ascontiguousarray(e_dof)), st.ptr,
                          C.byref(st.counters), nthreads)


def push(cfg, st: OracleState, dt, nthreads: int = 1):
    lib().orc_push(C.byref(cfg), st.ptr, dt, nthreads)


def save_last(st: OracleState):
    st.last_part_pos[:] = st.part_state[:, :3]
    st.last_elem[:] = st.elem


def track(cfg, mesh_struct, st: OracleState, nthreads: int = 1):
    lib().orc_track(C.byref(cfg), mesh_struct.ptr, st.ptr, C.byref(st.counters), nthreads)


def integrate_charge(mesh_struct, N, part_source) -> float:
    return float(lib().orc_integrate_charge(mesh_struct.ptr, N, dptr(np.ascontiguousarray(part_source))))


def lagrange_polys(x, xgp, wbary):
    xgp = np.ascontiguousarray(xgp, dtype=np.float64)
    wb = np.ascontiguousarray(wbary, dtype=np.float64)
    L = np.zeros(len(xgp))
    lib().orc_lagrange_polys(float(x), len(xgp) - 1, dptr(xgp), dptr(wb), dptr(L))
    return L


# ---- HDG Poisson solve ----------------------------------------------------------------------------
class HdgOracle:
    """Elem_Mat + HDGLinear of the oracle for one (BoxMesh, HdgMesh) pair."""

    def __init__(self, mesh, hmesh):
        self._keep = [np.ascontiguousarray(a) for a in (hmesh.elem_to_side.astype(np.int32),
                                                        hmesh.side_to_elem.astype(np.int32),
                                                        hmesh.metrics_f, hmesh.metrics_g, hmesh.metrics_h,
                                                        hmesh.sj, mesh.xgp, mesh.wgp,
                                                        np.asarray(hmesh.dirichlet_sides, np.int32))]
        e2s, s2e, mf, mg, mh, sj, xg, wg, ds = self._keep
        self.N, self.ne, self.n_sides = mesh.N, mesh.n_elems, hmesh.n_sides
        self.nd = mesh.N + 1
        self.nv, self.nf = self.nd ** 3, self.nd ** 2
        self.n_dir = len(ds)
        self.s = OrcHdgMesh(self.N, self.ne, self.n_sides, iptr(e2s), iptr(s2e), dptr(mf), dptr(mg), dptr(mh),
                            dptr(sj), dptr(xg), dptr(wg), self.n_dir, iptr(ds) if self.n_dir else C.POINTER(C.c_int32)())
        self.ehat = np.zeros((self.ne, 6, self.nv, self.nf))      # Ehat(nf,nv,6) per element
        self.inv_dhat = np.zeros((self.ne, self.nv, self.nv))
        self.smat = np.zeros((self.ne, 6, 6, self.nf, self.nf))   # Smat(nf,nf,6,6) -> [jS][iS][b][a]
        self.tau = np.zeros(self.ne)
        rc = lib().orc_hdg_elem_mat(C.byref(self.s), dptr(self.ehat), dptr(self.inv_dhat), dptr(self.smat),
                                    dptr(self.tau))
        if rc:
            raise RuntimeError(f"orc_hdg_elem_mat failed: {rc}")
        self.lam = np.zeros((self.n_sides, self.nf))

    def solve(self, resu, precond_type=0, eps_cg=1e-10, max_iter=10000, relative=False, lambda_dirichlet=None):
        """resu: CalcSourceHDG at the volume points, C [e][k][j][i].  Returns (phi, E, iterations, norm, rc)."""
        resu = np.ascontiguousarray(resu, dtype=np.float64).reshape(self.ne, self.nv)
        ld = (np.ascontiguousarray(lambda_dirichlet, dtype=np.float64) if lambda_dirichlet is not None
              else None)
        U = np.zeros((self.ne, self.nv))
        E = np.zeros((self.ne, self.nv, 3))
        it = C.c_int(0)
        nrm = C.c_double(0.0)
        rc = lib().orc_hdg_solve(C.byref(self.s), dptr(self.ehat), dptr(self.inv_dhat), dptr(self.smat),
                                 int(precond_type), float(eps_cg), int(max_iter), int(bool(relative)), dptr(resu),
                                 dptr(ld) if ld is not None else C.POINTER(C.c_double)(), dptr(self.lam),
                                 dptr(U), dptr(E), C.byref(it), C.byref(nrm))
        if rc > 0:
            raise RuntimeError(f"orc_hdg_solve failed: {rc}")
        return U, E, it.value, nrm.value, rc
