"""ctypes mirror of include/piclas_gpu.h.

The structures here are byte-for-byte the C-ABI structs; ``make_mesh_struct`` fills a
``PicMesh`` from a :class:`piclas_gb300.mesh.BoxMesh` (the arrays are already in the
reference's Fortran memory order) and keeps the numpy buffers alive alongside it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PIC_MAX_SPECIES = 8

PIC_TRACK_TRIA = 1
PIC_TRACK_REFMAPPING = 2
PIC_DEPO_CVWM = 1
PIC_DEPO_SHAPE_FUNCTION = 2
PIC_DEPO_SHAPE_FUNCTION_CC = 3
PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE = 4
PIC_PREC_FP64 = 0
PIC_PREC_MIXED = 1

PIC_STATUS_LOST_PARTICLE = 0x01
PIC_STATUS_NEWTON_FAILED = 0x02
PIC_STATUS_HOP_LIMIT = 0x04
PIC_STATUS_REF_TOLERANCE = 0x08
PIC_STATUS_BAD_ELEMENT = 0x10
PIC_STATUS_NOT_FINITE = 0x20
PIC_STATUS_CG_NOT_CONVERGED = 0x40
PIC_STATUS_CG_BREAKDOWN = 0x80
PIC_STATUS_WAIT_TIMEOUT = 0x100

ERROR_NAMES = {0: "PIC_OK", 1: "PIC_ERR_INVALID_ARGUMENT", 2: "PIC_ERR_CUDA", 3: "PIC_ERR_OUT_OF_MEMORY",
               4: "PIC_ERR_NO_DEVICE", 5: "PIC_ERR_STATE", 6: "PIC_ERR_CAPACITY"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class PicConfig(C.Structure):
    _fields_ = [
        ("n_dg", C.c_int32), ("tracking", C.c_int32), ("deposition", C.c_int32), ("precision", C.c_int32),
        ("max_particles", C.c_int32), ("n_species", C.c_int32),
        ("charge", C.c_double * PIC_MAX_SPECIES), ("mass", C.c_double * PIC_MAX_SPECIES),
        ("mpf", C.c_double * PIC_MAX_SPECIES), ("external_field", C.c_double * 6),
        ("refmapping_eps", C.c_double), ("sf_radius", C.c_double), ("sf_alpha", C.c_int32),
        ("sort_interval", C.c_int32), ("sf_dim", C.c_int32), ("sf_dir", C.c_int32), ("sf_depo3d", C.c_int32),
        ("time_step_factor", C.c_double * PIC_MAX_SPECIES),
        ("periodic_tracing", C.c_int32), ("ref_mapping_guess", C.c_int32),
    ]


class PicMesh(C.Structure):
    _fields_ = [
        ("n_elems", C.c_int32), ("n_geo", C.c_int32), ("n_nodes", C.c_int32), ("n_periodic_vectors", C.c_int32),
        ("periodic_vectors", C.c_double * 9), ("xmin_glob", C.c_double * 3), ("xmax_glob", C.c_double * 3),
        ("xi_cl_ngeo", _dp), ("wbary_cl_ngeo", _dp), ("xgp", _dp), ("wgp", _dp), ("wbary_gp", _dp),
        ("xcl_ngeo", _dp), ("dxcl_ngeo", _dp), ("elem_bary", _dp), ("xez_basis", _dp), ("slen_basis", _dp),
        ("elem_radius", _dp), ("eps_one_cell", _dp), ("elem_xgp", _dp), ("elem_sj", _dp),
        ("node_coords", _dp), ("elem_node", _ip), ("elem_side_node", _ip), ("side_nb_elem", _ip),
        ("side_pvid", _ip), ("concave_side", _ip),
        ("node_info", _ip), ("node_volume", _dp), ("periodic_n_nodes", _ip), ("periodic_offset", _ip),
        ("periodic_nodes", _ip), ("n_total_periodic_nodes", C.c_int32),
        ("fibgm_imax", C.c_int32 * 3), ("fibgm_deltas", C.c_double * 3), ("fibgm_n_elems", _ip),
        ("fibgm_offset", _ip), ("fibgm_element", _ip), ("fibgm_n_total", C.c_int32),
        ("side_bc", _ip), ("sf_elem_radius", _dp),
        ("n_bc_entries", C.c_int32), ("elem_to_bc_sides", _ip), ("bc_side_elem_loc", _ip), ("bc_side_distance", _dp),
        ("n_dg_mapping", _ip), ("n_inter", _dp), ("elem_curved", _ip), ("side_bezier", _dp), ("side_type", _ip),
    ]


class PicAdjointConfig(C.Structure):
    _fields_ = [("nsteps", C.c_int32), ("checkpoint_every", C.c_int32), ("precision", C.c_int32),
                ("dt", C.c_double), ("rho_scale", C.c_double), ("b_scale", C.c_double)]


class PicHdg(C.Structure):
    _fields_ = [("n_sides", C.c_int32), ("elem_to_side", _ip), ("side_to_elem", _ip), ("metrics_f", _dp),
                ("metrics_g", _dp), ("metrics_h", _dp), ("sj", _dp), ("n_dirichlet", C.c_int32),
                ("dirichlet_sides", _ip), ("precond_type", C.c_int32), ("max_iter_cg", C.c_int32),
                ("eps_cg", C.c_double), ("use_relative_abort", C.c_int32), ("solve_in_step", C.c_int32),
                ("cg_kernel", C.c_int32)]


class PicHdgStatus(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("norm_r", C.c_double),
                ("n_solves", C.c_int64)]


class PicStatus(C.Structure):
    _fields_ = [("error_word", C.c_uint32), ("n_lost", C.c_int32), ("n_inside", C.c_int32),
                ("n_newton_failed", C.c_int32), ("n_steps", C.c_int64)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_ip)


def u8ptr(a: np.ndarray):
    assert a.dtype == np.uint8 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_u8p)


def make_config(n_dg: int, tracking: int, deposition: int, precision: int, species, max_particles: int,
                external_field=(0.0,) * 6, refmapping_eps: float = 1e-4, sf_radius: float = 0.0,
                sf_alpha: int = 2, sort_interval: int = 0, sf_dim: int = 3, sf_dir: int = 1,
                sf_depo3d: bool = True, time_step_factor=None, periodic_tracing: bool = False,
                ref_mapping_guess: int = 0) -> PicConfig:
    """species: list of (charge, mass, mpf); time_step_factor: per species (Species%TimeStepFactor), None = 1;
    periodic_tracing: RefTracking traces periodic sides as BC sides (CartesianPeriodic = F); ref_mapping_guess:
    RefMappingGuess 1..4 (0 = 1)."""
    cfg = PicConfig()
    cfg.n_dg = n_dg
    cfg.tracking = tracking
    cfg.deposition = deposition
    cfg.precision = precision
    cfg.max_particles = max_particles
    cfg.n_species = len(species)
    for s, (q, m, w) in enumerate(species):
        cfg.charge[s] = q
        cfg.mass[s] = m
        cfg.mpf[s] = w
    for s, f in enumerate(time_step_factor or []):
        cfg.time_step_factor[s] = float(f)
    cfg.periodic_tracing = 1 if periodic_tracing else 0
    cfg.ref_mapping_guess = int(ref_mapping_guess)
    for i in range(6):
        cfg.external_field[i] = float(external_field[i])
    cfg.refmapping_eps = refmapping_eps
    cfg.sf_radius = sf_radius
    cfg.sf_alpha = sf_alpha
    cfg.sort_interval = sort_interval
    cfg.sf_dim = sf_dim
    cfg.sf_dir = sf_dir
    cfg.sf_depo3d = int(bool(sf_depo3d))
    return cfg


class MeshStruct:
    """A filled PicMesh plus the numpy arrays it points into."""

    def __init__(self, mesh):
        self.mesh = mesh
        keep = {}

        def d(name, arr):
            a = np.ascontiguousarray(arr, dtype=np.float64)
            keep[name] = a
            return dptr(a)

        def i(name, arr):
            a = np.ascontiguousarray(arr, dtype=np.int32)
            keep[name] = a
            return iptr(a)

        s = PicMesh()
        s.n_elems = mesh.n_elems
        s.n_geo = mesh.n_geo
        s.n_nodes = mesh.n_nodes
        pv = mesh.periodic_vectors  # column k = vector k
        s.n_periodic_vectors = int(pv.shape[1])
        for k in range(pv.shape[1]):
            for c in range(3):
                s.periodic_vectors[k * 3 + c] = float(pv[c, k])
        for c in range(3):
            s.xmin_glob[c] = float(mesh.lo[c])
            s.xmax_glob[c] = float(mesh.hi[c])
        s.xi_cl_ngeo = d("xi_cl", mesh.xi_cl_ngeo)
        s.wbary_cl_ngeo = d("wb_cl", mesh.wbary_cl_ngeo)
        s.xgp = d("xgp", mesh.xgp)
        s.wgp = d("wgp", mesh.wgp)
        s.wbary_gp = d("wbgp", mesh.wbary_gp)
        s.xcl_ngeo = d("xcl", mesh.xcl_ngeo)
        s.dxcl_ngeo = d("dxcl", mesh.dxcl_ngeo)
        s.elem_bary = d("bary", mesh.elem_bary)
        s.xez_basis = d("xez", mesh.xez_basis)
        s.slen_basis = d("slen", mesh.slen_basis)
        s.elem_radius = d("rad", mesh.elem_radius)
        s.eps_one_cell = d("eps1", mesh.eps_one_cell)
        s.elem_xgp = d("exgp", mesh.elem_xgp)
        s.elem_sj = d("esj", mesh.elem_sj)
        s.node_coords = d("nc", mesh.node_coords)
        s.elem_node = i("en", mesh.elem_node)
        s.elem_side_node = i("esn", mesh.elem_side_node)
        s.side_nb_elem = i("snb", mesh.side_nb_elem)
        s.side_pvid = i("spv", mesh.side_pvid)
        s.concave_side = i("cc", mesh.concave_side)
        s.node_info = i("ni", mesh.node_info)
        s.node_volume = d("nv", mesh.node_volume)
        s.periodic_n_nodes = i("pn", mesh.periodic_n_nodes)
        s.periodic_offset = i("po", mesh.periodic_offset)
        s.periodic_nodes = i("pnodes", mesh.periodic_nodes)
        s.n_total_periodic_nodes = int(mesh.periodic_n_nodes.sum())
        for c in range(3):
            s.fibgm_imax[c] = int(mesh.fibgm_imax[c])
            s.fibgm_deltas[c] = float(mesh.fibgm_deltas[c])
        s.fibgm_n_elems = i("fn", mesh.fibgm_n_elems)
        s.fibgm_offset = i("fo", mesh.fibgm_offset)
        s.fibgm_element = i("fe", mesh.fibgm_element)
        s.fibgm_n_total = int(len(mesh.fibgm_element))
        s.side_bc = i("sbc", mesh.side_bc) if mesh.side_bc is not None else C.POINTER(C.c_int32)()
        sfr = getattr(mesh, "sf_elem_radius", None)
        s.sf_elem_radius = d("sfr", sfr) if sfr is not None else C.POINTER(C.c_double)()
        e2b = getattr(mesh, "elem_to_bc_sides", None)
        if e2b is not None:
            s.n_bc_entries = int(len(mesh.bc_side_distance))
            s.elem_to_bc_sides = i("e2b", e2b)
            s.bc_side_elem_loc = i("bcl", mesh.bc_side_elem_loc)
            s.bc_side_distance = d("bcd", mesh.bc_side_distance)
        else:
            s.n_bc_entries = 0
            s.elem_to_bc_sides = C.POINTER(C.c_int32)()
            s.bc_side_elem_loc = C.POINTER(C.c_int32)()
            s.bc_side_distance = C.POINTER(C.c_double)()
        ndg = getattr(mesh, "n_dg_mapping", None)
        if ndg is not None:
            s.n_dg_mapping = i("ndg", ndg)
            s.n_inter = d("ninter", mesh.n_inter)
        else:
            s.n_dg_mapping = C.POINTER(C.c_int32)()
            s.n_inter = C.POINTER(C.c_double)()
        ec = getattr(mesh, "elem_curved", None)
        s.elem_curved = i("ecurv", ec) if ec is not None else C.POINTER(C.c_int32)()
        sbz = getattr(mesh, "side_bezier", None)
        s.side_bezier = d("sbez", sbz) if sbz is not None else C.POINTER(C.c_double)()
        sty = getattr(mesh, "side_type", None)
        s.side_type = i("stype", sty) if sty is not None else C.POINTER(C.c_int32)()
        self.struct = s
        self._keep = keep

    @property
    def ptr(self):
        return C.byref(self.struct)


def repo_root() -> str:
    return os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
