"""Seeded synthetic inputs for the particle-loop workloads.

The reference builds its particles through emission (``particle_emission_tools.f90``) and its
field through the HDG solver.  Neither is on the path, so the harness generates both with a
seeded numpy generator:

* ``plasma_wave``: unit cube, nx^3 linear hexahedra, fully periodic, electrons with density
  ``n0*(1+A sin(2 pi x))`` (inverse-CDF sampling in x, uniform in y, z), Maxwellian velocities,
  and the matching frozen field E_x = e n0 A/(2 pi eps0) cos(2 pi x) of an immobile neutralising
  ion background (the reference has no immobile-ion option; the ions are the field's constant).
* ``curved_two_species``: a box with interior nodes displaced by 0.05 h sin sin sin, electrons and
  ions (mass ratio 1836) uniform in space (sampled per element with a det(J) rejection so the
  element is known exactly), an external B_z and a frozen smooth synthetic E.

Constants follow the reference's globals (globals_vars.f90:53-90) and tutorials.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .mesh import BoxMesh, build_box_mesh

C_LIGHT = 299792458.0
EPS0 = 8.8541878176e-12
BOLTZMANN = 1.380648813e-23
EV2KELVIN = 1.16045250061657e4
Q_ELECTRON = -1.60217653e-19      # Part-SpeciesX-ChargeIC used by the PIC tutorials
M_ELECTRON = 9.1093826e-31        # ElectronMass


def maxwell_sigma(T_eV: float, mass: float) -> float:
    return math.sqrt(BOLTZMANN * T_eV * EV2KELVIN / mass)


@dataclass
class Workload:
    name: str
    mesh: BoxMesh
    species: list                   # [(charge, mass, mpf)]
    tracking: int
    deposition: int
    part_state: np.ndarray          # (n, 6)  PartState(1:6, n)
    elem: np.ndarray                # (n,)    1-based GlobalElemID
    part_species: np.ndarray        # (n,)    1-based
    e_dof: np.ndarray               # (nElems, nDOF, 3); with p-adaption packed (nDofs, 3)
    dt: float
    nsteps: int
    external_field: tuple = (0.0,) * 6
    sf_radius: float = 0.0
    sf_alpha: int = 2
    sf_dim: int = 3                 # PIC-shapefunction-dimension
    sf_dir: int = 1                 # PIC-shapefunction-direction
    sf_depo3d: bool = True          # PIC-shapefunction-3D-deposition
    time_step_factor: tuple | None = None   # Species(s)%TimeStepFactor per species (None: 1)
    periodic_tracing: bool = False          # RefTracking: periodic sides traced as BC sides (CartesianPeriodic = F)
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.part_state.shape[0])

    def config(self, precision: int = capi.PIC_PREC_FP64, max_particles: int | None = None,
               sort_interval: int = 0) -> capi.PicConfig:
        return capi.make_config(self.mesh.N, self.tracking, self.deposition, precision, self.species,
                                max_particles if max_particles is not None else self.n,
                                external_field=self.external_field, sf_radius=self.sf_radius,
                                sf_alpha=self.sf_alpha, sort_interval=sort_interval, sf_dim=self.sf_dim,
                                sf_dir=self.sf_dir, sf_depo3d=self.sf_depo3d,
                                time_step_factor=self.time_step_factor, periodic_tracing=self.periodic_tracing)


# --------------------------------------------------------------------------------------
def _inverse_cdf_sine(u: np.ndarray, amp: float) -> np.ndarray:
    """x in [0,1) with density (1 + amp sin(2 pi x)): Newton on F(x) = x + amp/(2pi)(1 - cos 2pi x)."""
    x = u.copy()
    k = amp / (2.0 * math.pi)
    for _ in range(30):
        f = x + k * (1.0 - np.cos(2.0 * math.pi * x)) - u
        fp = 1.0 + amp * np.sin(2.0 * math.pi * x)
        x = x - f / fp
    return np.clip(x, 0.0, np.nextafter(1.0, 0.0))


def _elem_of_uniform(mesh: BoxMesh, x: np.ndarray) -> np.ndarray:
    h = mesh.h
    idx = np.floor((x - mesh.lo) / h).astype(np.int64)
    idx[:, 0] = np.clip(idx[:, 0], 0, mesh.nx - 1)
    idx[:, 1] = np.clip(idx[:, 1], 0, mesh.ny - 1)
    idx[:, 2] = np.clip(idx[:, 2], 0, mesh.nz - 1)
    return (idx[:, 0] + mesh.nx * (idx[:, 1] + mesh.ny * idx[:, 2]) + 1).astype(np.int32)


def plasma_wave(n_cells: int = 8, N: int = 3, n_particles: int = 200_000, amp: float = 0.01, T_eV: float = 1.0,
                n0: float = 1.0e11, dt: float = 1.0e-11, nsteps: int = 100, seed: int = 0,
                tracking: int = capi.PIC_TRACK_TRIA, deposition: int = capi.PIC_DEPO_CVWM,
                mesh: BoxMesh | None = None) -> Workload:
    """The electrostatic plasma wave on the unit cube (8^3 hexahedra, N=3, 200k electrons, 1 eV)."""
    rng = np.random.default_rng(seed)
    if mesh is None:
        mesh = build_box_mesh(n_cells, n_cells, n_cells, N)
    n = n_particles
    x = np.empty((n, 3))
    x[:, 0] = _inverse_cdf_sine(rng.random(n), amp)
    x[:, 1] = rng.random(n)
    x[:, 2] = rng.random(n)
    x = mesh.lo + x * (mesh.hi - mesh.lo)
    sig = maxwell_sigma(T_eV, M_ELECTRON)
    v = rng.normal(0.0, sig, size=(n, 3))
    ps = np.ascontiguousarray(np.concatenate([x, v], axis=1))
    elem = _elem_of_uniform(mesh, x)
    vol = float(np.prod(mesh.hi - mesh.lo))
    mpf = n0 * vol / n
    # field of the perturbation with a neutralising background: dE_x/dx = rho/eps0
    ex0 = (-Q_ELECTRON) * n0 * amp / (2.0 * math.pi * EPS0)
    xg = mesh.elem_xgp.reshape(mesh.dof_shape(3))
    e_dof = np.zeros_like(xg)
    e_dof[..., 0] = ex0 * np.cos(2.0 * math.pi * (xg[..., 0] - mesh.lo[0]) / (mesh.hi[0] - mesh.lo[0]))
    return Workload(name=f"plasma_wave_{mesh.nx}^3_N{mesh.N}_{n}", mesh=mesh,
                    species=[(Q_ELECTRON, M_ELECTRON, mpf)], tracking=tracking, deposition=deposition,
                    part_state=ps, elem=elem, part_species=np.ones(n, np.int32), e_dof=np.ascontiguousarray(e_dof),
                    dt=dt, nsteps=nsteps, info=dict(amp=amp, T_eV=T_eV, n0=n0, mpf=mpf, seed=seed))


# --------------------------------------------------------------------------------------
def _trilinear(mesh: BoxMesh, e0: np.ndarray, xi: np.ndarray):
    """x(xi) and det J of the NGeo=1 map for elements e0 (0-based), vectorised."""
    X = mesh.xcl_ngeo.reshape(mesh.n_elems, 8, 3)[e0]          # corners, tensor order
    f = (0.5 * (1.0 - xi), 0.5 * (1.0 + xi))                    # Lagrange factors per corner side
    x = np.zeros((len(e0), 3))
    J = [np.zeros((len(e0), 3)) for _ in range(3)]
    for t in range(8):
        a, b, c = t & 1, (t >> 1) & 1, t >> 2
        wa, wb, wc = f[a][:, 0], f[b][:, 1], f[c][:, 2]
        Xt = X[:, t, :]
        x += (wa * wb * wc)[:, None] * Xt
        J[0] += ((a - 0.5) * wb * wc)[:, None] * Xt
        J[1] += ((b - 0.5) * wa * wc)[:, None] * Xt
        J[2] += ((c - 0.5) * wa * wb)[:, None] * Xt
    det = np.einsum("nd,nd->n", J[0], np.cross(J[1], J[2]))
    return x, det


def _lagrange_vec(x: np.ndarray, nodes, wbary) -> np.ndarray:
    """Lagrange basis on the nodes at every x (barycentric form; Kronecker at a node), shape (len(x), len(nodes))."""
    nodes = np.asarray(nodes, dtype=np.float64)
    d = x[:, None] - nodes[None, :]
    hit = d == 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.asarray(wbary)[None, :] / d
        L = t / t.sum(axis=1, keepdims=True)
    rows = hit.any(axis=1)
    L[rows] = hit[rows].astype(np.float64)
    return L


def _curved_map(mesh: BoxMesh, e0: np.ndarray, xi: np.ndarray):
    """x(xi) and det J of the NGeo map (Lagrange on the CL points) for elements e0 (0-based), vectorised."""
    ng1 = mesh.n_geo + 1
    L = [_lagrange_vec(xi[:, d], mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo) for d in range(3)]
    X = mesh.xcl_ngeo.reshape(mesh.n_elems, ng1, ng1, ng1, 3)[e0]
    DX = mesh.dxcl_ngeo.reshape(mesh.n_elems, ng1, ng1, ng1, 3, 3)[e0]
    w = np.einsum("na,nb,nc->ncba", L[0], L[1], L[2])
    x = np.einsum("ncba,ncbad->nd", w, X)
    J = np.einsum("ncba,ncbaij->nij", w, DX)              # [nn][dd] = d x_nn / d xi_dd
    return x, np.linalg.det(J)


def _uniform_in_mesh(mesh: BoxMesh, n: int, rng, chunk: int = 1 << 20) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Positions uniform in space, with their element and reference coordinates (chunked)."""
    x = np.empty((n, 3))
    e = np.empty(n, np.int32)
    xi = np.empty((n, 3))
    # rejection bound on det J: the displacement field is smooth, det J stays within a few
    # percent of h^3/8; the bound is checked on every sample
    dmax = float(np.prod(mesh.h)) / 8.0 * 1.25
    # bulged or sheared wall faces vary det J by more: then the bound comes from a probe sample
    pr = np.random.default_rng(12345)
    m = min(65536, 64 * mesh.n_elems)
    e_pr, xi_pr = pr.integers(0, mesh.n_elems, size=m), pr.random((m, 3)) * 2.0 - 1.0
    _, det = _trilinear(mesh, e_pr, xi_pr) if mesh.n_geo == 1 else _curved_map(mesh, e_pr, xi_pr)
    if det.max() >= dmax:
        dmax = 1.3 * float(det.max())
    got = 0
    while got < n:
        m = min(chunk, int((n - got) * 1.4) + 1024)
        e0 = rng.integers(0, mesh.n_elems, size=m)
        xr = rng.random((m, 3)) * 2.0 - 1.0
        xc, det = _trilinear(mesh, e0, xr) if mesh.n_geo == 1 else _curved_map(mesh, e0, xr)
        if det.max() >= dmax or det.min() <= 0.0:
            raise RuntimeError("element Jacobian outside the sampling bound")
        keep = np.nonzero(rng.random(m) * dmax < det)[0][: n - got]
        k = len(keep)
        x[got:got + k] = xc[keep]
        e[got:got + k] = e0[keep] + 1
        xi[got:got + k] = xr[keep]
        got += k
    return x, e, xi


def curved_two_species(n_cells: int = 32, N: int = 3, n_per_species: int = 8_000_000, perturb: float = 0.05,
                       Te_eV: float = 2.0, Ti_eV: float = 0.1, mass_ratio: float = 1836.0, Bz: float = 0.1,
                       E0: float = 100.0, n0: float = 1.0e12, dt: float = 5.0e-12, nsteps: int = 200,
                       sf_radius_cells: float = 1.5, seed: int = 0, mesh: BoxMesh | None = None) -> Workload:
    """Plain FP64 at scale: 32^3 curved box, 8M electrons + 8M ions, B_z, RefTracking, shape function."""
    rng = np.random.default_rng(seed)
    if mesh is None:
        mesh = build_box_mesh(n_cells, n_cells, n_cells, N, perturb=perturb)
    n = 2 * n_per_species
    x, elem, _ = _uniform_in_mesh(mesh, n, rng)
    m_i = mass_ratio * M_ELECTRON
    v = np.empty((n, 3))
    v[:n_per_species] = rng.normal(0.0, maxwell_sigma(Te_eV, M_ELECTRON), size=(n_per_species, 3))
    v[n_per_species:] = rng.normal(0.0, maxwell_sigma(Ti_eV, m_i), size=(n_per_species, 3))
    spec = np.ones(n, np.int32)
    spec[n_per_species:] = 2
    ps = np.ascontiguousarray(np.concatenate([x, v], axis=1))
    vol = float(np.prod(mesh.hi - mesh.lo))
    mpf = n0 * vol / n_per_species
    xg = mesh.elem_xgp.reshape(mesh.dof_shape(3))
    Lb = mesh.hi - mesh.lo
    e_dof = np.empty_like(xg)
    e_dof[..., 0] = E0 * np.sin(2.0 * math.pi * (xg[..., 1] - mesh.lo[1]) / Lb[1])
    e_dof[..., 1] = E0 * np.sin(2.0 * math.pi * (xg[..., 2] - mesh.lo[2]) / Lb[2])
    e_dof[..., 2] = E0 * np.sin(2.0 * math.pi * (xg[..., 0] - mesh.lo[0]) / Lb[0])
    h = float(mesh.h[0])
    return Workload(name=f"curved_{mesh.nx}^3_N{mesh.N}_{n}", mesh=mesh,
                    species=[(Q_ELECTRON, M_ELECTRON, mpf), (-Q_ELECTRON, m_i, mpf)],
                    tracking=capi.PIC_TRACK_REFMAPPING, deposition=capi.PIC_DEPO_SHAPE_FUNCTION,
                    part_state=ps, elem=elem, part_species=spec, e_dof=np.ascontiguousarray(e_dof), dt=dt,
                    nsteps=nsteps, external_field=(0.0, 0.0, 0.0, 0.0, 0.0, Bz), sf_radius=sf_radius_cells * h,
                    sf_alpha=2, info=dict(perturb=perturb, Te_eV=Te_eV, Ti_eV=Ti_eV, Bz=Bz, E0=E0, mpf=mpf,
                                          seed=seed))


def batch_instances(count: int = 32, seed: int = 0):
    """Parameters of the mixed-precision batch: meshes {4,8,12,16}^3, N=3, log-uniform 1e4..2e6
    particles, amplitudes U[0.005,0.05], 100 steps; instance i uses seed i."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        nc = int(rng.choice([4, 8, 12, 16]))
        npart = int(round(math.exp(rng.uniform(math.log(1e4), math.log(2e6)))))
        amp = float(rng.uniform(0.005, 0.05))
        out.append(dict(n_cells=nc, n_particles=npart, amp=amp, seed=i, nsteps=100))
    return out


def differentiable_loop(n_cells: int = 16, N: int = 2, n_particles: int = 1_000_000, T_eV: float = 1.0,
                        Bz: float = 0.05, E0: float = 1.0e3, n0: float = 1.0e11, dt: float = 1.0e-11,
                        nsteps: int = 50, seed: int = 0, mesh: BoxMesh | None = None) -> Workload:
    """Differentiable loop: 16^3 linear hex, N=2, 1M electrons uniform in space, Maxwellian 1 eV,
    B_z = 0.05 T, frozen field E_y = E0 sin(2 pi y), 50 push steps; the loss target at the DOFs is
    rho_target = 1 + 0.05 cos(2 pi y) in units of the mean charge density (``info['rho_scale']``)."""
    rng = np.random.default_rng(seed)
    if mesh is None:
        mesh = build_box_mesh(n_cells, n_cells, n_cells, N)
    n = n_particles
    x = mesh.lo + rng.random((n, 3)) * (mesh.hi - mesh.lo)
    v = rng.normal(0.0, maxwell_sigma(T_eV, M_ELECTRON), size=(n, 3))
    ps = np.ascontiguousarray(np.concatenate([x, v], axis=1))
    elem = _elem_of_uniform(mesh, x)
    vol = float(np.prod(mesh.hi - mesh.lo))
    mpf = n0 * vol / n
    xg = mesh.elem_xgp.reshape(mesh.dof_shape(3))
    Ly = mesh.hi[1] - mesh.lo[1]
    e_dof = np.zeros_like(xg)
    e_dof[..., 1] = E0 * np.sin(2.0 * math.pi * (xg[..., 1] - mesh.lo[1]) / Ly)
    target = 1.0 + 0.05 * np.cos(2.0 * math.pi * (xg[..., 1] - mesh.lo[1]) / Ly)
    rho_scale = Q_ELECTRON * mpf * n / vol
    return Workload(name=f"adjoint_{mesh.nx}^3_N{mesh.N}_{n}", mesh=mesh, species=[(Q_ELECTRON, M_ELECTRON, mpf)],
                    tracking=capi.PIC_TRACK_TRIA, deposition=capi.PIC_DEPO_CVWM, part_state=ps, elem=elem,
                    part_species=np.ones(n, np.int32), e_dof=np.ascontiguousarray(e_dof), dt=dt, nsteps=nsteps,
                    external_field=(0.0, 0.0, 0.0, 0.0, 0.0, Bz),
                    info=dict(rho_target=np.ascontiguousarray(target), rho_scale=rho_scale, Bz=Bz, E0=E0, seed=seed))
