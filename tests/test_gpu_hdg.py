"""GPU HDG Poisson solve (libpiclas_gpu.so through the C-ABI) against the oracle.

Tolerances: Elem_Mat (Ehat, InvDhat, Smat) bit-identical (same per-entry operation order, no FMA
contraction on either side); lambda, phi and E of a solve within 1e-9 of their maximum at epsCG = 1e-12
(the CG dot products are summed in a different order, so the iterates differ in the last bits); a
self-consistent PIC step (deposit -> HDG -> push -> track) keeps the same element ids and positions
within 1e-10 relative.
"""
import numpy as np
import pytest

import oracle
from piclas_gb300 import ParticleLoop, PicError, capi, workloads
from piclas_gb300.hdg_mesh import build_hdg_mesh, exact_func_105, grad_105, source_105
from piclas_gb300.mesh import build_box_mesh

pytestmark = pytest.mark.gpu
L2PI = 6.283185306


def _loop(mesh, precision=capi.PIC_PREC_FP64):
    cfg = capi.make_config(mesh.N, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, precision,
                           [(-1.60217653e-19, 9.1093826e-31, 1.0)], 1)
    return ParticleLoop(cfg, mesh)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("case", ["periodic_curved_N3", "dirichlet_N2", "mixed_N1", "dirichlet_N4"])
def test_elem_mat_bitexact(gpu_lib, oracle_lib, case):
    if case == "periodic_curved_N3":
        m = build_box_mesh(3, 2, 2, 3, perturb=0.08)
        fbc = None
    elif case == "dirichlet_N2":
        m = build_box_mesh(2, 3, 2, 2, lo=(-1, -1, -1), hi=(1, 1, 1), bc=("open",) * 3)
        fbc = None
    elif case == "mixed_N1":
        m = build_box_mesh(2, 2, 3, 1, bc=("periodic", "reflective", "open"))
        fbc = ("periodic", "dirichlet", "neumann")
    else:
        m = build_box_mesh(2, 2, 2, 4, lo=(-1, -1, -1), hi=(1, 1, 1), perturb=0.1, bc=("open",) * 3)
        fbc = None
    h = build_hdg_mesh(m, fbc)
    o = oracle.HdgOracle(m, h)
    loop = _loop(m)
    loop.hdg_init(h, precond_type=1)
    for e in range(m.n_elems):
        eh, di, sm = loop.hdg_elem_mat(e + 1)
        assert np.array_equal(eh, o.ehat[e]), f"Ehat of element {e + 1}"
        assert np.array_equal(di, o.inv_dhat[e]), f"InvDhat of element {e + 1}"
        assert np.array_equal(sm, o.smat[e]), f"Smat of element {e + 1}"
    loop.close()


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_periodic_exact_func_105_parity(gpu_lib, oracle_lib, precond):
    """The reference's CHE_poisson_periodic case: 4^3 periodic box (0,2pi)^3, N = 3, epsCG 1e-12."""
    m = build_box_mesh(4, 4, 4, 3, hi=(L2PI, L2PI, L2PI))
    h = build_hdg_mesh(m)
    o = oracle.HdgOracle(m, h)
    resu = source_105(m.elem_xgp).reshape(m.n_elems, -1)
    Uo, Eo, it_o, _, rc = o.solve(resu, precond_type=precond, eps_cg=1e-12)
    loop = _loop(m)
    loop.hdg_init(h, precond_type=precond, eps_cg=1e-12, max_iter_cg=10000)
    phi, E, st = loop.hdg_solve(resu)
    assert st["converged"] == 1 and abs(st["iterations"] - it_o) <= 3
    assert _rel(phi, Uo) <= 1e-9 and _rel(E, Eo) <= 1e-9
    assert _rel(loop.hdg_lambda(), o.lam) <= 1e-9
    # against the analytic field, as the reference's test does
    assert np.abs(E.reshape(m.elem_xgp.shape) + grad_105(m.elem_xgp)).max() < 3e-3
    loop.close()


@pytest.mark.parametrize("N,precond", [(1, 2), (2, 1), (3, 0), (4, 2)])
def test_dirichlet_curved_parity(gpu_lib, oracle_lib, N, precond):
    m = build_box_mesh(3, 3, 2, N, lo=(-1, -1, -1), hi=(1, 1, 1), perturb=0.08, bc=("open",) * 3)
    h = build_hdg_mesh(m)
    o = oracle.HdgOracle(m, h)
    lam_d = exact_func_105(h.face_xgp[h.dirichlet_sides - 1]).reshape(len(h.dirichlet_sides), -1)
    resu = source_105(m.elem_xgp).reshape(m.n_elems, -1)
    Uo, Eo, it_o, _, rc = o.solve(resu, precond_type=precond, eps_cg=1e-12, lambda_dirichlet=lam_d)
    loop = _loop(m)
    loop.hdg_init(h, precond_type=precond, eps_cg=1e-12, max_iter_cg=10000)
    loop.hdg_set_dirichlet(lam_d)
    phi, E, st = loop.hdg_solve(resu)
    assert st["converged"] == 1
    assert _rel(phi, Uo) <= 1e-9 and _rel(E, Eo) <= 1e-9
    loop.close()


def test_mixed_boundaries_parity_and_warm_start(gpu_lib, oracle_lib):
    m = build_box_mesh(3, 3, 3, 3, hi=(L2PI, L2PI, np.pi), bc=("periodic", "reflective", "open"))
    h = build_hdg_mesh(m, ("periodic", "dirichlet", "neumann"))
    o = oracle.HdgOracle(m, h)
    resu = source_105(m.elem_xgp).reshape(m.n_elems, -1)
    loop = _loop(m)
    loop.hdg_init(h, precond_type=2, eps_cg=1e-12, max_iter_cg=10000)
    for k in range(2):                                   # second solve starts from the first lambda
        Uo, Eo, it_o, _, rc = o.solve(resu * (1.0 + 0.1 * k), precond_type=2, eps_cg=1e-12)
        phi, E, st = loop.hdg_solve(resu * (1.0 + 0.1 * k))
        assert _rel(phi, Uo) <= 1e-9 and _rel(E, Eo) <= 1e-9
        assert st["n_solves"] == k + 1
    loop.close()


def test_solve_from_deposited_charge(gpu_lib, oracle_lib):
    """resu = -PartSource(4)/eps0 of the device deposition (CalcSourceHDG with particles)."""
    w = workloads.plasma_wave(n_cells=4, N=3, n_particles=20000, seed=3)
    h = build_hdg_mesh(w.mesh)
    loop = ParticleLoop(w.config(), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    loop.hdg_init(h, precond_type=2, eps_cg=1e-12, relative=True, max_iter_cg=10000)
    PS = loop.deposition()
    phi, E, st = loop.hdg_solve(None)
    o = oracle.HdgOracle(w.mesh, h)
    resu = -(PS[:, :, 3] / 8.8541878176e-12)
    Uo, Eo, it_o, _, rc = o.solve(resu, precond_type=2, eps_cg=1e-12, relative=True)
    assert st["converged"] == 1
    assert _rel(phi, Uo) <= 1e-8 and _rel(E, Eo) <= 1e-8
    loop.close()


def _neutral_plasma(n_cells, N, n, seed):
    """Plasma-wave electrons plus as many resting ions (q = +e, m = 1836 m_e) spread uniformly, so that
    the periodic potential problem has a neutral source."""
    w = workloads.plasma_wave(n_cells=n_cells, N=N, n_particles=n, seed=seed, T_eV=50.0)
    rng = np.random.default_rng(seed + 100)
    xi = rng.random((n, 3)) * (w.mesh.hi - w.mesh.lo) + w.mesh.lo
    el_i = workloads._elem_of_uniform(w.mesh, xi)
    q, m, mpf = w.species[0]
    ps = np.concatenate([w.part_state, np.concatenate([xi, np.zeros((n, 3))], axis=1)])
    return workloads.Workload(**{**w.__dict__, "species": [w.species[0], (-q, 1836.0 * m, mpf)], "part_state": ps,
                                 "elem": np.concatenate([w.elem, el_i]).astype(np.int32),
                                 "part_species": np.concatenate([w.part_species, np.full(n, 2, np.int32)])})


def _oracle_hdg_steps(w, h, nsteps, precond=2, eps=1e-10):
    cfg = w.config()
    ms = capi.MeshStruct(w.mesh)
    st = oracle.OracleState(w.part_state, w.elem, w.part_species)
    o = oracle.HdgOracle(w.mesh, h)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    for _ in range(nsteps):
        PS[:] = 0.0
        oracle.deposit(cfg, ms, st, PS)
        _, E, _, _, _ = o.solve(-(PS[:, :, 3] / 8.8541878176e-12), precond_type=precond, eps_cg=eps, relative=True)
        oracle.save_last(st)
        oracle.interpolate(cfg, ms, E, st)
        oracle.push(cfg, st, w.dt)
        oracle.track(cfg, ms, st)
    return st, PS


@pytest.mark.parametrize("prec", [capi.PIC_PREC_FP64, capi.PIC_PREC_MIXED])
def test_self_consistent_step_with_hdg(gpu_lib, oracle_lib, prec):
    """pic_step with solve_in_step: Deposition -> HDG -> InterpolateFieldToParticle -> push -> tracking."""
    w = _neutral_plasma(n_cells=4, N=3, n=3000, seed=5)
    h = build_hdg_mesh(w.mesh)
    loop = ParticleLoop(w.config(precision=prec), w.mesh)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    loop.hdg_init(h, precond_type=2, eps_cg=1e-10, relative=True, max_iter_cg=10000, solve_in_step=True)
    PSg = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    loop.time_step(w.dt, 4, PSg)
    g = loop.download_particles()
    stg = loop.status()
    loop.close()
    st, PS = _oracle_hdg_steps(w, h, 4)
    assert stg["error_word"] == 0
    assert np.array_equal(g["elem"], st.elem)
    x_scale = 1.0
    if prec == capi.PIC_PREC_FP64:
        assert np.max(np.abs(g["part_state"][:, :3] - st.part_state[:, :3])) <= 1e-12 * x_scale
        assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-9
        assert _rel(PSg, PS) <= 1e-11
    else:
        assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-5
        assert _rel(PSg, PS) <= 1e-6


def test_cg_not_converged_sets_status(gpu_lib):
    m = build_box_mesh(3, 3, 3, 2, hi=(L2PI, L2PI, L2PI))
    h = build_hdg_mesh(m)
    loop = _loop(m)
    loop.hdg_init(h, precond_type=0, eps_cg=1e-14, max_iter_cg=3)
    phi, E, st = loop.hdg_solve(source_105(m.elem_xgp).reshape(m.n_elems, -1))
    assert st["converged"] == 0 and st["iterations"] == 3
    assert loop.status()["error_word"] & capi.PIC_STATUS_CG_NOT_CONVERGED
    loop.close()


def test_hdg_rejects_bad_input(gpu_lib):
    m = build_box_mesh(2, 2, 2, 2)
    h = build_hdg_mesh(m)
    loop = _loop(m)
    with pytest.raises(PicError):
        loop.hdg_solve(np.zeros((m.n_elems, m.n_dof)))          # before init
    bad = build_hdg_mesh(m)
    bad.elem_to_side = bad.elem_to_side.copy()
    bad.elem_to_side[0, 0, 0] = bad.n_sides + 5
    with pytest.raises(PicError) as e:
        loop.hdg_init(bad)
    assert e.value.code == 1
    with pytest.raises(PicError):
        loop.hdg_init(h, precond_type=7)
    loop.hdg_init(h)
    with pytest.raises(PicError) as e:
        loop.hdg_init(h)                                        # twice
    assert e.value.code == 5
    loop.close()


def test_cooperative_cg_matches_graph_cg(gpu_lib, oracle_lib):
    """cg_kernel = 2 (one cooperative kernel with grid barriers) gives the solution of the default path."""
    m = build_box_mesh(4, 4, 4, 3, hi=(L2PI, L2PI, L2PI), perturb=0.05)
    h = build_hdg_mesh(m)
    resu = source_105(m.elem_xgp).reshape(m.n_elems, -1)
    out = {}
    for k in (1, 2):
        loop = _loop(m)
        loop.hdg_init(h, precond_type=2, eps_cg=1e-12, max_iter_cg=10000, cg_kernel=k)
        out[k] = loop.hdg_solve(resu)
        loop.close()
    assert out[2][2]["converged"] == 1 and abs(out[1][2]["iterations"] - out[2][2]["iterations"]) <= 2
    assert _rel(out[2][0], out[1][0]) <= 1e-9 and _rel(out[2][1], out[1][1]) <= 1e-9


def test_self_consistent_step_between_electrodes(gpu_lib, oracle_lib):
    """Reflective particle walls at x = 0, 1 that are grounded electrodes (Dirichlet phi = 0), periodic y/z:
    Deposition -> HDG -> push -> TriaTracking with wall reflections, against the oracle."""
    mesh = build_box_mesh(4, 4, 4, 2, bc=("reflective", "periodic", "periodic"))
    w = workloads.plasma_wave(mesh=mesh, n_particles=3000, T_eV=2000.0, seed=8, dt=2e-10)
    h = build_hdg_mesh(mesh)                                  # x faces: Dirichlet, lambda = 0
    assert len(h.dirichlet_sides) == 2 * 16
    loop = ParticleLoop(w.config(), w.mesh)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    loop.hdg_init(h, precond_type=1, eps_cg=1e-10, relative=True, max_iter_cg=10000, solve_in_step=True)
    PSg = np.zeros((mesh.n_elems, mesh.n_dof, 4))
    loop.time_step(w.dt, 5, PSg)
    g = loop.download_particles()
    stg = loop.status()
    loop.close()
    st, PS = _oracle_hdg_steps(w, h, 5, precond=1)
    assert stg["error_word"] == 0 and st.inside.all()
    assert np.array_equal(g["elem"], st.elem)
    assert np.max(np.abs(g["part_state"][:, :3] - st.part_state[:, :3])) <= 1e-12
    assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-9
    assert (np.sign(st.part_state[:, 3]) != np.sign(w.part_state[:, 3])).sum() > 20     # wall reflections
