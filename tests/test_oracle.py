"""CPU tests: the oracle against the reference's known answers and analytic solutions."""
import json
import math
import os

import numpy as np
import pytest

from piclas_gb300 import capi, workloads
from piclas_gb300.mesh import (barycentric_weights, build_box_mesh, cheby_gauss_lobatto_nodes, elem_map,
                               lagrange_polys, legendre_gauss_nodes, sf_adaptive_radius)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")


@pytest.fixture(scope="module")
def kat():
    with open(GOLDEN) as f:
        return json.load(f)


# ---- basis (basis.f90) -----------------------------------------------------------------------
def test_gauss_nodes_are_legendre_roots():
    for N in (1, 2, 3, 4):
        x, w = legendre_gauss_nodes(N)
        ref, wref = np.polynomial.legendre.leggauss(N + 1)
        assert np.allclose(x, ref, atol=1e-15, rtol=0)
        assert np.allclose(w, wref, atol=2e-15, rtol=0)


def test_lagrange_kronecker_and_partition(oracle_lib):
    x, _ = legendre_gauss_nodes(3)
    wb = barycentric_weights(x)
    for i, xi in enumerate(x):
        L = oracle_lib.lagrange_polys(xi, x, wb)
        assert np.array_equal(L, np.eye(4)[i])          # ALMOSTEQUAL_UNITY branch
    for t in np.linspace(-0.99, 0.99, 17):
        L = oracle_lib.lagrange_polys(t, x, wb)
        assert abs(L.sum() - 1.0) < 1e-15
        assert np.allclose(L, lagrange_polys(t, x, wb), rtol=0, atol=0)   # C and Python restatements agree


def test_cl_nodes_ngeo1():
    assert cheby_gauss_lobatto_nodes(1) == [-1.0, 1.0]
    assert barycentric_weights([-1.0, 1.0]) == [-0.5, 0.5]


# ---- cell_volweight_mean charge conservation (Plasma_Ball_cell_volweight_mean) ---------------
def _plasma_ball(kat, seed=0):
    k = kat["cvwm_plasma_ball"]
    mesh = build_box_mesh(10, 10, 10, k["N"], lo=(-1, -1, -1), hi=(1, 1, 1))
    rng = np.random.default_rng(seed)
    n = k["n_particles"]
    # uniform in a sphere of RadiusIC around the origin
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    r = k["sphere_radius"] * rng.random(n) ** (1.0 / 3.0)
    x = d * r[:, None]
    ps = np.concatenate([x, np.zeros((n, 3))], axis=1)
    elem = workloads._elem_of_uniform(mesh, x)
    cfg = capi.make_config(k["N"], capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64,
                           [(k["charge_ic"], 1.0, k["mpf"])], n)
    return mesh, cfg, ps, elem


def test_cvwm_total_charge_kat(oracle_lib, kat):
    k = kat["cvwm_plasma_ball"]
    mesh, cfg, ps, elem = _plasma_ball(kat)
    ms = capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(ps, elem, np.ones(len(elem), np.int32))
    PS = np.zeros((mesh.n_elems, mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS)
    q = oracle_lib.integrate_charge(ms, mesh.N, PS)
    assert abs(q - k["total_charge"]) <= k["tolerance_abs"], (q, k["total_charge"])


SF_BALL_CASES = ["1d_x-dir", "1d_x-dir-cc", "1d_x-dir-adaptive", "2d_z-dir", "2d_z-dir-cc", "2d_z-dir-adaptive"]


def sf_plasma_ball(kat, case, seed=0):
    """Plasma_Ball_Shape-function-xDir: 100000 resting particles in a ball of radius 0.5 at the origin on the
    4 x 4 x 1 periodic box [-5,5]^3, N = 3, deposited with the case's kernel (1D along x or 2D constant in z;
    shape_function, _cc, or _adaptive with smoothing).  Returns (mesh, cfg, part_state, elem)."""
    k = kat["sf_plasma_ball"]
    c = k["cases"][case]
    mesh = build_box_mesh(*k["n_elems"], k["N"], lo=tuple(k["box_lo"]), hi=tuple(k["box_hi"]))
    rng = np.random.default_rng(seed)
    n = k["n_particles"]
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    x = np.asarray(k["base_point"]) + d * (k["sphere_radius"] * rng.random(n) ** (1.0 / 3.0))[:, None]
    ps = np.concatenate([x, np.zeros((n, 3))], axis=1)
    elem = workloads._elem_of_uniform(mesh, x)
    dep = {"shape_function": capi.PIC_DEPO_SHAPE_FUNCTION, "shape_function_cc": capi.PIC_DEPO_SHAPE_FUNCTION_CC,
           "shape_function_adaptive": capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE}[c["deposition"]]
    if dep == capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE:
        mesh.sf_elem_radius = sf_adaptive_radius(mesh, smoothing=k["adaptive_smoothing"], dim=c["dimension"],
                                                 direction=c["direction"])
    cfg = capi.make_config(k["N"], capi.PIC_TRACK_REFMAPPING, dep, capi.PIC_PREC_FP64,
                           [(k["charge_ic"], 1.0, k["mpf"]), (workloads.Q_ELECTRON, workloads.M_ELECTRON, k["mpf"])],
                           n, sf_radius=k["sf_radius"], sf_alpha=k["sf_alpha"], sf_dim=c["dimension"],
                           sf_dir=c["direction"], sf_depo3d=k["depo3d"])
    return mesh, cfg, ps, elem


def sf_ball_charge_ok(k, case, q):
    c = k["cases"][case]
    if c["tolerance_type"] == "relative":
        return abs(q - c["total_charge"]) <= c["tolerance"] * abs(c["total_charge"])
    return abs(q - c["total_charge"]) <= c["tolerance"]


@pytest.mark.parametrize("case", SF_BALL_CASES)
def test_sf_plasma_ball_total_charge_kat(oracle_lib, kat, case):
    """The reference's shape-function plasma-ball known answers (1D x / 2D z kernels, plain within 5e-2
    relative, charge-conserving and adaptive within 1e-9 C absolute of 320.435306 C)."""
    mesh, cfg, ps, elem = sf_plasma_ball(kat, case)
    ms = capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(ps, elem, np.ones(len(elem), np.int32))
    PS = np.zeros((mesh.n_elems, mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS, os.cpu_count() or 1)
    q = oracle_lib.integrate_charge(ms, mesh.N, PS)
    assert sf_ball_charge_ok(kat["sf_plasma_ball"], case, q), (case, q)


def test_cvwm_charge_conservation_periodic_twins(oracle_lib):
    """Particles everywhere (incl. periodic corners): the integral still equals the charge."""
    w = workloads.plasma_wave(n_cells=4, N=2, n_particles=3000, seed=3)
    ms = capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(w.config(), ms, st, PS)
    total = w.n * w.species[0][0] * w.species[0][2]
    assert abs(oracle_lib.integrate_charge(ms, w.mesh.N, PS) - total) <= 1e-13 * abs(total)


# ---- Boris push convergence (NIG_convtest_t_poisson constant B_z, orders 2) -------------------
def _gyration_error(oracle_lib, case, dt, use_gamma):
    q, m = case["charge"], case["mass"]
    if use_gamma:
        g = case["gamma"]
        vperp = workloads.C_LIGHT * math.sqrt(1.0 - 1.0 / g ** 2)
        B = g * vperp
        omega = abs(q) * B / (g * m)
    else:
        vperp, B = 1.0, 1.0
        omega = abs(q) * B / m
    rc = vperp / omega
    phi = math.atan2(case["base_point"][1], case["base_point"][0])
    # InitAnalyticalParticleState (pic_interpolation.f90:572-584): x(0) and v(-dt/2) from the
    # analytic solution, IsNewPart = .FALSE.
    x0 = np.array([math.cos(phi) * rc, math.sin(phi) * rc, 0.0])
    th = omega * (-0.5 * dt) + phi
    v0 = np.array([-math.sin(th) * vperp, math.cos(th) * vperp, 0.0])
    cfg = capi.make_config(1, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64, [(q, m, 1.0)], 1)
    st = oracle_lib.OracleState(np.concatenate([x0, v0])[None, :], np.array([1]), np.array([1]),
                                is_new=np.zeros(1, np.uint8))
    st.field[0, 5] = B
    nsteps = int(round(case["tend"] / dt))
    for _ in range(nsteps):
        oracle_lib.push(cfg, st, dt)
    t = nsteps * dt
    ex = np.array([math.cos(omega * t + phi) * rc, math.sin(omega * t + phi) * rc, 0.0])
    return np.linalg.norm(st.part_state[0, :3] - ex) / rc


@pytest.mark.parametrize("which", ["nonrel", "rel"])
def test_boris_second_order(oracle_lib, kat, which):
    case = kat["boris_gyration_" + which]
    dts = case["dt"][1:4] if which == "nonrel" else case["dt"][:3]
    errs = [_gyration_error(oracle_lib, case, dt, which == "rel") for dt in dts]
    orders = [math.log(errs[i] / errs[i + 1]) / math.log(dts[i] / dts[i + 1]) for i in range(len(dts) - 1)]
    for o in orders:
        assert abs(o - case["order"]) <= case["order_tolerance"] * case["order"], (errs, orders)


# ---- tracking consistency ---------------------------------------------------------------------
def test_tria_tracking_matches_geometry(oracle_lib):
    w = workloads.plasma_wave(n_cells=6, N=2, n_particles=4000, seed=5, T_eV=2000.0)  # fast: many crossings
    ms = capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.step(w.config(), ms, w.e_dof, st, 2e-10, 5)
    assert st.counters.n_lost == 0
    assert (st.elem != w.elem).sum() > 100
    x = st.part_state[:, :3]
    assert np.all((x >= 0) & (x <= 1))
    assert np.array_equal(workloads._elem_of_uniform(w.mesh, x), st.elem)


def test_ref_tracking_curved_mesh(oracle_lib):
    w = workloads.curved_two_species(n_cells=6, n_per_species=1500, seed=2, Te_eV=5000.0)
    ms = capi.MeshStruct(w.mesh)
    cfg = w.config()
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.map_particles(cfg, ms, st)
    oracle_lib.step(cfg, ms, w.e_dof, st, 2e-11, 4)
    assert st.counters.n_ref_tolerance == 0
    assert (st.elem != w.elem).sum() > 50
    assert np.abs(st.part_pos_ref).max() < 1.0
    # x(xi) in the found element reproduces the particle position
    for i in range(0, st.n, 97):
        xe = elem_map(w.mesh, st.elem[i] - 1, st.part_pos_ref[i])
        assert np.linalg.norm(xe - st.part_state[i, :3]) < 1e-3 * w.mesh.h[0]


def test_shape_function_charge(oracle_lib):
    w = workloads.curved_two_species(n_cells=6, n_per_species=800, seed=1)
    ms = capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state[:800], w.elem[:800], w.part_species[:800])
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(w.config(), ms, st, PS)
    total = 800 * w.species[0][0] * w.species[0][2]
    q = oracle_lib.integrate_charge(ms, w.mesh.N, PS)
    assert abs(q - total) <= 2e-3 * abs(total)      # quadrature of the kernel on the DG grid


# ---- particle boundaries: open and reflective walls (TriaTracking) ----------------------------
def _wall_case(bc, n=4000, T_eV=2000.0, seed=9, cells=5, N=2, field=False):
    mesh = build_box_mesh(cells, cells, cells, N, bc=bc)
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, T_eV=T_eV, seed=seed, dt=2e-10)
    if not field:
        w.e_dof[:] = 0.0
    return w


def _oracle_steps(oracle_lib, w, nsteps):
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, nsteps)
    return st


def test_wall_mesh_arrays():
    m = build_box_mesh(3, 3, 3, 1, bc=("reflective", "open", "periodic"))
    assert m.periodic_vectors.shape == (3, 1) and m.periodic_vectors[2, 0] == 1.0
    walls = m.side_nb_elem == 0
    assert np.array_equal(walls, m.side_bc > 0)
    assert (m.side_bc == 2).sum() == 2 * 9 and (m.side_bc == 1).sum() == 2 * 9
    assert np.all(np.abs(m.side_pvid[walls]) == 0) and set(np.unique(np.abs(m.side_pvid))) == {0, 1}
    assert not m.concave_side[walls].any()
    # node twins only across the periodic z faces; node volumes still add up to the box volume
    assert m.periodic_n_nodes.max() == 1
    assert abs(m.node_volume.sum() - (1.0 + m.node_volume[m.periodic_n_nodes > 0].sum() / 2.0)) < 1e-12


def test_reflective_walls_keep_particles(oracle_lib):
    w = _wall_case(("reflective", "reflective", "reflective"))
    st = _oracle_steps(oracle_lib, w, 30)
    x, v0, v = st.part_state[:, :3], w.part_state[:, 3:], st.part_state[:, 3:]
    assert st.inside.all() and st.counters.n_lost == 0
    assert (x >= 0.0).all() and (x <= 1.0).all()
    # specular reflection keeps |v| (no field); many particles were reflected at least once
    assert np.allclose(np.linalg.norm(v, axis=1), np.linalg.norm(v0, axis=1), rtol=1e-13, atol=0.0)
    assert (np.sign(v) != np.sign(v0)).any(axis=1).sum() > 500
    assert np.array_equal(st.elem, workloads._elem_of_uniform(w.mesh, x))


def test_open_walls_remove_the_leaving_particles(oracle_lib):
    w = _wall_case(("open", "periodic", "periodic"))
    K = 30
    st = _oracle_steps(oracle_lib, w, K)
    # free streaming: a particle is removed iff its straight path ends outside 0 < x < 1
    xf = w.part_state[:, 0] + w.part_state[:, 3] * (w.dt * K)
    clear = (np.abs(xf) > 1e-9) & (np.abs(xf - 1.0) > 1e-9)
    expect = (xf > 0.0) & (xf < 1.0)
    assert np.array_equal(st.inside[clear].astype(bool), expect[clear])
    assert (~expect).sum() > 300 and st.counters.n_lost == 0
    kept = st.inside.astype(bool)
    assert np.array_equal(st.elem[kept], workloads._elem_of_uniform(w.mesh, st.part_state[kept, :3]))


def test_adaptive_with_uniform_radius_is_cc(oracle_lib):
    """shape_function_adaptive with every element radius = R is shape_function_cc with radius R."""
    w = workloads.curved_two_species(n_cells=5, n_per_species=800, seed=4, nsteps=1)
    w.mesh.sf_elem_radius = np.full(w.mesh.n_elems, w.sf_radius)
    out = {}
    for dep in (capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE):
        w.deposition = dep
        cfg, ms = w.config(), capi.MeshStruct(w.mesh)
        st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
        PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
        oracle_lib.deposit(cfg, ms, st, PS)
        out[dep] = PS
    assert np.array_equal(out[capi.PIC_DEPO_SHAPE_FUNCTION_CC], out[capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])


# ---- walls with RefTracking (ParticleBCTracking over planar wall sides) -----------------------------
def _ref_wall_steps(oracle_lib, w, nsteps):
    w.tracking = capi.PIC_TRACK_REFMAPPING
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    oracle_lib.map_particles(cfg, ms, st)
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, nsteps)
    return st


def test_bc_elem_distance_lists():
    m = build_box_mesh(4, 3, 3, 1, bc=("reflective", "open", "reflective"))
    e2b, loc, dist = m.elem_to_bc_sides, m.bc_side_elem_loc, m.bc_side_distance
    walls = {(e + 1, s + 1) for e in range(m.n_elems) for s in range(6) if m.side_nb_elem[e, s] == 0}
    assert len(walls) == 2 * (9 + 12 + 12)
    for e in range(m.n_elems):
        n, f = e2b[e]
        own = {(e + 1, s + 1) for s in range(6) if m.side_nb_elem[e, s] == 0}
        if n < 0:
            assert not own
            continue
        ent = [tuple(x) for x in loc[f:f + n]]
        assert own <= set(ent) and set(ent) <= walls and len(set(ent)) == n
        assert np.all(np.diff(dist[f:f + n]) >= 0.0)          # sorted by distance
    assert (e2b[:, 0] > 0).sum() == m.n_elems                 # halo = one element extent: all elements in reach


def test_reftracking_reflective_box_matches_triatracking(oracle_lib):
    w = _wall_case(("reflective", "reflective", "reflective"), n=3000, seed=12)
    tri = _oracle_steps(oracle_lib, w, 30)
    ref = _ref_wall_steps(oracle_lib, w, 30)
    assert ref.inside.all() and ref.counters.n_ref_tolerance == 0
    x = ref.part_state[:, :3]
    assert (x >= 0.0).all() and (x <= 1.0).all()
    # both trackers reflect at the same planes with the same normal: velocities identical, positions
    # equal up to the rounding of the two intersection formulas
    assert np.array_equal(ref.part_state[:, 3:], tri.part_state[:, 3:])
    assert np.max(np.abs(ref.part_state[:, :3] - tri.part_state[:, :3])) < 1e-13
    assert (np.sign(ref.part_state[:, 3:]) != np.sign(w.part_state[:, 3:])).any(axis=1).sum() > 500
    assert np.array_equal(ref.elem, workloads._elem_of_uniform(w.mesh, x))


def test_reftracking_open_walls_remove_the_leaving_particles(oracle_lib):
    w = _wall_case(("open", "open", "open"), n=3000, seed=13)
    K = 20
    ref = _ref_wall_steps(oracle_lib, w, K)
    xf = w.part_state[:, :3] + w.part_state[:, 3:] * (w.dt * K)
    clear = np.all((np.abs(xf) > 1e-9) & (np.abs(xf - 1.0) > 1e-9), axis=1)
    expect = np.all((xf > 0.0) & (xf < 1.0), axis=1)
    assert np.array_equal(ref.inside[clear].astype(bool), expect[clear])
    assert (~expect).sum() > 300 and ref.counters.n_ref_tolerance == 0


def test_reftracking_walls_curved_mesh(oracle_lib):
    """Interior nodes displaced, planar walls (reflective in x and z, open in y), no field: every particle
    follows the folded straight line, leaves iff its y path leaves (0,1), and ends in an element whose
    reference coordinates hold it."""
    mesh = build_box_mesh(4, 4, 4, 2, perturb=0.05, bc=("reflective", "open", "reflective"))
    w = workloads.plasma_wave(mesh=mesh, n_particles=3000, T_eV=2000.0, seed=14, dt=2e-10)
    w.e_dof[:] = 0.0
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(14))   # true (curved) elements
    w.part_state[:, :3] = x
    w.elem = e
    K = 20
    ref = _ref_wall_steps(oracle_lib, w, K)
    assert ref.counters.n_ref_tolerance == 0
    xs = w.part_state[:, :3] + w.part_state[:, 3:] * (w.dt * K)

    def fold(u):
        u = np.mod(u, 2.0)
        return np.where(u > 1.0, 2.0 - u, u)

    y = xs[:, 1]
    clear = (np.abs(y) > 1e-9) & (np.abs(y - 1.0) > 1e-9)
    expect = (y > 0.0) & (y < 1.0)
    assert np.array_equal(ref.inside[clear].astype(bool), expect[clear]) and (~expect).sum() > 100
    k = ref.inside.astype(bool)
    assert np.max(np.abs(ref.part_state[k, 0] - fold(xs[k, 0]))) < 1e-12
    assert np.max(np.abs(ref.part_state[k, 2] - fold(xs[k, 2]))) < 1e-12
    assert np.max(np.abs(ref.part_state[k, 1] - y[k])) < 1e-12
    assert np.max(np.abs(ref.part_pos_ref[k])) <= 1.0 + 1e-9


# ---- 1D and 2D shape functions (PIC-shapefunction-dimension / -direction) ---------------------------
def _sf_dim_case(dim, sf_dir, n=400, seed=21, depo3d=True):
    w = workloads.plasma_wave(n_cells=4, N=3, n_particles=n, seed=seed)
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION
    w.sf_radius = 0.3
    w.sf_alpha = 4
    w.sf_dim, w.sf_dir, w.sf_depo3d = dim, sf_dir, depo3d
    return w


def test_sf_1d_single_particle_matches_the_analytic_kernel(oracle_lib):
    from math import gamma, pi, sqrt
    w = _sf_dim_case(1, 1, n=1)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS)
    q = w.species[0][0] * w.species[0][2]
    R, a = w.sf_radius, w.sf_alpha
    wsf = gamma(a + 1.5) / (sqrt(pi) * R * gamma(a + 1)) / 1.0            # extent in y and z: 1 x 1
    x0 = w.part_state[0, 0]
    xg = w.mesh.elem_xgp.reshape(w.mesh.n_elems, -1, 3)[..., 0]
    expect = np.zeros_like(xg)
    for shift in (-1.0, 0.0, 1.0):                                        # the three periodic cases
        d2 = (xg - (x0 + shift)) ** 2
        expect += np.where(d2 <= R * R, (1.0 - d2 / (R * R)) ** a, 0.0) * wsf * q
    assert np.allclose(PS[..., 3], expect, rtol=1e-12, atol=1e-12 * np.abs(expect).max())


@pytest.mark.parametrize("dim,sf_dir", [(1, 1), (1, 3), (2, 1), (2, 2)])
def test_sf_1d_2d_conserve_charge_and_are_constant_across(oracle_lib, dim, sf_dir):
    w = _sf_dim_case(dim, sf_dir)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS)
    total = w.n * w.species[0][0] * w.species[0][2]
    assert abs(oracle_lib.integrate_charge(ms, w.mesh.N, PS) - total) <= 2e-3 * abs(total)
    # rho depends only on the kernel coordinates: equal at DOFs whose kernel coordinates are equal
    xg = w.mesh.elem_xgp.reshape(-1, 3)
    kdirs = [sf_dir - 1] if dim == 1 else [d for d in range(3) if d != sf_dir - 1]
    key = np.round(xg[:, kdirs], 12)
    rho = PS[..., 3].reshape(-1)
    _, inv = np.unique(key, axis=0, return_inverse=True)
    for k in range(inv.max() + 1):
        v = rho[inv == k]
        assert np.allclose(v, v[0], rtol=1e-11, atol=1e-11 * np.abs(rho).max())


# ---- shape_function_cc / _adaptive without periodic vectors (depoChargeOnDOFsSFChargeCon / ...Adaptive) ----
def _walled_sf_case(dep, n=300, seed=5, cells=4, N=2):
    mesh = build_box_mesh(cells, cells, cells, N, bc=("reflective", "open", "reflective"))
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, seed=seed)
    w.deposition = dep
    w.sf_radius = 0.4
    w.sf_alpha = 3
    h = 1.0 / cells
    w.mesh.sf_elem_radius = np.random.default_rng(seed).uniform(1.2 * h, 2.6 * h, mesh.n_elems)
    return w


def _sf_con_numpy(mesh, P, fac, R, alpha, elems):
    """The normalised kernel alpha (Fac S1) on the DOFs within R of P in the given elements (0-based)."""
    ne, nd = mesh.n_elems, mesh.n_dof
    xg = mesh.elem_xgp.reshape(ne, nd, 3)[elems]
    sj = mesh.elem_sj.reshape(ne, nd)[elems]
    w3 = np.einsum("k,j,i->kji", mesh.wgp, mesh.wgp, mesh.wgp).reshape(-1)
    r2 = ((P - xg) ** 2).sum(-1)
    S1 = np.where(r2 <= R * R, 1.0 - r2 / (R * R), 0.0) ** alpha
    tot = (w3 * fac[3] * S1 / sj).sum()
    out = np.zeros((ne, nd, 4))
    out[elems] = (fac[3] / tot) * S1[..., None] * fac
    return out


@pytest.mark.parametrize("dep", [capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])
def test_charge_conserving_sf_without_periodic_vectors(oracle_lib, dep):
    w = _walled_sf_case(dep)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS)
    q, mpf = w.species[0][0], w.species[0][2]
    total = w.n * q * mpf
    # every particle's charge is kept, also where the kernel is cut by a wall
    assert abs(oracle_lib.integrate_charge(ms, w.mesh.N, PS) - total) <= 1e-12 * abs(total)
    # single particles against an independent evaluation; adaptive: the particle's element and the
    # elements sharing a corner node with it (ElemToElemMapping), radius of the particle's element
    ni = w.mesh.node_info
    for ip in range(0, w.n, 37):
        e0 = int(w.elem[ip]) - 1
        one = oracle_lib.OracleState(w.part_state[ip:ip + 1], w.elem[ip:ip + 1], w.part_species[ip:ip + 1])
        ps1 = np.zeros_like(PS)
        oracle_lib.deposit(cfg, ms, one, ps1)
        P = w.part_state[ip, :3]
        fac = np.array([*w.part_state[ip, 3:], 1.0]) * (q * mpf)
        if dep == capi.PIC_DEPO_SHAPE_FUNCTION_CC:
            ref = _sf_con_numpy(w.mesh, P, fac, w.sf_radius, w.sf_alpha, np.arange(w.mesh.n_elems))
        else:
            nb = np.flatnonzero(np.isin(ni, ni[e0]).any(axis=1))
            ref = _sf_con_numpy(w.mesh, P, fac, w.mesh.sf_elem_radius[e0], w.sf_alpha, nb)
            outside = np.setdiff1d(np.arange(w.mesh.n_elems), nb)
            assert not ps1[outside].any()
        assert np.allclose(ps1, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


# ---- RefTracking walls that are bilinear (SideType BILINEAR) or planar non-rectangles -------------------
_FACES = {  # tensor-corner layout of the six hexahedron faces: axis, side (0 low / 1 high)
    "x-": (0, 0), "x+": (0, 1), "y-": (1, 0), "y+": (1, 1), "z-": (2, 0), "z+": (2, 1)}


def _face_corners(mesh, e, axis, hi):
    """The four corners of a face as X(u,v) = sum corner * (bilinear weights), u/v along the other axes."""
    C = mesh.xcl_ngeo.reshape(mesh.n_elems, 2, 2, 2, 3)[e]       # [k][j][i]
    o1, o2 = [a for a in range(3) if a != axis]
    P = np.zeros((2, 2, 3))
    for a in range(2):
        for b in range(2):
            idx = [0, 0, 0]
            idx[axis], idx[o1], idx[o2] = hi, a, b
            P[a, b] = C[idx[2], idx[1], idx[0]]
    return P


def _patch_hit(P, xl, d, tmax):
    """Newton for X(u,v) = xl + t d on the bilinear patch with corners P[a][b], u,v in [0,1]."""
    u = v = 0.5
    t = 0.0
    for _ in range(60):
        X = (P[0, 0] * (1 - u) * (1 - v) + P[1, 0] * u * (1 - v) + P[0, 1] * (1 - u) * v + P[1, 1] * u * v)
        Xu = (P[1, 0] - P[0, 0]) * (1 - v) + (P[1, 1] - P[0, 1]) * v
        Xv = (P[0, 1] - P[0, 0]) * (1 - u) + (P[1, 1] - P[1, 0]) * u
        F = X - xl - t * d
        J = np.stack([Xu, Xv, -d], axis=1)
        du, dv, dt = np.linalg.solve(J, -F)
        u, v, t = u + du, v + dv, t + dt
        if max(abs(du), abs(dv), abs(dt)) < 1e-16:
            break
    ok = -1e-12 <= u <= 1 + 1e-12 and -1e-12 <= v <= 1 + 1e-12 and 0.0 <= t <= tmax
    n = np.cross(Xu, Xv)
    return ok, t, n / np.linalg.norm(n)


def _walled_case(bulge=0.0, shear=0.0, bc=("reflective",) * 3, n=2000, seed=15):
    mesh = build_box_mesh(4, 4, 4, 2, bc=bc, wall_bulge=bulge, wall_shear=shear)
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, T_eV=2000.0, seed=seed, dt=2e-10)
    w.e_dof[:] = 0.0
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(seed))
    w.part_state[:, :3] = x
    w.elem = e
    return w


@pytest.mark.parametrize("bulge,shear", [(0.2, 0.0), (0.0, 0.15), (0.15, 0.1)])
def test_reftracking_nonplanar_reflective_walls_keep_particles(oracle_lib, bulge, shear):
    w = _walled_case(bulge, shear)
    ref = _ref_wall_steps(oracle_lib, w, 25)
    v0, v = w.part_state[:, 3:], ref.part_state[:, 3:]
    assert ref.inside.all() and ref.counters.n_lost == 0 and ref.counters.n_ref_tolerance == 0
    assert np.max(np.abs(ref.part_pos_ref)) <= 1.0 + 1e-9
    assert np.allclose(np.linalg.norm(v, axis=1), np.linalg.norm(v0, axis=1), rtol=1e-13, atol=0.0)
    assert (np.abs(v - v0).max(axis=1) > 0).sum() > 300          # many reflections


@pytest.mark.parametrize("bulge,shear", [(0.2, 0.0), (0.0, 0.15)])
@pytest.mark.parametrize("face", ["x-", "y+", "z-"])
def test_reftracking_nonplanar_wall_single_reflection(oracle_lib, bulge, shear, face):
    """One particle against one wall side: the hit point, the normal there (bilinear: d/dxi x d/deta at the
    hit; planar: the side normal) and the reflected state against an independent Newton solve."""
    w = _walled_case(bulge, shear, n=1)
    m = w.mesh
    axis, hi = _FACES[face]
    ijk = [2, 1, 2]
    ijk[axis] = 3 if hi else 0
    e = ijk[0] + 4 * (ijk[1] + 4 * ijk[2])
    P = _face_corners(m, e, axis, hi)
    target = P.mean(axis=(0, 1)) + 0.1 * (P[1, 0] - P[0, 0]) - 0.05 * (P[0, 1] - P[0, 0])
    start = m.elem_bary[e] + 0.2 * (m.elem_bary[e] - target)
    d = target - start
    L = np.linalg.norm(d)
    d /= L
    step = L + 0.4 * 0.25                                          # crosses the wall by 0.4 h
    w.dt = 1e-9
    w.part_state[0, :3] = start
    w.part_state[0, 3:] = d * step / w.dt
    w.elem = np.array([e + 1], np.int32)
    ok, t, n = _patch_hit(P, start, d, step)
    assert ok
    if np.dot(n, target - m.elem_bary[e]) < 0:
        n = -n
    poi = start + t * d
    d2 = d - 2.0 * np.dot(d, n) * n
    x_exp = poi + d2 * (step - t)
    v_exp = w.part_state[0, 3:] - 2.0 * np.dot(w.part_state[0, 3:], n) * n
    ref = _ref_wall_steps(oracle_lib, w, 1)
    assert ref.inside[0] == 1
    assert np.max(np.abs(ref.part_state[0, :3] - x_exp)) < 1e-12
    assert np.max(np.abs(ref.part_state[0, 3:] - v_exp)) < 1e-9 * np.linalg.norm(v_exp)
    if bulge:
        assert abs(abs(n[axis]) - 1.0) > 1e-6                       # the wall is tilted at the hit


def test_reftracking_bilinear_open_wall_removes(oracle_lib):
    """A particle that crosses the bulged open wall is removed; one stopping short of it stays."""
    for frac, kept in ((0.4, False), (-0.05, True)):
        w = _walled_case(0.2, 0.0, bc=("open", "reflective", "reflective"), n=1)
        m = w.mesh
        e = 0 + 4 * (2 + 4 * 1)
        P = _face_corners(m, e, 0, 0)
        target = P.mean(axis=(0, 1))
        start = m.elem_bary[e]
        d = target - start
        L = np.linalg.norm(d)
        d /= L
        w.dt = 1e-9
        w.part_state[0, :3] = start
        w.part_state[0, 3:] = d * (L + frac * 0.25) / w.dt
        w.elem = np.array([e + 1], np.int32)
        ref = _ref_wall_steps(oracle_lib, w, 1)
        assert bool(ref.inside[0]) == kept


def test_sf_adaptive_radius_init():
    """InitShapeFunctionAdaptive on uniform boxes: the nearest unshared neighbour corner is h away and the
    bounding-box length is h, so R = h (3 DOF/(4 pi))^(1/3) / (N+1) = 2h/(N+1) at the default DOF (4/3)pi 2^3;
    smoothing averages with the same h; a larger DOF scales R by the cube root."""
    from piclas_gb300.mesh import elem_to_elem, sf_adaptive_radius
    for N in (1, 2, 3):
        m = build_box_mesh(4, 3, 5, N, bc=("reflective", "open", "periodic"))
        h = float(np.min(m.h))
        r = sf_adaptive_radius(m)
        hmin = np.minimum.reduce([m.h[0], m.h[1], m.h[2]])
        assert np.allclose(r, 2.0 * hmin / (N + 1), rtol=1e-14)
        assert np.allclose(sf_adaptive_radius(m, smoothing=True), r * 0 + (hmin + np.prod(m.h) ** (1 / 3)) / 2 * 2 / (N + 1),
                           rtol=1e-14)
        if N > 1:
            assert np.allclose(sf_adaptive_radius(m, adaptive_dof=(4 / 3) * np.pi * 8 * 1.728), 1.2 * r, rtol=1e-12)
        assert h > 0
    nb = elem_to_elem(build_box_mesh(3, 3, 3, 1, bc=("open",) * 3))
    assert len(nb[13]) == 26 and len(nb[0]) == 7 and 13 not in nb[13]
    with pytest.raises(ValueError):
        sf_adaptive_radius(build_box_mesh(2, 2, 2, 1), adaptive_dof=40.0)


def test_adaptive_with_initialised_radius_conserves_charge(oracle_lib):
    from piclas_gb300.mesh import sf_adaptive_radius
    mesh = build_box_mesh(5, 5, 5, 3, bc=("reflective", "open", "reflective"), perturb=0.05)
    w = workloads.plasma_wave(mesh=mesh, n_particles=400, seed=16)
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(16))
    w.part_state[:, :3] = x
    w.elem = e
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE
    w.mesh.sf_elem_radius = sf_adaptive_radius(mesh)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS)
    total = w.n * w.species[0][0] * w.species[0][2]
    assert abs(oracle_lib.integrate_charge(ms, w.mesh.N, PS) - total) <= 1e-12 * abs(total)


# ---- 1D/2D shape_function_cc / _adaptive -------------------------------------------------------------
@pytest.mark.parametrize("dep", [capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])
@pytest.mark.parametrize("walls", [False, True])
@pytest.mark.parametrize("dim,sf_dir,depo3d", [(1, 1, True), (1, 3, False), (2, 2, True), (2, 1, False)])
def test_sf_1d_2d_charge_conserving(oracle_lib, dep, walls, dim, sf_dir, depo3d):
    """Integrated deposit per particle: q MPF, times dimFactorSF where the charge sits on a line / an area
    (3D-deposition = F) and the branch divides its total by it (the periodic branch and the Adaptive routine;
    ChargeCon without periodic vectors does not).  rho depends on the kernel coordinates only."""
    hi = (1.0, 0.5, 0.8)
    bc = ("reflective", "open", "reflective") if walls else ("periodic",) * 3
    mesh = build_box_mesh(4, 4, 4, 2, hi=hi, bc=bc)
    w = workloads.plasma_wave(mesh=mesh, n_particles=300, seed=22)
    w.deposition = dep
    w.sf_radius, w.sf_alpha = 0.3, 3
    w.sf_dim, w.sf_dir, w.sf_depo3d = dim, sf_dir, depo3d
    w.mesh.sf_elem_radius = np.random.default_rng(22).uniform(0.25, 0.45, mesh.n_elems)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS)
    d = sf_dir - 1
    dim_factor = float(np.prod([hi[a] for a in range(3) if a != d])) if dim == 1 else hi[d]
    divides = not depo3d and (not walls or dep == capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE)
    total = w.n * w.species[0][0] * w.species[0][2] * (dim_factor if divides else 1.0)
    assert abs(oracle_lib.integrate_charge(ms, w.mesh.N, PS) - total) <= 1e-12 * abs(total)
    if dep == capi.PIC_DEPO_SHAPE_FUNCTION_CC:
        xg = w.mesh.elem_xgp.reshape(-1, 3)
        kdirs = [d] if dim == 1 else [a for a in range(3) if a != d]
        _, inv = np.unique(np.round(xg[:, kdirs], 12), axis=0, return_inverse=True)
        rho = PS[..., 3].reshape(-1)
        for k in range(inv.max() + 1):
            v = rho[inv == k]
            assert np.allclose(v, v[0], rtol=1e-11, atol=1e-11 * np.abs(rho).max())


# ---- species-specific time step (VarTimeStep%UseSpeciesSpecific, Species%TimeStepFactor) ----------------
def test_species_time_step_factor_free_streaming(oracle_lib):
    """No field: species s moves by v dt factor_s per step (timedisc_TimeStepPoissonByBorisLeapfrog.f90:130-135),
    factor 0 meaning 1; through periodic faces with TriaTracking."""
    w = workloads.plasma_wave(n_cells=4, N=2, n_particles=600, seed=31, T_eV=500.0)
    w.e_dof[:] = 0.0
    q, m, mpf = w.species[0]
    w.species = [(q, m, mpf), (q, 4.0 * m, mpf)]
    w.part_species = np.where(np.arange(w.n) % 2 == 0, 1, 2).astype(np.int32)
    w.time_step_factor = (0.0, 0.25)
    K = 5
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, K)
    fac = np.where(w.part_species == 1, 1.0, 0.25)[:, None]
    x = w.part_state[:, :3]
    for _ in range(K):
        x = x + w.part_state[:, 3:] * (w.dt * fac)
    x = np.mod(x, 1.0)
    assert np.max(np.abs(np.mod(st.part_state[:, :3] - x + 0.5, 1.0) - 0.5)) < 1e-12
    assert st.inside.all() and np.array_equal(st.elem, workloads._elem_of_uniform(w.mesh, st.part_state[:, :3]))


def test_timing_build_matches_checker(oracle_lib):
    """The CPU baseline is timed with the oracle built like the reference's release build (-O3, FMA
    contraction).  It computes the same loop: element ids identical and the state within rounding of the
    checker build after 5 steps of the plasma wave and of the curved RefTracking/shape-function box."""
    for w in (workloads.plasma_wave(n_cells=4, N=3, n_particles=4000, seed=71, T_eV=200.0),
              workloads.curved_two_species(n_cells=4, n_per_species=2000, seed=72, nsteps=5)):
        cfg, ms = w.config(), capi.MeshStruct(w.mesh)
        res = []
        for timing in (False, True):
            oracle_lib.set_timing_build(timing)
            try:
                st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
                if w.tracking == capi.PIC_TRACK_REFMAPPING:
                    oracle_lib.map_particles(cfg, ms, st)
                PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
                oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, 5, PS)
                res.append((st, PS))
            finally:
                oracle_lib.set_timing_build(False)
        (a, pa), (b, pb) = res
        assert np.array_equal(a.elem, b.elem)
        assert np.max(np.abs(a.part_state - b.part_state)) <= 1e-10 * np.max(np.abs(a.part_state))
        assert np.max(np.abs(pa - pb)) <= 1e-10 * np.max(np.abs(pa))


# ---- RefTracking with periodic sides traced as BC sides (CartesianPeriodic = F) ------------------------
def _periodic_tracing_steps(oracle_lib, w, nsteps, tracing):
    w.tracking = capi.PIC_TRACK_REFMAPPING
    w.periodic_tracing = tracing
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    oracle_lib.map_particles(cfg, ms, st)
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, nsteps)
    return st


def test_periodic_tracing_lists_hold_the_periodic_sides():
    m = build_box_mesh(4, 4, 4, 1, perturb=0.05, periodic_tracing=True)
    e2b, loc, dist = m.elem_to_bc_sides, m.bc_side_elem_loc, m.bc_side_distance
    per = {(e + 1, s + 1) for e in range(m.n_elems) for s in range(6) if m.side_pvid[e, s] != 0}
    assert len(per) == 6 * 16
    for e in range(m.n_elems):
        n, f = e2b[e]
        own = {(e + 1, s + 1) for s in range(6) if m.side_pvid[e, s] != 0}
        if n < 0:
            assert not own
            continue
        ent = [tuple(x) for x in loc[f:f + n]]
        assert own <= set(ent) and set(ent) <= per and len(set(ent)) == n
        assert np.all(np.diff(dist[f:f + n]) >= 0.0)


def test_periodic_tracing_matches_cartesian_periodic(oracle_lib):
    """The reference's default periodic RefTracking (periodic sides traced as BC sides, PeriodicBoundary) and
    the CartesianPeriodic/FastPeriodic variant move particles across the periodic box alike: the same elements,
    velocities identical, positions equal up to the rounding of the two shift formulas."""
    mesh = build_box_mesh(6, 6, 6, 2, perturb=0.05, periodic_tracing=True)
    w = workloads.plasma_wave(mesh=mesh, n_particles=4000, T_eV=3000.0, seed=91, dt=1e-10)
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(91))
    w.part_state[:, :3] = x
    w.elem = e
    a = _periodic_tracing_steps(oracle_lib, w, 12, False)
    b = _periodic_tracing_steps(oracle_lib, w, 12, True)
    assert np.array_equal(a.elem, b.elem)
    assert np.array_equal(a.part_state[:, 3:], b.part_state[:, 3:])
    assert np.max(np.abs(a.part_state[:, :3] - b.part_state[:, :3])) < 1e-13
    assert np.max(np.abs(a.part_pos_ref - b.part_pos_ref)) < 1e-10
    assert b.counters.n_ref_tolerance == 0 and b.inside.all()
    crossed = np.any(np.abs(b.part_state[:, :3] - (w.part_state[:, :3] + w.part_state[:, 3:] * w.dt * 12)) > 0.5, axis=1)
    assert crossed.sum() > 200                              # many particles crossed a periodic side


def test_periodic_tracing_with_walls_free_streaming(oracle_lib):
    """Reflective walls in x, periodic y and z traced as BC sides, no field: every particle follows the straight
    line folded at x = 0, 1 and wrapped in y, z, and ends in the element that holds it."""
    mesh = build_box_mesh(5, 4, 4, 2, bc=("reflective", "periodic", "periodic"), periodic_tracing=True)
    w = workloads.plasma_wave(mesh=mesh, n_particles=4000, T_eV=3000.0, seed=92, dt=2e-10)
    w.e_dof[:] = 0.0
    K = 20
    st = _periodic_tracing_steps(oracle_lib, w, K, True)
    assert st.inside.all() and st.counters.n_ref_tolerance == 0
    xs = w.part_state[:, :3] + w.part_state[:, 3:] * (w.dt * K)
    u = np.mod(xs[:, 0], 2.0)
    fx = np.where(u > 1.0, 2.0 - u, u)
    want = np.stack([fx, np.mod(xs[:, 1], 1.0), np.mod(xs[:, 2], 1.0)], axis=1)
    d = st.part_state[:, :3] - want
    d[:, 1:] -= np.round(d[:, 1:])                           # y, z: modulo the period
    assert np.max(np.abs(d)) < 1e-12
    assert np.array_equal(st.elem, workloads._elem_of_uniform(w.mesh, st.part_state[:, :3]))


# ---- per-element polynomial degree (p-adaption, N_DG_Mapping) --------------------------------------------
def test_p_adaption_mapping_layout():
    """N_DG_Mapping(1:3,:) of Set_N_DG_Mapping: row 1 the running DOF offsets, row 2 the degrees, row 3 = row 1 on
    one process; N_Inter(1..NMax) blocks hold the Gauss nodes, weights and barycentric weights of each degree;
    Elem_xGP and sJ of an element of degree k equal those of the same element in a uniform degree-k mesh."""
    from piclas_gb300.mesh import p_adaption_degrees
    nl = p_adaption_degrees(4, 3, 2, "random", 1, 3, seed=4)
    assert set(np.unique(nl)) <= {1, 2, 3} and len(np.unique(nl)) == 3
    m = build_box_mesh(4, 3, 2, 3, perturb=0.05, n_loc=nl)
    g = m.n_dg_mapping
    assert np.array_equal(g[:, 1], nl) and np.array_equal(g[:, 0], g[:, 2])
    assert np.array_equal(g[:, 0], np.concatenate([[0], np.cumsum((nl + 1) ** 3)[:-1]]))
    assert m.n_dofs == int(((nl + 1) ** 3).sum())
    ni, off = m.n_inter, 0
    for k in (1, 2, 3):
        xg, wg = legendre_gauss_nodes(k)
        assert np.array_equal(ni[off:off + k + 1], xg)
        assert np.array_equal(ni[off + k + 1:off + 2 * (k + 1)], wg)
        assert np.array_equal(ni[off + 2 * (k + 1):off + 3 * (k + 1)], barycentric_weights(xg))
        off += 3 * (k + 1)
        mu = build_box_mesh(4, 3, 2, k, perturb=0.05)
        for e in np.nonzero(nl == k)[0]:
            assert np.array_equal(m.elem_dofs(m.elem_xgp, e), mu.elem_dofs(mu.elem_xgp, e))
            assert np.array_equal(m.elem_dofs(m.elem_sj, e), mu.elem_dofs(mu.elem_sj, e))
            assert m.eps_one_cell[e] == mu.eps_one_cell[e]
    hh = p_adaption_degrees(4, 1, 1, "half-half", 1, 3, lo=(-1, 0, 0), hi=(1, 1, 1))
    assert list(hh) == [1, 1, 3, 3]


@pytest.mark.parametrize("dep", [capi.PIC_DEPO_CVWM, capi.PIC_DEPO_SHAPE_FUNCTION, capi.PIC_DEPO_SHAPE_FUNCTION_CC])
def test_p_adaption_one_degree_equals_fixed_n(oracle_lib, dep):
    """A p-adapted mesh whose elements all have degree 2 (NMax = 3) runs the loop exactly as the uniform N = 2
    mesh: identical positions, velocities, elements, PartSource and integrated charge after 3 steps."""
    res = []
    for mesh in (build_box_mesh(4, 4, 4, 2, perturb=0.05), build_box_mesh(4, 4, 4, 3, perturb=0.05, n_loc=np.full(64, 2))):
        w = workloads.plasma_wave(mesh=mesh, n_particles=3000, seed=5, deposition=dep)
        w.sf_radius = 0.3
        cfg, ms = w.config(), capi.MeshStruct(mesh)
        st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
        PS = np.zeros(mesh.dof_shape(4))
        oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, 3, PS)
        res.append((st.part_state.copy(), st.elem.copy(), PS.reshape(-1), oracle_lib.integrate_charge(ms, mesh.N, PS)))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    assert np.array_equal(res[0][2], res[1][2]) and res[0][3] == res[1][3]


@pytest.mark.parametrize("dep", [capi.PIC_DEPO_CVWM, capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])
def test_p_adaption_deposition_conserves_charge(oracle_lib, dep):
    """Degrees 1..3 at random: cell_volweight_mean (NodeVolume and CellVolWeight(Nloc) per element) and the
    charge-conserving shape functions integrate, element by element with each element's own Gauss rule, to the
    deposited charge within 1e-12."""
    from piclas_gb300.mesh import p_adaption_degrees
    nl = p_adaption_degrees(5, 5, 5, "random", 1, 3, seed=7)
    mesh = build_box_mesh(5, 5, 5, 3, perturb=0.05, n_loc=nl)
    if dep == capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE:
        mesh.sf_elem_radius = sf_adaptive_radius(mesh)
    w = workloads.plasma_wave(mesh=mesh, n_particles=4000, seed=9, deposition=dep)
    w.sf_radius = 0.25
    cfg, ms = w.config(), capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros(mesh.dof_shape(4))
    oracle_lib.deposit(cfg, ms, st, PS, os.cpu_count() or 1)
    total = w.n * w.species[0][0] * w.species[0][2]
    assert abs(oracle_lib.integrate_charge(ms, mesh.N, PS) - total) <= 1e-12 * abs(total)


def test_p_adaption_interpolation_reproduces_trilinear_field(oracle_lib):
    """A field trilinear in the reference coordinates (here E linear in x on an unperturbed box) lies in every
    degree's polynomial space: EvaluateFieldAtRefPos with each element's Nloc returns it at the particles to
    rounding, for degrees 1..3 side by side."""
    from piclas_gb300.mesh import p_adaption_degrees
    nl = p_adaption_degrees(4, 4, 4, "random", 1, 3, seed=2)
    mesh = build_box_mesh(4, 4, 4, 3, n_loc=nl)
    w = workloads.plasma_wave(mesh=mesh, n_particles=2000, seed=3)
    A = np.array([[1.0, -2.0, 0.5], [0.3, 0.7, -1.1], [2.0, 0.1, 0.4]])
    b = np.array([0.2, -0.3, 0.9])
    e_dof = mesh.elem_xgp.reshape(-1, 3) @ A.T + b
    cfg, ms = w.config(), capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.interpolate(cfg, ms, e_dof, st)
    want = w.part_state[:, :3] @ A.T + b
    assert np.max(np.abs(st.field[:, :3] - want)) <= 1e-13 * np.max(np.abs(want))


# ---- RefMappingGuess 1..4 (GetRefNewtonStartValue) ----------------------------------------------------------
@pytest.mark.parametrize("guess", [1, 2, 3, 4])
def test_ref_mapping_guess_maps_particles(oracle_lib, guess):
    """Every start value of the Newton (linear guess, closest Gauss point, closest corner, zero) maps particles on
    a curved box and on a p-adapted one to xi with x(xi) = x within 1e-5 h (the Newton stops once
    |dxi|^2 <= RefMappingEps = 1e-4, so the last iterate carries the quadratic remainder), and RefTracking over 3
    steps gives the same elements as the default guess, states within 1e-9 (the field at slightly different xi)."""
    from piclas_gb300.mesh import p_adaption_degrees
    for nl in (None, p_adaption_degrees(4, 4, 4, "random", 1, 3, seed=6)):
        mesh = build_box_mesh(4, 4, 4, 3, perturb=0.08, n_loc=nl)
        w = workloads.curved_two_species(mesh=mesh, n_per_species=1000, seed=12, nsteps=3)
        ms = capi.MeshStruct(mesh)
        cfg = w.config()
        cfg.ref_mapping_guess = guess
        st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
        oracle_lib.map_particles(cfg, ms, st)
        x = np.array([elem_map(mesh, e - 1, xi) for e, xi in zip(w.elem, st.part_pos_ref)])
        assert np.max(np.abs(x - w.part_state[:, :3])) <= 1e-5 * float(mesh.h[0])
        oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, 3, None)
        cfg1 = w.config()
        st1 = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
        oracle_lib.map_particles(cfg1, ms, st1)
        oracle_lib.step(cfg1, ms, w.e_dof, st1, w.dt, 3, None)
        assert np.array_equal(st.elem, st1.elem)
        assert np.max(np.abs(st.part_state - st1.part_state) / np.max(np.abs(st1.part_state), axis=0)) <= 1e-9


def test_ref_mapping_guess_start_values(oracle_lib):
    """The start values themselves: with a Newton limited to no iteration effect (a particle exactly at a Gauss
    point, or at a corner) guesses 2 and 3 return that node's xi exactly."""
    mesh = build_box_mesh(2, 2, 2, 2, perturb=0.05)
    ms = capi.MeshStruct(mesh)
    xg, _ = legendre_gauss_nodes(2)
    e = 5
    P = mesh.elem_dofs(mesh.elem_xgp, e)
    r = 2 * 9 + 1 * 3 + 0                         # (i, j, k) = (0, 1, 2)
    cfg = capi.make_config(2, capi.PIC_TRACK_REFMAPPING, capi.PIC_DEPO_CVWM, 0, [(-1.0, 1.0, 1.0)], 1, ref_mapping_guess=2)
    st = oracle_lib.OracleState(np.concatenate([P[r], [0, 0, 0]])[None, :], np.array([e + 1]), np.array([1]))
    oracle_lib.map_particles(cfg, ms, st)
    assert np.array_equal(st.part_pos_ref[0], [xg[0], xg[1], xg[2]])
    X = mesh.xcl_ngeo.reshape(mesh.n_elems, 2, 2, 2, 3)[e]
    cfg.ref_mapping_guess = 3
    st = oracle_lib.OracleState(np.concatenate([X[1, 0, 1], [0, 0, 0]])[None, :], np.array([e + 1]), np.array([1]))
    oracle_lib.map_particles(cfg, ms, st)
    assert np.array_equal(st.part_pos_ref[0], [1.0, -1.0, 1.0])      # corner (i, j, k) = (1, 0, 1): X[k][j][i]


# ---- curved elements (NGeo > 1) ------------------------------------------------------------------------------
@pytest.mark.parametrize("ng", [2, 3])
def test_curved_mesh_geometry(ng):
    """The NGeo mesh: corners are the grid nodes, shared faces have identical CL points (conforming), the map
    reproduces XCL_NGeo at the CL points, every perturbed element is ElemCurved and an unperturbed one is not
    (then Elem_xGP, sJ and ElemBaryNGeo equal those of the NGeo = 1 box to rounding)."""
    m = build_box_mesh(4, 4, 4, 2, perturb=0.08, n_geo=ng)
    X = m.xcl_ngeo
    assert np.array_equal(m.node_coords[:, 0], X[:, 0, 0, 0]) and np.array_equal(m.node_coords[:, 7], X[:, -1, -1, -1])
    e = m.elem_index(1, 2, 1)
    assert np.array_equal(X[e][:, :, -1], X[m.elem_index(2, 2, 1)][:, :, 0])
    assert np.array_equal(X[e][:, -1, :], X[m.elem_index(1, 3, 1)][:, 0, :])
    xi_cl = m.xi_cl_ngeo
    for (a, b, c) in ((0, 0, 0), (1, 0, ng), (ng, ng - 1, 1)):
        assert np.allclose(elem_map(m, e, (xi_cl[a], xi_cl[b], xi_cl[c])), X[e, c, b, a], rtol=0, atol=1e-15)
    assert m.elem_curved.all()
    m0, m1 = build_box_mesh(3, 3, 3, 2, n_geo=ng), build_box_mesh(3, 3, 3, 2)
    assert not m0.elem_curved.any()
    for a in ("elem_xgp", "elem_sj", "elem_bary"):
        assert np.allclose(getattr(m0, a), getattr(m1, a), rtol=1e-14, atol=1e-15), a


@pytest.mark.parametrize("ng", [2, 3])
def test_curved_newton_and_loop(oracle_lib, ng):
    """RefElemNewton on XCL_NGeo: particles placed at known xi of curved elements are mapped back to it within the
    Newton's stopping rule (all four start values), RefTracking + shape function loses none of them over 5
    steps, and cell_volweight_mean on the curved box conserves the charge to 1e-12."""
    from piclas_gb300.workloads import _uniform_in_mesh
    mesh = build_box_mesh(4, 4, 4, 3, perturb=0.08, n_geo=ng)
    ms = capi.MeshStruct(mesh)
    rng = np.random.default_rng(4)
    x, e, xi0 = _uniform_in_mesh(mesh, 3000, rng)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=1500, seed=5, Te_eV=1000.0)
    w.part_state[:, :3] = x
    w.elem = e
    for guess in (1, 2, 3, 4):
        cfg = w.config()
        cfg.ref_mapping_guess = guess
        st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
        oracle_lib.map_particles(cfg, ms, st)
        assert np.max(np.abs(st.part_pos_ref - xi0)) <= 1e-4, guess
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.map_particles(w.config(), ms, st)
    oracle_lib.step(w.config(), ms, w.e_dof, st, w.dt * 20, 5, None)
    assert st.counters.n_lost == 0 and st.counters.n_ref_tolerance == 0 and (st.elem != w.elem).sum() > 20
    cfg = capi.make_config(3, capi.PIC_TRACK_REFMAPPING, capi.PIC_DEPO_CVWM, 0, w.species, w.n)
    st2 = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros(mesh.dof_shape(4))
    oracle_lib.deposit(cfg, ms, st2, PS)
    total = sum(w.species[s - 1][0] * w.species[s - 1][2] for s in w.part_species)
    scale = sum(abs(w.species[s - 1][0] * w.species[s - 1][2]) for s in w.part_species)
    assert abs(oracle_lib.integrate_charge(ms, mesh.N, PS) - total) <= 1e-12 * scale


# ---- curved wall sides (Bezier clipping) --------------------------------------------------------------------
def _face_point(mesh, e, s, u, v):
    """Point and tangents of the wall face of element e (0-based) at the face parameters (u, v): the element's
    NGeo map with the face's reference coordinate fixed (s: 'ylo' -> xi_2 = -1, u = xi_1, v = xi_3)."""
    assert s == "ylo"
    x = elem_map(mesh, e, (u, -1.0, v))
    d = 1e-5                                            # central differences (O(d^2) for the polynomial map)
    tu = (elem_map(mesh, e, (u + d, -1.0, v)) - elem_map(mesh, e, (u - d, -1.0, v))) / (2 * d)
    tv = (elem_map(mesh, e, (u, -1.0, v + d)) - elem_map(mesh, e, (u, -1.0, v - d))) / (2 * d)
    return x, tu, tv


def _line_face_hit(mesh, e, x0, dx):
    """(alpha, hit point, unit normal) of the segment x0 + alpha*dx (alpha in [0, 1]) and the lower y wall face of
    element e, by Newton's method on x(u, v) - x0 - alpha*dx = 0 (independent of the library's Bezier clipping)."""
    q = np.array([0.0, 0.0, 0.5])
    for _ in range(50):
        x, tu, tv = _face_point(mesh, e, "ylo", q[0], q[1])
        r = x - x0 - q[2] * dx
        J = np.stack([tu, tv, -dx], axis=1)
        q = q - np.linalg.solve(J, r)
        if np.max(np.abs(r)) < 1e-15:
            break
    x, tu, tv = _face_point(mesh, e, "ylo", q[0], q[1])
    n = np.cross(tu, tv)
    return q, x, n / np.linalg.norm(n)


@pytest.mark.parametrize("n_geo", [2, 3, 4])
def test_curved_wall_reflection_against_an_independent_solve(oracle_lib, n_geo):
    """Bulged (SideType CURVED) reflective walls: a particle that reaches the lower y wall within one step ends at
    the mirror image of its path in the wall's tangent plane at the hit point, with the velocity reflected there;
    hit point and normal from a plain Newton solve on the face of the element map (the Bezier clipping stops at
    ClipTol = 1e-8 in the face parameters: positions agree to 1e-8 h)."""
    mesh = build_box_mesh(4, 4, 4, 2, bc=("reflective", "reflective", "reflective"), wall_bulge=0.2, n_geo=n_geo)
    assert (mesh.side_type[mesh.side_nb_elem == 0] == 4).all()
    rng = np.random.default_rng(7)
    n = 40
    h = 0.25
    xz = rng.uniform(0.15, 0.85, size=(n, 2))
    p0 = np.column_stack([xz[:, 0], np.full(n, 0.06), xz[:, 1]])
    vel = np.column_stack([rng.uniform(-0.3, 0.3, n), -np.ones(n), rng.uniform(-0.3, 0.3, n)]) * 1.0e6
    dt = 0.035 / 1.0e6
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, seed=3, dt=dt)
    w.e_dof[:] = 0.0
    w.part_state[:, :3], w.part_state[:, 3:] = p0, vel
    ix, iz = np.floor(p0[:, 0] / h).astype(int), np.floor(p0[:, 2] / h).astype(int)
    w.elem = (ix + 4 * (0 + 4 * iz) + 1).astype(np.int32)
    w.tracking = capi.PIC_TRACK_REFMAPPING
    cfg, ms = w.config(), capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species, is_new=np.zeros(n, np.uint8))
    oracle_lib.map_particles(cfg, ms, st)
    assert np.abs(st.part_pos_ref).max() <= 1.0
    oracle_lib.step(cfg, ms, w.e_dof, st, dt, 1)
    assert st.inside.all() and st.counters.n_lost == 0
    checked = 0
    for i in range(n):
        dx = vel[i] * dt
        q, xh, nrm = _line_face_hit(mesh, w.elem[i] - 1, p0[i], dx)
        if not (-1.0 < q[0] < 1.0 and -1.0 < q[1] < 1.0 and 0.0 < q[2] < 1.0):
            continue                        # leaves the element's face patch first (hits a neighbour's face)
        v2 = vel[i] - 2.0 * np.dot(vel[i], nrm) * nrm
        x2 = xh + v2 * dt * (1.0 - q[2])
        assert np.max(np.abs(st.part_state[i, :3] - x2)) < 1e-8 * h, i
        assert np.max(np.abs(st.part_state[i, 3:] - v2)) < 1e-7 * np.linalg.norm(vel[i]), i
        checked += 1
    assert checked >= 25


def test_planar_curved_walls_fold_straight_paths(oracle_lib):
    """Sheared wall faces of an NGeo = 2 box stay in the box planes (SideType PLANAR_CURVED, in-plane CL points
    moved): reflective walls fold every straight path exactly as plane walls do, open walls remove the particles
    whose unfolded y path leaves (0, 1).  The hit points come from BezierNewton on the projected patch (stopped at
    a squared update below BezierNewtonTolerance2): the folded positions agree to 1e-9."""
    mesh = build_box_mesh(4, 4, 4, 2, bc=("reflective", "open", "reflective"), wall_shear=0.3, n_geo=2)
    assert (mesh.side_type[mesh.side_nb_elem == 0] == 3).all()
    w = workloads.plasma_wave(mesh=mesh, n_particles=3000, T_eV=2000.0, seed=15, dt=2e-10)
    w.e_dof[:] = 0.0
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(15))
    w.part_state[:, :3] = x
    w.elem = e
    K = 20
    ref = _ref_wall_steps(oracle_lib, w, K)
    assert ref.counters.n_ref_tolerance == 0 and ref.counters.n_lost == 0
    xs = w.part_state[:, :3] + w.part_state[:, 3:] * (w.dt * K)

    def fold(u):
        u = np.mod(u, 2.0)
        return np.where(u > 1.0, 2.0 - u, u)

    y = xs[:, 1]
    clear = (np.abs(y) > 1e-9) & (np.abs(y - 1.0) > 1e-9)
    expect = (y > 0.0) & (y < 1.0)
    assert np.array_equal(ref.inside[clear].astype(bool), expect[clear]) and (~expect).sum() > 100
    k = ref.inside.astype(bool)
    assert np.max(np.abs(ref.part_state[k, 0] - fold(xs[k, 0]))) < 1e-9
    assert np.max(np.abs(ref.part_state[k, 2] - fold(xs[k, 2]))) < 1e-9
    assert np.max(np.abs(ref.part_state[k, 1] - y[k])) < 1e-12
    assert np.max(np.abs(ref.part_pos_ref[k])) <= 1.0 + 1e-9


def test_curved_open_walls_remove_exactly_the_crossing_particles(oracle_lib):
    """Bulged open walls in y: particles moving along y (away from the x and z walls) are removed iff their end
    point lies beyond the wall surface at their (x, z); the survivors move on their straight paths, stay mapped
    within [-1, 1]^3 and their element map reproduces their position."""
    mesh = build_box_mesh(4, 4, 4, 2, perturb=0.05, bc=("reflective", "open", "reflective"), wall_bulge=0.2, n_geo=2)
    rng = np.random.default_rng(16)
    w = workloads.plasma_wave(mesh=mesh, n_particles=2000, T_eV=2000.0, seed=16, dt=2e-10)
    w.e_dof[:] = 0.0
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, rng)
    keep = np.all((x[:, [0, 2]] > 0.1) & (x[:, [0, 2]] < 0.9), axis=1)
    x, e = x[keep], e[keep]
    n = len(x)
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, T_eV=2000.0, seed=16, dt=2e-10)
    w.e_dof[:] = 0.0
    w.part_state[:, :3] = x
    w.part_state[:, 3] = 0.0
    w.part_state[:, 5] = 0.0
    w.part_state[:, 4] = rng.choice([-1.0, 1.0], n) * rng.uniform(0.1, 0.45, n) / (w.dt * 10)   # |v| < 0.76 c
    w.elem = e
    ref = _ref_wall_steps(oracle_lib, w, 10)
    assert ref.counters.n_lost == 0 and ref.counters.n_ref_tolerance == 0
    yend = x[:, 1] + w.part_state[:, 4] * w.dt * 10
    h = 0.25

    def wall_y(px, pz, top):
        # the wall face above/below (px, pz): solve x(u, +-1, v)[x, z] = (px, pz) on the wall element by Newton's
        # method (all particles at once, central differences: exact for the quadratic map), then take its y
        ix, iz = np.minimum((px / h).astype(int), 3), np.minimum((pz / h).astype(int), 3)
        eidx = ix + 4 * ((3 if top else 0) + 4 * iz)
        s2 = 1.0 if top else -1.0

        def xmap(q):
            return workloads._curved_map(mesh, eidx, np.column_stack([q[:, 0], np.full(len(q), s2), q[:, 1]]))[0]
        q = np.zeros((len(px), 2))
        d = 1e-5
        for _ in range(30):
            r = xmap(q)[:, [0, 2]] - np.column_stack([px, pz])
            J = np.empty((len(px), 2, 2))
            for a in range(2):
                dq = np.zeros(2)
                dq[a] = d
                J[:, :, a] = (xmap(q + dq) - xmap(q - dq))[:, [0, 2]] / (2 * d)
            q = q - np.linalg.solve(J, r[..., None])[..., 0]
        return xmap(q)[:, 1]

    ylo = wall_y(x[:, 0], x[:, 2], False)
    yhi = wall_y(x[:, 0], x[:, 2], True)
    expect = (yend > ylo) & (yend < yhi)
    clear = (np.abs(yend - ylo) > 1e-7) & (np.abs(yend - yhi) > 1e-7)
    got = ref.inside.astype(bool)
    assert np.array_equal(got[clear], expect[clear]) and (~expect).sum() > 50 and expect.sum() > 50
    k = got
    assert np.max(np.abs(ref.part_state[k, :3] - np.column_stack([x[:, 0], yend, x[:, 2]])[k])) < 1e-12
    assert np.max(np.abs(ref.part_pos_ref[k])) <= 1.0 + 1e-9
    for i in np.nonzero(k)[0][:50]:
        # PartPosRef from RefElemNewton, stopped by its tolerance (RefMappingEps = 1e-4 on the update)
        assert np.allclose(elem_map(mesh, ref.elem[i] - 1, ref.part_pos_ref[i]), ref.part_state[i, :3], atol=1e-4 * h)
