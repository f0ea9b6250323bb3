"""GPU parity: libpiclas_gpu.so (through the C-ABI) against the CPU oracle on seeded inputs.

Tolerances (FP64 variant): element ids bit-exact; positions and velocities bit-exact on the
CVWM/TriaTracking path (same evaluation order, no FMA contraction on either side) and within
1e-13 relative on the B-field path (CUDA's tan may differ from libm's in the last bit);
PartSource within 1e-12 of its maximum (atomic summation order).
Mixed variant: relative charge-density error <= 1e-6 against the FP64 oracle.
"""
import numpy as np
import pytest

from piclas_gb300 import ParticleLoop, PicError, capi, workloads
from piclas_gb300.mesh import build_box_mesh

pytestmark = pytest.mark.gpu


def _run_gpu(w, nsteps, precision=capi.PIC_PREC_FP64, dt=None, sort_interval=0):
    cfg = w.config(precision=precision, sort_interval=sort_interval)
    loop = ParticleLoop(cfg, w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    PS = np.zeros(w.mesh.dof_shape(4))
    loop.time_step(dt or w.dt, nsteps, PS)
    out = loop.download_particles(with_ref=True)
    out["PS"] = PS
    out["status"] = loop.status()
    loop.close()
    return out


def _run_oracle(oracle, w, nsteps, dt=None):
    cfg = w.config()
    ms = capi.MeshStruct(w.mesh)
    st = oracle.OracleState(w.part_state, w.elem, w.part_species)
    if w.tracking == capi.PIC_TRACK_REFMAPPING:
        oracle.map_particles(cfg, ms, st)
    PS = np.zeros(w.mesh.dof_shape(4))
    oracle.step(cfg, ms, w.e_dof, st, dt or w.dt, nsteps, PS)
    return st, PS


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _rho_species_scale(oracle, w, st, nthreads=1):
    """max over DOFs of sum_s |rho_s|: the oracle's charge density of each species deposited on its own from
    the final oracle state.  Electrons and ions cancel in the summed rho, so a mixed-precision error is
    measured against the magnitude the species deposit, not against their small difference."""
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    tot = np.zeros(w.mesh.dof_shape(4)[:-1])
    for s in np.unique(st.species):
        k = (st.species == s) & (st.inside == 1)
        if not k.any():
            continue
        sub = oracle.OracleState(st.part_state[k], st.elem[k], st.species[k], is_new=np.zeros(int(k.sum()), np.uint8),
                                 part_pos_ref=st.part_pos_ref[k])
        PSs = np.zeros(w.mesh.dof_shape(4))
        oracle.deposit(cfg, ms, sub, PSs, nthreads)
        tot += np.abs(PSs[..., 3])
    return float(tot.max())


def _rho_err_species(oracle, w, st, ps_gpu, ps_oracle, nthreads=1):
    """Mixed charge-density error: max |rho_gpu - rho_oracle| / max sum_s |rho_s| (bound: 1e-6)."""
    return float(np.max(np.abs(ps_gpu[..., 3] - ps_oracle[..., 3])) / _rho_species_scale(oracle, w, st, nthreads))


def test_plasma_wave_fp64_bitexact(gpu_lib, oracle_lib):
    w = workloads.plasma_wave(n_cells=8, N=3, n_particles=20000, nsteps=10, seed=0, T_eV=200.0)
    g = _run_gpu(w, 10)
    st, PS = _run_oracle(oracle_lib, w, 10)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["n_lost"] == 0 and g["status"]["error_word"] == 0
    assert (st.elem != w.elem).sum() > 50          # the walk crossed faces, incl. periodic ones


def test_plasma_wave_with_resort(gpu_lib, oracle_lib):
    w = workloads.plasma_wave(n_cells=4, N=2, n_particles=5000, nsteps=6, seed=4, T_eV=500.0)
    g = _run_gpu(w, 6, sort_interval=2)
    st, PS = _run_oracle(oracle_lib, w, 6)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12


def test_pieces_match_oracle(gpu_lib, oracle_lib):
    """interpolate / push / track / deposit called one by one, as the Fortran host would."""
    w = workloads.plasma_wave(n_cells=4, N=3, n_particles=3000, seed=7, T_eV=100.0)
    cfg = w.config()
    ms = capi.MeshStruct(w.mesh)
    loop = ParticleLoop(cfg, w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PSo = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PSo)
    PSg = loop.deposition()
    assert _rel(PSg, PSo) <= 1e-12
    oracle_lib.save_last(st)
    oracle_lib.interpolate(cfg, ms, w.e_dof, st)
    loop.interpolate_field_to_particle()
    assert np.array_equal(loop.field_at_particles(), st.field)
    oracle_lib.push(cfg, st, w.dt)
    loop.push(w.dt)
    oracle_lib.track(cfg, ms, st)
    loop.perform_tracking()
    g = loop.download_particles()
    assert np.array_equal(g["part_state"], st.part_state)
    assert np.array_equal(g["elem"], st.elem)
    loop.close()


def test_curved_sf_reftracking_fp64(gpu_lib, oracle_lib):
    w = workloads.curved_two_species(n_cells=6, n_per_species=2000, seed=3, Te_eV=1000.0, nsteps=4)
    g = _run_gpu(w, 4, dt=2e-11)
    st, PS = _run_oracle(oracle_lib, w, 4, dt=2e-11)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-13
    assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-13
    assert _rel(g["part_pos_ref"], st.part_pos_ref) <= 1e-10
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0


def test_cvwm_kat_on_gpu(gpu_lib):
    """Plasma_Ball_cell_volweight_mean: integral of the deposited charge = 10.68010874898 C."""
    import json, os
    import oracle
    k = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))["cvwm_plasma_ball"]
    from test_oracle import _plasma_ball
    mesh, cfg, ps, elem = _plasma_ball({"cvwm_plasma_ball": k})
    loop = ParticleLoop(cfg, mesh)
    loop.upload_particles(ps, elem, np.ones(len(elem), np.int32))
    PS = loop.deposition()
    q = oracle.integrate_charge(capi.MeshStruct(mesh), mesh.N, PS)
    assert abs(q - k["total_charge"]) <= k["tolerance_abs"]
    # the same check on the device (VerifyDepositedCharge through the C-ABI)
    num, ana = loop.verify_deposited_charge()
    assert abs(num - k["total_charge"]) <= k["tolerance_abs"]
    assert abs(ana - k["total_charge"]) <= k["tolerance_abs"]
    loop.close()


@pytest.mark.parametrize("kind", ["cvwm", "sf_1d_line"])
def test_verify_deposited_charge(gpu_lib, oracle_lib, kind):
    """pic_verify_deposited_charge (VerifyDepositedCharge, pic_analyze.f90:41-133) after pic_step: the numerical
    charge equals the oracle's integral of the same PartSource to 1e-12, the analytical one the sum of
    q * MPF over the particles inside (times dimFactorSF for a 1D kernel with its charge on a line)."""
    if kind == "cvwm":
        w = workloads.plasma_wave(n_cells=4, N=3, n_particles=8000, seed=61, T_eV=100.0)
        factor = 1.0
    else:
        mesh = build_box_mesh(6, 4, 4, 2, lo=(0.0, 0.0, 0.0), hi=(1.0, 0.5, 0.8))
        w = workloads.plasma_wave(mesh=mesh, n_particles=6000, seed=62, T_eV=100.0)
        w.deposition, w.sf_radius, w.sf_dim, w.sf_dir, w.sf_depo3d = capi.PIC_DEPO_SHAPE_FUNCTION, 0.25, 1, 1, False
        factor = 0.5 * 0.8                                   # dimFactorSF: the cross-section of the 1D kernel
    loop = ParticleLoop(w.config(), w.mesh)
    with pytest.raises(PicError):
        loop.verify_deposited_charge()                       # no particles / deposition yet
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    loop.time_step(w.dt, 2, PS)
    num, ana = loop.verify_deposited_charge()
    n_in = loop.status()["n_inside"]
    loop.close()
    qo = oracle_lib.integrate_charge(capi.MeshStruct(w.mesh), w.mesh.N, PS)
    assert abs(num - qo) <= 1e-12 * abs(qo)
    q, _, mpf = w.species[0]
    assert abs(ana - n_in * q * mpf * factor) <= 1e-12 * abs(ana)
    if kind == "cvwm":
        assert abs(num - ana) <= 1e-10 * abs(ana)           # CVWM conserves charge


def test_mixed_precision_rho_error(gpu_lib, oracle_lib):
    w = workloads.plasma_wave(n_cells=8, N=3, n_particles=50000, nsteps=5, seed=1)
    g = _run_gpu(w, 5, precision=capi.PIC_PREC_MIXED)
    st, PS = _run_oracle(oracle_lib, w, 5)
    rho_err = _rel(g["PS"][..., 3], PS[..., 3])
    assert rho_err <= 1e-6, rho_err
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-9
    assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-5


def test_mixed_sf_rho_error(gpu_lib, oracle_lib):
    w = workloads.curved_two_species(n_cells=6, n_per_species=3000, seed=5, nsteps=2)
    g = _run_gpu(w, 2, precision=capi.PIC_PREC_MIXED)
    st, PS = _run_oracle(oracle_lib, w, 2)
    assert _rho_err_species(oracle_lib, w, st, g["PS"], PS) <= 1e-6
    assert np.array_equal(g["elem"], st.elem)


# ---- edge cases ------------------------------------------------------------------------------
def test_empty_particle_set(gpu_lib):
    w = workloads.plasma_wave(n_cells=2, N=1, n_particles=10)
    loop = ParticleLoop(w.config(max_particles=10), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(np.zeros((0, 6)), np.zeros(0, np.int32), np.zeros(0, np.int32))
    PS = loop.deposition()
    assert np.all(PS == 0.0)
    loop.time_step(1e-11, 3)
    assert loop.status()["n_inside"] == 0
    loop.close()


def test_capacity_and_bad_ids_rejected(gpu_lib):
    w = workloads.plasma_wave(n_cells=2, N=1, n_particles=10)
    loop = ParticleLoop(w.config(max_particles=5), w.mesh)
    with pytest.raises(PicError) as e:
        loop.upload_particles(w.part_state, w.elem, w.part_species)
    assert e.value.code == 6
    bad = w.elem[:5].copy()
    bad[2] = 99
    with pytest.raises(PicError) as e:
        loop.upload_particles(w.part_state[:5], bad, w.part_species[:5])
    assert e.value.code == 1
    nan = w.part_state[:5].copy()
    nan[1, 0] = np.nan
    with pytest.raises(PicError):
        loop.upload_particles(nan, w.elem[:5], w.part_species[:5])
    with pytest.raises(PicError) as e:
        loop.time_step(1e-11, 1)                  # no field, no particles yet
    assert e.value.code == 5
    loop.close()


def test_particles_on_faces_nodes_and_holes(gpu_lib, oracle_lib):
    """Particles exactly on element faces, edges and corners (incl. periodic ones), plus holes."""
    mesh = build_box_mesh(4, 4, 4, 2)
    pts = []
    for x in (0.0, 0.25, 0.5, 0.999999999, 1.0):
        for y in (0.0, 0.25, 0.75):
            pts.append((x, y, 0.5))
            pts.append((x, y, 0.0))
    x = np.array(pts)
    n = len(x)
    rng = np.random.default_rng(0)
    v = rng.normal(0, 4e5, size=(n, 3))
    ps = np.ascontiguousarray(np.concatenate([x, v], axis=1))
    elem = workloads._elem_of_uniform(mesh, np.minimum(x, np.nextafter(1.0, 0)))
    inside = np.ones(n, np.uint8)
    inside[::7] = 0                              # holes in the particle vector
    cfg = capi.make_config(2, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64,
                           [(workloads.Q_ELECTRON, workloads.M_ELECTRON, 1e5)], n)
    e_dof = np.zeros((mesh.n_elems, mesh.n_dof, 3))
    loop = ParticleLoop(cfg, mesh)
    loop.set_field(e_dof)
    loop.upload_particles(ps, elem, np.ones(n, np.int32), inside=inside)
    PSg = np.zeros((mesh.n_elems, mesh.n_dof, 4))
    loop.time_step(5e-11, 3, PSg)
    g = loop.download_particles()
    ms = capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(ps, elem, np.ones(n, np.int32), inside=inside)
    PSo = np.zeros_like(PSg)
    oracle_lib.step(cfg, ms, e_dof, st, 5e-11, 3, PSo)
    assert np.array_equal(g["elem"][inside == 1], st.elem[inside == 1])
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["part_state"][inside == 1], st.part_state[inside == 1])
    assert _rel(PSg, PSo) <= 1e-12
    loop.close()


def test_full_size_plasma_wave_properties(gpu_lib):
    """200k electrons, 8^3, N=3, 100 steps: charge conservation each run, elements consistent
    with the geometry (uniform cubes), nothing lost."""
    import oracle
    w = workloads.plasma_wave()
    for prec in (capi.PIC_PREC_FP64, capi.PIC_PREC_MIXED):
        g = _run_gpu(w, w.nsteps, precision=prec, sort_interval=10)
        assert g["status"]["n_lost"] == 0 and g["status"]["error_word"] == 0
        x = g["part_state"][:, :3]
        assert np.array_equal(workloads._elem_of_uniform(w.mesh, x), g["elem"])
        q = oracle.integrate_charge(capi.MeshStruct(w.mesh), w.mesh.N, g["PS"])
        total = w.n * w.species[0][0] * w.species[0][2]
        # FP64: summation order only; mixed: FP32 corner weights sum to 1 within a few FP32 ulps
        tol = 1e-12 if prec == capi.PIC_PREC_FP64 else 1e-6
        assert abs(q - total) <= tol * abs(total), (prec, q, total)


def test_near_face_particles_element_ids_exact(gpu_lib, oracle_lib):
    """Particles at 1e-13..1e-3 cell widths on either side of faces, edges and corners: the FP32
    pre-filter of the inside test must hand all of them to the FP64 test, so element ids stay
    identical to the oracle's."""
    mesh = build_box_mesh(4, 4, 4, 2)
    h = 0.25
    rng = np.random.default_rng(3)
    pts = []
    for off in (1e-13, 1e-11, 1e-9, 1e-7, 1e-5, 1e-3):
        for sgn in (-1.0, 1.0):
            for k in range(40):
                base = rng.integers(1, 4, size=3) * h          # an interior grid node
                axes = rng.random(3) < 0.5                    # face / edge / corner neighbourhoods
                axes[rng.integers(0, 3)] = True
                jitter = np.where(axes, sgn * off * h, rng.random(3) * h * 0.9 + 0.05 * h)
                pts.append(base + jitter - np.where(axes, 0.0, 0.5 * h))
    x = np.array(pts)
    n = len(x)
    v = rng.normal(0, 4e5, size=(n, 3))
    ps = np.ascontiguousarray(np.concatenate([x, v], axis=1))
    # start each particle in the element the oracle's own tracking puts it in (walk from floor())
    elem0 = workloads._elem_of_uniform(mesh, x)
    cfg = capi.make_config(2, capi.PIC_TRACK_TRIA, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64,
                           [(workloads.Q_ELECTRON, workloads.M_ELECTRON, 1e5)], n)
    e_dof = np.zeros((mesh.n_elems, mesh.n_dof, 3))
    ms = capi.MeshStruct(mesh)
    st = oracle_lib.OracleState(ps, elem0, np.ones(n, np.int32), is_new=np.zeros(n, np.uint8))
    PSo = np.zeros((mesh.n_elems, mesh.n_dof, 4))
    oracle_lib.step(cfg, ms, e_dof, st, 1e-13, 2, PSo)       # tiny steps: particles stay near the faces
    loop = ParticleLoop(cfg, mesh)
    loop.set_field(e_dof)
    loop.upload_particles(ps, elem0, np.ones(n, np.int32), is_new=np.zeros(n, np.uint8))
    PSg = np.zeros_like(PSo)
    loop.time_step(1e-13, 2, PSg)
    g = loop.download_particles()
    loop.close()
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)


def test_mixed_error_per_step_plasma_wave(gpu_lib):
    """Mixed vs FP64 on the plasma wave, every step: rho, E at particles, x and v stay within the
    mixed variant's budget and element ids never differ."""
    from piclas_gb300 import precision_report
    w = workloads.plasma_wave(n_cells=8, N=3, n_particles=20000, nsteps=10, seed=3)
    rows = precision_report.mixed_vs_fp64_per_step(w, 10)
    assert len(rows) == 10
    for r in rows:
        assert r["rho"] <= 1e-6, r
        assert r["E"] <= 1e-5, r
        assert r["v"] <= 1e-5, r
        assert r["x_m"] <= 1e-9, r
        assert r["elem_mismatch"] == 0, r


@pytest.mark.parametrize("N", [1, 2])
def test_sf_gather_low_order(gpu_lib, oracle_lib, N):
    """Shape-function gather for N = 1, 2 (8 and 27 DOFs per element: one DOF half, four particle
    parities per CTA) in FP64 and mixed against the oracle."""
    w = workloads.curved_two_species(n_cells=5, N=N, n_per_species=1500, seed=11, nsteps=2)
    g = _run_gpu(w, 2)
    st, PS = _run_oracle(oracle_lib, w, 2)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["PS"], PS) <= 1e-12
    gm = _run_gpu(w, 2, precision=capi.PIC_PREC_MIXED)
    assert np.array_equal(gm["elem"], st.elem)
    assert _rho_err_species(oracle_lib, w, st, gm["PS"], PS) <= 1e-6


# ---- particle boundaries: open and reflective walls --------------------------------------------
def _wall_workload(seed=21, n=6000):
    mesh = build_box_mesh(5, 5, 5, 2, bc=("reflective", "open", "periodic"))
    return workloads.plasma_wave(mesh=mesh, n_particles=n, T_eV=2000.0, seed=seed, dt=2e-10)


@pytest.mark.parametrize("bulge,shear,dep", [(0.2, 0.0, capi.PIC_DEPO_CVWM), (0.15, 0.1, capi.PIC_DEPO_CVWM),
                                              (0.2, 0.0, capi.PIC_DEPO_SHAPE_FUNCTION_CC)])
def test_tria_walls_nonplanar_fp64_bitexact(gpu_lib, oracle_lib, bulge, shear, dep):
    """TriaTracking against bulged/sheared walls (each wall side as its two triangles, IntersectionWithWall):
    bit-exact against the oracle, with cell_volweight_mean and shape_function_cc."""
    mesh = build_box_mesh(5, 5, 5, 2, perturb=0.03, bc=("reflective", "open", "reflective"),
                          wall_bulge=bulge, wall_shear=shear)
    w = workloads.plasma_wave(mesh=mesh, n_particles=4000, T_eV=2000.0, seed=39, dt=2e-10)
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(39))
    w.part_state[:, :3] = x
    w.elem = e
    w.deposition = dep
    w.sf_radius = 1.5 / 5
    g = _run_gpu(w, 12)
    st, PS = _run_oracle(oracle_lib, w, 12)
    assert np.array_equal(g["inside"], st.inside) and np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    # a particle placed by the trilinear map next to a bent face can lie outside the element's triangles
    # (TriaTracking's geometry); both sides lose the same ones
    assert g["status"]["n_lost"] == st.counters.n_lost <= 3
    assert (np.sign(st.part_state[:, 3:]) != np.sign(w.part_state[:, 3:])).any(axis=1).sum() > 100
    assert (st.inside == 0).sum() > 50


def test_walls_fp64_bitexact(gpu_lib, oracle_lib):
    """Reflective x walls, open y walls, periodic z: 12 fused steps bit-exact against the oracle
    (removed particles keep their last state, inside = 0, and are not counted as lost)."""
    w = _wall_workload()
    g = _run_gpu(w, 12)
    st, PS = _run_oracle(oracle_lib, w, 12)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["n_lost"] == 0 and g["status"]["error_word"] == 0
    assert (st.inside == 0).sum() > 200                                   # the open walls removed particles
    assert (np.sign(st.part_state[:, 3]) != np.sign(w.part_state[:, 3])).sum() > 200   # reflections


def test_walls_separate_routines_and_mixed(gpu_lib, oracle_lib):
    """The same walls through pic_push + pic_track (FP64, bit-exact) and the mixed fused step."""
    w = _wall_workload(seed=22, n=3000)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    loop = ParticleLoop(cfg, w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    for _ in range(6):
        oracle_lib.save_last(st)
        oracle_lib.interpolate(cfg, ms, w.e_dof, st)
        loop.interpolate_field_to_particle()
        oracle_lib.push(cfg, st, w.dt)
        loop.push(w.dt)
        oracle_lib.track(cfg, ms, st)
        loop.perform_tracking()
    g = loop.download_particles()
    loop.close()
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    gm = _run_gpu(w, 6, precision=capi.PIC_PREC_MIXED)
    st6, PS6 = _run_oracle(oracle_lib, w, 6)
    assert abs(int(gm["inside"].sum()) - int(st6.inside.sum())) <= 2
    assert _rel(gm["PS"][..., 3], PS6[..., 3]) <= 1e-5


def test_walls_rejected_where_unsupported(gpu_lib):
    w = _wall_workload(n=100)
    cfg = capi.make_config(w.mesh.N, capi.PIC_TRACK_REFMAPPING, capi.PIC_DEPO_CVWM, capi.PIC_PREC_FP64, w.species, 100)
    with pytest.raises(PicError) as e:
        ParticleLoop(cfg, w.mesh)
    assert e.value.code == 1


# ---- shape_function_cc -----------------------------------------------------------------------------
def _cc_workload(n_cells=6, n_per_species=2000, seed=13):
    w = workloads.curved_two_species(n_cells=n_cells, n_per_species=n_per_species, seed=seed, nsteps=2)
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION_CC
    return w


def test_shape_function_cc_against_oracle(gpu_lib, oracle_lib):
    w = _cc_workload()
    g = _run_gpu(w, 2)
    st, PS = _run_oracle(oracle_lib, w, 2)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["PS"], PS) <= 1e-12
    gm = _run_gpu(w, 2, precision=capi.PIC_PREC_MIXED)
    assert _rho_err_species(oracle_lib, w, st, gm["PS"], PS) <= 1e-6
    assert g["status"]["error_word"] == 0


@pytest.mark.parametrize("prec,tol", [(capi.PIC_PREC_FP64, 1e-12), (capi.PIC_PREC_MIXED, 1e-5)])
def test_shape_function_cc_conserves_charge(gpu_lib, oracle_lib, prec, tol):
    """Charge-corrected deposition: the quadrature integral of each species' deposit equals its total
    charge (the defining property; plain shape_function misses it by the quadrature error)."""
    w = _cc_workload(n_cells=12, n_per_species=100_000, seed=5)
    ms = capi.MeshStruct(w.mesh)
    for sp in (1, 2):
        sel = w.part_species == sp
        loop = ParticleLoop(w.config(precision=prec), w.mesh)
        loop.set_field(w.e_dof)
        loop.upload_particles(w.part_state[sel], w.elem[sel], w.part_species[sel])
        PS = loop.deposition()
        loop.close()
        q = w.species[sp - 1][0] * w.species[sp - 1][2] * int(sel.sum())
        Q = oracle_lib.integrate_charge(ms, w.mesh.N, PS)
        assert abs(Q - q) <= tol * abs(q), (sp, Q, q)


def test_walls_with_resort(gpu_lib, oracle_lib):
    """Removed particles sort behind all elements at every re-sort; results stay bit-exact."""
    w = _wall_workload(seed=23, n=4000)
    g = _run_gpu(w, 12, sort_interval=3)
    st, PS = _run_oracle(oracle_lib, w, 12)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12


# ---- checkpoint layout and restart (FillParticleData / particle read-in) -------------------------
def _fill_particle_data(state, elem, inside, species, ne, offset=0):
    """FillParticleData restated in numpy: inside particles grouped by element, ascending index within."""
    idx = np.flatnonzero(inside)
    idx = idx[np.argsort(elem[idx], kind="stable")]
    pd = np.concatenate([state[idx], species[idx, None].astype(np.float64)], axis=1)
    counts = np.bincount(elem[idx] - 1, minlength=ne)
    first = offset + np.concatenate([[0], np.cumsum(counts)[:-1]])
    return pd, np.stack([first, first + counts], axis=1), idx


def test_part_data_layout_and_restart(gpu_lib):
    w = _wall_workload(seed=31, n=5000)            # open walls remove particles: holes in the caller order
    loop = ParticleLoop(w.config(), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    loop.time_step(w.dt, 6)
    g = loop.download_particles()
    pd, pi = loop.get_part_data(offset_npart=1000)
    ref_pd, ref_pi, order = _fill_particle_data(g["part_state"], g["elem"], g["inside"], w.part_species,
                                                w.mesh.n_elems, offset=1000)
    assert np.array_equal(pi, ref_pi) and np.array_equal(pd, ref_pd)
    assert pd.shape[0] == int(g["inside"].sum()) < w.n
    # restart a second context from the checkpoint; both continue identically
    loop2 = ParticleLoop(w.config(), w.mesh)
    loop2.set_field(w.e_dof)
    loop2.set_part_data(pd, pi, offset_npart=1000)
    loop.time_step(w.dt, 5)
    loop2.time_step(w.dt, 5)
    a, b = loop.download_particles(), loop2.download_particles()
    assert np.array_equal(a["part_state"][order], b["part_state"])
    assert np.array_equal(a["elem"][order], b["elem"])
    assert np.array_equal(a["inside"][order], b["inside"])
    loop.close()
    loop2.close()


def _adaptive_workload(n_cells=6, n_per_species=2000, seed=17):
    w = workloads.curved_two_species(n_cells=n_cells, n_per_species=n_per_species, seed=seed, nsteps=2)
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE
    h = 1.0 / n_cells
    w.mesh.sf_elem_radius = np.random.default_rng(seed).uniform(1.2 * h, 1.8 * h, w.mesh.n_elems)
    return w


def test_shape_function_adaptive_against_oracle(gpu_lib, oracle_lib):
    """Per-element radii between 1.2 h and 1.8 h: FP64 against the oracle, mixed rho within 1e-6 of the
    species-summed magnitude."""
    w = _adaptive_workload()
    g = _run_gpu(w, 2)
    st, PS = _run_oracle(oracle_lib, w, 2)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["PS"], PS) <= 1e-12
    gm = _run_gpu(w, 2, precision=capi.PIC_PREC_MIXED)
    assert _rho_err_species(oracle_lib, w, st, gm["PS"], PS) <= 1e-6
    assert g["status"]["error_word"] == 0


def test_shape_function_adaptive_conserves_charge(gpu_lib, oracle_lib):
    w = _adaptive_workload(n_cells=10, n_per_species=50_000, seed=6)
    ms = capi.MeshStruct(w.mesh)
    for prec, tol in ((capi.PIC_PREC_FP64, 1e-12), (capi.PIC_PREC_MIXED, 1e-5)):
        loop = ParticleLoop(w.config(precision=prec), w.mesh)
        loop.set_field(w.e_dof)
        sel = w.part_species == 1
        loop.upload_particles(w.part_state[sel], w.elem[sel], w.part_species[sel])
        PS = loop.deposition()
        loop.close()
        q = w.species[0][0] * w.species[0][2] * int(sel.sum())
        assert abs(oracle_lib.integrate_charge(ms, w.mesh.N, PS) - q) <= tol * abs(q)


def test_fp64_fma_rate_probe(gpu_lib):
    """The FP64 peak the FP64-bound kernels are compared against: a plausible GB300 figure (nominal
    1.25 TFLOP/s) that repeats within 10 %."""
    w = workloads.plasma_wave(n_cells=2, N=1, n_particles=10)
    loop = ParticleLoop(w.config(), w.mesh)
    r1, r2 = loop.fp64_fma_rate(), loop.fp64_fma_rate()
    loop.close()
    assert 200.0 < r1 < 20000.0, r1
    assert abs(r1 - r2) <= 0.1 * max(r1, r2), (r1, r2)


def test_fp32_fma_rate_probe(gpu_lib):
    """The FP32 peak the mixed kernels are compared against: plausible for GB300 (nominal 152 SMs x 128 lanes
    x 2 FLOP x 2.07 GHz = 80.5 TFLOP/s), repeatable within 10 %, far above the FP64 rate."""
    w = workloads.plasma_wave(n_cells=2, N=1, n_particles=10)
    loop = ParticleLoop(w.config(), w.mesh)
    r1, r2 = loop.fp32_fma_rate(), loop.fp32_fma_rate()
    r64 = loop.fp64_fma_rate()
    loop.close()
    assert 10000.0 < r1 < 200000.0, r1
    assert abs(r1 - r2) <= 0.1 * max(r1, r2), (r1, r2)
    assert r1 > 20.0 * r64


# ---- parity at the benchmark configurations --------------------------------------------------------
def test_plasma_wave_full_size_100_steps_bitexact(gpu_lib, oracle_lib):
    """The plasma-wave case as benchmarked (8^3, N=3, 200k electrons, 100 steps, re-sorting every 10):
    FP64 element ids, positions and velocities bit-identical to the oracle after 100 steps."""
    import os
    w = workloads.plasma_wave()
    g = _run_gpu(w, w.nsteps, sort_interval=10)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, w.nsteps, PS, os.cpu_count() or 1)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["n_lost"] == 0


def test_curved_32cube_mesh_parity(gpu_lib, oracle_lib):
    """The benchmark's 32^3 curved mesh (RefTracking + shape function, B_z = 0.1 T) with 400k particles,
    2 steps: element ids exact, state and PartSource as in the small-mesh test; mixed rho within 1e-6."""
    import os
    w = workloads.curved_two_species(n_per_species=200_000, seed=9, nsteps=2)
    g = _run_gpu(w, 2)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.map_particles(cfg, ms, st, os.cpu_count() or 1)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, 2, PS, os.cpu_count() or 1)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-13
    assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-13
    assert _rel(g["PS"], PS) <= 1e-12
    # the mixed variant on the same mesh and particles: element ids exact, rho within 1e-6 of the
    # species-summed magnitude
    gm = _run_gpu(w, 2, precision=capi.PIC_PREC_MIXED)
    assert np.array_equal(gm["elem"], st.elem)
    assert _rho_err_species(oracle_lib, w, st, gm["PS"], PS, os.cpu_count() or 1) <= 1e-6



# ---- fault injection on the host: bad inputs come back as error codes or status bits ---------------
def test_nan_upload_rejected(gpu_lib):
    w = workloads.plasma_wave(n_cells=4, N=2, n_particles=2000, seed=41)
    loop = ParticleLoop(w.config(), w.mesh)
    bad = w.part_state.copy()
    bad[5, 4] = np.nan
    with pytest.raises(PicError) as e:
        loop.upload_particles(bad, w.elem, w.part_species)
    assert e.value.code == 1
    loop.close()


@pytest.mark.parametrize("prec", [capi.PIC_PREC_FP64, capi.PIC_PREC_MIXED])
@pytest.mark.parametrize("fused", [True, False])
def test_non_finite_field_removes_particles(gpu_lib, prec, fused):
    """A field solve that diverged (Inf in one element's DOFs): the particles in that element leave the
    loop with PIC_STATUS_NOT_FINITE; every other particle and PartSource stay finite."""
    w = workloads.plasma_wave(n_cells=4, N=2, n_particles=4000, seed=43)
    hot = 7                                             # 0-based element with the diverged field
    e_bad = w.e_dof.copy()
    e_bad[hot] = np.inf
    loop = ParticleLoop(w.config(precision=prec), w.mesh)
    loop.set_field(e_bad)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    in_hot = w.elem == hot + 1
    assert in_hot.any()
    if fused:
        loop.time_step(w.dt, 1)
    else:
        loop.interpolate_field_to_particle()
        loop.push(w.dt)
        loop.perform_tracking()
    st = loop.status()
    g = loop.download_particles()
    assert st["error_word"] & capi.PIC_STATUS_NOT_FINITE
    assert st["n_inside"] == w.n - int(in_hot.sum())
    assert not g["inside"][in_hot].any() and g["inside"][~in_hot].all()
    assert np.isfinite(g["part_state"][~in_hot]).all()
    loop.set_field(w.e_dof)                             # the next field is sane again
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    loop.time_step(w.dt, 2, PS)
    assert np.isfinite(PS).all() and loop.status()["n_inside"] == w.n - int(in_hot.sum())
    loop.close()


def test_wrong_start_element_matches_oracle(gpu_lib, oracle_lib):
    """Particles uploaded with an element that does not contain them: TriaTracking walks (or loses) them
    exactly as the oracle does, and the deposition's inverse-distance fallback for failed Newton calls gives
    the oracle's PartSource."""
    w = workloads.plasma_wave(n_cells=4, N=2, n_particles=3000, seed=47)
    wrong = w.elem.copy()
    wrong[:40] = (wrong[:40] % w.mesh.n_elems) + 1
    w2 = workloads.Workload(**{**w.__dict__, "elem": wrong})
    g = _run_gpu(w2, 2)
    st, PS = _run_oracle(oracle_lib, w2, 2)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert g["status"]["n_lost"] == st.counters.n_lost
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    # one step: its Deposition (before tracking) runs the Newton of the wrongly labelled particles in the
    # wrong element; where it fails, cell_volweight_mean falls back to inverse-distance weights of the
    # element's corner nodes (pic_depo_method.f90:512-539) and the interpolation to GetEMFieldDW
    # (pic_interpolation_tools.f90:458-527) -- the same PartSource and state as the oracle
    g1 = _run_gpu(w2, 1)
    st1, PS1 = _run_oracle(oracle_lib, w2, 1)
    assert st1.counters.n_newton_failed > 0
    assert g1["status"]["n_newton_failed"] > 0
    assert _rel(g1["PS"], PS1) <= 1e-12
    assert np.array_equal(g1["elem"], st1.elem) and np.array_equal(g1["part_state"], st1.part_state)


# ---- walls with RefTracking (ParticleBCTracking over planar wall sides) ------------------------------
def _ref_wall_workload(bc, seed, n=4000, perturb=0.0, cells=5, bulge=0.0, shear=0.0):
    mesh = build_box_mesh(cells, cells, cells, 2, perturb=perturb, bc=bc, wall_bulge=bulge, wall_shear=shear)
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, T_eV=2000.0, seed=seed, dt=2e-10)
    if perturb or bulge or shear:
        x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(seed))
        w.part_state[:, :3] = x
        w.elem = e
    w.tracking = capi.PIC_TRACK_REFMAPPING
    return w


@pytest.mark.parametrize("bc,perturb", [(("reflective",) * 3, 0.0), (("reflective", "open", "reflective"), 0.05),
                                        (("open", "reflective", "open"), 0.0)])
def test_reftracking_walls_fp64_bitexact(gpu_lib, oracle_lib, bc, perturb):
    w = _ref_wall_workload(bc, seed=31, perturb=perturb)
    g = _run_gpu(w, 12)
    st, PS = _run_oracle(oracle_lib, w, 12)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0 and st.counters.n_ref_tolerance == 0
    assert (np.sign(st.part_state[:, 3:]) != np.sign(w.part_state[:, 3:])).any(axis=1).sum() > 100
    if "open" in bc:
        assert (st.inside == 0).sum() > 100


def test_reftracking_walls_separate_routines_and_mixed(gpu_lib, oracle_lib):
    w = _ref_wall_workload(("reflective", "open", "reflective"), seed=32, n=3000)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    loop = ParticleLoop(cfg, w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.map_particles(cfg, ms, st)
    for _ in range(6):
        oracle_lib.save_last(st)
        oracle_lib.interpolate(cfg, ms, w.e_dof, st)
        oracle_lib.push(cfg, st, w.dt)
        oracle_lib.track(cfg, ms, st)
        loop.interpolate_field_to_particle()
        loop.push(w.dt)
        loop.perform_tracking()
    g = loop.download_particles()
    loop.close()
    assert np.array_equal(g["inside"], st.inside) and np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    gm = _run_gpu(w, 6, precision=capi.PIC_PREC_MIXED)
    assert (gm["inside"] != st.inside).sum() <= 3
    k = (gm["inside"] == 1) & (st.inside == 1)
    assert np.max(np.abs(gm["part_state"][k, :3] - st.part_state[k, :3])) < 1e-6


@pytest.mark.parametrize("bc,bulge,shear", [(("reflective",) * 3, 0.2, 0.0), (("open", "reflective", "open"), 0.2, 0.0),
                                             (("reflective", "open", "reflective"), 0.0, 0.15),
                                             (("reflective",) * 3, 0.15, 0.1)])
def test_reftracking_nonplanar_walls_fp64_bitexact(gpu_lib, oracle_lib, bc, bulge, shear):
    """Bilinear wall sides (ComputeBiLinearIntersection, CalcNormAndTangBilinear) and planar non-rectangular
    ones: 12 fused steps bit-exact against the oracle; mixed: the same particles inside, positions close."""
    w = _ref_wall_workload(bc, seed=34, perturb=0.03, bulge=bulge, shear=shear)
    g = _run_gpu(w, 12)
    st, PS = _run_oracle(oracle_lib, w, 12)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0 and st.counters.n_ref_tolerance == 0
    assert (np.sign(st.part_state[:, 3:]) != np.sign(w.part_state[:, 3:])).any(axis=1).sum() > 100
    gm = _run_gpu(w, 12, precision=capi.PIC_PREC_MIXED)
    assert (gm["inside"] != st.inside).sum() <= 3
    k = (gm["inside"] == 1) & (st.inside == 1)
    assert np.max(np.abs(gm["part_state"][k, :3] - st.part_state[k, :3])) < 1e-6


def test_reftracking_walls_rejected_where_unsupported(gpu_lib):
    w = _ref_wall_workload(("reflective", "open", "periodic"), seed=33, n=100)
    with pytest.raises(PicError) as e:
        ParticleLoop(w.config(), w.mesh)                      # periodic sides + RefTracking walls
    assert e.value.code == 1
    w = _ref_wall_workload(("reflective",) * 3, seed=33, n=100)
    w.mesh.elem_to_bc_sides = None
    with pytest.raises(PicError):
        ParticleLoop(w.config(), w.mesh)                      # no BC-element lists


# ---- shape_function next to walls (no periodic sides: no images, the kernel ends at the walls) ---------
@pytest.mark.parametrize("tracking,bc", [(capi.PIC_TRACK_REFMAPPING, ("reflective",) * 3),
                                         (capi.PIC_TRACK_TRIA, ("reflective", "open", "reflective"))])
def test_shape_function_with_walls_fp64_bitexact(gpu_lib, oracle_lib, tracking, bc):
    mesh = build_box_mesh(5, 5, 5, 2, bc=bc)
    w = workloads.plasma_wave(mesh=mesh, n_particles=3000, T_eV=2000.0, seed=35, dt=2e-10)
    w.tracking = tracking
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION
    w.sf_radius = 1.5 / 5
    g = _run_gpu(w, 8)
    st, PS = _run_oracle(oracle_lib, w, 8)
    assert np.array_equal(g["inside"], st.inside) and np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0
    gm = _run_gpu(w, 8, precision=capi.PIC_PREC_MIXED)
    assert _rel(gm["PS"][..., 3], PS[..., 3]) <= 1e-6


def test_shape_function_with_walls_needs_a_nonperiodic_mesh(gpu_lib):
    mesh = build_box_mesh(4, 4, 4, 2, bc=("reflective", "open", "periodic"))
    w = workloads.plasma_wave(mesh=mesh, n_particles=100, seed=36)
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION
    w.sf_radius = 1.5 / 4
    with pytest.raises(PicError) as e:
        ParticleLoop(w.config(), w.mesh)
    assert e.value.code == 1


# ---- shape_function_cc / _adaptive without periodic vectors (walls all round) --------------------------
@pytest.mark.parametrize("dep", [capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])
@pytest.mark.parametrize("tracking", [capi.PIC_TRACK_TRIA, capi.PIC_TRACK_REFMAPPING])
def test_charge_conserving_sf_with_walls_against_oracle(gpu_lib, oracle_lib, dep, tracking):
    """depoChargeOnDOFsSFChargeCon / depoChargeOnDOFsSFAdaptive: the kernel cut by the walls (adaptive: also
    by the node neighbours of the particle's element) and renormalised to q MPF; FP64 within 1e-12 of the
    oracle's maximum, mixed within 1e-6, particles and elements bit-exact."""
    mesh = build_box_mesh(5, 5, 5, 2, bc=("reflective", "open", "reflective"))
    w = workloads.plasma_wave(mesh=mesh, n_particles=3000, T_eV=2000.0, seed=37, dt=2e-10)
    w.tracking, w.deposition = tracking, dep
    w.sf_radius = 1.5 / 5
    h = 1.0 / 5
    w.mesh.sf_elem_radius = np.random.default_rng(37).uniform(1.2 * h, 2.4 * h, mesh.n_elems)
    g = _run_gpu(w, 6)
    st, PS = _run_oracle(oracle_lib, w, 6)
    assert np.array_equal(g["inside"], st.inside) and np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0
    gm = _run_gpu(w, 6, precision=capi.PIC_PREC_MIXED)
    assert _rel(gm["PS"][..., 3], PS[..., 3]) <= 1e-6


@pytest.mark.parametrize("dep", [capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])
def test_charge_conserving_sf_with_walls_conserves_charge(gpu_lib, oracle_lib, dep):
    mesh = build_box_mesh(8, 8, 8, 3, bc=("reflective", "reflective", "open"))
    w = workloads.plasma_wave(mesh=mesh, n_particles=100_000, seed=38)
    w.deposition = dep
    w.sf_radius = 2.0 / 8
    w.mesh.sf_elem_radius = np.random.default_rng(38).uniform(1.2 / 8, 2.0 / 8, mesh.n_elems)
    ms = capi.MeshStruct(w.mesh)
    q = w.species[0][0] * w.species[0][2] * w.n
    for prec, tol in ((capi.PIC_PREC_FP64, 1e-12), (capi.PIC_PREC_MIXED, 1e-5)):
        loop = ParticleLoop(w.config(precision=prec), w.mesh)
        loop.set_field(w.e_dof)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        PS = loop.deposition()
        loop.close()
        Q = oracle_lib.integrate_charge(ms, w.mesh.N, PS)
        assert abs(Q - q) <= tol * abs(q), (prec, Q, q)


# ---- 1D and 2D shape functions -------------------------------------------------------------------------
@pytest.mark.parametrize("dim,sf_dir,depo3d", [(1, 1, True), (1, 2, False), (2, 3, True), (2, 1, True)])
def test_shape_function_1d_2d_against_oracle(gpu_lib, oracle_lib, dim, sf_dir, depo3d):
    w = workloads.plasma_wave(n_cells=4, N=3, n_particles=3000, seed=41, T_eV=200.0)
    w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION
    w.sf_radius, w.sf_alpha = 0.3, 4
    w.sf_dim, w.sf_dir, w.sf_depo3d = dim, sf_dir, depo3d
    g = _run_gpu(w, 4)
    st, PS = _run_oracle(oracle_lib, w, 4)
    assert np.array_equal(g["elem"], st.elem) and np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    gm = _run_gpu(w, 4, precision=capi.PIC_PREC_MIXED)
    assert _rel(gm["PS"][..., 3], PS[..., 3]) <= 1e-6


@pytest.mark.parametrize("dep", [capi.PIC_DEPO_SHAPE_FUNCTION_CC, capi.PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE])
@pytest.mark.parametrize("walls,dim,sf_dir,depo3d", [(False, 1, 1, False), (False, 2, 3, True),
                                                     (True, 1, 2, True), (True, 2, 1, False)])
def test_charge_conserving_sf_1d_2d_against_oracle(gpu_lib, oracle_lib, dep, walls, dim, sf_dir, depo3d):
    """1D/2D shape_function_cc / _adaptive (periodic images or walls, charge on the volume or on the line /
    area): FP64 within 1e-12 of the oracle's maximum, mixed within 1e-6, particles bit-exact."""
    bc = ("reflective", "open", "reflective") if walls else ("periodic",) * 3
    mesh = build_box_mesh(4, 4, 4, 2, hi=(1.0, 0.5, 0.8), bc=bc)
    w = workloads.plasma_wave(mesh=mesh, n_particles=3000, seed=42, T_eV=200.0)
    w.deposition = dep
    w.sf_radius, w.sf_alpha = 0.3, 3
    w.sf_dim, w.sf_dir, w.sf_depo3d = dim, sf_dir, depo3d
    w.mesh.sf_elem_radius = np.random.default_rng(42).uniform(0.25, 0.45, mesh.n_elems)
    g = _run_gpu(w, 4)
    st, PS = _run_oracle(oracle_lib, w, 4)
    assert np.array_equal(g["elem"], st.elem) and np.array_equal(g["part_state"], st.part_state)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0
    gm = _run_gpu(w, 4, precision=capi.PIC_PREC_MIXED)
    assert _rel(gm["PS"][..., 3], PS[..., 3]) <= 1e-6


@pytest.mark.parametrize("kind", ["cvwm_tria", "sf_ref"])
def test_species_time_step_factor(gpu_lib, oracle_lib, kind):
    """Species(s)%TimeStepFactor: each species pushed with dt * factor; FP64 bit-exact against the oracle,
    mixed within one particle; the adjoint refuses it."""
    if kind == "cvwm_tria":
        w = workloads.plasma_wave(n_cells=4, N=3, n_particles=6000, seed=43, T_eV=200.0)
        q, m, mpf = w.species[0]
        w.species = [(q, m, mpf), (-q, 1836.0 * m, mpf)]
        w.part_species = np.where(np.arange(w.n) % 3 == 0, 2, 1).astype(np.int32)
    else:
        w = workloads.curved_two_species(n_cells=4, n_per_species=3000, seed=43, nsteps=4)
    w.time_step_factor = (1.0, 0.25)     # the reference allows factors in (0, 1] only
    g = _run_gpu(w, 6)
    st, PS = _run_oracle(oracle_lib, w, 6)
    assert np.array_equal(g["elem"], st.elem)
    if kind == "cvwm_tria":
        assert np.array_equal(g["part_state"], st.part_state)
    else:   # B_z = 0.1 T: the Boris rotation's tan differs in the last bit between device and host libm
        assert _rel(g["part_state"], st.part_state) <= 1e-12
    assert _rel(g["PS"], PS) <= 1e-12 and g["status"]["error_word"] == 0
    w1 = workloads.Workload(**{**w.__dict__, "time_step_factor": None})
    st1, _ = _run_oracle(oracle_lib, w1, 6)
    sp2 = w.part_species == 2
    assert not np.array_equal(st1.part_state[sp2], st.part_state[sp2])          # the factor acted
    assert np.array_equal(st1.part_state[~sp2], st.part_state[~sp2])          # frozen field: others unchanged
    gm = _run_gpu(w, 6, precision=capi.PIC_PREC_MIXED)
    assert (gm["elem"] != st.elem).sum() <= 2
    if kind == "cvwm_tria":
        loop = ParticleLoop(w.config(), w.mesh)
        loop.set_field(w.e_dof)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        with pytest.raises(PicError):
            loop.adjoint(2, w.dt, np.zeros((w.mesh.n_elems, w.mesh.n_dof)), 1.0)
        loop.close()


# ---- several live contexts -----------------------------------------------------------------------------
def test_two_contexts_interleaved(gpu_lib, oracle_lib):
    """Two contexts with different meshes, species, external fields and methods (CVWM + TriaTracking on a
    4^3 plasma wave; shape function + RefTracking with B_z on a 6^3 curved box) live at the same time, their
    steps interleaved, one of them mixed: each matches its own oracle run (FP64 bit-exact / within 1e-12,
    mixed rho within 1e-6).  Every launch carries its own context's constants, so neither sees the other's
    charges, masses, periodic vectors, field or shape-function radius."""
    wa = workloads.plasma_wave(n_cells=4, N=3, n_particles=5000, seed=51, T_eV=300.0)
    wb = workloads.curved_two_species(n_cells=6, n_per_species=2500, seed=52, nsteps=4)
    wc = workloads.curved_two_species(n_cells=6, n_per_species=2500, seed=53, nsteps=4)
    loops = []
    for w, prec in ((wa, capi.PIC_PREC_FP64), (wb, capi.PIC_PREC_FP64), (wc, capi.PIC_PREC_MIXED)):
        lp = ParticleLoop(w.config(precision=prec), w.mesh)
        lp.set_field(w.e_dof)
        lp.upload_particles(w.part_state, w.elem, w.part_species)
        loops.append(lp)
    PSs = [np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4)) for w in (wa, wb, wc)]
    for _ in range(4):
        for lp, w, PS in zip(loops, (wa, wb, wc), PSs):
            lp.time_step(w.dt, 1, PS)
    outs = [lp.download_particles(with_ref=True) for lp in loops]
    stats = [lp.status() for lp in loops]
    for lp in loops:
        lp.close()
    st_a, PS_a = _run_oracle(oracle_lib, wa, 4)
    st_b, PS_b = _run_oracle(oracle_lib, wb, 4)
    st_c, PS_c = _run_oracle(oracle_lib, wc, 4)
    assert np.array_equal(outs[0]["elem"], st_a.elem) and np.array_equal(outs[0]["part_state"], st_a.part_state)
    assert _rel(PSs[0], PS_a) <= 1e-12
    assert np.array_equal(outs[1]["elem"], st_b.elem)
    assert _rel(outs[1]["part_state"], st_b.part_state) <= 1e-13
    assert _rel(PSs[1], PS_b) <= 1e-12
    assert np.array_equal(outs[2]["elem"], st_c.elem)
    assert _rho_err_species(oracle_lib, wc, st_c, PSs[2], PS_c) <= 1e-6
    assert all(s["error_word"] == 0 for s in stats)


def test_mixed_gather_hits_in_the_kernel_shell(gpu_lib, oracle_lib):
    """The mixed shape-function gather pre-tests candidates in packed FP16 (units of R, threshold 1.05) before
    its exact FP32 test.  Particles are placed at 0.98 R ... 0.9999 R from a DOF, so every particle has
    DOFs in the outer shell of its kernel, and kept more than 2 R apart, so each DOF sees at most one
    particle: the set of DOFs that receive charge is then each particle's hit set.  That set must equal
    the FP64 oracle's (DOFs within 1e-5 R of the kernel edge excluded: FP32 and FP64 may round them
    differently, with a weight below 1e-9), and the values must agree to 1e-6 of their maximum."""
    mesh = build_box_mesh(12, 12, 12, 3)
    R = 1.5 * float(mesh.h[0])
    xg = mesh.elem_xgp.reshape(-1, 3)
    L = mesh.hi - mesh.lo
    rng = np.random.default_rng(77)
    n_shell = 0
    for trial in range(3):
        pts = []
        for _ in range(4000):
            g = xg[rng.integers(len(xg))]
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            x = g + R * rng.uniform(0.98, 0.9999) * u
            x = mesh.lo + np.mod(x - mesh.lo, L)
            if all(np.linalg.norm((x - p) - L * np.round((x - p) / L)) > 2.0 * R + 1e-9 for p in pts):
                pts.append(x)
        x = np.array(pts)
        n = len(x)
        assert n >= 25
        w = workloads.plasma_wave(mesh=mesh, n_particles=n, seed=trial)
        v = rng.normal(0.0, 1e5, size=(n, 3))
        w.part_state = np.ascontiguousarray(np.concatenate([x, v], axis=1))
        w.elem = workloads._elem_of_uniform(mesh, x)
        w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION
        w.sf_radius = R
        loop = ParticleLoop(w.config(precision=capi.PIC_PREC_MIXED), mesh)
        loop.upload_particles(w.part_state, w.elem, w.part_species)
        PSg = loop.deposition()
        loop.close()
        st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species, is_new=np.zeros(n, np.uint8))
        PSo = np.zeros_like(PSg)
        oracle_lib.deposit(w.config(), capi.MeshStruct(mesh), st, PSo)
        # exact distance of every DOF to its nearest particle (minimum image), in units of R
        d = np.full(len(xg), np.inf)
        for p in x:
            dv = xg - p
            dv -= L * np.round(dv / L)
            d = np.minimum(d, np.linalg.norm(dv, axis=1) / R)
        keep = np.abs(d - 1.0) > 1e-5
        hit_g = (PSg[..., 3].reshape(-1) != 0.0)
        hit_o = (PSo[..., 3].reshape(-1) != 0.0)
        assert np.array_equal(hit_g[keep], hit_o[keep])
        assert np.array_equal(hit_o[keep], d[keep] <= 1.0)
        h = hit_o & keep
        rg, ro = PSg[..., 3].reshape(-1)[h], PSo[..., 3].reshape(-1)[h]
        assert np.max(np.abs(rg - ro)) <= 1e-6 * np.max(np.abs(ro))
        n_shell += int(((d >= 0.98) & (d < 1.0) & keep).sum())
    assert n_shell > 2000


@pytest.mark.parametrize("case", ["1d_x-dir", "1d_x-dir-cc", "1d_x-dir-adaptive", "2d_z-dir", "2d_z-dir-cc",
                                  "2d_z-dir-adaptive"])
def test_sf_plasma_ball_kat_on_gpu(gpu_lib, oracle_lib, case):
    """The reference's shape-function plasma-ball known answers on the GPU (Plasma_Ball_Shape-function-xDir:
    1D x / 2D z kernels of shape_function, _cc and _adaptive on a 4 x 4 x 1 periodic box): the integrated
    charge, from the oracle's integral of the GPU PartSource and from pic_verify_deposited_charge, within the
    reference's tolerance (plain 5e-2 relative, charge-conserving 1e-9 C absolute); PartSource within 1e-12
    of the oracle's; mixed within the plain tolerance and, charge-conserving, within 1e-5 relative."""
    import json
    import os
    from test_oracle import sf_ball_charge_ok, sf_plasma_ball
    kat = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))
    k = kat["sf_plasma_ball"]
    mesh, cfg, ps, elem = sf_plasma_ball(kat, case)
    ms = capi.MeshStruct(mesh)
    spec = np.ones(len(elem), np.int32)
    st = oracle_lib.OracleState(ps, elem, spec)
    PSo = np.zeros((mesh.n_elems, mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PSo, os.cpu_count() or 1)
    for prec in (capi.PIC_PREC_FP64, capi.PIC_PREC_MIXED):
        cfg.precision = prec
        loop = ParticleLoop(cfg, mesh)
        loop.upload_particles(ps, elem, spec)
        PS = loop.deposition()
        num, ana = loop.verify_deposited_charge()
        loop.close()
        q = oracle_lib.integrate_charge(ms, mesh.N, PS)
        assert abs(num - q) <= 1e-12 * abs(q)
        assert abs(ana - len(elem) * k["charge_ic"] * k["mpf"]) <= 1e-12 * abs(ana)
        if prec == capi.PIC_PREC_FP64:
            assert sf_ball_charge_ok(k, case, q), (case, q)
            assert _rel(PS, PSo) <= 1e-12
        elif k["cases"][case]["tolerance_type"] == "relative":
            assert sf_ball_charge_ok(k, case, q), (case, q)
        else:
            assert abs(q - k["cases"][case]["total_charge"]) <= 1e-5 * abs(q), (case, q)


def test_mixed_reftracking_100_steps_against_fp64(gpu_lib, oracle_lib):
    """Mixed RefTracking (FP32 field and push, FP64 positions, the NGeo = 1 map in monomial form with fused
    multiply-adds for the Newton) on the curved 16^3 box over 100 steps of the benchmark's time step: element
    ids identical to the FP64 run, and PartPosRef equal, within 1e-10, to the reference Newton (oracle) at
    the mixed run's own positions."""
    w = workloads.curved_two_species(n_cells=16, n_per_species=100_000, seed=81, nsteps=100)
    g64 = _run_gpu(w, 100)
    g32 = _run_gpu(w, 100, precision=capi.PIC_PREC_MIXED)
    assert np.array_equal(g32["elem"], g64["elem"])
    assert g32["status"]["error_word"] == 0
    st = oracle_lib.OracleState(g32["part_state"], g32["elem"], w.part_species)
    oracle_lib.map_particles(w.config(), capi.MeshStruct(w.mesh), st)
    assert np.max(np.abs(g32["part_pos_ref"] - st.part_pos_ref)) <= 1e-10


# ---- RefTracking with periodic sides traced as BC sides (periodic_tracing, CartesianPeriodic = F) ---------
@pytest.mark.parametrize("bc", [("periodic", "periodic", "periodic"), ("reflective", "periodic", "periodic"),
                                ("open", "reflective", "periodic")])
def test_periodic_tracing_against_oracle(gpu_lib, oracle_lib, bc):
    """The reference's default periodic RefTracking: periodic sides are BC sides of ParticleBCTracking, a
    crossing moves the particle by the periodic vector into the neighbour element (PeriodicBoundary), also
    together with open and reflective walls.  FP64 bit-exact against the oracle over 8 fast steps on curved
    boxes; mixed within 1e-6 m of it with at most two differing element ids."""
    mesh = build_box_mesh(6, 6, 6, 2, perturb=0.05, bc=bc, periodic_tracing=True)
    w = workloads.plasma_wave(mesh=mesh, n_particles=4000, T_eV=3000.0, seed=93, dt=1e-10)
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(93))
    w.part_state[:, :3] = x
    w.elem = e
    w.tracking = capi.PIC_TRACK_REFMAPPING
    w.periodic_tracing = True
    g = _run_gpu(w, 8)
    st, PS = _run_oracle(oracle_lib, w, 8)
    assert np.array_equal(g["inside"], st.inside) and np.array_equal(g["elem"], st.elem)
    assert np.array_equal(g["part_state"], st.part_state)
    assert np.max(np.abs(g["part_pos_ref"] - st.part_pos_ref)) <= 1e-12
    assert _rel(g["PS"], PS) <= 1e-12
    assert st.counters.n_ref_tolerance == 0 and g["status"]["error_word"] == 0
    if bc[0] == "open":
        assert (st.inside == 0).sum() > 30                   # the open wall removed particles
    gm = _run_gpu(w, 8, precision=capi.PIC_PREC_MIXED)
    k = (gm["inside"] == 1) & (st.inside == 1)
    assert (gm["elem"][k] != st.elem[k]).sum() <= 2
    d = gm["part_state"][k, :3] - st.part_state[k, :3]
    d -= np.round(d)                                          # a particle may sit on either side of a period
    assert np.max(np.abs(d)) < 1e-6


def test_periodic_tracing_curved_32cube(gpu_lib, oracle_lib):
    """The benchmark's 32^3 curved mesh (RefTracking + shape function, B_z = 0.1 T) with the periodic sides
    traced as BC sides: 200k particles, 2 steps, element ids exact, state within 1e-13, PartSource within
    1e-12 of the oracle's."""
    import os
    mesh = build_box_mesh(32, 32, 32, 3, perturb=0.05, periodic_tracing=True)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=100_000, seed=94, nsteps=2)
    w.periodic_tracing = True
    g = _run_gpu(w, 2)
    cfg, ms = w.config(), capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.map_particles(cfg, ms, st, os.cpu_count() or 1)
    PS = np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4))
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, 2, PS, os.cpu_count() or 1)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-13
    assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-13
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0


# ---- the 32-instance mixed-precision batch --------------------------------------------------------------
def test_batch_instances_mixed_vs_fp64_and_concurrent(gpu_lib):
    """Eight instances of the mixed-precision batch (the batch's own meshes, amplitudes and seeds, particle
    counts capped at 200k, 30 steps): each instance's mixed charge density within 1e-6 of its FP64 run, and the
    eight mixed contexts run concurrently, each on its own stream with all launches enqueued before any
    synchronisation, end with the same element ids and states as the same contexts run one after another
    (contexts carry their own constants) and PartSource within 1e-12 (node-sum atomic order)."""
    inst = workloads.batch_instances(32)[:8]
    ws = [workloads.plasma_wave(n_cells=p["n_cells"], N=3, n_particles=min(p["n_particles"], 200_000),
                                amp=p["amp"], seed=p["seed"], nsteps=30) for p in inst]
    seq = []
    for w in ws:
        g32 = _run_gpu(w, w.nsteps, precision=capi.PIC_PREC_MIXED, sort_interval=10)
        g64 = _run_gpu(w, w.nsteps, precision=capi.PIC_PREC_FP64, sort_interval=10)
        err = float(np.max(np.abs(g32["PS"][..., 3] - g64["PS"][..., 3])) / np.max(np.abs(g64["PS"][..., 3])))
        assert err <= 1e-6, (w.mesh.n_elems, w.n, err)
        assert (g32["elem"] != g64["elem"]).sum() <= 2
        assert g32["status"]["error_word"] == 0
        seq.append(g32)
    loops, out = [], []
    for w in ws:
        lp = ParticleLoop(w.config(precision=capi.PIC_PREC_MIXED, sort_interval=10), w.mesh)
        lp.set_field(w.e_dof)
        lp.upload_particles(w.part_state, w.elem, w.part_species)
        loops.append(lp)
    for lp in loops:
        lp.synchronize()
    PSs = [np.zeros((w.mesh.n_elems, w.mesh.n_dof, 4)) for w in ws]
    for lp, w in zip(loops, ws):
        lp.time_step(w.dt, w.nsteps - 1)           # enqueued on each context's stream, no wait in between
    for lp, w, PS in zip(loops, ws, PSs):
        lp.time_step(w.dt, 1, PS)
    for lp, PS, g in zip(loops, PSs, seq):
        c = lp.download_particles()
        assert np.array_equal(c["elem"], g["elem"])
        assert np.array_equal(c["part_state"], g["part_state"])
        assert _rel(PS, g["PS"]) <= 1e-12
        lp.close()


# ---- per-element polynomial degree (p-adaption, N_DG_Mapping) ---------------------------------------------
def _p_adapted(kind, seed, n=6000, precision_fp64=True):
    from piclas_gb300.mesh import p_adaption_degrees
    nl = p_adaption_degrees(5, 5, 5, "random", 1, 3, seed=seed)
    if kind == "cvwm":          # TriaTracking on the straight-sided box
        mesh = build_box_mesh(5, 5, 5, 3, n_loc=nl)
        return workloads.plasma_wave(mesh=mesh, n_particles=n, seed=seed, T_eV=2000.0, nsteps=6)
    mesh = build_box_mesh(5, 5, 5, 3, perturb=0.05, n_loc=nl)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=n // 2, seed=seed, Te_eV=1000.0, nsteps=4)
    w.dt *= 10.0
    if kind == "cc":
        w.deposition = capi.PIC_DEPO_SHAPE_FUNCTION_CC
    return w


@pytest.mark.parametrize("kind", ["cvwm", "sf", "cc"])
def test_p_adaption_against_oracle(gpu_lib, oracle_lib, kind):
    """Degrees 1..3 at random over a curved 5^3 box (NMax = 3): the particle kernels dispatch on each element's
    degree, the node -> DOF and gather kernels run per degree group.  FP64 against the oracle: CVWM +
    TriaTracking bit-exact (elements, positions, velocities), RefTracking + shape function (B_z) elements exact
    and states within 1e-13, PartSource within 1e-12 of its maximum.  Mixed: elements within two, rho within
    1e-6 of max sum_s |rho_s|.  The integrated charge (pic_verify_deposited_charge) equals the oracle's
    element-by-element integral."""
    w = _p_adapted(kind, seed=31)
    g = _run_gpu(w, w.nsteps)
    st, PS = _run_oracle(oracle_lib, w, w.nsteps)
    assert np.array_equal(g["elem"], st.elem) and np.array_equal(g["inside"], st.inside)
    if kind == "cvwm":
        assert np.array_equal(g["part_state"], st.part_state)
    else:
        assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-13
        assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-13
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0
    assert (st.elem != w.elem).sum() > 20                 # particles crossed into elements of other degrees
    loop = ParticleLoop(w.config(), w.mesh)
    loop.upload_particles(st.part_state, st.elem, st.species, inside=st.inside, is_new=st.is_new)
    PSd = loop.deposition()
    num, _ = loop.verify_deposited_charge()
    loop.close()
    q = oracle_lib.integrate_charge(capi.MeshStruct(w.mesh), w.mesh.N, PSd)
    scale = sum(abs(w.species[s - 1][0] * w.species[s - 1][2]) * int((st.species == s).sum()) for s in np.unique(st.species))
    assert abs(num - q) <= 1e-12 * scale
    gm = _run_gpu(w, w.nsteps, precision=capi.PIC_PREC_MIXED)
    assert (gm["elem"] != st.elem).sum() <= 2
    assert _rho_err_species(oracle_lib, w, st, gm["PS"], PS) <= 1e-6


@pytest.mark.parametrize("kind", ["cvwm", "sf"])
def test_p_adaption_one_degree_equals_fixed_n_on_gpu(gpu_lib, kind):
    """A p-adapted mesh whose elements all have degree 3 runs on the GPU exactly as the uniform N = 3 mesh:
    the degree-dispatching kernels and the grouped launches give identical elements and states, and
    PartSource within 1e-12 (atomic order)."""
    res = []
    for nl in (None, np.full(125, 3, np.int32)):
        mesh = build_box_mesh(5, 5, 5, 3, perturb=0.05, n_loc=nl)
        if kind == "cvwm":
            w = workloads.plasma_wave(mesh=mesh, n_particles=6000, seed=8, T_eV=50.0, nsteps=4)
        else:
            w = workloads.curved_two_species(mesh=mesh, n_per_species=3000, seed=8, nsteps=4)
        res.append(_run_gpu(w, 4))
    assert np.array_equal(res[0]["elem"], res[1]["elem"])
    assert np.array_equal(res[0]["part_state"], res[1]["part_state"])
    assert _rel(res[1]["PS"].reshape(res[0]["PS"].shape), res[0]["PS"]) <= 1e-12


def test_p_adaption_rejected_by_hdg_and_adjoint(gpu_lib):
    """The HDG solve and the differentiable loop need one degree for all elements: both return
    PIC_ERR_INVALID_ARGUMENT on a p-adapted mesh (the reference builds p-adaption with HDG only on PETSc)."""
    w = _p_adapted("cvwm", seed=3, n=2000)
    loop = ParticleLoop(w.config(), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    with pytest.raises(PicError):
        loop.adjoint(2, w.dt, np.zeros(w.mesh.n_elems * loop.nd), 1.0)
    import ctypes as C
    hdg = capi.PicHdg()
    hdg.n_sides = 1
    rc = gpu_lib.pic_hdg_init(loop.handle, C.byref(hdg))
    assert rc == 1
    loop.close()


# ---- RefMappingGuess 1..4 ----------------------------------------------------------------------------------
@pytest.mark.parametrize("guess", [2, 3, 4])
@pytest.mark.parametrize("kind", ["tria", "ref", "ref_padapt"])
def test_ref_mapping_guess_against_oracle(gpu_lib, oracle_lib, guess, kind):
    """The Newton start values of GetRefNewtonStartValue on the GPU: CVWM + TriaTracking (the Newton of the
    deposition and the interpolation) bit-exact, RefTracking + shape function (B_z) on a curved box and on a
    p-adapted one with exact elements and states within 1e-13, PartPosRef within 1e-10; mixed elements within
    two of the oracle's."""
    from piclas_gb300.mesh import p_adaption_degrees
    if kind == "tria":
        w = workloads.plasma_wave(n_cells=5, N=3, n_particles=6000, seed=17, T_eV=50.0, nsteps=4)
    else:
        nl = p_adaption_degrees(5, 5, 5, "random", 1, 3, seed=5) if kind == "ref_padapt" else None
        mesh = build_box_mesh(5, 5, 5, 3, perturb=0.08, n_loc=nl)
        w = workloads.curved_two_species(mesh=mesh, n_per_species=3000, seed=17, Te_eV=1000.0, nsteps=4)
    cfg = w.config()
    cfg.ref_mapping_guess = guess
    loop = ParticleLoop(cfg, w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    PS = np.zeros(w.mesh.dof_shape(4))
    loop.time_step(w.dt, w.nsteps, PS)
    g = loop.download_particles(with_ref=True)
    loop.close()
    ms = capi.MeshStruct(w.mesh)
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    if kind != "tria":
        oracle_lib.map_particles(cfg, ms, st)
    PSo = np.zeros(w.mesh.dof_shape(4))
    oracle_lib.step(cfg, ms, w.e_dof, st, w.dt, w.nsteps, PSo)
    assert np.array_equal(g["elem"], st.elem)
    if kind == "tria":
        assert np.array_equal(g["part_state"], st.part_state)
    else:
        assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-13
        assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-13
        assert np.max(np.abs(g["part_pos_ref"] - st.part_pos_ref)) <= 1e-10
    assert _rel(PS, PSo) <= 1e-12
    cfg.precision = capi.PIC_PREC_MIXED
    lm = ParticleLoop(cfg, w.mesh)
    lm.set_field(w.e_dof)
    lm.upload_particles(w.part_state, w.elem, w.part_species)
    lm.time_step(w.dt, w.nsteps)
    gm = lm.download_particles()
    lm.close()
    assert (gm["elem"] != st.elem).sum() <= 2


# ---- curved elements (NGeo > 1) --------------------------------------------------------------------------------
def _curved_ngeo(ng, deposition, seed, n=6000, tracking=capi.PIC_TRACK_REFMAPPING):
    mesh = build_box_mesh(5, 5, 5, 3, perturb=0.08, n_geo=ng)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=n // 2, seed=seed, Te_eV=1000.0, nsteps=5)
    w.dt *= 10.0
    w.deposition = deposition
    w.tracking = tracking
    return w


@pytest.mark.parametrize("ng,dep", [(2, capi.PIC_DEPO_SHAPE_FUNCTION), (3, capi.PIC_DEPO_SHAPE_FUNCTION),
                                    (2, capi.PIC_DEPO_CVWM), (2, capi.PIC_DEPO_SHAPE_FUNCTION_CC)])
def test_curved_ngeo_against_oracle(gpu_lib, oracle_lib, ng, dep):
    """Curved elements (NGeo 2, 3): the Newton on XCL_NGeo (RefTracking, the FIBGM candidate search, the deposition
    and the interpolation) against the oracle -- elements exact, states within 1e-13, PartPosRef within 1e-10,
    PartSource within 1e-12 of its maximum; mixed: elements within two, rho within 1e-6 of max sum_s |rho_s|."""
    w = _curved_ngeo(ng, dep, seed=41)
    g = _run_gpu(w, w.nsteps)
    st, PS = _run_oracle(oracle_lib, w, w.nsteps)
    assert np.array_equal(g["elem"], st.elem) and np.array_equal(g["inside"], st.inside)
    assert _rel(g["part_state"][:, :3], st.part_state[:, :3]) <= 1e-13
    assert _rel(g["part_state"][:, 3:], st.part_state[:, 3:]) <= 1e-13
    assert np.max(np.abs(g["part_pos_ref"] - st.part_pos_ref)) <= 1e-10
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0 and (st.elem != w.elem).sum() > 20
    gm = _run_gpu(w, w.nsteps, precision=capi.PIC_PREC_MIXED)
    assert (gm["elem"] != st.elem).sum() <= 2
    assert _rho_err_species(oracle_lib, w, st, gm["PS"], PS) <= 1e-6


def test_curved_ngeo_triatracking_against_oracle(gpu_lib, oracle_lib):
    """TriaTracking + cell_volweight_mean on an NGeo = 2 box: the tracking walks the triangulated corner faces,
    the deposition and the interpolation map x -> xi with the curved Newton; against the oracle with exact
    elements, including which particles the triangulated faces lose (curved faces bulge beyond them), and states
    within 1e-13 (B_z: CUDA's tan against libm's)."""
    w = _curved_ngeo(2, capi.PIC_DEPO_CVWM, seed=43, tracking=capi.PIC_TRACK_TRIA)
    g = _run_gpu(w, w.nsteps)
    st, PS = _run_oracle(oracle_lib, w, w.nsteps)
    assert np.array_equal(g["elem"], st.elem) and np.array_equal(g["inside"], st.inside)
    assert _rel(g["part_state"], st.part_state) <= 1e-13
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["n_lost"] == st.counters.n_lost


def test_curved_ngeo_uncurved_elements_use_corner_newton(gpu_lib, oracle_lib):
    """An NGeo = 2 box without perturbation has no curved element: GetPositionInRefElem then runs the NGeo = 1
    Newton on the corners with their dXCL_NGeo; GPU and oracle agree bit-for-bit, and both agree with the
    NGeo = 1 box to rounding."""
    res = []
    for ng in (2, 1):
        mesh = build_box_mesh(5, 5, 5, 3, n_geo=ng)
        w = workloads.curved_two_species(mesh=mesh, n_per_species=3000, seed=44, Te_eV=1000.0, nsteps=4)
        g = _run_gpu(w, 4)
        st, PS = _run_oracle(oracle_lib, w, 4)
        assert np.array_equal(g["elem"], st.elem)
        assert _rel(g["part_state"], st.part_state) <= 1e-13
        res.append(g)
    assert np.array_equal(res[0]["elem"], res[1]["elem"])
    assert _rel(res[0]["part_state"], res[1]["part_state"]) <= 1e-12


@pytest.mark.parametrize("ng", [2, 3])
def test_mixed_curved_newton_against_fp64(gpu_lib, oracle_lib, ng):
    """Mixed RefTracking on curved elements maps x -> xi with the NGeo map in power form (nested Horner, fused
    multiply-adds): over 30 steps the element ids equal the FP64 run's, and PartPosRef equals, within 1e-10, the
    reference Newton (oracle, Lagrange form) at the mixed run's own positions."""
    mesh = build_box_mesh(8, 8, 8, 3, perturb=0.08, n_geo=ng)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=20_000, seed=82, nsteps=30, Te_eV=1000.0)
    w.dt *= 5.0
    g64 = _run_gpu(w, 30)
    g32 = _run_gpu(w, 30, precision=capi.PIC_PREC_MIXED)
    assert (g32["elem"] != g64["elem"]).sum() <= 2
    assert g32["status"]["error_word"] == 0 and (g64["elem"] != w.elem).sum() > 100
    st = oracle_lib.OracleState(g32["part_state"], g32["elem"], w.part_species)
    oracle_lib.map_particles(w.config(), capi.MeshStruct(w.mesh), st)
    assert np.max(np.abs(g32["part_pos_ref"] - st.part_pos_ref)) <= 1e-10


# ---- curved wall sides (NGeo > 1: Bezier clipping, BezierNewton) ------------------------------------------------
def _curved_wall_workload(bc, ng, seed, bulge=0.0, shear=0.0, perturb=0.05, n=3000):
    mesh = build_box_mesh(4, 4, 4, 2, perturb=perturb, bc=bc, wall_bulge=bulge, wall_shear=shear, n_geo=ng)
    w = workloads.plasma_wave(mesh=mesh, n_particles=n, T_eV=2000.0, seed=seed, dt=2e-10)
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(seed))
    w.part_state[:, :3] = x
    w.elem = e
    w.tracking = capi.PIC_TRACK_REFMAPPING
    return w


@pytest.mark.parametrize("bc,ng,bulge,shear", [(("reflective",) * 3, 2, 0.2, 0.0),
                                               (("reflective", "open", "reflective"), 2, 0.2, 0.0),
                                               (("reflective", "open", "reflective"), 2, 0.0, 0.3),
                                               (("open", "reflective", "reflective"), 3, 0.15, 0.1),
                                               (("reflective", "reflective", "open"), 4, 0.2, 0.0)])
def test_reftracking_curved_walls_against_oracle(gpu_lib, oracle_lib, bc, ng, bulge, shear):
    """Curved wall sides of an NGeo = 2, 3 box: bulged faces (SideType CURVED, Bezier clipping) and sheared planar
    faces (PLANAR_CURVED, BezierNewton), reflective and open, 12 fused steps against the oracle -- the same
    particles inside, the same elements, states within 1e-13, PartSource within 1e-12 of its maximum, no status
    bit; mixed: the same particles inside but three, positions within 1e-6."""
    w = _curved_wall_workload(bc, ng, seed=51, bulge=bulge, shear=shear)
    g = _run_gpu(w, 12)
    st, PS = _run_oracle(oracle_lib, w, 12)
    assert np.array_equal(g["inside"], st.inside)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["part_state"], st.part_state) <= 1e-13
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0 and st.counters.n_ref_tolerance == 0 and st.counters.n_lost == 0
    assert (np.sign(st.part_state[:, 3:]) != np.sign(w.part_state[:, 3:])).any(axis=1).sum() > 100
    if "open" in bc:
        assert (st.inside == 0).sum() > 100
    gm = _run_gpu(w, 12, precision=capi.PIC_PREC_MIXED)
    assert (gm["inside"] != st.inside).sum() <= 3
    k = (gm["inside"] == 1) & (st.inside == 1)
    assert np.max(np.abs(gm["part_state"][k, :3] - st.part_state[k, :3])) < 1e-6


def test_reftracking_curved_periodic_tracing_against_oracle(gpu_lib, oracle_lib):
    """CartesianPeriodic = F on a curved NGeo = 2 box: the periodic sides are BC sides of the RefTracking lists
    (PLANAR_RECT faces of curved elements), together with a bulged reflective wall pair (CURVED); 8 steps against
    the oracle with the same elements and particles inside, states within 1e-13, no status bit."""
    mesh = build_box_mesh(6, 6, 6, 2, perturb=0.05, bc=("reflective", "periodic", "periodic"), wall_bulge=0.2,
                          n_geo=2, periodic_tracing=True)
    w = workloads.plasma_wave(mesh=mesh, n_particles=4000, T_eV=3000.0, seed=52, dt=1e-10)
    x, e, _ = workloads._uniform_in_mesh(mesh, w.n, np.random.default_rng(52))
    w.part_state[:, :3] = x
    w.elem = e
    w.tracking = capi.PIC_TRACK_REFMAPPING
    w.periodic_tracing = True
    g = _run_gpu(w, 8)
    st, PS = _run_oracle(oracle_lib, w, 8)
    assert np.array_equal(g["elem"], st.elem) and np.array_equal(g["inside"], st.inside)
    assert _rel(g["part_state"], st.part_state) <= 1e-13
    assert _rel(g["PS"], PS) <= 1e-12
    assert st.counters.n_hop_limit == 0 and st.counters.n_ref_tolerance == 0
    assert g["status"]["error_word"] == 0 and (st.elem != w.elem).sum() > 200


def test_reftracking_curved_walls_need_the_bezier_sides(gpu_lib):
    w = _curved_wall_workload(("reflective",) * 3, 2, seed=53, bulge=0.2, n=100)
    w.mesh.side_bezier = None
    with pytest.raises(PicError) as e:
        ParticleLoop(w.config(), w.mesh)
    assert e.value.code == 1 and "side_bezier" in str(e.value)


# ---- FP64 shape-function gather: particles covering the target's DOFs enter through moments ----------------------
@pytest.mark.parametrize("N,radius_cells", [(3, 1.5), (3, 3.0), (2, 3.0), (1, 2.0)])
def test_sf_gather_moments_against_oracle(gpu_lib, oracle_lib, N, radius_cells):
    """The FP64 gather sums the particles whose kernel covers every DOF of the target element (or, at N = 3, of
    one DOF half) as moments of (A_p + B_g + p'.g)^2 instead of per (particle, DOF) hit: at R = 3 h most of the
    hits go that way, at R = 1.5 h about a quarter.  PartSource within 1e-12 of the oracle's per-hit sum, the
    same for the deposition of a single step (no tracking between) and for 4 fused steps."""
    mesh = build_box_mesh(6, 6, 6, N, perturb=0.05)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=3000, seed=61, Te_eV=1000.0, nsteps=4,
                                     sf_radius_cells=radius_cells)
    cfg, ms = w.config(), capi.MeshStruct(mesh)
    loop = ParticleLoop(cfg, mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species)
    PSg = loop.deposition()
    loop.close()
    st = oracle_lib.OracleState(w.part_state, w.elem, w.part_species)
    oracle_lib.map_particles(cfg, ms, st)
    PSo = np.zeros(mesh.dof_shape(4))
    oracle_lib.deposit(cfg, ms, st, PSo)
    assert _rel(PSg, PSo) <= 1e-12
    g = _run_gpu(w, 4, dt=2e-11)
    st, PS = _run_oracle(oracle_lib, w, 4, dt=2e-11)
    assert np.array_equal(g["elem"], st.elem)
    assert _rel(g["PS"], PS) <= 1e-12
    assert g["status"]["error_word"] == 0


def test_mixed_newton_far_from_origin(gpu_lib, oracle_lib):
    """The mixed Newton works in double-FP32 on each element's map relative to its barycentre: on a box 1000 m from
    the origin (h = 1/8 m) 20 mixed steps keep the FP64 run's element ids but two, and PartPosRef equals the
    reference Newton (oracle) at the mixed run's own positions within 1e-10."""
    mesh = build_box_mesh(8, 8, 8, 3, lo=(1000.0, -500.0, 250.0), hi=(1001.0, -499.0, 251.0), perturb=0.08)
    w = workloads.curved_two_species(mesh=mesh, n_per_species=20_000, seed=83, nsteps=20, Te_eV=1000.0)
    w.dt *= 5.0
    g64 = _run_gpu(w, 20)
    g32 = _run_gpu(w, 20, precision=capi.PIC_PREC_MIXED)
    assert (g32["elem"] != g64["elem"]).sum() <= 2
    assert g32["status"]["error_word"] == 0 and (g64["elem"] != w.elem).sum() > 100
    st = oracle_lib.OracleState(g32["part_state"], g32["elem"], w.part_species)
    oracle_lib.map_particles(w.config(), capi.MeshStruct(w.mesh), st)
    assert np.max(np.abs(g32["part_pos_ref"] - st.part_pos_ref)) <= 1e-10
