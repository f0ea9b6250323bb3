"""Differentiable loop: the hand-written adjoint (pic_adjoint_run) against central finite differences
of its own FP64 forward (h = 1e-6), FP32 against FP64 gradients, checkpoint invariance, and a
torch.autograd.Function wrapper (test harness only).

Tolerances: FP64 adjoint vs central FD <= 1e-5 relative (directional derivatives over all particles
along gradient-shaped directions, and d/d|B|); FP32 adjoint vs FP64 adjoint <= 1e-3 (norm-wise; the FP32 forward itself drifts);
checkpoint intervals 1 / 10 / 50 agree to 1e-10 (only atomic summation order differs)."""
import numpy as np
import pytest

from piclas_gb300 import PIC_PREC_FP64, PIC_PREC_MIXED, ParticleLoop, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(gpu_lib):
    w = workloads.differentiable_loop()
    loop = ParticleLoop(w.config(), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    yield w, loop
    loop.close()


def _adj(loop, w, **kw):
    return loop.adjoint(w.nsteps, w.dt, w.info["rho_target"], w.info["rho_scale"], **kw)


def test_adjoint_vs_central_fd(case):
    """Directional central differences along two gradient-shaped directions: d = g and d = g * U(0.5, 1.5)
    (per-component weights, so an error in any single component shows).  Each direction is scaled so
    that particles move by about h * sigma_v; a random direction would give a derivative of 3M cancelling
    terms, below the summation-order noise of the loss."""
    w, loop = case
    L0, gv, gB = _adj(loop, w, checkpoint_every=10, precision=PIC_PREC_FP64)
    assert np.isfinite(L0) and np.all(np.isfinite(gv)) and np.isfinite(gB)
    rng = np.random.default_rng(7)
    sigma = workloads.maxwell_sigma(1.0, workloads.M_ELECTRON)
    h = 1e-6
    rms = float(np.sqrt(np.mean(gv * gv)))
    for d in (gv * (sigma / rms), gv * rng.uniform(0.5, 1.5, size=gv.shape) * (sigma / rms)):
        Ls = []
        for s in (+1, -1):
            ps = w.part_state.copy()
            ps[:, 3:] += s * h * d
            loop.upload_particles(ps, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
            Ls.append(_adj(loop, w, gradients=False))
        fd = (Ls[0] - Ls[1]) / (2 * h)
        ad = float(np.sum(gv * d))
        assert abs(fd - ad) <= 1e-5 * abs(fd), (fd, ad, L0)
    loop.upload_particles(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    # d/d|B| through the B scale factor
    Bz = w.info["Bz"]
    Lp = _adj(loop, w, gradients=False, b_scale=1 + h)
    Lm = _adj(loop, w, gradients=False, b_scale=1 - h)
    fdB = (Lp - Lm) / (2 * h * Bz)
    assert abs(fdB - gB) <= 1e-5 * abs(fdB), (fdB, gB)


def test_fp32_adjoint_against_fp64(case):
    w, loop = case
    _, g64, b64 = _adj(loop, w, precision=PIC_PREC_FP64)
    _, g32, b32 = _adj(loop, w, precision=PIC_PREC_MIXED)
    rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    assert rel <= 1e-3, rel
    assert abs(b32 - b64) <= 1e-3 * abs(b64), (b32, b64)


def test_checkpoint_interval_invariance(case):
    w, loop = case
    ref = _adj(loop, w, checkpoint_every=10)
    for k in (1, 50):
        L, g, b = _adj(loop, w, checkpoint_every=k)
        assert abs(L - ref[0]) <= 1e-12 * abs(ref[0])
        assert np.linalg.norm(g - ref[1]) <= 1e-10 * np.linalg.norm(ref[1])
        assert abs(b - ref[2]) <= 1e-10 * abs(ref[2])


def test_torch_autograd_wrapper(case):
    torch = pytest.importorskip("torch")
    w, loop = case

    class PicLoss(torch.autograd.Function):
        """loss(v0, |B|) of the differentiable loop; backward = pic_adjoint_run's reverse pass."""

        @staticmethod
        def forward(ctx, v0, b_scale):
            ps = w.part_state.copy()
            ps[:, 3:] = v0.detach().cpu().numpy()
            loop.upload_particles(ps, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
            L, gv, gb = _adj(loop, w, b_scale=float(b_scale))
            ctx.save_for_backward(torch.from_numpy(gv), torch.tensor(gb * w.info["Bz"], dtype=torch.float64))
            return torch.tensor(L, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            gv, gb = ctx.saved_tensors
            return gout * gv, gout * gb

    v0 = torch.tensor(w.part_state[:, 3:], dtype=torch.float64, requires_grad=True)
    b = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    loss = PicLoss.apply(v0, b)
    loss.backward()
    L, gv, gb = _adj(loop, w)
    assert abs(loss.item() - L) <= 1e-12 * abs(L)
    # a fresh upload regroups particles, so atomic summation order (and the last bits) may differ
    assert np.linalg.norm(v0.grad.numpy() - gv) <= 1e-9 * np.linalg.norm(gv)
    assert abs(b.grad.item() - gb * w.info["Bz"]) <= 1e-9 * abs(gb * w.info["Bz"])


def test_adjoint_forward_matches_oracle(gpu_lib, oracle_lib):
    """The adjoint's forward pass is the reference loop: its loss equals the loss of the oracle's nsteps of
    interpolation + Boris push + TriaTracking (B scaled by b_scale, IsNewPart off) followed by
    cell_volweight_mean deposition of the final state, and of the GPU's own pic_step + pic_deposit on the
    same inputs.  FP64 within 1e-12; FP32 within 2e-6 relative.  The FP32 bound is the loss's
    sensitivity: dL/L ~ 2 max|d rho^| / |rho^ - target| with |rho^ - target| ~ 0.2 here (particle noise),
    so 2e-6 on the loss holds rho^ to about 2e-7."""
    import os
    from piclas_gb300 import capi
    w = workloads.differentiable_loop(n_cells=8, N=2, n_particles=20000, nsteps=20, seed=3)
    b_scale = 1.3
    tgt, rs = w.info["rho_target"], w.info["rho_scale"]
    loop = ParticleLoop(w.config(), w.mesh)
    loop.set_field(w.e_dof)
    loop.upload_particles(w.part_state, w.elem, w.part_species, is_new=np.zeros(w.n, np.uint8))
    L64 = loop.adjoint(w.nsteps, w.dt, tgt, rs, b_scale=b_scale, checkpoint_every=5, gradients=False)
    L32 = loop.adjoint(w.nsteps, w.dt, tgt, rs, b_scale=b_scale, checkpoint_every=5, precision=PIC_PREC_MIXED,
                       gradients=False)
    loop.close()
    ext = list(w.external_field)
    ext[3:] = [b * b_scale for b in ext[3:]]
    w2 = workloads.Workload(**{**w.__dict__, "external_field": tuple(ext)})
    cfg, ms, nt = w2.config(), capi.MeshStruct(w2.mesh), os.cpu_count() or 1
    st = oracle_lib.OracleState(w2.part_state, w2.elem, w2.part_species, is_new=np.zeros(w2.n, np.uint8))
    oracle_lib.step(cfg, ms, w2.e_dof, st, w2.dt, w2.nsteps, None, nt)
    PS = np.zeros((w2.mesh.n_elems, w2.mesh.n_dof, 4))
    oracle_lib.deposit(cfg, ms, st, PS, nt)
    Lo = float(np.sum((PS[..., 3] / rs - tgt) ** 2))
    assert st.counters.n_lost == 0
    assert abs(L64 - Lo) <= 1e-12 * Lo, (L64, Lo)
    assert abs(L32 - Lo) <= 2e-6 * Lo, (L32, Lo)
    # the same through the drop-in loop
    lp = ParticleLoop(w2.config(), w2.mesh)
    lp.set_field(w2.e_dof)
    lp.upload_particles(w2.part_state, w2.elem, w2.part_species, is_new=np.zeros(w2.n, np.uint8))
    lp.time_step(w2.dt, w2.nsteps)
    PSg = lp.deposition()
    lp.close()
    Lg = float(np.sum((PSg[..., 3] / rs - tgt) ** 2))
    assert abs(Lg - Lo) <= 1e-12 * Lo, (Lg, Lo)
