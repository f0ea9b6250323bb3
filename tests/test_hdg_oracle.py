"""The oracle's HDG Poisson solve against analytic solutions (CPU only).

Pins: the reference's own HDG test cases are analytic -- CHE_poisson_periodic (IniExactFunc 105 on the
periodic box (0, 2pi)^3, N = 3, 4^3 elements, epsCG 1e-12, PrecondType 0 and 2; its .h5 reference state is
unreadable here) and NIG_convtest_poisson (h-convergence rate of the L2 error).  The discrete solution
must approach the exact one at the rate of a degree-N method; E = -grad(phi) is checked as well.
"""
import numpy as np
import pytest

import oracle
from piclas_gb300.hdg_mesh import build_hdg_mesh, exact_func_105, grad_105, source_105
from piclas_gb300.mesh import build_box_mesh

L2PI = 6.283185306          # li of the reference's periodic test mesh (hopr.ini)


def _solve(mesh, fbc=None, precond=2, eps=1e-12, phi_exact=exact_func_105, src=source_105):
    h = build_hdg_mesh(mesh, fbc)
    o = oracle.HdgOracle(mesh, h)
    lam_d = None
    if len(h.dirichlet_sides):
        lam_d = phi_exact(h.face_xgp[h.dirichlet_sides - 1]).reshape(len(h.dirichlet_sides), -1)
    U, E, it, nrm, rc = o.solve(src(mesh.elem_xgp), precond_type=precond, eps_cg=eps, lambda_dirichlet=lam_d)
    assert rc == 0, rc
    return h, o, U.reshape(mesh.elem_xgp.shape[:-1]), E.reshape(mesh.elem_xgp.shape), it


def test_periodic_exact_func_105_like_the_reference_case():
    errs = []
    for n in (2, 4):
        m = build_box_mesh(n, n, n, 3, hi=(L2PI, L2PI, L2PI))
        for pt in (0, 2):
            h, o, U, E, it = _solve(m, precond=pt)
            ph = exact_func_105(m.elem_xgp)
            c = float((ph - U).mean())                       # the pinned DOF fixes the constant
            ephi = float(np.abs(U + c - ph).max())
            eE = float(np.abs(E + grad_105(m.elem_xgp)).max())
            assert it > 0
            if pt == 0:
                errs.append((ephi, eE))
    (p2, e2), (p4, e4) = errs
    assert p4 < 2e-3 and e4 < 3e-3
    assert np.log2(p2 / p4) > 3.5 and np.log2(e2 / e4) > 3.0      # degree-3 method: order 4 in phi


def test_dirichlet_box_convergence_straight_and_curved():
    for pert in (0.0, 0.1):
        errs = []
        for n in (2, 4):
            m = build_box_mesh(n, n, n, 3, lo=(-1, -1, -1), hi=(1, 1, 1), perturb=pert, bc=("open",) * 3)
            h, o, U, E, it = _solve(m)
            assert len(h.dirichlet_sides) == 6 * n * n
            errs.append(float(np.abs(U - exact_func_105(m.elem_xgp)).max()))
        assert errs[1] < 1e-5 and np.log2(errs[0] / errs[1]) > 3.5


def test_mixed_periodic_dirichlet_neumann():
    """x periodic, y Dirichlet, z zero-gradient Neumann: phi = sin(x+1) sin(y+2) cos(z) on (0,2pi)^2 x (0,pi)."""
    def phi(x):
        return np.sin(x[..., 0] + 1.0) * np.sin(x[..., 1] + 2.0) * np.cos(x[..., 2])

    def src(x):
        return -3.0 * phi(x)

    errs = []
    for n in (2, 4):
        m = build_box_mesh(n, n, n, 3, hi=(L2PI, L2PI, np.pi), bc=("periodic", "reflective", "open"))
        h, o, U, E, it = _solve(m, fbc=("periodic", "dirichlet", "neumann"), phi_exact=phi, src=src)
        assert len(h.neumann_sides) == 2 * n * n
        errs.append(float(np.abs(U - phi(m.elem_xgp)).max()))
    assert errs[1] < 5e-3 and np.log2(errs[0] / errs[1]) > 3.0


@pytest.mark.parametrize("N", [1, 2, 4])
def test_other_degrees_converge(N):
    errs = []
    for n in (2, 4):
        m = build_box_mesh(n, n, n, N, lo=(-1, -1, -1), hi=(1, 1, 1), bc=("open",) * 3)
        h, o, U, E, it = _solve(m, precond=1)
        errs.append(float(np.abs(U - exact_func_105(m.elem_xgp)).max()))
    assert np.log2(errs[0] / errs[1]) > N + 0.5


def test_element_matrices_properties():
    m = build_box_mesh(3, 2, 2, 3, perturb=0.08)
    h = build_hdg_mesh(m)
    o = oracle.HdgOracle(m, h)
    # Smat(a,b,iS,jS) = Smat(b,a,jS,iS); InvDhat symmetric, negative definite
    assert np.abs(o.smat - o.smat.transpose(0, 2, 1, 4, 3)).max() <= 1e-15 * np.abs(o.smat).max()
    assert np.array_equal(o.inv_dhat, o.inv_dhat.transpose(0, 2, 1))
    assert np.all(np.linalg.eigvalsh(o.inv_dhat[0]) < 0)
    # Tau = 2 / vol^(1/3) with vol = the element volume
    vol = np.einsum("ekji,i,j,k->e", 1.0 / m.elem_sj, m.wgp, m.wgp, m.wgp)
    assert np.allclose(o.tau, 2.0 / np.cbrt(vol), rtol=1e-14)
    # the trace operator has the constants in its kernel on a periodic box (rows of Smat sum to ~0
    # once the two elements of every side are added): S * 1 = 0
    ones = np.ones((h.n_sides, (m.N + 1) ** 2))
    y = np.zeros_like(ones)
    for e in range(m.n_elems):
        for jl in range(6):
            sid = h.elem_to_side[e, jl, 0] - 1
            for loc in range(6):
                # Smat(a,b,jl,loc) = smat[e, loc, jl, b, a]
                y[sid] += o.smat[e, loc, jl].T @ ones[h.elem_to_side[e, loc, 0] - 1]
    assert np.abs(y).max() < 1e-10 * np.abs(o.smat).max()


def test_all_preconditioners_agree():
    m = build_box_mesh(3, 3, 3, 2, lo=(-1, -1, -1), hi=(1, 1, 1), perturb=0.05, bc=("open",) * 3)
    sols = [_solve(m, precond=pt)[2] for pt in (0, 1, 2)]
    assert np.abs(sols[0] - sols[1]).max() < 1e-9 and np.abs(sols[0] - sols[2]).max() < 1e-9
