"""Side connectivity, metric terms and field boundaries of a box mesh for the HDG Poisson solve.

The reference's HDG solver (src/hdg/) reads, besides sJ and the Gauss nodes:
  * ``ElemToSide(E2S_SIDE_ID/E2S_FLIP, 1:6, nElems)`` and ``SideToElem(1:5, nSides)``
    (src/mesh/mesh_vars.f90; numbering: boundary sides first, src/readIMD/ or HOPR order),
  * ``N_VolMesh(e)%Metrics_fTilde/gTilde/hTilde(1:3,0:N,0:N,0:N)`` = J grad(xi), J grad(eta), J grad(zeta)
    (src/mesh/metrics.f90:157-330),
  * the Dirichlet side list ``DirichletBC`` and, for BCType 2/5-8, the face Gauss points ``Face_xGP``
    to evaluate the boundary potential (src/hdg/hdg.f90:466-520, src/hdg/hdg_linear.f90:96-150).

This module derives them for :func:`piclas_gb300.mesh.build_box_mesh` meshes.  The metric terms are
the cross-product form ``Ja^1 = x_eta x x_zeta`` (cyclic) of the trilinear map at the Gauss points;
the reference's default curl form gives the same values for affine elements and, for trilinear
elements, the same polynomial (degree <= 2 per direction) whenever N >= 2.
Side-local coordinates follow the CGNS convention of ``CGNS_VolToSide`` and ``Flip_S2M``
(src/mesh/mapping.f90:147-278): a slave side's flip is derived from the geometry and checked against
the node-based flip of the particle mesh.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import SIDE_IS_PLUS, BoxMesh, lagrange_polys

FIELD_BCS = ("periodic", "dirichlet", "neumann")
# local sides 1..6 = zeta-, eta-, xi+, eta+, xi-, zeta+ (piclas.h: ZETA_MINUS=1 ... ZETA_PLUS=6)
_BACK = {0: 5, 5: 0, 1: 3, 3: 1, 2: 4, 4: 2}


@dataclass
class HdgMesh:
    """HDG arrays of one mesh, 1-based ids like the reference."""
    n_sides: int
    elem_to_side: np.ndarray        # (2,6,nElems) -> C [e][s][2]: SideID (1-based), flip
    side_to_elem: np.ndarray        # (5,nSides)   -> C [side][5]: elem, nb elem, loc side, nb loc side, flip (-1 = none)
    metrics_f: np.ndarray           # (3,0:N,0:N,0:N,nElems) -> C [e][k][j][i][3]
    metrics_g: np.ndarray
    metrics_h: np.ndarray
    sj: np.ndarray                  # (0:N,0:N,0:N,nElems)  -> C [e][k][j][i]
    dirichlet_sides: np.ndarray     # (nDirichlet) 1-based SideIDs
    neumann_sides: np.ndarray       # (nNeumann)   1-based SideIDs (BCType 10: zero gradient)
    face_xgp: np.ndarray            # (3,0:N,0:N,nSides) -> C [side][q][p][3], master side coordinates
    field_bc: tuple


def cgns_vol_to_side(N: int, i: int, j: int, k: int, s: int):
    """CGNS_VolToSide (mapping.f90:205-240) for the 0-based local side s: (p, q, normal index)."""
    return [(j, i, k), (i, k, j), (j, k, N - i), (N - i, k, N - j), (k, j, i), (i, j, N - k)][s]


def flip_s2m(N: int, p: int, q: int, flip: int):
    """Flip_S2M (mapping.f90:147-179): slave side coordinates -> master side coordinates."""
    return [(p, q), (q, p), (N - p, q), (N - q, N - p), (p, N - q)][flip]


def _face_xi(N: int, xgp, s: int, p: int, q: int):
    """Reference coordinates of the side point with CGNS coordinates (p, q) of local side s."""
    return [(xgp[q], xgp[p], -1.0), (xgp[p], -1.0, xgp[q]), (1.0, xgp[p], xgp[q]),
            (xgp[N - p], 1.0, xgp[q]), (-1.0, xgp[q], xgp[p]), (xgp[p], xgp[q], 1.0)][s]


def _map(mesh: BoxMesh, elems: np.ndarray, xi):
    """x(xi) of the trilinear map of every element in ``elems`` (0-based), shape (len, 3)."""
    La = lagrange_polys(float(xi[0]), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo)
    Lb = lagrange_polys(float(xi[1]), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo)
    Lc = lagrange_polys(float(xi[2]), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo)
    xc = mesh.xcl_ngeo[elems]
    x = np.zeros((len(elems), 3))
    for c in range(2):
        for b in range(2):
            for a in range(2):
                x = x + xc[:, c, b, a] * (La[a] * Lb[b] * Lc[c])
    return x


def metric_terms(mesh: BoxMesh):
    """(Metrics_fTilde, Metrics_gTilde, Metrics_hTilde) at the Gauss points, C [e][k][j][i][3]."""
    N = mesh.N
    nd = N + 1
    ne = mesh.n_elems
    lg = [lagrange_polys(float(x), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo) for x in mesh.xgp]
    f = np.zeros((ne, nd, nd, nd, 3))
    g = np.zeros_like(f)
    h = np.zeros_like(f)
    for k in range(nd):
        for j in range(nd):
            for i in range(nd):
                J = np.zeros((ne, 3, 3))             # [nn][dd] = d x_nn / d xi_dd
                for c in range(2):
                    for b in range(2):
                        for a in range(2):
                            J = J + mesh.dxcl_ngeo[:, c, b, a, :, :] * (lg[i][a] * lg[j][b] * lg[k][c])
                xs, ys, zs = J[:, :, 0], J[:, :, 1], J[:, :, 2]
                f[:, k, j, i] = np.cross(ys, zs)
                g[:, k, j, i] = np.cross(zs, xs)
                h[:, k, j, i] = np.cross(xs, ys)
    return f, g, h


def build_hdg_mesh(mesh: BoxMesh, field_bc=None) -> HdgMesh:
    """Unique sides (boundary sides first, then inner sides at their master element), flips,
    metric terms and boundary lists.  ``field_bc`` per axis: "periodic" (only where the mesh is
    periodic), "dirichlet" or "neumann"; default: periodic where the mesh is, else Dirichlet."""
    N = mesh.N
    nd = N + 1
    ne = mesh.n_elems
    periodic = tuple(b == "periodic" for b in mesh.bc)
    if field_bc is None:
        field_bc = tuple("periodic" if p else "dirichlet" for p in periodic)
    field_bc = tuple(field_bc)
    if len(field_bc) != 3 or any(b not in FIELD_BCS for b in field_bc):
        raise ValueError(f"field_bc must hold one of {FIELD_BCS} per axis, got {field_bc}")
    for d in range(3):
        if (field_bc[d] == "periodic") != periodic[d]:
            raise ValueError(f"axis {d}: field boundary {field_bc[d]!r} does not match the mesh ({mesh.bc[d]!r})")
    axis_of_side = (2, 1, 0, 1, 0, 2)

    side_id = -np.ones((ne, 6), dtype=np.int64)
    owners = []          # per unique side: [(elem, locside, flip), ...] master first
    bc_kind = []
    # boundary sides first (SideID 1..nBCSides), element order
    for e in range(ne):
        for s in range(6):
            if mesh.side_nb_elem[e, s] == 0:
                side_id[e, s] = len(owners)
                owners.append([(e, s, 0)])
                bc_kind.append(field_bc[axis_of_side[s]])
    # inner (and periodic) sides, numbered at their master (the + side of the pair)
    for e in range(ne):
        for s in range(6):
            if mesh.side_nb_elem[e, s] != 0 and SIDE_IS_PLUS[s]:
                side_id[e, s] = len(owners)
                owners.append([(e, s, 0)])
                bc_kind.append("inner")
    for e in range(ne):
        for s in range(6):
            if mesh.side_nb_elem[e, s] != 0 and not SIDE_IS_PLUS[s]:
                en = int(mesh.side_nb_elem[e, s]) - 1
                sid = side_id[en, _BACK[s]]
                assert sid >= 0
                side_id[e, s] = sid
                owners[sid].append((e, s, int(mesh.side_flip[e, s])))
    n_sides = len(owners)

    # geometric check of the slave flips: the master point (p,q) is the slave point Flip_S2M^-1(p,q)
    # (every flip is its own inverse), up to a periodic shift; checked at the four corners of each side
    pv = mesh.periodic_vectors
    shifts = [np.zeros(3)] + [sg * pv[:, k] for k in range(pv.shape[1]) for sg in (1.0, -1.0)]
    pairs = [(sid, o[0][0], o[0][1], o[1][0], o[1][1], o[1][2]) for sid, o in enumerate(owners) if len(o) > 1]
    groups = {}
    for sid, em, sm, es, ss, fl in pairs:
        groups.setdefault((sm, ss, fl), []).append((em, es))
    tol = 1e-12 * max(1.0, float(np.abs(mesh.node_coords).max()))
    for (sm, ss, fl), lst in groups.items():
        em = np.array([a for a, _ in lst])
        es = np.array([b for _, b in lst])
        for q in (0, N):
            for p in (0, N):
                ps, qs = flip_s2m(N, p, q, fl)
                xm = _map(mesh, em, _face_xi(N, mesh.xgp, sm, p, q))
                xs = _map(mesh, es, _face_xi(N, mesh.xgp, ss, ps, qs))
                ok = np.zeros(len(lst), dtype=bool)
                for sh in shifts:
                    ok |= np.all(np.abs(xm - xs - sh) <= tol, axis=1)
                assert ok.all(), f"flip {fl} does not map the slave face onto the master face (sides {sm},{ss})"

    e2s = np.zeros((ne, 6, 2), dtype=np.int32)
    s2e = -np.ones((n_sides, 5), dtype=np.int32)
    for sid, own in enumerate(owners):
        em, sm, _ = own[0]
        s2e[sid, 0] = em + 1
        s2e[sid, 2] = sm + 1
        s2e[sid, 4] = 0
        e2s[em, sm] = (sid + 1, 0)
        if len(own) > 1:
            es, ss, fl = own[1]
            s2e[sid, 1] = es + 1
            s2e[sid, 3] = ss + 1
            s2e[sid, 4] = fl
            e2s[es, ss] = (sid + 1, fl)

    f, g, h = metric_terms(mesh)
    face = np.zeros((n_sides, nd, nd, 3))
    master_e = np.array([o[0][0] for o in owners])
    master_s = np.array([o[0][1] for o in owners])
    for sm in range(6):
        sel = np.nonzero(master_s == sm)[0]
        if len(sel) == 0:
            continue
        for q in range(nd):
            for p in range(nd):
                face[sel, q, p] = _map(mesh, master_e[sel], _face_xi(N, mesh.xgp, sm, p, q))
    dirichlet = np.array([sid + 1 for sid in range(n_sides) if bc_kind[sid] == "dirichlet"], dtype=np.int32)
    neumann = np.array([sid + 1 for sid in range(n_sides) if bc_kind[sid] == "neumann"], dtype=np.int32)
    return HdgMesh(n_sides=n_sides, elem_to_side=e2s, side_to_elem=s2e,
                   metrics_f=np.ascontiguousarray(f), metrics_g=np.ascontiguousarray(g),
                   metrics_h=np.ascontiguousarray(h), sj=np.ascontiguousarray(mesh.elem_sj),
                   dirichlet_sides=dirichlet, neumann_sides=neumann, face_xgp=face, field_bc=field_bc)


# ---- exact functions of the reference's Poisson test cases (src/equations/poisson/equation.f90) -----
def exact_func_105(x):
    """IniExactFunc 105, the 3D periodic test case: phi = sin(x+1) sin(y+2) sin(z+3)."""
    x = np.asarray(x)
    return np.sin(x[..., 0] + 1.0) * np.sin(x[..., 1] + 2.0) * np.sin(x[..., 2] + 3.0)


def source_105(x):
    """CalcSourceHDG for IniExactFunc 105 (equation.f90:975-977): -3 sin(x+1) sin(y+2) sin(z+3)."""
    x = np.asarray(x)
    return -3.0 * np.sin(x[..., 0] + 1.0) * np.sin(x[..., 1] + 2.0) * np.sin(x[..., 2] + 3.0)


def grad_105(x):
    """Gradient of phi_105, for E = -grad(phi)."""
    x = np.asarray(x)
    a, b, c = x[..., 0] + 1.0, x[..., 1] + 2.0, x[..., 2] + 3.0
    return np.stack([np.cos(a) * np.sin(b) * np.sin(c), np.sin(a) * np.cos(b) * np.sin(c),
                     np.sin(a) * np.sin(b) * np.cos(c)], axis=-1)
