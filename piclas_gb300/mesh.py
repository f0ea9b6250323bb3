"""Structured hexahedral box meshes in the layout the PICLas particle loop consumes.

The reference reads HOPR ``.h5`` meshes and derives, at init, the arrays the particle
loop reads (``XCL_NGeo``, ``dXCL_NGeo``, side/node maps, ``NodeVolume``, periodic node
twins, the FIBGM background mesh ...).  This module generates the same arrays directly
for a periodic box of ``nx*ny*nz`` linear (NGeo=1) hexahedra, optionally with the interior
nodes displaced (curved-box test mesh).  Every array is returned in the reference's
Fortran memory order (first index fastest), so it can be handed to ``pic_create`` as is.

Reference routines restated (paths relative to the PICLas source tree):
  * Gauss / Chebyshev-Lobatto nodes, barycentric weights, Lagrange polynomials:
    src/interpolation/basis.f90:643-688, 719-754, 758-833, 952-976, 1011-1035, 1223-1264
  * dXCL_NGeo: src/mesh/metrics.f90:309-318;  sJ at Gauss points: metrics.f90 (1/detJac)
  * ElemBaryNGeo: src/particles/particle_mesh/particle_mesh_build.f90:1446-1466
  * XiEtaZetaBasis / slenXiEtaZetaBasis / ElemRadiusNGeo: particle_mesh_build.f90:1625-1678
  * ElemEpsOneCell: particle_mesh_build.f90:607-617
  * ElemSideNodeID / ConcaveElemSide: src/particles/particle_mesh/particle_mesh_tools.f90:1877-1930
  * CGNS corner map: src/mesh/mesh_tools.f90:728-769;  ElemNodeID: mesh_tools.f90:634-696
  * NodeVolume: src/particles/pic/deposition/pic_depo_tools.f90:224-355
  * Periodic node twins: src/particles/pic/deposition/pic_depo.f90:1218-2089
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

EPS_MACH = float(np.finfo(np.float64).eps)   # PP_RealTolerance = EPSILON(1.0D0)

# CGNS corner c (1..8) -> tensor-product corner index a + 2b + 4c (0-based), NGeo = 1.
# CNS(1:8) = 1, 2, 4, 3, 5, 6, 8, 7 (mesh_tools.f90:748-755) minus one.
CGNS_TO_TENSOR = (0, 1, 3, 2, 4, 5, 7, 6)
# NodeMapCGNS(1:4, side) in CGNS corner numbers (mesh_tools.f90:760-765)
SIDE_CGNS = ((1, 4, 3, 2), (1, 2, 6, 5), (2, 3, 7, 6), (3, 4, 8, 7), (1, 5, 8, 4), (5, 6, 7, 8))
# neighbour offset (di, dj, dk) of local sides 1..6 (zeta-, eta-, xi+, eta+, xi-, zeta+)
SIDE_OFFSET = ((0, 0, -1), (0, -1, 0), (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, 0, 1))
SIDE_DIR = (2, 1, 0, 1, 0, 2)          # axis normal to each local side
SIDE_IS_PLUS = (False, False, True, True, False, True)


# --------------------------------------------------------------------------------------
# 1D basis (basis.f90)
# --------------------------------------------------------------------------------------
def almost_equal_unity(x: float, y: float) -> bool:
    """ALMOSTEQUAL_UNITY, basis.f90:1011-1035."""
    if x == 0.0 or y == 0.0:
        return abs(x - y) <= 2.0 * EPS_MACH
    return abs(x - y) <= EPS_MACH * abs(x) and abs(x - y) <= EPS_MACH * abs(y)


def lagrange_polys(x: float, xgp, wbary):
    """LagrangeInterpolationPolys, basis.f90:1223-1264 (barycentric form, node-hit branch)."""
    n = len(xgp)
    L = [0.0] * n
    hit = False
    for i in range(n):
        if almost_equal_unity(x, float(xgp[i])):
            L[i] = 1.0
            hit = True
    if hit:
        return L
    s = 0.0
    for i in range(n):
        L[i] = float(wbary[i]) / (x - float(xgp[i]))
        s = s + L[i]
    return [L[i] / s for i in range(n)]


def barycentric_weights(xgp):
    """BarycentricWeights, basis.f90:952-976."""
    n = len(xgp)
    w = [1.0] * n
    for i in range(1, n):
        for j in range(i):
            w[j] = w[j] * (xgp[j] - xgp[i])
            w[i] = w[i] * (xgp[i] - xgp[j])
    return [1.0 / v for v in w]


def _legendre_and_derivative(n: int, x: float):
    """LegendrePolynomialAndDerivative, basis.f90:643-688 (normalised)."""
    if n == 0:
        L, Ld = 1.0, 0.0
    elif n == 1:
        L, Ld = x, 1.0
    else:
        Lm2, Lm1, Ldm2, Ldm1 = 1.0, x, 0.0, 1.0
        L = Ld = 0.0
        for i in range(2, n + 1):
            L = (float(2 * i - 1) * x * Lm1 - float(i - 1) * Lm2) / float(i)
            Ld = Ldm2 + float(2 * i - 1) * Lm1
            Lm2, Lm1 = Lm1, L
            Ldm2, Ldm1 = Ldm1, Ld
    s = math.sqrt(float(n) + 0.5)
    return L * s, Ld * s


def legendre_gauss_nodes(n: int):
    """LegendreGaussNodesAndWeights, basis.f90:758-833 (Newton from Chebyshev guesses)."""
    x = [0.0] * (n + 1)
    w = [0.0] * (n + 1)
    if n == 0:
        return [0.0], [2.0]
    if n == 1:
        x[0] = -math.sqrt(1.0 / 3.0)
        x[1] = -x[0]
        return x, [1.0, 1.0]
    tol = 1.0e-15
    cheb = 2.0 * math.atan(1.0) / float(n + 1)
    for i in range((n + 1) // 2):
        x[i] = -math.cos(cheb * float(2 * i + 1))
        for _ in range(11):
            L, Ld = _legendre_and_derivative(n + 1, x[i])
            dx = -L / Ld
            x[i] = x[i] + dx
            if abs(dx) < tol * abs(x[i]):
                break
        L, Ld = _legendre_and_derivative(n + 1, x[i])
        x[n - i] = -x[i]
        w[i] = (2.0 * n + 3) / ((1.0 - x[i] * x[i]) * Ld * Ld)
        w[n - i] = w[i]
    if n % 2 == 0:
        x[n // 2] = 0.0
        L, Ld = _legendre_and_derivative(n + 1, 0.0)
        w[n // 2] = (2.0 * n + 3) / (Ld * Ld)
    return x, w


def cheby_gauss_lobatto_nodes(n: int):
    """ChebyGaussLobNodesAndWeights, basis.f90:719-754 (nodes only)."""
    if n == 0:
        return [0.0]
    return [-math.cos(float(i) / float(n) * math.acos(-1.0)) for i in range(n + 1)]


# --------------------------------------------------------------------------------------
# mesh container
# --------------------------------------------------------------------------------------
@dataclass
class BoxMesh:
    """Arrays of a periodic hex box in reference (Fortran) memory order.

    Index arrays are 1-based like the reference.  ``shape`` comments use Fortran notation.
    """
    nx: int
    ny: int
    nz: int
    N: int
    lo: np.ndarray
    hi: np.ndarray
    n_elems: int
    n_nodes: int
    n_geo: int
    periodic_vectors: np.ndarray          # (3, nPeriodicVectors): column k = PeriodicVectors(:,k)
    xi_cl_ngeo: np.ndarray
    wbary_cl_ngeo: np.ndarray
    xgp: np.ndarray
    wgp: np.ndarray
    wbary_gp: np.ndarray
    xcl_ngeo: np.ndarray                  # (3,0:NGeo,0:NGeo,0:NGeo,nElems) -> C [e][c][b][a][3]
    dxcl_ngeo: np.ndarray                 # (3,3,0:NGeo,0:NGeo,0:NGeo,nElems) -> C [e][c][b][a][nn][dd]
    elem_bary: np.ndarray                 # (3,nElems)
    xez_basis: np.ndarray                 # (3,6,nElems)
    slen_basis: np.ndarray                # (6,nElems)
    elem_radius: np.ndarray               # (nElems)
    eps_one_cell: np.ndarray              # (nElems)
    elem_xgp: np.ndarray                  # (3,0:N,0:N,0:N,nElems) -> C [e][k][j][i][3]; with n_loc: packed (nDofs, 3)
    elem_sj: np.ndarray                   # (0:N,0:N,0:N,nElems); with n_loc: packed (nDofs)
    node_coords: np.ndarray               # (3,8*nElems): tensor-ordered element corners
    elem_node: np.ndarray                 # (8,nElems) CGNS order, 1-based into node_coords
    elem_side_node: np.ndarray            # (4,6,nElems) 1-based into node_coords
    side_nb_elem: np.ndarray              # (6,nElems) 1-based
    side_pvid: np.ndarray                 # (6,nElems)
    side_flip: np.ndarray                 # (6,nElems) SIDE_FLIP (0 for master sides)
    concave_side: np.ndarray              # (6,nElems)
    node_info: np.ndarray                 # (8,nElems) unique node ids, 1-based
    unique_node_coords: np.ndarray        # (3,nUniqueNodes)
    node_volume: np.ndarray               # (nUniqueNodes)
    periodic_n_nodes: np.ndarray
    periodic_offset: np.ndarray
    periodic_nodes: np.ndarray            # 1-based
    fibgm_imax: tuple
    fibgm_deltas: np.ndarray
    fibgm_n_elems: np.ndarray             # (imax,jmax,kmax) -> C [k][j][i]
    fibgm_offset: np.ndarray
    fibgm_element: np.ndarray             # 1-based
    canonical_node: np.ndarray = field(default=None)  # 0-based periodic-unique id per unique node
    side_bc: np.ndarray = field(default=None)         # (6,nElems) 1 open / 2 reflective wall, 0 otherwise; None: no walls
    bc: tuple = ("periodic", "periodic", "periodic")  # particle boundary per axis
    sf_elem_radius: np.ndarray = field(default=None)  # SFElemr2_Shared(1,:) for shape_function_adaptive
    # RefTracking with walls: BuildBCElemDistance output (see build_bc_elem_distance)
    n_loc: np.ndarray = field(default=None)          # per-element degree Nloc (p-adaption); None: N everywhere
    elem_curved: np.ndarray = field(default=None)    # ElemCurved (0/1) of an NGeo > 1 mesh; None at NGeo = 1
    side_bezier: np.ndarray = field(default=None)    # NGeo > 1: BezierControlPoints3D per (element, local side) [e][s][q][p][3]
    side_type: np.ndarray = field(default=None)      # NGeo > 1: SideType per (element, local side) (PLANAR_RECT 0 .. CURVED 4)
    dof_offset: np.ndarray = field(default=None)     # N_DG_Mapping(1,:): 0-based DOF offset of each element (nElems+1)
    elem_to_bc_sides: np.ndarray = field(default=None)
    bc_side_elem_loc: np.ndarray = field(default=None)
    bc_side_distance: np.ndarray = field(default=None)

    @property
    def n_dof(self) -> int:
        """(N+1)^3: the DOFs per element (with n_loc: of an element of the largest degree)."""
        return (self.N + 1) ** 3

    @property
    def n_dofs(self) -> int:
        """nDofsMapping: the DOFs of all elements."""
        return int(self.dof_offset[-1]) if self.n_loc is not None else self.n_elems * self.n_dof

    def dof_shape(self, ncomp: int) -> tuple:
        """Shape of a per-DOF array with ncomp components: (nElems, (N+1)^3, ncomp), or packed (nDofs, ncomp)."""
        return (self.n_dofs, ncomp) if self.n_loc is not None else (self.n_elems, self.n_dof, ncomp)

    def elem_dofs(self, a: np.ndarray, e: int) -> np.ndarray:
        """The (Nloc+1)^3 DOFs of element e (0-based) of a per-DOF array in either layout, as rows (DOF, component)."""
        if self.n_loc is None:
            return a.reshape(self.n_elems, self.n_dof, -1)[e]
        return a.reshape(self.n_dofs, -1)[self.dof_offset[e]:self.dof_offset[e + 1]]

    @property
    def n_dg_mapping(self) -> np.ndarray | None:
        """N_DG_Mapping(1:3, nElems): DOF offset, Nloc, compute-node offset (= the DOF offset on one process)."""
        if self.n_loc is None:
            return None
        off = self.dof_offset[:-1]
        return np.ascontiguousarray(np.stack([off, self.n_loc, off], axis=1), dtype=np.int32)

    @property
    def n_inter(self) -> np.ndarray | None:
        """N_Inter(Nloc)%xGP, %wGP, %wBary for Nloc = 1..N, one block of 3 (Nloc+1) values per degree."""
        if self.n_loc is None:
            return None
        out = []
        for k in range(1, self.N + 1):
            xg, wg = legendre_gauss_nodes(k)
            out += [np.asarray(xg), np.asarray(wg), np.asarray(barycentric_weights(xg))]
        return np.ascontiguousarray(np.concatenate(out), dtype=np.float64)

    @property
    def h(self) -> np.ndarray:
        return (self.hi - self.lo) / np.array([self.nx, self.ny, self.nz], dtype=np.float64)

    def elem_index(self, i, j, k):
        return i + self.nx * (j + self.ny * k)


def _wrap(v, n):
    return v % n


WALL_BC = {"open": 1, "reflective": 2}      # PartBound%TargetBoundCond


def build_box_mesh(nx: int, ny: int, nz: int, N: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0),
                   perturb: float = 0.0, refmapping_eps: float = 1.0e-4,
                   bc=("periodic", "periodic", "periodic"), bc_halo_eps: float | None = None,
                   wall_bulge: float = 0.0, wall_shear: float = 0.0, periodic_tracing: bool = False,
                   n_loc=None, n_geo: int = 1) -> BoxMesh:
    """Build a box of nx*ny*nz NGeo=1 hexahedra with DG degree N.

    ``n_loc`` (p-adaption): the degree Nloc of every element (1..N, N is then NMax); the DOF arrays are then
    packed element by element (N_DG_Mapping offsets), and NodeVolume and ElemEpsOneCell use each element's Nloc.
    ``n_geo`` > 1: curved elements of geometry degree NGeo -- XCL_NGeo at the Chebyshev-Gauss-Lobatto points of
    each element, displaced by the same smooth ``perturb`` field as the grid nodes (so the faces are curved,
    conforming and periodic), with dXCL_NGeo from the CL derivative matrix, ElemCurved, ElemRadiusNGeo from the
    sides' Bezier control points and the FIBGM from the elements' Bezier bounding boxes (periodic boxes only).

    ``perturb`` displaces every interior node by ``perturb*h*sin(2 pi x)sin(2 pi y)sin(2 pi z)``
    along each axis (h per axis); boundary nodes stay put so the periodic faces match.
    ``bc`` gives the particle boundary of both faces of each axis: "periodic" (a periodic vector, node
    twins for cell_volweight_mean), "open" or "reflective" (wall sides without a neighbour: SIDE_NBELEMID
    = 0, master orientation, convex).  Without periodic axes the BC-element lists of RefTracking are
    built with halo ``bc_halo_eps`` (default: the largest element extent); with ``periodic_tracing``
    (CartesianPeriodic = F) they include the periodic sides, and walls may be combined with periodic axes.
    ``wall_bulge`` moves the nodes of each open/reflective face inwards along its normal by
    ``wall_bulge*h*sin(pi u)sin(pi v)`` (u, v in [0,1] across the face): the wall sides become bilinear
    (SideType BILINEAR; at NGeo > 1 curved, CURVED, with the CL points inside the wall elements moved by the
    same bump fading linearly across the element layer).  ``wall_shear`` moves them within the face plane by
    ``wall_shear*h`` times the same bump along the first in-plane axis: planar sides that are no longer
    rectangles (PLANAR_NONRECT; at NGeo > 1 PLANAR_CURVED).  The face edges stay put.
    """
    bc = tuple(bc)
    if n_geo < 1 or n_geo > 4:
        raise ValueError("n_geo must be 1..4")

    if len(bc) != 3 or any(b not in ("periodic", "open", "reflective") for b in bc):
        raise ValueError(f"bc must hold 'periodic', 'open' or 'reflective' per axis, got {bc}")
    periodic = [b == "periodic" for b in bc]
    pv_index = {d: q + 1 for q, d in enumerate([d for d in range(3) if periodic[d]])}   # 1-based vector id
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    L = hi - lo
    hvec = L / np.array([nx, ny, nz], dtype=np.float64)
    ne = nx * ny * nz

    # ---- unique (periodic copies distinct) grid nodes --------------------------------
    gi = np.arange(nx + 1, dtype=np.float64)
    gj = np.arange(ny + 1, dtype=np.float64)
    gk = np.arange(nz + 1, dtype=np.float64)
    X = np.empty((nz + 1, ny + 1, nx + 1, 3), dtype=np.float64)
    X[..., 0] = lo[0] + gi[None, None, :] * hvec[0]
    X[..., 1] = lo[1] + gj[None, :, None] * hvec[1]
    X[..., 2] = lo[2] + gk[:, None, None] * hvec[2]
    X[:, :, nx, 0] = hi[0]
    X[:, ny, :, 1] = hi[1]
    X[nz, :, :, 2] = hi[2]
    if perturb != 0.0:
        interior = np.zeros((nz + 1, ny + 1, nx + 1), dtype=bool)
        interior[1:nz, 1:ny, 1:nx] = True
        s = (np.sin(2.0 * np.pi * (X[..., 0] - lo[0]) / L[0]) * np.sin(2.0 * np.pi * (X[..., 1] - lo[1]) / L[1])
             * np.sin(2.0 * np.pi * (X[..., 2] - lo[2]) / L[2]))
        for d in range(3):
            X[..., d] = np.where(interior, X[..., d] + perturb * hvec[d] * s, X[..., d])
    if wall_bulge != 0.0 or wall_shear != 0.0:
        U = [(X[..., d] - lo[d]) / L[d] for d in range(3)]
        for d in range(3):
            if periodic[d]:
                continue
            o1, o2 = [a for a in range(3) if a != d]
            bump = np.sin(np.pi * U[o1]) * np.sin(np.pi * U[o2])
            for face, sign in ((0, 1.0), (-1, -1.0)):
                sl = [slice(None)] * 3
                sl[2 - d] = face                       # X is indexed [k][j][i]
                sl = tuple(sl)
                b = bump[sl]
                X[sl + (d,)] = X[sl + (d,)] + sign * wall_bulge * hvec[d] * b
                X[sl + (o1,)] = X[sl + (o1,)] + wall_shear * hvec[o1] * b
    n_unique = (nx + 1) * (ny + 1) * (nz + 1)

    def uid(i, j, k):  # 0-based unique node id of grid node (i,j,k)
        return i + (nx + 1) * (j + (ny + 1) * k)

    unique_coords = np.ascontiguousarray(X.reshape(-1, 3))

    # ---- element corners (tensor order a + 2b + 4c) ---------------------------------
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei = ei.transpose(2, 1, 0).reshape(-1)   # element e = i + nx*(j + ny*k)
    ej = ej.transpose(2, 1, 0).reshape(-1)
    ek = ek.transpose(2, 1, 0).reshape(-1)
    corner_uid = np.empty((ne, 8), dtype=np.int64)
    xcl = np.empty((ne, 2, 2, 2, 3), dtype=np.float64)    # [e][c][b][a][3]
    for c in range(2):
        for b in range(2):
            for a in range(2):
                t = a + 2 * b + 4 * c
                corner_uid[:, t] = uid(ei + a, ej + b, ek + c)
                xcl[:, c, b, a, :] = unique_coords[corner_uid[:, t]]
    node_coords = np.ascontiguousarray(xcl.reshape(ne, 8, 3))   # NodeCoords_Shared(1:3, 8e+t+1)

    # ---- reference-element data ------------------------------------------------------
    ng1 = n_geo + 1
    xi_cl = cheby_gauss_lobatto_nodes(n_geo)
    wb_cl = barycentric_weights(xi_cl)
    xgp, wgp = legendre_gauss_nodes(N)
    wb_gp = barycentric_weights(xgp)
    if n_geo > 1:
        # XCL_NGeo: the unperturbed position of every CL point of the element, moved by the perturbation field
        # (points on the domain boundary stay put); the corner points coincide with the grid nodes above
        t = 0.5 * (np.asarray(xi_cl) + 1.0)
        xcl = np.empty((ne, ng1, ng1, ng1, 3))
        idx = np.stack([ei, ej, ek], axis=1).astype(np.float64)
        dims_f = np.array([nx, ny, nz], dtype=np.float64)
        for c in range(ng1):
            for b in range(ng1):
                for a in range(ng1):
                    g = idx + np.array([t[a], t[b], t[c]])          # grid-index coordinates
                    p0 = lo + g * hvec
                    p0 = np.where(g >= dims_f, hi, p0)
                    if perturb != 0.0:
                        inner = np.all((g > 0.0) & (g < dims_f), axis=1)
                        sv = (np.sin(2.0 * np.pi * (p0[:, 0] - lo[0]) / L[0]) * np.sin(2.0 * np.pi * (p0[:, 1] - lo[1]) / L[1])
                              * np.sin(2.0 * np.pi * (p0[:, 2] - lo[2]) / L[2]))
                        p0 = np.where(inner[:, None], p0 + perturb * hvec[None, :] * sv[:, None], p0)
                    if wall_bulge != 0.0 or wall_shear != 0.0:
                        # the wall faces' bump, as for the grid nodes: along the wall normal and within the plane,
                        # fading linearly to zero across the wall element layer (grid index distance 1), so that the
                        # CL points inside a wall element follow the face and no element folds over
                        U = (p0 - lo) / L
                        p0 = p0.copy()
                        for d in range(3):
                            if periodic[d]:
                                continue
                            o1, o2 = [q for q in range(3) if q != d]
                            bump = np.sin(np.pi * U[:, o1]) * np.sin(np.pi * U[:, o2])
                            wlo = np.clip(1.0 - g[:, d], 0.0, 1.0)
                            whi = np.clip(1.0 - (dims_f[d] - g[:, d]), 0.0, 1.0)
                            for wgt, sign in ((wlo, 1.0), (whi, -1.0)):
                                p0[:, d] = p0[:, d] + sign * wall_bulge * hvec[d] * bump * wgt
                                p0[:, o1] = p0[:, o1] + wall_shear * hvec[o1] * bump * wgt
                    xcl[:, c, b, a, :] = p0
        for c in range(2):
            for b in range(2):
                for a in range(2):
                    if not np.array_equal(xcl[:, c * n_geo, b * n_geo, a * n_geo, :], node_coords[:, a + 2 * b + 4 * c, :]):
                        raise RuntimeError("curved element corners differ from the grid nodes")

    # dXCL_NGeo(dd,nn,i,j,k) = sum_l D(i,l) X(nn,l,j,k) ... (metrics.f90:309-318), D the derivative matrix of the
    # Lagrange basis on the CL points (PolynomialDerivativeMatrix: D(i,j) = w_j/w_i/(x_i-x_j), D(i,i) = -sum);
    # at NGeo = 1 D = +-0.5
    D = np.zeros((ng1, ng1))
    for i in range(ng1):
        for j in range(ng1):
            if i != j:
                D[i, j] = wb_cl[j] / wb_cl[i] / (xi_cl[i] - xi_cl[j])
        D[i, i] = -sum(D[i, j] for j in range(ng1) if j != i)
    dxcl = np.zeros((ne, ng1, ng1, ng1, 3, 3), dtype=np.float64)  # [e][c][b][a][nn][dd]
    for c in range(ng1):
        for b in range(ng1):
            for a in range(ng1):
                acc = np.zeros((ne, 3, 3))
                for l in range(ng1):
                    acc[:, :, 0] = acc[:, :, 0] + D[a, l] * xcl[:, c, b, l, :]
                    acc[:, :, 1] = acc[:, :, 1] + D[b, l] * xcl[:, c, l, a, :]
                    acc[:, :, 2] = acc[:, :, 2] + D[c, l] * xcl[:, l, b, a, :]
                dxcl[:, c, b, a, :, :] = acc

    # ElemBaryNGeo: evaluate at xi = 0 (particle_mesh_build.f90:1446-1466)
    L0 = lagrange_polys(0.0, xi_cl, wb_cl)
    bary = np.zeros((ne, 3))
    for c in range(ng1):
        for b in range(ng1):
            buf = L0[b] * L0[c]
            for a in range(ng1):
                bary = bary + xcl[:, c, b, a, :] * L0[a] * buf

    # XiEtaZetaBasis, slenXiEtaZetaBasis, ElemRadiusNGeo (particle_mesh_build.f90:1625-1678)
    dirs = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (-1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (0.0, 0.0, -1.0))
    xez = np.zeros((ne, 6, 3))
    slen = np.zeros((ne, 6))
    for d, xi in enumerate(dirs):
        La = lagrange_polys(xi[0], xi_cl, wb_cl)
        Lb = lagrange_polys(xi[1], xi_cl, wb_cl)
        Lc = lagrange_polys(xi[2], xi_cl, wb_cl)
        xp = np.zeros((ne, 3))
        for c in range(ng1):
            for b in range(ng1):
                for a in range(ng1):
                    xp = xp + xcl[:, c, b, a, :] * La[a] * Lb[b] * Lc[c]
        v = xp - bary
        xez[:, d, :] = v
        slen[:, d] = 1.0 / np.einsum("ij,ij->i", v, v)
    if n_geo == 1:
        radius = np.sqrt(np.max(np.sum((node_coords - bary[:, None, :]) ** 2, axis=2), axis=1))
        elem_curved = None
        bez = None
        side_bezier = side_type = None
    else:
        # Bezier control points of the element (Bernstein coefficients of the map: solve V c = X along each axis,
        # V(i,j) = B_j(t_i) on the CL points), the sides' control points bound ElemRadiusNGeo (:1662-1672) and the
        # element's control points its bounding box (convex hull property)
        tt = 0.5 * (np.asarray(xi_cl) + 1.0)
        V = np.array([[math.comb(n_geo, j) * tt[i] ** j * (1.0 - tt[i]) ** (n_geo - j) for j in range(ng1)]
                      for i in range(ng1)])
        Vi = np.linalg.inv(V)
        bez = np.einsum("ai,ebcij->ebcaj", Vi, xcl)
        bez = np.einsum("bi,ecijk->ecbjk", Vi, bez)
        bez = np.einsum("ci,eijkl->ecjkl", Vi, bez)
        side_pts = np.concatenate([bez[:, 0].reshape(ne, -1, 3), bez[:, -1].reshape(ne, -1, 3),
                                   bez[:, :, 0].reshape(ne, -1, 3), bez[:, :, -1].reshape(ne, -1, 3),
                                   bez[:, :, :, 0].reshape(ne, -1, 3), bez[:, :, :, -1].reshape(ne, -1, 3)], axis=1)
        radius = np.sqrt(np.max(np.sum((side_pts - bary[:, None, :]) ** 2, axis=2), axis=1))
        # ElemCurved: XCL_NGeo differs by more than 1e-14 from the trilinear interpolation of its corners
        # (IdentifyElemAndSideType with PointsEqual, particle_mesh_tools.f90:953-967,1238-1268)
        lin = np.zeros_like(xcl)
        for c in range(ng1):
            for b in range(ng1):
                for a in range(ng1):
                    w = [(1.0 - tt[a], tt[a]), (1.0 - tt[b], tt[b]), (1.0 - tt[c], tt[c])]
                    for q in range(8):
                        qa, qb, qc = q & 1, (q >> 1) & 1, q >> 2
                        lin[:, c, b, a, :] += w[0][qa] * w[1][qb] * w[2][qc] * node_coords[:, q, :]
        elem_curved = np.any(np.abs(lin - xcl) > 1e-14, axis=(1, 2, 3, 4)).astype(np.int32)
        side_bezier, side_type = _curved_side_data(xcl, lin, elem_curved, bary, xi_cl, n_geo)

    # ---- Gauss points, Jacobian (trilinear map) -------------------------------------
    def dof_geometry(sel, Nd):
        """Elem_xGP [e][k][j][i][3] and sJ [e][k][j][i] of the elements sel at degree Nd."""
        xg_d, _ = legendre_gauss_nodes(Nd)
        lg = [lagrange_polys(float(x), xi_cl, wb_cl) for x in xg_d]   # lg[p][a]
        nd = Nd + 1
        m = len(sel)
        exg = np.zeros((m, nd, nd, nd, 3))
        jac = np.zeros((m, nd, nd, nd, 3, 3))      # J[a][b] = d x_a / d xi_b
        for k in range(nd):
            for j in range(nd):
                for i in range(nd):
                    xp = np.zeros((m, 3))
                    J = np.zeros((m, 3, 3))
                    for c in range(ng1):
                        for b in range(ng1):
                            for a in range(ng1):
                                w = lg[i][a] * lg[j][b] * lg[k][c]
                                xp = xp + xcl[sel, c, b, a, :] * w
                                J = J + dxcl[sel, c, b, a, :, :] * w      # [nn][dd]
                    exg[:, k, j, i, :] = xp
                    jac[:, k, j, i] = J
        Jm = jac
        detJ = (Jm[..., 0, 0] * (Jm[..., 1, 1] * Jm[..., 2, 2] - Jm[..., 2, 1] * Jm[..., 1, 2])
                + Jm[..., 0, 1] * (Jm[..., 1, 2] * Jm[..., 2, 0] - Jm[..., 1, 0] * Jm[..., 2, 2])
                + Jm[..., 0, 2] * (Jm[..., 1, 0] * Jm[..., 2, 1] - Jm[..., 1, 1] * Jm[..., 2, 0]))
        return exg, 1.0 / detJ

    if n_loc is None:
        elem_xgp, sJ = dof_geometry(np.arange(ne), N)
        groups_n = [(N, np.arange(ne))]
        scaleJ = sJ.reshape(ne, -1).max(axis=1) / sJ.reshape(ne, -1).min(axis=1)
        dof_offset = None
    else:
        n_loc = np.ascontiguousarray(n_loc, dtype=np.int32).reshape(-1)
        if n_loc.shape != (ne,) or n_loc.min() < 1 or n_loc.max() > N:
            raise ValueError(f"n_loc must hold one degree in 1..{N} per element")
        dof_offset = np.zeros(ne + 1, dtype=np.int64)
        dof_offset[1:] = np.cumsum((n_loc.astype(np.int64) + 1) ** 3)        # Set_N_DG_Mapping
        elem_xgp = np.zeros((int(dof_offset[-1]), 3))
        sJ = np.zeros(int(dof_offset[-1]))
        scaleJ = np.zeros(ne)
        groups_n = [(int(k), np.nonzero(n_loc == k)[0]) for k in np.unique(n_loc)]
        for k, sel in groups_n:
            exg, sj = dof_geometry(sel, k)
            nd3 = (k + 1) ** 3
            idx = (dof_offset[sel][:, None] + np.arange(nd3)[None, :]).reshape(-1)
            elem_xgp[idx] = exg.reshape(-1, 3)
            sJ[idx] = sj.reshape(-1)
            scaleJ[sel] = sj.reshape(len(sel), -1).max(axis=1) / sj.reshape(len(sel), -1).min(axis=1)
    # ElemEpsOneCell from the element's own ElemsJ (particle_mesh_build.f90:625)
    eps_one_cell = 1.0 + np.sqrt(3.0 * scaleJ * refmapping_eps)

    # ---- sides: neighbours, periodic vectors, node maps, concavity -----------------
    side_nb = np.zeros((ne, 6), dtype=np.int32)
    side_pvid = np.zeros((ne, 6), dtype=np.int32)
    side_flip = np.zeros((ne, 6), dtype=np.int32)
    side_node = np.zeros((ne, 6, 4), dtype=np.int32)
    concave = np.zeros((ne, 6), dtype=np.int32)
    dims = (nx, ny, nz)
    ijk = np.stack([ei, ej, ek], axis=1)

    def grid_of(base, t):
        """Unwrapped grid position of corner t of the element whose first corner sits at ``base``."""
        a, b, c = t & 1, (t >> 1) & 1, (t >> 2) & 1
        return (base[0] + a, base[1] + b, base[2] + c)

    side_bc = np.zeros((ne, 6), dtype=np.int32)
    for e in range(ne):
        for s in range(6):
            off = SIDE_OFFSET[s]
            n3 = [int(ijk[e, d]) + off[d] for d in range(3)]
            pv = 0
            wall = 0
            for d in range(3):
                if n3[d] < 0 or n3[d] >= dims[d]:
                    if periodic[d]:
                        # crossing the +face moves the particle by -PeriodicVector, the -face by +
                        pv = -pv_index[d] if n3[d] >= dims[d] else pv_index[d]
                    else:
                        wall = WALL_BC[bc[d]]
                n3[d] = _wrap(n3[d], dims[d])
            en = n3[0] + nx * (n3[1] + ny * n3[2])
            side_nb[e, s] = 0 if wall else en + 1
            side_pvid[e, s] = pv
            side_bc[e, s] = wall
            cg = SIDE_CGNS[s]
            if SIDE_IS_PLUS[s] or wall:      # walls are master sides (flip 0)
                nstart = 0
                side_flip[e, s] = 0
            else:
                # slave side: rotate so that node 1 coincides with the master's node 1
                # compare unwrapped grid positions: the neighbour sits at ijk(e) + offset, so that a
                # box with one element along an axis (its own periodic neighbour) matches unambiguously
                sm = {0: 5, 1: 3, 4: 2}[s]
                base_e = tuple(int(ijk[e, d]) for d in range(3))
                base_n = tuple(base_e[d] + off[d] for d in range(3))
                master_first = grid_of(base_n, CGNS_TO_TENSOR[SIDE_CGNS[sm][0] - 1])
                nstart = -1
                for r in range(4):
                    if grid_of(base_e, CGNS_TO_TENSOR[cg[r] - 1]) == master_first:
                        nstart = r
                        break
                assert nstart >= 0
                side_flip[e, s] = nstart + 1
            for q in range(4):
                t = CGNS_TO_TENSOR[cg[(nstart + q) % 4] - 1]
                side_node[e, s, q] = 8 * e + t + 1
    # ConcaveElemSide (particle_mesh_tools.f90:1909-1930); tie-break on planar sides by side IDs
    nc = node_coords.reshape(-1, 3)
    for e in range(ne):
        for s in range(6):
            p = [nc[side_node[e, s, q] - 1] for q in range(4)]
            A = [p[q] - p[3] for q in range(3)]   # A(:,NodeNum)
            detcon = ((A[0][1] * A[1][2] - A[0][2] * A[1][1]) * A[2][0]
                      + (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * A[2][1]
                      + (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * A[2][2])
            if detcon < 0.0:
                concave[e, s] = 1
            elif detcon == 0.0 and side_nb[e, s] > 0:      # walls: SIDE_NBSIDEID = 0, never concave
                en = side_nb[e, s] - 1
                # neighbour's local side facing back
                s_back = {0: 5, 5: 0, 1: 3, 3: 1, 2: 4, 4: 2}[s]
                side_id = 6 * e + s + 1
                nb_side_id = 6 * en + s_back + 1
                if side_id < nb_side_id:
                    concave[e, s] = 1

    # ---- element nodes (CGNS order) ---------------------------------------------------
    elem_node = np.zeros((ne, 8), dtype=np.int32)
    node_info = np.zeros((ne, 8), dtype=np.int32)
    for c in range(8):
        t = CGNS_TO_TENSOR[c]
        elem_node[:, c] = 8 * np.arange(ne) + t + 1
        node_info[:, c] = corner_uid[:, t] + 1

    # ---- NodeVolume (pic_depo_tools.f90:282-303, each element with its own Nloc) ----------
    NV = np.zeros(n_unique)
    signs = ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1))
    for kd, sel in groups_n:
        xg_d, wg_d = legendre_gauss_nodes(kd)
        xg = np.asarray(xg_d)
        wg = np.asarray(wg_d)
        nd = kd + 1
        if dof_offset is None:
            sj_sel = sJ
        else:
            idx = dof_offset[sel][:, None] + np.arange(nd ** 3)[None, :]
            sj_sel = sJ[idx].reshape(len(sel), nd, nd, nd)
        for i in range(nd):
            for j in range(nd):
                for k in range(nd):
                    sjv = sj_sel[:, k, j, i]
                    for c in range(8):
                        sx, sy, sz = signs[c]
                        w = (1.0 + sx * xg[i]) * (1.0 + sy * xg[j]) * (1.0 + sz * xg[k]) * wg[i] * wg[j] * wg[k] / 8.0
                        np.add.at(NV, node_info[sel, c] - 1, 1.0 / sjv * w)

    # ---- periodic twins (pic_depo.f90:1218-2089) --------------------------------------
    canon = np.empty(n_unique, dtype=np.int64)
    gk_, gj_, gi_ = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    px, py, pz = (nx if periodic[0] else nx + 1), (ny if periodic[1] else ny + 1), (nz if periodic[2] else nz + 1)
    canon[:] = ((gi_ % px) + px * ((gj_ % py) + py * (gk_ % pz))).reshape(-1)
    order = np.argsort(canon, kind="stable")
    groups = {}
    for u in order:
        groups.setdefault(int(canon[u]), []).append(int(u))
    per_n = np.zeros(n_unique, dtype=np.int32)
    per_off = np.zeros(n_unique, dtype=np.int32)
    per_nodes = []
    for u in range(n_unique):
        twins = [v for v in groups[int(canon[u])] if v != u]
        per_off[u] = len(per_nodes)
        per_n[u] = len(twins)
        per_nodes.extend(v + 1 for v in twins)
    per_nodes = np.asarray(per_nodes if per_nodes else [0], dtype=np.int32)
    NVper = np.zeros(n_unique)
    for u in range(n_unique):
        for q in range(per_n[u]):
            NVper[u] = NVper[u] + NV[per_nodes[per_off[u] + q] - 1]
    NV = NV + NVper

    # ---- FIBGM: one background cell per unperturbed element cell ----------------------
    fib_imax = (nx, ny, nz)
    fib_d = hvec.copy()
    bmin = node_coords.min(axis=1) if bez is None else bez.reshape(ne, -1, 3).min(axis=1)
    bmax = node_coords.max(axis=1) if bez is None else bez.reshape(ne, -1, 3).max(axis=1)
    cells = [[] for _ in range(nx * ny * nz)]
    for e in range(ne):
        imn = [max(int(math.floor((bmin[e, d] - lo[d]) / fib_d[d])) + 1, 1) for d in range(3)]
        imx = [min(int(math.ceil((bmax[e, d] - lo[d]) / fib_d[d])), fib_imax[d]) for d in range(3)]
        for kk in range(imn[2], imx[2] + 1):
            for jj in range(imn[1], imx[1] + 1):
                for ii in range(imn[0], imx[0] + 1):
                    cells[(ii - 1) + nx * ((jj - 1) + ny * (kk - 1))].append(e + 1)
    fib_n = np.array([len(c) for c in cells], dtype=np.int32)
    fib_off = np.zeros(len(cells), dtype=np.int32)
    fib_off[1:] = np.cumsum(fib_n)[:-1]
    fib_el = np.array([x for c in cells for x in c], dtype=np.int32)

    pv = np.zeros((3, len(pv_index)))                 # column k = PeriodicVectors(:,k)
    for d, q in pv_index.items():
        pv[d, q - 1] = L[d]

    mesh = BoxMesh(
        nx=nx, ny=ny, nz=nz, N=N, lo=lo, hi=hi, n_elems=ne, n_nodes=n_unique, n_geo=n_geo,
        periodic_vectors=pv,
        xi_cl_ngeo=np.asarray(xi_cl), wbary_cl_ngeo=np.asarray(wb_cl),
        xgp=np.asarray(xgp), wgp=np.asarray(wgp), wbary_gp=np.asarray(wb_gp),
        xcl_ngeo=np.ascontiguousarray(xcl), dxcl_ngeo=np.ascontiguousarray(dxcl),
        elem_bary=np.ascontiguousarray(bary), xez_basis=np.ascontiguousarray(xez),
        slen_basis=np.ascontiguousarray(slen), elem_radius=np.ascontiguousarray(radius),
        eps_one_cell=np.ascontiguousarray(eps_one_cell),
        elem_xgp=np.ascontiguousarray(elem_xgp), elem_sj=np.ascontiguousarray(sJ),
        node_coords=node_coords, elem_node=elem_node, elem_side_node=np.ascontiguousarray(side_node),
        side_nb_elem=side_nb, side_pvid=side_pvid, side_flip=side_flip, concave_side=concave,
        node_info=node_info, unique_node_coords=unique_coords, node_volume=NV,
        periodic_n_nodes=per_n, periodic_offset=per_off, periodic_nodes=per_nodes,
        fibgm_imax=fib_imax, fibgm_deltas=fib_d, fibgm_n_elems=fib_n, fibgm_offset=fib_off,
        fibgm_element=fib_el, canonical_node=canon,
        side_bc=side_bc if side_bc.any() else None, bc=bc, n_loc=n_loc, dof_offset=dof_offset,
        elem_curved=elem_curved, side_bezier=side_bezier, side_type=side_type,
    )
    if (side_bc.any() and not any(periodic)) or (periodic_tracing and any(periodic)):
        halo = float(hvec.max()) if bc_halo_eps is None else float(bc_halo_eps)
        mesh.elem_to_bc_sides, mesh.bc_side_elem_loc, mesh.bc_side_distance = build_bc_elem_distance(
            mesh, halo, include_periodic=periodic_tracing)
    return mesh


def p_adaption_degrees(nx: int, ny: int, nz: int, kind: str, nmin: int, nmax: int, lo=(0.0, 0.0, 0.0),
                       hi=(1.0, 1.0, 1.0), seed: int = 0) -> np.ndarray:
    """Initial element degrees of InitpAdaption (mesh_pAdaption.f90:98-145) for the box of build_box_mesh:
    "random" -- NMin + INT(U (NMax - NMin + 1)) per element (U from a seeded generator in place of the
    reference's RANDOM_NUMBER); "half-half" -- NMax where the element's x centre is above 0, else NMin (the
    reference takes (max + min)/2 of the node x coordinates; here the cell centre of the unperturbed grid)."""
    ne = nx * ny * nz
    if kind == "random":
        u = np.random.default_rng(seed).random(ne)
        return (nmin + (u * (nmax - nmin + 1)).astype(np.int64)).astype(np.int32)
    if kind == "half-half":
        i = np.arange(ne) % nx
        h = (hi[0] - lo[0]) / nx
        xc = lo[0] + (i + 0.5) * h
        return np.where(xc > 0.0, nmax, nmin).astype(np.int32)
    raise ValueError("kind must be 'random' or 'half-half'")


# CGNS_SideToVol2 of a master side at geometry degree n: point (p,q) of local side s -> volume index (a,b,c)
_SIDE_VOL = {
    0: lambda p, q, n: (q, p, 0),          # ZETA_MINUS
    1: lambda p, q, n: (p, 0, q),          # ETA_MINUS
    2: lambda p, q, n: (n, p, q),          # XI_PLUS
    3: lambda p, q, n: (n - p, n, q),      # ETA_PLUS
    4: lambda p, q, n: (0, q, p),          # XI_MINUS
    5: lambda p, q, n: (p, q, n),          # ZETA_PLUS
}


def _slab_bounding_box_empty(P) -> bool:
    """BoundingBoxIsEmpty of GetSideSlabNormalsAndIntervals (particle_surfaces.f90:619-816) for the control
    points P[q][p][3] of one side."""
    n = P.shape[0] - 1

    def crossnorm(a, b):
        c = np.cross(a, b)
        return c / math.sqrt(float(c @ c))
    s1 = ((P[0, n] - P[0, 0]) + P[n, n]) - P[n, 0]
    s1 = s1 / math.sqrt(float(s1 @ s1))
    s2 = crossnorm(s1, ((P[n, 0] - P[0, 0]) + P[n, n]) - P[0, n])
    s3 = crossnorm(s2, s1)
    iv = np.zeros(6)
    for q in range(n + 1):
        for p in range(n + 1):
            if p == 0 and q == 0:
                continue
            d = P[q, p] - P[0, 0]
            for i, sn in enumerate((s1, s2, s3)):
                sk = (d[0] * sn[0] + d[1] * sn[1]) + d[2] * sn[2]
                if sk < 0.0:
                    iv[2 * i] = min(iv[2 * i], sk)
                elif sk > 0.0:
                    iv[2 * i + 1] = max(iv[2 * i + 1], sk)
    dx, dy, dz = abs(iv[1] - iv[0]), abs(iv[3] - iv[2]), abs(iv[5] - iv[4])
    h, w, l = dy, min(dx, dz), max(dx, dz)
    if h / max(h, l, w) < 1.0e-6:
        h = 0.0
    return abs(h / math.sqrt(l * l + w * w + h * h)) <= 2.220446049250313e-16


def _curved_side_data(xcl, lin, elem_curved, bary, xi_cl, n):
    """BezierControlPoints3D and SideType of every (element, local side) of an NGeo mesh, each side in its
    element's own (master) orientation: the Bernstein coefficients of the side's CL interpolant (sVdm_Bezier of
    BuildBezierVdm, basis.f90:275-358), and IdentifyElemAndSideType (particle_mesh_tools.f90:953-1233): an
    element that is not curved has planar (BoundingBoxIsEmpty: PLANAR_RECT if the edges meet at right angles,
    else PLANAR_NONRECT) or BILINEAR sides; a curved element's side whose CL points differ from the trilinear
    interpolation of the corners (PointsEqual, 1e-14) is PLANAR_CURVED (empty box) or CURVED, its other sides
    as for an element that is not curved."""
    ne = xcl.shape[0]
    n1 = n + 1
    xc = np.asarray(xi_cl)
    V = np.array([[math.comb(n, j) / 2.0 ** n * (1.0 + xc[i]) ** j * (1.0 - xc[i]) ** (n - j) for j in range(n1)]
                  for i in range(n1)])
    sV = np.linalg.inv(V)
    bez = np.zeros((ne, 6, n1, n1, 3))
    stype = np.zeros((ne, 6), dtype=np.int32)
    eps = 2.220446049250313e-16

    def unit(v):
        ln = math.sqrt(float(v @ v))
        return v / ln if ln > 0.0 else v * 0.0
    for s in range(6):
        idx = [[_SIDE_VOL[s](p, q, n) for p in range(n1)] for q in range(n1)]
        Xs = np.stack([np.stack([xcl[:, c, b, a] for (a, b, c) in row], axis=1) for row in idx], axis=1)  # [e][q][p][3]
        Ls = np.stack([np.stack([lin[:, c, b, a] for (a, b, c) in row], axis=1) for row in idx], axis=1)
        B = np.einsum("pi,eqid->eqpd", sV, Xs)
        B = np.einsum("qj,ejpd->eqpd", sV, B)
        bez[:, s] = B
        curved_side = np.any(np.abs(Ls - Xs) > 1e-14, axis=(1, 2, 3))
        for e in range(ne):
            P = B[e]
            empty = _slab_bounding_box_empty(P)
            if elem_curved[e] and curved_side[e]:
                stype[e, s] = 3 if empty else 4
            elif empty:
                v1 = unit(P[n, 0] - P[0, 0])
                v2 = unit(P[0, n] - P[0, 0])
                v3 = unit(P[n, n] - P[n, 0])
                rect = abs(float(v1 @ v2)) <= eps and abs(float(v1 @ v3)) <= eps
                if rect:
                    v1 = unit(P[n, n] - P[0, n])
                    rect = abs(float(v1 @ v2)) <= eps and abs(float(v1 @ v3)) <= eps
                stype[e, s] = 0 if rect else 1
            else:
                stype[e, s] = 2
    return np.ascontiguousarray(bez), stype


# CGNS_SideToVol2 at NGeo = 1 for a master side: corner (p,q) of local side s -> tensor corner (a,b,c)
_SIDE_CORNER = {
    0: lambda p, q: (q, p, 0),        # ZETA_MINUS: (p,q) = (j,i)
    1: lambda p, q: (p, 0, q),        # ETA_MINUS:  (p,q) = (i,k)
    2: lambda p, q: (1, p, q),        # XI_PLUS:    (p,q) = (j,k)
    3: lambda p, q: (1 - p, 1, q),    # ETA_PLUS:   (p,q) = (1-i,k)
    4: lambda p, q: (0, q, p),        # XI_MINUS:   (p,q) = (k,j)
    5: lambda p, q: (p, q, 1),        # ZETA_PLUS:  (p,q) = (i,j)
}


def side_control_points(mesh: BoxMesh, e: int, s: int) -> np.ndarray:
    """BezierControlPoints3D(1:3,0:NGeo,0:NGeo) of local side s of element e (0-based), as [q][p][3]
    (particle_mesh_tools.f90:1748-1773 at NGeo = 1, where the Bezier and CL corner points coincide)."""
    if mesh.side_bezier is not None:
        return mesh.side_bezier[e, s]
    out = np.zeros((2, 2, 3))
    for q in range(2):
        for p in range(2):
            a, b, c = _SIDE_CORNER[s](p, q)
            out[q, p] = mesh.xcl_ngeo[e, c, b, a]
    return out


def elem_to_elem(mesh: BoxMesh) -> list[list[int]]:
    """ElemToElemMapping/ElemToElemInfo (particle_mesh_build.f90:1244-1380): per element (0-based) the other
    elements sharing one of its unique corner nodes, in the order met walking its corners (CGNS order) and,
    per node, the elements in ascending order (NodeToElemInfo, :1150-1243)."""
    ni = mesh.node_info
    node_elems: dict[int, list[int]] = {}
    for e in range(mesh.n_elems):
        for c in range(8):
            node_elems.setdefault(int(ni[e, c]), []).append(e)
    out = []
    for e in range(mesh.n_elems):
        seen: list[int] = []
        for c in range(8):
            for t in node_elems[int(ni[e, c])]:
                if t != e and t not in seen:
                    seen.append(t)
        out.append(seen)
    return out


def sf_adaptive_radius(mesh: BoxMesh, adaptive_dof: float | None = None, smoothing: bool = False, dim: int = 3,
                       direction: int = 1) -> np.ndarray:
    """SFElemr2_Shared(1,:) of InitShapeFunctionAdaptive (pic_depo.f90:680-815): the shortest distance (SFNorm)
    from the element's corners to the corners of its node neighbours that it does not share and that do not
    coincide with them in the kernel's projection (SFMeasureDistance, pic_depo.f90:1080-1109; else the mid
    point to its corners), averaged with the characteristic length when that is shorter (always with
    ``smoothing``, PIC-shapefunction-adaptive-smoothing), times SFDepoScaling/(minN_PP+1), minN_PP the lowest
    degree of the element and its node neighbours (N without p-adaption).  ``dim`` and ``direction``
    are PIC-shapefunction-dimension and -direction: SFNorm is |v(dir)| in 1D, the norm in the plane normal to
    dir in 2D (components dim_sf_dir1, dim_sf_dir2 of InitShapeFunctionDimensionalty), the 3D norm otherwise;
    the characteristic length is BoxVolume/dimFactorSF (1D), sqrt(BoxVolume/dimFactorSF) (2D) or
    BoxVolume^(1/3) (3D); SFDepoScaling = DOF/2, sqrt(DOF/pi), (3 DOF/(4 pi))^(1/3) with DOF =
    PIC-shapefunction-adaptive-DOF (defaults 2*2, pi*2^2, (4/3) pi 2^3; at most 2(N+1), pi(N+1)^2,
    (4/3) pi (N+1)^3)."""
    N1 = mesh.N + 1.0
    if dim == 1:
        default, dof_max, name = 2.0 * 2.0, 2.0 * N1, "2*(N+1)"
    elif dim == 2:
        default, dof_max, name = math.pi * 2.0 ** 2, math.pi * N1 ** 2, "PI*(N+1)**2"
    elif dim == 3:
        default, dof_max, name = (4.0 / 3.0) * math.pi * 2.0 ** 3, (4.0 / 3.0) * math.pi * N1 ** 3, "(4/3)*PI*(N+1)**3"
    else:
        raise ValueError("dim must be 1, 2 or 3")
    if adaptive_dof is None:
        adaptive_dof = default
    if adaptive_dof > dof_max:
        raise ValueError(f"PIC-shapefunction-adaptive-DOF > {name} = {dof_max} is not allowed")
    d0 = direction - 1
    d1 = 0 if direction == 2 else 1                    # dim_sf_dir1 = MERGE(1,2,dim_sf_dir.EQ.2)
    d2 = 0 if direction == 3 else 2                    # dim_sf_dir2 = MERGE(1,3,dim_sf_dir.EQ.3)
    if dim == 1:
        scaling = adaptive_dof / 2.0
    elif dim == 2:
        scaling = math.sqrt(adaptive_dof / math.pi)
    else:
        scaling = (3.0 * adaptive_dof / (4.0 * math.pi)) ** (1.0 / 3.0)
    ext = mesh.hi - mesh.lo
    if dim == 1:
        dim_factor = float((ext[1] * ext[2]) if d0 == 0 else (ext[0] * ext[2]) if d0 == 1 else (ext[0] * ext[1]))
    elif dim == 2:
        dim_factor = float(ext[d0])
    else:
        dim_factor = 1.0

    def sf_norm(v):
        if dim == 1:
            return abs(v[d0])
        if dim == 2:
            return math.sqrt(v[d1] ** 2 + v[d2] ** 2)
        return math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])

    def almost_equal_rel(a, b, tol=1e-6):
        return abs(a - b) <= max(abs(a), abs(b)) * tol

    def measure(v1, v2):
        if dim == 1:
            return not almost_equal_rel(v1[d0], v2[d0])
        if dim == 2:
            return not (almost_equal_rel(v1[d1], v2[d1]) and almost_equal_rel(v1[d2], v2[d2]))
        return True

    nb = elem_to_elem(mesh)
    ni = mesh.node_info
    corners = mesh.node_coords.reshape(mesh.n_elems, 8, 3)[:, CGNS_TO_TENSOR, :]     # CGNS corner order
    r = np.full(mesh.n_elems, np.finfo(np.float64).max)
    for e in range(mesh.n_elems):
        done = False
        own = set(int(u) for u in ni[e])
        for t in nb[e]:
            for jn in range(8):
                if int(ni[t, jn]) in own:
                    continue
                done = True
                v2 = corners[t, jn]
                for i in range(8):
                    if measure(corners[e, i], v2):
                        rt = sf_norm(corners[e, i] - v2)
                        if rt < r[e]:
                            r[e] = rt
        if not done:
            mid = corners[e].sum(axis=0) / 8.0
            for i in range(8):
                r[e] = min(r[e], sf_norm(mid - corners[e, i]))
        lo, hi = corners[e].min(axis=0), corners[e].max(axis=0)
        vol = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2])
        if dim == 1:
            char_len = vol / dim_factor
        elif dim == 2:
            char_len = math.sqrt(vol / dim_factor)
        else:
            char_len = vol ** (1.0 / 3.0)
        if char_len < r[e] or smoothing:
            r[e] = (r[e] + char_len) / 2.0
        min_n = mesh.N if mesh.n_loc is None else int(min([mesh.n_loc[e]] + [mesh.n_loc[t] for t in nb[e]]))
        r[e] = r[e] * scaling / (min_n + 1.0)
    return r


def build_bc_elem_distance(mesh: BoxMesh, bc_halo_eps: float, include_periodic: bool = False):
    """ElemToBCSides / SideBCMetrics of BuildBCElemDistance (particle_mesh_build.f90:645-1092, the halo
    branch of an MPI build): for every element its own BC sides (local side order), then every other
    BC side whose element and side lie within bc_halo_eps (+ radii) of it, ordered by
    SideBCMetrics(BCSIDE_DISTANCE) = |ElemBaryNGeo - origin| - ElemRadiusNGeo - side radius with the
    reference's stable InsertionSort.  BC sides are the open/reflective walls and, with ``include_periodic``
    (CartesianPeriodic = F: every side with SIDE_BCID > 0 counts), the periodic sides.  Side origin and radius:
    BuildSideOriginAndRadius (particle_mesh_build.f90:1795-1820; DeCasteljauInterpolation at (0,0)).
    Returns (elem_to_bc_sides (nElems,2) = (count or -1, 0-based first entry or -1),
             entries (n,2) = (element 1-based, local side 1-based), distance (n))."""
    ne = mesh.n_elems
    isbc = mesh.side_nb_elem == 0
    if include_periodic:
        isbc = isbc | (mesh.side_pvid != 0)
    we_arr, ws_arr = np.nonzero(isbc)                  # element-major, local side order
    nbc = len(we_arr)
    if nbc == 0:
        return None
    origin = np.zeros((nbc, 3))
    radius = np.zeros(nbc)
    for k in range(nbc):
        P = side_control_points(mesh, int(we_arr[k]), int(ws_arr[k]))
        n = P.shape[0] - 1
        R = P.copy()                                      # DeCasteljauInterpolation at xi = (0,0) (basis.f90:429-476)
        for l in range(n - 1, -1, -1):
            for q in range(l + 1):
                for p in range(l + 1):
                    R[q, p] = (((0.5 * R[q, p]) * 0.5 + (0.5 * R[q + 1, p]) * 0.5) + (0.5 * R[q, p + 1]) * 0.5) \
                        + (0.5 * R[q + 1, p + 1]) * 0.5
        o = R[0, 0]
        origin[k] = o
        rmax = 0.0
        for q in range(n + 1):
            for p in range(n + 1):
                v = P[q, p] - o
                rmax = max(rmax, float(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]))
        radius[k] = math.sqrt(rmax)
    bary = mesh.elem_bary
    rad = mesh.elem_radius

    def norm3(v):
        return np.sqrt(v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1] + v[..., 2] * v[..., 2])

    own_first = np.searchsorted(we_arr, np.arange(ne), side="left")
    own_last = np.searchsorted(we_arr, np.arange(ne), side="right")
    e2b = -np.ones((ne, 2), dtype=np.int32)
    entries, dists = [], []
    chunk = max(1, 4_000_000 // nbc)
    for c0 in range(0, ne, chunk):
        es = np.arange(c0, min(ne, c0 + chunk))
        d_el = norm3(bary[es][:, None, :] - bary[we_arr][None, :, :])
        keep = d_el <= bc_halo_eps + rad[es][:, None] + rad[we_arr][None, :]
        d_sd = norm3(bary[es][:, None, :] - origin[None, :, :])
        keep &= d_sd <= bc_halo_eps + rad[es][:, None] + radius[None, :]
        keep &= we_arr[None, :] != es[:, None]
        for r, e in enumerate(es):
            own = list(range(own_first[e], own_last[e]))
            lst = own + [int(k) for k in np.nonzero(keep[r])[0]]
            if not lst:
                continue
            lst = np.asarray(lst)
            vec = bary[e] - origin[lst]
            dist = np.sqrt((vec[:, 0] * vec[:, 0] + vec[:, 1] * vec[:, 1]) + vec[:, 2] * vec[:, 2]) - rad[e] - radius[lst]
            order = np.argsort(dist, kind="stable")     # InsertionSort (utils.f90:52-101): stable, ascending
            e2b[e] = (len(lst), len(entries))
            for i in order:
                k = int(lst[i])
                entries.append((int(we_arr[k]) + 1, int(ws_arr[k]) + 1))
                dists.append(float(dist[i]))
    return e2b, np.asarray(entries, dtype=np.int32), np.asarray(dists)


def elem_map(mesh: BoxMesh, e: int, xi) -> np.ndarray:
    """x(xi) of element e (0-based) through the Lagrange interpolation of XCL_NGeo on the CL points."""
    La = lagrange_polys(float(xi[0]), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo)
    Lb = lagrange_polys(float(xi[1]), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo)
    Lc = lagrange_polys(float(xi[2]), mesh.xi_cl_ngeo, mesh.wbary_cl_ngeo)
    x = np.zeros(3)
    ng1 = mesh.n_geo + 1
    for c in range(ng1):
        for b in range(ng1):
            for a in range(ng1):
                x = x + mesh.xcl_ngeo[e, c, b, a] * La[a] * Lb[b] * Lc[c]
    return x
