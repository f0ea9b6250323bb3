/*
 * pic_oracle.c -- CPU restatement of PICLas's Boris-Leapfrog PIC particle loop.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle that tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py check the GPU library against.  The product never calls it.
 *
 * Each routine follows the cited reference Fortran (paths relative to the PICLas source
 * tree) statement by statement, in the same floating-point evaluation order.  It is built
 * with -ffp-contract=off so that no multiply-add is fused.  1-based indices as in Fortran.
 *
 * Scope restated: NGeo = 1 hexahedra, conforming (no mortar) fully periodic meshes,
 * PP_nVar = 1 (Poisson/HDG) with Boris-Leapfrog (PP_TimeDiscMethod = 508), non-relativistic
 * PartRHS, external field = constant PIC-externalField, CVWM and 3D shape_function
 * deposition, TriaTracking, and RefTracking with CartesianPeriodic = FastPeriodic = T.
 */
#include "pic_oracle.h"
#include "pic_oracle_bezier.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double EPS_MACH = 2.220446049250313080847e-16;  /* EPSILON(0.0d0) */
static const double C_LIGHT = 299792458.0;                   /* globals_vars.f90:85 */

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------------------------
 * Lagrange basis (basis.f90)
 * ------------------------------------------------------------------------------------- */
/* ALMOSTEQUAL_UNITY, basis.f90:1011-1035 */
static int almost_equal_unity(double x, double y) {
  if (x == 0.0 || y == 0.0) return fabs(x - y) <= 2.0 * EPS_MACH;
  return (fabs(x - y) <= EPS_MACH * fabs(x)) && (fabs(x - y) <= EPS_MACH * fabs(y));
}

/* LagrangeInterpolationPolys, basis.f90:1223-1264 */
void orc_lagrange_polys(double x, int n, const double* xgp, const double* wbary, double* L) {
  int hit = 0;
  for (int i = 0; i <= n; ++i) {
    L[i] = 0.0;
    if (almost_equal_unity(x, xgp[i])) { L[i] = 1.0; hit = 1; }
  }
  if (hit) return;
  double s = 0.0;
  for (int i = 0; i <= n; ++i) { L[i] = wbary[i] / (x - xgp[i]); s = s + L[i]; }
  for (int i = 0; i <= n; ++i) L[i] = L[i] / s;
}

/* ---------------------------------------------------------------------------------------
 * mesh accessors (reference layouts, 1-based element ids)
 * ------------------------------------------------------------------------------------- */
#define NG1(m)                     ((m)->n_geo + 1)
#define XCL(m, c, i, j, k, e) \
  ((m)->xcl_ngeo[((((size_t)((e) - 1) * NG1(m) + (k)) * NG1(m) + (j)) * NG1(m) + (i)) * 3 + (c)])
#define DXCL(m, dd, nn, i, j, k, e) \
  ((m)->dxcl_ngeo[(((((size_t)((e) - 1) * NG1(m) + (k)) * NG1(m) + (j)) * NG1(m) + (i)) * 3 + (nn)) * 3 + (dd)])
#define NODE(m, c, n)              ((m)->node_coords[((size_t)(n) - 1) * 3 + (c)])
#define SIDENODE(m, q, s, e)       ((m)->elem_side_node[((size_t)((e) - 1) * 6 + (s)) * 4 + (q)])

/* per-element polynomial degree: Nloc = N_DG_Mapping(2,e) and the DOF offset N_DG_Mapping(1,e) (dg_vars.f90:38,
 * set by Set_N_DG_Mapping, mesh_pAdaption.f90:391-414); without a mapping every element has degree N */
static int elem_n(const pic_mesh_t* m, int N, int e) {
  return m->n_dg_mapping ? m->n_dg_mapping[(size_t)(e - 1) * 3 + 1] : N;
}
static size_t dof_off(const pic_mesh_t* m, int N, int e) {
  return m->n_dg_mapping ? (size_t)m->n_dg_mapping[(size_t)(e - 1) * 3] : (size_t)(e - 1) * (N + 1) * (N + 1) * (N + 1);
}
/* N_Inter(Nloc)%xGP (which 0), %wGP (1), %wBary (2) */
static const double* n_inter(const pic_mesh_t* m, int nloc, int which) {
  if (!m->n_dg_mapping) return which == 0 ? m->xgp : which == 1 ? m->wgp : m->wbary_gp;
  return m->n_inter + (size_t)3 * ((nloc - 1) * (nloc + 2) / 2) + (size_t)which * (nloc + 1);
}
size_t orc_n_dofs(const pic_mesh_t* m, int N) {
  const int nl = elem_n(m, N, m->n_elems);
  return dof_off(m, N, m->n_elems) + (size_t)(nl + 1) * (nl + 1) * (nl + 1);
}

/* ---------------------------------------------------------------------------------------
 * Reference mapping x -> xi (eval_xyz.f90)
 * ------------------------------------------------------------------------------------- */
static int elem_n(const pic_mesh_t* m, int N, int e);
static size_t dof_off(const pic_mesh_t* m, int N, int e);
static const double* n_inter(const pic_mesh_t* m, int nloc, int which);

/* GetRefNewtonStartValue, eval_xyz.f90:498-612: RefMappingGuess 1 (linear pseudo-Cartesian coordinates,
 * :549-562), 2 (xi of the closest Gauss point of the element's degree, :564-583), 3 (xi of the closest XCL_NGeo
 * point, :585-601), 4 (zero, :603-605) */
static void ref_newton_start(const pic_config_t* cfg, const pic_mesh_t* m, const double x[3], double xi[3], int e) {
  const int guess = cfg->ref_mapping_guess ? cfg->ref_mapping_guess : 1;
  if (guess == 2) {
    const int nl = elem_n(m, cfg->n_dg, e), n1 = nl + 1;
    const double* xg = n_inter(m, nl, 0);
    const double* P = &m->elem_xgp[dof_off(m, cfg->n_dg, e) * 3];
    double d0[3] = {x[0] - P[0], x[1] - P[1], x[2] - P[2]};
    double winner = sqrt(d0[0] * d0[0] + d0[1] * d0[1] + d0[2] * d0[2]);
    xi[0] = xi[1] = xi[2] = xg[0];
    for (int i = 0; i <= nl; ++i)
      for (int j = 0; j <= nl; ++j)
        for (int k = 0; k <= nl; ++k) {
          const double* Q = &P[(size_t)(k * n1 * n1 + j * n1 + i) * 3];
          double dX = fabs(x[0] - Q[0]);
          if (dX > winner) continue;
          double dY = fabs(x[1] - Q[1]);
          if (dY > winner) continue;
          double dZ = fabs(x[2] - Q[2]);
          if (dZ > winner) continue;
          double dist = sqrt(dX * dX + dY * dY + dZ * dZ);
          if (dist < winner) { winner = dist; xi[0] = xg[i]; xi[1] = xg[j]; xi[2] = xg[k]; }
        }
    return;
  }
  if (guess == 3) {
    double d0[3] = {x[0] - XCL(m, 0, 0, 0, 0, e), x[1] - XCL(m, 1, 0, 0, 0, e), x[2] - XCL(m, 2, 0, 0, 0, e)};
    double winner = sqrt(d0[0] * d0[0] + d0[1] * d0[1] + d0[2] * d0[2]);
    const double* xc = m->xi_cl_ngeo;
    xi[0] = xi[1] = xi[2] = xc[0];
    for (int i = 0; i <= m->n_geo; ++i)
      for (int j = 0; j <= m->n_geo; ++j)
        for (int k = 0; k <= m->n_geo; ++k) {
          double dX = fabs(x[0] - XCL(m, 0, i, j, k, e));
          if (dX > winner) continue;
          double dY = fabs(x[1] - XCL(m, 1, i, j, k, e));
          if (dY > winner) continue;
          double dZ = fabs(x[2] - XCL(m, 2, i, j, k, e));
          if (dZ > winner) continue;
          double dist = sqrt(dX * dX + dY * dY + dZ * dZ);
          if (dist < winner) { winner = dist; xi[0] = xc[i]; xi[1] = xc[j]; xi[2] = xc[k]; }
        }
    return;
  }
  if (guess == 4) { xi[0] = xi[1] = xi[2] = 0.0; return; }
  const double epsOne = 1.0 + cfg->refmapping_eps;
  double Ptild[3], xil[6];
  for (int c = 0; c < 3; ++c) Ptild[c] = x[c] - m->elem_bary[(size_t)(e - 1) * 3 + c];
  for (int d = 0; d < 6; ++d) {
    const double* b = &m->xez_basis[((size_t)(e - 1) * 6 + d) * 3];
    double dp = Ptild[0] * b[0] + Ptild[1] * b[1] + Ptild[2] * b[2];
    xil[d] = dp * m->slen_basis[(size_t)(e - 1) * 6 + d];
  }
  for (int d = 0; d < 3; ++d) xi[d] = 0.5 * (xil[d] - xil[d + 3]);
  double mx = fmax(fabs(xi[0]), fmax(fabs(xi[1]), fabs(xi[2])));
  if (mx > epsOne)
    for (int d = 0; d < 3; ++d) xi[d] = fmax(fmin(1.0, xi[d]), -1.0);
}

/* RefElemNewton, eval_xyz.f90:298-445, for N_In <= 4: X (N_In+1)^3 CL points [k][j][i][3] and their
 * derivatives D [k][j][i][nn][dd], on the nodes XiCL with barycentric weights wb.  Returns isSuccessful. */
static int ref_elem_newton_n(const pic_config_t* cfg, double xi[3], const double x[3], int nIn, const double* X,
                             const double* D, const double* xiCL, const double* wb) {
  const int n1 = nIn + 1;
  double Lag[3][5], F[3], xiOld[3], dxi[3], Jac[3][3], sJac[3][3];
  int success = 1;
  for (int d = 0; d < 3; ++d) orc_lagrange_polys(xi[d], nIn, xiCL, wb, Lag[d]);
  /* F(xi) = x(xi) - x_in with F = F + XCL*Lag(1,i)*buff (:342-350) */
  for (int c = 0; c < 3; ++c) F[c] = -x[c];
  for (int k = 0; k <= nIn; ++k)
    for (int j = 0; j <= nIn; ++j) {
      double buff = Lag[1][j] * Lag[2][k];
      for (int i = 0; i <= nIn; ++i)
        for (int c = 0; c < 3; ++c) F[c] = F[c] + X[((size_t)(k * n1 + j) * n1 + i) * 3 + c] * Lag[0][i] * buff;
    }
  double deltaXi2 = (fabs(F[0]) < EPS_MACH && fabs(F[1]) < EPS_MACH && fabs(F[2]) < EPS_MACH) ? 0.0 : 1.0;
  double normF = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
  double normFold;
  int iter = 0;
  while (deltaXi2 > cfg->refmapping_eps && iter < 100) {
    iter = iter + 1;
    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) Jac[a][b] = 0.0;
    for (int k = 0; k <= nIn; ++k)
      for (int j = 0; j <= nIn; ++j) {
        double buff = Lag[1][j] * Lag[2][k];
        for (int i = 0; i <= nIn; ++i) {
          double buff2 = Lag[0][i] * buff;
          const double* Dp = &D[((size_t)(k * n1 + j) * n1 + i) * 9];
          for (int nn = 0; nn < 3; ++nn)
            for (int dd = 0; dd < 3; ++dd) Jac[nn][dd] = Jac[nn][dd] + Dp[nn * 3 + dd] * buff2;
        }
      }
    /* getDet, eval_xyz.f90:464-466 */
    double sdet = (Jac[0][0] * Jac[1][1] - Jac[0][1] * Jac[1][0]) * Jac[2][2]
                + (Jac[0][1] * Jac[1][2] - Jac[0][2] * Jac[1][1]) * Jac[2][0]
                + (Jac[0][2] * Jac[1][0] - Jac[0][0] * Jac[1][2]) * Jac[2][1];
    if (sdet > 0.0) sdet = 1.0 / sdet;
    /* getInv, eval_xyz.f90:486-494 */
    sJac[0][0] = (Jac[1][1] * Jac[2][2] - Jac[1][2] * Jac[2][1]) * sdet;
    sJac[0][1] = (Jac[0][2] * Jac[2][1] - Jac[0][1] * Jac[2][2]) * sdet;
    sJac[0][2] = (Jac[0][1] * Jac[1][2] - Jac[0][2] * Jac[1][1]) * sdet;
    sJac[1][0] = (Jac[1][2] * Jac[2][0] - Jac[1][0] * Jac[2][2]) * sdet;
    sJac[1][1] = (Jac[0][0] * Jac[2][2] - Jac[0][2] * Jac[2][0]) * sdet;
    sJac[1][2] = (Jac[0][2] * Jac[1][0] - Jac[0][0] * Jac[1][2]) * sdet;
    sJac[2][0] = (Jac[1][0] * Jac[2][1] - Jac[1][1] * Jac[2][0]) * sdet;
    sJac[2][1] = (Jac[0][1] * Jac[2][0] - Jac[0][0] * Jac[2][1]) * sdet;
    sJac[2][2] = (Jac[0][0] * Jac[1][1] - Jac[0][1] * Jac[1][0]) * sdet;
    for (int r = 0; r < 3; ++r) dxi[r] = ((0.0 + sJac[r][0] * F[0]) + sJac[r][1] * F[1]) + sJac[r][2] * F[2];
    deltaXi2 = dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2];
    for (int d = 0; d < 3; ++d) xiOld[d] = xi[d];
    normFold = normF;
    normF = normF * 2.0;
    double lambda = 1.0;
    int iArmijo = 1;
    while (normF > normFold * (1.0 - 0.0001 * lambda) && iArmijo <= 8) {
      for (int d = 0; d < 3; ++d) xi[d] = xiOld[d] - lambda * dxi[d];
      for (int d = 0; d < 3; ++d) orc_lagrange_polys(xi[d], nIn, xiCL, wb, Lag[d]);
      for (int c = 0; c < 3; ++c) F[c] = -x[c];
      for (int k = 0; k <= nIn; ++k)
        for (int j = 0; j <= nIn; ++j) {
          double buff = Lag[1][j] * Lag[2][k];
          for (int i = 0; i <= nIn; ++i) {
            double buff2 = Lag[0][i] * buff;
            for (int c = 0; c < 3; ++c) F[c] = F[c] + X[((size_t)(k * n1 + j) * n1 + i) * 3 + c] * buff2;
          }
        }
      lambda = 0.2 * lambda;
      iArmijo = iArmijo + 1;
      normF = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
    }
    if (fabs(xi[0]) > 1.5 || fabs(xi[1]) > 1.5 || fabs(xi[2]) > 1.5) { success = 0; break; }
  }
  return success;
}

/* The Newton of GetPositionInRefElem (eval_xyz.f90:87-117): on XCL_NGeo at NGeo for NGeo = 1 or a curved
 * element, else on the element's eight corners with their dXCL_NGeo (XCL_NGeo1, dXCL_NGeo1 on XiCL_NGeo1). */
static int ref_elem_newton(const pic_config_t* cfg, const pic_mesh_t* m, double xi[3], const double x[3], int e) {
  const int ng = m->n_geo, n1 = ng + 1;
  const size_t n3 = (size_t)n1 * n1 * n1;
  if (ng == 1 || !m->elem_curved || m->elem_curved[e - 1])
    return ref_elem_newton_n(cfg, xi, x, ng, &m->xcl_ngeo[(size_t)(e - 1) * n3 * 3],
                             &m->dxcl_ngeo[(size_t)(e - 1) * n3 * 9], m->xi_cl_ngeo, m->wbary_cl_ngeo);
  double X1[24], D1[72];
  static const double xi1[2] = {-1.0, 1.0}, wb1[2] = {-0.5, 0.5};   /* ChebyGaussLobNodes(1), BarycentricWeights */
  for (int k = 0; k <= 1; ++k)
    for (int j = 0; j <= 1; ++j)
      for (int i = 0; i <= 1; ++i) {
        const int q = (k * 2 + j) * 2 + i;
        for (int c = 0; c < 3; ++c) X1[q * 3 + c] = XCL(m, c, i * ng, j * ng, k * ng, e);
        for (int nn = 0; nn < 3; ++nn)
          for (int dd = 0; dd < 3; ++dd) D1[q * 9 + nn * 3 + dd] = DXCL(m, dd, nn, i * ng, j * ng, k * ng, e);
      }
  return ref_elem_newton_n(cfg, xi, x, 1, X1, D1, xi1, wb1);
}

/* GetPositionInRefElem, eval_xyz.f90:35-123 (NGeo = 1 branch).  Without isSuccessful the
 * reference exits the Newton loop silently in Mode 2 (the only mode used on this path without
 * isSuccessful); the success flag is still returned here for bookkeeping. */
int orc_get_position_in_ref_elem(const pic_config_t* cfg, const pic_mesh_t* m, const double x[3], double xi[3],
                                 int elem, int want_success) {
  (void)want_success;
  ref_newton_start(cfg, m, x, xi, elem);
  return ref_elem_newton(cfg, m, xi, x, elem);
}

/* EvaluateFieldAtRefPos, eval_xyz.f90:167-215 with NVar_IN = 3 */
void orc_evaluate_field_at_ref_pos(const double xi[3], int N, const double* xgp, const double* wbary, const double* U,
                                   double out[3]) {
  double L[3][8];
  for (int d = 0; d < 3; ++d) orc_lagrange_polys(xi[d], N, xgp, wbary, L[d]);
  out[0] = out[1] = out[2] = 0.0;
  const int n1 = N + 1;
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N; ++j) {
      double Lez = L[1][j] * L[2][k];
      for (int i = 0; i <= N; ++i) {
        const double* u = &U[((size_t)(k * n1 + j) * n1 + i) * 3];
        for (int c = 0; c < 3; ++c) out[c] = out[c] + u[c] * L[0][i] * Lez;
      }
    }
}

/* GetEMFieldDW, pic_interpolation_tools.f90:458-527 (components 1:3) */
static void get_em_field_dw(const pic_mesh_t* m, int N, int e, const double* Ue, const double x[3], double out[3]) {
  const size_t e0 = dof_off(m, N, e);
  N = elem_n(m, N, e);
  const int n1 = N + 1, ndof = n1 * n1 * n1;
  double dist[512];
  for (int r = 0; r < ndof; ++r) dist[r] = 0.0;
  double DistSum = 0.0;
  /* DO k; DO l; DO m with Elem_xGP(1:3,k,l,m): k is the first (fastest) array index */
  for (int k = 0; k <= N; ++k)
    for (int l = 0; l <= N; ++l)
      for (int mm = 0; mm <= N; ++mm) {
        int r = k + n1 * (l + n1 * mm);
        const double* xg = &m->elem_xgp[(e0 + r) * 3];
        double v0 = xg[0] - x[0], v1 = xg[1] - x[1], v2 = xg[2] - x[2];
        double norm = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
        if (norm > 0.0) {
          dist[r] = 1.0 / norm;
        } else {
          for (int q = 0; q < ndof; ++q) dist[q] = 0.0;
          dist[r] = 1.0;
          DistSum = 1.0;
          break; /* EXIT leaves the innermost (m) loop only */
        }
        DistSum = DistSum + dist[r];
      }
  out[0] = out[1] = out[2] = 0.0;
  for (int k = 0; k <= N; ++k)
    for (int l = 0; l <= N; ++l)
      for (int mm = 0; mm <= N; ++mm) {
        int r = k + n1 * (l + n1 * mm);
        for (int c = 0; c < 3; ++c) out[c] = out[c] + dist[r] / DistSum * Ue[(size_t)r * 3 + c];
      }
}

/* ---------------------------------------------------------------------------------------
 * InterpolateFieldToParticle, pic_interpolation.f90:248-369 + tools:54-115,198-254,399-455
 * ------------------------------------------------------------------------------------- */
static void interpolate_single(const pic_config_t* cfg, const pic_mesh_t* m, const double* e_dof, orc_particles_t* p,
                               int ip, int64_t* nfail) {
  const int N = cfg->n_dg;
  double* F = &p->field[(size_t)ip * 6];
  const double* x = &p->part_state[(size_t)ip * 6];
  const int e = p->elem[ip];
  for (int c = 0; c < 6; ++c) F[c] = cfg->external_field[c];     /* GetExternalFieldAtParticle */
  double xi[3];
  int suc = 1;
  if (cfg->tracking != PIC_TRACK_REFMAPPING) {
    suc = orc_get_position_in_ref_elem(cfg, m, x, xi, e, 1);
    if (!suc) (*nfail)++;
  } else {
    for (int d = 0; d < 3; ++d) xi[d] = p->part_pos_ref[(size_t)ip * 3 + d];
  }
  double Eo[3];
  const double* Ue = &e_dof[dof_off(m, N, e) * 3];
  const int nl = elem_n(m, N, e);   /* Nloc = N_DG_Mapping(2,ElemID), pic_interpolation_tools.f90:430 */
  if (!suc && cfg->deposition == PIC_DEPO_CVWM)
    get_em_field_dw(m, N, e, Ue, x, Eo);
  else
    orc_evaluate_field_at_ref_pos(xi, nl, n_inter(m, nl, 0), n_inter(m, nl, 2), Ue, Eo);
  for (int c = 0; c < 3; ++c) F[c] = F[c] + Eo[c];
  /* components 4:6 of GetEMField are zero for PP_nVar = 1 */
  for (int c = 3; c < 6; ++c) F[c] = F[c] + 0.0;
}

int orc_interpolate(const pic_config_t* cfg, const pic_mesh_t* m, const double* e_dof, orc_particles_t* p,
                    orc_counters_t* c, int nthreads) {
  int64_t nfail = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) reduction(+ : nfail) schedule(static)
#endif
  for (int ip = 0; ip < p->n; ++ip) {
    if (!p->inside[ip]) continue;
    if (cfg->charge[p->species[ip] - 1] == 0.0) continue;   /* isInterpolateParticle */
    interpolate_single(cfg, m, e_dof, p, ip, &nfail);
  }
  (void)nthreads;
  if (c) c->n_newton_failed += nfail;
  return 0;
}

/* ---------------------------------------------------------------------------------------
 * Boris-Leapfrog push, timedisc_TimeStepPoissonByBorisLeapfrog.f90:109-198
 * ------------------------------------------------------------------------------------- */
static void push_single(const pic_config_t* cfg, orc_particles_t* p, int ip, double dt, double c2_inv) {
  double* s = &p->part_state[(size_t)ip * 6];
  const double* F = &p->field[(size_t)ip * 6];
  const int sp = p->species[ip] - 1;
  const double q = cfg->charge[sp], mass = cfg->mass[sp];
  /* dtVar = dt * Species(s)%TimeStepFactor (timedisc_TimeStepPoissonByBorisLeapfrog.f90:130-135; 0 = unset) */
  const double fac = cfg->time_step_factor[sp] > 0.0 ? cfg->time_step_factor[sp] : 1.0;
  const double dtVar = dt * fac, dtFrac = dtVar;
  const int push = fabs(q) > 0.0;               /* isPushParticle */
  if (p->is_new[ip]) {
    if (push) {
      /* CalcPartRHSSingleParticle -> PartRHS_NR, particle_rhs.f90:232-247 */
      double qmt = q / mass;
      double Pt[3] = {F[0] * qmt, F[1] * qmt, F[2] * qmt};
      for (int c = 0; c < 3; ++c) s[3 + c] = s[3 + c] - Pt[c] * dtVar * 0.5;
    }
    p->is_new[ip] = 0;
  }
  if (push) {
    double c1 = (q * dtFrac) / (mass * 2.0);
    double vv = s[3] * s[3] + s[4] * s[4] + s[5] * s[5];
    double gamma = 1.0 / sqrt(1.0 - (vv * c2_inv));
    double vmo[3], vm[3], t[3], vp[3], vpl[3], vn1[3];
    for (int c = 0; c < 3; ++c) vmo[c] = s[3 + c] * gamma;
    for (int c = 0; c < 3; ++c) vm[c] = vmo[c] + c1 * F[c];
    double gm = sqrt(1.0 + (vm[0] * vm[0] + vm[1] * vm[1] + vm[2] * vm[2]) * c2_inv);
    const double* B = &F[3];
    double Bn = sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    double tn = tan(c1 / gm * Bn);
    double u[3] = {0.0, 0.0, 0.0};                                 /* UNITVECTOR, globals.f90:916-940 */
    if (fabs(Bn) > 0.0) { double invL = 1.0 / Bn; for (int c = 0; c < 3; ++c) u[c] = B[c] * invL; }
    for (int c = 0; c < 3; ++c) t[c] = tn * u[c];
    double cr[3] = {vm[1] * t[2] - vm[2] * t[1], vm[2] * t[0] - vm[0] * t[2], vm[0] * t[1] - vm[1] * t[0]};
    for (int c = 0; c < 3; ++c) vp[c] = vm[c] + cr[c];
    double fac = 2.0 / (1.0 + (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
    double cr2[3] = {vp[1] * t[2] - vp[2] * t[1], vp[2] * t[0] - vp[0] * t[2], vp[0] * t[1] - vp[1] * t[0]};
    for (int c = 0; c < 3; ++c) vpl[c] = vm[c] + fac * cr2[c];
    for (int c = 0; c < 3; ++c) vn1[c] = vpl[c] + c1 * F[c];
    double den = sqrt(1.0 + (vn1[0] * vn1[0] + vn1[1] * vn1[1] + vn1[2] * vn1[2]) * c2_inv);
    for (int c = 0; c < 3; ++c) s[3 + c] = vn1[c] / den;
  }
  for (int c = 0; c < 3; ++c) s[c] = s[c] + s[3 + c] * dtFrac;
}

void orc_push(const pic_config_t* cfg, orc_particles_t* p, double dt, int nthreads) {
  const double c2 = C_LIGHT * C_LIGHT;
  const double c2_inv = 1.0 / c2;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(static)
#endif
  for (int ip = 0; ip < p->n; ++ip) {
    if (!p->inside[ip]) continue;
    push_single(cfg, p, ip, dt, c2_inv);
  }
  (void)nthreads;
}

/* ---------------------------------------------------------------------------------------
 * TriaTracking (particle_triatracking.f90:137-484 and helpers)
 * ------------------------------------------------------------------------------------- */
/* ParticleInsideQuad3D, particle_mesh_tools.f90:78-222 (regular sides) */
static int inside_quad3d(const pic_mesh_t* m, const double x[3], int e, double det[6][2]) {
  int inElem = 1;
  for (int s = 0; s < 6; ++s) {
    double A[3][4];
    for (int q = 0; q < 4; ++q) {
      int nid = SIDENODE(m, q, s, e);
      for (int c = 0; c < 3; ++c) A[c][q] = NODE(m, c, nid) - x[c];
    }
    double cp0 = A[1][0] * A[2][2] - A[2][0] * A[1][2];
    double cp1 = A[2][0] * A[0][2] - A[0][0] * A[2][2];
    double cp2 = A[0][0] * A[1][2] - A[1][0] * A[0][2];
    double d1 = cp0 * A[0][1] + cp1 * A[1][1] + cp2 * A[2][1];
    d1 = -d1;
    double d2 = cp0 * A[0][3] + cp1 * A[1][3] + cp2 * A[2][3];
    det[s][0] = d1;
    det[s][1] = d2;
    int neg = 0, pos = 0;
    if (d1 < 0.0) neg = 1; else pos = 1;
    if (d2 < 0.0) neg = 1; else pos = 1;
    if (m->concave_side[(size_t)(e - 1) * 6 + s]) { if (!pos) inElem = 0; }
    else { if (neg) inElem = 0; }
  }
  return inElem;
}

/* ParticleThroughSideCheck3DFast, particle_intersection.f90:167-280 (regular side) */
static int through_side_check(const pic_mesh_t* m, const double P[3], const double V[3], int s, int e, int triNum) {
  double Ax[3], Ay[3], Az[3];
  int nid = SIDENODE(m, 0, s, e);
  Ax[0] = NODE(m, 0, nid) - P[0]; Ay[0] = NODE(m, 1, nid) - P[1]; Az[0] = NODE(m, 2, nid) - P[2];
  for (int n = 1; n <= 2; ++n) {
    int q = n + triNum - 1;       /* NodeID = n + TriNum - 1 with n = 2,3 (1-based) */
    nid = SIDENODE(m, q, s, e);
    Ax[n] = NODE(m, 0, nid) - P[0]; Ay[n] = NODE(m, 1, nid) - P[1]; Az[n] = NODE(m, 2, nid) - P[2];
  }
  const double Vx = V[0], Vy = V[1], Vz = V[2];
  double dc[3][3];
  dc[0][0] = (Ay[0] * Vz - Az[0] * Vy) * Ax[2]; dc[0][1] = (Az[0] * Vx - Ax[0] * Vz) * Ay[2]; dc[0][2] = (Ax[0] * Vy - Ay[0] * Vx) * Az[2];
  dc[1][0] = (Ay[1] * Vz - Az[1] * Vy) * Ax[0]; dc[1][1] = (Az[1] * Vx - Ax[1] * Vz) * Ay[0]; dc[1][2] = (Ax[1] * Vy - Ay[1] * Vx) * Az[0];
  dc[2][0] = (Ay[2] * Vz - Az[2] * Vy) * Ax[1]; dc[2][1] = (Az[2] * Vx - Ax[2] * Vz) * Ay[1]; dc[2][2] = (Ax[2] * Vy - Ay[2] * Vx) * Az[1];
  for (int r = 0; r < 3; ++r) {
    double det = (dc[r][0] + dc[r][1]) + dc[r][2];
    double mn = DBL_MAX;                                  /* MINVAL over an empty mask = HUGE */
    for (int q = 0; q < 3; ++q) if (fabs(dc[r][q]) > 0.0 && fabs(dc[r][q]) < mn) mn = fabs(dc[r][q]);
    double minComp = -EPS_MACH * mn;
    if (!(det >= minComp)) return 0;
  }
  return 1;
}

/* ParticleThroughSideLastPosCheck, particle_intersection.f90:430-512 (regular side) */
static int last_pos_check(const pic_mesh_t* m, const double Pl[3], int s, int e, int triNum, double* detOut) {
  double NC[3][3], Ax[3], Ay[3], Az[3];
  int nid = SIDENODE(m, 0, s, e);
  for (int c = 0; c < 3; ++c) NC[c][0] = NODE(m, c, nid);
  for (int iN = 1; iN <= 2; ++iN) {
    nid = SIDENODE(m, iN + triNum - 1, s, e);
    for (int c = 0; c < 3; ++c) NC[c][iN] = NODE(m, c, nid);
  }
  for (int q = 0; q < 3; ++q) { Ax[q] = NC[0][q] - Pl[0]; Ay[q] = NC[1][q] - Pl[1]; Az[q] = NC[2][q] - Pl[2]; }
  double det = ((Ay[0] * Az[1] - Az[0] * Ay[1]) * Ax[2] + (Az[0] * Ax[1] - Ax[0] * Az[1]) * Ay[2] +
                (Ax[0] * Ay[1] - Ay[0] * Ax[1]) * Az[2]);
  *detOut = det;
  return !((det < 0.0) || (det != det));
}

/* IntersectionWithWall, particle_intersection.f90:79-164 -> TrackInfo%alpha */
static double intersection_with_wall(const pic_mesh_t* m, const double Pold[3], const double traj[3], int s, int e,
                                     int triNum) {
  int n0 = SIDENODE(m, 0, s, e);
  double xN = NODE(m, 0, n0), yN = NODE(m, 1, n0), zN = NODE(m, 2, n0);
  int n1 = SIDENODE(m, triNum, s, e), n2 = SIDENODE(m, triNum + 1, s, e);   /* Node1 = TriNum+1, Node2 = TriNum+2 */
  double V1[3] = {NODE(m, 0, n1) - xN, NODE(m, 1, n1) - yN, NODE(m, 2, n1) - zN};
  double V2[3] = {NODE(m, 0, n2) - xN, NODE(m, 1, n2) - yN, NODE(m, 2, n2) - zN};
  double nx = V1[1] * V2[2] - V1[2] * V2[1];
  double ny = V1[2] * V2[0] - V1[0] * V2[2];
  double nz = V1[0] * V2[1] - V1[1] * V2[0];
  double nVal = sqrt(nx * nx + ny * ny + nz * nz);
  nx = nx / nVal; ny = ny / nVal; nz = nz / nVal;
  double bx = Pold[0] - xN, by = Pold[1] - yN, bz = Pold[2] - zN;
  double ax = bx - nx * (bx * nx + by * ny + bz * nz);
  double ay = by - ny * (bx * nx + by * ny + bz * nz);
  double az = bz - nz * (bx * nx + by * ny + bz * nz);
  double dist = sqrt(((ay * bz - az * by) * (ay * bz - az * by) + (az * bx - ax * bz) * (az * bx - ax * bz) +
                      (ax * by - ay * bx) * (ax * by - ay * bx)) / (ax * ax + ay * ay + az * az));
  if (dist != dist) dist = sqrt(bx * bx + by * by + bz * bz);
  double alpha = traj[0] * nx + traj[1] * ny + traj[2] * nz;
  if (fabs(alpha) > 0.0) alpha = dist / alpha;
  return alpha;
}

/* CalcNormAndTangTriangle, particle_surfaces.f90:256-319 (TriaTracking): unit normal of triangle TriNum of
 * a side, (Node(TriNum+1)-Node1) x (Node(TriNum+2)-Node1) normalised (the routine's two sign flips cancel) */
static void triangle_normal(const pic_mesh_t* m, int s, int e, int triNum, double nrm[3]) {
  int n0 = SIDENODE(m, 0, s, e), n1 = SIDENODE(m, triNum, s, e), n2 = SIDENODE(m, triNum + 1, s, e);
  double V1[3] = {NODE(m, 0, n1) - NODE(m, 0, n0), NODE(m, 1, n1) - NODE(m, 1, n0), NODE(m, 2, n1) - NODE(m, 2, n0)};
  double V2[3] = {NODE(m, 0, n2) - NODE(m, 0, n0), NODE(m, 1, n2) - NODE(m, 1, n0), NODE(m, 2, n2) - NODE(m, 2, n0)};
  double nx = -V1[1] * V2[2] + V1[2] * V2[1];
  double ny = -V1[2] * V2[0] + V1[0] * V2[2];
  double nz = -V1[0] * V2[1] + V1[1] * V2[0];
  double nVal = sqrt(nx * nx + ny * ny + nz * nz);
  nrm[0] = -nx / nVal; nrm[1] = -ny / nVal; nrm[2] = -nz / nVal;
}

/* PerfectReflection, surfacemodel_tools.f90:81-256, without wall velocity or rotating frame: the velocity and
 * the remaining trajectory are mirrored at the point of intersection, which becomes LastPartPos */
static void perfect_reflection(double v[3], double x[3], double xl[3], const double traj_in[3], double len,
                               double alpha, const double nrm[3]) {
  double poi[3], traj[3] = {traj_in[0], traj_in[1], traj_in[2]};
  for (int c = 0; c < 3; ++c) poi[c] = xl[c] + traj[c] * alpha;
  double dv = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2];
  for (int c = 0; c < 3; ++c) v[c] = v[c] - 2.0 * dv * nrm[c];
  for (int c = 0; c < 3; ++c) xl[c] = poi[c];
  double dt = traj[0] * nrm[0] + traj[1] * nrm[1] + traj[2] * nrm[2];
  for (int c = 0; c < 3; ++c) traj[c] = traj[c] - 2.0 * dt * nrm[c];
  for (int c = 0; c < 3; ++c) x[c] = xl[c] + traj[c] * (len - alpha);
}

#define ORC_MAX_TRACK_LOOPS 10000

/* SingleParticleTriaTracking3D, particle_triatracking.f90:137-484 */
static void tria_track_single(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, int ip,
                              int64_t* nlost, int64_t* nhop) {
  (void)cfg;
  double* x = &p->part_state[(size_t)ip * 6];
  double* xl = &p->last_part_pos[(size_t)ip * 3];
  int elem = p->last_elem[ip];
  int doneLast[6][4];
  memset(doneLast, 0, sizeof(doneLast));
  for (int loop = 0;; ++loop) {
    if (loop >= ORC_MAX_TRACK_LOOPS) { (*nhop)++; p->inside[ip] = 0; return; }
    double det[6][2];
    if (inside_quad3d(m, x, elem, det)) { p->elem[ip] = elem; return; }
    int nThrough = 0, locS[6] = {0}, triT[6] = {0}, globS[6] = {0};
    int sideID = 0, localSide = 0;
    double traj[3] = {x[0] - xl[0], x[1] - xl[1], x[2] - xl[2]};
    double len = sqrt(traj[0] * traj[0] + traj[1] * traj[1] + traj[2] * traj[2]);
    if (fabs(len) > 0.0) for (int c = 0; c < 3; ++c) traj[c] = traj[c] / len;
    for (int s = 0; s < 6; ++s) {
      int gside = (elem - 1) * 6 + s + 1;   /* global (non-unique) side id */
      for (int tri = 1; tri <= 2; ++tri) {
        if (det[s][tri - 1] <= -0.0) {
          if (through_side_check(m, xl, traj, s, elem, tri)) {
            if (nThrough < 6) { locS[nThrough] = s; triT[nThrough] = tri; globS[nThrough] = gside; }
            nThrough++;
            sideID = gside; localSide = s;
          }
        }
      }
    }
    int triNum = triT[0];
    if (nThrough != 1) {
      if (nThrough == 0) { (*nlost)++; p->inside[ip] = 0; return; }
      int second = 0;
      double minRatio = 0.0;
      for (int ind2 = 0; ind2 < nThrough && ind2 < 6; ++ind2) {
        int doCheck = 1;
        for (int is = 1; is < 6; ++is)
          if (doneLast[is][0] == elem && doneLast[is][3] == globS[ind2] && doneLast[is][2] == triT[ind2]) doCheck = 0;
        if (!doCheck) continue;
        double detM;
        if (last_pos_check(m, xl, locS[ind2], elem, triT[ind2], &detM)) {
          double dPP = det[locS[ind2]][triT[ind2] - 1];
          if (detM == 0.0 && dPP == 0.0) continue;
          if (detM == 0.0 && minRatio == 0.0) {
            second++; sideID = globS[ind2]; localSide = locS[ind2]; triNum = triT[ind2];
          } else {
            if (detM == 0.0) continue;
            double ratio = dPP / detM;
            if (ratio < minRatio) {
              minRatio = ratio; second++; sideID = globS[ind2]; localSide = locS[ind2]; triNum = triT[ind2];
            }
          }
        }
      }
      if (second == 0) { (*nlost)++; p->inside[ip] = 0; return; }
    }
    const int pvid = m->side_pvid[(size_t)(elem - 1) * 6 + localSide];
    const int nb = m->side_nb_elem[(size_t)(elem - 1) * 6 + localSide];
    const int bc = m->side_bc ? m->side_bc[(size_t)(elem - 1) * 6 + localSide] : 0;
    /* particle boundary of a wall side (particle_triatracking.f90:409-433, GetBoundaryInteraction
     * particle_boundary_condition.f90:35-221) */
    if (bc == 1) { p->inside[ip] = 0; return; }            /* open: RemoveParticle, not a lost particle */
    if (bc == 2) {                                          /* reflective: PerfectReflection, same element */
      double alpha = intersection_with_wall(m, xl, traj, localSide, elem, triNum);
      double nrm[3];
      triangle_normal(m, localSide, elem, triNum, nrm);
      perfect_reflection(&p->part_state[(size_t)ip * 6 + 3], x, xl, traj, len, alpha, nrm);
      memset(doneLast, 0, sizeof(doneLast));
      continue;
    }
    for (int q = 5; q >= 1; --q) for (int c = 0; c < 4; ++c) doneLast[q][c] = doneLast[q - 1][c];
    doneLast[0][0] = elem; doneLast[0][1] = localSide; doneLast[0][2] = triNum; doneLast[0][3] = sideID;
    if (pvid != 0) {
      /* IntersectionWithWall + GetBoundaryInteraction -> PeriodicBoundary
       * (particle_boundary_condition.f90:224-284) */
      double alpha = intersection_with_wall(m, xl, traj, localSide, elem, triNum);
      int k = abs(pvid) - 1;
      double sgn = pvid > 0 ? 1.0 : -1.0;
      for (int c = 0; c < 3; ++c) xl[c] = xl[c] + traj[c] * alpha;
      for (int c = 0; c < 3; ++c) xl[c] = xl[c] + copysign(m->periodic_vectors[k * 3 + c], sgn);
      for (int c = 0; c < 3; ++c) x[c] = xl[c] + (len - alpha) * traj[c];
    }
    elem = nb;
  }
}

/* ---------------------------------------------------------------------------------------
 * RefTracking with CartesianPeriodic = FastPeriodic = T (particle_reftracking.f90:30-414, 697-985)
 * ------------------------------------------------------------------------------------- */
static void periodic_movement_fast(const pic_mesh_t* m, double x[3], double xl[3]) {
  const double* mn = m->xmin_glob;
  const double* mx = m->xmax_glob;
  for (int d = 0; d < 3; ++d) {
    int iPV = -1;
    for (int k = 0; k < m->n_periodic_vectors; ++k) if (m->periodic_vectors[k * 3 + d] != 0.0) { iPV = k; break; }
    if (iPV < 0) continue;   /* GEO%directions(d) = .FALSE. */
    const double* pv = &m->periodic_vectors[iPV * 3];
    if (x[d] > mx[d]) {
      double n = ceil(fabs(x[d] - mx[d]) / fabs(pv[d]));
      double mv[3] = {n * pv[0], n * pv[1], n * pv[2]};
      if (pv[d] > 0.0) { for (int c = 0; c < 3; ++c) { x[c] = x[c] - mv[c]; xl[c] = xl[c] - mv[c]; } }
      else { for (int c = 0; c < 3; ++c) { x[c] = x[c] + mv[c]; xl[c] = xl[c] + mv[c]; } }
    }
    if (x[d] < mn[d]) {
      double n = ceil(fabs(x[d] - mn[d]) / fabs(pv[d]));
      double mv[3] = {n * pv[0], n * pv[1], n * pv[2]};
      if (pv[d] > 0.0) { for (int c = 0; c < 3; ++c) { x[c] = x[c] + mv[c]; xl[c] = xl[c] + mv[c]; } }
      else { for (int c = 0; c < 3; ++c) { x[c] = x[c] - mv[c]; xl[c] = xl[c] - mv[c]; } }
    }
  }
}

static double maxabs3(const double v[3]) { return fmax(fabs(v[0]), fmax(fabs(v[1]), fabs(v[2]))); }

static int almost_equal(double x, double y) { return fabs(x - y) <= fmax(fabs(x), fabs(y)) * 4.441e-16; }

/* ---- RefTracking with walls (meshes without periodic vectors) ----------------------------------------
 * Wall side geometry of a planar rectangular side: BezierControlPoints3D at NGeo = 1 (the corner nodes in
 * CGNS side order, particle_mesh_tools.f90:1748-1773), BaseVectors0-2 (particle_mesh_build.f90:1916-1925),
 * SideNormVec / SideDistance oriented away from the element (particle_mesh_tools.f90:1011-1048). */
typedef struct {
  double bv0[3], bv1[3], bv2[3], bv3[3], n[3], dist, P[4][3];
  int bc, type;                     /* type: SideType PLANAR_RECT (0), PLANAR_NONRECT (1), BILINEAR (2),
                                       PLANAR_CURVED (3), CURVED (4) */
  int pvid, nb;                     /* bc = 3 (periodic): BoundaryType(BC_ALPHA) and SIDE_NBELEMID (1-based) */
  orc_bz_side_t bz;                 /* curved sides (NGeo > 1): Bezier points, slab normals and intervals */
} orc_bc_side_t;
enum { ORC_PLANAR_RECT = 0, ORC_PLANAR_NONRECT = 1, ORC_BILINEAR = 2, ORC_PLANAR_CURVED = 3, ORC_CURVED = 4 };

/* corner (p,q) in {0,1} of local side s of element e (0-based): XCL_NGeo at the volume index of CGNS_SideToVol2 */
static void side_corner(const pic_mesh_t* m, int e, int s, int p, int q, double out[3]) {
  const int ng = m->n_geo;
  int a, b, c;
  switch (s) {
    case 0: a = q; b = p; c = 0; break;
    case 1: a = p; b = 0; c = q; break;
    case 2: a = 1; b = p; c = q; break;
    case 3: a = 1 - p; b = 1; c = q; break;
    case 4: a = 0; b = q; c = p; break;
    default: a = p; b = q; c = 1; break;
  }
  for (int k = 0; k < 3; ++k) out[k] = XCL(m, k, a * ng, b * ng, c * ng, e + 1);
}

static void unit3(const double v[3], double u[3]) {
  double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (fabs(l) > 0.0) { l = 1.0 / l; u[0] = v[0] * l; u[1] = v[1] * l; u[2] = v[2] * l; }
  else { u[0] = u[1] = u[2] = 0.0; }
}

/* GetSideType for NGeo = 1 (particle_mesh_tools.f90:1001-1053; linear elements are never curved): a side
 * whose corners lie within 1e-6 of its extent of the averaged plane is planar (the slab test of
 * GetSideSlabNormalsAndIntervals, particle_surfaces.f90:740-815, restated on the four corners) with
 * SideNormVec oriented away from the element and SideDistance, PLANAR_RECT when its edges meet at right
 * angles (:1026-1041), PLANAR_NONRECT otherwise; a non-planar side is BILINEAR with the non-oriented
 * averaged normal.  Returns the type. */
static int orc_bc_side_geometry(const pic_mesh_t* m, int e, int s, orc_bc_side_t* g) {
  memset(g, 0, sizeof(*g));
  if (m->n_geo > 1) {
    /* curved mesh: the side's Bezier points and the reference's SideType; SideNormVec/SideDistance of a planar
     * side from its corners as below (IdentifyElemAndSideType, particle_mesh_tools.f90:991-1012) */
    const size_t n2 = (size_t)(m->n_geo + 1) * (m->n_geo + 1);
    orc_bz_side_init(&g->bz, m->n_geo, &m->side_bezier[((size_t)e * 6 + s) * n2 * 3]);
  }
  double P00[3], P10[3], P01[3], P11[3];
  side_corner(m, e, s, 0, 0, P00); side_corner(m, e, s, 1, 0, P10);
  side_corner(m, e, s, 0, 1, P01); side_corner(m, e, s, 1, 1, P11);
  double ctr[3];
  for (int c = 0; c < 3; ++c) {
    g->bv0[c] = ((+P00[c] + P10[c]) + P01[c]) + P11[c];
    g->bv1[c] = ((-P00[c] + P10[c]) - P01[c]) + P11[c];
    g->bv2[c] = ((-P00[c] - P10[c]) + P01[c]) + P11[c];
    g->bv3[c] = ((+P00[c] - P10[c]) - P01[c]) + P11[c];
    ctr[c] = 0.25 * (((P00[c] + P10[c]) + P01[c]) + P11[c]);
    g->P[0][c] = P00[c]; g->P[1][c] = P10[c]; g->P[2][c] = P01[c]; g->P[3][c] = P11[c];
  }
  const double* v1 = g->bv1;
  const double* v2 = g->bv2;
  double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
  double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int c = 0; c < 3; ++c) n[c] = n[c] / len;
  g->bc = m->side_bc ? m->side_bc[(size_t)e * 6 + s] : 0;
  g->pvid = m->side_pvid[(size_t)e * 6 + s];
  g->nb = m->side_nb_elem[(size_t)e * 6 + s];
  if (g->bc == 0 && g->pvid != 0) g->bc = 3;     /* a periodic side traced as a BC side */
  /* slab thickness along the averaged normal against the side's extent */
  const double* Pc[4] = {P00, P10, P01, P11};
  double hmin = DBL_MAX, hmax = -DBL_MAX;
  for (int k = 0; k < 4; ++k) {
    const double d = Pc[k][0] * n[0] + Pc[k][1] * n[1] + Pc[k][2] * n[2];
    hmin = fmin(hmin, d); hmax = fmax(hmax, d);
  }
  const double l1 = 0.5 * sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  const double l2 = 0.5 * sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  const double h = hmax - hmin, dmax = fmax(h, fmax(l1, l2));
  const int given = m->n_geo > 1 ? m->side_type[(size_t)e * 6 + s] : -1;
  if (given == ORC_BILINEAR || given == ORC_CURVED || (given < 0 && !(h < 1.0e-6 * dmax))) {
    for (int c = 0; c < 3; ++c) g->n[c] = n[c];
    g->dist = 0.0;
    g->type = given == ORC_CURVED ? ORC_CURVED : ORC_BILINEAR;
    return g->type;
  }
  const double* bary = &m->elem_bary[(size_t)e * 3];
  double vb[3] = {ctr[0] - bary[0], ctr[1] - bary[1], ctr[2] - bary[2]};
  if (vb[0] * n[0] + vb[1] * n[1] + vb[2] * n[2] < 0.0) for (int c = 0; c < 3; ++c) n[c] = -n[c];
  for (int c = 0; c < 3; ++c) g->n[c] = n[c];
  g->dist = ctr[0] * n[0] + ctr[1] * n[1] + ctr[2] * n[2];
  double d1[3], d2[3], d3[3], d4[3], u1[3], u2[3], u3[3], u4[3];
  for (int c = 0; c < 3; ++c) { d1[c] = P01[c] - P00[c]; d2[c] = P10[c] - P00[c]; d3[c] = P11[c] - P01[c]; d4[c] = P11[c] - P10[c]; }
  unit3(d1, u1); unit3(d2, u2); unit3(d3, u3); unit3(d4, u4);
#define DOT3(a, b) ((a)[0] * (b)[0] + (a)[1] * (b)[1] + (a)[2] * (b)[2])
  int rect = fabs(DOT3(u1, u2)) <= 2.22e-16 && fabs(DOT3(u1, u3)) <= 2.22e-16;
  if (rect) rect = fabs(DOT3(u4, u2)) <= 2.22e-16 && fabs(DOT3(u4, u3)) <= 2.22e-16;
#undef DOT3
  g->type = given >= 0 ? given : (rect ? ORC_PLANAR_RECT : ORC_PLANAR_NONRECT);
  return g->type;
}

/* QuadraticSolver, utils.f90:401-465 */
static int quadratic_solver(double A, double B, double C, double* r1, double* r2) {
  *r1 = 0.0; *r2 = 0.0;
  if (A != 0.0 && B == 0.0 && C == 0.0) return 1;
  if (A != 0.0) {
    const double q = 0.5 * B / A, radicant = q * q - (C / A);
    if (radicant < 0.0) return 0;
    const double ba = B / A;
    *r1 = -(0.5 * ba) - copysign(1.0, ba) * sqrt(radicant);
    *r2 = (C / A) / *r1;
    return 2;
  }
  if (B != 0.0) { *r1 = -C / B; return 1; }
  return 0;
}

/* ComputeXi, particle_intersection.f90:2241-2273; HUGE when the denominator vanishes */
static double compute_xi(double eta, const double A1[4], const double A2[4]) {
  const double a = eta * A2[0] + A2[1];
  const double b = (eta * (A2[0] - A1[0]) + A2[1]) - A1[1];
  if (fabs(b) >= fabs(a)) {
    if (fabs(b) <= 2.22e-16) return DBL_MAX;
    return (-(eta * (A2[2] - A1[2])) - (A2[3] - A1[3])) / b;
  }
  return (-(eta * A2[2]) - A2[3]) / a;
}

/* ComputeSurfaceDistance2, particle_intersection.f90:2209-2238 */
static double surface_distance2(const double BLC[4][3], double xi, double eta, const double traj[3]) {
  double v[3];
  for (int c = 0; c < 3; ++c) v[c] = (((xi * eta) * BLC[0][c] + xi * BLC[1][c]) + eta * BLC[2][c]) + BLC[3][c];
  return (v[0] * traj[0] + v[1] * traj[1]) + v[2] * traj[2];
}

/* ComputeBiLinearIntersection, particle_intersection.f90:855-1240, RefTracking on a wall side (BCID > 0):
 * the bilinear patch X(xi,eta) met by the line xl + t traj, eta from the quadratic of the two components
 * normal to the trajectory, xi from ComputeXi, t the distance along traj; of two hits the nearer.  alpha2 > -1
 * (the double check) drops a hit at alpha2.  Returns alpha or -1, and xi/eta of the hit; *bad is set where
 * the reference aborts ('Invalid intersection with bilinear side'). */
static double bilinear_alpha(const orc_bc_side_t* g, const double xl[3], const double traj[3], double len,
                             double alpha2, double* xi_out, double* eta_out, int* bad) {
  double BLC[4][3];
  for (int c = 0; c < 3; ++c) {
    BLC[0][c] = 0.25 * g->bv3[c]; BLC[1][c] = 0.25 * g->bv1[c];
    BLC[2][c] = 0.25 * g->bv2[c]; BLC[3][c] = 0.25 * g->bv0[c];
  }
  const double scaleFac = traj[0] * g->n[0] + traj[1] * g->n[1] + traj[2] * g->n[2];
  if (fabs(scaleFac) < 100.0 * EPS_MACH) return -1.0;                      /* epsilontol */
  for (int c = 0; c < 3; ++c) BLC[3][c] = BLC[3][c] - xl[c];
  double NC[4][3];
  for (int i = 0; i < 4; ++i) {
    const double d = (BLC[i][0] * traj[0] + BLC[i][1] * traj[1]) + BLC[i][2] * traj[2];
    for (int c = 0; c < 3; ++c) NC[i][c] = BLC[i][c] - d * traj[c];
  }
  double A1[4], A2[4];
  for (int i = 0; i < 4; ++i) { A1[i] = NC[i][2] - NC[i][0]; A2[i] = NC[i][2] - NC[i][1]; }
  const double A = A1[0] * A2[2] - A2[0] * A1[2];
  const double B = ((A1[0] * A2[3] - A2[0] * A1[3]) + A1[1] * A2[2]) - A2[1] * A1[2];
  const double C = A1[1] * A2[3] - A2[1] * A1[3];
  double eta[2], xi[2] = {0.0, 0.0}, t[2] = {-1.0, -1.0};
  const int nRoot = quadratic_solver(A, B, C, &eta[0], &eta[1]);
  int inter = 0;
  for (int r = 0; r < nRoot; ++r) {
    if (!(fabs(eta[r]) <= 1.0)) continue;
    xi[r] = compute_xi(eta[r], A1, A2);
    if (xi[r] == DBL_MAX) { *bad = 1; return -1.0; }
    if (!(fabs(xi[r]) <= 1.0)) continue;
    t[r] = surface_distance2(BLC, xi[r], eta[r], traj);
    if (alpha2 > -1.0 && almost_equal(t[r], alpha2)) t[r] = -1.0;
    const double alphaNorm = t[r] / len;
    if (alphaNorm <= 1.0 && alphaNorm >= 0.0) inter |= 1 << r;
    if (nRoot == 1) break;
  }
  int k;
  if (inter == 0) return -1.0;
  else if (inter == 1) k = 0;
  else if (inter == 2) k = 1;
  else k = t[0] < t[1] ? 0 : 1;
  *xi_out = xi[k];
  *eta_out = eta[k];
  return t[k];
}

/* CalcNormAndTangBilinear, particle_surfaces.f90:404-440: the unit normal d/dxi x d/deta at (xi,eta) */
static void bilinear_normal(const orc_bc_side_t* g, double xi, double eta, double nv[3]) {
  const double* P00 = g->P[0];
  const double* P10 = g->P[1];
  const double* P01 = g->P[2];
  const double* P11 = g->P[3];
  double a[3], b[3];
  for (int c = 0; c < 3; ++c) {
    const double twist = ((P00[c] - P10[c]) + P11[c]) - P01[c];
    b[c] = (xi * 0.25) * twist + 0.25 * (((-P00[c] - P10[c]) + P11[c]) + P01[c]);
    a[c] = (eta * 0.25) * twist + 0.25 * (((-P00[c] + P10[c]) + P11[c]) - P01[c]);
  }
  double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  const double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int c = 0; c < 3; ++c) nv[c] = n[c] / l;
}

/* ComputePlanarRectIntersection, particle_intersection.f90:515-684 (flip = 0: wall sides are masters);
 * returns alpha or -1 */
static double planar_rect_alpha(const orc_bc_side_t* g, const double xl[3], const double traj[3], double len) {
  const double* n = g->n;
  double coeffA = n[0] * traj[0] + n[1] * traj[1] + n[2] * traj[2];
  if (fabs(coeffA) <= 2.22e-16) return -1.0;                       /* parallel to the side */
  double locSideDistance = g->dist - (xl[0] * n[0] + xl[1] * n[1] + xl[2] * n[2]);
  double alpha = locSideDistance / coeffA;
  if (locSideDistance < -100.0 * EPS_MACH) return -1.0;
  double alphaNorm = alpha / len;
  if (alphaNorm > 1.0 || alphaNorm < -(100.0 * EPS_MACH)) return -1.0;   /* epsilontol = 100 epsMach */
  double P0[3], P1[3], P2[3];
  for (int c = 0; c < 3; ++c) {
    double inter = xl[c] + alpha * traj[c];
    P0[c] = -0.25 * g->bv0[c] + inter;
    P1[c] = 0.25 * g->bv1[c];
    P2[c] = 0.25 * g->bv2[c];
  }
  double A1 = P1[0] * P1[0] + P1[1] * P1[1] + P1[2] * P1[2];
  double B1 = P2[0] * P1[0] + P2[1] * P1[1] + P2[2] * P1[2];
  double C1 = P1[0] * P0[0] + P1[1] * P0[1] + P1[2] * P0[2];
  double A2 = B1;
  double B2 = P2[0] * P2[0] + P2[1] * P2[1] + P2[2] * P2[2];
  double C2 = P2[0] * P0[0] + P2[1] * P0[1] + P2[2] * P0[2];
  double sdet = A1 * B2 - A2 * B1;
  if (fabs(sdet) == 0.0) return -1.0;                              /* the reference aborts */
  sdet = 1.0 / sdet;
  const double epsLoc = 1.0 + 100.0 * EPS_MACH;
  double xi = (B2 * C1 - B1 * C2) * sdet;
  if (fabs(xi) > epsLoc) return -1.0;
  double eta = (-A2 * C1 + A1 * C2) * sdet;
  if (fabs(eta) > epsLoc) return -1.0;
  return alpha;
}

#define ORC_BC_CAP 64   /* wall sides within reach of one trajectory; more are not traced (same cap on the GPU) */

/* ParticleBCTracking, particle_reftracking.f90:417-694: trace the trajectory against the BC sides of the
 * element's list (sorted by SideBCMetrics distance, stopping beyond the trajectory length) -- open and
 * reflective walls, and with periodic_tracing the periodic sides.  A periodic crossing (GetBoundaryInteraction
 * -> PeriodicBoundary, particle_boundary_condition.f90:184-186, 224-284) moves LastPartPos to the crossing
 * point plus the periodic vector and the particle by the rest of its trajectory, and continues the trace in
 * the neighbour element (the reference's recursive call, here a loop).  *elem is that element on return.
 * Returns 1 when the particle is done -- it has not moved (PARTHASMOVED) or an open wall removed it. */
static int bc_tracking(const pic_mesh_t* m, const orc_bc_side_t* geo, int* elem, double x[3], double xl[3],
                       double v[3], uint8_t* inside, double* len0, int64_t* ncap) {
  for (int call = 0; call < ORC_MAX_TRACK_LOOPS; ++call) {
    const int e = *elem - 1;
    const int nloc = m->elem_to_bc_sides[2 * e] > 0 ? m->elem_to_bc_sides[2 * e] : 0;
    const int first = m->elem_to_bc_sides[2 * e + 1];
    double traj[3] = {x[0] - xl[0], x[1] - xl[1], x[2] - xl[2]};
    double len = sqrt(traj[0] * traj[0] + traj[1] * traj[1] + traj[2] * traj[2]);
    if (fabs(len / m->elem_radius[e]) <= 2.22e-16) return 1;
    for (int c = 0; c < 3; ++c) traj[c] = traj[c] / len;
    *len0 = fmax(*len0, len);
    int doubleCheck = 0, moved_elem = 0;
    double alphaOld = -1.0;
    for (int loop = 0; loop < ORC_MAX_TRACK_LOOPS; ++loop) {
      double alpha[ORC_BC_CAP], sxi[ORC_BC_CAP], seta[ORC_BC_CAP];
      int list[ORC_BC_CAP];
      int nc = 0, nInter = 0;
      for (int i = 0; i < nloc; ++i) {
        if (m->bc_side_distance[first + i] > *len0) break;
        if (nc == ORC_BC_CAP) { (*ncap)++; break; }
        const orc_bc_side_t* g = &geo[first + i];
        sxi[nc] = 0.0; seta[nc] = 0.0;
        if (g->type == ORC_PLANAR_RECT) {
          alpha[nc] = planar_rect_alpha(g, xl, traj, len);
        } else if (g->type == ORC_PLANAR_CURVED || g->type == ORC_CURVED) {
          int bad = 0;
          alpha[nc] = g->type == ORC_CURVED
                          ? orc_bz_curved(&g->bz, g->n, xl, x, traj, len, &sxi[nc], &seta[nc], &bad)
                          : orc_bz_planar_curved(&g->bz, g->n, g->dist, xl, traj, len, &sxi[nc], &seta[nc], &bad);
          if (bad) (*ncap)++;
        } else {
          int bad = 0;
          alpha[nc] = bilinear_alpha(g, xl, traj, len, doubleCheck ? alphaOld : -1.0, &sxi[nc], &seta[nc], &bad);
          if (bad) (*ncap)++;
        }
        list[nc] = i;
        if (alpha[nc] > -1.0) nInter++;
        nc++;
      }
      if (nInter == 0) return 0;
      int slot[ORC_BC_CAP];
      for (int i = 0; i < nc; ++i) slot[i] = i;
      for (int i = 1; i < nc; ++i) {              /* InsertionSort (stable) */
        double t = alpha[i];
        int ti = list[i], ts = slot[i], j = i - 1;
        while (j >= 0 && !(alpha[j] <= t)) { alpha[j + 1] = alpha[j]; list[j + 1] = list[j]; slot[j + 1] = slot[j]; j--; }
        alpha[j + 1] = t; list[j + 1] = ti; slot[j + 1] = ts;
      }
      for (int k = 0; k < nc; ++k)
        if (alpha[k] > -1.0) { alphaOld = alpha[k]; break; }
      int reflected = 0;
      for (int k = 0; k < nc; ++k) {
        if (!(alpha[k] > -1.0)) continue;
        const orc_bc_side_t* g = &geo[first + list[k]];
        /* GetBoundaryInteraction (particle_boundary_condition.f90:35-221), REFMAPPING branch: SideNormVec of
         * planar sides, CalcNormAndTangBilinear at the hit of bilinear ones */
        double nl[3] = {g->n[0], g->n[1], g->n[2]};
        if (g->type == ORC_BILINEAR) bilinear_normal(g, sxi[slot[k]], seta[slot[k]], nl);
        if (g->type == ORC_PLANAR_CURVED || g->type == ORC_CURVED) orc_bz_normal(&g->bz, sxi[slot[k]], seta[slot[k]], nl);
        if (nl[0] * traj[0] + nl[1] * traj[1] + nl[2] * traj[2] <= 0.0) { reflected = 0; continue; }
        reflected = 1;
        if (g->bc == 1) { *inside = 0; break; }                  /* RemoveParticle */
        if (g->bc == 3) {
          /* PeriodicBoundary: LastPartPos at the crossing plus the periodic vector, the rest of the trajectory */
          const int k3 = (g->pvid < 0 ? -g->pvid : g->pvid) - 1;
          const double sg = g->pvid < 0 ? -1.0 : 1.0;
          for (int c = 0; c < 3; ++c) xl[c] = xl[c] + traj[c] * alpha[k];
          for (int c = 0; c < 3; ++c) xl[c] = xl[c] + copysign(m->periodic_vectors[3 * k3 + c], sg);
          for (int c = 0; c < 3; ++c) x[c] = xl[c] + (len - alpha[k]) * traj[c];
          len = len - alpha[k];
          if (g->nb != *elem) {
            /* the trace continues in the neighbour; lengthPartTrajectory0 = the largest SideBCMetrics distance
             * of the element it left */
            if (m->n_periodic_vectors > 0) {
              double mx = -DBL_MAX;
              for (int i = 0; i < nloc; ++i) mx = fmax(mx, m->bc_side_distance[first + i]);
              *len0 = mx;
            }
            *elem = g->nb;
            moved_elem = 1;
          }
          break;
        }
        perfect_reflection(v, x, xl, traj, len, alpha[k], nl);
        for (int c = 0; c < 3; ++c) traj[c] = x[c] - xl[c];
        len = sqrt(traj[0] * traj[0] + traj[1] * traj[1] + traj[2] * traj[2]);
        if (fabs(len) <= 2.22e-16) len = 0.0;
        else for (int c = 0; c < 3; ++c) traj[c] = traj[c] / len;
        break;
      }
      if (moved_elem) break;
      if (!*inside) return 1;
      if (!reflected) {
        if (!doubleCheck) doubleCheck = 1;
        else return 0;
      }
    }
    if (!moved_elem) return 0;
  }
  return 0;
}

static void ref_track_single(const pic_config_t* cfg, const pic_mesh_t* m, const orc_bc_side_t* geo,
                             orc_particles_t* p, int ip, int64_t* ntol, int64_t* nhop) {
  double* x = &p->part_state[(size_t)ip * 6];
  double* v = x + 3;
  double* xl = &p->last_part_pos[(size_t)ip * 3];
  double* xi = &p->part_pos_ref[(size_t)ip * 3];
  int elem = p->last_elem[ip];
  const int bc_elem = geo && m->elem_to_bc_sides[2 * (elem - 1)] > 0;
  if (bc_elem) {
    /* BC element (particle_reftracking.f90:98-126); a periodic crossing changes the element */
    double len0 = 0.0;
    if (bc_tracking(m, geo, &elem, x, xl, v, &p->inside[ip], &len0, nhop)) { p->elem[ip] = elem; return; }
    orc_get_position_in_ref_elem(cfg, m, x, xi, elem, 0);
    if (maxabs3(xi) < 1.0) { p->elem[ip] = elem; return; }
  } else if (m->n_periodic_vectors > 0 && !cfg->periodic_tracing) {
    double lp[3] = {x[0], x[1], x[2]};
    periodic_movement_fast(m, x, xl);
    int guard = 0;
    while ((!almost_equal(lp[0], x[0]) || !almost_equal(lp[1], x[1]) || !almost_equal(lp[2], x[2])) && guard < 16) {
      lp[0] = x[0]; lp[1] = x[1]; lp[2] = x[2];
      periodic_movement_fast(m, x, xl);
      guard++;
    }
  }
  if (!bc_elem) {
    orc_get_position_in_ref_elem(cfg, m, x, xi, elem, 0);
    if (maxabs3(xi) < 1.0) { p->elem[ip] = elem; return; }
  }
  int oldElem = p->last_elem[ip];
  int cell[3];
  for (int d = 0; d < 3; ++d) {
    int cc = (int)floor((x[d] - m->xmin_glob[d]) / m->fibgm_deltas[d]);
    cc = (cc > 0 ? cc : 0) + 1;
    cell[d] = cc < m->fibgm_imax[d] ? cc : m->fibgm_imax[d];
  }
  size_t cidx = (size_t)(cell[0] - 1) + (size_t)m->fibgm_imax[0] * ((cell[1] - 1) + (size_t)m->fibgm_imax[1] * (cell[2] - 1));
  int nBGM = m->fibgm_n_elems[cidx];
  int off = m->fibgm_offset[cidx];
  double distv[256];
  int list[256];
  if (nBGM > 256) nBGM = 256;
  if (nBGM > 1) {
    for (int i = 0; i < nBGM; ++i) {
      int e = m->fibgm_element[off + i];
      list[i] = e;
      if (e == oldElem) distv[i] = -DBL_MAX;
      else {
        const double* b = &m->elem_bary[(size_t)(e - 1) * 3];
        double d0 = x[0] - b[0], d1 = x[1] - b[1], d2 = x[2] - b[2];
        distv[i] = (d0 * d0 + d1 * d1) + d2 * d2;
        double r = m->elem_radius[e - 1];
        if (distv[i] > r * r) distv[i] = -DBL_MAX;
      }
    }
    /* InsertionSort, utils.f90:52-101 */
    for (int i = 1; i < nBGM; ++i) {
      int j = i - 1;
      double tr = distv[i];
      int ti = list[i];
      while (j >= 0) {
        if (distv[j] <= tr) break;
        distv[j + 1] = distv[j]; list[j + 1] = list[j];
        j--;
      }
      distv[j + 1] = tr; list[j + 1] = ti;
    }
  } else if (nBGM == 1) {
    distv[0] = 0.0;
    list[0] = m->fibgm_element[off];
  }
  double oldXi[3] = {xi[0], xi[1], xi[2]};
  double newXi[3] = {DBL_MAX, DBL_MAX, DBL_MAX};
  int newElem = -1;
  for (int i = 0; i < nBGM; ++i) {
    if (distv[i] == -DBL_MAX) continue;
    int e = list[i];
    orc_get_position_in_ref_elem(cfg, m, x, xi, e, 0);
    if (maxabs3(xi) < 1.0) { p->elem[ip] = e; return; }
    if (maxabs3(xi) < maxabs3(newXi)) { newXi[0] = xi[0]; newXi[1] = xi[1]; newXi[2] = xi[2]; newElem = e; }
  }
  if (maxabs3(oldXi) < maxabs3(newXi)) {
    xi[0] = oldXi[0]; xi[1] = oldXi[1]; xi[2] = oldXi[2];
    p->elem[ip] = oldElem;
  } else {
    xi[0] = newXi[0]; xi[1] = newXi[1]; xi[2] = newXi[2];
    p->elem[ip] = newElem;
  }
  int te = p->elem[ip];
  double epsElement = (te >= 1) ? m->eps_one_cell[te - 1] : 1.0;
  if (te < 1 || maxabs3(xi) > epsElement) {
    if (te >= 1 && geo && m->elem_to_bc_sides[2 * (te - 1)] > 0) {
      /* BC element (particle_reftracking.f90:327-403): trace the BC sides again from TestElem (a periodic
       * crossing changes it; epsOneCell stays the one of the element the trace started in) */
      double len0 = 0.0;
      const double eps_te = m->eps_one_cell[te - 1];
      if (bc_tracking(m, geo, &te, x, xl, v, &p->inside[ip], &len0, nhop)) { p->elem[ip] = te; return; }
      orc_get_position_in_ref_elem(cfg, m, x, xi, te, 0);
      /* beyond epsOneCell the reference calls LocateParticleInElement and aborts when that fails */
      if (maxabs3(xi) > eps_te) (*ntol)++;
      else p->elem[ip] = te;
    } else {
      (*ntol)++;                                 /* the reference aborts here (internal element) */
    }
  }
}

/* the wall geometry of every BC entry, or NULL without RefTracking walls */
static orc_bc_side_t* bc_geometry(const pic_mesh_t* m) {
  if (!m->elem_to_bc_sides || m->n_bc_entries <= 0) return NULL;
  orc_bc_side_t* geo = (orc_bc_side_t*)malloc(sizeof(orc_bc_side_t) * (size_t)m->n_bc_entries);
  for (int k = 0; k < m->n_bc_entries; ++k)
    orc_bc_side_geometry(m, m->bc_side_elem_loc[2 * k] - 1, m->bc_side_elem_loc[2 * k + 1] - 1, &geo[k]);
  return geo;
}

void orc_track(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, orc_counters_t* c, int nthreads) {
  int64_t nlost = 0, nhop = 0, ntol = 0;
  orc_bc_side_t* geo = (cfg->tracking == PIC_TRACK_REFMAPPING && (m->n_periodic_vectors == 0 || cfg->periodic_tracing)) ? bc_geometry(m) : NULL;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) reduction(+ : nlost, nhop, ntol) schedule(static)
#endif
  for (int ip = 0; ip < p->n; ++ip) {
    if (!p->inside[ip]) continue;
    if (cfg->tracking == PIC_TRACK_TRIA) {
      if (p->last_elem[ip] == 0) continue;    /* particle_triatracking.f90:101 */
      tria_track_single(cfg, m, p, ip, &nlost, &nhop);
    } else {
      ref_track_single(cfg, m, geo, p, ip, &ntol, &nhop);
    }
  }
  free(geo);
  (void)nthreads;
  if (c) { c->n_lost += nlost; c->n_hop_limit += nhop; c->n_ref_tolerance += ntol; }
}

/* ---------------------------------------------------------------------------------------
 * Deposition (pic_depo.f90:944-1025)
 * ------------------------------------------------------------------------------------- */
/* one particle's CVWM node scatter, pic_depo_method.f90:471-544 */
static void cvwm_particle(const pic_config_t* cfg, const pic_mesh_t* m, const orc_particles_t* p, int ip,
                          double* NS, int64_t* nfail) {
  const double* s = &p->part_state[(size_t)ip * 6];
  const int sp = p->species[ip] - 1, e = p->elem[ip];
  double charge = cfg->charge[sp] * cfg->mpf[sp];
  double xi[3];
  int suc = orc_get_position_in_ref_elem(cfg, m, s, xi, e, 1);
  if (!suc) (*nfail)++;
  double TS[4] = {s[3] * charge, s[4] * charge, s[5] * charge, charge};
  double w[8];
  const int32_t* ni = &m->node_info[(size_t)(e - 1) * 8];
  if (suc) {
    double a1 = 0.5 * (xi[0] + 1.0), a2 = 0.5 * (xi[1] + 1.0), a3 = 0.5 * (xi[2] + 1.0);
    w[0] = (1 - a1) * (1 - a2) * (1 - a3);
    w[1] = (a1) * (1 - a2) * (1 - a3);
    w[2] = (a1) * (a2) * (1 - a3);
    w[3] = (1 - a1) * (a2) * (1 - a3);
    w[4] = (1 - a1) * (1 - a2) * (a3);
    w[5] = (a1) * (1 - a2) * (a3);
    w[6] = (a1) * (a2) * (a3);
    w[7] = (1 - a1) * (a2) * (a3);
    for (int iN = 0; iN < 8; ++iN) {
      int node = ni[iN];
      for (int v = 0; v < 4; ++v) NS[(size_t)(node - 1) * 4 + v] = NS[(size_t)(node - 1) * 4 + v] + (TS[v] * w[iN]);
      if (m->n_periodic_vectors > 0 && m->periodic_n_nodes[node - 1] > 0) {
        int o = m->periodic_offset[node - 1];
        for (int j = 0; j < m->periodic_n_nodes[node - 1]; ++j) {
          int tw = m->periodic_nodes[o + j];
          for (int v = 0; v < 4; ++v) NS[(size_t)(tw - 1) * 4 + v] = NS[(size_t)(tw - 1) * 4 + v] + (TS[v] * w[iN]);
        }
      }
    }
  } else {
    const int32_t* en = &m->elem_node[(size_t)(e - 1) * 8];
    for (int iN = 0; iN < 8; ++iN) {
      double v0 = NODE(m, 0, en[iN]) - s[0], v1 = NODE(m, 1, en[iN]) - s[1], v2 = NODE(m, 2, en[iN]) - s[2];
      double norm = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
      if (norm > 0.0) w[iN] = 1.0 / norm;
      else { for (int q = 0; q < 8; ++q) w[q] = 0.0; w[iN] = 1.0; break; }
    }
    double DistSum = 0.0;
    for (int iN = 0; iN < 8; ++iN) DistSum = DistSum + w[iN];
    for (int iN = 0; iN < 8; ++iN) {
      int node = ni[iN];
      for (int v = 0; v < 4; ++v) NS[(size_t)(node - 1) * 4 + v] = NS[(size_t)(node - 1) * 4 + v] + w[iN] / DistSum * TS[v];
      if (m->n_periodic_vectors > 0 && m->periodic_n_nodes[node - 1] > 0) {
        int o = m->periodic_offset[node - 1];
        for (int j = 0; j < m->periodic_n_nodes[node - 1]; ++j) {
          int tw = m->periodic_nodes[o + j];
          for (int v = 0; v < 4; ++v) NS[(size_t)(tw - 1) * 4 + v] = NS[(size_t)(tw - 1) * 4 + v] + w[iN] / DistSum * TS[v];
        }
      }
    }
  }
}

/* DepositionMethod_CVWM, pic_depo_method.f90:373-744 */
static int deposit_cvwm(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, double* PS, orc_counters_t* c,
                        int nthreads) {
  const int N0 = cfg->n_dg;
  const size_t nn = (size_t)m->n_nodes * 4;
  int nt = nthreads > 0 ? nthreads : 1;
  double* NS = (double*)calloc(nn * (size_t)nt, sizeof(double));
  if (!NS) return 1;
  int64_t nfail = 0;
  if (nt == 1) {
    for (int ip = 0; ip < p->n; ++ip) {
      if (!p->inside[ip]) continue;
      if (cfg->charge[p->species[ip] - 1] == 0.0) continue;    /* isDepositParticle */
      cvwm_particle(cfg, m, p, ip, NS, &nfail);
    }
  } else {
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(+ : nfail)
    {
      double* my = NS + nn * (size_t)omp_get_thread_num();
#pragma omp for schedule(static)
      for (int ip = 0; ip < p->n; ++ip) {
        if (!p->inside[ip]) continue;
        if (cfg->charge[p->species[ip] - 1] == 0.0) continue;
        cvwm_particle(cfg, m, p, ip, my, &nfail);
      }
    }
    for (int t = 1; t < nt; ++t)
      for (size_t q = 0; q < nn; ++q) NS[q] = NS[q] + NS[nn * (size_t)t + q];
#endif
  }
  for (int node = 0; node < m->n_nodes; ++node) {                    /* :692-695 */
    double V = m->node_volume[node];
    if (V > 0.0) for (int v = 0; v < 4; ++v) NS[(size_t)node * 4 + v] = NS[(size_t)node * 4 + v] / V;
  }
  for (int e = 1; e <= m->n_elems; ++e) {                            /* :710-733 */
    /* CellVolWeight(Nloc)%Fac, pic_depo.f90:274-275, with Nloc = N_DG_Mapping(2,e) (:714) */
    const int N = elem_n(m, N0, e), n1 = N + 1;
    const double* xgp = n_inter(m, N, 0);
    double Fac[8];
    for (int i = 0; i <= N; ++i) Fac[i] = (xgp[i] + 1.0) / 2.0;
    const int32_t* ni = &m->node_info[(size_t)(e - 1) * 8];
    double* ps = &PS[dof_off(m, N0, e) * 4];
    for (int kk = 0; kk <= N; ++kk)
      for (int ll = 0; ll <= N; ++ll)
        for (int mm = 0; mm <= N; ++mm) {
          double a1 = Fac[kk], a2 = Fac[ll], a3 = Fac[mm];
          int r = kk + n1 * (ll + n1 * mm);
          for (int v = 0; v < 4; ++v) {
            const double* S = NS + v;
            ps[(size_t)r * 4 + v] =
                S[(size_t)(ni[0] - 1) * 4] * (1 - a1) * (1 - a2) * (1 - a3) +
                S[(size_t)(ni[1] - 1) * 4] * (a1) * (1 - a2) * (1 - a3) +
                S[(size_t)(ni[2] - 1) * 4] * (a1) * (a2) * (1 - a3) +
                S[(size_t)(ni[3] - 1) * 4] * (1 - a1) * (a2) * (1 - a3) +
                S[(size_t)(ni[4] - 1) * 4] * (1 - a1) * (1 - a2) * (a3) +
                S[(size_t)(ni[5] - 1) * 4] * (a1) * (1 - a2) * (a3) +
                S[(size_t)(ni[6] - 1) * 4] * (a1) * (a2) * (a3) +
                S[(size_t)(ni[7] - 1) * 4] * (1 - a1) * (a2) * (a3);
          }
        }
  }
  free(NS);
  if (c) c->n_newton_failed += nfail;
  return 0;
}

/* w_sf for the 3D shape function, pic_depo_shapefunction_tools.f90:1243-1246 with beta()
 * from pic_depo_tools.f90:491-511 */
/* shape-function dimension (InitShapeFunctionDimensionalty, pic_depo_shapefunction_tools.f90:1131-1294):
 * dim 1: kernel along dir; dim 2: kernel in d1, d2, constant along dir (0-based directions) */
typedef struct { int dim, dir, d1, d2; } sf_geom_t;
static sf_geom_t sf_geom(const pic_config_t* cfg) {
  sf_geom_t g;
  g.dim = cfg->sf_dim ? cfg->sf_dim : 3;
  g.dir = (cfg->sf_dir >= 1 && cfg->sf_dir <= 3 ? cfg->sf_dir : 1) - 1;
  g.d1 = (g.dir == 1) ? 0 : 1;             /* dim_sf_dir1 = MERGE(1,2,dim_sf_dir.EQ.2) */
  g.d2 = (g.dir == 2) ? 0 : 2;             /* dim_sf_dir2 = MERGE(1,3,dim_sf_dir.EQ.3) */
  return g;
}
/* SFRadius2 and SFNorm (pic_depo_shapefunction_tools.f90:997-1058) */
static double sf_radius2(const sf_geom_t* g, const double v[3]) {
  if (g->dim == 1) return v[g->dir] * v[g->dir];
  if (g->dim == 2) return v[g->d1] * v[g->d1] + v[g->d2] * v[g->d2];
  return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
}
static double sf_norm(const sf_geom_t* g, const double v[3]) {
  if (g->dim == 1) return fabs(v[g->dir]);
  if (g->dim == 2) return sqrt(v[g->d1] * v[g->d1] + v[g->d2] * v[g->d2]);
  return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

/* dimFactorSF (InitShapeFunctionDimensionalty): 1D the cross-section across the kernel direction, 2D the
 * extent along the constant direction; 1 for the 3D kernel.  sf_charge_on_line: 1D/2D kernels with
 * PIC-shapefunction-3D-deposition = F, whose charge-conserving totals are divided by it */
static double sf_dim_factor(const pic_config_t* cfg, const pic_mesh_t* m) {
  const sf_geom_t g = sf_geom(cfg);
  double ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = m->xmax_glob[d] - m->xmin_glob[d];
  if (g.dim == 1) return (g.dir == 0) ? ext[1] * ext[2] : (g.dir == 1) ? ext[0] * ext[2] : ext[0] * ext[1];
  if (g.dim == 2) return ext[g.dir];
  return 1.0;
}
static int sf_charge_on_line(const pic_config_t* cfg) {
  const sf_geom_t g = sf_geom(cfg);
  return g.dim < 3 && !cfg->sf_depo3d;
}

static double sf_w(const pic_config_t* cfg, const pic_mesh_t* m, double r_sf, int alpha) {
  const double PI = acos(-1.0);
  const sf_geom_t g = sf_geom(cfg);
  const int depo3d = cfg->sf_dim == 0 || cfg->sf_depo3d;
  double ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = m->xmax_glob[d] - m->xmin_glob[d];
  if (g.dim == 1) {
    double dimFactor = (g.dir == 0) ? ext[1] * ext[2] : (g.dir == 1) ? ext[0] * ext[2] : ext[0] * ext[1];
    double a = tgamma((double)alpha + 1.5);
    double b = sqrt(PI) * r_sf * tgamma((double)(alpha + 1));
    return depo3d ? a / (b * dimFactor) : a / b;
  }
  if (g.dim == 2) {
    double dimFactor = ext[g.dir];
    return depo3d ? ((double)alpha + 1.0) / (PI * (r_sf * r_sf) * dimFactor) : ((double)alpha + 1.0) / (PI * (r_sf * r_sf));
  }
  double BetaFac = tgamma(1.5) * tgamma((double)alpha + 1.0) / tgamma(1.5 + ((double)alpha + 1.0));
  return 1.0 / (2.0 * BetaFac * (double)alpha + 2.0 * BetaFac) * ((double)alpha + 1.0) / (PI * (r_sf * r_sf * r_sf));
}

/* GetPartPosShifted (pic_depo_shapefunction_tools.f90:1061-1124) for periodic case ic (0-based) with
 * PeriodicSFCaseMatrix (pic_depo.f90:865-888); dims 1 and 2 on a box with one periodic vector per axis */
static void sf_shifted(const sf_geom_t* g, const pic_mesh_t* m, int ic, const double P[3], double Ps[3]) {
#define PV(i, k) m->periodic_vectors[3 * (k) + (i)]
  if (g->dim == 1) {
    const double c = (double)(1 - ic);
    Ps[0] = Ps[1] = Ps[2] = 0.0;
    Ps[g->dir] = P[g->dir] + c * PV(g->dir, g->dir);
  } else if (g->dim == 2) {
    const double c1 = (double)(1 - ic / 3), c2 = (double)(1 - ic % 3);
    const int v1 = g->d1, v2 = g->d2;          /* dim_periodic_vec1/2 for three periodic vectors */
    Ps[g->dir] = P[g->dir];
    Ps[g->d1] = P[g->d1] + c1 * PV(g->d1, v1);
    Ps[g->d2] = P[g->d2] + c1 * PV(g->d2, v1);
    Ps[g->d1] = Ps[g->d1] + c2 * PV(g->d1, v2);
    Ps[g->d2] = Ps[g->d2] + c2 * PV(g->d2, v2);
  } else {
    const double c1 = (double)(1 - ic / 9), c2 = (double)(1 - (ic / 3) % 3), c3 = (double)(1 - ic % 3);
    for (int d = 0; d < 3; ++d) Ps[d] = P[d] + c1 * PV(d, 0) + c2 * PV(d, 1) + c3 * PV(d, 2);
  }
#undef PV
}

/* depoChargeOnDOFsSF, pic_depo_shapefunction_tools.f90:292-422 */
static void depo_charge_on_dofs_sf(const pic_config_t* cfg, const pic_mesh_t* m, const double P[3], const double Fac[4],
                                   double r_sf, double r2_sf, double r2_sf_inv, double* PS, uint8_t* done) {
  const int N0 = cfg->n_dg;
  const sf_geom_t g = sf_geom(cfg);
  memset(done, 0, (size_t)m->n_elems);
  int kmax = (int)ceil((P[0] + r_sf - m->xmin_glob[0]) / m->fibgm_deltas[0]);
  int kmin = (int)floor((P[0] - r_sf - m->xmin_glob[0]) / m->fibgm_deltas[0] + 1);
  int lmax = (int)ceil((P[1] + r_sf - m->xmin_glob[1]) / m->fibgm_deltas[1]);
  int lmin = (int)floor((P[1] - r_sf - m->xmin_glob[1]) / m->fibgm_deltas[1] + 1);
  int mmax = (int)ceil((P[2] + r_sf - m->xmin_glob[2]) / m->fibgm_deltas[2]);
  int mmin = (int)floor((P[2] - r_sf - m->xmin_glob[2]) / m->fibgm_deltas[2] + 1);
  /* 1D/2D: every background cell across the directions without kernel (:346-377) */
  if (g.dim < 3) {
    int full[3] = {0, 0, 0};
    if (g.dim == 2) full[g.dir] = 1;
    else { full[0] = full[1] = full[2] = 1; full[g.dir] = 0; }
    if (full[0]) { kmin = 1; kmax = m->fibgm_imax[0]; }
    if (full[1]) { lmin = 1; lmax = m->fibgm_imax[1]; }
    if (full[2]) { mmin = 1; mmax = m->fibgm_imax[2]; }
  }
  if (kmax > m->fibgm_imax[0]) kmax = m->fibgm_imax[0];
  if (kmin < 1) kmin = 1;
  if (lmax > m->fibgm_imax[1]) lmax = m->fibgm_imax[1];
  if (lmin < 1) lmin = 1;
  if (mmax > m->fibgm_imax[2]) mmax = m->fibgm_imax[2];
  if (mmin < 1) mmin = 1;
  for (int kk = kmin; kk <= kmax; ++kk)
    for (int ll = lmin; ll <= lmax; ++ll)
      for (int mm = mmin; mm <= mmax; ++mm) {
        size_t cidx = (size_t)(kk - 1) + (size_t)m->fibgm_imax[0] * ((ll - 1) + (size_t)m->fibgm_imax[1] * (mm - 1));
        int nE = m->fibgm_n_elems[cidx], off = m->fibgm_offset[cidx];
        for (int q = 0; q < nE; ++q) {
          int e = m->fibgm_element[off + q];
          if (done[e - 1]) continue;
          const double* b = &m->elem_bary[(size_t)(e - 1) * 3];
          const double vb[3] = {P[0] - b[0], P[1] - b[1], P[2] - b[2]};
          if (sf_norm(&g, vb) > (r_sf + m->elem_radius[e - 1])) continue;
          const int N = elem_n(m, N0, e), n1 = N + 1;       /* Nloc, offSetDof: :398-399 */
          const double* xg = &m->elem_xgp[dof_off(m, N0, e) * 3];
          double* ps = &PS[dof_off(m, N0, e) * 4];
          for (int mz = 0; mz <= N; ++mz)
            for (int l = 0; l <= N; ++l)
              for (int k = 0; k <= N; ++k) {
                int r = mz * n1 * n1 + l * n1 + k;
                const double dv[3] = {P[0] - xg[(size_t)r * 3], P[1] - xg[(size_t)r * 3 + 1], P[2] - xg[(size_t)r * 3 + 2]};
                double radius2 = sf_radius2(&g, dv);
                if (radius2 <= r2_sf) {
                  double S = 1.0 - r2_sf_inv * radius2;
                  double S1 = S * S;
                  for (int ex = 3; ex <= cfg->sf_alpha; ++ex) S1 = S * S1;
                  for (int v = 0; v < 4; ++v) ps[(size_t)r * 4 + v] = ps[(size_t)r * 4 + v] + S1 * Fac[v];
                }
              }
          done[e - 1] = 1;
        }
      }
}

/* the FIBGM cell range of calcTotalChargePeriodic_cc / depoChargeOnDOFsSF(ChargeCon)
 * (pic_depo_shapefunction_tools.f90:330-377): within r_sf of P along the kernel directions, every cell
 * across the others, clamped to the grid */
static void sf_cell_range(const sf_geom_t* g, const pic_mesh_t* m, const double P[3], double r_sf, int lo[3], int hi[3]) {
  int full[3] = {0, 0, 0};
  if (g->dim == 2) full[g->dir] = 1;
  else if (g->dim == 1) { full[0] = full[1] = full[2] = 1; full[g->dir] = 0; }
  for (int d = 0; d < 3; ++d) {
    hi[d] = (int)ceil((P[d] + r_sf - m->xmin_glob[d]) / m->fibgm_deltas[d]);
    lo[d] = (int)floor((P[d] - r_sf - m->xmin_glob[d]) / m->fibgm_deltas[d] + 1);
    if (full[d]) { lo[d] = 1; hi[d] = m->fibgm_imax[d]; }
    if (hi[d] > m->fibgm_imax[d]) hi[d] = m->fibgm_imax[d];
    if (lo[d] < 1) lo[d] = 1;
  }
}

/* calcTotalChargePeriodic_cc, pic_depo_shapefunction_tools.f90:425-555: the quadrature integral
 * sum wGP(k) wGP(l) wGP(m) Fac S1 / sJ over the DOFs within r_sf (SFRadius2) of one (shifted) position, added
 * term by term to the running total (totalChargePeriodicSF is INOUT across the periodic cases) */
static double total_charge_cc(const pic_config_t* cfg, const pic_mesh_t* m, const double P[3], double Fac4,
                              double totalCharge, double r_sf, double r2_sf, double r2_sf_inv, uint8_t* done) {
  const int N0 = cfg->n_dg;
  const sf_geom_t g = sf_geom(cfg);
  memset(done, 0, (size_t)m->n_elems);
  int lo[3], hi[3];
  sf_cell_range(&g, m, P, r_sf, lo, hi);
  for (int kk = lo[0]; kk <= hi[0]; ++kk)
    for (int ll = lo[1]; ll <= hi[1]; ++ll)
      for (int mm = lo[2]; mm <= hi[2]; ++mm) {
        size_t cidx = (size_t)(kk - 1) + (size_t)m->fibgm_imax[0] * ((ll - 1) + (size_t)m->fibgm_imax[1] * (mm - 1));
        int nE = m->fibgm_n_elems[cidx], off = m->fibgm_offset[cidx];
        for (int q = 0; q < nE; ++q) {
          int e = m->fibgm_element[off + q];
          if (done[e - 1]) continue;
          const double* b = &m->elem_bary[(size_t)(e - 1) * 3];
          const double vb[3] = {P[0] - b[0], P[1] - b[1], P[2] - b[2]};
          if (sf_norm(&g, vb) > (r_sf + m->elem_radius[e - 1])) continue;
          const int N = elem_n(m, N0, e), n1 = N + 1;       /* Nloc, offSetDof(Node): :530-532 */
          const double* wgp = n_inter(m, N, 1);
          const double* xg = &m->elem_xgp[dof_off(m, N0, e) * 3];
          const double* sj = &m->elem_sj[dof_off(m, N0, e)];
          for (int mz = 0; mz <= N; ++mz)
            for (int l = 0; l <= N; ++l)
              for (int k = 0; k <= N; ++k) {
                int r = mz * n1 * n1 + l * n1 + k;
                const double dv[3] = {P[0] - xg[(size_t)r * 3], P[1] - xg[(size_t)r * 3 + 1], P[2] - xg[(size_t)r * 3 + 2]};
                double radius2 = sf_radius2(&g, dv);
                if (radius2 <= r2_sf) {
                  double S = 1.0 - r2_sf_inv * radius2;
                  double S1 = S * S;
                  for (int ex = 3; ex <= cfg->sf_alpha; ++ex) S1 = S * S1;
                  totalCharge = totalCharge + wgp[k] * wgp[l] * wgp[mz] * Fac4 * S1 / sj[r];
                }
              }
          done[e - 1] = 1;
        }
      }
  return totalCharge;
}

/* ElemToElemMapping/ElemToElemInfo of particle_mesh_build.f90:1244-1380: for every element, the other
 * elements sharing one of its unique corner nodes, in the order met when walking the corners (CGNS order)
 * and, per node, the elements of NodeToElemInfo (ascending, :1150-1243).  off has n_elems + 1 entries. */
static int build_elem_to_elem(const pic_mesh_t* m, int** off_out, int** info_out) {
  const int ne = m->n_elems;
  int nn = 0;
  for (size_t q = 0; q < (size_t)ne * 8; ++q) nn = m->node_info[q] > nn ? m->node_info[q] : nn;
  int* ncnt = (int*)calloc((size_t)nn + 1, sizeof(int));
  int* noff = (int*)calloc((size_t)nn + 2, sizeof(int));
  int* ninfo = (int*)malloc(sizeof(int) * (size_t)ne * 8);
  int* off = (int*)calloc((size_t)ne + 1, sizeof(int));
  int* info = (int*)malloc(sizeof(int) * (size_t)ne * 8 * 8);
  if (!ncnt || !noff || !ninfo || !off || !info) {
    free(ncnt); free(noff); free(ninfo); free(off); free(info);
    return 1;
  }
  for (size_t q = 0; q < (size_t)ne * 8; ++q) ncnt[m->node_info[q]]++;
  for (int u = 1; u <= nn; ++u) noff[u + 1] = noff[u] + ncnt[u];
  memset(ncnt, 0, sizeof(int) * ((size_t)nn + 1));
  for (int e = 0; e < ne; ++e)
    for (int c = 0; c < 8; ++c) {
      const int u = m->node_info[(size_t)e * 8 + c];
      ninfo[noff[u] + ncnt[u]++] = e + 1;
    }
  int tot = 0;
  for (int e = 0; e < ne; ++e) {
    const int start = tot;
    for (int c = 0; c < 8; ++c) {
      const int u = m->node_info[(size_t)e * 8 + c];
      for (int j = noff[u]; j < noff[u] + ncnt[u]; ++j) {
        const int t = ninfo[j];
        if (t == e + 1) continue;
        int dup = 0;
        for (int k = start; k < tot && !dup; ++k) dup = info[k] == t;
        if (!dup) info[tot++] = t;
      }
    }
    off[e + 1] = tot;
  }
  free(ncnt); free(noff); free(ninfo);
  *off_out = off;
  *info_out = info;
  return 0;
}

/* depoChargeOnDOFsSFChargeCon (pic_depo_shapefunction_tools.f90:558-755; shape_function_cc without periodic
 * vectors) and depoChargeOnDOFsSFAdaptive (:758-908; shape_function_adaptive without periodic vectors): the
 * kernel Fac S1 at every DOF within R of the particle in the listed elements, its quadrature integral
 * totalCharge = sum wGP(k) wGP(l) wGP(m) (Fac(4) S1) / sJ in visiting order, and the deposit
 * (Fac(4)/totalCharge) * (Fac S1).  The elements are visited in list order, skipping repeats (ChargeSFDone)
 * and those whose barycentre lies beyond R + ElemRadiusNGeo.  ChargeCon evaluates S = 1 - R^-2 r^2,
 * Adaptive S = 1 - r^2/R^2.  The pass that deposits repeats the first pass's arithmetic. */
static void depo_charge_con(const pic_config_t* cfg, const pic_mesh_t* m, const double P[3], const double Fac[4],
                            double r_sf, double r2_sf, double r2_sf_inv, int divide, double total_div,
                            const int* list, int nlist, double* PS, uint8_t* done, int* used) {
  const int N0 = cfg->n_dg;
  const sf_geom_t g = sf_geom(cfg);
  memset(done, 0, (size_t)m->n_elems);
  int nused = 0;
  double totalCharge = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass && total_div != 1.0) totalCharge = totalCharge / total_div;     /* the Adaptive branch, :881-884 */
    const double alpha = pass ? Fac[3] / totalCharge : 0.0;
    const int n = pass ? nused : nlist;
    for (int q = 0; q < n; ++q) {
      const int e = pass ? used[q] : list[q];
      if (!pass) {
        if (done[e - 1]) continue;
        const double* b = &m->elem_bary[(size_t)(e - 1) * 3];
        const double vb[3] = {P[0] - b[0], P[1] - b[1], P[2] - b[2]};
        if (sf_norm(&g, vb) > (r_sf + m->elem_radius[e - 1])) continue;
      }
      const int N = elem_n(m, N0, e), n1 = N + 1;           /* Nloc, offSetDof(Node): :682-684 */
      const double* wgp = n_inter(m, N, 1);
      const double* xg = &m->elem_xgp[dof_off(m, N0, e) * 3];
      const double* sj = &m->elem_sj[dof_off(m, N0, e)];
      double* ps = &PS[dof_off(m, N0, e) * 4];
      int hit = 0;
      for (int mz = 0; mz <= N; ++mz)
        for (int l = 0; l <= N; ++l)
          for (int k = 0; k <= N; ++k) {
            const int r = mz * n1 * n1 + l * n1 + k;
            const double dv[3] = {P[0] - xg[(size_t)r * 3], P[1] - xg[(size_t)r * 3 + 1], P[2] - xg[(size_t)r * 3 + 2]};
            const double radius2 = sf_radius2(&g, dv);
            if (!(radius2 <= r2_sf)) continue;
            hit = 1;
            const double S = divide ? 1.0 - radius2 / r2_sf : 1.0 - r2_sf_inv * radius2;
            double S1 = S * S;
            for (int ex = 3; ex <= cfg->sf_alpha; ++ex) S1 = S * S1;
            if (!pass) {
              totalCharge = totalCharge + wgp[k] * wgp[l] * wgp[mz] * (Fac[3] * S1) / sj[r];
            } else {
              for (int v = 0; v < 4; ++v) ps[(size_t)r * 4 + v] = ps[(size_t)r * 4 + v] + alpha * (Fac[v] * S1);
            }
          }
      if (!pass) {
        if (hit) used[nused++] = e;
        done[e - 1] = 1;
      }
    }
    if (!nused) return;
  }
}

/* the FIBGM cells of sf_cell_range, their elements in visiting order,
 * each at its first appearance (a later one is skipped or fails the same barycentre test) */
static int fibgm_visit_list(const pic_config_t* cfg, const pic_mesh_t* m, const double P[3], double r_sf, int* list,
                            uint8_t* seen) {
  int lo[3], hi[3], n = 0;
  const sf_geom_t g = sf_geom(cfg);
  memset(seen, 0, (size_t)m->n_elems);
  sf_cell_range(&g, m, P, r_sf, lo, hi);
  for (int kk = lo[0]; kk <= hi[0]; ++kk)
    for (int ll = lo[1]; ll <= hi[1]; ++ll)
      for (int mm = lo[2]; mm <= hi[2]; ++mm) {
        size_t cidx = (size_t)(kk - 1) + (size_t)m->fibgm_imax[0] * ((ll - 1) + (size_t)m->fibgm_imax[1] * (mm - 1));
        int nE = m->fibgm_n_elems[cidx], off = m->fibgm_offset[cidx];
        for (int q = 0; q < nE; ++q) {
          const int e = m->fibgm_element[off + q];
          if (!seen[e - 1]) { seen[e - 1] = 1; list[n++] = e; }
        }
      }
  return n;
}

/* DepositionMethod_SF, pic_depo_method.f90:851-1003 + calcSfSource (shapefunction_tools:30-164);
 * shape_function_cc with periodic images: calcSfSource:96-120 (totalChargePeriodicSF, Fac*Fac(4)/total) */
static int deposit_sf(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, double* PS, int nthreads) {
  const size_t nps = orc_n_dofs(m, cfg->n_dg) * 4;
  const double r_sf = cfg->sf_radius, r2_sf = r_sf * r_sf, r2_sf_inv = 1.0 / r2_sf;
  const double w_sf = sf_w(cfg, m, r_sf, cfg->sf_alpha);
  int nt = nthreads > 0 ? nthreads : 1;
  const sf_geom_t gsf = sf_geom(cfg);
  /* NbrOfPeriodicSFCases = 3**dim_sf with periodic vectors, else 0 (pic_depo.f90:849-861) */
  int nCases = (m->n_periodic_vectors > 0) ? (gsf.dim == 1 ? 3 : gsf.dim == 2 ? 9 : 27) : 0;
  double* acc = PS;
  if (nt > 1) { acc = (double*)calloc(nps * (size_t)nt, sizeof(double)); if (!acc) return 1; }
  uint8_t* doneAll = (uint8_t*)malloc((size_t)m->n_elems * (size_t)nt);
  if (!doneAll) { if (acc != PS) free(acc); return 1; }
  /* the non-periodic charge-conserving branches of calcSfSource (:136-160): element lists and scratch */
  const int con = nCases == 0 && (cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_CC ||
                                  cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE);
  int *e2e_off = NULL, *e2e_info = NULL, *lists = NULL;
  const int lcap = m->n_elems + 1;
  if (con) {
    if (cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE && build_elem_to_elem(m, &e2e_off, &e2e_info)) {
      if (acc != PS) free(acc);
      free(doneAll);
      return 1;
    }
    lists = (int*)malloc(sizeof(int) * (size_t)lcap * 2 * (size_t)nt);
    if (!lists) { if (acc != PS) free(acc); free(doneAll); free(e2e_off); free(e2e_info); return 1; }
  }
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double* my = (nt > 1) ? acc + nps * (size_t)tid : PS;
    uint8_t* done = doneAll + (size_t)m->n_elems * tid;
    const int adaptive = cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int ip = 0; ip < p->n; ++ip) {
      if (!p->inside[ip]) continue;
      const int sp = p->species[ip] - 1;
      if (cfg->charge[sp] == 0.0) continue;
      const double* s = &p->part_state[(size_t)ip * 6];
      double cm = cfg->charge[sp] * cfg->mpf[sp];
      double Fac[4] = {s[3] * cm, s[4] * cm, s[5] * cm, cm};
      /* shape_function_adaptive: the radius of the particle's element (calcSfSource:83-92) */
      double r_sf_p = r_sf, r2_sf_p = r2_sf, r2_sf_inv_p = r2_sf_inv;
      if (adaptive) {
        r_sf_p = m->sf_elem_radius[p->elem[ip] - 1];
        r2_sf_p = r_sf_p * r_sf_p;
        r2_sf_inv_p = 1.0 / r2_sf_p;
      }
      if (nCases > 1) {
        if (cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_CC || adaptive) {
          double totalCharge = 0.0;
          for (int ic = 0; ic < nCases; ++ic) {
            double Ps[3];
            sf_shifted(&gsf, m, ic, s, Ps);
            totalCharge = total_charge_cc(cfg, m, Ps, Fac[3], totalCharge, r_sf_p, r2_sf_p, r2_sf_inv_p, done);
          }
          if (sf_charge_on_line(cfg)) totalCharge = totalCharge / sf_dim_factor(cfg, m);   /* :117-119 */
          const double f4 = Fac[3];
          for (int v = 0; v < 4; ++v) Fac[v] = Fac[v] * f4 / totalCharge;
        } else {
          for (int v = 0; v < 4; ++v) Fac[v] = Fac[v] * w_sf;
        }
        for (int ic = 0; ic < nCases; ++ic) {
          double Ps[3];
          sf_shifted(&gsf, m, ic, s, Ps);
          depo_charge_on_dofs_sf(cfg, m, Ps, Fac, r_sf_p, r2_sf_p, r2_sf_inv_p, my, done);
        }
      } else if (con) {
        int* list = lists + (size_t)lcap * 2 * tid;
        int* used = list + lcap;
        int nl;
        if (adaptive) {
          const int e0 = p->elem[ip];
          list[0] = e0;
          nl = 1;
          for (int j = e2e_off[e0 - 1]; j < e2e_off[e0]; ++j) list[nl++] = e2e_info[j];
        } else {
          nl = fibgm_visit_list(cfg, m, s, r_sf, list, done);
        }
        /* only the Adaptive branch divides its total by dimFactorSF (:881-884; ChargeCon does not) */
        const double tdiv = adaptive && sf_charge_on_line(cfg) ? sf_dim_factor(cfg, m) : 1.0;
        depo_charge_con(cfg, m, s, Fac, r_sf_p, r2_sf_p, r2_sf_inv_p, adaptive, tdiv, list, nl, my, done, used);
      } else {
        double Fw[4];
        for (int v = 0; v < 4; ++v) Fw[v] = Fac[v] * w_sf;
        depo_charge_on_dofs_sf(cfg, m, s, Fw, r_sf, r2_sf, r2_sf_inv, my, done);
      }
    }
  }
  if (nt > 1) {
    for (size_t q = 0; q < nps; ++q) {
      double v = 0.0;
      for (int t = 0; t < nt; ++t) v = v + acc[nps * (size_t)t + q];
      PS[q] = v;
    }
    free(acc);
  }
  free(doneAll);
  free(lists);
  free(e2e_off);
  free(e2e_info);
  return 0;
}

int orc_deposit(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, double* part_source,
                orc_counters_t* c, int nthreads) {
  memset(part_source, 0, sizeof(double) * orc_n_dofs(m, cfg->n_dg) * 4);   /* pic_depo.f90:1004-1007 */
  if (cfg->deposition == PIC_DEPO_CVWM) return deposit_cvwm(cfg, m, p, part_source, c, nthreads);
  return deposit_sf(cfg, m, p, part_source, nthreads);
}

/* One TimeStepPoissonByBorisLeapfrog without HDG (the field stays frozen). */
int orc_step(const pic_config_t* cfg, const pic_mesh_t* m, const double* e_dof, orc_particles_t* p, double dt,
             int nsteps, double* part_source, orc_counters_t* c, int nthreads) {
  for (int it = 0; it < nsteps; ++it) {
    if (part_source) {
      int rc = orc_deposit(cfg, m, p, part_source, c, nthreads);                   /* :93 */
      if (rc) return rc;
    }
    for (int ip = 0; ip < p->n; ++ip) {                                            /* :109-110 */
      for (int d = 0; d < 3; ++d) p->last_part_pos[(size_t)ip * 3 + d] = p->part_state[(size_t)ip * 6 + d];
      p->last_elem[ip] = p->elem[ip];
    }
    orc_interpolate(cfg, m, e_dof, p, c, nthreads);                                /* :122 */
    orc_push(cfg, p, dt, nthreads);                                                /* :128-198 */
    orc_track(cfg, m, p, c, nthreads);                                             /* :211 */
  }
  return 0;
}

/* VerifyDepositedCharge, pic_analyze.f90:72-91, integrating each element on its own Gauss nodes (NAnalyze =
 * Nloc, an identity change of basis): the integrand -- the degree-Nloc interpolants of PartSource(4) and
 * 1/sJ -- has degree 2 Nloc per direction, which both this rule and the reference's NAnalyze grid with
 * NAnalyze > Nloc integrate exactly, so the two agree up to rounding */
double orc_integrate_charge(const pic_mesh_t* m, int N0, const double* PS) {
  double total = 0.0;
  for (int e = 0; e < m->n_elems; ++e) {
    const int N = elem_n(m, N0, e + 1), n1 = N + 1;
    const double* wgp = n_inter(m, N, 1);
    const size_t e0 = dof_off(m, N0, e + 1);
    double loc = 0.0;
    for (int mm = 0; mm <= N; ++mm)
      for (int l = 0; l <= N; ++l)
        for (int k = 0; k <= N; ++k) {
          int r = k + n1 * (l + n1 * mm);
          double J = 1.0 / m->elem_sj[e0 + r];
          double w = wgp[k] * wgp[l] * wgp[mm] * J;
          loc = loc + w * PS[(e0 + r) * 4 + 3];
        }
    total = total + loc;
  }
  return total;
}

void orc_map_particles(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(static)
#endif
  for (int ip = 0; ip < p->n; ++ip) {
    if (!p->inside[ip]) continue;
    orc_get_position_in_ref_elem(cfg, m, &p->part_state[(size_t)ip * 6], &p->part_pos_ref[(size_t)ip * 3], p->elem[ip], 0);
  }
  (void)nthreads;
}
