/*
 * pic_oracle_bezier.c -- CPU restatement of PICLas's intersections of a particle trajectory with curved
 * (Bezier) sides: GetSideSlabNormalsAndIntervals, the side bounding-box tests, BezierNewton, Bezier clipping
 * (BezierClipRecursive, CheckXiClip, CheckEtaClip, CalcSminSmax2, calcLineNormVec3,
 * ComputeBezierIntersectionPoint) and the two drivers ComputePlanarCurvedIntersection and
 * ComputeCurvedIntersection.
 *
 * TEST INFRASTRUCTURE ONLY: part of the oracle the tests check the GPU library against.
 *
 * Files (PICLas source tree): src/particles/tracking/particle_intersection.f90,
 * src/particles/particle_mesh/particle_surfaces.f90, src/interpolation/basis.f90.  Default parameters of
 * InitParticleSurfaces (particle_surfaces.f90:133-158): BezierNewtonAngle = pi/2 (every curved side is clipped),
 * BezierClipTolerance 1e-8, BezierNewtonTolerance 1e-4, BezierNewtonGuess 1, BezierNewtonMaxIter 100,
 * BezierSplitLimit 2 x 0.6, BezierClipMaxIter 100, BezierClipLineVectorMethod 2, epsilontol 100 epsMach,
 * BezierClipHit 1 + 100 BezierClipTolerance, BezierClipMaxIntersec 2 (NGeo+1); BezierElevation 0.
 *
 * The recursion of BezierClipRecursive <-> CheckXiClip/CheckEtaClip is restated as a loop with an explicit
 * stack: at a split the first half is clipped next, and the second half is pushed together with the state the
 * reference saves around the first recursive call (clip counters, line vectors, ClipMode); when a branch
 * returns, the next pending half continues with that state -- the reference's visiting order.  The stack holds
 * 8 nested splits (as the GPU library's); deeper nesting raises the error flag, as more than
 * BezierClipMaxIntersec hits and a degenerated patch do, where the reference aborts.  Floating-point order
 * follows the Fortran (built with -ffp-contract=off).
 */
#include "pic_oracle_bezier.h"

#include <float.h>
#include <math.h>
#include <string.h>

#define BZ_EPS_MACH 2.220446049250313080847e-16
#define BZ_CLIP_TOL 1e-8
#define BZ_NEWTON_TOL2 1e-8                     /* BezierNewtonTolerance**2 */
#define BZ_NEWTON_MAXITER 100
#define BZ_SPLIT_LIMIT 1.2                      /* 2 x 0.6 */
#define BZ_CLIP_MAXITER 100
#define BZ_EPSILONTOL (100.0 * BZ_EPS_MACH)
#define BZ_CLIP_HIT (1.0 + 100.0 * BZ_CLIP_TOL)

static int almostzero(double a) { return fabs(a) <= BZ_EPS_MACH; }

static void bz_crossnorm(const double a[3], const double b[3], double n[3]) {
  n[0] = a[1] * b[2] - a[2] * b[1];
  n[1] = a[2] * b[0] - a[0] * b[2];
  n[2] = a[0] * b[1] - a[1] * b[0];
  double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  n[0] = n[0] / l; n[1] = n[1] / l; n[2] = n[2] / l;
}

/* UNITVECTOR (globals.f90) */
static void bz_unit(const double v[3], double u[3]) {
  double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (fabs(l) > 0.0) { l = 1.0 / l; u[0] = v[0] * l; u[1] = v[1] * l; u[2] = v[2] * l; }
  else { u[0] = u[1] = u[2] = 0.0; }
}

static double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r = r * x;
  return r;
}

/* FacNchooseK (BuildBezierVdm, basis.f90:275-358), Xi_NGeo (particle_mesh_tools.f90:1470-1473) and D_Bezier
 * (BuildBezierDMat, basis.f90:361-402) */
void orc_bz_basis_init(orc_bz_basis_t* B, int ng) {
  memset(B, 0, sizeof(*B));
  B->ng = ng;
  for (int i = 0; i <= ng; ++i)
    for (int j = 0; j <= i; ++j) {
      double c = 1.0;
      for (int q = 0; q < j; ++q) c = c * (double)(i - q) / (double)(q + 1);
      B->fnk[i][j] = (1.0 / ipow(2.0, i)) * c;
    }
  for (int i = 0; i <= ng; ++i) B->xi_ng[i] = 2.0 / (double)ng * (double)i - 1.0;
  for (int i = 0; i <= ng; ++i) B->dbez[i][0] = -B->fnk[ng][0] * (double)ng * ipow(1 - B->xi_ng[i], ng - 1);
  for (int i = 0; i <= ng; ++i) B->dbez[i][ng] = B->fnk[ng][ng] * (double)ng * ipow(B->xi_ng[i] + 1, ng - 1);
  for (int j = 1; j <= ng - 1; ++j)
    for (int i = 0; i <= ng; ++i) {
      const double XiPlus = B->xi_ng[i] + 1.0, XiMinus = 1.0 - B->xi_ng[i];
      B->dbez[i][j] = B->fnk[ng][j] * ((double)j * ipow(XiPlus, j - 1) * ipow(XiMinus, ng - j) -
                                       (double)(ng - j) * ipow(XiPlus, j) * ipow(XiMinus, ng - j - 1));
    }
}

/* EvaluateBezierPolynomialAndGradient, particle_surfaces.f90:474-616, for 2 or 3 components (isz); cp holds
 * the points (isz components, p fastest): cp[(q*(n+1)+p)*isz + c]; dcp (optional) the pre-computed derivatives
 * [(q*(n+1)+p)*2*isz + dd*isz + c]; point/grad optional (grad[dd*isz + c]) */
static void bz_eval(const orc_bz_basis_t* B, const double xi[2], int isz, const double* cp, const double* dcp,
                    double* point, double* grad) {
  const int n = B->ng, n1 = n + 1, M = n - 1;
  double xiup[BZ_NP], etaup[BZ_NP], xidown[BZ_NP], etadown[BZ_NP], xitild[BZ_NP], etatild[BZ_NP];
  const double MinusXi = 1.0 - xi[0], PlusXi = 1.0 + xi[0], MinusEta = 1.0 - xi[1], PlusEta = 1.0 + xi[1];
  xiup[0] = 1.0; etaup[0] = 1.0; xidown[n] = 1.0; etadown[n] = 1.0;
  for (int p = 1; p <= n; ++p) {
    xiup[p] = xiup[p - 1] * PlusXi;
    etaup[p] = etaup[p - 1] * PlusEta;
    xidown[n - p] = xidown[n - p + 1] * MinusXi;
    etadown[n - p] = etadown[n - p + 1] * MinusEta;
  }
  for (int p = 0; p <= n; ++p) { xitild[p] = xiup[p] * xidown[p]; etatild[p] = etaup[p] * etadown[p]; }
  if (point) {
    for (int c = 0; c < isz; ++c) point[c] = 0.0;
    for (int q = 0; q <= n; ++q)
      for (int p = 0; p <= n; ++p)
        for (int c = 0; c < isz; ++c)
          point[c] = point[c] + cp[(q * n1 + p) * isz + c] * B->fnk[n][p] * xitild[p] * B->fnk[n][q] * etatild[q];
  }
  if (grad) {
    for (int c = 0; c < 2 * isz; ++c) grad[c] = 0.0;
    if (dcp) {
      for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p)
          for (int dd = 0; dd < 2; ++dd)
            for (int c = 0; c < isz; ++c)
              grad[dd * isz + c] = grad[dd * isz + c] + dcp[(q * n1 + p) * 2 * isz + dd * isz + c] * B->fnk[n][p] *
                                                           xitild[p] * B->fnk[n][q] * etatild[q];
    } else {
      for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= M; ++p)
          for (int c = 0; c < isz; ++c) {
            grad[c] = grad[c] + (cp[(q * n1 + p + 1) * isz + c] - cp[(q * n1 + p) * isz + c]) * B->fnk[M][p] *
                                    xiup[p] * xidown[p + 1] * B->fnk[n][q] * etatild[q];
            grad[isz + c] = grad[isz + c] + (cp[((p + 1) * n1 + q) * isz + c] - cp[(p * n1 + q) * isz + c]) *
                                                B->fnk[n][q] * xitild[q] * B->fnk[M][p] * etaup[p] * etadown[p + 1];
          }
      for (int c = 0; c < 2 * isz; ++c) grad[c] = 0.5 * (double)n * grad[c];
    }
  }
}

/* CalcNormAndTangBezier, particle_surfaces.f90:443-471: the unit normal d/dxi x d/deta at (xi, eta) */
void orc_bz_normal(const orc_bz_side_t* S, double xi, double eta, double nv[3]) {
  const double x2[2] = {xi, eta};
  double g[6];
  bz_eval(&S->B, x2, 3, S->cp, NULL, NULL, g);
  bz_crossnorm(&g[0], &g[3], nv);
}

/* GetSideSlabNormalsAndIntervals, particle_surfaces.f90:619-816 (BezierElevation = 0).  Returns 1 when the
 * reference aborts (degenerated side). */
int orc_bz_side_init(orc_bz_side_t* S, int ng, const double* bcp) {
  memset(S, 0, sizeof(*S));
  orc_bz_basis_init(&S->B, ng);
  const int n1 = ng + 1;
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p)
      for (int c = 0; c < 3; ++c) S->cp[(q * n1 + p) * 3 + c] = bcp[(q * n1 + p) * 3 + c];
#define CP(p, q, c) S->cp[((q) * n1 + (p)) * 3 + (c)]
  double n1v[3], n2v[3], n3v[3], t[3];
  for (int c = 0; c < 3; ++c) n1v[c] = ((CP(ng, 0, c) - CP(0, 0, c)) + CP(ng, ng, c)) - CP(0, ng, c);
  if (n1v[0] == 0.0 && n1v[1] == 0.0 && n1v[2] == 0.0) return 1;
  double l = sqrt(n1v[0] * n1v[0] + n1v[1] * n1v[1] + n1v[2] * n1v[2]);
  for (int c = 0; c < 3; ++c) n1v[c] = n1v[c] / l;
  for (int c = 0; c < 3; ++c) t[c] = ((CP(0, ng, c) - CP(0, 0, c)) + CP(ng, ng, c)) - CP(ng, 0, c);
  bz_crossnorm(n1v, t, n2v);
  bz_crossnorm(n2v, n1v, n3v);
  for (int c = 0; c < 3; ++c) { S->slab_n[0][c] = n1v[c]; S->slab_n[1][c] = n2v[c]; S->slab_n[2][c] = n3v[c]; }
  for (int k = 0; k < 6; ++k) S->slab_i[k] = 0.0;
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p) {
      if (p == 0 && q == 0) continue;
      double d[3] = {CP(p, q, 0) - CP(0, 0, 0), CP(p, q, 1) - CP(0, 0, 1), CP(p, q, 2) - CP(0, 0, 2)};
      for (int i = 0; i < 3; ++i) {
        const double sk = (d[0] * S->slab_n[i][0] + d[1] * S->slab_n[i][1]) + d[2] * S->slab_n[i][2];
        if (sk < 0.0) S->slab_i[2 * i] = fmin(S->slab_i[2 * i], sk);
        else if (sk > 0.0) S->slab_i[2 * i + 1] = fmax(S->slab_i[2 * i + 1], sk);
      }
    }
#undef CP
  const double dx = fabs(S->slab_i[1] - S->slab_i[0]), dy = fabs(S->slab_i[3] - S->slab_i[2]),
               dz = fabs(S->slab_i[5] - S->slab_i[4]);
  double h = dy;
  const double w = fmin(dx, dz), len = fmax(dx, dz);
  const double dMax = fmax(h, fmax(len, w));
  if (len / dMax < 1.0e-6 || w / dMax < 1.0e-6) return 1;
  if (h / dMax < 1.0e-6) { S->slab_i[2] = 0.0; S->slab_i[3] = 0.0; h = 0.0; }
  S->bb_empty = almostzero(h / sqrt(len * len + w * w + h * h));
  return 0;
}

/* InsideBoundingBox, particle_intersection.f90:1991-2038 */
static int bz_inside_bb(const orc_bz_side_t* S, const double x[3]) {
  const double P[3] = {x[0] - S->cp[0], x[1] - S->cp[1], x[2] - S->cp[2]};
  const double e = 100.0 * BZ_EPS_MACH;
  const double y = (P[0] * S->slab_n[1][0] + P[1] * S->slab_n[1][1]) + P[2] * S->slab_n[1][2];
  if (y < S->slab_i[2] - e || y > S->slab_i[3] + e) return 0;
  const double xx = (P[0] * S->slab_n[0][0] + P[1] * S->slab_n[0][1]) + P[2] * S->slab_n[0][2];
  if (xx < S->slab_i[0] - e || xx > S->slab_i[1] + e) return 0;
  const double z = (P[0] * S->slab_n[2][0] + P[1] * S->slab_n[2][1]) + P[2] * S->slab_n[2][2];
  if (z < S->slab_i[4] - e || z > S->slab_i[5] + e) return 0;
  return 1;
}

static double bz_dot(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* the slab entry/exit parameters of direction i (BoundingBoxIntersection / FlatBoundingBoxIntersection) */
static void bz_slab_alpha(const orc_bz_side_t* S, int i, double dnk, const double xl[3], double* a1, double* a2) {
  const double d[3] = {S->cp[0] - xl[0], S->cp[1] - xl[1], S->cp[2] - xl[2]};
  const double base = bz_dot(d, S->slab_n[i]);
  if (dnk < 0.0) {
    *a1 = (base + S->slab_i[2 * i + 1]) / dnk;
    *a2 = (base + S->slab_i[2 * i]) / dnk;
  } else {
    *a1 = (base + S->slab_i[2 * i]) / dnk;
    *a2 = (base + S->slab_i[2 * i + 1]) / dnk;
  }
}

/* BoundingBoxIntersection, particle_intersection.f90:2040-2110 */
static int bz_bb_intersection(const orc_bz_side_t* S, const double traj[3], double len, const double xl[3]) {
  double a[2][3];
  for (int i = 0; i < 3; ++i) {
    double dnk = bz_dot(traj, S->slab_n[i]);
    if (fabs(dnk) < 100.0 * BZ_EPS_MACH) dnk = 100.0 * BZ_EPS_MACH;
    bz_slab_alpha(S, i, dnk, xl, &a[0][i], &a[1][i]);
  }
  const double maxv = fmax(fmax(a[0][0], a[0][1]), a[0][2]);
  const double minv = fmin(fmin(a[1][0], a[1][1]), a[1][2]);
  if (maxv <= minv) return (maxv < len + 100 * BZ_EPS_MACH) && (maxv + 100 * BZ_EPS_MACH > 0.0);
  return 0;
}

/* FlatBoundingBoxIntersection, particle_intersection.f90:2112-2207 */
static int bz_flat_bb_intersection(const orc_bz_side_t* S, const double traj[3], double len, const double xl[3]) {
  double a[2][3];
  for (int i = 0; i < 3; i += 2) {
    const double dnk = bz_dot(traj, S->slab_n[i]);
    if (fabs(dnk) < 100.0 * BZ_EPS_MACH) { a[0][i] = -DBL_MAX; a[1][i] = DBL_MAX; }
    else bz_slab_alpha(S, i, dnk, xl, &a[0][i], &a[1][i]);
  }
  const double maxv = fmax(a[0][0], a[0][2]), minv = fmin(a[1][0], a[1][2]);
  if (maxv <= minv) {
    if (maxv < 0 && minv > 0) return 1;
    return (maxv < len + 100.0 * BZ_EPS_MACH) && (maxv + 100.0 * BZ_EPS_MACH > 0.0);
  }
  return 0;
}

/* ---- Bezier clipping ----------------------------------------------------------------------------------- */
typedef struct {
  const orc_bz_side_t* S;
  const double *xl, *traj;
  double len, localTol;
  double XiArray[BZ_CLIP_MAXITER + 2][2], EtaArray[BZ_CLIP_MAXITER + 2][2];
  double locAlpha[2 * BZ_NP], locXi[2 * BZ_NP], locEta[2 * BZ_NP];
  int nInter, maxInter, err;
} bz_clip_t;

/* calcLineNormVec3, particle_intersection.f90:3285-3364 */
static int bz_line_norm_vec(int ng, const double* cp, double lnv[2][2]) {
  const int n1 = ng + 1;
#define C2(p, q, c) cp[((q) * n1 + (p)) * 2 + (c)]
  double LXi[2], Leta[2];
  for (int c = 0; c < 2; ++c) LXi[c] = (C2(0, ng, c) - C2(0, 0, c)) + (C2(ng, ng, c) - C2(ng, 0, c));
  double Length = sqrt(LXi[0] * LXi[0] + LXi[1] * LXi[1]);
  if (Length == 0.0) return 1;                                     /* the reference stops */
  LXi[0] = LXi[0] / Length; LXi[1] = LXi[1] / Length;
  for (int c = 0; c < 2; ++c) Leta[c] = (C2(ng, 0, c) - C2(0, 0, c)) + (C2(ng, ng, c) - C2(0, ng, c));
  Length = sqrt(Leta[0] * Leta[0] + Leta[1] * Leta[1]);
  if (Length == 0.0) return 1;
  Leta[0] = Leta[0] / Length; Leta[1] = Leta[1] / Length;
#undef C2
  lnv[0][0] = -LXi[1]; lnv[0][1] = LXi[0];    /* LineNormVec(1:2,1) */
  lnv[1][0] = -Leta[1]; lnv[1][1] = Leta[0];  /* LineNormVec(1:2,2) */
  return 0;
}

/* CalcSminSmax2, particle_intersection.f90:3366-3451 */
static void bz_sminmax(const orc_bz_basis_t* B, const double mm[2][BZ_NP], double* smin, double* smax, int iter) {
  const int ng = B->ng;
  double Smin = 1.5, Smax = -1.5;
  for (int p = 0; p <= ng; ++p)
    for (int q = 0; q <= ng; ++q) {
      if (p == q) continue;
      if (mm[1][p] * mm[1][q] <= 0.0) {
        const double m = (mm[1][q] - mm[1][p]) / (B->xi_ng[q] - B->xi_ng[p]);
        if (m < 0.0) Smax = fmax(Smax, B->xi_ng[q] - mm[1][q] / m);
        if (m > 0.0) Smin = fmin(Smin, B->xi_ng[q] - mm[1][q] / m);
      }
      if (mm[0][p] * mm[0][q] <= 0.0) {
        const double m = (mm[0][q] - mm[0][p]) / (B->xi_ng[q] - B->xi_ng[p]);
        if (m > 0.0) Smax = fmax(Smax, B->xi_ng[q] - mm[0][q] / m);
        if (m < 0.0) Smin = fmin(Smin, B->xi_ng[q] - mm[0][q] / m);
      }
    }
  if (mm[0][0] * mm[1][0] < 0.0) Smin = -1.0;
  if (mm[0][ng] * mm[1][ng] < 0.0) Smax = 1.0;
  if (Smax > -1.5) Smax = fmin(Smax + 20.0 * BZ_CLIP_TOL, 1.0);
  if (Smin < 1.5) Smin = fmax(Smin - 20.0 * BZ_CLIP_TOL, -1.0);
  if (iter == 0) {
    if (Smin == 1.5) Smin = -1.0;
    if (Smax == -1.5) Smax = 1.0;
  }
  *smin = Smin; *smax = Smax;
}

/* the de Casteljau products of CheckXiClip/CheckEtaClip: the Bernstein weights XiBuf(p,l) = up^l down^(p-l)
 * FacNchooseK(p,l) with up = plus, down = minus */
static void bz_buf(const orc_bz_basis_t* B, double plus, double minus, double buf[BZ_NP][BZ_NP]) {
  const int ng = B->ng;
  double up[BZ_NP], down[BZ_NP];
  up[0] = 1.0; down[0] = 1.0;
  for (int l = 1; l <= ng; ++l) { up[l] = up[l - 1] * plus; down[l] = down[l - 1] * minus; }
  for (int p = 0; p <= ng; ++p)
    for (int l = 0; l <= p; ++l) buf[p][l] = up[l] * down[p - l] * B->fnk[p][l];
}

/* out(:, p, q) = sum_l in(:, l, q) buf(p, l) along direction dir (0: xi index p, 1: eta index),
 * from the low end (rev 0) or mirrored from the high end (rev 1: out(:, N-p) = sum_l in(:, N-l) buf(p, l)) */
static void bz_sub(int ng, const double buf[BZ_NP][BZ_NP], const double* in, double* out, int dir, int rev) {
  const int n1 = ng + 1;
  for (int k = 0; k < n1 * n1 * 2; ++k) out[k] = 0.0;
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p)
      for (int l = 0; l <= p; ++l) {
        const int po = rev ? ng - p : p, li = rev ? ng - l : l;
        const int o = dir == 0 ? (q * n1 + po) : (po * n1 + q);   /* dir 1: (:, q, po) in Fortran = row po, col q */
        const int i = dir == 0 ? (q * n1 + li) : (li * n1 + q);
        for (int c = 0; c < 2; ++c) out[o * 2 + c] = out[o * 2 + c] + in[i * 2 + c] * buf[p][l];
      }
}

/* ComputeBezierIntersectionPoint, particle_intersection.f90:2276-2457 */
static void bz_intersection_point(bz_clip_t* K, int nXiClip, int nEtaClip) {
  const orc_bz_side_t* S = K->S;
  const int ng = S->B.ng;
  double Xi, Eta;
  if (nXiClip == 0) Xi = 0.0;
  else {
    Xi = 0.5 * (K->XiArray[nXiClip][0] + K->XiArray[nXiClip][1]);
    for (int i = nXiClip - 1; i >= 1; --i) Xi = K->XiArray[i][0] + 0.5 * (Xi + 1) * (K->XiArray[i][1] - K->XiArray[i][0]);
  }
  if (nEtaClip == 0) Eta = 0.0;
  else {
    Eta = 0.5 * (K->EtaArray[nEtaClip][0] + K->EtaArray[nEtaClip][1]);
    for (int i = nEtaClip - 1; i >= 1; --i)
      Eta = K->EtaArray[i][0] + 0.5 * (Eta + 1) * (K->EtaArray[i][1] - K->EtaArray[i][0]);
  }
  const double tmpXi = Xi, tmpEta = Eta;
  Xi = 0.5 * (Xi + 1);
  Eta = 0.5 * (Eta + 1);
  if (fabs(Eta) > BZ_CLIP_HIT || fabs(Xi) > BZ_CLIP_HIT) return;
  const double MinusXi = 1.0 - Xi, MinusEta = 1.0 - Eta;
  double R[BZ_NP][BZ_NP][3];
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p)
      for (int c = 0; c < 3; ++c) R[q][p][c] = S->cp[(q * (ng + 1) + p) * 3 + c];
  int l = ng - 1;
  for (int it = 1; it <= ng; ++it) {
    for (int q = 0; q <= l; ++q)
      for (int p = 0; p <= l; ++p)
        for (int c = 0; c < 3; ++c)
          R[q][p][c] = ((MinusXi * R[q][p][c] * MinusEta + MinusXi * R[q + 1][p][c] * Eta) +
                        Xi * R[q][p + 1][c] * MinusEta) + Xi * R[q + 1][p + 1][c] * Eta;
    l = l - 1;
  }
  const double iv[3] = {R[0][0][0] - K->xl[0], R[0][0][1] - K->xl[1], R[0][0][2] - K->xl[2]};
  const double alpha = bz_dot(iv, K->traj), alphaNorm = alpha / K->len;
  if (alphaNorm <= 1.0 && alphaNorm > -BZ_EPSILONTOL) {
    if (K->nInter >= K->maxInter) { K->err = 1; return; }        /* the reference stops */
    if (K->nInter == 0) {
      K->locAlpha[0] = alpha; K->locXi[0] = tmpXi; K->locEta[0] = tmpEta; K->nInter = 1;
    } else {
      int isNew = 1;
      for (int i = 0; i < K->nInter; ++i) {
        if (fabs(K->locXi[i] - tmpXi) > 0.01) continue;
        if (fabs(K->locEta[i] - tmpEta) > 0.01) continue;
        isNew = 0;
        break;
      }
      if (isNew) {
        K->locAlpha[K->nInter] = alpha; K->locXi[K->nInter] = tmpXi; K->locEta[K->nInter] = tmpEta; K->nInter++;
      }
    }
  }
}

typedef struct {
  double cp[BZ_NP * BZ_NP * 2];
  double lnv[2][2];
  double a0, a1;                  /* the interval the pending half clips to (XiArray/EtaArray at nClip) */
  int clipMode, iClipIter, nXi, nEta, eta;
} bz_pending_t;
#define BZ_STACK 8   /* nested splits held (the library holds the same number) */

/* CheckXiClip (dir 0, particle_intersection.f90:2459-2851) / CheckEtaClip (dir 1, :2853-3243) on the patch cp.
 * Returns 1 at a split: the first half is in cp, the second half in *pend (to be clipped after the first). */
static int bz_check_clip(bz_clip_t* K, int dir, double* cp, double lnv[2][2], int* clipMode, int* iClipIter,
                         int* nXi, int* nEta, bz_pending_t* pend) {
  const orc_bz_basis_t* B = &K->S->B;
  const int ng = B->ng, n1 = ng + 1;
  double c1[BZ_NP][BZ_NP];   /* BezierControlPoints1D(p,q) -> c1[q][p] */
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p) c1[q][p] = cp[(q * n1 + p) * 2] * lnv[dir][0] + cp[(q * n1 + p) * 2 + 1] * lnv[dir][1];
  double mm[2][BZ_NP];
  for (int l = 0; l <= ng; ++l) {
    double mn = DBL_MAX, mx = -DBL_MAX;
    for (int k = 0; k <= ng; ++k) {
      const double v = dir == 0 ? c1[k][l] : c1[l][k];   /* xi: MINVAL(1D(l,:)); eta: MINVAL(1D(:,l)) */
      mn = fmin(mn, v); mx = fmax(mx, v);
    }
    mm[0][l] = mn; mm[1][l] = mx;
  }
  double dmin = DBL_MAX, dmax = -DBL_MAX;
  for (int l = 0; l <= ng; ++l) { dmin = fmin(dmin, mm[0][l]); dmax = fmax(dmax, mm[1][l]); }
  if (dmax * dmin > 0.0) { *clipMode = -1; return 0; }
  if (fabs(dmax - dmin) < K->localTol) {
    if (dir == 0) *clipMode = (*clipMode == 3) ? 5 : 4;
    else *clipMode = (*clipMode == 4) ? 5 : 3;
    return 0;
  }
  *clipMode = dir == 0 ? 2 : 1;
  int* nClip = dir == 0 ? nXi : nEta;
  double (*Arr)[2] = dir == 0 ? K->XiArray : K->EtaArray;
  double smin, smax;
  bz_sminmax(B, (const double(*)[BZ_NP])mm, &smin, &smax, *nClip);
  if (smin == 1.5 || smax == -1.5) { *clipMode = -1; return 0; }
  if (smin > smax) { const double t = smax; smax = smin; smin = t; }
  *nClip = *nClip + 1;
  if (*nClip > BZ_CLIP_MAXITER) { K->err = 1; *clipMode = -1; return 0; }
  double buf[BZ_NP][BZ_NP], tmp[BZ_NP * BZ_NP * 2], tmp2[BZ_NP * BZ_NP * 2];
  if (smax - smin > BZ_SPLIT_LIMIT) {
    const double split = 0.5 * (smax + smin);
    Arr[*nClip][0] = split; Arr[*nClip][1] = smax;
    if (smax != 1.0) { bz_buf(B, 1.0 + smax, 1.0 - smax, buf); bz_sub(ng, buf, cp, tmp, dir, 0); }
    else memcpy(tmp, cp, sizeof(double) * n1 * n1 * 2);
    double plus = (split + 1.0) / (smax + 1.0), minus = 2.0 * plus;
    plus = 2.0 - 2.0 * plus;
    bz_buf(B, plus, minus, buf);
    bz_sub(ng, buf, tmp, tmp2, dir, 1);                            /* first half: [split, smax] */
    /* the second half [smin, split], from the same patch */
    bz_buf(B, 1.0 + split, 1.0 - split, buf);
    bz_sub(ng, buf, cp, tmp, dir, 0);
    if (smin != -1.0) {
      plus = (smin + 1.0) / (split + 1.0); minus = 2.0 * plus;
      plus = 2.0 - 2.0 * plus;
      bz_buf(B, plus, minus, buf);
      bz_sub(ng, buf, tmp, pend->cp, dir, 1);
    } else {
      memcpy(pend->cp, tmp, sizeof(double) * n1 * n1 * 2);
    }
    memcpy(pend->lnv, lnv, sizeof(pend->lnv));
    pend->a0 = smin; pend->a1 = split;
    pend->clipMode = *clipMode; pend->iClipIter = *iClipIter; pend->nXi = *nXi; pend->nEta = *nEta; pend->eta = dir;
    memcpy(cp, tmp2, sizeof(double) * n1 * n1 * 2);
    return 1;
  }
  Arr[*nClip][0] = smin; Arr[*nClip][1] = smax;
  if (smax != 1.0) {
    bz_buf(B, 1.0 + smax, 1.0 - smax, buf);
    bz_sub(ng, buf, cp, tmp, dir, 0);
    memcpy(cp, tmp, sizeof(double) * n1 * n1 * 2);
  }
  if (smin != -1.0) {
    double plus = (smin + 1.0) / (smax + 1.0), minus = 2.0 * plus;
    plus = 2.0 - 2.0 * plus;
    bz_buf(B, plus, minus, buf);
    bz_sub(ng, buf, cp, tmp, dir, 1);
    memcpy(cp, tmp, sizeof(double) * n1 * n1 * 2);
  }
  return 0;
}

/* BezierClipRecursive, particle_intersection.f90:1635-1748, with the recursion as an explicit stack */
static void bz_clip(bz_clip_t* K, const double* cp2d_in, int clipMode0) {
  const int ng = K->S->B.ng, n1 = ng + 1;
  double cp[BZ_NP * BZ_NP * 2];
  memcpy(cp, cp2d_in, sizeof(double) * n1 * n1 * 2);
  double lnv[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  int clipMode = clipMode0, iClipIter = 0, nXi = 0, nEta = 0;
  bz_pending_t stack[BZ_STACK];
  int top = 0;
  for (int guard = 0; guard < 100000; ++guard) {
    int done = 0;   /* the current branch returned */
    if (iClipIter > BZ_CLIP_MAXITER) { K->err = 1; done = 1; }   /* the reference stops */
    else {
      iClipIter = iClipIter + 1;
      int split = 0;
      switch (clipMode) {
        case -1: done = 1; break;
        case 1:
        case 2:
          if (iClipIter % 2 == 1 && bz_line_norm_vec(ng, cp, lnv)) { K->err = 1; done = 1; break; }
          if (top == BZ_STACK) { K->err = 1; done = 1; break; }
          split = bz_check_clip(K, clipMode == 1 ? 0 : 1, cp, lnv, &clipMode, &iClipIter, &nXi, &nEta, &stack[top]);
          break;
        case 3:
        case 4:
          if (top == BZ_STACK) { K->err = 1; done = 1; break; }
          split = bz_check_clip(K, clipMode == 3 ? 0 : 1, cp, lnv, &clipMode, &iClipIter, &nXi, &nEta, &stack[top]);
          break;
        case 5: bz_intersection_point(K, nXi, nEta); done = 1; break;
        default: K->err = 1; done = 1; break;
      }
      if (split) top++;
    }
    if (!done) continue;
    if (top == 0) return;
    bz_pending_t* P = &stack[--top];
    memcpy(cp, P->cp, sizeof(double) * n1 * n1 * 2);
    memcpy(lnv, P->lnv, sizeof(lnv));
    clipMode = P->clipMode; iClipIter = P->iClipIter; nXi = P->nXi; nEta = P->nEta;
    if (P->eta) { K->EtaArray[nEta][0] = P->a0; K->EtaArray[nEta][1] = P->a1; }
    else { K->XiArray[nXi][0] = P->a0; K->XiArray[nXi][1] = P->a1; }
  }
  K->err = 1;
}

/* BezierClipLocalTol = MIN(dXi, dEta) BezierClipTolerance with the extents of the projected patch; returns the
 * extents in d[2] too */
static double bz_extents(int ng, const double* cp2d, double d[2]) {
  const int n1c = ng + 1;
  double mn0 = DBL_MAX, mx0 = -DBL_MAX, mn1 = DBL_MAX, mx1 = -DBL_MAX;
  for (int k = 0; k < n1c * n1c; ++k) {
    mn0 = fmin(mn0, cp2d[2 * k]); mx0 = fmax(mx0, cp2d[2 * k]);
    mn1 = fmin(mn1, cp2d[2 * k + 1]); mx1 = fmax(mx1, cp2d[2 * k + 1]);
  }
  d[0] = mx0 - mn0; d[1] = mx1 - mn1;
  return fmin(d[0], d[1]) * BZ_CLIP_TOL;
}
static double bz_local_tol(int ng, const double* cp2d) { double d[2]; return bz_extents(ng, cp2d, d); }

/* the trajectory's projection of the side onto the plane normal to it (n1, n2 of the drivers) */
static void bz_project(const orc_bz_side_t* S, const double xl[3], const double traj[3], int swap, double* cp2d) {
  const int ng = S->B.ng, n1c = ng + 1;
  double n1[3], n2[3], t[3];
  if (fabs(traj[2]) < 0.0) { t[0] = -traj[1] - traj[2]; t[1] = traj[0]; t[2] = traj[0]; }
  else { t[0] = traj[2]; t[1] = traj[2]; t[2] = -traj[0] - traj[1]; }
  bz_unit(t, n1);
  bz_crossnorm(traj, n1, n2);
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p) {
      const double* P = &S->cp[(q * n1c + p) * 3];
      const double d[3] = {P[0] - xl[0], P[1] - xl[1], P[2] - xl[2]};
      const double a = bz_dot(d, n1), b = bz_dot(d, n2);
      cp2d[(q * n1c + p) * 2] = swap ? b : a;
      cp2d[(q * n1c + p) * 2 + 1] = swap ? a : b;
    }
}

/* BezierNewton, particle_intersection.f90:1750-1989 (BezierNewtonGuess 1).  Returns alpha or -1; *failed when
 * it ran out of iterations. */
static double bz_newton(const orc_bz_side_t* S, const double* cp2d, const double xl[3], const double traj[3],
                        double len, double Xi[2], int* failed) {
  const orc_bz_basis_t* B = &S->B;
  const int ng = B->ng, n1 = ng + 1;
  *failed = 0;
  double MinMax[2][2];
  int hasInter = 1;
  for (int l = 0; l < 2; ++l) {
    double mn = DBL_MAX, mx = -DBL_MAX;
    for (int k = 0; k < n1 * n1; ++k) { mn = fmin(mn, cp2d[2 * k + l]); mx = fmax(mx, cp2d[2 * k + l]); }
    MinMax[0][l] = mn; MinMax[1][l] = mx;
    if (mn * mx > 0.0) hasInter = 0;
  }
  if (!hasInter) return -1.0;
  for (int l = 0; l < 2; ++l) Xi[l] = -1.0 - 2 * MinMax[0][l] / (MinMax[1][l] - MinMax[0][l]);
  double dcp[BZ_NP * BZ_NP * 4];      /* dBezierControlPoints2D(dd, nn, i, j) -> [(j*n1+i)*4 + dd*2 + nn] */
  for (int k = 0; k < n1 * n1 * 4; ++k) dcp[k] = 0.0;
  for (int nn = 0; nn < 2; ++nn)
    for (int dd = 0; dd < 2; ++dd)
      for (int j = 0; j <= ng; ++j)
        for (int i = 0; i <= ng; ++i)
          for (int l = 0; l <= ng; ++l) {
            const int ci = dd == 0 ? l : i, cj = dd == 0 ? j : l;
            const int cyc = dd == 0 ? i : j;
            dcp[(j * n1 + i) * 4 + dd * 2 + nn] =
                dcp[(j * n1 + i) * 4 + dd * 2 + nn] + B->dbez[cyc][l] * cp2d[(cj * n1 + ci) * 2 + nn];
          }
  double P[2], g[4];
  bz_eval(B, Xi, 2, cp2d, dcp, P, g);          /* g[dd*2 + nn] = d P(nn) / d xi(dd): gradXi(dd, nn) */
  double normP = P[0] * P[0] + P[1] * P[1];
  double dXi2 = 1.0;
  int nIter = 1;
  while (dXi2 > BZ_NEWTON_TOL2 && nIter <= BZ_NEWTON_MAXITER) {
    double sdet = g[0] * g[3] - g[1] * g[2];  /* gradXi(1,1) gradXi(2,2) - gradXi(1,2) gradXi(2,1) */
    if (fabs(sdet) > BZ_EPS_MACH) sdet = 1.0 / sdet;         /* epsilon(0.) with -fdefault-real-8 */
    else { Xi[0] = 1.5; Xi[1] = 1.5; return -1.0; }
    double dXi[2];
    dXi[0] = g[3] * P[0] - g[2] * P[1];
    dXi[1] = -g[1] * P[0] + g[0] * P[1];
    dXi[0] = sdet * dXi[0]; dXi[1] = sdet * dXi[1];
    dXi2 = dXi[0] * dXi[0] + dXi[1] * dXi[1];
    const double Xi_old[2] = {Xi[0], Xi[1]};
    double lambda = 1.0;
    const double normPold = normP;
    normP = normP * 2.0;
    for (int iArmijo = 1; normP > normPold * (1.0 - 0.0001 * lambda) && iArmijo <= 6; ++iArmijo) {
      Xi[0] = Xi_old[0] - lambda * dXi[0];
      Xi[1] = Xi_old[1] - lambda * dXi[1];
      bz_eval(B, Xi, 2, cp2d, NULL, P, g);
      normP = P[0] * P[0] + P[1] * P[1];
      lambda = 0.3 * lambda;
    }
    if (nIter >= 4 && (fabs(Xi[0]) > 1.5 || fabs(Xi[1]) > 1.5)) { Xi[0] = 1.5; Xi[1] = 1.5; break; }
    nIter = nIter + 1;
  }
  if (nIter > BZ_NEWTON_MAXITER) { *failed = 1; return -1.0; }
  if (fabs(Xi[0]) > 1.002 || fabs(Xi[1]) > 1.002) return -1.0;
  double ip[3];
  bz_eval(B, Xi, 3, S->cp, NULL, ip, NULL);
  const double iv[3] = {ip[0] - xl[0], ip[1] - xl[1], ip[2] - xl[2]};
  const double alpha = bz_dot(iv, traj), alphaNorm = alpha / len;
  if (alphaNorm <= 1.0 && alphaNorm > -BZ_EPSILONTOL) return alpha;
  return -1.0;
}

/* ComputePlanarCurvedIntersection, particle_intersection.f90:687-852, with the side's normal nv and distance dist
 * oriented away from the element (flip = 0).  Returns alpha or -1, and xi/eta of the hit; *err on a reference
 * abort. */
double orc_bz_planar_curved(const orc_bz_side_t* S, const double nv[3], double dist, const double xl[3],
                            const double traj[3], double len, double* xi, double* eta, int* err) {
  *xi = 2.0; *eta = 2.0;
  const double coeffA = bz_dot(nv, traj);
  if (coeffA <= 0.0) return -1.0;
  double locSideDistance = dist - bz_dot(xl, nv);
  locSideDistance = locSideDistance / coeffA;
  if (locSideDistance > len) return -1.0;
  if (!bz_flat_bb_intersection(S, traj, len, xl)) return -1.0;
  const int ng = S->B.ng;
  double cp2d[BZ_NP * BZ_NP * 2];
  bz_project(S, xl, traj, 0, cp2d);
  double Xn[2] = {0.0, 0.0};
  int failed;
  double alpha = bz_newton(S, cp2d, xl, traj, len, Xn, &failed);
  double lx = Xn[0], le = Xn[1];
  if (failed) {
    /* the reference clips with BezierClipLocalTol as an earlier ComputeCurvedIntersection left it; here it is
     * set as that routine sets it, from this patch */
    bz_clip_t K;
    memset(&K, 0, sizeof(K));
    K.S = S; K.xl = xl; K.traj = traj; K.len = len; K.maxInter = 2 * (ng + 1);
    K.localTol = bz_local_tol(ng, cp2d);
    bz_clip(&K, cp2d, 1);
    if (K.err) *err = 1;
    alpha = K.nInter > 0 ? K.locAlpha[0] : -1.0;
    lx = K.nInter > 0 ? K.locXi[0] : lx;
    le = K.nInter > 0 ? K.locEta[0] : le;
  }
  if (!(alpha > -1.0)) return -1.0;
  *xi = lx; *eta = le;
  return alpha;
}

/* ComputeCurvedIntersection, particle_intersection.f90:1243-1632, RefTracking (no ElemCheck).  x is the new
 * position (InsideBoundingBox of PartState). */
double orc_bz_curved(const orc_bz_side_t* S, const double nv[3], const double xl[3], const double x[3],
                     const double traj[3], double len, double* xi, double* eta, int* err) {
  *xi = 2.0; *eta = 2.0;
  if (S->bb_empty) {
    if (bz_dot(nv, traj) < 0.0) return -1.0;
    if (!bz_flat_bb_intersection(S, traj, len, xl)) return -1.0;
  } else {
    if (!bz_inside_bb(S, xl) && !bz_inside_bb(S, x) && !bz_bb_intersection(S, traj, len, xl)) return -1.0;
  }
  const int ng = S->B.ng;
  double cp2d[BZ_NP * BZ_NP * 2];
  bz_project(S, xl, traj, 1, cp2d);    /* BezierControlPoints2D(1) = . n2, (2) = . n1 */
  double ext[2];
  const double tol = bz_extents(ng, cp2d, ext);
  bz_clip_t K;
  memset(&K, 0, sizeof(K));
  K.S = S; K.xl = xl; K.traj = traj; K.len = len; K.maxInter = 2 * (ng + 1);
  K.localTol = tol;
  const double PartFaceAngle = fabs(0.5 * acos(-1.0) - acos(bz_dot(traj, S->slab_n[1])));
  if (PartFaceAngle < 1.570796326) {
    /* BezierNewtonAngle (default): clip, in the wider direction first */
    bz_clip(&K, cp2d, ext[0] > ext[1] ? 1 : 2);
  } else {
    /* a trajectory along SideSlabNormals(:,2): clip a copy (at most one intersection), then BezierNewton, whose
     * root is taken (BezierClipLocalTol as for the clip branch, which the reference leaves from earlier calls) */
    bz_clip(&K, cp2d, 1);
    if (K.nInter > 1) *err = 1;
    double Xn[2] = {0.0, 0.0};
    int failed;
    const double a = bz_newton(S, cp2d, xl, traj, len, Xn, &failed);
    if (failed) *err = 1;
    K.locAlpha[0] = a;
    K.nInter = a > -1.0 ? 1 : 0;
    K.locXi[0] = Xn[0]; K.locEta[0] = Xn[1];
  }
  if (K.err) *err = 1;
  if (K.nInter == 0) return -1.0;
  if (K.nInter == 1) { *xi = K.locXi[0]; *eta = K.locEta[0]; return K.locAlpha[0]; }
  /* more than one: InsertionSort of the alphas, the first one > -1 (RefTracking) */
  int id[2 * BZ_NP];
  double a[2 * BZ_NP];
  for (int i = 0; i < K.nInter; ++i) { id[i] = i; a[i] = K.locAlpha[i]; }
  for (int i = 1; i < K.nInter; ++i) {
    const double t = a[i];
    const int ti = id[i];
    int j = i - 1;
    while (j >= 0 && !(a[j] <= t)) { a[j + 1] = a[j]; id[j + 1] = id[j]; j--; }
    a[j + 1] = t; id[j + 1] = ti;
  }
  for (int i = 0; i < K.nInter; ++i)
    if (a[i] > -1.0) { *xi = K.locXi[id[i]]; *eta = K.locEta[id[i]]; return a[i]; }
  return -1.0;
}
