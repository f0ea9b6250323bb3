// pic_bezier.cuh -- intersections of a particle trajectory with curved (Bezier) wall sides, RefTracking on
// meshes of geometry degree NGeo = 2..4: the side bounding-box tests, BezierNewton, Bezier clipping and the
// two drivers ComputePlanarCurvedIntersection (SideType PLANAR_CURVED) and ComputeCurvedIntersection (CURVED).
//
// PICLas sources: src/particles/tracking/particle_intersection.f90 (drivers :687-852 and :1243-1632,
// BezierClipRecursive :1635-1748, BezierNewton :1750-1989, InsideBoundingBox :1991-2038,
// BoundingBoxIntersection :2040-2110, FlatBoundingBoxIntersection :2112-2207, ComputeBezierIntersectionPoint
// :2276-2457, CheckXiClip :2459-2851, CheckEtaClip :2853-3243, calcLineNormVec3 :3285-3364, CalcSminSmax2
// :3366-3451), src/particles/particle_mesh/particle_surfaces.f90 (EvaluateBezierPolynomialAndGradient
// :474-616, CalcNormAndTangBezier :443-471).  Default parameters of InitParticleSurfaces
// (particle_surfaces.f90:133-158): BezierNewtonAngle pi/2 (every curved side is clipped), BezierClipTolerance
// 1e-8, BezierNewtonTolerance 1e-4, BezierNewtonMaxIter 100, BezierSplitLimit 2 x 0.6, BezierClipMaxIter 100,
// BezierClipLineVectorMethod 2, epsilontol 100 epsMach, BezierClipHit 1 + 100 BezierClipTolerance,
// BezierClipMaxIntersec 2 (NGeo+1); BezierElevation 0.
//
// One thread per particle, FP64 in the reference's operation order (the library builds with -fmad=false).  The
// mutual recursion BezierClipRecursive <-> CheckXiClip/CheckEtaClip runs as a loop with an explicit stack of
// pending second halves: at a split the first half is clipped next and the second half is pushed with the
// state the reference keeps across its first recursive call (clip counters, line vectors, ClipMode), so that
// the halves are visited in the reference's order.  The stack holds kBzStack nested splits; deeper nesting,
// more than BezierClipMaxIntersec hits or a degenerated patch raise the error flag (status bit) instead of the
// reference's abort.  Every loop is bounded.
#pragma once

namespace pic {

constexpr int kBzNP = kMaxNGeo + 1;               // control points per direction (NGeo <= 4)
constexpr int kBzGeo = 96;                        // doubles per BC-side entry of DevMesh::bc_bz
constexpr int kBzSlabN = 75, kBzSlabI = 84, kBzEmpty = 90;
constexpr int kBzClipMaxIter = 100;               // BezierClipMaxIter
constexpr int kBzMaxInter = 2 * kBzNP;            // BezierClipMaxIntersec at NGeo = 4
constexpr int kBzStack = 8;                       // nested splits held
constexpr double kBzClipTol = 1e-8;               // BezierClipTolerance
constexpr double kBzNewtonTol2 = 1e-8;            // BezierNewtonTolerance**2
constexpr double kBzSplitLimit = 1.2;             // 2 x BezierSplitLimit
constexpr double kBzEpsilonTol = 100.0 * kEpsMach;
constexpr double kBzClipHit = 1.0 + 100.0 * kBzClipTol;


__device__ __forceinline__ double bz_dot(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

__device__ __forceinline__ void bz_crossnorm(const double a[3], const double b[3], double n[3]) {
  n[0] = a[1] * b[2] - a[2] * b[1];
  n[1] = a[2] * b[0] - a[0] * b[2];
  n[2] = a[0] * b[1] - a[1] * b[0];
  const double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  n[0] = n[0] / l; n[1] = n[1] / l; n[2] = n[2] / l;
}

// EvaluateBezierPolynomialAndGradient for ISZ components; cp[(q*(ng+1)+p)*ISZ + c]; dcp (optional): the
// pre-computed derivatives [(q*(ng+1)+p)*2*ISZ + dd*ISZ + c]; point/grad optional (grad[dd*ISZ + c])
template <int ISZ>
static __device__ __noinline__ void bz_eval(const BzBasis& B, const double xi[2], const double* cp, const double* dcp, double* point,
                                            double* grad) {
  const int n = B.ng, n1 = n + 1, M = n - 1;
  double xiup[kBzNP], etaup[kBzNP], xidown[kBzNP], etadown[kBzNP], xitild[kBzNP], etatild[kBzNP];
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
    for (int c = 0; c < ISZ; ++c) point[c] = 0.0;
    for (int q = 0; q <= n; ++q)
      for (int p = 0; p <= n; ++p)
        for (int c = 0; c < ISZ; ++c)
          point[c] = point[c] + cp[(q * n1 + p) * ISZ + c] * B.fnk[n][p] * xitild[p] * B.fnk[n][q] * etatild[q];
  }
  if (grad) {
    for (int c = 0; c < 2 * ISZ; ++c) grad[c] = 0.0;
    if (dcp) {
      for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p)
          for (int dd = 0; dd < 2; ++dd)
            for (int c = 0; c < ISZ; ++c)
              grad[dd * ISZ + c] = grad[dd * ISZ + c] + dcp[(q * n1 + p) * 2 * ISZ + dd * ISZ + c] * B.fnk[n][p] *
                                                            xitild[p] * B.fnk[n][q] * etatild[q];
    } else {
      for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= M; ++p)
          for (int c = 0; c < ISZ; ++c) {
            grad[c] = grad[c] + (cp[(q * n1 + p + 1) * ISZ + c] - cp[(q * n1 + p) * ISZ + c]) * B.fnk[M][p] *
                                    xiup[p] * xidown[p + 1] * B.fnk[n][q] * etatild[q];
            grad[ISZ + c] = grad[ISZ + c] + (cp[((p + 1) * n1 + q) * ISZ + c] - cp[(p * n1 + q) * ISZ + c]) *
                                                B.fnk[n][q] * xitild[q] * B.fnk[M][p] * etaup[p] * etadown[p + 1];
          }
      for (int c = 0; c < 2 * ISZ; ++c) grad[c] = 0.5 * (double)n * grad[c];
    }
  }
}

// CalcNormAndTangBezier: the unit normal d/dxi x d/deta of the side at (xi, eta)
static __device__ __noinline__ void bz_normal(const BzBasis& B, const double* __restrict__ S, double xi, double eta, double nv[3]) {
  const double x2[2] = {xi, eta};
  double g[6];
  bz_eval<3>(B, x2, S, nullptr, nullptr, g);
  bz_crossnorm(&g[0], &g[3], nv);
}

// InsideBoundingBox
__device__ __forceinline__ bool bz_inside_bb(const double* __restrict__ S, const double x[3]) {
  const double P[3] = {x[0] - __ldg(S), x[1] - __ldg(S + 1), x[2] - __ldg(S + 2)};
  const double e = 100.0 * kEpsMach;
  const double* sn = S + kBzSlabN;
  const double* si = S + kBzSlabI;
  const double y = (P[0] * __ldg(sn + 3) + P[1] * __ldg(sn + 4)) + P[2] * __ldg(sn + 5);
  if (y < __ldg(si + 2) - e || y > __ldg(si + 3) + e) return false;
  const double xx = (P[0] * __ldg(sn) + P[1] * __ldg(sn + 1)) + P[2] * __ldg(sn + 2);
  if (xx < __ldg(si) - e || xx > __ldg(si + 1) + e) return false;
  const double z = (P[0] * __ldg(sn + 6) + P[1] * __ldg(sn + 7)) + P[2] * __ldg(sn + 8);
  if (z < __ldg(si + 4) - e || z > __ldg(si + 5) + e) return false;
  return true;
}

// the slab entry/exit parameters of direction i (BoundingBoxIntersection / FlatBoundingBoxIntersection)
__device__ __forceinline__ void bz_slab_alpha(const double* __restrict__ S, int i, double dnk, const double xl[3],
                                              double& a1, double& a2) {
  const double d[3] = {__ldg(S) - xl[0], __ldg(S + 1) - xl[1], __ldg(S + 2) - xl[2]};
  const double sn[3] = {__ldg(S + kBzSlabN + 3 * i), __ldg(S + kBzSlabN + 3 * i + 1), __ldg(S + kBzSlabN + 3 * i + 2)};
  const double base = bz_dot(d, sn);
  const double lo = __ldg(S + kBzSlabI + 2 * i), hi = __ldg(S + kBzSlabI + 2 * i + 1);
  if (dnk < 0.0) { a1 = (base + hi) / dnk; a2 = (base + lo) / dnk; }
  else { a1 = (base + lo) / dnk; a2 = (base + hi) / dnk; }
}

__device__ __forceinline__ double bz_slab_dot(const double* __restrict__ S, int i, const double t[3]) {
  const double sn[3] = {__ldg(S + kBzSlabN + 3 * i), __ldg(S + kBzSlabN + 3 * i + 1), __ldg(S + kBzSlabN + 3 * i + 2)};
  return bz_dot(t, sn);
}

// BoundingBoxIntersection
static __device__ __noinline__ bool bz_bb_intersection(const double* __restrict__ S, const double traj[3], double len,
                                                       const double xl[3]) {
  double a0[3], a1[3];
  for (int i = 0; i < 3; ++i) {
    double dnk = bz_slab_dot(S, i, traj);
    if (fabs(dnk) < 100.0 * kEpsMach) dnk = 100.0 * kEpsMach;
    bz_slab_alpha(S, i, dnk, xl, a0[i], a1[i]);
  }
  const double maxv = fmax(fmax(a0[0], a0[1]), a0[2]);
  const double minv = fmin(fmin(a1[0], a1[1]), a1[2]);
  if (maxv <= minv) return (maxv < len + 100 * kEpsMach) && (maxv + 100 * kEpsMach > 0.0);
  return false;
}

// FlatBoundingBoxIntersection
static __device__ __noinline__ bool bz_flat_bb_intersection(const double* __restrict__ S, const double traj[3],
                                                            double len, const double xl[3]) {
  double a0[3] = {0.0, 0.0, 0.0}, a1[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 3; i += 2) {
    const double dnk = bz_slab_dot(S, i, traj);
    if (fabs(dnk) < 100.0 * kEpsMach) { a0[i] = -1.7976931348623157e308; a1[i] = 1.7976931348623157e308; }
    else bz_slab_alpha(S, i, dnk, xl, a0[i], a1[i]);
  }
  const double maxv = fmax(a0[0], a0[2]), minv = fmin(a1[0], a1[2]);
  if (maxv <= minv) {
    if (maxv < 0 && minv > 0) return true;
    return (maxv < len + 100.0 * kEpsMach) && (maxv + 100.0 * kEpsMach > 0.0);
  }
  return false;
}

// ---- Bezier clipping ------------------------------------------------------------------------------------
struct BzPending {
  double cp[kBzNP * kBzNP * 2];
  double lnv[2][2];
  double a0, a1;                  // the interval the pending half clips to (XiArray/EtaArray at nClip)
  int clipMode, iClipIter, nXi, nEta, eta;
};

struct BzClip {
  const BzBasis* B;
  const double* S;
  double xl[3], traj[3];
  double len, localTol;
  double xiA[kBzClipMaxIter + 2][2], etaA[kBzClipMaxIter + 2][2];
  double locAlpha[kBzMaxInter], locXi[kBzMaxInter], locEta[kBzMaxInter];
  int nInter, maxInter, err;
};

// calcLineNormVec3; returns true on a degenerated patch (the reference stops)
__device__ __forceinline__ bool bz_line_norm_vec(const BzBasis& B, const double* cp, double lnv[2][2]) {
  const int ng = B.ng, n1 = ng + 1;
  auto C2 = [&](int p, int q, int c) { return cp[(q * n1 + p) * 2 + c]; };
  double LXi[2], Leta[2];
  for (int c = 0; c < 2; ++c) LXi[c] = (C2(0, ng, c) - C2(0, 0, c)) + (C2(ng, ng, c) - C2(ng, 0, c));
  double Length = sqrt(LXi[0] * LXi[0] + LXi[1] * LXi[1]);
  if (Length == 0.0) return true;
  LXi[0] = LXi[0] / Length; LXi[1] = LXi[1] / Length;
  for (int c = 0; c < 2; ++c) Leta[c] = (C2(ng, 0, c) - C2(0, 0, c)) + (C2(ng, ng, c) - C2(0, ng, c));
  Length = sqrt(Leta[0] * Leta[0] + Leta[1] * Leta[1]);
  if (Length == 0.0) return true;
  Leta[0] = Leta[0] / Length; Leta[1] = Leta[1] / Length;
  lnv[0][0] = -LXi[1]; lnv[0][1] = LXi[0];
  lnv[1][0] = -Leta[1]; lnv[1][1] = Leta[0];
  return false;
}

// CalcSminSmax2
__device__ __forceinline__ void bz_sminmax(const BzBasis& B, const double mm[2][kBzNP], double& smin, double& smax, int iter) {
  const int ng = B.ng;
  double Smin = 1.5, Smax = -1.5;
  for (int p = 0; p <= ng; ++p)
    for (int q = 0; q <= ng; ++q) {
      if (p == q) continue;
      if (mm[1][p] * mm[1][q] <= 0.0) {
        const double m = (mm[1][q] - mm[1][p]) / (B.xi[q] - B.xi[p]);
        if (m < 0.0) Smax = fmax(Smax, B.xi[q] - mm[1][q] / m);
        if (m > 0.0) Smin = fmin(Smin, B.xi[q] - mm[1][q] / m);
      }
      if (mm[0][p] * mm[0][q] <= 0.0) {
        const double m = (mm[0][q] - mm[0][p]) / (B.xi[q] - B.xi[p]);
        if (m > 0.0) Smax = fmax(Smax, B.xi[q] - mm[0][q] / m);
        if (m < 0.0) Smin = fmin(Smin, B.xi[q] - mm[0][q] / m);
      }
    }
  if (mm[0][0] * mm[1][0] < 0.0) Smin = -1.0;
  if (mm[0][ng] * mm[1][ng] < 0.0) Smax = 1.0;
  if (Smax > -1.5) Smax = fmin(Smax + 20.0 * kBzClipTol, 1.0);
  if (Smin < 1.5) Smin = fmax(Smin - 20.0 * kBzClipTol, -1.0);
  if (iter == 0) {
    if (Smin == 1.5) Smin = -1.0;
    if (Smax == -1.5) Smax = 1.0;
  }
  smin = Smin; smax = Smax;
}

// the de Casteljau weights of CheckXiClip/CheckEtaClip: buf(p,l) = plus^l minus^(p-l) FacNchooseK(p,l)
__device__ __forceinline__ void bz_buf(const BzBasis& B, double plus, double minus, double buf[kBzNP][kBzNP]) {
  const int ng = B.ng;
  double up[kBzNP], down[kBzNP];
  up[0] = 1.0; down[0] = 1.0;
  for (int l = 1; l <= ng; ++l) { up[l] = up[l - 1] * plus; down[l] = down[l - 1] * minus; }
  for (int p = 0; p <= ng; ++p)
    for (int l = 0; l <= p; ++l) buf[p][l] = up[l] * down[p - l] * B.fnk[p][l];
}

// out(:, p, q) = sum_l in(:, l, q) buf(p, l) along direction dir (0: xi, 1: eta), from the low end (rev 0) or
// mirrored from the high end (rev 1: out(:, N-p) = sum_l in(:, N-l) buf(p, l))
static __device__ __noinline__ void bz_sub(const BzBasis& B, const double buf[kBzNP][kBzNP], const double* in, double* out, int dir,
                                           int rev) {
  const int ng = B.ng, n1 = ng + 1;
  for (int k = 0; k < n1 * n1 * 2; ++k) out[k] = 0.0;
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p)
      for (int l = 0; l <= p; ++l) {
        const int po = rev ? ng - p : p, li = rev ? ng - l : l;
        const int o = dir == 0 ? (q * n1 + po) : (po * n1 + q);
        const int i = dir == 0 ? (q * n1 + li) : (li * n1 + q);
        for (int c = 0; c < 2; ++c) out[o * 2 + c] = out[o * 2 + c] + in[i * 2 + c] * buf[p][l];
      }
}

// ComputeBezierIntersectionPoint
static __device__ __noinline__ void bz_intersection_point(BzClip& K, int nXiClip, int nEtaClip) {
  const BzBasis& B = *K.B;
  const int ng = B.ng, n1 = ng + 1;
  double Xi, Eta;
  if (nXiClip == 0) Xi = 0.0;
  else {
    Xi = 0.5 * (K.xiA[nXiClip][0] + K.xiA[nXiClip][1]);
    for (int i = nXiClip - 1; i >= 1; --i) Xi = K.xiA[i][0] + 0.5 * (Xi + 1) * (K.xiA[i][1] - K.xiA[i][0]);
  }
  if (nEtaClip == 0) Eta = 0.0;
  else {
    Eta = 0.5 * (K.etaA[nEtaClip][0] + K.etaA[nEtaClip][1]);
    for (int i = nEtaClip - 1; i >= 1; --i) Eta = K.etaA[i][0] + 0.5 * (Eta + 1) * (K.etaA[i][1] - K.etaA[i][0]);
  }
  const double tmpXi = Xi, tmpEta = Eta;
  Xi = 0.5 * (Xi + 1);
  Eta = 0.5 * (Eta + 1);
  if (fabs(Eta) > kBzClipHit || fabs(Xi) > kBzClipHit) return;
  const double MinusXi = 1.0 - Xi, MinusEta = 1.0 - Eta;
  double R[kBzNP][kBzNP][3];
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p)
      for (int c = 0; c < 3; ++c) R[q][p][c] = __ldg(K.S + (q * n1 + p) * 3 + c);
  int l = ng - 1;
  for (int it = 1; it <= ng; ++it) {
    for (int q = 0; q <= l; ++q)
      for (int p = 0; p <= l; ++p)
        for (int c = 0; c < 3; ++c)
          R[q][p][c] = ((MinusXi * R[q][p][c] * MinusEta + MinusXi * R[q + 1][p][c] * Eta) +
                        Xi * R[q][p + 1][c] * MinusEta) + Xi * R[q + 1][p + 1][c] * Eta;
    l = l - 1;
  }
  const double iv[3] = {R[0][0][0] - K.xl[0], R[0][0][1] - K.xl[1], R[0][0][2] - K.xl[2]};
  const double alpha = bz_dot(iv, K.traj), alphaNorm = alpha / K.len;
  if (alphaNorm <= 1.0 && alphaNorm > -kBzEpsilonTol) {
    if (K.nInter >= K.maxInter) { K.err = 1; return; }
    if (K.nInter == 0) {
      K.locAlpha[0] = alpha; K.locXi[0] = tmpXi; K.locEta[0] = tmpEta; K.nInter = 1;
    } else {
      bool isNew = true;
      for (int i = 0; i < K.nInter; ++i) {
        if (fabs(K.locXi[i] - tmpXi) > 0.01) continue;
        if (fabs(K.locEta[i] - tmpEta) > 0.01) continue;
        isNew = false;
        break;
      }
      if (isNew) {
        K.locAlpha[K.nInter] = alpha; K.locXi[K.nInter] = tmpXi; K.locEta[K.nInter] = tmpEta; K.nInter++;
      }
    }
  }
}

// CheckXiClip (dir 0) / CheckEtaClip (dir 1) on the patch cp.  Returns true at a split: the first half is in
// cp, the second half in pend (clipped after the first).
static __device__ __noinline__ bool bz_check_clip(BzClip& K, int dir, double* cp, double lnv[2][2], int& clipMode,
                                                  int& iClipIter, int& nXi, int& nEta, BzPending& pend) {
  const BzBasis& B = *K.B;
  const int ng = B.ng, n1 = ng + 1;
  double c1[kBzNP][kBzNP];
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p) c1[q][p] = cp[(q * n1 + p) * 2] * lnv[dir][0] + cp[(q * n1 + p) * 2 + 1] * lnv[dir][1];
  double mm[2][kBzNP];
  for (int l = 0; l <= ng; ++l) {
    double mn = 1.7976931348623157e308, mx = -1.7976931348623157e308;
    for (int k = 0; k <= ng; ++k) {
      const double v = dir == 0 ? c1[k][l] : c1[l][k];
      mn = fmin(mn, v); mx = fmax(mx, v);
    }
    mm[0][l] = mn; mm[1][l] = mx;
  }
  double dmin = 1.7976931348623157e308, dmax = -1.7976931348623157e308;
  for (int l = 0; l <= ng; ++l) { dmin = fmin(dmin, mm[0][l]); dmax = fmax(dmax, mm[1][l]); }
  if (dmax * dmin > 0.0) { clipMode = -1; return false; }
  if (fabs(dmax - dmin) < K.localTol) {
    if (dir == 0) clipMode = (clipMode == 3) ? 5 : 4;
    else clipMode = (clipMode == 4) ? 5 : 3;
    return false;
  }
  clipMode = dir == 0 ? 2 : 1;
  int& nClip = dir == 0 ? nXi : nEta;
  double (*Arr)[2] = dir == 0 ? K.xiA : K.etaA;
  double smin, smax;
  bz_sminmax(B, mm, smin, smax, nClip);
  if (smin == 1.5 || smax == -1.5) { clipMode = -1; return false; }
  if (smin > smax) { const double t = smax; smax = smin; smin = t; }
  nClip = nClip + 1;
  if (nClip > kBzClipMaxIter) { K.err = 1; clipMode = -1; return false; }
  double buf[kBzNP][kBzNP], tmp[kBzNP * kBzNP * 2], tmp2[kBzNP * kBzNP * 2];
  const int ncp = n1 * n1 * 2;
  if (smax - smin > kBzSplitLimit) {
    const double split = 0.5 * (smax + smin);
    Arr[nClip][0] = split; Arr[nClip][1] = smax;
    if (smax != 1.0) { bz_buf(B, 1.0 + smax, 1.0 - smax, buf); bz_sub(B, buf, cp, tmp, dir, 0); }
    else for (int k = 0; k < ncp; ++k) tmp[k] = cp[k];
    double plus = (split + 1.0) / (smax + 1.0), minus = 2.0 * plus;
    plus = 2.0 - 2.0 * plus;
    bz_buf(B, plus, minus, buf);
    bz_sub(B, buf, tmp, tmp2, dir, 1);                              // first half: [split, smax]
    bz_buf(B, 1.0 + split, 1.0 - split, buf);                       // the second half [smin, split]
    bz_sub(B, buf, cp, tmp, dir, 0);
    if (smin != -1.0) {
      plus = (smin + 1.0) / (split + 1.0); minus = 2.0 * plus;
      plus = 2.0 - 2.0 * plus;
      bz_buf(B, plus, minus, buf);
      bz_sub(B, buf, tmp, pend.cp, dir, 1);
    } else {
      for (int k = 0; k < ncp; ++k) pend.cp[k] = tmp[k];
    }
    pend.lnv[0][0] = lnv[0][0]; pend.lnv[0][1] = lnv[0][1]; pend.lnv[1][0] = lnv[1][0]; pend.lnv[1][1] = lnv[1][1];
    pend.a0 = smin; pend.a1 = split;
    pend.clipMode = clipMode; pend.iClipIter = iClipIter; pend.nXi = nXi; pend.nEta = nEta; pend.eta = dir;
    for (int k = 0; k < ncp; ++k) cp[k] = tmp2[k];
    return true;
  }
  Arr[nClip][0] = smin; Arr[nClip][1] = smax;
  if (smax != 1.0) {
    bz_buf(B, 1.0 + smax, 1.0 - smax, buf);
    bz_sub(B, buf, cp, tmp, dir, 0);
    for (int k = 0; k < ncp; ++k) cp[k] = tmp[k];
  }
  if (smin != -1.0) {
    double plus = (smin + 1.0) / (smax + 1.0), minus = 2.0 * plus;
    plus = 2.0 - 2.0 * plus;
    bz_buf(B, plus, minus, buf);
    bz_sub(B, buf, cp, tmp, dir, 1);
    for (int k = 0; k < ncp; ++k) cp[k] = tmp[k];
  }
  return false;
}

// BezierClipRecursive with the recursion as an explicit stack
static __device__ __noinline__ void bz_clip(BzClip& K, const double* cp2d_in, int clipMode0) {
  const BzBasis& B = *K.B;
  const int ng = B.ng, n1 = ng + 1, ncp = n1 * n1 * 2;
  double cp[kBzNP * kBzNP * 2];
  for (int k = 0; k < ncp; ++k) cp[k] = cp2d_in[k];
  double lnv[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  int clipMode = clipMode0, iClipIter = 0, nXi = 0, nEta = 0;
  BzPending stack[kBzStack];
  int top = 0;
  for (int guard = 0; guard < 100000; ++guard) {
    bool done = false;   // the current branch returned
    if (iClipIter > kBzClipMaxIter) { K.err = 1; done = true; }
    else {
      iClipIter = iClipIter + 1;
      bool split = false;
      switch (clipMode) {
        case -1: done = true; break;
        case 1:
        case 2:
          if (iClipIter % 2 == 1 && bz_line_norm_vec(B, cp, lnv)) { K.err = 1; done = true; break; }
          if (top == kBzStack) { K.err = 1; done = true; break; }
          split = bz_check_clip(K, clipMode == 1 ? 0 : 1, cp, lnv, clipMode, iClipIter, nXi, nEta, stack[top]);
          break;
        case 3:
        case 4:
          if (top == kBzStack) { K.err = 1; done = true; break; }
          split = bz_check_clip(K, clipMode == 3 ? 0 : 1, cp, lnv, clipMode, iClipIter, nXi, nEta, stack[top]);
          break;
        case 5: bz_intersection_point(K, nXi, nEta); done = true; break;
        default: K.err = 1; done = true; break;
      }
      if (split) top++;
    }
    if (!done) continue;
    if (top == 0) return;
    const BzPending& P = stack[--top];
    for (int k = 0; k < ncp; ++k) cp[k] = P.cp[k];
    lnv[0][0] = P.lnv[0][0]; lnv[0][1] = P.lnv[0][1]; lnv[1][0] = P.lnv[1][0]; lnv[1][1] = P.lnv[1][1];
    clipMode = P.clipMode; iClipIter = P.iClipIter; nXi = P.nXi; nEta = P.nEta;
    if (P.eta) { K.etaA[nEta][0] = P.a0; K.etaA[nEta][1] = P.a1; }
    else { K.xiA[nXi][0] = P.a0; K.xiA[nXi][1] = P.a1; }
  }
  K.err = 1;
}

// BezierClipLocalTol = MIN(dXi, dEta) BezierClipTolerance from the extents of the projected patch (d[2])
__device__ __forceinline__ double bz_extents(const BzBasis& B, const double* cp2d, double d[2]) {
  const int n1 = B.ng + 1;
  double mn0 = 1.7976931348623157e308, mx0 = -1.7976931348623157e308, mn1 = mn0, mx1 = mx0;
  for (int k = 0; k < n1 * n1; ++k) {
    mn0 = fmin(mn0, cp2d[2 * k]); mx0 = fmax(mx0, cp2d[2 * k]);
    mn1 = fmin(mn1, cp2d[2 * k + 1]); mx1 = fmax(mx1, cp2d[2 * k + 1]);
  }
  d[0] = mx0 - mn0; d[1] = mx1 - mn1;
  return fmin(d[0], d[1]) * kBzClipTol;
}

// the side projected onto the plane normal to the trajectory (n1, n2 of the drivers); swap: (. n2, . n1)
static __device__ __noinline__ void bz_project(const BzBasis& B, const double* __restrict__ S, const double xl[3], const double traj[3],
                                               int swap, double* cp2d) {
  const int ng = B.ng, n1c = ng + 1;
  double n1[3], n2[3], t[3];
  if (fabs(traj[2]) < 0.0) { t[0] = -traj[1] - traj[2]; t[1] = traj[0]; t[2] = traj[0]; }
  else { t[0] = traj[2]; t[1] = traj[2]; t[2] = -traj[0] - traj[1]; }
  {
    double l = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);    // UNITVECTOR
    if (fabs(l) > 0.0) { l = 1.0 / l; n1[0] = t[0] * l; n1[1] = t[1] * l; n1[2] = t[2] * l; }
    else { n1[0] = n1[1] = n1[2] = 0.0; }
  }
  bz_crossnorm(traj, n1, n2);
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p) {
      const double* P = S + (q * n1c + p) * 3;
      const double d[3] = {__ldg(P) - xl[0], __ldg(P + 1) - xl[1], __ldg(P + 2) - xl[2]};
      const double a = bz_dot(d, n1), b = bz_dot(d, n2);
      cp2d[(q * n1c + p) * 2] = swap ? b : a;
      cp2d[(q * n1c + p) * 2 + 1] = swap ? a : b;
    }
}

// BezierNewton (BezierNewtonGuess 1).  Returns alpha or -1; failed when it ran out of iterations.
static __device__ __noinline__ double bz_newton(const BzBasis& B, const double* __restrict__ S, const double* cp2d, const double xl[3],
                                                const double traj[3], double len, double Xi[2], bool& failed) {
  const int ng = B.ng, n1 = ng + 1;
  failed = false;
  double MinMax[2][2];
  bool hasInter = true;
  for (int l = 0; l < 2; ++l) {
    double mn = 1.7976931348623157e308, mx = -1.7976931348623157e308;
    for (int k = 0; k < n1 * n1; ++k) { mn = fmin(mn, cp2d[2 * k + l]); mx = fmax(mx, cp2d[2 * k + l]); }
    MinMax[0][l] = mn; MinMax[1][l] = mx;
    if (mn * mx > 0.0) hasInter = false;
  }
  if (!hasInter) return -1.0;
  for (int l = 0; l < 2; ++l) Xi[l] = -1.0 - 2 * MinMax[0][l] / (MinMax[1][l] - MinMax[0][l]);
  double dcp[kBzNP * kBzNP * 4];
  for (int k = 0; k < n1 * n1 * 4; ++k) dcp[k] = 0.0;
  for (int nn = 0; nn < 2; ++nn)
    for (int dd = 0; dd < 2; ++dd)
      for (int j = 0; j <= ng; ++j)
        for (int i = 0; i <= ng; ++i)
          for (int l = 0; l <= ng; ++l) {
            const int ci = dd == 0 ? l : i, cj = dd == 0 ? j : l;
            const int cyc = dd == 0 ? i : j;
            dcp[(j * n1 + i) * 4 + dd * 2 + nn] =
                dcp[(j * n1 + i) * 4 + dd * 2 + nn] + B.dbez[cyc][l] * cp2d[(cj * n1 + ci) * 2 + nn];
          }
  double P[2], g[4];
  bz_eval<2>(B, Xi, cp2d, dcp, P, g);
  double normP = P[0] * P[0] + P[1] * P[1];
  double dXi2 = 1.0;
  int nIter = 1;
  while (dXi2 > kBzNewtonTol2 && nIter <= 100) {
    double sdet = g[0] * g[3] - g[1] * g[2];
    if (fabs(sdet) > kEpsMach) sdet = 1.0 / sdet;
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
      bz_eval<2>(B, Xi, cp2d, nullptr, P, g);
      normP = P[0] * P[0] + P[1] * P[1];
      lambda = 0.3 * lambda;
    }
    if (nIter >= 4 && (fabs(Xi[0]) > 1.5 || fabs(Xi[1]) > 1.5)) { Xi[0] = 1.5; Xi[1] = 1.5; break; }
    nIter = nIter + 1;
  }
  if (nIter > 100) { failed = true; return -1.0; }
  if (fabs(Xi[0]) > 1.002 || fabs(Xi[1]) > 1.002) return -1.0;
  double ip[3];
  bz_eval<3>(B, Xi, S, nullptr, ip, nullptr);
  const double iv[3] = {ip[0] - xl[0], ip[1] - xl[1], ip[2] - xl[2]};
  const double alpha = bz_dot(iv, traj), alphaNorm = alpha / len;
  if (alphaNorm <= 1.0 && alphaNorm > -kBzEpsilonTol) return alpha;
  return -1.0;
}

__device__ __forceinline__ void bz_clip_init(BzClip& K, const BzBasis& B, const double* S, const double xl[3], const double traj[3],
                                             double len, double tol) {
  K.B = &B;
  K.S = S;
  for (int c = 0; c < 3; ++c) { K.xl[c] = xl[c]; K.traj[c] = traj[c]; }
  K.len = len; K.localTol = tol;
  K.nInter = 0; K.maxInter = 2 * (B.ng + 1); K.err = 0;
}

// ComputePlanarCurvedIntersection with the side's normal nv and distance dist oriented away from the element.
// Returns alpha or -1, xi/eta of the hit; err where the reference aborts.
static __device__ __noinline__ double bz_planar_curved(const BzBasis& B, const double* __restrict__ S, const double nv[3], double dist,
                                                       const double xl[3], const double traj[3], double len,
                                                       double& xi, double& eta, bool& err) {
  xi = 2.0; eta = 2.0;
  const double coeffA = bz_dot(nv, traj);
  if (coeffA <= 0.0) return -1.0;
  double locSideDistance = dist - bz_dot(xl, nv);
  locSideDistance = locSideDistance / coeffA;
  if (locSideDistance > len) return -1.0;
  if (!bz_flat_bb_intersection(S, traj, len, xl)) return -1.0;
  double cp2d[kBzNP * kBzNP * 2];
  bz_project(B, S, xl, traj, 0, cp2d);
  double Xn[2] = {0.0, 0.0};
  bool failed;
  double alpha = bz_newton(B, S, cp2d, xl, traj, len, Xn, failed);
  double lx = Xn[0], le = Xn[1];
  if (failed) {
    // the reference clips with BezierClipLocalTol as an earlier ComputeCurvedIntersection left it; here it is
    // set as that routine sets it, from this patch
    BzClip K;
    double d[2];
    bz_clip_init(K, B, S, xl, traj, len, bz_extents(B, cp2d, d));
    bz_clip(K, cp2d, 1);
    if (K.err) err = true;
    alpha = K.nInter > 0 ? K.locAlpha[0] : -1.0;
    lx = K.nInter > 0 ? K.locXi[0] : lx;
    le = K.nInter > 0 ? K.locEta[0] : le;
  }
  if (!(alpha > -1.0)) return -1.0;
  xi = lx; eta = le;
  return alpha;
}

// ComputeCurvedIntersection (RefTracking, no ElemCheck); x is the new position (InsideBoundingBox of PartState)
static __device__ __noinline__ double bz_curved(const BzBasis& B, const double* __restrict__ S, const double xl[3], const double x[3],
                                                const double traj[3], double len, double& xi, double& eta, bool& err) {
  xi = 2.0; eta = 2.0;
  if (__ldg(S + kBzEmpty) != 0.0) {
    if (bz_slab_dot(S, 1, traj) < 0.0) return -1.0;
    if (!bz_flat_bb_intersection(S, traj, len, xl)) return -1.0;
  } else {
    if (!bz_inside_bb(S, xl) && !bz_inside_bb(S, x) && !bz_bb_intersection(S, traj, len, xl)) return -1.0;
  }
  double cp2d[kBzNP * kBzNP * 2];
  bz_project(B, S, xl, traj, 1, cp2d);    // BezierControlPoints2D(1) = . n2, (2) = . n1
  double ext[2];
  const double tol = bz_extents(B, cp2d, ext);
  BzClip K;
  bz_clip_init(K, B, S, xl, traj, len, tol);
  const double PartFaceAngle = fabs(0.5 * acos(-1.0) - acos(bz_slab_dot(S, 1, traj)));
  if (PartFaceAngle < 1.570796326) {
    bz_clip(K, cp2d, ext[0] > ext[1] ? 1 : 2);     // BezierNewtonAngle: clip, in the wider direction first
  } else {
    // a trajectory along SideSlabNormals(:,2): clip (at most one intersection), then BezierNewton, whose root
    // is taken
    bz_clip(K, cp2d, 1);
    if (K.nInter > 1) err = true;
    double Xn[2] = {0.0, 0.0};
    bool failed;
    const double a = bz_newton(B, S, cp2d, xl, traj, len, Xn, failed);
    if (failed) err = true;
    K.locAlpha[0] = a;
    K.nInter = a > -1.0 ? 1 : 0;
    K.locXi[0] = Xn[0]; K.locEta[0] = Xn[1];
  }
  if (K.err) err = true;
  if (K.nInter == 0) return -1.0;
  if (K.nInter == 1) { xi = K.locXi[0]; eta = K.locEta[0]; return K.locAlpha[0]; }
  // more than one: InsertionSort of the alphas, the first one > -1 (RefTracking)
  int id[kBzMaxInter];
  double a[kBzMaxInter];
  for (int i = 0; i < K.nInter; ++i) { id[i] = i; a[i] = K.locAlpha[i]; }
  for (int i = 1; i < K.nInter; ++i) {
    const double t = a[i];
    const int ti = id[i];
    int j = i - 1;
    while (j >= 0 && !(a[j] <= t)) { a[j + 1] = a[j]; id[j + 1] = id[j]; j--; }
    a[j + 1] = t; id[j + 1] = ti;
  }
  for (int i = 0; i < K.nInter; ++i)
    if (a[i] > -1.0) { xi = K.locXi[id[i]]; eta = K.locEta[id[i]]; return a[i]; }
  return -1.0;
}

}  // namespace pic
