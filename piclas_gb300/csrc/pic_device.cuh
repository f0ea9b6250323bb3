// pic_device.cuh -- device data layout and per-particle routines of the GB300 particle loop.
//
// FP64 routines keep the reference's floating-point evaluation order (the library is compiled
// with -fmad=false, so no multiply-add is contracted behind our back); element decisions are
// therefore bit-identical to the reference's CPU arithmetic.  FP32 routines of the mixed
// variant request fused multiply-adds explicitly with fmaf().
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pic {

constexpr int kMaxN = 5;                 // highest DG degree instantiated
constexpr int kMaxNGeo = 4;              // highest geometry degree (curved elements)
constexpr int kMaxTrackLoops = 10000;    // hop cap of the tracking walks (status bit on overflow)
constexpr double kEpsMach = 2.220446049250313080847e-16;

// ---- device status word -------------------------------------------------------------
struct DevStatus {
  unsigned int error_word;
  int n_lost;
  int n_newton_failed;
  int n_ref_tolerance;
};

// the Bernstein tables of the mesh's NGeo for curved wall sides: FacNchooseK(n,k) = C(n,k)/2^n, Xi_NGeo
// (equidistant nodes on [-1,1]) and D_Bezier (BuildBezierVdm, BuildBezierDMat: basis.f90:275-402)
struct BzBasis {
  int ng;
  double fnk[kMaxNGeo + 1][kMaxNGeo + 1];
  double xi[kMaxNGeo + 1];
  double dbez[kMaxNGeo + 1][kMaxNGeo + 1];
};

// ---- run-time constants (constant memory) -------------------------------------------
struct Consts {
  int N, n1, ndof, n_species;
  double q[8], m[8], mpf[8], qm[8];            // charge, mass, MPF, charge*MPF
  double ext[6];                               // PIC-externalField
  double refmapping_eps;
  double c2_inv;
  double xgp[kMaxN + 1], wbary_gp[kMaxN + 1], fac_gp[kMaxN + 1];
  float xgp_f[kMaxN + 1], wbary_gp_f[kMaxN + 1];
  double xi_cl[2], wbary_cl[2];
  int n_pv;
  double pv[9];                                // PeriodicVectors(1:3,k) at pv[3k..3k+2]
  double xmin[3], xmax[3];
  int fib_imax[3];
  double fib_delta[3];
  double sf_r, sf_r2, sf_r2_inv, sf_w;
  float sf_r_inv;                              // 1/R (FP16 pre-test of the mixed gather)
  double dt_fac[8];                            // Species(s)%TimeStepFactor (1 unless set)
  double sf_cc_div;                            // charge-conserving total divided by dimFactorSF (else 1)
  int sf_alpha;
  int pv_dir[3];                               // periodic vector index per axis (-1: none)
  int sf_keep[3];                              // 1D/2D shape function: 1 in the kernel directions
  int periodic_tracing;                        // RefTracking: periodic sides traced as BC sides (CartesianPeriodic = F)
  int ref_guess;                               // RefMappingGuess 1..4
  int ngeo;                                    // NGeo (curved elements when > 1)
  double xi_cl_ng[kMaxNGeo + 1], wbary_cl_ng[kMaxNGeo + 1];   // XiCL_NGeo, wBaryCL_NGeo (xi_cl: of NGeo = 1)
  BzBasis bz;                                  // curved wall sides (NGeo > 1)
  // mixed Newton in double-FP32 arithmetic: RefMappingEps, 1 + RefMappingEps, and per Armijo step k (lambda_k =
  // 0.2^k in FP64) -lambda_k and 1 - 1e-4 lambda_k, each as a (hi, lo) pair
  float2 df_eps, df_one_eps, df_lam[9], df_arm[9];
  // N_Inter(k)%xGP, %wBary and CellVolWeight(k)%Fac for every degree k (row k; rows up to NMax are set), FP64
  // and FP32: the kernels of degree k read row k, so elements of different degrees (p-adaption) share them
  double xgp_n[kMaxN + 1][kMaxN + 1], wbary_n[kMaxN + 1][kMaxN + 1], fac_n[kMaxN + 1][kMaxN + 1];
  float xgp_nf[kMaxN + 1][kMaxN + 1], wbary_nf[kMaxN + 1][kMaxN + 1];
};

// ---- mesh (device arrays) ---------------------------------------------------------------
struct DevMesh {
  int ne;
  const double* xcl;       // [ne][8][3] corners in tensor order (= NodeCoords of the element)
  const double* dxcl;      // [ne][8][3 nn][3 dd]
  const double* bary;      // [ne][3]
  const double* xez;       // [ne][6][3]
  const double* slen;      // [ne][6]
  const double* radius;    // [ne]
  const double* eps1;      // [ne]
  const int* side_nb;      // [ne][6] 0-based neighbour
  const uint32_t* side_info;  // [ne][6]: bits 0-11 corner ids (4x3), bit 12 concave, bits 16-23 pvid (int8)
  const int* canon_node;   // [ne][8] periodic-unique node (CGNS corner order)
  const double* node_vol;  // [n_canon]
  const double* elem_xgp;  // [ne][ndof][3]
  const int* fib_n;        // FIBGM cells
  const int* fib_off;
  const int* fib_elem;     // 0-based
  const float* xclr;       // [ne][8][3] FP32 corners minus the barycentre (inside-test pre-filter)
  // RefTracking with walls: per element (ELEM_NBR_BCSIDES, first entry) or (-1,-1); per entry kBcGeo doubles
  const int* bc_e2b;
  const double* bc_geo;
  // curved meshes (NGeo > 1): per BC-side entry kBzGeo doubles -- BezierControlPoints3D [(q (NGeo+1) + p) 3 + c],
  // SideSlabNormals [75..83], SideSlabIntervals [84..89], BoundingBoxIsEmpty [90]
  const double* bc_bz;
  // shape-function DOF coordinates: elem_xgp, or for a 1D/2D kernel its directions only (others zero)
  const double* sf_xgp;

  // per-element polynomial degree (p-adaption): N_DG_Mapping(1,:) as 0-based DOF offsets [ne+1] and
  // N_DG_Mapping(2,:) [ne]; both null when every element has degree N (DOF offset e (N+1)^3)
  const int* dof_off;
  const int* elem_n;
  // curved elements (NGeo > 1): XCL_NGeo [ne][(NGeo+1)^3][3] and dXCL_NGeo [ne][(NGeo+1)^3][9] ([k][j][i] order),
  // ElemCurved [ne] (null: all curved); xcl/dxcl above then hold each element's corners (XCL_NGeo1, dXCL_NGeo1)
  const double* xcl_ng;
  const double* dxcl_ng;
  const int* curved;
  // mixed variant: the NGeo = 1 map in monomial form, x(xi) = c0 + c1 xi1 + c2 xi2 + c3 xi3 + c12 xi1 xi2
  // + c13 xi1 xi3 + c23 xi2 xi3 + c123 xi1 xi2 xi3 (from the corners at pic_create), relative to the element's
  // barycentre (c0 - bary) and divided by s_e, the power of two nearest the element's size (exact; the map is O(1)
  // wherever the element lies, far from the FP32 range limits), as double-FP32 pairs (hi, lo) for the Newton in
  // double-FP32 arithmetic: [ne][kDfLin], 24 coefficients, (s_e, 1/s_e), then the start-value data of
  // RefMappingGuess 1 in the same frame and units: the barycentre (0, 0, 0), XiEtaZetaBasis (18),
  // slenXiEtaZetaBasis s_e (6)
  const float2* tcoef_df;
  // curved elements: the NGeo map in power form, x(xi) = sum C[c][b][a] xi1^a xi2^b xi3^c, the same way (constant
  // term relative to the barycentre, over s_e), [ne][(NGeo+1)^3 3 + 1 + 27] in that index order, then (s_e, 1/s_e)
  // and the start-value data
  const float2* tcoef_ng_df;
  // run-time constants of the context; kernels take DevMesh as a __grid_constant__ parameter, so these are
  // read from the launch's parameter bank (each launch carries its own context's copy)
  Consts k;
};
// per BC-side entry: BaseVectors0-2 [0..8], SideNormVec (away from the element) [9..11], SideDistance [12],
// SideBCMetrics(BCSIDE_DISTANCE) [13], boundary [14] (1 open, 2 reflective, 3 periodic), SideType [15]
// (0 PLANAR_RECT, 1 PLANAR_NONRECT, 2 BILINEAR, 3 PLANAR_CURVED, 4 CURVED), BaseVectors3 [16..18], the corners P00, P10, P01, P11
// [19..30], periodic sides: 16 (neighbour element, 0-based) + (BoundaryType(BC_ALPHA) + 8) [31]
constexpr int kBcGeo = 32;
constexpr int kDfStart = 27, kDfLin = 25 + kDfStart;   // double-FP32 start-value data; trilinear block size
constexpr int kBcCap = 64;   // wall sides traced per trajectory (entries within reach beyond it are not)

// ---- particles (SoA) ---------------------------------------------------------------------
struct DevParticles {
  int n;
  double *x, *y, *z;           // PartState(1:3)
  double *vx, *vy, *vz;        // PartState(4:6) in FP64 mode
  float *vxf, *vyf, *vzf;      // PartState(4:6) in mixed mode
  double *lx, *ly, *lz;        // LastPartPos
  double *xi0, *xi1, *xi2;     // PartPosRef
  int* elem;                   // 0-based GlobalElemID-1
  int* last_elem;
  uint8_t* species;            // 0-based
  uint8_t* flags;              // bit0 inside, bit1 IsNewPart
  double* field;               // FieldAtParticle [6][cap]
  int cap;
};

constexpr uint8_t kInside = 1, kNew = 2;

__device__ __forceinline__ void flag_status(DevStatus* st, unsigned int bit) { atomicOr(&st->error_word, bit); }

// ==========================================================================================
// Lagrange basis, basis.f90:1011-1035 and 1223-1264
// ==========================================================================================
__device__ __forceinline__ bool almost_equal_unity(double x, double y) {
  if (x == 0.0 || y == 0.0) return fabs(x - y) <= 2.0 * kEpsMach;
  return (fabs(x - y) <= kEpsMach * fabs(x)) && (fabs(x - y) <= kEpsMach * fabs(y));
}

template <int NP>
__device__ __forceinline__ void lagrange(double x, const double* xgp, const double* wb, double* L) {
  bool hit = false;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    L[i] = 0.0;
    if (almost_equal_unity(x, xgp[i])) { L[i] = 1.0; hit = true; }
  }
  if (hit) return;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NP; ++i) { L[i] = wb[i] / (x - xgp[i]); s = s + L[i]; }
#pragma unroll
  for (int i = 0; i < NP; ++i) L[i] = L[i] / s;
}

// FP32 variant (mixed precision): same barycentric formula, node hit within FP32 eps
template <int NP>
__device__ __forceinline__ void lagrange_f(float x, const float* xgp, const float* wb, float* L) {
  bool hit = false;
  const float eps = 1.1920929e-07f;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    L[i] = 0.0f;
    float d = fabsf(x - xgp[i]);
    if (d <= eps * fabsf(xgp[i]) || (xgp[i] == 0.0f && d <= 2.0f * eps)) { L[i] = 1.0f; hit = true; }
  }
  if (hit) return;
  float s = 0.0f;
#pragma unroll
  for (int i = 0; i < NP; ++i) { L[i] = __fdiv_rn(wb[i], x - xgp[i]); s += L[i]; }
  const float inv = __frcp_rn(s);
#pragma unroll
  for (int i = 0; i < NP; ++i) L[i] = L[i] * inv;
}

// ==========================================================================================
// x -> xi: GetRefNewtonStartValue (eval_xyz.f90:498-612) + RefElemNewton (:298-445)
// ==========================================================================================
// RefMappingGuess 2 and 3 (:564-601): xi of the closest Gauss point of the element's degree, or of the closest
// corner (XCL_NGeo at NGeo = 1); distances in the reference's order with its per-axis early exits
static __device__ __noinline__ void newton_start_closest(const DevMesh& M, int e, const double x[3], double xi[3]) {
  const Consts& kc = M.k;
  if (kc.ref_guess == 2) {
    const int nl = M.elem_n ? __ldg(M.elem_n + e) : kc.N, n1 = nl + 1;
    const double* xg = kc.xgp_n[nl];
    const double* P = M.elem_xgp + (M.dof_off ? (size_t)__ldg(M.dof_off + e) : (size_t)e * kc.ndof) * 3;
    const double d0 = x[0] - __ldg(P), d1 = x[1] - __ldg(P + 1), d2 = x[2] - __ldg(P + 2);
    double winner = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    xi[0] = xi[1] = xi[2] = xg[0];
    for (int i = 0; i < n1; ++i)
      for (int j = 0; j < n1; ++j)
        for (int k = 0; k < n1; ++k) {
          const double* Q = P + (size_t)(k * n1 * n1 + j * n1 + i) * 3;
          const double dX = fabs(x[0] - __ldg(Q));
          if (dX > winner) continue;
          const double dY = fabs(x[1] - __ldg(Q + 1));
          if (dY > winner) continue;
          const double dZ = fabs(x[2] - __ldg(Q + 2));
          if (dZ > winner) continue;
          const double dist = sqrt(dX * dX + dY * dY + dZ * dZ);
          if (dist < winner) { winner = dist; xi[0] = xg[i]; xi[1] = xg[j]; xi[2] = xg[k]; }
        }
    return;
  }
  // XCL_NGeo: corner (i, j, k) at tensor index i + 2 j + 4 k (NGeo = 1), CL point (i, j, k) of XCL_NGeo else
  const int g1 = kc.ngeo + 1;
  const double* X = M.xcl_ng ? M.xcl_ng + (size_t)e * g1 * g1 * g1 * 3 : M.xcl + (size_t)e * 24;
  const double* xcl = M.xcl_ng ? kc.xi_cl_ng : kc.xi_cl;
  const double d0 = x[0] - __ldg(X), d1 = x[1] - __ldg(X + 1), d2 = x[2] - __ldg(X + 2);
  double winner = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
  xi[0] = xi[1] = xi[2] = xcl[0];
  for (int i = 0; i < g1; ++i)
    for (int j = 0; j < g1; ++j)
      for (int k = 0; k < g1; ++k) {
        const double* Q = X + (i + g1 * (j + g1 * k)) * 3;
        const double dX = fabs(x[0] - __ldg(Q));
        if (dX > winner) continue;
        const double dY = fabs(x[1] - __ldg(Q + 1));
        if (dY > winner) continue;
        const double dZ = fabs(x[2] - __ldg(Q + 2));
        if (dZ > winner) continue;
        const double dist = sqrt(dX * dX + dY * dY + dZ * dZ);
        if (dist < winner) { winner = dist; xi[0] = xcl[i]; xi[1] = xcl[j]; xi[2] = xcl[k]; }
      }
}

__device__ __forceinline__ void newton_start(const DevMesh& M, int e, const double x[3], double xi[3]) {
  const Consts& kc = M.k;
  if (kc.ref_guess != 1) {
    if (kc.ref_guess == 4) { xi[0] = xi[1] = xi[2] = 0.0; return; }
    newton_start_closest(M, e, x, xi);
    return;
  }
  const double epsOne = 1.0 + kc.refmapping_eps;
  const double* b = M.bary + (size_t)e * 3;
  double P0 = x[0] - __ldg(b + 0), P1 = x[1] - __ldg(b + 1), P2 = x[2] - __ldg(b + 2);
  double xil[6];
  const double* B = M.xez + (size_t)e * 18;
  const double* S = M.slen + (size_t)e * 6;
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    double dp = P0 * __ldg(B + 3 * d) + P1 * __ldg(B + 3 * d + 1) + P2 * __ldg(B + 3 * d + 2);
    xil[d] = dp * __ldg(S + d);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) xi[d] = 0.5 * (xil[d] - xil[d + 3]);
  double mx = fmax(fabs(xi[0]), fmax(fabs(xi[1]), fabs(xi[2])));
  if (mx > epsOne) {
#pragma unroll
    for (int d = 0; d < 3; ++d) xi[d] = fmax(fmin(1.0, xi[d]), -1.0);
  }
}

// Returns isSuccessful (false when the iterate left |xi| <= 1.5).
__device__ __forceinline__ bool ref_elem_newton_lin(const DevMesh& M, int e, const double x[3], double xi[3]) {
  const Consts& kc = M.k;
  const double* X = M.xcl + (size_t)e * 24;
  const double* DX = M.dxcl + (size_t)e * 72;
  double Xl[24];
#pragma unroll
  for (int q = 0; q < 24; ++q) Xl[q] = __ldg(X + q);
  double L[3][2];
#pragma unroll
  for (int d = 0; d < 3; ++d) lagrange<2>(xi[d], kc.xi_cl, kc.wbary_cl, L[d]);
  double F[3] = {-x[0], -x[1], -x[2]};
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      double buff = L[1][j] * L[2][k];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int t = i + 2 * j + 4 * k;
#pragma unroll
        for (int c = 0; c < 3; ++c) F[c] = F[c] + Xl[3 * t + c] * L[0][i] * buff;
      }
    }
  double deltaXi2 = (fabs(F[0]) < kEpsMach && fabs(F[1]) < kEpsMach && fabs(F[2]) < kEpsMach) ? 0.0 : 1.0;
  double normF = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
  int iter = 0;
  bool success = true;
  while (deltaXi2 > kc.refmapping_eps && iter < 100) {
    iter = iter + 1;
    double J[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) J[a][b] = 0.0;
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        double buff = L[1][j] * L[2][k];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          double buff2 = L[0][i] * buff;
          const int t = i + 2 * j + 4 * k;
#pragma unroll
          for (int nn = 0; nn < 3; ++nn)
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) J[nn][dd] = J[nn][dd] + __ldg(DX + 9 * t + 3 * nn + dd) * buff2;
        }
      }
    double sdet = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * J[2][2] + (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * J[2][0] +
                  (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * J[2][1];
    if (sdet > 0.0) sdet = 1.0 / sdet;
    double sJ[3][3];
    sJ[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * sdet;
    sJ[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * sdet;
    sJ[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * sdet;
    sJ[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * sdet;
    sJ[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * sdet;
    sJ[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * sdet;
    sJ[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * sdet;
    sJ[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * sdet;
    sJ[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * sdet;
    double dxi[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) dxi[r] = ((0.0 + sJ[r][0] * F[0]) + sJ[r][1] * F[1]) + sJ[r][2] * F[2];
    deltaXi2 = dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2];
    double xo[3] = {xi[0], xi[1], xi[2]};
    double normFold = normF;
    normF = normF * 2.0;
    double lambda = 1.0;
    int iArmijo = 1;
    while (normF > normFold * (1.0 - 0.0001 * lambda) && iArmijo <= 8) {
#pragma unroll
      for (int d = 0; d < 3; ++d) xi[d] = xo[d] - lambda * dxi[d];
#pragma unroll
      for (int d = 0; d < 3; ++d) lagrange<2>(xi[d], kc.xi_cl, kc.wbary_cl, L[d]);
      F[0] = -x[0]; F[1] = -x[1]; F[2] = -x[2];
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          double buff = L[1][j] * L[2][k];
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            double buff2 = L[0][i] * buff;
            const int t = i + 2 * j + 4 * k;
#pragma unroll
            for (int c = 0; c < 3; ++c) F[c] = F[c] + Xl[3 * t + c] * buff2;
          }
        }
      lambda = 0.2 * lambda;
      iArmijo = iArmijo + 1;
      normF = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
    }
    if (fabs(xi[0]) > 1.5 || fabs(xi[1]) > 1.5 || fabs(xi[2]) > 1.5) { success = false; break; }
  }
  return success;
}

// ---- double-FP32 ("double-float") arithmetic: a value is the unevaluated sum hi + lo of two floats, |lo| <= ulp(hi)/2,
// about 48 significant bits.  Error-free transforms after Dekker (1971, "A floating-point technique for extending
// the available precision") and Knuth (TwoSum, TAOCP vol. 2, 4.2.2), the product error from one fused multiply-add,
// and the accurate addition of Hida, Li and Bailey (QD library, 2001).  GB300 runs FP32 at about 70x its FP64 rate.
struct DF { float hi, lo; };
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {      // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  const DF s = df_two_sum(x.hi, y.hi), t = df_two_sum(x.lo, y.lo);
  const DF u = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
__device__ __forceinline__ DF df_mul(DF x, DF y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) { return df_add(df_mul(a, b), c); }
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_div(DF a, DF b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const DF r = df_add(a, df_neg(df_mul(DF{q1, 0.f}, b)));
  return df_fast_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ DF df_of(double d) {
  const float h = __double2float_rn(d);
  return DF{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double df_val(DF a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ DF df_ld(const float2* __restrict__ p) { const float2 v = __ldg(p); return DF{v.x, v.y}; }
__device__ __forceinline__ DF df_c(float2 v) { return DF{v.x, v.y}; }
// a > b for normalised pairs
__device__ __forceinline__ bool df_gt(DF a, DF b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ DF df_abs(DF a) { return a.hi < 0.f ? df_neg(a) : a; }

// GetRefNewtonStartValue, RefMappingGuess 1 (eval_xyz.f90:498-535) in double-FP32 arithmetic on the scaled
// data S (bary / s_e, XiEtaZetaBasis, slen s_e) and the scaled position xs
__device__ __forceinline__ void df_start(const Consts& kc, const float2* __restrict__ S, const DF xs[3], DF z[3]) {
  const DF P[3] = {df_add(xs[0], df_neg(df_ld(S))), df_add(xs[1], df_neg(df_ld(S + 1))), df_add(xs[2], df_neg(df_ld(S + 2)))};
  DF xil[6];
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    const DF dp = df_add(df_add(df_mul(P[0], df_ld(S + 3 + 3 * d)), df_mul(P[1], df_ld(S + 4 + 3 * d))),
                         df_mul(P[2], df_ld(S + 5 + 3 * d)));
    xil[d] = df_mul(dp, df_ld(S + 21 + d));
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) z[d] = df_mul(DF{0.5f, 0.f}, df_add(xil[d], df_neg(xil[d + 3])));
  const DF one_eps = df_c(kc.df_one_eps);
  if (df_gt(df_abs(z[0]), one_eps) || df_gt(df_abs(z[1]), one_eps) || df_gt(df_abs(z[2]), one_eps)) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (df_gt(z[d], DF{1.f, 0.f})) z[d] = DF{1.f, 0.f};
      if (df_gt(DF{-1.f, 0.f}, z[d])) z[d] = DF{-1.f, 0.f};
    }
  }
}

// Newton of the mixed variant: the same start value, stopping rule (||dxi||^2 <= RefMappingEps, 100 iterations,
// taken in FP64 from the double-FP32 value), Armijo damping and plausibility bound as RefElemNewton, but on the
// NGeo = 1 map in monomial form (DevMesh::tcoef_df: the residual in 18 and the Jacobian in 30 multiply-adds instead
// of the tensor-product sums over 8 corners, one reciprocal of det(J) per iteration) and in double-FP32 arithmetic
// (relative error ~1e-14 instead of ~1e-16): the same map, so the iterates follow the FP64 ones to ~1e-13 in xi.  The map is scaled by the element's power-of-two size s_e
// (exact): dxi and the Armijo ratios do not change, the initial |F| < epsMach test compares |F/s_e| s_e.
// one Newton iteration's common tail in double-FP32 arithmetic: dxi = J^-1 F from the cofactors, ||dxi||^2, and
// the Armijo line search on F; EVAL(z, F) evaluates the residual.  Returns false when |xi| left 1.5.
template <class EVAL>
__device__ __forceinline__ bool df_newton_step(const Consts& kc, const DF (*J)[3], DF z[3], DF F[3], DF& normF,
                                               DF& deltaXi2, bool& moved, EVAL&& eval) {
  auto norm2 = [&](const DF v[3]) { return df_fma(v[0], v[0], df_fma(v[1], v[1], df_mul(v[2], v[2]))); };
  auto cof = [&](const DF& a, const DF& b, const DF& cc, const DF& d) { return df_add(df_mul(a, b), df_neg(df_mul(cc, d))); };
  const DF c00 = cof(J[1][1], J[2][2], J[1][2], J[2][1]);
  const DF c01 = cof(J[0][2], J[2][1], J[0][1], J[2][2]);
  const DF c02 = cof(J[0][1], J[1][2], J[0][2], J[1][1]);
  const DF c10 = cof(J[1][2], J[2][0], J[1][0], J[2][2]);
  const DF c11 = cof(J[0][0], J[2][2], J[0][2], J[2][0]);
  const DF c12 = cof(J[0][2], J[1][0], J[0][0], J[1][2]);
  const DF c20 = cof(J[1][0], J[2][1], J[1][1], J[2][0]);
  const DF c21 = cof(J[0][1], J[2][0], J[0][0], J[2][1]);
  const DF c22 = cof(J[0][0], J[1][1], J[0][1], J[1][0]);
  const DF det = df_fma(J[0][0], c00, df_fma(J[0][1], c10, df_mul(J[0][2], c20)));
  const DF sd = det.hi > 0.f ? df_div(DF{1.f, 0.f}, det) : det;
  DF dxi[3];
  dxi[0] = df_mul(df_fma(c00, F[0], df_fma(c01, F[1], df_mul(c02, F[2]))), sd);
  dxi[1] = df_mul(df_fma(c10, F[0], df_fma(c11, F[1], df_mul(c12, F[2]))), sd);
  dxi[2] = df_mul(df_fma(c20, F[0], df_fma(c21, F[1], df_mul(c22, F[2]))), sd);
  deltaXi2 = norm2(dxi);
  const DF zo[3] = {z[0], z[1], z[2]};
  const DF normFold = normF;
  // Armijo: the first trial always runs unless ||F||^2 = 0 (2 ||F||^2 > (1 - 1e-4) ||F||^2); lambda_k = 0.2^k
  bool go = normFold.hi > 0.f;
  for (int k = 0; go && k < 8; ++k) {
    moved = true;
    const DF lam = df_c(kc.df_lam[k]);
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) z[dd] = df_fma(lam, dxi[dd], zo[dd]);
    eval(z, F);
    normF = norm2(F);
    go = df_gt(normF, df_mul(normFold, df_c(kc.df_arm[k + 1])));
  }
  return !(fabsf(z[0].hi) > 1.5f || fabsf(z[1].hi) > 1.5f || fabsf(z[2].hi) > 1.5f);
}

// Newton of the mixed variant: the same start value, stopping rule (||dxi||^2 <= RefMappingEps, 100 iterations),
// Armijo damping and plausibility bound as RefElemNewton, but on the NGeo = 1 map in monomial form
// (DevMesh::tcoef_df: the residual in 18 and the Jacobian in 30 multiply-adds instead of the tensor-product sums
// over 8 corners, one reciprocal of det(J) per iteration) and in double-FP32 arithmetic (relative error ~1e-14
// instead of ~1e-16), the start value of RefMappingGuess 1 too (start): the same map, so the iterates follow the
// FP64 ones to ~1e-13 in xi.  The map is scaled by the element's power-of-two size s_e (exact): dxi and the
// Armijo ratios do not change, the initial |F| < epsMach test compares |F/s_e| s_e.
__device__ __forceinline__ bool ref_elem_newton_df_lin(const DevMesh& M, int e, const double x[3], double xi[3],
                                                       bool start) {
  const Consts& kc = M.k;
  const float2* Cg = M.tcoef_df + (size_t)e * kDfLin;
  DF c[8][3];
#pragma unroll
  for (int q = 0; q < 8; ++q)
#pragma unroll
    for (int k = 0; k < 3; ++k) c[q][k] = df_ld(Cg + 3 * q + k);
  const float2 sc = __ldg(Cg + 24);
  const double* by = M.bary + (size_t)e * 3;       // the map is stored relative to the barycentre
  const DF xs[3] = {df_of((x[0] - __ldg(by)) * (double)sc.y), df_of((x[1] - __ldg(by + 1)) * (double)sc.y),
                    df_of((x[2] - __ldg(by + 2)) * (double)sc.y)};
#pragma unroll
  for (int k = 0; k < 3; ++k) c[0][k] = df_add(c[0][k], df_neg(xs[k]));
  auto residual = [&](const DF z[3], DF F[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const DF t = df_add(df_mul(z[1], df_fma(z[2], c[7][k], c[4][k])), df_fma(z[2], c[5][k], c[1][k]));
      const DF u = df_fma(z[2], c[6][k], c[2][k]);
      F[k] = df_fma(z[0], t, df_fma(z[1], u, df_fma(z[2], c[3][k], c[0][k])));
    }
  };
  DF z[3];
  if (start) df_start(kc, Cg + 25, xs, z);
  else { z[0] = df_of(xi[0]); z[1] = df_of(xi[1]); z[2] = df_of(xi[2]); }
  DF F[3];
  residual(z, F);
  const float eps = (float)kEpsMach;
  bool moved = start;
  bool more = !(fabsf(F[0].hi) * sc.x < eps && fabsf(F[1].hi) * sc.x < eps && fabsf(F[2].hi) * sc.x < eps);
  DF normF = df_fma(F[0], F[0], df_fma(F[1], F[1], df_mul(F[2], F[2])));
  bool success = true;
  const DF eps_map = df_c(kc.df_eps);
  for (int iter = 0; iter < 100 && more; ++iter) {
    const DF z12 = df_mul(z[0], z[1]), z13 = df_mul(z[0], z[2]), z23 = df_mul(z[1], z[2]);
    DF J[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      J[k][0] = df_fma(z23, c[7][k], df_fma(z[2], c[5][k], df_fma(z[1], c[4][k], c[1][k])));
      J[k][1] = df_fma(z13, c[7][k], df_fma(z[2], c[6][k], df_fma(z[0], c[4][k], c[2][k])));
      J[k][2] = df_fma(z12, c[7][k], df_fma(z[1], c[6][k], df_fma(z[0], c[5][k], c[3][k])));
    }
    DF d2;
    if (!df_newton_step(kc, J, z, F, normF, d2, moved, residual)) { success = false; break; }
    more = df_gt(d2, eps_map);
  }
  if (moved) { xi[0] = df_val(z[0]); xi[1] = df_val(z[1]); xi[2] = df_val(z[2]); }
  return success;
}

static __device__ __noinline__ void lagrange_rt(double x, int np, const double* xgp, const double* wb, double* L) {
  bool hit = false;
  for (int i = 0; i < np; ++i) {
    L[i] = 0.0;
    if (almost_equal_unity(x, xgp[i])) { L[i] = 1.0; hit = true; }
  }
  if (hit) return;
  double s = 0.0;
  for (int i = 0; i < np; ++i) { L[i] = wb[i] / (x - xgp[i]); s = s + L[i]; }
  for (int i = 0; i < np; ++i) L[i] = L[i] / s;
}

// RefElemNewton (eval_xyz.f90:298-445) on the NGeo map of a curved element, in the reference's order
__device__ __forceinline__ bool ref_elem_newton_ng(const DevMesh& M, int e, const double x[3], double xi[3]) {
  const Consts& kc = M.k;
  const int n1 = kc.ngeo + 1;
  const size_t n3 = (size_t)n1 * n1 * n1;
  const double* X = M.xcl_ng + (size_t)e * n3 * 3;
  const double* DX = M.dxcl_ng + (size_t)e * n3 * 9;
  double L[3][kMaxNGeo + 1];
  for (int d = 0; d < 3; ++d) lagrange_rt(xi[d], n1, kc.xi_cl_ng, kc.wbary_cl_ng, L[d]);
  double F[3] = {-x[0], -x[1], -x[2]};
  for (int k = 0; k < n1; ++k)
    for (int j = 0; j < n1; ++j) {
      const double buff = L[1][j] * L[2][k];
      for (int i = 0; i < n1; ++i) {
        const double* P = X + ((size_t)(k * n1 + j) * n1 + i) * 3;
        for (int c = 0; c < 3; ++c) F[c] = F[c] + __ldg(P + c) * L[0][i] * buff;
      }
    }
  double deltaXi2 = (fabs(F[0]) < kEpsMach && fabs(F[1]) < kEpsMach && fabs(F[2]) < kEpsMach) ? 0.0 : 1.0;
  double normF = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
  int iter = 0;
  bool success = true;
  while (deltaXi2 > kc.refmapping_eps && iter < 100) {
    iter = iter + 1;
    double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int k = 0; k < n1; ++k)
      for (int j = 0; j < n1; ++j) {
        const double buff = L[1][j] * L[2][k];
        for (int i = 0; i < n1; ++i) {
          const double buff2 = L[0][i] * buff;
          const double* D = DX + ((size_t)(k * n1 + j) * n1 + i) * 9;
#pragma unroll
          for (int nn = 0; nn < 3; ++nn)
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) J[nn][dd] = J[nn][dd] + __ldg(D + 3 * nn + dd) * buff2;
        }
      }
    double sdet = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * J[2][2] + (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * J[2][0] +
                  (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * J[2][1];
    if (sdet > 0.0) sdet = 1.0 / sdet;
    double sJ[3][3];
    sJ[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * sdet;
    sJ[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * sdet;
    sJ[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * sdet;
    sJ[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * sdet;
    sJ[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * sdet;
    sJ[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * sdet;
    sJ[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * sdet;
    sJ[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * sdet;
    sJ[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * sdet;
    double dxi[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) dxi[r] = ((0.0 + sJ[r][0] * F[0]) + sJ[r][1] * F[1]) + sJ[r][2] * F[2];
    deltaXi2 = dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2];
    const double xo[3] = {xi[0], xi[1], xi[2]};
    const double normFold = normF;
    normF = normF * 2.0;
    double lambda = 1.0;
    for (int iArmijo = 1; normF > normFold * (1.0 - 0.0001 * lambda) && iArmijo <= 8; ++iArmijo) {
      for (int d = 0; d < 3; ++d) xi[d] = xo[d] - lambda * dxi[d];
      for (int d = 0; d < 3; ++d) lagrange_rt(xi[d], n1, kc.xi_cl_ng, kc.wbary_cl_ng, L[d]);
      F[0] = -x[0]; F[1] = -x[1]; F[2] = -x[2];
      for (int k = 0; k < n1; ++k)
        for (int j = 0; j < n1; ++j) {
          const double buff = L[1][j] * L[2][k];
          for (int i = 0; i < n1; ++i) {
            const double buff2 = L[0][i] * buff;
            const double* P = X + ((size_t)(k * n1 + j) * n1 + i) * 3;
            for (int c = 0; c < 3; ++c) F[c] = F[c] + __ldg(P + c) * buff2;
          }
        }
      lambda = 0.2 * lambda;
      normF = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
    }
    if (fabs(xi[0]) > 1.5 || fabs(xi[1]) > 1.5 || fabs(xi[2]) > 1.5) { success = false; break; }
  }
  return success;
}

// GetPositionInRefElem (eval_xyz.f90:87-117): the NGeo Newton for a curved element of an NGeo > 1 mesh, the
// NGeo = 1 Newton on the corners otherwise
__device__ __forceinline__ bool elem_curved(const DevMesh& M, int e) {
  return M.xcl_ng && (!M.curved || __ldg(M.curved + e) != 0);
}

// One out-of-line Newton per call site (the curved and the trilinear forms inside): the kernels call it from
// many places, and a second out-of-line callee per site multiplies the compile time
static __device__ __noinline__ bool ref_elem_newton(const DevMesh& M, int e, const double x[3], double xi[3]) {
  return elem_curved(M, e) ? ref_elem_newton_ng(M, e, x, xi) : ref_elem_newton_lin(M, e, x, xi);
}

__device__ __forceinline__ bool position_in_ref_elem(const DevMesh& M, int e, const double x[3], double xi[3]) {
  newton_start(M, e, x, xi);
  return ref_elem_newton(M, e, x, xi);
}

// Mixed variant, curved element: the Newton of ref_elem_newton_df_lin on the NGeo map in power form (nested Horner
// for x(xi) and its Jacobian, no divisions) instead of the barycentric Lagrange sums over the (NGeo+1)^3 CL points,
// in double-FP32 arithmetic with the map scaled by the element's power-of-two size; the same start value, stopping
// rule, Armijo damping and bound as RefElemNewton on the same map
// x(z) - x (scaled) of the power form and, with WJ, its Jacobian J[nn][dd] = d x_nn / d xi_dd (nested Horner)
template <int NG, bool WJ>
static __device__ __noinline__ void df_eval_ng(const float2* __restrict__ Cg, const DF xs[3], const DF z[3], DF F[3],
                                               DF (*J)[3]) {
  constexpr int n1 = NG + 1;
  auto ld = [&](int i) { const float2 v = __ldg(Cg + i); return DF{v.x, v.y}; };
#pragma unroll 1
  for (int k = 0; k < 3; ++k) {
    const DF zero{0.f, 0.f};
    DF q = zero, q0 = zero, q1 = zero, q2 = zero;
#pragma unroll 1
    for (int c = NG; c >= 0; --c) {
      DF r = zero, r0 = zero, r1 = zero;
#pragma unroll 1
      for (int b = NG; b >= 0; --b) {
        const int base = ((c * n1 + b) * n1) * 3 + k;
        DF p = ld(base + 3 * NG), dp = zero;
#pragma unroll
        for (int a = NG - 1; a >= 0; --a) {
          if (WJ) dp = df_fma(dp, z[0], p);
          p = df_fma(p, z[0], ld(base + 3 * a));
        }
        if (WJ) { r1 = df_fma(r1, z[1], r); r0 = df_fma(r0, z[1], dp); }
        r = df_fma(r, z[1], p);
      }
      if (WJ) { q2 = df_fma(q2, z[2], q); q0 = df_fma(q0, z[2], r0); q1 = df_fma(q1, z[2], r1); }
      q = df_fma(q, z[2], r);
    }
    F[k] = df_add(q, df_neg(xs[k]));
    if (WJ) { J[k][0] = q0; J[k][1] = q1; J[k][2] = q2; }
  }
}

template <int NG>
static __device__ __noinline__ bool ref_elem_newton_df_ng(const DevMesh& M, int e, const double x[3], double xi[3],
                                                          bool start) {
  const Consts& kc = M.k;
  constexpr int n1 = NG + 1, n3 = n1 * n1 * n1;
  const float2* Cg = M.tcoef_ng_df + (size_t)e * (n3 * 3 + 1 + kDfStart);
  const float2 sc = __ldg(Cg + n3 * 3);
  const double* by = M.bary + (size_t)e * 3;       // the map is stored relative to the barycentre
  const DF xs[3] = {df_of((x[0] - __ldg(by)) * (double)sc.y), df_of((x[1] - __ldg(by + 1)) * (double)sc.y),
                    df_of((x[2] - __ldg(by + 2)) * (double)sc.y)};
  DF z[3];
  if (start) df_start(kc, Cg + n3 * 3 + 1, xs, z);
  else { z[0] = df_of(xi[0]); z[1] = df_of(xi[1]); z[2] = df_of(xi[2]); }
  auto residual = [&](const DF zz[3], DF F[3]) { df_eval_ng<NG, false>(Cg, xs, zz, F, nullptr); };
  DF F[3];
  residual(z, F);
  const float eps = (float)kEpsMach;
  bool moved = start;
  bool more = !(fabsf(F[0].hi) * sc.x < eps && fabsf(F[1].hi) * sc.x < eps && fabsf(F[2].hi) * sc.x < eps);
  DF normF = df_fma(F[0], F[0], df_fma(F[1], F[1], df_mul(F[2], F[2])));
  bool success = true;
  const DF eps_map = df_c(kc.df_eps);
  for (int iter = 0; iter < 100 && more; ++iter) {
    DF J[3][3], Fd[3];
    df_eval_ng<NG, true>(Cg, xs, z, Fd, J);
    DF d2;
    if (!df_newton_step(kc, J, z, F, normF, d2, moved, residual)) { success = false; break; }
    more = df_gt(d2, eps_map);
  }
  if (moved) { xi[0] = df_val(z[0]); xi[1] = df_val(z[1]); xi[2] = df_val(z[2]); }
  return success;
}

__device__ __forceinline__ bool ref_elem_newton_fast_curved(const DevMesh& M, int e, const double x[3], double xi[3],
                                                            bool start) {
  switch (M.k.ngeo) {
    case 2: return ref_elem_newton_df_ng<2>(M, e, x, xi, start);
    case 3: return ref_elem_newton_df_ng<3>(M, e, x, xi, start);
    default: return ref_elem_newton_df_ng<4>(M, e, x, xi, start);
  }
}

// the mixed variant's Newton: power forms of the trilinear or the curved map in double-FP32 arithmetic; with start
// it takes RefMappingGuess 1 itself (in double-FP32), else xi holds the start value
static __device__ __noinline__ bool ref_elem_newton_fast(const DevMesh& M, int e, const double x[3], double xi[3],
                                                        bool start) {
  if (elem_curved(M, e)) {
    if (M.tcoef_ng_df) return ref_elem_newton_fast_curved(M, e, x, xi, start);
    if (start) newton_start(M, e, x, xi);
    return ref_elem_newton_ng(M, e, x, xi);
  }
  if (M.tcoef_df) return ref_elem_newton_df_lin(M, e, x, xi, start);
  if (start) newton_start(M, e, x, xi);
  return ref_elem_newton_lin(M, e, x, xi);
}

template <bool FAST>
__device__ __forceinline__ bool position_in_ref_elem_t(const DevMesh& M, int e, const double x[3], double xi[3]) {
  if (FAST && M.k.ref_guess == 1) return ref_elem_newton_fast(M, e, x, xi, true);
  newton_start(M, e, x, xi);
  return FAST ? ref_elem_newton_fast(M, e, x, xi, false) : ref_elem_newton(M, e, x, xi);
}

// ==========================================================================================
// Field at a reference position: EvaluateFieldAtRefPos, eval_xyz.f90:167-215 (NVar_in = 3)
// ==========================================================================================
template <int N>
__device__ __forceinline__ void eval_field(const Consts& kc, const double* __restrict__ U, const double xi[3], double out[3]) {
  constexpr int n1 = N + 1;
  double L[3][n1];
#pragma unroll
  for (int d = 0; d < 3; ++d) lagrange<n1>(xi[d], kc.xgp_n[N], kc.wbary_n[N], L[d]);
  out[0] = out[1] = out[2] = 0.0;
#pragma unroll
  for (int k = 0; k < n1; ++k)
#pragma unroll
    for (int j = 0; j < n1; ++j) {
      double Lez = L[1][j] * L[2][k];
#pragma unroll
      for (int i = 0; i < n1; ++i) {
        const double* u = U + ((k * n1 + j) * n1 + i) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c] = out[c] + __ldg(u + c) * L[0][i] * Lez;
      }
    }
}

// GetEMFieldDW, pic_interpolation_tools.f90:458-527 (inverse-distance fallback when Newton failed)
// (U and xg: the element's field and DOF coordinates)
template <int N>
static __device__ __noinline__ void eval_field_dw(const double* __restrict__ U, const double* __restrict__ xg,
                                                  const double x[3], double out[3]) {
  constexpr int n1 = N + 1, nd = n1 * n1 * n1;
  double dist[nd];
#pragma unroll
  for (int r = 0; r < nd; ++r) dist[r] = 0.0;
  double DistSum = 0.0;
  for (int k = 0; k < n1; ++k)
    for (int l = 0; l < n1; ++l)
      for (int mm = 0; mm < n1; ++mm) {
        int r = k + n1 * (l + n1 * mm);
        double v0 = __ldg(xg + 3 * r) - x[0], v1 = __ldg(xg + 3 * r + 1) - x[1], v2 = __ldg(xg + 3 * r + 2) - x[2];
        double norm = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
        if (norm > 0.0) {
          dist[r] = 1.0 / norm;
        } else {
          for (int q = 0; q < nd; ++q) dist[q] = 0.0;
          dist[r] = 1.0;
          DistSum = 1.0;
          break;
        }
        DistSum = DistSum + dist[r];
      }
  out[0] = out[1] = out[2] = 0.0;
  for (int k = 0; k < n1; ++k)
    for (int l = 0; l < n1; ++l)
      for (int mm = 0; mm < n1; ++mm) {
        int r = k + n1 * (l + n1 * mm);
        for (int c = 0; c < 3; ++c) out[c] = out[c] + dist[r] / DistSum * __ldg(U + 3 * r + c);
      }
}

// ---- per-element polynomial degree (p-adaption) ---------------------------------------------
// Kernels instantiated for a degree N > 0 address the DOFs of element e at e (N+1)^3, or at its
// N_DG_Mapping(1,e) offset on a p-adapted mesh (element-parallel kernels run per degree group there).
// N = 0 instantiates the particle kernels for p-adapted meshes: they dispatch on the element's own degree.
template <int N>
__device__ __forceinline__ size_t dof_base(const DevMesh& M, int e) {
  if constexpr (N == 0) return (size_t)__ldg(M.dof_off + e);
  else return M.dof_off ? (size_t)__ldg(M.dof_off + e) : (size_t)e * ((N + 1) * (N + 1) * (N + 1));
}

// EvaluateFieldAtRefPos with Nloc (pic_interpolation_tools.f90:427-433): E of element e at xi
template <int N>
__device__ __forceinline__ void field_at(const DevMesh& M, const double* __restrict__ E, int e, const double xi[3],
                                         double out[3]) {
  if constexpr (N > 0) {
    eval_field<N>(M.k, E + (size_t)e * ((N + 1) * (N + 1) * (N + 1)) * 3, xi, out);
  } else {
    const double* U = E + (size_t)__ldg(M.dof_off + e) * 3;
    switch (__ldg(M.elem_n + e)) {
      case 1: eval_field<1>(M.k, U, xi, out); break;
      case 2: eval_field<2>(M.k, U, xi, out); break;
      case 3: eval_field<3>(M.k, U, xi, out); break;
      default: eval_field<4>(M.k, U, xi, out); break;     // degrees are 1..4 (checked at pic_create)
    }
  }
}

// GetEMFieldDW with Nloc: the inverse-distance fallback of element e at x
template <int N>
__device__ __forceinline__ void field_dw_at(const DevMesh& M, const double* __restrict__ E, int e, const double x[3],
                                            double out[3]) {
  if constexpr (N > 0) {
    const size_t b = (size_t)e * ((N + 1) * (N + 1) * (N + 1));
    eval_field_dw<N>(E + b * 3, M.elem_xgp + b * 3, x, out);
  } else {
    const size_t b = (size_t)__ldg(M.dof_off + e);
    switch (__ldg(M.elem_n + e)) {
      case 1: eval_field_dw<1>(E + b * 3, M.elem_xgp + b * 3, x, out); break;
      case 2: eval_field_dw<2>(E + b * 3, M.elem_xgp + b * 3, x, out); break;
      case 3: eval_field_dw<3>(E + b * 3, M.elem_xgp + b * 3, x, out); break;
      default: eval_field_dw<4>(E + b * 3, M.elem_xgp + b * 3, x, out); break;
    }
  }
}

// ==========================================================================================
// Boris-Leapfrog push, timedisc_TimeStepPoissonByBorisLeapfrog.f90:128-197 (FP64)
// ==========================================================================================
__device__ __forceinline__ void boris_push(const Consts& kc, double v[3], const double F[6], int sp, bool& is_new, double dt) {
  const double q = kc.q[sp], mass = kc.m[sp];
  const bool push = fabs(q) > 0.0;
  if (is_new) {
    if (push) {
      double qmt = q / mass;
#pragma unroll
      for (int c = 0; c < 3; ++c) v[c] = v[c] - (F[c] * qmt) * dt * 0.5;
    }
    is_new = false;
  }
  if (!push) return;
  const double c2_inv = kc.c2_inv;
  double c1 = (q * dt) / (mass * 2.0);
  double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  double gamma = 1.0 / sqrt(1.0 - (vv * c2_inv));
  double vm[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) vm[c] = v[c] * gamma + c1 * F[c];
  double gm = sqrt(1.0 + (vm[0] * vm[0] + vm[1] * vm[1] + vm[2] * vm[2]) * c2_inv);
  double Bn = sqrt(F[3] * F[3] + F[4] * F[4] + F[5] * F[5]);
  double t[3] = {0.0, 0.0, 0.0};
  if (fabs(Bn) > 0.0) {
    double tn = tan(c1 / gm * Bn);
    double invL = 1.0 / Bn;
#pragma unroll
    for (int c = 0; c < 3; ++c) t[c] = tn * (F[3 + c] * invL);
  } else {
    double tn = tan(c1 / gm * Bn);   // tan(0): keeps the reference's evaluation (t = tan(.)*0)
#pragma unroll
    for (int c = 0; c < 3; ++c) t[c] = tn * 0.0;
  }
  double vp[3] = {vm[0] + (vm[1] * t[2] - vm[2] * t[1]), vm[1] + (vm[2] * t[0] - vm[0] * t[2]),
                  vm[2] + (vm[0] * t[1] - vm[1] * t[0])};
  double fac = 2.0 / (1.0 + (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
  double vn1[3];
  vn1[0] = vm[0] + fac * (vp[1] * t[2] - vp[2] * t[1]);
  vn1[1] = vm[1] + fac * (vp[2] * t[0] - vp[0] * t[2]);
  vn1[2] = vm[2] + fac * (vp[0] * t[1] - vp[1] * t[0]);
#pragma unroll
  for (int c = 0; c < 3; ++c) vn1[c] = vn1[c] + c1 * F[c];
  double den = sqrt(1.0 + (vn1[0] * vn1[0] + vn1[1] * vn1[1] + vn1[2] * vn1[2]) * c2_inv);
#pragma unroll
  for (int c = 0; c < 3; ++c) v[c] = vn1[c] / den;
}

// ==========================================================================================
// TriaTracking, particle_triatracking.f90:137-484 with the helpers of particle_mesh_tools.f90
// and particle_intersection.f90 (regular, non-mortar sides)
// ==========================================================================================
__device__ __forceinline__ int side_corner(uint32_t info, int q) { return (info >> (3 * q)) & 7; }
__device__ __forceinline__ bool side_concave(uint32_t info) { return (info >> 12) & 1; }
// particle boundary of a wall side: 0 none (inner or periodic), 1 open, 2 reflective
__device__ __forceinline__ int side_wall(uint32_t info) { return (info >> 24) & 3; }
__device__ __forceinline__ int side_pvid(uint32_t info) { return (int)(int8_t)((info >> 16) & 0xff); }

// ParticleInsideQuad3D, particle_mesh_tools.f90:78-222
__device__ __forceinline__ bool inside_quad3d(const double* __restrict__ X, const uint32_t* __restrict__ sinfo,
                                              const double x[3], double det[6][2]) {
  bool in = true;
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    const uint32_t info = __ldg(sinfo + s);
    double A[3][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int t = side_corner(info, q);
#pragma unroll
      for (int c = 0; c < 3; ++c) A[c][q] = __ldg(X + 3 * t + c) - x[c];
    }
    double cp0 = A[1][0] * A[2][2] - A[2][0] * A[1][2];
    double cp1 = A[2][0] * A[0][2] - A[0][0] * A[2][2];
    double cp2 = A[0][0] * A[1][2] - A[1][0] * A[0][2];
    double d1 = cp0 * A[0][1] + cp1 * A[1][1] + cp2 * A[2][1];
    d1 = -d1;
    double d2 = cp0 * A[0][3] + cp1 * A[1][3] + cp2 * A[2][3];
    det[s][0] = d1;
    det[s][1] = d2;
    bool neg = (d1 < 0.0) || (d2 < 0.0);
    bool pos = !(d1 < 0.0) || !(d2 < 0.0);
    if (side_concave(info)) { if (!pos) in = false; }
    else { if (neg) in = false; }
  }
  return in;
}

// ParticleThroughSideCheck3DFast, particle_intersection.f90:167-280
__device__ __forceinline__ bool through_side(const double* __restrict__ X, uint32_t info, const double P[3],
                                             const double V[3], int tri) {
  double Ax[3], Ay[3], Az[3];
  int t = side_corner(info, 0);
  Ax[0] = __ldg(X + 3 * t) - P[0]; Ay[0] = __ldg(X + 3 * t + 1) - P[1]; Az[0] = __ldg(X + 3 * t + 2) - P[2];
#pragma unroll
  for (int n = 1; n <= 2; ++n) {
    t = side_corner(info, n + tri - 1);
    Ax[n] = __ldg(X + 3 * t) - P[0]; Ay[n] = __ldg(X + 3 * t + 1) - P[1]; Az[n] = __ldg(X + 3 * t + 2) - P[2];
  }
  const double Vx = V[0], Vy = V[1], Vz = V[2];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int a = r, b = (r + 2) % 3;   // row r uses node r and node (r+2)%3
    double c0 = (Ay[a] * Vz - Az[a] * Vy) * Ax[b];
    double c1 = (Az[a] * Vx - Ax[a] * Vz) * Ay[b];
    double c2 = (Ax[a] * Vy - Ay[a] * Vx) * Az[b];
    double det = (c0 + c1) + c2;
    double mn = 1.7976931348623157e308;
    if (fabs(c0) > 0.0 && fabs(c0) < mn) mn = fabs(c0);
    if (fabs(c1) > 0.0 && fabs(c1) < mn) mn = fabs(c1);
    if (fabs(c2) > 0.0 && fabs(c2) < mn) mn = fabs(c2);
    if (!(det >= -kEpsMach * mn)) return false;
  }
  return true;
}

// ParticleThroughSideLastPosCheck, particle_intersection.f90:430-512
__device__ __forceinline__ bool last_pos_check(const double* __restrict__ X, uint32_t info, const double Pl[3], int tri,
                                               double& detOut) {
  double Ax[3], Ay[3], Az[3];
  int t0 = side_corner(info, 0), t1 = side_corner(info, tri), t2 = side_corner(info, tri + 1);
  const int ts[3] = {t0, t1, t2};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    Ax[q] = __ldg(X + 3 * ts[q]) - Pl[0];
    Ay[q] = __ldg(X + 3 * ts[q] + 1) - Pl[1];
    Az[q] = __ldg(X + 3 * ts[q] + 2) - Pl[2];
  }
  double det = ((Ay[0] * Az[1] - Az[0] * Ay[1]) * Ax[2] + (Az[0] * Ax[1] - Ax[0] * Az[1]) * Ay[2] +
                (Ax[0] * Ay[1] - Ay[0] * Ax[1]) * Az[2]);
  detOut = det;
  return !((det < 0.0) || (det != det));
}

// IntersectionWithWall, particle_intersection.f90:79-164 -> alpha
__device__ __forceinline__ double wall_alpha(const double* __restrict__ X, uint32_t info, const double Pold[3],
                                             const double traj[3], int tri) {
  int t0 = side_corner(info, 0), t1 = side_corner(info, tri), t2 = side_corner(info, tri + 1);
  double xN = __ldg(X + 3 * t0), yN = __ldg(X + 3 * t0 + 1), zN = __ldg(X + 3 * t0 + 2);
  double V1[3] = {__ldg(X + 3 * t1) - xN, __ldg(X + 3 * t1 + 1) - yN, __ldg(X + 3 * t1 + 2) - zN};
  double V2[3] = {__ldg(X + 3 * t2) - xN, __ldg(X + 3 * t2 + 1) - yN, __ldg(X + 3 * t2 + 2) - zN};
  double nx = V1[1] * V2[2] - V1[2] * V2[1];
  double ny = V1[2] * V2[0] - V1[0] * V2[2];
  double nz = V1[0] * V2[1] - V1[1] * V2[0];
  double nVal = sqrt(nx * nx + ny * ny + nz * nz);
  nx = nx / nVal; ny = ny / nVal; nz = nz / nVal;
  double bx = Pold[0] - xN, by = Pold[1] - yN, bz = Pold[2] - zN;
  double pr = bx * nx + by * ny + bz * nz;
  double ax = bx - nx * pr, ay = by - ny * pr, az = bz - nz * pr;
  double dist = sqrt(((ay * bz - az * by) * (ay * bz - az * by) + (az * bx - ax * bz) * (az * bx - ax * bz) +
                      (ax * by - ay * bx) * (ax * by - ay * bx)) / (ax * ax + ay * ay + az * az));
  if (dist != dist) dist = sqrt(bx * bx + by * by + bz * bz);
  double alpha = traj[0] * nx + traj[1] * ny + traj[2] * nz;
  if (fabs(alpha) > 0.0) alpha = dist / alpha;
  return alpha;
}

// FP32 pre-filter of ParticleInsideQuad3D: true only if all 12 signed volumes are positive with a
// margin far above the FP32 error, so that the FP64 volumes have the same (positive) signs and the
// particle is inside for convex and concave sides alike; otherwise the caller runs the FP64 test.
// Error bound (L1 norms n_q of the edge vectors A_q, S = |p|_1 + sqrt(3) * element radius >= every
// |corner|_1, |p|_1, |A_q|_1): inputs are off by <= 1.8e-7 S per vector and the FP32 evaluation adds
// <= 3e-7 n_a n_b n_c, so |det32 - det| <= 1.8e-7 S (n_a n_b + n_a n_c + n_b n_c) + 3e-7 n_a n_b n_c.
// The thresholds below are 1e-5 times the same terms (>= 33x margin).
__device__ __forceinline__ bool certainly_inside_f32(const DevMesh& M, int e, const double x[3]) {
  if (!M.xclr) return false;
  const double* b = M.bary + (size_t)e * 3;
  const float p[3] = {(float)(x[0] - __ldg(b)), (float)(x[1] - __ldg(b + 1)), (float)(x[2] - __ldg(b + 2))};
  const float S = fabsf(p[0]) + fabsf(p[1]) + fabsf(p[2]) + 1.7320509f * (float)__ldg(M.radius + e) * 1.0001f;
  const float* X = M.xclr + (size_t)e * 24;
  const uint32_t* sinfo = M.side_info + (size_t)e * 6;
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    const uint32_t info = __ldg(sinfo + s);
    float A[4][3], n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int t = side_corner(info, q);
#pragma unroll
      for (int c = 0; c < 3; ++c) A[q][c] = __ldg(X + 3 * t + c) - p[c];
      n[q] = fabsf(A[q][0]) + fabsf(A[q][1]) + fabsf(A[q][2]);
    }
    // crossP = A1 x A3 ; det1 = -(crossP . A2) ; det2 = crossP . A4  (same vectors as the FP64 test)
    const float cp0 = A[0][1] * A[2][2] - A[0][2] * A[2][1];
    const float cp1 = A[0][2] * A[2][0] - A[0][0] * A[2][2];
    const float cp2 = A[0][0] * A[2][1] - A[0][1] * A[2][0];
    const float d1 = -(cp0 * A[1][0] + cp1 * A[1][1] + cp2 * A[1][2]);
    const float d2 = cp0 * A[3][0] + cp1 * A[3][1] + cp2 * A[3][2];
    const float n02 = n[0] * n[2];
    const float T1 = 1e-5f * (S * (n02 + n[0] * n[1] + n[2] * n[1]) + n02 * n[1]);
    const float T2 = 1e-5f * (S * (n02 + n[0] * n[3] + n[2] * n[3]) + n02 * n[3]);
    if (!(d1 > T1) || !(d2 > T2)) return false;
  }
  return true;
}

// A particle whose position or velocity overflowed in the push (extreme fields) leaves the loop with
// PIC_STATUS_NOT_FINITE instead of walking the mesh with NaN coordinates (NaN passes no test, so the
// inside test would keep it where it is and its deposit would poison PartSource).
__device__ __forceinline__ bool state_finite(const double x[3], double v0, double v1, double v2) {
  return isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(v0) && isfinite(v1) && isfinite(v2);
}

// CalcNormAndTangTriangle, particle_surfaces.f90:256-319 (TriaTracking): unit normal of triangle `tri`,
// (P(tri+1)-P1) x (P(tri+2)-P1) normalised (the routine's two sign flips cancel)
__device__ __forceinline__ void triangle_normal(const double* __restrict__ X, uint32_t info, int tri, double n[3]) {
  const int t0 = side_corner(info, 0), t1 = side_corner(info, tri), t2 = side_corner(info, tri + 1);
  double V1[3], V2[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double p0 = __ldg(X + 3 * t0 + c);
    V1[c] = __ldg(X + 3 * t1 + c) - p0;
    V2[c] = __ldg(X + 3 * t2 + c) - p0;
  }
  const double nx = -V1[1] * V2[2] + V1[2] * V2[1];
  const double ny = -V1[2] * V2[0] + V1[0] * V2[2];
  const double nz = -V1[0] * V2[1] + V1[1] * V2[0];
  const double nVal = sqrt(nx * nx + ny * ny + nz * nz);
  n[0] = -nx / nVal; n[1] = -ny / nVal; n[2] = -nz / nVal;
}

// PerfectReflection, surfacemodel_tools.f90:81-256, without wall velocity or rotating frame: velocity and the
// rest of the trajectory mirrored at the point of intersection, which becomes LastPartPos
__device__ __forceinline__ void perfect_reflection(double v[3], double x[3], double xl[3], const double traj_in[3],
                                                   double len, double alpha, const double n[3]) {
  double poi[3], traj[3] = {traj_in[0], traj_in[1], traj_in[2]};
#pragma unroll
  for (int c = 0; c < 3; ++c) poi[c] = xl[c] + traj[c] * alpha;
  const double dv = v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
#pragma unroll
  for (int c = 0; c < 3; ++c) v[c] = v[c] - 2.0 * dv * n[c];
#pragma unroll
  for (int c = 0; c < 3; ++c) xl[c] = poi[c];
  const double dt = traj[0] * n[0] + traj[1] * n[1] + traj[2] * n[2];
#pragma unroll
  for (int c = 0; c < 3; ++c) traj[c] = traj[c] - 2.0 * dt * n[c];
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = xl[c] + traj[c] * (len - alpha);
}

// Walk from `elem` (= LastElem); updates x / xl at periodic crossings and x / xl / v at reflective walls.
// Returns the new element, -1 if the particle is lost, -2 if the hop cap was hit, -3 if it left through an
// open boundary (RemoveParticle; not a lost particle).
static __device__ __noinline__ int tria_track(const DevMesh& M, int elem, double x[3], double xl[3], double v[3]) {
  const Consts& kc = M.k;
  if (certainly_inside_f32(M, elem, x)) return elem;     // same decision as the FP64 test below
  int doneE[6] = {0, 0, 0, 0, 0, 0}, doneS[6] = {0, 0, 0, 0, 0, 0}, doneT[6] = {0, 0, 0, 0, 0, 0};
  // doneE/doneS/doneT hold DoneLastElem(1/4/3, 1:6) with 1-based element and side ids (0 = empty)
  for (int loop = 0; loop < kMaxTrackLoops; ++loop) {
    const double* X = M.xcl + (size_t)elem * 24;
    const uint32_t* sinfo = M.side_info + (size_t)elem * 6;
    double det[6][2];
    if (inside_quad3d(X, sinfo, x, det)) return elem;
    int nThrough = 0, locS[6], triT[6];
    int localSide = 0;
    double traj[3] = {x[0] - xl[0], x[1] - xl[1], x[2] - xl[2]};
    double len = sqrt(traj[0] * traj[0] + traj[1] * traj[1] + traj[2] * traj[2]);
    if (fabs(len) > 0.0) { traj[0] = traj[0] / len; traj[1] = traj[1] / len; traj[2] = traj[2] / len; }
    for (int s = 0; s < 6; ++s) {
      const uint32_t info = __ldg(sinfo + s);
      for (int tri = 1; tri <= 2; ++tri) {
        if (det[s][tri - 1] <= -0.0) {
          if (through_side(X, info, xl, traj, tri)) {
            if (nThrough < 6) { locS[nThrough] = s; triT[nThrough] = tri; }
            nThrough++;
            localSide = s;
          }
        }
      }
    }
    int triNum = triT[0];
    if (nThrough != 1) {
      if (nThrough == 0) return -1;
      int second = 0;
      double minRatio = 0.0;
      const int gElem = elem + 1;
      for (int ind2 = 0; ind2 < nThrough && ind2 < 6; ++ind2) {
        const int gSide = elem * 6 + locS[ind2] + 1;
        bool doCheck = true;
        for (int is = 1; is < 6; ++is)
          if (doneE[is] == gElem && doneS[is] == gSide && doneT[is] == triT[ind2]) doCheck = false;
        if (!doCheck) continue;
        double detM;
        if (last_pos_check(X, __ldg(sinfo + locS[ind2]), xl, triT[ind2], detM)) {
          double dPP = det[locS[ind2]][triT[ind2] - 1];
          if (detM == 0.0 && dPP == 0.0) continue;
          if (detM == 0.0 && minRatio == 0.0) {
            second++; localSide = locS[ind2]; triNum = triT[ind2];
          } else {
            if (detM == 0.0) continue;
            double ratio = dPP / detM;
            if (ratio < minRatio) { minRatio = ratio; second++; localSide = locS[ind2]; triNum = triT[ind2]; }
          }
        }
      }
      if (second == 0) return -1;
    }
    const uint32_t info = __ldg(sinfo + localSide);
    const int pvid = side_pvid(info);
    const int nb = __ldg(M.side_nb + (size_t)elem * 6 + localSide);
    // particle boundary of a wall side (particle_triatracking.f90:409-433, GetBoundaryInteraction
    // particle_boundary_condition.f90:35-221)
    const int wall = side_wall(info);
    if (wall == 1) return -3;
    if (wall == 2) {
      const double alpha = wall_alpha(X, info, xl, traj, triNum);
      double n[3];
      triangle_normal(X, info, triNum, n);
      perfect_reflection(v, x, xl, traj, len, alpha, n);
#pragma unroll
      for (int q = 0; q < 6; ++q) { doneE[q] = 0; doneS[q] = 0; doneT[q] = 0; }
      continue;
    }
#pragma unroll
    for (int q = 5; q >= 1; --q) { doneE[q] = doneE[q - 1]; doneS[q] = doneS[q - 1]; doneT[q] = doneT[q - 1]; }
    doneE[0] = elem + 1; doneS[0] = elem * 6 + localSide + 1; doneT[0] = triNum;
    if (pvid != 0) {
      // IntersectionWithWall + PeriodicBoundary, particle_boundary_condition.f90:224-284
      double alpha = wall_alpha(X, info, xl, traj, triNum);
      const int k = abs(pvid) - 1;
      const double sg = pvid > 0 ? 1.0 : -1.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) xl[c] = xl[c] + traj[c] * alpha;
#pragma unroll
      for (int c = 0; c < 3; ++c) xl[c] = xl[c] + copysign(kc.pv[3 * k + c], sg);
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c] = xl[c] + (len - alpha) * traj[c];
    }
    elem = nb;
  }
  return -2;
}

// ==========================================================================================
// RefTracking with CartesianPeriodic = FastPeriodic = T (particle_reftracking.f90:30-414, 697-985)
// ==========================================================================================
__device__ __forceinline__ void periodic_movement_fast(const Consts& kc, double x[3], double xl[3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int k = kc.pv_dir[d];
    if (k < 0) continue;
    const double* pv = kc.pv + 3 * k;
    if (x[d] > kc.xmax[d]) {
      double n = ceil(fabs(x[d] - kc.xmax[d]) / fabs(pv[d]));
      double mv[3] = {n * pv[0], n * pv[1], n * pv[2]};
      if (pv[d] > 0.0) { for (int c = 0; c < 3; ++c) { x[c] = x[c] - mv[c]; xl[c] = xl[c] - mv[c]; } }
      else { for (int c = 0; c < 3; ++c) { x[c] = x[c] + mv[c]; xl[c] = xl[c] + mv[c]; } }
    }
    if (x[d] < kc.xmin[d]) {
      double n = ceil(fabs(x[d] - kc.xmin[d]) / fabs(pv[d]));
      double mv[3] = {n * pv[0], n * pv[1], n * pv[2]};
      if (pv[d] > 0.0) { for (int c = 0; c < 3; ++c) { x[c] = x[c] + mv[c]; xl[c] = xl[c] + mv[c]; } }
      else { for (int c = 0; c < 3; ++c) { x[c] = x[c] - mv[c]; xl[c] = xl[c] - mv[c]; } }
    }
  }
}

__device__ __forceinline__ double maxabs3(const double v[3]) { return fmax(fabs(v[0]), fmax(fabs(v[1]), fabs(v[2]))); }
__device__ __forceinline__ bool almost_equal(double a, double b) { return fabs(a - b) <= fmax(fabs(a), fabs(b)) * 4.441e-16; }

constexpr int kMaxBgmCand = 64;

// ComputePlanarRectIntersection, particle_intersection.f90:515-684 (flip 0: wall sides are master sides);
// alpha or -1
__device__ __forceinline__ double planar_rect_alpha(const double* __restrict__ g, const double xl[3],
                                                    const double traj[3], double len) {
  const double n0 = g[9], n1 = g[10], n2 = g[11];
  const double coeffA = n0 * traj[0] + n1 * traj[1] + n2 * traj[2];
  if (fabs(coeffA) <= 2.22e-16) return -1.0;
  const double locSideDistance = g[12] - (xl[0] * n0 + xl[1] * n1 + xl[2] * n2);
  const double alpha = locSideDistance / coeffA;
  if (locSideDistance < -100.0 * kEpsMach) return -1.0;
  const double alphaNorm = alpha / len;
  if (alphaNorm > 1.0 || alphaNorm < -(100.0 * kEpsMach)) return -1.0;
  double P0[3], P1[3], P2[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double inter = xl[c] + alpha * traj[c];
    P0[c] = -0.25 * g[c] + inter;
    P1[c] = 0.25 * g[3 + c];
    P2[c] = 0.25 * g[6 + c];
  }
  const double A1 = P1[0] * P1[0] + P1[1] * P1[1] + P1[2] * P1[2];
  const double B1 = P2[0] * P1[0] + P2[1] * P1[1] + P2[2] * P1[2];
  const double C1 = P1[0] * P0[0] + P1[1] * P0[1] + P1[2] * P0[2];
  const double A2 = B1;
  const double B2 = P2[0] * P2[0] + P2[1] * P2[1] + P2[2] * P2[2];
  const double C2 = P2[0] * P0[0] + P2[1] * P0[1] + P2[2] * P0[2];
  double sdet = A1 * B2 - A2 * B1;
  if (fabs(sdet) == 0.0) return -1.0;
  sdet = 1.0 / sdet;
  const double epsLoc = 1.0 + 100.0 * kEpsMach;
  const double xi = (B2 * C1 - B1 * C2) * sdet;
  if (fabs(xi) > epsLoc) return -1.0;
  const double eta = (-A2 * C1 + A1 * C2) * sdet;
  if (fabs(eta) > epsLoc) return -1.0;
  return alpha;
}

// QuadraticSolver, utils.f90:401-465
__device__ __forceinline__ int quadratic_solver(double A, double B, double C, double& r1, double& r2) {
  r1 = 0.0;
  r2 = 0.0;
  if (A != 0.0 && B == 0.0 && C == 0.0) return 1;
  if (A != 0.0) {
    const double q = 0.5 * B / A, radicant = q * q - (C / A);
    if (radicant < 0.0) return 0;
    const double ba = B / A;
    r1 = -(0.5 * ba) - copysign(1.0, ba) * sqrt(radicant);
    r2 = (C / A) / r1;
    return 2;
  }
  if (B != 0.0) { r1 = -C / B; return 1; }
  return 0;
}

// ComputeBiLinearIntersection, particle_intersection.f90:855-1240 (RefTracking, wall side): eta from the
// quadratic of the trajectory-normal components, xi from ComputeXi (:2241-2273), t from
// ComputeSurfaceDistance2 (:2209-2238); of two hits the nearer; alpha2 > -1 drops a hit at alpha2.  Returns
// alpha or -1 with xi/eta of the hit; bad where the reference aborts (ComputeXi's HUGE).
static __device__ __noinline__ double bilinear_alpha(const double* __restrict__ g, const double xl[3], const double traj[3],
                                              double len, double alpha2, double& xi_out, double& eta_out, bool& bad) {
  double BLC[4][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    BLC[0][c] = 0.25 * __ldg(g + 16 + c);
    BLC[1][c] = 0.25 * __ldg(g + 3 + c);
    BLC[2][c] = 0.25 * __ldg(g + 6 + c);
    BLC[3][c] = 0.25 * __ldg(g + c);
  }
  const double scaleFac = traj[0] * __ldg(g + 9) + traj[1] * __ldg(g + 10) + traj[2] * __ldg(g + 11);
  if (fabs(scaleFac) < 100.0 * kEpsMach) return -1.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) BLC[3][c] = BLC[3][c] - xl[c];
  double A1[4], A2[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double d = (BLC[i][0] * traj[0] + BLC[i][1] * traj[1]) + BLC[i][2] * traj[2];
    const double n0 = BLC[i][0] - d * traj[0], n1 = BLC[i][1] - d * traj[1], n2 = BLC[i][2] - d * traj[2];
    A1[i] = n2 - n0;
    A2[i] = n2 - n1;
  }
  const double A = A1[0] * A2[2] - A2[0] * A1[2];
  const double B = ((A1[0] * A2[3] - A2[0] * A1[3]) + A1[1] * A2[2]) - A2[1] * A1[2];
  const double C = A1[1] * A2[3] - A2[1] * A1[3];
  double eta[2], xi[2] = {0.0, 0.0}, t[2] = {-1.0, -1.0};
  const int nRoot = quadratic_solver(A, B, C, eta[0], eta[1]);
  int inter = 0;
  for (int r = 0; r < nRoot; ++r) {
    if (!(fabs(eta[r]) <= 1.0)) continue;
    const double e = eta[r];
    const double a = e * A2[0] + A2[1];
    const double b = (e * (A2[0] - A1[0]) + A2[1]) - A1[1];
    if (fabs(b) >= fabs(a)) {
      if (fabs(b) <= 2.22e-16) { bad = true; return -1.0; }
      xi[r] = (-(e * (A2[2] - A1[2])) - (A2[3] - A1[3])) / b;
    } else {
      xi[r] = (-(e * A2[2]) - A2[3]) / a;
    }
    if (!(fabs(xi[r]) <= 1.0)) continue;
    double sv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) sv[c] = (((xi[r] * e) * BLC[0][c] + xi[r] * BLC[1][c]) + e * BLC[2][c]) + BLC[3][c];
    t[r] = (sv[0] * traj[0] + sv[1] * traj[1]) + sv[2] * traj[2];
    if (alpha2 > -1.0 && almost_equal(t[r], alpha2)) t[r] = -1.0;
    const double alphaNorm = t[r] / len;
    if (alphaNorm <= 1.0 && alphaNorm >= 0.0) inter |= 1 << r;
    if (nRoot == 1) break;
  }
  if (inter == 0) return -1.0;
  const int k = inter == 1 ? 0 : inter == 2 ? 1 : (t[0] < t[1] ? 0 : 1);
  xi_out = xi[k];
  eta_out = eta[k];
  return t[k];
}

// CalcNormAndTangBilinear, particle_surfaces.f90:404-440: unit d/dxi x d/deta at (xi, eta)
__device__ __forceinline__ void bilinear_normal(const double* __restrict__ g, double xi, double eta, double nv[3]) {
  double a[3], b[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double P00 = __ldg(g + 19 + c), P10 = __ldg(g + 22 + c), P01 = __ldg(g + 25 + c), P11 = __ldg(g + 28 + c);
    const double twist = ((P00 - P10) + P11) - P01;
    b[c] = (xi * 0.25) * twist + 0.25 * (((-P00 - P10) + P11) + P01);
    a[c] = (eta * 0.25) * twist + 0.25 * (((-P00 + P10) + P11) - P01);
  }
  const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  const double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) nv[c] = n[c] / l;
}

}  // namespace pic
#include "pic_bezier.cuh"
namespace pic {

// ParticleBCTracking, particle_reftracking.f90:417-694, for wall sides only (the element never changes).
// Returns true when the particle is done: it has not moved (PARTHASMOVED) or an open wall removed it.
static __device__ __noinline__ bool bc_tracking(const DevMesh& M, int& elem, double x[3], double xl[3], double v[3],
                                         bool& removed, double& len0, bool& cap_hit) {
  const Consts& kc = M.k;
  // each pass is one call of the reference's recursive ParticleBCTracking; a periodic crossing into another
  // element starts the next pass (the recursion is a tail call)
  for (int call = 0; call < 10000; ++call) {
    const int nl0 = __ldg(M.bc_e2b + 2 * elem);
    const int nloc = nl0 > 0 ? nl0 : 0, first = __ldg(M.bc_e2b + 2 * elem + 1);
    double traj[3] = {x[0] - xl[0], x[1] - xl[1], x[2] - xl[2]};
    double len = sqrt(traj[0] * traj[0] + traj[1] * traj[1] + traj[2] * traj[2]);
    if (fabs(len / __ldg(M.radius + elem)) <= 2.22e-16) return true;
#pragma unroll
    for (int c = 0; c < 3; ++c) traj[c] = traj[c] / len;
    len0 = fmax(len0, len);
    bool doubleCheck = false, moved_elem = false;
    double alphaOld = -1.0;
    for (int loop = 0; loop < 10000; ++loop) {
      double alpha[kBcCap], sxi[kBcCap], seta[kBcCap];
      int list[kBcCap];
      int nc = 0, nInter = 0;
      const double alpha2 = doubleCheck ? alphaOld : -1.0;
      for (int i = 0; i < nloc; ++i) {
        const double* g = M.bc_geo + (size_t)kBcGeo * (first + i);
        if (__ldg(g + 13) > len0) break;
        if (nc == kBcCap) { cap_hit = true; break; }
        const double type = __ldg(g + 15);
        sxi[nc] = 0.0;
        seta[nc] = 0.0;
        if (type == 0.0) {
          alpha[nc] = planar_rect_alpha(g, xl, traj, len);
        } else if (type >= 3.0) {
          // curved side: ComputeCurvedIntersection / ComputePlanarCurvedIntersection on its Bezier patch
          const double* S = M.bc_bz + (size_t)kBzGeo * (first + i);
          bool bad = false;
          if (type == 4.0) {
            alpha[nc] = bz_curved(kc.bz, S, xl, x, traj, len, sxi[nc], seta[nc], bad);
          } else {
            const double nv[3] = {__ldg(g + 9), __ldg(g + 10), __ldg(g + 11)};
            alpha[nc] = bz_planar_curved(kc.bz, S, nv, __ldg(g + 12), xl, traj, len, sxi[nc], seta[nc], bad);
          }
          if (bad) cap_hit = true;
        } else {
          double sxi, seta;
          bool bad = false;
          alpha[nc] = bilinear_alpha(g, xl, traj, len, alpha2, sxi, seta, bad);
          if (bad) cap_hit = true;
        }
        list[nc] = i;
        if (alpha[nc] > -1.0) nInter++;
        nc++;
      }
      if (nInter == 0) return false;
      for (int i = 1; i < nc; ++i) {                       // InsertionSort (stable)
        const double t = alpha[i], txi = sxi[i], teta = seta[i];
        const int ti = list[i];
        int j = i - 1;
        while (j >= 0 && !(alpha[j] <= t)) {
          alpha[j + 1] = alpha[j]; list[j + 1] = list[j]; sxi[j + 1] = sxi[j]; seta[j + 1] = seta[j];
          j--;
        }
        alpha[j + 1] = t;
        list[j + 1] = ti;
        sxi[j + 1] = txi;
        seta[j + 1] = teta;
      }
      for (int k = 0; k < nc; ++k)
        if (alpha[k] > -1.0) { alphaOld = alpha[k]; break; }
      bool reflected = false;
      for (int k = 0; k < nc; ++k) {
        if (!(alpha[k] > -1.0)) continue;
        const double* g = M.bc_geo + (size_t)kBcGeo * (first + list[k]);
        double n[3] = {__ldg(g + 9), __ldg(g + 10), __ldg(g + 11)};
        const double type = __ldg(g + 15);
        if (type == 2.0) {
          // the hit's xi/eta: the same call as above (xl, traj, len and alpha2 are unchanged until an interaction)
          double bxi = 0.0, beta = 0.0;
          bool bad = false;
          bilinear_alpha(g, xl, traj, len, alpha2, bxi, beta, bad);
          bilinear_normal(g, bxi, beta, n);
        } else if (type >= 3.0) {
          bz_normal(kc.bz, M.bc_bz + (size_t)kBzGeo * (first + list[k]), sxi[k], seta[k], n);   // CalcNormAndTangBezier
        }
        // GetBoundaryInteraction, REFMAPPING branch (particle_boundary_condition.f90:35-221)
        if (n[0] * traj[0] + n[1] * traj[1] + n[2] * traj[2] <= 0.0) { reflected = false; continue; }
        reflected = true;
        const double bc = __ldg(g + 14);
        if (bc == 1.0) { removed = true; break; }                    // RemoveParticle
        if (bc == 3.0) {
          // PeriodicBoundary (particle_boundary_condition.f90:224-284): LastPartPos at the crossing plus the
          // periodic vector, the particle at the rest of its trajectory, the trace goes on in the neighbour
          const double code = __ldg(g + 31);
          const int nb = (int)(code / 16.0);
          const int pvid = (int)(code - 16.0 * (double)nb) - 8;
          const int k3 = (pvid < 0 ? -pvid : pvid) - 1;
          const double sg = pvid < 0 ? -1.0 : 1.0;
#pragma unroll
          for (int c = 0; c < 3; ++c) xl[c] = xl[c] + traj[c] * alpha[k];
#pragma unroll
          for (int c = 0; c < 3; ++c) xl[c] = xl[c] + copysign(kc.pv[3 * k3 + c], sg);
#pragma unroll
          for (int c = 0; c < 3; ++c) x[c] = xl[c] + (len - alpha[k]) * traj[c];
          len = len - alpha[k];
          if (nb != elem) {
            // lengthPartTrajectory0 = the largest SideBCMetrics distance of the element left behind
            if (kc.n_pv > 0) {
              double mx = -1.7976931348623157e308;
              for (int i = 0; i < nloc; ++i) mx = fmax(mx, __ldg(M.bc_geo + (size_t)kBcGeo * (first + i) + 13));
              len0 = mx;
            }
            elem = nb;
            moved_elem = true;
          }
          break;
        }
        perfect_reflection(v, x, xl, traj, len, alpha[k], n);
#pragma unroll
        for (int c = 0; c < 3; ++c) traj[c] = x[c] - xl[c];
        len = sqrt(traj[0] * traj[0] + traj[1] * traj[1] + traj[2] * traj[2]);
        if (fabs(len) <= 2.22e-16) len = 0.0;
        else {
#pragma unroll
          for (int c = 0; c < 3; ++c) traj[c] = traj[c] / len;
        }
        break;
      }
      if (moved_elem) break;
      if (removed) return true;
      if (!reflected) {
        if (!doubleCheck) doubleCheck = true;
        else return false;
      }
    }
    if (!moved_elem) return false;
  }
  return false;
}

// Returns the new element (0-based); sets tol_fail when the reference would abort, removed when an open
// wall took the particle.  FAST selects the mixed variant's Newton (ref_elem_newton_fast).  v is only
// changed by reflective walls.
template <bool FAST>
__device__ __noinline__ int ref_track(const DevMesh& M, int last_elem, double x[3], double xl[3], double xi[3],
                                      double v[3], bool& tol_fail, bool& removed, bool& cap_hit) {
  const Consts& kc = M.k;
  tol_fail = false;
  removed = false;
  const bool bc_elem = M.bc_e2b && __ldg(M.bc_e2b + 2 * last_elem) > 0;
  int elem = last_elem;
  if (bc_elem) {
    // BC element (particle_reftracking.f90:98-126); a periodic crossing changes the element
    double len0 = 0.0;
    if (bc_tracking(M, elem, x, xl, v, removed, len0, cap_hit)) return elem;
    position_in_ref_elem_t<FAST>(M, elem, x, xi);
    if (maxabs3(xi) < 1.0) return elem;
  } else if (kc.n_pv > 0 && !kc.periodic_tracing) {
    double lp[3] = {x[0], x[1], x[2]};
    periodic_movement_fast(kc, x, xl);
    int guard = 0;
    while ((!almost_equal(lp[0], x[0]) || !almost_equal(lp[1], x[1]) || !almost_equal(lp[2], x[2])) && guard < 16) {
      lp[0] = x[0]; lp[1] = x[1]; lp[2] = x[2];
      periodic_movement_fast(kc, x, xl);
      guard++;
    }
  }
  if (!bc_elem) {
    position_in_ref_elem_t<FAST>(M, last_elem, x, xi);
    if (maxabs3(xi) < 1.0) return last_elem;
  }
  const int oldElem = last_elem;
  int cell[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int cc = (int)floor((x[d] - kc.xmin[d]) / kc.fib_delta[d]);
    cc = (cc > 0 ? cc : 0) + 1;
    cell[d] = cc < kc.fib_imax[d] ? cc : kc.fib_imax[d];
  }
  const size_t cidx = (size_t)(cell[0] - 1) + (size_t)kc.fib_imax[0] * ((cell[1] - 1) + (size_t)kc.fib_imax[1] * (cell[2] - 1));
  int nBGM = __ldg(M.fib_n + cidx);
  const int off = __ldg(M.fib_off + cidx);
  if (nBGM > kMaxBgmCand) nBGM = kMaxBgmCand;      // pic_create rejects FIBGM cells with more
  double dist[kMaxBgmCand];
  int list[kMaxBgmCand];
  if (nBGM > 1) {
    for (int i = 0; i < nBGM; ++i) {
      const int e = __ldg(M.fib_elem + off + i);
      list[i] = e;
      if (e == oldElem) {
        dist[i] = -1.7976931348623157e308;
      } else {
        double d0 = x[0] - __ldg(M.bary + 3 * e), d1 = x[1] - __ldg(M.bary + 3 * e + 1), d2 = x[2] - __ldg(M.bary + 3 * e + 2);
        dist[i] = (d0 * d0 + d1 * d1) + d2 * d2;
        double r = __ldg(M.radius + e);
        if (dist[i] > r * r) dist[i] = -1.7976931348623157e308;
      }
    }
    for (int i = 1; i < nBGM; ++i) {   // InsertionSort, utils.f90:52-101
      int j = i - 1;
      double tr = dist[i];
      int ti = list[i];
      while (j >= 0) {
        if (dist[j] <= tr) break;
        dist[j + 1] = dist[j]; list[j + 1] = list[j];
        j--;
      }
      dist[j + 1] = tr; list[j + 1] = ti;
    }
  } else if (nBGM == 1) {
    dist[0] = 0.0;
    list[0] = __ldg(M.fib_elem + off);
  }
  double oldXi[3] = {xi[0], xi[1], xi[2]};
  double newXi[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
  int newElem = -1;
  for (int i = 0; i < nBGM; ++i) {
    if (dist[i] == -1.7976931348623157e308) continue;
    const int e = list[i];
    position_in_ref_elem_t<FAST>(M, e, x, xi);
    if (maxabs3(xi) < 1.0) return e;
    if (maxabs3(xi) < maxabs3(newXi)) { newXi[0] = xi[0]; newXi[1] = xi[1]; newXi[2] = xi[2]; newElem = e; }
  }
  int te;
  if (maxabs3(oldXi) < maxabs3(newXi)) {
    xi[0] = oldXi[0]; xi[1] = oldXi[1]; xi[2] = oldXi[2];
    te = oldElem;
  } else {
    xi[0] = newXi[0]; xi[1] = newXi[1]; xi[2] = newXi[2];
    te = newElem;
  }
  if (te < 0 || maxabs3(xi) > __ldg(M.eps1 + te)) {
    if (te >= 0 && M.bc_e2b && __ldg(M.bc_e2b + 2 * te) > 0) {
      // BC element (particle_reftracking.f90:327-403): trace the BC sides again from TestElem (a periodic
      // crossing changes it; epsOneCell stays the one of the element the trace started in)
      double len0 = 0.0;
      const double eps_te = __ldg(M.eps1 + te);
      int tn = te;
      if (bc_tracking(M, tn, x, xl, v, removed, len0, cap_hit)) return tn;
      position_in_ref_elem_t<FAST>(M, tn, x, xi);
      // beyond epsOneCell the reference calls LocateParticleInElement and aborts when that fails
      if (maxabs3(xi) > eps_te) tol_fail = true;
      else te = tn;
    } else {
      tol_fail = true;
    }
  }
  return te < 0 ? oldElem : te;
}

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------------
// warp reduce-scatter: lane k ends with the warp sum of v[k] (k = node*4 + component)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double reduce_scatter32(double v[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool upper = (lane & h) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const double a = v[j], b = v[j + h];
      const double recv = __shfl_xor_sync(kFull, upper ? a : b, h);
      v[j] = (upper ? b : a) + recv;
    }
  }
  return v[0];
}

// Knuth TwoSum
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// compensated variant: (hi, lo) pairs, exact partial sums carried in lo
__device__ __forceinline__ double reduce_scatter32_ts(float hi[32], float lo[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool upper = (lane & h) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const float ah = hi[j], bh = hi[j + h], al = lo[j], bl = lo[j + h];
      const float rh = __shfl_xor_sync(kFull, upper ? ah : bh, h);
      const float rl = __shfl_xor_sync(kFull, upper ? al : bl, h);
      float s, e;
      two_sum(upper ? bh : ah, rh, s, e);
      hi[j] = s;
      lo[j] = __fadd_rn(__fadd_rn(upper ? bl : al, rl), e);
    }
  }
  return (double)hi[0] + (double)lo[0];
}

// Scatter one particle's 8 corner contributions (contrib[k], k = node*4+comp) to the
// periodic-unique node sums.  Called by all 32 lanes; lanes with active=false add nothing.
__device__ __forceinline__ void cvwm_scatter(const DevMesh& M, bool active, int e, double contrib[32], double* NS) {
  const int lane = threadIdx.x & 31;
  const unsigned act = __ballot_sync(kFull, active);
  if (act == 0) return;
  const int leader = __ffs(act) - 1;
  const int e0 = __shfl_sync(kFull, e, leader);
  const bool same = __all_sync(kFull, !active || e == e0);
  if (same) {
    if (!active) {
#pragma unroll
      for (int k = 0; k < 32; ++k) contrib[k] = 0.0;
    }
    const double s = reduce_scatter32(contrib);
    const int node = __ldg(M.canon_node + (size_t)e0 * 8 + (lane >> 2));
    atomicAdd(NS + (size_t)node * 4 + (lane & 3), s);
  } else if (active) {
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int node = __ldg(M.canon_node + (size_t)e * 8 + n);
#pragma unroll
      for (int c = 0; c < 4; ++c) atomicAdd(NS + (size_t)node * 4 + c, contrib[4 * n + c]);
    }
  }
}

__device__ __forceinline__ void cvwm_scatter_ts(const DevMesh& M, bool active, int e, float hi[32], double* NS) {
  const int lane = threadIdx.x & 31;
  const unsigned act = __ballot_sync(kFull, active);
  if (act == 0) return;
  const int leader = __ffs(act) - 1;
  const int e0 = __shfl_sync(kFull, e, leader);
  const bool same = __all_sync(kFull, !active || e == e0);
  if (same) {
    float lo[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) { lo[k] = 0.0f; if (!active) hi[k] = 0.0f; }
    const double s = reduce_scatter32_ts(hi, lo);
    const int node = __ldg(M.canon_node + (size_t)e0 * 8 + (lane >> 2));
    atomicAdd(NS + (size_t)node * 4 + (lane & 3), s);
  } else if (active) {
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int node = __ldg(M.canon_node + (size_t)e * 8 + n);
#pragma unroll
      for (int c = 0; c < 4; ++c) atomicAdd(NS + (size_t)node * 4 + c, (double)hi[4 * n + c]);
    }
  }
}

// CVWM corner weights of one particle (pic_depo_method.f90:479-539) in FP64, as contributions.
__device__ __forceinline__ void cvwm_contrib(const DevMesh& M, int e, bool suc, const double xi[3], const double x[3],
                                             const double TS[4], double out[32]) {
  double w[8];
  if (suc) {
    const double a1 = 0.5 * (xi[0] + 1.0), a2 = 0.5 * (xi[1] + 1.0), a3 = 0.5 * (xi[2] + 1.0);
    w[0] = (1 - a1) * (1 - a2) * (1 - a3);
    w[1] = (a1) * (1 - a2) * (1 - a3);
    w[2] = (a1) * (a2) * (1 - a3);
    w[3] = (1 - a1) * (a2) * (1 - a3);
    w[4] = (1 - a1) * (1 - a2) * (a3);
    w[5] = (a1) * (1 - a2) * (a3);
    w[6] = (a1) * (a2) * (a3);
    w[7] = (1 - a1) * (a2) * (a3);
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int c = 0; c < 4; ++c) out[4 * n + c] = TS[c] * w[n];
  } else {
    // inverse-distance weights to the corners (CGNS corner order)
    const double* X = M.xcl + (size_t)e * 24;
    const int cg2t[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    for (int n = 0; n < 8; ++n) w[n] = 0.0;
    for (int n = 0; n < 8; ++n) {
      const int t = cg2t[n];
      double v0 = __ldg(X + 3 * t) - x[0], v1 = __ldg(X + 3 * t + 1) - x[1], v2 = __ldg(X + 3 * t + 2) - x[2];
      double norm = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
      if (norm > 0.0) w[n] = 1.0 / norm;
      else { for (int q = 0; q < 8; ++q) w[q] = 0.0; w[n] = 1.0; break; }
    }
    double ds = 0.0;
    for (int n = 0; n < 8; ++n) ds = ds + w[n];
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int c = 0; c < 4; ++c) out[4 * n + c] = w[n] / ds * TS[c];
  }
}


// NodeSource / NodeVolume once per node (pic_depo_method.f90:684-690), in place, so that the DOF
// kernel below reads normalised sums instead of dividing 32 times per DOF (FP64 division is slow).
static __global__ void k_node_normalize(const double* __restrict__ node_vol, double* __restrict__ NS, int n_nodes) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_nodes * 4) return;
  const double V = __ldg(node_vol + t / 4);
  if (V > 0.0) NS[t] = NS[t] / V;
}

// Node sums -> DOFs (pic_depo_method.f90:692-733): PartSource(1:4,k,l,m) of every element.
// NORMALIZED: NS already holds NodeSource / NodeVolume (k_node_normalize ran first).
// N = 0 (p-adaption): threads cover (NMax+1)^3 DOFs per element; each element uses CellVolWeight(Nloc)%Fac
// (pic_depo_method.f90:714-720) and writes its (Nloc+1)^3 DOFs at its N_DG_Mapping offset.
template <int N, bool NORMALIZED = false>
__global__ void k_node_to_dof(const __grid_constant__ DevMesh M, const double* __restrict__ NS, double* __restrict__ PS) {
  const Consts& kc = M.k;
  const int nmax1 = N > 0 ? N + 1 : kc.N + 1, ndmax = nmax1 * nmax1 * nmax1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.ne * ndmax) return;
  const int e = t / ndmax, r = t - e * ndmax;
  const int nl = N > 0 ? N : __ldg(M.elem_n + e), n1 = nl + 1;
  if (r >= n1 * n1 * n1) return;
  const int kk = r % n1, ll = (r / n1) % n1, mm = r / (n1 * n1);
  const double a1 = kc.fac_n[nl][kk], a2 = kc.fac_n[nl][ll], a3 = kc.fac_n[nl][mm];
  double S[8][4];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int node = __ldg(M.canon_node + (size_t)e * 8 + n);
    if constexpr (NORMALIZED) {
#pragma unroll
      for (int c = 0; c < 4; ++c) S[n][c] = __ldg(NS + (size_t)node * 4 + c);
    } else {
      const double V = __ldg(M.node_vol + node);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double s = __ldg(NS + (size_t)node * 4 + c);
        S[n][c] = V > 0.0 ? s / V : s;
      }
    }
  }
  double out[4];
#pragma unroll
  for (int c = 0; c < 4; ++c)
    out[c] = S[0][c] * (1 - a1) * (1 - a2) * (1 - a3) + S[1][c] * (a1) * (1 - a2) * (1 - a3) +
             S[2][c] * (a1) * (a2) * (1 - a3) + S[3][c] * (1 - a1) * (a2) * (1 - a3) +
             S[4][c] * (1 - a1) * (1 - a2) * (a3) + S[5][c] * (a1) * (1 - a2) * (a3) +
             S[6][c] * (a1) * (a2) * (a3) + S[7][c] * (1 - a1) * (a2) * (a3);
  double2* o = reinterpret_cast<double2*>(PS + (N > 0 ? (size_t)t : dof_base<0>(M, e) + r) * 4);
  o[0] = make_double2(out[0], out[1]);
  o[1] = make_double2(out[2], out[3]);
}

}  // namespace pic
