// pic_adjoint.cu -- differentiable particle loop: reverse-mode adjoint of interpolation + Boris push
// + cell_volweight_mean deposition, with element ids replayed from the forward pass.
//
// Forward (field frozen, per step n = 0..nsteps-1, per particle):
//   xi_n = x -> xi Newton in elem_n (FP64, as the loop), E_n = sum U L L L (T), B = b_scale * B_ext,
//   v_{n+1/2} = Boris(v_{n-1/2}, E_n, B) (T), x_{n+1} = x_n + v_{n+1/2} dt (FP64),
//   elem_{n+1} = TriaTracking (FP64; integer result, replayed in the reverse pass).
// Then rho = CVWM deposition of x_N, loss = sum_DOF (rho/rho_scale - rho_target)^2.
// Reverse: dL/drho -> dL/d(node sums) -> dL/dx_N per particle -> per step the transposed Jacobians
// of x_{n+1} = x_n + v dt, the Boris map and the field interpolation E(x(xi)); dL/dB accumulates
// over particles and steps.  Checkpoints of (x, v, elem) every k steps; each segment is recomputed
// forward with its per-step states recorded, then reversed.
// T = double (FP64 reference gradient) or float (the FP32 adjoint); positions stay FP64.
#include "pic_ctx.h"

#include <vector>

using namespace pic;

namespace {

// Lagrange values and derivatives at x (product form), nodes kc.xgp[0..NP-1]
template <int NP, class T>
__device__ __forceinline__ void lagrange_d(const Consts& kc, T x, T L[NP], T dL[NP]) {
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    T l = T(1), d = T(0);
#pragma unroll
    for (int m = 0; m < NP; ++m) {
      if (m == i) continue;
      const T den = T(kc.xgp[i] - kc.xgp[m]);
      const T f = (x - T(kc.xgp[m])) / den;
      d = d * f + l / den;      // product rule, running
      l = l * f;
    }
    L[i] = l;
    dL[i] = d;
  }
}

// E(xi) and dE/dxi (3x3: [component][direction])
template <int N, class T>
__device__ __forceinline__ void field_and_grad(const Consts& kc, const T* __restrict__ U, const double xi[3], T E[3], T G[3][3]) {
  constexpr int n1 = N + 1;
  T L[3][n1], D[3][n1];
#pragma unroll
  for (int d = 0; d < 3; ++d) lagrange_d<n1, T>(kc, T(xi[d]), L[d], D[d]);
#pragma unroll
  for (int c = 0; c < 3; ++c) { E[c] = T(0); G[c][0] = G[c][1] = G[c][2] = T(0); }
  for (int k = 0; k < n1; ++k)
    for (int j = 0; j < n1; ++j)
#pragma unroll
      for (int i = 0; i < n1; ++i) {
        const T* u = U + ((k * n1 + j) * n1 + i) * 3;
        const T w = L[0][i] * L[1][j] * L[2][k];
        const T w0 = D[0][i] * L[1][j] * L[2][k], w1 = L[0][i] * D[1][j] * L[2][k], w2 = L[0][i] * L[1][j] * D[2][k];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T uc = __ldg(u + c);
          E[c] += uc * w;
          G[c][0] += uc * w0; G[c][1] += uc * w1; G[c][2] += uc * w2;
        }
      }
}

// J^{-T} applied to a vector: solves J^T y = b with J the trilinear map's Jacobian at xi (FP64)
__device__ __forceinline__ void jinvT(const DevMesh& M, int e, const double xi[3], const double b[3], double y[3]) {
  const double* DX = M.dxcl + (size_t)e * 72;
  const double l[3][2] = {{0.5 * (1.0 - xi[0]), 0.5 * (1.0 + xi[0])}, {0.5 * (1.0 - xi[1]), 0.5 * (1.0 + xi[1])},
                          {0.5 * (1.0 - xi[2]), 0.5 * (1.0 + xi[2])}};
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int t = 0; t < 8; ++t) {
    const double w = l[0][t & 1] * l[1][(t >> 1) & 1] * l[2][t >> 2];
    for (int nn = 0; nn < 3; ++nn)
      for (int dd = 0; dd < 3; ++dd) J[nn][dd] += __ldg(DX + 9 * t + 3 * nn + dd) * w;
  }
  // (J^T)^{-1} = (J^{-1})^T ; J^{-1} = adj(J)/det
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  const double c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1], c10 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0], c12 = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  const double c20 = J[1][0] * J[2][1] - J[1][1] * J[2][0], c21 = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  const double c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const double det = J[0][0] * c00 + J[0][1] * c10 + J[0][2] * c20;
  const double s = 1.0 / det;
  // Jinv[r][c] = c_rc * s ; y = Jinv^T b -> y[c] = sum_r Jinv[r][c] b[r]
  y[0] = (c00 * b[0] + c10 * b[1] + c20 * b[2]) * s;
  y[1] = (c01 * b[0] + c11 * b[1] + c21 * b[2]) * s;
  y[2] = (c02 * b[0] + c12 * b[1] + c22 * b[2]) * s;
}

template <class T>
struct BorisTape {
  T v[3], E[3], gamma, vm[3], gm, theta, tn, t[3], vp[3], f, vpl[3], vn1[3], den;
};

// relativistic Boris step (timedisc_TimeStepPoissonByBorisLeapfrog.f90:165-189), B = Bn * bhat
template <class T>
__device__ __forceinline__ void boris_fwd(BorisTape<T>& s, const T vin[3], const T E[3], T Bn, const T bh[3], T c1, T c2i) {
#pragma unroll
  for (int c = 0; c < 3; ++c) { s.v[c] = vin[c]; s.E[c] = E[c]; }
  const T vv = vin[0] * vin[0] + vin[1] * vin[1] + vin[2] * vin[2];
  s.gamma = T(1) / sqrt(T(1) - vv * c2i);
#pragma unroll
  for (int c = 0; c < 3; ++c) s.vm[c] = vin[c] * s.gamma + c1 * E[c];
  s.gm = sqrt(T(1) + (s.vm[0] * s.vm[0] + s.vm[1] * s.vm[1] + s.vm[2] * s.vm[2]) * c2i);
  s.theta = c1 / s.gm * Bn;
  s.tn = tan(s.theta);
#pragma unroll
  for (int c = 0; c < 3; ++c) s.t[c] = s.tn * bh[c];
  s.vp[0] = s.vm[0] + (s.vm[1] * s.t[2] - s.vm[2] * s.t[1]);
  s.vp[1] = s.vm[1] + (s.vm[2] * s.t[0] - s.vm[0] * s.t[2]);
  s.vp[2] = s.vm[2] + (s.vm[0] * s.t[1] - s.vm[1] * s.t[0]);
  s.f = T(2) / (T(1) + (s.t[0] * s.t[0] + s.t[1] * s.t[1] + s.t[2] * s.t[2]));
  s.vpl[0] = s.vm[0] + s.f * (s.vp[1] * s.t[2] - s.vp[2] * s.t[1]);
  s.vpl[1] = s.vm[1] + s.f * (s.vp[2] * s.t[0] - s.vp[0] * s.t[2]);
  s.vpl[2] = s.vm[2] + s.f * (s.vp[0] * s.t[1] - s.vp[1] * s.t[0]);
#pragma unroll
  for (int c = 0; c < 3; ++c) s.vn1[c] = s.vpl[c] + c1 * E[c];
  s.den = sqrt(T(1) + (s.vn1[0] * s.vn1[0] + s.vn1[1] * s.vn1[1] + s.vn1[2] * s.vn1[2]) * c2i);
}

__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1]; c[1] = a[2] * b[0] - a[0] * b[2]; c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ void cross3(const float* a, const float* b, float* c) {
  c[0] = a[1] * b[2] - a[2] * b[1]; c[1] = a[2] * b[0] - a[0] * b[2]; c[2] = a[0] * b[1] - a[1] * b[0];
}

// Reverse of boris_fwd: given dL/dv_out, return dL/dv_in, dL/dE, dL/dBn
template <class T>
__device__ __forceinline__ void boris_bwd(const BorisTape<T>& s, const T gout[3], const T bh[3], T c1, T c2i, T gv[3],
                                          T gE[3], T& gBn) {
  T gvn1[3], gvpl[3], gvm[3] = {0, 0, 0}, gvp[3], gt[3] = {0, 0, 0};
  // v_out = vn1 / den, den = sqrt(1 + |vn1|^2 c2i)
  T gden = T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) { gvn1[c] = gout[c] / s.den; gden -= gout[c] * s.vn1[c] / (s.den * s.den); }
#pragma unroll
  for (int c = 0; c < 3; ++c) gvn1[c] += gden * c2i / s.den * s.vn1[c];
  // vn1 = vpl + c1 E
#pragma unroll
  for (int c = 0; c < 3; ++c) { gvpl[c] = gvn1[c]; gE[c] = c1 * gvn1[c]; }
  // vpl = vm + f (vp x t)
  T cpt[3];
  cross3(s.vp, s.t, cpt);
  T gf = gvpl[0] * cpt[0] + gvpl[1] * cpt[1] + gvpl[2] * cpt[2];
  T cb[3] = {s.f * gvpl[0], s.f * gvpl[1], s.f * gvpl[2]};
  T tmp[3];
  cross3(s.t, cb, tmp);            // d/d(vp) of cb.(vp x t) = t x cb
#pragma unroll
  for (int c = 0; c < 3; ++c) { gvm[c] += gvpl[c]; gvp[c] = tmp[c]; }
  cross3(cb, s.vp, tmp);           // d/dt = cb x vp
#pragma unroll
  for (int c = 0; c < 3; ++c) gt[c] += tmp[c];
  // f = 2/(1+|t|^2)
#pragma unroll
  for (int c = 0; c < 3; ++c) gt[c] += -gf * s.f * s.f * s.t[c];
  // vp = vm + vm x t
#pragma unroll
  for (int c = 0; c < 3; ++c) gvm[c] += gvp[c];
  cross3(s.t, gvp, tmp);
#pragma unroll
  for (int c = 0; c < 3; ++c) gvm[c] += tmp[c];
  cross3(gvp, s.vm, tmp);
#pragma unroll
  for (int c = 0; c < 3; ++c) gt[c] += tmp[c];
  // t = tn * bh ; tn = tan(theta) ; theta = c1 Bn / gm
  const T gtn = gt[0] * bh[0] + gt[1] * bh[1] + gt[2] * bh[2];
  const T gth = gtn * (T(1) + s.tn * s.tn);
  gBn = gth * c1 / s.gm;
  const T ggm = -gth * s.theta / s.gm;
  // gm = sqrt(1 + |vm|^2 c2i)
#pragma unroll
  for (int c = 0; c < 3; ++c) gvm[c] += ggm * c2i / s.gm * s.vm[c];
  // vm = v gamma + c1 E
  T ggam = T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) { gv[c] = gvm[c] * s.gamma; ggam += gvm[c] * s.v[c]; gE[c] += c1 * gvm[c]; }
  // gamma = (1 - |v|^2 c2i)^(-1/2)
  const T g3 = s.gamma * s.gamma * s.gamma;
#pragma unroll
  for (int c = 0; c < 3; ++c) gv[c] += ggam * c2i * g3 * s.v[c];
}

struct AdjState {
  int n;
  double *x, *y, *z;       // current positions
  void *vx, *vy, *vz;      // T
  int* e;
  const uint8_t* sp;
};

template <class T>
struct Rec {
  double* x;     // [slot][3][n]
  T* v;          // [slot][3][n]
  int* e;        // [slot][n]
};

template <int N, class T, bool RECORD>
__global__ void __launch_bounds__(128) k_adj_fwd(const __grid_constant__ DevMesh M, AdjState S, const T* __restrict__ E, double dt, double b_scale,
                                                 Rec<T> R, int slot, DevStatus* st) {
  const Consts& kc = M.k;
  constexpr int n1 = N + 1, nd = n1 * n1 * n1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.n) return;
  double x[3] = {S.x[i], S.y[i], S.z[i]};
  T* vx = (T*)S.vx; T* vy = (T*)S.vy; T* vz = (T*)S.vz;
  T v[3] = {vx[i], vy[i], vz[i]};
  int e = S.e[i];
  const int sp = S.sp[i];
  if (RECORD) {
    const size_t o = (size_t)slot * 3 * S.n;
    R.x[o + i] = x[0]; R.x[o + S.n + i] = x[1]; R.x[o + 2 * (size_t)S.n + i] = x[2];
    R.v[o + i] = v[0]; R.v[o + S.n + i] = v[1]; R.v[o + 2 * (size_t)S.n + i] = v[2];
    R.e[(size_t)slot * S.n + i] = e;
  }
  double xi[3];
  position_in_ref_elem(M, e, x, xi);
  T Ef[3], G[3][3];
  field_and_grad<N, T>(kc, E + (size_t)e * nd * 3, xi, Ef, G);
#pragma unroll
  for (int c = 0; c < 3; ++c) Ef[c] += T(kc.ext[c]);
  const double Bx = kc.ext[3] * b_scale, By = kc.ext[4] * b_scale, Bz = kc.ext[5] * b_scale;
  const double Bn = sqrt(Bx * Bx + By * By + Bz * Bz);
  const T bh[3] = {T(Bn > 0 ? Bx / Bn : 0), T(Bn > 0 ? By / Bn : 0), T(Bn > 0 ? Bz / Bn : 0)};
  const T c1 = T(kc.q[sp] * dt / (kc.m[sp] * 2.0)), c2i = T(kc.c2_inv);
  BorisTape<T> tape;
  boris_fwd<T>(tape, v, Ef, T(Bn), bh, c1, c2i);
#pragma unroll
  for (int c = 0; c < 3; ++c) v[c] = tape.vn1[c] / tape.den;
  double xl[3] = {x[0], x[1], x[2]};
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = x[c] + (double)v[c] * dt;
  double vw[3] = {0.0, 0.0, 0.0};     // the adjoint runs on meshes without walls: no reflection
  int ne = tria_track(M, e, x, xl, vw);
  if (ne < 0) { flag_status(st, ne == -1 ? 0x01u : 0x04u); ne = e; }
  S.x[i] = x[0]; S.y[i] = x[1]; S.z[i] = x[2];
  vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
  S.e[i] = ne;
}

// CVWM charge only (component 4): node sums of q*MPF*w
template <class T>
__global__ void __launch_bounds__(128) k_adj_deposit(const __grid_constant__ DevMesh M, AdjState S, double* __restrict__ NS1) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.n) return;
  const double x[3] = {S.x[i], S.y[i], S.z[i]};
  const int e = S.e[i], sp = S.sp[i];
  double xi[3];
  position_in_ref_elem(M, e, x, xi);
  const T a[3] = {T(0.5 * (xi[0] + 1.0)), T(0.5 * (xi[1] + 1.0)), T(0.5 * (xi[2] + 1.0))};
  const T ch = T(kc.qm[sp]);
  const int cg2t[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  for (int c = 0; c < 8; ++c) {
    const int t = cg2t[c];
    const T w = ((t & 1) ? a[0] : T(1) - a[0]) * (((t >> 1) & 1) ? a[1] : T(1) - a[1]) * ((t >> 2) ? a[2] : T(1) - a[2]);
    atomicAdd(NS1 + __ldg(M.canon_node + (size_t)e * 8 + c), (double)(ch * w));
  }
}

// rho at the DOFs, loss, and dL/drho
__global__ void k_adj_loss(const __grid_constant__ DevMesh M, int nd, int n1, const double* __restrict__ NS1, const double* __restrict__ target,
                           double rho_scale, double* __restrict__ grho, double* __restrict__ loss) {
  const Consts& kc = M.k;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (tid < M.ne * nd) {
    const int e = tid / nd, r = tid - e * nd;
    const double a1 = kc.fac_gp[r % n1], a2 = kc.fac_gp[(r / n1) % n1], a3 = kc.fac_gp[r / (n1 * n1)];
    const double tri[8] = {(1 - a1) * (1 - a2) * (1 - a3), a1 * (1 - a2) * (1 - a3), a1 * a2 * (1 - a3), (1 - a1) * a2 * (1 - a3),
                           (1 - a1) * (1 - a2) * a3, a1 * (1 - a2) * a3, a1 * a2 * a3, (1 - a1) * a2 * a3};
    double rho = 0.0;
    for (int c = 0; c < 8; ++c) {
      const int node = __ldg(M.canon_node + (size_t)e * 8 + c);
      rho += NS1[node] / __ldg(M.node_vol + node) * tri[c];
    }
    const double d = rho / rho_scale - target[tid];
    l = d * d;
    grho[tid] = 2.0 * d / rho_scale;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

__global__ void k_adj_node_grad(const __grid_constant__ DevMesh M, int nd, int n1, const double* __restrict__ grho, double* __restrict__ gN) {
  const Consts& kc = M.k;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= M.ne * nd) return;
  const int e = tid / nd, r = tid - e * nd;
  const double a1 = kc.fac_gp[r % n1], a2 = kc.fac_gp[(r / n1) % n1], a3 = kc.fac_gp[r / (n1 * n1)];
  const double tri[8] = {(1 - a1) * (1 - a2) * (1 - a3), a1 * (1 - a2) * (1 - a3), a1 * a2 * (1 - a3), (1 - a1) * a2 * (1 - a3),
                         (1 - a1) * (1 - a2) * a3, a1 * (1 - a2) * a3, a1 * a2 * a3, (1 - a1) * a2 * a3};
  for (int c = 0; c < 8; ++c) {
    const int node = __ldg(M.canon_node + (size_t)e * 8 + c);
    atomicAdd(gN + node, grho[tid] * tri[c] / __ldg(M.node_vol + node));
  }
}

// dL/dx at the final positions from the CVWM weights
template <class T>
__global__ void __launch_bounds__(128) k_adj_deposit_bwd(const __grid_constant__ DevMesh M, AdjState S, const double* __restrict__ gN, T* gx,
                                                         T* gy, T* gz) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.n) return;
  const double x[3] = {S.x[i], S.y[i], S.z[i]};
  const int e = S.e[i], sp = S.sp[i];
  double xi[3];
  position_in_ref_elem(M, e, x, xi);
  const double a[3] = {0.5 * (xi[0] + 1.0), 0.5 * (xi[1] + 1.0), 0.5 * (xi[2] + 1.0)};
  const double ch = kc.qm[sp];
  const int cg2t[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  double gxi[3] = {0, 0, 0};
  for (int c = 0; c < 8; ++c) {
    const int t = cg2t[c];
    const int bx = t & 1, by = (t >> 1) & 1, bz = t >> 2;
    const double f0 = bx ? a[0] : 1.0 - a[0], f1 = by ? a[1] : 1.0 - a[1], f2 = bz ? a[2] : 1.0 - a[2];
    const double g = gN[__ldg(M.canon_node + (size_t)e * 8 + c)] * ch;
    gxi[0] += g * (bx ? 0.5 : -0.5) * f1 * f2;
    gxi[1] += g * f0 * (by ? 0.5 : -0.5) * f2;
    gxi[2] += g * f0 * f1 * (bz ? 0.5 : -0.5);
  }
  double gxx[3];
  jinvT(M, e, xi, gxi, gxx);
  gx[i] = T(gxx[0]); gy[i] = T(gxx[1]); gz[i] = T(gxx[2]);
}

// one reverse step: from (dL/dx_{n+1}, dL/dv_{n+1/2}) to (dL/dx_n, dL/dv_{n-1/2})
template <int N, class T>
__global__ void __launch_bounds__(128) k_adj_bwd(const __grid_constant__ DevMesh M, int n, const uint8_t* __restrict__ spv, const T* __restrict__ E,
                                                 double dt, double b_scale, Rec<T> R, int slot, T* gx, T* gy, T* gz,
                                                 T* gvx, T* gvy, T* gvz, double* gB) {
  const Consts& kc = M.k;
  constexpr int n1 = N + 1, nd = n1 * n1 * n1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double gBl = 0.0;
  if (i < n) {
    const size_t o = (size_t)slot * 3 * n;
    const double x[3] = {R.x[o + i], R.x[o + n + i], R.x[o + 2 * (size_t)n + i]};
    const T v[3] = {R.v[o + i], R.v[o + n + i], R.v[o + 2 * (size_t)n + i]};
    const int e = R.e[(size_t)slot * n + i];
    const int sp = spv[i];
    T lx[3] = {gx[i], gy[i], gz[i]};
    T lv[3] = {gvx[i], gvy[i], gvz[i]};
    // x_{n+1} = x_n + v_{n+1/2} dt
#pragma unroll
    for (int c = 0; c < 3; ++c) lv[c] += lx[c] * T(dt);
    double xi[3];
    position_in_ref_elem(M, e, x, xi);
    T Ef[3], G[3][3];
    field_and_grad<N, T>(kc, E + (size_t)e * nd * 3, xi, Ef, G);
#pragma unroll
    for (int c = 0; c < 3; ++c) Ef[c] += T(kc.ext[c]);
    const double Bx = kc.ext[3] * b_scale, By = kc.ext[4] * b_scale, Bz = kc.ext[5] * b_scale;
    const double Bn = sqrt(Bx * Bx + By * By + Bz * Bz);
    const T bh[3] = {T(Bn > 0 ? Bx / Bn : 0), T(Bn > 0 ? By / Bn : 0), T(Bn > 0 ? Bz / Bn : 0)};
    const T c1 = T(kc.q[sp] * dt / (kc.m[sp] * 2.0)), c2i = T(kc.c2_inv);
    BorisTape<T> tape;
    boris_fwd<T>(tape, v, Ef, T(Bn), bh, c1, c2i);
    T gv[3], gE[3], gBn;
    boris_bwd<T>(tape, lv, bh, c1, c2i, gv, gE, gBn);
    // E(x) = E(xi(x)): dL/dx += J^{-T} (dE/dxi)^T gE
    double gxi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) gxi[d] = (double)(G[0][d] * gE[0] + G[1][d] * gE[1] + G[2][d] * gE[2]);
    double gxe[3];
    jinvT(M, e, xi, gxi, gxe);
#pragma unroll
    for (int c = 0; c < 3; ++c) lx[c] += T(gxe[c]);
    gx[i] = lx[0]; gy[i] = lx[1]; gz[i] = lx[2];
    gvx[i] = gv[0]; gvy[i] = gv[1]; gvz[i] = gv[2];
    // dL/d|B| at fixed direction
    gBl = (double)gBn;
  }
  for (int o = 16; o > 0; o >>= 1) gBl += __shfl_xor_sync(0xffffffffu, gBl, o);
  if ((threadIdx.x & 31) == 0 && gBl != 0.0) atomicAdd(gB, gBl);
}

template <class TIn, class T>
__global__ void k_copy_cast(const TIn* __restrict__ a, T* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (T)a[i];
}

struct DevBuf {
  std::vector<void*> p;
  ~DevBuf() { for (void* q : p) cudaFree(q); }
  template <class X>
  bool get(X** out, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, (n ? n : 1) * sizeof(X)) != cudaSuccess) return false;
    p.push_back(q);
    *out = (X*)q;
    return true;
  }
};

template <int N, class T>
int run(pic_ctx_t* c, const pic_adjoint_cfg_t* a, const double* target_h, double* loss_h, double* gv_h, double* gB_h) {
  const int n = c->P.n, ne = c->ne, nd = c->nd, n1 = c->N + 1;
  const int K = a->checkpoint_every > 0 ? a->checkpoint_every : a->nsteps;
  const int nseg = a->nsteps > 0 ? (a->nsteps + K - 1) / K : 0;
  cudaStream_t s = c->stream;
  DevBuf B;
  double *x, *y, *z, *NS1, *grho, *gN, *loss, *gB, *target, *ck_x;
  T *vx, *vy, *vz, *E, *gx, *gy, *gz, *gvx, *gvy, *gvz, *ck_v;
  int *el, *ck_e;
  Rec<T> R{};
  const size_t nn = (size_t)std::max(n, 1);
  if (!B.get(&x, nn) || !B.get(&y, nn) || !B.get(&z, nn) || !B.get(&vx, nn) || !B.get(&vy, nn) || !B.get(&vz, nn) ||
      !B.get(&el, nn) || !B.get(&NS1, (size_t)c->n_canon) || !B.get(&grho, (size_t)ne * nd) || !B.get(&gN, (size_t)c->n_canon) ||
      !B.get(&loss, 1) || !B.get(&gB, 1) || !B.get(&target, (size_t)ne * nd) || !B.get(&E, (size_t)ne * nd * 3) ||
      !B.get(&gx, nn) || !B.get(&gy, nn) || !B.get(&gz, nn) || !B.get(&gvx, nn) || !B.get(&gvy, nn) || !B.get(&gvz, nn) ||
      !B.get(&ck_x, 3 * nn * (size_t)std::max(nseg, 1)) || !B.get(&ck_v, 3 * nn * (size_t)std::max(nseg, 1)) ||
      !B.get(&ck_e, nn * (size_t)std::max(nseg, 1)) || !B.get(&R.x, 3 * nn * (size_t)K) || !B.get(&R.v, 3 * nn * (size_t)K) ||
      !B.get(&R.e, nn * (size_t)K))
    return pic_internal::set_error(PIC_ERR_OUT_OF_MEMORY, "adjoint buffers");
  const int gb = (n + 127) / 128;
  const size_t bd = sizeof(double) * (size_t)n;
  cudaMemcpyAsync(x, c->P.x, bd, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(y, c->P.y, bd, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(z, c->P.z, bd, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(el, c->P.elem, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  if (n > 0) {
    if (c->mixed) {
      k_copy_cast<float, T><<<gb, 128, 0, s>>>(c->P.vxf, vx, n);
      k_copy_cast<float, T><<<gb, 128, 0, s>>>(c->P.vyf, vy, n);
      k_copy_cast<float, T><<<gb, 128, 0, s>>>(c->P.vzf, vz, n);
    } else {
      k_copy_cast<double, T><<<gb, 128, 0, s>>>(c->P.vx, vx, n);
      k_copy_cast<double, T><<<gb, 128, 0, s>>>(c->P.vy, vy, n);
      k_copy_cast<double, T><<<gb, 128, 0, s>>>(c->P.vz, vz, n);
    }
  }
  const size_t ftot = (size_t)ne * nd * 3;
  k_copy_cast<double, T><<<(unsigned)((ftot + 255) / 256), 256, 0, s>>>(c->E, E, (int)ftot);
  cudaMemcpyAsync(target, target_h, sizeof(double) * (size_t)ne * nd, cudaMemcpyHostToDevice, s);
  AdjState S{n, x, y, z, vx, vy, vz, el, c->P.species};
  auto save_ck = [&](int k) {
    cudaMemcpyAsync(ck_x + 3 * nn * k, x, bd, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(ck_x + 3 * nn * k + nn, y, bd, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(ck_x + 3 * nn * k + 2 * nn, z, bd, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(ck_v + 3 * nn * k, vx, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(ck_v + 3 * nn * k + nn, vy, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(ck_v + 3 * nn * k + 2 * nn, vz, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(ck_e + nn * k, el, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  };
  auto load_ck = [&](int k) {
    cudaMemcpyAsync(x, ck_x + 3 * nn * k, bd, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(y, ck_x + 3 * nn * k + nn, bd, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(z, ck_x + 3 * nn * k + 2 * nn, bd, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vx, ck_v + 3 * nn * k, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vy, ck_v + 3 * nn * k + nn, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vz, ck_v + 3 * nn * k + 2 * nn, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(el, ck_e + nn * k, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  };
  // ---- forward with checkpoints ---------------------------------------------------------------
  for (int it = 0; it < a->nsteps; ++it) {
    if (it % K == 0) save_ck(it / K);
    if (n > 0) k_adj_fwd<N, T, false><<<gb, 128, 0, s>>>(c->M, S, E, a->dt, a->b_scale, R, 0, c->st);
  }
  cudaMemsetAsync(NS1, 0, sizeof(double) * c->n_canon, s);
  cudaMemsetAsync(loss, 0, sizeof(double), s);
  if (n > 0) k_adj_deposit<T><<<gb, 128, 0, s>>>(c->M, S, NS1);
  const int gd = (ne * nd + 255) / 256;
  k_adj_loss<<<gd, 256, 0, s>>>(c->M, nd, n1, NS1, target, a->rho_scale, grho, loss);
  if (cudaMemcpyAsync(loss_h, loss, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return pic_internal::set_error(PIC_ERR_CUDA, std::string("adjoint forward: ") + cudaGetErrorString(cudaGetLastError()));
  if (!gv_h && !gB_h) return PIC_OK;
  // ---- reverse ---------------------------------------------------------------------------------
  cudaMemsetAsync(gN, 0, sizeof(double) * c->n_canon, s);
  cudaMemsetAsync(gB, 0, sizeof(double), s);
  k_adj_node_grad<<<gd, 256, 0, s>>>(c->M, nd, n1, grho, gN);
  if (n > 0) k_adj_deposit_bwd<T><<<gb, 128, 0, s>>>(c->M, S, gN, gx, gy, gz);
  cudaMemsetAsync(gvx, 0, sizeof(T) * n, s);
  cudaMemsetAsync(gvy, 0, sizeof(T) * n, s);
  cudaMemsetAsync(gvz, 0, sizeof(T) * n, s);
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * K, s1 = std::min(a->nsteps, s0 + K);
    load_ck(seg);
    for (int it = s0; it < s1; ++it)
      if (n > 0) k_adj_fwd<N, T, true><<<gb, 128, 0, s>>>(c->M, S, E, a->dt, a->b_scale, R, it - s0, c->st);
    for (int it = s1 - 1; it >= s0; --it)
      if (n > 0)
        k_adj_bwd<N, T><<<gb, 128, 0, s>>>(c->M, n, c->P.species, E, a->dt, a->b_scale, R, it - s0, gx, gy, gz, gvx, gvy,
                                           gvz, gB);
  }
  std::vector<T> hv(3 * nn);
  std::vector<int> pm(nn);
  cudaMemcpyAsync(hv.data(), gvx, sizeof(T) * n, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(hv.data() + nn, gvy, sizeof(T) * n, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(hv.data() + 2 * nn, gvz, sizeof(T) * n, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(pm.data(), c->perm, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, s);
  double gb_host = 0.0;
  cudaMemcpyAsync(&gb_host, gB, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t err = cudaStreamSynchronize(s);
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err != cudaSuccess) return pic_internal::set_error(PIC_ERR_CUDA, std::string("adjoint: ") + cudaGetErrorString(err));
  if (gv_h)
    for (int j = 0; j < n; ++j)
      for (int d = 0; d < 3; ++d) gv_h[(size_t)pm[j] * 3 + d] = (double)hv[d * nn + j];
  if (gB_h) *gB_h = gb_host;
  return PIC_OK;
}

}  // namespace

extern "C" int pic_adjoint_run(pic_ctx_t* c, const pic_adjoint_cfg_t* a, const double* rho_target, double* loss,
                               double* dL_dv0, double* dL_dB) {
  if (!c || !a || !rho_target || !loss) return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (c->cfg.deposition != PIC_DEPO_CVWM || c->cfg.tracking != PIC_TRACK_TRIA)
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "the adjoint loop needs cell_volweight_mean + TriaTracking");
  if (a->nsteps < 0 || a->checkpoint_every < 0 || !(a->rho_scale != 0.0) || !(a->dt > 0.0) || !(a->b_scale > 0.0))
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "adjoint configuration");
  if (a->precision != PIC_PREC_FP64 && a->precision != PIC_PREC_MIXED)
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "adjoint precision");
  if (c->has_walls)
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "the adjoint loop needs a mesh without open/reflective sides");
  if (c->var_n)
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "the adjoint loop needs one polynomial degree for all elements");
  if (c->M.xcl_ng)
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "the adjoint loop needs NGeo = 1 (trilinear elements)");
  for (int s = 0; s < c->cfg.n_species; ++s)
    if (c->M.k.dt_fac[s] != 1.0)
      return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "the adjoint loop needs one time step for all species");
  if (!c->field_set || !c->have_particles) return pic_internal::set_error(PIC_ERR_STATE, "field and particles must be set first");
  const bool f32 = a->precision == PIC_PREC_MIXED;
  switch (c->N) {
    case 1: return f32 ? run<1, float>(c, a, rho_target, loss, dL_dv0, dL_dB) : run<1, double>(c, a, rho_target, loss, dL_dv0, dL_dB);
    case 2: return f32 ? run<2, float>(c, a, rho_target, loss, dL_dv0, dL_dB) : run<2, double>(c, a, rho_target, loss, dL_dv0, dL_dB);
    case 3: return f32 ? run<3, float>(c, a, rho_target, loss, dL_dv0, dL_dB) : run<3, double>(c, a, rho_target, loss, dL_dv0, dL_dB);
    default: return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "adjoint supports N = 1..3");
  }
}
