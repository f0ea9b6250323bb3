// pic_kernels.cu -- sm_103a kernels of the Boris-Leapfrog PIC particle loop.
//
// Layout: particles in SoA (x,y,z / vx,vy,vz / elem / flags), kept grouped by element by a
// counting sort so that a warp mostly works on one element: its corner nodes, DOFs and field
// stay in L1, and CVWM charge is reduced across the warp before the global atomics.
#include "pic_kernels.cuh"

#include <cstdio>
#include <cuda_fp16.h>

namespace pic {




// ---------------------------------------------------------------------------------------------
// Mixed-precision (FP32) mapping on linear, uncurved elements: Newton in element-local
// coordinates relative to the barycentre.  Only used with TriaTracking meshes.
// ---------------------------------------------------------------------------------------------


// RefMappingGuess 1 in FP32; the other guesses take the FP64 start value of x (newton_start)
__device__ __forceinline__ bool position_in_ref_elem_f(const DevMesh& M, const MeshF& F, int e, const double x[3],
                                                       const float p[3], float xi[3]) {
  const Consts& kc = M.k;
  if (elem_curved(M, e)) {        // NGeo > 1: the FP64 Newton on the NGeo map (power form)
    double xd[3];
    const bool suc = position_in_ref_elem_t<true>(M, e, x, xd);
    xi[0] = (float)xd[0]; xi[1] = (float)xd[1]; xi[2] = (float)xd[2];
    return suc;
  }
  if (kc.ref_guess != 1) {
    double xs[3];
    newton_start(M, e, x, xs);
    xi[0] = (float)xs[0]; xi[1] = (float)xs[1]; xi[2] = (float)xs[2];
  } else {
    const float* B = F.xez + (size_t)e * 18;
    const float* S = F.slen + (size_t)e * 6;
    float xil[6];
#pragma unroll
    for (int d = 0; d < 6; ++d)
      xil[d] = fmaf(p[0], __ldg(B + 3 * d), fmaf(p[1], __ldg(B + 3 * d + 1), p[2] * __ldg(B + 3 * d + 2))) * __ldg(S + d);
#pragma unroll
    for (int d = 0; d < 3; ++d) xi[d] = 0.5f * (xil[d] - xil[d + 3]);
    const float epsOne = 1.0f + (float)kc.refmapping_eps;
    if (fmaxf(fabsf(xi[0]), fmaxf(fabsf(xi[1]), fabsf(xi[2]))) > epsOne) {
#pragma unroll
      for (int d = 0; d < 3; ++d) xi[d] = fmaxf(fminf(1.0f, xi[d]), -1.0f);
    }
  }
  const float* X = F.xclr + (size_t)e * 24;
  const float* DX = F.dxcl + (size_t)e * 72;
  bool success = true;
  float deltaXi2 = 1.0f;
  for (int iter = 0; iter < 100 && deltaXi2 > (float)kc.refmapping_eps; ++iter) {
    float l[3][2];
#pragma unroll
    for (int d = 0; d < 3; ++d) { l[d][0] = 0.5f * (1.0f - xi[d]); l[d][1] = 0.5f * (1.0f + xi[d]); }
    float Fr[3] = {-p[0], -p[1], -p[2]}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const float w = l[0][t & 1] * l[1][(t >> 1) & 1] * l[2][t >> 2];
#pragma unroll
      for (int c = 0; c < 3; ++c) Fr[c] = fmaf(__ldg(X + 3 * t + c), w, Fr[c]);
#pragma unroll
      for (int nn = 0; nn < 3; ++nn)
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) J[nn][dd] = fmaf(__ldg(DX + 9 * t + 3 * nn + dd), w, J[nn][dd]);
    }
    float det = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * J[2][2] + (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * J[2][0] +
                (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * J[2][1];
    const float sd = 1.0f / det;
    float dxi[3];
    dxi[0] = ((J[1][1] * J[2][2] - J[1][2] * J[2][1]) * Fr[0] + (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * Fr[1] +
              (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * Fr[2]) * sd;
    dxi[1] = ((J[1][2] * J[2][0] - J[1][0] * J[2][2]) * Fr[0] + (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * Fr[1] +
              (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * Fr[2]) * sd;
    dxi[2] = ((J[1][0] * J[2][1] - J[1][1] * J[2][0]) * Fr[0] + (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * Fr[1] +
              (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * Fr[2]) * sd;
    deltaXi2 = dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2];
#pragma unroll
    for (int d = 0; d < 3; ++d) xi[d] -= dxi[d];
    if (fabsf(xi[0]) > 1.5f || fabsf(xi[1]) > 1.5f || fabsf(xi[2]) > 1.5f) { success = false; break; }
  }
  return success;
}

template <int N>
__device__ __forceinline__ void eval_field_f(const Consts& kc, const float* __restrict__ U, const float xi[3], float out[3]) {
  constexpr int n1 = N + 1;
  float L[3][n1];
#pragma unroll
  for (int d = 0; d < 3; ++d) lagrange_f<n1>(xi[d], kc.xgp_nf[N], kc.wbary_nf[N], L[d]);
  out[0] = out[1] = out[2] = 0.0f;
#pragma unroll
  for (int k = 0; k < n1; ++k)
#pragma unroll
    for (int j = 0; j < n1; ++j) {
      const float Lez = L[1][j] * L[2][k];
#pragma unroll
      for (int i = 0; i < n1; ++i) {
        const float* u = U + ((k * n1 + j) * n1 + i) * 3;
        const float w = L[0][i] * Lez;
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c] = fmaf(__ldg(u + c), w, out[c]);
      }
    }
}

// FP32 field of element e at xi (mixed variant); N = 0 dispatches on the element's degree (p-adaption)
template <int N>
__device__ __forceinline__ void field_at_f(const DevMesh& M, const float* __restrict__ E32, int e, const float xi[3],
                                           float out[3]) {
  if constexpr (N > 0) {
    eval_field_f<N>(M.k, E32 + (size_t)e * ((N + 1) * (N + 1) * (N + 1)) * 3, xi, out);
  } else {
    const float* U = E32 + (size_t)__ldg(M.dof_off + e) * 3;
    switch (__ldg(M.elem_n + e)) {
      case 1: eval_field_f<1>(M.k, U, xi, out); break;
      case 2: eval_field_f<2>(M.k, U, xi, out); break;
      case 3: eval_field_f<3>(M.k, U, xi, out); break;
      default: eval_field_f<4>(M.k, U, xi, out); break;
    }
  }
}

// FP32 Boris push (mixed variant)
__device__ __forceinline__ void boris_push_f(const Consts& kc, float v[3], const float F[6], int sp, bool& is_new, float dt) {
  const float q = (float)kc.q[sp], qmt = (float)(kc.q[sp] / kc.m[sp]);
  const bool push = fabsf(q) > 0.0f;
  if (is_new) {
    if (push) {
#pragma unroll
      for (int c = 0; c < 3; ++c) v[c] = fmaf(-F[c] * qmt, dt * 0.5f, v[c]);
    }
    is_new = false;
  }
  if (!push) return;
  const float c2i = (float)kc.c2_inv;
  const float c1 = 0.5f * qmt * dt;
  const float vv = fmaf(v[0], v[0], fmaf(v[1], v[1], v[2] * v[2]));
  const float gamma = rsqrtf(1.0f - vv * c2i);
  float vm[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) vm[c] = fmaf(v[c], gamma, c1 * F[c]);
  const float gm = sqrtf(fmaf(fmaf(vm[0], vm[0], fmaf(vm[1], vm[1], vm[2] * vm[2])), c2i, 1.0f));
  const float Bn = sqrtf(fmaf(F[3], F[3], fmaf(F[4], F[4], F[5] * F[5])));
  float t[3] = {0.0f, 0.0f, 0.0f};
  if (Bn > 0.0f) {
    const float s = tanf(c1 / gm * Bn) / Bn;
#pragma unroll
    for (int c = 0; c < 3; ++c) t[c] = s * F[3 + c];
  }
  const float vp[3] = {vm[0] + (vm[1] * t[2] - vm[2] * t[1]), vm[1] + (vm[2] * t[0] - vm[0] * t[2]),
                       vm[2] + (vm[0] * t[1] - vm[1] * t[0])};
  const float fac = 2.0f / (1.0f + fmaf(t[0], t[0], fmaf(t[1], t[1], t[2] * t[2])));
  float vn[3];
  vn[0] = fmaf(fac, vp[1] * t[2] - vp[2] * t[1], vm[0]) + c1 * F[0];
  vn[1] = fmaf(fac, vp[2] * t[0] - vp[0] * t[2], vm[1]) + c1 * F[1];
  vn[2] = fmaf(fac, vp[0] * t[1] - vp[1] * t[0], vm[2]) + c1 * F[2];
  const float inv = rsqrtf(fmaf(fmaf(vn[0], vn[0], fmaf(vn[1], vn[1], vn[2] * vn[2])), c2i, 1.0f));
#pragma unroll
  for (int c = 0; c < 3; ++c) v[c] = vn[c] * inv;
}

// =============================================================================================
// Fused step for cell_volweight_mean + TriaTracking
// =============================================================================================
// resident CTAs per SM the mixed variant is compiled for (register cap 65536 / (256 x this))
#ifndef PIC_CVWM_MIXED_MINB
#define PIC_CVWM_MIXED_MINB 4   // 4 x 256 threads: 64 registers, a few spills; 1.13x faster than 2 CTAs/SM
#endif
#ifndef PIC_CVWM_MINB
#define PIC_CVWM_MINB 1         // FP64 variant
#endif
template <int N, bool MIXED>
__global__ void __launch_bounds__(256, MIXED ? PIC_CVWM_MIXED_MINB : PIC_CVWM_MINB) k_step_cvwm_tria(const __grid_constant__ DevMesh M, MeshF MF, DevParticles P, const double* __restrict__ E,
                                                        const float* __restrict__ E32, double* __restrict__ NS,
                                                        double dt, DevStatus* st) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in_range = i < P.n;
  const uint8_t fl = in_range ? P.flags[i] : 0;
  const bool inside = (fl & kInside) != 0;
  const int sp = inside ? P.species[i] : 0;
  const bool charged = inside && (kc.q[sp] != 0.0);
  int e = inside ? P.elem[i] : 0;
  double x[3] = {0.0, 0.0, 0.0};
  if (inside) { x[0] = P.x[i]; x[1] = P.y[i]; x[2] = P.z[i]; }

  // ---- Deposition (CVWM) and interpolation share one x -> xi mapping ------------------------
  double Fd[6];
  float Ff[6];
  if constexpr (!MIXED) {
    double v[3] = {0.0, 0.0, 0.0};
    if (inside) { v[0] = P.vx[i]; v[1] = P.vy[i]; v[2] = P.vz[i]; }
    double xi[3] = {0.0, 0.0, 0.0};
    bool suc = true;
    if (charged) {
      suc = position_in_ref_elem(M, e, x, xi);
      if (!suc) { atomicAdd(&st->n_newton_failed, 1); flag_status(st, 0x02u); }
    }
    {
      double contrib[32];
      if (charged) {
        const double ch = kc.qm[sp];
        const double TS[4] = {v[0] * ch, v[1] * ch, v[2] * ch, ch};
        cvwm_contrib(M, e, suc, xi, x, TS, contrib);
      }
      cvwm_scatter(M, charged, e, contrib, NS);
    }
    if (!inside) return;
#pragma unroll
    for (int c = 0; c < 6; ++c) Fd[c] = kc.ext[c];
    if (charged) {
      double Eo[3];
      if (suc) field_at<N>(M, E, e, xi, Eo);
      else field_dw_at<N>(M, E, e, x, Eo);
#pragma unroll
      for (int c = 0; c < 3; ++c) Fd[c] = Fd[c] + Eo[c];
#pragma unroll
      for (int c = 3; c < 6; ++c) Fd[c] = Fd[c] + 0.0;
    }
    bool isnew = (fl & kNew) != 0;
    const double dtv = dt * kc.dt_fac[sp];
    boris_push(kc, v, Fd, sp, isnew, dtv);
    double xl[3] = {x[0], x[1], x[2]};
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = x[c] + v[c] * dtv;
    if (!state_finite(x, v[0], v[1], v[2])) {
      flag_status(st, 0x20u);
      P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2];
      P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
      P.flags[i] = (isnew ? (fl | kNew) : (fl & ~kNew)) & ~kInside;
      return;
    }
    int ne = tria_track(M, e, x, xl, v);
    P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2];
    uint8_t nf = isnew ? (fl | kNew) : (fl & ~kNew);
    if (ne < 0) {
      nf &= ~kInside;
      if (ne == -1) { atomicAdd(&st->n_lost, 1); flag_status(st, 0x01u); }
      else if (ne == -2) flag_status(st, 0x04u);
      ne = e;
    }
    P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
    P.elem[i] = ne;
    P.flags[i] = nf;
  } else {
    float v[3] = {0.0f, 0.0f, 0.0f};
    if (inside) { v[0] = P.vxf[i]; v[1] = P.vyf[i]; v[2] = P.vzf[i]; }
    float xi[3] = {0.0f, 0.0f, 0.0f};
    bool suc = true;
    if (charged) {
      const double* b = M.bary + (size_t)e * 3;
      const float p[3] = {(float)(x[0] - __ldg(b)), (float)(x[1] - __ldg(b + 1)), (float)(x[2] - __ldg(b + 2))};
      suc = position_in_ref_elem_f(M, MF, e, x, p, xi);
      if (!suc) {
        // fall back to the FP64 mapping so that the inverse-distance branch matches the reference's
        double xd[3];
        suc = position_in_ref_elem(M, e, x, xd);
        xi[0] = (float)xd[0]; xi[1] = (float)xd[1]; xi[2] = (float)xd[2];
        if (!suc) { atomicAdd(&st->n_newton_failed, 1); flag_status(st, 0x02u); }
      }
    }
    {
      float hi[32];
      if (charged) {
        const float ch = (float)kc.qm[sp];
        const float TS[4] = {v[0] * ch, v[1] * ch, v[2] * ch, ch};
        if (suc) {
          const float a1 = 0.5f * (xi[0] + 1.0f), a2 = 0.5f * (xi[1] + 1.0f), a3 = 0.5f * (xi[2] + 1.0f);
          const float b1 = 1.0f - a1, b2 = 1.0f - a2, b3 = 1.0f - a3;
          const float w[8] = {b1 * b2 * b3, a1 * b2 * b3, a1 * a2 * b3, b1 * a2 * b3,
                              b1 * b2 * a3, a1 * b2 * a3, a1 * a2 * a3, b1 * a2 * a3};
#pragma unroll
          for (int n = 0; n < 8; ++n)
#pragma unroll
            for (int c = 0; c < 4; ++c) hi[4 * n + c] = TS[c] * w[n];
        } else {
          double TSd[4] = {(double)TS[0], (double)TS[1], (double)TS[2], (double)TS[3]};
          double xd[3] = {0, 0, 0}, cd[32];
          cvwm_contrib(M, e, false, xd, x, TSd, cd);
#pragma unroll
          for (int k = 0; k < 32; ++k) hi[k] = (float)cd[k];
        }
      }
      cvwm_scatter_ts(M, charged, e, hi, NS);
    }
    if (!inside) return;
#pragma unroll
    for (int c = 0; c < 6; ++c) Ff[c] = (float)kc.ext[c];
    if (charged) {
      float Eo[3];
      if (suc) {
        field_at_f<N>(M, E32, e, xi, Eo);
      } else {
        double Ed[3];
        field_dw_at<N>(M, E, e, x, Ed);
        Eo[0] = (float)Ed[0]; Eo[1] = (float)Ed[1]; Eo[2] = (float)Ed[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) Ff[c] += Eo[c];
    }
    bool isnew = (fl & kNew) != 0;
    const double dtv = dt * kc.dt_fac[sp];
    boris_push_f(kc, v, Ff, sp, isnew, (float)dtv);
    double xl[3] = {x[0], x[1], x[2]};
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = x[c] + (double)v[c] * dtv;
    if (!state_finite(x, v[0], v[1], v[2])) {
      flag_status(st, 0x20u);
      P.vxf[i] = v[0]; P.vyf[i] = v[1]; P.vzf[i] = v[2];
      P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
      P.flags[i] = (isnew ? (fl | kNew) : (fl & ~kNew)) & ~kInside;
      return;
    }
    double vd[3] = {(double)v[0], (double)v[1], (double)v[2]};   // reflective walls mirror it in FP64
    int ne = tria_track(M, e, x, xl, vd);
    P.vxf[i] = (float)vd[0]; P.vyf[i] = (float)vd[1]; P.vzf[i] = (float)vd[2];
    uint8_t nf = isnew ? (fl | kNew) : (fl & ~kNew);
    if (ne < 0) {
      nf &= ~kInside;
      if (ne == -1) { atomicAdd(&st->n_lost, 1); flag_status(st, 0x01u); }
      else if (ne == -2) flag_status(st, 0x04u);
      ne = e;
    }
    P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
    P.elem[i] = ne;
    P.flags[i] = nf;
  }
}

// =============================================================================================
// Separate loop pieces (the reference's individual routines)
// =============================================================================================
template <int N, bool MIXED>
__global__ void __launch_bounds__(256) k_interpolate(const __grid_constant__ DevMesh M, MeshF MF, DevParticles P, const double* __restrict__ E,
                                                     const float* __restrict__ E32, DevStatus* st, bool refmap,
                                                     bool cvwm) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = P.flags[i];
  if (!(fl & kInside)) return;
  const int sp = P.species[i];
  if (kc.q[sp] == 0.0) return;   // isInterpolateParticle
  const int e = P.elem[i];
  const double x[3] = {P.x[i], P.y[i], P.z[i]};
  double F[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) F[c] = kc.ext[c];
  double Eo[3];
  if constexpr (!MIXED) {
    double xi[3];
    bool suc = true;
    if (!refmap) {
      suc = position_in_ref_elem(M, e, x, xi);
      if (!suc) { atomicAdd(&st->n_newton_failed, 1); flag_status(st, 0x02u); }
    } else {
      xi[0] = P.xi0[i]; xi[1] = P.xi1[i]; xi[2] = P.xi2[i];
    }
    if (!suc && cvwm) field_dw_at<N>(M, E, e, x, Eo);
    else field_at<N>(M, E, e, xi, Eo);
  } else {
    float xi[3];
    bool suc = true;
    if (!refmap) {
      const double* b = M.bary + (size_t)e * 3;
      const float p[3] = {(float)(x[0] - __ldg(b)), (float)(x[1] - __ldg(b + 1)), (float)(x[2] - __ldg(b + 2))};
      suc = position_in_ref_elem_f(M, MF, e, x, p, xi);
      if (!suc) {
        double xd[3];
        suc = position_in_ref_elem(M, e, x, xd);
        xi[0] = (float)xd[0]; xi[1] = (float)xd[1]; xi[2] = (float)xd[2];
        if (!suc) { atomicAdd(&st->n_newton_failed, 1); flag_status(st, 0x02u); }
      }
    } else {
      xi[0] = (float)P.xi0[i]; xi[1] = (float)P.xi1[i]; xi[2] = (float)P.xi2[i];
    }
    if (!suc && cvwm) {
      field_dw_at<N>(M, E, e, x, Eo);
    } else {
      float Ef[3];
      field_at_f<N>(M, E32, e, xi, Ef);
      Eo[0] = Ef[0]; Eo[1] = Ef[1]; Eo[2] = Ef[2];
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) F[c] = F[c] + Eo[c];
#pragma unroll
  for (int c = 0; c < 6; ++c) P.field[(size_t)c * P.cap + i] = F[c];
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_push(const __grid_constant__ Consts kc, DevParticles P, double dt, DevStatus* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = P.flags[i];
  if (!(fl & kInside)) return;
  const int sp = P.species[i];
  double x[3] = {P.x[i], P.y[i], P.z[i]};
  P.lx[i] = x[0]; P.ly[i] = x[1]; P.lz[i] = x[2];      // LastPartPos (timedisc...:109-110)
  P.last_elem[i] = P.elem[i];
  bool isnew = (fl & kNew) != 0;
  bool finite;
  if constexpr (!MIXED) {
    double F[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) F[c] = P.field[(size_t)c * P.cap + i];
    double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
    const double dtv = dt * kc.dt_fac[sp];
    boris_push(kc, v, F, sp, isnew, dtv);
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = x[c] + v[c] * dtv;
    P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2];
    finite = state_finite(x, v[0], v[1], v[2]);
  } else {
    float F[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) F[c] = (float)P.field[(size_t)c * P.cap + i];
    float v[3] = {P.vxf[i], P.vyf[i], P.vzf[i]};
    const double dtv = dt * kc.dt_fac[sp];
    boris_push_f(kc, v, F, sp, isnew, (float)dtv);
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = x[c] + (double)v[c] * dtv;
    P.vxf[i] = v[0]; P.vyf[i] = v[1]; P.vzf[i] = v[2];
    finite = state_finite(x, v[0], v[1], v[2]);
  }
  P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
  uint8_t nf = isnew ? (fl | kNew) : (fl & ~kNew);
  if (!finite) { flag_status(st, 0x20u); nf &= ~kInside; }
  P.flags[i] = nf;
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_track_tria(const __grid_constant__ DevMesh M, DevParticles P, DevStatus* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = P.flags[i];
  if (!(fl & kInside)) return;
  const int le = P.last_elem[i];
  if (le < 0) return;
  double x[3] = {P.x[i], P.y[i], P.z[i]};
  double xl[3] = {P.lx[i], P.ly[i], P.lz[i]};
  double v[3];
  if constexpr (MIXED) { v[0] = P.vxf[i]; v[1] = P.vyf[i]; v[2] = P.vzf[i]; }
  else { v[0] = P.vx[i]; v[1] = P.vy[i]; v[2] = P.vz[i]; }
  int ne = tria_track(M, le, x, xl, v);
  if constexpr (MIXED) { P.vxf[i] = (float)v[0]; P.vyf[i] = (float)v[1]; P.vzf[i] = (float)v[2]; }
  else { P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2]; }
  if (ne < 0) {
    P.flags[i] = fl & ~kInside;
    if (ne == -1) { atomicAdd(&st->n_lost, 1); flag_status(st, 0x01u); }
    else if (ne == -2) flag_status(st, 0x04u);
    ne = le;
  }
  P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
  P.lx[i] = xl[0]; P.ly[i] = xl[1]; P.lz[i] = xl[2];
  P.elem[i] = ne;
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_track_ref(const __grid_constant__ DevMesh M, DevParticles P, DevStatus* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = P.flags[i];
  if (!(fl & kInside)) return;
  double x[3] = {P.x[i], P.y[i], P.z[i]};
  double xl[3] = {P.lx[i], P.ly[i], P.lz[i]};
  double xi[3] = {P.xi0[i], P.xi1[i], P.xi2[i]};
  double v[3];
  if constexpr (MIXED) { v[0] = P.vxf[i]; v[1] = P.vyf[i]; v[2] = P.vzf[i]; }
  else { v[0] = P.vx[i]; v[1] = P.vy[i]; v[2] = P.vz[i]; }
  bool tol = false, removed = false, cap = false;
  const int ne = ref_track<false>(M, P.last_elem[i], x, xl, xi, v, tol, removed, cap);
  if (tol) { atomicAdd(&st->n_ref_tolerance, 1); flag_status(st, 0x08u); }
  if (cap) flag_status(st, 0x04u);
  if constexpr (MIXED) { P.vxf[i] = (float)v[0]; P.vyf[i] = (float)v[1]; P.vzf[i] = (float)v[2]; }
  else { P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2]; }
  if (removed) P.flags[i] = fl & ~kInside;
  P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
  P.lx[i] = xl[0]; P.ly[i] = xl[1]; P.lz[i] = xl[2];
  P.xi0[i] = xi[0]; P.xi1[i] = xi[1]; P.xi2[i] = xi[2];
  P.elem[i] = ne;
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_deposit_cvwm(const __grid_constant__ DevMesh M, MeshF MF, DevParticles P, double* __restrict__ NS,
                                                      DevStatus* st) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in_range = i < P.n;
  const uint8_t fl = in_range ? P.flags[i] : 0;
  const bool inside = (fl & kInside) != 0;
  const int sp = inside ? P.species[i] : 0;
  const bool charged = inside && (kc.q[sp] != 0.0);
  const int e = inside ? P.elem[i] : 0;
  double x[3] = {0.0, 0.0, 0.0};
  if (inside) { x[0] = P.x[i]; x[1] = P.y[i]; x[2] = P.z[i]; }
  if constexpr (!MIXED) {
    double contrib[32];
    if (charged) {
      double xi[3];
      const bool suc = position_in_ref_elem(M, e, x, xi);
      if (!suc) { atomicAdd(&st->n_newton_failed, 1); flag_status(st, 0x02u); }
      const double ch = kc.qm[sp];
      const double TS[4] = {P.vx[i] * ch, P.vy[i] * ch, P.vz[i] * ch, ch};
      cvwm_contrib(M, e, suc, xi, x, TS, contrib);
    }
    cvwm_scatter(M, charged, e, contrib, NS);
  } else {
    float hi[32];
    if (charged) {
      const double* b = M.bary + (size_t)e * 3;
      const float p[3] = {(float)(x[0] - __ldg(b)), (float)(x[1] - __ldg(b + 1)), (float)(x[2] - __ldg(b + 2))};
      float xi[3];
      bool suc = position_in_ref_elem_f(M, MF, e, x, p, xi);
      const float ch = (float)kc.qm[sp];
      const float TS[4] = {P.vxf[i] * ch, P.vyf[i] * ch, P.vzf[i] * ch, ch};
      if (!suc) {
        double xd[3];
        suc = position_in_ref_elem(M, e, x, xd);
        if (!suc) { atomicAdd(&st->n_newton_failed, 1); flag_status(st, 0x02u); }
        double TSd[4] = {TS[0], TS[1], TS[2], TS[3]}, cd[32];
        cvwm_contrib(M, e, suc, xd, x, TSd, cd);
#pragma unroll
        for (int k = 0; k < 32; ++k) hi[k] = (float)cd[k];
      } else {
        const float a1 = 0.5f * (xi[0] + 1.0f), a2 = 0.5f * (xi[1] + 1.0f), a3 = 0.5f * (xi[2] + 1.0f);
        const float b1 = 1.0f - a1, b2 = 1.0f - a2, b3 = 1.0f - a3;
        const float w[8] = {b1 * b2 * b3, a1 * b2 * b3, a1 * a2 * b3, b1 * a2 * b3,
                            b1 * b2 * a3, a1 * b2 * a3, a1 * a2 * a3, b1 * a2 * a3};
#pragma unroll
        for (int n = 0; n < 8; ++n)
#pragma unroll
          for (int c = 0; c < 4; ++c) hi[4 * n + c] = TS[c] * w[n];
      }
    }
    cvwm_scatter_ts(M, charged, e, hi, NS);
  }
}

// =============================================================================================
// Counting sort by element (integer keys: element ids are exact)
// =============================================================================================
// Counting-sort slot for `key`, one atomic per distinct key of the warp: particles grouped by element
// mostly share the key within a warp.  Every lane of the warp calls it (valid = false adds nothing);
// returns the slot, or -1 for invalid lanes.  Slots of one key follow lane order within the warp.
__device__ __forceinline__ int warp_slot(int* __restrict__ cursor, int key, bool valid) {
  const unsigned act = __ballot_sync(kFull, valid);
  if (!valid) return -1;
  const unsigned peers = __match_any_sync(act, key);
  const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(cursor + key, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(256) k_hist(DevParticles P, int* __restrict__ count, int ne) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;      // the grid covers whole warps: no early return
  const bool valid = i < P.n;
  const int key = valid ? ((P.flags[i] & kInside) ? P.elem[i] : ne) : 0;
  warp_slot(count, key, valid);
}

// single-CTA exclusive scan of count[0..n) into offset[0..n] (offset[n] = total)
__global__ void __launch_bounds__(1024) k_scan(const int* __restrict__ count, int* __restrict__ offset,
                                               int* __restrict__ cursor, int n) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int base = 0; base < n; base += 1024) {
    const int idx = base + threadIdx.x;
    const int v = idx < n ? count[idx] : 0;
    int s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(kFull, s, o);
      if (lane >= o) s += t;
    }
    if (lane == 31) warp_tot[wid] = s;
    __syncthreads();
    if (wid == 0) {
      int w = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, w, o);
        if (lane >= o) w += t;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const int excl = carry + (wid > 0 ? warp_tot[wid - 1] : 0) + s - v;
    if (idx < n) { offset[idx] = excl; cursor[idx] = excl; }
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) offset[n] = carry;
}

// =============================================================================================
// Shape-function deposition: pack particles by element, then gather per target element
// =============================================================================================
// Sub-cell binning of the pack (mixed gather with octant warps): key 8 e + octant of the FP32 position relative to
// the element's DOF centre, computed exactly as the pack computes the record (same conversion, same sign test).
__device__ __forceinline__ int sf_sub_key(const Consts& kc, const DevParticles& P, int i, int e,
                                          const double* __restrict__ dofc) {
  const double x = kc.sf_keep[0] ? P.x[i] : 0.0, y = kc.sf_keep[1] ? P.y[i] : 0.0, z = kc.sf_keep[2] ? P.z[i] : 0.0;
  const double* c = dofc + (size_t)e * 3;
  const float rx = (float)(x - __ldg(c)), ry = (float)(y - __ldg(c + 1)), rz = (float)(z - __ldg(c + 2));
  return 8 * e + (rx > 0.0f ? 1 : 0) + (ry > 0.0f ? 2 : 0) + (rz > 0.0f ? 4 : 0);
}

__global__ void __launch_bounds__(256) k_hist8(const __grid_constant__ Consts kc, DevParticles P,
                                               const double* __restrict__ dofc, int* __restrict__ count8, int ne) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;      // the grid covers whole warps: no early return
  const bool valid = i < P.n;
  const bool in = valid && (P.flags[i] & kInside);
  const int key = in ? sf_sub_key(kc, P, i, P.elem[i], dofc) : 8 * ne;
  warp_slot(count8, key, valid);
}

// element counts from the sub-cell counts (count[ne] = particles not inside)
__global__ void __launch_bounds__(256) k_sum8(const int* __restrict__ count8, int* __restrict__ count, int ne) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e > ne) return;
  int sum = 0;
  if (e < ne) {
#pragma unroll
    for (int c = 0; c < 8; ++c) sum += count8[8 * e + c];
  } else {
    sum = count8[8 * ne];
  }
  count[e] = sum;
}

// sub-cell offsets inside each element's range, and the pack cursors
__global__ void __launch_bounds__(256) k_sub_offsets(const int* __restrict__ count8, const int* __restrict__ offset,
                                                     int* __restrict__ off8, int* __restrict__ cursor8, int ne) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e > ne) return;
  if (e == ne) { off8[8 * ne] = offset[ne]; cursor8[8 * ne] = offset[ne]; return; }
  int o = offset[e];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    off8[8 * e + c] = o;
    cursor8[8 * e + c] = o;
    o += count8[8 * e + c];
  }
}

template <bool MIXED, bool SUB>
__global__ void __launch_bounds__(256) k_sf_pack(const __grid_constant__ Consts kc, DevParticles P, int* __restrict__ cursor, const double* __restrict__ dofc,
                                                 SfPack K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < P.n && (P.flags[i] & kInside);
  const int e = valid ? P.elem[i] : 0;
  // SUB: records ordered by (element, sub-cell) through the sub-cell cursors
  const int slot = warp_slot(cursor, SUB && valid ? sf_sub_key(kc, P, i, e, dofc) : e, valid);
  if (!valid) return;
  const int sp = P.species[i];
  const double qm = kc.qm[sp];
  // 1D/2D shape function: the coordinates without kernel are zero, as in the DOF coordinates
  const double x = kc.sf_keep[0] ? P.x[i] : 0.0, y = kc.sf_keep[1] ? P.y[i] : 0.0, z = kc.sf_keep[2] ? P.z[i] : 0.0;
  const double* c = dofc + (size_t)e * 3;
  const float4 rel = make_float4((float)(x - __ldg(c)), (float)(y - __ldg(c + 1)), (float)(z - __ldg(c + 2)), 0.0f);
  reinterpret_cast<float4*>(K.posf)[slot] = rel;
  if constexpr (!MIXED) {
    const double w = kc.sf_w;
    // Fac(1:3) = PartVelo*ChargeMPF, Fac(4) = ChargeMPF, Fac = Fac*w_sf (shapefunction_tools:78-100)
    const double f0 = (P.vx[i] * qm) * w, f1 = (P.vy[i] * qm) * w, f2 = (P.vz[i] * qm) * w, f3 = qm * w;
    K.pos[(size_t)slot * 3] = x; K.pos[(size_t)slot * 3 + 1] = y; K.pos[(size_t)slot * 3 + 2] = z;
    double2* fp = reinterpret_cast<double2*>(K.fac + (size_t)slot * 4);
    fp[0] = make_double2(f0, f1);
    fp[1] = make_double2(f2, f3);
  } else {
    const float w = (float)(kc.sf_w * qm);
    reinterpret_cast<float4*>(K.facf)[slot] = make_float4(P.vxf[i] * w, P.vyf[i] * w, P.vzf[i] * w, w);
  }
}

constexpr int kSfChunk = 256;

template <int N>
struct SfShape {
  static constexpr int n1 = N + 1, nd = n1 * n1 * n1;
  static constexpr int split = nd >= 128 ? 1 : 128 / nd;
  static constexpr int threads = ((nd * split + 31) / 32) * 32;
};

// FP64 gather.  An FP32 pre-test on coordinates relative to the target element's DOF centre
// discards pairs outside (1+1e-4) R; the rest is evaluated exactly as the reference does in FP64.
template <int N>
__global__ void __launch_bounds__(SfShape<N>::threads) k_sf_gather_fp64(const __grid_constant__ DevMesh M, SfLists L, const int* __restrict__ off,
                                                                        SfPack K, double* __restrict__ PS) {
  const Consts& kc = M.k;
  using S = SfShape<N>;
  constexpr int nd = S::nd, split = S::split;
  __shared__ double s_pos[kSfChunk][3];
  __shared__ double s_fac[kSfChunk][4];
  __shared__ float4 s_rel[kSfChunk];
  __shared__ double s_red[split > 1 ? S::threads : 1][4];
  const int e = L.order ? __ldg(L.order + blockIdx.x) : blockIdx.x;
  const int t = threadIdx.x;
  const int dof = t % nd, part = t / nd;
  const bool active = t < nd * split;
  const double* ce = L.dof_center + (size_t)e * 3;
  const double cex = __ldg(ce), cey = __ldg(ce + 1), cez = __ldg(ce + 2);
  double xg[3] = {0, 0, 0};
  float xgf[3] = {0, 0, 0};
  if (active) {
    const double* g = M.sf_xgp + (dof_base<N>(M, e) + dof) * 3;
    xg[0] = __ldg(g); xg[1] = __ldg(g + 1); xg[2] = __ldg(g + 2);
    xgf[0] = (float)(xg[0] - cex); xgf[1] = (float)(xg[1] - cey); xgf[2] = (float)(xg[2] - cez);
  }
  const double R2 = kc.sf_r2, R2inv = kc.sf_r2_inv;
  const float R2f = (float)(R2 * (1.0 + 1.0e-4));
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int p0 = __ldg(L.nb_off + e), p1 = __ldg(L.nb_off + e + 1);
  for (int p = p0; p < p1; ++p) {
    const int s = __ldg(L.nb_src + p);
    double sh[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int k = kc.pv_dir[d];
      sh[d] = k >= 0 ? (double)L.nb_shift[3 * p + d] * kc.pv[3 * k + d] : 0.0;
    }
    const double* cs = L.dof_center + (size_t)s * 3;
    const float ox = (float)((__ldg(cs) + sh[0]) - cex), oy = (float)((__ldg(cs + 1) + sh[1]) - cey),
                oz = (float)((__ldg(cs + 2) + sh[2]) - cez);
    const int b0 = __ldg(off + s), cnt = __ldg(off + s + 1) - b0;
    for (int base = 0; base < cnt; base += kSfChunk) {
      const int nl = min(kSfChunk, cnt - base);
      __syncthreads();
      for (int q = t; q < nl; q += S::threads) {
        const size_t j = (size_t)b0 + base + q;
        const float4 r = reinterpret_cast<const float4*>(K.posf)[j];
        s_rel[q] = make_float4(r.x + ox, r.y + oy, r.z + oz, 0.0f);
        s_pos[q][0] = K.pos[3 * j] + sh[0];
        s_pos[q][1] = K.pos[3 * j + 1] + sh[1];
        s_pos[q][2] = K.pos[3 * j + 2] + sh[2];
        const double2* fp = reinterpret_cast<const double2*>(K.fac + 4 * j);
        const double2 f01 = fp[0], f23 = fp[1];
        s_fac[q][0] = f01.x; s_fac[q][1] = f01.y; s_fac[q][2] = f23.x; s_fac[q][3] = f23.y;
      }
      __syncthreads();
      if (active) {
        for (int q = part; q < nl; q += split) {
          const float4 r = s_rel[q];
          const float dx = r.x - xgf[0], dy = r.y - xgf[1], dz = r.z - xgf[2];
          const float r2f = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (r2f <= R2f) {
            const double d0 = s_pos[q][0] - xg[0], d1 = s_pos[q][1] - xg[1], d2 = s_pos[q][2] - xg[2];
            const double r2 = (d0 * d0 + d1 * d1) + d2 * d2;
            if (r2 <= R2) {
              const double Sv = 1.0 - R2inv * r2;
              double S1 = Sv * Sv;
              for (int ex = 3; ex <= kc.sf_alpha; ++ex) S1 = Sv * S1;
#pragma unroll
              for (int c = 0; c < 4; ++c) acc[c] = acc[c] + S1 * s_fac[q][c];
            }
          }
        }
      }
    }
  }
  if constexpr (split > 1) {
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 4; ++c) s_red[t][c] = acc[c];
    __syncthreads();
    if (t < nd) {
      for (int k = 1; k < split; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s_red[t + k * nd][c];
    }
  }
  if (t < nd) {
    double2* o = reinterpret_cast<double2*>(PS + (dof_base<N>(M, e) + dof) * 4);
    o[0] = make_double2(acc[0], acc[1]);
    o[1] = make_double2(acc[2], acc[3]);
  }
}

// Mixed gather: FP32 distances and weights, per-DOF TwoSum-compensated FP32 sums, FP64 result.
template <int N>
__global__ void __launch_bounds__(SfShape<N>::threads) k_sf_gather_mixed(const __grid_constant__ DevMesh M, SfLists L, const int* __restrict__ off,
                                                                         SfPack K, double* __restrict__ PS) {
  const Consts& kc = M.k;
  using S = SfShape<N>;
  constexpr int nd = S::nd, split = S::split;
  __shared__ float4 s_rel[kSfChunk];
  __shared__ float4 s_fac[kSfChunk];
  __shared__ float s_red[split > 1 ? S::threads : 1][8];
  const int e = L.order ? __ldg(L.order + blockIdx.x) : blockIdx.x;
  const int t = threadIdx.x;
  const int dof = t % nd, part = t / nd;
  const bool active = t < nd * split;
  const double* ce = L.dof_center + (size_t)e * 3;
  const double cex = __ldg(ce), cey = __ldg(ce + 1), cez = __ldg(ce + 2);
  float xgf[3] = {0, 0, 0};
  if (active) {
    const double* g = M.sf_xgp + (dof_base<N>(M, e) + dof) * 3;
    xgf[0] = (float)(__ldg(g) - cex); xgf[1] = (float)(__ldg(g + 1) - cey); xgf[2] = (float)(__ldg(g + 2) - cez);
  }
  const float R2 = (float)kc.sf_r2, R2inv = (float)kc.sf_r2_inv;
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  const int p0 = __ldg(L.nb_off + e), p1 = __ldg(L.nb_off + e + 1);
  for (int p = p0; p < p1; ++p) {
    const int s = __ldg(L.nb_src + p);
    double sh[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int k = kc.pv_dir[d];
      sh[d] = k >= 0 ? (double)L.nb_shift[3 * p + d] * kc.pv[3 * k + d] : 0.0;
    }
    const double* cs = L.dof_center + (size_t)s * 3;
    const float ox = (float)((__ldg(cs) + sh[0]) - cex), oy = (float)((__ldg(cs + 1) + sh[1]) - cey),
                oz = (float)((__ldg(cs + 2) + sh[2]) - cez);
    const int b0 = __ldg(off + s), cnt = __ldg(off + s + 1) - b0;
    for (int base = 0; base < cnt; base += kSfChunk) {
      const int nl = min(kSfChunk, cnt - base);
      __syncthreads();
      for (int q = t; q < nl; q += S::threads) {
        const size_t j = (size_t)b0 + base + q;
        const float4 r = reinterpret_cast<const float4*>(K.posf)[j];
        s_rel[q] = make_float4(r.x + ox, r.y + oy, r.z + oz, 0.0f);
        s_fac[q] = reinterpret_cast<const float4*>(K.facf)[j];
      }
      __syncthreads();
      if (active) {
        for (int q = part; q < nl; q += split) {
          const float4 r = s_rel[q];
          const float dx = r.x - xgf[0], dy = r.y - xgf[1], dz = r.z - xgf[2];
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (r2 <= R2) {
            const float Sv = fmaf(-R2inv, r2, 1.0f);
            float S1 = Sv * Sv;
            for (int ex = 3; ex <= kc.sf_alpha; ++ex) S1 = Sv * S1;
            const float4 f = s_fac[q];
            const float fc[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              float sm, er;
              two_sum(hi[c], S1 * fc[c], sm, er);
              hi[c] = sm;
              lo[c] += er;
            }
          }
        }
      }
    }
  }
  double acc[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) acc[c] = (double)hi[c] + (double)lo[c];
  if constexpr (split > 1) {
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 4; ++c) { s_red[t][c] = hi[c]; s_red[t][4 + c] = lo[c]; }
    __syncthreads();
    if (t < nd) {
      for (int k = 1; k < split; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + ((double)s_red[t + k * nd][c] + (double)s_red[t + k * nd][4 + c]);
    }
  }
  if (t < nd) {
    double2* o = reinterpret_cast<double2*>(PS + (dof_base<N>(M, e) + dof) * 4);
    o[0] = make_double2(acc[0], acc[1]);
    o[1] = make_double2(acc[2], acc[3]);
  }
}

// Two-phase gather (N <= 3, nd <= 64).  Per (source element, periodic image) pair the CTA stages
// the source's particles that lie within R + (DOF-box radius) of the target's DOF centre.  Then:
//   phase A: every lane owns one DOF and tests every staged particle of its half in FP32 against
//            (1+1e-4) R^2; hits go to a per-lane list in shared memory (column per lane);
//   phase B: each lane walks its own list and evaluates (1 - r^2/R^2)^alpha * Fac -- exactly in
//            FP64 (decision r^2 <= R^2 in FP64 as the reference), or in FP32 with TwoSum-compensated
//            per-DOF sums (mixed).  Lanes are busy in proportion to their hit counts instead of
//            executing the evaluation for every particle any lane of the warp hits.
[[maybe_unused]] constexpr int kSf2Chunk = 256;   // used by the PIC_SF_GATHER=2 build
constexpr int kSf2Threads = 128;   // 4 warps: (DOF half) x (particle parity)

template <int N, bool MIXED>
__global__ void __launch_bounds__(kSf2Threads) k_sf_gather2(const __grid_constant__ DevMesh M, SfLists L, const int* __restrict__ off,
                                                            SfPack K, double* __restrict__ PS) {
  const Consts& kc = M.k;
  constexpr int n1 = N + 1, nd = n1 * n1 * n1;
  static_assert(nd <= 64, "two-phase gather holds at most 64 DOFs per element");
  __shared__ float4 s_rel[kSf2Chunk];
  __shared__ float4 s_facf[MIXED ? kSf2Chunk : 1];
  __shared__ double s_pos[MIXED ? 1 : kSf2Chunk][3];
  __shared__ double s_fac[MIXED ? 1 : kSf2Chunk][4];
  __shared__ uint8_t s_list[4][kSf2Chunk / 2][32];
  __shared__ int s_cnt;
  __shared__ double s_red[2][64][4];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int dof = (w & 1) * 32 + lane, parity = w >> 1;
  const bool active = dof < nd;
  const int e = L.order ? __ldg(L.order + blockIdx.x) : blockIdx.x;
  const double* ce = L.dof_center + (size_t)e * 3;
  const double cex = __ldg(ce), cey = __ldg(ce + 1), cez = __ldg(ce + 2);
  double xg[3] = {0, 0, 0};
  float xgf[3] = {0, 0, 0};
  if (active) {
    const double* g = M.sf_xgp + (dof_base<N>(M, e) + dof) * 3;
    xg[0] = __ldg(g); xg[1] = __ldg(g + 1); xg[2] = __ldg(g + 2);
    xgf[0] = (float)(xg[0] - cex); xgf[1] = (float)(xg[1] - cey); xgf[2] = (float)(xg[2] - cez);
  }
  const double R2 = kc.sf_r2, R2inv = kc.sf_r2_inv;
  const float R2f = (float)(R2 * (1.0 + 1.0e-4));
  const float cull = (float)kc.sf_r + __ldg(L.dof_radius + e);
  const float cull2 = cull * cull * 1.0001f;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  const int p0 = __ldg(L.nb_off + e), p1 = __ldg(L.nb_off + e + 1);
  for (int p = p0; p < p1; ++p) {
    const int s = __ldg(L.nb_src + p);
    double sh[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int k = kc.pv_dir[d];
      sh[d] = k >= 0 ? (double)L.nb_shift[3 * p + d] * kc.pv[3 * k + d] : 0.0;
    }
    const double* cs = L.dof_center + (size_t)s * 3;
    const float ox = (float)((__ldg(cs) + sh[0]) - cex), oy = (float)((__ldg(cs + 1) + sh[1]) - cey),
                oz = (float)((__ldg(cs + 2) + sh[2]) - cez);
    const int b0 = __ldg(off + s), cnt = __ldg(off + s + 1) - b0;
    for (int base = 0; base < cnt; base += kSf2Chunk) {
      const int nl = min(kSf2Chunk, cnt - base);
      __syncthreads();
      if (t == 0) s_cnt = 0;
      __syncthreads();
      for (int q = t; q < nl; q += kSf2Threads) {
        const size_t j = (size_t)b0 + base + q;
        const float4 r = reinterpret_cast<const float4*>(K.posf)[j];
        const float rx = r.x + ox, ry = r.y + oy, rz = r.z + oz;
        if (fmaf(rx, rx, fmaf(ry, ry, rz * rz)) <= cull2) {
          const int slot = atomicAdd(&s_cnt, 1);
          s_rel[slot] = make_float4(rx, ry, rz, 0.0f);
          if constexpr (MIXED) {
            s_facf[slot] = reinterpret_cast<const float4*>(K.facf)[j];
          } else {
            s_pos[slot][0] = K.pos[3 * j] + sh[0];
            s_pos[slot][1] = K.pos[3 * j + 1] + sh[1];
            s_pos[slot][2] = K.pos[3 * j + 2] + sh[2];
            const double2* fp = reinterpret_cast<const double2*>(K.fac + 4 * j);
            const double2 f01 = fp[0], f23 = fp[1];
            s_fac[slot][0] = f01.x; s_fac[slot][1] = f01.y; s_fac[slot][2] = f23.x; s_fac[slot][3] = f23.y;
          }
        }
      }
      __syncthreads();
      const int nst = s_cnt;
      if (!active) continue;
      // phase A: FP32 test, per-lane hit lists
      int nh = 0;
      for (int q = parity; q < nst; q += 2) {
        const float4 r = s_rel[q];
        const float dx = r.x - xgf[0], dy = r.y - xgf[1], dz = r.z - xgf[2];
        const float r2f = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (r2f <= R2f) s_list[w][nh++][lane] = (uint8_t)q;
      }
      // phase B: evaluate this lane's hits
      for (int k = 0; k < nh; ++k) {
        const int q = s_list[w][k][lane];
        if constexpr (MIXED) {
          const float4 r = s_rel[q];
          const float dx = r.x - xgf[0], dy = r.y - xgf[1], dz = r.z - xgf[2];
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (r2 <= (float)R2) {
            const float Sv = fmaf(-(float)R2inv, r2, 1.0f);
            float S1 = Sv * Sv;
            for (int ex = 3; ex <= kc.sf_alpha; ++ex) S1 = Sv * S1;
            const float4 f = s_facf[q];
            const float fc[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              float sm, er;
              two_sum(hi[c], S1 * fc[c], sm, er);
              hi[c] = sm;
              lo[c] += er;
            }
          }
        } else {
          // FP64 with fused multiply-adds (12 FP64 instructions per hit instead of 19); differs from
          // the reference's unfused order by rounding only (no decision depends on it)
          const double d0 = s_pos[q][0] - xg[0], d1 = s_pos[q][1] - xg[1], d2 = s_pos[q][2] - xg[2];
          const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
          if (r2 <= R2) {
            const double Sv = fma(-R2inv, r2, 1.0);
            double S1 = Sv * Sv;
            for (int ex = 3; ex <= kc.sf_alpha; ++ex) S1 = Sv * S1;
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[c] = fma(S1, s_fac[q][c], acc[c]);
          }
        }
      }
    }
  }
  if constexpr (MIXED) {
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c] = (double)hi[c] + (double)lo[c];
  }
  __syncthreads();
  if (active && parity == 1) {
#pragma unroll
    for (int c = 0; c < 4; ++c) s_red[w & 1][lane][c] = acc[c];
  }
  __syncthreads();
  if (active && parity == 0) {
    double2* o = reinterpret_cast<double2*>(PS + (dof_base<N>(M, e) + dof) * 4);
    const double* rr = s_red[w & 1][lane];
    o[0] = make_double2(acc[0] + rr[0], acc[1] + rr[1]);
    o[1] = make_double2(acc[2] + rr[2], acc[3] + rr[3]);
  }
}

// Round-robin gather, one DOF per lane (N <= 3).  Candidates of all (source, image) pairs of the target
// are taken row by row (particle r of every pair, then r+1, ...) and the staging set is filled to at
// least kSf5Chunk - kSf5Threads entries, so every set surrounds the target evenly and each DOF's
// hit count is close to the mean: per-lane hit lists then keep the lanes of a warp about equally busy
// (simulated 86 % of lane slots carry a hit, 46 % with sets from one source element at a time).
// Warps: (DOF half) x (particle parity) for nd > 32, four parities for nd <= 32.
// FP64: with p, g the particle and DOF positions relative to the target's DOF centre,
// 1 - |p-g|^2/R^2 = A_p + B_g + p'.g with A_p = -|p|^2/R^2, p' = 2p/R^2 (per staged particle) and
// B_g = 1 - |g|^2/R^2 (per DOF): one add and three fused multiply-adds per hit, 9 FP64 instructions
// per hit in all.  It differs from the reference's (1 - r^2/R^2) by rounding only (|terms| <= 8, so
// ~1e-15 absolute); the reference keeps r^2 <= R^2, here 1 - r^2/R^2 >= 0 (read from the sign bit).
// Mixed: FP32 distances and weights; per staged set each lane sums its hits in FP32 (fused
// multiply-adds, at most kSf5Chunk / npar terms, ~30 on average) and adds that partial to its DOF's
// (hi, lo) pair with TwoSum; the FP64 result is hi + lo.  Against the same accumulation with TwoSum per
// hit: 15 % less time, rho error vs FP64 1.7e-7 instead of 1.3e-7 (32^3 curved, 16M particles).
// FP64 with alpha = 2 and one radius: a staged particle whose kernel covers every DOF of a DOF group -- the
// target element, or (N = 3) one of its two DOF halves -- adds S_g^2 = (u.v_g + B_g)^2 to each of them,
// u = (p', A_p), v_g = (g, 1).  Summed over such particles that is v^T Q_c v + 2 B_g v.L_c + B_g^2 Z_c with
// the moments Q_c = sum f_c u u^T, L_c = sum f_c u, Z_c = sum f_c (15 per component), accumulated by 60
// threads per particle and evaluated per DOF at the end: 2 FP64 instructions per thread and particle instead
// of 9 per hit (at R = 1.5 h and N = 3 about 16 % of the hits are covered by the element test, 27 % with the
// halves).  Covered means the group's DOF box lies within R (1 - 1e-4) of the particle in an FP32 test with
// the box rounded outwards, so every reference test r^2 <= R^2 of the group holds.
constexpr int kSf5Chunk = 256;
constexpr int kSf5Threads = 128;
constexpr int kSf5Pairs = 152;

// (1 - r^2/R^2)^alpha from Sv = 1 - r^2/R^2: S*S, then alpha - 2 more factors (runtime alpha unless A2)
template <bool A2, typename T>
__device__ __forceinline__ T sf_power(const Consts& kc, T Sv) {
  T S1 = Sv * Sv;
  if constexpr (!A2)
    for (int ex = 3; ex <= kc.sf_alpha; ++ex) S1 = Sv * S1;
  return S1;
}

template <int N, bool MIXED, bool ADAPT, bool A2>
__global__ void __launch_bounds__(kSf5Threads) k_sf_gather5(const __grid_constant__ DevMesh M, SfLists L, const int* __restrict__ off,
                                                            SfPack K, double* __restrict__ PS) {
  const Consts& kc = M.k;
  constexpr int n1 = N + 1, nd = n1 * n1 * n1;
  static_assert(nd <= 64, "one DOF per lane, at most two DOF halves");
  constexpr int halves = nd > 32 ? 2 : 1, npar = 4 / halves;
  constexpr int cap = kSf5Chunk / npar;                  // hit-list entries per lane
  __shared__ float4 s_rel[kSf5Chunk];
  __shared__ float4 s_facf[MIXED ? kSf5Chunk : 1];
  __shared__ __align__(16) double2 s_pq[2 * kSf5Chunk];  // FP64: (p'x, p'y), (p'z, A_p); per-DOF sums at the end
  __shared__ double2 s_fac[MIXED ? 1 : 2 * kSf5Chunk];
  __shared__ uint8_t s_list[kSf5Threads / 32][cap][32];
  __shared__ uint8_t s_nh[kSf5Threads / 32][32];         // hit-list lengths (pooled phase B)
  __shared__ int s_j[kSf5Chunk];
  __shared__ uint8_t s_pr[kSf5Chunk];
  __shared__ int s_b0[kSf5Pairs], s_n[kSf5Pairs];
  __shared__ float s_o[kSf5Pairs][3];
  __shared__ double s_off[MIXED ? 1 : kSf5Pairs][3];
  // shape_function_adaptive: radius of each pair's source element
  __shared__ float s_r2f[ADAPT ? kSf5Pairs : 1];                  // (1+1e-4) R_s^2, FP32 pre-test
  __shared__ double s_rinv[ADAPT && !MIXED ? kSf5Pairs : 1];      // 1/R_s^2
  __shared__ float2 s_rpf[ADAPT && MIXED ? kSf5Pairs : 1];        // (R_s^2, 1/R_s^2)
  __shared__ float2 s_rp[ADAPT && MIXED ? kSf5Chunk : 1];         // the same per staged particle
  // mixed, one radius: the pre-test on two staged particles per instruction in packed FP16, positions in
  // units of R relative to the target's DOF centre; entry i*npar + p holds the slots p + npar*2i and
  // p + npar*(2i+1) of parity p (see the comment at phase A)
  // (mixed uses s_pq only for the final per-DOF sums, so the FP16 copy lives there)
  constexpr bool H2 = MIXED && !ADAPT;
  constexpr bool MOM = !MIXED && !ADAPT && A2;
  // moments: DOF boxes (FP32, rounded outwards) of the halves and of the element, [group][lo, hi][axis]; the
  // slots of the staged particles covering the element or one half (which: the bits in s_rel[slot].w)
  __shared__ float s_box[3][2][3];
  __shared__ int s_nfull;
  __shared__ uint8_t s_flist[MOM ? kSf5Chunk : 1];
  __shared__ int s_cnt, s_max;
  static_assert(sizeof(double) * 4 * npar * (halves * 32) <= sizeof(double2) * 2 * kSf5Chunk, "sums alias s_pq");
  static_assert(sizeof(__half2) * 3 * (kSf5Chunk / 2 + 4) <= sizeof(double2) * 2 * kSf5Chunk, "FP16 set aliases s_pq");
  __half2 (*s_h)[3] = reinterpret_cast<__half2 (*)[3]>(s_pq);
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int dof = (w % halves) * 32 + lane, parity = w / halves;
  const bool active = dof < nd;
  const int e = L.order ? __ldg(L.order + blockIdx.x) : blockIdx.x;
  const double* ce = L.dof_center + (size_t)e * 3;
  const double cex = __ldg(ce), cey = __ldg(ce + 1), cez = __ldg(ce + 2);
  const double R2inv = kc.sf_r2_inv;
  const float R2f = (float)(kc.sf_r2 * (1.0 + 1.0e-4));
  const float cull = (float)kc.sf_r + __ldg(L.dof_radius + e);
  const float cull2 = cull * cull * 1.0001f;
  // FP16 pre-test where |p|/R + |g|/R <= 5 (DOF-box radius <= 2R), which bounds its r^2/R^2 error by 1.5e-2
  const bool h2 = H2 && __ldg(L.dof_radius + e) <= 2.0f * (float)kc.sf_r;
  double gd[4] = {0.0, 0.0, 0.0, 0.0};
  float gf[3] = {0.f, 0.f, 0.f};
  if (active) {
    const double* g = M.sf_xgp + (dof_base<N>(M, e) + dof) * 3;
    const double gx = __ldg(g) - cex, gy = __ldg(g + 1) - cey, gz = __ldg(g + 2) - cez;
    gd[0] = gx; gd[1] = gy; gd[2] = gz;
    // B_g = 1 - |g|^2/R^2; adaptive: |g|^2 (the particle's own radius enters at each hit)
    gd[3] = ADAPT ? fma(gx, gx, fma(gy, gy, gz * gz)) : fma(-R2inv, fma(gx, gx, fma(gy, gy, gz * gz)), 1.0);
    gf[0] = (float)gx; gf[1] = (float)gy; gf[2] = (float)gz;
  }
  // moments: thread (half mh, index mm < 60) accumulates moment mm (component mm / 15; 0..9 Q_ij, 10..13 L_i,
  // 14 Z) over the covering particles of its half; u[4] stands for 1
  const int mh = t >> 6, mm = t & 63, mk = mm % 15;
  const int mi = mk < 10 ? (mk < 4 ? 0 : mk < 7 ? 1 : mk < 9 ? 2 : 3) : (mk < 14 ? mk - 10 : 4);
  const int mj = mk < 10 ? (mk < 4 ? mk : mk < 7 ? mk - 3 : mk < 9 ? mk - 5 : 3) : 4;
  double mom = 0.0, momh = 0.0;            // the element's moment (two copies) and half mh's
  if constexpr (MOM) {
    // per-warp DOF boxes (a warp holds DOFs of one half); the parity-0 warps write their half's box
    float lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = active ? __double2float_rd(gd[d]) : 3.0e38f;
      hi[d] = active ? __double2float_ru(gd[d]) : -3.0e38f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
        hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
      }
    }
    if (parity == 0 && lane == 0)
#pragma unroll
      for (int d = 0; d < 3; ++d) { s_box[w][0][d] = lo[d]; s_box[w][1][d] = hi[d]; }
    __syncthreads();
    if (t < 3) {
      s_box[2][0][t] = halves == 2 ? fminf(s_box[0][0][t], s_box[1][0][t]) : s_box[0][0][t];
      s_box[2][1][t] = halves == 2 ? fmaxf(s_box[0][1][t], s_box[1][1][t]) : s_box[0][1][t];
    }
  }
  const float cover2 = (float)(kc.sf_r2 * (1.0 - 1.0e-4));
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  const double t2 = 2.0 * R2inv;
  const int p0 = __ldg(L.nb_off + e), p1 = __ldg(L.nb_off + e + 1);
  for (int pw = p0; pw < p1; pw += kSf5Pairs) {
    const int npw = min(kSf5Pairs, p1 - pw);
    __syncthreads();                       // the previous window is finished with the pair tables
    if (t == 0) s_max = 0;
    __syncthreads();
    for (int i = t; i < npw; i += kSf5Threads) {
      const int p = pw + i;
      const int src = __ldg(L.nb_src + p);
      double sh[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int k = kc.pv_dir[d];
        sh[d] = k >= 0 ? (double)L.nb_shift[3 * p + d] * kc.pv[3 * k + d] : 0.0;
      }
      const double* cs = L.dof_center + (size_t)src * 3;
      s_o[i][0] = (float)((__ldg(cs) + sh[0]) - cex);
      s_o[i][1] = (float)((__ldg(cs + 1) + sh[1]) - cey);
      s_o[i][2] = (float)((__ldg(cs + 2) + sh[2]) - cez);
      if constexpr (!MIXED) { s_off[i][0] = sh[0] - cex; s_off[i][1] = sh[1] - cey; s_off[i][2] = sh[2] - cez; }
      if constexpr (ADAPT) {
        const double r = __ldg(L.elem_r + src), r2 = r * r;
        s_r2f[i] = (float)(r2 * (1.0 + 1.0e-4));
        if constexpr (MIXED) s_rpf[i] = make_float2((float)r2, (float)(1.0 / r2));
        else s_rinv[i] = 1.0 / r2;
      }
      const int b0 = __ldg(off + src), n = __ldg(off + src + 1) - b0;
      s_b0[i] = b0;
      s_n[i] = n;
      atomicMax(&s_max, n);
    }
    __syncthreads();
    const long long total = (long long)npw * s_max;    // candidates (row, pair), row-major
    long long cursor = 0;
    while (cursor < total) {
      __syncthreads();                     // the previous set is evaluated
      if (t == 0) { s_cnt = 0; s_nfull = 0; }
      __syncthreads();
      int nst = 0;
      while (cursor < total && nst <= kSf5Chunk - kSf5Threads) {
        const long long c = cursor + t;
        bool app = false;
        if (c < total) {
          const long long rowl = c / npw;
          const int pr = (int)(c - rowl * npw);
          if (rowl < s_n[pr]) {
            const int j = s_b0[pr] + (int)rowl;
            const float4 r = reinterpret_cast<const float4*>(K.posf)[j];
            const float rx = r.x + s_o[pr][0], ry = r.y + s_o[pr][1], rz = r.z + s_o[pr][2];
            if (fmaf(rx, rx, fmaf(ry, ry, rz * rz)) <= cull2) {
              const int slot = atomicAdd(&s_cnt, 1);
              unsigned cov = 0;       // moments: bit h = the particle covers DOF half h (both: the element)
              if constexpr (MOM) {
                const float rr[3] = {rx, ry, rz};
                auto far2 = [&](int b) {
                  float sum = 0.f;
#pragma unroll
                  for (int d = 0; d < 3; ++d) {
                    const float a = fmaxf(fabsf(rr[d] - s_box[b][0][d]), fabsf(rr[d] - s_box[b][1][d]));
                    sum = fmaf(a, a, sum);
                  }
                  return sum;
                };
                if (far2(2) <= cover2) cov = halves == 2 ? 3u : 1u;
                else if (halves == 2) cov = far2(0) <= cover2 ? 1u : far2(1) <= cover2 ? 2u : 0u;
                if (cov) s_flist[atomicAdd(&s_nfull, 1)] = (uint8_t)slot;
              }
              s_rel[slot] = make_float4(rx, ry, rz, ADAPT ? s_r2f[pr] : __uint_as_float(cov));
              if constexpr (MIXED) {
                s_facf[slot] = reinterpret_cast<const float4*>(K.facf)[j];
                if constexpr (ADAPT) s_rp[slot] = s_rpf[pr];
              } else {
                s_j[slot] = j;
                s_pr[slot] = (uint8_t)pr;
              }
              app = true;
            }
          }
        }
        nst += __syncthreads_count(app);
        cursor += kSf5Threads;
      }
      if constexpr (!MIXED) {
        // FP64 staging over the compacted set
        for (int slot = t; slot < nst; slot += kSf5Threads) {
          const size_t j = (size_t)s_j[slot];
          const int pr = s_pr[slot];
          const double px = K.pos[3 * j] + s_off[pr][0], py = K.pos[3 * j + 1] + s_off[pr][1],
                       pz = K.pos[3 * j + 2] + s_off[pr][2];
          if constexpr (ADAPT) {
            // 1 - |p-g|^2/R^2 = (1 - |p|^2/R^2) + (2p/R^2).g - |g|^2/R^2 with the source's R
            const double ri = s_rinv[pr], tt = 2.0 * ri;
            s_pq[2 * slot] = make_double2(px * tt, py * tt);
            s_pq[2 * slot + 1] = make_double2(pz * tt, fma(-ri, fma(px, px, fma(py, py, pz * pz)), 1.0));
          } else {
            s_pq[2 * slot] = make_double2(px * t2, py * t2);
            s_pq[2 * slot + 1] = make_double2(pz * t2, -R2inv * fma(px, px, fma(py, py, pz * pz)));
          }
          const double2* fp = reinterpret_cast<const double2*>(K.fac + 4 * j);
          s_fac[2 * slot] = fp[0];
          s_fac[2 * slot + 1] = fp[1];
        }
        __syncthreads();
        if constexpr (MOM) {
          // thread group mh (two warps): the element-covering entries of its parity into mom, the entries
          // covering half mh into momh (the branches are uniform per warp)
          if (mm < 60) {
            const int c = mm / 15;
            const unsigned all = halves == 2 ? 3u : 1u;
            const int nf = s_nfull;
            for (int f = 0; f < nf; ++f) {
              const int q = s_flist[f];
              const unsigned cov = __float_as_uint(s_rel[q].w);
              const bool el = cov == all;
              if (el ? (f & 1) != mh : cov != (1u << mh)) continue;
              const double* u = reinterpret_cast<const double*>(&s_pq[2 * q]);
              const double ua = mi < 4 ? u[mi & 3] : 1.0, ub = mj < 4 ? u[mj & 3] : 1.0;
              const double fc = reinterpret_cast<const double*>(&s_fac[2 * q])[c];
              if (el) mom = fma(ua * ub, fc, mom);
              else momh = fma(ua * ub, fc, momh);
            }
          }
        }
      }
      const int nper = (nst + npar - 1) / npar, np2 = (nper + 1) / 2;   // slots and slot pairs per parity
      if (h2) {
        // packed FP16 copy of the set for the pre-test (a missing partner sits far away: r^2 overflows)
        for (int i = t; i < npar * np2; i += kSf5Threads) {
          const int p = i % npar, k = i / npar;
          const int a = p + npar * (2 * k), b = a + npar;
          const float4 ra = a < nst ? s_rel[a] : make_float4(1e3f, 1e3f, 1e3f, 0.f);
          const float4 rb = b < nst ? s_rel[b] : make_float4(1e3f, 1e3f, 1e3f, 0.f);
          const float ir = kc.sf_r_inv;
          s_h[i][0] = __floats2half2_rn(ra.x * ir, rb.x * ir);
          s_h[i][1] = __floats2half2_rn(ra.y * ir, rb.y * ir);
          s_h[i][2] = __floats2half2_rn(ra.z * ir, rb.z * ir);
        }
        __syncthreads();
      }
      int nh = 0;
      if (active) {
        // phase A: test of this lane's DOF against its parity's particles, into the lane's hit list (slot
        // index / npar, ascending).  FP32 with (1+1e-4) R^2; mixed with one radius and a DOF box within 2R:
        // packed FP16 in units of R against 1.05 (error of r^2/R^2 below 1.5e-2 near the threshold), two
        // particles per instruction.  Either way phase B repeats the exact test, so only the work changes.
        if (h2) {
          const float ir = kc.sf_r_inv;
          const __half2 gx = __float2half2_rn(gf[0] * ir), gy = __float2half2_rn(gf[1] * ir),
                        gz = __float2half2_rn(gf[2] * ir);
          const __half2 thr = __float2half2_rn(1.05f);
          for (int k = 0; k < np2; ++k) {
            const __half2* e = s_h[k * npar + parity];
            const __half2 dx = __hsub2(e[0], gx), dy = __hsub2(e[1], gy), dz = __hsub2(e[2], gz);
            const __half2 r2 = __hfma2(dx, dx, __hfma2(dy, dy, __hmul2(dz, dz)));
            const unsigned msk = __hle2_mask(r2, thr);
            if (msk & 0xFFFFu) s_list[w][nh++][lane] = (uint8_t)(2 * k);
            if (msk & 0xFFFF0000u) s_list[w][nh++][lane] = (uint8_t)(2 * k + 1);
          }
        } else {
          // moments: a particle covering this lane's DOF half is in the moments instead
          const unsigned hbit = 1u << (w % halves);
          for (int m = 0; parity + npar * m < nst; ++m) {
            const float4 r = s_rel[parity + npar * m];
            const float dx = r.x - gf[0], dy = r.y - gf[1], dz = r.z - gf[2];
            const bool in = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= (ADAPT ? r.w : R2f);
            if (MOM ? (in && !(__float_as_uint(r.w) & hbit)) : in) s_list[w][nh++][lane] = (uint8_t)m;
          }
        }
      }
      // FP64: the npar warps holding a DOF (one per particle parity) pool its hit lists and take equal shares:
      // the longest share of a warp is closer to the mean than the longest own list (mixed: the FP32 hits are
      // too cheap for the extra barrier and bookkeeping, each lane takes its own list)
      if constexpr (!MIXED) {
        s_nh[w][lane] = (uint8_t)nh;
        __syncthreads();
      }
      if (!active) continue;
      // phase B: this lane's share of its DOF's pooled hits (the lists of parities 0..npar-1 in turn)
      int pre[npar + 1];
      pre[0] = 0;
#pragma unroll
      for (int k = 0; k < npar; ++k)
        pre[k + 1] = pre[k] + (MIXED ? (k == parity ? nh : 0) : (int)s_nh[w % halves + halves * k][lane]);
      const int plo = MIXED ? 0 : (parity * pre[npar]) / npar, phi = MIXED ? nh : ((parity + 1) * pre[npar]) / npar;
      float part[4] = {0.f, 0.f, 0.f, 0.f};      // mixed: this staged set's FP32 partial sums
      for (int pos = plo; pos < phi; ++pos) {
        int kp = 0;
#pragma unroll
        for (int k = 1; k < npar; ++k) kp += pos >= pre[k] ? 1 : 0;
        const int base = kp == 0 ? 0 : kp == 1 ? pre[1] : kp == 2 ? pre[2] : pre[npar - 1];
        const int q = MIXED ? parity + npar * (int)s_list[w][pos][lane]
                            : kp + npar * (int)s_list[w % halves + halves * kp][pos - base][lane];
        if constexpr (MIXED) {
          const float4 r = s_rel[q];
          const float dx = r.x - gf[0], dy = r.y - gf[1], dz = r.z - gf[2];
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const float2 rp = ADAPT ? s_rp[q] : make_float2((float)kc.sf_r2, (float)R2inv);
          if (r2 <= rp.x) {
            const float Sv = fmaf(-rp.y, r2, 1.0f);
            const float S1 = sf_power<A2>(kc, Sv);
            const float4 f = s_facf[q];
            part[0] = fmaf(S1, f.x, part[0]);
            part[1] = fmaf(S1, f.y, part[1]);
            part[2] = fmaf(S1, f.z, part[2]);
            part[3] = fmaf(S1, f.w, part[3]);
          }
        } else {
          const double2 pa = s_pq[2 * q], pb = s_pq[2 * q + 1];
          const double Sv = ADAPT ? fma(pa.x, gd[0], fma(pa.y, gd[1], fma(pb.x, gd[2], fma(-gd[3], s_rinv[s_pr[q]], pb.y))))
                                  : fma(pa.x, gd[0], fma(pa.y, gd[1], fma(pb.x, gd[2], pb.y + gd[3])));
          // Sv >= 0 read from the sign bit (integer pipe); -0.0 is skipped, its contribution is 0
          if (__double_as_longlong(Sv) >= 0) {
            const double S1 = sf_power<A2>(kc, Sv);
            const double2 f01 = s_fac[2 * q], f23 = s_fac[2 * q + 1];
            acc[0] = fma(S1, f01.x, acc[0]);
            acc[1] = fma(S1, f01.y, acc[1]);
            acc[2] = fma(S1, f23.x, acc[2]);
            acc[3] = fma(S1, f23.y, acc[3]);
          }
        }
      }
      if constexpr (MIXED) {
        // the set's partial joins the DOF sum through TwoSum: (hi, lo) carries the exact rounding errors
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          float sm, er;
          two_sum(hi[c], part[c], sm, er);
          hi[c] = sm;
          lo[c] += er;
        }
      }
    }
  }
  if constexpr (MIXED) {
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c] = (double)hi[c] + (double)lo[c];
  }
  // per-DOF sums over the particle parities
  __syncthreads();
  double (*s_red)[halves * 32][4] = reinterpret_cast<double (*)[halves * 32][4]>(s_pq);
  if (active) {
#pragma unroll
    for (int c = 0; c < 4; ++c) s_red[parity][dof][c] = acc[c];
  }
  // the moments (element: two copies, then half 0 and half 1), in s_pq behind the per-DOF sums
  double (*s_mom)[64] = reinterpret_cast<double (*)[64]>(s_pq) + 2 * npar * halves;
  static_assert(sizeof(double) * (4 * npar * halves * 32 + 4 * 64) <= sizeof(double2) * 2 * kSf5Chunk, "moments alias s_pq");
  if constexpr (MOM) { s_mom[mh][mm] = mom; s_mom[2 + mh][mm] = momh; }
  __syncthreads();
  if (t < nd) {
    double o[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      o[c] = s_red[0][t][c];
      for (int k = 1; k < npar; ++k) o[c] = o[c] + s_red[k][t][c];
    }
    if constexpr (MOM) {
      // the covering particles: v^T Q_c v + B (2 v.L_c + B Z_c), v = (g, 1), for the DOF of thread t (dof == t,
      // in half t / 32)
      const double v[4] = {gd[0], gd[1], gd[2], 1.0}, B = gd[3];
      const int hrow = 2 + (halves == 2 ? t / 32 : 0);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double m[15];
#pragma unroll
        for (int k = 0; k < 15; ++k)
          m[k] = (s_mom[0][15 * c + k] + s_mom[1][15 * c + k]) + (halves == 2 ? s_mom[hrow][15 * c + k] : 0.0);
        const double quad = v[0] * (v[0] * m[0] + 2.0 * (v[1] * m[1] + v[2] * m[2] + v[3] * m[3])) +
                            v[1] * (v[1] * m[4] + 2.0 * (v[2] * m[5] + v[3] * m[6])) +
                            v[2] * (v[2] * m[7] + 2.0 * v[3] * m[8]) + v[3] * v[3] * m[9];
        const double lin = v[0] * m[10] + v[1] * m[11] + v[2] * m[12] + v[3] * m[13];
        o[c] = o[c] + (quad + B * (2.0 * lin + B * m[14]));
      }
    }
    double2* out = reinterpret_cast<double2*>(PS + (dof_base<N>(M, e) + t) * 4);
    out[0] = make_double2(o[0], o[1]);
    out[1] = make_double2(o[2], o[3]);
  }
}

// =============================================================================================
// Mixed shape-function gather for N = 3 with one radius, fed by a TMA bulk-copy ring.
//
// The particle records of the target's (source element, periodic image) pairs are contiguous per source
// element (the pack sorts them by element, and inside an element by 2x2x2 sub-cell), so their concatenation
// is a stream of 16-byte records (position relative to the source's DOF centre, and w q MPF (v, 1)).
// Thread 0 copies that stream into a ring of kSf7Stages shared-memory stages of kSf7Cap records with one
// cp.async.bulk per (pair, stage) segment; each stage has a "full" mbarrier (the copies complete their
// bytes on it) and an "empty" one (each of the 8 warps arrives when it is done with the stage).  The
// producer keeps kSf7Ahead fills in flight and refills a stage only after every warp released it, so warps
// may drift apart by a few fills and the global loads are never waited for by the CTA as a whole.
// The 8 warps each own one DOF octant (2x2x2 DOFs in registers).  Per stage a warp skips the sub-cells whose
// box lies beyond R + (octant radius) of its octant's centre, culls the records of the others to that
// radius (about 1.5 candidates per hit), compacts the survivors with a ballot and evaluates them
// lane-parallel without branches: with p and g relative to the target's DOF centre,
// 1 - r^2/R^2 = A_p + B_g + p'.g (A_p = 1 - |p|^2/R^2, p' = 2 p/R^2, B_g = -|g|^2/R^2), then
// S = max(., 0)^alpha and 4 fused multiply-adds: 10 FP32 instructions per pair.  Each lane sums its pairs in
// FP32 for at most kSf7Fold particles; the warp then reduce-scatters the 32 partials (8 DOFs x 4 components)
// so that lane k holds value k, which joins the lane's (hi, lo) pair through TwoSum: the FP64 result
// hi + lo carries every fold exactly, FP32 rounding stays within windows of 16 x 32 terms.
// Every wait is bounded (kMbarPolls polls); a wait that gives up sets PIC_STATUS_WAIT_TIMEOUT, the CTA
// skips the rest of its work, and thread 0 waits (bounded) for the copies it issued before it returns.
// =============================================================================================
constexpr int kSf7Warps = 8, kSf7Threads = kSf7Warps * 32;
constexpr int kSf7Stages = 4, kSf7Cap = 512, kSf7Ahead = 2;   // refill the stage released kStages-kAhead fills ago
constexpr int kSf7Pairs = 160;
constexpr int kSf7Fold = 16;
constexpr int kMbarPolls = 1 << 22;
constexpr unsigned kStatusWaitTimeout = 0x100u;               // PIC_STATUS_WAIT_TIMEOUT
static_assert(kSf7Ahead < kSf7Stages, "the producer must refill a stage released earlier");
static_assert(kSf7Cap <= 65536 && kSf7Pairs <= 65536, "compacted entries pack slot and pair in 16 bits each");

struct Sf7Smem {
  float4 pos[kSf7Stages][kSf7Cap];       // 16-byte aligned (bulk-copy destinations)
  float4 fac[kSf7Stages][kSf7Cap];
  uint32_t list[kSf7Warps][kSf7Cap];     // compacted (slot | pair << 16) per warp
  float4 off[kSf7Pairs];                 // source DOF centre + image shift - target DOF centre
  float4 blo[kSf7Pairs], bhi[kSf7Pairs]; // the source's padded particle box in the target frame
  int sub[kSf7Pairs][9];                 // first record of each sub-cell relative to the pair's first record
  int b0[kSf7Pairs], n[kSf7Pairs], g[kSf7Pairs + 1];
  uint8_t okeep[kSf7Warps][kSf7Pairs];   // per warp (octant): the pair's sub-cells within its reach
  int sp[kSf7Stages];                    // first pair of the fill a stage holds
  unsigned long long full[kSf7Stages], empty[kSf7Stages];
  int abort_flag;
};

__device__ __forceinline__ float reduce_scatter32f(float v[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool upper = (lane & h) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const float a = v[j], b = v[j + h];
      const float recv = __shfl_xor_sync(kFull, upper ? a : b, h);
      v[j] = __fadd_rn(upper ? b : a, recv);
    }
  }
  return v[0];
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase of the given parity; false after kMbarPolls polls
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (int i = 0; i < kMbarPolls; ++i)
    if (mbar_test(bar, parity)) return true;
  return false;
}
// 1D bulk copy global -> shared (TMA), completion counted in bytes on the mbarrier
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

template <bool A2>
__global__ void __launch_bounds__(kSf7Threads, 2) k_sf_gather7(const __grid_constant__ DevMesh M, SfLists L,
                                                               const int* __restrict__ off, SfPack K,
                                                               double* __restrict__ PS, DevStatus* st) {
  const Consts& kc = M.k;
  extern __shared__ __align__(128) unsigned char sf7_raw[];
  Sf7Smem& S = *reinterpret_cast<Sf7Smem*>(sf7_raw);
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int e = L.order ? __ldg(L.order + blockIdx.x) : blockIdx.x;
  const double* ce = L.dof_center + (size_t)e * 3;
  const double cex = __ldg(ce), cey = __ldg(ce + 1), cez = __ldg(ce + 2);
  const float R = (float)kc.sf_r, R2inv = (float)kc.sf_r2_inv, tR2 = 2.0f * R2inv;
  // this warp's octant: DOF (i, j, k) = (2 ox + a, 2 oy + b, 2 oz + c), r = i + 4 (j + 4 k)
  const int ox = w & 1, oy = (w >> 1) & 1, oz = w >> 2;
  float gx[8], gy[8], gz[8], bg[8];
  float lo3[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi3[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
#pragma unroll
  for (int d = 0; d < 8; ++d) {
    const int r = (2 * ox + (d & 1)) + 4 * ((2 * oy + ((d >> 1) & 1)) + 4 * (2 * oz + (d >> 2)));
    const double* g = M.sf_xgp + (dof_base<3>(M, e) + r) * 3;
    gx[d] = (float)(__ldg(g) - cex); gy[d] = (float)(__ldg(g + 1) - cey); gz[d] = (float)(__ldg(g + 2) - cez);
    bg[d] = -R2inv * fmaf(gx[d], gx[d], fmaf(gy[d], gy[d], gz[d] * gz[d]));
    lo3[0] = fminf(lo3[0], gx[d]); hi3[0] = fmaxf(hi3[0], gx[d]);
    lo3[1] = fminf(lo3[1], gy[d]); hi3[1] = fmaxf(hi3[1], gy[d]);
    lo3[2] = fminf(lo3[2], gz[d]); hi3[2] = fmaxf(hi3[2], gz[d]);
  }
  const float ocx = 0.5f * (lo3[0] + hi3[0]), ocy = 0.5f * (lo3[1] + hi3[1]), ocz = 0.5f * (lo3[2] + hi3[2]);
  float orad2 = 0.0f;
#pragma unroll
  for (int d = 0; d < 8; ++d) {
    const float dx = gx[d] - ocx, dy = gy[d] - ocy, dz = gz[d] - ocz;
    orad2 = fmaxf(orad2, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
  }
  const float ocull = R + sqrtf(orad2);
  const float ocull2 = ocull * ocull * 1.0001f;
  if (t == 0) {
    for (int q = 0; q < kSf7Stages; ++q) {
      mbar_init(&S.full[q], 1);
      mbar_init(&S.empty[q], kSf7Warps);
    }
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  float part[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) part[k] = 0.0f;
  float hi = 0.0f, lo = 0.0f;
  int since_fold = 0;
  auto fold = [&]() {
    float v = reduce_scatter32f(part);
    float sm, er;
    two_sum(hi, v, sm, er);
    hi = sm;
    lo = __fadd_rn(lo, er);
#pragma unroll
    for (int k = 0; k < 32; ++k) part[k] = 0.0f;
  };
  volatile int* abort_flag = &S.abort_flag;
  auto give_up = [&]() {
    *abort_flag = 1;
    flag_status(st, kStatusWaitTimeout);
  };
  int fill = 0;            // global fill index (fills continue across pair windows)
  int issued = 0;          // thread 0: fills issued so far
  int pc = 0;              // thread 0: first pair not yet fully copied in this window
  const int p0 = __ldg(L.nb_off + e), p1 = __ldg(L.nb_off + e + 1);
  for (int pw = p0; pw < p1; pw += kSf7Pairs) {
    const int npw = min(kSf7Pairs, p1 - pw);
    __syncthreads();                       // every warp is done with the previous window's tables
    for (int i = t; i < npw; i += kSf7Threads) {
      const int p = pw + i;
      const int src = __ldg(L.nb_src + p);
      double sh[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int k = kc.pv_dir[d];
        sh[d] = k >= 0 ? (double)L.nb_shift[3 * p + d] * kc.pv[3 * k + d] : 0.0;
      }
      const double* cs = L.dof_center + (size_t)src * 3;
      const float4 o = make_float4((float)((__ldg(cs) + sh[0]) - cex), (float)((__ldg(cs + 1) + sh[1]) - cey),
                                   (float)((__ldg(cs + 2) + sh[2]) - cez), 0.0f);
      S.off[i] = o;
      const float4 bl = __ldg(reinterpret_cast<const float4*>(L.elem_box) + 2 * (size_t)src);
      const float4 bh = __ldg(reinterpret_cast<const float4*>(L.elem_box) + 2 * (size_t)src + 1);
      S.blo[i] = make_float4(bl.x + o.x, bl.y + o.y, bl.z + o.z, 0.0f);
      S.bhi[i] = make_float4(bh.x + o.x, bh.y + o.y, bh.z + o.z, 0.0f);
      const int b0 = __ldg(K.sub_off + 8 * (size_t)src);
      S.b0[i] = b0;
#pragma unroll
      for (int c = 0; c <= 8; ++c) S.sub[i][c] = __ldg(K.sub_off + 8 * (size_t)src + c) - b0;
      S.n[i] = S.sub[i][8];
    }
    __syncthreads();
    if (t == 0) {
      S.g[0] = 0;
      for (int i = 0; i < npw; ++i) S.g[i + 1] = S.g[i] + S.n[i];
    }
    // each warp: which sub-cells of every pair come within R + (octant radius) of its octant's centre (the
    // sub-cell's box is the source's padded particle box split at the source's DOF centre o), once per window
    for (int i = lane; i < npw; i += 32) {
      const float4 o = S.off[i], bl = S.blo[i], bh = S.bhi[i];
      unsigned keep = 0;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float lx = (c & 1) ? o.x : bl.x, hx = (c & 1) ? bh.x : o.x;
        const float ly = (c & 2) ? o.y : bl.y, hy = (c & 2) ? bh.y : o.y;
        const float lz = (c & 4) ? o.z : bl.z, hz = (c & 4) ? bh.z : o.z;
        const float ex = fmaxf(fmaxf(lx - ocx, ocx - hx), 0.0f), ey = fmaxf(fmaxf(ly - ocy, ocy - hy), 0.0f),
                    ez = fmaxf(fmaxf(lz - ocz, ocz - hz), 0.0f);
        if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= ocull2 && S.sub[i][c + 1] > S.sub[i][c]) keep |= 1u << c;
      }
      S.okeep[w][i] = (uint8_t)keep;
    }
    __syncthreads();
    const int total = S.g[npw];
    const int nfill = (total + kSf7Cap - 1) / kSf7Cap;
    const int f0 = fill;
    // thread 0: issue fill jj (window-relative jj - f0) after every warp released the stage's previous fill
    auto issue = [&](int jj) {
      const int s = jj % kSf7Stages;
      if (*abort_flag) return;
      if (jj >= kSf7Stages && !mbar_wait(&S.empty[s], (unsigned)((jj / kSf7Stages) - 1) & 1u)) {
        give_up();
        return;
      }
      const int r0 = (jj - f0) * kSf7Cap, r1 = min(r0 + kSf7Cap, total);
      while (S.g[pc + 1] <= r0) ++pc;
      S.sp[s] = pc;
      mbar_arrive_expect_tx(&S.full[s], (unsigned)(r1 - r0) * 32u);
      for (int p = pc; p < npw && S.g[p] < r1; ++p) {
        const int a = max(S.g[p], r0), b = min(S.g[p + 1], r1);
        if (b > a) {
          const size_t src0 = (size_t)S.b0[p] + (size_t)(a - S.g[p]);
          bulk_g2s(&S.pos[s][a - r0], reinterpret_cast<const float4*>(K.posf) + src0, (unsigned)(b - a) * 16u, &S.full[s]);
          bulk_g2s(&S.fac[s][a - r0], reinterpret_cast<const float4*>(K.facf) + src0, (unsigned)(b - a) * 16u, &S.full[s]);
        }
      }
      issued = jj + 1;
    };
    if (t == 0) {
      pc = 0;
      for (int i = 0; i < min(nfill, kSf7Ahead); ++i) issue(f0 + i);
    }
    for (int i = 0; i < nfill; ++i) {
      const int j = f0 + i, s = j % kSf7Stages;
      if (t == 0 && i + kSf7Ahead < nfill) issue(j + kSf7Ahead);
      __syncwarp();
      if (*abort_flag) continue;
      // every lane observes the phase itself (acquire of the bulk-copied bytes); the outcome is made uniform
      if (!__all_sync(kFull, mbar_wait(&S.full[s], (unsigned)(j / kSf7Stages) & 1u))) {
        if (lane == 0) give_up();
        __syncwarp();
        continue;
      }
      const int r0 = i * kSf7Cap, r1 = min(r0 + kSf7Cap, total);
      // this warp's octant: compact the stage's records within R + octant radius of its centre.  Sub-cells
      // whose box lies beyond that reach are skipped (masks of the window); consecutive kept sub-cells form one
      // run of records, tested 4 x 32 at a time (independent shared-memory loads in flight).
      int cnt = 0;
      for (int p = S.sp[s]; p < npw && S.g[p] < r1; ++p) {
        const float4 o = S.off[p];
        unsigned keep = S.okeep[w][p];
        const float qx = o.x - ocx, qy = o.y - ocy, qz = o.z - ocz;   // record -> octant-centre frame
        const uint32_t tag = (uint32_t)p << 16;
        while (keep) {
          const int c0 = __ffs(keep) - 1;
          const int c1 = c0 + __ffs(~(keep >> c0)) - 1;                 // end of the run of kept sub-cells
          keep &= ~((c1 >= 32 ? 0u : (1u << c1)) - (1u << c0));
          const int a = max(S.g[p] + S.sub[p][c0], r0) - r0, b = min(S.g[p] + S.sub[p][c1], r1) - r0;
          for (int base = a; base < b; base += 128) {
            float4 rr[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int k = base + 32 * u + lane;
              rr[u] = k < b ? S.pos[s][k] : make_float4(3e18f, 3e18f, 3e18f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float dx = rr[u].x + qx, dy = rr[u].y + qy, dz = rr[u].z + qz;
              const bool ok = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= ocull2;
              const unsigned m = __ballot_sync(kFull, ok);
              if (ok) S.list[w][cnt + __popc(m & ((1u << lane) - 1u))] = (uint32_t)(base + 32 * u + lane) | tag;
              cnt += __popc(m);
            }
          }
        }
      }
      __syncwarp();
      // evaluation, with the next entry's records loaded while the current one is evaluated
      const int qend = (cnt + 31) & ~31;
      float4 rn = make_float4(0.f, 0.f, 0.f, 0.f), on = rn, fn = rn;
      bool vn = false;
      if (lane < cnt) {
        const uint32_t v = S.list[w][lane];
        rn = S.pos[s][v & 0xFFFFu]; on = S.off[v >> 16]; fn = S.fac[s][v & 0xFFFFu];
        vn = true;
      }
      for (int q = lane; q < qend; q += 32) {
        const float4 r = rn, o = on, f = vn ? fn : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool valid = vn;
        vn = false;
        if (q + 32 < cnt) {
          const uint32_t v = S.list[w][q + 32];
          rn = S.pos[s][v & 0xFFFFu]; on = S.off[v >> 16]; fn = S.fac[s][v & 0xFFFFu];
          vn = true;
        }
        const float x = r.x + o.x, y = r.y + o.y, z = r.z + o.z;
        const float A = valid ? fmaf(-R2inv, fmaf(x, x, fmaf(y, y, z * z)), 1.0f) : -1.0f;
        const float px = valid ? tR2 * x : 0.f, py = valid ? tR2 * y : 0.f, pz = valid ? tR2 * z : 0.f;
#pragma unroll
        for (int d = 0; d < 8; ++d) {
          const float Sv = fmaxf(fmaf(pz, gz[d], fmaf(py, gy[d], fmaf(px, gx[d], bg[d]))) + A, 0.0f);
          const float S1 = sf_power<A2>(kc, Sv);
          part[4 * d] = fmaf(S1, f.x, part[4 * d]);
          part[4 * d + 1] = fmaf(S1, f.y, part[4 * d + 1]);
          part[4 * d + 2] = fmaf(S1, f.z, part[4 * d + 2]);
          part[4 * d + 3] = fmaf(S1, f.w, part[4 * d + 3]);
        }
        if (++since_fold == kSf7Fold) {    // warp-uniform: every lane runs the same iterations
          fold();
          since_fold = 0;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.empty[s]);
    }
    fill = f0 + nfill;
  }
  if (*abort_flag) {
    // give the copies this CTA issued time to land before its shared memory goes away
    if (t == 0)
      for (int jj = max(issued - kSf7Stages, 0); jj < issued; ++jj)
        (void)mbar_wait(&S.full[jj % kSf7Stages], (unsigned)(jj / kSf7Stages) & 1u);
    return;
  }
  fold();
  // lane k holds value k = 4 d + c of this octant
  const int dl = lane >> 2;
  const int r_out = (2 * ox + (dl & 1)) + 4 * ((2 * oy + ((dl >> 1) & 1)) + 4 * (2 * oz + (dl >> 2)));
  PS[(dof_base<3>(M, e) + r_out) * 4 + (lane & 3)] = (double)hi + (double)lo;
}

// =============================================================================================
// shape_function_cc normalisation (calcSfSource:96-120 with calcTotalChargePeriodic_cc:425-555).
// One CTA per source element, one thread per packed particle of it.  Per round the CTA stages the DOFs
// of four (target, image) pairs of the source, taken at stride npairs/4 so that they lie on different
// sides (a single target leaves the particles on the far side of the source idle): each DOF shifted back
// by the image (FP64, with the weight wGP^3/sJ) and its FP32 position relative to the source's DOF
// centre.  Each thread tests its particle in FP32 against (1+1e-4) R^2 into a hit list, then evaluates
// the hits exactly (FP64: r^2 <= R^2 and (1 - r^2/R^2)^alpha wGP^3/sJ; mixed: FP32).  The packed Fac (q MPF (v,1)) is multiplied by
// 1/sum, i.e. Fac * Fac(4) / totalCharge of the reference up to rounding.
// =============================================================================================
constexpr int kCcThreads = 128;
// pairs staged per round (taken at stride npairs/round: targets on all sides); 2 for N = 4 (48 KB smem)
template <int N>
__host__ __device__ constexpr int cc_round() { return (N + 1) * (N + 1) * (N + 1) > 64 ? 2 : 4; }
constexpr int kCcCap = 256;       // hit-list entries per thread: a whole round (ns <= 256), so no lane flushes alone

template <int N, bool MIXED, bool A2>
__device__ __forceinline__ void cc_eval(const Consts& kc, const double (*s_g)[5], const float4* s_gf, const uint8_t (*s_list)[kCcThreads],
                                        int nh, const double p[4], const float pf[3], double R2, double R2inv,
                                        double& acc, float& accf) {
  const int t = threadIdx.x;
  for (int k = 0; k < nh; ++k) {
    const int d = s_list[k][t];
    if constexpr (MIXED) {
      const float4 g = s_gf[d];
      const float dx = pf[0] - g.x, dy = pf[1] - g.y, dz = pf[2] - g.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (r2 <= (float)R2) {
        const float Sv = fmaf(-(float)R2inv, r2, 1.0f);
        accf = fmaf(g.w, sf_power<A2>(kc, Sv), accf);
      }
    } else {
      // 1 - |p-g|^2/R^2 = A_p + p'.g + B_g (p' = 2p/R^2, A_p = 1 - |p|^2/R^2, B_g = -|g|^2/R^2, all relative to
      // the source's DOF centre): one add and three fused multiply-adds; r^2 <= R^2 read from the sign
      const double Sv = fma(p[0], s_g[d][0], fma(p[1], s_g[d][1], fma(p[2], s_g[d][2], p[3] + s_g[d][4])));
      if (__double_as_longlong(Sv) >= 0) acc = fma(s_g[d][3], sf_power<A2>(kc, Sv), acc);
    }
  }
}

template <int N, bool MIXED, bool A2>
__global__ void __launch_bounds__(kCcThreads) k_sf_cc_norm(const __grid_constant__ DevMesh M, SfLists L, const int* __restrict__ off, SfPack K,
                                                           DevStatus* st) {
  const Consts& kc = M.k;
  constexpr int n1 = N + 1, nd = n1 * n1 * n1, ns = cc_round<N>() * nd;
  __shared__ double s_g[MIXED ? 1 : ns][5];     // DOF position minus the image shift, relative to the source's
                                                // DOF centre; wGP^3/sJ; -|g|^2/R^2
  __shared__ float4 s_gf[ns];                   // FP32 position relative to the source's DOF centre; w = weight
  __shared__ uint8_t s_list[kCcCap][kCcThreads];
  static_assert(ns <= kCcCap, "a round's DOFs must fit one hit list");
  const int s = L.order ? __ldg(L.order + blockIdx.x) : blockIdx.x;
  const int t = threadIdx.x;
  const int b0 = __ldg(off + s), cnt = __ldg(off + s + 1) - b0;
  const double* cs = L.dof_center + (size_t)s * 3;
  const double csx = __ldg(cs), csy = __ldg(cs + 1), csz = __ldg(cs + 2);
  // radius of the source element (shape_function_adaptive) or the global one
  double R2 = kc.sf_r2, R2inv = kc.sf_r2_inv;
  if (L.elem_r) { const double r = __ldg(L.elem_r + s); R2 = r * r; R2inv = 1.0 / R2; }
  const float R2f = (float)(R2 * (1.0 + 1.0e-4));
  const int q0 = __ldg(L.t_off + s), npair = __ldg(L.t_off + s + 1) - q0;
  const int stride = (npair + cc_round<N>() - 1) / cc_round<N>();
  for (int base = 0; base < cnt; base += kCcThreads) {
    const int j = b0 + base + t;
    const bool act = base + t < cnt;
    double p[4] = {0.0, 0.0, 0.0, 0.0};           // FP64: p' = 2p/R^2 and A_p = 1 - |p|^2/R^2
    float pf[3] = {0.f, 0.f, 0.f};
    if (act) {
      const float4 r = reinterpret_cast<const float4*>(K.posf)[j];     // relative to the source DOF centre
      pf[0] = r.x; pf[1] = r.y; pf[2] = r.z;
      if constexpr (!MIXED) {
        const double px = K.pos[3 * (size_t)j] - csx, py = K.pos[3 * (size_t)j + 1] - csy,
                     pz = K.pos[3 * (size_t)j + 2] - csz;
        const double t2 = 2.0 * R2inv;
        p[0] = px * t2; p[1] = py * t2; p[2] = pz * t2;
        p[3] = fma(-R2inv, fma(px, px, fma(py, py, pz * pz)), 1.0);
      }
    }
    double acc = 0.0;
    float accf = 0.f;
    for (int r = 0; r < stride; ++r) {
      __syncthreads();                          // the previous round's DOFs are no longer read
      for (int i = t; i < ns; i += kCcThreads) {
        const int kq = i / nd, d = i - kq * nd, pi = r + kq * stride;
        if (pi >= npair) { s_gf[i] = make_float4(1e30f, 1e30f, 1e30f, 0.0f); continue; }   // never a hit
        const int q = q0 + pi;
        const int e = __ldg(L.t_tgt + q);
        if (M.elem_n) {          // p-adaption: slots beyond the target's (Nloc+1)^3 DOFs hold no DOF
          const int nl1 = __ldg(M.elem_n + e) + 1;
          if (d >= nl1 * nl1 * nl1) { s_gf[i] = make_float4(1e30f, 1e30f, 1e30f, 0.0f); continue; }
        }
        double sh[3];
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
          const int k = kc.pv_dir[dd];
          sh[dd] = k >= 0 ? (double)L.t_shift[3 * q + dd] * kc.pv[3 * k + dd] : 0.0;
        }
        const double* g = M.sf_xgp + (dof_base<N>(M, e) + d) * 3;
        const double gx = __ldg(g) - sh[0], gy = __ldg(g + 1) - sh[1], gz = __ldg(g + 2) - sh[2];
        const double wgt = __ldg(L.dof_w + dof_base<N>(M, e) + d);
        const double rx = gx - csx, ry = gy - csy, rz = gz - csz;
        if constexpr (!MIXED) {
          s_g[i][0] = rx; s_g[i][1] = ry; s_g[i][2] = rz; s_g[i][3] = wgt;
          s_g[i][4] = -R2inv * fma(rx, rx, fma(ry, ry, rz * rz));
        }
        s_gf[i] = make_float4((float)rx, (float)ry, (float)rz, (float)wgt);
      }
      __syncthreads();
      if (!act) continue;
      int nh = 0;
      for (int i = 0; i < ns; ++i) {
        const float4 g = s_gf[i];
        const float dx = pf[0] - g.x, dy = pf[1] - g.y, dz = pf[2] - g.z;
        if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= R2f) s_list[nh++][t] = (uint8_t)i;
      }
      cc_eval<N, MIXED, A2>(kc, s_g, s_gf, s_list, nh, p, pf, R2, R2inv, acc, accf);
    }
    if (act) {
      const double tot = (MIXED ? (double)accf : acc) / kc.sf_cc_div;
      const bool ok = tot > 0.0;
      // no DOF within R: with periodic images the reference divides by zero (calcSfSource:122); without,
      // it deposits nothing (nUsedElems = 0), as the zero scale does here
      if (!ok && kc.n_pv > 0) flag_status(st, 0x20u);
      const double sc = ok ? 1.0 / tot : 0.0;
      if constexpr (MIXED) {
        float4* f = reinterpret_cast<float4*>(K.facf) + j;
        const float4 v = *f;
        const float scf = (float)sc;
        *f = make_float4(v.x * scf, v.y * scf, v.z * scf, v.w * scf);
      } else {
        double2* f = reinterpret_cast<double2*>(K.fac + 4 * (size_t)j);
        const double2 a = f[0], b = f[1];
        f[0] = make_double2(a.x * sc, a.y * sc);
        f[1] = make_double2(b.x * sc, b.y * sc);
      }
    }
  }
}

// =============================================================================================
// Fused remainder for RefTracking: interpolation at PartPosRef + push + RefTracking
// =============================================================================================
// resident CTAs per SM the RefTracking step is compiled for (FP64 / mixed): 2 x 256 threads caps it at 128
// registers (no spills); against 1 CTA/SM (170 registers) 62.4 vs 64.1 ms (FP64) and 14.0 vs 16.0 ms (mixed)
// per step at 32^3 / 16M particles
#ifndef PIC_REF_MINB
#define PIC_REF_MINB 2
#endif
#ifndef PIC_REF_MIXED_MINB
#define PIC_REF_MIXED_MINB 2
#endif
template <int N, bool MIXED>
__global__ void __launch_bounds__(256, MIXED ? PIC_REF_MIXED_MINB : PIC_REF_MINB) k_step_ref(const __grid_constant__ DevMesh M, DevParticles P, const double* __restrict__ E,
                                                  const float* __restrict__ E32, double dt, DevStatus* st) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = P.flags[i];
  if (!(fl & kInside)) return;
  const int sp = P.species[i];
  const bool charged = kc.q[sp] != 0.0;
  const int e = P.elem[i];
  double x[3] = {P.x[i], P.y[i], P.z[i]};
  double xi[3] = {P.xi0[i], P.xi1[i], P.xi2[i]};
  bool isnew = (fl & kNew) != 0;
  if constexpr (!MIXED) {
    double F[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) F[c] = kc.ext[c];
    if (charged) {
      double Eo[3];
      field_at<N>(M, E, e, xi, Eo);
#pragma unroll
      for (int c = 0; c < 3; ++c) F[c] = F[c] + Eo[c];
    }
    double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
    const double dtv = dt * kc.dt_fac[sp];
    boris_push(kc, v, F, sp, isnew, dtv);
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = x[c] + v[c] * dtv;
    P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2];
  } else {
    float F[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) F[c] = (float)kc.ext[c];
    if (charged) {
      float Eo[3];
      const float xf[3] = {(float)xi[0], (float)xi[1], (float)xi[2]};
      field_at_f<N>(M, E32, e, xf, Eo);
#pragma unroll
      for (int c = 0; c < 3; ++c) F[c] += Eo[c];
    }
    float v[3] = {P.vxf[i], P.vyf[i], P.vzf[i]};
    const double dtv = dt * kc.dt_fac[sp];
    boris_push_f(kc, v, F, sp, isnew, (float)dtv);
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = x[c] + (double)v[c] * dtv;
    P.vxf[i] = v[0]; P.vyf[i] = v[1]; P.vzf[i] = v[2];
  }
  double xl[3] = {P.x[i], P.y[i], P.z[i]};
  const bool finite = MIXED ? state_finite(x, P.vxf[i], P.vyf[i], P.vzf[i]) : state_finite(x, P.vx[i], P.vy[i], P.vz[i]);
  if (!finite) {
    flag_status(st, 0x20u);
    P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
    P.flags[i] = (isnew ? (fl | kNew) : (fl & ~kNew)) & ~kInside;
    return;
  }
  bool tol = false, removed = false, cap = false;
  double v[3];
  if constexpr (MIXED) { v[0] = P.vxf[i]; v[1] = P.vyf[i]; v[2] = P.vzf[i]; }
  else { v[0] = P.vx[i]; v[1] = P.vy[i]; v[2] = P.vz[i]; }
  const int ne = ref_track<MIXED>(M, e, x, xl, xi, v, tol, removed, cap);
  if (tol) { atomicAdd(&st->n_ref_tolerance, 1); flag_status(st, 0x08u); }
  if (cap) flag_status(st, 0x04u);
  if (M.bc_e2b) {                                   // reflective walls change v
    if constexpr (MIXED) { P.vxf[i] = (float)v[0]; P.vyf[i] = (float)v[1]; P.vzf[i] = (float)v[2]; }
    else { P.vx[i] = v[0]; P.vy[i] = v[1]; P.vz[i] = v[2]; }
  }
  P.x[i] = x[0]; P.y[i] = x[1]; P.z[i] = x[2];
  P.xi0[i] = xi[0]; P.xi1[i] = xi[1]; P.xi2[i] = xi[2];
  P.elem[i] = ne;
  const uint8_t f2 = isnew ? (fl | kNew) : (fl & ~kNew);
  P.flags[i] = removed ? (f2 & ~kInside) : f2;
}

// =============================================================================================
// Reorder the particle arrays by element (counting-sort scatter)
// =============================================================================================
template <bool MIXED>
__global__ void __launch_bounds__(256) k_reorder(DevParticles P, DevParticles Q, const int* __restrict__ perm_in,
                                                 int* __restrict__ perm_out, int* __restrict__ cursor, int ne) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < P.n;
  const uint8_t fl = valid ? P.flags[i] : 0;
  const int key = (fl & kInside) ? P.elem[i] : ne;
  const int j = warp_slot(cursor, key, valid);
  if (!valid) return;
  Q.x[j] = P.x[i]; Q.y[j] = P.y[i]; Q.z[j] = P.z[i];
  if constexpr (!MIXED) { Q.vx[j] = P.vx[i]; Q.vy[j] = P.vy[i]; Q.vz[j] = P.vz[i]; }
  else { Q.vxf[j] = P.vxf[i]; Q.vyf[j] = P.vyf[i]; Q.vzf[j] = P.vzf[i]; }
  Q.xi0[j] = P.xi0[i]; Q.xi1[j] = P.xi1[i]; Q.xi2[j] = P.xi2[i];
  Q.elem[j] = P.elem[i];
  Q.last_elem[j] = P.last_elem[i];
  Q.species[j] = P.species[i];
  Q.flags[j] = fl;
  perm_out[j] = perm_in[i];
}

__global__ void __launch_bounds__(256) k_map_particles(const __grid_constant__ DevMesh M, DevParticles P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  if (!(P.flags[i] & kInside)) return;
  const double x[3] = {P.x[i], P.y[i], P.z[i]};
  double xi[3];
  position_in_ref_elem(M, P.elem[i], x, xi);
  P.xi0[i] = xi[0]; P.xi1[i] = xi[1]; P.xi2[i] = xi[2];
}

__global__ void k_count_inside(DevParticles P, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int v = (i < P.n && (P.flags[i] & kInside)) ? 1 : 0;
  v = __reduce_add_sync(kFull, v);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

// VerifyDepositedCharge (pic_analyze.f90:72-91; the change of basis to NAnalyze is left out: for Gauss nodes the
// N+1-point rule already integrates PartSource(4)/sJ, a product of two degree-N interpolants, exactly).  One warp
// per element sums w * PartSource(4) over its DOFs; one block then adds the element sums in index order, so the
// result does not depend on scheduling.
// dof_off: the elements' DOF offsets on a p-adapted mesh (else null: nd DOFs each)
__global__ void __launch_bounds__(256) k_charge_elem(const double* __restrict__ PS, const double* __restrict__ w, int ne,
                                                     int nd, const int* __restrict__ dof_off, double* __restrict__ elem_sum) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (e >= ne) return;
  const size_t b = dof_off ? (size_t)__ldg(dof_off + e) : (size_t)e * nd;
  const int nde = dof_off ? __ldg(dof_off + e + 1) - __ldg(dof_off + e) : nd;
  double s = 0.0;
  for (int r = lane; r < nde; r += 32) s = s + __ldg(w + b + r) * __ldg(PS + (b + r) * 4 + 3);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = s + __shfl_down_sync(kFull, s, o);
  if (lane == 0) elem_sum[e] = s;
}

__global__ void __launch_bounds__(1024) k_sum_ordered(const double* __restrict__ a, int n, double* __restrict__ out) {
  __shared__ double part[1024];
  const int t = threadIdx.x;
  const int per = (n + 1023) / 1024, b = t * per, end = min(n, b + per);
  double s = 0.0;
  for (int i = b; i < end; ++i) s = s + a[i];
  part[t] = s;
  __syncthreads();
  for (int h = 512; h > 0; h >>= 1) {
    if (t < h) part[t] = part[t] + part[t + h];
    __syncthreads();
  }
  if (t == 0) *out = part[0];
}

__global__ void k_count_species(DevParticles P, int* __restrict__ counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n || !(P.flags[i] & kInside)) return;
  atomicAdd(counts + P.species[i], 1);
}

// =============================================================================================
// launch wrappers
// =============================================================================================
static inline int nblk(int n, int b) { return (n + b - 1) / b; }

#define PIC_DISPATCH_N(Nv, ...)                               \
  switch (Nv) {                                               \
    case 1: { constexpr int NN = 1; __VA_ARGS__; } break;     \
    case 2: { constexpr int NN = 2; __VA_ARGS__; } break;     \
    case 3: { constexpr int NN = 3; __VA_ARGS__; } break;     \
    case 4: { constexpr int NN = 4; __VA_ARGS__; } break;     \
    default: break;                                           \
  }
// the same for kernels with a per-element-degree instance (NN = 0 on p-adapted meshes)
#define PIC_DISPATCH_NV(A, ...)                                             \
  if ((A).M.dof_off) { constexpr int NN = 0; __VA_ARGS__; }                 \
  else { PIC_DISPATCH_N((A).N, __VA_ARGS__); }

// Mixed variant of node -> DOF: the node sums stay FP64; NodeSource / NodeVolume and the trilinear node ->
// DOF weights (deposition weights) in FP32, one kernel; PartSource written in FP64.
// N = 0 (p-adaption): as k_node_to_dof, each element with its own degree.
template <int N>
__global__ void __launch_bounds__(256) k_node_to_dof_f(const __grid_constant__ DevMesh M, const double* __restrict__ NS, double* __restrict__ PS) {
  const Consts& kc = M.k;
  const int nmax1 = N > 0 ? N + 1 : kc.N + 1, ndmax = nmax1 * nmax1 * nmax1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.ne * ndmax) return;
  const int e = t / ndmax, r = t - e * ndmax;
  const int nl = N > 0 ? N : __ldg(M.elem_n + e), n1 = nl + 1;
  if (r >= n1 * n1 * n1) return;
  const float a1 = (float)kc.fac_n[nl][r % n1], a2 = (float)kc.fac_n[nl][(r / n1) % n1],
              a3 = (float)kc.fac_n[nl][r / (n1 * n1)];
  const float w[8] = {(1 - a1) * (1 - a2) * (1 - a3), a1 * (1 - a2) * (1 - a3), a1 * a2 * (1 - a3), (1 - a1) * a2 * (1 - a3),
                      (1 - a1) * (1 - a2) * a3,       a1 * (1 - a2) * a3,       a1 * a2 * a3,       (1 - a1) * a2 * a3};
  float out[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int node = __ldg(M.canon_node + (size_t)e * 8 + n);
    const double V = __ldg(M.node_vol + node);
    const float s = V > 0.0 ? w[n] / (float)V : w[n];
    const double2 a = __ldg(reinterpret_cast<const double2*>(NS + (size_t)node * 4));
    const double2 b = __ldg(reinterpret_cast<const double2*>(NS + (size_t)node * 4) + 1);
    out[0] = fmaf((float)a.x, s, out[0]);
    out[1] = fmaf((float)a.y, s, out[1]);
    out[2] = fmaf((float)b.x, s, out[2]);
    out[3] = fmaf((float)b.y, s, out[3]);
  }
  double2* o = reinterpret_cast<double2*>(PS + (N > 0 ? (size_t)t : dof_base<0>(M, e) + r) * 4);
  o[0] = make_double2(out[0], out[1]);
  o[1] = make_double2(out[2], out[3]);
}

int launch_node_to_dof(const LaunchArgs& A, double* PS) {
  // A.nd = (NMax+1)^3: on a p-adapted mesh the NN = 0 instance skips each element's DOFs beyond its degree
  if (A.mixed) {
    PIC_DISPATCH_NV(A, { k_node_to_dof_f<NN><<<nblk(A.M.ne * A.nd, 256), 256, 0, A.s>>>(A.M, A.NS, PS); });
    return 1;
  }
  k_node_normalize<<<nblk(A.n_canon * 4, 256), 256, 0, A.s>>>(A.M.node_vol, A.NS, A.n_canon);
  PIC_DISPATCH_NV(A, { k_node_to_dof<NN, true><<<nblk(A.M.ne * A.nd, 256), 256, 0, A.s>>>(A.M, A.NS, PS); });
  return 2;
}

int launch_cvwm_fused(const LaunchArgs& A, const DevParticles& P, double dt) {
  cudaMemsetAsync(A.NS, 0, sizeof(double) * 4 * (size_t)A.n_canon, A.s);
  if (P.n <= 0) return 0;
  PIC_DISPATCH_NV(A, {
    if (A.mixed) k_step_cvwm_tria<NN, true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, A.MF, P, A.E, A.E32, A.NS, dt, A.st);
    else k_step_cvwm_tria<NN, false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, A.MF, P, A.E, A.E32, A.NS, dt, A.st);
  });
  return 1;
}

int launch_step_cvwm_tria(const LaunchArgs& A, const DevParticles& P, double* PS, double dt) {
  int launches = launch_cvwm_fused(A, P, dt);
  if (PS) launches += launch_node_to_dof(A, PS);
  return launches;
}

int launch_interpolate(const LaunchArgs& A, const DevParticles& P, bool refmap, bool cvwm) {
  if (P.n <= 0) return 0;
  PIC_DISPATCH_NV(A, {
    if (A.mixed) k_interpolate<NN, true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, A.MF, P, A.E, A.E32, A.st, refmap, cvwm);
    else k_interpolate<NN, false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, A.MF, P, A.E, A.E32, A.st, refmap, cvwm);
  });
  return 1;
}

int launch_push(const LaunchArgs& A, const DevParticles& P, double dt) {
  if (P.n <= 0) return 0;
  if (A.mixed) k_push<true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M.k, P, dt, A.st);
  else k_push<false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M.k, P, dt, A.st);
  return 1;
}

int launch_track(const LaunchArgs& A, const DevParticles& P, bool refmap) {
  if (P.n <= 0) return 0;
  if (refmap && A.mixed) k_track_ref<true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P, A.st);
  else if (refmap) k_track_ref<false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P, A.st);
  else if (A.mixed) k_track_tria<true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P, A.st);
  else k_track_tria<false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P, A.st);
  return 1;
}

int launch_deposit_cvwm(const LaunchArgs& A, const DevParticles& P, double* PS) {
  int launches = 0;
  cudaMemsetAsync(A.NS, 0, sizeof(double) * 4 * (size_t)A.n_canon, A.s);
  if (P.n > 0) {
    if (A.mixed) k_deposit_cvwm<true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, A.MF, P, A.NS, A.st);
    else k_deposit_cvwm<false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, A.MF, P, A.NS, A.st);
    launches++;
  }
  return launches + launch_node_to_dof(A, PS);
}

int launch_sort_offsets(const LaunchArgs& A, const DevParticles& P, const SortBuffers& B) {
  cudaMemsetAsync(B.count, 0, sizeof(int) * (B.ne + 1), A.s);
  if (P.n > 0) k_hist<<<nblk(P.n, 256), 256, 0, A.s>>>(P, B.count, B.ne);
  k_scan<<<1, 1024, 0, A.s>>>(B.count, B.offset, B.cursor, B.ne + 1);
  return P.n > 0 ? 2 : 1;
}

int launch_sf_pack(const LaunchArgs& A, const DevParticles& P, const SortBuffers& B, const SfLists& L, const SfPack& K) {
  if (L.elem_box) {
    // (element, sub-cell) bins: sub-cell histogram, element counts and offsets (B, as the other kernels read
    // them), then the sub-cell offsets and cursors inside each element
    const int ne = B.ne;
    cudaMemsetAsync(K.sub_count, 0, sizeof(int) * (8 * (size_t)ne + 1), A.s);
    if (P.n > 0) k_hist8<<<nblk(P.n, 256), 256, 0, A.s>>>(A.M.k, P, L.dof_center, K.sub_count, ne);
    k_sum8<<<nblk(ne + 1, 256), 256, 0, A.s>>>(K.sub_count, B.count, ne);
    k_scan<<<1, 1024, 0, A.s>>>(B.count, B.offset, B.cursor, ne + 1);
    k_sub_offsets<<<nblk(ne + 1, 256), 256, 0, A.s>>>(K.sub_count, B.offset, K.sub_off, K.sub_cursor, ne);
    if (P.n > 0) k_sf_pack<true, true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M.k, P, K.sub_cursor, L.dof_center, K);
    return P.n > 0 ? 5 : 3;
  }
  int launches = launch_sort_offsets(A, P, B);
  if (P.n > 0) {
    if (A.mixed) k_sf_pack<true, false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M.k, P, B.cursor, L.dof_center, K);
    else k_sf_pack<false, false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M.k, P, B.cursor, L.dof_center, K);
    launches++;
  }
  return launches;
}

// Shape-function gather variant for N <= 3 (compile-time choice, 5 by default): 5 = round-robin staging,
// one DOF per lane; 2 = staging one source element at a time, one DOF per lane.
#ifndef PIC_SF_GATHER
#define PIC_SF_GATHER 5
#endif

// ntgt target elements: L.order[0 .. ntgt), all of degree N
template <int N, bool MIXED>
static void launch_gather_n(const LaunchArgs& A, const SortBuffers& B, const SfLists& L, const SfPack& K, double* PS,
                            int ntgt) {
  if constexpr (N >= 4) {   // nd > 64: one thread per DOF, single phase
    if (MIXED) k_sf_gather_mixed<N><<<ntgt, SfShape<N>::threads, 0, A.s>>>(A.M, L, B.offset, K, PS);
    else k_sf_gather_fp64<N><<<ntgt, SfShape<N>::threads, 0, A.s>>>(A.M, L, B.offset, K, PS);
    return;
  } else {
#if PIC_SF_GATHER == 5
  if constexpr (N == 3 && MIXED) {
    // one radius: octant warps fed by the bulk-copy ring (sub-cell culling, no hit lists)
    if (!L.elem_r && L.elem_box) {
      const bool a2 = A.sf_alpha == 2;     // the attribute is per device: set it at every launch (cheap)
      if (a2) cudaFuncSetAttribute(k_sf_gather7<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sf7Smem));
      else cudaFuncSetAttribute(k_sf_gather7<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sf7Smem));
      if (a2) k_sf_gather7<true><<<ntgt, kSf7Threads, sizeof(Sf7Smem), A.s>>>(A.M, L, B.offset, K, PS, A.st);
      else k_sf_gather7<false><<<ntgt, kSf7Threads, sizeof(Sf7Smem), A.s>>>(A.M, L, B.offset, K, PS, A.st);
      return;
    }
  }
  if (L.elem_r) k_sf_gather5<N, MIXED, true, false><<<ntgt, kSf5Threads, 0, A.s>>>(A.M, L, B.offset, K, PS);
  else if (A.sf_alpha == 2) k_sf_gather5<N, MIXED, false, true><<<ntgt, kSf5Threads, 0, A.s>>>(A.M, L, B.offset, K, PS);
  else k_sf_gather5<N, MIXED, false, false><<<ntgt, kSf5Threads, 0, A.s>>>(A.M, L, B.offset, K, PS);
#else
  k_sf_gather2<N, MIXED><<<ntgt, kSf2Threads, 0, A.s>>>(A.M, L, B.offset, K, PS);
#endif
  }
}

int launch_sf_cc_norm(const LaunchArgs& A, const SortBuffers& B, const SfLists& L, const SfPack& K) {
  PIC_DISPATCH_N(A.N, {
    if (A.sf_alpha == 2) {
      if (A.mixed) k_sf_cc_norm<NN, true, true><<<A.M.ne, kCcThreads, 0, A.s>>>(A.M, L, B.offset, K, A.st);
      else k_sf_cc_norm<NN, false, true><<<A.M.ne, kCcThreads, 0, A.s>>>(A.M, L, B.offset, K, A.st);
    } else {
      if (A.mixed) k_sf_cc_norm<NN, true, false><<<A.M.ne, kCcThreads, 0, A.s>>>(A.M, L, B.offset, K, A.st);
      else k_sf_cc_norm<NN, false, false><<<A.M.ne, kCcThreads, 0, A.s>>>(A.M, L, B.offset, K, A.st);
    }
  });
  return 1;
}

int sf_gather_variant() { return PIC_SF_GATHER; }

// FP64 fused multiply-add throughput probe: 8 independent chains per thread keep the FP64 pipe busy;
// the result is stored only if it is non-finite, so the chains cannot be removed.
__global__ void __launch_bounds__(256) k_fp64_fma_probe(int iters, double b, double c, double* sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (!isfinite(s)) sink[blockIdx.x] = s;
}

double fp64_fma_rate(cudaStream_t st, double* sink, int sms) {
  const int blocks = sms * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma_probe<<<blocks, 256, 0, st>>>(iters / 8, 0.9999999, 1e-7, sink);     // warm-up
  cudaEventRecord(e0, st);
  k_fp64_fma_probe<<<blocks, 256, 0, st>>>(iters, 0.9999999, 1e-7, sink);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;
  return ms > 0.f ? flops / (ms * 1e-3) / 1e9 : 0.0;
}

// FP32 counterpart: independent fmaf chains (16 per thread), the peak the FP32 work of the mixed kernels is
// compared against
__global__ void __launch_bounds__(256) k_fp32_fma_probe(int iters, float b, float c, float* sink) {
  float a[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = 1.0f + 1e-3f * (float)(threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 16; ++k) s += a[k];
  if (!isfinite(s)) sink[blockIdx.x] = s;
}

double fp32_fma_rate(cudaStream_t st, float* sink, int sms) {
  const int blocks = sms * 8, iters = 8192;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp32_fma_probe<<<blocks, 256, 0, st>>>(iters / 8, 0.9999999f, 1e-7f, sink);     // warm-up
  cudaEventRecord(e0, st);
  k_fp32_fma_probe<<<blocks, 256, 0, st>>>(iters, 0.9999999f, 1e-7f, sink);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 16.0 * (double)iters * 256.0 * (double)blocks;
  return ms > 0.f ? flops / (ms * 1e-3) / 1e9 : 0.0;
}

int launch_sf_gather(const LaunchArgs& A, const SortBuffers& B, const SfLists& L, const SfPack& K, double* PS) {
  if (!A.M.dof_off) {
    PIC_DISPATCH_N(A.N, {
      if (A.mixed) launch_gather_n<NN, true>(A, B, L, K, PS, A.M.ne);
      else launch_gather_n<NN, false>(A, B, L, K, PS, A.M.ne);
    });
    return 1;
  }
  // p-adapted mesh: one launch per degree over that degree's targets
  int launches = 0;
  for (int k = 1; k <= kMaxN; ++k) {
    const int ntgt = L.grp_off[k + 1] - L.grp_off[k];
    if (ntgt <= 0) continue;
    SfLists Lk = L;
    Lk.order = L.order + L.grp_off[k];
    PIC_DISPATCH_N(k, {
      if (A.mixed) launch_gather_n<NN, true>(A, B, Lk, K, PS, ntgt);
      else launch_gather_n<NN, false>(A, B, Lk, K, PS, ntgt);
    });
    ++launches;
  }
  return launches;
}

int launch_deposit_sf(const LaunchArgs& A, const DevParticles& P, const SortBuffers& B, const SfLists& L,
                      const SfPack& K, double* PS) {
  return launch_sf_pack(A, P, B, L, K) + launch_sf_gather(A, B, L, K, PS);
}

int launch_step_ref(const LaunchArgs& A, const DevParticles& P, double dt) {
  if (P.n <= 0) return 0;
  PIC_DISPATCH_NV(A, {
    if (A.mixed) k_step_ref<NN, true><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P, A.E, A.E32, dt, A.st);
    else k_step_ref<NN, false><<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P, A.E, A.E32, dt, A.st);
  });
  return 1;
}

int launch_reorder(const LaunchArgs& A, DevParticles& P, DevParticles& Q, int* perm, int* perm_tmp,
                   const SortBuffers& B) {
  if (P.n <= 0) return 0;
  int launches = launch_sort_offsets(A, P, B);
  if (A.mixed) k_reorder<true><<<nblk(P.n, 256), 256, 0, A.s>>>(P, Q, perm, perm_tmp, B.cursor, B.ne);
  else k_reorder<false><<<nblk(P.n, 256), 256, 0, A.s>>>(P, Q, perm, perm_tmp, B.cursor, B.ne);
  return launches + 1;
}

int launch_map_particles(const LaunchArgs& A, const DevParticles& P) {
  if (P.n <= 0) return 0;
  k_map_particles<<<nblk(P.n, 256), 256, 0, A.s>>>(A.M, P);
  return 1;
}


int launch_charge_integral(const LaunchArgs& A, const double* PS, const double* w, double* elem_sum, double* out) {
  const int ne = A.M.ne;
  k_charge_elem<<<nblk(ne * 32, 256), 256, 0, A.s>>>(PS, w, ne, A.nd, A.M.dof_off, elem_sum);
  k_sum_ordered<<<1, 1024, 0, A.s>>>(elem_sum, ne, out);
  return 2;
}

int launch_count_species(const LaunchArgs& A, const DevParticles& P, int* counts) {
  cudaMemsetAsync(counts, 0, sizeof(int) * 8, A.s);
  if (P.n <= 0) return 0;
  k_count_species<<<nblk(P.n, 256), 256, 0, A.s>>>(P, counts);
  return 1;
}

int launch_count_inside(const LaunchArgs& A, const DevParticles& P, int* out) {
  cudaMemsetAsync(out, 0, sizeof(int), A.s);
  if (P.n <= 0) return 0;
  k_count_inside<<<nblk(P.n, 256), 256, 0, A.s>>>(P, out);
  return 1;
}

}  // namespace pic
