// pic_hdg.cu -- PICLas's linear HDG Poisson solve (src/hdg/) on the device, FP64.
//
// Layout in HBM (element-major, the reference's Fortran order inside each element):
//   ehat  [e][6][nv][nf]       Ehat(1:nf,1:nv,1:6)              (elem_mat.f90:193-226)
//   invd  [e][nv][nv]          InvDhat (symmetric)                (elem_mat.f90:262-268)
//   smat  [e][6 jS][6 iS][nf][nf]  Smat(a,b,iS,jS) at a + nf*(b + nf*(iS + 6*jS))
//   pre   [side][nf][nf] upper Cholesky factor (PrecondType 1) or [side][nf] 1/diag (PrecondType 2)
//   lam, rhs, R, V, Z  [side][nf]   lambda etc. in the master side's (p,q) order, r = q*(N+1)+p
//
// Kernels:
//   k_elem_mat      one CTA per element builds Dhat (shared memory), factors -Dhat (Cholesky),
//                   inverts it and forms Ehat and Smat; same per-entry operation order as the oracle's
//                   restatement of Elem_Mat, so the matrices agree bit for bit (no FMA contraction).
//   k_build_precond one thread per side: BuildPrecond.
//   k_rhs           one CTA per element: RHS_vol, InvDhat(-RHS_vol), Ehat_s * that per side.
//   CG iteration    k_matvec (one CTA per element: the 36 Smat blocks times lambda of its 6 sides),
//                   k_gather (per side DOF: sum of the two elements, Dirichlet/zero-potential masking,
//                   dot product), k_update, k_precond, k_vupdate.  Dot products end in the last CTA
//                   to finish (ticket counter, fixed summation order), which also updates the CG
//                   scalars on the device, so the host never reads them inside the loop; a chunk of
//                   iterations is captured once as a CUDA graph and replayed until the device flag
//                   says converged.
//   k_post          one CTA per element: U = InvDhat(-(RHS_vol + sum_s Ehat_s^T lambda_s)) and
//                   E = PostProcessGradientHDG, written into the context's field array.
// Bounds: k_matvec streams Smat (36*nf^2*8 B per element and iteration) -> HBM-bound for large meshes,
// L2-resident for small ones; the rest is latency-bound.
#include "pic_ctx.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace pic_hdg {

constexpr int kMaxND = 5;                      // N <= 4
constexpr double kEps0 = 8.8541878176e-12;     // eps0 (src/globals/globals_vars.f90:84)

struct Tabs {                                  // N_Inter(N) tables (hdg.f90:473-497)
  int N, nd, nv, nf;
  double w[kMaxND], Lm[kMaxND], Lp[kMaxND], Lom_m[kMaxND], Lom_p[kMaxND];
  double Dom[kMaxND][kMaxND], LLm[kMaxND][kMaxND], LLp[kMaxND][kMaxND];
};

enum { F_DONE = 0, F_ITER = 1, F_STATUS = 2, F_TICKET = 3, F_CONV = 4, F_BARRIER = 5 };
enum { S_RZ1 = 0, S_OMEGA = 1, S_BETA = 2, S_RR = 3, S_ABORT2 = 4 };
enum { ST_NOT_CONVERGED = 1, ST_BREAKDOWN = 2, ST_ELEM_MAT = 4, ST_PRECOND = 8 };

struct Dev {
  int ne, ns, precond, zero_side, max_iter, relative;
  double eps_cg;
  const int* e2s;          // [e][6][2]: side (0-based), flip
  const int* s2e;          // [side][4]: elem, nb elem, loc, nb loc (0-based, -1)
  const uint8_t* masked;   // [side] Dirichlet
  const double *mf, *mg, *mh, *sj, *tau;
  double *ehat, *invd, *smat, *pre;
  double* smat_u;           // [e][stride]: the 21 blocks Smat(:,:,i,j), i <= j
  double *lam, *rhs, *R, *Pr, *Ax, *V0, *V1, *rhs_vol, *contrib, *U;
  double* red;             // partial sums, one per CTA of a side-DOF kernel (the cooperative kernel: 4 per CTA)
  double* sc;              // CG scalars
  int* flags;
};

__host__ __device__ inline int vidx(int i, int j, int k, int nd) { return i + nd * (j + nd * k); }

// CGNS_VolToSide + Flip_S2M (mapping.f90:147-240, 359-384): master-side (p,q) of volume point (i,j,k)
__device__ inline void vol_to_side(int N, int i, int j, int k, int flip, int s, int& p, int& q) {
  int a, b;
  switch (s) {
    case 4: a = k; b = j; break;
    case 2: a = j; b = k; break;
    case 1: a = i; b = k; break;
    case 3: a = N - i; b = k; break;
    case 0: a = j; b = i; break;
    default: a = i; b = j; break;
  }
  switch (flip) {
    case 0: p = a; q = b; break;
    case 1: p = b; q = a; break;
    case 2: p = N - a; q = b; break;
    case 3: p = N - b; q = N - a; break;
    default: p = a; q = N - b; break;
  }
}
__device__ inline void vol_to_side_ijk(int i, int j, int k, int s, int& l1, int& l2) {
  switch (s) {
    case 4: l1 = k; l2 = j; break;
    case 2: l1 = j; l2 = k; break;
    case 1: case 3: l1 = i; l2 = k; break;
    case 0: l1 = j; l2 = i; break;
    default: l1 = i; l2 = j; break;
  }
}
__device__ __constant__ int c_side_dir[6] = {2, 1, 0, 1, 0, 2};
__device__ __constant__ int c_pm[6] = {0, 0, 1, 1, 0, 1};
__device__ __constant__ int c_dir_pm[3][2] = {{4, 2}, {1, 3}, {0, 5}};

// ---------------------------------------------------------------------------------------------------
// Elem_Mat (elem_mat.f90:42-349).  Shared memory: Dh[nv*nv] | K[nv*9] | TauS[nv*6] | surf[6*nf] | tmp
// ---------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_elem_mat(Dev H, Tabs T) {
  extern __shared__ double sm[];
  const int e = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int N = T.N, nd = T.nd, nv = T.nv, nf = T.nf;
  double* Dh = sm;                       // column-major nv x nv; after the factorisation: U (upper)
  double* Ks = Dh + nv * nv;             // [g][3][3]
  double* Ts = Ks + nv * 9;              // [g][2][3]
  double* surf = Ts + nv * 6;            // [s][q][p]
  double* St1 = surf + 6 * nf;           // [b][r]  Stmp1(r,b) at r + nv*b
  __shared__ int fail;
  const int* e2s = H.e2s + 12 * e;
  const double* Mf = H.mf + (size_t)3 * nv * e;
  const double* Mg = H.mg + (size_t)3 * nv * e;
  const double* Mh = H.mh + (size_t)3 * nv * e;
  const double* sJ = H.sj + (size_t)nv * e;
  const double tau = H.tau[e];
  double* Eh = H.ehat + (size_t)nf * nv * 6 * e;
  double* Sm = H.smat + (size_t)nf * nf * 36 * e;
  double* Di = H.invd + (size_t)nv * nv * e;
  if (tid == 0) fail = 0;
  for (int i = tid; i < nf * nv * 6; i += nt) Eh[i] = 0.0;
  for (int i = tid; i < nf * nf * 36; i += nt) Sm[i] = 0.0;
  for (int i = tid; i < nv * nv; i += nt) Dh[i] = 0.0;
  // SurfElemLoc: |Ja^dir| prolonged to the side (ProlongToFace_Side, Gauss nodes) in master coordinates
  for (int t = tid; t < 6 * nf; t += nt) {
    const int s = t / nf, pq = t % nf, p = pq % nd, q = pq / nd;
    const int flip = e2s[2 * s + 1];
    int ps, qs;
    switch (flip) {
      case 0: ps = p; qs = q; break;
      case 1: ps = q; qs = p; break;
      case 2: ps = N - p; qs = q; break;
      case 3: ps = N - q; qs = N - p; break;
      default: ps = p; qs = N - q; break;
    }
    const double* Ja = (c_side_dir[s] == 0) ? Mf : (c_side_dir[s] == 1) ? Mg : Mh;
    const double* L = c_pm[s] ? T.Lp : T.Lm;
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (int l = 0; l < nd; ++l) {
      int i, j, k;
      switch (s) {
        case 4: i = l; j = qs; k = ps; break;
        case 1: i = ps; j = l; k = qs; break;
        case 0: i = qs; j = ps; k = l; break;
        case 2: i = l; j = ps; k = qs; break;
        case 3: i = N - ps; j = l; k = qs; break;
        default: i = ps; j = qs; k = l; break;
      }
      const double* u = Ja + 3 * vidx(i, j, k, nd);
      if (l == 0) { v0 = u[0] * L[0]; v1 = u[1] * L[0]; v2 = u[2] * L[0]; }
      else { v0 = v0 + u[0] * L[l]; v1 = v1 + u[1] * L[l]; v2 = v2 + u[2] * L[l]; }
    }
    surf[s * nf + q * nd + p] = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
  }
  __syncthreads();
  // Ktilde (chi = identity) scaled by sJ*wGP_vol, and TauS
  for (int g = tid; g < nv; g += nt) {
    const int g1 = g % nd, g2 = (g / nd) % nd, g3 = g / (nd * nd);
    const double* f = Mf + 3 * g;
    const double* gg = Mg + 3 * g;
    const double* h = Mh + 3 * g;
    double K[3][3];
    K[0][0] = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    K[1][1] = gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2];
    K[2][2] = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
    K[1][0] = gg[0] * f[0] + gg[1] * f[1] + gg[2] * f[2];
    K[2][0] = h[0] * f[0] + h[1] * f[1] + h[2] * f[2];
    K[2][1] = h[0] * gg[0] + h[1] * gg[1] + h[2] * gg[2];
    K[0][1] = K[1][0]; K[0][2] = K[2][0]; K[1][2] = K[2][1];
    const double sc = sJ[g] * (T.w[g1] * T.w[g2] * T.w[g3]);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) Ks[g * 9 + 3 * a + b] = sc * K[a][b];
    for (int s = 0; s < 6; ++s) {
      int p, q, l1, l2;
      vol_to_side(N, g1, g2, g3, e2s[2 * s + 1], s, p, q);
      vol_to_side_ijk(g1, g2, g3, s, l1, l2);
      Ts[g * 6 + 3 * c_pm[s] + c_side_dir[s]] = (T.w[l1] * T.w[l2] * surf[s * nf + q * nd + p]) * tau;
    }
  }
  __syncthreads();
  // Dhat: thread j owns column j; contributions in the reference's order (g ascending; the surface
  // term, then jDir, q, iDir, p)
  for (int j = tid; j < nv; j += nt) {
    const int jx[3] = {j % nd, (j / nd) % nd, j / (nd * nd)};
    for (int g = 0; g < nv; ++g) {
      const int gd[3] = {g % nd, (g / nd) % nd, g / (nd * nd)};
      const int diff = (gd[0] != jx[0]) + (gd[1] != jx[1]) + (gd[2] != jx[2]);
      if (diff > 1) continue;
      const double* Kg = Ks + 9 * g;
      const double* Tg = Ts + 6 * g;
      if (g == j) {
        for (int iDir = 0; iDir < 3; ++iDir) {
          int idx[3] = {gd[0], gd[1], gd[2]};
          for (int l = 0; l < nd; ++l) {
            idx[iDir] = l;
            const int i = vidx(idx[0], idx[1], idx[2], nd);
            Dh[i + nv * j] = Dh[i + nv * j] - (Tg[iDir] * T.LLm[l][gd[iDir]] + Tg[3 + iDir] * T.LLp[l][gd[iDir]]);
          }
        }
      }
      for (int jDir = 0; jDir < 3; ++jDir) {
        bool hit = true;
        for (int c = 0; c < 3; ++c)
          if (c != jDir && gd[c] != jx[c]) hit = false;
        if (!hit) continue;
        const int q = jx[jDir];
        for (int iDir = 0; iDir < 3; ++iDir) {
          int idx[3] = {gd[0], gd[1], gd[2]};
          for (int p = 0; p < nd; ++p) {
            idx[iDir] = p;
            const int i = vidx(idx[0], idx[1], idx[2], nd);
            Dh[i + nv * j] = Dh[i + nv * j] - Kg[3 * iDir + jDir] * T.Dom[p][gd[iDir]] * T.Dom[q][gd[jDir]];
          }
        }
      }
    }
  }
  __syncthreads();
  // -Dhat = U^T U (upper Cholesky, column by column, as the oracle)
  for (int i = tid; i < nv * nv; i += nt) Dh[i] = -Dh[i];
  __syncthreads();
  for (int j = 0; j < nv; ++j) {
    if (tid == 0) {
      double s = Dh[j + nv * j];
      for (int k = 0; k < j; ++k) s = s - Dh[k + nv * j] * Dh[k + nv * j];
      if (!(s > 0.0)) { fail = 1; s = 1.0; }
      Dh[j + nv * j] = sqrt(s);
    }
    __syncthreads();
    const double d = Dh[j + nv * j];
    for (int i = j + 1 + tid; i < nv; i += nt) {
      double t = Dh[j + nv * i];
      for (int k = 0; k < j; ++k) t = t - Dh[k + nv * j] * Dh[k + nv * i];
      Dh[j + nv * i] = t / d;
    }
    __syncthreads();
  }
  // inverse, one column per thread: forward and back substitution with U; InvDhat = -(-Dhat)^{-1}
  for (int c = tid; c < nv; c += nt) {
    double y[kMaxND * kMaxND * kMaxND];
    for (int i = 0; i < nv; ++i) {
      double t = (i == c) ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) t = t - Dh[k + nv * i] * y[k];
      y[i] = t / Dh[i + nv * i];
    }
    for (int i = nv - 1; i >= 0; --i) {
      double t = y[i];
      for (int k = i + 1; k < nv; ++k) t = t - Dh[i + nv * k] * y[k];   // y[k] already holds x[k]
      y[i] = t / Dh[i + nv * i];
    }
    for (int i = 0; i <= c; ++i) Di[i + nv * c] = y[i];                 // upper triangle of column c
  }
  __syncthreads();
  for (int t = tid; t < nv * nv; t += nt) {
    const int i = t % nv, c = t / nv;
    if (i > c) Di[i + nv * c] = Di[c + nv * i];
  }
  __syncthreads();
  for (int t = tid; t < nv * nv; t += nt) Di[t] = -Di[t];
  // Ehat = E - B A^{-1} C^T: thread per (side, row a); the normal line of a, g ascending
  for (int t = tid; t < 6 * nf; t += nt) {
    const int s = t / nf, a = t % nf;
    const int iDir = c_side_dir[s], pmS = c_pm[s];
    const double* Lom = pmS ? T.Lom_p : T.Lom_m;
    double* Es = Eh + (size_t)nf * nv * s;
    for (int g = 0; g < nv; ++g) {
      const int g1 = g % nd, g2 = (g / nd) % nd, g3 = g / (nd * nd);
      int p, q;
      vol_to_side(N, g1, g2, g3, e2s[2 * s + 1], s, p, q);
      if (q * nd + p != a) continue;
      const double* Kg = Ks + 9 * g;
      const int gi = (iDir == 0) ? g1 : (iDir == 1) ? g2 : g3;
      const double tsv = Ts[6 * g + 3 * pmS + iDir];
      Es[a + nf * g] = Es[a + nf * g] + (pmS ? tsv * T.w[gi] * (T.Lom_p[gi]) : tsv * T.w[gi] * (-T.Lom_m[gi]));
      for (int qq = 0; qq < nd; ++qq) {
        int j = vidx(qq, g2, g3, nd);
        Es[a + nf * j] = Es[a + nf * j] + Kg[0 * 3 + iDir] * T.Dom[qq][g1] * Lom[gi];
        j = vidx(g1, qq, g3, nd);
        Es[a + nf * j] = Es[a + nf * j] + Kg[1 * 3 + iDir] * T.Dom[qq][g2] * Lom[gi];
        j = vidx(g1, g2, qq, nd);
        Es[a + nf * j] = Es[a + nf * j] + Kg[2 * 3 + iDir] * T.Dom[qq][g3] * Lom[gi];
      }
    }
  }
  __syncthreads();
  // Smat: C A^{-1} C^T, thread per (row side iS, row a)
  for (int t = tid; t < 6 * nf; t += nt) {
    const int iS = t / nf, a = t % nf;
    const int iDir = c_side_dir[iS];
    const double* LomI = c_pm[iS] ? T.Lom_p : T.Lom_m;
    for (int g = 0; g < nv; ++g) {
      const int g1 = g % nd, g2 = (g / nd) % nd, g3 = g / (nd * nd);
      int p, q;
      vol_to_side(N, g1, g2, g3, e2s[2 * iS + 1], iS, p, q);
      if (q * nd + p != a) continue;
      const int gd[3] = {g1, g2, g3};
      for (int jDir = 0; jDir < 3; ++jDir) {
        const double kk = Ks[9 * g + 3 * iDir + jDir];
        for (int m = 0; m < 2; ++m) {
          const int jS = c_dir_pm[jDir][m];
          vol_to_side(N, g1, g2, g3, e2s[2 * jS + 1], jS, p, q);
          const int b = q * nd + p;
          const double lj = m ? T.Lom_p[gd[jDir]] : T.Lom_m[gd[jDir]];
          double* ent = Sm + a + nf * (b + nf * (iS + 6 * jS));
          *ent = *ent + kk * LomI[gd[iDir]] * lj;
        }
      }
    }
  }
  __syncthreads();
  // Smat += Ehat_i InvDhat Ehat_j^T, and the side mass term on the diagonal blocks
  for (int jS = 0; jS < 6; ++jS) {
    const double* Ej = Eh + (size_t)nf * nv * jS;
    for (int t = tid; t < nv * nf; t += nt) {
      const int r = t % nv, b = t / nv;
      double acc = 0.0;
      for (int c = 0; c < nv; ++c) acc = acc + Di[r + nv * c] * Ej[b + nf * c];
      St1[r + nv * b] = acc;
    }
    __syncthreads();
    for (int iS = jS; iS < 6; ++iS) {
      const double* Ei = Eh + (size_t)nf * nv * iS;
      for (int t = tid; t < nf * nf; t += nt) {
        const int a = t % nf, b = t / nf;
        double acc = 0.0;
        for (int r = 0; r < nv; ++r) acc = acc + Ei[a + nf * r] * St1[r + nv * b];
        if (iS == jS) {
          double* ent = Sm + a + nf * (b + nf * (jS + 6 * jS));
          *ent = *ent + acc;
          if (a == b) {
            const int p = a % nd, q = a / nd;
            const double fd = -tau * T.w[p] * T.w[q] * surf[jS * nf + q * nd + p];
            *ent = *ent - fd;
          }
        } else {
          double* e1 = Sm + a + nf * (b + nf * (iS + 6 * jS));
          double* e2 = Sm + b + nf * (a + nf * (jS + 6 * iS));
          *e1 = *e1 + acc;
          *e2 = *e2 + acc;
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0 && fail) atomicOr(&H.flags[F_STATUS], ST_ELEM_MAT);
}

// BuildPrecond (elem_mat.f90:513-618): one thread per side
__global__ void k_build_precond(Dev H, int nf) {
  const int sid = blockIdx.x * blockDim.x + threadIdx.x;
  if (sid >= H.ns) return;
  const int* se = H.s2e + 4 * sid;
  if (H.precond == 1) {
    double* P = H.pre + (size_t)nf * nf * sid;
    for (int i = 0; i < nf * nf; ++i) P[i] = 0.0;
    for (int m = 0; m < 2; ++m) {
      if (se[2 + m] < 0) continue;
      const int e = se[m], loc = se[2 + m];
      const double* blk = H.smat + (size_t)nf * nf * (36 * e + loc + 6 * loc);
      for (int i = 0; i < nf * nf; ++i) P[i] = P[i] + blk[i];
    }
    if (H.masked[sid]) return;
    for (int j = 0; j < nf; ++j) {                    // DPOTRF 'U'
      double s = P[j + nf * j];
      for (int k = 0; k < j; ++k) s = s - P[k + nf * j] * P[k + nf * j];
      if (!(s > 0.0)) { atomicOr(&H.flags[F_STATUS], ST_PRECOND); return; }
      const double d = sqrt(s);
      P[j + nf * j] = d;
      for (int i = j + 1; i < nf; ++i) {
        double t = P[j + nf * i];
        for (int k = 0; k < j; ++k) t = t - P[k + nf * j] * P[k + nf * i];
        P[j + nf * i] = t / d;
      }
    }
  } else if (H.precond == 2) {
    double* P = H.pre + (size_t)nf * sid;
    for (int a = 0; a < nf; ++a) P[a] = 0.0;
    for (int m = 0; m < 2; ++m) {
      if (se[2 + m] < 0) continue;
      const int e = se[m], loc = se[2 + m];
      const double* blk = H.smat + (size_t)nf * nf * (36 * e + loc + 6 * loc);
      for (int a = 0; a < nf; ++a) P[a] = P[a] + blk[a + nf * a];
    }
    if (H.masked[sid]) return;
    double mx = 0.0;
    for (int a = 0; a < nf; ++a) mx = fmax(mx, fabs(P[a]));
    if (!(mx > 1.0e-12)) { atomicOr(&H.flags[F_STATUS], ST_PRECOND); return; }
    for (int a = 0; a < nf; ++a) P[a] = 1.0 / P[a];
  }
}

// ---------------------------------------------------------------------------------------------------
// RHS (hdg_linear.f90:191-233): resu from the deposited PartSource (src_ps) or from a given array
// ---------------------------------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(128) k_rhs(Dev H, Tabs T, const double* __restrict__ part_source,
                                             const double* __restrict__ resu_in) {
  constexpr int nv = ND * ND * ND, nf = ND * ND;
  __shared__ double rv[nv], rt[nv];
  const int e = blockIdx.x, tid = threadIdx.x;
  const double* sJ = H.sj + (size_t)nv * e;
  for (int r = tid; r < nv; r += blockDim.x) {
    const int i = r % ND, j = (r / ND) % ND, k = r / (ND * ND);
    const double jw = T.w[i] * T.w[j] * T.w[k] / sJ[r];
    const double resu = part_source ? -(part_source[((size_t)nv * e + r) * 4 + 3] / kEps0) : resu_in[(size_t)nv * e + r];
    rv[r] = -jw * resu;
    H.rhs_vol[(size_t)nv * e + r] = rv[r];
  }
  __syncthreads();
  const double* Di = H.invd + (size_t)nv * nv * e;
  for (int r = tid; r < nv; r += blockDim.x) {
    double acc = 0.0;
    for (int c = 0; c < nv; ++c) acc = acc + (-rv[c]) * Di[r + nv * c];
    rt[r] = acc;
  }
  __syncthreads();
  for (int t = tid; t < 6 * nf; t += blockDim.x) {
    const int s = t / nf, a = t % nf;
    const double* Es = H.ehat + (size_t)nf * nv * (s + 6 * e);
    double acc = 0.0;
    for (int c = 0; c < nv; ++c) acc = acc + rt[c] * Es[a + nf * c];
    H.contrib[((size_t)6 * e + s) * nf + a] = acc;
  }
}

// per side DOF: the two element contributions in element order (the reference's assembly order)
__device__ inline double side_sum(const Dev& H, const double* __restrict__ contrib, int sid, int a, int nf) {
  const int* se = H.s2e + 4 * sid;
  const int e0 = se[0], l0 = se[2], e1 = se[1], l1 = se[3];
  const double c0 = contrib[((size_t)6 * e0 + l0) * nf + a];
  if (l1 < 0) return c0;
  const double c1 = contrib[((size_t)6 * e1 + l1) * nf + a];
  const bool first0 = (e0 < e1) || (e0 == e1 && l0 < l1);
  return first0 ? c0 + c1 : c1 + c0;
}

__global__ void k_rhs_face(Dev H, int nf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= H.ns * nf) return;
  H.rhs[t] = side_sum(H, H.contrib, t / nf, t % nf, nf);
}

__global__ void k_set_dirichlet(Dev H, const double* __restrict__ vals, const int* __restrict__ dir_sides, int n_dir,
                                int nf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_dir * nf) H.lam[(size_t)dir_sides[t / nf] * nf + t % nf] = vals ? vals[t] : 0.0;
  if (t == 0 && H.zero_side >= 0) H.lam[(size_t)H.zero_side * nf] = 0.0;
}

// ---------------------------------------------------------------------------------------------------
// CG (hdg_tools.f90:41-234).  One iteration = three kernels:
//   k_matvec   (per element) V_new = P^{-1}R + beta V_old for the element's sides (the master element
//              of a side writes it), y = S V_new from the 21 stored blocks of Smat
//   k_gather   (per side DOF) Ax = the two elements' y, masked; v.Ax -> omega
//   k_update   lambda += omega V, R -= omega Ax, Pr = P^{-1} R; r.r and r.Pr -> convergence, beta
// The reference's order (MatVec, omega, update, test, ApplyPrecond, beta, V = Z + beta V) is kept; the
// V update just moves to the start of the next iteration.  Two V buffers alternate between iterations.
// The matvec is bound by the FP64 pipe (GB300: about 2 FP64 lanes per clock and SM), so its products
// are explicit fused multiply-adds (one instruction, one rounding) although the library is built
// with -fmad=false; the CG is compared with the oracle within a tolerance, not bit for bit.
// ---------------------------------------------------------------------------------------------------
constexpr int kRedThreads = 256;

// block sums of (v0, v1), then the last CTA to arrive sums the partials in index order and runs fin
template <class Fin>
__device__ inline void reduce_and_finish(const Dev& H, double v0, double v1, Fin fin) {
  __shared__ double ws[2][kRedThreads / 32];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, o);
    v1 += __shfl_down_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) == 0) { ws[0][threadIdx.x >> 5] = v0; ws[1][threadIdx.x >> 5] = v1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s0 += ws[0][w]; s1 += ws[1][w]; }
    H.red[2 * blockIdx.x] = s0;
    H.red[2 * blockIdx.x + 1] = s1;
    __threadfence();
    const int ticket = atomicAdd(&H.flags[F_TICKET], 1);
    last = (ticket == (int)gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s0 = 0.0, s1 = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    s0 += __ldcg(H.red + 2 * b);
    s1 += __ldcg(H.red + 2 * b + 1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { ws[0][threadIdx.x >> 5] = s0; ws[1][threadIdx.x >> 5] = s1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t0 += ws[0][w]; t1 += ws[1][w]; }
    H.flags[F_TICKET] = 0;
    fin(t0, t1);
  }
}

// upper block (i <= j) index in the packed Smat: (0,0) (0,1) .. (0,5) (1,1) .. (5,5)
__host__ __device__ constexpr int upper_block(int i, int j) { return i * 6 - (i * (i - 1)) / 2 + (j - i); }

// copy the 21 blocks Smat(:,:,i,j), i <= j, of every element to the packed array used by k_matvec
__global__ void k_pack_upper(Dev H, int nf, size_t stride) {
  const int e = blockIdx.x;
  const double* Sm = H.smat + (size_t)nf * nf * 36 * e;
  for (int t = threadIdx.x; t < 21 * nf * nf; t += blockDim.x) {
    const int blk = t / (nf * nf), ab = t % (nf * nf);
    int i = 0;
    while (upper_block(i, 5) < blk) ++i;
    const int j = i + (blk - upper_block(i, i));
    H.smat_u[stride * e + t] = Sm[ab + (size_t)nf * nf * (i + 6 * j)];
  }
}

template <int ND>
__host__ __device__ constexpr int matvec_threads_t() { return ((21 * ND * ND + 31) / 32) * 32; }

// y = S x per element.  UPDATE: x = V_new = Pr + beta V_old (the side's master element stores it in Vnew);
// otherwise x = xin.  Shared memory: the 21 blocks (column stride nf+1), x of the 6 sides, row/col parts.
template <int ND, bool UPDATE>
__device__ __forceinline__ void matvec_element(const Dev& H, int e, const double* __restrict__ xin,
                                               const double* __restrict__ vold, double* __restrict__ vnew,
                                               size_t stride, double beta, double* sm) {
  constexpr int nf = ND * ND, ld = nf + 1;
  double* Sb = sm;                       // [21][nf][ld]
  double* xs = Sb + 21 * nf * ld;        // [6][nf]
  double* pr = xs + 6 * nf;              // [21][nf] row parts
  double* pc = pr + 21 * nf;             // [21][nf] column parts
  const int tid = threadIdx.x, nt = blockDim.x;
  const double* src = H.smat_u + stride * e;
  // every load of the thread issued before the first store: 16..25 independent loads in flight per thread
  // (launched with exactly matvec_threads_t<ND>() threads)
  constexpr int NT = matvec_threads_t<ND>(), TOT = 21 * nf * nf, PER = (TOT + NT - 1) / NT;
  double v[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int t = tid + k * NT;
    v[k] = t < TOT ? src[t] : 0.0;
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int t = tid + k * NT;
    if (t < TOT) {
      const int blk = t / (nf * nf), ab = t % (nf * nf);
      Sb[blk * nf * ld + (ab / nf) * ld + ab % nf] = v[k];
    }
  }
  const int* e2s = H.e2s + 12 * e;
  for (int t = tid; t < 6 * nf; t += nt) {
    const int loc = t / nf, b = t % nf;
    const int sid = e2s[2 * loc];
    const size_t g = (size_t)sid * nf + b;
    double x;
    if (UPDATE) {
      x = __fma_rn(beta, vold[g], H.Pr[g]);
      const int* se = H.s2e + 4 * sid;
      if (se[0] == e && se[2] == loc) vnew[g] = x;
    } else {
      x = xin[g];
    }
    xs[t] = x;
  }
  __syncthreads();
  if (tid < 21 * nf) {
    const int blk = tid / nf, t = tid % nf;
    int i = 0;
    while (upper_block(i, 5) < blk) ++i;
    const int j = i + (blk - upper_block(i, i));
    const double* B = Sb + blk * nf * ld;
    double r = 0.0;
#pragma unroll
    for (int b = 0; b < nf; ++b) r = __fma_rn(B[b * ld + t], xs[j * nf + b], r);
    pr[blk * nf + t] = r;
    if (i != j) {
      double c = 0.0;
#pragma unroll
      for (int a = 0; a < nf; ++a) c = __fma_rn(B[t * ld + a], xs[i * nf + a], c);
      pc[blk * nf + t] = c;
    }
  }
  __syncthreads();
  for (int t = tid; t < 6 * nf; t += nt) {
    const int i = t / nf, a = t % nf;
    double y = 0.0;
    for (int j = 0; j < 6; ++j) y = y + (j >= i ? pr[upper_block(i, j) * nf + a] : pc[upper_block(j, i) * nf + a]);
    H.contrib[((size_t)6 * e + i) * nf + a] = y;
  }
}

template <int ND, bool UPDATE>
__global__ void __launch_bounds__(matvec_threads_t<ND>()) k_matvec(Dev H, const double* __restrict__ xin,
                                                                   const double* __restrict__ vold,
                                                                   double* __restrict__ vnew, size_t stride) {
  if (__ldcg(&H.flags[F_DONE])) return;
  extern __shared__ double sm[];
  matvec_element<ND, UPDATE>(H, blockIdx.x, xin, vold, vnew, stride, UPDATE ? __ldcg(&H.sc[S_BETA]) : 0.0, sm);
}

// MODE 0: EvalResidual (R = RHS - S lambda, |R|^2, start test); MODE 1: Ax = S V and v.Ax -> omega
template <int MODE>
__global__ void __launch_bounds__(kRedThreads) k_gather(Dev H, const double* __restrict__ v, int nf) {
  if (__ldcg(&H.flags[F_DONE])) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (t < H.ns * nf) {
    const int sid = t / nf, a = t % nf;
    const bool zero = H.masked[sid] || (sid == H.zero_side && a == 0);
    double y = side_sum(H, H.contrib, sid, a, nf);
    if (zero) y = 0.0;
    if (MODE == 0) {
      const double r = zero ? 0.0 : H.rhs[t] - y;
      H.R[t] = r;
      acc = r * r;
    } else {
      H.Ax[t] = y;
      acc = v[t] * y;
    }
  }
  reduce_and_finish(H, acc, 0.0, [&](double tot, double) {
    if (MODE == 0) {
      H.sc[S_RR] = tot;
      const double e2 = H.eps_cg * H.eps_cg;
      const bool conv = H.relative ? (tot < 1e-16) : (tot < e2);
      H.sc[S_ABORT2] = H.relative ? tot * e2 : e2;
      H.flags[F_ITER] = 0;
      if (conv) { H.flags[F_CONV] = 1; H.flags[F_DONE] = 1; }
    } else {
      if (fabs(tot) <= 0.0) { H.flags[F_STATUS] |= ST_BREAKDOWN; H.flags[F_DONE] = 1; }
      else H.sc[S_OMEGA] = H.sc[S_RZ1] / tot;
    }
  });
}

// Pr = P^{-1} r for one side (ApplyPrecond), returns r.Pr over the side
__device__ inline double apply_precond_side(const Dev& H, int sid, int nf, const double* r, double* o) {
  double v = 0.0;
  if (H.precond == 0) {
    for (int a = 0; a < nf; ++a) { o[a] = r[a]; v += r[a] * r[a]; }
  } else if (H.masked[sid]) {
    for (int a = 0; a < nf; ++a) o[a] = 0.0;
  } else if (H.precond == 2) {
    const double* P = H.pre + (size_t)nf * sid;
    for (int a = 0; a < nf; ++a) { o[a] = P[a] * r[a]; v += r[a] * o[a]; }
  } else {
    const double* U = H.pre + (size_t)nf * nf * sid;        // DPOTRS with the upper factor
    double y[kMaxND * kMaxND];
    for (int i = 0; i < nf; ++i) {
      double t = r[i];
      for (int k = 0; k < i; ++k) t = t - U[k + nf * i] * y[k];
      y[i] = t / U[i + nf * i];
    }
    for (int i = nf - 1; i >= 0; --i) {
      double t = y[i];
      for (int k = i + 1; k < nf; ++k) t = t - U[i + nf * k] * y[k];
      y[i] = t / U[i + nf * i];
    }
    for (int a = 0; a < nf; ++a) { o[a] = y[a]; v += r[a] * y[a]; }
  }
  return v;
}

// FIRST (after EvalResidual): Pr = P^{-1}R, rz1 = r.Pr, beta = 0.
// Otherwise: lambda += omega V, R -= omega Ax, |R|^2 and the tests, Pr = P^{-1}R, beta = rz2/rz1.
// PrecondType 1 runs one thread per side, the others one thread per side DOF.
template <bool FIRST>
__global__ void __launch_bounds__(kRedThreads) k_update(Dev H, const double* __restrict__ v, int nf) {
  if (__ldcg(&H.flags[F_DONE])) return;
  const double om = FIRST ? 0.0 : __ldcg(&H.sc[S_OMEGA]);
  double rr = 0.0, rz = 0.0;
  if (H.precond == 1) {
    const int sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid < H.ns) {
      double r[kMaxND * kMaxND];
      for (int a = 0; a < nf; ++a) {
        const size_t g = (size_t)sid * nf + a;
        if (!FIRST) {
          H.lam[g] = H.lam[g] + om * v[g];
          H.R[g] = H.R[g] - om * H.Ax[g];
        }
        r[a] = H.R[g];
        rr += r[a] * r[a];
      }
      rz = apply_precond_side(H, sid, nf, r, H.Pr + (size_t)sid * nf);
    }
  } else {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < H.ns * nf) {
      double r = H.R[t];
      if (!FIRST) {
        H.lam[t] = H.lam[t] + om * v[t];
        r = r - om * H.Ax[t];
        H.R[t] = r;
      }
      double z = r;
      if (H.precond == 2) z = H.masked[t / nf] ? 0.0 : H.pre[t] * r;
      H.Pr[t] = z;
      rr = r * r;
      rz = r * z;
    }
  }
  reduce_and_finish(H, rr, rz, [&](double trr, double trz) {
    if (FIRST) {
      H.sc[S_RZ1] = trz;
      H.sc[S_BETA] = 0.0;
      return;
    }
    const int it = H.flags[F_ITER] + 1;
    H.flags[F_ITER] = it;
    H.sc[S_RR] = trr;
    if (isnan(trr)) { H.flags[F_STATUS] |= ST_BREAKDOWN; H.flags[F_DONE] = 1; return; }
    if (trr < H.sc[S_ABORT2]) { H.flags[F_CONV] = 1; H.flags[F_DONE] = 1; return; }
    if (it >= H.max_iter) { H.flags[F_STATUS] |= ST_NOT_CONVERGED; H.flags[F_DONE] = 1; return; }
    H.sc[S_BETA] = trz / H.sc[S_RZ1];
    H.sc[S_RZ1] = trz;
  });
}

// ---------------------------------------------------------------------------------------------------
// The whole CG in one cooperative launch (every CTA resident): the three phases of an iteration are
// separated by grid barriers instead of kernel boundaries.  Each CTA adds all CTAs' partial sums in the
// same order, so every CTA takes the same decisions (omega, convergence, beta) from the same values.
// The barrier wait is bounded: on timeout the CTA raises F_BARRIER and returns, and the others follow at
// their next barrier; the host then restores lambda and solves with the kernel-per-phase path.
// ---------------------------------------------------------------------------------------------------
constexpr unsigned long long kBarrierSpins = 1ull << 22;   // x ~0.1-0.3 us per poll
#ifndef PIC_HDG_COOP_MINB
#define PIC_HDG_COOP_MINB 1
#endif

__device__ bool grid_barrier(const Dev& H, unsigned* bar) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* gen = bar + 1;
    volatile int* err = H.flags + F_BARRIER;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned long long it = 0;
      while (*gen == g) {
        if (*err || ++it > kBarrierSpins) { atomicExch(H.flags + F_BARRIER, 1); ok = 0; break; }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// sum of (a, b) over the block; the result in every thread
__device__ inline void block_sum2(double& a, double& b, double* ws) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int nw = (int)(blockDim.x >> 5);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { ws[2 * (threadIdx.x >> 5)] = a; ws[2 * (threadIdx.x >> 5) + 1] = b; }
  __syncthreads();
  double s0 = 0.0, s1 = 0.0;
  for (int w = 0; w < nw; ++w) { s0 += ws[2 * w]; s1 += ws[2 * w + 1]; }
  a = s0;
  b = s1;
}

// every CTA: the sum of all CTAs' partials in index order
__device__ inline void grid_total2(const double* red, double& a, double& b, double* ws) {
  double s0 = 0.0, s1 = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    s0 += __ldcg(red + 2 * k);
    s1 += __ldcg(red + 2 * k + 1);
  }
  block_sum2(s0, s1, ws);
  a = s0;
  b = s1;
}

template <int ND>
__global__ void __launch_bounds__(matvec_threads_t<ND>(), PIC_HDG_COOP_MINB) k_cg_persistent(Dev H, size_t stride, unsigned* bar) {
  constexpr int nf = ND * ND;
  extern __shared__ double sm[];
  __shared__ double ws[2 * 32];
  if (__ldcg(&H.flags[F_DONE])) return;                        // set before the launch: uniform
  const int nthr = gridDim.x * blockDim.x, gtid = blockIdx.x * blockDim.x + threadIdx.x;
  double rz1 = __ldcg(&H.sc[S_RZ1]);
  const double abort2 = __ldcg(&H.sc[S_ABORT2]);
  double beta = 0.0;
  int it = __ldcg(&H.flags[F_ITER]);
  int par = 0;
  double* redB = H.red;                                        // v.Ax partials
  double* redC = H.red + 2 * gridDim.x;                        // r.r and r.Pr partials
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  for (;;) {
    const double* vold = par ? H.V1 : H.V0;
    double* vnew = par ? H.V0 : H.V1;
    // A: V_new = P^{-1}R + beta V_old, y = S V_new (element by element)
    for (int e = blockIdx.x; e < H.ne; e += gridDim.x) {
      matvec_element<ND, true>(H, e, nullptr, vold, vnew, stride, beta, sm);
      __syncthreads();
    }
    if (!grid_barrier(H, bar)) return;
    // B: Ax = the two elements' y (masked), v.Ax
    double acc = 0.0, dummy = 0.0;
    for (int t = gtid; t < H.ns * nf; t += nthr) {
      const int sid = t / nf, a = t % nf;
      double y = side_sum(H, H.contrib, sid, a, nf);
      if (H.masked[sid] || (sid == H.zero_side && a == 0)) y = 0.0;
      H.Ax[t] = y;
      acc += vnew[t] * y;
    }
    block_sum2(acc, dummy, ws);
    if (threadIdx.x == 0) { redB[2 * blockIdx.x] = acc; redB[2 * blockIdx.x + 1] = 0.0; }
    if (!grid_barrier(H, bar)) return;
    double vz, unused;
    grid_total2(redB, vz, unused, ws);
    if (fabs(vz) <= 0.0) {
      if (leader) { H.flags[F_STATUS] |= ST_BREAKDOWN; H.flags[F_DONE] = 1; H.flags[F_ITER] = it; }
      return;
    }
    const double om = rz1 / vz;
    // C: lambda += omega V, R -= omega Ax, Pr = P^{-1} R, r.r and r.Pr
    double rr = 0.0, rz = 0.0;
    if (H.precond == 1) {
      for (int sid = gtid; sid < H.ns; sid += nthr) {
        double r[kMaxND * kMaxND];
        for (int a = 0; a < nf; ++a) {
          const size_t g = (size_t)sid * nf + a;
          H.lam[g] = H.lam[g] + om * vnew[g];
          H.R[g] = H.R[g] - om * H.Ax[g];
          r[a] = H.R[g];
          rr += r[a] * r[a];
        }
        rz += apply_precond_side(H, sid, nf, r, H.Pr + (size_t)sid * nf);
      }
    } else {
      for (int t = gtid; t < H.ns * nf; t += nthr) {
        H.lam[t] = H.lam[t] + om * vnew[t];
        const double r = H.R[t] - om * H.Ax[t];
        H.R[t] = r;
        double z = r;
        if (H.precond == 2) z = H.masked[t / nf] ? 0.0 : H.pre[t] * r;
        H.Pr[t] = z;
        rr += r * r;
        rz += r * z;
      }
    }
    block_sum2(rr, rz, ws);
    if (threadIdx.x == 0) { redC[2 * blockIdx.x] = rr; redC[2 * blockIdx.x + 1] = rz; }
    if (!grid_barrier(H, bar)) return;
    double trr, trz;
    grid_total2(redC, trr, trz, ws);
    ++it;
    if (isnan(trr) || trr < abort2 || it >= H.max_iter) {
      if (leader) {
        H.flags[F_ITER] = it;
        H.sc[S_RR] = trr;
        if (isnan(trr)) H.flags[F_STATUS] |= ST_BREAKDOWN;
        else if (trr < abort2) H.flags[F_CONV] = 1;
        else H.flags[F_STATUS] |= ST_NOT_CONVERGED;
        H.flags[F_DONE] = 1;
      }
      return;
    }
    beta = trz / rz1;
    rz1 = trz;
    par ^= 1;
  }
}

// ---------------------------------------------------------------------------------------------------
// post processing (hdg_linear.f90:531-546) and PostProcessGradientHDG (elem_mat.f90:621-719)
// ---------------------------------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(128) k_post(Dev H, Tabs T, double* __restrict__ E) {
  constexpr int N = ND - 1, nv = ND * ND * ND, nf = ND * ND;
  __shared__ double lam6[6 * nf], rv[nv], u[nv];
  const int e = blockIdx.x, tid = threadIdx.x;
  const int* e2s = H.e2s + 12 * e;
  for (int t = tid; t < 6 * nf; t += blockDim.x) lam6[t] = H.lam[(size_t)e2s[2 * (t / nf)] * nf + t % nf];
  __syncthreads();
  for (int c = tid; c < nv; c += blockDim.x) {
    double r = H.rhs_vol[(size_t)nv * e + c];
    for (int s = 0; s < 6; ++s) {
      const double* Es = H.ehat + (size_t)nf * nv * (s + 6 * e);
      double acc = 0.0;
      for (int a = 0; a < nf; ++a) acc = acc + Es[a + nf * c] * lam6[s * nf + a];
      r = r + acc;
    }
    rv[c] = r;
  }
  __syncthreads();
  const double* Di = H.invd + (size_t)nv * nv * e;
  for (int r = tid; r < nv; r += blockDim.x) {
    double acc = 0.0;
    for (int c = 0; c < nv; ++c) acc = acc + (-rv[c]) * Di[r + nv * c];
    u[r] = acc;
    H.U[(size_t)nv * e + r] = acc;
  }
  __syncthreads();
  const double* sJ = H.sj + (size_t)nv * e;
  for (int g = tid; g < nv; g += blockDim.x) {
    const int gd[3] = {g % ND, (g / ND) % ND, g / (ND * ND)};
    double ex = 0.0, ey = 0.0, ez = 0.0;
    for (int jDir = 0; jDir < 3; ++jDir) {
      double ql = 0.0;
      int jdx[3] = {gd[0], gd[1], gd[2]};
      for (int q = 0; q < ND; ++q) {
        jdx[jDir] = q;
        ql = ql + T.Dom[q][gd[jDir]] * u[vidx(jdx[0], jdx[1], jdx[2], ND)];
      }
      const int mS = c_dir_pm[jDir][0], pS = c_dir_pm[jDir][1];
      int p, q;
      vol_to_side(N, gd[0], gd[1], gd[2], e2s[2 * mS + 1], mS, p, q);
      const int im = q * ND + p;
      vol_to_side(N, gd[0], gd[1], gd[2], e2s[2 * pS + 1], pS, p, q);
      const int ip = q * ND + p;
      ql = ql - T.Lom_m[gd[jDir]] * lam6[mS * nf + im];
      ql = ql - T.Lom_p[gd[jDir]] * lam6[pS * nf + ip];
      const double* a = ((jDir == 0) ? H.mf : (jDir == 1) ? H.mg : H.mh) + ((size_t)nv * e + g) * 3;
      ex = ex + sJ[g] * a[0] * ql;
      ey = ey + sJ[g] * a[1] * ql;
      ez = ez + sJ[g] * a[2] * ql;
    }
    double* o = E + ((size_t)nv * e + g) * 3;
    o[0] = ex; o[1] = ey; o[2] = ez;
  }
}

__global__ void k_field_to_float(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

}  // namespace pic_hdg

using namespace pic_hdg;

// ---------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------
struct HdgState {
  Dev D{};
  Tabs T{};
  int N = 0, nd = 0, nv = 0, nf = 0, n_dir = 0;
  int* dir_sides = nullptr;       // device, 0-based
  double* dir_vals = nullptr;     // device (nf, n_dir), null: zeros
  bool solve_in_step = false;
  int red_blocks = 0;
  cudaGraphExec_t chunk = nullptr;
  int chunk_iters = 0;
  size_t upper_stride = 0;        // doubles per element in the packed Smat
  int coop_grid = 0;              // CTAs of the cooperative CG kernel (0: kernel-per-phase path only)
  bool use_coop = true;           // cleared after a failed cooperative solve
  unsigned* bar = nullptr;        // its grid barrier (count, generation)
  double* lam_bak = nullptr;      // lambda at the start of a solve, for the fallback
  pic_hdg_status_t status{};
  std::vector<double> tau;
};

namespace {

int fail(int code, const std::string& m) { return pic_internal::set_error(code, m); }

void make_tabs(int N, const double* xgp, const double* wgp, Tabs& T) {
  // BarycentricWeights, LagrangeInterpolationPolys at -1/+1, PolynomialDerivativeMatrix (basis.f90)
  T.N = N; T.nd = N + 1; T.nv = T.nd * T.nd * T.nd; T.nf = T.nd * T.nd;
  double x[kMaxND], wb[kMaxND];
  for (int i = 0; i < T.nd; ++i) { x[i] = xgp[i]; T.w[i] = wgp[i]; wb[i] = 1.0; }
  for (int i = 1; i < T.nd; ++i)
    for (int k = 0; k < i; ++k) { wb[k] = wb[k] * (x[k] - x[i]); wb[i] = wb[i] * (x[i] - x[k]); }
  for (int i = 0; i < T.nd; ++i) wb[i] = 1.0 / wb[i];
  for (int side = 0; side < 2; ++side) {
    const double xx = side ? 1.0 : -1.0;
    double* L = side ? T.Lp : T.Lm;
    double tmp = 0.0;
    for (int j = 0; j < T.nd; ++j) { L[j] = wb[j] / (xx - x[j]); tmp = tmp + L[j]; }
    for (int j = 0; j < T.nd; ++j) L[j] = L[j] / tmp;
  }
  double D[kMaxND][kMaxND] = {};
  for (int l = 0; l < T.nd; ++l)
    for (int g = 0; g < T.nd; ++g)
      if (l != g) {
        D[g][l] = wb[l] / (wb[g] * (x[g] - x[l]));
        D[g][g] = D[g][g] - D[g][l];
      }
  for (int i = 0; i < T.nd; ++i) {
    for (int j = 0; j < T.nd; ++j) {
      T.LLm[i][j] = T.Lm[i] * T.Lm[j];
      T.LLp[i][j] = T.Lp[i] * T.Lp[j];
      T.Dom[i][j] = T.w[i] / T.w[j] * D[i][j];
    }
    T.Lom_m[i] = -T.Lm[i] / T.w[i];
    T.Lom_p[i] = +T.Lp[i] / T.w[i];
  }
}

#define HDG_DISPATCH(ND_, CALL) \
  switch (ND_) { case 2: { constexpr int ND = 2; CALL; } break; case 3: { constexpr int ND = 3; CALL; } break; \
                 case 4: { constexpr int ND = 4; CALL; } break; case 5: { constexpr int ND = 5; CALL; } break; default: break; }

int side_blocks(const HdgState* h) { return (h->D.ns * h->nf + kRedThreads - 1) / kRedThreads; }
int update_blocks(const HdgState* h) {
  return h->D.precond == 1 ? (h->D.ns + kRedThreads - 1) / kRedThreads : side_blocks(h);
}
template <int ND>
size_t matvec_smem() { constexpr int nf = ND * ND; return sizeof(double) * (21 * nf * (nf + 1) + 6 * nf + 42 * nf); }
template <int ND>
cudaError_t set_matvec_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_matvec<ND, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)matvec_smem<ND>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_matvec<ND, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)matvec_smem<ND>());
  return e;
}

template <int ND>
int coop_blocks_per_sm() {
  int n = 0;
  if (cudaFuncSetAttribute(k_cg_persistent<ND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)matvec_smem<ND>()) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cg_persistent<ND>, matvec_threads_t<ND>(), matvec_smem<ND>()) !=
      cudaSuccess)
    return 0;
  return n;
}

template <int ND>
cudaError_t launch_coop(HdgState* h, cudaStream_t s) {
  void* args[] = {(void*)&h->D, (void*)&h->upper_stride, (void*)&h->bar};
  return cudaLaunchCooperativeKernel((const void*)k_cg_persistent<ND>, dim3(h->coop_grid), dim3(matvec_threads_t<ND>()),
                                     args, matvec_smem<ND>(), s);
}

// CG iteration `parity`: V_old = V[parity], V_new = V[1 - parity]
int launch_iteration(HdgState* h, cudaStream_t s, int parity) {
  const int nf = h->nf;
  double* vold = parity ? h->D.V1 : h->D.V0;
  double* vnew = parity ? h->D.V0 : h->D.V1;
  HDG_DISPATCH(h->nd, (k_matvec<ND, true><<<h->D.ne, matvec_threads_t<ND>(), matvec_smem<ND>(), s>>>(
                           h->D, nullptr, vold, vnew, h->upper_stride)));
  k_gather<1><<<side_blocks(h), kRedThreads, 0, s>>>(h->D, vnew, nf);
  k_update<false><<<update_blocks(h), kRedThreads, 0, s>>>(h->D, vnew, nf);
  return 3;
}

int launch_chunk(HdgState* h, cudaStream_t s, int iters) {
  int n = 0;
  for (int i = 0; i < iters; ++i) n += launch_iteration(h, s, i & 1);
  return n;
}

}  // namespace

int hdg_destroy(pic_ctx_t* c) {
  if (c && c->hdg) {
    if (c->hdg->chunk) cudaGraphExecDestroy(c->hdg->chunk);
    delete c->hdg;
    c->hdg = nullptr;
  }
  return PIC_OK;
}

extern "C" int pic_hdg_init(pic_ctx_t* c, const pic_hdg_t* g) {
  if (!c || !g) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (c->hdg) return fail(PIC_ERR_STATE, "HDG already initialised for this context");
  const int N = c->N, nd = N + 1, nv = nd * nd * nd, nf = nd * nd, ne = c->ne;
  if (N < 1 || N > 4) return fail(PIC_ERR_INVALID_ARGUMENT, "the HDG solve supports N = 1..4");
  // p-adaption with HDG needs PETSc in the reference (mesh_pAdaption.f90:83-85); this solve has one N
  if (c->var_n) return fail(PIC_ERR_INVALID_ARGUMENT, "the HDG solve needs one polynomial degree for all elements");
  if (g->n_sides <= 0 || !g->elem_to_side || !g->side_to_elem || !g->metrics_f || !g->metrics_g || !g->metrics_h ||
      !g->sj)
    return fail(PIC_ERR_INVALID_ARGUMENT, "pic_hdg_t: missing array");
  if (g->precond_type < 0 || g->precond_type > 2) return fail(PIC_ERR_INVALID_ARGUMENT, "PrecondType must be 0, 1 or 2");
  if (g->max_iter_cg < 1 || !(g->eps_cg > 0.0)) return fail(PIC_ERR_INVALID_ARGUMENT, "MaxIterCG/epsCG");
  if (g->cg_kernel < 0 || g->cg_kernel > 2) return fail(PIC_ERR_INVALID_ARGUMENT, "cg_kernel must be 0, 1 or 2");
  if (g->n_dirichlet < 0 || (g->n_dirichlet > 0 && !g->dirichlet_sides))
    return fail(PIC_ERR_INVALID_ARGUMENT, "dirichlet_sides");
  const int ns = g->n_sides;
  // connectivity checks and conversion to 0-based
  std::vector<int> e2s(12 * (size_t)ne), s2e(4 * (size_t)ns);
  std::vector<int> seen(ns, 0);
  for (int e = 0; e < ne; ++e)
    for (int s = 0; s < 6; ++s) {
      const int sid = g->elem_to_side[12 * e + 2 * s], fl = g->elem_to_side[12 * e + 2 * s + 1];
      if (sid < 1 || sid > ns || fl < 0 || fl > 4) return fail(PIC_ERR_INVALID_ARGUMENT, "ElemToSide out of range");
      e2s[12 * e + 2 * s] = sid - 1;
      e2s[12 * e + 2 * s + 1] = fl;
      seen[sid - 1]++;
    }
  for (int sid = 0; sid < ns; ++sid) {
    const int32_t* r = g->side_to_elem + 5 * sid;
    if (r[0] < 1 || r[0] > ne || r[2] < 1 || r[2] > 6) return fail(PIC_ERR_INVALID_ARGUMENT, "SideToElem: master");
    const bool has_nb = r[1] != -1;
    if (has_nb && (r[1] < 1 || r[1] > ne || r[3] < 1 || r[3] > 6)) return fail(PIC_ERR_INVALID_ARGUMENT, "SideToElem: neighbour");
    if (seen[sid] != (has_nb ? 2 : 1)) return fail(PIC_ERR_INVALID_ARGUMENT, "SideToElem and ElemToSide disagree");
    if (e2s[12 * (r[0] - 1) + 2 * (r[2] - 1)] != sid || (has_nb && e2s[12 * (r[1] - 1) + 2 * (r[3] - 1)] != sid))
      return fail(PIC_ERR_INVALID_ARGUMENT, "SideToElem and ElemToSide disagree");
    s2e[4 * sid + 0] = r[0] - 1;
    s2e[4 * sid + 1] = has_nb ? r[1] - 1 : -1;
    s2e[4 * sid + 2] = r[2] - 1;
    s2e[4 * sid + 3] = has_nb ? r[3] - 1 : -1;
  }
  std::vector<uint8_t> masked(ns, 0);
  std::vector<int> dsides(g->n_dirichlet);
  for (int i = 0; i < g->n_dirichlet; ++i) {
    const int sid = g->dirichlet_sides[i];
    if (sid < 1 || sid > ns) return fail(PIC_ERR_INVALID_ARGUMENT, "DirichletBC out of range");
    masked[sid - 1] = 1;
    dsides[i] = sid - 1;
  }
  for (size_t i = 0; i < (size_t)nv * ne; ++i)
    if (!(g->sj[i] > 0.0)) return fail(PIC_ERR_INVALID_ARGUMENT, "sJ must be positive");

  HdgState* h = new HdgState();
  c->hdg = h;
  h->N = N; h->nd = nd; h->nv = nv; h->nf = nf; h->n_dir = g->n_dirichlet;
  h->solve_in_step = g->solve_in_step != 0;
  make_tabs(N, c->xgp_h.data(), c->wgp_h.data(), h->T);
  // Tau(iElem) = 2/(SUM(JwGP_vol))**(1/3) (hdg.f90:527), on the host like the oracle
  h->tau.resize(ne);
  for (int e = 0; e < ne; ++e) {
    double vol = 0.0;
    for (int k = 0; k < nd; ++k)
      for (int j = 0; j < nd; ++j)
        for (int i = 0; i < nd; ++i)
          vol = vol + h->T.w[i] * h->T.w[j] * h->T.w[k] / g->sj[(size_t)nv * e + vidx(i, j, k, nd)];
    h->tau[e] = 2.0 / std::pow(vol, 1.0 / 3.0);
  }
  Dev& D = h->D;
  D.ne = ne; D.ns = ns; D.precond = g->precond_type; D.max_iter = g->max_iter_cg; D.relative = g->use_relative_abort != 0;
  D.eps_cg = g->eps_cg;
  D.zero_side = g->n_dirichlet == 0 ? e2s[0] : -1;                 // ElemToSide(E2S_SIDE_ID,1,1)
  int rc = 0;
  int *d_e2s = nullptr, *d_s2e = nullptr;
  uint8_t* d_mask = nullptr;
  double *mf = nullptr, *mg = nullptr, *mh = nullptr, *sj = nullptr, *tau = nullptr;
  const size_t nsf = (size_t)ns * nf;
  rc = rc ? rc : c->alloc(&d_e2s, e2s.size());
  rc = rc ? rc : c->alloc(&d_s2e, s2e.size());
  rc = rc ? rc : c->alloc(&d_mask, (size_t)ns);
  rc = rc ? rc : c->alloc(&mf, (size_t)3 * nv * ne);
  rc = rc ? rc : c->alloc(&mg, (size_t)3 * nv * ne);
  rc = rc ? rc : c->alloc(&mh, (size_t)3 * nv * ne);
  rc = rc ? rc : c->alloc(&sj, (size_t)nv * ne);
  rc = rc ? rc : c->alloc(&tau, (size_t)ne);
  rc = rc ? rc : c->alloc(&D.ehat, (size_t)nf * nv * 6 * ne);
  rc = rc ? rc : c->alloc(&D.invd, (size_t)nv * nv * ne);
  rc = rc ? rc : c->alloc(&D.smat, (size_t)nf * nf * 36 * ne);
  rc = rc ? rc : c->alloc(&D.pre, g->precond_type == 1 ? nsf * nf : nsf);
  rc = rc ? rc : c->alloc(&D.lam, nsf);
  rc = rc ? rc : c->alloc(&D.rhs, nsf);
  rc = rc ? rc : c->alloc(&D.R, nsf);
  rc = rc ? rc : c->alloc(&D.Pr, nsf);
  rc = rc ? rc : c->alloc(&D.Ax, nsf);
  rc = rc ? rc : c->alloc(&D.V0, nsf);
  rc = rc ? rc : c->alloc(&D.V1, nsf);
  h->upper_stride = ((size_t)21 * nf * nf + 1) / 2 * 2;
  rc = rc ? rc : c->alloc(&D.smat_u, h->upper_stride * ne);
  rc = rc ? rc : c->alloc(&D.rhs_vol, (size_t)nv * ne);
  rc = rc ? rc : c->alloc(&D.contrib, (size_t)6 * nf * ne);
  rc = rc ? rc : c->alloc(&D.U, (size_t)nv * ne);
  const int nred = std::max((int)((nsf + kRedThreads - 1) / kRedThreads), 1);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  rc = rc ? rc : c->alloc(&D.red, (size_t)std::max(2 * nred, 4 * 8 * std::max(sms, 1)));
  rc = rc ? rc : c->alloc(&h->bar, 2);
  rc = rc ? rc : c->alloc(&h->lam_bak, nsf);
  rc = rc ? rc : c->alloc(&D.sc, 8);
  rc = rc ? rc : c->alloc(&D.flags, 8);
  if (g->n_dirichlet > 0) {
    rc = rc ? rc : c->alloc(&h->dir_sides, (size_t)g->n_dirichlet);
    rc = rc ? rc : c->alloc(&h->dir_vals, (size_t)g->n_dirichlet * nf);
  }
  if (rc) { hdg_destroy(c); return rc; }
  cudaStream_t s = c->stream;
#define H2D(dst, src, bytes) CUDA_CHECK_HDG(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s))
#define CUDA_CHECK_HDG(x) do { cudaError_t err_ = (x); if (err_ != cudaSuccess) { hdg_destroy(c); \
      return fail(PIC_ERR_CUDA, std::string("HDG init: ") + cudaGetErrorString(err_)); } } while (0)
  H2D(d_e2s, e2s.data(), e2s.size() * sizeof(int));
  H2D(d_s2e, s2e.data(), s2e.size() * sizeof(int));
  H2D(d_mask, masked.data(), masked.size());
  H2D(mf, g->metrics_f, sizeof(double) * 3 * nv * (size_t)ne);
  H2D(mg, g->metrics_g, sizeof(double) * 3 * nv * (size_t)ne);
  H2D(mh, g->metrics_h, sizeof(double) * 3 * nv * (size_t)ne);
  H2D(sj, g->sj, sizeof(double) * nv * (size_t)ne);
  H2D(tau, h->tau.data(), sizeof(double) * ne);
  if (g->n_dirichlet > 0) {
    H2D(h->dir_sides, dsides.data(), dsides.size() * sizeof(int));
    CUDA_CHECK_HDG(cudaMemsetAsync(h->dir_vals, 0, sizeof(double) * nf * (size_t)g->n_dirichlet, s));
  }
  CUDA_CHECK_HDG(cudaMemsetAsync(D.lam, 0, sizeof(double) * nsf, s));
  CUDA_CHECK_HDG(cudaMemsetAsync(D.V0, 0, sizeof(double) * nsf, s));
  CUDA_CHECK_HDG(cudaMemsetAsync(D.V1, 0, sizeof(double) * nsf, s));
  CUDA_CHECK_HDG(cudaMemsetAsync(D.flags, 0, sizeof(int) * 8, s));
  CUDA_CHECK_HDG(cudaMemsetAsync(D.sc, 0, sizeof(double) * 8, s));
  D.e2s = d_e2s; D.s2e = d_s2e; D.masked = d_mask; D.mf = mf; D.mg = mg; D.mh = mh; D.sj = sj; D.tau = tau;
  h->red_blocks = nred;
  // Elem_Mat
  const size_t smem = sizeof(double) * ((size_t)nv * nv + (size_t)nv * 9 + (size_t)nv * 6 + 6 * nf + (size_t)nv * nf);
  CUDA_CHECK_HDG(cudaFuncSetAttribute(k_elem_mat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_elem_mat<<<ne, 256, smem, s>>>(D, h->T);
  CUDA_CHECK_HDG(cudaGetLastError());
  k_build_precond<<<(ns + 127) / 128, 128, 0, s>>>(D, nf);
  CUDA_CHECK_HDG(cudaGetLastError());
  k_pack_upper<<<ne, 256, 0, s>>>(D, nf, h->upper_stride);
  CUDA_CHECK_HDG(cudaGetLastError());
  c->launches += 3;
  {
    cudaError_t ea = cudaSuccess;
    HDG_DISPATCH(nd, (ea = set_matvec_smem<ND>()));
    CUDA_CHECK_HDG(ea);
    // the cooperative CG kernel: as many CTAs as can be resident at once (at most 8 per SM)
    int coop = 0, per_sm = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (coop) {
      HDG_DISPATCH(nd, (per_sm = coop_blocks_per_sm<ND>()));
      h->coop_grid = std::min(per_sm, 8) * sms;
    }
    cudaGetLastError();
    // auto = the graph of three kernels per iteration: on GB300 the cooperative form measured slower
    // (8^3, N=3: 41 us per iteration with 2 CTAs/SM, 81 us with 4, against 34 us) -- the grid barriers
    // cost more than the kernel boundaries of a replayed graph
    h->use_coop = h->coop_grid > 0 && g->cg_kernel == 2;
  }
  int fl[8];
  CUDA_CHECK_HDG(cudaMemcpyAsync(fl, D.flags, sizeof(fl), cudaMemcpyDeviceToHost, s));
  CUDA_CHECK_HDG(cudaStreamSynchronize(s));
  if (fl[F_STATUS] & ST_ELEM_MAT) { hdg_destroy(c); return fail(PIC_ERR_INVALID_ARGUMENT, "Elem_Mat: -Dhat is not positive definite"); }
  if (fl[F_STATUS] & ST_PRECOND) { hdg_destroy(c); return fail(PIC_ERR_INVALID_ARGUMENT, "BuildPrecond: matrix inversion failed"); }
  // the CG chunk as a CUDA graph (8 iterations); plain launches if capture is unavailable
  h->chunk_iters = 8;
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    launch_chunk(h, s, h->chunk_iters);
    if (cudaStreamEndCapture(s, &graph) == cudaSuccess && graph) {
      if (cudaGraphInstantiate(&h->chunk, graph, 0) != cudaSuccess) h->chunk = nullptr;
      cudaGraphDestroy(graph);
    }
  }
  cudaGetLastError();
  return PIC_OK;
#undef H2D
}

extern "C" int pic_hdg_set_dirichlet(pic_ctx_t* c, const double* lambda_bc) {
  if (!c || !lambda_bc) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  HdgState* h = c->hdg;
  if (!h) return fail(PIC_ERR_STATE, "pic_hdg_init first");
  if (h->n_dir == 0) return PIC_OK;
  cudaError_t err = cudaMemcpyAsync(h->dir_vals, lambda_bc, sizeof(double) * h->nf * (size_t)h->n_dir,
                                    cudaMemcpyHostToDevice, c->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  return PIC_OK;
}

// HDGLinear on the device; source: device PartSource (ps_dev) or host resu
int hdg_solve_device(pic_ctx_t* c, const double* ps_dev, const double* resu_host) {
  HdgState* h = c->hdg;
  Dev& D = h->D;
  cudaStream_t s = c->stream;
  const int nf = h->nf, nv = h->nv;
  const double* resu_dev = nullptr;
  if (resu_host) {
    double* buf = D.rhs_vol;     // staging: k_rhs reads resu before it overwrites rhs_vol element by element
    cudaError_t err = cudaMemcpyAsync(buf, resu_host, sizeof(double) * nv * (size_t)D.ne, cudaMemcpyHostToDevice, s);
    if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
    resu_dev = buf;
  }
  int n = 0;
  // Dirichlet values and the zero-potential DOF
  const int nd_t = std::max(h->n_dir * nf, 1);
  k_set_dirichlet<<<(nd_t + 255) / 256, 256, 0, s>>>(D, h->dir_vals, h->dir_sides, h->n_dir, nf); ++n;
  HDG_DISPATCH(h->nd, (k_rhs<ND><<<D.ne, 128, 0, s>>>(D, h->T, ps_dev, resu_dev))); ++n;
  k_rhs_face<<<(D.ns * nf + 255) / 256, 256, 0, s>>>(D, nf); ++n;
  // EvalResidual and the first preconditioner application
  auto cg_start = [&]() {
    cudaMemsetAsync(D.flags, 0, sizeof(int) * 8, s);
    cudaMemsetAsync(D.V0, 0, sizeof(double) * (size_t)D.ns * nf, s);    // V_old of the first iteration
    HDG_DISPATCH(h->nd, (k_matvec<ND, false><<<D.ne, matvec_threads_t<ND>(), matvec_smem<ND>(), s>>>(
                             D, D.lam, nullptr, nullptr, h->upper_stride))); ++n;
    k_gather<0><<<side_blocks(h), kRedThreads, 0, s>>>(D, nullptr, nf); ++n;
    k_update<true><<<update_blocks(h), kRedThreads, 0, s>>>(D, nullptr, nf); ++n;
  };
  cudaError_t err = cudaMemcpyAsync(h->lam_bak, D.lam, sizeof(double) * (size_t)D.ns * nf, cudaMemcpyDeviceToDevice, s);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  cg_start();
  err = cudaGetLastError();
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  int fl[8] = {0};
  bool coop_done = false;
  if (h->coop_grid > 0 && h->use_coop) {
    // the whole CG in one cooperative launch; on a launch error or a barrier timeout: restore lambda
    // and run the kernel-per-phase path below
    cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), s);
    HDG_DISPATCH(h->nd, (err = launch_coop<ND>(h, s)));
    if (err == cudaSuccess) {
      ++n;
      err = cudaMemcpyAsync(fl, D.flags, sizeof(fl), cudaMemcpyDeviceToHost, s);
      if (err == cudaSuccess) err = cudaStreamSynchronize(s);
      if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
      coop_done = fl[F_DONE] && !fl[F_BARRIER];
    } else {
      cudaGetLastError();
    }
    if (!coop_done) {
      h->use_coop = false;
      err = cudaMemcpyAsync(D.lam, h->lam_bak, sizeof(double) * (size_t)D.ns * nf, cudaMemcpyDeviceToDevice, s);
      if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
      cg_start();
    }
  }
  const int max_chunks = coop_done ? 0 : (D.max_iter + h->chunk_iters - 1) / h->chunk_iters + 1;
  for (int ch = 0; ch < max_chunks; ++ch) {
    if (h->chunk) { err = cudaGraphLaunch(h->chunk, s); n += 3 * h->chunk_iters; }
    else n += launch_chunk(h, s, h->chunk_iters);
    if (err == cudaSuccess) err = cudaMemcpyAsync(fl, D.flags, sizeof(fl), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
    if (fl[F_DONE]) break;
  }
  HDG_DISPATCH(h->nd, (k_post<ND><<<D.ne, 128, 0, s>>>(D, h->T, c->E))); ++n;
  if (c->mixed) {
    const size_t m = (size_t)D.ne * nv * 3;
    k_field_to_float<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(c->E, c->E32, m); ++n;
  }
  err = cudaGetLastError();
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  double sc[8];
  err = cudaMemcpyAsync(sc, D.sc, sizeof(sc), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  c->launches += n;
  h->status.iterations = fl[F_ITER];
  h->status.converged = fl[F_CONV];
  h->status.norm_r = std::sqrt(sc[S_RR]);
  h->status.n_solves++;
  c->field_set = true;
  if (fl[F_STATUS] & (ST_NOT_CONVERGED | ST_BREAKDOWN)) {
    pic::DevStatus st{};
    cudaMemcpy(&st, c->st, sizeof(st), cudaMemcpyDeviceToHost);
    st.error_word |= (fl[F_STATUS] & ST_NOT_CONVERGED) ? PIC_STATUS_CG_NOT_CONVERGED : 0u;
    st.error_word |= (fl[F_STATUS] & ST_BREAKDOWN) ? PIC_STATUS_CG_BREAKDOWN : 0u;
    cudaMemcpy(c->st, &st, sizeof(st), cudaMemcpyHostToDevice);
  }
  return PIC_OK;
}

extern "C" int pic_hdg_solve(pic_ctx_t* c, const double* source, double* phi, double* e_field,
                             pic_hdg_status_t* status) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  HdgState* h = c->hdg;
  if (!h) return fail(PIC_ERR_STATE, "pic_hdg_init first");
  if (!source && !c->ps_valid) return fail(PIC_ERR_STATE, "no deposited charge: call pic_deposit or pass a source");
  int rc = hdg_solve_device(c, source ? nullptr : c->PS, source);
  if (rc) return rc;
  cudaError_t err = cudaSuccess;
  const size_t nvne = (size_t)h->nv * c->ne;
  if (phi) err = cudaMemcpyAsync(phi, h->D.U, sizeof(double) * nvne, cudaMemcpyDeviceToHost, c->stream);
  if (e_field && err == cudaSuccess)
    err = cudaMemcpyAsync(e_field, c->E, sizeof(double) * nvne * 3, cudaMemcpyDeviceToHost, c->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  if (status) *status = h->status;
  return PIC_OK;
}

extern "C" int pic_hdg_get_lambda(pic_ctx_t* c, double* lambda) {
  if (!c || !lambda) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  HdgState* h = c->hdg;
  if (!h) return fail(PIC_ERR_STATE, "pic_hdg_init first");
  cudaError_t err = cudaMemcpyAsync(lambda, h->D.lam, sizeof(double) * h->nf * (size_t)h->D.ns,
                                    cudaMemcpyDeviceToHost, c->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  return PIC_OK;
}

extern "C" int pic_hdg_set_lambda(pic_ctx_t* c, const double* lambda) {
  if (!c || !lambda) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  HdgState* h = c->hdg;
  if (!h) return fail(PIC_ERR_STATE, "pic_hdg_init first");
  cudaError_t err = cudaMemcpyAsync(h->D.lam, lambda, sizeof(double) * h->nf * (size_t)h->D.ns,
                                    cudaMemcpyHostToDevice, c->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  return PIC_OK;
}

extern "C" int pic_hdg_get_elem_mat(pic_ctx_t* c, int32_t elem, double* ehat, double* inv_dhat, double* smat) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  HdgState* h = c->hdg;
  if (!h) return fail(PIC_ERR_STATE, "pic_hdg_init first");
  if (elem < 1 || elem > c->ne) return fail(PIC_ERR_INVALID_ARGUMENT, "element out of range");
  const size_t e = (size_t)elem - 1, nv = h->nv, nf = h->nf;
  cudaError_t err = cudaSuccess;
  if (ehat) err = cudaMemcpyAsync(ehat, h->D.ehat + nf * nv * 6 * e, sizeof(double) * nf * nv * 6, cudaMemcpyDeviceToHost, c->stream);
  if (inv_dhat && err == cudaSuccess)
    err = cudaMemcpyAsync(inv_dhat, h->D.invd + nv * nv * e, sizeof(double) * nv * nv, cudaMemcpyDeviceToHost, c->stream);
  if (smat && err == cudaSuccess)
    err = cudaMemcpyAsync(smat, h->D.smat + nf * nf * 36 * e, sizeof(double) * nf * nf * 36, cudaMemcpyDeviceToHost, c->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  if (err != cudaSuccess) return fail(PIC_ERR_CUDA, cudaGetErrorString(err));
  return PIC_OK;
}

bool hdg_solve_in_step(const pic_ctx_t* c) { return c->hdg && c->hdg->solve_in_step; }
