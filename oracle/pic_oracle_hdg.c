/*
 * pic_oracle_hdg.c -- CPU restatement of PICLas's linear HDG Poisson solve.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU HDG solve of libpiclas_gpu.so.  Nothing in the
 * product links or calls this file.
 *
 * Follows, in the same loop order (no FMA contraction: -ffp-contract=off):
 *   Tau, JwGP_vol, Lomega/Domega/LL tables ... src/hdg/hdg.f90:473-529
 *   Elem_Mat (Dhat, Ehat, Smat, InvDhat) ..... src/hdg/elem_mat.f90:42-349
 *   ProlongToFace_Side (Gauss nodes) ......... src/interpolation/prolongtoface.f90:405-555
 *   VolToSide / Flip_S2M / CGNS_VolToSide .... src/mesh/mapping.f90:147-278, 359-384
 *   BuildPrecond (PrecondType 0/1/2) ......... src/hdg/elem_mat.f90:513-618
 *   HDGLinear (RHS, solve, post) ............. src/hdg/hdg_linear.f90:37-565
 *   CG_solver / MatVec / EvalResidual / ApplyPrecond / solveSPD
 *                                               src/hdg/hdg_tools.f90:41-807
 *   PostProcessGradientHDG ................... src/hdg/elem_mat.f90:621-719
 *   CalcSourceHDG with particles ............. src/equations/poisson/equation.f90:1039-1041
 * The reference calls LAPACK (DPOTRF/DPOTRI/DPOTRS) and BLAS (DSYMV/DGEMV/DGEMM/DSYMM); they are
 * restated here as textbook Cholesky factorisation, inverse, triangular solves and plain loops.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pic_oracle.h"

/* local sides 0..5 = ZETA_MINUS, ETA_MINUS, XI_PLUS, ETA_PLUS, XI_MINUS, ZETA_PLUS (piclas.h:204-209 minus one) */
static const int kSideDir[6] = {2, 1, 0, 1, 0, 2};  /* SideDir: normal direction of each side        */
static const int kPm[6] = {0, 0, 1, 1, 0, 1};       /* pm: 0 minus, 1 plus                           */
static const int kDirPm[3][2] = {{4, 2}, {1, 3}, {0, 5}};  /* dirPm2iSide(1:2,1:3) minus one      */

static void cgns_vol_to_side(int N, int i, int j, int k, int s, int* p, int* q) {
  switch (s) {
    case 4: *p = k; *q = j; break;          /* XI_MINUS   (k,j,i)      */
    case 2: *p = j; *q = k; break;          /* XI_PLUS    (j,k,N-i)    */
    case 1: *p = i; *q = k; break;          /* ETA_MINUS  (i,k,j)      */
    case 3: *p = N - i; *q = k; break;      /* ETA_PLUS   (N-i,k,N-j)  */
    case 0: *p = j; *q = i; break;          /* ZETA_MINUS (j,i,k)      */
    default: *p = i; *q = j; break;         /* ZETA_PLUS  (i,j,N-k)    */
  }
}

static void flip_s2m(int N, int p, int q, int flip, int* pm, int* qm) {
  switch (flip) {
    case 0: *pm = p; *qm = q; break;
    case 1: *pm = q; *qm = p; break;
    case 2: *pm = N - p; *qm = q; break;
    case 3: *pm = N - q; *qm = N - p; break;
    default: *pm = p; *qm = N - q; break;
  }
}

/* VolToSideA(1:2,i,j,k,flip,s) */
static void vol_to_side(int N, int i, int j, int k, int flip, int s, int* p, int* q) {
  int a, b;
  cgns_vol_to_side(N, i, j, k, s, &a, &b);
  flip_s2m(N, a, b, flip, p, q);
}

/* VolToSideIJKA(1:2,...): the two tangential volume indices */
static void vol_to_side_ijk(int i, int j, int k, int s, int* l1, int* l2) {
  switch (s) {
    case 4: *l1 = k; *l2 = j; break;
    case 2: *l1 = j; *l2 = k; break;
    case 1: case 3: *l1 = i; *l2 = k; break;
    case 0: *l1 = j; *l2 = i; break;
    default: *l1 = i; *l2 = j; break;
  }
}

/* 1D tables of N_Inter(N) used by HDG */
typedef struct {
  int N, nd, nv, nf;
  double x[ORC_HDG_MAXND], w[ORC_HDG_MAXND];
  double Lm[ORC_HDG_MAXND], Lp[ORC_HDG_MAXND];       /* L_minus, L_plus              */
  double D[ORC_HDG_MAXND][ORC_HDG_MAXND];             /* D(i,j) = l_j'(x_i)          */
  double Dom[ORC_HDG_MAXND][ORC_HDG_MAXND];           /* Domega(i,j) = w_i/w_j D(i,j) */
  double Lom_m[ORC_HDG_MAXND], Lom_p[ORC_HDG_MAXND];  /* Lomega_m/p                   */
  double LLm[ORC_HDG_MAXND][ORC_HDG_MAXND], LLp[ORC_HDG_MAXND][ORC_HDG_MAXND];
} Tables;

static void lagrange_at(const Tables* T, const double* wb, double x, double* L) {
  /* LagrangeInterpolationPolys (basis.f90:1223-1264) */
  int n = T->nd;
  for (int j = 0; j < n; ++j) {
    double dx = x - T->x[j];
    int hit = (x == 0.0 || T->x[j] == 0.0) ? (fabs(dx) <= 2.0 * 2.220446049250313e-16)
                                           : (fabs(dx) <= 2.220446049250313e-16 * fabs(x) &&
                                              fabs(dx) <= 2.220446049250313e-16 * fabs(T->x[j]));
    if (hit) {
      for (int k = 0; k < n; ++k) L[k] = 0.0;
      L[j] = 1.0;
      return;
    }
  }
  double tmp = 0.0;
  for (int j = 0; j < n; ++j) {
    L[j] = wb[j] / (x - T->x[j]);
    tmp = tmp + L[j];
  }
  for (int j = 0; j < n; ++j) L[j] = L[j] / tmp;
}

static void make_tables(int N, const double* xgp, const double* wgp, Tables* T) {
  T->N = N; T->nd = N + 1; T->nv = T->nd * T->nd * T->nd; T->nf = T->nd * T->nd;
  double wb[ORC_HDG_MAXND] = {0.0};
  for (int i = 0; i < T->nd; ++i) { T->x[i] = xgp[i]; T->w[i] = wgp[i]; }
  /* BarycentricWeights (basis.f90:952-976) */
  for (int i = 0; i < T->nd; ++i) wb[i] = 1.0;
  for (int i = 1; i < T->nd; ++i)
    for (int k = 0; k < i; ++k) {
      wb[k] = wb[k] * (T->x[k] - T->x[i]);
      wb[i] = wb[i] * (T->x[i] - T->x[k]);
    }
  for (int i = 0; i < T->nd; ++i) wb[i] = 1.0 / wb[i];
  lagrange_at(T, wb, -1.0, T->Lm);
  lagrange_at(T, wb, 1.0, T->Lp);
  /* PolynomialDerivativeMatrix (basis.f90:980-1007) */
  for (int i = 0; i < T->nd; ++i)
    for (int j = 0; j < T->nd; ++j) T->D[i][j] = 0.0;
  for (int l = 0; l < T->nd; ++l)
    for (int g = 0; g < T->nd; ++g)
      if (l != g) {
        T->D[g][l] = wb[l] / (wb[g] * (T->x[g] - T->x[l]));
        T->D[g][g] = T->D[g][g] - T->D[g][l];
      }
  for (int i = 0; i < T->nd; ++i) {
    for (int j = 0; j < T->nd; ++j) {
      T->LLm[i][j] = T->Lm[i] * T->Lm[j];
      T->LLp[i][j] = T->Lp[i] * T->Lp[j];
      T->Dom[i][j] = T->w[i] / T->w[j] * T->D[i][j];
    }
    T->Lom_m[i] = -T->Lm[i] / T->w[i];
    T->Lom_p[i] = +T->Lp[i] / T->w[i];
  }
}

static inline int vidx(int i, int j, int k, int nd) { return i + nd * (j + nd * k); }

/* Cholesky A = U^T U (upper, column-major n x n); returns 0 on success (DPOTRF 'U') */
static int chol_upper(int n, double* A) {
  for (int j = 0; j < n; ++j) {
    double s = A[j + n * j];
    for (int k = 0; k < j; ++k) s = s - A[k + n * j] * A[k + n * j];
    if (!(s > 0.0)) return 1;
    double d = sqrt(s);
    A[j + n * j] = d;
    for (int i = j + 1; i < n; ++i) {
      double t = A[j + n * i];
      for (int k = 0; k < j; ++k) t = t - A[k + n * j] * A[k + n * i];
      A[j + n * i] = t / d;
    }
  }
  return 0;
}

/* solve (U^T U) x = b with the upper factor (DPOTRS 'U') */
static void chol_solve(int n, const double* U, const double* b, double* x) {
  double y[ORC_HDG_MAXNV];
  for (int i = 0; i < n; ++i) {
    double t = b[i];
    for (int k = 0; k < i; ++k) t = t - U[k + n * i] * y[k];
    y[i] = t / U[i + n * i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double t = y[i];
    for (int k = i + 1; k < n; ++k) t = t - U[i + n * k] * x[k];
    x[i] = t / U[i + n * i];
  }
}

/* inverse of an SPD matrix: A^{-1}, symmetric (getSPDInverse = DPOTRF + DPOTRI, basis.f90) */
static int spd_inverse(int n, const double* A, double* Ainv) {
  double* U = (double*)malloc(sizeof(double) * n * n);
  memcpy(U, A, sizeof(double) * n * n);
  int rc = chol_upper(n, U);
  if (!rc) {
    double e[ORC_HDG_MAXNV], col[ORC_HDG_MAXNV];
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < n; ++i) e[i] = (i == j) ? 1.0 : 0.0;
      chol_solve(n, U, e, col);
      for (int i = 0; i < n; ++i) Ainv[i + n * j] = col[i];
    }
    for (int j = 0; j < n; ++j)          /* keep the upper triangle, mirror it */
      for (int i = j + 1; i < n; ++i) Ainv[i + n * j] = Ainv[j + n * i];
  }
  free(U);
  return rc;
}

int orc_hdg_elem_mat(const OrcHdgMesh* H, double* ehat, double* inv_dhat, double* smat, double* tau_out) {
  Tables T;
  make_tables(H->N, H->xgp, H->wgp, &T);
  const int N = T.N, nd = T.nd, nv = T.nv, nf = T.nf;
  if (nd > ORC_HDG_MAXND) return 1;
  double* Dhat = (double*)malloc(sizeof(double) * nv * nv);
  double* Stmp1 = (double*)malloc(sizeof(double) * nv * nf);
  double Stmp2[ORC_HDG_MAXNF * ORC_HDG_MAXNF];
  double surf[6][ORC_HDG_MAXND][ORC_HDG_MAXND];   /* SurfElemLoc(p,q,s) -> surf[s][q][p] */
  int rc = 0;
  for (int e = 0; e < H->ne && !rc; ++e) {
    const int32_t* e2s = H->e2s + 12 * e;          /* ElemToSide(1:2,1:6,e) */
    int flip[6];
    for (int s = 0; s < 6; ++s) flip[s] = e2s[2 * s + 1];
    const double* Mf = H->mf + (size_t)3 * nv * e;
    const double* Mg = H->mg + (size_t)3 * nv * e;
    const double* Mh = H->mh + (size_t)3 * nv * e;
    const double* sJ = H->sj + (size_t)nv * e;
    double* Eh = ehat + (size_t)nf * nv * 6 * e;       /* Ehat(nf,nv,6)   */
    double* Sm = smat + (size_t)nf * nf * 36 * e;      /* Smat(nf,nf,6,6) */
    double* Di = inv_dhat + (size_t)nv * nv * e;
    for (int i = 0; i < nf * nv * 6; ++i) Eh[i] = 0.0;
    for (int i = 0; i < nf * nf * 36; ++i) Sm[i] = 0.0;
    /* Tau(iElem) = 2/(SUM(JwGP_vol))**(1/3) (hdg.f90:527) */
    double vol = 0.0;
    for (int k = 0; k < nd; ++k)
      for (int j = 0; j < nd; ++j)
        for (int i = 0; i < nd; ++i) {
          int r = vidx(i, j, k, nd);
          vol = vol + T.w[i] * T.w[j] * T.w[k] / sJ[r];
        }
    const double tau = 2.0 / pow(vol, 1.0 / 3.0);
    if (tau_out) tau_out[e] = tau;
    /* SurfElemLoc: |Ja^dir| prolonged to each side in master coordinates (elem_mat.f90:103-121) */
    for (int s = 0; s < 6; ++s) {
      const double* Ja = (kSideDir[s] == 0) ? Mf : (kSideDir[s] == 1) ? Mg : Mh;
      const double* L = kPm[s] ? T.Lp : T.Lm;
      double face[ORC_HDG_MAXND][ORC_HDG_MAXND][3];   /* Uface(:,ps,qs) -> face[qs][ps] */
      for (int qs = 0; qs < nd; ++qs)
        for (int ps = 0; ps < nd; ++ps)
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
            for (int c = 0; c < 3; ++c)
              face[qs][ps][c] = (l == 0) ? u[c] * L[0] : face[qs][ps][c] + u[c] * L[l];
          }
      for (int q = 0; q < nd; ++q)
        for (int p = 0; p < nd; ++p) {
          int ps, qs;
          switch (flip[s]) {     /* USide(:,p,q) = Uface(:,...) (prolongtoface.f90:527-553) */
            case 0: ps = p; qs = q; break;
            case 1: ps = q; qs = p; break;
            case 2: ps = N - p; qs = q; break;
            case 3: ps = N - q; qs = N - p; break;
            default: ps = p; qs = N - q; break;
          }
          const double* v = face[qs][ps];
          surf[s][q][p] = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        }
    }
    for (int i = 0; i < nv * nv; ++i) Dhat[i] = 0.0;
    for (int g3 = 0; g3 < nd; ++g3)
      for (int g2 = 0; g2 < nd; ++g2)
        for (int g1 = 0; g1 < nd; ++g1) {
          const int gr = vidx(g1, g2, g3, nd);
          const double* f = Mf + 3 * gr;
          const double* g = Mg + 3 * gr;
          const double* h = Mh + 3 * gr;
          double K[3][3];
          K[0][0] = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
          K[1][1] = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
          K[2][2] = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
          K[1][0] = g[0] * f[0] + g[1] * f[1] + g[2] * f[2];
          K[2][0] = h[0] * f[0] + h[1] * f[1] + h[2] * f[2];
          K[2][1] = h[0] * g[0] + h[1] * g[1] + h[2] * g[2];
          K[0][1] = K[1][0]; K[0][2] = K[2][0]; K[1][2] = K[2][1];
          const double sc = sJ[gr] * (T.w[g1] * T.w[g2] * T.w[g3]);
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) K[a][b] = sc * K[a][b];
          double TauS[2][3];
          for (int s = 0; s < 6; ++s) {
            int p, q, l1, l2;
            vol_to_side(N, g1, g2, g3, flip[s], s, &p, &q);
            vol_to_side_ijk(g1, g2, g3, s, &l1, &l2);
            TauS[kPm[s]][kSideDir[s]] = T.w[l1] * T.w[l2] * surf[s][q][p];
          }
          for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 3; ++b) TauS[a][b] = TauS[a][b] * tau;
          const int gdx[3] = {g1, g2, g3};
          /* D surface contribution */
          for (int iDir = 0; iDir < 3; ++iDir) {
            int idx[3] = {g1, g2, g3};
            for (int l = 0; l < nd; ++l) {
              idx[iDir] = l;
              const int i = vidx(idx[0], idx[1], idx[2], nd);
              Dhat[i + nv * gr] = Dhat[i + nv * gr] -
                  (TauS[0][iDir] * T.LLm[l][gdx[iDir]] + TauS[1][iDir] * T.LLp[l][gdx[iDir]]);
            }
          }
          /* [- B A^{-1} B^T] */
          for (int jDir = 0; jDir < 3; ++jDir) {
            int jdx[3] = {g1, g2, g3};
            for (int q = 0; q < nd; ++q) {
              jdx[jDir] = q;
              const int j = vidx(jdx[0], jdx[1], jdx[2], nd);
              for (int iDir = 0; iDir < 3; ++iDir) {
                int idx[3] = {g1, g2, g3};
                for (int p = 0; p < nd; ++p) {
                  idx[iDir] = p;
                  const int i = vidx(idx[0], idx[1], idx[2], nd);
                  Dhat[i + nv * j] = Dhat[i + nv * j] - K[iDir][jDir] * T.Dom[p][gdx[iDir]] * T.Dom[q][gdx[jDir]];
                }
              }
            }
          }
          /* Ehat = E - B A^{-1} C^T */
          for (int iDir = 0; iDir < 3; ++iDir) {
            const int mS = kDirPm[iDir][0], pS = kDirPm[iDir][1];
            int p, q;
            vol_to_side(N, g1, g2, g3, flip[mS], mS, &p, &q);
            const int i_m = q * nd + p;
            vol_to_side(N, g1, g2, g3, flip[pS], pS, &p, &q);
            const int i_p = q * nd + p;
            double* Em = Eh + (size_t)nf * nv * mS;
            double* Ep = Eh + (size_t)nf * nv * pS;
            const int gi = gdx[iDir];
            Em[i_m + nf * gr] = Em[i_m + nf * gr] + TauS[0][iDir] * T.w[gi] * (-T.Lom_m[gi]);
            Ep[i_p + nf * gr] = Ep[i_p + nf * gr] + TauS[1][iDir] * T.w[gi] * (T.Lom_p[gi]);
            for (int qq = 0; qq < nd; ++qq) {
              int j = vidx(qq, g2, g3, nd);
              Em[i_m + nf * j] = Em[i_m + nf * j] + K[0][iDir] * T.Dom[qq][g1] * T.Lom_m[gi];
              Ep[i_p + nf * j] = Ep[i_p + nf * j] + K[0][iDir] * T.Dom[qq][g1] * T.Lom_p[gi];
              j = vidx(g1, qq, g3, nd);
              Em[i_m + nf * j] = Em[i_m + nf * j] + K[1][iDir] * T.Dom[qq][g2] * T.Lom_m[gi];
              Ep[i_p + nf * j] = Ep[i_p + nf * j] + K[1][iDir] * T.Dom[qq][g2] * T.Lom_p[gi];
              j = vidx(g1, g2, qq, nd);
              Em[i_m + nf * j] = Em[i_m + nf * j] + K[2][iDir] * T.Dom[qq][g3] * T.Lom_m[gi];
              Ep[i_p + nf * j] = Ep[i_p + nf * j] + K[2][iDir] * T.Dom[qq][g3] * T.Lom_p[gi];
            }
          }
          /* Smat: C A^{-1} C^T */
          for (int jDir = 0; jDir < 3; ++jDir) {
            const int jm = kDirPm[jDir][0], jp = kDirPm[jDir][1];
            int p, q;
            vol_to_side(N, g1, g2, g3, flip[jm], jm, &p, &q);
            const int j_m = q * nd + p;
            vol_to_side(N, g1, g2, g3, flip[jp], jp, &p, &q);
            const int j_p = q * nd + p;
            for (int iDir = 0; iDir < 3; ++iDir) {
              const int im = kDirPm[iDir][0], ip = kDirPm[iDir][1];
              vol_to_side(N, g1, g2, g3, flip[im], im, &p, &q);
              const int i_m = q * nd + p;
              vol_to_side(N, g1, g2, g3, flip[ip], ip, &p, &q);
              const int i_p = q * nd + p;
              const double kk = K[iDir][jDir];
              const int gi = gdx[iDir], gj = gdx[jDir];
#define SM(a, b, is, js) Sm[(a) + nf * ((b) + nf * ((is) + 6 * (js)))]
              SM(i_m, j_m, im, jm) = SM(i_m, j_m, im, jm) + kk * T.Lom_m[gi] * T.Lom_m[gj];
              SM(i_p, j_m, ip, jm) = SM(i_p, j_m, ip, jm) + kk * T.Lom_p[gi] * T.Lom_m[gj];
              SM(i_m, j_p, im, jp) = SM(i_m, j_p, im, jp) + kk * T.Lom_m[gi] * T.Lom_p[gj];
              SM(i_p, j_p, ip, jp) = SM(i_p, j_p, ip, jp) + kk * T.Lom_p[gi] * T.Lom_p[gj];
            }
          }
        }
    /* InvDhat = -getSPDInverse(-Dhat) */
    for (int i = 0; i < nv * nv; ++i) Dhat[i] = -Dhat[i];
    if (spd_inverse(nv, Dhat, Di)) { rc = 2; break; }
    for (int i = 0; i < nv * nv; ++i) Di[i] = -Di[i];
    /* Smat += Ehat InvDhat Ehat^T, minus the side mass term */
    for (int jS = 0; jS < 6; ++jS) {
      const double* Ej = Eh + (size_t)nf * nv * jS;
      for (int b = 0; b < nf; ++b)
        for (int r = 0; r < nv; ++r) {
          double t = 0.0;
          for (int c = 0; c < nv; ++c) t = t + Di[r + nv * c] * Ej[b + nf * c];
          Stmp1[r + nv * b] = t;
        }
      for (int iS = jS; iS < 6; ++iS) {
        const double* Ei = Eh + (size_t)nf * nv * iS;
        for (int b = 0; b < nf; ++b)
          for (int a = 0; a < nf; ++a) {
            double t = 0.0;
            for (int r = 0; r < nv; ++r) t = t + Ei[a + nf * r] * Stmp1[r + nv * b];
            Stmp2[a + nf * b] = t;
          }
        if (iS == jS) {
          for (int b = 0; b < nf; ++b)
            for (int a = 0; a < nf; ++a) SM(a, b, jS, jS) = SM(a, b, jS, jS) + Stmp2[a + nf * b];
          for (int q = 0; q < nd; ++q)
            for (int p = 0; p < nd; ++p) {
              const int i = q * nd + p;
              const double fd = -tau * T.w[p] * T.w[q] * surf[jS][q][p];
              SM(i, i, jS, jS) = SM(i, i, jS, jS) - fd;
            }
        } else {
          for (int b = 0; b < nf; ++b)
            for (int a = 0; a < nf; ++a) {
              SM(a, b, iS, jS) = SM(a, b, iS, jS) + Stmp2[a + nf * b];
              SM(b, a, jS, iS) = SM(b, a, jS, iS) + Stmp2[a + nf * b];
            }
        }
      }
    }
#undef SM
  }
  free(Dhat);
  free(Stmp1);
  return rc;
}

/* ---- HDGLinear ---------------------------------------------------------------------------------- */
typedef struct {
  const OrcHdgMesh* H;
  int nf, nv, nd;
  const double* ehat; const double* inv_dhat; const double* smat;
  const uint8_t* masked;   /* Dirichlet sides */
  int zero_side;           /* ZeroPotentialSide (0-based) or -1 */
} Sys;

static void matvec(const Sys* S, const double* x, double* y) {
  const OrcHdgMesh* H = S->H;
  const int nf = S->nf;
  double tmp[ORC_HDG_MAXNF];
  for (size_t i = 0; i < (size_t)H->n_sides * nf; ++i) y[i] = 0.0;
  for (int sid = 0; sid < H->n_sides; ++sid) {
    const int32_t* se = H->s2e + 5 * sid;
    for (int m = 0; m < 2; ++m) {                           /* master, then neighbour */
      const int loc = se[m ? 3 : 2] - 1;
      if (se[m ? 3 : 2] == -1) continue;
      const int e = se[m ? 1 : 0] - 1;
      const double* lam = x + (size_t)nf * sid;
      const double* Sm = S->smat + (size_t)nf * nf * 36 * e;
      for (int jl = 0; jl < 6; ++jl) {
        const int s2 = H->e2s[12 * e + 2 * jl] - 1;
        const double* blk = Sm + (size_t)nf * nf * (jl + 6 * loc);    /* Smat(:,:,jLocSide,locSideID) */
        for (int a = 0; a < nf; ++a) tmp[a] = 0.0;
        for (int b = 0; b < nf; ++b) {
          const double t = lam[b];
          for (int a = 0; a < nf; ++a) tmp[a] = tmp[a] + t * blk[a + nf * b];
        }
        for (int a = 0; a < nf; ++a) y[(size_t)nf * s2 + a] = y[(size_t)nf * s2 + a] + tmp[a];
      }
    }
  }
  for (int sid = 0; sid < H->n_sides; ++sid)
    if (S->masked[sid])
      for (int a = 0; a < nf; ++a) y[(size_t)nf * sid + a] = 0.0;
  if (S->zero_side >= 0) y[(size_t)nf * S->zero_side] = 0.0;
}

static double dot(const double* a, const double* b, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s = s + a[i] * b[i];
  return s;
}

int orc_hdg_solve(const OrcHdgMesh* H, const double* ehat, const double* inv_dhat, const double* smat,
                  int precond_type, double eps_cg, int max_iter_cg, int use_relative, const double* resu,
                  const double* lambda_dirichlet, double* lambda, double* U, double* E, int* iterations,
                  double* norm_out) {
  Tables T;
  make_tables(H->N, H->xgp, H->wgp, &T);
  const int N = T.N, nd = T.nd, nv = T.nv, nf = T.nf, ns = H->n_sides;
  const size_t nl = (size_t)ns * nf;
  Sys S = {H, nf, nv, nd, ehat, inv_dhat, smat, NULL, -1};
  uint8_t* masked = (uint8_t*)calloc(ns, 1);
  for (int i = 0; i < H->n_dir; ++i) masked[H->dir_sides[i] - 1] = 1;
  S.masked = masked;
  if (H->n_dir == 0) S.zero_side = H->e2s[0] - 1;         /* ElemToSide(E2S_SIDE_ID,1,1) */
  double* rhs_vol = (double*)malloc(sizeof(double) * nv * H->ne);
  double* rhs_face = (double*)calloc(nl, sizeof(double));
  double* R = (double*)malloc(sizeof(double) * nl);
  double* V = (double*)malloc(sizeof(double) * nl);
  double* Z = (double*)malloc(sizeof(double) * nl);
  double* P = NULL;
  double* Pdiag = NULL;
  double rt[ORC_HDG_MAXNV], ft[ORC_HDG_MAXNF];
  int rc = 0;
  /* Dirichlet values and the zero-potential DOF */
  for (int i = 0; i < H->n_dir; ++i)
    for (int a = 0; a < nf; ++a) lambda[(size_t)nf * (H->dir_sides[i] - 1) + a] = lambda_dirichlet ? lambda_dirichlet[(size_t)nf * i + a] : 0.0;
  if (S.zero_side >= 0) lambda[(size_t)nf * S.zero_side] = 0.0;
  /* RHS_vol = -JwGP_vol * resu; RHS_face = sum over elements of Ehat InvDhat (-RHS_vol) */
  for (int e = 0; e < H->ne; ++e) {
    const double* sJ = H->sj + (size_t)nv * e;
    double* rv = rhs_vol + (size_t)nv * e;
    for (int k = 0; k < nd; ++k)
      for (int j = 0; j < nd; ++j)
        for (int i = 0; i < nd; ++i) {
          const int r = vidx(i, j, k, nd);
          const double jw = T.w[i] * T.w[j] * T.w[k] / sJ[r];
          rv[r] = -jw * resu[(size_t)nv * e + r];
        }
    const double* Di = inv_dhat + (size_t)nv * nv * e;
    for (int r = 0; r < nv; ++r) rt[r] = 0.0;
    for (int c = 0; c < nv; ++c) {
      const double t = -rv[c];
      for (int r = 0; r < nv; ++r) rt[r] = rt[r] + t * Di[r + nv * c];
    }
    for (int s = 0; s < 6; ++s) {
      const double* Es = ehat + (size_t)nf * nv * (s + 6 * e);
      for (int a = 0; a < nf; ++a) ft[a] = 0.0;
      for (int c = 0; c < nv; ++c) {
        const double t = rt[c];
        for (int a = 0; a < nf; ++a) ft[a] = ft[a] + t * Es[a + nf * c];
      }
      const int sid = H->e2s[12 * e + 2 * s] - 1;
      for (int a = 0; a < nf; ++a) rhs_face[(size_t)nf * sid + a] = rhs_face[(size_t)nf * sid + a] + ft[a];
    }
  }
  /* BuildPrecond */
  if (precond_type == 1) {
    P = (double*)calloc((size_t)ns * nf * nf, sizeof(double));
    for (int sid = 0; sid < ns && !rc; ++sid) {
      const int32_t* se = H->s2e + 5 * sid;
      double* Ps = P + (size_t)nf * nf * sid;
      for (int m = 0; m < 2; ++m) {
        if (se[m ? 3 : 2] == -1) continue;
        const int e = se[m ? 1 : 0] - 1, loc = se[m ? 3 : 2] - 1;
        const double* blk = smat + (size_t)nf * nf * (36 * e + loc + 6 * loc);
        for (int i = 0; i < nf * nf; ++i) Ps[i] = Ps[i] + blk[i];
      }
      if (!masked[sid] && chol_upper(nf, Ps)) rc = 3;
    }
  } else if (precond_type == 2) {
    Pdiag = (double*)calloc(nl, sizeof(double));
    for (int sid = 0; sid < ns && !rc; ++sid) {
      const int32_t* se = H->s2e + 5 * sid;
      for (int m = 0; m < 2; ++m) {
        if (se[m ? 3 : 2] == -1) continue;
        const int e = se[m ? 1 : 0] - 1, loc = se[m ? 3 : 2] - 1;
        const double* blk = smat + (size_t)nf * nf * (36 * e + loc + 6 * loc);
        for (int a = 0; a < nf; ++a) Pdiag[(size_t)nf * sid + a] = Pdiag[(size_t)nf * sid + a] + blk[a + nf * a];
      }
      if (masked[sid]) continue;
      double mx = 0.0;
      for (int a = 0; a < nf; ++a) mx = fmax(mx, fabs(Pdiag[(size_t)nf * sid + a]));
      if (!(mx > 1.0e-12)) { rc = 3; break; }
      for (int a = 0; a < nf; ++a) Pdiag[(size_t)nf * sid + a] = 1.0 / Pdiag[(size_t)nf * sid + a];
    }
  }
  int it_done = 0;
  double norm_r2 = 0.0;
  if (!rc) {
    /* CG_solver */
    matvec(&S, lambda, Z);                                             /* EvalResidual */
    for (size_t i = 0; i < nl; ++i) R[i] = rhs_face[i] - Z[i];
    for (int sid = 0; sid < ns; ++sid)
      if (masked[sid]) for (int a = 0; a < nf; ++a) R[(size_t)nf * sid + a] = 0.0;
    if (S.zero_side >= 0) R[(size_t)nf * S.zero_side] = 0.0;
    norm_r2 = dot(R, R, nl);
    const int converged0 = use_relative ? (norm_r2 < 1e-16) : (norm_r2 < eps_cg * eps_cg);
    if (!converged0) {
      const double abort2 = use_relative ? norm_r2 * eps_cg * eps_cg : eps_cg * eps_cg;
#define PRECOND(IN, OUT)                                                                         \
      for (int sid = 0; sid < ns; ++sid) {                                                       \
        double* o = OUT + (size_t)nf * sid;                                                      \
        const double* in = IN + (size_t)nf * sid;                                                \
        if (precond_type == 0) { for (int a = 0; a < nf; ++a) o[a] = in[a]; continue; }          \
        if (masked[sid]) { for (int a = 0; a < nf; ++a) o[a] = 0.0; continue; }                  \
        if (precond_type == 1) chol_solve(nf, P + (size_t)nf * nf * sid, in, o);                 \
        else for (int a = 0; a < nf; ++a) o[a] = Pdiag[(size_t)nf * sid + a] * in[a];            \
      }
      PRECOND(R, V)
      double rz1 = dot(R, V, nl);
      int conv = 0;
      for (int iter = 1; iter <= max_iter_cg; ++iter) {
        matvec(&S, V, Z);
        const double vz = dot(V, Z, nl);
        if (fabs(vz) <= 0.0) { rc = 4; it_done = iter; break; }
        const double omega = rz1 / vz;
        for (size_t i = 0; i < nl; ++i) {
          lambda[i] = lambda[i] + omega * V[i];
          R[i] = R[i] - omega * Z[i];
        }
        const double rr = dot(R, R, nl);
        if (isnan(rr)) { rc = 5; it_done = iter; break; }
        it_done = iter;
        norm_r2 = rr;
        if (rr < abort2) { conv = 1; break; }
        PRECOND(R, Z)
        const double rz2 = dot(R, Z, nl);
        const double beta = rz2 / rz1;
        for (size_t i = 0; i < nl; ++i) V[i] = Z[i] + beta * V[i];
        rz1 = rz2;
      }
#undef PRECOND
      if (!conv && !rc) rc = -1;                                       /* not converged: reference warns */
    }
  }
  /* post processing: U = InvDhat (-(RHS_vol + sum_s Ehat_s^T lambda_s)), then the gradient */
  if (rc == 0 || rc == -1) {
    double lam6[6][ORC_HDG_MAXNF];
    for (int e = 0; e < H->ne; ++e) {
      double* rv = rhs_vol + (size_t)nv * e;
      for (int s = 0; s < 6; ++s) {
        const int sid = H->e2s[12 * e + 2 * s] - 1;
        const double* Es = ehat + (size_t)nf * nv * (s + 6 * e);
        for (int c = 0; c < nv; ++c) {
          double t = 0.0;
          for (int a = 0; a < nf; ++a) t = t + Es[a + nf * c] * lambda[(size_t)nf * sid + a];
          rv[c] = rv[c] + t;
        }
        for (int a = 0; a < nf; ++a) lam6[s][a] = lambda[(size_t)nf * sid + a];
      }
      const double* Di = inv_dhat + (size_t)nv * nv * e;
      double* u = U + (size_t)nv * e;
      for (int r = 0; r < nv; ++r) u[r] = 0.0;
      for (int c = 0; c < nv; ++c) {
        const double t = -rv[c];
        for (int r = 0; r < nv; ++r) u[r] = u[r] + t * Di[r + nv * c];
      }
      /* PostProcessGradientHDG */
      const int32_t* e2s = H->e2s + 12 * e;
      const double* sJ = H->sj + (size_t)nv * e;
      const double* M3[3] = {H->mf + (size_t)3 * nv * e, H->mg + (size_t)3 * nv * e, H->mh + (size_t)3 * nv * e};
      double* Eo = E + (size_t)3 * nv * e;
      for (int g3 = 0; g3 < nd; ++g3)
        for (int g2 = 0; g2 < nd; ++g2)
          for (int g1 = 0; g1 < nd; ++g1) {
            const int gr = vidx(g1, g2, g3, nd);
            double ex = 0.0, ey = 0.0, ez = 0.0;
            const int gdx[3] = {g1, g2, g3};
            for (int jDir = 0; jDir < 3; ++jDir) {
              double ql = 0.0;
              int jdx[3] = {g1, g2, g3};
              for (int q = 0; q < nd; ++q) {
                jdx[jDir] = q;
                ql = ql + T.Dom[q][gdx[jDir]] * u[vidx(jdx[0], jdx[1], jdx[2], nd)];
              }
              const int mS = kDirPm[jDir][0], pS = kDirPm[jDir][1];
              int p, q;
              vol_to_side(N, g1, g2, g3, e2s[2 * mS + 1], mS, &p, &q);
              const int idx_m = q * nd + p;
              vol_to_side(N, g1, g2, g3, e2s[2 * pS + 1], pS, &p, &q);
              const int idx_p = q * nd + p;
              ql = ql - T.Lom_m[gdx[jDir]] * lam6[mS][idx_m];
              ql = ql - T.Lom_p[gdx[jDir]] * lam6[pS][idx_p];
              const double* a = M3[jDir] + 3 * gr;
              ex = ex + sJ[gr] * a[0] * ql;
              ey = ey + sJ[gr] * a[1] * ql;
              ez = ez + sJ[gr] * a[2] * ql;
            }
            Eo[3 * gr + 0] = ex;
            Eo[3 * gr + 1] = ey;
            Eo[3 * gr + 2] = ez;
          }
    }
  }
  if (iterations) *iterations = it_done;
  if (norm_out) *norm_out = sqrt(norm_r2);
  free(masked); free(rhs_vol); free(rhs_face); free(R); free(V); free(Z); free(P); free(Pdiag);
  return rc;
}
