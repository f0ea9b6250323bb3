/* pic_oracle_bezier.h -- curved-side intersections of the oracle (test infrastructure; see pic_oracle_bezier.c). */
#ifndef PIC_ORACLE_BEZIER_H
#define PIC_ORACLE_BEZIER_H

#define BZ_MAXN 4
#define BZ_NP (BZ_MAXN + 1)

typedef struct {
  int ng;                           /* NGeo */
  double fnk[BZ_NP][BZ_NP];         /* FacNchooseK(n,k) = C(n,k) / 2^n */
  double xi_ng[BZ_NP];              /* Xi_NGeo: equidistant nodes on [-1,1] */
  double dbez[BZ_NP][BZ_NP];        /* D_Bezier */
} orc_bz_basis_t;

typedef struct {
  orc_bz_basis_t B;
  double cp[BZ_NP * BZ_NP * 3];     /* BezierControlPoints3D(1:3,p,q) at cp[(q*(NGeo+1)+p)*3 + c] */
  double slab_n[3][3];              /* SideSlabNormals(:,i) at slab_n[i] */
  double slab_i[6];                 /* SideSlabIntervals */
  int bb_empty;                     /* BoundingBoxIsEmpty */
} orc_bz_side_t;

void orc_bz_basis_init(orc_bz_basis_t* B, int ng);
int orc_bz_side_init(orc_bz_side_t* S, int ng, const double* bcp);
void orc_bz_normal(const orc_bz_side_t* S, double xi, double eta, double nv[3]);
double orc_bz_planar_curved(const orc_bz_side_t* S, const double nv[3], double dist, const double xl[3],
                            const double traj[3], double len, double* xi, double* eta, int* err);
double orc_bz_curved(const orc_bz_side_t* S, const double nv[3], const double xl[3], const double x[3],
                     const double traj[3], double len, double* xi, double* eta, int* err);

#endif
