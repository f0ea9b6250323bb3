/*
 * pic_oracle.h -- CPU restatement of PICLas's Boris-Leapfrog particle loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked against
 * (tests/, __graft_entry__.smoke() and bench.py's CPU baseline).  Nothing in the
 * piclas_gb300 package links, loads or calls it.
 *
 * Every routine restates the cited reference Fortran in the same floating-point
 * evaluation order (built with -ffp-contract=off, no FMA contraction).  Arrays use the
 * reference's memory layout and 1-based element / species / node indices, and the mesh
 * is passed in the same pic_mesh_t the GPU library takes.
 */
#ifndef PIC_ORACLE_H
#define PIC_ORACLE_H

#include <stdint.h>
#include "../include/piclas_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_particles_t {
  int32_t  n;               /* PDM%ParticleVecLength                       */
  double*  part_state;      /* PartState(1:6,n)                            */
  double*  last_part_pos;   /* LastPartPos(1:3,n)                          */
  double*  part_pos_ref;    /* PartPosRef(1:3,n)                           */
  double*  field;           /* FieldAtParticle(1:6,n)                      */
  int32_t* elem;            /* PEM%GlobalElemID (1-based)                  */
  int32_t* last_elem;       /* PEM%LastGlobalElemID                        */
  int32_t* species;         /* PartSpecies (1-based)                       */
  uint8_t* inside;          /* PDM%ParticleInside                          */
  uint8_t* is_new;          /* PDM%IsNewPart                               */
} orc_particles_t;

typedef struct orc_counters_t {
  int64_t n_lost;           /* NbrOfLostParticles                          */
  int64_t n_newton_failed;  /* isSuccessful=.FALSE. returns                 */
  int64_t n_ref_tolerance;  /* RefTracking tolerance aborts                */
  int64_t n_hop_limit;      /* walks cut by the iteration cap              */
} orc_counters_t;

/* basis.f90:1223-1264 */
void orc_lagrange_polys(double x, int n, const double* xgp, const double* wbary, double* L);
/* eval_xyz.f90:35-123 with GetRefNewtonStartValue (guess 1) and RefElemNewton.
 * Returns 1 if successful (or success not requested), 0 if isSuccessful=.FALSE. */
int orc_get_position_in_ref_elem(const pic_config_t* cfg, const pic_mesh_t* m, const double x[3],
                                 double xi[3], int elem, int want_success);
/* eval_xyz.f90:167-215, NVar_in = 3 */
void orc_evaluate_field_at_ref_pos(const double xi[3], int N, const double* xgp, const double* wbary,
                                   const double* U /*(3,0:N,0:N,0:N)*/, double out[3]);

int  orc_interpolate(const pic_config_t* cfg, const pic_mesh_t* m, const double* e_dof,
                     orc_particles_t* p, orc_counters_t* c, int nthreads);
void orc_push(const pic_config_t* cfg, orc_particles_t* p, double dt, int nthreads);
void orc_track(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, orc_counters_t* c,
               int nthreads);
/* part_source: PS_N(e)%PartSource(1:4,0:N,0:N,0:N) for all e (4*(N+1)^3*nElems) */
int  orc_deposit(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, double* part_source,
                 orc_counters_t* c, int nthreads);
/* nsteps x {Deposition, save LastPartPos, InterpolateFieldToParticle, push, PerformTracking} */
int  orc_step(const pic_config_t* cfg, const pic_mesh_t* m, const double* e_dof, orc_particles_t* p,
              double dt, int nsteps, double* part_source, orc_counters_t* c, int nthreads);

/* VerifyDepositedCharge (pic_analyze.f90:41-133) for NAnalyze = N */
double orc_integrate_charge(const pic_mesh_t* m, int N, const double* part_source);

/* PartPosRef of every particle in its element (insertion-time mapping for RefTracking) */
void orc_map_particles(const pic_config_t* cfg, const pic_mesh_t* m, orc_particles_t* p, int nthreads);

int orc_max_threads(void);

/* ---- HDG Poisson solve (pic_oracle_hdg.c) --------------------------------------------------------- */
#define ORC_HDG_MAXND 6
#define ORC_HDG_MAXNF (ORC_HDG_MAXND * ORC_HDG_MAXND)
#define ORC_HDG_MAXNV (ORC_HDG_MAXNF * ORC_HDG_MAXND)
typedef struct OrcHdgMesh {
  int N, ne, n_sides;
  const int32_t* e2s;        /* ElemToSide(1:2,1:6,nElems): SideID (1-based), flip */
  const int32_t* s2e;        /* SideToElem(1:5,nSides), -1 = none                  */
  const double* mf;          /* Metrics_fTilde(1:3,0:N,0:N,0:N,nElems)             */
  const double* mg;
  const double* mh;
  const double* sj;          /* sJ(0:N,0:N,0:N,nElems)                             */
  const double* xgp;         /* Gauss nodes and weights                            */
  const double* wgp;
  int n_dir;                 /* nDirichletBCSides                                  */
  const int32_t* dir_sides;  /* DirichletBC(:), 1-based                            */
} OrcHdgMesh;
/* Elem_Mat: Ehat(nf,nv,6), InvDhat(nv,nv), Smat(nf,nf,6,6) per element; Tau per element.  0 = ok */
int orc_hdg_elem_mat(const OrcHdgMesh* H, double* ehat, double* inv_dhat, double* smat, double* tau);
/* HDGLinear with CG_solver: resu = CalcSourceHDG at every volume point (nv,nElems); lambda (nf,nSides)
 * is the start value and the result; U (nv,nElems), E (3,nv,nElems).  0 ok, -1 not converged,
 * >0 failure (3 preconditioner, 4 vz = 0, 5 NaN residual) */
int orc_hdg_solve(const OrcHdgMesh* H, const double* ehat, const double* inv_dhat, const double* smat,
                  int precond_type, double eps_cg, int max_iter_cg, int use_relative, const double* resu,
                  const double* lambda_dirichlet, double* lambda, double* U, double* E, int* iterations,
                  double* norm_out);

#ifdef __cplusplus
}
#endif
#endif
