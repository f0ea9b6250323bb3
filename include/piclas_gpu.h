/*
 * piclas_gpu.h -- C-ABI of the GB300 (sm_103a) PIC particle loop.
 *
 * The entry points replace the argument-less Fortran routines of PICLas's
 * Boris-Leapfrog particle loop.  A Fortran host binds them with ISO_C_BINDING
 * (BIND(C) interfaces with the same names); every pointer is a plain host pointer to a contiguous
 * array laid out exactly like the reference's Fortran array (column-major,
 * first index fastest).  Index arrays are 1-based, as in the reference.
 *
 * Reference routines replaced (paths relative to the PICLas source tree):
 *   pic_create             InitParticleMesh / InitializeDeposition / InitializeParticleInterpolation
 *                          (src/particles/particle_mesh/particle_mesh.f90:141,
 *                           src/particles/pic/deposition/pic_depo.f90:83,
 *                           src/particles/pic/interpolation/pic_interpolation.f90:105)
 *   pic_set_field          hand-over of U_N(e)%E(1:3,0:N,0:N,0:N) after HDG()
 *                          (src/timedisc/timedisc_TimeStepPoissonByBorisLeapfrog.f90:99)
 *   pic_upload_particles / pic_download_particles
 *                          PartState(1:6,:), PEM%GlobalElemID, PartSpecies, PDM%ParticleInside,
 *                          PDM%IsNewPart, PartPosRef (src/particles/particle_vars.f90:50-167)
 *   pic_interpolate        InterpolateFieldToParticle (pic_interpolation.f90:248)
 *   pic_push               LastPartPos/LastElem save + Boris push loop
 *                          (timedisc_TimeStepPoissonByBorisLeapfrog.f90:109-198)
 *   pic_track              PerformTracking (src/particles/tracking/particle_tracking.f90:32)
 *   pic_deposit            Deposition (src/particles/pic/deposition/pic_depo.f90:944)
 *   pic_step               TimeStepPoissonByBorisLeapfrog with the field frozen
 *                          (timedisc_TimeStepPoissonByBorisLeapfrog.f90:32-286 minus HDG)
 *   pic_get_status         NbrOfLostParticles and the abort conditions of the loop
 *                          (particle_triatracking.f90:293-308, eval_xyz.f90:424-441)
 *   pic_get_part_data / pic_set_part_data
 *                          FillParticleData and the particle read-in of a restart
 *                          (src/io_hdf5/hdf5_output_particle.f90:1531, src/particles/restart/particle_readin.f90)
 *   pic_get_field_at_particles  FieldAtParticle(1:6,:) (src/particles/pic/interpolation/pic_interpolation_vars.f90:26)
 *   pic_verify_deposited_charge VerifyDepositedCharge (src/particles/pic/analyze/pic_analyze.f90:41)
 *   pic_hdg_init           InitHDG + Elem_Mat + BuildPrecond (src/hdg/hdg.f90:90, src/hdg/elem_mat.f90:42,513)
 *   pic_hdg_set_dirichlet  the Dirichlet branch of HDGLinear (src/hdg/hdg_linear.f90:96-150)
 *   pic_hdg_solve          HDG -> HDGLinear -> CG_solver + PostProcessGradientHDG
 *                          (src/hdg/hdg.f90:734, hdg_linear.f90:37, src/hdg/hdg_tools.f90:41, elem_mat.f90:621);
 *                          with pic_hdg_t.solve_in_step, pic_step calls it after every Deposition
 *                          (timedisc_TimeStepPoissonByBorisLeapfrog.f90:99)
 *   pic_hdg_get_lambda / pic_hdg_set_lambda / pic_hdg_get_elem_mat
 *                          HDG_Surf_N(:)%lambda, HDG_Vol_N(e)%Ehat/InvDhat/Smat (src/hdg/hdg_vars.f90)
 *   pic_adjoint_run        no reference counterpart (differentiable loop, see its comment)
 *   pic_deposit_cvwm_noalloc, pic_profile*, pic_launch_count, pic_stream, pic_fp64_fma_rate, pic_fp32_fma_rate
 *                          no reference counterpart (allocation-free entry point, instrumentation)
 *
 * Error convention: every int-returning call returns PIC_OK (0) or a positive
 * pic_error_t.  The library never aborts the host process: where the reference
 * calls abort(), the library records an error bit in the status word instead.
 */
#ifndef PICLAS_GPU_H
#define PICLAS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes (return values) --------------------------------------- */
typedef enum pic_error_t {
  PIC_OK = 0,
  PIC_ERR_INVALID_ARGUMENT = 1,  /* null pointer, bad size, unsupported option          */
  PIC_ERR_CUDA = 2,              /* a CUDA runtime call failed (message in pic_last_error) */
  PIC_ERR_OUT_OF_MEMORY = 3,     /* device allocation failed                             */
  PIC_ERR_NO_DEVICE = 4,         /* no CUDA device visible                               */
  PIC_ERR_STATE = 5,             /* call out of order (e.g. deposit before upload)       */
  PIC_ERR_CAPACITY = 6           /* more particles than pic_config_t.max_particles       */
} pic_error_t;

/* ---- status bits (pic_status_t.error_word), set by device code ------------- */
#define PIC_STATUS_LOST_PARTICLE   0x01u  /* TriaTracking found no side: particle removed  */
#define PIC_STATUS_NEWTON_FAILED   0x02u  /* Newton left |xi|>1.5 (isSuccessful=.FALSE.)    */
#define PIC_STATUS_HOP_LIMIT       0x04u  /* tracking walk exceeded its iteration cap      */
#define PIC_STATUS_REF_TOLERANCE   0x08u  /* RefTracking: |xi| > epsOneCell (reference aborts) */
#define PIC_STATUS_BAD_ELEMENT     0x10u  /* element index out of range in particle data   */
#define PIC_STATUS_NOT_FINITE      0x20u  /* NaN/Inf position or velocity                  */
#define PIC_STATUS_CG_NOT_CONVERGED 0x40u /* HDG CG reached MaxIterCG (reference: warning)    */
#define PIC_STATUS_CG_BREAKDOWN    0x80u  /* HDG CG: v.z = 0 or NaN residual (reference aborts) */
#define PIC_STATUS_WAIT_TIMEOUT    0x100u /* a kernel's bounded wait on its own copies gave up (no reference
                                             counterpart; the kernel's output is then incomplete)         */

/* ---- option enums ------------------------------------------------------- */
enum { PIC_TRACK_TRIA = 1, PIC_TRACK_REFMAPPING = 2 };     /* TrackingMethod           */
/* PIC-Deposition-Type: cell_volweight_mean, shape_function, shape_function_cc (charge-corrected: each
 * particle's deposit scaled so that its quadrature integral is exactly q*MPF; with three periodic
 * vectors over the 27 images, without any over the DOFs left inside the walls), shape_function_adaptive (as
 * _cc with the radius of the particle's element, pic_mesh_t.sf_elem_radius; without periodic vectors only
 * on the particle's element and the elements sharing a corner node with it) */
enum { PIC_DEPO_CVWM = 1, PIC_DEPO_SHAPE_FUNCTION = 2, PIC_DEPO_SHAPE_FUNCTION_CC = 3,
       PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE = 4 };
enum { PIC_PREC_FP64 = 0, PIC_PREC_MIXED = 1 };            /* arithmetic variant       */

#define PIC_MAX_SPECIES 8

/* Run-time options (the ini parameters the path reads). */
typedef struct pic_config_t {
  int32_t n_dg;                 /* N: DG polynomial degree (1..4; NMax with p-adaption)  */
  int32_t tracking;             /* PIC_TRACK_*                                          */
  int32_t deposition;           /* PIC_DEPO_*                                           */
  int32_t precision;            /* PIC_PREC_*                                           */
  int32_t max_particles;        /* capacity of the device particle arrays               */
  int32_t n_species;            /* 1..PIC_MAX_SPECIES                                   */
  double  charge[PIC_MAX_SPECIES];   /* Species(s)%ChargeIC                            */
  double  mass[PIC_MAX_SPECIES];     /* Species(s)%MassIC                              */
  double  mpf[PIC_MAX_SPECIES];      /* Species(s)%MacroParticleFactor                 */
  double  external_field[6];    /* PIC-externalField (Ex,Ey,Ez,Bx,By,Bz)                */
  double  refmapping_eps;       /* RefMappingEps (default 1e-4)                         */
  double  sf_radius;            /* PIC-shapefunction-radius                             */
  int32_t sf_alpha;             /* PIC-shapefunction-alpha (>=2)                        */
  int32_t sort_interval;        /* re-sort particles by element every k steps (0: never) */
  /* PIC-shapefunction-dimension (1, 2, 3; 0 = 3), -direction (1D: the direction of the kernel, 2D: the
   * direction in which it is constant) and -3D-deposition (1: charge over the volume, 0: over the line /
   * area); for every shape-function deposition (InitShapeFunctionDimensionalty,
   * pic_depo_shapefunction_tools.f90:1131-1294) */
  int32_t sf_dim;
  int32_t sf_dir;
  int32_t sf_depo3d;
  /* Part-Species[s]-TimeStepFactor with Part-VariableTimeStep-...-Species (VarTimeStep%UseSpeciesSpecific):
   * the push of species s advances by dt * factor (timedisc_TimeStepPoissonByBorisLeapfrog.f90:130-135);
   * 0 = not set = 1; a factor above 1 is rejected (PIC_ERR_INVALID_ARGUMENT), as the reference stops on it
   * (particle_emission_init.f90:218-219) */
  double  time_step_factor[PIC_MAX_SPECIES];
  /* RefTracking on meshes with periodic sides: 0 = CartesianPeriodic = T with FastPeriodic (a particle that
   * left the box is moved back by the periodic vectors, PeriodicMovement, particle_reftracking.f90:697-985);
   * 1 = CartesianPeriodic = F, the reference's default (particle_mesh.f90:97-101): periodic sides are BC
   * sides traced by ParticleBCTracking, a crossing moves the particle by the side's periodic vector into the
   * neighbour element (GetBoundaryInteraction -> PeriodicBoundary, particle_boundary_condition.f90:184-186,
   * 224-284).  With 1 the BC-element lists (pic_mesh_t.elem_to_bc_sides ...) must include the periodic sides
   * (BuildBCElemDistance counts every side with SIDE_BCID > 0); open/reflective walls may then be combined
   * with periodic sides. */
  int32_t periodic_tracing;
  /* RefMappingGuess, the start value of the Newton x -> xi (GetRefNewtonStartValue, eval_xyz.f90:498-612):
   * 1 = linear pseudo-Cartesian coordinates (the reference's default on linear meshes, particle_mesh.f90:
   * 350-366), 2 = xi of the element's closest Gauss point (Elem_xGP at the element's degree), 3 = xi of the
   * closest XCL_NGeo point (the corners at NGeo = 1), 4 = (0,0,0); 0 = 1. */
  int32_t ref_mapping_guess;
} pic_config_t;

/* Mesh arrays as the reference holds them after init (NGeo = 1 hexahedra).
 * Shapes are given in the reference's Fortran notation; memory is column-major. */
typedef struct pic_mesh_t {
  int32_t n_elems;              /* nElems                                               */
  int32_t n_geo;                /* NGeo (1..4; NGeo > 1: see elem_curved)                */
  int32_t n_nodes;              /* nUniqueGlobalNodes (periodic copies are distinct)    */
  int32_t n_periodic_vectors;   /* GEO%nPeriodicVectors (0..3)                          */
  double  periodic_vectors[9];  /* GEO%PeriodicVectors(1:3,1:3)                         */
  double  xmin_glob[3], xmax_glob[3];  /* GEO%x/y/zminglob, x/y/zmaxglob                */
  /* reference-element data */
  const double* xi_cl_ngeo;     /* XiCL_NGeo(0:NGeo)                                    */
  const double* wbary_cl_ngeo;  /* wBaryCL_NGeo(0:NGeo)                                 */
  const double* xgp;            /* N_Inter(N)%xGP(0:N)  Gauss nodes                     */
  const double* wgp;            /* N_Inter(N)%wGP(0:N)                                  */
  const double* wbary_gp;       /* N_Inter(N)%wBary(0:N)                                */
  /* element geometry */
  const double* xcl_ngeo;       /* XCL_NGeo(1:3,0:NGeo,0:NGeo,0:NGeo,nElems) at XiCL_NGeo */
  const double* dxcl_ngeo;      /* dXCL_NGeo(1:3,1:3,0:NGeo,0:NGeo,0:NGeo,nElems)        */
  const double* elem_bary;      /* ElemBaryNGeo(1:3,nElems)                             */
  const double* xez_basis;      /* XiEtaZetaBasis(1:3,1:6,nElems)                       */
  const double* slen_basis;     /* slenXiEtaZetaBasis(1:6,nElems)                       */
  const double* elem_radius;    /* ElemRadiusNGeo(nElems)                               */
  const double* eps_one_cell;   /* ElemEpsOneCell(nElems)                               */
  const double* elem_xgp;       /* Elem_xGP_Shared(1:3,(N+1)^3*nElems)                  */
  const double* elem_sj;        /* ElemsJ((N+1)^3*nElems)                               */
  /* linear-element connectivity (TriaTracking) */
  const double* node_coords;    /* NodeCoords_Shared(1:3,8*nElems): corners, tensor order */
  const int32_t* elem_node;     /* ElemNodeID_Shared(1:8,nElems): CGNS corner order, 1-based into node_coords */
  const int32_t* elem_side_node;/* ElemSideNodeID_Shared(1:4,1:6,nElems)+1, 1-based into node_coords */
  const int32_t* side_nb_elem;  /* SideInfo_Shared(SIDE_NBELEMID) per (1:6,nElems), 1-based; 0 at walls */
  const int32_t* side_pvid;     /* BoundaryType(SIDE_BCID,BC_ALPHA) per (1:6,nElems): 0 inner, +-k periodic */
  const int32_t* concave_side;  /* ConcaveElemSide_Shared(1:6,nElems) as 0/1             */
  /* cell_volweight_mean */
  const int32_t* node_info;     /* NodeInfo_Shared(ElemNodeID(1:8,e)) per (1:8,nElems): unique node, 1-based */
  const double* node_volume;    /* NodeVolume(nUniqueGlobalNodes)                       */
  const int32_t* periodic_n_nodes;   /* Periodic_nNodes(nUniqueGlobalNodes)            */
  const int32_t* periodic_offset;    /* Periodic_offsetNode(nUniqueGlobalNodes)        */
  const int32_t* periodic_nodes;     /* Periodic_Nodes(nTotalPeriodicNodes), 1-based    */
  int32_t n_total_periodic_nodes;
  /* Fast-Init background mesh (RefTracking candidates, shape-function search) */
  int32_t fibgm_imax[3];        /* FIBGMimax/jmax/kmax (imin=jmin=kmin=1)               */
  double  fibgm_deltas[3];      /* GEO%FIBGMdeltas                                      */
  const int32_t* fibgm_n_elems; /* FIBGM_nElems(i,j,k)                                  */
  const int32_t* fibgm_offset;  /* FIBGM_offsetElem(i,j,k)                              */
  const int32_t* fibgm_element; /* FIBGM_Element(:), 1-based                            */
  int32_t fibgm_n_total;
  /* particle boundaries of non-periodic sides (TriaTracking + cell_volweight_mean only):
   * PartBound%TargetBoundCond of the side's BC per (1:6,nElems): 1 open (RemoveParticle),
   * 2 reflective (PerfectReflection: MomentumACC = 0, no wall velocity), 0 for inner and periodic
   * sides; a side with side_nb_elem = 0 must be 1 or 2.  NULL: every side is inner or periodic. */
  const int32_t* side_bc;
  /* shape_function_adaptive: SFElemr2_Shared(1,nElems), the shape-function radius of each element
   * (InitShapeFunctionAdaptive, pic_depo.f90:727-815); NULL otherwise */
  const double* sf_elem_radius;
  /* RefTracking with BC sides -- open/reflective walls, and with pic_config_t.periodic_tracing = 1 also the
   * periodic sides: the BC-element lists of BuildBCElemDistance (particle_mesh_build.f90:645-1092).
   * elem_to_bc_sides(1:2, nElems) = (ELEM_NBR_BCSIDES, ELEM_FIRST_BCSIDE): the number of BC sides in reach of
   * the element and the 0-based first entry, -1/-1 for none; entry k (sorted by distance within an element)
   * is the BC side bc_side_elem_loc(1:2,k) = (element 1-based, local side 1..6) with
   * SideBCMetrics(BCSIDE_DISTANCE) = bc_side_distance(k).  Sides may be planar (rectangular or not) or
   * bilinear.  NULL/0 for TriaTracking, or for periodic meshes with periodic_tracing = 0. */
  int32_t n_bc_entries;
  const int32_t* elem_to_bc_sides;
  const int32_t* bc_side_elem_loc;
  const double* bc_side_distance;
  /* per-element polynomial degree (p-adaption, dg_vars.f90:38): N_DG_Mapping(1:3, nElems) -- row 1 the
   * element's 0-based offset into the DOF arrays (the running sum of (Nloc+1)^3 over the elements before it,
   * Set_N_DG_Mapping, mesh_pAdaption.f90:391-414), row 2 its degree Nloc in 1..pic_config_t.n_dg (n_dg is
   * then NMax), row 3 (the compute-node offset) is not read -- and n_inter = N_Inter(Nloc)%xGP(0:Nloc),
   * %wGP(0:Nloc), %wBary(0:Nloc) for Nloc = 1..n_dg, one block of 3 (Nloc+1) values per degree in that order.
   * With a mapping every per-DOF array is packed by row 1 (each element's (0:Nloc)^3 block in turn,
   * nDofsMapping DOFs in all): elem_xgp, elem_sj, the field of pic_set_field (U_N(e)%E) and PartSource
   * (PS_N(e)%PartSource); node_volume is CalcCellLocNodeVolumes with each element's own Nloc.  NULL: every
   * element has degree n_dg, with xgp/wgp/wbary_gp = N_Inter(n_dg).  Rejected by the HDG solve (the
   * reference builds p-adaption with HDG only on PETSc) and the differentiable loop. */
  const int32_t* n_dg_mapping;
  const double* n_inter;
  /* curved elements (NGeo > 1): ElemCurved(nElems) as 0/1 (IdentifyElemAndSideType, particle_mesh_tools.f90:
   * 848-1235: the element's XCL_NGeo differs from the trilinear interpolation of its corners).  The Newton x -> xi
   * runs on XCL_NGeo/dXCL_NGeo at NGeo for a curved element and on its eight corners (with dXCL_NGeo of the
   * corners) otherwise (GetPositionInRefElem, eval_xyz.f90:87-117); NULL: every element curved.  node_coords
   * holds the corners; elem_bary, xez_basis, slen_basis, elem_radius, elem_xgp, elem_sj and the FIBGM are
   * those of the curved map; BC sides need side_bezier and side_type below.  The differentiable loop needs
   * NGeo = 1. */
  const int32_t* elem_curved;
  /* BC sides of curved elements (NGeo > 1 with BC-element lists): BezierControlPoints3D(1:3,0:NGeo,0:NGeo) of
   * every local side (1:6) of every element in the element's own orientation (its master orientation;
   * RotateMasterToSlave, particle_surfaces.f90:1171-1202, of the master's points for a slave side), and SideType
   * of those sides (PLANAR_RECT 0, PLANAR_NONRECT 1, BILINEAR 2, PLANAR_CURVED 3, CURVED 4; IdentifyElemAndSideType,
   * particle_mesh_tools.f90:848-1235).  PLANAR_CURVED sides are traced by ComputePlanarCurvedIntersection, CURVED
   * ones by ComputeCurvedIntersection (Bezier clipping); NULL at NGeo = 1 (the corners give the side geometry).
   * Layout: side_bezier[((e * 6 + s) * (NGeo+1) + q) * (NGeo+1) + p][3] (p the first Bezier index), side_type[e * 6 + s].
   * Only the sides of the BC-element lists are read; pic_create rejects a degenerated one
   * (GetSideSlabNormalsAndIntervals) and RefTracking with BC sides on a curved mesh without these arrays. */
  const double* side_bezier;
  const int32_t* side_type;
} pic_mesh_t;

typedef struct pic_status_t {
  uint32_t error_word;          /* OR of PIC_STATUS_* seen since the last reset         */
  int32_t  n_lost;              /* NbrOfLostParticles                                   */
  int32_t  n_inside;            /* particles with PDM%ParticleInside                    */
  int32_t  n_newton_failed;     /* Newton calls that returned isSuccessful=.FALSE.      */
  int64_t  n_steps;             /* steps taken by pic_step/pic_push since create        */
} pic_status_t;

typedef struct pic_ctx pic_ctx_t;

/* Library / device ---------------------------------------------------------- */
const char* pic_version(void);
const char* pic_last_error(void);          /* message of the last failed call (thread-local) */

/* Context ------------------------------------------------------------------- */
int  pic_create(const pic_config_t* cfg, const pic_mesh_t* mesh, pic_ctx_t** ctx_out);
void pic_destroy(pic_ctx_t* ctx);

/* Field: U_N(e)%E(1:3,0:N,0:N,0:N) for e=1..nElems, contiguous (3*(N+1)^3*nElems doubles). */
int pic_set_field(pic_ctx_t* ctx, const double* e_dof, int32_t n_elems);

/* Particles: part_state is PartState(1:6,1:n); elem is PEM%GlobalElemID (1-based);
 * species is PartSpecies (1-based); inside / is_new are PDM%ParticleInside / PDM%IsNewPart. */
int pic_upload_particles(pic_ctx_t* ctx, const double* part_state, const int32_t* elem,
                         const int32_t* species, const uint8_t* inside, const uint8_t* is_new,
                         int32_t n);
/* Same arrays back in the caller's particle order.  part_pos_ref (PartPosRef(1:3,n)) may be NULL. */
int pic_download_particles(pic_ctx_t* ctx, double* part_state, int32_t* elem, uint8_t* inside,
                           uint8_t* is_new, double* part_pos_ref, int32_t n);

/* Loop pieces in reference order.  pic_push also saves LastPartPos/LastElem. */
int pic_interpolate(pic_ctx_t* ctx);
int pic_push(pic_ctx_t* ctx, double dt);
int pic_track(pic_ctx_t* ctx);
/* Deposition on the current particle state.  part_source is PS_N(e)%PartSource(1:4,0:N,0:N,0:N)
 * for all elements (4*(N+1)^3*nElems doubles); NULL keeps the result on the device. */
int pic_deposit(pic_ctx_t* ctx, double* part_source);
/* FieldAtParticle(1:6,1:n) of the last pic_interpolate (the fused pic_step keeps the field in registers), caller's particle order. */
int pic_get_field_at_particles(pic_ctx_t* ctx, double* field, int32_t n);

/* nsteps x {Deposition, InterpolateFieldToParticle, push, PerformTracking} with the field frozen.
 * part_source (may be NULL) receives the deposition of the last step. */
int pic_step(pic_ctx_t* ctx, double dt, int32_t nsteps, double* part_source);

int pic_get_status(pic_ctx_t* ctx, pic_status_t* status);

/* VerifyDepositedCharge (src/particles/pic/analyze/pic_analyze.f90:41-133; called by Deposition with
 * PIC-VerifyCharge = T, pic_depo.f90:1012-1015) on the last deposition of this context:
 * charge_numerical = the integral of PartSource(4) over the mesh (sum over elements and DOFs of
 * wGP(k) wGP(l) wGP(m) / sJ * PartSource(4)), charge_analytical = the sum of ChargeIC * MacroParticleFactor over
 * the particles inside (times dimFactorSF for a 1D/2D shape function with PIC-shapefunction-3D-deposition = F).
 * Needs pic_mesh_t.elem_sj at pic_create and a deposition (pic_deposit or pic_step) before the call;
 * PIC_ERR_STATE otherwise.  Synchronises the context's stream. */
int pic_verify_deposited_charge(pic_ctx_t* ctx, double* charge_numerical, double* charge_analytical);

/* Instrumentation (no reference counterpart): sustained FP64 fused multiply-add rate of this GPU in GFLOP/s,
 * from independent FMA chains on every SM (~0.1 s); the peak the FP64-bound kernels are compared against. */
int pic_fp64_fma_rate(pic_ctx_t* ctx, double* gflops);
/* The same for FP32 fused multiply-adds (fmaf chains): the peak of the mixed variant's FP32 work. */
int pic_fp32_fma_rate(pic_ctx_t* ctx, double* gflops);

/* Particle state in the reference's checkpoint layout (FillParticleData, src/io_hdf5/hdf5_output_particle.f90:1531):
 * the particles inside the domain grouped by element, in ascending caller index within an element
 * (UpdateNextFreePosition order); part_data(1:7, n_out) = PartState(1:6), Species; part_int(1:2, nElems) =
 * (FirstPartID, LastPartID) = offset_npart + the element's range, LastPartID - FirstPartID particles.
 * part_data may be NULL to query n_out first; capacity is the number of particles part_data holds. */
int pic_get_part_data(pic_ctx_t* ctx, double* part_data, int64_t* part_int, int64_t offset_npart, int32_t capacity,
                      int32_t* n_out);
/* Restart from that layout (particle_readin.f90): particle k of part_data lies in the element whose
 * part_int range holds offset_npart + k; uploaded with ParticleInside = T, IsNewPart = F. */
int pic_set_part_data(pic_ctx_t* ctx, const double* part_data, const int64_t* part_int, int64_t offset_npart,
                      int32_t n_part);

/* ---- HDG Poisson solve (linear, PP_nVar = 1; src/hdg/) ----------------------------------------------
 * Solves  -div(grad phi) = rho/eps0  (CalcSourceHDG: resu = -PartSource(4)/eps0) by PICLas's hybridised
 * DG method: element matrices Ehat, InvDhat, Smat (Elem_Mat), the trace system for lambda on the sides by
 * preconditioned CG (CG_solver, MatVec), the element-local potential U and E = PostProcessGradientHDG.
 * Everything runs on the device in FP64; E is written into the context's field (as pic_set_field would),
 * so InterpolateFieldToParticle sees it without a host round trip.  Conforming meshes with one N
 * (1..4), vacuum (chi = identity), Dirichlet (BCType 2/4-8: values set by pic_hdg_set_dirichlet, default
 * 0) and zero-gradient Neumann (BCType 10) sides; without Dirichlet sides the first DOF of
 * ElemToSide(E2S_SIDE_ID,1,1) is pinned to 0 (ZeroPotentialSide).  lambda is kept between solves and is
 * the start value of the next CG (as the reference's HDG_Surf_N(:)%lambda). */
typedef struct pic_hdg_t {
  int32_t n_sides;                /* nSides                                                           */
  const int32_t* elem_to_side;    /* ElemToSide(1:2,1:6,nElems): E2S_SIDE_ID (1-based), E2S_FLIP      */
  const int32_t* side_to_elem;    /* SideToElem(1:5,nSides): S2E_ELEM_ID, S2E_NB_ELEM_ID, S2E_LOC_SIDE_ID,
                                     S2E_NB_LOC_SIDE_ID, S2E_FLIP; -1 where a side has no such element  */
  const double* metrics_f;        /* N_VolMesh(e)%Metrics_fTilde(1:3,0:N,0:N,0:N) for all elements    */
  const double* metrics_g;        /* N_VolMesh(e)%Metrics_gTilde                                       */
  const double* metrics_h;        /* N_VolMesh(e)%Metrics_hTilde                                       */
  const double* sj;               /* N_VolMesh(e)%sJ(0:N,0:N,0:N) for all elements                     */
  int32_t n_dirichlet;            /* nDirichletBCSides                                                 */
  const int32_t* dirichlet_sides; /* DirichletBC(1:nDirichletBCSides), 1-based SideIDs                 */
  int32_t precond_type;           /* PrecondType: 0 none, 1 side-block Cholesky, 2 diagonal            */
  int32_t max_iter_cg;            /* MaxIterCG                                                         */
  double  eps_cg;                 /* epsCG                                                             */
  int32_t use_relative_abort;     /* useRelativeAbortCrit                                              */
  int32_t solve_in_step;          /* 1: pic_step solves after every Deposition (HDG(), :99)            */
  int32_t cg_kernel;              /* CG launch form (no reference counterpart): 0 auto (= 1), 1 three
                                     kernels per iteration replayed as a CUDA graph, 2 the whole CG in
                                     one cooperative kernel with grid barriers (slower on GB300)        */
} pic_hdg_t;
typedef struct pic_hdg_status_t {
  int32_t iterations;             /* CG iterations of the last solve                                   */
  int32_t converged;              /* 1: |r|^2 below the abort criterion                                */
  double  norm_r;                 /* sqrt(r.r) at the end of the last solve                            */
  int64_t n_solves;               /* solves since pic_hdg_init                                         */
} pic_hdg_status_t;
int pic_hdg_init(pic_ctx_t* ctx, const pic_hdg_t* hdg);
/* lambda on the Dirichlet sides, (nGP_face, nDirichletBCSides) in DirichletBC order */
int pic_hdg_set_dirichlet(pic_ctx_t* ctx, const double* lambda_bc);
/* One HDGLinear solve.  source = NULL: the charge density of the last deposition on the device
 * (resu = -PartSource(4)/eps0); otherwise resu itself, (0:N,0:N,0:N, nElems) on the host.  phi and e_field
 * (U_N(e)%U(1,...), U_N(e)%E(1:3,...)) are copied to the host when non-NULL; status may be NULL. */
int pic_hdg_solve(pic_ctx_t* ctx, const double* source, double* phi, double* e_field, pic_hdg_status_t* status);
int pic_hdg_get_lambda(pic_ctx_t* ctx, double* lambda /* (nGP_face, nSides) */);
/* lambda from a restart state (DG_SolutionLambda, src/restart/restart_field.f90:652-672): the start value
 * of the next CG */
int pic_hdg_set_lambda(pic_ctx_t* ctx, const double* lambda /* (nGP_face, nSides) */);
/* Elem_Mat of one element (1-based): Ehat(nGP_face,nGP_vol,6), InvDhat(nGP_vol,nGP_vol), Smat(nGP_face,
 * nGP_face,6,6); any pointer may be NULL */
int pic_hdg_get_elem_mat(pic_ctx_t* ctx, int32_t elem, double* ehat, double* inv_dhat, double* smat);

/* Differentiable loop (no reference counterpart; the reference has no adjoint).  Starting from the
 * uploaded particles (taken as x_0 and v_{-1/2}; IsNewPart is not applied), runs nsteps of
 * {interpolation, Boris push, TriaTracking} with the field frozen and B = b_scale * B_ext, deposits
 * the charge with cell_volweight_mean and returns
 *     loss = sum over all DOFs of (rho/rho_scale - rho_target)^2 ,
 * rho_target given as (nDOF, nElems).  If dL_dv0 (3,n) or dL_dB is non-NULL, a hand-written
 * reverse pass returns dL/dv_{-1/2} per particle (caller order) and dL/d|B|.  Element ids of the
 * forward pass are replayed in the reverse pass; (x, v, elem) are checkpointed every
 * checkpoint_every steps and each segment is recomputed.  precision PIC_PREC_FP64 gives the FP64
 * gradient, PIC_PREC_MIXED the FP32 adjoint (positions stay FP64).  The context's own particle
 * state is not modified.  Requires cell_volweight_mean + TriaTracking and N <= 3. */
typedef struct pic_adjoint_cfg_t {
  int32_t nsteps;
  int32_t checkpoint_every;
  int32_t precision;
  double  dt;
  double  rho_scale;
  double  b_scale;
} pic_adjoint_cfg_t;
int pic_adjoint_run(pic_ctx_t* ctx, const pic_adjoint_cfg_t* cfg, const double* rho_target, double* loss,
                    double* dL_dv0, double* dL_dB);
int pic_reset_status(pic_ctx_t* ctx);
/* Block the host until all work queued on the context's stream has finished. */
int pic_synchronize(pic_ctx_t* ctx);
/* Per-phase CUDA-event timing on the context's stream (no reference counterpart: the GPU analogue
 * of the reference's LBStartTime/LBSplitTime timers, loadbalance_timers.f90:70-172).
 * pic_profile(ctx,1) clears and starts collection, pic_profile(ctx,0) stops it.  pic_profile_read
 * returns accumulated milliseconds and kernel launches per phase:
 *   0 dominant deposition kernel (shape-function gather, or the fused CVWM+push+tracking kernel)
 *   1 sort-by-element + pack   2 interpolation+push+tracking   3 node -> DOF
 *   4 particle reorder         5 stand-alone CVWM deposition   6 HDG solve */
#define PIC_N_PHASES 7
int pic_profile(pic_ctx_t* ctx, int32_t enable);
int pic_profile_read(pic_ctx_t* ctx, double* ms, int64_t* launches, int32_t nphase);
/* cell_volweight_mean deposition that makes no device allocation (no reference counterpart).
 * For callers that cannot call cudaMalloc while their time loop runs (e.g. a host whose device
 * memory belongs to another runtime or to a fixed pool): the particles and the result stay in the
 * caller's device arrays -- d_part_state is PartState(1:6,n), d_elem / d_species are 1-based
 * PEM%GlobalElemID / PartSpecies, d_inside is PDM%ParticleInside as 0/1 bytes (NULL: every particle
 * inside; particles with 0 are skipped, as the reference skips them, pic_depo_method.f90:472),
 * d_part_source receives PartSource(1:4,0:N,0:N,0:N,nElems) -- and the node-sum scratch is a fixed
 * file-scope device array for at most 131072 periodic-unique mesh nodes (4 MiB per GPU, held until
 * the process exits; larger meshes return PIC_ERR_CAPACITY).  Element or species ids out of range
 * skip the particle and set PIC_STATUS_BAD_ELEMENT.
 * The work is queued on `stream` (a cudaStream_t, NULL = default stream) and not waited for; the
 * context's own stream is made to wait for it, so a later pic_get_status reports its status bits
 * (except while `stream` is being captured: then synchronise `stream` before pic_get_status).
 * Calls share the array: calls that overlap on the GPU race, so order them on one stream.  The
 * first call on a device looks up the array's address; make it before any stream capture. */
int pic_deposit_cvwm_noalloc(pic_ctx_t* ctx, const double* d_part_state, const int32_t* d_elem,
                             const int32_t* d_species, const uint8_t* d_inside, int32_t n, double* d_part_source,
                             void* stream);
/* Kernels launched through this context so far (no reference counterpart: instrumentation). */
int64_t pic_launch_count(pic_ctx_t* ctx);
/* The cudaStream_t the context enqueues on, as void* (no reference counterpart: lets a caller
 * time or order its own work against the loop). */
void* pic_stream(pic_ctx_t* ctx);

#ifdef __cplusplus
}
#endif
#endif /* PICLAS_GPU_H */
