// pic_kernels.cuh -- kernel declarations shared by the C-ABI layer and the kernel units.
#pragma once
#include "pic_device.cuh"

namespace pic {

// FP32 copies of the mapping data (mixed variant, linear uncurved elements)
struct MeshF {
  const float* xclr;   // [ne][8][3] corners minus barycentre
  const float* dxcl;   // [ne][8][9]
  const float* xez;    // [ne][6][3]
  const float* slen;   // [ne][6]
};

// everything a launch needs besides the particle arrays
struct LaunchArgs {
  DevMesh M;
  MeshF MF;
  int N, nd, n_canon;
  bool mixed;
  int sf_alpha;          // PIC-shapefunction-alpha (the gather has a compile-time branch for 2)
  const double* E;       // [ne][nd][3]
  const float* E32;      // [ne][nd][3] (mixed)
  double* NS;            // [n_canon][4] CVWM node sums
  DevStatus* st;
  cudaStream_t s;
};

// counting sort by element
struct SortBuffers {
  int* count;        // [ne+1]
  int* offset;       // [ne+2]
  int* cursor;       // [ne+1]
  int ne;
};

// shape-function deposition (gather over element neighbour lists)
struct SfLists {
  const int* nb_off;      // [ne+1]
  const int* nb_src;      // [n_pairs] source element (0-based)
  const int8_t* nb_shift; // [n_pairs][3] periodic image in units of the periodic vectors
  int n_pairs;
  const double* dof_center;   // [ne][3] centre of the element's DOF bounding box
  const float* dof_radius;    // [ne] largest distance of a DOF from dof_center
  const int* order;           // [ne] target elements in Morton order of their DOF centres (L2 reuse); on a
                              // p-adapted mesh grouped by degree, Morton order within each group
  int grp_off[kMaxN + 2];     // p-adapted mesh: the degree-k targets are order[grp_off[k] .. grp_off[k+1])
  // shape_function_cc: the same pairs seen from the source element, and the quadrature weight per DOF
  const int* t_off;           // [ne+1] per source element
  const int* t_tgt;           // [n_pairs] target element (0-based)
  const int8_t* t_shift;      // [n_pairs][3] periodic image of the source particles
  const double* dof_w;        // per DOF (packed like PartSource): wGP(k) wGP(l) wGP(m) / sJ of the element's degree
  const double* elem_r;       // [ne] shape_function_adaptive: radius of the source element (else NULL)
  // particle box of each element relative to its DOF centre, padded (lo.xyz, 0, hi.xyz, 0); set where the
  // pack bins particles into 2x2x2 sub-cells (mixed N = 3 with one radius), else NULL
  const float* elem_box;      // [ne][8]
};
struct SfPack {
  double* pos;     // [cap][3] FP64 position (FP64 variant)
  double* fac;     // [cap][4] w_sf*q*MPF*(v,1) (FP64 variant)
  float* posf;     // [cap][4] position relative to the source element's DOF centre (FP32), 4th = pad
  float* facf;     // [cap][4] (mixed variant)
  // sub-cell binning (SfLists::elem_box set): records ordered by (element, sub-cell), sub-cell = the octant of
  // the position relative to the element's DOF centre (bit 0: x > 0, bit 1: y > 0, bit 2: z > 0)
  int* sub_count;  // [8 ne + 1] (last: particles not inside)
  int* sub_off;    // [8 ne + 1] first record of each (element, sub-cell); sub_off[8 ne] = records inside
  int* sub_cursor; // [8 ne + 1]
};

// Launch wrappers; each returns the number of kernels it launched.
int launch_interpolate(const LaunchArgs& A, const DevParticles& P, bool refmap, bool cvwm);
int launch_push(const LaunchArgs& A, const DevParticles& P, double dt);
int launch_track(const LaunchArgs& A, const DevParticles& P, bool refmap);
int launch_deposit_cvwm(const LaunchArgs& A, const DevParticles& P, double* part_source);
// fused: Deposition (CVWM) + InterpolateFieldToParticle + push + TriaTracking
int launch_step_cvwm_tria(const LaunchArgs& A, const DevParticles& P, double* part_source, double dt);
int launch_cvwm_fused(const LaunchArgs& A, const DevParticles& P, double dt);
int launch_node_to_dof(const LaunchArgs& A, double* part_source);
int launch_sort_offsets(const LaunchArgs& A, const DevParticles& P, const SortBuffers& B);
int launch_sf_pack(const LaunchArgs& A, const DevParticles& P, const SortBuffers& B, const SfLists& L, const SfPack& K);
int sf_gather_variant();   // compile-time shape-function gather variant (PIC_SF_GATHER)
double fp64_fma_rate(cudaStream_t st, double* sink, int sms);   // GFLOP/s of independent FP64 FMA chains
double fp32_fma_rate(cudaStream_t st, float* sink, int sms);    // GFLOP/s of independent FP32 FMA chains
// shape_function_cc: scales each packed particle's Fac by q*MPF / (its quadrature charge over all DOFs
// within R), so that every particle deposits exactly its charge
int launch_sf_cc_norm(const LaunchArgs& A, const SortBuffers& B, const SfLists& L, const SfPack& K);
int launch_sf_gather(const LaunchArgs& A, const SortBuffers& B, const SfLists& L, const SfPack& K, double* part_source);
int launch_deposit_sf(const LaunchArgs& A, const DevParticles& P, const SortBuffers& B, const SfLists& L,
                      const SfPack& K, double* part_source);
// fused remainder for RefTracking: interpolation at PartPosRef + push + RefTracking
int launch_step_ref(const LaunchArgs& A, const DevParticles& P, double dt);
int launch_reorder(const LaunchArgs& A, DevParticles& P, DevParticles& Q, int* perm, int* perm_tmp,
                   const SortBuffers& B);
int launch_map_particles(const LaunchArgs& A, const DevParticles& P);
int launch_count_inside(const LaunchArgs& A, const DevParticles& P, int* out);
// VerifyDepositedCharge: sum over elements (in index order) of sum_DOF w * PartSource(4); inside particles per species
int launch_charge_integral(const LaunchArgs& A, const double* PS, const double* w, double* elem_sum, double* out);
int launch_count_species(const LaunchArgs& A, const DevParticles& P, int* counts);

}  // namespace pic
