// pic_ctx.h -- the context behind pic_ctx_t (private to the library's .cu files).
#pragma once
#include "../../include/piclas_gpu.h"
#include "pic_kernels.cuh"

#include <string>
#include <vector>

struct HdgState;            // HDG Poisson solve (pic_hdg.cu)
struct pic_ctx;
int hdg_destroy(pic_ctx* c);
int hdg_solve_device(pic_ctx* c, const double* part_source_dev, const double* resu_host);
bool hdg_solve_in_step(const pic_ctx* c);

namespace pic_internal {
int dalloc_bytes(void** p, size_t bytes);   // cudaMalloc with the library's error reporting
int set_error(int code, const std::string& msg);
}

struct pic_ctx {
  pic_config_t cfg{};
  int N = 0, nd = 0, ne = 0, n_canon = 0;
  bool mixed = false, refmap = false, sf = false;
  bool has_walls = false;       // some side is an open or reflective particle boundary
  bool cc = false;              // shape_function_cc or _adaptive: per-particle charge normalisation
  bool adaptive = false;        // shape_function_adaptive: radius per source element (SfLists::elem_r)
  double sf_rmax = 0.0;         // largest shape-function radius
  // per-element polynomial degree (pic_mesh_t.n_dg_mapping): each element's degree and DOF offset (without a
  // mapping N and e (N+1)^3), and the DOFs of all elements; var_n when the mesh is p-adapted (N is then NMax)
  bool var_n = false;
  std::vector<int> elem_n_h, dof_off_h;    // [ne], [ne+1]
  size_t ndofs = 0;
  int nd_of(int e) const { const int k = elem_n_h[e] + 1; return k * k * k; }
  cudaStream_t stream = nullptr;
  cudaEvent_t noalloc_done = nullptr;   // orders the context's stream after pic_deposit_cvwm_noalloc
  std::vector<void*> allocs;
  // mesh
  pic::DevMesh M{};
  pic::MeshF MF{};
  // field
  double* E = nullptr;
  float* E32 = nullptr;
  bool field_set = false;
  // deposition
  double* NS = nullptr;
  double* PS = nullptr;
  bool ps_valid = false;        // PS holds a deposition
  // VerifyDepositedCharge: wGP^3/sJ per DOF, per-element partial integrals, result, inside particles per species
  double* charge_w = nullptr;
  double* charge_elem = nullptr;
  double* charge_out = nullptr;
  int* species_count = nullptr;
  double charge_dim_factor = 1.0;
  // HDG field solve (pic_hdg_init)
  HdgState* hdg = nullptr;
  std::vector<double> xgp_h, wgp_h;   // N_Inter(N)%xGP, wGP
  pic::SortBuffers sortb{};
  pic::SfLists sfl{};
  pic::SfPack sfk{};
  // particles
  pic::DevParticles P{}, Q{};
  int* perm = nullptr;
  int* perm_tmp = nullptr;
  bool have_particles = false;
  // status
  pic::DevStatus* st = nullptr;
  int* d_count = nullptr;
  int64_t n_steps = 0;
  int64_t launches = 0;
  // per-phase CUDA-event timing (pic_profile)
  bool prof = false;
  struct Rec { int phase; cudaEvent_t a, b; int launches; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  double prof_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t prof_launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};

  template <class T>
  int alloc(T** p, size_t n) {
    if (n == 0) n = 1;
    int rc = pic_internal::dalloc_bytes((void**)p, n * sizeof(T));
    if (rc == PIC_OK) allocs.push_back((void*)*p);
    return rc;
  }
  cudaEvent_t take_event() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  // run fn() (which enqueues kernels and returns how many), bracketed by events when profiling
  template <class F>
  void phase(int ph, F&& fn) {
    if (!prof) { launches += fn(); return; }
    cudaEvent_t a = take_event(), b = take_event();
    cudaEventRecord(a, stream);
    const int n = fn();
    cudaEventRecord(b, stream);
    launches += n;
    recs.push_back(Rec{ph, a, b, n});
  }
  void collect() {
    for (auto& r : recs) {
      float ms = 0.f;
      cudaEventSynchronize(r.b);
      cudaEventElapsedTime(&ms, r.a, r.b);
      prof_ms[r.phase] += ms;
      prof_launches[r.phase] += r.launches;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    recs.clear();
  }
  pic::LaunchArgs args() const {
    pic::LaunchArgs a;
    a.M = M; a.MF = MF; a.N = N; a.nd = nd; a.n_canon = n_canon; a.mixed = mixed; a.sf_alpha = cfg.sf_alpha;
    a.E = E; a.E32 = E32; a.NS = NS; a.st = st; a.s = stream;
    return a;
  }
};
