// pic_capi.cu -- extern "C" boundary of the GB300 particle loop (see include/piclas_gpu.h).
//
// The context owns every device array.  Mesh arrays arrive in the reference's layout and are
// converted once at pic_create:
//   * periodic node copies (Periodic_Nodes twins) are merged into one periodic-unique node, so
//     CVWM deposits once per corner instead of once per copy;
//   * per-element side data is packed into one 32-bit word per side;
//   * FP32 copies of the mapping data are made for the mixed variant;
//   * shape-function neighbour lists (source element, periodic image) are built per target
//     element from the FIBGM, so deposition is a gather without atomics.
#include "../../include/piclas_gpu.h"
#include "pic_kernels.cuh"
#include "pic_ctx.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace pic;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                            \
  do {                                                                                            \
    cudaError_t _e = (expr);                                                                      \
    if (_e != cudaSuccess) {                                                                      \
      return fail(_e == cudaErrorMemoryAllocation ? PIC_ERR_OUT_OF_MEMORY : PIC_ERR_CUDA,         \
                  std::string(#expr) + ": " + cudaGetErrorString(_e));                            \
    }                                                                                             \
  } while (0)

template <class T>
int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) return fail(PIC_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return PIC_OK;
}

}  // namespace

namespace pic_internal {
int dalloc_bytes(void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return fail(PIC_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return PIC_OK;
}
int set_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace pic_internal



// ---------------------------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------------------------
namespace {

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

template <class T>
int upload(pic_ctx* c, T** dst, const std::vector<T>& src) {
  int rc = c->alloc(dst, src.size());
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return PIC_OK;
}

// 3D shape function weight, pic_depo_shapefunction_tools.f90:1243-1246 with beta() of
// pic_depo_tools.f90:491-511
double sf_weight(double r, int alpha) {
  const double PI = std::acos(-1.0);
  const double beta = std::tgamma(1.5) * std::tgamma((double)alpha + 1.0) / std::tgamma(1.5 + ((double)alpha + 1.0));
  return 1.0 / (2.0 * beta * (double)alpha + 2.0 * beta) * ((double)alpha + 1.0) / (PI * (r * r * r));
}

// 1D / 2D shape-function weight (InitShapeFunctionDimensionalty, pic_depo_shapefunction_tools.f90:1162-1232):
// the kernel normalised along its line / over its area, divided by the extent of the remaining
// directions when the charge is spread over the volume (PIC-shapefunction-3D-deposition)
double sf_weight_dim(const pic_config_t* cfg, const pic_mesh_t* m, double r, int alpha) {
  const int dim = cfg->sf_dim ? cfg->sf_dim : 3, dir = cfg->sf_dir - 1;
  if (dim == 3) return sf_weight(r, alpha);
  const double PI = std::acos(-1.0);
  double ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = m->xmax_glob[d] - m->xmin_glob[d];
  if (dim == 1) {
    const double dimFactor = (dir == 0) ? ext[1] * ext[2] : (dir == 1) ? ext[0] * ext[2] : ext[0] * ext[1];
    const double a = std::tgamma((double)alpha + 1.5);
    const double b = std::sqrt(PI) * r * std::tgamma((double)(alpha + 1));
    return cfg->sf_depo3d ? a / (b * dimFactor) : a / b;
  }
  return cfg->sf_depo3d ? ((double)alpha + 1.0) / (PI * (r * r) * ext[dir]) : ((double)alpha + 1.0) / (PI * (r * r));
}

// dimFactorSF (InitShapeFunctionDimensionalty): 1D the cross-section across the kernel direction, 2D the
// extent along the constant direction, 1 for the 3D kernel
static double sf_dim_factor(const pic_config_t* cfg, const pic_mesh_t* m) {
  const int dim = cfg->sf_dim ? cfg->sf_dim : 3, dir = cfg->sf_dir - 1;
  double ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = m->xmax_glob[d] - m->xmin_glob[d];
  if (dim == 1) return (dir == 0) ? ext[1] * ext[2] : (dir == 1) ? ext[0] * ext[2] : ext[0] * ext[1];
  if (dim == 2) return ext[dir];
  return 1.0;
}

// directions in which a 1D/2D shape function has its kernel (the others are zeroed in the DOF and particle
// coordinates the gather reads, so the kernel sees SFRadius2, pic_depo_shapefunction_tools.f90:1029-1058)
void sf_kernel_dirs(const pic_config_t* cfg, bool keep[3]) {
  const int dim = cfg->sf_dim ? cfg->sf_dim : 3, dir = cfg->sf_dir - 1;
  for (int d = 0; d < 3; ++d) keep[d] = dim == 3 || (dim == 1 ? d == dir : d != dir);
}

int validate(const pic_config_t* cfg, const pic_mesh_t* m) {
  if (!cfg || !m) return fail(PIC_ERR_INVALID_ARGUMENT, "null config or mesh");
  if (cfg->sf_dim < 0 || cfg->sf_dim > 3) return fail(PIC_ERR_INVALID_ARGUMENT, "sf_dim must be 1, 2 or 3 (0 = 3)");
  if (cfg->sf_dim == 1 || cfg->sf_dim == 2) {
    if (cfg->deposition == PIC_DEPO_CVWM)
      return fail(PIC_ERR_INVALID_ARGUMENT, "sf_dim applies to the shape-function depositions");
    if (cfg->sf_dir < 1 || cfg->sf_dir > 3) return fail(PIC_ERR_INVALID_ARGUMENT, "sf_dir must be 1..3");
    if (m->n_periodic_vectors != 0 && m->n_periodic_vectors != 3)
      return fail(PIC_ERR_INVALID_ARGUMENT, "1D/2D shape functions need a mesh with no or three periodic vectors");
  }
  if (cfg->n_dg < 1 || cfg->n_dg > 4) return fail(PIC_ERR_INVALID_ARGUMENT, "n_dg must be 1..4");
  // 'Wrong guessing method for mapping from physical space in reference space.' (particle_mesh.f90:374-376)
  if (cfg->ref_mapping_guess < 0 || cfg->ref_mapping_guess > 4)
    return fail(PIC_ERR_INVALID_ARGUMENT, "ref_mapping_guess must be 1..4 (0: 1)");
  if (cfg->tracking != PIC_TRACK_TRIA && cfg->tracking != PIC_TRACK_REFMAPPING)
    return fail(PIC_ERR_INVALID_ARGUMENT, "unknown tracking method");
  if (cfg->deposition < PIC_DEPO_CVWM || cfg->deposition > PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE)
    return fail(PIC_ERR_INVALID_ARGUMENT, "unknown deposition method");
  // the 3D kernel visits 27 images (three periodic vectors) or none (InitPeriodicSFCaseMatrix, pic_depo.f90:828-910)
  if (cfg->deposition != PIC_DEPO_CVWM && (cfg->sf_dim == 0 || cfg->sf_dim == 3) && m->n_periodic_vectors != 0 &&
      m->n_periodic_vectors != 3)
    return fail(PIC_ERR_INVALID_ARGUMENT, "3D shape functions need a mesh with no or three periodic vectors");
  if (cfg->precision != PIC_PREC_FP64 && cfg->precision != PIC_PREC_MIXED)
    return fail(PIC_ERR_INVALID_ARGUMENT, "unknown precision");
  if (cfg->n_species < 1 || cfg->n_species > PIC_MAX_SPECIES) return fail(PIC_ERR_INVALID_ARGUMENT, "n_species");
  if (cfg->max_particles < 0) return fail(PIC_ERR_INVALID_ARGUMENT, "max_particles");
  for (int s = 0; s < cfg->n_species; ++s) {
    if (!(cfg->mass[s] > 0.0)) return fail(PIC_ERR_INVALID_ARGUMENT, "species mass must be > 0");
    // Species(s)%TimeStepFactor: the reference stops on factors above 1 ('Species-specific time step only
    // allows factors below 1!', particle_emission_init.f90:218-219)
    if (!(cfg->time_step_factor[s] >= 0.0) || !(cfg->time_step_factor[s] <= 1.0))
      return fail(PIC_ERR_INVALID_ARGUMENT, "time_step_factor must lie in [0, 1] (0: not set = 1); the reference "
                                            "only allows species-specific factors below 1");
  }
  if (m->n_elems < 1) return fail(PIC_ERR_INVALID_ARGUMENT, "n_elems must be positive");
  if (m->n_geo < 1 || m->n_geo > 4) return fail(PIC_ERR_INVALID_ARGUMENT, "NGeo must be 1..4");
  if (m->n_geo > 1 && cfg->tracking == PIC_TRACK_REFMAPPING && (m->side_bc || cfg->periodic_tracing) &&
      (!m->side_bezier || !m->side_type))
    return fail(PIC_ERR_INVALID_ARGUMENT, "RefTracking with BC sides on curved elements (NGeo > 1) needs side_bezier "
                                          "and side_type");
  if (m->n_periodic_vectors < 0 || m->n_periodic_vectors > 3) return fail(PIC_ERR_INVALID_ARGUMENT, "n_periodic_vectors");
  const void* req[] = {m->xi_cl_ngeo, m->wbary_cl_ngeo, m->xgp, m->wgp, m->wbary_gp, m->xcl_ngeo, m->dxcl_ngeo,
                       m->elem_bary, m->xez_basis, m->slen_basis, m->elem_radius, m->elem_xgp, m->node_coords,
                       m->elem_side_node, m->side_nb_elem, m->side_pvid, m->concave_side, m->node_info};
  for (const void* p : req)
    if (!p) return fail(PIC_ERR_INVALID_ARGUMENT, "missing mesh array");
  if (cfg->deposition == PIC_DEPO_CVWM && !m->node_volume) return fail(PIC_ERR_INVALID_ARGUMENT, "node_volume");
  const bool sf = cfg->deposition == PIC_DEPO_SHAPE_FUNCTION || cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_CC ||
                  cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE;
  if ((cfg->tracking == PIC_TRACK_REFMAPPING || sf) &&
      (!m->fibgm_n_elems || !m->fibgm_offset || !m->fibgm_element || !m->eps_one_cell))
    return fail(PIC_ERR_INVALID_ARGUMENT, "FIBGM arrays required for RefTracking / shape function");
  if (sf && cfg->sf_alpha < 2) return fail(PIC_ERR_INVALID_ARGUMENT, "shape function alpha must be >= 2");
  if (cfg->tracking == PIC_TRACK_REFMAPPING) {
    // RefTracking sorts the candidates of one FIBGM cell in registers (at most 64, pic_device.cuh)
    const size_t ncell = (size_t)std::max(m->fibgm_imax[0], 1) * std::max(m->fibgm_imax[1], 1) * std::max(m->fibgm_imax[2], 1);
    for (size_t q = 0; q < ncell; ++q)
      if (m->fibgm_n_elems[q] > 64)
        return fail(PIC_ERR_INVALID_ARGUMENT, "a FIBGM cell holds more than 64 elements: refine the background mesh");
  }
  if (cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE) {
    if (!m->sf_elem_radius) return fail(PIC_ERR_INVALID_ARGUMENT, "shape_function_adaptive needs sf_elem_radius");
    for (int e = 0; e < m->n_elems; ++e)
      if (!(m->sf_elem_radius[e] > 0.0) || !std::isfinite(m->sf_elem_radius[e]))
        return fail(PIC_ERR_INVALID_ARGUMENT, "sf_elem_radius must be positive and finite");
  } else if (sf && !(cfg->sf_radius > 0.0)) {
    return fail(PIC_ERR_INVALID_ARGUMENT, "shape function radius");
  }
  if (m->n_dg_mapping) {
    // N_DG_Mapping(1:3,:): degrees 1..NMax and the DOF offsets of Set_N_DG_Mapping (mesh_pAdaption.f90:391-414)
    if (!m->n_inter) return fail(PIC_ERR_INVALID_ARGUMENT, "n_dg_mapping needs n_inter (N_Inter(1..n_dg))");
    int64_t off = 0;
    for (int e = 0; e < m->n_elems; ++e) {
      const int nl = m->n_dg_mapping[(size_t)e * 3 + 1];
      if (nl < 1 || nl > cfg->n_dg)
        return fail(PIC_ERR_INVALID_ARGUMENT, "n_dg_mapping: element degrees must lie in 1..n_dg");
      if (m->n_dg_mapping[(size_t)e * 3] != off)
        return fail(PIC_ERR_INVALID_ARGUMENT, "n_dg_mapping: DOF offsets must be the running sum of (Nloc+1)^3");
      off += (int64_t)(nl + 1) * (nl + 1) * (nl + 1);
      if (off > INT32_MAX) return fail(PIC_ERR_INVALID_ARGUMENT, "n_dg_mapping: more than 2^31 DOFs");
    }
  }
  return PIC_OK;
}

// Bounding box of element e: its corners (NGeo = 1), or the Bezier control points of its NGeo map (Bernstein
// coefficients of the Lagrange interpolant on the CL points, which hold the element by the convex hull property)
void elem_bbox(const pic_mesh_t* m, int e, double lo[3], double hi[3]) {
  const int ng = m->n_geo, n1 = ng + 1;
  for (int d = 0; d < 3; ++d) { lo[d] = 1e300; hi[d] = -1e300; }
  if (ng == 1) {
    for (int t = 0; t < 8; ++t)
      for (int d = 0; d < 3; ++d) {
        const double v = m->xcl_ngeo[((size_t)e * 8 + t) * 3 + d];
        lo[d] = std::min(lo[d], v); hi[d] = std::max(hi[d], v);
      }
    return;
  }
  // V(i,j) = B_j(t_i), t = (xi_i + 1)/2 on the CL points; Vi = V^-1 (Gauss-Jordan, n1 <= 5)
  double V[5][10];
  for (int i = 0; i < n1; ++i) {
    const double t = 0.5 * (m->xi_cl_ngeo[i] + 1.0);
    for (int j = 0; j < n1; ++j) {
      double b = 1.0;
      for (int q = 0; q < j; ++q) b = b * (double)(ng - q) / (double)(q + 1);
      V[i][j] = b * std::pow(t, j) * std::pow(1.0 - t, ng - j);
      V[i][n1 + j] = i == j ? 1.0 : 0.0;
    }
  }
  for (int c = 0; c < n1; ++c) {
    int p = c;
    for (int r = c + 1; r < n1; ++r) if (std::fabs(V[r][c]) > std::fabs(V[p][c])) p = r;
    for (int k = 0; k < 2 * n1; ++k) std::swap(V[c][k], V[p][k]);
    const double piv = V[c][c];
    for (int k = 0; k < 2 * n1; ++k) V[c][k] /= piv;
    for (int r = 0; r < n1; ++r)
      if (r != c) { const double f = V[r][c]; for (int k = 0; k < 2 * n1; ++k) V[r][k] -= f * V[c][k]; }
  }
  const double* X = m->xcl_ngeo + (size_t)e * n1 * n1 * n1 * 3;
  for (int d = 0; d < 3; ++d) {
    double A[125], B[125];
    for (int q = 0; q < n1 * n1 * n1; ++q) A[q] = X[(size_t)q * 3 + d];
    for (int ax = 0; ax < 3; ++ax) {              // apply Vi along i, then j, then k
      const int st = ax == 0 ? 1 : ax == 1 ? n1 : n1 * n1;
      for (int q = 0; q < n1 * n1 * n1; ++q) {
        const int a = (q / st) % n1, base = q - a * st;
        double v = 0.0;
        for (int l = 0; l < n1; ++l) v += V[a][n1 + l] * A[base + l * st];
        B[q] = v;
      }
      for (int q = 0; q < n1 * n1 * n1; ++q) A[q] = B[q];
    }
    for (int q = 0; q < n1 * n1 * n1; ++q) { lo[d] = std::min(lo[d], A[q]); hi[d] = std::max(hi[d], A[q]); }
  }
}

// N_Inter(Nloc)%wGP of element e (N_Inter(N) without a mapping)
const double* elem_wgp(const pic_ctx* c, const pic_mesh_t* m, int e) {
  if (!c->var_n) return m->wgp;
  const int kd = c->elem_n_h[e];
  return m->n_inter + 3 * ((kd - 1) * (kd + 2) / 2) + (kd + 1);
}

// Shape-function gather lists: for every target element, the (source element, periodic image)
// pairs whose bounding box lies within R of at least one DOF of the target.  Enumerated from
// the FIBGM cells covering the target's DOF box grown by R, with cell indices outside the grid
// wrapped onto their periodic image.
int build_sf_lists(pic_ctx* c, const pic_mesh_t* m, const std::vector<double>& dofc, const std::vector<double>& sfx,
                   const bool kdir[3]) {
  const int ne = m->n_elems;
  const double R = c->sf_rmax;
  auto R2src = [&](int s) { const double r = c->adaptive ? m->sf_elem_radius[s] : c->cfg.sf_radius; return r * r; };
  std::vector<double> bmin((size_t)ne * 3), bmax((size_t)ne * 3), dmin((size_t)ne * 3), dmax((size_t)ne * 3);
  for (int e = 0; e < ne; ++e)
    for (int d = 0; d < 3; ++d) {
      double lo, hi, dl = 1e300, dh = -1e300;
      {
        double blo[3], bhi[3];
        elem_bbox(m, e, blo, bhi);
        lo = blo[d]; hi = bhi[d];
      }
      for (int r = 0; r < c->nd_of(e); ++r) {
        double v = sfx[((size_t)c->dof_off_h[e] + r) * 3 + d];
        dl = std::min(dl, v); dh = std::max(dh, v);
      }
      bmin[e * 3 + d] = lo; bmax[e * 3 + d] = hi; dmin[e * 3 + d] = dl; dmax[e * 3 + d] = dh;
    }
  // periodic vector per axis (axis-aligned boxes only)
  double Lax[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    int k = -1;
    for (int q = 0; q < m->n_periodic_vectors; ++q) {
      const double* pv = m->periodic_vectors + 3 * q;
      if (pv[d] != 0.0) {
        for (int o = 0; o < 3; ++o)
          if (o != d && pv[o] != 0.0) return fail(PIC_ERR_INVALID_ARGUMENT, "shape function needs axis-aligned periodic vectors");
        k = q;
      }
    }
    Lax[d] = k >= 0 ? m->periodic_vectors[3 * k + d] : 0.0;
  }
  // ElemToElemMapping as a set: elements sharing a unique corner node (particle_mesh_build.f90:1244-1380)
  const bool near_only = c->adaptive && m->n_periodic_vectors == 0;
  std::vector<std::vector<int>> node_elems;
  if (near_only) {
    int nn = 0;
    for (size_t q = 0; q < (size_t)ne * 8; ++q) {
      if (m->node_info[q] < 1) return fail(PIC_ERR_INVALID_ARGUMENT, "node_info out of range");
      nn = std::max(nn, m->node_info[q]);
    }
    node_elems.resize((size_t)nn + 1);
    for (int e = 0; e < ne; ++e)
      for (int t = 0; t < 8; ++t) node_elems[m->node_info[(size_t)e * 8 + t]].push_back(e);
  }
  auto shares_node = [&](int a, int b) {
    for (int t = 0; t < 8; ++t)
      for (int x : node_elems[m->node_info[(size_t)a * 8 + t]])
        if (x == b) return true;
    return false;
  };
  std::vector<int> off(ne + 1, 0), src;
  std::vector<int8_t> shift;
  std::vector<int> seen(ne, -1);
  std::vector<int> seen_shift(ne, 0);
  const int* imax = m->fibgm_imax;
  for (int e = 0; e < ne; ++e) {
    int clo[3], chi[3];
    for (int d = 0; d < 3; ++d) {
      if (!kdir[d]) { clo[d] = 1; chi[d] = imax[d]; continue; }   // no kernel along d: every cell, no image
      clo[d] = (int)std::floor((dmin[e * 3 + d] - R - m->xmin_glob[d]) / m->fibgm_deltas[d]) + 1;
      chi[d] = (int)std::ceil((dmax[e * 3 + d] + R - m->xmin_glob[d]) / m->fibgm_deltas[d]);
    }
    std::vector<std::pair<int, int>> cand;  // (src, packed shift)
    for (int kk = clo[2]; kk <= chi[2]; ++kk)
      for (int jj = clo[1]; jj <= chi[1]; ++jj)
        for (int ii = clo[0]; ii <= chi[0]; ++ii) {
          int cidx[3] = {ii, jj, kk}, sh[3] = {0, 0, 0};
          bool ok = true;
          for (int d = 0; d < 3; ++d) {
            while (cidx[d] < 1) { if (Lax[d] == 0.0) { ok = false; break; } cidx[d] += imax[d]; sh[d] -= 1; }
            while (cidx[d] > imax[d]) { if (Lax[d] == 0.0) { ok = false; break; } cidx[d] -= imax[d]; sh[d] += 1; }
            if (sh[d] < -1 || sh[d] > 1) ok = false;   // the reference visits the 27 images only
          }
          if (!ok) continue;
          size_t ci = (size_t)(cidx[0] - 1) + (size_t)imax[0] * ((cidx[1] - 1) + (size_t)imax[1] * (cidx[2] - 1));
          int n = m->fibgm_n_elems[ci], o = m->fibgm_offset[ci];
          // a cell index below 1 wrapped to the top of the grid holds sources near xmax: their
          // particles are seen from the target at x + sh*L with sh = -1 (and +1 above the grid)
          for (int q = 0; q < n; ++q) {
            int s = m->fibgm_element[o + q] - 1;
            int pk = ((sh[0] + 1) * 9) + ((sh[1] + 1) * 3) + (sh[2] + 1);
            cand.emplace_back(s, pk);
          }
        }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    for (auto& pr : cand) {
      const int s = pr.first, pk = pr.second;
      // shape_function_adaptive without periodic vectors deposits on the particle's element and the
      // elements sharing a corner node with it only (depoChargeOnDOFsSFAdaptive over ElemToElemMapping)
      if (near_only && s != e && !shares_node(s, e)) continue;
      const int sx = pk / 9 - 1, sy = (pk / 3) % 3 - 1, sz = pk % 3 - 1;
      const double shv[3] = {sx * Lax[0], sy * Lax[1], sz * Lax[2]};
      // exact-conservative test: min over target DOFs of the distance to the shifted source box
      bool keep = false;
      for (int r = 0; r < c->nd_of(e) && !keep; ++r) {
        double d2 = 0.0;
        for (int d = 0; d < 3; ++d) {
          if (!kdir[d]) continue;
          const double p = sfx[((size_t)c->dof_off_h[e] + r) * 3 + d];
          const double lo = bmin[s * 3 + d] + shv[d], hi = bmax[s * 3 + d] + shv[d];
          const double q = p < lo ? lo - p : (p > hi ? p - hi : 0.0);
          d2 += q * q;
        }
        if (d2 <= R2src(s) * (1.0 + 1e-6)) keep = true;
      }
      if (!keep) continue;
      src.push_back(s);
      shift.push_back((int8_t)sx); shift.push_back((int8_t)sy); shift.push_back((int8_t)sz);
    }
    off[e + 1] = (int)src.size();
  }
  // DOF-box radius per element (staging cull) and a Morton order of the targets
  std::vector<float> drad(ne);
  std::vector<std::pair<uint64_t, int>> mort(ne);
  for (int e = 0; e < ne; ++e) {
    double r2 = 0.0;
    for (int r = 0; r < c->nd_of(e); ++r) {
      double q = 0.0;
      for (int d = 0; d < 3; ++d) {
        const double v = sfx[((size_t)c->dof_off_h[e] + r) * 3 + d] - dofc[(size_t)e * 3 + d];
        q += v * v;
      }
      r2 = std::max(r2, q);
    }
    drad[e] = (float)(std::sqrt(r2) * (1.0 + 1e-6));
    uint64_t code = 0;
    uint32_t ic[3];
    for (int d = 0; d < 3; ++d) {
      double u = (dofc[(size_t)e * 3 + d] - m->xmin_glob[d]) / std::max(m->xmax_glob[d] - m->xmin_glob[d], 1e-300);
      u = std::min(std::max(u, 0.0), 1.0);
      ic[d] = (uint32_t)(u * 1048575.0);
    }
    for (int b = 19; b >= 0; --b)
      for (int d = 2; d >= 0; --d) code = (code << 1) | ((ic[d] >> b) & 1u);
    // p-adapted mesh: grouped by degree (one gather launch per degree), Morton order within a group
    if (c->var_n) code |= (uint64_t)c->elem_n_h[e] << 60;
    mort[e] = {code, e};
  }
  std::sort(mort.begin(), mort.end());
  std::vector<int> order(ne);
  for (int e = 0; e < ne; ++e) order[e] = mort[e].second;
  for (int k = 0; k <= kMaxN + 1; ++k) c->sfl.grp_off[k] = 0;
  for (int e = 0; e < ne; ++e) c->sfl.grp_off[c->elem_n_h[e] + 1]++;
  for (int k = 1; k <= kMaxN + 1; ++k) c->sfl.grp_off[k] += c->sfl.grp_off[k - 1];
  int* d_off; int* d_src; int8_t* d_sh; double* d_c; float* d_r; int* d_o;
  int rc;
  if (c->mixed && c->N == 3 && !c->var_n && !c->adaptive && pic::sf_gather_variant() == 5) {
    // the particle box of every element relative to its DOF centre (kernel directions only): the corners'
    // bounding box, padded by 5 % of its extent on every side (RefTracking keeps particles within
    // epsOneCell ~ 1 + sqrt(3 RefMappingEps) of the element), for the sub-cell culling of the mixed gather
    std::vector<float> ebox((size_t)ne * 8, 0.0f);
    for (int e = 0; e < ne; ++e)
      for (int d = 0; d < 3; ++d) {
        if (!kdir[d]) continue;
        double blo[3], bhi[3];
        elem_bbox(m, e, blo, bhi);
        const double lo = blo[d] - dofc[(size_t)e * 3 + d], hi = bhi[d] - dofc[(size_t)e * 3 + d];
        const double pad = 0.05 * (hi - lo);
        ebox[(size_t)e * 8 + d] = (float)(lo - pad);
        ebox[(size_t)e * 8 + 4 + d] = (float)(hi + pad);
      }
    float* d_eb;
    if ((rc = upload(c, &d_eb, ebox))) return rc;
    c->sfl.elem_box = d_eb;
  }
  if (c->cc) {
    // the pairs transposed to (source -> target, image), and wGP(k) wGP(l) wGP(m) / sJ per DOF
    std::vector<int> toff(ne + 1, 0), ttgt(src.size());
    std::vector<int8_t> tsh(shift.size());
    for (size_t q = 0; q < src.size(); ++q) toff[src[q] + 1]++;
    for (int e = 0; e < ne; ++e) toff[e + 1] += toff[e];
    std::vector<int> cur(toff.begin(), toff.end() - 1);
    for (int e = 0; e < ne; ++e)
      for (int q = off[e]; q < off[e + 1]; ++q) {
        const int t = cur[src[q]]++;
        ttgt[t] = e;
        for (int d = 0; d < 3; ++d) tsh[3 * (size_t)t + d] = shift[3 * (size_t)q + d];
      }
    std::vector<double> dw(c->ndofs);
    for (int e = 0; e < ne; ++e) {
      const int n1 = c->elem_n_h[e] + 1;
      const double* wg = elem_wgp(c, m, e);
      const size_t b = (size_t)c->dof_off_h[e];
      for (int r = 0; r < c->nd_of(e); ++r) {
        const int k = r % n1, l = (r / n1) % n1, mm = r / (n1 * n1);
        dw[b + r] = wg[k] * wg[l] * wg[mm] / m->elem_sj[b + r];
      }
    }
    int* d_toff; int* d_ttgt; int8_t* d_tsh; double* d_dw;
    if ((rc = upload(c, &d_toff, toff)) || (rc = upload(c, &d_ttgt, ttgt)) || (rc = upload(c, &d_tsh, tsh)) ||
        (rc = upload(c, &d_dw, dw)))
      return rc;
    c->sfl.t_off = d_toff; c->sfl.t_tgt = d_ttgt; c->sfl.t_shift = d_tsh; c->sfl.dof_w = d_dw;
  }
  if (c->adaptive) {
    std::vector<double> er(m->sf_elem_radius, m->sf_elem_radius + ne);
    double* d_er;
    if ((rc = upload(c, &d_er, er))) return rc;
    c->sfl.elem_r = d_er;
  }
  if ((rc = upload(c, &d_off, off))) return rc;
  if ((rc = upload(c, &d_src, src))) return rc;
  if ((rc = upload(c, &d_sh, shift))) return rc;
  if ((rc = upload(c, &d_c, dofc))) return rc;
  if ((rc = upload(c, &d_r, drad))) return rc;
  if ((rc = upload(c, &d_o, order))) return rc;
  c->sfl.nb_off = d_off; c->sfl.nb_src = d_src; c->sfl.nb_shift = d_sh; c->sfl.n_pairs = (int)src.size();
  c->sfl.dof_center = d_c; c->sfl.dof_radius = d_r; c->sfl.order = d_o;
  return PIC_OK;
}

int alloc_particles(pic_ctx* c, DevParticles& P, int cap, bool with_aux) {
  int rc;
  P.cap = cap;
  P.n = 0;
  const size_t n = (size_t)std::max(cap, 1);
  if ((rc = c->alloc(&P.x, n)) || (rc = c->alloc(&P.y, n)) || (rc = c->alloc(&P.z, n))) return rc;
  if (c->mixed) {
    if ((rc = c->alloc(&P.vxf, n)) || (rc = c->alloc(&P.vyf, n)) || (rc = c->alloc(&P.vzf, n))) return rc;
  } else {
    if ((rc = c->alloc(&P.vx, n)) || (rc = c->alloc(&P.vy, n)) || (rc = c->alloc(&P.vz, n))) return rc;
  }
  if ((rc = c->alloc(&P.xi0, n)) || (rc = c->alloc(&P.xi1, n)) || (rc = c->alloc(&P.xi2, n))) return rc;
  if ((rc = c->alloc(&P.elem, n)) || (rc = c->alloc(&P.last_elem, n))) return rc;
  if ((rc = c->alloc(&P.species, n)) || (rc = c->alloc(&P.flags, n))) return rc;
  if (with_aux) {
    if ((rc = c->alloc(&P.lx, n)) || (rc = c->alloc(&P.ly, n)) || (rc = c->alloc(&P.lz, n))) return rc;
    if ((rc = c->alloc(&P.field, 6 * n))) return rc;
  }
  return PIC_OK;
}

int device_sync(pic_ctx* c) {
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cudaGetLastError());
  return PIC_OK;
}

}  // namespace

// =============================================================================================
extern "C" {

const char* pic_version(void) {
  static const std::string v = "piclas_gb300 0.1 (sm_103a; sf gather " + std::to_string(pic::sf_gather_variant()) + ")";
  return v.c_str();
}
const char* pic_last_error(void) { return g_last_error.c_str(); }

// Wall side geometry of a BC element for RefTracking, in the oracle's operation order: GetSideType for
// NGeo = 1 (particle_mesh_tools.f90:1001-1053) and BaseVectors0-3 (particle_mesh_build.f90:1916-1925);
// corners in the side's BezierControlPoints3D order (CGNS side order, particle_mesh_tools.f90:1748-1773),
// planar when they lie within 1e-6 of the side's extent of the
// averaged plane (then SideNormVec oriented away from the element, SideDistance, PLANAR_RECT or
// PLANAR_NONRECT), else BILINEAR with the non-oriented averaged normal.  Fills kBcGeo doubles.  On curved
// meshes the side's type is given (the mesh's SideType, GetSideType for NGeo > 1): BILINEAR and CURVED sides
// keep the non-oriented averaged normal, planar ones (PLANAR_RECT, _NONRECT, _CURVED) get SideNormVec and
// SideDistance from their corners as above (IdentifyElemAndSideType, particle_mesh_tools.f90:991-1012).
static void wall_side_geometry(const double* xcl, const double* bary, int e, int s, double* g, int given) {
  auto corner = [&](int p, int q, double out[3]) {
    int a, b, cc;
    switch (s) {
      case 0: a = q; b = p; cc = 0; break;
      case 1: a = p; b = 0; cc = q; break;
      case 2: a = 1; b = p; cc = q; break;
      case 3: a = 1 - p; b = 1; cc = q; break;
      case 4: a = 0; b = q; cc = p; break;
      default: a = p; b = q; cc = 1; break;
    }
    const double* X = xcl + ((size_t)e * 8 + (a + 2 * b + 4 * cc)) * 3;
    out[0] = X[0]; out[1] = X[1]; out[2] = X[2];
  };
  double P00[3], P10[3], P01[3], P11[3], ctr[3];
  corner(0, 0, P00); corner(1, 0, P10); corner(0, 1, P01); corner(1, 1, P11);
  for (int c = 0; c < 3; ++c) {
    g[c] = ((+P00[c] + P10[c]) + P01[c]) + P11[c];
    g[3 + c] = ((-P00[c] + P10[c]) - P01[c]) + P11[c];
    g[6 + c] = ((-P00[c] - P10[c]) + P01[c]) + P11[c];
    g[16 + c] = ((+P00[c] - P10[c]) - P01[c]) + P11[c];
    ctr[c] = 0.25 * (((P00[c] + P10[c]) + P01[c]) + P11[c]);
    g[19 + c] = P00[c]; g[22 + c] = P10[c]; g[25 + c] = P01[c]; g[28 + c] = P11[c];
  }
  const double* v1 = g + 3;
  const double* v2 = g + 6;
  double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
  const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int c = 0; c < 3; ++c) n[c] = n[c] / len;
  const double* Pc[4] = {P00, P10, P01, P11};
  double hmin = 1e300, hmax = -1e300;
  for (int k = 0; k < 4; ++k) {
    const double d = Pc[k][0] * n[0] + Pc[k][1] * n[1] + Pc[k][2] * n[2];
    hmin = std::min(hmin, d); hmax = std::max(hmax, d);
  }
  const double l1 = 0.5 * std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  const double l2 = 0.5 * std::sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  const double h = hmax - hmin, dmax = std::max(h, std::max(l1, l2));
  if (given == 2 || given == 4 || (given < 0 && !(h < 1.0e-6 * dmax))) {
    for (int c = 0; c < 3; ++c) g[9 + c] = n[c];
    g[12] = 0.0;
    g[15] = given == 4 ? 4.0 : 2.0;                // CURVED / BILINEAR
    return;
  }
  const double* b = bary + (size_t)e * 3;
  const double vb[3] = {ctr[0] - b[0], ctr[1] - b[1], ctr[2] - b[2]};
  if (vb[0] * n[0] + vb[1] * n[1] + vb[2] * n[2] < 0.0)
    for (int c = 0; c < 3; ++c) n[c] = -n[c];
  for (int c = 0; c < 3; ++c) g[9 + c] = n[c];
  g[12] = ctr[0] * n[0] + ctr[1] * n[1] + ctr[2] * n[2];
  auto unit = [](const double a[3], const double b0[3], double u[3]) {
    double d[3] = {a[0] - b0[0], a[1] - b0[1], a[2] - b0[2]};
    double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (std::fabs(l) > 0.0) { l = 1.0 / l; u[0] = d[0] * l; u[1] = d[1] * l; u[2] = d[2] * l; }
    else { u[0] = u[1] = u[2] = 0.0; }
  };
  double u1[3], u2[3], u3[3], u4[3];
  unit(P01, P00, u1); unit(P10, P00, u2); unit(P11, P01, u3); unit(P11, P10, u4);
  auto dz = [](const double a[3], const double bb[3]) { return std::fabs(a[0] * bb[0] + a[1] * bb[1] + a[2] * bb[2]) <= 2.22e-16; };
  const bool rect = dz(u1, u2) && dz(u1, u3) && dz(u4, u2) && dz(u4, u3);
  g[15] = given >= 0 ? (double)given : (rect ? 0.0 : 1.0);   // PLANAR_RECT / PLANAR_NONRECT (/ PLANAR_CURVED)
}

// FacNchooseK, Xi_NGeo and D_Bezier of NGeo (BuildBezierVdm, basis.f90:275-358; particle_mesh_tools.f90:
// 1470-1473; BuildBezierDMat, basis.f90:361-402)
static void bezier_basis(int ng, pic::BzBasis& B) {
  std::memset(&B, 0, sizeof(B));
  B.ng = ng;
  auto ipow = [](double x, int n) { double r = 1.0; for (int i = 0; i < n; ++i) r = r * x; return r; };
  for (int i = 0; i <= ng; ++i)
    for (int j = 0; j <= i; ++j) {
      double c = 1.0;
      for (int q = 0; q < j; ++q) c = c * (double)(i - q) / (double)(q + 1);
      B.fnk[i][j] = (1.0 / ipow(2.0, i)) * c;
    }
  for (int i = 0; i <= ng; ++i) B.xi[i] = 2.0 / (double)ng * (double)i - 1.0;
  for (int i = 0; i <= ng; ++i) B.dbez[i][0] = -B.fnk[ng][0] * (double)ng * ipow(1 - B.xi[i], ng - 1);
  for (int i = 0; i <= ng; ++i) B.dbez[i][ng] = B.fnk[ng][ng] * (double)ng * ipow(B.xi[i] + 1, ng - 1);
  for (int j = 1; j <= ng - 1; ++j)
    for (int i = 0; i <= ng; ++i) {
      const double XiPlus = B.xi[i] + 1.0, XiMinus = 1.0 - B.xi[i];
      B.dbez[i][j] = B.fnk[ng][j] * ((double)j * ipow(XiPlus, j - 1) * ipow(XiMinus, ng - j) -
                                     (double)(ng - j) * ipow(XiPlus, j) * ipow(XiMinus, ng - j - 1));
    }
}

// GetSideSlabNormalsAndIntervals (particle_surfaces.f90:619-816, BezierElevation = 0) of a side's Bezier
// points bcp[(q (NGeo+1) + p) 3 + c]: fills kBzGeo doubles (points, slab normals and intervals,
// BoundingBoxIsEmpty).  Returns false where the reference aborts (a degenerated side).
static bool bezier_side_slab(int ng, const double* bcp, double* S) {
  const int n1 = ng + 1;
  for (int k = 0; k < n1 * n1 * 3; ++k) S[k] = bcp[k];
  auto CP = [&](int p, int q, int c) { return bcp[(q * n1 + p) * 3 + c]; };
  auto crossnorm = [](const double a[3], const double b[3], double n[3]) {
    n[0] = a[1] * b[2] - a[2] * b[1];
    n[1] = a[2] * b[0] - a[0] * b[2];
    n[2] = a[0] * b[1] - a[1] * b[0];
    const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] = n[0] / l; n[1] = n[1] / l; n[2] = n[2] / l;
  };
  double n1v[3], n2v[3], n3v[3], t[3];
  for (int c = 0; c < 3; ++c) n1v[c] = ((CP(ng, 0, c) - CP(0, 0, c)) + CP(ng, ng, c)) - CP(0, ng, c);
  if (n1v[0] == 0.0 && n1v[1] == 0.0 && n1v[2] == 0.0) return false;
  const double l = std::sqrt(n1v[0] * n1v[0] + n1v[1] * n1v[1] + n1v[2] * n1v[2]);
  for (int c = 0; c < 3; ++c) n1v[c] = n1v[c] / l;
  for (int c = 0; c < 3; ++c) t[c] = ((CP(0, ng, c) - CP(0, 0, c)) + CP(ng, ng, c)) - CP(ng, 0, c);
  crossnorm(n1v, t, n2v);
  crossnorm(n2v, n1v, n3v);
  double* sn = S + pic::kBzSlabN;
  double* si = S + pic::kBzSlabI;
  for (int c = 0; c < 3; ++c) { sn[c] = n1v[c]; sn[3 + c] = n2v[c]; sn[6 + c] = n3v[c]; }
  for (int k = 0; k < 6; ++k) si[k] = 0.0;
  for (int q = 0; q <= ng; ++q)
    for (int p = 0; p <= ng; ++p) {
      if (p == 0 && q == 0) continue;
      const double d[3] = {CP(p, q, 0) - CP(0, 0, 0), CP(p, q, 1) - CP(0, 0, 1), CP(p, q, 2) - CP(0, 0, 2)};
      for (int i = 0; i < 3; ++i) {
        const double sk = (d[0] * sn[3 * i] + d[1] * sn[3 * i + 1]) + d[2] * sn[3 * i + 2];
        if (sk < 0.0) si[2 * i] = std::fmin(si[2 * i], sk);
        else if (sk > 0.0) si[2 * i + 1] = std::fmax(si[2 * i + 1], sk);
      }
    }
  const double dx = std::fabs(si[1] - si[0]), dy = std::fabs(si[3] - si[2]), dz = std::fabs(si[5] - si[4]);
  double h = dy;
  const double w = std::fmin(dx, dz), len = std::fmax(dx, dz);
  const double dMax = std::fmax(h, std::fmax(len, w));
  if (len / dMax < 1.0e-6 || w / dMax < 1.0e-6) return false;
  if (h / dMax < 1.0e-6) { si[2] = 0.0; si[3] = 0.0; h = 0.0; }
  S[pic::kBzEmpty] = std::fabs(h / std::sqrt(len * len + w * w + h * h)) <= pic::kEpsMach ? 1.0 : 0.0;
  return true;
}

int pic_create(const pic_config_t* cfg, const pic_mesh_t* m, pic_ctx_t** out) {
  if (!out) return fail(PIC_ERR_INVALID_ARGUMENT, "ctx_out is null");
  *out = nullptr;
  int rc = validate(cfg, m);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(PIC_ERR_NO_DEVICE, "no CUDA device");
  pic_ctx* c = new pic_ctx();
  c->cfg = *cfg;
  c->N = cfg->n_dg;
  const int n1 = c->N + 1;
  c->nd = n1 * n1 * n1;
  c->ne = m->n_elems;
  c->mixed = cfg->precision == PIC_PREC_MIXED;
  c->refmap = cfg->tracking == PIC_TRACK_REFMAPPING;
  c->sf = cfg->deposition != PIC_DEPO_CVWM;
  c->adaptive = cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_ADAPTIVE;
  c->cc = cfg->deposition == PIC_DEPO_SHAPE_FUNCTION_CC || c->adaptive;     // both normalise per particle
  c->sf_rmax = cfg->sf_radius;
  const int ne = c->ne, nd = c->nd;
  auto bail = [&](int code) { pic_destroy(c); return code; };
  // degree and DOF offset of every element (N_DG_Mapping rows 2 and 1; e (N+1)^3 without a mapping)
  c->var_n = m->n_dg_mapping != nullptr;
  c->elem_n_h.assign(ne, c->N);
  c->dof_off_h.assign(ne + 1, 0);
  for (int e = 0; e < ne; ++e) {
    if (c->var_n) c->elem_n_h[e] = m->n_dg_mapping[(size_t)e * 3 + 1];
    c->dof_off_h[e + 1] = c->dof_off_h[e] + c->nd_of(e);
  }
  c->ndofs = (size_t)c->dof_off_h[ne];
  if (c->adaptive && (cfg->n_dg > 3 || pic::sf_gather_variant() != 5))
    return bail(fail(PIC_ERR_INVALID_ARGUMENT, "shape_function_adaptive needs N <= 3 and the round-robin gather"));
  if (c->adaptive) {
    c->sf_rmax = 0.0;
    for (int e = 0; e < m->n_elems; ++e) c->sf_rmax = std::max(c->sf_rmax, m->sf_elem_radius[e]);
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(PIC_ERR_CUDA, "cudaStreamCreate failed"));
  if (cudaEventCreateWithFlags(&c->noalloc_done, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(PIC_ERR_CUDA, "cudaEventCreate failed"));

  // ---- element geometry -------------------------------------------------------------------
  // each element's corners and their dXCL_NGeo (XCL_NGeo1, dXCL_NGeo1 of GetPositionInRefElem; XCL_NGeo itself at
  // NGeo = 1), tensor order i + 2 j + 4 k
  const int ng = m->n_geo, g1 = ng + 1;
  const size_t g3 = (size_t)g1 * g1 * g1;
  std::vector<double> xcl((size_t)ne * 24), dxcl((size_t)ne * 72);
  for (int e = 0; e < ne; ++e)
    for (int t = 0; t < 8; ++t) {
      const size_t q = (size_t)e * g3 + (size_t)((t >> 2) * ng * g1 + ((t >> 1) & 1) * ng) * g1 + (t & 1) * ng;
      for (int c = 0; c < 3; ++c) xcl[((size_t)e * 8 + t) * 3 + c] = m->xcl_ngeo[q * 3 + c];
      for (int c = 0; c < 9; ++c) dxcl[((size_t)e * 8 + t) * 9 + c] = m->dxcl_ngeo[q * 9 + c];
    }
  std::vector<double> bary(m->elem_bary, m->elem_bary + (size_t)ne * 3);
  std::vector<double> xez(m->xez_basis, m->xez_basis + (size_t)ne * 18);
  std::vector<double> slen(m->slen_basis, m->slen_basis + (size_t)ne * 6);
  std::vector<double> rad(m->elem_radius, m->elem_radius + ne);
  std::vector<double> eps1(ne, 1.0);
  if (m->eps_one_cell) eps1.assign(m->eps_one_cell, m->eps_one_cell + ne);
  std::vector<double> exgp(m->elem_xgp, m->elem_xgp + c->ndofs * 3);
  std::vector<int> side_nb((size_t)ne * 6);
  std::vector<uint32_t> side_info((size_t)ne * 6);
  for (int e = 0; e < ne; ++e) {
    for (int t = 0; t < 8; ++t)
      for (int d = 0; d < 3; ++d)
        if (m->node_coords[((size_t)e * 8 + t) * 3 + d] != xcl[((size_t)e * 8 + t) * 3 + d])
          return bail(fail(PIC_ERR_INVALID_ARGUMENT, "node_coords must hold each element's 8 corners (tensor order)"));
    for (int s = 0; s < 6; ++s) {
      const int nb = m->side_nb_elem[e * 6 + s];
      const int bc = m->side_bc ? m->side_bc[e * 6 + s] : 0;
      if (bc < 0 || bc > 3) return bail(fail(PIC_ERR_INVALID_ARGUMENT, "side_bc must be 0..3"));
      const bool wall = bc == 1 || bc == 2;
      if (wall ? nb != 0 : (nb < 1 || nb > ne))
        return bail(fail(PIC_ERR_INVALID_ARGUMENT, "side_nb_elem must be 1..nElems, or 0 exactly at open/reflective sides"));
      // shape functions near walls: no images, the kernel ends at the wall (calcSfSource with
      // NbrOfPeriodicSFCases = 0; _cc and _adaptive renormalise what is left)
      if (wall && !(cfg->deposition == PIC_DEPO_CVWM || m->n_periodic_vectors == 0))
        return bail(fail(PIC_ERR_INVALID_ARGUMENT,
                         "open/reflective particle boundaries need cell_volweight_mean, or a shape function on a mesh "
                         "without periodic sides"));
      if (wall && cfg->tracking == PIC_TRACK_REFMAPPING &&
          ((m->n_periodic_vectors > 0 && !cfg->periodic_tracing) || !m->elem_to_bc_sides))
        return bail(fail(PIC_ERR_INVALID_ARGUMENT,
                         "RefTracking with walls needs elem_to_bc_sides, and periodic_tracing = 1 on a mesh with "
                         "periodic sides"));
      c->has_walls = c->has_walls || wall;
      side_nb[e * 6 + s] = wall ? -1 : nb - 1;
      uint32_t info = 0;
      for (int q = 0; q < 4; ++q) {
        const int t = m->elem_side_node[((size_t)e * 6 + s) * 4 + q] - 1 - 8 * e;
        if (t < 0 || t > 7) return bail(fail(PIC_ERR_INVALID_ARGUMENT, "elem_side_node must point at the element's own corners"));
        info |= (uint32_t)t << (3 * q);
      }
      if (m->concave_side[e * 6 + s]) info |= 1u << 12;
      const int pv = m->side_pvid[e * 6 + s];
      if (pv < -m->n_periodic_vectors || pv > m->n_periodic_vectors)
        return bail(fail(PIC_ERR_INVALID_ARGUMENT, "side_pvid out of range"));
      info |= ((uint32_t)(uint8_t)(int8_t)pv) << 16;
      if (wall) info |= (uint32_t)bc << 24;     // 1 open, 2 reflective
      side_info[e * 6 + s] = info;
    }
  }
  // ---- RefTracking wall sides: BC-element lists and planar-side geometry ------------------------
  std::vector<int> bc_e2b;
  std::vector<double> bc_geo, bc_bz;
  // BC sides: the open/reflective walls, and with periodic_tracing (CartesianPeriodic = F) the periodic sides
  const bool bc_lists = cfg->tracking == PIC_TRACK_REFMAPPING &&
                        (m->n_periodic_vectors > 0 ? cfg->periodic_tracing != 0 : c->has_walls);
  if (bc_lists) {
    const int nent = m->n_bc_entries;
    if (nent < 1 || !m->elem_to_bc_sides || !m->bc_side_elem_loc || !m->bc_side_distance)
      return bail(fail(PIC_ERR_INVALID_ARGUMENT,
                       "elem_to_bc_sides/n_bc_entries/bc_side_elem_loc/bc_side_distance missing"));
    bc_e2b.assign(m->elem_to_bc_sides, m->elem_to_bc_sides + (size_t)ne * 2);
    for (int e = 0; e < ne; ++e) {
      const int n = bc_e2b[2 * e], f = bc_e2b[2 * e + 1];
      if (n > 0 ? (f < 0 || f + n > nent) : (n != -1 && n != 0))
        return bail(fail(PIC_ERR_INVALID_ARGUMENT, "elem_to_bc_sides out of range"));
      if (n <= 0) { bc_e2b[2 * e] = -1; bc_e2b[2 * e + 1] = -1; }
    }
    bc_geo.assign((size_t)nent * kBcGeo, 0.0);
    if (ng > 1) bc_bz.assign((size_t)nent * pic::kBzGeo, 0.0);
    for (int k = 0; k < nent; ++k) {
      const int e = m->bc_side_elem_loc[2 * k] - 1, sd = m->bc_side_elem_loc[2 * k + 1] - 1;
      const bool periodic_side = e >= 0 && e < ne && sd >= 0 && sd <= 5 && cfg->periodic_tracing &&
                                 m->side_pvid[e * 6 + sd] != 0 && m->side_nb_elem[e * 6 + sd] != 0;
      if (e < 0 || e >= ne || sd < 0 || sd > 5 || (m->side_nb_elem[e * 6 + sd] != 0 && !periodic_side))
        return bail(fail(PIC_ERR_INVALID_ARGUMENT, "bc_side_elem_loc must name open/reflective wall sides, or "
                                                   "periodic sides with periodic_tracing"));
      int given = -1;
      if (ng > 1) {
        // the side's SideType and Bezier patch (BezierControlPoints3D, slab normals and intervals)
        given = m->side_type[e * 6 + sd];
        if (given < 0 || given > 4) return bail(fail(PIC_ERR_INVALID_ARGUMENT, "side_type must be 0..4"));
        if (!bezier_side_slab(ng, m->side_bezier + ((size_t)e * 6 + sd) * g1 * g1 * 3, &bc_bz[(size_t)k * pic::kBzGeo]))
          return bail(fail(PIC_ERR_INVALID_ARGUMENT, "degenerated Bezier side (GetSideSlabNormalsAndIntervals)"));
      }
      wall_side_geometry(xcl.data(), bary.data(), e, sd, &bc_geo[(size_t)k * kBcGeo], given);
      bc_geo[(size_t)k * kBcGeo + 13] = m->bc_side_distance[k];
      if (periodic_side) {
        // PeriodicBC: the neighbour element (0-based) and BoundaryType(BC_ALPHA) of the side
        bc_geo[(size_t)k * kBcGeo + 14] = 3.0;
        bc_geo[(size_t)k * kBcGeo + 31] =
            (double)(m->side_nb_elem[e * 6 + sd] - 1) * 16.0 + (double)(m->side_pvid[e * 6 + sd] + 8);
      } else {
        bc_geo[(size_t)k * kBcGeo + 14] = (double)m->side_bc[e * 6 + sd];
      }
    }
  }
  // ---- periodic-unique nodes (merge Periodic_Nodes twins) ----------------------------------
  const int nn = m->n_nodes;
  std::vector<int> rep(nn);
  for (int u = 0; u < nn; ++u) {
    int r = u;
    if (m->periodic_n_nodes && m->periodic_offset && m->periodic_nodes)
      for (int j = 0; j < m->periodic_n_nodes[u]; ++j) r = std::min(r, m->periodic_nodes[m->periodic_offset[u] + j] - 1);
    rep[u] = r;
  }
  std::vector<int> canon_id(nn, -1);
  int ncanon = 0;
  for (int u = 0; u < nn; ++u)
    if (rep[u] == u) canon_id[u] = ncanon++;
  for (int u = 0; u < nn; ++u) canon_id[u] = canon_id[rep[u]];
  std::vector<double> nvol(ncanon, 0.0);
  for (int u = 0; u < nn; ++u)
    if (rep[u] == u) nvol[canon_id[u]] = m->node_volume ? m->node_volume[u] : 1.0;
  std::vector<int> ecan((size_t)ne * 8);
  for (size_t q = 0; q < (size_t)ne * 8; ++q) {
    const int u = m->node_info[q] - 1;
    if (u < 0 || u >= nn) return bail(fail(PIC_ERR_INVALID_ARGUMENT, "node_info out of range"));
    ecan[q] = canon_id[u];
  }
  c->n_canon = ncanon;
  // ---- FP32 mapping copies (mixed) ----------------------------------------------------------
  std::vector<float> xclr((size_t)ne * 24), dxclf((size_t)ne * 72), xezf((size_t)ne * 18), slenf((size_t)ne * 6);
  for (int e = 0; e < ne; ++e) {
    for (int t = 0; t < 8; ++t)
      for (int d = 0; d < 3; ++d) xclr[(e * 8 + t) * 3 + d] = (float)(xcl[(e * 8 + t) * 3 + d] - bary[e * 3 + d]);
    for (int q = 0; q < 72; ++q) dxclf[(size_t)e * 72 + q] = (float)dxcl[(size_t)e * 72 + q];
    for (int q = 0; q < 18; ++q) xezf[(size_t)e * 18 + q] = (float)xez[(size_t)e * 18 + q];
    for (int q = 0; q < 6; ++q) slenf[(size_t)e * 6 + q] = (float)slen[(size_t)e * 6 + q];
  }
  // ---- FIBGM -------------------------------------------------------------------------------
  std::vector<int> fn, fo, fe;
  if (m->fibgm_n_elems) {
    const size_t ncell = (size_t)m->fibgm_imax[0] * m->fibgm_imax[1] * m->fibgm_imax[2];
    fn.assign(m->fibgm_n_elems, m->fibgm_n_elems + ncell);
    fo.assign(m->fibgm_offset, m->fibgm_offset + ncell);
    fe.resize(m->fibgm_n_total);
    for (int q = 0; q < m->fibgm_n_total; ++q) fe[q] = m->fibgm_element[q] - 1;
  } else {
    fn.assign(1, 0); fo.assign(1, 0); fe.assign(1, 0);
  }
  // ---- upload mesh ---------------------------------------------------------------------------
  double *d_xcl, *d_dxcl, *d_bary, *d_xez, *d_slen, *d_rad, *d_eps1, *d_exgp, *d_nvol;
  int *d_snb, *d_ecan, *d_fn, *d_fo, *d_fe;
  uint32_t* d_sinfo;
  float *d_xclr, *d_dxclf, *d_xezf, *d_slenf;
  if ((rc = upload(c, &d_xcl, xcl)) || (rc = upload(c, &d_dxcl, dxcl)) || (rc = upload(c, &d_bary, bary)) ||
      (rc = upload(c, &d_xez, xez)) || (rc = upload(c, &d_slen, slen)) || (rc = upload(c, &d_rad, rad)) ||
      (rc = upload(c, &d_eps1, eps1)) || (rc = upload(c, &d_exgp, exgp)) || (rc = upload(c, &d_nvol, nvol)) ||
      (rc = upload(c, &d_snb, side_nb)) || (rc = upload(c, &d_sinfo, side_info)) || (rc = upload(c, &d_ecan, ecan)) ||
      (rc = upload(c, &d_fn, fn)) || (rc = upload(c, &d_fo, fo)) || (rc = upload(c, &d_fe, fe)) ||
      (rc = upload(c, &d_xclr, xclr)) || (rc = upload(c, &d_dxclf, dxclf)) || (rc = upload(c, &d_xezf, xezf)) ||
      (rc = upload(c, &d_slenf, slenf)))
    return bail(rc);
  c->M = DevMesh{ne, d_xcl, d_dxcl, d_bary, d_xez, d_slen, d_rad, d_eps1, d_snb, d_sinfo, d_ecan, d_nvol, d_exgp,
                 d_fn, d_fo, d_fe, d_xclr};
  c->M.sf_xgp = d_exgp;
  if (ng > 1) {
    std::vector<double> xng(m->xcl_ngeo, m->xcl_ngeo + (size_t)ne * g3 * 3), dng(m->dxcl_ngeo, m->dxcl_ngeo + (size_t)ne * g3 * 9);
    std::vector<int> crv(ne, 1);
    if (m->elem_curved)
      for (int e = 0; e < ne; ++e) crv[e] = m->elem_curved[e] ? 1 : 0;
    double *d_xng = nullptr, *d_dng = nullptr;
    int* d_crv = nullptr;
    if ((rc = upload(c, &d_xng, xng)) || (rc = upload(c, &d_dng, dng)) || (rc = upload(c, &d_crv, crv))) return bail(rc);
    c->M.xcl_ng = d_xng; c->M.dxcl_ng = d_dng; c->M.curved = d_crv;
  }
  if (c->var_n) {
    int *d_doff = nullptr, *d_en = nullptr;
    if ((rc = upload(c, &d_doff, c->dof_off_h)) || (rc = upload(c, &d_en, c->elem_n_h))) return bail(rc);
    c->M.dof_off = d_doff;
    c->M.elem_n = d_en;
  }
  if (!bc_e2b.empty()) {
    int* d_be = nullptr;
    double* d_bg = nullptr;
    if ((rc = upload(c, &d_be, bc_e2b)) || (rc = upload(c, &d_bg, bc_geo))) return bail(rc);
    c->M.bc_e2b = d_be;
    c->M.bc_geo = d_bg;
    if (!bc_bz.empty()) {
      double* d_bz = nullptr;
      if ((rc = upload(c, &d_bz, bc_bz))) return bail(rc);
      c->M.bc_bz = d_bz;
    }
  }
  c->MF = MeshF{d_xclr, d_dxclf, d_xezf, d_slenf};
  if (c->mixed) {
    // the NGeo = 1 map in monomial form for the mixed Newton: x = 1/8 sum_t X_t (1 + s_a xi1)(1 + s_b xi2)(1 + s_c xi3),
    // s = -1 / +1 for the corner's low / high index; coefficients (c0, c1, c2, c3, c12, c13, c23, c123)
    std::vector<double> tc((size_t)ne * 24, 0.0);
    for (int e = 0; e < ne; ++e)
      for (int t = 0; t < 8; ++t) {
        const double sa = (t & 1) ? 1.0 : -1.0, sb = (t & 2) ? 1.0 : -1.0, sc = (t & 4) ? 1.0 : -1.0;
        const double w[8] = {1.0, sa, sb, sc, sa * sb, sa * sc, sb * sc, sa * sb * sc};
        for (int q = 0; q < 8; ++q)
          for (int k = 0; k < 3; ++k) tc[(size_t)e * 24 + 3 * q + k] += 0.125 * w[q] * xcl[(size_t)e * 24 + 3 * t + k];
      }
    // the same coefficients relative to the element's barycentre (c0 - bary) over s_e = 2^round(log2 max|c1..c3|)
    // as double-FP32 pairs, then (s_e, 1/s_e) and the start-value data of RefMappingGuess 1 in the same frame and
    // units (bary - bary = 0, XiEtaZetaBasis, slen s_e): every value O(1) wherever the element lies
    auto pair = [](double v) { const float hi = (float)v; return make_float2(hi, (float)(v - (double)hi)); };
    auto start_data = [&](int e, double sc, float2* out) {
      for (int d = 0; d < 3; ++d) out[d] = make_float2(0.f, 0.f);
      for (int d = 0; d < 18; ++d) out[3 + d] = pair(xez[(size_t)e * 18 + d]);
      for (int d = 0; d < 6; ++d) out[21 + d] = pair(slen[(size_t)e * 6 + d] * sc);
    };
    std::vector<float2> tdf((size_t)ne * pic::kDfLin);
    for (int e = 0; e < ne; ++e) {
      double mx = 0.0;
      for (int q = 1; q <= 3; ++q)
        for (int k = 0; k < 3; ++k) mx = std::max(mx, std::fabs(tc[(size_t)e * 24 + 3 * q + k]));
      const double sc = mx > 0.0 ? std::ldexp(1.0, (int)std::lround(std::log2(mx))) : 1.0;
      for (int j = 0; j < 24; ++j)
        tdf[(size_t)e * pic::kDfLin + j] = pair((j < 3 ? tc[(size_t)e * 24 + j] - bary[(size_t)e * 3 + j] : tc[(size_t)e * 24 + j]) / sc);
      tdf[(size_t)e * pic::kDfLin + 24] = make_float2((float)sc, (float)(1.0 / sc));
      start_data(e, sc, &tdf[(size_t)e * pic::kDfLin + 25]);
    }
    float2* d_tdf = nullptr;
    if ((rc = upload(c, &d_tdf, tdf))) return bail(rc);
    c->M.tcoef_df = d_tdf;
    if (ng > 1) {
      // the NGeo map in power form: along each axis C_a = sum_i T(a,i) X_i with T = V^-1, V(i,a) = XiCL_i^a
      double V[5][10];
      for (int i = 0; i < g1; ++i)
        for (int a = 0; a < g1; ++a) {
          V[i][a] = std::pow(m->xi_cl_ngeo[i], a);
          V[i][g1 + a] = i == a ? 1.0 : 0.0;
        }
      for (int col = 0; col < g1; ++col) {
        int p = col;
        for (int r = col + 1; r < g1; ++r) if (std::fabs(V[r][col]) > std::fabs(V[p][col])) p = r;
        for (int q = 0; q < 2 * g1; ++q) std::swap(V[col][q], V[p][q]);
        const double piv = V[col][col];
        for (int q = 0; q < 2 * g1; ++q) V[col][q] /= piv;
        for (int r = 0; r < g1; ++r)
          if (r != col) { const double fct = V[r][col]; for (int q = 0; q < 2 * g1; ++q) V[r][q] -= fct * V[col][q]; }
      }
      std::vector<double> pc((size_t)ne * g3 * 3);
      for (int e = 0; e < ne; ++e)
        for (int k = 0; k < 3; ++k) {
          double A[125], B[125];
          for (size_t q = 0; q < g3; ++q) A[q] = m->xcl_ngeo[((size_t)e * g3 + q) * 3 + k];
          for (int ax = 0; ax < 3; ++ax) {
            const int st = ax == 0 ? 1 : ax == 1 ? g1 : g1 * g1;
            for (int q = 0; q < (int)g3; ++q) {
              const int aa = (q / st) % g1, base = q - aa * st;
              double v = 0.0;
              for (int l = 0; l < g1; ++l) v += V[aa][g1 + l] * A[base + l * st];
              B[q] = v;
            }
            for (size_t q = 0; q < g3; ++q) A[q] = B[q];
          }
          for (size_t q = 0; q < g3; ++q) pc[((size_t)e * g3 + q) * 3 + k] = A[q];
        }
      // the same over s_e = 2^round(log2 max |first-order coefficient|) as double-FP32 pairs, then (s_e, 1/s_e)
      const size_t nb = g3 * 3 + 1 + pic::kDfStart;
      std::vector<float2> pdf((size_t)ne * nb);
      for (int e = 0; e < ne; ++e) {
        double mx = 0.0;
        const size_t first[3] = {1, (size_t)g1, (size_t)g1 * g1};     // the xi1, xi2, xi3 terms
        for (int a = 0; a < 3; ++a)
          for (int k = 0; k < 3; ++k) mx = std::max(mx, std::fabs(pc[((size_t)e * g3 + first[a]) * 3 + k]));
        const double sc = mx > 0.0 ? std::ldexp(1.0, (int)std::lround(std::log2(mx))) : 1.0;
        for (size_t j = 0; j < g3 * 3; ++j)   // j < 3: the constant term, relative to the barycentre
          pdf[(size_t)e * nb + j] = pair((j < 3 ? pc[(size_t)e * g3 * 3 + j] - bary[(size_t)e * 3 + j] : pc[(size_t)e * g3 * 3 + j]) / sc);
        pdf[(size_t)e * nb + g3 * 3] = make_float2((float)sc, (float)(1.0 / sc));
        start_data(e, sc, &pdf[(size_t)e * nb + g3 * 3 + 1]);
      }
      float2* d_pdf = nullptr;
      if ((rc = upload(c, &d_pdf, pdf))) return bail(rc);
      c->M.tcoef_ng_df = d_pdf;
    }
  }

  // ---- constants -------------------------------------------------------------------------------
  Consts k{};
  k.N = c->N; k.n1 = n1; k.ndof = nd; k.n_species = cfg->n_species;
  for (int s = 0; s < 8; ++s) k.dt_fac[s] = 1.0;
  for (int s = 0; s < cfg->n_species; ++s) {
    k.q[s] = cfg->charge[s]; k.m[s] = cfg->mass[s]; k.mpf[s] = cfg->mpf[s];
    k.qm[s] = cfg->charge[s] * cfg->mpf[s];
    if (cfg->time_step_factor[s] > 0.0) k.dt_fac[s] = cfg->time_step_factor[s];
  }
  for (int q = 0; q < 6; ++q) k.ext[q] = cfg->external_field[q];
  k.periodic_tracing = (cfg->tracking == PIC_TRACK_REFMAPPING && cfg->periodic_tracing) ? 1 : 0;
  k.ref_guess = cfg->ref_mapping_guess ? cfg->ref_mapping_guess : 1;
  k.refmapping_eps = cfg->refmapping_eps > 0.0 ? cfg->refmapping_eps : 1e-4;
  const double c2 = 299792458.0 * 299792458.0;
  k.c2_inv = 1.0 / c2;
  c->xgp_h.assign(m->xgp, m->xgp + n1);
  c->wgp_h.assign(m->wgp, m->wgp + n1);
  for (int i = 0; i < n1; ++i) {
    k.xgp[i] = m->xgp[i]; k.wbary_gp[i] = m->wbary_gp[i];
    k.fac_gp[i] = (m->xgp[i] + 1.0) / 2.0;    // CellVolWeight%Fac, pic_depo.f90:274-275
    k.xgp_f[i] = (float)m->xgp[i]; k.wbary_gp_f[i] = (float)m->wbary_gp[i];
  }
  // the tables per degree: N_Inter(1..NMax) of a p-adapted mesh, else row N = N_Inter(N)
  for (int kd = 1; kd <= c->N; ++kd) {
    if (!c->var_n && kd != c->N) continue;
    const double* xg = c->var_n ? m->n_inter + 3 * ((kd - 1) * (kd + 2) / 2) : m->xgp;
    const double* wb = c->var_n ? xg + 2 * (kd + 1) : m->wbary_gp;
    for (int i = 0; i <= kd; ++i) {
      k.xgp_n[kd][i] = xg[i]; k.wbary_n[kd][i] = wb[i];
      k.fac_n[kd][i] = (xg[i] + 1.0) / 2.0;   // CellVolWeight(Nloc)%Fac
      k.xgp_nf[kd][i] = (float)xg[i]; k.wbary_nf[kd][i] = (float)wb[i];
    }
  }
  k.ngeo = ng;
  if (ng > 1) bezier_basis(ng, k.bz);
  {
    // the mixed Newton's constants in double-FP32: RefMappingEps, 1 + RefMappingEps, -lambda_k and 1 - 1e-4 lambda_k
    auto pair = [](double v) { const float hi = (float)v; return make_float2(hi, (float)(v - (double)hi)); };
    k.df_eps = pair(k.refmapping_eps);
    k.df_one_eps = pair(1.0 + k.refmapping_eps);
    double lambda = 1.0;
    for (int j = 0; j < 9; ++j) {
      k.df_lam[j] = pair(-lambda);
      k.df_arm[j] = pair(1.0 - 0.0001 * lambda);
      lambda = 0.2 * lambda;
    }
  }
  for (int i = 0; i <= ng; ++i) { k.xi_cl_ng[i] = m->xi_cl_ngeo[i]; k.wbary_cl_ng[i] = m->wbary_cl_ngeo[i]; }
  if (ng == 1) {
    k.xi_cl[0] = m->xi_cl_ngeo[0]; k.xi_cl[1] = m->xi_cl_ngeo[1];
    k.wbary_cl[0] = m->wbary_cl_ngeo[0]; k.wbary_cl[1] = m->wbary_cl_ngeo[1];
  } else {   // XiCL_NGeo1 = ChebyGaussLobNodes(1), wBaryCL_NGeo1 = its barycentric weights
    k.xi_cl[0] = -1.0; k.xi_cl[1] = 1.0;
    k.wbary_cl[0] = -0.5; k.wbary_cl[1] = 0.5;
  }
  k.n_pv = m->n_periodic_vectors;
  for (int q = 0; q < 9; ++q) k.pv[q] = m->periodic_vectors[q];
  for (int d = 0; d < 3; ++d) {
    k.xmin[d] = m->xmin_glob[d]; k.xmax[d] = m->xmax_glob[d];
    k.fib_imax[d] = m->fibgm_imax[d] > 0 ? m->fibgm_imax[d] : 1;
    k.fib_delta[d] = m->fibgm_deltas[d] > 0.0 ? m->fibgm_deltas[d] : 1.0;
    k.pv_dir[d] = -1;
    for (int q = 0; q < m->n_periodic_vectors; ++q)
      if (m->periodic_vectors[3 * q + d] != 0.0) { k.pv_dir[d] = q; break; }   // GEO%DirPeriodicVectors
  }
  if (c->sf) {
    // the largest radius (adaptive: the per-element radii bound the searches; exact per-particle radii in the kernels)
    k.sf_r = c->sf_rmax; k.sf_r2 = c->sf_rmax * c->sf_rmax; k.sf_r2_inv = 1.0 / k.sf_r2;
    k.sf_r_inv = (float)(1.0 / c->sf_rmax);
    k.sf_alpha = cfg->sf_alpha;
    k.sf_w = c->cc ? 1.0 : sf_weight_dim(cfg, m, cfg->sf_radius, cfg->sf_alpha);   // cc: Fac = q MPF (v,1), normalised later
    // 1D/2D charge-conserving kernels with the charge on a line / an area (PIC-shapefunction-3D-deposition
    // = F): the periodic branch and the Adaptive routine divide their totals by dimFactorSF
    // (calcSfSource:117-119, depoChargeOnDOFsSFAdaptive:881-884); depoChargeOnDOFsSFChargeCon does not
    const bool on_line = (cfg->sf_dim == 1 || cfg->sf_dim == 2) && !cfg->sf_depo3d;
    k.sf_cc_div = (c->cc && on_line && (m->n_periodic_vectors > 0 || c->adaptive)) ? sf_dim_factor(cfg, m) : 1.0;
    bool keep[3];
    sf_kernel_dirs(cfg, keep);
    for (int d = 0; d < 3; ++d) k.sf_keep[d] = keep[d] ? 1 : 0;
  }
  c->M.k = k;   // travels with every launch (kernel parameter), so contexts do not share constants

  // ---- work arrays -------------------------------------------------------------------------------
  if ((rc = c->alloc(&c->E, c->ndofs * 3)) || (rc = c->alloc(&c->E32, c->ndofs * 3)) ||
      (rc = c->alloc(&c->NS, (size_t)ncanon * 4)) || (rc = c->alloc(&c->PS, c->ndofs * 4)) ||
      (rc = c->alloc(&c->st, 1)) || (rc = c->alloc(&c->d_count, 1)) ||
      (rc = c->alloc(&c->sortb.count, ne + 1)) || (rc = c->alloc(&c->sortb.offset, ne + 2)) ||
      (rc = c->alloc(&c->sortb.cursor, ne + 1)))
    return bail(rc);
  c->sortb.ne = ne;
  cudaMemset(c->st, 0, sizeof(DevStatus));
  cudaMemset(c->PS, 0, sizeof(double) * c->ndofs * 4);
  if ((rc = alloc_particles(c, c->P, cfg->max_particles, true)) || (rc = alloc_particles(c, c->Q, cfg->max_particles, false)) ||
      (rc = c->alloc(&c->perm, std::max(cfg->max_particles, 1))) || (rc = c->alloc(&c->perm_tmp, std::max(cfg->max_particles, 1))))
    return bail(rc);
  // the reorder buffer shares the auxiliary arrays (LastPartPos, field) of P
  c->Q.lx = c->P.lx; c->Q.ly = c->P.ly; c->Q.lz = c->P.lz; c->Q.field = c->P.field;
  if (c->sf) {
    // DOF coordinates the gather reads: the kernel directions only (all three for a 3D shape function)
    bool keep[3];
    sf_kernel_dirs(cfg, keep);
    std::vector<double> sfx(exgp);
    if (!(keep[0] && keep[1] && keep[2])) {
      for (size_t q = 0; q < c->ndofs; ++q)
        for (int d = 0; d < 3; ++d)
          if (!keep[d]) sfx[q * 3 + d] = 0.0;
      double* d_sfx = nullptr;
      if ((rc = upload(c, &d_sfx, sfx))) return bail(rc);
      c->M.sf_xgp = d_sfx;
    }
    std::vector<double> dofc((size_t)ne * 3);
    for (int e = 0; e < ne; ++e)
      for (int d = 0; d < 3; ++d) {
        double lo = 1e300, hi = -1e300;
        for (int r = 0; r < c->nd_of(e); ++r) {
          const double v = sfx[((size_t)c->dof_off_h[e] + r) * 3 + d];
          lo = std::min(lo, v); hi = std::max(hi, v);
        }
        dofc[(size_t)e * 3 + d] = 0.5 * (lo + hi);
      }
    if ((rc = build_sf_lists(c, m, dofc, sfx, keep))) return bail(rc);
    const size_t cap = (size_t)std::max(cfg->max_particles, 1);
    if ((rc = c->alloc(&c->sfk.posf, cap * 4))) return bail(rc);
    if (c->mixed) {
      if ((rc = c->alloc(&c->sfk.facf, cap * 4))) return bail(rc);
      if (c->sfl.elem_box &&
          ((rc = c->alloc(&c->sfk.sub_count, 8 * (size_t)ne + 1)) || (rc = c->alloc(&c->sfk.sub_off, 8 * (size_t)ne + 1)) ||
           (rc = c->alloc(&c->sfk.sub_cursor, 8 * (size_t)ne + 1))))
        return bail(rc);
    } else {
      if ((rc = c->alloc(&c->sfk.pos, cap * 3)) || (rc = c->alloc(&c->sfk.fac, cap * 4))) return bail(rc);
    }
  }
  // VerifyDepositedCharge (pic_analyze.f90:41-133): quadrature weight wGP(k) wGP(l) wGP(m) / sJ of every DOF, and the
  // factor of the analytical charge (dimFactorSF for a 1D/2D shape function whose charge sits on a line / area)
  if (m->elem_sj) {
    std::vector<double> wq(c->ndofs);
    for (int e = 0; e < ne; ++e) {
      const int n1e = c->elem_n_h[e] + 1;
      const double* wg = elem_wgp(c, m, e);
      const size_t b = (size_t)c->dof_off_h[e];
      for (int mm = 0; mm < n1e; ++mm)
        for (int l = 0; l < n1e; ++l)
          for (int k = 0; k < n1e; ++k) {
            const int r = k + n1e * (l + n1e * mm);
            wq[b + r] = wg[k] * wg[l] * wg[mm] * (1.0 / m->elem_sj[b + r]);
          }
    }
    if ((rc = upload(c, &c->charge_w, wq)) || (rc = c->alloc(&c->charge_elem, ne)) ||
        (rc = c->alloc(&c->charge_out, 1)) || (rc = c->alloc(&c->species_count, PIC_MAX_SPECIES)))
      return bail(rc);
  }
  c->charge_dim_factor = (c->sf && (cfg->sf_dim == 1 || cfg->sf_dim == 2) && !cfg->sf_depo3d) ? sf_dim_factor(cfg, m) : 1.0;
  if ((rc = device_sync(c))) return bail(rc);
  *out = c;
  return PIC_OK;
}

void pic_destroy(pic_ctx_t* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  hdg_destroy(c);
  for (auto& r : c->recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto e : c->pool) cudaEventDestroy(e);
  for (void* p : c->allocs) cudaFree(p);
  if (c->noalloc_done) cudaEventDestroy(c->noalloc_done);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int pic_set_field(pic_ctx_t* c, const double* e_dof, int32_t n_elems) {
  if (!c || !e_dof) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (n_elems != c->ne) return fail(PIC_ERR_INVALID_ARGUMENT, "n_elems does not match the mesh");
  const size_t n = c->ndofs * 3;
  CUDA_TRY(cudaMemcpyAsync(c->E, e_dof, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->mixed) k_to_float<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->E, c->E32, n);
  CUDA_TRY(cudaGetLastError());
  c->field_set = true;
  return PIC_OK;
}

__global__ void k_iota(int* p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = i;
}

int pic_upload_particles(pic_ctx_t* c, const double* ps, const int32_t* elem, const int32_t* species,
                         const uint8_t* inside, const uint8_t* is_new, int32_t n) {
  if (!c || (n > 0 && (!ps || !elem || !species))) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (n < 0) return fail(PIC_ERR_INVALID_ARGUMENT, "negative particle count");
  if (n > c->P.cap) return fail(PIC_ERR_CAPACITY, "more particles than max_particles");
  std::vector<double> x(n), y(n), z(n), vx(n), vy(n), vz(n);
  std::vector<float> vxf, vyf, vzf;
  std::vector<int> el(n);
  std::vector<uint8_t> sp(n), fl(n);
  for (int i = 0; i < n; ++i) {
    const double* s = ps + (size_t)i * 6;
    x[i] = s[0]; y[i] = s[1]; z[i] = s[2]; vx[i] = s[3]; vy[i] = s[4]; vz[i] = s[5];
    const bool in = inside ? inside[i] != 0 : true;
    if (in && (elem[i] < 1 || elem[i] > c->ne)) return fail(PIC_ERR_INVALID_ARGUMENT, "element id out of range");
    if (species[i] < 1 || species[i] > c->cfg.n_species) return fail(PIC_ERR_INVALID_ARGUMENT, "species id out of range");
    bool finite = std::isfinite(s[0]) && std::isfinite(s[1]) && std::isfinite(s[2]) && std::isfinite(s[3]) &&
                  std::isfinite(s[4]) && std::isfinite(s[5]);
    if (in && !finite) return fail(PIC_ERR_INVALID_ARGUMENT, "non-finite particle state");
    el[i] = in ? elem[i] - 1 : 0;
    sp[i] = (uint8_t)(species[i] - 1);
    fl[i] = (uint8_t)((in ? kInside : 0) | ((is_new ? is_new[i] != 0 : false) ? kNew : 0));
  }
  cudaStream_t s = c->stream;
  const size_t bd = sizeof(double) * (size_t)n;
  CUDA_TRY(cudaMemcpyAsync(c->P.x, x.data(), bd, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(c->P.y, y.data(), bd, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(c->P.z, z.data(), bd, cudaMemcpyHostToDevice, s));
  if (c->mixed) {
    vxf.assign(vx.begin(), vx.end()); vyf.assign(vy.begin(), vy.end()); vzf.assign(vz.begin(), vz.end());
    CUDA_TRY(cudaMemcpyAsync(c->P.vxf, vxf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->P.vyf, vyf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->P.vzf, vzf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
  } else {
    CUDA_TRY(cudaMemcpyAsync(c->P.vx, vx.data(), bd, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->P.vy, vy.data(), bd, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->P.vz, vz.data(), bd, cudaMemcpyHostToDevice, s));
  }
  CUDA_TRY(cudaMemcpyAsync(c->P.elem, el.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(c->P.last_elem, el.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(c->P.species, sp.data(), n, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(c->P.flags, fl.data(), n, cudaMemcpyHostToDevice, s));
  c->P.n = n;
  c->Q.n = n;
  if (n > 0) k_iota<<<(n + 255) / 256, 256, 0, s>>>(c->perm, n);
  LaunchArgs A = c->args();
  if (c->refmap) launch_map_particles(A, c->P);       // PartPosRef at insertion
  // group by element
  launch_reorder(A, c->P, c->Q, c->perm, c->perm_tmp, c->sortb);
  std::swap(c->P.x, c->Q.x); std::swap(c->P.y, c->Q.y); std::swap(c->P.z, c->Q.z);
  std::swap(c->P.vx, c->Q.vx); std::swap(c->P.vy, c->Q.vy); std::swap(c->P.vz, c->Q.vz);
  std::swap(c->P.vxf, c->Q.vxf); std::swap(c->P.vyf, c->Q.vyf); std::swap(c->P.vzf, c->Q.vzf);
  std::swap(c->P.xi0, c->Q.xi0); std::swap(c->P.xi1, c->Q.xi1); std::swap(c->P.xi2, c->Q.xi2);
  std::swap(c->P.elem, c->Q.elem); std::swap(c->P.last_elem, c->Q.last_elem);
  std::swap(c->P.species, c->Q.species); std::swap(c->P.flags, c->Q.flags);
  std::swap(c->perm, c->perm_tmp);
  int rc = device_sync(c);
  if (rc) return rc;
  c->have_particles = true;
  return PIC_OK;
}

static void swap_sorted(pic_ctx* c) {
  std::swap(c->P.x, c->Q.x); std::swap(c->P.y, c->Q.y); std::swap(c->P.z, c->Q.z);
  std::swap(c->P.vx, c->Q.vx); std::swap(c->P.vy, c->Q.vy); std::swap(c->P.vz, c->Q.vz);
  std::swap(c->P.vxf, c->Q.vxf); std::swap(c->P.vyf, c->Q.vyf); std::swap(c->P.vzf, c->Q.vzf);
  std::swap(c->P.xi0, c->Q.xi0); std::swap(c->P.xi1, c->Q.xi1); std::swap(c->P.xi2, c->Q.xi2);
  std::swap(c->P.elem, c->Q.elem); std::swap(c->P.last_elem, c->Q.last_elem);
  std::swap(c->P.species, c->Q.species); std::swap(c->P.flags, c->Q.flags);
  std::swap(c->perm, c->perm_tmp);
}

int pic_download_particles(pic_ctx_t* c, double* ps, int32_t* elem, uint8_t* inside, uint8_t* is_new,
                           double* part_pos_ref, int32_t n) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (n != c->P.n) return fail(PIC_ERR_INVALID_ARGUMENT, "n does not match the uploaded particle count");
  int rc = device_sync(c);
  if (rc) return rc;
  std::vector<double> x(n), y(n), z(n), vx(n), vy(n), vz(n), a(n), b(n), d(n);
  std::vector<float> vf(n);
  std::vector<int> el(n), pm(n);
  std::vector<uint8_t> fl(n);
  const size_t bd = sizeof(double) * (size_t)n;
  if (n > 0) {
    CUDA_TRY(cudaMemcpy(x.data(), c->P.x, bd, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(y.data(), c->P.y, bd, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(z.data(), c->P.z, bd, cudaMemcpyDeviceToHost));
    if (c->mixed) {
      CUDA_TRY(cudaMemcpy(vf.data(), c->P.vxf, sizeof(float) * n, cudaMemcpyDeviceToHost));
      for (int i = 0; i < n; ++i) vx[i] = vf[i];
      CUDA_TRY(cudaMemcpy(vf.data(), c->P.vyf, sizeof(float) * n, cudaMemcpyDeviceToHost));
      for (int i = 0; i < n; ++i) vy[i] = vf[i];
      CUDA_TRY(cudaMemcpy(vf.data(), c->P.vzf, sizeof(float) * n, cudaMemcpyDeviceToHost));
      for (int i = 0; i < n; ++i) vz[i] = vf[i];
    } else {
      CUDA_TRY(cudaMemcpy(vx.data(), c->P.vx, bd, cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(vy.data(), c->P.vy, bd, cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(vz.data(), c->P.vz, bd, cudaMemcpyDeviceToHost));
    }
    CUDA_TRY(cudaMemcpy(el.data(), c->P.elem, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(fl.data(), c->P.flags, n, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(pm.data(), c->perm, sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (part_pos_ref) {
      CUDA_TRY(cudaMemcpy(a.data(), c->P.xi0, bd, cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(b.data(), c->P.xi1, bd, cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(d.data(), c->P.xi2, bd, cudaMemcpyDeviceToHost));
    }
  }
  for (int j = 0; j < n; ++j) {
    const int i = pm[j];
    if (i < 0 || i >= n) return fail(PIC_ERR_STATE, "corrupt particle permutation");
    if (ps) {
      double* s = ps + (size_t)i * 6;
      s[0] = x[j]; s[1] = y[j]; s[2] = z[j]; s[3] = vx[j]; s[4] = vy[j]; s[5] = vz[j];
    }
    if (elem) elem[i] = el[j] + 1;
    if (inside) inside[i] = (fl[j] & kInside) ? 1 : 0;
    if (is_new) is_new[i] = (fl[j] & kNew) ? 1 : 0;
    if (part_pos_ref) { part_pos_ref[(size_t)i * 3] = a[j]; part_pos_ref[(size_t)i * 3 + 1] = b[j]; part_pos_ref[(size_t)i * 3 + 2] = d[j]; }
  }
  return PIC_OK;
}

int pic_interpolate(pic_ctx_t* c) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (!c->field_set || !c->have_particles) return fail(PIC_ERR_STATE, "field and particles must be set first");
  c->launches += launch_interpolate(c->args(), c->P, c->refmap, !c->sf);
  CUDA_TRY(cudaGetLastError());
  return PIC_OK;
}

int pic_push(pic_ctx_t* c, double dt) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (!c->have_particles) return fail(PIC_ERR_STATE, "particles must be uploaded first");
  c->launches += launch_push(c->args(), c->P, dt);
  CUDA_TRY(cudaGetLastError());
  return PIC_OK;
}

int pic_track(pic_ctx_t* c) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (!c->have_particles) return fail(PIC_ERR_STATE, "particles must be uploaded first");
  c->launches += launch_track(c->args(), c->P, c->refmap);
  CUDA_TRY(cudaGetLastError());
  return PIC_OK;
}

enum { PH_MAIN = 0, PH_PACK = 1, PH_PARTICLE = 2, PH_NODE2DOF = 3, PH_REORDER = 4, PH_OTHER = 5, PH_HDG = 6 };

static int deposit_device(pic_ctx* c) {
  const LaunchArgs A = c->args();
  if (c->sf) {
    c->phase(PH_PACK, [&] { return launch_sf_pack(A, c->P, c->sortb, c->sfl, c->sfk); });
    if (c->cc) c->phase(PH_MAIN, [&] { return launch_sf_cc_norm(A, c->sortb, c->sfl, c->sfk); });
    c->phase(PH_MAIN, [&] { return launch_sf_gather(A, c->sortb, c->sfl, c->sfk, c->PS); });
  } else {
    c->phase(PH_OTHER, [&] { return launch_deposit_cvwm(A, c->P, c->PS); });
  }
  c->ps_valid = true;
  return PIC_OK;
}

int pic_deposit(pic_ctx_t* c, double* part_source) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (!c->have_particles) return fail(PIC_ERR_STATE, "particles must be uploaded first");
  deposit_device(c);
  CUDA_TRY(cudaGetLastError());
  if (part_source) {
    CUDA_TRY(cudaMemcpyAsync(part_source, c->PS, sizeof(double) * c->ndofs * 4, cudaMemcpyDeviceToHost,
                             c->stream));
    return device_sync(c);
  }
  return PIC_OK;
}

int pic_get_part_data(pic_ctx_t* c, double* part_data, int64_t* part_int, int64_t offset_npart, int32_t capacity,
                      int32_t* n_out) {
  if (!c || !part_int || !n_out) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  const int n = c->P.n, ne = c->ne;
  std::vector<double> ps((size_t)n * 6);
  std::vector<int32_t> el(n);
  std::vector<uint8_t> ins(n), sp(n);
  std::vector<int> pm(n);
  int rc = pic_download_particles(c, ps.data(), el.data(), ins.data(), nullptr, nullptr, n);
  if (rc) return rc;
  if (n > 0) {
    CUDA_TRY(cudaMemcpy(sp.data(), c->P.species, n, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(pm.data(), c->perm, sizeof(int) * n, cudaMemcpyDeviceToHost));
  }
  std::vector<int> spc(n, 0);
  for (int j = 0; j < n; ++j) spc[pm[j]] = sp[j] + 1;
  // stable counting sort by element: ascending caller index within an element
  std::vector<int64_t> first(ne + 1, 0);
  for (int i = 0; i < n; ++i)
    if (ins[i]) first[el[i]]++;                       // el is 1-based: counts land in first[1..ne]
  for (int e = 0; e < ne; ++e) first[e + 1] += first[e];
  const int64_t total = first[ne];
  *n_out = (int32_t)total;
  for (int e = 0; e < ne; ++e) {
    part_int[2 * (size_t)e] = offset_npart + first[e];
    part_int[2 * (size_t)e + 1] = offset_npart + first[e + 1];
  }
  if (!part_data) return PIC_OK;
  if (total > capacity) return fail(PIC_ERR_CAPACITY, "part_data holds fewer particles than are inside");
  std::vector<int64_t> cur(first.begin(), first.end() - 1);
  for (int i = 0; i < n; ++i) {
    if (!ins[i]) continue;
    double* d = part_data + 7 * (size_t)cur[el[i] - 1]++;
    for (int q = 0; q < 6; ++q) d[q] = ps[(size_t)i * 6 + q];
    d[6] = (double)spc[i];
  }
  return PIC_OK;
}

int pic_set_part_data(pic_ctx_t* c, const double* part_data, const int64_t* part_int, int64_t offset_npart,
                      int32_t n_part) {
  if (!c || !part_int || (n_part > 0 && !part_data)) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (n_part < 0) return fail(PIC_ERR_INVALID_ARGUMENT, "negative particle count");
  std::vector<double> ps((size_t)n_part * 6);
  std::vector<int32_t> el(n_part, 0), spc(n_part, 0);
  for (int e = 0; e < c->ne; ++e) {
    const int64_t a = part_int[2 * (size_t)e] - offset_npart, b = part_int[2 * (size_t)e + 1] - offset_npart;
    if (a < 0 || b < a || b > n_part) return fail(PIC_ERR_INVALID_ARGUMENT, "part_int range outside part_data");
    for (int64_t k = a; k < b; ++k) {
      if (el[k] != 0) return fail(PIC_ERR_INVALID_ARGUMENT, "part_int ranges overlap");
      el[k] = e + 1;
    }
  }
  for (int k = 0; k < n_part; ++k) {
    if (el[k] == 0) return fail(PIC_ERR_INVALID_ARGUMENT, "particle outside every part_int range");
    const double* d = part_data + 7 * (size_t)k;
    for (int q = 0; q < 6; ++q) ps[(size_t)k * 6 + q] = d[q];
    spc[k] = (int32_t)d[6];
    if ((double)spc[k] != d[6]) return fail(PIC_ERR_INVALID_ARGUMENT, "species column is not an integer");
  }
  std::vector<uint8_t> inside(n_part, 1), is_new(n_part, 0);
  return pic_upload_particles(c, ps.data(), el.data(), spc.data(), inside.data(), is_new.data(), n_part);
}

int pic_get_field_at_particles(pic_ctx_t* c, double* field, int32_t n) {
  if (!c || !field) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (n != c->P.n) return fail(PIC_ERR_INVALID_ARGUMENT, "n does not match the particle count");
  int rc = device_sync(c);
  if (rc) return rc;
  std::vector<double> f((size_t)6 * c->P.cap);
  std::vector<int> pm(n);
  if (n > 0) {
    CUDA_TRY(cudaMemcpy(f.data(), c->P.field, sizeof(double) * 6 * (size_t)c->P.cap, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(pm.data(), c->perm, sizeof(int) * n, cudaMemcpyDeviceToHost));
  }
  for (int j = 0; j < n; ++j)
    for (int q = 0; q < 6; ++q) field[(size_t)pm[j] * 6 + q] = f[(size_t)q * c->P.cap + j];
  return PIC_OK;
}

int pic_step(pic_ctx_t* c, double dt, int32_t nsteps, double* part_source) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (nsteps < 0) return fail(PIC_ERR_INVALID_ARGUMENT, "nsteps < 0");
  const bool solve = hdg_solve_in_step(c);
  if (!(c->field_set || solve) || !c->have_particles) return fail(PIC_ERR_STATE, "field and particles must be set first");
  const int sort_every = c->cfg.sort_interval;
  for (int it = 0; it < nsteps; ++it) {
    LaunchArgs A = c->args();
    if (sort_every > 0 && c->n_steps > 0 && (c->n_steps % sort_every) == 0) {
      c->phase(PH_REORDER, [&] { return launch_reorder(A, c->P, c->Q, c->perm, c->perm_tmp, c->sortb); });
      swap_sorted(c);
      A = c->args();
    }
    if (!c->sf && !c->refmap && !solve) {
      // Deposition + InterpolateFieldToParticle + push + TriaTracking in one kernel, then node -> DOF
      c->phase(PH_MAIN, [&] { return launch_cvwm_fused(A, c->P, dt); });
      c->phase(PH_NODE2DOF, [&] { return launch_node_to_dof(A, c->PS); });
      c->ps_valid = true;
    } else {
      deposit_device(c);                                  // Deposition on x_n
      if (solve) {                                        // HDG(): the field of rho_n
        int rc = PIC_OK;
        c->phase(PH_HDG, [&] { rc = hdg_solve_device(c, c->PS, nullptr); return 0; });
        if (rc) return rc;
      }
      if (c->refmap) {
        c->phase(PH_PARTICLE, [&] { return launch_step_ref(A, c->P, dt); });   // interpolation + push + RefTracking
      } else {
        c->phase(PH_PARTICLE, [&] {
          return launch_interpolate(A, c->P, false, !c->sf) + launch_push(A, c->P, dt) + launch_track(A, c->P, false);
        });
      }
    }
    c->n_steps++;
  }
  CUDA_TRY(cudaGetLastError());
  if (part_source) {
    CUDA_TRY(cudaMemcpyAsync(part_source, c->PS, sizeof(double) * c->ndofs * 4, cudaMemcpyDeviceToHost,
                             c->stream));
    return device_sync(c);
  }
  return PIC_OK;
}

int pic_fp64_fma_rate(pic_ctx_t* c, double* gflops) {
  if (!c || !gflops) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* sink = nullptr;
  int rc = c->alloc(&sink, (size_t)sms * 8);
  if (rc) return rc;
  *gflops = pic::fp64_fma_rate(c->stream, sink, sms);
  CUDA_TRY(cudaGetLastError());
  return PIC_OK;
}

int pic_fp32_fma_rate(pic_ctx_t* c, double* gflops) {
  if (!c || !gflops) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  float* sink = nullptr;
  int rc = c->alloc(&sink, (size_t)sms * 8);
  if (rc) return rc;
  *gflops = pic::fp32_fma_rate(c->stream, sink, sms);
  CUDA_TRY(cudaGetLastError());
  return PIC_OK;
}

int pic_get_status(pic_ctx_t* c, pic_status_t* out) {
  if (!c || !out) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  launch_count_inside(c->args(), c->P, c->d_count);
  int rc = device_sync(c);
  if (rc) return rc;
  DevStatus s{};
  int cnt = 0;
  CUDA_TRY(cudaMemcpy(&s, c->st, sizeof(DevStatus), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(&cnt, c->d_count, sizeof(int), cudaMemcpyDeviceToHost));
  out->error_word = s.error_word;
  out->n_lost = s.n_lost;
  out->n_inside = cnt;
  out->n_newton_failed = s.n_newton_failed;
  out->n_steps = c->n_steps;
  return PIC_OK;
}

int pic_verify_deposited_charge(pic_ctx_t* c, double* charge_numerical, double* charge_analytical) {
  if (!c || !charge_numerical || !charge_analytical) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  if (!c->charge_w) return fail(PIC_ERR_STATE, "the charge check needs pic_mesh_t.elem_sj at pic_create");
  if (!c->ps_valid) return fail(PIC_ERR_STATE, "no deposition to check: call pic_deposit or pic_step first");
  if (!c->have_particles) return fail(PIC_ERR_STATE, "particles must be uploaded first");
  launch_charge_integral(c->args(), c->PS, c->charge_w, c->charge_elem, c->charge_out);
  launch_count_species(c->args(), c->P, c->species_count);
  double num = 0.0;
  int cnt[PIC_MAX_SPECIES] = {0};
  CUDA_TRY(cudaMemcpyAsync(&num, c->charge_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(cnt, c->species_count, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  int rc = device_sync(c);
  if (rc) return rc;
  double ana = 0.0;   // ChargeAnalytical: sum over particles inside of ChargeIC * MacroParticleFactor
  for (int s = 0; s < c->cfg.n_species; ++s) ana = ana + (double)cnt[s] * (c->cfg.charge[s] * c->cfg.mpf[s]);
  *charge_numerical = num;
  *charge_analytical = ana * c->charge_dim_factor;
  return PIC_OK;
}

int pic_reset_status(pic_ctx_t* c) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  CUDA_TRY(cudaMemsetAsync(c->st, 0, sizeof(DevStatus), c->stream));
  return device_sync(c);
}

int pic_synchronize(pic_ctx_t* c) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  return device_sync(c);
}

int pic_profile(pic_ctx_t* c, int32_t enable) {
  if (!c) return fail(PIC_ERR_INVALID_ARGUMENT, "null context");
  int rc = device_sync(c);
  if (rc) return rc;
  c->collect();
  for (int q = 0; q < 8; ++q) { c->prof_ms[q] = 0.0; c->prof_launches[q] = 0; }
  c->prof = enable != 0;
  return PIC_OK;
}

int pic_profile_read(pic_ctx_t* c, double* ms, int64_t* launches, int32_t nphase) {
  if (!c || !ms || !launches || nphase < 1) return fail(PIC_ERR_INVALID_ARGUMENT, "null argument");
  int rc = device_sync(c);
  if (rc) return rc;
  c->collect();
  for (int q = 0; q < nphase && q < 8; ++q) { ms[q] = c->prof_ms[q]; launches[q] = c->prof_launches[q]; }
  return PIC_OK;
}

// number of kernels launched through this context (for the benchmark's launch count)
int64_t pic_launch_count(pic_ctx_t* c) { return c ? c->launches : 0; }

// the context's CUDA stream (for event timing by a caller that shares the device)
void* pic_stream(pic_ctx_t* c) { return c ? (void*)c->stream : nullptr; }

}  // extern "C"
