// pic_noalloc.cu -- cell_volweight_mean deposition that makes no device allocation.
//
// Who needs it: a host that cannot call cudaMalloc while its time loop runs -- for example a
// Fortran code whose device memory belongs to another runtime or to a fixed pool, or a loop that
// runs under a hard device-memory budget.  Such a caller keeps the particles and PartSource in
// its own device arrays and passes them in; the only scratch the deposition needs (the CVWM node
// sums) lives in the fixed-size file-scope device array below instead of a cudaMalloc'ed buffer.
//
// Limits and rules of use:
//   * at most kNoallocMaxNodes periodic-unique mesh nodes (131072 nodes, 4 MiB of FP64 sums);
//     larger meshes are rejected with PIC_ERR_CAPACITY;
//   * the array exists once per GPU that loads the library and stays allocated until the process
//     exits; every call shares it and it keeps the last call's contents (each call clears the part
//     it uses before depositing);
//   * calls that overlap on the GPU (different streams, or different host threads) race on the
//     array: order them on one stream or serialise them;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current; make that first call before any stream capture;
//   * particles whose ParticleInside flag is 0 (optional mask) are skipped; element or species ids out
//     of range skip the particle and set PIC_STATUS_BAD_ELEMENT, which pic_get_status reports (the
//     context's stream waits for the call).
#include "pic_ctx.h"

#include <mutex>

using namespace pic;

namespace {

constexpr int kNoallocMaxNodes = 1 << 17;
constexpr int kMaxDevices = 64;

// node sums [node][4], FP64
static __device__ __align__(256) double g_node_scratch[(size_t)kNoallocMaxNodes * 4];

// device address of g_node_scratch, per device ordinal (filled by the set-up below)
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

int scratch_for_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return pic_internal::set_error(PIC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_node_scratch);
    if (e != cudaSuccess || !p)
      return pic_internal::set_error(PIC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return PIC_OK;
}

// Same corner scatter as the context's FP64 CVWM kernel, reading the caller's PartState(1:6,n),
// 1-based element / species ids and (optionally) PDM%ParticleInside straight from device memory.
// Particles with ParticleInside = .FALSE. are skipped before their element is read, as the reference
// skips them (pic_depo_method.f90:472): a removed particle keeps a stale element id.
__global__ void __launch_bounds__(256) k_noalloc_cvwm(const __grid_constant__ DevMesh M, const double* __restrict__ ps,
                                                      const int32_t* __restrict__ elem1,
                                                      const int32_t* __restrict__ spec1,
                                                      const uint8_t* __restrict__ inside, int n,
                                                      double* __restrict__ NS, DevStatus* st) {
  const Consts& kc = M.k;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n && (inside == nullptr || inside[i] != 0);
  int e = valid ? elem1[i] - 1 : 0;
  int sp = valid ? spec1[i] - 1 : 0;
  if (valid && (e < 0 || e >= M.ne || sp < 0 || sp >= kc.n_species)) {
    flag_status(st, 0x10u);            // PIC_STATUS_BAD_ELEMENT: skipped, nothing read out of range
    valid = false;
  }
  if (!valid) { e = 0; sp = 0; }
  const bool charged = valid && (kc.q[sp] != 0.0);
  double contrib[32];
  if (charged) {
    const double* s = ps + (size_t)i * 6;
    const double x[3] = {s[0], s[1], s[2]};
    double xi[3];
    const bool suc = position_in_ref_elem(M, e, x, xi);
    if (!suc) flag_status(st, 0x02u);
    const double ch = kc.qm[sp];
    const double TS[4] = {s[3] * ch, s[4] * ch, s[5] * ch, ch};
    cvwm_contrib(M, e, suc, xi, x, TS, contrib);
  }
  cvwm_scatter(M, charged, e, contrib, NS);
}

}  // namespace

extern "C" int pic_deposit_cvwm_noalloc(pic_ctx_t* ctx, const double* d_part_state, const int32_t* d_elem,
                                        const int32_t* d_species, const uint8_t* d_inside, int32_t n,
                                        double* d_part_source, void* stream) {
  if (!ctx) return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "null context");
  if (ctx->cfg.deposition != PIC_DEPO_CVWM)
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "the allocation-free deposition is cell_volweight_mean only");
  if (n < 0 || !d_part_source || (n > 0 && (!d_part_state || !d_elem || !d_species)))
    return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "null device pointer or negative particle count");
  if (ctx->n_canon > kNoallocMaxNodes)
    return pic_internal::set_error(PIC_ERR_CAPACITY,
                                   "mesh has " + std::to_string(ctx->n_canon) +
                                       " periodic-unique nodes; the allocation-free deposition holds at most " +
                                       std::to_string(kNoallocMaxNodes));
  double* NS = nullptr;
  int rc = scratch_for_current_device(&NS);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(NS, 0, sizeof(double) * 4 * (size_t)ctx->n_canon, s);
  if (e != cudaSuccess) return pic_internal::set_error(PIC_ERR_CUDA, std::string("set-up: ") + cudaGetErrorString(e));
  if (n > 0)
    k_noalloc_cvwm<<<(n + 255) / 256, 256, 0, s>>>(ctx->M, d_part_state, d_elem, d_species, d_inside, n, NS, ctx->st);
  const int tot = ctx->M.ne * ctx->nd;
  switch (ctx->var_n ? 0 : ctx->N) {
    case 0: k_node_to_dof<0><<<(tot + 255) / 256, 256, 0, s>>>(ctx->M, NS, d_part_source); break;   // p-adapted
    case 1: k_node_to_dof<1><<<(tot + 255) / 256, 256, 0, s>>>(ctx->M, NS, d_part_source); break;
    case 2: k_node_to_dof<2><<<(tot + 255) / 256, 256, 0, s>>>(ctx->M, NS, d_part_source); break;
    case 3: k_node_to_dof<3><<<(tot + 255) / 256, 256, 0, s>>>(ctx->M, NS, d_part_source); break;
    case 4: k_node_to_dof<4><<<(tot + 255) / 256, 256, 0, s>>>(ctx->M, NS, d_part_source); break;
    default: return pic_internal::set_error(PIC_ERR_INVALID_ARGUMENT, "unsupported N");
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return pic_internal::set_error(PIC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  // The kernels above set status bits (PIC_STATUS_BAD_ELEMENT, _NEWTON_FAILED) in the context's status word
  // from the caller's stream.  pic_get_status and pic_reset_status work on the context's own stream, so that
  // stream waits for this call (an event, no allocation): a later pic_get_status sees this call's bits.
  // While the caller's stream is being captured the wait is not added (it would pull the context's stream
  // into the capture); the caller then synchronises its stream before reading the status.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) {
    e = cudaEventRecord(ctx->noalloc_done, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->noalloc_done, 0);
    if (e != cudaSuccess) return pic_internal::set_error(PIC_ERR_CUDA, std::string("status ordering: ") + cudaGetErrorString(e));
  } else {
    (void)cudaGetLastError();
  }
  return PIC_OK;
}
