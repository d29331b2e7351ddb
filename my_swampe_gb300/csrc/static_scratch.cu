// Allocation-free variant of swp_adjoint_step.
//
// swp_adjoint_step needs a scratch buffer (lam_y: the adjoint of the step's
// Fourier outputs, written by the grid adjoint kernel and read by the
// spectral adjoint kernel) that the caller allocates.  Some callers cannot
// allocate device memory at the point where they run the adjoint: code that
// executes inside another framework's custom-call or callback (for example an
// XLA/JAX custom call or a plugin invoked from a host callback), where the
// host framework owns the allocator and forbids cudaMalloc/cudaFree; code
// running inside a real-time or hard-latency loop where a synchronising
// cudaMalloc/cudaFree is not acceptable; and embedded callers that link the C
// ABI without any memory manager.  For them swp_adjoint_step_noalloc keeps
// that scratch in a fixed, file-scope device array instead.
#include <mutex>
#include "swp_internal.h"

namespace swp {
int adjoint_step_dispatch(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                          const swp_group_adjoint* adj, const swp_flags* f, int t, cudaStream_t s);
int plan_groups(const swp_plan* p);
size_t plan_lamy_bytes(const swp_plan* p, int g);
int plan_fail(swp_plan* p, int code, const char* msg);
int adjoint_step_checks(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                        const swp_group_adjoint* adj, const swp_flags* f, bool need_lamy);
}  // namespace swp

// Every device that loads this library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_swp_adjoint_scratch[SWP_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device, resolved once
// per device (the name is only a host-side stand-in for the device symbol).
// The cache is never invalidated: after cudaDeviceReset the library's module
// is loaded anew and the cached address may be stale, so resetting a device
// after the first call on it is not supported.
int scratch_address(void** out, std::string& err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return SWP_ERR_CUDA; }
  if (dev < 0 || dev >= kMaxDevices) { err = "device ordinal out of range"; return SWP_ERR_ARG; }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_swp_adjoint_scratch);
    if (e != cudaSuccess || !ptr) {
      err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
      return SWP_ERR_CUDA;
    }
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return SWP_OK;
}
}  // namespace

extern "C" int swp_adjoint_step_noalloc(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                                        const swp_group_adjoint* adj, const swp_flags* f, int t, void* stream) {
  using namespace swp;
  // the same argument checks as swp_adjoint_step, except that lam_y is not the caller's
  if (int rc = adjoint_step_checks(p, st_in, st_out, adj, f, false)) return rc;
  int ng = plan_groups(p);
  // lam_y of every group is carved out of the static array, 256-byte aligned
  size_t need = 0;
  size_t off[SWP_MAX_GROUPS] = {};
  for (int g = 0; g < ng; ++g) {
    off[g] = need;
    need += (plan_lamy_bytes(p, g) + 255) / 256 * 256;
  }
  if (need > (size_t)SWP_NOALLOC_SCRATCH_BYTES) {
    return plan_fail(p, SWP_ERR_ARG,
                     "swp_adjoint_step_noalloc: the plan needs more scratch than SWP_NOALLOC_SCRATCH_BYTES "
                     "(5*(M+1)*B*J complex values per group); use swp_adjoint_step with a caller buffer");
  }
  void* base = nullptr;
  std::string err;
  int rc = scratch_address(&base, err);
  if (rc != SWP_OK) return plan_fail(p, rc, err.c_str());
  swp_group_adjoint a[SWP_MAX_GROUPS];
  for (int g = 0; g < ng; ++g) {
    a[g] = adj[g];
    a[g].lam_y = (char*)base + off[g];
  }
  return adjoint_step_dispatch(p, st_in, st_out, a, f, t, (cudaStream_t)stream);
}
