// fo_solve_static: the integrator without a caller-provided workspace and
// without any device allocation.
//
// Some callers cannot allocate device memory when they integrate: an
// atmospheric model that hands the whole device to its own memory pool at
// start-up and forbids allocations afterwards, or a model time step on a path
// where the implicit device-wide synchronization of cudaMalloc/cudaFree is not
// acceptable. For them this entry point takes its scratch from one
// file-scope device array of FO_STATIC_SCRATCH_BYTES, which every GPU that
// loads the library holds until the process exits.
//
// The array's name is only a host-side stand-in in host code: its device
// address is obtained once per device with cudaGetSymbolAddress, on the first
// call made while that device is current, and passed to the kernel. That
// first call should therefore be made before any stream capture begins. The
// address is kept for the life of the process: after cudaDeviceReset, which
// destroys the primary context and with it the module, the array may move, so
// the entry point must not be used again in that process.
//
// All calls share the one array and it keeps the last call's contents; the
// only state that must start at zero, the queue counter of the persistent
// launch, is cleared by every call. Calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on the array: order
// them on one stream.
#include <cuda_runtime.h>

#include <mutex>

#include "fastode_gb300.h"

// The scratch: the queue counter at offset 0, then as many group slots as fit.
static __device__ __align__(256) unsigned char g_static_scratch[FO_STATIC_SCRATCH_BYTES];

namespace fo {
int set_last_error(int code, const char* what);  // abi.cu
}  // namespace fo

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_address[kMaxDevices] = {};

// The device address of the scratch on the current device (looked up once).
int static_scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fo::set_last_error(FO_E_CUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= kMaxDevices) return fo::set_last_error(FO_E_UNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (g_address[dev] == nullptr) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (e != cudaSuccess || ptr == nullptr)
      return fo::set_last_error(FO_E_CUDA, "cudaGetSymbolAddress of the static scratch failed");
    g_address[dev] = ptr;
  }
  *out = g_address[dev];
  return FO_OK;
}

}  // namespace

extern "C" int fo_solve_static(const fo_plan* plan, const fo_options* opt, int32_t ngroups,
                               const int32_t* group_offsets, int32_t max_group_cells, double* Y,
                               int64_t y_cell_stride, int64_t y_species_stride, const double* k,
                               int64_t k_cell_stride, int64_t k_reaction_stride, const double* atol, double rtol,
                               double dt, double* memory, int64_t* counts, int32_t* status, void* stream) {
  if (!plan || ngroups < 0 || max_group_cells <= 0)
    return fo::set_last_error(FO_E_INVALID, "null plan or bad group sizes");
  if (ngroups == 0) return FO_OK;
  // slots of the static scratch: one group in flight per slot
  size_t one = 0;
  int rc = fo_workspace_bytes(plan, 1, max_group_cells, &one);
  if (rc != FO_OK) return rc;
  size_t two = 0;
  rc = fo_workspace_bytes(plan, 2, max_group_cells, &two);
  if (rc != FO_OK) return rc;
  const size_t slot = two - one, header = one - slot;
  if (one > (size_t)FO_STATIC_SCRATCH_BYTES)
    return fo::set_last_error(FO_E_UNSUPPORTED,
                              "one group of this mechanism needs more scratch than the static "
                              "FO_STATIC_SCRATCH_BYTES array holds: use fo_solve with a workspace");
  size_t fit = ((size_t)FO_STATIC_SCRATCH_BYTES - header) / slot;
  const int32_t slots = (int32_t)(fit < (size_t)ngroups ? fit : (size_t)ngroups);
  void* scratch = nullptr;
  rc = static_scratch_address(&scratch);
  if (rc != FO_OK) return rc;
  return fo_solve(plan, opt, ngroups, group_offsets, max_group_cells, Y, y_cell_stride, y_species_stride, k,
                  k_cell_stride, k_reaction_stride, atol, rtol, dt, memory, counts, status, scratch,
                  (size_t)FO_STATIC_SCRATCH_BYTES, slots, nullptr, 0, nullptr, stream);
}
