// spmm_static.cu — smat_spmm_static_scratch: the SpMM with its packed-B
// scratch in a fixed, file-scope device array instead of caller-provided
// workspace.
//
// Some callers can neither allocate device memory nor hand in scratch:
// a launcher bound to a fixed signature that has no workspace parameter
// (such as the reference's HGEMM_FUNC_SPARSE2 launchers), or code running
// where allocating is not allowed — cudaMalloc can synchronise the device
// and stall every stream, and a service that budgets its memory at start-up
// may forbid allocations afterwards. This entry point serves them: it calls
// no cudaMalloc, cudaFree or allocating library routine. The scratch is
// g_spmm_scratch below, SMAT_SPMM_STATIC_SCRATCH_BYTES (32 MiB) per device,
// reserved when the library's device code is loaded on that device.
//
// Host code cannot use g_spmm_scratch as a pointer (on the host the name
// stands for the symbol, not a device address). The first call on each
// device therefore looks the address up with cudaGetSymbolAddress, with
// that device current, and keeps it for later calls on that device. Make
// that first call on each device before any stream capture begins. The
// address belongs to the device's primary context: every call compares that
// context's ID with the one the address was looked up in, and looks it up
// again when they differ (after cudaDeviceReset the module is loaded anew
// and the array can move), so such a call also belongs outside a capture.
//
// Every call on a device shares the one array and leaves its contents
// behind. The packed B is rewritten in full (padding included) by the pack
// kernel before the contraction reads it; the only part that must start at
// zero, the split-panel counters, is cleared by smat_spmm_packed on the
// call's stream before each contraction. Calls that overlap in time — on
// different streams, or from different threads — race on the array and
// corrupt each other's results.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "smat_internal.h"

namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint8_t g_spmm_scratch[SMAT_SPMM_STATIC_SCRATCH_BYTES];

std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // ID of the context the address belongs to

// Device address of g_spmm_scratch on `dev`, looked up in the device's
// current primary context (again whenever that context changed).
smat_status scratch_on(int dev, void** out) {
  if (dev < 0 || dev >= kMaxDevices) return smat::fail(SMAT_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return smat::fail(SMAT_ERR_CUDA, "cudaGetDevice failed");
  // cudaSetDevice binds the device's primary context to this thread (also
  // when dev is already current), so that the driver query below sees it
  if (cudaSetDevice(dev) != cudaSuccess) return smat::fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  smat_status st = SMAT_OK;
  using CtxGetCurrent = CUresult (*)(CUcontext*);
  using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
  static const auto get_current = reinterpret_cast<CtxGetCurrent>(smat::driver_fn("cuCtxGetCurrent"));
  static const auto get_id = reinterpret_cast<CtxGetId>(smat::driver_fn("cuCtxGetId"));
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) {
    st = smat::fail(SMAT_ERR_CUDA, "no current CUDA context for the static scratch");
  } else if (!g_scratch_addr[dev] || g_scratch_ctx[dev] != id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_spmm_scratch);
    if (e != cudaSuccess || !p) {
      st = smat::fail(SMAT_ERR_CUDA, std::string("cudaGetSymbolAddress(g_spmm_scratch): ") + cudaGetErrorString(e));
    } else {
      g_scratch_addr[dev] = p;
      g_scratch_ctx[dev] = id;
    }
  }
  if (prev != dev) cudaSetDevice(prev);
  if (st != SMAT_OK) return st;
  *out = g_scratch_addr[dev];
  return SMAT_OK;
}

}  // namespace

smat_status smat_spmm_static_scratch(const smat_bcsr* A, int32_t form, const void* B, int32_t b_dtype,
                                     int32_t b_layout, int64_t ldb, void* C, int32_t c_dtype, int64_t ldc,
                                     int64_t N, void* stream) {
  if (!A || !B || !C) return smat::fail(SMAT_ERR_INVALID, "null argument");
  size_t need = 0;
  smat_status st = smat_spmm_workspace_size(A, form, b_dtype, N, &need);
  if (st != SMAT_OK) return st;
  if (need > (size_t)SMAT_SPMM_STATIC_SCRATCH_BYTES)
    return smat::fail(SMAT_ERR_UNSUPPORTED,
                      "packed B needs " + std::to_string(need) + " bytes but the static scratch holds " +
                          std::to_string((size_t)SMAT_SPMM_STATIC_SCRATCH_BYTES) +
                          "; use smat_spmm with a caller-provided workspace");
  void* scratch = nullptr;
  st = scratch_on(smat::bcsr_device(A), &scratch);
  if (st != SMAT_OK) return st;
  return smat_spmm(A, form, B, b_dtype, b_layout, ldb, C, c_dtype, ldc, N, scratch,
                   (size_t)SMAT_SPMM_STATIC_SCRATCH_BYTES, stream);
}
