// libbasefold_gpu.so: multilinear evaluation without any allocation.
//
// bf_eval needs scratch for the chain of variable fixings and takes it from
// device memory it allocates.  Some callers cannot allocate at that point:
// a proving service that has carved all device memory into fixed per-request
// slots for admission control (an extra cudaMalloc would fail or break its
// accounting), or a latency-critical loop where cudaMalloc/cudaFree would
// synchronise the device.  bf_eval_noalloc gives them the same evaluation
// with the scratch in a fixed array that lives in the library's device image.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "api_common.h"

using namespace bfapi;

namespace {

// Largest evaluation this entry point handles: 2^(num_vars-1) scratch
// elements, num_vars <= kNoAllocMaxVars.  The array (1 MiB) is part of the
// library's device image: every GPU that loads the library holds it until the
// process exits.
constexpr int kNoAllocMaxVars = 17;
constexpr size_t kNoAllocScratchElems = (size_t)1 << (kNoAllocMaxVars - 1);

// Fixed scratch shared by every call on a device; it keeps whatever the last
// call left.  Calls whose GPU work overlaps (different streams, or different
// host threads without ordering) race on it.
static __device__ __align__(256) uint4 g_noalloc_scratch[kNoAllocScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
uint4* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (in host code
// the array's name is only a host-side stand-in, never a device address).
// Looked up once per device, with that device current, by the first call
// made on it; make that first call before any stream capture.  The address
// is kept for the life of the process: resetting the device
// (cudaDeviceReset) after the first call is not supported, since the
// reloaded module may place the array elsewhere.
int scratch_for_current_device(uint4** out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(BF_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(BF_ERR_CUDA, "cudaGetSymbolAddress(noalloc scratch) on device %d: %s", dev, cudaGetErrorString(e));
    g_scratch_ptr[dev] = reinterpret_cast<uint4*>(p);
  }
  *out = g_scratch_ptr[dev];
  return BF_OK;
}

}  // namespace

extern "C" int bf_eval_noalloc(const void* d_evals, int num_vars, const uint8_t* point, void* d_value, void* stream) {
  if (!d_evals || !d_value || (num_vars > 0 && !point)) return fail(BF_ERR_ARG, "null argument");
  if (num_vars < 0) return fail(BF_ERR_ARG, "num_vars must be >= 0");
  if (num_vars > kNoAllocMaxVars)
    return fail(BF_ERR_ARG,
                "num_vars %d exceeds the fixed scratch of bf_eval_noalloc (at most %d variables, %zu elements); "
                "use bf_eval",
                num_vars, kNoAllocMaxVars, kNoAllocScratchElems);
  if ((reinterpret_cast<uintptr_t>(d_evals) | reinterpret_cast<uintptr_t>(d_value)) & 15)
    return fail(BF_ERR_ARG, "device pointers must be 16-byte aligned");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (num_vars == 0) {
    CU(cudaMemcpyAsync(d_value, d_evals, 16, cudaMemcpyDeviceToDevice, st));
    return BF_OK;
  }
  uint4* scratch = nullptr;
  TRY(scratch_for_current_device(&scratch));
  // MultiPoly::evaluate (multilinear.rs:124-141): fix the top variable with
  // the last coordinate, repeatedly — the large levels one launch each, the
  // last (at most kEvalTailMaxVars) in one block, as bf_eval does.  Every
  // level writes the entries the next one reads, so nothing in the scratch
  // needs clearing between calls.
  auto coord = [&](int k) {
    uint4 r;
    std::memcpy(&r, point + 16 * k, 16);
    return r;
  };
  const int tail = num_vars - 1 < bf::kEvalTailMaxVars ? num_vars - 1 : bf::kEvalTailMaxVars;
  CU(bf::launch_fix(reinterpret_cast<const uint4*>(d_evals), scratch, (size_t)1 << (num_vars - 1),
                    coord(num_vars - 1), nullptr, 0, nullptr, st));
  for (int k = num_vars - 2; k >= tail; --k)
    CU(bf::launch_fix(scratch, scratch, (size_t)1 << k, coord(k), nullptr, 0, nullptr, st));
  if (tail > 0) {
    bf::EvalTail et{};
    et.nvars = tail;
    et.rp = nullptr;
    for (int k = 0; k < tail; ++k) et.r[k] = coord(k);
    CU(bf::launch_eval_tail(scratch, et, st));
  }
  CU(cudaMemcpyAsync(d_value, scratch, 16, cudaMemcpyDeviceToDevice, st));
  return BF_OK;
}
