// eval_eq for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need this operation: host libraries
// that embed the prover behind an allocator they do not control, callers holding a fixed memory
// budget, or code that must not allocate at the call site. whir_eval_eq_noalloc takes only caller-owned device buffers and keeps its one piece of
// scratch (the two eq tables) in a file-scope device array, so it performs no allocation at all.
//
// The scratch array lives for as long as the library is loaded, on every device that loads it.
// Host code cannot use the array's name as a device address (in host code the symbol is only a
// host-side stand-in), so the device address is looked up with cudaGetSymbolAddress, with the
// device current (see scratch_address for when a call reuses an earlier lookup).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/whir_gb300.h"
#include "field.cuh"
#include "kernels.hpp"

namespace {

// Room for the hi and lo eq tables: 2^ceil(nvars/2) + 2^floor(nvars/2) elements.
constexpr size_t NOALLOC_SCRATCH_BYTES = 256 * 1024;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void* g_scratch_ptr[MAX_DEVICES] = {nullptr};
thread_local std::string g_err;

int fail(int code, const std::string& m) {
  g_err = m;
  return code;
}

// Device address of the scratch array on the current device. Looked up again on every call (the
// lookup is cheap, and a fresh one stays valid after a device reset or in a context other than the
// one of an earlier call), except while `stream` reports an active capture, when the address found
// by the last looking-up call on this device is reused.
int scratch_address(int device, cudaStream_t stream, void** out) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const cudaError_t qe = cudaStreamIsCapturing(stream, &cs);
  if (qe != cudaSuccess) cudaGetLastError();  // the query's error must not reach the launch check
  std::lock_guard<std::mutex> g(g_mu);
  if (qe == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(WHIR_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[device] = p;
  } else if (!g_scratch_ptr[device]) {
    return fail(WHIR_ERR_INVALID, "the first call on a device must be made outside a stream capture");
  }
  *out = g_scratch_ptr[device];
  return 0;
}

template <class T>
int run(uint64_t* acc, const uint64_t* point, size_t nvars, const uint64_t* scalar, cudaStream_t stream,
        void* scratch) {
  const size_t h = nvars / 2, l = nvars - h;
  const size_t need = ((size_t(1) << h) + (size_t(1) << l)) * sizeof(T);
  if (need > NOALLOC_SCRATCH_BYTES)
    return fail(WHIR_ERR_INVALID, "nvars too large for the no-allocation scratch (" + std::to_string(need) +
                                      " bytes needed, " + std::to_string(NOALLOC_SCRATCH_BYTES) + " available)");
  T s;
  for (int d = 0; d < T::LIMBS; ++d) {
    if (scalar[d] >= whir::GL_P) return fail(WHIR_ERR_INVALID, "non-canonical scalar");
    reinterpret_cast<uint64_t*>(&s)[d] = scalar[d];
  }
  cudaError_t e = whir::launch_eval_eq<T>(reinterpret_cast<T*>(acc), reinterpret_cast<const T*>(point), (int)nvars,
                                          s, reinterpret_cast<T*>(scratch), stream);
  if (e != cudaSuccess) return fail(WHIR_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return 0;
}

}  // namespace

extern "C" {

const char* whir_noalloc_last_error(void) { return g_err.c_str(); }

size_t whir_eval_eq_noalloc_max_scratch(void) { return NOALLOC_SCRATCH_BYTES; }

int whir_eval_eq_noalloc(int field, uint64_t* acc_dev, const uint64_t* point_dev, size_t nvars,
                         const uint64_t* scalar, void* stream) {
  g_err.clear();
  if (!acc_dev || !scalar || (nvars > 0 && !point_dev)) return fail(WHIR_ERR_INVALID, "null argument");
  if (nvars == 0 || nvars > 62) return fail(WHIR_ERR_INVALID, "nvars must be in [1, 62]");
  int device = -1;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return fail(WHIR_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (device < 0 || device >= MAX_DEVICES) return fail(WHIR_ERR_INVALID, "device index out of range");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  int rc = scratch_address(device, s, &scratch);
  if (rc) return rc;
  switch (field) {
    case WHIR_GOLDILOCKS1: return run<whir::Gl>(acc_dev, point_dev, nvars, scalar, s, scratch);
    case WHIR_GOLDILOCKS2: return run<whir::Gl2>(acc_dev, point_dev, nvars, scalar, s, scratch);
    case WHIR_GOLDILOCKS3: return run<whir::Gl3>(acc_dev, point_dev, nvars, scalar, s, scratch);
    default: return fail(WHIR_ERR_INVALID, "unsupported field id");
  }
}

}  // extern "C"
