// Likelihood evaluation that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc.  A host application may
// reserve the GPU's memory up front for its own pool allocator, so that a
// driver allocation by a library fails or fragments that pool; a sampler may
// run its likelihood calls on a latency-critical path where the device-wide
// synchronisation of cudaMalloc / cudaFree is not acceptable.  For them
// gwl_eval_device_noalloc runs the mixed-precision TaylorF2 launch sequence
// (per-point prologue, band-end ordering, fused likelihood kernel and its
// accurate variant for the points whose error bound exceeds the tolerance,
// finalize) with its work space -- the device status word, the ordering
// histogram with the count of marked points, the per-point records, the
// split-K partial sums and the ordering -- in one statically allocated device
// buffer of kNoAllocScratchBytes
// that every GPU loading this library holds until the process exits.
//
// The caller passes the parameter block and the result buffer.  The first
// call on each device looks up that device's address of the buffer; make it
// before any stream capture.  All calls share the buffer, which keeps the
// contents of the last call: calls whose launches overlap on the GPU (two
// streams, two threads) race on it and must be serialised by the caller.
// The kernels' status word (a bounded wait that gave up, an ordering key out
// of range) lives in the buffer too; gwl_noalloc_status reads and clears it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "gwl_internal.h"

namespace gwl {
namespace {

constexpr size_t kNoAllocScratchBytes = 32u << 20;  // 32 MiB
constexpr size_t kAlign = 256;
constexpr int kMaxDevices = 64;

// The work space.  In host code this name is a host-side stand-in, not a
// device address: only the address from cudaGetSymbolAddress goes to a kernel.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

}  // namespace
}  // namespace gwl

using namespace gwl;

extern "C" int gwl_eval_device_noalloc(gwl_analysis* a, const double* params, int64_t B, double* out,
                                       void* stream) {
  if (!a || B < 0 || (B > 0 && (!params || !out))) {
    set_error("null argument or negative batch size");
    return GWL_ERR_ARGUMENT;
  }
  if (B == 0) return GWL_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error(std::string("gwl_eval_device_noalloc: no usable current device: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  void* base = nullptr;
  {
    // set-up, once per device, with that device current
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        set_error(std::string("gwl_eval_device_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        return GWL_ERR_CUDA;
      }
      g_scratch_ptr[dev] = p;
    }
    base = g_scratch_ptr[dev];
  }
  LaunchArgs L;
  size_t rec_bytes = 0, part_bytes = 0;
  int rc = noalloc_launch_args(a, B, &L, &rec_bytes, &part_bytes);
  if (rc) return rc;
  // the status word, then the ordering histogram and the marked count: one memset clears them
  ordering_with_marks(L);
  const size_t head_bytes = sizeof(int) + sizeof(int32_t) * (2 * (size_t)L.order_keys + 1);
  const size_t rec_off = align_up(head_bytes);
  const size_t part_off = rec_off + align_up(rec_bytes);
  const size_t order_off = part_off + align_up(part_bytes);
  const size_t order_bytes = (size_t)B * sizeof(int32_t);
  const size_t need = order_off + order_bytes;
  if (need > kNoAllocScratchBytes) {
    const size_t per_point = rec_bytes / (size_t)B + part_bytes / (size_t)B + sizeof(int32_t);
    set_error("gwl_eval_device_noalloc: " + std::to_string(B) + " points need " + std::to_string(need) +
              " bytes of scratch, more than the " + std::to_string(kNoAllocScratchBytes) +
              "-byte static buffer; at most about " +
              std::to_string((kNoAllocScratchBytes - rec_off - 3 * kAlign) / per_point) +
              " points fit for this analysis");
    return GWL_ERR_ARGUMENT;
  }
  unsigned char* scratch = static_cast<unsigned char*>(base);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  L.params = params;
  L.out = out;
  L.status = reinterpret_cast<int*>(scratch);
  L.rec = reinterpret_cast<PointRec*>(scratch + rec_off);
  L.part = reinterpret_cast<double*>(scratch + part_off);
  L.dh_out = nullptr;
  L.hh_out = nullptr;
  L.order_hist = reinterpret_cast<int32_t*>(scratch + sizeof(int));
  L.rf_count = L.order_hist + 2 * L.order_keys;
  L.order = reinterpret_cast<int32_t*>(scratch + order_off);
  // The buffer keeps the previous call's contents: the status word, the
  // histogram and the marked count must start at zero; the records, partial
  // sums and ordering are fully written before being read.
  if ((e = cudaMemsetAsync(scratch, 0, head_bytes, s)) != cudaSuccess ||
      (e = launch_prologue(L, s)) != cudaSuccess || (e = launch_order(L, s)) != cudaSuccess ||
      (e = launch_mixed(L, s)) != cudaSuccess || (e = launch_mixed_acc(L, s)) != cudaSuccess ||
      (e = launch_finalize(L, s)) != cudaSuccess) {
    set_error(std::string("gwl_eval_device_noalloc: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  return GWL_OK;
}

extern "C" int gwl_noalloc_status(void* stream, int* device_status) {
  if (!device_status) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *device_status = kDevStatusOk;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error(std::string("gwl_noalloc_status: no usable current device: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> g(g_mu);
    base = g_scratch_ptr[dev];
  }
  if (!base) return GWL_OK;  // no call on this device yet
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int word = 0;
  if ((e = cudaMemcpyAsync(&word, base, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess) {
    set_error(std::string("gwl_noalloc_status: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  *device_status = word;
  if (word == kDevStatusOk) return GWL_OK;
  if ((e = cudaMemsetAsync(base, 0, sizeof(int), s)) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess) {
    set_error(std::string("gwl_noalloc_status: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  if (word == kDevStatusTimeout) {
    set_error("gwl_eval_device_noalloc: a bounded device wait gave up (bulk copy did not complete)");
    return GWL_ERR_TIMEOUT;
  }
  set_error("gwl_eval_device_noalloc: a point's ordering key was out of range");
  return GWL_ERR_ARGUMENT;
}
