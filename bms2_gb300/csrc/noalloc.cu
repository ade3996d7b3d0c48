// GMCR offsets without any device allocation.
//
// bms_gmcr_offsets_static turns per-data-graph pair counts into the GMCR
// data_graph_offsets (an exclusive prefix sum with the total in the last slot)
// using the library's multi-block scan.  The scan needs scratch words for its
// per-block partial sums; everywhere else the library allocates them, here they
// live in a fixed array in this file, so the call itself never allocates.
//
// It exists for callers that must not allocate device memory at call time:
// applications whose device memory is owned by their own pool allocator (a
// cudaMalloc from inside would fail once the pool has reserved the device, or
// fragment it), and latency-sensitive pipelines that cannot afford the implicit
// device-wide synchronisation of cudaMalloc/cudaFree while other streams run.
#include <mutex>
#include <string>

#include "../../include/bms.h"
#include "graphs.h"
#include "internal.h"

namespace bms {
namespace {

// Scratch of the scan: kStaticScanWords 32-bit words, shared by every call of
// the entry point on a device.  scan_scratch_words(kMaxStaticScanItems) fits.
constexpr size_t kStaticScanWords = 65536;  // 256 KiB per device
constexpr uint64_t kMaxStaticScanItems = 100000000ull;

static __device__ __align__(256) uint32_t g_scan_scratch[kStaticScanWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
// Per device: the context the address was looked up in, and the address.  A
// module's globals live per context, so a caller that makes another context
// current on the same device (driver API) gets its own lookup.
void* g_scratch_ctx[kMaxDevices] = {};
uint32_t* g_scratch_addr[kMaxDevices] = {};

// cuCtxGetCurrent through the runtime's driver entry point (no libcuda link).
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

// Device address of g_scan_scratch in the current context of `device`, looked
// up once per (device, context): the host-side symbol is only a stand-in,
// never a device address.
int scratch_address(int device, uint32_t** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  void* cur = nullptr;
  if (CtxGetCurrentFn f = ctx_get_current()) f(&cur);
  if (!g_scratch_addr[device] || g_scratch_ctx[device] != cur) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_thread_error(std::string("cudaGetSymbolAddress of the static scan scratch failed: ") +
                       cudaGetErrorString(e));
      return BMS_ECUDA;
    }
    g_scratch_addr[device] = static_cast<uint32_t*>(p);
    // the first runtime call above may have created the primary context
    if (CtxGetCurrentFn f = ctx_get_current()) f(&cur);
    g_scratch_ctx[device] = cur;
  }
  *out = g_scratch_addr[device];
  return BMS_OK;
}

}  // namespace
}  // namespace bms

extern "C" int bms_gmcr_offsets_static(const uint32_t* counts, uint32_t* offsets, uint64_t n, void* stream) {
  using namespace bms;
  if (!offsets || (n && !counts)) {
    set_thread_error("bms_gmcr_offsets_static: counts and offsets must be device pointers");
    return BMS_EINVAL;
  }
  if (n > kMaxStaticScanItems || scan_scratch_words(n) > kStaticScanWords) {
    set_thread_error("bms_gmcr_offsets_static: " + std::to_string(n) + " data graphs exceed the limit of " +
                     std::to_string(kMaxStaticScanItems));
    return BMS_EUNSUPPORTED;
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess || device < 0 || device >= kMaxDevices) {
    cudaGetLastError();
    set_thread_error("bms_gmcr_offsets_static: no usable current device");
    return BMS_ENODEV;
  }
  uint32_t* scratch = nullptr;
  const int r = scratch_address(device, &scratch);
  if (r != BMS_OK) return r;
  // Every scratch word the scan reads is written earlier in the same call, so
  // nothing has to be cleared between calls.
  e = launch_scan_u32(counts, offsets, n, scratch, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_thread_error(std::string("bms_gmcr_offsets_static: launch failed: ") + cudaGetErrorString(e));
    return BMS_ECUDA;
  }
  return BMS_OK;
}
