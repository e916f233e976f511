// noalloc.cu -- filter + project into caller-owned buffers without any device
// allocation.
//
// Some callers cannot allocate device memory at the point where they evaluate a
// batch: an engine whose memory resource owns the whole device budget (all
// device memory is handed out by its own pool, so allocations made behind its
// back break its accounting and can fail when the pool has reserved the rest of
// the GPU), or a hot per-batch path that must never enter an allocator.  For
// them gx_plan_execute_noalloc runs the same fused single-pass filter kernel as
// gx_plan_execute, with two differences: the outputs are the caller's buffers,
// and the kernel's scratch (tile ticket, row count, error flag and one
// look-back status word per tile) lives in the fixed array below, which every
// GPU that loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>
#include <unordered_map>

#include "runtime.h"

namespace gx {
namespace {

// 4 MiB: 4 header words + up to GX_NOALLOC_MAX_TILES tile status words.
constexpr long long kScratchWords = 4 + GX_NOALLOC_MAX_TILES;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

std::mutex g_mu;
std::unordered_map<int, unsigned long long*> g_addr;  // device -> address of g_noalloc_scratch

// The array's name in host code is only a host-side handle, not a device
// address: resolve the device address once per device, with that device current.
unsigned long long* scratch_on_current_device() {
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_addr.find(dev);
  if (it != g_addr.end()) return it->second;
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) {
    cudaGetLastError();
    fail(GX_ERR_CUDA, std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(e));
  }
  g_addr[dev] = static_cast<unsigned long long*>(p);
  return g_addr[dev];
}

}  // namespace

void run_filter_noalloc(const CompiledPlan& cp, const std::vector<ColumnView>& cols, gx_column* out,
                        int64_t* out_rows, cudaStream_t s) {
  cp.execute_with_scratch(cols, out, out_rows, scratch_on_current_device(), kScratchWords, s);
}

const CompiledPlan* single_chunk(const gx_plan* plan);  // capi.cpp

}  // namespace gx

extern "C" int gx_plan_execute_noalloc(const gx_plan* plan, const gx_column_view* columns, int num_columns,
                                       gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status) {
  auto set = [&](int code, const char* msg) {
    if (status) {
      status->code = code;
      std::snprintf(status->message, sizeof status->message, "%s", msg);
    }
    return code;
  };
  try {
    const gx::CompiledPlan* cp = gx::single_chunk(plan);
    if (!cp) return set(GX_ERR_INVALID, "gx_plan_execute_noalloc needs a plan with at most 32 outputs "
                                          "over at most 64 columns");
    if (!out && cp->plan().outputs.size() > 0) return set(GX_ERR_INVALID, "null output array");
    gx::run_filter_noalloc(*cp, gx::to_views(columns, num_columns), out, out_rows, (cudaStream_t)stream);
    return set(GX_OK, "");
  } catch (const gx::Error& e) {
    return set(e.code, e.what());
  } catch (const std::exception& e) {
    return set(GX_ERR_INVALID, e.what());
  }
}
