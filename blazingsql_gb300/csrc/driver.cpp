// driver.cpp -- run-time resolution of driver API entry points (see driver.h).
#include "driver.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "gx_common.h"

namespace gx {
namespace {

template <class F>
void resolve(const char* sym, F& fn) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  cudaError_t e = cudaGetDriverEntryPointByVersion(sym, &p, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    cudaGetLastError();
    fail(GX_ERR_CUDA, std::string("CUDA driver entry point unavailable: ") + sym);
  }
  fn = reinterpret_cast<F>(p);
}

DriverApi g_api;
std::once_flag g_once;

}  // namespace

const DriverApi& driver() {
  std::call_once(g_once, [] {
    resolve("cuModuleLoadData", g_api.ModuleLoadData);
    resolve("cuModuleUnload", g_api.ModuleUnload);
    resolve("cuModuleGetFunction", g_api.ModuleGetFunction);
    resolve("cuLaunchKernel", g_api.LaunchKernel);
    resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", g_api.OccupancyMaxActiveBlocksPerMultiprocessor);
    resolve("cuFuncGetAttribute", g_api.FuncGetAttribute);
    resolve("cuFuncSetAttribute", g_api.FuncSetAttribute);
    resolve("cuGetErrorString", g_api.GetErrorString);
  });
  return g_api;
}

const char* driver_error_string(CUresult r) {
  const char* s = nullptr;
  if (g_api.GetErrorString) g_api.GetErrorString(r, &s);
  return s ? s : "unknown CUDA driver error";
}

}  // namespace gx
