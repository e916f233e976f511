// jit.cpp -- NVRTC -> cubin -> driver-API module cache (see jit.h).
#include "jit.h"

#include <cuda_runtime.h>
#include <nvrtc.h>

#include <cctype>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <mutex>
#include <sstream>
#include <unordered_map>
#include <vector>

#include "driver.h"
#include "gx_common.h"

namespace gx {
namespace {

// device runtime prelude, embedded at build time from device_rt.cuh
const char* kPrelude =
#include "device_rt.inc"
    ;

struct Entry {
  CUmodule mod = nullptr;
  JitKernel k;
};

std::mutex g_mu;
std::unordered_map<std::string, Entry> g_cache;
long long g_compiles = 0;
double g_compile_ms = 0.0;

uint64_t fnv1a(const std::string& s) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

void check_cu(CUresult r, const char* what) {
  if (r != CUDA_SUCCESS)
    fail(r == CUDA_ERROR_OUT_OF_MEMORY ? GX_ERR_OOM : GX_ERR_CUDA, std::string(what) + ": " + driver_error_string(r));
}

std::string cubin_cache_path(uint64_t h) {
  const char* dir = std::getenv("GX_JIT_CACHE_DIR");
  if (!dir || !*dir) return "";
  char buf[64];
  std::snprintf(buf, sizeof buf, "/gx_%016llx.cubin", (unsigned long long)h);
  return std::string(dir) + buf;
}

// ptxas_log (optional) receives the assembler's resource report
std::vector<char> compile_cubin(const std::string& src, const std::string& name, std::string* ptxas_log = nullptr) {
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), (name + ".cu").c_str(), 0, nullptr, nullptr) != NVRTC_SUCCESS)
    fail(GX_ERR_CUDA, "nvrtcCreateProgram failed");
  const char* opts[] = {"--gpu-architecture=sm_103a", "--fmad=false", "-default-device", "--std=c++17",
                        "-lineinfo", "--ptxas-options=-v"};
  const int nopts = (int)(sizeof(opts) / sizeof(opts[0])) - (ptxas_log ? 0 : 1);
  nvrtcResult r = nvrtcCompileProgram(prog, nopts, opts);
  if (r != NVRTC_SUCCESS) {
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    std::string log(ls, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    // GX_JIT_DUMP names a directory that receives the failing source
    const char* dump = std::getenv("GX_JIT_DUMP");
    if (dump && *dump) {
      std::ofstream f(std::string(dump) + "/gx_failed_" + name + ".cu");
      f << src;
    }
    fail(GX_ERR_CUDA, "NVRTC compile of " + name + " failed: " + log.substr(0, 400));
  }
  if (ptxas_log) {
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    ptxas_log->assign(ls, '\0');
    nvrtcGetProgramLog(prog, &(*ptxas_log)[0]);
  }
  size_t cs = 0;
  nvrtcGetCUBINSize(prog, &cs);
  std::vector<char> cubin(cs);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  return cubin;
}

}  // namespace

int device_sm_count() {
  static std::mutex mu;
  static std::unordered_map<int, int> counts;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = counts.find(dev);
  if (it != counts.end()) return it->second;
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    fail(GX_ERR_CUDA, "cannot query SM count");
  counts[dev] = n;
  return n;
}

JitKernel jit_get(const std::string& body, const std::string& name, int block_threads, unsigned dyn_smem) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) fail(GX_ERR_CUDA, "no CUDA device");
  const std::string src = std::string(kPrelude) + "\n" + body;
  const uint64_t h = fnv1a(src);
  char keybuf[64];
  std::snprintf(keybuf, sizeof keybuf, "%016llx:%d:%u", (unsigned long long)h, dev, dyn_smem);
  const std::string key(keybuf);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) return it->second.k;
  }
  // make the runtime's primary context current for the driver API calls
  cudaFree(nullptr);
  auto t0 = std::chrono::steady_clock::now();
  std::vector<char> cubin;
  const std::string path = cubin_cache_path(h);
  if (!path.empty()) {
    std::ifstream f(path, std::ios::binary);
    if (f) cubin.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  }
  if (cubin.empty()) {
    cubin = compile_cubin(src, name);
    if (!path.empty()) {
      std::ofstream f(path, std::ios::binary);
      f.write(cubin.data(), (std::streamsize)cubin.size());
    }
  }
  Entry e;
  const DriverApi& d = driver();
  check_cu(d.ModuleLoadData(&e.mod, cubin.data()), "cuModuleLoadData");
  check_cu(d.ModuleGetFunction(&e.k.fn, e.mod, name.c_str()), "cuModuleGetFunction");
  // static + dynamic shared memory above 48 KiB needs the opt-in; set it for every dynamic size
  if (dyn_smem > 0u)
    check_cu(d.FuncSetAttribute(e.k.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)dyn_smem),
             "cuFuncSetAttribute(max dynamic shared memory)");
  e.k.dyn_smem = dyn_smem;
  check_cu(d.OccupancyMaxActiveBlocksPerMultiprocessor(&e.k.max_blocks_per_sm, e.k.fn, block_threads, dyn_smem),
           "cuOccupancyMaxActiveBlocksPerMultiprocessor");
  d.FuncGetAttribute(&e.k.num_regs, CU_FUNC_ATTRIBUTE_NUM_REGS, e.k.fn);
  e.k.block_threads = block_threads;
  if (e.k.max_blocks_per_sm < 1) e.k.max_blocks_per_sm = 1;
  auto t1 = std::chrono::steady_clock::now();
  e.k.compile_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cache.find(key);
  if (it != g_cache.end()) {  // another thread won the race
    d.ModuleUnload(e.mod);
    return it->second.k;
  }
  g_compiles++;
  g_compile_ms += e.k.compile_ms;
  g_cache[key] = e;
  return e.k;
}

void jit_compile_check(const std::string& body, const std::string& name) {
  compile_cubin(std::string(kPrelude) + "\n" + body, name);
}

static int number_before(const std::string& log, const std::string& suffix) {
  const size_t at = log.find(suffix);
  if (at == std::string::npos) return 0;
  size_t b = at;
  while (b > 0 && log[b - 1] == ' ') b--;
  size_t e = b;
  while (b > 0 && std::isdigit((unsigned char)log[b - 1])) b--;
  return b < e ? std::atoi(log.substr(b, e - b).c_str()) : 0;
}

KernelResources jit_resources(const std::string& body, const std::string& name) {
  std::string log;
  compile_cubin(std::string(kPrelude) + "\n" + body, name, &log);
  KernelResources r;
  r.registers = number_before(log, "registers");
  r.spill_bytes = number_before(log, "bytes spill stores");
  r.shared_bytes = number_before(log, "bytes smem");
  return r;
}

const char* jit_prelude() { return kPrelude; }

long long jit_compile_count() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_compiles;
}

double jit_compile_ms_total() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_compile_ms;
}

}  // namespace gx
