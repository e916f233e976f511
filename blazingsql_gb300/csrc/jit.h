// jit.h -- NVRTC compilation of generated plan kernels for sm_103a, with a
// process-wide cache keyed by (source hash, device).
#pragma once

#include <cuda.h>

#include <string>

namespace gx {

struct JitKernel {
  CUfunction fn = nullptr;
  int max_blocks_per_sm = 0;   // occupancy at the kernel's block size
  int block_threads = 0;
  int num_regs = 0;
  unsigned dyn_smem = 0;       // dynamic shared memory per block, bytes
  double compile_ms = 0.0;
};

// Compiles (or fetches from cache) kernel `name` defined in `body` (appended to
// the device runtime prelude) for the current device.
// dyn_smem: dynamic shared memory bytes each launch of the kernel gets.
JitKernel jit_get(const std::string& body, const std::string& name, int block_threads, unsigned dyn_smem = 0);

// Assembler resource report of a kernel (NVRTC + ptxas, no device needed).
struct KernelResources {
  int registers = 0;
  int spill_bytes = 0;
  int shared_bytes = 0;
};
KernelResources jit_resources(const std::string& body, const std::string& name);

// NVRTC compile only (no device needed); throws GX_ERR_CUDA with the log.
void jit_compile_check(const std::string& body, const std::string& name);

// The device runtime prelude prepended to every plan kernel.
const char* jit_prelude();

// Number of SMs of the current device (cached).
int device_sm_count();

// Statistics for diagnostics / autotuning.
long long jit_compile_count();
double jit_compile_ms_total();

}  // namespace gx
