// driver.h -- CUDA driver API entry points resolved at run time through the
// runtime's cudaGetDriverEntryPointByVersion, so the library does not link
// libcuda and loads on hosts without a GPU driver (CPU-side tests).
#pragma once

#include <cuda.h>

namespace gx {

struct DriverApi {
  CUresult (*ModuleLoadData)(CUmodule*, const void*);
  CUresult (*ModuleUnload)(CUmodule);
  CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*);
  CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
                           void**, void**);
  CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t);
  CUresult (*FuncGetAttribute)(int*, CUfunction_attribute, CUfunction);
  CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int);
  CUresult (*GetErrorString)(CUresult, const char**);
};

// Resolves the entry points once (throws GX_ERR_CUDA if unavailable).
const DriverApi& driver();

// Message for a driver result code.
const char* driver_error_string(CUresult r);

}  // namespace gx
