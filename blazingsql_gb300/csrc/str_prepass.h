// str_prepass.h -- the string pre-pass (str_prepass.cu): string operators over string
// columns evaluated into BOOL8 / INT32 columns before the plan kernels run.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "frontend.h"
#include "runtime.h"

namespace gx {

// one operator over string column `op.col`, writing `out` (library column of
// op.size rows: BOOL8, INT32 for CHAR_LENGTH); pattern_dev holds op.literal
void launch_string_op(const ColumnView& col, const StringOp& op, const void* pattern_dev, gx_column& out,
                      cudaStream_t s);

// Evaluates `ops` over `cols` and appends their columns to `cols` (column
// ncols + i is op i).  The returned columns are the caller's to free once the
// work that reads them has been enqueued.
std::vector<gx_column> run_string_prepass(std::vector<ColumnView>& cols, const std::vector<StringOp>& ops,
                                          cudaStream_t s);

}  // namespace gx
