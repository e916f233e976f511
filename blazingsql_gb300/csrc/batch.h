// batch.h -- batch runner (batch.cu): a table of batches of one filter plan
// through one persistent kernel in a captured CUDA graph, with an autotuned
// tile shape.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "runtime.h"

namespace gx {

class BatchRunner {
 public:
  // max_batches / max_rows bound one run; autotune picks warps x words on the
  // first run of at least 2^20 rows (cached per plan, column mix and device)
  BatchRunner(const CompiledPlan& base, int max_batches, int64_t max_rows, bool autotune);
  ~BatchRunner();
  BatchRunner(const BatchRunner&) = delete;
  BatchRunner& operator=(const BatchRunner&) = delete;

  // out: batches.size() x outputs columns (batch-major); caller buffers when
  // out[0].data is set, else one library allocation shared by all of them
  void run(const std::vector<std::vector<ColumnView>>& batches, gx_column* out, int64_t* out_rows, cudaStream_t s);
  int warps() const { return warps_; }
  int words() const { return words_; }

 private:
  void release();
  void ensure_buffers();
  int64_t max_tiles(int words, int warps) const;
  std::shared_ptr<CompiledPlan> variant(int warps, int words);
  int64_t stage(const std::vector<std::vector<ColumnView>>& batches, const gx_column* out, int warps, int words);
  void enqueue(const JitKernel& k, cudaStream_t s, bool timed);
  void capture(const JitKernel& k);
  std::string tune_key(const std::vector<bool>& nullable) const;
  void tune(const std::vector<std::vector<ColumnView>>& batches, gx_column* out, const std::vector<bool>& nullable,
            cudaStream_t s);

  Plan plan_;
  KernelConfig base_cfg_;
  int max_batches_;
  int64_t max_rows_;
  bool autotune_;
  bool tuned_ = false;
  int warps_ = 4, words_ = 4;
  int64_t scratch_tiles_ = 0;
  std::map<std::pair<int, int>, std::shared_ptr<CompiledPlan>> variants_;
  // device buffers: descriptors, tile offsets, header, scratch (per batch 4
  // header words, then the tile status words of every batch)
  KernelArgs* dargs_ = nullptr;
  long long* dbase_ = nullptr;
  BatchHeader* dhdr_ = nullptr;
  uint64_t* dscratch_ = nullptr;
  // pinned host staging the graph copies from / to
  KernelArgs* hargs_ = nullptr;
  long long* hbase_ = nullptr;
  BatchHeader* hhdr_ = nullptr;
  unsigned long long* hres_ = nullptr;
  cudaStream_t cap_stream_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  CUfunction captured_fn_ = nullptr;
};

}  // namespace gx
