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

// A queue of batches of one filter plan evaluated by one persistent kernel
// (FUSED_STREAM) that runs while the host appends batches: start() launches
// the kernel, which waits for work; push() copies a batch's descriptor and
// tile offsets to the device and then publishes its tiles (ordered copies on a
// side stream, no host synchronisation); finish() closes the queue, waits for
// the kernel and returns every batch's output.  Each batch's output is what
// gx_plan_execute returns for it alone.  A kernel that waits longer than
// wait_polls x ~2 us for a batch gives up (GX_ERR_TIMEOUT at finish).
class BatchStream {
 public:
  BatchStream(const CompiledPlan& base, int max_batches, int64_t max_rows, int warps, int words);
  ~BatchStream();
  BatchStream(const BatchStream&) = delete;
  BatchStream& operator=(const BatchStream&) = delete;

  void start(cudaStream_t s);
  // the batch's columns must stay valid until finish(); returns its index
  int push(const std::vector<ColumnView>& cols);
  // out: num_outputs() columns per pushed batch (batch-major), all views of
  // one allocation released with the last of them; out_rows: rows per batch
  void finish(gx_column* out, int64_t* out_rows, int max_out_batches);
  int pushed() const { return count_; }
  bool running() const { return running_; }
  int num_outputs() const { return (int)plan_.outputs.size(); }
  void set_wait_polls(unsigned polls) { wait_polls_ = polls; }

 private:
  void release();
  Plan plan_;
  std::shared_ptr<CompiledPlan> variant_;
  JitKernel kernel_{};
  int max_batches_;
  int64_t max_rows_;
  int64_t tile_rows_ = 0;
  int64_t max_tiles_ = 0;
  int64_t arena_rows_ = 0;
  unsigned wait_polls_ = 1u << 22;
  // session state
  bool running_ = false;
  cudaStream_t s_ = nullptr;
  int count_ = 0;
  int64_t tiles_ = 0, rows_used_ = 0;
  char* arena_ = nullptr;               // this session's outputs: every output's masks, then data
  std::vector<size_t> moff_, doff_;     // per output: byte offset of its mask / data region
  std::vector<int64_t> row_off_, rows_in_;
  // device
  KernelArgs* dargs_ = nullptr;
  long long* dbase_ = nullptr;
  BatchHeader* dhdr_ = nullptr;
  uint64_t* dscratch_ = nullptr;        // per batch 4 words (row count at [1], error at [2]), then tile statuses
  int* dwerr_ = nullptr;
  // pinned host staging of the pushes' copies (one slot per batch: a copy may
  // run after the host moved on)
  KernelArgs* hargs_ = nullptr;
  long long* hbase_ = nullptr;
  long long* hpub_ = nullptr;
  int* hflag_ = nullptr;                // [0] = 1 (closes the queue), [1] = the kernel's wait error
  unsigned long long* hres_ = nullptr;
  cudaStream_t push_stream_ = nullptr;
  cudaEvent_t started_ = nullptr;
};

}  // namespace gx
