// runtime.h -- plan execution on the device: output allocation, kernel
// launches, compaction bookkeeping.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "jit.h"
#include "plan.h"

namespace gx {

struct ColumnView {
  int type;
  const void* data;
  const uint32_t* mask;
  int64_t offset;
  int64_t size;
  const int32_t* str_offsets = nullptr;  // STRING columns: cudf offsets (data = characters)
};

std::vector<ColumnView> to_views(const gx_column_view* cols, int n);

// stream-ordered device allocation from the device's memory pool; failures
// raise GX_ERR_OOM (retryable)
void* dev_alloc(size_t bytes, cudaStream_t s);
// output columns sharing one device allocation (see alloc_outputs in runtime.cu):
// types[i] / caps[i] per column; masks zeroed when zero_masks
void alloc_output_set(const std::vector<int>& types, const std::vector<int64_t>& caps, bool zero_masks,
                      gx_column* out, cudaStream_t s);
// output columns of one call in one allocation: [scratch | masks | data];
// returns the scratch (scratch_bytes > 0) or nullptr
void* alloc_outputs(const std::vector<int>& types, int64_t capacity, size_t scratch_bytes, bool zero_masks,
                    gx_column* out, cudaStream_t s);
int64_t mask_words_for(int64_t rows);  // padded 32-bit mask words an output of `rows` rows holds
// Outputs of a queue of filter calls in one allocation and one memset: for
// batch b, types.size() columns of capacity caps[b] with zeroed masks
// (out[b * types.size() + j]) and status_words[b] zeroed tile-status words
// (status[b]); the allocation starts with a zeroed kQueueHeaderBytes header
// per batch (the returned base).  Released when the last column is freed.
constexpr size_t kQueueHeaderBytes = 256;
void* alloc_output_queue(const std::vector<int>& types, const std::vector<int64_t>& caps,
                         const std::vector<int64_t>& status_words, gx_column* out, uint64_t** status,
                         cudaStream_t s);
// Makes n columns that view distinct parts of one allocation `base` (from
// dev_alloc) owners of it: the allocation is released with the last of them.
void adopt_output_views(void* base, gx_column* cols, int n);
// The headers and tile-status words of a queue without its outputs (a queue
// whose outputs are allocated batch by batch): the same layout, zeroed; the
// caller releases the returned base with dev_free once the queue completed.
void* alloc_queue_scratch(const std::vector<int64_t>& status_words, uint64_t** status, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);
void check_cuda(cudaError_t e, const char* what);
// host-side fault injection for tests: fail the n-th next allocation (n >= 1)
void debug_fail_allocation(int n);

// allocates an output column holding `capacity` rows (data + padded mask)
gx_column alloc_column(int type, int64_t capacity, cudaStream_t s);
void free_column(gx_column& c, cudaStream_t s);

// Per-launch extras of a filter execution (learned ordering, label counting).
struct ExecExtras {
  const int* order = nullptr;              // runtime conjunct order (runtime_order kernels)
  const int* order_dev = nullptr;          // or the order in device memory (read by the kernel)
  int num_order = 0;
  unsigned long long* conj_counts = nullptr;  // device counters, one per conjunct (conj_stats count pass)
  unsigned long long* conj_counts_host = nullptr;  // optional host copy of them, made before the count sync
  int64_t capacity_hint = -1;              // library-allocated outputs: rows to allocate (-1: all input rows)
  // diagnostics: the tile ticket starts here, so tiles before it are never
  // claimed and their look-back status is never published; and the polls a
  // bounded device wait makes before it gives up (0: default)
  int64_t first_tile = 0;
  uint32_t spin_limit = 0;
};

struct ExecStats {
  double kernel_ms = 0;      // not measured unless requested
  int64_t tiles = 0;
  int grid = 0;
  int block = 0;
  int regs = 0;
};

class CompiledPlan {
 public:
  struct Shape {
    int warps, words;  // block shape of a filter kernel: warps x 32-row words per warp
    int regs = 0;      // registers per thread the kernel is held to (0: the configured cap, if any)
  };
  // the single-pass filter's block shape now: the tuned one once chosen
  Shape current_shape() const;
  CompiledPlan(Plan p, KernelConfig cfg, int mode) : plan_(std::move(p)), cfg_(std::move(cfg)), mode_(mode) {}

  // Fused single-pass filter into the caller's buffers (out[j].data / null_mask /
  // capacity), with the kernel's scratch taken from `scratch` (scratch_words
  // 8-byte words) instead of the memory pool.  Makes no device allocation.
  void execute_with_scratch(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                            unsigned long long* scratch, long long scratch_words, cudaStream_t s) const;

  // Runs the plan over `cols`.  out must hold plan.outputs.size() entries.  If
  // out[0].data is non-null, caller-supplied buffers are used (capacity rows).
  void execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows, cudaStream_t s,
               const ExecExtras* extras = nullptr) const;

  // Queue form of a filter call: only the plan's kernels go on the stream (no
  // allocation, memset, copy or synchronisation).  out[j] come from the caller
  // with room for every input row and zeroed masks; `hdr` (4 words: tile
  // counter, single-pass row count, error flag, two-pass row count) and
  // `tile_status` (tiles_for(n) words) are zeroed device memory.  The call is
  // completed by finish_queued() on a host copy of hdr once the stream has
  // reached it.  Needs can_defer().
  void enqueue_filter(const std::vector<ColumnView>& cols, gx_column* out, unsigned long long* hdr,
                      uint64_t* tile_status, const ExecExtras* extras, cudaStream_t s) const;
  void finish_queued(const unsigned long long* hdr, int64_t n, gx_column* out, int64_t* out_rows) const;
  // Host-to-host execution: `cols` and out[j].data / null_mask are host
  // memory (inputs at offset 0; pinned memory gives full copy bandwidth),
  // out[j].capacity the rows the host buffers hold.  A filter plan without
  // literal outputs runs as a pipeline of row chunks whose copies in, kernels
  // and copies out overlap; other plans copy in, run and copy out.  Returns
  // after the outputs are in host memory.
  void execute_host(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows, cudaStream_t s) const;
  // a filter plan whose outputs are all computed per row (none a literal)
  bool can_defer() const;
  // tile-status words a filter over n rows uses
  int64_t tiles_for(int64_t n) const;
  // single-pass calls over these columns run on the tile-staged kernel
  bool tma_path(const std::vector<ColumnView>& cols) const;
  // dynamic shared memory a tile ring may take (the rest of the 227 KiB a
  // block can have holds the kernel's kept-row lists and branch results)
  static constexpr unsigned kTmaMaxDynSmem = 176u * 1024u;

  // kernel handle of this plan for a given kind and set of columns with masks
  JitKernel kernel_for(KernelKind kind, const std::vector<bool>& nullable) const { return kernel(kind, nullable); }

  const Plan& plan() const { return plan_; }
  const KernelConfig& config() const { return cfg_; }
  int mode() const { return mode_; }
  mutable ExecStats last;

 private:
  // warps / words / regs: a block shape and register cap other than the configured ones (0: configured)
  JitKernel kernel(KernelKind kind, const std::vector<bool>& nullable, int warps = 0, int words = 0,
                   int regs = 0) const;
  // Block shape of a single-pass filter call over n rows.  With tune_shape,
  // calls of at least kShapeTuneRows rows first run the first candidate once
  // unmeasured (a warm-up), then each candidate once (*explore = its index;
  // the caller reports its time to shape_measured), then every call takes the
  // fastest.
  Shape filter_shape(int64_t n, int* explore) const;
  void shape_measured(int idx, float ms) const;
  static constexpr int64_t kShapeTuneRows = int64_t(1) << 22;
  mutable std::mutex tmu_;
  mutable std::vector<float> cand_ms_;  // per candidate, < 0 until measured
  mutable int next_cand_ = 0;
  mutable int chosen_ = -1;
  mutable std::atomic<bool> tune_compile_{false};  // compile every candidate on the next call
  void run_project(const std::vector<ColumnView>& cols, gx_column* out, bool caller_bufs, cudaStream_t s) const;
  void run_filter(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows, bool caller_bufs,
                  const ExecExtras* extras,
                  cudaStream_t s) const;

  Plan plan_;
  KernelConfig cfg_;
  int mode_;
  // kernel handles by (kind, nullable columns, device): generating and hashing
  // the source is host work worth skipping on every batch
  mutable std::mutex kmu_;
  mutable std::unordered_map<std::string, JitKernel> kcache_;
};

// no-allocation variant of the fused filter (noalloc.cu)
void run_filter_noalloc(const CompiledPlan& cp, const std::vector<ColumnView>& cols, gx_column* out,
                        int64_t* out_rows, cudaStream_t s);

// diagnostics: per-thread kernel timing and a global launch counter
void set_kernel_timing(bool on);
bool kernel_timing_enabled();
double kernel_ms(bool reset);
int64_t launch_count();
void add_launches(int64_t n);  // kernels launched outside CompiledPlan (learner)

// launch helpers for precompiled kernels (runtime.cu)
void launch_copy_mask(const uint32_t* src, int64_t src_bit, uint32_t* dst, int64_t nrows, int64_t dst_words,
                      cudaStream_t s);
void launch_fill(void* dst, int width, uint64_t value, int64_t n, cudaStream_t s);
void launch_fill_mask(uint32_t* dst, int64_t nrows, bool valid, int64_t dst_words, cudaStream_t s);
void launch_scan_tiles(uint64_t* counts, int64_t n, unsigned long long* total, cudaStream_t s);
// launches a plan kernel with an arbitrary parameter list (counted, optionally timed)
void launch_raw(const JitKernel& k, int grid, cudaStream_t s, void** params, bool timed);

}  // namespace gx
