// plan.h -- expression DAG, planning and CUDA code generation.
//
// The reference encodes each expression separately into (left, right, out, op)
// slot arrays with first-free slot reuse and no sharing
// (engine/src/Interpreter/interpreter_cpp.cu:274-438), then interprets that list
// per row.  Here all expressions of one call (filter condition + projections)
// become one DAG with hash-consed common sub-expressions; the DAG is emitted as
// straight-line CUDA in SSA form (the CUDA compiler allocates registers), so the
// kernel never dispatches on operator or type at run time.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "frontend.h"
#include "gx_common.h"

namespace gx {

struct Node {
  enum Kind { COL, LIT, OP } kind = OP;
  Op op = OP_NONE;
  int col = -1;
  int lit_type = EMPTY;
  bool lit_valid = false;
  uint64_t lit_bits = 0;
  int vtype = EMPTY;
  int ktype = EMPTY;
  int a = -1, b = -1;        // operand node ids
  int rand_id = -1;          // RAND ordinal (post-order within its expression group)
  bool rand_out_row = false; // RAND keyed by output (compacted) row instead of input row
  bool exact_null = false;   // data under NULL is observable (feeds CASE's magic test)
};

struct OutSpec {
  enum Kind { NODE, COPY, BROADCAST } kind = NODE;
  int node = -1;       // NODE
  int col = -1;        // COPY
  int type = EMPTY;    // output column type
  uint64_t lit_bits = 0;
  bool lit_valid = false;
  // BROADCAST: the element bits of the literal in the output type
  uint64_t lit_bits_as_element() const;
};

constexpr int kNativeAddSub = 1, kNativeMul = 2, kNativeConvert = 4, kNativeCompare = 8, kNativeRound = 16,
              kNativeDiv = 32, kNativeConstDiv = 64, kNativeIntDiv = 128;

struct KernelConfig {
  int warps = 8;           // warps per CTA
  int words = 2;           // 32-row words per warp per step
  bool emulate_fp64 = true;  // binary64 compares / divides / conversions on the integer pipes
  // with emulate_fp64, operation classes that still use the FP64 pipe (both
  // forms are exact IEEE binary64): kNativeAddSub, kNativeMul, kNativeConvert,
  // kNativeConstDiv (division by a literal: two FMAs and a multiply),
  // kNativeIntDiv (division by an integer value: the same with a table reciprocal),
  // kNativeCompare, kNativeRound, kNativeDiv; -1: chosen per plan
  int native_f64_ops = -1;
  bool dense = true;         // filter kernels: projections on warp-compacted kept rows
  bool lazy_case = true;     // dense phase: expensive CASE branches only for the rows that select them
  bool runtime_order = false;  // short-circuit AND conjuncts in the order given at launch (KernelArgs::order)
  bool staged = false;         // runtime_order: stage conjunct columns in shared memory by bulk copies
  int stream_slots = 0;        // runtime_order: words in flight per warp, refilled as words finish (0: lockstep)
  bool conj_stats = false;     // COUNT_FILTER also counts each conjunct's passing rows
  bool short_circuit = false;
  std::vector<int> conjunct_order;  // indices into Plan::conjuncts
  // single-pass filter calls choose the block shape online among a few
  // candidates (the shape is not fixed by the caller or the environment)
  bool tune_shape = false;
  // registers per thread the kernel is held to (0: the compiler's choice),
  // as launch bounds asking for 65536 / (max_regs x threads) resident blocks
  int max_regs = 0;
  // Single-pass filters on the tile-staged kernel (FUSED_TMA): -1 when the
  // plan qualifies (fixed conjunct order, dense projections), 0 never, 1 always
  // when it qualifies; its consumer warps, 32-row words per consumer warp and
  // input stages (>= 2) of its shared-memory tile ring
  int use_tma = -1;
  int tma_warps = 8;
  int tma_words = 2;
  int stages = 3;
};

struct Plan {
  std::vector<int> schema;
  std::vector<bool> nullable;
  std::vector<Node> nodes;
  int predicate = -1;                 // filter condition node (-1: no filter)
  std::vector<int> conjuncts;         // top-level AND operands of the condition
  std::vector<OutSpec> outputs;
  bool filter_copies_all = false;     // process_filter: outputs are every input column
  uint64_t rand_seed = 0;

  bool has_filter() const { return predicate >= 0; }
  // nodes computed per row by the kernels (outputs of kind NODE + predicate)
  bool needs_kernel() const;
};

// Builds a plan.  condition may be empty (no filter).  When filter_all is set the
// outputs are COPY outputs of every input column (process_filter).  RAND()
// calls in the expressions are numbered from first_rand_id (post-order), so a
// long expression list split over several plans keeps one numbering;
// *rand_count (optional) receives how many the expressions used.
Plan build_plan(const std::vector<int>& schema, const std::vector<bool>& nullable, const std::string& condition,
                const std::vector<std::string>& expressions, bool filter_all, bool rand_by_output_row,
                int first_rand_id = 0, int* rand_count = nullptr, bool all_nodes = false);
// (all_nodes: every expression, a bare column reference included, becomes a
// NODE output computed in the kernel -- the aggregation kernel reads values
// from nodes only; a bare literal is rejected there)

// Fused filter + group-by aggregation (gx_filter_aggregate): the plan's
// outputs are the key columns then the non-empty aggregation inputs, all NODE
// outputs.  The kernel keeps a hash table of groups per block in shared memory
// and merges it into a global table (GxAggArgs) when the block finishes.
struct AggLayout {
  std::vector<int> key_nodes;   // node of each key column
  std::vector<int> kinds;       // gx_agg_kind per aggregation
  std::vector<int> in_nodes;    // input node per aggregation (-1: COUNT(*))
  int smem_slots = 256;         // shared-memory table slots per block (power of two)
  // the lanes of one group combine their inputs over a warp tree before one
  // lane applies them (true), or every lane applies its own row (false)
  bool warp_combine = true;
};
std::string generate_agg_kernel(const Plan& plan, const AggLayout& L, const KernelConfig& cfg, const std::string& name);
// Accumulators (bit j of L's accumulator j) whose input is never NULL under
// plan.nullable: the aggregation kernel keeps no valid count for them, and
// the group's row count stands for it.
uint64_t agg_counts_are_rows(const Plan& plan, const AggLayout& L);

// Outputs per plan kernel; longer expression lists are split into several
// plans (the reference splits at 64 interpreter slots, LogicalProject.cpp:906-922).
constexpr int GX_OUTPUTS_PER_KERNEL = 32;

// FUSED_STREAM: the batched kernel fed by a queue that the host extends while
// it runs (BatchStream, batch.cu)
enum class KernelKind {
  PROJECT, FUSED_FILTER, COUNT_FILTER, WRITE_FILTER, FUSED_BATCHED, FUSED_STAGED, FUSED_TMA, FUSED_STREAM
};

// Shared-memory layout of the tile-staged fused filter (FUSED_TMA): a ring of
// `stages` input stages, each holding one tile (consumer warps x words x 32
// rows) of every column the plan reads -- its data bytes and, for a column
// with a validity mask, its mask words -- copied in by one bulk copy per
// column and tile; then a ring of output staging buffers.
struct TileLayout {
  int tile_rows = 0;
  int stages = 0;
  std::vector<int> cols;             // staged columns, ascending
  std::vector<uint32_t> data_off;    // per staged column: data slot offset within a stage
  std::vector<uint32_t> mask_off;    // mask slot offset (UINT32_MAX: no mask)
  std::vector<int> mask_index;       // index among the masked staged columns (-1: none)
  int num_masked = 0;
  uint32_t stage_bytes = 0;
  // output staging: out_stages buffers of out_stage_bytes from out_base, each
  // with a data slot (out_off) and validity bytes (out_valid_off) per output
  std::vector<uint32_t> out_width, out_off, out_valid_off;
  uint32_t out_stage_bytes = 0;
  uint32_t out_base = 0;
  int out_stages = 3;                // a tile is written out this many tiles after its projections
  uint32_t dyn_smem = 0;             // stages x stage_bytes + out_stages x out_stage_bytes
};
// (plan.nullable tells which columns carry a mask at run time)
TileLayout tile_layout(const Plan& plan, int warps, int words, int stages);

// Header of a batch table run by the FUSED_BATCHED kernel (device memory).
struct BatchHeader {
  unsigned long long tile_counter;  // next tile to claim, over all batches
  long long total_tiles;
  int nbatch;
  int pad;
};

// Distinct columns read by conjunct c (index into Plan::conjuncts), ascending.
std::vector<int> conjunct_columns(const Plan& plan, int c);

// CUDA source of one plan kernel.  The kernel is named by `name`.
std::string generate_kernel(const Plan& plan, KernelKind kind, const KernelConfig& cfg, const std::string& name);

// Parameter block layout shared by generated kernels and the host launcher.
constexpr int GX_MAX_COLS = 64;
constexpr int GX_MAX_OUTS = 64;

struct KernelArgs {
  const void* in_data[GX_MAX_COLS];
  const uint32_t* in_mask[GX_MAX_COLS];
  int64_t in_off[GX_MAX_COLS];
  void* out_data[GX_MAX_OUTS];
  uint32_t* out_mask[GX_MAX_OUTS];
  int64_t n;                 // input rows
  int64_t capacity;          // output rows available (filter kernels)
  uint64_t* tile_status;     // FUSED: look-back status; COUNT/WRITE: per-tile counts / offsets
  unsigned long long* tile_counter;
  unsigned long long* out_count;
  int* err;
  uint64_t seed;
  unsigned long long* conj_counts;  // COUNT_FILTER with conj_stats: passes per conjunct
  int32_t order[16];                // runtime conjunct order (runtime_order kernels)
  const int32_t* order_dev;         // if set: the order in device memory (written by an earlier kernel)
  uint32_t spin_limit;              // polls a bounded device wait makes before it gives up (0: default)
};

// Bytes between two batch descriptors of a batch stream (a multiple of the
// 128-byte cache line, at least sizeof(KernelArgs)).
constexpr size_t kStreamArgsStride = (sizeof(KernelArgs) + 255) / 256 * 256;

}  // namespace gx
