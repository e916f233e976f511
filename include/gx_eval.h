/*
 * gx_eval.h -- C ABI of the GB300-native row-wise expression evaluator.
 *
 * Drop-in boundary for the path behind BlazingSQL's LogicalProject /
 * LogicalFilter: the entry points below take the same inputs as the
 * reference's C++ functions (a table of fixed-width columns in the cudf layout
 * plus Calcite RexNode expression text) and return owning device columns.
 *
 * Column layout (cudf 21.08, as read by engine/src/Interpreter/interpreter_ops.cuh):
 *   - data: device pointer to element 0; row r of the view is element offset + r;
 *   - null_mask: device pointer to uint32 words, bit (offset + r) % 32 of word
 *     (offset + r) / 32 is row r, 1 = valid (Arrow order); NULL = no nulls;
 *   - type ids: numbering of cudf::type_id (GX_TYPE_* below).
 * Outputs always carry a validity mask, zero-padded to 64 bytes.
 *
 * Errors never cross the ABI as exceptions: every call returns a gx_status code
 * and fills gx_status_info (code + message) when one is passed.
 * Streams are cudaStream_t passed as void*; NULL means the legacy default stream.
 * All entry points are reentrant; a compiled gx_plan is immutable and may be
 * shared between threads.
 */
#ifndef GX_EVAL_H
#define GX_EVAL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GX_ABI_VERSION 2

/* cudf::type_id numbering (cudf 21.08) */
enum gx_type_id {
  GX_TYPE_EMPTY = 0,
  GX_TYPE_INT8 = 1, GX_TYPE_INT16 = 2, GX_TYPE_INT32 = 3, GX_TYPE_INT64 = 4,
  GX_TYPE_UINT8 = 5, GX_TYPE_UINT16 = 6, GX_TYPE_UINT32 = 7, GX_TYPE_UINT64 = 8,
  GX_TYPE_FLOAT32 = 9, GX_TYPE_FLOAT64 = 10, GX_TYPE_BOOL8 = 11,
  GX_TYPE_TIMESTAMP_DAYS = 12, GX_TYPE_TIMESTAMP_SECONDS = 13, GX_TYPE_TIMESTAMP_MILLISECONDS = 14,
  GX_TYPE_TIMESTAMP_MICROSECONDS = 15, GX_TYPE_TIMESTAMP_NANOSECONDS = 16,
  GX_TYPE_DURATION_DAYS = 17, GX_TYPE_DURATION_SECONDS = 18, GX_TYPE_DURATION_MILLISECONDS = 19,
  GX_TYPE_DURATION_MICROSECONDS = 20, GX_TYPE_DURATION_NANOSECONDS = 21,
  GX_TYPE_DICTIONARY32 = 22, GX_TYPE_STRING = 23
};

/* Status codes.  GX_ERR_OOM is retryable (the reference maps rmm::bad_alloc to
 * task_status::RETRY, engine/src/execution_kernels/BatchProcessing.cpp:379-384). */
typedef enum gx_status {
  GX_OK = 0,
  GX_ERR_PARSE = 1,          /* malformed RexNode text                       */
  GX_ERR_UNSUPPORTED = 2,    /* operator / type outside this evaluator        */
  GX_ERR_TYPE = 3,           /* type rule violation (e.g. non-BOOL8 filter)   */
  GX_ERR_OOM = 4,            /* device allocation failed: retry later         */
  GX_ERR_CUDA = 5,           /* CUDA runtime / NVRTC failure                  */
  GX_ERR_TIMEOUT = 6,        /* a bounded device-side wait gave up            */
  GX_ERR_INVALID = 7,        /* bad argument (null pointer, size mismatch...) */
  GX_ERR_CAPACITY = 8        /* output capacity too small (plan API)          */
} gx_status;

typedef struct gx_status_info {
  int32_t code;
  char message[500];
} gx_status_info;

typedef struct gx_column_view {
  int32_t type_id;          /* enum gx_type_id */
  int32_t reserved;
  const void* data;         /* device memory (GX_TYPE_STRING: the characters) */
  const uint32_t* null_mask;/* device memory or NULL */
  int64_t offset;           /* in elements (rows) */
  int64_t size;             /* rows */
  /* GX_TYPE_STRING only (cudf's strings column: offsets child + chars): device
   * int32 offsets, row r spanning data[string_offsets[offset + r]] up to
   * data[string_offsets[offset + r + 1]]; NULL for every other type.  String
   * columns are read by the string pre-pass (LIKE, CHAR_LENGTH, comparisons,
   * CASE with string results, the string functions and CASTs of
   * evaluate_string_functions), passed through as outputs ($i) and compacted
   * by gx_process_filter / gx_filter_project. */
  const int32_t* string_offsets;
} gx_column_view;

typedef struct gx_column {
  int32_t type_id;
  int32_t reserved;
  void* data;               /* device memory owned by this library */
  uint32_t* null_mask;      /* device memory owned by this library, always present */
  int64_t size;             /* rows */
  int64_t capacity;         /* rows the buffers can hold (>= size) */
  /* GX_TYPE_STRING outputs (a cudf strings column): `data` holds the
   * characters, string_offsets the size + 1 int32 offsets (row r spans
   * data[string_offsets[r]] up to data[string_offsets[r + 1]]; a NULL row is
   * empty) and string_bytes = string_offsets[size].  All three are owned by
   * the column and released by gx_free_columns.  NULL / 0 for other types. */
  int32_t* string_offsets;
  int64_t string_bytes;
} gx_column;

/* ---- reference-shaped entry points ------------------------------------ */

/* ral::processor::evaluate_expressions(const cudf::table_view&, const std::vector<std::string>&)
 * (engine/src/execution_kernels/LogicalProject.h:24-25, LogicalProject.cpp:796-941).
 * out[i] receives the column of expressions[i]. */
int gx_evaluate_expressions(const gx_column_view* columns, int num_columns,
                            const char* const* expressions, int num_expressions,
                            gx_column* out, void* stream, gx_status_info* status);

/* ral::processor::process_project(std::unique_ptr<BlazingTable>, const std::string& query_part, Context*)
 * (LogicalProject.h:27-30, LogicalProject.cpp:943-969).  query_part is the
 * LogicalProject(...) text; *num_out receives the number of projections and
 * out_names (optional, max_out entries of name_len bytes) their names. */
int gx_process_project(const gx_column_view* columns, int num_columns, const char* query_part,
                       gx_column* out, int max_out, int* num_out, char* out_names, int name_len,
                       void* stream, gx_status_info* status);

/* ral::processor::process_filter(const BlazingTableView&, const std::string& query_part, Context*)
 * (LogicalFilter.h:18-21, LogicalFilter.cpp:31-52).  Evaluates condition=[..]
 * (or filters=[..]) and compacts every input column, keeping row order.
 * out receives num_columns columns; *out_rows the surviving row count. */
int gx_process_filter(const gx_column_view* columns, int num_columns, const char* query_part,
                      gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status);

/* Fused filter + project in one device pass:
 * process_project(process_filter(table, condition), expressions).
 * A NULL / empty condition keeps every row. */
int gx_filter_project(const gx_column_view* columns, int num_columns, const char* condition,
                      const char* const* expressions, int num_expressions,
                      gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status);

/* The query's current timestamp, "YYYY-MM-DD hh:mm:ss[.fraction]" (the value
 * BlazingSQL's engine Context keeps, Context::getCurrentTimestamp,
 * engine/src/execution_graph/Context.h:47), for the calls the calling thread
 * makes afterwards: CURRENT_TIMESTAMP (and CURRENT_TIME) becomes it to the
 * millisecond and CURRENT_DATE its date, as get_current_date_or_timestamp does
 * (engine/src/parser/expression_utils.cpp:1494-1518).  NULL or "" clears it;
 * without one such expressions are rejected with GX_ERR_UNSUPPORTED.  It stands
 * in for the Context* the reference's process_filter / process_project take. */
int gx_set_current_timestamp(const char* timestamp, gx_status_info* status);

/* Releases columns returned by this library (stream-ordered). */
void gx_free_columns(gx_column* columns, int num_columns, void* stream);

/* Copies a column's first `size` rows and its mask words to host memory.  For
 * a GX_TYPE_STRING column host_data receives the string_bytes characters. */
int gx_column_to_host(const gx_column* column, void* host_data, uint32_t* host_mask,
                      void* stream, gx_status_info* status);

/* LIKE(text, 'pattern') through the byte automaton the string pre-pass
 * builds for the pattern, evaluated on the host exactly as the kernel walks it
 * (no GPU needed): *result = 1 match, 0 no match, -1 when the pattern runs on
 * the backtracking matcher instead. */
int gx_debug_like_automaton(const char* pattern, const char* text, int64_t text_len, int32_t* result,
                            gx_status_info* status);

/* The size + 1 offsets of a GX_TYPE_STRING column, to host memory. */
int gx_string_offsets_to_host(const gx_column* column, int32_t* host_offsets, void* stream,
                              gx_status_info* status);

/* ---- compiled plans (batched execution-graph path) --------------------- */

typedef struct gx_plan gx_plan;

typedef enum gx_filter_mode {
  GX_FILTER_AUTO = 0,       /* library picks (single pass, worst-case capacity)      */
  GX_FILTER_TWO_PASS = 1,   /* count pass + write pass, exact output size            */
  GX_FILTER_SINGLE_PASS = 2 /* decoupled look-back compaction into caller capacity   */
} gx_filter_mode;

typedef struct gx_plan_options {
  int32_t filter_mode;      /* gx_filter_mode */
  int32_t block_threads;    /* 0 = autotuned / default */
  int32_t words_per_warp;   /* 32-row validity words per warp per step, 0 = default */
  int32_t use_tma;          /* -1 auto, 0 direct loads, 1 TMA bulk staging */
  int32_t short_circuit;    /* 1: evaluate AND conjuncts in `conjunct_order`, skip dead warps */
  int32_t num_conjuncts;    /* entries in conjunct_order (0 = textual order) */
  int32_t conjunct_order[16];
  uint64_t rand_seed;       /* seed of RAND() streams */
} gx_plan_options;

void gx_plan_options_init(gx_plan_options* options);

/* Compiles condition + expressions for a column schema.  Nullability is a
 * per-column hint (1 = may have nulls); a NULL null_mask at run time is always
 * accepted.  Any number of columns and expressions: the plan runs as kernels
 * of at most 32 outputs, each binding at most 64 of the columns (the ones its
 * expressions read, over tables wider than that), as the reference splits its
 * interpreter plans at 64 slots (LogicalProject.cpp:906-922). */
gx_plan* gx_plan_compile(const int32_t* column_types, const uint8_t* column_nullable, int num_columns,
                         const char* condition, const char* const* expressions, int num_expressions,
                         const gx_plan_options* options, gx_status_info* status);

/* Number and types of the plan's output columns. */
int gx_plan_num_outputs(const gx_plan* plan);
int32_t gx_plan_output_type(const gx_plan* plan, int index);
/* Number of top-level AND conjuncts in the condition (1 if not an AND). */
int gx_plan_num_conjuncts(const gx_plan* plan);

/* Runs the plan over one batch.  If out[i].data is NULL the library allocates
 * the outputs; otherwise the caller's buffers (capacity rows) are used and
 * GX_ERR_CAPACITY is returned, with *out_rows set to the needed row count,
 * when they are too small. */
int gx_plan_execute(const gx_plan* plan, const gx_column_view* columns, int num_columns,
                    gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status);

/* Runs a filter plan (condition required, at most 32 outputs over a table of
 * at most 64 columns) into the
 * caller's buffers without allocating any device memory.  No counterpart in
 * the reference.
 *
 * For callers that cannot allocate device memory while they evaluate a batch:
 * an engine whose own memory pool owns the whole device budget (allocations
 * made outside it break its accounting, and fail once it has reserved the
 * rest of the GPU), or a per-batch path that must not enter an allocator.
 * Same results as gx_plan_execute in GX_FILTER_SINGLE_PASS mode, from the same
 * direct-load fused filter kernel at the configured block shape (4 warps x 4
 * words, 512-row tiles, unless GX_WARPS / GX_WORDS say otherwise; never the
 * shape gx_plan_execute may pick online); the kernel's scratch (row-count,
 * ticket and error words plus one status word per tile) comes from a fixed
 * 4 MiB array in the library's device memory that every GPU loading the library
 * keeps until the process exits.
 *
 * - out[i].data, out[i].null_mask and out[i].capacity must be set by the
 *   caller; null_mask must hold ((capacity + 511) / 512) * 64 bytes (>= 64).
 * - Batches needing more than GX_NOALLOC_MAX_TILES tiles (more than
 *   268,433,408 rows with the default 512-row tile) are rejected with
 *   GX_ERR_INVALID.  When the selected rows exceed the outputs' capacity the
 *   call returns GX_ERR_CAPACITY with the needed count in *out_rows and writes
 *   nothing past the buffers.
 * - The call waits for its stream to finish the batch before it returns (it
 *   reads the row count back into host memory of its own stack frame).
 * - All calls share the one array (it keeps the last call's contents and is
 *   cleared at the start of each call), so calls whose work overlaps on the
 *   GPU -- on different streams or host threads at the same time -- race:
 *   serialise them.
 * - The first call on each device does set-up: it looks up the array's device
 *   address and compiles/loads the plan's kernel if no earlier call did.  Make
 *   that first call before any stream capture. */
#define GX_NOALLOC_MAX_TILES 524284
int gx_plan_execute_noalloc(const gx_plan* plan, const gx_column_view* columns, int num_columns,
                            gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status);

/* Runs the plan from host memory to host memory.  No counterpart in the
 * reference, whose tables are already on the device when the evaluator runs.
 *
 * columns[i].data / null_mask are host pointers (offset 0; pinned memory
 * gives the full copy bandwidth, pageable memory works at a lower rate);
 * out[i].data / null_mask are caller host buffers holding out[i].capacity
 * rows (null_mask: (capacity + 31) / 32 words).  A filter plan whose outputs
 * are all computed per row runs as a pipeline of row chunks (at least 2^22
 * rows, at most 64 chunks): each chunk's inputs are copied up on one copy
 * stream, its kernel runs on `stream` once they are in, and its output rows
 * are copied down on another copy stream as soon as its row count is known,
 * so copies in, kernels and copies out overlap.  Other plans copy in, run and
 * copy out.  Returns once the outputs are in host memory; GX_ERR_CAPACITY (and
 * the needed count in *out_rows) when the host buffers are too small.
 * Per-thread copy streams and a small pinned block are made on a thread's
 * first call and kept. */
int gx_plan_execute_host(const gx_plan* plan, const gx_column_view* columns, int num_columns,
                         gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status);

void gx_plan_destroy(gx_plan* plan);

/* ---- fused filter + group-by aggregation ---------------------------------
 *
 * The aggregation step of a Filter -> Projection -> Aggregate chain in one
 * device pass: ral::operators::compute_aggregations_with_groupby
 * (engine/src/operators/GroupBy.cpp:316-416), or compute_aggregations_without_groupby
 * (GroupBy.cpp:217-314) when there are no group columns, applied to the rows of
 * `columns` that pass `condition`, with each aggregation input expression
 * (what the reference evaluates through evaluate_expressions,
 * GroupBy.cpp:246-250 / :348-352) computed in the same pass.  No column of
 * the filtered table or of the aggregation inputs is materialised.
 *
 * - group_columns: input column indices of the keys (integer, BOOL8,
 *   timestamp or duration columns); NULL keys form their own group
 *   (cudf::null_policy::INCLUDE, GroupBy.cpp:380).
 * - agg_inputs[i]: a RexNode expression over the input columns, or "" for
 *   COUNT(*) (GX_AGG_COUNT_ALL).
 * - Output: out[0 .. num_group_columns) the key columns (their input types),
 *   then out[num_group_columns + i] aggregation i.  Types: COUNT -> INT64;
 *   SUM / SUM0 -> INT64 for an integer input, FLOAT64 for a floating one (the
 *   widening of GroupBy.cpp:33-40); MIN / MAX -> the input expression's type;
 *   MEAN -> FLOAT64.  SUM / MIN / MAX / MEAN of a group without a valid input
 *   are NULL; SUM0 is 0 there (GroupBy.cpp:394-397); COUNT_VALID counts valid
 *   inputs, COUNT_ALL rows.  Integer sums wrap (two's complement).
 * - With group columns the groups come out in no particular order (as the
 *   reference's hash group-by); *out_groups receives their number.  Without
 *   group columns there is exactly one output row, empty input included.
 * - Floating-point sums and means add in an order that depends on the GPU's
 *   scheduling (as cudf's hash aggregation does): results agree with a
 *   sequential sum to rounding, not bit for bit.  Everything else is exact. */
typedef enum gx_agg_kind {
  GX_AGG_SUM = 0, GX_AGG_SUM0 = 1, GX_AGG_MIN = 2, GX_AGG_MAX = 3,
  GX_AGG_COUNT_VALID = 4, GX_AGG_COUNT_ALL = 5, GX_AGG_MEAN = 6
} gx_agg_kind;

#define GX_AGG_MAX_KEYS 8
#define GX_AGG_MAX_AGGS 24

int gx_filter_aggregate(const gx_column_view* columns, int num_columns, const char* condition,
                        const int* group_columns, int num_group_columns, const char* const* agg_inputs,
                        const int* agg_kinds, int num_aggs, gx_column* out, int64_t* out_groups, void* stream,
                        gx_status_info* status);

/* Builds the aggregation kernel of a gx_filter_aggregate call for a column
 * schema (types, which columns carry a mask) and compiles it with NVRTC (no
 * GPU needed); registers, spill bytes and static shared memory per thread /
 * block from ptxas (each may be NULL). */
int gx_debug_aggregate_check(const int32_t* column_types, const uint8_t* column_has_mask, int num_columns,
                             const char* condition, const int* group_columns, int num_group_columns,
                             const char* const* agg_inputs, const int* agg_kinds, int num_aggs, int32_t* registers,
                             int32_t* spill_bytes, int32_t* shared_bytes, gx_status_info* status);

/* ---- skip-data: row groups a TableScan's condition can skip ---------------
 *
 * ral::skip_data::process_skipdata_for_table (engine/src/skip_data/
 * SkipDataProcessor.cpp:252-350).  `metadata` is the table of row-group
 * statistics with its column names: "min_<i>_<name>" / "max_<i>_<name>" per
 * input column i that has statistics, and as its last two columns the file
 * handle index and the row-group index.  column_names are the scanned
 * table's column names.  The scan's condition=[..] (or filters=[..]) over its
 * projects=[[..]] columns is restated over the statistics (a comparison over
 * a column becomes one over its min and max; operators that cannot be
 * restated are removed, an AND keeping its other side) and evaluated on the
 * GPU over the metadata rows.  out[0], out[1] receive the two id columns of
 * the row groups that may hold matching rows; *unusable is 1 (and out empty)
 * when the condition allows no pruning (read every row group), as the
 * reference's `true` result. */
int gx_skip_data_filter(const gx_column_view* metadata, const char* const* metadata_names, int num_metadata_columns,
                        const char* const* column_names, int num_columns, const char* table_scan, gx_column* out,
                        int64_t* out_rows, int* unusable, void* stream, gx_status_info* status);

/* The statistics form of a condition alone (no GPU): columns listed in
 * dropped_columns have no statistics; buf receives the rewritten condition
 * text, or with prefix_form the reference's prefix notation of the tree
 * (as its tests print it); *usable is 0 when nothing usable is left. */
int gx_skip_data_rewrite(const char* condition, const int* dropped_columns, int num_dropped, int prefix_form,
                         char* buf, int buf_len, int* usable, gx_status_info* status);

/* ---- batch runner: many batches, one persistent launch (no counterpart in
 * the reference) -------------------------------------------------------------
 *
 * The batched execution graph calls the filter once per batch
 * (engine/src/execution_kernels/BatchProcessing.cpp:371-476); each call of the
 * reference interpreter allocates, uploads, launches and synchronises
 * (engine/src/Interpreter/interpreter_cpp.cu:440-594), which dominates batches
 * of a few thousand rows.  A batch runner takes a whole table of batches of one
 * plan and runs them with one persistent kernel whose blocks take tiles from
 * every batch in turn, replayed from a captured CUDA graph (descriptor upload,
 * scratch and mask clear, kernel, row-count readback).  Each batch's output is
 * exactly what gx_plan_execute returns for it alone.  With autotune set, the
 * first run of at least 2^20 rows times a few block shapes (threads per block
 * x 32-row words per warp) on that run's batches and keeps the fastest, cached
 * per plan, column mix and device (and in $GX_AUTOTUNE_CACHE/gx_autotune.txt
 * when that variable names a directory).  A runner is not reentrant: one run
 * at a time. */
typedef struct gx_batch_runner gx_batch_runner;

/* plan: a compiled filter plan (condition + at most 32 outputs, at most 64
 * columns); a run takes at
 * most max_batches batches of max_total_rows rows in all. */
gx_batch_runner* gx_batch_runner_create(const gx_plan* plan, int max_batches, int64_t max_total_rows, int autotune,
                                        gx_status_info* status);

/* columns: num_batches x num_columns views, batch-major; out: num_batches x
 * num_outputs columns, batch-major (caller buffers when out[0].data is set,
 * else library-owned columns sharing one allocation, each released by
 * gx_free_columns); out_rows[b]: batch b's surviving rows. */
int gx_batch_runner_run(gx_batch_runner* runner, const gx_column_view* columns, int num_batches, int num_columns,
                        gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status);

/* The block shape in use (after autotuning). */
int gx_batch_runner_config(const gx_batch_runner* runner, int32_t* block_threads, int32_t* words_per_warp);
void gx_batch_runner_destroy(gx_batch_runner* runner);

/* ---- batch stream: a persistent kernel fed while it runs ------------------
 *
 * The batched execution graph hands the Filter kernel batches one by one as
 * they come out of the previous kernel (engine/src/execution_kernels/
 * BatchProcessing.cpp:371-476, run by execution_graph/executor.cpp:217-255);
 * the reference launches the interpreter per batch.  A batch stream keeps one
 * persistent kernel running per plan: gx_batch_stream_start launches it and it
 * waits for work; each gx_batch_stream_push hands it one more batch (its
 * descriptor and tile offsets are copied to the device, then its tiles are
 * published, by ordered asynchronous copies on a side stream -- no host
 * synchronisation), and the kernel's blocks take the new tiles as they
 * appear; gx_batch_stream_finish closes the queue, waits for the kernel and
 * returns every batch's output, each exactly what gx_plan_execute returns for
 * it alone.  A pushed batch's columns must stay valid until finish.  The
 * kernel gives up after waiting about 8 s for a batch that does not come
 * (finish then returns GX_ERR_TIMEOUT).  One session at a time per stream
 * object.  No counterpart in the reference. */
typedef struct gx_batch_stream gx_batch_stream;

/* plan: a compiled filter plan (condition, at most 32 outputs, at most 64
 * columns, no literal
 * outputs); a session takes at most max_batches batches of max_total_rows rows
 * in all; block_threads / words_per_warp: the kernel's block shape (0: the
 * plan's). */
gx_batch_stream* gx_batch_stream_create(const gx_plan* plan, int max_batches, int64_t max_total_rows,
                                        int block_threads, int words_per_warp, gx_status_info* status);
/* Starts a session: launches the kernel on `stream`. */
int gx_batch_stream_start(gx_batch_stream* st, void* stream, gx_status_info* status);
/* Appends one batch (num_columns views); *batch_index: its position. */
int gx_batch_stream_push(gx_batch_stream* st, const gx_column_view* columns, int num_columns, int* batch_index,
                         gx_status_info* status);
/* Closes the session: out receives num_outputs columns per pushed batch,
 * batch-major (library-owned views of one allocation, each released by
 * gx_free_columns), out_rows[b] batch b's surviving rows; max_batches: the
 * batches `out` / `out_rows` have room for. */
int gx_batch_stream_finish(gx_batch_stream* st, gx_column* out, int64_t* out_rows, int max_batches,
                           gx_status_info* status);
void gx_batch_stream_destroy(gx_batch_stream* st);
/* Test hook: the polls (about 2 us apart) the kernel waits for a batch before
 * it gives up (default 2^22). */
int gx_debug_batch_stream_wait_polls(gx_batch_stream* st, uint32_t polls);

/* ---- learned conjunct ordering (no counterpart in the reference) ---------
 *
 * A learner wraps a compiled filter plan (condition = AND of side-effect-free
 * conjuncts, at most 16) for a stream of batches of one schema, as the batched
 * execution graph's Filter kernel produces them (BatchProcessing.cpp:371-476).
 * Per batch it sketches every column (min, max, 8-bin histogram, null
 * fraction of a sample of 32-row words), predicts each conjunct's selectivity
 * with a small FP32 MLP (features -> 64 -> 64 -> conjuncts), evaluates the
 * conjuncts in predicted order with per-word short-circuit in one fused pass
 * into outputs sized from the predicted row count, and re-runs with the exact
 * count when the prediction was too small.  The plain fixed-order two-pass
 * evaluator runs the warm-up batches and every relabel_every-th batch after;
 * its per-conjunct pass counts are the training labels, and the network is
 * trained on the GPU after each of them.  Output is bit-identical to
 * gx_plan_execute with the same plan whatever the policy or prediction. */
typedef struct gx_learner gx_learner;

enum {
  GX_LEARN_POLICY_LEARNED = 0, /* network order + predicted capacity (warm-up / relabel on the plain path) */
  GX_LEARN_POLICY_PLAIN = 1,   /* always the plain fixed-order two-pass path */
  GX_LEARN_POLICY_TEXTUAL = 2  /* single pass, conjuncts short-circuited in textual order, full capacity */
};

typedef struct gx_learner_options {
  int32_t policy;          /* GX_LEARN_POLICY_* */
  int32_t warmup_batches;  /* plain labelled batches before the network is used (default 8) */
  int32_t relabel_every;   /* later batches: every n-th runs the plain path and trains (default 8; 0 never) */
  int32_t train_steps;     /* Adam steps per labelled batch (default 16) */
  float learning_rate;     /* default 3e-3 */
  int32_t hidden;          /* hidden width (default 64, at most 256) */
  double capacity_margin;  /* rows allocated = predicted rows x margin + slack (default 1.5) */
  int64_t capacity_slack;  /* default 4096 */
  int64_t sketch_stride_words; /* sketch every n-th 32-row word (default 256) */
  int32_t async_training;  /* 1: train on a side stream, overlapped with later batches */
  int32_t fast_words_per_warp; /* 32-row words per warp of the single-pass kernel (0: the plan's) */
  uint64_t seed;           /* parameter initialisation */
  int32_t size_outputs;    /* 1 (default): read the prediction back and allocate outputs of the predicted
                              size (one extra host round trip per batch); 0: the kernel takes the order
                              from device memory right after the prediction, outputs have full size */
  int32_t reserved;
} gx_learner_options;

/* Per-batch report of gx_learner_execute. */
typedef struct gx_learned_batch_info {
  int32_t path;             /* 0 plain two-pass (labelled), 1 single pass */
  int32_t reruns;           /* single-pass re-runs after an output-size misprediction */
  int64_t rows;
  int64_t predicted_rows;
  float train_loss;         /* loss of the latest finished training round */
  int32_t num_conjuncts;
  int32_t order[16];        /* evaluation order used (single pass) */
  double predicted_sel[16]; /* network's selectivity per conjunct (single pass) */
  double measured_sel[16];  /* plain path's measured selectivity per conjunct (path 0) */
} gx_learned_batch_info;

void gx_learner_options_init(gx_learner_options* options);

/* Creates a learner for a plan made by gx_plan_compile (with a condition, at
 * most 32 outputs and at most 64 columns).  The plan may be destroyed afterwards. */
gx_learner* gx_learner_create(const gx_plan* plan, const gx_learner_options* options, gx_status_info* status);

/* Filters one batch; same arguments and output contract as gx_plan_execute
 * (library-allocated outputs when out[0].data is NULL).  info may be NULL. */
int gx_learner_execute(gx_learner* learner, const gx_column_view* columns, int num_columns, gx_column* out,
                       int64_t* out_rows, gx_learned_batch_info* info, void* stream, gx_status_info* status);

/* Optional look-ahead for a stream of batches: sketches a batch that a later
 * gx_learner_execute call will receive, and runs the network on it, on the
 * learner's side stream (after `stream` reaches this point, so the columns may
 * still be being produced there).  Call it for batch b+1 before executing batch
 * b: the next call then finds its prediction ready instead of computing it on
 * its critical path.  A prepared batch is recognised by its column pointers,
 * offsets and row count; two may be pending at a time. */
int gx_learner_prepare(gx_learner* learner, const gx_column_view* columns, int num_columns, void* stream,
                       gx_status_info* status);

/* A queue of batches in one call: gx_learner_execute on batches[0] …
 * batches[num_batches-1] in order (each num_columns views), each next batch
 * prepared (as gx_learner_prepare) while the current one runs.  out holds
 * (plan outputs) columns per batch, batch-major, all with data == NULL on
 * entry (library-allocated, freed with gx_free_columns); out_rows and infos
 * (may be NULL) one entry per batch.  Every batch's columns are checked
 * against the plan before any batch runs.  On an error the message names the
 * failing batch; out_rows[b] stays -1 for every batch that did not complete,
 * and the outputs of those that did are valid and the caller's to free. */
int gx_learner_execute_batches(gx_learner* learner, const gx_column_view* const* batches, int num_columns,
                               int num_batches, gx_column* out, int64_t* out_rows, gx_learned_batch_info* infos,
                               void* stream, gx_status_info* status);

/* Network parameters to / from a file (the plan's shape must match). */
int gx_learner_save(const gx_learner* learner, const char* path, gx_status_info* status);
int gx_learner_load(gx_learner* learner, const char* path, gx_status_info* status);
void gx_learner_destroy(gx_learner* learner);

/* Library version / build information string. */
const char* gx_version(void);

/* ---- diagnostics (no counterpart in the reference) --------------------- */

/* Generated CUDA source of a plan kernel: kind 0 project, 1 fused single-pass
 * filter, 2 filter count pass, 3 filter write pass, 4 the learner's fused pass
 * (conjunct order given at launch), 5 the learner's labelling count pass
 * (per-conjunct pass counts), 6 the batch runner's persistent kernel, 7 the
 * learner's staged fused pass (conjunct columns copied to shared memory by TMA), 8 the tile-staged
 * single-pass filter (every column's tile copied to shared memory by bulk copies), 9 the batch
 * stream's persistent kernel.  Writes at most buf_len
 * bytes (NUL-terminated) and returns the full length, or -1 on error. */
int64_t gx_debug_kernel_source(const gx_plan* plan, int kind, const uint8_t* column_has_mask, char* buf,
                               int64_t buf_len, gx_status_info* status);

/* Compiles a plan kernel with NVRTC for sm_103a without loading it (no GPU
 * needed).  Returns GX_OK or GX_ERR_CUDA with the compiler log in status. */
int gx_debug_compile_check(const gx_plan* plan, int kind, const uint8_t* column_has_mask, gx_status_info* status);

/* Registers per thread, spill-store bytes and static shared memory of a plan
 * kernel as the assembler reports them for sm_103a (no GPU needed). */
int gx_debug_kernel_resources(const gx_plan* plan, int kind, const uint8_t* column_has_mask, int32_t* registers,
                              int32_t* spill_bytes, int32_t* shared_bytes, gx_status_info* status);

/* Host-side fault injection for tests: the n-th next device allocation made by
 * this library fails with GX_ERR_OOM (n <= 0 disables). */
void gx_debug_fail_allocation(int n);

/* Test of the bounded device waits, with no fault and no endless wait: runs a
 * single-pass filter plan over the columns (library outputs, released again)
 * with its tile ticket starting at first_tile, so tiles 0 .. first_tile-1 are
 * never claimed and never publish their look-back status, and with every
 * bounded wait giving up after spin_limit polls (0: the default).  With
 * first_tile >= 1 and more rows than first_tile tiles the look-backs of the
 * claimed tiles cannot finish: the kernel must return and the call report
 * GX_ERR_TIMEOUT, leaving the device usable. */
int gx_debug_filter_timeout(const gx_plan* plan, const gx_column_view* columns, int num_columns, int64_t first_tile,
                            uint32_t spin_limit, gx_status_info* status);

/* JIT statistics: number of NVRTC compilations and their total milliseconds. */
void gx_debug_jit_stats(int64_t* compiles, double* total_ms);

/* Kernel timing: when enabled, the main plan kernel of each call is bracketed
 * by CUDA events on the caller's stream; gx_debug_kernel_ms returns the summed
 * milliseconds of the calling thread since the last reset (the call
 * synchronises the stream when timing is on). */
void gx_debug_set_kernel_timing(int enable);
double gx_debug_kernel_ms(int reset);

/* Number of device kernels this library has launched (all threads). */
int64_t gx_debug_launch_count(void);

/* The text rewrites of preprocess_expression (engine/src/parser/expression_utils.cpp:1624-1632) on one
 * expression for a column schema, only those in `stages`: 1 unary minus, 2 CURRENT_DATE /
 * CURRENT_TIMESTAMP, 4 millisecond-to-nanosecond units, 8 Reinterpret casts, 16 interval units
 * (31: all, as every entry point applies them). */
int gx_debug_preprocess_expression(const char* expression, const int32_t* column_types, int num_columns, int stages,
                                   char* buf, int buf_len, gx_status_info* status);

/* Parses and lowers one RexNode expression (normalisation, AND/OR nesting,
 * CASE / ROUND / CAST-literal lowering) and writes it back as text, the way the
 * reference's parse_tree::rebuildExpression prints it. */
int gx_debug_rebuild_expression(const char* expression, char* buf, int buf_len, gx_status_info* status);

/* One forward + backward pass of the learner's MLP on the GPU, for checking
 * gradients: params (gx_learner MLP layout W1[H*F] b1[H] W2[H*H] b2[H] W3[O*H]
 * b3[O], row-major out x in), X[M*F], Y[M*O] are host arrays; writes the
 * gradient of loss = mean((log sigmoid(z) - Y)^2) into grad (same layout), the
 * loss and the outputs z[M*O].  M*H <= 4096, M*O <= 1024, H <= 256. */
/* The learner's sketch of one batch: ncols x 11 features (per column: min and
 * max of t / 16, the 8-bin histogram of t as cumulative fractions, the null
 * fraction; t = sign(d) log1p(|d|), d = value - anchor, on every
 * sketch_stride_words-th 32-row word), and optionally the per-column anchors
 * (doubles).  LEARNED policy only. */
int gx_debug_learner_features(gx_learner* learner, const gx_column_view* columns, int num_columns, float* features,
                              int max_features, int* num_features, double* anchors, void* stream,
                              gx_status_info* status);

int gx_debug_mlp_grad(int F, int H, int O, const float* params, const float* X, int M, const float* Y, float* grad,
                      float* loss, float* z, gx_status_info* status);

#ifdef __cplusplus
}
#endif

#endif /* GX_EVAL_H */
