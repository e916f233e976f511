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

#define GX_ABI_VERSION 1

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
  const void* data;         /* device memory */
  const uint32_t* null_mask;/* device memory or NULL */
  int64_t offset;           /* in elements */
  int64_t size;             /* rows */
} gx_column_view;

typedef struct gx_column {
  int32_t type_id;
  int32_t reserved;
  void* data;               /* device memory owned by this library */
  uint32_t* null_mask;      /* device memory owned by this library, always present */
  int64_t size;             /* rows */
  int64_t capacity;         /* rows the buffers can hold (>= size) */
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

/* Releases columns returned by this library (stream-ordered). */
void gx_free_columns(gx_column* columns, int num_columns, void* stream);

/* Copies a column's first `size` rows and its mask words to host memory. */
int gx_column_to_host(const gx_column* column, void* host_data, uint32_t* host_mask,
                      void* stream, gx_status_info* status);

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
 * accepted. */
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

/* Runs a filter plan (condition required, at most 32 outputs) into the
 * caller's buffers without allocating any device memory.  No counterpart in
 * the reference.
 *
 * For callers that cannot allocate device memory while they evaluate a batch:
 * an engine whose own memory pool owns the whole device budget (allocations
 * made outside it break its accounting, and fail once it has reserved the
 * rest of the GPU), or a per-batch path that must not enter an allocator.
 * Same kernel and results as gx_plan_execute in GX_FILTER_SINGLE_PASS mode;
 * the kernel's scratch (row-count, ticket and error words plus one status word
 * per 1024-row tile) comes from a fixed 4 MiB array in the library's device
 * memory that every GPU loading the library keeps until the process exits.
 *
 * - out[i].data, out[i].null_mask and out[i].capacity must be set by the
 *   caller; null_mask must hold ((capacity + 511) / 512) * 64 bytes (>= 64).
 * - Batches needing more than GX_NOALLOC_MAX_TILES tiles (more than
 *   536,866,816 rows with the default tile) are rejected with GX_ERR_INVALID.
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

void gx_plan_destroy(gx_plan* plan);

/* Library version / build information string. */
const char* gx_version(void);

/* ---- diagnostics (no counterpart in the reference) --------------------- */

/* Generated CUDA source of a plan kernel: kind 0 project, 1 fused single-pass
 * filter, 2 filter count pass, 3 filter write pass.  Writes at most buf_len
 * bytes (NUL-terminated) and returns the full length, or -1 on error. */
int64_t gx_debug_kernel_source(const gx_plan* plan, int kind, const uint8_t* column_has_mask, char* buf,
                               int64_t buf_len, gx_status_info* status);

/* Compiles a plan kernel with NVRTC for sm_103a without loading it (no GPU
 * needed).  Returns GX_OK or GX_ERR_CUDA with the compiler log in status. */
int gx_debug_compile_check(const gx_plan* plan, int kind, const uint8_t* column_has_mask, gx_status_info* status);

/* Host-side fault injection for tests: the n-th next device allocation made by
 * this library fails with GX_ERR_OOM (n <= 0 disables). */
void gx_debug_fail_allocation(int n);

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

/* Parses and lowers one RexNode expression (normalisation, AND/OR nesting,
 * CASE / ROUND / CAST-literal lowering) and writes it back as text, the way the
 * reference's parse_tree::rebuildExpression prints it. */
int gx_debug_rebuild_expression(const char* expression, char* buf, int buf_len, gx_status_info* status);

#ifdef __cplusplus
}
#endif

#endif /* GX_EVAL_H */
