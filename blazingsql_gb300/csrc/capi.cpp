// capi.cpp -- extern "C" entry points of include/gx_eval.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <new>
#include <unordered_map>

#include "frontend.h"
#include "plan.h"
#include "runtime.h"
#include "aggregate.h"
#include "str_prepass.h"

namespace gx {
namespace {

void set_status(gx_status_info* st, int code, const char* msg) {
  if (!st) return;
  st->code = code;
  std::snprintf(st->message, sizeof st->message, "%s", msg ? msg : "");
}

template <class F>
int guarded(gx_status_info* st, F&& f) {
  try {
    f();
    set_status(st, GX_OK, "");
    return GX_OK;
  } catch (const Error& e) {
    set_status(st, e.code, e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_status(st, GX_ERR_OOM, "host allocation failed");
    return GX_ERR_OOM;
  } catch (const std::exception& e) {
    set_status(st, GX_ERR_INVALID, e.what());
    return GX_ERR_INVALID;
  }
}

int env_int(const char* name, int dflt) {
  const char* v = std::getenv(name);
  return (v && *v) ? std::atoi(v) : dflt;
}

KernelConfig default_config() {
  KernelConfig c;
  c.warps = env_int("GX_WARPS", 4);
  c.words = env_int("GX_WORDS", 4);
  c.tune_shape = !std::getenv("GX_WARPS") && !std::getenv("GX_WORDS");
  c.emulate_fp64 = env_int("GX_NATIVE_FP64", 0) == 0;
  c.native_f64_ops = env_int("GX_NATIVE_F64_OPS", -1);
  c.dense = env_int("GX_DENSE", 1) != 0;
  c.lazy_case = env_int("GX_LAZY_CASE", 1) != 0;
  c.max_regs = env_int("GX_MAX_REGS", 0);
  c.use_tma = env_int("GX_TMA", 0);  // opt-in until it beats the direct-load kernel
  c.tma_warps = env_int("GX_TMA_WARPS", c.tma_warps);
  c.tma_words = env_int("GX_TMA_WORDS", c.tma_words);
  c.stages = env_int("GX_TMA_STAGES", c.stages);
  return c;
}

// The columns a text reads ($k outside quoted literals) appended to *used,
// or, with map, the text with each $k renumbered to $map[k].
static std::string map_columns(const std::string& t, std::vector<int>* used, const std::vector<int>* map) {
  std::string r;
  bool quoted = false;
  for (size_t i = 0; i < t.size();) {
    const char c = t[i];
    if (c == '\'') {
      if (quoted && i + 1 < t.size() && t[i + 1] == '\'') {  // '' inside a literal
        r += "''";
        i += 2;
        continue;
      }
      quoted = !quoted;
    } else if (!quoted && c == '$' && i + 1 < t.size() && std::isdigit((unsigned char)t[i + 1])) {
      size_t j = i + 1;
      long k = 0;
      while (j < t.size() && std::isdigit((unsigned char)t[j]) && k < (1L << 30)) k = k * 10 + (t[j++] - '0');
      if (used) used->push_back((int)k);
      r += "$" + std::to_string(map && k < (long)map->size() && (*map)[k] >= 0 ? (*map)[k] : k);
      i = j;
      continue;
    }
    r += c;
    i++;
  }
  return r;
}

// One call's plans: expression lists longer than GX_OUTPUTS_PER_KERNEL run as
// several kernels (chunks), each writing its slice of the outputs.  A kernel
// binds at most GX_MAX_COLS columns: over a wider table each chunk binds only
// the columns its texts read (col_maps[c], renumbered in order), and chunks
// also end where one more output would pass that limit -- the reference
// splits its plans at 64 slots the same way (LogicalProject.cpp:906-922).
struct PlanSet {
  std::vector<std::shared_ptr<CompiledPlan>> chunks;
  std::vector<int> first_output;
  std::vector<std::vector<int>> col_maps;  // per chunk: the table columns it binds (empty: all)
  int num_outputs = 0;
  int num_conjuncts = 0;
  std::vector<int> output_types;

  bool binds_all() const {
    for (const auto& m : col_maps)
      if (!m.empty()) return false;
    return true;
  }
  // the views chunk c binds
  const std::vector<ColumnView>& chunk_cols(size_t c, const std::vector<ColumnView>& cols,
                                            std::vector<ColumnView>& sub) const {
    if (col_maps[c].empty()) return cols;
    sub.clear();
    for (int k : col_maps[c]) {
      if (k >= (int)cols.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
      sub.push_back(cols[k]);
    }
    return sub;
  }

  void execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows, cudaStream_t s) const {
    const bool caller_bufs = num_outputs > 0 && out[0].data != nullptr;
    int64_t rows = -1;
    size_t done = 0;
    std::vector<ColumnView> sub;
    try {
      for (size_t c = 0; c < chunks.size(); c++) {
        int64_t r = 0;
        chunks[c]->execute(chunk_cols(c, cols, sub), out + first_output[c], &r, s);
        done = c + 1;
        if (rows >= 0 && r != rows) fail(GX_ERR_CUDA, "chunks of one plan disagree on the row count");
        rows = r;
      }
    } catch (...) {
      if (!caller_bufs)  // release the outputs of the chunks that completed
        for (size_t c = 0; c < done; c++)
          for (size_t j = 0; j < chunks[c]->plan().outputs.size(); j++) free_column(out[first_output[c] + j], s);
      throw;
    }
    if (out_rows) *out_rows = rows < 0 ? 0 : rows;
  }
};

std::shared_ptr<PlanSet> make_plan_set(const std::vector<int>& schema, const std::vector<bool>& nullable,
                                       const std::string& cond, const std::vector<std::string>& exprs,
                                       bool rand_by_out, const KernelConfig& cfg, int mode, uint64_t seed) {
  auto ps = std::make_shared<PlanSet>();
  int rand_base = 0;
  const bool wide = schema.size() > (size_t)GX_MAX_COLS;
  std::vector<int> cond_cols;
  map_columns(cond, &cond_cols, nullptr);
  for (size_t i = 0; i < exprs.size() || (i == 0 && exprs.empty());) {
    // this chunk's outputs: at most GX_OUTPUTS_PER_KERNEL, and over a wide
    // table no more than keep its columns within GX_MAX_COLS
    std::vector<int> bound = cond_cols;
    size_t j = i;
    while (j < exprs.size() && j - i < (size_t)GX_OUTPUTS_PER_KERNEL) {
      std::vector<int> t = bound;
      map_columns(exprs[j], &t, nullptr);
      std::sort(t.begin(), t.end());
      t.erase(std::unique(t.begin(), t.end()), t.end());
      if (wide && j > i && t.size() > (size_t)GX_MAX_COLS) break;
      bound = std::move(t);
      j++;
    }
    std::vector<std::string> part(exprs.begin() + i, exprs.begin() + j);
    std::vector<int> col_map;
    std::vector<int> sub_schema = schema;
    std::vector<bool> sub_nullable = nullable;
    std::string sub_cond = cond;
    if (wide) {
      std::sort(bound.begin(), bound.end());
      bound.erase(std::unique(bound.begin(), bound.end()), bound.end());
      if (bound.empty()) bound.push_back(0);  // a column to carry the row count
      std::vector<int> renum(schema.size(), -1);
      sub_schema.clear();
      sub_nullable.clear();
      for (int k : bound) {
        if (k < 0 || k >= (int)schema.size()) fail(GX_ERR_PARSE, "column index out of range: $" + std::to_string(k));
        renum[k] = (int)sub_schema.size();
        sub_schema.push_back(schema[k]);
        sub_nullable.push_back(nullable[k]);
      }
      sub_cond = map_columns(cond, nullptr, &renum);
      for (auto& e : part) e = map_columns(e, nullptr, &renum);
      col_map = bound;
    }
    int used = 0;
    Plan p = build_plan(sub_schema, sub_nullable, sub_cond, part, false, rand_by_out, rand_base, &used);
    ps->col_maps.push_back(col_map);
    i = j;
    rand_base += used;
    p.rand_seed = seed;
    if (ps->chunks.empty()) ps->num_conjuncts = (int)p.conjuncts.size();
    for (const auto& o : p.outputs) ps->output_types.push_back(o.type);
    ps->first_output.push_back(ps->num_outputs);
    ps->num_outputs += (int)p.outputs.size();
    KernelConfig c = cfg;
    if (!c.conjunct_order.empty() && c.conjunct_order.size() != p.conjuncts.size())
      fail(GX_ERR_INVALID, "conjunct order must list every conjunct");
    ps->chunks.push_back(std::make_shared<CompiledPlan>(std::move(p), c, mode));
    if (exprs.empty()) break;
  }
  return ps;
}

// Host-side cache of compiled plans keyed by the call's text + schema, so the
// per-batch host work of the execution graph's many small batches is a lookup
// (the reference re-parses with std::regex on every batch).
class PlanCache {
 public:
  std::shared_ptr<PlanSet> get(const std::string& key) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = map_.find(key);
    if (it == map_.end()) return nullptr;
    lru_.splice(lru_.begin(), lru_, it->second.second);
    return it->second.first;
  }
  void put(const std::string& key, std::shared_ptr<PlanSet> p) {
    std::lock_guard<std::mutex> lk(mu_);
    if (map_.count(key)) return;
    lru_.push_front(key);
    map_[key] = {std::move(p), lru_.begin()};
    while (map_.size() > 256) {
      map_.erase(lru_.back());
      lru_.pop_back();
    }
  }

 private:
  std::mutex mu_;
  std::list<std::string> lru_;
  std::unordered_map<std::string, std::pair<std::shared_ptr<PlanSet>, std::list<std::string>::iterator>> map_;
};

PlanCache& cache() {
  static PlanCache c;
  return c;
}

std::string cache_key(const char* kind, const std::vector<ColumnView>& cols, const std::string& cond,
                      const std::vector<std::string>& exprs, const KernelConfig& cfg, int mode) {
  std::string k = kind;
  k += '|';
  for (const auto& c : cols) {
    k += std::to_string(c.type);
    k += c.mask ? 'n' : '-';
    k += ',';
  }
  k += '|' + cond + '|';
  for (const auto& e : exprs) {
    k += e;
    k += '\x1f';
  }
  k += '|' + std::to_string(cfg.warps) + ':' + std::to_string(cfg.words) + ':' + std::to_string(mode) + ':' +
       std::to_string(cfg.emulate_fp64) + std::to_string(cfg.dense) + std::to_string(cfg.lazy_case) + ':' +
       std::to_string(cfg.native_f64_ops) + ':' + std::to_string(cfg.max_regs) + ':' + std::to_string(cfg.use_tma) +
       ':' + std::to_string(cfg.tma_warps) + 'x' + std::to_string(cfg.tma_words) + 'x' + std::to_string(cfg.stages);
  return k;
}

std::shared_ptr<PlanSet> plan_for(const char* kind, const std::vector<ColumnView>& cols, const std::string& cond,
                                  const std::vector<std::string>& exprs, bool rand_by_out) {
  const KernelConfig cfg = default_config();
  const int mode = env_int("GX_FILTER_MODE", GX_FILTER_AUTO);
  const std::string key = cache_key(kind, cols, cond, exprs, cfg, mode);
  if (auto p = cache().get(key)) return p;
  std::vector<int> schema;
  std::vector<bool> nullable;
  for (const auto& c : cols) {
    schema.push_back(c.type);
    nullable.push_back(c.mask != nullptr);
  }
  auto ps = make_plan_set(schema, nullable, cond, exprs, rand_by_out, cfg, mode, 0);
  cache().put(key, ps);
  return ps;
}

std::vector<int> schema_of(const std::vector<ColumnView>& cols) {
  std::vector<int> s;
  for (const auto& c : cols) s.push_back(c.type);
  return s;
}

}  // namespace
}  // namespace gx

struct gx_plan {
  std::shared_ptr<gx::PlanSet> ps;
};

namespace gx {
// The compiled plan of a gx_plan with one kernel (at most GX_OUTPUTS_PER_KERNEL
// outputs), or null.
const CompiledPlan* single_chunk(const gx_plan* plan) {
  if (!plan || plan->ps->chunks.size() != 1 || !plan->ps->binds_all()) return nullptr;
  return plan->ps->chunks[0].get();
}
}  // namespace gx

using namespace gx;

extern "C" {

const char* gx_version(void) {
  static const char* v = "gx-eval 0.1 (sm_103a; NVRTC plan kernels; abi " "2" ")";
  return v;
}

void gx_plan_options_init(gx_plan_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->filter_mode = GX_FILTER_AUTO;
  o->use_tma = -1;
}

// The string pre-pass of one call: the columns it computed, released (stream
// ordered) when the call's work has been enqueued, unless an output took one.
struct StringPrepass {
  std::vector<gx_column> made;
  std::vector<StringOp> ops;
  std::vector<bool> defer;  // per op: made after the filter, for the kept rows only
  cudaStream_t s = nullptr;
  ~StringPrepass() {
    for (auto& c : made)
      if (c.data || c.null_mask) free_column(c, s);
  }
};

// A CASE condition of the pre-pass evaluated into a BOOL8 column.
static gx_column eval_condition(const std::vector<ColumnView>& cols, const std::string& text, cudaStream_t s) {
  auto ps = plan_for("eval", cols, "", {text}, false);
  gx_column out{};
  int64_t rows = 0;
  ps->execute(cols, &out, &rows, s);
  return out;
}

// String operators over string columns in `cond` / `exprs` become columns
// appended to `cols` (function_evaluator_transformer, LogicalProject.cpp:671-742).
// Under a filter, an operator whose column is read only as a whole output
// (and by nothing else: not the condition, another expression or another
// operator) is deferred: it is made after the filter for the kept rows alone,
// instead of for every row and then gathered.  The outputs are the same.
static void string_prepass(std::vector<ColumnView>& cols, std::string* cond, std::vector<std::string>& exprs,
                           StringPrepass& pp, bool filtering) {
  const std::vector<int> schema = schema_of(cols);
  std::vector<std::string> texts;
  if (cond) texts.push_back(*cond);
  texts.insert(texts.end(), exprs.begin(), exprs.end());
  std::vector<StringOp> ops;
  rewrite_string_ops(texts, schema, ops);
  if (ops.empty()) return;
  size_t i = 0;
  if (cond) *cond = texts[i++];
  for (auto& e : exprs) e = texts[i++];
  pp.ops = ops;
  pp.defer.assign(ops.size(), false);
  if (filtering) {
    std::vector<int> read;  // columns read other than as a whole output
    if (cond) map_columns(*cond, &read, nullptr);
    for (const auto& e : exprs)
      if (passthrough_column(e) < 0) map_columns(e, &read, nullptr);
    for (const auto& op : ops) {
      read.push_back(op.col);
      read.push_back(op.col2);
      read.insert(read.end(), op.more_cols.begin(), op.more_cols.end());
      map_columns(op.cond, &read, nullptr);
      map_columns(op.pos0, &read, nullptr);
      map_columns(op.pos1, &read, nullptr);
    }
    for (size_t k = 0; k < ops.size(); k++)
      pp.defer[k] = is_deferrable(ops[k]) &&
                    std::find(read.begin(), read.end(), (int)(schema.size() + k)) == read.end();
  }
  const cudaStream_t s = pp.s;
  pp.made = run_string_prepass(
      cols, ops, s, [s](const std::vector<ColumnView>& c, const std::string& t) { return eval_condition(c, t, s); },
      &pp.defer);
}

// evaluate_expressions / process_filter / filter + project over a table that
// may hold string columns.  The string pre-pass runs first.  Expressions that
// are a whole string column or string literal are string outputs: without a
// condition a string column is copied (the reference deep-copies `$i`
// outputs, LogicalProject.cpp:829, and moves a computed one, :885-887) and a
// literal repeated (:825); with a condition the plan kernel also writes each
// kept row's input row (GX_ROW_INDEX), and the string outputs are gathered
// through it (apply_boolean_mask's gather, LogicalFilter.cpp:22-29).  Every
// other expression runs in one plan kernel.
static void evaluate_with_strings(std::vector<ColumnView> cols, std::string cond, std::vector<std::string> ex,
                                  bool filtering, gx_column* out, int64_t* out_rows, cudaStream_t s,
                                  const char* kind, bool rand_by_out) {
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const size_t ncols0 = cols.size();
  StringPrepass pp;
  pp.s = s;
  string_prepass(cols, filtering ? &cond : nullptr, ex, pp, filtering);
  if (filtering) {
    const int c = passthrough_column(cond);
    if ((c >= 0 && c < (int)cols.size() && cols[c].type == STRING) || string_literal_value(cond, nullptr))
      fail(GX_ERR_TYPE, "the condition is a string");
  }
  // classify the outputs: -2 plan output, -1 string literal, >= 0 string column
  std::vector<int> src(ex.size(), -2);
  std::vector<std::string> lit(ex.size());
  std::vector<std::string> num;
  std::vector<int> num_pos;
  bool gather = false;
  for (size_t i = 0; i < ex.size(); i++) {
    const int c = passthrough_column(ex[i]);
    if (c >= 0 && c < (int)cols.size() && cols[c].type == STRING) {
      src[i] = c;
      gather |= filtering;
    } else if (string_literal_value(ex[i], &lit[i])) {
      src[i] = -1;
    } else {
      num.push_back(ex[i]);
      num_pos.push_back((int)i);
    }
  }
  // a filter whose outputs are all literals still needs its row count
  const bool row_index = filtering && (gather || num.empty());
  if (row_index) num.push_back("GX_ROW_INDEX()");
  std::vector<gx_column> tmp(num.size());
  for (auto& c : tmp) c = gx_column{};
  for (size_t i = 0; i < ex.size(); i++) out[i] = gx_column{};
  int64_t rows = n;
  try {
    if (!num.empty()) {
      auto ps = plan_for(kind, cols, filtering ? cond : std::string(), num, rand_by_out);
      ps->execute(cols, tmp.data(), &rows, s);
      for (size_t j = 0; j < num_pos.size(); j++) {
        out[num_pos[j]] = tmp[j];
        tmp[j] = gx_column{};
      }
    }
    const int32_t* map = row_index ? (const int32_t*)tmp.back().data : nullptr;
    for (size_t i = 0; i < ex.size(); i++) {
      if (src[i] == -2) continue;
      StrSource a, none;
      if (src[i] == -1) {
        a.kind = StrSource::LITERAL;
        a.literal = lit[i];
        out[i] = build_strings(a, none, nullptr, nullptr, rows, s);
        continue;
      }
      const size_t k = (size_t)src[i] - ncols0;
      if (src[i] >= (int)ncols0 && k < pp.defer.size() && pp.defer[k]) {  // made now, for the kept rows
        out[i] = transform_column(pp.ops[k], cols, filtering ? map : nullptr, rows, s,
                                  [s](const std::vector<ColumnView>& c, const std::string& t) {
                                    return eval_condition(c, t, s);
                                  });
        continue;
      }
      if (!filtering && src[i] >= (int)ncols0 && k < pp.made.size() && pp.made[k].data) {
        out[i] = pp.made[k];  // a computed string column moves to the output
        pp.made[k] = gx_column{};
        continue;
      }
      a.kind = StrSource::COLUMN;
      a.col = cols[src[i]];
      out[i] = build_strings(a, none, filtering ? map : nullptr, nullptr, rows, s);
    }
  } catch (...) {
    for (size_t i = 0; i < ex.size(); i++)
      if (out[i].data || out[i].null_mask) free_column(out[i], s);
    for (auto& c : tmp)
      if (c.data || c.null_mask) free_column(c, s);
    throw;
  }
  for (auto& c : tmp)
    if (c.data || c.null_mask) free_column(c, s);
  if (out_rows) *out_rows = rows;
}

int gx_evaluate_expressions(const gx_column_view* columns, int num_columns, const char* const* expressions,
                            int num_expressions, gx_column* out, void* stream, gx_status_info* status) {
  return guarded(status, [&] {
    if (num_expressions < 0 || (num_expressions > 0 && (!expressions || !out))) fail(GX_ERR_INVALID, "bad arguments");
    auto cols = to_views(columns, num_columns);
    std::vector<std::string> ex;
    for (int i = 0; i < num_expressions; i++) {
      if (!expressions[i]) fail(GX_ERR_INVALID, "null expression");
      ex.emplace_back(expressions[i]);
    }
    if (ex.empty()) return;
    evaluate_with_strings(cols, "", ex, false, out, nullptr, (cudaStream_t)stream, "eval", false);
  });
}

int gx_process_project(const gx_column_view* columns, int num_columns, const char* query_part, gx_column* out,
                       int max_out, int* num_out, char* out_names, int name_len, void* stream,
                       gx_status_info* status) {
  return guarded(status, [&] {
    if (!query_part || !out || !num_out) fail(GX_ERR_INVALID, "bad arguments");
    auto cols = to_views(columns, num_columns);
    std::vector<std::string> names, exprs;
    split_projections(query_part, names, exprs);
    if ((int)exprs.size() > max_out) fail(GX_ERR_INVALID, "output array too small for the projections");
    const std::vector<int> schema = schema_of(cols);
    for (auto& e : exprs) {
      if (e.find(" OVER ") != std::string::npos) fail(GX_ERR_UNSUPPORTED, "window functions are out of scope");
      e = preprocess_expression(e, schema);
    }
    if (!exprs.empty())
      evaluate_with_strings(cols, "", exprs, false, out, nullptr, (cudaStream_t)stream, "eval", false);
    *num_out = (int)exprs.size();
    if (out_names && name_len > 0)
      for (size_t i = 0; i < names.size(); i++)
        std::snprintf(out_names + i * name_len, (size_t)name_len, "%s", names[i].c_str());
  });
}

int gx_process_filter(const gx_column_view* columns, int num_columns, const char* query_part, gx_column* out,
                      int64_t* out_rows, void* stream, gx_status_info* status) {
  return guarded(status, [&] {
    if (!query_part || (num_columns > 0 && !out)) fail(GX_ERR_INVALID, "bad arguments");
    auto cols = to_views(columns, num_columns);
    const cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = cols.empty() ? 0 : cols[0].size;
    if (n == 0) {  // LogicalFilter.cpp:36-38: empty input -> empty_like, no parsing
      for (int i = 0; i < num_columns; i++) out[i] = gx_column{};
      try {
        for (int i = 0; i < num_columns; i++) {
          if (cols[i].type == STRING) {
            out[i] = build_strings(StrSource{}, StrSource{}, nullptr, nullptr, 0, s);
          } else {
            out[i] = alloc_column(cols[i].type, 0, s);
            launch_fill_mask(out[i].null_mask, 0, false, 16, s);
          }
        }
      } catch (...) {
        for (int i = 0; i < num_columns; i++)
          if (out[i].data || out[i].null_mask) free_column(out[i], s);
        throw;
      }
      if (out_rows) *out_rows = 0;
      return;
    }
    const std::string qp(query_part);
    std::string cond = named_expression(qp, "condition");
    if (cond.empty()) cond = named_expression(qp, "filters");
    if (cond.empty()) fail(GX_ERR_PARSE, "no condition=[...] or filters=[...] in: " + qp);
    cond = preprocess_expression(cond, schema_of(cols));
    // every input column compacted = the projections $0..$k-1 of the filtered rows
    std::vector<std::string> all;
    for (int i = 0; i < num_columns; i++) all.push_back("$" + std::to_string(i));
    evaluate_with_strings(cols, cond, all, true, out, out_rows, s, "filter", false);
  });
}

int gx_filter_project(const gx_column_view* columns, int num_columns, const char* condition,
                      const char* const* expressions, int num_expressions, gx_column* out, int64_t* out_rows,
                      void* stream, gx_status_info* status) {
  return guarded(status, [&] {
    if (num_expressions <= 0 || !expressions || !out) fail(GX_ERR_INVALID, "bad arguments");
    auto cols = to_views(columns, num_columns);
    const std::vector<int> schema = schema_of(cols);
    std::string cond = condition ? std::string(condition) : std::string();
    if (!cond.empty()) cond = preprocess_expression(cond, schema);
    std::vector<std::string> ex;
    for (int i = 0; i < num_expressions; i++) {
      if (!expressions[i]) fail(GX_ERR_INVALID, "null expression");
      ex.push_back(preprocess_expression(expressions[i], schema));
    }
    evaluate_with_strings(cols, cond, ex, !cond.empty(), out, out_rows, (cudaStream_t)stream, "fused", true);
  });
}

static std::shared_ptr<AggPlan> agg_plan_for(const std::vector<int>& schema, const std::vector<bool>& nullable,
                                             const char* condition, const int* group_columns, int nk,
                                             const char* const* agg_inputs, const int* agg_kinds, int na) {
  if (nk < 0 || na <= 0 || (nk > 0 && !group_columns) || !agg_inputs || !agg_kinds)
    fail(GX_ERR_INVALID, "bad aggregation arguments");
  std::string cond = condition ? std::string(condition) : std::string();
  if (!cond.empty()) cond = preprocess_expression(cond, schema);
  std::vector<int> keys(group_columns, group_columns + nk);
  std::vector<std::string> inputs;
  std::vector<int> kinds(agg_kinds, agg_kinds + na);
  for (int i = 0; i < na; i++) {
    const std::string e = agg_inputs[i] ? std::string(agg_inputs[i]) : std::string();
    inputs.push_back(e.empty() ? e : preprocess_expression(e, schema));
  }
  KernelConfig cfg = default_config();
  if (cfg.tune_shape) {
    // one-warp blocks of 8 words: each warp owns its block's group table, so
    // its shared-memory atomics meet no other warp's.  Measured on the Q1
    // shape (2^27 rows): 1 x 8 3.88 ms; 1 x 16 4.00; 2 x 8 4.02; 2 x 4 4.04;
    // 4 x 8 4.07; 4 x 4 4.10; 8 x 4 4.20; 8 x 2 4.45.
    cfg.warps = 1;
    cfg.words = 8;
  }
  std::string key;
  for (size_t i = 0; i < schema.size(); i++) key += std::to_string(schema[i]) + (nullable[i] ? "n," : "-,");
  key += "|" + cond + "|";
  for (int c : keys) key += std::to_string(c) + ",";
  key += "|";
  for (int i = 0; i < na; i++) key += std::to_string(kinds[i]) + ":" + inputs[i] + "\x1f";
  key += "|" + std::to_string(cfg.warps) + ":" + std::to_string(cfg.words) + ":" + std::to_string(cfg.native_f64_ops);
  const char* wc = std::getenv("GX_AGG_COMBINE");
  key += (wc && *wc == '0') ? ":direct" : ":combine";
  if (const char* kb = std::getenv("GX_AGG_SMEM_KB")) key += std::string(":smem") + kb;
  static std::mutex mu;
  static std::unordered_map<std::string, std::shared_ptr<AggPlan>> plans;
  {
    std::lock_guard<std::mutex> g(mu);
    auto it = plans.find(key);
    if (it != plans.end()) return it->second;
  }
  auto p = std::make_shared<AggPlan>(schema, nullable, cond, keys, inputs, kinds, cfg);
  std::lock_guard<std::mutex> g(mu);
  if (plans.size() > 256) plans.clear();
  plans[key] = p;
  return p;
}

int gx_filter_aggregate(const gx_column_view* columns, int num_columns, const char* condition,
                        const int* group_columns, int num_group_columns, const char* const* agg_inputs,
                        const int* agg_kinds, int num_aggs, gx_column* out, int64_t* out_groups, void* stream,
                        gx_status_info* status) {
  return guarded(status, [&] {
    if (!out) fail(GX_ERR_INVALID, "null output array");
    auto cols = to_views(columns, num_columns);
    std::vector<bool> nullable;
    for (const auto& c : cols) nullable.push_back(c.mask != nullptr);
    auto ap = agg_plan_for(schema_of(cols), nullable, condition, group_columns, num_group_columns, agg_inputs,
                           agg_kinds, num_aggs);
    for (int i = 0; i < ap->num_outputs(); i++) out[i] = gx_column{};
    ap->execute(cols, out, out_groups, (cudaStream_t)stream);
  });
}

int gx_debug_aggregate_check(const int32_t* column_types, const uint8_t* column_has_mask, int num_columns,
                             const char* condition, const int* group_columns, int num_group_columns,
                             const char* const* agg_inputs, const int* agg_kinds, int num_aggs, int32_t* registers,
                             int32_t* spill_bytes, int32_t* shared_bytes, gx_status_info* status) {
  return guarded(status, [&] {
    if (num_columns < 0 || (num_columns > 0 && !column_types)) fail(GX_ERR_INVALID, "bad column types");
    std::vector<int> schema(column_types, column_types + num_columns);
    std::vector<bool> nullable;
    for (int i = 0; i < num_columns; i++) nullable.push_back(column_has_mask ? column_has_mask[i] != 0 : true);
    auto ap = agg_plan_for(schema, nullable, condition, group_columns, num_group_columns, agg_inputs, agg_kinds,
                           num_aggs);
    const KernelResources r = jit_resources(ap->kernel_source(nullable), "gx_filter_aggregate");
    if (registers) *registers = r.registers;
    if (spill_bytes) *spill_bytes = r.spill_bytes;
    if (shared_bytes) *shared_bytes = r.shared_bytes;
  });
}

int gx_skip_data_rewrite(const char* condition, const int* dropped_columns, int num_dropped, int prefix_form,
                         char* buf, int buf_len, int* usable, gx_status_info* status) {
  return guarded(status, [&] {
    if (!condition || (num_dropped > 0 && !dropped_columns)) fail(GX_ERR_INVALID, "bad arguments");
    std::vector<int> dropped(dropped_columns, dropped_columns + std::max(num_dropped, 0));
    std::string prefix;
    const std::string text = skip_data_rewrite(condition, dropped, &prefix);
    if (usable) *usable = text.empty() ? 0 : 1;
    const std::string& r = prefix_form ? prefix : text;
    if (buf && buf_len > 0) std::snprintf(buf, (size_t)buf_len, "%s", r.c_str());
  });
}

int gx_skip_data_filter(const gx_column_view* metadata, const char* const* metadata_names, int num_metadata_columns,
                        const char* const* column_names, int num_columns, const char* table_scan, gx_column* out,
                        int64_t* out_rows, int* unusable, void* stream, gx_status_info* status) {
  return guarded(status, [&] {
    if (!metadata || !metadata_names || num_metadata_columns < 2 || !column_names || num_columns < 0 || !table_scan ||
        !out || !unusable)
      fail(GX_ERR_INVALID, "bad arguments");
    *unusable = 1;
    out[0] = gx_column{};
    out[1] = gx_column{};
    if (out_rows) *out_rows = 0;
    const std::string scan(table_scan);
    std::string cond = named_expression(scan, "condition");
    if (cond.empty()) cond = named_expression(scan, "filters");
    if (cond.empty()) return;  // no condition: every row group is read
    std::vector<int> projected;
    const std::string projects = named_expression(scan, "projects");
    if (projects.empty()) {
      for (int i = 0; i < num_columns; i++) projected.push_back(i);
    } else {
      for (const auto& item : split_expression_list(projects, true)) projected.push_back(std::stoi(item));
    }
    auto meta = to_views(metadata, num_metadata_columns);
    const int64_t rows = meta[0].size;
    auto find = [&](const std::string& name) {
      for (int i = 0; i < num_metadata_columns; i++)
        if (metadata_names[i] && name == metadata_names[i]) return i;
      return -1;
    };
    // [min, max] per projected column (a dummy pair for one without
    // statistics, dropped from the condition), then the two id columns
    std::vector<ColumnView> table;
    std::vector<int> dropped;
    void* dummy = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    for (size_t i = 0; i < projected.size(); i++) {
      const int c = projected[i];
      if (c < 0 || c >= num_columns || !column_names[c]) fail(GX_ERR_INVALID, "projected column out of range");
      const std::string suffix = std::to_string(c) + "_" + column_names[c];
      const int mn = find("min_" + suffix), mx = find("max_" + suffix);
      if (mn >= 0 && mx >= 0) {
        table.push_back(meta[mn]);
        table.push_back(meta[mx]);
      } else {
        dropped.push_back((int)i);
        if (!dummy) dummy = dev_alloc((size_t)std::max<int64_t>(rows, 1), s);
        table.push_back({INT8, dummy, nullptr, 0, rows});
        table.push_back({INT8, dummy, nullptr, 0, rows});
      }
    }
    const int id0 = (int)table.size();
    table.push_back(meta[num_metadata_columns - 2]);
    table.push_back(meta[num_metadata_columns - 1]);
    try {
      const std::string expr = skip_data_rewrite(cond, dropped, nullptr);
      if (!expr.empty()) {
        auto ps = plan_for("skipdata", table, expr, {"$" + std::to_string(id0), "$" + std::to_string(id0 + 1)}, false);
        ps->execute(table, out, out_rows, s);
        *unusable = 0;
      }
    } catch (...) {
      dev_free(dummy, s);
      throw;
    }
    dev_free(dummy, s);
  });
}

void gx_free_columns(gx_column* columns, int num_columns, void* stream) {
  if (!columns) return;
  for (int i = 0; i < num_columns; i++) free_column(columns[i], (cudaStream_t)stream);
}

int gx_column_to_host(const gx_column* column, void* host_data, uint32_t* host_mask, void* stream,
                      gx_status_info* status) {
  return guarded(status, [&] {
    if (!column) fail(GX_ERR_INVALID, "null column");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t bytes = column->type_id == STRING ? (size_t)column->string_bytes
                                                   : (size_t)column->size * type_size(column->type_id);
    if (bytes && host_data)
      check_cuda(cudaMemcpyAsync(host_data, column->data, bytes, cudaMemcpyDeviceToHost, s), "column to host");
    if (host_mask) {
      const size_t words = (size_t)((column->size + 31) / 32);
      if (words)
        check_cuda(cudaMemcpyAsync(host_mask, column->null_mask, words * 4, cudaMemcpyDeviceToHost, s), "mask to host");
    }
    check_cuda(cudaStreamSynchronize(s), "column to host sync");
  });
}

int gx_debug_like_automaton(const char* pattern, const char* text, int64_t text_len, int32_t* result,
                            gx_status_info* status) {
  return guarded(status, [&] {
    if (!pattern || (!text && text_len > 0) || text_len < 0 || !result) fail(GX_ERR_INVALID, "bad arguments");
    *result = like_dfa_host_match(pattern, (const unsigned char*)text, text_len);
  });
}

int gx_string_offsets_to_host(const gx_column* column, int32_t* host_offsets, void* stream,
                              gx_status_info* status) {
  return guarded(status, [&] {
    if (!column || !host_offsets) fail(GX_ERR_INVALID, "null argument");
    if (column->type_id != STRING || !column->string_offsets) fail(GX_ERR_TYPE, "not a string column");
    cudaStream_t s = (cudaStream_t)stream;
    check_cuda(cudaMemcpyAsync(host_offsets, column->string_offsets, (size_t)(column->size + 1) * 4,
                               cudaMemcpyDeviceToHost, s),
               "offsets to host");
    check_cuda(cudaStreamSynchronize(s), "offsets to host sync");
  });
}

gx_plan* gx_plan_compile(const int32_t* column_types, const uint8_t* column_nullable, int num_columns,
                         const char* condition, const char* const* expressions, int num_expressions,
                         const gx_plan_options* options, gx_status_info* status) {
  gx_plan* out = nullptr;
  guarded(status, [&] {
    if (num_columns < 0 || (num_columns > 0 && !column_types)) fail(GX_ERR_INVALID, "bad schema");
    std::vector<int> schema(column_types, column_types + num_columns);
    std::vector<bool> nullable(num_columns, true);
    if (column_nullable)
      for (int i = 0; i < num_columns; i++) nullable[i] = column_nullable[i] != 0;
    gx_plan_options o;
    gx_plan_options_init(&o);
    if (options) o = *options;
    std::string cond = condition ? std::string(condition) : std::string();
    if (!cond.empty()) cond = preprocess_expression(cond, schema);
    std::vector<std::string> ex;
    for (int i = 0; i < num_expressions; i++) ex.push_back(preprocess_expression(expressions[i], schema));
    KernelConfig cfg = default_config();
    if (o.block_threads > 0) cfg.warps = o.block_threads / 32;
    if (o.words_per_warp > 0) cfg.words = o.words_per_warp;
    if (o.block_threads > 0 || o.words_per_warp > 0) cfg.tune_shape = false;
    cfg.short_circuit = o.short_circuit != 0;
    if (o.use_tma == 0 || o.use_tma == 1) cfg.use_tma = o.use_tma;
    for (int i = 0; i < o.num_conjuncts && i < 16; i++) {
      if (o.conjunct_order[i] < 0 || o.conjunct_order[i] >= 16) fail(GX_ERR_INVALID, "conjunct order index out of range");
      cfg.conjunct_order.push_back(o.conjunct_order[i]);
    }
    if (!cfg.conjunct_order.empty()) {
      std::vector<int> sorted = cfg.conjunct_order;
      std::sort(sorted.begin(), sorted.end());
      for (size_t i = 0; i < sorted.size(); i++)
        if (sorted[i] != (int)i) fail(GX_ERR_INVALID, "conjunct order must be a permutation");
    }
    out = new gx_plan{make_plan_set(schema, nullable, cond, ex, true, cfg, o.filter_mode, o.rand_seed)};
  });
  return out;
}

int gx_plan_num_outputs(const gx_plan* plan) { return plan ? plan->ps->num_outputs : -1; }

int32_t gx_plan_output_type(const gx_plan* plan, int index) {
  if (!plan || index < 0 || index >= plan->ps->num_outputs) return -1;
  return plan->ps->output_types[index];
}

int gx_plan_num_conjuncts(const gx_plan* plan) { return plan ? plan->ps->num_conjuncts : -1; }

int gx_plan_execute(const gx_plan* plan, const gx_column_view* columns, int num_columns, gx_column* out,
                    int64_t* out_rows, void* stream, gx_status_info* status) {
  return guarded(status, [&] {
    if (!plan || !out) fail(GX_ERR_INVALID, "bad arguments");
    auto cols = to_views(columns, num_columns);
    plan->ps->execute(cols, out, out_rows, (cudaStream_t)stream);
  });
}

int gx_plan_execute_host(const gx_plan* plan, const gx_column_view* host_columns, int num_columns,
                         gx_column* host_out, int64_t* out_rows, void* stream, gx_status_info* status) {
  return guarded(status, [&] {
    if (!plan || !host_out) fail(GX_ERR_INVALID, "bad arguments");
    auto cols = to_views(host_columns, num_columns);
    // a plan of more than one kernel (over 32 outputs) runs each one in turn
    const PlanSet& ps = *plan->ps;
    int64_t rows = -1;
    std::vector<ColumnView> sub;
    for (size_t c = 0; c < ps.chunks.size(); c++) {
      int64_t r = 0;
      try {
        ps.chunks[c]->execute_host(ps.chunk_cols(c, cols, sub), host_out + ps.first_output[c], &r,
                                   (cudaStream_t)stream);
      } catch (const Error& e) {
        if (out_rows && e.code == GX_ERR_CAPACITY) *out_rows = r;  // the count the buffers need
        throw;
      }
      if (rows >= 0 && r != rows) fail(GX_ERR_CUDA, "chunks of one plan disagree on the row count");
      rows = r;
    }
    if (out_rows) *out_rows = rows < 0 ? 0 : rows;
  });
}

void gx_plan_destroy(gx_plan* plan) { delete plan; }

static KernelKind kind_of(int k) {
  switch (k) {
    case 0: return KernelKind::PROJECT;
    case 1: case 4: return KernelKind::FUSED_FILTER;
    case 2: case 5: return KernelKind::COUNT_FILTER;
    case 3: return KernelKind::WRITE_FILTER;
    case 6: return KernelKind::FUSED_BATCHED;
    case 7: return KernelKind::FUSED_STAGED;
    case 8: return KernelKind::FUSED_TMA;
    case 9: return KernelKind::FUSED_STREAM;
    default: fail(GX_ERR_INVALID, "kernel kind must be 0..9");
  }
}

// kinds 4 and 5 are the learner's variants: the fused pass with the conjunct
// order taken at launch, and the count pass with per-conjunct pass counts
static std::string debug_source(const gx_plan* plan, int kind, const uint8_t* has_mask) {
  if (!plan) fail(GX_ERR_INVALID, "null plan");
  if (!plan->ps->binds_all()) fail(GX_ERR_UNSUPPORTED, "diagnostics of a plan over more than 64 columns");
  Plan p = plan->ps->chunks.at(0)->plan();
  for (size_t i = 0; i < p.nullable.size(); i++) p.nullable[i] = has_mask ? has_mask[i] != 0 : true;
  KernelConfig cfg = plan->ps->chunks.at(0)->config();
  if (kind == 4 || kind == 5 || kind == 7) {
    cfg.short_circuit = false;
    cfg.conjunct_order.clear();
    cfg.runtime_order = kind == 4 || kind == 7;
    cfg.staged = kind == 7;
    if (kind == 4) {  // as the learner builds it
      const char* st = std::getenv("GX_STREAM");
      cfg.stream_slots = st && *st ? std::atoi(st) : 0;
    }
    cfg.conj_stats = kind == 5;
    if (kind == 4 || kind == 7) cfg.dense = true;
  }
  if (kind == 8) {  // the tile-staged kernel at the plan's configured shape
    cfg.warps = cfg.tma_warps;
    cfg.words = cfg.tma_words;
  }
  return generate_kernel(p, kind_of(kind), cfg, "gx_kernel");
}

int64_t gx_debug_kernel_source(const gx_plan* plan, int kind, const uint8_t* column_has_mask, char* buf,
                               int64_t buf_len, gx_status_info* status) {
  int64_t n = -1;
  guarded(status, [&] {
    const std::string s = std::string(jit_prelude()) + "\n" + debug_source(plan, kind, column_has_mask);
    n = (int64_t)s.size();
    if (buf && buf_len > 0) std::snprintf(buf, (size_t)buf_len, "%s", s.c_str());
  });
  return n;
}

int gx_debug_compile_check(const gx_plan* plan, int kind, const uint8_t* column_has_mask, gx_status_info* status) {
  return guarded(status, [&] { jit_compile_check(debug_source(plan, kind, column_has_mask), "gx_kernel"); });
}

int gx_debug_kernel_resources(const gx_plan* plan, int kind, const uint8_t* column_has_mask, int32_t* registers,
                              int32_t* spill_bytes, int32_t* shared_bytes, gx_status_info* status) {
  return guarded(status, [&] {
    const KernelResources r = jit_resources(debug_source(plan, kind, column_has_mask), "gx_kernel");
    if (registers) *registers = r.registers;
    if (spill_bytes) *spill_bytes = r.spill_bytes;
    if (shared_bytes) *shared_bytes = r.shared_bytes;
  });
}

void gx_debug_fail_allocation(int n) { debug_fail_allocation(n); }

int gx_debug_filter_timeout(const gx_plan* plan, const gx_column_view* columns, int num_columns, int64_t first_tile,
                            uint32_t spin_limit, gx_status_info* status) {
  return guarded(status, [&] {
    if (!plan || !plan->ps->binds_all()) fail(GX_ERR_INVALID, "null plan or a plan over more than 64 columns");
    const CompiledPlan& cp = *plan->ps->chunks.at(0);
    if (!cp.plan().has_filter()) fail(GX_ERR_INVALID, "the wait test runs a filter plan");
    auto cols = to_views(columns, num_columns);
    std::vector<gx_column> out(cp.plan().outputs.size());
    for (auto& c : out) std::memset(&c, 0, sizeof c);
    ExecExtras ex;
    ex.first_tile = first_tile;
    ex.spin_limit = spin_limit;
    int64_t rows = 0;
    cp.execute(cols, out.data(), &rows, nullptr, &ex);
    // reached only when no wait gave up: release the outputs
    for (auto& c : out) free_column(c, nullptr);
    cudaStreamSynchronize(nullptr);
  });
}

void gx_debug_set_kernel_timing(int enable) { set_kernel_timing(enable != 0); }

double gx_debug_kernel_ms(int reset) { return kernel_ms(reset != 0); }

int64_t gx_debug_launch_count(void) { return launch_count(); }

int gx_set_current_timestamp(const char* timestamp, gx_status_info* status) {
  return guarded(status, [&] { set_current_timestamp(timestamp ? std::string(timestamp) : std::string()); });
}

int gx_debug_preprocess_expression(const char* expression, const int32_t* column_types, int num_columns, int stages,
                                   char* buf, int buf_len, gx_status_info* status) {
  return guarded(status, [&] {
    if (!expression || !buf || buf_len <= 0 || num_columns < 0 || (num_columns > 0 && !column_types))
      fail(GX_ERR_INVALID, "bad arguments");
    std::vector<int> schema(column_types, column_types + num_columns);
    std::snprintf(buf, (size_t)buf_len, "%s", preprocess_stages(expression, schema, stages).c_str());
  });
}

int gx_debug_rebuild_expression(const char* expression, char* buf, int buf_len, gx_status_info* status) {
  return guarded(status, [&] {
    if (!expression || !buf || buf_len <= 0) fail(GX_ERR_INVALID, "bad arguments");
    std::snprintf(buf, (size_t)buf_len, "%s", rebuild(parse_and_lower(expression)).c_str());
  });
}

void gx_debug_jit_stats(int64_t* compiles, double* total_ms) {
  if (compiles) *compiles = jit_compile_count();
  if (total_ms) *total_ms = jit_compile_ms_total();
}

}  // extern "C"
