// gx_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// This file restates, on the CPU, the algorithm of BlazingSQL's row-wise
// expression evaluator behind LogicalFilter / LogicalProject, so the CUDA
// implementation in blazingsql_gb300/ can be checked against it on the same
// inputs.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// may load it; the product never links or calls it.
//
// Reference files restated here (paths inside the BlazingSQL source tree):
//   engine/src/parser/expression_utils.cpp         normalisation, type rules, operator map
//   engine/src/parser/CalciteExpressionParsing.cpp literal scalars, n-ary AND/OR nesting
//   engine/src/parser/expression_tree.{hpp,cpp}    lexer, parser, CASE / ROUND / CAST lowering
//   engine/src/utilities/scalar_timestamp_parser.cpp  date / timestamp literal parsing
//   engine/src/Interpreter/interpreter_ops.cuh     per-row op semantics (InterpreterFunctor)
//   engine/src/Interpreter/interpreter_cpp.cu      per-op input/output type resolution
//   engine/src/execution_kernels/LogicalProject.cpp evaluate_expressions / process_project
//   engine/src/execution_kernels/LogicalFilter.cpp  process_filter / applyBooleanFilter
//
// Value model.  The reference keeps every intermediate as a 64-bit slot that is
// read as int64 or double depending on whether the op's *kernel input type* is a
// float type (interpreter_ops.cuh:479-498), plus one validity bit.  We keep the
// same model: a value is (uint64 bits, valid).  Two type annotations are carried
// per node, exactly as the reference computes them:
//   vtype  -- expr_output_type_visitor (LogicalProject.cpp:748-794): decides the
//             output column type;
//   ktype  -- perform_interpreter_operation (interpreter_cpp.cu:507-550): decides
//             how the kernel reads each operand (a null literal is EMPTY here).
//
// Deliberate, documented divergences from the reference (each marked DIVERGENCE):
//   * data under a NULL *computed* value is defined as 0 (the reference leaves a
//     stale slot value); it is only observable through CASE's magic-number test;
//   * integer MOD by 0 yields NULL (undefined in the reference);
//   * IS_NOT_DISTINCT_FROM has type BOOL8 (the reference's binary type rule
//     returns EMPTY and fails when it is the root);
//   * EXP is accepted (absent from the reference operator map);
//   * a validity mask with a non-zero column offset is read at the offset (the
//     reference reads word row/32 ignoring the offset, interpreter_ops.cuh:397-404);
//   * the boolean literal lexer is anchored (the reference's `^true|false` pattern
//     matches `false` anywhere in the remaining text);
//   * RAND is a Philox4x32-10 stream keyed by (seed, RAND ordinal, row) so runs are
//     reproducible; the reference draws from curand with a random seed;
//   * ROUND's scale factor 10^d uses the correctly rounded double for |d| <= 22.
//
// Build: see oracle/Makefile (g++ -O2 -ffp-contract=off, no fast-math).

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <regex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// Types: numbering follows cudf::type_id (cudf 21.08), the layout the reference
// evaluator consumes.
// ---------------------------------------------------------------------------
enum TypeId : int32_t {
  EMPTY = 0, INT8, INT16, INT32, INT64, UINT8, UINT16, UINT32, UINT64, FLOAT32, FLOAT64, BOOL8,
  TIMESTAMP_DAYS, TIMESTAMP_SECONDS, TIMESTAMP_MILLISECONDS, TIMESTAMP_MICROSECONDS, TIMESTAMP_NANOSECONDS,
  DURATION_DAYS, DURATION_SECONDS, DURATION_MILLISECONDS, DURATION_MICROSECONDS, DURATION_NANOSECONDS,
  DICTIONARY32, STRING, LIST, DECIMAL32, DECIMAL64, STRUCT, NUM_TYPE_IDS
};

static bool is_float(int t) { return t == FLOAT32 || t == FLOAT64; }
static bool is_integer(int t) { return t >= INT8 && t <= UINT64; }
static bool is_timestamp(int t) { return t >= TIMESTAMP_DAYS && t <= TIMESTAMP_NANOSECONDS; }
static bool is_duration(int t) { return t >= DURATION_DAYS && t <= DURATION_NANOSECONDS; }

static int size_of(int t) {
  switch (t) {
    case INT8: case UINT8: case BOOL8: return 1;
    case INT16: case UINT16: return 2;
    case INT32: case UINT32: case FLOAT32: case TIMESTAMP_DAYS: case DURATION_DAYS: return 4;
    case INT64: case UINT64: case FLOAT64: case TIMESTAMP_SECONDS: case TIMESTAMP_MILLISECONDS:
    case TIMESTAMP_MICROSECONDS: case TIMESTAMP_NANOSECONDS: case DURATION_SECONDS:
    case DURATION_MILLISECONDS: case DURATION_MICROSECONDS: case DURATION_NANOSECONDS: return 8;
    default: return 0;
  }
}

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
enum { E_OK = 0, E_PARSE = 1, E_UNSUPPORTED = 2, E_TYPE = 3 };

// ---------------------------------------------------------------------------
// Operators (expression_utils.hpp:11-93)
// ---------------------------------------------------------------------------
enum Op {
  OP_INVALID,
  OP_RAND,
  OP_NOT, OP_ABS, OP_FLOOR, OP_CEIL, OP_SIN, OP_COS, OP_ASIN, OP_ACOS, OP_TAN, OP_COTAN, OP_ATAN,
  OP_LN, OP_LOG, OP_EXP, OP_YEAR, OP_MONTH, OP_DAY, OP_DAYOFWEEK, OP_HOUR, OP_MINUTE, OP_SECOND,
  OP_IS_NULL, OP_IS_NOT_NULL, OP_IS_TRUE, OP_IS_NOT_TRUE, OP_IS_NOT_FALSE,
  OP_CAST_TINYINT, OP_CAST_SMALLINT, OP_CAST_INTEGER, OP_CAST_BIGINT, OP_CAST_FLOAT, OP_CAST_DOUBLE,
  OP_CAST_DATE, OP_CAST_TIMESTAMP_SECONDS, OP_CAST_TIMESTAMP_MILLISECONDS, OP_CAST_TIMESTAMP_MICROSECONDS,
  OP_CAST_TIMESTAMP,
  OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MOD, OP_POW, OP_ROUND,
  OP_EQUAL, OP_NOT_EQUAL, OP_LESS, OP_GREATER, OP_LESS_EQUAL, OP_GREATER_EQUAL,
  OP_AND, OP_OR, OP_FIRST_NON_MAGIC, OP_MAGIC_IF_NOT, OP_IS_NOT_DISTINCT_FROM,
  // string operators: recognised so they can be rejected as out of scope
  OP_STRING_FN,
};

static bool is_unary(Op op) { return op >= OP_NOT && op <= OP_CAST_TIMESTAMP; }
static bool is_binary(Op op) { return op >= OP_ADD && op <= OP_IS_NOT_DISTINCT_FROM; }

// map_to_operator_type (expression_utils.cpp:268-352)
static Op map_op(const std::string& tok) {
  static const std::map<std::string, Op> M = {
    {"BLZ_RND", OP_RAND},
    {"NOT", OP_NOT}, {"IS NOT TRUE", OP_IS_NOT_TRUE}, {"IS NOT FALSE", OP_IS_NOT_FALSE}, {"IS TRUE", OP_IS_TRUE},
    {"SIN", OP_SIN}, {"ASIN", OP_ASIN}, {"COS", OP_COS}, {"ACOS", OP_ACOS}, {"TAN", OP_TAN}, {"ATAN", OP_ATAN},
    {"COT", OP_COTAN},
    {"FLOOR", OP_FLOOR}, {"CEIL", OP_CEIL}, {"ABS", OP_ABS}, {"LOG10", OP_LOG}, {"LN", OP_LN}, {"EXP", OP_EXP},
    {"BL_YEAR", OP_YEAR}, {"BL_MONTH", OP_MONTH}, {"BL_DAY", OP_DAY}, {"BL_DOW", OP_DAYOFWEEK},
    {"BL_HOUR", OP_HOUR}, {"BL_MINUTE", OP_MINUTE}, {"BL_SECOND", OP_SECOND},
    {"IS_NULL", OP_IS_NULL}, {"IS_NOT_NULL", OP_IS_NOT_NULL},
    {"CAST_TINYINT", OP_CAST_TINYINT}, {"CAST_SMALLINT", OP_CAST_SMALLINT}, {"CAST_INTEGER", OP_CAST_INTEGER},
    {"CAST_BIGINT", OP_CAST_BIGINT}, {"CAST_FLOAT", OP_CAST_FLOAT}, {"CAST_DOUBLE", OP_CAST_DOUBLE},
    {"CAST_DATE", OP_CAST_DATE}, {"CAST_TIMESTAMP_SECONDS", OP_CAST_TIMESTAMP_SECONDS},
    {"CAST_TIMESTAMP_MILLISECONDS", OP_CAST_TIMESTAMP_MILLISECONDS},
    {"CAST_TIMESTAMP_MICROSECONDS", OP_CAST_TIMESTAMP_MICROSECONDS}, {"CAST_TIMESTAMP", OP_CAST_TIMESTAMP},
    {"=", OP_EQUAL}, {"<>", OP_NOT_EQUAL}, {">", OP_GREATER}, {">=", OP_GREATER_EQUAL}, {"<", OP_LESS},
    {"<=", OP_LESS_EQUAL}, {"+", OP_ADD}, {"-", OP_SUB}, {"*", OP_MUL}, {"/", OP_DIV}, {"POWER", OP_POW},
    {"ROUND", OP_ROUND}, {"MOD", OP_MOD}, {"AND", OP_AND}, {"OR", OP_OR}, {"FIRST_NON_MAGIC", OP_FIRST_NON_MAGIC},
    {"MAGIC_IF_NOT", OP_MAGIC_IF_NOT}, {"IS_NOT_DISTINCT_FROM", OP_IS_NOT_DISTINCT_FROM},
    {"CAST_VARCHAR", OP_STRING_FN}, {"CAST_CHAR", OP_STRING_FN}, {"CHAR_LENGTH", OP_STRING_FN},
    {"LOWER", OP_STRING_FN}, {"UPPER", OP_STRING_FN}, {"INITCAP", OP_STRING_FN}, {"REVERSE", OP_STRING_FN},
    {"LIKE", OP_STRING_FN}, {"SUBSTRING", OP_STRING_FN}, {"REGEXP_REPLACE", OP_STRING_FN},
    {"REPLACE", OP_STRING_FN}, {"TO_DATE", OP_STRING_FN}, {"TO_TIMESTAMP", OP_STRING_FN},
    {"||", OP_STRING_FN}, {"CONCAT", OP_STRING_FN}, {"TRIM", OP_STRING_FN}, {"LEFT", OP_STRING_FN},
    {"RIGHT", OP_STRING_FN},
  };
  auto it = M.find(tok);
  if (it == M.end()) throw Error(E_UNSUPPORTED, "Unsupported operator: " + tok);
  if (it->second == OP_STRING_FN) throw Error(E_UNSUPPORTED, "string operator out of scope: " + tok);
  return it->second;
}

// get_output_type, unary form (expression_utils.cpp:127-200)
static int out_type_unary(Op op, int l) {
  switch (op) {
    case OP_CAST_TINYINT: return INT8;
    case OP_CAST_SMALLINT: return INT16;
    case OP_CAST_INTEGER: return INT32;
    case OP_CAST_BIGINT: return INT64;
    case OP_CAST_FLOAT: return FLOAT32;
    case OP_CAST_DOUBLE: return FLOAT64;
    case OP_CAST_DATE: return TIMESTAMP_DAYS;
    case OP_CAST_TIMESTAMP_SECONDS: return TIMESTAMP_SECONDS;
    case OP_CAST_TIMESTAMP_MILLISECONDS: return TIMESTAMP_MILLISECONDS;
    case OP_CAST_TIMESTAMP_MICROSECONDS: return TIMESTAMP_MICROSECONDS;
    case OP_CAST_TIMESTAMP: return TIMESTAMP_NANOSECONDS;
    case OP_YEAR: case OP_MONTH: case OP_DAY: case OP_DAYOFWEEK: case OP_HOUR: case OP_MINUTE: case OP_SECOND:
      return INT16;
    case OP_SIN: case OP_COS: case OP_ASIN: case OP_ACOS: case OP_TAN: case OP_COTAN: case OP_ATAN:
    case OP_LN: case OP_LOG: case OP_EXP: case OP_FLOOR: case OP_CEIL:
      return is_float(l) ? l : FLOAT64;
    case OP_ABS: return l;
    case OP_NOT: case OP_IS_TRUE: case OP_IS_NULL: case OP_IS_NOT_NULL: case OP_IS_NOT_TRUE: case OP_IS_NOT_FALSE:
      return BOOL8;
    default: return EMPTY;
  }
}

// get_output_type, binary form (expression_utils.cpp:202-262)
static int out_type_binary(Op op, int l, int r) {
  if (l == EMPTY && r == EMPTY) throw Error(E_TYPE, "In get_output_type function: both operands types are empty");
  if (l == EMPTY) l = r; else if (r == EMPTY) r = l;
  switch (op) {
    case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_MOD:
      if (is_float(l) && is_float(r)) return size_of(l) >= size_of(r) ? l : r;
      if (is_float(l)) return l;
      if (is_float(r)) return r;
      return size_of(l) >= size_of(r) ? l : r;
    case OP_EQUAL: case OP_NOT_EQUAL: case OP_LESS: case OP_GREATER: case OP_LESS_EQUAL: case OP_GREATER_EQUAL:
    case OP_AND: case OP_OR:
      return BOOL8;
    case OP_POW: case OP_ROUND:
      return size_of(l) <= size_of(FLOAT32) ? FLOAT32 : FLOAT64;
    case OP_MAGIC_IF_NOT: return r;
    case OP_FIRST_NON_MAGIC: return size_of(l) >= size_of(r) ? l : r;
    case OP_IS_NOT_DISTINCT_FROM: return BOOL8;  // DIVERGENCE: reference returns EMPTY here
    default: return EMPTY;
  }
}

// ---------------------------------------------------------------------------
// String helpers
// ---------------------------------------------------------------------------
static void replace_all(std::string& s, const std::string& from, const std::string& to) {
  if (from.empty()) return;
  size_t pos = 0;
  while ((pos = s.find(from, pos)) != std::string::npos) {
    s.replace(pos, from.size(), to);
    pos += to.size();
  }
}
static std::string replace_first(const std::string& s, const std::string& from, const std::string& to) {
  std::string r = s;
  size_t p = r.find(from);
  if (p != std::string::npos) r.replace(p, from.size(), to);
  return r;
}
// StringUtil::replace (io/src/Util/StringUtil.cpp:371-380): every occurrence,
// left to right, scanning on after each replacement
static std::string string_replace(const std::string& s, const std::string& from, const std::string& to) {
  std::string r = s;
  size_t p = 0;
  while ((p = r.find(from, p)) != std::string::npos) {
    r.replace(p, from.size(), to);
    p += to.size();
  }
  return r;
}
static std::string ltrim(const std::string& s) {
  size_t i = 0;
  while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
  return s.substr(i);
}
static std::string trim(const std::string& s) {
  std::string t = ltrim(s);
  size_t j = t.size();
  while (j > 0 && std::isspace((unsigned char)t[j - 1])) j--;
  return t.substr(0, j);
}
static size_t count_of(const std::string& s, const std::string& needle) {
  size_t c = 0, p = 0;
  while ((p = s.find(needle, p)) != std::string::npos) { c++; p += needle.size(); }
  return c;
}

// replace_calcite_regex (expression_utils.cpp:1068-1113)
static std::string replace_calcite_regex(const std::string& expr) {
  std::string ret = expr;
  static const std::regex char_collate_re{R"((?:\(\d+\))? CHARACTER SET ".+?" COLLATE ".+?")", std::regex_constants::icase};
  ret = std::regex_replace(ret, char_collate_re, "");
  static const std::regex timestamp_re{R"(TIMESTAMP\(\d+\))", std::regex_constants::icase};
  ret = std::regex_replace(ret, timestamp_re, "TIMESTAMP");
  static const std::regex decimal_re{R"(DECIMAL\(\d+, \d+\))", std::regex_constants::icase};
  ret = std::regex_replace(ret, decimal_re, "DOUBLE");
  static const std::regex char_re{R"(:CHAR\(\d+\))", std::regex_constants::icase};
  ret = std::regex_replace(ret, char_re, ":VARCHAR");
  replace_all(ret, "IS NOT DISTINCT FROM", "IS_NOT_DISTINCT_FROM");
  replace_all(ret, "IS NOT NULL", "IS_NOT_NULL");
  replace_all(ret, "IS NULL", "IS_NULL");
  replace_all(ret, " NOT NULL", "");
  replace_all(ret, "RAND()", "BLZ_RND()");
  replace_all(ret, "EXTRACT(FLAG(YEAR), ", "BL_YEAR(");
  replace_all(ret, "EXTRACT(FLAG(MONTH), ", "BL_MONTH(");
  replace_all(ret, "EXTRACT(FLAG(DAY), ", "BL_DAY(");
  replace_all(ret, "EXTRACT(FLAG(DOW), ", "BL_DOW(");
  replace_all(ret, "EXTRACT(FLAG(HOUR), ", "BL_HOUR(");
  replace_all(ret, "EXTRACT(FLAG(MINUTE), ", "BL_MINUTE(");
  replace_all(ret, "EXTRACT(FLAG(SECOND), ", "BL_SECOND(");
  replace_all(ret, "DAY TO SECOND", "SECOND");
  replace_all(ret, "HOUR TO SECOND", "SECOND");
  replace_all(ret, "MINUTE TO SECOND", "SECOND");
  replace_all(ret, "/INT(", "/(");
  return ret;
}

// get_expressions_from_expression_list (expression_utils.cpp:1012-1066)
static std::vector<std::string> split_expression_list(std::string& combined, bool do_trim) {
  combined = replace_calcite_regex(combined);
  std::vector<std::string> out;
  size_t cur = 0, start = 0;
  bool in_quotes = false;
  int paren = 0, sq = 0;
  while (cur < combined.size()) {
    char c = combined[cur];
    if (in_quotes) {
      if (c == '\'' && !(cur + 1 < combined.size() && combined[cur + 1] == '\'')) in_quotes = false;
    } else {
      if (c == '\'') in_quotes = true;
      else if (c == '(') paren++;
      else if (c == ')') paren--;
      else if (c == '[') sq++;
      else if (c == ']') sq--;
      else if (c == ',' && paren == 0 && sq == 0) {
        std::string e = combined.substr(start, cur - start);
        out.push_back(do_trim ? ltrim(e) : e);
        start = cur + 1;
      }
    }
    cur++;
  }
  if (start < combined.size()) {
    std::string e = combined.substr(start, cur - start);
    out.push_back(do_trim ? trim(e) : e);
  }
  return out;
}

// get_named_expression (expression_utils.cpp:537-547)
static std::string get_named_expression(const std::string& qp, const std::string& name) {
  if (qp.find(name + "=[") == std::string::npos) return "";
  size_t start;
  if (qp.find(name + "=[[") != std::string::npos) start = qp.find(name + "=[[") + 3 + name.size();
  else start = qp.find(name + "=[") + 2 + name.size();
  size_t end = qp.find("]", start);
  return qp.substr(start, end - start);
}

// get_query_part (expression_utils.cpp:764-769)
static std::string get_query_part(const std::string& plan) {
  size_t a = plan.find("(");
  size_t b = plan.rfind(")");
  if (a == std::string::npos || b == std::string::npos || b < a) throw Error(E_PARSE, "malformed relational node: " + plan);
  return plan.substr(a + 1, b - a - 1);
}

// find_closing_char (CalciteExpressionParsing.cpp:295-328)
static int find_closing(const std::string& e, int start) {
  char open = e[start], close = open == '(' ? ')' : open == '[' ? ']' : 0;
  if (!close) return -1;
  size_t i = start + 1;
  int depth = 1;
  bool inq = false;
  while (i < e.size()) {
    if (inq) {
      if (e[i] == '\'' && !(i + 1 < e.size() && e[i + 1] == '\'')) inq = false;
    } else {
      if (e[i] == '\'') inq = true;
      else if (e[i] == open) depth++;
      else if (e[i] == close) { if (--depth == 0) return (int)i; }
    }
    i++;
  }
  return -1;
}

// quoted-ness vector + first-occurrence-not-in-quotes (io StringUtil helpers)
static int find_first_not_in_quotes(const std::string& s, const std::string& needle, size_t from) {
  std::vector<bool> quoted(s.size(), false);
  bool inq = false;
  for (size_t i = 0; i < s.size(); i++) {
    if (s[i] == '\'') { inq = !inq; quoted[i] = true; continue; }
    quoted[i] = inq;
  }
  size_t p = from;
  while ((p = s.find(needle, p)) != std::string::npos) {
    if (!quoted[p]) return (int)p;
    p++;
  }
  return -1;
}

// expand_if_logical_op (CalciteExpressionParsing.cpp:331-398): n-ary AND(/OR( to
// left-deep binary nesting.  OR is not expanded when the text contains FLOOR.
static std::string expand_if_logical_op(std::string expression) {
  std::string output = expression;
  size_t start_pos = 0;
  while (start_pos < expression.size()) {
    int first_and = find_first_not_in_quotes(expression, "AND(", start_pos);
    int first_or = -1;
    if (expression.find("FLOOR") == std::string::npos) first_or = find_first_not_in_quotes(expression, "OR(", start_pos);
    int first;
    std::string op;
    if (first_and >= 0) {
      if (first_or >= 0 && first_or < first_and) { first = first_or; op = "OR("; }
      else { first = first_and; op = "AND("; }
    } else { first = first_or; op = "OR("; }
    if (first < 0) return output;
    int es = first + (int)op.size() - 1;
    int ee = find_closing(expression, es);
    if (ee < 0) throw Error(E_PARSE, "unbalanced parentheses in: " + expression);
    std::string rest = expression.substr(es + 1, ee - (es + 1));
    std::vector<std::string> parts = split_expression_list(rest, false);
    if (parts.size() == 2) { start_pos = es; continue; }
    if (parts.size() < 2) throw Error(E_PARSE, "logical operator with fewer than two operands: " + expression);
    start_pos = first;
    output = expression.substr(0, first);
    for (size_t i = 0; i + 1 < parts.size(); i++) { output += op; start_pos += op.size(); }
    output += parts[0] + ",";
    for (size_t i = 1; i + 1 < parts.size(); i++) output += parts[i] + "),";
    output += parts.back() + ")";
    if ((size_t)ee < expression.size() - 1) output += expression.substr(ee + 1);
    expression = output;
  }
  return output;
}

// fill_minus_op_with_zero (expression_utils.cpp:1155-1164)
static std::string fill_minus_op_with_zero(std::string e) {
  if (!e.empty() && e[0] == '-' && count_of(e, "$") == 1 && e.find(",") == std::string::npos) {
    std::string l = e.substr(0, 2), r = e.substr(2);
    e = l + "0, " + r;
  }
  return e;
}

// convert_ms_to_ns_units (expression_utils.cpp:1316-1350)
static std::string convert_ms_to_ns_units(std::string e) {
  bool cts = e.find("CAST(") != std::string::npos && e.find(":TIMESTAMP") != std::string::npos;
  bool cdt = e.find("CAST(") != std::string::npos && e.find(":DATE") != std::string::npos;
  if (!cts && !cdt) return e;
  const std::string ns = "000000";
  if (e.find("Reinterpret(") != std::string::npos) {
    for (const char* u : {"86400000", "3600000", "60000", "1000"}) {
      if (e.find(u) != std::string::npos) return string_replace(e, u, std::string(u) + ns);
    }
  }
  size_t ip = e.find(":INTERVAL");
  if (ip != std::string::npos) {
    size_t sp = e.find(", ") + 2;
    std::string tv = e.substr(sp, ip - sp);
    return string_replace(e, tv, tv + ns);
  }
  return e;
}

static bool re_match(const std::string& s, const char* pat) {
  std::regex re(pat);
  return std::regex_match(s, re);
}
static bool is_date_dash(const std::string& s) { return re_match(s, R"([0-9]{4}-[0-9]{2}-[0-9]{2})"); }
static bool is_date_bar(const std::string& s) { return re_match(s, R"([0-9]{4}/[0-9]{2}/[0-9]{2})"); }
static bool is_date(const std::string& s) { return is_date_bar(s) || is_date_dash(s); }
static bool is_ts_dec(const std::string& s, int digits) {
  char a[256], b[256];
  snprintf(a, sizeof a, "([0-9]{4})-([0-9]{2})-([0-9]{2})?[ T]?([0-9]{2}):([0-9]{2}):([0-9]{2}).([0-9]{%d})?[Z]?", digits);
  snprintf(b, sizeof b, "([0-9]{4})/([0-9]{2})/([0-9]{2})?[ T]?([0-9]{2}):([0-9]{2}):([0-9]{2}).([0-9]{%d})?[Z]?", digits);
  return re_match(s, a) || re_match(s, b);
}
static bool is_ts_with_decimals(const std::string& s) { return is_ts_dec(s, 3) || is_ts_dec(s, 6) || is_ts_dec(s, 9); }
static bool is_timestamp_str(const std::string& s) {
  return re_match(s, "([0-9]{4})/([0-9]{2})/([0-9]{2})?[ T]?([0-9]{2}):([0-9]{2}):([0-9]{2})?[Z]?") ||
         re_match(s, "([0-9]{4})-([0-9]{2})-([0-9]{2})?[ T]?([0-9]{2}):([0-9]{2}):([0-9]{2})?[Z]?") ||
         is_ts_with_decimals(s);
}

// reinterpret_timestamp (expression_utils.cpp:1371-1420)
static std::string reinterpret_timestamp(std::string e, const std::vector<int>& schema) {
  if (schema.empty()) return e;
  const std::string key = "Reinterpret(-(";
  size_t p = e.find(key);
  if (p == std::string::npos) return e;
  std::string red = e.substr(p + key.size());
  red = red.substr(0, red.find("))"));
  std::vector<std::string> parts = split_expression_list(red, false);
  if (parts.size() != 2) return e;
  auto idx_of = [](std::string x) -> size_t {
    if (x[0] == '$') return (size_t)std::stoi(x.substr(1));
    size_t a = x.find('$') + 1, b = x.find(')');
    return (size_t)std::stoi(x.substr(a, b - a));
  };
  std::string ts;
  size_t col;
  if (is_timestamp_str(parts[0])) { ts = parts[0]; col = idx_of(parts[1]); }
  else if (is_timestamp_str(parts[1])) { ts = parts[1]; col = idx_of(parts[0]); }
  else return e;
  if (col >= schema.size()) throw Error(E_PARSE, "column index out of range in Reinterpret");
  const char* unit = schema[col] == TIMESTAMP_SECONDS ? "TIMESTAMP_SECONDS"
                   : schema[col] == TIMESTAMP_MILLISECONDS ? "TIMESTAMP_MILLISECONDS"
                   : schema[col] == TIMESTAMP_MICROSECONDS ? "TIMESTAMP_MICROSECONDS" : "TIMESTAMP";
  return string_replace(e, ts, "CAST(" + ts + "):" + unit);
}

// apply_interval_conversion (expression_utils.cpp:1425-1460)
static std::string apply_interval_conversion(std::string e, const std::vector<int>& schema) {
  const std::string iv = ":INTERVAL";
  if (schema.empty() || e.find(iv) == std::string::npos) return e;
  if (e.find("+") != std::string::npos || e.find("-") != std::string::npos) {
    size_t sp = 0;
    if (e.find("+($") != std::string::npos) sp = e.find("+($") + 3;
    else if (e.find("-($") != std::string::npos) sp = e.find("-($") + 3;
    std::string ne = e.substr(sp);
    ne = ne.substr(0, ne.find(", "));
    int col = std::stoi(ne);
    if (col < 0 || (size_t)col >= schema.size()) throw Error(E_PARSE, "column index out of range in interval");
    if (schema[col] == DURATION_SECONDS) return string_replace(e, "000" + iv, iv);
    if (schema[col] == DURATION_MICROSECONDS) return string_replace(e, "000" + iv, "000000" + iv);
    if (schema[col] == DURATION_NANOSECONDS) return string_replace(e, "000" + iv, "000000000" + iv);
    return e;
  }
  if (e.find("$") == std::string::npos && e.find("000:INTERVAL") != std::string::npos) return string_replace(e, "000" + iv, iv);
  return e;
}

// preprocess_expression (expression_utils.cpp:1624-1632).  CURRENT_DATE /
// CURRENT_TIMESTAMP need the engine Context; with no Context they are rejected.
static std::string preprocess_expression(std::string e, const std::vector<int>& schema) {
  e = fill_minus_op_with_zero(e);
  if (e.find("CONCAT") != std::string::npos) throw Error(E_UNSUPPORTED, "string operator out of scope: CONCAT");
  if (e.find("CURRENT_DATE") != std::string::npos || e.find("CURRENT_TIME") != std::string::npos)
    throw Error(E_UNSUPPORTED, "CURRENT_DATE/CURRENT_TIMESTAMP need an engine context");
  e = convert_ms_to_ns_units(e);
  e = reinterpret_timestamp(e, schema);
  e = apply_interval_conversion(e, schema);
  return e;
}

// ---------------------------------------------------------------------------
// Lexer / parser (expression_tree.hpp:258-330, expression_tree.cpp:33-279)
// ---------------------------------------------------------------------------
enum Tok { T_LP, T_RP, T_COMMA, T_COLON, T_VAR, T_NULL, T_BOOL, T_NUM, T_DUR_S, T_DUR_MS, T_TS_D, T_TS_S, T_TS_MS,
           T_TS_NS, T_STR, T_IDENT, T_EOF };
struct Token { Tok t; std::string v; };

struct Lexer {
  std::string text;
  size_t pos = 0;
  explicit Lexer(const std::string& s) : text(trim(s)) {}
  Token next() {
    if (pos >= text.size()) return {T_EOF, ""};
    while (pos < text.size() && text[pos] == ' ') pos++;
    if (pos >= text.size()) return {T_EOF, ""};
    char c = text[pos];
    if (c == '(') { pos++; return {T_LP, "("}; }
    if (c == ')') { pos++; return {T_RP, ")"}; }
    if (c == ',') { pos++; return {T_COMMA, ","}; }
    if (c == ':') { pos++; return {T_COLON, ":"}; }
    static const std::regex var_re{R"(^\$\d+)"}, null_re{R"(^null)"}, bool_re{R"(^(?:true|false))"},
        dur_s_re{R"(^\d{2}:\d{2}:\d{2})"},
        ts_us_re{R"(^\d{4}-\d{2}-\d{2}(?:[ T]?\d{2}:\d{2}:\d{2}.\d{6}))"},
        ts_ms_re{R"(^\d{4}-\d{2}-\d{2}(?:[ T]?\d{2}:\d{2}:\d{2}.\d{3}))"},
        ts_s_re{R"(^\d{4}-\d{2}-\d{2}(?:[ T]?\d{2}:\d{2}:\d{2}))"}, ts_d_re{R"(^\d{4}-\d{2}-\d{2})"},
        num_re{R"(^[-+]?\d*\.?\d+([eE][-+]?\d+)?)"}, str_re{R"(^(["'])(?:(?!\1|\\).|\\.)*?\1)"};
    std::smatch m;
    std::string rem = text.substr(pos);
    auto take = [&](const std::regex& re, Tok t, Token& out) {
      if (std::regex_search(rem, m, re)) { pos += m.length(0); out = {t, m.str(0)}; return true; }
      return false;
    };
    Token tk;
    if (take(var_re, T_VAR, tk)) return tk;
    if (take(null_re, T_NULL, tk)) return tk;
    if (take(bool_re, T_BOOL, tk)) return tk;  // DIVERGENCE: anchored alternation
    if (take(dur_s_re, T_DUR_S, tk)) return tk;
    // the reference tests its nanosecond token with the microsecond pattern first
    if (take(ts_us_re, T_TS_NS, tk)) return tk;
    if (take(ts_ms_re, T_TS_MS, tk)) return tk;
    if (take(ts_s_re, T_TS_S, tk)) return tk;
    if (take(ts_d_re, T_TS_D, tk)) return tk;
    if (take(num_re, T_NUM, tk)) return tk;
    if (take(str_re, T_STR, tk)) return tk;
    size_t len = 0;
    do {
      char ch = text[pos + len];
      if (ch == '(' || ch == ')' || ch == ',' || ch == ':') break;
    } while (pos + (++len) < text.size());
    std::string v = text.substr(pos, len);
    pos += len;
    return {T_IDENT, v};
  }
};

enum NodeKind { N_OP, N_LIT, N_VAR };
struct Node {
  NodeKind kind;
  std::string value;   // operator token / literal text / "$i"
  int lit_type = EMPTY;
  int var_index = -1;
  std::vector<std::unique_ptr<Node>> ch;
  // annotations
  Op op = OP_INVALID;
  int vtype = EMPTY, ktype = EMPTY;
};

// type_from_type_token (expression_tree.cpp:324-375)
static int type_from_token(const std::string& v) {
  if (v == "NULL" || v == "BOOLEAN") return BOOL8;
  if (v == "TINYINT") return INT8;
  if (v == "SMALLINT") return INT16;
  if (v == "INTEGER") return INT32;
  if (v == "INTERVAL SECOND" || v == "INTERVAL MINUTE" || v == "INTERVAL HOUR" || v == "INTERVAL DAY") return DURATION_SECONDS;
  if (v == "INTERVAL MONTH" || v == "INTERVAL YEAR") throw Error(E_UNSUPPORTED, "operation over MONTH or YEAR units are not currently supported.");
  if (v == "BIGINT") return INT64;
  if (v == "FLOAT") return FLOAT32;
  if (v == "DOUBLE") return FLOAT64;
  if (v == "DATE") return TIMESTAMP_DAYS;
  if (v == "TIMESTAMP_SECONDS") return TIMESTAMP_SECONDS;
  if (v == "TIMESTAMP_MILLISECONDS") return TIMESTAMP_MILLISECONDS;
  if (v == "TIMESTAMP_MICROSECONDS") return TIMESTAMP_MICROSECONDS;
  if (v == "TIMESTAMP") return TIMESTAMP_NANOSECONDS;
  if (v == "VARCHAR") return STRING;
  throw Error(E_PARSE, "Invalid literal cast type: " + v);
}

// infer_type_from_literal_token (expression_tree.cpp:281-322)
static int infer_literal_type(const Token& t) {
  switch (t.t) {
    case T_NULL: return EMPTY;
    case T_BOOL: return BOOL8;
    case T_NUM: {
      if (t.v.find_first_of(".eE") != std::string::npos) {
        double d = std::stod(t.v);
        float f = (float)d;
        return (d == (double)f) ? FLOAT32 : FLOAT64;
      }
      long long v;
      try { v = std::stoll(t.v); } catch (...) { throw Error(E_PARSE, "integer literal out of range: " + t.v); }
      return v > 2147483647LL ? INT64 : INT32;
    }
    case T_DUR_S: return DURATION_SECONDS;
    case T_DUR_MS: return DURATION_MILLISECONDS;
    case T_TS_NS: return TIMESTAMP_NANOSECONDS;
    case T_TS_MS: return TIMESTAMP_MILLISECONDS;
    case T_TS_S: return TIMESTAMP_SECONDS;
    case T_TS_D: return TIMESTAMP_DAYS;
    default: return STRING;
  }
}

struct Parser {
  Lexer lx;
  Token tok;
  explicit Parser(const std::string& s) : lx(s) { tok = lx.next(); }
  bool accept(Tok t) {
    if (tok.t == t) { tok = lx.next(); return true; }
    return false;
  }
  std::unique_ptr<Node> expr() {
    auto r = term();
    if (!r) r = func();
    if (!r) throw Error(E_PARSE, "Couldn't parse calcite expression");
    return r;
  }
  std::unique_ptr<Node> term() {
    Token t = tok;
    if (accept(T_VAR)) {
      auto n = std::make_unique<Node>();
      n->kind = N_VAR;
      n->value = t.v;
      n->var_index = std::stoi(t.v.substr(1));
      return n;
    }
    return literal();
  }
  std::unique_ptr<Node> func() {
    Token name = tok;
    if (!accept(T_IDENT)) return nullptr;
    accept(T_LP);
    std::vector<std::unique_ptr<Node>> args;
    if (!accept(T_RP)) {
      args.push_back(expr());
      while (accept(T_COMMA)) args.push_back(expr());
      accept(T_RP);
    }
    std::string id = name.v;
    if (accept(T_COLON)) {
      Token rt = tok;
      accept(T_IDENT);
      id += "_" + rt.v;
    }
    auto n = std::make_unique<Node>();
    n->kind = N_OP;
    n->value = id;
    n->ch = std::move(args);
    return n;
  }
  std::unique_ptr<Node> literal() {
    Token t = tok;
    if (accept(T_NULL) || accept(T_BOOL) || accept(T_NUM) || accept(T_DUR_S) || accept(T_DUR_MS) || accept(T_TS_D) ||
        accept(T_TS_S) || accept(T_TS_MS) || accept(T_TS_NS) || accept(T_STR)) {
      int type;
      if (accept(T_COLON)) {
        Token tt = tok;
        accept(T_IDENT);
        type = type_from_token(tt.v);
      } else {
        type = infer_literal_type(t);
      }
      auto n = std::make_unique<Node>();
      n->kind = N_LIT;
      n->value = t.v;
      n->lit_type = type;
      return n;
    }
    return nullptr;
  }
};

// get_common_type(strict) compatibility check used by CAST-of-literal lowering
// (utilities/CommonOperations.cpp:185-230)
static void check_common_type(int a, int b) {
  if (a == b) return;
  if ((is_float(a) && is_float(b)) || (is_integer(a) && is_integer(b))) return;
  if (is_timestamp(a) && is_timestamp(b)) return;
  if (is_duration(a) && is_duration(b)) return;
  if (a == STRING && is_timestamp(b)) return;
  throw Error(E_TYPE, "No common type between " + std::to_string(a) + " and " + std::to_string(b));
}

// custom_op_transformer (expression_tree.hpp:181-258), applied bottom-up.
static std::unique_ptr<Node> lower_case(std::vector<std::unique_ptr<Node>>& c, size_t i) {
  if (i == c.size() - 1) return std::move(c[i]);
  auto mif = std::make_unique<Node>();
  mif->kind = N_OP;
  mif->value = "MAGIC_IF_NOT";
  mif->ch.push_back(std::move(c[i]));
  mif->ch.push_back(std::move(c[i + 1]));
  auto fnm = std::make_unique<Node>();
  fnm->kind = N_OP;
  fnm->value = "FIRST_NON_MAGIC";
  fnm->ch.push_back(std::move(mif));
  fnm->ch.push_back(lower_case(c, i + 2));
  return fnm;
}

static std::unique_ptr<Node> custom_ops(std::unique_ptr<Node> n) {
  if (n->kind != N_OP) return n;
  for (auto& c : n->ch) c = custom_ops(std::move(c));
  if (n->value == "CASE") {
    if (n->ch.size() < 3 || n->ch.size() % 2 == 0) throw Error(E_PARSE, "CASE needs an odd number (>=3) of operands");
    return lower_case(n->ch, 0);
  }
  if (n->value == "Reinterpret") {
    if (n->ch.size() != 1) throw Error(E_PARSE, "Reinterpret takes one operand");
    return std::move(n->ch[0]);
  }
  if (n->value == "ROUND") {
    if (n->ch.size() == 1) {
      auto z = std::make_unique<Node>();
      z->kind = N_LIT;
      z->value = "0";
      z->lit_type = INT8;
      n->ch.push_back(std::move(z));
    }
    return n;
  }
  if (n->value.rfind("CAST", 0) == 0) {
    if (n->ch.size() != 1) throw Error(E_PARSE, "CAST takes one operand");
    if (n->ch[0]->kind == N_LIT) {
      Op cop = map_op(n->value);
      int nt = out_type_unary(cop, n->ch[0]->lit_type);
      check_common_type(n->ch[0]->lit_type, nt);
      auto l = std::move(n->ch[0]);
      l->lit_type = nt;
      return l;
    }
  }
  return n;
}

// ---------------------------------------------------------------------------
// Literal scalars (CalciteExpressionParsing.cpp:138-262, scalar_timestamp_parser.cpp)
// ---------------------------------------------------------------------------
struct Scalar { uint64_t bits = 0; bool valid = false; int type = EMPTY; };

static uint64_t d2b(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static double b2d(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }

// days_from_civil, the era-based algorithm used by the reference's parser
// (scalar_timestamp_parser.cpp timestamp_from_parts).
static int64_t days_from_parts(int32_t y, int32_t m, int32_t d) {
  y -= (m <= 2) ? 1 : 0;
  const int32_t eras_days = 146097, eras_years = eras_days / 365;
  int32_t era = (y >= 0 ? y : y - 399) / eras_years;
  int32_t yoe = y - era * eras_years;
  int32_t doy = m == 0 ? d : ((153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1);
  int32_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return (int32_t)(era * eras_days + doe - 719468);
}

static int32_t str2int(const char* p, int n) {
  int32_t v = 0;
  for (int i = 0; i < n; i++) {
    char c = p[i];
    if (c < '0' || c > '9') break;
    v = v * 10 + (c - '0');
  }
  return v;
}

// Parses "%Y-%m-%d[ %H:%M:%S[.%f]]" by fixed positions into the unit of `type`.
static int64_t parse_timestamp(const std::string& s, int type, bool with_time, bool with_frac) {
  int fl = type == TIMESTAMP_MILLISECONDS ? 3 : type == TIMESTAMP_NANOSECONDS ? 9 : 6;
  size_t need = with_time ? (with_frac ? 20 + fl : 19) : 10;
  if (s.size() < need) throw Error(E_PARSE, "format string cannot be parsed from datetime string: " + s);
  int32_t y = str2int(s.c_str(), 4), mo = str2int(s.c_str() + 5, 2), d = str2int(s.c_str() + 8, 2);
  int64_t days = days_from_parts(y, mo, d);
  if (type == TIMESTAMP_DAYS) return days;
  int32_t h = 0, mi = 0, se = 0, sub = 0;
  if (with_time) {
    h = str2int(s.c_str() + 11, 2);
    mi = str2int(s.c_str() + 14, 2);
    se = str2int(s.c_str() + 17, 2);
    if (with_frac) sub = str2int(s.c_str() + 20, fl);
  }
  int64_t t = days * 24LL * 3600LL + h * 3600LL + mi * 60LL + se;
  if (type == TIMESTAMP_SECONDS) return t;
  if (type == TIMESTAMP_MILLISECONDS) t *= 1000LL;
  else if (type == TIMESTAMP_MICROSECONDS) t *= 1000000LL;
  else t *= 1000000000LL;
  return t + sub;
}

static Scalar make_scalar(const std::string& text, int type) {
  Scalar s;
  s.type = type;
  if (text == "null") { s.valid = false; return s; }
  s.valid = true;
  try {
    switch (type) {
      case BOOL8: s.bits = (text == "true") ? 1 : 0; return s;
      case INT8: s.bits = (uint64_t)(int64_t)(int8_t)std::stoi(text); return s;
      case INT16: s.bits = (uint64_t)(int64_t)(int16_t)std::stoi(text); return s;
      case INT32: s.bits = (uint64_t)(int64_t)(int32_t)std::stoi(text); return s;
      case INT64: s.bits = (uint64_t)(int64_t)std::stoll(text); return s;
      case UINT8: s.bits = (uint64_t)(uint8_t)std::stoul(text); return s;
      case UINT16: s.bits = (uint64_t)(uint16_t)std::stoul(text); return s;
      case UINT32: s.bits = (uint64_t)(uint32_t)std::stoul(text); return s;
      case UINT64: s.bits = (uint64_t)std::stoull(text); return s;
      case FLOAT32: s.bits = d2b((double)std::stof(text)); return s;
      case FLOAT64: s.bits = d2b(std::stod(text)); return s;
      case DURATION_SECONDS: case DURATION_MILLISECONDS: case DURATION_MICROSECONDS: case DURATION_NANOSECONDS:
        s.bits = (uint64_t)(int64_t)std::stoll(text); return s;
      default: break;
    }
  } catch (const std::exception&) {
    throw Error(E_PARSE, "cannot convert literal '" + text + "'");
  }
  if (type == STRING) throw Error(E_UNSUPPORTED, "string literal out of scope: " + text);
  std::string c = text;
  if (!c.empty() && (c[0] == '\'' || c.back() == '\'')) c = c.substr(1, c.size() - 2);
  if (type == TIMESTAMP_DAYS) {
    if (!is_date(c)) throw Error(E_PARSE, "not recognized format TIMESTAMP_DAYS for: " + text);
    s.bits = (uint64_t)(int64_t)(int32_t)parse_timestamp(c, type, false, false);
    return s;
  }
  if (type == TIMESTAMP_SECONDS) {
    if (!is_timestamp_str(c)) throw Error(E_PARSE, "not recognized format TIMESTAMP_SECONDS for: " + c);
    s.bits = (uint64_t)parse_timestamp(c, type, true, false);
    return s;
  }
  if (type == TIMESTAMP_MILLISECONDS || type == TIMESTAMP_MICROSECONDS || type == TIMESTAMP_NANOSECONDS) {
    if (is_ts_with_decimals(c)) s.bits = (uint64_t)parse_timestamp(c, type, true, true);
    else if (is_timestamp_str(c)) s.bits = (uint64_t)parse_timestamp(c, type, true, false);
    else throw Error(E_PARSE, "not recognized format TIMESTAMP for: " + c);
    return s;
  }
  throw Error(E_UNSUPPORTED, "unsupported literal type");
}

// ---------------------------------------------------------------------------
// Annotation: operator ids, vtype and ktype
// ---------------------------------------------------------------------------
static void annotate(Node* n, const std::vector<int>& col_types) {
  if (n->kind == N_VAR) {
    if (n->var_index < 0 || (size_t)n->var_index >= col_types.size()) throw Error(E_PARSE, "column index out of range: " + n->value);
    int t = col_types[n->var_index];
    if (t == STRING) throw Error(E_UNSUPPORTED, "string column out of scope");
    n->vtype = n->ktype = t;
    return;
  }
  if (n->kind == N_LIT) {
    if (n->lit_type == STRING) throw Error(E_UNSUPPORTED, "string literal out of scope");
    n->vtype = n->lit_type;
    n->ktype = (n->value == "null") ? EMPTY : n->lit_type;
    return;
  }
  for (auto& c : n->ch) annotate(c.get(), col_types);
  n->op = map_op(n->value);
  if (n->op == OP_RAND) {
    n->vtype = n->ktype = FLOAT64;
  } else if (is_unary(n->op)) {
    if (n->ch.empty()) throw Error(E_PARSE, "unary operator without operand: " + n->value);
    if (n->ch[0]->kind == N_LIT) throw Error(E_UNSUPPORTED, "Unary operations on literals is not supported");
    n->vtype = out_type_unary(n->op, n->ch[0]->vtype);
    n->ktype = out_type_unary(n->op, n->ch[0]->ktype);
  } else if (is_binary(n->op)) {
    if (n->ch.size() < 2) throw Error(E_PARSE, "binary operator needs two operands: " + n->value);
    if (n->ch[0]->kind == N_LIT && n->ch[1]->kind == N_LIT) throw Error(E_UNSUPPORTED, "Operations between literals is not supported");
    n->vtype = out_type_binary(n->op, n->ch[0]->vtype, n->ch[1]->vtype);
    n->ktype = out_type_binary(n->op, n->ch[0]->ktype, n->ch[1]->ktype);
  } else {
    throw Error(E_UNSUPPORTED, "unsupported operator " + n->value);
  }
}

// ---------------------------------------------------------------------------
// Flat evaluation program (post-order, one op per tree node; no sharing)
// ---------------------------------------------------------------------------
enum SrcKind { S_COL, S_LIT, S_NULL, S_TMP, S_NONE };
struct Src { SrcKind k = S_NONE; int idx = -1; Scalar lit; int ktype = EMPTY; };
struct Step {
  Op op;
  Src l, r;
  int out;        // temp index
  int ktype;      // kernel output type (informational)
  int rand_id = -1;
};

struct Program {
  std::vector<Step> steps;
  int ntemps = 0;
  int nrand = 0;
};

static Src emit(Node* n, Program& p, int& rand_counter) {
  Src s;
  s.ktype = n->ktype;
  if (n->kind == N_VAR) { s.k = S_COL; s.idx = n->var_index; return s; }
  if (n->kind == N_LIT) {
    Scalar sc = make_scalar(n->value, n->lit_type);
    if (!sc.valid) { s.k = S_NULL; s.ktype = EMPTY; return s; }
    s.k = S_LIT; s.lit = sc;
    return s;
  }
  Step st;
  st.op = n->op;
  if (n->op == OP_RAND) {
    st.rand_id = rand_counter++;
  } else {
    // the reference visits every child (an un-expanded n-ary OR keeps its extra
    // operands in the tree) but its op reads only children[0] and children[1]
    std::vector<Src> kids;
    for (auto& c : n->ch) kids.push_back(emit(c.get(), p, rand_counter));
    st.l = kids[0];
    if (is_binary(n->op)) st.r = kids[1];
  }
  st.out = p.ntemps++;
  st.ktype = n->ktype;
  p.steps.push_back(st);
  s.k = S_TMP;
  s.idx = st.out;
  return s;
}

// ---------------------------------------------------------------------------
// Per-row semantics (interpreter_ops.cuh:479-925)
// ---------------------------------------------------------------------------
static const int64_t MAGIC_I = std::numeric_limits<int64_t>::max() - 13LL;
static const double MAGIC_D = 1.7976931348623123e+308;

// double -> int64 conversion with the GPU's cvt.rzi.s64.f64 behaviour
// (truncate, saturate out-of-range, NaN -> 0); the reference ran on the GPU.
static int64_t d2ll(double x) {
  if (x != x) return 0;
  if (x >= 9223372036854775808.0) return std::numeric_limits<int64_t>::max();
  if (x < -9223372036854775808.0) return std::numeric_limits<int64_t>::min();
  return (int64_t)x;
}

static double pow10_scale(double d) {
  static const double P[23] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11,
                               1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
  static const double N[23] = {1e-0, 1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11,
                               1e-12, 1e-13, 1e-14, 1e-15, 1e-16, 1e-17, 1e-18, 1e-19, 1e-20, 1e-21, 1e-22};
  if (d == std::floor(d) && d >= -22 && d <= 22) {
    int k = (int)d;
    return k >= 0 ? P[k] : N[-k];
  }
  return std::pow(10.0, d);
}

// ns per unit for timestamps / durations (cudf::timestamp_ns conversion)
static int64_t ns_per_unit(int t) {
  switch (t) {
    case TIMESTAMP_DAYS: case DURATION_DAYS: return 86400000000000LL;
    case TIMESTAMP_SECONDS: case DURATION_SECONDS: return 1000000000LL;
    case TIMESTAMP_MILLISECONDS: case DURATION_MILLISECONDS: return 1000000LL;
    case TIMESTAMP_MICROSECONDS: case DURATION_MICROSECONDS: return 1000LL;
    default: return 1;
  }
}
// the representation count of a timestamp is int32 for DAYS (cudf::timestamp_D)
static int64_t ts_count(int t, int64_t v) { return (t == TIMESTAMP_DAYS || t == DURATION_DAYS) ? (int64_t)(int32_t)v : v; }
static int64_t to_ns(int t, int64_t v) { return (int64_t)((uint64_t)ts_count(t, v) * (uint64_t)ns_per_unit(t)); }

static int64_t floor_div(int64_t a, int64_t b) { int64_t q = a / b; if ((a % b != 0) && ((a < 0) != (b < 0))) q--; return q; }

// extract_component_operator (interpreter_ops.cuh:69-99): civil-from-days
static int64_t extract(Op op, int t, int64_t v) {
  if (!is_timestamp(t)) return 0;
  int64_t per_day = ns_per_unit(t) == 86400000000000LL ? 1 : 86400000000000LL / ns_per_unit(t);
  int64_t cnt = ts_count(t, v);
  int64_t days = (t == TIMESTAMP_DAYS) ? cnt : floor_div(cnt, per_day);
  int64_t tsm = (t == TIMESTAMP_DAYS) ? 0 : cnt - days * per_day;
  int64_t per_hour = per_day / 24, per_min = per_hour / 60, per_sec = per_min / 60;
  if (op == OP_HOUR) return t == TIMESTAMP_DAYS ? 0 : tsm / per_hour;
  if (op == OP_MINUTE) return t == TIMESTAMP_DAYS ? 0 : (tsm % per_hour) / per_min;
  if (op == OP_SECOND) return t == TIMESTAMP_DAYS ? 0 : (tsm % per_min) / per_sec;
  if (op == OP_DAYOFWEEK) {
    int64_t wd = ((days % 7) + 7 + 4) % 7;  // 0 = Sunday
    return wd == 0 ? 7 : wd;
  }
  // civil_from_days (H. Hinnant's published algorithm)
  int64_t z = days + 719468;
  int64_t era = (z >= 0 ? z : z - 146096) / 146097;
  int64_t doe = z - era * 146097;
  int64_t yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  int64_t y = yoe + era * 400;
  int64_t doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  int64_t mp = (5 * doy + 2) / 153;
  int64_t d = doy - (153 * mp + 2) / 5 + 1;
  int64_t m = mp < 10 ? mp + 3 : mp - 9;
  y += (m <= 2);
  if (op == OP_YEAR) return y;
  if (op == OP_MONTH) return m;
  return d;  // OP_DAY
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
// as 1, 2, 3", SC'11) -> uniform double in (0, 1].
static double philox_uniform(uint64_t seed, uint32_t rand_id, uint64_t row) {
  uint32_t c0 = (uint32_t)row, c1 = (uint32_t)(row >> 32), c2 = rand_id, c3 = 0x5EED;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int i = 0; i < 10; i++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  uint64_t m = ((uint64_t)c0 << 21) | (c1 >> 11);
  return (double)(m + 1) * (1.0 / 9007199254740992.0);
}

struct Column { int type; const uint8_t* data; const uint32_t* mask; int64_t offset; int64_t size; };

static inline uint64_t read_bits(const Column& c, int64_t row) {
  int64_t i = c.offset + row;
  switch (c.type) {
    case INT8: return (uint64_t)(int64_t)((const int8_t*)c.data)[i];
    case INT16: return (uint64_t)(int64_t)((const int16_t*)c.data)[i];
    case INT32: case TIMESTAMP_DAYS: case DURATION_DAYS: return (uint64_t)(int64_t)((const int32_t*)c.data)[i];
    case UINT8: case BOOL8: {
      uint8_t b = ((const uint8_t*)c.data)[i];
      return c.type == BOOL8 ? (uint64_t)(b != 0) : (uint64_t)b;
    }
    case UINT16: return (uint64_t)((const uint16_t*)c.data)[i];
    case UINT32: return (uint64_t)((const uint32_t*)c.data)[i];
    case FLOAT32: return d2b((double)((const float*)c.data)[i]);
    default: return ((const uint64_t*)c.data)[i];  // 8-byte types
  }
}
static inline bool read_valid(const Column& c, int64_t row) {
  if (!c.mask) return true;
  int64_t b = c.offset + row;
  return (c.mask[b >> 5] >> (b & 31)) & 1u;
}

static const int CHUNK = 1024;

struct Scratch {
  std::vector<uint64_t> bits;
  std::vector<uint8_t> valid;
  int ntemps = 0;
  void init(int nt) { ntemps = nt; bits.assign((size_t)nt * CHUNK, 0); valid.assign((size_t)nt * CHUNK, 0); }
  uint64_t* b(int t) { return &bits[(size_t)t * CHUNK]; }
  uint8_t* v(int t) { return &valid[(size_t)t * CHUNK]; }
};

static inline void load_src(const Src& s, const std::vector<Column>& cols, Scratch& sc, int64_t row0, int n,
                            const uint64_t*& bp, const uint8_t*& vp, std::vector<uint64_t>& tb, std::vector<uint8_t>& tv) {
  if (s.k == S_TMP) { bp = sc.b(s.idx); vp = sc.v(s.idx); return; }
  tb.resize(CHUNK); tv.resize(CHUNK);
  if (s.k == S_COL) {
    const Column& c = cols[s.idx];
    for (int i = 0; i < n; i++) { tb[i] = read_bits(c, row0 + i); tv[i] = read_valid(c, row0 + i); }
  } else if (s.k == S_LIT) {
    // get_scalar_value<T>: a float-typed scalar reads as double, others as int64
    for (int i = 0; i < n; i++) { tb[i] = s.lit.bits; tv[i] = 1; }
  } else {  // S_NULL: uninitialised value in the reference; defined as 0
    for (int i = 0; i < n; i++) { tb[i] = 0; tv[i] = 0; }
  }
  bp = tb.data(); vp = tv.data();
}

static inline bool nz(uint64_t b, bool isf) { return isf ? (b2d(b) != 0.0) : (b != 0); }

static void run_step(const Step& st, const std::vector<Column>& cols, Scratch& sc, int64_t row0, int n, uint64_t seed,
                     std::vector<uint64_t>& lb, std::vector<uint8_t>& lv, std::vector<uint64_t>& rb, std::vector<uint8_t>& rv) {
  uint64_t* ob = sc.b(st.out);
  uint8_t* ov = sc.v(st.out);
  const Op op = st.op;
  if (op == OP_RAND) {
    for (int i = 0; i < n; i++) { ob[i] = d2b(philox_uniform(seed, (uint32_t)st.rand_id, (uint64_t)(row0 + i))); ov[i] = 1; }
    return;
  }
  const uint64_t* L; const uint8_t* LV;
  load_src(st.l, cols, sc, row0, n, L, LV, lb, lv);
  const int lt = st.l.ktype;
  const bool lf = is_float(lt);
  if (is_unary(op)) {
    for (int i = 0; i < n; i++) {
      const uint64_t x = L[i];
      const bool v = LV[i];
      const double xd = lf ? b2d(x) : (double)(int64_t)x;   // static_cast<double>(left_value)
      const int64_t xi = lf ? d2ll(b2d(x)) : (int64_t)x;     // static_cast<int64_t>(left_value)
      uint64_t r = 0;
      bool rvld = v;
      switch (op) {
        case OP_IS_NOT_TRUE: r = !(v && (lf ? b2d(x) == 1.0 : (int64_t)x == 1)); rvld = true; break;
        case OP_IS_NOT_FALSE: r = !(v && (lf ? b2d(x) == 0.0 : (int64_t)x == 0)); rvld = true; break;
        case OP_IS_NULL: r = !v; rvld = true; break;
        case OP_IS_NOT_NULL: r = v; rvld = true; break;
        default:
          if (!v) { r = 0; break; }  // DIVERGENCE: data under NULL defined as 0
          switch (op) {
            case OP_FLOOR: r = d2b(std::floor(xd)); break;
            case OP_CEIL: r = d2b(std::ceil(xd)); break;
            case OP_SIN: r = d2b(std::sin(xd)); break;
            case OP_COS: r = d2b(std::cos(xd)); break;
            case OP_ASIN: r = d2b(std::asin(xd)); break;
            case OP_ACOS: r = d2b(std::acos(xd)); break;
            case OP_TAN: r = d2b(std::tan(xd)); break;
            case OP_COTAN: r = d2b(std::cos(xd) / std::sin(xd)); break;
            case OP_ATAN: r = d2b(std::atan(xd)); break;
            case OP_ABS:
              if (lf) r = d2b(std::fabs(b2d(x)));
              else r = ((int64_t)x < 0) ? (uint64_t)0 - x : x;
              break;
            case OP_NOT: r = !nz(x, lf); break;
            case OP_IS_TRUE: r = (uint64_t)xi; break;
            case OP_LN: r = d2b(std::log(xd)); break;
            case OP_LOG: r = d2b(std::log10(xd)); break;
            case OP_EXP: r = d2b(std::exp(xd)); break;
            case OP_YEAR: case OP_MONTH: case OP_DAY: case OP_DAYOFWEEK: case OP_HOUR: case OP_MINUTE: case OP_SECOND:
              r = (uint64_t)extract(op, lt, (int64_t)x); break;
            case OP_CAST_TINYINT: case OP_CAST_SMALLINT: case OP_CAST_INTEGER: case OP_CAST_BIGINT:
              r = (uint64_t)xi; break;
            case OP_CAST_FLOAT: case OP_CAST_DOUBLE: r = d2b(xd); break;
            case OP_CAST_DATE: {
              int64_t d;
              switch (lt) {
                case TIMESTAMP_SECONDS: d = xi / 86400LL; break;
                case TIMESTAMP_MILLISECONDS: d = xi / 86400000LL; break;
                case TIMESTAMP_MICROSECONDS: d = xi / 86400000000LL; break;
                case TIMESTAMP_NANOSECONDS: d = xi / 86400000000000LL; break;
                default: d = xi; break;
              }
              r = (uint64_t)(int64_t)(int32_t)d;
              break;
            }
            case OP_CAST_TIMESTAMP_SECONDS: case OP_CAST_TIMESTAMP_MILLISECONDS:
            case OP_CAST_TIMESTAMP_MICROSECONDS: case OP_CAST_TIMESTAMP:
              r = is_timestamp(lt) ? (uint64_t)to_ns(lt, xi) : (uint64_t)xi;
              break;
            default: break;
          }
      }
      ob[i] = r;
      ov[i] = rvld;
    }
    return;
  }
  const uint64_t* R; const uint8_t* RV;
  load_src(st.r, cols, sc, row0, n, R, RV, rb, rv);
  const int rt = st.r.ktype;
  const bool rf = is_float(rt);
  const bool anyf = lf || rf;
  const bool ts_cmp = is_timestamp(lt) && is_timestamp(rt);
  for (int i = 0; i < n; i++) {
    const uint64_t a = L[i], b = R[i];
    const bool av = LV[i], bv = RV[i];
    const double ad = lf ? b2d(a) : (double)(int64_t)a, bd = rf ? b2d(b) : (double)(int64_t)b;
    const int64_t ai = (int64_t)a, bi = (int64_t)b;
    uint64_t r = 0;
    bool rvld = false;
    switch (op) {
      case OP_MAGIC_IF_NOT:
        if (av && nz(a, lf)) { r = b; rvld = bv; }
        else { r = rf ? d2b(MAGIC_D) : (uint64_t)MAGIC_I; rvld = false; }
        break;
      case OP_FIRST_NON_MAGIC: {
        bool is_magic = lf ? (b2d(a) == MAGIC_D) : (ai == MAGIC_I);
        if (is_magic) { r = b; rvld = bv; } else { r = a; rvld = av; }
        break;
      }
      case OP_OR:
        if (av && bv) { r = (uint64_t)(nz(a, lf) || nz(b, rf)); rvld = true; }
        else if (av) { r = a; rvld = nz(a, lf); }
        else if (bv) { r = b; rvld = true; }
        else { r = 0; rvld = false; }
        break;
      case OP_IS_NOT_DISTINCT_FROM:
        if (!av && !bv) r = 1;
        else if (!av || !bv) r = 0;
        else r = anyf ? (ad == bd) : (ai == bi);
        rvld = true;
        break;
      default:
        if (!(av && bv)) { r = 0; rvld = false; break; }  // DIVERGENCE: data under NULL defined as 0
        rvld = true;
        switch (op) {
          case OP_AND: r = nz(a, lf) && nz(b, rf); break;
          case OP_ADD: r = anyf ? d2b(ad + bd) : (uint64_t)a + (uint64_t)b; break;
          case OP_SUB: r = anyf ? d2b(ad - bd) : (uint64_t)a - (uint64_t)b; break;
          case OP_MUL: r = anyf ? d2b(ad * bd) : (uint64_t)a * (uint64_t)b; break;
          case OP_DIV:
            if (anyf) r = d2b(ad / bd);
            else if (bi == 0) r = 0;
            else if (bi == -1) r = (uint64_t)0 - a;
            else r = (uint64_t)(ai / bi);
            if (rf ? (bd == 0.0) : (bi == 0)) { rvld = false; r = 0; }
            break;
          case OP_MOD:
            if (anyf) r = d2b(std::fmod(ad, bd));
            else if (bi == 0) { r = 0; rvld = false; }  // DIVERGENCE: integer MOD by 0 is NULL
            else if (bi == -1) r = 0;
            else r = (uint64_t)(ai % bi);
            break;
          case OP_POW: r = d2b(std::pow(ad, bd)); break;
          case OP_ROUND: {
            double f = pow10_scale(bd);
            double prod = ad * f;
            r = d2b(std::round(prod) / f);
            break;
          }
          case OP_EQUAL: case OP_NOT_EQUAL: case OP_LESS: case OP_GREATER: case OP_LESS_EQUAL: case OP_GREATER_EQUAL: {
            int c;  // -1, 0, 1, or 2 for unordered
            if (ts_cmp) {
              int64_t x = to_ns(lt, ai), y = to_ns(rt, bi);
              c = x < y ? -1 : (x > y ? 1 : 0);
            } else if (anyf) {
              c = ad < bd ? -1 : (ad > bd ? 1 : (ad == bd ? 0 : 2));
            } else {
              c = ai < bi ? -1 : (ai > bi ? 1 : 0);
            }
            bool res;
            switch (op) {
              case OP_EQUAL: res = c == 0; break;
              case OP_NOT_EQUAL: res = c != 0; break;
              case OP_LESS: res = c == -1; break;
              case OP_GREATER: res = c == 1; break;
              case OP_LESS_EQUAL: res = c == -1 || c == 0; break;
              default: res = c == 1 || c == 0; break;
            }
            r = res;
            break;
          }
          default: break;
        }
    }
    ob[i] = r;
    ov[i] = rvld;
  }
}

// store into an output column of type `t` (device_ptr_write_from_buffer,
// interpreter_ops.cuh:329-395): integer columns take static_cast<T>(int64 bits),
// float columns static_cast<T>(double of bits), timestamps the int64 count.
static void store_value(uint8_t* data, int t, int64_t row, uint64_t bits) {
  switch (t) {
    case INT8: ((int8_t*)data)[row] = (int8_t)(int64_t)bits; break;
    case INT16: ((int16_t*)data)[row] = (int16_t)(int64_t)bits; break;
    case INT32: case TIMESTAMP_DAYS: case DURATION_DAYS: ((int32_t*)data)[row] = (int32_t)(int64_t)bits; break;
    case UINT8: ((uint8_t*)data)[row] = (uint8_t)bits; break;
    case BOOL8: ((uint8_t*)data)[row] = bits != 0; break;
    case UINT16: ((uint16_t*)data)[row] = (uint16_t)bits; break;
    case UINT32: ((uint32_t*)data)[row] = (uint32_t)bits; break;
    case FLOAT32: ((float*)data)[row] = (float)b2d(bits); break;
    case FLOAT64: ((double*)data)[row] = b2d(bits); break;
    default: ((uint64_t*)data)[row] = bits; break;
  }
}

// ---------------------------------------------------------------------------
// Compiled expression set
// ---------------------------------------------------------------------------
struct OutSpec {
  enum Kind { OP_RESULT, COPY_COL, BROADCAST } kind;
  int type;           // output column type
  int temp = -1;      // OP_RESULT: temp index
  int col = -1;       // COPY_COL: source column
  Scalar lit;         // BROADCAST
};

struct Compiled {
  Program prog;
  std::vector<OutSpec> outs;
};

static std::unique_ptr<Node> build_tree(const std::string& raw) {
  std::string e = replace_calcite_regex(raw);
  e = expand_if_logical_op(e);
  Parser ps(e);
  auto root = ps.expr();
  return custom_ops(std::move(root));
}

static Compiled compile(const std::vector<std::string>& exprs, const std::vector<int>& col_types) {
  Compiled C;
  int rand_counter = 0;
  for (const auto& raw : exprs) {
    auto root = build_tree(raw);
    annotate(root.get(), col_types);
    OutSpec o;
    if (root->kind == N_LIT) {
      o.kind = OutSpec::BROADCAST;
      o.type = root->lit_type;
      if (o.type == EMPTY) throw Error(E_TYPE, "a bare null literal has no column type");
      o.lit = make_scalar(root->value, root->lit_type);
    } else if (root->kind == N_VAR) {
      o.kind = OutSpec::COPY_COL;
      o.col = root->var_index;
      o.type = col_types[o.col];
    } else {
      o.kind = OutSpec::OP_RESULT;
      o.type = root->vtype;
      if (o.type == EMPTY || o.type == STRING || size_of(o.type) == 0) throw Error(E_TYPE, "expression has no fixed-width output type");
      Src s = emit(root.get(), C.prog, rand_counter);
      o.temp = s.idx;
    }
    C.outs.push_back(o);
  }
  C.prog.nrand = rand_counter;
  return C;
}

struct OutCol { int type; uint8_t* data; uint32_t* mask; int64_t size; };

static void parallel_for_chunks(int64_t nrows, int nthreads, const std::function<void(int64_t, int64_t)>& fn) {
  // contiguous per-thread ranges aligned to 32-row words
  if (nthreads <= 1 || nrows < 4096) { fn(0, nrows); return; }
  int64_t words = (nrows + 31) / 32;
  int64_t per = (words + nthreads - 1) / nthreads;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++) {
    int64_t a = std::min(nrows, t * per * 32), b = std::min(nrows, (t + 1) * per * 32);
    if (a >= b) break;
    th.emplace_back([&, a, b] { fn(a, b); });
  }
  for (auto& x : th) x.join();
}

static void eval_range(const Compiled& C, const std::vector<Column>& cols, int64_t a, int64_t b, uint64_t seed,
                       std::vector<OutCol>& outs) {
  Scratch sc;
  sc.init(std::max(1, C.prog.ntemps));
  std::vector<uint64_t> lb, rb;
  std::vector<uint8_t> lv, rv;
  for (int64_t r0 = a; r0 < b; r0 += CHUNK) {
    int n = (int)std::min<int64_t>(CHUNK, b - r0);
    for (const auto& st : C.prog.steps) run_step(st, cols, sc, r0, n, seed, lb, lv, rb, rv);
    for (size_t k = 0; k < C.outs.size(); k++) {
      const OutSpec& o = C.outs[k];
      OutCol& oc = outs[k];
      for (int i = 0; i < n; i++) {
        int64_t row = r0 + i;
        uint64_t bits;
        bool v;
        if (o.kind == OutSpec::OP_RESULT) { bits = sc.b(o.temp)[i]; v = sc.v(o.temp)[i]; }
        else if (o.kind == OutSpec::COPY_COL) { bits = read_bits(cols[o.col], row); v = read_valid(cols[o.col], row); }
        else { bits = o.lit.bits; v = o.lit.valid; }
        if (o.kind == OutSpec::COPY_COL) {
          // deep copy keeps the raw element (no 64-bit round trip)
          const Column& c = cols[o.col];
          int w = size_of(c.type);
          memcpy(oc.data + row * w, c.data + (c.offset + row) * w, w);
        } else {
          store_value(oc.data, o.type, row, bits);
        }
        // each 32-row word belongs to exactly one thread (ranges are word aligned)
        if (v) oc.mask[row >> 5] |= (1u << (row & 31));
        else oc.mask[row >> 5] &= ~(1u << (row & 31));
      }
    }
  }
}

static OutCol alloc_out(int type, int64_t n) {
  OutCol o;
  o.type = type;
  o.size = n;
  int w = size_of(type);
  o.data = (uint8_t*)calloc((size_t)std::max<int64_t>(1, n) * w, 1);
  int64_t words = (n + 31) / 32;
  o.mask = (uint32_t*)calloc((size_t)std::max<int64_t>(1, (words + 15) / 16 * 16), 4);
  return o;
}

static std::vector<OutCol> evaluate(const std::vector<Column>& cols, const std::vector<std::string>& exprs, int nthreads,
                                    uint64_t seed) {
  std::vector<int> types;
  int64_t n = cols.empty() ? 0 : cols[0].size;
  for (auto& c : cols) types.push_back(c.type);
  Compiled C = compile(exprs, types);
  std::vector<OutCol> outs;
  for (auto& o : C.outs) outs.push_back(alloc_out(o.type, n));
  parallel_for_chunks(n, nthreads, [&](int64_t a, int64_t b) { eval_range(C, cols, a, b, seed, outs); });
  return outs;
}

// applyBooleanFilter -> cudf::apply_boolean_mask: keep row iff the mask row is
// valid and true; stable order; every input column is compacted.
static std::vector<OutCol> compact(const std::vector<Column>& cols, const OutCol& mask, int nthreads, int64_t& out_rows) {
  int64_t n = mask.size;
  int T = (nthreads <= 1 || n < 4096) ? 1 : nthreads;
  int64_t words = (n + 31) / 32, per = (words + T - 1) / T;
  std::vector<int64_t> cnt(T + 1, 0);
  auto keep = [&](int64_t r) { return ((mask.mask[r >> 5] >> (r & 31)) & 1u) && mask.data[r] != 0; };
  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) {
    th.emplace_back([&, t] {
      int64_t a = std::min(n, t * per * 32), b = std::min(n, (t + 1) * per * 32), c = 0;
      for (int64_t r = a; r < b; r++) c += keep(r);
      cnt[t + 1] = c;
    });
  }
  for (auto& x : th) x.join();
  th.clear();
  for (int t = 0; t < T; t++) cnt[t + 1] += cnt[t];
  out_rows = cnt[T];
  std::vector<OutCol> outs;
  for (auto& c : cols) outs.push_back(alloc_out(c.type, out_rows));
  for (int t = 0; t < T; t++) {
    th.emplace_back([&, t] {
      int64_t a = std::min(n, t * per * 32), b = std::min(n, (t + 1) * per * 32), o = cnt[t];
      for (int64_t r = a; r < b; r++) {
        if (!keep(r)) continue;
        for (size_t k = 0; k < cols.size(); k++) {
          const Column& c = cols[k];
          int w = size_of(c.type);
          memcpy(outs[k].data + o * w, c.data + (c.offset + r) * w, w);
          if (read_valid(c, r)) __atomic_fetch_or(&outs[k].mask[o >> 5], 1u << (o & 31), __ATOMIC_RELAXED);
        }
        o++;
      }
    });
  }
  for (auto& x : th) x.join();
  return outs;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface used by the tests and the bench's CPU-baseline leg
// ---------------------------------------------------------------------------
extern "C" {

typedef struct oracle_column {
  int32_t type_id;
  int32_t pad_;
  const void* data;
  const uint32_t* null_mask;
  int64_t offset;
  int64_t size;
} oracle_column;

typedef struct oracle_out_column {
  int32_t type_id;
  int32_t pad_;
  void* data;
  uint32_t* null_mask;
  int64_t size;
} oracle_out_column;

static std::vector<orc::Column> to_cols(const oracle_column* c, int n) {
  std::vector<orc::Column> v;
  for (int i = 0; i < n; i++) v.push_back({c[i].type_id, (const uint8_t*)c[i].data, c[i].null_mask, c[i].offset, c[i].size});
  return v;
}

static int fail(const orc::Error& e, char* err, int errlen) {
  if (err && errlen > 0) snprintf(err, errlen, "%s", e.what());
  return e.code;
}

static void export_cols(const std::vector<orc::OutCol>& o, oracle_out_column* out) {
  for (size_t i = 0; i < o.size(); i++) out[i] = {o[i].type, 0, o[i].data, o[i].mask, o[i].size};
}

int oracle_evaluate_expressions(const oracle_column* cols, int ncols, const char* const* exprs, int nexprs,
                                oracle_out_column* out, int nthreads, uint64_t seed, char* err, int errlen) {
  try {
    std::vector<std::string> e(exprs, exprs + nexprs);
    export_cols(orc::evaluate(to_cols(cols, ncols), e, nthreads, seed), out);
    return 0;
  } catch (const orc::Error& x) {
    return fail(x, err, errlen);
  } catch (const std::exception& x) {
    return fail(orc::Error(orc::E_PARSE, x.what()), err, errlen);
  }
}

// process_filter (LogicalFilter.cpp:31-52).  `out` receives ncols columns.
int oracle_process_filter(const oracle_column* cols, int ncols, const char* query_part, oracle_out_column* out,
                          int64_t* out_rows, int nthreads, char* err, int errlen) {
  try {
    auto cv = to_cols(cols, ncols);
    int64_t n = ncols ? cv[0].size : 0;
    if (n == 0) {
      for (int i = 0; i < ncols; i++) { auto o = orc::alloc_out(cv[i].type, 0); out[i] = {o.type, 0, o.data, o.mask, 0}; }
      *out_rows = 0;
      return 0;
    }
    std::string qp(query_part);
    std::string cond = orc::get_named_expression(qp, "condition");
    if (cond.empty()) cond = orc::get_named_expression(qp, "filters");
    std::vector<int> schema;
    for (auto& c : cv) schema.push_back(c.type);
    cond = orc::preprocess_expression(cond, schema);
    auto m = orc::evaluate(cv, {cond}, nthreads, 0);
    if (m[0].type != orc::BOOL8) {
      free(m[0].data); free(m[0].mask);
      throw orc::Error(orc::E_TYPE, "Expression does not evaluate to a boolean mask");
    }
    auto o = orc::compact(cv, m[0], nthreads, *out_rows);
    free(m[0].data); free(m[0].mask);
    export_cols(o, out);
    return 0;
  } catch (const orc::Error& x) {
    return fail(x, err, errlen);
  } catch (const std::exception& x) {
    return fail(orc::Error(orc::E_PARSE, x.what()), err, errlen);
  }
}

// process_project (LogicalProject.cpp:943-969).  Returns the number of output
// columns in *nout (out must hold at least max_out entries).
int oracle_process_project(const oracle_column* cols, int ncols, const char* query_part, oracle_out_column* out,
                           int max_out, int* nout, int nthreads, uint64_t seed, char* err, int errlen) {
  try {
    auto cv = to_cols(cols, ncols);
    std::string combined = orc::get_query_part(query_part);
    auto named = orc::split_expression_list(combined, false);
    std::vector<int> schema;
    for (auto& c : cv) schema.push_back(c.type);
    std::vector<std::string> exprs;
    for (auto& ne : named) {
      size_t p = ne.find("=[");
      if (p == std::string::npos) throw orc::Error(orc::E_PARSE, "project item without name=[expr]: " + ne);
      std::string e = ne.substr(p + 2, ne.size() - p - 3);
      if (e.find(" OVER ") != std::string::npos) throw orc::Error(orc::E_UNSUPPORTED, "window functions out of scope");
      exprs.push_back(orc::preprocess_expression(e, schema));
    }
    if ((int)exprs.size() > max_out) throw orc::Error(orc::E_PARSE, "too many projections for output buffer");
    export_cols(orc::evaluate(cv, exprs, nthreads, seed), out);
    *nout = (int)exprs.size();
    return 0;
  } catch (const orc::Error& x) {
    return fail(x, err, errlen);
  } catch (const std::exception& x) {
    return fail(orc::Error(orc::E_PARSE, x.what()), err, errlen);
  }
}

// Filter then project on the surviving rows: process_project(process_filter(T)).
int oracle_filter_project(const oracle_column* cols, int ncols, const char* condition, const char* const* exprs,
                          int nexprs, oracle_out_column* out, int64_t* out_rows, int nthreads, uint64_t seed, char* err,
                          int errlen) {
  try {
    auto cv = to_cols(cols, ncols);
    std::vector<int> schema;
    for (auto& c : cv) schema.push_back(c.type);
    std::string cond = orc::preprocess_expression(condition, schema);
    int64_t n = ncols ? cv[0].size : 0;
    std::vector<orc::OutCol> filtered;
    int64_t rows = 0;
    if (n > 0) {
      auto m = orc::evaluate(cv, {cond}, nthreads, seed);
      if (m[0].type != orc::BOOL8) {
        free(m[0].data); free(m[0].mask);
        throw orc::Error(orc::E_TYPE, "Expression does not evaluate to a boolean mask");
      }
      filtered = orc::compact(cv, m[0], nthreads, rows);
      free(m[0].data); free(m[0].mask);
    } else {
      for (auto& c : cv) filtered.push_back(orc::alloc_out(c.type, 0));
    }
    std::vector<orc::Column> fc;
    for (auto& f : filtered) fc.push_back({f.type, f.data, f.mask, 0, rows});
    std::vector<std::string> e;
    for (int i = 0; i < nexprs; i++) e.push_back(orc::preprocess_expression(exprs[i], schema));
    auto o = orc::evaluate(fc, e, nthreads, seed);
    for (auto& f : filtered) { free(f.data); free(f.mask); }
    export_cols(o, out);
    *out_rows = rows;
    return 0;
  } catch (const orc::Error& x) {
    return fail(x, err, errlen);
  } catch (const std::exception& x) {
    return fail(orc::Error(orc::E_PARSE, x.what()), err, errlen);
  }
}

// Parse + normalise + lower an expression and print the rebuilt tree (used by
// the parser tests: CASE lowering, CAST renaming, n-ary AND nesting).
int oracle_rebuild_expression(const char* expr, char* out, int outlen) {
  try {
    std::string e = orc::replace_calcite_regex(expr);
    e = orc::expand_if_logical_op(e);
    orc::Parser ps(e);
    auto root = orc::custom_ops(ps.expr());
    std::function<std::string(const orc::Node*)> rb = [&](const orc::Node* n) -> std::string {
      if (n->kind != orc::N_OP) return n->value;
      std::string s;
      for (auto& c : n->ch) s += (s.empty() ? "" : ", ") + rb(c.get());
      return n->value + "(" + s + ")";
    };
    snprintf(out, outlen, "%s", rb(root.get()).c_str());
    return 0;
  } catch (const orc::Error& x) {
    snprintf(out, outlen, "%s", x.what());
    return x.code;
  }
}

int oracle_string_transform(const char* which, const char* in, char* out, int outlen) {
  std::string w(which), s(in), r;
  try {
    if (w == "fill_minus_op_with_zero") r = orc::fill_minus_op_with_zero(s);
    else if (w == "expand_if_logical_op") r = orc::expand_if_logical_op(s);
    else if (w == "replace_calcite_regex") r = orc::replace_calcite_regex(s);
    else if (w == "get_query_part") r = orc::get_query_part(s);
    else return -1;
  } catch (const orc::Error& x) {
    snprintf(out, outlen, "%s", x.what());
    return x.code;
  }
  snprintf(out, outlen, "%s", r.c_str());
  return 0;
}

double oracle_round_scale(double d) { return orc::pow10_scale(d); }
double oracle_philox_uniform(uint64_t seed, uint32_t rand_id, uint64_t row) { return orc::philox_uniform(seed, rand_id, row); }

void oracle_free_columns(oracle_out_column* cols, int n) {
  for (int i = 0; i < n; i++) { free(cols[i].data); free(cols[i].null_mask); cols[i].data = nullptr; cols[i].null_mask = nullptr; }
}

}  // extern "C"
