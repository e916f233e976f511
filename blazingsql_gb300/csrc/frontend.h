// frontend.h -- RexNode text -> typed expression tree.
//
// Accepts the Calcite RexNode grammar BlazingSQL's parser accepts
// (engine/src/parser/expression_tree.cpp:183-279) and applies the same
// normalisation (expression_utils.cpp:1068-1113, 1624-1632), n-ary AND/OR
// nesting (CalciteExpressionParsing.cpp:330-398), CASE / ROUND / CAST-literal
// lowering (expression_tree.hpp:181-258) and result-type rules
// (expression_utils.cpp:115-266).  No std::regex: the lexer is a hand-written
// scanner (the reference runs ~14 regex searches per token).
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "gx_common.h"

namespace gx {

struct Expr;
using ExprPtr = std::shared_ptr<Expr>;

struct Expr {
  enum Kind { COL, LIT, OP } kind = OP;
  Op op = OP_NONE;
  std::string token;          // operator token / literal text (diagnostics, rebuild)
  int col = -1;               // COL
  int lit_type = EMPTY;       // LIT: declared / inferred type
  bool lit_valid = false;     // LIT: false for a null literal
  uint64_t lit_bits = 0;      // LIT: value as the kernel reads it (int64 or double bits)
  std::string lit_type_token; // LIT: the explicit ":TYPE" of the text, if any
  int vtype = EMPTY;          // result type as expr_output_type_visitor computes it
  int ktype = EMPTY;          // result type as perform_interpreter_operation computes it
  std::vector<ExprPtr> ch;
};

// Whole-expression pipeline of evaluate_expressions for one expression:
// normalise, nest n-ary AND/OR, parse, lower CASE/ROUND/CAST-literal, type.
ExprPtr compile_expression(const std::string& text, const std::vector<int>& schema);

// preprocess_expression (expression_utils.cpp:1624-1632)
std::string preprocess_expression(const std::string& text, const std::vector<int>& schema);
// the same with only some of its rewrites: unary minus, CURRENT_DATE /
// CURRENT_TIMESTAMP, millisecond-to-nanosecond units, Reinterpret casts,
// interval units (expression_utils.cpp:1155-1164, 1494-1518, 1316-1350,
// 1371-1420, 1425-1460)
constexpr int kPreMinus = 1, kPreCurrent = 2, kPreMsToNs = 4, kPreReinterpret = 8, kPreInterval = 16, kPreAll = 31;
std::string preprocess_stages(const std::string& text, const std::vector<int>& schema, int stages);
// The calling thread's query timestamp ("YYYY-MM-DD hh:mm:ss[.fraction]", as the
// engine Context keeps it, Context.h:47; empty: none), which CURRENT_DATE,
// CURRENT_TIME and CURRENT_TIMESTAMP take in the calls that thread makes.
void set_current_timestamp(const std::string& ts);
std::string current_timestamp();

// get_named_expression (expression_utils.cpp:537-547)
std::string named_expression(const std::string& query_part, const std::string& name);

// get_query_part (expression_utils.cpp:764-769)
std::string query_part_of(const std::string& plan_text);

// get_expressions_from_expression_list (expression_utils.cpp:1012-1066); applies
// the Calcite normalisation to the text first, as the reference does.
std::vector<std::string> split_expression_list(std::string text, bool trim_items);

// Splits a LogicalProject(...) query part into (names, expressions).
void split_projections(const std::string& plan_text, std::vector<std::string>& names,
                       std::vector<std::string>& exprs);

// Rebuilds a (lowered) expression tree as text: "OP(a, b)".
std::string rebuild(const ExprPtr& e);

// Parse + lower without typing (used by tests of the lowering rules).
ExprPtr parse_and_lower(const std::string& text);

constexpr int kMaxConcatParts = 8;  // parts one CONCAT operator of the pre-pass joins

// A string operator of the string pre-pass (the operators of
// evaluate_string_functions, LogicalProject.cpp:103-603, and the
// interpreter's string comparisons).
struct StringOp {
  enum Kind {
    LIKE = 0, EQ, NE, LT, LE, GT, GE, CHAR_LENGTH,
    CASE,       // THEN (col / literal / null) where cond is true, else ELSE (col2 / literal2 / null)
    SLICE,      // cudf::strings::slice_strings by characters: [i0, i1) with validity flags, step (+1 / -1),
                // or [pos0, pos1) per row
    UPPER, LOWER, INITCAP,
    TRIM,       // side i0 (0 both, 1 leading, 2 trailing), characters to strip in `literal`
    REPLACE,    // every `literal` by `literal2`
    CONCAT,     // (col | literal) followed by (col2 | literal2)
    TO_STRING,  // CAST to VARCHAR of column `col` (or of the expression `cond`), formatted by its type
    PARSE,      // CAST of string column `col` to `type` (integers, floating point, DATE, TIMESTAMPs)
    REGEXP_REPLACE  // matches of pattern `literal` replaced by template `literal2`, after the first i0
                    // characters when i0_valid
  };
  Kind kind = LIKE;
  int col = -1;         // the (first) string column; CASE: the THEN column, or -1
  std::string literal;  // pattern / literal, quotes removed; CASE: the THEN literal
  int col2 = -1;        // comparisons: the right-hand string column; CASE: the ELSE column, or -1
  // CASE: `cond` (text over the columns before this operator) selects THEN
  // where it is true, ELSE where it is false or NULL
  // (evaluate_string_case_when_else, LogicalProject.cpp:612-659); an operand
  // without a column is its literal, or NULL when *_null is set.
  // TO_STRING: the expression whose column is formatted when col < 0.
  std::string cond;
  std::string literal2;  // the ELSE / second literal
  bool then_null = false, else_null = false;
  int i0 = 0, i1 = 0, step = 1;
  bool i0_valid = false, i1_valid = false;
  // SLICE with positions per row (SUBSTRING whose start or length is not a
  // literal): the texts of the zero-based start and of the stop (empty: to
  // the end), over the columns before this operator; i0 / i1 are then unused
  std::string pos0, pos1;
  int type = 0;  // PARSE: the result type
  // CONCAT of more than two parts: parts 3, 4, ... (a column, or -1 and the literal)
  std::vector<int> more_cols;
  std::vector<std::string> more_lits;
  bool operator==(const StringOp& o) const {
    return kind == o.kind && col == o.col && literal == o.literal && col2 == o.col2 && cond == o.cond &&
           literal2 == o.literal2 && then_null == o.then_null && else_null == o.else_null && i0 == o.i0 &&
           i1 == o.i1 && step == o.step && i0_valid == o.i0_valid && i1_valid == o.i1_valid && type == o.type &&
           more_cols == o.more_cols && more_lits == o.more_lits && pos0 == o.pos0 && pos1 == o.pos1;
  }
  int result_type() const {
    switch (kind) {
      case CHAR_LENGTH: return INT32;
      case PARSE: return type;
      case LIKE: case EQ: case NE: case LT: case LE: case GT: case GE: return BOOL8;
      default: return STRING;
    }
  }
};

// The string pre-pass of function_evaluator_transformer
// (LogicalProject.cpp:671-742), children before parents as the reference's
// node_transformer visits them: in each (preprocessed) expression text, every
// string operator becomes the column $(schema.size() + i) of op i (shared by
// equal operators), so a later operator can read an earlier one's column.
// A string column (read or made) may then remain only as a whole expression
// (a string output); anywhere else it fails with GX_ERR_UNSUPPORTED.
// Texts without string columns or string literals are returned as they are.
void rewrite_string_ops(std::vector<std::string>& texts, const std::vector<int>& schema,
                        std::vector<StringOp>& ops);

// The column a (rewritten) expression text passes through whole ("$n"), or -1.
int passthrough_column(const std::string& text);

// True when the whole expression is a string literal; *value receives it
// without quotes.
bool string_literal_value(const std::string& text, std::string* value);

// The row-group pruning form of a TableScan condition (ral::skip_data,
// engine/src/skip_data/SkipDataProcessor.cpp:215-232 and :23-212): operands
// $i listed in `dropped` (columns without statistics) are removed, operators
// other than = < <= > >= + - AND OR are removed (an AND keeps its other side,
// anything else loses the whole comparison), then each comparison is
// restated over $2i (min) and $2i+1 (max) of the columns.  Returns the new
// condition's text, or "" when nothing usable is left; *prefix_form (optional)
// receives the tree in the reference's prefix notation ("NONE" when unusable).
std::string skip_data_rewrite(const std::string& condition, const std::vector<int>& dropped,
                              std::string* prefix_form);

}  // namespace gx
