// str_prepass.h -- the string pre-pass (str_prepass.cu): string operators over string
// columns evaluated into BOOL8 / INT32 / string columns before the plan kernels
// run, and the builder of string output columns (copies, gathers, CASE).
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

#include "frontend.h"
#include "runtime.h"

namespace gx {

struct LikeDfa;

// LIKE of `text` through the pattern's byte automaton, run on the host as the
// kernel runs it: 1 match, 0 no match, -1 when the pattern is left to the
// backtracking matcher (no automaton)
int like_dfa_host_match(const std::string& pattern, const unsigned char* text, int64_t n);

// one operator over string column `op.col` (and `col2`, the right-hand column
// of a comparison of two columns, or null), writing `out` (library column of
// col.size rows: BOOL8, INT32 for CHAR_LENGTH); pattern_dev holds op.literal,
// or for a LIKE with an automaton (dfa) the automaton's bytes
void launch_string_op(const ColumnView& col, const ColumnView* col2, const StringOp& op, const void* pattern_dev,
                      gx_column& out, cudaStream_t s, const LikeDfa* dfa = nullptr);

// Where the rows of a string column being built come from: a string column
// (`col`), a literal (`literal`, host bytes that build_strings copies to the
// device), NULL, or (a CONCAT part) a typed column `col` formatted as CAST to
// VARCHAR formats it.
struct StrSource {
  enum Kind { COLUMN = 0, LITERAL = 1, NUL = 2, FORMAT = 3 } kind = NUL;
  ColumnView col{};
  std::string literal;
};

// Builds a cudf strings column of `rows` rows (library-owned: characters in
// `data`, offsets in `string_offsets`, validity always present):
//  * map set: row o is a's row map[o] (a gather, a: a column);
//  * cond set (a BOOL8 view of `rows` rows): row o is a's where cond is valid
//    and true, else b's (cudf::copy_if_else, which the reference's string CASE
//    calls, LogicalProject.cpp:639-655);
//  * neither: row o is a's row o (a copy, or a literal repeated).
// A NULL row is empty.  Returns once the column is complete on the stream
// (the character count is read back to size the characters).
gx_column build_strings(const StrSource& a, const StrSource& b, const int32_t* map, const ColumnView* cond,
                        int64_t rows, cudaStream_t s);

// Evaluates `ops` over `cols` and appends their columns to `cols` (column
// ncols + i is op i).  eval_bool evaluates an expression's text over the
// columns so far into a column: a CASE condition (BOOL8), the operand of a
// CAST to VARCHAR, a SUBSTRING's start or stop (integers).  The returned columns are the caller's
// to free once the work that reads them has been enqueued.
using EvalText = std::function<gx_column(const std::vector<ColumnView>&, const std::string&)>;
// defer (optional, per op): ops to skip here, for transform_column to make
// later over the kept rows; their columns are appended as empty placeholders.
std::vector<gx_column> run_string_prepass(std::vector<ColumnView>& cols, const std::vector<StringOp>& ops,
                                          cudaStream_t s, const EvalText& eval_bool,
                                          const std::vector<bool>* defer = nullptr);

// The operators whose result is built row by row from the rows of their
// inputs (casts to VARCHAR, slices, case mappings, TRIM, REPLACE, CONCAT,
// REGEXP_REPLACE): these can be made after a filter, for its kept rows only.
bool is_deferrable(const StringOp& op);

// Such an operator over `cols` (every input row) into a string column of
// `rows` rows; with map, output row o is made from input row map[o] (the
// kept rows of a filter, LogicalFilter.cpp:22-29, gathered while building).
gx_column transform_column(const StringOp& op, const std::vector<ColumnView>& cols, const int32_t* map,
                           int64_t rows, cudaStream_t s, const EvalText& eval_bool);

}  // namespace gx
