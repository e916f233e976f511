// gx_common.h -- shared host-side definitions of the evaluator library.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gx_eval.h"

namespace gx {

// cudf::type_id numbering (see include/gx_eval.h)
enum TypeId : int32_t {
  EMPTY = 0, INT8, INT16, INT32, INT64, UINT8, UINT16, UINT32, UINT64, FLOAT32, FLOAT64, BOOL8,
  TIMESTAMP_DAYS, TIMESTAMP_SECONDS, TIMESTAMP_MILLISECONDS, TIMESTAMP_MICROSECONDS, TIMESTAMP_NANOSECONDS,
  DURATION_DAYS, DURATION_SECONDS, DURATION_MILLISECONDS, DURATION_MICROSECONDS, DURATION_NANOSECONDS,
  DICTIONARY32, STRING
};

inline bool is_float(int t) { return t == FLOAT32 || t == FLOAT64; }
inline bool is_integer(int t) { return t >= INT8 && t <= UINT64; }
inline bool is_timestamp(int t) { return t >= TIMESTAMP_DAYS && t <= TIMESTAMP_NANOSECONDS; }
inline bool is_duration(int t) { return t >= DURATION_DAYS && t <= DURATION_NANOSECONDS; }
inline int type_size(int t) {
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

// Row-wise operators (the reference's operator_type, engine/src/parser/expression_utils.hpp:11-93,
// restricted to the fixed-width ops the interpreter evaluates, plus EXP).
enum Op : int32_t {
  OP_NONE = 0,
  OP_RAND,
  OP_ROW_INDEX,  // internal: the input row of the current row (compaction maps)
  // unary
  OP_NOT, OP_ABS, OP_FLOOR, OP_CEIL, OP_SIN, OP_COS, OP_ASIN, OP_ACOS, OP_TAN, OP_COTAN, OP_ATAN,
  OP_LN, OP_LOG10, OP_EXP, OP_YEAR, OP_MONTH, OP_DAY, OP_DAYOFWEEK, OP_HOUR, OP_MINUTE, OP_SECOND,
  OP_IS_NULL, OP_IS_NOT_NULL, OP_IS_TRUE, OP_IS_NOT_TRUE, OP_IS_NOT_FALSE,
  OP_CAST_TINYINT, OP_CAST_SMALLINT, OP_CAST_INTEGER, OP_CAST_BIGINT, OP_CAST_FLOAT, OP_CAST_DOUBLE,
  OP_CAST_DATE, OP_CAST_TIMESTAMP_SECONDS, OP_CAST_TIMESTAMP_MILLISECONDS, OP_CAST_TIMESTAMP_MICROSECONDS,
  OP_CAST_TIMESTAMP,
  // binary
  OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MOD, OP_POW, OP_ROUND,
  OP_EQ, OP_NE, OP_LT, OP_GT, OP_LE, OP_GE,
  OP_AND, OP_OR, OP_FIRST_NON_MAGIC, OP_MAGIC_IF_NOT, OP_IS_NOT_DISTINCT_FROM,
};

inline bool op_is_unary(Op op) { return op >= OP_NOT && op <= OP_CAST_TIMESTAMP; }
inline bool op_is_binary(Op op) { return op >= OP_ADD && op <= OP_IS_NOT_DISTINCT_FROM; }

struct Error : std::runtime_error {
  gx_status code;
  Error(gx_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(gx_status c, const std::string& m) { throw Error(c, m); }

}  // namespace gx
