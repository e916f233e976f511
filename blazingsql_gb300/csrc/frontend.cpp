// frontend.cpp -- RexNode text -> typed expression tree (see frontend.h).
#include "frontend.h"
#include "regex.h"

#include <functional>

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>

namespace gx {
namespace {

// ---------------------------------------------------------------- text utils
bool digit(char c) { return c >= '0' && c <= '9'; }

void replace_all(std::string& s, const std::string& from, const std::string& to) {
  size_t p = 0;
  while ((p = s.find(from, p)) != std::string::npos) {
    s.replace(p, from.size(), to);
    p += to.size();
  }
}

std::string replace_first(const std::string& s, const std::string& from, const std::string& to) {
  std::string r = s;
  size_t p = r.find(from);
  if (p != std::string::npos) r.replace(p, from.size(), to);
  return r;
}

std::string ltrim(const std::string& s) {
  size_t i = 0;
  while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
  return s.substr(i);
}

std::string trim(const std::string& s) {
  std::string t = ltrim(s);
  size_t j = t.size();
  while (j > 0 && std::isspace((unsigned char)t[j - 1])) j--;
  return t.substr(0, j);
}

bool ieq(char a, char b) { return std::toupper((unsigned char)a) == std::toupper((unsigned char)b); }

// case-insensitive match of `word` at s[p]
bool imatch(const std::string& s, size_t p, const char* word) {
  size_t n = std::strlen(word);
  if (p + n > s.size()) return false;
  for (size_t i = 0; i < n; i++)
    if (!ieq(s[p + i], word[i])) return false;
  return true;
}

size_t count_digits(const std::string& s, size_t p) {
  size_t n = 0;
  while (p + n < s.size() && digit(s[p + n])) n++;
  return n;
}

// Rewrites "<word>(<digits>[, <digits>])" case-insensitively (the reference's
// TIMESTAMP(\d+), DECIMAL(\d+, \d+) and :CHAR(\d+) regex rules).
std::string rewrite_paren_digits(const std::string& s, const char* word, bool two, const char* repl) {
  std::string out;
  size_t i = 0, wl = std::strlen(word);
  while (i < s.size()) {
    if (imatch(s, i, word) && i + wl < s.size() && s[i + wl] == '(') {
      size_t j = i + wl + 1, d = count_digits(s, j);
      if (d > 0) {
        j += d;
        bool ok = true;
        if (two) {
          if (s.compare(j, 2, ", ") == 0 && count_digits(s, j + 2) > 0) j += 2 + count_digits(s, j + 2);
          else ok = false;
        }
        if (ok && j < s.size() && s[j] == ')') {
          out += repl;
          i = j + 1;
          continue;
        }
      }
    }
    out += s[i++];
  }
  return out;
}

// "(\d+)? CHARACTER SET "..." COLLATE "..."" -> "" (string collation annotations)
std::string drop_collation(const std::string& s) {
  const std::string key = " CHARACTER SET \"";
  std::string out = s;
  size_t p;
  while ((p = out.find(key)) != std::string::npos) {
    size_t q = out.find("\" COLLATE \"", p + key.size());
    if (q == std::string::npos) break;
    size_t r = out.find('"', q + 11);
    if (r == std::string::npos) break;
    size_t start = p;
    if (start > 0 && out[start - 1] == ')') {
      size_t k = start - 1, d = 0;
      while (k > 0 && digit(out[k - 1])) { k--; d++; }
      if (d > 0 && k > 0 && out[k - 1] == '(') start = k - 1;
    }
    out.erase(start, r + 1 - start);
  }
  return out;
}

// replace_calcite_regex (expression_utils.cpp:1068-1113)
std::string normalize_calcite(const std::string& in) {
  std::string s = drop_collation(in);
  s = rewrite_paren_digits(s, "TIMESTAMP", false, "TIMESTAMP");
  s = rewrite_paren_digits(s, "DECIMAL", true, "DOUBLE");
  s = rewrite_paren_digits(s, ":CHAR", false, ":VARCHAR");
  replace_all(s, "IS NOT DISTINCT FROM", "IS_NOT_DISTINCT_FROM");
  replace_all(s, "IS NOT NULL", "IS_NOT_NULL");
  replace_all(s, "IS NULL", "IS_NULL");
  replace_all(s, " NOT NULL", "");
  replace_all(s, "RAND()", "BLZ_RND()");
  static const char* parts[] = {"YEAR", "MONTH", "DAY", "DOW", "HOUR", "MINUTE", "SECOND"};
  for (const char* p : parts) replace_all(s, std::string("EXTRACT(FLAG(") + p + "), ", std::string("BL_") + p + "(");
  replace_all(s, "DAY TO SECOND", "SECOND");
  replace_all(s, "HOUR TO SECOND", "SECOND");
  replace_all(s, "MINUTE TO SECOND", "SECOND");
  replace_all(s, "/INT(", "/(");
  replace_all(s, "TRIM(FLAG(BOTH),", "TRIM(\"BOTH\",");
  replace_all(s, "TRIM(FLAG(LEADING),", "TRIM(\"LEADING\",");
  replace_all(s, "TRIM(FLAG(TRAILING),", "TRIM(\"TRAILING\",");
  return s;
}

// ------------------------------------------------------------ date patterns
bool is_dd(const std::string& s, size_t p, size_t n) {
  if (p + n > s.size()) return false;
  for (size_t i = 0; i < n; i++)
    if (!digit(s[p + i])) return false;
  return true;
}
// dddd<sep>dd<sep>dd at p
bool date_at(const std::string& s, size_t p, char sep) {
  return is_dd(s, p, 4) && p + 4 < s.size() && s[p + 4] == sep && is_dd(s, p + 5, 2) && p + 7 < s.size() &&
         s[p + 7] == sep && is_dd(s, p + 8, 2);
}
bool time_at(const std::string& s, size_t p) {
  return is_dd(s, p, 2) && p + 2 < s.size() && s[p + 2] == ':' && is_dd(s, p + 3, 2) && p + 5 < s.size() &&
         s[p + 5] == ':' && is_dd(s, p + 6, 2);
}
bool is_date_text(const std::string& s) {
  return s.size() == 10 && (date_at(s, 0, '-') || date_at(s, 0, '/'));
}
// date + optional [ T] + time + optional ".fff" (frac digits) + optional Z, full match
bool is_timestamp_text(const std::string& s, int frac) {
  if (!(date_at(s, 0, '-') || date_at(s, 0, '/'))) return false;
  size_t p = 10;
  if (p < s.size() && (s[p] == ' ' || s[p] == 'T')) p++;
  if (!time_at(s, p)) return false;
  p += 8;
  if (frac > 0) {
    if (p >= s.size()) return false;
    p++;  // any separator character
    if (!is_dd(s, p, frac)) return false;
    p += frac;
  }
  if (p < s.size() && s[p] == 'Z') p++;
  return p == s.size();
}
bool is_timestamp_any(const std::string& s) {
  return is_timestamp_text(s, 0) || is_timestamp_text(s, 3) || is_timestamp_text(s, 6) || is_timestamp_text(s, 9);
}
bool is_timestamp_decimals(const std::string& s) {
  return is_timestamp_text(s, 3) || is_timestamp_text(s, 6) || is_timestamp_text(s, 9);
}

// ---------------------------------------------------------------- lexer
enum Tok { T_LP, T_RP, T_COMMA, T_COLON, T_VAR, T_NULL, T_BOOL, T_NUM, T_DUR_S, T_TS_D, T_TS_S, T_TS_MS, T_TS_NS,
           T_STR, T_IDENT, T_EOF };
struct Token {
  Tok t;
  std::string v;
};

// Token classes and their order follow expression_tree.cpp:33-160.
class Lexer {
 public:
  explicit Lexer(const std::string& s) : text_(trim(s)) {}

  Token next() {
    while (pos_ < text_.size() && text_[pos_] == ' ') pos_++;
    if (pos_ >= text_.size()) return {T_EOF, ""};
    const char c = text_[pos_];
    if (c == '(') return punct(T_LP);
    if (c == ')') return punct(T_RP);
    if (c == ',') return punct(T_COMMA);
    if (c == ':') return punct(T_COLON);
    size_t n;
    if ((n = var_len())) return take(T_VAR, n);
    if (text_.compare(pos_, 4, "null") == 0) return take(T_NULL, 4);
    if (text_.compare(pos_, 4, "true") == 0) return take(T_BOOL, 4);
    if (text_.compare(pos_, 5, "false") == 0) return take(T_BOOL, 5);
    if (time_at(text_, pos_)) return take(T_DUR_S, 8);
    if ((n = ts_len(6))) return take(T_TS_NS, n);  // the reference's ns token uses the 6-digit pattern
    if ((n = ts_len(3))) return take(T_TS_MS, n);
    if ((n = ts_len(0))) return take(T_TS_S, n);
    if (date_at(text_, pos_, '-')) return take(T_TS_D, 10);
    if ((n = num_len())) return take(T_NUM, n);
    if ((n = str_len())) return take(T_STR, n);
    size_t len = 0;
    while (pos_ + len < text_.size()) {
      char ch = text_[pos_ + len];
      if (ch == '(' || ch == ')' || ch == ',' || ch == ':') break;
      len++;
    }
    if (len == 0) len = 1;
    return take(T_IDENT, len);
  }

 private:
  Token punct(Tok t) { return take(t, 1); }
  Token take(Tok t, size_t n) {
    Token tk{t, text_.substr(pos_, n)};
    pos_ += n;
    return tk;
  }
  size_t var_len() const {
    if (text_[pos_] != '$') return 0;
    size_t d = count_digits(text_, pos_ + 1);
    return d ? d + 1 : 0;
  }
  // dddd-dd-dd([ T]?dd:dd:dd(.d{frac})?)
  size_t ts_len(int frac) const {
    if (!date_at(text_, pos_, '-')) return 0;
    size_t p = pos_ + 10;
    if (p < text_.size() && (text_[p] == ' ' || text_[p] == 'T') && time_at(text_, p + 1)) p++;
    if (!time_at(text_, p)) return 0;
    p += 8;
    if (frac > 0) {
      if (p >= text_.size() || text_[p] == '\n') return 0;
      if (!is_dd(text_, p + 1, frac)) return 0;
      p += 1 + frac;
    }
    return p - pos_;
  }
  // [-+]?\d*\.?\d+([eE][-+]?\d+)?
  size_t num_len() const {
    size_t i = pos_;
    if (text_[i] == '-' || text_[i] == '+') i++;
    size_t d1 = count_digits(text_, i), j = i + d1, end;
    if (j < text_.size() && text_[j] == '.' && count_digits(text_, j + 1) > 0) end = j + 1 + count_digits(text_, j + 1);
    else if (d1 > 0) end = j;
    else return 0;
    if (end < text_.size() && (text_[end] == 'e' || text_[end] == 'E')) {
      size_t m = end + 1;
      if (m < text_.size() && (text_[m] == '-' || text_[m] == '+')) m++;
      size_t de = count_digits(text_, m);
      if (de > 0) end = m + de;
    }
    return end - pos_;
  }
  // (["'])(?:(?!\1|\\).|\\.)*?\1
  size_t str_len() const {
    char q = text_[pos_];
    if (q != '\'' && q != '"') return 0;
    size_t i = pos_ + 1;
    while (i < text_.size()) {
      char c = text_[i];
      if (c == q) return i + 1 - pos_;
      if (c == '\\') {
        if (i + 1 >= text_.size()) return 0;
        i += 2;
        continue;
      }
      if (c == '\n') return 0;
      i++;
    }
    return 0;
  }

  std::string text_;
  size_t pos_ = 0;
};

// ---------------------------------------------------------------- literals
int type_from_token(const std::string& v) {
  static const std::unordered_map<std::string, int> M = {
      {"NULL", BOOL8}, {"BOOLEAN", BOOL8}, {"TINYINT", INT8}, {"SMALLINT", INT16}, {"INTEGER", INT32},
      {"INTERVAL SECOND", DURATION_SECONDS}, {"INTERVAL MINUTE", DURATION_SECONDS},
      {"INTERVAL HOUR", DURATION_SECONDS}, {"INTERVAL DAY", DURATION_SECONDS}, {"BIGINT", INT64},
      {"FLOAT", FLOAT32}, {"DOUBLE", FLOAT64}, {"DATE", TIMESTAMP_DAYS},
      {"TIMESTAMP_SECONDS", TIMESTAMP_SECONDS}, {"TIMESTAMP_MILLISECONDS", TIMESTAMP_MILLISECONDS},
      {"TIMESTAMP_MICROSECONDS", TIMESTAMP_MICROSECONDS}, {"TIMESTAMP", TIMESTAMP_NANOSECONDS}, {"VARCHAR", STRING}};
  if (v == "INTERVAL MONTH" || v == "INTERVAL YEAR")
    fail(GX_ERR_UNSUPPORTED, "operation over MONTH or YEAR units are not currently supported.");
  auto it = M.find(v);
  if (it == M.end()) fail(GX_ERR_PARSE, "Invalid literal cast type: " + v);
  return it->second;
}

long long parse_ll(const std::string& s, long long lo, long long hi) {
  errno = 0;
  char* end = nullptr;
  long long v = std::strtoll(s.c_str(), &end, 10);
  if (end == s.c_str() || errno == ERANGE || v < lo || v > hi) fail(GX_ERR_PARSE, "cannot convert literal '" + s + "'");
  return v;
}
unsigned long long parse_ull(const std::string& s) {
  errno = 0;
  char* end = nullptr;
  unsigned long long v = std::strtoull(s.c_str(), &end, 10);
  if (end == s.c_str() || errno == ERANGE) fail(GX_ERR_PARSE, "cannot convert literal '" + s + "'");
  return v;
}

int infer_literal_type(const Token& t) {
  switch (t.t) {
    case T_NULL: return EMPTY;
    case T_BOOL: return BOOL8;
    case T_NUM: {
      if (t.v.find_first_of(".eE") != std::string::npos) {
        double d = std::strtod(t.v.c_str(), nullptr);
        return d == (double)(float)d ? FLOAT32 : FLOAT64;
      }
      long long v = parse_ll(t.v, INT64_MIN, INT64_MAX);
      return v > 2147483647LL ? INT64 : INT32;
    }
    case T_DUR_S: return DURATION_SECONDS;
    case T_TS_NS: return TIMESTAMP_NANOSECONDS;
    case T_TS_MS: return TIMESTAMP_MILLISECONDS;
    case T_TS_S: return TIMESTAMP_SECONDS;
    case T_TS_D: return TIMESTAMP_DAYS;
    default: return STRING;
  }
}

uint64_t dbits(double d) {
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
}

int32_t fixed_int(const std::string& s, size_t p, size_t n) {
  int32_t v = 0;
  for (size_t i = 0; i < n && p + i < s.size(); i++) {
    char c = s[p + i];
    if (!digit(c)) break;
    v = v * 10 + (c - '0');
  }
  return v;
}

// days since 1970-01-01 from a proleptic Gregorian date (era-based day count,
// as engine/src/utilities/scalar_timestamp_parser.cpp timestamp_from_parts)
int64_t civil_days(int32_t y, int32_t m, int32_t d) {
  y -= m <= 2 ? 1 : 0;
  const int32_t era = (y >= 0 ? y : y - 399) / 400;
  const int32_t yoe = y - era * 400;
  const int32_t doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
  const int32_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return (int32_t)(era * 146097 + doe - 719468);
}

int64_t timestamp_value(const std::string& s, int type, bool with_time, bool with_frac) {
  const int fl = type == TIMESTAMP_MILLISECONDS ? 3 : type == TIMESTAMP_NANOSECONDS ? 9 : 6;
  const size_t need = with_time ? (with_frac ? 20 + fl : 19) : 10;
  if (s.size() < need) fail(GX_ERR_PARSE, "format string cannot be parsed from datetime string: " + s);
  int64_t days = civil_days(fixed_int(s, 0, 4), fixed_int(s, 5, 2), fixed_int(s, 8, 2));
  if (type == TIMESTAMP_DAYS) return days;
  int64_t t = days * 86400LL;
  int32_t sub = 0;
  if (with_time) {
    t += fixed_int(s, 11, 2) * 3600LL + fixed_int(s, 14, 2) * 60LL + fixed_int(s, 17, 2);
    if (with_frac) sub = fixed_int(s, 20, fl);
  }
  if (type == TIMESTAMP_SECONDS) return t;
  if (type == TIMESTAMP_MILLISECONDS) t *= 1000LL;
  else if (type == TIMESTAMP_MICROSECONDS) t *= 1000000LL;
  else t *= 1000000000LL;
  return t + sub;
}

// get_scalar_from_string (CalciteExpressionParsing.cpp:138-262): the value as the
// kernel reads it -- int64 bits for integral/timestamp scalars, double bits for floats.
void literal_value(Expr& e) {
  const std::string& s = e.token;
  const int t = e.lit_type;
  if (s == "null") {
    e.lit_valid = false;
    e.lit_bits = 0;
    return;
  }
  e.lit_valid = true;
  switch (t) {
    case BOOL8: e.lit_bits = s == "true"; return;
    case INT8: e.lit_bits = (uint64_t)(int64_t)(int8_t)parse_ll(s, INT32_MIN, INT32_MAX); return;
    case INT16: e.lit_bits = (uint64_t)(int64_t)(int16_t)parse_ll(s, INT32_MIN, INT32_MAX); return;
    case INT32: e.lit_bits = (uint64_t)(int64_t)(int32_t)parse_ll(s, INT32_MIN, INT32_MAX); return;
    case INT64: e.lit_bits = (uint64_t)parse_ll(s, INT64_MIN, INT64_MAX); return;
    case UINT8: e.lit_bits = (uint8_t)parse_ull(s); return;
    case UINT16: e.lit_bits = (uint16_t)parse_ull(s); return;
    case UINT32: e.lit_bits = (uint32_t)parse_ull(s); return;
    case UINT64: e.lit_bits = parse_ull(s); return;
    case FLOAT32: {
      errno = 0;
      char* end = nullptr;
      float f = std::strtof(s.c_str(), &end);
      if (end == s.c_str() || errno == ERANGE) fail(GX_ERR_PARSE, "cannot convert literal '" + s + "'");
      e.lit_bits = dbits((double)f);
      return;
    }
    case FLOAT64: {
      errno = 0;
      char* end = nullptr;
      double d = std::strtod(s.c_str(), &end);
      if (end == s.c_str() || errno == ERANGE) fail(GX_ERR_PARSE, "cannot convert literal '" + s + "'");
      e.lit_bits = dbits(d);
      return;
    }
    case DURATION_SECONDS: case DURATION_MILLISECONDS: case DURATION_MICROSECONDS: case DURATION_NANOSECONDS:
      e.lit_bits = (uint64_t)parse_ll(s, INT64_MIN, INT64_MAX);
      return;
    case STRING: fail(GX_ERR_UNSUPPORTED, "string literal out of scope: " + s);
    default: break;
  }
  std::string c = s;
  if (!c.empty() && (c[0] == '\'' || c.back() == '\'')) c = c.substr(1, c.size() - 2);
  if (t == TIMESTAMP_DAYS) {
    if (!is_date_text(c)) fail(GX_ERR_PARSE, "not recognized format TIMESTAMP_DAYS for: " + s);
    e.lit_bits = (uint64_t)(int64_t)(int32_t)timestamp_value(c, t, false, false);
    return;
  }
  if (t == TIMESTAMP_SECONDS) {
    if (!is_timestamp_any(c)) fail(GX_ERR_PARSE, "not recognized format TIMESTAMP_SECONDS for: " + c);
    e.lit_bits = (uint64_t)timestamp_value(c, t, true, false);
    return;
  }
  if (t == TIMESTAMP_MILLISECONDS || t == TIMESTAMP_MICROSECONDS || t == TIMESTAMP_NANOSECONDS) {
    if (is_timestamp_decimals(c)) e.lit_bits = (uint64_t)timestamp_value(c, t, true, true);
    else if (is_timestamp_any(c)) e.lit_bits = (uint64_t)timestamp_value(c, t, true, false);
    else fail(GX_ERR_PARSE, "not recognized format TIMESTAMP for: " + c);
    return;
  }
  fail(GX_ERR_UNSUPPORTED, "unsupported literal type for '" + s + "'");
}

// ---------------------------------------------------------------- parser
class Parser {
 public:
  explicit Parser(const std::string& s) : lx_(s) { tok_ = lx_.next(); }

  ExprPtr expr() {
    ExprPtr r = term();
    if (!r) r = func();
    if (!r) fail(GX_ERR_PARSE, "Couldn't parse calcite expression");
    return r;
  }

 private:
  bool accept(Tok t) {
    if (tok_.t != t) return false;
    tok_ = lx_.next();
    return true;
  }
  ExprPtr term() {
    Token t = tok_;
    if (accept(T_VAR)) {
      auto e = std::make_shared<Expr>();
      e->kind = Expr::COL;
      e->token = t.v;
      e->col = (int)parse_ll(t.v.substr(1), 0, INT32_MAX);
      return e;
    }
    return literal();
  }
  ExprPtr func() {
    Token name = tok_;
    if (!accept(T_IDENT)) return nullptr;
    accept(T_LP);
    auto e = std::make_shared<Expr>();
    e->kind = Expr::OP;
    if (!accept(T_RP)) {
      e->ch.push_back(expr());
      while (accept(T_COMMA)) e->ch.push_back(expr());
      accept(T_RP);
    }
    e->token = name.v;
    if (accept(T_COLON)) {
      Token rt = tok_;
      accept(T_IDENT);
      e->token += "_" + rt.v;
    }
    return e;
  }
  ExprPtr literal() {
    Token t = tok_;
    switch (t.t) {
      case T_NULL: case T_BOOL: case T_NUM: case T_DUR_S: case T_TS_D: case T_TS_S: case T_TS_MS: case T_TS_NS:
      case T_STR: break;
      default: return nullptr;
    }
    tok_ = lx_.next();
    auto e = std::make_shared<Expr>();
    e->kind = Expr::LIT;
    e->token = t.v;
    if (accept(T_COLON)) {
      Token tt = tok_;
      accept(T_IDENT);
      e->lit_type = type_from_token(tt.v);
      e->lit_type_token = tt.v;
    } else {
      e->lit_type = infer_literal_type(t);
    }
    return e;
  }

  Lexer lx_;
  Token tok_;
};

// ---------------------------------------------------------------- operators
const std::unordered_map<std::string, Op>& op_table() {
  static const std::unordered_map<std::string, Op> M = {
      {"BLZ_RND", OP_RAND}, {"GX_ROW_INDEX", OP_ROW_INDEX}, {"NOT", OP_NOT}, {"IS NOT TRUE", OP_IS_NOT_TRUE}, {"IS NOT FALSE", OP_IS_NOT_FALSE},
      {"IS TRUE", OP_IS_TRUE}, {"SIN", OP_SIN}, {"ASIN", OP_ASIN}, {"COS", OP_COS}, {"ACOS", OP_ACOS},
      {"TAN", OP_TAN}, {"ATAN", OP_ATAN}, {"COT", OP_COTAN}, {"FLOOR", OP_FLOOR}, {"CEIL", OP_CEIL},
      {"ABS", OP_ABS}, {"LOG10", OP_LOG10}, {"LN", OP_LN}, {"EXP", OP_EXP}, {"BL_YEAR", OP_YEAR},
      {"BL_MONTH", OP_MONTH}, {"BL_DAY", OP_DAY}, {"BL_DOW", OP_DAYOFWEEK}, {"BL_HOUR", OP_HOUR},
      {"BL_MINUTE", OP_MINUTE}, {"BL_SECOND", OP_SECOND}, {"IS_NULL", OP_IS_NULL}, {"IS_NOT_NULL", OP_IS_NOT_NULL},
      {"CAST_TINYINT", OP_CAST_TINYINT}, {"CAST_SMALLINT", OP_CAST_SMALLINT}, {"CAST_INTEGER", OP_CAST_INTEGER},
      {"CAST_BIGINT", OP_CAST_BIGINT}, {"CAST_FLOAT", OP_CAST_FLOAT}, {"CAST_DOUBLE", OP_CAST_DOUBLE},
      {"CAST_DATE", OP_CAST_DATE}, {"CAST_TIMESTAMP_SECONDS", OP_CAST_TIMESTAMP_SECONDS},
      {"CAST_TIMESTAMP_MILLISECONDS", OP_CAST_TIMESTAMP_MILLISECONDS},
      {"CAST_TIMESTAMP_MICROSECONDS", OP_CAST_TIMESTAMP_MICROSECONDS}, {"CAST_TIMESTAMP", OP_CAST_TIMESTAMP},
      {"=", OP_EQ}, {"<>", OP_NE}, {">", OP_GT}, {">=", OP_GE}, {"<", OP_LT}, {"<=", OP_LE}, {"+", OP_ADD},
      {"-", OP_SUB}, {"*", OP_MUL}, {"/", OP_DIV}, {"POWER", OP_POW}, {"ROUND", OP_ROUND}, {"MOD", OP_MOD},
      {"AND", OP_AND}, {"OR", OP_OR}, {"FIRST_NON_MAGIC", OP_FIRST_NON_MAGIC}, {"MAGIC_IF_NOT", OP_MAGIC_IF_NOT},
      {"IS_NOT_DISTINCT_FROM", OP_IS_NOT_DISTINCT_FROM}};
  return M;
}

bool is_string_op(const std::string& t) {
  static const char* S[] = {"CAST_VARCHAR", "CAST_CHAR", "CHAR_LENGTH", "LOWER", "UPPER", "INITCAP", "REVERSE",
                            "LIKE", "SUBSTRING", "REGEXP_REPLACE", "REPLACE", "TO_DATE", "TO_TIMESTAMP", "||",
                            "CONCAT", "TRIM", "LEFT", "RIGHT"};
  for (const char* x : S)
    if (t == x) return true;
  return false;
}

Op op_of(const std::string& token) {
  auto it = op_table().find(token);
  if (it != op_table().end()) return it->second;
  if (is_string_op(token)) fail(GX_ERR_UNSUPPORTED, "string operator out of scope: " + token);
  fail(GX_ERR_UNSUPPORTED, "Unsupported operator: " + token);
}

// get_output_type, unary (expression_utils.cpp:127-200)
int unary_type(Op op, int l) {
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
    case OP_SIN: case OP_COS: case OP_ASIN: case OP_ACOS: case OP_TAN: case OP_COTAN: case OP_ATAN: case OP_LN:
    case OP_LOG10: case OP_EXP: case OP_FLOOR: case OP_CEIL:
      return is_float(l) ? l : FLOAT64;
    case OP_ABS: return l;
    case OP_NOT: case OP_IS_TRUE: case OP_IS_NULL: case OP_IS_NOT_NULL: case OP_IS_NOT_TRUE: case OP_IS_NOT_FALSE:
      return BOOL8;
    default: return EMPTY;
  }
}

// get_output_type, binary (expression_utils.cpp:202-262)
int binary_type(Op op, int l, int r) {
  if (l == EMPTY && r == EMPTY) fail(GX_ERR_TYPE, "In get_output_type function: both operands types are empty");
  if (l == EMPTY) l = r;
  else if (r == EMPTY) r = l;
  switch (op) {
    case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_MOD:
      if (is_float(l) && is_float(r)) return type_size(l) >= type_size(r) ? l : r;
      if (is_float(l)) return l;
      if (is_float(r)) return r;
      return type_size(l) >= type_size(r) ? l : r;
    case OP_EQ: case OP_NE: case OP_LT: case OP_GT: case OP_LE: case OP_GE: case OP_AND: case OP_OR:
      return BOOL8;
    case OP_POW: case OP_ROUND: return type_size(l) <= 4 ? FLOAT32 : FLOAT64;
    case OP_MAGIC_IF_NOT: return r;
    case OP_FIRST_NON_MAGIC: return type_size(l) >= type_size(r) ? l : r;
    case OP_IS_NOT_DISTINCT_FROM: return BOOL8;  // reference's binary rule has no entry (EMPTY)
    default: return EMPTY;
  }
}

// get_common_type(..., strict=true) (utilities/CommonOperations.cpp:185-230)
void check_common_type(int a, int b) {
  if (a == b) return;
  if ((is_float(a) && is_float(b)) || (is_integer(a) && is_integer(b))) return;
  if ((is_timestamp(a) && is_timestamp(b)) || (is_duration(a) && is_duration(b))) return;
  if (a == STRING && is_timestamp(b)) return;
  fail(GX_ERR_TYPE, "No common type between " + std::to_string(a) + " and " + std::to_string(b));
}

ExprPtr make_op(const char* token, ExprPtr a, ExprPtr b) {
  auto e = std::make_shared<Expr>();
  e->kind = Expr::OP;
  e->token = token;
  e->ch = {std::move(a), std::move(b)};
  return e;
}

// n-ary AND(/OR( -> left-deep binary nesting (CalciteExpressionParsing.cpp:330-398).
// OR is left n-ary when the text contains FLOOR (the reference skips it then);
// the interpreter then reads only its first two operands.
void nest_logical(ExprPtr& e, bool expand_or) {
  if (e->kind != Expr::OP) return;
  for (auto& c : e->ch) nest_logical(c, expand_or);
  const bool is_and = e->token == "AND", is_or = e->token == "OR";
  if ((is_and || (is_or && expand_or)) && e->ch.size() > 2) {
    ExprPtr acc = make_op(e->token.c_str(), e->ch[0], e->ch[1]);
    for (size_t i = 2; i < e->ch.size(); i++) acc = make_op(e->token.c_str(), acc, e->ch[i]);
    e = acc;
  }
  if ((is_and || is_or) && e->ch.size() < 2) fail(GX_ERR_PARSE, "logical operator with fewer than two operands");
}

ExprPtr lower_case(std::vector<ExprPtr>& c, size_t i) {
  if (i == c.size() - 1) return c[i];
  ExprPtr mif = make_op("MAGIC_IF_NOT", c[i], c[i + 1]);
  return make_op("FIRST_NON_MAGIC", mif, lower_case(c, i + 2));
}

// custom_op_transformer (expression_tree.hpp:181-258), bottom-up.
ExprPtr lower(ExprPtr e) {
  if (e->kind != Expr::OP) return e;
  for (auto& c : e->ch) c = lower(c);
  if (e->token == "CASE") {
    if (e->ch.size() < 3 || e->ch.size() % 2 == 0) fail(GX_ERR_PARSE, "CASE needs an odd number (>= 3) of operands");
    return lower_case(e->ch, 0);
  }
  if (e->token == "Reinterpret") {
    if (e->ch.size() != 1) fail(GX_ERR_PARSE, "Reinterpret takes one operand");
    return e->ch[0];
  }
  if (e->token == "ROUND") {
    if (e->ch.size() == 1) {
      auto z = std::make_shared<Expr>();
      z->kind = Expr::LIT;
      z->token = "0";
      z->lit_type = INT8;
      e->ch.push_back(z);
    }
    return e;
  }
  if (e->token.rfind("CAST", 0) == 0 && e->ch.size() == 1 && e->ch[0]->kind == Expr::LIT) {
    if (is_string_op(e->token)) fail(GX_ERR_UNSUPPORTED, "string operator out of scope: " + e->token);
    Op cop = op_of(e->token);
    int nt = unary_type(cop, e->ch[0]->lit_type);
    check_common_type(e->ch[0]->lit_type, nt);
    auto l = std::make_shared<Expr>(*e->ch[0]);
    l->lit_type = nt;
    return l;
  }
  return e;
}

void annotate(Expr& e, const std::vector<int>& schema) {
  if (e.kind == Expr::COL) {
    if (e.col < 0 || (size_t)e.col >= schema.size()) fail(GX_ERR_PARSE, "column index out of range: " + e.token);
    const int t = schema[e.col];
    if (t == STRING) fail(GX_ERR_UNSUPPORTED, "string column out of scope: " + e.token);
    if (type_size(t) == 0) fail(GX_ERR_UNSUPPORTED, "unsupported column type " + std::to_string(t));
    e.vtype = e.ktype = t;
    return;
  }
  if (e.kind == Expr::LIT) {
    literal_value(e);
    e.vtype = e.lit_type;
    e.ktype = e.lit_valid ? e.lit_type : EMPTY;
    return;
  }
  for (auto& c : e.ch) annotate(*c, schema);
  e.op = op_of(e.token);
  if (e.op == OP_RAND) {
    e.vtype = e.ktype = FLOAT64;
    return;
  }
  if (e.op == OP_ROW_INDEX) {
    e.vtype = e.ktype = INT32;
    return;
  }
  if (op_is_unary(e.op)) {
    if (e.ch.empty()) fail(GX_ERR_PARSE, "unary operator without operand: " + e.token);
    if (e.ch[0]->kind == Expr::LIT) fail(GX_ERR_UNSUPPORTED, "Unary operations on literals is not supported");
    e.vtype = unary_type(e.op, e.ch[0]->vtype);
    e.ktype = unary_type(e.op, e.ch[0]->ktype);
    return;
  }
  if (op_is_binary(e.op)) {
    if (e.ch.size() < 2) fail(GX_ERR_PARSE, "binary operator needs two operands: " + e.token);
    if (e.ch[0]->kind == Expr::LIT && e.ch[1]->kind == Expr::LIT)
      fail(GX_ERR_UNSUPPORTED, "Operations between literals is not supported");
    e.vtype = binary_type(e.op, e.ch[0]->vtype, e.ch[1]->vtype);
    e.ktype = binary_type(e.op, e.ch[0]->ktype, e.ch[1]->ktype);
    return;
  }
  fail(GX_ERR_UNSUPPORTED, "unsupported operator " + e.token);
}

}  // namespace

// ---------------------------------------------------------------- public API
ExprPtr parse_and_lower(const std::string& text) {
  const std::string norm = normalize_calcite(text);
  Parser p(norm);
  ExprPtr root = p.expr();
  nest_logical(root, norm.find("FLOOR") == std::string::npos);
  return lower(root);
}

ExprPtr compile_expression(const std::string& text, const std::vector<int>& schema) {
  ExprPtr root = parse_and_lower(text);
  annotate(*root, schema);
  return root;
}

std::vector<std::string> split_expression_list(std::string text, bool trim_items) {
  text = normalize_calcite(text);
  std::vector<std::string> out;
  size_t start = 0;
  bool in_quotes = false;
  int paren = 0, sq = 0;
  for (size_t i = 0; i < text.size(); i++) {
    const char c = text[i];
    if (in_quotes) {
      if (c == '\'' && !(i + 1 < text.size() && text[i + 1] == '\'')) in_quotes = false;
      continue;
    }
    if (c == '\'') in_quotes = true;
    else if (c == '(') paren++;
    else if (c == ')') paren--;
    else if (c == '[') sq++;
    else if (c == ']') sq--;
    else if (c == ',' && paren == 0 && sq == 0) {
      std::string item = text.substr(start, i - start);
      out.push_back(trim_items ? ltrim(item) : item);
      start = i + 1;
    }
  }
  if (start < text.size()) {
    std::string item = text.substr(start);
    out.push_back(trim_items ? trim(item) : item);
  }
  return out;
}

std::string named_expression(const std::string& qp, const std::string& name) {
  if (qp.find(name + "=[") == std::string::npos) return "";
  size_t start;
  size_t dbl = qp.find(name + "=[[");
  if (dbl != std::string::npos) start = dbl + 3 + name.size();
  else start = qp.find(name + "=[") + 2 + name.size();
  size_t end = qp.find(']', start);
  return qp.substr(start, end == std::string::npos ? std::string::npos : end - start);
}

std::string query_part_of(const std::string& plan) {
  size_t a = plan.find('('), b = plan.rfind(')');
  if (a == std::string::npos || b == std::string::npos || b < a) fail(GX_ERR_PARSE, "malformed relational node: " + plan);
  return plan.substr(a + 1, b - a - 1);
}

void split_projections(const std::string& plan, std::vector<std::string>& names, std::vector<std::string>& exprs) {
  std::vector<std::string> items = split_expression_list(query_part_of(plan), false);
  for (const auto& it : items) {
    size_t p = it.find("=[");
    if (p == std::string::npos || it.size() < p + 3) fail(GX_ERR_PARSE, "projection without name=[expr]: " + it);
    names.push_back(trim(it.substr(0, p)));
    exprs.push_back(it.substr(p + 2, it.size() - p - 3));
  }
}

namespace {
thread_local std::string t_current_timestamp;  // the calling thread's query timestamp ("" = none)

std::string replaced_all(std::string s, const std::string& from, const std::string& to) {
  size_t p = 0;
  while ((p = s.find(from, p)) != std::string::npos) {
    s.replace(p, from.size(), to);
    p += to.size();
  }
  return s;
}
}  // namespace

void set_current_timestamp(const std::string& ts) {
  if (!ts.empty()) {
    // "YYYY-MM-DD hh:mm:ss[.f...]": the form the engine Context keeps
    auto digits = [&](size_t a, size_t n) {
      for (size_t i = a; i < a + n; i++)
        if (i >= ts.size() || ts[i] < '0' || ts[i] > '9') return false;
      return true;
    };
    const bool ok = ts.size() >= 19 && digits(0, 4) && ts[4] == '-' && digits(5, 2) && ts[7] == '-' &&
                    digits(8, 2) && ts[10] == ' ' && digits(11, 2) && ts[13] == ':' && digits(14, 2) &&
                    ts[16] == ':' && digits(17, 2) && (ts.size() == 19 || (ts[19] == '.' && digits(20, ts.size() - 20)));
    if (!ok) fail(GX_ERR_INVALID, "current timestamp must look like YYYY-MM-DD hh:mm:ss[.fraction]: " + ts);
  }
  t_current_timestamp = ts;
}

std::string current_timestamp() { return t_current_timestamp; }

std::string preprocess_expression(const std::string& text, const std::vector<int>& schema) {
  return preprocess_stages(text, schema, kPreAll);
}

std::string preprocess_stages(const std::string& text, const std::vector<int>& schema, int stages) {
  std::string e = text;
  // fill_minus_op_with_zero (expression_utils.cpp:1155-1164)
  if (stages & kPreMinus) {
    size_t dollars = 0;
    for (char c : e) dollars += c == '$';
    if (!e.empty() && e[0] == '-' && dollars == 1 && e.find(',') == std::string::npos && e.size() >= 2)
      e = e.substr(0, 2) + "0, " + e.substr(2);
  }
  // convert_nary_to_binary_concat (:1620) happens in the string pre-pass
  // (rewrite_string_ops nests an n-ary CONCAT before evaluating it)
  // get_current_date_or_timestamp (expression_utils.cpp:1494-1518): the
  // query's timestamp replaces CURRENT_TIMESTAMP (to milliseconds) or
  // CURRENT_DATE (the date); CURRENT_TIME means CURRENT_TIMESTAMP; when both
  // appear only CURRENT_DATE is replaced, as there
  if ((stages & kPreCurrent) &&
      (e.find("CURRENT_DATE") != std::string::npos || e.find("CURRENT_TIME") != std::string::npos)) {
    if (t_current_timestamp.empty())
      fail(GX_ERR_UNSUPPORTED,
           "CURRENT_DATE/CURRENT_TIMESTAMP need the query's timestamp: set it with gx_set_current_timestamp");
    if (e.find("CURRENT_TIMESTAMP") == std::string::npos) e = replaced_all(e, "CURRENT_TIME", "CURRENT_TIMESTAMP");
    std::string ts = t_current_timestamp.substr(0, 23), what = "CURRENT_TIMESTAMP";
    if (e.find("CURRENT_DATE") != std::string::npos) {
      what = "CURRENT_DATE";
      ts = ts.substr(0, 10);
    }
    e = replaced_all(e, what, ts);
  }
  // convert_ms_to_ns_units (expression_utils.cpp:1316-1350)
  const bool ms_ns = (stages & kPreMsToNs) != 0;
  const bool cast_ts = ms_ns && e.find("CAST(") != std::string::npos && e.find(":TIMESTAMP") != std::string::npos;
  const bool cast_dt = ms_ns && e.find("CAST(") != std::string::npos && e.find(":DATE") != std::string::npos;
  if (cast_ts || cast_dt) {
    bool done = false;
    if (e.find("Reinterpret(") != std::string::npos) {
      for (const char* u : {"86400000", "3600000", "60000", "1000"}) {
        if (e.find(u) != std::string::npos) {
          e = replaced_all(e, u, std::string(u) + "000000");
          done = true;
          break;
        }
      }
    }
    size_t ip = e.find(":INTERVAL");
    if (!done && ip != std::string::npos) {
      size_t sp = e.find(", ") + 2;
      std::string tv = e.substr(sp, ip - sp);
      e = replaced_all(e, tv, tv + "000000");
    }
  }
  if (schema.empty()) return e;
  // reinterpret_timestamp (expression_utils.cpp:1371-1420)
  const std::string key = "Reinterpret(-(";
  size_t rp = (stages & kPreReinterpret) ? e.find(key) : std::string::npos;
  if (rp != std::string::npos) {
    std::string red = e.substr(rp + key.size());
    red = red.substr(0, red.find("))"));
    std::vector<std::string> parts = split_expression_list(red, false);
    if (parts.size() == 2) {
      auto idx_of = [](const std::string& x) -> size_t {
        if (!x.empty() && x[0] == '$') return (size_t)parse_ll(x.substr(1), 0, INT32_MAX);
        size_t a = x.find('$') + 1, b = x.find(')');
        return (size_t)parse_ll(x.substr(a, b - a), 0, INT32_MAX);
      };
      std::string ts;
      size_t col = 0;
      bool hit = true;
      if (is_timestamp_any(parts[0])) { ts = parts[0]; col = idx_of(parts[1]); }
      else if (is_timestamp_any(parts[1])) { ts = parts[1]; col = idx_of(parts[0]); }
      else hit = false;
      if (hit) {
        if (col >= schema.size()) fail(GX_ERR_PARSE, "column index out of range in Reinterpret");
        const char* unit = schema[col] == TIMESTAMP_SECONDS ? "TIMESTAMP_SECONDS"
                         : schema[col] == TIMESTAMP_MILLISECONDS ? "TIMESTAMP_MILLISECONDS"
                         : schema[col] == TIMESTAMP_MICROSECONDS ? "TIMESTAMP_MICROSECONDS" : "TIMESTAMP";
        e = replaced_all(e, ts, "CAST(" + ts + "):" + unit);
      }
    }
  }
  // apply_interval_conversion (expression_utils.cpp:1425-1460)
  const std::string iv = ":INTERVAL";
  if ((stages & kPreInterval) && e.find(iv) != std::string::npos) {
    if (e.find('+') != std::string::npos || e.find('-') != std::string::npos) {
      size_t sp = 0;
      if (e.find("+($") != std::string::npos) sp = e.find("+($") + 3;
      else if (e.find("-($") != std::string::npos) sp = e.find("-($") + 3;
      std::string ne = e.substr(sp);
      ne = ne.substr(0, ne.find(", "));
      long long col = parse_ll(ne, 0, INT32_MAX);
      if ((size_t)col >= schema.size()) fail(GX_ERR_PARSE, "column index out of range in interval");
      if (schema[col] == DURATION_SECONDS) e = replaced_all(e, "000" + iv, iv);
      else if (schema[col] == DURATION_MICROSECONDS) e = replaced_all(e, "000" + iv, "000000" + iv);
      else if (schema[col] == DURATION_NANOSECONDS) e = replaced_all(e, "000" + iv, "000000000" + iv);
    } else if (e.find('$') == std::string::npos && e.find("000:INTERVAL") != std::string::npos) {
      e = replaced_all(e, "000" + iv, iv);
    }
  }
  return e;
}

std::string rebuild(const ExprPtr& e) {
  if (e->kind != Expr::OP) return e->token;
  std::string s;
  for (const auto& c : e->ch) s += (s.empty() ? "" : ", ") + rebuild(c);
  return e->token + "(" + s + ")";
}


// ---------------------------------------------------------------- skip data
// Row-group pruning predicate (ral::skip_data, engine/src/skip_data/
// SkipDataProcessor.cpp): a TableScan condition over column $i becomes a
// condition over its row-group statistics, $2i = min and $2i+1 = max.
namespace {

ExprPtr sd_none() {
  auto e = std::make_shared<Expr>();
  e->kind = Expr::OP;
  e->token = "NONE";
  return e;
}

bool sd_unary(const std::string& token) {
  if (token == "NONE") return true;
  auto it = op_table().find(token);
  return it != op_table().end() && op_is_unary(it->second);
}

// skip_data_drop_transformer (:23-45): every node named v becomes NONE
ExprPtr sd_drop(ExprPtr e, const std::string& v) {
  if (e->kind == Expr::OP)
    for (auto& c : e->ch) c = sd_drop(c, v);
  if (e->token == v) return sd_none();
  return e;
}

// skip_data_reducer (:167-212) with is_unsupported_binary_op / is_exclusion_unary_op
// (skip_data/utils.cpp:12-37), children first
ExprPtr sd_reduce(ExprPtr e) {
  if (e->kind != Expr::OP) return e;
  for (auto& c : e->ch) c = sd_reduce(c);
  static const char* kSupported[] = {"=", ">", ">=", "<", "<=", "+", "-", "AND", "OR"};
  bool supported = false;
  for (const char* t : kSupported) supported |= e->token == t;
  if (!supported || e->ch.size() != 2) return sd_none();
  const bool l = e->ch[0]->kind == Expr::OP && sd_unary(e->ch[0]->token);
  const bool r = e->ch[1]->kind == Expr::OP && sd_unary(e->ch[1]->token);
  if (l && !r) return e->token == "AND" ? e->ch[1] : sd_none();
  if (r && !l) return e->token == "AND" ? e->ch[0] : sd_none();
  if (l && r) return sd_none();
  return e;
}

ExprPtr sd_op(const std::string& token, ExprPtr a, ExprPtr b) {
  auto e = std::make_shared<Expr>();
  e->kind = Expr::OP;
  e->token = token;
  e->ch = {std::move(a), std::move(b)};
  return e;
}

// transform_inc (:69-101): a column to its min (k 0) or max (k 1) statistic,
// the "&&&" pair of a transformed sum / difference to its min or max form
ExprPtr sd_inc(const ExprPtr& n, int k) {
  if (n->kind == Expr::COL) {
    auto e = std::make_shared<Expr>(*n);
    e->col = 2 * n->col + k;
    e->token = "$" + std::to_string(e->col);
    return e;
  }
  if (n->kind == Expr::OP && n->token == "&&&") return n->ch[k];
  return n;
}

// skip_data_transformer (:48-165), children first
ExprPtr sd_transform(ExprPtr e) {
  if (e->kind != Expr::OP) return e;
  for (auto& c : e->ch) c = sd_transform(c);
  const std::string& op = e->token;
  if (e->ch.size() != 2) return e;
  const ExprPtr& n = e->ch[0];
  const ExprPtr& m = e->ch[1];
  if (op == "=")
    return sd_op("AND", sd_op("<=", sd_inc(n, 0), sd_inc(m, 1)), sd_op(">=", sd_inc(n, 1), sd_inc(m, 0)));
  if (op == "<" || op == "<=") return sd_op(op, sd_inc(n, 0), sd_inc(m, 1));
  if (op == ">" || op == ">=") return sd_op(op, sd_inc(n, 1), sd_inc(m, 0));
  if (op == "+" || op == "-")
    return sd_op("&&&", sd_op(op, sd_inc(n, 0), sd_inc(m, 0)), sd_op(op, sd_inc(n, 1), sd_inc(m, 1)));
  return e;
}

// tokenizer_helper (parser/expression_tree.hpp:164-179): prefix form
std::string sd_prefix(const ExprPtr& e) {
  if (e->kind != Expr::OP || e->token.empty()) return e->token;
  std::string s;
  for (const auto& c : e->ch) s += (s.empty() ? "" : " ") + sd_prefix(c);
  return e->token + (s.empty() ? "" : " " + s);
}

}  // namespace

std::string skip_data_rewrite(const std::string& condition, const std::vector<int>& dropped,
                              std::string* prefix_form) {
  // replace_calcite_regex + expand_if_logical_op, then the parse tree
  // (process_skipdata_for_table, SkipDataProcessor.cpp:270-271, 310)
  const std::string norm = normalize_calcite(condition);
  Parser p(norm);
  ExprPtr root = p.expr();
  nest_logical(root, norm.find("FLOOR") == std::string::npos);
  for (int c : dropped) root = sd_drop(root, "$" + std::to_string(c));
  // apply_skip_data_rules (:220-232)
  root = sd_reduce(root);
  if (root->token == "NONE") {
    if (prefix_form) *prefix_form = "NONE";
    return "";
  }
  root = sd_transform(root);
  if (prefix_form) *prefix_form = sd_prefix(root);
  return rebuild(root);
}


// ---------------------------------------------------------------- string pre-pass
namespace {

std::string unquote(const std::string& t) {
  if (t.size() >= 2 && (t.front() == '\'' || t.front() == '"') && t.back() == t.front()) {
    std::string r;
    const std::string in = t.substr(1, t.size() - 2);
    for (size_t i = 0; i < in.size(); i++) {
      r += in[i];
      if (in[i] == '\'' && i + 1 < in.size() && in[i + 1] == '\'') i++;  // '' -> '
    }
    return r;
  }
  return t;
}

bool is_string_literal(const ExprPtr& e) {
  return e->kind == Expr::LIT && !e->token.empty() && (e->token.front() == '\'' || e->token.front() == '"');
}

// rebuild() keeping literals' explicit types, so a rewritten text types its
// literals as the original did
std::string rebuild_typed(const ExprPtr& e) {
  if (e->kind == Expr::LIT) return e->lit_type_token.empty() ? e->token : e->token + ":" + e->lit_type_token;
  if (e->kind != Expr::OP) return e->token;
  std::string s;
  for (const auto& c : e->ch) s += (s.empty() ? "" : ", ") + rebuild_typed(c);
  return e->token + "(" + s + ")";
}

bool is_null_literal(const ExprPtr& e) { return e->kind == Expr::LIT && e->token == "null"; }

}  // namespace

int passthrough_column(const std::string& text) {
  size_t b = 0, e = text.size();
  while (b < e && std::isspace((unsigned char)text[b])) b++;
  while (e > b && std::isspace((unsigned char)text[e - 1])) e--;
  if (e - b < 2 || text[b] != '$') return -1;
  for (size_t i = b + 1; i < e; i++)
    if (!std::isdigit((unsigned char)text[i])) return -1;
  return e - b > 10 ? -1 : std::atoi(text.c_str() + b + 1);
}

bool string_literal_value(const std::string& text, std::string* value) {
  if (text.find('\'') == std::string::npos) return false;
  const std::string norm = normalize_calcite(text);
  Parser p(norm);
  ExprPtr root = p.expr();
  if (!is_string_literal(root)) return false;
  if (value) *value = unquote(root->token);
  return true;
}

void rewrite_string_ops(std::vector<std::string>& texts, const std::vector<int>& schema,
                        std::vector<StringOp>& ops) {
  bool any = false;
  for (int t : schema) any |= t == STRING;
  // a CAST to VARCHAR / CHAR makes a string column from typed ones
  for (const auto& t : texts) any |= t.find('\'') != std::string::npos || t.find("CHAR") != std::string::npos;
  if (!any) return;
  // the schema grows by one column per operator
  std::vector<int> types = schema;
  auto strcol = [&](const ExprPtr& c) {
    return c->kind == Expr::COL && c->col >= 0 && c->col < (int)types.size() && types[c->col] == STRING;
  };
  auto column_of = [&](const StringOp& op) {
    size_t k = 0;
    while (k < ops.size() && !(ops[k] == op)) k++;
    if (k == ops.size()) {
      ops.push_back(op);
      types.push_back(op.result_type());
    }
    auto c = std::make_shared<Expr>();
    c->kind = Expr::COL;
    c->col = (int)(schema.size() + k);
    c->token = "$" + std::to_string(c->col);
    return c;
  };
  // a CASE operand evaluate_string_case_when_else takes: a string column, a
  // string literal or a null literal (LogicalProject.cpp:616-623)
  auto string_operand = [&](const ExprPtr& e) { return strcol(e) || is_string_literal(e) || is_null_literal(e); };
  auto int_literal = [&](const ExprPtr& e, int* v) {
    if (e->kind != Expr::LIT || e->token.empty() || is_string_literal(e) || is_null_literal(e)) return false;
    char* end = nullptr;
    const long long x = std::strtoll(e->token.c_str(), &end, 10);
    if (!end || *end != '\0' || x < INT32_MIN || x > INT32_MAX) return false;
    *v = (int)x;
    return true;
  };
  auto need_strcol = [&](const ExprPtr& e, const char* fn) {
    if (!strcol(e))
      fail(GX_ERR_UNSUPPORTED, std::string(fn) + " argument must be a column of type string");
  };
  // the functions of evaluate_string_functions (LogicalProject.cpp:103-603)
  // other than LIKE; false when `e` is none of them
  std::function<bool(const ExprPtr&, StringOp&)> string_function = [&](const ExprPtr& e, StringOp& op) {
    const std::string& t = e->token;
    const auto& a = e->ch;
    if (t == "SUBSTRING" && (a.size() == 2 || a.size() == 3)) {
      // :212-220: start = max(start, 1) - 1; stop = start + length when a length >= 0 is given
      int st = 0, len = -1;
      need_strcol(a[0], "SUBSTRING");
      op.kind = StringOp::SLICE;
      op.col = a[0]->col;
      const bool lit_start = int_literal(a[1], &st);
      if (!lit_start || (a.size() == 3 && !int_literal(a[2], &len))) {
        // :221-300, positions from columns or expressions: a literal start is
        // max(start, 1), any start then one less (transform_start_to_zero_based_indexing,
        // utilities/transform.cu:44-68); the stop is start + length
        // (transform_length_to_end, transform.cu:15-42); no length: to the end
        op.pos0 = lit_start ? std::to_string(std::max(st, 1) - 1) : "-(" + rebuild_typed(a[1]) + ", 1)";
        if (a.size() == 3) op.pos1 = "+(" + op.pos0 + ", " + rebuild_typed(a[2]) + ")";
        return true;
      }
      op.i0 = std::max(st, 1) - 1;
      op.i0_valid = true;
      op.i1 = len >= 0 ? op.i0 + len : 0;
      op.i1_valid = a.size() == 3 && len >= 0;
      return true;
    }
    if ((t == "LEFT" || t == "RIGHT") && a.size() == 2) {
      int n = 0;
      need_strcol(a[0], t.c_str());
      if (!int_literal(a[1], &n)) fail(GX_ERR_UNSUPPORTED, t + " with a non-literal length");
      n = std::max(n, 0);
      op.kind = StringOp::SLICE;
      op.col = a[0]->col;
      if (t == "LEFT") {  // :186-191: [0, n)
        op.i0 = 0;
        op.i1 = n;
        op.i0_valid = op.i1_valid = true;
      } else {  // :200-201: [-n, end), or [0, 0) when n < 1
        op.i0 = -n;
        op.i0_valid = true;
        op.i1 = 0;
        op.i1_valid = n < 1;
      }
      return true;
    }
    if (t == "REVERSE" && a.size() == 1) {  // :573-585: step -1
      need_strcol(a[0], "REVERSE");
      op.kind = StringOp::SLICE;
      op.col = a[0]->col;
      op.step = -1;
      return true;
    }
    if ((t == "UPPER" || t == "LOWER" || t == "INITCAP") && a.size() == 1) {
      need_strcol(a[0], t.c_str());
      op.kind = t == "UPPER" ? StringOp::UPPER : t == "LOWER" ? StringOp::LOWER : StringOp::INITCAP;
      op.col = a[0]->col;
      return true;
    }
    if (t == "TRIM" && a.size() == 3 && is_string_literal(a[0]) && is_string_literal(a[1])) {
      need_strcol(a[2], "TRIM");
      const std::string side = unquote(a[0]->token);
      op.kind = StringOp::TRIM;
      op.col = a[2]->col;
      op.i0 = side == "LEADING" ? 1 : side == "TRAILING" ? 2 : 0;
      op.literal = unquote(a[1]->token);
      return true;
    }
    if (t == "REGEXP_REPLACE" && a.size() >= 3 && a.size() <= 6) {
      // :149-183: a string column, a pattern, a replacement and an optional position
      if (a.size() > 4) fail(GX_ERR_UNSUPPORTED, "Optional parameters occurrence and match_type are not yet supported.");
      if (a[0]->kind == Expr::LIT) fail(GX_ERR_UNSUPPORTED, "REGEXP_REPLACE function not supported for string literals");
      need_strcol(a[0], "REGEXP_REPLACE");
      if (!is_string_literal(a[1]) || !is_string_literal(a[2]))
        fail(GX_ERR_UNSUPPORTED, "REGEXP_REPLACE with a non-literal pattern or replacement");
      op.kind = StringOp::REGEXP_REPLACE;
      op.col = a[0]->col;
      op.literal = unquote(a[1]->token);
      op.literal2 = unquote(a[2]->token);
      if (a.size() == 4) {
        int st = 0;
        if (!int_literal(a[3], &st)) fail(GX_ERR_UNSUPPORTED, "REGEXP_REPLACE with a non-literal position");
        if (st - 1 < 0) fail(GX_ERR_INVALID, "Position must be greater than zero.");  // :164
        op.i0 = st - 1;
        op.i0_valid = true;
      }
      std::string program, tmpl;
      compile_regex_replace(op.literal, op.literal2, &program, &tmpl);  // rejects what is not supported now
      return true;
    }
    if (t == "REPLACE" && a.size() == 3) {
      need_strcol(a[0], "REPLACE");
      if (!is_string_literal(a[1]) || !is_string_literal(a[2]))
        fail(GX_ERR_UNSUPPORTED, "REPLACE with non-literal target or replacement");
      op.kind = StringOp::REPLACE;
      op.col = a[0]->col;
      op.literal = unquote(a[1]->token);
      op.literal2 = unquote(a[2]->token);
      if (op.literal.empty()) fail(GX_ERR_UNSUPPORTED, "REPLACE with an empty target");
      return true;
    }
    if ((t == "CAST_VARCHAR" || t == "CAST_CHAR") && a.size() == 1) {
      if (a[0]->kind == Expr::LIT) fail(GX_ERR_UNSUPPORTED, "CAST operator not supported for literals");
      op.kind = StringOp::TO_STRING;
      if (a[0]->kind == Expr::COL) op.col = a[0]->col;
      else op.cond = rebuild_typed(a[0]);
      return true;
    }
    static const std::map<std::string, int> parse_types = {
        {"CAST_TINYINT", INT8}, {"CAST_SMALLINT", INT16}, {"CAST_INTEGER", INT32}, {"CAST_BIGINT", INT64},
        {"CAST_DATE", TIMESTAMP_DAYS}, {"CAST_TIMESTAMP_SECONDS", TIMESTAMP_SECONDS},
        {"CAST_TIMESTAMP_MILLISECONDS", TIMESTAMP_MILLISECONDS},
        {"CAST_TIMESTAMP_MICROSECONDS", TIMESTAMP_MICROSECONDS}, {"CAST_TIMESTAMP", TIMESTAMP_NANOSECONDS},
        {"CAST_FLOAT", FLOAT32}, {"CAST_DOUBLE", FLOAT64}};
    auto pt = parse_types.find(t);
    if (pt != parse_types.end() && a.size() == 1 && strcol(a[0])) {
      op.kind = StringOp::PARSE;
      op.col = a[0]->col;
      op.type = pt->second;
      // to_timestamps' formats for the CASTs (LogicalProject.cpp:468-528)
      if (pt->second == TIMESTAMP_DAYS) op.literal = "%Y-%m-%d";
      else if (pt->second != INT8 && pt->second != INT16 && pt->second != INT32 && pt->second != INT64 &&
               pt->second != FLOAT32 && pt->second != FLOAT64)
        op.literal = "%Y-%m-%d %H:%M:%S";
      return true;
    }
    if ((t == "TO_DATE" || t == "TO_TIMESTAMP") && a.size() == 2) {
      // :530-552: a string column and a string format
      if (!strcol(a[0]) || !is_string_literal(a[1]))
        fail(GX_ERR_UNSUPPORTED, t + " operator arguments must be a column and a string format");
      op.kind = StringOp::PARSE;
      op.col = a[0]->col;
      op.type = t == "TO_DATE" ? TIMESTAMP_DAYS : TIMESTAMP_NANOSECONDS;
      op.literal = unquote(a[1]->token);
      const std::string& f = op.literal;
      if (f.find("%Y") == std::string::npos || f.find("%m") == std::string::npos ||
          f.find("%d") == std::string::npos)
        fail(GX_ERR_UNSUPPORTED, t + " format without %Y, %m and %d: " + f);
      return true;
    }
    return false;
  };
  for (auto& text : texts) {
    if (text.empty()) continue;
    const std::string norm = normalize_calcite(text);
    Parser p(norm);
    ExprPtr root = p.expr();
    nest_logical(root, norm.find("FLOOR") == std::string::npos);
    bool touched = false;
    std::function<ExprPtr(ExprPtr)> walk = [&](ExprPtr e) -> ExprPtr {
      if (e->kind != Expr::OP) return e;
      if ((e->token == "CONCAT" || e->token == "||") && e->ch.size() >= 2) {
        // The reference nests CONCAT(a, b, c) as CONCAT(CONCAT(a, b), c)
        // (convert_nary_to_binary_concat, expression_utils.cpp:1620) and
        // evaluates each pair, NULL if either side is.  That is one
        // concatenation of all parts, NULL if any is: nested CONCATs are
        // flattened into parts, up to kMaxConcatParts per operator.  Its
        // innermost pair of literals is still refused (:311).
        // a part CAST($k):VARCHAR of a typed column stays that column: the
        // CONCAT formats it in place (the pre-pass would format it into a
        // string column first)
        std::vector<ExprPtr> parts;
        std::vector<bool> formatted;
        std::function<void(const ExprPtr&)> flat = [&](const ExprPtr& x) {
          if (x->kind == Expr::OP && (x->token == "CONCAT" || x->token == "||") && x->ch.size() >= 2) {
            if (is_string_literal(x->ch[0]) && is_string_literal(x->ch[1]))
              fail(GX_ERR_UNSUPPORTED, "CONCAT operator between literals is not supported");
            for (const auto& c : x->ch) flat(c);
          } else if (x->kind == Expr::OP && (x->token == "CAST_VARCHAR" || x->token == "CAST_CHAR") &&
                     x->ch.size() == 1 && x->ch[0]->kind == Expr::COL && x->ch[0]->col >= 0 &&
                     x->ch[0]->col < (int)types.size() && types[x->ch[0]->col] != STRING) {
            parts.push_back(x->ch[0]);
            formatted.push_back(true);
          } else {
            parts.push_back(walk(x));
            formatted.push_back(false);
          }
        };
        flat(e);
        for (size_t k = 0; k < parts.size(); k++)
          if (!formatted[k] && !strcol(parts[k]) && !is_string_literal(parts[k]))
            fail(GX_ERR_UNSUPPORTED, "CONCAT of something other than strings");
        ExprPtr cur;
        for (size_t k = 0; k < parts.size();) {
          StringOp op;
          op.kind = StringOp::CONCAT;
          std::vector<ExprPtr> group;
          if (cur) group.push_back(cur);
          while (k < parts.size() && (int)group.size() < kMaxConcatParts) group.push_back(parts[k++]);
          for (size_t g = 0; g < group.size(); g++) {
            const int c = group[g]->kind == Expr::COL ? group[g]->col : -1;
            const std::string lit = c < 0 ? unquote(group[g]->token) : std::string();
            if (g == 0) { op.col = c; op.literal = lit; }
            else if (g == 1) { op.col2 = c; op.literal2 = lit; }
            else { op.more_cols.push_back(c); op.more_lits.push_back(lit); }
          }
          cur = column_of(op);
        }
        touched = true;
        return cur;
      }
      for (auto& c : e->ch) c = walk(c);
      const std::string& t = e->token;
      StringOp op;
      if (t == "LIKE" && e->ch.size() == 2 && strcol(e->ch[0]) && is_string_literal(e->ch[1])) {
        op.kind = StringOp::LIKE;
        op.col = e->ch[0]->col;
        op.literal = unquote(e->ch[1]->token);
        // the reference hands the pattern to a regular-expression engine
        // (LogicalProject.cpp:31-47, 128-131); only '%' and '_' are restated here
        if (op.literal.find_first_of(".^$*+?()[]{}|\\") != std::string::npos)
          fail(GX_ERR_UNSUPPORTED, "LIKE pattern with regular-expression characters: " + op.literal);
      } else if (t == "CHAR_LENGTH" && e->ch.size() == 1 && strcol(e->ch[0])) {
        op.kind = StringOp::CHAR_LENGTH;
        op.col = e->ch[0]->col;
      } else if ((t == "=" || t == "<>" || t == "<" || t == "<=" || t == ">" || t == ">=") && e->ch.size() == 2 &&
                 (strcol(e->ch[0]) || strcol(e->ch[1])) &&
                 (strcol(e->ch[0]) || is_string_literal(e->ch[0])) &&
                 (strcol(e->ch[1]) || is_string_literal(e->ch[1]))) {
        const bool swapped = !strcol(e->ch[0]);
        std::string o = t;
        if (swapped) o = o == "<" ? ">" : o == ">" ? "<" : o == "<=" ? ">=" : o == ">=" ? "<=" : o;
        op.kind = o == "=" ? StringOp::EQ : o == "<>" ? StringOp::NE : o == "<" ? StringOp::LT
                : o == "<=" ? StringOp::LE : o == ">" ? StringOp::GT : StringOp::GE;
        const ExprPtr& l = e->ch[swapped ? 1 : 0];
        const ExprPtr& r = e->ch[swapped ? 0 : 1];
        op.col = l->col;
        if (strcol(r)) op.col2 = r->col;
        else op.literal = unquote(r->token);
      } else if ((t == "CAST_VARCHAR" || t == "CAST_CHAR") && e->ch.size() == 1 && e->ch[0]->kind == Expr::LIT &&
                 !is_null_literal(e->ch[0])) {
        // CAST(literal):VARCHAR is a VARCHAR literal before the pre-pass runs
        // (transform_cast_literal, expression_tree.hpp:238-256)
        auto l = std::make_shared<Expr>(*e->ch[0]);
        if (!is_string_literal(l)) l->token = "'" + l->token + "'";
        l->lit_type_token.clear();
        touched = true;
        return l;
      } else if (t == "CASE" && e->ch.size() >= 3 && e->ch.size() % 2 == 1) {
        // CASE(c1, v1, ..., ck, vk, else) is FIRST_NON_MAGIC(MAGIC_IF_NOT(c1,
        // v1), ...) nested to the right (expression_tree.hpp:200-220); from
        // the innermost pair out, each pair whose THEN and ELSE are string
        // operands becomes a string column, until one is not
        ExprPtr cur = e->ch.back();
        size_t i = e->ch.size() - 1;
        bool folded = false;
        while (i >= 2 && string_operand(e->ch[i - 1]) && string_operand(cur) &&
               !(is_null_literal(e->ch[i - 1]) && is_null_literal(cur))) {
          const ExprPtr& c = e->ch[i - 2];
          const ExprPtr& v = e->ch[i - 1];
          if (c->kind == Expr::LIT)  // RAL_EXPECTS, LogicalProject.cpp:627
            fail(GX_ERR_UNSUPPORTED, "CASE operator not supported for condition expression literals");
          StringOp cs;
          cs.kind = StringOp::CASE;
          cs.cond = rebuild_typed(c);
          if (strcol(v)) cs.col = v->col;
          else if (is_null_literal(v)) cs.then_null = true;
          else cs.literal = unquote(v->token);
          if (strcol(cur)) cs.col2 = cur->col;
          else if (is_null_literal(cur)) cs.else_null = true;
          else cs.literal2 = unquote(cur->token);
          cur = column_of(cs);
          folded = true;
          i -= 2;
        }
        if (!folded) return e;
        touched = true;
        if (i == 0) return cur;
        e->ch.resize(i);
        e->ch.push_back(cur);
        return e;
      } else if (!string_function(e, op)) {
        return e;
      }
      touched = true;
      return column_of(op);
    };
    root = walk(root);
    // a string column left anywhere but the root is an unsupported use
    std::function<void(const ExprPtr&, bool)> check = [&](const ExprPtr& e, bool top) {
      if (strcol(e) && !top)
        fail(GX_ERR_UNSUPPORTED, "string column " + e->token +
                                     " used outside LIKE, CHAR_LENGTH, a comparison or a CASE with string results");
      if (e->kind == Expr::LIT && is_string_literal(e) && !top)
        fail(GX_ERR_UNSUPPORTED, "string literal " + e->token + " used outside a string operator");
      for (const auto& c : e->ch) check(c, false);
    };
    check(root, true);
    if (touched) text = rebuild_typed(root);
  }
}

}  // namespace gx
