// str_prepass.cu -- the string pre-pass of the evaluator: the string operators of an
// expression over cudf-layout string columns (int32 offsets + UTF-8
// characters) evaluated into BOOL8 / INT32 columns that replace them in the
// expression, as the reference's function_evaluator_transformer does
// (engine/src/execution_kernels/LogicalProject.cpp:671-742, with
// evaluate_string_functions :103-603) before its interpreter runs.
//
// LIKE follows the reference's translation of the pattern into a regular
// expression (like_expression_to_regex_str, LogicalProject.cpp:31-47): '%' ->
// "(?:.*?)", '_' -> "(?:.)", anchored at the ends the pattern does not start
// or end with '%', matched by cudf::strings::contains_re; "." stands for one
// character (UTF-8) other than a newline.  An empty pattern is the empty
// regular expression, which every string contains.  Patterns holding other
// regular-expression metacharacters are rejected (the reference hands them
// to the regex engine as they are).  Comparisons with a string literal follow
// the interpreter's string_view comparison (interpreter_ops.cuh:623-719):
// bytes in lexicographic order.  CHAR_LENGTH counts characters
// (cudf::strings::count_characters).  A NULL string gives NULL.
#include "str_prepass.h"

#include <algorithm>
#include <cstring>

namespace gx {

namespace {

__device__ __forceinline__ int utf8_len(unsigned char c) {
  return c < 0x80 ? 1 : (c >> 5) == 0x6 ? 2 : (c >> 4) == 0xE ? 3 : (c >> 3) == 0x1E ? 4 : 1;
}

// The LIKE pattern's regular expression searched in s: '%' between other
// pattern characters is a run of characters but a newline, '_' one character
// but a newline.  A leading '%' (no '^' anchor) lets the match start
// anywhere, a trailing one (no '$' anchor) end anywhere, newlines included.
// Greedy with backtracking to the last '%'.
__device__ bool like_match(const unsigned char* s, int n, const unsigned char* p, int m) {
  if (m == 0) return true;
  int lead = 0;  // the leading run of '%'
  while (lead < m && p[lead] == '%') lead++;
  if (lead == m) return true;
  int tail = m;  // pattern positions >= tail are the trailing run of '%'
  while (tail > lead && p[tail - 1] == '%') tail--;
  int i = 0, j = lead, star_j = lead > 0 ? lead - 1 : -1, star_i = 0;
  while (true) {
    if (j >= tail) {
      if (tail < m || i == n) return true;  // a trailing '%' takes any rest
    } else if (i < n) {
      if (p[j] == '%') {
        star_j = j++;
        star_i = i;
        continue;
      }
      if (p[j] == '_' ? s[i] != '\n' : p[j] == s[i]) {
        i += p[j] == '_' ? utf8_len(s[i]) : 1;
        j++;
        continue;
      }
    }
    // retry from the last '%' one character further; an inner '%' stops at a
    // newline, the leading one does not
    if (star_j < 0 || star_i >= n) return false;
    if (star_j >= lead && s[star_i] == '\n') return false;
    star_i += utf8_len(s[star_i]);
    i = star_i;
    j = star_j + 1;
  }
}

__device__ int compare_bytes(const unsigned char* s, int n, const unsigned char* p, int m) {
  const int k = n < m ? n : m;
  for (int i = 0; i < k; i++)
    if (s[i] != p[i]) return s[i] < p[i] ? -1 : 1;
  return n < m ? -1 : (n > m ? 1 : 0);
}

struct StrArgs {
  const int32_t* offs;
  const unsigned char* chars;
  int64_t off;
  const uint32_t* mask;
  int64_t n;
  const unsigned char* pat;
  int plen;
  int op;  // StringOp::Kind
  void* out;
  uint32_t* out_mask;
};

// one warp per 32 rows: a lane per row, the warp's validity word by ballot
__global__ void k_string_op(StrArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t nwords = (a.n + 31) / 32;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; w < nwords;
       w += ((int64_t)gridDim.x * blockDim.x) / 32) {
    const int64_t r = w * 32 + lane;
    bool valid = false;
    if (r < a.n) {
      const int64_t q = a.off + r;
      valid = !a.mask || ((a.mask[q >> 5] >> (q & 31)) & 1u);
      const int32_t b = a.offs[q], e = a.offs[q + 1];
      const unsigned char* s = a.chars + b;
      const int len = e - b;
      if (a.op == StringOp::CHAR_LENGTH) {
        int c = 0;
        for (int i = 0; i < len; i++) c += (s[i] & 0xC0) != 0x80;
        ((int32_t*)a.out)[r] = valid ? c : 0;
      } else {
        bool v = false;
        if (valid) {
          if (a.op == StringOp::LIKE) {
            v = like_match(s, len, a.pat, a.plen);
          } else {
            const int c = compare_bytes(s, len, a.pat, a.plen);
            switch (a.op) {
              case StringOp::EQ: v = c == 0; break;
              case StringOp::NE: v = c != 0; break;
              case StringOp::LT: v = c < 0; break;
              case StringOp::LE: v = c <= 0; break;
              case StringOp::GT: v = c > 0; break;
              default: v = c >= 0; break;
            }
          }
        }
        ((unsigned char*)a.out)[r] = v ? 1 : 0;
      }
    }
    const uint32_t word = __ballot_sync(0xffffffffu, r < a.n && valid);
    if (lane == 0) a.out_mask[w] = word;
  }
}

}  // namespace

void launch_string_op(const ColumnView& col, const StringOp& op, const void* pattern_dev, gx_column& out,
                      cudaStream_t s) {
  StrArgs a{};
  a.offs = col.str_offsets;
  a.chars = (const unsigned char*)col.data;
  a.off = col.offset;
  a.mask = col.mask;
  a.n = col.size;
  a.pat = (const unsigned char*)pattern_dev;
  a.plen = (int)op.literal.size();
  a.op = op.kind;
  a.out = out.data;
  a.out_mask = out.null_mask;
  if (a.n == 0) return;
  const int64_t warps = (a.n + 31) / 32;
  const int grid = (int)std::min<int64_t>((warps + 7) / 8, 152 * 32);
  k_string_op<<<grid, 256, 0, s>>>(a);
  check_cuda(cudaGetLastError(), "k_string_op");
  add_launches(1);
}

std::vector<gx_column> run_string_prepass(std::vector<ColumnView>& cols, const std::vector<StringOp>& ops,
                                          cudaStream_t s) {
  std::vector<gx_column> made;
  if (ops.empty()) return made;
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  size_t pbytes = 0;
  for (const auto& op : ops) pbytes += (op.literal.size() + 15) / 16 * 16;
  std::string host(std::max<size_t>(pbytes, 16), '\0');
  std::vector<size_t> poff;
  size_t at = 0;
  for (const auto& op : ops) {
    poff.push_back(at);
    std::memcpy(&host[at], op.literal.data(), op.literal.size());
    at += (op.literal.size() + 15) / 16 * 16;
  }
  char* pdev = (char*)dev_alloc(host.size(), s);
  try {
    check_cuda(cudaMemcpyAsync(pdev, host.data(), host.size(), cudaMemcpyHostToDevice, s), "string patterns");
    for (size_t i = 0; i < ops.size(); i++) {
      const StringOp& op = ops[i];
      const ColumnView c = cols.at(op.col);  // a copy: cols grows below
      if (c.type != STRING) fail(GX_ERR_TYPE, "string operator over a non-string column");
      gx_column out = alloc_column(op.kind == StringOp::CHAR_LENGTH ? INT32 : BOOL8, n, s);
      made.push_back(out);
      launch_string_op(c, op, pdev + poff[i], out, s);
      ColumnView v{out.type_id, out.data, out.null_mask, 0, n};
      cols.push_back(v);
    }
  } catch (...) {
    for (auto& c : made) free_column(c, s);
    dev_free(pdev, s);
    throw;
  }
  // the copy of the patterns must finish before their host buffer goes away
  check_cuda(cudaStreamSynchronize(s), "string pre-pass");
  dev_free(pdev, s);
  return made;
}

}  // namespace gx
