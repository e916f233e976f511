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
  // comparisons of two string columns: the right-hand column (offs2 set)
  const int32_t* offs2;
  const unsigned char* chars2;
  int64_t off2;
  const uint32_t* mask2;
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
      const unsigned char* pat = a.pat;
      int plen = a.plen;
      if (a.offs2) {
        const int64_t q2 = a.off2 + r;
        valid = valid && (!a.mask2 || ((a.mask2[q2 >> 5] >> (q2 & 31)) & 1u));
        pat = a.chars2 + a.offs2[q2];
        plen = a.offs2[q2 + 1] - a.offs2[q2];
      }
      if (a.op == StringOp::CHAR_LENGTH) {
        int c = 0;
        for (int i = 0; i < len; i++) c += (s[i] & 0xC0) != 0x80;
        ((int32_t*)a.out)[r] = valid ? c : 0;
      } else {
        bool v = false;
        if (valid) {
          if (a.op == StringOp::LIKE) {
            v = like_match(s, len, pat, plen);
          } else {
            const int c = compare_bytes(s, len, pat, plen);
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

// ------------------------------------------------------------ string builder
// A strings column is built in three launches: row sizes and validity (and a
// character total per block), an exclusive scan of the block totals, then
// offsets and characters.  A block covers kBuildWarps x kBuildWords 32-row
// words; a warp copies the characters of its rows one row at a time, lanes
// on consecutive bytes.
constexpr int kBuildWarps = 8, kBuildWords = 8;
constexpr int64_t kBuildRows = kBuildWarps * kBuildWords * 32;

struct BuildSrc {
  const int32_t* offs;
  const unsigned char* chars;
  const uint32_t* mask;
  int64_t off;
  const unsigned char* lit;
  int32_t lit_len;
  int32_t kind;  // StrSource::Kind
};

struct BuildArgs {
  BuildSrc a, b;
  const int32_t* map;
  const unsigned char* cond;
  const uint32_t* cond_mask;
  int64_t cond_off;
  int64_t m;
  int32_t* out_offs;
  uint32_t* out_mask;
  unsigned char* out_chars;
  uint64_t* block_sums;
};

__device__ __forceinline__ bool bit_of(const uint32_t* mask, int64_t q) {
  return !mask || ((mask[q >> 5] >> (q & 31)) & 1u);
}

__device__ __forceinline__ void resolve(const BuildArgs& a, int64_t o, const unsigned char*& p, int& len,
                                        bool& valid) {
  bool use_a = true;
  if (a.cond) {
    const int64_t q = a.cond_off + o;
    use_a = bit_of(a.cond_mask, q) && a.cond[q] != 0;
  }
  const BuildSrc& s = use_a ? a.a : a.b;
  p = nullptr;
  len = 0;
  valid = false;
  if (s.kind == StrSource::NUL) return;
  if (s.kind == StrSource::LITERAL) {
    p = s.lit;
    len = s.lit_len;
    valid = true;
    return;
  }
  const int64_t q = s.off + (a.map ? (int64_t)a.map[o] : o);
  if (!bit_of(s.mask, q)) return;
  const int32_t b0 = s.offs[q];
  p = s.chars + b0;
  len = s.offs[q + 1] - b0;
  valid = true;
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

__global__ void __launch_bounds__(kBuildWarps * 32) k_str_sizes(BuildArgs a) {
  __shared__ uint64_t s_sum[kBuildWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = ((int64_t)blockIdx.x * kBuildWarps + warp) * kBuildWords;
  uint64_t total = 0;
  for (int k = 0; k < kBuildWords; k++) {
    const int64_t o = (w0 + k) * 32 + lane;
    if ((w0 + k) * 32 >= a.m) break;
    const unsigned char* p;
    int len = 0;
    bool valid = false;
    if (o < a.m) resolve(a, o, p, len, valid);
    const uint32_t word = __ballot_sync(0xffffffffu, valid);
    if (lane == 0) a.out_mask[w0 + k] = word;
    total += (uint64_t)warp_sum(len);
  }
  if (lane == 0) s_sum[warp] = total;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t = 0;
    for (int i = 0; i < kBuildWarps; i++) t += s_sum[i];
    a.block_sums[blockIdx.x] = t;
  }
}

// block_sums hold each block's first character position (exclusive scan)
__global__ void __launch_bounds__(kBuildWarps * 32) k_str_write(BuildArgs a) {
  __shared__ uint64_t s_sum[kBuildWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = ((int64_t)blockIdx.x * kBuildWarps + warp) * kBuildWords;
  uint64_t total = 0;
  for (int k = 0; k < kBuildWords; k++) {
    const int64_t o = (w0 + k) * 32 + lane;
    if ((w0 + k) * 32 >= a.m) break;
    const unsigned char* p;
    int len = 0;
    bool valid = false;
    if (o < a.m) resolve(a, o, p, len, valid);
    total += (uint64_t)warp_sum(len);
  }
  if (lane == 0) s_sum[warp] = total;
  __syncthreads();
  uint64_t pos = a.block_sums[blockIdx.x];
  for (int i = 0; i < warp; i++) pos += s_sum[i];
  for (int k = 0; k < kBuildWords; k++) {
    const int64_t o = (w0 + k) * 32 + lane;
    if ((w0 + k) * 32 >= a.m) break;
    const unsigned char* p = nullptr;
    int len = 0;
    bool valid = false;
    if (o < a.m) resolve(a, o, p, len, valid);
    int incl = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    const uint64_t dst = pos + (uint64_t)(incl - len);
    if (o < a.m) {
      a.out_offs[o] = (int32_t)dst;
      if (o == a.m - 1) a.out_offs[a.m] = (int32_t)(dst + (uint64_t)len);
    }
    for (int j = 0; j < 32; j++) {
      const int lj = __shfl_sync(0xffffffffu, len, j);
      if (lj == 0) continue;
      const unsigned char* pj = (const unsigned char*)__shfl_sync(0xffffffffu, (unsigned long long)p, j);
      const uint64_t dj = __shfl_sync(0xffffffffu, (unsigned long long)dst, j);
      for (int b = lane; b < lj; b += 32) a.out_chars[dj + b] = pj[b];
    }
    pos += (uint64_t)__shfl_sync(0xffffffffu, incl, 31);
  }
}

BuildSrc device_source(const StrSource& s, const unsigned char* lit_dev) {
  BuildSrc b{};
  b.kind = s.kind;
  if (s.kind == StrSource::COLUMN) {
    if (s.col.type != STRING || !s.col.str_offsets) fail(GX_ERR_TYPE, "string source is not a string column");
    b.offs = s.col.str_offsets;
    b.chars = (const unsigned char*)s.col.data;
    b.mask = s.col.mask;
    b.off = s.col.offset;
  } else if (s.kind == StrSource::LITERAL) {
    b.lit = lit_dev;
    b.lit_len = (int32_t)s.literal.size();
  }
  return b;
}

}  // namespace

gx_column build_strings(const StrSource& a, const StrSource& b, const int32_t* map, const ColumnView* cond,
                        int64_t rows, cudaStream_t s) {
  if (rows < 0 || rows > INT32_MAX) fail(GX_ERR_UNSUPPORTED, "string columns hold at most 2^31 - 1 rows");
  if (map && a.kind != StrSource::COLUMN) fail(GX_ERR_INVALID, "a gather reads a column");
  if (cond && cond->type != BOOL8)
    fail(GX_ERR_TYPE, "Expression does not evaluate to a boolean mask");  // LogicalProject.cpp:636
  const int64_t nblocks = (rows + kBuildRows - 1) / kBuildRows;
  const int64_t words = mask_words_for(rows);
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  // [mask | offsets | block sums + total | literals]
  const size_t mask_b = al((size_t)words * 4), offs_b = al((size_t)(rows + 1) * 4);
  const size_t sums_b = al((size_t)(nblocks + 1) * 8);
  const size_t la = a.kind == StrSource::LITERAL ? al(a.literal.size() + 1) : 0;
  const size_t lb = b.kind == StrSource::LITERAL ? al(b.literal.size() + 1) : 0;
  char* base = (char*)dev_alloc(mask_b + offs_b + sums_b + la + lb, s);
  gx_column out{};
  out.type_id = STRING;
  out.null_mask = (uint32_t*)base;
  out.string_offsets = (int32_t*)(base + mask_b);
  out.size = rows;
  out.capacity = rows;
  try {
    uint64_t* sums = (uint64_t*)(base + mask_b + offs_b);
    unsigned char* lit_a = (unsigned char*)(base + mask_b + offs_b + sums_b);
    unsigned char* lit_b = lit_a + la;
    check_cuda(cudaMemsetAsync(base, 0, mask_b + offs_b, s), "string column clear");
    if (la && !a.literal.empty())
      check_cuda(cudaMemcpyAsync(lit_a, a.literal.data(), a.literal.size(), cudaMemcpyHostToDevice, s), "literal");
    if (lb && !b.literal.empty())
      check_cuda(cudaMemcpyAsync(lit_b, b.literal.data(), b.literal.size(), cudaMemcpyHostToDevice, s), "literal");
    BuildArgs args{};
    args.a = device_source(a, lit_a);
    args.b = device_source(b, lit_b);
    args.map = map;
    if (cond) {
      args.cond = (const unsigned char*)cond->data;
      args.cond_mask = cond->mask;
      args.cond_off = cond->offset;
    }
    args.m = rows;
    args.out_offs = out.string_offsets;
    args.out_mask = out.null_mask;
    args.block_sums = sums;
    uint64_t total = 0;
    if (rows > 0) {
      k_str_sizes<<<(unsigned)nblocks, kBuildWarps * 32, 0, s>>>(args);
      check_cuda(cudaGetLastError(), "k_str_sizes");
      launch_scan_tiles(sums, nblocks, (unsigned long long*)(sums + nblocks), s);
      check_cuda(cudaMemcpyAsync(&total, sums + nblocks, 8, cudaMemcpyDeviceToHost, s), "string size");
      add_launches(1);
    }
    // the literals' host bytes and `total` must outlive the copies
    check_cuda(cudaStreamSynchronize(s), "string size sync");
    if (total > (uint64_t)INT32_MAX) fail(GX_ERR_UNSUPPORTED, "string column over 2^31 - 1 characters");
    out.data = dev_alloc(al(total ? total : 1), s);
    out.string_bytes = (int64_t)total;
    if (rows > 0) {
      args.out_chars = (unsigned char*)out.data;
      k_str_write<<<(unsigned)nblocks, kBuildWarps * 32, 0, s>>>(args);
      check_cuda(cudaGetLastError(), "k_str_write");
      add_launches(1);
    }
  } catch (...) {
    if (out.data) dev_free(out.data, s);
    dev_free(base, s);
    throw;
  }
  return out;
}

void launch_string_op(const ColumnView& col, const ColumnView* col2, const StringOp& op, const void* pattern_dev,
                      gx_column& out, cudaStream_t s) {
  StrArgs a{};
  a.offs = col.str_offsets;
  a.chars = (const unsigned char*)col.data;
  a.off = col.offset;
  a.mask = col.mask;
  if (col2) {
    a.offs2 = col2->str_offsets;
    a.chars2 = (const unsigned char*)col2->data;
    a.off2 = col2->offset;
    a.mask2 = col2->mask;
  }
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

std::vector<gx_column> run_string_prepass(
    std::vector<ColumnView>& cols, const std::vector<StringOp>& ops, cudaStream_t s,
    const std::function<gx_column(const std::vector<ColumnView>&, const std::string&)>& eval_bool) {
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
  auto string_col = [&](int c) {
    const ColumnView v = cols.at(c);
    if (v.type != STRING) fail(GX_ERR_TYPE, "string operator over a non-string column");
    return v;
  };
  try {
    check_cuda(cudaMemcpyAsync(pdev, host.data(), host.size(), cudaMemcpyHostToDevice, s), "string patterns");
    for (size_t i = 0; i < ops.size(); i++) {
      const StringOp& op = ops[i];
      gx_column out{};
      if (op.kind == StringOp::CASE) {
        StrSource a, b;
        if (op.col >= 0) {
          a.kind = StrSource::COLUMN;
          a.col = string_col(op.col);
        } else if (!op.then_null) {
          a.kind = StrSource::LITERAL;
          a.literal = op.literal;
        }
        if (op.col2 >= 0) {
          b.kind = StrSource::COLUMN;
          b.col = string_col(op.col2);
        } else if (!op.else_null) {
          b.kind = StrSource::LITERAL;
          b.literal = op.literal2;
        }
        gx_column mask = eval_bool(cols, op.cond);
        try {
          const ColumnView mv{mask.type_id, mask.data, mask.null_mask, 0, n};
          out = build_strings(a, b, nullptr, &mv, n, s);
        } catch (...) {
          free_column(mask, s);
          throw;
        }
        free_column(mask, s);
      } else {
        const ColumnView c = string_col(op.col);  // a copy: cols grows below
        ColumnView c2{};
        if (op.col2 >= 0) c2 = string_col(op.col2);
        out = alloc_column(op.result_type(), n, s);
        launch_string_op(c, op.col2 >= 0 ? &c2 : nullptr, op, pdev + poff[i], out, s);
      }
      made.push_back(out);
      cols.push_back(ColumnView{out.type_id, out.data, out.null_mask, 0, n, out.string_offsets});
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
