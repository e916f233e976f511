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

#include "regex_vm.h"

#include <algorithm>
#include <array>
#include <cstring>
#include <map>

namespace gx {

namespace {

__device__ __forceinline__ int utf8_len(unsigned char c) {
  return c < 0x80 ? 1 : (c >> 5) == 0x6 ? 2 : (c >> 4) == 0xE ? 3 : (c >> 3) == 0x1E ? 4 : 1;
}

// The LIKE pattern's regular expression searched in s: '%' between other
// pattern characters is a run of characters but a newline, '_' one character
// but a newline.  A trailing '%' (no '$' anchor) lets the match end anywhere.
// A leading '%' (no '^' anchor) lets it start anywhere: each start t is tried
// in turn.  From a start, a greedy match that backtracks to its last inner
// '%' (the classic wildcard algorithm; inner '%'s cannot cross a newline, so
// none of them can take over where the last one stops).  A start fails over
// to the next when a newline or a mismatch before the first inner '%' stops
// it; when the last inner '%' has run to the end of s, no later start can
// match either.
__device__ bool like_match(const unsigned char* s, int n, const unsigned char* p, int m) {
  if (m == 0) return true;
  int lead = 0;  // the leading run of '%'
  while (lead < m && p[lead] == '%') lead++;
  if (lead == m) return true;
  int tail = m;  // pattern positions >= tail are the trailing run of '%'
  while (tail > lead && p[tail - 1] == '%') tail--;
  const int c0 = p[lead] == '_' ? -1 : p[lead];  // a match starts with this byte, when not -1
  for (int t = 0;; t += utf8_len(s[t])) {
    if (lead > 0 && c0 >= 0) {  // next start: the next c0
      while (t < n && s[t] != c0) t++;
      if (t >= n) return false;
    }
    int i = t, j = lead, star_j = -1, star_i = 0;
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
      // retry from the last inner '%' one character further, and on to the
      // next byte that can continue the match (when a literal follows it)
      if (star_j < 0) break;  // no inner '%' yet: the next start
      const int nj = star_j + 1;
      const int cj = (nj < tail && p[nj] != '_' && p[nj] != '%') ? p[nj] : -1;
      bool next_start = false;
      while (true) {
        if (star_i >= n) return false;  // ran to the end: no start can match
        if (s[star_i] == '\n') {        // an inner '%' stops at a newline
          next_start = true;
          break;
        }
        star_i += utf8_len(s[star_i]);
        if (cj < 0 || star_i >= n || s[star_i] == cj) break;
      }
      if (next_start) break;
      if (star_i >= n && cj >= 0) return false;
      i = star_i;
      j = nj;
    }
    if (lead == 0 || t >= n) return false;
  }
}

__device__ int compare_bytes(const unsigned char* s, int n, const unsigned char* p, int m) {
  const int k = n < m ? n : m;
  for (int i = 0; i < k; i++) {
    const unsigned char c = s[i];
    if (c != p[i]) return c < p[i] ? -1 : 1;
  }
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
  // LIKE as a byte automaton (LikeDfa), or null: [byte class 256 | flags S |
  // transitions S x C], copied to shared memory by each block
  const unsigned char* dfa;
  int dfa_states, dfa_classes, dfa_start;
  void* out;
  uint32_t* out_mask;
};

// one warp per 32 rows: a lane per row, the warp's validity word by ballot
__global__ void k_string_op(StrArgs a) {
  extern __shared__ unsigned char s_dfa[];
  if (a.dfa) {  // uniform over the block
    const int bytes = a.dfa_classes ? 256 + a.dfa_states * (1 + a.dfa_classes) : a.dfa_states * 257;
    for (int i = threadIdx.x; i < bytes; i += blockDim.x) s_dfa[i] = a.dfa[i];
    __syncthreads();
  }
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
        // characters = bytes that are not UTF-8 continuation bytes (10xxxxxx),
        // counted four at a time over the aligned words of the row
        int c = 0, i = 0;
        for (; i < len && ((uintptr_t)(s + i) & 3u); i++) c += (s[i] & 0xC0) != 0x80;
        for (; i + 4 <= len; i += 4) {
          const uint32_t w = *(const uint32_t*)(s + i);
          c += 4 - __popc((w >> 7) & ~(w >> 6) & 0x01010101u);
        }
        for (; i < len; i++) c += (s[i] & 0xC0) != 0x80;
        ((int32_t*)a.out)[r] = valid ? c : 0;
      } else {
        bool v = false;
        if (valid) {
          if (a.op == StringOp::LIKE && a.dfa && a.dfa_classes == 0) {
            // byte-indexed automaton: one shared-memory read per byte; bit 7
            // of a state marks an absorbing one (the answer is decided)
            const unsigned char* tr = s_dfa;
            const unsigned char* flags = s_dfa + a.dfa_states * 256;
            unsigned st = (unsigned)a.dfa_start | ((flags[a.dfa_start] & 2) ? 0x80u : 0u);
            int i = 0;
            for (; i < len && !(st & 0x80u) && ((uintptr_t)(s + i) & 3u); i++) st = tr[((st & 0x7Fu) << 8) | s[i]];
            for (; !(st & 0x80u) && i + 4 <= len; i += 4) {
              const uint32_t w = *(const uint32_t*)(s + i);
              st = tr[((st & 0x7Fu) << 8) | (w & 0xFFu)];
              st = tr[((st & 0x7Fu) << 8) | ((w >> 8) & 0xFFu)];
              st = tr[((st & 0x7Fu) << 8) | ((w >> 16) & 0xFFu)];
              st = tr[((st & 0x7Fu) << 8) | (w >> 24)];
            }
            for (; i < len && !(st & 0x80u); i++) st = tr[((st & 0x7Fu) << 8) | s[i]];
            v = flags[st & 0x7Fu] & 1;
          } else if (a.op == StringOp::LIKE && a.dfa) {
            // a table step per byte, the same instructions in every lane; the
            // row's aligned middle is read a 4-byte word at a time
            const unsigned char* flags = s_dfa + 256;
            const unsigned char* tr = flags + a.dfa_states;
            const int nc = a.dfa_classes;
            int st = a.dfa_start, i = 0;
            bool done = false;
            for (; i < len && ((uintptr_t)(s + i) & 3u); i++) {
              st = tr[st * nc + s_dfa[s[i]]];
              if (flags[st] & 2) {  // absorbing: decided
                done = true;
                break;
              }
            }
            // (an absorbing state keeps itself on every byte, so one check
            // per word decides as early as a check per byte would)
            for (; !done && i + 4 <= len; i += 4) {
              const uint32_t w = *(const uint32_t*)(s + i);
              const int c0 = s_dfa[w & 0xFFu], c1 = s_dfa[(w >> 8) & 0xFFu], c2 = s_dfa[(w >> 16) & 0xFFu],
                        c3 = s_dfa[w >> 24];
              st = tr[st * nc + c0];
              st = tr[st * nc + c1];
              st = tr[st * nc + c2];
              st = tr[st * nc + c3];
              done = (flags[st] & 2) != 0;
            }
            for (; !done && i < len; i++) {
              st = tr[st * nc + s_dfa[s[i]]];
              if (flags[st] & 2) break;
            }
            v = flags[st] & 1;
          } else if (a.op == StringOp::LIKE) {
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
// words.  A warp's rows are copied together by warp_copy when they are long,
// a lane per row when they are short.
constexpr int kBuildWarps = 8, kBuildWords = 8;
constexpr int64_t kBuildRows = kBuildWarps * kBuildWords * 32;

struct BuildSrc {
  const int32_t* offs;
  const unsigned char* chars;
  const uint32_t* mask;
  int64_t off;
  int64_t end;  // the view's row end (off + size): its characters end at offs[end]
  const void* num;  // FORMAT: the typed column's data (mask, off as above)
  int32_t num_type;
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

// Rows longer than this on average (bytes) are copied by warp_copy; shorter
// ones by a lane each, which takes fewer instructions.
constexpr int kWarpCopyBytes = 32;

// The characters of a warp's 32 rows as one contiguous range of `total`
// bytes at out: lane l's row starts at byte ex (its exclusive prefix) and is
// n1 bytes from p1 followed by the rest from p2.  Lanes copy consecutive bytes
// (coalesced loads and stores), each finding its byte's row by a binary search
// over the lanes' prefixes.
__device__ __forceinline__ void warp_copy(unsigned char* out, int ex, int n1, const unsigned char* p1,
                                          const unsigned char* p2, int total, int lane) {
  for (int base = 0; base < total; base += 32) {
    const int k = base + lane;
    int lo = 0;  // the last lane whose row starts at or before byte k
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int e = __shfl_sync(0xffffffffu, ex, lo + step);
      if (e <= k) lo += step;
    }
    const int exj = __shfl_sync(0xffffffffu, ex, lo);
    const int n1j = __shfl_sync(0xffffffffu, n1, lo);
    const unsigned char* a1 = (const unsigned char*)__shfl_sync(0xffffffffu, (unsigned long long)p1, lo);
    const unsigned char* a2 = (const unsigned char*)__shfl_sync(0xffffffffu, (unsigned long long)p2, lo);
    if (k < total) {
      const int r = k - exj;
      out[k] = r < n1j ? a1[r] : a2[r - n1j];
    }
  }
}

// Rows of one 32-row word whose bytes total at most kStageBytes are written
// by their lanes into a per-warp shared-memory stage, then copied out by the
// whole warp with coalesced 4-byte stores (byte stores only at the two
// ends); the stage starts at pos % 4 so stage and output words line up.
constexpr int kStageBytes = 32 * kWarpCopyBytes;

__device__ __forceinline__ void stage_flush(unsigned char* out, uint64_t pos, const unsigned char* st, int wtot,
                                            int lane) {
  const int sh = (int)(pos & 3u);
  const int head = min(wtot, (4 - sh) & 3);
  if (lane < head) out[pos + lane] = st[sh + lane];
  const int nw = (wtot - head) >> 2;
  uint32_t* gw = (uint32_t*)(out + pos + head);
  const uint32_t* sw = (const uint32_t*)(st + sh + head);
  for (int w = lane; w < nw; w += 32) gw[w] = sw[w];
  const int t0 = head + nw * 4;
  if (lane < wtot - t0) out[pos + t0 + lane] = st[sh + t0 + lane];
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
  __shared__ __align__(16) unsigned char s_stage[kBuildWarps][kStageBytes + 8];
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
    const int wtot = __shfl_sync(0xffffffffu, incl, 31);
    if (wtot > kStageBytes) {  // long rows: the warp copies them together
      warp_copy(a.out_chars + pos, incl - len, len, p, nullptr, wtot, lane);
    } else {  // short rows: each lane stages its own, the warp writes them out
      unsigned char* st = s_stage[warp] + (pos & 3u) + (incl - len);
      for (int i = 0; i < len; i++) st[i] = p[i];
      __syncwarp();
      stage_flush(a.out_chars, pos, s_stage[warp], wtot, lane);
      __syncwarp();
    }
    pos += (uint64_t)wtot;
  }
}

// ------------------------------------------------------ string transforms
// Row-wise string functions (slices, case, trim, replace, concatenation,
// formatting of typed values), a thread per row: the same three launches as
// build_strings, each row's bytes produced by xform_row (sizing when d is
// null, writing otherwise).
struct XformArgs {
  int kind;  // StringOp::Kind
  BuildSrc a, b;
  BuildSrc more[kMaxConcatParts - 2];  // CONCAT: parts 3, 4, ...
  int nmore;
  const void* num;  // TO_STRING: the typed column
  const uint32_t* num_mask;
  int64_t num_off;
  int num_type;
  int i0, i1, step, i0v, i1v;
  // SLICE with positions per row: the start and stop columns (integer types,
  // offset 0; no stop column: to the end), a NULL position read as 0
  const void* p0;
  const void* p1;
  const uint32_t* p0m;
  const uint32_t* p1m;
  int p0t, p1t;
  const unsigned char* s1;  // TRIM: characters to strip; REPLACE: target
  int l1;
  const unsigned char* s2;  // REPLACE: replacement
  int l2;
  int64_t m;
  const int32_t* map;  // set: output row o is built from input row map[o] (a gather)
  int32_t* out_offs;
  uint32_t* out_mask;
  unsigned char* out_chars;
  uint64_t* block_sums;
};

__device__ __forceinline__ void source_row(const BuildSrc& s, int64_t o, const unsigned char*& p, int& len,
                                           bool& valid) {
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
  const int64_t q = s.off + o;
  if (!bit_of(s.mask, q)) return;
  const int32_t b0 = s.offs[q];
  p = s.chars + b0;
  len = s.offs[q + 1] - b0;
  valid = true;
}

__device__ __forceinline__ int put(unsigned char* d, int at, const unsigned char* src, int n) {
  if (d)
    for (int i = 0; i < n; i++) d[at + i] = src[i];
  return at + n;
}

// the character (as its byte count) of strip set `set` that matches s[i..]
__device__ bool in_set(const unsigned char* s, int i, int k, const unsigned char* set, int sl) {
  if (sl == 0) return k == 1 && s[i] <= ' ';  // no characters given: whitespace
  for (int j = 0; j < sl;) {
    const int cl = utf8_len(set[j]);
    if (cl == k) {
      bool eq = true;
      for (int t = 0; t < k; t++) eq = eq && set[j + t] == s[i + t];
      if (eq) return true;
    }
    j += cl;
  }
  return false;
}

// the decimal digits of v (as unsigned), zero-padded to `width`, at d + at;
// counted first, then written from the last digit (no buffer)
__device__ __forceinline__ int civil_digits(unsigned char* d, int at, int64_t v, int width) {
  uint64_t u = (uint64_t)v;
  int n = 1;
  for (uint64_t t = u; t >= 10; t /= 10) n++;
  if (n < width) n = width;
  if (d)
    for (int i = n - 1; i >= 0; i--) {
      d[at + i] = (unsigned char)('0' + u % 10);
      u /= 10;
    }
  return at + n;
}

// days since 1970-01-01 -> (y, m, d): the proleptic Gregorian conversion of
// H. Hinnant's "chrono-Compatible Low-Level Date Algorithms" (civil_from_days)
__device__ void civil_from_days(int64_t z, int64_t& y, int& m, int& dd) {
  z += 719468;
  const int64_t era = (z >= 0 ? z : z - 146096) / 146097;
  const int64_t doe = z - era * 146097;
  const int64_t yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  y = yoe + era * 400;
  const int64_t doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  const int64_t mp = (5 * doy + 2) / 153;
  dd = (int)(doy - (153 * mp + 2) / 5 + 1);
  m = (int)(mp < 10 ? mp + 3 : mp - 9);
  y += m <= 2;
}

__device__ __forceinline__ int64_t floor_div(int64_t a, int64_t b) {
  const int64_t q = a / b;
  return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

// A double as cudf::strings::from_floats writes it (the CAST to VARCHAR of
// FLOAT and DOUBLE columns, LogicalProject.cpp:62-92): NaN, Inf, -Inf; values
// in [1e-4, 1e9) in fixed notation, others scaled into [1, 10) by the binary
// decomposition of their decimal exponent and followed by e, its sign and at
// least two digits; at most 9 significant digits (the integer part's digits
// taken from 9 decimal places), the last rounded half up from the scaled
// remainder, trailing zeros dropped but one decimal place kept.  Every
// product, quotient and difference is a single correctly rounded operation
// (no contraction into fused multiply-adds), so the digits are those of the
// same steps in any IEEE binary64 arithmetic.
__device__ int format_double(double x, unsigned char* d) {
  const unsigned char* nan_t = (const unsigned char*)"NaN";
  const unsigned char* inf_t = (const unsigned char*)"-Inf";
  if (isnan(x)) return put(d, 0, nan_t, 3);
  const bool neg = signbit(x);
  if (isinf(x)) return neg ? put(d, 0, inf_t, 4) : put(d, 0, inf_t + 1, 3);
  int at = 0;
  if (neg) at = put(d, 0, inf_t, 1);
  double v = fabs(x);
  if (v == 0.0) return put(d, at, (const unsigned char*)"0.0", 3);
  const int fx[9] = {256, 128, 64, 32, 16, 8, 4, 2, 1};
  const double up[9] = {1e256, 1e128, 1e64, 1e32, 1e16, 1e8, 1e4, 1e2, 1e1};
  const double lo[9] = {1e-255, 1e-127, 1e-63, 1e-31, 1e-15, 1e-7, 1e-3, 1e-1, 1e0};
  int exp10 = 0;
  if (v >= 1e9) {
    for (int k = 0; k < 9; k++)
      if (v >= up[k]) {
        v = __ddiv_rn(v, up[k]);
        exp10 += fx[k];
      }
  } else if (v < 1e-4) {
    for (int k = 0; k < 9; k++)
      if (v < lo[k]) {
        v = __dmul_rn(v, up[k]);
        exp10 -= fx[k];
      }
  }
  uint64_t whole = (uint64_t)v;  // below 1e9 here
  int places = 9;
  uint64_t width = 1000000000ull;
  for (uint64_t i = whole; i >= 10; i /= 10) {
    places--;
    width /= 10;
  }
  const double frac = __dmul_rn(__dsub_rn(v, (double)whole), (double)width);
  uint64_t dec = (uint64_t)frac;
  dec += (uint64_t)__dmul_rn(2.0, __dsub_rn(frac, (double)dec));
  if (dec >= width) {
    dec = 0;
    whole++;
    if (exp10 != 0 && whole >= 10) {
      exp10++;
      whole = 1;
    }
  }
  while (places > 0 && dec % 10 == 0) {
    dec /= 10;
    places--;
  }
  const unsigned char dot = '.', e = 'e', plus = '+', minus = '-', zero = '0';
  at = civil_digits(d, at, (int64_t)whole, 1);
  at = put(d, at, &dot, 1);
  at = places > 0 ? civil_digits(d, at, (int64_t)dec, places) : put(d, at, &zero, 1);
  if (exp10 != 0) {
    at = put(d, at, &e, 1);
    at = put(d, at, exp10 < 0 ? &minus : &plus, 1);
    at = civil_digits(d, at, exp10 < 0 ? -exp10 : exp10, 2);
  }
  return at;
}

// formats row o of the typed column (cast_to_str_functor, LogicalProject.cpp:62-92)
__device__ int format_typed(const void* num, const uint32_t* mask, int64_t off, int type, int64_t o,
                             unsigned char* d, bool& valid) {
  const int64_t q = off + o;
  valid = bit_of(mask, q);
  if (!valid) return 0;
  int at = 0;
  switch (type) {
    case BOOL8: {  // cudf::strings::from_booleans: "true" / "false"
      const bool v = ((const uint8_t*)num)[q] != 0;
      const unsigned char* t = (const unsigned char*)(v ? "true" : "false");
      return put(d, 0, t, v ? 4 : 5);
    }
    case INT8: case INT16: case INT32: case INT64: {  // cudf::strings::from_integers
      int64_t v = type == INT8 ? ((const int8_t*)num)[q] : type == INT16 ? ((const int16_t*)num)[q]
                : type == INT32 ? ((const int32_t*)num)[q] : ((const int64_t*)num)[q];
      uint64_t u = (uint64_t)v;
      if (v < 0) {
        if (d) d[at] = '-';
        at++;
        u = 0 - u;
      }
      return civil_digits(d, at, (int64_t)u, 1);
    }
    case UINT8: case UINT16: case UINT32: case UINT64: {
      const uint64_t u = type == UINT8 ? ((const uint8_t*)num)[q] : type == UINT16
                       ? ((const uint16_t*)num)[q] : type == UINT32 ? ((const uint32_t*)num)[q]
                       : ((const uint64_t*)num)[q];
      return civil_digits(d, 0, (int64_t)u, 1);
    }
    case FLOAT32: return format_double((double)((const float*)num)[q], d);
    case FLOAT64: return format_double(((const double*)num)[q], d);
    default: break;
  }
  // timestamps: "%Y-%m-%d" for days, "%Y-%m-%d %H:%M:%S" otherwise
  int64_t days, sod = 0;
  if (type == TIMESTAMP_DAYS) {
    days = ((const int32_t*)num)[q];
  } else {
    const int64_t v = ((const int64_t*)num)[q];
    const int64_t per = type == TIMESTAMP_SECONDS ? 1 : type == TIMESTAMP_MILLISECONDS ? 1000
                      : type == TIMESTAMP_MICROSECONDS ? 1000000 : 1000000000;
    const int64_t secs = floor_div(v, per);
    days = floor_div(secs, 86400);
    sod = secs - days * 86400;
  }
  int64_t y;
  int m, dd;
  civil_from_days(days, y, m, dd);
  const unsigned char dash = '-', colon = ':', space = ' ';
  at = civil_digits(d, 0, y, 4);
  at = put(d, at, &dash, 1);
  at = civil_digits(d, at, m, 2);
  at = put(d, at, &dash, 1);
  at = civil_digits(d, at, dd, 2);
  if (type != TIMESTAMP_DAYS) {
    at = put(d, at, &space, 1);
    at = civil_digits(d, at, sod / 3600, 2);
    at = put(d, at, &colon, 1);
    at = civil_digits(d, at, sod / 60 % 60, 2);
    at = put(d, at, &colon, 1);
    at = civil_digits(d, at, sod % 60, 2);
  }
  return at;
}

__device__ __forceinline__ int format_value(const XformArgs& a, int64_t o, unsigned char* d, bool& valid) {
  return format_typed(a.num, a.num_mask, a.num_off, a.num_type, o, d, valid);
}

// The functions whose result is one or two byte ranges of their inputs
// (slices by a positive step, TRIM, CONCAT): the row is n1 bytes at p1, then
// len - n1 bytes at p2.  Returns len.
__device__ __forceinline__ bool is_segment_kind(const XformArgs& a) {
  return (a.kind == StringOp::SLICE && a.step > 0) || a.kind == StringOp::TRIM ||
         (a.kind == StringOp::CONCAT && a.nmore == 0 && a.a.kind != StrSource::FORMAT &&
          a.b.kind != StrSource::FORMAT);
}

// row o of an integer position column, 0 where it is NULL
__device__ __forceinline__ int64_t row_position(const void* p, const uint32_t* m, int t, int64_t o) {
  if (!bit_of(m, o)) return 0;
  switch (t) {
    case INT8: return ((const int8_t*)p)[o];
    case INT16: return ((const int16_t*)p)[o];
    case INT32: return ((const int32_t*)p)[o];
    case UINT8: return ((const uint8_t*)p)[o];
    case UINT16: return ((const uint16_t*)p)[o];
    case UINT32: return ((const uint32_t*)p)[o];
    default: return ((const int64_t*)p)[o];  // INT64, UINT64
  }
}

// the first lim bytes at p are all ASCII (read a 4-byte word at a time where
// aligned, so the loads do not wait on one another)
__device__ __forceinline__ bool ascii_prefix(const unsigned char* p, int lim) {
  uint32_t acc = 0;
  int i = 0;
  for (; i < lim && ((uintptr_t)(p + i) & 3u); i++) acc |= p[i];
  for (; i + 4 <= lim; i += 4) acc |= *(const uint32_t*)(p + i);
  for (; i < lim; i++) acc |= p[i];
  return (acc & 0x80808080u) == 0;
}

__device__ int xform_segments(const XformArgs& a, int64_t o, const unsigned char*& p1, int& n1,
                              const unsigned char*& p2, bool& valid) {
  const unsigned char* p;
  int n;
  source_row(a.a, o, p, n, valid);
  p1 = p2 = nullptr;
  n1 = 0;
  if (a.kind == StringOp::CONCAT) {  // cudf::strings::concatenate: NULL if either side is
    const unsigned char* q;
    int m;
    bool v2;
    source_row(a.b, o, q, m, v2);
    valid = valid && v2;
    if (!valid) return 0;
    p1 = p;
    n1 = n;
    p2 = q;
    return n + m;
  }
  if (!valid) return 0;
  if (a.kind == StringOp::SLICE && a.p0) {
    // cudf::strings::slice_strings with a start and a stop per row: the start
    // clamped at 0, a stop below 0 or past the end meaning the end, empty when
    // the start is not before the stop
    const int64_t s0 = row_position(a.p0, a.p0m, a.p0t, o);
    const int64_t s1 = a.p1 ? row_position(a.p1, a.p1m, a.p1t, o) : -1;
    int L = 0;
    for (int i = 0; i < n; i++) L += (p[i] & 0xC0) != 0x80;
    const int64_t b = s0 > 0 ? s0 : 0;
    if (b >= L) return 0;
    const int64_t e = (s1 < 0 || s1 > L) ? L : s1;
    if (b >= e) return 0;
    int bb = 0, c = 0;
    while (c < b) { bb += utf8_len(p[bb]); c++; }
    int eb = bb;
    while (c < e) { eb += utf8_len(p[eb]); c++; }
    p1 = p + bb;
    n1 = eb - bb;
    return n1;
  }
  if (a.kind == StringOp::SLICE && a.i0v && a.i1v && a.i0 >= 0 && a.i1 >= 0) {
    // [i0, i1) from the front (SUBSTRING with a length, LEFT).  When the
    // first min(n, i1) bytes are ASCII, characters are bytes: the slice is
    // [i0, min(n, i1)), found without a dependent walk
    const int lim = min(n, a.i1);
    if (ascii_prefix(p, lim)) {
      if (a.i0 >= lim) return 0;
      p1 = p + a.i0;
      n1 = lim - a.i0;
      return n1;
    }
    // otherwise walk at most i1 characters; the same clipping as below,
    // without counting the rest
    int i = 0, c = 0, bb = 0;
    while (i < n && c < a.i1) {
      if (c == a.i0) bb = i;
      i += utf8_len(p[i]);
      c++;
    }
    if (a.i0 >= c) return 0;  // begins at or after the end
    i = min(i, n);
    p1 = p + bb;
    n1 = i - bb;
    return n1;
  }
  if (a.kind == StringOp::SLICE) {  // cudf::strings::slice_strings, characters [begin, end)
    int L = 0;
    for (int i = 0; i < n; i++) L += (p[i] & 0xC0) != 0x80;
    int b = 0, e = L;
    if (a.i0v) b = a.i0 >= 0 ? (a.i0 < L ? a.i0 : L) : (L + a.i0 >= 0 ? L + a.i0 : 0);
    if (a.i1v) e = a.i1 >= 0 ? (a.i1 < L ? a.i1 : L) : (L + a.i1 >= 0 ? L + a.i1 : 0);
    if (b >= e) return 0;
    int bb = 0, c = 0;
    while (c < b) { bb += utf8_len(p[bb]); c++; }
    int eb = bb;
    while (c < e) { eb += utf8_len(p[eb]); c++; }
    p1 = p + bb;
    n1 = eb - bb;
    return n1;
  }
  // TRIM: cudf::strings::strip
  int b = 0, e = n;
  if (a.i0 != 2)
    while (b < e) {
      const int k = utf8_len(p[b]);
      if (!in_set(p, b, k, a.s1, a.l1)) break;
      b += k;
    }
  if (a.i0 != 1)
    while (e > b) {
      int k = e - 1;
      while (k > b && (p[k] & 0xC0) == 0x80) k--;
      if (!in_set(p, k, e - k, a.s1, a.l1)) break;
      e = k;
    }
  p1 = p + b;
  n1 = e - b;
  return n1;
}

// REGEXP_REPLACE of row o (cudf::strings::replace_with_backrefs,
// LogicalProject.cpp:149-183), by the Pike VM of regex_vm.h
__device__ int regex_row(const XformArgs& a, int64_t o, unsigned char* d, bool& valid) {
  const unsigned char* p;
  int n;
  source_row(a.a, o, p, n, valid);
  if (!valid) return 0;
  return regex_replace_row(a.s1, a.s2, a.l2, p, n, a.i0v ? a.i0 : 0, d);
}

// ------------------------------------------------------ case mapping
// Unicode case mappings and alphabetic ranges, sorted by code point
#include "case_tables.inc"

__device__ __forceinline__ int find_cp(const uint32_t* keys, int count, uint32_t c) {
  int lo = 0, hi = count - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const uint32_t k = keys[mid];
    if (k == c) return mid;
    if (k < c) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

// c's upper- or lowercase mapping into m (1 to 3 code points); returns the count
__device__ int case_map(uint32_t c, bool upper, uint32_t* m) {
  int k = upper ? find_cp(kUpperFrom, kUpperCount, c) : find_cp(kLowerFrom, kLowerCount, c);
  if (k >= 0) {
    m[0] = upper ? kUpperTo[k] : kLowerTo[k];
    return 1;
  }
  k = upper ? find_cp(kUpperMultiFrom, kUpperMultiCount, c) : find_cp(kLowerMultiFrom, kLowerMultiCount, c);
  if (k < 0) {
    m[0] = c;
    return 1;
  }
  const uint32_t* t = (upper ? kUpperMultiTo : kLowerMultiTo) + 3 * k;
  int n = 0;
  for (int j = 0; j < 3 && t[j]; j++) m[n++] = t[j];
  return n;
}

__device__ bool is_alpha_cp(uint32_t c) {
  int lo = 0, hi = kAlphaCount - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (c < kAlphaLo[mid]) hi = mid - 1;
    else if (c > kAlphaHi[mid]) lo = mid + 1;
    else return true;
  }
  return false;
}

// c as UTF-8 at d + at (counted only when d is null)
__device__ __forceinline__ int put_utf8(unsigned char* d, int at, uint32_t c) {
  const int n = c < 0x80 ? 1 : c < 0x800 ? 2 : c < 0x10000 ? 3 : 4;
  if (d) {
    if (n == 1) {
      d[at] = (unsigned char)c;
    } else {
      const unsigned char lead = n == 2 ? 0xC0 : n == 3 ? 0xE0 : 0xF0;
      d[at] = (unsigned char)(lead | (c >> (6 * (n - 1))));
      for (int j = 1; j < n; j++) d[at + j] = (unsigned char)(0x80 | ((c >> (6 * (n - 1 - j))) & 0x3F));
    }
  }
  return at + n;
}

__device__ int xform_row(const XformArgs& a, int64_t o, unsigned char* d, bool& valid) {
  if (a.kind == StringOp::TO_STRING) return format_value(a, o, d, valid);
  if (is_segment_kind(a)) {
    const unsigned char *p1, *p2;
    int n1;
    const int len = xform_segments(a, o, p1, n1, p2, valid);
    if (d) {
      put(d, 0, p1, n1);
      put(d, n1, p2, len - n1);
    }
    return len;
  }
  if (a.kind == StringOp::CONCAT) {  // more than two parts or a formatted part, NULL if any is
    int at = 0;
#pragma unroll
    for (int k = 0; k < kMaxConcatParts; k++) {  // unrolled: the parts stay in parameter space
      if (k >= 2 + a.nmore) break;
      const BuildSrc& ps = k == 0 ? a.a : k == 1 ? a.b : a.more[k >= 2 ? k - 2 : 0];
      if (ps.kind == StrSource::FORMAT) {  // CAST(column):VARCHAR in place
        at += format_typed(ps.num, ps.mask, ps.off, ps.num_type, o, d ? d + at : nullptr, valid);
        if (!valid) return 0;
        continue;
      }
      const unsigned char* q;
      int m;
      source_row(ps, o, q, m, valid);
      if (!valid) return 0;
      at = put(d, at, q, m);
    }
    return at;
  }
  const unsigned char* p;
  int n;
  source_row(a.a, o, p, n, valid);
  if (!valid) return 0;
  switch (a.kind) {
    case StringOp::SLICE: {  // a negative step: the whole string, characters in reverse order
      int at = 0, e = n;
      while (e > 0) {
        int b = e - 1;
        while (b > 0 && (p[b] & 0xC0) == 0x80) b--;
        if (d)
          for (int i = b; i < e; i++) d[at + i - b] = p[i];
        at += e - b;
        e = b;
      }
      return at;
    }
    case StringOp::UPPER: case StringOp::LOWER: case StringOp::INITCAP: {
      // per code point (cudf::strings::to_upper / to_lower / title): INITCAP
      // maps the first alphabetic character of each run of them to upper
      // case and the rest to lower case
      bool word = false;
      int at = 0;
      for (int i = 0; i < n;) {
        const unsigned char b = p[i];
        if (b < 0x80) {  // ASCII
          unsigned char c = b;
          const bool up = c >= 'A' && c <= 'Z', lo = c >= 'a' && c <= 'z';
          const bool to_up = a.kind == StringOp::INITCAP ? !word : a.kind == StringOp::UPPER;
          if (to_up && lo) c = (unsigned char)(c - 32);
          if (!to_up && up) c = (unsigned char)(c + 32);
          word = up || lo;
          if (d) d[at] = c;
          at++;
          i++;
          continue;
        }
        int len = utf8_len(b);
        bool ok = len > 1 && i + len <= n;
        uint32_t c = len == 2 ? (b & 0x1Fu) : len == 3 ? (b & 0x0Fu) : (b & 0x07u);
        for (int k = 1; ok && k < len; k++) {
          ok = (p[i + k] & 0xC0) == 0x80;
          c = (c << 6) | (p[i + k] & 0x3Fu);
        }
        if (!ok) {  // not a UTF-8 sequence: the byte as it is
          if (d) d[at] = b;
          at++;
          i++;
          word = false;
          continue;
        }
        bool to_up = a.kind == StringOp::UPPER, map = true;
        if (a.kind == StringOp::INITCAP) {
          const bool alpha = is_alpha_cp(c);
          to_up = !word;
          map = alpha;
          word = alpha;
        }
        uint32_t m[3] = {c, 0, 0};
        const int k = map ? case_map(c, to_up, m) : 1;
        for (int j = 0; j < k; j++) at = put_utf8(d, at, m[j]);
        i += len;
      }
      return at;
    }
    case StringOp::REPLACE: {  // cudf::strings::replace, every occurrence, left to right
      int at = 0, i = 0;
      while (i < n) {
        bool hit = i + a.l1 <= n;
        for (int t = 0; hit && t < a.l1; t++) hit = p[i + t] == a.s1[t];
        if (hit) {
          at = put(d, at, a.s2, a.l2);
          i += a.l1;
        } else {
          if (d) d[at] = p[i];
          at++;
          i++;
        }
      }
      return at;
    }
    default: return 0;
  }
}

// kRegex: REGEXP_REPLACE rows (a separate instantiation keeps the Pike VM's
// thread lists out of the other transforms' local memory)
template <bool kRegex>
__global__ void __launch_bounds__(kBuildWarps * 32) k_xf_sizes(XformArgs a) {
  __shared__ uint64_t s_sum[kBuildWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = ((int64_t)blockIdx.x * kBuildWarps + warp) * kBuildWords;
  uint64_t total = 0;
  for (int k = 0; k < kBuildWords; k++) {
    const int64_t o = (w0 + k) * 32 + lane;
    if ((w0 + k) * 32 >= a.m) break;
    const int64_t src = (o < a.m && a.map) ? (int64_t)a.map[o] : o;  // the input row
    bool valid = false;
    int len = 0;
    if (o < a.m) {
      if constexpr (kRegex) len = regex_row(a, src, nullptr, valid);
      else len = xform_row(a, src, nullptr, valid);
      a.out_offs[o] = len;  // the row's length, read back by k_xf_write (which then writes offsets)
    }
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

template <bool kRegex>
__global__ void __launch_bounds__(kBuildWarps * 32) k_xf_write(XformArgs a) {
  __shared__ uint64_t s_sum[kBuildWarps];
  __shared__ __align__(16) unsigned char s_stage[kBuildWarps][kStageBytes + 8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = ((int64_t)blockIdx.x * kBuildWarps + warp) * kBuildWords;
  uint64_t total = 0;
  for (int k = 0; k < kBuildWords; k++) {
    const int64_t o = (w0 + k) * 32 + lane;
    if ((w0 + k) * 32 >= a.m) break;
    const int len = o < a.m ? a.out_offs[o] : 0;  // k_xf_sizes' row lengths
    total += (uint64_t)warp_sum(len);
  }
  if (lane == 0) s_sum[warp] = total;
  __syncthreads();
  uint64_t pos = a.block_sums[blockIdx.x];
  for (int i = 0; i < warp; i++) pos += s_sum[i];
  for (int k = 0; k < kBuildWords; k++) {
    const int64_t o = (w0 + k) * 32 + lane;
    if ((w0 + k) * 32 >= a.m) break;
    const int64_t src = (o < a.m && a.map) ? (int64_t)a.map[o] : o;  // the input row
    const bool seg = !kRegex && is_segment_kind(a);  // warp-uniform
    const unsigned char *p1 = nullptr, *p2 = nullptr;
    int n1 = 0, len = 0;
    bool valid = false;
    if (o < a.m) {
      if (seg) len = xform_segments(a, src, p1, n1, p2, valid);
      else len = a.out_offs[o];  // k_xf_sizes' row length
    }
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
    const int wtot = __shfl_sync(0xffffffffu, incl, 31);
    if (seg && wtot > 32 * kWarpCopyBytes) {  // long rows: the warp copies them together
      warp_copy(a.out_chars + pos, incl - len, n1, p1, p2, wtot, lane);
    } else if (seg) {  // short rows: staged by their lanes, written out by the warp
      unsigned char* st = s_stage[warp] + (pos & 3u) + (incl - len);
      for (int i = 0; i < n1; i++) st[i] = p1[i];
      for (int i = n1; i < len; i++) st[i] = p2[i - n1];
      __syncwarp();
      stage_flush(a.out_chars, pos, s_stage[warp], wtot, lane);
      __syncwarp();
    } else if (o < a.m && len > 0) {
      if constexpr (kRegex) regex_row(a, src, a.out_chars + dst, valid);
      else xform_row(a, src, a.out_chars + dst, valid);
    }
    pos += (uint64_t)wtot;
  }
}

// string -> integer / floating point / DATE / TIMESTAMP (cudf::strings::to_integers, to_floats and
// to_timestamps with "%Y-%m-%d" / "%Y-%m-%d %H:%M:%S", LogicalProject.cpp:379-528)
constexpr int kMaxFormatItems = 32;
struct ParseArgs {
  BuildSrc a;
  int type;
  int64_t m;
  void* out;
  uint32_t* out_mask;
  // DATE / TIMESTAMP: the format's items in order, each a field (index into
  // Y m d H M S) or a literal (-1), and its width in bytes
  int nitems;
  signed char field[kMaxFormatItems];
  unsigned char width[kMaxFormatItems];
};

// digits from s[0..n) up to the first non-digit
__device__ __forceinline__ int64_t leading_digits(const unsigned char* s, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; i++) {
    if (s[i] < '0' || s[i] > '9') break;
    v = v * 10 + (uint64_t)(s[i] - '0');
  }
  return (int64_t)v;
}

// days since 1970-01-01 of (y, m, d): H. Hinnant's days_from_civil
__device__ int64_t days_from_civil(int64_t y, int64_t m, int64_t d) {
  y -= m <= 2;
  const int64_t era = (y >= 0 ? y : y - 399) / 400;
  const int64_t yoe = y - era * 400;
  const int64_t doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
  const int64_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 719468;
}

// A string as cudf::strings::to_floats reads it: an optional sign, then NaN,
// Inf, or digits with one optional decimal point and an optional e / E
// exponent.  Up to 19 significant digits are accumulated into an integer
// (later ones only move the decimal exponent), which is then scaled by exact
// powers of ten -- multiplied for a positive exponent, divided for a negative
// one, in steps of 1e22 -- each step one correctly rounded operation, so
// values of up to 15 digits with |exponent| <= 22 convert exactly rounded.
// Reading stops at the first other character (no digits: 0).
__device__ double parse_double(const unsigned char* p, int n) {
  int i = 0;
  bool neg = false;
  if (i < n && (p[i] == '+' || p[i] == '-')) {
    neg = p[i] == '-';
    i++;
  }
  if (i + 3 <= n && p[i] == 'N' && p[i + 1] == 'a' && p[i + 2] == 'N') return __longlong_as_double(0x7ff8000000000000ll);
  if (i + 3 <= n && p[i] == 'I' && p[i + 1] == 'n' && p[i + 2] == 'f')
    return __longlong_as_double(neg ? (long long)0xfff0000000000000ull : 0x7ff0000000000000ll);
  uint64_t mant = 0;
  int digits = 0, exp10 = 0;
  bool dot = false;
  for (; i < n; i++) {
    const unsigned char c = p[i];
    if (c == '.' && !dot) {
      dot = true;
    } else if (c >= '0' && c <= '9') {
      if (digits < 19) {
        mant = mant * 10 + (c - '0');
        if (mant) digits++;
        if (dot) exp10--;
      } else if (!dot) {
        exp10++;
      }
    } else {
      break;
    }
  }
  if (i < n && (p[i] == 'e' || p[i] == 'E')) {
    int j = i + 1, e = 0;
    bool eneg = false;
    if (j < n && (p[j] == '+' || p[j] == '-')) {
      eneg = p[j] == '-';
      j++;
    }
    for (; j < n && p[j] >= '0' && p[j] <= '9'; j++) e = min(e * 10 + (p[j] - '0'), 100000);
    exp10 += eneg ? -e : e;
  }
  // 1e0 .. 1e22: every one exact in binary64
  const double pow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                            1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
  double x = __ull2double_rn(mant);
  if (exp10 >= 0) {
    for (; exp10 > 22; exp10 -= 22) x = __dmul_rn(x, 1e22);
    x = __dmul_rn(x, pow10[exp10]);
  } else {
    int e = -exp10;
    for (; e > 22; e -= 22) x = __ddiv_rn(x, 1e22);
    x = __ddiv_rn(x, pow10[e]);
  }
  return neg ? -x : x;
}

__global__ void k_parse(ParseArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t nwords = (a.m + 31) / 32;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; w < nwords;
       w += ((int64_t)gridDim.x * blockDim.x) / 32) {
    const int64_t r = w * 32 + lane;
    bool valid = false;
    if (r < a.m) {
      const unsigned char* p;
      int n;
      source_row(a.a, r, p, n, valid);
      int64_t v = 0;
      double fv = 0.0;
      if (valid && (a.type == FLOAT32 || a.type == FLOAT64)) {
        fv = parse_double(p, n);
      } else if (valid && (a.type == TIMESTAMP_DAYS || a.type == TIMESTAMP_SECONDS || a.type == TIMESTAMP_MILLISECONDS ||
                    a.type == TIMESTAMP_MICROSECONDS || a.type == TIMESTAMP_NANOSECONDS)) {
        // the format's items in order, each taking its width (less at the end of
        // the string); a field reads its digits up to the first non-digit
        int64_t f[6] = {0, 0, 0, 0, 0, 0};
        int at = 0;
        for (int k = 0; k < a.nitems; k++) {
          const int w = max(0, min((int)a.width[k], n - at));
          if (a.field[k] >= 0) f[a.field[k]] = leading_digits(p + at, w);
          at += w;
        }
        const int64_t days = days_from_civil(f[0], f[1], f[2]);
        if (a.type == TIMESTAMP_DAYS) {
          v = days;
        } else {
          const int64_t secs = days * 86400 + f[3] * 3600 + f[4] * 60 + f[5];
          const int64_t per = a.type == TIMESTAMP_SECONDS ? 1 : a.type == TIMESTAMP_MILLISECONDS ? 1000
                            : a.type == TIMESTAMP_MICROSECONDS ? 1000000 : 1000000000;
          v = secs * per;
        }
      } else if (valid && n > 0) {
        int i = 0;
        bool neg = false;
        if (p[0] == '-' || p[0] == '+') {
          neg = p[0] == '-';
          i = 1;
        }
        const uint64_t u = (uint64_t)leading_digits(p + i, n - i);
        v = (int64_t)(neg ? 0 - u : u);
      }
      switch (a.type) {
        case INT8: ((int8_t*)a.out)[r] = (int8_t)v; break;
        case INT16: ((int16_t*)a.out)[r] = (int16_t)v; break;
        case INT32: case TIMESTAMP_DAYS: ((int32_t*)a.out)[r] = (int32_t)v; break;
        case FLOAT32: ((float*)a.out)[r] = __double2float_rn(fv); break;
        case FLOAT64: ((double*)a.out)[r] = fv; break;
        default: ((int64_t*)a.out)[r] = v; break;
      }
    }
    const uint32_t word = __ballot_sync(0xffffffffu, r < a.m && valid);
    if (lane == 0) a.out_mask[w] = word;
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
    b.end = s.col.offset + s.col.size;
  } else if (s.kind == StrSource::LITERAL) {
    b.lit = lit_dev;
    b.lit_len = (int32_t)s.literal.size();
  } else if (s.kind == StrSource::FORMAT) {
    if (s.col.type == STRING || type_size(s.col.type) == 0 || s.col.type >= DURATION_DAYS)
      fail(GX_ERR_UNSUPPORTED, "CAST to VARCHAR of type " + std::to_string(s.col.type));
    b.num = s.col.data;
    b.mask = s.col.mask;
    b.off = s.col.offset;
    b.num_type = s.col.type;
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

gx_column build_transform(const StringOp& op, const StrSource& a, const StrSource& b, const ColumnView* num,
                          int64_t rows, cudaStream_t s, const std::vector<StrSource>& more,
                          const ColumnView* pos0 = nullptr, const ColumnView* pos1 = nullptr,
                          const int32_t* map = nullptr) {
  if (more.size() > (size_t)(kMaxConcatParts - 2)) fail(GX_ERR_INVALID, "too many CONCAT parts");
  if (rows < 0 || rows > INT32_MAX) fail(GX_ERR_UNSUPPORTED, "string columns hold at most 2^31 - 1 rows");
  const int64_t nblocks = (rows + kBuildRows - 1) / kBuildRows;
  const int64_t words = mask_words_for(rows);
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  // [mask | offsets | block sums + total | a, b, literal, literal2]
  const size_t mask_b = al((size_t)words * 4), offs_b = al((size_t)(rows + 1) * 4);
  const size_t sums_b = al((size_t)(nblocks + 1) * 8);
  std::vector<std::string> lits = {a.kind == StrSource::LITERAL ? a.literal : std::string(),
                                   b.kind == StrSource::LITERAL ? b.literal : std::string(), op.literal,
                                   op.literal2};
  for (const auto& x : more) lits.push_back(x.kind == StrSource::LITERAL ? x.literal : std::string());
  const int nl = (int)lits.size();
  std::vector<size_t> loff(nl);
  size_t lb = 0;
  for (int i = 0; i < nl; i++) {
    loff[i] = lb;
    lb += al(lits[i].size() + 1);
  }
  char* base = (char*)dev_alloc(mask_b + offs_b + sums_b + lb, s);
  gx_column out{};
  out.type_id = STRING;
  out.null_mask = (uint32_t*)base;
  out.string_offsets = (int32_t*)(base + mask_b);
  out.size = rows;
  out.capacity = rows;
  try {
    uint64_t* sums = (uint64_t*)(base + mask_b + offs_b);
    unsigned char* ldev = (unsigned char*)(base + mask_b + offs_b + sums_b);
    check_cuda(cudaMemsetAsync(base, 0, mask_b + offs_b + sums_b, s), "string column clear");
    for (int i = 0; i < nl; i++)
      if (!lits[i].empty())
        check_cuda(cudaMemcpyAsync(ldev + loff[i], lits[i].data(), lits[i].size(), cudaMemcpyHostToDevice, s),
                   "string literal");
    XformArgs x{};
    x.kind = op.kind;
    x.a = device_source(a, ldev + loff[0]);
    x.b = device_source(b, ldev + loff[1]);
    x.nmore = (int)more.size();
    for (size_t k = 0; k < more.size(); k++) x.more[k] = device_source(more[k], ldev + loff[4 + k]);
    if (num) {
      x.num = num->data;
      x.num_mask = num->mask;
      x.num_off = num->offset;
      x.num_type = num->type;
    }
    if (pos0) {
      x.p0 = pos0->data;
      x.p0m = pos0->mask;
      x.p0t = pos0->type;
    }
    if (pos1) {
      x.p1 = pos1->data;
      x.p1m = pos1->mask;
      x.p1t = pos1->type;
    }
    x.i0 = op.i0;
    x.i1 = op.i1;
    x.step = op.step;
    x.i0v = op.i0_valid;
    x.i1v = op.i1_valid;
    x.s1 = ldev + loff[2];
    x.l1 = (int)op.literal.size();
    x.s2 = ldev + loff[3];
    x.l2 = (int)op.literal2.size();
    x.m = rows;
    x.map = map;
    x.out_offs = out.string_offsets;
    x.out_mask = out.null_mask;
    x.block_sums = sums;
    uint64_t host[1] = {0};
    if (rows > 0) {
      if (op.kind == StringOp::REGEXP_REPLACE) k_xf_sizes<true><<<(unsigned)nblocks, kBuildWarps * 32, 0, s>>>(x);
      else k_xf_sizes<false><<<(unsigned)nblocks, kBuildWarps * 32, 0, s>>>(x);
      check_cuda(cudaGetLastError(), "k_xf_sizes");
      launch_scan_tiles(sums, nblocks, (unsigned long long*)(sums + nblocks), s);
      check_cuda(cudaMemcpyAsync(host, sums + nblocks, 8, cudaMemcpyDeviceToHost, s), "string size");
      add_launches(1);
    }
    check_cuda(cudaStreamSynchronize(s), "string size sync");
    const uint64_t total = host[0];
    if (total > (uint64_t)INT32_MAX) fail(GX_ERR_UNSUPPORTED, "string column over 2^31 - 1 characters");
    out.data = dev_alloc(al(total ? total : 1), s);
    out.string_bytes = (int64_t)total;
    if (rows > 0) {
      x.out_chars = (unsigned char*)out.data;
      if (op.kind == StringOp::REGEXP_REPLACE) k_xf_write<true><<<(unsigned)nblocks, kBuildWarps * 32, 0, s>>>(x);
      else k_xf_write<false><<<(unsigned)nblocks, kBuildWarps * 32, 0, s>>>(x);
      check_cuda(cudaGetLastError(), "k_xf_write");
      add_launches(1);
    }
  } catch (...) {
    if (out.data) dev_free(out.data, s);
    dev_free(base, s);
    throw;
  }
  return out;
}

void launch_parse(const ColumnView& col, int type, const std::string& format, gx_column& out, cudaStream_t s) {
  ParseArgs a{};
  // cudf::strings::to_timestamps' items: %Y 4 bytes, %m %d %H %M %S 2, any
  // other character (and %%) 1
  for (size_t i = 0; i < format.size(); i++) {
    if (a.nitems == kMaxFormatItems) fail(GX_ERR_UNSUPPORTED, "timestamp format too long: " + format);
    int field = -1, width = 1;
    if (format[i] == '%' && i + 1 < format.size()) {
      const char c = format[++i];
      static const char* kFields = "YmdHMS";
      const char* at = c == '%' ? nullptr : std::strchr(kFields, c);
      if (c != '%' && !at) fail(GX_ERR_UNSUPPORTED, std::string("timestamp format specifier %") + c);
      if (at) {
        field = (int)(at - kFields);
        width = c == 'Y' ? 4 : 2;
      }
    }
    a.field[a.nitems] = (signed char)field;
    a.width[a.nitems] = (unsigned char)width;
    a.nitems++;
  }
  StrSource src;
  src.kind = StrSource::COLUMN;
  src.col = col;
  a.a = device_source(src, nullptr);
  a.type = type;
  a.m = col.size;
  a.out = out.data;
  a.out_mask = out.null_mask;
  if (a.m == 0) return;
  const int64_t warps = (a.m + 31) / 32;
  const int grid = (int)std::min<int64_t>((warps + 7) / 8, 152 * 32);
  k_parse<<<grid, 256, 0, s>>>(a);
  check_cuda(cudaGetLastError(), "k_parse");
  add_launches(1);
}

// ----------------------------------------------------------- LIKE automaton
// The LIKE pattern's regular expression (see like_match) as a byte automaton
// for the search: an NFA over the pattern's middle (between its leading and
// trailing '%' runs) whose states are (token k, continuation bytes still due
// for a '_' character), a new start after every byte when the pattern starts
// with '%', made deterministic by subset construction, with an absorbing
// accept state when it ends with '%'.  Bytes that behave alike share a class.
// False (the matcher is used) for a middle over 15 bytes or over 128 states.
struct LikeDfa {
  int states = 0, classes = 0, start = 0;
  // classes > 0: [class of each byte 256 | flags per state | transitions states x classes];
  // direct (classes == 0, at most kDirectStates states): [transitions states x 256
  // bytes, each the next state with bit 7 set when that state is absorbing |
  // flags per state] -- one table read per byte, no class lookup
  std::string blob;
};
constexpr int kDirectStates = 64;

static int host_utf8_len(unsigned char c) {
  return c < 0x80 ? 1 : (c >> 5) == 0x6 ? 2 : (c >> 4) == 0xE ? 3 : (c >> 3) == 0x1E ? 4 : 1;
}

static bool build_like_dfa(const std::string& pat, LikeDfa& d) {
  const int m = (int)pat.size();
  int lead = 0;
  while (lead < m && pat[lead] == '%') lead++;
  if (lead == m) return false;  // every string matches: the matcher answers at once
  int tail = m;
  while (tail > lead && pat[tail - 1] == '%') tail--;
  const std::string tok = pat.substr(lead, tail - lead);
  const int M = (int)tok.size();
  if (M > 15) return false;
  const bool anchored_start = lead == 0, anchored_end = tail == m;
  auto bit = [](int k, int c) { return 1ull << (k * 4 + c); };
  auto closure = [&](uint64_t x) {
    for (int k = 0; k < M; k++)
      if ((x & bit(k, 0)) && tok[k] == '%') x |= bit(k + 1, 0);
    return x;
  };
  const uint64_t start = closure(bit(0, 0)), acc = bit(M, 0);
  const uint64_t kAccept = ~0ull;  // the absorbing accept state of a pattern ending with '%'
  auto step = [&](uint64_t S, unsigned char b) {
    uint64_t nx = 0;
    for (int k = 0; k < M; k++)
      for (int c = 0; c < 4; c++) {
        if (!(S & bit(k, c))) continue;
        if (c > 0) {  // inside a '_' character
          if ((b & 0xC0) == 0x80) nx |= c > 1 ? bit(k, c - 1) : bit(k + 1, 0);
          continue;
        }
        const unsigned char t = (unsigned char)tok[k];
        if (t == '%') {
          if (b != '\n') nx |= bit(k, 0);
        } else if (t == '_') {
          if (b == '\n' || (b & 0xC0) == 0x80) continue;
          const int L = host_utf8_len(b);
          nx |= L == 1 ? bit(k + 1, 0) : bit(k, L - 1);
        } else if (b == t) {
          nx |= bit(k + 1, 0);
        }
      }
    nx = closure(nx);
    if (!anchored_start) nx |= start;
    return nx;
  };
  std::map<uint64_t, int> id;
  std::vector<uint64_t> sets;
  auto sid = [&](uint64_t S) {
    if (!anchored_end && (S & acc)) S = kAccept;
    auto it = id.find(S);
    if (it != id.end()) return it->second;
    id[S] = (int)sets.size();
    sets.push_back(S);
    return (int)sets.size() - 1;
  };
  d.start = sid(start);
  std::vector<std::array<int, 256>> tr;
  for (size_t i = 0; i < sets.size(); i++) {
    if (sets.size() > 128) return false;
    std::array<int, 256> row{};
    for (int b = 0; b < 256; b++) row[b] = sets[i] == kAccept ? (int)i : sid(step(sets[i], (unsigned char)b));
    tr.push_back(row);
  }
  if (sets.size() > 128) return false;
  d.states = (int)sets.size();
  // byte classes: bytes whose transitions agree in every state
  std::map<std::vector<int>, int> cls_of;
  std::vector<int> cls(256);
  for (int b = 0; b < 256; b++) {
    std::vector<int> col(d.states);
    for (int i = 0; i < d.states; i++) col[i] = tr[i][b];
    auto it = cls_of.find(col);
    if (it == cls_of.end()) it = cls_of.emplace(col, (int)cls_of.size()).first;
    cls[b] = it->second;
  }
  d.classes = (int)cls_of.size();
  d.blob.assign(256 + d.states * (1 + d.classes), '\0');
  for (int b = 0; b < 256; b++) d.blob[b] = (char)cls[b];
  for (int i = 0; i < d.states; i++) {
    const uint64_t S = sets[i];
    const bool accept = S == kAccept || (S & acc);
    const bool absorbing = S == kAccept || (S == 0 && anchored_start);
    d.blob[256 + i] = (char)((accept ? 1 : 0) | (absorbing ? 2 : 0));
  }
  for (int b = 0; b < 256; b++)
    for (int i = 0; i < d.states; i++) d.blob[256 + d.states + i * d.classes + cls[b]] = (char)tr[i][b];
  if (d.states <= kDirectStates) {  // byte-indexed form
    std::string direct((size_t)d.states * 256 + d.states, '\0');
    for (int i = 0; i < d.states; i++) {
      for (int b = 0; b < 256; b++) {
        const int nx = tr[i][b];
        const bool absorbing = (d.blob[256 + nx] & 2) != 0;
        direct[(size_t)i * 256 + b] = (char)(nx | (absorbing ? 0x80 : 0));
      }
      direct[(size_t)d.states * 256 + i] = d.blob[256 + i];
    }
    d.blob = direct;
    d.classes = 0;
  }
  return true;
}

int like_dfa_host_match(const std::string& pattern, const unsigned char* text, int64_t n) {
  LikeDfa d;
  if (!build_like_dfa(pattern, d)) return -1;
  // the same walk as k_string_op's
  if (d.classes == 0) {  // byte-indexed
    const unsigned char* tr = (const unsigned char*)d.blob.data();
    const unsigned char* flags = tr + (size_t)d.states * 256;
    unsigned st = (unsigned)d.start | ((flags[d.start] & 2) ? 0x80u : 0u);
    for (int64_t i = 0; i < n && !(st & 0x80u); i++) st = tr[((st & 0x7Fu) << 8) | text[i]];
    return flags[st & 0x7Fu] & 1;
  }
  const unsigned char* cls = (const unsigned char*)d.blob.data();
  const unsigned char* flags = cls + 256;
  const unsigned char* tr = flags + d.states;
  int st = d.start;
  for (int64_t i = 0; i < n; i++) {
    st = tr[st * d.classes + cls[text[i]]];
    if (flags[st] & 2) break;
  }
  return flags[st] & 1;
}

void launch_string_op(const ColumnView& col, const ColumnView* col2, const StringOp& op, const void* pattern_dev,
                      gx_column& out, cudaStream_t s, const LikeDfa* dfa) {
  StrArgs a{};
  size_t smem = 0;
  if (dfa) {  // pattern_dev holds the automaton
    a.dfa = (const unsigned char*)pattern_dev;
    a.dfa_states = dfa->states;
    a.dfa_classes = dfa->classes;
    a.dfa_start = dfa->start;
    smem = dfa->blob.size();
  }
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
  k_string_op<<<grid, 256, smem, s>>>(a);
  check_cuda(cudaGetLastError(), "k_string_op");
  add_launches(1);
}

// column c of cols, which a string operator reads as a string column
static ColumnView string_column(const std::vector<ColumnView>& cols, int c) {
  const ColumnView v = cols.at(c);
  if (v.type != STRING) fail(GX_ERR_TYPE, "string operator over a non-string column");
  return v;
}

bool is_deferrable(const StringOp& op) {
  switch (op.kind) {
    case StringOp::TO_STRING: case StringOp::SLICE: case StringOp::UPPER: case StringOp::LOWER:
    case StringOp::INITCAP: case StringOp::TRIM: case StringOp::REPLACE: case StringOp::CONCAT:
    case StringOp::REGEXP_REPLACE:
      return true;
    default:
      return false;
  }
}

gx_column transform_column(const StringOp& op, const std::vector<ColumnView>& cols, const int32_t* map,
                           int64_t rows, cudaStream_t s, const EvalText& eval_bool) {
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  auto string_col = [&](int c) { return string_column(cols, c); };
  gx_column out{};
  if (op.kind == StringOp::TO_STRING) {
    gx_column tmp{};
    ColumnView v = op.col >= 0 ? cols.at(op.col) : ColumnView{};
    if (op.col < 0) {
      tmp = eval_bool(cols, op.cond);
      v = ColumnView{tmp.type_id, tmp.data, tmp.null_mask, 0, n, tmp.string_offsets};
    }
    try {
      if (v.type == STRING) {
        StrSource a, none;
        a.kind = StrSource::COLUMN;
        a.col = v;
        out = build_strings(a, none, map, nullptr, rows, s);
      } else {
        if (type_size(v.type) == 0 || v.type >= DURATION_DAYS)
          fail(GX_ERR_UNSUPPORTED, "CAST to VARCHAR of type " + std::to_string(v.type));
        out = build_transform(op, StrSource{}, StrSource{}, &v, rows, s, {}, nullptr, nullptr, map);
      }
    } catch (...) {
      if (tmp.data || tmp.null_mask) free_column(tmp, s);
      throw;
    }
    if (tmp.data || tmp.null_mask) free_column(tmp, s);
    return out;
  }
  // a part: a string column, a literal, or (CONCAT) a typed column to format
  auto part = [&](int c, const std::string& lit) {
    StrSource x;
    if (c < 0) {
      x.kind = StrSource::LITERAL;
      x.literal = lit;
    } else if (op.kind == StringOp::CONCAT && cols.at(c).type != STRING) {
      x.kind = StrSource::FORMAT;
      x.col = cols.at(c);
    } else {
      x.kind = StrSource::COLUMN;
      x.col = string_col(c);
    }
    return x;
  };
  StrSource a = part(op.col, op.literal), b;
  if (op.kind == StringOp::CONCAT) b = part(op.col2, op.literal2);
  std::vector<StrSource> more;
  for (size_t k = 0; k < op.more_cols.size(); k++) more.push_back(part(op.more_cols[k], op.more_lits[k]));
  StringOp xo = op;
  if (op.kind == StringOp::CONCAT) xo.literal.clear(), xo.literal2.clear();
  if (op.kind == StringOp::REGEXP_REPLACE) compile_regex_replace(op.literal, op.literal2, &xo.literal, &xo.literal2);
  if (op.kind == StringOp::SLICE && !op.pos0.empty()) {
    // the start and stop columns (LogicalProject.cpp:241-300), made by
    // the same evaluator as a CASE condition over every input row
    gx_column pc[2] = {};
    auto release = [&] {
      for (auto& c : pc)
        if (c.data || c.null_mask) free_column(c, s);
    };
    try {
      ColumnView pv[2];
      for (int k = 0; k < 2; k++) {
        const std::string& text = k == 0 ? op.pos0 : op.pos1;
        if (text.empty()) continue;
        pc[k] = eval_bool(cols, text);
        const int t = pc[k].type_id;
        if (t != INT8 && t != INT16 && t != INT32 && t != INT64 && t != UINT8 && t != UINT16 && t != UINT32 &&
            t != UINT64)
          fail(GX_ERR_TYPE, "Expression does not evaluate to an integer column");  // :252
        pv[k] = ColumnView{t, pc[k].data, pc[k].null_mask, 0, n};
      }
      out = build_transform(xo, a, b, nullptr, rows, s, more, &pv[0], op.pos1.empty() ? nullptr : &pv[1], map);
    } catch (...) {
      release();
      throw;
    }
    release();
    return out;
  }
  return build_transform(xo, a, b, nullptr, rows, s, more, nullptr, nullptr, map);
}

std::vector<gx_column> run_string_prepass(std::vector<ColumnView>& cols, const std::vector<StringOp>& ops,
                                          cudaStream_t s, const EvalText& eval_bool,
                                          const std::vector<bool>* defer) {
  std::vector<gx_column> made;
  if (ops.empty()) return made;
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  // each operator's device bytes: its literal, or a LIKE pattern's automaton
  std::vector<LikeDfa> dfas(ops.size());
  std::vector<const std::string*> bytes(ops.size());
  for (size_t i = 0; i < ops.size(); i++) {
    bytes[i] = &ops[i].literal;
    if (ops[i].kind == StringOp::LIKE && ops[i].col2 < 0 && build_like_dfa(ops[i].literal, dfas[i]))
      bytes[i] = &dfas[i].blob;
  }
  size_t pbytes = 0;
  // a 16-byte aligned slot of 16 bytes or more per operator
  auto slot = [](size_t len) { return (std::max<size_t>(len, 1) + 15) / 16 * 16; };
  for (const auto* b : bytes) pbytes += slot(b->size());
  std::string host(std::max<size_t>(pbytes, 16), '\0');
  std::vector<size_t> poff;
  size_t at = 0;
  for (const auto* b : bytes) {
    poff.push_back(at);
    std::memcpy(&host[at], b->data(), b->size());
    at += slot(b->size());
  }
  char* pdev = (char*)dev_alloc(host.size(), s);
  auto string_col = [&](int c) { return string_column(cols, c); };
  try {
    check_cuda(cudaMemcpyAsync(pdev, host.data(), host.size(), cudaMemcpyHostToDevice, s), "string patterns");
    for (size_t i = 0; i < ops.size(); i++) {
      const StringOp& op = ops[i];
      gx_column out{};
      if (defer && i < defer->size() && (*defer)[i]) {
        // made later over the kept rows only (transform_column with a row
        // map); nothing before the plan reads it
        made.push_back(out);
        cols.push_back(ColumnView{STRING, nullptr, nullptr, 0, n, nullptr});
        continue;
      }
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
      } else if (is_deferrable(op)) {
        out = transform_column(op, cols, nullptr, n, s, eval_bool);
      } else if (op.kind == StringOp::PARSE) {
        const ColumnView c = string_col(op.col);
        out = alloc_column(op.type, n, s);
        launch_parse(c, op.type, op.literal, out, s);
      } else {
        const ColumnView c = string_col(op.col);  // a copy: cols grows below
        ColumnView c2{};
        if (op.col2 >= 0) c2 = string_col(op.col2);
        out = alloc_column(op.result_type(), n, s);
        launch_string_op(c, op.col2 >= 0 ? &c2 : nullptr, op, pdev + poff[i], out, s,
                         dfas[i].states ? &dfas[i] : nullptr);
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
