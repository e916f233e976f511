// regex_vm.h -- the REGEXP_REPLACE matcher: a Pike VM over the program that
// compile_regex_replace (regex.cpp) makes, one subject row per call.  The
// string pre-pass runs it per row on the device; the functions are also
// host-callable so that a host test can drive the same code.
//
// The threads of one subject position are kept in priority order, each a
// program counter with its capture slots; a state already taken by a
// higher-priority thread at the same position is not taken again, and a
// MATCH drops the threads below it.  The match found is therefore the
// leftmost-first one: the one a backtracking matcher that tries alternatives
// and repeats in order would report.
#pragma once

#include <cstdint>

#include "regex.h"

#ifdef __CUDACC__
#define GX_RE_FN __host__ __device__ __forceinline__
#else
#define GX_RE_FN inline
#endif

namespace gx {

struct ReList {
  int n;
  uint8_t pc[kReMaxInst];
  int32_t cap[kReMaxInst * kReMaxSlots];
};

struct ReVm {
  const ReInst* prog;
  const ReRange* ranges;
  int nslots;
  const unsigned char* p;
  int from, n;  // the subject is p[from, n)
  uint32_t gen;
  uint32_t mark[kReMaxInst];
  int32_t stk[kReMaxInst + 1][2];  // a pc to explore, or (-slot - 1, value) to restore
};

GX_RE_FN int re_utf8_len(unsigned char c) {
  return c < 0x80 ? 1 : (c >> 5) == 0x6 ? 2 : (c >> 4) == 0xE ? 3 : (c >> 3) == 0x1E ? 4 : 1;
}

GX_RE_FN bool re_word(unsigned char c) {
  return (c >= '0' && c <= '9') || (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || c == '_';
}

// Adds the threads that pc0 reaches without consuming a character at byte i
// to l, in priority order (a SPLIT's x before its y).  caps is restored on
// return.  Every instruction is entered at most once per position (mark), so
// the stack holds at most one entry per instruction plus the first.
GX_RE_FN void re_add(ReVm& vm, ReList& l, int pc0, int32_t* caps, int i) {
  int sp = 0;
  vm.stk[sp++][0] = pc0;
  while (sp > 0) {
    --sp;
    const int e = vm.stk[sp][0];
    if (e < 0) {
      caps[-e - 1] = vm.stk[sp][1];
      continue;
    }
    int pc = e;
    for (;;) {
      if (vm.mark[pc] == vm.gen) break;
      vm.mark[pc] = vm.gen;
      const ReInst in = vm.prog[pc];
      if (in.op == RE_JMP) {
        pc = in.x;
      } else if (in.op == RE_SPLIT) {
        vm.stk[sp++][0] = in.y;
        pc = in.x;
      } else if (in.op == RE_SAVE) {
        if (in.x < vm.nslots) {
          vm.stk[sp][0] = -(int)in.x - 1;
          vm.stk[sp++][1] = caps[in.x];
          caps[in.x] = i;
        }
        pc++;
      } else if (in.op == RE_BOL || in.op == RE_EOL || in.op == RE_WORDB || in.op == RE_NWORDB) {
        bool ok;
        if (in.op == RE_BOL) ok = i == vm.from;
        else if (in.op == RE_EOL) ok = i == vm.n;
        else ok = ((i > vm.from && re_word(vm.p[i - 1])) != (i < vm.n && re_word(vm.p[i]))) == (in.op == RE_WORDB);
        if (!ok) break;
        pc++;
      } else {  // CHAR, ANY, CLASS, MATCH: a thread of the list
        const int k = l.n++;
        l.pc[k] = (uint8_t)pc;
        for (int t = 0; t < vm.nslots; t++) l.cap[k * kReMaxSlots + t] = caps[t];
        break;
      }
    }
  }
}

GX_RE_FN bool re_step(const ReVm& vm, const ReInst& in, uint32_t c) {
  if (in.op == RE_CHAR) return c == (uint32_t)in.y;
  if (in.op == RE_ANY) return c != '\n';
  if (in.op != RE_CLASS) return false;
  const uint32_t cnt = (uint32_t)in.y & 0x7fffffffu;
  bool hit = false;
  for (uint32_t k = 0; k < cnt; k++) {  // sorted, disjoint ranges
    const ReRange r = vm.ranges[in.x + k];
    if (c < r.lo) break;
    if (c <= r.hi) {
      hit = true;
      break;
    }
  }
  return hit != (in.y < 0);
}

// The leftmost-first match starting at byte pos or later: its capture slots in best.
GX_RE_FN bool re_search(ReVm& vm, ReList* cl, ReList* nl, int pos, int32_t* best) {
  int32_t caps[kReMaxSlots];
  bool matched = false;
  cl->n = 0;
  vm.gen++;
  for (int i = pos;;) {
    if (!matched) {  // a thread starting here, below every earlier-starting one
      for (int t = 0; t < vm.nslots; t++) caps[t] = -1;
      re_add(vm, *cl, 0, caps, i);
    }
    if (cl->n == 0 && matched) break;  // (without a match, later starts remain)
    uint32_t c = 0;
    int clen = 0;
    if (i < vm.n) {  // the code point at i (a truncated sequence reads as its first byte)
      const unsigned char b = vm.p[i];
      clen = re_utf8_len(b);
      if (i + clen > vm.n) clen = 1;
      c = clen == 1 ? b : clen == 2 ? (b & 0x1Fu) : clen == 3 ? (b & 0x0Fu) : (b & 0x07u);
      for (int k = 1; k < clen; k++) c = (c << 6) | (vm.p[i + k] & 0x3Fu);
    }
    vm.gen++;
    nl->n = 0;
    for (int k = 0; k < cl->n; k++) {
      const int pc = cl->pc[k];
      const ReInst in = vm.prog[pc];
      if (in.op == RE_MATCH) {  // the threads below this one are dropped
        matched = true;
        for (int t = 0; t < vm.nslots; t++) best[t] = cl->cap[k * kReMaxSlots + t];
        break;
      }
      if (clen > 0 && re_step(vm, in, c)) {
        for (int t = 0; t < vm.nslots; t++) caps[t] = cl->cap[k * kReMaxSlots + t];
        re_add(vm, *nl, pc + 1, caps, i + clen);
      }
    }
    ReList* t = cl;
    cl = nl;
    nl = t;
    if (clen == 0) break;
    i += clen;
  }
  return matched;
}

GX_RE_FN int re_put(unsigned char* d, int at, const unsigned char* src, int n) {
  if (d)
    for (int i = 0; i < n; i++) d[at + i] = src[i];
  return at + n;
}

// REGEXP_REPLACE of one row p[0, n) (cudf::strings::replace_with_backrefs,
// LogicalProject.cpp:149-183): the first `keep` characters (the position
// argument) as they are, then every match, left to right, replaced by the
// template `tmpl` (tl bytes), whose group references take the group's text
// (empty when the group did not take part).  Writes to d unless it is null;
// returns the row's length.
GX_RE_FN int regex_replace_row(const unsigned char* program, const unsigned char* tmpl, int tl,
                               const unsigned char* p, int n, int keep, unsigned char* d) {
  const ReHeader* h = (const ReHeader*)program;
  ReVm vm;
  vm.prog = (const ReInst*)(h + 1);
  vm.ranges = (const ReRange*)(vm.prog + h->ninst);
  vm.nslots = h->nslots;
  vm.p = p;
  vm.n = n;
  vm.gen = 0;
  for (int k = 0; k < kReMaxInst; k++) vm.mark[k] = 0;
  int from = 0;
  for (int c = 0; c < keep && from < n; c++) from += re_utf8_len(p[from]);
  if (from > n) from = n;
  vm.from = from;
  ReList l1, l2;
  int32_t best[kReMaxSlots];
  int at = re_put(d, 0, p, from);
  int pos = from;
  while (pos < n && re_search(vm, &l1, &l2, pos, best)) {
    at = re_put(d, at, p + pos, best[0] - pos);
    for (int t = 0; t < tl;) {
      if (tmpl[t] == 0xFF && t + 1 < tl) {
        const int g = tmpl[t + 1];
        if (g == 0xFF) {
          at = re_put(d, at, tmpl + t, 1);
        } else if (best[2 * g] >= 0 && best[2 * g + 1] >= best[2 * g]) {
          at = re_put(d, at, p + best[2 * g], best[2 * g + 1] - best[2 * g]);
        }
        t += 2;
      } else {
        at = re_put(d, at, tmpl + t, 1);
        t++;
      }
    }
    if (best[1] <= pos) break;  // cannot happen: the pattern never matches the empty string
    pos = best[1];
  }
  return re_put(d, at, p + pos, n - pos);
}

}  // namespace gx
