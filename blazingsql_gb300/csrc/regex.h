// regex.h -- REGEXP_REPLACE: a regular expression compiled on the host into a
// small program that the string pre-pass runs per row on the device.
//
// The reference hands the pattern to cudf::strings::replace_with_backrefs
// (LogicalProject.cpp:149-183), a libcudf regular-expression engine outside
// the reference tree.  This build restates a subset with leftmost-first
// semantics (the first alternative and the greedy choice win; matches do not
// overlap and are replaced left to right):
//   literals (UTF-8 code points), escaped punctuation, \t \n \r \f \v;
//   .  (any code point but \n);  [...] / [^...] with ranges and \d \w \s;
//   \d \w \s \D \W \S (ASCII classes);  \b \B (ASCII word boundaries);
//   ^ $ (start / end of the subject only);  (...), (?:...), |;
//   * + ? {n} {n,} {n,m} {,m}, each optionally lazy (a trailing ?).
// Patterns that can match the empty string, quantifiers over subpatterns
// that can, and anything else (back references, look-around, flags) are
// rejected with GX_ERR_UNSUPPORTED.  The replacement may refer to groups
// 0..4 as \N or ${N}.
#pragma once

#include <cstdint>
#include <string>

namespace gx {

enum ReOp : uint8_t {
  RE_CHAR = 0,  // y: the code point
  RE_ANY,       // any code point but '\n'
  RE_CLASS,     // x: first range, y: range count | negated << 31
  RE_SPLIT,     // try x first, then y
  RE_JMP,       // x
  RE_SAVE,      // record the position in capture slot x
  RE_MATCH,
  RE_BOL,       // at the start of the subject
  RE_EOL,       // at the end of the subject
  RE_WORDB,     // at an ASCII word boundary
  RE_NWORDB     // not at one
};

struct ReInst {
  uint8_t op;
  uint8_t pad;
  uint16_t x;
  int32_t y;
};

struct ReRange {
  uint32_t lo, hi;  // inclusive
};

// A compiled program: this header, then `ninst` instructions, then `nranges` ranges.
struct ReHeader {
  int32_t ninst, nranges, nslots, pad;
};

constexpr int kReMaxInst = 64;     // instructions of one program
constexpr int kReMaxSlots = 10;    // capture slots: groups 0..4
constexpr int kReMaxRanges = 256;  // class ranges of one program

// Compiles `pattern` and the replacement template `repl` for REGEXP_REPLACE.
// *program receives the program (header, instructions, ranges); *tmpl the
// replacement with literal bytes as they are, a group reference as 0xFF and
// the group number, and a literal 0xFF byte as 0xFF 0xFF.  Fails with
// GX_ERR_UNSUPPORTED or GX_ERR_INVALID (a reference to a missing group).
void compile_regex_replace(const std::string& pattern, const std::string& repl, std::string* program,
                           std::string* tmpl);

}  // namespace gx
