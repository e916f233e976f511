// regex.cpp -- the REGEXP_REPLACE pattern compiler (see regex.h): a
// recursive-descent parser into a syntax tree, checks, then a Thompson-style
// program whose SPLIT instructions order the alternatives (first = preferred),
// which the device runs as a Pike VM.
#include "regex.h"

#include <algorithm>
#include <vector>

#include "gx_common.h"

namespace gx {
namespace {

struct Node {
  enum Kind { CHAR, ANY, CLASS, BOL, EOL, WORDB, NWORDB, CAT, ALT, REP, GROUP } kind = CAT;
  uint32_t c = 0;
  std::vector<ReRange> ranges;
  bool neg = false;
  std::vector<Node> kids;
  int min = 0, max = -1;  // REP: max -1 is unbounded
  bool lazy = false;
  int group = 0;  // GROUP: capture index (0: non-capturing)
};

[[noreturn]] void bad(const std::string& why, const std::string& pattern) {
  fail(GX_ERR_UNSUPPORTED, "REGEXP_REPLACE pattern " + why + ": " + pattern);
}

std::vector<ReRange> normalise(std::vector<ReRange> r) {
  std::sort(r.begin(), r.end(), [](const ReRange& a, const ReRange& b) { return a.lo < b.lo; });
  std::vector<ReRange> out;
  for (const auto& x : r) {
    if (!out.empty() && x.lo <= out.back().hi + 1) out.back().hi = std::max(out.back().hi, x.hi);
    else out.push_back(x);
  }
  return out;
}

std::vector<ReRange> complement(const std::vector<ReRange>& r) {
  std::vector<ReRange> out;
  uint32_t next = 0;
  for (const auto& x : normalise(r)) {
    if (x.lo > next) out.push_back({next, x.lo - 1});
    next = x.hi + 1;
  }
  if (next <= 0x10FFFF) out.push_back({next, 0x10FFFF});
  return out;
}

// \d \w \s and their complements, ASCII only
bool class_escape(char e, std::vector<ReRange>& r) {
  std::vector<ReRange> base;
  switch (e) {
    case 'd': case 'D': base = {{'0', '9'}}; break;
    case 'w': case 'W': base = {{'0', '9'}, {'A', 'Z'}, {'_', '_'}, {'a', 'z'}}; break;
    case 's': case 'S': base = {{'\t', '\r'}, {' ', ' '}}; break;  // \t \n \v \f \r and space
    default: return false;
  }
  if (e >= 'A' && e <= 'Z') base = complement(base);
  r.insert(r.end(), base.begin(), base.end());
  return true;
}

class Parser {
 public:
  explicit Parser(const std::string& p) : p_(p) {}
  Node parse() {
    Node n = alt();
    if (i_ < p_.size()) bad("has an unmatched ')'", p_);
    return n;
  }
  int groups() const { return groups_; }

 private:
  const std::string& p_;
  size_t i_ = 0;
  int groups_ = 0;

  bool more() const { return i_ < p_.size(); }
  char peek() const { return p_[i_]; }

  uint32_t code_point() {  // the UTF-8 code point at i_
    const unsigned char b = (unsigned char)p_[i_];
    int len = b < 0x80 ? 1 : (b >> 5) == 0x6 ? 2 : (b >> 4) == 0xE ? 3 : (b >> 3) == 0x1E ? 4 : 0;
    if (len == 0 || i_ + len > p_.size()) bad("is not valid UTF-8", p_);
    uint32_t c = len == 1 ? b : len == 2 ? (b & 0x1F) : len == 3 ? (b & 0x0F) : (b & 0x07);
    for (int k = 1; k < len; k++) {
      const unsigned char t = (unsigned char)p_[i_ + k];
      if ((t & 0xC0) != 0x80) bad("is not valid UTF-8", p_);
      c = (c << 6) | (t & 0x3F);
    }
    i_ += len;
    return c;
  }

  // an escape's single code point: \t \n \r \f \v or escaped punctuation
  uint32_t escaped_char(char e) {
    switch (e) {
      case 't': return '\t';
      case 'n': return '\n';
      case 'r': return '\r';
      case 'f': return '\f';
      case 'v': return '\v';
      default: break;
    }
    if ((e >= '0' && e <= '9') || (e >= 'A' && e <= 'Z') || (e >= 'a' && e <= 'z') || (unsigned char)e >= 0x80)
      bad(std::string("uses the escape \\") + e, p_);
    return (unsigned char)e;
  }

  Node alt() {
    Node first = seq();
    if (!more() || peek() != '|') return first;
    Node n;
    n.kind = Node::ALT;
    n.kids.push_back(std::move(first));
    while (more() && peek() == '|') {
      i_++;
      n.kids.push_back(seq());
    }
    return n;
  }

  Node seq() {
    Node n;
    n.kind = Node::CAT;
    while (more() && peek() != '|' && peek() != ')') {
      Node a = atom();
      quantify(a);
      n.kids.push_back(std::move(a));
    }
    return n;
  }

  bool number(int* v) {
    size_t j = i_;
    long x = 0;
    while (j < p_.size() && p_[j] >= '0' && p_[j] <= '9' && x <= 100000) x = x * 10 + (p_[j++] - '0');
    if (j == i_) return false;
    i_ = j;
    *v = (int)std::min<long>(x, 100000);
    return true;
  }

  void quantify(Node& a) {
    if (!more()) return;
    int mn = 0, mx = -1;
    const char q = peek();
    if (q == '*') {
      i_++;
    } else if (q == '+') {
      mn = 1;
      i_++;
    } else if (q == '?') {
      mx = 1;
      i_++;
    } else if (q == '{') {
      i_++;
      const bool has_min = number(&mn);
      if (more() && peek() == '}' && has_min) {
        mx = mn;
      } else if (more() && peek() == ',') {
        i_++;
        if (!number(&mx)) mx = -1;
        if (!has_min) mn = 0;
        if (!has_min && mx < 0) bad("has a malformed {...}", p_);
      } else {
        bad("has a malformed {...}", p_);
      }
      if (!more() || peek() != '}') bad("has a malformed {...}", p_);
      i_++;
      if (mx >= 0 && mx < mn) bad("has a repeat whose minimum exceeds its maximum", p_);
      if (mn > 1000 || mx > 1000) bad("repeats more than 1000 times", p_);
    } else {
      return;
    }
    bool lazy = false;
    if (more() && peek() == '?') {
      lazy = true;
      i_++;
    }
    if (more() && (peek() == '*' || peek() == '+' || peek() == '?' || peek() == '{')) bad("repeats a repeat", p_);
    if (a.kind == Node::BOL || a.kind == Node::EOL || a.kind == Node::WORDB || a.kind == Node::NWORDB)
      bad("repeats an anchor", p_);
    Node r;
    r.kind = Node::REP;
    r.min = mn;
    r.max = mx;
    r.lazy = lazy;
    r.kids.push_back(std::move(a));
    a = std::move(r);
  }

  Node atom() {
    Node n;
    const char c = peek();
    if (c == '(') {
      i_++;
      n.kind = Node::GROUP;
      if (more() && peek() == '?') {
        if (i_ + 1 < p_.size() && p_[i_ + 1] == ':') i_ += 2;
        else bad("uses a (?...) construct other than (?:...)", p_);
      } else {
        n.group = ++groups_;
      }
      n.kids.push_back(alt());
      if (!more() || peek() != ')') bad("has an unmatched '('", p_);
      i_++;
      return n;
    }
    if (c == '[') return char_class();
    if (c == '*' || c == '+' || c == '?' || c == '{' || c == '}') bad("has nothing to repeat or a stray brace", p_);
    i_++;
    if (c == '.') {
      n.kind = Node::ANY;
      return n;
    }
    if (c == '^') {
      n.kind = Node::BOL;
      return n;
    }
    if (c == '$') {
      n.kind = Node::EOL;
      return n;
    }
    if (c == '\\') {
      if (!more()) bad("ends with '\\'", p_);
      const char e = p_[i_++];
      if (e == 'b' || e == 'B') {
        n.kind = e == 'b' ? Node::WORDB : Node::NWORDB;
        return n;
      }
      if (class_escape(e, n.ranges)) {
        n.kind = Node::CLASS;
        n.ranges = normalise(n.ranges);
        return n;
      }
      n.kind = Node::CHAR;
      n.c = escaped_char(e);
      return n;
    }
    i_--;
    n.kind = Node::CHAR;
    n.c = code_point();
    return n;
  }

  Node char_class() {
    i_++;  // '['
    Node n;
    n.kind = Node::CLASS;
    if (more() && peek() == '^') {
      n.neg = true;
      i_++;
    }
    bool first = true;
    for (;;) {
      if (!more()) bad("has an unterminated [...]", p_);
      if (peek() == ']' && !first) {
        i_++;
        break;
      }
      first = false;
      uint32_t lo;
      if (peek() == '\\') {
        i_++;
        if (!more()) bad("ends with '\\'", p_);
        const char e = p_[i_++];
        if (class_escape(e, n.ranges)) {
          if (more() && peek() == '-' && i_ + 1 < p_.size() && p_[i_ + 1] != ']') bad("has a bad character range", p_);
          continue;
        }
        if (e == 'b' || e == 'B') bad("uses \\b inside [...]", p_);
        lo = escaped_char(e);
      } else {
        lo = code_point();
      }
      uint32_t hi = lo;
      if (more() && peek() == '-' && i_ + 1 < p_.size() && p_[i_ + 1] != ']') {
        i_++;
        if (peek() == '\\') {
          i_++;
          if (!more()) bad("ends with '\\'", p_);
          const char e = p_[i_++];
          std::vector<ReRange> dummy;
          if (class_escape(e, dummy) || e == 'b' || e == 'B') bad("has a bad character range", p_);
          hi = escaped_char(e);
        } else {
          hi = code_point();
        }
        if (hi < lo) bad("has a bad character range", p_);
      }
      n.ranges.push_back({lo, hi});
    }
    n.ranges = normalise(n.ranges);
    return n;
  }
};

// can match without consuming a character
bool nullable(const Node& n) {
  switch (n.kind) {
    case Node::CHAR: case Node::ANY: case Node::CLASS: return false;
    case Node::BOL: case Node::EOL: case Node::WORDB: case Node::NWORDB: return true;
    case Node::CAT:
      for (const auto& k : n.kids)
        if (!nullable(k)) return false;
      return true;
    case Node::ALT:
      for (const auto& k : n.kids)
        if (nullable(k)) return true;
      return false;
    case Node::REP: return n.min == 0 || nullable(n.kids[0]);
    case Node::GROUP: return nullable(n.kids[0]);
  }
  return true;
}

void check(const Node& n, const std::string& p) {
  if (n.kind == Node::REP && nullable(n.kids[0])) bad("repeats a subpattern that can match the empty string", p);
  for (const auto& k : n.kids) check(k, p);
}

class Emitter {
 public:
  Emitter(int max_group, const std::string& p) : max_group_(max_group), p_(p) {}
  std::vector<ReInst> code;
  std::vector<ReRange> ranges;

  int emit(ReOp op, int x = 0, int32_t y = 0) {
    if ((int)code.size() >= kReMaxInst) bad("compiles to more than 64 instructions", p_);
    code.push_back(ReInst{(uint8_t)op, 0, (uint16_t)x, y});
    return (int)code.size() - 1;
  }
  int here() const { return (int)code.size(); }

  void node(const Node& n) {
    switch (n.kind) {
      case Node::CHAR: emit(RE_CHAR, 0, (int32_t)n.c); break;
      case Node::ANY: emit(RE_ANY); break;
      case Node::CLASS: {
        if (ranges.size() + n.ranges.size() > (size_t)kReMaxRanges) bad("has more than 256 class ranges", p_);
        const int at = (int)ranges.size();
        ranges.insert(ranges.end(), n.ranges.begin(), n.ranges.end());
        emit(RE_CLASS, at, (int32_t)((uint32_t)n.ranges.size() | (n.neg ? 0x80000000u : 0u)));
        break;
      }
      case Node::BOL: emit(RE_BOL); break;
      case Node::EOL: emit(RE_EOL); break;
      case Node::WORDB: emit(RE_WORDB); break;
      case Node::NWORDB: emit(RE_NWORDB); break;
      case Node::CAT:
        for (const auto& k : n.kids) node(k);
        break;
      case Node::ALT: {
        // SPLIT next_alt; body; JMP end; ... the last alternative without a SPLIT
        std::vector<int> jumps;
        for (size_t k = 0; k < n.kids.size(); k++) {
          int split = -1;
          if (k + 1 < n.kids.size()) split = emit(RE_SPLIT);
          if (split >= 0) code[split].x = (uint16_t)here();
          node(n.kids[k]);
          if (k + 1 < n.kids.size()) {
            jumps.push_back(emit(RE_JMP));
            code[split].y = here();
          }
        }
        for (int j : jumps) code[j].x = (uint16_t)here();
        break;
      }
      case Node::GROUP: {
        const bool cap = n.group > 0 && n.group <= max_group_;
        if (cap) emit(RE_SAVE, 2 * n.group);
        node(n.kids[0]);
        if (cap) emit(RE_SAVE, 2 * n.group + 1);
        break;
      }
      case Node::REP: {
        const Node& e = n.kids[0];
        if (n.max < 0) {
          for (int k = 0; k + 1 < n.min; k++) node(e);
          if (n.min >= 1) {  // L: e; SPLIT L, end
            const int L = here();
            node(e);
            const int s = emit(RE_SPLIT);
            prefer(s, L, here(), n.lazy);
          } else {  // L: SPLIT body, end; body: e; JMP L
            const int L = emit(RE_SPLIT);
            node(e);
            emit(RE_JMP, L);
            prefer(L, L + 1, here(), n.lazy);
          }
        } else {
          for (int k = 0; k < n.min; k++) node(e);
          // the optional copies: skipping one skips the rest
          std::vector<int> splits;
          for (int k = n.min; k < n.max; k++) {
            splits.push_back(emit(RE_SPLIT));
            node(e);
          }
          for (int s : splits) prefer(s, s + 1, here(), n.lazy);
        }
        break;
      }
    }
  }

 private:
  // SPLIT s: the body first (greedy) or the exit first (lazy)
  void prefer(int s, int body, int exit, bool lazy) {
    code[s].x = (uint16_t)(lazy ? exit : body);
    code[s].y = lazy ? body : exit;
  }
  int max_group_;
  const std::string& p_;
};

}  // namespace

void compile_regex_replace(const std::string& pattern, const std::string& repl, std::string* program,
                           std::string* tmpl) {
  if (pattern.empty()) bad("is empty", pattern);
  Parser ps(pattern);
  const Node root = ps.parse();
  if (nullable(root)) bad("can match the empty string", pattern);
  check(root, pattern);
  // the replacement: \N or ${N} refer to group N
  std::string t;
  int max_ref = 0;
  for (size_t i = 0; i < repl.size();) {
    int g = -1;
    size_t next = i + 1;
    if (repl[i] == '\\' && i + 1 < repl.size() && repl[i + 1] >= '0' && repl[i + 1] <= '9') {
      g = repl[i + 1] - '0';
      next = i + 2;
    } else if (repl[i] == '$' && i + 1 < repl.size() && repl[i + 1] == '{') {
      size_t j = i + 2;
      long v = 0;
      while (j < repl.size() && repl[j] >= '0' && repl[j] <= '9' && v < 1000) v = v * 10 + (repl[j++] - '0');
      if (j > i + 2 && j < repl.size() && repl[j] == '}') {
        g = (int)v;
        next = j + 1;
      }
    }
    if (g < 0) {
      const unsigned char b = (unsigned char)repl[i];
      t.push_back((char)b);
      if (b == 0xFF) t.push_back((char)0xFF);
      i = next;
      continue;
    }
    if (g > ps.groups())
      fail(GX_ERR_INVALID, "REGEXP_REPLACE replacement refers to group " + std::to_string(g) + " of a pattern with " +
                               std::to_string(ps.groups()) + " groups");
    if (2 * g + 1 >= kReMaxSlots) fail(GX_ERR_UNSUPPORTED, "REGEXP_REPLACE replacement refers to a group above 4");
    max_ref = std::max(max_ref, g);
    t.push_back((char)0xFF);
    t.push_back((char)g);
    i = next;
  }
  Emitter em(max_ref, pattern);
  em.emit(RE_SAVE, 0);
  em.node(root);
  em.emit(RE_SAVE, 1);
  em.emit(RE_MATCH);
  ReHeader h{(int32_t)em.code.size(), (int32_t)em.ranges.size(), 2 * (max_ref + 1), 0};
  program->assign((const char*)&h, sizeof(h));
  program->append((const char*)em.code.data(), em.code.size() * sizeof(ReInst));
  program->append((const char*)em.ranges.data(), em.ranges.size() * sizeof(ReRange));
  *tmpl = t;
}

}  // namespace gx
