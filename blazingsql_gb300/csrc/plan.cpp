// plan.cpp -- expression DAG + CUDA code generation (see plan.h).
#include "plan.h"

#include "fp64emu.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <set>
#include <sstream>

namespace gx {
namespace {

std::string hex64(uint64_t v) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "0x%016llxull", (unsigned long long)v);
  return buf;
}

struct Builder {
  Plan& p;
  std::map<std::string, int> memo;
  int rand_counter = 0;
  bool rand_out_row = false;

  int push(Node n, const std::string& key) {
    if (!key.empty()) {
      auto it = memo.find(key);
      if (it != memo.end()) return it->second;
    }
    p.nodes.push_back(n);
    int id = (int)p.nodes.size() - 1;
    if (!key.empty()) memo[key] = id;
    return id;
  }

  int add(const ExprPtr& e) {
    if (e->kind == Expr::COL) {
      Node n;
      n.kind = Node::COL;
      n.col = e->col;
      n.vtype = e->vtype;
      n.ktype = e->ktype;
      return push(n, "c" + std::to_string(e->col));
    }
    if (e->kind == Expr::LIT) {
      Node n;
      n.kind = Node::LIT;
      n.lit_type = e->lit_type;
      n.lit_valid = e->lit_valid;
      n.lit_bits = e->lit_bits;
      n.vtype = e->vtype;
      n.ktype = e->ktype;
      return push(n, "l" + std::to_string(e->vtype) + ":" + std::to_string(e->ktype) + ":" +
                         std::to_string(e->lit_valid) + ":" + std::to_string(e->lit_bits));
    }
    // every operand is visited (RAND ordinals follow the reference's post-order
    // visit, which also walks the extra operands of an un-nested OR)
    std::vector<int> kids;
    for (const auto& c : e->ch) kids.push_back(add(c));
    Node n;
    n.kind = Node::OP;
    n.op = e->op;
    n.vtype = e->vtype;
    n.ktype = e->ktype;
    if (!kids.empty()) n.a = kids[0];
    if (op_is_binary(e->op) && kids.size() > 1) n.b = kids[1];
    if (e->op == OP_RAND) {
      n.rand_id = rand_counter++;
      n.rand_out_row = rand_out_row;
      return push(n, "");  // never shared
    }
    return push(n, "o" + std::to_string(n.op) + ":" + std::to_string(n.a) + ":" + std::to_string(n.b) + ":" +
                       std::to_string(n.vtype) + ":" + std::to_string(n.ktype));
  }
};

void flatten_and(const Plan& p, int id, std::vector<int>& out) {
  const Node& n = p.nodes[id];
  if (n.kind == Node::OP && n.op == OP_AND) {
    flatten_and(p, n.a, out);
    flatten_and(p, n.b, out);
  } else {
    out.push_back(id);
  }
}

}  // namespace

uint64_t OutSpec::lit_bits_as_element() const {
  if (type == FLOAT32) {
    double d;
    std::memcpy(&d, &lit_bits, 8);
    const float f = (float)d;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
  }
  if (type == BOOL8) return lit_bits != 0;
  return lit_bits;
}

bool Plan::needs_kernel() const {
  if (has_filter()) return true;
  for (const auto& o : outputs)
    if (o.kind == OutSpec::NODE) return true;
  return false;
}

Plan build_plan(const std::vector<int>& schema, const std::vector<bool>& nullable, const std::string& condition,
                const std::vector<std::string>& expressions, bool filter_all, bool rand_by_output_row,
                int first_rand_id, int* rand_count, bool all_nodes) {
  Plan p;
  p.schema = schema;
  p.nullable = nullable;
  Builder b{p};
  if (!condition.empty()) {
    ExprPtr c = compile_expression(condition, schema);
    if (c->vtype != BOOL8) fail(GX_ERR_TYPE, "Expression does not evaluate to a boolean mask");
    p.predicate = b.add(c);
    flatten_and(p, p.predicate, p.conjuncts);
  }
  b.rand_counter = first_rand_id;
  b.rand_out_row = rand_by_output_row && !condition.empty();
  if (filter_all) {
    p.filter_copies_all = true;
    for (size_t i = 0; i < schema.size(); i++) {
      OutSpec o;
      o.kind = OutSpec::COPY;
      o.col = (int)i;
      o.type = schema[i];
      p.outputs.push_back(o);
    }
  } else {
    for (const auto& text : expressions) {
      ExprPtr e = compile_expression(text, schema);
      OutSpec o;
      if (e->kind == Expr::LIT && all_nodes) {
        fail(GX_ERR_UNSUPPORTED, "a literal aggregation input");
      } else if (e->kind == Expr::LIT) {
        o.kind = OutSpec::BROADCAST;
        o.type = e->lit_type;
        o.lit_bits = e->lit_bits;
        o.lit_valid = e->lit_valid;
        if (o.type == EMPTY || type_size(o.type) == 0) fail(GX_ERR_TYPE, "a bare null literal has no column type");
      } else if (e->kind == Expr::COL && !all_nodes) {
        o.kind = OutSpec::COPY;
        o.col = e->col;
        o.type = schema[e->col];
      } else {
        o.kind = OutSpec::NODE;
        o.node = b.add(e);
        o.type = e->vtype;
        if (type_size(o.type) == 0) fail(GX_ERR_TYPE, "expression has no fixed-width output type");
      }
      p.outputs.push_back(o);
    }
  }
  if (rand_count) *rand_count = b.rand_counter - first_rand_id;
  if (p.outputs.size() > (size_t)GX_MAX_OUTS) fail(GX_ERR_UNSUPPORTED, "too many output columns in one plan");
  if (schema.size() > (size_t)GX_MAX_COLS) fail(GX_ERR_UNSUPPORTED, "too many input columns in one plan");
  // data under NULL is observable where it reaches CASE's magic-number test
  for (int i = (int)p.nodes.size() - 1; i >= 0; i--) {
    Node& n = p.nodes[i];
    if (n.kind != Node::OP) continue;
    if (n.op == OP_MAGIC_IF_NOT && n.b >= 0) p.nodes[n.b].exact_null = true;
    if (n.op == OP_FIRST_NON_MAGIC) {
      p.nodes[n.a].exact_null = true;
      if (n.exact_null) p.nodes[n.b].exact_null = true;
    }
  }
  return p;
}

// =============================================================== code generation
namespace {

const char* load_fn(int t) {
  switch (t) {
    case INT8: return "gx_ld_i8";
    case UINT8: case BOOL8: return "gx_ld_u8";
    case INT16: return "gx_ld_i16";
    case UINT16: return "gx_ld_u16";
    case INT32: case TIMESTAMP_DAYS: case DURATION_DAYS: return "gx_ld_i32";
    case UINT32: return "gx_ld_u32";
    case FLOAT32: return "gx_ld_f32";
    default: return "gx_ld_64";
  }
}

const char* load_fn_emu(int t) { return t == FLOAT32 ? "gx_ld_f32e" : load_fn(t); }

// store of 64-bit value bits into an output column of type t
// (device_ptr_write_from_buffer, interpreter_ops.cuh:329-395)
std::string store_stmt(int t, const std::string& ptr, const std::string& idx, const std::string& bits) {
  switch (t) {
    case BOOL8: return "gx_st_8(" + ptr + ", " + idx + ", (u64)((" + bits + ") != 0ull));";
    case INT8: case UINT8: return "gx_st_8(" + ptr + ", " + idx + ", " + bits + ");";
    case INT16: case UINT16: return "gx_st_16(" + ptr + ", " + idx + ", " + bits + ");";
    case INT32: case UINT32: case TIMESTAMP_DAYS: case DURATION_DAYS:
      return "gx_st_32(" + ptr + ", " + idx + ", " + bits + ");";
    case FLOAT32: return "gx_st_f32(" + ptr + ", " + idx + ", " + bits + ");";
    default: return "gx_st_64(" + ptr + ", " + idx + ", " + bits + ");";
  }
}

// raw element copy for COPY outputs of filter kernels
std::string raw_type(int t) {
  switch (type_size(t)) {
    case 1: return "unsigned char";
    case 2: return "unsigned short";
    case 4: return "unsigned int";
    default: return "unsigned long long";
  }
}

uint64_t magic_double_bits() {
  const double m = 1.7976931348623123e+308;  // interpreter_ops.cuh:47
  uint64_t u;
  std::memcpy(&u, &m, 8);
  return u;
}

int64_t ns_per_unit(int t) {
  switch (t) {
    case TIMESTAMP_DAYS: case DURATION_DAYS: return 86400000000000LL;
    case TIMESTAMP_SECONDS: case DURATION_SECONDS: return 1000000000LL;
    case TIMESTAMP_MILLISECONDS: case DURATION_MILLISECONDS: return 1000000LL;
    case TIMESTAMP_MICROSECONDS: case DURATION_MICROSECONDS: return 1000LL;
    default: return 1;
  }
}

class Gen {
 public:
  Gen(const Plan& p, const KernelConfig& c) : p_(p), cfg_(c) {}

  // operand views for node id in word-slot k
  std::string B(int id) const { return value_bits(id); }
  std::string V(int id) const { return value_valid(id); }

  std::string value_bits(int id) const {
    const Node& n = p_.nodes[id];
    if (n.kind == Node::LIT) return n.lit_valid ? hex64(n.lit_bits) : std::string("0ull");
    return "b" + std::to_string(id) + "[k]";
  }
  std::string value_valid(int id) const {
    const Node& n = p_.nodes[id];
    if (n.kind == Node::LIT) return n.lit_valid ? "true" : "false";
    return "v" + std::to_string(id) + "[k]";
  }
  bool kind_f(int id) const { return is_float(p_.nodes[id].ktype); }
  // operand as a double value (native FP64 arithmetic follows)
  std::string asD(int id) const {
    if (kind_f(id)) return "gx_D(" + B(id) + ")";
    return emu_op(kNativeConvert) ? "gx_D(gxe_i2d((i64)(" + B(id) + ")))" : "gx_I2D(" + B(id) + ")";
  }
  // operand as the bits of its double value (integer-pipe binary64 routines follow)
  std::string asDB(int id) const {
    if (kind_f(id)) return B(id);
    return emu_op(kNativeConvert) ? "gxe_i2d((i64)(" + B(id) + "))" : "gx_B(gx_I2D(" + B(id) + "))";
  }
  std::string asI(int id) const {
    if (!kind_f(id)) return "(i64)(" + B(id) + ")";
    return emu_op(kNativeConvert) ? "gxe_d2ll(" + B(id) + ")" : "gx_D2LL(gx_D(" + B(id) + "))";
  }
  std::string nz(int id) const {
    if (!kind_f(id)) return "(" + B(id) + " != 0ull)";
    return emu_op(kNativeCompare) ? "gxe_nz(" + B(id) + ")" : "(gx_D(" + B(id) + ") != 0.0)";
  }
  bool emu() const { return cfg_.emulate_fp64; }
  // this class of binary64 operation runs on the integer pipes
  bool emu_op(int cls) const { return cfg_.emulate_fp64 && !(cfg_.native_f64_ops & cls); }

  // a valid literal's value as binary64 bits (integer literals converted exactly
  // as the kernels convert them)
  uint64_t literal_double_bits(int id) const {
    const Node& n = p_.nodes[id];
    return kind_f(id) ? n.lit_bits : gxe_i2d((gxe_i64)n.lit_bits);
  }
  // A divisor whose value is an integer (an integer-kind node, or its CAST
  // to DOUBLE / FLOAT, which keeps the exact value inside a plan): the node
  // holding that integer, or -1.  Divisions by it may take the reciprocal
  // table (gxe_div_small) when the plan puts literal divisions on the FMA unit.
  int int_divisor(int y) const {
    const Node& n = p_.nodes[y];
    if (n.kind == Node::LIT) return -1;
    if (!kind_f(y)) return y;
    if (n.kind == Node::OP && (n.op == OP_CAST_DOUBLE || n.op == OP_CAST_FLOAT) && !kind_f(n.a) &&
        p_.nodes[n.a].kind != Node::LIT)
      return n.a;
    return -1;
  }
  bool small_div(int id) const {
    const Node& n = p_.nodes[id];
    return n.kind == Node::OP && n.op == OP_DIV && (kind_f(n.a) || kind_f(n.b)) && emu_op(kNativeDiv) &&
           !emu_op(kNativeIntDiv) && !const_divisor(n.b) && int_divisor(n.b) >= 0;
  }
  // the reciprocal table gxe_div_small reads, when some division of the plan uses it
  void emit_rcp_table(std::ostringstream& o) const {
    bool any = false;
    for (size_t i = 0; i < p_.nodes.size() && !any; i++) any = small_div((int)i);
    if (!any) return;
    o << "#define GX_RCP_N " << kRcpTable << "\n__device__ const unsigned long long gx_rcp_[GX_RCP_N] = {";
    for (int k = 1; k <= kRcpTable; k++) {
      const double y = 1.0 / (double)k;
      uint64_t b;
      std::memcpy(&b, &y, 8);
      o << (k > 1 ? "," : "") << (k % 8 == 1 ? "\n  " : "") << hex64(b);
    }
    o << "};\n";
  }
  static constexpr int kRcpTable = 1024;
  // a literal divisor that is a normal finite nonzero double
  bool const_divisor(int id) const {
    const Node& n = p_.nodes[id];
    if (n.kind != Node::LIT || !n.lit_valid) return false;
    const int e = (int)((literal_double_bits(id) >> 52) & 0x7FF);
    return e >= 1 && e <= 2046;
  }

  // statements computing node id for slot k; row / out-row expressions given
  void emit_node(std::ostringstream& o, int id, const std::string& ind) const {
    const Node& n = p_.nodes[id];
    const std::string b = "b" + std::to_string(id) + "[k]", v = "v" + std::to_string(id) + "[k]";
    if (n.kind == Node::LIT) return;
    if (n.kind == Node::COL) {
      const int c = n.col;
      if (tile_mode_) {
        // the tile's rows of column c are in shared memory: element trow at
        // byte offset sd_<c> + trow * width, validity bit trow of the tile's
        // re-aligned mask words vmw_<c>
        const std::string gfn = emu() ? load_fn_emu(p_.schema[c]) : load_fn(p_.schema[c]);
        const std::string sfn = "gx_sld_" + gfn.substr(6);  // gx_ld_X -> gx_sld_X
        o << ind << b << " = inr ? (u64)" << sfn << "(sd_" << c << " + trow * " << type_size(p_.schema[c])
          << "u) : 0ull;\n";
        if (p_.nullable[c]) o << ind << v << " = inr && ((vmw_" << c << "[trow >> 5] >> (trow & 31u)) & 1u);\n";
        else o << ind << v << " = inr;\n";
        return;
      }
      auto st = staged_.find(c);
      if (st != staged_.end()) {
        // full words are staged in shared memory at (buffer, index); a partial
        // last word is read from global memory
        const std::string gfn = emu() ? load_fn_emu(p_.schema[c]) : load_fn(p_.schema[c]);
        const std::string sfn = "gx_lds_" + gfn.substr(6);  // gx_ld_X -> gx_lds_X
        o << ind << b << " = inr ? (full_word_ ? (u64)" << sfn << "(" << st->second.first << ", " << st->second.second
          << ") : (u64)" << gfn << "(a.in_data[" << c << "], a.in_off[" << c << "] + row)) : 0ull;\n";
      } else {
        std::string fn = emu() ? load_fn_emu(p_.schema[c]) : load_fn(p_.schema[c]);
        if (reread_cols_.count(c)) fn = "gx_ldg_" + fn.substr(6);  // gx_ld_X -> gx_ldg_X
        o << ind << b << " = inr ? (u64)" << fn << "(a.in_data[" << c << "], a.in_off[" << c << "] + row) : 0ull;\n";
      }
      if (p_.nullable[c]) o << ind << v << " = inr && gx_valid(a.in_mask[" << c << "], a.in_off[" << c << "] + row);\n";
      else o << ind << v << " = inr;\n";
      return;
    }
    std::string r, vv;
    const Op op = n.op;
    if (op == OP_RAND) {
      o << ind << b << " = gx_B(gx_philox_uniform(a.seed, " << n.rand_id << "u, (u64)("
        << (n.rand_out_row ? "orow" : "row") << ")));\n";
      o << ind << v << " = true;\n";
      return;
    }
    if (op == OP_ROW_INDEX) {
      o << ind << b << " = (u64)row;\n";
      o << ind << v << " = true;\n";
      return;
    }
    if (op_is_unary(op)) {
      const int x = n.a;
      const int lt = p_.nodes[x].ktype;
      const bool lf = kind_f(x);
      const std::string X = B(x), XV = V(x);
      bool always_valid = false;
      switch (op) {
        case OP_IS_NOT_TRUE:
          r = "(u64)(!(" + XV + " && " + (lf ? "(" + X + ") == 0x3ff0000000000000ull" : "(i64)(" + X + ") == 1LL") +
              "))";
          always_valid = true;
          break;
        case OP_IS_NOT_FALSE:
          r = "(u64)(!(" + XV + " && " + (lf ? "((" + X + ") << 1) == 0ull" : "(i64)(" + X + ") == 0LL") + "))";
          always_valid = true;
          break;
        case OP_IS_NULL: r = "(u64)(!" + XV + ")"; always_valid = true; break;
        case OP_IS_NOT_NULL: r = "(u64)(" + XV + ")"; always_valid = true; break;
        case OP_FLOOR: r = emu_op(kNativeRound) ? "gxe_floor(" + asDB(x) + ")" : "gx_B(floor(" + asD(x) + "))"; break;
        case OP_CEIL: r = emu_op(kNativeRound) ? "gxe_ceil(" + asDB(x) + ")" : "gx_B(ceil(" + asD(x) + "))"; break;
        case OP_SIN: r = "gx_B(sin(" + asD(x) + "))"; break;
        case OP_COS: r = "gx_B(cos(" + asD(x) + "))"; break;
        case OP_ASIN: r = "gx_B(asin(" + asD(x) + "))"; break;
        case OP_ACOS: r = "gx_B(acos(" + asD(x) + "))"; break;
        case OP_TAN: r = "gx_B(tan(" + asD(x) + "))"; break;
        case OP_COTAN: r = "gx_B(cos(" + asD(x) + ") / sin(" + asD(x) + "))"; break;
        case OP_ATAN: r = "gx_B(atan(" + asD(x) + "))"; break;
        case OP_LN: r = "gx_B(log(" + asD(x) + "))"; break;
        case OP_LOG10: r = "gx_B(log10(" + asD(x) + "))"; break;
        case OP_EXP: r = "gx_B(exp(" + asD(x) + "))"; break;
        case OP_ABS:
          r = lf ? "((" + X + ") & 0x7fffffffffffffffull)" : "((i64)(" + X + ") < 0LL ? 0ull - (" + X + ") : (" + X + "))";
          break;
        case OP_NOT: r = "(u64)(!" + nz(x) + ")"; break;
        case OP_IS_TRUE: r = "(u64)" + asI(x); break;
        case OP_YEAR: case OP_MONTH: case OP_DAY: case OP_DAYOFWEEK: case OP_HOUR: case OP_MINUTE: case OP_SECOND: {
          if (!is_timestamp(lt)) { r = "0ull"; break; }
          const int which = op == OP_YEAR ? 0 : op == OP_MONTH ? 1 : op == OP_DAY ? 2 : op == OP_DAYOFWEEK ? 3
                          : op == OP_HOUR ? 4 : op == OP_MINUTE ? 5 : 6;
          const long long per_day = lt == TIMESTAMP_DAYS ? 1LL : 86400000000000LL / ns_per_unit(lt);
          const std::string cnt = lt == TIMESTAMP_DAYS ? "gx_days32((i64)(" + X + "))" : "(i64)(" + X + ")";
          r = "(u64)gx_extract(" + cnt + ", " + std::to_string(per_day) + "LL, " + std::to_string(which) + ")";
          break;
        }
        case OP_CAST_TINYINT: case OP_CAST_SMALLINT: case OP_CAST_INTEGER: case OP_CAST_BIGINT:
          r = "(u64)" + asI(x);
          break;
        case OP_CAST_FLOAT: case OP_CAST_DOUBLE: r = asDB(x); break;
        case OP_CAST_DATE: {
          long long div = lt == TIMESTAMP_SECONDS ? 86400LL : lt == TIMESTAMP_MILLISECONDS ? 86400000LL
                        : lt == TIMESTAMP_MICROSECONDS ? 86400000000LL : lt == TIMESTAMP_NANOSECONDS ? 86400000000000LL : 1;
          r = div == 1 ? "(u64)(i64)(int)" + asI(x) : "(u64)(i64)(int)(" + asI(x) + " / " + std::to_string(div) + "LL)";
          break;
        }
        case OP_CAST_TIMESTAMP_SECONDS: case OP_CAST_TIMESTAMP_MILLISECONDS: case OP_CAST_TIMESTAMP_MICROSECONDS:
        case OP_CAST_TIMESTAMP:
          if (is_timestamp(lt)) {
            const std::string cnt = lt == TIMESTAMP_DAYS ? "(u64)gx_days32(" + asI(x) + ")" : "(u64)" + asI(x);
            r = "(" + cnt + " * " + std::to_string(ns_per_unit(lt)) + "ull)";
          } else {
            r = "(u64)" + asI(x);
          }
          break;
        default: fail(GX_ERR_UNSUPPORTED, "no code for unary operator");
      }
      vv = always_valid ? "true" : XV;
      if (!always_valid && n.exact_null) r = "(" + vv + " ? " + r + " : 0ull)";
      o << ind << b << " = " << r << ";\n" << ind << v << " = " << vv << ";\n";
      return;
    }
    // binary
    const int x = n.a, y = n.b;
    const bool lf = kind_f(x), rf = kind_f(y), anyf = lf || rf;
    const int lt = p_.nodes[x].ktype, rt = p_.nodes[y].ktype;
    const std::string X = B(x), Y = B(y), XV = V(x), YV = V(y);
    switch (op) {
      case OP_MAGIC_IF_NOT: {
        const std::string cond = "(" + XV + " && " + nz(x) + ")";
        o << ind << "{ const bool c_ = " << cond << ";\n";
        o << ind << "  " << b << " = c_ ? " << Y << " : " << (rf ? "gx_B(GX_MAGIC_D)" : "(u64)GX_MAGIC_I")
          << ";\n";
        o << ind << "  " << v << " = c_ ? " << YV << " : false; }\n";
        return;
      }
      case OP_FIRST_NON_MAGIC: {
        // double equality with the (non-zero, finite) magic value is bit equality
        const std::string magic = lf ? "((" + X + ") == " + hex64(magic_double_bits()) + ")"
                                     : "((i64)(" + X + ") == GX_MAGIC_I)";
        o << ind << "{ const bool m_ = " << magic << ";\n";
        o << ind << "  " << b << " = m_ ? " << Y << " : " << X << ";\n";
        o << ind << "  " << v << " = m_ ? " << YV << " : " << XV << "; }\n";
        return;
      }
      case OP_OR:
        o << ind << b << " = (" << XV << " && " << YV << ") ? (u64)(" << nz(x) << " || " << nz(y) << ") : (" << XV
          << " ? " << X << " : (" << YV << " ? " << Y << " : 0ull));\n";
        o << ind << v << " = (" << XV << " && " << YV << ") || (" << XV << " ? " << nz(x) << " : " << YV << ");\n";
        return;
      case OP_IS_NOT_DISTINCT_FROM: {
        const std::string eq = !anyf ? "(" + X + " == " + Y + ")"
                               : emu_op(kNativeCompare) ? "gxe_eq(" + asDB(x) + ", " + asDB(y) + ")"
                                       : "(" + asD(x) + " == " + asD(y) + ")";
        o << ind << b << " = (u64)((!" << XV << " && !" << YV << ") || (" << XV << " && " << YV << " && " << eq
          << "));\n";
        o << ind << v << " = true;\n";
        return;
      }
      default: break;
    }
    vv = "(" + XV + " && " + YV + ")";
    const bool ts_cmp = is_timestamp(lt) && is_timestamp(rt);
    auto cmp = [&](const char* opstr) -> std::string {
      if (ts_cmp) {
        auto to_ns = [&](int id, int t) {
          const std::string cnt = t == TIMESTAMP_DAYS ? "(u64)gx_days32((i64)(" + B(id) + "))" : "(u64)(" + B(id) + ")";
          return "(i64)(" + cnt + " * " + std::to_string(ns_per_unit(t)) + "ull)";
        };
        return std::string("(u64)(") + to_ns(x, lt) + " " + opstr + " " + to_ns(y, rt) + ")";
      }
      if (anyf && emu_op(kNativeCompare)) {
        const std::string X2 = asDB(x), Y2 = asDB(y), o2 = opstr;
        if (o2 == "<") return "(u64)gxe_lt(" + X2 + ", " + Y2 + ")";
        if (o2 == ">") return "(u64)gxe_lt(" + Y2 + ", " + X2 + ")";
        if (o2 == "<=") return "(u64)gxe_le(" + X2 + ", " + Y2 + ")";
        if (o2 == ">=") return "(u64)gxe_le(" + Y2 + ", " + X2 + ")";
        if (o2 == "==") return "(u64)gxe_eq(" + X2 + ", " + Y2 + ")";
        return "(u64)(!gxe_eq(" + X2 + ", " + Y2 + "))";
      }
      if (anyf) return std::string("(u64)(") + asD(x) + " " + opstr + " " + asD(y) + ")";
      return std::string("(u64)((i64)(") + X + ") " + opstr + " (i64)(" + Y + "))";
    };
    switch (op) {
      case OP_AND: r = "(u64)(" + nz(x) + " && " + nz(y) + ")"; break;
      case OP_ADD:
        r = !anyf ? "(" + X + " + " + Y + ")"
            : emu_op(kNativeAddSub) ? "gxe_add(" + asDB(x) + ", " + asDB(y) + ")" : "gx_B(" + asD(x) + " + " + asD(y) + ")";
        break;
      case OP_SUB:
        r = !anyf ? "(" + X + " - " + Y + ")"
            : emu_op(kNativeAddSub) ? "gxe_sub(" + asDB(x) + ", " + asDB(y) + ")" : "gx_B(" + asD(x) + " - " + asD(y) + ")";
        break;
      case OP_MUL:
        r = !anyf ? "(" + X + " * " + Y + ")"
            : emu_op(kNativeMul) ? "gxe_mul(" + asDB(x) + ", " + asDB(y) + ")" : "gx_B(" + asD(x) + " * " + asD(y) + ")";
        break;
      case OP_DIV:
        if (anyf && emu_op(kNativeDiv) && const_divisor(y) && !emu_op(kNativeConstDiv)) {
          // the FMA unit's correctly rounded constant division, the integer
          // pipes' form outside its exponent window
          const uint64_t db = literal_double_bits(y);
          double bd, yd;
          std::memcpy(&bd, &db, 8);
          yd = 1.0 / bd;
          uint64_t yb;
          std::memcpy(&yb, &yd, 8);
          int lo = 0, hi = 0;
          gxe_div_c_window((int)((db >> 52) & 0x7FF), &lo, &hi);
          r = "gxe_div_c(" + asDB(x) + ", " + hex64(db) + ", " + hex64(gxe_recip_fixed((db & GXE_FRAC) | GXE_HIDDEN)) +
              ", " + hex64(yb) + ", " + std::to_string(lo) + ", " + std::to_string(hi) + ")";
        } else if (small_div(id)) {  // an integer divisor: RN(1/|k|) from the table for small |k|
          r = "gxe_div_small(" + asDB(x) + ", (i64)(" + B(int_divisor(y)) + "), gx_rcp_, GX_RCP_N)";
        } else if (anyf && emu_op(kNativeDiv) && const_divisor(y)) {
          // constant divisor: its fixed-point reciprocal is computed here
          const uint64_t db = literal_double_bits(y);
          r = "gxe_div_r(" + asDB(x) + ", " + hex64(db) + ", " +
              hex64(gxe_recip_fixed((db & GXE_FRAC) | GXE_HIDDEN)) + ")";
        } else {
          r = !anyf ? "gx_div_ii(" + X + ", " + Y + ")"
              : emu_op(kNativeDiv) ? "gxe_div(" + asDB(x) + ", " + asDB(y) + ")" : "gx_B(" + asD(x) + " / " + asD(y) + ")";
        }
        vv = "(" + vv + " && " + (rf ? nz(y) : "(i64)(" + Y + ") != 0LL") + ")";
        break;
      case OP_MOD:
        if (anyf) {
          r = "gx_B(fmod(" + asD(x) + ", " + asD(y) + "))";
        } else {
          r = "gx_mod_ii(" + X + ", " + Y + ")";
          vv = "(" + vv + " && (i64)(" + Y + ") != 0LL)";
        }
        break;
      case OP_POW: r = "gx_B(pow(" + asD(x) + ", " + asD(y) + "))"; break;
      case OP_ROUND: r = "gx_B(gx_round_to(" + asD(x) + ", " + asD(y) + "))"; break;
      case OP_EQ: r = cmp("=="); break;
      case OP_NE: r = cmp("!="); break;
      case OP_LT: r = cmp("<"); break;
      case OP_GT: r = cmp(">"); break;
      case OP_LE: r = cmp("<="); break;
      case OP_GE: r = cmp(">="); break;
      default: fail(GX_ERR_UNSUPPORTED, "no code for binary operator");
    }
    if (n.exact_null) {
      o << ind << v << " = " << vv << ";\n";
      o << ind << b << " = " << v << " ? " << r << " : 0ull;\n";
    } else {
      o << ind << b << " = " << r << ";\n" << ind << v << " = " << vv << ";\n";
    }
  }

  // ids of OP / COL nodes reachable from roots, ascending (topological)
  std::vector<int> cone(const std::vector<int>& roots) const {
    std::set<int> seen;
    std::function<void(int)> go = [&](int id) {
      if (id < 0 || seen.count(id)) return;
      seen.insert(id);
      const Node& n = p_.nodes[id];
      if (n.kind == Node::OP) { go(n.a); go(n.b); }
    };
    for (int r : roots) go(r);
    std::vector<int> v;
    for (int id : seen)
      if (p_.nodes[id].kind != Node::LIT) v.push_back(id);
    return v;
  }

  void decl(std::ostringstream& o, const std::vector<int>& ids, const std::string& ind) const {
    for (int id : ids) o << ind << "u64 b" << id << "[GX_V]; bool v" << id << "[GX_V];\n";
  }

  // keep expression of conjunct c (index into p_.conjuncts) for slot k
  std::string conj_keep(int cid) const {
    if (cid < 0) return "true";
    const Node& n = p_.nodes[cid];
    if (n.kind == Node::LIT) return (n.lit_valid && n.lit_bits != 0) ? "inr" : "false";
    if (p_.conjuncts.size() == 1 && cid == p_.predicate)  // the root itself: BOOL8 column semantics
      return "(" + V(cid) + " && " + B(cid) + " != 0ull)";
    return "(" + V(cid) + " && " + nz(cid) + ")";
  }

  // Evaluates nodes `ids` for the warp's GX_V words: first a loop issuing every
  // column load of every word (so the loads are in flight together), then a
  // loop computing the operators and `tail` (a statement per word).  `inr` is
  // the per-row condition that loads are predicated on.
  void emit_words(std::ostringstream& o, const std::vector<int>& ids, const std::string& ind, const std::string& inr,
                  const std::string& tail) const {
    const std::string rowdef =
        tile_mode_ ? "const u32 trow = (u32)(wl0 + k) * 32u + (u32)lane; const i64 row = tb0 + (i64)trow; "
                     "const bool inr = " + inr + "; (void)inr; (void)row;\n"
                   : "const i64 row = (w0 + k) * 32 + lane; const bool inr = " + inr + "; (void)inr;\n";
    bool any_col = false;
    for (int id : ids) any_col |= p_.nodes[id].kind == Node::COL;
    if (any_col) {
      o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) {\n" << ind << "  " << rowdef;
      for (int id : ids)
        if (p_.nodes[id].kind == Node::COL) emit_node(o, id, ind + "  ");
      o << ind << "}\n";
    }
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) {\n" << ind << "  " << rowdef;
    for (int id : ids)
      if (p_.nodes[id].kind != Node::COL) emit_node(o, id, ind + "  ");
    if (!tail.empty()) o << ind << "  " << tail << "\n";
    o << ind << "}\n";
  }

  // predicate phase: fills keep bits bal[k]; with short-circuit, conjuncts are
  // evaluated in cfg order and later conjuncts skipped for all-dead warps
  void emit_predicate(std::ostringstream& o, const std::string& ind) const {
    std::vector<int> order;
    if (!cfg_.conjunct_order.empty()) {
      for (int i : cfg_.conjunct_order) order.push_back(p_.conjuncts.at(i));
    } else {
      order = p_.conjuncts;
    }
    o << ind << "bool alive[GX_V];\n";
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) alive[k] = (w0 + k) * 32 + lane < a.n;\n";
    if (cfg_.runtime_order) {
      if (cfg_.stream_slots > 0 && streamable())
        emit_predicate_stream(o, ind);
      else
        emit_predicate_runtime_order(o, ind);
      return;
    }
    std::set<int> done;
    if (!cfg_.short_circuit) {
      // fixed order: evaluate every conjunct for every row
      std::string keep = "inr";
      for (int c : order) keep += " && " + conj_keep(c);
      emit_words(o, cone(order), ind, "row < a.n", "alive[k] = " + keep + ";");
      return;
    }
    o << ind << "bool any_alive = true;\n";
    for (size_t j = 0; j < order.size(); j++) {
      std::vector<int> ids;
      for (int id : cone({order[j]}))
        if (!done.count(id)) ids.push_back(id);
      // loads predicated on the row being alive, issued for all words before
      // the ballots
      o << ind << "if (any_alive) {\n";
      emit_words(o, ids, ind + "  ", "alive[k]", "alive[k] = alive[k] && " + conj_keep(order[j]) + ";");
      o << ind << "  u32 any_ = 0;\n";
      o << ind << "  #pragma unroll\n" << ind << "  for (int k = 0; k < GX_V; k++) any_ |= __ballot_sync(GX_FULL, alive[k]);\n";
      o << ind << "  any_alive = any_ != 0u;\n";
      o << ind << "}\n";
      for (int id : ids) done.insert(id);
    }
  }

  // Short-circuit evaluation in the order a.order[] given at launch: one
  // warp-uniform switch per conjunct, each case evaluating its conjunct's whole
  // cone (no value crosses conjuncts) for the warp's GX_V words.  Column loads
  // are predicated on the row still being alive, so sectors whose rows all
  // died are not read; the words' loads are issued together (no ballot between
  // them), and the warp stops once none of its rows is alive.
  void emit_predicate_runtime_order(std::ostringstream& o, const std::string& ind) const {
    const int nc = (int)p_.conjuncts.size();
    o << ind << "u32 live_[GX_V];\n";
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) live_[k] = __ballot_sync(GX_FULL, alive[k]);\n";
    o << ind << "for (int j_ = 0; j_ < " << nc << "; j_++) {\n";
    o << ind << "  bool keep_[GX_V];\n";
    o << ind << "  switch (a.order_dev ? __ldg(a.order_dev + j_) : a.order[j_]) {\n";
    for (int c = 0; c < nc; c++) {
      const int cid = p_.conjuncts[c];
      o << ind << "    case " << c << ": {\n";
      std::vector<int> ids = cone({cid});
      decl(o, ids, ind + "      ");
      emit_words(o, ids, ind + "      ", "alive[k]", "keep_[k] = " + conj_keep(cid) + ";");
      o << ind << "      break; }\n";
    }
    o << ind << "    default:\n";
    o << ind << "      #pragma unroll\n" << ind << "      for (int k = 0; k < GX_V; k++) keep_[k] = false;\n";
    o << ind << "  }\n";
    o << ind << "  u32 any_ = 0u;\n";
    o << ind << "  #pragma unroll\n" << ind << "  for (int k = 0; k < GX_V; k++) {\n";
    o << ind << "    alive[k] = alive[k] && keep_[k];\n";
    o << ind << "    live_[k] = __ballot_sync(GX_FULL, alive[k]);\n";
    o << ind << "    any_ |= live_[k];\n";
    o << ind << "  }\n";
    o << ind << "  if (any_ == 0u) break;\n";
    o << ind << "}\n";
  }

  // every conjunct reads exactly one column (or none)
  bool streamable() const {
    for (size_t c = 0; c < p_.conjuncts.size(); c++)
      if (conjunct_columns(p_, (int)c).size() > 1) return false;
    return true;
  }

  // Streaming short-circuit in the launch order: the warp keeps S word slots in
  // flight, each at its own conjunct step; a slot whose word has no live row
  // left, or has passed every conjunct, takes the warp's next word.  Each round
  // issues the loads of every slot before evaluating any, so the warp always has
  // S words' loads outstanding instead of a shrinking lockstep set, and the
  // number of dependent load rounds is about (words x steps per word) / S
  // rather than the longest chain per group of words.  Word masks live in shared
  // memory (indexed by a slot's word).
  void emit_predicate_stream(std::ostringstream& o, const std::string& ind) const {
    const int nc = (int)p_.conjuncts.size();
    const int S = cfg_.stream_slots;
    std::vector<int> col_of(nc, -1);
    for (int c = 0; c < nc; c++) {
      const std::vector<int> cols = conjunct_columns(p_, c);
      if (!cols.empty()) col_of[c] = cols[0];
    }
    const std::string S_ = std::to_string(S);
    o << ind << "__shared__ u32 s_aw_[GX_WARPS][GX_V];\n";
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) {\n";
    o << ind << "  const u32 m_ = __ballot_sync(GX_FULL, alive[k]);\n";
    o << ind << "  if (lane == 0) s_aw_[warp][k] = m_;\n";
    o << ind << "}\n";
    o << ind << "__syncwarp();\n";
    o << ind << "int sw_[" << S_ << "], sj_[" << S_ << "]; u64 val_[" << S_ << "]; bool vv_[" << S_ << "];\n";
    o << ind << "int nx_ = 0;\n";
    o << ind << "#pragma unroll\n" << ind << "for (int q = 0; q < " << S_ << "; q++) {\n";
    o << ind << "  sw_[q] = -1; sj_[q] = 0; val_[q] = 0ull; vv_[q] = false;\n";
    o << ind << "  while (nx_ < GX_V && s_aw_[warp][nx_] == 0u) nx_++;\n";
    o << ind << "  if (nx_ < GX_V) { sw_[q] = nx_; nx_++; }\n";
    o << ind << "}\n";
    o << ind << "while (true) {\n";
    o << ind << "  bool act_ = false;\n";
    o << ind << "  #pragma unroll\n" << ind << "  for (int q = 0; q < " << S_ << "; q++) act_ |= sw_[q] >= 0;\n";
    o << ind << "  if (!act_) break;\n";
    // loads of every slot
    o << ind << "  #pragma unroll\n" << ind << "  for (int q = 0; q < " << S_ << "; q++) {\n";
    o << ind << "    if (sw_[q] < 0) continue;\n";
    o << ind << "    const int wk_ = sw_[q];\n";
    o << ind << "    const i64 row = (w0 + wk_) * 32 + lane;\n";
    o << ind << "    const bool inr = ((s_aw_[warp][wk_] >> lane) & 1u) != 0u;\n";
    o << ind << "    switch (a.order_dev ? __ldg(a.order_dev + sj_[q]) : a.order[sj_[q]]) {\n";
    for (int c = 0; c < nc; c++) {
      const int col = col_of[c];
      if (col < 0) continue;
      const std::string gfn = emu() ? load_fn_emu(p_.schema[col]) : load_fn(p_.schema[col]);
      o << ind << "      case " << c << ": val_[q] = inr ? (u64)" << gfn << "(a.in_data[" << col << "], a.in_off[" << col
        << "] + row) : 0ull; vv_[q] = inr" << (p_.nullable[col] ? " && gx_valid(a.in_mask[" + std::to_string(col) +
                                                                      "], a.in_off[" + std::to_string(col) + "] + row)"
                                                                : std::string())
        << "; break;\n";
    }
    o << ind << "      default: break;\n    }\n";
    o << ind << "  }\n";
    // evaluation, mask update, refill
    o << ind << "  #pragma unroll\n" << ind << "  for (int q = 0; q < " << S_ << "; q++) {\n";
    o << ind << "    if (sw_[q] < 0) continue;\n";
    o << ind << "    const int wk_ = sw_[q];\n";
    o << ind << "    const i64 row = (w0 + wk_) * 32 + lane; (void)row;\n";
    o << ind << "    const bool inr = ((s_aw_[warp][wk_] >> lane) & 1u) != 0u;\n";
    o << ind << "    const int k = 0;\n";
    o << ind << "    bool keep_ = false;\n";
    o << ind << "    switch (a.order_dev ? __ldg(a.order_dev + sj_[q]) : a.order[sj_[q]]) {\n";
    for (int c = 0; c < nc; c++) {
      const int cid = p_.conjuncts[c];
      o << ind << "      case " << c << ": {\n";
      const std::vector<int> ids = cone({cid});
      for (int id : ids) o << ind << "        u64 b" << id << "[1]; bool v" << id << "[1];\n";
      for (int id : ids) {
        if (p_.nodes[id].kind == Node::COL)
          o << ind << "        b" << id << "[0] = val_[q]; v" << id << "[0] = vv_[q];\n";
      }
      for (int id : ids)
        if (p_.nodes[id].kind != Node::COL) emit_node(o, id, ind + "        ");
      o << ind << "        keep_ = " << conj_keep(cid) << ";\n";
      o << ind << "        break; }\n";
    }
    o << ind << "      default: break;\n    }\n";
    o << ind << "    const u32 m_ = s_aw_[warp][wk_] & __ballot_sync(GX_FULL, inr && keep_);\n";
    o << ind << "    __syncwarp();\n";
    o << ind << "    if (lane == 0) s_aw_[warp][wk_] = m_;\n";
    o << ind << "    __syncwarp();\n";
    o << ind << "    sj_[q]++;\n";
    o << ind << "    if (m_ == 0u || sj_[q] >= " << nc << ") {\n";
    o << ind << "      sw_[q] = -1; sj_[q] = 0;\n";
    o << ind << "      while (nx_ < GX_V && s_aw_[warp][nx_] == 0u) nx_++;\n";
    o << ind << "      if (nx_ < GX_V) { sw_[q] = nx_; nx_++; }\n";
    o << ind << "    }\n";
    o << ind << "  }\n";
    o << ind << "}\n";
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) alive[k] = ((s_aw_[warp][k] >> lane) & 1u) != 0u;\n";
    o << ind << "__syncwarp();\n";  // s_aw_ is rewritten by the warp's next tile
  }

  // per-conjunct pass counts of this warp's rows, accumulated in shared memory
  void emit_conj_stats(std::ostringstream& o, const std::string& ind) const {
    const int nc = (int)p_.conjuncts.size();
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) {\n";
    o << ind << "  const i64 row = (w0 + k) * 32 + lane; const bool inr = row < a.n; (void)inr;\n";
    for (int c = 0; c < nc; c++) {
      o << ind << "  { const u32 b_ = __ballot_sync(GX_FULL, inr && " << conj_keep(p_.conjuncts[c]) << ");\n";
      o << ind << "    if (lane == 0) atomicAdd(&s_conj[" << c << "], (unsigned long long)__popc(b_)); }\n";
    }
    o << ind << "}\n";
  }

  std::vector<int> predicate_cone() const { return p_.has_filter() ? cone(p_.conjuncts) : std::vector<int>{}; }

  // ids of OP / COL nodes reachable from roots without descending below the
  // nodes in `stop` (which are included themselves), ascending
  std::vector<int> cone_stop(const std::vector<int>& roots, const std::set<int>& stop) const {
    std::set<int> seen;
    std::function<void(int)> go = [&](int id) {
      if (id < 0 || seen.count(id)) return;
      seen.insert(id);
      const Node& n = p_.nodes[id];
      if (n.kind == Node::OP && !stop.count(id)) { go(n.a); go(n.b); }
    };
    for (int r : roots) go(r);
    std::vector<int> v;
    for (int id : seen)
      if (p_.nodes[id].kind != Node::LIT) v.push_back(id);
    return v;
  }

  // A CASE branch (the value operand of a MAGIC_IF_NOT) whose subtree is used
  // by nothing else, reads only columns and literals, and is expensive
  // (transcendentals, divisions): the dense phase evaluates it only for the
  // kept rows whose condition selects it, packed into full warps.  Rows whose
  // condition is false take the magic value whatever the branch computes, so
  // skipping them changes no result.
  struct Lazy {
    int consumer = -1;  // the MAGIC_IF_NOT node
    int cond = -1;      // its condition operand
    int root = -1;      // the branch value operand
    std::vector<int> nodes;  // OP and COL nodes of the branch, ascending
  };

  static int op_cost(Op op) {
    switch (op) {
      case OP_LN: case OP_LOG10: case OP_EXP: case OP_POW: case OP_SIN: case OP_COS: case OP_TAN: case OP_ASIN:
      case OP_ACOS: case OP_ATAN: case OP_COTAN:
        return 64;
      case OP_DIV: case OP_MOD: case OP_ROUND:
        return 16;
      default:
        return 1;
    }
  }

  std::vector<Lazy> lazy_branches(const std::vector<int>& roots) const {
    std::vector<Lazy> out;
    if (!cfg_.lazy_case) return out;
    const std::vector<int> all = cone(roots);
    std::map<int, std::vector<int>> users;
    for (int id : all) {
      const Node& n = p_.nodes[id];
      if (n.kind != Node::OP) continue;
      if (n.a >= 0) users[n.a].push_back(id);
      if (n.b >= 0 && n.b != n.a) users[n.b].push_back(id);
    }
    const std::set<int> external(roots.begin(), roots.end());
    std::set<int> taken;
    // outermost consumers first (a parent's id is above its operands')
    for (auto it = all.rbegin(); it != all.rend(); ++it) {
      const int m = *it;
      const Node& mn = p_.nodes[m];
      if (mn.kind != Node::OP || mn.op != OP_MAGIC_IF_NOT || taken.count(m)) continue;
      const int y = mn.b;
      if (y < 0 || p_.nodes[y].kind != Node::OP || external.count(y) || taken.count(y)) continue;
      if (users[y].size() != 1 || users[y][0] != m) continue;
      const std::vector<int> ycone = cone({y});
      std::set<int> S{y};
      for (bool grown = true; grown;) {
        grown = false;
        for (int id : ycone) {
          if (S.count(id) || p_.nodes[id].kind != Node::OP || external.count(id)) continue;
          bool excl = true;
          for (int u : users[id])
            if (!S.count(u)) { excl = false; break; }
          if (excl) { S.insert(id); grown = true; }
        }
      }
      bool ok = true;
      int cost = 0;
      for (int id : ycone) {
        const Node& n = p_.nodes[id];
        if (n.kind != Node::OP) continue;
        if (!S.count(id) || taken.count(id)) { ok = false; break; }
        cost += op_cost(n.op);
      }
      if (!ok || cost < 32) continue;
      Lazy lz;
      lz.consumer = m;
      lz.cond = mn.a;
      lz.root = y;
      lz.nodes = ycone;
      for (int id : ycone)
        if (p_.nodes[id].kind == Node::OP) taken.insert(id);
      out.push_back(lz);
    }
    return out;
  }

  std::vector<int> output_roots() const {
    std::vector<int> r;
    for (const auto& o : p_.outputs)
      if (o.kind == OutSpec::NODE) r.push_back(o.node);
    return r;
  }

  const Plan& p_;
  const KernelConfig& cfg_;
  // columns read from a shared-memory staging buffer: col -> (buffer, index)
  mutable std::map<int, std::pair<std::string, std::string>> staged_;
  // tile-staged kernels: every column is read from the tile's shared-memory
  // stage (row trow of the tile; see emit_fused_tma)
  mutable bool tile_mode_ = false;
  // columns whose data both the predicate and the projections read: loaded
  // with the default cache policy so the projections' re-read hits L2
  mutable std::set<int> reread_cols_;

  // validity of node id is true for every row in range (no NULL can arise):
  // non-nullable columns, valid literals, and operators that propagate only
  // their operands' validity or divide by a nonzero literal
  bool never_null(int id) const {
    const Node& n = p_.nodes[id];
    if (n.kind == Node::LIT) return n.lit_valid;
    if (n.kind == Node::COL) return !p_.nullable[n.col];
    switch (n.op) {
      case OP_RAND: case OP_ROW_INDEX:
      case OP_IS_NOT_TRUE: case OP_IS_NOT_FALSE: case OP_IS_NULL: case OP_IS_NOT_NULL: case OP_IS_NOT_DISTINCT_FROM:
        return true;
      case OP_MAGIC_IF_NOT: return false;
      default: break;
    }
    if (op_is_unary(n.op)) return never_null(n.a);
    if (!never_null(n.a) || !never_null(n.b)) return false;
    if (n.op == OP_DIV || (n.op == OP_MOD && !kind_f(n.a) && !kind_f(n.b))) {
      const Node& d = p_.nodes[n.b];
      return d.kind == Node::LIT && d.lit_valid && (d.lit_bits & 0x7fffffffffffffffull) != 0;
    }
    return true;
  }
};

void emit_prelude(std::ostringstream& o, const KernelConfig& cfg) {
  o << "#define GX_V " << cfg.words << "\n#define GX_WARPS " << cfg.warps << "\n";
  // a register cap becomes a resident-block count in the launch bounds; without
  // one the bounds name the block size only (a minimum of one block lets ptxas
  // take more registers than its default choice)
  if (cfg.max_regs > 0)
    o << "#define GX_LB __launch_bounds__(GX_WARPS * 32, "
      << std::max(1, 65536 / (cfg.max_regs * cfg.warps * 32)) << ")\n";
  else
    o << "#define GX_LB __launch_bounds__(GX_WARPS * 32)\n";
  o << "#define GX_TILE_WORDS (GX_WARPS * GX_V)\n";
  o << "#define GX_MAX_COLS " << GX_MAX_COLS << "\n#define GX_MAX_OUTS " << GX_MAX_OUTS << "\n";
  o << "struct GxArgs {\n"
       "  const void* in_data[GX_MAX_COLS]; const u32* in_mask[GX_MAX_COLS]; i64 in_off[GX_MAX_COLS];\n"
       "  void* out_data[GX_MAX_OUTS]; u32* out_mask[GX_MAX_OUTS];\n"
       "  i64 n; i64 capacity; u64* tile_status; unsigned long long* tile_counter; unsigned long long* out_count;\n"
       "  int* err; u64 seed; unsigned long long* conj_counts; int order[16]; const int* order_dev;\n"
       "  u32 spin_limit;\n};\n"
       // polls a bounded wait makes before it gives up (0: the default)
       "#define GX_SPINS (a.spin_limit ? a.spin_limit : (1u << 22))\n";
}

// phase 2 of the filter kernels: projections for the kept rows of each word,
// written at positions pos.. (warp-uniform), plus validity bit streams.
// Stores output j for the current lane (dense rounds) and returns its validity
// expression for the round's ballot ("" for a broadcast output, filled after
// the launch).
std::string emit_dense_store(std::ostringstream& o, const Gen& g, const Plan& p, size_t j, const std::string& ind) {
  const OutSpec& os = p.outputs[j];
  if (os.kind == OutSpec::NODE) {
    o << ind << "if (wr) " << store_stmt(os.type, "a.out_data[" + std::to_string(j) + "]", "orow", g.B(os.node)) << "\n";
    return g.V(os.node);
  }
  if (os.kind != OutSpec::COPY) return "";
  const int c = os.col;
  const std::string rt = raw_type(p.schema[c]);
  o << ind << "if (wr) ((" << rt << "*)a.out_data[" << j << "])[orow] = __ldcs((const " << rt << "*)a.in_data[" << c
    << "] + a.in_off[" << c << "] + row);\n";
  return p.nullable[c] ? "gx_valid(a.in_mask[" + std::to_string(c) + "], a.in_off[" + std::to_string(c) + "] + row)"
                       : "true";
}

// outputs that carry a validity bit stream (broadcasts are filled after the launch)
std::vector<size_t> masked_outputs(const Plan& p) {
  std::vector<size_t> v;
  for (size_t j = 0; j < p.outputs.size(); j++)
    if (p.outputs[j].kind != OutSpec::BROADCAST) v.push_back(j);
  return v;
}

// Dense phase 2: the warp's kept rows, in row order, are dealt to lanes in
// rounds of 32 (lane l of round r takes the warp's (32r + l)-th kept row), so
// projections are computed only for surviving rows and every output store and
// validity word of a round is contiguous.  Operands are re-read with the
// gathered row index (predicate columns hit L1/L2).
// statements mapping kept rank t_ of the warp (0 <= t_ < total_) to its row
// through the warp's kept-row list in shared memory
void emit_rank_to_row(std::ostringstream& o, const std::string& ind) {
  o << ind << "const i64 row = w0 * 32 + (act ? (i64)s_kept_[warp][t_] : 0); const bool inr = act; (void)inr;\n";
  o << ind << "const i64 orow = (i64)pos + (i64)t_; (void)orow;\n";
  o << ind << "const int k = 0;\n";
}

// nodes ids for one row per lane: gathers first, then operators; lazy branch
// roots (lz_root -> index) are read from the branch results in shared memory
void emit_row_nodes(std::ostringstream& o, const Gen& g, const Plan& p, const std::vector<int>& ids,
                    const std::map<int, int>& lz_root, const std::string& ind) {
  g.decl(o, ids, ind);
  for (int id : ids)
    if (p.nodes[id].kind == Node::COL) g.emit_node(o, id, ind);
  for (int id : ids) {
    if (p.nodes[id].kind == Node::COL) continue;
    auto it = lz_root.find(id);
    if (it != lz_root.end()) {
      o << ind << "b" << id << "[k] = s_lzb_[" << it->second << "][warp][t_]; v" << id << "[k] = s_lzv_["
        << it->second << "][warp][t_] != 0;\n";
    } else {
      g.emit_node(o, id, ind);
    }
  }
}

// Dense phase 2: the warp's kept rows, in row order, are dealt to lanes in
// rounds of 32 (lane l of round r takes the warp's (32r + l)-th kept row), so
// projections are computed only for surviving rows and every output store and
// validity word of a round is contiguous.  Operands are re-read with the
// gathered row index (predicate columns hit L1/L2).  Expensive CASE branches
// (Gen::lazy_branches) are first evaluated for the kept rows whose condition
// selects them, packed into full warps, into shared memory.
void emit_filter_writes_dense(std::ostringstream& o, const Gen& g, const Plan& p, const std::string& ind) {
  const std::vector<int> roots = g.output_roots();
  const std::vector<Gen::Lazy> lz = g.lazy_branches(roots);
  std::map<int, int> lz_root;
  std::set<int> stop;
  for (size_t i = 0; i < lz.size(); i++) {
    lz_root[lz[i].root] = (int)i;
    stop.insert(lz[i].root);
  }
  const std::vector<int> proj = g.cone_stop(roots, stop);
  // the warp's kept rows in order: offsets from its first row, by kept rank
  o << ind << "__shared__ unsigned short s_kept_[GX_WARPS][GX_V * 32];\n";
  o << ind << "u32 total_ = 0u;\n";
  o << ind << "#pragma unroll\n" << ind << "for (int kk = 0; kk < GX_V; kk++) {\n";
  o << ind << "  if ((bal[kk] >> lane) & 1u) s_kept_[warp][total_ + __popc(bal[kk] & ((1u << lane) - 1u))] = (unsigned short)(kk * 32 + lane);\n";
  o << ind << "  total_ += __popc(bal[kk]);\n";
  o << ind << "}\n";
  o << ind << "__syncwarp();\n";
  if (!lz.empty()) {
    const int nl = (int)lz.size();
    o << ind << "__shared__ u64 s_lzb_[" << nl << "][GX_WARPS][GX_V * 32];\n";
    o << ind << "__shared__ unsigned char s_lzv_[" << nl << "][GX_WARPS][GX_V * 32];\n";
    // pass 1: which kept rows select each branch
    std::vector<int> conds;
    for (const auto& l : lz) conds.push_back(l.cond);
    const std::vector<int> cond_ids = g.cone(conds);
    o << ind << "u32 dmd_[" << nl << "][GX_V];\n";
    o << ind << "__shared__ unsigned short s_dem_[GX_WARPS][GX_V * 32];\n";
    o << ind << "#pragma unroll\n" << ind << "for (int r_ = 0; r_ < GX_V; r_++) {\n";
    const std::string i2 = ind + "  ";
    o << i2 << "#pragma unroll\n" << i2 << "for (int l_ = 0; l_ < " << nl << "; l_++) dmd_[l_][r_] = 0u;\n";
    o << i2 << "if ((u32)r_ * 32u < total_) {\n";
    const std::string i3 = i2 + "  ";
    o << i3 << "const u32 t_ = (u32)r_ * 32u + (u32)lane; const bool act = t_ < total_;\n";
    emit_rank_to_row(o, i3);
    emit_row_nodes(o, g, p, cond_ids, {}, i3);
    for (int i = 0; i < nl; i++) {
      const int c = lz[i].cond;
      o << i3 << "dmd_[" << i << "][r_] = __ballot_sync(GX_FULL, act && (" << g.V(c) << " && " << g.nz(c) << "));\n";
    }
    o << i2 << "}\n";
    o << ind << "}\n";
    // pass 2: each branch over its selecting rows, 32 at a time
    for (int i = 0; i < nl; i++) {
      o << ind << "{\n";
      // the kept ranks selecting branch i, in order, listed in shared memory
      o << i2 << "u32 dtot_ = 0u;\n";
      o << i2 << "#pragma unroll\n" << i2 << "for (int r_ = 0; r_ < GX_V; r_++) {\n";
      o << i2 << "  const u32 db_ = dmd_[" << i << "][r_];\n";
      o << i2 << "  if ((db_ >> lane) & 1u) s_dem_[warp][dtot_ + __popc(db_ & ((1u << lane) - 1u))] = (unsigned short)(r_ * 32 + lane);\n";
      o << i2 << "  dtot_ += __popc(db_);\n";
      o << i2 << "}\n";
      o << i2 << "__syncwarp();\n";
      o << i2 << "for (u32 db_ = 0; db_ < dtot_; db_ += 32u) {\n";
      o << i3 << "const u32 q_ = db_ + (u32)lane; const bool act = q_ < dtot_;\n";
      o << i3 << "const u32 t_ = act ? (u32)s_dem_[warp][q_] : 0u;\n";
      emit_rank_to_row(o, i3);
      emit_row_nodes(o, g, p, lz[i].nodes, {}, i3);
      o << i3 << "if (act) { s_lzb_[" << i << "][warp][t_] = " << g.B(lz[i].root) << "; s_lzv_[" << i
        << "][warp][t_] = " << g.V(lz[i].root) << " ? 1 : 0; }\n";
      o << i2 << "}\n";
      o << i2 << "__syncwarp();\n";  // s_dem_ is rewritten for the next branch
      o << ind << "}\n";
    }
    o << ind << "__syncwarp();\n";
  }
  // validity bit streams: one position shared by all outputs (every round
  // appends the same number of bits to each), one accumulator per output
  // whose validity varies and one shared by the outputs that are never NULL;
  // the first word may be shared with the previous warp's range and the last
  // with the next one (atomicOr), words in between are stored
  const std::vector<size_t> mo = masked_outputs(p);
  std::vector<int> slot(p.outputs.size(), -1);
  int nslots = 0, nn_slot = -1;
  for (size_t j : mo) {
    const OutSpec& os = p.outputs[j];
    if (os.kind == OutSpec::COPY ? !p.nullable[os.col] : g.never_null(os.node)) {
      if (nn_slot < 0) nn_slot = nslots++;
      slot[j] = nn_slot;
    } else {
      slot[j] = nslots++;
    }
  }
  const int nacc = std::max(nslots, 1);
  o << ind << "u64 acc_[" << nacc << "];\n";
  o << ind << "#pragma unroll\n" << ind << "for (int j = 0; j < " << nacc << "; j++) acc_[j] = 0ull;\n";
  o << ind << "int bf_ = (int)(pos & 31ull); i64 bword_ = (i64)(pos >> 5); bool bfirst_ = bf_ != 0;\n";
  o << ind << "const i64 cap_words = (a.capacity + 31) >> 5;\n";
  o << ind << "for (u32 base_ = 0; base_ < total_; base_ += 32u) {\n";
  const std::string in2 = ind + "  ";
  o << in2 << "const u32 t_ = base_ + (u32)lane; const bool act = t_ < total_;\n";
  emit_rank_to_row(o, in2);
  emit_row_nodes(o, g, p, proj, lz_root, in2);
  o << in2 << "const bool wr = act && orow < a.capacity;\n";
  o << in2 << "const int nb = (int)min(32u, total_ - base_);\n";
  std::vector<std::string> vexpr(p.outputs.size());
  for (size_t j = 0; j < p.outputs.size(); j++) vexpr[j] = emit_dense_store(o, g, p, j, in2);
  for (int sl = 0; sl < nslots; sl++) {
    std::string e = "act";
    if (sl != nn_slot)
      for (size_t j : mo)
        if (slot[j] == sl) e = "act && " + vexpr[j];
    o << in2 << "acc_[" << sl << "] |= (u64)__ballot_sync(GX_FULL, " << e << ") << bf_;\n";
  }
  o << in2 << "const int nf_ = bf_ + nb;\n";
  o << in2 << "if (nf_ >= 32) {\n";
  o << in2 << "  if (lane == 0 && bword_ < cap_words) {\n";
  for (size_t j : mo)
    o << in2 << "    if (bfirst_) atomicOr(a.out_mask[" << j << "] + bword_, (u32)acc_[" << slot[j] << "]); else a.out_mask["
      << j << "][bword_] = (u32)acc_[" << slot[j] << "];\n";
  o << in2 << "  }\n";
  o << in2 << "  #pragma unroll\n" << in2 << "  for (int j = 0; j < " << nacc << "; j++) acc_[j] >>= 32;\n";
  o << in2 << "  bfirst_ = false; bword_++; bf_ = nf_ - 32;\n";
  o << in2 << "} else {\n" << in2 << "  bf_ = nf_;\n" << in2 << "}\n";
  o << ind << "}\n";
  o << ind << "__syncwarp();\n";  // the kept-row list and branch results are rewritten by the next tile
  o << ind << "if (bf_ > 0 && lane == 0 && bword_ < cap_words) {\n";
  for (size_t j : mo) o << ind << "  atomicOr(a.out_mask[" << j << "] + bword_, (u32)acc_[" << slot[j] << "]);\n";
  o << ind << "}\n";
}

void emit_filter_writes(std::ostringstream& o, const Gen& g, const Plan& p, const std::vector<int>& pred_ids,
                        const std::string& ind) {
  if (g.cfg_.dense) {
    emit_filter_writes_dense(o, g, p, ind);
    return;
  }
  std::vector<int> proj = g.cone(g.output_roots());
  std::set<int> have(pred_ids.begin(), pred_ids.end());
  std::vector<int> fresh;
  for (int id : proj)
    if (!have.count(id)) fresh.push_back(id);
  g.decl(o, fresh, ind);
  o << ind << "GxBitWriter bw_[" << p.outputs.size() << "];\n";
  o << ind << "#pragma unroll\n" << ind << "for (int j = 0; j < " << p.outputs.size() << "; j++) bw_[j].init((i64)pos);\n";
  o << ind << "const i64 cap_words = (a.capacity + 31) >> 5;\n";
  o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) {\n";
  o << ind << "  const u32 bk = bal[k];\n";
  o << ind << "  if (bk == 0u) continue;\n";
  o << ind << "  const i64 row = (w0 + k) * 32 + lane; const bool inr = row < a.n; (void)inr;\n";
  o << ind << "  const bool keep = (bk >> lane) & 1u;\n";
  o << ind << "  const i64 orow = (i64)pos + __popc(bk & ((1u << lane) - 1u)); (void)orow;\n";
  for (int id : fresh) g.emit_node(o, id, ind + "  ");
  o << ind << "  const bool wr = keep && orow < a.capacity;\n";
  o << ind << "  const int nb = __popc(bk);\n";
  o << ind << "  const int q = (int)(orow - (i64)pos);\n";
  for (size_t j = 0; j < p.outputs.size(); j++) {
    const OutSpec& os = p.outputs[j];
    std::string vexpr;
    if (os.kind == OutSpec::NODE) {
      o << ind << "  if (wr) " << store_stmt(os.type, "a.out_data[" + std::to_string(j) + "]", "orow", g.B(os.node))
        << "\n";
      vexpr = g.V(os.node);
    } else if (os.kind == OutSpec::COPY) {
      const int c = os.col;
      const std::string rt = raw_type(p.schema[c]);
      o << ind << "  if (wr) ((" << rt << "*)a.out_data[" << j << "])[orow] = __ldcs((const " << rt << "*)a.in_data[" << c
        << "] + a.in_off[" << c << "] + row);\n";
      vexpr = p.nullable[c] ? "gx_valid(a.in_mask[" + std::to_string(c) + "], a.in_off[" + std::to_string(c) + "] + row)"
                            : "true";
    } else {
      continue;  // broadcast outputs are filled after the launch
    }
    o << ind << "  { const u32 vb_ = __reduce_or_sync(GX_FULL, (keep && " << vexpr << ") ? (1u << (q & 31)) : 0u);\n";
    o << ind << "    if (bw_[" << j << "].word < cap_words) bw_[" << j << "].append(a.out_mask[" << j
      << "], vb_, nb); else { bw_[" << j << "].fill = 0; } }\n";
  }
  o << ind << "  pos += (u64)nb;\n";
  o << ind << "}\n";
  for (size_t j = 0; j < p.outputs.size(); j++) {
    if (p.outputs[j].kind == OutSpec::BROADCAST) continue;
    o << ind << "if (bw_[" << j << "].word < cap_words) bw_[" << j << "].flush(a.out_mask[" << j << "]);\n";
  }
}

// Fused single-pass filter (dense projections) as a two-stage tile pipeline:
// a block claims tile t+1 and evaluates its predicate before it resolves tile
// t's output offset by look-back, so the look-back of t waits on tiles that
// had a whole tile's time to publish, and the next tile's loads are in flight
// meanwhile.  Tile t's keep masks stay in registers between the stages (dense
// projections recompute outputs from the gathered rows).  A claimed tile's
// aggregate is published before the block waits on anything, and a tile's
// look-back only needs earlier tiles, so the pipeline cannot deadlock.
void emit_fused_pipelined(std::ostringstream& o, const Gen& g, const Plan& p, const std::vector<int>& pred_ids) {
  // with conj_stats (fixed order, every conjunct evaluated for every row): each
  // conjunct's passing rows, counted per warp in registers and added to
  // a.conj_counts once per warp at the end
  const bool stats = g.cfg_.conj_stats && !g.cfg_.runtime_order && !g.cfg_.short_circuit;
  const int nc = (int)p.conjuncts.size();
  auto count_conjuncts = [&](const std::string& ind) {
    if (!stats) return;
    o << ind << "#pragma unroll\n" << ind << "for (int k = 0; k < GX_V; k++) {\n";
    o << ind << "  const i64 row = (w0 + k) * 32 + lane; const bool inr = row < a.n; (void)inr;\n";
    for (int c = 0; c < nc; c++)
      o << ind << "  cst_[" << c << "] += (u32)__popc(__ballot_sync(GX_FULL, inr && " << g.conj_keep(p.conjuncts[c])
        << "));\n";
    o << ind << "}\n";
  };
  if (stats) o << "  u32 cst_[" << nc << "] = {};\n";
  o << "  __shared__ unsigned long long s_claim;\n";
  o << "  __shared__ u32 s_cnt[2][GX_WARPS];\n";
  o << "  __shared__ u64 s_off[2][GX_WARPS];\n";
  o << "  __shared__ u64 s_base;\n";
  o << "  const i64 ntiles = (nwords + GX_TILE_WORDS - 1) / GX_TILE_WORDS;\n";
  o << "  if (threadIdx.x == 0) s_claim = atomicAdd(a.tile_counter, 1ull);\n";
  o << "  __syncthreads();\n";
  o << "  i64 tile = (i64)s_claim;\n";
  o << "  if (tile >= ntiles) return;\n";
  o << "  u32 bal[GX_V]; u32 wcnt = 0u; int par = 0; u64 ptotal = 0ull;\n";
  o << "  {\n";
  o << "    const i64 w0 = tile * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  g.decl(o, pred_ids, "    ");
  g.emit_predicate(o, "    ");
  count_conjuncts("    ");
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) { bal[k] = __ballot_sync(GX_FULL, alive[k]); wcnt += __popc(bal[k]); }\n";
  o << "    if (lane == 0) s_cnt[0][warp] = wcnt;\n";
  o << "  }\n";
  o << "  __syncthreads();\n";
  o << "  if (warp == 0) ptotal = gx_tile_publish(a.tile_status, tile, s_cnt[0], s_off[0], GX_WARPS);\n";
  o << "  while (true) {\n";
  o << "    if (threadIdx.x == 0) s_claim = atomicAdd(a.tile_counter, 1ull);\n";
  o << "    __syncthreads();\n";
  o << "    const i64 next = (i64)s_claim;\n";
  o << "    const int npar = par ^ 1;\n";
  o << "    u32 nbal[GX_V]; u32 nwcnt = 0u;\n";
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) nbal[k] = 0u;\n";
  o << "    if (next < ntiles) {\n";
  o << "      const i64 w0 = next * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  g.decl(o, pred_ids, "      ");
  g.emit_predicate(o, "      ");
  count_conjuncts("      ");
  o << "      #pragma unroll\n      for (int k = 0; k < GX_V; k++) { nbal[k] = __ballot_sync(GX_FULL, alive[k]); nwcnt += __popc(nbal[k]); }\n";
  o << "      if (lane == 0) s_cnt[npar][warp] = nwcnt;\n";
  o << "    }\n";
  o << "    __syncthreads();\n";
  o << "    if (warp == 0) {\n";
  o << "      u64 ntotal = 0ull;\n";
  o << "      if (next < ntiles) ntotal = gx_tile_publish(a.tile_status, next, s_cnt[npar], s_off[npar], GX_WARPS);\n";
  o << "      const u64 excl = gx_lookback_resolve(a.tile_status, tile, ptotal, a.err, GX_SPINS);\n";
  o << "      if (lane == 0) {\n";
  o << "        s_base = excl;\n";
  o << "        if (tile == ntiles - 1 && excl != ~0ull) *a.out_count = excl + ptotal;\n";
  o << "      }\n";
  o << "      ptotal = ntotal;\n";
  o << "    }\n";
  o << "    __syncthreads();\n";
  o << "    const u64 base_t = s_base;\n";
  o << "    if (base_t == ~0ull) break;\n";  // look-back gave up: error already recorded
  o << "    if (wcnt != 0u) {\n";
  o << "      u64 pos = base_t + s_off[par][warp];\n";
  o << "      const i64 w0 = tile * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  emit_filter_writes_dense(o, g, p, "      ");
  o << "    }\n";
  o << "    if (next >= ntiles) break;\n";
  o << "    tile = next; par = npar; wcnt = nwcnt;\n";
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) bal[k] = nbal[k];\n";
  o << "  }\n";
  if (stats) {
    o << "  if (lane == 0) {\n";
    for (int c = 0; c < nc; c++)
      o << "    if (cst_[" << c << "]) atomicAdd(&a.conj_counts[" << c << "], (unsigned long long)cst_[" << c << "]);\n";
    o << "  }\n";
  }
  o << "}\n";
}

// Columns read by the predicate and the outputs (COPY outputs included), ascending.
std::vector<int> referenced_columns(const Plan& p) {
  std::set<int> cols, seen;
  std::function<void(int)> go = [&](int id) {
    if (id < 0 || seen.count(id)) return;
    seen.insert(id);
    const Node& n = p.nodes[id];
    if (n.kind == Node::COL) cols.insert(n.col);
    if (n.kind == Node::OP) { go(n.a); go(n.b); }
  };
  if (p.has_filter()) go(p.predicate);
  for (const auto& os : p.outputs) {
    if (os.kind == OutSpec::NODE) go(os.node);
    if (os.kind == OutSpec::COPY) cols.insert(os.col);
  }
  return std::vector<int>(cols.begin(), cols.end());
}

// Store of an output value into its shared-memory staging slot at byte
// offset `off`, with the conversion store_stmt applies to a global store.
std::string sstore_stmt(int t, const std::string& off, const std::string& bits) {
  const std::string at = "(gx_smem + " + off + ")";
  switch (t) {
    case BOOL8: return "*(unsigned char*)" + at + " = (unsigned char)((" + bits + ") != 0ull);";
    case INT8: case UINT8: return "*(unsigned char*)" + at + " = (unsigned char)(" + bits + ");";
    case INT16: case UINT16: return "*(unsigned short*)" + at + " = (unsigned short)(" + bits + ");";
    case INT32: case UINT32: case TIMESTAMP_DAYS: case DURATION_DAYS:
      return "*(unsigned*)" + at + " = (unsigned)(" + bits + ");";
    case FLOAT32: return "*(float*)" + at + " = (float)gx_D(" + bits + ");";
    default: return "*(u64*)" + at + " = (" + bits + ");";
  }
}

// kept rank t_ of the consumer warp -> its tile row, and its rank tk_ among
// the tile's kept rows
void emit_ws_rank_row(std::ostringstream& o, const std::string& in) {
  o << in << "const u32 trow = act ? (u32)s_kept_w[warp][t_] : 0u; const i64 row = tb0 + (i64)trow; const bool inr = act;"
             " (void)row; (void)inr;\n";
  o << in << "const u32 tk_ = woff + t_; (void)tk_;\n";
  o << in << "const int k = 0;\n";
}

// Projections of one consumer warp's kept rows of a tile (wcnt rows, tile
// rows in s_kept_w[warp]), computed in rounds of 32 and staged in shared
// memory at the rows' tile-level kept ranks (woff + rank): data in the output's
// slot, validity as one byte per row.  Expensive CASE branches are first
// evaluated for the warp's kept rows whose condition selects them, packed into
// full rounds (per-warp lists, no block barrier).
void emit_ws_dense(std::ostringstream& o, const Gen& g, const Plan& p, const TileLayout& L, const std::string& ind) {
  const std::vector<int> roots = g.output_roots();
  const std::vector<Gen::Lazy> lz = g.lazy_branches(roots);
  std::map<int, int> lz_root;
  std::set<int> stop;
  for (size_t i = 0; i < lz.size(); i++) {
    lz_root[lz[i].root] = (int)i;
    stop.insert(lz[i].root);
  }
  const std::vector<int> proj = g.cone_stop(roots, stop);
  const std::string i2 = ind + "  ", i3 = i2 + "  ";
  if (!lz.empty()) {
    const int nl = (int)lz.size();
    std::vector<int> conds;
    for (const auto& l : lz) conds.push_back(l.cond);
    const std::vector<int> cond_ids = g.cone(conds);
    o << ind << "u32 dmd_[" << nl << "][GX_V];\n";
    o << ind << "#pragma unroll\n" << ind << "for (int r_ = 0; r_ < GX_V; r_++) {\n";
    o << i2 << "#pragma unroll\n" << i2 << "for (int l_ = 0; l_ < " << nl << "; l_++) dmd_[l_][r_] = 0u;\n";
    o << i2 << "if ((u32)r_ * 32u < wcnt) {\n";
    o << i3 << "const u32 t_ = (u32)r_ * 32u + (u32)lane; const bool act = t_ < wcnt;\n";
    emit_ws_rank_row(o, i3);
    emit_row_nodes(o, g, p, cond_ids, {}, i3);
    for (int i = 0; i < nl; i++) {
      const int c = lz[i].cond;
      o << i3 << "dmd_[" << i << "][r_] = __ballot_sync(GX_FULL, act && (" << g.V(c) << " && " << g.nz(c) << "));\n";
    }
    o << i2 << "}\n";
    o << ind << "}\n";
    for (int i = 0; i < nl; i++) {
      o << ind << "{\n";
      o << i2 << "u32 dtot_ = 0u;\n";
      o << i2 << "#pragma unroll\n" << i2 << "for (int r_ = 0; r_ < GX_V; r_++) {\n";
      o << i3 << "const u32 db_ = dmd_[" << i << "][r_];\n";
      o << i3 << "if ((db_ >> lane) & 1u) s_dem_[warp][dtot_ + __popc(db_ & ((1u << lane) - 1u))] = "
                 "(unsigned short)(r_ * 32 + lane);\n";
      o << i3 << "dtot_ += __popc(db_);\n";
      o << i2 << "}\n";
      o << i2 << "__syncwarp();\n";
      o << i2 << "for (u32 db_ = 0; db_ < dtot_; db_ += 32u) {\n";
      o << i3 << "const u32 q_ = db_ + (u32)lane; const bool act = q_ < dtot_;\n";
      o << i3 << "const u32 t_ = act ? (u32)s_dem_[warp][q_] : 0u;\n";
      emit_ws_rank_row(o, i3);
      emit_row_nodes(o, g, p, lz[i].nodes, {}, i3);
      o << i3 << "if (act) { s_lzb_[" << i << "][warp][t_] = " << g.B(lz[i].root) << "; s_lzv_[" << i
        << "][warp][t_] = " << g.V(lz[i].root) << " ? 1 : 0; }\n";
      o << i2 << "}\n";
      o << i2 << "__syncwarp();\n";  // s_dem_ is rewritten for the next branch
      o << ind << "}\n";
    }
  }
  o << ind << "for (u32 base_ = 0; base_ < wcnt; base_ += 32u) {\n";
  o << i2 << "const u32 t_ = base_ + (u32)lane; const bool act = t_ < wcnt;\n";
  emit_ws_rank_row(o, i2);
  emit_row_nodes(o, g, p, proj, lz_root, i2);
  for (size_t j = 0; j < p.outputs.size(); j++) {
    const OutSpec& os = p.outputs[j];
    if (os.kind == OutSpec::BROADCAST) continue;
    const std::string w = std::to_string(L.out_width[j]);
    const std::string doff = "ost + " + std::to_string(L.out_off[j]) + "u + tk_ * " + w + "u";
    const std::string voff = "ost + " + std::to_string(L.out_valid_off[j]) + "u + tk_";
    if (os.kind == OutSpec::NODE) {
      o << i2 << "if (act) { " << sstore_stmt(os.type, doff, g.B(os.node)) << " gx_smem[" << voff << "] = "
        << g.V(os.node) << " ? 1 : 0; }\n";
    } else {
      const int c = os.col;
      const std::string cs = std::to_string(c), rt = raw_type(p.schema[c]);
      const std::string vexpr = p.nullable[c] ? "((vmw_" + cs + "[trow >> 5] >> (trow & 31u)) & 1u)" : "1u";
      o << i2 << "if (act) { *(" << rt << "*)(gx_smem + " << doff << ") = *(const " << rt << "*)(gx_smem + sd_" << cs
        << " + trow * " << w << "u); gx_smem[" << voff << "] = (unsigned char)" << vexpr << "; }\n";
    }
  }
  o << ind << "}\n";
}

// Write-out of a tile's staged outputs (K_w rows at output rows base_w..) by
// every consumer warp: data element by element (coalesced), validity words
// rebuilt from the staged bytes by ballots; the first and last words of the
// tile's range may be shared with the neighbouring tiles and are OR-ed in
// atomically (the masks were zeroed before the launch).
void emit_ws_writeout(std::ostringstream& o, const Plan& p, const TileLayout& L, const std::string& ind) {
  const std::string i2 = ind + "  ";
  o << ind << "const u32 tid_ = (u32)warp * 32u + (u32)lane;\n";
  for (size_t j = 0; j < p.outputs.size(); j++) {
    if (p.outputs[j].kind == OutSpec::BROADCAST) continue;
    const std::string rt = raw_type(p.outputs[j].kind == OutSpec::COPY ? p.schema[p.outputs[j].col] : p.outputs[j].type);
    o << ind << "for (u32 t = tid_; t < K_w; t += GX_WARPS * 32u) {\n";
    o << i2 << "const i64 orow = (i64)base_w + (i64)t;\n";
    o << i2 << "if (orow < a.capacity) __stcs((" << rt << "*)a.out_data[" << j << "] + orow, *(const " << rt
      << "*)(gx_smem + osw + " << L.out_off[j] << "u + t * " << L.out_width[j] << "u));\n";
    o << ind << "}\n";
  }
  o << ind << "const u32 bf_ = (u32)(base_w & 31ull); const u32 nw_ = K_w ? (bf_ + K_w + 31u) >> 5 : 0u;\n";
  o << ind << "const i64 w0_ = (i64)(base_w >> 5); const i64 cap_words = (a.capacity + 31) >> 5;\n";
  o << ind << "for (u32 kw = (u32)warp; kw < nw_; kw += GX_WARPS) {\n";
  o << i2 << "const int t = (int)(kw * 32u + (u32)lane) - (int)bf_;\n";
  o << i2 << "const bool in_ = t >= 0 && (u32)t < K_w;\n";
  o << i2 << "const bool shared_ = (kw == 0u && bf_ != 0u) || kw + 1u == nw_;\n";
  for (size_t j = 0; j < p.outputs.size(); j++) {
    if (p.outputs[j].kind == OutSpec::BROADCAST) continue;
    o << i2 << "{ const u32 word_ = __ballot_sync(GX_FULL, in_ && gx_smem[osw + " << L.out_valid_off[j]
      << "u + (u32)(in_ ? t : 0)] != 0);\n";
    o << i2 << "  if (lane == 0 && w0_ + (i64)kw < cap_words) { if (shared_) atomicOr(a.out_mask[" << j
      << "] + w0_ + kw, word_); else a.out_mask[" << j << "][w0_ + kw] = word_; } }\n";
  }
  o << ind << "}\n";
}

// Tile-staged fused filter + project (single pass, stable order), with the
// warps of a block in three roles.
//
//  * warp 0 (producer): claims tiles in order from the ticket and, for each,
//    issues one bulk copy per column (its data bytes, and its mask words when
//    it has a mask) into the next free stage of a GX_NS-stage ring in shared
//    memory, completing on the stage's "full" mbarrier; it reuses a stage once
//    every consumer warp has arrived on the stage's "empty" mbarrier.
//  * warp 1 (resolver): for each tile, once the consumers have published its
//    aggregate and the block's next tile has been counted too, resolves its
//    output offset by decoupled look-back -- a 256-wide window per poll that
//    stops at the block's previous tile, whose inclusive prefix it already
//    has -- and hands it back through a "based" mbarrier.
//  * warps 2.. (consumers): slot j of their loop evaluates the predicate of
//    the block's j-th tile from shared memory (lane per row; the mask words are
//    first re-aligned to the tile's rows), lists each warp's kept rows, meets
//    at one named barrier to total the tile (one thread publishes the
//    aggregate and passes it to the resolver); then computes the projections
//    of the (j-1)-th tile's kept rows into a ring of shared-memory output
//    staging buffers and releases that tile's stage; then writes the
//    (j - GX_NR)-th tile's staged outputs to their final rows.
//
// A block thus publishes its newest aggregate before it waits on any
// look-back, and a tile's look-back waits only on earlier tiles, so the kernel
// cannot deadlock.  Every wait is bounded: a look-back that gives up records
// error 1 (the block goes on without writing that tile); a copy or hand-over
// wait that gives up records error 2, and the consumers wait (bounded) for the
// copies still in flight to land before the block returns.
void emit_fused_tma(std::ostringstream& o, const Gen& g, const Plan& p, const TileLayout& L, const std::string& name) {
  g.tile_mode_ = true;
  const std::vector<int> pred_ids = g.predicate_cone();
  const std::vector<Gen::Lazy> lz = g.lazy_branches(g.output_roots());
  const int nl = (int)lz.size();
  o << "#undef GX_LB\n#define GX_LB __launch_bounds__((GX_WARPS + 2) * 32)\n";
  o << "#define GX_TR " << L.tile_rows << "\n#define GX_NS " << L.stages << "\n#define GX_STAGE " << L.stage_bytes
    << "u\n#define GX_OBASE " << L.out_base << "u\n#define GX_OSTAGE " << L.out_stage_bytes << "u\n#define GX_NR "
    << L.out_stages << "\n#define GX_RR (GX_NR + 1)\n";
  o << "#define GX_WAIT (1u << 21)\n";
  // the copies of one tile into the stage at shared address stg
  o << "__device__ __forceinline__ void gx_issue_tile_(const GxArgs& a, long long t, u32 stg, u64* bar) {\n";
  o << "  const i64 r0 = (i64)t * GX_TR; const i64 r1 = min(a.n, r0 + (i64)GX_TR);\n";
  for (size_t i = 0; i < L.cols.size(); i++) {
    const int c = L.cols[i];
    const std::string cs = std::to_string(c), w = std::to_string(type_size(p.schema[c]));
    o << "  const u64 lo" << cs << " = (u64)a.in_data[" << cs << "] + (u64)(a.in_off[" << cs << "] + r0) * " << w
      << "ull, hi" << cs << " = (u64)a.in_data[" << cs << "] + (u64)(a.in_off[" << cs << "] + r1) * " << w << "ull;\n";
    if (L.mask_off[i] != UINT32_MAX)
      o << "  const u64 mlo" << cs << " = (u64)(a.in_mask[" << cs << "] + ((a.in_off[" << cs << "] + r0) >> 5)), mhi"
        << cs << " = (u64)(a.in_mask[" << cs << "] + ((a.in_off[" << cs << "] + r1 - 1) >> 5) + 1);\n";
  }
  o << "  u32 tot = 0u;\n";
  for (size_t i = 0; i < L.cols.size(); i++) {
    const std::string cs = std::to_string(L.cols[i]);
    o << "  tot += gx_bulk_span(0u, lo" << cs << ", hi" << cs << ", bar, false);\n";
    if (L.mask_off[i] != UINT32_MAX) o << "  tot += gx_bulk_span(0u, mlo" << cs << ", mhi" << cs << ", bar, false);\n";
  }
  o << "  gx_mbar_arrive_tx(bar, tot);\n";
  for (size_t i = 0; i < L.cols.size(); i++) {
    const std::string cs = std::to_string(L.cols[i]);
    o << "  gx_bulk_span(stg + " << L.data_off[i] << "u, lo" << cs << ", hi" << cs << ", bar, true);\n";
    if (L.mask_off[i] != UINT32_MAX)
      o << "  gx_bulk_span(stg + " << L.mask_off[i] << "u, mlo" << cs << ", mhi" << cs << ", bar, true);\n";
  }
  o << "}\n";

  o << "extern \"C\" __global__ void GX_LB " << name << "(const GxArgs a) {\n";
  o << "  const int lane = threadIdx.x & 31; const int wid_ = threadIdx.x >> 5;\n";
  o << "  const i64 ntiles = (a.n + GX_TR - 1) / GX_TR;\n";
  o << "  __shared__ __align__(8) u64 s_full_[GX_NS];\n";
  o << "  __shared__ __align__(8) u64 s_empty_[GX_NS];\n";
  o << "  __shared__ __align__(8) u64 s_counted_[GX_RR];\n";
  o << "  __shared__ __align__(8) u64 s_based_[GX_RR];\n";
  o << "  __shared__ long long s_tile_[GX_NS];\n";
  o << "  __shared__ long long s_rtile_[GX_RR];\n";
  o << "  __shared__ u64 s_ragg_[GX_RR];\n";
  o << "  __shared__ u64 s_base_[GX_RR];\n";
  o << "  __shared__ u32 s_cnt_[2][GX_WARPS];\n";
  o << "  __shared__ unsigned short s_kept_[2][GX_WARPS][GX_V * 32];\n";
  if (L.num_masked > 0) o << "  __shared__ u32 s_vm_[2][" << L.num_masked << "][GX_TR / 32];\n";
  if (nl > 0) {
    o << "  __shared__ unsigned short s_dem_[GX_WARPS][GX_V * 32];\n";
    o << "  __shared__ u64 s_lzb_[" << nl << "][GX_WARPS][GX_V * 32];\n";
    o << "  __shared__ unsigned char s_lzv_[" << nl << "][GX_WARPS][GX_V * 32];\n";
  }
  o << "  const u32 smem0_ = gx_saddr(gx_smem);\n";
  // bulk copies land on 16-byte boundaries of the dynamic shared memory
  o << "  if ((smem0_ & 15u) != 0u) { if (threadIdx.x == 0) atomicExch(a.err, 3); return; }\n";
  o << "  if (threadIdx.x == 0) {\n";
  o << "    for (int q = 0; q < GX_NS; q++) { gx_mbar_init(&s_full_[q], 1u); gx_mbar_init(&s_empty_[q], GX_WARPS); }\n";
  o << "    for (int q = 0; q < GX_RR; q++) { gx_mbar_init(&s_counted_[q], 1u); gx_mbar_init(&s_based_[q], 1u); }\n";
  o << "    gx_mbar_init_fence();\n";
  o << "  }\n";
  o << "  __syncthreads();\n";
  // ---- producer
  o << "  if (wid_ == 0) {\n";
  o << "    if (lane == 0) {\n";
  o << "      for (int j = 0; ; j++) {\n";
  o << "        const int q = j % GX_NS;\n";
  o << "        if (j >= GX_NS && !gx_mbar_wait(&s_empty_[q], (u32)(j / GX_NS - 1) & 1u, GX_WAIT)) {\n";
  o << "          atomicExch(a.err, 2);\n";
  o << "          break;\n";
  o << "        }\n";
  o << "        long long t = (long long)atomicAdd(a.tile_counter, 1ull);\n";
  o << "        if (t >= ntiles) t = -1;\n";
  o << "        s_tile_[q] = t;\n";
  o << "        if (t < 0) { gx_mbar_arrive(&s_full_[q]); break; }\n";
  o << "        gx_fence_async_smem();\n";
  o << "        gx_issue_tile_(a, t, smem0_ + (u32)q * GX_STAGE, &s_full_[q]);\n";
  o << "      }\n";
  o << "    }\n";
  o << "    return;\n";
  o << "  }\n";
  // ---- resolver
  o << "  if (wid_ == 1) {\n";
  o << "    long long tk = -1; u64 pk = 0ull;\n";  // the block's last resolved tile and its inclusive prefix
  o << "    for (int j = 0; ; j++) {\n";
  o << "      const int b = j % GX_RR;\n";
  o << "      if (!gx_mbar_wait(&s_counted_[b], (u32)(j / GX_RR) & 1u, GX_WAIT)) {\n";
  o << "        if (lane == 0) atomicExch(a.err, 2);\n";
  o << "        return;\n";
  o << "      }\n";
  o << "      const long long t = s_rtile_[b]; const u64 agg = s_ragg_[b];\n";
  o << "      if (t < 0) return;\n";
  // start once the block's next tile is counted too: by then the tiles other
  // blocks claimed before this one have mostly published their aggregates
  o << "      gx_mbar_wait(&s_counted_[(j + 1) % GX_RR], (u32)((j + 1) / GX_RR) & 1u, GX_WAIT);\n";
  o << "      const u64 ex = gx_lookback_wide<8>(a.tile_status, t, agg, a.err, GX_SPINS, tk, pk);\n";
  o << "      if (ex != ~0ull) { tk = t; pk = ex + agg; } else { tk = -1; pk = 0ull; }\n";
  o << "      if (lane == 0) {\n";
  o << "        s_base_[b] = ex;\n";
  o << "        if (t == ntiles - 1 && ex != ~0ull) *a.out_count = ex + agg;\n";
  o << "        gx_mbar_arrive(&s_based_[b]);\n";
  o << "      }\n";
  o << "      __syncwarp();\n";
  o << "    }\n";
  o << "  }\n";
  // ---- consumers
  o << "  const int warp = wid_ - 2;\n";
  // per-column shifts: the byte of element 0 within its 16-byte block, and
  // for masks the byte of the first word within its block and the bit of row
  // 0 within that word -- the same for every tile (tiles are multiples of 128 rows)
  for (size_t i = 0; i < L.cols.size(); i++) {
    const int c = L.cols[i];
    const std::string cs = std::to_string(c);
    o << "  const u32 h_" << cs << " = (u32)(((u64)a.in_data[" << cs << "] + (u64)a.in_off[" << cs << "] * "
      << type_size(p.schema[c]) << "ull) & 15ull);\n";
    if (L.mask_off[i] != UINT32_MAX) {
      o << "  const u32 mh_" << cs << " = (u32)((u64)(a.in_mask[" << cs << "] + (a.in_off[" << cs << "] >> 5)) & 15ull);\n";
      o << "  const u32 ms_" << cs << " = (u32)(a.in_off[" << cs << "] & 31);\n";
    }
  }
  o << "  long long tile_p = -1; u32 wcnt_p = 0u, woff_p = 0u;\n";  // the (j-1)-th tile, awaiting its projections
  o << "  for (int j = 0; ; j++) {\n";
  o << "    const int q = j % GX_NS; const int vp = j & 1; const int rr = j % GX_RR;\n";
  o << "    const bool ok_ = gx_mbar_wait(&s_full_[q], (u32)(j / GX_NS) & 1u, GX_WAIT);\n";
  o << "    const long long tile = ok_ ? s_tile_[q] : -1;\n";
  o << "    u32 wcnt = 0u;\n";
  o << "    if (tile >= 0) {\n";
  o << "      const i64 tb0 = (i64)tile * GX_TR; const int wl0 = warp * GX_V;\n";
  o << "      const u32 stg = (u32)q * GX_STAGE;\n";
  for (size_t i = 0; i < L.cols.size(); i++) {
    const std::string cs = std::to_string(L.cols[i]);
    o << "      const u32 sd_" << cs << " = stg + " << L.data_off[i] << "u + h_" << cs << "; (void)sd_" << cs << ";\n";
    if (L.mask_off[i] != UINT32_MAX) {
      o << "      const u32* vmw_" << cs << " = s_vm_[vp][" << L.mask_index[i] << "]; (void)vmw_" << cs << ";\n";
      o << "      if (lane < GX_V) {\n";
      o << "        const u32 wk_ = (u32)(wl0 + lane);\n";
      o << "        const u32* raw_ = (const u32*)(gx_smem + stg + " << L.mask_off[i] << "u + mh_" << cs << ");\n";
      o << "        s_vm_[vp][" << L.mask_index[i] << "][wk_] = __funnelshift_r(raw_[wk_], raw_[wk_ + 1], ms_" << cs
        << ");\n";
      o << "      }\n";
    }
  }
  o << "      __syncwarp();\n";
  o << "      const i64 w0 = (i64)tile * GX_TILE_WORDS + wl0;\n";
  g.decl(o, pred_ids, "      ");
  g.emit_predicate(o, "      ");
  o << "      u32 r_ = 0u;\n";
  o << "      #pragma unroll\n      for (int k = 0; k < GX_V; k++) {\n";
  o << "        const u32 bk_ = __ballot_sync(GX_FULL, alive[k]);\n";
  o << "        if ((bk_ >> lane) & 1u) s_kept_[vp][warp][r_ + __popc(bk_ & ((1u << lane) - 1u))] = "
       "(unsigned short)((wl0 + k) * 32 + lane);\n";
  o << "        r_ += __popc(bk_);\n";
  o << "      }\n";
  o << "      wcnt = r_;\n";
  o << "      __syncwarp();\n";
  o << "    }\n";
  o << "    if (lane == 0) s_cnt_[vp][warp] = wcnt;\n";
  o << "    if (!gx_bar_and(ok_, GX_WARPS * 32)) {\n";
  // a copy never landed: wait (bounded) for the copies in flight, then leave
  o << "      if (warp == 0 && lane == 0) atomicExch(a.err, 2);\n";
  o << "      for (int d_ = 0; d_ < GX_NS; d_++) gx_mbar_wait(&s_full_[(j + d_) % GX_NS], (u32)((j + d_) / GX_NS) & 1u, "
       "GX_WAIT);\n";
  o << "      return;\n";
  o << "    }\n";
  o << "    u32 tot_ = 0u, woff = 0u;\n";
  o << "    if (tile >= 0) woff = gx_block_excl(s_cnt_[vp], GX_WARPS, &tot_, warp);\n";
  o << "    if (warp == 0 && lane == 0) {\n";
  o << "      if (tile >= 0) gx_st_release(a.tile_status + tile, (tile == 0 ? GX_ST_PFX : GX_ST_AGG) | (u64)tot_);\n";
  o << "      s_rtile_[rr] = tile; s_ragg_[rr] = (u64)tot_;\n";
  o << "      gx_mbar_arrive(&s_counted_[rr]);\n";
  o << "    }\n";
  // projections of the previous slot's tile
  o << "    if (tile_p >= 0) {\n";
  o << "      const int jp = j - 1; const int qp = jp % GX_NS; const int pp = jp & 1;\n";
  o << "      const u32 ost = GX_OBASE + (u32)(jp % GX_NR) * GX_OSTAGE;\n";
  o << "      const u32 wcnt = wcnt_p, woff = woff_p;\n";
  o << "      const i64 tb0 = (i64)tile_p * GX_TR;\n";
  o << "      const u32 stg = (u32)qp * GX_STAGE;\n";
  o << "      const unsigned short (*s_kept_w)[GX_V * 32] = s_kept_[pp];\n";
  for (size_t i = 0; i < L.cols.size(); i++) {
    const std::string cs = std::to_string(L.cols[i]);
    o << "      const u32 sd_" << cs << " = stg + " << L.data_off[i] << "u + h_" << cs << "; (void)sd_" << cs << ";\n";
    if (L.mask_off[i] != UINT32_MAX)
      o << "      const u32* vmw_" << cs << " = s_vm_[pp][" << L.mask_index[i] << "]; (void)vmw_" << cs << ";\n";
  }
  emit_ws_dense(o, g, p, L, "      ");
  o << "      __syncwarp();\n";
  o << "      if (lane == 0) gx_mbar_arrive(&s_empty_[qp]);\n";
  o << "    }\n";
  // after the last tile every staged tile is written out, the one just
  // projected included: all consumer warps must have staged it first
  o << "    if (tile < 0) gx_bar_and(true, GX_WARPS * 32);\n";
  o << "    for (int jw = j - GX_NR; jw <= (tile >= 0 ? j - GX_NR : j - 1); jw++) {\n";
  o << "      if (jw < 0) continue;\n";
  o << "      const int pr = jw % GX_RR;\n";
  o << "      if (s_rtile_[pr] < 0) continue;\n";
  o << "      const bool okb = gx_mbar_wait(&s_based_[pr], (u32)(jw / GX_RR) & 1u, GX_WAIT);\n";
  o << "      if (!okb && warp == 0 && lane == 0) atomicExch(a.err, 2);\n";
  o << "      const u64 base_w = okb ? s_base_[pr] : ~0ull;\n";
  o << "      if (base_w != ~0ull) {\n";
  o << "        const u32 K_w = (u32)s_ragg_[pr]; const u32 osw = GX_OBASE + (u32)(jw % GX_NR) * GX_OSTAGE;\n";
  emit_ws_writeout(o, p, L, "        ");
  o << "      }\n";
  o << "    }\n";
  o << "    if (tile < 0) break;\n";
  o << "    tile_p = tile; wcnt_p = wcnt; woff_p = woff;\n";
  o << "  }\n";
  o << "}\n";
  g.tile_mode_ = false;
}

// Batched persistent form of the pipelined fused filter: one launch runs a
// whole table of batches (GxArgs per batch).  Batch b owns the tiles
// [tile_base[b], tile_base[b + 1]) of one tile sequence that blocks claim in
// order from one counter; every batch has its own look-back segment and row
// counter, so a block's pending and next tiles may belong to different
// batches, and each batch's result is exactly that of running it alone.
// (streaming: the host appends batches while the kernel runs -- descriptors,
// tile offsets, then the published tile count, each by an ordered copy -- and
// closes the queue by setting hdr->pad; a block that claims a tile past the
// published count waits for it (bounded: `wait_polls` polls 2 us apart, then
// *werr = 1) or, once the queue is closed without it, stops.  Tile offsets of
// unpublished batches hold INT64_MAX, so a lookup never passes the last
// published batch.)
void emit_fused_batched(std::ostringstream& o, const Gen& g, const Plan& p, const std::vector<int>& pred_ids,
                        const std::string& name, bool streaming = false) {
  o << "struct GxBatchHdr { unsigned long long tile_counter; long long total_tiles; int nbatch; int pad; };\n";
  // a batch's descriptor: streaming descriptors sit kArgsStride bytes apart,
  // so that no cache line holds two of them (one is written while the kernel
  // may have read its neighbour)
  if (streaming)
    o << "#define GX_BATCH(b) (*(const GxArgs*)((const char*)A + (size_t)(b) * " << kStreamArgsStride << "u))\n";
  else
    o << "#define GX_BATCH(b) (A[(b)])\n";
  if (streaming) {
    o << "extern \"C\" __global__ void GX_LB " << name
      << "(const GxArgs* A, const volatile long long* tile_base, GxBatchHdr* hdr, int* werr, unsigned wait_polls) {\n";
    o << "  const int nbatch = 0x7fffffff; (void)nbatch;\n";
    // claim a tile; -1 once the queue is closed below it (or the wait gave up)
    o << "  auto claim_ = [&]() -> long long {\n";
    o << "    long long t = (long long)atomicAdd(&hdr->tile_counter, 1ull);\n";
    o << "    unsigned polls = 0;\n";
    o << "    while (true) {\n";
    o << "      if (t < *(volatile long long*)&hdr->total_tiles) break;\n";
    o << "      if (*(volatile int*)&hdr->pad != 0) {\n";  // closed: the published count is final
    o << "        if (t < *(volatile long long*)&hdr->total_tiles) break;\n";
    o << "        return -1;\n";
    o << "      }\n";
    o << "      if (*(volatile int*)werr != 0) return -1;\n";
    o << "      if (++polls > wait_polls) { atomicExch(werr, 1); return -1; }\n";
    o << "      __nanosleep(2000);\n";
    o << "    }\n";
    o << "    __threadfence();\n";  // the batch's descriptor and tile offsets were copied before its tiles were published
    o << "    return t;\n";
    o << "  };\n";
  } else {
    o << "extern \"C\" __global__ void GX_LB " << name
      << "(const GxArgs* __restrict__ A, const long long* __restrict__ tile_base, GxBatchHdr* hdr) {\n";
    o << "  const i64 total_tiles = hdr->total_tiles; const int nbatch = hdr->nbatch;\n";
  }
  o << "  const int lane = threadIdx.x & 31; const int warp = threadIdx.x >> 5;\n";
  o << "  __shared__ unsigned long long s_claim;\n";
  o << "  __shared__ u32 s_cnt[2][GX_WARPS];\n";
  o << "  __shared__ u64 s_off[2][GX_WARPS];\n";
  o << "  __shared__ u64 s_base;\n";
  if (streaming) {
    o << "  if (threadIdx.x == 0) s_claim = (unsigned long long)claim_();\n";
    o << "  __syncthreads();\n";
    o << "  const i64 gt0 = (i64)s_claim;\n";
    o << "  if (gt0 < 0) return;\n";
  } else {
    o << "  if (threadIdx.x == 0) s_claim = atomicAdd(&hdr->tile_counter, 1ull);\n";
    o << "  __syncthreads();\n";
    o << "  const i64 gt0 = (i64)s_claim;\n";
    o << "  if (gt0 >= total_tiles) return;\n";
  }
  o << "  int pb = 0;\n";
  o << "  while (pb + 1 < nbatch && tile_base[pb + 1] <= gt0) pb++;\n";
  o << "  i64 tile = gt0 - tile_base[pb];\n";
  o << "  u32 bal[GX_V]; u32 wcnt = 0u; int par = 0; u64 ptotal = 0ull;\n";
  o << "  {\n";
  o << "    const GxArgs& a = GX_BATCH(pb);\n";
  o << "    const i64 w0 = tile * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  g.decl(o, pred_ids, "    ");
  g.emit_predicate(o, "    ");
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) { bal[k] = __ballot_sync(GX_FULL, alive[k]); wcnt += __popc(bal[k]); }\n";
  o << "    if (lane == 0) s_cnt[0][warp] = wcnt;\n";
  o << "  }\n";
  o << "  __syncthreads();\n";
  o << "  if (warp == 0) ptotal = gx_tile_publish(GX_BATCH(pb).tile_status, tile, s_cnt[0], s_off[0], GX_WARPS);\n";
  o << "  while (true) {\n";
  if (streaming) o << "    if (threadIdx.x == 0) s_claim = (unsigned long long)claim_();\n";
  else o << "    if (threadIdx.x == 0) s_claim = atomicAdd(&hdr->tile_counter, 1ull);\n";
  o << "    __syncthreads();\n";
  o << "    const i64 ngt = (i64)s_claim;\n";
  o << "    int nb = pb; i64 next = -1;\n";
  o << "    if (" << (streaming ? "ngt >= 0" : "ngt < total_tiles") << ") {\n";
  o << "      while (nb + 1 < nbatch && tile_base[nb + 1] <= ngt) nb++;\n";
  o << "      next = ngt - tile_base[nb];\n";
  o << "    }\n";
  o << "    const int npar = par ^ 1;\n";
  o << "    u32 nbal[GX_V]; u32 nwcnt = 0u;\n";
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) nbal[k] = 0u;\n";
  o << "    if (next >= 0) {\n";
  o << "      const GxArgs& a = GX_BATCH(nb);\n";
  o << "      const i64 w0 = next * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  g.decl(o, pred_ids, "      ");
  g.emit_predicate(o, "      ");
  o << "      #pragma unroll\n      for (int k = 0; k < GX_V; k++) { nbal[k] = __ballot_sync(GX_FULL, alive[k]); nwcnt += __popc(nbal[k]); }\n";
  o << "      if (lane == 0) s_cnt[npar][warp] = nwcnt;\n";
  o << "    }\n";
  o << "    __syncthreads();\n";
  o << "    if (warp == 0) {\n";
  o << "      u64 ntotal = 0ull;\n";
  o << "      if (next >= 0) ntotal = gx_tile_publish(GX_BATCH(nb).tile_status, next, s_cnt[npar], s_off[npar], GX_WARPS);\n";
  o << "      const GxArgs& a = GX_BATCH(pb);\n";
  o << "      const i64 ntiles = (((a.n + 31) >> 5) + GX_TILE_WORDS - 1) / GX_TILE_WORDS;\n";
  o << "      const u64 excl = gx_lookback_resolve(a.tile_status, tile, ptotal, a.err, GX_SPINS);\n";
  o << "      if (lane == 0) {\n";
  o << "        s_base = excl;\n";
  o << "        if (tile == ntiles - 1 && excl != ~0ull) *a.out_count = excl + ptotal;\n";
  o << "      }\n";
  o << "      ptotal = ntotal;\n";
  o << "    }\n";
  o << "    __syncthreads();\n";
  o << "    const u64 base_t = s_base;\n";
  o << "    if (base_t == ~0ull) break;\n";  // look-back gave up: error already recorded
  o << "    if (wcnt != 0u) {\n";
  o << "      const GxArgs& a = GX_BATCH(pb);\n";
  o << "      u64 pos = base_t + s_off[par][warp];\n";
  o << "      const i64 w0 = tile * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  emit_filter_writes_dense(o, g, p, "      ");
  o << "    }\n";
  o << "    if (next < 0) break;\n";
  o << "    tile = next; pb = nb; par = npar; wcnt = nwcnt;\n";
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) bal[k] = nbal[k];\n";
  o << "  }\n";
  o << "}\n";
}

// Staged short-circuit filter (runtime conjunct order, dense projections).
// Each block keeps GX_D tiles in flight.  A tile's conjuncts are evaluated one
// at a time in the launch order; before each step, warp 0 copies the 32-row
// words of that conjunct's columns that still have a live row into the tile's
// shared-memory slot with asynchronous copies (completion on the slot's
// mbarrier) and the block moves on to the next slot, so the copies of several
// tiles are in flight while it evaluates one.  (Bulk copies of one 256-byte
// word each were measured an order of magnitude slower than 16-byte
// asynchronous copies spread over the warp: small bulk copies serialise.)  A tile whose rows are all dead, or that has
// passed every conjunct, publishes its aggregate at once; tiles are resolved
// (look-back) and written in claim order, so a block never waits on one of its
// own unpublished tiles.  A partial last word is read from global memory
// directly.  Every column a conjunct reads must start on a 16-byte boundary
// (the host checks and otherwise runs the unstaged kernel).
void emit_staged_filter(std::ostringstream& o, const Gen& g, const Plan& p, const std::string& name) {
  const int nc = (int)p.conjuncts.size();
  std::vector<std::vector<int>> cc(nc);
  std::vector<std::vector<int>> coff(nc);  // byte offset of each column's region in a slot, per word
  std::vector<int> cwb(nc, 0);             // bytes per word of all the conjunct's columns
  int wbmax = 16;
  for (int c = 0; c < nc; c++) {
    cc[c] = conjunct_columns(p, c);
    for (int col : cc[c]) {
      coff[c].push_back(cwb[c]);
      cwb[c] += 32 * type_size(p.schema[col]);
    }
    wbmax = std::max(wbmax, cwb[c]);
  }
  o << "#define GX_T (GX_WARPS * GX_V)\n#define GX_D 4\n";
  o << "extern \"C\" __global__ void GX_LB " << name << "(const GxArgs a) {\n";
  o << "  const int lane = threadIdx.x & 31; const int warp = threadIdx.x >> 5;\n";
  o << "  const i64 nwords = (a.n + 31) >> 5;\n";
  o << "  const i64 ntiles = (nwords + GX_T - 1) / GX_T;\n";
  // slot layout for conjunct c: column i's words at GX_T * coff[c][i] + kw * 32 * w
  o << "  __shared__ __align__(128) unsigned char s_buf[GX_D][GX_T * " << wbmax << "];\n";
  o << "  __shared__ __align__(8) u64 s_bar[GX_D];\n";
  o << "  __shared__ long long s_tile[GX_D];\n";
  o << "  __shared__ int s_step[GX_D], s_done[GX_D], s_pend[GX_D], s_seq[GX_D];\n";
  o << "  __shared__ u32 s_par[GX_D];\n";
  o << "  __shared__ u32 s_alive[GX_D][GX_T];\n";
  o << "  __shared__ u32 s_cnt[GX_WARPS];\n";
  o << "  __shared__ u64 s_off[GX_D][GX_WARPS];\n";
  o << "  __shared__ u64 s_total[GX_D];\n";
  o << "  __shared__ u64 s_base;\n";
  o << "  __shared__ int s_cseq, s_rseq, s_abort, s_ready;\n";
  o << "  __shared__ long long s_lbpred;\n";   // look-back progress of the oldest tile
  o << "  __shared__ u64 s_lbexcl;\n";
  o << "  __shared__ u32 s_lbpolls;\n";
  o << "  const u32 spin_limit = 1u << 22;\n";
  o << "  const u32 mbar_limit = 1u << 20;  // polls of a slot's barrier (each try_wait may suspend briefly)\n";

  // warp 0: copies of conjunct order[step]'s live full words of slot s, as
  // 16-byte asynchronous copies spread over the warp's lanes; every lane then
  // arrives on the slot's barrier when its copies have landed (32 arrivals)
  o << "  auto issue_ = [&](int s, long long tile, int step) {\n";
  o << "    const int cj = a.order_dev ? __ldg(a.order_dev + step) : a.order[step];\n";
  o << "    int nwt_ = 0;\n";
  o << "    for (int kb = 0; kb < GX_T; kb += 32) {\n";
  o << "      const int kw = kb + lane;\n";
  o << "      const i64 wd = tile * GX_T + kw;\n";
  o << "      nwt_ += __popc(__ballot_sync(GX_FULL, kw < GX_T && s_alive[s][kw] != 0u && (wd + 1) * 32 <= a.n));\n";
  o << "    }\n";
  o << "    if (lane == 0) s_pend[s] = nwt_ != 0 ? 1 : 0;\n";
  o << "    if (nwt_ == 0) return;\n";
  o << "    gx_fence_async_smem();\n";
  o << "    for (int kb = 0; kb < GX_T; kb += 32) {\n";
  o << "      const int kwl = kb + lane;\n";
  o << "      const u32 wm_ = __ballot_sync(GX_FULL, kwl < GX_T && s_alive[s][kwl] != 0u && (tile * GX_T + kwl + 1) * 32 <= a.n);\n";
  o << "      const int nw_ = __popc(wm_);\n";
  o << "      switch (cj) {\n";
  for (int c = 0; c < nc; c++) {
    const int ch = cwb[c] / 16;  // 16-byte chunks per word, all the conjunct's columns
    o << "        case " << c << ":\n";
    o << "          for (int q = lane; q < nw_ * " << ch << "; q += 32) {\n";
    o << "            const int kw = kb + (int)__fns(wm_, 0u, q / " << ch << " + 1);\n";
    o << "            const int ck = q % " << ch << ";\n";
    o << "            const i64 wd = tile * GX_T + kw;\n";
    int chk = 0;
    for (size_t i = 0; i < cc[c].size(); i++) {
      const int col = cc[c][i];
      const int w = type_size(p.schema[col]);
      const int cn = 2 * w;  // chunks of this column per word (32 * w / 16)
      o << "            " << (i ? "else " : "") << "if (ck < " << chk + cn << ") gx_cp16(s_buf[s] + GX_T * " << coff[c][i]
        << " + kw * " << 32 * w << " + (ck - " << chk << ") * 16, (const char*)a.in_data[" << col << "] + (a.in_off["
        << col << "] + wd * 32) * " << w << " + (ck - " << chk << ") * 16);\n";
      chk += cn;
    }
    o << "          }\n";
    o << "          break;\n";
  }
  o << "        default: break;\n      }\n    }\n";
  o << "    gx_cp_arrive(&s_bar[s]);\n";
  o << "  };\n";

  // thread 0: claim the next tile into slot s; returns whether one was claimed
  o << "  auto claim_ = [&](int s) {\n";
  o << "    const long long t = (long long)atomicAdd(a.tile_counter, 1ull);\n";
  o << "    if (t >= ntiles) { s_tile[s] = -1; return; }\n";
  o << "    s_tile[s] = t; s_step[s] = 0; s_done[s] = 0; s_pend[s] = 0; s_seq[s] = s_cseq++;\n";
  o << "  };\n";
  // warp 0: alive masks of a newly claimed tile (rows < n)
  o << "  auto init_alive_ = [&](int s, long long tile) {\n";
  o << "    for (int kw = lane; kw < GX_T; kw += 32) {\n";
  o << "      const i64 r0 = (tile * GX_T + kw) * 32;\n";
  o << "      const i64 left = a.n - r0;\n";
  o << "      s_alive[s][kw] = left >= 32 ? 0xffffffffu : (left <= 0 ? 0u : ((1u << left) - 1u));\n";
  o << "    }\n";
  o << "    __syncwarp();\n";
  o << "  };\n";

  // setup: barriers and the first GX_D tiles
  o << "  if (threadIdx.x == 0) {\n";
  o << "    s_cseq = 0; s_rseq = 0; s_abort = 0;\n";
  o << "    for (int s = 0; s < GX_D; s++) { gx_mbar_init(&s_bar[s], 32u); s_par[s] = 0u; }\n";
  o << "    gx_mbar_init_fence();\n";
  o << "    for (int s = 0; s < GX_D; s++) claim_(s);\n";
  o << "  }\n";
  o << "  __syncthreads();\n";
  o << "  if (warp == 0) {\n";
  o << "    for (int s = 0; s < GX_D; s++) {\n";
  o << "      const long long t = s_tile[s];\n";
  o << "      if (t < 0) continue;\n";
  o << "      init_alive_(s, t);\n";
  o << "      issue_(s, t, 0);\n";
  o << "    }\n";
  o << "  }\n";

  o << "  while (true) {\n";
  o << "    __syncthreads();\n";
  o << "    bool any_ = false;\n";
  o << "    #pragma unroll\n    for (int s = 0; s < GX_D; s++) any_ |= s_tile[s] >= 0;\n";
  o << "    if (!any_ || s_abort) break;\n";
  o << "    for (int s = 0; s < GX_D; s++) {\n";
  o << "      __syncthreads();\n";
  o << "      const long long tile = s_tile[s];\n";
  o << "      if (tile < 0) continue;\n";
  // ---- one conjunct step
  o << "      if (s_done[s] == 0) {\n";
  o << "        if (s_pend[s]) {\n";
  o << "          const u32 par_ = s_par[s];\n";
  o << "          u32 sp_ = 0u;\n";
  o << "          while (!gx_mbar_try_wait(&s_bar[s], par_)) {\n";
  o << "            if (++sp_ > mbar_limit) { atomicExch(a.err, 1); s_abort = 1; break; }\n";
  o << "            __nanosleep(20);\n";
  o << "          }\n";
  o << "        }\n";
  o << "        const int cj = a.order_dev ? __ldg(a.order_dev + s_step[s]) : a.order[s_step[s]];\n";
  o << "        bool keep_[GX_V];\n";
  o << "        bool inr_[GX_V];\n";
  o << "        switch (cj) {\n";
  for (int c = 0; c < nc; c++) {
    const int cid = p.conjuncts[c];
    o << "          case " << c << ": {\n";
    g.staged_.clear();
    for (size_t i = 0; i < cc[c].size(); i++)
      g.staged_[cc[c][i]] = {"(const void*)(s_buf[s] + GX_T * " + std::to_string(coff[c][i]) + ")",
                             "(i64)(kw * 32 + lane)"};
    const std::vector<int> ids = g.cone({cid});
    g.decl(o, ids, "            ");
    o << "            #pragma unroll\n            for (int k = 0; k < GX_V; k++) {\n";
    o << "              const int kw = warp * GX_V + k;\n";
    o << "              const i64 row = (tile * GX_T + kw) * 32 + lane;\n";
    o << "              const bool full_word_ = (tile * GX_T + kw + 1) * 32 <= a.n; (void)full_word_;\n";
    o << "              const bool inr = ((s_alive[s][kw] >> lane) & 1u) != 0u;\n";
    for (int id : ids)
      if (p.nodes[id].kind == Node::COL) g.emit_node(o, id, "              ");
    for (int id : ids)
      if (p.nodes[id].kind != Node::COL) g.emit_node(o, id, "              ");
    o << "              keep_[k] = " << g.conj_keep(cid) << "; inr_[k] = inr;\n";
    o << "            }\n";
    o << "            break; }\n";
  }
  g.staged_.clear();
  o << "          default:\n";
  o << "            #pragma unroll\n            for (int k = 0; k < GX_V; k++) { keep_[k] = false; inr_[k] = false; }\n";
  o << "        }\n";
  o << "        #pragma unroll\n        for (int k = 0; k < GX_V; k++) {\n";
  o << "          const u32 nb_ = __ballot_sync(GX_FULL, inr_[k] && keep_[k]);\n";
  o << "          if (lane == 0) s_alive[s][warp * GX_V + k] &= nb_;\n";
  o << "        }\n";
  o << "        __syncthreads();\n";
  // warp 0: next step or done
  o << "        if (warp == 0) {\n";
  o << "          if (lane == 0) { if (s_pend[s]) s_par[s] ^= 1u; s_step[s] += 1; }\n";
  o << "          __syncwarp();\n";
  o << "          u32 live_ = 0u;\n";
  o << "          for (int kw = lane; kw < GX_T; kw += 32) live_ |= s_alive[s][kw];\n";
  o << "          const bool anyl_ = __any_sync(GX_FULL, live_ != 0u);\n";
  o << "          if (!anyl_ || s_step[s] >= " << nc << ") {\n";
  o << "            if (lane == 0) { s_done[s] = 1; s_pend[s] = 0; }\n";
  o << "          } else {\n";
  o << "            issue_(s, tile, s_step[s]);\n";
  o << "          }\n";
  o << "        }\n";
  o << "        __syncthreads();\n";
  o << "      }\n";
  // ---- publish the aggregate of a finished tile
  o << "      if (s_done[s] == 1) {\n";
  o << "        u32 c_ = 0u;\n";
  o << "        #pragma unroll\n        for (int k = 0; k < GX_V; k++) c_ += __popc(s_alive[s][warp * GX_V + k]);\n";
  o << "        if (lane == 0) s_cnt[warp] = c_;\n";
  o << "        __syncthreads();\n";
  o << "        if (warp == 0) {\n";
  o << "          const u64 tot_ = gx_tile_publish(a.tile_status, tile, s_cnt, s_off[s], GX_WARPS);\n";
  o << "          if (lane == 0) { s_total[s] = tot_; s_done[s] = 2; }\n";
  o << "          if (lane == 0 && s_seq[s] == s_rseq) { s_lbpred = tile - 1; s_lbexcl = 0ull; s_lbpolls = 0u; }\n";
  o << "        }\n";
  o << "        __syncthreads();\n";
  o << "      }\n";
  // ---- resolve and write, in claim order
  // the oldest tile's look-back is polled, never waited on: while predecessors
  // are missing the block goes on with its other tiles, whose aggregates other
  // blocks may be waiting for
  o << "      if (s_done[s] == 2 && s_seq[s] == s_rseq) {\n";
  o << "        if (warp == 0) {\n";
  o << "          long long pr_ = s_lbpred; u64 ex_ = s_lbexcl;\n";
  o << "          const bool ok_ = gx_lookback_poll(a.tile_status, tile, s_total[s], &pr_, &ex_);\n";
  o << "          if (lane == 0) {\n";
  o << "            s_lbpred = pr_; s_lbexcl = ex_; s_ready = ok_ ? 1 : 0;\n";
  o << "            if (ok_) {\n";
  o << "              s_base = ex_;\n";
  o << "              if (tile == ntiles - 1) *a.out_count = ex_ + s_total[s];\n";
  o << "            } else if (++s_lbpolls > spin_limit) {\n";
  o << "              atomicExch(a.err, 1); s_abort = 1;\n";
  o << "            } else {\n";
  o << "              __nanosleep(64);\n";
  o << "            }\n";
  o << "          }\n";
  o << "        }\n";
  o << "        __syncthreads();\n";
  o << "        if (!s_ready) continue;\n";
  o << "        {\n";
  o << "          u32 bal[GX_V]; u32 wcnt = 0u;\n";
  o << "          #pragma unroll\n          for (int k = 0; k < GX_V; k++) { bal[k] = s_alive[s][warp * GX_V + k]; wcnt += __popc(bal[k]); }\n";
  o << "          if (wcnt != 0u) {\n";
  o << "            u64 pos = s_base + s_off[s][warp];\n";
  o << "            const i64 w0 = tile * GX_T + (i64)warp * GX_V;\n";
  emit_filter_writes_dense(o, g, p, "            ");
  o << "          }\n";
  o << "        }\n";
  o << "        __syncthreads();\n";
  o << "        if (threadIdx.x == 0) {\n";
  o << "          s_rseq++;\n";
  o << "          claim_(s);\n";
  o << "          for (int q = 0; q < GX_D; q++)  // the next oldest, if already published\n";
  o << "            if (s_tile[q] >= 0 && s_done[q] == 2 && s_seq[q] == s_rseq) { s_lbpred = s_tile[q] - 1; s_lbexcl = 0ull; s_lbpolls = 0u; }\n";
  o << "        }\n";
  o << "        __syncthreads();\n";
  o << "        if (warp == 0 && s_tile[s] >= 0) {\n";
  o << "          init_alive_(s, s_tile[s]);\n";
  o << "          issue_(s, s_tile[s], 0);\n";
  o << "        }\n";
  o << "      }\n";
  o << "    }\n";
  o << "  }\n";
  // an abandoned run (a wait gave up): let copies still in flight land before exit
  o << "  __syncthreads();\n";
  o << "  if (s_abort && threadIdx.x == 0) {\n";
  o << "    for (int s = 0; s < GX_D; s++) {\n";
  o << "      if (s_tile[s] < 0 || !s_pend[s] || s_done[s] != 0) continue;\n";
  o << "      u32 sp_ = 0u;\n";
  o << "      while (!gx_mbar_try_wait(&s_bar[s], s_par[s]) && ++sp_ < mbar_limit) __nanosleep(20);\n";
  o << "    }\n";
  o << "  }\n";
  o << "}\n";
}

}  // namespace

TileLayout tile_layout(const Plan& p, int warps, int words, int stages) {
  TileLayout L;
  L.tile_rows = warps * words * 32;
  L.stages = stages;
  if (L.tile_rows % 128 != 0) fail(GX_ERR_INVALID, "tile-staged kernels need tiles of a multiple of 128 rows");
  if (stages < 2) fail(GX_ERR_INVALID, "tile-staged kernels need at least 2 stages");
  if (warps > 32) fail(GX_ERR_INVALID, "tile-staged kernels take at most 32 consumer warps");
  L.cols = referenced_columns(p);
  uint32_t off = 0;
  for (int c : L.cols) {
    // data: the tile's bytes from the 16-byte block of its first element up to
    // the block past its last; mask: its words plus the next one (re-alignment
    // to the tile's rows reads one word ahead), from the first word's block
    L.data_off.push_back(off);
    off += (uint32_t)L.tile_rows * (uint32_t)type_size(p.schema[c]) + 32u;
    if (p.nullable[c]) {
      L.mask_off.push_back(off);
      L.mask_index.push_back(L.num_masked++);
      off += (uint32_t)L.tile_rows / 8u + 32u;
    } else {
      L.mask_off.push_back(UINT32_MAX);
      L.mask_index.push_back(-1);
    }
  }
  L.stage_bytes = (off + 127u) & ~127u;
  // output staging: per non-literal output its data slot and one validity
  // byte per row, by the row's kept rank within the tile
  uint32_t oo = 0;
  for (const auto& os : p.outputs) {
    const int t = os.kind == OutSpec::COPY ? p.schema[os.col] : os.type;
    const uint32_t w = os.kind == OutSpec::BROADCAST ? 0u : (uint32_t)type_size(t);
    L.out_width.push_back(w);
    L.out_off.push_back(oo);
    oo += ((uint32_t)L.tile_rows * w + 15u) & ~15u;
    L.out_valid_off.push_back(oo);
    if (os.kind != OutSpec::BROADCAST) oo += (uint32_t)L.tile_rows;
  }
  L.out_stage_bytes = (oo + 127u) & ~127u;
  L.out_base = L.stage_bytes * (uint32_t)stages;
  L.dyn_smem = L.out_base + (uint32_t)L.out_stages * L.out_stage_bytes;
  return L;
}

std::vector<int> conjunct_columns(const Plan& p, int c) {
  std::set<int> cols;
  std::function<void(int)> go = [&](int id) {
    if (id < 0) return;
    const Node& n = p.nodes[id];
    if (n.kind == Node::COL) cols.insert(n.col);
    if (n.kind == Node::OP) { go(n.a); go(n.b); }
  };
  go(p.conjuncts.at(c));
  return std::vector<int>(cols.begin(), cols.end());
}

// Which binary64 operation classes go to the FP64 pipe when the plan leaves it
// to the library.  Both forms are exact; the choice balances the two pipes.
// Add, subtract and multiply cost about as much natively (one FP64-pipe
// instruction, at 1/64 of the FP32 rate) as emulated (about 25 integer
// instructions), so moving them to the otherwise idle FP64 pipe frees the
// integer pipes.  Integer-to-double conversions go there too.  Compares go
// there only when the plan has no transcendental (LN / EXP / trigonometric /
// POWER / ROUND, which already load the FP64 pipe): with one they cost more
// time there than they free.  So does division by a literal (a multiply and
// two FMAs instead of about 100 integer instructions).  Other division stays
// emulated: natively it is a reciprocal and Newton steps, several FP64-pipe
// instructions.  Measured on
// GB300 against all-emulated: 25 % on the deep plan (with LN / EXP; the
// conversions are 6.5 % of it), 10 % on the plain filter + divide.
int auto_native_f64_ops(const Plan& p) {
  bool transcendental = false;
  for (const auto& n : p.nodes)
    if (n.kind == Node::OP) switch (n.op) {
        case OP_SIN: case OP_COS: case OP_ASIN: case OP_ACOS: case OP_TAN: case OP_COTAN: case OP_ATAN:
        case OP_LN: case OP_LOG10: case OP_EXP: case OP_POW: case OP_ROUND:
          transcendental = true;
          break;
        default: break;
      }
  return transcendental ? (kNativeAddSub | kNativeMul | kNativeConvert)
                        : (kNativeAddSub | kNativeMul | kNativeConvert | kNativeCompare | kNativeConstDiv |
                           kNativeIntDiv);
}

std::string generate_kernel(const Plan& p, KernelKind kind, const KernelConfig& cfg_in, const std::string& name) {
  KernelConfig cfg = cfg_in;
  if (cfg.native_f64_ops < 0) cfg.native_f64_ops = auto_native_f64_ops(p);
  Gen g(p, cfg);
  if (p.has_filter() && cfg.dense) {
    // columns whose data the predicate reads (not only their validity, as
    // IS [NOT] NULL does) and the dense projections read again by kept row
    std::set<int> pred_cols;
    const std::vector<int> pc = g.predicate_cone();
    for (int id : pc) {
      const Node& n = p.nodes[id];
      if (n.kind != Node::OP || n.op == OP_IS_NULL || n.op == OP_IS_NOT_NULL) continue;
      for (int x : {n.a, n.b})
        if (x >= 0 && p.nodes[x].kind == Node::COL) pred_cols.insert(p.nodes[x].col);
    }
    for (int c : p.conjuncts)  // a BOOL8 column as a conjunct is read as data
      if (p.nodes[c].kind == Node::COL) pred_cols.insert(p.nodes[c].col);
    for (int id : g.cone(g.output_roots()))
      if (p.nodes[id].kind == Node::COL && pred_cols.count(p.nodes[id].col)) g.reread_cols_.insert(p.nodes[id].col);
    for (const auto& os : p.outputs)
      if (os.kind == OutSpec::COPY && pred_cols.count(os.col)) g.reread_cols_.insert(os.col);
  }
  std::ostringstream o;
  emit_prelude(o, cfg);
  g.emit_rcp_table(o);
  if (kind == KernelKind::FUSED_STAGED) {
    if (!p.has_filter() || p.conjuncts.size() > 16) fail(GX_ERR_INVALID, "the staged kernel runs filters of at most 16 conjuncts");
    KernelConfig c = cfg;
    c.dense = true;
    c.runtime_order = true;
    Gen gs(p, c);
    emit_staged_filter(o, gs, p, name);
    return o.str();
  }
  if (kind == KernelKind::FUSED_TMA) {
    if (!p.has_filter()) fail(GX_ERR_INVALID, "the tile-staged kernel runs filter plans");
    if (cfg.runtime_order || cfg.short_circuit || !cfg.dense)
      fail(GX_ERR_INVALID, "the tile-staged kernel evaluates conjuncts in plan order with dense projections");
    const TileLayout L = tile_layout(p, cfg.warps, cfg.words, cfg.stages);
    emit_fused_tma(o, g, p, L, name);
    return o.str();
  }
  if (kind == KernelKind::FUSED_BATCHED || kind == KernelKind::FUSED_STREAM) {
    if (!p.has_filter()) fail(GX_ERR_INVALID, "the batched kernel runs filter plans");
    if (cfg.runtime_order || cfg.short_circuit) fail(GX_ERR_INVALID, "the batched kernel evaluates conjuncts in plan order");
    KernelConfig c = cfg;
    c.dense = true;
    Gen gb(p, c);
    gb.reread_cols_ = g.reread_cols_;
    emit_fused_batched(o, gb, p, gb.predicate_cone(), name, kind == KernelKind::FUSED_STREAM);
    return o.str();
  }
  o << "extern \"C\" __global__ void GX_LB " << name << "(const GxArgs a) {\n";
  o << "  const int lane = threadIdx.x & 31; const int warp = threadIdx.x >> 5;\n";
  o << "  const i64 nwords = (a.n + 31) >> 5;\n";
  if (kind == KernelKind::PROJECT) {
    std::vector<int> ids = g.cone(g.output_roots());
    o << "  for (i64 w0 = ((i64)blockIdx.x * GX_WARPS + warp) * GX_V; w0 < nwords;"
         " w0 += (i64)gridDim.x * GX_WARPS * GX_V) {\n";
    g.decl(o, ids, "    ");
    // every column load of the warp's words first, then operators and stores
    o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) {\n";
    o << "      const i64 row = (w0 + k) * 32 + lane; const bool inr = row < a.n; (void)inr;\n";
    for (int id : ids)
      if (p.nodes[id].kind == Node::COL) g.emit_node(o, id, "      ");
    o << "    }\n";
    o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) {\n";
    o << "      const i64 row = (w0 + k) * 32 + lane; const bool inr = row < a.n; (void)inr;\n";
    o << "      const i64 orow = row; (void)orow;\n";
    for (int id : ids)
      if (p.nodes[id].kind != Node::COL) g.emit_node(o, id, "      ");
    for (size_t j = 0; j < p.outputs.size(); j++) {
      const OutSpec& os = p.outputs[j];
      if (os.kind != OutSpec::NODE) continue;
      o << "      if (inr) " << store_stmt(os.type, "a.out_data[" + std::to_string(j) + "]", "row", g.B(os.node)) << "\n";
      o << "      { const u32 vb_ = __ballot_sync(GX_FULL, inr && " << g.V(os.node) << ");\n";
      o << "        if (lane == 0 && w0 + k < nwords) a.out_mask[" << j << "][w0 + k] = vb_; }\n";
    }
    o << "    }\n  }\n}\n";
    return o.str();
  }

  if ((cfg.runtime_order || cfg.conj_stats) && p.conjuncts.size() > 16)
    fail(GX_ERR_UNSUPPORTED, "learned ordering supports at most 16 AND conjuncts");
  // dense phase 2 recomputes every output from the gathered row; the word mode
  // would reuse predicate values that a runtime-ordered predicate never computed
  if (cfg.runtime_order && !cfg.dense) fail(GX_ERR_INVALID, "runtime conjunct order needs dense projections");
  const std::vector<int> pred_ids = g.predicate_cone();
  // per-conjunct pass counts (training labels) only in the plain fixed-order count pass
  const bool stats = kind == KernelKind::COUNT_FILTER && cfg.conj_stats && !cfg.runtime_order && !cfg.short_circuit;
  if (stats) {
    o << "  __shared__ unsigned long long s_conj[16];\n";
    o << "  if (threadIdx.x < 16) s_conj[threadIdx.x] = 0ull;\n";
    o << "  __syncthreads();\n";
  }
  if (kind == KernelKind::FUSED_FILTER && cfg.dense) {
    emit_fused_pipelined(o, g, p, pred_ids);
    return o.str();
  }
  o << "  __shared__ unsigned long long s_tile;\n";
  o << "  __shared__ u64 s_w[GX_WARPS];\n";
  o << "  const i64 ntiles = (nwords + GX_TILE_WORDS - 1) / GX_TILE_WORDS;\n";
  if (kind == KernelKind::FUSED_FILTER) {
    o << "  while (true) {\n";
    o << "    if (threadIdx.x == 0) s_tile = atomicAdd(a.tile_counter, 1ull);\n";
    o << "    __syncthreads();\n";
    o << "    const i64 tile = (i64)s_tile;\n";
    o << "    if (tile >= ntiles) break;\n";
  } else {
    o << "  for (i64 tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {\n";
  }
  o << "    const i64 w0 = tile * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  g.decl(o, pred_ids, "    ");
  g.emit_predicate(o, "    ");
  if (stats) g.emit_conj_stats(o, "    ");
  o << "    u32 bal[GX_V]; u32 wcnt = 0;\n";
  o << "    #pragma unroll\n    for (int k = 0; k < GX_V; k++) { bal[k] = __ballot_sync(GX_FULL, alive[k]); wcnt += __popc(bal[k]); }\n";
  // per-warp exclusive offsets within the tile
  o << "    if (lane == 0) s_w[warp] = wcnt;\n";
  o << "    __syncthreads();\n";
  o << "    if (warp == 0) {\n";
  o << "      u64 c = lane < GX_WARPS ? s_w[lane] : 0ull; u64 incl = c;\n";
  o << "      #pragma unroll\n      for (int d = 1; d < 32; d <<= 1) { u64 t = __shfl_up_sync(GX_FULL, incl, d); if (lane >= d) incl += t; }\n";
  o << "      const u64 total = __shfl_sync(GX_FULL, incl, 31);\n";
  if (kind == KernelKind::FUSED_FILTER) {
    o << "      const u64 excl_tile = gx_lookback(a.tile_status, tile, total, a.err, GX_SPINS);\n";
    o << "      if (tile == ntiles - 1 && lane == 0 && excl_tile != ~0ull) *a.out_count = excl_tile + total;\n";
  } else if (kind == KernelKind::COUNT_FILTER) {
    o << "      if (lane == 0) a.tile_status[tile] = total;\n";
    o << "      const u64 excl_tile = 0ull;\n";
  } else {
    o << "      const u64 excl_tile = a.tile_status[tile];\n";
  }
  o << "      if (lane < GX_WARPS) s_w[lane] = excl_tile == ~0ull ? ~0ull : excl_tile + incl - c;\n";
  o << "    }\n";
  o << "    __syncthreads();\n";
  if (kind != KernelKind::COUNT_FILTER) {
    o << "    u64 pos = s_w[warp];\n";
    o << "    if (pos == ~0ull) break;\n";  // look-back gave up: error already recorded
    o << "    if (wcnt != 0u) {\n";
    emit_filter_writes(o, g, p, pred_ids, "      ");
    o << "    }\n";
  }
  o << "    __syncthreads();\n";  // s_tile / s_w reuse by the next tile
  o << "  }\n";
  if (stats) {
    o << "  __syncthreads();\n";
    o << "  if (threadIdx.x < " << p.conjuncts.size() << ") atomicAdd(&a.conj_counts[threadIdx.x], s_conj[threadIdx.x]);\n";
  }
  o << "}\n";
  return o.str();
}


// ------------------------------------------------------------ aggregation
// Fused filter + group-by aggregation kernel (gx_filter_aggregate).  Blocks
// claim tiles; each warp evaluates the condition on its words, lists its kept
// rows, and deals them to lanes in rounds of 32.  A lane computes its row's
// keys and aggregation inputs and finds the row's group in the block's hash
// table in shared memory.  The lanes of one group then combine their inputs
// over a tree within the warp, and the group's first lane applies them with
// shared-memory atomics: one atomic per group and warp round.  A row whose
// group finds no room along the probe of the block's table goes to the global
// table directly.  When the tiles run out, each block merges its table into the
// global one.
static std::string agg_identity(int kind, bool flt) {
  if (kind == 2) return "0x7FFFFFFFFFFFFFFFull";                 // MIN: +largest (ordered)
  if (kind == 3) return "0x8000000000000000ull";                 // MAX: -largest (ordered)
  (void)flt;
  return "0ull";                                                 // sums (0 and +0.0 share bits)
}

uint64_t agg_counts_are_rows(const Plan& p, const AggLayout& L) {
  KernelConfig cfg;
  cfg.native_f64_ops = 0;
  Gen g(p, cfg);
  uint64_t m = 0;
  for (size_t j = 0; j < L.in_nodes.size() && j < 64; j++)
    if (L.in_nodes[j] >= 0 && g.never_null(L.in_nodes[j])) m |= 1ull << j;
  return m;
}

std::string generate_agg_kernel(const Plan& p, const AggLayout& L, const KernelConfig& cfg_in,
                                const std::string& name) {
  KernelConfig cfg = cfg_in;
  // the aggregation's floating sums and combining trees already load the FP64
  // pipe: divisions stay on the integer pipes (Q1 shape: 3.72 ms, against
  // 3.93 ms with the literal division and 3.91 ms with the integer-value
  // division on the FMA unit)
  if (cfg.native_f64_ops < 0) cfg.native_f64_ops = auto_native_f64_ops(p) & ~(kNativeConstDiv | kNativeIntDiv);
  cfg.short_circuit = false;
  cfg.runtime_order = false;
  cfg.conjunct_order.clear();
  Gen g(p, cfg);
  std::ostringstream o;
  emit_prelude(o, cfg);
  g.emit_rcp_table(o);
  const int nk = (int)L.key_nodes.size(), na = (int)L.kinds.size(), S = L.smem_slots;
  const uint64_t rows_cnt = agg_counts_are_rows(p, L);
  if (S < 16 || (S & (S - 1)) != 0) fail(GX_ERR_INVALID, "aggregation table slots must be a power of two >= 16");
  o << "#define GXA_S " << S << "\n#define GXA_NK " << std::max(nk, 1) << "\n#define GXA_NA " << std::max(na, 1)
    << "\n#define GXA_PROBES 32\n";
  // key hash (null keys hash as zero with their null bit set)
  // (multiply by odd constants per key, then the high half folded onto the
  // low one, which the table index takes)
  o << "__device__ __forceinline__ u64 gxa_hash(const u64* kv, u32 kn) {\n"
       "  u64 h = (0x9E3779B97F4A7C15ull ^ (u64)kn) * 0xBF58476D1CE4E5B9ull;\n";
  for (int j = 0; j < nk; j++) o << "  h = (h ^ kv[" << j << "]) * 0x94D049BB133111EBull;\n";
  o << "  return h ^ (h >> 32) ^ (h >> 47);\n}\n";
  auto same_keys = [&](const std::string& ks, const std::string& stride, const std::string& pos) {
    std::string r = "true";
    for (int j = 0; j < nk; j++)
      r += " && *(volatile u64*)(" + ks + " + " + std::to_string(j) + "ull * " + stride + " + " + pos + ") == kv[" +
           std::to_string(j) + "]";
    return r;
  };
  auto write_keys = [&](std::ostringstream& os, const std::string& ks, const std::string& stride,
                        const std::string& pos, const std::string& ind) {
    for (int j = 0; j < nk; j++)
      os << ind << ks << "[" << j << "ull * " << stride << " + " << pos << "] = kv[" << j << "];\n";
  };
  // the block's table: -1 when the probe finds no room, -2 after a wait gave up
  o << "__device__ int gxa_find_smem(u32* st, u32* nm, u64* ks, const u64* kv, u32 kn, u64 h, int* err) {\n"
       "  u32 pos = (u32)h & (GXA_S - 1);\n"
       "  for (int pr = 0; pr < GXA_PROBES; pr++) {\n"
       "    u32 s = *(volatile u32*)(st + pos);\n"
       "    if (s == 0u) {\n"
       "      s = atomicCAS(st + pos, 0u, 1u);\n"
       "      if (s == 0u) {\n";
  write_keys(o, "ks", "GXA_S", "pos", "        ");
  o << "        nm[pos] = kn;\n"
       "        __threadfence_block();\n"
       "        atomicExch(st + pos, 2u);\n"
       "        return (int)pos;\n"
       "      }\n"
       "    }\n"
       "    u32 spins = 0;\n"
       "    while (s == 1u) {\n"
       "      if (++spins > (1u << 20)) { atomicExch(err, 1); return -2; }\n"
       "      __nanosleep(16);\n"
       "      s = *(volatile u32*)(st + pos);\n"
       "    }\n"
       "    __threadfence_block();\n"
       "    if (*(volatile u32*)(nm + pos) == kn && " << same_keys("ks", "GXA_S", "pos") << ") return (int)pos;\n"
       "    pos = (pos + 1u) & (GXA_S - 1);\n"
       "  }\n"
       "  return -1;\n"
       "}\n";
  // the global table: -1 when the whole table was probed (overflow) or a wait gave up
  o << "__device__ long long gxa_find_global(const GxAggArgs& g, const u64* kv, u32 kn, u64 h) {\n"
       "  u64 pos = h & (g.cap - 1ull);\n"
       "  for (u64 pr = 0; pr < g.cap; pr++) {\n"
       "    u32 s = *(volatile u32*)(g.state + pos);\n"
       "    if (s == 0u) {\n"
       "      s = atomicCAS(g.state + pos, 0u, 1u);\n"
       "      if (s == 0u) {\n";
  write_keys(o, "g.keys", "g.cap", "pos", "        ");
  o << "        g.nullm[pos] = kn;\n"
       "        __threadfence();\n"
       "        atomicExch(g.state + pos, 2u);\n"
       "        atomicAdd(g.groups, 1ull);\n"
       "        return (long long)pos;\n"
       "      }\n"
       "    }\n"
       "    u32 spins = 0;\n"
       "    while (s == 1u) {\n"
       "      if (++spins > (1u << 22)) { atomicExch(g.err, 1); return -1; }\n"
       "      __nanosleep(32);\n"
       "      s = *(volatile u32*)(g.state + pos);\n"
       "    }\n"
       "    __threadfence();\n"
       "    if (*(volatile u32*)(g.nullm + pos) == kn && " << same_keys("g.keys", "g.cap", "pos") << ") return (long long)pos;\n"
       "    pos = (pos + 1ull) & (g.cap - 1ull);\n"
       "  }\n"
       "  atomicExch(g.overflow, 1);\n"
       "  return -1;\n"
       "}\n";

  // per aggregation: value type, input value, identity, combine, atomic update
  struct AggCode {
    std::string ty, val, id, comb, atom;  // atom: format with @A@ (address) and @X@ (value)
  };
  std::vector<AggCode> ac(na);
  for (int j = 0; j < na; j++) {
    const int kind = L.kinds[j], in = L.in_nodes[j];
    const bool flt = in >= 0 && g.kind_f(in);
    AggCode& c = ac[j];
    if (kind == 4 || kind == 5) continue;  // counts only
    if (kind == 2 || kind == 3) {
      c.ty = "long long";
      c.val = flt ? "gx_ord64(" + g.B(in) + ")" : "(long long)(" + g.B(in) + ")";
      c.id = kind == 2 ? "(long long)0x7FFFFFFFFFFFFFFFull" : "(long long)0x8000000000000000ull";
      c.comb = kind == 2 ? "min" : "max";
      c.atom = kind == 2 ? "atomicMin((long long*)(@A@), @X@);" : "atomicMax((long long*)(@A@), @X@);";
    } else if (flt) {
      c.ty = "double";
      c.val = "__longlong_as_double((long long)(" + g.B(in) + "))";
      c.id = "0.0";
      c.comb = "+";
      c.atom = "atomicAdd((double*)(@A@), @X@);";
    } else {
      c.ty = "u64";
      c.val = "(u64)(" + g.B(in) + ")";
      c.id = "0ull";
      c.comb = "+";
      c.atom = "atomicAdd((unsigned long long*)(@A@), (unsigned long long)(@X@));";
    }
  }
  auto atom = [&](int j, const std::string& addr, const std::string& x) {
    std::string a = ac[j].atom;
    a.replace(a.find("@A@"), 3, addr);
    a.replace(a.find("@X@"), 3, x);
    return a;
  };
  auto combine = [&](int j, const std::string& x, const std::string& t) {
    if (ac[j].comb == "+") return x + " += " + t + ";";
    return x + " = " + ac[j].comb + "(" + x + ", " + t + ");";
  };
  std::vector<int> roots = L.key_nodes;
  for (int in : L.in_nodes)
    if (in >= 0) roots.push_back(in);
  const std::vector<int> row_ids = g.cone(roots);
  const std::vector<int> pred_ids = g.predicate_cone();

  o << "extern \"C\" __global__ void GX_LB " << name
    << "(const GxArgs a, const GxAggArgs ga) {\n";
  o << "  const int lane = threadIdx.x & 31; const int warp = threadIdx.x >> 5;\n";
  o << "  const i64 nwords = (a.n + 31) >> 5;\n";
  o << "  const i64 ntiles = (nwords + GX_TILE_WORDS - 1) / GX_TILE_WORDS;\n";
  o << "  __shared__ u32 s_st_[GXA_S]; __shared__ u32 s_nm_[GXA_S]; __shared__ u64 s_rows_[GXA_S];\n";
  o << "  __shared__ u64 s_ks_[GXA_NK * GXA_S]; __shared__ u64 s_acc_[GXA_NA * GXA_S];\n";
  o << "  __shared__ u64 s_cnt_[GXA_NA * GXA_S];\n";
  o << "  __shared__ unsigned short s_kept_[GX_WARPS][GX_V * 32];\n";
  o << "  __shared__ unsigned long long s_claim;\n";
  o << "  for (int i = threadIdx.x; i < GXA_S; i += blockDim.x) {\n";
  o << "    s_st_[i] = 0u; s_nm_[i] = 0u; s_rows_[i] = 0ull;\n";
  for (int j = 0; j < na; j++)
    o << "    s_acc_[" << j << " * GXA_S + i] = " << agg_identity(L.kinds[j], false) << "; s_cnt_[" << j
      << " * GXA_S + i] = 0ull;\n";
  o << "  }\n  __syncthreads();\n";
  o << "  while (true) {\n";
  o << "    if (threadIdx.x == 0) s_claim = atomicAdd(a.tile_counter, 1ull);\n";
  o << "    __syncthreads();\n";
  o << "    const i64 tile = (i64)s_claim;\n";
  o << "    __syncthreads();\n";
  o << "    if (tile >= ntiles) break;\n";
  o << "    const i64 w0 = tile * GX_TILE_WORDS + (i64)warp * GX_V;\n";
  o << "    u32 bal[GX_V];\n";
  o << "    {\n";
  if (p.has_filter()) {
    g.decl(o, pred_ids, "      ");
    g.emit_predicate(o, "      ");
  } else {
    o << "      bool alive[GX_V];\n";
    o << "      #pragma unroll\n      for (int k = 0; k < GX_V; k++) alive[k] = (w0 + k) * 32 + lane < a.n;\n";
  }
  o << "      #pragma unroll\n      for (int k = 0; k < GX_V; k++) bal[k] = __ballot_sync(GX_FULL, alive[k]);\n";
  o << "    }\n";
  o << "    u32 total_ = 0u;\n";
  o << "    #pragma unroll\n    for (int kk = 0; kk < GX_V; kk++) {\n";
  o << "      if ((bal[kk] >> lane) & 1u) s_kept_[warp][total_ + __popc(bal[kk] & ((1u << lane) - 1u))] = "
       "(unsigned short)(kk * 32 + lane);\n";
  o << "      total_ += __popc(bal[kk]);\n";
  o << "    }\n";
  o << "    __syncwarp();\n";
  o << "    const u64 pos = 0ull; (void)pos;\n";
  o << "    for (u32 base_ = 0; base_ < total_; base_ += 32u) {\n";
  const std::string in2 = "      ";
  o << in2 << "const u32 t_ = base_ + (u32)lane; const bool act = t_ < total_;\n";
  emit_rank_to_row(o, in2);
  emit_row_nodes(o, g, p, row_ids, {}, in2);
  o << in2 << "u64 kv[GXA_NK]; u32 kn_ = 0u; kv[0] = 0ull;\n";
  for (int j = 0; j < nk; j++) {
    const int id = L.key_nodes[j];
    o << in2 << "kv[" << j << "] = " << g.V(id) << " ? (u64)(" << g.B(id) << ") : 0ull; if (!(" << g.V(id)
      << ")) kn_ |= " << (1u << j) << "u;\n";
  }
  o << in2 << "const u64 h_ = gxa_hash(kv, kn_);\n";
  o << in2 << "const int sl_ = act ? gxa_find_smem(s_st_, s_nm_, s_ks_, kv, kn_, h_, ga.err) : -3;\n";
  o << in2 << "const bool sm_ = sl_ >= 0;\n";
  if (!L.warp_combine) {
    // every lane applies its own row with shared-memory atomics
    o << in2 << "if (sm_) {\n";
    o << in2 << "  atomicAdd((unsigned long long*)&s_rows_[sl_], 1ull);\n";
    for (int j = 0; j < na; j++) {
      const int in = L.in_nodes[j];
      o << in2 << "  if (" << (in >= 0 ? g.V(in) : std::string("true")) << ") {\n";
      if (!((rows_cnt >> j) & 1ull))
        o << in2 << "    atomicAdd((unsigned long long*)&s_cnt_[" << j << " * GXA_S + sl_], 1ull);\n";
      if (!ac[j].ty.empty())
        o << in2 << "    " << atom(j, "&s_acc_[" + std::to_string(j) + " * GXA_S + sl_]", ac[j].val) << "\n";
      o << in2 << "  }\n";
    }
    o << in2 << "}\n";
  } else {
    o << in2 << "const u32 peers_ = __match_any_sync(GX_FULL, sm_ ? (u32)sl_ : (0x80000000u | (u32)lane));\n";
    o << in2 << "GxPeers pr_; pr_.init(peers_);\n";
    for (int j = 0; j < na; j++) {
      const int in = L.in_nodes[j];
      const std::string vj = in >= 0 ? "(sm_ && " + g.V(in) + ")" : "sm_";
      o << in2 << "const bool vl" << j << "_ = " << vj << ";\n";
      if ((rows_cnt >> j) & 1ull)  // never NULL: the count is the group's rows
        o << in2 << "const u64 c" << j << "_ = (u64)__popc(peers_);\n";
      else
        o << in2 << "const u64 c" << j << "_ = (u64)__popc(__ballot_sync(GX_FULL, vl" << j << "_) & peers_);\n";
      if (!ac[j].ty.empty())
        o << in2 << ac[j].ty << " x" << j << "_ = vl" << j << "_ ? " << ac[j].val << " : " << ac[j].id << ";\n";
    }
    // a tree over each group's lanes: log2 of the largest group's lanes steps
    o << in2 << "const int mx_ = (int)__reduce_max_sync(GX_FULL, (u32)__popc(peers_));\n";
    o << in2 << "#pragma unroll\n" << in2 << "for (int s_ = 1; s_ < 32; s_ <<= 1) {\n";
    o << in2 << "  if (s_ >= mx_) break;\n";
    o << in2 << "  const int src_ = pr_.partner(); const bool rcv_ = pr_.receives(s_);\n";
    for (int j = 0; j < na; j++) {
      if (ac[j].ty.empty()) continue;
      o << in2 << "  { const " << ac[j].ty << " t_ = __shfl_sync(GX_FULL, x" << j << "_, src_); if (rcv_) "
        << combine(j, "x" + std::to_string(j) + "_", "t_") << " }\n";
    }
    o << in2 << "  pr_.step(s_);\n";
    o << in2 << "}\n";
    // With one warp per block the table is the warp's own, and the leaders
    // of one round hold distinct slots: plain read-modify-writes replace the
    // shared-memory atomics (a __syncwarp orders them before the next round).
    const bool own = cfg.warps == 1;
    auto plain = [&](int j, const std::string& slot, const std::string& x) {
      if (ac[j].ty == "double")
        return "{ double* q_ = (double*)&" + slot + "; *q_ = *q_ + " + x + "; }";
      if (ac[j].ty == "long long")
        return "{ long long* q_ = (long long*)&" + slot + "; *q_ = " + ac[j].comb + "(*q_, " + x + "); }";
      return slot + " += (u64)(" + x + ");";
    };
    o << in2 << "if (sm_ && pr_.rank == 0) {\n";
    if (own) o << in2 << "  s_rows_[sl_] += (u64)__popc(peers_);\n";
    else o << in2 << "  atomicAdd((unsigned long long*)&s_rows_[sl_], (unsigned long long)__popc(peers_));\n";
    for (int j = 0; j < na; j++) {
      const std::string cs = "s_cnt_[" + std::to_string(j) + " * GXA_S + sl_]";
      const std::string as = "s_acc_[" + std::to_string(j) + " * GXA_S + sl_]";
      const std::string xj = "x" + std::to_string(j) + "_";
      o << in2 << "  if (c" << j << "_ != 0ull) {\n";
      if (!((rows_cnt >> j) & 1ull)) {
        if (own) o << in2 << "    " << cs << " += c" << j << "_;\n";
        else o << in2 << "    atomicAdd((unsigned long long*)&" << cs << ", (unsigned long long)c" << j << "_);\n";
      }
      if (!ac[j].ty.empty()) o << in2 << "    " << (own ? plain(j, as, xj) : atom(j, "&" + as, xj)) << "\n";
      o << in2 << "  }\n";
    }
    o << in2 << "}\n";
    if (own) o << in2 << "__syncwarp();\n";
  }
  // rows whose group found no room in the block's table go to the global one
  o << in2 << "if (act && sl_ == -1) {\n";
  o << in2 << "  const long long gs_ = gxa_find_global(ga, kv, kn_, h_);\n";
  o << in2 << "  if (gs_ >= 0) {\n";
  o << in2 << "    atomicAdd((unsigned long long*)(ga.rows + gs_), 1ull);\n";
  for (int j = 0; j < na; j++) {
    const int in = L.in_nodes[j];
    const std::string vj = in >= 0 ? g.V(in) : "true";
    o << in2 << "    if (" << vj << ") {\n";
    if (!((rows_cnt >> j) & 1ull))
      o << in2 << "      atomicAdd((unsigned long long*)(ga.cnt + " << j << "ull * ga.cap + gs_), 1ull);\n";
    if (!ac[j].ty.empty())
      o << in2 << "      " << atom(j, "ga.acc + " + std::to_string(j) + "ull * ga.cap + gs_", ac[j].val) << "\n";
    o << in2 << "    }\n";
  }
  o << in2 << "  }\n";
  o << in2 << "}\n";
  o << "    }\n";  // rounds
  o << "  }\n";    // tiles
  // merge the block's table into the global one
  o << "  __syncthreads();\n";
  o << "  for (int i = threadIdx.x; i < GXA_S; i += blockDim.x) {\n";
  o << "    if (s_st_[i] != 2u || s_rows_[i] == 0ull) continue;\n";
  o << "    u64 kv[GXA_NK]; kv[0] = 0ull;\n";
  for (int j = 0; j < nk; j++) o << "    kv[" << j << "] = s_ks_[" << j << " * GXA_S + i];\n";
  o << "    const u32 kn_ = s_nm_[i];\n";
  o << "    const long long gs_ = gxa_find_global(ga, kv, kn_, gxa_hash(kv, kn_));\n";
  o << "    if (gs_ < 0) continue;\n";
  o << "    atomicAdd((unsigned long long*)(ga.rows + gs_), (unsigned long long)s_rows_[i]);\n";
  for (int j = 0; j < na; j++) {
    const bool rc = (rows_cnt >> j) & 1ull;  // no valid count kept: every row of the group is valid
    o << "    if (" << (rc ? std::string("s_rows_[i]") : "s_cnt_[" + std::to_string(j) + " * GXA_S + i]")
      << " != 0ull) {\n";
    if (!rc)
      o << "      atomicAdd((unsigned long long*)(ga.cnt + " << j << "ull * ga.cap + gs_), (unsigned long long)s_cnt_["
        << j << " * GXA_S + i]);\n";
    if (!ac[j].ty.empty()) {
      std::string x;
      if (ac[j].ty == "double") x = "__longlong_as_double((long long)s_acc_[" + std::to_string(j) + " * GXA_S + i])";
      else if (ac[j].ty == "long long") x = "(long long)s_acc_[" + std::to_string(j) + " * GXA_S + i]";
      else x = "s_acc_[" + std::to_string(j) + " * GXA_S + i]";
      o << "      " << atom(j, "ga.acc + " + std::to_string(j) + "ull * ga.cap + gs_", x) << "\n";
    }
    o << "    }\n";
  }
  o << "  }\n";
  o << "}\n";
  return o.str();
}
}  // namespace gx
