// aggregate.cu -- fused filter + group-by aggregation: plan building, the
// global group table, the launch of the generated aggregation kernel, and the
// finalisation of the table into output columns.
//
// Semantics follow ral::operators::compute_aggregations_with_groupby and
// compute_aggregations_without_groupby (engine/src/operators/GroupBy.cpp:217-416):
// aggregation inputs are expressions over the input table; keys group with
// NULL as a value of its own (null_policy::INCLUDE, :380); SUM0 of a group
// without valid inputs is 0 (:394-397); output columns are the keys then the
// aggregations (:383-405).  Output types widen sums as :33-40 does.
#include "aggregate.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "jit.h"

namespace gx {

namespace {

// host image of GxAggArgs (device_rt.cuh): same field order, all 8-byte
struct AggTable {
  uint32_t* state;
  uint32_t* nullm;
  uint64_t* keys;
  uint64_t* acc;
  uint64_t* cnt;
  uint64_t* rows;
  uint64_t cap;
  int* overflow;
  int* err;
  unsigned long long* groups;
};

constexpr int kMaxKeys = 8;
constexpr int kMaxAggs = 24;

struct AggFinal {
  int nk, na;
  int key_w[kMaxKeys];
  int kind[kMaxAggs];
  int acc_of[kMaxAggs];  // accumulator of aggregation j (-1: the group's row count)
  int in_flt[kMaxAggs];
  int out_w[kMaxAggs];
  int out_f32[kMaxAggs];
  void* out_data[kMaxKeys + kMaxAggs];
  uint32_t* out_mask[kMaxKeys + kMaxAggs];
  AggTable t;
  unsigned long long* counter;
  int empty_group;  // no group keys and no row: one row of empty aggregates
  unsigned long long cnt_rows;  // accumulators whose valid count is the group's row count (input never NULL)
};

__device__ __forceinline__ void store_w(void* d, uint64_t p, int w, uint64_t v) {
  switch (w) {
    case 1: ((unsigned char*)d)[p] = (unsigned char)v; break;
    case 2: ((unsigned short*)d)[p] = (unsigned short)v; break;
    case 4: ((unsigned int*)d)[p] = (unsigned int)v; break;
    default: ((unsigned long long*)d)[p] = v; break;
  }
}

__device__ __forceinline__ void set_valid(uint32_t* m, uint64_t p) { atomicOr(m + (p >> 5), 1u << (p & 31)); }

__device__ __forceinline__ uint64_t unord64(uint64_t o) {
  return o ^ (((uint64_t)((long long)o >> 63)) & 0x7FFFFFFFFFFFFFFFull);
}

// one output row p from table slot i (i < 0: the empty group)
__device__ void write_row(const AggFinal& f, long long i, uint64_t p) {
  const uint64_t cap = f.t.cap;
  for (int j = 0; j < f.nk; j++) {
    const uint64_t v = f.t.keys[j * cap + i];
    store_w(f.out_data[j], p, f.key_w[j], v);
    if (!((f.t.nullm[i] >> j) & 1u)) set_valid(f.out_mask[j], p);
  }
  for (int j = 0; j < f.na; j++) {
    const int o = f.nk + j;
    const int q = f.acc_of[j];
    const uint64_t c = i < 0 ? 0ull : (q < 0 || ((f.cnt_rows >> q) & 1ull)) ? f.t.rows[i] : f.t.cnt[q * cap + i];
    const uint64_t a = (i < 0 || q < 0) ? 0ull : f.t.acc[q * cap + i];
    const int kind = f.kind[j];
    if (kind == 4 || kind == 5) {  // COUNT_VALID, COUNT_ALL
      store_w(f.out_data[o], p, 8, c);
      set_valid(f.out_mask[o], p);
    } else if (kind == 0 || kind == 1) {  // SUM, SUM0
      store_w(f.out_data[o], p, 8, c ? a : 0ull);
      if (c || kind == 1) set_valid(f.out_mask[o], p);
    } else if (kind == 6) {  // MEAN
      if (c) {
        const double s = f.in_flt[j] ? __longlong_as_double((long long)a) : (double)(long long)a;
        store_w(f.out_data[o], p, 8, (uint64_t)__double_as_longlong(s / (double)c));
        set_valid(f.out_mask[o], p);
      } else {
        store_w(f.out_data[o], p, 8, 0ull);
      }
    } else {  // MIN, MAX (ordered bits for floating inputs)
      uint64_t v = c ? (f.in_flt[j] ? unord64(a) : a) : 0ull;
      if (f.out_f32[j]) {
        const float x = (float)__longlong_as_double((long long)v);
        v = (uint64_t)__float_as_uint(x);
      }
      store_w(f.out_data[o], p, f.out_w[j], v);
      if (c) set_valid(f.out_mask[o], p);
    }
  }
}

__global__ void k_agg_finalize(AggFinal f) {
  if (f.empty_group) {
    if (blockIdx.x == 0 && threadIdx.x == 0) write_row(f, -1, 0);
    return;
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < f.t.cap;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (f.t.state[i] != 2u) continue;
    const uint64_t p = atomicAdd(f.counter, 1ull);
    write_row(f, (long long)i, p);
  }
}

// MIN / MAX accumulators start at the far end of the ordered range
__global__ void k_agg_init(AggTable t, int na, unsigned long long min_mask, unsigned long long max_mask) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < t.cap; i += (uint64_t)gridDim.x * blockDim.x)
    for (int j = 0; j < na; j++) {
      if ((min_mask >> j) & 1ull) t.acc[j * t.cap + i] = 0x7FFFFFFFFFFFFFFFull;
      if ((max_mask >> j) & 1ull) t.acc[j * t.cap + i] = 0x8000000000000000ull;
    }
}

bool key_type_ok(int t) {
  return (t >= INT8 && t <= UINT64) || t == BOOL8 || (t >= TIMESTAMP_DAYS && t <= DURATION_NANOSECONDS);
}

uint64_t next_pow2(uint64_t x) {
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace

AggPlan::AggPlan(const std::vector<int>& schema, const std::vector<bool>& nullable, const std::string& condition,
                 const std::vector<int>& key_cols, const std::vector<std::string>& inputs,
                 const std::vector<int>& kinds, const KernelConfig& cfg)
    : cfg_(cfg) {
  if (key_cols.size() > (size_t)kMaxKeys) fail(GX_ERR_UNSUPPORTED, "at most 8 group columns");
  if (inputs.size() != kinds.size()) fail(GX_ERR_INVALID, "one kind per aggregation input");
  if (kinds.empty() || kinds.size() > (size_t)kMaxAggs) fail(GX_ERR_UNSUPPORTED, "1 to 24 aggregations");
  // the plan's outputs: the keys, then every non-empty aggregation input
  std::vector<std::string> exprs;
  for (int c : key_cols) {
    if (c < 0 || c >= (int)schema.size()) fail(GX_ERR_INVALID, "group column index out of range");
    if (!key_type_ok(schema[c])) fail(GX_ERR_UNSUPPORTED, "group columns must be integer, BOOL8, timestamp or duration");
    exprs.push_back("$" + std::to_string(c));
    key_types_.push_back(schema[c]);
  }
  for (size_t i = 0; i < kinds.size(); i++) {
    if (kinds[i] < 0 || kinds[i] > 6) fail(GX_ERR_INVALID, "unknown aggregation kind");
    if (inputs[i].empty() != (kinds[i] == 5)) fail(GX_ERR_INVALID, "COUNT(*) takes no input; the others take one");
    if (!inputs[i].empty()) exprs.push_back(inputs[i]);
  }
  plan_ = build_plan(schema, nullable, condition, exprs, false, false, 0, nullptr, true);
  for (size_t j = 0; j < key_cols.size(); j++) layout_.key_nodes.push_back(plan_.outputs[j].node);
  // accumulators: one per (sum | min | max, input node); SUM, SUM0 and MEAN of
  // one input share a sum, COUNT(x) takes the valid count of any accumulator
  // on x (a count-only one when there is none), COUNT(*) the group's rows
  size_t next = key_cols.size();
  for (size_t i = 0; i < kinds.size(); i++) {
    int node = -1;
    if (kinds[i] != 5) node = plan_.outputs[next++].node;
    agg_node_.push_back(node);
    in_float_.push_back(node >= 0 && is_float(plan_.nodes[node].ktype));
  }
  auto acc_for = [&](int cls, int node) {
    for (size_t q = 0; q < layout_.kinds.size(); q++)
      if (layout_.kinds[q] == cls && layout_.in_nodes[q] == node) return (int)q;
    layout_.kinds.push_back(cls);
    layout_.in_nodes.push_back(node);
    return (int)layout_.kinds.size() - 1;
  };
  acc_of_.assign(kinds.size(), -1);
  for (size_t i = 0; i < kinds.size(); i++) {
    const int k = kinds[i];
    if (k == 0 || k == 1 || k == 6) acc_of_[i] = acc_for(0, agg_node_[i]);
    else if (k == 2 || k == 3) acc_of_[i] = acc_for(k, agg_node_[i]);
  }
  for (size_t i = 0; i < kinds.size(); i++) {
    if (kinds[i] != 4) continue;
    for (size_t q = 0; q < layout_.kinds.size() && acc_of_[i] < 0; q++)
      if (layout_.in_nodes[q] == agg_node_[i]) acc_of_[i] = (int)q;
    if (acc_of_[i] < 0) acc_of_[i] = acc_for(4, agg_node_[i]);
  }
  agg_kind_ = kinds;
  // output types: keys keep theirs; COUNT INT64; SUM widened; MEAN FLOAT64; MIN/MAX the input's
  out_types_ = key_types_;
  for (size_t i = 0; i < kinds.size(); i++) {
    const int k = kinds[i], node = agg_node_[i];
    if (k == 4 || k == 5) out_types_.push_back(INT64);
    else if (k == 6) out_types_.push_back(FLOAT64);
    else if (k == 0 || k == 1) out_types_.push_back(in_float_[i] ? FLOAT64 : INT64);
    else {
      const int vt = plan_.nodes[node].vtype;
      if (type_size(vt) == 0) fail(GX_ERR_TYPE, "MIN / MAX input has no fixed-width type");
      out_types_.push_back(vt);
    }
  }
  // shared-memory table: as many slots (a power of two, at most 256) as fit in
  // about 8 KB.  A larger table costs blocks per SM, and the kernel is
  // instruction bound.  Measured on GB300 at 2^26 order-line rows: the Q1 shape
  // (6 groups) takes 2.48 / 2.49 / 3.01 ms with 8 / 20 / 40 KB tables; grouped
  // by ship date (2557 groups, mostly in the global table) 8.1 / 8.8 / 16.8 ms.
  const size_t per_slot = 4 + 4 + 8 + 8 * std::max<size_t>(key_cols.size(), 1) +
                          16 * std::max<size_t>(layout_.kinds.size(), 1);
  int slots = 256;
  const int budget = std::getenv("GX_AGG_SMEM_KB") ? std::atoi(std::getenv("GX_AGG_SMEM_KB")) : 8;
  while (slots > 16 && (size_t)slots * per_slot > (size_t)budget * 1024) slots >>= 1;
  layout_.smem_slots = slots;
  const char* wc = std::getenv("GX_AGG_COMBINE");
  layout_.warp_combine = !(wc && *wc == '0');
}

std::string AggPlan::kernel_source(const std::vector<bool>& nullable) const {
  Plan p = plan_;
  p.nullable = nullable;
  return generate_agg_kernel(p, layout_, cfg_, "gx_filter_aggregate");
}

JitKernel AggPlan::kernel(const std::vector<bool>& nullable) const {
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::string key = std::to_string(dev) + ":";
  for (bool b : nullable) key += b ? '1' : '0';
  {
    std::lock_guard<std::mutex> g(mu_);
    auto it = kcache_.find(key);
    if (it != kcache_.end()) return it->second;
  }
  const JitKernel k = jit_get(kernel_source(nullable), "gx_filter_aggregate", cfg_.warps * 32);
  std::lock_guard<std::mutex> g(mu_);
  kcache_[key] = k;
  return k;
}

void AggPlan::execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_groups, cudaStream_t s) const {
  if (cols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < cols.size(); i++)
    if (cols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const int nk = (int)layout_.key_nodes.size(), na = (int)layout_.kinds.size();  // na: accumulators
  const int nagg = (int)agg_kind_.size();
  const int nout = nk + nagg;
  std::vector<bool> nb(cols.size());
  for (size_t i = 0; i < cols.size(); i++) nb[i] = cols[i].mask != nullptr;
  const JitKernel k = kernel(nb);  // compiled before any allocation of this call
  unsigned long long min_mask = 0, max_mask = 0;
  for (int j = 0; j < na; j++) {
    if (layout_.kinds[j] == 2) min_mask |= 1ull << j;
    if (layout_.kinds[j] == 3) max_mask |= 1ull << j;
  }
  // the global table: a start size that fits few groups cheaply, grown (and
  // the pass repeated) when a probe walks the whole table
  uint64_t cap = next_pow2((uint64_t)std::max<int64_t>(1024, std::min<int64_t>(2 * n, int64_t(1) << 17)));
  const uint64_t max_cap = next_pow2((uint64_t)std::max<int64_t>(1024, 2 * n + 16));
  const int64_t tile_rows = (int64_t)cfg_.warps * cfg_.words * 32;
  const int64_t ntiles = (n + tile_rows - 1) / tile_rows;
  unsigned long long* hflags = nullptr;  // overflow, err, groups (pinned per thread)
  thread_local unsigned long long* tflags = nullptr;
  if (!tflags) check_cuda(cudaMallocHost((void**)&tflags, 64), "pinned flags");
  hflags = tflags;
  AggTable t{};
  char* base = nullptr;
  unsigned long long groups = 0;
  while (true) {
    const size_t tb = (size_t)cap * (4 + 4 + 8 + 8 * nk + 16 * na);
    const size_t bytes = tb + 256;
    base = (char*)dev_alloc(bytes, s);
    char* q = base;
    t.state = (uint32_t*)q; q += cap * 4;
    t.nullm = (uint32_t*)q; q += cap * 4;
    t.rows = (uint64_t*)q; q += cap * 8;
    t.keys = (uint64_t*)q; q += cap * 8 * nk;
    t.acc = (uint64_t*)q; q += cap * 8 * na;
    t.cnt = (uint64_t*)q; q += cap * 8 * na;
    unsigned long long* flags = (unsigned long long*)(base + tb);  // [0] overflow, [1] err, [2] groups, [3] tiles, [4] rows out
    t.cap = cap;
    t.overflow = (int*)(flags + 0);
    t.err = (int*)(flags + 1);
    t.groups = flags + 2;
    try {
      check_cuda(cudaMemsetAsync(base, 0, bytes, s), "aggregation table clear");
      if (min_mask | max_mask) {
        k_agg_init<<<(unsigned)std::min<uint64_t>((cap + 255) / 256, 4096), 256, 0, s>>>(t, na, min_mask, max_mask);
        check_cuda(cudaGetLastError(), "k_agg_init");
        add_launches(1);
      }
      if (n > 0) {
        KernelArgs a{};
        for (size_t i = 0; i < cols.size(); i++) {
          a.in_data[i] = cols[i].data;
          a.in_mask[i] = cols[i].mask;
          a.in_off[i] = cols[i].offset;
        }
        a.n = n;
        a.tile_counter = flags + 3;
        a.err = t.err;
        a.seed = plan_.rand_seed;
        for (int i = 0; i < 16; i++) a.order[i] = i;
        int64_t grid = (int64_t)device_sm_count() * k.max_blocks_per_sm;
        grid = std::min<int64_t>(grid, std::max<int64_t>(ntiles, 1));
        void* params[] = {&a, &t};
        launch_raw(k, (int)grid, s, params, true);
      }
      check_cuda(cudaMemcpyAsync(hflags, flags, 24, cudaMemcpyDeviceToHost, s), "aggregation flags");
      check_cuda(cudaStreamSynchronize(s), "aggregation sync");
    } catch (...) {
      dev_free(base, s);
      throw;
    }
    if ((int)hflags[1] != 0) {
      dev_free(base, s);
      fail(GX_ERR_TIMEOUT, "aggregation table wait timed out");
    }
    if ((int)hflags[0] == 0) {
      groups = hflags[2];
      break;
    }
    dev_free(base, s);
    if (cap >= max_cap) fail(GX_ERR_CUDA, "aggregation table overflow at its largest size");
    cap = std::min<uint64_t>(cap * 16, max_cap);
  }
  const bool empty_group = nk == 0 && groups == 0;
  const int64_t G = empty_group ? 1 : (int64_t)groups;
  std::vector<gx_column> made;
  try {
    alloc_outputs(out_types_, G, 0, true, out, s);
    made.assign(out, out + nout);
    AggFinal f{};
    f.nk = nk;
    f.na = nagg;
    for (int j = 0; j < nk; j++) f.key_w[j] = type_size(key_types_[j]);
    for (int j = 0; j < nagg; j++) {
      f.kind[j] = agg_kind_[j];
      f.acc_of[j] = acc_of_[j];
      f.in_flt[j] = in_float_[j] ? 1 : 0;
      f.out_w[j] = type_size(out_types_[nk + j]);
      f.out_f32[j] = out_types_[nk + j] == FLOAT32 ? 1 : 0;
    }
    for (int j = 0; j < nout; j++) {
      f.out_data[j] = out[j].data;
      f.out_mask[j] = out[j].null_mask;
    }
    f.t = t;
    f.counter = (unsigned long long*)(base + (size_t)cap * (4 + 4 + 8 + 8 * nk + 16 * na)) + 4;
    f.empty_group = empty_group ? 1 : 0;
    {
      Plan p = plan_;
      p.nullable = nb;
      f.cnt_rows = agg_counts_are_rows(p, layout_);
    }
    const unsigned grid = (unsigned)std::min<uint64_t>((cap + 255) / 256, (uint64_t)device_sm_count() * 8);
    k_agg_finalize<<<grid, 256, 0, s>>>(f);
    check_cuda(cudaGetLastError(), "k_agg_finalize");
    add_launches(1);
  } catch (...) {
    for (auto& c : made) free_column(c, s);
    dev_free(base, s);
    throw;
  }
  dev_free(base, s);
  for (int j = 0; j < nout; j++) out[j].size = G;
  if (out_groups) *out_groups = G;
}

}  // namespace gx
