// aggregate.h -- fused filter + group-by aggregation (aggregate.cu): the
// aggregation step of a Filter -> Projection -> Aggregate chain
// (ral::operators::compute_aggregations_with_groupby / _without_groupby,
// engine/src/operators/GroupBy.cpp:217-416) over the rows that pass a
// condition, with the aggregation inputs evaluated in the same device pass.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "runtime.h"

namespace gx {

class AggPlan {
 public:
  // key_cols: input column indices of the group keys; inputs[i]: expression
  // text of aggregation i ("" for COUNT(*)); kinds[i]: gx_agg_kind
  AggPlan(const std::vector<int>& schema, const std::vector<bool>& nullable, const std::string& condition,
          const std::vector<int>& key_cols, const std::vector<std::string>& inputs, const std::vector<int>& kinds,
          const KernelConfig& cfg);

  // out: keys then aggregations (library-allocated); *out_groups the groups
  void execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_groups, cudaStream_t s) const;

  int num_outputs() const { return (int)out_types_.size(); }
  const std::vector<int>& output_types() const { return out_types_; }
  // the generated aggregation kernel's source (diagnostics, compile checks)
  std::string kernel_source(const std::vector<bool>& nullable) const;

 private:
  JitKernel kernel(const std::vector<bool>& nullable) const;

  Plan plan_;
  AggLayout layout_;
  KernelConfig cfg_;
  std::vector<int> key_types_;
  std::vector<int> agg_kind_;   // gx_agg_kind per aggregation
  std::vector<int> agg_node_;   // input node per aggregation (-1: COUNT(*))
  std::vector<int> acc_of_;     // accumulator per aggregation (-1: the group's rows)
  std::vector<bool> in_float_;  // per aggregation: floating-point input
  std::vector<int> out_types_;
  mutable std::mutex mu_;
  mutable std::unordered_map<std::string, JitKernel> kcache_;
};

}  // namespace gx
