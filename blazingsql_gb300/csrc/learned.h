// learned.h -- learned conjunct ordering and output sizing (learned.cu).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "runtime.h"

namespace gx {

constexpr int kMaxSketchCols = 32;
constexpr int kSketchParts = 64;  // CTAs per column of the sketch kernel
constexpr int kTrainRing = 64;    // labelled examples kept for training
constexpr int kPredSlots = 3;     // prediction buffers: 0 for in-call sketches, 1-2 for look-ahead

struct LearnerOptions {
  int policy = GX_LEARN_POLICY_LEARNED;
  int warmup_batches = 8;     // labelled batches before the network is used
  int relabel_every = 8;      // every n-th later batch runs the plain path and trains
  int train_steps = 16;       // Adam steps per labelled batch
  float lr = 3e-3f;
  double capacity_margin = 1.5;   // output rows allocated = predicted x margin + slack
  int64_t capacity_slack = 4096;
  int64_t stride_words = 256;  // sketch reads every n-th 32-row word
  int hidden = 64;
  int fast_words = 0;         // words per warp of the single-pass kernel (0: the plan's)
  bool size_outputs = true;   // prediction read back: outputs of the predicted size
  bool async_training = false;  // train on a side stream (overlapped; prediction timing then varies)
  uint64_t seed = 1;
};


// Parameters of an F -> H -> H -> O ReLU MLP, flattened:
// W1[H*F] b1[H] W2[H*H] b2[H] W3[O*H] b3[O] (row-major, out x in).
int mlp_param_count(int F, int H, int O);

// One forward + backward pass of the MLP over M rows of dX on the GPU:
// gradient of loss = mean over M*O of (log sigmoid(z) - Y)^2 into dG, the loss
// into *dloss; dact holds 2*M*H + M*O floats (hidden activations, then z).
void mlp_grad(const float* dP, int F, int H, int O, const float* dX, int M, const float* dY, float* dG, float* dloss,
              float* dact, cudaStream_t s);

// Per column of the plan: the constant a conjunct compares it with (the
// sketch's centre), 0 when none.
std::vector<double> sketch_anchors(const Plan& p, int ncols);

class Learner {
 public:
  // Builds from `base` the plain fixed-order two-pass variant (counting each
  // conjunct's passes under the LEARNED policy) and the fused single-pass
  // variant that takes the conjunct order at launch.
  Learner(const CompiledPlan& base, const LearnerOptions& opt);
  ~Learner();
  Learner(const Learner&) = delete;
  Learner& operator=(const Learner&) = delete;

  void execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows, gx_learned_batch_info* info,
               cudaStream_t s);
  // Look-ahead: sketches (and predicts) a batch that a later execute() will
  // receive, on a side stream, so that execute() finds its prediction ready.
  // report_dev / report_host: where the sketch kernel leaves the prediction
  // for the batch report (mapped host memory; default: the slot's own).
  void prepare(const std::vector<ColumnView>& cols, cudaStream_t s, float* report_dev = nullptr,
               float* report_host = nullptr);
  // execute() on each batch in order, each next batch prepared while the
  // current one runs; out holds num_outputs() columns per batch, batch-major.
  // Single-pass policies with full-size outputs run the whole queue with one
  // host synchronisation at the end.
  void execute_batches(const std::vector<std::vector<ColumnView>>& batches, gx_column* out, int64_t* out_rows,
                       gx_learned_batch_info* infos, cudaStream_t s);
  void save(const std::string& path) const;
  void load(const std::string& path);
  // the sketch features of one batch (diagnostics)
  std::vector<float> features(const std::vector<ColumnView>& cols, cudaStream_t s);
  const std::vector<double>& anchors() const { return anchors_; }
  int num_conjuncts() const { return nconj_; }
  int num_outputs() const { return (int)fast_->plan().outputs.size(); }

 private:
  // host-side record of a batch enqueued without a synchronisation
  struct Deferred {
    unsigned long long* hdr_dev = nullptr;   // device, zeroed: filter header [0, 4), conjunct counts [4, 20)
    uint64_t* status = nullptr;              // device, zeroed: tile status words
    const unsigned long long* hdr = nullptr; // pinned host copy of hdr_dev, valid after the queue's sync
    float* report = nullptr;                 // mapped: z[16] then order[16] (host view)
    float* report_dev = nullptr;             // the same, device view
    const float* feat = nullptr;             // device: the batch's sketch features (queue sketch)
    int* order_dev = nullptr;                // device: the predicted conjunct order (in the header)
    cudaEvent_t pred_ready = nullptr;        // recorded after the batch's prediction
    bool labelled = false;                   // ran the plain fixed-order evaluator (labels)
    int64_t capacity = -1;                   // sized outputs: rows allocated from the prediction
    int64_t pred_rows = -1;                  // sized outputs: the predicted row count
  };
  void execute_one(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                   gx_learned_batch_info* info, cudaStream_t s, Deferred* d);
  // false when the batch's outputs, sized from its prediction, were too small
  // (its row count is then in *out_rows and it must run again)
  bool finish_one(const Deferred& d, int64_t n, gx_column* out, int64_t* out_rows, gx_learned_batch_info* info);
  // the batch's outputs in one allocation of `capacity` rows, masks zeroed
  void alloc_batch_outputs(gx_column* out, int64_t capacity, cudaStream_t s) const;
  bool can_defer() const;
  // queue buffers for up to nb batches (made at construction for kQueueReserve)
  struct QueueSketchLayout {
    size_t o_n = 0, o_tk = 0, o_part = 0, o_feat = 0, total = 0;
  };
  QueueSketchLayout queue_sketch_layout(size_t nb) const;
  void reserve_queue(size_t nb);
  static constexpr size_t kQueueReserve = 64;
  // the loss of the last finished training round, when one has finished
  void poll_training();
  // sketch features of the batch into a prediction slot (and, with predict, the network's z and order)
  void sketch(const std::vector<ColumnView>& cols, bool predict, cudaStream_t s, int slot,
              float* report_dev = nullptr, float* report_host = nullptr);
  std::vector<float> predict_log_sel(const std::vector<ColumnView>& cols, cudaStream_t s);
  void add_example(const unsigned long long* counts, int64_t n, cudaStream_t s, const float* feat);
  // a queue's sketches of every batch in one launch on the side stream, and
  // the prediction of one of its batches
  void sketch_queue(const std::vector<std::vector<ColumnView>>& batches, std::vector<Deferred>& d, cudaStream_t s);
  void predict_queued(Deferred& d, int ev, cudaStream_t s);
  std::vector<uintptr_t> batch_key(const std::vector<ColumnView>& cols) const;
  int take_prepared(const std::vector<ColumnView>& cols, cudaStream_t s);
  void train(int steps, cudaStream_t s);
  void sync_inference_params(cudaStream_t s);
  void release();

  // plain_: the fixed-order two-pass evaluator (the PLAIN policy, and the
  // judge); label_: the fixed-order single pass that also counts each
  // conjunct's passing rows (labelled batches); fast_: the single pass in the
  // order given at launch
  std::shared_ptr<CompiledPlan> plain_, label_, fast_;
  LearnerOptions opt_;
  int ncols_ = 0, nconj_ = 0, F_ = 0, H_ = 0, O_ = 0, nparams_ = 0;
  std::vector<double> conj_cost_;  // bytes per row the conjunct's columns read
  std::vector<double> anchors_;    // per column: the constant its sketch is centred on
  // device buffers
  float* dparams_ = nullptr;  // training copy; dgrad_, dmom_, dvel_ follow
  float* dgrad_ = nullptr;
  float* dmom_ = nullptr;
  float* dvel_ = nullptr;
  float* dinfer_ = nullptr;   // inference copy of the parameters
  struct PredSlot {
    float* feat = nullptr;       // F features of the sketched batch
    float* z = nullptr;          // network outputs (16)
    int* order = nullptr;        // conjunct order (16)
    float* partial = nullptr;    // sketch partials
    unsigned int* ticket = nullptr;
    float* report = nullptr;      // mapped host copy of z[16] then order[16] (host view)
    float* report_dev = nullptr;  // the same memory, device view
    const float* cur_report = nullptr;  // where the current prediction's report goes (host view)
    cudaEvent_t ready = nullptr;
    std::vector<uintptr_t> key;  // the batch it holds (column starts, rows)
    bool valid = false;
  };
  PredSlot slots_[kPredSlots];
  int prep_next_ = 1;
  float* dslots_ = nullptr;   // one allocation for every slot
  cudaEvent_t prep_in_ = nullptr;
  float* dtrainX_ = nullptr;  // ring of labelled examples
  float* dtrainY_ = nullptr;
  float* dsnapX_ = nullptr;   // snapshot of the ring a side-stream round trains on
  float* dsnapY_ = nullptr;
  float* dact_ = nullptr;     // training activations
  unsigned long long* dcounts_ = nullptr;
  float* dcost_ = nullptr;           // per conjunct: bytes per row its columns read
  float* hpinned_ = nullptr;  // pinned host: predictions + loss
  unsigned long long* hcounts_ = nullptr;  // pinned host: per-conjunct pass counts
  char* hqueue_ = nullptr;                 // pinned, mapped: per-batch slots of a deferred queue
  size_t queue_cap_ = 0;                   // batches hqueue_ holds
  // a queue's sketch: device [column descriptors | rows | tickets | partials |
  // features] and its pinned staging for the first three
  char* dqsk_ = nullptr;
  char* hqsk_ = nullptr;
  size_t qsk_cap_ = 0;                     // batches they hold
  static constexpr int kPredAhead = 3;  // a queued batch's prediction is made this many batches ahead
  static constexpr int kPredEvents = 8;  // prediction events, in rotation (> kPredAhead)
  cudaEvent_t qev_[kPredEvents] = {};
  cudaEvent_t qdone_[8] = {};              // batch completion events of a queue, in rotation
  cudaEvent_t qsketch_done_ = nullptr;
  bool qsketch_pending_ = false;           // the main stream has not waited for the queue sketch yet
  cudaStream_t train_stream_ = nullptr;
  cudaStream_t aux_stream_ = nullptr;   // prediction readback for the batch report
  cudaEvent_t train_done_ = nullptr, labels_ready_ = nullptr;
  bool params_pending_ = false;
  bool train_pending_ = false;   // a round was asked for while another ran  // training finished a version not yet copied to dinfer_
  uint64_t seen_ = 0, labelled_ = 0, batches_ = 0;
  int since_label_ = 0;  // single-pass batches since the last labelled one
  int adam_t_ = 0;
  float loss_ = 0.f;
};

}  // namespace gx
