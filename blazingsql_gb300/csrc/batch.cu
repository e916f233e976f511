// batch.cu -- batch runner: many execution-graph batches of one filter plan
// through one persistent kernel launch inside a captured CUDA graph.
//
// The reference evaluates each batch with its own interpreter launch, device
// allocations, uploads and a host synchronisation
// (engine/src/Interpreter/interpreter_cpp.cu:440-594 via
// engine/src/execution_kernels/BatchProcessing.cpp:371-476), a fixed cost that
// dominates small batches.  Here the host writes one descriptor per batch into
// pinned memory and replays a graph of five nodes: descriptor upload, scratch
// clear, the persistent FUSED_BATCHED kernel over every batch's tiles, and the
// per-batch row-count readback.  The block size and rows per warp are chosen
// by an autotuner on the first run and cached per plan, column mix and device.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "batch.h"
#include "jit.h"

namespace gx {

namespace {

uint64_t fnv1a(const std::string& s) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

// autotune results: key -> (warps, words), in memory and optionally on disk
std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tuned;

std::string tune_file() {
  const char* d = std::getenv("GX_AUTOTUNE_CACHE");
  return (d && *d) ? std::string(d) + "/gx_autotune.txt" : std::string();
}

bool tune_lookup(const std::string& key, int* warps, int* words) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  auto it = g_tuned.find(key);
  if (it == g_tuned.end()) {
    const std::string f = tune_file();
    if (!f.empty()) {
      std::ifstream in(f);
      std::string k;
      int w, v;
      while (in >> k >> w >> v) g_tuned[k] = {w, v};
      it = g_tuned.find(key);
    }
  }
  if (it == g_tuned.end()) return false;
  *warps = it->second.first;
  *words = it->second.second;
  return true;
}

void tune_store(const std::string& key, int warps, int words) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tuned[key] = {warps, words};
  const std::string f = tune_file();
  if (!f.empty()) {
    std::ofstream out(f, std::ios::app);
    out << key << ' ' << warps << ' ' << words << '\n';
  }
}

// Zeroes every batch's output masks (the filter kernel ORs boundary words):
// block i clears output i % nout of batch i / nout; blocks past the batch
// count exit.
__global__ void k_clear_masks(const KernelArgs* __restrict__ A, const BatchHeader* __restrict__ hdr, int nout) {
  const int b = blockIdx.x / nout, j = blockIdx.x % nout;
  if (b >= hdr->nbatch) return;
  const KernelArgs& a = A[b];
  uint32_t* m = a.out_mask[j];
  int64_t words = (a.capacity + 31) / 32;
  words = words < 16 ? 16 : (words + 15) / 16 * 16;
  for (int64_t w = threadIdx.x; w < words; w += blockDim.x) m[w] = 0u;
}

}  // namespace

BatchRunner::BatchRunner(const CompiledPlan& base, int max_batches, int64_t max_rows, bool autotune)
    : plan_(base.plan()), base_cfg_(base.config()), max_batches_(max_batches), max_rows_(max_rows),
      autotune_(autotune) {
  if (!plan_.has_filter()) fail(GX_ERR_INVALID, "the batch runner runs plans with a condition");
  if (max_batches < 1 || max_rows < 0) fail(GX_ERR_INVALID, "bad batch runner limits");
  base_cfg_.short_circuit = false;
  base_cfg_.conjunct_order.clear();
  base_cfg_.runtime_order = false;
  base_cfg_.conj_stats = false;
  base_cfg_.dense = true;
  warps_ = base_cfg_.warps;
  words_ = base_cfg_.words;
}

BatchRunner::~BatchRunner() { release(); }

void BatchRunner::release() {
  if (exec_) cudaGraphExecDestroy(exec_);
  if (cap_stream_) cudaStreamDestroy(cap_stream_);
  cudaFree(dargs_);
  cudaFree(dbase_);
  cudaFree(dhdr_);
  cudaFree(dscratch_);
  if (hargs_) cudaFreeHost(hargs_);
  if (hbase_) cudaFreeHost(hbase_);
  if (hhdr_) cudaFreeHost(hhdr_);
  if (hres_) cudaFreeHost(hres_);
  exec_ = nullptr;
  cap_stream_ = nullptr;
  dargs_ = nullptr;
  dbase_ = nullptr;
  dhdr_ = nullptr;
  dscratch_ = nullptr;
  hargs_ = nullptr;
  hbase_ = nullptr;
  hhdr_ = nullptr;
  hres_ = nullptr;
}

int64_t BatchRunner::max_tiles(int words, int warps) const {
  const int64_t tile_rows = (int64_t)words * warps * 32;
  return max_rows_ / tile_rows + max_batches_ + 1;
}

void BatchRunner::ensure_buffers() {
  if (dargs_) return;
  // scratch sized for the smallest tile any candidate uses
  scratch_tiles_ = max_tiles(2, 4);
  auto dmalloc = [](void** p, size_t b, const char* what) {
    const cudaError_t e = cudaMalloc(p, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(e == cudaErrorMemoryAllocation ? GX_ERR_OOM : GX_ERR_CUDA, what);
    }
  };
  try {
    dmalloc((void**)&dargs_, sizeof(KernelArgs) * max_batches_, "batch descriptors");
    dmalloc((void**)&dbase_, 8 * (size_t)(max_batches_ + 1), "batch tile offsets");
    dmalloc((void**)&dhdr_, sizeof(BatchHeader), "batch header");
    dmalloc((void**)&dscratch_, 8 * (size_t)(4 * max_batches_ + scratch_tiles_), "batch scratch");
    check_cuda(cudaMallocHost((void**)&hargs_, sizeof(KernelArgs) * max_batches_), "pinned descriptors");
    check_cuda(cudaMallocHost((void**)&hbase_, 8 * (size_t)(max_batches_ + 1)), "pinned tile offsets");
    check_cuda(cudaMallocHost((void**)&hhdr_, sizeof(BatchHeader)), "pinned header");
    check_cuda(cudaMallocHost((void**)&hres_, 8 * 4 * (size_t)max_batches_), "pinned results");
    check_cuda(cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking), "capture stream");
  } catch (...) {
    release();
    throw;
  }
}

std::shared_ptr<CompiledPlan> BatchRunner::variant(int warps, int words) {
  auto& v = variants_[{warps, words}];
  if (!v) {
    KernelConfig c = base_cfg_;
    c.warps = warps;
    c.words = words;
    c.tune_shape = false;  // the runner tunes its own shape
    v = std::make_shared<CompiledPlan>(plan_, c, GX_FILTER_SINGLE_PASS);
  }
  return v;
}

// Writes the descriptors of `batches` for tiles of words x warps into the
// pinned staging buffers; returns the total tile count.
int64_t BatchRunner::stage(const std::vector<std::vector<ColumnView>>& batches, const gx_column* out,
                           int warps, int words) {
  const int nb = (int)batches.size();
  const int nout = (int)plan_.outputs.size();
  const int64_t tile_rows = (int64_t)words * warps * 32;
  uint64_t* status = dscratch_ + 4 * (size_t)max_batches_;
  int64_t tiles = 0;
  for (int b = 0; b < nb; b++) {
    KernelArgs& a = hargs_[b];
    std::memset(&a, 0, sizeof a);
    const auto& cols = batches[b];
    const int64_t n = cols.empty() ? 0 : cols[0].size;
    for (size_t i = 0; i < cols.size(); i++) {
      a.in_data[i] = cols[i].data;
      a.in_mask[i] = cols[i].mask;
      a.in_off[i] = cols[i].offset;
    }
    for (int j = 0; j < nout; j++) {
      a.out_data[j] = out[(size_t)b * nout + j].data;
      a.out_mask[j] = out[(size_t)b * nout + j].null_mask;
    }
    int64_t cap = nout ? out[(size_t)b * nout].capacity : 0;
    for (int j = 1; j < nout; j++) cap = std::min<int64_t>(cap, out[(size_t)b * nout + j].capacity);
    a.n = n;
    a.capacity = cap;
    a.tile_status = status + tiles;
    a.out_count = (unsigned long long*)(dscratch_ + 4 * (size_t)b + 1);
    a.err = (int*)(dscratch_ + 4 * (size_t)b + 2);
    a.seed = plan_.rand_seed;
    for (int i = 0; i < 16; i++) a.order[i] = i;
    hbase_[b] = tiles;
    tiles += (n + tile_rows - 1) / tile_rows;
  }
  hbase_[nb] = tiles;
  if (tiles > scratch_tiles_) fail(GX_ERR_INVALID, "batches exceed the runner's row limit");
  hhdr_->tile_counter = 0;
  hhdr_->total_tiles = tiles;
  hhdr_->nbatch = nb;
  hhdr_->pad = 0;
  return tiles;
}

// the run's device work on stream s: upload, clear, persistent kernel, readback
void BatchRunner::enqueue(const JitKernel& k, cudaStream_t s, bool timed) {
  check_cuda(cudaMemcpyAsync(dargs_, hargs_, sizeof(KernelArgs) * max_batches_, cudaMemcpyHostToDevice, s),
             "descriptor upload");
  check_cuda(cudaMemcpyAsync(dbase_, hbase_, 8 * (size_t)(max_batches_ + 1), cudaMemcpyHostToDevice, s),
             "tile offsets upload");
  check_cuda(cudaMemcpyAsync(dhdr_, hhdr_, sizeof(BatchHeader), cudaMemcpyHostToDevice, s), "header upload");
  check_cuda(cudaMemsetAsync(dscratch_, 0, 8 * (size_t)(4 * max_batches_ + scratch_tiles_), s), "scratch clear");
  const int nout = (int)plan_.outputs.size();
  k_clear_masks<<<max_batches_ * nout, 256, 0, s>>>(dargs_, dhdr_, nout);
  check_cuda(cudaGetLastError(), "k_clear_masks");
  KernelArgs* pa = dargs_;
  long long* pb = dbase_;
  BatchHeader* ph = dhdr_;
  void* params[] = {&pa, &pb, &ph};
  const int grid = device_sm_count() * k.max_blocks_per_sm;
  launch_raw(k, grid, s, params, timed);
  check_cuda(cudaMemcpyAsync(hres_, dscratch_, 8 * 4 * (size_t)max_batches_, cudaMemcpyDeviceToHost, s),
             "result readback");
}

void BatchRunner::capture(const JitKernel& k) {
  if (exec_ && captured_fn_ == k.fn) return;
  if (exec_) {
    cudaGraphExecDestroy(exec_);
    exec_ = nullptr;
  }
  cudaGraph_t graph = nullptr;
  check_cuda(cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
  try {
    enqueue(k, cap_stream_, false);
  } catch (...) {
    cudaStreamEndCapture(cap_stream_, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  check_cuda(cudaStreamEndCapture(cap_stream_, &graph), "end capture");
  const cudaError_t e = cudaGraphInstantiate(&exec_, graph, 0);
  cudaGraphDestroy(graph);
  check_cuda(e, "graph instantiate");
  captured_fn_ = k.fn;
}

std::string BatchRunner::tune_key(const std::vector<bool>& nullable) const {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof prop);
  cudaGetDeviceProperties(&prop, dev);
  std::string name = prop.name;
  for (char& c : name)
    if (c == ' ') c = '_';
  std::vector<bool> nb = nullable;
  Plan p = plan_;
  p.nullable = nb;
  const std::string src = generate_kernel(p, KernelKind::FUSED_BATCHED, base_cfg_, "k");
  char buf[32];
  std::snprintf(buf, sizeof buf, "%016llx", (unsigned long long)fnv1a(src));
  return std::string(buf) + "/" + name;
}

// Times each candidate (block warps x words per warp) on this run's batches and
// keeps the fastest.  The candidates' outputs are written and overwritten in
// the run's own output buffers; the final run rewrites them.
void BatchRunner::tune(const std::vector<std::vector<ColumnView>>& batches, gx_column* out,
                       const std::vector<bool>& nullable, cudaStream_t s) {
  const std::string key = tune_key(nullable);
  int w = 0, v = 0;
  if (tune_lookup(key, &w, &v)) {
    warps_ = w;
    words_ = v;
    tuned_ = true;
    return;
  }
  static const int cand[][2] = {{4, 2}, {4, 4}, {4, 8}, {8, 2}, {8, 4}, {2, 8}, {1, 16}};
  float best = 1e30f;
  cudaEvent_t e0, e1;
  check_cuda(cudaEventCreate(&e0), "event");
  check_cuda(cudaEventCreate(&e1), "event");
  for (const auto& c : cand) {
    const JitKernel k = variant(c[0], c[1])->kernel_for(KernelKind::FUSED_BATCHED, nullable);
    stage(batches, out, c[0], c[1]);
    float ms = 0.f;
    for (int rep = 0; rep < 2; rep++) {  // the first run warms caches and the module
      check_cuda(cudaEventRecord(e0, s), "event");
      enqueue(k, s, false);
      check_cuda(cudaEventRecord(e1, s), "event");
      check_cuda(cudaEventSynchronize(e1), "event");
      cudaEventElapsedTime(&ms, e0, e1);
    }
    if (ms < best) {
      best = ms;
      warps_ = c[0];
      words_ = c[1];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  tune_store(key, warps_, words_);
  tuned_ = true;
}

void BatchRunner::run(const std::vector<std::vector<ColumnView>>& batches, gx_column* out, int64_t* out_rows,
                      cudaStream_t s) {
  const int nb = (int)batches.size();
  if (nb > max_batches_) fail(GX_ERR_INVALID, "more batches than the runner was created for");
  const int nout = (int)plan_.outputs.size();
  if (nout == 0) fail(GX_ERR_INVALID, "plan has no outputs");
  int64_t rows_total = 0;
  std::vector<bool> nullable(plan_.schema.size(), false);
  for (const auto& cols : batches) {
    if (cols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
    for (size_t i = 0; i < cols.size(); i++) {
      if (cols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
      if (cols[i].mask) nullable[i] = true;
    }
    rows_total += cols.empty() ? 0 : cols[0].size;
  }
  if (rows_total > max_rows_) fail(GX_ERR_INVALID, "batches exceed the runner's row limit");
  ensure_buffers();
  const bool caller_bufs = out[0].data != nullptr;
  std::vector<gx_column> made;
  try {
    if (!caller_bufs) {
      std::vector<int> types;
      std::vector<int64_t> caps;
      for (const auto& cols : batches)
        for (int j = 0; j < nout; j++) {
          types.push_back(plan_.outputs[j].type);
          caps.push_back(cols.empty() ? 0 : cols[0].size);
        }
      alloc_output_set(types, caps, false, out, s);  // the graph clears the masks
      made.assign(out, out + (size_t)nb * nout);
    } else {
      for (size_t b = 0; b < (size_t)nb; b++)
        for (int j = 0; j < nout; j++) {
          gx_column& c = out[b * nout + j];
          if (!c.data || !c.null_mask) fail(GX_ERR_INVALID, "caller output buffer missing");
          c.type_id = plan_.outputs[j].type;
        }
    }
    if (autotune_ && !tuned_ && rows_total >= (int64_t)1 << 20) tune(batches, out, nullable, s);
    const JitKernel k = variant(warps_, words_)->kernel_for(KernelKind::FUSED_BATCHED, nullable);
    stage(batches, out, warps_, words_);
    capture(k);
    const bool timed = kernel_timing_enabled();
    if (timed) {
      // timing mode: the same work outside the graph, with events around the kernel
      enqueue(k, s, true);
    } else {
      check_cuda(cudaGraphLaunch(exec_, s), "graph launch");
      add_launches(1);
    }
    check_cuda(cudaStreamSynchronize(s), "batch sync");
    int64_t err = 0;
    for (int b = 0; b < nb; b++) {
      const int64_t rows = (int64_t)hres_[4 * (size_t)b + 1];
      err |= (int64_t)(hres_[4 * (size_t)b + 2] & 0xFFFFFFFFull);
      if (out_rows) out_rows[b] = rows;
      for (int j = 0; j < nout; j++) out[(size_t)b * nout + j].size = rows;
    }
    if (err) fail(GX_ERR_TIMEOUT, "compaction look-back wait timed out");
    for (int b = 0; b < nb; b++)
      for (int j = 0; j < nout; j++) {
        gx_column& c = out[(size_t)b * nout + j];
        if (c.size > c.capacity) fail(GX_ERR_CAPACITY, "output capacity too small");
        const OutSpec& os = plan_.outputs[j];
        if (os.kind == OutSpec::BROADCAST) {
          launch_fill(c.data, type_size(os.type), os.lit_bits_as_element(), c.size, s);
          launch_fill_mask(c.null_mask, c.size, os.lit_valid, mask_words_for(c.capacity), s);
        }
      }
  } catch (...) {
    for (auto& c : made) free_column(c, s);
    throw;
  }
}


// ------------------------------------------------------------------ stream
BatchStream::BatchStream(const CompiledPlan& base, int max_batches, int64_t max_rows, int warps, int words)
    : plan_(base.plan()), max_batches_(max_batches), max_rows_(max_rows) {
  if (!plan_.has_filter()) fail(GX_ERR_INVALID, "a batch stream runs plans with a condition");
  if (!base.can_defer()) fail(GX_ERR_INVALID, "a batch stream needs a plan without literal outputs");
  if (max_batches < 1 || max_rows < 0) fail(GX_ERR_INVALID, "bad batch stream limits");
  KernelConfig c = base.config();
  c.short_circuit = false;
  c.conjunct_order.clear();
  c.runtime_order = false;
  c.conj_stats = false;
  c.dense = true;
  c.tune_shape = false;
  if (warps > 0) c.warps = warps;
  if (words > 0) c.words = words;
  if (c.warps < 1 || c.warps > 32 || c.words < 1 || c.words > 32) fail(GX_ERR_INVALID, "bad block shape");
  variant_ = std::make_shared<CompiledPlan>(plan_, c, GX_FILTER_SINGLE_PASS);
  tile_rows_ = (int64_t)c.warps * c.words * 32;
  max_tiles_ = max_rows_ / tile_rows_ + max_batches_ + 1;
  // a batch's output rows start on a 32-row boundary (its mask words are its own)
  arena_rows_ = max_rows_ + 32 * (int64_t)max_batches_;
  // the kernel reads validity through a mask pointer that may be null, so one
  // kernel serves batches with and without masks
  kernel_ = variant_->kernel_for(KernelKind::FUSED_STREAM, std::vector<bool>(plan_.schema.size(), true));
  auto dmalloc = [](void** p, size_t b, const char* what) {
    const cudaError_t e = cudaMalloc(p, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(e == cudaErrorMemoryAllocation ? GX_ERR_OOM : GX_ERR_CUDA, what);
    }
  };
  try {
    dmalloc((void**)&dargs_, kStreamArgsStride * max_batches_, "stream descriptors");
    dmalloc((void**)&dbase_, 8 * (size_t)(max_batches_ + 1), "stream tile offsets");
    dmalloc((void**)&dhdr_, sizeof(BatchHeader), "stream header");
    dmalloc((void**)&dscratch_, 8 * (size_t)(4 * max_batches_ + max_tiles_), "stream scratch");
    dmalloc((void**)&dwerr_, 16, "stream wait flag");
    check_cuda(cudaMallocHost((void**)&hargs_, kStreamArgsStride * max_batches_), "pinned descriptors");
    check_cuda(cudaMallocHost((void**)&hbase_, 8 * (size_t)(max_batches_ + 1)), "pinned tile offsets");
    check_cuda(cudaMallocHost((void**)&hpub_, 8 * (size_t)max_batches_), "pinned published counts");
    check_cuda(cudaMallocHost((void**)&hflag_, 16), "pinned flags");
    check_cuda(cudaMallocHost((void**)&hres_, 8 * 4 * (size_t)max_batches_), "pinned results");
    check_cuda(cudaStreamCreateWithFlags(&push_stream_, cudaStreamNonBlocking), "push stream");
    check_cuda(cudaEventCreateWithFlags(&started_, cudaEventDisableTiming), "event");
  } catch (...) {
    release();
    throw;
  }
}

BatchStream::~BatchStream() {
  if (running_) {
    // close the queue so the kernel stops before its buffers go
    hflag_[0] = 1;
    cudaMemcpyAsync(&dhdr_->pad, hflag_, 4, cudaMemcpyHostToDevice, push_stream_);
    cudaStreamSynchronize(push_stream_);
    cudaStreamSynchronize(s_);
    dev_free(arena_, s_);
    cudaStreamSynchronize(s_);
  }
  release();
}

void BatchStream::release() {
  if (push_stream_) cudaStreamDestroy(push_stream_);
  if (started_) cudaEventDestroy(started_);
  cudaFree(dargs_);
  cudaFree(dbase_);
  cudaFree(dhdr_);
  cudaFree(dscratch_);
  cudaFree(dwerr_);
  if (hargs_) cudaFreeHost(hargs_);
  if (hbase_) cudaFreeHost(hbase_);
  if (hpub_) cudaFreeHost(hpub_);
  if (hflag_) cudaFreeHost(hflag_);
  if (hres_) cudaFreeHost(hres_);
  push_stream_ = nullptr;
  started_ = nullptr;
  dargs_ = nullptr;
  dbase_ = nullptr;
  dhdr_ = nullptr;
  dscratch_ = nullptr;
  dwerr_ = nullptr;
  hargs_ = nullptr;
  hbase_ = nullptr;
  hpub_ = nullptr;
  hflag_ = nullptr;
  hres_ = nullptr;
}

void BatchStream::start(cudaStream_t s) {
  if (running_) fail(GX_ERR_INVALID, "the batch stream is already running");
  const int nout = num_outputs();
  // this session's outputs: [masks of every output | data of every output]
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  moff_.assign(nout, 0);
  doff_.assign(nout, 0);
  size_t total = 0;
  for (int j = 0; j < nout; j++) {
    moff_[j] = total;
    total += al((size_t)(arena_rows_ / 32 + 16) * 4);
  }
  const size_t masks = total;
  for (int j = 0; j < nout; j++) {
    doff_[j] = total;
    total += al(std::max<size_t>(64, (size_t)arena_rows_ * type_size(plan_.outputs[j].type)));
  }
  arena_ = (char*)dev_alloc(total, s);
  try {
    check_cuda(cudaMemsetAsync(arena_, 0, masks, s), "stream masks");
    check_cuda(cudaMemsetAsync(dscratch_, 0, 8 * (size_t)(4 * max_batches_ + max_tiles_), s), "stream scratch");
    // tile offsets of unpublished batches read as INT64_MAX-like (0x7f..7f)
    check_cuda(cudaMemsetAsync(dbase_, 0x7f, 8 * (size_t)(max_batches_ + 1), s), "stream offsets");
    check_cuda(cudaMemsetAsync(dbase_, 0, 8, s), "stream offsets");
    check_cuda(cudaMemsetAsync(dhdr_, 0, sizeof(BatchHeader), s), "stream header");
    check_cuda(cudaMemsetAsync(dwerr_, 0, 16, s), "stream wait flag");
    check_cuda(cudaEventRecord(started_, s), "stream event");
    check_cuda(cudaStreamWaitEvent(push_stream_, started_, 0), "stream wait");
    KernelArgs* pa = dargs_;
    long long* pb = dbase_;
    BatchHeader* ph = dhdr_;
    int* pw = dwerr_;
    unsigned polls = wait_polls_;
    void* params[] = {&pa, &pb, &ph, &pw, &polls};
    const int grid = device_sm_count() * kernel_.max_blocks_per_sm;
    launch_raw(kernel_, grid, s, params, false);
  } catch (...) {
    dev_free(arena_, s);
    arena_ = nullptr;
    throw;
  }
  add_launches(1);
  hbase_[0] = 0;
  s_ = s;
  running_ = true;
  count_ = 0;
  tiles_ = 0;
  rows_used_ = 0;
  row_off_.clear();
  rows_in_.clear();
}

int BatchStream::push(const std::vector<ColumnView>& cols) {
  if (!running_) fail(GX_ERR_INVALID, "the batch stream is not running");
  if (count_ >= max_batches_) fail(GX_ERR_INVALID, "more batches than the stream was created for");
  if (cols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < cols.size(); i++)
    if (cols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const int64_t tiles = (n + tile_rows_ - 1) / tile_rows_;
  const int64_t need = (std::max<int64_t>(n, 1) + 31) / 32 * 32;  // distinct, word-aligned output rows
  if (tiles_ + tiles > max_tiles_ || rows_used_ + need > arena_rows_)
    fail(GX_ERR_INVALID, "batches exceed the stream's row limit");
  const int b = count_;
  const int nout = num_outputs();
  KernelArgs& a = *(KernelArgs*)((char*)hargs_ + (size_t)b * kStreamArgsStride);
  std::memset(&a, 0, sizeof a);
  for (size_t i = 0; i < cols.size(); i++) {
    a.in_data[i] = cols[i].data;
    a.in_mask[i] = cols[i].mask;
    a.in_off[i] = cols[i].offset;
  }
  for (int j = 0; j < nout; j++) {
    a.out_data[j] = arena_ + doff_[j] + (size_t)rows_used_ * type_size(plan_.outputs[j].type);
    a.out_mask[j] = (uint32_t*)(arena_ + moff_[j]) + rows_used_ / 32;
  }
  a.n = n;
  a.capacity = n;
  a.tile_status = dscratch_ + 4 * (size_t)max_batches_ + tiles_;
  a.out_count = (unsigned long long*)(dscratch_ + 4 * (size_t)b + 1);
  a.err = (int*)(dscratch_ + 4 * (size_t)b + 2);
  a.seed = plan_.rand_seed;
  for (int i = 0; i < 16; i++) a.order[i] = i;
  hbase_[b + 1] = tiles_ + tiles;
  hpub_[b] = tiles_ + tiles;
  // descriptor and offsets first; the published tile count last (the kernel
  // reads a batch's descriptor only after seeing its tiles published)
  check_cuda(cudaMemcpyAsync((char*)dargs_ + (size_t)b * kStreamArgsStride, &a, sizeof(KernelArgs),
                             cudaMemcpyHostToDevice, push_stream_),
             "stream descriptor");
  check_cuda(cudaMemcpyAsync(dbase_ + b + 1, hbase_ + b + 1, 8, cudaMemcpyHostToDevice, push_stream_),
             "stream offsets");
  check_cuda(cudaMemcpyAsync(&dhdr_->total_tiles, hpub_ + b, 8, cudaMemcpyHostToDevice, push_stream_),
             "stream publish");
  row_off_.push_back(rows_used_);
  rows_in_.push_back(n);
  tiles_ += tiles;
  rows_used_ += need;
  return count_++;
}

void BatchStream::finish(gx_column* out, int64_t* out_rows, int max_out_batches) {
  if (!running_) fail(GX_ERR_INVALID, "the batch stream is not running");
  if (count_ > max_out_batches) fail(GX_ERR_INVALID, "output array too small for the pushed batches");
  running_ = false;
  hflag_[0] = 1;
  const int nb = count_;
  const int nout = num_outputs();
  cudaError_t e = cudaMemcpyAsync(&dhdr_->pad, hflag_, 4, cudaMemcpyHostToDevice, push_stream_);
  if (e == cudaSuccess && nb > 0)
    e = cudaMemcpyAsync(hres_, dscratch_, 8 * 4 * (size_t)nb, cudaMemcpyDeviceToHost, s_);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hflag_ + 1, dwerr_, 4, cudaMemcpyDeviceToHost, s_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(push_stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
  if (e != cudaSuccess) {
    dev_free(arena_, s_);
    arena_ = nullptr;
    check_cuda(e, "stream finish");
  }
  int64_t err = hflag_[1] ? 1 : 0;
  for (int b = 0; b < nb; b++) err |= (int64_t)(hres_[4 * (size_t)b + 2] & 0xFFFFFFFFull);
  if (err || nb == 0) {
    dev_free(arena_, s_);
    arena_ = nullptr;
    if (hflag_[1]) fail(GX_ERR_TIMEOUT, "the stream's kernel waited too long for a batch");
    if (err) fail(GX_ERR_TIMEOUT, "compaction look-back wait timed out");
    return;
  }
  for (int b = 0; b < nb; b++) {
    const int64_t rows = (int64_t)hres_[4 * (size_t)b + 1];
    if (out_rows) out_rows[b] = rows;
    for (int j = 0; j < nout; j++) {
      gx_column& c = out[(size_t)b * nout + j];
      c = gx_column{};
      c.type_id = plan_.outputs[j].type;
      c.data = arena_ + doff_[j] + (size_t)row_off_[b] * type_size(plan_.outputs[j].type);
      c.null_mask = (uint32_t*)(arena_ + moff_[j]) + row_off_[b] / 32;
      c.size = rows;
      c.capacity = std::max<int64_t>(rows_in_[b], 0);
    }
  }
  adopt_output_views(arena_, out, nb * nout);
  arena_ = nullptr;
}

}  // namespace gx

// ------------------------------------------------------------------ C ABI
struct gx_batch_runner {
  std::unique_ptr<gx::BatchRunner> r;
};
struct gx_batch_stream {
  std::unique_ptr<gx::BatchStream> s;
};

namespace gx {
const CompiledPlan* single_chunk(const gx_plan* plan);  // capi.cpp
}  // namespace gx

namespace {
void put_status(gx_status_info* st, int code, const char* msg) {
  if (!st) return;
  st->code = code;
  std::snprintf(st->message, sizeof st->message, "%s", msg ? msg : "");
}

template <class F>
int guarded_call(gx_status_info* st, F&& f) {
  try {
    f();
    put_status(st, GX_OK, "");
    return GX_OK;
  } catch (const gx::Error& e) {
    put_status(st, e.code, e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    put_status(st, GX_ERR_OOM, "host allocation failed");
    return GX_ERR_OOM;
  } catch (const std::exception& e) {
    put_status(st, GX_ERR_INVALID, e.what());
    return GX_ERR_INVALID;
  }
}
}  // namespace

extern "C" {

gx_batch_runner* gx_batch_runner_create(const gx_plan* plan, int max_batches, int64_t max_total_rows, int autotune,
                                        gx_status_info* status) {
  gx_batch_runner* out = nullptr;
  guarded_call(status, [&] {
    const gx::CompiledPlan* cp = gx::single_chunk(plan);
    if (!cp) gx::fail(GX_ERR_INVALID, "a batch runner needs a compiled plan with at most 32 outputs "
                                      "over at most 64 columns");
    out = new gx_batch_runner{std::make_unique<gx::BatchRunner>(*cp, max_batches, max_total_rows, autotune != 0)};
  });
  return out;
}

int gx_batch_runner_run(gx_batch_runner* runner, const gx_column_view* columns, int num_batches, int num_columns,
                        gx_column* out, int64_t* out_rows, void* stream, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!runner || !out || num_batches < 1 || num_columns < 0 || (num_columns > 0 && !columns))
      gx::fail(GX_ERR_INVALID, "bad arguments");
    std::vector<std::vector<gx::ColumnView>> batches;
    batches.reserve(num_batches);
    for (int b = 0; b < num_batches; b++)
      batches.push_back(gx::to_views(columns + (size_t)b * num_columns, num_columns));
    runner->r->run(batches, out, out_rows, (cudaStream_t)stream);
  });
}

int gx_batch_runner_config(const gx_batch_runner* runner, int32_t* block_threads, int32_t* words_per_warp) {
  if (!runner) return GX_ERR_INVALID;
  if (block_threads) *block_threads = runner->r->warps() * 32;
  if (words_per_warp) *words_per_warp = runner->r->words();
  return GX_OK;
}

void gx_batch_runner_destroy(gx_batch_runner* runner) { delete runner; }

gx_batch_stream* gx_batch_stream_create(const gx_plan* plan, int max_batches, int64_t max_total_rows,
                                        int block_threads, int words_per_warp, gx_status_info* status) {
  gx_batch_stream* out = nullptr;
  guarded_call(status, [&] {
    const gx::CompiledPlan* cp = gx::single_chunk(plan);
    if (!cp) gx::fail(GX_ERR_INVALID, "a batch stream needs a compiled plan with at most 32 outputs "
                                      "over at most 64 columns");
    if (block_threads % 32 != 0) gx::fail(GX_ERR_INVALID, "block_threads must be a multiple of 32");
    out = new gx_batch_stream{std::make_unique<gx::BatchStream>(*cp, max_batches, max_total_rows, block_threads / 32,
                                                                 words_per_warp)};
  });
  return out;
}

int gx_batch_stream_start(gx_batch_stream* st, void* stream, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!st) gx::fail(GX_ERR_INVALID, "null batch stream");
    st->s->start((cudaStream_t)stream);
  });
}

int gx_batch_stream_push(gx_batch_stream* st, const gx_column_view* columns, int num_columns, int* batch_index,
                         gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!st || num_columns < 0 || (num_columns > 0 && !columns)) gx::fail(GX_ERR_INVALID, "bad arguments");
    const int b = st->s->push(gx::to_views(columns, num_columns));
    if (batch_index) *batch_index = b;
  });
}

int gx_batch_stream_finish(gx_batch_stream* st, gx_column* out, int64_t* out_rows, int max_batches,
                           gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!st || (max_batches > 0 && !out)) gx::fail(GX_ERR_INVALID, "bad arguments");
    st->s->finish(out, out_rows, max_batches);
  });
}

void gx_batch_stream_destroy(gx_batch_stream* st) { delete st; }

int gx_debug_batch_stream_wait_polls(gx_batch_stream* st, uint32_t polls) {
  if (!st) return GX_ERR_INVALID;
  st->s->set_wait_polls(polls);
  return GX_OK;
}

}  // extern "C"
