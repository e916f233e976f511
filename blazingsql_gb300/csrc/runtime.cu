// runtime.cu -- plan execution and the library's precompiled helper kernels.
#include "runtime.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <unordered_map>

#include "driver.h"

namespace gx {

// ------------------------------------------------------------------ helpers
void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  cudaGetLastError();  // clear sticky-free errors
  fail(e == cudaErrorMemoryAllocation ? GX_ERR_OOM : GX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {
std::atomic<bool> g_timing{false};
std::atomic<int64_t> g_launches{0};
thread_local double t_kernel_ms = 0.0;
std::atomic<int> g_fail_countdown{0};
std::mutex g_pool_mu;
std::unordered_map<int, bool> g_pool_ready;

void ensure_pool() {
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (g_pool_ready[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;  // keep freed blocks cached in the pool
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  g_pool_ready[dev] = true;
}
}  // namespace

void debug_fail_allocation(int n) { g_fail_countdown.store(n); }

void set_kernel_timing(bool on) { g_timing.store(on); }
bool kernel_timing_enabled() { return g_timing.load(); }
double kernel_ms(bool reset) {
  const double v = t_kernel_ms;
  if (reset) t_kernel_ms = 0.0;
  return v;
}
void add_launches(int64_t n) { g_launches.fetch_add(n); }

int64_t launch_count() { return g_launches.load(); }

void* dev_alloc(size_t bytes, cudaStream_t s) {
  int c = g_fail_countdown.load();
  while (c > 0) {
    if (g_fail_countdown.compare_exchange_weak(c, c - 1)) {
      if (c == 1) fail(GX_ERR_OOM, "injected allocation failure");
      break;
    }
  }
  ensure_pool();
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes ? bytes : 64, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? GX_ERR_OOM : GX_ERR_CUDA,
         std::string("cudaMallocAsync(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
  }
  return p;
}

void dev_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

std::vector<ColumnView> to_views(const gx_column_view* cols, int n) {
  if (n < 0 || (n > 0 && !cols)) fail(GX_ERR_INVALID, "null column array");
  std::vector<ColumnView> v;
  for (int i = 0; i < n; i++) {
    const gx_column_view& c = cols[i];
    const bool str = c.type_id == STRING;
    if (str && !c.string_offsets) fail(GX_ERR_INVALID, "a string column needs its offsets");
    if (!str && type_size(c.type_id) == 0)
      fail(GX_ERR_UNSUPPORTED, "unsupported column type " + std::to_string(c.type_id));
    if (c.size < 0 || c.offset < 0) fail(GX_ERR_INVALID, "negative column size/offset");
    if (!str && c.size > 0 && !c.data) fail(GX_ERR_INVALID, "column data pointer is null");
    if (i > 0 && c.size != cols[0].size) fail(GX_ERR_INVALID, "columns of one table must have equal sizes");
    ColumnView cv{c.type_id, c.data, c.null_mask, c.offset, c.size};
    if (str) cv.str_offsets = c.string_offsets;
    v.push_back(cv);
  }
  return v;
}

static int64_t mask_words_padded(int64_t rows) {
  int64_t w = (rows + 31) / 32;
  w = (w + 15) / 16 * 16;
  return w < 16 ? 16 : w;
}

gx_column alloc_column(int type, int64_t capacity, cudaStream_t s) {
  gx_column c{};
  c.type_id = type;
  c.capacity = capacity;
  c.size = 0;
  size_t bytes = (size_t)capacity * type_size(type);
  bytes = (bytes + 63) / 64 * 64;
  c.data = dev_alloc(bytes ? bytes : 64, s);
  try {
    c.null_mask = (uint32_t*)dev_alloc((size_t)mask_words_padded(capacity) * 4, s);
  } catch (...) {
    dev_free(c.data, s);
    throw;
  }
  return c;
}

// Output columns of one call share one allocation (an arena) laid out as
// [scratch | every mask | every data buffer]; the arena is released when the
// last of its columns is freed.  Columns are found by their data pointer.
struct OutputArena {
  void* base;
  int refs;
};
static std::mutex g_arena_mu;
static std::unordered_map<void*, OutputArena*> g_arena_of;

void* alloc_outputs(const std::vector<int>& types, int64_t capacity, size_t scratch_bytes, bool zero_masks,
                    gx_column* out, cudaStream_t s) {
  const int nout = (int)types.size();
  if (nout == 0) fail(GX_ERR_INVALID, "no output columns");
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t sb = al(scratch_bytes);
  const size_t mb = al((size_t)mask_words_padded(capacity) * 4);
  size_t total = sb + mb * nout;
  std::vector<size_t> doff(nout);
  for (int j = 0; j < nout; j++) {
    doff[j] = total;
    total += al(std::max<size_t>(64, (size_t)capacity * type_size(types[j])));
  }
  char* base = (char*)dev_alloc(total, s);
  const size_t zero = zero_masks ? sb + mb * nout : sb;
  if (zero) {
    const cudaError_t e = cudaMemsetAsync(base, 0, zero, s);
    if (e != cudaSuccess) {
      dev_free(base, s);
      check_cuda(e, "output arena memset");
    }
  }
  auto* ar = new OutputArena{base, nout};
  std::lock_guard<std::mutex> g(g_arena_mu);
  for (int j = 0; j < nout; j++) {
    out[j] = gx_column{};
    out[j].type_id = types[j];
    out[j].data = base + doff[j];
    out[j].null_mask = (uint32_t*)(base + sb + mb * j);
    out[j].capacity = capacity;
    g_arena_of[out[j].data] = ar;
  }
  return sb ? base : nullptr;
}

void alloc_output_set(const std::vector<int>& types, const std::vector<int64_t>& caps, bool zero_masks,
                      gx_column* out, cudaStream_t s) {
  const size_t nout = types.size();
  if (nout == 0) return;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t mtotal = 0;
  std::vector<size_t> moff(nout), doff(nout);
  for (size_t j = 0; j < nout; j++) {
    moff[j] = mtotal;
    mtotal += al((size_t)mask_words_padded(caps[j]) * 4);
  }
  size_t total = mtotal;
  for (size_t j = 0; j < nout; j++) {
    doff[j] = total;
    total += al(std::max<size_t>(64, (size_t)caps[j] * type_size(types[j])));
  }
  char* base = (char*)dev_alloc(total, s);
  if (zero_masks) {
    const cudaError_t e = cudaMemsetAsync(base, 0, mtotal, s);
    if (e != cudaSuccess) {
      dev_free(base, s);
      check_cuda(e, "output set memset");
    }
  }
  auto* ar = new OutputArena{base, (int)nout};
  std::lock_guard<std::mutex> g(g_arena_mu);
  for (size_t j = 0; j < nout; j++) {
    out[j] = gx_column{};
    out[j].type_id = types[j];
    out[j].data = base + doff[j];
    out[j].null_mask = (uint32_t*)(base + moff[j]);
    out[j].capacity = caps[j];
    g_arena_of[out[j].data] = ar;
  }
}

void adopt_output_views(void* base, gx_column* cols, int n) {
  if (n <= 0) return;
  auto* ar = new OutputArena{base, n};
  std::lock_guard<std::mutex> g(g_arena_mu);
  for (int i = 0; i < n; i++) g_arena_of[cols[i].data] = ar;
}

void* alloc_queue_scratch(const std::vector<int64_t>& status_words, uint64_t** status, cudaStream_t s) {
  const size_t nb = status_words.size();
  if (nb == 0) return nullptr;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t total = al(nb * kQueueHeaderBytes);
  std::vector<size_t> soff(nb);
  for (size_t b = 0; b < nb; b++) {
    soff[b] = total;
    total += al((size_t)std::max<int64_t>(status_words[b], 1) * 8);
  }
  char* base = (char*)dev_alloc(total, s);
  const cudaError_t e = cudaMemsetAsync(base, 0, total, s);
  if (e != cudaSuccess) {
    dev_free(base, s);
    check_cuda(e, "queue scratch memset");
  }
  for (size_t b = 0; b < nb; b++) status[b] = (uint64_t*)(base + soff[b]);
  return base;
}

void* alloc_output_queue(const std::vector<int>& types, const std::vector<int64_t>& caps,
                         const std::vector<int64_t>& status_words, gx_column* out, uint64_t** status,
                         cudaStream_t s) {
  const size_t nout = types.size();
  const size_t nb = caps.size();
  if (nout == 0) fail(GX_ERR_INVALID, "no output columns");
  if (nb == 0) return nullptr;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  // [headers: 256 bytes per batch | per batch: tile status, masks | data]
  size_t total = al(nb * kQueueHeaderBytes);
  std::vector<size_t> soff(nb), moff(nb * nout), doff(nb * nout);
  for (size_t b = 0; b < nb; b++) {
    soff[b] = total;
    total += al((size_t)std::max<int64_t>(status_words[b], 1) * 8);
    for (size_t j = 0; j < nout; j++) {
      moff[b * nout + j] = total;
      total += al((size_t)mask_words_padded(caps[b]) * 4);
    }
  }
  const size_t zero = total;
  for (size_t b = 0; b < nb; b++)
    for (size_t j = 0; j < nout; j++) {
      doff[b * nout + j] = total;
      total += al(std::max<size_t>(64, (size_t)caps[b] * type_size(types[j])));
    }
  char* base = (char*)dev_alloc(total, s);
  const cudaError_t e = cudaMemsetAsync(base, 0, zero, s);
  if (e != cudaSuccess) {
    dev_free(base, s);
    check_cuda(e, "output queue memset");
  }
  auto* ar = new OutputArena{base, (int)(nb * nout)};
  std::lock_guard<std::mutex> g(g_arena_mu);
  for (size_t b = 0; b < nb; b++) {
    status[b] = (uint64_t*)(base + soff[b]);
    for (size_t j = 0; j < nout; j++) {
      gx_column& c = out[b * nout + j];
      c = gx_column{};
      c.type_id = types[j];
      c.data = base + doff[b * nout + j];
      c.null_mask = (uint32_t*)(base + moff[b * nout + j]);
      c.capacity = caps[b];
      g_arena_of[c.data] = ar;
    }
  }
  return base;
}

int64_t mask_words_for(int64_t rows) { return mask_words_padded(rows); }

void free_column(gx_column& c, cudaStream_t s) {
  bool in_arena = false;
  void* release = nullptr;
  if (c.data) {
    std::lock_guard<std::mutex> g(g_arena_mu);
    auto it = g_arena_of.find(c.data);
    if (it != g_arena_of.end()) {
      in_arena = true;
      OutputArena* ar = it->second;
      g_arena_of.erase(it);
      if (--ar->refs == 0) {
        release = ar->base;
        delete ar;
      }
    }
  }
  if (in_arena) {
    dev_free(release, s);
  } else {
    dev_free(c.data, s);
    dev_free(c.null_mask, s);
  }
  c.data = nullptr;
  c.null_mask = nullptr;
}

// ---------------------------------------------------- precompiled kernels
__global__ void k_copy_mask(const uint32_t* __restrict__ src, int64_t src_bit, uint32_t* __restrict__ dst,
                            int64_t nrows, int64_t dst_words) {
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < dst_words; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row0 = w * 32;
    uint32_t v = 0;
    if (row0 < nrows) {
      if (src == nullptr) {
        v = 0xffffffffu;
      } else {
        const int64_t b = src_bit + row0;
        const int sh = (int)(b & 31);
        const int64_t i = b >> 5;
        const uint32_t lo = src[i];
        // the high word is read only if bits of it are needed by a row < nrows
        const uint32_t hi = (sh != 0 && row0 + (32 - sh) < nrows) ? src[i + 1] : 0u;
        v = sh ? __funnelshift_r(lo, hi, sh) : lo;
      }
      const int64_t left = nrows - row0;
      if (left < 32) v &= (1u << left) - 1u;
    }
    dst[w] = v;
  }
}

__global__ void k_fill(void* dst, int width, uint64_t value, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    switch (width) {
      case 1: ((uint8_t*)dst)[i] = (uint8_t)value; break;
      case 2: ((uint16_t*)dst)[i] = (uint16_t)value; break;
      case 4: ((uint32_t*)dst)[i] = (uint32_t)value; break;
      default: ((uint64_t*)dst)[i] = value; break;
    }
  }
}

__global__ void k_fill_mask(uint32_t* dst, int64_t nrows, bool valid, int64_t dst_words) {
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < dst_words; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row0 = w * 32;
    uint32_t v = 0;
    if (valid && row0 < nrows) v = (nrows - row0 >= 32) ? 0xffffffffu : ((1u << (nrows - row0)) - 1u);
    dst[w] = v;
  }
}

// Exclusive scan of per-tile counts in place (one CTA of 1024 threads walks
// the array in chunks); *total receives the sum.
__global__ void __launch_bounds__(1024) k_scan_tiles(uint64_t* counts, int64_t n, unsigned long long* total) {
  __shared__ uint64_t s_warp[32];
  __shared__ uint64_t s_carry;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) s_carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t i = base + t;
    const uint64_t v = i < n ? counts[i] : 0ull;
    uint64_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint64_t w = s_warp[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= d) w += y;
      }
      s_warp[lane] = w;
    }
    __syncthreads();
    const uint64_t carry = s_carry;
    const uint64_t incl = x + (warp > 0 ? s_warp[warp - 1] : 0ull);
    if (i < n) counts[i] = carry + incl - v;
    __syncthreads();
    if (t == 1023) s_carry = carry + incl;
    __syncthreads();
  }
  if (t == 0) *total = s_carry;
}

static int grid_for(int64_t items, int threads) {
  int64_t g = (items + threads - 1) / threads;
  int64_t cap = (int64_t)device_sm_count() * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

void launch_copy_mask(const uint32_t* src, int64_t src_bit, uint32_t* dst, int64_t nrows, int64_t dst_words,
                      cudaStream_t s) {
  k_copy_mask<<<grid_for(dst_words, 256), 256, 0, s>>>(src, src_bit, dst, nrows, dst_words);
  g_launches.fetch_add(1);
  check_cuda(cudaGetLastError(), "k_copy_mask launch");
}

void launch_fill(void* dst, int width, uint64_t value, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  k_fill<<<grid_for(n, 256), 256, 0, s>>>(dst, width, value, n);
  g_launches.fetch_add(1);
  check_cuda(cudaGetLastError(), "k_fill launch");
}

void launch_fill_mask(uint32_t* dst, int64_t nrows, bool valid, int64_t dst_words, cudaStream_t s) {
  k_fill_mask<<<grid_for(dst_words, 256), 256, 0, s>>>(dst, nrows, valid, dst_words);
  g_launches.fetch_add(1);
  check_cuda(cudaGetLastError(), "k_fill_mask launch");
}

void launch_scan_tiles(uint64_t* counts, int64_t n, unsigned long long* total, cudaStream_t s) {
  k_scan_tiles<<<1, 1024, 0, s>>>(counts, n, total);
  g_launches.fetch_add(1);
  check_cuda(cudaGetLastError(), "k_scan_tiles launch");
}

// ------------------------------------------------------------ plan execution
static const char* kind_name(KernelKind k) {
  switch (k) {
    case KernelKind::PROJECT: return "gx_project";
    case KernelKind::FUSED_FILTER: return "gx_filter_fused";
    case KernelKind::COUNT_FILTER: return "gx_filter_count";
    case KernelKind::FUSED_BATCHED: return "gx_filter_batched";
    case KernelKind::FUSED_STAGED: return "gx_filter_staged";
    case KernelKind::FUSED_TMA: return "gx_filter_tma";
    case KernelKind::FUSED_STREAM: return "gx_filter_stream";
    default: return "gx_filter_write";
  }
}

// Candidate block shapes (warps x words, register cap) of a tuned single-pass
// filter: the first is used until the others have been measured.  Measured on
// GB300: the deep C2 plan is fastest at 4 x 8, the order-line C5 plan at 1 x 16
// (no block barrier between warps), the light C1 plan at 4 x 8 held to 40
// registers (more resident warps for a latency-bound pass: 0.179 ms against
// 0.191 at 1 x 16 and 0.220 at 4 x 8 uncapped, 2^24 rows).
static const CompiledPlan::Shape kShapes[] = {{4, 8, 0}, {1, 16, 0}, {2, 8, 0}, {4, 8, 40}};
static constexpr int kNumShapes = 4;

// The first large call runs the first candidate unmeasured (it pays the
// first touches of fresh output memory), the next ones measure each candidate.
CompiledPlan::Shape CompiledPlan::filter_shape(int64_t n, int* explore) const {
  *explore = -1;
  if (!cfg_.tune_shape) return {cfg_.warps, cfg_.words, 0};
  std::lock_guard<std::mutex> g(tmu_);
  if (chosen_ >= 0) return kShapes[chosen_];
  if (cand_ms_.empty()) cand_ms_.assign(kNumShapes, -1.f);
  if (n >= kShapeTuneRows && next_cand_ <= kNumShapes) {
    const int k = next_cand_++;
    if (k == 0) {  // warm-up; every candidate is compiled now, so no trial pays a compile
      tune_compile_ = true;
      return kShapes[0];
    }
    *explore = k - 1;
    return kShapes[*explore];
  }
  return kShapes[0];
}

CompiledPlan::Shape CompiledPlan::current_shape() const {
  if (!cfg_.tune_shape) return {cfg_.warps, cfg_.words, 0};
  std::lock_guard<std::mutex> g(tmu_);
  return chosen_ >= 0 ? kShapes[chosen_] : kShapes[0];
}

void CompiledPlan::shape_measured(int idx, float ms) const {
  std::lock_guard<std::mutex> g(tmu_);
  if (idx < 0 || idx >= (int)cand_ms_.size()) return;
  cand_ms_[idx] = ms;
  int best = -1;
  for (int i = 0; i < kNumShapes; i++) {
    if (cand_ms_[i] < 0) return;  // not all measured yet
    if (best < 0 || cand_ms_[i] < cand_ms_[best]) best = i;
  }
  chosen_ = best;
}

JitKernel CompiledPlan::kernel(KernelKind kind, const std::vector<bool>& nullable, int warps, int words,
                               int regs) const {
  if (warps <= 0) warps = cfg_.warps;
  if (words <= 0) words = cfg_.words;
  if (regs <= 0) regs = cfg_.max_regs;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::string key = std::to_string((int)kind) + ":" + std::to_string(dev) + ":" + std::to_string(warps) + "x" +
                    std::to_string(words) + "x" + std::to_string(cfg_.stages) + "r" + std::to_string(regs) + ":";
  for (bool b : nullable) key += b ? '1' : '0';
  {
    std::lock_guard<std::mutex> g(kmu_);
    auto it = kcache_.find(key);
    if (it != kcache_.end()) return it->second;
  }
  Plan p = plan_;
  p.nullable = nullable;
  KernelConfig c = cfg_;
  c.warps = warps;
  c.words = words;
  c.max_regs = regs;
  // the single pass in a conjunct order given at launch (learned ordering) is
  // named apart, so that profiles can tell it from the fixed-order pass
  const std::string name =
      kind == KernelKind::FUSED_FILTER && c.runtime_order ? std::string("gx_filter_ordered") : kind_name(kind);
  const std::string src = generate_kernel(p, kind, c, name);
  // the tile-staged kernel runs a producer and a resolver warp beside its consumer warps
  const bool tma = kind == KernelKind::FUSED_TMA;
  const unsigned dyn = tma ? tile_layout(p, warps, words, c.stages).dyn_smem : 0u;
  const JitKernel k = jit_get(src, name, (tma ? warps + 2 : warps) * 32, dyn);
  std::lock_guard<std::mutex> g(kmu_);
  kcache_[key] = k;
  return k;
}

// Launches a plan kernel; with timing on, brackets it with events on `s`
// (timed=true for the call's main kernel) and adds its duration to the
// calling thread's total.
void launch_raw(const JitKernel& k, int grid, cudaStream_t s, void** params, bool timed) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool tm = timed && g_timing.load();
  if (tm) {
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    check_cuda(cudaEventRecord(e0, s), "event record");
  }
  CUresult r = driver().LaunchKernel(k.fn, (unsigned)grid, 1, 1, (unsigned)k.block_threads, 1, 1, k.dyn_smem,
                                     (CUstream)s, params, nullptr);
  if (r != CUDA_SUCCESS) fail(GX_ERR_CUDA, std::string("cuLaunchKernel: ") + driver_error_string(r));
  g_launches.fetch_add(1);
  if (tm) {
    check_cuda(cudaEventRecord(e1, s), "event record");
    check_cuda(cudaEventSynchronize(e1), "event sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    t_kernel_ms += ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
}

// The calling thread's pinned 4-word buffer for a filter's scratch header:
// a copy into pageable memory would be staged by the driver.  A call reads it
// back and synchronises before it returns, so one buffer per thread suffices.
static unsigned long long* pinned_header() {
  thread_local unsigned long long* buf = nullptr;
  if (!buf) check_cuda(cudaMallocHost((void**)&buf, 64), "pinned header");
  for (int i = 0; i < 4; i++) buf[i] = 0;
  return buf;
}

// The error word a filter kernel leaves in its scratch header: 1 a look-back
// wait gave up, 2 a wait for a tile's bulk copies (or a hand-over between the
// warps of a tile-staged block) gave up, 3 the dynamic shared memory was not
// 16-byte aligned (nothing was copied).
static void raise_kernel_error(unsigned long long word) {
  const int e = (int)(word & 0xffffffffull);
  if (e == 0) return;
  if (e == 1) fail(GX_ERR_TIMEOUT, "compaction look-back wait timed out");
  if (e == 2) fail(GX_ERR_TIMEOUT, "tile-staged kernel: a wait for bulk copies or a warp hand-over timed out");
  fail(GX_ERR_CUDA, "tile-staged kernel: dynamic shared memory not 16-byte aligned");
}

static std::vector<bool> runtime_nullable(const Plan& p, const std::vector<ColumnView>& cols) {
  std::vector<bool> nb(cols.size());
  for (size_t i = 0; i < cols.size(); i++) nb[i] = cols[i].mask != nullptr;
  (void)p;
  return nb;
}

// bulk copies need every column a conjunct reads to start on a 16-byte boundary
static bool staging_aligned(const Plan& p, const std::vector<ColumnView>& cols) {
  for (size_t c = 0; c < p.conjuncts.size(); c++)
    for (int col : conjunct_columns(p, (int)c)) {
      const uintptr_t start = (uintptr_t)cols[col].data + (uintptr_t)(cols[col].offset * type_size(cols[col].type));
      if (start % 16 != 0) return false;
    }
  return true;
}

static void launch(const JitKernel& k, int grid, cudaStream_t s, KernelArgs& args, bool timed = false) {
  void* params[] = {&args};
  launch_raw(k, grid, s, params, timed);
}

static void fill_args_inputs(KernelArgs& a, const std::vector<ColumnView>& cols) {
  std::memset(&a, 0, sizeof a);
  for (size_t i = 0; i < cols.size(); i++) {
    a.in_data[i] = cols[i].data;
    a.in_mask[i] = cols[i].mask;
    a.in_off[i] = cols[i].offset;
  }
  a.n = cols.empty() ? 0 : cols[0].size;
}

void CompiledPlan::execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                           cudaStream_t s, const ExecExtras* extras) const {
  if (cols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < cols.size(); i++)
    if (cols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
  const bool caller_bufs = !plan_.outputs.empty() && out[0].data != nullptr;
  if (plan_.has_filter()) {
    run_filter(cols, out, out_rows, caller_bufs, extras, s);
  } else {
    run_project(cols, out, caller_bufs, s);
    if (out_rows) *out_rows = cols.empty() ? 0 : cols[0].size;
  }
}

bool CompiledPlan::can_defer() const {
  if (!plan_.has_filter()) return false;
  for (const auto& o : plan_.outputs)
    if (o.kind == OutSpec::BROADCAST) return false;
  return true;
}

void CompiledPlan::finish_queued(const unsigned long long* hdr, int64_t n, gx_column* out, int64_t* out_rows) const {
  raise_kernel_error(hdr[2]);
  const int64_t rows = n == 0 ? 0 : mode_ == GX_FILTER_TWO_PASS ? (int64_t)hdr[3] : (int64_t)hdr[1];
  if (out_rows) *out_rows = rows;
  for (size_t j = 0; j < plan_.outputs.size(); j++) {
    if (rows > out[j].capacity) fail(GX_ERR_CAPACITY, "output capacity too small");
    out[j].size = rows;
  }
}

// Single-pass filters run on the tile-staged kernel (FUSED_TMA) unless the
// plan evaluates its conjuncts in a runtime order, projects per word, keys
// RAND by output row (the output row is known only at the write-out), was told
// not to, reads a column that is not fixed-width or not naturally aligned, or
// its tile ring does not fit in shared memory.
bool CompiledPlan::tma_path(const std::vector<ColumnView>& cols) const {
  if (cfg_.use_tma == 0 || mode_ == GX_FILTER_TWO_PASS || !plan_.has_filter()) return false;
  if (!cfg_.dense || cfg_.runtime_order || cfg_.short_circuit || cfg_.staged) return false;
  for (const Node& nd : plan_.nodes)
    if (nd.kind == Node::OP && nd.op == OP_RAND && nd.rand_out_row) return false;
  // elements are read from shared memory at their natural alignment
  for (const ColumnView& c : cols) {
    const int w = type_size(c.type);
    if (w > 1 && ((uintptr_t)c.data + (uintptr_t)(c.offset * w)) % (uintptr_t)w != 0) return false;
  }
  Plan p = plan_;
  p.nullable = runtime_nullable(plan_, cols);
  const TileLayout L = tile_layout(p, cfg_.tma_warps, cfg_.tma_words, cfg_.stages);
  for (int c : L.cols)
    if (type_size(p.schema[c]) == 0) return false;  // only fixed-width columns are staged
  return L.dyn_smem <= kTmaMaxDynSmem;
}

int64_t CompiledPlan::tiles_for(int64_t n) const {
  const int64_t tile_rows = (int64_t)cfg_.warps * cfg_.words * 32;
  return (n + tile_rows - 1) / tile_rows;
}

void CompiledPlan::enqueue_filter(const std::vector<ColumnView>& cols, gx_column* out, unsigned long long* hdr,
                                  uint64_t* tile_status, const ExecExtras* extras, cudaStream_t s) const {
  if (!can_defer()) fail(GX_ERR_INVALID, "a queued filter needs a filter plan without literal outputs");
  if (cols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < cols.size(); i++)
    if (cols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const int nout = (int)plan_.outputs.size();
  // outputs may hold fewer rows than the batch (sized from a prediction): the
  // kernel writes nothing past the smallest capacity and finish_queued reports
  // a row count above it as GX_ERR_CAPACITY
  int64_t capacity = n;
  for (int j = 0; j < nout; j++) {
    if (!out[j].data || !out[j].null_mask) fail(GX_ERR_INVALID, "queued filter outputs missing");
    out[j].type_id = plan_.outputs[j].type;
    capacity = std::min<int64_t>(capacity, out[j].capacity);
  }
  if (n == 0) return;
  const int64_t ntiles = tiles_for(n);
  const std::vector<bool> nb = runtime_nullable(plan_, cols);
  KernelArgs a{};
  fill_args_inputs(a, cols);
  a.tile_status = tile_status;
  a.tile_counter = hdr + 0;
  a.out_count = hdr + 1;
  a.err = (int*)(hdr + 2);
  a.seed = plan_.rand_seed;
  a.capacity = capacity;
  for (int i = 0; i < 16; i++) a.order[i] = i;
  if (extras) {
    for (int i = 0; i < extras->num_order && i < 16; i++) a.order[i] = extras->order[i];
    a.order_dev = extras->order_dev;
    a.conj_counts = extras->conj_counts;
  }
  for (int j = 0; j < nout; j++) {
    a.out_data[j] = out[j].data;
    a.out_mask[j] = out[j].null_mask;
  }
  const bool two_pass = mode_ == GX_FILTER_TWO_PASS;
  if (two_pass) {
    const JitKernel kc = kernel(KernelKind::COUNT_FILTER, nb);
    int64_t grid = (int64_t)device_sm_count() * kc.max_blocks_per_sm;
    if (grid > ntiles) grid = ntiles;
    launch(kc, (int)grid, s, a, true);
    launch_scan_tiles(tile_status, ntiles, hdr + 3, s);
  }
  const JitKernel k = kernel(two_pass ? KernelKind::WRITE_FILTER : KernelKind::FUSED_FILTER, nb);
  int64_t grid = (int64_t)device_sm_count() * k.max_blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  launch(k, (int)grid, s, a, true);
}

void CompiledPlan::run_project(const std::vector<ColumnView>& cols, gx_column* out, bool caller_bufs,
                               cudaStream_t s) const {
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const int nout = (int)plan_.outputs.size();
  std::vector<gx_column> made;
  try {
    if (!caller_bufs && nout > 0) {
      std::vector<int> types;
      for (const auto& o : plan_.outputs) types.push_back(o.type);
      alloc_outputs(types, n, 0, false, out, s);
      made.assign(out, out + nout);
    }
    for (int j = 0; j < nout; j++) {
      if (caller_bufs) {
        if (out[j].capacity < n || !out[j].data || !out[j].null_mask) fail(GX_ERR_CAPACITY, "output buffer too small");
        out[j].type_id = plan_.outputs[j].type;
      }
      out[j].size = n;
    }
    const int64_t words = mask_words_padded(n), nwords = (n + 31) / 32;
    for (int j = 0; j < nout; j++) {
      const OutSpec& o = plan_.outputs[j];
      const int w = type_size(o.type);
      if (o.kind == OutSpec::COPY) {
        const ColumnView& c = cols[o.col];
        if (n > 0)
          check_cuda(cudaMemcpyAsync(out[j].data, (const char*)c.data + c.offset * w, (size_t)n * w,
                                     cudaMemcpyDeviceToDevice, s), "copy column");
        launch_copy_mask(c.mask, c.offset, out[j].null_mask, n, words, s);
      } else if (o.kind == OutSpec::BROADCAST) {
        launch_fill(out[j].data, w, o.lit_bits_as_element(), n, s);
        launch_fill_mask(out[j].null_mask, n, o.lit_valid, words, s);
      } else if (words > nwords) {
        check_cuda(cudaMemsetAsync(out[j].null_mask + nwords, 0, (size_t)(words - nwords) * 4, s), "mask pad");
      }
    }
    if (n > 0 && plan_.needs_kernel()) {
      const JitKernel k = kernel(KernelKind::PROJECT, runtime_nullable(plan_, cols));
      KernelArgs a{};
      fill_args_inputs(a, cols);
      for (int j = 0; j < nout; j++) {
        a.out_data[j] = out[j].data;
        a.out_mask[j] = out[j].null_mask;
      }
      a.seed = plan_.rand_seed;
      const int64_t steps = (nwords + cfg_.words * cfg_.warps - 1) / (cfg_.words * cfg_.warps);
      int64_t grid = (int64_t)device_sm_count() * k.max_blocks_per_sm;
      if (grid > steps) grid = steps;
      last.grid = (int)grid;
      last.block = k.block_threads;
      last.regs = k.num_regs;
      launch(k, (int)grid, s, a, true);
    }
  } catch (...) {
    for (auto& c : made) free_column(c, s);
    throw;
  }
}

void CompiledPlan::run_filter(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                              bool caller_bufs, const ExecExtras* extras, cudaStream_t s) const {
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const int nout = (int)plan_.outputs.size();
  const int64_t nwords = (n + 31) / 32;
  const bool two_pass = mode_ == GX_FILTER_TWO_PASS;
  // the single-pass fused kernel's block shape (tuned online when allowed)
  int explore = -1;
  Shape sh{cfg_.warps, cfg_.words};
  const std::vector<bool> nb = runtime_nullable(plan_, cols);
  const bool tma = !two_pass && tma_path(cols);
  if (tma) sh = {cfg_.tma_warps, cfg_.tma_words};
  else if (!two_pass && !(cfg_.staged && cfg_.runtime_order)) sh = filter_shape(n, &explore);
  const int64_t tile_words = (int64_t)sh.warps * sh.words;
  const int64_t ntiles = (nwords + tile_words - 1) / tile_words;
  std::vector<gx_column> made;
  void* scratch = nullptr;
  cudaEvent_t te0 = nullptr, te1 = nullptr;
  try {
    if (n == 0) {
      for (int j = 0; j < nout; j++) {
        if (!caller_bufs) {
          out[j] = alloc_column(plan_.outputs[j].type, 0, s);
          made.push_back(out[j]);
        }
        out[j].size = 0;
        launch_fill_mask(out[j].null_mask, 0, false, mask_words_padded(0), s);
      }
      if (out_rows) *out_rows = 0;
      return;
    }
    // scratch: [0] tile counter, [1] out count, [2] err (int), [3] total, then per-tile status
    const size_t sbytes = (size_t)(4 + ntiles) * 8;
    int64_t capacity = n;
    if (extras && extras->capacity_hint >= 0 && extras->capacity_hint < n) capacity = extras->capacity_hint;
    // single pass into library outputs: scratch and outputs in one arena, one
    // memset for scratch + masks; otherwise a scratch allocation of its own
    const bool arena = !two_pass && !caller_bufs && nout > 0;
    void* sbase = nullptr;
    if (arena) {
      std::vector<int> types;
      for (const auto& o : plan_.outputs) types.push_back(o.type);
      sbase = alloc_outputs(types, capacity, sbytes, true, out, s);
      made.assign(out, out + nout);
    } else {
      scratch = dev_alloc(sbytes, s);
      sbase = scratch;
      check_cuda(cudaMemsetAsync(scratch, 0, sbytes, s), "scratch memset");
    }
    unsigned long long* hdr = (unsigned long long*)sbase;
    uint64_t* status = (uint64_t*)sbase + 4;
    KernelArgs a{};
    fill_args_inputs(a, cols);
    a.tile_status = status;
    a.tile_counter = hdr + 0;
    a.out_count = hdr + 1;
    a.err = (int*)(hdr + 2);
    a.seed = plan_.rand_seed;
    for (int i = 0; i < 16; i++) a.order[i] = i;
    if (extras) {
      for (int i = 0; i < extras->num_order && i < 16; i++) a.order[i] = extras->order[i];
      a.order_dev = extras->order_dev;
      a.conj_counts = extras->conj_counts;
    }
    unsigned long long* host_hdr = pinned_header();
    if (extras) {
      a.spin_limit = extras->spin_limit;
      if (extras->first_tile > 0 && !two_pass) {
        host_hdr[0] = (unsigned long long)extras->first_tile;
        check_cuda(cudaMemcpyAsync(hdr, host_hdr, 8, cudaMemcpyHostToDevice, s), "ticket start");
      }
    }
    if (two_pass) {
      const JitKernel kc = kernel(KernelKind::COUNT_FILTER, nb);
      int64_t grid = (int64_t)device_sm_count() * kc.max_blocks_per_sm;
      if (grid > ntiles) grid = ntiles;
      launch(kc, (int)grid, s, a, true);
      launch_scan_tiles(status, ntiles, hdr + 3, s);
      if (extras && extras->conj_counts && extras->conj_counts_host)
        check_cuda(cudaMemcpyAsync(extras->conj_counts_host, extras->conj_counts, 16 * 8, cudaMemcpyDeviceToHost, s),
                   "conjunct counts readback");
      check_cuda(cudaMemcpyAsync(host_hdr, hdr, 4 * 8, cudaMemcpyDeviceToHost, s), "count readback");
      check_cuda(cudaStreamSynchronize(s), "count sync");
      capacity = (int64_t)host_hdr[3];
    }
    if (caller_bufs) {
      for (int j = 0; j < nout; j++) {
        if (!out[j].data || !out[j].null_mask) fail(GX_ERR_INVALID, "caller output buffer missing");
        out[j].type_id = plan_.outputs[j].type;
      }
      capacity = out[0].capacity;
      for (int j = 1; j < nout; j++) capacity = std::min<int64_t>(capacity, out[j].capacity);
      if (two_pass && capacity < (int64_t)host_hdr[3]) {
        if (out_rows) *out_rows = (int64_t)host_hdr[3];
        fail(GX_ERR_CAPACITY, "output capacity too small");
      }
      for (int j = 0; j < nout; j++)
        check_cuda(cudaMemsetAsync(out[j].null_mask, 0, (size_t)mask_words_padded(capacity) * 4, s), "mask zero");
    } else if (!arena && nout > 0) {
      std::vector<int> types;
      for (const auto& o : plan_.outputs) types.push_back(o.type);
      alloc_outputs(types, capacity, 0, true, out, s);
      made.assign(out, out + nout);
    }
    for (int j = 0; j < nout; j++) {
      a.out_data[j] = out[j].data;
      a.out_mask[j] = out[j].null_mask;
    }
    a.capacity = capacity;
    KernelKind kind = two_pass ? KernelKind::WRITE_FILTER : tma ? KernelKind::FUSED_TMA : KernelKind::FUSED_FILTER;
    if (!two_pass && cfg_.staged && cfg_.runtime_order && staging_aligned(plan_, cols)) kind = KernelKind::FUSED_STAGED;
    if (kind == KernelKind::FUSED_FILTER && tune_compile_.exchange(false))
      for (const Shape& c : kShapes) kernel(kind, nb, c.warps, c.words, c.regs);
    const JitKernel k = two_pass ? kernel(kind, nb) : kernel(kind, nb, sh.warps, sh.words, sh.regs);
    int64_t grid = (int64_t)device_sm_count() * k.max_blocks_per_sm;
    if (grid > ntiles) grid = ntiles;
    last.grid = (int)grid;
    last.block = k.block_threads;
    last.regs = k.num_regs;
    last.tiles = ntiles;
    if (explore >= 0) {
      check_cuda(cudaEventCreate(&te0), "event");
      check_cuda(cudaEventCreate(&te1), "event");
      check_cuda(cudaEventRecord(te0, s), "event record");
    }
    launch(k, (int)grid, s, a, true);
    if (explore >= 0) check_cuda(cudaEventRecord(te1, s), "event record");
    if (!two_pass && extras && extras->conj_counts && extras->conj_counts_host)
      check_cuda(cudaMemcpyAsync(extras->conj_counts_host, extras->conj_counts, 16 * 8, cudaMemcpyDeviceToHost, s),
                 "conjunct counts readback");
    check_cuda(cudaMemcpyAsync(host_hdr, hdr, 4 * 8, cudaMemcpyDeviceToHost, s), "count readback");
    check_cuda(cudaStreamSynchronize(s), "filter sync");
    if (explore >= 0) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, te0, te1) == cudaSuccess) shape_measured(explore, ms);
      cudaEventDestroy(te0);
      cudaEventDestroy(te1);
      te0 = te1 = nullptr;
    }
    raise_kernel_error(host_hdr[2]);
    const int64_t rows = two_pass ? (int64_t)host_hdr[3] : (int64_t)host_hdr[1];
    if (out_rows) *out_rows = rows;
    if (rows > capacity) fail(GX_ERR_CAPACITY, "output capacity too small");
    for (int j = 0; j < nout; j++) {
      out[j].size = rows;
      const OutSpec& o = plan_.outputs[j];
      if (o.kind == OutSpec::BROADCAST) {
        launch_fill(out[j].data, type_size(o.type), o.lit_bits_as_element(), rows, s);
        launch_fill_mask(out[j].null_mask, rows, o.lit_valid, mask_words_padded(capacity), s);
      }
    }
    dev_free(scratch, s);
    scratch = nullptr;
  } catch (...) {
    if (te0) cudaEventDestroy(te0);
    if (te1) cudaEventDestroy(te1);
    if (scratch) dev_free(scratch, s);
    for (auto& c : made) free_column(c, s);
    throw;
  }
}

void CompiledPlan::execute_with_scratch(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                                        unsigned long long* scratch, long long scratch_words, cudaStream_t s) const {
  if (!plan_.has_filter()) fail(GX_ERR_INVALID, "the no-allocation entry point needs a plan with a condition");
  if (cols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < cols.size(); i++)
    if (cols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
  const int nout = (int)plan_.outputs.size();
  for (int j = 0; j < nout; j++) {
    if (!out[j].data || !out[j].null_mask || out[j].capacity < 0)
      fail(GX_ERR_INVALID, "the no-allocation entry point writes into caller buffers: out[].data, "
                           "out[].null_mask and out[].capacity must be set");
    out[j].type_id = plan_.outputs[j].type;
  }
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  const int64_t nwords = (n + 31) / 32;
  const int64_t tile_words = (int64_t)cfg_.warps * cfg_.words;
  const int64_t ntiles = (nwords + tile_words - 1) / tile_words;
  if (4 + ntiles > scratch_words)
    fail(GX_ERR_INVALID, "batch of " + std::to_string(n) + " rows needs " + std::to_string(ntiles) +
                             " tile slots; the no-allocation scratch holds " + std::to_string(scratch_words - 4) +
                             " (at most " + std::to_string((scratch_words - 4) * tile_words * 32) + " rows)");
  int64_t capacity = nout ? out[0].capacity : 0;
  for (int j = 1; j < nout; j++) capacity = std::min<int64_t>(capacity, out[j].capacity);
  for (int j = 0; j < nout; j++)
    check_cuda(cudaMemsetAsync(out[j].null_mask, 0, (size_t)mask_words_padded(capacity) * 4, s), "mask zero");
  if (n == 0) {
    for (int j = 0; j < nout; j++) out[j].size = 0;
    if (out_rows) *out_rows = 0;
    return;
  }
  // the array keeps the previous call's contents: ticket, count, error flag and
  // tile status words must start at zero
  check_cuda(cudaMemsetAsync(scratch, 0, (size_t)(4 + ntiles) * 8, s), "scratch zero");
  KernelArgs a{};
  fill_args_inputs(a, cols);
  a.tile_status = (uint64_t*)scratch + 4;
  a.tile_counter = scratch + 0;
  a.out_count = scratch + 1;
  a.err = (int*)(scratch + 2);
  a.seed = plan_.rand_seed;
  a.capacity = capacity;
  for (int i = 0; i < 16; i++) a.order[i] = i;  // plan order (as run_filter)
  for (int j = 0; j < nout; j++) {
    a.out_data[j] = out[j].data;
    a.out_mask[j] = out[j].null_mask;
  }
  // the configured block shape (cfg_.warps x cfg_.words, 512-row tiles by
  // default), never the online-tuned one: the scratch's tile limit is fixed
  const JitKernel k = kernel(KernelKind::FUSED_FILTER, runtime_nullable(plan_, cols));
  int64_t grid = (int64_t)device_sm_count() * k.max_blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  launch(k, (int)grid, s, a, true);
  // read back into this frame, not a pinned block: this path allocates nothing
  unsigned long long host_hdr[4] = {0, 0, 0, 0};
  check_cuda(cudaMemcpyAsync(host_hdr, scratch, 4 * 8, cudaMemcpyDeviceToHost, s), "count readback");
  check_cuda(cudaStreamSynchronize(s), "filter sync");
  raise_kernel_error(host_hdr[2]);
  const int64_t rows = (int64_t)host_hdr[1];
  if (out_rows) *out_rows = rows;
  if (rows > capacity) fail(GX_ERR_CAPACITY, "output capacity too small");
  for (int j = 0; j < nout; j++) {
    out[j].size = rows;
    const OutSpec& o = plan_.outputs[j];
    if (o.kind == OutSpec::BROADCAST) {
      launch_fill(out[j].data, type_size(o.type), o.lit_bits_as_element(), rows, s);
      launch_fill_mask(out[j].null_mask, rows, o.lit_valid, mask_words_padded(capacity), s);
    }
  }
}


// ------------------------------------------------------------ host to host
namespace {
constexpr int kMaxHostChunks = 64;

// Per-thread resources of host-to-host execution, made on first use and kept
// for the thread's lifetime: a copy stream each way, an event pool, and a
// pinned, mapped block for the chunks' row counts and the counter values.
struct HostExecRes {
  int device = -1;
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t ev[2 * kMaxHostChunks + 2] = {};
  unsigned long long* blk = nullptr;      // host view: [0, 64) row counts, [64, 128) counters, [128] error
  unsigned long long* blk_dev = nullptr;  // device view
};

HostExecRes& host_exec_res() {
  thread_local HostExecRes r;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "device");
  if (r.device != dev) {
    // a thread that moves to another device gets new resources (the old ones
    // belong to the other device's context and stay with it)
    r = HostExecRes{};
    check_cuda(cudaStreamCreateWithFlags(&r.h2d, cudaStreamNonBlocking), "copy stream");
    check_cuda(cudaStreamCreateWithFlags(&r.d2h, cudaStreamNonBlocking), "copy stream");
    for (auto& e : r.ev) check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    check_cuda(cudaHostAlloc((void**)&r.blk, 2048, cudaHostAllocMapped | cudaHostAllocPortable), "pinned block");
    check_cuda(cudaHostGetDevicePointer((void**)&r.blk_dev, r.blk, 0), "mapped block");
    r.device = dev;
  }
  return r;
}
}  // namespace

void CompiledPlan::execute_host(const std::vector<ColumnView>& hcols, gx_column* hout, int64_t* out_rows,
                                cudaStream_t s) const {
  if (hcols.size() != plan_.schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < hcols.size(); i++) {
    if (hcols[i].type != plan_.schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
    if (hcols[i].offset != 0) fail(GX_ERR_INVALID, "host columns must start at offset 0");
  }
  const int nout = (int)plan_.outputs.size();
  const int64_t n = hcols.empty() ? 0 : hcols[0].size;
  int64_t capacity = nout ? hout[0].capacity : 0;
  for (int j = 0; j < nout; j++) {
    if (!hout[j].data || !hout[j].null_mask) fail(GX_ERR_INVALID, "host output buffers missing");
    capacity = std::min<int64_t>(capacity, hout[j].capacity);
    hout[j].type_id = plan_.outputs[j].type;
  }
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  // device copies of the inputs
  std::vector<size_t> in_off(hcols.size()), in_moff(hcols.size());
  size_t in_bytes = 0;
  const int64_t nwords = (n + 31) / 32;
  for (size_t i = 0; i < hcols.size(); i++) {
    in_off[i] = in_bytes;
    in_bytes += al(std::max<size_t>(64, (size_t)n * type_size(hcols[i].type)));
    in_moff[i] = in_bytes;
    if (hcols[i].mask) in_bytes += al((size_t)std::max<int64_t>(nwords, 1) * 4);
  }
  const bool pipelined = plan_.has_filter() && can_defer() && mode_ != GX_FILTER_TWO_PASS && n > 0;
  if (!pipelined) {
    // whole-table form: copy in, evaluate, copy out (a plan with literal
    // outputs or no condition, the two-pass mode, or no rows)
    char* din = (char*)dev_alloc(std::max<size_t>(in_bytes, 64), s);
    std::vector<gx_column> dout(nout);
    try {
      std::vector<ColumnView> dcols = hcols;
      for (size_t i = 0; i < hcols.size(); i++) {
        const size_t bytes = (size_t)n * type_size(hcols[i].type);
        dcols[i].data = din + in_off[i];
        if (bytes) check_cuda(cudaMemcpyAsync(din + in_off[i], hcols[i].data, bytes, cudaMemcpyHostToDevice, s), "input");
        if (hcols[i].mask) {
          dcols[i].mask = (const uint32_t*)(din + in_moff[i]);
          if (nwords)
            check_cuda(cudaMemcpyAsync(din + in_moff[i], hcols[i].mask, (size_t)nwords * 4, cudaMemcpyHostToDevice, s),
                       "input mask");
        }
      }
      int64_t rows = 0;
      execute(dcols, dout.data(), &rows, s);
      if (out_rows) *out_rows = rows;
      if (rows > capacity) fail(GX_ERR_CAPACITY, "host output capacity too small");
      for (int j = 0; j < nout; j++) {
        const size_t bytes = (size_t)rows * type_size(dout[j].type_id);
        if (bytes) check_cuda(cudaMemcpyAsync(hout[j].data, dout[j].data, bytes, cudaMemcpyDeviceToHost, s), "output");
        if (rows)
          check_cuda(cudaMemcpyAsync(hout[j].null_mask, dout[j].null_mask, (size_t)((rows + 31) / 32) * 4,
                                     cudaMemcpyDeviceToHost, s), "output mask");
        hout[j].size = rows;
      }
      check_cuda(cudaStreamSynchronize(s), "host output sync");
    } catch (...) {
      for (auto& c : dout)
        if (c.data) free_column(c, s);
      dev_free(din, s);
      throw;
    }
    for (auto& c : dout) free_column(c, s);
    dev_free(din, s);
    return;
  }
  // Pipelined form: the rows are cut into chunks of whole tiles.  Chunk k's
  // inputs go up on a copy stream, its kernel runs on `s` once they are in,
  // and its output rows go down on the other copy stream once its row count
  // is known, so the three overlap across chunks.  The kernels of all chunks
  // form one tile sequence over full-size device buffers: chunk k claims the
  // tiles [k T, (k + 1) T) from a counter that starts at k T, and its first
  // tile's look-back finds chunk k - 1's last inclusive prefix already
  // published, so every output row lands at its final position (and mask bit).
  HostExecRes& R = host_exec_res();
  const Shape sh = current_shape();
  const int64_t tile_rows = (int64_t)sh.warps * sh.words * 32;
  const int64_t ntiles = (n + tile_rows - 1) / tile_rows;
  int64_t chunk_tiles = std::max<int64_t>((int64_t(1) << 22) / tile_rows, (ntiles + 15) / 16);
  chunk_tiles = std::max<int64_t>(chunk_tiles, (ntiles + kMaxHostChunks - 1) / kMaxHostChunks);
  const int64_t chunk_rows = chunk_tiles * tile_rows;
  const int nchunks = (int)((ntiles + chunk_tiles - 1) / chunk_tiles);
  std::vector<size_t> out_off(nout), out_moff(nout);
  size_t total = in_bytes;
  for (int j = 0; j < nout; j++) {
    out_off[j] = total;
    total += al(std::max<size_t>(64, (size_t)n * type_size(plan_.outputs[j].type)));
  }
  const size_t zero_from = total;  // output masks, tile statuses and the error word start zeroed
  for (int j = 0; j < nout; j++) {
    out_moff[j] = total;
    total += al((size_t)mask_words_padded(n) * 4);
  }
  const size_t st_off = total;
  total += al((size_t)ntiles * 8);
  const size_t err_off = total;
  total += 256;
  const size_t ctr_off = total;
  total += al((size_t)nchunks * 8);
  char* dbase = (char*)dev_alloc(total, s);
  unsigned long long* counts = R.blk;  // chunk k's row count after its kernel (mapped)
  for (int k = 0; k < nchunks; k++) {
    counts[k] = 0;
    R.blk[64 + k] = (unsigned long long)(k * chunk_tiles);
  }
  R.blk[128] = 0;
  cudaEvent_t ready = R.ev[2 * kMaxHostChunks], drained = R.ev[2 * kMaxHostChunks + 1];
  bool launched = false;
  int64_t rows = 0;
  bool over = false;
  try {
    check_cuda(cudaMemsetAsync(dbase + zero_from, 0, ctr_off - zero_from, s), "host pipeline zero");
    check_cuda(cudaMemcpyAsync(dbase + ctr_off, R.blk + 64, (size_t)nchunks * 8, cudaMemcpyHostToDevice, s),
               "chunk counters");
    check_cuda(cudaEventRecord(ready, s), "event");
    check_cuda(cudaStreamWaitEvent(R.h2d, ready, 0), "event wait");
    launched = true;
    for (int k = 0; k < nchunks; k++) {
      const int64_t r0 = k * chunk_rows, r1 = std::min<int64_t>(n, r0 + chunk_rows);
      for (size_t i = 0; i < hcols.size(); i++) {
        const size_t w = type_size(hcols[i].type);
        if (w)
          check_cuda(cudaMemcpyAsync(dbase + in_off[i] + r0 * w, (const char*)hcols[i].data + r0 * w, (r1 - r0) * w,
                                     cudaMemcpyHostToDevice, R.h2d), "input chunk");
        if (hcols[i].mask) {
          const int64_t w0 = r0 / 32, w1 = (r1 + 31) / 32;
          check_cuda(cudaMemcpyAsync(dbase + in_moff[i] + w0 * 4, hcols[i].mask + w0, (size_t)(w1 - w0) * 4,
                                     cudaMemcpyHostToDevice, R.h2d), "input mask chunk");
        }
      }
      check_cuda(cudaEventRecord(R.ev[2 * k], R.h2d), "event");
    }
    std::vector<bool> nb(hcols.size());
    for (size_t i = 0; i < hcols.size(); i++) nb[i] = hcols[i].mask != nullptr;
    const JitKernel kern = kernel(KernelKind::FUSED_FILTER, nb, sh.warps, sh.words, sh.regs);
    for (int k = 0; k < nchunks; k++) {
      const int64_t r1 = std::min<int64_t>(n, (k + 1) * chunk_rows);
      check_cuda(cudaStreamWaitEvent(s, R.ev[2 * k], 0), "event wait");
      KernelArgs a{};
      for (size_t i = 0; i < hcols.size(); i++) {
        a.in_data[i] = dbase + in_off[i];
        a.in_mask[i] = hcols[i].mask ? (const uint32_t*)(dbase + in_moff[i]) : nullptr;
        a.in_off[i] = 0;
      }
      a.n = r1;
      a.capacity = n;
      a.tile_status = (uint64_t*)(dbase + st_off);
      a.tile_counter = (unsigned long long*)(dbase + ctr_off) + k;
      a.out_count = R.blk_dev + k;
      a.err = (int*)(dbase + err_off);
      a.seed = plan_.rand_seed;
      for (int i = 0; i < 16; i++) a.order[i] = i;
      for (int j = 0; j < nout; j++) {
        a.out_data[j] = dbase + out_off[j];
        a.out_mask[j] = (uint32_t*)(dbase + out_moff[j]);
      }
      int64_t grid = (int64_t)device_sm_count() * kern.max_blocks_per_sm;
      grid = std::min<int64_t>(grid, std::min<int64_t>(ntiles, (k + 1) * chunk_tiles) - k * chunk_tiles);
      launch(kern, (int)grid, s, a, true);
      check_cuda(cudaEventRecord(R.ev[2 * k + 1], s), "event");
    }
    // each chunk's rows go down as soon as its count is known
    int64_t prev = 0;
    for (int k = 0; k < nchunks; k++) {
      check_cuda(cudaEventSynchronize(R.ev[2 * k + 1]), "chunk sync");
      const int64_t rk = (int64_t)((volatile unsigned long long*)counts)[k];
      if (rk < prev) break;  // the chunk's kernel gave up (error word set): reported below
      if (rk > capacity) over = true;
      if (!over && rk > prev) {
        check_cuda(cudaStreamWaitEvent(R.d2h, R.ev[2 * k + 1], 0), "event wait");
        for (int j = 0; j < nout; j++) {
          const size_t w = type_size(plan_.outputs[j].type);
          check_cuda(cudaMemcpyAsync((char*)hout[j].data + prev * w, dbase + out_off[j] + prev * w,
                                     (size_t)(rk - prev) * w, cudaMemcpyDeviceToHost, R.d2h), "output chunk");
          const int64_t w0 = prev / 32, w1 = (rk + 31) / 32;
          check_cuda(cudaMemcpyAsync(hout[j].null_mask + w0, dbase + out_moff[j] + w0 * 4, (size_t)(w1 - w0) * 4,
                                     cudaMemcpyDeviceToHost, R.d2h), "output mask chunk");
        }
      }
      prev = std::max(prev, rk);
    }
    rows = prev;
    check_cuda(cudaEventRecord(drained, R.d2h), "event");
    check_cuda(cudaStreamWaitEvent(s, drained, 0), "event wait");
    check_cuda(cudaMemcpyAsync(R.blk + 128, dbase + err_off, 4, cudaMemcpyDeviceToHost, s), "error word");
    check_cuda(cudaStreamSynchronize(s), "host pipeline sync");
  } catch (...) {
    if (launched) {
      cudaStreamSynchronize(R.h2d);
      cudaStreamSynchronize(R.d2h);
    }
    dev_free(dbase, s);
    throw;
  }
  dev_free(dbase, s);
  if ((int)R.blk[128] != 0) fail(GX_ERR_TIMEOUT, "compaction look-back wait timed out");
  if (out_rows) *out_rows = rows;
  if (over) fail(GX_ERR_CAPACITY, "host output capacity too small");
  for (int j = 0; j < nout; j++) hout[j].size = rows;
}

}  // namespace gx
