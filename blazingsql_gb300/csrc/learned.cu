// learned.cu -- learned conjunct ordering and output sizing for filter plans.
//
// Per batch: a sampled column sketch (min, max, 8-bin histogram and null
// fraction per column, on every `stride`-th 32-row word) feeds a small FP32
// MLP (features -> 64 -> 64 -> one output per AND conjunct) that predicts each
// conjunct's selectivity.  The filter then runs single pass, evaluating the
// conjuncts most-selective first with per-word short-circuit (dead 32-row words
// skip the remaining conjuncts' column loads), into outputs sized from the
// predicted row count; a misprediction that overflows re-runs with the exact
// count, so results are always identical to the plain path.  The plain
// fixed-order evaluator supplies the training labels on warm-up batches and
// every `relabel_every`-th batch: in one fused pass (no short-circuit, every
// conjunct evaluated for every row) that also counts each conjunct's passing
// rows.  The plain fixed-order two-pass evaluator remains the PLAIN policy and
// the judge.  Forward, backward and Adam run in the kernels below.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "learned.h"

namespace gx {

// ------------------------------------------------------------------ sketches
// Each column is sketched in a signed log distance from its anchor -- the
// constant the condition compares it with (0 when none): t = sign(d) *
// log1p(|d|), d = x - anchor.  Features per column: min t / 16, max t / 16, the
// 8-bin histogram of t as cumulative fractions (bins t < -8, [-8, -4), [-4, -1),
// [-1, 0), t == 0, (0, 1], (1, 4], > 4: the bins around 0 separate x < anchor,
// x == anchor and x > anchor, so a conjunct's pass fraction is close to a sum
// of bins), and the null fraction.
constexpr int kSketchBins = 8;
constexpr int kFeatPerCol = kSketchBins + 3;   // min, max, cumulative hist[8], null fraction
constexpr int kPartial = kSketchBins + 4;      // min, max, hist[8], valid count, null count

struct SketchCols {
  const void* data[kMaxSketchCols];
  const uint32_t* mask[kMaxSketchCols];
  int64_t off[kMaxSketchCols];
  int type[kMaxSketchCols];
  double anchor[kMaxSketchCols];
};

__device__ __forceinline__ double sketch_value(const void* d, int type, int64_t i) {
  switch (type) {
    case INT8: return (double)((const signed char*)d)[i];
    case UINT8: case BOOL8: return (double)((const unsigned char*)d)[i];
    case INT16: return (double)((const short*)d)[i];
    case UINT16: return (double)((const unsigned short*)d)[i];
    case INT32: case TIMESTAMP_DAYS: case DURATION_DAYS: return (double)((const int*)d)[i];
    case UINT32: return (double)((const unsigned*)d)[i];
    case FLOAT32: return (double)((const float*)d)[i];
    case FLOAT64: return ((const double*)d)[i];
    case UINT64: return (double)((const unsigned long long*)d)[i];
    default: return (double)((const long long*)d)[i];
  }
}

__device__ __forceinline__ int sketch_bin(float t) {
  if (t < 0.f) return t < -8.f ? 0 : (t < -4.f ? 1 : (t < -1.f ? 2 : 3));
  if (t == 0.f) return 4;
  return t <= 1.f ? 5 : (t <= 4.f ? 6 : 7);
}

// Partial sketch of column blockIdx.y over this block's share of the sampled
// words, written to partial[col][blockIdx.x][kPartial].
__device__ void sketch_partial_block(const SketchCols& c, int64_t n, int64_t stride_words, float* partial) {
  const int col = blockIdx.y, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nwords = (n + 31) / 32;
  // columns without a fixed width (none among a valid plan's inputs) are not read
  const int64_t nsamp = c.data[col] == nullptr ? 0 : (nwords + stride_words - 1) / stride_words;
  const double anchor = c.anchor[col];
  float mn = INFINITY, mx = -INFINITY;
  float hist[kSketchBins];
#pragma unroll
  for (int i = 0; i < kSketchBins; i++) hist[i] = 0.f;
  float valid_n = 0.f, null_n = 0.f;
  const int64_t step = (int64_t)gridDim.x * 8;
  // four sampled words per warp at a time: their loads are in flight together
  for (int64_t s0 = (int64_t)blockIdx.x * 8 + warp; s0 < nsamp; s0 += 4 * step) {
    double v[4];
    int st[4];  // 0 absent, 1 null, 2 valid
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int64_t s = s0 + q * step;
      const int64_t row = s * stride_words * 32 + lane;
      st[q] = 0;
      v[q] = 0.0;
      if (s < nsamp && row < n) {
        const int64_t bit = c.off[col] + row;
        const bool valid = c.mask[col] == nullptr || ((c.mask[col][bit >> 5] >> (bit & 31)) & 1u);
        st[q] = valid ? 2 : 1;
        if (valid) v[q] = sketch_value(c.data[col], c.type[col], c.off[col] + row);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (st[q] == 1) null_n += 1.f;
      if (st[q] != 2) continue;
      const float d = (float)(v[q] - anchor);
      const float t = copysignf(log1pf(fabsf(d)), d);
      mn = fminf(mn, t);
      mx = fmaxf(mx, t);
      const int b = sketch_bin(t);
#pragma unroll
      for (int i = 0; i < kSketchBins; i++) hist[i] += (i == b) ? 1.f : 0.f;
      valid_n += 1.f;
    }
  }
  __shared__ float red[8][kPartial];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    valid_n += __shfl_xor_sync(0xffffffffu, valid_n, o);
    null_n += __shfl_xor_sync(0xffffffffu, null_n, o);
#pragma unroll
    for (int i = 0; i < kSketchBins; i++) hist[i] += __shfl_xor_sync(0xffffffffu, hist[i], o);
  }
  if (lane == 0) {
    red[warp][0] = mn;
    red[warp][1] = mx;
    for (int i = 0; i < kSketchBins; i++) red[warp][2 + i] = hist[i];
    red[warp][2 + kSketchBins] = valid_n;
    red[warp][3 + kSketchBins] = null_n;
  }
  __syncthreads();
  if (threadIdx.x < kPartial) {
    const int k = threadIdx.x;
    float v = red[0][k];
    for (int w = 1; w < 8; w++) v = k == 0 ? fminf(v, red[w][k]) : (k == 1 ? fmaxf(v, red[w][k]) : v + red[w][k]);
    partial[((int64_t)col * gridDim.x + blockIdx.x) * kPartial + k] = v;
  }
}

// One warp reduces column `col`'s partials (written by other blocks: read
// past L1) into its 11 features f[] (lane 0 writes).
__device__ void sketch_final_warp(const float* partial, int col, int nparts, float* f) {
  const int lane = threadIdx.x & 31;
  float mn = INFINITY, mx = -INFINITY, valid_n = 0.f, null_n = 0.f;
  float hist[kSketchBins];
#pragma unroll
  for (int i = 0; i < kSketchBins; i++) hist[i] = 0.f;
  for (int b = lane; b < nparts; b += 32) {
    const float* p = partial + ((int64_t)col * nparts + b) * kPartial;
    mn = fminf(mn, __ldcg(p + 0));
    mx = fmaxf(mx, __ldcg(p + 1));
#pragma unroll
    for (int i = 0; i < kSketchBins; i++) hist[i] += __ldcg(p + 2 + i);
    valid_n += __ldcg(p + 2 + kSketchBins);
    null_n += __ldcg(p + 3 + kSketchBins);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    valid_n += __shfl_xor_sync(0xffffffffu, valid_n, o);
    null_n += __shfl_xor_sync(0xffffffffu, null_n, o);
#pragma unroll
    for (int i = 0; i < kSketchBins; i++) hist[i] += __shfl_xor_sync(0xffffffffu, hist[i], o);
  }
  if (lane == 0) {
    f[0] = valid_n > 0.f ? mn * (1.f / 16.f) : 0.f;
    f[1] = valid_n > 0.f ? mx * (1.f / 16.f) : 0.f;
    float cum = 0.f;
    for (int i = 0; i < kSketchBins; i++) {
      cum += hist[i];
      f[2 + i] = valid_n > 0.f ? cum / valid_n : 0.f;
    }
    f[2 + kSketchBins] = (valid_n + null_n) > 0.f ? null_n / (valid_n + null_n) : 0.f;
  }
}

// ------------------------------------------------------------------ MLP
// Parameter layout (floats): W1[H*F] b1[H] W2[H*H] b2[H] W3[O*H] b3[O].
// Output z_o; predicted selectivity s_o = sigmoid(z_o); log s_o = -softplus(-z_o).
// The block-level routines below are run by every thread of one CTA.
__device__ __forceinline__ float softplusf(float x) { return fmaxf(x, 0.f) + log1pf(expf(-fabsf(x))); }

// y[m][j] = act(b[j] + sum_i W[j][i] x[m][i]) for every sample m and unit j:
// each warp takes 4 (m, j) dot products at a time, lanes striding over i, so
// weight rows are read coalesced and four rows' loads are in flight together.
__device__ void dense_layer_block(const float* W, const float* bias, int In, int Out, const float* X, int M,
                                  float* Y, bool relu) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int units = M * Out;
  for (int u0 = warp * 4; u0 < units; u0 += nw * 4) {
    const float* w[4];
    const float* x[4];
    float acc[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int u = min(u0 + q, units - 1);
      w[q] = W + (int64_t)(u % Out) * In;
      x[q] = X + (int64_t)(u / Out) * In;
      acc[q] = 0.f;
    }
    for (int i = lane; i < In; i += 32) {
#pragma unroll
      for (int q = 0; q < 4; q++) acc[q] += w[q][i] * x[q][i];
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
    }
    if (lane < 4 && u0 + lane < units) {
      float v = acc[0];
#pragma unroll
      for (int q = 1; q < 4; q++) v = lane == q ? acc[q] : v;
      const int u = u0 + lane;
      v += bias[u % Out];
      Y[u] = relu ? fmaxf(v, 0.f) : v;
    }
  }
}

// forward over M samples: H1, H2 (M*H) and Z (M*O) in global memory
__device__ void mlp_forward_block(const float* P, int F, int H, int O, const float* X, int M, float* H1, float* H2,
                                  float* Z) {
  const float* W1 = P;
  const float* b1 = W1 + H * F;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + O * H;
  dense_layer_block(W1, b1, F, H, X, M, H1, true);
  __syncthreads();
  dense_layer_block(W2, b2, H, H, H1, M, H2, true);
  __syncthreads();
  dense_layer_block(W3, b3, H, O, H2, M, Z, false);
  __syncthreads();
}

// Gradients of L = mean_{m,o} (log sigmoid(z_mo) - Y_mo)^2 into G (layout of
// P) and the loss into *loss; sm holds M*O + 2*M*H floats.
__device__ void mlp_backward_block(const float* P, int F, int H, int O, const float* X, int M, const float* H1,
                                   const float* H2, const float* Z, const float* Y, float* G, float* loss, float* sm) {
  float* dz = sm;                 // M*O
  float* dh2 = dz + M * O;        // M*H
  float* dh1 = dh2 + M * H;       // M*H
  const int t = threadIdx.x, nt = blockDim.x;
  const float* W2 = P + H * F + H;
  const float* W3 = W2 + H * H + H;
  float* gW1 = G;
  float* gb1 = gW1 + H * F;
  float* gW2 = gb1 + H;
  float* gb2 = gW2 + H * H;
  float* gW3 = gb2 + H;
  float* gb3 = gW3 + O * H;
  const float inv = 1.f / (float)(M * O);
  for (int i = t; i < M * O; i += nt) {
    const float z = Z[i];
    const float ls = -softplusf(-z);
    const float sig_neg = 1.f / (1.f + expf(z));  // d log(sigmoid(z)) / dz
    dz[i] = 2.f * inv * (ls - Y[i]) * sig_neg;
  }
  __syncthreads();
  if (loss && t == 0) {
    float l = 0.f;
    for (int i = 0; i < M * O; i++) {
      const float d = -softplusf(-Z[i]) - Y[i];
      l += d * d;
    }
    *loss = l * inv;
  }
  for (int i = t; i < O * H; i += nt) {
    const int o = i / H, k = i % H;
    float g = 0.f;
    for (int m = 0; m < M; m++) g += dz[m * O + o] * H2[m * H + k];
    gW3[i] = g;
  }
  for (int o = t; o < O; o += nt) {
    float g = 0.f;
    for (int m = 0; m < M; m++) g += dz[m * O + o];
    gb3[o] = g;
  }
  for (int i = t; i < M * H; i += nt) {
    const int m = i / H, k = i % H;
    float g = 0.f;
    for (int o = 0; o < O; o++) g += dz[m * O + o] * W3[o * H + k];
    dh2[i] = H2[i] > 0.f ? g : 0.f;
  }
  __syncthreads();
  for (int i = t; i < H * H; i += nt) {
    const int j = i / H, k = i % H;
    float g = 0.f;
    for (int m = 0; m < M; m++) g += dh2[m * H + j] * H1[m * H + k];
    gW2[i] = g;
  }
  for (int j = t; j < H; j += nt) {
    float g = 0.f;
    for (int m = 0; m < M; m++) g += dh2[m * H + j];
    gb2[j] = g;
  }
  for (int i = t; i < M * H; i += nt) {
    const int m = i / H, k = i % H;
    float g = 0.f;
    for (int j = 0; j < H; j++) g += dh2[m * H + j] * W2[j * H + k];
    dh1[i] = H1[i] > 0.f ? g : 0.f;
  }
  __syncthreads();
  for (int i = t; i < H * F; i += nt) {
    const int j = i / F, f = i % F;
    float g = 0.f;
    for (int m = 0; m < M; m++) g += dh1[m * H + j] * X[(int64_t)m * F + f];
    gW1[i] = g;
  }
  for (int j = t; j < H; j += nt) {
    float g = 0.f;
    for (int m = 0; m < M; m++) g += dh1[m * H + j];
    gb1[j] = g;
  }
  __syncthreads();
}

__device__ void forward_and_order(const float* s_x, const float* P, int F, int H, int O,
                                  const float* __restrict__ cost, float* s_h, float* Z, int* __restrict__ order,
                                  float* __restrict__ report);

// Sketch of every column plus, in the last block to finish, the feature rows
// and the network's forward pass for them (one launch per batch).  grid
// (kSketchParts, ncols); *ticket is zero on entry and left zero.
__global__ void __launch_bounds__(256) k_sketch_predict(SketchCols c, int64_t n, int64_t stride_words, int ncols,
                                                        float* __restrict__ partial, unsigned int* ticket,
                                                        const float* P, int H, int O,
                                                        float* __restrict__ features, float* __restrict__ Z,
                                                        const float* __restrict__ cost, int* __restrict__ order,
                                                        int stage_w, float* __restrict__ report) {
  // the last block reads the network's weights: one warp pulls them into L2
  // while the sample loads are in flight
  if (P && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 32) {
    const int np = H * (ncols * kFeatPerCol) + H + H * H + H + O * H + O;
    for (int i = threadIdx.x * 32; i < np; i += 32 * 32)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(P + i));
  }
  sketch_partial_block(c, n, stride_words, partial);
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int total = gridDim.x * gridDim.y;
    s_last = atomicAdd(ticket, 1u) == total - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int F = ncols * kFeatPerCol;
  // with dynamic shared memory for them, the weights are copied in first
  // (their loads overlap the partials' reduction) and read from there
  extern __shared__ float4 s_w4[];
  const bool wsm = P && stage_w;
  if (wsm) {
    const int np = H * F + H + H * H + H + O * H + O;
    const float4* P4 = reinterpret_cast<const float4*>(P);
#pragma unroll 4
    for (int i = threadIdx.x; i < np / 4; i += blockDim.x) s_w4[i] = __ldg(P4 + i);
    float* s_wf = reinterpret_cast<float*>(s_w4);
    for (int i = (np / 4) * 4 + threadIdx.x; i < np; i += blockDim.x) s_wf[i] = __ldg(P + i);
  }
  // features into shared memory (the forward pass reads them) and global
  // memory (a labelled batch's training example)
  __shared__ float s_x[kMaxSketchCols * kFeatPerCol];
  __shared__ float s_h[2 * 256];
  for (int col = threadIdx.x >> 5; col < ncols; col += blockDim.x >> 5)
    sketch_final_warp(partial, col, gridDim.x, s_x + col * kFeatPerCol);
  __syncthreads();
  if (wsm) P = reinterpret_cast<const float*>(s_w4);
  for (int i = threadIdx.x; i < F; i += blockDim.x) features[i] = s_x[i];
  if (threadIdx.x == 0) *ticket = 0u;
  if (P) forward_and_order(s_x, P, F, H, O, cost, s_h, Z, order, report);
}

// The network's forward pass on one feature row x (shared memory) by the whole
// block, its outputs to Z, and (when `order` is given) the conjunct order
// ranked on them, to `order` and, when given, with Z to the mapped `report`.
// s_h: 512 floats of shared memory.
__device__ void forward_and_order(const float* s_x, const float* P, int F, int H, int O,
                                  const float* __restrict__ cost, float* s_h, float* Z, int* __restrict__ order,
                                  float* __restrict__ report) {
  const float* W1 = P;
  const float* b1 = W1 + H * F;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + O * H;
  dense_layer_block(W1, b1, F, H, s_x, 1, s_h, true);
  __syncthreads();
  dense_layer_block(W2, b2, H, H, s_h, 1, s_h + 256, true);
  __syncthreads();
  dense_layer_block(W3, b3, H, O, s_h + 256, 1, Z, false);
  if (!order) return;
  // conjunct order from the prediction: rank = cost / (1 - selectivity),
  // ascending, ties by index (the host computes the same ranks)
  __syncthreads();
  if (threadIdx.x == 0) {
    float rank[16];
    int ord[16];
    for (int c = 0; c < O; c++) {
      const float z = Z[c];
      const float ls = -(fmaxf(-z, 0.f) + log1pf(expf(-fabsf(z))));
      rank[c] = cost[c] / fmaxf(1e-9f, 1.f - expf(ls));
      ord[c] = c;
    }
    for (int i = 1; i < O; i++) {
      const int v = ord[i];
      int j = i - 1;
      while (j >= 0 && rank[ord[j]] > rank[v]) {
        ord[j + 1] = ord[j];
        j--;
      }
      ord[j + 1] = v;
    }
    for (int c = 0; c < O; c++) order[c] = ord[c];
    // the batch report's copy, in mapped host memory: the host reads it
    // after its stream synchronisation, without a copy of its own
    if (report) {
      for (int c = 0; c < O; c++) {
        report[c] = Z[c];
        reinterpret_cast<int*>(report)[16 + c] = ord[c];
      }
    }
  }
}

// Sketches of every batch of a queue in one launch: grid (parts, ncols,
// batches), qc[b] / qn[b] batch b's columns and rows; the last block of each
// batch (tickets[b], zero on entry) reduces the batch's partials into its
// features (F = ncols * 11 floats at features + b * F).
__global__ void __launch_bounds__(256) k_sketch_queue(const SketchCols* __restrict__ qc,
                                                      const int64_t* __restrict__ qn, int64_t stride_words, int ncols,
                                                      float* __restrict__ partial, unsigned int* tickets,
                                                      float* __restrict__ features) {
  const int b = blockIdx.z;
  float* pb = partial + (size_t)b * ncols * gridDim.x * kPartial;
  sketch_partial_block(qc[b], qn[b], stride_words, pb);
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&tickets[b], 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  float* f = features + (size_t)b * ncols * kFeatPerCol;
  for (int col = threadIdx.x >> 5; col < ncols; col += blockDim.x >> 5)
    sketch_final_warp(pb, col, gridDim.x, f + col * kFeatPerCol);
}

// One batch's prediction from its features: forward pass, order to `order`
// (device) and the report (mapped host).  One block of 256 threads.
__global__ void __launch_bounds__(256) k_predict(const float* __restrict__ feat, int F, const float* __restrict__ P,
                                                 int H, int O, const float* __restrict__ cost,
                                                 int* __restrict__ order, float* __restrict__ report) {
  __shared__ float s_x[kMaxSketchCols * kFeatPerCol];
  __shared__ float s_h[2 * 256];
  __shared__ float s_z[16];
  for (int i = threadIdx.x; i < F; i += blockDim.x) s_x[i] = feat[i];
  __syncthreads();
  forward_and_order(s_x, P, F, H, O, cost, s_h, s_z, order, report);
}

// `steps` full-batch Adam steps over the M stored examples, one CTA; the loss
// of the last step's forward pass goes to *loss.
__global__ void __launch_bounds__(256) k_mlp_train(float* __restrict__ P, float* __restrict__ G,
                                                   float* __restrict__ Mo, float* __restrict__ Ve, int F, int H,
                                                   int O, const float* __restrict__ X, int M,
                                                   const float* __restrict__ Y, float* __restrict__ act, int steps,
                                                   int t0, float lr, float* __restrict__ loss) {
  extern __shared__ float sm[];
  const int np = H * F + H + H * H + H + O * H + O;
  float* H1 = act;
  float* H2 = H1 + M * H;
  float* Z = H2 + M * H;
  for (int it = 0; it < steps; it++) {
    mlp_forward_block(P, F, H, O, X, M, H1, H2, Z);
    mlp_backward_block(P, F, H, O, X, M, H1, H2, Z, Y, G, it == steps - 1 ? loss : nullptr, sm);
    const float tt = (float)(t0 + it + 1);
    const float c1 = 1.f - powf(0.9f, tt), c2 = 1.f - powf(0.999f, tt);
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const float g = G[i];
      const float m = 0.9f * Mo[i] + 0.1f * g;
      const float v = 0.999f * Ve[i] + 0.001f * g * g;
      Mo[i] = m;
      Ve[i] = v;
      P[i] -= lr * (m / c1) / (sqrtf(v / c2) + 1e-8f);
    }
    __syncthreads();
  }
}

// Shared-memory floats of k_mlp_train_smem: parameters and gradients, the
// examples and their labels, both hidden activations, the outputs and the
// backward pass's scratch.
__host__ __device__ inline size_t train_smem_floats(int F, int H, int O, int M) {
  const size_t np = (size_t)H * F + H + (size_t)H * H + H + (size_t)O * H + O;
  const size_t npa = (np + 3) / 4 * 4;
  return 2 * npa + (size_t)M * F + (size_t)M * O + 2 * (size_t)M * H + (size_t)M * O +
         ((size_t)M * O + 2 * (size_t)M * H);
}

// k_mlp_train with everything a step touches in shared memory (the Adam
// moments stay in global memory, read and written once per step) and 1024
// threads: the rounds are bound by dependent shared-memory arithmetic instead
// of L1/L2 latency.
__global__ void __launch_bounds__(1024) k_mlp_train_smem(float* __restrict__ P, float* __restrict__ Mo,
                                                         float* __restrict__ Ve, int F, int H, int O,
                                                         const float* __restrict__ X, int M,
                                                         const float* __restrict__ Y, int steps, int t0, float lr,
                                                         float* __restrict__ loss) {
  extern __shared__ float4 sm4[];
  float* sm = reinterpret_cast<float*>(sm4);
  const int np = H * F + H + H * H + H + O * H + O;
  const int npa = (np + 3) / 4 * 4;
  float* sP = sm;
  float* sG = sP + npa;
  float* sX = sG + npa;
  float* sY = sX + M * F;
  float* sH1 = sY + M * O;
  float* sH2 = sH1 + M * H;
  float* sZ = sH2 + M * H;
  float* sB = sZ + M * O;
  for (int i = threadIdx.x; i < np; i += blockDim.x) sP[i] = P[i];
  for (int i = threadIdx.x; i < M * F; i += blockDim.x) sX[i] = X[i];
  for (int i = threadIdx.x; i < M * O; i += blockDim.x) sY[i] = Y[i];
  __syncthreads();
  for (int it = 0; it < steps; it++) {
    mlp_forward_block(sP, F, H, O, sX, M, sH1, sH2, sZ);
    mlp_backward_block(sP, F, H, O, sX, M, sH1, sH2, sZ, sY, sG, it == steps - 1 ? loss : nullptr, sB);
    const float tt = (float)(t0 + it + 1);
    const float c1 = 1.f - powf(0.9f, tt), c2 = 1.f - powf(0.999f, tt);
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const float g = sG[i];
      const float m = 0.9f * Mo[i] + 0.1f * g;
      const float v = 0.999f * Ve[i] + 0.001f * g * g;
      Mo[i] = m;
      Ve[i] = v;
      sP[i] -= lr * (m / c1) / (sqrtf(v / c2) + 1e-8f);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < np; i += blockDim.x) P[i] = sP[i];
}

// one forward + backward pass (gradient checks)
__global__ void __launch_bounds__(256) k_mlp_grad(const float* __restrict__ P, float* __restrict__ G, int F, int H,
                                                  int O, const float* __restrict__ X, int M,
                                                  const float* __restrict__ Y, float* __restrict__ act,
                                                  float* __restrict__ loss) {
  extern __shared__ float sm[];
  float* H1 = act;
  float* H2 = H1 + M * H;
  float* Z = H2 + M * H;
  mlp_forward_block(P, F, H, O, X, M, H1, H2, Z);
  mlp_backward_block(P, F, H, O, X, M, H1, H2, Z, Y, G, loss, sm);
}

// labelled example `slot`: the batch's features and log pass-rate per conjunct
__global__ void k_add_example(const float* __restrict__ feat, const unsigned long long* __restrict__ counts,
                              long long n, int F, int O, float* __restrict__ X, float* __restrict__ Y) {
  for (int i = threadIdx.x; i < F; i += blockDim.x) X[i] = feat[i];
  if (threadIdx.x < O) Y[threadIdx.x] = logf((float)((double)counts[threadIdx.x] / (double)n) + 1e-6f);
}

// ------------------------------------------------------------------ host side
int mlp_param_count(int F, int H, int O) { return H * F + H + H * H + H + O * H + O; }

static void check_mlp_shape(int F, int H, int O, int M) {
  if (F <= 0 || F > 4096 || H <= 0 || O <= 0 || H > 256 || O > 256 || M <= 0 || M * H > 4096 || M * O > 1024)
    fail(GX_ERR_INVALID, "MLP shape out of range");
}

static int backward_smem(int H, int O, int M) { return (M * O + 2 * M * H) * 4; }

void mlp_grad(const float* dP, int F, int H, int O, const float* dX, int M, const float* dY, float* dG, float* dloss,
              float* dact, cudaStream_t s) {
  check_mlp_shape(F, H, O, M);
  k_mlp_grad<<<1, 256, backward_smem(H, O, M), s>>>(dP, dG, F, H, O, dX, M, dY, dact, dloss);
  check_cuda(cudaGetLastError(), "k_mlp_grad");
  add_launches(1);
}

static void* must_alloc(size_t bytes) {
  void* p = nullptr;
  const cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? GX_ERR_OOM : GX_ERR_CUDA, "learner device buffers");
  }
  return p;
}

static std::shared_ptr<CompiledPlan> variant(const CompiledPlan& base, int mode, bool stats, bool runtime_order,
                                             int words = 0) {
  KernelConfig c = base.config();
  if (words > 0) c.words = words;
  c.tune_shape = false;  // the learner's variants keep one shape
  c.short_circuit = false;
  c.conjunct_order.clear();
  c.conj_stats = stats;
  c.runtime_order = runtime_order;
  if (runtime_order) {
    c.dense = true;
    // conjunct columns staged in shared memory by asynchronous copies: measured
    // slower than direct predicated loads on the C4 batches, so on request only
    const char* e = std::getenv("GX_STAGED");
    c.staged = e && *e == '1';
    // word slots in flight per warp for the short-circuit chain: measured slower
    // than the lockstep words of a 4 x 8 block on the C4 batches (83 vs 60 us),
    // so on request only (GX_STREAM=<slots>)
    const char* st = std::getenv("GX_STREAM");
    c.stream_slots = st && *st ? std::atoi(st) : 0;
  }
  return std::make_shared<CompiledPlan>(base.plan(), c, mode);
}

// nanoseconds per unit of a timestamp / duration type (1 for other types)
static double unit_ns(int t) {
  switch (t) {
    case TIMESTAMP_DAYS: case DURATION_DAYS: return 86400e9;
    case TIMESTAMP_SECONDS: case DURATION_SECONDS: return 1e9;
    case TIMESTAMP_MILLISECONDS: case DURATION_MILLISECONDS: return 1e6;
    case TIMESTAMP_MICROSECONDS: case DURATION_MICROSECONDS: return 1e3;
    default: return 1.0;
  }
}

static double literal_value(const Node& n) {
  if (n.lit_type == FLOAT64 || n.lit_type == FLOAT32) {
    double d;
    std::memcpy(&d, &n.lit_bits, 8);
    return d;
  }
  if (n.lit_type == UINT64) return (double)n.lit_bits;
  return (double)(int64_t)n.lit_bits;
}

// The sketch anchor of each column: the first literal a conjunct compares the
// column with (through casts), in the column's own units; 0 when none.
std::vector<double> sketch_anchors(const Plan& p, int ncols) {
  std::vector<double> a(ncols, 0.0);
  std::vector<bool> set(ncols, false);
  auto col_of = [&](int id) {
    while (id >= 0 && p.nodes[id].kind == Node::OP && p.nodes[id].op >= OP_CAST_TINYINT &&
           p.nodes[id].op <= OP_CAST_TIMESTAMP)
      id = p.nodes[id].a;
    return (id >= 0 && p.nodes[id].kind == Node::COL) ? p.nodes[id].col : -1;
  };
  for (int cid : p.conjuncts) {
    const Node& n = p.nodes[cid];
    if (n.kind != Node::OP || n.op < OP_EQ || n.op > OP_GE) continue;
    for (int side = 0; side < 2; side++) {
      const int ci = col_of(side == 0 ? n.a : n.b);
      const int li = side == 0 ? n.b : n.a;
      if (ci < 0 || ci >= ncols || set[ci] || li < 0 || p.nodes[li].kind != Node::LIT || !p.nodes[li].lit_valid)
        continue;
      const Node& lit = p.nodes[li];
      double v = literal_value(lit);
      const int ct = p.schema[ci];
      if ((is_timestamp(ct) || is_duration(ct)) && (is_timestamp(lit.lit_type) || is_duration(lit.lit_type)))
        v = v * unit_ns(lit.lit_type) / unit_ns(ct);
      a[ci] = v;
      set[ci] = true;
    }
  }
  return a;
}

Learner::Learner(const CompiledPlan& base, const LearnerOptions& opt) : opt_(opt) {
  const Plan& p = base.plan();
  if (!p.has_filter()) fail(GX_ERR_INVALID, "a learner needs a plan with a condition");
  if (p.conjuncts.size() > 16) fail(GX_ERR_UNSUPPORTED, "learned ordering supports at most 16 AND conjuncts");
  if (opt_.hidden < 1 || opt_.hidden > 256) fail(GX_ERR_INVALID, "hidden width must be 1..256");
  if (opt_.policy < GX_LEARN_POLICY_LEARNED || opt_.policy > GX_LEARN_POLICY_TEXTUAL)
    fail(GX_ERR_INVALID, "unknown learner policy");
  if (opt_.stride_words < 1) opt_.stride_words = 1;
  plain_ = variant(base, GX_FILTER_TWO_PASS, false, false);
  label_ = variant(base, GX_FILTER_SINGLE_PASS, true, false, opt_.fast_words);
  fast_ = variant(base, GX_FILTER_SINGLE_PASS, false, true, opt_.fast_words);
  ncols_ = std::min((int)p.schema.size(), kMaxSketchCols);
  nconj_ = (int)p.conjuncts.size();
  // cost of a conjunct: bytes per row of the distinct columns its cone reads
  for (int c = 0; c < nconj_; c++) {
    std::vector<int> stack{p.conjuncts[c]}, seen(p.nodes.size(), 0), colseen(p.schema.size(), 0);
    double bytes = 0;
    while (!stack.empty()) {
      const int id = stack.back();
      stack.pop_back();
      if (id < 0 || seen[id]) continue;
      seen[id] = 1;
      const Node& nd = p.nodes[id];
      if (nd.kind == Node::COL && !colseen[nd.col]) {
        colseen[nd.col] = 1;
        bytes += type_size(p.schema[nd.col]) + 0.125;
      } else if (nd.kind == Node::OP) {
        stack.push_back(nd.a);
        stack.push_back(nd.b);
      }
    }
    conj_cost_.push_back(bytes > 0 ? bytes : 0.125);
  }
  anchors_ = sketch_anchors(p, ncols_);
  F_ = ncols_ * kFeatPerCol;
  H_ = opt_.hidden;
  O_ = nconj_;
  nparams_ = mlp_param_count(F_, H_, O_);
  if (opt_.policy != GX_LEARN_POLICY_LEARNED) {
    // the comparison policies need no network; the textual one may run queues
    if (opt_.policy == GX_LEARN_POLICY_TEXTUAL) {
      try {
        reserve_queue(kQueueReserve);
      } catch (...) {
        release();
        throw;
      }
    }
    return;
  }
  try {
    dparams_ = (float*)must_alloc((size_t)nparams_ * 4 * 5);  // P, G, Adam m, v, inference copy
    dgrad_ = dparams_ + nparams_;
    dmom_ = dgrad_ + nparams_;
    dvel_ = dmom_ + nparams_;
    dinfer_ = dvel_ + nparams_;
    dtrainX_ = (float*)must_alloc((size_t)F_ * 4 * kTrainRing);
    // prediction slots: features, z, order, partials, ticket (each part 16-float aligned)
    const size_t fpart = ((size_t)F_ + 15) / 16 * 16;
    const size_t ppart = (size_t)kPartial * kMaxSketchCols * kSketchParts;
    const size_t per = fpart + 16 + 16 + ppart + 16;
    dslots_ = (float*)must_alloc(4 * per * kPredSlots);
    for (int q = 0; q < kPredSlots; q++) {
      float* b = dslots_ + per * q;
      slots_[q].feat = b;
      slots_[q].z = b + fpart;
      slots_[q].order = (int*)(b + fpart + 16);
      slots_[q].partial = b + fpart + 32;
      slots_[q].ticket = (unsigned int*)(b + fpart + 32 + ppart);
    }
    dtrainY_ = (float*)must_alloc((size_t)O_ * 4 * kTrainRing);
    dsnapX_ = (float*)must_alloc((size_t)(F_ + O_) * 4 * kTrainRing);
    dsnapY_ = dsnapX_ + (size_t)F_ * kTrainRing;
    dact_ = (float*)must_alloc((size_t)4 * (2 * kTrainRing * H_ + kTrainRing * O_ + 4));
    dcounts_ = (unsigned long long*)must_alloc(8 * 16);
    dcost_ = (float*)must_alloc(4 * 16);
    // pinned, mapped host block: predictions z[16], the loss at [16], conjunct
    // counts from byte 256, each slot's report (z[16], order[16]) from byte 512
    check_cuda(cudaHostAlloc((void**)&hpinned_, 512 + 128 * kPredSlots, cudaHostAllocMapped | cudaHostAllocPortable),
               "pinned host buffer");
    std::memset(hpinned_, 0, 512 + 128 * kPredSlots);
    hcounts_ = (unsigned long long*)((char*)hpinned_ + 256);
    float* dpinned = nullptr;
    check_cuda(cudaHostGetDevicePointer((void**)&dpinned, hpinned_, 0), "mapped host buffer");
    for (int q = 0; q < kPredSlots; q++) {
      slots_[q].report = hpinned_ + 128 + 32 * q;
      slots_[q].report_dev = dpinned + 128 + 32 * q;
    }
    check_cuda(cudaStreamCreateWithFlags(&aux_stream_, cudaStreamNonBlocking), "aux stream");
    check_cuda(cudaEventCreateWithFlags(&prep_in_, cudaEventDisableTiming), "event");
    for (int q = 0; q < kPredSlots; q++)
      check_cuda(cudaEventCreateWithFlags(&slots_[q].ready, cudaEventDisableTiming), "event");
    for (int q = 0; q < kPredEvents; q++) check_cuda(cudaEventCreateWithFlags(&qev_[q], cudaEventDisableTiming), "event");
    check_cuda(cudaEventCreateWithFlags(&qsketch_done_, cudaEventDisableTiming), "event");
    if (opt_.async_training) {
      check_cuda(cudaStreamCreateWithFlags(&train_stream_, cudaStreamNonBlocking), "training stream");
      check_cuda(cudaEventCreateWithFlags(&train_done_, cudaEventDisableTiming), "event");
      check_cuda(cudaEventCreateWithFlags(&labels_ready_, cudaEventDisableTiming), "event");
    }
  } catch (...) {
    release();
    throw;
  }
  // uniform(-a, a) initialisation with a = sqrt(6 / fan_in), from a fixed seed
  std::vector<float> init(nparams_, 0.f);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ (opt_.seed * 0xD1B54A32D192ED03ull);
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return ((double)(st >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
  };
  size_t o = 0;
  for (int i = 0; i < H_ * F_; i++) init[o++] = (float)(rnd() * std::sqrt(6.0 / F_));
  o += H_;
  for (int i = 0; i < H_ * H_; i++) init[o++] = (float)(rnd() * std::sqrt(6.0 / H_));
  o += H_;
  for (int i = 0; i < O_ * H_; i++) init[o++] = (float)(rnd() * std::sqrt(3.0 / H_));
  try {
    check_cuda(cudaMemcpy(dparams_, init.data(), (size_t)nparams_ * 4, cudaMemcpyHostToDevice), "init params");
    check_cuda(cudaMemcpy(dinfer_, init.data(), (size_t)nparams_ * 4, cudaMemcpyHostToDevice), "init params");
    check_cuda(cudaMemset(dmom_, 0, (size_t)nparams_ * 8), "init adam");
    check_cuda(cudaMemset(dslots_, 0, 4 * (slots_[1].feat - slots_[0].feat) * kPredSlots), "init slots");
    std::vector<float> cost(16, 0.f);
    for (int c = 0; c < nconj_; c++) cost[c] = (float)conj_cost_[c];
    check_cuda(cudaMemcpy(dcost_, cost.data(), 4 * 16, cudaMemcpyHostToDevice), "init costs");
    reserve_queue(kQueueReserve);
  } catch (...) {
    release();
    throw;
  }
}

void Learner::release() {
  if (train_stream_) cudaStreamSynchronize(train_stream_);
  cudaFree(dparams_);
  cudaFree(dtrainX_);
  cudaFree(dslots_);
  cudaFree(dtrainY_);
  cudaFree(dsnapX_);
  cudaFree(dact_);
  cudaFree(dcounts_);
  cudaFree(dcost_);
  if (hpinned_) cudaFreeHost(hpinned_);
  if (hqueue_) cudaFreeHost(hqueue_);
  hqueue_ = nullptr;
  queue_cap_ = 0;
  cudaFree(dqsk_);
  if (hqsk_) cudaFreeHost(hqsk_);
  dqsk_ = hqsk_ = nullptr;
  qsk_cap_ = 0;
  for (int q = 0; q < kPredEvents; q++) {
    if (qev_[q]) cudaEventDestroy(qev_[q]);
    qev_[q] = nullptr;
  }
  for (int q = 0; q < 8; q++) {
    if (qdone_[q]) cudaEventDestroy(qdone_[q]);
    qdone_[q] = nullptr;
  }
  if (qsketch_done_) cudaEventDestroy(qsketch_done_);
  qsketch_done_ = nullptr;
  if (train_done_) cudaEventDestroy(train_done_);
  if (labels_ready_) cudaEventDestroy(labels_ready_);
  if (train_stream_) cudaStreamDestroy(train_stream_);
  if (aux_stream_) cudaStreamDestroy(aux_stream_);
  aux_stream_ = nullptr;
  for (int q = 0; q < kPredSlots; q++) {
    if (slots_[q].ready) cudaEventDestroy(slots_[q].ready);
    slots_[q] = PredSlot{};
  }
  if (prep_in_) cudaEventDestroy(prep_in_);
  prep_in_ = nullptr;
  dparams_ = dtrainX_ = dtrainY_ = dact_ = hpinned_ = dsnapX_ = dsnapY_ = dslots_ = nullptr;
  dcounts_ = nullptr;
  dcost_ = nullptr;
  train_done_ = labels_ready_ = nullptr;
  train_stream_ = nullptr;
}

Learner::~Learner() { release(); }

void Learner::sketch(const std::vector<ColumnView>& cols, bool predict, cudaStream_t s, int slot,
                     float* report_dev, float* report_host) {
  PredSlot& ps = slots_[slot];
  if (!report_dev) {
    report_dev = ps.report_dev;
    report_host = ps.report;
  }
  ps.cur_report = report_host;
  SketchCols c{};
  for (int i = 0; i < ncols_; i++) {
    c.data[i] = cols[i].data;
    c.mask[i] = cols[i].mask;
    c.off[i] = cols[i].offset;
    c.type[i] = cols[i].type;
    c.anchor[i] = anchors_[i];
    if (type_size(cols[i].type) == 0) c.data[i] = nullptr;
  }
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  dim3 grid(kSketchParts, ncols_);
  // weights in dynamic shared memory when they fit the default 48 KB
  const size_t wbytes = (size_t)nparams_ * 4;
  const bool stage_w = predict && wbytes <= 48 * 1024;
  k_sketch_predict<<<grid, 256, stage_w ? wbytes : 0, s>>>(
      c, n, opt_.stride_words, ncols_, ps.partial, ps.ticket, predict ? dinfer_ : nullptr, H_, O_, ps.feat, ps.z,
      dcost_, predict ? ps.order : nullptr, stage_w ? 1 : 0, predict ? report_dev : nullptr);
  check_cuda(cudaGetLastError(), "k_sketch_predict");
  add_launches(1);
}

std::vector<float> Learner::features(const std::vector<ColumnView>& cols, cudaStream_t s) {
  if (!dslots_) fail(GX_ERR_INVALID, "this learner has no network (policy is not LEARNED)");
  if ((int)cols.size() != (int)plain_->plan().schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  std::vector<float> f(F_, 0.f);
  if (!cols.empty() && cols[0].size > 0) sketch(cols, false, s, 0);
  else check_cuda(cudaMemsetAsync(slots_[0].feat, 0, (size_t)F_ * 4, s), "features");
  check_cuda(cudaMemcpyAsync(f.data(), slots_[0].feat, (size_t)F_ * 4, cudaMemcpyDeviceToHost, s), "features");
  check_cuda(cudaStreamSynchronize(s), "features");
  return f;
}

std::vector<uintptr_t> Learner::batch_key(const std::vector<ColumnView>& cols) const {
  std::vector<uintptr_t> k;
  for (int i = 0; i < ncols_ && i < (int)cols.size(); i++) {
    k.push_back((uintptr_t)cols[i].data);
    k.push_back((uintptr_t)cols[i].offset);
    k.push_back((uintptr_t)cols[i].mask);
  }
  k.push_back(cols.empty() ? 0 : (uintptr_t)cols[0].size);
  return k;
}

// The look-ahead slot holding this batch, if any: the stream waits for it and
// the slot is released.
int Learner::take_prepared(const std::vector<ColumnView>& cols, cudaStream_t s) {
  bool any = false;
  for (int q = 1; q < kPredSlots; q++) any |= slots_[q].valid;
  if (!any) return -1;
  const std::vector<uintptr_t> key = batch_key(cols);
  for (int q = 1; q < kPredSlots; q++) {
    if (!slots_[q].valid || slots_[q].key != key) continue;
    check_cuda(cudaStreamWaitEvent(s, slots_[q].ready, 0), "wait look-ahead");
    slots_[q].valid = false;
    return q;
  }
  return -1;
}

void Learner::prepare(const std::vector<ColumnView>& cols, cudaStream_t s, float* report_dev, float* report_host) {
  if (opt_.policy != GX_LEARN_POLICY_LEARNED || !dslots_) return;
  const auto& schema = plain_->plan().schema;
  if (cols.size() != schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  for (size_t i = 0; i < cols.size(); i++)
    if (cols[i].type != schema[i]) fail(GX_ERR_INVALID, "column type does not match the plan");
  if (cols.empty() || cols[0].size == 0) return;
  const int q = prep_next_;
  prep_next_ = prep_next_ + 1 < kPredSlots ? prep_next_ + 1 : 1;
  // the columns are ready once the caller's stream reaches this point
  check_cuda(cudaEventRecord(prep_in_, s), "look-ahead event");
  check_cuda(cudaStreamWaitEvent(aux_stream_, prep_in_, 0), "wait columns");
  sync_inference_params(aux_stream_);
  sketch(cols, true, aux_stream_, q, report_dev, report_host);
  check_cuda(cudaEventRecord(slots_[q].ready, aux_stream_), "look-ahead ready");
  slots_[q].key = batch_key(cols);
  slots_[q].valid = true;
}

void Learner::sync_inference_params(cudaStream_t s) {
  if (!params_pending_) return;
  if (train_stream_) {
    if (cudaEventQuery(train_done_) != cudaSuccess) {
      cudaGetLastError();  // still training: keep predicting with the previous version
      return;
    }
    check_cuda(cudaStreamWaitEvent(s, train_done_, 0), "wait training");
  }
  check_cuda(cudaMemcpyAsync(dinfer_, dparams_, (size_t)nparams_ * 4, cudaMemcpyDeviceToDevice, s), "params copy");
  params_pending_ = false;
}

std::vector<float> Learner::predict_log_sel(const std::vector<ColumnView>& cols, cudaStream_t s) {
  int slot = take_prepared(cols, s);
  if (slot < 0) {
    sync_inference_params(s);
    sketch(cols, true, s, 0);
    slot = 0;
  }
  check_cuda(cudaMemcpyAsync(hpinned_, slots_[slot].z, O_ * 4, cudaMemcpyDeviceToHost, s), "prediction");
  check_cuda(cudaStreamSynchronize(s), "prediction sync");
  std::vector<float> ls(O_);
  for (int o = 0; o < O_; o++) {
    const float z = hpinned_[o];
    ls[o] = -(std::max(-z, 0.f) + std::log1p(std::exp(-std::fabs(z))));  // log sigmoid(z)
  }
  return ls;
}

void Learner::add_example(const unsigned long long* counts, int64_t n, cudaStream_t s, const float* feat) {
  const int slot = (int)(seen_ % (uint64_t)kTrainRing);
  // (a side-stream training round reads a snapshot of the ring, not the ring)
  k_add_example<<<1, 128, 0, s>>>(feat, counts, (long long)n, F_, O_, dtrainX_ + (size_t)slot * F_,
                                  dtrainY_ + (size_t)slot * O_);
  check_cuda(cudaGetLastError(), "k_add_example");
  add_launches(1);
  seen_++;
}

// Dynamic shared memory the shared-memory training kernel may use on the
// current device (its opt-in limit, raised once per device).
static size_t train_smem_limit() {
  static std::mutex mu;
  static std::unordered_map<int, size_t> lim;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "device");
  std::lock_guard<std::mutex> g(mu);
  auto it = lim.find(dev);
  if (it != lim.end()) return it->second;
  int optin = 0;
  check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "shared memory limit");
  size_t v = 0;
  if (cudaFuncSetAttribute(k_mlp_train_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) == cudaSuccess)
    v = (size_t)optin;
  cudaGetLastError();
  lim[dev] = v;
  return v;
}

void Learner::train(int steps, cudaStream_t s) {
  // full-batch Adam over every stored example (the ring's order is irrelevant)
  const int M = (int)std::min<uint64_t>({seen_, (uint64_t)kTrainRing, (uint64_t)(4096 / H_), (uint64_t)(1024 / O_)});
  if (M == 0 || steps <= 0) return;
  check_mlp_shape(F_, H_, O_, M);
  cudaStream_t ts = s;
  const float* X = dtrainX_;
  const float* Y = dtrainY_;
  if (train_stream_) {
    // one round at a time on the side stream; a round asked for meanwhile
    // starts once the running one has finished (execute checks)
    if (cudaEventQuery(train_done_) != cudaSuccess) {
      cudaGetLastError();
      train_pending_ = true;
      return;
    }
    // the round trains on a snapshot, so later batches may add examples
    // without waiting for it
    check_cuda(cudaMemcpyAsync(dsnapX_, dtrainX_, (size_t)M * F_ * 4, cudaMemcpyDeviceToDevice, s), "snapshot X");
    check_cuda(cudaMemcpyAsync(dsnapY_, dtrainY_, (size_t)M * O_ * 4, cudaMemcpyDeviceToDevice, s), "snapshot Y");
    check_cuda(cudaEventRecord(labels_ready_, s), "labels event");
    check_cuda(cudaStreamWaitEvent(train_stream_, labels_ready_, 0), "wait labels");
    ts = train_stream_;
    X = dsnapX_;
    Y = dsnapY_;
  }
  train_pending_ = false;
  float* dloss = dact_ + 2 * kTrainRing * H_ + kTrainRing * O_;
  const size_t smem = train_smem_floats(F_, H_, O_, M) * 4;
  if (smem <= train_smem_limit()) {
    k_mlp_train_smem<<<1, 1024, smem, ts>>>(dparams_, dmom_, dvel_, F_, H_, O_, X, M, Y, steps, adam_t_, opt_.lr,
                                             dloss);
  } else {
    k_mlp_train<<<1, 256, backward_smem(H_, O_, M), ts>>>(dparams_, dgrad_, dmom_, dvel_, F_, H_, O_, X, M, Y, dact_,
                                                          steps, adam_t_, opt_.lr, dloss);
  }
  check_cuda(cudaGetLastError(), "k_mlp_train");
  add_launches(1);
  adam_t_ += steps;
  check_cuda(cudaMemcpyAsync(hpinned_ + 16, dloss, 4, cudaMemcpyDeviceToHost, ts), "loss");
  if (train_stream_) check_cuda(cudaEventRecord(train_done_, ts), "training event");
  params_pending_ = true;
}

void Learner::poll_training() {
  if (train_stream_ && cudaEventQuery(train_done_) == cudaSuccess) loss_ = hpinned_[16];
  cudaGetLastError();  // a round still running answers cudaErrorNotReady
}

void Learner::execute(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                      gx_learned_batch_info* info, cudaStream_t s) {
  execute_one(cols, out, out_rows, info, s, nullptr);
}

void Learner::execute_one(const std::vector<ColumnView>& cols, gx_column* out, int64_t* out_rows,
                          gx_learned_batch_info* info, cudaStream_t s, Deferred* d) {
  gx_learned_batch_info bi;
  std::memset(&bi, 0, sizeof bi);
  bi.num_conjuncts = nconj_;
  const int64_t n = cols.empty() ? 0 : cols[0].size;
  if ((int)cols.size() != (int)plain_->plan().schema.size()) fail(GX_ERR_INVALID, "column count does not match the plan");
  batches_++;
  if (opt_.policy == GX_LEARN_POLICY_PLAIN) {
    plain_->execute(cols, out, out_rows, s);
    bi.rows = out_rows ? *out_rows : 0;
    if (info) *info = bi;
    return;
  }
  if (opt_.policy == GX_LEARN_POLICY_TEXTUAL) {
    ExecExtras ex;
    std::vector<int> order(nconj_);
    std::iota(order.begin(), order.end(), 0);
    ex.order = order.data();
    ex.num_order = nconj_;
    if (d) fast_->enqueue_filter(cols, out, d->hdr_dev, d->status, &ex, s);
    else fast_->execute(cols, out, out_rows, s, &ex);
    for (int o = 0; o < nconj_; o++) bi.order[o] = o;
    bi.path = 1;
    bi.rows = out_rows ? *out_rows : 0;
    if (info) *info = bi;
    return;
  }
  // a training round asked for while the previous one ran starts now if it can
  if (train_pending_ && train_stream_ && cudaEventQuery(train_done_) == cudaSuccess) train(opt_.train_steps, s);
  cudaGetLastError();
  const bool warm = labelled_ < (uint64_t)opt_.warmup_batches;
  const bool relabel = !warm && opt_.relabel_every > 0 && since_label_ >= opt_.relabel_every;
  if (warm || relabel || n == 0) {
    since_label_ = 0;
    // the plain fixed-order evaluator in one pass (every conjunct evaluated for
    // every row): output + per-conjunct pass counts (queued: the counters sit in
    // the batch's zeroed header, read after the queue)
    unsigned long long* counts = d ? d->hdr_dev + 4 : dcounts_;
    ExecExtras ex;
    ex.conj_counts = counts;
    if (d) {
      d->labelled = true;
      if (!out[0].data) alloc_batch_outputs(out, n, s);  // a queue with outputs made per batch
      label_->enqueue_filter(cols, out, d->hdr_dev, d->status, &ex, s);
    } else {
      check_cuda(cudaMemsetAsync(dcounts_, 0, 8 * 16, s), "counts zero");
      ex.conj_counts_host = hcounts_;  // read back with the pass's own readback
      label_->execute(cols, out, out_rows, s, &ex);  // synchronises the stream
    }
    bi.path = 0;
    if (n > 0) {
      const float* feat = nullptr;
      if (d && d->feat) {
        if (qsketch_pending_) {
          check_cuda(cudaStreamWaitEvent(s, qsketch_done_, 0), "wait queue sketch");
          qsketch_pending_ = false;
        }
        feat = d->feat;
      } else {
        int fs = take_prepared(cols, s);
        if (fs < 0) {
          sketch(cols, false, s, 0);
          fs = 0;
        }
        feat = slots_[fs].feat;
      }
      if (!d)
        for (int o = 0; o < nconj_; o++) bi.measured_sel[o] = (double)hcounts_[o] / (double)n;
      add_example(counts, n, s, feat);
      labelled_++;
      train(opt_.train_steps, s);
      if (!train_stream_) {
        check_cuda(cudaStreamSynchronize(s), "training sync");
        loss_ = hpinned_[16];
      }
    }
    poll_training();
    bi.train_loss = loss_;
    bi.rows = out_rows ? *out_rows : 0;
    if (info) *info = bi;
    return;
  }
  since_label_++;
  if (!opt_.size_outputs) {
    // order decided on the device: no host round trip before the filter
    ExecExtras ex;
    int ps = -1;
    if (d && d->pred_ready) {
      check_cuda(cudaStreamWaitEvent(s, d->pred_ready, 0), "wait prediction");
      ex.order_dev = d->order_dev;
    } else {
      ps = take_prepared(cols, s);
      if (ps < 0) {
        sync_inference_params(s);
        sketch(cols, true, s, 0, d ? d->report_dev : nullptr, d ? d->report : nullptr);
        ps = 0;
      }
      ex.order_dev = slots_[ps].order;
    }
    if (d) fast_->enqueue_filter(cols, out, d->hdr_dev, d->status, &ex, s);
    else fast_->execute(cols, out, out_rows, s, &ex);  // synchronises the stream
    if (!d) {
      // the sketch kernel (ordered before the filter) left its prediction in
      // a mapped host report
      const float* rz = slots_[ps].cur_report;
      const int* rorder = reinterpret_cast<const int*>(rz + 16);
      for (int o = 0; o < O_; o++) {
        const float z = rz[o];
        bi.predicted_sel[o] = std::exp(-(std::max(-z, 0.f) + std::log1p(std::exp(-std::fabs(z)))));
        bi.order[o] = rorder[o];
      }
    }
    poll_training();
    bi.train_loss = loss_;
    bi.path = 1;
    bi.rows = out_rows ? *out_rows : 0;
    if (info) *info = bi;
    return;
  }
  if (d) {
    // queued: the prediction was made on the side stream while the previous
    // batch ran; the host reads it (mapped report), sizes the outputs and puts
    // the filter on the stream without waiting for the device
    if (!d->pred_ready) fail(GX_ERR_INVALID, "queued batch without a prediction");
    check_cuda(cudaEventSynchronize(d->pred_ready), "prediction wait");
    double log_all = 0.0;
    for (int o = 0; o < O_; o++) {
      const float z = d->report[o];
      log_all += -(std::max(-z, 0.f) + std::log1p(std::exp(-std::fabs(z))));  // log sigmoid(z)
    }
    const double pred_rows = (double)n * std::exp(std::min(0.0, log_all));
    d->pred_rows = (int64_t)pred_rows;
    d->capacity =
        (int64_t)std::min<double>((double)n, pred_rows * opt_.capacity_margin + (double)opt_.capacity_slack);
    alloc_batch_outputs(out, d->capacity, s);
    check_cuda(cudaStreamWaitEvent(s, d->pred_ready, 0), "wait prediction");
    ExecExtras ex;
    ex.order_dev = d->order_dev;
    fast_->enqueue_filter(cols, out, d->hdr_dev, d->status, &ex, s);
    poll_training();
    bi.train_loss = loss_;
    bi.path = 1;
    if (info) *info = bi;
    return;
  }
  const std::vector<float> ls = predict_log_sel(cols, s);
  poll_training();
  // order by rank = cost / (1 - selectivity): cheap conjuncts that remove most rows first
  std::vector<int> order(nconj_);
  std::iota(order.begin(), order.end(), 0);
  std::vector<double> rank(nconj_);
  double log_all = 0.0;
  for (int o = 0; o < nconj_; o++) {
    const double sel = std::exp((double)ls[o]);
    bi.predicted_sel[o] = sel;
    rank[o] = conj_cost_[o] / std::max(1e-9, 1.0 - sel);
    log_all += ls[o];
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rank[a] < rank[b]; });
  for (int o = 0; o < nconj_; o++) bi.order[o] = order[o];
  // output capacity from the prediction (conjuncts taken as independent), with margin
  const double pred_rows = (double)n * std::exp(std::min(0.0, log_all));
  bi.predicted_rows = (int64_t)pred_rows;
  ExecExtras ex;
  ex.order = order.data();
  ex.num_order = nconj_;
  ex.capacity_hint =
      (int64_t)std::min<double>((double)n, pred_rows * opt_.capacity_margin + (double)opt_.capacity_slack);
  const bool caller_bufs = out[0].data != nullptr;
  try {
    fast_->execute(cols, out, out_rows, s, &ex);
  } catch (const Error& e) {
    if (e.code != GX_ERR_CAPACITY || caller_bufs || !out_rows) throw;
    // misprediction: the outputs were released; re-run with the exact row count
    bi.reruns = 1;
    ex.capacity_hint = *out_rows;
    for (int j = 0; j < num_outputs(); j++) out[j] = gx_column{};
    fast_->execute(cols, out, out_rows, s, &ex);
  }
  bi.train_loss = loss_;
  bi.path = 1;
  bi.rows = out_rows ? *out_rows : 0;
  if (info) *info = bi;
}

// Host side of a deferred batch: the row count, the labels or the prediction,
// all read after the queue's one synchronisation.
void Learner::alloc_batch_outputs(gx_column* out, int64_t capacity, cudaStream_t s) const {
  std::vector<int> types;
  for (const auto& o : fast_->plan().outputs) types.push_back(o.type);
  alloc_output_set(types, std::vector<int64_t>(types.size(), capacity), true, out, s);
}

bool Learner::finish_one(const Deferred& d, int64_t n, gx_column* out, int64_t* out_rows,
                         gx_learned_batch_info* info) {
  const CompiledPlan& ran = d.labelled ? *label_ : *fast_;
  if (info && d.pred_rows >= 0) info->predicted_rows = d.pred_rows;
  // (a kernel error word is raised by finish_queued below)
  if (!d.labelled && d.capacity >= 0 && n > 0 && d.hdr[2] == 0 && (int64_t)d.hdr[1] > d.capacity) {
    if (out_rows) *out_rows = (int64_t)d.hdr[1];
    return false;
  }
  int64_t rows = 0;
  ran.finish_queued(d.hdr, n, out, &rows);
  if (out_rows) *out_rows = rows;
  if (!info) return true;
  info->rows = rows;
  if (d.labelled && n > 0)
    for (int o = 0; o < nconj_; o++) info->measured_sel[o] = (double)d.hdr[4 + o] / (double)n;
  if (!d.labelled && opt_.policy == GX_LEARN_POLICY_LEARNED) {
    const int* rorder = reinterpret_cast<const int*>(d.report + 16);
    for (int o = 0; o < O_; o++) {
      const float z = d.report[o];
      info->predicted_sel[o] = std::exp(-(std::max(-z, 0.f) + std::log1p(std::exp(-std::fabs(z)))));
      info->order[o] = rorder[o];
    }
  }
  return true;
}

bool Learner::can_defer() const {
  const bool single_pass = opt_.policy == GX_LEARN_POLICY_TEXTUAL || opt_.policy == GX_LEARN_POLICY_LEARNED;
  return single_pass && fast_->can_defer() && label_->can_defer();
}

constexpr int kQueueParts = 16;  // sketch blocks per column of a queued batch
constexpr size_t kQueueDepth = 4;  // batches of a queue the host runs ahead of the device
constexpr size_t kHostSlot = kQueueHeaderBytes + 128;  // per batch: header copy + mapped report

Learner::QueueSketchLayout Learner::queue_sketch_layout(size_t nb) const {
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  QueueSketchLayout q;
  q.o_n = al(nb * sizeof(SketchCols));
  q.o_tk = q.o_n + al(nb * 8);
  q.o_part = q.o_tk + al(nb * 4);
  q.o_feat = q.o_part + al(nb * (size_t)ncols_ * kQueueParts * kPartial * 4);
  q.total = q.o_feat + al(nb * (size_t)F_ * 4);
  return q;
}

void Learner::reserve_queue(size_t nb) {
  if (nb == 0) return;
  if (queue_cap_ < nb) {
    if (hqueue_) cudaFreeHost(hqueue_);
    hqueue_ = nullptr;
    queue_cap_ = 0;
    check_cuda(cudaHostAlloc((void**)&hqueue_, nb * kHostSlot, cudaHostAllocMapped | cudaHostAllocPortable),
               "pinned queue slots");
    queue_cap_ = nb;
  }
  for (int q = 0; q < 8; q++)
    if (!qdone_[q]) check_cuda(cudaEventCreateWithFlags(&qdone_[q], cudaEventDisableTiming), "event");
  if (opt_.policy == GX_LEARN_POLICY_LEARNED && qsk_cap_ < nb) {
    const QueueSketchLayout q = queue_sketch_layout(nb);
    cudaFree(dqsk_);
    if (hqsk_) cudaFreeHost(hqsk_);
    dqsk_ = hqsk_ = nullptr;
    qsk_cap_ = 0;
    dqsk_ = (char*)must_alloc(q.total);
    check_cuda(cudaMallocHost((void**)&hqsk_, q.o_part), "pinned sketch descriptors");
    qsk_cap_ = nb;
  }
}

void Learner::sketch_queue(const std::vector<std::vector<ColumnView>>& batches, std::vector<Deferred>& d,
                           cudaStream_t s) {
  const size_t nb = batches.size();
  reserve_queue(nb);
  const QueueSketchLayout q = queue_sketch_layout(nb);
  const size_t o_n = q.o_n, o_tk = q.o_tk, o_part = q.o_part, o_feat = q.o_feat;
  // the previous queue's upload has been consumed: its queue synchronised
  std::memset(hqsk_, 0, o_part);
  auto* desc = (SketchCols*)hqsk_;
  auto* rows = (int64_t*)(hqsk_ + o_n);
  for (size_t b = 0; b < nb; b++) {
    const auto& cols = batches[b];
    for (int i = 0; i < ncols_; i++) {
      desc[b].data[i] = type_size(cols[i].type) == 0 ? nullptr : cols[i].data;
      desc[b].mask[i] = cols[i].mask;
      desc[b].off[i] = cols[i].offset;
      desc[b].type[i] = cols[i].type;
      desc[b].anchor[i] = anchors_[i];
    }
    rows[b] = cols.empty() ? 0 : cols[0].size;
    d[b].feat = (const float*)(dqsk_ + o_feat) + b * (size_t)F_;
  }
  check_cuda(cudaMemcpyAsync(dqsk_, hqsk_, o_part, cudaMemcpyHostToDevice, s), "sketch descriptors");
  // the side stream starts once the main stream has the descriptors (and the
  // caller's columns are ready)
  check_cuda(cudaEventRecord(prep_in_, s), "queue event");
  check_cuda(cudaStreamWaitEvent(aux_stream_, prep_in_, 0), "wait queue");
  k_sketch_queue<<<dim3(kQueueParts, ncols_, (unsigned)nb), 256, 0, aux_stream_>>>(
      (const SketchCols*)dqsk_, (const int64_t*)(dqsk_ + o_n), opt_.stride_words, ncols_, (float*)(dqsk_ + o_part),
      (unsigned int*)(dqsk_ + o_tk), (float*)(dqsk_ + o_feat));
  check_cuda(cudaGetLastError(), "k_sketch_queue");
  add_launches(1);
  check_cuda(cudaEventRecord(qsketch_done_, aux_stream_), "queue sketch event");
  qsketch_pending_ = true;
}

void Learner::predict_queued(Deferred& d, int ev, cudaStream_t) {
  sync_inference_params(aux_stream_);
  k_predict<<<1, 256, 0, aux_stream_>>>(d.feat, F_, dinfer_, H_, O_, dcost_, d.order_dev, d.report_dev);
  check_cuda(cudaGetLastError(), "k_predict");
  add_launches(1);
  check_cuda(cudaEventRecord(qev_[ev], aux_stream_), "prediction event");
  d.pred_ready = qev_[ev];
}

void Learner::execute_batches(const std::vector<std::vector<ColumnView>>& batches, gx_column* out,
                              int64_t* out_rows, gx_learned_batch_info* infos, cudaStream_t s) {
  const size_t nb = batches.size();
  const int nout = num_outputs();
  const auto& schema = plain_->plan().schema;
  for (size_t b = 0; b < nb; b++) {
    bool ok = batches[b].size() == schema.size();
    for (size_t i = 0; ok && i < schema.size(); i++) ok = batches[b][i].type == schema[i];
    if (!ok) fail(GX_ERR_INVALID, "batch " + std::to_string(b) + ": columns do not match the plan");
  }
  if (out_rows)
    for (size_t b = 0; b < nb; b++) out_rows[b] = -1;  // set as each batch completes
  auto rows_of = [&](size_t b) { return batches[b].empty() ? (int64_t)0 : batches[b][0].size; };
  if (!can_defer()) {
    // every batch completes before the next starts (the plain policy)
    size_t at = 0;  // the batch being prepared or executed
    try {
      if (nb > 0) prepare(batches[0], s);
      for (size_t b = 0; b < nb; b++) {
        if (b + 1 < nb) {
          at = b + 1;
          prepare(batches[b + 1], s);
        }
        at = b;
        execute_one(batches[b], out + b * nout, out_rows ? out_rows + b : nullptr, infos ? infos + b : nullptr, s,
                    nullptr);
      }
    } catch (const Error& e) {
      fail(e.code, "batch " + std::to_string(at) + ": " + e.what());
    }
    return;
  }
  // Queued: every batch's outputs, masks, tile statuses and headers come from
  // one allocation cleared by one memset, and each batch puts only its
  // kernels on the stream (no host round trip); one copy of all headers and
  // one synchronisation complete the queue.  With outputs sized from the
  // predictions, the headers and statuses are one allocation and each batch's
  // outputs are allocated when its prediction is read (the side stream makes
  // it while the previous batch runs); a batch whose rows overflow its
  // prediction runs again after the queue with the exact row count.
  if (nb == 0) return;
  const bool sized = opt_.policy == GX_LEARN_POLICY_LEARNED && opt_.size_outputs;
  reserve_queue(nb);
  std::memset(hqueue_, 0, queue_cap_ * kHostSlot);
  char* dqueue = nullptr;
  check_cuda(cudaHostGetDevicePointer((void**)&dqueue, hqueue_, 0), "mapped queue slots");
  std::vector<int> types;
  for (const auto& o : fast_->plan().outputs) types.push_back(o.type);
  std::vector<int64_t> caps(nb), status_words(nb);
  for (size_t b = 0; b < nb; b++) {
    caps[b] = rows_of(b);
    status_words[b] = std::max(fast_->tiles_for(caps[b]), label_->tiles_for(caps[b]));
  }
  std::vector<uint64_t*> status(nb);
  char* base = nullptr;
  if (sized) {
    base = (char*)alloc_queue_scratch(status_words, status.data(), s);
    for (size_t c = 0; c < nb * (size_t)nout; c++) out[c] = gx_column{};
  } else {
    base = (char*)alloc_output_queue(types, caps, status_words, out, status.data(), s);
  }
  std::vector<Deferred> d(nb);
  const size_t rep0 = queue_cap_ * kQueueHeaderBytes;
  for (size_t b = 0; b < nb; b++) {
    d[b].hdr_dev = (unsigned long long*)(base + b * kQueueHeaderBytes);
    d[b].status = status[b];
    d[b].hdr = (const unsigned long long*)(hqueue_ + b * kQueueHeaderBytes);
    d[b].report = (float*)(hqueue_ + rep0 + b * 128);
    d[b].report_dev = (float*)(dqueue + rep0 + b * 128);
    d[b].order_dev = (int*)(d[b].hdr_dev + 20);
  }
  const bool learned = opt_.policy == GX_LEARN_POLICY_LEARNED;
  std::vector<gx_learned_batch_info> local(infos ? 0 : nb);
  gx_learned_batch_info* inf = infos ? infos : local.data();
  size_t at = 0;
  size_t enqueued = 0;  // batches whose work is on the stream
  std::string err;
  int code = GX_OK;
  try {
    // every batch's sketch in one launch; each batch's prediction kPredAhead
    // batches ahead on the side stream, so that the one-block prediction
    // kernel never sits between two filters (it runs beside them)
    if (learned) {
      sketch_queue(batches, d, s);
      for (size_t b = 0; b < std::min<size_t>(nb, kPredAhead); b++)
        if (rows_of(b) > 0) predict_queued(d[b], (int)(b % kPredEvents), s);
    }
    for (size_t b = 0; b < nb; b++) {
      // at most kQueueDepth batches ahead of the device: the host then sees
      // training rounds finish while the queue runs, and later predictions
      // use their parameters (the device never waits for the host)
      if (b >= kQueueDepth)
        check_cuda(cudaEventSynchronize(qdone_[(b - kQueueDepth) % 8]), "queue pacing");
      const size_t pb = b + kPredAhead;
      if (learned && pb < nb && rows_of(pb) > 0) {
        at = pb;
        predict_queued(d[pb], (int)(pb % kPredEvents), s);
      }
      at = b;
      execute_one(batches[b], out + b * nout, nullptr, inf + b, s, &d[b]);
      check_cuda(cudaEventRecord(qdone_[b % 8], s), "batch event");
      enqueued = b + 1;
    }
  } catch (const Error& e) {
    code = e.code;
    err = e.what();
  }
  // batches that never ran release their outputs (the allocation goes with the last column)
  for (size_t c = enqueued; c < nb; c++)
    for (int j = 0; j < nout; j++) {
      free_column(out[c * nout + j], s);
      out[c * nout + j] = gx_column{};
    }
  cudaError_t se = cudaSuccess;
  if (enqueued > 0) se = cudaMemcpyAsync(hqueue_, base, enqueued * kQueueHeaderBytes, cudaMemcpyDeviceToHost, s);
  if (se == cudaSuccess) se = cudaStreamSynchronize(s);
  if (se != cudaSuccess) {
    if (code == GX_OK) {
      code = GX_ERR_CUDA;
      err = std::string("queue completion: ") + cudaGetErrorString(se);
      at = 0;
    }
    // no batch is known to have completed
    for (size_t c = 0; c < enqueued; c++)
      for (int j = 0; j < nout; j++) {
        free_column(out[c * nout + j], s);
        out[c * nout + j] = gx_column{};
      }
    enqueued = 0;
  }
  for (size_t b = 0; b < enqueued; b++) {
    try {
      int64_t rows = 0;
      if (!finish_one(d[b], rows_of(b), out + b * nout, &rows, inf + b)) {
        // misprediction: the batch runs again into outputs of its exact row count
        for (int j = 0; j < nout; j++) {
          free_column(out[b * nout + j], s);
          out[b * nout + j] = gx_column{};
        }
        ExecExtras ex;
        std::vector<int> order(nconj_);
        const int* rorder = reinterpret_cast<const int*>(d[b].report + 16);
        for (int o = 0; o < nconj_; o++) order[o] = rorder[o];
        ex.order = order.data();
        ex.num_order = nconj_;
        ex.capacity_hint = rows;
        fast_->execute(batches[b], out + b * nout, &rows, s, &ex);
        inf[b].reruns = 1;
        inf[b].rows = rows;
      }
      if (out_rows) out_rows[b] = rows;
    } catch (const Error& e) {
      if (code == GX_OK) {
        code = e.code;
        err = e.what();
        at = b;
      }
      // this batch and the later ones do not complete
      for (size_t c = b; c < enqueued; c++) {
        for (int j = 0; j < nout; j++) {
          free_column(out[c * nout + j], s);
          out[c * nout + j] = gx_column{};
        }
        if (out_rows) out_rows[c] = -1;
      }
      break;
    }
  }
  if (qsketch_pending_) {
    // no labelled batch waited for the queue sketch: the next queue's upload
    // must not overwrite its descriptors while it runs
    check_cuda(cudaStreamWaitEvent(s, qsketch_done_, 0), "wait queue sketch");
    qsketch_pending_ = false;
  }

  if (sized) dev_free(base, s);  // headers and statuses (the outputs are the columns')
  poll_training();
  if (code != GX_OK) fail((gx_status)code, "batch " + std::to_string(at) + ": " + err);
}

void Learner::save(const std::string& path) const {
  if (!dparams_) fail(GX_ERR_INVALID, "this learner has no network (policy is not LEARNED)");
  if (train_stream_) check_cuda(cudaStreamSynchronize(train_stream_), "training sync");
  std::vector<float> p(nparams_);
  check_cuda(cudaMemcpy(p.data(), dparams_, (size_t)nparams_ * 4, cudaMemcpyDeviceToHost), "save params");
  std::ofstream f(path, std::ios::binary);
  // header, the sketch anchors the features were computed against, the parameters
  const int32_t hdr[6] = {0x47584D4C /* "GXML" */, 3, F_, H_, O_, ncols_};
  f.write((const char*)hdr, sizeof hdr);
  f.write((const char*)anchors_.data(), (std::streamsize)anchors_.size() * 8);
  f.write((const char*)p.data(), (std::streamsize)p.size() * 4);
  if (!f) fail(GX_ERR_INVALID, "cannot write " + path);
}

void Learner::load(const std::string& path) {
  if (!dparams_) fail(GX_ERR_INVALID, "this learner has no network (policy is not LEARNED)");
  std::ifstream f(path, std::ios::binary);
  int32_t hdr[6] = {0};
  f.read((char*)hdr, sizeof hdr);
  if (!f || hdr[0] != 0x47584D4C || hdr[1] != 3 || hdr[2] != F_ || hdr[3] != H_ || hdr[4] != O_ || hdr[5] != ncols_)
    fail(GX_ERR_INVALID, "model file does not match this plan: " + path);
  std::vector<double> anchors(ncols_);
  std::vector<float> p(nparams_);
  f.read((char*)anchors.data(), (std::streamsize)anchors.size() * 8);
  f.read((char*)p.data(), (std::streamsize)p.size() * 4);
  if (f && anchors != anchors_) fail(GX_ERR_INVALID, "model file was trained for other comparison constants: " + path);
  if (!f) fail(GX_ERR_INVALID, "truncated model file: " + path);
  if (train_stream_) check_cuda(cudaStreamSynchronize(train_stream_), "training sync");
  check_cuda(cudaMemcpy(dparams_, p.data(), (size_t)nparams_ * 4, cudaMemcpyHostToDevice), "load params");
  check_cuda(cudaMemcpy(dinfer_, p.data(), (size_t)nparams_ * 4, cudaMemcpyHostToDevice), "load params");
  params_pending_ = false;
  // a loaded network is used at once
  labelled_ = std::max<uint64_t>(labelled_, (uint64_t)opt_.warmup_batches);
}

}  // namespace gx

// ------------------------------------------------------------------ C ABI
struct gx_learner {
  std::unique_ptr<gx::Learner> l;
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

void gx_learner_options_init(gx_learner_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  const gx::LearnerOptions d;
  o->policy = d.policy;
  o->warmup_batches = d.warmup_batches;
  o->relabel_every = d.relabel_every;
  o->train_steps = d.train_steps;
  o->learning_rate = d.lr;
  o->hidden = d.hidden;
  o->capacity_margin = d.capacity_margin;
  o->capacity_slack = d.capacity_slack;
  o->sketch_stride_words = d.stride_words;
  o->async_training = d.async_training ? 1 : 0;
  o->seed = d.seed;
  o->fast_words_per_warp = d.fast_words;
  o->size_outputs = d.size_outputs ? 1 : 0;
}

gx_learner* gx_learner_create(const gx_plan* plan, const gx_learner_options* options, gx_status_info* status) {
  gx_learner* out = nullptr;
  guarded_call(status, [&] {
    const gx::CompiledPlan* cp = gx::single_chunk(plan);
    if (!cp) gx::fail(GX_ERR_INVALID, "a learner needs a compiled plan with at most 32 outputs "
                                      "over at most 64 columns");
    gx_learner_options o;
    gx_learner_options_init(&o);
    if (options) o = *options;
    gx::LearnerOptions lo;
    lo.policy = o.policy;
    lo.warmup_batches = std::max(1, o.warmup_batches);
    lo.relabel_every = std::max(0, o.relabel_every);
    lo.train_steps = std::max(0, o.train_steps);
    lo.lr = o.learning_rate > 0.f ? o.learning_rate : 3e-3f;
    lo.hidden = o.hidden > 0 ? o.hidden : 64;
    lo.capacity_margin = o.capacity_margin >= 1.0 ? o.capacity_margin : 1.0;
    lo.capacity_slack = std::max<int64_t>(0, o.capacity_slack);
    lo.stride_words = o.sketch_stride_words > 0 ? o.sketch_stride_words : 256;
    lo.async_training = o.async_training != 0;
    lo.seed = o.seed;
    lo.fast_words = o.fast_words_per_warp > 0 ? std::min(o.fast_words_per_warp, 32) : 0;
    lo.size_outputs = o.size_outputs != 0;
    out = new gx_learner{std::make_unique<gx::Learner>(*cp, lo)};
  });
  return out;
}

int gx_learner_execute(gx_learner* learner, const gx_column_view* columns, int num_columns, gx_column* out,
                       int64_t* out_rows, gx_learned_batch_info* info, void* stream, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!learner || !out || (num_columns > 0 && !columns)) gx::fail(GX_ERR_INVALID, "null argument");
    learner->l->execute(gx::to_views(columns, num_columns), out, out_rows, info, (cudaStream_t)stream);
  });
}

int gx_learner_execute_batches(gx_learner* learner, const gx_column_view* const* batches, int num_columns,
                               int num_batches, gx_column* out, int64_t* out_rows, gx_learned_batch_info* infos,
                               void* stream, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!learner || num_batches < 0 || (num_batches > 0 && (!batches || !out)))
      gx::fail(GX_ERR_INVALID, "null argument");
    std::vector<std::vector<gx::ColumnView>> b(num_batches);
    for (int i = 0; i < num_batches; i++) {
      if (num_columns > 0 && !batches[i]) gx::fail(GX_ERR_INVALID, "null batch");
      b[i] = gx::to_views(batches[i], num_columns);
    }
    learner->l->execute_batches(b, out, out_rows, infos, (cudaStream_t)stream);
  });
}

int gx_learner_prepare(gx_learner* learner, const gx_column_view* columns, int num_columns, void* stream,
                       gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!learner || (num_columns > 0 && !columns)) gx::fail(GX_ERR_INVALID, "null argument");
    learner->l->prepare(gx::to_views(columns, num_columns), (cudaStream_t)stream);
  });
}

int gx_learner_save(const gx_learner* learner, const char* path, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!learner || !path) gx::fail(GX_ERR_INVALID, "null argument");
    learner->l->save(path);
  });
}

int gx_learner_load(gx_learner* learner, const char* path, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!learner || !path) gx::fail(GX_ERR_INVALID, "null argument");
    learner->l->load(path);
  });
}

void gx_learner_destroy(gx_learner* learner) { delete learner; }

int gx_debug_learner_features(gx_learner* learner, const gx_column_view* columns, int num_columns, float* features,
                              int max_features, int* num_features, double* anchors, void* stream,
                              gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!learner || !features || (num_columns > 0 && !columns)) gx::fail(GX_ERR_INVALID, "null argument");
    const std::vector<float> f =
        learner->l->features(gx::to_views(columns, num_columns), (cudaStream_t)stream);
    if ((int)f.size() > max_features) gx::fail(GX_ERR_INVALID, "feature buffer too small");
    std::memcpy(features, f.data(), f.size() * 4);
    if (num_features) *num_features = (int)f.size();
    if (anchors) {
      const std::vector<double>& a = learner->l->anchors();
      std::memcpy(anchors, a.data(), a.size() * 8);
    }
  });
}

int gx_debug_mlp_grad(int F, int H, int O, const float* params, const float* X, int M, const float* Y, float* grad,
                      float* loss, float* z, gx_status_info* status) {
  return guarded_call(status, [&] {
    if (!params || !X || !Y || !grad || !loss || !z) gx::fail(GX_ERR_INVALID, "null argument");
    gx::check_mlp_shape(F, H, O, M);
    const size_t np = (size_t)gx::mlp_param_count(F, H, O);
    const size_t floats = np * 2 + (size_t)M * F + (size_t)M * O + 2 * (size_t)M * H + (size_t)M * O + 4;
    float* d = nullptr;
    gx::check_cuda(cudaMalloc(&d, floats * 4), "mlp check buffers");
    float *dP = d, *dG = dP + np, *dX = dG + np, *dY = dX + (size_t)M * F, *dA = dY + (size_t)M * O,
          *dZ = dA + 2 * (size_t)M * H, *dL = dZ + (size_t)M * O;
    try {
      gx::check_cuda(cudaMemcpy(dP, params, np * 4, cudaMemcpyHostToDevice), "params");
      gx::check_cuda(cudaMemcpy(dX, X, (size_t)M * F * 4, cudaMemcpyHostToDevice), "X");
      gx::check_cuda(cudaMemcpy(dY, Y, (size_t)M * O * 4, cudaMemcpyHostToDevice), "Y");
      gx::mlp_grad(dP, F, H, O, dX, M, dY, dG, dL, dA, 0);
      gx::check_cuda(cudaMemcpy(grad, dG, np * 4, cudaMemcpyDeviceToHost), "grad");
      gx::check_cuda(cudaMemcpy(loss, dL, 4, cudaMemcpyDeviceToHost), "loss");
      gx::check_cuda(cudaMemcpy(z, dZ, (size_t)M * O * 4, cudaMemcpyDeviceToHost), "z");
    } catch (...) {
      cudaFree(d);
      throw;
    }
    cudaFree(d);
  });
}

}  // extern "C"
