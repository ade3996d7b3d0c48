// Learned query-vertex ordering: features, cost-model inference and training.
//
// No reference counterpart (the reference only ever searches in query-index
// order, isomorphism.hpp:414-448).  The cost model is a 12-64-64-1 ReLU MLP with
// bfloat16 weights and fp32 accumulation that predicts a query vertex's
// root-level search-tree size: log2 of the mean number of DFS assignments it
// receives per pair when the search starts at it.
// The order only permutes the search; EXACT counts do not depend on it.
#include <cuda_bf16.h>

#include "device_common.cuh"

namespace bms {
namespace {

unsigned grid_for(uint64_t work, unsigned threads, unsigned per_sm = 8) {
  uint64_t want = (work + threads - 1) / threads;
  uint64_t cap = uint64_t(sm_count()) * per_sm;
  if (want < 1) want = 1;
  return unsigned(want < cap ? want : cap);
}

// parameter layout
constexpr int oW1 = 0, oB1 = 768, oW2 = 832, oB2 = 4928, oW3 = 4992, oB3 = 5056;
static_assert(oB3 + 1 == kParams, "parameter layout");

__device__ __forceinline__ float bf16_to_f(uint16_t h) { return __bfloat162float(__ushort_as_bfloat16(h)); }

// ------------------------------------------------------------------ features
__global__ void record_stats_kernel(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, DGraphs q,
                                    const uint64_t* arena, unsigned int* per_query, unsigned int* cand_sum) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  // a deterministic sample: records of every s-th data graph (all when n is small)
  const uint32_t s = 1u + uint32_t(n >> 19);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const PairRec r = recs[i];
    if (r.d % s) continue;
    atomicAdd(&per_query[r.q], 1u);
    const uint32_t qoff = q.goff[r.q], nq = q.goff[r.q + 1] - qoff;
    for (uint32_t u = 0; u < nq; ++u) atomicAdd(&cand_sum[qoff + u], b_pop(ld_b128(arena + 2 * (uint64_t(r.c_row) + u))));
  }
}

__global__ void features_kernel(DFeatureArgs a) {
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < a.q.N; u += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t qg = graph_of(a.q.goff, a.q.G, uint32_t(u));
    const uint32_t qoff = a.q.goff[qg], n = a.q.goff[qg + 1] - qoff;
    const uint64_t* rec = a.qs.frec + uint64_t(kRecWords) * u;
    const uint32_t l = uint32_t(rec[0] & 0xFFu), deg = uint32_t(rec[0] >> 32);
    const uint64_t cyc = rec[1];
    const uint32_t c5 = uint32_t(cyc & 0xFFFFu) + uint32_t((cyc >> 16) & 0xFFFFu);
    const uint32_t c6 = uint32_t((cyc >> 32) & 0xFFFFu) + uint32_t((cyc >> 48) & 0xFFFFu);
    const uint32_t pbits = __popcll(rec[2]) + __popcll(rec[3]) + __popcll(rec[4]) + __popcll(rec[5]);
    const uint64_t nb = a.qs.adj[2 * u];
    const uint32_t ul = uint32_t(u) - qoff;
    uint32_t same_q = 0, same_nb = 0, nb_deg = 0;
    uint64_t reach = (uint64_t(1) << ul) | nb;
    for (uint32_t i = 0; i < n; ++i) {
      const uint64_t w0 = a.qs.frec[uint64_t(kRecWords) * (qoff + i)];
      const bool same = uint32_t(w0 & 0xFFu) == l;
      same_q += same;
      if ((nb >> i) & 1ull) {
        same_nb += same;
        nb_deg += uint32_t(w0 >> 32);
        reach |= a.qs.adj[2 * (uint64_t(qoff) + i)];
      }
    }
    const uint32_t recs = a.recs_per_query[qg];
    const float mean_c = recs ? float(a.cand_sum[u]) / float(recs) : 0.f;
    const float nbc = float(__popcll(nb));
    float* f = a.features + uint64_t(kFeatures) * u;
    f[0] = log2f(1.f + mean_c);
    f[1] = float(deg) * 0.25f;
    f[2] = l == kWildcard ? 1.f : (a.data_nodes ? float(double(a.label_count[l]) / double(a.data_nodes)) : 0.f);
    f[3] = float(same_q) / float(n);
    f[4] = c5 ? 1.f : 0.f;
    f[5] = c6 ? 1.f : 0.f;
    f[6] = log2f(1.f + float(c5 + c6));
    f[7] = float(n) * (1.f / 64.f);
    f[8] = nbc > 0.f ? float(same_nb) / nbc : 0.f;
    f[9] = float(pbits) * (1.f / 256.f);
    f[10] = float(nb_deg) * (1.f / 16.f);
    f[11] = float(__popcll(reach)) / float(n);
  }
}

// ------------------------------------------------------------------ inference
__global__ void mlp_predict_kernel(const float* x, uint64_t n, const uint16_t* wbf, float* cost) {
  __shared__ float w[kParams];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = bf16_to_f(wbf[i]);
  __syncthreads();
  for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < n; s += uint64_t(gridDim.x) * blockDim.x) {
    float xi[kFeatures];
#pragma unroll
    for (int i = 0; i < kFeatures; ++i) xi[i] = x[uint64_t(kFeatures) * s + i];
    float h1[kHidden];
#pragma unroll 8
    for (int j = 0; j < kHidden; ++j) {
      float acc = w[oB1 + j];
#pragma unroll
      for (int i = 0; i < kFeatures; ++i) acc = fmaf(w[oW1 + j * kFeatures + i], xi[i], acc);
      h1[j] = fmaxf(acc, 0.f);
    }
    float out = w[oB3];
    for (int j = 0; j < kHidden; ++j) {
      float acc = w[oB2 + j];
#pragma unroll
      for (int i = 0; i < kHidden; ++i) acc = fmaf(w[oW2 + j * kHidden + i], h1[i], acc);
      out = fmaf(w[oW3 + j], fmaxf(acc, 0.f), out);
    }
    cost[s] = out;
  }
}

// Greedy connected order per query: the root is the vertex of lowest predicted
// cost; each next vertex is the frontier vertex (adjacent to the placed set,
// any vertex if none is) minimising cost - (number of placed neighbours).
__global__ void learned_order_kernel(DGraphs q, DSigs qs, const float* cost, DOrder o) {
  for (uint32_t qg = blockIdx.x * blockDim.x + threadIdx.x; qg < q.G; qg += gridDim.x * blockDim.x) {
    const uint32_t qoff = q.goff[qg], n = q.goff[qg + 1] - qoff;
    uint8_t* perm = o.perm + uint64_t(qg) * kMaxQueryNodes;
    uint64_t placed = 0, frontier = 0;
    for (uint32_t t = 0; t < n; ++t) {
      const uint64_t all = n >= 64 ? ~0ull : ((uint64_t(1) << n) - 1);
      uint64_t pool = frontier & ~placed;
      if (!pool) pool = all & ~placed;
      float best = 3.0e38f;
      uint32_t pick = 0;
      for (uint64_t p = pool; p; p &= p - 1) {
        const uint32_t v = uint32_t(__ffsll((long long)p) - 1);
        const uint64_t row = qs.adj[2 * (uint64_t(qoff) + v)];
        const float score = cost[qoff + v] - float(__popcll(row & placed));
        if (score < best) {
          best = score;
          pick = v;
        }
      }
      perm[t] = uint8_t(pick);
      placed |= uint64_t(1) << pick;
      frontier |= qs.adj[2 * (uint64_t(qoff) + pick)];
    }
  }
}

// ------------------------------------------------------------------ training
constexpr int kSamplesPerBlock = 32;

__global__ void __launch_bounds__(256) mlp_grad_kernel(const float* x, const float* y, uint32_t n, uint32_t n_total,
                                                       const uint16_t* wbf, float* grad_partial, float* pred,
                                                       float* loss_partial) {
  __shared__ float w[kParams];
  __shared__ float X[kSamplesPerBlock][kFeatures];
  __shared__ float H1[kSamplesPerBlock][kHidden];
  __shared__ float H2[kSamplesPerBlock][kHidden];
  __shared__ float dy[kSamplesPerBlock];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = bf16_to_f(wbf[i]);
  const uint32_t s0 = blockIdx.x * kSamplesPerBlock;
  for (int i = threadIdx.x; i < kSamplesPerBlock * kFeatures; i += blockDim.x) {
    const uint32_t s = s0 + i / kFeatures;
    X[i / kFeatures][i % kFeatures] = s < n ? x[uint64_t(s) * kFeatures + i % kFeatures] : 0.f;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kSamplesPerBlock * kHidden; k += blockDim.x) {
    const int s = k / kHidden, j = k % kHidden;
    float acc = w[oB1 + j];
    for (int i = 0; i < kFeatures; ++i) acc = fmaf(w[oW1 + j * kFeatures + i], X[s][i], acc);
    H1[s][j] = fmaxf(acc, 0.f);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kSamplesPerBlock * kHidden; k += blockDim.x) {
    const int s = k / kHidden, j = k % kHidden;
    float acc = w[oB2 + j];
    for (int i = 0; i < kHidden; ++i) acc = fmaf(w[oW2 + j * kHidden + i], H1[s][i], acc);
    H2[s][j] = fmaxf(acc, 0.f);
  }
  __syncthreads();
  if (threadIdx.x < kSamplesPerBlock) {
    const int s = threadIdx.x;
    float o = w[oB3];
    for (int j = 0; j < kHidden; ++j) o = fmaf(w[oW3 + j], H2[s][j], o);
    const bool live = s0 + s < n;
    const float e = live ? o - y[s0 + s] : 0.f;
    if (live && pred) pred[s0 + s] = o;
    dy[s] = 2.f * e / float(n_total);
    float l = e * e;
    for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
    if (s == 0) loss_partial[blockIdx.x] = l;
  }
  __syncthreads();
  float* g = grad_partial + uint64_t(blockIdx.x) * kParams;
  // output layer
  for (int j = threadIdx.x; j < kHidden; j += blockDim.x) {
    float acc = 0.f;
    for (int s = 0; s < kSamplesPerBlock; ++s) acc = fmaf(dy[s], H2[s][j], acc);
    g[oW3 + j] = acc;
  }
  if (threadIdx.x == 0) {
    float acc = 0.f;
    for (int s = 0; s < kSamplesPerBlock; ++s) acc += dy[s];
    g[oB3] = acc;
  }
  __syncthreads();
  // dH2 in place of H2
  for (int k = threadIdx.x; k < kSamplesPerBlock * kHidden; k += blockDim.x) {
    const int s = k / kHidden, j = k % kHidden;
    H2[s][j] = H2[s][j] > 0.f ? dy[s] * w[oW3 + j] : 0.f;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kHidden * kHidden; k += blockDim.x) {
    const int j = k / kHidden, i = k % kHidden;
    float acc = 0.f;
    for (int s = 0; s < kSamplesPerBlock; ++s) acc = fmaf(H2[s][j], H1[s][i], acc);
    g[oW2 + k] = acc;
  }
  for (int j = threadIdx.x; j < kHidden; j += blockDim.x) {
    float acc = 0.f;
    for (int s = 0; s < kSamplesPerBlock; ++s) acc += H2[s][j];
    g[oB2 + j] = acc;
  }
  __syncthreads();
  // dH1 in place of H1
  for (int k = threadIdx.x; k < kSamplesPerBlock * kHidden; k += blockDim.x) {
    const int s = k / kHidden, i = k % kHidden;
    float acc = 0.f;
    for (int j = 0; j < kHidden; ++j) acc = fmaf(H2[s][j], w[oW2 + j * kHidden + i], acc);
    H1[s][i] = H1[s][i] > 0.f ? acc : 0.f;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kHidden * kFeatures; k += blockDim.x) {
    const int j = k / kFeatures, i = k % kFeatures;
    float acc = 0.f;
    for (int s = 0; s < kSamplesPerBlock; ++s) acc = fmaf(H1[s][j], X[s][i], acc);
    g[oW1 + k] = acc;
  }
  for (int j = threadIdx.x; j < kHidden; j += blockDim.x) {
    float acc = 0.f;
    for (int s = 0; s < kSamplesPerBlock; ++s) acc += H1[s][j];
    g[oB1 + j] = acc;
  }
}

__global__ void mlp_reduce_kernel(const float* partial, int blocks, float* grad, const float* loss_partial, float* loss,
                                  uint32_t n) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kParams; p += gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int b = 0; b < blocks; ++b) acc += partial[uint64_t(b) * kParams + p];
    grad[p] = acc;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && loss) {
    float l = 0.f;
    for (int b = 0; b < blocks; ++b) l += loss_partial[b];
    *loss = n ? l / float(n) : 0.f;
  }
}

__global__ void adam_kernel(float* master, uint16_t* wbf, const float* grad, float* m, float* v, float lr, float b1,
                            float b2, float eps, int step) {
  const float c1 = 1.f - powf(b1, float(step)), c2 = 1.f - powf(b2, float(step));
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kParams; p += gridDim.x * blockDim.x) {
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.f - b1) * g;
    const float vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float w = master[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    master[p] = w;
    wbf[p] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
  }
}

__global__ void to_bf16_kernel(const float* master, uint16_t* wbf, int n) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    wbf[p] = __bfloat16_as_ushort(__float2bfloat16_rn(master[p]));
}

}  // namespace

cudaError_t launch_record_stats(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, const DGraphs& q,
                                const uint64_t* arena, unsigned int* per_query, unsigned int* cand_sum,
                                cudaStream_t st) {
  if (rec_cap == 0) return cudaSuccess;
  record_stats_kernel<<<grid_for(rec_cap, 256, 4), 256, 0, st>>>(recs, ctr, rec_cap, q, arena, per_query, cand_sum); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_features(const DFeatureArgs& a, cudaStream_t st) {
  if (a.q.N == 0) return cudaSuccess;
  features_kernel<<<grid_for(a.q.N, 128), 128, 0, st>>>(a); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const float* features, uint64_t n, const uint16_t* wbf16, float* cost, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  mlp_predict_kernel<<<grid_for(n, 128, 2), 128, 0, st>>>(features, n, wbf16, cost); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_learned_order(const DGraphs& q, const DSigs& qs, const float* cost, DOrder o, cudaStream_t st) {
  if (q.G == 0) return cudaSuccess;
  learned_order_kernel<<<grid_for(q.G, 64), 64, 0, st>>>(q, qs, cost, o); note_launch();
  return cudaGetLastError();
}

int mlp_grad_blocks(uint32_t n) { return int((n + kSamplesPerBlock - 1) / kSamplesPerBlock); }

cudaError_t launch_mlp_grad(const float* x, const float* y, uint32_t n, uint32_t n_total, const uint16_t* wbf16,
                            float* grad_partial, float* pred, float* loss_partial, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  mlp_grad_kernel<<<mlp_grad_blocks(n), 256, 0, st>>>(x, y, n, n_total, wbf16, grad_partial, pred, loss_partial); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_mlp_reduce(const float* grad_partial, int blocks, float* grad, const float* loss_partial, float* loss,
                              uint32_t n, cudaStream_t st) {
  mlp_reduce_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(grad_partial, blocks, grad, loss_partial, loss, n); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_adam(float* master, uint16_t* wbf16, const float* grad, float* m, float* v, float lr, float b1,
                        float b2, float eps, int step, cudaStream_t st) {
  adam_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(master, wbf16, grad, m, v, lr, b1, b2, eps, step); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* master, uint16_t* wbf16, int n, cudaStream_t st) {
  to_bf16_kernel<<<(n + 255) / 256, 256, 0, st>>>(master, wbf16, n); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
