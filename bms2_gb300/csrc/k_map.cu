// Mapping and bookkeeping kernels: GMCR offsets and query indices (gmcr.hpp:
// 92-127, with a parallel scan in place of the reference's single-work-item
// prefix sum), query preparation, search orders, task emission, totals, the
// scatter of per-pair results into GMCR order, and the grouping of a data
// batch's graphs by size class at upload.
#include "device_common.cuh"

namespace bms {
namespace {

unsigned grid_for(uint64_t work, unsigned threads, unsigned per_sm = 8) {
  uint64_t want = (work + threads - 1) / threads;
  uint64_t cap = uint64_t(sm_count()) * per_sm;
  if (want < 1) want = 1;
  return unsigned(want < cap ? want : cap);
}

// ------------------------------------------------------------------ labels
__global__ void label_count_kernel(DGraphs d, unsigned long long* counts) {
  __shared__ unsigned int h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < d.N; v += uint64_t(gridDim.x) * blockDim.x)
    atomicAdd(&h[d.lab[v]], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&counts[i], (unsigned long long)h[i]);
}

// One warp per query, lane i owning vertices i and i + 32.
//  - order: the vertex order of the validity test, rarest data label first
//    (wildcards last), then higher degree, then lower index;
//  - dup[v]: the vertex earliest in that order whose filter record (label,
//    degree, cycle, path and the first R shells) equals v's, 0xFF if none or
//    if v is itself the earliest.  Equal records give equal candidate rows.
__global__ void query_prep_kernel(DGraphs q, DSigs qs, const unsigned long long* label_count, uint8_t* order,
                                  uint8_t* dup) {
  const uint32_t lane = lane_id();
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  const int R = qs.R;
  for (uint32_t qg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; qg < q.G; qg += warps) {
    const uint32_t qoff = q.goff[qg], n = q.goff[qg + 1] - qoff;
    unsigned long long key[2];
    uint64_t h[2];
    for (int r = 0; r < 2; ++r) {
      const uint32_t i = lane + 32 * r;
      key[r] = ~0ull;
      h[r] = 0;
      if (i < n) {
        const uint64_t* rec = qs.frec + uint64_t(kRecWords) * (qoff + i);
        const uint64_t w0 = rec[0];
        const uint32_t l = uint32_t(w0 & 0xFFu), deg = uint32_t(w0 >> 32);
        const unsigned long long freq = l == kWildcard ? 0xFFFFFFFFFFull : (label_count[l] & 0xFFFFFFFFFFull);
        const uint32_t dk = 0xFFFFu - (deg > 0xFFFFu ? 0xFFFFu : deg);
        key[r] = (freq << 22) | (uint64_t(dk) << 6) | i;
        uint64_t x = 0x9e3779b97f4a7c15ull;
        for (int w = 0; w < 6 + R; ++w) x = (x ^ rec[w]) * 0x100000001b3ull + (x >> 29);
        h[r] = x;
      }
    }
    // rank of each vertex in the order
    uint32_t rank[2] = {0, 0};
    for (uint32_t j = 0; j < n; ++j) {
      const unsigned long long kj = __shfl_sync(0xffffffffu, key[j >> 5], j & 31);
      for (int r = 0; r < 2; ++r) rank[r] += kj < key[r];
    }
    uint8_t* o = order + uint64_t(qg) * kMaxQueryNodes;
    uint8_t* dd = dup + uint64_t(qg) * kMaxQueryNodes;
    for (int r = 0; r < 2; ++r) {
      const uint32_t i = lane + 32 * r;
      if (i < n) o[rank[r]] = uint8_t(i);
    }
    // duplicate records: earliest-ranked vertex with an equal record
    for (int r = 0; r < 2; ++r) {
      const uint32_t i = lane + 32 * r;
      uint32_t best = 0xFFu, best_rank = rank[r];
      for (uint32_t j = 0; j < n; ++j) {
        const uint64_t hj = __shfl_sync(0xffffffffu, h[j >> 5], j & 31);
        const uint32_t rj = __shfl_sync(0xffffffffu, rank[j >> 5], j & 31);
        if (i < n && j != i && hj == h[r] && rj < best_rank) {
          const uint64_t* a = qs.frec + uint64_t(kRecWords) * (qoff + i);
          const uint64_t* b = qs.frec + uint64_t(kRecWords) * (qoff + j);
          bool same = true;
          for (int w = 0; w < 6 + R && same; ++w) same = a[w] == b[w];
          if (same) {
            best = j;
            best_rank = rj;
          }
        }
      }
      if (i < n) dd[i] = uint8_t(best);
    }
  }
}

// ------------------------------------------------------------------ scan
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint64_t kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* s_warp, uint32_t& total) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= uint32_t(o)) inc += y;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (blockDim.x >> 5) ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= uint32_t(o)) wi += y;
    }
    if (lane < (blockDim.x >> 5)) s_warp[lane] = wi - w;
    if (lane == 31) s_warp[32] = wi;
  }
  __syncthreads();
  const uint32_t r = s_warp[warp] + inc - x;
  total = s_warp[32];
  __syncthreads();
  return r;
}

// out[i] = exclusive prefix within the block chunk; sums[b] = chunk total
__global__ void __launch_bounds__(kScanThreads) scan_chunks(const uint32_t* in, uint32_t* out, uint64_t n,
                                                            uint32_t* sums) {
  __shared__ uint32_t s_warp[33];
  const uint64_t base = uint64_t(blockIdx.x) * kScanBlock + uint64_t(threadIdx.x) * kScanItems;
  uint32_t v[kScanItems];
  uint32_t local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? in[base + i] : 0u;
    local += v[i];
  }
  uint32_t total;
  uint32_t pre = block_exclusive_scan(local, s_warp, total);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_add(uint32_t* out, uint64_t n, const uint32_t* offs) {
  const uint64_t base = uint64_t(blockIdx.x) * kScanBlock;
  const uint32_t add = offs[blockIdx.x];
  for (uint64_t i = base + threadIdx.x; i < base + kScanBlock && i < n; i += blockDim.x) out[i] += add;
}

__global__ void scan_total(const uint32_t* in, const uint32_t* out, uint64_t n, uint32_t* last) {
  *last = n ? out[n - 1] + in[n - 1] : 0u;
}

// ------------------------------------------------------------------ GMCR
__global__ void gmcr_indices_kernel(const uint32_t* valid, uint32_t QW, uint32_t Q, uint32_t D, const uint32_t* offsets,
                                    uint32_t* qidx) {
  for (uint32_t dg = blockIdx.x * blockDim.x + threadIdx.x; dg < D; dg += gridDim.x * blockDim.x) {
    uint32_t pos = offsets[dg];
    const uint32_t* row = valid + uint64_t(dg) * QW;
    for (uint32_t w = 0; w < QW; ++w)
      for (uint32_t bits = row[w]; bits; bits &= bits - 1) qidx[pos++] = w * 32 + uint32_t(__ffs(bits) - 1);
  }
}

__global__ void pair_positions_kernel(PairRec* recs, const Counters* ctr, uint64_t rec_cap, const uint32_t* valid,
                                      uint32_t QW, const uint32_t* offsets) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const PairRec r = recs[i];
    const uint32_t* row = valid + uint64_t(r.d) * QW;
    uint32_t rank = 0;
    for (uint32_t w = 0; w < (r.q >> 5); ++w) rank += __popc(row[w]);
    rank += __popc(row[r.q >> 5] & ((1u << (r.q & 31u)) - 1u));
    recs[i].gpos = offsets[r.d] + rank;
  }
}

// ------------------------------------------------------------------ orders
__global__ void plain_order_kernel(DGraphs q, DOrder o) {
  for (uint32_t qg = blockIdx.x * blockDim.x + threadIdx.x; qg < q.G; qg += gridDim.x * blockDim.x) {
    const uint32_t n = q.goff[qg + 1] - q.goff[qg];
    for (uint32_t t = 0; t < n && t < kMaxQueryNodes; ++t) o.perm[uint64_t(qg) * kMaxQueryNodes + t] = uint8_t(t);
  }
}

// dadj[t] bit i  <=>  perm[i] is in the CSR row of perm[t]
__global__ void order_adjacency_kernel(DGraphs q, DSigs qs, DOrder o) {
  const uint64_t total = uint64_t(q.G) * kMaxQueryNodes;
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < total; k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t qg = uint32_t(k / kMaxQueryNodes), t = uint32_t(k % kMaxQueryNodes);
    const uint32_t qoff = q.goff[qg], n = q.goff[qg + 1] - qoff;
    if (t >= n) continue;
    const uint8_t* perm = o.perm + uint64_t(qg) * kMaxQueryNodes;
    const uint64_t row = qs.adj[2 * (uint64_t(qoff) + perm[t])];  // queries have at most 64 nodes
    uint64_t m = 0;
    for (uint32_t i = 0; i < t; ++i) m |= ((row >> perm[i]) & 1ull) << i;
    o.dadj[k] = m;
  }
}

// ------------------------------------------------------------------ tasks
// Warp-aggregated: one atomic per warp reserves the tasks of 32 records.
__global__ void task_emit_kernel(const PairRec* recs, uint64_t rec_cap, DGraphs q, DOrder o, const uint64_t* arena,
                                 Task* tasks, uint64_t task_cap, Counters* ctr, uint32_t* err) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  const uint32_t lane = lane_id();
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t base_i = uint64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u); base_i < n; base_i += stride) {
    const uint64_t i = base_i + lane;
    B128 c{0, 0};
    if (i < n) {
      const PairRec r = recs[i];
      const uint32_t root = o.perm[uint64_t(r.q) * kMaxQueryNodes];
      c = ld_b128(arena + 2 * (uint64_t(r.c_row) + root));
    }
    const uint32_t k = b_pop(c);
    uint32_t incl = k;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= uint32_t(d)) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(&ctr->tasks, (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!total) continue;
    if (base + total > task_cap) {
      if (lane == 0) atomicOr(err, kErrOverflow);
      continue;
    }
    unsigned long long pos = base + incl - k;
    for (uint32_t j = 0; j < k; ++j) {
      tasks[pos + j] = Task{uint32_t(i), b_low(c)};
      c = b_clear_low(c);
    }
  }
}

// ------------------------------------------------------------------ totals
__global__ void totals_kernel(const Counters* ctr_in, uint64_t rec_cap, const unsigned long long* pair_count,
                              const unsigned long long* pair_exp, const uint32_t* pair_flag, int find_first,
                              Counters* ctr) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr_in->recs);
  unsigned long long c = 0, e = 0, inc = 0;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const unsigned long long k = pair_count[i];
    c += find_first ? (k ? 1ull : 0ull) : k;
    e += pair_exp[i];
    inc += (pair_flag[i] >> 1) & 1u;
  }
  for (int o = 16; o > 0; o >>= 1) {
    c += __shfl_down_sync(0xffffffffu, c, o);
    e += __shfl_down_sync(0xffffffffu, e, o);
    inc += __shfl_down_sync(0xffffffffu, inc, o);
  }
  if (lane_id() == 0) {
    if (c) atomicAdd(&ctr->total, c);
    if (e) atomicAdd(&ctr->expansions, e);
    if (inc) atomicAdd(&ctr->incomplete, inc);
  }
}

__global__ void scatter_kernel(const PairRec* recs, const Counters* ctr, uint64_t rec_cap,
                               const unsigned long long* pair_count, const unsigned long long* pair_exp,
                               const uint32_t* pair_flag, int find_first, uint64_t* counts, uint64_t* exps,
                               uint8_t* status) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t g = recs[i].gpos;
    const unsigned long long k = pair_count[i];
    if (counts) counts[g] = find_first ? (k ? 1ull : 0ull) : k;
    if (exps) exps[g] = pair_exp[i];
    if (status) status[g] = uint8_t((pair_flag[i] >> 1) & 1u);
  }
}

// Batch slices: row offsets and column ids of a slice arrive with global
// values and are rebased to the slice.
__global__ void rebase_kernel(uint32_t* rowp, uint64_t n_rowp, uint32_t entry_base, uint32_t* col, uint64_t n_col,
                              uint32_t node_base) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n_rowp; i += stride) rowp[i] -= entry_base;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n_col; i += stride) col[i] -= node_base;
}

// per_query[q] += the matches of every record with query q (find-first: the
// records with a match); a shared-memory histogram per block when Q is small.
__global__ void query_totals_kernel(const PairRec* recs, const Counters* ctr, uint64_t rec_cap,
                                    const unsigned long long* pair_count, int find_first, uint32_t Q,
                                    unsigned long long* per_query, int use_smem) {
  extern __shared__ unsigned long long s_hist[];
  if (use_smem) {
    for (uint32_t i = threadIdx.x; i < Q; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
  }
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const unsigned long long k = pair_count[i];
    const unsigned long long v = find_first ? (k ? 1ull : 0ull) : k;
    if (!v) continue;
    const uint32_t q = recs[i].q;
    if (use_smem) atomicAdd(&s_hist[q], v);
    else atomicAdd(&per_query[q], v);
  }
  if (use_smem) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < Q; i += blockDim.x)
      if (s_hist[i]) atomicAdd(&per_query[i], s_hist[i]);
  }
}


// Data graphs grouped by size class (65..128 nodes, then 33..64, then <= 32),
// each class in batch order: per tile of kClassTile graphs the class counts,
// then (after scans of those counts) each tile places its graphs.
constexpr uint32_t kClassTile = 2048;
constexpr uint32_t kClassThreads = 256;

__device__ __forceinline__ uint32_t size_class(const uint32_t* goff, uint32_t g) {
  const uint32_t m = goff[g + 1] - goff[g];
  return uint32_t(m > 32u) + uint32_t(m > 64u);
}

__global__ void __launch_bounds__(kClassThreads) class_count_kernel(const uint32_t* goff, uint32_t G, uint32_t* n2,
                                                                    uint32_t* n1) {
  __shared__ uint32_t s2[kClassThreads / 32], s1[kClassThreads / 32];
  const uint32_t t0 = blockIdx.x * kClassTile, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t c2 = 0, c1 = 0;
  for (uint32_t i = threadIdx.x; i < kClassTile; i += kClassThreads) {
    const uint32_t g = t0 + i;
    if (g < G) {
      const uint32_t k = size_class(goff, g);
      c2 += k == 2u;
      c1 += k == 1u;
    }
  }
  c2 = __reduce_add_sync(0xffffffffu, c2);
  c1 = __reduce_add_sync(0xffffffffu, c1);
  if (lane == 0) {
    s2[warp] = c2;
    s1[warp] = c1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t a = 0, b = 0;
    for (uint32_t w = 0; w < kClassThreads / 32; ++w) {
      a += s2[w];
      b += s1[w];
    }
    n2[blockIdx.x] = a;
    n1[blockIdx.x] = b;
  }
}

// p2, p1: exclusive scans of the tiles' class-2 and class-1 counts (p[tiles] =
// the class's total).  A graph's place: its class's start, the class's graphs
// in earlier tiles, then those before it in its tile.
__global__ void __launch_bounds__(kClassThreads) class_place_kernel(const uint32_t* goff, uint32_t G,
                                                                    const uint32_t* p2, const uint32_t* p1,
                                                                    uint32_t tiles, uint32_t* dperm) {
  __shared__ uint32_t w2[kClassThreads / 32], w1[kClassThreads / 32];
  const uint32_t t0 = blockIdx.x * kClassTile, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t total2 = p2[tiles], total1 = p1[tiles];
  const uint32_t b2 = p2[blockIdx.x], b1 = p1[blockIdx.x];
  const uint32_t b0 = t0 - b2 - b1;  // class-0 graphs in earlier tiles
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t run2 = 0, run1 = 0;  // the tile's class-2 / class-1 graphs in earlier rounds
  for (uint32_t i0 = 0; i0 < kClassTile; i0 += kClassThreads) {
    const uint32_t i = i0 + threadIdx.x, g = t0 + i;
    const bool in = g < G;
    const uint32_t k = in ? size_class(goff, g) : 3u;
    const uint32_t m2 = __ballot_sync(0xffffffffu, k == 2u), m1 = __ballot_sync(0xffffffffu, k == 1u);
    if (lane == 0) {
      w2[warp] = uint32_t(__popc(m2));
      w1[warp] = uint32_t(__popc(m1));
    }
    __syncthreads();
    uint32_t r2 = run2 + uint32_t(__popc(m2 & lt)), r1 = run1 + uint32_t(__popc(m1 & lt));
    for (uint32_t w = 0; w < kClassThreads / 32; ++w) {
      const uint32_t a = w2[w], b = w1[w];
      if (w < warp) {
        r2 += a;
        r1 += b;
      }
      run2 += a;
      run1 += b;
    }
    if (in) {
      uint32_t pos;
      if (k == 2u) pos = b2 + r2;
      else if (k == 1u) pos = total2 + b1 + r1;
      else pos = total2 + total1 + b0 + (i - r2 - r1);
      dperm[pos] = g;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_label_count(const DGraphs& d, unsigned long long* counts, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(counts, 0, 256 * sizeof(unsigned long long), st);
  if (e != cudaSuccess || d.N == 0) return e;
  label_count_kernel<<<grid_for(d.N, 256, 4), 256, 0, st>>>(d, counts); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_query_prep(const DGraphs& q, const DSigs& qs, const unsigned long long* label_count,
                              uint8_t* filter_order, uint8_t* dup, cudaStream_t st) {
  if (q.G == 0) return cudaSuccess;
  query_prep_kernel<<<grid_for(uint64_t(q.G) * 32, 128), 128, 0, st>>>(q, qs, label_count, filter_order, dup); note_launch();
  return cudaGetLastError();
}

size_t scan_scratch_words(uint64_t n) {
  size_t w = 0;
  while (n > kScanBlock) {
    n = (n + kScanBlock - 1) / kScanBlock;
    w += 2 * n + 1;
  }
  return w + 2;
}

cudaError_t launch_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* scratch, cudaStream_t st) {
  if (n == 0) return cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
  const uint64_t blocks = (n + kScanBlock - 1) / kScanBlock;
  if (blocks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  uint32_t* sums = scratch;
  uint32_t* sums_scan = scratch + blocks;
  scan_chunks<<<unsigned(blocks), kScanThreads, 0, st>>>(in, out, n, sums); note_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (blocks > 1) {
    e = launch_scan_u32(sums, sums_scan, blocks, scratch + 2 * blocks + 1, st);
    if (e != cudaSuccess) return e;
    scan_add<<<unsigned(blocks), 256, 0, st>>>(out, n, sums_scan); note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  scan_total<<<1, 1, 0, st>>>(in, out, n, out + n); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_gmcr_indices(const uint32_t* valid, uint32_t QW, uint32_t Q, uint32_t D, const uint32_t* offsets,
                                uint32_t* qidx, cudaStream_t st) {
  if (D == 0) return cudaSuccess;
  gmcr_indices_kernel<<<grid_for(D, 128, 16), 128, 0, st>>>(valid, QW, Q, D, offsets, qidx); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_pair_positions(PairRec* recs, const Counters* ctr, uint64_t rec_cap, const uint32_t* valid,
                                  uint32_t QW, const uint32_t* offsets, cudaStream_t st) {
  if (rec_cap == 0) return cudaSuccess;
  pair_positions_kernel<<<grid_for(rec_cap, 256, 4), 256, 0, st>>>(recs, ctr, rec_cap, valid, QW, offsets); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_plain_order(const DGraphs& q, DOrder o, cudaStream_t st) {
  if (q.G == 0) return cudaSuccess;
  plain_order_kernel<<<grid_for(q.G, 128), 128, 0, st>>>(q, o); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_order_adjacency(const DGraphs& q, const DSigs& qs, DOrder o, cudaStream_t st) {
  if (q.G == 0) return cudaSuccess;
  order_adjacency_kernel<<<grid_for(uint64_t(q.G) * kMaxQueryNodes, 256), 256, 0, st>>>(q, qs, o); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_task_emit(const PairRec* recs, uint64_t rec_cap, const DGraphs& q, DOrder o, const uint64_t* arena,
                             Task* tasks, uint64_t task_cap, Counters* ctr, uint32_t* err, cudaStream_t st) {
  if (rec_cap == 0) return cudaSuccess;
  task_emit_kernel<<<grid_for(rec_cap, 256, 4), 256, 0, st>>>(recs, rec_cap, q, o, arena, tasks, task_cap, ctr, err); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_totals(const Counters* ctr_in, uint64_t rec_cap, const unsigned long long* pair_count,
                          const unsigned long long* pair_exp, const uint32_t* pair_flag, int find_first, Counters* ctr,
                          cudaStream_t st) {
  if (rec_cap == 0) return cudaSuccess;
  totals_kernel<<<grid_for(rec_cap, 256, 4), 256, 0, st>>>(ctr_in, rec_cap, pair_count, pair_exp, pair_flag,
                                                            find_first, ctr); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_scatter(const PairRec* recs, const Counters* ctr, uint64_t rec_cap,
                           const unsigned long long* pair_count, const unsigned long long* pair_exp,
                           const uint32_t* pair_flag, int find_first, uint64_t* counts, uint64_t* exps,
                           uint8_t* status, cudaStream_t st) {
  if (rec_cap == 0) return cudaSuccess;
  scatter_kernel<<<grid_for(rec_cap, 256, 4), 256, 0, st>>>(recs, ctr, rec_cap, pair_count, pair_exp, pair_flag,
                                                             find_first, counts, exps, status); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_rebase(uint32_t* rowp, uint64_t n_rowp, uint32_t entry_base, uint32_t* col, uint64_t n_col,
                          uint32_t node_base, cudaStream_t st) {
  if (!entry_base && !node_base) return cudaSuccess;
  rebase_kernel<<<grid_for(n_rowp > n_col ? n_rowp : n_col, 256, 4), 256, 0, st>>>(rowp, n_rowp, entry_base, col, n_col,
                                                                                   node_base); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_query_totals(const PairRec* recs, const Counters* ctr, uint64_t rec_cap,
                                const unsigned long long* pair_count, int find_first, uint32_t Q,
                                unsigned long long* per_query, cudaStream_t st) {
  if (rec_cap == 0 || Q == 0) return cudaSuccess;
  const size_t smem = size_t(Q) * sizeof(unsigned long long);
  const int use_smem = smem <= (48u << 10);
  query_totals_kernel<<<grid_for(rec_cap, 256, 4), 256, use_smem ? smem : 0, st>>>(recs, ctr, rec_cap, pair_count,
                                                                                  find_first, Q, per_query, use_smem); note_launch();
  return cudaGetLastError();
}

uint64_t class_scratch_words(uint32_t G) {
  const uint64_t tiles = (uint64_t(G) + kClassTile - 1) / kClassTile;
  return 4 * (tiles + 1) + scan_scratch_words(tiles);
}

cudaError_t launch_size_classes(const uint32_t* goff, uint32_t G, uint32_t* scratch, uint32_t* dperm, cudaStream_t st) {
  if (G == 0) return cudaSuccess;
  const uint32_t tiles = uint32_t((uint64_t(G) + kClassTile - 1) / kClassTile);
  uint32_t* n2 = scratch;
  uint32_t* n1 = n2 + (tiles + 1);
  uint32_t* p2 = n1 + (tiles + 1);
  uint32_t* p1 = p2 + (tiles + 1);
  uint32_t* ss = p1 + (tiles + 1);
  class_count_kernel<<<tiles, kClassThreads, 0, st>>>(goff, G, n2, n1); note_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = launch_scan_u32(n2, p2, tiles, ss, st)) != cudaSuccess) return e;
  if ((e = launch_scan_u32(n1, p1, tiles, ss, st)) != cudaSuccess) return e;
  class_place_kernel<<<tiles, kClassThreads, 0, st>>>(goff, G, p2, p1, tiles, dperm); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
