// Staged, reference-shaped stages on the dense query-major candidate matrix
// (Candidates, candidates.hpp:10-24: one row of ceil(data_nodes/32) uint32 words
// per query node).
//   filter_dense   <- FilterCandidatesKernel_v2  isomorphism.hpp:30-104
//   refine_dense   <- RefineCandidatesKernel_v3  isomorphism.hpp:106-203
//   gmcr_dense     <- GMCR kernel 1              gmcr.hpp:54-88
//   gather_pairs   <- the per-task candidate counts/selects of the join
//                     (isomorphism.hpp:371-391, candidates.hpp:82-158), done once
//                     per pair into 128-bit local rows
#include "device_common.cuh"

namespace bms {
namespace {

constexpr int kTileNodes = 512;  // data nodes per filter tile (16 words)
constexpr int kTileWords = kTileNodes / 32;
constexpr int kQueryTile = 64;

__global__ void __launch_bounds__(256) filter_dense_kernel(DGraphs q, DSigs qs, DGraphs d, DSigs ds, uint32_t* cand,
                                                          uint64_t W) {
  __shared__ uint32_t s_lab[kTileNodes], s_deg[kTileNodes];
  __shared__ uint64_t s_p0[kTileNodes], s_p1[kTileNodes], s_p2[kTileNodes], s_p3[kTileNodes], s_cyc[kTileNodes];
  const uint64_t base = uint64_t(blockIdx.x) * kTileNodes;
  for (int i = threadIdx.x; i < kTileNodes; i += blockDim.x) {
    const uint64_t v = base + i;
    if (v < d.N) {
      const uint64_t* r = ds.frec + kRecWords * v;
      const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(r);
      const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(r + 2);
      const ulonglong2 c = *reinterpret_cast<const ulonglong2*>(r + 4);
      s_lab[i] = uint32_t(a.x & 0xFFu);
      s_deg[i] = uint32_t(a.x >> 32);
      s_cyc[i] = a.y;
      s_p0[i] = b.x;
      s_p1[i] = b.y;
      s_p2[i] = c.x;
      s_p3[i] = c.y;
    } else {
      s_lab[i] = 0x100u;  // never equal to a query label
      s_deg[i] = 0;
      s_cyc[i] = s_p0[i] = s_p1[i] = s_p2[i] = s_p3[i] = 0;
    }
  }
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint64_t word0 = uint64_t(blockIdx.x) * kTileWords;
  for (uint32_t k = warp; k < kQueryTile; k += blockDim.x >> 5) {
    const uint64_t u = uint64_t(blockIdx.y) * kQueryTile + k;
    if (u >= q.N) break;
    const uint64_t* qr = qs.frec + kRecWords * u;
    const uint64_t w0 = qr[0], qc = qr[1], q0 = qr[2], q1 = qr[3], q2 = qr[4], q3 = qr[5];
    const uint32_t ql = uint32_t(w0 & 0xFFu), qd = uint32_t(w0 >> 32);
    uint32_t mine = 0;
    for (int w = 0; w < kTileWords; ++w) {
      const int i = w * 32 + lane;
      // filterCandidates test order: label (or wildcard), degree, path, cycle
      bool ok = (ql == s_lab[i] || (ql == kWildcard && s_lab[i] < 0x100u)) && qd <= s_deg[i];
      uint32_t word = 0;
      if (__any_sync(0xffffffffu, ok)) {
        ok = ok && (s_p0[i] & q0) == q0 && (s_p1[i] & q1) == q1 && (s_p2[i] & q2) == q2 && (s_p3[i] & q3) == q3 &&
             cyc_ge(s_cyc[i], qc);
        word = __ballot_sync(0xffffffffu, ok);
      }
      if (lane == uint32_t(w)) mine = word;
    }
    if (lane < kTileWords && word0 + lane < W) cand[u * W + word0 + lane] = mine;
  }
}

__global__ void refine_dense_kernel(DSigs qs, uint64_t Qn, DSigs ds, uint64_t Dn, int step, uint32_t* cand,
                                    uint64_t W) {
  const uint64_t total = Qn * W;
  const uint64_t chunks = (total + 3) / 4;
  for (uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < chunks; c += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t f0 = c * 4;
    uint32_t w[4];
    const bool full = f0 + 4 <= total;
    if (full) {
      const uint4 v = *reinterpret_cast<const uint4*>(cand + f0);
      w[0] = v.x, w[1] = v.y, w[2] = v.z, w[3] = v.w;
    } else {
      for (int j = 0; j < 4; ++j) w[j] = f0 + j < total ? cand[f0 + j] : 0u;
    }
    if ((w[0] | w[1] | w[2] | w[3]) == 0) continue;
    uint64_t u = f0 / W;
    uint64_t wi = f0 - u * W;
    bool changed = false;
    uint64_t qsig = qs.frec[kRecWords * u + 6 + step - 1];
    for (int j = 0; j < 4; ++j) {
      if (j > 0 && ++wi == W) {
        wi = 0;
        ++u;
        if (u < Qn) qsig = qs.frec[kRecWords * u + 6 + step - 1];
      }
      uint32_t nb = w[j];
      for (uint32_t bits = w[j]; bits; bits &= bits - 1) {
        const uint32_t bit = uint32_t(__ffs(bits) - 1);
        const uint64_t v = wi * 32 + bit;
        const bool keep = v < Dn && nib_le(qsig, ds.frec[kRecWords * v + 6 + step - 1]);
        if (!keep) nb &= ~(1u << bit);
      }
      changed |= nb != w[j];
      w[j] = nb;
    }
    if (!changed) continue;
    if (full) {
      *reinterpret_cast<uint4*>(cand + f0) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
      for (int j = 0; j < 4; ++j)
        if (f0 + j < total) cand[f0 + j] = w[j];
    }
  }
}

// popcount of bits [s, e) of a row of uint32 words
__device__ __forceinline__ uint32_t range_pop(const uint32_t* row, uint32_t s, uint32_t e) {
  uint32_t c = 0;
  while (s < e) {
    const uint32_t wi = s >> 5, lo = s & 31u;
    const uint32_t take = min(32u - lo, e - s);
    uint32_t x = row[wi] >> lo;
    if (take < 32) x &= (1u << take) - 1u;
    c += __popc(x);
    s += take;
  }
  return c;
}

// One thread per data graph; consecutive threads read consecutive words of a row.
__global__ void gmcr_dense_kernel(DGraphs q, DGraphs d, const uint32_t* cand, uint64_t W, uint32_t* valid, uint32_t QW,
                                  uint32_t* vcounts) {
  for (uint32_t dg = blockIdx.x * blockDim.x + threadIdx.x; dg < d.G; dg += gridDim.x * blockDim.x) {
    const uint32_t s = d.goff[dg], e = d.goff[dg + 1];
    uint32_t word = 0, total = 0;
    for (uint32_t qg = 0; qg < q.G; ++qg) {
      const uint32_t qoff = q.goff[qg], n = q.goff[qg + 1] - qoff;
      bool ok = n > 1;  // gmcr.hpp:64
      for (uint32_t i = 0; i < n && ok; ++i) ok = range_pop(cand + uint64_t(qoff + i) * W, s, e) > 0;
      word |= uint32_t(ok) << (qg & 31u);
      if ((qg & 31u) == 31u || qg + 1 == q.G) {
        valid[uint64_t(dg) * QW + (qg >> 5)] = word;
        total += __popc(word);
        word = 0;
      }
    }
    vcounts[dg] = total;
  }
}

__global__ void pair_nodes_kernel(DGraphs q, const uint32_t* qidx, uint64_t T, uint32_t* nodes) {
  for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < T; t += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t qg = qidx[t];
    nodes[t] = q.goff[qg + 1] - q.goff[qg];
  }
}

// One warp per data graph: its GMCR pairs in order.
__global__ void gather_pairs_kernel(DGraphs q, DGraphs d, const uint32_t* cand, uint64_t W, const uint32_t* offsets,
                                    const uint32_t* qidx, const uint32_t* row_off, PairRec* recs, uint64_t* arena) {
  const uint32_t lane = lane_id();
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t dg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; dg < d.G; dg += warps) {
    const uint32_t s = d.goff[dg], m = d.goff[dg + 1] - s;
    for (uint32_t t = offsets[dg]; t < offsets[dg + 1]; ++t) {
      const uint32_t qg = qidx[t];
      const uint32_t qoff = q.goff[qg], n = q.goff[qg + 1] - qoff;
      const uint32_t r0 = row_off[t];
      for (uint32_t u = lane; u < n; u += 32)
        st_b128(arena + 2 * (uint64_t(r0) + u), extract_row(cand + uint64_t(qoff + u) * W, W, s, m));
      if (lane == 0) recs[t] = PairRec{qg, dg, t, r0};
    }
  }
}

__global__ void set_counter_kernel(unsigned long long* dst, unsigned long long v) { *dst = v; }

}  // namespace

thread_local unsigned long long g_launches = 0;

int sm_count() {
  static int cached = 0;
  if (!cached) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached = n > 0 ? n : 152;
  }
  return cached;
}

static unsigned grid_for(uint64_t work, unsigned threads, unsigned per_sm = 8) {
  uint64_t want = (work + threads - 1) / threads;
  uint64_t cap = uint64_t(sm_count()) * per_sm;
  if (want < 1) want = 1;
  return unsigned(want < cap ? want : cap);
}

cudaError_t launch_filter_dense(const DGraphs& q, const DSigs& qs, const DGraphs& d, const DSigs& ds, uint32_t* cand,
                                uint64_t W, cudaStream_t st) {
  if (q.N == 0 || W == 0) return cudaSuccess;
  const uint64_t tiles = (d.N + kTileNodes - 1) / kTileNodes;
  const uint64_t qt = (q.N + kQueryTile - 1) / kQueryTile;
  if (tiles > 0x7FFFFFFFull || qt > 65535) return cudaErrorInvalidValue;
  // words of the last tile beyond the data nodes are zero-filled by the kernel
  filter_dense_kernel<<<dim3(unsigned(tiles ? tiles : 1), unsigned(qt)), 256, 0, st>>>(q, qs, d, ds, cand, W); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_refine_dense(const DSigs& qs, uint64_t Qn, const DSigs& ds, uint64_t Dn, int step, uint32_t* cand,
                                uint64_t W, cudaStream_t st) {
  if (Qn == 0 || W == 0) return cudaSuccess;
  refine_dense_kernel<<<grid_for((Qn * W + 3) / 4, 256, 16), 256, 0, st>>>(qs, Qn, ds, Dn, step, cand, W); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_gmcr_dense(const DGraphs& q, const DGraphs& d, const uint32_t* cand, uint64_t W, uint32_t* valid,
                              uint32_t QW, uint32_t* vcounts, cudaStream_t st) {
  if (d.G == 0) return cudaSuccess;
  gmcr_dense_kernel<<<grid_for(d.G, 128, 16), 128, 0, st>>>(q, d, cand, W, valid, QW, vcounts); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_pair_nodes(const DGraphs& q, const uint32_t* qidx, uint64_t T, uint32_t* nodes, cudaStream_t st) {
  if (T == 0) return cudaSuccess;
  pair_nodes_kernel<<<grid_for(T, 256), 256, 0, st>>>(q, qidx, T, nodes); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_gather_pairs(const DGraphs& q, const DGraphs& d, const uint32_t* cand, uint64_t W,
                                const uint32_t* offsets, const uint32_t* qidx, const uint32_t* row_off, PairRec* recs,
                                uint64_t* arena, cudaStream_t st) {
  if (d.G == 0) return cudaSuccess;
  gather_pairs_kernel<<<grid_for(uint64_t(d.G) * 32, 256), 256, 0, st>>>(q, d, cand, W, offsets, qidx, row_off, recs,
                                                                         arena); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_set_counter(unsigned long long* dst, unsigned long long value, cudaStream_t st) {
  set_counter_kernel<<<1, 1, 0, st>>>(dst, value); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
