// Fused filter + refine + GMCR validity, per (query, data graph) pair.
//
// The reference builds a dense candidate matrix over ALL query nodes x ALL data
// nodes (filterCandidates, isomorphism.hpp:30-104), streams it once per
// refinement step (refineCandidates, :106-203) and then tests every pair for
// validity (GMCR kernel 1, gmcr.hpp:54-88).  Candidate bits only ever matter
// inside a pair's own data graph, so here a warp owns one data graph at a time:
// lane j holds the filter records of data nodes j, j+32, ... in registers, and
// for every query the warp evaluates the full predicate (label, degree, path,
// cycle and every distance shell) node by node, forming each 128-bit candidate
// row with warp ballots.  A pair dies at its first empty row (the validity test
// needs nothing more), and the rows of pairs that go on to the join are written
// once to a compact arena.  The dense matrix never exists.
//
// Before any node is evaluated, 32 queries at a time are screened against the
// data graph's label set: a query using a label the graph lacks has an empty
// candidate row and is GMCR-invalid.  With EXACT semantics, a query whose label
// multiset does not fit into the graph's has no injective embedding; its
// validity is still established exactly, but it is not sent to the join.
#include "device_common.cuh"

namespace bms {
namespace {

template <int ROUNDS, int PWMAX>
struct DataNodes {
  uint32_t lab[ROUNDS], deg[ROUNDS];
  uint64_t cyc[ROUNDS], p[ROUNDS][4], sh[ROUNDS][PWMAX];
  bool live[ROUNDS];
};

// Candidate row of one query node: label (or wildcard) and degree, then path
// containment and cycle counts, then every distance shell; a warp-uniform
// early exit follows each group.
template <int ROUNDS, int PWMAX>
__device__ __forceinline__ B128 eval_rows(const DataNodes<ROUNDS, PWMAX>& dn, const uint64_t* __restrict__ qr,
                                          const uint64_t* __restrict__ qp, uint32_t PW) {
  const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(qr);
  const uint32_t ql = uint32_t(a.x & 0xFFu), qd = uint32_t(a.x >> 32);
  bool ok[ROUNDS];
  bool any = false;
#pragma unroll
  for (int r = 0; r < ROUNDS; ++r) {
    ok[r] = dn.live[r] && (ql == dn.lab[r] || ql == kWildcard) && qd <= dn.deg[r];
    any |= ok[r];
  }
  if (!__any_sync(0xffffffffu, any)) return B128{0, 0};
  const ulonglong2 p01 = *reinterpret_cast<const ulonglong2*>(qr + 2);
  const ulonglong2 p23 = *reinterpret_cast<const ulonglong2*>(qr + 4);
  any = false;
#pragma unroll
  for (int r = 0; r < ROUNDS; ++r) {
    const uint64_t miss = (p01.x & ~dn.p[r][0]) | (p01.y & ~dn.p[r][1]) | (p23.x & ~dn.p[r][2]) | (p23.y & ~dn.p[r][3]);
    ok[r] = ok[r] && miss == 0 && cyc_ge(dn.cyc[r], a.y);
    any |= ok[r];
  }
  if (!__any_sync(0xffffffffu, any)) return B128{0, 0};
  uint64_t q[PWMAX];
#pragma unroll
  for (int w = 0; w < PWMAX; ++w) q[w] = uint32_t(w) < PW ? qp[w] : 0ull;
  uint32_t ballots[4] = {0, 0, 0, 0};
#pragma unroll
  for (int r = 0; r < ROUNDS; ++r) {
    uint64_t acc = kHiBit;
#pragma unroll
    for (int w = 0; w < PWMAX; ++w)
      if (uint32_t(w) < PW) acc &= nib_le_bits(q[w], dn.sh[r][w]);
    ballots[r] = __ballot_sync(0xffffffffu, ok[r] && (acc & kHiBit) == kHiBit);
  }
  return B128{uint64_t(ballots[0]) | (uint64_t(ballots[1]) << 32), uint64_t(ballots[2]) | (uint64_t(ballots[3]) << 32)};
}

template <int ROUNDS, int PWMAX>
__global__ void __launch_bounds__(ROUNDS <= 2 ? 256 : 128) pair_filter_kernel(PairFilterArgs a) {
  constexpr int kWarpsPerBlock = (ROUNDS <= 2 ? 256 : 128) / 32;
  __shared__ B128 s_rows[kWarpsPerBlock][kMaxQueryNodes];
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  B128* rows = s_rows[warp];
  const int R = a.ds.R;
  const uint32_t Q = a.q.G;
  for (;;) {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(&a.ctr->work[a.class_id], 1u);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (a.class_begin + idx >= a.class_end) break;
    const uint32_t dg = a.dperm[a.class_begin + idx];
    const uint32_t start = a.d.goff[dg], m = a.d.goff[dg + 1] - start;
    if (m == 0) {  // an empty data graph has no candidates: every pair is invalid
      for (uint32_t w = lane; w < a.QW; w += 32) a.valid[uint64_t(dg) * a.QW + w] = 0u;
      if (lane == 0) a.vcounts[dg] = 0u;
      continue;
    }
    DataNodes<ROUNDS, PWMAX> dn;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
      const uint32_t v = lane + 32 * r;
      dn.live[r] = v < m;
      const uint64_t* rec = a.ds.frec + uint64_t(kRecWords) * (uint64_t(start) + (dn.live[r] ? v : 0));
      const ulonglong2 w01 = *reinterpret_cast<const ulonglong2*>(rec);
      const ulonglong2 w23 = *reinterpret_cast<const ulonglong2*>(rec + 2);
      const ulonglong2 w45 = *reinterpret_cast<const ulonglong2*>(rec + 4);
      dn.lab[r] = uint32_t(w01.x & 0xFFu);
      dn.deg[r] = uint32_t(w01.x >> 32);
      dn.cyc[r] = w01.y;
      dn.p[r][0] = w23.x;
      dn.p[r][1] = w23.y;
      dn.p[r][2] = w45.x;
      dn.p[r][3] = w45.y;
      uint64_t sh[kMaxSteps];
#pragma unroll
      for (int k = 0; k < kMaxSteps; ++k) sh[k] = k < R ? rec[6 + k] : 0ull;
#pragma unroll
      for (int w = 0; w < PWMAX; ++w) dn.sh[r][w] = uint32_t(w) < a.sp.PW ? packed_word(sh, R, w, a.sp) : 0ull;
    }
    const uint64_t dhist = a.ds.ghist[dg];
    const uint32_t dlab = a.ds.glabset[dg];
    uint32_t nvalid = 0;
    for (uint32_t qb = 0; qb < Q; qb += 32) {
      const uint32_t qg = qb + lane;
      bool p1 = false, p2 = false;
      if (qg < Q) {
        const uint32_t n = a.q.goff[qg + 1] - a.q.goff[qg];
        p1 = n > 1 && (a.qs.glabset[qg] & ~dlab) == 0;  // gmcr.hpp:64 and label presence
        p2 = p1 && (!a.skip_by_labels || nib_le(a.qs.ghist[qg], dhist));
      }
      uint32_t m1 = __ballot_sync(0xffffffffu, p1);
      const uint32_t m2 = __ballot_sync(0xffffffffu, p2);
      uint32_t vb = 0;
      while (m1) {
        const int i = __ffs(m1) - 1;
        m1 &= m1 - 1;
        const uint32_t q = qb + uint32_t(i);
        const bool join = (m2 >> i) & 1u;
        const uint32_t qoff = a.q.goff[q], n = a.q.goff[q + 1] - qoff;
        const uint8_t* ord = a.filter_order + uint64_t(q) * kMaxQueryNodes;
        const uint8_t* dup = a.dup + uint64_t(q) * kMaxQueryNodes;
        bool valid = true;
        for (uint32_t t = 0; t < n; ++t) {
          const uint32_t ul = ord[t];
          const uint32_t src = dup[ul];
          B128 c;
          if (src != 0xFFu) {
            __syncwarp();
            c = rows[src];  // identical record, evaluated earlier in this pair
          } else {
            c = eval_rows<ROUNDS, PWMAX>(dn, a.qs.frec + uint64_t(kRecWords) * (qoff + ul),
                                         a.qpack + 8 * (uint64_t(qoff) + ul), a.sp.PW);
            if (!b_any(c)) {
              valid = false;
              break;
            }
          }
          if (lane == 0) rows[ul] = c;
        }
        if (!valid) continue;
        vb |= 1u << i;
        if (!join) continue;
        unsigned long long rec = 0, row = 0;
        if (lane == 0) {
          rec = atomicAdd(&a.ctr->recs, 1ull);
          row = atomicAdd(&a.ctr->rows, (unsigned long long)n);
        }
        rec = __shfl_sync(0xffffffffu, rec, 0);
        row = __shfl_sync(0xffffffffu, row, 0);
        __syncwarp();
        if (rec >= a.rec_cap || row + n > a.row_cap) {
          if (lane == 0) atomicOr(a.err, kErrOverflow);
          continue;
        }
        if (lane == 0) a.recs[rec] = PairRec{q, dg, 0u, uint32_t(row)};
        for (uint32_t t = lane; t < n; t += 32) {
          const B128 c = rows[t];
          st_b128(a.arena + 2 * (row + t), c);
          if (a.cand_sum) atomicAdd(&a.cand_sum[qoff + t], b_pop(c));
        }
        __syncwarp();
      }
      if (lane == 0) a.valid[uint64_t(dg) * a.QW + (qb >> 5)] = vb;
      nvalid += __popc(vb);
    }
    if (lane == 0) a.vcounts[dg] = nvalid;
  }
}

__global__ void pack_query_shells_kernel(DGraphs q, DSigs qs, ShellPack sp, uint64_t* qpack) {
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < q.N; u += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t sh[kMaxSteps];
    for (int k = 0; k < kMaxSteps; ++k) sh[k] = k < qs.R ? qs.frec[uint64_t(kRecWords) * u + 6 + k] : 0ull;
    for (int w = 0; w < 8; ++w) qpack[8 * u + w] = uint32_t(w) < sp.PW ? packed_word(sh, qs.R, w, sp) : 0ull;
  }
}

template <int ROUNDS, int PWMAX>
void launch_rounds(const PairFilterArgs& a, unsigned blocks, unsigned threads, cudaStream_t st) {
  pair_filter_kernel<ROUNDS, PWMAX><<<blocks, threads, 0, st>>>(a); note_launch();
}

template <int ROUNDS>
void launch_pw(const PairFilterArgs& a, unsigned blocks, unsigned threads, cudaStream_t st) {
  if (a.sp.PW <= 2) launch_rounds<ROUNDS, 2>(a, blocks, threads, st);
  else if (a.sp.PW <= 4) launch_rounds<ROUNDS, 4>(a, blocks, threads, st);
  else launch_rounds<ROUNDS, 8>(a, blocks, threads, st);
}

}  // namespace

cudaError_t launch_pack_query_shells(const DGraphs& q, const DSigs& qs, ShellPack sp, uint64_t* qpack,
                                     cudaStream_t st) {
  if (q.N == 0) return cudaSuccess;
  const uint64_t want = (q.N + 127) / 128, cap = uint64_t(sm_count()) * 4;
  pack_query_shells_kernel<<<unsigned(want < cap ? want : cap), 128, 0, st>>>(q, qs, sp, qpack); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_pair_filter(const PairFilterArgs& a, int rounds, cudaStream_t st) {
  if (a.class_end <= a.class_begin) return cudaSuccess;
  const uint32_t graphs = a.class_end - a.class_begin;
  const uint64_t sms = uint64_t(sm_count());
  if (rounds <= 1) {
    launch_pw<1>(a, unsigned(std::min<uint64_t>((graphs + 7) / 8, sms * 8)), 256, st);
  } else if (rounds == 2) {
    launch_pw<2>(a, unsigned(std::min<uint64_t>((graphs + 7) / 8, sms * 8)), 256, st);
  } else {
    launch_pw<4>(a, unsigned(std::min<uint64_t>((graphs + 3) / 4, sms * 8)), 128, st);
  }
  return cudaGetLastError();
}

}  // namespace bms
