// Clustered join, REFERENCE_DFS semantics: the reference driver's --use-cs
// flow (BMS2.cpp:218-296) restated literally.  (EXACT runs inside the join
// kernels, k_join.cu, as round 0 of the join.)
//
// The query batch is one cluster: query 0 is the prototype P, and every member
// lists P's nodes first, in P's order (generate_cs.py:338-362, 555-577).  The
// reference runs two kernels: joinPartialCandidates2 (isomorphism.hpp:1021-1178)
// writes every match of P's nodes 0..end-1 (end = |V(P)|) in every data graph to
// a global array, and joinWithPartialMatches (isomorphism.hpp:756-977) gives
// each stored match a subgroup that extends it with every query of its data
// graph's GMCR row.  Here one warp owns a data graph from start to end: its
// lanes enumerate P's matches (each lane a share of the roots) into a 64-entry
// shared-memory buffer, then the whole warp extends the buffered matches, one
// (match, query) item per lane, before it refills the buffer.
//
// Per item (match of graph d, query q of d's GMCR row, n = |V(q)|): n < end
// adds nothing, n == end adds 1, otherwise every branch root (a candidate of
// q's node `end` outside the match that passes the induced test against it)
// starts a DFS over q's candidate rows.  Both loops are the reference's: a
// frame never clears the visited bit of a candidate it moves past, an
// exhausted frame clears the bit of mapping[k] (the last value written at depth
// k in this root's search, nothing before the first write), step 1 records a
// match at depth `end` and pops without touching visited, and step 2 starts
// each branch root with visited = match + root.
#include "device_common.cuh"

namespace bms {
namespace {

constexpr int kCsWarps = 4;     // warps per block
constexpr int kCsBuf = 64;      // prototype matches buffered per warp
constexpr int kCsChunk = 4;     // data graphs taken per work-queue atomic

__global__ void pos_desc_kernel(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, DGraphs q, uint4* out) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const PairRec r = recs[i];
    if (r.gpos < rec_cap) out[r.gpos] = make_uint4(uint32_t(i), r.c_row, q.goff[r.q + 1] - q.goff[r.q], r.q);
  }
}

// Candidates at depth j of a query (rows `crow`, order adjacency `dadj`) given
// the path f[0..j-1]: v is kept iff it is in the rows of the images of j's
// earlier query neighbours and in no row of the images of its earlier
// non-neighbours (isValidMapping_fast_bitwise, isomorphism.hpp:266-285).  The
// path may hold a node twice (a stale clear unmarks a path node), so the
// non-neighbour images are collected position by position; path nodes are
// left to the visited set.
__device__ __forceinline__ B128 level(const uint64_t* crow, const uint64_t* dadj, const uint64_t* arow,
                                      const uint64_t* irow, uint32_t j, const uint8_t* f) {
  B128 c = ld_b128(crow + 2 * uint64_t(j));
  const uint64_t adj = __ldg(reinterpret_cast<const unsigned long long*>(dadj) + j);
  for (uint64_t pm = adj; pm; pm &= pm - 1) c = b_and(c, ld_b128(arow + 2 * uint64_t(f[__ffsll((long long)pm) - 1])));
  B128 nset{0, 0};
  for (uint64_t nm = ~adj & ((uint64_t(1) << j) - 1); nm; nm &= nm - 1)
    nset = b_or(nset, b_bit(f[__ffsll((long long)nm) - 1]));
  B128 res{0, 0};
  for (B128 r = c; b_any(r); r = b_clear_low(r)) {
    const uint32_t v = b_low(r);
    if (!b_any(b_and(ld_b128(irow + 2 * uint64_t(v)), nset))) res = b_or(res, b_bit(v));
  }
  return res;
}

// A lane's enumeration of prototype matches (joinPartialCandidates2's DFS).
struct Enum {
  B128 roots;  // roots not started yet
  B128 vis;    // the visited set
  uint64_t mpset;
  int t;       // current depth, -1 = start the next root
  bool done;
};

__device__ __forceinline__ bool next_match(Enum& e, uint32_t end, const uint64_t* crow, const uint64_t* dadj,
                                           const uint64_t* arow, const uint64_t* irow, uint8_t* f, B128* F, uint8_t* mp,
                                           unsigned long long& exps) {
  for (;;) {
    if (e.t < 0) {
      if (!b_any(e.roots)) return false;
      const uint32_t v0 = b_low(e.roots);
      e.roots = b_clear_low(e.roots);
      f[0] = uint8_t(v0);
      ++exps;
      if (end == 1) return true;
      e.vis = b_bit(v0);
      e.mpset = 0;
      F[1] = level(crow, dadj, arow, irow, 1, f);
      e.t = 1;
    }
    int t = e.t;
    if (!b_any(F[t])) {  // frame t exhausted: mapping[t] leaves visited
      if ((e.mpset >> t) & 1ull) e.vis = b_andn(e.vis, b_bit(mp[t]));
      if (t == 1) {
        e.t = -1;
        continue;
      }
      e.t = t - 1;
      continue;
    }
    const uint32_t v = b_low(F[t]);
    F[t] = b_clear_low(F[t]);
    if (b_has(e.vis, v)) continue;
    mp[t] = uint8_t(v);
    e.mpset |= uint64_t(1) << t;
    e.vis = b_or(e.vis, b_bit(v));
    f[t] = uint8_t(v);
    ++exps;
    if (uint32_t(t) + 1 == end) return true;  // depth `end`: recorded, popped at once
    F[t + 1] = level(crow, dadj, arow, irow, uint32_t(t) + 1, f);
    e.t = t + 1;
  }
}

// Literal extension (joinWithPartialMatches' loop over branch roots and its DFS).
template <bool kFind>
__device__ unsigned long long extend_literal(uint32_t end, uint32_t n, const uint64_t* crow, const uint64_t* dadj,
                                             const uint64_t* arow, const uint64_t* irow, uint8_t* f, B128* F,
                                             uint8_t* mp, unsigned long long& exps) {
  B128 pre{0, 0};
  for (uint32_t k = 0; k < end; ++k) pre = b_or(pre, b_bit(f[k]));
  // branch roots: induced-consistent with the prefix and not in it
  const B128 roots = b_andn(level(crow, dadj, arow, irow, end, f), pre);
  unsigned long long cnt = 0;
  for (B128 rr = roots; b_any(rr); rr = b_clear_low(rr)) {
    const uint32_t b = b_low(rr);
    ++exps;
    if (end + 1 == n) {
      ++cnt;
      if (kFind) return cnt;
      continue;
    }
    f[end] = uint8_t(b);
    B128 vis = b_or(pre, b_bit(b));
    uint64_t mpset = 0;
    uint32_t t = end + 1;
    F[t] = level(crow, dadj, arow, irow, t, f);
    if (t + 1 == n) {  // the first frame is the leaf frame
      const uint32_t pc = b_pop(b_andn(F[t], vis));
      cnt += pc;
      exps += pc;
      if (kFind && cnt) return cnt;
      continue;
    }
    for (;;) {
      if (!b_any(F[t])) {  // frame t exhausted
        if ((mpset >> t) & 1ull) vis = b_andn(vis, b_bit(mp[t]));
        if (t == end + 1) break;
        --t;
        continue;
      }
      const uint32_t v = b_low(F[t]);
      F[t] = b_clear_low(F[t]);
      if (b_has(vis, v)) continue;
      f[t] = uint8_t(v);
      mp[t] = uint8_t(v);
      mpset |= uint64_t(1) << t;
      vis = b_or(vis, b_bit(v));
      ++exps;
      const B128 nf = level(crow, dadj, arow, irow, t + 1, f);
      if (t + 2 == n) {
        // frame n-1: every unvisited candidate is pushed and popped at depth n
        const uint32_t last = n - 1;
        const B128 acc = b_andn(nf, vis);
        const uint32_t pc = b_pop(acc);
        cnt += pc;
        exps += pc;
        if (kFind && cnt) return cnt;
        if (pc) {
          vis = b_or(vis, acc);
          mp[last] = uint8_t(b_high(acc));
          mpset |= uint64_t(1) << last;
        }
        if ((mpset >> last) & 1ull) vis = b_andn(vis, b_bit(mp[last]));  // frame n-1 exhausted
        continue;
      }
      F[++t] = nf;
    }
  }
  return cnt;
}

template <bool kFind>
__global__ void __launch_bounds__(kCsWarps * 32) cs_join_kernel(CsArgs a) {
  __shared__ __align__(16) uint8_t s_buf[kCsWarps][kCsBuf * kMaxQueryNodes];
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  uint8_t* buf = s_buf[warp];
  const uint32_t end = a.end, D = a.d.G;
  const uint32_t p_off = a.q.goff[0];
  uint8_t fa[kMaxQueryNodes], fb[kMaxQueryNodes], mpa[kMaxQueryNodes], mpb[kMaxQueryNodes];
  B128 Fa[kMaxQueryNodes], Fb[kMaxQueryNodes];
  unsigned long long parts = 0, pexps = 0;
  for (;;) {
    uint32_t i0 = 0;
    if (lane == 0) i0 = atomicAdd(&a.ctr->cs_head, uint32_t(kCsChunk));
    i0 = __shfl_sync(0xffffffffu, i0, 0);
    if (i0 >= D) break;
    for (uint32_t i = i0; i < i0 + kCsChunk && i < D; ++i) {
      const uint32_t d = a.dperm ? a.dperm[i] : i;
      const uint32_t start = a.d.goff[d], m = a.d.goff[d + 1] - start;
      const uint32_t g0 = a.gmcr_off[d], vcount = a.gmcr_off[d + 1] - g0;
      if (m == 0) continue;
      const uint64_t* crow_p = nullptr;
      B128 roots;
      if (end == 1) {
        roots = prototype_row(a.qs.frec, a.ds.frec, a.ds.R, a.dense, a.W, p_off, start, m);
        if (vcount == 0) {  // no query to extend: only the matches are counted
          if (lane == 0) {
            parts += b_pop(roots);
            pexps += b_pop(roots);
          }
          continue;
        }
      } else {
        // the prototype's own pair heads the row when it is valid (query ids ascend)
        const uint4 p0 = vcount && g0 < a.rec_cap ? a.pos_desc[g0] : make_uint4(kNoRecord, 0, 0, 0);
        if (p0.x == kNoRecord || p0.w != 0) continue;
        crow_p = a.arena + 2 * uint64_t(p0.y);
        roots = ld_b128(crow_p);
      }
      const uint64_t* arow = a.ds.adj + 2 * uint64_t(start);
      const uint64_t* irow = a.ds.adjin + 2 * uint64_t(start);
      Enum e;
      e.roots = B128{0, 0};
      {  // this lane's roots: every 32nd set bit from its rank on
        uint32_t k = 0;
        for (B128 r = roots; b_any(r); r = b_clear_low(r), ++k)
          if ((k & 31u) == lane) e.roots = b_or(e.roots, b_bit(b_low(r)));
      }
      e.vis = B128{0, 0};
      e.mpset = 0;
      e.t = -1;
      e.done = false;
      uint32_t nb = 0;
      for (;;) {
        // fill the buffer with prototype matches
        for (;;) {
          bool have = false;
          if (!e.done) {
            have = next_match(e, end, crow_p, a.o.dadj, arow, irow, fa, Fa, mpa, pexps);
            e.done = !have;
          }
          const uint32_t bal = __ballot_sync(0xffffffffu, have);
          if (have) {
            uint8_t* dst = buf + (nb + __popc(bal & ((1u << lane) - 1u))) * kMaxQueryNodes;
            for (uint32_t k = 0; k < end; ++k) dst[k] = fa[k];
            ++parts;
          }
          nb += __popc(bal);
          if (nb + 32 > kCsBuf || __all_sync(0xffffffffu, e.done)) break;
        }
        __syncwarp();
        // extend every buffered match with every query of the graph
        const uint32_t items = nb * vcount;
        for (uint32_t k = lane; k < items; k += 32) {
          const uint32_t p = k / vcount, j = k - p * vcount;
          if (uint64_t(g0) + j >= a.rec_cap) continue;
          const uint4 pd = a.pos_desc[g0 + j];
          const uint32_t rec = pd.x, n = pd.z;
          if (rec == kNoRecord) continue;
          if (n < end) continue;
          if (kFind && (a.pair_flag[rec] & 1u)) continue;
          unsigned long long cnt = 1, ex = 0;
          if (n > end) {
            const uint8_t* src = buf + p * kMaxQueryNodes;
            for (uint32_t t = 0; t < end; ++t) fb[t] = src[t];
            const uint64_t* crow = a.arena + 2 * uint64_t(pd.y);
            const uint64_t* dadj = a.o.dadj + uint64_t(pd.w) * kMaxQueryNodes;
            cnt = extend_literal<kFind>(end, n, crow, dadj, arow, irow, fb, Fb, mpb, ex);
          }
          if (cnt) {
            if (kFind) {
              atomicOr(a.pair_flag + rec, 1u);
              a.pair_count[rec] = 1ull;
            } else {
              atomicAdd(a.pair_count + rec, cnt);
            }
          }
          if (ex) atomicAdd(a.pair_exp + rec, ex);
        }
        __syncwarp();
        nb = 0;
        if (__all_sync(0xffffffffu, e.done)) break;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    parts += __shfl_down_sync(0xffffffffu, parts, o);
    pexps += __shfl_down_sync(0xffffffffu, pexps, o);
  }
  if (lane == 0) {
    if (parts) atomicAdd(&a.ctr->partials, parts);
    if (pexps) {
      atomicAdd(&a.ctr->partial_exps, pexps);
      atomicAdd(&a.ctr->expansions, pexps);
    }
  }
}

}  // namespace

cudaError_t launch_pos_desc(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, const DGraphs& q, uint4* desc,
                               cudaStream_t st) {
  if (rec_cap == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(desc, 0xFF, sizeof(uint4) * rec_cap, st);
  if (e != cudaSuccess) return e;
  pos_desc_kernel<<<sm_count() * 4, 256, 0, st>>>(recs, ctr, rec_cap, q, desc); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_cs_join(const CsArgs& a, bool find_first, cudaStream_t st) {
  if (a.d.G == 0 || a.end == 0) return cudaSuccess;
  const int blocks = sm_count() * 8, threads = kCsWarps * 32;
  if (find_first) cs_join_kernel<true><<<blocks, threads, 0, st>>>(a);
  else cs_join_kernel<false><<<blocks, threads, 0, st>>>(a);
  note_launch();
  return cudaGetLastError();
}

}  // namespace bms
