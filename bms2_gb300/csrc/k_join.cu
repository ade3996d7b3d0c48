// Persistent, work-stealing DFS join.
//
// Replaces join::joinCandidates / JoinCandidates3Optimized (isomorphism.hpp:
// 291-472).  The reference gives a sub-group one (query, data graph) pair;
// lanes stride over root candidates, select each candidate by rank with an
// O(words) scan (candidates.hpp:128-158) and test adjacency with a linear CSR
// scan (graph.hpp:68-73).  Here every task is one (pair, root) and every lane
// of a persistent warp runs its own task.  A warp takes a contiguous chunk of
// tasks from the global queue with one atomic (chunks shrink as the queue
// drains) and hands them to its lanes; a lane that finishes takes the next one
// at once, so lanes never wait for a slow neighbour's task.
//
// The search state is bitsets over the data graph's local ids (<= 128 nodes):
// `cur` holds the candidates left at the current depth t: the vertices v of
// C[order[t]], not yet mapped, that pass the induced test of
// isValidMapping_fast_bitwise (isomorphism.hpp:268-288) against every earlier
// depth i (v in row(f_i) iff query vertex order[i] is in the row of order[t]).
// The test is evaluated in two parts: C is intersected with the rows of the
// nodes mapped at the query-adjacent earlier depths (usually one or two), and
// each surviving candidate v is kept iff every mapped node whose row contains
// v (v's in-row, intersected with the mapped set) sits at one of those depths.
// On molecular graphs (degree <= 4) that is a few independent 16-byte loads per
// level.  The last depth is never expanded: its candidates are counted with one
// popcount.  `cur` lives in registers; the per-thread stack (interleaved local
// memory) is touched only on descend and backtrack.
//
// EXACT semantics count every injective induced embedding.  REFERENCE_DFS
// (literal) restates the reference DFS: a frame never clears the visited bit of
// a candidate it moves past, and an exhausted frame clears the bit of mapping[k]
// (the last value written at depth k in this root's search, nothing before the
// first write) — isomorphism.hpp:414-448, with mapping[] reset per root.
#include "device_common.cuh"

namespace bms {
namespace {

struct Lane {
  bool active;
  bool done_fetching;
  uint32_t rec, n, qoff;
  const uint64_t* crow;  // candidate rows of the pair
  const uint64_t* arow;  // out-rows of the data graph
  const uint64_t* irow;  // in-rows of the data graph
  const uint8_t* perm;
  const uint64_t* dadj;
  int t;
  B128 cur;       // candidates left at depth t
  B128 mapped;    // nodes mapped at depths < t
  B128 vis;       // REFERENCE_DFS: the reference's visited bitset
  uint64_t mpset; // REFERENCE_DFS: depths whose mapping[] has been written
  unsigned long long cnt, exps;
  uint32_t since_check;
};

__device__ __forceinline__ B128 compute_level(const Lane& L, uint32_t j, const uint8_t* f, bool literal) {
  B128 c = ld_b128(L.crow + 2 * uint64_t(L.perm[j]));
  if (!literal) c = b_andn(c, L.mapped);
  B128 pset{0, 0};
  for (uint64_t pm = L.dadj[j]; pm; pm &= pm - 1) {
    const uint32_t x = f[__ffsll((long long)pm) - 1];
    c = b_and(c, ld_b128(L.arow + 2 * uint64_t(x)));
    pset = b_or(pset, b_bit(x));
  }
  B128 res{0, 0};
  for (B128 r = c; b_any(r); r = b_clear_low(r)) {
    const uint32_t v = b_low(r);
    const B128 bad = b_andn(b_and(ld_b128(L.irow + 2 * uint64_t(v)), L.mapped), pset);
    if (!b_any(bad)) res = b_or(res, b_bit(v));
  }
  return res;
}

__device__ __forceinline__ void finish(Lane& L, const JoinArgs& a, const uint32_t* expd) {
  if (L.cnt) atomicAdd(&a.pair_count[L.rec], L.cnt);
  if (L.exps) atomicAdd(&a.pair_exp[L.rec], L.exps);
  if (a.find_first && L.cnt) atomicOr(&a.pair_flag[L.rec], 1u);
  if (a.vertex_exp)
    for (uint32_t t = 0; t < L.n; ++t)
      if (expd[t]) atomicAdd(&a.vertex_exp[L.qoff + L.perm[t]], (unsigned long long)expd[t]);
  L.active = false;
}

// One DFS step of an active lane.
__device__ __forceinline__ void step(Lane& L, const JoinArgs& a, uint8_t* f, uint8_t* mp, B128* F, uint32_t* expd) {
  const int t = L.t;
  if (!b_any(L.cur)) {  // frame t exhausted
    if (a.literal && ((L.mpset >> t) & 1ull)) L.vis = b_andn(L.vis, b_bit(mp[t]));
    if (t == 0) {
      finish(L, a, expd);
      return;
    }
    L.t = t - 1;
    L.cur = F[t - 1];
    L.mapped = b_andn(L.mapped, b_bit(f[t - 1]));  // back in frame t-1: its node leaves the path
    return;
  }
  const uint32_t v = b_low(L.cur);
  L.cur = b_clear_low(L.cur);
  if (a.literal) {
    if (b_has(L.vis, v)) return;
    mp[t] = uint8_t(v);
    L.mpset |= uint64_t(1) << t;
    L.vis = b_or(L.vis, b_bit(v));
  }
  f[t] = uint8_t(v);
  L.mapped = b_or(L.mapped, b_bit(v));
  L.exps += 1;
  if (a.vertex_exp) expd[t] += 1;
  const B128 nf = compute_level(L, uint32_t(t) + 1, f, a.literal);
  if (uint32_t(t) + 2 == L.n) {
    // depth n-1 is the leaf level: count it without expanding
    const uint32_t last = L.n - 1;
    B128 acc = nf;
    if (a.literal) acc = b_andn(nf, L.vis);
    const uint32_t pc = b_pop(acc);
    L.cnt += pc;
    L.exps += pc;
    if (a.vertex_exp) expd[last] += pc;
    if (a.literal && pc) {
      L.vis = b_or(L.vis, acc);
      mp[last] = uint8_t(b_high(acc));
      L.mpset |= uint64_t(1) << last;
    }
    if (a.find_first && pc) {
      finish(L, a, expd);
      return;
    }
    if (a.literal && ((L.mpset >> last) & 1ull)) L.vis = b_andn(L.vis, b_bit(mp[last]));  // frame n-1 exhausted
    L.mapped = b_andn(L.mapped, b_bit(v));  // frame t moves on
  } else {
    F[t] = L.cur;
    L.t = t + 1;
    L.cur = nf;
  }
  if (a.budget && L.exps > a.budget) {
    atomicOr(&a.pair_flag[L.rec], 2u);
    finish(L, a, expd);
    return;
  }
  if (a.find_first && ++L.since_check >= 64) {
    L.since_check = 0;
    if (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u) finish(L, a, expd);
  }
}

__global__ void __launch_bounds__(256) join_kernel(JoinArgs a) {
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const unsigned long long ntasks = min((unsigned long long)a.task_cap, a.ctr->tasks);
  const unsigned long long nwarps = (unsigned long long)(gridDim.x * blockDim.x) >> 5;
  Lane L;
  L.active = false;
  L.done_fetching = false;
  uint8_t f[kMaxQueryNodes], mp[kMaxQueryNodes];
  B128 F[kMaxQueryNodes];
  uint32_t expd[kMaxQueryNodes];
  unsigned long long qbase = 0, qend = 0;  // this warp's chunk of the task queue (warp-uniform)
  bool queue_empty = false;
  for (;;) {
    uint32_t need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    while (need) {
      if (qbase >= qend) {
        if (queue_empty) break;
        unsigned long long base = 0, chunk = 0;
        if (lane == 0) {
          const unsigned long long head = *(volatile const unsigned long long*)&a.ctr->task_fetch;
          const unsigned long long left = head < ntasks ? ntasks - head : 0;
          chunk = left / (4 * nwarps);
          chunk = chunk < 32 ? 32 : (chunk > 256 ? 256 : chunk);
          base = atomicAdd(&a.ctr->task_fetch, chunk);
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        qbase = base < ntasks ? base : ntasks;
        qend = base + chunk < ntasks ? base + chunk : ntasks;
        if (qbase >= qend) {
          queue_empty = true;
          break;
        }
      }
      const unsigned long long avail = qend - qbase;
      const uint32_t rank = __popc(need & lt_mask);
      const bool mine = ((need >> lane) & 1u) && rank < avail;
      const uint32_t took = uint64_t(__popc(need)) < avail ? uint32_t(__popc(need)) : uint32_t(avail);
      if (mine) {
        const Task tk = a.tasks[qbase + rank];
        const PairRec r = a.recs[tk.pair];
        L.rec = tk.pair;
        L.qoff = a.q.goff[r.q];
        L.n = a.q.goff[r.q + 1] - L.qoff;
        L.crow = a.arena + 2 * uint64_t(r.c_row);
        L.arow = a.ds.adj + 2 * uint64_t(a.d.goff[r.d]);
        L.irow = a.ds.adjin + 2 * uint64_t(a.d.goff[r.d]);
        L.perm = a.o.perm + uint64_t(r.q) * kMaxQueryNodes;
        L.dadj = a.o.dadj + uint64_t(r.q) * kMaxQueryNodes;
        L.cnt = 0;
        L.exps = 0;
        L.since_check = 0;
        L.t = 0;
        L.cur = b_bit(tk.root);
        L.mapped = B128{0, 0};
        L.vis = B128{0, 0};
        L.mpset = 0;
        L.active = true;
        if (a.vertex_exp)
          for (uint32_t t = 0; t < L.n; ++t) expd[t] = 0;
        if (a.find_first && (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u)) finish(L, a, expd);
      }
      qbase += took;
      need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    }
    if (queue_empty && !L.active) L.done_fetching = true;
    if (__all_sync(0xffffffffu, !L.active && L.done_fetching)) break;
    for (int s = 0; s < a.steps; ++s) {
      if (L.active) step(L, a, f, mp, F, expd);
      if (__any_sync(0xffffffffu, !L.active && !L.done_fetching)) break;
    }
  }
}

}  // namespace

cudaError_t launch_join(const JoinArgs& a, int blocks, int threads, cudaStream_t st) {
  join_kernel<<<blocks, threads, 0, st>>>(a); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
