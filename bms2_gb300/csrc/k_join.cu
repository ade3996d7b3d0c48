// Persistent, work-stealing DFS join.
//
// Replaces join::joinCandidates / JoinCandidates3Optimized (isomorphism.hpp:
// 291-472).  The reference gives a sub-group one (query, data graph) pair;
// lanes stride over root candidates, select each candidate by rank with an
// O(words) scan (candidates.hpp:128-158) and test adjacency with a linear CSR
// scan (graph.hpp:68-73).  Here every task is one (pair, root) and every lane
// of a persistent warp runs its own task; a lane that finishes takes the next
// task with one warp-aggregated atomic on a global head, so there is no
// per-workgroup chunking and long tasks never hold idle neighbours hostage.
// The search state is bitsets over the data graph's local ids (<= 128 nodes):
//   F[t]   candidates left at depth t: the vertices v of C[order[t]] not yet
//          mapped that satisfy the induced test of isValidMapping_fast_bitwise
//          (isomorphism.hpp:268-288) against every earlier depth i, i.e.
//          v in row(f_i) iff query vertex order[i] is in the row of order[t].
// The test is evaluated in two parts: C is intersected with the rows of the
// nodes mapped at the query-adjacent earlier depths (usually one or two), and
// each surviving candidate v is kept iff every mapped node whose row contains
// v (v's in-row, intersected with the mapped set) sits at one of those
// depths.  On molecular graphs (degree <= 4) that is a handful of independent
// 16-byte loads per level instead of one dependent load per earlier depth.
// The last depth is never expanded: its candidates are counted with one
// popcount.  Stacks live in per-thread local memory, interleaved per lane.
//
// EXACT semantics count every injective induced embedding.  REFERENCE_DFS
// (literal) restates the reference DFS: a frame never clears the visited bit of
// a candidate it moves past, and an exhausted frame clears the bit of mapping[k]
// (the last value written at depth k, NULL before the first write) —
// isomorphism.hpp:414-448, with mapping[] reset per root.
#include "device_common.cuh"

namespace bms {
namespace {

constexpr uint8_t kNull8 = 0xFF;

struct Lane {
  bool active;
  bool done_fetching;
  uint32_t rec, n, qoff;
  const uint64_t* crow;
  const uint64_t* arow;  // out-rows of the data graph
  const uint64_t* irow;  // in-rows of the data graph
  const uint8_t* perm;
  const uint64_t* dadj;
  int t;
  B128 mapped;  // nodes mapped at depths 0..t-1 of the current path
  B128 vis;     // REFERENCE_DFS: the reference's visited bitset
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
  atomicAdd(&a.pair_exp[L.rec], L.exps);
  if (a.find_first && L.cnt) atomicOr(&a.pair_flag[L.rec], 1u);
  if (a.vertex_exp)
    for (uint32_t t = 0; t < L.n; ++t)
      if (expd[t]) atomicAdd(&a.vertex_exp[L.qoff + L.perm[t]], (unsigned long long)expd[t]);
  L.active = false;
}

// Leaf depth n-1 reached with candidate set nf.  Returns true if the task ends
// (find-first hit).
__device__ __forceinline__ bool leaf(Lane& L, const JoinArgs& a, B128 nf, uint8_t* mp, uint32_t* expd) {
  const uint32_t last = L.n - 1;
  if (!a.literal) {
    const uint32_t pc = b_pop(nf);
    L.cnt += pc;
    L.exps += pc;
    if (a.vertex_exp) expd[last] += pc;
    return a.find_first && pc;
  }
  const B128 acc = b_andn(nf, L.vis);
  const uint32_t pc = b_pop(acc);
  L.cnt += pc;
  L.exps += pc;
  if (a.vertex_exp) expd[last] += pc;
  if (pc) {
    L.vis = b_or(L.vis, acc);
    mp[last] = uint8_t(b_high(acc));
  }
  if (a.find_first && pc) return true;
  if (mp[last] != kNull8) L.vis = b_andn(L.vis, b_bit(mp[last]));  // frame n-1 exhausted
  return false;
}

__global__ void __launch_bounds__(256) join_kernel(JoinArgs a) {
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const unsigned long long ntasks = min((unsigned long long)a.task_cap, a.ctr->tasks);
  Lane L;
  L.active = false;
  L.done_fetching = false;
  L.cnt = L.exps = 0;
  uint8_t f[kMaxQueryNodes], mp[kMaxQueryNodes];
  B128 F[kMaxQueryNodes];
  uint32_t expd[kMaxQueryNodes];
  for (;;) {
    const uint32_t need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (int(lane) == leader) base = atomicAdd(&a.ctr->task_fetch, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!L.active && !L.done_fetching) {
        const unsigned long long my = base + __popc(need & lt_mask);
        if (my >= ntasks) {
          L.done_fetching = true;
        } else {
          const Task tk = a.tasks[my];
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
          L.exps = 1;
          L.since_check = 0;
          L.active = true;
          if (a.vertex_exp)
            for (uint32_t t = 0; t < L.n; ++t) expd[t] = t == 0 ? 1u : 0u;
          if (a.find_first && (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u)) {
            L.exps = 0;
            if (a.vertex_exp) expd[0] = 0;
            finish(L, a, expd);
          } else {
            const uint32_t root = tk.root;
            f[0] = uint8_t(root);
            mp[0] = uint8_t(root);
            for (uint32_t t = 1; t < L.n; ++t) mp[t] = kNull8;
            L.vis = b_bit(root);
            L.mapped = L.vis;
            const B128 nf = compute_level(L, 1, f, a.literal);
            if (L.n == 2) {
              leaf(L, a, nf, mp, expd);
              finish(L, a, expd);
            } else {
              L.t = 1;
              F[1] = nf;
            }
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, !L.active && L.done_fetching)) break;
    for (int s = 0; s < a.steps && L.active; ++s) {
      const int t = L.t;
      const B128 cur = F[t];
      if (!b_any(cur)) {
        // frame t exhausted; back in frame t-1, whose node leaves the path
        if (a.literal && mp[t] != kNull8) L.vis = b_andn(L.vis, b_bit(mp[t]));
        L.t = t - 1;
        if (L.t == 0) {
          finish(L, a, expd);
          continue;
        }
        L.mapped = b_andn(L.mapped, b_bit(f[L.t]));
        continue;
      }
      const uint32_t v = b_low(cur);
      F[t] = b_clear_low(cur);
      if (a.literal) {
        if (b_has(L.vis, v)) continue;
        mp[t] = uint8_t(v);
        L.vis = b_or(L.vis, b_bit(v));
      }
      f[t] = uint8_t(v);
      L.mapped = b_or(L.mapped, b_bit(v));
      L.exps += 1;
      if (a.vertex_exp) expd[t] += 1;
      const B128 nf = compute_level(L, uint32_t(t) + 1, f, a.literal);
      if (uint32_t(t) + 1 == L.n - 1) {
        if (leaf(L, a, nf, mp, expd)) {
          finish(L, a, expd);
          continue;
        }
        L.mapped = b_andn(L.mapped, b_bit(v));  // frame t moves on
      } else {
        L.t = t + 1;
        F[t + 1] = nf;
      }
      if (a.budget && L.exps > a.budget) {
        atomicOr(&a.pair_flag[L.rec], 2u);
        finish(L, a, expd);
        continue;
      }
      if (a.find_first && ++L.since_check >= 64) {
        L.since_check = 0;
        if (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u) finish(L, a, expd);
      }
    }
  }
}

}  // namespace

cudaError_t launch_join(const JoinArgs& a, int blocks, int threads, cudaStream_t st) {
  join_kernel<<<blocks, threads, 0, st>>>(a); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
