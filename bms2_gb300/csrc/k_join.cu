// Persistent, work-stealing DFS join.
//
// Replaces join::joinCandidates / JoinCandidates3Optimized (isomorphism.hpp:
// 291-472).  The reference gives a sub-group one (query, data graph) pair;
// lanes stride over root candidates, select each candidate by rank with an
// O(words) scan (candidates.hpp:128-158) and test adjacency with a linear CSR
// scan (graph.hpp:68-73).  Here every lane of a persistent warp runs its own
// task — a whole pair, or one (pair, root) when pairs are split — and a warp
// takes a contiguous chunk of tasks from the global queue with one atomic
// (chunks shrink as the queue drains).  Idle lanes are refilled as soon as a
// few of them are waiting, so lanes never wait long for a slow neighbour.
//
// The search state is bitsets over the data graph's local ids (one 64-bit word
// for graphs of <= 64 nodes, two up to 128): `cur` holds the candidates left at
// the current depth t: the vertices v of C[order[t]], not yet mapped, that pass
// the induced test of isValidMapping_fast_bitwise (isomorphism.hpp:268-288)
// against every earlier depth i (v in row(f_i) iff query vertex order[i] is in
// the row of order[t]).  The test is evaluated in two parts: C is intersected
// with the rows of the nodes mapped at the query-adjacent earlier depths
// (usually one or two), and each surviving candidate v is kept iff every mapped
// node whose row contains v (v's in-row, intersected with the mapped set) sits
// at one of those depths.  On molecular graphs (degree <= 4) that is a few
// independent loads per level.  The last depth is never expanded: its
// candidates are counted with one popcount.  `cur` lives in registers; the
// per-thread stack (interleaved local memory) is touched only on descend and
// backtrack, and a step first pops every exhausted frame, so each step is one
// assignment.
//
// EXACT semantics count every injective induced embedding.  REFERENCE_DFS
// (literal) restates the reference DFS: a frame never clears the visited bit of
// a candidate it moves past, and an exhausted frame clears the bit of mapping[k]
// (the last value written at depth k in this root's search, nothing before the
// first write) — isomorphism.hpp:414-448, with mapping[] reset per root.  In
// that mode tasks are always (pair, root): the reference searches every root
// with a fresh visited set.
#include "device_common.cuh"

namespace bms {
namespace {

template <int W>
struct Bits {
  uint64_t w[W];
};
template <int W>
__device__ __forceinline__ Bits<W> z() {
  Bits<W> r;
#pragma unroll
  for (int i = 0; i < W; ++i) r.w[i] = 0;
  return r;
}
template <int W>
__device__ __forceinline__ Bits<W> band(Bits<W> a, Bits<W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] &= b.w[i];
  return a;
}
template <int W>
__device__ __forceinline__ Bits<W> bandn(Bits<W> a, Bits<W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] &= ~b.w[i];
  return a;
}
template <int W>
__device__ __forceinline__ Bits<W> bor(Bits<W> a, Bits<W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] |= b.w[i];
  return a;
}
template <int W>
__device__ __forceinline__ bool bany(Bits<W> a) {
  uint64_t x = 0;
#pragma unroll
  for (int i = 0; i < W; ++i) x |= a.w[i];
  return x != 0;
}
template <int W>
__device__ __forceinline__ uint32_t bpop(Bits<W> a) {
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i < W; ++i) c += __popcll(a.w[i]);
  return c;
}
template <int W>
__device__ __forceinline__ Bits<W> bbit(uint32_t v) {
  Bits<W> r = z<W>();
#pragma unroll
  for (int i = 0; i < W; ++i) r.w[i] = (v >> 6) == uint32_t(i) ? (uint64_t(1) << (v & 63u)) : 0ull;
  return r;
}
template <int W>
__device__ __forceinline__ bool bhas(Bits<W> a, uint32_t v) {
  uint64_t x = a.w[0];
  if (W > 1 && v >= 64) x = a.w[W - 1];
  return (x >> (v & 63u)) & 1u;
}
template <int W>
__device__ __forceinline__ uint32_t blow(Bits<W> a) {
  if (W == 1 || a.w[0]) return uint32_t(__ffsll((long long)a.w[0]) - 1);
  return uint32_t(64 + __ffsll((long long)a.w[W - 1]) - 1);
}
template <int W>
__device__ __forceinline__ uint32_t bhigh(Bits<W> a) {
  if (W > 1 && a.w[W - 1]) return uint32_t(127 - __clzll((long long)a.w[W - 1]));
  return uint32_t(63 - __clzll((long long)a.w[0]));
}
template <int W>
__device__ __forceinline__ Bits<W> bclear_low(Bits<W> a) {
  if (W == 1 || a.w[0]) {
    a.w[0] &= a.w[0] - 1;
  } else {
    a.w[W - 1] &= a.w[W - 1] - 1;
  }
  return a;
}
// rows are stored as two 64-bit words; a 1-word search reads the low word
template <int W>
__device__ __forceinline__ Bits<W> bload(const uint64_t* p) {
  Bits<W> r;
  if (W == 1) {
    r.w[0] = *p;
  } else {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
    r.w[0] = v.x;
    r.w[W - 1] = v.y;
  }
  return r;
}

template <int W>
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
  Bits<W> cur;     // candidates left at depth t
  Bits<W> mapped;  // nodes mapped at depths < t
  Bits<W> vis;     // REFERENCE_DFS: the reference's visited bitset
  uint64_t mpset;  // REFERENCE_DFS: depths whose mapping[] has been written
  unsigned long long cnt, exps;
  uint32_t since_check;
};

template <int W>
__device__ __forceinline__ Bits<W> compute_level(const Lane<W>& L, uint32_t j, const uint8_t* f, bool literal) {
  Bits<W> c = bload<W>(L.crow + 2 * uint64_t(L.perm[j]));
  if (!literal) c = bandn(c, L.mapped);
  Bits<W> pset = z<W>();
  for (uint64_t pm = L.dadj[j]; pm; pm &= pm - 1) {
    const uint32_t x = f[__ffsll((long long)pm) - 1];
    c = band(c, bload<W>(L.arow + 2 * uint64_t(x)));
    pset = bor(pset, bbit<W>(x));
  }
  Bits<W> res = z<W>();
  for (Bits<W> r = c; bany(r); r = bclear_low(r)) {
    const uint32_t v = blow(r);
    const Bits<W> bad = bandn(band(bload<W>(L.irow + 2 * uint64_t(v)), L.mapped), pset);
    if (!bany(bad)) res = bor(res, bbit<W>(v));
  }
  return res;
}

template <int W>
__device__ __forceinline__ void finish(Lane<W>& L, const JoinArgs& a, const uint32_t* expd) {
  if (L.cnt) atomicAdd(&a.pair_count[L.rec], L.cnt);
  if (L.exps) atomicAdd(&a.pair_exp[L.rec], L.exps);
  if (a.find_first && L.cnt) atomicOr(&a.pair_flag[L.rec], 1u);
  if (a.vertex_exp)
    for (uint32_t t = 0; t < L.n; ++t)
      if (expd[t]) atomicAdd(&a.vertex_exp[L.qoff + L.perm[t]], (unsigned long long)expd[t]);
  L.active = false;
}

// One assignment of an active lane: pop exhausted frames, take the next
// candidate, compute the next level (or count the leaf level).
template <int W>
__device__ __forceinline__ void step(Lane<W>& L, const JoinArgs& a, uint8_t* f, uint8_t* mp, Bits<W>* F,
                                     uint32_t* expd) {
  int t = L.t;
  while (!bany(L.cur)) {  // frame t exhausted
    if (a.literal && ((L.mpset >> t) & 1ull)) L.vis = bandn(L.vis, bbit<W>(mp[t]));
    if (t == 0) {
      finish(L, a, expd);
      return;
    }
    --t;
    L.cur = F[t];
    L.mapped = bandn(L.mapped, bbit<W>(f[t]));  // back in frame t: its node leaves the path
  }
  L.t = t;
  const uint32_t v = blow(L.cur);
  L.cur = bclear_low(L.cur);
  if (a.literal) {
    if (bhas(L.vis, v)) return;
    mp[t] = uint8_t(v);
    L.mpset |= uint64_t(1) << t;
    L.vis = bor(L.vis, bbit<W>(v));
  }
  f[t] = uint8_t(v);
  L.mapped = bor(L.mapped, bbit<W>(v));
  L.exps += 1;
  if (a.vertex_exp) expd[t] += 1;
  const Bits<W> nf = compute_level(L, uint32_t(t) + 1, f, a.literal);
  if (uint32_t(t) + 2 == L.n) {
    // depth n-1 is the leaf level: count it without expanding
    const uint32_t last = L.n - 1;
    Bits<W> acc = nf;
    if (a.literal) acc = bandn(nf, L.vis);
    const uint32_t pc = bpop(acc);
    L.cnt += pc;
    L.exps += pc;
    if (a.vertex_exp) expd[last] += pc;
    if (a.literal && pc) {
      L.vis = bor(L.vis, acc);
      mp[last] = uint8_t(bhigh(acc));
      L.mpset |= uint64_t(1) << last;
    }
    if (a.find_first && pc) {
      finish(L, a, expd);
      return;
    }
    if (a.literal && ((L.mpset >> last) & 1ull)) L.vis = bandn(L.vis, bbit<W>(mp[last]));  // frame n-1 exhausted
    L.mapped = bandn(L.mapped, bbit<W>(v));  // frame t moves on
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

template <int W>
__global__ void __launch_bounds__(256) join_kernel(JoinArgs a) {
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  // task range: records [0, recs_wide) need two words, the rest one word
  const unsigned long long recs = min((unsigned long long)a.rec_cap, a.ctr->recs);
  const unsigned long long wide = min(recs, a.ctr->recs_wide);
  unsigned long long first, ntasks;
  if (a.per_pair) {
    first = W == 2 ? 0 : wide;
    ntasks = W == 2 ? wide : recs - wide;
  } else {
    first = 0;
    ntasks = min((unsigned long long)a.task_cap, a.ctr->tasks);
  }
  unsigned long long* head = W == 2 ? &a.ctr->task_fetch_wide : &a.ctr->task_fetch;
  const unsigned long long nwarps = (unsigned long long)(gridDim.x * blockDim.x) >> 5;
  Lane<W> L;
  L.active = false;
  L.done_fetching = false;
  uint8_t f[kMaxQueryNodes], mp[kMaxQueryNodes];
  Bits<W> F[kMaxQueryNodes];
  uint32_t expd[kMaxQueryNodes];
  unsigned long long qbase = 0, qend = 0;  // this warp's chunk of the queue (warp-uniform)
  bool queue_empty = false;
  for (;;) {
    uint32_t need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    while (need) {
      if (qbase >= qend) {
        if (queue_empty) break;
        unsigned long long base = 0, chunk = 0;
        if (lane == 0) {
          const unsigned long long h = *(volatile const unsigned long long*)head;
          const unsigned long long left = h < ntasks ? ntasks - h : 0;
          chunk = left / (4 * nwarps);
          chunk = chunk < 32 ? 32 : (chunk > 256 ? 256 : chunk);
          base = atomicAdd(head, chunk);
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
        uint32_t rec;
        Bits<W> roots;
        bool take = true;
        if (a.per_pair) {
          rec = uint32_t(first + qbase + rank);
        } else {
          const Task tk = a.tasks[qbase + rank];
          rec = tk.pair;
          take = (rec < wide) == (W == 2);
          roots = bbit<W>(tk.root);
        }
        L.active = take;
        if (take) {
          const PairRec r = a.recs[rec];
          L.rec = rec;
          L.qoff = a.q.goff[r.q];
          L.n = a.q.goff[r.q + 1] - L.qoff;
          L.crow = a.arena + 2 * uint64_t(r.c_row);
          L.arow = a.ds.adj + 2 * uint64_t(a.d.goff[r.d]);
          L.irow = a.ds.adjin + 2 * uint64_t(a.d.goff[r.d]);
          L.perm = a.o.perm + uint64_t(r.q) * kMaxQueryNodes;
          L.dadj = a.o.dadj + uint64_t(r.q) * kMaxQueryNodes;
          if (a.per_pair) roots = bload<W>(L.crow + 2 * uint64_t(L.perm[0]));
          L.cnt = 0;
          L.exps = 0;
          L.since_check = 0;
          L.t = 0;
          L.cur = roots;
          L.mapped = z<W>();
          L.vis = z<W>();
          L.mpset = 0;
          if (a.vertex_exp)
            for (uint32_t t = 0; t < L.n; ++t) expd[t] = 0;
          if (a.find_first && (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u)) finish(L, a, expd);
        }
      }
      qbase += took;
      need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    }
    if (queue_empty && !L.active) L.done_fetching = true;
    if (__all_sync(0xffffffffu, !L.active && L.done_fetching)) break;
    for (int s = 0; s < a.steps; ++s) {
      if (L.active) step(L, a, f, mp, F, expd);
      const uint32_t idle = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
      if (__popc(idle) >= 4 || (idle && !__any_sync(0xffffffffu, L.active))) break;
    }
  }
}

}  // namespace

cudaError_t launch_join(const JoinArgs& a, int blocks, int threads, cudaStream_t st) {
  join_kernel<2><<<blocks, threads, 0, st>>>(a); note_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  join_kernel<1><<<blocks, threads, 0, st>>>(a); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
