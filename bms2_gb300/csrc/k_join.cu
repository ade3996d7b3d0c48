// Persistent, work-stealing DFS join.
//
// Replaces join::joinCandidates / JoinCandidates3Optimized (isomorphism.hpp:
// 291-472).  The reference gives a sub-group one (query, data graph) pair;
// lanes stride over root candidates, select each candidate by rank with an
// O(words) scan (candidates.hpp:128-158) and test adjacency with a linear CSR
// scan (graph.hpp:68-73).  Here every lane of a persistent warp runs its own
// task — a whole pair, or one (pair, root) when pairs are split — and a warp
// takes a contiguous chunk of tasks from the global queue with one atomic
// (chunks shrink as the queue drains).  Idle lanes are refilled once `refill`
// of them are waiting (a schedule column: refilling often keeps more lanes
// busy, refilling rarely costs fewer refills).
//
// The search state is bitsets over the data graph's local ids: one 32-bit word
// for graphs of <= 32 nodes, one 64-bit word up to 64, two up to 128 (records
// arrive grouped by these classes and each class has its own kernel).  `cur`
// holds the candidates left at the current depth t: the vertices v of
// C[order[t]], not yet mapped, that pass the induced test of
// isValidMapping_fast_bitwise (isomorphism.hpp:268-288) against every earlier
// depth i (v in row(f_i) iff query vertex order[i] is in the row of order[t]).
// C is intersected with the rows of the nodes mapped at the query-adjacent
// earlier depths (usually one or two); a surviving v must then lie in the row
// of no other mapped node.  Two ways to test that:
//  - counted (EXACT semantics, every in-degree <= 7): each lane keeps, for
//    every data node, the number of mapped nodes whose row contains it, as
//    three bit planes updated with ripple-carry adds and borrows when a node
//    is mapped or unmapped.  v passes iff its count equals the number of
//    query-adjacent earlier depths: one plane comparison for the whole level,
//    no per-candidate load.
//  - in-row (REFERENCE_DFS, or larger in-degrees): each surviving v is kept iff
//    its in-row, intersected with the mapped set, holds only nodes mapped at
//    the adjacent depths: one load per candidate.
// Each kernel reads the side's largest in-degree on the device and returns at
// once when the other variant applies, so no host round trip decides it.  The
// last depth is never expanded: its candidates are counted with one popcount.
// `cur` lives in registers; the per-thread stack (interleaved local memory) is
// touched only on descend and backtrack, and a step first pops every exhausted
// frame, so each step is one assignment.
//
// EXACT semantics count every injective induced embedding.  REFERENCE_DFS
// (literal) restates the reference DFS: a frame never clears the visited bit of
// a candidate it moves past, and an exhausted frame clears the bit of mapping[k]
// (the last value written at depth k in this root's search, nothing before the
// first write) — isomorphism.hpp:414-448, with mapping[] reset per root.  In
// that mode tasks are always (pair, root): the reference searches every root
// with a fresh visited set.
#include <type_traits>

#include "device_common.cuh"

namespace bms {
namespace {

constexpr int kPlanes = 3;  // counted test: counts 0..7

// Run modes a join kernel is compiled for (their per-step checks vanish):
// count-all, find-first, count-all with per-vertex expansion logging.
constexpr int kModeCount = 0, kModeFind = 1, kModeLog = 2;


__device__ __forceinline__ uint32_t wpop(uint32_t x) { return uint32_t(__popc(x)); }
__device__ __forceinline__ uint32_t wpop(uint64_t x) { return uint32_t(__popcll(x)); }
__device__ __forceinline__ uint32_t wlow(uint32_t x) { return uint32_t(__ffs(int(x)) - 1); }
__device__ __forceinline__ uint32_t wlow(uint64_t x) { return uint32_t(__ffsll((long long)x) - 1); }
__device__ __forceinline__ uint32_t whigh(uint32_t x) { return uint32_t(31 - __clz(int(x))); }
__device__ __forceinline__ uint32_t whigh(uint64_t x) { return uint32_t(63 - __clzll((long long)x)); }

// A set of local ids: W words of type T.
template <typename T, int W>
struct Bits {
  static constexpr uint32_t kBits = 8 * sizeof(T);
  T w[W];
};
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> z() {
  Bits<T, W> r;
#pragma unroll
  for (int i = 0; i < W; ++i) r.w[i] = 0;
  return r;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> ones() {
  Bits<T, W> r;
#pragma unroll
  for (int i = 0; i < W; ++i) r.w[i] = T(~T(0));
  return r;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> band(Bits<T, W> a, Bits<T, W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] &= b.w[i];
  return a;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bandn(Bits<T, W> a, Bits<T, W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] &= T(~b.w[i]);
  return a;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bor(Bits<T, W> a, Bits<T, W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] |= b.w[i];
  return a;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bxor(Bits<T, W> a, Bits<T, W> b) {
#pragma unroll
  for (int i = 0; i < W; ++i) a.w[i] ^= b.w[i];
  return a;
}
template <typename T, int W>
__device__ __forceinline__ bool bany(Bits<T, W> a) {
  T x = 0;
#pragma unroll
  for (int i = 0; i < W; ++i) x |= a.w[i];
  return x != 0;
}
template <typename T, int W>
__device__ __forceinline__ uint32_t bpop(Bits<T, W> a) {
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i < W; ++i) c += wpop(a.w[i]);
  return c;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bbit(uint32_t v) {
  constexpr uint32_t kB = Bits<T, W>::kBits;
  Bits<T, W> r;
#pragma unroll
  for (int i = 0; i < W; ++i) r.w[i] = v / kB == uint32_t(i) ? T(T(1) << (v % kB)) : T(0);
  return r;
}
template <typename T, int W>
__device__ __forceinline__ bool bhas(Bits<T, W> a, uint32_t v) {
  constexpr uint32_t kB = Bits<T, W>::kBits;
  T x = a.w[0];
#pragma unroll
  for (int i = 1; i < W; ++i)
    if (v / kB == uint32_t(i)) x = a.w[i];
  return (x >> (v % kB)) & 1u;
}
template <typename T, int W>
__device__ __forceinline__ uint32_t blow(Bits<T, W> a) {
  constexpr uint32_t kB = Bits<T, W>::kBits;
  uint32_t r = wlow(a.w[W - 1]) + (W - 1) * kB;
#pragma unroll
  for (int i = W - 2; i >= 0; --i)
    if (a.w[i]) r = uint32_t(i) * kB + wlow(a.w[i]);
  return r;
}
template <typename T, int W>
__device__ __forceinline__ uint32_t bhigh(Bits<T, W> a) {
  constexpr uint32_t kB = Bits<T, W>::kBits;
  uint32_t r = whigh(a.w[0]);
#pragma unroll
  for (int i = 1; i < W; ++i)
    if (a.w[i]) r = uint32_t(i) * kB + whigh(a.w[i]);
  return r;
}
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bclear_low(Bits<T, W> a) {
  bool done = false;
#pragma unroll
  for (int i = 0; i < W; ++i) {
    if (!done && a.w[i]) {
      a.w[i] &= a.w[i] - 1;
      done = true;
    }
  }
  return a;
}
// Rows are stored as two 64-bit words (little-endian); a search reads as many
// of its words as its set holds: 32, 64 or 128 bits, in 32- or 64-bit words.
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bload(const uint64_t* p) {
  static_assert(sizeof(T) * 8 * W <= 128, "rows hold 128 bits");
  Bits<T, W> r;
  if constexpr (sizeof(T) * 8 * W == 32) {
    r.w[0] = T(__ldg(reinterpret_cast<const unsigned int*>(p)));
  } else if constexpr (sizeof(T) * 8 * W == 64) {
    const unsigned long long x = __ldg(reinterpret_cast<const unsigned long long*>(p));
    if constexpr (W == 1) {
      r.w[0] = T(x);
    } else {
      r.w[0] = T(uint32_t(x));
      r.w[1] = T(uint32_t(x >> 32));
    }
  } else {
    const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p));
    if constexpr (W == 2) {
      r.w[0] = T(v.x);
      r.w[1] = T(v.y);
    } else {
      r.w[0] = T(uint32_t(v.x));
      r.w[1] = T(uint32_t(v.x >> 32));
      r.w[2] = T(uint32_t(v.y));
      r.w[3] = T(uint32_t(v.y >> 32));
    }
  }
  return r;
}
// A set given as its low and high 64 bits (subtree records).
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bfrom64(uint64_t lo, uint64_t hi) {
  Bits<T, W> r;
  if constexpr (sizeof(T) == 8) {
    r.w[0] = T(lo);
    if constexpr (W == 2) r.w[1] = T(hi);
  } else {
    r.w[0] = T(uint32_t(lo));
    if constexpr (W >= 2) r.w[1] = T(uint32_t(lo >> 32));
    if constexpr (W == 4) {
      r.w[2] = T(uint32_t(hi));
      r.w[3] = T(uint32_t(hi >> 32));
    }
  }
  return r;
}
// The members of `a` whose rank (0 = lowest) is g modulo 2^lg: lane g of a
// group of 2^lg lanes searching one pair takes these roots.
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> bstride(Bits<T, W> a, uint32_t g, uint32_t lg) {
  if (lg == 0) return a;
  const uint32_t mask = (1u << lg) - 1u;
  Bits<T, W> r = z<T, W>();
  uint32_t k = 0;
  for (; bany(a); a = bclear_low(a), ++k)
    if ((k & mask) == g) r = bor(r, bbit<T, W>(blow(a)));
  return r;
}

// Per-node counts of mapped in-neighbours as kPlanes bit planes.
template <typename T, int W>
struct Planes {
  Bits<T, W> p[kPlanes];
};
template <typename T, int W>
__device__ __forceinline__ void padd(Planes<T, W>& P, Bits<T, W> carry) {
#pragma unroll
  for (int b = 0; b < kPlanes; ++b) {
    const Bits<T, W> nc = band(P.p[b], carry);
    P.p[b] = bxor(P.p[b], carry);
    carry = nc;
  }
}
template <typename T, int W>
__device__ __forceinline__ void psub(Planes<T, W>& P, Bits<T, W> borrow) {
#pragma unroll
  for (int b = 0; b < kPlanes; ++b) {
    const Bits<T, W> nb = bandn(borrow, P.p[b]);
    P.p[b] = bxor(P.p[b], borrow);
    borrow = nb;
  }
}
// nodes whose count plus their bit in `add` equals k (k < 2^kPlanes): the
// sum is formed plane by plane (ripple carry) without storing it
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> peq_added(const Planes<T, W>& P, Bits<T, W> carry, uint32_t k) {
  Bits<T, W> m = ones<T, W>();
#pragma unroll
  for (int b = 0; b < kPlanes; ++b) {
    const Bits<T, W> sum = bxor(P.p[b], carry);
    carry = band(P.p[b], carry);
    m = ((k >> b) & 1u) ? band(m, sum) : bandn(m, sum);
  }
  return m;
}

template <typename T, int W>
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
  int base;           // depth the task starts at (a subtree's prefix length)
  bool no_split;      // the subtree buffer was full: keep the work
  Bits<T, W> cur;     // candidates left at depth t
  Bits<T, W> mapped;  // nodes mapped at depths < t
  Bits<T, W> vis;     // REFERENCE_DFS: the reference's visited bitset
  Planes<T, W> P;     // counted test: mapped in-neighbour counts
  uint64_t mpset;     // REFERENCE_DFS: depths whose mapping[] has been written
  unsigned long long cnt, exps;
  uint32_t since_check;
};

// Per-thread stacks, indexed by depth.
template <typename T, int W>
struct Stack {
  uint8_t f[kMaxQueryNodes];         // node mapped at each depth
  uint8_t mp[kMaxQueryNodes];        // REFERENCE_DFS: mapping[] as the reference writes it
  Bits<T, W> F[kMaxQueryNodes];      // candidates left in each frame
  uint32_t expd[kMaxQueryNodes];     // per-depth expansions (logging)
};

template <typename T, int W, int kMode>
__device__ __forceinline__ void finish(Lane<T, W>& L, const JoinArgs& a, const uint32_t* expd) {
  constexpr bool kFindFirst = kMode == kModeFind, kLogVertices = kMode == kModeLog;
  if (L.cnt) atomicAdd(&a.pair_count[L.rec], L.cnt);
  if (L.exps) atomicAdd(&a.pair_exp[L.rec], L.exps);
  if (kFindFirst && L.cnt) atomicOr(&a.pair_flag[L.rec], 1u);
  if (kLogVertices)
    for (uint32_t t = 0; t < L.n; ++t)
      if (expd[t]) atomicAdd(&a.vertex_exp[L.qoff + L.perm[t]], (unsigned long long)expd[t]);
  L.active = false;
}

// Hand every unexplored subtree of the search to the next round: frame i in
// [base, t) still holds F[i], frame t holds cur; each candidate left in them
// becomes its own SubTask with the prefix f[0..i), so the next round spreads
// the search over as many lanes as it has branches.  Returns false (and keeps
// the work) when the buffer has no room.
template <typename T, int W>
__device__ bool split(Lane<T, W>& L, const JoinArgs& a, const Stack<T, W>& S) {
  uint32_t m = bpop(L.cur);
  for (int i = L.base; i < L.t; ++i) m += bpop(S.F[i]);
  if (m == 0) return false;  // nothing left: the next step finishes
  SubTask* out = a.sub[(a.round + 1) & 1];
  const unsigned long long b = atomicAdd(&a.ctr->sub_n[a.round + 1], (unsigned long long)m);
  if (b + m > a.sub_cap) {
    for (unsigned long long k = b; k < a.sub_cap && k < b + m; ++k) out[k].rec = kNoRecord;
    return false;
  }
  unsigned long long k = b;
  for (int i = L.base; i <= L.t; ++i) {
    for (Bits<T, W> c = i < L.t ? S.F[i] : L.cur; bany(c); c = bclear_low(c)) {
      const uint32_t v = blow(c);
      SubTask& o = out[k++];
      o.rec = L.rec;
      o.depth = uint32_t(i);
      o.cand[0] = v < 64 ? uint64_t(1) << v : 0ull;
      o.cand[1] = v >= 64 ? uint64_t(1) << (v - 64) : 0ull;
      for (int j = 0; j < i; ++j) o.f[j] = S.f[j];
    }
  }
  return true;
}

template <typename T, int W, int kMode>
__device__ __forceinline__ bool after_step(Lane<T, W>& L, const JoinArgs& a, const Stack<T, W>& S) {
  constexpr bool kFindFirst = kMode == kModeFind;
  const uint32_t* expd = S.expd;
  if (a.budget && L.exps > a.budget) {
    atomicOr(&a.pair_flag[L.rec], 2u);
    finish<T, W, kMode>(L, a, expd);
    return false;
  }
  if (a.split_budget && L.exps >= a.split_budget && !L.no_split) {
    if (split(L, a, S)) {
      finish<T, W, kMode>(L, a, expd);
      return false;
    }
    L.no_split = true;
  }
  if (kFindFirst && ++L.since_check >= 64) {
    L.since_check = 0;
    if (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u) {
      finish<T, W, kMode>(L, a, expd);
      return false;
    }
  }
  return true;
}

// ----------------------------------------------------------- counted test
// One assignment: pop exhausted frames, take the next candidate v of depth t,
// compute depth t+1 with v mapped; count it when it is the leaf level, else
// push.  Leaf and dead-end steps write no stack state.
template <typename T, int W, int kMode>
__device__ __forceinline__ void step_counted(Lane<T, W>& L, const JoinArgs& a, Stack<T, W>& S) {
  constexpr bool kFindFirst = kMode == kModeFind, kLogVertices = kMode == kModeLog;
  int t = L.t;
  while (!bany(L.cur)) {  // frame t exhausted
    if (t == L.base) {
      finish<T, W, kMode>(L, a, S.expd);
      return;
    }
    --t;
    L.cur = S.F[t];
    L.mapped = bandn(L.mapped, bbit<T, W>(S.f[t]));  // back in frame t: its node leaves the path
    psub(L.P, bload<T, W>(L.arow + 2 * uint64_t(S.f[t])));
  }
  L.t = t;
  const uint32_t v = blow(L.cur);
  L.cur = bclear_low(L.cur);
  const uint32_t j = uint32_t(t) + 1;
  const Bits<T, W> row = bload<T, W>(L.arow + 2 * uint64_t(v));
  const uint64_t dm = __ldg(reinterpret_cast<const unsigned long long*>(L.dadj) + j);
  Bits<T, W> c = bload<T, W>(L.crow + 2 * uint64_t(__ldg(L.perm + j)));
  const Bits<T, W> mapped = bor(L.mapped, bbit<T, W>(v));
  c = bandn(c, mapped);
  if ((dm >> t) & 1ull) c = band(c, row);
  for (uint64_t pm = dm & ~(uint64_t(1) << t); pm; pm &= pm - 1)
    c = band(c, bload<T, W>(L.arow + 2 * uint64_t(S.f[__ffsll((long long)pm) - 1])));
  const uint32_t k = uint32_t(__popcll(dm));
  c = k < (1u << kPlanes) ? band(c, peq_added(L.P, row, k)) : z<T, W>();
  L.exps += 1;
  if (kLogVertices) S.expd[t] += 1;
  if (j + 1 == L.n) {  // depth j is the leaf level: count it without expanding
    const uint32_t pc = bpop(c);
    L.cnt += pc;
    L.exps += pc;
    if (kLogVertices) S.expd[j] += pc;
    if (kFindFirst && pc) {
      finish<T, W, kMode>(L, a, S.expd);
      return;
    }
  } else if (bany(c)) {
    S.F[t] = L.cur;
    S.f[t] = uint8_t(v);
    padd(L.P, row);
    L.mapped = mapped;
    L.t = int(j);
    L.cur = c;
  }
  after_step<T, W, kMode>(L, a, S);
}

// ----------------------------------------------------------- in-row test
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> compute_level(const Lane<T, W>& L, uint32_t j, const uint8_t* f, bool literal) {
  Bits<T, W> c = bload<T, W>(L.crow + 2 * uint64_t(__ldg(L.perm + j)));
  if (!literal) c = bandn(c, L.mapped);
  const uint64_t adj = __ldg(reinterpret_cast<const unsigned long long*>(L.dadj) + j);
  Bits<T, W> pset = z<T, W>();
  for (uint64_t pm = adj; pm; pm &= pm - 1) {
    const uint32_t x = f[__ffsll((long long)pm) - 1];
    c = band(c, bload<T, W>(L.arow + 2 * uint64_t(x)));
    pset = bor(pset, bbit<T, W>(x));
  }
  // images of the earlier non-neighbours: EXACT paths are injective (mapped
  // minus pset); a literal path can hold a node twice (a stale clear unmarks a
  // path node), so it collects them position by position
  Bits<T, W> nset = bandn(L.mapped, pset);
  if (literal) {
    nset = z<T, W>();
    for (uint64_t nm = ~adj & ((uint64_t(1) << j) - 1); nm; nm &= nm - 1)
      nset = bor(nset, bbit<T, W>(f[__ffsll((long long)nm) - 1]));
  }
  Bits<T, W> res = z<T, W>();
  for (Bits<T, W> r = c; bany(r); r = bclear_low(r)) {
    const uint32_t v = blow(r);
    if (!bany(band(bload<T, W>(L.irow + 2 * uint64_t(v)), nset))) res = bor(res, bbit<T, W>(v));
  }
  return res;
}

template <typename T, int W, int kMode>
__device__ __forceinline__ void step_inrow(Lane<T, W>& L, const JoinArgs& a, Stack<T, W>& S) {
  constexpr bool kFindFirst = kMode == kModeFind, kLogVertices = kMode == kModeLog;
  int t = L.t;
  while (!bany(L.cur)) {  // frame t exhausted
    if (a.literal && ((L.mpset >> t) & 1ull)) L.vis = bandn(L.vis, bbit<T, W>(S.mp[t]));
    if (t == L.base) {
      finish<T, W, kMode>(L, a, S.expd);
      return;
    }
    --t;
    L.cur = S.F[t];
    L.mapped = bandn(L.mapped, bbit<T, W>(S.f[t]));  // back in frame t: its node leaves the path
  }
  L.t = t;
  const uint32_t v = blow(L.cur);
  L.cur = bclear_low(L.cur);
  if (a.literal) {
    if (bhas(L.vis, v)) return;
    S.mp[t] = uint8_t(v);
    L.mpset |= uint64_t(1) << t;
    L.vis = bor(L.vis, bbit<T, W>(v));
  }
  S.f[t] = uint8_t(v);
  L.mapped = bor(L.mapped, bbit<T, W>(v));
  L.exps += 1;
  if (kLogVertices) S.expd[t] += 1;
  const Bits<T, W> nf = compute_level(L, uint32_t(t) + 1, S.f, a.literal);
  if (uint32_t(t) + 2 == L.n) {
    // depth n-1 is the leaf level: count it without expanding
    const uint32_t last = L.n - 1;
    Bits<T, W> acc = nf;
    if (a.literal) acc = bandn(nf, L.vis);
    const uint32_t pc = bpop(acc);
    L.cnt += pc;
    L.exps += pc;
    if (kLogVertices) S.expd[last] += pc;
    if (a.literal && pc) {
      L.vis = bor(L.vis, acc);
      S.mp[last] = uint8_t(bhigh(acc));
      L.mpset |= uint64_t(1) << last;
    }
    if (kFindFirst && pc) {
      finish<T, W, kMode>(L, a, S.expd);
      return;
    }
    if (a.literal && ((L.mpset >> last) & 1ull)) L.vis = bandn(L.vis, bbit<T, W>(S.mp[last]));  // frame n-1 exhausted
    L.mapped = bandn(L.mapped, bbit<T, W>(v));  // frame t moves on
  } else {
    S.F[t] = L.cur;
    L.t = t + 1;
    L.cur = nf;
  }
  after_step<T, W, kMode>(L, a, S);
}

// ----------------------------------------------------------- clustered join
// The clustered join, EXACT semantics (the reference driver's --use-cs,
// BMS2.cpp:218-296): joinPartialCandidates2 (isomorphism.hpp:1021-1178) finds
// the prototype's matches, joinWithPartialMatches (:756-977) extends each with
// every query of its data graph's GMCR row.  Here round 0 of the join is
//   cs_enum_kernel: one warp per data graph; its lanes enumerate the matches
//     of query 0 over its own candidate rows (each lane a share of the roots)
//     and write one entry per (match, run of up to kCsMembers members) into
//     the array of the graph's size class;
//   cs_extend_kernel<K>: the class's entries by work stealing; the members of
//     a warp's current entry go to its idle lanes as consecutive items, each
//     lane builds the match's prefix state and starts its member with the
//     steps, refills and splits of the plain join (a member of the prototype's
//     size counts one, a smaller one nothing).
// Later rounds run the subtrees that long searches handed over, as for the
// plain join.

// EXACT candidates at depth j (plain order) given the path f[0..j-1] = `mapped`.
template <typename T, int W>
__device__ __forceinline__ Bits<T, W> cs_level(const uint64_t* crow, const uint64_t* dadj, const uint64_t* arow,
                                               const uint64_t* irow, uint32_t j, const uint8_t* f, Bits<T, W> mapped) {
  Bits<T, W> c = bandn(bload<T, W>(crow + 2 * uint64_t(j)), mapped);
  Bits<T, W> pset = z<T, W>();
  for (uint64_t pm = __ldg(reinterpret_cast<const unsigned long long*>(dadj) + j); pm; pm &= pm - 1) {
    const uint32_t x = f[__ffsll((long long)pm) - 1];
    c = band(c, bload<T, W>(arow + 2 * uint64_t(x)));
    pset = bor(pset, bbit<T, W>(x));
  }
  const Bits<T, W> nset = bandn(mapped, pset);
  Bits<T, W> res = z<T, W>();
  for (Bits<T, W> r = c; bany(r); r = bclear_low(r)) {
    const uint32_t v = blow(r);
    if (!bany(band(bload<T, W>(irow + 2 * uint64_t(v)), nset))) res = bor(res, bbit<T, W>(v));
  }
  return res;
}

// A lane's enumeration of prototype matches.
template <typename T, int W>
struct CsEnum {
  Bits<T, W> roots;   // roots not started yet
  Bits<T, W> mapped;  // path nodes below the current depth
  int t;              // current depth, -1: start the next root
  bool done;
  uint8_t f[kMaxQueryNodes];
  Bits<T, W> F[kMaxQueryNodes];
};

// The next match into e.f[0..end-1]; false when the lane's roots are exhausted.
template <typename T, int W>
__device__ bool cs_next(CsEnum<T, W>& e, uint32_t end, const uint64_t* crow, const uint64_t* dadj,
                        const uint64_t* arow, const uint64_t* irow, unsigned long long& exps) {
  for (;;) {
    if (e.t < 0) {
      if (!bany(e.roots)) return false;
      const uint32_t v0 = blow(e.roots);
      e.roots = bclear_low(e.roots);
      e.f[0] = uint8_t(v0);
      ++exps;
      if (end == 1) return true;
      e.mapped = bbit<T, W>(v0);
      e.F[1] = cs_level<T, W>(crow, dadj, arow, irow, 1, e.f, e.mapped);
      e.t = 1;
    }
    int t = e.t;
    if (!bany(e.F[t])) {  // frame t exhausted
      if (t == 1) {
        e.t = -1;
        continue;
      }
      e.t = --t;
      e.mapped = bandn(e.mapped, bbit<T, W>(e.f[t]));
      continue;
    }
    const uint32_t v = blow(e.F[t]);
    e.F[t] = bclear_low(e.F[t]);
    e.f[t] = uint8_t(v);
    ++exps;
    if (uint32_t(t) + 1 == end) return true;
    e.mapped = bor(e.mapped, bbit<T, W>(v));
    e.F[t + 1] = cs_level<T, W>(crow, dadj, arow, irow, uint32_t(t) + 1, e.f, e.mapped);
    e.t = t + 1;
  }
}

__global__ void __launch_bounds__(256) cs_enum_kernel(JoinArgs a) {
  using T = uint64_t;
  constexpr int W = 2;
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t end = a.cs_end, D = a.d.G;
  CsEnum<T, W> E;
  unsigned long long parts = 0, pexps = 0;
  for (;;) {
    uint32_t i = 0;
    if (lane == 0) i = atomicAdd(&a.ctr->cs_ghead, 1u);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= D) break;
    const uint32_t d = a.dperm[i];
    const uint32_t d_start = a.d.goff[d], m = a.d.goff[d + 1] - d_start;
    const uint32_t g0 = a.gmcr_off[d], vcount = a.gmcr_off[d + 1] - g0;
    if (m == 0) continue;
    const uint64_t* crow_p = nullptr;
    B128 roots;
    if (end == 1) {
      roots = prototype_row(a.qs.frec, a.ds.frec, a.ds.R, a.dense, a.dense_w, a.q.goff[0], d_start, m);
      if (vcount == 0) {  // nothing to extend: only the matches are counted
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
    const int cls = m > 64 ? 2 : (m > 32 ? 1 : 0);
    const uint32_t nchunk = (vcount + kCsMembers - 1) / kCsMembers;
    uint8_t* out = a.cs_ent[cls];
    const uint64_t* arow = a.ds.adj + 2 * uint64_t(d_start);
    const uint64_t* irow = a.ds.adjin + 2 * uint64_t(d_start);
    E.roots = z<T, W>();
    {  // this lane's roots: every 32nd set bit from its rank on
      uint32_t k = 0;
      for (B128 r = roots; b_any(r); r = b_clear_low(r), ++k)
        if ((k & 31u) == lane) E.roots = bor(E.roots, bbit<T, W>(b_low(r)));
    }
    E.t = -1;
    E.done = !bany(E.roots);
    while (!__all_sync(0xffffffffu, E.done)) {
      bool got = false;
      if (!E.done) {
        got = cs_next<T, W>(E, end, crow_p, a.o.dadj, arow, irow, pexps);
        E.done = !got;
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, got);
      if (!bal) continue;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&a.ctr->cs_n[cls], (unsigned long long)__popc(bal) * nchunk);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (got) {
        ++parts;
        const unsigned long long k0 = base + (unsigned long long)__popc(bal & lt_mask) * nchunk;
        for (uint32_t c = 0; c < nchunk; ++c) {
          if (k0 + c >= a.cs_cap) {
            atomicOr(a.err, kErrOverflow);
            break;
          }
          uint8_t* e = out + (k0 + c) * a.cs_stride;
          *reinterpret_cast<CsEntry*>(e) = CsEntry{d, c * kCsMembers};
          for (uint32_t t = 0; t < end; ++t) e[sizeof(CsEntry) + t] = E.f[t];
        }
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

// The prefix state of a match at depth `end` (S.f, counting planes,
// mapped).  Built by every lane that starts a member of the entry; lanes of a
// warp take consecutive members of the same entry, so they load the same rows.
template <typename T, int W, bool kCounted>
__device__ __forceinline__ void cs_prefix(Lane<T, W>& L, Stack<T, W>& S, uint32_t end, const uint8_t* pre,
                                          const uint64_t* arow) {
  L.mapped = z<T, W>();
#pragma unroll
  for (int b = 0; b < kPlanes; ++b) L.P.p[b] = z<T, W>();
  for (uint32_t j = 0; j < end; ++j) {
    const uint32_t x = pre[j];
    S.f[j] = uint8_t(x);
    L.mapped = bor(L.mapped, bbit<T, W>(x));
    if constexpr (kCounted) {
      const Bits<T, W> row = bload<T, W>(arow + 2 * uint64_t(x));
      padd(L.P, row);
    }
  }
}

// Member j of the graph's GMCR row against the entry's match: a query of the
// prototype's size counts one; otherwise depth `end` is computed with the
// lane's test and, when it holds candidates, the lane starts the search there
// (a leaf-level depth `end` is counted at once).  `held` is the entry whose
// prefix state the lane holds (kNoRecord: none).
template <typename T, int W, bool kCounted, int kMode>
__device__ __forceinline__ void cs_start_member(Lane<T, W>& L, Stack<T, W>& S, uint32_t& held, const JoinArgs& a,
                                                uint32_t entry, const uint8_t* pre, uint32_t g0, uint32_t j,
                                                uint32_t d_start) {
  constexpr bool kFindFirst = kMode == kModeFind, kLogVertices = kMode == kModeLog;
  const uint32_t end = a.cs_end;
  if (uint64_t(g0) + j >= a.rec_cap) return;
  const uint4 pd = a.pos_desc[g0 + j];  // {record, first row, query nodes, query}
  const uint32_t rec = pd.x, n = pd.z;
  if (rec == kNoRecord || n < end) return;
  if (kFindFirst && (*(volatile const uint32_t*)&a.pair_flag[rec] & 1u)) return;
  if (n == end) {
    atomicAdd(&a.pair_count[rec], 1ull);
    if (kFindFirst) atomicOr(&a.pair_flag[rec], 1u);
    return;
  }
  const uint64_t* arow = a.ds.adj + 2 * uint64_t(d_start);
  if (held != entry || L.t != L.base) {  // another match, or a search that stopped below the prefix
    cs_prefix<T, W, kCounted>(L, S, end, pre, arow);
    L.t = L.base = int(end);
    held = entry;
  }
  L.crow = a.arena + 2 * uint64_t(pd.y);
  L.perm = a.o.perm + uint64_t(pd.w) * kMaxQueryNodes;
  L.dadj = a.o.dadj + uint64_t(pd.w) * kMaxQueryNodes;
  Bits<T, W> c;
  if constexpr (kCounted) {
    const uint64_t dm = __ldg(reinterpret_cast<const unsigned long long*>(L.dadj) + end);
    c = bandn(bload<T, W>(L.crow + 2 * uint64_t(__ldg(L.perm + end))), L.mapped);
    for (uint64_t pm = dm; pm; pm &= pm - 1) c = band(c, bload<T, W>(arow + 2 * uint64_t(S.f[__ffsll((long long)pm) - 1])));
    const uint32_t k = uint32_t(__popcll(dm));
    c = k < (1u << kPlanes) ? band(c, peq_added(L.P, z<T, W>(), k)) : z<T, W>();
  } else {
    c = cs_level<T, W>(L.crow, L.dadj, arow, a.ds.adjin + 2 * uint64_t(d_start), end, S.f, L.mapped);
  }
  if (!bany(c)) return;  // no branch root: nothing to count, no expansion
  if (end + 1 == n) {    // depth `end` is the leaf level
    const uint32_t pc = bpop(c);
    atomicAdd(&a.pair_count[rec], (unsigned long long)pc);
    atomicAdd(&a.pair_exp[rec], (unsigned long long)pc);
    if (kFindFirst) atomicOr(&a.pair_flag[rec], 1u);
    return;
  }
  L.rec = rec;
  L.qoff = a.q.goff[pd.w];
  L.n = n;
  L.arow = arow;
  L.irow = a.ds.adjin + 2 * uint64_t(d_start);
  L.cnt = 0;
  L.exps = 0;
  L.since_check = 0;
  L.no_split = false;
  L.vis = z<T, W>();
  L.mpset = 0;
  if (kLogVertices)
    for (uint32_t t = 0; t < n; ++t) S.expd[t] = 0;
  L.cur = c;
  L.active = true;
}

// The class's entries by chunked work stealing.  The warp walks its entries
// one at a time; the members of the current entry go to the lanes that need
// work as consecutive items, so those lanes build the same prefix and test
// their members side by side.
template <int K, bool kCounted, int kMode>
__global__ void __launch_bounds__(256) cs_extend_kernel(JoinArgs a) {
  using T = typename std::conditional<K == 0, uint32_t, uint64_t>::type;
  constexpr int W = K == 2 ? 2 : 1;
  const bool counted_applies = *a.ds.maxin < (1u << kPlanes);
  if (counted_applies != kCounted) return;  // the other variant runs this class
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const unsigned long long ntasks = min((unsigned long long)a.cs_cap, a.ctr->cs_n[K]);
  if (ntasks == 0) return;
  const uint8_t* ent = a.cs_ent[K];
  unsigned long long* head = &a.ctr->join_head[0][K];
  const unsigned long long nwarps = (unsigned long long)(gridDim.x * blockDim.x) >> 5;
  Lane<T, W> L;
  L.active = false;
  L.done_fetching = false;
  L.t = L.base = 0;
  Stack<T, W> S;
  uint32_t held = kNoRecord;
  // warp-uniform: this warp's chunk of the queue and the entry being handed out
  unsigned long long qbase = 0, qend = 0;
  bool queue_empty = false;
  uint32_t e_id = 0, e_g0 = 0, e_j0 = 0, e_dstart = 0, nmem = 0, m = 0;
  const uint8_t* e_pre = nullptr;
  for (;;) {
    uint32_t need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    while (need) {
      if (m >= nmem) {  // the next entry
        if (qbase >= qend) {
          if (queue_empty) break;
          unsigned long long base = 0, chunk = 0;
          if (lane == 0) {
            const unsigned long long h = *(volatile const unsigned long long*)head;
            const unsigned long long left = h < ntasks ? ntasks - h : 0;
            chunk = left / (8 * nwarps);
            chunk = chunk < 1 ? 1 : (chunk > 16 ? 16 : chunk);
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
        const uint8_t* e = ent + qbase * a.cs_stride;
        const CsEntry h = *reinterpret_cast<const CsEntry*>(e);
        e_id = uint32_t(qbase);
        e_pre = e + sizeof(CsEntry);
        e_dstart = a.d.goff[h.d];
        e_g0 = a.gmcr_off[h.d];
        e_j0 = h.j0;
        nmem = min(a.gmcr_off[h.d + 1] - e_g0 - h.j0, kCsMembers);
        m = 0;
        ++qbase;
        continue;
      }
      const uint32_t left = nmem - m;
      const uint32_t rank = __popc(need & lt_mask);
      const uint32_t took = uint32_t(__popc(need)) < left ? uint32_t(__popc(need)) : left;
      if (((need >> lane) & 1u) && rank < left)
        cs_start_member<T, W, kCounted, kMode>(L, S, held, a, e_id, e_pre, e_g0, e_j0 + m + rank, e_dstart);
      m += took;
      need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    }
    if (queue_empty && m >= nmem && !L.active) L.done_fetching = true;
    if (__all_sync(0xffffffffu, !L.active && L.done_fetching)) break;
    for (int s = 0; s < a.steps; ++s) {
      if (L.active) {
        if constexpr (kCounted) step_counted<T, W, kMode>(L, a, S);
        else step_inrow<T, W, kMode>(L, a, S);
      }
      const uint32_t idle = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
      if (__popc(idle) >= a.refill || (idle && !__any_sync(0xffffffffu, L.active))) break;
    }
  }
}

// Record class K: 2 = data graphs of 65..128 nodes (128-bit sets), 1 = 33..64
// nodes (64 bits), 0 = up to 32 nodes (32 bits); kWordBits: the sets' machine
// word (32 or 64 bits, at most the set's width).  kCounted selects the counted
// test (EXACT, in-degrees <= 7) or the in-row test.
template <int K, int kWordBits, bool kCounted, int kMode>
__global__ void __launch_bounds__(256) join_kernel(JoinArgs a) {
  constexpr bool kFindFirst = kMode == kModeFind, kLogVertices = kMode == kModeLog;
  using T = typename std::conditional<kWordBits == 32, uint32_t, uint64_t>::type;
  constexpr int kSetBits = 32 << K;
  static_assert(kWordBits <= kSetBits, "a word wider than the set");
  constexpr int W = kSetBits / kWordBits;
  const bool counted_applies = !a.literal && *a.ds.maxin < (1u << kPlanes);
  if (counted_applies != kCounted) return;  // the other variant runs this class
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  // record ranges: [0, wide) two words, [wide, mid) one word, [mid, recs) 32 bits
  const unsigned long long recs = min((unsigned long long)a.rec_cap, a.ctr->recs);
  const unsigned long long wide = min(recs, a.ctr->recs_wide);
  const unsigned long long mid = max(wide, min(recs, a.ctr->recs_mid));
  const unsigned long long lo = K == 2 ? 0 : (K == 1 ? wide : mid);
  const unsigned long long hi = K == 2 ? wide : (K == 1 ? mid : recs);
  // round 0: records (per-pair tasks) or (pair, root) tasks; later rounds:
  // the subtrees the previous round handed over
  const bool subtrees = a.round > 0;
  const SubTask* sub_in = a.sub[a.round & 1];
  unsigned long long first, ntasks;
  if (subtrees) {
    first = 0;
    ntasks = min((unsigned long long)a.sub_cap, a.ctr->sub_n[a.round]);
  } else if (a.per_pair) {  // 2^lanes_log2 lanes per record, each a share of its roots
    first = lo;
    ntasks = (hi - lo) << a.lanes_log2;
  } else {
    first = 0;
    ntasks = min((unsigned long long)a.task_cap, a.ctr->tasks);
  }
  if (ntasks == 0) return;
  unsigned long long* head = &a.ctr->join_head[a.round][K];
  const unsigned long long nwarps = (unsigned long long)(gridDim.x * blockDim.x) >> 5;
  Lane<T, W> L;
  L.active = false;
  L.done_fetching = false;
  Stack<T, W> S;
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
        Bits<T, W> roots;
        bool take = true;
        const SubTask* sub = nullptr;
        if (subtrees) {
          sub = sub_in + (qbase + rank);
          rec = sub->rec;
          take = (K == 2 || rec >= lo) && rec < hi;  // kNoRecord is never in range
        } else if (a.per_pair) {
          rec = uint32_t(first + ((qbase + rank) >> a.lanes_log2));
        } else {
          const Task tk = a.tasks[qbase + rank];
          rec = tk.pair;
          take = (K == 2 || rec >= lo) && rec < hi;  // class 2 starts at record 0
          roots = bbit<T, W>(tk.root);
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
          if (a.per_pair && !subtrees)
            roots = bstride(bload<T, W>(L.crow + 2 * uint64_t(L.perm[0])),
                            uint32_t(qbase + rank) & ((1u << a.lanes_log2) - 1u), a.lanes_log2);
          L.cnt = 0;
          L.exps = 0;
          L.since_check = 0;
          L.t = 0;
          L.base = 0;
          L.no_split = false;
          L.mapped = z<T, W>();
          L.vis = z<T, W>();
#pragma unroll
          for (int b = 0; b < kPlanes; ++b) L.P.p[b] = z<T, W>();
          L.mpset = 0;
          if (subtrees) {  // rebuild the prefix state of the subtree
            const int dep = int(sub->depth);
            L.t = dep;
            L.base = dep;
            roots = bfrom64<T, W>(sub->cand[0], sub->cand[1]);
            for (int j = 0; j < dep; ++j) {
              const uint32_t x = sub->f[j];
              S.f[j] = uint8_t(x);
              L.mapped = bor(L.mapped, bbit<T, W>(x));
              if constexpr (kCounted) {
                const Bits<T, W> row = bload<T, W>(L.arow + 2 * uint64_t(x));
                padd(L.P, row);
              }
            }
          }
          L.cur = roots;
          if (kLogVertices)
            for (uint32_t t = 0; t < L.n; ++t) S.expd[t] = 0;
          if (kFindFirst && (*(volatile const uint32_t*)&a.pair_flag[L.rec] & 1u)) finish<T, W, kMode>(L, a, S.expd);
        }
      }
      qbase += took;
      need = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
    }
    if (queue_empty && !L.active) L.done_fetching = true;
    if (__all_sync(0xffffffffu, !L.active && L.done_fetching)) break;
    for (int s = 0; s < a.steps; ++s) {
      if (L.active) {
        if constexpr (kCounted) step_counted<T, W, kMode>(L, a, S);
        else step_inrow<T, W, kMode>(L, a, S);
      }
      const uint32_t idle = __ballot_sync(0xffffffffu, !L.active && !L.done_fetching);
      if (__popc(idle) >= a.refill || (idle && !__any_sync(0xffffffffu, L.active))) break;
    }
  }
}

template <int K, int kWordBits, int kMode>
cudaError_t launch_mode(const JoinArgs& a, int blocks, int threads, cudaStream_t st) {
  if constexpr (kMode != kModeLog) {
    if (a.cs_end && a.round == 0) {  // the clustered entries of this class
      cs_extend_kernel<K, true, kMode><<<blocks, threads, 0, st>>>(a); note_launch();
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      cs_extend_kernel<K, false, kMode><<<blocks, threads, 0, st>>>(a); note_launch();
      return cudaGetLastError();
    }
  }
  if (!a.literal) {
    join_kernel<K, kWordBits, true, kMode><<<blocks, threads, 0, st>>>(a); note_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  join_kernel<K, kWordBits, false, kMode><<<blocks, threads, 0, st>>>(a); note_launch();
  return cudaGetLastError();
}

template <int K, int kWordBits>
cudaError_t launch_width(const JoinArgs& a, int blocks, int threads, cudaStream_t st) {
  if (a.vertex_exp) return launch_mode<K, kWordBits, kModeLog>(a, blocks, threads, st);
  if (a.find_first) return launch_mode<K, kWordBits, kModeFind>(a, blocks, threads, st);
  return launch_mode<K, kWordBits, kModeCount>(a, blocks, threads, st);
}

// Class 0 sets hold 32 bits: one 32-bit word.  Classes 1 and 2 run with 32- or
// 64-bit words (the schedule's word_bits).
template <int K>
cudaError_t launch_class(const JoinArgs& a, int blocks, int threads, int word_bits, cudaStream_t st) {
  if constexpr (K == 0) {
    (void)word_bits;
    return launch_width<0, 32>(a, blocks, threads, st);
  } else {
    if (word_bits == 32) return launch_width<K, 32>(a, blocks, threads, st);
    return launch_width<K, 64>(a, blocks, threads, st);
  }
}

}  // namespace

cudaError_t launch_join(const JoinArgs& args, const ClassLaunch cl[3], cudaStream_t st, cudaEvent_t (*timers)[3][2],
                        const JoinStreams* js) {
  // the reference DFS's visited state does not survive a split
  bool splits = false;
  for (int k = 0; k < 3; ++k) splits = splits || (cl[k].split_budget != 0 && !args.literal);
  const int rounds = splits ? kJoinRounds : 1;
  cudaError_t e = cudaSuccess;
  for (int r = 0; r < rounds && e == cudaSuccess; ++r) {
    if (r == 0 && args.cs_end) {  // clustered join: the prototype's matches first
      cs_enum_kernel<<<sm_count() * 8, 256, 0, st>>>(args); note_launch();
      e = cudaGetLastError();
    }
    const bool fork = js && !timers;
    if (fork && e == cudaSuccess) {  // classes 1 and 0 on the side streams, after everything before
      e = cudaEventRecord(js->fork, st);
      for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(js->side[i], js->fork, 0);
    }
    for (int k = 2; k >= 0 && e == cudaSuccess; --k) {
      const cudaStream_t ks = fork && k < 2 ? js->side[1 - k] : st;
      JoinArgs a = args;
      a.round = r;
      a.per_pair = args.literal ? 0 : cl[k].per_pair;
      a.steps = cl[k].steps;
      a.refill = cl[k].refill;
      a.split_budget = !args.literal && r + 1 < kJoinRounds ? cl[k].split_budget : 0u;
      a.lanes_log2 = cl[k].lanes_log2;
      if (timers) e = cudaEventRecord(timers[r][k][0], st);
      if (e != cudaSuccess) break;
      e = k == 2 ? launch_class<2>(a, cl[k].blocks, cl[k].threads, cl[k].word_bits, ks)
                 : (k == 1 ? launch_class<1>(a, cl[k].blocks, cl[k].threads, cl[k].word_bits, ks)
                           : launch_class<0>(a, cl[k].blocks, cl[k].threads, cl[k].word_bits, ks));
      if (timers && e == cudaSuccess) e = cudaEventRecord(timers[r][k][1], st);
    }
    if (fork)  // the next round (and everything after) waits for all three classes
      for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaEventRecord(js->done[i], js->side[i]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, js->done[i], 0);
      }
  }
  return e;
}

}  // namespace bms
