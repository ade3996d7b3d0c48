// Node signatures of a graph batch, one warp per graph.
//
// Replaces, for one side (data or queries), the reference kernels
//   GenerateDataSignaturesKernel      signature.hpp:124-151   -> label_gen
//   GenerateCSRPathSignaturesKernel   signature.hpp:472-519   -> path
//   GenerateCSRCycleSignaturesKernel  signature.hpp:591-719   -> cycle
//   RefineDataSignaturesKernel (x R)  signature.hpp:335-389   -> shells[k]
// in a single pass.  The graph's adjacency is staged in shared memory as one
// 128-bit set per node, so every walk, path and BFS runs on on-chip bitsets.
// Semantics are the reference's with bitsets as wide as the graph (no 64-node
// aliasing, no 128-entry stack cap, cycle signatures for every graph size).
// The grid is persistent (as many blocks as fit the SMs at once) and warps
// take graphs from a counter, so graphs of uneven cost leave no tail.
#include "device_common.cuh"

namespace bms {
namespace {

constexpr int kWarps = 4;
constexpr int kBlocksPerSm = 7;  // 6.4 KB of shared memory per warp: seven 4-warp blocks fit an SM

// Shared memory of one warp.  Two arrays of node sets serve in turn: first the
// reach sets of the distance shells; then scratch[0] holds the in-sets of an
// asymmetric graph, or the (s0, a) item offsets of the cycle enumeration, and
// at last the lanes' path filters, while scratch[1] holds the cycle counters
// of a canonical graph or the same-label sets of a non-canonical one.
struct WarpSmem {
  B128 adj[kMaxDataNodes];  // out-neighbour set of every node (row as a set)
  B128 scratch[2][kMaxDataNodes];
  B128 labmask[16];         // nodes of each label < 16
  uint8_t lab[kMaxDataNodes];
};
static_assert(sizeof(WarpSmem) % 16 == 0, "per-warp areas keep 16-byte alignment");
static_assert(sizeof(uint16_t) * (kMaxDataNodes + 1) <= sizeof(B128) * kMaxDataNodes, "item offsets fit");
static_assert(sizeof(uint32_t) * 32 * 8 <= sizeof(B128) * kMaxDataNodes, "32 path filters fit");
static_assert(sizeof(uint32_t) * 4 * kMaxDataNodes <= sizeof(B128) * kMaxDataNodes, "cycle counters fit");

__device__ __forceinline__ uint16_t* item_first(WarpSmem& s) { return reinterpret_cast<uint16_t*>(s.scratch[0]); }
__device__ __forceinline__ uint32_t* lane_bloom(WarpSmem& s, uint32_t lane) {
  return reinterpret_cast<uint32_t*>(s.scratch[0]) + 8 * lane;
}
typedef uint32_t CycRow[4];
__device__ __forceinline__ CycRow* cyc_counts(WarpSmem& s) { return reinterpret_cast<CycRow*>(s.scratch[1]); }

// CSR row access of the current graph with local ids, from global memory (the
// degrees, and the paths for rows with repeated entries; out-of-graph columns,
// already flagged as an error of the batch, read node 0).
struct Rows {
  const uint32_t* rowp;
  const uint32_t* col;
  uint32_t start, m;
  __device__ uint32_t begin(uint32_t v) const { return rowp[start + v]; }
  __device__ uint32_t end(uint32_t v) const { return rowp[start + v + 1]; }
  __device__ uint32_t at(uint32_t i) const {
    const uint32_t l = col[i] - start;
    return l < m ? l : 0u;
  }
};

// 64-bit node sets for graphs of at most 64 nodes (96% of molecules): the B128
// operations on one word, for the walks and the cycle enumeration, whose
// integer set arithmetic bounds the kernel
__device__ __forceinline__ uint64_t b_and(uint64_t a, uint64_t b) { return a & b; }
__device__ __forceinline__ uint64_t b_or(uint64_t a, uint64_t b) { return a | b; }
__device__ __forceinline__ uint64_t b_andn(uint64_t a, uint64_t b) { return a & ~b; }
__device__ __forceinline__ bool b_any(uint64_t a) { return a != 0; }
__device__ __forceinline__ uint32_t b_pop(uint64_t a) { return uint32_t(__popcll(a)); }
__device__ __forceinline__ uint32_t b_low(uint64_t a) { return uint32_t(__ffsll((long long)a) - 1); }
__device__ __forceinline__ uint64_t b_clear_low(uint64_t a) { return a & (a - 1); }
template <class Set> __device__ __forceinline__ Set set_bit(uint32_t i);
template <> __device__ __forceinline__ uint64_t set_bit<uint64_t>(uint32_t i) { return uint64_t(1) << i; }
template <> __device__ __forceinline__ B128 set_bit<B128>(uint32_t i) { return b_bit(i); }
template <class Set> __device__ __forceinline__ Set set_of(const B128& b);
template <> __device__ __forceinline__ uint64_t set_of<uint64_t>(const B128& b) { return b.lo; }
template <> __device__ __forceinline__ B128 set_of<B128>(const B128& b) { return b; }

// path signature of node v: walks v-a-w (w != v) and v-a-w-x (x != a, x != v),
// as one flat loop with one Bloom insert per iteration, so lanes whose nodes
// have different neighbourhoods still hash in step (inserts commute).  The
// filter's bits accumulate in the lane's own shared words (one OR per
// position, PathSignatureDevice::insert, signature.hpp:418-430).
template <class Set>
__device__ __forceinline__ void path_walks(const WarpSmem& s, uint32_t v, uint32_t lu, uint32_t* bl) {
  const Set bv = set_bit<Set>(v);
  Set ra = set_of<Set>(s.adj[v]), rw{}, rx{};
  uint32_t a = 0, h2 = 0;
  while (true) {
    uint32_t h;
    if (b_any(rx)) {  // next x of the current v-a-w; the hash depends on x's
      // label only, so every other x of that label is dropped with it
      const uint32_t lx = s.lab[b_low(rx)];
      h = hcombine(h2, lx);
      rx = lx < 16 ? b_andn(rx, set_of<Set>(s.labmask[lx])) : b_clear_low(rx);
    } else {  // next w, moving on to the next a with a continuation
      while (!b_any(rw) && b_any(ra)) {
        a = b_low(ra);
        ra = b_clear_low(ra);
        rw = b_andn(set_of<Set>(s.adj[a]), bv);
      }
      if (!b_any(rw)) break;
      const uint32_t w = b_low(rw);
      rw = b_clear_low(rw);
      h2 = hcombine(lu, hcombine(s.lab[a], s.lab[w]));
      h = h2;
      rx = b_andn(set_of<Set>(s.adj[w]), b_or(set_bit<Set>(a), bv));
    }
    uint32_t x = fmix32(h);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const uint32_t idx = x & 255u;
      atomicOr(&bl[idx >> 5], 1u << (idx & 31u));
      x = fmix32(x);
    }
  }
}

// The two-word instance out of line: it keeps the hot loop of the one-word
// instance (graphs of at most 64 nodes) compact in the instruction cache.
__device__ __noinline__ void path_walks_wide(const WarpSmem& s, uint32_t v, uint32_t lu, uint32_t* bl) {
  path_walks<B128>(s, v, lu, bl);
}

// Saturating nibble histogram (signature.hpp:22-53) of the labels < 16 of a
// node set: per present label, min(15, nodes of the set with that label).
__device__ __forceinline__ uint64_t label_hist(const WarpSmem& s, uint32_t present, B128 set) {
  uint64_t h = 0;
  for (uint32_t pl = present; pl; pl &= pl - 1) {
    const uint32_t l = uint32_t(__ffs(int(pl)) - 1);
    const uint32_t c = b_pop(b_and(set, s.labmask[l]));
    h |= uint64_t(c < 15u ? c : 15u) << (4 * l);
  }
  return h;
}

// Exact-distance shells 1..R (signature.hpp:335-389 refines with BFS levels),
// level-synchronous over the warp: reach_k(v) = reach_{k-1}(v) | reach_{k-1}(u)
// for every u in the row of v, and shell k of v (the nodes first reached after
// k steps) is reach_k(v) minus reach_{k-1}(v).  Every lane runs one union per
// neighbour of its nodes per level, so lanes stay in step whatever the BFS
// frontiers look like.  The reach sets live in the two scratch arrays; once no
// set grows, the remaining shells are empty.
// Writes record words 6..13 (shells 1..8; steps >= R stay zero).
template <class Set>
__device__ __forceinline__ void shells_levels_t(WarpSmem& s, const DSigs& out, uint32_t start, uint32_t m,
                                                uint32_t lane, uint32_t present) {
  Set* cur = reinterpret_cast<Set*>(s.scratch[0]);
  Set* nxt = reinterpret_cast<Set*>(s.scratch[1]);
  for (uint32_t v = lane; v < m; v += 32) cur[v] = set_bit<Set>(v);
  __syncwarp();
  bool grows = out.R > 0;
  for (int k = 0; k < kMaxSteps; ++k) {
    bool grew = false;
    for (uint32_t v = lane; v < m; v += 32) {
      uint64_t h = 0;
      if (grows && k < out.R) {
        const Set prev = cur[v];
        Set r = prev;
        for (Set a = set_of<Set>(s.adj[v]); b_any(a); a = b_clear_low(a)) r = b_or(r, cur[b_low(a)]);
        nxt[v] = r;
        const Set shell = b_andn(r, prev);
        if (b_any(shell)) {
          grew = true;
          for (uint32_t pl = present; pl; pl &= pl - 1) {
            const uint32_t l = uint32_t(__ffs(int(pl)) - 1);
            const uint32_t c = b_pop(b_and(shell, set_of<Set>(s.labmask[l])));
            h |= uint64_t(c < 15u ? c : 15u) << (4 * l);
          }
        }
      }
      out.frec[uint64_t(kRecWords) * (uint64_t(start) + v) + 6 + k] = h;
    }
    grows = __any_sync(0xffffffffu, grew);
    __syncwarp();
    Set* t = cur;
    cur = nxt;
    nxt = t;
  }
  __syncwarp();
}

__device__ void shells_levels(WarpSmem& s, const DSigs& out, uint32_t start, uint32_t m, uint32_t lane,
                              uint32_t present) {
  if (m <= 64) shells_levels_t<uint64_t>(s, out, start, m, lane, present);
  else shells_levels_t<B128>(s, out, start, m, lane, present);
}

__device__ __noinline__ uint32_t mult(const Rows& r, uint32_t a, uint32_t target) {
  uint32_t k = 0;
  for (uint32_t i = r.begin(a); i < r.end(a); ++i) k += r.at(i) == target;
  return k;
}

// Cycle closures through v following CSR entries (multi-edge graphs).
__device__ __noinline__ void cycles_entries(const WarpSmem& s, const Rows& r, uint32_t v, uint32_t c[4]) {
  const uint32_t lv = s.lab[v];
  for (uint32_t i1 = r.begin(v); i1 < r.end(v); ++i1) {
    const uint32_t a = r.at(i1);
    const bool s1 = s.lab[a] == lv;
    const B128 m1 = b_or(b_bit(v), b_bit(a));
    for (uint32_t i2 = r.begin(a); i2 < r.end(a); ++i2) {
      const uint32_t b = r.at(i2);
      if (b == v || b_has(m1, b)) continue;
      const bool s2 = s1 && s.lab[b] == lv;
      const B128 m2 = b_or(m1, b_bit(b));
      for (uint32_t i3 = r.begin(b); i3 < r.end(b); ++i3) {
        const uint32_t cc = r.at(i3);
        if (cc == v || b_has(m2, cc)) continue;
        const bool s3 = s2 && s.lab[cc] == lv;
        const B128 m3 = b_or(m2, b_bit(cc));
        for (uint32_t i4 = r.begin(cc); i4 < r.end(cc); ++i4) {
          const uint32_t d = r.at(i4);
          if (d == v || b_has(m3, d)) continue;
          const bool s4 = s3 && s.lab[d] == lv;
          const uint32_t k4 = mult(r, d, v);
          c[s4 ? 0 : 1] += k4;
          const B128 m4 = b_or(m3, b_bit(d));
          for (uint32_t i5 = r.begin(d); i5 < r.end(d); ++i5) {
            const uint32_t e = r.at(i5);
            if (e == v || b_has(m4, e)) continue;
            const bool s5 = s4 && s.lab[e] == lv;
            c[s5 ? 2 : 3] += mult(r, e, v);
          }
        }
      }
    }
  }
}

// Every 5- and 6-cycle of a symmetric graph without repeated entries, once:
// from its smallest node s0, through larger nodes only, second node below the
// last.  Each member gets +2 in the same/different-label counter of the
// cycle's length — exactly what the per-node walk counts (the cycle in both
// directions), so the halved signature is unchanged.  A cycle is "same" iff
// all its nodes carry one label (the per-node rule: every node after v on the
// path has v's label).  Counters in scratch[1]; lanes take (s0, first edge)
// items, whose offsets sit in scratch[0].
template <class Set>
__device__ __forceinline__ void cycles_canonical_t(WarpSmem& s, uint32_t m, uint32_t lane) {
  const Set all = set_of<Set>(b_lowmask(m));
  CycRow* cyc = cyc_counts(s);
  uint16_t* first = item_first(s);
  // work items: (s0, a) with a an upper neighbour of s0, spread over the lanes
  // first[v] = items of the nodes before v: a warp scan per 32 nodes
  uint32_t carry = 0;
  for (uint32_t v0 = 0; v0 < m; v0 += 32) {
    const uint32_t v = v0 + lane;
    uint32_t n = 0;
    if (v < m) {
      for (int t = 0; t < 4; ++t) cyc[v][t] = 0;
      n = b_pop(b_and(set_of<Set>(s.adj[v]), b_andn(all, set_of<Set>(b_lowmask(v + 1)))));
    }
    uint32_t incl = n;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= uint32_t(d)) incl += y;
    }
    if (v < m) first[v + 1] = uint16_t(carry + incl);
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) first[0] = 0;
  __syncwarp();
  const uint32_t items = first[m];
  for (uint32_t k = lane; k < items; k += 32) {
    uint32_t lo = 0, hi = m;  // first[lo] <= k < first[hi]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (first[mid] <= k) lo = mid;
      else hi = mid;
    }
    const uint32_t s0 = lo;
    const Set gt = b_andn(all, set_of<Set>(b_lowmask(s0 + 1)));
    Set up = b_and(set_of<Set>(s.adj[s0]), gt);
    for (uint32_t r = k - first[s0]; r > 0; --r) up = b_clear_low(up);
    const uint32_t a = b_low(up);
    const uint32_t l0 = s.lab[s0];
    const Set ns = set_of<Set>(s.adj[s0]);
    const bool s1 = s.lab[a] == l0;
    const Set v1 = set_bit<Set>(a);
    // the cycle's last node is a neighbour of s0 above a (orientation)
    const Set last = b_and(ns, b_andn(gt, set_of<Set>(b_lowmask(a + 1))));
    if (!b_any(last)) continue;
    // only paths that can still close are walked: the 4th node closes a
    // 5-cycle (it is in last) or precedes the last node of a 6-cycle (it is
    // next to last), and the 3rd node is next to such a 4th node
    Set q4 = last;
    for (Set r = last; b_any(r); r = b_clear_low(r)) q4 = b_or(q4, set_of<Set>(s.adj[b_low(r)]));
    q4 = b_and(q4, gt);
    Set q3{};
    for (Set r = q4; b_any(r); r = b_clear_low(r)) q3 = b_or(q3, set_of<Set>(s.adj[b_low(r)]));
    q3 = b_and(q3, gt);
    for (Set r2 = b_andn(b_and(set_of<Set>(s.adj[a]), gt), v1); b_any(r2); r2 = b_clear_low(r2)) {
      const uint32_t b = b_low(r2);
      const bool s2 = s1 && s.lab[b] == l0;
      const Set v2 = b_or(v1, set_bit<Set>(b));
      for (Set r3 = b_andn(b_and(set_of<Set>(s.adj[b]), q3), v2); b_any(r3); r3 = b_clear_low(r3)) {
        const uint32_t c = b_low(r3);
        const bool s3 = s2 && s.lab[c] == l0;
        const Set v3 = b_or(v2, set_bit<Set>(c));
        for (Set r4 = b_andn(b_and(set_of<Set>(s.adj[c]), q4), v3); b_any(r4); r4 = b_clear_low(r4)) {
          const uint32_t d = b_low(r4);
          const bool s4 = s3 && s.lab[d] == l0;
          if (b_any(b_and(last, set_bit<Set>(d)))) {
            const int t = s4 ? 0 : 1;
            atomicAdd(&cyc[s0][t], 2u);
            atomicAdd(&cyc[a][t], 2u);
            atomicAdd(&cyc[b][t], 2u);
            atomicAdd(&cyc[c][t], 2u);
            atomicAdd(&cyc[d][t], 2u);
          }
          const Set v4 = b_or(v3, set_bit<Set>(d));
          for (Set r5 = b_andn(b_and(set_of<Set>(s.adj[d]), last), v4); b_any(r5); r5 = b_clear_low(r5)) {
            const uint32_t e = b_low(r5);
            const int t = (s4 && s.lab[e] == l0) ? 2 : 3;
            atomicAdd(&cyc[s0][t], 2u);
            atomicAdd(&cyc[a][t], 2u);
            atomicAdd(&cyc[b][t], 2u);
            atomicAdd(&cyc[c][t], 2u);
            atomicAdd(&cyc[d][t], 2u);
            atomicAdd(&cyc[e][t], 2u);
          }
        }
      }
    }
  }
  __syncwarp();
}

// The enumeration on one-word sets when the graph has at most 64 nodes.
__device__ void cycles_canonical(WarpSmem& s, uint32_t m, uint32_t lane) {
  if (m <= 64) cycles_canonical_t<uint64_t>(s, m, lane);
  else cycles_canonical_t<B128>(s, m, lane);
}

// Cycle closures through v on adjacency sets (graphs without repeated entries).
// At depth 5 the closing nodes are counted in one step: they are the unvisited
// out-neighbours of the depth-4 node whose rows contain v.
__device__ __noinline__ void cycles_sets(const WarpSmem& s, B128 inv, B128 eq, uint32_t v, uint32_t c[4]) {
  const uint32_t lv = s.lab[v];
  for (B128 r1 = s.adj[v]; b_any(r1); r1 = b_clear_low(r1)) {
    const uint32_t a = b_low(r1);
    const bool s1 = s.lab[a] == lv;
    const B128 m1 = b_or(b_bit(v), b_bit(a));
    for (B128 r2 = b_andn(s.adj[a], m1); b_any(r2); r2 = b_clear_low(r2)) {
      const uint32_t b = b_low(r2);
      const bool s2 = s1 && s.lab[b] == lv;
      const B128 m2 = b_or(m1, b_bit(b));
      for (B128 r3 = b_andn(s.adj[b], m2); b_any(r3); r3 = b_clear_low(r3)) {
        const uint32_t cc = b_low(r3);
        const bool s3 = s2 && s.lab[cc] == lv;
        const B128 m3 = b_or(m2, b_bit(cc));
        for (B128 r4 = b_andn(s.adj[cc], m3); b_any(r4); r4 = b_clear_low(r4)) {
          const uint32_t d = b_low(r4);
          const bool s4 = s3 && s.lab[d] == lv;
          if (b_has(inv, d)) c[s4 ? 0 : 1] += 1;
          const B128 close = b_and(b_andn(s.adj[d], b_or(m3, b_bit(d))), inv);
          const uint32_t all = b_pop(close);
          const uint32_t same = s4 ? b_pop(b_and(close, eq)) : 0u;
          c[2] += same;
          c[3] += all - same;
        }
      }
    }
  }
}

// In-sets of an asymmetric graph, by scattering every row, written out here
// (scratch[0] serves the path filters later), and the same-label sets in
// scratch[1] for the set-based cycle count.  Returns the lane's largest
// in-degree.  Out of line: asymmetric graphs are rare.
__device__ __noinline__ uint32_t asym_sets(WarpSmem& s, const DSigs& out, uint32_t start, uint32_t m, uint32_t lane) {
  B128* ins = s.scratch[0];
  for (uint32_t v = lane; v < m; v += 32) ins[v] = B128{0, 0};
  __syncwarp();
  for (uint32_t v = lane; v < m; v += 32) {
    const B128 bv = b_bit(v);
    for (B128 r = s.adj[v]; b_any(r); r = b_clear_low(r)) {
      const uint32_t w = b_low(r);
      atomicOr(reinterpret_cast<unsigned long long*>(&ins[w].lo), (unsigned long long)bv.lo);
      atomicOr(reinterpret_cast<unsigned long long*>(&ins[w].hi), (unsigned long long)bv.hi);
    }
  }
  __syncwarp();
  uint32_t max_in = 0;
  for (uint32_t v = lane; v < m; v += 32) {
    const B128 i = ins[v];
    max_in = max(max_in, b_pop(i));
    st_b128(out.adjin + 2 * (uint64_t(start) + v), i);
    const uint8_t l = s.lab[v];
    B128 eq{0, 0};
    if (l < 16) {
      eq = s.labmask[l];
    } else {
      for (uint32_t y = 0; y < m; ++y)
        if (s.lab[y] == l) eq = b_or(eq, b_bit(y));
    }
    s.scratch[1][v] = eq;
  }
  return max_in;
}

// One graph on one warp: its rows staged as node sets, the symmetry check and
// label masks, then the shells, the canonical cycle enumeration and the
// per-node label, path and cycle signatures.
__device__ __forceinline__ void signatures_graph(const DGraphs& g, const DSigs& out, uint32_t max_nodes,
                                                 uint32_t* err, WarpSmem& s, uint32_t gi, uint32_t lane) {
  const uint32_t start = g.goff[gi];
  const uint32_t m = g.goff[gi + 1] - start;
  if (m > max_nodes) {
    if (lane == 0) atomicOr(err, kErrTooLarge);
    return;
  }
  // stage labels; rows as adjacency sets.  Row offsets must be non-decreasing
  // and inside [0, E]; a lane reads a row's entries only once its two offsets
  // passed, four entries per round of loads.
  uint32_t bad = 0;
  bool multi = false, rows_ok = true;
  if (lane < 16) s.labmask[lane] = B128{0, 0};
  if (m == 0 && lane == 0) rows_ok = g.rowp[start] <= g.E;
  for (uint32_t v = lane; v < m; v += 32) {
    s.lab[v] = g.lab[start + v];
    const uint32_t rb = g.rowp[start + v], re = g.rowp[start + v + 1];
    B128 a{0, 0};
    if (rb <= re && re <= g.E) {
      for (uint32_t i = rb; i < re; i += 4) {
        uint32_t cc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) cc[j] = i + j < re ? g.col[i + j] : start;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (i + j >= re) break;
          uint32_t lc = cc[j] - start;
          if (cc[j] < start || lc >= m) {
            bad |= kErrColumn;
            lc = 0;  // keep the entry inside the graph; the batch is rejected
          }
          if (b_has(a, lc)) multi = true;
          a = b_or(a, b_bit(lc));
        }
      }
    } else {
      rows_ok = false;
    }
    s.adj[v] = a;
  }
  if (!__all_sync(0xffffffffu, rows_ok)) {
    if (lane == 0) atomicOr(err, kErrRows);
    __syncwarp();
    return;
  }
  multi = __any_sync(0xffffffffu, multi);
  __syncwarp();
  // label masks: one 32-node word per label and chunk of nodes, stored by the
  // chunk's first lane with that label
  for (uint32_t v0 = 0; v0 < m; v0 += 32) {
    const uint32_t v = v0 + lane;
    const uint32_t l = v < m ? uint32_t(s.lab[v]) : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xffffffffu, l);
    if (l < 16 && lane == uint32_t(__ffs(int(peers)) - 1))
      reinterpret_cast<uint32_t*>(&s.labmask[l])[v0 >> 5] = peers;
  }
  // symmetry as sets (w in the row of v implies v in the row of w), read off
  // the staged rows; the in-sets of a symmetric graph are its rows
  bool sym = true;
  uint32_t max_in = 0;
  for (uint32_t v = lane; v < m; v += 32) {
    const B128 a = s.adj[v];
    for (B128 r = a; b_any(r); r = b_clear_low(r)) sym = sym && b_has(s.adj[b_low(r)], v);
    max_in = max(max_in, b_pop(a));
  }
  const bool asym = !__all_sync(0xffffffffu, sym);
  __syncwarp();
  // labels < 16 present in the graph: label histograms are popcounts of their masks
  const uint32_t present = __ballot_sync(0xffffffffu, lane < 16 && b_any(s.labmask[lane]));
  shells_levels(s, out, start, m, lane, present);
  if (asym) {
    max_in = asym_sets(s, out, start, m, lane);
    bad |= kErrAsym;
  }
  max_in = __reduce_max_sync(0xffffffffu, max_in);
  if (lane == 0 && max_in) atomicMax(out.maxin, max_in);
  bad = __reduce_or_sync(0xffffffffu, bad);
  if (bad && lane == 0) atomicOr(err, bad);
  __syncwarp();
  const Rows rows{g.rowp, g.col, start, m};
  // symmetric graphs without repeated entries: every cycle found once
  const bool canonical = !multi && !asym;
  if (canonical) cycles_canonical(s, m, lane);
  const CycRow* cyc = cyc_counts(s);
  for (uint32_t v = lane; v < m; v += 32) {
    const uint64_t u = uint64_t(start) + v;
    const uint32_t lu = s.lab[v];
    const uint32_t rb = rows.begin(v), re = rows.end(v);
    // label signature: +1 per CSR entry on the neighbour's label
    uint64_t lg = 0;
    if (multi) {
      for (uint32_t i = rb; i < re; ++i) nib_inc(lg, s.lab[rows.at(i)]);
    } else {  // every entry distinct: the row as a set
      lg = label_hist(s, present, s.adj[v]);
    }
    // path signature (path_walks), into the lane's own 256-bit filter
    uint32_t* bl = lane_bloom(s, lane);
    reinterpret_cast<uint4*>(bl)[0] = make_uint4(0, 0, 0, 0);
    reinterpret_cast<uint4*>(bl)[1] = make_uint4(0, 0, 0, 0);
    if (m <= 64) path_walks<uint64_t>(s, v, lu, bl);
    else path_walks_wide(s, v, lu, bl);
    const uint4 bq0 = reinterpret_cast<const uint4*>(bl)[0], bq1 = reinterpret_cast<const uint4*>(bl)[1];
    const uint64_t p0 = uint64_t(bq0.x) | (uint64_t(bq0.y) << 32), p1 = uint64_t(bq0.z) | (uint64_t(bq0.w) << 32);
    const uint64_t p2 = uint64_t(bq1.x) | (uint64_t(bq1.y) << 32), p3 = uint64_t(bq1.z) | (uint64_t(bq1.w) << 32);
    // cycle signature
    uint32_t c[4] = {0, 0, 0, 0};
    if (canonical) {
      for (int t = 0; t < 4; ++t) c[t] = cyc[v][t];
    } else if (multi) {
      cycles_entries(s, rows, v, c);
    } else {
      cycles_sets(s, ld_b128(out.adjin + 2 * u), s.scratch[1][v], v, c);
    }
    const uint64_t cy = uint64_t((c[0] & 0xFFFFu) >> 1) | (uint64_t((c[1] & 0xFFFFu) >> 1) << 16) |
                        (uint64_t((c[2] & 0xFFFFu) >> 1) << 32) | (uint64_t((c[3] & 0xFFFFu) >> 1) << 48);
    // record words 6..13 (distance shells) were written by shells_levels
    const uint32_t deg = re - rb;
    ulonglong2* rec = reinterpret_cast<ulonglong2*>(out.frec + uint64_t(kRecWords) * u);
    rec[0] = make_ulonglong2(uint64_t(lu) | (uint64_t(deg) << 32), cy);
    rec[1] = make_ulonglong2(p0, p1);
    rec[2] = make_ulonglong2(p2, p3);
    rec[7] = make_ulonglong2(lg, 0ull);
    st_b128(out.adj + 2 * u, s.adj[v]);
    if (!asym) st_b128(out.adjin + 2 * u, s.adj[v]);
  }
  __syncwarp();
  // per-graph label histogram (labels < 16) and label set
  uint32_t cnt = 0;
  if (lane < 16) cnt = b_pop(s.labmask[lane]);
  const uint32_t nib = lane < 16 ? (cnt > 15 ? 15u : cnt) : 0u;
  const uint32_t lo = __reduce_or_sync(0xffffffffu, lane < 8 ? nib << (4 * lane) : 0u);
  const uint32_t hi = __reduce_or_sync(0xffffffffu, (lane >= 8 && lane < 16) ? nib << (4 * (lane - 8)) : 0u);
  if (lane == 0) {
    out.ghist[gi] = uint64_t(lo) | (uint64_t(hi) << 32);
    out.glabset[gi] = present & 0xFFFFu;
  }
  __syncwarp();
}

// Graphs are taken one at a time from out.maxin[1] (zero before the launch);
// the next graph is claimed while the current one runs.
__global__ void __launch_bounds__(kWarps * 32, kBlocksPerSm) signatures_kernel(DGraphs g, DSigs out,
                                                                              uint32_t max_nodes, uint32_t* err) {
  __shared__ WarpSmem smem[kWarps];
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  uint32_t* head = out.maxin + 1;
  uint32_t gi = lane == 0 ? atomicAdd(head, 1u) : 0u;
  gi = __shfl_sync(0xffffffffu, gi, 0);
  while (gi < g.G) {
    uint32_t next = 0;
    if (lane == 0) next = atomicAdd(head, 1u);
    signatures_graph(g, out, max_nodes, err, smem[warp], gi, lane);
    gi = __shfl_sync(0xffffffffu, next, 0);
  }
}

}  // namespace

cudaError_t launch_signatures(const DGraphs& g, DSigs s, uint32_t max_nodes, uint32_t* err, cudaStream_t st) {
  if (g.G == 0) return cudaSuccess;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, signatures_kernel, kWarps * 32, 0);
  if (e != cudaSuccess) return e;
  const uint64_t want = (uint64_t(g.G) + kWarps - 1) / kWarps;
  const uint64_t cap = uint64_t(sms > 0 ? sms : 152) * uint64_t(per_sm > 0 ? per_sm : 1);
  const unsigned blocks = unsigned(want < cap ? want : cap);
  signatures_kernel<<<blocks, kWarps * 32, 0, st>>>(g, s, max_nodes, err); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
