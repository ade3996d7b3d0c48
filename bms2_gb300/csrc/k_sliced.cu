// Fused filter + refine + GMCR validity with bit-sliced threshold masks.
//
// The reference tests every (query node, data node) pair of the batch with the
// full predicate (filterCandidates, isomorphism.hpp:30-104, then R passes of
// refineCandidates, :106-203) and then every (query, data graph) pair for
// validity (GMCR kernel 1, gmcr.hpp:54-88).  Every clause of that predicate is
// a threshold on one data-node attribute:
//   label == l (or any label for the wildcard)      -> LAB[l]
//   degree >= k                                     -> DEG[k]
//   cycle count of type t >= c (4 types)            -> CYC[t][c]
//   path-filter bit b set (the query's bit b is set) -> PATH[b]
//   shell k nibble of label l >= c                  -> SHELL[k][l][c]
// So for one data graph, the candidate row of a query node is the AND of the
// node masks of the clauses its own signature selects.  A block owns one data
// graph at a time: it builds, in shared memory, the masks any query uses (a
// warp per clause family and 32-node chunk, bit-transposed across the warp),
// then evaluates the queries level by level in their selectivity order with
// one thread per still-alive query: each evaluation is a walk over the query
// node's precomputed clause list ("program"), ANDing node masks of 32 bits
// (graphs of <= 32 nodes), 64 bits (<= 64) or 128 bits, one launch per size
// class.  A query dies at its first
// empty row; its output rows are allocated once its first row is non-empty.
// Queries whose label multiset cannot embed (EXACT semantics) keep being tested
// for GMCR validity but write no rows and reach no join.
#include "device_common.cuh"

namespace bms {
namespace {

constexpr uint32_t kMLab = 0, kMDeg = 16, kMCyc = 32, kMPath = 64, kMShell = 320;
constexpr uint32_t kMaxMaskIds = kClauseIds;  // 2240
constexpr uint8_t kSlowLabel = 1, kSlowDeg = 2, kSlowCyc = 4;
constexpr uint32_t kNoRow = 0xFFFFFFFFu;

// Node masks of one data graph: W 64-bit words (graphs of up to 64 W nodes),
// or for W = 0 one 32-bit word (graphs of up to 32 nodes: half the mask table
// and one 32-bit operation per mask AND).
template <int W>
struct MaskWord {
  using T = uint64_t;
  static constexpr int n = W;
  static constexpr uint32_t bits = 64;
};
template <>
struct MaskWord<0> {
  using T = uint32_t;
  static constexpr int n = 1;
  static constexpr uint32_t bits = 32;
};
template <int W>
struct Mask {
  typename MaskWord<W>::T w[MaskWord<W>::n];
};
template <int W>
constexpr uint32_t kMaxNodesOf = W == 0 ? 32u : 64u * W;
template <int W>
constexpr uint32_t kHalvesOf = W == 0 ? 1u : 2u * W;  // 32-bit chunks per mask
template <int W>
__device__ __forceinline__ Mask<W> mand(Mask<W> a, Mask<W> b) {
#pragma unroll
  for (int i = 0; i < MaskWord<W>::n; ++i) a.w[i] &= b.w[i];
  return a;
}
template <int W>
__device__ __forceinline__ bool many(Mask<W> a) {
  typename MaskWord<W>::T x = 0;
#pragma unroll
  for (int i = 0; i < MaskWord<W>::n; ++i) x |= a.w[i];
  return x != 0;
}
template <int W>
__device__ __forceinline__ Mask<W> mlow(uint32_t m) {
  using T = typename MaskWord<W>::T;
  constexpr uint32_t B = MaskWord<W>::bits;
  Mask<W> r;
#pragma unroll
  for (int i = 0; i < MaskWord<W>::n; ++i) {
    const uint32_t lo = B * i;
    r.w[i] = m <= lo ? T(0) : (m >= lo + B ? ~T(0) : T((T(1) << (m - lo)) - 1));
  }
  return r;
}
template <int W>
__device__ __forceinline__ void mclear(Mask<W>& a, uint32_t v) {
  using T = typename MaskWord<W>::T;
  constexpr uint32_t B = MaskWord<W>::bits;
  a.w[v / B] &= ~(T(1) << (v % B));
}
template <int W>
__device__ __forceinline__ B128 to128(Mask<W> a) {
  return W <= 1 ? B128{uint64_t(a.w[0]), 0ull} : B128{a.w[0], a.w[MaskWord<W>::n - 1]};
}

// ------------------------------------------------------------- query side
// Clause list of one query node, most selective clauses first: label, degree,
// cycles, shells, path bits.  Clauses that do not fit the mask table (labels
// 16..254, degree > 16, cycle counts > 8) set a slow-path flag instead.
template <bool kWrite>
__device__ uint32_t query_clauses(const uint64_t* rec, int R, const ShellPack& sp, uint16_t* out, uint8_t* slow,
                                  uint32_t* used) {
  uint32_t n = 0;
  auto emit = [&](uint32_t id) {
    if (kWrite) out[n] = uint16_t(id);
    else atomicOr(&used[id >> 5], 1u << (id & 31));
    ++n;
  };
  uint8_t s = 0;
  const uint32_t l = uint32_t(rec[0] & 0xFFu), deg = uint32_t(rec[0] >> 32);
  if (l < 16) emit(kMLab + l);
  else if (l != kWildcard) s |= kSlowLabel;
  if (deg >= 1) {
    if (deg <= 16) emit(kMDeg + deg - 1);
    else s |= kSlowDeg;
  }
  for (int t = 0; t < 4; ++t) {
    const uint32_t c = uint32_t(rec[1] >> (16 * t)) & 0xFFFFu;
    if (c) {
      if (c <= 8) emit(kMCyc + 8 * t + c - 1);
      else s |= kSlowCyc;
    }
  }
  for (int k = 0; k < R; ++k) {
    const uint64_t sh = rec[6 + k];
    for (uint32_t j = 0; j < sp.K; ++j) {
      const uint32_t c = uint32_t(sh >> (4 * sp.pos[j])) & 15u;
      if (c) emit(kMShell + (uint32_t(k) * sp.K + j) * 15 + c - 1);
    }
  }
  for (int w = 0; w < 4; ++w)
    for (uint64_t b = rec[2 + w]; b; b &= b - 1) emit(kMPath + 64 * w + uint32_t(__ffsll((long long)b) - 1));
  if (kWrite && slow) *slow = s;
  return n;
}

// Programs are padded to whole groups of 8 clause indices (16 bytes) with the
// index of an all-ones mask, so the filter reads a group with one load.
constexpr uint32_t kGroup = 8;

__global__ void program_count_kernel(DGraphs q, DSigs qs, ShellPack sp, uint32_t* len, uint32_t* used) {
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < q.N; u += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t n = query_clauses<false>(qs.frec + uint64_t(kRecWords) * u, qs.R, sp, nullptr, nullptr, used);
    len[u] = (n + kGroup - 1) / kGroup * kGroup;
  }
}

// compact index of every used mask id (single block)
__global__ void program_compact_kernel(const uint32_t* used, uint16_t* remap, uint16_t* used_ids, uint32_t* n_used) {
  __shared__ uint32_t base[kMaxMaskIds / 32 + 1];
  if (threadIdx.x == 0) {
    uint32_t b = 0;
    for (uint32_t w = 0; w < kMaxMaskIds / 32; ++w) {
      base[w] = b;
      b += __popc(used[w]);
    }
    *n_used = b;
  }
  __syncthreads();
  for (uint32_t id = threadIdx.x; id < kMaxMaskIds; id += blockDim.x) {
    const uint32_t w = id >> 5, bit = id & 31u;
    if ((used[w] >> bit) & 1u) {
      const uint32_t k = base[w] + __popc(used[w] & ((1u << bit) - 1u));
      remap[id] = uint16_t(k);
      used_ids[k] = uint16_t(id);
    }
  }
}

// the all-ones mask sits right after the used ones, at index n_used
__global__ void program_fill_kernel(DGraphs q, DSigs qs, ShellPack sp, const uint32_t* off, const uint16_t* remap,
                                    const uint32_t* n_used, uint16_t* prog, uint8_t* slow) {
  const uint16_t pad = uint16_t(*n_used);
  for (uint64_t u = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < q.N; u += uint64_t(gridDim.x) * blockDim.x) {
    uint16_t* p = prog + off[u];
    const uint32_t n = query_clauses<true>(qs.frec + uint64_t(kRecWords) * u, qs.R, sp, p, slow + u, nullptr);
    for (uint32_t i = 0; i < n; ++i) p[i] = remap[p[i]];
    for (uint32_t i = n; i < off[u + 1] - off[u]; ++i) p[i] = pad;
  }
}

// Screen record of the i-th query in screening order (decreasing size):
// {query, size | label set << 16, label histogram low, high}.
__global__ void screen_kernel(DGraphs q, DSigs qs, const uint32_t* qorder, uint4* screen) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < q.G; i += gridDim.x * blockDim.x) {
    const uint32_t qg = qorder[i];
    const uint32_t n = q.goff[qg + 1] - q.goff[qg];
    const uint64_t h = qs.ghist[qg];
    screen[i] = make_uint4(qg, (n & 0xFFFFu) | ((qs.glabset[qg] & 0xFFFFu) << 16), uint32_t(h), uint32_t(h >> 32));
  }
}

// One descriptor per (query, level of its filter order); see desc_vertex.
__global__ void level_desc_kernel(DGraphs q, const uint8_t* filter_order, const uint8_t* dup, const uint32_t* prog_off,
                                  const uint8_t* slow, uint2* desc) {
  const uint64_t total = uint64_t(q.G) * kMaxQueryNodes;
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < total; k += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t qg = uint32_t(k / kMaxQueryNodes), level = uint32_t(k % kMaxQueryNodes);
    const uint32_t qoff = q.goff[qg], n = q.goff[qg + 1] - qoff;
    if (level >= n) continue;
    const uint32_t ul = filter_order[k];
    const uint64_t u = uint64_t(qoff) + ul;
    const uint32_t pb = prog_off[u], pe = prog_off[u + 1];
    const uint32_t src = dup[uint64_t(qg) * kMaxQueryNodes + ul];
    desc[k] = make_uint2(pb / kGroup, ((pe - pb) / kGroup) | (ul << 8) | (src << 16) | (uint32_t(slow[u]) << 24));
  }
}

// ------------------------------------------------------------- data side


// The data graph a block works on: its mask table and staged attributes.
template <int W>
struct GraphCtx {
  const Mask<W>* tab;
  const uint8_t* lab;
  const uint64_t* cyc;
  uint32_t start, m;
  Mask<W> all;
};

// Alive-list entries: query id (24 bits), size (7 bits), join-eligible (bit 31).
__device__ __forceinline__ uint32_t entry(uint32_t qg, uint32_t n, bool join) {
  return qg | (n << 24) | (join ? 0x80000000u : 0u);
}
__device__ __forceinline__ uint32_t entry_query(uint32_t e) { return e & 0xFFFFFFu; }
__device__ __forceinline__ uint32_t entry_size(uint32_t e) { return (e >> 24) & 0x7Fu; }
__device__ __forceinline__ bool entry_join(uint32_t e) { return (e >> 31) != 0; }

// Per (query, level) descriptor, built once per run: x = first clause group of
// the vertex's program; y = groups | vertex << 8 | dup source << 16 | slow << 24.
__device__ __forceinline__ uint32_t desc_vertex(uint2 d) { return (d.y >> 8) & 0xFFu; }

// Candidate row of the query vertex at one level of query qg's filter order
// (its descriptor dsc).  A vertex whose record equals an earlier one in that
// order (dup) repeats that row (read back from the arena when the query has
// rows, row0).  Returns whether the row is non-empty.
template <int W>
__device__ __forceinline__ bool eval_node(const SlicedArgs& a, const GraphCtx<W>& g, uint32_t qg, uint2 dsc,
                                          uint32_t row0, Mask<W>& row) {
  const uint32_t ul = desc_vertex(dsc), src = (dsc.y >> 16) & 0xFFu;
  if (src != 0xFFu) {  // same record as an earlier, non-empty row
    if (row0 != kNoRow) {
      const B128 c = ld_b128(a.arena + 2 * (uint64_t(row0) + src));
      row.w[0] = typename MaskWord<W>::T(c.lo);
      if (W > 1) row.w[MaskWord<W>::n - 1] = c.hi;
    }
    return true;
  }
  row = g.all;
  const uint4* grp = reinterpret_cast<const uint4*>(a.prog) + dsc.x;
  const uint32_t groups = dsc.y & 0xFFu;
  for (uint32_t k = 0; k < groups; ++k) {
    const uint4 w = __ldg(grp + k);
    row = mand(row, mand(mand(g.tab[w.x & 0xFFFFu], g.tab[w.x >> 16]), mand(g.tab[w.y & 0xFFFFu], g.tab[w.y >> 16])));
    row = mand(row, mand(mand(g.tab[w.z & 0xFFFFu], g.tab[w.z >> 16]), mand(g.tab[w.w & 0xFFFFu], g.tab[w.w >> 16])));
    if (!many(row)) return false;
  }
  const uint32_t slow = dsc.y >> 24;
  if (slow && many(row)) {
    const uint64_t u = uint64_t(a.q.goff[qg]) + ul;
    const uint64_t rec0 = a.qs.frec[uint64_t(kRecWords) * u], rec1 = a.qs.frec[uint64_t(kRecWords) * u + 1];
    const uint32_t ql = uint32_t(rec0 & 0xFFu), qd = uint32_t(rec0 >> 32);
    for (uint32_t v = 0; v < g.m; ++v) {
      bool ok = true;
      if (slow & kSlowLabel) ok = ok && g.lab[v] == ql;
      if (slow & kSlowDeg) {
        const uint64_t* dr = a.ds.frec + uint64_t(kRecWords) * (uint64_t(g.start) + v);
        ok = ok && uint32_t(dr[0] >> 32) >= qd;
      }
      if (slow & kSlowCyc) ok = ok && cyc_ge(g.cyc[v], rec1);
      if (!ok) mclear(row, v);
    }
  }
  return many(row);
}

// 32 x 32 bit transpose across the warp: lane r holds row r (bit c = A[r][c]);
// afterwards lane c holds column c (bit r = A[r][c]).  Five exchange stages
// swap the off-diagonal blocks of size 16, 8, 4, 2, 1.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, uint32_t lane) {
  const uint32_t keep[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const uint32_t j = 16u >> k;
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~keep[k]) | ((y >> j) & keep[k])) : ((x & keep[k]) | ((y << j) & ~keep[k]));
  }
  return x;
}

// Chunk ch (32 nodes) of the mask of clause id, if some query uses it; the
// halves from zero_from on (past the graph's last node) are cleared.
template <int W>
__device__ __forceinline__ void put_chunk(uint32_t* tab32, const uint32_t* used, const uint16_t* remap, uint32_t id,
                                          uint32_t ch, uint32_t bits, uint32_t zero_from) {
  if ((used[id >> 5] >> (id & 31u)) & 1u) {
    uint32_t* p = tab32 + uint32_t(remap[id]) * kHalvesOf<W>;
    p[ch] = bits;
    for (uint32_t z = zero_from; z < kHalvesOf<W>; ++z) p[z] = 0;
  }
}

template <int W>
__global__ void __launch_bounds__(256) sliced_filter_kernel(SlicedArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr uint32_t MAXN = kMaxNodesOf<W>;
  const int R = a.ds.R;
  // shared layout
  uint64_t* s_path = reinterpret_cast<uint64_t*>(smem);            // [MAXN*4]
  uint64_t* s_cyc = s_path + 4 * MAXN;                              // [MAXN]
  uint64_t* s_sh = s_cyc + MAXN;                                    // [MAXN*R]
  Mask<W>* s_tab = reinterpret_cast<Mask<W>*>(s_sh + MAXN * (R > 0 ? R : 1));  // [n_used]
  uint32_t* s_aq = reinterpret_cast<uint32_t*>(s_tab + (a.n_used_cap ? a.n_used_cap : 1));  // [2][Q] query | join << 31
  uint32_t* s_as = s_aq + 2 * a.q.G;                                // [2][Q] first output row or kNoRow
  uint32_t* s_valid = s_as + 2 * a.q.G;                             // [QW]
  uint8_t* s_lab = reinterpret_cast<uint8_t*>(s_valid + a.QW);      // [MAXN]
  uint8_t* s_deg = s_lab + MAXN;                                    // [MAXN]
  __shared__ uint32_t s_count[2], s_graph, s_nvalid, s_next, s_nrec;
  __shared__ unsigned long long s_recbase;
  __shared__ uint32_t s_used[kMaxMaskIds / 32 + 1];
  __shared__ uint16_t s_remap[kMaxMaskIds];
  const uint32_t tid = threadIdx.x, lane = lane_id();
  const uint32_t Q = a.q.G;
  for (uint32_t w = tid; w < kMaxMaskIds / 32 + 1; w += blockDim.x) s_used[w] = a.used_bits[w];
  __syncthreads();
  for (uint32_t id = tid; id < kMaxMaskIds; id += blockDim.x)
    if ((s_used[id >> 5] >> (id & 31u)) & 1u) s_remap[id] = a.remap[id];
  if (tid == 0) {  // the all-ones mask that pads programs; used masks never overwrite it
    Mask<W> ones;
#pragma unroll
    for (int x = 0; x < MaskWord<W>::n; ++x) ones.w[x] = ~typename MaskWord<W>::T(0);
    s_tab[min(*a.n_used, a.n_used_cap - 1)] = ones;
  }
  for (;;) {
    __syncthreads();
    if (tid == 0) s_graph = atomicAdd(&a.ctr->work[a.class_id], 1u);
    __syncthreads();
    if (a.class_begin + s_graph >= a.class_end) break;
    const uint32_t dg = a.dperm[a.class_begin + s_graph];
    const uint32_t start = a.d.goff[dg], m = a.d.goff[dg + 1] - start;
    // stage node attributes: the graph's records are contiguous, so the block
    // reads them as 16-byte pieces in order (piece q of node v holds record
    // words 2q and 2q + 1) and scatters the words it needs
    {
      const uint32_t pieces = 3u + uint32_t(R + 1) / 2u;  // label/degree/cycle, path, shells 1..R
      const ulonglong2* rec2 = reinterpret_cast<const ulonglong2*>(a.ds.frec + uint64_t(kRecWords) * start);
      for (uint32_t idx = tid; idx < m * 8u; idx += blockDim.x) {
        const uint32_t v = idx >> 3, q = idx & 7u;
        if (q >= pieces) continue;
        const ulonglong2 x = rec2[idx];
        if (q == 0) {
          s_lab[v] = uint8_t(x.x & 0xFFu);
          const uint32_t dgv = uint32_t(x.x >> 32);
          s_deg[v] = uint8_t(dgv > 255u ? 255u : dgv);
          s_cyc[v] = x.y;
        } else if (q < 3) {
          s_path[4 * v + 2 * (q - 1)] = x.x;
          s_path[4 * v + 2 * (q - 1) + 1] = x.y;
        } else {
          const uint32_t k = 2 * (q - 3);
          s_sh[uint32_t(R) * v + k] = x.x;
          if (k + 1 < uint32_t(R)) s_sh[uint32_t(R) * v + k + 1] = x.y;
        }
      }
    }
    for (uint32_t w = tid; w < a.QW; w += blockDim.x) s_valid[w] = 0;
    if (tid < 2) s_count[tid] = 0;
    if (tid == 0) {
      s_nvalid = 0;
      s_next = 0;
      s_nrec = 0;
    }
    __syncthreads();
    // The mask table: a warp takes one clause family and one 32-node chunk of
    // the graph, lane = node.  Each lane writes its node's 32 clause bits of
    // the family as one word (one-hot label, degree and cycle thermometers, a
    // 32-bit slice of the path filter, shell-count thermometers of two labels),
    // and a 32 x 32 bit transpose across the warp leaves lane i holding the
    // mask of the family's clause i, so the used masks are stored in parallel.
    // Families: labels + degrees, cycles, 8 path slices, then per shell step
    // one per pair of packed labels.
    {
      const uint32_t chunks = (m + 31) >> 5;
      const uint32_t shell_items = (a.sp.K + 1) / 2;
      const uint32_t n_items = 10 + uint32_t(R) * shell_items;
      uint32_t* tab32 = reinterpret_cast<uint32_t*>(s_tab);
      for (uint32_t it = tid >> 5; it < n_items * chunks; it += blockDim.x >> 5) {
        const uint32_t item = it / chunks, ch = it - item * chunks;
        const uint32_t v = ch * 32 + lane;
        const bool in = v < m;
        const uint32_t zero_from = ch + 1 == chunks ? chunks : kHalvesOf<W>;  // halves past the graph
        uint32_t row = 0, id = 0;
        bool used = false;
        if (item < 10) {
          if (in) {
            if (item == 0) {
              const uint32_t l = s_lab[v], dg = min(uint32_t(s_deg[v]), 16u);
              row = (l < 16 ? 1u << l : 0u) | (((1u << dg) - 1u) << 16);
            } else if (item == 1) {
              for (int t = 0; t < 4; ++t) {
                const uint32_t cnt = min(uint32_t((s_cyc[v] >> (16 * t)) & 0xFFFFull), 8u);
                row |= ((1u << cnt) - 1u) << (8 * t);
              }
            } else {
              const uint32_t w = item - 2;
              row = uint32_t(s_path[4 * v + (w >> 1)] >> (32 * (w & 1u)));
            }
          }
          id = item == 0 ? kMLab + lane : (item == 1 ? kMCyc + lane : kMPath + (item - 2) * 32 + lane);
          used = (s_used[id >> 5] >> (id & 31u)) & 1u;
        } else {
          const uint32_t k = (item - 10) / shell_items, j0 = 2 * ((item - 10) % shell_items);
          const uint32_t j = j0 + (lane >> 4), c = lane & 15u;  // lane -> (label j, count c + 1)
          id = kMShell + (k * a.sp.K + j) * 15 + c;
          used = c < 15 && j < a.sp.K && ((s_used[id >> 5] >> (id & 31u)) & 1u);
          if (!__any_sync(0xffffffffu, used)) continue;
          if (in) {
            const uint64_t sh = s_sh[uint32_t(R) * v + k];
            const uint32_t n0 = uint32_t(sh >> (4 * a.sp.pos[j0])) & 15u;
            const uint32_t n1 = j0 + 1 < a.sp.K ? uint32_t(sh >> (4 * a.sp.pos[j0 + 1])) & 15u : 0u;
            row = ((1u << n0) - 1u) | (((1u << n1) - 1u) << 16);
          }
        }
        const uint32_t mask = warp_transpose32(row, lane);
        if (used) put_chunk<W>(tab32, s_used, s_remap, id, ch, mask, zero_from);
      }
    }
    // screening: label set, more than one node, label multiset (join)
    const uint64_t dhist = a.ds.ghist[dg];
    const uint32_t dlab = a.ds.glabset[dg];
    for (uint32_t qb = 0; qb < Q; qb += blockDim.x) {
      // screen records in screening order (longest queries first)
      const uint4 sr = qb + tid < Q ? __ldg(a.screen + qb + tid) : make_uint4(Q, 0, 0, 0);
      const uint32_t qg = sr.x, n = sr.y & 0xFFFFu;
      bool p1 = false, p2 = false;
      if (qg < Q && m > 0) {
        p1 = n > 1 && ((sr.y >> 16) & ~dlab) == 0;  // gmcr.hpp:64 and label presence
        p2 = p1 && (!a.skip_by_labels || nib_le(uint64_t(sr.z) | (uint64_t(sr.w) << 32), dhist));
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, p1);
      uint32_t base = 0;
      if (lane == 0 && bal) base = atomicAdd(&s_count[0], __popc(bal));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (p1) {
        const uint32_t k = base + __popc(bal & ((1u << lane) - 1u));
        s_aq[k] = entry(qg, n, p2);
        s_as[k] = kNoRow;
      }
    }
    __syncthreads();
    const Mask<W> all = mlow<W>(m);
    const GraphCtx<W> g{s_tab, s_lab, s_cyc, start, m, all};
    // Level 0 over the screened queries, block-parallel: it ends most pairs.
    // Survivors get their output rows (warp-aggregated allocation) and go to
    // list 1.
    {
      const uint32_t count = s_count[0];
      for (uint32_t i0 = 0; i0 < count; i0 += blockDim.x) {
        const uint32_t i = i0 + tid;
        const bool live = i < count;
        uint32_t qg = 0, n = 0;
        uint2 dsc0 = make_uint2(0, 0);
        bool join = false, alive = false;
        Mask<W> row = all;
        if (live) {
          const uint32_t e = s_aq[i];
          qg = entry_query(e);
          join = entry_join(e);
          n = entry_size(e);
          dsc0 = __ldg(a.desc + uint64_t(qg) * kMaxQueryNodes);
          alive = eval_node<W>(a, g, qg, dsc0, kNoRow, row);
        }
        const bool need = live && alive && join;
        uint32_t row0 = kNoRow;
        const uint32_t nb = __ballot_sync(0xffffffffu, need);
        if (nb) {
          uint32_t incl = need ? n : 0u;
          for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= uint32_t(d)) incl += y;
          }
          unsigned long long base = 0;
          const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
          if (lane == 31) base = atomicAdd(&a.ctr->rows, (unsigned long long)tot);
          base = __shfl_sync(0xffffffffu, base, 31);
          if (need) {
            const unsigned long long b = base + incl - n;
            if (b + n > a.row_cap) {
              atomicOr(a.err, kErrOverflow);
              join = false;
            } else {
              row0 = uint32_t(b);
              st_b128(a.arena + 2 * (uint64_t(row0) + desc_vertex(dsc0)), to128(row));
            }
          }
        }
        const bool cont = live && alive;
        const uint32_t cb = __ballot_sync(0xffffffffu, cont);
        if (cb) {
          uint32_t base = 0;
          if (lane == __ffs(cb) - 1) base = atomicAdd(&s_count[1], __popc(cb));
          base = __shfl_sync(0xffffffffu, base, __ffs(cb) - 1);
          if (cont) {
            const uint32_t k = base + __popc(cb & ((1u << lane) - 1u));
            s_aq[Q + k] = entry(qg, n, join);
            s_as[Q + k] = row0;
          }
        }
      }
    }
    __syncthreads();
    // Levels 1.. : each survivor runs to completion on one thread, taken from
    // a shared counter (queries were screened longest first).  Finished
    // join-eligible queries are collected in list 0 and written out with one
    // global atomic per graph.
    {
      const uint32_t count = s_count[1];
      for (;;) {
        const uint32_t i = atomicAdd(&s_next, 1u);
        if (i >= count) break;
        const uint32_t e = s_aq[Q + i];
        const uint32_t qg = entry_query(e), n = entry_size(e);
        const bool join = entry_join(e);
        const uint32_t row0 = s_as[Q + i];
        bool alive = true;
        const uint2* qdesc = a.desc + uint64_t(qg) * kMaxQueryNodes;
        uint2 dnext = n > 1 ? __ldg(qdesc + 1) : make_uint2(0, 0);
        for (uint32_t level = 1; level < n && alive; ++level) {
          Mask<W> row = all;
          const uint2 dsc = dnext;
          if (level + 1 < n) dnext = __ldg(qdesc + level + 1);  // next level's descriptor in flight
          alive = eval_node<W>(a, g, qg, dsc, join ? row0 : kNoRow, row);
          if (alive && join && row0 != kNoRow) st_b128(a.arena + 2 * (uint64_t(row0) + desc_vertex(dsc)), to128(row));
        }
        if (alive) {
          atomicOr(&s_valid[qg >> 5], 1u << (qg & 31u));
          if (join && row0 != kNoRow) {
            const uint32_t k = atomicAdd(&s_nrec, 1u);
            s_aq[k] = qg;
            s_as[k] = row0;
          }
        }
      }
    }
    __syncthreads();
    {
      const uint32_t nrec = s_nrec;
      if (tid == 0 && nrec) s_recbase = atomicAdd(&a.ctr->recs, (unsigned long long)nrec);
      __syncthreads();
      for (uint32_t k = tid; k < nrec; k += blockDim.x) {
        const unsigned long long r = s_recbase + k;
        if (r < a.rec_cap) a.recs[r] = PairRec{s_aq[k], dg, 0u, s_as[k]};
        else atomicOr(a.err, kErrOverflow);
      }
    }
    // validity bits and per-graph count
    uint32_t nv = 0;
    for (uint32_t w = tid; w < a.QW; w += blockDim.x) {
      const uint32_t bits = s_valid[w];
      a.valid[uint64_t(dg) * a.QW + w] = bits;
      nv += __popc(bits);
    }
    for (int d = 16; d > 0; d >>= 1) nv += __shfl_down_sync(0xffffffffu, nv, d);
    if (lane == 0 && nv) atomicAdd(&s_nvalid, nv);
    __syncthreads();
    if (tid == 0) a.vcounts[dg] = s_nvalid;
  }
}

template <int W>
size_t sliced_smem(const SlicedArgs& a) {
  constexpr size_t MAXN = kMaxNodesOf<W>;
  const size_t R = size_t(a.ds.R > 0 ? a.ds.R : 1);
  size_t b = 8 * (4 * MAXN + MAXN + MAXN * R);
  b += sizeof(Mask<W>) * (a.n_used_cap ? a.n_used_cap : 1);
  b += 4 * (4 * size_t(a.q.G) + a.QW);
  b += 2 * MAXN;
  return (b + 15) & ~size_t(15);
}

}  // namespace

size_t sliced_smem_bytes(const SlicedArgs& a, int words) {
  return words == 0 ? sliced_smem<0>(a) : (words == 1 ? sliced_smem<1>(a) : sliced_smem<2>(a));
}

cudaError_t launch_query_programs(const DGraphs& q, const DSigs& qs, ShellPack sp, uint32_t* len, uint32_t* prog_off,
                                  uint32_t* scan_scratch, uint32_t* used, uint16_t* remap, uint16_t* used_ids,
                                  uint32_t* n_used, uint16_t* prog, uint8_t* slow, uint64_t prog_cap,
                                  uint32_t* prog_total_host, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(used, 0, sizeof(uint32_t) * (kMaxMaskIds / 32 + 1), st);
  if (e != cudaSuccess || q.N == 0) return e;
  const uint64_t want = (q.N + 127) / 128, cap = uint64_t(sm_count()) * 4;
  const unsigned blocks = unsigned(want < cap ? want : cap);
  program_count_kernel<<<blocks, 128, 0, st>>>(q, qs, sp, len, used); note_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = launch_scan_u32(len, prog_off, q.N, scan_scratch, st)) != cudaSuccess) return e;
  program_compact_kernel<<<1, 256, 0, st>>>(used, remap, used_ids, n_used); note_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  (void)prog_cap;
  (void)prog_total_host;
  program_fill_kernel<<<blocks, 128, 0, st>>>(q, qs, sp, prog_off, remap, n_used, prog, slow); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_screen(const DGraphs& q, const DSigs& qs, const uint32_t* qorder, uint4* screen, cudaStream_t st) {
  if (q.G == 0) return cudaSuccess;
  screen_kernel<<<(q.G + 255) / 256, 256, 0, st>>>(q, qs, qorder, screen); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_level_desc(const DGraphs& q, const uint8_t* filter_order, const uint8_t* dup,
                              const uint32_t* prog_off, const uint8_t* slow, uint2* desc, cudaStream_t st) {
  if (q.G == 0) return cudaSuccess;
  const uint64_t want = (uint64_t(q.G) * kMaxQueryNodes + 255) / 256, cap = uint64_t(sm_count()) * 8;
  level_desc_kernel<<<unsigned(want < cap ? want : cap), 256, 0, st>>>(q, filter_order, dup, prog_off, slow, desc); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_sliced_filter(const SlicedArgs& a, int words, size_t smem, cudaStream_t st) {
  if (a.class_end <= a.class_begin) return cudaSuccess;
  const uint32_t graphs = a.class_end - a.class_begin;
  const uint64_t per_sm = smem ? std::max<uint64_t>(1, std::min<uint64_t>(8, (200u << 10) / smem)) : 8;
  const unsigned blocks = unsigned(std::min<uint64_t>(graphs, uint64_t(sm_count()) * per_sm));
  if (words == 0) {
    cudaFuncSetAttribute(sliced_filter_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    sliced_filter_kernel<0><<<blocks, 256, smem, st>>>(a); note_launch();
  } else if (words == 1) {
    cudaFuncSetAttribute(sliced_filter_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    sliced_filter_kernel<1><<<blocks, 256, smem, st>>>(a); note_launch();
  } else {
    cudaFuncSetAttribute(sliced_filter_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    sliced_filter_kernel<2><<<blocks, 256, smem, st>>>(a); note_launch();
  }
  return cudaGetLastError();
}

}  // namespace bms
