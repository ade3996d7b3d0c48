// Embedding output for one (query, data graph) pair.
//
// The reference only counts (isomorphism.hpp:291-472, "# Matches"); this
// enumerates the injective induced embeddings the EXACT join counts, from the
// pair's candidate rows and the search order of the last run.  One thread per
// root candidate runs the DFS of the join (in-row induced test, two 64-bit
// words per set) and writes every complete mapping by query vertex:
// out[k * n + u] = local data id of query vertex u.  Slots are reserved with an
// atomic counter; the host sorts the mappings, so the output is deterministic.
#include "device_common.cuh"

namespace bms {
namespace {

__device__ __forceinline__ B128 rd(const uint64_t* p) { return ld_b128(p); }

__global__ void find_record_kernel(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, uint32_t gpos,
                                   unsigned long long* out) {
  const uint64_t n = min((unsigned long long)rec_cap, ctr->recs);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    if (recs[i].gpos == gpos) *out = i;
}

__global__ void __launch_bounds__(128) embed_kernel(EmbedArgs a) {
  const uint32_t root = threadIdx.x;
  const PairRec r = a.recs[a.rec];
  const uint32_t qoff = a.q.goff[r.q], n = a.q.goff[r.q + 1] - qoff;
  const uint8_t* perm = a.o.perm + uint64_t(r.q) * kMaxQueryNodes;
  const uint64_t* dadj = a.o.dadj + uint64_t(r.q) * kMaxQueryNodes;
  const uint64_t* crow = a.arena + 2 * uint64_t(r.c_row);
  const uint64_t* arow = a.ds.adj + 2 * uint64_t(a.d.goff[r.d]);
  const uint64_t* irow = a.ds.adjin + 2 * uint64_t(a.d.goff[r.d]);
  if (n < 2 || !b_has(rd(crow + 2 * uint64_t(perm[0])), root)) return;
  uint8_t f[kMaxQueryNodes];
  B128 F[kMaxQueryNodes];
  f[0] = uint8_t(root);
  B128 mapped = b_bit(root);
  // candidates of depth j given the nodes mapped at depths < j
  auto level = [&](uint32_t j) -> B128 {
    B128 c = b_andn(rd(crow + 2 * uint64_t(perm[j])), mapped);
    B128 pset{0, 0};
    for (uint64_t pm = dadj[j]; pm; pm &= pm - 1) {
      const uint32_t x = f[__ffsll((long long)pm) - 1];
      c = b_and(c, rd(arow + 2 * uint64_t(x)));
      pset = b_or(pset, b_bit(x));
    }
    B128 res{0, 0};
    for (B128 w = c; b_any(w); w = b_clear_low(w)) {
      const uint32_t v = b_low(w);
      if (!b_any(b_andn(b_and(rd(irow + 2 * uint64_t(v)), mapped), pset))) res = b_or(res, b_bit(v));
    }
    return res;
  };
  uint32_t t = 1;
  F[1] = level(1);
  for (;;) {
    if (!b_any(F[t])) {
      if (t == 1) break;
      --t;
      mapped = b_andn(mapped, b_bit(f[t]));  // back at depth t: its node leaves the path
      continue;
    }
    const uint32_t v = b_low(F[t]);
    F[t] = b_clear_low(F[t]);
    if (t + 1 == n) {  // a complete embedding
      const unsigned long long k = atomicAdd(a.count, 1ull);
      if (k < a.cap) {
        uint8_t* o = a.out + k * n;
        for (uint32_t i = 0; i + 1 < n; ++i) o[perm[i]] = f[i];
        o[perm[n - 1]] = uint8_t(v);
      }
      continue;
    }
    f[t] = uint8_t(v);
    mapped = b_or(mapped, b_bit(v));
    ++t;
    F[t] = level(t);
  }
}

}  // namespace

cudaError_t launch_find_record(const PairRec* recs, const Counters* ctr, uint64_t rec_cap, uint32_t gpos,
                               unsigned long long* out, cudaStream_t st) {
  find_record_kernel<<<sm_count() * 4, 256, 0, st>>>(recs, ctr, rec_cap, gpos, out); note_launch();
  return cudaGetLastError();
}

cudaError_t launch_embed(const EmbedArgs& a, cudaStream_t st) {
  embed_kernel<<<1, 128, 0, st>>>(a); note_launch();
  return cudaGetLastError();
}

}  // namespace bms
