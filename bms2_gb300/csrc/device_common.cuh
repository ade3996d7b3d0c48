// Device helpers shared by the kernels: nibble signatures, hashes, 128-bit
// local-id bitsets, warp utilities.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace bms {

// ---------------------------------------------------------------- nibbles
// Signature<PowerGraph,4>::SignatureDevice (signature.hpp:22-53): 16 saturating
// 4-bit label counters; labels >= 16 are ignored.
__device__ __forceinline__ void nib_inc(uint64_t& s, uint32_t l) {
  if (l >= 16) return;
  const uint32_t sh = 4 * l;
  const uint32_t c = uint32_t(s >> sh) & 15u;
  if (c < 15) s += uint64_t(1) << sh;
}

constexpr uint64_t kLoNib = 0x0F0F0F0F0F0F0F0Full;
constexpr uint64_t kHiBit = 0x8080808080808080ull;

// True iff every nibble of q is <= the same nibble of d.  Even and odd nibbles
// are spread into bytes; (d_byte | 0x80) - q_byte keeps bit 7 iff d >= q and
// never borrows across bytes because both values are below 16.
__device__ __forceinline__ uint64_t nib_le_bits(uint64_t q, uint64_t d) {
  const uint64_t qe = q & kLoNib, qo = (q >> 4) & kLoNib;
  const uint64_t de = (d & kLoNib) | kHiBit, dob = ((d >> 4) & kLoNib) | kHiBit;
  return (de - qe) & (dob - qo);
}
__device__ __forceinline__ bool nib_le(uint64_t q, uint64_t d) { return (nib_le_bits(q, d) & kHiBit) == kHiBit; }

// Shell k projected onto ShellPack positions, packed two per word when K <= 8.
__device__ __forceinline__ uint64_t project_shell(uint64_t s, const ShellPack& sp) {
  uint64_t c = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j)
    if (uint32_t(j) < sp.K) c |= ((s >> (4 * sp.pos[j])) & 15ull) << (4 * j);
  return c;
}
__device__ __forceinline__ uint64_t packed_word(const uint64_t* shells, int R, int w, const ShellPack& sp) {
  if (sp.K <= 8) {
    const int k0 = 2 * w, k1 = 2 * w + 1;
    const uint64_t a = k0 < R ? project_shell(shells[k0], sp) : 0ull;
    const uint64_t b = k1 < R ? project_shell(shells[k1], sp) : 0ull;
    return a | (b << 32);
  }
  return w < R ? project_shell(shells[w], sp) : 0ull;
}

// CycleSignatureDevice::contains (signature.hpp:551-554) on 4 packed uint16.
__device__ __forceinline__ bool cyc_ge(uint64_t d, uint64_t q) {
  const uint32_t dl = uint32_t(d), dh = uint32_t(d >> 32), ql = uint32_t(q), qh = uint32_t(q >> 32);
  return (__vcmpgeu2(dl, ql) & __vcmpgeu2(dh, qh)) == 0xFFFFFFFFu;
}

// ---------------------------------------------------------------- hashes
// signature.hpp:393-404: MurmurHash3 fmix32 finalizer, boost-style combine.
__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
__device__ __forceinline__ uint32_t hcombine(uint32_t a, uint32_t b) { return a ^ (b + 0x9e3779b9u + (a << 6) + (a >> 2)); }
// PathSignatureDevice::insert (signature.hpp:418-430) into four words.
__device__ __forceinline__ void bloom_insert(uint64_t& b0, uint64_t& b1, uint64_t& b2, uint64_t& b3, uint32_t v) {
  uint32_t h = v;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const uint32_t idx = h & 255u;
    const uint64_t bit = uint64_t(1) << (idx & 63u);
    const uint32_t w = idx >> 6;
    b0 |= (w == 0) ? bit : 0;
    b1 |= (w == 1) ? bit : 0;
    b2 |= (w == 2) ? bit : 0;
    b3 |= (w == 3) ? bit : 0;
    h = fmix32(h);
  }
}

// ---------------------------------------------------------------- bitsets
struct B128 {
  uint64_t lo, hi;
};
__device__ __forceinline__ B128 b_and(B128 a, B128 b) { return {a.lo & b.lo, a.hi & b.hi}; }
__device__ __forceinline__ B128 b_or(B128 a, B128 b) { return {a.lo | b.lo, a.hi | b.hi}; }
__device__ __forceinline__ B128 b_andn(B128 a, B128 b) { return {a.lo & ~b.lo, a.hi & ~b.hi}; }
__device__ __forceinline__ bool b_any(B128 a) { return (a.lo | a.hi) != 0; }
__device__ __forceinline__ uint32_t b_pop(B128 a) { return uint32_t(__popcll(a.lo) + __popcll(a.hi)); }
__device__ __forceinline__ B128 b_bit(uint32_t i) {
  return i < 64 ? B128{uint64_t(1) << i, 0} : B128{0, uint64_t(1) << (i - 64)};
}
__device__ __forceinline__ bool b_has(B128 a, uint32_t i) { return ((i < 64 ? a.lo >> i : a.hi >> (i - 64)) & 1u) != 0; }
// lowest set bit index (a must be non-zero)
__device__ __forceinline__ uint32_t b_low(B128 a) {
  return a.lo ? uint32_t(__ffsll((long long)a.lo) - 1) : uint32_t(64 + __ffsll((long long)a.hi) - 1);
}
// highest set bit index (a must be non-zero)
__device__ __forceinline__ uint32_t b_high(B128 a) {
  return a.hi ? uint32_t(127 - __clzll((long long)a.hi)) : uint32_t(63 - __clzll((long long)a.lo));
}
__device__ __forceinline__ B128 b_clear_low(B128 a) {
  return a.lo ? B128{a.lo & (a.lo - 1), a.hi} : B128{0, a.hi & (a.hi - 1)};
}
__device__ __forceinline__ B128 ld_b128(const uint64_t* p) {
  const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
  return {v.x, v.y};
}
__device__ __forceinline__ void st_b128(uint64_t* p, B128 a) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(a.lo, a.hi);
}
// mask of the low n bits (n <= 128)
__device__ __forceinline__ B128 b_lowmask(uint32_t n) {
  if (n >= 128) return {~0ull, ~0ull};
  if (n >= 64) return {~0ull, n == 64 ? 0ull : (~0ull >> (128 - n))};
  return {n == 0 ? 0ull : (~0ull >> (64 - n)), 0};
}

// bits [s, s+m) of a dense row as a 128-bit local row
__device__ __forceinline__ B128 extract_row(const uint32_t* row, uint64_t W, uint32_t s, uint32_t m) {
  uint32_t part[4] = {0, 0, 0, 0};
  for (uint32_t k = 0; k < 4 && 32 * k < m; ++k) {
    const uint32_t pos = s + 32 * k;
    const uint32_t wi = pos >> 5, sh = pos & 31u;
    uint32_t x = row[wi] >> sh;
    if (sh && wi + 1 < W) x |= row[wi + 1] << (32 - sh);
    const uint32_t rem = m - 32 * k;
    if (rem < 32) x &= (1u << rem) - 1u;
    part[k] = x;
  }
  return {uint64_t(part[0]) | (uint64_t(part[1]) << 32), uint64_t(part[2]) | (uint64_t(part[3]) << 32)};
}

// Candidates of a one-node prototype (global query node u) in data graph
// [start, start+m): its row of the dense matrix (staged pipeline), or the
// filter and refine tests of u against every data node (isomorphism.hpp:30-104,
// 106-203: label or wildcard, degree, path superset, cycle counts, shells
// 1..R).  Warp-uniform: every lane returns the whole row.
__device__ __forceinline__ B128 prototype_row(const uint64_t* qfrec, const uint64_t* dfrec, int R,
                                              const uint32_t* dense, uint64_t W, uint32_t u, uint32_t start,
                                              uint32_t m) {
  if (dense) return extract_row(dense + uint64_t(u) * W, W, start, m);
  const uint64_t* qr = qfrec + uint64_t(kRecWords) * u;
  const uint64_t w0 = qr[0], qc = qr[1], q0 = qr[2], q1 = qr[3], q2 = qr[4], q3 = qr[5];
  const uint32_t ql = uint32_t(w0 & 0xFFu), qd = uint32_t(w0 >> 32);
  uint32_t part[4] = {0, 0, 0, 0};
  for (uint32_t k = 0; k < 4 && 32 * k < m; ++k) {
    const uint32_t v = 32 * k + (threadIdx.x & 31u);
    bool ok = false;
    if (v < m) {
      const uint64_t* r = dfrec + uint64_t(kRecWords) * (start + v);
      const uint32_t dl = uint32_t(r[0] & 0xFFu), dd = uint32_t(r[0] >> 32);
      ok = (ql == dl || ql == kWildcard) && qd <= dd && (r[2] & q0) == q0 && (r[3] & q1) == q1 &&
           (r[4] & q2) == q2 && (r[5] & q3) == q3 && cyc_ge(r[1], qc);
      for (int s = 0; s < R && ok; ++s) ok = nib_le(qr[6 + s], r[6 + s]);
    }
    part[k] = __ballot_sync(0xffffffffu, ok);
  }
  return {uint64_t(part[0]) | (uint64_t(part[1]) << 32), uint64_t(part[2]) | (uint64_t(part[3]) << 32)};
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// graph id of a global node id: upper bound search on graph offsets
__device__ __forceinline__ uint32_t graph_of(const uint32_t* goff, uint32_t G, uint32_t node) {
  uint32_t lo = 0, hi = G;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (goff[mid + 1] <= node) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

}  // namespace bms
