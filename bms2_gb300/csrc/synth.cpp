// Seeded synthetic molecular graphs and queries.
//
// The reference converts public SMARTS sets with rdkit (generate_data.py); those
// datasets cannot be converted here, so seeded synthetic molecules with the
// stated element, bond, ring and size distributions stand in for them.  No
// dataset item is reproduced.  PRNG: splitmix64 (Steele, Lea, Flood 2014) seeds
// a PCG32 XSH-RR generator (O'Neill 2014).
#include <algorithm>
#include <cmath>
#include <new>
#include <numeric>
#include <vector>

#include "graphs.h"

namespace {

struct Rng {
  uint64_t state, inc;
  static uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) {
    uint64_t s = seed;
    state = splitmix(s);
    inc = splitmix(s) | 1u;
    next();
  }
  uint32_t next() {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = uint32_t(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  double uniform() { return (double(next() >> 5) * 67108864.0 + double(next() >> 6)) / 9007199254740992.0; }
  uint32_t below(uint32_t n) { return n ? uint32_t(uniform() * n) % n : 0; }
  uint32_t range(uint32_t lo, uint32_t hi) { return lo + below(hi - lo + 1); }
  double normal() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
  bool coin(double p) { return uniform() < p; }
};

// Label ids of the reference converter (generate_data.py:8).
enum : uint8_t { N_ = 0, Cl = 1, Br = 3, O_ = 7, C_ = 8, S_ = 9, F_ = 10 };

uint8_t draw_element(Rng& r) {
  // C 72%, N 12%, O 11%, S 2%, F 1.5%, Cl 1%, Br 0.5%
  double u = r.uniform() * 100.0;
  if (u < 72.0) return C_;
  if (u < 84.0) return N_;
  if (u < 95.0) return O_;
  if (u < 97.0) return S_;
  if (u < 98.5) return F_;
  if (u < 99.5) return Cl;
  return Br;
}

uint8_t max_valence(uint8_t l) {
  switch (l) {
    case C_: return 4;
    case S_: return 4;
    case N_: return 3;
    case O_: return 2;
    default: return 1;  // halogens
  }
}

uint8_t draw_bond(Rng& r) {
  // bond ids of generate_data.py:9-15: single 1, double 2, triple 3, aromatic 4
  double u = r.uniform() * 100.0;
  if (u < 60.0) return 1;
  if (u < 80.0) return 2;
  if (u < 82.0) return 3;
  return 4;
}

struct Mol {
  std::vector<uint8_t> lab;
  std::vector<std::vector<uint32_t>> adj;
  std::vector<bms::Edge> edges;
  bool has_edge(uint32_t a, uint32_t b) const {
    for (uint32_t x : adj[a])
      if (x == b) return true;
    return false;
  }
  bool free(uint32_t a) const { return adj[a].size() < max_valence(lab[a]); }
  void bond(uint32_t a, uint32_t b, uint8_t l) {
    adj[a].push_back(b);
    adj[b].push_back(a);
    edges.emplace_back(a, b, l);
  }
};

uint32_t draw_size(Rng& r, const bms_mol_params& p) {
  double v;
  switch (p.size_dist) {
    case BMS_SIZE_NORMAL: v = p.p0 + p.p1 * r.normal(); break;
    case BMS_SIZE_LOGNORMAL: v = std::exp(std::log(p.p0) + p.p1 * r.normal()); break;
    default: return r.range(p.min_nodes, p.max_nodes);
  }
  long n = std::lround(v);
  return uint32_t(std::min<long>(std::max<long>(n, p.min_nodes), p.max_nodes));
}

// One molecule: labels drawn i.i.d.; rings (5/6-membered, some fused) built
// from atoms of valence >= 2; the rest attached as a random tree respecting
// valence (halogens terminal).  Atoms are renumbered in a random depth-first
// order, like the atom order of a SMILES string.
Mol make_molecule(Rng& r, uint32_t n, uint32_t rings) {
  Mol m;
  m.lab.resize(n);
  m.adj.assign(n, {});
  for (uint32_t i = 0; i < n; ++i) m.lab[i] = draw_element(r);
  std::vector<uint32_t> order(n);
  std::iota(order.begin(), order.end(), 0u);
  for (uint32_t i = n; i > 1; --i) std::swap(order[i - 1], order[r.below(i)]);
  std::vector<uint32_t> pool;  // ring-capable atoms not yet used
  std::vector<uint32_t> rest;
  for (uint32_t a : order) (max_valence(m.lab[a]) >= 2 ? pool : rest).push_back(a);
  std::vector<char> placed(n, 0);
  std::vector<std::vector<uint32_t>> ring_list;
  std::vector<int> comp(n, -1);
  int ncomp = 0;
  for (uint32_t k = 0; k < rings; ++k) {
    uint32_t size = r.coin(0.6) ? 6 : 5;
    bool fused = !ring_list.empty() && r.coin(0.4);
    if (fused) {
      // share one bond (a, b) of an existing ring: add size-2 new atoms a-x1..-b
      const auto& base = ring_list[r.below(uint32_t(ring_list.size()))];
      uint32_t i = r.below(uint32_t(base.size()));
      uint32_t a = base[i], b = base[(i + 1) % base.size()];
      if (!m.free(a) || !m.free(b) || pool.size() < size - 2) fused = false;
      if (fused) {
        std::vector<uint32_t> ring{a};
        uint32_t prev = a;
        for (uint32_t j = 0; j < size - 2; ++j) {
          uint32_t x = pool.back();
          pool.pop_back();
          m.bond(prev, x, 1);
          placed[x] = 1;
          comp[x] = comp[a];
          ring.push_back(x);
          prev = x;
        }
        m.bond(prev, b, 1);
        ring.push_back(b);
        ring_list.push_back(ring);
        continue;
      }
    }
    if (pool.size() < size) break;
    std::vector<uint32_t> ring;
    for (uint32_t j = 0; j < size; ++j) {
      ring.push_back(pool.back());
      pool.pop_back();
    }
    for (uint32_t j = 0; j < size; ++j) {
      m.bond(ring[j], ring[(j + 1) % size], 1);
      placed[ring[j]] = 1;
      comp[ring[j]] = ncomp;
    }
    ++ncomp;
    ring_list.push_back(ring);
  }
  // aromatic 6-rings with p = 0.5; other bonds drawn from the bond mix
  std::vector<char> arom(ring_list.size(), 0);
  for (size_t i = 0; i < ring_list.size(); ++i) arom[i] = ring_list[i].size() == 6 && r.coin(0.5);
  for (auto& e : m.edges) std::get<2>(e) = draw_bond(r);
  for (size_t i = 0; i < ring_list.size(); ++i) {
    if (!arom[i]) continue;
    const auto& ring = ring_list[i];
    for (size_t j = 0; j < ring.size(); ++j) {
      uint32_t a = ring[j], b = ring[(j + 1) % ring.size()];
      for (auto& e : m.edges)
        if ((std::get<0>(e) == a && std::get<1>(e) == b) || (std::get<0>(e) == b && std::get<1>(e) == a))
          std::get<2>(e) = 4;
    }
  }
  // connect: start from the first ring (or the first atom) and attach the rest
  std::vector<uint32_t> connected;
  std::vector<char> in_conn(n, 0);
  auto absorb_comp = [&](int c) {
    for (uint32_t a = 0; a < n; ++a)
      if (comp[a] == c && !in_conn[a]) {
        in_conn[a] = 1;
        connected.push_back(a);
      }
  };
  std::vector<uint32_t> todo;
  for (uint32_t a : pool) todo.push_back(a);
  for (uint32_t a : rest) todo.push_back(a);
  for (uint32_t i = uint32_t(todo.size()); i > 1; --i) std::swap(todo[i - 1], todo[r.below(i)]);
  std::vector<int> comps_left;
  for (int c = 0; c < ncomp; ++c) comps_left.push_back(c);
  if (ncomp > 0) {
    absorb_comp(comps_left.front());
    comps_left.erase(comps_left.begin());
  } else if (!todo.empty()) {
    // prefer a non-halogen seed
    size_t s = 0;
    for (size_t i = 0; i < todo.size(); ++i)
      if (max_valence(m.lab[todo[i]]) >= 2) {
        s = i;
        break;
      }
    uint32_t a = todo[s];
    todo.erase(todo.begin() + long(s));
    if (max_valence(m.lab[a]) < 2) m.lab[a] = C_;
    in_conn[a] = 1;
    connected.push_back(a);
  }
  auto pick_free = [&]() -> int64_t {
    std::vector<uint32_t> cand;
    for (uint32_t a : connected)
      if (m.free(a)) cand.push_back(a);
    if (cand.empty()) return -1;
    return cand[r.below(uint32_t(cand.size()))];
  };
  // interleave remaining ring components and single atoms
  while (!todo.empty() || !comps_left.empty()) {
    bool take_comp = !comps_left.empty() && (todo.empty() || r.coin(0.5));
    int64_t host = pick_free();
    if (host < 0) {
      // no free valence left: turn a connected halogen-free atom into carbon
      for (uint32_t a : connected)
        if (m.lab[a] != C_ && max_valence(m.lab[a]) < 4) {
          m.lab[a] = C_;
          break;
        }
      host = pick_free();
      if (host < 0) break;  // cannot happen for n >= 2 with carbon conversion
    }
    if (take_comp) {
      int c = comps_left.back();
      comps_left.pop_back();
      std::vector<uint32_t> members;
      for (uint32_t a = 0; a < n; ++a)
        if (comp[a] == c && m.free(a)) members.push_back(a);
      if (members.empty()) continue;
      uint32_t a = members[r.below(uint32_t(members.size()))];
      m.bond(uint32_t(host), a, draw_bond(r));
      absorb_comp(c);
    } else {
      uint32_t a = todo.back();
      todo.pop_back();
      m.bond(uint32_t(host), a, draw_bond(r));
      in_conn[a] = 1;
      connected.push_back(a);
    }
  }
  // random depth-first renumbering
  std::vector<uint32_t> newid(n, 0xFFFFFFFFu);
  uint32_t next = 0;
  std::vector<uint32_t> st;
  uint32_t start = r.below(n);
  for (uint32_t s0 = 0; s0 < n; ++s0) {
    uint32_t s = (start + s0) % n;
    if (newid[s] != 0xFFFFFFFFu) continue;
    st.push_back(s);
    while (!st.empty()) {
      uint32_t a = st.back();
      st.pop_back();
      if (newid[a] != 0xFFFFFFFFu) continue;
      newid[a] = next++;
      std::vector<uint32_t> nb = m.adj[a];
      for (uint32_t i = uint32_t(nb.size()); i > 1; --i) std::swap(nb[i - 1], nb[r.below(i)]);
      for (uint32_t b : nb)
        if (newid[b] == 0xFFFFFFFFu) st.push_back(b);
    }
  }
  Mol out;
  out.lab.resize(n);
  out.adj.assign(n, {});
  for (uint32_t a = 0; a < n; ++a) out.lab[newid[a]] = m.lab[a];
  std::vector<bms::Edge> es;
  for (const auto& e : m.edges) {
    uint32_t a = newid[std::get<0>(e)], b = newid[std::get<1>(e)];
    if (a > b) std::swap(a, b);
    es.emplace_back(a, b, std::get<2>(e));
  }
  std::sort(es.begin(), es.end());
  for (const auto& e : es) out.bond(std::get<0>(e), std::get<1>(e), std::get<2>(e));
  return out;
}

void append_mol(bms_graphs& g, const Mol& m) { bms::append_graph(g, m.lab, m.edges); }

// Connected induced subgraph of `src` graph gi with k nodes, numbered in a
// random depth-first discovery order.
bool extract_query(Rng& r, const bms_graphs& src, uint32_t gi, uint32_t k, Mol& q) {
  const uint32_t b = src.goff[gi], e = src.goff[gi + 1], n = e - b;
  if (n < k || k == 0) return false;
  std::vector<char> in(n, 0);
  std::vector<uint32_t> sel{r.below(n)};
  in[sel[0]] = 1;
  while (sel.size() < k) {
    std::vector<uint32_t> frontier;
    for (uint32_t a : sel)
      for (uint32_t i = src.rowp[b + a]; i < src.rowp[b + a + 1]; ++i) {
        uint32_t w = src.col[i] - b;
        if (!in[w]) frontier.push_back(w);
      }
    if (frontier.empty()) return false;  // component smaller than k
    uint32_t w = frontier[r.below(uint32_t(frontier.size()))];
    in[w] = 1;
    sel.push_back(w);
  }
  // DFS discovery order over the induced subgraph
  std::vector<uint32_t> newid(n, 0xFFFFFFFFu);
  uint32_t next = 0;
  std::vector<uint32_t> st{sel[0]};
  while (!st.empty()) {
    uint32_t a = st.back();
    st.pop_back();
    if (newid[a] != 0xFFFFFFFFu) continue;
    newid[a] = next++;
    std::vector<uint32_t> nb;
    for (uint32_t i = src.rowp[b + a]; i < src.rowp[b + a + 1]; ++i) {
      uint32_t w = src.col[i] - b;
      if (in[w] && newid[w] == 0xFFFFFFFFu) nb.push_back(w);
    }
    for (uint32_t i = uint32_t(nb.size()); i > 1; --i) std::swap(nb[i - 1], nb[r.below(i)]);
    for (uint32_t w : nb) st.push_back(w);
  }
  q.lab.assign(k, 0);
  q.adj.assign(k, {});
  q.edges.clear();
  for (uint32_t a : sel) q.lab[newid[a]] = src.lab[b + a];
  std::vector<bms::Edge> es;
  for (uint32_t a : sel)
    for (uint32_t i = src.rowp[b + a]; i < src.rowp[b + a + 1]; ++i) {
      uint32_t w = src.col[i] - b;
      if (!in[w] || w <= a) continue;
      uint32_t x = newid[a], y = newid[w];
      if (x > y) std::swap(x, y);
      es.emplace_back(x, y, src.elab[i]);
    }
  std::sort(es.begin(), es.end());
  es.erase(std::unique(es.begin(), es.end(), [](const bms::Edge& p, const bms::Edge& s) {
             return std::get<0>(p) == std::get<0>(s) && std::get<1>(p) == std::get<1>(s);
           }),
           es.end());
  for (const auto& ed : es) q.bond(std::get<0>(ed), std::get<1>(ed), std::get<2>(ed));
  return true;
}

// Pure-carbon chain (numbered along the chain) or a carbon ring with a chain
// tail (numbered around the ring, then along the tail).
Mol carbon_query(Rng& r, uint32_t k) {
  Mol q;
  q.lab.assign(k, C_);
  q.adj.assign(k, {});
  if (k >= 5 && r.coin(0.5)) {
    uint32_t rs = (k >= 6 && r.coin(0.7)) ? 6 : 5;
    for (uint32_t i = 0; i < rs; ++i) q.bond(i, (i + 1) % rs, rs == 6 ? 4 : 1);
    uint32_t anchor = r.below(rs);
    for (uint32_t i = rs; i < k; ++i) {
      q.bond(i == rs ? anchor : i - 1, i, 1);
    }
  } else {
    for (uint32_t i = 1; i < k; ++i) q.bond(i - 1, i, 1);
  }
  return q;
}

// Adversarial symmetric patterns: linearly fused carbon 6-rings, long carbon
// chains, or a carbon chain carrying repeated halogen substituents.
Mol adversarial_query(Rng& r, uint32_t k) {
  Mol q;
  uint32_t kind = r.below(3);
  if (kind == 0 && k >= 6) {
    // linear acene: each new hexagon shares the bond opposite to the one its
    // predecessor shared; n = 4 * rings + 2
    uint32_t rings = std::max<uint32_t>(1, (k - 2) / 4);
    uint32_t n = 4 * rings + 2;
    q.lab.assign(n, C_);
    q.adj.assign(n, {});
    uint32_t c[6] = {0, 1, 2, 3, 4, 5};
    for (uint32_t i = 0; i < 6; ++i) q.bond(c[i], c[(i + 1) % 6], 4);
    uint32_t next = 6;
    for (uint32_t ring = 1; ring < rings; ++ring) {
      uint32_t a = c[3], b = c[4];
      uint32_t n1 = next, n2 = next + 1, n3 = next + 2, n4 = next + 3;
      next += 4;
      q.bond(a, n1, 4);
      q.bond(n1, n2, 4);
      q.bond(n2, n3, 4);
      q.bond(n3, n4, 4);
      q.bond(n4, b, 4);
      uint32_t nc[6] = {b, a, n1, n2, n3, n4};
      std::copy(nc, nc + 6, c);
    }
    return q;
  }
  if (kind == 1 || k < 4) {
    q.lab.assign(k, C_);
    q.adj.assign(k, {});
    for (uint32_t i = 1; i < k; ++i) q.bond(i - 1, i, 1);
    return q;
  }
  // halogen star chain: backbone of carbons, each with up to two halogens
  uint8_t hal = r.coin(0.5) ? F_ : Cl;
  uint32_t backbone = std::max<uint32_t>(2, k / 3);
  q.lab.assign(backbone, C_);
  q.adj.assign(backbone, {});
  for (uint32_t i = 1; i < backbone; ++i) q.bond(i - 1, i, 1);
  uint32_t n = backbone;
  for (uint32_t i = 0; i < backbone && n < k; ++i)
    for (int j = 0; j < 2 && n < k; ++j) {
      if (!q.free(i)) break;
      q.lab.push_back(hal);
      q.adj.emplace_back();
      q.bond(i, n, 1);
      ++n;
    }
  return q;
}

}  // namespace

extern "C" {

int bms_synth_molecules(const bms_mol_params* p, uint64_t seed, bms_graphs** out) {
  if (!p || !out || p->min_nodes == 0 || p->min_nodes > p->max_nodes || p->min_rings > p->max_rings) {
    bms::set_thread_error("invalid molecule parameters");
    return BMS_EINVAL;
  }
  if ((p->size_dist == BMS_SIZE_LOGNORMAL && p->p0 <= 0) || p->size_dist > BMS_SIZE_LOGNORMAL) {
    bms::set_thread_error("invalid size distribution");
    return BMS_EINVAL;
  }
  *out = nullptr;
  bms_graphs* g = new (std::nothrow) bms_graphs();
  if (!g) return BMS_ENOMEM;
  try {
    Rng r(seed);
    for (uint32_t i = 0; i < p->n_graphs; ++i) {
      uint32_t n = draw_size(r, *p);
      uint32_t rings = r.range(p->min_rings, p->max_rings);
      append_mol(*g, make_molecule(r, n, rings));
    }
  } catch (const std::bad_alloc&) {
    delete g;
    return BMS_ENOMEM;
  }
  *out = g;
  return BMS_OK;
}

int bms_synth_queries(const bms_query_params* p, const bms_graphs* src, uint64_t seed, bms_graphs** out) {
  if (!p || !src || !out || p->min_nodes == 0 || p->min_nodes > p->max_nodes || src->n_graphs() == 0) {
    bms::set_thread_error("invalid query parameters");
    return BMS_EINVAL;
  }
  *out = nullptr;
  bms_graphs* g = new (std::nothrow) bms_graphs();
  if (!g) return BMS_ENOMEM;
  try {
    Rng r(seed ^ 0x51ed2701a3c5f0e9ull);
    const uint32_t G = src->n_graphs();
    for (uint32_t i = 0; i < p->n_queries; ++i) {
      uint32_t k = r.range(p->min_nodes, p->max_nodes);
      double u = r.uniform();
      Mol q;
      if (u < p->frac_adversarial) {
        q = adversarial_query(r, k);
      } else if (u < p->frac_adversarial + p->frac_carbon) {
        q = carbon_query(r, k);
      } else {
        bool ok = false;
        for (int attempt = 0; attempt < 64 && !ok; ++attempt) ok = extract_query(r, *src, r.below(G), k, q);
        if (!ok) {
          // largest source graph that can hold a connected k-subgraph, shrinking k
          for (uint32_t kk = k; kk >= 1 && !ok; --kk)
            for (int attempt = 0; attempt < 256 && !ok; ++attempt) ok = extract_query(r, *src, r.below(G), kk, q);
        }
        if (!ok) q = carbon_query(r, k);
      }
      append_mol(*g, q);
    }
  } catch (const std::bad_alloc&) {
    delete g;
    return BMS_ENOMEM;
  }
  *out = g;
  return BMS_OK;
}

}  // extern "C"
