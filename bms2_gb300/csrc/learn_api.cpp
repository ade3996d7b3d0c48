// Learned search order and schedule entry points of the C ABI.  The cost model
// and the autotuner have no counterpart in the reference: its only ordering
// hook, defineMatchingOrder (isomorphism.hpp:476-502), is never called.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"

using namespace bms;

namespace {

const char* const kFeatureNames[kFeatures] = {
    "log2_mean_candidates",   // log2(1 + mean candidate-set size over the query's join pairs)
    "degree",                 // query degree / 4
    "data_label_freq",        // share of data nodes carrying the vertex's label (wildcard: 1)
    "query_label_share",      // share of the query's vertices with the same label
    "in_5_ring",              // the vertex closes a 5-ring (cycle signature)
    "in_6_ring",              // the vertex closes a 6-ring
    "log2_ring_closures",     // log2(1 + all 5/6-ring closures)
    "query_size",             // query node count / 64
    "same_label_neighbours",  // share of neighbours with the vertex's label
    "path_density",           // set bits of the 256-bit path filter / 256
    "neighbour_degree",       // sum of neighbour degrees / 16
    "two_hop_reach",          // query vertices within distance 2 / query size
};

constexpr char kMagic[8] = {'B', 'M', 'S', 'M', 'L', 'P', '0', '1'};

}  // namespace

extern "C" {

const char* bms_feature_name(int i) { return (i >= 0 && i < kFeatures) ? kFeatureNames[i] : ""; }

int bms_model_get(bms_ctx* c, float* params) {
  GUARD(c);
  if (!params) return fail(c, BMS_EINVAL, "params is null");
  if (!c->model_set) return fail(c, BMS_ESTATE, "no model: train, set or load one");
  CK(cudaMemcpyAsync(params, c->model_master.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
}

int bms_model_set(bms_ctx* c, const float* params) {
  GUARD(c);
  if (!params) return fail(c, BMS_EINVAL, "params is null");
  for (int i = 0; i < kParams; ++i)
    if (!(params[i] == params[i]) || params[i] > 1e30f || params[i] < -1e30f)
      return fail(c, BMS_EINVAL, "model parameters must be finite");
  CK(c->model_master.ensure(sizeof(float) * kParams));
  CK(c->model_bf16.ensure(sizeof(uint16_t) * kParams));
  CK(cudaMemcpyAsync(c->model_master.p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, c->st));
  CK(launch_to_bf16(c->model_master.as<float>(), c->model_bf16.as<uint16_t>(), kParams, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->model_set = true;
  return BMS_OK;
}

int bms_model_save(bms_ctx* c, const char* path) {
  GUARD(c);
  if (!path) return fail(c, BMS_EINVAL, "path is null");
  std::vector<float> p(kParams);
  int r = bms_model_get(c, p.data());
  if (r) return r;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(c, BMS_EIO, std::string("cannot open ") + path);
  bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(p.data(), sizeof(float), kParams, f) == size_t(kParams);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BMS_OK : fail(c, BMS_EIO, std::string("write error on ") + path);
}

int bms_model_load(bms_ctx* c, const char* path) {
  GUARD(c);
  if (!path) return fail(c, BMS_EINVAL, "path is null");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(c, BMS_EIO, std::string("cannot open ") + path);
  char magic[8];
  std::vector<float> p(kParams);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0 &&
            std::fread(p.data(), sizeof(float), kParams, f) == size_t(kParams);
  std::fclose(f);
  if (!ok) return fail(c, BMS_EINVAL, std::string("not a cost-model file: ") + path);
  return bms_model_set(c, p.data());
}

}  // extern "C"

namespace {

// splitmix64 (Steele, Lea, Flood 2014): seeds initialisation and shuffles
uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double unit(uint64_t& s) { return double(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

bool have_records(const bms_ctx* c) { return c->have_results; }

}  // namespace

int bms::compute_features(bms_ctx* c) {
  const uint64_t Qn = c->q.N ? c->q.N : 1;
  CK(c->cand_sum.ensure(sizeof(unsigned int) * Qn));
  CK(c->recs_per_query.ensure(sizeof(unsigned int) * (c->q.G ? c->q.G : 1)));
  CK(c->features.ensure(sizeof(float) * kFeatures * Qn));
  CK(c->label_count.ensure(256 * sizeof(unsigned long long)));
  CK(cudaMemsetAsync(c->cand_sum.p, 0, sizeof(unsigned int) * Qn, c->st));
  CK(cudaMemsetAsync(c->recs_per_query.p, 0, sizeof(unsigned int) * (c->q.G ? c->q.G : 1), c->st));
  CK(launch_record_stats(c->recs.as<PairRec>(), c->ctr.as<Counters>(), c->rec_cap, c->q.dg(), c->arena.as<uint64_t>(),
                         c->recs_per_query.as<unsigned int>(), c->cand_sum.as<unsigned int>(), c->st));
  CK(launch_label_count(c->d.dg(), c->label_count.as<unsigned long long>(), c->st));
  DFeatureArgs fa{};
  fa.q = c->q.dg();
  fa.qs = c->q.ds();
  fa.label_count = c->label_count.as<unsigned long long>();
  fa.data_nodes = c->d.N;
  fa.cand_sum = c->cand_sum.as<unsigned int>();
  fa.recs_per_query = c->recs_per_query.as<unsigned int>();
  fa.features = c->features.as<float>();
  CK(launch_features(fa, c->st));
  return BMS_OK;
}

int bms::learned_order(bms_ctx* c) {
  if (!c->model_set) return fail(c, BMS_ESTATE, "the learned order needs a cost model: train, set or load one");
  int r = compute_features(c);
  if (r) return r;
  CK(c->cost.ensure(sizeof(float) * (c->q.N ? c->q.N : 1)));
  CK(launch_mlp_predict(c->features.as<float>(), c->q.N, c->model_bf16.as<uint16_t>(), c->cost.as<float>(), c->st));
  CK(launch_learned_order(c->q.dg(), c->q.ds(), c->cost.as<float>(),
                          DOrder{c->perm.as<uint8_t>(), c->dadj.as<uint64_t>()}, c->st));
  return BMS_OK;
}

extern "C" {

int bms_query_features(bms_ctx* c, float* out) {
  GUARD(c);
  if (!out) return fail(c, BMS_EINVAL, "out is null");
  if (!have_records(c)) return fail(c, BMS_ESTATE, "run bms_run or bms_join first");
  int r = compute_features(c);
  if (r) return r;
  if (c->q.N) CK(cudaMemcpyAsync(out, c->features.p, sizeof(float) * kFeatures * c->q.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
}

int bms_vertex_expansions(bms_ctx* c, uint64_t* out) {
  GUARD(c);
  if (!out) return fail(c, BMS_EINVAL, "out is null");
  if (!c->have_vexp)
    return fail(c, BMS_ESTATE, "no vertex log: enable bms_set_logging and run count-all, GMCR or given order, EXACT");
  if (c->q.N)
    CK(cudaMemcpyAsync(out, c->vertex_exp.p, sizeof(uint64_t) * c->q.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return BMS_OK;
}

int bms_model_predict(bms_ctx* c, float* cost, uint8_t* order) {
  GUARD(c);
  if (!have_records(c)) return fail(c, BMS_ESTATE, "run bms_run or bms_join first");
  const uint64_t Qslots = uint64_t(c->q.G ? c->q.G : 1) * kMaxQueryNodes;
  CK(c->perm.ensure(Qslots));
  CK(c->dadj.ensure(sizeof(uint64_t) * Qslots));
  int r = learned_order(c);
  if (r) return r;
  if (cost && c->q.N) CK(cudaMemcpyAsync(cost, c->cost.p, sizeof(float) * c->q.N, cudaMemcpyDeviceToHost, c->st));
  std::vector<uint8_t> perm(Qslots);
  CK(cudaMemcpyAsync(perm.data(), c->perm.p, Qslots, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (order) {
    for (uint32_t qg = 0; qg < c->q.G; ++qg) {
      const uint32_t qoff = c->q.h_goff[qg], n = c->q.h_goff[qg + 1] - qoff;
      for (uint32_t t = 0; t < n; ++t) order[qoff + t] = perm[uint64_t(qg) * kMaxQueryNodes + t];
    }
  }
  // the order buffers now hold the learned order; the next join recomputes its own
  return BMS_OK;
}

int bms_model_grad(bms_ctx* c, const float* params, const float* x, const float* y, uint32_t n, float* y_out,
                   float* grad, float* loss) {
  GUARD(c);
  if (!params || !x || !y || n == 0) return fail(c, BMS_EINVAL, "params, x, y and n > 0 are required");
  DevBuf master, wbf, dx, dy, partial, dgrad, lpart, dloss, dpred;
  const int blocks = mlp_grad_blocks(n);
  CK(master.ensure(sizeof(float) * kParams));
  CK(wbf.ensure(sizeof(uint16_t) * kParams));
  CK(dx.ensure(sizeof(float) * kFeatures * n));
  CK(dy.ensure(sizeof(float) * n));
  CK(dpred.ensure(sizeof(float) * n));
  CK(partial.ensure(sizeof(float) * kParams * blocks));
  CK(dgrad.ensure(sizeof(float) * kParams));
  CK(lpart.ensure(sizeof(float) * blocks));
  CK(dloss.ensure(sizeof(float)));
  CK(cudaMemcpyAsync(master.p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(dx.p, x, sizeof(float) * kFeatures * n, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(dy.p, y, sizeof(float) * n, cudaMemcpyHostToDevice, c->st));
  CK(launch_to_bf16(master.as<float>(), wbf.as<uint16_t>(), kParams, c->st));
  CK(launch_mlp_grad(dx.as<float>(), dy.as<float>(), n, n, wbf.as<uint16_t>(), partial.as<float>(), dpred.as<float>(),
                     lpart.as<float>(), c->st));
  CK(launch_mlp_reduce(partial.as<float>(), blocks, dgrad.as<float>(), lpart.as<float>(), dloss.as<float>(), n, c->st));
  if (y_out) CK(cudaMemcpyAsync(y_out, dpred.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->st));
  if (grad) CK(cudaMemcpyAsync(grad, dgrad.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, c->st));
  float l = 0.f;
  CK(cudaMemcpyAsync(&l, dloss.p, sizeof(float), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (loss) *loss = l;
  return BMS_OK;
}

int bms_model_train(bms_ctx* c, const float* x, const float* y, uint32_t n, uint32_t epochs, uint32_t batch, float lr,
                    uint64_t seed, float* final_loss) {
  GUARD(c);
  if (!x || !y || n == 0 || batch == 0 || epochs == 0 || !(lr > 0.f))
    return fail(c, BMS_EINVAL, "x, y, n > 0, epochs > 0, batch > 0 and lr > 0 are required");
  uint64_t s = seed ^ 0x6a09e667f3bcc908ull;
  if (!c->model_set) {
    // He-uniform initialisation, zero biases
    std::vector<float> p(kParams, 0.f);
    const float a1 = std::sqrt(6.f / float(kFeatures)), a2 = std::sqrt(6.f / float(kHidden));
    for (int i = 0; i < kHidden * kFeatures; ++i) p[i] = float((2.0 * unit(s) - 1.0) * a1);
    for (int i = 0; i < kHidden * kHidden; ++i) p[832 + i] = float((2.0 * unit(s) - 1.0) * a2);
    for (int i = 0; i < kHidden; ++i) p[4992 + i] = float((2.0 * unit(s) - 1.0) * a2);
    int r = bms_model_set(c, p.data());
    if (r) return r;
  }
  const uint32_t B = std::min(batch, n);
  const int blocks = mlp_grad_blocks(B);
  CK(c->adam_m.ensure(sizeof(float) * kParams));
  CK(c->adam_v.ensure(sizeof(float) * kParams));
  CK(c->grad.ensure(sizeof(float) * kParams));
  CK(c->grad_partial.ensure(sizeof(float) * kParams * blocks));
  CK(c->loss_buf.ensure(sizeof(float) * (blocks + 1)));
  CK(c->train_x.ensure(sizeof(float) * kFeatures * n));
  CK(c->train_y.ensure(sizeof(float) * n));
  CK(cudaMemsetAsync(c->adam_m.p, 0, sizeof(float) * kParams, c->st));
  CK(cudaMemsetAsync(c->adam_v.p, 0, sizeof(float) * kParams, c->st));
  std::vector<uint32_t> idx(n);
  std::vector<float> xs(size_t(kFeatures) * n), ys(n), losses;
  for (uint32_t i = 0; i < n; ++i) idx[i] = i;
  DevBuf dlosses;
  const uint32_t steps_per_epoch = (n + B - 1) / B;
  CK(dlosses.ensure(sizeof(float) * steps_per_epoch));
  int step = 0;
  float last = 0.f;
  for (uint32_t e = 0; e < epochs; ++e) {
    for (uint32_t i = n; i > 1; --i) std::swap(idx[i - 1], idx[splitmix(s) % i]);
    for (uint32_t i = 0; i < n; ++i) {
      std::memcpy(&xs[size_t(kFeatures) * i], x + size_t(kFeatures) * idx[i], sizeof(float) * kFeatures);
      ys[i] = y[idx[i]];
    }
    CK(cudaMemcpyAsync(c->train_x.p, xs.data(), sizeof(float) * kFeatures * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->train_y.p, ys.data(), sizeof(float) * n, cudaMemcpyHostToDevice, c->st));
    for (uint32_t k = 0; k < steps_per_epoch; ++k) {
      const uint32_t lo = k * B, cnt = std::min(B, n - lo);
      const int nb = mlp_grad_blocks(cnt);
      CK(launch_mlp_grad(c->train_x.as<float>() + size_t(kFeatures) * lo, c->train_y.as<float>() + lo, cnt, cnt,
                         c->model_bf16.as<uint16_t>(), c->grad_partial.as<float>(), nullptr, c->loss_buf.as<float>(),
                         c->st));
      CK(launch_mlp_reduce(c->grad_partial.as<float>(), nb, c->grad.as<float>(), c->loss_buf.as<float>(),
                           dlosses.as<float>() + k, cnt, c->st));
      CK(launch_adam(c->model_master.as<float>(), c->model_bf16.as<uint16_t>(), c->grad.as<float>(),
                     c->adam_m.as<float>(), c->adam_v.as<float>(), lr, 0.9f, 0.999f, 1e-8f, ++step, c->st));
    }
    losses.resize(steps_per_epoch);
    CK(cudaMemcpyAsync(losses.data(), dlosses.p, sizeof(float) * steps_per_epoch, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    double tot = 0;
    for (uint32_t k = 0; k < steps_per_epoch; ++k) {
      const uint32_t cnt = std::min(B, n - k * B);
      tot += double(losses[k]) * cnt;
    }
    last = float(tot / n);
  }
  if (final_loss) *final_loss = last;
  return BMS_OK;
}

// Times the join of the loaded workload under candidate schedules and keeps
// the fastest.  Tasks are emitted once; every trial re-runs the join over
// them from a reset work head.  The schedule table records the shape per query
// size bucket (one shape serves all buckets of the single persistent launch).
// Coordinate search over the join schedule, all buckets at once: every
// candidate value of one column is tried for the three buckets together, each
// bucket's kernels are timed on their own (best of two runs), and each bucket
// keeps its fastest value before the next column is searched.
int bms_autotune(bms_ctx* c, int R, int mode, int order, bms_schedule* out) {
  GUARD(c);
  if (c->use_cs) return bms::fail(c, BMS_EINVAL, "the autotuner times the plain join; switch the clustered join off");
  uint64_t total = 0;
  int r = bms_run(c, R, mode, order, BMS_SEM_EXACT, &total);
  if (r && r != BMS_EINCOMPLETE) return r;
  bms_schedule best = c->sched;
  float best_ms[3];
  auto timed = [&](const bms_schedule& s, float cms[3]) -> int {
    float ms = 0.f, a[3], b[3];
    int rr = rejoin_timed(c, s, &ms, a);
    if (rr) return rr;
    rr = rejoin_timed(c, s, &ms, b);
    if (rr) return rr;
    for (int k = 0; k < 3; ++k) cms[k] = std::min(a[k], b[k]);
    return BMS_OK;
  };
  r = timed(best, best_ms);
  if (r) return r;
  struct Shape {
    uint32_t bps, wpb;
  };
  const Shape shapes[] = {{2, 8}, {3, 8}, {4, 8}, {6, 4}, {8, 4}, {12, 2}};  // <= 256 threads per block
  const uint32_t budgets[] = {256, 1024, 4096, 0};
  const uint32_t steps[] = {16, 32, 64};
  const uint32_t refills[] = {1, 2, 4, 8};
  const uint32_t depths[] = {0, 1};
  const uint32_t lanes[] = {1, 2, 4, 8, 32};
  const uint32_t words[] = {32, 64};
  auto sweep = [&](int n, auto apply) -> int {
    for (int i = 0; i < n; ++i) {
      bms_schedule s = best;
      for (int k = 0; k < 3; ++k) apply(s, k, i);
      float cms[3];
      const int rr = timed(s, cms);
      if (rr) return rr;
      for (int k = 0; k < 3; ++k)
        if (cms[k] < best_ms[k]) {
          best_ms[k] = cms[k];
          bms_schedule pick = best;
          apply(pick, k, i);
          best.blocks_per_sm[k] = pick.blocks_per_sm[k];
          best.warps_per_block[k] = pick.warps_per_block[k];
          best.split_budget[k] = pick.split_budget[k];
          best.steps[k] = pick.steps[k];
          best.refill[k] = pick.refill[k];
          best.split_depth[k] = pick.split_depth[k];
          best.lanes_per_pair[k] = pick.lanes_per_pair[k];
          best.word_bits[k] = pick.word_bits[k];
        }
    }
    return BMS_OK;
  };
  r = sweep(int(sizeof(shapes) / sizeof(shapes[0])), [&](bms_schedule& s, int k, int i) {
    s.blocks_per_sm[k] = shapes[i].bps;
    s.warps_per_block[k] = shapes[i].wpb;
  });
  if (r) return r;
  r = sweep(4, [&](bms_schedule& s, int k, int i) { s.split_budget[k] = budgets[i]; });
  if (r) return r;
  r = sweep(3, [&](bms_schedule& s, int k, int i) { s.steps[k] = steps[i]; });
  if (r) return r;
  r = sweep(4, [&](bms_schedule& s, int k, int i) { s.refill[k] = refills[i]; });
  if (r) return r;
  r = sweep(2, [&](bms_schedule& s, int k, int i) { s.split_depth[k] = depths[i]; });
  if (r) return r;
  // lanes per pair (per-pair tasks only): 1 lane, a few lanes, one warp per
  // pair as the reference's sub-group decomposition (isomorphism.hpp:401)
  r = sweep(int(sizeof(lanes) / sizeof(lanes[0])), [&](bms_schedule& s, int k, int i) { s.lanes_per_pair[k] = lanes[i]; });
  if (r) return r;
  // machine word of the search sets: 32- or 64-bit words for the 64- and
  // 128-bit buckets (the 32-bit bucket has one 32-bit word)
  r = sweep(2, [&](bms_schedule& s, int k, int i) { s.word_bits[k] = k == 0 ? 32u : words[i]; });
  if (r) return r;
  for (int k = 0; k < 3; ++k) best.ms[k] = best_ms[k];
  best.ms[3] = 0.f;
  c->sched = best;
  if (out) *out = c->sched;
  return BMS_OK;
}

}  // extern "C"
