// A host-only stand-in for the part of SYCL 2020 that the reference's headers
// use, so that their kernels can run on the CPU and produce reference outputs.
//
// Test infrastructure only (it builds the checker's fixtures).  Nothing here is
// SYCL's implementation; it follows the SYCL 2020 specification's semantics
// for the calls named below, restated serially:
//   - queue::submit / parallel_for / single_task run the kernel to completion
//     before returning (every command is synchronous; events are no-ops);
//   - range<1>/range<2> kernels run their items in row-major order;
//   - nd_range<1> kernels run one work-group after another; inside a
//     work-group every work-item is a cooperative fiber (ucontext), started in
//     local-id order, switched only at group collectives.  Sub-groups are 32
//     consecutive work-items.  group_barrier, select_from_group, any_of_group
//     and reduce_over_group complete once every member has arrived;
//   - atomic_ref operations are plain read-modify-writes (one thread);
//   - malloc_device/host/shared return zero-filled host memory (the only
//     deterministic reading of memory the reference reads before writing);
//   - a fiber's stack is filled with 0xFF bytes before each work-item starts,
//     so private arrays the reference reads before writing hold all-ones
//     (NULL_NODE for node ids).
#pragma once

#include <ucontext.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#define SYCL_EXTERNAL

namespace sycl {

// ------------------------------------------------------------------ index space
template <int D = 1>
struct range {
  size_t v[D > 0 ? D : 1] = {};
  range() = default;
  template <int E = D, typename = std::enable_if_t<E == 1>>
  range(size_t a) { v[0] = a; }
  template <int E = D, typename = std::enable_if_t<E == 2>>
  range(size_t a, size_t b) { v[0] = a; v[1] = b; }
  size_t operator[](int i) const { return v[i]; }
  size_t& operator[](int i) { return v[i]; }
  size_t get(int i) const { return v[i]; }
  size_t size() const {
    size_t s = 1;
    for (int i = 0; i < D; ++i) s *= v[i];
    return s;
  }
};
range(size_t) -> range<1>;
range(size_t, size_t) -> range<2>;

template <int D = 1>
struct id {
  size_t v[D] = {};
  size_t operator[](int i) const { return v[i]; }
  size_t get(int i) const { return v[i]; }
  template <int E = D, typename = std::enable_if_t<E == 1>>
  operator size_t() const { return v[0]; }
};

template <int D = 1>
struct item {
  id<D> i;
  range<D> r;
  size_t get_id(int d) const { return i.v[d]; }
  id<D> get_id() const { return i; }
  size_t operator[](int d) const { return i.v[d]; }
  size_t get_range(int d) const { return r.v[d]; }
  range<D> get_range() const { return r; }
  size_t get_linear_id() const { return D == 1 ? i.v[0] : i.v[0] * r.v[1] + i.v[1]; }
  template <int E = D, typename = std::enable_if_t<E == 1>>
  operator size_t() const { return i.v[0]; }
};

template <int D = 1>
struct nd_range {
  range<D> global, local;
  nd_range(range<D> g, range<D> l) : global(g), local(l) {}
  range<D> get_global_range() const { return global; }
  range<D> get_local_range() const { return local; }
};

namespace detail {

// one work-group being executed: its fibers and collective state
struct GroupRun {
  size_t group_id = 0, n_groups = 1, wg_size = 1, sg_size = 32, global_size = 1;
  size_t current = 0;
  ucontext_t sched;
  std::vector<ucontext_t> ctx;
  std::vector<char> done;
  size_t live = 0;
  // barriers: arrivals and generation, for the work-group and each sub-group
  size_t wg_arrived = 0, wg_gen = 0;
  std::vector<size_t> sg_arrived, sg_gen;
  // one 16-byte slot per work-item for collective operands
  std::vector<unsigned char> slots;
  uint64_t progress = 0;
  bool waiting = false;
};

inline thread_local GroupRun* g_run = nullptr;

inline void yield_waiting() {
  GroupRun& g = *g_run;
  g.waiting = true;
  swapcontext(&g.ctx[g.current], &g.sched);
  g.waiting = false;
}

inline void wg_barrier() {
  GroupRun& g = *g_run;
  const size_t gen = g.wg_gen;
  if (++g.wg_arrived == g.wg_size) {
    g.wg_arrived = 0;
    ++g.wg_gen;
    ++g.progress;
    return;
  }
  while (g.wg_gen == gen) yield_waiting();
}

inline size_t sg_of(size_t lid) { return lid / g_run->sg_size; }
inline size_t sg_members(size_t sg) {
  GroupRun& g = *g_run;
  const size_t beg = sg * g.sg_size;
  return std::min(g.sg_size, g.wg_size - beg);
}

inline void sg_barrier() {
  GroupRun& g = *g_run;
  const size_t s = sg_of(g.current);
  const size_t gen = g.sg_gen[s];
  if (++g.sg_arrived[s] == sg_members(s)) {
    g.sg_arrived[s] = 0;
    ++g.sg_gen[s];
    ++g.progress;
    return;
  }
  while (g.sg_gen[s] == gen) yield_waiting();
}

template <typename T>
void put_slot(size_t lid, const T& x) {
  static_assert(sizeof(T) <= 16, "collective operand too large");
  std::memcpy(&g_run->slots[lid * 16], &x, sizeof(T));
}
template <typename T>
T get_slot(size_t lid) {
  T x;
  std::memcpy(&x, &g_run->slots[lid * 16], sizeof(T));
  return x;
}

}  // namespace detail

struct sub_group {
  size_t lid;  // work-group local id of the work-item
  size_t get_local_linear_id() const { return lid % detail::g_run->sg_size; }
  range<1> get_local_range() const { return range<1>(detail::sg_members(detail::sg_of(lid))); }
  range<1> get_max_local_range() const { return range<1>(detail::g_run->sg_size); }
  size_t get_group_linear_id() const { return detail::sg_of(lid); }
  bool leader() const { return get_local_linear_id() == 0; }
};

template <int D = 1>
struct group {
  size_t lid;
  size_t get_group_linear_id() const { return detail::g_run->group_id; }
  size_t get_group_id(int) const { return detail::g_run->group_id; }
  size_t get_local_linear_id() const { return lid; }
  range<1> get_local_range() const { return range<1>(detail::g_run->wg_size); }
  size_t get_group_linear_range() const { return detail::g_run->n_groups; }
  range<1> get_group_range() const { return range<1>(detail::g_run->n_groups); }
  bool leader() const { return lid == 0; }
};

template <int D = 1>
struct nd_item {
  size_t lid;
  size_t get_global_id(int) const { return detail::g_run->group_id * detail::g_run->wg_size + lid; }
  size_t get_global_linear_id() const { return get_global_id(0); }
  size_t get_local_id(int) const { return lid; }
  size_t get_local_linear_id() const { return lid; }
  size_t get_global_range(int) const { return detail::g_run->global_size; }
  size_t get_local_range(int) const { return detail::g_run->wg_size; }
  size_t get_group_linear_id() const { return detail::g_run->group_id; }
  group<D> get_group() const { return group<D>{lid}; }
  sub_group get_sub_group() const { return sub_group{lid}; }
};

// ------------------------------------------------------------------ collectives
template <typename G>
void group_barrier(const G&) {
  if constexpr (std::is_same_v<G, sub_group>)
    detail::sg_barrier();
  else
    detail::wg_barrier();
}

template <typename T = void>
struct plus {
  template <typename A, typename B>
  auto operator()(const A& a, const B& b) const { return a + b; }
};
template <typename T = void>
struct maximum {
  template <typename A, typename B>
  auto operator()(const A& a, const B& b) const { return a < b ? b : a; }
};
template <typename T = void>
struct minimum {
  template <typename A, typename B>
  auto operator()(const A& a, const B& b) const { return b < a ? b : a; }
};

template <typename T>
T select_from_group(const sub_group& sg, T x, size_t src) {
  const size_t base = detail::sg_of(sg.lid) * detail::g_run->sg_size;
  detail::put_slot(sg.lid, x);
  detail::sg_barrier();
  T r = detail::get_slot<T>(base + src);
  detail::sg_barrier();
  return r;
}

inline bool any_of_group(const sub_group& sg, bool p) {
  const size_t s = detail::sg_of(sg.lid), base = s * detail::g_run->sg_size, n = detail::sg_members(s);
  detail::put_slot(sg.lid, p);
  detail::sg_barrier();
  bool r = false;
  for (size_t i = 0; i < n; ++i) r = r || detail::get_slot<bool>(base + i);
  detail::sg_barrier();
  return r;
}

template <typename T, typename Op>
T reduce_over_group(const sub_group& sg, T x, Op op) {
  const size_t s = detail::sg_of(sg.lid), base = s * detail::g_run->sg_size, n = detail::sg_members(s);
  detail::put_slot(sg.lid, x);
  detail::sg_barrier();
  T r = detail::get_slot<T>(base);
  for (size_t i = 1; i < n; ++i) r = static_cast<T>(op(r, detail::get_slot<T>(base + i)));
  detail::sg_barrier();
  return r;
}

template <int D, typename T, typename Op>
T reduce_over_group(const group<D>& g, T x, Op op) {
  detail::put_slot(g.lid, x);
  detail::wg_barrier();
  T r = detail::get_slot<T>(0);
  for (size_t i = 1; i < detail::g_run->wg_size; ++i) r = static_cast<T>(op(r, detail::get_slot<T>(i)));
  detail::wg_barrier();
  return r;
}

// ------------------------------------------------------------------ atomics
enum class memory_order { relaxed, acquire, release, acq_rel, seq_cst };
enum class memory_scope { work_item, sub_group, work_group, device, system };
namespace access {
enum class address_space { global_space, local_space, constant_space, private_space, generic_space };
}

template <typename T, memory_order O = memory_order::relaxed, memory_scope S = memory_scope::device,
          access::address_space A = access::address_space::generic_space>
struct atomic_ref {
  T& r;
  explicit atomic_ref(T& x) : r(x) {}
  T load() const { return r; }
  void store(T v) const { r = v; }
  operator T() const { return r; }
  T operator=(T v) const { return r = v; }
  T fetch_add(T v) const { T o = r; r = static_cast<T>(r + v); return o; }
  T fetch_sub(T v) const { T o = r; r = static_cast<T>(r - v); return o; }
  T fetch_or(T v) const { T o = r; r = static_cast<T>(r | v); return o; }
  T fetch_and(T v) const { T o = r; r = static_cast<T>(r & v); return o; }
  T fetch_max(T v) const { T o = r; r = std::max(r, v); return o; }
  T fetch_min(T v) const { T o = r; r = std::min(r, v); return o; }
  T exchange(T v) const { T o = r; r = v; return o; }
  bool compare_exchange_strong(T& expected, T desired) const {
    if (r == expected) { r = desired; return true; }
    expected = r;
    return false;
  }
  T operator+=(T v) const { return r = static_cast<T>(r + v); }
  T operator-=(T v) const { return r = static_cast<T>(r - v); }
  T operator|=(T v) const { return r = static_cast<T>(r | v); }
  T operator&=(T v) const { return r = static_cast<T>(r & v); }
  T operator++(int) const { return fetch_add(1); }
  T operator++() const { return r = static_cast<T>(r + 1); }
};

// ------------------------------------------------------------------ math / bits
template <typename T>
T popcount(T x) { return static_cast<T>(__builtin_popcountll(static_cast<unsigned long long>(x))); }
template <typename T>
T ctz(T x) {
  if (x == 0) return static_cast<T>(sizeof(T) * 8);
  return static_cast<T>(__builtin_ctzll(static_cast<unsigned long long>(x)));
}
inline float sqrt(float x) { return std::sqrt(x); }
inline double sqrt(double x) { return std::sqrt(x); }
template <typename T>
T min(T a, T b) { return b < a ? b : a; }
template <typename T>
T max(T a, T b) { return a < b ? b : a; }

template <typename T, int N>
struct vec {
  T v[N] = {};
  vec() = default;
  template <typename... A>
  vec(A... a) : v{static_cast<T>(a)...} {}
  T& operator[](int i) { return v[i]; }
  const T& operator[](int i) const { return v[i]; }
};

// ------------------------------------------------------------------ info / events
namespace info {
namespace device {
struct global_mem_size { using return_type = size_t; };
struct max_work_group_size { using return_type = size_t; };
struct name { using return_type = std::string; };
}  // namespace device
namespace queue {
struct device;
}
namespace event_profiling {
struct command_start {};
struct command_end {};
}  // namespace event_profiling
}  // namespace info

class device {
 public:
  template <typename P>
  typename P::return_type get_info() const {
    if constexpr (std::is_same_v<P, info::device::name>) return std::string("host shim");
    else if constexpr (std::is_same_v<P, info::device::global_mem_size>) return size_t(1) << 34;
    else return size_t(1024);
  }
};
namespace info {
namespace queue {
struct device { using return_type = sycl::device; };
}
}  // namespace info

class event {
 public:
  void wait() {}
  void wait_and_throw() {}
  template <typename P>
  uint64_t get_profiling_info() const { return 0; }
};

namespace property {
namespace queue {
struct enable_profiling {};
struct in_order {};
}  // namespace queue
}  // namespace property
struct property_list {
  template <typename... P>
  property_list(P...) {}
};
inline constexpr int gpu_selector_v = 0;
inline constexpr int cpu_selector_v = 0;
inline constexpr int default_selector_v = 0;

// ------------------------------------------------------------------ kernel launch
namespace detail {

constexpr size_t kFiberStack = 64 * 1024;

struct NdLaunch {
  const void* fn;
  void (*call)(const void*, nd_item<1>);
};
inline thread_local NdLaunch g_launch;

inline void fiber_entry() {
  GroupRun& g = *g_run;
  const size_t lid = g.current;
  g_launch.call(g_launch.fn, nd_item<1>{lid});
  g.done[lid] = 1;
  --g.live;
  ++g.progress;
  // returning resumes uc_link (the scheduler)
}

template <typename F>
void run_nd(const nd_range<1>& r, const F& f) {
  const size_t wg = r.local[0];
  const size_t global = r.global[0];
  if (wg == 0 || global % wg) throw std::runtime_error("nd_range: global size not a multiple of the local size");
  const size_t n_groups = global / wg;
  static thread_local std::vector<char> stacks;
  if (stacks.size() < wg * kFiberStack) stacks.assign(wg * kFiberStack, 0);
  GroupRun g;
  g.wg_size = wg;
  g.n_groups = n_groups;
  g.global_size = global;
  g.ctx.resize(wg);
  g.done.assign(wg, 0);
  g.slots.assign(wg * 16, 0);
  const size_t n_sg = (wg + g.sg_size - 1) / g.sg_size;
  g_launch = NdLaunch{&f, [](const void* p, nd_item<1> it) { (*static_cast<const F*>(p))(it); }};
  GroupRun* prev = g_run;
  g_run = &g;
  for (size_t grp = 0; grp < n_groups; ++grp) {
    g.group_id = grp;
    g.wg_arrived = g.wg_gen = 0;
    g.sg_arrived.assign(n_sg, 0);
    g.sg_gen.assign(n_sg, 0);
    std::fill(g.done.begin(), g.done.end(), 0);
    g.live = wg;
    for (size_t i = 0; i < wg; ++i) {
      char* st = stacks.data() + i * kFiberStack;
      std::memset(st, 0xFF, kFiberStack);
      getcontext(&g.ctx[i]);
      g.ctx[i].uc_stack.ss_sp = st;
      g.ctx[i].uc_stack.ss_size = kFiberStack;
      g.ctx[i].uc_link = &g.sched;
      makecontext(&g.ctx[i], fiber_entry, 0);
    }
    // round-robin until every work-item has returned
    while (g.live) {
      const uint64_t before = g.progress;
      bool all_waiting = true;
      for (size_t i = 0; i < wg; ++i) {
        if (g.done[i]) continue;
        g.current = i;
        swapcontext(&g.sched, &g.ctx[i]);
        if (!g.done[i] && !g.waiting) all_waiting = false;
        if (g.done[i]) all_waiting = false;
      }
      if (g.live && all_waiting && g.progress == before) {
        g_run = prev;
        throw std::runtime_error("nd_range kernel: work-items wait on a collective that cannot complete");
      }
    }
  }
  g_run = prev;
}

template <int D, typename F>
void run_range(const range<D>& r, const F& f) {
  if constexpr (D == 1) {
    for (size_t i = 0; i < r.v[0]; ++i) {
      item<1> it;
      it.i.v[0] = i;
      it.r = r;
      if constexpr (std::is_invocable_v<F, item<1>>) f(it);
      else f(id<1>{{i}});
    }
  } else {
    for (size_t a = 0; a < r.v[0]; ++a)
      for (size_t b = 0; b < r.v[1]; ++b) {
        item<2> it;
        it.i.v[0] = a;
        it.i.v[1] = b;
        it.r = r;
        f(it);
      }
  }
}

}  // namespace detail

class handler;

template <typename T, int D = 1>
class local_accessor {
 public:
  std::shared_ptr<std::vector<T>> mem;
  local_accessor(range<D> r, handler&) : mem(std::make_shared<std::vector<T>>(r.size())) {}
  T& operator[](size_t i) const { return (*mem)[i]; }
  T* get_pointer() const { return mem->data(); }
};

class handler {
 public:
  template <typename Name = void, typename F>
  void parallel_for(const nd_range<1>& r, const F& f) { detail::run_nd(r, f); }
  template <typename Name = void, int D, typename F>
  void parallel_for(const range<D>& r, const F& f) { detail::run_range(r, f); }
  template <typename Name = void, typename F>
  void parallel_for(size_t n, const F& f) { detail::run_range(range<1>(n), f); }
  template <typename Name = void, typename F>
  void single_task(const F& f) { f(); }
  void depends_on(const event&) {}
  void depends_on(const std::vector<event>&) {}
  template <typename T>
  void fill(void* p, const T& v, size_t n) {
    T* q = static_cast<T*>(p);
    for (size_t i = 0; i < n; ++i) q[i] = v;
  }
  template <typename T>
  void copy(const T* s, T* d, size_t n) { std::memmove(d, s, n * sizeof(T)); }
  void memcpy(void* d, const void* s, size_t n) { std::memmove(d, s, n); }
  void memset(void* d, int v, size_t n) { std::memset(d, v, n); }
};

class queue {
 public:
  queue() = default;
  template <typename... A>
  explicit queue(A&&...) {}
  template <typename F>
  event submit(F&& f) {
    handler h;
    f(h);
    return event{};
  }
  template <typename Name = void, typename F>
  event parallel_for(const nd_range<1>& r, const F& f) { detail::run_nd(r, f); return {}; }
  template <typename Name = void, int D, typename F>
  event parallel_for(const range<D>& r, const F& f) { detail::run_range(r, f); return {}; }
  template <typename Name = void, typename F>
  event single_task(const F& f) { f(); return {}; }
  template <typename T>
  event fill(void* p, const T& v, size_t n) {
    T* q = static_cast<T*>(p);
    for (size_t i = 0; i < n; ++i) q[i] = v;
    return {};
  }
  template <typename T>
  event copy(const T* s, T* d, size_t n) { std::memmove(d, s, n * sizeof(T)); return {}; }
  event memcpy(void* d, const void* s, size_t n) { std::memmove(d, s, n); return {}; }
  event memset(void* d, int v, size_t n) { std::memset(d, v, n); return {}; }
  void wait() {}
  void wait_and_throw() {}
  sycl::device get_device() const { return {}; }
  template <typename P>
  typename P::return_type get_info() const { return typename P::return_type{}; }
};

// ------------------------------------------------------------------ memory
template <typename T>
T* malloc_device(size_t n, const queue&) {
  return static_cast<T*>(std::calloc(n ? n : 1, sizeof(T)));
}
template <typename T>
T* malloc_host(size_t n, const queue&) {
  return static_cast<T*>(std::calloc(n ? n : 1, sizeof(T)));
}
template <typename T>
T* malloc_shared(size_t n, const queue&) {
  return static_cast<T*>(std::calloc(n ? n : 1, sizeof(T)));
}
inline void free(void* p, const queue&) { std::free(p); }

template <typename T, int D = 1>
class buffer {
 public:
  std::shared_ptr<std::vector<T>> mem;
  explicit buffer(range<D> r) : mem(std::make_shared<std::vector<T>>(r.size())) {}
  explicit buffer(size_t n) : mem(std::make_shared<std::vector<T>>(n)) {}
};

template <typename T, int D = 1>
class host_accessor {
 public:
  std::shared_ptr<std::vector<T>> mem;
  explicit host_accessor(buffer<T, D>& b) : mem(b.mem) {}
  T& operator[](size_t i) const { return (*mem)[i]; }
};

}  // namespace sycl
