// Host graph batches: text parsing and writing in the reference format, CSR
// construction, size filtering.  Follows library/include/graph.hpp:147-310 and
// io.hpp:43-52 of the reference.
#include "graphs.h"

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <system_error>
#include <thread>
#include <fstream>
#include <new>
#include <sstream>

namespace bms {

static thread_local std::string g_thread_error;
void set_thread_error(const std::string& msg) { g_thread_error = msg; }
const char* thread_error() { return g_thread_error.c_str(); }

void append_graph(bms_graphs& g, const std::vector<uint8_t>& labels, const std::vector<Edge>& edges) {
  const uint32_t n = uint32_t(labels.size());
  const uint32_t node_base = uint32_t(g.lab.size());
  const uint32_t entry_base = uint32_t(g.col.size());
  // rows[i]: start of node i's row (local), then its fill cursor
  thread_local std::vector<uint32_t> rows;
  rows.assign(size_t(n) + 1, 0);
  for (const Edge& e : edges) {
    rows[std::get<0>(e) + 1]++;
    rows[std::get<1>(e) + 1]++;
  }
  for (uint32_t i = 1; i <= n; ++i) rows[i] += rows[i - 1];
  const uint32_t entries = rows[n];
  const size_t r0 = g.rowp.size();
  g.rowp.resize(r0 + n);
  for (uint32_t i = 0; i < n; ++i) g.rowp[r0 + i] = entry_base + rows[i + 1];
  // an entry never written (the second slot of a self-loop) holds local id 0
  g.col.resize(size_t(entry_base) + entries, node_base);
  g.elab.resize(size_t(entry_base) + entries, 0);
  uint32_t* col = g.col.data() + entry_base;
  uint8_t* el = g.elab.data() + entry_base;
  for (const Edge& e : edges) {
    // both ends are written before either cursor moves (graph.hpp:229-240): a
    // self-loop writes one slot twice and skips the next
    const uint32_t a = std::get<0>(e), b = std::get<1>(e);
    const uint8_t l = std::get<2>(e);
    const uint32_t ia = rows[a], ib = rows[b];
    col[ia] = node_base + b;
    el[ia] = l;
    col[ib] = node_base + a;
    el[ib] = l;
    rows[a]++;
    rows[b]++;
  }
  g.lab.insert(g.lab.end(), labels.begin(), labels.end());
  g.goff.push_back(node_base + n);
  g.max_nodes = std::max(g.max_nodes, n);
}

namespace {

// whitespace (the characters isspace accepts in the C locale), as a table
struct SpaceTable {
  bool ws[256] = {};
  constexpr SpaceTable() {
    ws[uint8_t(' ')] = ws[uint8_t('\t')] = ws[uint8_t('\r')] = ws[uint8_t('\n')] = true;
    ws[uint8_t('\f')] = ws[uint8_t('\v')] = true;
  }
};
constexpr SpaceTable kSpace{};

// whitespace tokenizer over one line
struct Tok {
  const char* p;
  const char* e;
  bool next(const char*& b, size_t& n) {
    while (p < e && kSpace.ws[uint8_t(*p)]) ++p;
    if (p >= e) return false;
    b = p;
    while (p < e && !kSpace.ws[uint8_t(*p)]) ++p;
    n = size_t(p - b);
    return true;
  }
};

bool to_u64(const char* b, size_t n, uint64_t& out) {
  if (n == 0 || n > 20) return false;
  uint64_t v = 0;
  for (size_t i = 0; i < n; ++i) {
    if (b[i] < '0' || b[i] > '9') return false;
    v = v * 10 + uint64_t(b[i] - '0');
  }
  out = v;
  return true;
}

bool to_i64(const char* b, size_t n, int64_t& out) {
  bool neg = false;
  if (n > 0 && (b[0] == '-' || b[0] == '+')) {
    neg = b[0] == '-';
    ++b;
    --n;
  }
  uint64_t u;
  if (!to_u64(b, n, u)) return false;
  out = neg ? -int64_t(u) : int64_t(u);
  return true;
}

// "n#12": the reference drops the first two characters (token.substr(2)).
bool header(Tok& t, uint64_t& v) {
  const char* b;
  size_t n;
  if (!t.next(b, n) || n < 3) return false;
  return to_u64(b + 2, n - 2, v);
}

}  // namespace

bool parse_line(const char* s, size_t len, std::vector<uint8_t>& labels, std::vector<Edge>& edges, std::string& err) {
  Tok t{s, s + len};
  uint64_t n = 0, nl = 0, ne = 0;
  if (!header(t, n)) {
    err = "expected n#<nodes>";
    return false;
  }
  if (!header(t, nl)) {
    err = "expected l#<labels>";
    return false;
  }
  if (n > (uint64_t(1) << 31)) {
    err = "node count too large";
    return false;
  }
  labels.assign(n, 0);
  for (uint64_t i = 0; i < n; ++i) {
    const char *b1, *b2;
    size_t n1, n2;
    uint64_t id;
    int64_t lab;
    if (!t.next(b1, n1) || !t.next(b2, n2) || !to_u64(b1, n1, id) || !to_i64(b2, n2, lab)) {
      err = "malformed node entry";
      return false;
    }
    if (id >= n) {
      err = "node id out of range";
      return false;
    }
    labels[id] = uint8_t(lab);  // label_t = uint8 (types.hpp:12), int truncated
  }
  if (!header(t, ne)) {
    err = "expected e#<edges>";
    return false;
  }
  thread_local std::vector<std::pair<const char*, size_t>> toks;
  toks.clear();
  const char* b;
  size_t k;
  while (t.next(b, k)) toks.emplace_back(b, k);
  edges.clear();
  size_t per;
  if (toks.size() == ne * 3) per = 3;
  else if (toks.size() == ne * 2) per = 2;
  else {
    err = "Invalid graph format";  // graph.hpp:200
    return false;
  }
  edges.reserve(ne);
  for (uint64_t i = 0; i < ne; ++i) {
    uint64_t u, v;
    int64_t l = 0;
    if (!to_u64(toks[i * per].first, toks[i * per].second, u) ||
        !to_u64(toks[i * per + 1].first, toks[i * per + 1].second, v) ||
        (per == 3 && !to_i64(toks[i * per + 2].first, toks[i * per + 2].second, l))) {
      err = "malformed edge entry";
      return false;
    }
    if (u >= n || v >= n) {
      err = "edge endpoint out of range";
      return false;
    }
    edges.emplace_back(uint32_t(u), uint32_t(v), uint8_t(l));
  }
  return true;
}

}  // namespace bms

using bms::set_thread_error;

namespace {

// Serial parse of one buffer; a malformed line is reported with its number
// counted from first_line, or (bad_line given) that number is stored there and
// the message carries only ": <reason>".
int parse_serial(const char* text, size_t len, uint32_t max_graphs, int skip_invalid, size_t first_line,
                 bms_graphs** out, size_t* bad_line = nullptr) {
  if (!out) return BMS_EINVAL;
  *out = nullptr;
  bms_graphs* g = new (std::nothrow) bms_graphs();
  if (!g) return BMS_ENOMEM;
  std::vector<uint8_t> labels;
  std::vector<bms::Edge> edges;
  std::string err;
  size_t line_no = first_line;
  const char* p = text;
  const char* end = text + len;
  try {
    while (p < end) {
      const char* nl = static_cast<const char*>(std::memchr(p, '\n', size_t(end - p)));
      const char* le = nl ? nl : end;
      ++line_no;
      bool blank = true;
      for (const char* q = p; q < le; ++q)
        if (!(*q == ' ' || *q == '\t' || *q == '\r')) {
          blank = false;
          break;
        }
      if (!blank) {
        if (max_graphs && g->n_graphs() >= max_graphs) break;
        if (bms::parse_line(p, size_t(le - p), labels, edges, err)) {
          if (g->lab.size() + labels.size() > 0xFFFFFFF0ull || g->col.size() + 2 * edges.size() > 0xFFFFFFF0ull) {
            delete g;
            set_thread_error("batch exceeds 32-bit node or entry ids");
            return BMS_EUNSUPPORTED;
          }
          bms::append_graph(*g, labels, edges);
        } else if (!skip_invalid) {
          delete g;
          if (bad_line) {  // the caller numbers the line
            *bad_line = line_no;
            set_thread_error(": " + err);
          } else {
            set_thread_error("line " + std::to_string(line_no) + ": " + err);
          }
          return BMS_EINVAL;
        }
      }
      p = nl ? nl + 1 : end;
    }
  } catch (const std::bad_alloc&) {
    delete g;
    set_thread_error("out of host memory while parsing");
    return BMS_ENOMEM;
  }
  *out = g;
  return BMS_OK;
}

// Concatenate the pieces of a parallel parse into one batch (ids rebased):
// the result is sized once and every piece copies its part in its own
// thread.  False if the 32-bit id space overflows.
bool merge_batches(const std::vector<bms_graphs*>& part, bms_graphs& g) {
  const size_t n = part.size();
  std::vector<uint64_t> g0(n + 1, 0), n0(n + 1, 0), e0(n + 1, 0);
  for (size_t k = 0; k < n; ++k) {
    g0[k + 1] = g0[k] + part[k]->n_graphs();
    n0[k + 1] = n0[k] + part[k]->lab.size();
    e0[k + 1] = e0[k] + part[k]->col.size();
  }
  if (n0[n] > 0xFFFFFFF0ull || e0[n] > 0xFFFFFFF0ull) return false;
  g.goff.assign(g0[n] + 1, 0);
  g.rowp.assign(n0[n] + 1, 0);
  g.col.resize(e0[n]);
  g.lab.resize(n0[n]);
  g.elab.resize(e0[n]);
  g.max_nodes = 0;
  for (const bms_graphs* b : part) g.max_nodes = std::max(g.max_nodes, b->max_nodes);
  auto copy = [&](size_t k) {
    const bms_graphs& b = *part[k];
    const uint32_t nb = uint32_t(n0[k]), eb = uint32_t(e0[k]);
    for (size_t i = 1; i < b.goff.size(); ++i) g.goff[g0[k] + i] = nb + b.goff[i];
    for (size_t i = 1; i < b.rowp.size(); ++i) g.rowp[n0[k] + i] = eb + b.rowp[i];
    for (size_t i = 0; i < b.col.size(); ++i) g.col[e0[k] + i] = nb + b.col[i];
    std::copy(b.lab.begin(), b.lab.end(), g.lab.begin() + ptrdiff_t(n0[k]));
    std::copy(b.elab.begin(), b.elab.end(), g.elab.begin() + ptrdiff_t(e0[k]));
  };
  std::vector<std::thread> pool;
  for (size_t k = 1; k < n; ++k) {
    try {
      pool.emplace_back(copy, k);
    } catch (const std::system_error&) {
      copy(k);  // no thread to spare: this piece on the calling thread
    }
  }
  copy(0);
  for (auto& t : pool) t.join();
  return true;
}

// Large buffers without a graph limit are split at line boundaries and parsed
// by several threads; the pieces are concatenated in order, so the result (and
// the line number of the first malformed line) equals a serial parse.
int parse_buffer(const char* text, size_t len, uint32_t max_graphs, int skip_invalid, bms_graphs** out) {
  constexpr size_t kMinPiece = 8u << 20;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t pieces = std::min<size_t>(std::min<size_t>(hw, 64), len / kMinPiece);
  if (max_graphs || pieces < 2) return parse_serial(text, len, max_graphs, skip_invalid, 0, out);
  if (!out) return BMS_EINVAL;
  *out = nullptr;
  std::vector<size_t> cut{0};
  for (size_t k = 1; k < pieces; ++k) {
    size_t at = std::max(cut.back(), len * k / pieces);
    const void* nl = at < len ? std::memchr(text + at, '\n', len - at) : nullptr;
    at = nl ? size_t(static_cast<const char*>(nl) - text) + 1 : len;
    cut.push_back(at);
  }
  cut.push_back(len);
  const size_t n = cut.size() - 1;
  std::vector<bms_graphs*> part(n, nullptr);
  std::vector<int> status(n, BMS_OK);
  std::vector<size_t> lines(n, 0), bad_line(n, 0);  // lines of each piece; a malformed line's number in it
  std::vector<std::string> msg(n);
  auto piece = [&](size_t k) {
    const char* b = text + cut[k];
    const size_t m = cut[k + 1] - cut[k];
    status[k] = parse_serial(b, m, 0, skip_invalid, 0, &part[k], &bad_line[k]);
    if (status[k] != BMS_OK) msg[k] = bms::thread_error();
    lines[k] = size_t(std::count(b, b + m, '\n'));
  };
  std::vector<std::thread> pool;
  for (size_t k = 0; k < n; ++k) {
    try {
      pool.emplace_back(piece, k);
    } catch (const std::system_error&) {
      piece(k);  // no thread to spare: this piece on the calling thread
    }
  }
  for (auto& t : pool) t.join();
  int r = BMS_OK;
  size_t before = 0;  // lines before piece k
  for (size_t k = 0; k < n && r == BMS_OK; ++k) {
    if (status[k] != BMS_OK) {
      r = status[k];
      // a malformed line: its number counted from the start of the buffer
      set_thread_error(bad_line[k] ? "line " + std::to_string(before + bad_line[k]) + msg[k] : msg[k]);
    }
    before += lines[k];
  }
  bms_graphs* g = nullptr;
  if (r == BMS_OK) {
    g = new (std::nothrow) bms_graphs();
    if (!g) {
      set_thread_error("out of host memory while parsing");
      r = BMS_ENOMEM;
    }
  }
  try {
    if (r == BMS_OK && !merge_batches(part, *g)) {
      set_thread_error("batch exceeds 32-bit node or entry ids");
      r = BMS_EUNSUPPORTED;
    }
  } catch (const std::bad_alloc&) {
    set_thread_error("out of host memory while parsing");
    r = BMS_ENOMEM;
  }
  for (bms_graphs* b : part) delete b;
  if (r != BMS_OK) {
    delete g;
    return r;
  }
  *out = g;
  return BMS_OK;
}

}  // namespace

extern "C" {

const char* bms_status_name(int s) {
  switch (s) {
    case BMS_OK: return "BMS_OK";
    case BMS_EINVAL: return "BMS_EINVAL";
    case BMS_ENOMEM: return "BMS_ENOMEM";
    case BMS_ECUDA: return "BMS_ECUDA";
    case BMS_EIO: return "BMS_EIO";
    case BMS_ESTATE: return "BMS_ESTATE";
    case BMS_EUNSUPPORTED: return "BMS_EUNSUPPORTED";
    case BMS_ETIMEDOUT: return "BMS_ETIMEDOUT";
    case BMS_EINCOMPLETE: return "BMS_EINCOMPLETE";
    case BMS_ENODEV: return "BMS_ENODEV";
    default: return "BMS_E?";
  }
}

int bms_abi_version(void) { return BMS_ABI_VERSION; }

int bms_graphs_parse_text(const char* text, size_t len, uint32_t max_graphs, int skip_invalid, bms_graphs** out) {
  if (!text && len) return BMS_EINVAL;
  return parse_buffer(text ? text : "", len, max_graphs, skip_invalid, out);
}

int bms_graphs_parse_file(const char* path, uint32_t max_graphs, int skip_invalid, bms_graphs** out) {
  if (!path || !out) return BMS_EINVAL;
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_thread_error(std::string("cannot open ") + path + ": " + std::strerror(errno));
    return BMS_EIO;
  }
  // one read of the file's size where it has one, then any remainder in chunks
  std::vector<char> buf;
  size_t len = 0;
  if (std::fseek(f, 0, SEEK_END) == 0) {
    const long sz = std::ftell(f);
    if (sz > 0) buf.reserve(size_t(sz));
    std::rewind(f);
  }
  try {
    if (buf.capacity()) {
      buf.resize(buf.capacity());
      len = std::fread(buf.data(), 1, buf.size(), f);
    }
    char chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) {
      if (len + k > buf.size()) buf.resize(std::max(buf.size() * 2, len + k));
      std::memcpy(buf.data() + len, chunk, k);
      len += k;
    }
  } catch (const std::bad_alloc&) {
    std::fclose(f);
    set_thread_error("out of host memory while reading");
    return BMS_ENOMEM;
  }
  bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) {
    set_thread_error(std::string("read error on ") + path);
    return BMS_EIO;
  }
  return parse_buffer(buf.data(), len, max_graphs, skip_invalid, out);
}

int bms_graphs_from_csr(uint32_t G, const uint32_t* goff, const uint32_t* rowp, const uint32_t* col,
                        const uint8_t* lab, const uint8_t* elab, bms_graphs** out) {
  if (!out || !goff || (G && (!rowp || !lab))) return BMS_EINVAL;
  *out = nullptr;
  if (goff[0] != 0) {
    set_thread_error("graph_offsets[0] must be 0");
    return BMS_EINVAL;
  }
  for (uint32_t i = 0; i < G; ++i)
    if (goff[i + 1] < goff[i]) {
      set_thread_error("graph_offsets must be non-decreasing");
      return BMS_EINVAL;
    }
  const uint64_t N = goff[G];
  if (N && rowp[0] != 0) {
    set_thread_error("row_offsets[0] must be 0");
    return BMS_EINVAL;
  }
  for (uint64_t v = 0; v < N; ++v)
    if (rowp[v + 1] < rowp[v]) {
      set_thread_error("row_offsets must be non-decreasing");
      return BMS_EINVAL;
    }
  const uint64_t E = N ? rowp[N] : 0;
  if (E && !col) return BMS_EINVAL;
  bms_graphs* g = new (std::nothrow) bms_graphs();
  if (!g) return BMS_ENOMEM;
  try {
    g->goff.assign(goff, goff + G + 1);
    g->rowp.assign(rowp, rowp + N + 1);
    if (!N) g->rowp.assign(1, 0);
    g->col.assign(col, col + E);
    g->lab.assign(lab, lab + N);
    if (elab) g->elab.assign(elab, elab + E);
    else g->elab.assign(E, 0);
  } catch (const std::bad_alloc&) {
    delete g;
    return BMS_ENOMEM;
  }
  for (uint32_t i = 0; i < G; ++i) g->max_nodes = std::max(g->max_nodes, goff[i + 1] - goff[i]);
  *out = g;
  return BMS_OK;
}

int bms_graphs_view_of(const bms_graphs* g, bms_graphs_view* v) {
  if (!g || !v) return BMS_EINVAL;
  v->n_graphs = g->n_graphs();
  v->max_nodes = g->max_nodes;
  v->n_nodes = g->lab.size();
  v->n_entries = g->col.size();
  v->graph_offsets = g->goff.data();
  v->row_offsets = g->rowp.data();
  v->column_indices = g->col.data();
  v->node_labels = g->lab.data();
  v->edge_labels = g->elab.data();
  return BMS_OK;
}

// One line per graph: "n#N l#11 0 L0 1 L1 ... e#E u v l ...".  Each undirected
// edge is written once, taken from the CSR entries with u <= v in row order;
// a CSR built by append_graph from such a line reproduces the same batch when
// the graph has no self-loops.
int bms_graphs_write_file(const bms_graphs* g, const char* path) {
  if (!g || !path) return BMS_EINVAL;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    set_thread_error(std::string("cannot open ") + path + ": " + std::strerror(errno));
    return BMS_EIO;
  }
  std::string line;
  bool ok = true;
  for (uint32_t gi = 0; gi < g->n_graphs() && ok; ++gi) {
    const uint32_t b = g->goff[gi], e = g->goff[gi + 1];
    line.clear();
    line += "n#" + std::to_string(e - b) + " l#11";
    for (uint32_t v = b; v < e; ++v) line += " " + std::to_string(v - b) + " " + std::to_string(unsigned(g->lab[v]));
    std::string el;
    uint64_t ne = 0;
    for (uint32_t v = b; v < e; ++v)
      for (uint32_t i = g->rowp[v]; i < g->rowp[v + 1]; ++i) {
        const uint32_t w = g->col[i];
        if (w < v) continue;
        el += " " + std::to_string(v - b) + " " + std::to_string(w - b) + " " + std::to_string(unsigned(g->elab[i]));
        ++ne;
      }
    line += " e#" + std::to_string(ne) + el + "\n";
    ok = std::fwrite(line.data(), 1, line.size(), f) == line.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    set_thread_error(std::string("write error on ") + path);
    return BMS_EIO;
  }
  return BMS_OK;
}

int bms_graphs_filter_size(const bms_graphs* g, uint32_t min_nodes, uint32_t max_nodes, bms_graphs** out) {
  if (!g || !out) return BMS_EINVAL;
  bms_graphs* r = new (std::nothrow) bms_graphs();
  if (!r) return BMS_ENOMEM;
  for (uint32_t gi = 0; gi < g->n_graphs(); ++gi) {
    const uint32_t b = g->goff[gi], e = g->goff[gi + 1], n = e - b;
    if (n < min_nodes || n > max_nodes) continue;
    const uint32_t node_base = uint32_t(r->lab.size());
    const uint32_t entry_base = uint32_t(r->col.size());
    for (uint32_t v = b; v < e; ++v) {
      r->lab.push_back(g->lab[v]);
      r->rowp.push_back(entry_base + (g->rowp[v + 1] - g->rowp[b]));
    }
    for (uint32_t i = g->rowp[b]; i < g->rowp[e]; ++i) {
      r->col.push_back(g->col[i] - b + node_base);
      r->elab.push_back(g->elab[i]);
    }
    r->goff.push_back(node_base + n);
    r->max_nodes = std::max(r->max_nodes, n);
  }
  *out = r;
  return BMS_OK;
}

void bms_graphs_free(bms_graphs* g) { delete g; }

}  // extern "C"
