// Plan façade: executes the reference's JSON plans (the operator names and
// fields of core/olap/lib/plan/plan-parser.cpp) on resident device columns
// by lowering each operator onto the C ABI.
//
// Operators: scan (plugin.name + projections, plan-parser.cpp scan cases),
// select (p), project (e), sort (e[{expression, direction}], :353-389),
// hash-rearrange / hash-pack (e, projections, buckets; :1424-1458),
// hashjoin-chained (build_input, probe_input, build_k, probe_k,
// hash_bits, maxBuildInputSize; plan-parser.cpp:977-1006),
// partitioned-hashjoin-chained (:851-976) and join (radix; p{eq},
// leftInput, rightInput; :1007-1139), groupby / hashgroupby-chained (input,
// k, e[{e, m, packet, offset}], hash_bits, maxInputSize; :479-530) and
// reduce (e, accumulator, p; :248-286), nest (RadixNest: f, p, e,
// accumulator, aggrLabels, g, fields; :1140-1268), print / project /
// materializer over a result, and the data-movement operators that leave a
// relation unchanged on one GPU (block-to-tuples, unpack, pack,
// tuples-to-block, cpu-to-gpu, gpu-to-cpu, mem-move-device,
// mem-broadcast-device, mem-move-local-to, router, exchange).  Expressions
// (expression-parser.cpp): recordProjection, argument, int, int64, bool,
// cast, eq, lt, le, gt, ge, and, multiply.  Accumulators: sum, max, min, or,
// and.  Every field of an operator is either honoured or rejected: an
// operator or field the façade does not know (or a value it cannot honour)
// fails with GBJ_ERR_UNSUPPORTED and a message naming it.  Placement and
// layout fields (gpu, blockwise, output, build_w / build_e packets, ...)
// select where and in which packed layout the reference runs an operator;
// here every operator runs on this GPU over columns, so they do not change
// a result and are accepted.
//
// Lowering: reduce over a join whose output expressions read at most one
// build column and one probe column runs as one fused probe + aggregate
// (gbj_join_probe_agg for hashjoin-chained, gbj_radix_join_agg for the
// partitioned / radix joins), as the reference's generated pipeline fuses
// them; other joins materialise (build row, probe row) pairs and gather the
// columns their parents read.  Sizing fields are capacity hints.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "gbj_internal.cuh"

using namespace gbj;

namespace {

// ------------------------------------------------------------------- JSON
struct JVal {
  enum Type { Null, Bool, Num, Str, Arr, Obj } t = Null;
  bool b = false;
  double num = 0;
  int64_t i = 0;
  bool is_int = false;
  std::string s;
  std::vector<JVal> a;
  std::vector<std::pair<std::string, JVal>> o;
  const JVal *get(const char *k) const {
    if (t != Obj) return nullptr;
    for (const auto &kv : o)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct PlanError {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string &msg) { throw PlanError{code, msg}; }

class JsonParser {
 public:
  explicit JsonParser(const char *p) : p_(p) {}
  JVal parse() {
    JVal v = value();
    ws();
    if (*p_) fail(GBJ_ERR_INVALID, "plan: trailing characters after JSON value");
    return v;
  }

 private:
  const char *p_;
  int depth_ = 0;
  void ws() {
    while (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r') ++p_;
  }
  JVal value() {
    if (++depth_ > 256) fail(GBJ_ERR_INVALID, "plan: JSON nested too deeply");
    ws();
    JVal v;
    const char c = *p_;
    if (c == '{') {
      v.t = JVal::Obj;
      ++p_;
      ws();
      if (*p_ == '}') {
        ++p_;
      } else {
        for (;;) {
          ws();
          if (*p_ != '"') fail(GBJ_ERR_INVALID, "plan: expected a string key");
          std::string k = str();
          ws();
          if (*p_ != ':') fail(GBJ_ERR_INVALID, "plan: expected ':'");
          ++p_;
          v.o.emplace_back(std::move(k), value());
          ws();
          if (*p_ == ',') { ++p_; continue; }
          if (*p_ == '}') { ++p_; break; }
          fail(GBJ_ERR_INVALID, "plan: expected ',' or '}'");
        }
      }
    } else if (c == '[') {
      v.t = JVal::Arr;
      ++p_;
      ws();
      if (*p_ == ']') {
        ++p_;
      } else {
        for (;;) {
          v.a.push_back(value());
          ws();
          if (*p_ == ',') { ++p_; continue; }
          if (*p_ == ']') { ++p_; break; }
          fail(GBJ_ERR_INVALID, "plan: expected ',' or ']'");
        }
      }
    } else if (c == '"') {
      v.t = JVal::Str;
      v.s = str();
    } else if (!strncmp(p_, "true", 4)) {
      v.t = JVal::Bool, v.b = true, p_ += 4;
    } else if (!strncmp(p_, "false", 5)) {
      v.t = JVal::Bool, v.b = false, p_ += 5;
    } else if (!strncmp(p_, "null", 4)) {
      p_ += 4;
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      v.t = JVal::Num;
      const char *st = p_;
      if (*p_ == '-') ++p_;
      while (*p_ >= '0' && *p_ <= '9') ++p_;
      v.is_int = !(*p_ == '.' || *p_ == 'e' || *p_ == 'E');
      if (v.is_int) {
        v.i = strtoll(st, nullptr, 10);
        v.num = (double)v.i;
      } else {
        char *end = nullptr;
        v.num = strtod(st, &end);
        p_ = end;
        v.i = (int64_t)v.num;
      }
    } else {
      fail(GBJ_ERR_INVALID, "plan: malformed JSON");
    }
    --depth_;
    return v;
  }
  std::string str() {
    std::string out;
    ++p_;  // opening quote
    while (*p_ && *p_ != '"') {
      if (*p_ == '\\') {
        ++p_;
        switch (*p_) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u':  // names here are ASCII: a \uXXXX escape becomes '?'
            out += '?';
            for (int k = 0; k < 4 && p_[1]; ++k) ++p_;
            break;
          default: out += *p_;
        }
        if (*p_) ++p_;
      } else {
        out += *p_++;
      }
    }
    if (*p_ != '"') fail(GBJ_ERR_INVALID, "plan: unterminated string");
    ++p_;
    return out;
  }
};

const JVal &need(const JVal &v, const char *k, const char *op) {
  const JVal *x = v.get(k);
  if (!x) fail(GBJ_ERR_INVALID, std::string("plan: operator '") + op + "' needs field '" + k + "'");
  return *x;
}

std::string op_name(const JVal &v) {
  const JVal *o = v.get("operator");
  if (!o || o->t != JVal::Str) fail(GBJ_ERR_INVALID, "plan: node without an \"operator\" string");
  return o->s;
}

std::string expr_name(const JVal &e) {
  const JVal *x = e.get("expression");
  if (!x || x->t != JVal::Str) fail(GBJ_ERR_INVALID, "plan: expression without an \"expression\" string");
  return x->s;
}

// Strips cast wrappers (int64 accumulation is how the library aggregates).
const JVal &uncast(const JVal &e) {
  const JVal *x = &e;
  while (expr_name(*x) == "cast") x = &need(*x, "e", "cast");
  return *x;
}

// (relName, attrName) of a recordProjection.
std::pair<std::string, std::string> projection(const JVal &e) {
  const JVal &x = uncast(e);
  if (expr_name(x) != "recordProjection")
    fail(GBJ_ERR_UNSUPPORTED, "plan: expected a column (recordProjection), got '" + expr_name(x) + "'");
  const JVal &a = need(x, "attribute", "recordProjection");
  const JVal *rel = a.get("relName"), *attr = a.get("attrName");
  if (!attr || attr->t != JVal::Str) fail(GBJ_ERR_INVALID, "plan: attribute without attrName");
  return {rel && rel->t == JVal::Str ? rel->s : std::string(), attr->s};
}

bool is_const(const JVal &e, int64_t *v) {
  const JVal &x = uncast(e);
  const std::string n = expr_name(x);
  if (n != "int" && n != "int64") return false;
  const JVal *c = x.get("v");
  if (!c || c->t != JVal::Num) fail(GBJ_ERR_INVALID, "plan: constant without \"v\"");
  *v = c->i;
  return true;
}

// expression-parser.cpp:781-800 (parseAccumulator); or / and are the
// logical monoids (gmonoids.cpp:363-376).
int monoid(const std::string &m) {
  if (m == "sum") return GBJ_AGG_SUM;
  if (m == "max") return GBJ_AGG_MAX;
  if (m == "min") return GBJ_AGG_MIN;
  if (m == "or") return GBJ_AGG_OR;
  if (m == "and") return GBJ_AGG_AND;
  fail(GBJ_ERR_UNSUPPORTED,
       "plan: accumulator '" + m + "' is not supported (sum, max, min, or, and are)");
}

// Operators that move or re-route a relation without changing it (the
// reference's device crossings, packers and routers): on one GPU over
// resident columns they are the identity.
bool passthrough(const std::string &op) {
  static const std::set<std::string> k = {"block-to-tuples", "unpack", "pack", "tuples-to-block",
                                          "cpu-to-gpu", "gpu-to-cpu", "mem-move-device",
                                          "mem-broadcast-device", "mem-move-local-to", "router",
                                          "exchange"};
  return k.count(op) != 0;
}

// The fields each operator may carry: the ones plan-parser.cpp reads for it,
// plus the placement / layout fields its plans carry.  Anything else is
// refused, so no field is ever silently ignored.
void check_fields(const JVal &v, const std::string &op) {
  static const std::set<std::string> placement = {"operator", "gpu", "blockwise", "output",
                                                  "max_line_estimate", "jumpTo"};
  static const std::map<std::string, std::set<std::string>> fields = {
      {"scan", {"plugin"}},
      {"select", {"input", "p"}},
      {"project", {"input", "e", "relName"}},
      {"print", {"input", "e", "plugin"}},
      {"materializer", {"input", "e", "w"}},
      {"sort", {"input", "e", "granularity", "rowType"}},
      {"hashjoin-chained",
       {"build_input", "probe_input", "build_k", "probe_k", "hash_bits", "maxBuildInputSize", "build_e",
        "build_w", "probe_e", "probe_w"}},
      {"partitioned-hashjoin-chained",
       {"build_input", "probe_input", "build_k", "probe_k", "build_k_minor", "probe_k_minor", "hash_bits",
        "maxBuildInputSize", "maxProbeInputSize", "build_e", "build_w", "probe_e", "probe_w"}},
      {"join",
       {"p", "leftInput", "rightInput", "leftFields", "rightFields", "build_e", "build_w", "probe_e",
        "probe_w"}},
      {"groupby", {"input", "k", "e", "hash_bits", "maxInputSize", "w"}},
      {"hashgroupby-chained", {"input", "k", "e", "hash_bits", "maxInputSize", "w"}},
      {"reduce", {"input", "e", "accumulator", "p"}},
      {"nest", {"input", "accumulator", "aggrLabels", "e", "p", "f", "g", "fields"}},
      {"hash-rearrange", {"input", "e", "projections", "buckets", "hashProject"}},
      {"hash-pack", {"input", "e", "projections", "buckets", "hashProject"}},
      {"block-to-tuples", {"input", "projections"}},
      {"unpack", {"input", "projections"}},
      {"pack", {"input", "projections", "trait"}},
      {"tuples-to-block", {"input", "projections", "trait"}},
      {"cpu-to-gpu", {"input", "projections", "queueSize", "granularity"}},
      {"gpu-to-cpu", {"input", "projections", "queueSize", "granularity"}},
      {"mem-move-device", {"input", "projections", "do_transfer", "split_id", "to_cpu", "slack"}},
      {"mem-broadcast-device", {"input", "projections", "always_share", "num_of_targets", "to_cpu"}},
      {"mem-move-local-to", {"input", "projections", "slack"}},
      {"router",
       {"input", "numOfParents", "num_of_targets", "slack", "target", "cpu_targets", "numa_local",
        "rand_local_cpu", "producers", "projections", "split_id"}},
      {"exchange",
       {"input", "numOfParents", "num_of_targets", "slack", "target", "cpu_targets", "numa_local",
        "rand_local_cpu", "producers", "projections", "split_id"}},
  };
  auto it = fields.find(op);
  if (it == fields.end()) return;
  for (const auto &kv : v.o)
    if (!placement.count(kv.first) && !it->second.count(kv.first))
      fail(GBJ_ERR_UNSUPPORTED, "plan: field '" + kv.first + "' of operator '" + op + "' is not supported");
}

// Walks a plan checking operator names and fields (no GPU work).
void validate(const JVal &v) {
  const std::string op = op_name(v);
  check_fields(v, op);
  if (passthrough(op)) {
    validate(need(v, "input", op.c_str()));
  } else if (op == "print") {
    validate(need(v, "input", "print"));
  } else if (op == "materializer") {
    need(v, "e", "materializer");
    validate(need(v, "input", "materializer"));
  } else if (op == "nest") {
    const JVal &acc = need(v, "accumulator", "nest");
    const JVal &e = need(v, "e", "nest");
    const JVal &labels = need(v, "aggrLabels", "nest");
    if (acc.a.size() != e.a.size() || labels.a.size() != e.a.size())
      fail(GBJ_ERR_INVALID, "plan: nest needs one accumulator and one label per expression");
    for (const JVal &a : acc.a) monoid(a.s);
    need(v, "f", "nest");
    need(v, "p", "nest");
    validate(need(v, "input", "nest"));
  } else if (op == "scan") {
    const JVal &pl = need(v, "plugin", "scan");
    need(pl, "name", "scan plugin");
  } else if (op == "select") {
    need(v, "p", "select");
    validate(need(v, "input", "select"));
  } else if (op == "hashjoin-chained" || op == "partitioned-hashjoin-chained") {
    need(v, "build_k", op.c_str());
    need(v, "probe_k", op.c_str());
    if (!v.get("build_k_minor") != !v.get("probe_k_minor"))
      fail(GBJ_ERR_INVALID, "plan: " + op + " needs build_k_minor and probe_k_minor together "
                            "(the reference checks the minor key only when both are given)");
    validate(need(v, "build_input", op.c_str()));
    validate(need(v, "probe_input", op.c_str()));
  } else if (op == "join") {
    need(v, "p", "join");
    validate(need(v, "leftInput", "join"));
    validate(need(v, "rightInput", "join"));
  } else if (op == "groupby" || op == "hashgroupby-chained") {
    need(v, "k", op.c_str());
    const JVal &e = need(v, "e", op.c_str());
    for (const JVal &x : e.a) {
      need(x, "e", op.c_str());
      monoid(need(x, "m", op.c_str()).s);
    }
    validate(need(v, "input", op.c_str()));
  } else if (op == "reduce") {
    const JVal &acc = need(v, "accumulator", "reduce");
    for (const JVal &a : acc.a) monoid(a.s);
    need(v, "e", "reduce");
    validate(need(v, "input", "reduce"));
  } else if (op == "sort") {
    const JVal &e = need(v, "e", "sort");
    for (const JVal &x : e.a) {
      need(x, "expression", "sort");
      const std::string d = need(x, "direction", "sort").s;
      if (d != "ASC" && d != "DESC" && d != "NONE")
        fail(GBJ_ERR_INVALID, "plan: sort direction '" + d + "' (ASC, DESC, NONE)");
    }
    validate(need(v, "input", "sort"));
  } else if (op == "project") {
    need(v, "e", "project");
    validate(need(v, "input", "project"));
  } else if (op == "hash-rearrange" || op == "hash-pack") {
    need(v, "e", op.c_str());
    need(v, "projections", op.c_str());
    validate(need(v, "input", op.c_str()));
  } else {
    fail(GBJ_ERR_UNSUPPORTED, "plan: operator '" + op +
                                  "' is not supported (scan, select, project, print, materializer, sort, "
                                  "hashjoin-chained, partitioned-hashjoin-chained, join, groupby, "
                                  "hashgroupby-chained, nest, reduce, hash-rearrange, hash-pack and the "
                                  "data-movement operators are)");
  }
}

// Output name of an expression: its register_as attribute, else `dflt`.
std::string out_name(const JVal &e, const std::string &dflt) {
  if (const JVal *r = e.get("register_as"))
    if (const JVal *a = r->get("attrName"))
      if (a->t == JVal::Str) return a->s;
  return dflt;
}

// ---------------------------------------------------------- kernels
// truth[i] = lo <= col[i] <= hi (mode 0) or col[i] != 0 (mode 1); with
// and_into the result is ANDed into truth.
__global__ void k_truth(const int32_t *__restrict__ col, uint64_t n, int mode, int32_t lo, int32_t hi,
                        int and_into, int32_t *__restrict__ truth) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t v = col[i];
    const int32_t t = mode == 0 ? (v >= lo && v <= hi) : (v != 0);
    truth[i] = and_into ? (truth[i] & t) : t;
  }
}

__global__ void k_widen(const int32_t *__restrict__ col, uint64_t n, int64_t *__restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = col[i];
}

// flag[i] = bminor[brow[i]] == pminor[prow[i]] (the minor-key check over
// materialised join pairs).
__global__ void k_pair_eq(const int32_t *__restrict__ bminor, const int32_t *__restrict__ pminor,
                          const int32_t *__restrict__ brow, const int32_t *__restrict__ prow, uint64_t n,
                          int32_t *__restrict__ flag) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    flag[i] = bminor[brow[i]] == pminor[prow[i]];
}

}  // namespace

// ------------------------------------------------------------- catalog
struct gbj_catalog {
  gbj_ctx *ctx = nullptr;
  struct Col {
    const int32_t *d;
    uint64_t n;
  };
  std::map<std::pair<std::string, std::string>, Col> cols;
  std::map<std::string, std::vector<std::string>> rel_attrs;
  std::vector<void *> owned;  // pool blocks of columns loaded from files
};

struct gbj_result {
  std::vector<std::string> names;
  std::vector<std::vector<int64_t>> cols;
  uint64_t rows = 0;
};

namespace {

// A relation during execution: int32 device columns of equal length.
struct Rel {
  uint64_t n = 0;
  struct C {
    std::string rel, attr;
    const int32_t *d;
  };
  std::vector<C> cols;
  const C *find(const std::pair<std::string, std::string> &ra) const {
    for (const C &c : cols)
      if (c.attr == ra.second && (ra.first.empty() || c.rel.empty() || c.rel == ra.first)) return &c;
    return nullptr;
  }
};

class Exec {
 public:
  Exec(gbj_catalog *cat) : cat_(cat), ctx_(cat->ctx) {}
  ~Exec() {
    for (void *p : allocs_) gbj_pool_free(ctx_, p);
  }

  static bool is_agg(const std::string &op) {
    return op == "reduce" || op == "groupby" || op == "hashgroupby-chained" || op == "nest";
  }
  // Whether an aggregate sits below print / project / materializer / sort
  // wrappers (their lists then select from the aggregate's result).
  static bool agg_below(const JVal &v) {
    const std::string op = op_name(v);
    if (is_agg(op)) return true;
    if (op == "print" || op == "project" || op == "materializer" || op == "sort")
      return agg_below(need(v, "input", op.c_str()));
    return false;
  }

  gbj_result *run(const JVal &root) {
    auto res = std::make_unique<gbj_result>();
    // print and, over an aggregate, project / materializer only choose and
    // rename result columns: peel them, apply their lists at the end
    std::vector<const JVal *> lists;  // outermost first
    const JVal *node = &root;
    for (;;) {
      const std::string op = op_name(*node);
      if (op != "print" && op != "project" && op != "materializer") break;
      const JVal &in = need(*node, "input", op.c_str());
      if (op != "print" && !agg_below(in)) break;
      if (const JVal *e = node->get("e")) lists.push_back(e);
      node = &in;
    }
    const std::string op = op_name(*node);
    const std::string iop = op == "sort" ? op_name(need(*node, "input", "sort")) : std::string();
    if (is_agg(op)) {
      aggregate(*node, res.get());
    } else if (op == "sort" && is_agg(iop)) {
      // ORDER BY over an aggregate's (small, int64) result: ordered on the host
      aggregate(need(*node, "input", "sort"), res.get());
      host_sort(*node, res.get());
    } else {
      const Rel r = rel(*node);
      res->rows = r.n;
      for (const auto &c : r.cols) {
        res->names.push_back(c.rel.empty() ? c.attr : c.rel + "." + c.attr);
        res->cols.push_back(to_host32(c.d, r.n));
      }
    }
    for (auto it = lists.rbegin(); it != lists.rend(); ++it) select_columns(**it, res.get());
    return res.release();
  }

 private:
  void aggregate(const JVal &v, gbj_result *res) {
    const std::string op = op_name(v);
    if (op == "reduce") reduce(v, res);
    else if (op == "nest") nest(v, res);
    else groupby(v, res);
  }

  // A print / project list over a result: each entry names a result column
  // (recordProjection) and may rename it (register_as).
  void select_columns(const JVal &list, gbj_result *res) {
    std::vector<std::string> names;
    std::vector<std::vector<int64_t>> cols;
    for (const JVal &e : list.a) {
      const auto ra = projection(e);
      int c = -1;
      for (size_t j = 0; j < res->names.size() && c < 0; ++j) {
        const std::string &n = res->names[j];
        if (n == ra.second || n == ra.first + "." + ra.second ||
            (n.size() > ra.second.size() && n.compare(n.size() - ra.second.size() - 1, std::string::npos,
                                                       "." + ra.second) == 0))
          c = (int)j;
      }
      if (c < 0) fail(GBJ_ERR_INVALID, "plan: output column " + ra.second + " is not in the result");
      names.push_back(out_name(e, ra.second));
      cols.push_back(res->cols[c]);
    }
    res->names.swap(names);
    res->cols.swap(cols);
  }

  gbj_catalog *cat_;
  gbj_ctx *ctx_;
  std::vector<void *> allocs_;
  std::set<std::pair<std::string, std::string>> absent_;
  int grid(uint64_t n) const { return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 4096)); }
  void launched(const char *name) { ck(after_launch(ctx_, name, ctx_->stream), name); }

  void ck(int rc, const char *what) {
    if (rc != GBJ_OK) fail(rc, std::string(what) + ": " + gbj_last_error(ctx_));
  }
  template <typename T>
  T *alloc(uint64_t n) {
    void *p = nullptr;
    ck(gbj_pool_alloc(ctx_, std::max<uint64_t>(n, 1) * sizeof(T), &p), "pool");
    allocs_.push_back(p);
    return static_cast<T *>(p);
  }
  void sync() { ck(gbj_sync(ctx_, nullptr), "sync"); }
  template <typename T>
  T read1(const T *d) {
    T v{};
    sync();
    if (cudaMemcpy(&v, d, sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess) fail(GBJ_ERR_CUDA, "plan: copy");
    return v;
  }
  std::vector<int64_t> to_host32(const int32_t *d, uint64_t n) {
    std::vector<int32_t> h(n);
    sync();
    if (n && cudaMemcpy(h.data(), d, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) fail(GBJ_ERR_CUDA, "plan: copy");
    return std::vector<int64_t>(h.begin(), h.end());
  }
  std::vector<int64_t> to_host64(const int64_t *d, uint64_t n) {
    std::vector<int64_t> h(n);
    sync();
    if (n && cudaMemcpy(h.data(), d, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) fail(GBJ_ERR_CUDA, "plan: copy");
    return h;
  }

  const int32_t *column(const Rel &r, const JVal &e) {
    const auto ra = projection(e);
    const Rel::C *c = r.find(ra);
    if (!c && absent_.count(ra))
      fail(GBJ_ERR_UNSUPPORTED, "plan: column " + ra.first + "." + ra.second +
                                    " is not an int32 column of the catalog (only int32 columns are loaded)");
    if (!c) fail(GBJ_ERR_INVALID, "plan: column " + ra.first + "." + ra.second + " is not in the operator's input");
    return c->d;
  }

  Rel rel(const JVal &v) {
    const std::string op = op_name(v);
    if (passthrough(op) || op == "print") return rel(need(v, "input", op.c_str()));
    if (op == "materializer") return project(v);
    if (op == "scan") return scan(v);
    if (op == "select") return select(v);
    if (op == "hashjoin-chained" || op == "partitioned-hashjoin-chained" || op == "join") return join(v);
    if (op == "sort") return sort(v);
    if (op == "project") return project(v);
    if (op == "hash-rearrange" || op == "hash-pack") return rearrange(v);
    if (is_agg(op))
      fail(GBJ_ERR_UNSUPPORTED, "plan: '" + op + "' is supported only as the plan's root (under print, "
                                "project or sort)");
    validate(v);  // raises the unsupported-operator error
    fail(GBJ_ERR_UNSUPPORTED, "plan: operator '" + op + "'");
  }

  // ORDER BY: stable device sorts from the last key to the first.
  Rel sort(const JVal &v) {
    Rel r = rel(need(v, "input", "sort"));
    const JVal &es = need(v, "e", "sort");
    if (r.cols.empty() || r.n == 0) return r;
    if (r.cols.size() > GBJ_SORT_MAX_COLS) fail(GBJ_ERR_UNSUPPORTED, "plan: sort of more than 16 columns");
    for (size_t k = es.a.size(); k-- > 0;) {
      const std::string dir = need(es.a[k], "direction", "sort").s;
      if (dir == "NONE") continue;
      const auto ra = projection(need(es.a[k], "expression", "sort"));
      int key = -1;
      for (size_t c = 0; c < r.cols.size(); ++c)
        if (r.find(ra) == &r.cols[c]) key = (int)c;
      if (key < 0) fail(GBJ_ERR_INVALID, "plan: sort key " + ra.second + " is not in its input");
      std::vector<const int32_t *> in;
      std::vector<int32_t *> out;
      for (auto &c : r.cols) {
        in.push_back(c.d);
        out.push_back(alloc<int32_t>(r.n));
      }
      ck(gbj_sort_by_key(ctx_, in.data(), (int32_t)in.size(), r.n, key, dir == "DESC", out.data(), nullptr),
         "sort");
      for (size_t c = 0; c < r.cols.size(); ++c) r.cols[c].d = out[c];
    }
    return r;
  }

  Rel project(const JVal &v) {
    const std::string op = op_name(v);
    const Rel r = rel(need(v, "input", op.c_str()));
    Rel o;
    o.n = r.n;
    for (const JVal &e : need(v, "e", op.c_str()).a) {
      const auto ra = projection(e);
      const Rel::C *c = r.find(ra);
      if (!c) fail(GBJ_ERR_INVALID, "plan: project column " + ra.second + " is not in its input");
      o.cols.push_back(*c);
    }
    return o;
  }

  // Router-side partition: rows bucket-major by hash(e) mod buckets.
  Rel rearrange(const JVal &v) {
    const std::string op = op_name(v);
    const Rel r = rel(need(v, "input", op.c_str()));
    const auto key = projection(need(v, "e", op.c_str()));
    int32_t buckets = 2;  // the reference's default
    if (const JVal *b = v.get("buckets")) buckets = (int32_t)b->i;
    Rel o;
    o.n = r.n;
    std::vector<const int32_t *> in;
    std::vector<int32_t *> out;
    int key_col = -1;
    for (const JVal &p : need(v, "projections", op.c_str()).a) {
      const auto ra = projection(p);
      const Rel::C *c = r.find(ra);
      if (!c) fail(GBJ_ERR_INVALID, "plan: " + op + " column " + ra.second + " is not in its input");
      if (ra.second == key.second && (key.first.empty() || ra.first.empty() || ra.first == key.first))
        key_col = (int)in.size();
      in.push_back(c->d);
      out.push_back(alloc<int32_t>(r.n));
      o.cols.push_back({c->rel, c->attr, out.back()});
    }
    if (key_col < 0) {  // the hash key need not be projected
      const Rel::C *c = r.find(key);
      if (!c) fail(GBJ_ERR_INVALID, "plan: " + op + " key " + key.second + " is not in its input");
      key_col = (int)in.size();
      in.push_back(c->d);
      out.push_back(alloc<int32_t>(r.n));
    }
    if (in.size() > GBJ_REARRANGE_MAX_COLS) fail(GBJ_ERR_UNSUPPORTED, "plan: more than 16 columns to rearrange");
    uint64_t *off = alloc<uint64_t>((uint64_t)buckets + 1);
    ck(gbj_hash_rearrange(ctx_, in.data(), (int32_t)in.size(), r.n, key_col, (uint32_t)buckets, out.data(), off,
                          nullptr),
       op.c_str());
    return o;
  }

  // ORDER BY over an aggregate's host result (stable, last key first).
  void host_sort(const JVal &v, gbj_result *res) {
    const JVal &es = need(v, "e", "sort");
    std::vector<size_t> order(res->rows);
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    for (size_t k = es.a.size(); k-- > 0;) {
      const std::string dir = need(es.a[k], "direction", "sort").s;
      if (dir == "NONE") continue;
      const auto ra = projection(need(es.a[k], "expression", "sort"));
      int c = -1;
      for (size_t j = 0; j < res->names.size(); ++j)
        if (res->names[j] == ra.second || res->names[j] == ra.first + "." + ra.second) c = (int)j;
      if (c < 0) fail(GBJ_ERR_INVALID, "plan: sort key " + ra.second + " is not an output column");
      const auto &col = res->cols[c];
      std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return dir == "DESC" ? col[a] > col[b] : col[a] < col[b];
      });
    }
    for (auto &col : res->cols) {
      std::vector<int64_t> t(col.size());
      for (size_t i = 0; i < order.size(); ++i) t[i] = col[order[i]];
      col.swap(t);
    }
  }

  Rel scan(const JVal &v) {
    const JVal &pl = need(v, "plugin", "scan");
    const std::string name = need(pl, "name", "scan plugin").s;
    auto it = cat_->rel_attrs.find(name);
    if (it == cat_->rel_attrs.end()) fail(GBJ_ERR_INVALID, "plan: relation '" + name + "' is not in the catalog");
    std::vector<std::string> attrs = it->second;
    if (const JVal *pr = pl.get("projections")) {
      attrs.clear();
      for (const JVal &a : pr->a) {
        const JVal *an = a.get("attrName");
        if (!an) fail(GBJ_ERR_INVALID, "plan: projection without attrName");
        attrs.push_back(an->s);
      }
    }
    // the relation's row count, also for a scan that projects nothing
    Rel r;
    r.n = cat_->cols.at({name, it->second.front()}).n;
    for (const std::string &a : attrs) {
      auto c = cat_->cols.find({name, a});
      if (c == cat_->cols.end()) {
        // a projected attribute the catalog does not hold (a string or float
        // column of the reference's schema): an error only if an operator reads it
        absent_.insert({name, a});
        continue;
      }
      if (c->second.n != r.n) fail(GBJ_ERR_INVALID, "plan: columns of " + name + " differ in length");
      r.cols.push_back({name, a, c->second.d});
    }
    return r;
  }

  // Conjunction of column-vs-constant comparisons -> per-column [lo, hi].
  void ranges(const JVal &p, std::vector<std::tuple<std::pair<std::string, std::string>, int32_t, int32_t>> &out) {
    const JVal &x = uncast(p);
    const std::string n = expr_name(x);
    if (n == "bool") {
      const JVal *b = x.get("v");
      if (b && b->t == JVal::Bool && b->b) return;
      out.push_back({{"", ""}, 1, 0});  // always false: empty range
      return;
    }
    if (n == "and") {
      ranges(need(x, "left", "and"), out);
      ranges(need(x, "right", "and"), out);
      return;
    }
    if (n != "eq" && n != "lt" && n != "le" && n != "gt" && n != "ge")
      fail(GBJ_ERR_UNSUPPORTED, "plan: predicate '" + n + "' is not supported (eq, lt, le, gt, ge, and are)");
    const JVal &l = need(x, "left", n.c_str()), &r = need(x, "right", n.c_str());
    int64_t c = 0;
    std::string cmp = n;
    const JVal *col = &l;
    if (is_const(l, &c)) {  // constant on the left: mirror the comparison
      col = &r;
      cmp = n == "lt" ? "gt" : n == "le" ? "ge" : n == "gt" ? "lt" : n == "ge" ? "le" : n;
    } else if (!is_const(r, &c)) {
      fail(GBJ_ERR_UNSUPPORTED, "plan: predicates compare a column with a constant");
    }
    int64_t lo = INT32_MIN, hi = INT32_MAX;
    if (cmp == "eq") lo = hi = c;
    if (cmp == "lt") hi = c - 1;
    if (cmp == "le") hi = c;
    if (cmp == "gt") lo = c + 1;
    if (cmp == "ge") lo = c;
    if (lo > INT32_MAX || hi < INT32_MIN || lo > hi) {
      out.push_back({{"", ""}, 1, 0});
      return;
    }
    out.push_back({projection(*col), (int32_t)std::max<int64_t>(lo, INT32_MIN),
                   (int32_t)std::min<int64_t>(hi, INT32_MAX)});
  }

  // Rows of `r` kept by `rows` (positions), every column gathered.
  Rel gather(const Rel &r, const int32_t *rows, uint64_t n) {
    Rel o;
    o.n = n;
    for (const auto &c : r.cols) {
      int32_t *d = alloc<int32_t>(n);
      if (n) ck(gbj_gather(ctx_, c.d, rows, n, d, nullptr), "gather");
      o.cols.push_back({c.rel, c.attr, d});
    }
    return o;
  }

  Rel select(const JVal &v) { return filter(rel(need(v, "input", "select")), need(v, "p", "select")); }

  // True for an absent predicate or the constant true.
  static bool always_true(const JVal *p) {
    if (!p) return true;
    const JVal &x = uncast(*p);
    if (expr_name(x) != "bool") return false;
    const JVal *b = x.get("v");
    return b && b->t == JVal::Bool && b->b;
  }

  // The rows of `in` a conjunction of column-vs-constant comparisons keeps.
  Rel filter(Rel in, const JVal &p) {
    std::vector<std::tuple<std::pair<std::string, std::string>, int32_t, int32_t>> rg;
    ranges(p, rg);
    for (const auto &t : rg) {
      if (std::get<1>(t) > std::get<2>(t)) return gather(in, nullptr, 0);  // always false
      const Rel::C *c = in.find(std::get<0>(t));
      if (!c) fail(GBJ_ERR_INVALID, "plan: select column " + std::get<0>(t).second + " is not in its input");
      int32_t *rows = alloc<int32_t>(in.n);
      uint64_t *cnt = alloc<uint64_t>(1);
      ck(gbj_select_range(ctx_, c->d, in.n, std::get<1>(t), std::get<2>(t), rows, cnt, nullptr), "select");
      const uint64_t k = read1(cnt);
      in = gather(in, rows, k);
    }
    return in;
  }

  struct JoinSides {
    const JVal *build, *probe, *bk, *pk;
    const JVal *bkm = nullptr, *pkm = nullptr;  // minor keys (partitioned join)
    int32_t hash_bits = 0;
    uint64_t max_build = 0;
    bool radix = false;
  };
  JoinSides sides(const JVal &v) {
    const std::string op = op_name(v);
    JoinSides s{};
    if (op == "join") {
      const JVal &p = uncast(need(v, "p", "join"));
      if (expr_name(p) != "eq") fail(GBJ_ERR_UNSUPPORTED, "plan: join predicates must be eq");
      s.build = &need(v, "leftInput", "join");
      s.probe = &need(v, "rightInput", "join");
      s.bk = &need(p, "left", "eq");
      s.pk = &need(p, "right", "eq");
      s.radix = true;
    } else {
      s.build = &need(v, "build_input", op.c_str());
      s.probe = &need(v, "probe_input", op.c_str());
      s.bk = &need(v, "build_k", op.c_str());
      s.pk = &need(v, "probe_k", op.c_str());
      if (const JVal *h = v.get("hash_bits")) s.hash_bits = (int32_t)h->i;
      if (const JVal *m = v.get("maxBuildInputSize")) s.max_build = (uint64_t)std::max<int64_t>(m->i, 0);
      s.radix = op == "partitioned-hashjoin-chained";
      s.bkm = v.get("build_k_minor");
      s.pkm = v.get("probe_k_minor");
      if (!s.bkm != !s.pkm) fail(GBJ_ERR_INVALID, "plan: build_k_minor and probe_k_minor go together");
    }
    return s;
  }

  Rel join(const JVal &v) {
    const JoinSides s = sides(v);
    const Rel b = rel(*s.build), p = rel(*s.probe);
    const int32_t *bk = column(b, *s.bk), *pk = column(p, *s.pk);
    gbj_table *t = nullptr;
    ck(gbj_join_build(ctx_, bk, nullptr, b.n, s.hash_bits, std::max<uint64_t>(s.max_build, b.n), nullptr, &t),
       "join build");
    struct TableGuard {
      gbj_ctx *c;
      gbj_table *t;
      ~TableGuard() { gbj_table_destroy(c, t); }
    } guard{ctx_, t};
    // count the matches, then write the pairs
    const gbj_agg cnt_agg{GBJ_AGG_COUNT, GBJ_VAL_ONE};
    int64_t *dcnt = alloc<int64_t>(1);
    ck(gbj_join_probe_agg(ctx_, t, pk, nullptr, p.n, &cnt_agg, 1, dcnt, nullptr), "join probe");
    const uint64_t m = (uint64_t)read1(dcnt);
    int32_t *br = alloc<int32_t>(m), *pr = alloc<int32_t>(m);
    uint64_t *dm = alloc<uint64_t>(1);
    ck(gbj_join_probe_pairs(ctx_, t, pk, nullptr, p.n, br, pr, m, dm, nullptr), "join pairs");
    uint64_t k = m;
    if (s.bkm && m) {
      // the minor-key check (gpu-partitioned-hash-join-chained.cpp:1284-1333)
      // over the key matches: keep the pairs whose minor keys are equal
      const int32_t *bm = column(b, *s.bkm), *pm = column(p, *s.pkm);
      int32_t *flag = alloc<int32_t>(m), *keep = alloc<int32_t>(m);
      k_pair_eq<<<grid(m), 256, 0, ctx_->stream>>>(bm, pm, br, pr, m, flag);
      launched("k_pair_eq");
      uint64_t *kc = alloc<uint64_t>(1);
      ck(gbj_select_range(ctx_, flag, m, 1, 1, keep, kc, nullptr), "minor key");
      k = read1(kc);
      int32_t *br2 = alloc<int32_t>(k), *pr2 = alloc<int32_t>(k);
      if (k) {
        ck(gbj_gather(ctx_, br, keep, k, br2, nullptr), "gather");
        ck(gbj_gather(ctx_, pr, keep, k, pr2, nullptr), "gather");
      }
      br = br2, pr = pr2;
    }
    sync();
    Rel o = gather(b, br, k);
    const Rel po = gather(p, pr, k);
    o.cols.insert(o.cols.end(), po.cols.begin(), po.cols.end());
    return o;
  }

  // Operand of a fused join aggregate, or -1 if the expression needs more.
  struct Operand {
    int operand;
    int64_t scale;  // constants: sum of v over n rows = v * count
  };
  bool fusable(const JVal &e, const Rel &b, const Rel &p, const JoinSides &s, const int32_t **bcol,
               const int32_t **pcol, Operand *out) {
    const JVal &x = uncast(e);
    int64_t c = 0;
    if (is_const(x, &c)) {
      *out = {GBJ_VAL_ONE, c};
      return true;
    }
    auto side_of = [&](const JVal &col, int *which, const int32_t **d) {
      const auto ra = projection(col);
      if (const Rel::C *bc = b.find(ra)) {
        *which = 0, *d = bc->d;
        return true;
      }
      if (const Rel::C *pc = p.find(ra)) {
        *which = 1, *d = pc->d;
        return true;
      }
      return false;
    };
    auto take = [&](int which, const int32_t *d) {
      const int32_t **slot = which == 0 ? bcol : pcol;
      if (*slot && *slot != d) return false;
      *slot = d;
      return true;
    };
    const std::string n = expr_name(x);
    if (n == "recordProjection") {
      int w;
      const int32_t *d;
      if (!side_of(x, &w, &d)) return false;
      if (w == 0 && projection(x) == projection(*s.bk)) {
        *out = {GBJ_VAL_BUILD_KEY, 1};
        return true;
      }
      if (!take(w, d)) return false;
      *out = {w == 0 ? GBJ_VAL_BUILD : GBJ_VAL_PROBE, 1};
      return true;
    }
    if (n == "multiply") {
      int w1, w2;
      const int32_t *d1, *d2;
      if (!side_of(uncast(need(x, "left", "multiply")), &w1, &d1) ||
          !side_of(uncast(need(x, "right", "multiply")), &w2, &d2) || w1 == w2)
        return false;
      if (!take(w1, d1) || !take(w2, d2)) return false;
      *out = {GBJ_VAL_PRODUCT, 1};
      return true;
    }
    return false;
  }

  // Aggregate of a constant operand over `n` rows (or `n` join matches).
  static int64_t const_agg(int m, int64_t c, int64_t n) {
    switch (m) {
      case GBJ_AGG_SUM: return c * n;
      case GBJ_AGG_OR: return (n && c) ? 1 : 0;
      case GBJ_AGG_AND: return (!n || c) ? 1 : 0;
      default: return n ? c : (m == GBJ_AGG_MAX ? INT64_MIN : INT64_MAX);
    }
  }

  // A value operand of an aggregate: a column, a constant, or a
  // column-vs-constant comparison (materialised as a 0/1 column).  With
  // `truth`, a column is turned into its truth value (!= 0), as the logical
  // accumulators read it.
  struct Val {
    const int32_t *d = nullptr;
    bool is_const = false;
    int64_t c = 0;
  };
  Val value(const Rel &r, const JVal &e, bool truth) {
    Val out;
    const JVal &x = uncast(e);
    const std::string n = expr_name(x);
    int64_t c = 0;
    if (is_const(x, &c)) {
      out.is_const = true;
      out.c = truth ? (c != 0) : c;
      return out;
    }
    if (n == "bool") {
      out.is_const = true;
      out.c = always_true(&x) ? 1 : 0;
      return out;
    }
    if (n == "eq" || n == "lt" || n == "le" || n == "gt" || n == "ge" || n == "and") {
      std::vector<std::tuple<std::pair<std::string, std::string>, int32_t, int32_t>> rg;
      ranges(x, rg);
      int32_t *t = alloc<int32_t>(r.n);
      bool first = true;
      for (const auto &q : rg) {
        const bool never = std::get<1>(q) > std::get<2>(q);
        const Rel::C *col = never ? nullptr : r.find(std::get<0>(q));
        if (!never && !col) fail(GBJ_ERR_INVALID, "plan: column " + std::get<0>(q).second + " is not in the input");
        if (r.n) {
          // an always-false range: every row fails (a column compared with an empty range)
          const int32_t *src = col ? col->d : t;
          k_truth<<<grid(r.n), 256, 0, ctx_->stream>>>(src, r.n, 0, never ? 1 : std::get<1>(q),
                                                       never ? 0 : std::get<2>(q), first ? 0 : 1, t);
          launched("k_truth");
        }
        first = false;
      }
      out.d = t;
      return out;
    }
    const int32_t *col = column(r, e);
    if (!truth) {
      out.d = col;
      return out;
    }
    int32_t *t = alloc<int32_t>(r.n);
    if (r.n) {
      k_truth<<<grid(r.n), 256, 0, ctx_->stream>>>(col, r.n, 1, 0, 0, 0, t);
      launched("k_truth");
    }
    out.d = t;
    return out;
  }

  void reduce(const JVal &v, gbj_result *res) {
    const JVal &es = need(v, "e", "reduce"), &acc = need(v, "accumulator", "reduce");
    if (es.a.size() != acc.a.size() || es.a.empty() || es.a.size() > GBJ_MAX_AGGS)
      fail(GBJ_ERR_INVALID, "plan: reduce needs 1..8 expressions, one accumulator each");
    const JVal &in = need(v, "input", "reduce");
    const JVal *pred = v.get("p");
    const std::string iop = op_name(in);
    std::vector<int64_t> out(es.a.size());
    bool done = false;
    if (always_true(pred) &&
        (iop == "hashjoin-chained" || iop == "partitioned-hashjoin-chained" || iop == "join")) {
      const JoinSides s = sides(in);
      const Rel b = rel(*s.build), p = rel(*s.probe);
      const int32_t *bcol = nullptr, *pcol = nullptr;
      std::vector<Operand> ops(es.a.size());
      bool ok = true;
      for (size_t j = 0; j < es.a.size() && ok; ++j) ok = fusable(es.a[j], b, p, s, &bcol, &pcol, &ops[j]);
      if (ok) {
        // constant operands are computed from the match count
        std::vector<gbj_agg> aggs(es.a.size());
        for (size_t j = 0; j < es.a.size(); ++j)
          aggs[j] = {ops[j].operand == GBJ_VAL_ONE ? GBJ_AGG_COUNT : monoid(acc.a[j].s), ops[j].operand};
        int64_t *d = alloc<int64_t>(aggs.size());
        const int32_t *bk = column(b, *s.bk), *pk = column(p, *s.pk);
        if (s.bkm) {
          ck(gbj_radix_join_agg_minor(ctx_, bk, column(b, *s.bkm), bcol, b.n, pk, column(p, *s.pkm), pcol, p.n,
                                      nullptr, aggs.data(), (int32_t)aggs.size(), d, nullptr),
             "radix join (minor key)");
        } else if (s.radix) {
          ck(gbj_radix_join_agg(ctx_, bk, bcol, b.n, pk, pcol, p.n, nullptr, aggs.data(), (int32_t)aggs.size(), d,
                                nullptr),
             "radix join");
        } else {
          gbj_table *t = nullptr;
          ck(gbj_join_build(ctx_, bk, bcol, b.n, s.hash_bits, std::max<uint64_t>(s.max_build, b.n), nullptr, &t),
             "join build");
          const int rc = gbj_join_probe_agg(ctx_, t, pk, pcol, p.n, aggs.data(), (int32_t)aggs.size(), d, nullptr);
          gbj_table_destroy(ctx_, t);
          ck(rc, "join probe");
        }
        const std::vector<int64_t> h = to_host64(d, aggs.size());
        for (size_t j = 0; j < aggs.size(); ++j)
          out[j] = ops[j].operand == GBJ_VAL_ONE ? const_agg(monoid(acc.a[j].s), ops[j].scale, h[j]) : h[j];
        done = true;
      }
    }
    if (!done) {
      Rel r = rel(in);
      if (!always_true(pred)) r = filter(r, *pred);
      for (size_t j = 0; j < es.a.size(); ++j) {
        const int m = monoid(acc.a[j].s);
        const Val x = value(r, es.a[j], false);
        if (x.is_const) {
          out[j] = const_agg(m, x.c, (int64_t)r.n);
          continue;
        }
        const gbj_agg a{m, GBJ_VAL_PROBE};
        int64_t *d = alloc<int64_t>(1);
        ck(gbj_reduce(ctx_, x.d, nullptr, r.n, &a, 1, d, nullptr), "reduce");
        out[j] = to_host64(d, 1)[0];
      }
    }
    res->rows = 1;
    for (size_t j = 0; j < out.size(); ++j) {
      res->names.push_back(out_name(es.a[j], acc.a[j].s + "_" + std::to_string(j)));
      res->cols.push_back({out[j]});
    }
  }

  // Per-group aggregates over one key column: COUNT, SUM, MIN, MAX of each
  // distinct value column (logical accumulators read MAX / MIN of the
  // operand's truth column), sorted by key.
  struct GroupSpec {
    int m;        // accumulator
    int vi;       // value column index, -1 for a constant
    int64_t c;    // the constant
  };
  void group_values(const Rel &r, const JVal &es, const char *op, const std::vector<std::string> &accs,
                    std::vector<const int32_t *> &vcols, std::vector<GroupSpec> &spec,
                    bool nested_e) {
    for (size_t j = 0; j < es.a.size(); ++j) {
      const JVal &x = nested_e ? need(es.a[j], "e", op) : es.a[j];
      const int m = monoid(accs[j]);
      const Val val = value(r, x, m == GBJ_AGG_OR || m == GBJ_AGG_AND);
      if (val.is_const) {
        spec.push_back({m, -1, val.c});
        continue;
      }
      auto it = std::find(vcols.begin(), vcols.end(), val.d);
      spec.push_back({m, (int)(it - vcols.begin()), 0});
      if (it == vcols.end()) vcols.push_back(val.d);
    }
  }
  static int64_t group_value(const GroupSpec &g, const std::vector<int64_t> &row) {
    const int64_t cnt = row[4 * std::max(g.vi, 0)];
    if (g.vi < 0) return const_agg(g.m, g.c, cnt);
    const int64_t *a = &row[4 * g.vi];
    switch (g.m) {
      case GBJ_AGG_SUM: return a[1];
      case GBJ_AGG_MIN: case GBJ_AGG_AND: return a[2];
      default: return a[3];  // MAX, OR
    }
  }

  void groupby(const JVal &v, gbj_result *res) {
    const char *op = "groupby";
    const JVal &ks = need(v, "k", op), &es = need(v, "e", op);
    if (ks.t != JVal::Arr || ks.a.size() != 1)
      fail(GBJ_ERR_UNSUPPORTED, "plan: group-by takes one int32 key expression");
    const Rel r = rel(need(v, "input", op));
    const int32_t *key = column(r, ks.a[0]);
    gbj_groupby_params prm{};
    if (const JVal *h = v.get("hash_bits")) prm.hash_bits = (int32_t)h->i;
    if (const JVal *m = v.get("maxInputSize")) prm.max_input_size = (uint64_t)std::max<int64_t>(m->i, 0);
    std::vector<std::string> accs;
    for (const JVal &x : es.a) accs.push_back(need(x, "m", op).s);
    // one gbj_groupby per distinct value column; constants need only the counts
    std::vector<const int32_t *> vcols;
    std::vector<GroupSpec> spec;
    group_values(r, es, op, accs, vcols, spec, true);
    if (vcols.empty()) vcols.push_back(key);  // counts of the key column
    const uint64_t cap = std::max<uint64_t>(r.n, 1);
    std::map<int32_t, std::vector<int64_t>> groups;  // key -> per value column: cnt, sum, min, max
    for (size_t i = 0; i < vcols.size(); ++i) {
      int32_t *ok = alloc<int32_t>(cap);
      int64_t *oc = alloc<int64_t>(cap), *os = alloc<int64_t>(cap);
      int32_t *omn = alloc<int32_t>(cap), *omx = alloc<int32_t>(cap);
      uint64_t *ng = alloc<uint64_t>(1);
      ck(gbj_groupby(ctx_, key, vcols[i], r.n, &prm, ok, oc, os, omn, omx, cap, ng, nullptr), "groupby");
      const uint64_t n = read1(ng);
      const auto hk = to_host32(ok, n), hmn = to_host32(omn, n), hmx = to_host32(omx, n);
      const auto hc = to_host64(oc, n), hs = to_host64(os, n);
      for (uint64_t g = 0; g < n; ++g) {
        auto &row = groups[(int32_t)hk[g]];
        row.resize(4 * vcols.size());
        row[4 * i] = hc[g], row[4 * i + 1] = hs[g], row[4 * i + 2] = hmn[g], row[4 * i + 3] = hmx[g];
      }
    }
    res->rows = groups.size();
    res->names.push_back(projection(ks.a[0]).second);
    res->cols.emplace_back();
    for (size_t j = 0; j < es.a.size(); ++j) {
      res->names.push_back(out_name(need(es.a[j], "e", op), accs[j] + "_" + std::to_string(j)));
      res->cols.emplace_back();
    }
    for (const auto &kv : groups) {  // sorted by key
      res->cols[0].push_back(kv.first);
      for (size_t j = 0; j < spec.size(); ++j) res->cols[1 + j].push_back(group_value(spec[j], kv.second));
    }
  }

  // RadixNest (radix-nest.cpp:326-700; plan fields plan-parser.cpp:1140-1268):
  // group by f over the rows p keeps, one aggregate per e / accumulator,
  // named by aggrLabels.  The key and each value column are widened to
  // int64 and grouped by gbj_nest_i64, as the reference nests on 64-bit
  // keys (radix-aggr.cpp, KEY_8B).  g (nulls to zeros) has no effect on
  // non-null int32 columns; fields lists what the reference materialises.
  void nest(const JVal &v, gbj_result *res) {
    const char *op = "nest";
    const JVal &es = need(v, "e", op), &acc = need(v, "accumulator", op), &labels = need(v, "aggrLabels", op);
    Rel r = rel(need(v, "input", op));
    if (!always_true(v.get("p"))) r = filter(r, need(v, "p", op));
    const JVal &f = need(v, "f", op);
    const int32_t *key = column(r, f);
    std::vector<std::string> accs;
    for (const JVal &a : acc.a) accs.push_back(a.s);
    std::vector<const int32_t *> vcols;
    std::vector<GroupSpec> spec;
    group_values(r, es, op, accs, vcols, spec, false);
    const uint64_t n = r.n, cap = std::max<uint64_t>(n, 1);
    int64_t *k64 = alloc<int64_t>(cap);
    if (n) {
      k_widen<<<grid(n), 256, 0, ctx_->stream>>>(key, n, k64);
      launched("k_widen");
    }
    std::map<int64_t, std::vector<int64_t>> groups;  // key -> per value column: cnt, sum, min, max
    const size_t passes = std::max<size_t>(vcols.size(), 1);
    for (size_t i = 0; i < passes; ++i) {
      int64_t *v64 = nullptr;
      if (i < vcols.size()) {
        v64 = alloc<int64_t>(cap);
        if (n) {
          k_widen<<<grid(n), 256, 0, ctx_->stream>>>(vcols[i], n, v64);
          launched("k_widen");
        }
      }
      int64_t *ok = alloc<int64_t>(cap), *oc = alloc<int64_t>(cap), *os = alloc<int64_t>(cap);
      int64_t *omn = alloc<int64_t>(cap), *omx = alloc<int64_t>(cap);
      uint64_t *ng = alloc<uint64_t>(1);
      ck(gbj_nest_i64(ctx_, k64, v64, n, 0, ok, oc, os, omn, omx, cap, ng, nullptr), "nest");
      const uint64_t g = read1(ng);
      const auto hk = to_host64(ok, g), hc = to_host64(oc, g), hs = to_host64(os, g);
      const auto hmn = to_host64(omn, g), hmx = to_host64(omx, g);
      for (uint64_t q = 0; q < g; ++q) {
        auto &row = groups[hk[q]];
        row.resize(4 * passes);
        row[4 * i] = hc[q], row[4 * i + 1] = hs[q], row[4 * i + 2] = hmn[q], row[4 * i + 3] = hmx[q];
      }
    }
    res->rows = groups.size();
    res->names.push_back(projection(f).second);
    res->cols.emplace_back();
    for (size_t j = 0; j < es.a.size(); ++j) {
      const JVal &l = labels.a[j];
      res->names.push_back(l.t == JVal::Str ? l.s : accs[j] + "_" + std::to_string(j));
      res->cols.emplace_back();
    }
    for (const auto &kv : groups) {  // sorted by key
      res->cols[0].push_back(kv.first);
      for (size_t j = 0; j < spec.size(); ++j) res->cols[1 + j].push_back(group_value(spec[j], kv.second));
    }
  }

};

}  // namespace

extern "C" int gbj_catalog_create(gbj_ctx *ctx, gbj_catalog **out) {
  if (!ctx || !out) return GBJ_ERR_INVALID;
  *out = new gbj_catalog();
  (*out)->ctx = ctx;
  return GBJ_OK;
}

extern "C" int gbj_catalog_add_column(gbj_catalog *cat, const char *rel, const char *attr, const int32_t *d_col,
                                      uint64_t n) {
  if (!cat || !rel || !attr || (n && !d_col)) return GBJ_ERR_INVALID;
  const std::pair<std::string, std::string> k{rel, attr};
  auto &attrs = cat->rel_attrs[rel];
  if (!cat->cols.count(k)) attrs.push_back(attr);
  cat->cols[k] = {d_col, n};
  return GBJ_OK;
}

extern "C" int gbj_catalog_destroy(gbj_catalog *cat) {
  if (!cat) return GBJ_ERR_INVALID;
  if (!cat->owned.empty()) cudaDeviceSynchronize();
  for (void *p : cat->owned) gbj_pool_free(cat->ctx, p);
  delete cat;
  return GBJ_OK;
}

namespace {

// Streams one binary column file into a pool block: reads go into two pinned
// staging buffers alternately, so the next read overlaps the previous copy.
int load_column_file(gbj_catalog *cat, const std::string &file, uint64_t *n_out, void **d_out) {
  gbj_ctx *ctx = cat->ctx;
  FILE *f = fopen(file.c_str(), "rb");
  if (!f) return set_error(ctx, GBJ_ERR_INVALID, "catalog: cannot open " + file);
  fseek(f, 0, SEEK_END);
  const long long bytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (bytes < 0 || bytes % 4) {
    fclose(f);
    return set_error(ctx, GBJ_ERR_INVALID, "catalog: " + file + " is not a whole number of int32 values");
  }
  void *d = nullptr;
  int rc = gbj_pool_alloc(ctx, std::max<uint64_t>((uint64_t)bytes, 16), &d);
  if (rc) {
    fclose(f);
    return rc;
  }
  constexpr size_t kChunk = 64u << 20;
  void *stage[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  cudaStream_t s = ctx->stream;
  for (int i = 0; i < 2 && rc == GBJ_OK; ++i) {
    if (cudaHostAlloc(&stage[i], kChunk, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess)
      rc = set_error(ctx, GBJ_ERR_CUDA, "catalog: staging buffers");
  }
  uint64_t off = 0;
  for (int k = 0; rc == GBJ_OK && off < (uint64_t)bytes; ++k) {
    const int b = k & 1;
    if (k >= 2) cudaEventSynchronize(done[b]);  // its previous copy has finished
    const size_t want = (size_t)std::min<uint64_t>(kChunk, (uint64_t)bytes - off);
    if (fread(stage[b], 1, want, f) != want) {
      rc = set_error(ctx, GBJ_ERR_INVALID, "catalog: short read of " + file);
      break;
    }
    if (cudaMemcpyAsync(static_cast<char *>(d) + off, stage[b], want, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaEventRecord(done[b], s) != cudaSuccess)
      rc = set_error(ctx, GBJ_ERR_CUDA, "catalog: copy of " + file);
    off += want;
  }
  cudaStreamSynchronize(s);
  for (int i = 0; i < 2; ++i) {
    if (stage[i]) cudaFreeHost(stage[i]);
    if (done[i]) cudaEventDestroy(done[i]);
  }
  fclose(f);
  if (rc) {
    gbj_pool_free(ctx, d);
    return rc;
  }
  *n_out = (uint64_t)bytes / 4;
  *d_out = d;
  return GBJ_OK;
}

}  // namespace

// Loads int32 columns described by a catalog.json in the reference's
// columnar layout (tools/prepare_data.py: one binary file per column,
// "<path>.<attrName>", int / boolean / dictionary-coded string columns as
// 4-byte little-endian values; relation name = the entry's "path").
// Columns of other types (int64, date, float) are skipped.
extern "C" int gbj_catalog_load(gbj_catalog *cat, const char *catalog_json, const char *base_dir,
                                const char *relation, uint64_t *columns_loaded) {
  if (!cat || !catalog_json) return GBJ_ERR_INVALID;
  gbj_ctx *ctx = cat->ctx;
  std::string text;
  {
    FILE *f = fopen(catalog_json, "rb");
    if (!f) return set_error(ctx, GBJ_ERR_INVALID, std::string("catalog: cannot open ") + catalog_json);
    char buf[1 << 16];
    size_t k;
    while ((k = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, k);
    fclose(f);
  }
  uint64_t loaded = 0;
  try {
    const JVal root = JsonParser(text.c_str()).parse();
    if (root.t != JVal::Obj) fail(GBJ_ERR_INVALID, "catalog: top level is not an object");
    const std::string base = base_dir && *base_dir ? std::string(base_dir) + "/" : std::string();
    for (const auto &kv : root.o) {
      const JVal &e = kv.second;
      const JVal *path = e.get("path");
      if (!path || path->t != JVal::Str) continue;
      if (relation && *relation && kv.first != relation && path->s != relation) continue;
      const JVal *ty = e.get("type");
      const JVal *inner = ty ? ty->get("inner") : nullptr;
      const JVal *attrs = inner ? inner->get("attributes") : nullptr;
      if (!attrs || attrs->t != JVal::Arr) fail(GBJ_ERR_INVALID, "catalog: " + kv.first + " has no attributes");
      for (const JVal &a : attrs->a) {
        const JVal *an = a.get("attrName");
        const JVal *at = a.get("type");
        const JVal *tn = at ? at->get("type") : nullptr;
        if (!an || !tn) continue;
        if (tn->s != "int" && tn->s != "dstring" && tn->s != "boolean") continue;
        uint64_t n = 0;
        void *d = nullptr;
        const int rc = load_column_file(cat, base + path->s + "." + an->s, &n, &d);
        if (rc) fail(rc, gbj_last_error(ctx));
        cat->owned.push_back(d);
        const int rc2 = gbj_catalog_add_column(cat, path->s.c_str(), an->s.c_str(), static_cast<int32_t *>(d), n);
        if (rc2) fail(rc2, "catalog: register " + an->s);
        ++loaded;
      }
    }
  } catch (const PlanError &e) {
    return set_error(ctx, e.code, e.msg);
  }
  if (columns_loaded) *columns_loaded = loaded;
  return GBJ_OK;
}

extern "C" int gbj_plan_validate(const char *plan_json, char *err, uint64_t err_len) {
  if (!plan_json) return GBJ_ERR_INVALID;
  try {
    validate(JsonParser(plan_json).parse());
    if (err && err_len) err[0] = 0;
    return GBJ_OK;
  } catch (const PlanError &e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.msg.c_str());
    return e.code;
  }
}

extern "C" int gbj_plan_execute(gbj_catalog *cat, const char *plan_json, gbj_result **out) {
  if (!cat || !plan_json || !out) return GBJ_ERR_INVALID;
  *out = nullptr;
  try {
    const JVal root = JsonParser(plan_json).parse();
    validate(root);
    Exec ex(cat);
    *out = ex.run(root);
    return GBJ_OK;
  } catch (const PlanError &e) {
    return set_error(cat->ctx, e.code, e.msg);
  } catch (const std::exception &e) {
    return set_error(cat->ctx, GBJ_ERR_INVALID, std::string("plan: ") + e.what());
  }
}

extern "C" int gbj_result_shape(const gbj_result *r, int32_t *n_cols, uint64_t *n_rows) {
  if (!r) return GBJ_ERR_INVALID;
  if (n_cols) *n_cols = (int32_t)r->cols.size();
  if (n_rows) *n_rows = r->rows;
  return GBJ_OK;
}

extern "C" const char *gbj_result_name(const gbj_result *r, int32_t col) {
  if (!r || col < 0 || col >= (int32_t)r->names.size()) return nullptr;
  return r->names[col].c_str();
}

extern "C" int gbj_result_column(const gbj_result *r, int32_t col, int64_t *h_out) {
  if (!r || !h_out || col < 0 || col >= (int32_t)r->cols.size()) return GBJ_ERR_INVALID;
  std::copy(r->cols[col].begin(), r->cols[col].end(), h_out);
  return GBJ_OK;
}

extern "C" void gbj_result_destroy(gbj_result *r) { delete r; }
