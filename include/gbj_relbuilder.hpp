// gbj_relbuilder.hpp -- C++ plan builder with the call shapes of the
// reference's RelBuilder (core/olap/include/olap/plan/relbuilder.hpp:
// scan, filter, join(build, build_k, probe_k, hash_bits, maxBuildInputSize)
// at :466-486 / :655-675, groupby(k, e, hash_bits, maxInputSize) at
// :537-541 / :612-614, reduce(e, accumulators) at :532-535) and a
// PreparedStatement whose execute() runs the plan (prepared-statement.cpp:
// 41-135).  The builder records the plan in the reference's JSON plan format
// and execution goes through gbj_plan_execute on catalog columns.
//
// Header-only; link against libgbjoin.so.
#ifndef GBJ_RELBUILDER_HPP
#define GBJ_RELBUILDER_HPP

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbjoin.h"

namespace gbj {

// An expression in the reference's JSON expression form.
class Expr {
 public:
  explicit Expr(std::string json) : json_(std::move(json)) {}
  const std::string &json() const { return json_; }

  static Expr col(const std::string &rel, const std::string &attr) {
    const std::string a = "{\"relName\":" + q(rel) + ",\"attrName\":" + q(attr) + "}";
    return Expr("{\"expression\":\"recordProjection\",\"type\":{\"type\":\"int\"},\"e\":{\"expression\":"
                "\"argument\",\"argNo\":-1,\"type\":{\"type\":\"record\",\"relName\":" +
                q(rel) + "},\"attributes\":[" + a + "]},\"attribute\":" + a + "}");
  }
  static Expr lit(int64_t v) { return Expr("{\"expression\":\"int\",\"v\":" + std::to_string(v) + "}"); }
  static Expr lit(bool v) { return Expr(std::string("{\"expression\":\"bool\",\"v\":") + (v ? "true" : "false") + "}"); }
  Expr cast64() const { return Expr("{\"expression\":\"cast\",\"type\":{\"type\":\"int64\"},\"e\":" + json_ + "}"); }

  Expr operator==(const Expr &o) const { return bin("eq", o); }
  Expr operator<(const Expr &o) const { return bin("lt", o); }
  Expr operator<=(const Expr &o) const { return bin("le", o); }
  Expr operator>(const Expr &o) const { return bin("gt", o); }
  Expr operator>=(const Expr &o) const { return bin("ge", o); }
  Expr operator&&(const Expr &o) const { return bin("and", o); }
  Expr operator*(const Expr &o) const { return bin("multiply", o); }
  Expr operator==(int64_t v) const { return *this == lit(v); }
  Expr operator<(int64_t v) const { return *this < lit(v); }
  Expr operator<=(int64_t v) const { return *this <= lit(v); }
  Expr operator>(int64_t v) const { return *this > lit(v); }
  Expr operator>=(int64_t v) const { return *this >= lit(v); }

  static std::string q(const std::string &s) {
    std::string o = "\"";
    for (char c : s) {
      if (c == '"' || c == '\\') o += '\\';
      o += c;
    }
    return o + "\"";
  }

 private:
  Expr bin(const char *name, const Expr &o) const {
    return Expr(std::string("{\"expression\":\"") + name + "\",\"left\":" + json_ + ",\"right\":" + o.json_ + "}");
  }
  std::string json_;
};

// An aggregate output expression of a group-by (GpuAggrMatExpr's (e, m)).
struct AggExpr {
  Expr e;
  std::string monoid;  // sum, max, min
};

// Query results: int64 host columns by name.
struct Result {
  std::vector<std::string> names;
  std::vector<std::vector<int64_t>> cols;
  uint64_t rows = 0;
  const std::vector<int64_t> &operator[](const std::string &n) const {
    for (size_t i = 0; i < names.size(); ++i)
      if (names[i] == n) return cols[i];
    throw std::out_of_range("no result column " + n);
  }
};

class PreparedStatement {
 public:
  PreparedStatement(gbj_catalog *cat, std::string plan) : cat_(cat), plan_(std::move(plan)) {}
  const std::string &plan() const { return plan_; }
  // Throws std::runtime_error with the library's message on failure.
  Result execute() const {
    gbj_result *r = nullptr;
    const int rc = gbj_plan_execute(cat_, plan_.c_str(), &r);
    if (rc != GBJ_OK) throw std::runtime_error("gbj_plan_execute failed (" + std::to_string(rc) + ")");
    std::unique_ptr<gbj_result, void (*)(gbj_result *)> hold(r, gbj_result_destroy);
    Result out;
    int32_t nc = 0;
    gbj_result_shape(r, &nc, &out.rows);
    for (int32_t i = 0; i < nc; ++i) {
      out.names.emplace_back(gbj_result_name(r, i));
      out.cols.emplace_back(out.rows);
      if (out.rows) gbj_result_column(r, i, out.cols.back().data());
    }
    return out;
  }

 private:
  gbj_catalog *cat_;
  std::string plan_;
};

// Immutable: every call returns a builder rooted at the new operator.
class RelBuilder {
 public:
  static RelBuilder scan(const std::string &rel, const std::vector<std::string> &attrs) {
    std::string pr;
    for (const auto &a : attrs)
      pr += (pr.empty() ? "" : ",") + std::string("{\"relName\":") + Expr::q(rel) + ",\"attrName\":" + Expr::q(a) + "}";
    return RelBuilder("{\"operator\":\"scan\",\"plugin\":{\"name\":" + Expr::q(rel) +
                      ",\"type\":\"gpu\",\"projections\":[" + pr + "]}}");
  }
  RelBuilder filter(const Expr &p) const {
    return RelBuilder("{\"operator\":\"select\",\"p\":" + p.json() + ",\"input\":" + json_ + "}");
  }
  // `this` is the probe side, as for the reference's RelBuilder::join.
  RelBuilder join(const RelBuilder &build, const Expr &build_k, const Expr &probe_k, int hash_bits = 0,
                  uint64_t maxBuildInputSize = 0) const {
    std::string j = "{\"operator\":\"hashjoin-chained\",\"build_input\":" + build.json_ +
                    ",\"probe_input\":" + json_ + ",\"build_k\":" + build_k.json() + ",\"probe_k\":" + probe_k.json();
    if (hash_bits) j += ",\"hash_bits\":" + std::to_string(hash_bits);
    if (maxBuildInputSize) j += ",\"maxBuildInputSize\":" + std::to_string(maxBuildInputSize);
    return RelBuilder(j + "}");
  }
  RelBuilder groupby(const std::vector<Expr> &k, const std::vector<AggExpr> &e, int hash_bits,
                     uint64_t maxInputSize) const {
    std::string ks, es;
    for (const auto &x : k) ks += (ks.empty() ? "" : ",") + x.json();
    for (size_t i = 0; i < e.size(); ++i)
      es += (i ? "," : "") + std::string("{\"e\":") + e[i].e.json() + ",\"m\":" + Expr::q(e[i].monoid) +
            ",\"packet\":1,\"offset\":" + std::to_string(32 * (i + 1)) + "}";
    return RelBuilder("{\"operator\":\"hashgroupby-chained\",\"input\":" + json_ + ",\"gpu\":true,\"k\":[" + ks +
                      "],\"e\":[" + es + "],\"hash_bits\":" + std::to_string(hash_bits) +
                      ",\"maxInputSize\":" + std::to_string(maxInputSize) + "}");
  }
  RelBuilder reduce(const std::vector<Expr> &e, const std::vector<std::string> &accs) const {
    std::string es, as;
    for (const auto &x : e) es += (es.empty() ? "" : ",") + x.json();
    for (const auto &a : accs) as += (as.empty() ? "" : ",") + Expr::q(a);
    return RelBuilder("{\"operator\":\"reduce\",\"input\":" + json_ + ",\"e\":[" + es + "],\"accumulator\":[" +
                      as + "],\"p\":{\"expression\":\"bool\",\"v\":true}}");
  }
  // ORDER BY: (expression, "ASC" | "DESC" | "NONE") per key (reference's sort).
  RelBuilder sort(const std::vector<std::pair<Expr, std::string>> &keys) const {
    std::string es;
    for (const auto &k : keys)
      es += (es.empty() ? "" : ",") + std::string("{\"expression\":") + k.first.json() +
            ",\"direction\":" + Expr::q(k.second) + "}";
    return RelBuilder("{\"operator\":\"sort\",\"input\":" + json_ + ",\"e\":[" + es + "]}");
  }
  PreparedStatement prepare(gbj_catalog *cat) const { return PreparedStatement(cat, json_); }
  const std::string &json() const { return json_; }

 private:
  explicit RelBuilder(std::string json) : json_(std::move(json)) {}
  std::string json_;
};

}  // namespace gbj

#endif  // GBJ_RELBUILDER_HPP
