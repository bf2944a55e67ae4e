// Drives gbj_relbuilder.hpp the way the reference's operator tests drive
// RelBuilder (core/olap/tests/operator-tests/tests-join-sailors.cpp).
//   relbuilder_main validate        -> one line per plan: name status
//   relbuilder_main run TABLES.txt  -> one line per plan: name col=v,v,...;
// TABLES.txt lines: "<relation> <attribute> v1 v2 ...".
#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "gbj_relbuilder.hpp"

using gbj::AggExpr;
using gbj::Expr;
using gbj::RelBuilder;

static const std::string S = "inputs/sailors.csv", R = "inputs/reserves.csv", B = "inputs/boats.csv",
                         L = "inputs/lineitem.tbl";

static std::vector<std::pair<std::string, RelBuilder>> plans() {
  std::vector<std::pair<std::string, RelBuilder>> v;
  {
    auto j = RelBuilder::scan(S, {"sid"}).join(RelBuilder::scan(R, {"sid", "bid"}), Expr::col(R, "sid"),
                                               Expr::col(S, "sid"), 16, 128);
    j = j.join(RelBuilder::scan(B, {"bid"}), Expr::col(B, "bid"), Expr::col(R, "bid"), 16, 128);
    v.push_back({"sailorsJoinLeft3", j.reduce({Expr::col(S, "sid"), Expr::col(S, "sid").cast64(), Expr::lit((int64_t)1)},
                                              {"max", "sum", "sum"})});
  }
  v.push_back({"multinestReserves",
               RelBuilder::scan(R, {"sid", "bid"})
                   .groupby({Expr::col(R, "sid")}, {{Expr::lit((int64_t)1), "sum"}, {Expr::col(R, "bid"), "max"}}, 4, 16)});
  v.push_back({"nestBagTPCH", RelBuilder::scan(L, {"l_orderkey", "l_linenumber", "l_quantity"})
                                  .filter(Expr::col(L, "l_orderkey") < 4)
                                  .groupby({Expr::col(L, "l_linenumber")},
                                           {{Expr::lit((int64_t)1), "sum"}, {Expr::col(L, "l_quantity"), "max"}}, 4, 16)});
  return v;
}

int main(int argc, char **argv) {
  if (argc >= 2 && std::string(argv[1]) == "validate") {
    for (auto &p : plans()) {
      char err[256];
      const int rc = gbj_plan_validate(p.second.json().c_str(), err, sizeof(err));
      std::printf("%s %d %s\n", p.first.c_str(), rc, err);
    }
    return 0;
  }
  if (argc < 3) return 2;
  gbj_ctx *ctx = nullptr;
  if (gbj_ctx_create(0, 1ull << 28, &ctx) != GBJ_OK) return 3;
  gbj_catalog *cat = nullptr;
  gbj_catalog_create(ctx, &cat);
  std::vector<int32_t *> bufs;
  std::ifstream in(argv[2]);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string rel, attr;
    ls >> rel >> attr;
    std::vector<int32_t> vals;
    for (int64_t x; ls >> x;) vals.push_back((int32_t)x);
    int32_t *d = nullptr;
    cudaMalloc(&d, vals.size() * 4 + 4);
    cudaMemcpy(d, vals.data(), vals.size() * 4, cudaMemcpyHostToDevice);
    bufs.push_back(d);
    gbj_catalog_add_column(cat, rel.c_str(), attr.c_str(), d, vals.size());
  }
  int rc = 0;
  for (auto &p : plans()) {
    try {
      const gbj::Result r = p.second.prepare(cat).execute();
      std::printf("%s", p.first.c_str());
      for (size_t i = 0; i < r.names.size(); ++i) {
        std::printf(" %s=", r.names[i].c_str());
        for (uint64_t j = 0; j < r.rows; ++j) std::printf("%s%lld", j ? "," : "", (long long)r.cols[i][j]);
      }
      std::printf("\n");
    } catch (const std::exception &e) {
      std::printf("%s ERROR %s %s\n", p.first.c_str(), e.what(), gbj_last_error(ctx));
      rc = 1;
    }
  }
  gbj_catalog_destroy(cat);
  for (auto *d : bufs) cudaFree(d);
  gbj_ctx_destroy(ctx);
  return rc;
}
