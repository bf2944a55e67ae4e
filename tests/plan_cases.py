"""The reference's golden test cases written as plans (reference plan format)
with the RelBuilder mirror; shared by the plan tests."""
from proteus_gb300.plan import RelBuilder, cast64, col, lit

S, R, B, L = "inputs/sailors.csv", "inputs/reserves.csv", "inputs/boats.csv", "inputs/lineitem.tbl"


def sailors_join_left3():
    # tests-join-sailors.cpp:127-165: sailors probes reserves, then boats
    j = RelBuilder.scan(S, ["sid"]).join(RelBuilder.scan(R, ["sid", "bid"]), col(R, "sid"), col(S, "sid"),
                                         16, 128)
    j = j.join(RelBuilder.scan(B, ["bid"]), col(B, "bid"), col(R, "bid"), 16, 128)
    return j.reduce([col(S, "sid"), cast64(col(S, "sid")), lit(1)], ["max", "sum", "sum"])


def three_way_join():
    # tests-output.cpp:240-281: reserves probes sailors (4, 16), then boats
    j = RelBuilder.scan(R, ["sid", "bid"]).join(RelBuilder.scan(S, ["sid"]), col(S, "sid"), col(R, "sid"), 4, 16)
    j = j.join(RelBuilder.scan(B, ["bid"]), col(B, "bid"), col(R, "bid"), 4, 16)
    return j.reduce([col(S, "sid"), col(S, "sid"), lit(1)], ["max", "sum", "sum"])


def reduce_join():
    # tests-plan-parsing.cpp:96-101: radix join sailors.sid = reserves.sid, SUM 1
    j = RelBuilder.scan(S, ["sid"]).radix_join(RelBuilder.scan(R, ["sid"]), col(S, "sid"), col(R, "sid"))
    return j.reduce([lit(1)], ["sum"])


def nest_reserves():
    return RelBuilder.scan(R, ["sid"]).groupby([col(R, "sid")], [(lit(1), "sum")], 4, 16)


def multinest_reserves():
    return RelBuilder.scan(R, ["sid", "bid"]).groupby([col(R, "sid")], [(lit(1), "sum"), (col(R, "bid"), "max")],
                                                      4, 16)


def nest_bag_tpch():
    return (RelBuilder.scan(L, ["l_orderkey", "l_linenumber", "l_quantity"])
            .filter(col(L, "l_orderkey") < 4)
            .groupby([col(L, "l_linenumber")], [(lit(1), "sum"), (col(L, "l_quantity"), "max")], 4, 16))


ALL = {"sailorsJoinLeft3": sailors_join_left3, "3wayJoin": three_way_join, "reduce-join": reduce_join,
       "nestReserves": nest_reserves, "multinestReserves": multinest_reserves, "nestBagTPCH": nest_bag_tpch}
