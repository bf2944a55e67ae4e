"""Loading relations from the reference's columnar file layout into device
memory and querying them with plans."""
import numpy as np
import pytest

from gpu_util import cpu_threads
from proteus_gb300 import abi, columnar
from proteus_gb300.plan import Catalog, RelBuilder, col, lit

pytestmark = pytest.mark.gpu

LO, D = "inputs/ssb/lineorder.csv", "inputs/ssb/date.csv"


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    base = tmp_path_factory.mktemp("columnar")
    rng = np.random.default_rng(9)
    n, nd = (1 << 20) + 5, 2557
    lo = {"lo_orderdate": rng.integers(0, nd, n).astype(np.int32) + 19920101,
          "lo_quantity": rng.integers(1, 51, n).astype(np.int32),
          "lo_revenue": rng.integers(0, 1 << 20, n).astype(np.int32),
          "lo_ordtotalprice64": rng.integers(0, 1 << 40, n).astype(np.int64)}  # skipped: int64
    d = {"d_datekey": np.arange(nd, dtype=np.int32) + 19920101,
         "d_year": (1992 + np.arange(nd) // 365).astype(np.int32)}
    cat = {"lineorder": columnar.write_relation(str(base), LO, lo),
           "date": columnar.write_relation(str(base), D, d)}
    columnar.write_catalog(str(base / "catalog.json"), cat)
    return base, lo, d


def test_load_and_query(ctx, files):
    base, lo, d = files
    c = Catalog(ctx)
    assert c.load(str(base / "catalog.json"), str(base)) == 5  # the int64 column is skipped
    plan = (RelBuilder.scan(LO, ["lo_orderdate", "lo_quantity", "lo_revenue"])
            .filter(col(LO, "lo_quantity") < 25)
            .join(RelBuilder.scan(D, ["d_datekey", "d_year"]), col(D, "d_datekey"), col(LO, "lo_orderdate"))
            .groupby([col(D, "d_year")], [(col(LO, "lo_revenue"), "sum"), (lit(1), "sum")], 10, 1 << 21))
    out = c.execute(plan)
    keep = lo["lo_quantity"] < 25
    years = d["d_year"][lo["lo_orderdate"][keep] - 19920101]
    exp_years = np.unique(years)
    assert out["d_year"].tolist() == exp_years.tolist()
    assert out["sum_0"].tolist() == [int(lo["lo_revenue"][keep][years == y].astype(np.int64).sum()) for y in exp_years]
    assert out["sum_1"].tolist() == [int((years == y).sum()) for y in exp_years]
    c.close()


def test_load_one_relation_and_errors(ctx, files, tmp_path):
    base, lo, d = files
    c = Catalog(ctx)
    assert c.load(str(base / "catalog.json"), str(base), relation="date") == 2
    out = c.execute(RelBuilder.scan(D, ["d_year"]).reduce([col(D, "d_year"), lit(1)], ["max", "sum"]))
    assert [int(v[0]) for v in out.values()] == [int(d["d_year"].max()), len(d["d_year"])]
    with pytest.raises(abi.GbjError):
        c.load(str(tmp_path / "missing.json"))
    bad = tmp_path / "cat.json"
    columnar.write_catalog(str(bad), {"x": {"path": "nowhere/x.csv", "type": {"type": "bag", "inner": {
        "type": "record", "attributes": [{"type": {"type": "int"}, "relName": "nowhere/x.csv", "attrName": "a"}]}}}})
    with pytest.raises(abi.GbjError) as e:
        c.load(str(bad), str(tmp_path))
    assert "cannot open" in str(e.value)
    c.close()
