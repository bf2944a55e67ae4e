"""The C ABI library loads, exports every declared entry point, and its host
side (generators, argument checks) behaves without a GPU."""
import math
import os
import re

import numpy as np
import pytest

import datagen
from proteus_gb300 import abi, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header=None):
    """gbj_* entry points declared in include/*.h (or in one header)."""
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h") and (header is None or f == header):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gbj_[a-z0-9_]+)\s*\(", src))
    return names


# each header, the library exporting it and its ctypes binding
LIBRARIES = {"gbjoin.h": (abi.load, abi.SIGNATURES), "gbj_datagen.h": (datagen.load, datagen.SIGNATURES)}


def test_every_header_has_a_library():
    headers = sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h"))
    assert headers == sorted(LIBRARIES)


@pytest.mark.parametrize("header", sorted(LIBRARIES))
def test_exports_every_declared_symbol(lib, header):
    load, _ = LIBRARIES[header]
    names = declared_symbols(header)
    assert len(names) >= 10
    so = load()
    missing = [n for n in sorted(names) if getattr(so, n, None) is None]
    assert not missing, missing


@pytest.mark.parametrize("header", sorted(LIBRARIES))
def test_binding_covers_header(lib, header):
    _, sigs = LIBRARIES[header]
    names = declared_symbols(header)
    unbound = sorted(n for n in names if n not in sigs)
    assert not unbound, unbound
    stale = sorted(n for n in sigs if n not in names)
    assert not stale, stale


def test_generators_live_apart_from_the_gpu_library(lib):
    """The generators are not in libgbjoin.so: a process that only generates
    inputs (the benchmark's CPU arm) never maps the GPU library."""
    assert getattr(lib, "gbj_gen_rand", None) is None
    assert not any(n.startswith("gbj_gen_") for n in declared_symbols("gbjoin.h"))


def test_ctx_create_without_gpu_fails_cleanly(lib):
    import ctypes as C

    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    h = C.c_void_p()
    rc = lib.gbj_ctx_create(0, 1 << 20, C.byref(h))
    assert rc in (abi.ERR_CUDA, abi.ERR_INVALID)
    assert h.value is None


def test_null_context_is_rejected(lib):
    assert lib.gbj_sync(None, None) == abi.ERR_INVALID
    assert lib.gbj_ctx_destroy(None) == abi.ERR_INVALID


def test_build_side_is_permutation(lib):
    for n in (1, 2, 3, 1000, 1 << 16, 100003):
        k, p = engine.gen_build_side(42, n)
        assert sorted(k.tolist()) == list(range(1, n + 1))
        assert p.min() >= 0 and p.max() < 1000


def test_probe_uniform_range(lib):
    k, p = engine.gen_probe_uniform(1, 1 << 16, 1000)
    assert k.min() >= 1 and k.max() <= 1000
    assert p.min() >= 0 and p.max() < 1000


@pytest.mark.parametrize("theta", [0.0, 0.5, 1.0])
def test_probe_zipf_shape(lib, theta):
    nr = 1 << 12
    k, _ = engine.gen_probe_zipf(3, 1 << 17, nr, theta, 0.5)
    hits = (k <= nr)
    assert abs(hits.mean() - 0.5) < 0.01
    assert k[hits].min() >= 1
    assert k[~hits].min() >= nr + 1 and k[~hits].max() <= 2 * nr
    counts = np.bincount(k[hits], minlength=nr + 1)[1:]
    top = np.sort(counts)[::-1]
    if theta == 1.0:
        # Zipf(1): most frequent rank ~ 1/H_N of the hits
        hn = sum(1.0 / i for i in range(1, nr + 1))
        assert abs(top[0] / hits.sum() - 1 / hn) < 0.01
    if theta == 0.0:
        assert top[0] < 5 * hits.sum() / nr


def test_zipf_sampler_distribution(lib):
    n, theta = 100, 1.0
    xs = np.array([datagen.load().gbj_gen_zipf(9, 1, n, theta, i) for i in range(40000)])
    assert xs.min() >= 1 and xs.max() <= n
    hn = sum(1.0 / i for i in range(1, n + 1))
    for r in (1, 2, 10):
        assert abs((xs == r).mean() - (1 / r) / hn) < 0.01


def test_deterministic_math(lib):
    for x in (1e-300, 1e-5, 0.3, 1.0, 1.5, 2.0, 10.0, 12345.678, 1e300):
        assert abs(datagen.load().gbj_gen_det_log(x) - math.log(x)) <= 1e-14 * max(1.0, abs(math.log(x)))
    for x in (-700.0, -5.0, -1e-3, 0.0, 0.5, 1.0, 3.7, 100.0, 700.0):
        assert abs(datagen.load().gbj_gen_det_exp(x) - math.exp(x)) <= 1e-14 * math.exp(x)


def test_generators_thread_count_independent(lib):
    a = engine.gen_groupby(5, 300000, 1 << 10, 1.0, threads=1)
    b = engine.gen_groupby(5, 300000, 1 << 10, 1.0, threads=7)
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    c = engine.gen_probe_zipf(5, 300000, 1 << 12, 0.5, 0.5, threads=1)
    d = engine.gen_probe_zipf(5, 300000, 1 << 12, 0.5, 0.5, threads=5)
    assert (c[0] == d[0]).all()


def test_groupby_generator_cardinality(lib):
    k, v = engine.gen_groupby(11, 1 << 18, 1 << 10, 0.0)
    assert len(np.unique(k)) == 1 << 10
    assert v.min() >= -(1 << 20) and v.max() < (1 << 20)
    kz, _ = engine.gen_groupby(11, 1 << 18, 1 << 10, 1.0)
    assert len(np.unique(kz)) <= 1 << 10
