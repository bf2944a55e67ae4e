"""Seeded synthetic inputs of the workload shapes (libgbj_datagen.so, the C
ABI of include/gbj_datagen.h).

A library of its own, so that code which must not load the GPU library (the
benchmark's CPU arm, which times the oracle alone) can still generate the
exact columns the GPU arm uses.  Every generator is a pure function of its
seed and row index: the same arrays come out on every host, for any thread
count.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbj_datagen.so")

vp, u64, i32, dbl = C.c_void_p, C.c_uint64, C.c_int32, C.c_double

# name -> (restype, argtypes); mirrors include/gbj_datagen.h
SIGNATURES = {
    "gbj_gen_build_side": (C.c_int, [u64, u64, vp, vp, C.c_int]),
    "gbj_gen_probe_uniform": (C.c_int, [u64, u64, u64, vp, vp, C.c_int]),
    "gbj_gen_probe_zipf": (C.c_int, [u64, u64, u64, dbl, dbl, vp, vp, C.c_int]),
    "gbj_gen_groupby": (C.c_int, [u64, u64, u64, dbl, vp, vp, C.c_int]),
    "gbj_gen_uniform_i32": (C.c_int, [u64, u64, u64, i32, i32, vp, C.c_int]),
    "gbj_gen_serve_query": (C.c_int, [u64, u64, u64, dbl, u64, vp, vp, vp, vp, C.c_int]),
    "gbj_gen_rand": (u64, [u64, u64, u64]),
    "gbj_gen_perm": (u64, [u64, u64, u64, u64]),
    "gbj_gen_zipf": (u64, [u64, u64, u64, dbl, u64]),
    "gbj_gen_det_log": (dbl, [dbl]),
    "gbj_gen_det_exp": (dbl, [dbl]),
}

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def load() -> C.CDLL:
    """The generator library (built in-tree when missing: plain host C++)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(rc, what):
    if rc:
        raise ValueError(f"{what}: bad argument (status {rc})")


def gen_build_side(seed: int, n: int, payload=True, threads=0):
    """Build side of the joins: keys a seeded permutation of 1..n, payload U[0, 1000)."""
    k = np.empty(n, dtype=np.int32)
    p = np.empty(n, dtype=np.int32) if payload else None
    _check(load().gbj_gen_build_side(seed, n, _p(k), _p(p), threads), "gen_build_side")
    return k, p


def gen_probe_uniform(seed: int, n: int, n_build: int, payload=True, threads=0):
    """Probe side hitting a uniform build key 1..n_build, payload U[0, 1000)."""
    k = np.empty(n, dtype=np.int32)
    p = np.empty(n, dtype=np.int32) if payload else None
    _check(load().gbj_gen_probe_uniform(seed, n, n_build, _p(k), _p(p), threads), "gen_probe_uniform")
    return k, p


def gen_probe_zipf(seed: int, n: int, n_build: int, theta: float, hit_rate=0.5, payload=False,
                   threads=0):
    """Probe side: a hit (probability hit_rate) is a build key of Zipf(theta)
    rank, a miss a key in n_build+1..2 n_build."""
    k = np.empty(n, dtype=np.int32)
    p = np.empty(n, dtype=np.int32) if payload else None
    _check(load().gbj_gen_probe_zipf(seed, n, n_build, theta, hit_rate, _p(k), _p(p), threads),
           "gen_probe_zipf")
    return k, p


def gen_groupby(seed: int, n: int, cardinality: int, theta: float = 0.0, threads=0):
    """Group-by input: `cardinality` distinct keys (uniform or Zipf), values U[-2^20, 2^20)."""
    k = np.empty(n, dtype=np.int32)
    v = np.empty(n, dtype=np.int32)
    _check(load().gbj_gen_groupby(seed, n, cardinality, theta, _p(k), _p(v), threads), "gen_groupby")
    return k, v


def gen_uniform_i32(seed: int, stream: int, n: int, lo: int, hi: int, threads=0):
    out = np.empty(n, dtype=np.int32)
    _check(load().gbj_gen_uniform_i32(seed, stream, n, lo, hi, _p(out), threads), "gen_uniform_i32")
    return out


def gen_serve_query(seed: int, n_build: int, n_probe: int, match_rate: float, cardinality: int,
                    threads=0):
    """(build keys, build groups, probe keys, probe values) of one served query."""
    bk, bg = np.empty(n_build, np.int32), np.empty(n_build, np.int32)
    pk, pv = np.empty(n_probe, np.int32), np.empty(n_probe, np.int32)
    _check(load().gbj_gen_serve_query(seed, n_build, n_probe, match_rate, cardinality, _p(bk), _p(bg),
                                      _p(pk), _p(pv), threads), "gen_serve_query")
    return bk, bg, pk, pv


def rand(seed: int, stream: int, i: int) -> int:
    return int(load().gbj_gen_rand(seed, stream, i))
