"""Helpers shared by the GPU parity tests."""
import numpy as np

from proteus_gb300 import abi


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


CONFIG1_AGGS = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_PRODUCT)]
CONFIG2_AGGS = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_ROWID_XOR)]


def sort_groups(keys, cnt, s, mn, mx, n):
    n = int(n)
    k = keys[:n]
    order = np.argsort(k, kind="stable")
    return k[order], cnt[:n][order], s[:n][order], mn[:n][order], mx[:n][order]


def cpu_threads():
    import os

    return max(1, os.cpu_count() or 1)
