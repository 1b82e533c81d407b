"""sdemc_price_noalloc: pricing for callers that cannot allocate device memory.

Hosts that own all GPU memory through their own pool, or that must not call
cudaMalloc while building a CUDA graph, call this entry point with only their
inputs and outputs; its scratch is a fixed array inside the library.  This file
is collected after the other kernel tests, so that a run stopping at the first
failure has already run them; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from sde_mc_gb300 import _native as N
from sde_mc_gb300 import kernels as K
from tests.cases import indep2d, inst_for, merton1d


def _noalloc(inst, payoffs=None):
    lib = N.load()
    out = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.sdemc_price_noalloc(ctypes.byref(inst), None, N.ptr(out), N.ptr(payoffs),
                                 N.stream_handle(out.device))
    N.check(rc, "sdemc_price_noalloc")
    return out


@pytest.mark.gpu
def test_noalloc_matches_price_on_two_calls_in_a_row():
    N.require_cuda()
    first = inst_for(indep2d(256), num_paths=300_000, seed=5, path_offset=0)
    second = inst_for(merton1d(100), num_paths=123_457, seed=9, path_offset=77)
    for inst in (first, second):
        n = int(inst.num_paths)
        pay_a = torch.empty(n, dtype=torch.float32, device="cuda")
        pay_b = torch.empty(n, dtype=torch.float32, device="cuda")
        got = _noalloc(inst, pay_a).cpu().numpy()
        ref = K.price(inst, payoffs=pay_b).cpu().numpy()
        # same kernels, same reduction order: the outputs agree bit for bit
        np.testing.assert_array_equal(got, ref)
        np.testing.assert_array_equal(pay_a.cpu().numpy(), pay_b.cpu().numpy())
        assert got[2] == n and got[5] == 0
    # a third call reuses the array left over from the second one
    again = _noalloc(second).cpu().numpy()
    np.testing.assert_array_equal(again, K.price(second).cpu().numpy())


@pytest.mark.gpu
def test_noalloc_rejects_sizes_over_the_limit():
    N.require_cuda()
    lib = N.load()
    assert lib.sdemc_price_noalloc_scratch_bytes() >= 256 + (1 << 23) // 32 * 24
    inst = inst_for(merton1d(10), num_paths=(1 << 23) + 1, seed=1)
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    rc = lib.sdemc_price_noalloc(ctypes.byref(inst), None, N.ptr(out), None, N.stream_handle(out.device))
    assert rc == N.ENOMEM
    assert "no-allocation limit" in N.last_error()
