"""Bounded device-side waits driven to their limit.

The inter-CTA and asynchronous waits of the library are bounded: the radix
sort's look-back on its predecessors' published counts and the waits for the
tensor-core MMAs of the priority MLP.  mdas_test_set_wait_limit sets the number
of polls after which each of them reports MDAS_ERR_TIMEOUT; these tests set it
to one poll and check that the status reaches the caller, that the GPU keeps
answering, and (for the MMA waits, which wait on for their MMAs) that the
results are still those of an undisturbed run.  No wait is made to hang: the
MMAs complete by themselves, the look-back gives up.
"""
import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.fixture
def wait_limit(cuda):
    lib = N.load()

    def set_limit(polls):
        N.check(lib.mdas_test_set_wait_limit(int(polls)), "mdas_test_set_wait_limit")

    yield set_limit
    set_limit(0)  # the waits' own limits again


def test_sort_lookback_gives_up_and_reports(cuda, wait_limit):
    import torch
    n = 1 << 22
    g = torch.Generator().manual_seed(5)
    keys = torch.randint(0, 1 << 62, (n,), generator=g, dtype=torch.int64).cuda()
    wait_limit(1)
    with pytest.raises(N.MdasError) as ei:
        P.radix_sort_pairs(keys, None, 0, 64)
    assert ei.value.status == N.MDAS_ERR_TIMEOUT
    wait_limit(0)
    sk, order = P.radix_sort_pairs(keys, None, 0, 64)  # the GPU still answers, the sort is whole again
    k = keys.cpu().numpy().view(np.uint64)
    np.testing.assert_array_equal(order.cpu().numpy().astype(np.int64), np.argsort(k, kind="stable"))
    np.testing.assert_array_equal(sk.cpu().numpy().view(np.uint64), np.sort(k))


def test_mlp_wait_reports_and_keeps_results(cuda, wait_limit):
    import torch
    g = torch.Generator().manual_seed(3)
    params = (torch.randn(N.MLP_PARAMS, generator=g) * 0.1).cuda()
    feats = torch.randn(4096, 16, generator=g).cuda()
    want = P.mlp_forward(params, feats).cpu()
    wait_limit(1)
    out = torch.empty(4096, dtype=torch.float32, device="cuda")
    rc = N.load().mdas_mlp_forward(params.data_ptr(), feats.data_ptr(), 4096, out.data_ptr(), None)
    wait_limit(0)
    assert rc == N.MDAS_ERR_TIMEOUT
    torch.testing.assert_close(out.cpu(), want, rtol=0, atol=0)
    # and the same call with the waits' own limits reports no timeout
    torch.testing.assert_close(P.mlp_forward(params, feats).cpu(), want, rtol=0, atol=0)
