"""The give-up path of the bounded mbarrier waits in the tensor-core kernels.

sdemc_wait_probe runs one warp that waits, through the same wait as K5tc,
K6tc and K7, on an mbarrier that nothing arrives at: the wait must give up
after its poll limit, record SDEMC_ETIMEOUT in the status word and return,
and the context must stay usable.  The wait is bounded, so the test cannot
hang the device.  Collected last, after every other kernel test.
"""

import numpy as np
import pytest
import torch

from sde_mc_gb300 import _native as N
from sde_mc_gb300 import kernels as K
from tests.cases import inst_for, merton1d


@pytest.mark.gpu
def test_bounded_wait_gives_up_with_a_status_and_the_context_survives():
    N.require_cuda()
    lib = N.load()
    inst = inst_for(merton1d(50), num_paths=100_000, seed=3)
    before = K.price(inst).cpu().numpy()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    for spins in (1, 256):
        status.zero_()
        N.check(lib.sdemc_wait_probe(spins, N.ptr(status), N.stream_handle(status.device)), "sdemc_wait_probe")
        torch.cuda.synchronize()
        assert int(status.item()) == N.ETIMEOUT
    # the same kernels give the same bits afterwards
    after = K.price(inst).cpu().numpy()
    np.testing.assert_array_equal(before, after)
    assert after[5] == 0
