"""The bounded-wait error path of the tensor-core kernels.

Every wait between the roles of a tcgen05 kernel (TMA producer, MMA issuer,
accumulator drain) gives up after a limit of %globaltimer time.  Setting the
limit to 1 ns (nla_set_wait_limit_ns) makes nearly every wait that does not
complete at once give up, on an ordinary update whose waits would otherwise
all complete: the kernel must then report NLA_ERR_TIMEOUT through
nla_device_status, drain its own in-flight loads and MMAs, release its tensor
memory and return, so that the next call with the default limit runs and
returns the same bits as before.  No wait here is left without an end: the
drain waits keep the default 2 s limit.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cm(rng, r, c, dev):
    import torch

    return torch.tensor(rng.uniform(-1, 1, (c, r)), device=dev, dtype=torch.float64).T


@pytest.mark.parametrize("split_terms,K", [(7, 1500), (7, 200), (3, 700)])
def test_timeout_reports_and_next_call_recovers(pkg, lib, cuda, split_terms, K):
    import torch

    from nextla_gb300 import _lib

    rng = np.random.default_rng(K)
    M, N = 640, 384
    A, B, C0 = _cm(rng, M, K, cuda), _cm(rng, K, N, cuda), _cm(rng, M, N, cuda)

    def update():
        C = torch.empty_like(C0.T).T
        C.copy_(C0)
        pkg.matmul_mixed_(C, A, B, -1.0, split_terms=split_terms)
        return C

    ref = update()
    pkg.device_status(ref)
    try:
        _lib.check(lib.nla_set_wait_limit_ns(1))
        update()
        with pytest.raises(_lib.NLAError) as err:
            pkg.device_status()
        assert err.value.code == _lib.NLA_ERR_TIMEOUT
    finally:
        _lib.check(lib.nla_set_wait_limit_ns(0))
    pkg.device_status()  # the error word was cleared by the report above
    for _ in range(2):
        again = update()
        pkg.device_status(again)
        assert torch.equal(again, ref)
