"""The bounded-wait error path of the tensor-core kernels (mlc_selftest_wait_timeout): a
wait on an mbarrier that nothing arrives at, with no copy or MMA feeding it, gives up after
its poll limit, the call returns MLC_ERR_TIMEOUT, the tensor memory the CTA allocated is
released, and the context keeps working: the tensor-core pair kernel (which allocates tensor
memory on every SM it runs on) then matches the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
MLC_ERR_TIMEOUT = 4


@pytest.mark.parametrize("polls", [1, 2000])
def test_wait_gives_up_releases_tmem_and_context_stays_usable(ctx, polls):
    import microsn_gb300 as mlc
    st, rep = mlc.selftest_wait_timeout(ctx, polls)
    assert st == MLC_ERR_TIMEOUT
    assert "gave up" in ctx.L.mlc_ctx_last_error(ctx.h).decode()
    assert rep[0] == 1 and rep[1] == polls and rep[2] == 1, rep
    ctx.synchronize()
    rng = np.random.default_rng(5)
    NA, NB, T = 300, 200, 40
    A = (np.cumsum(rng.normal(0, 0.05, (NA, T)), axis=1) + rng.normal(0, 0.3, (NA, 1))).astype(np.float32)
    B = (np.cumsum(rng.normal(0, 0.05, (NB, T)), axis=1) + rng.normal(0, 0.3, (NB, 1))).astype(np.float32)
    w = 1.0 / rng.uniform(0.02, 0.1, T) ** 2
    d = rng.normal(0, 0.02, T)
    r = mlc.pair_chi2_magdiff(ctx, torch.as_tensor(A, device=DEV), torch.as_tensor(B, device=DEV), w, d, True,
                              method="tensor", nbins=100, lo=-6, hi=8, k=5, want_matrix=True)
    got = r["matrix"].cpu().numpy().astype(np.float64).ravel()
    ref = oracle.pair_chi2_magdiff(A, B, w, d, True)
    assert (np.abs(got - ref) / np.maximum(ref, 1e-300)).max() < 1e-5


def test_poll_limit_is_checked(ctx):
    import microsn_gb300 as mlc
    st, _ = mlc.selftest_wait_timeout(ctx, 0)
    assert st == 1  # MLC_ERR_ARG
