"""The synthetic map generator on the GPU (mlc_rayshoot) against the oracle's ray shooter.

Both do the same IEEE FP32 operations in the same order (explicitly rounded on the GPU,
-ffp-contract=off on the host), so the ray counts are equal pixel for pixel.  The FP64
numpy restatement (synth.rayshoot_numpy) differs only by rays landing within FP32
rounding of a pixel edge.  The reference reads such maps from gerlumph files
(magnification_map.cpp:7-40); it has no generator of its own.
"""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,kappa,gamma,seed,rpp", [(300, 0.45, 0.35, 2, 4.0), (512, 0.4, 0.4, 0, 8.0),
                                                    (200, 0.3, 0.55, 9, 2.0)])
def test_rayshoot_counts_equal_oracle(ctx, N, kappa, gamma, seed, rpp):
    mp, meta = synth.rayshoot_gpu(ctx, N, 20.0, kappa, gamma, seed=seed, rays_per_pixel=rpp, dtype=torch.float64)
    counts_o, map_o = oracle.rayshoot(N, 20.0, kappa, gamma, seed, rpp)
    got = np.rint(mp.cpu().numpy() * meta["avgN"]).astype(np.int64)
    assert np.array_equal(got, counts_o.astype(np.int64))
    np.testing.assert_allclose(mp.cpu().numpy(), map_o, rtol=1e-15, atol=0)
    # the FP64 restatement: only rays within rounding of an edge move, to a neighbouring pixel
    _, counts_np, _ = synth.rayshoot_numpy(N, 20.0, kappa, gamma, seed, rpp)
    moved = int(np.abs(counts_np.astype(np.int64) - counts_o).sum())
    assert counts_np.sum() - counts_o.sum() in range(-moved, moved + 1)
    assert moved <= 1e-3 * counts_o.sum()
