"""fnd_rt_tonemap (linear RGB -> R8G8B8A8_UNORM) against the oracle's display
encoding: every curve, host and device buffers, exposure, special values;
codes equal up to one step (the device evaluates x^(1/2.4) with powf)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_tonemap_matches_oracle(built):
    import torch
    import foundation_gb300 as fg
    rng = np.random.default_rng(5)
    h, w = 61, 97
    rgb = (rng.lognormal(-1.0, 2.0, (h, w, 3))).astype(np.float32)
    rgb[0, :5] = [[0, 0, 0], [-1, -2, -3], [np.nan, 1, np.inf], [0.0031308, 0.0031309, 1e-8], [1, 1, 1]]
    with fg.Context(0) as ctx:
        for mode in (fg.TONEMAP_CLAMP, fg.TONEMAP_REINHARD, fg.TONEMAP_ACES):
            for exposure in (1.0, 0.25, 4.0):
                got = ctx.tonemap(rgb, w, h, exposure, mode)
                want = O.tonemap_rgba8(rgb, exposure, mode)
                d = np.abs(got.astype(int) - want.astype(int))
                assert d.max() <= 1 and (d > 0).mean() < 0.01, (mode, exposure, d.max())
        dev_in = torch.from_numpy(rgb.reshape(-1)).cuda()
        dev_out = torch.empty(h * w * 4, dtype=torch.uint8, device="cuda")
        ctx.tonemap(dev_in, w, h, 1.0, fg.TONEMAP_ACES, out=dev_out)
        ctx.sync()
        assert np.array_equal(dev_out.cpu().numpy().reshape(h, w, 4), ctx.tonemap(rgb, w, h, 1.0, fg.TONEMAP_ACES))
        with pytest.raises(fg.FndError):
            ctx.tonemap(rgb, w, h, 1.0, 7)
        with pytest.raises(fg.FndError):
            ctx.tonemap(rgb, w, h, -1.0, 0)
