"""The depth Gaussian blur on the GPU equals the oracle's restatement bit for bit: kernel
half-widths 0..31, integer and fractional spreads, ragged sizes, host and device buffers, and
the splat depth of a real frame."""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("W,H,N,spread", [(1, 1, 0, 1.0), (1, 1, 5, 1.0), (17, 5, 2, 1.0), (64, 48, 8, 1.0),
                                          (64, 48, 8, 2.5), (33, 20, 31, 1.0), (40, 30, 3, 7.3)])
def test_blur_matches_oracle(fmlib, ctx, W, H, N, spread):
    rng = np.random.default_rng(W * 1000 + H + N)
    depth = rng.uniform(0.2, 1.0, W * H).astype(np.float32)
    depth[rng.random(W * H) < 0.3] = 1.0
    want = O.depth_blur(depth, W, H, N, spread)
    got = fmlib.depth_blur(ctx, depth, W, H, N, spread)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    d = torch.from_numpy(depth).cuda()
    o = torch.empty_like(d)
    fmlib.depth_blur(ctx, d, W, H, N, spread, out=o)
    ctx.sync()
    assert np.array_equal(o.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_blur_of_splat_depth(fmlib, ctx):
    sc = scenes.small_scene(seed=3, n=8000, width=160, height=120)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    z = np.zeros(cam.width * cam.height, np.float32)
    fmlib.splat_depth(s, cam, z)
    got = fmlib.depth_blur(ctx, z, cam.width, cam.height)  # the reference's defaults: N 8, spread 1
    want = O.depth_blur(z, cam.width, cam.height, 8, 1.0)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.any(got != z)
    s.close()


def test_blur_rejects_bad_arguments(fmlib, ctx):
    z = np.zeros(16, np.float32)
    for args in ((4, 4, 32, 1.0), (4, 4, -1, 1.0), (0, 4, 2, 1.0), (4, 4, 2, 0.0), (4, 4, 2, float("nan"))):
        with pytest.raises(fmlib.FmError):
            fmlib.depth_blur(ctx, z, *args)
