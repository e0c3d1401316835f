"""The depth Gaussian blur (GaussRenderPass.cpp:13-57, gauss.frag) in the oracle, pinned against the
reference's own restatement of the pass (tools/gauss.py: the same kernel in double precision,
nearest texel with the index clamped to the image) and the kernel formula; no GPU."""

import math

import numpy as np
import pytest

import oracle as O


def reference_tool_blur(depth, W, H, N):
    """tools/gauss.py restated with numpy: exp(-r^2/2) weights normalised over the grid, the
    clamped neighbourhood summed in double."""
    ii, jj = np.meshgrid(np.arange(-N, N + 1), np.arange(-N, N + 1), indexing="ij")
    k = np.exp(-0.5 * (ii * ii + jj * jj))
    k /= k.sum()
    img = depth.reshape(H, W).astype(np.float64)
    out = np.zeros((H, W))
    for a in range(-N, N + 1):
        for b in range(-N, N + 1):
            xs = np.clip(np.arange(W) + a, 0, W - 1)
            ys = np.clip(np.arange(H) + b, 0, H - 1)
            out += k[a + N, b + N] * img[np.ix_(ys, xs)]
    return out.reshape(-1)


@pytest.mark.parametrize("n", [0, 1, 2, 8, 31])
def test_weights(n):
    w = O.gauss_weights(n).astype(np.float64)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    g = np.exp(-0.5 * (ii * ii + jj * jj))
    full = g[0, 0] + 2 * g[0, 1:].sum() + 2 * g[1:, 0].sum() + 4 * g[1:, 1:].sum()
    # the FP32 exponent -r^2/2 carries the rounding of r = sqrt(i^2 + j^2): relative error ~ r^2/2 ulps
    # (weights below the FP32 normal range come out subnormal or 0)
    tol = 2e-6 + 1.5e-7 * 0.5 * (ii * ii + jj * jj)
    ref = g / full
    normal = ref > 1e-36
    assert np.all(np.abs(w - ref)[normal] <= (tol * ref)[normal])
    assert np.all(w[~normal] <= 1e-36)
    total = w[0, 0] + 2 * w[0, 1:].sum() + 2 * w[1:, 0].sum() + 4 * w[1:, 1:].sum()
    assert total == pytest.approx(1.0, abs=1e-6)
    assert np.array_equal(w, w.T)


@pytest.mark.parametrize("W,H,N", [(1, 1, 3), (17, 5, 2), (40, 30, 8)])
def test_blur_matches_reference_tool(W, H, N):
    rng = np.random.default_rng(W * 100 + H)
    depth = rng.uniform(0.2, 1.0, W * H).astype(np.float32)
    depth[rng.random(W * H) < 0.3] = 1.0  # no particle
    got = O.depth_blur(depth, W, H, N, 1.0)
    want = reference_tool_blur(depth, W, H, N)
    assert np.allclose(got, want, rtol=2e-6, atol=0)


def test_blur_spread_interpolates_between_texels():
    W, H = 24, 16
    x = np.tile(np.arange(W, dtype=np.float32), H) / W
    # a horizontal ramp is linear, so the blur of it with any spread stays the ramp away from the edges
    got = O.depth_blur(x, W, H, 2, 1.5).reshape(H, W)
    assert np.allclose(got[:, 6:-6], x.reshape(H, W)[:, 6:-6], atol=2e-6)
    const = np.full(W * H, 0.625, np.float32)
    assert np.allclose(O.depth_blur(const, W, H, 4, 3.7), 0.625, rtol=1e-6)
