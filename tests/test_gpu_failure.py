"""Failure detection on the GPU without a fault: bounded waits report and return.

The tensor-core kernels wait on mbarriers for their MMAs with a bounded number
of polls; when the limit runs out the kernel sets a status bit, the host turns
it into FM_ERR_DEVICE, and the context stays usable.  The test makes such a
wait run out on a barrier that never completes (one of two arrivals made),
then marches a scene on the same context and checks it against the oracle.
"""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_and_context_survives(fmlib, ctx):
    L = ctx.L
    assert L.fm_selftest_wait_timeout(ctx.h, 0) == fmlib.FM_ERR_INVALID
    for polls in (1, 1000, 20000):
        assert L.fm_selftest_wait_timeout(ctx.h, polls) == fmlib.FM_ERR_DEVICE
        assert b"status word 8" in L.fm_last_error(ctx.h)
    # the status word was cleared and the context still marches correctly
    sc = scenes.small_scene(seed=21, n=6000, width=80, height=60)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    g = fmlib.render(s, cam, fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_EXACT))
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, g["start_depth"])
    for k in ("position", "normal", "depth", "colour"):
        assert np.array_equal(g[k].view(np.uint32), o[k].view(np.uint32)), k
    s.close()
