"""Batched views and work splits against single-view marches and the oracle.

A batch renders many views of many scenes (uneven particle counts,
resolutions and march settings) with one launch per pass under a CUDA graph;
every view must come out bit-identical to the same view rendered alone, and
the single-view march must not depend on the work split (tile shape, tiles
per claim, deferral limit, long-ray queue size).
"""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

KEYS = ("position", "normal", "depth", "colour", "start_depth")
SHAPE = {"position": 4, "normal": 4, "depth": 1, "colour": 4, "start_depth": 1}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def device_outputs(cam):
    npx = cam.width * cam.height
    return {k: torch.zeros((npx, SHAPE[k]) if SHAPE[k] > 1 else (npx,), dtype=torch.float32, device="cuda")
            for k in KEYS}


def host(out):
    return {k: v.cpu().numpy() for k, v in out.items()}


def single(fm, scene, cam, params):
    npx = cam.width * cam.height
    out = {"position": np.zeros((npx, 4), np.float32), "normal": np.zeros((npx, 4), np.float32),
           "depth": np.zeros(npx, np.float32), "colour": np.zeros((npx, 4), np.float32),
           "start_depth": np.zeros(npx, np.float32)}
    fm.march(scene, cam, params, out["position"], out["normal"], out["depth"], out["colour"], out["start_depth"])
    return out


def assert_same(a, b, what=""):
    for k in KEYS:
        if k not in a or k not in b:
            continue
        x, y = bits(a[k]), bits(b[k])
        bad = np.nonzero(np.any((x != y).reshape(x.shape[0], -1), axis=1))[0]
        assert bad.size == 0, f"{what} {k}: {bad.size} pixels differ, first {bad[:5]}"


@pytest.fixture(scope="module")
def small_batch(fmlib, ctx):
    """Six scenes of the sloshing family, 1-3 views each, mixed settings."""
    specs = [(3000, 64, 48), (9000, 120, 90), (1500, 33, 17), (20000, 160, 96), (6000, 96, 64), (12000, 80, 120)]
    rng = np.random.default_rng(5)
    items = []
    for i, (n, w, h) in enumerate(specs):
        sc = scenes.small_scene(seed=100 + i, n=n, width=w, height=h, max_steps=200)
        s = fmlib.Scene(ctx, sc.xyz, sc.support)
        for k in range(1 + i % 3):
            ang = rng.uniform(0, 2 * np.pi)
            eye = (0.5 + 1.8 * np.cos(ang), 1.2, 0.5 + 1.8 * np.sin(ang))
            cam = scenes.make_camera(eye, (0.5, 0.3, 0.5), w + 7 * k, h + 3 * k)
            params = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, (0, 8, 3)[k % 3], (i + k) % 3)
            items.append((sc, s, cam, params))
    return items


def make_views(fmlib, items):
    views, outs = [], []
    for sc, s, cam, params in items:
        o = device_outputs(cam)
        outs.append(o)
        views.append(fmlib.View(s, cam, params, **o))
    return views, outs


def test_batch_matches_single_views(fmlib, ctx, small_batch):
    views, outs = make_views(fmlib, small_batch)
    b = fmlib.Batch(ctx, views)
    info = b.info()
    assert info["n_views"] == len(views)
    assert info["graph_nodes"] >= 8  # counter reset, 5 depth-pass launches, 2 march launches
    b.run()
    ctx.sync()
    for i, (sc, s, cam, params) in enumerate(small_batch):
        assert_same(host(outs[i]), single(fmlib, s, cam, params), f"view {i}")
    # a second graph launch gives the same frame
    for o in outs:
        for v in o.values():
            v.zero_()
    b.run()
    ctx.sync()
    for i, (sc, s, cam, params) in enumerate(small_batch):
        assert_same(host(outs[i]), single(fmlib, s, cam, params), f"rerun view {i}")
    b.close()


def test_batch_view_matches_oracle(fmlib, ctx, small_batch, oracle_lib):
    sc, s, cam, params = small_batch[3]
    views, outs = make_views(fmlib, [small_batch[3]])
    b = fmlib.Batch(ctx, views)
    b.run()
    ctx.sync()
    g = host(outs[0])
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    assert np.array_equal(bits(g["start_depth"]), bits(depth))
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, params.bisect, depth, skip_mode=params.skip_mode)
    assert_same(g, o, "oracle")
    b.close()


def test_bench_batch_every_view_matches_oracle(fmlib, ctx, oracle_lib):
    """The benchmark's batch (64 sloshing-family scenes, 50k..2M particles, 146 views at 640x480 /
    1280x720 / 1920x1080, exact skip, 8 bisections) in one graph launch with the work split its
    autotuner picks (8x4 tiles, deferral after 64 sums): in every view, a seeded sample of 1,000 started pixels and 200 pixels anywhere bit-exact against
    the oracle's march of that view from the batch's start depths."""
    bs = scenes.batch_scenes()
    keep, views, outs, where = [], [], [], []
    for sc in bs:
        s = fmlib.Scene(ctx, sc.xyz, sc.support)
        keep.append(s)
        p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, sc.bisect, fmlib.FM_SKIP_EXACT)
        for cam in sc.cameras:
            o = device_outputs(cam)
            outs.append(o)
            views.append(fmlib.View(s, cam, p, **o))
            where.append((sc, cam))
    assert len(views) == 146
    b = fmlib.Batch(ctx, views, dict(tile_width=8, tiles_per_claim=1, defer_iters=64))
    b.run()
    ctx.sync()
    rng = np.random.default_rng(146)
    frames = {}
    checked = 0
    for o, (sc, cam) in zip(outs, where):
        if id(sc) not in frames:
            frames.clear()  # views of a scene are consecutive: keep one oracle frame at a time
            frames[id(sc)] = O.build_frame(sc.xyz, sc.support)
        fr = frames[id(sc)]
        z = o["start_depth"].cpu().numpy()
        started = np.nonzero(z < 1)[0]
        assert started.size > 1000
        pix = np.unique(np.concatenate([rng.choice(started, 1000, replace=False),
                                        rng.integers(0, cam.width * cam.height, 200)])).astype(np.int64)
        idx = torch.from_numpy(pix).cuda()
        g = {k: o[k].index_select(0, idx).cpu().numpy() for k in ("position", "normal", "depth", "colour")}
        ref = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, sc.bisect, z, pixels=pix)
        assert_same(g, {k: ref[k][pix] for k in g}, f"view {checked} ({cam.width}x{cam.height}, {sc.n} particles)")
        checked += 1
    assert checked == 146
    b.close()
    for s in keep:
        s.close()


@pytest.mark.parametrize("cfg", [
    dict(tile_width=1), dict(tile_width=2), dict(tile_width=4), dict(tile_width=16), dict(tile_width=32),
    dict(tile_width=8, tiles_per_claim=4), dict(tile_width=8, defer_iters=1), dict(tile_width=8, defer_iters=4096),
    dict(tile_width=8, long_queue=3), dict(tile_width=16, defer_iters=2, long_queue=1),
    dict(tile_width=8, regroup_iters=0), dict(tile_width=8, defer_iters=4, regroup_iters=1),
    dict(tile_width=4, defer_iters=8, regroup_iters=4096, defer_lanes=8),
])
def test_tile_config_does_not_change_results(fmlib, ctx, cfg):
    sc = scenes.small_scene(seed=44, n=12000, width=130, height=70)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1)
    ref = single(fmlib, s, cam, p)
    old = ctx.tile_config()
    try:
        ctx.set_tile_config(**cfg)
        ctx.set_stats(True)
        got = single(fmlib, s, cam, p)
        st = ctx.stats()
    finally:
        ctx.set_stats(False)
        ctx.set_tile_config(**old)
    assert_same(got, ref, str(cfg))
    if cfg.get("defer_iters") == 1 and "long_queue" not in cfg:
        assert st["deferred"] + st["regrouped"] > 0


def test_batch_tile_configs_and_autotune(fmlib, ctx, small_batch):
    views, outs = make_views(fmlib, small_batch[:5])
    b = fmlib.Batch(ctx, views, tile_config=dict(tile_width=32, tiles_per_claim=2, defer_iters=8, long_queue=2))
    b.run()
    ctx.sync()
    first = [host(o) for o in outs]
    best, ms = b.autotune(reps=1, candidates=[dict(tile_width=4), dict(tile_width=8, defer_iters=64)])
    assert best["tile_width"] in (4, 8) and ms > 0
    assert b.info()["config"]["tile_width"] == best["tile_width"]
    best, ms = b.autotune(reps=1)
    assert best["tile_width"] in (4, 8, 16, 32) and ms > 0
    for o in outs:
        for v in o.values():
            v.zero_()
    b.run()
    ctx.sync()
    for i in range(len(outs)):
        assert_same(host(outs[i]), first[i], f"view {i} after tuning")
    b.close()


def test_batch_counters(fmlib, ctx, small_batch):
    views, outs = make_views(fmlib, small_batch)
    b = fmlib.Batch(ctx, views)
    ctx.set_stats(True)
    try:
        b.run()
        ctx.sync()
        st = ctx.stats()
    finally:
        ctx.set_stats(False)
    assert st["rays"] == b.info()["pixels"]
    assert st["hits"] == sum(int((o["depth"] > 0).sum()) for o in outs)
    b.close()


def test_batch_scene_update_needs_refresh(fmlib, ctx):
    sc = scenes.small_scene(seed=61, n=6000, width=80, height=60)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1)
    views, outs = make_views(fmlib, [(sc, s, cam, p)])
    b = fmlib.Batch(ctx, views)
    moved = (sc.xyz + np.float32(0.01)).astype(np.float32)
    s.update(moved)
    with pytest.raises(fmlib.FmError):
        b.run()
    b.refresh()
    b.run()
    ctx.sync()
    assert_same(host(outs[0]), single(fmlib, s, cam, p), "after refresh")
    b.close()
    s.close()


def test_march_batch_one_shot(fmlib, ctx, small_batch):
    views, outs = make_views(fmlib, small_batch[:3])
    fmlib.march_batch(ctx, views)
    for i, (sc, s, cam, params) in enumerate(small_batch[:3]):
        assert_same(host(outs[i]), single(fmlib, s, cam, params), f"one-shot view {i}")


def test_batch_rejects_bad_views(fmlib, ctx, small_batch):
    sc, s, cam, params = small_batch[0]
    o = device_outputs(cam)
    with pytest.raises(fmlib.FmError):
        fmlib.Batch(ctx, [])
    bad = fmlib.MarchParams(params.iso, -1.0, params.max_steps)
    with pytest.raises(fmlib.FmError):
        fmlib.Batch(ctx, [fmlib.View(s, cam, bad, **o)])
    with pytest.raises(fmlib.FmError):
        fmlib.Batch(ctx, [fmlib.View(s, cam, params, **o)], tile_config=dict(tile_width=3))
    with pytest.raises(ValueError):
        fmlib.View(s, cam, params, position=np.zeros((cam.width * cam.height, 4), np.float32)).cstruct()


@pytest.mark.parametrize("which", ["constant", "trained"])
def test_batch_with_learned_views(fmlib, ctx, small_batch, which):
    """Views with FM_MARCH_PROPOSAL in a batch equal the same learned views marched alone.

    Half the views use the proposal, the others march every sample; the batch
    keeps its own copy of the proposal, so destroying the context's proposal
    after fm_batch_create changes nothing.
    """
    from fluidmarch import proposal as prop_mod
    if which == "constant":
        P = np.zeros(fmlib.FM_PROPOSAL_PARAMS, np.float32)
        P[-2:] = (0.6, 3.0)  # every ray: samples ks+1 .. kf with ks = floor(0.6 H / step)
        pr = fmlib.Proposal(ctx, P)
    else:
        P, _ = prop_mod.load()
        pr = fmlib.Proposal(ctx, P, margin_lo=0.5, margin_hi=0.5, min_near=2.0)
    fmlib.set_proposal(ctx, pr)
    items = []
    for i, (sc, s, cam, params) in enumerate(small_batch):
        learned = i % 2 == 0
        skip = params.skip_mode if not learned or params.skip_mode != fmlib.FM_SKIP_REFERENCE else fmlib.FM_SKIP_EXACT
        p = fmlib.MarchParams(params.iso, params.step, params.max_steps, params.bisect, skip, proposal=learned)
        items.append((sc, s, cam, p))
    try:
        want = [single(fmlib, s, cam, p) for sc, s, cam, p in items]
        views, outs = make_views(fmlib, items)
        b = fmlib.Batch(ctx, views)
        fmlib.set_proposal(ctx, None)
        pr.close()
        ctx.set_stats(True)
        try:
            b.run()
            ctx.sync()
            st = ctx.stats()
        finally:
            ctx.set_stats(False)
        for i in range(len(items)):
            assert_same(host(outs[i]), want[i], f"{which} view {i}")
        assert st["proposed"] > 0
        assert st["rays"] == b.info()["pixels"]
        b.close()
    finally:
        fmlib.set_proposal(ctx, None)
        pr.close()


def test_batch_learned_view_needs_a_proposal(fmlib, ctx, small_batch):
    sc, s, cam, params = small_batch[1]
    fmlib.set_proposal(ctx, None)
    o = device_outputs(cam)
    p = fmlib.MarchParams(params.iso, params.step, params.max_steps, 8, fmlib.FM_SKIP_EXACT, proposal=True)
    with pytest.raises(fmlib.FmError):
        fmlib.Batch(ctx, [fmlib.View(s, cam, p, **o)])
    pr = fmlib.Proposal(ctx, np.zeros(fmlib.FM_PROPOSAL_PARAMS, np.float32))
    fmlib.set_proposal(ctx, pr)
    try:
        bad = fmlib.MarchParams(params.iso, params.step, params.max_steps, 8, fmlib.FM_SKIP_REFERENCE, proposal=True)
        with pytest.raises(fmlib.FmError):
            fmlib.Batch(ctx, [fmlib.View(s, cam, bad, **o)])
        aniso = fmlib.MarchParams(params.iso, params.step, params.max_steps, 8, fmlib.FM_SKIP_EXACT, anisotropic=True,
                                  proposal=True)
        with pytest.raises(fmlib.FmError):
            fmlib.Batch(ctx, [fmlib.View(s, cam, aniso, **o)])
    finally:
        fmlib.set_proposal(ctx, None)
        pr.close()


def test_batch_with_anisotropic_views(fmlib, ctx, small_batch):
    """Anisotropic views (skip off and the reference's flags) next to isotropic ones in one batch
    equal the same views marched alone; the batch keeps the kernel settings it was created with."""
    ctx.set_anisotropy(2.0, 0.5, 2.0, 2000.0, 1)
    items = []
    for i, (sc, s, cam, params) in enumerate(small_batch[:6]):
        aniso = i % 2 == 1
        skip = (fmlib.FM_SKIP_OFF, fmlib.FM_SKIP_REFERENCE, fmlib.FM_SKIP_EXACT)[i % 3] if aniso else params.skip_mode
        p = fmlib.MarchParams(params.iso, params.step, params.max_steps, params.bisect, skip, anisotropic=aniso)
        items.append((sc, s, cam, p))
    want = [single(fmlib, s, cam, p) for sc, s, cam, p in items]
    views, outs = make_views(fmlib, items)
    b = fmlib.Batch(ctx, views)
    ctx.set_anisotropy(1.5, 0.4, 3.0, 1000.0, 2)  # not seen by the batch
    try:
        ctx.set_stats(True)
        try:
            b.run()
            ctx.sync()
            st = ctx.stats()
        finally:
            ctx.set_stats(False)
        for i in range(len(items)):
            assert_same(host(outs[i]), want[i], f"view {i}")
        assert st["rays"] == b.info()["pixels"]
        for o in outs:
            for v in o.values():
                v.zero_()
        b.run()  # the captured graph
        ctx.sync()
        for i in range(len(items)):
            assert_same(host(outs[i]), want[i], f"graph view {i}")
    finally:
        ctx.set_anisotropy(2.0, 0.5, 2.0, 2000.0, 1)
        b.close()
