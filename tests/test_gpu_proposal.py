"""The learned hit-interval proposal: tensor-core MLP, trainer, interval march, judge.

* The BF16 tcgen05 MLP equals a numpy evaluation of the same network with the
  same BF16 roundings (FP32 accumulation order aside).
* The trainer's forward / backward / Adam kernels agree with torch autograd.
* The learned march (FM_MARCH_PROPOSAL) is bit-identical to the oracle's
  interval march (fm_oracle.cpp) given the same intervals, and never changes a
  hit mask against the plain march.
"""

import math

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NF, NH = 32, 64
oW1, oB1 = 0, 64 * 32
oW2 = oB1 + 64
oB2 = oW2 + 64 * 64
oW3 = oB2 + 64
oB3 = oW3 + 2 * 64
NP = oB3 + 2


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def bf16(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def gelu(x):
    x = np.asarray(x, np.float64)
    return 0.5 * x * (1.0 + np.vectorize(math.erf)(x / math.sqrt(2.0)))


def unpack(P):
    P = np.asarray(P, np.float64)
    return (P[oW1:oB1].reshape(64, 32), P[oB1:oW2], P[oW2:oB2].reshape(64, 64), P[oB2:oW3],
            P[oW3:oB3].reshape(2, 64), P[oB3:oB3 + 2])


def mlp(P, X, bf=False):
    W1, b1, W2, b2, W3, b3 = unpack(P)
    r = (lambda a: bf16(a).astype(np.float64)) if bf else (lambda a: np.asarray(a, np.float64))
    h1 = r(gelu(r(X) @ r(W1).T + b1))
    h2 = r(gelu(h1 @ r(W2).T + b2))
    return h2 @ r(W3).T + b3


@pytest.fixture(scope="module")
def scene_setup(fmlib, ctx):
    sc = scenes.small_scene(seed=91, n=9000, width=128, height=96, max_steps=200)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    npx = cam.width * cam.height
    z = torch.zeros(npx, dtype=torch.float32, device="cuda")
    fmlib.splat_depth(s, cam, out=z)
    ctx.sync()
    return sc, cam, s, z


def random_params(seed, bias_scale=0.5):
    rng = np.random.default_rng(seed)
    P = np.zeros(NP, np.float32)
    P[oW1:oB1] = rng.uniform(-1, 1, 2048) * math.sqrt(6 / 32)
    P[oW2:oB2] = rng.uniform(-1, 1, 4096) * math.sqrt(6 / 64)
    P[oW3:oB3] = rng.uniform(-1, 1, 128) * math.sqrt(6 / 64)
    P[oB1:oW2] = rng.normal(0, bias_scale, 64)
    P[oB2:oW3] = rng.normal(0, bias_scale, 64)
    P[oB3:] = (1.0, 3.0)
    return P


def features(fmlib, s, cam, z):
    npx = cam.width * cam.height
    f = torch.zeros((npx, NF), dtype=torch.float32, device="cuda")
    t0 = torch.zeros(npx, dtype=torch.float32, device="cuda")
    fmlib.proposal_features(s, cam, z, f, t0)
    return f, t0


def intervals(fmlib, ctx, s, cam, sc, z, P, bisect=8, skip=1):
    prop = fmlib.Proposal(ctx, P)
    fmlib.set_proposal(ctx, prop)
    npx = cam.width * cam.height
    iv = torch.zeros((npx, 2), dtype=torch.int32, device="cuda")
    nf = torch.zeros((npx, 2), dtype=torch.float32, device="cuda")
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, bisect, skip, proposal=True)
    fmlib.proposal_intervals(s, cam, p, z, iv, nf)
    ctx.sync()
    return prop, iv.cpu().numpy(), nf.cpu().numpy()


def test_features_are_sane(fmlib, ctx, scene_setup):
    sc, cam, s, z = scene_setup
    f, t0 = features(fmlib, s, cam, z)
    ctx.sync()
    f = f.cpu().numpy()
    ray = z.cpu().numpy() < 1
    assert ray.sum() > 500
    assert np.all(np.isfinite(f))
    assert np.all(f[~ray] == 0)
    occ = f[ray, :16]
    assert occ.min() >= 0
    assert (occ.max(axis=1) > 0).mean() > 0.9  # rays start at a particle: density along them
    # the occupancy is the density over W(0) at the voxel centres, sampled
    # trilinearly: check the 16 samples of a few rays against the oracle's density
    g = s.grid()
    fr = O.build_frame(sc.xyz, sc.support)
    vox = (g["max"].astype(np.float64) - g["min"]) / 64
    sig = 8.0 / (math.pi * np.float64(np.float32(sc.support)) ** 3)
    cam_pos = np.asarray(cam.position, np.float64)
    t0h = t0.cpu().numpy()
    rows = np.nonzero(ray)[0][:: max(1, int(ray.sum()) // 6)][:6]
    for i in rows:
        d = f[i, 17:20].astype(np.float64)
        p0 = cam_pos + d * t0h[i]
        for j in range(16):
            q = p0 + d * sc.support * (0.25 + 0.5 * j)
            u = (q - g["min"]) / vox - 0.5
            b = np.floor(u).astype(int)
            w = u - b
            val = 0.0
            for c in range(8):
                o = np.array([c & 1, (c >> 1) & 1, c >> 2])
                v = b + o
                if np.any(v < 0) or np.any(v >= 64):
                    continue
                cen = (g["min"] + (v + 0.5) * vox).astype(np.float32)[None]
                wt = np.prod(np.where(o == 1, w, 1 - w))
                val += wt * float(O.density(fr, cen)[0]) / sig
            assert f[i, j] == pytest.approx(val, rel=5e-3, abs=0.05), (i, j)
    d = f[ray, 17:20]
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
    assert f[ray, 16].max() <= 0 and f[ray, 16].min() >= -4.0
    assert np.all((f[ray, 20:23] > -0.01) & (f[ray, 20:23] < 1.01))
    assert np.all(f[:, 23:] == 0)
    assert np.all(t0.cpu().numpy()[ray] > 0)


def test_tensor_core_mlp_matches_bf16_reference(fmlib, ctx, scene_setup):
    sc, cam, s, z = scene_setup
    P = random_params(7)
    f, _ = features(fmlib, s, cam, z)
    prop, iv, nf = intervals(fmlib, ctx, s, cam, sc, z, P)
    ray = z.cpu().numpy() < 1
    X = f.cpu().numpy()[ray]
    ref = mlp(P, X, bf=True)
    got = nf[ray]
    err = np.abs(got - ref) / (1.0 + np.abs(ref))
    assert np.median(err) < 1e-3, np.median(err)
    assert err.max() < 3e-2, err.max()
    # against the unrounded FP32 network: BF16 operands, FP32 accumulation
    ref32 = mlp(P, X, bf=False)
    assert np.median(np.abs(got - ref32) / (1.0 + np.abs(ref32))) < 2e-2
    # pixels without a ray get the full march
    assert np.all(iv[~ray] == [0, -1])
    fmlib.set_proposal(ctx, None)
    prop.close()


@pytest.mark.parametrize("which", ["constant", "random"])
def test_learned_march_matches_oracle(fmlib, ctx, scene_setup, which):
    sc, cam, s, z = scene_setup
    if which == "constant":
        P = np.zeros(NP, np.float32)
        P[oB3:] = (0.6, 3.0)  # every ray: samples ks+1 .. kf with ks = floor(0.6 H / step)
    else:
        P = random_params(11, bias_scale=1.0)
    prop, iv, _ = intervals(fmlib, ctx, s, cam, sc, z, P)
    ray = z.cpu().numpy() < 1
    used = (iv[:, 1] > 0) & ray
    assert used.sum() > 200
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1, proposal=True)
    npx = cam.width * cam.height
    g = {"position": np.zeros((npx, 4), np.float32), "normal": np.zeros((npx, 4), np.float32),
         "depth": np.zeros(npx, np.float32), "colour": np.zeros((npx, 4), np.float32)}
    ctx.set_stats(True)
    try:
        fmlib.march(s, cam, p, g["position"], g["normal"], g["depth"], g["colour"])
        st = ctx.stats()
    finally:
        ctx.set_stats(False)
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, depth, intervals=iv)
    for k in ("position", "normal", "depth", "colour"):
        bad = np.nonzero(np.any((bits(g[k]) != bits(o[k])).reshape(npx, -1), axis=1))[0]
        assert bad.size == 0, f"{k}: {bad.size} pixels differ, first {bad[:5]}"
    plain = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, depth)
    assert np.array_equal(g["depth"] > 0, plain["depth"] > 0)
    assert st["proposed"] == int(used.sum())
    assert 0 < st["fallbacks"] <= st["proposed"]
    fmlib.set_proposal(ctx, None)
    prop.close()


def test_learned_march_needs_a_proposal(fmlib, ctx, scene_setup):
    sc, cam, s, z = scene_setup
    fmlib.set_proposal(ctx, None)
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1, proposal=True)
    with pytest.raises(fmlib.FmError):
        fmlib.render(s, cam, p)
    bad = np.zeros(NP, np.float32)
    bad[5] = np.nan
    with pytest.raises(fmlib.FmError):
        fmlib.Proposal(ctx, bad)


def test_trainer_matches_torch(fmlib, ctx):
    rng = np.random.default_rng(2)
    n = 777
    X = rng.normal(0, 1, (n, NF)).astype(np.float32)
    X[:, 23:] = 0
    T = (2.0 + X[:, 0] - 0.5 * X[:, 3] + 0.2 * rng.normal(0, 1, n)).astype(np.float32)
    P0 = random_params(5, bias_scale=0.2)
    tr = fmlib.Trainer(ctx, init=P0)
    Xd = torch.from_numpy(X).cuda()
    Td = torch.from_numpy(T).cuda()
    out = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    tr.predict(Xd, n, out)
    ctx.sync()
    assert np.allclose(out.cpu().numpy(), mlp(P0, X), rtol=1e-4, atol=1e-4)
    # torch autograd of the same loss
    tl, th = 0.05, 0.95
    Pt = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
    W1 = Pt[oW1:oB1].view(64, 32)
    W2 = Pt[oW2:oB2].view(64, 64)
    W3 = Pt[oW3:oB3].view(2, 64)
    x = torch.tensor(X, dtype=torch.float64)
    t = torch.tensor(T, dtype=torch.float64)
    g = torch.nn.functional.gelu
    y = g(g(x @ W1.T + Pt[oB1:oW2]) @ W2.T + Pt[oB2:oW3]) @ W3.T + Pt[oB3:]
    e0, e1 = t - y[:, 0], t - y[:, 1]
    loss = (torch.maximum(tl * e0, (tl - 1) * e0) + torch.maximum(th * e1, (th - 1) * e1)).mean()
    loss.backward()
    grad = Pt.grad.numpy()
    lr = 1e-3
    got_loss = tr.step(Xd, Td, n, lr, tl, th, want_loss=True)
    assert got_loss == pytest.approx(float(loss.detach()), rel=1e-4)
    P1 = tr.params()
    # first Adam step: delta = -lr * g / (|g| + eps)
    sig = np.abs(grad) > 1e-4
    assert sig.sum() > 1000
    delta = (P1 - P0)[sig]
    assert np.allclose(delta, -lr * np.sign(grad[sig]), rtol=1e-2, atol=1e-6)
    tr.close()


def test_trainer_checkpoint_resumes_exactly(fmlib, ctx, tmp_path):
    """Steps 1-6 in one go equal steps 1-3, a checkpoint, a fresh trainer from it, steps 4-6 (bits)."""
    from fluidmarch import proposal as PR

    rng = np.random.default_rng(9)
    n = 3000
    X = torch.from_numpy(rng.normal(0, 1, (6, n, NF)).astype(np.float32)).cuda()
    T = torch.from_numpy(rng.uniform(0, 10, (6, n)).astype(np.float32)).cuda()
    P0 = random_params(4)
    a = fmlib.Trainer(ctx, init=P0)
    for k in range(6):
        a.step(X[k], T[k], n, 3e-3, 0.05, 0.97)
    want, want_step = a.state()
    b = fmlib.Trainer(ctx, init=P0)
    for k in range(3):
        b.step(X[k], T[k], n, 3e-3, 0.05, 0.97)
    path = str(tmp_path / "trainer.ckpt")
    PR.save_checkpoint(path, b, {"epoch": 0, "batch": 3})
    b.close()
    c, head = PR.load_checkpoint(path, ctx)
    assert head["step"] == 3 and head["meta"]["batch"] == 3
    for k in range(3, 6):
        c.step(X[k], T[k], n, 3e-3, 0.05, 0.97)
    got, got_step = c.state()
    assert got_step == want_step == 6
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the same six steps again give the same bits (the gradient reduction has a fixed order)
    d = fmlib.Trainer(ctx, init=P0)
    for k in range(6):
        d.step(X[k], T[k], n, 3e-3, 0.05, 0.97)
    assert np.array_equal(d.state()[0].view(np.uint32), want.view(np.uint32))
    bad = want.copy()
    bad[2 * fmlib.FM_PROPOSAL_PARAMS] = -1.0  # a negative second moment
    with pytest.raises(fmlib.FmError):
        c.set_state(bad, 6)
    with open(path, "r+b") as f:
        f.write(b"XXXX")
    with pytest.raises(ValueError):
        PR.load_checkpoint(path, ctx)
    for t in (a, c, d):
        t.close()


def test_trainer_learns(fmlib, ctx):
    rng = np.random.default_rng(8)
    n = 16384
    X = rng.normal(0, 1, (n, NF)).astype(np.float32)
    X[:, 23:] = 0
    T = (3.0 + np.tanh(X[:, 0]) - 0.5 * X[:, 5]).astype(np.float32)
    tr = fmlib.Trainer(ctx, seed=1)
    Xd = torch.from_numpy(X).cuda()
    Td = torch.from_numpy(T).cuda()
    first = tr.step(Xd, Td, n, 3e-3, 0.5, 0.5, want_loss=True)
    for _ in range(400):
        last = tr.step(Xd, Td, n, 3e-3, 0.5, 0.5, want_loss=False)
    last = tr.step(Xd, Td, n, 1e-3, 0.5, 0.5, want_loss=True)
    assert last < 0.2 * first, (first, last)
    tr.close()


def test_judge(fmlib, ctx):
    rng = np.random.default_rng(3)
    n = 100_003
    a = np.where(rng.random(n) < 0.6, rng.uniform(1, 3, n), 0).astype(np.float32)
    b = a.copy()
    k = rng.choice(np.nonzero(a > 0)[0], 500, replace=False)
    b[k[:300]] += rng.uniform(0, 2e-4, 300).astype(np.float32)
    b[k[300:]] = 0
    m = rng.choice(np.nonzero(a == 0)[0], 77, replace=False)
    b[m] = 2.0
    r = fmlib.judge(ctx, torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), 1e-4)
    both = (a > 0) & (b > 0)
    err = np.abs(b - a)
    assert r["hits_ref"] == int((a > 0).sum()) and r["hits_test"] == int((b > 0).sum())
    assert r["mask_mismatch"] == 277
    assert r["within_tol"] == int((both & (err <= np.float32(1e-4))).sum())
    assert r["max_err"] == pytest.approx(float(err[both].max()), rel=1e-6)


def _judge_sample(width, height, seq, stride):
    """The per-frame judge's sample of frame `seq`: pixels of the 8x4 blocks whose index, hashed with
    lowbias32 after an xor with the frame's seed, is 0 modulo the stride."""
    py, px = np.divmod(np.arange(width * height, dtype=np.uint64), np.uint64(width))
    blk = (py >> np.uint64(2)) * np.uint64((width + 7) // 8) + (px >> np.uint64(3))
    x = ((blk ^ np.uint64((seq * 0x9E3779B9) & 0xFFFFFFFF)) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    with np.errstate(over="ignore"):
        x ^= x >> np.uint32(16)
        x *= np.uint32(0x7FEB352D)
        x ^= x >> np.uint32(15)
        x *= np.uint32(0x846CA68B)
        x ^= x >> np.uint32(16)
    return x % np.uint32(stride) == 0


def test_per_frame_judge(fmlib, scene_setup):
    """fm_set_judge: every learned march also marches a changing sample of 8x4 pixel blocks plainly and compares the
    hit distances on the device; the accumulated counts equal a host count over the same samples."""
    sc, cam, _, _ = scene_setup
    ctx = fmlib.Context(0)
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    prop = fmlib.Proposal(ctx, random_params(12, bias_scale=1.0))
    fmlib.set_proposal(ctx, prop)
    stride, frames = 4, 3
    tol = 1e-4 * float(np.max(sc.xyz.max(0) - sc.xyz.min(0)))
    ctx.set_judge(stride, tol)
    plain = fmlib.render(s, cam, fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1))
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1, proposal=True)
    outs = [fmlib.render(s, cam, p) for _ in range(frames)]
    j = ctx.judge_frames(reset=True)
    npx = cam.width * cam.height
    ref = plain["depth"]
    started = plain["start_depth"] < 1
    want = dict(frames=frames, sampled=0, hits_ref=0, hits_test=0, mask_mismatch=0, within_tol=0)
    max_err = 0.0
    for k, o in enumerate(outs):
        m = _judge_sample(cam.width, cam.height, k, stride) & started
        hr, ht = ref[m] > 0, o["depth"][m] > 0
        both = hr & ht
        err = np.abs(o["depth"][m][both] - ref[m][both])
        want["sampled"] += int(m.sum())
        want["hits_ref"] += int(hr.sum())
        want["hits_test"] += int(ht.sum())
        want["mask_mismatch"] += int((hr != ht).sum())
        want["within_tol"] += int((err <= np.float32(tol)).sum())
        max_err = max(max_err, float(err.max()) if err.size else 0.0)
    assert {k: j[k] for k in want} == want
    assert j["max_err"] == pytest.approx(max_err, abs=0.0)
    assert want["sampled"] > 3 * 0.1 * started.sum() and want["hits_ref"] > 100
    assert ctx.judge_frames()["frames"] == 0  # reset
    ctx.set_judge(0, 0.0)
    fmlib.render(s, cam, p)
    assert ctx.judge_frames()["frames"] == 0  # off
    with pytest.raises(fmlib.FmError):
        ctx.set_judge(4, float("nan"))
    fmlib.set_proposal(ctx, None)
    prop.close()
    s.close()
    ctx.close()
