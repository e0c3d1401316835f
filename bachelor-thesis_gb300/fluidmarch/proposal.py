"""Training data, training and evaluation of the learned hit-interval proposal.

The proposal is trained only on first-hit distances that the plain GPU march
produces: seeded scenes of the sloshing family are generated on the GPU,
rendered at 1920x1080 from seeded orbit cameras with the plain march, and the
hit pixels give (features, distance) pairs:

    target = (hit distance - ray-start distance) / support radius

The MLP (3 layers, width 64, GELU) is trained with the library's FP32 kernels
(``fm_trainer_*``: forward, backward, Adam) on a pinball loss: ``near`` at a low
quantile, ``far`` at a high one.  A held-out split of scenes measures how often
the first hit lies inside the interval and how wide the interval is.

    python -m fluidmarch.proposal --train 2000 --heldout 200 --out proposal_sloshing.npz
"""

from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

import fluidmarch as fm
from fluidmarch import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "proposal_sloshing.npz")
TRAIN_SEED0, HELDOUT_SEED0 = 100_000, 200_000


def _torch():
    import torch

    return torch


def sloshing_xyz_gpu(seed: int, n: int = 1_000_000):
    """Sloshing-family particles generated on the GPU (torch RNG, training data only).

    Same layout as ``scenes.sloshing``: 95% below y = 0.4 + 0.08 sin(2 pi x)
    cos(3 pi z) + N(0, 0.005) in the unit column, 5% spray above it up to 0.9.
    """
    torch = _torch()
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    n_fluid = int(round(0.95 * n))
    parts, got = [], 0
    lo = torch.tensor([1.0, 0.5, 1.0], device="cuda")
    while got < n_fluid:
        m = max(1024, int((n_fluid - got) * 1.35))
        p = torch.rand((m, 3), generator=g, device="cuda", dtype=torch.float64) * lo
        top = 0.4 + 0.08 * torch.sin(2 * math.pi * p[:, 0]) * torch.cos(3 * math.pi * p[:, 2])
        top = top + 0.005 * torch.randn(m, generator=g, device="cuda", dtype=torch.float64)
        p = p[p[:, 1] < top][: n_fluid - got]
        parts.append(p)
        got += p.shape[0]
    hi = torch.tensor([1.0, 0.9, 1.0], device="cuda")
    n_spray, got = n - n_fluid, 0
    while got < n_spray:
        m = max(1024, int((n_spray - got) * 2.2))
        p = torch.rand((m, 3), generator=g, device="cuda", dtype=torch.float64) * hi
        top = 0.4 + 0.08 * torch.sin(2 * math.pi * p[:, 0]) * torch.cos(3 * math.pi * p[:, 2])
        p = p[p[:, 1] > top][: n_spray - got]
        parts.append(p)
        got += p.shape[0]
    return torch.cat(parts).to(torch.float32).contiguous()


def orbit_camera(rng: np.random.Generator, width: int = 1920, height: int = 1080):
    ang = rng.uniform(0, 2 * math.pi)
    rad = rng.uniform(1.5, 2.1)
    eye = (0.5 + rad * math.cos(ang), rng.uniform(0.8, 1.6), 0.5 + rad * math.sin(ang))
    tgt = (0.5 + rng.uniform(-0.1, 0.1), 0.3 + rng.uniform(-0.05, 0.05), 0.5 + rng.uniform(-0.1, 0.1))
    return scenes.make_camera(eye, tgt, width, height)


def family_settings(n: int = 1_000_000):
    """Support radius, iso density, step, max steps of the sloshing family at n particles."""
    h = 0.02 * (1_000_000 / n) ** (1.0 / 3.0)
    H = 2 * h
    spacing = (0.4 / (0.95 * n)) ** (1.0 / 3.0)
    rho0 = scenes.lattice_rest_density(spacing, H)
    return float(np.float32(H)), float(np.float32(0.5 * rho0)), float(np.float32(0.25 * h)), 1024


def collect(ctx: fm.Context, seeds, per_scene: int = 4096, n: int = 1_000_000, width: int = 1920,
            height: int = 1080, log=None):
    """(features, targets) of up to per_scene hit rays of each seeded scene, on the device."""
    torch = _torch()
    H, iso, step, max_steps = family_settings(n)
    npx = width * height
    dev = dict(device="cuda", dtype=torch.float32)
    depth = torch.zeros(npx, **dev)
    z = torch.zeros(npx, **dev)
    feat = torch.zeros((npx, fm.FM_PROPOSAL_FEATURES), **dev)
    t0 = torch.zeros(npx, **dev)
    params = fm.MarchParams(iso, step, max_steps, 8, fm.FM_SKIP_EXACT)
    X, T = [], []
    scene = None
    t_start = time.time()
    for k, seed in enumerate(seeds):
        xyz = sloshing_xyz_gpu(seed, n)
        torch.cuda.synchronize()
        if scene is None:
            scene = fm.Scene(ctx, xyz, H)
        else:
            scene.update(xyz)
        cam = orbit_camera(np.random.default_rng(seed), width, height)
        fm.march(scene, cam, params, depth=depth, start_depth=z)
        fm.proposal_features(scene, cam, z, feat, t0)
        ctx.sync()
        hit = torch.nonzero((depth > 0) & (z < 1)).flatten()
        if hit.numel() == 0:
            continue
        g = torch.Generator(device="cuda")
        g.manual_seed(int(seed))
        pick = hit[torch.randperm(hit.numel(), generator=g, device="cuda")[:per_scene]]
        X.append(feat[pick].clone())
        T.append(((depth[pick] - t0[pick]) / H).clone())
        if log and (k + 1) % 100 == 0:
            log(f"collected {k + 1}/{len(seeds)} scenes, {sum(x.shape[0] for x in X)} rays, "
                f"{time.time() - t_start:.1f} s")
    if scene is not None:
        scene.close()
    return torch.cat(X), torch.cat(T)


def train(ctx: fm.Context, X, T, epochs: int = 12, batch: int = 8192, lr: float = 2e-3, tau_lo: float = 0.05,
          tau_hi: float = 0.97, seed: int = 0, log=None, init=None) -> np.ndarray:
    """Adam on the pinball loss with a cosine learning-rate decay; returns the FP32 parameters.

    init: parameters to start from (fine-tuning), else a seeded initialisation.
    """
    torch = _torch()
    n = X.shape[0]
    tr = fm.Trainer(ctx, seed=seed, init=init)
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    steps_per_epoch = max(1, n // batch)
    total = epochs * steps_per_epoch
    it = 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g, device="cuda")
        Xs, Ts = X[perm].contiguous(), T[perm].contiguous()
        losses = []
        for b in range(steps_per_epoch):
            lr_t = 1e-5 + 0.5 * (lr - 1e-5) * (1 + math.cos(math.pi * it / total))
            xb = Xs[b * batch:(b + 1) * batch]
            tb = Ts[b * batch:(b + 1) * batch]
            want = b == steps_per_epoch - 1
            l = tr.step(xb, tb, xb.shape[0], lr_t, tau_lo, tau_hi, want_loss=want)
            if want:
                losses.append(l)
            it += 1
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {losses[-1]:.4f}")
    P = tr.params()
    tr.close()
    return P


def evaluate(ctx: fm.Context, P: np.ndarray, X, T, H: float = None, step: float = None) -> dict:
    """Coverage and width of the FP32 network's intervals on (X, T)."""
    torch = _torch()
    n = X.shape[0]
    tr = fm.Trainer(ctx, init=P)
    out = torch.zeros((n, 2), device="cuda", dtype=torch.float32)
    tr.predict(X, n, out)
    ctx.sync()
    tr.close()
    near, far = out[:, 0], out[:, 1]
    r = {
        "rays": int(n),
        "near_below_hit": float(((near <= T)).float().mean()),
        "far_above_hit": float(((far >= T)).float().mean()),
        "covered": float(((near <= T) & (far >= T)).float().mean()),
        "mean_width_support_radii": float((far - near).clamp(min=0).mean()),
        "mean_hit_distance_support_radii": float(T.mean()),
        "mean_near_support_radii": float(near.clamp(min=0).mean()),
    }
    return r


CKPT_MAGIC = b"FMTRAIN\0"
CKPT_VERSION = 1


def save_checkpoint(path: str, trainer: fm.Trainer, meta: dict | None = None) -> None:
    """Trainer checkpoint: magic, version (uint32), JSON header length (uint32), the JSON header
    (layout, Adam step, caller metadata), then the state as little-endian float32 (parameters,
    Adam first moments, second moments: 3 x FM_PROPOSAL_PARAMS).  Written to a temporary file
    and renamed, so a crash never leaves a torn checkpoint."""
    state, step = trainer.state()
    head = json.dumps({"version": CKPT_VERSION, "params": fm.FM_PROPOSAL_PARAMS, "step": step,
                       "layout": ["parameters", "adam_m", "adam_v"], "dtype": "<f4",
                       "meta": meta or {}}).encode()
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(CKPT_MAGIC)
        f.write(np.array([CKPT_VERSION, len(head)], "<u4").tobytes())
        f.write(head)
        f.write(state.astype("<f4").tobytes())
    os.replace(tmp, path)


def load_checkpoint(path: str, ctx: fm.Context) -> tuple:
    """(trainer restored from the checkpoint, its JSON header)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != CKPT_MAGIC:
        raise ValueError(f"{path}: not a trainer checkpoint")
    version, hlen = np.frombuffer(data[8:16], "<u4")
    if version != CKPT_VERSION:
        raise ValueError(f"{path}: checkpoint version {version}, expected {CKPT_VERSION}")
    head = json.loads(data[16:16 + hlen].decode())
    if head["params"] != fm.FM_PROPOSAL_PARAMS:
        raise ValueError(f"{path}: {head['params']} parameters, expected {fm.FM_PROPOSAL_PARAMS}")
    state = np.frombuffer(data[16 + hlen:], "<f4")
    if state.size != 3 * fm.FM_PROPOSAL_PARAMS:
        raise ValueError(f"{path}: truncated state")
    tr = fm.Trainer(ctx, init=state[: fm.FM_PROPOSAL_PARAMS])
    tr.set_state(state, head["step"])
    return tr, head


def load(path: str = WEIGHTS):
    d = np.load(path, allow_pickle=False)
    meta = json.loads(str(d["meta"])) if "meta" in d else {}
    return d["params"].astype(np.float32), meta


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--train", type=int, default=2000, help="training scenes")
    ap.add_argument("--heldout", type=int, default=200, help="held-out scenes")
    ap.add_argument("--per-scene", type=int, default=4096)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--tau-lo", type=float, default=0.05)
    ap.add_argument("--tau-hi", type=float, default=0.97)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)  # noqa: E731
    ctx = fm.Context(0)
    t = time.time()
    Xtr, Ttr = collect(ctx, range(TRAIN_SEED0, TRAIN_SEED0 + args.train), args.per_scene, log=log)
    Xte, Tte = collect(ctx, range(HELDOUT_SEED0, HELDOUT_SEED0 + args.heldout), args.per_scene, log=log)
    t_collect = time.time() - t
    log(f"data: {Xtr.shape[0]} training rays, {Xte.shape[0]} held-out rays ({t_collect:.1f} s)")
    t = time.time()
    P = train(ctx, Xtr, Ttr, epochs=args.epochs, tau_lo=args.tau_lo, tau_hi=args.tau_hi, log=log)
    t_train = time.time() - t
    ev_tr = evaluate(ctx, P, Xtr, Ttr)
    ev_te = evaluate(ctx, P, Xte, Tte)
    meta = {"train_scenes": args.train, "heldout_scenes": args.heldout, "per_scene": args.per_scene,
            "epochs": args.epochs, "tau_lo": args.tau_lo, "tau_hi": args.tau_hi, "train_seed0": TRAIN_SEED0,
            "heldout_seed0": HELDOUT_SEED0, "collect_s": t_collect, "train_s": t_train, "train": ev_tr,
            "heldout": ev_te}
    log(json.dumps(meta))
    np.savez(args.out, params=P, meta=json.dumps(meta))
    ctx.close()


if __name__ == "__main__":
    main()
