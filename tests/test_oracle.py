"""The CPU oracle, pinned against known answers, the reference's own code and
the golden vectors the reference wrote (tests/golden).  No GPU needed."""

import glob
import math
import os

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def sigma(H):
    return 8.0 / (math.pi * H ** 3)


@pytest.fixture(scope="module")
def L(oracle_lib):
    return oracle_lib.lib()


# ---- kernel known answers (Kernel.cpp:9-52) --------------------------------

def test_w_known_answers(L):
    H = 0.1
    s = np.float32(8.0) / (np.float32(np.pi) * np.float32(H) * np.float32(H) * np.float32(H))
    assert L.orc_sigma(H) == pytest.approx(sigma(H), rel=1e-6)
    assert L.orc_W(H, 0, 0, 0) == pytest.approx(float(s), rel=1e-7)          # W(0) = sigma (Kernel.h W0)
    assert L.orc_W(H, 0.01, 0, 0) == pytest.approx(2408.97, rel=2e-6)       # closed form at q = 0.1
    # continuity at q = 0.5: both branches give sigma / 4
    lo = L.orc_W(H, 0.5 * H * (1 - 1e-6), 0, 0)
    hi = L.orc_W(H, 0.5 * H, 0, 0)
    assert lo == pytest.approx(sigma(H) / 4, rel=1e-4)
    assert hi == pytest.approx(sigma(H) / 4, rel=1e-4)
    assert L.orc_W(H, H, 0, 0) == 0.0
    assert L.orc_W(H, 0, 0, 0.2) == 0.0


def test_gradw_reference_formula(L):
    """gradQ = normalize(r) / (|r| H): the reference's extra 1/|r| factor is kept."""
    H = 0.1
    g = np.zeros(3, np.float32)
    L.orc_gradW(H, 0.03, 0, 0, g)
    q = 0.3
    expect = sigma(H) * (1.0 / (0.03 * H)) * 6.0 * (3 * q * q - 2 * q)
    assert g[0] == pytest.approx(expect, rel=1e-5)
    assert g[1] == 0 and g[2] == 0
    L.orc_gradW(H, 0, 0, -0.07, g)
    q = 0.7
    expect = -sigma(H) * (-1.0 / (0.07 * H)) * 6.0 * (1 - q) ** 2
    assert g[2] == pytest.approx(expect, rel=1e-5)
    L.orc_gradW(H, 0, 0, 0, g)  # r = 0 guarded (the reference would return NaN)
    assert np.all(g == 0)


def test_cos_poly_accuracy(L):
    t = np.linspace(0, math.pi / 2, 2001, dtype=np.float32)
    got = np.array([L.orc_cos_poly(float(x)) for x in t])
    assert np.max(np.abs(got - np.cos(t.astype(np.float64)))) < 3e-7


# ---- oracle vs the reference's compiled translation units ------------------

needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference tree absent: oracle/_ref not built")


@needs_ref
def test_kernel_bitwise_vs_reference(L):
    R = O.ref()
    rng = np.random.default_rng(3)
    g1 = np.zeros(3, np.float32)
    g2 = np.zeros(3, np.float32)
    for H in (0.1, 0.04, 0.0252):
        r = rng.uniform(-1.1 * H, 1.1 * H, size=(500, 3)).astype(np.float32)
        for x, y, z in r:
            assert np.float32(L.orc_W(H, x, y, z)).view(np.uint32) == np.float32(R.ref_W(H, x, y, z)).view(np.uint32)
            L.orc_gradW(H, x, y, z, g1)
            R.ref_gradW(H, x, y, z, g2)
            assert np.array_equal(g1.view(np.uint32), g2.view(np.uint32))


@needs_ref
def test_cells_match_query_density_grid():
    """Per-particle cell = Frame::QueryDensityGrid index (Dataset.cpp:26-47), bit-exact."""
    sc = scenes.small_scene(seed=5, n=5000)
    fr = O.build_frame(sc.xyz, sc.support)
    # query with the sorted particles (the reference's frame stores them z-sorted)
    q = np.ascontiguousarray(fr.sorted[:, :3])
    out = np.empty(q.shape[0], np.int64)
    O.ref().ref_query_cells(np.ascontiguousarray(sc.xyz), sc.n, sc.support, q, q.shape[0], out)
    assert np.array_equal(out.astype(np.uint32), fr.cells[fr.perm])


@needs_ref
@pytest.mark.parametrize("box_mode", [0, 1])
@pytest.mark.parametrize("which", ["dam", "slosh"])
def test_march_bitwise_vs_reference(which, box_mode):
    if which == "dam":
        sc = scenes.dam_break(width=96, height=72)
    else:
        sc = scenes.small_scene(seed=9, n=6000, width=96, height=72)
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    a = O.ref_march(sc.xyz, sc.support, cam, depth, sc.max_steps, sc.step, sc.iso, box_mode=box_mode)
    b = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, skip_mode=2 if box_mode else 0, threads=4)
    assert np.array_equal(a["sorted"], fr.sorted[:, :3])
    last = cam.width * cam.height - 1  # the reference never marches pixel W*H-1 (ThreadPool.cpp:50)
    for k in ("position", "normal"):
        x = b[k].copy()
        x[last] = 0
        assert np.array_equal(a[k].view(np.uint32), x.view(np.uint32)), k
    assert (a["position"][:, 3] == 1).sum() > 100


@needs_ref
def test_neighbour_clamp_is_where_reference_and_restatement_part():
    """The reference keeps at most MAX_NEIGHBORS = 8192 neighbours per sample (RayMarcher.cpp:14,312);
    the restatement (and the GPU march) sums every particle within the support radius.  A cluster of
    particles much smaller than the support radius puts all of them in range of the samples near it:
    with 8192 particles the two agree bit for bit, with 9000 the reference sums only the first 8192 of
    its neighbour list and its hit points and normals differ."""
    H = 0.1
    cam = scenes.make_camera((0.0, 0.0, -1.0), (0.0, 0.0, 0.0), 17, 17)
    rng = np.random.default_rng(11)
    w06 = 2.0 * sigma(H) * (1.0 - 0.6) ** 3  # W at q = 0.6
    results = {}
    for m in (8192, 9000):
        xyz = rng.uniform(-0.005, 0.005, (m, 3)).astype(np.float32)
        iso = float(np.float32(m * w06))  # crossing near 0.6 H from the cluster, every particle in range
        fr = O.build_frame(xyz, H)
        depth = O.splat(xyz, H, cam)
        a = O.ref_march(xyz, H, cam, depth, 200, 0.005, iso)
        b = O.march(fr, cam, iso, 0.005, 200, 0, depth, threads=2)
        last = cam.width * cam.height - 1
        same = True
        for k in ("position", "normal"):
            x = b[k].copy()
            x[last] = 0
            same &= np.array_equal(a[k].view(np.uint32), x.view(np.uint32))
        hits = int((b["position"][:, 3] == 1).sum())
        assert hits > 0
        results[m] = same
    assert results == {8192: True, 9000: False}


# ---- golden vectors written by the reference --------------------------------

class _Cam:
    def __init__(self, z):
        self.view, self.proj, self.inv_proj_view = z["view"], z["proj"], z["inv_proj_view"]
        self.position, self.width, self.height = z["cam_pos"], int(z["width"]), int(z["height"])


def load_golden(path):
    z = dict(np.load(path))
    return z, _Cam(z)


@pytest.mark.skipif(not GOLDEN, reason="no golden vectors")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_golden(path):
    z, cam = load_golden(path)
    fr = O.build_frame(z["xyz"], float(z["support"]))
    assert np.array_equal(fr.sorted[:, :3], z["ref_sorted"])
    depth = O.splat(z["xyz"], float(z["support"]), cam)
    assert np.array_equal(depth, z["start_depth"])
    skip = 2 if int(z["box_mode"]) == 1 else 0
    b = O.march(fr, cam, float(z["iso"]), float(z["step"]), int(z["max_steps"]), 0, z["start_depth"],
                skip_mode=skip, threads=2)
    last = cam.width * cam.height - 1
    for k in ("position", "normal"):
        x = b[k].copy()
        x[last] = 0
        assert np.array_equal(z["ref_" + k].view(np.uint32), x.view(np.uint32)), k


# ---- self-made known answers --------------------------------------------------

def test_lattice_rest_density():
    assert scenes.lattice_rest_density(0.025, 0.1) == pytest.approx(64005, rel=1e-4)
    assert scenes.lattice_rest_density((0.4 / 950000) ** (1 / 3), 0.04) == pytest.approx(2.376e6, rel=1e-3)


def test_oracle_density_matches_lattice_sum():
    s, H = 0.025, 0.1
    i = np.arange(-6, 7) * s
    x, y, z = np.meshgrid(i, i, i, indexing="ij")
    xyz = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32)
    fr = O.build_frame(xyz, H)
    d64 = O.density(fr, np.zeros((1, 3), np.float32), precision=64)[0]
    # positions are float32, so the sum differs from the exact lattice in the 8th digit
    assert d64 == pytest.approx(scenes.lattice_rest_density(s, H), rel=1e-6)


def test_single_particle_sphere_hit():
    """One particle: the iso surface of W is a sphere; the bisected hit lies on it."""
    H = 0.1
    xyz = np.array([[0.0, 0.0, 0.0]], np.float32)
    fr = O.build_frame(xyz, H)
    iso = np.float32(sigma(H) * 0.25)  # W = sigma/4 at q = 0.5
    cam = scenes.make_camera((0.0, 0.0, -1.0), (0.0, 0.0, 0.0), 129, 129)
    depth = O.splat(xyz, H, cam)
    out = O.march(fr, cam, float(iso), 0.002, 400, 12, depth, threads=1)
    hit = out["position"][:, 3] == 1
    # iso sphere radius 0.05 at distance 1 with a 60 degree view: about 5.6 pixels across
    assert hit.sum() > 40
    r = np.linalg.norm(out["position"][hit, :3], axis=1)
    assert np.allclose(r, 0.5 * H, atol=2e-6)
    centre = 64 * 129 + 64
    assert hit[centre]
    # the normal points away from the fluid (towards the camera at the centre pixel)
    n = out["normal"][centre, :3]
    assert n[2] < -0.99


def test_splat_single_particle_centre_depth():
    H = 0.1
    xyz = np.array([[0.0, 0.0, 0.0]], np.float32)
    cam = scenes.make_camera((0.0, 0.0, -1.0), (0.0, 0.0, 0.0), 31, 31)
    depth = O.splat(xyz, H, cam).reshape(31, 31)
    P = cam.proj.astype(np.float64)
    zv = 1.0 - H
    expect = (P[10] * zv + P[14]) / (P[11] * zv + P[15])
    assert depth[15, 15] == pytest.approx(expect, abs=1e-6)
    assert depth[0, 0] == 1.0


def test_fp64_twin_close_to_fp32():
    sc = scenes.small_scene(seed=4, n=4000, width=64, height=48)
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    # 12 bisections: the final interval (step / 4096) is well below the 1e-4 extent tolerance
    a = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 12, depth, threads=4, precision=32)
    b = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 12, depth, threads=4, precision=64)
    ha, hb = a["position"][:, 3] == 1, b["position"][:, 3] == 1
    assert (ha != hb).sum() <= 2
    both = ha & hb
    ext = float(np.max(sc.xyz.max(0) - sc.xyz.min(0)))
    assert np.quantile(np.abs(a["depth"][both] - b["depth"][both]), 0.999) < 1e-4 * ext


# ---- the learned march's interval semantics --------------------------------

def test_interval_march_semantics():
    """A proposed interval (ks, kf) never changes a hit mask; a hit only moves
    deeper, and only when the plain march crosses at or before sample ks."""
    sc = scenes.small_scene(seed=33, n=6000, width=96, height=72, max_steps=160)
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    npx = cam.width * cam.height
    plain = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth)
    rng = np.random.default_rng(4)
    ks = rng.integers(1, 12, npx).astype(np.int32)
    kf = (ks + rng.integers(1, 30, npx)).astype(np.int32)
    ivl = np.stack([ks, kf], axis=1)
    got = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, intervals=ivl)
    hit_p, hit_g = plain["depth"] > 0, got["depth"] > 0
    assert np.array_equal(hit_p, hit_g)
    # with bisection 0 and skipping off, a hit ray's evaluations = its hit sample number
    h = plain["evals"]
    later = hit_p & (h > ks)
    assert np.array_equal(got["position"][later], plain["position"][later])
    early = hit_p & (h <= ks)
    same = np.all(got["position"] == plain["position"], axis=1)
    moved = early & ~same
    assert np.all(got["depth"][moved] > plain["depth"][moved])
    assert later.sum() > 100 and early.sum() > 20
    # intervals that are not usable (ks < 1, kf <= ks, kf > max_steps) mean the full march
    bad = np.stack([np.zeros(npx, np.int32), np.full(npx, 5, np.int32)], axis=1)
    got0 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, intervals=bad)
    assert np.array_equal(got0["position"], plain["position"])


def _aniso_iso(fr, xyz, aniso=(2.0, 0.5, 2.0, 2000.0, 1)):
    inner = xyz[(xyz[:, 1] < 0.2) & (xyz[:, 0] > 0.3) & (xyz[:, 0] < 0.7) & (xyz[:, 2] > 0.3) & (xyz[:, 2] < 0.7)]
    return float(np.float32(0.5 * np.median(O.density_aniso(fr, inner[:200], aniso))))


@pytest.mark.skipif(not O.ref_available(), reason="reference build not available")
@pytest.mark.parametrize("n,w,h", [(3000, 48, 36), (12000, 64, 48)])
def test_aniso_march_vs_reference(n, w, h):
    """The anisotropic march restatement against the reference's own PerPixel_Anisotropic
    (RayMarcher.cpp:346-423 with Eigen's solver): same hits, same sample positions,
    normals within 0.5 degrees (the eigen-decompositions differ in the last bits)."""
    sc = scenes.small_scene(seed=5, n=n, width=w, height=h, max_steps=120)
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    iso = _aniso_iso(fr, sc.xyz)
    depth = O.splat(sc.xyz, sc.support, cam)
    b = O.march_aniso(fr, cam, iso, sc.step, sc.max_steps, 0, depth)
    r = O.ref_march(sc.xyz, sc.support, cam, depth, sc.max_steps, sc.step, iso, aniso=(2.0, 0.5, 2.0, 2000.0, 1))
    hb, ha = b["position"][:, 3] > 0, r["position"][:, 3] > 0
    ha[-1] = hb[-1]  # the reference never marches the last pixel (ThreadPool.cpp:50)
    assert np.array_equal(ha, hb) and ha.sum() > 200
    assert np.array_equal(b["position"][ha], r["position"][ha])
    nb, na = b["normal"][ha, :3], r["normal"][ha, :3]
    cosang = np.sum(nb * na, 1) / np.linalg.norm(nb, axis=1) / np.linalg.norm(na, axis=1)
    assert np.degrees(np.arccos(np.clip(cosang, -1, 1))).max() < 0.5
