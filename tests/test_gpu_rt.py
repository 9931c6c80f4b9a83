"""Ray-tracer parity: the persistent per-tile GPU render (every bounce in one
launch, one queue per tile) and the stream-compaction baseline against the serial
CPU renders of the oracle.  Both sides perform the same float operations in the
same order without contraction (device and host), so the images are identical;
TOL = 0 is the bar."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 0.0


@pytest.fixture(scope="module")
def cpu_images(oracle_lib):
    out = {}
    for scene in (0, 1):
        img = np.zeros((720, 1280, 3), np.float32)
        n = oracle_lib.lib().oracle_rt_render(scene, 1280, 720, 4, img.ctypes.data)
        out[scene] = (img, n)
    return out


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "wfq", "sfq"])
@pytest.mark.parametrize("scene", [0, 1])
def test_rt_reference_scene(gcq, cpu_images, kind, scene):
    # the reference configuration: 1280x720, 8x8 tiles, 1024 threads per tile, 4 bounces
    r, img = gcq.rt_render(kind, scene=scene)
    want, rays = cpu_images[scene]
    assert r["leftover"] == 0
    assert r["total_rays"] == rays
    assert r["primary_rays"] == 1280 * 720
    diff = np.abs(img - want)
    assert diff.max() <= TOL, (float(diff.max()), int((diff > TOL).sum()))


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "wfq"])
def test_rt_other_tilings(gcq, oracle_lib, kind):
    # uneven tiles, fewer threads per tile than pixels, 2 bounces
    want = np.zeros((240, 320, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_render(1, 320, 240, 2, want.ctypes.data)
    r, img = gcq.rt_render(kind, scene=1, width=320, height=240, tiles_x=3, tiles_y=5, threads_per_tile=96,
                           max_bounces=2, queue_log2=13)
    assert r["total_rays"] == n and r["leftover"] == 0
    assert np.abs(img - want).max() <= TOL


def test_rt_rejects_small_queue(gcq):
    with pytest.raises(gcq.GcqError) as e:
        gcq.rt_render("gwfq", scene=0, queue_log2=12)   # a 160x90 tile does not fit 4096 slots
    assert e.value.status == gcq.ECAPACITY


# ------------------------------------------------- the stream-compaction baseline
@pytest.mark.parametrize("scene", [0, 1, 2])
def test_rt_compact_reference_size(gcq, oracle_lib, scene):
    """rt_compaction.cpp's renderer at its own size (1280x720, 4 bounces): the image
    equals the serial restatement of its shading bit for bit, and every pass's rays
    are counted."""
    want = np.zeros((720, 1280, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_compact_render(scene, 1280, 720, 4, want.ctypes.data)
    r, img = gcq.rt_compact_render(scene=scene, max_bounces=4)
    assert r["primary_rays"] == 1280 * 720
    assert r["total_rays"] == n
    assert np.array_equal(img, want), float(np.abs(img - want).max())


def test_rt_compact_deep_tunnel(gcq, oracle_lib):
    # the mirror tunnel keeps most rays alive for many bounces
    want = np.zeros((180, 320, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_compact_render(2, 320, 180, 12, want.ctypes.data)
    r, img = gcq.rt_compact_render(scene=2, width=320, height=180, max_bounces=12)
    assert r["total_rays"] == n and n > 320 * 180 * 6
    assert np.array_equal(img, want)


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "wfq"])
def test_rt_queue_tunnel_scene(gcq, oracle_lib, kind):
    # the queue renderer on the compaction baseline's scene 2, its own shading
    want = np.zeros((180, 320, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_render(2, 320, 180, 8, want.ctypes.data)
    r, img = gcq.rt_render(kind, scene=2, width=320, height=180, tiles_x=4, tiles_y=4, threads_per_tile=256,
                           max_bounces=8)
    assert r["leftover"] == 0 and r["total_rays"] == n
    assert np.abs(img - want).max() <= TOL


def test_rt_compact_rejects(gcq):
    for kw in [dict(scene=3), dict(width=0), dict(max_bounces=-1)]:
        with pytest.raises(gcq.GcqError) as e:
            gcq.rt_compact_render(**kw)
        assert e.value.status == gcq.EINVAL


# ------------------------------------ benchmark scenes: 1024x1024, 1 spp, 4 bounces
BOUNCE_TOL = 1e-4   # per fp32 channel; the two renders perform the same operations


def _bounce_cpu(oracle_lib, scene, w, h, bounces, seed=1):
    img = np.zeros((h, w, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_bounce_render(scene, w, h, bounces, seed, 16, img.ctypes.data)
    assert n > 0
    return img, n


@pytest.fixture(scope="module")
def bounce_images(oracle_lib):
    return {s: _bounce_cpu(oracle_lib, s, 1024, 1024, 4) for s in (0, 1)}


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "wfq", "sfq"])
@pytest.mark.parametrize("scene", [0, 1])
def test_rt_bounce_full_size(gcq, bounce_images, kind, scene):
    """The benchmark configuration: 1024x1024, 32x32-pixel tiles, 1024 threads per
    tile, queue 2^15 per tile, 4 bounces; image and ray count equal the serial render."""
    r, img = gcq.rt_bounce_render(kind, scene=scene)
    want, rays = bounce_images[scene]
    assert r["leftover"] == 0
    assert r["primary_rays"] == 1024 * 1024
    assert r["total_rays"] == rays
    diff = np.abs(img - want)
    assert diff.max() <= BOUNCE_TOL, (float(diff.max()), int((diff > BOUNCE_TOL).sum()))
    assert np.isfinite(img).all()


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "wfq", "sfq"])
@pytest.mark.parametrize("case", [
    dict(width=100, height=70, tile_px=32, threads_per_tile=1024, max_bounces=4, queue_log2=10),  # ragged tiles
    dict(width=96, height=96, tile_px=16, threads_per_tile=40, max_bounces=6, queue_log2=8),      # fewer threads
    dict(width=64, height=48, tile_px=8, threads_per_tile=512, max_bounces=0, queue_log2=9),      # primary only
    dict(width=1, height=1, tile_px=32, threads_per_tile=32, max_bounces=4, queue_log2=10),       # one pixel
])
@pytest.mark.parametrize("scene", [0, 1])
def test_rt_bounce_edge_cases(gcq, oracle_lib, kind, case, scene):
    want, rays = _bounce_cpu(oracle_lib, scene, case["width"], case["height"], case["max_bounces"], seed=7)
    r, img = gcq.rt_bounce_render(kind, scene=scene, seed=7, **case)
    assert r["leftover"] == 0 and r["total_rays"] == rays
    assert np.abs(img - want).max() <= BOUNCE_TOL


def test_rt_ymc_reuses_tiles_and_pool(gcq, oracle_lib):
    """YMC tile queues rendered again from the same context (rings and pools
    re-initialised between renders), tile lists in another order: the tiles equal
    the serial render each time and no pool runs dry."""
    want, _ = _bounce_cpu(oracle_lib, 1, 256, 256, 4)
    with gcq.RtTiles("wfq", scene=1, width=256, height=256, max_tiles=16) as c:
        tiles = np.arange(64, dtype=np.int32)
        for rep in range(2):
            for chunk in (tiles[::-1][:16], tiles[16:32], tiles[32:48], tiles[48:]):
                c.render(np.ascontiguousarray(chunk))
        r, img = c.render(tiles[:16], image=True)
    assert np.abs(img - want).max() <= BOUNCE_TOL


def test_rt_bounce_seed_changes_scene(gcq, oracle_lib):
    a = gcq.rt_bounce_render("gwfq", scene=0, width=128, height=128, seed=1)[1]
    b = gcq.rt_bounce_render("gwfq", scene=0, width=128, height=128, seed=2)[1]
    want, _ = _bounce_cpu(oracle_lib, 0, 128, 128, 4, seed=2)
    assert np.abs(a - b).max() > 0.1
    assert np.abs(b - want).max() <= BOUNCE_TOL


def test_rt_bounce_rejects(gcq):
    for kwargs, status in [(dict(queue_log2=9), gcq.ECAPACITY),          # a 32x32 tile needs 1024 slots
                           (dict(scene=2), gcq.EINVAL),
                           (dict(max_bounces=-1), gcq.EINVAL),
                           (dict(width=0), gcq.EINVAL)]:
        with pytest.raises(gcq.GcqError) as e:
            gcq.rt_bounce_render(**kwargs)
        assert e.value.status == status, kwargs
