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


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "sfq"])
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


@pytest.mark.parametrize("kind", ["gwfq", "glfq"])
def test_rt_other_tilings(gcq, oracle_lib, kind):
    # uneven tiles, fewer threads per tile than pixels, 2 bounces
    want = np.zeros((240, 320, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_render(1, 320, 240, 2, want.ctypes.data)
    r, img = gcq.rt_render(kind, scene=1, width=320, height=240, tiles_x=3, tiles_y=5, threads_per_tile=96,
                           max_bounces=2, queue_log2=13)
    assert r["total_rays"] == n and r["leftover"] == 0
    assert np.abs(img - want).max() <= TOL


def test_rt_rejects_ymc_and_small_queue(gcq):
    with pytest.raises(gcq.GcqError) as e:
        gcq.rt_render("wfq", scene=0)
    assert e.value.status == gcq.EUNSUPPORTED
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


@pytest.mark.parametrize("kind", ["gwfq", "glfq"])
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
