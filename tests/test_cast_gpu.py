"""GPU parity of the extend (closest-hit) and shadow (any-hit) kernels through
the C ABI: bit-exact hit triangle, object, t and barycentrics, and bit-exact
occlusion, against the reference's golden outputs and the oracle."""
import numpy as np
import pytest

import oracle
from conftest import golden
from yar_gb300 import native, scenes
from yar_gb300.scene import FlatScene, Mesh, make_object

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_same_hits(got, want):
    t, prim, obj, bary = got
    wt, wprim, wobj, wbary = want
    assert np.array_equal(prim, wprim), np.nonzero(prim != wprim)[0][:10]
    assert np.array_equal(obj, wobj)
    assert np.array_equal(bits(t), bits(wt))
    assert np.array_equal(bits(bary), bits(wbary))


@pytest.mark.parametrize("name", ["raycast_small", "transform_small", "cornell_c1_64"])
def test_golden_scene_casts(gpu_ctx, name):
    s = FlatScene.read(golden(name + ".yfs"))
    gpu_ctx.upload_scene(s)
    if name == "cornell_c1_64":
        lo, hi = scenes.scene_box(s)
        rays = scenes.random_rays(lo, hi, 8192, 5)
        want = oracle.cast_closest(s, rays)
        shadow = scenes.random_shadow_rays(lo, hi, 8192, 6)
        want_occ = oracle.cast_any(s, shadow)
    else:
        g = np.load(golden(name + ".npz"))
        rays, shadow = g["rays"], g["shadow_rays"]
        want = (g["t"], g["prim"], g["obj"], g["bary"])
        want_occ = g["occluded"]
    assert_same_hits(gpu_ctx.cast_closest(rays), want)
    assert np.array_equal(gpu_ctx.cast_any(shadow), want_occ)


@pytest.mark.parametrize("k", [0, 1])
def test_kdtree_regression_meshes(gpu_ctx, k):
    g = np.load(golden("kdtree_regression.npz"))
    s = FlatScene()
    s.meshes = [Mesh(g["mesh%d_vertices" % k], g["mesh%d_indices" % k], bounds=g["mesh%d_bounds" % k],
                     nodes=g["mesh%d_nodes" % k])]
    s.objects = np.array([make_object(0)])
    s.build_scene_kdtree()
    rays = np.zeros((g["mesh%d_rays" % k].shape[0], 8), np.float32)
    rays[:, 0:3] = g["mesh%d_rays" % k][:, 0:3]
    rays[:, 4:7] = g["mesh%d_rays" % k][:, 3:6]
    rays[:, 3] = np.inf
    gpu_ctx.upload_scene(s)
    t, prim, obj, bary = gpu_ctx.cast_closest(rays)
    assert np.array_equal(bits(t), bits(g["mesh%d_t" % k]))
    assert np.array_equal(prim, g["mesh%d_prim" % k])


@pytest.fixture(scope="module")
def medium_scene():
    return scenes.raycast_scene(seed=4, grid=256, spheres=64, level=4, build=True)


def test_medium_scene_against_oracle(gpu_ctx, medium_scene):
    s = medium_scene
    gpu_ctx.upload_scene(s)
    lo, hi = scenes.scene_box(s)
    rays = scenes.random_rays(lo, hi, 300_000, 17)
    assert_same_hits(gpu_ctx.cast_closest(rays), oracle.cast_closest(s, rays))
    shadow = scenes.random_shadow_rays(lo, hi, 300_000, 18)
    assert np.array_equal(gpu_ctx.cast_any(shadow), oracle.cast_any(s, shadow))


def test_edge_case_rays(gpu_ctx, medium_scene):
    """Axis-parallel directions (zero components, +-inf inverse), origins
    exactly on split planes, zero tmax, rays starting outside and pointing
    away, and empty batches."""
    s = medium_scene
    gpu_ctx.upload_scene(s)
    lo, hi = scenes.scene_box(s)
    rng = np.random.default_rng(1)
    n = 60_000
    rays = scenes.random_rays(lo, hi, n, 19)
    axis = rng.integers(0, 3, n)
    sign = np.where(rng.random(n) < 0.5, -1.0, 1.0).astype(np.float32)
    rays[: n // 3, 4:7] = 0.0
    rays[np.arange(n // 3), 4 + axis[: n // 3]] = sign[: n // 3]
    # origins on split planes of the terrain tree
    nodes = s.meshes[0].nodes
    interior = nodes[(nodes[:, 0] & 3) != 3]
    pick = rng.integers(0, interior.shape[0], n // 3)
    planes = interior[pick, 1].view(np.float32)
    ax = (interior[pick, 0] & 3).astype(np.int64)
    sl = slice(n // 3, 2 * n // 3)
    rays[sl][np.arange(n // 3), ax] = planes
    rays[2 * n // 3: 2 * n // 3 + 1000, 3] = 0.0          # tmax = 0: nothing can hit
    rays[-1000:, 0:3] = hi + 1.0                            # outside, pointing away
    rays[-1000:, 4:7] = np.abs(rays[-1000:, 4:7])
    assert_same_hits(gpu_ctx.cast_closest(rays), oracle.cast_closest(s, rays))
    shadow = rays.copy()
    shadow[:, 3] = np.where(np.isinf(shadow[:, 3]), 0.5, shadow[:, 3])
    assert np.array_equal(gpu_ctx.cast_any(shadow), oracle.cast_any(s, shadow))
    empty = np.zeros((0, 8), np.float32)
    assert gpu_ctx.cast_closest(empty)[0].shape == (0,)
    assert gpu_ctx.cast_any(empty).shape == (0,)


def test_visibility_flags_and_degenerate_triangles(gpu_ctx):
    """Invisible meshes are skipped by both casts, no-shadow meshes only by the
    any-hit cast (src/ref/scene_context.cpp:98-106); degenerate triangles never
    report a hit (src/ref/kdtree.cpp:27-29)."""
    v = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0], [0.5, 0.5, 0], [0.5, 0.5, 0]], np.float32)
    tri = np.array([[0, 1, 2]], np.int32)
    degenerate = np.array([[3, 4, 0], [0, 1, 2]], np.int32)
    s = FlatScene()
    s.meshes = [Mesh(v, tri, visibility=0), Mesh(v, tri, visibility=1), Mesh(v, tri, visibility=2),
                Mesh(v, degenerate)]
    m = lambda z: np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, z], np.float32)
    s.objects = np.array([make_object(0, m(0.0)), make_object(1, m(-1.0)), make_object(2, m(-2.0)),
                          make_object(3, m(-3.0))])
    s.build_kdtrees(1)
    gpu_ctx.upload_scene(s)
    rays = np.zeros((4, 8), np.float32)
    rays[:, 0:3] = [0.0, -0.2, 5.0]
    rays[:, 4:7] = [0, 0, -1]
    rays[:, 3] = [np.inf, 5.5, 6.5, 7.5]
    t, prim, obj, _ = gpu_ctx.cast_closest(rays)
    want = oracle.cast_closest(s, rays)
    assert np.array_equal(obj, want[2]) and np.array_equal(prim, want[1])
    assert obj[0] == 0
    shadow = rays.copy()
    shadow[0:3, 0:3] = [0.0, -0.2, -0.5]      # below object 0: only the no-shadow/invisible ones in range
    occ = gpu_ctx.cast_any(shadow)
    assert np.array_equal(occ, oracle.cast_any(s, shadow))


def test_device_buffers_match_host_buffers(gpu_ctx, medium_scene):
    torch = pytest.importorskip("torch")
    s = medium_scene
    gpu_ctx.upload_scene(s)
    lo, hi = scenes.scene_box(s)
    rays = scenes.random_rays(lo, hi, 100_000, 23)
    host = gpu_ctx.cast_closest(rays)
    d_rays = torch.from_numpy(rays).cuda()
    n = rays.shape[0]
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    obj = torch.empty(n, dtype=torch.int32, device="cuda")
    bary = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ms = gpu_ctx.cast_closest_device(d_rays.data_ptr(), n, t.data_ptr(), prim.data_ptr(), obj.data_ptr(),
                                     bary.data_ptr(), timed=True)
    assert ms > 0
    dev = (t.cpu().numpy(), prim.cpu().numpy().view(np.uint32), obj.cpu().numpy().view(np.uint32),
           bary.cpu().numpy())
    assert_same_hits(dev, host)
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    gpu_ctx.cast_any_device(d_rays.data_ptr(), n, occ.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(occ.cpu().numpy(), gpu_ctx.cast_any(rays))


def test_pipelined_host_casts_match_device_casts(medium_scene):
    """Host-buffer batches of two or more pipeline chunks overlap their copies
    with the traversal (the first call of a scene tunes the kernel and runs
    unpipelined): a ragged 3,145,745-ray batch in 1M-ray chunks gives the
    device-buffer results bit for bit, without the output it leaves out (bary)."""
    torch = pytest.importorskip("torch")
    from yar_gb300 import native
    import ctypes as C
    from conftest import cuda_available
    if not cuda_available():
        pytest.skip("no CUDA device")
    s = medium_scene
    gpu_ctx = native.Context(0, pipeline_chunk_rays=1 << 20)
    gpu_ctx.upload_scene(s)
    lo, hi = scenes.scene_box(s)
    n = 3 * (1 << 20) + 17
    rays = scenes.random_rays(lo, hi, n, 31)
    shadow = scenes.random_shadow_rays(lo, hi, n, 32)
    first = gpu_ctx.cast_closest(rays)  # tunes
    gpu_ctx.cast_any(shadow)
    t = np.empty(n, np.float32)
    prim = np.empty(n, np.uint32)
    obj = np.empty(n, np.uint32)
    hits = native.HitSoa(t.ctypes.data, prim.ctypes.data, obj.ctypes.data, None)
    assert native.lib().yar_gpu_cast_closest(gpu_ctx._h, rays.ctypes.data, n, C.byref(hits),
                                             native.YAR_BUFFERS_HOST) == 0
    host_occ = gpu_ctx.cast_any(shadow)
    d_rays = torch.from_numpy(rays).cuda()
    d_shadow = torch.from_numpy(shadow).cuda()
    dt = torch.empty(n, dtype=torch.float32, device="cuda")
    dprim = torch.empty(n, dtype=torch.int32, device="cuda")
    dobj = torch.empty(n, dtype=torch.int32, device="cuda")
    dbary = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    docc = torch.empty(n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    gpu_ctx.cast_closest_device(d_rays.data_ptr(), n, dt.data_ptr(), dprim.data_ptr(), dobj.data_ptr(),
                                dbary.data_ptr())
    gpu_ctx.cast_any_device(d_shadow.data_ptr(), n, docc.data_ptr())
    torch.cuda.synchronize()
    dev = (dt.cpu().numpy(), dprim.cpu().numpy().view(np.uint32), dobj.cpu().numpy().view(np.uint32),
           dbary.cpu().numpy())
    assert np.array_equal(bits(t), bits(dev[0])) and np.array_equal(prim, dev[1]) and np.array_equal(obj, dev[2])
    assert_same_hits(first, dev)
    assert np.array_equal(host_occ, docc.cpu().numpy())
    gpu_ctx.close()


def test_malformed_scene_is_rejected_on_the_host(gpu_ctx):
    s = FlatScene.read(golden("raycast_small.yfs"))
    bad = FlatScene.read(golden("raycast_small.yfs"))
    nodes = bad.meshes[0].nodes.copy()
    interior = np.nonzero((nodes[:, 0] & 3) != 3)[0][0]
    nodes[interior, 0] = (nodes[interior, 0] & 3) | (np.uint32(nodes.shape[0] + 5) << np.uint32(2))
    bad.meshes[0].nodes = nodes
    with pytest.raises(native.YarError) as e:
        gpu_ctx.upload_scene(bad)
    assert e.value.code == native.YAR_ERR_INVALID
    with pytest.raises(native.YarError):
        gpu_ctx.cast_closest(np.zeros((4, 8), np.float32))   # no scene after a failed upload
    gpu_ctx.upload_scene(s)                                  # the context stays usable
    g = np.load(golden("raycast_small.npz"))
    assert np.array_equal(gpu_ctx.cast_closest(g["rays"])[1], g["prim"])


def test_batch_capacity_error():
    if not pytest.importorskip("torch").cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = native.Context(0, max_batch_rays=1000)
    try:
        ctx.upload_scene(FlatScene.read(golden("raycast_small.yfs")))
        with pytest.raises(native.YarError) as e:
            ctx.cast_closest(np.zeros((1001, 8), np.float32))
        assert e.value.code == native.YAR_ERR_CAPACITY
        ctx.cast_closest(np.zeros((1000, 8), np.float32))
    finally:
        ctx.close()


@pytest.mark.parametrize("kernel", [native.TRAVERSAL_PERSISTENT_64, native.TRAVERSAL_PERSISTENT_128,
                                    native.TRAVERSAL_PER_RAY, native.TRAVERSAL_PER_RAY_VOTE])
def test_every_traversal_kernel_matches_oracle(medium_scene, kernel):
    if not pytest.importorskip("torch").cuda.is_available():
        pytest.skip("no CUDA device")
    s = medium_scene
    ctx = native.Context(0, traversal_kernel=kernel)
    try:
        ctx.upload_scene(s)
        lo, hi = scenes.scene_box(s)
        rays = scenes.random_rays(lo, hi, 200_000, 31)
        assert_same_hits(ctx.cast_closest(rays), oracle.cast_closest(s, rays))
        shadow = scenes.random_shadow_rays(lo, hi, 200_000, 32)
        assert np.array_equal(ctx.cast_any(shadow), oracle.cast_any(s, shadow))
    finally:
        ctx.close()


def test_tuned_batch_matches_fixed_kernel(gpu_ctx, medium_scene):
    """A batch large enough to trigger the per-scene kernel timing returns the
    same results as a fixed kernel, on the timing call and after it."""
    s = medium_scene
    lo, hi = scenes.scene_box(s)
    rays = scenes.random_rays(lo, hi, (1 << 20) + 3, 33)
    shadow = scenes.random_shadow_rays(lo, hi, (1 << 20) + 3, 34)
    fixed = native.Context(0, traversal_kernel=native.TRAVERSAL_PER_RAY)
    try:
        fixed.upload_scene(s)
        want, want_occ = fixed.cast_closest(rays), fixed.cast_any(shadow)
    finally:
        fixed.close()
    gpu_ctx.upload_scene(s)
    for _ in range(2):
        assert_same_hits(gpu_ctx.cast_closest(rays), want)
        assert np.array_equal(gpu_ctx.cast_any(shadow), want_occ)


def test_invalid_traversal_kernel_option():
    if not pytest.importorskip("torch").cuda.is_available():
        pytest.skip("no CUDA device")
    with pytest.raises(native.YarError) as e:
        native.Context(0, traversal_kernel=7)
    assert e.value.code == native.YAR_ERR_INVALID


@pytest.mark.parametrize("kernel", [native.TRAVERSAL_PERSISTENT_64, native.TRAVERSAL_PER_RAY])
def test_alpha_test_matches_oracle(kernel):
    """Both casts skip triangle hits whose alpha texture reads red 0 at the hit's
    uv (src/ref/kdtree.cpp:31-38, :69-77): bit-identical to the oracle on rays
    through the cut-out fence of cornell_alpha_64, and different from the same
    scene without its alpha texture."""
    s = FlatScene.read(golden("cornell_alpha_64.yfs"))
    fence = [i for i, m in enumerate(s.meshes) if m.alpha_texture]
    assert fence
    ctx = native.Context(0, traversal_kernel=kernel)
    try:
        ctx.upload_scene(s)
        lo, hi = scenes.scene_box(s)
        rays = scenes.random_rays(lo, hi, 200_000, 23)
        got = ctx.cast_closest(rays)
        assert_same_hits(got, oracle.cast_closest(s, rays))
        shadow = scenes.random_shadow_rays(lo, hi, 200_000, 24)
        occ = ctx.cast_any(shadow)
        assert np.array_equal(occ, oracle.cast_any(s, shadow))
        fence_objects = [k for k, o in enumerate(s.objects) if o["mesh_index"] in fence]
        assert np.isin(got[2], fence_objects).sum() > 1000  # the fence's kept parts are hit
        for i in fence:
            s.meshes[i].alpha_texture = 0
        ctx.upload_scene(s)
        assert not np.array_equal(ctx.cast_any(shadow), occ)
    finally:
        ctx.close()
