"""Ray-cast parity on the GPU through the C-ABI: the hit primitive index is
bit-exact against the fp64 oracle on the same BVH, and t is float32 of the
oracle's fp64 distance (the contract allows 2 ULP; the exact re-test gives 0).
"""
import numpy as np
import pytest

from bcgx import scenes

pytestmark = pytest.mark.gpu


def _ulp_diff(a, b):
    """Distance in units in the last place, on the ordered-integer line (+0 == -0)."""
    def ordered(x):
        i = x.astype(np.float32).view(np.int32).astype(np.int64)
        return np.where(i < 0, -(i & 0x7FFFFFFF), i)
    return np.abs(ordered(a) - ordered(b))


def _check(ctx, orc_scene, rays, max_ulp=0):
    """Bit-exact hit index on every ray, exact fp64 ties included: where several
    primitives share the minimal fp64 distance (coplanar faces, t == +0 == -0),
    the GPU returns the one the reference's binary traversal keeps."""
    t_gpu, p_gpu = ctx.raycast(rays)
    t_ref, p_ref, _ = orc_scene.hit_f32(rays)
    mism = np.nonzero(p_gpu != p_ref)[0]
    assert len(mism) == 0, f"{len(mism)} hit-index mismatches, first {mism[:5]}: gpu {p_gpu[mism[:5]]} ref {p_ref[mism[:5]]}"
    hit = p_ref >= 0
    assert np.all(t_gpu[~hit] == -1.0)
    d = _ulp_diff(t_gpu[hit], t_ref[hit].astype(np.float32))
    assert d.max(initial=0) <= max_ulp
    return hit


def test_random_triangles_parity(gpu_ctx, orc):
    spec = scenes.random_triangles(100_000, seed=scenes.SEED_TRIS)
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    ref = orc.OracleScene.from_spec(spec)
    rays = scenes.random_rays(262_144, seed=5)
    hit = _check(gpu_ctx, ref, rays)
    assert 0.05 < hit.mean() < 0.99


def test_gpu_consumes_callers_tree(gpu_ctx, orc):
    """Drop-in: the GPU traverses the tree the caller built (here the oracle's),
    handed over as plain arrays like the Go Scene."""
    spec = scenes.random_triangles(30_000, seed=3)
    ref = orc.OracleScene.from_spec(spec)
    gpu_ctx.upload(ref.arrays(), scene_id=991, topology_rev=1, geometry_rev=1)
    _check(gpu_ctx, ref, scenes.random_rays(65_536, seed=9))


@pytest.mark.parametrize("maker", ["stress", "showcase", "cornell_ref", "c1"])
def test_builtin_scenes_parity(gpu_ctx, orc, maker):
    spec, cam = {"stress": scenes.stress_scene, "showcase": scenes.showcase_scene,
                 "cornell_ref": scenes.cornell_reference_scene,
                 "c1": lambda: scenes.cornell_box()[:2]}[maker]()
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    ref = orc.OracleScene.from_spec(spec)
    rng = np.random.default_rng(17)
    n = 65_536
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = np.asarray(cam.position, np.float32)
    tgt = np.asarray(cam.target) + (rng.random((n, 3)) - 0.5) * 14
    rays[:, 4:7] = (tgt - np.asarray(cam.position)).astype(np.float32)
    rays[:, 3] = 1e-4
    rays[:, 7] = 1e30
    # secondary-ray-like origins inside the scene
    rays[n // 2:, 0:3] = (np.asarray(cam.target) + (rng.random((n - n // 2, 3)) - 0.5) * 6).astype(np.float32)
    _check(gpu_ctx, ref, rays)


def test_occluded_parity_and_closest_equivalence(gpu_ctx, orc):
    """TestOccludedMatchesClosestHit (renderer_test.go:658) on the GPU path."""
    spec, cam = scenes.stress_scene()
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    ref = orc.OracleScene.from_spec(spec)
    rng = np.random.default_rng(424242)
    n = 3000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = np.asarray(cam.position, np.float32)
    tgt = np.asarray(cam.target) + (rng.random((n, 3)) - 0.5) * np.array([24, 8, 24])
    rays[:, 4:7] = (tgt - np.asarray(cam.position)).astype(np.float32)
    rays[:, 3] = 1e-4
    rays[:, 7] = (0.25 + rng.random(n) * 30).astype(np.float32)
    occ = gpu_ctx.occluded(rays)
    _, p = gpu_ctx.raycast(rays)
    assert np.array_equal(occ, p >= 0)
    occ_ref, _ = ref.occluded_f32(rays)
    assert np.array_equal(occ, occ_ref)


def test_edge_rays(gpu_ctx, orc):
    """Zero direction components, origins on box faces and on triangle planes,
    tmax cut-offs, zero-length and NaN directions."""
    spec, _, _ = scenes.cornell_box()
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    ref = orc.OracleScene.from_spec(spec)
    rng = np.random.default_rng(1)
    rays = []
    for _ in range(4000):
        o = rng.uniform(-1, 1, 3)
        # snap some coordinates onto walls / boxes' planes exactly
        if rng.random() < 0.3:
            o[rng.integers(3)] = rng.choice([-1.0, 1.0, 0.999])
        d = rng.normal(size=3)
        k = rng.random()
        if k < 0.3:
            d[rng.integers(3)] = 0.0
        elif k < 0.4:
            d[:] = 0
            d[rng.integers(3)] = rng.choice([-1.0, 1.0])
        tmin = 1e-4 if rng.random() < 0.8 else 0.0
        tmax = 1e30 if rng.random() < 0.7 else rng.uniform(0.01, 2)
        rays.append([o[0], o[1], o[2], tmin, d[0], d[1], d[2], tmax])
    rays = np.array(rays, np.float32)
    cnt, _ = ref.tie_sets_f32(rays)
    assert (cnt >= 2).sum() >= 5  # the set holds exact fp64 ties, resolved as the reference resolves them
    _check(gpu_ctx, ref, rays)
    odd = np.array([[0, 0, 0, 1e-4, 0, 0, 0, 1e30], [0.1, 0.2, 0.3, 1e-4, np.nan, 1, 0, 1e30],
                    [0, 0, 0, 1e-4, 1, 0, 0, np.nan]], np.float32)
    t, p = gpu_ctx.raycast(odd)
    tr, pr, _ = ref.hit_f32(odd)
    assert p[0] == pr[0] == -1  # zero-length direction: no hit
    # NaN inputs have no meaningful reference answer; they must still return a valid record
    assert np.all((p >= -1) & (p < len(a_prims(spec))))


def a_prims(spec):
    return np.zeros(spec.n_triangles())


def test_empty_and_errors(gpu_ctx, native_lib):
    import bcgx
    t, p = gpu_ctx.raycast(np.zeros((0, 8), np.float32))
    assert len(t) == 0 and len(p) == 0
    # bad scenes are rejected on the host with BC_ERR_BAD_SCENE
    spec = scenes.random_triangles(1000, seed=2)
    a = scenes.to_scene(spec).arrays()
    bad = scenes.to_scene(spec).arrays()
    bad.node_count = bad.node_count.copy()
    bad.node_count[np.nonzero(bad.node_count)[0][0]] = 17
    with pytest.raises(bcgx.BCError) as e:
        gpu_ctx.upload(bad, scene_id=77, topology_rev=1, geometry_rev=1)
    assert e.value.status == 3
    bad2 = scenes.to_scene(spec).arrays()
    bad2.order = bad2.order.copy()
    bad2.order[0] = bad2.order[1]
    with pytest.raises(bcgx.BCError):
        gpu_ctx.upload(bad2, scene_id=78, topology_rev=1, geometry_rev=1)
    bad3 = scenes.to_scene(spec).arrays()
    bad3.node_left = bad3.node_left.copy()
    bad3.node_left[0] = 0
    with pytest.raises(bcgx.BCError):
        gpu_ctx.upload(bad3, scene_id=79, topology_rev=1, geometry_rev=1)
    gpu_ctx.upload(a, scene_id=80, topology_rev=1, geometry_rev=1)
    st = gpu_ctx.scene_stats()
    assert st["slots"] == len(a.prim_kind) and st["stack_need"] <= 256


def test_full_size_raycast_properties_and_sample(gpu_ctx, orc):
    """Workload 2 at full size: 1M triangles, 4M rays. Exact parity on a seeded
    sample of 131072 rays; size-independent properties on all rays."""
    spec = scenes.random_triangles(1_000_000, seed=scenes.SEED_TRIS)
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    rays = scenes.random_rays(4_194_304)
    t, p = gpu_ctx.raycast(rays)
    hit = p >= 0
    assert np.all((p[hit] >= 0) & (p[hit] < 1_000_000))
    assert np.all(t[hit] >= np.float32(1e-4)) and np.all(t[~hit] == -1)
    # any-hit agrees with closest-hit existence on every ray
    occ = gpu_ctx.occluded(rays)
    assert np.array_equal(occ, hit)
    ref = orc.OracleScene.from_spec(spec)
    idx = np.random.default_rng(0).choice(len(rays), 131_072, replace=False)
    tr, pr, _ = ref.hit_f32(rays[idx])
    assert np.array_equal(p[idx], pr)
    h = pr >= 0
    assert np.all(_ulp_diff(t[idx][h], tr[h].astype(np.float32)) == 0)


def _stacked_triangles(n_base=300, copies=8, seed=41):
    """Large random triangles, each repeated `copies` times: the first six copies
    coincide, the others are offset by 1e-7 along z. A ray through a stack meets
    at least six certain hits with the same distance interval, more contenders
    than the walk's list holds (four), which sends it to the third pass of the
    split form."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.1, 0.9, (n_base, 3))
    e1 = rng.normal(size=(n_base, 3)) * 0.15
    e2 = rng.normal(size=(n_base, 3)) * 0.15
    a = c - (e1 + e2) / 3
    base = np.concatenate([a, a + e1, a + e2], axis=1)
    layers = []
    for k in range(copies):
        off = np.zeros(9)
        off[2::3] = max(0, k - 5) * 1e-7
        layers.append(base + off)
    sp = scenes.SceneSpec(name="stacked", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)
    m = sp.material(scenes.Material(scenes.MAT_DIFFUSE, (0.5, 0.5, 0.5)))
    sp.triangles(np.concatenate(layers), m)
    return sp


@pytest.mark.parametrize("which", ["random", "stacked", "edge"])
def test_split_passes_parity(gpu_ctx, orc, which):
    """raycast_split 1 (the default: walk pass without fp64 code, fp64 settlement
    pass, and a pass that re-traces rays whose contender list overflowed) returns
    the same hits and distances as the one-kernel exact form (raycast_split 0),
    and both match the oracle; the same for the any hit."""
    if which == "random":
        spec = scenes.random_triangles(100_000, seed=scenes.SEED_TRIS + 7)
        rays = scenes.random_rays(262_144, seed=15)
    elif which == "stacked":
        spec = _stacked_triangles()
        rays = scenes.random_rays(131_072, seed=16)
    else:
        spec, _, _ = scenes.cornell_box()
        rng = np.random.default_rng(2)
        rays = scenes.random_rays(20_000, seed=17)
        rays[:, 0:3] = rng.uniform(-1, 1, (len(rays), 3))
        rays[::3, 4 + rng.integers(3)] = 0.0  # zero direction components
        rays[1::7, 1] = -1.0  # origins on the floor plane
    gpu_ctx.upload(scenes.to_scene(spec))
    ref = orc.OracleScene.from_spec(spec)
    assert gpu_ctx.get_option("raycast_split") == 1
    _check(gpu_ctx, ref, rays)
    two = gpu_ctx.raycast(rays)
    occ2 = gpu_ctx.occluded(rays)
    try:
        gpu_ctx.set_option("raycast_split", 0)
        _check(gpu_ctx, ref, rays)
        one = gpu_ctx.raycast(rays)
        occ1 = gpu_ctx.occluded(rays)
    finally:
        gpu_ctx.set_option("raycast_split", 1)
    assert np.array_equal(one[1], two[1]) and np.array_equal(one[0], two[0])
    # any hit: both forms, the oracle's Occluded, and closest-hit existence agree
    occ_ref, _ = ref.occluded_f32(rays)
    assert np.array_equal(occ2, occ1) and np.array_equal(occ2, occ_ref)
    assert np.array_equal(occ2, two[1] >= 0)
    # the split passes without the coherent ray order give the same answers
    try:
        gpu_ctx.set_option("raycast_sort", 0)
        three = gpu_ctx.raycast(rays)
        occ3 = gpu_ctx.occluded(rays)
    finally:
        gpu_ctx.set_option("raycast_sort", 1)
    assert np.array_equal(three[1], two[1]) and np.array_equal(three[0], two[0])
    assert np.array_equal(occ3, occ2)


def test_device_call_status_reaches_its_own_sync(gpu_ctx, native_lib):
    """A kernel status raised during bc_raycast_device / bc_occluded_device is
    returned by that call's bc_sync, and no later unrelated call sees it. The
    status bit is raised by the test hook "test_status_bits" (a one-thread
    kernel ORs it into the device-pointer calls' status word on their stream),
    as a traversal stack overflow would; nothing faults."""
    torch = pytest.importorskip("torch")
    import bcgx
    spec = scenes.random_triangles(20_000, seed=21)
    gpu_ctx.upload(scenes.to_scene(spec))
    rays = scenes.random_rays(4096, seed=22)
    dev = torch.device("cuda", 0)
    d_rays = torch.from_numpy(rays).to(dev)
    d_t = torch.empty(len(rays), dtype=torch.float32, device=dev)
    d_p = torch.empty(len(rays), dtype=torch.int32, device=dev)
    d_o = torch.empty(len(rays), dtype=torch.uint8, device=dev)
    s = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()
    # clean calls: sync is OK
    gpu_ctx.raycast_device(d_rays.data_ptr(), len(rays), d_t.data_ptr(), d_p.data_ptr(), s.cuda_stream)
    gpu_ctx.sync(s.cuda_stream)
    kStatusStackOverflow = 1
    for call in ("closest", "any"):
        gpu_ctx.set_option("test_status_bits", kStatusStackOverflow)
        if call == "closest":
            gpu_ctx.raycast_device(d_rays.data_ptr(), len(rays), d_t.data_ptr(), d_p.data_ptr(), s.cuda_stream)
        else:
            gpu_ctx.occluded_device(d_rays.data_ptr(), len(rays), d_o.data_ptr(), s.cuda_stream)
        # an unrelated host call in between does not pick the bit up
        t_h, p_h = gpu_ctx.raycast(rays)
        with pytest.raises(bcgx.BCError) as e:
            gpu_ctx.sync(s.cuda_stream)
        assert e.value.status == 9  # BC_ERR_CAPACITY: the stack-overflow status of this call
        gpu_ctx.sync(s.cuda_stream)  # cleared by the sync that returned it
        torch.cuda.synchronize()
        if call == "closest":  # the results themselves are unaffected by the hook
            assert np.array_equal(d_p.cpu().numpy(), p_h)


@pytest.mark.parametrize("which", ["random", "stacked"])
def test_merged_leaves_parity(gpu_ctx, orc, which):
    """With BVH8 leaf merging forced on (option scene_leaf_merge 1: binary
    subtrees of up to 8 primitives packed as one leaf), closest hits, exact ties
    included, and any hits still match the oracle and the unmerged packing."""
    if which == "random":
        spec = scenes.random_triangles(100_000, seed=scenes.SEED_TRIS + 9)
        rays = scenes.random_rays(262_144, seed=19)
    else:
        spec = _stacked_triangles(seed=43)
        rays = scenes.random_rays(131_072, seed=20)
    ref = orc.OracleScene.from_spec(spec)
    s = scenes.to_scene(spec)
    assert gpu_ctx.get_option("scene_leaf_merge") == -1
    gpu_ctx.upload(s)
    plain = gpu_ctx.raycast(rays)
    try:
        gpu_ctx.set_option("scene_leaf_merge", 1)
        gpu_ctx.upload(s)  # same scene: the changed option repacks it
        _check(gpu_ctx, ref, rays)
        merged = gpu_ctx.raycast(rays)
        occ = gpu_ctx.occluded(rays)
    finally:
        gpu_ctx.set_option("scene_leaf_merge", -1)
    assert np.array_equal(merged[1], plain[1]) and np.array_equal(merged[0], plain[0])
    occ_ref, _ = ref.occluded_f32(rays)
    assert np.array_equal(occ, occ_ref)
