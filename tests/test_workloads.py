"""Shapes of the seeded synthetic workloads (no GPU)."""
from bcgx import scenes


def test_batch_workload_generator_shapes():
    specs, views = scenes.batch_views(n_views=64, sizes=(1000, 2000, 3000, 4000))
    assert [s.n_triangles() for s in specs] == [1002, 2002, 3002, 4002]
    Ws = [st.width for _, _, st in views]
    Hs = [st.height for _, _, st in views]
    assert min(Ws) >= 128 and max(Ws) <= 1920 and min(Hs) >= 128 and max(Hs) <= 1080
    assert all(4 <= st.spp <= 64 and st.bounces == 8 for _, _, st in views)
    assert [k for k, _, _ in views] == [v % 4 for v in range(64)]
    # same seed, same workload
    _, again = scenes.batch_views(n_views=64, sizes=(1000, 2000, 3000, 4000))
    assert [(st.width, st.height, st.spp, st.seed) for _, _, st in views] == \
           [(st.width, st.height, st.spp, st.seed) for _, _, st in again]
