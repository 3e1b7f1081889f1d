"""The allocation-free post-processing entry point (bc_post_process_noalloc).

Some callers cannot allocate device memory when they post-process a frame
(an engine or plugin host that owns the GPU memory budget, an allocation-free
real-time loop, code that must not synchronise the device). This entry point
takes the caller's device buffers and keeps its scratch in a static device
array. It must give the same result as bc_post_process, which allocates.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test; it passes alone and after them.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BC_ERR_INVALID_ARG = 7


def _frame(w, h, seed):
    rng = np.random.default_rng(seed)
    img = rng.gamma(1.5, 0.6, size=(h, w, 3)).astype(np.float32)
    n = rng.normal(size=(h, w, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    depth = rng.uniform(1, 6, size=(h, w, 1))
    depth[rng.random((h, w, 1)) < 0.05] = -1.0  # pixels without a first hit
    return img, np.concatenate([n, depth], -1).astype(np.float32)


@pytest.fixture(scope="module")
def post_ctx(native_lib):
    import bcgx
    ctx = bcgx.Context(0)
    yield ctx
    ctx.close()


def _noalloc(L, st, img, g, want_rgba):
    """Runs the entry point on device copies of img and g; returns host copies of its outputs."""
    import torch
    h, w = img.shape[:2]
    dev = torch.device("cuda", 0)
    d_in = torch.from_numpy(img).to(dev)
    d_g = torch.from_numpy(g).to(dev) if g is not None else None
    d_out = torch.full_like(d_in, float("nan"))  # a pass that writes nothing shows up
    d_rgba = torch.zeros((h, w), dtype=torch.int32, device=dev) if want_rgba else None
    sc = st.c()
    torch.cuda.synchronize()
    rc = L.bc_post_process_noalloc(w, h, d_in.data_ptr(), d_g.data_ptr() if d_g is not None else None, C.byref(sc),
                                   d_out.data_ptr(), d_rgba.data_ptr() if d_rgba is not None else None, None)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    rgba = d_rgba.cpu().numpy().view(np.uint32) if d_rgba is not None else None
    return rc, out, rgba


# Every routing of the passes through the output and the static scratch:
# denoise alone (the last pass lands in the output), bloom alone (it reads the
# input directly), both (the last pass lands in scratch), neither (a copy), an
# odd and an even number of a-trous passes, a pass count of zero or less
# (taa = txaa = -2: the input passes through), and with and without RGBA.
CASES = [
    # denoise, bloom, taa, txaa, rgba
    (True, 1, 1, 0, True),     # 3 passes + bloom (the Ultra Realism post stack)
    (True, 0, 1, 0, True),     # 3 passes, denoise only
    (True, 0, 0, 0, False),    # 2 passes, denoise only, no RGBA
    (True, 2, 3, 0, True),     # 5 passes + bloom level 2
    (True, 1, 0, 2, False),    # 4 passes via txaa + bloom, no RGBA
    (False, 1, 0, 0, True),    # bloom only
    (False, 0, 0, 0, True),    # neither: copy + tone map
    (False, 0, 0, 0, False),   # neither, no RGBA
    (True, 0, -2, -2, True),   # zero passes: input unchanged
    (True, 1, -3, -2, True),   # zero passes, then bloom
]


@pytest.mark.parametrize("denoise,bloom,taa,txaa,want_rgba", CASES)
def test_noalloc_post_matches_allocating_entry(post_ctx, denoise, bloom, taa, txaa, want_rgba):
    pytest.importorskip("torch")
    import bcgx
    from bcgx._lib import lib

    L = lib()
    for call, (w, h, seed) in enumerate([(320, 200, 1), (256, 144, 2)]):  # two calls in a row
        img, g = _frame(w, h, seed + 10 * int(denoise) + bloom)
        st = bcgx.ultra_realism_settings("CPU")  # ACES tone map, gamma 2.2
        st.denoise, st.bloom, st.taa, st.txaa = denoise, bloom, taa, txaa
        st.exposure = 0.25 * call
        ref_lin, ref_rgba = post_ctx.post_process(img, g, st, want_rgba=want_rgba)
        rc, out, rgba = _noalloc(L, st, img, g, want_rgba)
        assert rc == 0, rc
        # same kernels in the same order: equal up to fp32 reassociation (1e-6 relative)
        assert np.allclose(out, ref_lin, rtol=1e-6, atol=1e-7), call
        if want_rgba:
            assert np.array_equal(rgba, ref_rgba), call
        if denoise and 2 + min(3, max(taa, txaa)) <= 0 and not bloom:
            assert np.array_equal(out, img)  # nothing to do: the input comes back


def test_noalloc_rejects_bad_arguments(native_lib):
    torch = pytest.importorskip("torch")
    import bcgx
    from bcgx._lib import lib

    L = lib()
    st = bcgx.ultra_realism_settings("CPU")
    sc = st.c()
    dev = torch.device("cuda", 0)
    w, h = 64, 48
    a = torch.zeros((h, w, 3), dtype=torch.float32, device=dev)
    b = torch.zeros((h, w, 3), dtype=torch.float32, device=dev)
    g = torch.zeros((h, w, 4), dtype=torch.float32, device=dev)
    rgba = torch.zeros((h, w), dtype=torch.int32, device=dev)
    big = torch.zeros((1500 * 1000 * 3,), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    # frames beyond the static scratch are rejected, not truncated
    assert L.bc_post_process_noalloc(1500, 1000, big.data_ptr(), None, C.byref(sc), big.data_ptr(), None,
                                     None) == BC_ERR_INVALID_ARG
    # denoise without guides
    assert L.bc_post_process_noalloc(w, h, a.data_ptr(), None, C.byref(sc), b.data_ptr(), None,
                                     None) == BC_ERR_INVALID_ARG
    # output equal to, or overlapping, the input
    assert L.bc_post_process_noalloc(w, h, a.data_ptr(), g.data_ptr(), C.byref(sc), a.data_ptr(), None,
                                     None) == BC_ERR_INVALID_ARG
    assert L.bc_post_process_noalloc(w, h, a.data_ptr(), g.data_ptr(), C.byref(sc), a.data_ptr() + 12, None,
                                     None) == BC_ERR_INVALID_ARG
    # output overlapping the guides, RGBA overlapping the linear output
    assert L.bc_post_process_noalloc(w, h, a.data_ptr(), g.data_ptr(), C.byref(sc), g.data_ptr() + 16, None,
                                     None) == BC_ERR_INVALID_ARG
    assert L.bc_post_process_noalloc(w, h, a.data_ptr(), g.data_ptr(), C.byref(sc), b.data_ptr(),
                                     b.data_ptr() + 4 * w, None) == BC_ERR_INVALID_ARG
    # separate buffers are accepted
    assert L.bc_post_process_noalloc(w, h, a.data_ptr(), g.data_ptr(), C.byref(sc), b.data_ptr(), rgba.data_ptr(),
                                     None) == 0
    torch.cuda.synchronize()
