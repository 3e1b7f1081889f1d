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


def _frame(w, h, seed):
    rng = np.random.default_rng(seed)
    img = rng.gamma(1.5, 0.6, size=(h, w, 3)).astype(np.float32)
    n = rng.normal(size=(h, w, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    depth = rng.uniform(1, 6, size=(h, w, 1))
    depth[rng.random((h, w, 1)) < 0.05] = -1.0  # pixels without a first hit
    return img, np.concatenate([n, depth], -1).astype(np.float32)


def test_noalloc_post_matches_allocating_entry(native_lib):
    torch = pytest.importorskip("torch")
    import bcgx
    from bcgx._lib import lib

    L = lib()
    ctx = bcgx.Context(0)
    try:
        for call, (w, h, seed) in enumerate([(320, 200, 1), (256, 144, 2)]):  # two calls in a row
            img, g = _frame(w, h, seed)
            st = bcgx.ultra_realism_settings("CPU")  # denoise 3 passes, bloom 1, ACES
            st.exposure = 0.25 * call
            ref_lin, ref_rgba = ctx.post_process(img, g, st)
            dev = torch.device("cuda", 0)
            d_in = torch.from_numpy(img).to(dev)
            d_g = torch.from_numpy(g).to(dev)
            d_out = torch.empty_like(d_in)
            d_rgba = torch.empty((h, w), dtype=torch.int32, device=dev)
            sc = st.c()
            torch.cuda.synchronize()
            rc = L.bc_post_process_noalloc(w, h, d_in.data_ptr(), d_g.data_ptr(), C.byref(sc), d_out.data_ptr(),
                                           d_rgba.data_ptr(), None)
            assert rc == 0, rc
            torch.cuda.synchronize()
            out = d_out.cpu().numpy()
            rgba = d_rgba.cpu().numpy().view(np.uint32)
            # same kernels, same order: identical up to fp32 reassociation (tolerance 1e-6 relative)
            assert np.allclose(out, ref_lin, rtol=1e-6, atol=1e-7), call
            assert np.array_equal(rgba, ref_rgba), call
        # frames beyond the static scratch are rejected, not truncated
        big = torch.zeros((1500 * 1000 * 3,), dtype=torch.float32, device="cuda")
        rc = L.bc_post_process_noalloc(1500, 1000, big.data_ptr(), big.data_ptr(), C.byref(sc), big.data_ptr(), None,
                                       None)
        assert rc == 7  # BC_ERR_INVALID_ARG
    finally:
        ctx.close()
