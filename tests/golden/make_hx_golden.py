"""Writes tests/golden/hx_closest.npz: the closest hits the reference's own C++
code (beamcast::hx::PackedScene::hit, source/src/hx.cpp:237-270, with its fp32
Moller-Trumbore test at hx.cpp:223-231) finds for seeded random triangles and
rays. It runs the reference library that `make -C oracle ref` compiles from the
reference's sources into oracle/_ref/, so it needs the reference tree; the
fixture lets the pin run without it.

Usage: python tests/golden/make_hx_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "beamcast-gx-v1.0-beta-_gb300"), os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
from bcgx import scenes  # noqa: E402

N_TRIS, TRI_SEED = 20_000, 0xBEAC0102
N_RAYS, RAY_SEED = 65_536, 0xBEAC0103


def main():
    oracle.build()
    verts = scenes.random_triangle_verts(N_TRIS, TRI_SEED)
    rays = scenes.random_rays(N_RAYS, seed=RAY_SEED)
    out = oracle.hx_reference_closest(verts, rays)
    if out is None:
        raise SystemExit("the reference library is not built (no reference tree here)")
    t, prim = out
    np.savez_compressed(os.path.join(HERE, "hx_closest.npz"), t=t, prim=prim, n_tris=N_TRIS, tri_seed=TRI_SEED,
                        n_rays=N_RAYS, ray_seed=RAY_SEED)
    print(f"{(prim >= 0).sum()} hits of {N_RAYS} rays")


if __name__ == "__main__":
    main()
