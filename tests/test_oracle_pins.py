"""Pins the CPU oracle before it is trusted as the checker.

The reference ships no renderer output, no swscale golden and no tests
(the renderer lives in an un-vendored external project, README.md:5), so
render and swscale parity are unpinned.  These tests pin the oracle's parts
against facts that hold independently of it: the resolution rule, hash
indices worked out from the primes, trilinear interpolation identities,
spherical-harmonic orthonormality, the BT.601 colour-bar values, an
independent float32 restatement of the ray set-up, and the committed golden
render (cross-host determinism).
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

T19 = 1 << 19
P1, P2 = 2654435761, 805459861


def test_resolution_table(oracle_mod):
    b = (2048 / 16) ** (1 / 15)
    expect = [math.floor(16 * b ** l) for l in range(15)] + [2048]
    assert list(oracle_mod.resolutions()) == expect
    assert expect[:5] == [16, 22, 30, 42, 58] and expect[-1] == 2048


def test_dt_constant(oracle_mod):
    assert oracle_mod.dt() == np.float32(math.sqrt(3) / 1024)


def test_grid_index_known_answers(oracle_mod):
    # Level 0: N=16, 17^3 <= 2^19 -> dense, x fastest.
    assert oracle_mod.grid_index(0, T19, 1, 2, 3) == 1 + 17 * 2 + 17 * 17 * 3
    assert oracle_mod.grid_index(4, T19, 58, 58, 58) == 58 + 59 * 58 + 59 * 59 * 58
    # Level 5: N=80, 81^3 = 531441 > 2^19 -> hashed: (x*1 ^ y*P1 ^ z*P2) mod 2^32 mod T.
    for (x, y, z) in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (80, 80, 80), (17, 33, 65), (2048, 2047, 1)]:
        h = ((x * 1) ^ ((y * P1) & 0xFFFFFFFF) ^ ((z * P2) & 0xFFFFFFFF)) & 0xFFFFFFFF
        assert oracle_mod.grid_index(5 if x <= 81 else 15, T19, x, y, z) == h % T19
    assert oracle_mod.grid_index(5, T19, 0, 1, 0) == 2654435761 % T19
    # At 2^14 only levels 0 and 1 are dense.
    assert oracle_mod.grid_index(1, 1 << 14, 22, 22, 22) == 22 + 23 * 22 + 23 * 23 * 22
    assert oracle_mod.grid_index(2, 1 << 14, 0, 0, 1) == P2 % (1 << 14)


def test_trilinear_partition_of_unity(oracle_mod):
    s = oracle_mod.Scene(3, 14)
    s.set_param(0, np.full(16 * (1 << 14) * 2, 0.25, np.float32))
    rng = np.random.default_rng(0)
    for _ in range(50):
        f = s.encode(rng.uniform(0, 1, 3))
        assert np.allclose(f, 0.25, atol=1e-14)


def test_encoding_at_vertex_is_table_entry(oracle_mod):
    s = oracle_mod.Scene(0, 19)
    table = s.param(0).reshape(16, T19, 2)
    res = oracle_mod.resolutions()
    v = np.array([5, 9, 13])
    for l in (0, 3, 7, 15):
        x = v / res[l]
        feat = s.encode(x)
        idx = oracle_mod.grid_index(l, T19, *[int(c) for c in v])
        assert np.allclose(feat[2 * l:2 * l + 2], table[l, idx], atol=1e-12)


def test_sh_orthonormal_by_quadrature(oracle_mod):
    nt, nphi = 24, 48
    ct, wt = np.polynomial.legendre.leggauss(nt)
    gram = np.zeros((16, 16))
    for c, w in zip(ct, wt):
        st = math.sqrt(1 - c * c)
        for k in range(nphi):
            phi = 2 * math.pi * k / nphi
            y = oracle_mod.sh16([st * math.cos(phi), st * math.sin(phi), c])
            gram += np.outer(y, y) * w * (2 * math.pi / nphi)
    assert np.allclose(gram, np.eye(16), atol=1e-10)


# 100% colour bars, ITU-R BT.601 8-bit studio range (Y, Cb, Cr).
COLOUR_BARS = [((255, 255, 255), (235, 128, 128)), ((255, 255, 0), (210, 16, 146)),
               ((0, 255, 255), (170, 166, 16)), ((0, 255, 0), (145, 54, 34)),
               ((255, 0, 255), (106, 202, 222)), ((255, 0, 0), (81, 90, 240)),
               ((0, 0, 255), (41, 240, 110)), ((0, 0, 0), (16, 128, 128))]


@pytest.mark.parametrize("rgb,ycc", COLOUR_BARS)
def test_yuv_colour_bars(oracle_mod, rgb, ycc):
    img = np.tile(np.array(rgb, np.uint8), (4, 4))  # 4x4 flat patch
    y, u, v = oracle_mod.rgb24_to_yuv420p(img, 4, 4, 12, [4, 2, 2])
    assert set(y.tolist()) == {ycc[0]} and set(u.tolist()) == {ycc[1]} and set(v.tolist()) == {ycc[2]}


def test_gray8_is_grey_rgb(oracle_mod):
    g = np.arange(256, dtype=np.uint8).reshape(16, 16)
    rgb = np.repeat(g[:, :, None], 3, axis=2).reshape(16, 48)
    gy, gu, gv = oracle_mod.gray8_to_yuv420p(g, 16, 16, 16, [16, 8, 8])
    y, u, v = oracle_mod.rgb24_to_yuv420p(rgb, 16, 16, 48, [16, 8, 8])
    assert np.array_equal(gy, y)
    assert set(gu.tolist()) == {128} and set(gv.tolist()) == {128}
    assert gy[0] == 16 and gy[-1] == 235


def test_depth_pack_known_answers(oracle_mod):
    d = np.array([0.0, 0.0004, 0.0005, 1.2345, 65.5349, 65.535, 65.6, 1e9, -1.0, np.nan, np.inf, -np.inf],
                 np.float32)
    expect = [0, 0, 1, 1235, 65535, 65535, 65535, 65535, 0, 0, 65535, 0]
    # 1.2345 in FP32 is 1.23450005..., * 1000 -> 1234.5 (rounded) -> 1235.
    assert oracle_mod.depth_pack_u16mm(d).tolist() == expect


def _ray_setup_np(M, W, H, f, px, py):
    """Independent float32 restatement of the ray set-up (numpy float32
    arithmetic rounds every operation, like the CUDA *_rn intrinsics)."""
    f32 = np.float32
    M = np.asarray(M, f32)
    u = (f32(px) + f32(0.5) - f32(0.5) * f32(W)) / f32(f)
    v = (f32(py) + f32(0.5) - f32(0.5) * f32(H)) / f32(f)
    dv = [(M[a * 4] * u + M[a * 4 + 1] * v) + M[a * 4 + 2] for a in range(3)]
    n = np.sqrt((dv[0] * dv[0] + dv[1] * dv[1]) + dv[2] * dv[2])
    d = [x / n for x in dv]
    o = [M[3], M[7], M[11]]
    tn, tf = f32(-np.inf), f32(np.inf)
    with np.errstate(divide="ignore", invalid="ignore"):
        for a in range(3):
            inv = f32(1.0) / d[a]
            t0 = (f32(0.0) - o[a]) * inv
            t1 = (f32(1.0) - o[a]) * inv
            tn = np.fmax(tn, np.fmin(t0, t1))
            tf = np.fmin(tf, np.fmax(t0, t1))
    ts = np.fmax(tn, f32(0.0))
    if not tf > ts:
        return 0, ts
    q = np.floor((tf - ts) / f32(math.sqrt(3) / 1024))
    return (1024 if q >= 1024 else int(q)), ts


def test_ray_setup_matches_float32_restatement(oracle_mod, nes_lib):
    rng = np.random.default_rng(1)
    poses = nes_lib.shell_poses(0, 6, 1.2, 2.0) + [[1, 0, 0, .5, 0, -1, 0, .5, 0, 0, -1, .5]]
    for M in poses:
        W, H = 97, 61
        f = nes_lib.focal_from_fov(W, 100.0)
        for _ in range(200):
            px, py = int(rng.integers(0, W)), int(rng.integers(0, H))
            n, o, d, ts = oracle_mod.ray_setup(M, W, H, f, px, py)
            n2, ts2 = _ray_setup_np(M, W, H, f, px, py)
            assert n == n2 and np.float32(ts) == ts2


def test_camera_inside_cube_marches_to_wall(oracle_mod):
    # The reference's initial pose puts the eye at the cube centre looking
    # down -z (include/base/camera_manager.h:18-19): every ray hits, the
    # centre ray has 0.5 / dt samples.
    M = [1, 0, 0, .5, 0, -1, 0, .5, 0, 0, -1, .5]
    n, o, d, ts = oracle_mod.ray_setup(M, 64, 64, 32.0, 32, 32)
    assert ts == 0.0
    assert d[2] < -0.999 and n == math.floor(0.5 / abs(d[2]) / (math.sqrt(3) / 1024))


def test_render_properties(scene0, nes_lib):
    M = nes_lib.shell_poses(0, 1, 1.5, 1.5)[0]
    rgb, depth, samples = scene0.render(M, 24, 24, nes_lib.focal_from_fov(24, 90.0))
    assert samples > 0
    assert np.all(rgb >= 0) and np.all(rgb <= 1) and np.all(depth >= 0)
    # A corner pixel at 90 deg from r = 1.5 misses the cube: black, depth 0.
    assert np.all(rgb[0] == 0) and depth[0] == 0


def test_oracle_matches_golden_render(scene0):
    g = np.load(os.path.join(GOLDEN, "render_seed0.npz"))
    rgb, depth, samples = scene0.render(g["pose"], int(g["W"]), int(g["H"]), float(g["focal"]))
    assert samples == int(g["samples"])
    assert np.allclose(rgb, g["rgb"], rtol=0, atol=1e-12)
    assert np.allclose(depth, g["depth"], rtol=0, atol=1e-12)


def test_overlay_glyph_placement(oracle_mod):
    # '1' (rows 00100 01100 00100 00100 00100 00100 01110) at 2x, pen at the
    # left-top anchor (50, 50), bottom row on the baseline: 10 set bits -> 40
    # white pixels, top-left set pixel at (54, 36).
    w = h = 100
    out = oracle_mod.overlay_text(np.zeros(h * w * 3, np.uint8), w, h, w * 3, "1", 0).reshape(h, w, 3)
    white = np.argwhere(out[:, :, 0] == 255)
    assert len(white) == 40 and np.all(out[out[:, :, 0] == 255] == 255)
    assert white[:, 0].min() == 36 and white[:, 0].max() == 49
    assert tuple(white[0]) == (36, 54)
    # '\n' returns to the anchor column 20 px lower; unknown glyphs only advance.
    a = oracle_mod.overlay_text(np.zeros(h * w * 3, np.uint8), w, h, w * 3, "#\n1", 0).reshape(h, w, 3)
    assert np.argwhere(a[:, :, 0] == 255)[:, 0].min() == 56


def test_oracle_matches_golden_yuv(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "yuv_small.npz"))
    w, h, ls = int(g["w"]), int(g["h"]), [int(v) for v in g["ls"]]
    y, u, v = oracle_mod.rgb24_to_yuv420p(g["rgb"], w, h, w * 3, ls)
    assert np.array_equal(y, g["y"]) and np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
    gy, gu, gv = oracle_mod.gray8_to_yuv420p(g["gray"], w, h, w, ls)
    assert np.array_equal(gy, g["gy"]) and np.array_equal(gu, g["gu"])
    assert np.array_equal(oracle_mod.depth_pack_u16mm(g["depth"]), g["depth_mm"])


def test_fp32_cpu_render_matches_fp64_oracle(scene0, nes_lib):
    """The plain FP32 CPU render (the bench's CPU baseline) evaluates the same
    samples as the FP64 oracle and agrees with it within the spec
    tolerances (PSNR >= 45 dB, max |delta depth| <= 1e-3)."""
    import numpy as np
    import oracle
    M = nes_lib.shell_poses(0, 3, 1.5, 1.5)[2]
    W, H = 32, 24
    f = nes_lib.focal_from_fov(W, 90.0)
    rgb64, dep64, n64 = scene0.render(M, W, H, f)
    rgb32, dep32, n32 = scene0.render_f32(M, W, H, f)
    assert n32 == n64 > 0
    assert oracle.psnr(rgb32.astype(np.float64), rgb64) >= 45.0
    assert np.abs(dep32.astype(np.float64) - dep64).max() <= 1e-3


def test_renders_independent_of_thread_count(scene0, nes_lib):
    """The oracle and the FP32 CPU render split pixels between threads and
    compute each pixel alone: the same bytes and sample counts for 1, 3 and
    8 threads, over all pixels and over a scattered pixel list."""
    M = nes_lib.shell_poses(4, 1, 1.3, 1.3)[0]
    W, H = 20, 14
    f = nes_lib.focal_from_fov(W, 80.0)
    pix = np.random.default_rng(9).permutation(W * H)[:120].astype(np.int32)
    for fn in (scene0.render, scene0.render_f32):
        for p in (None, pix):
            ref = fn(M, W, H, f, pixels=p, nthreads=1)
            assert ref[2] > 0
            for nt in (3, 8):
                got = fn(M, W, H, f, pixels=p, nthreads=nt)
                assert got[2] == ref[2]
                assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
