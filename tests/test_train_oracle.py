"""Pins the oracle's training gradient (FP64 reverse-mode sweeps) against
central finite differences of its own FP64 loss, before the GPU gradient is
checked against it.  CPU only."""
import numpy as np
import pytest

LOG2T = 14


def _setup(oracle_mod, nes_lib, nrays=8, seed=5):
    sc = oracle_mod.Scene(2, LOG2T)
    M = nes_lib.shell_poses(1, 1, 1.4, 1.4)[0]
    W = H = 16
    f = nes_lib.focal_from_fov(W, 30.0)
    views = [(M, W, H, f)]
    rng = np.random.default_rng(seed)
    pairs = np.stack([np.zeros(nrays, np.int32), rng.integers(0, W * H, nrays).astype(np.int32)], 1)
    rays = sc.rays(views, pairs)
    assert np.all(rays[3] > 0), "test rays must hit the cube"
    target = np.concatenate([rng.uniform(0, 1, (nrays, 3)), rng.uniform(1.0, 2.0, (nrays, 1))], 1)
    return sc, rays, target


def _fd(sc, rays, target, which, index, h):
    """Central difference in FP64 of the loss over the FP32-stored parameter;
    the applied steps are the exact FP32 differences."""
    if which == 0:
        arr, setter = sc.param(0), lambda a: sc.set_param(0, a)
    else:
        arr, setter = sc.weights_blob(), sc.set_weights_blob
    p0 = arr[index]
    hi, lo = np.float32(p0 + h), np.float32(p0 - h)
    a = arr.copy()
    a[index] = hi
    setter(a)
    lp = sc.loss_grad(rays, target, grad=False)
    a[index] = lo
    setter(a)
    lm = sc.loss_grad(rays, target, grad=False)
    setter(arr)
    return (lp - lm) / (float(hi) - float(lo))


def _fd_err(sc, rays, target, which, index, g):
    """Smallest |FD - g| over three step sizes: a step that straddles a ReLU
    kink of any sample spoils one size, not all three."""
    return min(abs(_fd(sc, rays, target, which, index, h) - g) for h in (1e-4, 1e-5, 1e-6))


def test_oracle_gradient_matches_finite_differences(oracle_mod, nes_lib):
    sc, rays, target = _setup(oracle_mod, nes_lib)
    loss, gt, gw = sc.loss_grad(rays, target)
    assert loss > 0 and np.isfinite(loss)
    # Weights: the largest entries of every layer plus a few random ones.
    offs = [0, 2048, 3072, 5120, 9216, 9408]
    rng = np.random.default_rng(0)
    picks = []
    for a, b in zip(offs[:-1], offs[1:]):
        picks.append(a + int(np.argmax(np.abs(gw[a:b]))))
        picks.append(int(rng.integers(a, b)))
    for i in picks:
        err = _fd_err(sc, rays, target, 1, i, gw[i])
        assert err <= 1e-5 * abs(gw[i]) + 1e-10, (i, err, gw[i])
    # Table: the largest gradients of a coarse and a fine level.
    for lvl in (0, 9, 15):
        seg = slice(lvl * (1 << LOG2T) * 2, (lvl + 1) * (1 << LOG2T) * 2)
        i = seg.start + int(np.argmax(np.abs(gt[seg])))
        err = _fd_err(sc, rays, target, 0, i, gt[i])
        assert err <= 1e-5 * abs(gt[i]) + 1e-10, (lvl, i, err, gt[i])


def test_oracle_gradient_zero_when_target_is_own_render(oracle_mod, nes_lib):
    sc, rays, _ = _setup(oracle_mod, nes_lib, nrays=4)
    # Target = the scene's own render of those rays: loss 0 and gradient 0.
    o, d, ts, ns = rays
    tgt = np.zeros((4, 4))
    for i in range(4):
        rgb = np.zeros(3)
        dep = np.zeros(1)
        oracle_mod.load().oracle_march_ray(sc.h, None, o[i].ctypes.data, d[i].ctypes.data, float(ts[i]), int(ns[i]),
                                           rgb.ctypes.data, dep.ctypes.data, None)
        tgt[i, :3], tgt[i, 3] = rgb, dep[0]
    loss, gt, gw = sc.loss_grad(rays, tgt)
    assert loss < 1e-28 and np.abs(gt).max() < 1e-14 and np.abs(gw).max() < 1e-14
