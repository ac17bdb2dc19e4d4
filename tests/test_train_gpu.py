"""GPU training path (nes_trainer_*): the FP32 loss and gradient against
the FP64 oracle's reverse-mode gradient on the same rays, against central
finite differences of the GPU's own FP64 loss, the Adam step, the refit's
loss curve and the error paths.

Tolerances: loss relative 1e-5; gradients (FP32 accumulation with atomics
in nondeterministic order against FP64) relative L2 error <= 1e-4 per
parameter block and |delta| <= 1e-3 of the block's largest entry; finite
differences relative 1e-3.  `exact_weight_grads=1` (per-sample MLP recompute,
backpropagation and weight gradients in FP32 on the CUDA cores) is held to
these FP32 tolerances throughout.  The default runs the ten per-sample layer
products and the weight-gradient GEMMs on the tensor cores in TF32 (10-bit
mantissa operands, FP32 accumulation).  Against the FP32 path on 4,096 rays
it is held to relative L2 2e-2 and 5e-2 of the block's largest entry
(TF32_REL, TF32_PEAK; measured 0.2-0.5 %).  Against the FP64 oracle on 64
rays the fine levels' entries each gather one or two samples, and a hidden
unit whose TF32 pre-activation lands on the other side of zero than in FP32
changes that sample's whole contribution: measured 0.2-1.9 % relative L2 and
up to 15 % of a block's largest entry, held to ORACLE_TF32 = (3e-2, 0.25).
The loss keeps the FP32 tolerance in both modes: the default evaluates the
forward with 3xTF32 products (TF32 high part and FP32 remainder of every
operand, three products per layer), FP32-level accuracy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOG2T = 14
TABLE_FLOATS = 16 * (1 << LOG2T) * 2
W = H = 16
BLOCKS = {"dw1": (0, 2048), "dw2": (2048, 3072), "cw1": (3072, 5120), "cw2": (5120, 9216), "cw3": (9216, 9408)}


def _views(nes_lib):
    f = nes_lib.focal_from_fov(W, 30.0)
    return [(M, W, H, f) for M in nes_lib.shell_poses(1, 2, 1.3, 1.6)]


@pytest.fixture(scope="module")
def setup(nes_lib, cuda):
    torch = cuda
    views = _views(nes_lib)
    nv = len(views)
    # Teacher (seed 1) renders the targets into device buffers.
    teacher = nes_lib.Renderer(precision=nes_lib.PREC_FP32, seed=1, log2_table_size=LOG2T, max_pixels=nv * W * H)
    rgb = torch.empty((nv * W * H, 3), device="cuda", dtype=torch.float32)
    dep = torch.empty((nv * W * H,), device="cuda", dtype=torch.float32)
    teacher.render_views([nes_lib.make_view(*v) for v in views],
                         [rgb[i * W * H:].data_ptr() for i in range(nv)], [dep[i * W * H:].data_ptr() for i in range(nv)])
    torch.cuda.synchronize()
    teacher.close()
    yield views, rgb, dep


def _student(nes_lib, setup, **kw):
    views, rgb, dep = setup
    r = nes_lib.Renderer(precision=nes_lib.PREC_FP32, seed=2, log2_table_size=LOG2T, max_pixels=W * H * 4)
    cfg = dict(batch_rays=4096)
    cfg.update(kw)
    t = nes_lib.Trainer(r, **cfg)
    t.set_targets([nes_lib.make_view(*v) for v in views], rgb.data_ptr(), dep.data_ptr())
    return r, t


def _pairs(n, nviews, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, nviews, n), rng.integers(0, W * H, n)], 1).astype(np.int32)


def _oracle_grad(oracle_mod, r, views, pairs, rgb, dep):
    sc = oracle_mod.Scene(2, LOG2T)
    occ = r.occupancy()
    rays = sc.rays(views, pairs)
    rgb_h, dep_h = rgb.cpu().numpy(), dep.cpu().numpy()
    q = pairs[:, 0] * W * H + pairs[:, 1]
    target = np.concatenate([rgb_h[q].astype(np.float64), dep_h[q, None].astype(np.float64)], 1)
    # Sample positions and grid cells rounded as the kernels round them:
    # FP64 positions alone move the fine-level gradients by up to a few % at
    # samples whose cell flips (checked on the CPU: dw1 by 3e-4 relative).
    loss, gt, gw = sc.loss_grad(rays, target, depth_w=0.1, occ=occ, fp32_positions=True)
    # Samples the oracle evaluates on those rays, for the exact count check.
    import ctypes
    o, d, ts, ns = rays
    lib = oracle_mod.load()
    occ_arr = np.ascontiguousarray(occ, np.uint32)
    count = 0
    buf = np.zeros(3)
    dd = np.zeros(1)
    for i in range(len(ns)):
        count += lib.oracle_march_ray(sc.h, occ_arr.ctypes.data, o[i].ctypes.data, d[i].ctypes.data, float(ts[i]),
                                      int(ns[i]), buf.ctypes.data, dd.ctypes.data, None)
    return loss, gt, gw, count


def _errs(a, b):
    """(relative L2 error, max |a - b| / max |b|)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb, mb = np.linalg.norm(b), np.abs(b).max()
    return (np.linalg.norm(a - b) / nb if nb else np.linalg.norm(a), np.abs(a - b).max() / mb if mb else 0.0)


TF32_REL, TF32_PEAK = 2e-2, 5e-2
ORACLE_TF32 = (3e-2, 0.25)


def _close(a, b, rel=1e-4, peak=1e-3):
    e_rel, e_peak = _errs(a, b)
    return e_rel <= rel and e_peak <= peak


@pytest.mark.parametrize("exact", [1, 0])
def test_gradient_matches_oracle(nes_lib, oracle_mod, setup, exact):
    views, rgb, dep = setup
    r, t = _student(nes_lib, setup, exact_weight_grads=exact)
    rel, peak = (1e-4, 1e-3) if exact else ORACLE_TF32
    pairs = _pairs(64, len(views), 3)
    loss, gt, gw = t.grad(pairs, TABLE_FLOATS)
    samples = t.last_samples()
    oloss, ogt, ogw, ocount = _oracle_grad(oracle_mod, r, views, pairs, rgb, dep)
    assert samples == ocount
    assert abs(loss - oloss) <= 1e-5 * oloss
    errs = {name: _errs(gw[a:b], ogw[a:b]) for name, (a, b) in BLOCKS.items()}
    for lvl in range(16):
        seg = slice(lvl * (1 << LOG2T) * 2, (lvl + 1) * (1 << LOG2T) * 2)
        errs[lvl] = _errs(gt[seg], ogt[seg])
    print("gradient errors vs FP64 oracle (exact=%d):" % exact,
          {k: (round(float(a), 6), round(float(b), 6)) for k, (a, b) in errs.items()})
    bad = [(k, e) for k, e in errs.items() if not (e[0] <= rel and e[1] <= peak)]
    assert not bad, bad
    # The gradient call changes nothing: a second call gives the same loss.
    loss2, _, _ = t.grad(pairs, TABLE_FLOATS)
    assert abs(loss2 - loss) <= 1e-6 * loss
    t.close()
    r.close()


def test_gradient_matches_gpu_finite_differences(nes_lib, setup):
    views, rgb, dep = setup
    r, t = _student(nes_lib, setup, exact_weight_grads=1)
    pairs = _pairs(128, len(views), 4)
    loss, gt, gw = t.grad(pairs, TABLE_FLOATS)
    l64 = t.loss_fp64(pairs)
    assert abs(l64 - loss) <= 1e-5 * l64
    checks = []
    rng = np.random.default_rng(1)
    for a, b in BLOCKS.values():
        order = a + np.argsort(-np.abs(gw[a:b]))
        checks += [(1, int(i), gw[i]) for i in order[:6]] + [(1, int(i), gw[i]) for i in rng.integers(a, b, 2)]
    for lvl in (0, 4, 8, 12, 15):
        seg = gt[lvl * (1 << LOG2T) * 2:(lvl + 1) * (1 << LOG2T) * 2]
        order = np.argsort(-np.abs(seg))[:4] + lvl * (1 << LOG2T) * 2
        checks += [(0, int(i), gt[i]) for i in order]
    # Every +-h evaluation for both step sizes in one launch.
    hs = (1e-3, 1e-4)
    wh = [c[0] for c in checks] * 4
    ix = [c[1] for c in checks] * 4
    dl = [sgn * h for h in hs for sgn in (1.0, -1.0) for _ in checks]
    ls = t.loss_fp64_batch(pairs, wh, ix, dl).reshape(len(hs), 2, len(checks))
    bad = []
    for j, (which, idx, g) in enumerate(checks):
        errs = [abs((ls[k, 0, j] - ls[k, 1, j]) / (2 * h) - g) for k, h in enumerate(hs)]
        if min(errs) > 1e-3 * abs(g) + 1e-9:
            bad.append((which, idx, g, min(errs)))
    assert not bad, bad
    t.close()
    r.close()


def test_tensor_core_weight_gradients_match_exact(nes_lib, setup):
    """4,096 rays (~0.9 M samples, ~28 k weight-gradient tiles, ~7 k
    backward tiles): every CTA of the TF32 kernels wraps its loop many times
    and ends on a partial tile."""
    views, rgb, dep = setup
    pairs = _pairs(4096, len(views), 7)
    out = {}
    for exact in (1, 0):
        r, t = _student(nes_lib, setup, exact_weight_grads=exact)
        out[exact] = t.grad(pairs, TABLE_FLOATS)
        t.close()
        r.close()
    (l1, gt1, gw1), (l0, gt0, gw0) = out[1], out[0]
    # The tensor-core mode evaluates the forward with 3xTF32 products, the
    # exact mode in FP32 on the CUDA cores: their losses agree to the bar both
    # meet against the FP64 oracle (measured: 3e-6 relative on these rays).
    assert l0 == pytest.approx(l1, rel=1e-5)
    print("tensor-core vs FP32 gradients: table", _errs(gt0, gt1),
          {name: _errs(gw0[a:b], gw1[a:b]) for name, (a, b) in BLOCKS.items()})
    assert _close(gt0, gt1, TF32_REL, TF32_PEAK), _errs(gt0, gt1)
    bad = [(name, _errs(gw0[a:b], gw1[a:b])) for name, (a, b) in BLOCKS.items()
           if not _close(gw0[a:b], gw1[a:b], TF32_REL, TF32_PEAK)]
    assert not bad, bad


def test_adam_first_step_moves_by_lr(nes_lib, setup):
    views, rgb, dep = setup
    r, t = _student(nes_lib, setup, lr=1e-3)
    pairs = _pairs(256, len(views), 5)
    _, gt, gw = t.grad(pairs, TABLE_FLOATS)
    w0 = np.concatenate([r.scene_param(k, n) for k, n in zip(range(1, 6), (2048, 1024, 2048, 4096, 192))])
    t0 = r.scene_param(0, TABLE_FLOATS)
    t.step_rays(pairs)
    w1 = np.concatenate([r.scene_param(k, n) for k, n in zip(range(1, 6), (2048, 1024, 2048, 4096, 192))])
    t1 = r.scene_param(0, TABLE_FLOATS)
    # Step 1 of Adam: m^ = g, v^ = g^2 -> delta = -lr g / (|g| + eps) = -lr sign(g).
    for p0, p1, g in ((w0, w1, gw), (t0, t1, gt)):
        big = np.abs(g) > 1e-7
        assert big.sum() > 10
        assert np.allclose((p1 - p0)[big], -1e-3 * np.sign(g[big]), rtol=1e-3, atol=2e-7)
        assert np.array_equal(p1[g == 0], p0[g == 0])
    t.close()
    r.close()


def test_refit_loss_decreases(nes_lib, setup):
    views, rgb, dep = setup
    r, t = _student(nes_lib, setup, batch_rays=2048)
    losses = [t.step(seed) for seed in range(40)]
    assert all(np.isfinite(losses))
    assert np.mean(losses[-5:]) < 0.6 * np.mean(losses[:3]), losses
    t.close()
    r.close()


def test_trainer_errors(nes_lib, setup, cuda):
    views, rgb, dep = setup
    tc = nes_lib.Renderer(precision=nes_lib.PREC_FP16_TC, seed=2, log2_table_size=LOG2T, max_pixels=W * H)
    with pytest.raises(nes_lib.NesError):
        nes_lib.Trainer(tc)
    tc.close()
    r = nes_lib.Renderer(precision=nes_lib.PREC_FP32, seed=2, log2_table_size=LOG2T, max_pixels=W * H)
    with pytest.raises(nes_lib.NesError):
        nes_lib.Trainer(r, batch_rays=0)
    t = nes_lib.Trainer(r, batch_rays=64)
    with pytest.raises(nes_lib.NesError):  # no targets yet
        t.step(0)
    t.set_targets([nes_lib.make_view(*v) for v in views], rgb.data_ptr(), dep.data_ptr())
    with pytest.raises(nes_lib.NesError):  # more rays than the batch
        t.step_rays(_pairs(65, len(views), 0))
    with pytest.raises(nes_lib.NesError):  # view index out of range
        t.step_rays(np.array([[len(views), 0]], np.int32))
    with pytest.raises(nes_lib.NesError):  # pixel out of range
        t.grad(np.array([[0, W * H]], np.int32), TABLE_FLOATS)
    with pytest.raises(nes_lib.NesError):
        t.loss_fp64(_pairs(4, len(views), 0), which=1, index=9408)
    # Still usable after the rejected calls.
    assert np.isfinite(t.step_rays(_pairs(64, len(views), 1)))
    t.close()
    r.close()


@pytest.mark.parametrize("exact", [1, 0])
def test_batch_whose_rays_all_miss(nes_lib, cuda, exact):
    """Rays of a view that looks away from the volume: no samples, so the
    sample list, the records and the backward chunks are all empty; the loss
    is the targets' own (student and teacher both render 0 there), the
    gradient is 0, and a batch mixing such rays with hitting ones gives the
    hitting rays' gradient scaled by the batch size."""
    torch = cuda
    away = (nes_lib.look_at((0.5, 0.5, 3.0), (0.5, 0.5, 6.0)), W, H, nes_lib.focal_from_fov(W, 30.0))
    views = _views(nes_lib) + [away]
    nv = len(views)
    teacher = nes_lib.Renderer(precision=nes_lib.PREC_FP32, seed=1, log2_table_size=LOG2T, max_pixels=nv * W * H)
    rgb = torch.empty((nv * W * H, 3), device="cuda", dtype=torch.float32)
    dep = torch.empty((nv * W * H,), device="cuda", dtype=torch.float32)
    teacher.render_views([nes_lib.make_view(*v) for v in views],
                         [rgb[i * W * H:].data_ptr() for i in range(nv)], [dep[i * W * H:].data_ptr() for i in range(nv)])
    torch.cuda.synchronize()
    teacher.close()
    r, t = _student(nes_lib, (views, rgb, dep), exact_weight_grads=exact)
    try:
        miss = np.stack([np.full(64, nv - 1), np.arange(64) % (W * H)], 1).astype(np.int32)
        loss, gt, gw = t.grad(miss, TABLE_FLOATS)
        assert t.last_samples() == 0
        assert loss == 0.0 and not gt.any() and not gw.any()
        hits = _pairs(64, nv - 1, 11)
        lh, gth, gwh = t.grad(hits, TABLE_FLOATS)
        lm, gtm, gwm = t.grad(np.concatenate([hits, miss]), TABLE_FLOATS)
        # The loss is a mean over the batch: the missing rays add 0 and halve it.
        assert lm == pytest.approx(lh / 2, rel=1e-6)
        assert _close(2 * gtm, gth, 1e-5, 1e-4) and _close(2 * gwm, gwh, 1e-5, 1e-4)
    finally:
        t.close()
        r.close()
