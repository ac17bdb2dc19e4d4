"""The differentiation form as configured: teacher scene seed 1 and student
seed 2 (T = 2^19), 64 teacher views of 800x800 (60 deg FOV, r = 1.2..2.0
shell).  The hand-written gradient is checked

  - against central FP64 finite differences (h = 1e-4) of the GPU's own FP64
    loss on 1,024 seeded random parameters: 100 in each of the five weight
    blocks and 524 table entries spread over the 16 levels (entries that the
    batch's samples touch, plus untouched ones whose gradient must be 0);
  - against the FP64 oracle's reverse-mode gradient on a 64-ray batch, in
    both modes: FP32 (exact_weight_grads = 1) to relative L2 1e-4 and 1e-3
    of each block's largest entry; the default tensor-core mode (TF32
    operands): each weight block (a sum over every sample) to 1e-2 relative
    L2 and 1e-2 of its largest entry, each table level to 3e-2 relative L2
    and, on entries fed by at least SUPPORT_MIN samples, to 5e-2 of the
    level's largest entry.  Entries fed by one or two
    samples are left to the L2 bound: where a hidden unit's pre-activation
    lands on the other side of zero in TF32 than in FP32, that sample's whole
    contribution changes.  The loss is held to 1e-5 relative in both modes
    (the default's forward evaluates its products as 3xTF32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOG2T = 19
T = 1 << LOG2T
TABLE_FLOATS = 16 * T * 2
SIDE = 800
NVIEWS = 64
BLOCKS = {"dw1": (0, 2048), "dw2": (2048, 3072), "cw1": (3072, 5120), "cw2": (5120, 9216), "cw3": (9216, 9408)}
RES = [16, 22, 30, 42, 58, 80, 111, 153, 212, 294, 406, 561, 776, 1072, 1482, 2048]
P1, P2 = np.uint32(2654435761), np.uint32(805459861)
SUPPORT_MIN = 8
# Tensor-core mode against the oracle (measured on this batch: weight blocks
# 0.2-0.5 % relative L2 and of the block's largest entry; table levels
# 0.4-1.9 % relative L2, at most 4.5 % of the level's largest entry on
# entries fed by >= 8 samples, up to 10 % on entries fed by fewer).
TC_W_REL, TC_W_PEAK = 1e-2, 1e-2
TC_REL, TC_PEAK = 3e-2, 5e-2


def _views(nes_lib):
    f = nes_lib.focal_from_fov(SIDE, 60.0)
    return [(M, SIDE, SIDE, f) for M in nes_lib.shell_poses(11, NVIEWS, 1.2, 2.0)]


@pytest.fixture(scope="module")
def teacher(nes_lib, cuda):
    torch = cuda
    views = _views(nes_lib)
    px = SIDE * SIDE
    rgb = torch.empty((NVIEWS * px, 3), device="cuda", dtype=torch.float32)
    dep = torch.empty((NVIEWS * px,), device="cuda", dtype=torch.float32)
    with nes_lib.Renderer(precision=nes_lib.PREC_FP32, seed=1, log2_table_size=LOG2T,
                          max_pixels=NVIEWS * px) as r:
        r.render_views([nes_lib.make_view(*v) for v in views], [rgb[i * px:].data_ptr() for i in range(NVIEWS)],
                       [dep[i * px:].data_ptr() for i in range(NVIEWS)])
        torch.cuda.synchronize()
    yield views, rgb, dep


def _student(nes_lib, teacher, **kw):
    views, rgb, dep = teacher
    r = nes_lib.Renderer(precision=nes_lib.PREC_FP32, seed=2, log2_table_size=LOG2T, max_pixels=SIDE * SIDE)
    cfg = dict(batch_rays=4096)
    cfg.update(kw)
    t = nes_lib.Trainer(r, **cfg)
    t.set_targets([nes_lib.make_view(*v) for v in views], rgb.data_ptr(), dep.data_ptr())
    return r, t


def _pairs(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, NVIEWS, n), rng.integers(0, SIDE * SIDE, n)], 1).astype(np.int32)


def _errs(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb, mb = np.linalg.norm(b), np.abs(b).max()
    return (np.linalg.norm(a - b) / nb if nb else np.linalg.norm(a), np.abs(a - b).max() / mb if mb else 0.0)


def _table_support(rays, dt):
    """Samples touching each table entry (float2 index l*T + e) for the
    batch's rays, positions in FP32 as the kernels place them (every sample
    of this scene is occupied and no ray terminates early)."""
    o, d, ts, ns = rays
    counts = np.zeros(16 * T, np.int64)
    for i in range(len(ns)):
        k = np.arange(int(ns[i]), dtype=np.float32)
        t = ((k + np.float32(0.5)) * np.float32(dt) + np.float32(ts[i])).astype(np.float32)
        x = np.clip(o[i][None, :] + t[:, None] * d[i][None, :], 0.0, 1.0).astype(np.float32)
        for lvl, n in enumerate(RES):
            c = np.minimum(np.floor(x * np.float32(n)).astype(np.int64), n - 1).astype(np.uint32)
            dense = (n + 1) ** 3 <= T
            for corner in range(8):
                cx = c[:, 0] + np.uint32(corner & 1)
                cy = c[:, 1] + np.uint32((corner >> 1) & 1)
                cz = c[:, 2] + np.uint32((corner >> 2) & 1)
                if dense:
                    e = cx + np.uint32(n + 1) * (cy + np.uint32(n + 1) * cz)
                else:
                    e = (cx ^ (cy * P1) ^ (cz * P2)) & np.uint32(T - 1)
                np.add.at(counts, lvl * T + e.astype(np.int64), 1)
    return counts


@pytest.mark.parametrize("exact", [1, 0])
def test_gradient_vs_oracle_64_rays(nes_lib, oracle_mod, teacher, cuda, exact):
    torch = cuda
    views, rgb, dep = teacher
    r, t = _student(nes_lib, teacher, exact_weight_grads=exact)
    try:
        pairs = _pairs(64, 3)
        loss, gt, gw = t.grad(pairs, TABLE_FLOATS)
        samples = t.last_samples()
        occ = r.occupancy()
    finally:
        t.close()
        r.close()
    sc = oracle_mod.Scene(2, LOG2T)
    rays = sc.rays(views, pairs)
    q = torch.from_numpy((pairs[:, 0].astype(np.int64) * SIDE * SIDE + pairs[:, 1])).cuda()
    rgb_h = rgb.index_select(0, q).cpu().numpy()
    dep_h = dep.index_select(0, q).cpu().numpy()
    target = np.concatenate([rgb_h.astype(np.float64), dep_h[:, None].astype(np.float64)], 1)
    oloss, ogt, ogw = sc.loss_grad(rays, target, depth_w=0.1, occ=occ, fp32_positions=True)
    # The samples the oracle marches on those rays, exactly.
    lib = oracle_mod.load()
    o, d, ts, ns = rays
    occ_arr = np.ascontiguousarray(occ, np.uint32)
    buf, dd = np.zeros(3), np.zeros(1)
    count = sum(lib.oracle_march_ray(sc.h, occ_arr.ctypes.data, o[i].ctypes.data, d[i].ctypes.data, float(ts[i]),
                                     int(ns[i]), buf.ctypes.data, dd.ctypes.data, None) for i in range(len(ns)))
    assert samples == count
    assert abs(loss - oloss) <= 1e-5 * oloss
    support = np.repeat(_table_support(rays, oracle_mod.dt()), 2)  # per float of the table
    report, bad = {}, []
    for name, (a, b) in BLOCKS.items():
        e = _errs(gw[a:b], ogw[a:b])
        report[name] = e
        lim = (1e-4, 1e-3) if exact else (TC_W_REL, TC_W_PEAK)
        if not (e[0] <= lim[0] and e[1] <= lim[1]):
            bad.append((name, e))
    for lvl in range(16):
        seg = slice(lvl * T * 2, (lvl + 1) * T * 2)
        g, og, sup = gt[seg], ogt[seg], support[seg]
        rel, peak = _errs(g, og)
        mx = np.abs(og).max()
        well = sup >= SUPPORT_MIN
        peak_well = float(np.abs(g[well] - og[well]).max() / mx) if well.any() and mx else 0.0
        report[lvl] = (rel, peak, peak_well, int(well.sum()), int((sup > 0).sum()))
        if exact:
            if not (rel <= 1e-4 and peak <= 1e-3):
                bad.append((lvl, report[lvl]))
        elif not (rel <= TC_REL and peak_well <= TC_PEAK):
            bad.append((lvl, report[lvl]))
    print("gradient vs FP64 oracle, exact=%d:" % exact,
          {k: tuple(round(float(x), 6) if isinstance(x, float) else x for x in v) for k, v in report.items()})
    assert not bad, bad


def test_finite_differences_1024_params(nes_lib, oracle_mod, teacher):
    """Central FP64 differences with h = 1e-4 on 1,024 seeded random
    parameters, on 64 rays.  Each check allows 1e-3 of the gradient, plus
    1e-3 of the largest gradient in the parameter's block (weight block or
    table level: the FP32 gradient is a sum of thousands of per-sample terms
    of both signs -- a coarse level's entry gathers every sample of its large
    cells -- so a small entry carries an absolute error of a few parts in 1e4
    of the block's largest; measured worst 6e-4, on a level-1 entry), plus
    twice the difference's own truncation error, estimated from a second
    central difference at h / 2.  A parameter whose loss has a kink inside
    [-h, h] (a ReLU pre-activation or a cell boundary crossing zero there)
    has no derivative for the difference to match: such a parameter is
    recognised by its two one-sided differences disagreeing, and at most 1 %
    of the checks may be kinks."""
    views, rgb, dep = teacher
    r, t = _student(nes_lib, teacher, exact_weight_grads=1)
    try:
        pairs = _pairs(64, 4)
        loss, gt, gw = t.grad(pairs, TABLE_FLOATS)
        l0 = t.loss_fp64(pairs)
        assert abs(l0 - loss) <= 1e-5 * l0
        rng = np.random.default_rng(1024)
        checks = []
        for a, b in BLOCKS.values():
            scale = float(np.abs(gw[a:b]).max())
            checks += [(1, int(i), float(gw[i]), scale) for i in rng.choice(np.arange(a, b), 100, replace=False)]
        touched = np.flatnonzero(gt)
        per_level = []
        for lvl in range(16):
            lo, hi = lvl * T * 2, (lvl + 1) * T * 2
            cand = touched[(touched >= lo) & (touched < hi)]
            per_level.append(cand)
        quota = [33] * 12 + [32] * 4  # 524 table entries
        for lvl, cand in enumerate(per_level):
            n_touch = min(len(cand), quota[lvl] - 2)
            pick = list(rng.choice(cand, n_touch, replace=False)) if n_touch > 0 else []
            lo = lvl * T * 2
            while len(pick) < quota[lvl]:  # untouched entries: gradient 0
                i = int(rng.integers(lo, lo + T * 2))
                if gt[i] == 0.0 and i not in pick:
                    pick.append(i)
            scale = float(np.abs(gt[lo:lo + T * 2]).max())
            checks += [(0, int(i), float(gt[i]), scale) for i in pick]
        assert len(checks) == 1024
        h = 1e-4
        # Every +h and -h evaluation in one launch (one block of rays each).
        wh = [c[0] for c in checks] * 2
        ix = [c[1] for c in checks] * 2
        dl = [h] * len(checks) + [-h] * len(checks)
        ls = t.loss_fp64_batch(pairs, wh, ix, dl)
        # The same at h / 2: the difference of the two estimates measures the
        # O(h^2) truncation error of the h = 1e-4 difference (~1e-9 here,
        # several parts in 1e4 of a weight block's largest gradient).
        ls2 = t.loss_fp64_batch(pairs, wh, ix, [d / 2 for d in dl])
        # The batched form agrees with single evaluations.
        for j in (0, 517, 1023):
            assert ls[j] == pytest.approx(t.loss_fp64(pairs, checks[j][0], checks[j][1], h), rel=1e-12)
        fails, kinks = [], []
        worst = 0.0
        for j, (which, idx, g, scale) in enumerate(checks):
            lp, lm = ls[j], ls[len(checks) + j]
            fd = (lp - lm) / (2 * h)
            fd2 = (ls2[j] - ls2[len(checks) + j]) / h
            tol = 1e-3 * abs(g) + 1e-3 * scale + 2.0 * abs(fd - fd2) + 1e-12
            right, left = (lp - l0) / h, (l0 - lm) / h
            if abs(fd - g) > tol and abs(right - left) > 10 * tol:
                kinks.append((which, idx, g, fd, left, right))
                continue
            worst = max(worst, abs(fd - g) / tol)
            if abs(fd - g) > tol:
                fails.append((which, idx, g, fd))
        print("FD: %d checks, %d kinks, %d failures, worst error / tolerance %.3f"
              % (len(checks), len(kinks), len(fails), worst))
        assert not fails, fails[:10]
        assert len(kinks) <= 10, kinks
    finally:
        t.close()
        r.close()
