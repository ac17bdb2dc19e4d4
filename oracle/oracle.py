"""ctypes wrapper of the CPU oracle (oracle/nes_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py, always as the checker or the timed CPU
baseline, never on the product path.  Parity is unpinned against reference
output (the reference ships no renderer, no swscale call that can run here,
and no test vectors); see the header of nes_oracle.c for what pins it.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_P = ctypes.c_void_p
_SIGS = {
    "oracle_scene_new": (_P, [ctypes.c_uint64, ctypes.c_uint32]),
    "oracle_scene_free": (None, [_P]),
    "oracle_scene_param": (_P, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "oracle_scene_set_param": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t]),
    "oracle_resolutions": (None, [_P]),
    "oracle_dt": (ctypes.c_float, []),
    "oracle_grid_index": (ctypes.c_uint32, [ctypes.c_uint32] * 5),
    "oracle_encode": (None, [_P, _P, _P]),
    "oracle_sh16": (None, [_P, _P]),
    "oracle_query": (None, [_P, _P, _P, _P, _P]),
    "oracle_density": (ctypes.c_double, [_P, _P]),
    "oracle_ray_setup": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                        ctypes.c_int, _P, _P, _P]),
    "oracle_occupancy": (None, [_P, ctypes.c_double, _P, ctypes.c_int]),
    "oracle_march_ray": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_float, ctypes.c_int, _P, _P, _P]),
    "oracle_render": (ctypes.c_longlong, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_float, _P,
                                          ctypes.c_long, _P, _P, ctypes.c_int]),
    "oracle_rgb24_to_yuv420p": (None, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P]),
    "oracle_gray8_to_yuv420p": (None, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P]),
    "oracle_depth_pack_u16mm": (None, [_P, ctypes.c_long, _P]),
    "oracle_depth_to_gray8": (None, [_P, ctypes.c_long, ctypes.c_float, _P]),
    "oracle_rgb_to_rgb24": (None, [_P, ctypes.c_long, _P]),
    "oracle_stream_key": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_uint32]),
    "oracle_overlay_text": (None, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]),
    "oracle_render_f32": (ctypes.c_longlong, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_float, _P,
                                              ctypes.c_long, _P, _P, ctypes.c_int]),
    "oracle_train_loss_grad": (ctypes.c_double, [_P, _P, _P, _P, _P, _P, ctypes.c_int, _P, ctypes.c_double,
                                                 ctypes.c_int, _P, _P]),
}


def overlay_text(rgb, w, h, ls, text, anchor):
    """Draws text into a copy of the RGB24 frame (uint8, h*ls bytes)."""
    out = np.ascontiguousarray(rgb, dtype=np.uint8).copy()
    load().oracle_overlay_text(out.ctypes.data, w, h, ls, text.encode(), anchor)
    return out

_lib = None


def load():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build_oracle.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        lib = ctypes.CDLL(mod.build())
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None else None


PARAM_NAMES = ["table", "dw1", "dw2", "cw1", "cw2", "cw3"]


class Scene:
    """The seeded scene, generated independently of the product."""

    def __init__(self, seed=0, log2T=19):
        self.lib = load()
        self.h = self.lib.oracle_scene_new(seed, log2T)
        if not self.h:
            raise ValueError("bad scene parameters")
        self.seed, self.log2T = seed, log2T

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_scene_free(self.h)
            self.h = None

    def param(self, which):
        n = ctypes.c_size_t(0)
        p = self.lib.oracle_scene_param(self.h, which, ctypes.byref(n))
        buf = (ctypes.c_float * n.value).from_address(p)
        return np.frombuffer(buf, dtype=np.float32).copy()

    def set_param(self, which, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float32)
        if self.lib.oracle_scene_set_param(self.h, which, arr.ctypes.data, arr.size) != 0:
            raise ValueError("size mismatch")

    def encode(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(32, dtype=np.float64)
        self.lib.oracle_encode(self.h, x.ctypes.data, out.ctypes.data)
        return out

    def query(self, x, d):
        x = np.ascontiguousarray(x, dtype=np.float64)
        d = np.ascontiguousarray(d, dtype=np.float64)
        sigma = ctypes.c_double(0)
        rgb = np.empty(3, dtype=np.float64)
        self.lib.oracle_query(self.h, x.ctypes.data, d.ctypes.data, ctypes.byref(sigma), rgb.ctypes.data)
        return sigma.value, rgb

    def occupancy(self, threshold=0.0, nthreads=None):
        bits = np.zeros(65536, dtype=np.uint32)
        self.lib.oracle_occupancy(self.h, threshold, bits.ctypes.data, nthreads or os.cpu_count() or 1)
        return bits

    def render(self, matrix, W, H, focal, pixels=None, occ=None, nthreads=None):
        """FP64 render.  Returns (rgb [n,3] f64, depth [n] f64, samples)."""
        M = np.ascontiguousarray(matrix, dtype=np.float32)
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels, dtype=np.int32)
            n = pixels.size
        else:
            n = W * H
        rgb = np.empty((n, 3), dtype=np.float64)
        depth = np.empty(n, dtype=np.float64)
        occ_arr = None if occ is None else np.ascontiguousarray(occ, dtype=np.uint32)
        samples = self.lib.oracle_render(self.h, _ptr(occ_arr), M.ctypes.data, W, H, focal, _ptr(pixels), n,
                                         rgb.ctypes.data, depth.ctypes.data, nthreads or os.cpu_count() or 1)
        return rgb, depth, samples

    def render_f32(self, matrix, W, H, focal, pixels=None, occ=None, nthreads=None):
        """Plain FP32 CPU render (a speed baseline, not the checker).
        Returns (rgb [n,3] f32, depth [n] f32, samples)."""
        M = np.ascontiguousarray(matrix, dtype=np.float32)
        if pixels is not None:
            pixels = np.ascontiguousarray(pixels, dtype=np.int32)
            n = pixels.size
        else:
            n = W * H
        rgb = np.empty((n, 3), dtype=np.float32)
        depth = np.empty(n, dtype=np.float32)
        occ_arr = None if occ is None else np.ascontiguousarray(occ, dtype=np.uint32)
        samples = self.lib.oracle_render_f32(self.h, _ptr(occ_arr), M.ctypes.data, W, H, focal, _ptr(pixels), n,
                                             rgb.ctypes.data, depth.ctypes.data, nthreads or os.cpu_count() or 1)
        return rgb, depth, samples

    def rays(self, views, pairs):
        """FP32 ray set-up of (view, pixel) pairs; views = [(M, W, H, focal)].
        Returns (o [n,3] f32, d [n,3] f32, ts [n] f32, nsteps [n] i32)."""
        n = len(pairs)
        o = np.zeros((n, 3), np.float32)
        d = np.zeros((n, 3), np.float32)
        ts = np.zeros(n, np.float32)
        ns = np.zeros(n, np.int32)
        for i, (v, p) in enumerate(pairs):
            M, W, H, f = views[int(v)]
            ns[i], o[i], d[i], ts[i] = ray_setup(M, W, H, f, int(p) % W, int(p) // W)
        return o, d, ts, ns

    def loss_grad(self, rays, target, depth_w=0.1, occ=None, grad=True, fp32_positions=False):
        """Training loss (mean over rays) and its FP64 gradient.
        rays: output of rays(); target: [n,4] (r, g, b, depth);
        fp32_positions: sample positions rounded as the CUDA kernels round
        them.  Returns (loss, g_table [16*T*2] f64, g_w [9408] f64) or the
        loss alone."""
        o, d, ts, ns = rays
        tgt = np.ascontiguousarray(target, dtype=np.float64)
        occ_arr = None if occ is None else np.ascontiguousarray(occ, dtype=np.uint32)
        gt = np.zeros(16 * (1 << self.log2T) * 2, np.float64) if grad else None
        gw = np.zeros(9408, np.float64) if grad else None
        loss = self.lib.oracle_train_loss_grad(self.h, _ptr(occ_arr), o.ctypes.data, d.ctypes.data, ts.ctypes.data,
                                               ns.ctypes.data, len(ns), tgt.ctypes.data, depth_w,
                                               1 if fp32_positions else 0, _ptr(gt), _ptr(gw))
        return (loss, gt, gw) if grad else loss

    def weights_blob(self):
        """The five weight matrices concatenated (dw1|dw2|cw1|cw2|cw3)."""
        return np.concatenate([self.param(k) for k in range(1, 6)])

    def set_weights_blob(self, blob):
        blob = np.asarray(blob, np.float32)
        off = 0
        for k in range(1, 6):
            n = self.param(k).size
            self.set_param(k, blob[off:off + n])
            off += n


def focal_from_fov(width, fov_deg):
    """Focal length in pixels for a horizontal FOV: (W/2) / tan(FOV/2) in
    double, rounded once to float32 (the camera convention of the scene
    specification, the same rounding the CUDA library applies)."""
    half = 0.5 * float(np.float32(fov_deg)) * 3.14159265358979323846 / 180.0
    return float(np.float32(0.5 * float(width) / math.tan(half)))


def ray_setup(matrix, W, H, focal, px, py):
    lib = load()
    M = np.ascontiguousarray(matrix, dtype=np.float32)
    o = np.empty(3, dtype=np.float32)
    d = np.empty(3, dtype=np.float32)
    ts = ctypes.c_float(0)
    n = lib.oracle_ray_setup(M.ctypes.data, W, H, focal, px, py, o.ctypes.data, d.ctypes.data, ctypes.byref(ts))
    return n, o, d, ts.value


def grid_index(level, T, x, y, z):
    return load().oracle_grid_index(level, T, x, y, z)


def resolutions():
    out = np.empty(16, dtype=np.int32)
    load().oracle_resolutions(out.ctypes.data)
    return out


def dt():
    return load().oracle_dt()


def sh16(d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.empty(16, dtype=np.float64)
    load().oracle_sh16(d.ctypes.data, out.ctypes.data)
    return out


def yuv_planes(w, h, ls):
    ch = (h + 1) // 2
    return (np.zeros(ls[0] * h, np.uint8), np.zeros(ls[1] * ch, np.uint8), np.zeros(ls[2] * ch, np.uint8))


def rgb24_to_yuv420p(rgb, w, h, rgb_ls, ls):
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    y, u, v = yuv_planes(w, h, ls)
    lsa = np.asarray(ls, dtype=np.int32)
    load().oracle_rgb24_to_yuv420p(rgb.ctypes.data, w, h, rgb_ls, y.ctypes.data, u.ctypes.data, v.ctypes.data,
                                   lsa.ctypes.data)
    return y, u, v


def gray8_to_yuv420p(g, w, h, g_ls, ls):
    g = np.ascontiguousarray(g, dtype=np.uint8)
    y, u, v = yuv_planes(w, h, ls)
    lsa = np.asarray(ls, dtype=np.int32)
    load().oracle_gray8_to_yuv420p(g.ctypes.data, w, h, g_ls, y.ctypes.data, u.ctypes.data, v.ctypes.data,
                                   lsa.ctypes.data)
    return y, u, v


def depth_pack_u16mm(d):
    d = np.ascontiguousarray(d, dtype=np.float32)
    out = np.empty(d.size, dtype=np.uint16)
    load().oracle_depth_pack_u16mm(d.ctypes.data, d.size, out.ctypes.data)
    return out


def depth_to_gray8(d, dmax):
    d = np.ascontiguousarray(d, dtype=np.float32)
    out = np.empty(d.size, dtype=np.uint8)
    load().oracle_depth_to_gray8(d.ctypes.data, d.size, dmax, out.ctypes.data)
    return out


def rgb_to_rgb24(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.size, dtype=np.uint8)
    load().oracle_rgb_to_rgb24(x.ctypes.data, x.size, out.ctypes.data)
    return out


def psnr(a, b, peak=1.0):
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)
