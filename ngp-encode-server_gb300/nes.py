"""ctypes binding of libnes_gb300.so (the C ABI in include/nes_gb300.h).

This is the host-side mirror a Python caller (tests, the benchmark, a
serving driver) uses.  It adds no compute of its own: every call goes through
the CUDA library, and loading fails loudly when the library is missing.

Reference interfaces mirrored:
  - Renderer.render(request_bytes) -> RenderedFrame bytes: the renderer round
    trip of src/server.cpp:161-194 (FrameRequest out, RenderedFrame back).
  - rgb24_to_yuv420p / gray8_to_yuv420p: RenderedFrame::convert_frame
    (include/base/video/rendered_frame.h:24-33).
Errors: negative errno-style codes, raised as NesError (the reference returns
-errno from its socket helpers, src/server.cpp:23-43, and throws
std::runtime_error from the receive path, src/server.cpp:91-112).
"""
import ctypes
import math
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnes_gb300.so")
HEADER = os.path.normpath(os.path.join(HERE, "..", "include", "nes_gb300.h"))

NES_OK = 0
NES_MAX_BATCH_FRAMES = 64  # include/nes_gb300.h
NES_EIO = -5
NES_EAGAIN = -11
NES_ENOMEM = -12
NES_ENODEV = -19
NES_EINVAL = -22
NES_EPROTO = -71
NES_ENOBUFS = -105
NES_ETIMEDOUT = -110

PREC_FP32 = 0
PREC_FP16_TC = 1


class NesError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__("%s: %s (%d)" % (what, _strerror(code), code))


class NesConfig(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("log2_table_size", ctypes.c_uint32),
                ("precision", ctypes.c_int32), ("fov_deg", ctypes.c_float),
                ("depth_gray_max", ctypes.c_float), ("device", ctypes.c_int32),
                ("max_pixels", ctypes.c_uint32), ("record_levels", ctypes.c_uint32)]


class NesView(ctypes.Structure):
    _fields_ = [("matrix", ctypes.c_float * 12), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("focal_px", ctypes.c_float),
                ("flags", ctypes.c_uint32)]


class NesFrameRequest(ctypes.Structure):
    _fields_ = [("index", ctypes.c_uint64), ("is_left", ctypes.c_int32),
                ("has_camera", ctypes.c_int32),
                ("camera_is_left", ctypes.c_int32), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("matrix_len", ctypes.c_uint32),
                ("matrix", ctypes.c_float * 12)]


class NesServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_batch_pixels", ctypes.c_uint32),
                ("max_inflight_batches", ctypes.c_uint32), ("max_pending", ctypes.c_uint32),
                ("use_graphs", ctypes.c_int32), ("max_queue_ms", ctypes.c_float)]


class NesRequest(ctypes.Structure):
    _fields_ = [("nviews", ctypes.c_uint32), ("views", NesView * 2)]


class NesResult(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("status", ctypes.c_int32), ("nviews", ctypes.c_uint32),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("linesize", ctypes.c_int32 * 3),
                ("y_dev", ctypes.c_void_p * 2), ("u_dev", ctypes.c_void_p * 2), ("v_dev", ctypes.c_void_p * 2),
                ("depth_mm_dev", ctypes.c_void_p * 2), ("latency_ms", ctypes.c_double),
                ("batch_id", ctypes.c_uint64), ("batch_requests", ctypes.c_uint32),
                ("batch_views", ctypes.c_uint32)]


class NesServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "rejected", "completed", "batches", "pixels",
                                               "samples", "graph_instantiations", "graph_updates",
                                               "budget_used_bytes")]


class NesTrainConfig(ctypes.Structure):
    _fields_ = [("batch_rays", ctypes.c_uint32), ("lr", ctypes.c_float), ("beta1", ctypes.c_float),
                ("beta2", ctypes.c_float), ("eps", ctypes.c_float), ("depth_weight", ctypes.c_float),
                ("exact_weight_grads", ctypes.c_int32)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_SZ = ctypes.c_size_t
_SIGS = {
    "nes_config_default": (None, [ctypes.POINTER(NesConfig)]),
    "nes_create": (_I, [ctypes.POINTER(NesConfig), ctypes.POINTER(_P)]),
    "nes_destroy": (None, [_P]),
    "nes_strerror": (ctypes.c_char_p, [_I]),
    "nes_focal_from_fov": (ctypes.c_float, [ctypes.c_uint32, ctypes.c_float]),
    "nes_rendered_frame_capacity": (_SZ, [ctypes.c_uint32, ctypes.c_uint32]),
    "nes_render": (_I, [_P, _P, _SZ, _P, _SZ, ctypes.POINTER(_SZ)]),
    "nes_render_views": (_I, [_P, _P, _I, _P, _P, _P]),
    "nes_render_yuv": (_I, [_P, _P, _P, _P, _P, ctypes.POINTER(_I), _P]),
    "nes_render_yuv_views": (_I, [_P, _P, _I, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                                  ctypes.POINTER(_I), ctypes.POINTER(_P)]),
    "nes_rgb24_to_yuv420p": (_I, [_P, _I, _I, _I, _P, _P, _P, ctypes.POINTER(_I), _P]),
    "nes_gray8_to_yuv420p": (_I, [_P, _I, _I, _I, _P, _P, _P, ctypes.POINTER(_I), _P]),
    "nes_depth_pack_u16mm": (_I, [_P, _SZ, _P, _P]),
    "nes_scene_set_param": (_I, [_P, _I, _P, _SZ]),
    "nes_rgb24_to_yuv420p_batch": (_I, [_I, ctypes.POINTER(_P), _I, _I, _I, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                        ctypes.POINTER(_P), ctypes.POINTER(_I), _P]),
    "nes_gray8_to_yuv420p_batch": (_I, [_I, ctypes.POINTER(_P), _I, _I, _I, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                        ctypes.POINTER(_P), ctypes.POINTER(_I), _P]),
    "nes_depth_pack_u16mm_batch": (_I, [_I, ctypes.POINTER(_P), _SZ, ctypes.POINTER(_P), _P]),
    "nes_depth_to_gray8": (_I, [_P, _SZ, ctypes.c_float, _P, _P]),
    "nes_rgb_to_rgb24": (_I, [_P, _SZ, _P, _P]),
    "nes_scene_param": (_I, [_P, _I, _P, _SZ]),
    "nes_occupancy": (_I, [_P, _P]),
    "nes_rebuild_occupancy": (_I, [_P, ctypes.c_float]),
    "nes_last_sample_count": (_I, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "nes_render_view_noalloc": (_I, [_P, ctypes.c_uint32, _P, _P, ctypes.POINTER(NesView), _P, _P, _P]),
    "nes_server_config_default": (None, [ctypes.POINTER(NesServerConfig)]),
    "nes_server_create": (_I, [_P, ctypes.POINTER(NesServerConfig), ctypes.POINTER(_P)]),
    "nes_server_destroy": (None, [_P]),
    "nes_submit": (_I, [_P, ctypes.POINTER(NesRequest), ctypes.POINTER(ctypes.c_uint64)]),
    "nes_wait": (_I, [_P, ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(NesResult)]),
    "nes_release": (_I, [_P, ctypes.c_uint64]),
    "nes_server_stats_get": (_I, [_P, ctypes.POINTER(NesServerStats)]),
    "nes_copy_to_host": (_I, [_P, _P, _SZ]),
    "nes_overlay_text": (_I, [_P, _I, _I, _I, ctypes.c_char_p, _I, _P]),
    "nes_tcp_serve": (_I, [_P, ctypes.c_char_p, ctypes.c_uint16, ctypes.POINTER(ctypes.c_int),
                           ctypes.POINTER(ctypes.c_uint16), ctypes.POINTER(ctypes.c_uint64)]),
    "nes_selftest_bounded_wait": (_I, [_P, ctypes.c_uint32, _I]),
    "nes_probe_gather": (_I, [_P, ctypes.c_uint64, _I, ctypes.c_uint32, ctypes.c_uint32, _P, _P]),
    "nes_probe_gather_replay": (_I, [_P, _P, _I, _I, _P, _SZ, ctypes.POINTER(ctypes.c_float)]),
    "nes_set_profiling": (_I, [_P, _I]),
    "nes_last_timings": (_I, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "nes_scene_generate": (_I, [ctypes.c_uint64, ctypes.c_uint32, _P, _P]),
    "nes_parse_frame_request": (_I, [_P, _SZ, ctypes.POINTER(NesFrameRequest)]),
    "nes_write_rendered_frame": (_I, [ctypes.POINTER(NesFrameRequest), _P, _SZ, _P, _SZ,
                                      _P, _SZ, ctypes.POINTER(_SZ)]),
    "nes_train_config_default": (None, [ctypes.POINTER(NesTrainConfig)]),
    "nes_trainer_create": (_I, [_P, ctypes.POINTER(NesTrainConfig), ctypes.POINTER(_P)]),
    "nes_trainer_destroy": (None, [_P]),
    "nes_trainer_set_targets": (_I, [_P, _P, _I, _P, _P]),
    "nes_trainer_step": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]),
    "nes_trainer_step_rays": (_I, [_P, _P, _I, ctypes.POINTER(ctypes.c_double)]),
    "nes_trainer_grad": (_I, [_P, _P, _I, ctypes.POINTER(ctypes.c_double), _P, _P]),
    "nes_trainer_loss_fp64": (_I, [_P, _P, _I, _I, ctypes.c_uint64, ctypes.c_double,
                                   ctypes.POINTER(ctypes.c_double)]),
    "nes_trainer_loss_fp64_batch": (_I, [_P, _P, _I, _I, _P, _P, _P, _P]),
    "nes_trainer_last_samples": (ctypes.c_uint64, [_P]),
    "nes_trainer_last_timings": (_I, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(ctypes.c_float)]),
}

_lib = None


def header_symbols():
    """Names of every function declared in include/nes_gb300.h."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nes_[a-z0-9_]+)\s*\(", text)))


def load(path=None):
    """Loads the CUDA library; raises OSError when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(path or LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _strerror(code):
    try:
        return load().nes_strerror(code).decode()
    except OSError:
        return "error"


def check(rc, what):
    if rc != NES_OK:
        raise NesError(rc, what)


def focal_from_fov(width, fov_deg):
    return load().nes_focal_from_fov(width, fov_deg)


def make_view(matrix, width, height, focal):
    v = NesView()
    for i in range(12):
        v.matrix[i] = float(matrix[i])
    v.width = width
    v.height = height
    v.focal_px = focal
    v.flags = 0
    return v


def default_config(**kw):
    cfg = NesConfig()
    load().nes_config_default(ctypes.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def linesizes(width, align=32):
    """av_image_alloc-style YUV420P linesizes (FrameManager aligns to 32,
    include/base/video/type_managers.h:164)."""
    cw = (width + 1) // 2
    a = lambda x: (x + align - 1) // align * align
    return [a(width), a(cw), a(cw)]


class Renderer:
    """One rendering context (scene + device buffers) on one GPU."""

    def __init__(self, **kw):
        self.lib = load()
        self.cfg = default_config(**kw)
        h = _P()
        check(self.lib.nes_create(ctypes.byref(self.cfg), ctypes.byref(h)), "nes_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.nes_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def render(self, request: bytes) -> bytes:
        """FrameRequest bytes -> RenderedFrame bytes (wire-compatible)."""
        n = _SZ(0)
        buf = ctypes.create_string_buffer(request, len(request))
        rc = self.lib.nes_render(self.h, buf, len(request), None, 0, ctypes.byref(n))
        if rc not in (NES_OK, NES_ENOBUFS):
            raise NesError(rc, "nes_render")
        out = ctypes.create_string_buffer(n.value)
        check(self.lib.nes_render(self.h, buf, len(request), out, n.value, ctypes.byref(n)),
              "nes_render")
        return out.raw[:n.value]

    def render_views(self, views, rgb_ptrs, depth_ptrs, stream=0):
        nv = len(views)
        arr = (NesView * nv)(*views)
        rgb = (_P * nv)(*[p or None for p in rgb_ptrs]) if rgb_ptrs is not None else None
        dep = (_P * nv)(*[p or None for p in depth_ptrs]) if depth_ptrs is not None else None
        check(self.lib.nes_render_views(self.h, arr, nv, rgb, dep, _P(stream) if stream else None),
              "nes_render_views")

    def render_yuv(self, view, y_ptr, u_ptr, v_ptr, ls, depth_ptr=None):
        lsa = (_I * 3)(*ls)
        check(self.lib.nes_render_yuv(self.h, ctypes.byref(view), _P(y_ptr), _P(u_ptr), _P(v_ptr), lsa,
                                      _P(depth_ptr) if depth_ptr else None), "nes_render_yuv")

    def render_yuv_views(self, views, y_ptrs, u_ptrs, v_ptrs, ls, depth_ptrs=None):
        """Pose -> YUV for several views of one size (e.g. a stereo pair) in
        one batch, planes copied to the given host buffers."""
        nv = len(views)
        arr = (NesView * nv)(*views)
        lsa = (_I * 3)(*ls)
        dep = _ptrs(depth_ptrs) if depth_ptrs else None
        check(self.lib.nes_render_yuv_views(self.h, arr, nv, _ptrs(y_ptrs), _ptrs(u_ptrs), _ptrs(v_ptrs), lsa, dep),
              "nes_render_yuv_views")

    def scene_param(self, which, count):
        import numpy as np
        out = np.empty(count, dtype=np.float32)
        check(self.lib.nes_scene_param(self.h, which, out.ctypes.data, count), "nes_scene_param")
        return out

    def set_scene_param(self, which, arr):
        import numpy as np
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(-1)
        check(self.lib.nes_scene_set_param(self.h, which, a.ctypes.data, a.size), "nes_scene_set_param")

    def occupancy(self):
        import numpy as np
        out = np.empty(65536, dtype=np.uint32)
        check(self.lib.nes_occupancy(self.h, out.ctypes.data), "nes_occupancy")
        return out

    def rebuild_occupancy(self, threshold):
        check(self.lib.nes_rebuild_occupancy(self.h, threshold), "nes_rebuild_occupancy")

    def last_sample_count(self):
        v = ctypes.c_uint64(0)
        check(self.lib.nes_last_sample_count(self.h, ctypes.byref(v)), "nes_last_sample_count")
        return v.value

    def set_profiling(self, on=True):
        check(self.lib.nes_set_profiling(self.h, 1 if on else 0), "nes_set_profiling")

    def last_timings(self):
        """(raygen_ms, march_ms) of the last render, from CUDA events."""
        a, b = ctypes.c_float(0), ctypes.c_float(0)
        check(self.lib.nes_last_timings(self.h, ctypes.byref(a), ctypes.byref(b)), "nes_last_timings")
        return a.value, b.value


class Trainer:
    """Refits an FP32 Renderer's scene to target renders (nes_trainer_*).

    Targets are device buffers (HWC FP32 RGB and FP32 depth, views
    concatenated) that must outlive the trainer's use of them."""

    def __init__(self, renderer, **kw):
        self.lib = load()
        self.renderer = renderer  # keeps the student context alive
        self.cfg = NesTrainConfig()
        self.lib.nes_train_config_default(ctypes.byref(self.cfg))
        for k, v in kw.items():
            setattr(self.cfg, k, v)
        h = _P()
        check(self.lib.nes_trainer_create(renderer.h, ctypes.byref(self.cfg), ctypes.byref(h)),
              "nes_trainer_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.nes_trainer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_targets(self, views, rgb_ptr, depth_ptr):
        arr = (NesView * len(views))(*views)
        check(self.lib.nes_trainer_set_targets(self.h, arr, len(views), _P(rgb_ptr), _P(depth_ptr)),
              "nes_trainer_set_targets")

    @staticmethod
    def _pairs(pairs):
        import numpy as np
        return np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)

    def step(self, seed):
        loss = ctypes.c_double(0)
        check(self.lib.nes_trainer_step(self.h, seed, ctypes.byref(loss)), "nes_trainer_step")
        return loss.value

    def step_rays(self, pairs):
        p = self._pairs(pairs)
        loss = ctypes.c_double(0)
        check(self.lib.nes_trainer_step_rays(self.h, p.ctypes.data, len(p), ctypes.byref(loss)),
              "nes_trainer_step_rays")
        return loss.value

    def grad(self, pairs, table_floats):
        """(loss, grad_table [table_floats] f32, grad_weights [9408] f32)."""
        import numpy as np
        p = self._pairs(pairs)
        gt = np.empty(table_floats, np.float32)
        gw = np.empty(9408, np.float32)
        loss = ctypes.c_double(0)
        check(self.lib.nes_trainer_grad(self.h, p.ctypes.data, len(p), ctypes.byref(loss), gt.ctypes.data,
                                        gw.ctypes.data), "nes_trainer_grad")
        return loss.value, gt, gw

    def loss_fp64(self, pairs, which=0, index=0, delta=0.0):
        p = self._pairs(pairs)
        loss = ctypes.c_double(0)
        check(self.lib.nes_trainer_loss_fp64(self.h, p.ctypes.data, len(p), which, index, delta,
                                             ctypes.byref(loss)), "nes_trainer_loss_fp64")
        return loss.value

    def loss_fp64_batch(self, pairs, which, index, delta):
        """FP64 loss for many single-parameter perturbations in one launch."""
        import numpy as np
        p = self._pairs(pairs)
        w = np.ascontiguousarray(which, dtype=np.int32)
        i = np.ascontiguousarray(index, dtype=np.uint64)
        d = np.ascontiguousarray(delta, dtype=np.float64)
        out = np.empty(len(w), np.float64)
        check(self.lib.nes_trainer_loss_fp64_batch(self.h, p.ctypes.data, len(p), len(w), w.ctypes.data,
                                                   i.ctypes.data, d.ctypes.data, out.ctypes.data),
              "nes_trainer_loss_fp64_batch")
        return out

    def last_samples(self):
        return self.lib.nes_trainer_last_samples(self.h)

    def last_timings(self):
        """(forward_ms, backward_ms, adam_ms) of the last step, CUDA events."""
        a, b, c = ctypes.c_float(0), ctypes.c_float(0), ctypes.c_float(0)
        check(self.lib.nes_trainer_last_timings(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
              "nes_trainer_last_timings")
        return a.value, b.value, c.value


def rgb24_to_yuv420p(rgb_ptr, w, h, rgb_ls, y, u, v, ls, stream=0):
    lsa = (_I * 3)(*ls)
    check(load().nes_rgb24_to_yuv420p(_P(rgb_ptr), w, h, rgb_ls, _P(y), _P(u), _P(v), lsa,
                                      _P(stream) if stream else None), "nes_rgb24_to_yuv420p")


def gray8_to_yuv420p(g_ptr, w, h, g_ls, y, u, v, ls, stream=0):
    lsa = (_I * 3)(*ls)
    check(load().nes_gray8_to_yuv420p(_P(g_ptr), w, h, g_ls, _P(y), _P(u), _P(v), lsa,
                                      _P(stream) if stream else None), "nes_gray8_to_yuv420p")


def _ptrs(ptrs):
    return (_P * len(ptrs))(*[_P(p) for p in ptrs])


def yuv420p_batch(src_ptrs, w, h, src_ls, y_ptrs, u_ptrs, v_ptrs, ls, stream=0, gray=False):
    """Batched RGB24 (or GRAY8) -> YUV420P: one launch for all frames."""
    lsa = (_I * 3)(*ls)
    fn = load().nes_gray8_to_yuv420p_batch if gray else load().nes_rgb24_to_yuv420p_batch
    check(fn(len(src_ptrs), _ptrs(src_ptrs), w, h, src_ls, _ptrs(y_ptrs), _ptrs(u_ptrs), _ptrs(v_ptrs), lsa,
             _P(stream) if stream else None), "yuv420p_batch")


def depth_pack_u16mm_batch(d_ptrs, n, out_ptrs, stream=0):
    check(load().nes_depth_pack_u16mm_batch(len(d_ptrs), _ptrs(d_ptrs), n, _ptrs(out_ptrs),
                                            _P(stream) if stream else None), "nes_depth_pack_u16mm_batch")


def depth_pack_u16mm(d_ptr, n, out_ptr, stream=0):
    check(load().nes_depth_pack_u16mm(_P(d_ptr), n, _P(out_ptr), _P(stream) if stream else None),
          "nes_depth_pack_u16mm")


def scene_generate(seed, log2T):
    """Host-side scene generation (no GPU): (table, weights) as numpy."""
    import numpy as np
    T = 1 << log2T
    table = np.empty(16 * T * 2, dtype=np.float32)
    weights = np.empty(9408, dtype=np.float32)
    check(load().nes_scene_generate(seed, log2T, table.ctypes.data, weights.ctypes.data),
          "nes_scene_generate")
    return table, weights


# ---------------------------------------------------------------------------
# Poses (host side).  SplitMix64 stream 6 of the workload seed: pose k uses
# draws 3k, 3k+1, 3k+2 for z = 1 - 2u, phi = 2 pi u, r = rmin + (rmax-rmin) u;
# the eye sits at centre + r * (sqrt(1-z^2) cos phi, sqrt(1-z^2) sin phi, z)
# looking at the cube centre (0.5, 0.5, 0.5).
# ---------------------------------------------------------------------------
_M64 = (1 << 64) - 1


def _mix64(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return z ^ (z >> 31)


def _u01(key, i):
    return (_mix64((key + (i + 1) * 0x9E3779B97F4A7C15) & _M64) >> 11) * 2.0 ** -53


def look_at(eye, centre=(0.5, 0.5, 0.5)):
    """3x4 row-major pose: columns right, down, forward, eye."""
    f = [centre[i] - eye[i] for i in range(3)]
    n = math.sqrt(sum(v * v for v in f))
    f = [v / n for v in f]
    up = (0.0, 0.0, 1.0) if abs(f[2]) < 0.99 else (0.0, 1.0, 0.0)
    r = [f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]]
    n = math.sqrt(sum(v * v for v in r))
    r = [v / n for v in r]
    d = [f[1] * r[2] - f[2] * r[1], f[2] * r[0] - f[0] * r[2], f[0] * r[1] - f[1] * r[0]]
    return [r[0], d[0], f[0], eye[0], r[1], d[1], f[1], eye[1], r[2], d[2], f[2], eye[2]]


def shell_poses(seed, count, rmin, rmax, centre=(0.5, 0.5, 0.5)):
    key = _mix64((seed * 256 + 6) & _M64)
    out = []
    for k in range(count):
        z = 1.0 - 2.0 * _u01(key, 3 * k)
        phi = 2.0 * math.pi * _u01(key, 3 * k + 1)
        r = rmin + (rmax - rmin) * _u01(key, 3 * k + 2)
        s = math.sqrt(max(0.0, 1.0 - z * z))
        eye = (centre[0] + r * s * math.cos(phi), centre[1] + r * s * math.sin(phi), centre[2] + r * z)
        out.append(look_at(eye, centre))
    return out


def stereo_pair(pose, ipd):
    """Left/right eye poses: the eye moves by -/+ ipd/2 along the right axis."""
    out = []
    for sgn in (-0.5, 0.5):
        m = list(pose)
        for row in range(3):
            m[row * 4 + 3] = pose[row * 4 + 3] + sgn * ipd * pose[row * 4 + 0]
        out.append(m)
    return out


class TcpEndpoint:
    """nes_tcp_serve in a background thread: the renderer endpoint neserver
    connects to with --renderer host:port."""

    def __init__(self, renderer, port=0, bind="127.0.0.1"):
        import threading
        import time
        self.lib = load()
        self.stop = ctypes.c_int(0)
        self.port = ctypes.c_uint16(0)
        self.served = ctypes.c_uint64(0)
        self.rc = None

        def run():
            self.rc = self.lib.nes_tcp_serve(renderer.h, bind.encode(), port, ctypes.byref(self.stop),
                                             ctypes.byref(self.port), ctypes.byref(self.served))
        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()
        t0 = time.time()
        while self.port.value == 0 and self.rc is None and time.time() - t0 < 10:
            time.sleep(0.01)
        if self.port.value == 0:
            raise NesError(self.rc if self.rc is not None else NES_ETIMEDOUT, "nes_tcp_serve")

    def close(self):
        self.stop.value = 1
        self.thread.join()
        return self.served.value


class Server:
    """Continuously batched serving loop on one Renderer (nes_server_*)."""

    def __init__(self, renderer, **kw):
        self.lib = load()
        self.renderer = renderer
        cfg = NesServerConfig()
        self.lib.nes_server_config_default(ctypes.byref(cfg))
        for k, v in kw.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        h = _P()
        check(self.lib.nes_server_create(renderer.h, ctypes.byref(cfg), ctypes.byref(h)), "nes_server_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.nes_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, views):
        """Admits a mono ([view]) or stereo ([left, right]) request; returns
        its ticket, or None when it was dropped (budget / queue full)."""
        req = NesRequest()
        req.nviews = len(views)
        for i, v in enumerate(views):
            req.views[i] = v
        t = ctypes.c_uint64(0)
        rc = self.lib.nes_submit(self.h, ctypes.byref(req), ctypes.byref(t))
        if rc == NES_EAGAIN:
            return None
        check(rc, "nes_submit")
        return t.value

    def wait(self, ticket, timeout_ns=-1):
        res = NesResult()
        rc = self.lib.nes_wait(self.h, ticket, timeout_ns, ctypes.byref(res))
        if rc == NES_ETIMEDOUT:
            return None
        check(rc, "nes_wait")
        return res

    def release(self, ticket):
        check(self.lib.nes_release(self.h, ticket), "nes_release")

    def stats(self):
        st = NesServerStats()
        check(self.lib.nes_server_stats_get(self.h, ctypes.byref(st)), "nes_server_stats_get")
        return {n: getattr(st, n) for n, _ in NesServerStats._fields_}

    def fetch(self, res, view=0):
        """Copies one served view to host: (y, u, v, depth_mm) numpy arrays."""
        import numpy as np
        h, ls = res.height, list(res.linesize)
        ch = (h + 1) // 2
        out = []
        for ptr, n in ((res.y_dev[view], ls[0] * h), (res.u_dev[view], ls[1] * ch), (res.v_dev[view], ls[2] * ch)):
            a = np.empty(n, np.uint8)
            check(self.lib.nes_copy_to_host(a.ctypes.data, ptr, n), "nes_copy_to_host")
            out.append(a)
        d = np.empty(res.width * h, np.uint16)
        check(self.lib.nes_copy_to_host(d.ctypes.data, res.depth_mm_dev[view], d.nbytes), "nes_copy_to_host")
        out.append(d)
        return out
