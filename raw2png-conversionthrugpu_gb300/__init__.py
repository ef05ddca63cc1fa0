"""raw2png GB300 encoder -- Python binding of the C ABI in include/r2p.h.

The product is libr2p.so (CUDA kernels for sm_103a + C ABI); this module is a
thin ctypes face over it for tests, benchmarks and Python callers.  There is
no CPU fallback: if libr2p.so is missing or no GPU is present, calls raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libr2p.so")

OK, EINVAL, ENOMEM, EBUDGET, ECUDA, ETIMEOUT, ENOSPC, ECANCELED, ENOTFOUND = range(9)
WINDOW_NONE, WINDOW_SWAP16, WINDOW_DICOM16, WINDOW_BATCH8 = range(4)
MANY_SLOTS = 4          # R2P_MANY_SLOTS: images in flight in Engine.encode_png_many
BLOCK64 = 65520
BLOCK32 = 32752


class R2PError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("r2p status %d (%s): %s" % (status, STATUS.get(status, "?"), msg))
        self.status = status


STATUS = {OK: "ok", EINVAL: "invalid argument", ENOMEM: "out of memory", EBUDGET: "HBM budget exceeded",
          ECUDA: "CUDA error", ETIMEOUT: "timed out", ENOSPC: "output buffer too small",
          ECANCELED: "cancelled", ENOTFOUND: "unknown ticket"}


class DicomParams(ctypes.Structure):
    """r2p_dicom_params: same layout as the reference's DicomPixelParams."""
    _fields_ = [
        ("bits_allocated", ctypes.c_int),
        ("bits_stored", ctypes.c_int),
        ("high_bit", ctypes.c_int),
        ("pixel_rep", ctypes.c_int),
        ("apply_rescale", ctypes.c_int),
        ("rescale_slope", ctypes.c_float),
        ("rescale_intercept", ctypes.c_float),
        ("apply_window", ctypes.c_int),
        ("window_center", ctypes.c_float),
        ("window_width", ctypes.c_float),
    ]

    @classmethod
    def make(cls, bits_allocated=16, bits_stored=16, high_bit=None, pixel_rep=0, slope=None, intercept=None,
             wc=None, ww=None):
        """Fill the fields the way src/dicom_loader.cpp:372-397 does: rescale
        only when slope != 1 or intercept != 0, window only when WW > 0."""
        p = cls()
        p.bits_allocated = bits_allocated
        p.bits_stored = bits_stored
        p.high_bit = bits_stored - 1 if high_bit is None else high_bit
        p.pixel_rep = pixel_rep
        p.rescale_slope, p.rescale_intercept = 1.0, 0.0
        if slope is not None or intercept is not None:
            s = 1.0 if slope is None else slope
            b = 0.0 if intercept is None else intercept
            if abs(s - 1.0) > 1e-9 or abs(b) > 1e-9:
                p.apply_rescale = 1
                p.rescale_slope, p.rescale_intercept = s, b
        p.window_center, p.window_width = 32768.0, 65536.0
        if wc is not None and ww is not None and ww > 0:
            p.apply_window = 1
            p.window_center, p.window_width = wc, ww
        return p


class Tuning(ctypes.Structure):
    """r2p_tuning: one image-size class of the autotuned table."""
    _fields_ = [("max_raw_bytes", ctypes.c_uint64), ("block_size", ctypes.c_int), ("band_rows", ctypes.c_int),
                ("hash_bits", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_size_t), ("host_pool_bytes", ctypes.c_size_t),
                ("max_inflight_batches", ctypes.c_int), ("max_batch_images", ctypes.c_int),
                ("max_batch_bytes", ctypes.c_size_t)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("png", ctypes.POINTER(ctypes.c_uint8)), ("png_len", ctypes.c_size_t),
                ("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64), ("canceled", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("pending", ctypes.c_uint64), ("mean_batch_images", ctypes.c_double),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("device_bytes_in_use", ctypes.c_size_t), ("device_bytes_peak", ctypes.c_size_t)]


class Image(ctypes.Structure):
    """r2p_image."""
    _fields_ = [
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("channels", ctypes.c_int),
        ("bytes_per_sample", ctypes.c_int),
        ("window_mode", ctypes.c_int),
        ("dicom", DicomParams),
        ("level", ctypes.c_int),
        ("strip_height", ctypes.c_int),
        ("block_size", ctypes.c_int),
    ]

    @classmethod
    def make(cls, width, height, channels=1, bytes_per_sample=2, window_mode=WINDOW_NONE, dicom=None, level=0,
             strip_height=256, block_size=0):
        im = cls()
        im.width, im.height, im.channels = width, height, channels
        im.bytes_per_sample, im.window_mode = bytes_per_sample, window_mode
        im.dicom = dicom if dicom is not None else DicomParams.make(8 * bytes_per_sample, 8 * bytes_per_sample)
        im.level, im.strip_height, im.block_size = level, strip_height, block_size
        return im

    @property
    def out_bytes_per_sample(self):
        return 1 if self.window_mode == WINDOW_BATCH8 else self.bytes_per_sample

    @property
    def row_bytes(self):
        return self.width * self.channels * self.out_bytes_per_sample

    @property
    def raw_bytes(self):
        return self.width * self.height * self.channels * self.bytes_per_sample

    @property
    def filtered_bytes(self):
        return self.height * (self.row_bytes + 1)


_lib = None
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_u64p = ctypes.POINTER(ctypes.c_uint64)

# name -> (restype, argtypes); every symbol include/r2p.h declares
SIGNATURES = {
    "r2p_version": (ctypes.c_int, []),
    "r2p_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "r2p_last_error": (ctypes.c_char_p, []),
    "r2p_engine_create": (ctypes.c_int, [ctypes.c_int, _sz, ctypes.POINTER(_vp)]),
    "r2p_engine_destroy": (None, [_vp]),
    "r2p_png_bound": (_sz, [ctypes.POINTER(Image)]),
    "r2p_encode_png": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _vp, _sz, ctypes.POINTER(_sz)]),
    "r2p_encode_png_device": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _vp, _sz, _vp, _vp]),
    "r2p_encode_png_many": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Image), ctypes.POINTER(_vp),
                                           ctypes.POINTER(_vp), ctypes.POINTER(_sz), ctypes.POINTER(_sz),
                                           ctypes.POINTER(ctypes.c_int)]),
    "r2p_encode_batch_device": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Image), ctypes.POINTER(_vp),
                                               ctypes.POINTER(_vp), ctypes.POINTER(_sz), _vp, _vp]),
    "r2p_window_filter_device": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _vp, _vp, _vp]),
    "r2p_window_filter_device_ex": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _vp, _vp, _vp, _vp]),
    "r2p_bmp_bound": (_sz, [ctypes.POINTER(Image)]),
    "r2p_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                                                 ctypes.POINTER(ctypes.c_int)]),
    "r2p_encode_bmp": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _vp, _sz, ctypes.POINTER(_sz)]),
    "r2p_encode_bmp_device": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _vp, _sz, _vp]),
    "r2p_zlib_compress_device": (ctypes.c_int, [_vp, _vp, _sz, ctypes.c_int, ctypes.c_int, _vp, _sz, _vp, _vp]),
    "r2p_zlib_bound": (_sz, [_sz, ctypes.c_int, ctypes.c_int]),
    "r2p_deflate_raw_device": (ctypes.c_int, [_vp, _vp, _sz, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _sz, _vp,
                                              _vp]),
    "r2p_zlib_compress_noalloc": (ctypes.c_int, [_vp, _sz, ctypes.c_int, ctypes.c_int, _vp, _sz, _vp, _vp]),
    "r2p_adler32_device": (ctypes.c_int, [_vp, _vp, _sz, _vp, _vp]),
    "r2p_crc32_device": (ctypes.c_int, [_vp, _vp, _sz, _vp, _vp]),
    "r2p_crc32_combine": (ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]),
    "r2p_adler32_combine": (ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]),
    "r2p_device_alloc": (ctypes.c_int, [_sz, ctypes.POINTER(_vp)]),
    "r2p_device_free": (ctypes.c_int, [_vp]),
    "r2p_host_alloc_pinned": (ctypes.c_int, [_sz, ctypes.POINTER(_vp)]),
    "r2p_host_free_pinned": (ctypes.c_int, [_vp]),
    "r2p_memcpy": (ctypes.c_int, [_vp, _vp, _sz, _vp]),
    "r2p_memset_device": (ctypes.c_int, [_vp, ctypes.c_int, _sz, _vp]),
    "r2p_stream_create": (ctypes.c_int, [ctypes.POINTER(_vp)]),
    "r2p_stream_destroy": (ctypes.c_int, [_vp]),
    "r2p_stream_synchronize": (ctypes.c_int, [_vp]),
    "r2p_event_create": (ctypes.c_int, [ctypes.POINTER(_vp)]),
    "r2p_event_destroy": (ctypes.c_int, [_vp]),
    "r2p_event_record": (ctypes.c_int, [_vp, _vp]),
    "r2p_event_elapsed_ms": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(ctypes.c_float)]),
    "r2p_stream_wait_event": (ctypes.c_int, [_vp, _vp]),
    "r2p_kernel_launch_count": (ctypes.c_uint64, []),
    "r2p_engine_set_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "r2p_batch_create": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Image), ctypes.POINTER(_vp),
                                        ctypes.POINTER(_vp), ctypes.POINTER(_sz), _vp, ctypes.POINTER(_vp)]),
    "r2p_batch_launch": (ctypes.c_int, [_vp, _vp]),
    "r2p_batch_launch_graph": (ctypes.c_int, [_vp, _vp]),
    "r2p_batch_device_bytes": (_sz, [_vp]),
    "r2p_batch_destroy": (None, [_vp]),
    "r2p_engine_set_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Tuning)]),
    "r2p_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "r2p_server_set_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Tuning)]),
    "r2p_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, _u64p]),
    "r2p_server_submit_ex": (ctypes.c_int, [_vp, ctypes.POINTER(Image), _vp, ctypes.c_uint32, _u64p]),
    "r2p_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(Result)]),
    "r2p_server_cancel": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "r2p_server_release": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "r2p_server_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "r2p_server_reset_stats": (ctypes.c_int, [_vp]),
    "r2p_server_destroy": (None, [_vp]),
    "r2p_engine_get_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_int)]),
    "r2p_engine_stage_times": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), _u64p]),
}

STAGES = ["prepare_window", "window_filter", "stored_blocks", "lz77_blocks", "finish", "unused"]
KERNELS = ["k_prepare_window", "k_window_filter", "k_stored_blocks", "k_lz77_blocks", "k_finish", None]


def filter_kernel(img):
    """The filter kernel the engine runs for img (pixels 16-byte aligned):
    k_filter_rows for rows of 2048 filtered bytes or more whose raw row is a
    multiple of 16 bytes and whose window table fits 32 KB; else
    k_window_filter_reg for rows of up to 8 KB with a table of up to 16 KB;
    else k_window_filter."""
    pitch = img.width * img.channels * img.bytes_per_sample
    bs = img.dicom.bits_stored
    lut = 0
    if img.window_mode == WINDOW_DICOM16:
        lut = ((1 << bs if bs < 16 else 65536) if img.bytes_per_sample == 2 else 256) * img.out_bytes_per_sample
    elif img.window_mode == WINDOW_BATCH8:
        lut = 1 << bs
    if img.row_bytes >= 2048 and pitch % 16 == 0 and lut <= 32768:
        return "k_filter_rows"
    ok = img.row_bytes <= 8192 and pitch % 16 == 0 and lut <= 16384
    return "k_window_filter_reg" if ok else "k_window_filter"


def lib():
    """Load libr2p.so; raises if it was not built (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libr2p.so not built: run __graft_entry__.build() (nvcc, sm_103a)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != OK:
        raise R2PError(status, lib().r2p_last_error().decode(errors="replace"))
    return status


def png_bound(img):
    return lib().r2p_png_bound(ctypes.byref(img))


def selftest_bounded_wait(arrive, limit_us, device=0):
    """Status the bounded device wait reports (r2p_selftest_bounded_wait)."""
    st = ctypes.c_int()
    check(lib().r2p_selftest_bounded_wait(device, 1 if arrive else 0, limit_us, ctypes.byref(st)))
    return st.value


def bmp_bound(img):
    return lib().r2p_bmp_bound(ctypes.byref(img))


def zlib_bound(n, level, block_size=0):
    return lib().r2p_zlib_bound(n, level, block_size)


def crc32_combine(c1, c2, len2):
    return lib().r2p_crc32_combine(c1, c2, len2)


def adler32_combine(a1, a2, len2):
    return lib().r2p_adler32_combine(a1, a2, len2)


def launch_count():
    return lib().r2p_kernel_launch_count()


# ------------------------------------------------------------ device memory
class DeviceBuffer:
    """Device allocation owned by Python (freed on close / GC)."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = _vp()
        check(lib().r2p_device_alloc(self.nbytes, ctypes.byref(p)))
        self.ptr = p.value

    @classmethod
    def from_array(cls, arr, stream=None):
        a = np.ascontiguousarray(arr)
        b = cls(max(a.nbytes, 1))
        b.upload(a, stream)
        return b

    def upload(self, arr, stream=None):
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        check(lib().r2p_memcpy(self.ptr, a.ctypes.data, a.nbytes, stream))
        if stream is None:
            check(lib().r2p_stream_synchronize(None))

    def download(self, nbytes=None, offset=0, stream=None):
        n = self.nbytes - offset if nbytes is None else int(nbytes)
        out = np.empty(n, np.uint8)
        check(lib().r2p_memcpy(out.ctypes.data, self.ptr + offset, n, stream))
        check(lib().r2p_stream_synchronize(stream))
        return out

    def memset(self, value=0, stream=None):
        check(lib().r2p_memset_device(self.ptr, value, self.nbytes, stream))

    def close(self):
        if getattr(self, "ptr", None):
            lib().r2p_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host buffer viewed as a numpy uint8 array."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = _vp()
        check(lib().r2p_host_alloc_pinned(max(self.nbytes, 1), ctypes.byref(p)))
        self.ptr = p.value
        self.array = np.ctypeslib.as_array((ctypes.c_uint8 * max(self.nbytes, 1)).from_address(self.ptr))

    def close(self):
        if getattr(self, "ptr", None):
            lib().r2p_host_free_pinned(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Stream:
    def __init__(self):
        p = _vp()
        check(lib().r2p_stream_create(ctypes.byref(p)))
        self.ptr = p.value

    def sync(self):
        check(lib().r2p_stream_synchronize(self.ptr))

    def wait(self, event):
        """Later work on this stream waits for `event`."""
        check(lib().r2p_stream_wait_event(self.ptr, event.ptr))

    def close(self):
        if getattr(self, "ptr", None):
            lib().r2p_stream_destroy(self.ptr)
            self.ptr = None


class Event:
    def __init__(self):
        p = _vp()
        check(lib().r2p_event_create(ctypes.byref(p)))
        self.ptr = p.value

    def record(self, stream=None):
        check(lib().r2p_event_record(self.ptr, stream.ptr if isinstance(stream, Stream) else stream))

    def elapsed_ms(self, end):
        ms = ctypes.c_float()
        check(lib().r2p_event_elapsed_ms(self.ptr, end.ptr, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "ptr", None):
            lib().r2p_event_destroy(self.ptr)
            self.ptr = None


def _sp(stream):
    return stream.ptr if isinstance(stream, Stream) else stream


# ------------------------------------------------------------------ engine
class Engine:
    """Device-owning encoder (r2p_engine)."""

    def __init__(self, device=0, hbm_budget=0):
        p = _vp()
        check(lib().r2p_engine_create(device, hbm_budget, ctypes.byref(p)))
        self.h = p.value

    def close(self):
        if getattr(self, "h", None):
            lib().r2p_engine_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def encode_png(self, img, pixels):
        """Host pixels -> PNG bytes (blocking)."""
        px = np.ascontiguousarray(pixels).view(np.uint8).reshape(-1)
        assert px.nbytes == img.raw_bytes, (px.nbytes, img.raw_bytes)
        cap = png_bound(img)
        if cap == 0:
            check(EINVAL)
        out = np.empty(cap, np.uint8)
        n = _sz()
        check(lib().r2p_encode_png(self.h, ctypes.byref(img), px.ctypes.data, out.ctypes.data, cap, ctypes.byref(n)))
        return out[:n.value].tobytes()

    def encode_bmp(self, img, pixels):
        """Host pixels -> BMP file bytes (blocking; r2p_encode_bmp)."""
        px = np.ascontiguousarray(pixels).view(np.uint8).reshape(-1)
        assert px.nbytes == img.raw_bytes, (px.nbytes, img.raw_bytes)
        cap = bmp_bound(img)
        if cap == 0:
            check(EINVAL)
        out = np.empty(cap, np.uint8)
        n = _sz()
        check(lib().r2p_encode_bmp(self.h, ctypes.byref(img), px.ctypes.data, out.ctypes.data, cap, ctypes.byref(n)))
        return out[:n.value].tobytes()

    def encode_bmp_device(self, img, d_pixels, d_bmp, cap, stream=None):
        """Device pixels -> BMP file in device memory (r2p_encode_bmp_device)."""
        check(lib().r2p_encode_bmp_device(self.h, ctypes.byref(img), d_pixels, d_bmp, cap, _sp(stream)))

    def encode_png_many(self, imgs, inputs, outputs=None):
        """Host images -> PNGs with up to MANY_SLOTS images in flight
        (r2p_encode_png_many).  inputs: numpy arrays or PinnedBuffers;
        outputs: optional PinnedBuffers (>= png_bound each; may repeat with a
        period that is a multiple of MANY_SLOTS).  Returns (statuses,
        PNG bytes, or PNG lengths when outputs are given)."""
        n = len(imgs)
        arr_imgs = (Image * n)(*imgs)
        keep = []
        ptr_in = (_vp * n)()
        for i, x in enumerate(inputs):
            if isinstance(x, PinnedBuffer):
                ptr_in[i] = x.ptr
            else:
                a = np.ascontiguousarray(x).view(np.uint8).reshape(-1)
                keep.append(a)
                ptr_in[i] = a.ctypes.data
        caps = (_sz * n)(*[png_bound(im) for im in imgs])
        ptr_out = (_vp * n)()
        own = None
        if outputs is None:
            own = [np.empty(caps[i], np.uint8) for i in range(n)]
            for i in range(n):
                ptr_out[i] = own[i].ctypes.data
        else:
            for i, o in enumerate(outputs):
                ptr_out[i] = o.ptr
                caps[i] = o.nbytes
        lens = (_sz * n)()
        sts = (ctypes.c_int * n)()
        lib().r2p_encode_png_many(self.h, n, arr_imgs, ptr_in, ptr_out, caps, lens, sts)
        statuses = list(sts)
        if own is None:
            return statuses, [int(lens[i]) for i in range(n)]
        return statuses, [own[i][:lens[i]].tobytes() if statuses[i] == OK else None for i in range(n)]

    def encode_png_device(self, img, d_pixels, d_png, png_cap, d_len, stream=None):
        check(lib().r2p_encode_png_device(self.h, ctypes.byref(img), d_pixels, d_png, png_cap, d_len, _sp(stream)))

    def encode_batch_device(self, imgs, d_pixels, d_pngs, caps, d_lens, stream=None):
        n = len(imgs)
        arr = (Image * n)(*imgs)
        px = (_vp * n)(*d_pixels)
        pg = (_vp * n)(*d_pngs)
        cp = (_sz * n)(*caps)
        check(lib().r2p_encode_batch_device(self.h, n, arr, px, pg, cp, d_lens, _sp(stream)))

    def window_filter_device(self, img, d_pixels, d_filtered, d_prior=None, stream=None, d_last_row=None):
        check(lib().r2p_window_filter_device_ex(self.h, ctypes.byref(img), d_pixels, d_prior, d_filtered, d_last_row,
                                                _sp(stream)))

    def zlib_compress_device(self, d_in, n, level, d_out, out_cap, d_len, block_size=0, stream=None):
        check(lib().r2p_zlib_compress_device(self.h, d_in, n, level, block_size, d_out, out_cap, d_len, _sp(stream)))

    def adler32_device(self, d_data, n, d_result, stream=None):
        check(lib().r2p_adler32_device(self.h, d_data, n, d_result, _sp(stream)))

    def crc32_device(self, d_data, n, d_result, stream=None):
        check(lib().r2p_crc32_device(self.h, d_data, n, d_result, _sp(stream)))

    def set_timing(self, enable=True):
        check(lib().r2p_engine_set_timing(self.h, 1 if enable else 0))

    def stage_times(self):
        """{stage: (total ms, launches)} since the last query."""
        ms = (ctypes.c_double * len(STAGES))()
        n = (ctypes.c_uint64 * len(STAGES))()
        check(lib().r2p_engine_stage_times(self.h, ms, n))
        return {STAGES[i]: (ms[i], int(n[i])) for i in range(len(STAGES))}

    def set_tuning(self, classes):
        """classes: list of (max_raw_bytes, block_size, band_rows, hash_bits)."""
        arr = (Tuning * len(classes))(*[Tuning(*c) for c in classes]) if classes else None
        check(lib().r2p_engine_set_tuning(self.h, len(classes), arr))

    def get_tuning(self):
        arr = (Tuning * 64)()
        n = ctypes.c_int()
        check(lib().r2p_engine_get_tuning(self.h, 64, arr, ctypes.byref(n)))
        return [(t.max_raw_bytes, t.block_size, t.band_rows, t.hash_bits) for t in arr[:n.value]]

    def batch(self, imgs, d_pixels, d_pngs, caps, d_lens):
        return Batch(self, imgs, d_pixels, d_pngs, caps, d_lens)

    # convenience wrappers that move data through host memory (tests)
    def filter_image(self, img, pixels, prior=None):
        px = DeviceBuffer.from_array(np.ascontiguousarray(pixels).view(np.uint8).reshape(-1))
        out = DeviceBuffer(img.filtered_bytes + 64)
        pr = DeviceBuffer.from_array(np.ascontiguousarray(prior, np.uint8)) if prior is not None else None
        self.window_filter_device(img, px.ptr, out.ptr, pr.ptr if pr else None)
        return out.download(img.filtered_bytes)

    def zlib_compress(self, data, level, block_size=0):
        data = np.ascontiguousarray(data, np.uint8).reshape(-1)
        src = DeviceBuffer.from_array(data)
        cap = zlib_bound(data.size, level, block_size)
        dst = DeviceBuffer(cap)
        ln = DeviceBuffer(8)
        self.zlib_compress_device(src.ptr, data.size, level, dst.ptr, cap, ln.ptr, block_size)
        n = int(ln.download(8).view(np.uint64)[0])
        if n >> 63:
            raise R2PError(n & 0xFF, "device reported an error")
        return dst.download(n).tobytes()

    def deflate_raw(self, data, level, final_part, block_size=0):
        """Raw DEFLATE of one stream part: (stream bytes, Adler-32 of data)."""
        data = np.ascontiguousarray(data, np.uint8).reshape(-1)
        src = DeviceBuffer.from_array(data)
        cap = zlib_bound(data.size, level, block_size)
        dst = DeviceBuffer(cap)
        ln = DeviceBuffer(8)
        check(lib().r2p_deflate_raw_device(self.h, src.ptr, data.size, level, block_size, 1 if final_part else 0,
                                           dst.ptr, cap, ln.ptr, None))
        n = int(ln.download(8).view(np.uint64)[0])
        if n >> 63:
            raise R2PError(n & 0xFF, "device reported an error")
        out = dst.download(n + 4).tobytes()
        return out[:n], int.from_bytes(out[n:], "big")

    def checksum(self, data, kind):
        data = np.ascontiguousarray(data, np.uint8).reshape(-1)
        src = DeviceBuffer.from_array(data) if data.size else DeviceBuffer(1)
        res = DeviceBuffer(4)
        (self.adler32_device if kind == "adler32" else self.crc32_device)(src.ptr, data.size, res.ptr)
        return int(res.download(4).view(np.uint32)[0])


class Batch:
    """A planned batch (r2p_batch): launch directly or as a CUDA graph."""

    def __init__(self, engine, imgs, d_pixels, d_pngs, caps, d_lens):
        n = len(imgs)
        arr = (Image * n)(*imgs)
        px = (_vp * n)(*d_pixels)
        pg = (_vp * n)(*d_pngs)
        cp = (_sz * n)(*caps)
        p = _vp()
        check(lib().r2p_batch_create(engine.h, n, arr, px, pg, cp, d_lens, ctypes.byref(p)))
        self.h = p.value
        self.engine = engine

    @property
    def device_bytes(self):
        return lib().r2p_batch_device_bytes(self.h)

    def launch(self, stream=None):
        check(lib().r2p_batch_launch(self.h, _sp(stream)))

    def launch_graph(self, stream=None):
        check(lib().r2p_batch_launch_graph(self.h, _sp(stream)))

    def close(self):
        if getattr(self, "h", None):
            lib().r2p_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request server (r2p_server)."""

    def __init__(self, device=0, hbm_budget=0, host_pool_bytes=0, max_inflight_batches=0, max_batch_images=0,
                 max_batch_bytes=0):
        cfg = ServerConfig(hbm_budget, host_pool_bytes, max_inflight_batches, max_batch_images, max_batch_bytes)
        p = _vp()
        check(lib().r2p_server_create(device, ctypes.byref(cfg), ctypes.byref(p)))
        self.h = p.value

    def set_tuning(self, classes):
        arr = (Tuning * len(classes))(*[Tuning(*c) for c in classes]) if classes else None
        check(lib().r2p_server_set_tuning(self.h, len(classes), arr))

    def submit(self, img, pixels, borrow=False):
        """Queue one image.  borrow=True: no copy; `pixels` (a numpy array or
        a PinnedBuffer) must stay alive and unchanged until wait() returns."""
        if isinstance(pixels, PinnedBuffer):
            ptr, nbytes = pixels.ptr, pixels.nbytes
        else:
            px = np.ascontiguousarray(pixels).view(np.uint8).reshape(-1)
            ptr, nbytes = px.ctypes.data, px.nbytes
        assert nbytes >= img.raw_bytes
        t = ctypes.c_uint64()
        check(lib().r2p_server_submit_ex(self.h, ctypes.byref(img), ptr, 1 if borrow else 0, ctypes.byref(t)))
        return t.value

    def wait(self, ticket, timeout_ms=-1, release=True, fetch=True):
        """(status, png bytes (or its length when fetch=False) or None, latency_ms, queue_ms)."""
        r = Result()
        st = lib().r2p_server_wait(self.h, ticket, timeout_ms, ctypes.byref(r))
        if st == ETIMEOUT:
            return ETIMEOUT, None, None, None
        png = None
        if st == OK and r.png_len:
            png = ctypes.string_at(r.png, r.png_len) if fetch else r.png_len
        if release:
            lib().r2p_server_release(self.h, ticket)
        return st, png, r.latency_ms, r.queue_ms

    def cancel(self, ticket):
        return lib().r2p_server_cancel(self.h, ticket)

    def stats(self):
        st = ServerStats()
        check(lib().r2p_server_get_stats(self.h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def reset_stats(self):
        check(lib().r2p_server_reset_stats(self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().r2p_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
