"""goofy_gb300 -- GB300-native (sm_103a) Goofy BC1 / ETC1s block encoder.

Python mirror of the reference's public interface (GoofyTC/goofy_tc.h:10-13)
over the C ABI of ``libgoofy_gb300.so`` (include/goofy_gpu.h):

* ``compressDXT1(result, input, width, height, stride)`` /
  ``compressETC1(...)`` -- same names, argument meaning and return codes as
  ``goofy::compressDXT1/compressETC1`` (0, -1 for width % 16, -2 for
  height % 4); buffers are host memory (numpy arrays, bytearrays or raw
  addresses).  They run on the GPU; there is no CPU fallback: if the library
  is not built, importing the functions raises.
* ``compress_device(codec, dst, src, width, height, stride, stream)`` --
  device pointers, asynchronous on a CUDA stream (width % 4 is enough).
* ``compress_host(codec, dst, src, width, height, stride)`` -- host memory,
  width % 4 is enough.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgoofy_gb300.so")
SYNTH_PATH = os.path.join(HERE, "_build", "libgoofy_synth.so")

OK = 0
ERR_WIDTH = -1
ERR_HEIGHT = -2
ERR_INVALID = -3
ERR_ALIGNMENT = -4
ERR_CUDA = -5
ERR_NOMEM = -6
ERR_TIMEOUT = -7
ERR_BUSY = -8
ERR_NO_DEVICE = -9
ERR_TOO_LARGE = -10

CODEC_BC1 = 0
CODEC_ETC1S = 1
CODEC_BOTH = 2  # the two-codec pass: compress_both_*, and its tile in get_tile / set_tile
NOALLOC_MAX_IMAGES = 256
CODECS = {"bc1": CODEC_BC1, "dxt1": CODEC_BC1, "etc1s": CODEC_ETC1S, "etc1": CODEC_ETC1S}

_lib = None
_synth = None

_VP = ctypes.c_void_p
_U32 = ctypes.c_uint32


HOST_PATH_AUTO = 0
HOST_PATH_STAGED = 1
HOST_PATH_DIRECT = 2

SERVER_STAGED = 0
SERVER_DIRECT = 1
COMPLETION_CALLBACK = 0
COMPLETION_EVENT = 1


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("mode", ctypes.c_int32), ("device_budget_bytes", ctypes.c_uint64),
                ("max_batch_images", ctypes.c_uint32), ("max_inflight_batches", ctypes.c_uint32),
                ("max_requests", ctypes.c_uint32), ("quality", ctypes.c_uint32), ("completion", ctypes.c_uint32)]


class Request(ctypes.Structure):
    """goofy_gpu_request: one host-memory encode request."""
    _fields_ = [("src", ctypes.c_void_p), ("dst", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("stride", ctypes.c_uint32), ("codec", ctypes.c_int32)]


class RequestTimes(ctypes.Structure):
    _fields_ = [("submit_ns", ctypes.c_int64), ("admit_ns", ctypes.c_int64), ("launch_ns", ctypes.c_int64),
                ("done_ns", ctypes.c_int64), ("psnr_rgb", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64), ("requests_done", ctypes.c_uint64), ("pixels_done", ctypes.c_uint64),
                ("max_batch", ctypes.c_uint64), ("waiting", ctypes.c_uint64), ("inflight_bytes", ctypes.c_uint64),
                ("max_enqueue_ns", ctypes.c_uint64), ("max_kernel_ns", ctypes.c_uint64),
                ("max_launch_ns", ctypes.c_uint64), ("slowest_enqueue_ns", ctypes.c_uint64),
                ("slowest_gpu_span_ns", ctypes.c_uint64), ("slowest_kernel_ns", ctypes.c_uint64)]


class Level(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("stride", ctypes.c_uint32)]


class Quality(ctypes.Structure):
    """goofy_gpu_quality: the harness's MsePsnr record."""
    _fields_ = [(n, ctypes.c_double) for n in ("mse_r", "mse_g", "mse_b", "mse_a", "mse_max", "mse_rgb", "mse_y",
                                                "psnr_r", "psnr_g", "psnr_b", "psnr_a", "psnr_min", "psnr_rgb",
                                                "psnr_y")] + [("unsupported_blocks", ctypes.c_uint64)]


class Tile(ctypes.Structure):
    _fields_ = [("threads_per_cta", ctypes.c_uint32), ("blocks_per_thread", ctypes.c_uint32),
                ("persistent", ctypes.c_uint32)]


class Image(ctypes.Structure):
    """goofy_gpu_image: one device image of a batch."""
    _fields_ = [("src", ctypes.c_void_p), ("dst", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("stride", ctypes.c_uint32), ("codec", ctypes.c_int32)]


class BatchTile(ctypes.Structure):
    _fields_ = [("threads_per_cta", ctypes.c_uint32), ("blocks_per_thread", ctypes.c_uint32),
                ("unit_blocks", ctypes.c_uint32), ("pipeline", ctypes.c_uint32)]


def _declare(lib):
    sigs = {
        "goofy_gpu_init": (ctypes.c_int, [ctypes.c_int]),
        "goofy_gpu_shutdown": (None, []),
        "goofy_gpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "goofy_gpu_last_error": (ctypes.c_char_p, []),
        "goofy_gpu_compress_device": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _U32, _U32, _U32, _VP]),
        "goofy_gpu_compress_bc1_device": (ctypes.c_int, [_VP, _VP, _U32, _U32, _U32, _VP]),
        "goofy_gpu_compress_etc1s_device": (ctypes.c_int, [_VP, _VP, _U32, _U32, _U32, _VP]),
        "goofy_gpu_compress_host": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _U32, _U32, _U32]),
        "goofy_gpu_compress_bc1_host": (ctypes.c_int, [_VP, _VP, _U32, _U32, _U32]),
        "goofy_gpu_compress_etc1s_host": (ctypes.c_int, [_VP, _VP, _U32, _U32, _U32]),
        "goofy_gpu_compress_both_device": (ctypes.c_int, [_VP, _VP, _VP, _U32, _U32, _U32, _VP]),
        "goofy_gpu_compress_both_host": (ctypes.c_int, [_VP, _VP, _VP, _U32, _U32, _U32]),
        "goofy_gpu_host_alloc": (_VP, [ctypes.c_size_t]),
        "goofy_gpu_set_host_path": (ctypes.c_int, [ctypes.c_int]),
        "goofy_gpu_get_host_path": (ctypes.c_int, []),
        "goofy_gpu_host_free": (None, [_VP]),
        "goofy_gpu_get_tile": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(Tile)]),
        "goofy_gpu_set_tile": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(Tile)]),
        "goofy_gpu_reset_tiles": (ctypes.c_int, []),
        "goofy_gpu_autotune_pair": (ctypes.c_int, [_VP, _VP, _VP, _U32, _U32, _U32, _U32, ctypes.POINTER(Tile),
                                                   ctypes.POINTER(Tile), ctypes.POINTER(ctypes.c_float)]),
        "goofy_gpu_set_tile_cache_path": (ctypes.c_int, [ctypes.c_char_p]),
        "goofy_gpu_get_tile_cache_path": (ctypes.c_size_t, [ctypes.c_char_p, ctypes.c_size_t]),
        "goofy_gpu_device_key": (ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_U32)]),
        "goofy_gpu_tile_cache_store": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _U32, ctypes.c_int,
                                                      ctypes.POINTER(Tile), ctypes.c_float]),
        "goofy_gpu_tile_cache_lookup": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _U32, ctypes.c_int,
                                                       ctypes.POINTER(Tile)]),
        "goofy_gpu_load_tile_cache": (ctypes.c_int, [ctypes.c_int]),
        "goofy_gpu_autotune": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _U32, _U32, _U32, _U32, ctypes.POINTER(Tile),
                                              ctypes.POINTER(ctypes.c_float)]),
        "goofy_gpu_batch_create": (ctypes.c_int, [ctypes.POINTER(_VP), _U32, ctypes.c_int]),
        "goofy_gpu_batch_destroy": (None, [_VP]),
        "goofy_gpu_batch_encode": (ctypes.c_int, [_VP, ctypes.POINTER(Image), _U32, _VP]),
        "goofy_gpu_batch_set_graphs": (ctypes.c_int, [_VP, ctypes.c_int]),
        "goofy_gpu_batch_get_tile": (ctypes.c_int, [_VP, ctypes.POINTER(BatchTile)]),
        "goofy_gpu_batch_set_tile": (ctypes.c_int, [_VP, ctypes.POINTER(BatchTile)]),
        "goofy_gpu_batch_autotune": (ctypes.c_int, [_VP, ctypes.POINTER(Image), _U32, _U32, ctypes.POINTER(BatchTile),
                                                    ctypes.POINTER(ctypes.c_float)]),
        "goofy_gpu_batch_encode_noalloc": (ctypes.c_int, [ctypes.POINTER(Image), _U32, _VP]),
        "goofy_gpu_decode_device": (ctypes.c_int, [ctypes.c_int, _VP, _U32, _VP, _U32, _U32, _VP, _VP]),
        "goofy_gpu_block_error_device": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _U32, _U32, _U32, _VP, _VP]),
        "goofy_gpu_psnr_rgb": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _U32, _U32, _U32,
                                              ctypes.POINTER(ctypes.c_double), _VP]),
        "goofy_gpu_pipeline_timeouts": (ctypes.c_int, [ctypes.POINTER(_U32), ctypes.c_int]),
        "goofy_gpu_selftest_bounded_wait": (ctypes.c_int, [ctypes.POINTER(_U32)]),
        "goofy_gpu_mse_psnr": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _U32, _U32, _U32, ctypes.POINTER(Quality)]),
        "goofy_gpu_png_info": (ctypes.c_int, [_VP, ctypes.c_size_t, ctypes.POINTER(_U32), ctypes.POINTER(_U32)]),
        "goofy_gpu_png_decode": (ctypes.c_int, [_VP, ctypes.c_size_t, _VP, ctypes.c_size_t, _U32, ctypes.c_int,
                                                ctypes.POINTER(_U32), ctypes.POINTER(_U32)]),
        "goofy_gpu_mip_count": (_U32, [_U32, _U32]),
        "goofy_gpu_mip_arena_bytes": (ctypes.c_size_t, [_U32, _U32]),
        "goofy_gpu_generate_mips": (ctypes.c_int, [_VP, _U32, _U32, _U32, _VP, ctypes.c_size_t, ctypes.POINTER(Level),
                                                   _U32, ctypes.POINTER(_U32), _VP]),
        "goofy_gpu_tga_size": (ctypes.c_size_t, [_U32, _U32]),
        "goofy_gpu_write_tga": (ctypes.c_int, [_VP, _U32, _U32, _U32, _VP, ctypes.c_size_t]),
        "goofy_gpu_container_size": (ctypes.c_size_t, [ctypes.c_int, _VP, _VP, _U32]),
        "goofy_gpu_write_container": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _VP, _U32, _VP, ctypes.c_size_t]),
        "goofy_gpu_server_default_config": (None, [ctypes.POINTER(ServerConfig)]),
        "goofy_gpu_server_create": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.POINTER(ServerConfig)]),
        "goofy_gpu_server_destroy": (None, [_VP]),
        "goofy_gpu_server_submit": (ctypes.c_int, [_VP, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
        "goofy_gpu_server_wait": (ctypes.c_int, [_VP, ctypes.c_uint64, _U32, ctypes.POINTER(RequestTimes)]),
        "goofy_gpu_server_get_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ServerStats)]),
        "goofy_gpu_now_ns": (ctypes.c_int64, []),
        "goofy_gpu_server_replay": (ctypes.c_int, [_VP, ctypes.POINTER(Request), _VP, _U32, _VP, ctypes.POINTER(ctypes.c_int64),
                                                   ctypes.POINTER(RequestTimes)]),
        "goofy_gpu_plain_replay": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(Request), _VP, _U32, _VP,
                                                  ctypes.POINTER(ctypes.c_int64)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    # C++ drop-in symbols (Itanium mangling of goofy::compressDXT1/ETC1)
    for mangled in ("_ZN5goofy12compressDXT1EPhPKhjjj", "_ZN5goofy12compressETC1EPhPKhjjj"):
        fn = getattr(lib, mangled)
        fn.restype = ctypes.c_int
        fn.argtypes = [_VP, _VP, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint]
    return lib


def lib():
    """The loaded C-ABI library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgoofy_gb300.so is not built (run goofy_gb300.build.build()); "
                               "there is no CPU fallback")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            raise RuntimeError("libgoofy_synth.so is not built (run goofy_gb300.build.build())")
        s = ctypes.CDLL(SYNTH_PATH)
        s.goofy_synth_scene.restype = ctypes.c_int
        s.goofy_synth_scene.argtypes = [_VP, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint64,
                                        ctypes.c_uint, ctypes.c_uint, ctypes.c_int]
        s.goofy_synth_stress.restype = ctypes.c_int
        s.goofy_synth_stress.argtypes = [_VP, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint64]
        s.goofy_synth_downsample.restype = ctypes.c_int
        s.goofy_synth_downsample.argtypes = [_VP, ctypes.c_uint, _VP, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint]
        s.goofy_synth_texture_spec.restype = None
        s.goofy_synth_texture_spec.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint),
                                               ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_int),
                                               ctypes.POINTER(ctypes.c_int)]
        s.goofy_synth_pcg32.restype = ctypes.c_uint32
        s.goofy_synth_pcg32.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32]
        _synth = s
    return _synth


def _addr(buf):
    """Address of a host buffer: numpy array, bytearray, ctypes object or int."""
    if buf is None:
        return None
    if isinstance(buf, int):
        return buf
    if hasattr(buf, "ctypes"):  # numpy
        return buf.ctypes.data
    if isinstance(buf, bytearray):
        return ctypes.addressof((ctypes.c_char * len(buf)).from_buffer(buf))
    if hasattr(buf, "data_ptr"):  # torch tensor
        return buf.data_ptr()
    return ctypes.addressof(buf)


def status_string(code):
    return lib().goofy_gpu_status_string(code).decode()


def last_error():
    return lib().goofy_gpu_last_error().decode()


# ---- reference-named entry points (goofy_tc.h:10-13) ----
def compressDXT1(result, input, width, height, stride):
    """goofy::compressDXT1 on the GPU: host buffers, returns 0 / -1 / -2 (or a GOOFY_ERR_*)."""
    return lib()._ZN5goofy12compressDXT1EPhPKhjjj(_addr(result), _addr(input), width, height, stride)


def compressETC1(result, input, width, height, stride):
    """goofy::compressETC1 on the GPU: host buffers, returns 0 / -1 / -2 (or a GOOFY_ERR_*)."""
    return lib()._ZN5goofy12compressETC1EPhPKhjjj(_addr(result), _addr(input), width, height, stride)


def compress_host(codec, dst, src, width, height, stride):
    return lib().goofy_gpu_compress_host(codec, _addr(dst), _addr(src), width, height, stride)


def compress_device(codec, dst, src, width, height, stride, stream=None):
    """Device pointers (ints or torch tensors); `stream` is a cudaStream_t handle (int) or None."""
    return lib().goofy_gpu_compress_device(codec, _addr(dst), _addr(src), width, height, stride, stream)


def compress_both_device(dst_bc1, dst_etc1s, src, width, height, stride, stream=None):
    """BC1 and ETC1s blocks of one device image from one pass over it (device
    pointers or torch tensors), each bit-identical to its single-codec call."""
    return lib().goofy_gpu_compress_both_device(_addr(dst_bc1), _addr(dst_etc1s), _addr(src), width, height, stride,
                                                stream)


def compress_both_host(dst_bc1, dst_etc1s, src, width, height, stride):
    """The same from host buffers, synchronous (the drop-in's host paths)."""
    return lib().goofy_gpu_compress_both_host(_addr(dst_bc1), _addr(dst_etc1s), _addr(src), width, height, stride)


def init(device=0):
    return lib().goofy_gpu_init(device)


def shutdown():
    lib().goofy_gpu_shutdown()


def set_host_path(path):
    return lib().goofy_gpu_set_host_path(path)


def get_host_path():
    return lib().goofy_gpu_get_host_path()


def host_alloc(nbytes):
    return lib().goofy_gpu_host_alloc(nbytes)


def host_free(ptr):
    lib().goofy_gpu_host_free(ptr)


def get_tile(codec):
    t = Tile()
    rc = lib().goofy_gpu_get_tile(codec, ctypes.byref(t))
    if rc != OK:
        raise ValueError(status_string(rc))
    return (t.threads_per_cta, t.blocks_per_thread, t.persistent)


def set_tile(codec, threads_per_cta, blocks_per_thread, persistent=0):
    t = Tile(threads_per_cta, blocks_per_thread, persistent)
    return lib().goofy_gpu_set_tile(codec, ctypes.byref(t))


def reset_tiles():
    """Back to the compiled default tiles; the tile cache is read again on the
    next goofy_gpu_init or encode call."""
    return lib().goofy_gpu_reset_tiles()


def _enc(s):
    return None if s is None else os.fsencode(s)


def set_tile_cache_path(path):
    """Use `path` as the tile cache ("" disables it, None restores
    $GOOFY_TILE_CACHE / the per-user default)."""
    return lib().goofy_gpu_set_tile_cache_path(_enc(path))


def tile_cache_path():
    n = lib().goofy_gpu_get_tile_cache_path(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    lib().goofy_gpu_get_tile_cache_path(buf, n + 1)
    return os.fsdecode(buf.value)


def device_key(device=0):
    """(GPU name, SM count): the key of a device's tile cache entries."""
    buf = ctypes.create_string_buffer(256)
    sms = _U32()
    rc = lib().goofy_gpu_device_key(device, buf, 256, ctypes.byref(sms))
    if rc != OK:
        raise RuntimeError("device_key: %s %s" % (status_string(rc), last_error()))
    return buf.value.decode(), sms.value


def tile_cache_store(path, gpu_name, sm_count, codec, tile, us):
    t = Tile(*tile)
    return lib().goofy_gpu_tile_cache_store(_enc(path), gpu_name.encode(), sm_count, codec, ctypes.byref(t), us)


def tile_cache_lookup(path, gpu_name, sm_count, codec):
    """The recorded tile (threads, blocks a thread, mode) or None."""
    t = Tile()
    rc = lib().goofy_gpu_tile_cache_lookup(_enc(path), gpu_name.encode(), sm_count, codec, ctypes.byref(t))
    return (t.threads_per_cta, t.blocks_per_thread, t.persistent) if rc == OK else None


def load_tile_cache(device=0):
    """Install the cached tiles of `device` (codecs not set explicitly); the count installed."""
    return lib().goofy_gpu_load_tile_cache(device)


def pipeline_timeouts(reset=False):
    """Bulk-copy pipeline waits that gave up on the current device (0 when healthy)."""
    n = _U32()
    rc = lib().goofy_gpu_pipeline_timeouts(ctypes.byref(n), 1 if reset else 0)
    if rc != OK:
        raise RuntimeError("pipeline_timeouts: %s %s" % (status_string(rc), last_error()))
    return n.value


def selftest_bounded_wait():
    """(status, elapsed ms) of goofy_gpu_selftest_bounded_wait: a pipeline wait
    on a barrier nothing completes gives up after its limit and is counted."""
    ms = _U32()
    rc = lib().goofy_gpu_selftest_bounded_wait(ctypes.byref(ms))
    return rc, ms.value


def autotune(codec, dst, src, width, height, stride, reps=9):
    """Time every tile shape on a device image, install the fastest; returns
    ((threads_per_cta, blocks_per_thread, persistent), mean microseconds a launch)."""
    t = Tile()
    us = ctypes.c_float()
    rc = lib().goofy_gpu_autotune(codec, _addr(dst), _addr(src), width, height, stride, reps, ctypes.byref(t),
                                  ctypes.byref(us))
    if rc != OK:
        raise RuntimeError("autotune failed: %s %s" % (status_string(rc), last_error()))
    return (t.threads_per_cta, t.blocks_per_thread, t.persistent), us.value


def autotune_pair(dst_bc1, dst_etc1s, src, width, height, stride, reps=5):
    """Tune both codecs for alternating BC1 / ETC1s calls on one image; installs
    the pair.  Returns (bc1 tile, etc1s tile, mean microseconds of one pair)."""
    t0, t1 = Tile(), Tile()
    us = ctypes.c_float()
    rc = lib().goofy_gpu_autotune_pair(_addr(dst_bc1), _addr(dst_etc1s), _addr(src), width, height, stride, reps,
                                       ctypes.byref(t0), ctypes.byref(t1), ctypes.byref(us))
    if rc != OK:
        raise RuntimeError("autotune_pair failed: %s %s" % (status_string(rc), last_error()))
    return ((t0.threads_per_cta, t0.blocks_per_thread, t0.persistent),
            (t1.threads_per_cta, t1.blocks_per_thread, t1.persistent), us.value)


def out_size(width, height):
    """Bytes of encoded output: (width/4)*(height/4) blocks of 8 bytes."""
    return (width // 4) * (height // 4) * 8


def images_array(images):
    """ctypes array of Image from (src, dst, width, height, stride, codec) tuples or Image objects."""
    arr = (Image * len(images))()
    for i, im in enumerate(images):
        arr[i] = im if isinstance(im, Image) else Image(_addr(im[0]), _addr(im[1]), *im[2:])
    return arr


class Batch:
    """goofy_gpu_batch: many device images of uneven sizes per persistent launch."""

    def __init__(self, max_images, device=0):
        h = ctypes.c_void_p()
        rc = lib().goofy_gpu_batch_create(ctypes.byref(h), max_images, device)
        if rc != OK:
            raise RuntimeError("goofy_gpu_batch_create: %s %s" % (status_string(rc), last_error()))
        self._h = h

    def encode(self, images, stream=None):
        arr = images if isinstance(images, ctypes.Array) else images_array(images)
        return lib().goofy_gpu_batch_encode(self._h, arr, len(arr), stream)

    def set_graphs(self, enable):
        return lib().goofy_gpu_batch_set_graphs(self._h, 1 if enable else 0)

    def get_tile(self):
        """(threads_per_cta, blocks_per_thread, unit_blocks, pipeline)"""
        t = BatchTile()
        assert lib().goofy_gpu_batch_get_tile(self._h, ctypes.byref(t)) == OK
        return (t.threads_per_cta, t.blocks_per_thread, t.unit_blocks, t.pipeline)

    def set_tile(self, threads_per_cta, blocks_per_thread, unit_blocks, pipeline=0):
        t = BatchTile(threads_per_cta, blocks_per_thread, unit_blocks, pipeline)
        return lib().goofy_gpu_batch_set_tile(self._h, ctypes.byref(t))

    def autotune(self, images, reps=5):
        arr = images if isinstance(images, ctypes.Array) else images_array(images)
        t = BatchTile()
        us = ctypes.c_float()
        rc = lib().goofy_gpu_batch_autotune(self._h, arr, len(arr), reps, ctypes.byref(t), ctypes.byref(us))
        if rc != OK:
            raise RuntimeError("batch autotune: %s %s" % (status_string(rc), last_error()))
        return (t.threads_per_cta, t.blocks_per_thread, t.unit_blocks, t.pipeline), us.value

    def close(self):
        if self._h:
            lib().goofy_gpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_encode_noalloc(images, stream=None):
    """goofy_gpu_batch_encode_noalloc: a batch of at most NOALLOC_MAX_IMAGES
    images encoded without any allocation (scratch in a fixed device array of
    the library; calls sharing it must not overlap on the GPU)."""
    arr = images if isinstance(images, ctypes.Array) else images_array(images)
    return lib().goofy_gpu_batch_encode_noalloc(arr, len(arr), stream)


def requests_array(reqs):
    """ctypes array of Request from (src, dst, width, height, stride, codec) tuples."""
    arr = (Request * len(reqs))()
    for i, q in enumerate(reqs):
        arr[i] = q if isinstance(q, Request) else Request(_addr(q[0]), _addr(q[1]), *q[2:])
    return arr


class Server:
    """goofy_gpu_server: continuous-batching server for host-memory requests."""

    def __init__(self, mode=SERVER_STAGED, device_budget_bytes=16 << 30, max_batch_images=1024,
                 max_inflight_batches=4, max_requests=1 << 20, device=0, quality=False,
                 completion=None):
        cfg = ServerConfig()
        lib().goofy_gpu_server_default_config(ctypes.byref(cfg))
        cfg.device, cfg.mode, cfg.device_budget_bytes = device, mode, device_budget_bytes
        cfg.quality = 1 if quality else 0
        if completion is not None:
            cfg.completion = completion
        cfg.max_batch_images, cfg.max_inflight_batches, cfg.max_requests = (max_batch_images, max_inflight_batches,
                                                                            max_requests)
        h = ctypes.c_void_p()
        rc = lib().goofy_gpu_server_create(ctypes.byref(h), ctypes.byref(cfg))
        if rc != OK:
            raise RuntimeError("goofy_gpu_server_create: %s %s" % (status_string(rc), last_error()))
        self._h = h

    def submit(self, codec, dst, src, width, height, stride):
        """Returns (status, ticket)."""
        t = ctypes.c_uint64()
        q = Request(_addr(src), _addr(dst), width, height, stride, codec)
        rc = lib().goofy_gpu_server_submit(self._h, ctypes.byref(q), ctypes.byref(t))
        return rc, t.value

    def wait(self, ticket, timeout_ms=60000):
        """Returns (status, RequestTimes)."""
        tm = RequestTimes()
        rc = lib().goofy_gpu_server_wait(self._h, ticket, timeout_ms, ctypes.byref(tm))
        return rc, tm

    def stats(self):
        st = ServerStats()
        assert lib().goofy_gpu_server_get_stats(self._h, ctypes.byref(st)) == OK
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def replay(self, reqs, arrival_ns, with_times=False):
        """Open-loop replay; returns (status, latency_ns int64 array, wall_ns)
        and, with `with_times`, an (n, 4) int64 array of submit / admit /
        launch / done stamps."""
        import numpy as np

        arr = reqs if isinstance(reqs, ctypes.Array) else requests_array(reqs)
        arrival = np.ascontiguousarray(arrival_ns, dtype=np.int64)
        lat = np.zeros(len(arr), np.int64)
        wall = ctypes.c_int64()
        times = (RequestTimes * len(arr))() if with_times else None
        rc = lib().goofy_gpu_server_replay(self._h, arr, arrival.ctypes.data, len(arr), lat.ctypes.data,
                                           ctypes.byref(wall), times)
        if not with_times:
            return rc, lat, wall.value
        raw = np.ctypeslib.as_array(times)
        stamps = np.stack([raw[k] for k in ("submit_ns", "admit_ns", "launch_ns", "done_ns")], axis=1)
        self.last_psnr = np.array(raw["psnr_rgb"])
        return rc, lat, wall.value, stamps

    def close(self):
        if self._h:
            lib().goofy_gpu_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plain_replay(reqs, arrival_ns, device=0):
    """The plain loop (one request per launch, sequential); (status, latency_ns, wall_ns)."""
    import numpy as np

    arr = reqs if isinstance(reqs, ctypes.Array) else requests_array(reqs)
    arrival = np.ascontiguousarray(arrival_ns, dtype=np.int64)
    lat = np.zeros(len(arr), np.int64)
    wall = ctypes.c_int64()
    rc = lib().goofy_gpu_plain_replay(device, arr, arrival.ctypes.data, len(arr), lat.ctypes.data, ctypes.byref(wall))
    return rc, lat, wall.value


def pinned_array(nbytes):
    """numpy uint8 view of a fresh pinned host buffer (freed with free_pinned)."""
    import numpy as np

    p = host_alloc(nbytes)
    if not p:
        raise MemoryError("pinned allocation of %d bytes failed" % nbytes)
    return np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p)), p


def decode_device(codec, rgba, rgba_stride, blocks, width, height, d_unsupported, stream=None):
    """GPU decode of device blocks into device RGBA8 rows (see goofy_gpu_decode_device)."""
    return lib().goofy_gpu_decode_device(codec, _addr(rgba), rgba_stride, _addr(blocks), width, height,
                                         _addr(d_unsupported), stream)


ERROR_SUMS = 6  # device accumulators goofy_gpu_block_error_device adds to


def block_error_device(codec, blocks, src, width, height, stride, d_sums, stream=None):
    """Adds the six error sums (see goofy_gpu_block_error_device) to device uint64[6] `d_sums`."""
    if hasattr(d_sums, "numel") and d_sums.numel() * d_sums.element_size() < 8 * ERROR_SUMS:
        raise ValueError("d_sums must hold %d uint64 accumulators" % ERROR_SUMS)
    return lib().goofy_gpu_block_error_device(codec, _addr(blocks), _addr(src), width, height, stride,
                                              _addr(d_sums), stream)


def psnr_rgb(codec, blocks, src, width, height, stride):
    """(status, RGB PSNR as the reference reports it, [sumR, sumG, sumB, sumA, unsupported])."""
    import numpy as np

    out = ctypes.c_double()
    sums = np.zeros(5, np.uint64)
    rc = lib().goofy_gpu_psnr_rgb(codec, _addr(blocks), _addr(src), width, height, stride, ctypes.byref(out),
                                  sums.ctypes.data)
    return rc, out.value, sums


def mse_psnr(codec, blocks, src, width, height, stride):
    """The harness's getMsePsnr of device `src` against its decoded device
    `blocks`, computed on the GPU; a dict of the MsePsnr fields."""
    q = Quality()
    rc = lib().goofy_gpu_mse_psnr(codec, _addr(blocks), _addr(src), width, height, stride, ctypes.byref(q))
    if rc != OK:
        raise RuntimeError("mse_psnr: %s %s" % (status_string(rc), last_error()))
    return {n: getattr(q, n) for n, _ in Quality._fields_}


def container(codec, levels):
    """DDS (BC1) / KTX (ETC1s) file bytes from [(blocks, width, height), ...] host levels."""
    import numpy as np

    n = len(levels)
    blocks = [np.ascontiguousarray(b, dtype=np.uint8) for b, _, _ in levels]
    ptrs = (ctypes.c_void_p * n)(*[b.ctypes.data for b in blocks])
    ws = (ctypes.c_uint32 * n)(*[w for _, w, _ in levels])
    hs = (ctypes.c_uint32 * n)(*[h for _, _, h in levels])
    size = lib().goofy_gpu_container_size(codec, ws, hs, n)
    if size == 0:
        raise ValueError("invalid container levels")
    out = np.zeros(size, np.uint8)
    rc = lib().goofy_gpu_write_container(codec, ptrs, ws, hs, n, out.ctypes.data, size)
    if rc != OK:
        raise RuntimeError(status_string(rc))
    return out.tobytes()


def generate_mips(src, width, height, stride, arena, arena_bytes, stream=None):
    """Device mip chain of `src` into `arena`; returns [(ptr, w, h, stride), ...] (level 0 = src)."""
    n = lib().goofy_gpu_mip_count(width, height)
    levels = (Level * max(n, 1))()
    count = ctypes.c_uint32()
    rc = lib().goofy_gpu_generate_mips(_addr(src), width, height, stride, _addr(arena), arena_bytes, levels,
                                       max(n, 1), ctypes.byref(count), stream)
    if rc != OK:
        raise RuntimeError("generate_mips: %s %s" % (status_string(rc), last_error()))
    return [(levels[i].data, levels[i].width, levels[i].height, levels[i].stride) for i in range(count.value)]


def read_png(source, opaque=True, stride=None):
    """Decode a PNG (path or bytes) with the library's decoder into a numpy
    RGBA8 image of shape (height, stride); returns (image, width, height)."""
    import numpy as np

    data = source if isinstance(source, (bytes, bytearray)) else open(source, "rb").read()
    buf = ctypes.create_string_buffer(bytes(data), len(data))
    w, h = _U32(), _U32()
    rc = lib().goofy_gpu_png_info(buf, len(data), ctypes.byref(w), ctypes.byref(h))
    if rc != OK:
        raise ValueError("png: %s %s" % (status_string(rc), last_error()))
    stride = stride or 4 * w.value
    img = np.zeros((h.value, stride), np.uint8)
    rc = lib().goofy_gpu_png_decode(buf, len(data), img.ctypes.data, img.nbytes, stride, 1 if opaque else 0,
                                    ctypes.byref(w), ctypes.byref(h))
    if rc != OK:
        raise ValueError("png: %s %s" % (status_string(rc), last_error()))
    return img, w.value, h.value


def tga(rgba, width, height):
    """The harness's TGA file bytes (saveTga) of a host RGBA8 image (rows of its stride)."""
    import numpy as np

    img = np.ascontiguousarray(rgba)
    n = lib().goofy_gpu_tga_size(width, height)
    if n == 0:
        raise ValueError("tga: unsupported size %dx%d" % (width, height))
    out = np.zeros(n, np.uint8)
    rc = lib().goofy_gpu_write_tga(img.ctypes.data, img.strides[0], width, height, out.ctypes.data, n)
    if rc != OK:
        raise RuntimeError("tga: %s %s" % (status_string(rc), last_error()))
    return out.tobytes()
