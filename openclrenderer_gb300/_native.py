"""Build and load libgbr.so, the CUDA sm_103a pipeline behind include/gbr.h.

There is no fallback: if the library cannot be built or loaded, every call
raises.  The library is built in-tree (openclrenderer_gb300/_lib/).
"""
import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libgbr.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
SOURCES = ["gbr_kernels.cu", "gbr_api.cu", "gbr_batch.cu", "gbr_noalloc.cu", "gbr_server.cu", "gbr_post.cu"]
HEADERS = ["gbr_math.h", "gbr_internal.h", "gbr_scene.h", "gbr_post.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(INCLUDE, "gbr.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile every translation unit for sm_103a (in parallel) and link libgbr.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class GbrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"gbr status {status}: {msg}")
        self.status = status


STATUS = {0: "GBR_OK", 1: "GBR_INVALID_ARG", 2: "GBR_OOM", 3: "GBR_BIN_OVERFLOW_RETRY",
          4: "GBR_DEVICE_TIMEOUT", 5: "GBR_INTERNAL", 6: "GBR_CUDA_ERROR", 7: "GBR_ADMISSION_REJECTED"}

# exported symbols and their ctypes signatures (must match include/gbr.h)
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
SIGNATURES = {
    "gbr_last_error_string": (ctypes.c_char_p, []),
    "gbr_fov_const_from_hfov": (ctypes.c_float, [ctypes.c_float, ctypes.c_int32]),
    "gbr_scene_create": (ctypes.c_int, [_P]),
    "gbr_scene_destroy": (ctypes.c_int, [_P]),
    "gbr_scene_set_triangles": (ctypes.c_int, [_P, _P, _U32]),
    "gbr_scene_set_descriptors": (ctypes.c_int, [_P, _P, _U32]),
    "gbr_scene_set_lights": (ctypes.c_int, [_P, _P, _U32]),
    "gbr_scene_set_textures": (ctypes.c_int, [_P, _U32, _P, _P]),
    "gbr_scene_texture_layout": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "gbr_scene_buffer": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "gbr_scene_read_buffer": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_size_t, ctypes.c_size_t]),
    "gbr_texture_pack": (ctypes.c_int, [_U32, _P, _P, _P, _P, _P]),
    "gbr_shadow_pass": (ctypes.c_int, [_P, _P]),
    "gbr_render_view": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "gbr_render_view_host": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "gbr_render_batch": (ctypes.c_int, [_P, _U32, _P, _P, _P, _P]),
    "gbr_scene_stats": (ctypes.c_int, [_P, _P]),
    "gbr_scene_profile": (ctypes.c_int, [_P, ctypes.c_int32]),
    "gbr_framebuffer_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P]),
    "gbr_framebuffer_outputs": (ctypes.c_int, [_P, _P, _P, _P]),
    "gbr_framebuffer_read": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_size_t]),
    "gbr_framebuffer_destroy": (ctypes.c_int, [_P]),
    "gbr_scene_set_tuning": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    "gbr_scene_get_tuning": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    "gbr_batch_create": (ctypes.c_int, [_P, _U32, _P, _P, ctypes.c_int32, _P]),
    "gbr_batch_launch": (ctypes.c_int, [_P, _P, _P]),
    "gbr_batch_wait": (ctypes.c_int, [_P]),
    "gbr_batch_wait_for": (ctypes.c_int, [_P, ctypes.c_int32]),
    "gbr_batch_render": (ctypes.c_int, [_P, _P, _P]),
    "gbr_batch_autotune": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P, _P, _P]),
    "gbr_batch_set_tuning": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    "gbr_batch_get_tuning": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    "gbr_batch_get_info": (ctypes.c_int, [_P, _P]),
    "gbr_batch_destroy": (ctypes.c_int, [_P]),
    "gbr_render_view_noalloc": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "gbr_post_godrays": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "gbr_render_view_blend": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "gbr_post_pseudo_aa": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "gbr_post_reflections": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "gbr_post_motion_blur": (ctypes.c_int, [_P, _P, _P, _P, _U32, ctypes.c_float, ctypes.c_float, _P, _P, _P, _P,
                                            _P]),
    "gbr_scene_flush_objects": (ctypes.c_int, [_P, _P, _U32]),
    "gbr_atomic_rate": (ctypes.c_int, [ctypes.c_int32, _P]),
    "gbr_scene_get_descriptors": (ctypes.c_int, [_P, _P, _U32]),
    "gbr_server_create": (ctypes.c_int, [_P, _U32, _P, _P]),
    "gbr_server_submit": (ctypes.c_int, [_P, _P, _P]),
    "gbr_server_poll": (ctypes.c_int, [_P, _P, _U32, _P, ctypes.c_int32]),
    "gbr_server_drain": (ctypes.c_int, [_P]),
    "gbr_server_drain_for": (ctypes.c_int, [_P, ctypes.c_int32]),
    "gbr_server_stats_get": (ctypes.c_int, [_P, _P]),
    "gbr_server_destroy": (ctypes.c_int, [_P]),
}

_lib = None


def load(path=None):
    """Load libgbr.so (building it if needed) and bind every symbol."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None:
        build()
        path = LIB
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status):
    if status != 0:
        msg = load().gbr_last_error_string().decode(errors="replace")
        raise GbrError(STATUS.get(status, status), msg)
