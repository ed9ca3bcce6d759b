"""Loader for the in-tree C-ABI library libmm3e_cuda.so (built by mm3e_cuda.build).

There is no fallback: if the library is missing, every entry point raises. The library is
never installed into site-packages, so the process maps it from this package directory.
"""
import ctypes as C
import os

from . import abi

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_lib", "libmm3e_cuda.so")

_lib = None


class NativeLibraryMissing(RuntimeError):
    pass


def _declare(lib):
    P = C.POINTER
    f = C.c_float
    sig = {
        "mm3e_abi_version": (C.c_int, []),
        "mm3e_camera_look_at": (None, [P(f), P(f), P(f), f, P(abi.Camera)]),
        "mm3e_orbit_camera": (None, [P(f), f, f, f, f, P(abi.Camera)]),
        "mm3e_mat3_from_euler": (None, [f, f, f, P(f)]),
        "mm3e_quat_to_mat3": (None, [P(f), P(f)]),
        "mm3e_light_directional": (None, [P(f), P(f), P(abi.Light)]),
        "mm3e_scene_validate": (C.c_int, [P(abi.SceneDesc), C.c_char_p, C.c_size_t]),
        "mm3e_scene_tape_bytes": (C.c_int, [P(abi.SceneDesc), P(C.c_size_t)]),
        "mm3e_ctx_create": (C.c_int, [C.c_int, P(C.c_void_p)]),
        "mm3e_ctx_destroy": (None, [C.c_void_p]),
        "mm3e_last_error": (C.c_char_p, [C.c_void_p]),
        "mm3e_ctx_sync": (C.c_int, [C.c_void_p]),
        "mm3e_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
        "mm3e_ctx_device_info": (C.c_int, [C.c_void_p, P(C.c_int), P(C.c_int)]),
        "mm3e_scene_compile": (C.c_int, [C.c_void_p, P(abi.SceneDesc), P(C.c_void_p)]),
        "mm3e_scene_destroy": (None, [C.c_void_p]),
        "mm3e_render": (C.c_int, [C.c_void_p, P(abi.Camera), P(abi.DynSphere), C.c_size_t, C.c_uint32, C.c_void_p,
                                  C.c_size_t, P(abi.RenderStats)]),
        "mm3e_render_linear": (C.c_int, [C.c_void_p, P(abi.Camera), P(f), C.c_size_t]),
        "mm3e_render_device": (C.c_int, [C.c_void_p, P(abi.Camera), C.c_uint32, C.c_void_p, C.c_size_t]),
        "mm3e_bake_gi": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
        "mm3e_scene_get_gi": (C.c_int, [C.c_void_p, P(f), P(f), P(C.c_uint32), P(f), C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _declare_extra(lib)


def _declare_extra(lib):
    """Entry points beyond the core set (diagnostics, batched and served forms)."""
    P = C.POINTER
    extra = {
        "mm3e_render_hits": (C.c_int, [C.c_void_p, P(abi.Camera), P(C.c_float), P(C.c_uint32), P(C.c_uint32),
                                       P(C.c_float)]),
        "mm3e_march_rays": (C.c_int, [C.c_void_p, P(C.c_float), C.c_size_t, P(C.c_float), P(C.c_uint32),
                                      P(C.c_uint32)]),
        "mm3e_field": (C.c_int, [C.c_void_p, P(C.c_float), C.c_size_t, P(C.c_float), P(C.c_uint32)]),
        "mm3e_march_rays_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                              C.c_void_p]),
        "mm3e_ctx_set_tuning": (C.c_int, [C.c_void_p, P(abi.Tuning)]),
        "mm3e_ctx_get_tuning": (C.c_int, [C.c_void_p, P(abi.Tuning)]),
        "mm3e_ctx_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
        "mm3e_ctx_set_host_writes": (C.c_int, [C.c_void_p, C.c_int, P(C.c_int)]),
        "mm3e_ctx_set_tape_wait": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int]),
        "mm3e_ctx_kernel_times": (C.c_int, [C.c_void_p, P(abi.KernelTime), C.c_uint32, P(C.c_uint32)]),
        "mm3e_scene_device_bytes": (C.c_int, [C.c_void_p, P(C.c_size_t)]),
        "mm3e_batch_configure": (C.c_int, [C.c_void_p, P(abi.BatchConfig)]),
        "mm3e_render_batch": (C.c_int, [C.c_void_p, P(abi.Job), C.c_size_t, P(abi.BatchStats)]),
        "mm3e_bake_mesh_sdf": (C.c_int, [C.c_void_p, P(abi.Mesh), C.c_uint32, C.c_float, P(abi.Volume),
                                         C.c_void_p, C.c_size_t, C.c_int]),
        "mm3e_server_create": (C.c_int, [C.c_void_p, P(abi.ServerConfig), P(C.c_void_p)]),
        "mm3e_server_add_scene": (C.c_int, [C.c_void_p, P(abi.SceneDesc), P(C.c_uint32)]),
        "mm3e_server_submit": (C.c_int, [C.c_void_p, P(abi.Request), P(C.c_uint64)]),
        "mm3e_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, P(abi.RequestResult)]),
        "mm3e_server_get_stats": (C.c_int, [C.c_void_p, P(abi.ServerStats)]),
        "mm3e_server_replay": (C.c_int, [C.c_void_p, P(abi.Request), P(C.c_double), C.c_size_t,
                                         P(abi.RequestResult)]),
        "mm3e_server_destroy": (None, [C.c_void_p]),
        "mm3e_scene_specialize": (C.c_int, [C.c_void_p, C.c_int, P(C.c_double)]),
        "mm3e_scene_is_specialized": (C.c_int, [C.c_void_p]),
        "mm3e_scene_spec_source": (C.c_int, [P(abi.SceneDesc), C.c_char_p, C.c_size_t, P(C.c_size_t)]),
        "mm3e_scene_tape": (C.c_int, [P(abi.SceneDesc), C.c_void_p, C.c_size_t, P(C.c_size_t)]),
        "mm3e_spec_compile_check": (C.c_int, [P(abi.SceneDesc), C.c_char_p, C.c_size_t, P(C.c_double)]),
        "mm3e_render_film": (C.c_int, [C.c_void_p, P(abi.Camera), C.c_float, C.c_float, P(C.c_float), P(C.c_float),
                                       P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_uint32)]),
        "mm3e_render_gbuffer": (C.c_int, [C.c_void_p, P(abi.Camera), P(C.c_float), C.c_uint32, P(C.c_uint8),
                                          P(C.c_float), P(C.c_int32)]),
        "mm3e_reproject": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, P(abi.Camera), P(C.c_uint8), P(C.c_float),
                                     P(C.c_int32), P(abi.Camera), P(C.c_float), C.c_uint32, C.c_void_p,
                                     P(C.c_uint8)]),
        "mm3e_scene_parse_mm3e": (C.c_int, [C.c_char_p, P(C.c_void_p), C.c_char_p, C.c_size_t]),
        "mm3e_parsed_scene_desc": (P(abi.SceneDesc), [C.c_void_p]),
        "mm3e_parsed_scene_camera": (C.c_int, [C.c_void_p, P(abi.Camera)]),
        "mm3e_parsed_scene_free": (None, [C.c_void_p]),
        "mm3e_scene_write_mm3e": (C.c_int, [P(abi.SceneDesc), P(abi.Camera), C.c_char_p, C.c_size_t, P(C.c_size_t),
                                            C.c_char_p, C.c_size_t]),
        "mm3e_volume_parse_sdfv": (C.c_int, [P(C.c_uint8), C.c_size_t, P(abi.Volume), P(C.c_float), C.c_size_t,
                                             P(C.c_size_t), C.c_char_p, C.c_size_t]),
        "mm3e_volume_write_sdfv": (C.c_int, [P(abi.Volume), P(C.c_uint8), C.c_size_t, P(C.c_size_t), C.c_char_p,
                                             C.c_size_t]),
        "mm3e_scene_autotune": (C.c_int, [C.c_void_p, P(abi.Camera), C.c_int, P(abi.Tuning), C.c_uint32, C.c_uint32,
                                          P(abi.Tuning), P(abi.TuneEntry), C.c_uint32, P(C.c_uint32)]),
        "mm3e_autotune": (C.c_int, [C.c_void_p, P(abi.Job), C.c_size_t, C.c_uint32, P(abi.Tuning),
                                    P(abi.TuneEntry), C.c_uint32, P(C.c_uint32)]),
    }
    for name, (res, args) in extra.items():
        fn = getattr(lib, name, None)
        if fn is not None:
            fn.restype = res
            fn.argtypes = args


def lib():
    """The loaded library (raises NativeLibraryMissing if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryMissing(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        l = C.CDLL(LIB_PATH)
        _declare(l)
        if l.mm3e_abi_version() != abi.ABI_VERSION:
            raise NativeLibraryMissing("libmm3e_cuda.so ABI version mismatch; rebuild")
        _lib = l
    return _lib


def fptr(seq, n=None):
    arr = (C.c_float * (n if n is not None else len(seq)))(*seq)
    return arr
