"""Loader for the in-tree native libraries.

The CUDA library is mandatory: there is no CPU fallback for any operation of
this package, so a missing or unloadable library raises immediately.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

_libs = {}

GBT_OK = 0
STATUS = {0: "GBT_OK", 1: "GBT_E_INVALID", 2: "GBT_E_CUDA", 3: "GBT_E_OOM", 4: "GBT_E_CAPACITY", 5: "GBT_E_TIMEOUT", 6: "GBT_E_TOO_LARGE"}


class GbtError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s%s" % (STATUS.get(code, code), (": " + msg) if msg else ""))
        self.code = code


def _load(name):
    if name in _libs:
        return _libs[name]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        raise RuntimeError(
            "%s is not built (expected at %s); run cuimg_gb300.build.build() or __graft_entry__.build()" % (name, path))
    lib = ctypes.CDLL(path)
    _libs[name] = lib
    return lib


def cuda_lib():
    lib = _load("libcuimg_gb300.so")
    if not getattr(lib, "_typed", False):
        _declare(lib)
        lib._typed = True
    return lib


def synth_lib():
    lib = _load("libgbt_synth.so")
    if not getattr(lib, "_typed", False):
        lib.synth_create.restype = ctypes.c_void_p
        lib.synth_create.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
        lib.synth_destroy.argtypes = [ctypes.c_void_p]
        lib.synth_frame_u8.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.synth_frame_rgb.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.synth_frame_f32.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_void_p]
        lib.synth_true_flow.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        lib._typed = True
    return lib


class gbt_config(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "rows", "cols", "nscales", "detector_threshold", "detector_n", "detector_frequency",
        "filtering_frequency", "k", "with_merge", "detector", "detector_step", "detector_grad_th", "matcher")]


def _declare(lib):
    P = ctypes.c_void_p
    I32 = ctypes.c_int32
    I32P = ctypes.POINTER(ctypes.c_int32)
    lib.gbt_config_default.argtypes = [ctypes.POINTER(gbt_config), I32, I32, I32]
    lib.gbt_config_default.restype = None
    lib.gbt_sizes_ok.argtypes = [I32, I32, I32]
    lib.gbt_create.argtypes = [ctypes.POINTER(gbt_config), I32, I32, ctypes.POINTER(P)]
    lib.gbt_create_ex.argtypes = [ctypes.POINTER(gbt_config), I32, I32, I32, ctypes.POINTER(P)]
    lib.gbt_groups.argtypes = [P, ctypes.POINTER(I32)]
    lib.gbt_destroy.argtypes = [P]
    lib.gbt_last_error.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    lib.gbt_run.argtypes = [P, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_int64), I32]
    lib.gbt_run_resident.argtypes = [P]
    lib.gbt_input_slot.argtypes = [P, I32, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_int64)]
    lib.gbt_use_graphs.argtypes = [P, I32]
    lib.gbt_test_withhold_tile_copies.argtypes = [P, I32]
    lib.gbt_test_tile_capacity.argtypes = [P, I32]
    lib.gbt_test_tile_fallbacks.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    lib.gbt_sync.argtypes = [P]
    lib.gbt_stream.argtypes = [P, ctypes.POINTER(P)]
    lib.gbt_nparticles.argtypes = [P, I32, I32, I32P]
    lib.gbt_get_particles.argtypes = [P, I32, I32, P, P, P, P, P, I32P, I32P]
    lib.gbt_get_particles_f.argtypes = [P, I32, I32, P, P, P, P, I32P, I32P]
    lib.gbt_get_stage.argtypes = [P, I32, I32, I32, I32, P]
    lib.gbt_bins.argtypes = [P, I32, I32, I32P, I32P]
    lib.gbt_get_bins.argtypes = [P, I32, I32, P, P, P, P]
    lib.gbt_frame_count.argtypes = [P, I32, I32, I32P]
    lib.gbt_kernels_per_frame.argtypes = [P, I32P]
    lib.gbt_kernel_launches.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    lib.gbt_trajectories_enable.argtypes = [P, I32]
    lib.gbt_set_rgb_to_gray.argtypes = [P, I32]
    lib.gbt_checkpoint_size.argtypes = [P, ctypes.POINTER(ctypes.c_size_t)]
    lib.gbt_checkpoint_save.argtypes = [P, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    lib.gbt_checkpoint_load.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    lib.gbt_get_trajectories.argtypes = [P, I32, I32, P, P, I32P, I32P]
    lib.gbt_read_counts.argtypes = [P, P, I32]
    lib.gbt_read_counts_async.argtypes = [P, P, I32]
    lib.gbt_set_tuning.argtypes = [P, I32, I32]
    lib.gbt_get_tuning.argtypes = [P, I32, I32P]
    lib.gbt_profile_enable.argtypes = [P, I32]
    lib.gbt_profile_read.argtypes = [P, I32, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double), I32P]
    lib.gbt_set_param.argtypes = [P, I32, I32, I32, I32]
    lib.gbt_get_param.argtypes = [P, I32, I32, I32, I32P]
    if hasattr(lib, "gbt_gaussian_taps"):
        lib.gbt_gaussian_taps.argtypes = [ctypes.c_float, P, I32P]
        lib.gbt_gaussian_f32.argtypes = [P, ctypes.c_int64, P, ctypes.c_int64, I32, I32, ctypes.c_float, P]
        lib.gbt_gaussian_f32_batch.argtypes = [P, ctypes.c_int64, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int64,
                                               I32, I32, I32, ctypes.c_float, P]
        lib.gbt_gaussian_pyramid_f32.argtypes = [P, ctypes.c_int64, I32, I32, I32, P, P]
        lib.gbt_pyramid_u8.argtypes = [P, ctypes.c_int64, I32, I32, I32, P, P]


def check(code, ctx=None):
    if code != GBT_OK:
        msg = ""
        if ctx:
            buf = ctypes.create_string_buffer(512)
            cuda_lib().gbt_last_error(ctx, buf, 512)
            msg = buf.value.decode(errors="replace")
        raise GbtError(code, msg)
