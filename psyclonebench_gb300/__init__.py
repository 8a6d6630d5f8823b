"""GB300-native NEMOLite2D time step behind the PSyKAl C boundary of
stfc/PSycloneBench's manual C/C++ version.

The compute path is the in-tree C-ABI library ``_lib/libnl2d_gpu.so``
(hand-written sm_103a CUDA; declared in ``include/nl2d_gpu.h``).  There is
no CPU fallback: importing the bindings without the built library raises.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libnl2d_gpu.so")

NL2D_OK = 0
NL2D_ERR_CUDA = 1
NL2D_ERR_ARGS = 2
NL2D_ERR_STATE = 3
NL2D_ERR_UNKNOWN_FIELD = 4
NL2D_ERR_NONFINITE = 5
NL2D_ERR_TOO_LARGE = 6
NL2D_ERR_IO = 7
NL2D_ERR_PARSE = 8
NL2D_MODE_AUTO = 0
NL2D_MODE_REFERENCE = 1

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p

# Argument list of c_invoke_time_step (psykal_cpp/time_step.cpp:10-51 plus
# height, psykal_cpp/time_step_mod.f90:8-31).
STEP_ARGTYPES = ([_DP] * 13 + [_IP] + [_DP] * 11 + [ctypes.c_int] * 7 +
                 [ctypes.c_double] * 6)
REGISTER_ARGTYPES = ([_DP] * 13 + [_IP] + [_DP] * 11 + [ctypes.c_int] * 6 +
                     [ctypes.c_double] * 6)

# Every symbol include/nl2d_gpu.h declares, with (restype, argtypes).
EXPORTS = {
    "c_invoke_time_step": (None, STEP_ARGTYPES),
    "c_read_from_device": (None, [_VP, _VP] + [ctypes.c_int] * 4 + [ctypes.c_bool]),
    "c_write_to_device": (None, [_VP, _VP] + [ctypes.c_int] * 4 + [ctypes.c_bool]),
    "nl2d_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "nl2d_finalize": (None, []),
    "nl2d_set_mode": (ctypes.c_int, [ctypes.c_int]),
    "nl2d_last_path": (ctypes.c_int, []),
    "nl2d_set_precision": (ctypes.c_int, [ctypes.c_int]),
    "nl2d_register": (ctypes.c_int, REGISTER_ARGTYPES),
    "nl2d_run_steps": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _DP]),
    "nl2d_timed_run": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP]),
    "nl2d_checksums": (ctypes.c_int, [_DP]),
    "nl2d_field_checksum": (ctypes.c_int, [_VP] + [ctypes.c_int] * 4 + [_DP]),
    "nl2d_field_checksum_noalloc": (ctypes.c_int, [_VP] + [ctypes.c_int] * 5 + [_VP, _VP]),
    "nl2d_selftest_exact": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_ulonglong,
                                            ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_longlong)]),
    "nl2d_selftest_intfp": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_ulonglong,
                                            ctypes.POINTER(ctypes.c_longlong)]),
    "nl2d_ens_create": (ctypes.c_int, [ctypes.c_int, _IP, _DP, _DP, _DP]),
    "nl2d_ens_set_domain": (ctypes.c_int, [ctypes.c_int, _IP, _DP, _DP, _DP]),
    "nl2d_ens_schedule": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "nl2d_ens_tile": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "nl2d_host_register": (ctypes.c_int, [_VP, ctypes.c_size_t]),
    "nl2d_host_unregister": (ctypes.c_int, [_VP]),
    "nl2d_speculation_counts": (ctypes.c_int, [_IP]),
    "nl2d_ens_run": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _DP, _DP]),
    "nl2d_ens_read": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _DP]),
    "nl2d_ens_info": (ctypes.c_int, [ctypes.POINTER(ctypes.c_longlong), _IP, _IP]),
    "nl2d_ens_reset": (ctypes.c_int, []),
    "nl2d_ens_set_precision": (ctypes.c_int, [ctypes.c_int]),
    "nl2d_ens_destroy": (None, []),
    "nl2d_emu_conv3x3": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP] + [ctypes.c_int] * 6 +
                         [_VP, _VP]),
    "nl2d_emu_flip_transpose": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_int, _VP]),
    "nl2d_emu_conv_wgrad": (ctypes.c_int, [_VP, _VP, _VP, _VP] + [ctypes.c_int] * 5 +
                            [_VP, _VP]),
    "nl2d_emu_relu_bwd": (ctypes.c_int, [_VP, _VP, _VP, ctypes.c_longlong, _VP]),
    "nl2d_emu_mse": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_longlong, ctypes.c_int,
                                    ctypes.c_int, _VP]),
    "nl2d_emu_adam": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_int] +
                      [ctypes.c_float] * 4 + [ctypes.c_int, _VP]),
    "nl2d_emu_assemble": (ctypes.c_int, [_VP] * 6 + [ctypes.c_ulonglong, _VP, _VP] +
                          [ctypes.c_int] * 4 + [_VP]),
    "nl2d_emu_advance": (ctypes.c_int, [_VP] * 6 + [ctypes.c_longlong, ctypes.c_longlong,
                                                 ctypes.c_int, _VP]),
    "nl2d_ens_export_interior": (ctypes.c_int, [_VP]),
    "nl2d_ens_uses_march": (ctypes.c_int, []),
    "nl2d_selftest_wait": (ctypes.c_int, [ctypes.c_longlong, _IP]),
    "nl2d_selftest_df": (ctypes.c_int, [_DP, ctypes.c_longlong, _VP, _VP, _DP, _DP]),
    "nl2d_checkpoint_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "nl2d_checkpoint_read": (ctypes.c_int, [ctypes.c_char_p, _IP]),
    "nl2d_ens_import_interior": (ctypes.c_int, [_VP]),
    "nl2d_read_namelist": (ctypes.c_int, [ctypes.c_char_p, _IP, _DP]),
    "nl2d_setup_model": (ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_double] * 3 +
                         [ctypes.c_int] * 2 + [ctypes.POINTER(_DP), _IP, ctypes.POINTER(_DP),
                                               _DP, _DP]),
    "nl2d_model_write": (ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_int] * 7 + [_DP] * 6),
    "nl2d_dump_tmask": (ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_int] * 5 + [_IP] +
                        [ctypes.c_int] * 4 + [_DP, _DP]),
    "nl2d_read_grid_file": (ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_int] * 4 + [_VP]),
    "nl2d_face_depths": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, _DP, _DP]),
    "nl2d_format_e": (ctypes.c_int, [ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_char_p, ctypes.c_int]),
    "tra_adv_compute": (None, [_DP] * 12 + [ctypes.c_int] * 3),
    "tra_adv_run": (ctypes.c_int, [ctypes.c_int, _DP]),
    "tra_adv_read": (ctypes.c_int, [_DP]),
    "tra_adv_checksum": (ctypes.c_int, [_DP]),
    "tra_adv_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "tra_adv_finalize": (None, []),
    "nl2d_sync": (ctypes.c_int, []),
    "nl2d_transfer_bytes": (ctypes.c_int, [ctypes.POINTER(ctypes.c_longlong)]),
    "nl2d_measure_pipe_rates": (ctypes.c_int, [_DP]),
    "nl2d_device_ptr": (ctypes.c_void_p, [_VP]),
}

_lib = None


class Nl2dError(RuntimeError):
    pass


def load_library(path=LIB_PATH):
    """Loads the CUDA library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise Nl2dError(
            "libnl2d_gpu.so is missing (%s); build it with "
            "`python -m psyclonebench_gb300.build` or __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc=None, what="nl2d"):
    """Raises Nl2dError if `rc` (or the library's sticky status) is an error."""
    lib = load_library()
    if rc is None or rc != NL2D_OK:
        buf = ctypes.create_string_buffer(512)
        st = lib.nl2d_last_error(buf, 512)
        if rc is None:
            rc = st
        if rc != NL2D_OK:
            raise Nl2dError("%s failed (%d): %s" % (what, rc, buf.value.decode()))
