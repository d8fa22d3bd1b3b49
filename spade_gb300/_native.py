"""Loader for libgbns.so (the CUDA library).  No fallback: if the library is
missing or fails to load, every entry point raises."""
import ctypes
import os

from . import _abi

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libgbns.so")


class SpadeError(RuntimeError):
    """Raised for any nonzero libgbns return code (the reference raises
    except::sp_exception, core/except.h:12-15)."""

    def __init__(self, code, msg):
        super().__init__("gbns error %d: %s" % (code, msg))
        self.code = code


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise SpadeError(_abi.ERR_UNSUPPORTED,
                         "libgbns.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    L.gbns_version.restype = ctypes.c_int
    L.gbns_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.gbns_array_size.argtypes = [P(_abi.GridDesc), P(ctypes.c_size_t)]
    L.gbns_flux_div.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, ctypes.c_int, vp]
    L.gbns_flux_div_variant.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, ctypes.c_int, ctypes.c_int, vp]
    L.gbns_flux_variant_count.argtypes = [P(_abi.SchemeDesc)]
    L.gbns_fill_ghosts.argtypes = [P(_abi.GridDesc), P(_abi.BcDesc), vp, vp]
    L.gbns_exchange_plan_create.argtypes = [P(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            vp, ctypes.c_int, vp]
    L.gbns_exchange_plan_run.argtypes = [vp, vp, vp]
    L.gbns_exchange_plan_waves.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                           ctypes.c_int, vp]
    L.gbns_exchange_plan_destroy.argtypes = [vp]
    L.gbns_rk_stage.argtypes = [P(_abi.GridDesc), P(_abi.GasDesc), vp, vp, vp, ctypes.c_int, vp]
    L.gbns_reduce.argtypes = [P(_abi.GridDesc), P(_abi.GasDesc), vp, ctypes.c_int, vp, vp]
    L.gbns_reduce_scratch_size.argtypes = [P(_abi.GridDesc), P(ctypes.c_size_t), P(ctypes.c_size_t)]
    L.gbns_reduce_async.argtypes = [P(_abi.GridDesc), P(_abi.GasDesc), vp, ctypes.c_int, vp, ctypes.c_size_t, vp]
    L.gbns_reduce_noalloc.argtypes = [P(_abi.GridDesc), P(_abi.GasDesc), vp, ctypes.c_int, vp, vp]
    L.gbns_flux_div_rk.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp]
    L.gbns_copy_fill_ghosts.argtypes = [P(_abi.GridDesc), P(_abi.BcDesc), vp, vp, vp]
    L.gbns_ssprk3_step.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), P(_abi.BcDesc), vp, vp, ctypes.c_double, vp]
    L.gbns_ssprk3_run.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), P(_abi.BcDesc), vp, vp, ctypes.c_double,
                                  ctypes.c_int, vp]
    L.gbns_ssprk3_step_host.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), P(_abi.BcDesc), vp, vp, vp,
                                        ctypes.c_double, ctypes.c_int, vp, vp]
    L.gbns_source_term.argtypes = [P(_abi.GridDesc), P(_abi.SourceDesc), vp, vp, vp]
    L.gbns_flux_div_host.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, ctypes.c_int, vp]
    L.gbns_flux_div_blocks.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, vp, ctypes.c_int, vp]
    L.gbns_flux_div_blocks_host.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, vp, ctypes.c_int, vp]
    L.gbns_ssprk3_step_blocks.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, P(_abi.BcDesc), vp, vp,
                                          ctypes.c_double, vp]
    L.gbns_wall_fill_blocks.argtypes = [P(_abi.GridDesc), vp, P(_abi.BcDesc), vp, vp]
    L.gbns_boundary_flux.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), vp, vp, P(ctypes.c_int), vp]
    L.gbns_selftest_wait_timeout.argtypes = [P(ctypes.c_int), vp]
    L.gbns_selftest_dmul_int.argtypes = [ctypes.c_uint64, ctypes.c_uint64, P(ctypes.c_uint64), vp]
    L.gbns_device_status.argtypes = [P(ctypes.c_int), ctypes.c_int, vp]
    L.gbns_batch_create.argtypes = [P(vp), ctypes.c_size_t, ctypes.c_int, ctypes.c_int, vp]
    L.gbns_batch_destroy.argtypes = [vp]
    L.gbns_batch_add.argtypes = [vp, P(_abi.GridDesc), P(_abi.SchemeDesc), P(_abi.BcDesc), ctypes.c_double, vp, P(ctypes.c_int)]
    L.gbns_batch_remove.argtypes = [vp, ctypes.c_int]
    L.gbns_batch_step.argtypes = [vp, ctypes.c_int]
    L.gbns_batch_state.argtypes = [vp, ctypes.c_int, P(vp), P(ctypes.c_longlong)]
    L.gbns_batch_usage.argtypes = [vp, P(ctypes.c_size_t), P(ctypes.c_size_t), P(ctypes.c_int), P(ctypes.c_longlong)]
    L.gbns_batch_instance_bytes.argtypes = [P(_abi.GridDesc)]
    L.gbns_batch_instance_bytes.restype = ctypes.c_size_t
    L.gbns_batch_autotune.argtypes = [vp, ctypes.c_int, P(ctypes.c_int)]
    L.gbns_batch_set_steps.argtypes = [vp, ctypes.c_int, ctypes.c_longlong]
    L.gbns_batch_steps_left.argtypes = [vp, ctypes.c_int, P(ctypes.c_longlong)]
    L.gbns_batch_set_variant.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.gbns_batch_class_count.argtypes = []
    L.gbns_batch_class_variant_info.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P(ctypes.c_int)]
    if L.gbns_version() != _abi.ABI_VERSION:
        raise SpadeError(_abi.ERR_UNSUPPORTED, "libgbns ABI version mismatch")
    _LIB = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().gbns_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != 0:
        raise SpadeError(rc, last_error())
    return rc
