"""ctypes binding of libgapgpu.so (include/gapgpu.h).

The library is the product: there is no Python or CPU compute path behind these
bindings.  If the shared library is missing it is built; if no GPU is usable every
compute entry point returns GAPGPU_ERR_CUDA and the Python side raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgapgpu.so")

OK, ERR_ARG, ERR_XML, ERR_UNSUPPORTED, ERR_CUDA, ERR_ATOMS, ERR_TIMEOUT = range(7)
FP64, MIXED_BF16X3, MIXED_TF32, MIXED_F16 = 0, 1, 2, 3
PRECISIONS = {"fp64": FP64, "bf16x3": MIXED_BF16X3, "tf32": MIXED_TF32, "fp16": MIXED_F16}

# Every symbol declared in include/gapgpu.h.
EXPORTS = ["gapgpu_last_error", "gapgpu_model_create", "gapgpu_model_cutoff", "gapgpu_model_info",
           "gapgpu_model_destroy", "gapgpu_context_create", "gapgpu_context_set_stream", "gapgpu_context_destroy",
           "gapgpu_calc", "gapgpu_calc_device", "gapgpu_context_sync", "gapgpu_neighbours", "gapgpu_descriptors",
           "gapgpu_context_timings", "gapgpu_context_launches", "gapgpu_neighbours_static", "gapgpu_calc_batch",
           "gapgpu_context_set_option", "gapgpu_model_footprint", "gapgpu_md_create", "gapgpu_md_step", "gapgpu_md_state",
           "gapgpu_md_counters", "gapgpu_md_context", "gapgpu_md_destroy", "gapgpu_tuning_report",
           "gapgpu_selftest_bounded_wait", "gapgpu_calc_lammps", "gapgpu_energy_per_coordinate",
           "gapgpu_probe_fp32_rate", "gapgpu_context_neighbours", "gapgpu_gap_variance",
           "gapgpu_gap_variance_instances"]


class GapGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gapgpu error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load(build_if_missing=True):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError("libgapgpu.so is not built")
        from . import build
        build.build()
    L = ctypes.CDLL(LIB_PATH)
    c_int, c_double, c_size_t, c_char_p, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_void_p
    P = ctypes.POINTER
    i64 = ctypes.c_int64
    L.gapgpu_last_error.restype = c_char_p
    L.gapgpu_model_create.argtypes = [c_char_p, c_size_t, c_char_p, c_char_p, P(c_void_p)]
    L.gapgpu_model_cutoff.argtypes = [c_void_p, P(c_double)]
    L.gapgpu_model_info.argtypes = [c_void_p, P(c_int), P(c_int), P(c_int), c_int]
    L.gapgpu_model_destroy.argtypes = [c_void_p]
    L.gapgpu_model_destroy.restype = None
    L.gapgpu_context_create.argtypes = [c_void_p, c_int, P(c_void_p)]
    L.gapgpu_context_set_stream.argtypes = [c_void_p, c_void_p]
    L.gapgpu_context_destroy.argtypes = [c_void_p]
    L.gapgpu_context_destroy.restype = None
    L.gapgpu_context_sync.argtypes = [c_void_p]
    L.gapgpu_calc.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_char_p]
    L.gapgpu_calc_device.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p]
    L.gapgpu_neighbours.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                    c_void_p, i64, P(i64)]
    L.gapgpu_neighbours_static.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p, c_void_p,
                                           i64, P(i64), c_void_p]
    L.gapgpu_descriptors.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, i64,
                                     P(c_int)]
    L.gapgpu_calc_batch.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_char_p]
    L.gapgpu_context_set_option.argtypes = [c_void_p, c_char_p, c_int]
    L.gapgpu_model_footprint.argtypes = [c_void_p, c_int, i64, c_double, P(i64)]
    L.gapgpu_md_create.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_double, c_double, P(c_void_p)]
    L.gapgpu_md_step.argtypes = [c_void_p, c_int]
    L.gapgpu_md_state.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
    L.gapgpu_md_counters.argtypes = [c_void_p, P(i64), P(i64), P(i64)]
    L.gapgpu_md_context.argtypes = [c_void_p]
    L.gapgpu_md_context.restype = c_void_p
    L.gapgpu_md_destroy.argtypes = [c_void_p]
    L.gapgpu_md_destroy.restype = None
    L.gapgpu_tuning_report.argtypes = [c_char_p, c_int]
    L.gapgpu_selftest_bounded_wait.argtypes = [c_void_p, i64]
    L.gapgpu_calc_lammps.argtypes = [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
    L.gapgpu_context_timings.argtypes = [c_void_p, P(c_double), c_int]
    L.gapgpu_context_launches.argtypes = [c_void_p, P(i64)]
    L.gapgpu_probe_fp32_rate.argtypes = [c_void_p, P(c_double)]
    L.gapgpu_gap_variance.argtypes = [c_void_p, c_void_p, c_void_p, c_int]
    L.gapgpu_gap_variance_instances.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, P(c_int)]
    L.gapgpu_context_neighbours.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, i64, P(i64)]
    L.gapgpu_energy_per_coordinate.argtypes = [c_void_p, c_void_p, c_int, P(c_int)]
    _lib = L
    return L


def tuning_report():
    """The GEMM autotuner's choices so far (text, one line per shape)."""
    L = load()
    n = L.gapgpu_tuning_report(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    L.gapgpu_tuning_report(buf, n + 1)
    return buf.value.decode()


def check(code):
    if code != OK:
        raise GapGpuError(code, load().gapgpu_last_error().decode())


def ptr(a):
    """Raw data pointer of a numpy array (or None)."""
    return None if a is None else a.ctypes.data
