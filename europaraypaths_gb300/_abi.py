"""ctypes mirror of include/raypath.h and the loader of libraypath.so.

The library is built in-tree (``europaraypaths_gb300/_build/libraypath.so``)
by ``europaraypaths_gb300.build``.  There is no fallback: if the library is
missing or fails to load, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libraypath.so")

RP_OK = 0
RP_FORM_PLAIN_F64 = 0
RP_FORM_FAST_F32 = 1

ERRORS = {
    -1: "RP_ERR_ARG", -2: "RP_ERR_IO", -3: "RP_ERR_PARSE", -4: "RP_ERR_CUDA",
    -5: "RP_ERR_NOMEM", -6: "RP_ERR_UNSUPPORTED", -7: "RP_ERR_BUDGET",
    -8: "RP_ERR_TIMEOUT", -9: "RP_ERR_INTERNAL", -10: "RP_ERR_CANCELLED",
}

_D = ctypes.c_double
_I = ctypes.c_int32


class RpJob(ctypes.Structure):
    """struct rp_job (include/raypath.h)."""
    _fields_ = [("scene", ctypes.c_void_p), ("d_traces", ctypes.c_void_p), ("ns", ctypes.c_int64),
                ("d_out", ctypes.c_void_p), ("counts", ctypes.c_void_p)]


class RpParams(ctypes.Structure):
    """struct rp_params (include/raypath.h); field order must match."""
    _fields_ = [
        ("frequency", _D), ("bandwidth", _D), ("power", _D), ("aperture", _D),
        ("surface_gain", _D), ("subsurface_gain", _D), ("rms_height", _D), ("buff", _D),
        ("eps_1", _D), ("eps_2", _D), ("sig_1", _D), ("sig_2", _D),
        ("rx_sample_rate", _D), ("rx_window_m", _D), ("rx_window_offset_m", _D),
        ("fs", _D), ("source_normal_multiplier", _D), ("altitude", _D),
        ("sx0", _D), ("sdx", _D), ("sy", _D), ("sz", _D),
        ("ns", _I), ("rerad_funct", _I), ("convolution", _I), ("convolution_linear", _I),
        ("specular", _I), ("lossless", _I), ("incoherent", _I), ("disable_surface", _I),
        ("debug_surface", _I), ("pol", _I),
        ("c", _D), ("lam", _D), ("k", _D), ("rng_res", _D), ("grefl_lin", _D), ("grefr_lin", _D),
        ("ks", _D), ("c_1", _D), ("c_2", _D), ("nu_1", _D), ("nu_2", _D),
        ("alpha1", _D), ("alpha2", _D), ("dr", _D),
        ("nr", _I), ("reserved", _I),
        ("incoherent_seed", ctypes.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class RaypathError(RuntimeError):
    """A libraypath call returned a non-zero status."""

    def __init__(self, func, rc, text):
        self.rc = rc
        super().__init__(f"{func} failed: {ERRORS.get(rc, rc)}: {text}")


_lib = None

_SIGS = {
    "rp_version": ([], ctypes.c_char_p),
    "rp_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "rp_params_derive": ([ctypes.c_void_p], ctypes.c_int),
    "rp_prism_alpha": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p], ctypes.c_int),
    "rp_scene_create": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                         ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                         ctypes.c_void_p], ctypes.c_int),
    "rp_scene_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rp_scene_footprint": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_query_footprint_traces": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                   ctypes.c_void_p], ctypes.c_int),
    "rp_query_footprint": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p],
                           ctypes.c_int),
    "rp_simulate": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                     ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
                    ctypes.c_int),
    "rp_simulate_device": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_last_launch_count": ([ctypes.c_void_p], ctypes.c_int),
    "rp_set_timing": ([ctypes.c_int], ctypes.c_int),
    "rp_last_timing": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rp_surface_noalloc": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                            ctypes.c_void_p], ctypes.c_int),
    "rp_workspace_create": ([ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rp_workspace_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rp_workspace_bytes": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_simulate_ws": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_simulate_batch": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_autotune": ([ctypes.c_int], ctypes.c_int),
    "rp_split_parts": ([ctypes.c_int], ctypes.c_int),
    "rp_autotune_query": ([ctypes.c_int, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rp_server_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                          ctypes.c_void_p], ctypes.c_int),
    "rp_server_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rp_server_configure": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "rp_graph_create": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                         ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "rp_graph_create_batch": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
                              ctypes.c_int),
    "rp_graph_launch": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_graph_check": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_graph_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "rp_submit": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_poll": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int], ctypes.c_int),
    "rp_cancel": ([ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "rp_server_drain": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rp_server_stats": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "rp_count_records": ([ctypes.c_char_p, ctypes.c_void_p], ctypes.c_int),
    "rp_read_facets": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "rp_read_targets": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "rp_read_sources": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "rp_read_gains": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p], ctypes.c_int),
    "rp_read_rx_window": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "rp_read_prisms": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
                       ctypes.c_int),
    "rp_write_trace": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "rp_check_directory": ([ctypes.c_char_p], ctypes.c_int),
    "rp_clear_traces": ([ctypes.c_char_p, ctypes.c_void_p], ctypes.c_int),
    "rp_focus_aperture": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                           ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p],
                          ctypes.c_int),
    "rp_focus_geometry": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_focus_center": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "rp_store_kind": ([ctypes.c_char_p, ctypes.c_void_p], ctypes.c_int),
    "rp_write_store": ([ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "rp_map_store": ([ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                     ctypes.c_int),
    "rp_unmap_store": ([ctypes.c_void_p], ctypes.c_int),
    "rp_write_radargram": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int],
                           ctypes.c_int),
    "rp_radargram_info": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "rp_read_radargram": ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int],
                          ctypes.c_int),
}


def lib():
    """Load libraypath.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libraypath.so not found at {LIB_PATH}; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first")
        l = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(l, name)
            fn.argtypes = args
            fn.restype = res
        _lib = l
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().rp_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(func, rc):
    if rc != RP_OK:
        raise RaypathError(func, rc, last_error())
    return rc
