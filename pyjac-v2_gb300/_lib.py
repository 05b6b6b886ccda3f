"""ctypes binding of the C ABI (include/pyjac_gb300.h).

The library is the in-tree ``_build/libpyjac_gb300.so``.  There is no CPU
fallback: if the library is missing or does not load, every entry point raises
``RuntimeError``.
"""
import ctypes
import os

from . import build as _build

_I32P = ctypes.POINTER(ctypes.c_int32)
_DP = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


class PjgTables(ctypes.Structure):
    _fields_ = [("ns", ctypes.c_int32), ("nr", ctypes.c_int32), ("flags", ctypes.c_int32),
                ("rxn", _VP), ("species", _DP), ("thd_spec", _I32P), ("thd_coef", _DP),
                ("n_thd", ctypes.c_int32), ("aux", _DP), ("n_aux", ctypes.c_int32),
                ("nnz", ctypes.c_int32), ("crs_row_ptr", _I32P), ("crs_col_ind", _I32P),
                ("ccs_col_ptr", _I32P), ("ccs_row_ind", _I32P)]


# (name, restype, argtypes) of every exported function
SIGNATURES = [
    ("pjg_mech_create", ctypes.c_int, [ctypes.POINTER(PjgTables), ctypes.POINTER(_VP)]),
    ("pjg_mech_destroy", ctypes.c_int, [_VP]),
    ("pjg_mech_info", ctypes.c_int, [_VP, _I32P, _I32P, _I32P]),
    ("pjg_jacobian_indices", ctypes.c_int, [_VP, ctypes.c_char, _I32P, _I32P, _I32P]),
    ("pjg_species_rates", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, _VP, _VP, _VP, _VP]),
    ("pjg_jacobian", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP]),
    ("pjg_jacobian_rates", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP, _VP]),
    ("pjg_vjp", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, _VP, _VP, _VP, _VP, _VP]),
    ("pjg_vjp_noalloc", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, _VP, _VP, _VP, _VP, _VP]),
    ("pjg_kernel_create", ctypes.c_int,
     [_VP, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_char, ctypes.c_int,
      ctypes.c_int, ctypes.POINTER(_VP)]),
    ("pjg_kernel_resize", ctypes.c_int, [_VP, ctypes.c_size_t, ctypes.c_size_t]),
    ("pjg_kernel_call", ctypes.c_int, [_VP, _VP, _VP, _VP]),
    ("pjg_kernel_required_memory", ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_size_t)]),
    ("pjg_kernel_destroy", ctypes.c_int, [_VP]),
    ("pjg_last_error", ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    ("pjg_mlp_linear", ctypes.c_int,
     [_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _VP,
      ctypes.c_int, _VP, ctypes.c_int64, _VP, ctypes.c_int64, _VP, ctypes.c_int64, _VP,
      ctypes.c_int64, _VP, ctypes.c_int64, _VP, _VP]),
    ("pjg_mlp_wgrad", ctypes.c_int,
     [_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _VP,
      ctypes.c_int64, _VP]),
    ("pjg_mlp_status", ctypes.c_int, [ctypes.c_int]),
    ("pjg_surrogate_features", ctypes.c_int,
     [ctypes.c_int64, ctypes.c_int32, _VP, _VP, _VP, _VP, ctypes.c_double, _VP]),
    ("pjg_surrogate_outputs", ctypes.c_int,
     [ctypes.c_int64, ctypes.c_int32, _VP, _VP, _VP, _VP, ctypes.c_int32, _VP, _VP, _VP]),
    ("pjg_mlp_forward", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(_VP), ctypes.POINTER(_VP), _VP,
      ctypes.c_int64, _VP]),
    ("pjg_host_register", ctypes.c_int, [_VP, ctypes.c_size_t]),
    ("pjg_host_unregister", ctypes.c_int, [_VP]),
    ("pjg_launch_count", ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    ("pjg_fp64_peak", ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    ("pjg_profile_begin", ctypes.c_int, []),
    ("pjg_profile_end", ctypes.c_int, [ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_double)]),
    ("pjg_math_exp", ctypes.c_int, [_VP, _VP, ctypes.c_int64, _VP]),
    ("pjg_reaction_order", ctypes.c_int,
     [ctypes.POINTER(PjgTables), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
      ctypes.POINTER(ctypes.c_int32)]),
    ("pjg_eval_chunk", ctypes.c_int,
     [_VP, ctypes.c_int, ctypes.c_int64, ctypes.c_char, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    ("pjg_read_initial_conditions", ctypes.c_int,
     [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_char, _VP, _VP]),
    ("pjg_write_initial_conditions", ctypes.c_int,
     [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_char, _VP, _VP]),
    ("pjg_chem_utils", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, _VP, _VP, _VP, _VP, _VP]),
    ("pjg_lu_factor", ctypes.c_int,
     [ctypes.c_int32, ctypes.c_int64, ctypes.c_char, ctypes.c_double, _VP, ctypes.c_double, _VP,
      _VP, _VP, _VP, _VP]),
    ("pjg_lu_solve", ctypes.c_int,
     [ctypes.c_int32, ctypes.c_int64, ctypes.c_char, _VP, _VP, _VP, _VP]),
    ("pjg_ros2_step", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_int, _VP, _VP, _VP, ctypes.c_double, ctypes.c_int,
      _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    ("pjg_lu_symbolic", ctypes.c_int,
     [ctypes.c_int32, _VP, _VP, _VP, _VP, ctypes.POINTER(ctypes.c_int64)]),
    ("pjg_lu_plan_info", ctypes.c_int, [_VP, _VP, _VP, ctypes.POINTER(ctypes.c_int64)]),
    ("pjg_lu_factor_sparse", ctypes.c_int,
     [_VP, ctypes.c_int64, ctypes.c_char, ctypes.c_double, _VP, ctypes.c_double, _VP, _VP, _VP,
      _VP]),
    ("pjg_lu_solve_sparse", ctypes.c_int, [_VP, ctypes.c_int64, ctypes.c_char, _VP, _VP, _VP]),
]


def launch_count():
    c = ctypes.c_int64()
    check("pjg_launch_count", load().pjg_launch_count(ctypes.byref(c)))
    return c.value


def eval_chunk(handle, kind, n, order, jac_format=0):
    """States per launch of an evaluation of n states (pjg_eval_chunk)."""
    c = ctypes.c_int64()
    check("pjg_eval_chunk", load().pjg_eval_chunk(handle, int(kind), int(n), order.encode(),
                                                  int(jac_format), ctypes.byref(c)))
    return c.value


def profile_begin():
    check("pjg_profile_begin", load().pjg_profile_begin())


def profile_end():
    """Return (evaluation-kernel launches, summed milliseconds) since profile_begin."""
    n = ctypes.c_int64()
    ms = ctypes.c_double()
    check("pjg_profile_end", load().pjg_profile_end(ctypes.byref(n), ctypes.byref(ms)))
    return n.value, ms.value

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load the CUDA library; raise RuntimeError if it is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("pyjac-v2_gb300 CUDA library not built (%s); run "
                               "__graft_entry__.build() or python pyjac-v2_gb300/build.py" % path)
    try:
        lib = ctypes.CDLL(path)
    except OSError as e:
        raise RuntimeError("cannot load %s: %s" % (path, e))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(512)
    lib.pjg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class PjgError(RuntimeError):
    def __init__(self, fn, code):
        self.code = code
        super(PjgError, self).__init__("%s failed (%d): %s" % (fn, code, last_error()))


def check(fn, code):
    if code != 0:
        raise PjgError(fn, code)
    return code
