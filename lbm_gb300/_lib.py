"""ctypes binding of liblbm_gb300.so (declared in include/lbm_gb300.h).

The library is built in-tree by ``lbm_gb300._build.build()``.  There is no
fallback: if the shared object is missing or a call fails, an exception is
raised.
"""
import ctypes
import os

from . import _build

# Status codes, enums and flags (include/lbm_gb300.h).
LBM_OK = 0
LBM_ERR_ARG = 1
LBM_ERR_CUDA = 2
LBM_ERR_NONFINITE = 3
LBM_ERR_UNSUPPORTED = 5

PREC_F64, PREC_F32, PREC_F16S, PREC_BF16S, PREC_Q60, PREC_F16SR, PREC_BF16SR = range(7)
PRECISIONS = {"f64": PREC_F64, "f32": PREC_F32, "f16s": PREC_F16S, "bf16s": PREC_BF16S,
              "q60": PREC_Q60, "f16sr": PREC_F16SR, "bf16sr": PREC_BF16SR}

WALL_LEFT_VELOCITY = 0
WALL_RIGHT_VELOCITY = 1
WALL_RIGHT_PRESSURE = 2
WALL_TOP_VELOCITY = 3
WALL_BOTTOM_VELOCITY = 4

CORNER_BOTTOM_LEFT, CORNER_TOP_LEFT, CORNER_TOP_RIGHT, CORNER_BOTTOM_RIGHT = 0, 1, 2, 3

MODE_COLLIDE_FROM_G, MODE_STEP, MODE_FINISH = 0, 1, 2
FLAG_MACRO_LAST, FLAG_CHECK_FINITE, FLAG_WALL_MACRO, FLAG_BULK_REGISTERS = 1, 2, 4, 8
FLAG_TEST_STALL = 16


class LbmError(RuntimeError):
    """A liblbm_gb300 call returned a non-zero status."""

    def __init__(self, fn, code, msg):
        super().__init__("%s failed (status %d): %s" % (fn, code, msg))
        self.code = code


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_d = ctypes.c_double


class Problem(ctypes.Structure):
    """Mirror of ``struct lbm_problem``."""

    _fields_ = [
        ("nx", _i32), ("ny", _i32), ("precision", _i32), ("ibb", _i32),
        ("om_p", _d), ("om_m", _d), ("rho0", _d),
        ("n_wall_ops", _i32), ("wall_ops", _i32 * 5),
        ("n_corner_ops", _i32), ("corner_ops", _i32 * 4),
        ("corner_nb_special", _i32 * 4), ("corner_special", _i32 * 4),
        ("f", _vp * 2),
        ("bc_base", _vp), ("bc_vec", _vp), ("bc_scale", _vp),
        ("bc_scale_it0", _i64), ("bc_scale_len", _i64),
        ("n_special", _i32), ("special_cell", _vp), ("special_link_start", _vp),
        ("n_links", _i32), ("link_cell", _vp), ("link_q", _vp), ("link_nb1", _vp),
        ("link_nb2", _vp), ("link_p", _vp), ("special_link_ids", _vp),
        ("n_obstacles", _i32), ("obstacle_link_start", _vp),
        ("scratch", _vp), ("scratch_bytes", ctypes.c_size_t),
        ("drag_hist", _vp), ("drag_cap", _i64),
        ("rho_out", _vp), ("u_out", _vp), ("g_out", _vp), ("status_flags", _vp),
        ("row_pitch", _i32),
        ("link_coef", _vp),
    ]


class BatchConfig(ctypes.Structure):
    """Mirror of ``struct lbm_batch_config``."""

    _fields_ = [("bulk_threads", _i32), ("bulk_blocks_per_sm", _i32),
                ("special_blocks_per_sm", _i32), ("scalar_tile_cells", _i32),
                ("persistent", _i32), ("vec_bytes", _i32), ("tile_rounds", _i32),
                ("bulk_tma", _i32)]


class Adjoint(ctypes.Structure):
    """Mirror of ``struct lbm_adjoint``."""

    _fields_ = [("obj_it_first", _i64), ("obj_it_last", _i64), ("obj_w", _vp),
                ("is_special", _vp), ("adj_pulled", _vp), ("link_adj", _vp),
                ("corner_seed", _vp), ("grad_bc_base", _vp), ("grad_bc_vec", _vp),
                ("grad_omega", _vp), ("grad_omega_len", _i32)]


_SIGS = {
    "lbm_abi_version": ([], ctypes.c_int),
    "lbm_last_error_string": ([], ctypes.c_char_p),
    "lbm_device_info": ([_vp, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "lbm_macro_f64": ([_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp], ctypes.c_int),
    "lbm_equilibrium_f64": ([_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp], ctypes.c_int),
    "lbm_collision_stream_f64": ([_vp, _vp, _vp, _d, _d, ctypes.c_int, ctypes.c_int, _vp],
                                 ctypes.c_int),
    "lbm_bounce_back_f64": ([ctypes.c_int, _vp, _i64, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                             _vp], ctypes.c_int),
    "lbm_drag_lift_scratch_bytes": ([_i64], ctypes.c_size_t),
    "lbm_drag_lift_f64": ([_vp, _i64, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp],
                          ctypes.c_int),
    "lbm_drag_lift_f64_noalloc": ([_vp, _i64, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp],
                                  ctypes.c_int),
    "lbm_zou_he_f64": ([ctypes.c_int, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp],
                       ctypes.c_int),
    "lbm_mv_avg_chunk": ([_vp, _i64, _i64, _i32, _d, _d, _i32, _vp, _vp, _vp, _vp, _vp],
                         ctypes.c_int),
    "lbm_zou_he_corner_f64": ([ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp],
                              ctypes.c_int),
    "lbm_problem_scratch_bytes": ([ctypes.POINTER(Problem)], ctypes.c_size_t),
    "lbm_advance": ([ctypes.POINTER(Problem), ctypes.c_int, _i64, ctypes.c_int, ctypes.c_int,
                     ctypes.c_uint32, _vp], ctypes.c_int),
    "lbm_advance_graph": ([ctypes.POINTER(Problem), _i64, ctypes.c_int, ctypes.c_int,
                           ctypes.c_uint32, _vp], ctypes.c_int),
    "lbm_profile_steps": ([ctypes.POINTER(Problem), _i64, ctypes.c_int, ctypes.c_int,
                           ctypes.c_uint32, ctypes.POINTER(ctypes.c_double), _vp], ctypes.c_int),
    "lbm_graph_cache_clear": ([], ctypes.c_int),
    "lbm_measure_dfma_scratch_bytes": ([], ctypes.c_size_t),
    "lbm_measure_dfma_rate": ([ctypes.POINTER(ctypes.c_double), _vp, ctypes.c_size_t, _vp],
                              ctypes.c_int),
    "lbm_batch_create": ([ctypes.POINTER(_vp), ctypes.POINTER(Problem), _i32,
                          ctypes.POINTER(BatchConfig)], ctypes.c_int),
    "lbm_batch_destroy": ([_vp], ctypes.c_int),
    "lbm_batch_info": ([_vp, ctypes.POINTER(_i64)], ctypes.c_int),
    "lbm_batch_advance": ([_vp, _i64, ctypes.c_int, ctypes.c_int, _vp], ctypes.c_int),
    "lbm_batch_advance_graph": ([_vp, _i64, ctypes.c_int, ctypes.c_int, _vp], ctypes.c_int),
    "lbm_adjoint_omega_slots": ([ctypes.POINTER(Problem)], ctypes.c_size_t),
    "lbm_adjoint_step": ([ctypes.POINTER(Problem), ctypes.POINTER(Adjoint), _i64, _vp, _vp, _vp,
                          _vp], ctypes.c_int),
    "lbm_adjoint_recompute": ([ctypes.POINTER(Problem), _i64, ctypes.c_int, _vp, _i64, _vp],
                              ctypes.c_int),
    "lbm_adjoint_sweep": ([ctypes.POINTER(Problem), ctypes.POINTER(Adjoint), _i64, ctypes.c_int,
                           _vp, _i64, _vp, _vp, ctypes.c_int, _vp], ctypes.c_int),
    "lbm_adjoint_initial": ([ctypes.POINTER(Problem), ctypes.POINTER(Adjoint), _vp, _vp, _vp,
                             _vp], ctypes.c_int),
    "lbm_pack_f64": ([ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _vp],
                     ctypes.c_int),
    "lbm_unpack_f64": ([ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d,
                        _vp], ctypes.c_int),
}

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("liblbm_gb300.so is not built (%s); run lbm_gb300._build.build()" % path)
    L = ctypes.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def exported_symbols():
    return list(_SIGS)


def call(name, *args):
    """Call ``name`` and raise LbmError on a non-zero status."""
    L = load()
    rc = getattr(L, name)(*args)
    if rc != LBM_OK:
        msg = L.lbm_last_error_string()
        raise LbmError(name, rc, msg.decode() if msg else "")
    return rc
