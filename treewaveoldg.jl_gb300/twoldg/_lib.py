"""ctypes binding of libtwoldg (include/twoldg.h).

The library is the only compute path: if it is not built, or the process has
no CUDA device, the calls that need it raise instead of falling back to any
CPU implementation.
"""
import ctypes
import os

from . import nativebuild as _build

TWOLDG_OK, TWOLDG_EINVAL, TWOLDG_ECUDA, TWOLDG_ENOMEM, TWOLDG_EUNSUP = range(5)
F64, F32, F32C = 0, 1, 2

# Every function include/twoldg.h declares; tests check the library exports them.
EXPORTS = [
    "twoldg_last_error", "twoldg_version", "twoldg_element_tables",
    "twoldg_problem_create", "twoldg_problem_destroy", "twoldg_state_words", "twoldg_min_spacing",
    "twoldg_rhs", "twoldg_truncate", "twoldg_rk4_step", "twoldg_reset_compensation",
    "twoldg_energy", "twoldg_norm", "twoldg_modal_indicator", "twoldg_mode_amplitude",
    "twoldg_synchronize", "twoldg_batch_create", "twoldg_batch_destroy", "twoldg_batch_offsets",
    "twoldg_batch_rk4_step", "twoldg_batch_synchronize", "twoldg_batch_stream", "twoldg_profile_step",
    "twoldg_profile_kernels",
    "twoldg_stream", "twoldg_boundary_faces", "twoldg_set_boundary_values",
    "twoldg_rhs_static", "twoldg_autotune", "twoldg_batch_autotune", "twoldg_transfer", "twoldg_gather",
    "twoldg_transfer_plan_create", "twoldg_transfer_plan_update", "twoldg_transfer_plan_destroy",
    "twoldg_transfer_plan_counts",
    "twoldg_transfer_points", "twoldg_project_values", "twoldg_project_density", "twoldg_transfer_table",
    "twoldg_average_shared", "twoldg_pairing", "twoldg_support_elements",
]


class Desc(ctypes.Structure):
    """twoldg_desc."""
    _fields_ = [
        ("dim", ctypes.c_int32), ("order", ctypes.c_int32), ("elems", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("truncate", ctypes.c_int32), ("nblocks", ctypes.c_int32),
        ("roots", ctypes.c_int32 * 3), ("periodic", ctypes.c_int32 * 3),
        ("reflecting", ctypes.c_int32 * 3), ("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
        ("level", ctypes.POINTER(ctypes.c_int32)), ("corner", ctypes.POINTER(ctypes.c_int64)),
        ("coef", ctypes.POINTER(ctypes.c_double)), ("trunc_modes", ctypes.POINTER(ctypes.c_double)),
        ("trunc_duals", ctypes.POINTER(ctypes.c_double)),
        ("metric", ctypes.c_int32), ("face_nb", ctypes.POINTER(ctypes.c_int32)),
        ("face_code", ctypes.POINTER(ctypes.c_int32)), ("elem_slot", ctypes.POINTER(ctypes.c_int32)),
        ("elem_w", ctypes.POINTER(ctypes.c_double)), ("elem_chol", ctypes.POINTER(ctypes.c_double)),
        ("elem_ntab", ctypes.c_int32), ("wave_k", ctypes.c_double * 3), ("wave_phi", ctypes.c_double),
        ("bnd_x", ctypes.POINTER(ctypes.c_double)),
        ("boundary", ctypes.c_int32), ("kappa", ctypes.c_double), ("inv_r", ctypes.c_double),
        ("fac_slot", ctypes.POINTER(ctypes.c_int32)), ("fac_radial", ctypes.POINTER(ctypes.c_int32)),
        ("fac_rmodes", ctypes.POINTER(ctypes.c_double)), ("fac_rduals", ctypes.POINTER(ctypes.c_double)),
        ("fac_aslot", ctypes.POINTER(ctypes.c_int32)), ("fac_aw", ctypes.POINTER(ctypes.c_double)),
        ("fac_achol", ctypes.POINTER(ctypes.c_double)), ("fac_ntab", ctypes.c_int32),
    ]


class Particle(ctypes.Structure):
    """twoldg_particle."""
    _fields_ = [("z", ctypes.c_double * 3), ("v", ctypes.c_double * 3), ("ell", ctypes.c_double),
                ("charge", ctypes.c_double)]


class TransferDesc(ctypes.Structure):
    """twoldg_transfer_desc."""
    _fields_ = [
        ("origins", ctypes.POINTER(ctypes.c_double)), ("spacings", ctypes.POINTER(ctypes.c_double)),
        ("levels", ctypes.POINTER(ctypes.c_int32)), ("mask", ctypes.POINTER(ctypes.c_uint8)),
        ("h_e", ctypes.c_double), ("ball_centre", ctypes.c_double * 3), ("ball_radius", ctypes.c_double),
        ("particles", ctypes.POINTER(Particle)), ("nparticles", ctypes.c_int32), ("rnear", ctypes.c_double),
        ("q", ctypes.c_int32), ("nsinh", ctypes.c_int32), ("nmid", ctypes.c_int32), ("ninner", ctypes.c_int32),
        ("nbands", ctypes.c_int32), ("band_from", ctypes.POINTER(ctypes.c_double)),
        ("band_points", ctypes.POINTER(ctypes.c_int32)), ("rfar", ctypes.c_double),
    ]


class TwoldgError(RuntimeError):
    """A failure reported by libtwoldg (CUDA error, allocation, unsupported shape)."""


_lib = None


def lib():
    """The loaded library; builds nothing, raises if it is missing."""
    global _lib
    if _lib is None:
        path = _build.lib_path()
        if not os.path.exists(path):
            raise TwoldgError("libtwoldg.so is not built (%s): run __graft_entry__.build()" % path)
        L = ctypes.CDLL(path)
        vp, i32, i64, d = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        sig = {
            "twoldg_last_error": (ctypes.c_char_p, []),
            "twoldg_version": (ctypes.c_char_p, []),
            "twoldg_element_tables": (ctypes.c_int, [i32, i32, ctypes.c_char_p, vp]),
            "twoldg_problem_create": (ctypes.c_int, [ctypes.POINTER(Desc), ctypes.POINTER(vp)]),
            "twoldg_problem_destroy": (ctypes.c_int, [vp]),
            "twoldg_state_words": (ctypes.c_int, [vp, ctypes.POINTER(i64)]),
            "twoldg_min_spacing": (ctypes.c_int, [vp, ctypes.POINTER(d)]),
            "twoldg_rhs": (ctypes.c_int, [vp, vp, vp, d]),
            "twoldg_truncate": (ctypes.c_int, [vp, vp]),
            "twoldg_rk4_step": (ctypes.c_int, [vp, vp, d, d, i32]),
            "twoldg_reset_compensation": (ctypes.c_int, [vp]),
            "twoldg_energy": (ctypes.c_int, [vp, vp, d, ctypes.POINTER(d)]),
            "twoldg_norm": (ctypes.c_int, [vp, vp, vp, i32, i32, ctypes.POINTER(d)]),
            "twoldg_modal_indicator": (ctypes.c_int, [vp, vp, i32, i32, vp]),
            "twoldg_mode_amplitude": (ctypes.c_int, [vp, vp, i32, i32, vp]),
            "twoldg_synchronize": (ctypes.c_int, [vp]),
            "twoldg_batch_create": (ctypes.c_int, [i32, ctypes.POINTER(Desc), ctypes.POINTER(vp)]),
            "twoldg_batch_destroy": (ctypes.c_int, [vp]),
            "twoldg_batch_offsets": (ctypes.c_int, [vp, ctypes.POINTER(i64), ctypes.POINTER(i64)]),
            "twoldg_batch_rk4_step": (ctypes.c_int, [vp, vp, ctypes.POINTER(d), i32]),
            "twoldg_batch_synchronize": (ctypes.c_int, [vp]),
            "twoldg_batch_stream": (vp, [vp]),
            "twoldg_profile_step": (ctypes.c_int, [vp, vp, d, ctypes.POINTER(ctypes.c_float)]),
            "twoldg_profile_kernels": (ctypes.c_int, [vp, vp, ctypes.POINTER(ctypes.c_float), i32]),
            "twoldg_stream": (vp, [vp]),
            "twoldg_boundary_faces": (ctypes.c_int, [vp, vp, ctypes.POINTER(i32)]),
            "twoldg_set_boundary_values": (ctypes.c_int, [vp, vp, i32, d, d]),
            "twoldg_rhs_static": (ctypes.c_int, [ctypes.POINTER(Desc), vp, vp, d, vp]),
            "twoldg_autotune": (ctypes.c_int, [vp, vp, d, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]),
            "twoldg_transfer": (ctypes.c_int, [ctypes.POINTER(Desc), vp, ctypes.POINTER(Desc), vp, vp]),
            "twoldg_gather": (ctypes.c_int, [vp, vp, i32, i64, i32, vp, vp, vp]),
            "twoldg_batch_autotune": (ctypes.c_int, [vp, vp, ctypes.POINTER(d), ctypes.c_char_p, ctypes.c_char_p,
                                                     ctypes.c_size_t]),
            "twoldg_transfer_plan_create": (ctypes.c_int, [vp, ctypes.POINTER(TransferDesc), ctypes.POINTER(vp)]),
            "twoldg_transfer_plan_update": (ctypes.c_int, [vp, ctypes.POINTER(Particle), i32]),
            "twoldg_transfer_plan_destroy": (ctypes.c_int, [vp]),
            "twoldg_transfer_plan_counts": (ctypes.c_int, [vp, ctypes.POINTER(i64)]),
            "twoldg_transfer_points": (ctypes.c_int, [vp, vp]),
            "twoldg_project_values": (ctypes.c_int, [vp, vp, vp, d, i32]),
            "twoldg_project_density": (ctypes.c_int, [vp, vp, d, i32]),
            "twoldg_average_shared": (ctypes.c_int, [vp, vp, i32]),
            "twoldg_pairing": (ctypes.c_int, [vp, vp, i32, i32, vp]),
            "twoldg_support_elements": (ctypes.c_int, [vp, i32, vp, vp]),
            "twoldg_transfer_table": (ctypes.c_int, [i32, i32, ctypes.c_char_p, i32, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def tune_report(text):
    """The autotuner's report lines ('"key": {"kernel": k, ...}') as a dict."""
    import json
    body = ",".join(line for line in text.splitlines() if line.strip())
    return json.loads("{" + body + "}") if body else {}


def check(rc):
    """Raise the library's error for a non-zero status: ValueError for a
    rejected argument (the reference's ArgumentError), TwoldgError else."""
    if rc == TWOLDG_OK:
        return
    msg = lib().twoldg_last_error().decode(errors="replace")
    if rc == TWOLDG_EINVAL:
        raise ValueError(msg)
    raise TwoldgError("libtwoldg error %d: %s" % (rc, msg))
