"""ctypes binding of the C ABI declared in include/treetime_gb300.h.

The shared library is built in-tree (``treetime_gb300/_lib``); importing this
module without it, or on a machine without a CUDA device, raises -- there is
no CPU fallback for any kernel.
"""

import ctypes as C
import os

from .errors import DeviceError, MissingDataError

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libtreetime_gb300.so")

TT_OK, TT_ERR_INVALID, TT_ERR_NUMERIC, TT_ERR_OOM, TT_ERR_TIMEOUT, TT_ERR_CUDA, TT_ERR_UNSUPPORTED, \
    TT_ERR_BRACKET = range(8)
TT_PREC_F64, TT_PREC_F32 = 0, 1

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
f64 = C.c_double


class TTTree(C.Structure):
    _fields_ = [("node_base", i64), ("level_base", i64), ("pat_base", i64), ("tip_base", i64),
                ("prof_base", i64), ("tipprof_base", i64), ("state_base", i64),
                ("n_int", i32), ("n_tip", i32), ("n_levels", i32), ("n_patterns", i32),
                ("model", i32), ("reserved", i32)]


class TTForest(C.Structure):
    _fields_ = [("n_trees", i32), ("n_states", i32), ("width", i32), ("max_levels", i32),
                ("n_nodes", i64), ("n_patterns", i64),
                ("trees", vp), ("level_off", vp), ("child_off", vp), ("child_idx", vp), ("parent", vp),
                ("tip_row", vp), ("mask_off", vp), ("masks", vp), ("bl", vp), ("tip_codes", vp), ("mult", vp),
                ("work", vp), ("n_work", i32), ("warps_per_block", i32), ("max_blocks", i32),
                ("lanes_per_pattern", i32), ("work_f32", vp), ("n_work_f32", i32), ("reserved1", i32),
                ("node_rec", vp), ("child_pair", vp), ("pair_slot", vp), ("threads_f32", i32),
                ("ctas_per_sm_f32", i32)]


class TTModel(C.Structure):
    _fields_ = [("n_models", i32), ("n_states", i32), ("V", vp), ("Vinv", vp), ("lam", vp), ("mu", vp),
                ("pi", vp), ("lut", vp), ("lut_log2", vp), ("logpi2", vp)]


class TTPmats(C.Structure):
    _fields_ = [("p64", vp), ("p32", vp), ("logp64", vp), ("p32_pair", vp), ("logp2", vp), ("logp2_pair", vp)]


class TTSSF32(C.Structure):
    _fields_ = [("n_sites", i32), ("n_grid", i32), ("V", vp), ("Vinv", vp), ("mulam", vp), ("pi", vp),
                ("em1_grid", vp), ("grid", vp), ("lut", vp), ("rate_scale", C.c_double)]


class TTSSModel(C.Structure):
    _fields_ = [("n_states", i32), ("n_grid", i32), ("approximate", i32), ("reserved", i32),
                ("rate_scale", C.c_double), ("lam", vp), ("V", vp), ("Vinv", vp), ("mu", vp), ("pi", vp),
                ("lut", vp), ("grid", vp), ("stack", vp)]


class TTMarginalOut(C.Structure):
    _fields_ = [("partial", vp), ("posterior", vp), ("outgroup", vp), ("tip_posterior", vp),
                ("tip_outgroup", vp), ("states", vp), ("site_lh", vp), ("tree_lh", vp), ("n_diff", vp),
                ("root_uniform", vp), ("reconstruct_tips", i32), ("count_diff", i32), ("node_uniform", vp)]


class TTJointOut(C.Structure):
    _fields_ = [("msg", vp), ("cx", vp), ("states", vp), ("site_lh", vp), ("tree_lh", vp), ("n_diff", vp),
                ("root_uniform", vp), ("reconstruct_tips", i32), ("count_diff", i32), ("rows", C.c_int64)]


P = C.POINTER
_SIGS = {
    "tt_abi_version": (i32, []),
    "tt_status_string": (C.c_char_p, [i32]),
    "tt_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "tt_device_sm_count": (i32, []),
    "tt_branch_pmats": (i32, [P(TTForest), P(TTModel), TTPmats, vp, vp]),
    "tt_propagate": (i32, [i32, i64, vp, vp, vp, i32, i32, vp, vp]),
    "tt_marginal": (i32, [P(TTForest), P(TTModel), P(TTPmats), i32, P(TTMarginalOut), vp, vp]),
    "tt_outgroups_f32": (i32, [P(TTForest), P(TTModel), P(TTPmats), vp, vp, vp, vp, vp]),
    "tt_count_changes": (i32, [P(TTForest), vp, vp, i32, vp, vp]),
    "tt_marginal_ss": (i32, [P(TTForest), vp, vp, vp, vp, vp, vp, vp, i32, f64, i32, i32, P(TTMarginalOut), vp, vp]),
    "tt_marginal_ss_f32": (i32, [P(TTForest), P(TTSSF32), vp, i32, P(TTMarginalOut), vp, vp]),
    "tt_joint": (i32, [P(TTForest), P(TTModel), P(TTPmats), P(TTJointOut), vp, vp]),
    "tt_joint_noalloc": (i32, [P(TTForest), P(TTModel), i64, vp, vp, vp, vp, vp, i32, i32, vp, vp]),
    "tt_ss_pstack": (i32, [P(TTSSModel), i32, vp, vp]),
    "tt_joint_ss": (i32, [P(TTForest), P(TTSSModel), vp, i32, i32, i32, P(TTJointOut), vp, vp]),
    "tt_mutation_counts_ss": (i32, [P(TTForest), P(TTSSModel), i32, i32, i64, vp, vp, vp, vp, vp, i32, vp, vp, vp,
                                    i64, vp]),
    "tt_state_pairs": (i32, [P(TTForest), vp, vp, i32, i32, i32, vp, vp, vp]),
    "tt_optimal_t_pairs": (i32, [i32, i64, vp, vp, P(TTModel), f64, vp, vp, vp]),
    "tt_prob_t_pairs": (i32, [i32, i64, vp, vp, P(TTModel), vp, vp, vp]),
    "tt_optimal_t_profiles": (i32, [P(TTForest), P(TTModel), i64, vp, vp, vp, vp, vp, i32, i32, i32, f64, vp, vp,
                                    vp, i64, vp]),
    "tt_prob_t_profiles_grid": (i32, [P(TTForest), P(TTModel), i64, vp, vp, vp, vp, vp, i32, i32, i32, vp, i32, vp,
                                      vp, i64, vp]),
    "tt_prob_t_pairs_grid": (i32, [i32, i64, vp, vp, P(TTModel), vp, i32, vp, vp]),
    "tt_fma_probe": (i32, [i64, i32, i32, vp, vp]),
    "tt_fitch_up": (i32, [P(TTForest), vp, vp, vp, vp]),
    "tt_fitch_down": (i32, [P(TTForest), vp, vp, vp, vp, vp, vp, vp, vp]),
    "tt_mutation_counts": (i32, [P(TTForest), P(TTModel), i32, i32, i64, vp, vp, vp, vp, vp, i32, vp, vp, vp, vp,
                                 i64, vp]),
    "tt_mutation_counts_joint": (i32, [P(TTForest), i32, i32, i64, vp, vp, vp, i32, vp, vp, vp, vp, i64, vp]),
    "tt_branch_mutation_matrix": (i32, [P(TTForest), P(TTModel), i32, i32, vp, vp, vp, vp, vp, i32, vp, vp, vp]),
    "tt_branch_mutation_matrix_ss": (i32, [P(TTForest), P(TTSSModel), i32, i32, vp, vp, vp, vp, vp, i32, vp, vp]),
    "tt_compress_columns": (i32, [vp, i64, i64, i32, vp, vp, vp]),
}

_lib = None


def exported_names():
    return sorted(_SIGS)


def load(path=LIB_PATH):
    """Load the library and bind every entry point (raises if missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("treetime_gb300 CUDA library not built: %s (run treetime_gb300.build.build())" % path)
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.tt_abi_version() != 1:
        raise ImportError("treetime_gb300 ABI mismatch")
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = C.create_string_buffer(2048)
    lib.tt_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


def check(status, what):
    """Map a tt_status to the exception TreeTime raises for the same condition."""
    if status == TT_OK:
        return
    msg = "%s: %s" % (what, last_error() or load().tt_status_string(status).decode())
    if status == TT_ERR_NUMERIC:
        raise ValueError("Error in computing exp(Q * t): Q has positive eigenvalues or the branch length t is too "
                         "large. This is most likely caused by incorrect input data.")
    if status == TT_ERR_BRACKET:
        raise ValueError("Bracketing values (xa, xb, xc) do not fulfill this requirement: (f(xb) < f(xa)) and "
                         "(f(xb) < f(xc))")
    if status == TT_ERR_INVALID:
        raise ValueError(msg)
    if status == TT_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise DeviceError(status, msg)
