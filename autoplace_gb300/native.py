"""ctypes binding of libgp103.so (include/gp103.h). No fallback: if the library is missing or fails to load, every
entry point raises. Streams are passed as raw cudaStream_t handles (torch.cuda.Stream.cuda_stream)."""
import ctypes
import os

from . import build as _build

_LIB = None

OK, ERR_ARG, ERR_CUDA, ERR_SHAPE = 0, 1, 2, 3
OPT_PDL, OPT_WAIT_MS, OPT_TEST_STALL_FIELD, OPT_WA_FUSED, OPT_FIELD_EARLY = 0, 1, 2, 3, 4
# the waits of the tensor-core field (gp103_device_error codes)
DEVICE_ERRORS = {1: "a TMA stage's slot", 2: "an accumulator's buffer", 3: "a TMA stage's data",
                 4: "an accumulator's result"}
FIELD_FP32, FIELD_BF16X3, FIELD_BF16X6, FIELD_F16X3, FIELD_TF32X3 = 0, 1, 2, 3, 4
FIELD_MODES = {"fp32": FIELD_FP32, "bf16x3": FIELD_BF16X3, "bf16x6": FIELD_BF16X6, "f16x3": FIELD_F16X3,
               "tf32x3": FIELD_TF32X3}
PHASE_START, PHASE_DENSITY = 0, 1
PASS_SORT = 0x100
PASS_JOIN_FIELD = 0x200
T = dict(alpha=0, a=1, iter=2, loop_it=3, done=4, stop=5, accept=6, hpwl=7, wa=8, evals=9, nwa=10, start_tol=11,
         inner=12, ring=16)
T_SIZE = 32

_vp, _i, _f, _d, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_size_t


class Plan(ctypes.Structure):
    """gp103_plan, field for field."""
    _fields_ = [
        ("num_nodes", _i), ("num_mov", _i), ("num_nets", _i), ("num_pins", _i),
        ("nbx", _i), ("nby", _i), ("jnbx", _i), ("jnby", _i), ("field_mode", _i),
        ("pin_cell", _vp), ("pin_off", _vp), ("net_start", _vp), ("cell_start", _vp), ("cell_pin", _vp),
        ("size", _vp), ("ratio", _vp), ("pins", _vp), ("area", _vp), ("lo", _vp), ("hi", _vp),
        ("bx", _f), ("by", _f), ("target", _f),
        ("fixed", _vp),
        ("ovf_scale", _d),
        ("jsize", _vp), ("jratio", _vp), ("jfixed", _vp), ("jbx", _f), ("jby", _f), ("jovf_scale", _d),
        ("field_const", _vp), ("field_work", _vp), ("ex", _vp), ("ey", _vp),
        ("u", _vp * 2), ("v", _vp * 2), ("g", _vp * 2), ("best", _vp), ("cur", _vp),
        ("S", _vp), ("T", _vp), ("kp", _vp), ("c", _vp),
        ("pin_grad", _vp), ("map", _vp), ("jmap", _vp), ("red", _vp), ("counters", _vp),
        ("pin_slot", _vp), ("net_split", _i),
        ("order", _vp), ("order_counts", _vp), ("order_cursor", _vp),
        ("net_mid", _i), ("net_two", _i), ("net_three", _i),
        ("field_shift", _f),
        ("net_g8", _i), ("net_g16", _i),
        ("wa_long_share", _i),
    ]


class Sizes(ctypes.Structure):
    _fields_ = [("field_const", ctypes.c_size_t), ("field_work", ctypes.c_size_t), ("red", ctypes.c_size_t)]


class BeginArgs(ctypes.Structure):
    """gp103_begin_args, field for field."""
    _fields_ = [(n, _d) for n in ("lr", "gamma", "lam", "start_tol", "inner_iter", "iter", "loop_it", "hpwl_prev")]


_SIGS = {
    "gp103_version": ([], _i),
    "gp103_status_string": ([_i], ctypes.c_char_p),
    "gp103_launch_count": ([], ctypes.c_ulonglong),
    "gp103_set_option": ([_i, _i], _i),
    "gp103_profile_begin": ([_vp], _i),
    "gp103_profile_end": ([ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_char_p), _i], _i),
    "gp103_wa": ([_vp] * 6 + [_i, _i] + [_vp] * 4 + [_vp], _i),
    "gp103_density_map": ([_vp, _vp, _vp, _i, _i, _f, _f, _i, _i, _vp, _vp, _f, _vp, _vp, _vp], _i),
    "gp103_density_map_noalloc": ([_vp, _vp, _vp, _i, _i, _f, _f, _i, _i, _vp, _f, _vp, _vp, _vp], _i),
    "gp103_nesterov_step": ([_vp] * 7 + [_i, _vp, _vp, _vp], _i),
    "gp103_density_grad": ([_vp] * 7 + [_i, _i, _vp, _vp, _f, _f, _i, _i, _vp, _vp], _i),
    "gp103_control": ([_vp] * 8 + [_vp], _i),
    "gp103_select": ([_vp] * 8 + [_i, _vp], _i),
    "gp103_plan_offsets": ([ctypes.POINTER(ctypes.c_size_t), _i], _i),
    "gp103_plan_sizes": ([_i, _i, _i, ctypes.POINTER(Sizes)], _i),
    "gp103_field_constants": ([ctypes.POINTER(Plan), _vp], _i),
    "gp103_pass": ([ctypes.POINTER(Plan), _i, _vp], _i),
    "gp103_eval": ([ctypes.POINTER(Plan), _vp, _vp, _vp, _d, _d, _i, _vp, _vp], _i),
    "gp103_probe": ([ctypes.POINTER(Plan), _vp, _vp, _d, _vp, _vp, _vp], _i),
    "gp103_field": ([ctypes.POINTER(Plan), _vp, _vp, _vp, _vp], _i),
    "gp103_finish": ([ctypes.POINTER(Plan), _vp], _i),
    "gp103_start_to_density": ([ctypes.POINTER(Plan), _d, _d, _d, _vp, _vp, _vp], _i),
    "gp103_begin": ([ctypes.POINTER(Plan), ctypes.POINTER(BeginArgs), _vp, _vp, _vp, _vp], _i),
    "gp103_device_error": ([ctypes.POINTER(Plan), _i, ctypes.POINTER(_i), _vp], _i),
    "gp103_hpwl": ([_vp] * 4 + [_i, _i, _vp, _vp, _vp], _i),
    "gp103_net_order_scratch": ([_i, _i, _i], ctypes.c_size_t),
    "gp103_cluster_scratch": ([_i, _i, _i], ctypes.c_size_t),
    "gp103_cluster_edges": ([_vp, _vp, _i, _i, _i, _i, _i, _vp, ctypes.c_size_t, _vp, _vp, _vp, _vp, _vp], _i),
    "gp103_cluster_round": ([_vp, _vp, _vp, _i, _i, _vp, _vp, ctypes.c_longlong, ctypes.c_longlong, _i, _vp,
                             ctypes.c_size_t, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i),
    "gp103_cluster_relabel": ([_vp, _i, _vp, _vp], _i),
    "gp103_coarse_pins_scratch": ([_i], ctypes.c_size_t),
    "gp103_coarse_pins": ([_vp, _vp, _vp, _i, _i, _vp, _i, _vp, _vp, ctypes.c_size_t, _vp, _vp, _vp, _vp, _vp], _i),
    "gp103_expand": ([_vp] * 5 + [_i, _vp, _vp], _i),
    "gp103_seeded_uniform": ([ctypes.c_ulonglong, ctypes.c_longlong, _vp, _vp], _i),
    "gp103_cluster_members": ([_vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp], _i),
    "gp103_pass_split": ([ctypes.POINTER(Plan), _i, _vp, _vp, _vp, _vp], _i),
    "gp103_event_create": ([ctypes.POINTER(_vp)], _i),
    "gp103_event_destroy": ([_vp], _i),
    "gp103_build_csr_scratch": ([_i, _i, _i], ctypes.c_size_t),
    "gp103_build_csr": ([_vp, _vp, _vp, _i, _i, _i, _i, _vp, ctypes.c_size_t] + [_vp] * 8 + [_vp], _i),
    "gp103_smooth_nodes": ([_vp, _i, _i, _d, _d, _f, _f] + [_vp] * 7 + [_vp], _i),
    "gp103_net_order": ([_vp] * 4 + [_i, _i, _i, _vp, ctypes.c_size_t] + [_vp] * 5 + [_vp], _i),
    "gp103_exact_overflow": ([_vp, _vp, _i, _f, _f, _i, _i, _vp, _f, _d, _vp, _vp, _vp, _vp], _i),
    "gp103_macro_fraction": ([_vp, _i, _d, _d, _i, _i, _vp, _vp], _i),
    # batches of instances in one graph
    "gp103_batch_create": ([ctypes.POINTER(_vp)], _i),
    "gp103_batch_add": ([_vp, ctypes.POINTER(Plan), _i, _i, _i, _i, _vp, _vp, _vp], _i),
    "gp103_batch_add_run": ([_vp, ctypes.POINTER(Plan), ctypes.POINTER(BeginArgs), _i, _i, _i, _i, _d, _d, _d, _vp,
                             _vp, _vp, _vp, _vp, _vp], _i),
    "gp103_batch_launch": ([_vp, _vp, _vp], _i),
    "gp103_batch_destroy": ([_vp], _i),
    # the learned start
    "gp103_learn_graph_scratch": ([_i, _i], _sz),
    "gp103_learn_graph": ([_vp] * 4 + [_i, _i, _i, _vp, _sz] + [_vp] * 6 + [_vp], _i),
    "gp103_seg_gather": ([_vp, _i, _vp, _vp, _vp, _i, _i, _vp, _vp], _i),
    "gp103_dense_fwd": ([_vp, _i, _i, _vp, _i, _vp, _vp, _vp, _i, _i, _vp, _vp], _i),
    "gp103_dense_bwd_scratch": ([_i, _i, _i], _sz),
    "gp103_dense_bwd": ([_vp, _i, _i, _vp, _i, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp,
                         _vp], _i),
    "gp103_mse": ([_vp, _vp, _i, _i, _vp, _vp, _vp, _vp], _i),
    "gp103_adam": ([_vp, _vp, _vp, _vp, _vp, _i, _f, _f, _f, _f, _i, _f, _vp], _i),
    "gp103_learn_features_scratch": ([_i, _i], _sz),
    "gp103_learn_features": ([_vp] * 4 + [_i, _i, _i] + [_vp] * 6 + [_d, _f, _f, _i, _i, _vp, _sz, _vp, _vp], _i),
}
EVAL_SCRATCH_BYTES = 16640


def library_path():
    return _build.LIB


def lib():
    """Load libgp103.so (building it first if it is missing or older than its sources)."""
    global _LIB
    if _LIB is None:
        if not _build.up_to_date():
            _build.build()
        path = _build.LIB
        if not os.path.exists(path):
            raise RuntimeError("libgp103.so is not built (python -m autoplace_gb300.build)")
        L = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def check(status, what):
    if status != OK:
        msg = lib().gp103_status_string(status).decode()
        raise RuntimeError("%s failed: %s (status %d)" % (what, msg, status))


def call(name, *args):
    check(getattr(lib(), name)(*args), name)


def device_error(plan_ref, stream_handle, clear=False):
    """The plan's device error flag (0: none; else the tensor-core field wait that ran out, DEVICE_ERRORS), read after
    the work queued on the stream; clear=True resets it."""
    code = _i(0)
    call("gp103_device_error", plan_ref, int(bool(clear)), ctypes.byref(code), stream_handle)
    return int(code.value)


def raise_device_error(code, what):
    raise RuntimeError("%s: the tensor-core field gave up waiting for %s (device error %d); its outputs were not "
                       "written" % (what, DEVICE_ERRORS.get(code, "?"), code))


def exported_symbols():
    return list(_SIGS)


def launch_count():
    return int(lib().gp103_launch_count())


def profile(stream_handle, fn):
    """Run fn() with the launch profile open: -> [(launcher name, ms)] in launch order."""
    call("gp103_profile_begin", stream_handle)
    try:
        fn()
    finally:
        ms = (ctypes.c_float * 512)()
        names = (ctypes.c_char_p * 512)()
        k = lib().gp103_profile_end(ms, names, 512)
    if k < 0:
        raise RuntimeError("gp103_profile_end failed")
    return [(names[i].decode(), float(ms[i])) for i in range(k)]
