"""ctypes binding of libissm103.so (include/issm.h).

This is the only route from Python to the GPU kernels. There is no CPU
fallback: if the library or a CUDA device is missing, `require()` raises.
Tensors are passed as raw device pointers; the current torch stream is used
unless a stream is given.
"""
import contextlib
import ctypes as C
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY = os.path.join(HERE, "libissm103.so")

F32, F64 = 0, 1
GAUSSIAN, STUDENT_T = 0, 1
SCALE_FACTOR, SCALE_DIAGONAL, SCALE_SPHERICAL = 0, 1, 2
DENOM_FULL, DENOM_GENERATING, DENOM_PARTIAL, DENOM_PREFIX = 0, 1, 2, 3
PREC_NATIVE, PREC_TF32, PREC_BF16 = 0, 1, 2
PREC_BF16X1 = 3  # regression likelihood only: one bf16 product per K slice

REASON_TARGET_NAN = 0x0100
REASON_TARGET_POS_INF = 0x0200
REASON_PROPOSAL_INVALID = 0x0400
REASON_GENERATED_NONFINITE = 0x0800
REASON_LOGWEIGHT_INVALID = 0x1000
REASON_DRAW_EXHAUSTED = 0x0010
REASON_MOMENT_FIT_INVALID = 0x2000

E_ALL_ZERO = -5


class NativeError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = _lib.issm_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{where}: {msg} (status {status})")


class Bank(C.Structure):
    _fields_ = [("dim", C.c_int32), ("count", C.c_int32), ("family", C.c_int32),
                ("scale_kind", C.c_int32), ("dtype", C.c_int32), ("reserved", C.c_int32),
                ("locations", C.c_void_p), ("scales", C.c_void_p), ("lognormalizers", C.c_void_p),
                ("dofs", C.c_void_p), ("range_risk", C.c_void_p), ("inverse_factors", C.c_void_p)]


class Denominator(C.Structure):
    _fields_ = [("kind", C.c_int32), ("terms", C.c_int32), ("logcoefficients", C.c_void_p),
                ("group_of_slot", C.c_void_p)]


class Target(C.Structure):
    _fields_ = [("kind", C.c_int32), ("dim", C.c_int32), ("count", C.c_int32), ("dtype", C.c_int32),
                ("a", C.c_void_p), ("b", C.c_void_p), ("c", C.c_void_p), ("p0", C.c_double), ("p1", C.c_double)]


class AmisRunDesc(C.Structure):
    """issm_amis_run_desc (include/issm.h)."""
    _fields_ = [("history", Bank), ("target", C.c_void_p), ("rounds", C.c_int32), ("precision", C.c_int32),
                ("round_sizes", C.c_void_p), ("logconstant", C.c_double), ("seed", C.c_uint64),
                ("normal_offset", C.c_uint64), ("counter", C.c_void_p), ("logcounts", C.c_void_p),
                ("round_ids_init", C.c_void_p), ("initial_location", C.c_void_p), ("initial_factor", C.c_void_p),
                ("initial_lognormalizer", C.c_void_p), ("samples", C.c_void_p), ("logtargets", C.c_void_p),
                ("lognum", C.c_void_p), ("logweights", C.c_void_p), ("round_ids", C.c_void_p),
                ("summaries", C.c_void_p), ("round_failures", C.c_void_p), ("mean", C.c_void_p),
                ("cov", C.c_void_p), ("shift", C.c_void_p), ("cand_location", C.c_void_p),
                ("cand_factor", C.c_void_p), ("cand_lognormalizer", C.c_void_p), ("workspace", C.c_void_p),
                ("workspace_bytes", C.c_size_t), ("target_operand", C.c_void_p), ("target_precision", C.c_int32),
                ("reserved", C.c_int32), ("target_bank", C.c_void_p), ("target_den", C.c_void_p),
                ("target_bank_precision", C.c_int32), ("reserved2", C.c_int32)]


TARGET_GAUSS_MIX, TARGET_STUDENT_T, TARGET_LINREG, TARGET_LOGISTIC, TARGET_STD_NORMAL, TARGET_QUADRATIC = range(6)

# (name, restype, argtypes) for every entry point of include/issm.h
_p, _i32, _i64, _u64, _d, _sz = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_size_t
_bank, _den = C.POINTER(Bank), C.POINTER(Denominator)
SIGNATURES = [
    ("issm_version", C.c_char_p, []),
    ("issm_status_string", C.c_char_p, [C.c_int]),
    ("issm_kernel_launches", C.c_uint64, []),
    ("issm_failure_reset", C.c_int, [_p, _p]),
    ("issm_fill_normals", C.c_int, [_u64, _u64, _i64, _p, _i32, _p]),
    ("issm_fill_uniforms", C.c_int, [_u64, _u64, _i64, _p, _i32, _p]),
    ("issm_fill_normals_at", C.c_int, [_u64, _p, _u64, _i64, _p, _i32, _p]),
    ("issm_fill_uniforms_at", C.c_int, [_u64, _p, _u64, _i64, _p, _i32, _p]),
    ("issm_counter_advance", C.c_int, [_p, _u64, _p]),
    ("issm_static_assign", C.c_int, [_p, _i32, _p, _i64, _i32, _p, _i32, _p]),
    ("issm_draw", C.c_int, [_bank, _p, _i32, _p, _p, _i32, _p, _i32, _i64, _p, _p, _i64, _p]),
    ("issm_draw_philox", C.c_int, [_bank, _i32, _u64, _p, _u64, _p, _i32, _p, _i32, _i64, _p, _p, _i64, _p]),
    ("issm_mixture_logdensity", C.c_int, [_bank, _den, _p, _i64, _p, _i32, _p, _p, _p, _i64, _i32, _p]),
    ("issm_mis_round", C.c_int, [_bank, _den, _p, _p, _p, _i32, _p, _i32, _p, _i64, _p, _p, _p, _p, _p,
                                 _i32, _p]),
    ("issm_add_target_values", C.c_int, [_p, _p, _i64, _i32, _p, _i64, _p]),
    ("issm_subtract_logweights", C.c_int, [_p, _p, _i64, _i32, _p, _p, _i64, _p]),
    ("issm_check_target_values", C.c_int, [_p, _i64, _i32, _p, _p, _i64, _p]),
    ("issm_amis_append", C.c_int, [_bank, _i32, _p, _p, _i64, _p, _p, _i32, _p]),
    ("issm_amis_form", C.c_int, [_p, _p, _p, _d, _i64, _i32, _p, _p, _p]),
    ("issm_amis_form_summary", C.c_int, [_p, _p, _p, _d, _i64, _i32, _p, _p, _p, _p, _sz, _p]),
    ("issm_reduce_workspace_bytes", _sz, [_i64]),
    ("issm_logweight_summary", C.c_int, [_p, _i64, _i32, _p, _p, _sz, _p]),
    ("issm_normalize", C.c_int, [_p, _i64, _i32, _p, _p, _p]),
    ("issm_resampling_cdf", C.c_int, [_p, _i64, _i32, _p, _p, _sz, _p]),
    ("issm_resampling_cdf_static_max", _i64, []),
    ("issm_resampling_cdf_static", C.c_int, [_p, _i64, _i32, _p, _p]),
    ("issm_resample_select", C.c_int, [_p, _p, _i64, _p, _i64, _i32, _p, _p]),
    ("issm_resample_workspace_bytes", _sz, [_i64]),
    ("issm_resample_multinomial", C.c_int, [_p, _i64, _i32, _p, _i64, _p, _p, _sz, _p]),
    ("issm_resample_systematic", C.c_int, [_p, _i64, _i32, _d, _i64, _p, _p, _sz, _p]),
    ("issm_gather", C.c_int, [_p, _i32, _i64, _p, _i64, _i32, _p, _p]),
    ("issm_local_resample", C.c_int, [_p, _p, _i32, _p, _p, _i32, _i32, _p, _p, _p]),
    ("issm_moments_workspace_bytes", _sz, [_i64, _i32]),
    ("issm_weighted_moments", C.c_int, [_p, _i32, _i64, _p, _i32, _p, _p, _p, _p, _p, _sz, _p]),
    ("issm_fit_factor", C.c_int, [_p, _p, _i32, _p, _d, _d, _i32, _p, _p, _p, _p, _i64, _p]),
    ("issm_fit_factor_ex", C.c_int, [_p, _p, _i32, _p, _d, _d, _i32, _p, _p, _p, _p, _p, _i64, _p]),
    ("issm_fit_factor_reg", C.c_int, [_p, _p, _i32, _p, _d, _d, _i32, _d, _p, _p, _p, _p, _p, _i64, _p]),
    ("issm_group_run_bytes", _sz, []),
    ("issm_group_step", C.c_int, [_p, _i32, _i64, _i64, _i64, _p]),
    ("issm_weighted_sum_workspace_bytes", _sz, [_i64, _i32]),
    ("issm_weighted_sum", C.c_int, [_p, _i32, _i64, _p, _i32, _p, _p, _p, _sz, _p]),
    ("issm_weighted_quantile_workspace_bytes", _sz, [_i32, _i32]),
    ("issm_weighted_quantile", C.c_int, [_p, _i32, _i64, _p, _i32, _p, _p, _i32, _p, _p, _sz, _p]),
    ("issm_glm_operand_bytes", _sz, [_i32, _i32, _i32]),
    ("issm_glm_prepare", C.c_int, [C.POINTER(Target), _i32, _p, _sz, _p]),
    ("issm_glm_logdensity", C.c_int, [C.POINTER(Target), _i32, _p, _p, _i64, _p, _p, _p]),
    ("issm_select_workspace_bytes", _sz, []),
    ("issm_select_kth", C.c_int, [_p, _i64, _i64, _i32, _p, _p, _sz, _p]),
    ("issm_npmc_clip", C.c_int, [_p, _i64, _i32, _p, _p, _p, _sz, _p]),
    ("issm_population_local_weights", C.c_int, [_p, _p, _i32, _i32, _p, _p, _p, _i32, _d, _i32, _p, _p, _p, _p,
                                                _p, _p]),
    ("issm_population_covariances", C.c_int, [_p, _i32, _i32, _p, _p, _p, _p, _bank, _p, _p, _i32, _p, _p, _p]),
    ("issm_population_factors", C.c_int, [_p, _i32, _i32, _i32, _p, _p, _p, _p, _p]),
    ("issm_target_logdensity", C.c_int, [C.POINTER(Target), _p, _i64, _p, _p]),
    ("issm_tc_selftest", C.c_int, [_p, _p, _p, _i32, _i32, _i32, _p, _p]),
    ("issm_amis_run_workspace_bytes", _sz, [_i32, _i64, _i32]),
    ("issm_amis_run", C.c_int, [C.POINTER(AmisRunDesc), _p]),
    ("issm_amis_run_desc_bytes", _sz, []),
    ("issm_amis_run_desc_workspace_offset", _sz, []),
    ("issm_tc_workspace_bytes", _sz, [_i32, _i32]),
    ("issm_invert_factors", C.c_int, [_bank, _i32, _i32, _p, _p]),
    ("issm_mixture_logdensity_ws", C.c_int, [_bank, _den, _p, _i64, _p, _i32, _p, _p, _p, _i64, _i32, _p, _sz,
                                             _p]),
    ("issm_amis_append_ws", C.c_int, [_bank, _i32, _p, _p, _i64, _p, _p, _i32, _p, _sz, _p]),
    ("issm_weighted_moments_ws", C.c_int, [_p, _i32, _i64, _p, _i32, _p, _p, _p, _p, _p, _i32, _p, _sz, _p]),
]

_lib = None


def library_path():
    return LIBRARY


def load():
    """Load libissm103.so and declare every entry point (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBRARY):
        raise RuntimeError(
            f"libissm103.so is not built at {LIBRARY}; run __graft_entry__.build() (needs nvcc)")
    lib = C.CDLL(LIBRARY)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def require():
    """Fail loudly unless the native library and a CUDA device are usable."""
    load()
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required: the importance-sampling path has no CPU fallback")


def lib():
    return load()


def dtype_code(dtype):
    if dtype == torch.float32:
        return F32
    if dtype == torch.float64:
        return F64
    raise TypeError(f"unsupported dtype {dtype}; use float32 or float64")


def ptr(t):
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_contiguous():
        raise ValueError("tensors passed to libissm103.so must be contiguous (raw column-major layouts)")
    return t.data_ptr()


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def check(status, where):
    if status != 0:
        raise NativeError(status, where)


def call(name, *args):
    fn = getattr(lib(), name)
    st = fn(*args)
    check(st, name)
    return st


_replayed = [0]


def note_replay(launches):
    """Count the kernels of a replayed CUDA graph (their host launch calls ran
    once, at capture)."""
    _replayed[0] += int(launches)


def launches():
    """Kernels launched by this process: direct launches plus graph replays."""
    return int(lib().issm_kernel_launches()) + _replayed[0]


_workspaces = {}
_retired = []  # outgrown workspaces stay allocated: a recorded CUDA graph may still address them
_scope = threading.local()


@contextlib.contextmanager
def workspace_scope(name):
    """Give the launches inside the block their own scratch buffers (keyed by
    `name`), so work running concurrently on other streams never shares one."""
    prev = getattr(_scope, "name", None)
    _scope.name = name
    try:
        yield
    finally:
        _scope.name = prev


def release_scope(name):
    """Free the scratch buffers of a scope once its work has completed."""
    for key in [k for k in _workspaces if k[2] == name]:
        del _workspaces[key]


def workspace(nbytes, device=None, tag="default", zero=False):
    """A cached device scratch buffer of at least nbytes (per device, tag and
    workspace scope); zero=True allocates it zero-filled (sticky error words
    live at its end)."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    key = (str(device), tag, getattr(_scope, "name", None))
    buf = _workspaces.get(key)
    if buf is None or buf.numel() < nbytes:
        if buf is not None:
            _retired.append(buf)
        alloc = torch.zeros if zero else torch.empty
        buf = alloc(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _workspaces[key] = buf
    return buf


def scoped_workspace(device, tag):
    """The current scope's buffer for `tag`, or None."""
    return _workspaces.get((str(device), tag, getattr(_scope, "name", None)))


def tc_error(device=None):
    """The sticky tensor-core wait-timeout word of the device's tc workspace."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    buf = scoped_workspace(device, "tc")
    if buf is None:
        return 0
    return int(buf[-64:-60].view(torch.int32).item())
