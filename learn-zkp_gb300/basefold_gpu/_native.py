"""ctypes binding of libbasefold_gpu.so (the C ABI of include/basefold_gpu.h).

There is no fallback: if the library is missing or a call fails, an exception
is raised.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libbasefold_gpu.so")

# Every symbol declared in include/basefold_gpu.h.
EXPORTS = [
    "bf_last_error", "bf_device_info", "bf_kernel_launches", "bf_pcs_setup", "bf_pcs_free", "bf_pcs_num_queries", "bf_pcs_proof_size",
    "bf_commit", "bf_commit_device", "bf_commitment_free", "bf_commitment_root", "bf_commitment_data", "bf_eval",
    "bf_open", "bf_open_start", "bf_open_round", "bf_open_challenge", "bf_open_poll", "bf_open_final",
    "bf_open_finish", "bf_open_session_free", "bf_verify", "bf_challenger_new", "bf_challenger_clone", "bf_challenger_free",
    "bf_challenger_observe", "bf_challenger_sample_ext", "bf_challenger_sample_bits", "bf_challenger_state",
    "bf_challenger_from_state", "bf_sumcheck_prove", "bf_sumcheck_prove_device", "bf_profile_enable",
    "bf_profile_read", "bf_test_gf_mul", "bf_test_keccak_f", "bf_engine_create", "bf_engine_free",
    "bf_engine_proof_size", "bf_engine_prove", "bf_engine_start", "bf_engine_stop", "bf_engine_submit",
    "bf_engine_poll", "bf_eval_noalloc", "bf_pcs_autotune", "bf_pcs_get_tune", "bf_pcs_set_tune",
    "bf_engine_autotune", "bf_engine_graphs", "bf_engine_stats", "bf_verify_batch", "bf_engine_set_tune", "bf_engine_cancel", "bf_engine_schedule",
    "bf_eval_data", "bf_tune_cache_load", "bf_tune_cache_save", "bf_tune_cache_clear",
    "bf_bb_pcs_setup", "bf_bb_pcs_setup_generic", "bf_bb_pcs_free", "bf_bb_pcs_num_queries", "bf_bb_pcs_proof_size", "bf_bb_commit",
    "bf_bb_commit_device", "bf_bb_commitment_root", "bf_bb_commitment_free", "bf_bb_eval", "bf_bb_eval_data", "bf_bb_open",
    "bf_bb_verify", "bf_challenger_sample_bb_ext",
]

BF_OK = 0
BF_ERR_ARG = -1
BF_ERR_CUDA = -2
BF_ERR_OOM = -3
BF_ERR_BUFFER = -4
BF_ERR_UNSUPPORTED = -5
BF_ERR_NOT_INVERTIBLE = -6
BF_ERR_CHECK = -7
BF_ERR_CANCELLED = -8


class BfJob(C.Structure):
    """bf_job of include/basefold_gpu.h."""
    _fields_ = [
        ("num_vars", C.c_int32), ("status", C.c_int32), ("evals", C.c_void_p), ("point", C.c_void_p),
        ("proof", C.c_void_p), ("proof_cap", C.c_size_t), ("proof_len", C.c_size_t), ("latency_ms", C.c_double),
        ("root", C.c_uint8 * 32), ("value", C.c_uint8 * 16),
    ]


class BfVerifyJob(C.Structure):
    """bf_verify_job of include/basefold_gpu.h."""
    _fields_ = [
        ("root", C.c_void_p), ("point", C.c_void_p), ("values", C.c_void_p), ("width", C.c_size_t),
        ("challenger", C.c_void_p), ("proof", C.c_void_p), ("proof_len", C.c_size_t), ("result", C.c_int32),
    ]


class BasefoldGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built: run `python learn-zkp_gb300/build.py` "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    u8p = C.c_void_p
    vp = C.c_void_p
    sz = C.c_size_t
    i = C.c_int
    decl = {
        "bf_last_error": ([C.c_char_p, sz], i),
        "bf_device_info": ([i, C.POINTER(i), C.POINTER(i), C.POINTER(i)], i),
        "bf_kernel_launches": ([C.POINTER(C.c_uint64)], i),
        "bf_pcs_setup": ([i, i, i, i, vp, C.POINTER(vp)], i),
        "bf_pcs_free": ([vp], None),
        "bf_pcs_num_queries": ([vp], sz),
        "bf_pcs_proof_size": ([vp, sz, i], sz),
        "bf_commit": ([vp, u8p, sz, C.POINTER(vp), u8p], i),
        "bf_commit_device": ([vp, vp, sz, C.POINTER(vp), u8p], i),
        "bf_commitment_free": ([vp], None),
        "bf_commitment_root": ([vp, u8p], i),
        "bf_commitment_data": ([vp, u8p, sz], i),
        "bf_eval": ([vp, vp, u8p, u8p], i),
        "bf_eval_data": ([vp, vp, i, sz, u8p, u8p], i),
        "bf_tune_cache_load": ([C.c_char_p], i),
        "bf_tune_cache_save": ([C.c_char_p], i),
        "bf_tune_cache_clear": ([], i),
        "bf_open": ([vp, vp, u8p, u8p, i, vp, u8p, sz, C.POINTER(sz)], i),
        "bf_open_start": ([vp, vp, u8p, u8p, u8p, vp, C.POINTER(vp)], i),
        "bf_open_round": ([vp, C.POINTER(i), u8p, u8p], i),
        "bf_open_challenge": ([vp, u8p], i),
        "bf_open_poll": ([vp], i),
        "bf_open_final": ([vp, u8p], i),
        "bf_open_finish": ([vp, C.POINTER(C.c_uint64), sz, u8p, sz, C.POINTER(sz)], i),
        "bf_open_session_free": ([vp], None),
        "bf_verify": ([vp, u8p, u8p, u8p, sz, i, vp, u8p, sz], i),
        "bf_challenger_new": ([u8p, sz, C.POINTER(vp)], i),
        "bf_challenger_clone": ([vp, C.POINTER(vp)], i),
        "bf_challenger_free": ([vp], None),
        "bf_challenger_observe": ([vp, u8p, sz], i),
        "bf_challenger_sample_ext": ([vp, u8p], i),
        "bf_challenger_sample_bits": ([vp, i, C.POINTER(C.c_uint64)], i),
        "bf_challenger_state": ([vp, u8p, sz, C.POINTER(sz)], i),
        "bf_challenger_from_state": ([u8p, sz, C.POINTER(vp)], i),
        "bf_sumcheck_prove": ([i, i, i, u8p, u8p, vp, u8p], i),
        "bf_sumcheck_prove_device": ([vp, i, i, vp, u8p, vp, u8p], i),
        "bf_profile_enable": ([vp, i], i),
        "bf_profile_read": ([vp, C.POINTER(C.c_double), C.POINTER(C.c_uint64), i], i),
        "bf_test_gf_mul": ([i, u8p, u8p, u8p, sz], i),
        "bf_test_keccak_f": ([i, C.POINTER(C.c_uint64), sz], i),
        "bf_engine_create": ([i, i, i, i, sz, C.POINTER(vp)], i),
        "bf_engine_free": ([vp], None),
        "bf_engine_proof_size": ([vp, i], sz),
        "bf_engine_prove": ([vp, C.POINTER(BfJob), sz, i], i),
        "bf_engine_start": ([vp], i),
        "bf_engine_stop": ([vp], i),
        "bf_engine_submit": ([vp, C.POINTER(BfJob), i], i),
        "bf_engine_poll": ([vp, C.POINTER(C.POINTER(BfJob)), sz, C.POINTER(sz)], i),
        "bf_eval_noalloc": ([vp, i, u8p, vp, vp], i),
        "bf_pcs_autotune": ([vp, i, C.c_char_p, sz], i),
        "bf_pcs_get_tune": ([vp, C.POINTER(C.c_int), i], i),
        "bf_pcs_set_tune": ([vp, C.POINTER(C.c_int), i], i),
        "bf_engine_autotune": ([vp, i], i),
        "bf_engine_graphs": ([vp, i], i),
        "bf_engine_stats": ([vp, C.POINTER(C.c_double), i], i),
        "bf_verify_batch": ([vp, C.POINTER(BfVerifyJob), sz], i),
        "bf_engine_set_tune": ([vp, C.POINTER(i), i], i),
        "bf_engine_cancel": ([vp, vp], i),
        "bf_engine_schedule": ([vp, i, i], i),
        "bf_bb_pcs_setup": ([i, i, i, i, vp, C.POINTER(vp)], i),
        "bf_bb_pcs_setup_generic": ([i, i, i, i, i, vp, sz, vp, C.POINTER(vp)], i),
        "bf_bb_pcs_free": ([vp], None),
        "bf_bb_pcs_num_queries": ([vp], sz),
        "bf_bb_pcs_proof_size": ([vp, sz, i], sz),
        "bf_bb_commit": ([vp, vp, sz, C.POINTER(vp), u8p], i),
        "bf_bb_commit_device": ([vp, vp, sz, C.POINTER(vp), u8p], i),
        "bf_bb_commitment_root": ([vp, u8p], i),
        "bf_bb_commitment_free": ([vp], None),
        "bf_bb_eval": ([vp, vp, u8p, u8p], i),
        "bf_bb_eval_data": ([vp, vp, i, sz, u8p, u8p], i),
        "bf_bb_open": ([vp, vp, u8p, u8p, i, vp, u8p, sz, C.POINTER(sz)], i),
        "bf_bb_verify": ([vp, u8p, u8p, u8p, sz, i, vp, u8p, sz], i),
        "bf_challenger_sample_bb_ext": ([vp, u8p], i),
    }
    for name, (args, res) in decl.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().bf_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int) -> int:
    if rc < 0:
        raise BasefoldGpuError(rc, last_error())
    return rc
