"""Loader and ctypes signatures of the C ABI (include/effsc_gpu.h).

The CUDA library must have been built in-tree (``efficient-sumcheck_gb300/
_build/libeffsc_gpu.so``); there is no CPU fallback, so a missing library is
an error.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_DIR, "_build", "libeffsc_gpu.so")

u64p = ctypes.POINTER(ctypes.c_uint64)
u8p = ctypes.POINTER(ctypes.c_uint8)
vp = ctypes.c_void_p
sz = ctypes.c_size_t
ci = ctypes.c_int

# name -> (restype, argtypes); every symbol include/effsc_gpu.h declares
SIGNATURES = {
    "effsc_last_error": (ctypes.c_char_p, []),
    "effsc_status_str": (ctypes.c_char_p, [ci]),
    "effsc_launch_count": (ctypes.c_uint64, []),
    "effsc_launch_count_reset": (None, []),
    "effsc_profile_enable": (ci, [ci]),
    "effsc_profile_count": (sz, []),
    "effsc_profile_get": (ci, [sz, ctypes.c_char_p, sz, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]),
    "effsc_profile_clear": (None, []),
    "effsc_diag_mulmod_rate": (ci, [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "effsc_diag_accumulate_rate": (ci, [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "effsc_ctx_create": (ci, [ci, ctypes.POINTER(vp)]),
    "effsc_ctx_destroy": (ci, [vp]),
    "effsc_ctx_set_stream": (ci, [vp, vp]),
    "effsc_ctx_synchronize": (ci, [vp]),
    "effsc_prover_create": (ci, [vp, ci, ci, ci, ci, ci, ctypes.POINTER(u64p), ctypes.POINTER(sz),
                                 ctypes.POINTER(ci), ctypes.POINTER(vp)]),
    "effsc_eqf_create": (ci, [vp, ci, ci, u64p, sz, u64p, sz, ci, ctypes.POINTER(vp)]),
    "effsc_prover_create_device": (ci, [vp, ci, ci, ci, ci, ctypes.POINTER(u64p), ctypes.POINTER(sz),
                                        ctypes.POINTER(ci), ctypes.POINTER(vp)]),
    "effsc_prover_destroy": (ci, [vp]),
    "effsc_prover_degree": (ci, [vp]),
    "effsc_prover_round": (ci, [vp, u64p, u64p, u64p]),
    "effsc_prover_finalize": (ci, [vp, u64p]),
    "effsc_prover_final_value": (ci, [vp, u64p]),
    "effsc_prover_table_len": (ci, [vp, ci, ctypes.POINTER(sz)]),
    "effsc_prover_read_table": (ci, [vp, ci, u64p]),
    "effsc_prover_reset": (ci, [vp]),
    "effsc_prove": (ci, [vp, sz, vp, u8p, sz, ci, u64p, u64p, u64p]),
    "effsc_transcript_create": (ci, [ci, ci, ci, u8p, sz, ctypes.c_uint64, ctypes.POINTER(vp)]),
    "effsc_transcript_destroy": (ci, [vp]),
    "effsc_transcript_clone": (ci, [vp, ctypes.POINTER(vp)]),
    "effsc_transcript_absorb": (ci, [vp, u8p, sz]),
    "effsc_transcript_squeeze": (ci, [vp, u8p, sz]),
    "effsc_transcript_send": (ci, [vp, u64p]),
    "effsc_transcript_challenge": (ci, [vp, u64p]),
    "effsc_verify": (ci, [ci, ci, u64p, sz, sz, vp, u8p, sz, u64p, u64p, u64p]),
    "effsc_fold": (ci, [vp, ci, ci, u64p, sz, ci, u64p, u64p, ctypes.POINTER(sz)]),
    "effsc_compute_sumcheck_polynomial": (ci, [vp, ci, ci, u64p, sz, ci, u64p]),
    "effsc_coef_expr_create": (ci, [vp, ci, ci, ci, ci, ci, ctypes.POINTER(u64p), ctypes.POINTER(ci), ci,
                                    ctypes.POINTER(u64p), ctypes.POINTER(sz), ctypes.POINTER(ci), sz, vp, sz,
                                    ctypes.POINTER(vp)]),
    "effsc_fused_fold_and_compute_polynomial": (ci, [vp, ci, ci, u64p, sz, ci, u64p, u64p, ctypes.POINTER(sz), u64p]),
    "effsc_build_eq_table": (ci, [vp, ci, ci, u64p, sz, u64p]),
    "effsc_gen_uniform": (ci, [vp, ctypes.c_uint64, ctypes.c_uint64, u64p, u64p]),
    "effsc_table_seed": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_uint64]),
    "effsc_prover_create_host": (ci, [vp, ci, ci, ci, ci, ctypes.POINTER(u64p), ctypes.POINTER(sz),
                                      ctypes.POINTER(ci), ctypes.POINTER(vp)]),
    "effsc_reorder_msb": (ci, [vp, u64p, sz, ci, u64p]),
    "effsc_stream_claim": (ci, [vp, ci, ci, ctypes.POINTER(u64p), sz, ci, u64p]),
    "effsc_protogalaxy_fold": (ci, [vp, ci, u64p, sz, u64p, sz, sz, u64p, ctypes.POINTER(sz)]),
    "effsc_diag_transcript_latency": (ci, [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "effsc_verify_batch": (ci, [vp, ci, sz, u64p, ci, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(vp), u8p, sz,
                                u64p, u64p, u64p]),
    "effsc_gkr_create": (ci, [vp, ci, ci, u64p, u64p, u64p, sz, ci, ctypes.POINTER(vp)]),
    "effsc_gkr_claimed_w_values": (ci, [vp, u64p]),
    "effsc_diag_bounded_wait": (ci, [vp, ctypes.c_uint64, ci, ctypes.POINTER(ctypes.c_uint32)]),
    "effsc_prover_set_tail": (ci, [vp, sz]),
    "effsc_prover_set_first_rounds": (ci, [vp, ci]),
    "effsc_prover_set_persistent": (ci, [vp, sz]),
    "effsc_batch_create": (ci, [vp, ci, ci, sz, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(u64p), u64p,
                                ctypes.POINTER(vp)]),
    "effsc_batch_destroy": (ci, [vp]),
    "effsc_batch_prove": (ci, [vp, ctypes.POINTER(vp), ci, u64p, u64p, u64p]),
    "effsc_batch_set_quads_per_thread": (ci, [vp, ci]),
    "effsc_batch_set_tail": (ci, [vp, ctypes.c_uint64]),
    "effsc_batch_tune": (ci, [vp, ctypes.POINTER(vp), ctypes.c_char_p, ctypes.POINTER(ci), u64p]),
    "effsc_batch_device_table": (ci, [vp, sz, ci, ctypes.POINTER(u64p)]),
    "effsc_server_create": (ci, [vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(vp)]),
    "effsc_server_destroy": (ci, [vp]),
    "effsc_server_submit": (ci, [vp, ci, ci, ctypes.c_uint32, ctypes.POINTER(u64p), u64p, vp, u64p]),
    "effsc_server_progress": (ci, [vp, ci, ctypes.POINTER(ctypes.c_uint32)]),
    "effsc_server_take": (ci, [vp, u64p, ctypes.POINTER(ctypes.c_uint32), u64p, u64p, u64p,
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "effsc_server_run_trace": (ci, [vp, sz, ctypes.POINTER(ci), ci, ctypes.POINTER(ctypes.c_uint32), u64p,
                                    ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), u64p, u64p,
                                    u64p]),
    "effsc_server_run_trace_host": (ci, [vp, sz, ctypes.POINTER(ci), ci, ctypes.POINTER(ctypes.c_uint32),
                                         ctypes.POINTER(u64p), ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), u64p, u64p,
                                         u64p]),
    "effsc_ip_round_noalloc": (ci, [vp, vp, vp, vp, sz, u64p, vp, ci, vp]),
    "effsc_device_alloc": (ci, [vp, sz, ctypes.POINTER(vp)]),
    "effsc_device_free": (ci, [vp, vp]),
    "effsc_memcpy_h2d": (ci, [vp, vp, vp, sz]),
    "effsc_memcpy_d2h": (ci, [vp, vp, vp, sz]),
}

_lib = None


class EffscError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("effsc status %d (%s): %s" % (status, STATUS.get(status, "?"), msg))
        self.status = status


class ReferencePanic(EffscError):
    """Raised where the reference crate panics (e.g. unequal table lengths)."""


STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "CUDA error",
          4: "timeout", 5: "unsupported", 6: "reference panics"}


def load(path=None):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("the CUDA library %s is missing: run __graft_entry__.build() "
                          "(there is no CPU fallback)" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != 0:
        msg = load().effsc_last_error().decode(errors="replace")
        if rc == 6:
            raise ReferencePanic(rc, msg)
        raise EffscError(rc, msg)
