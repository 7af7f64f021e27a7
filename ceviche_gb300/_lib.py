"""ctypes binding of libcevgpu.so (the C ABI declared in include/cevgpu.h).

The library is built in-tree by ``ceviche_gb300.build``.  There is no CPU
fallback: every entry point raises if the library or a CUDA device is missing.
"""
import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcevgpu.so")

CEV_OK = 0
CEV_ERR_INVALID = -1
CEV_ERR_CUDA = -2
CEV_ERR_WORKSPACE = -3
CEV_ERR_NUMERIC = -4
CEV_NOT_CONVERGED = 1
CEV_STAGNATED = 2
POL_EZ, POL_HZ = 0, 1
PREC_C64, PREC_C128 = 0, 1
PRECOND = {"none": 0, "shifted_laplacian": 1, "learned": 2, "separable": 3, "direct": 4}
STATUS_NAMES = {0: "converged", 1: "not converged", 2: "stagnated", -1: "invalid argument",
                -2: "CUDA error", -3: "workspace", -4: "non-finite values"}


class SolveOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("inner_rtol", C.c_double), ("max_iters", C.c_int),
                ("restart", C.c_int), ("precond", C.c_int), ("transpose", C.c_int),
                ("use_x0", C.c_int), ("reorth", C.c_int), ("max_stall", C.c_int),
                ("mg_levels", C.c_int), ("mg_shift", C.c_double), ("learned", C.c_void_p),
                ("separable", C.c_void_p), ("direct", C.c_void_p)]


class SolveInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("cycles", C.c_int),
                ("reserved", C.c_int), ("residual", C.c_double), ("bnorm", C.c_double)]


class FDTDState(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in
                ("hx", "hy", "dz", "icex", "icey", "idz", "hz", "dx", "dy", "ihz", "ichx", "ichy")]


class FDTDIOTE(C.Structure):
    _fields_ = [("n_src", C.c_int), ("src_idx", C.c_void_p), ("src_wx", C.c_void_p),
                ("src_wy", C.c_void_p), ("amps", C.c_void_p), ("n_probe", C.c_int),
                ("probe_idx", C.c_void_p), ("probe_out", C.c_void_p)]


class FDTDIO(C.Structure):
    _fields_ = [("n_src", C.c_int), ("src_idx", C.c_void_p), ("src_w", C.c_void_p),
                ("amps", C.c_void_p), ("n_probe", C.c_int), ("probe_idx", C.c_void_p),
                ("probe_out", C.c_void_p)]


P = C.c_void_p
I = C.c_int
D = C.c_double
S = C.c_size_t
PP = C.POINTER(C.c_void_p)

# name: (restype, argtypes) -- one line per declaration of include/cevgpu.h
SIGNATURES = {
    "cev_last_error_string": (C.c_char_p, []),
    "cev_version": (I, []),
    "cev_fdfd_plan_create": (I, [PP, I, I, I, I, D, C.POINTER(C.c_double), I, I, D, D]),
    "cev_fdfd_plan_destroy": (I, [P]),
    "cev_fdfd_plan_set_eps_complex": (I, [P, I]),
    "cev_sep_precond_create": (I, [PP, P, I, P, P, P, P, P]),
    "cev_sep_precond_destroy": (I, [P]),
    "cev_nd_precond_create": (I, [PP, P, P, I, I, D, P]),
    "cev_nd_precond_apply": (I, [P, P, P, P]),
    "cev_nd_precond_info": (I, [P, C.POINTER(S), C.POINTER(D), C.POINTER(I)]),
    "cev_nd_precond_destroy": (I, [P]),
    "cev_nd_analyse": (I, [I, I, C.POINTER(S), C.POINTER(I), C.POINTER(S), C.POINTER(D),
                           C.POINTER(S), C.POINTER(C.c_longlong)]),
    "cev_learned_param_count": (I, [I, C.POINTER(S)]),
    "cev_learned_create": (I, [PP, I, I, I, I]),
    "cev_learned_set_params": (I, [P, P, P]),
    "cev_learned_forward": (I, [P, P, P, I, P, P, P]),
    "cev_learned_backward": (I, [P, P, P, P]),
    "cev_adam_step": (I, [P, P, P, P, S, C.c_float, C.c_float, C.c_float, C.c_float, I, P]),
    "cev_learned_set_conv_impl": (I, [I]),
    "cev_learned_tc_fault": (I, [C.POINTER(I)]),
    "cev_learned_destroy": (I, [P]),
    "cev_fdfd_axis_matrix": (I, [P, I, I, I, P]),
    "cev_fdfd_plan_scale": (D, [P]),
    "cev_fdfd_apply": (I, [P, P, I, P, P, I, I, I, P]),
    "cev_solve_opts_default": (None, [C.POINTER(SolveOpts)]),
    "cev_fdfd_solve_workspace_size": (S, [P, C.POINTER(SolveOpts)]),
    "cev_fdfd_solve": (I, [P, P, I, P, P, C.POINTER(SolveOpts), C.POINTER(SolveInfo), P, S, P]),
    "cev_fdfd_fields": (I, [P, P, I, P, P, P, P]),
    "cev_fdfd_fields_adjoint": (I, [P, P, I, P, P, P, P, P, P]),
    "cev_fdfd_grad_eps": (I, [P, P, I, P, P, P, P]),
    "cev_fdfd_jvp_rhs": (I, [P, P, I, P, P, P, P]),
    "cev_fdfd_fields_jvp": (I, [P, P, I, P, P, P, P, P]),
    "cev_fdfd_mf_plan_create": (I, [PP, I, I, D, D, D, I, I, I, D, D]),
    "cev_fdfd_mf_apply": (I, [P, P, I, P, P, P, I, P]),
    "cev_fdfd_mf_solve_workspace_size": (S, [P, I, C.POINTER(SolveOpts)]),
    "cev_fdfd_mf_solve": (I, [P, P, I, P, P, P, C.POINTER(SolveOpts), C.POINTER(SolveInfo), P, S,
                              P]),
    "cev_fdfd_mf_grad": (I, [P, I, P, P, P, P, P]),
    "cev_csr_apply": (I, [I, I, P, P, P, P, P, P]),
    "cev_csr_solve_workspace_size": (S, [I, I, C.POINTER(SolveOpts)]),
    "cev_csr_solve": (I, [I, I, P, P, P, D, P, P, C.POINTER(SolveOpts), C.POINTER(SolveInfo), P, S,
                          P]),
    "cev_probe_measure": (I, [I, P, P, P, P, I, I, C.c_longlong, P, C.c_longlong, P]),
    "cev_mode_workspace_size": (S, [I, I, I]),
    "cev_mode_solve": (I, [I, I, P, D, D, I, I, D, I, P, P, P, P, P, S, P]),
    "cev_dense_eig": (I, [I, P, P, P]),
    "cev_fdtd_plan_create": (I, [PP, I, I, D, I, I, I, P, P]),
    "cev_fdtd_plan_destroy": (I, [P]),
    "cev_fdtd_set_eps": (I, [P, P, P]),
    "cev_fdtd_dt": (D, [P]),
    "cev_fdtd_step": (I, [P, C.POINTER(FDTDState), P, P, P, I, P]),
    "cev_fdtd_e_fields": (I, [P, C.POINTER(FDTDState), P, P, P, P]),
    "cev_fdtd_run_tm": (I, [P, C.POINTER(FDTDState), I, C.POINTER(FDTDIO), P]),
    "cev_fdtd_run_te": (I, [P, C.POINTER(FDTDState), I, C.POINTER(FDTDIOTE), P]),
    "cev_fdtd_run_tm_noalloc": (I, [I, I, D, I, I, P, C.POINTER(FDTDState), I, C.POINTER(FDTDIO),
                                    P]),
    "cev_fdtd_step_adjoint_tm": (I, [P, P, P, P, C.POINTER(FDTDState), P, P, P]),
    "cev_fdtd_adjoint_workspace_size": (S, [P, I, I]),
    "cev_fdtd_adjoint_tm": (I, [P, I, I, C.POINTER(FDTDIO), P, P, P, S, P]),
}

_lib = None
_lock = threading.Lock()


class CevError(RuntimeError):
    """Error status returned by the GPU library."""


def load(path=LIB_PATH):
    """Load libcevgpu.so (no CUDA call is made).  Raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise CevError(f"{path} not found: build it with "
                           f"`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc, what=""):
    """Raise CevError for negative statuses; return rc otherwise."""
    if rc < 0:
        msg = load().cev_last_error_string().decode(errors="replace")
        raise CevError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {msg}")
    return rc


def stream_ptr(torch_stream=None):
    import torch
    s = torch_stream if torch_stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def ptr(t):
    """Device pointer of a torch tensor (None -> NULL)."""
    if t is None:
        return None
    if t.is_conj() or t.is_neg():
        raise ValueError("lazily conjugated/negated tensor: call resolve_conj()/resolve_neg()")
    return C.c_void_p(t.data_ptr())
