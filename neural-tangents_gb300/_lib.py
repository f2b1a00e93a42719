"""ctypes binding of libntgb300.so (the C ABI declared in include/nt_gb300.h).

The library is loaded from this package directory. On a CUDA machine a
missing or unloadable library is an error: there is no CPU fallback for any
kernel of this package.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libntgb300.so')

NTG_ACT_NONE, NTG_ACT_ABRELU, NTG_ACT_ERF = 0, 1, 2
NTG_ACT_SIN, NTG_ACT_RBF, NTG_ACT_GELU = 3, 4, 5
NTG_PAD_ZERO, NTG_PAD_CIRCULAR = 0, 1
NTG_TUNE_STENCIL_RING = 0
CHAIN_MAX_SEG, CHAIN_MAX_LAYERS = 4, 16

ERRORS = {
    1: 'invalid argument', 2: 'CUDA error', 3: 'unsupported', 4: 'not positive definite',
    5: 'wait timeout', 6: 'no device scratch',
}


class Act(C.Structure):
    _fields_ = [('kind', C.c_int32), ('a', C.c_float), ('b', C.c_float), ('c', C.c_float),
                ('compensated', C.c_int32), ('stabilize', C.c_float)]


class Affine(C.Structure):
    _fields_ = [('w2', C.c_float), ('b2', C.c_float), ('ntk_w2', C.c_float),
                ('ntk_nn', C.c_float), ('ntk_c', C.c_float), ('nn_scaled', C.c_int32)]


class Var(C.Structure):
    _fields_ = [('base', C.c_void_p), ('s_n', C.c_int64), ('s_a', C.c_int64),
                ('s_c', C.c_int64)]


class Chain(C.Structure):
    _fields_ = [('nseg', C.c_int32), ('s0', C.c_int32), ('channels', C.c_int32),
                ('readout', C.c_int32), ('nconv', C.c_int32 * CHAIN_MAX_SEG),
                ('aff', Affine * CHAIN_MAX_LAYERS), ('act', Act * CHAIN_MAX_LAYERS),
                ('var_off', C.c_int64 * CHAIN_MAX_LAYERS), ('var_stride', C.c_int64)]


_P, _I64, _I32, _F = C.c_void_p, C.c_int64, C.c_int32, C.c_float

SIGNATURES = {
    'ntg_last_error': ([], C.c_char_p),
    'ntg_version': ([], C.c_char_p),
    'ntg_launch_count': ([], C.c_uint64),
    'ntg_device_status': ([], C.c_int),
    'ntg_tune_set': ([_I32, _I32], C.c_int),
    'ntg_tune_get': ([_I32], C.c_int32),
    'ntg_gram': ([_P, _P, _P, _I64, _I64, _I64, _P, _I32, _P, C.c_size_t], C.c_int),
    'ntg_gram_workspace_bytes': ([_I64, _I64, _I64], C.c_size_t),
    'ntg_gemm': ([_P, _P, _P, _P, _I64, _I64, _I64, _I32], C.c_int),
    'ntg_cov_diag': ([_P, _P, _I64, _I64, _P], C.c_int),
    'ntg_input_fs': ([_P, _P, _P, _I64, _I64, _I64, _I64, _I64, _I32, _P], C.c_int),
    'ntg_input_ds': ([_P, _P, _P, _I64, _I64, _I64, _I64, _P], C.c_int),
    'ntg_conv_fs': ([_P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, _I32, _I32, _I32, _I32,
                     _I32, _I32, _I64, _I64, _I32, Affine, Act, Var, Var], C.c_int),
    'ntg_conv_act_fs': ([_P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, Affine, Act, Var,
                         Var], C.c_int),
    'ntg_conv_input_fs': ([_P, _P, _P, _I64, _I64, _I64, _I64, _I64, _P, _P, Affine, Act, Var,
                           Var], C.c_int),
    'ntg_conv_ds': ([_P, _P, _P, _P, _P, _I64, _I64, _I64, _I32, _I32, _I32, _I32, _I32, _I32,
                     _I64, _I64, _I32, Affine], C.c_int),
    'ntg_affine_act': ([_P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, _I32, _I32, Affine, Act,
                        Var, Var], C.c_int),
    'ntg_max_abs': ([_P, _P, _I64, _P], C.c_int),
    'ntg_pool': ([_P, _P, _P, _I64, _I64, _I64, _I32, _I32, _I32, _I32, _I32, _I32, _I64, _I64,
                  _I32, _I32, _I32, _I32], C.c_int),
    'ntg_global_pool': ([_P, _P, _P, _I64, _I64, _I32, _F], C.c_int),
    'ntg_flatten_fs': ([_P, _P, _P, _I64, _I64, _I64], C.c_int),
    'ntg_chain_fwd': ([_P, C.POINTER(Chain), _P, _P, _I64, _I64, _I64, _I64, _P, _P, _P, _P,
                       _I64], C.c_int),
    'ntg_chain_fwd_sym': ([_P, C.POINTER(Chain), _P, _I64, _I64, _I64, _I64, _P, _P, _P, _I64],
                          C.c_int),
    'ntg_act_bwd': ([_P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, _I32, Act, Var, Var, _P,
                     _P], C.c_int),
    'ntg_act_pool_bwd': ([_P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, Act, Var, Var, _P,
                          _P], C.c_int),
    'ntg_conv_act_pool_fs': ([_P, _P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, Affine, Act,
                             Var, Var], C.c_int),
    'ntg_input_conv_act_fs': ([_P, _P, _P, _I64, _I64, _I64, _P, _P, _P, Affine, Act, Var, Var],
                              C.c_int),
    'ntg_conv_act_bwd': ([_P, _P, _P, _P, _P, _I32, _P, _P, _I64, _I64, _I64, _F, Act, Var, Var,
                          _P, _P], C.c_int),
    'ntg_affine_bwd': ([_P, _P, _P, _P, _P, _I64, Affine, _F], C.c_int),
    'ntg_affine_hyper_bwd': ([_P, _P, _P, _P, _P, _I64, _F, _F, _P], C.c_int),
    'ntg_stencil_bwd': ([_P, _P, _P, _I64, _I64, _I64, _I32, _I32, _I32, _I32, _I32, _I32, _I64,
                         _I64, _I32, _I32], C.c_int),
    'ntg_pool_bwd': ([_P, _P, _P, _I64, _I64, _I64, _I32, _I32, _I32, _I32, _I32, _I32, _I64,
                      _I64, _I32, _I32, _I32, _I32], C.c_int),
    'ntg_readout_bwd': ([_P, _P, _P, _I64, _I64, _I64, _I32, _I64, _F], C.c_int),
    'ntg_input_fs_bwd': ([_P, _P, _P, _P, _I64, _I64, _I64, _I64, _I64, _I64, _I32], C.c_int),
    'ntg_input_fs_bwd2': ([_P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, _I64], C.c_int),
    'ntg_input_ds_bwd': ([_P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _I64], C.c_int),
    'ntg_gemm_ex': ([_P, _P, _P, _P, _I64, _I64, _I64, _I32, _F, _I32], C.c_int),
    'ntg_cov_diag_bwd': ([_P, _P, _P, _P, _I64, _I64], C.c_int),
    'ntg_diag_add': ([_P, _P, _P, _I64, _I64, _I64, _I64, _I64, _I64], C.c_int),
    'ntg_chol_factor': ([_P, _P, _I64, C.c_double, _I32, _P, _P, _P], C.c_int),
    'ntg_chol_logdet': ([_P, _P, _I64, _P], C.c_int),
    'ntg_nll_grad': ([_P, _P, _P, _I64, _I64, _F, C.c_double, _P, _P], C.c_int),
    'ntg_chol_workspace_bytes': ([_I64, _I64], C.c_size_t),
    'ntg_chol_solve': ([_P, _P, _P, _P, _I64, _P, _I64, _P, _I32, _P, C.c_size_t, _P], C.c_int),
    'ntg_chol_solve_noalloc': ([_P, _P, _P, _P, _I64, _P, _I64, _P, _I32, _P], C.c_int),
    'ntg_gemm_tc': ([_P, _P, _I64, _P, _I64, _P, _I64, _I64, _I64, _I64, _F, _F, _I32], C.c_int),
    'ntg_chol_factor_tc_workspace_bytes': ([_I64, _I64], C.c_size_t),
    'ntg_chol_factor_tc': ([_P, _P, _I64, C.c_double, _I32, _P, _I64, _P, _P, _P, C.c_size_t],
                           C.c_int),
    'ntg_chol_solve_tc_workspace_bytes': ([_I64, _I64, _I64], C.c_size_t),
    'ntg_chol_solve_tc': ([_P, _P, _P, _I64, _P, _P, _I64, _P, _I64, _P, _I32, _P, C.c_size_t,
                           _P, _P, _P], C.c_int),
    'ntg_gemm_df_workspace_bytes': ([_I64, _I64, _I64], C.c_size_t),
    'ntg_gemm_df': ([_P, _P, _I64, _I64, _I64, _P, _I64, _P, _P, _P, _P, C.c_size_t], C.c_int),
    'ntg_chol_logdet_tc': ([_P, _P, _I64, _I64, _P], C.c_int),
    'ntg_eigh_workspace_bytes': ([_I64], C.c_size_t),
    'ntg_eigh': ([_P, _P, _I64, C.c_double, _P, _P, _I32, C.c_double, _I32, _P, C.c_size_t,
                  _P], C.c_int),
    'ntg_spectral_scale': ([_P, _P, _P, _I64, _I32, C.c_double, _P, _I64, _I64, _P], C.c_int),
}

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Loads the library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            from . import _build
            _build.build()
        lib = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                raise RuntimeError(f'{LIB_PATH} does not export {name}')
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


class NtgError(RuntimeError):
    pass


_pinned = threading.local()


def _keep(t) -> None:
    lst = getattr(_pinned, 'tensors', None)
    if lst is None:
        lst = _pinned.tensors = []
    lst.append(t)


def call(name: str, *args) -> None:
    """Calls an entry point; raises NtgError with the library message on failure.

    Tensors whose pointers were taken by ptr() since the previous call stay
    referenced until this call has enqueued its work: a temporary such as
    ptr(x.contiguous()) would otherwise return its memory to the caching
    allocator before the kernel that reads it is launched, and the next
    temporary of the same argument list could take over that block."""
    lib = load()
    try:
        rc = getattr(lib, name)(*args)
    finally:
        _pinned.tensors = []
    if rc != 0:
        msg = lib.ntg_last_error().decode()
        raise NtgError(f'{name} failed ({ERRORS.get(rc, rc)}): {msg}')


_depth = threading.local()


def check_device(where: str) -> None:
    """Raises NtgError when a bounded wait of a device kernel ran out since the last check.

    The streamed, adjoint and tensor-core kernels bound every pipeline wait; one that runs
    out sets a device error word and the kernel winds down with its results incomplete.
    The current stream is synchronised first, so that every kernel it carries has finished,
    then ntg_device_status reads and clears the words (one 4-byte read per word)."""
    if not torch.cuda.is_available():
        return  # nothing of this library can have run
    torch.cuda.current_stream().synchronize()
    lib = load()
    rc = lib.ntg_device_status()
    if rc != 0:
        raise NtgError(f'{where}: {ERRORS.get(rc, rc)}: {lib.ntg_last_error().decode()}')


@contextlib.contextmanager
def boundary(where: str):
    """A public call of the package: on its normal exit, and only at the outermost level
    (calls nest, e.g. nt.batch calls kernel_fn per tile), the device error words are
    checked with check_device."""
    d = getattr(_depth, 'n', 0)
    _depth.n = d + 1
    try:
        yield
    finally:
        _depth.n = d
    if d == 0:
        check_device(where)


def launch_count() -> int:
    return int(load().ntg_launch_count())


def stream() -> int:
    """The current torch CUDA stream as a raw cudaStream_t value."""
    return torch.cuda.current_stream().cuda_stream


def ptr(t) -> int | None:
    if t is None:
        return None
    if not t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
        raise ValueError('nt_gb300 kernels take contiguous float32 CUDA tensors')
    _keep(t)
    return t.data_ptr()


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError('nt_gb300 needs a CUDA device (sm_103a); there is no CPU fallback')
    return torch.device('cuda', torch.cuda.current_device())
