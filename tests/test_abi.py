"""The C-ABI library loads and exports every entry point include/nt_gb300.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'nt_gb300.h')
LIB = os.path.join(ROOT, 'neural-tangents_gb300', 'libntgb300.so')


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(ntg_[a-z0-9_]+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib():
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            'ntg_build', os.path.join(ROOT, 'neural-tangents_gb300', '_build.py'))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert 'ntg_chain_fwd' in syms and 'ntg_conv_fs' in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_channel(lib):
    lib.ntg_version.restype = ctypes.c_char_p
    assert b'sm_103a' in lib.ntg_version()
    lib.ntg_last_error.restype = ctypes.c_char_p
    lib.ntg_gram.restype = ctypes.c_int
    # invalid arguments are rejected on the host before any CUDA call
    rc = lib.ntg_gram(None, None, None, ctypes.c_int64(1), ctypes.c_int64(1), ctypes.c_int64(1),
                      None, 0, None, ctypes.c_size_t(0))
    assert rc == 1
    assert b'null pointer' in lib.ntg_last_error()


def test_python_binding_signatures_cover_header():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        'ntg_lib', os.path.join(ROOT, 'neural-tangents_gb300', '_lib.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    missing = [s for s in declared_symbols() if s not in mod.SIGNATURES]
    assert not missing, missing


def test_tuning_knobs_are_checked(lib):
    lib.ntg_tune_get.restype = ctypes.c_int32
    lib.ntg_tune_set.restype = ctypes.c_int
    assert lib.ntg_tune_get(0) == 4            # stencil ring default
    assert lib.ntg_tune_get(99) == -1
    assert lib.ntg_tune_set(0, 5) == 1         # not a supported ring depth
    assert lib.ntg_tune_set(7, 1) == 1         # unknown knob
    assert lib.ntg_tune_set(0, 6) == 0 and lib.ntg_tune_get(0) == 6
    assert lib.ntg_tune_set(0, 4) == 0 and lib.ntg_tune_get(0) == 4


def test_argument_checks_before_any_launch(lib):
    """Host-side validation of the C ABI rejects bad sizes and layouts with an error code and
    message, without touching a device (the pointers below are never dereferenced)."""
    lib.ntg_last_error.restype = ctypes.c_char_p
    i64 = ctypes.c_int64
    fake = ctypes.c_void_p(256)
    # ntg_conv_fs: empty batch
    lib.ntg_conv_fs.restype = ctypes.c_int
    assert lib.ntg_chol_workspace_bytes(i64(10), i64(3)) >= 10 * 3 * 12
    rc = lib.ntg_pool_bwd(None, fake, fake, i64(0), i64(4), i64(4), 2, 2, 2, 2, 0, 0, i64(2),
                          i64(2), 0, 0, 1, 0)
    assert rc == 1 and b'bad arguments' in lib.ntg_last_error()
    rc = lib.ntg_input_fs_bwd2(None, fake, fake, None, fake, None, i64(2), i64(3), i64(4),
                               i64(4), i64(3))
    assert rc == 1 and b'pairs need x2' in lib.ntg_last_error()
    rc = lib.ntg_chol_solve(None, fake, fake, fake, i64(4), fake, i64(2), fake, 17, None,
                            ctypes.c_size_t(0), None)
    assert rc == 1 and b'refinement' in lib.ntg_last_error()


def test_tensor_core_solver_entries_check_arguments(lib):
    """The tensor-core Cholesky, its solve, the double-float product and the eigensolver reject
    bad sizes, pointers and workspaces with an error code and message before any launch."""
    lib.ntg_last_error.restype = ctypes.c_char_p
    i64, sz = ctypes.c_int64, ctypes.c_size_t
    fake = ctypes.c_void_p(256)
    for fn in ('ntg_gemm_df_workspace_bytes', 'ntg_chol_factor_tc_workspace_bytes',
               'ntg_chol_solve_tc_workspace_bytes', 'ntg_eigh_workspace_bytes'):
        getattr(lib, fn).restype = ctypes.c_size_t
    size_max = ctypes.c_size_t(-1).value
    assert lib.ntg_gemm_df_workspace_bytes(i64(0), i64(5), i64(3)) == size_max
    assert lib.ntg_gemm_df_workspace_bytes(i64(7), i64(5), i64(3)) > 5 * 3 * 8
    assert lib.ntg_chol_factor_tc_workspace_bytes(i64(100), i64(99)) == size_max  # ldl < n
    # ntg_gemm_df: no output at all, then a workspace too small for rows x n x m
    rc = lib.ntg_gemm_df(None, fake, i64(8), i64(4), i64(8), fake, i64(2), None, None, None,
                         fake, sz(1 << 20))
    assert rc == 1 and b'null pointer' in lib.ntg_last_error()
    rc = lib.ntg_gemm_df(None, fake, i64(8), i64(4), i64(8), fake, i64(2), None, fake, None,
                         fake, sz(16))
    assert rc == 1 and b'workspace' in lib.ntg_last_error()
    # ntg_chol_factor_tc: ldl not a multiple of 4
    rc = lib.ntg_chol_factor_tc(None, fake, i64(10), ctypes.c_double(1e-4), 0, fake, i64(11),
                                fake, fake, fake, sz(1 << 30))
    assert rc == 1 and b'ldl' in lib.ntg_last_error()
    # ntg_chol_solve_tc: refinement steps out of range
    rc = lib.ntg_chol_solve_tc(None, fake, fake, i64(12), fake, fake, i64(10), fake, i64(2), fake,
                               65, fake, sz(1 << 30), None, None, None)
    assert rc == 1 and b'refinement' in lib.ntg_last_error()
    # ntg_eigh: sweeps out of range
    rc = lib.ntg_eigh(None, fake, i64(10), ctypes.c_double(0.), fake, fake, 0,
                      ctypes.c_double(1e-5), 2, fake, sz(1 << 30), None)
    assert rc == 1 and b'max_sweeps' in lib.ntg_last_error()
