"""The C ABI library loads and exports every symbol include/gbpc.h declares (no GPU)."""

import ctypes
import re

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "gbpc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbpc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("gbpc_fsai_setup", "gbpc_fsai_pack", "gbpc_csr_transpose",
                     "gbpc_op_fsai", "gbpc_op_sqlap", "gbpc_op_block_jacobi", "gbpc_op_bilu0",
                     "gbpc_krylov", "gbpc_op_apply"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from warp_preconditioners_gb300 import _build

    lib = ctypes.CDLL(str(_build.build()))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.gbpc_version.restype = ctypes.c_int
    assert lib.gbpc_version() == 1
    lib.gbpc_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.gbpc_last_error(), bytes)


def test_argument_errors_need_no_gpu():
    # Validation happens before any device work, with the reference's wording.
    from warp_preconditioners_gb300 import _lib

    lib = _lib.load()
    status = (ctypes.c_int32 * 3)()
    dummy = ctypes.c_void_p(8)  # never dereferenced: validation fails first
    rc = lib.gbpc_fsai_setup(4, dummy, dummy, dummy, 0, 65, 1, 1e-3, 1e-12, dummy, dummy, dummy,
                             dummy, status, None)
    assert rc == _lib.ERR_ARG
    assert "max_row_size" in _lib.last_error()
    rc = lib.gbpc_fsai_setup(4, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), 0, 8,
                             0, 1e-3, 1e-12, ctypes.c_void_p(8), ctypes.c_void_p(8),
                             ctypes.c_void_p(8), ctypes.c_void_p(8), status, None)
    assert rc == _lib.ERR_ARG and "max_step_size" in _lib.last_error()
