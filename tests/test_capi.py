"""CPU tests of the C ABI: the library loads and exports every entry point
declared in include/qfgpu.h; statuses are reported, not aborts."""
import ctypes
import os
import re

import pytest

from quickfoil_gb300 import _capi as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(qfg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("qfg_evaluate_group", "qfg_evaluate_step", "qfg_evaluate_per_literal",
                 "qfg_radix_partition", "qfg_build_hash_table_on_partitions",
                 "qfg_left_semijoin", "qfg_right_semijoin", "qfg_extend_bindings"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = C.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    bound = {s[0] for s in C.SIGNATURES}
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_status_strings():
    lib = C.load()
    assert lib.qfg_version() >= 1
    assert lib.qfg_status_string(C.QFG_OK) == b"ok"
    assert lib.qfg_status_string(C.QFG_ERR_BUDGET) == b"HBM budget exceeded"
    assert lib.qfg_status_string(12345) == b"unknown status"


def test_null_arguments_are_rejected_without_a_device():
    lib = C.load()
    assert lib.qfg_ctx_destroy(None) == C.QFG_ERR_INVALID
    assert lib.qfg_evaluate_step(None, None, 0, None, None, 0) == C.QFG_ERR_INVALID
    assert lib.qfg_radix_partition(None, None, 0, 5, None, None) == C.QFG_ERR_INVALID
    assert lib.qfg_ctx_create(0, 0, None) == C.QFG_ERR_INVALID


def test_context_creation_fails_cleanly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = C.load()
    h = ctypes.c_void_p()
    assert lib.qfg_ctx_create(0, 0, ctypes.byref(h)) == C.QFG_ERR_CUDA
    assert not h.value


def test_misaligned_partition_tuples_are_rejected_without_a_device():
    """A PartitionTuple is stored as one 8-byte word, so an output array that
    is only 4-byte aligned is refused with a status before any device work.
    Run only where no GPU is present: the addresses are never dereferenced,
    because the arguments are checked first."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = C.load()
    err = ctypes.create_string_buffer(128)
    rc = lib.qfg_radix_partition_static(None, 0x10000, 10, 5, 0x20004, 0x30000, err, len(err))
    assert rc == C.QFG_ERR_INVALID
    assert b"8-byte aligned" in err.value


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c++", "c++17")])
def test_header_compiles_cleanly_for_c_and_cpp_callers(tmp_path, lang, std):
    """include/qfgpu.h is the boundary a C (cgo, ctypes, JNI glue) or C++
    caller includes: it must compile on its own without warnings."""
    import shutil
    import subprocess
    cc = "gcc" if lang == "c" else "g++"
    if shutil.which(cc) is None:
        pytest.skip(f"{cc} not installed")
    src = tmp_path / "use_header.c"
    src.write_text('#include "qfgpu.h"\nint main(void) { return qfg_version() > 0 ? 0 : 1; }\n')
    r = subprocess.run([cc, "-x", lang, f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I", os.path.join(ROOT, "include"), "-c", str(src), "-o",
                        str(tmp_path / "use_header.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
