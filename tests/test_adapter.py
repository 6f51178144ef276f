"""The C++ drop-in adapter (quickfoil_gb300/adapter) compiles against the
reference's own headers and links with the reference's learner objects in
place of learner/CandidateLiteralEvaluator.cpp, with libqfgpu resolving every
C ABI call (no undefined symbol).  A renamed accessor of FoilClause /
FoilLiteral / TableView, a wrong CandidateLiteralInfo field or a changed C ABI
signature fails here.  Runs where the reference sources and its objects
(oracle/build_ref.sh) are present; skipped elsewhere."""
import glob
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "quickfoil_gb300", "adapter")
SOURCES = ["qfgpu_adapter.cpp", "CandidateLiteralEvaluator_gpu.cpp"]


def _reference_dir():
    res = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), "--where"],
                         capture_output=True, text=True)
    return res.stdout.strip() if res.returncode == 0 else None


def _flags(ref):
    return ["-std=c++14", "-I", os.path.join(ROOT, "oracle", "shims"), "-I", ref,
            "-I", os.path.join(ROOT, "include"), "-I", ADAPTER]


def test_adapter_compiles_against_reference_headers():
    ref = _reference_dir()
    if ref is None:
        pytest.skip("reference sources absent")
    for src in SOURCES:
        res = subprocess.run(["g++", "-fsyntax-only", "-Wall", *_flags(ref), os.path.join(ADAPTER, src)],
                             capture_output=True, text=True)
        assert res.returncode == 0, res.stderr


def test_adapter_links_with_the_reference_learner_and_libqfgpu():
    ref = _reference_dir()
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
            if not any(x in o for x in ("learner_CandidateLiteralEvaluator", "ref_driver",
                                        "ref_loader"))]
    lib = os.path.join(ROOT, "quickfoil_gb300", "_lib", "libqfgpu.so")
    if ref is None or not objs or not os.path.exists(lib):
        pytest.skip("reference objects or libqfgpu absent")
    assert any("learner_QuickFoil.o" in o for o in objs)
    with tempfile.TemporaryDirectory() as d:
        mine = []
        for src in SOURCES:
            out = os.path.join(d, src + ".o")
            res = subprocess.run(["g++", "-O1", "-fPIC", "-w", *_flags(ref), "-c",
                                  os.path.join(ADAPTER, src), "-o", out], capture_output=True,
                                 text=True)
            assert res.returncode == 0, res.stderr
            mine.append(out)
        so = os.path.join(d, "liblearner_gpu.so")
        res = subprocess.run(["g++", "-shared", "-o", so, *mine, *objs, "-L", os.path.dirname(lib),
                              "-lqfgpu", "-Wl,--no-undefined"], capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        syms = subprocess.run(["nm", "-D", so], capture_output=True, text=True).stdout
        for name in ("qfg_evaluate_group", "qfg_coverage", "qfg_bindings_create"):
            assert f" U {name}" in syms
        # The learner's Evaluate now comes from the adapter.
        assert "CandidateLiteralEvaluator8Evaluate" in subprocess.run(
            ["nm", mine[1]], capture_output=True, text=True).stdout
