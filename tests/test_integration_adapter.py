"""The Jolt-side adapter (include/jsb_jolt_adapter.h, described in INTEGRATION.md) compiles against the
reference's own headers and the C ABI (include/jsb.h). Runs where the reference sources are available
(oracle/_ref/ref_dir.txt, written by oracle/Makefile.ref, or JSB_REFERENCE_DIR); skipped elsewhere."""
import os
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def reference_dir():
    d = os.environ.get("JSB_REFERENCE_DIR")
    marker = os.path.join(REPO, "oracle", "_ref", "ref_dir.txt")
    if not d and os.path.exists(marker):
        d = open(marker).read().strip()
    return d if d and os.path.exists(os.path.join(d, "Jolt", "Jolt.h")) else None


def test_adapter_compiles_against_the_reference():
    ref = reference_dir()
    if ref is None:
        pytest.skip("the reference's sources are not available here")
    src = '#include "jsb_jolt_adapter.h"\n' \
          "void use(jsb_jolt::GpuSoftBodyStepper &s, JPH::PhysicsSystem &p) { s.Step(p, 1.0f / 60.0f, 1, nullptr); }\n"
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "adapter.cpp")
        open(path, "w").write(src)
        cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-Wno-unused-function", f"-I{ref}",
               f"-I{os.path.join(REPO, 'include')}", path]
        res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
