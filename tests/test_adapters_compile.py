"""The C++ adapters of include/nlgpu_reference_adapters.hpp (the GPU ILLT behind
the reference's preconditioner_base plug-in point, the whole CG in one call)
compile against the reference's own solver headers and the Eigen API shim and
link against libnlgpu.so (oracle/check_adapters.sh; skipped where the
reference sources are absent, as on the GPU machines)."""
import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_reference_adapters_compile_and_link():
    from nonlocal_gb300 import build
    build.build()
    r = subprocess.run(["bash", str(ROOT / "oracle" / "check_adapters.sh")], capture_output=True, text=True,
                       timeout=600)
    if r.returncode == 2:
        pytest.skip("reference sources not present")
    assert r.returncode == 0, r.stdout + r.stderr
