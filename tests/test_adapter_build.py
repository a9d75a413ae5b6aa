"""The ForceCalculationMethod adapter compiles against the reference's own
headers and links with the reference objects and libsolveit_gpu.so (only
where the reference tree is available; running it needs a GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("SOLVEIT_REFERENCE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(REFERENCE), reason="reference tree not present")
def test_adapter_builds_against_reference_headers():
    lib = os.path.join(ROOT, "solveit-code_gb300", "_build", "libsolveit_gpu.so")
    if not os.path.exists(lib):
        pytest.skip("libsolveit_gpu.so not built")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "adapter", f"REF={REFERENCE}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "stock", "adapter_check"))
