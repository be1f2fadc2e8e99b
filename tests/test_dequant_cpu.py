"""The traversal kernels form each child bound as one fused multiply-add,
fmaf(q, 2^(e-8), Origin), where the reference adds an exact ldexpf(q, e-8) to
Origin (vulkan_acceleration_structure_util.h:499-508).  dequant_fma.c checks
that the two agree bit for bit over every 8-bit q and int8 exponent e and a
spread of origins, with the host's IEEE fmaf (the device's FFMA rounds the
same way)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fused_child_bound_equals_reference_add(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "dequant_fma")
    subprocess.run([cc, "-O2", "-ffp-contract=off", os.path.join(HERE, "dequant_fma.c"), "-o", exe, "-lm"],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout
