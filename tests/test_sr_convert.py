"""The bf16 write-back rounds with the hardware stochastic-rounding convert
(cvt.rs.satfinite.bf16x2.f32).  It must equal the software rule the library documents --
bf16 bits = (fp32 bits + 16 random bits) >> 16, upper element with the high random half --
so that bf16 results do not depend on which form computed them."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.gpu
def test_hardware_sr_equals_software_rule(ng, gpu_ok, tmp_path):
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    exe = str(tmp_path / "sr_check")
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O2", "-o", exe,
                    os.path.join(HERE, "sr_convert_check.cu")], check=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 of" in r.stdout
