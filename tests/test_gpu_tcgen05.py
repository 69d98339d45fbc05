"""GPU: the tcgen05 measurements behind the contraction's design.

``tests/tcgen05/layout_probe.cu`` checks the tcgen05 operand encodings
(shared-memory descriptors, instruction descriptor, A in shared or tensor
memory, accumulators read back from tensor memory) against a host product
that is exact; ``tests/tcgen05/mma_rate.cu`` measures the issue cost of
kind::tf32 MMAs of M = 128, K = 8 by N and by the number of independent
accumulators. The Green-block contraction has N = 16 (four mirror points x
two sources x real/imaginary parts), and at that width one MMA costs about
46 SM cycles whatever the accumulator count: the contraction stays on the
legacy warp-level MMAs (profiles/tcgen05_mma_rate.md).

Both programs are built here with nvcc for sm_103a.
"""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tcgen05")


def _build_run(tmp_path, name):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / name)
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", exe,
                    os.path.join(HERE, name + ".cu")], check=True)
    return subprocess.run([exe], capture_output=True, text=True, timeout=120)


def test_tcgen05_operand_encodings_are_exact(tmp_path):
    p = _build_run(tmp_path, "layout_probe")
    print(p.stdout)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "max_err_smem_a 0 max_err_tmem_a 0" in p.stdout


def test_tcgen05_mma_issue_cost(tmp_path):
    p = _build_run(tmp_path, "mma_rate")
    print(p.stdout)
    assert p.returncode == 0, p.stdout + p.stderr
    rows = re.findall(r"CH=(\d+) N=\s*(\d+) A=(\w+): no error status 0\s+([\d.]+) cycles/MMA", p.stdout)
    assert len(rows) == 7, p.stdout
    for ch, n, a, cyc in rows:
        assert float(cyc) > 0
