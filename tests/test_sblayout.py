"""CPU: the complex64 Green copy's sub-block layout (egx_sblayout.cuh),
compiled for the host by the system C++ compiler.

* every stored entry is reached and the repack's inverse names the packed
  complex128 entry of the same (row, col) (bijective up to the symmetric
  blocks' shared entries), for nz in {16, 32, 48};
* the pair rule the FP16 contraction kernels load by (neighbour at ^1, or ^4
  in transposed sub-blocks);
* the checkerboard keeps those kernels' A-fragment loads within 15 % of
  the conflict-free shared-memory wavefront count (4.6 % at nz = 48, where
  the diagonal tiles that mix in-place and transposed reads are fewest;
  twice the count without the swizzle).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "extreme_gb300", "csrc")


@pytest.fixture(scope="module")
def layout_lines(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("sblayout") / "sblayout_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, "-o", exe, os.path.join(HERE, "sblayout_check.cpp")],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    rows = {}
    for line in out.strip().splitlines():
        f = line.split()
        rows[int(f[1])] = {f[k]: int(f[k + 1]) for k in range(2, len(f), 2)}
    return rows


@pytest.mark.parametrize("nz", [16, 32, 48])
def test_layout_is_consistent(layout_lines, nz):
    row = layout_lines[nz]
    nb = nz // 4
    assert row["entries"] == 4 * nb * (nb + 1) // 2 * 16 + 2 * nb * nb * 16
    assert row["errors"] == 0


@pytest.mark.parametrize("nz", [16, 32, 48])
def test_fragment_loads_nearly_conflict_free(layout_lines, nz):
    row = layout_lines[nz]
    assert row["wavefronts"] <= 1.15 * row["ideal"], row
