"""The output mapping of the continuation rows (row_slots in kernels.h),
checked on the host: whatever the number of branches per solved centre, the
initial solve and the continuation rows write every slot (branch, column) of
the reference's output layout exactly once.

With seg = 1 (every centre solved, the reference's scheme) row (c, 1) ends in
column 2 half of branch c and row (c + 1, 0) in column 0 of branch c + 1;
with seg > 1 a row from a solved centre crosses branch boundaries and writes
both slots of a boundary phase itself."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "kernels.h"
#include <cstdio>
#include <vector>
int main()
{
    const int cases[][3] = {{1, 50, 1}, {8, 32, 1}, {8, 32, 2}, {8, 32, 4}, {8, 32, 8}, {6, 5, 3}, {6, 5, 2},
                            {128, 40, 32}, {128, 40, 64}, {12, 1, 4}, {3, 7, 3}, {2, 1, 2}};
    int bad = 0;
    for (auto& t : cases)
    {
        const int nb = t[0], half = t[1], seg = t[2];
        const int cols = 2 * half + 1;
        std::vector<int> cnt(nb * cols, 0);
        for (int q = 0; q < nb / seg; q++)
        {
            const int c = q * seg;
            cnt[c * cols + half]++;                       /* the initial solve */
            for (int side = 0; side < 2; side++)
            {
                const int steps = seg == 1 ? half : (side ? seg * half : seg * half - 1);
                for (int j = 1; j <= steps; j++)
                {
                    int b[2], k[2];
                    const int n = ccf::row_slots(nb, half, seg, c, side, j, b, k);
                    for (int m = 0; m < n; m++) cnt[b[m] * cols + k[m]]++;
                }
            }
        }
        for (int i = 0; i < nb * cols; i++)
            if (cnt[i] != 1)
            {
                std::printf("nb %d half %d seg %d: branch %d column %d written %d times\n", nb, half, seg, i / cols,
                    i % cols, cnt[i]);
                bad++;
            }
    }
    std::printf("bad %d\n", bad);
    return bad != 0;
}
"""


def test_every_output_slot_is_written_once(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "slots.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "slots"
    r = subprocess.run([nvcc, "-std=c++20", "-I", os.path.join(ROOT, "ccf_gb300", "csrc"), "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("bad 0")
