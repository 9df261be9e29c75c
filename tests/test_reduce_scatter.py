"""The trimmed warp reduce-scatter of csrc/bsfit_device.cuh (reduce_scatter,
RsSources) on the CPU: a float32 model of the 32 lanes shows that every value's
total equals the padded 32-wide butterfly's bit for bit (the property the 3D and
4D fits rely on to keep their results unchanged), and the source table the
kernels gather from, evaluated by nvcc on the host, matches the model's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "gpu-based-b-spline-fitter_gb300", "csrc")
LEVELS = (16, 8, 4, 2, 1)


def butterfly32(parts):
    """Padded form: 32 values, lane t ends with the total of value t."""
    v = parts.copy()
    for o in LEVELS:
        nv = v.copy()
        for lane in range(32):
            p = lane ^ o
            for i in range(o):
                keep = v[lane, i + o] if lane & o else v[lane, i]
                recv = v[p, i] if p & o else v[p, i + o]
                nv[lane, i] = np.float32(keep + recv)
        v = nv
    return v[:, 0]


def trimmed(parts, c):
    """Trimmed form: returns per-lane slot values and slot -> value maps."""
    v = parts.copy()
    maps = [list(range(c)) for _ in range(32)]
    for o in LEVELS:
        half = c // 2
        nv = v.copy()
        for lane in range(32):
            p = lane ^ o
            up, pup = bool(lane & o), bool(p & o)
            for i in range(half):
                keep = v[lane, i + half] if up else v[lane, i]
                recv = v[p, i] if pup else v[p, i + half]
                nv[lane, i] = np.float32(keep + recv)
            if c & 1:
                nv[lane, half] = np.float32(v[lane, 2 * half] + v[p, 2 * half])
            m = [maps[lane][i + (half if up else 0)] for i in range(half)]
            if c & 1:
                m.append(maps[lane][2 * half])
            maps[lane] = m
        c = half + (c & 1)
        v = nv
    return v[:, :c], maps


def sources(c):
    _, maps = trimmed(np.zeros((32, 64), np.float32), c)
    src = [-1] * c
    for lane in range(32):
        for slot, x in enumerate(maps[lane]):
            if src[x] < 0:
                src[x] = 2 * lane + slot
    return src


@pytest.mark.parametrize("c", [20, 27, 44, 1, 5, 32, 33, 64])
def test_trimmed_totals_bit_identical_to_padded(c):
    rng = np.random.default_rng(c)
    parts = (rng.standard_normal((32, 64)) * 10.0 ** rng.uniform(-4, 4, (32, 64))).astype(np.float32)
    parts[:, c:] = 0.0
    ref = np.concatenate([butterfly32(parts[:, h:h + 32]) for h in range(0, 64, 32)])
    vals, maps = trimmed(parts, c)
    held = set()
    for lane in range(32):
        for slot, x in enumerate(maps[lane]):
            held.add(x)
            assert vals[lane, slot].tobytes() == ref[x].tobytes(), (c, lane, slot, x)
    assert held == set(range(c))


def test_source_table_matches_the_model(tmp_path):
    if not shutil.which("nvcc"):
        pytest.skip("no nvcc")
    counts = (20, 27, 44, 32, 64)
    body = "\n".join(
        f"  {{ constexpr bsfit::RsSources<{c}> t{{}}; printf(\"%d\", bsfit::rs_slots({c}));"
        f" for (int x = 0; x < {c}; ++x) printf(\" %d\", t.src[x]); printf(\"\\n\"); }}"
        for c in counts)
    src = f"""#include <cstdio>
#include "bsfit_device.cuh"
int main() {{
{body}
  return 0;
}}
"""
    cu = tmp_path / "rs.cu"
    cu.write_text(src)
    exe = tmp_path / "rs"
    r = subprocess.run(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", CSRC, str(cu), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    # printing only: the table is evaluated at compile time, no GPU is touched
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for c, line in zip(counts, out):
        got = [int(x) for x in line.split()]
        _, maps = trimmed(np.zeros((32, 64), np.float32), c)
        assert got[0] == len(maps[0]), (c, got[0])
        assert got[1:] == sources(c), c
