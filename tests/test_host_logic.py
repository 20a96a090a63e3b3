"""Host-side logic checked on the CPU: the chunk plan of the pipelined host-buffer path
(csrc/rt_chunks.hpp, compiled here with g++), and the committed ncu summaries that bench.py
reads its per-launch DRAM traffic and launch counts from."""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHUNK = 1 << 21

_PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include "rt_chunks.hpp"
int main(int argc, char **argv) {
    for (int a = 1; a < argc; ++a) {
        const size_t n = strtoull(argv[a], nullptr, 10);
        const std::vector<size_t> v = rgb::chunk_plan(n, size_t(1) << 21);
        printf("%zu", n);
        for (size_t c : v) printf(" %zu", c);
        printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def plan_tool(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("chunks")
    src, exe = d / "plan.cpp", d / "plan"
    src.write_text(_PROGRAM)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "rendu_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)

    def plans(ns):
        out = subprocess.run([str(exe)] + [str(n) for n in ns], check=True, capture_output=True, text=True).stdout
        res = {}
        for line in out.strip().splitlines():
            v = [int(x) for x in line.split()]
            res[v[0]] = v[1:]
        return res

    return plans


def test_chunk_plan_covers_every_record_once(plan_tool):
    tail = [CHUNK // 2, CHUNK // 4, CHUNK // 8]
    ns = [0, 1, 100, CHUNK - 1, CHUNK, CHUNK + 1, 2 * CHUNK, 2 * CHUNK + sum(tail) - 1, 2 * CHUNK + sum(tail),
          (1 << 24) - 12345, 1 << 24, (1 << 24) + 12345, 5 * CHUNK + 7, 100 * CHUNK + 3]
    plans = plan_tool(ns)
    for n in ns:
        v = plans[n]
        assert sum(v) == n, n
        assert all(0 < c <= CHUNK for c in v), n
        if n >= 2 * CHUNK + sum(tail):
            # the last three halve; the others are as equal as the count allows
            assert v[-3:] == tail, n
            mid = v[:-3]
            assert max(mid) - min(mid) <= 1 and len(mid) == -(-(n - sum(tail)) // CHUNK), n
        else:
            # equal chunks but the last
            assert all(c == CHUNK for c in v[:-1]), n
    # the 16M-ray workload: 8 chunks of 1,867,776, then 1M, 512K, 256K
    v = plans[1 << 24]
    assert v == [1867776] * 8 + tail


def test_profiles_carry_the_lines_bench_reads():
    sys.path.insert(0, ROOT)
    import bench

    for name in bench.PT_CONFIGS:
        p = bench._profile_traffic(f"pathtracer_{name}.txt")
        for k in ("trace", "shade"):
            assert p[k]["traffic_bytes_per_launch"] > 0 and p[k]["launches_per_render"] >= 1, (name, k)
    b = bench._profile_traffic("pathtracer_batch_64.txt")
    assert b["trace"]["launches_per_render"] >= 1
    assert bench._profile_traffic("denoiser_conv_1080p.txt")["k_conv_fold"]["traffic_bytes_per_launch"] > 0
    with open(os.path.join(ROOT, "profiles", "raycaster_closest_16M.txt")) as f:
        assert any(ln.startswith("traffic_bytes_per_launch:") for ln in f)
