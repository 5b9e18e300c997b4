"""The batched runners' host-side planning (calcir_gb300/csrc/cir_plan.h), compiled on its own
with the host compiler: chunk lengths against the tridiagonalisation's waves, and the first
part of a chunk's eigensolver batch when it is split over two streams."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER_DIR = os.path.join(os.path.dirname(HERE), "calcir_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include "cir_plan.h"
int main() {
    int K, St, kn, wave, nmat;
    while (std::scanf("%d %d %d %d %d", &K, &St, &kn, &wave, &nmat) == 5)
        std::printf("%d %d\n", cir_plan_chunk(K, St, kn, wave), cir_split_first_part(nmat, wave));
    return 0;
}
"""


@pytest.fixture(scope="module")
def planner():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tempfile.mkdtemp(prefix="cir_plan_")
    src, exe = os.path.join(d, "plan.cpp"), os.path.join(d, "plan")
    with open(src, "w") as f:
        f.write(DRIVER)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", HEADER_DIR, src, "-o", exe], check=True)

    def run(cases):
        inp = "".join(f"{K} {St} {kn} {w} {nm}\n" for K, St, kn, w, nm in cases)
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split()
        return [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(len(cases))]
    yield run
    shutil.rmtree(d, ignore_errors=True)


def test_chunks_avoid_nearly_empty_last_waves(planner):
    (kn_a, _), (kn_b, _), (kn_c, _), (kn_d, _) = planner([
        (200, 32, 101, 456, 0),   # order 1024, 32 origins, memory for 101 steps: 101 + 99 (6400 = 7.09 + 6.95 waves)
        (200, 32, 100, 456, 0),   # 100 + 100 would leave two nearly empty waves: the planner still has 2 chunks
        (250, 10, 250, 456, 0),   # the headline job fits in one chunk
        (200, 32, 40, 456, 0),    # five chunks of 40 steps (1280 = 2.81 waves each)
    ])
    assert kn_a == 101
    assert kn_b == 100
    assert kn_c == 250
    assert kn_d == 40


def test_chunk_length_bounds(planner):
    res = planner([(K, St, km, w, 0) for K, St, km, w in [(7, 3, 1, 456, ), (7, 3, 100, 456), (1, 1, 5, 1), (50, 1000, 3, 456)]])
    assert res[0][0] == 1            # kn_max = 1
    assert res[1][0] == 7            # never more than K
    assert res[2][0] == 1
    assert 1 <= res[3][0] <= 3


def test_split_first_part_is_whole_waves_but_the_last(planner):
    res = planner([(1, 1, 1, 456, 2500), (1, 1, 1, 456, 911), (1, 1, 1, 456, 912), (1, 1, 1, 304, 1250)])
    assert res[0][1] == 1824         # 5 whole waves of 456 in 2500: the first 4 on one stream
    assert res[1][1] == 0            # fewer than two waves: one stream
    assert res[2][1] == 456
    assert res[3][1] == 912          # order 2048, two blocks per SM
