"""The serving loop's further-step policy (csrc/launch_plan.hpp), compiled on
the host with g++: light launches stay one step per scene, heavy launches give
further steps to the deepest queues level by level within the caps."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "novaphy_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "launch_plan.hpp"
int main() {
    long long cap, min_step;
    int max_steps, n;
    if (std::scanf("%lld %lld %d %d", &cap, &min_step, &max_steps, &n) != 4) return 2;
    std::vector<pbf_plan::PlanItem> items((size_t)n);
    for (auto& it : items)
        if (std::scanf("%lld %d %lld", &it.n, &it.avail, &it.depth) != 3) return 3;
    for (int s : pbf_plan::plan_steps(items, cap, min_step, max_steps)) std::printf("%d ", s);
    std::printf("\n");
    return 0;
}
"""

M = 1 << 20


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("plan")
    (d / "p.cpp").write_text(PROGRAM)
    exe = str(d / "p")
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{CSRC}", str(d / "p.cpp"), "-o", exe],
                   check=True)

    def run(items, cap=16 * M, min_step=M, max_steps=16):
        inp = f"{cap} {min_step} {max_steps} {len(items)}\n" + "".join(
            f"{n} {a} {dp}\n" for n, a, dp in items)
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True)
        return [int(t) for t in out.stdout.split()]

    return run


def test_light_launch_stays_one_step_per_scene(plan):
    assert plan([(20_000, 15, 15)]) == [1]
    assert plan([(20_000, 15, 15), (50_000, 3, 3)]) == [1, 1]
    assert plan([]) == []


def test_without_a_minimum_a_launch_at_most_doubles(plan):
    # extra work <= the launch's own particles
    assert plan([(20_000, 15, 15)], min_step=0) == [2]
    assert plan([(20_000, 15, 15), (20_000, 0, 0)], min_step=0) == [3, 1]


def test_heavy_launch_gives_the_deepest_queues_further_steps(plan):
    items = [(M, 8, 8 - k) for k in range(6)] + [(M, 0, 0)] * 4  # 10M particles
    # cap 16M: 6M more; level 1 takes all six (6M >= 2.5M); level 2 no longer fits
    assert plan(items) == [2] * 6 + [1] * 4
    # a tighter cap keeps the deepest first
    assert plan(items, cap=13 * M) == [2, 2, 2, 1, 1, 1] + [1] * 4


def test_a_small_level_is_not_added(plan):
    items = [(M, 8, 8), (M, 8, 7)] + [(M, 0, 0)] * 8  # level 1 would hold 2M < 2.5M
    assert plan(items) == [1] * 10


def test_levels_respect_availability_and_max_steps(plan):
    # 4M particles: extra cap 8M (twice), level minimum 1M; item 0 has one
    # further step available, item 1 many: levels 2 and 3 hold item 1 alone
    items = [(M, 1, 9), (M, 9, 9), (2 * M, 0, 0)]
    assert plan(items) == [2, 4, 1]
    assert plan([(M, 30, 30)], min_step=0, max_steps=4) == [2]
    assert plan([(M, 30, 30)], min_step=0, cap=64 * M, max_steps=4) == [2]
    many = [(M, 30, 30), (M, 30, 30), (M, 30, 30), (M, 30, 30)]
    assert plan(many, min_step=0, max_steps=4) == [2, 2, 2, 2]
