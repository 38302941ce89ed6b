"""The serving loop's fixed-memory latency histogram (csrc/latency_hist.hpp),
compiled on the host with g++: its percentiles match numpy's exact ones to
within a quarter of a percent, over a heavy-tailed sample, zeros, a single
value and a cleared histogram."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "novaphy_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "latency_hist.hpp"
int main() {
    pbf_stats::LatencyHist h;
    int n = 0;
    if (std::scanf("%d", &n) != 1) return 2;
    for (int i = 0; i < n; ++i) {
        double v;
        if (std::scanf("%lf", &v) != 1) return 3;
        h.add(v);
    }
    const double qs[] = {0, 1, 25, 50, 90, 99, 99.9, 100};
    for (double q : qs) std::printf("%.17g\n", h.percentile(q));
    h.clear();
    std::printf("%.17g %llu\n", h.percentile(50), (unsigned long long)h.count());
    return 0;
}
"""
QS = [0, 1, 25, 50, 90, 99, 99.9, 100]


@pytest.fixture(scope="module")
def hist_bin(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("hist")
    src = d / "h.cpp"
    src.write_text(PROGRAM)
    exe = d / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{CSRC}", str(src), "-o", str(exe)], check=True)
    return str(exe)


def run(exe, values):
    inp = f"{len(values)}\n" + "\n".join(repr(float(v)) for v in values) + "\n"
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout
    lines = out.split("\n")
    pcts = [float(t) for t in lines[: len(QS)]]
    cleared = lines[len(QS)].split()
    return pcts, float(cleared[0]), int(cleared[1])


def test_heavy_tailed_sample(hist_bin):
    rng = np.random.default_rng(7)
    v = np.concatenate([rng.lognormal(3.0, 1.5, 20000), rng.uniform(1e4, 3e4, 200)])
    got, cleared, cnt = run(hist_bin, v)
    want = np.percentile(v, QS)
    assert np.allclose(got, want, rtol=2.6e-3, atol=0), (got, want)
    assert got[0] == v.min() and got[-1] == v.max()
    assert cleared == 0.0 and cnt == 0


def test_zeros_and_single_values(hist_bin):
    got, _, _ = run(hist_bin, [0.0] * 10)
    assert got == [0.0] * len(QS)
    got, _, _ = run(hist_bin, [42.5])
    assert got == [42.5] * len(QS)
    got, _, _ = run(hist_bin, [0.0, 0.0, 0.0, 10.0])
    want = np.percentile([0.0, 0.0, 0.0, 10.0], QS)
    assert np.allclose(got, want, rtol=2.6e-3, atol=1e-12)
    got, _, _ = run(hist_bin, [])
    assert got == [0.0] * len(QS)
