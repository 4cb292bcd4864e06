"""Writes tests/golden/samples/mt19937_uniform.npz: the draws the reference's pairing-instability
sample takes (src/sample/pairing_instability.cpp:29-35: std::mt19937 engine(1) and
std::uniform_real_distribution<real>(-0.05 dx, 0.05 dx) with dx = 1/64), produced by the GNU C++
standard library itself, for the Python restatement in sphcode_gb300/ics.py to be pinned to.

    python tests/golden/make_sample_golden.py
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
COUNT = 2 * 64 * 64

PROGRAM = r"""
#include <cstdio>
#include <random>
int main() {
    std::mt19937 raw(1);
    for (int i = 0; i < 16; ++i) std::printf("%u\n", (unsigned)raw());
    const double dx = 1.0 / 64;
    std::mt19937 engine(1);
    std::uniform_real_distribution<double> dist(-dx * 0.05, dx * 0.05);
    for (int i = 0; i < %d; ++i) std::printf("%%a\n", dist(engine));
    return 0;
}
"""


def main():
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "mt.cpp")
        exe = os.path.join(tmp, "mt")
        with open(src, "w") as f:
            f.write(PROGRAM.replace("%d", str(COUNT)).replace("%%", "%"))
        subprocess.check_call(["g++", "-O0", "-std=c++14", src, "-o", exe])
        out = subprocess.check_output([exe], text=True).split()
    raw = np.array([int(x) for x in out[:16]], dtype=np.uint64)
    draws = np.array([float.fromhex(x) for x in out[16:]], dtype=np.float64)
    assert draws.size == COUNT
    np.savez_compressed(os.path.join(HERE, "samples", "mt19937_uniform.npz"), raw=raw, draws=draws)


if __name__ == "__main__":
    main()
