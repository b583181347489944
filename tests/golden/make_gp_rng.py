"""Writes gp_rng.json: the first draws of the reference's general-position
perturbation sequence (preproc.cpp:2621-2627: a thread_local
std::default_random_engine seeded 1 seeds a std::mt19937, and
std::uniform_real_distribution<double>(-1, 1) draws from it), produced by
compiling that expression with the host's C++ standard library.

    python tests/golden/make_gp_rng.py
"""
import json
import os
import subprocess
import tempfile

N = 24
SRC = r"""
#include <cstdio>
#include <random>
int main() {
    static thread_local std::default_random_engine random_engine(1);
    static thread_local std::mt19937 mersenne_twister_generator(random_engine());
    static thread_local std::uniform_real_distribution<double> uniform_distribution(-1.0, 1.0);
    for (int i = 0; i < %d; ++i) std::printf("%%a\n", uniform_distribution(mersenne_twister_generator));
}
""" % N


def main():
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "rng.cpp"), os.path.join(d, "rng")
        with open(src, "w") as f:
            f.write(SRC)
        subprocess.run(["g++", "-O2", "-o", exe, src], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    draws = [float.fromhex(x) for x in out]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gp_rng.json")
    with open(path, "w") as f:
        json.dump({"source": "std::mt19937(std::default_random_engine(1)()), uniform_real_distribution<double>(-1, 1)",
                   "draws_hex": [d.hex() for d in draws]}, f, indent=1)
    print(path, len(draws))


if __name__ == "__main__":
    main()
