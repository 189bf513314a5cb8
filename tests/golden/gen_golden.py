"""Regenerate the golden input fixtures of this directory.

Compiles gen_inputs.cpp with g++ (libstdc++'s mt19937 and
uniform_real_distribution<float>, the generators the reference's tests use)
and writes grid_8193.bin and neighbors_257.bin next to this script.
"""

import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "gen_inputs")
        subprocess.check_call(["g++", "-O1", "-std=c++17", "-o", exe,
                               os.path.join(HERE, "gen_inputs.cpp")])
        subprocess.check_call([exe, HERE])


if __name__ == "__main__":
    main()
