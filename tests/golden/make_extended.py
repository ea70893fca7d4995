"""Generate tests/golden/ext_poiseuille_256x64_20000.npz: the 256 x 64
Poiseuille channel after 20,000 steps of lbc's step evaluated in long double
(tests/golden/poiseuille_extended.c), the exact-arithmetic reference against
which the FP64 kernels' rounding is measured. Run on x86-64, where long double
has a 64-bit significand:

    python tests/golden/make_extended.py
"""
import os
import platform
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STEPS = 20000


def main():
    if platform.machine() not in ("x86_64", "AMD64"):
        raise SystemExit("run on x86-64 (long double with a 64-bit significand)")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "poiseuille_extended")
        subprocess.run(["gcc", "-std=c99", "-O2", "-o", exe, os.path.join(HERE, "poiseuille_extended.c")], check=True)
        out = subprocess.run([exe, str(STEPS)], check=True, capture_output=True, text=True).stdout
    vals = np.array([[float(x) for x in line.split()] for line in out.strip().splitlines()])
    np.savez_compressed(os.path.join(HERE, f"ext_poiseuille_256x64_{STEPS}.npz"), rho=vals[:, 0], u=vals[:, 1],
                        steps=STEPS)
    print("wrote", vals.shape)


if __name__ == "__main__":
    main()
