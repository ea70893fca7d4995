"""Generate the golden fixtures in tests/golden/ from lbc itself.

Runs lbc's own FP64 solver (oracle/_ref/libref_lbc.so, compiled from lbc's
src/ by oracle/build_ref.sh) on every case of tests/casezoo.py and stores the
final state and the per-step force of each run, and copies the first records
of lbc's shipped cylinder force history
(cases/cylinder/sol/forces_IBB_res_20_Re_20.00_tau_0.90.bin).

    python tests/golden/make_golden.py [LBC_SOURCE_DIR]
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from lbc_gb300.abi import LbcAbi  # noqa: E402
import casezoo  # noqa: E402


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LBC_REF", "/root/reference")
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), src], check=True)
    ref = LbcAbi(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_lbc.so")), "ref_")
    for name, builder, steps in casezoo.standard_cases():
        case, st = builder()
        forces = ref.run(case, st, steps, record_forces=True)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), f=st.f, f_new=st.f_new,
                            rho=st.rho, u=st.u, v=st.v, forces=forces, steps=steps)
        print("wrote", name, steps, "steps")
    g = np.fromfile(os.path.join(src, "cases", "cylinder", "sol",
                                 "forces_IBB_res_20_Re_20.00_tau_0.90.bin")).reshape(-1, 3)
    np.save(os.path.join(HERE, "lbc_cylinder_forces_res20_first300.npy"), g[:300])
    print("wrote cylinder force records", g[:300].shape)


if __name__ == "__main__":
    main()
