"""Generate the golden fixtures in tests/golden/ from lbc itself.

Runs lbc's own FP64 solver (oracle/_ref/libref_lbc.so, compiled from lbc's
src/ by oracle/build_ref.sh) on every case of tests/casezoo.py and stores the
final state and the per-step force of each run, and copies the first records
of lbc's shipped cylinder force history
(cases/cylinder/sol/forces_IBB_res_20_Re_20.00_tau_0.90.bin).

    python tests/golden/make_golden.py [LBC_SOURCE_DIR] [--vtk-only] [--only=NAME,NAME]

It also writes lbc_small.vtk: lbc's write_vtk_binary_2D on a small seeded field.
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


VTK_ARGS = (7, 5, 0.5, 2.0, 3.0)  # Nx, Ny, dx, cu, crho


def vtk_inputs():
    rng = np.random.default_rng(7)
    Nx, Ny = VTK_ARGS[:2]
    u = rng.uniform(-0.1, 0.1, (Ny, Nx))
    v = rng.uniform(-0.1, 0.1, (Ny, Nx))
    rho = 1.0 + rng.uniform(-0.01, 0.01, (Ny, Nx))
    u[2, 3] = np.nan  # lbc's moments are NaN at solid nodes
    return u, v, rho


def write_vtk_fixture(lib):
    """lbc's write_vtk_binary_2D on a small seeded field -> lbc_small.vtk."""
    Nx, Ny, dx, cu, crho = VTK_ARGS
    u, v, rho = vtk_inputs()
    fn = lib.ref_write_vtk_binary_2D
    dp = C.POINTER(C.c_double)
    fn.restype = None
    fn.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, dp, dp, dp, C.c_double, C.c_double]
    out = os.path.join(HERE, "lbc_small.vtk")
    fn(out.encode(), Nx, Ny, dx, u.ctypes.data_as(dp), v.ctypes.data_as(dp), rho.ctypes.data_as(dp), cu, crho)
    print("wrote", out)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    # lbc's sources: the argument, else what oracle/build_ref.sh finds.
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")] + args[:1], check=True)
    with open(os.path.join(ROOT, "oracle", "_ref", "SOURCE")) as fh:
        src = fh.read().strip()
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_lbc.so"))
    write_vtk_fixture(lib)
    if "--vtk-only" in sys.argv:
        return
    ref = LbcAbi(lib, "ref_")
    only = [a.split("=", 1)[1].split(",") for a in sys.argv[1:] if a.startswith("--only=")]
    for name, builder, steps in casezoo.standard_cases():
        if only and name not in only[0]:
            continue
        case, st = builder()
        forces = ref.run(case, st, steps, record_forces=True)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), f=st.f, f_new=st.f_new,
                            rho=st.rho, u=st.u, v=st.v, forces=forces, steps=steps)
        print("wrote", name, steps, "steps")
    if only:
        return
    g = np.fromfile(os.path.join(src, "cases", "cylinder", "sol",
                                 "forces_IBB_res_20_Re_20.00_tau_0.90.bin")).reshape(-1, 3)
    np.save(os.path.join(HERE, "lbc_cylinder_forces_res20_first300.npy"), g[:300])
    print("wrote cylinder force records", g[:300].shape)


if __name__ == "__main__":
    main()
