"""Run one named case on the GPU for a number of steps (device-resident).

    python -m lbc_gb300.runcase --case taylor_green --n 2048 --storage f32 --steps 20

Prints one line with the wall time of the run (CUDA events) and MLUPS. Used to
profile a single kernel on a small case, and as a command-line case main.
"""
import argparse
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from lbc_gb300 import STORAGE, GpuSolver, cases  # noqa: E402

BUILDERS = {
    "taylor_green": lambda n, ny: cases.taylor_green(n, ny or n, 0.04, 0.56),
    "poiseuille": lambda n, ny: cases.poiseuille(n, ny or max(8, n // 4), 0.8, 1e-6),
    "cavity": lambda n, ny: cases.cavity_moving_wall(n, 0.1, 1000.0),
    "cavity_zouhe": lambda n, ny: cases.cavity_zouhe(n, 0.1, 1000.0),
    "cylinder": lambda n, ny: cases.cylinder_wake(n, ny or n // 4, D=max(8.0, n / 32), xc=n / 4,
                                                  yc=(ny or n // 4) / 2),
}


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--case", default="taylor_green", choices=sorted(BUILDERS))
    p.add_argument("--n", type=int, default=2048)
    p.add_argument("--ny", type=int, default=0)
    p.add_argument("--storage", default="f32", choices=sorted(STORAGE))
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=2)
    p.add_argument("--block", default="", help="bx,by thread block of the fused step")
    p.add_argument("--ducts", type=int, default=0, help="run this many seeded liner ducts as one batch")
    p.add_argument("--serve", type=int, default=0, help="serve a seeded stream of this many requests")
    p.add_argument("--scale", type=float, default=1.0, help="step-count scale of the served stream")
    p.add_argument("--rate", type=float, default=200.0, help="arrival rate of the served stream (1/s)")
    p.add_argument("--max-active", type=int, default=64)
    p.add_argument("--chunk", type=int, default=1000)
    p.add_argument("--wake", type=int, default=0,
                   help="cylinder wake (2048 x 512, Re 100): Cd, Cl, St after this many steps")
    p.add_argument("--vs-f64", action="store_true",
                   help="also run the case in FP64 for the same steps; report the u L2 error against it")
    p.add_argument("--autotune", action="store_true",
                   help="tune block / tile shapes on the warm-up steps (LBM_GPU_AUTOTUNE=1)")
    a = p.parse_args(argv)
    if a.autotune:
        os.environ["LBM_GPU_AUTOTUNE"] = "1"
        a.warmup = max(a.warmup, 80)
    if a.wake:
        from lbc_gb300 import wake
        h = wake.cylinder_forces(STORAGE[a.storage], a.wake)
        r = wake.summary(h)
        r.update({"storage": a.storage, "steps": a.wake})
        print(json.dumps(r))
        return
    if a.serve:
        from lbc_gb300 import serving
        stream = serving.make_stream(a.serve, rate=a.rate, scale=a.scale)
        r = serving.serve(stream, a.max_active, a.chunk, prebuild=a.serve <= 400)
        r.pop("latencies_s")
        r["serial_fp64"] = serving.serial_fp64_estimate(stream)
        print(json.dumps(r))
        return
    if a.ducts:
        from lbc_gb300 import impedance as imp
        r = imp.run_liner_batch(a.ducts, a.steps, STORAGE[a.storage])
        print(json.dumps({k: v for k, v in r.items()}))
        return
    case, st = BUILDERS[a.case](a.n, a.ny)
    s = GpuSolver(case, STORAGE[a.storage])
    if a.block:
        bx, by = (int(x) for x in a.block.split(","))
        s.set_block(bx, by)
    s.set_state(st)
    s.run(a.warmup)
    ms = s.run_timed(a.steps)
    tuned, blk, us = s.autotune_status()
    out = {"case": a.case, "Nx": case.Nx, "Ny": case.Ny, "storage": a.storage,
           "steps": a.steps, "ms": round(ms, 3),
           "mlups": round(case.nodes * a.steps / (ms / 1e3) / 1e6, 1),
           "block": list(blk), "tuned": tuned}
    if a.vs_f64:
        import numpy as np
        r, u, v = s.get_fields()
        ref = GpuSolver(case, STORAGE["f64"])
        ref.set_state(st)
        ref.run(a.warmup)
        ms64 = ref.run_timed(a.steps)
        r64, u64, v64 = ref.get_fields()
        m = case.solid_mask == 0
        out["f64_mlups"] = round(case.nodes * a.steps / (ms64 / 1e3) / 1e6, 1)
        out["u_l2_rel_vs_f64"] = float(np.sqrt(np.sum((u[m] - u64[m]) ** 2 + (v[m] - v64[m]) ** 2) /
                                               np.sum(u64[m] ** 2 + v64[m] ** 2)))
        out["mass_rel_vs_f64"] = float(np.sum(r[m]) / np.sum(r64[m]) - 1.0)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
