"""Run one hot-path operation at a chosen size (for profiler captures).

    python -m fluidlets_gb300.profile_cases sum --kind wall --targets 65536 --sources 262144 --precision mixed
    python -m fluidlets_gb300.profile_cases lu --n 4608 --lu tf32

Inputs are the seeded synthetic workloads of bench.py at reduced size.
"""
from __future__ import annotations

import argparse
import time

import numpy as np
import torch


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("op", choices=["sum", "assemble", "lu", "resistance"])
    p.add_argument("--kind", default="wall", choices=["stokeslet", "wall", "brinkman"])
    p.add_argument("--alpha", type=complex, default=0.0)
    p.add_argument("--targets", type=int, default=65536)
    p.add_argument("--sources", type=int, default=262144)
    p.add_argument("--precision", default="mixed")
    p.add_argument("--n", type=int, default=1536, help="points for assemble/lu/resistance")
    p.add_argument("--lu", default="tf32")
    p.add_argument("--reps", type=int, default=2)
    a = p.parse_args(argv)

    import fluidlets_gb300 as fl
    from fluidlets_gb300 import core
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing, wall_sum_workload

    dev = torch.device("cuda")
    kern = {"stokeslet": fl.Stokeslet3D(), "wall": fl.WallStokeslet3D()}.get(a.kind) or fl.Brinkmanlet3D(a.alpha)
    if a.op == "sum":
        T, S, F, eps = wall_sum_workload(a.sources, a.targets, 0, 0.01, seed=0)
        Td, Sd, Fd = (torch.from_numpy(x).to(dev) for x in (T, S, F))
        for _ in range(a.reps):
            fl.evaluate(kern, Td, Sd, Fd, eps, precision=a.precision)
        torch.cuda.synchronize()
    else:
        X = fibonacci_sphere(a.n) + (np.array([0, 0, 1.5]) if a.kind == "wall" else 0)
        eps = 0.25 * mean_nn_spacing(X)
        Xd = torch.from_numpy(X).to(dev)
        U = torch.zeros_like(Xd)
        U[:, 0] = 1.0
        for _ in range(a.reps):
            t0 = time.perf_counter()
            if a.op == "assemble":
                fl.assemble(kern, Xd, Xd, eps)
            elif a.op == "lu":
                core.resistance(kern, Xd, U, eps, method="lu", precision=a.precision, lu=a.lu)
            else:
                core.resistance(kern, Xd, U, eps, precision=a.precision, lu=a.lu)
            torch.cuda.synchronize()
            print(f"{a.op} n={a.n}: {1e3 * (time.perf_counter() - t0):.2f} ms")


if __name__ == "__main__":
    main()
