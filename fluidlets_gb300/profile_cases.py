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
    p.add_argument("op", choices=["sum", "assemble", "lu", "resistance", "breakdown", "swim"])
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
    elif a.op == "breakdown":
        breakdown(a, kern)
    elif a.op == "swim":
        swim_case(a)
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


def swim_case(a):
    """swim() of the biflagellate swimmer over one beat period (RK45, rtol 1e-6): FP64 solves per
    stage vs the captured mixed-precision stage graph; time per right-hand side.  Flagellum
    amplitude 0.08, so the two mirror-image flagella (attached at z = +-0.1) never touch (with 0.2
    they cross and the system is near-singular there); nearest map fixed at t = 0 (the flagellum
    quadrature points sit midway between force points, so a recomputed map would flip and make
    the right-hand side discontinuous)."""
    import fluidlets_gb300 as fl
    from fluidlets_gb300.geometry import biflagellate_shape

    calls = {"n": 0}

    def shape_at(t):
        calls["n"] += 1
        return biflagellate_shape(t, amplitude=0.08)

    s0 = biflagellate_shape(0.0, amplitude=0.08)
    out = {}
    for prec in ("fp64", "mixed", "mixed"):  # the second mixed run is timed warm
        calls["n"] = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr = fl.swim(shape_at, (0.0, 1.0), 0.02, rtol=1e-6, atol=1e-9, fixed_nearest=True, precision=prec)
        torch.cuda.synchronize()
        out[prec] = (time.perf_counter() - t0, calls["n"], tr)
    t64, n64, tr64 = out["fp64"]
    tmx, nmx, trmx = out["mixed"]
    dx = np.abs(tr64.x0[-1] - trmx.x0[-1]).max()
    print(f"swim: N={len(s0.x)} force / {len(s0.X)} quadrature points, n={3 * len(s0.x) + 6}; "
          f"fp64 {t64 * 1e3:.0f} ms for {n64} right-hand sides ({t64 / n64 * 1e3:.2f} ms each); "
          f"mixed {tmx * 1e3:.0f} ms for {nmx} ({tmx / nmx * 1e3:.2f} ms each); final position difference {dx:.1e}")


def breakdown(a, kern):
    """Phase times of one mixed-precision dense resistance solve (assembly, FP32 copy,
    tensor-core LU, FP64 GMRES-IR, final FP64 residual) and of the FP64 LU."""
    import ctypes

    from fluidlets_gb300 import _lib, core
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    L = _lib.load()
    dev = torch.device("cuda")
    X = fibonacci_sphere(a.n) + (np.array([0, 0, 1.5]) if a.kind == "wall" else 0)
    eps = 0.25 * mean_nn_spacing(X)
    Xd = torch.from_numpy(X).to(dev)
    e = torch.full((a.n,), eps, dtype=torch.float64, device=dev)
    U = torch.zeros_like(Xd)
    U[:, 0] = 1.0
    b = U.reshape(-1).contiguous()

    def t(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, 1e3 * (time.perf_counter() - t0)

    for rep in range(a.reps):
        L.flg_profile_enable(1)
        K, t_asm = t(lambda: core._assemble_dev(kern, Xd, Xd, e, 1.0, sym_eps=eps, reciprocal=True))
        (K32, ld32, dinv, A32), t_lu = t(lambda: core._lowp_factor_dev(K, a.lu))
        (x, it, outer, res), t_ir = t(lambda: core._gmres_ir_dense_dev(K, K32, ld32, dinv, b, 1e-12, 60, 200,
                                                                        required=1e-10, A32=A32))
        _, t_res = t(lambda: core._evaluate_dev(kern, Xd, Xd, x.reshape(-1, 3), e, 1.0, "fp64"))
        slots = {}
        for name, k in _lib.SLOT.items():
            ms, n = ctypes.c_double(0), ctypes.c_int64(0)
            L.flg_profile_read(k, ctypes.byref(ms), ctypes.byref(n))
            if n.value:
                slots[name] = (round(ms.value, 3), n.value)
        L.flg_profile_enable(0)
        print(f"[mixed {a.lu}] n={3 * a.n}: assemble {t_asm:.2f} ms, convert+LU {t_lu:.2f} ms, GMRES-IR {t_ir:.2f} ms "
              f"({it} it, {outer} IR, resid {res:.2e}), residual {t_res:.2f} ms; kernel slots (ms, launches): {slots}")
    if a.n > 4096:  # the FP64 factorizations take seconds at this size
        return
    K = core._assemble_dev(kern, Xd, Xd, e, 1.0)
    L.flg_profile_enable(1)
    _, t64 = t(lambda: core._lu_solve_dev(K.clone(), b))
    slots = {}
    for name, k in _lib.SLOT.items():
        ms, n = ctypes.c_double(0), ctypes.c_int64(0)
        L.flg_profile_read(k, ctypes.byref(ms), ctypes.byref(n))
        if n.value:
            slots[name] = (round(ms.value, 3), n.value)
    L.flg_profile_enable(0)
    print(f"[fp64] kernel slots (ms, launches): {slots}")
    torch.linalg.solve(K, b)  # library initialization outside the timing
    _, tcs = t(lambda: torch.linalg.solve(K, b))
    print(f"[fp64] LU factor+solve {t64:.2f} ms; cuSOLVER (torch.linalg.solve) {tcs:.2f} ms")


if __name__ == "__main__":
    main()
