"""The oracle port's speed against the reference's own compiled code on the
same point solves, one thread each (test infrastructure: it shows what the
CPU baseline, which is the port, stands for).

The reference side is `oracle/_ref/libspac_ref.so` (the reference's sources
compiled unmodified against the shim, `make -C oracle ref`), driven through
`ref_point_solve` = FeynmanKacSolver::Solve_OMP_Analytic(X0, N, h, rho, bvp)
(Solvers/FeynmanKacSolver.cpp:335-342) with one OpenMP thread; the port is
`orc_point_solve` on the same problem, point, N and h with its sequential
random stream (the reference's draws).  Both run here, where the reference
sources exist; prints one JSON line per case.

    OMP_NUM_THREADS=1 python oracle/time_port_vs_ref.py
"""
import ctypes as C
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import oracle_py as orc  # noqa: E402

_dp = C.POINTER(C.c_double)
CASES = [  # name, problem, point, N, h
    ("franke (config 1 point)", 0, (0.3, 0.4), 20000, 1e-3),
    ("aniso", 2, (0.25, 0.75), 20000, 1e-3),
]


def ref_lib():
    orc.build(ref=True)
    L = C.CDLL(os.path.join(HERE, "_ref", "libspac_ref.so"))
    L.ref_solver_new.restype = C.c_void_p
    L.ref_solver_new.argtypes = [C.c_int]
    L.ref_point_solve.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, _dp, C.c_double, C.c_double, C.c_uint,
                                  C.c_double, _dp]
    return L


def main():
    R = ref_lib()
    rs = R.ref_solver_new(1)
    s = orc.Session(orc.RNG_SEQUENTIAL)  # draws what the one-thread reference draws, call after call
    for name, problem, (x, y), N, h in CASES:
        out = (C.c_double * 9)()
        dom = (C.c_double * 4)(0, 0, 1, 1)
        t0 = time.perf_counter()
        R.ref_point_solve(rs, problem, 0, dom, 0, None, x, y, N, h, out)
        t_ref = time.perf_counter() - t0
        b = orc.bvp(problem)
        t0 = time.perf_counter()
        o = s.point_solve(b, x, y, N, h)
        t_port = time.perf_counter() - t0
        print(json.dumps({"case": name, "paths": N, "h": h, "reference_paths_per_s": N / t_ref,
                          "port_paths_per_s": N / t_port, "port_over_reference": t_ref / t_port,
                          "phi_reference": out[0], "phi_port": o["phi"]}))


if __name__ == "__main__":
    main()
