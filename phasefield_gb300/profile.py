"""Runs a few increments of a named workload on cuda:0 (for profilers such as ncu).

  python -m phasefield_gb300.profile --workload cahn_hilliard_3d --refine 6 --steps 3

The workloads are those of phasefield_gb300.workloads with their default parameters except
the refinement level; the command exits non-zero if the run reports an error.
"""
from __future__ import annotations

import argparse
import sys

from . import workloads as W


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cahn_hilliard_3d",
                    choices=["allen_cahn_2d", "cahn_hilliard_3d", "coupled_acch_2d"])
    ap.add_argument("--refine", type=int, default=None)
    ap.add_argument("--steps", type=int, default=3)
    args = ap.parse_args(argv)
    kw = {} if args.refine is None else {"refine": args.refine}
    wl = getattr(W, args.workload)(**kw)
    p = wl.make_problem()
    p.solve(args.steps)
    p.synchronize()
    p.close()
    print(f"{args.workload}: {args.steps} increments ok")
    return 0


if __name__ == "__main__":
    sys.exit(main())
