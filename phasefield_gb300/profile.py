"""Runs a short, fixed piece of a named workload on cuda:0 (for profilers such as ncu).

  python -m phasefield_gb300.profile --workload cahn_hilliard_3d --refine 6 --steps 3
  python -m phasefield_gb300.profile --workload eshelby_3d --refine 5 --mixed 1
  python -m phasefield_gb300.profile --workload eshelby_3d --refine 6 --preconditioner 1
  python -m phasefield_gb300.profile --workload ensemble --steps 3
  python -m phasefield_gb300.profile --workload cahn_hilliard_amr_3d --steps 3

Explicit workloads run `steps` increments; eshelby_3d runs one preconditioned CG solve
(--preconditioner 2: GMG with --mg-depth levels, default refine + 1; 1: Chebyshev on the fine
level only; Chebyshev degree 4; FP32 smoothing levels with --mixed 1); ensemble runs `steps`
steps of the 256-instance Allen-Cahn ensemble; cahn_hilliard_amr_3d is periodic Cahn-Hilliard
Q2 on [0,64]^3 with an adaptive mesh of levels 5..7 (refined where |grad c| > 0.15, about 112k
cells after the initial passes, dt 1e-5), run for `steps` increments after its initial
refinement. The command exits non-zero if a run reports an error.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from . import workloads as W


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cahn_hilliard_3d",
                    choices=["allen_cahn_2d", "cahn_hilliard_3d", "coupled_acch_2d", "eshelby_3d", "ensemble",
                             "cahn_hilliard_amr_3d"])
    ap.add_argument("--refine", type=int, default=None)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--mixed", type=int, default=0)
    ap.add_argument("--preconditioner", type=int, default=2, choices=[0, 1, 2])
    ap.add_argument("--mg-depth", type=int, default=None)
    args = ap.parse_args(argv)
    kw = {} if args.refine is None else {"refine": args.refine}
    if args.workload == "ensemble":
        from . import ensemble as E
        meshes, mw, ka, ics = E.allen_cahn_ensemble(n_instances=256)
        ens = E.Ensemble(meshes, mw, ka, 0.01)
        for i, ic in enumerate(ics):
            ens.upload(i, ic)
        ens.run(args.steps, use_graph=False)
        ens.synchronize()
        ens.close()
    elif args.workload == "eshelby_3d":
        wl = W.eshelby_3d(**kw)
        p = wl.make_problem()
        b = p.apply(0, 0, None, scale=0)
        depth = args.mg_depth if args.mg_depth else wl.mesh.global_refinement + 1
        p.set_linear_params(0, tolerance_type=0, tolerance=1e-10 * float(np.linalg.norm(b)), max_iterations=2000,
                            preconditioner=args.preconditioner, mg_depth=depth, smoother_degree=4,
                            mixed_precision=args.mixed)
        its, _ = p.linear_solve(0)
        print("phases (ms):", {k: round(v, 2) for k, v in p.linear_stats(0).items()})
        p.close()
        print(f"eshelby_3d: preconditioner {args.preconditioner} CG {its} iterations ok")
        return 0
    elif args.workload == "cahn_hilliard_amr_3d":
        wl = W.cahn_hilliard_amr(3, refine=6, degree=2, min_level=5, max_level=7, period=0, size=64.0, dt=1e-5,
                                 gradient_bound=0.15)
        p = wl.make_problem()
        p.solve(args.steps)
        p.synchronize()
        print(f"cahn_hilliard_amr_3d: {p.n_cells} cells, {p.n_nodes} DoFs per field")
        p.close()
    else:
        wl = getattr(W, args.workload)(**kw)
        p = wl.make_problem()
        p.solve(args.steps)
        p.synchronize()
        p.close()
    print(f"{args.workload}: {args.steps} steps ok")
    return 0


if __name__ == "__main__":
    sys.exit(main())
