"""Generates the golden fixtures of tests/golden/ in a container that holds the reference.

- sod_exact_t0.2.npz: exact solution of the Sod problem of the sod workload (diaphragm at x=0.5,
  (rho,u,p) = (1,0,1) | (0.125,0,0.1), gamma=1.4) at t=0.2 on 401 points, computed by the
  reference's own exact Riemann solver utilities/shockTubeSoln.py (imported from the reference
  tree; the solver works in (p, T) with R=287, so T = p/(rho R) is passed).
- oracle_sod_rhs.npz: a small oracle regression vector (40-cell Sod workload: the state after 15
  RK steps and its RHS), used to check that the oracle computes the same numbers on every host.

Run from the repository root:
    python tests/golden/make_golden.py --reference <path of the reference checkout>
(or with the PLENS_REFERENCE environment variable naming that path).
"""
import argparse
import contextlib
import io
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def sod_exact(reference: Path):
    sys.path.insert(0, str(reference / "utilities"))
    from shockTubeSoln import shockTubeSoln  # noqa: E402  (the reference's utility)
    R = 287.0
    x = np.linspace(0.0, 1.0, 401)
    with contextlib.redirect_stdout(io.StringIO()):
        out = shockTubeSoln(1.0, 0.1, 1.0 / (1.0 * R), 0.1 / (0.125 * R), 0.0, 0.0, x - 0.5, 0.2, gamma=1.4, R=R)
    return x, out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default=os.environ.get("PLENS_REFERENCE"),
                    help="root of the reference checkout (holds utilities/shockTubeSoln.py)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give --reference or set PLENS_REFERENCE")
    x, out = sod_exact(Path(args.reference))
    out = np.asarray(out, dtype=float)  # columns: x, T, p, u, rho
    p, u, rho = out[:, 2], out[:, 3], out[:, 4]
    np.savez(Path(__file__).parent / "sod_exact_t0.2.npz", x=x, rho=rho, u=u, p=p)

    from oracle.pyoracle import Oracle
    from plens_gb300 import configs
    case = configs.make_case(configs.sod(n=40))
    o = Oracle(case, threads=1)
    o.set_state(case.initial_state(), 0.0)
    o.advance(15)
    U, t, _, _ = o.get_state()
    o.set_state(U, t)
    Rr, a, ad = o.rhs()
    np.savez(Path(__file__).parent / "oracle_sod_rhs.npz", U=U, t=t, R=Rr, alpha=a)


if __name__ == "__main__":
    main()
