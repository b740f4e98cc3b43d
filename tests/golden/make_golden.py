"""Generate the golden fixture tests/golden/oracle_golden.npz.

The reference ships no tests, fixtures or decks, and it cannot be compiled
here, so these vectors come from the oracle (the C restatement of the
reference MG path) on small seeded inputs after it passed the reference's own
known-answer test.  They pin the oracle (and, on the GPU, the kernels) against
regressions.  Run:  python -m tests.golden.make_golden
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "oracle_golden.npz"


def compute():
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from oracle.oracle import Oracle
    from tests.helpers import oracle_stagnated

    out = {}
    # 2D known-answer case, n = 16 (Poisson_Tester)
    kat = P.kat2d(16, restol_Poisson=1e-12)
    r = Oracle(kat).solve()
    out["kat16_p"] = r["p"][1:17, 1:17, 1]
    out["kat16_hist"] = r["hist"]
    # 2D random box, one MG_Solver call from zero
    box = P.box2d(16, seed=11)
    o = Oracle(box)
    v = np.zeros(box.shape, order="F")
    o.subtract_average(v)
    o.mg_solver(v, box.nlu0)
    out["box16_nlu0"] = box.nlu0[1:17, 1:17, 1]
    out["box16_mg1"] = v[1:17, 1:17, 1]
    # 3D sphere 12^3 uniform: geometry integers, compatible RHS, converged solve
    sp = P.sphere(12, stretch=None, seed=13)
    c = P.make_compatible(sp, oracle_stagnated(sp))
    out["sph12_shift"] = np.array([c])
    out["sph12_iblank"] = sp.geom.iblank[1:13, 1:13, 1:13].copy()
    out["sph12_ghost_ijk"] = np.stack([sp.geom.iG, sp.geom.jG, sp.geom.kG])
    out["sph12_cell_ijk"] = np.stack([sp.geom.iCI, sp.geom.jCI, sp.geom.kCI])
    out["sph12_coeff"] = sp.geom.coeff.copy()
    sp.params.restol_Poisson = 1e-10 * abs(sp.nlu0).max()
    r = Oracle(sp).solve()
    out["sph12_p"] = r["p"][1:13, 1:13, 1:13]
    out["sph12_hist"] = r["hist"]
    return out


if __name__ == "__main__":
    data = compute()
    np.savez_compressed(GOLDEN, **data)
    print(GOLDEN, {k: v.shape for k, v in data.items()})
