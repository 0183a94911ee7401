"""Full-length benchmark scenes against the reference's own CPU solver.

The reference build ran c0 (2000 steps) and c1 (8000 steps) to produce the
golden recorder series.  Two bars, side by side:
  * reference arithmetic (FP32, the reference's tables and update order)
    within 1e-4 relative L2 of the reference's CPU solver;
  * accurate arithmetic (the default) within 1e-4 of the FP64 GPU oracle,
    and no farther from the reference's CPU solver than that solver's own
    FP32 rounding puts it from FP64 (+1e-5).
All cross errors are printed (pytest -s)."""
import numpy as np
import pytest

import ard_gb300 as A
from ard_gb300 import configs as K
from helpers import load_run, rel_l2

pytestmark = pytest.mark.gpu


def _run(g, precision, arithmetic):
    sc = g["scene"]
    p = sc["params"]
    T = sc["steps"]
    scene = A.build_scene(sc["air"], sc["sources"], sc["recorders"], p["dh"], p["dt"], p["c0"], p["pml_layers"])
    sim = A.Simulation(scene, precision=precision, max_steps=T, arithmetic=arithmetic)
    sim.set_source_series(0, g["sources"][0])
    sim.run(T)
    out = sim.recorders(f64=True)
    sim.close()
    return out


@pytest.mark.parametrize("name", ["c0_full", "c1_full"])
def test_full_length(name):
    """Reference arithmetic: within 1e-4 of the reference's CPU solver.
    Accurate arithmetic (the default): within 1e-4 of the FP64 GPU oracle.
    All cross errors are printed (pytest -s)."""
    g = load_run(name)
    if g is None:
        pytest.skip(f"golden {name} not generated")
    want = g["recorders"].astype(np.float64)
    f64 = _run(g, A.PREC_F64, A.ARITH_ACCURATE)
    acc = _run(g, A.PREC_F32, A.ARITH_ACCURATE)
    ref = _run(g, A.PREC_F32, A.ARITH_REFERENCE)
    for r in range(want.shape[1]):
        e = dict(ref_vs_reference=rel_l2(ref[:, r], want[:, r]), acc_vs_fp64=rel_l2(acc[:, r], f64[:, r]),
                 acc_vs_reference=rel_l2(acc[:, r], want[:, r]), ref_vs_fp64=rel_l2(ref[:, r], f64[:, r]),
                 fp64_vs_reference=rel_l2(f64[:, r], want[:, r]))
        print(name, "recorder", r, " ".join(f"{k}={v:.2e}" for k, v in e.items()))
        assert e["ref_vs_reference"] < 1e-4
        assert e["acc_vs_fp64"] < 1e-4
        # the default (accurate) arithmetic against the reference's CPU solver: no farther than the
        # reference's own FP32 solution lies from FP64, plus 1e-5
        assert e["acc_vs_reference"] <= e["fp64_vs_reference"] + 1e-5
