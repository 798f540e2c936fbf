"""The committed FP64 oracle of the configured mixed-precision LP
(tests/golden/transport_20m_1e8.json, written on GB300 by
tests/golden/make_transport_oracle.py): the reference's own single-GPU solve
and this library's FP64 solve of the 20M-nnz transport LP to 1e-8."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "transport_20m_1e8.json")


def rel(a, b):
    return abs(a - b) / (1.0 + abs(b))


def test_transport_oracle_fixture_pins_ours_to_the_reference_at_1e8():
    with open(GOLDEN) as f:
        g = json.load(f)
    assert g["eps"] == 1e-8
    ref, ours = g["reference_fp64"], g["ours_fp64"]
    assert ref["status"] == ours["status"] == "OPTIMAL"
    # same iteration for iteration, objectives within the 1e-6 bar
    # (recorded: equal to 1e-14), both at the requested tolerance
    assert ours["total_count"] == ref["total_count"]
    for k in ("primal_objective_value", "dual_objective_value"):
        assert rel(ours[k], ref[k]) <= 1e-6
    for r in (ref, ours):
        for k in ("relative_primal_residual", "relative_dual_residual",
                  "relative_objective_gap"):
            assert r[k] <= 1e-8
