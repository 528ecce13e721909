"""bin/energy_conditions.rs as one batched device job: the 99 numbers equal the
oracle's deterministic-math mode bit for bit, and the printed report equals the
reference's committed stdout line for line."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_energy_conditions_bit_exact(geon, orc):
    from geon_gb300 import energy
    v = energy.values()
    assert np.array_equal(v, orc.energy_conditions(orc.GEON))
    assert np.allclose(v, orc.energy_conditions(orc.LIBM), rtol=0, atol=1e-6)


def test_energy_conditions_report(geon):
    from geon_gb300 import energy
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "energy_conditions_stdout.json"),
                          encoding="utf-8"))["lines"]
    assert energy.report() == gold
    r = energy.energy_conditions()
    assert abs(r["morris_thorne"]["throat_T_diag"][0] + 1.0 / (8.0 * np.pi)) < 1e-6
