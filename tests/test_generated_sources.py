"""Generated sources: christoffel_sparse.cuh is exactly what its generator
writes (no hand edits), and the generator's operation counts, which the
benchmark's config-3 roofline uses, are those of the emitted code."""
import importlib.util
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "geon_gb300", "csrc")


@pytest.fixture(scope="module")
def gen():
    spec = importlib.util.spec_from_file_location("gen_sparse_christoffel",
                                                  os.path.join(CSRC, "gen_sparse_christoffel.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_sparse_christoffel_header_is_generated(gen):
    with open(os.path.join(CSRC, "christoffel_sparse.cuh")) as f:
        assert f.read() == gen.header_text()


def test_op_counts(gen):
    c = gen.op_counts()
    for name, points, evals in (("alcubierre", 7, 17), ("morris_thorne", 5, 5)):
        k = c[name]
        assert k["metric_points_per_rhs"] == points
        assert k["flops_per_rhs"] == sum(k["ops_per_rhs"].values()) + points * evals
        assert k["flops_per_step"] == 4 * k["flops_per_rhs"] + 104
    # the emitted Alcubierre code: 138 multiplications, 42 additions, 18
    # subtractions and 10 divisions per right-hand side
    assert c["alcubierre"]["ops_per_rhs"] == {"mul": 138, "add": 42, "sub": 18, "div": 10}
    assert c["alcubierre"]["calls_per_step"] == {"sqrt": 28, "tanh": 56}


def test_sincos_constants_match_their_derivation():
    """The constants of the deterministic FP64 sin/cos in devmath.cuh are the
    doubles nearest pi/2 (three parts), 2/pi and +-1/n! (gen_math_constants.py)."""
    mp = pytest.importorskip("mpmath")
    import re
    mp.mp.prec = 300
    with open(os.path.join(CSRC, "devmath.cuh")) as f:
        text = f.read()
    got = {m.group(1): float.fromhex(m.group(2))
           for m in re.finditer(r"constexpr double (\w+) = (-?0x[0-9a-fA-Fp.+-]+);", text)}
    pio2 = mp.pi / 2
    p1 = float(pio2)
    p2 = float(pio2 - p1)
    p3 = float(pio2 - p1 - p2)
    want = {"PIO2_1": p1, "PIO2_2": p2, "PIO2_3": p3, "TWO_OVER_PI": float(2 / mp.pi)}
    for n in range(3, 18, 2):
        want[f"S{n}"] = float((-1) ** ((n - 1) // 2) / mp.factorial(n))
    for n in range(4, 19, 2):
        want[f"C{n}"] = float((-1) ** (n // 2) / mp.factorial(n))
    for name, v in want.items():
        assert got[name] == v, name
