"""bin/energy_conditions.rs on the GPU: the bin's 99 numbers from one batched
device job (geon_energy_conditions), and its printed report.

`report()` formats the numbers as the bin prints them (energy_conditions.rs:
22-34 print_row and the println! lines of main), so a caller gets the bin's
stdout from the GPU path.
"""
import numpy as np

from . import _ffi
from ._util import check

N = 99


def values():
    """The 99 numbers in the bin's order (see geon_energy_conditions)."""
    out = np.empty(N)
    check(_ffi.load().geon_energy_conditions(out.ctypes.data_as(_ffi.c_double_p)))
    return out


def energy_conditions():
    """The bin's results by metric."""
    v = values()
    sch = v[2:8].reshape(3, 2)
    alc = v[8:52]
    mt = v[52:99]
    return {
        "minkowski": {"nec": v[0], "ricci_scalar": v[1]},
        "schwarzschild": {r: {"nec": sch[i, 0], "ricci_scalar": sch[i, 1]} for i, r in enumerate((5.0, 10.0, 30.0))},
        "alcubierre": {"x": -4.0 + 0.2 * np.arange(41), "nec": alc[:41], "min": alc[41], "min_x": alc[42],
                       "integral_negative": alc[43]},
        "morris_thorne": {"l": -4.0 + 0.2 * np.arange(41), "nec": mt[:41], "min": mt[41], "min_l": mt[42],
                          "throat_T_diag": mt[43:47]},
    }


def _exp(v, sign=True):
    """Rust's `{:+.4e}` / `{:.4e}`: 4 fractional digits, bare exponent (e-5, e0)."""
    s = f"{v:+.4e}" if sign else f"{v:.4e}"
    mant, ex = s.split("e")
    return f"{mant}e{int(ex)}"


def _row(label, val, threshold, note):
    # print_row (energy_conditions.rs:26-34)
    if val < -threshold:
        flag = "NEC VIOLATED"
    elif abs(val) < threshold:
        flag = "≈ 0"
    else:
        flag = "NEC ok"
    return f"  {label:<28}  {_exp(val):>13}   [{flag}]  {note}"


def report(v=None):
    """The bin's stdout, as lines, for the 99 numbers v (default: computed on the GPU)."""
    v = values() if v is None else np.asarray(v, dtype=np.float64)
    out = ["", "== Minkowski (sanity, T = 0 expected) =="]
    out.append(_row("T_μν k^μ k^ν", v[0], 1e-10, "should be 0"))
    out.append(_row("Ricci scalar", v[1], 1e-10, "should be 0"))
    out += ["", "== Schwarzschild (sanity, vacuum: T = 0, R = 0) =="]
    for i, r in enumerate((5, 10, 30)):
        out.append(_row(f"r = {r:>4}  NEC contraction", v[2 + 2 * i], 1e-4, "vacuum → ~0"))
        out.append(_row(f"r = {r:>4}  Ricci scalar", v[3 + 2 * i], 1e-4, "vacuum → ~0"))
    out += ["", "== Alcubierre warp bubble (expecting NEC violation across bubble wall) =="]
    out.append("  scanning along x at y=z=0:")
    for n in range(0, 41, 4):
        out.append(_row(f"x = {-4.0 + 0.2 * n:>6.2f}", v[8 + n], 1e-6, ""))
    out.append(f"  minimum T_μν k^μ k^ν = {_exp(v[49])} at x = {v[50]:.2f}  (negative = exotic matter required)")
    out.append(f"  ∫ T_kk dx (negative part only, axis only) ≈ {_exp(v[51])}  (rough exotic-mass proxy)")
    out += ["", "== Morris–Thorne wormhole (expecting NEC violation near throat) =="]
    out.append("  scanning along l (proper radial) at θ=π/2, φ=0:")
    for n in range(0, 41, 4):
        out.append(_row(f"l = {-4.0 + 0.2 * n:>6.2f}", v[52 + n], 1e-6, ""))
    out.append(f"  minimum T_μν k^μ k^ν = {_exp(v[93])} at l = {v[94]:.2f}  (negative ⇒ exotic matter at throat)")
    out += ["", "  T^μ_ν diagonal at throat (l=0):"]
    for i in range(4):
        out.append(f"    T[{i}][{i}] = {_exp(v[95 + i])}")
    return out
