"""Regenerate the golden fixtures from the reference's own printed results.

Reads, as text, the known-answer output the reference commits
(docs/energy_conditions.txt, the stdout of bin/energy_conditions.rs, kept both
as parsed values and line for line) and the
shadow-validation lines of its README (README.md:43-45, the stdout of
bin/validate_shadow.rs), and writes them as JSON next to this script. Run in a
checkout where the reference sits at GEON_REFERENCE_DIR (default: a checkout
named "reference" beside this repository); the JSON files are committed so the
tests never need the reference itself.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: GEON_REFERENCE_DIR, else a checkout named "reference"
# beside this repository
REF = os.environ.get("GEON_REFERENCE_DIR") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")
NUM = r"[+-]?\d+\.\d+e[+-]?\d+"


def energy_conditions():
    txt = open(os.path.join(REF, "docs", "energy_conditions.txt"), encoding="utf-8").read()
    out = {"source": "docs/energy_conditions.txt", "sig_digits": 5}
    lines = txt.splitlines()
    sec = None
    rows = {"minkowski": [], "schwarzschild": [], "alcubierre": [], "morris_thorne": []}
    extra = {}
    for ln in lines:
        if ln.startswith("== Minkowski"):
            sec = "minkowski"
        elif ln.startswith("== Schwarzschild"):
            sec = "schwarzschild"
        elif ln.startswith("== Alcubierre"):
            sec = "alcubierre"
        elif ln.startswith("== Morris"):
            sec = "morris_thorne"
        m = re.search(r"minimum T_μν k\^μ k\^ν = (" + NUM + r") at [xl] = ([+-]?\d+\.\d+)", ln)
        if m:
            extra[sec + "_min"] = float(m.group(1))
            extra[sec + "_min_at"] = float(m.group(2))
            continue
        m = re.search(r"∫ T_kk dx .* ≈ (" + NUM + ")", ln)
        if m:
            extra["alcubierre_integral"] = float(m.group(1))
            continue
        m = re.search(r"T\[(\d)\]\[\d\] = (" + NUM + ")", ln)
        if m:
            extra.setdefault("morris_thorne_throat_T_diag", []).append(float(m.group(2)))
            continue
        m = re.search(r"\s(" + NUM + r")\s+\[", ln)
        if m and sec:
            rows[sec].append({"label": " ".join(ln[:m.start(1)].split()), "value": float(m.group(1))})
    out.update(rows)
    out.update(extra)
    return out


def shadow():
    txt = open(os.path.join(REF, "README.md"), encoding="utf-8").read()
    a = re.search(r"analytic: b_c = 3√3 M = (\d+\.\d+), α_c = (\d+\.\d+)°", txt)
    m = re.search(r"measured: b_c =\s+(\d+\.\d+), α_c = (\d+\.\d+)°", txt)
    e = re.search(r"relative error: (\d+\.\d+e-?\d+)", txt)
    nr = re.search(r"\|g_μν p\^μ p\^ν\| ≈ (\d+e-?\d+)", txt)
    return {"source": "README.md:43-50 (bin/validate_shadow.rs settings: r_obs 20, h 0.01, "
                      "max 200000, 60 bisections of [0, pi/2 - 1e-3])",
            "b_c_analytic": float(a.group(1)), "alpha_c_analytic_deg": float(a.group(2)),
            "b_c_measured": float(m.group(1)), "alpha_c_measured_deg": float(m.group(2)),
            "rel_err": float(e.group(1)), "minkowski_null_residual_order": float(nr.group(1))}


def energy_conditions_stdout():
    # the bin's stdout as the reference committed it, line for line
    return open(os.path.join(REF, "docs", "energy_conditions.txt"), encoding="utf-8").read().splitlines()


def main():
    ec = energy_conditions()
    sh = shadow()
    for name, obj in (("energy_conditions.json", ec), ("validate_shadow.json", sh),
                      ("energy_conditions_stdout.json", {"source": "docs/energy_conditions.txt",
                                                         "lines": energy_conditions_stdout()})):
        with open(os.path.join(HERE, name), "w", encoding="utf-8") as f:
            json.dump(obj, f, indent=1, ensure_ascii=False)
            f.write("\n")
    print(json.dumps(sh), file=sys.stderr)
    print({k: (len(v) if isinstance(v, list) else v) for k, v in ec.items()}, file=sys.stderr)


if __name__ == "__main__":
    main()
