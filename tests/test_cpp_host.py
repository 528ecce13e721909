"""The C++ host side: include/geon.hpp (the crate's API over the C ABI) and the
C++ ports of the reference's executables (bin/validate_shadow.rs,
bin/energy_conditions.rs, bin/render.rs). CPU tests build them and check
argument handling and the Rust-style number formatting; GPU tests run them
and compare their output with the reference's committed output."""
import json
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def programs():
    from geon_gb300 import build
    build.build()
    return dict(zip(build.PROGRAMS, build.build_programs()))


def test_programs_build_and_parse_arguments(programs):
    r = subprocess.run([programs["render"], "--metric", "kerr"], capture_output=True, text=True)
    assert r.returncode == 2 and "invalid value 'kerr'" in r.stderr
    r = subprocess.run([programs["render"], "--width"], capture_output=True, text=True)
    assert r.returncode == 2 and "needs a value" in r.stderr


def test_rust_number_formatting(tmp_path):
    src = tmp_path / "fmt.cpp"
    src.write_text('#include <cstdio>\n#include "rust_fmt.hpp"\nint main(){using namespace rustfmt;'
                   'for (double v : {3.5496e-7, -2.4626e-2, 0.0, -0.0, 12345.678, 1.0e-300})'
                   ' std::printf("%s|%s|%s\\n", exp(v, 4).c_str(), exp(v, 4, true).c_str(), display(v).c_str());'
                   'std::printf("%s|%s|%s\\n", display(20.0).c_str(), display(0.05).c_str(), fixed(2.4, 2).c_str());}')
    exe = tmp_path / "fmt"
    subprocess.run(["g++", "-std=c++17", f"-I{os.path.join(ROOT, 'geon_gb300', 'cpp')}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    # Rust: format!("{:.4e}|{:+.4e}|{}", v, v, v)
    assert out[0] == "3.5496e-7|+3.5496e-7|0.00000035496"
    assert out[1] == "-2.4626e-2|-2.4626e-2|-0.024626"
    assert out[2] == "0.0000e0|+0.0000e0|0"
    assert out[3] == "-0.0000e0|-0.0000e0|-0"
    assert out[4] == "1.2346e4|+1.2346e4|12345.678"
    assert out[6] == "20|0.05|2.40"


@pytest.mark.gpu
def test_energy_conditions_program(programs):
    gold = json.load(open(os.path.join(GOLD, "energy_conditions_stdout.json"), encoding="utf-8"))["lines"]
    r = subprocess.run([programs["energy_conditions"]], capture_output=True, text=True, check=True)
    assert r.stdout.splitlines() == gold


@pytest.mark.gpu
def test_validate_shadow_program(programs):
    g = json.load(open(os.path.join(GOLD, "validate_shadow.json")))
    r = subprocess.run([programs["validate_shadow"]], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "== Schwarzschild shadow validation ==" and lines[1] == "M = 1, r_obs = 20"
    assert lines[2].startswith(f"analytic: b_c = 3√3 M = {g['b_c_analytic']:.6f}, α_c = ")
    assert lines[2].endswith(f"{g['alpha_c_analytic_deg']:.4f}°")
    assert lines[3].startswith(f"measured: b_c = {g['b_c_measured']:.6f}, α_c = ")
    assert lines[3].endswith(f"{g['alpha_c_measured_deg']:.4f}°")
    rel = float(lines[4].split(": ")[1])
    assert abs(rel - g["rel_err"]) < 5e-10 and lines[5] == "PASS (< 1% error)"


def png_pixels(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", 0
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert zlib.crc32(tag + body) == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[j * (3 * w + 1) + 1:(j + 1) * (3 * w + 1)] for j in range(h)]
    return np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(h, w, 3)


@pytest.mark.gpu
def test_render_program(programs, geon, tmp_path):
    out = tmp_path / "sub" / "s.png"
    r = subprocess.run([programs["render"], "--metric", "schwarzschild", "--width", "64", "--height", "48",
                        "--max-steps", "5000", "--out", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "rendering Schwarzschild @ 64x48, fov 60°, r_obs 20, step 0.05"
    m = geon.Schwarzschild(1.0)
    cam = geon.Camera([0.0, 20.0, np.pi / 2, 0.0], 60.0, 64, 48)
    rgb8, st = geon.render_u8(m, cam, geon.RenderConfig(max_steps=5000, show_stars=True))
    assert lines[1] == (f"done. captured={st.captured}, escaped={st.escaped}, diverged={st.diverged}, "
                        f"avg_steps={st.avg_steps:.1f}, max_null_residual="
                        + f"{st.max_null_residual:.3e}".replace("e-0", "e-").replace("e+0", "e").replace("e+", "e"))
    assert lines[2] == f"wrote {out}"
    assert np.array_equal(png_pixels(out), rgb8)
