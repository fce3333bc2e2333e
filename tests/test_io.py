"""Host-side I/O of the C ABI (no GPU): .stinput reader and the write_output CSV format."""
import os

import numpy as np
import pytest

from optixsoltracedemos_gb300 import native, scenes
from tests.golden import cases

# the reference's own .stinput fixture, read where CSP_REFERENCE_DIR names the reference checkout
REF_TOY = os.path.join(os.environ.get("CSP_REFERENCE_DIR", ""), "data", "stinput", "toy_problem_parabolic.stinput")


def _write_stinput(path, elements, sun, sigma_mrad, optics=True):
    """Write a SolTrace .stinput (version 2012.7.6 layout) for a scene: heliostats in stage 1 and
    the receiver in stage 2.  Cylinder receivers use the 'l'/'t' section type (radius as 1/tok[18],
    origin y shifted back by the radius) followed by the two end caps ('c'/'f') that readers skip."""
    L = ["# SOLTRACE VERSION 2012.7.6 INPUT FILE -- GENERATED BY test_io",
         f"SUN\tPTSRC\t0\tSHAPE\tp\tSIGMA\t{sigma_mrad:f}\tHALFWIDTH\t{sigma_mrad:f}",
         f"XYZ\t{sun[0]:f}\t{sun[1]:f}\t{sun[2]:f}\tUSELDH\t0\tLDH\t0.000000\t0.000000\t0.000000",
         "USER SHAPE DATA\t2", "0.0\t1.0", "4.65\t1.0",
         "OPTICS LIST COUNT\t2",
         "OPTICAL PAIR\tReflector",
         "OPTICAL\tg\t3\t1\t4\t0.930000\t0.000000\t1.500000\t0.200000\t0\t0\t0\t0\t0\t0\t1\t2",
         "0.0 0.93", "90.0 0.90",
         "OPTICAL\tg\t3\t1\t4\t0.960000\t0.000000\t0.950000\t0.200000\t0\t0\t0\t0\t0\t0",
         "OPTICAL PAIR\tAbsorber",
         "OPTICAL\tg\t3\t1\t4\t0.000000\t0.000000\t0.950000\t0.200000\t0\t0\t0\t0\t0\t0",
         "OPTICAL\tg\t3\t1\t4\t0.960000\t0.000000\t0.950000\t0.200000\t0\t0\t0\t0\t0\t0",
         "STAGE LIST COUNT\t2"]
    n = len(elements) - 1

    def elem_line(e, recv):
        o, a = e["origin"], e["aim_point"]
        if int(e["surface"]) == scenes.SURFACE_CYLINDER:
            r = float(e["width"]) / 2
            geo = ["l", "0", "0", f"{float(e['height']):f}"] + ["0"] * 5 + ["t", f"{1 / r:.12g}", "0"] + ["0"] * 6
            o = (o[0], o[1] - r, o[2])
        else:
            surf = "p" if int(e["surface"]) == scenes.SURFACE_PARABOLIC else "f"
            geo = ["r", f"{float(e['width']):f}", f"{float(e['height']):f}"] + ["0"] * 6 + \
                  [surf, f"{float(e['curv_x']):f}", f"{float(e['curv_y']):f}"] + ["0"] * 6
        vals = ["1", *(f"{v:.9f}" for v in o), *(f"{v:.9f}" for v in a), f"{float(e['zrot_deg']):f}", *geo,
                "", "Absorber" if recv else "Reflector", "2"]
        return "\t".join(vals) + "\t"

    L.append(f"STAGE\tXYZ\t0\t0\t0\tAIM\t0\t0\t1\tZROT\t0\tVIRTUAL\t0\tMULTIHIT\t1\tELEMENTS\t{n}\tTRACETHROUGH\t0")
    L.append("Heliostat field")
    L += [elem_line(e, False) for e in elements[:-1]]
    recv = elements[-1]
    caps = 2 if int(recv["surface"]) == scenes.SURFACE_CYLINDER else 0
    L.append(f"STAGE\tXYZ\t0\t0\t0\tAIM\t0\t0\t1\tZROT\t0\tVIRTUAL\t0\tMULTIHIT\t1\tELEMENTS\t{1 + caps}\tTRACETHROUGH\t0")
    L.append("Receiver")
    L.append(elem_line(recv, True))
    for _ in range(caps):
        L.append("\t".join(["1", "0", "0", "0", "0", "0", "1", "0", "c", "1", "0", "0"] + ["0"] * 5 +
                           ["f"] + ["0"] * 8 + ["", "Absorber", "2"]) + "\t")
    with open(path, "w") as f:
        f.write("\r\n".join(L) + "\r\n")


@pytest.mark.parametrize("sc", [scenes.three_heliostats(), scenes.single_parabolic(),
                                scenes.large_field(n_heliostats=50)], ids=lambda s: s.name)
def test_stinput_roundtrip(native_lib, tmp_path, sc):
    p = str(tmp_path / "scene.stinput")
    _write_stinput(p, sc.elements, sc.sun_dir, 4.65)
    el, sun, ang = native.parse_stinput(p)
    assert len(el) == len(sc.elements)
    np.testing.assert_allclose(sun, sc.sun_dir, atol=1e-6)
    assert ang == pytest.approx(4.65e-3)
    for f in ("origin", "aim_point", "width", "height", "curv_x", "curv_y", "zrot_deg"):
        np.testing.assert_allclose(el[f], sc.elements[f], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(el["surface"], sc.elements["surface"])
    # the reference discards the optical pairs ...
    assert np.all(el["reflectivity"] == 1.0) and np.all(el["slope_error"] == 0.0)
    # ... unless asked: front surface of each element's named pair
    el2, _, _ = native.parse_stinput(p, apply_optics=True)
    assert np.all(el2["reflectivity"][:-1] == 0.93)
    assert np.allclose(el2["slope_error"][:-1], 1.5e-3)
    assert el2["reflectivity"][-1] == 0.0


def test_stinput_errors(native_lib, tmp_path):
    bad = tmp_path / "bad.stinput"
    bad.write_text("SOLTRACE without the hash\n")
    with pytest.raises(native.CspError) as e:
        native.parse_stinput(str(bad))
    assert e.value.status == -8
    with pytest.raises(native.CspError) as e:
        native.parse_stinput(str(tmp_path / "missing.stinput"))
    assert e.value.status == -7
    sc = scenes.three_heliostats()
    p = str(tmp_path / "trunc.stinput")
    _write_stinput(p, sc.elements, sc.sun_dir, 4.65)
    txt = open(p).read().replace("\tr\t1.000000", "\tq\t1.000000", 1)   # unknown aperture letter
    open(p, "w").write(txt)
    with pytest.raises(native.CspError):
        native.parse_stinput(p)


@pytest.mark.skipif(not os.environ.get("CSP_REFERENCE_DIR") or not os.path.exists(REF_TOY),
                    reason="CSP_REFERENCE_DIR does not name the reference checkout")
def test_reference_toy_stinput(native_lib):
    el, sun, ang = native.parse_stinput(REF_TOY)
    exp = cases.toy_problem_parabolic()[0]
    np.testing.assert_allclose(sun, exp.sun_dir)
    assert ang == pytest.approx(4.65e-3)
    for f in ("origin", "aim_point", "width", "height", "curv_x", "curv_y", "zrot_deg"):
        np.testing.assert_allclose(el[f], exp.elements[f], atol=1e-9)
    np.testing.assert_array_equal(el["surface"], exp.elements["surface"])


def reference_csv_rows(hits, max_depth=5):
    """Line-by-line restatement of SolTraceSystem::write_output (lib/soltrace_system.cpp:221-255)."""
    rows, current, stage = [], 1, 0
    for r in hits.reshape(-1, 4):
        if r[1] == 0 and r[2] == 0 and r[3] == 0:
            if stage > 0:
                current += 1
                stage = 0
            continue
        if stage < max_depth:
            rows.append(f"{current},{r[0]:g},{r[1]:g},{r[2]:g},{r[3]:g}")
            stage += 1
        else:
            current += 1
            stage = 0
            rows.append(f"{current},{r[0]:g},{r[1]:g},{r[2]:g},{r[3]:g}")
            stage += 1
    return rows


def test_csv_writer_matches_reference_format(native_lib, tmp_path, oracle32):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "three_heliostats.npz"))
    hits = g["hits"].copy()
    # exercise the corner cases of the format: a ray with all five slots used, an all-zero ray
    hits[3] = [[0, 1.5, 2.5, 3.5], [1, 1e-7, -0.0, 123456789.0], [1, 4, 5, 6], [1, 7, 8, 9], [2, 1, 2, 3]]
    hits[4] = 0
    hits[5, 0] = [0, 0, 0, 1e-30]
    p = str(tmp_path / "out.csv")
    native.write_hits_csv(hits, p)
    lines = open(p).read().splitlines()
    assert lines[0] == "number,stage,loc_x,loc_y,loc_z"
    assert lines[1:] == reference_csv_rows(hits)
    # large input takes the multi-block path
    big = np.tile(hits, (300, 1, 1))
    native.write_hits_csv(big, p)
    assert open(p).read().splitlines()[1:] == reference_csv_rows(big)


def test_csv_float_text_equals_stream_format(tmp_path):
    """The CSV writer's float formatter (csp_format.h) gives the text of std::to_chars with six
    significant digits in general format (the C++ stream default the reference's writer uses) on
    every 97th float bit pattern and next to every power of ten (a host program compiled from the
    formatter's header; the whole 2^32 range passes with stride 1)."""
    import shutil
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "format_g6_check")
    subprocess.run([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-pthread", "-I",
                    os.path.join(root, "optixsoltracedemos_gb300", "csrc"),
                    os.path.join(root, "tests", "cpp", "format_g6_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "97"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert r.stdout.strip().endswith("0 mismatches"), r.stdout[-500:]
