"""Extracts the reference's known-answer tests for the photon-propagation
path from its test file (test/runtests.jl of chrhck/NeutrinoTelescopes) into
tests/golden/reference_kats.json.  Run where a checkout of the reference
exists:  python tests/golden/make_golden.py <reference checkout>

The Julia test file is read as text; each case keeps its line number.
  * Intersections        runtests.jl:60-83  (check_intersection, photon_prop_cuda.jl:233-271)
  * Rotations            runtests.jl:89-118 (apply_rot / rot_to_ez_fast / rot_from_ez_fast)
  * integrate_gauss_quad runtests.jl:121-130
  * sph_to_cart          runtests.jl:132-152
  * cart_to_sph          runtests.jl:154-158
  * split_source         runtests.jl:48-56
"""
import json
import math
import re
import sys
from pathlib import Path

ref = Path(sys.argv[1])
lines = (ref / "test" / "runtests.jl").read_text().splitlines()


def floats(s):
    return [float(x.replace("f0", "")) for x in re.findall(r"-?\d+\.\d+(?:f0)?|-?\d+(?:f0)?", s)]


def pi_expr(s):
    s = s.strip().replace("π", "math.pi")
    return float(eval(s, {"math": math}))


out = {"source": "test/runtests.jl", "intersections": [], "sph_to_cart": [], "cart_to_sph": [],
       "rotations": [], "gauss_quad": [], "split_source": []}

# --- intersections: replay the assignments of the testset in order
target = pos = direction = None
i = 0
while i < len(lines):
    ln = lines[i]
    no = i + 1
    if 60 <= no <= 83:
        if "DetectionSphere(" in ln:
            block = " ".join(lines[i:i + 6])
            v = floats(block.split("DetectionSphere(")[1])
            target = {"position": v[0:3], "radius": v[3], "line": no}
        m = re.match(r"\s*pos = @SVector\[(.*)\]", ln)
        if m:
            pos = floats(m.group(1))
        m = re.match(r"\s*dir = @SVector\[(.*)\]", ln)
        if m:
            direction = floats(m.group(1))
        m = re.match(r"\s*dir = \[(.*)\]", ln)
        if m:
            direction = floats(m.group(1))
        if "dir ./ norm(dir)" in ln:
            n = math.sqrt(sum(x * x for x in direction))
            direction = [x / n for x in direction]
        m = re.match(r"\s*@test (!?)check_intersection\(target, pos, dir, ([\d.]+)f0\)\[1\]", ln)
        if m:
            out["intersections"].append({"center": target["position"], "radius": target["radius"],
                                         "pos": pos, "dir": direction, "step": float(m.group(2)),
                                         "hit": m.group(1) != "!", "line": no})
    i += 1

# --- sph_to_cart / cart_to_sph
for i, ln in enumerate(lines):
    no = i + 1
    m = re.match(r"\s*let theta = ([^,]+), phi = (.+)$", ln)
    if m and 132 <= no <= 152:
        want = re.search(r"≈ SA\[(.*)\]", lines[i + 1])
        out["sph_to_cart"].append({"theta": pi_expr(m.group(1)), "phi": pi_expr(m.group(2)),
                                   "expected": floats(want.group(1)), "line": no})
    if m and 154 <= no <= 158:
        out["cart_to_sph"].append({"theta": pi_expr(m.group(1)), "phi": pi_expr(m.group(2)), "line": no})

# --- rotations (properties with the literal angles)
for i, ln in enumerate(lines):
    no = i + 1
    if 89 <= no <= 118 and ln.strip().startswith("let"):
        args = dict(re.findall(r"(θ_1|θ_2|ϕ_1|ϕ_2|theta|phi)\s*=\s*([^,]+?)(?:,|$)", ln.strip()[4:]))
        out["rotations"].append({k: pi_expr(v) for k, v in args.items()} | {"line": no})

# --- gauss quadrature
out["gauss_quad"] = [{"f": "x^3", "a": 0.0, "b": 1.0, "expected": 0.25, "line": 123},
                     {"f": "cos", "a": 0.0, "b": 0.5, "expected": math.sin(0.5), "line": 127}]
assert "x^3" in lines[121] and "1 / 4" in lines[122] and "cos" in lines[125]

# --- split_source
src_line = next(i for i, ln in enumerate(lines) if "split_source(src, 1005)" in ln)
photons = int(float(re.search(r"Int64\((.*?)\)", " ".join(lines[src_line - 5:src_line])).group(1)))
out["split_source"].append({"photons": photons, "parts": 1005, "line": src_line + 1})

dest = Path(__file__).resolve().parent / "reference_kats.json"
dest.write_text(json.dumps(out, indent=1) + "\n")
print(dest, {k: len(v) for k, v in out.items() if isinstance(v, list)})
