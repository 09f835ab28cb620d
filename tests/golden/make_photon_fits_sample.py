"""Extracts a slice of the reference's statistical fixture
assets/photon_fits.parquet (chrhck/NeutrinoTelescopes) into
tests/golden/photon_fits_sample.json.  Run where a checkout of the reference
exists:  python tests/golden/make_photon_fits_sample.py <reference checkout>

The fixture holds, per (distance, observation angle), the fraction of the
photons of a point-like Cherenkov emitter at the origin that is detected by a
module at (0, 0, distance), weighted by absorption and the PMT acceptance
(det_fraction = sum(abs_weight * p_one_pmt_acc(wavelength)) / photons, from
make_photon_fits / fit_photon_dist, src/photon_propagation/modelling.jl:60-167,
Cascadia Basin water, Frank-Tamm spectrum 300-800 nm).  Kept: every row at
the three distances closest to 10, 25 and 50 m (250 observation angles each).
"""
import json
import sys
from pathlib import Path

import numpy as np
import pyarrow.parquet as pq

ref = Path(sys.argv[1])
t = pq.read_table(ref / "assets" / "photon_fits.parquet").to_pydict()
dist = np.asarray(t["distance"])
angle = np.asarray(t["obs_angle"])
frac = np.asarray(t["det_fraction"])
levels = np.unique(dist)
out = {"source": "assets/photon_fits.parquet", "rows": []}
for want in (10.0, 25.0, 50.0):
    d = levels[np.argmin(np.abs(levels - want))]
    sel = np.flatnonzero(dist == d)
    sel = sel[np.argsort(angle[sel])]
    for i in sel:
        out["rows"].append([float(dist[i]), float(angle[i]), float(frac[i])])
Path(__file__).with_name("photon_fits_sample.json").write_text(json.dumps(out))
print(len(out["rows"]), "rows")
