"""Regenerates the two measurement tables this package ships, from the
reference's assets (run where a checkout of chrhck/NeutrinoTelescopes exists):

  straw_abs_len.csv    assets/attenuation_length_straw_fit.parquet  (101 knots,
                       absorption length in m vs wavelength in nm; read by
                       AbsLengthStrawFromFit, src/photon_propagation/medium.jl:392-404)
  pmt_acceptance.csv   assets/PMTAcc.csv  (56 knots, single-PMT wavelength
                       acceptance; read at src/photon_propagation/detection.jl:161-163)

Usage: python make_tables.py <path to the reference checkout>
"""
import sys
from pathlib import Path

import pyarrow.parquet as pq

here = Path(__file__).resolve().parent
root = Path(sys.argv[1])
t = pq.read_table(root / "assets" / "attenuation_length_straw_fit.parquet").to_pydict()
with open(here / "straw_abs_len.csv", "w") as f:
    f.write("wavelength_nm,abs_len_m\n")
    for w, a in zip(t["wavelength"], t["abs_len"]):
        f.write(f"{w!r},{a!r}\n")
with open(here / "pmt_acceptance.csv", "w") as f:
    f.write("wavelength_nm,acceptance\n")
    for line in (root / "assets" / "PMTAcc.csv").read_text().splitlines():
        if line.strip():
            w, a = (float(x) for x in line.split(","))
            f.write(f"{w!r},{a!r}\n")
