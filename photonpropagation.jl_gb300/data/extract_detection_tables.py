"""Extract the DOM and generic multi-PMT detection tables from the reference's
assets (run once; the committed CSVs are what the package reads).

* assets/as.set50_p0=-0.27_p1=-0.042 -> dom_angular_acceptance.csv: the
  polynomial's maximum, then its coefficients in ascending powers of
  cos(zenith) (DOMAcceptance, src/dom.jl:14-26).
* assets/icecube_wl_acc.csv -> dom_wl_acceptance.csv (wavelength, acceptance):
  the effective area divided by the DOM's cross-section pi * 0.16510^2, as
  DOMAcceptance stores it (src/dom.jl:19-23).
* assets/R6091_relqe.csv -> multipmt_qe.csv (wavelength, qe): QE / 100, the
  InterpQuantumEff that make_generic_multipmt_om reads (src/generic_multipmt.jl:36,
  src/detection.jl:170-184 with relative = false).

Usage: python extract_detection_tables.py [reference_root]
"""
import csv
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DOM_RADIUS = 0.16510


def _columns(path):
    with open(path, newline="") as f:
        rows = list(csv.DictReader(f))
    return {k: [float(r[k]) for r in rows] for k in rows[0]}


def main(root):
    assets = os.path.join(root, "assets")
    with open(os.path.join(assets, "as.set50_p0=-0.27_p1=-0.042")) as f:
        values = [float(line) for line in f if line.strip()]
    with open(os.path.join(HERE, "dom_angular_acceptance.csv"), "w") as f:
        f.write("# polymax, then coefficients in ascending powers of cos(zenith)\n")
        for v in values:
            f.write(f"{v!r}\n")

    wl = _columns(os.path.join(assets, "icecube_wl_acc.csv"))
    area = math.pi * DOM_RADIUS ** 2
    with open(os.path.join(HERE, "dom_wl_acceptance.csv"), "w") as f:
        f.write("wavelength,acceptance\n")
        for w, a in zip(wl["wl"], wl["acc"]):
            f.write(f"{w!r},{a / area!r}\n")

    qe = _columns(os.path.join(assets, "R6091_relqe.csv"))
    with open(os.path.join(HERE, "multipmt_qe.csv"), "w") as f:
        f.write("wavelength,qe\n")
        for w, q in zip(qe["wavelength"], qe["QE"]):
            f.write(f"{w!r},{q / 100.0!r}\n")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PP_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s <reference checkout> (or set PP_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
