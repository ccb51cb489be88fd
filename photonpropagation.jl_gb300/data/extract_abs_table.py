"""Regenerate attenuation_length_straw_fit.csv from PhotonPropagation.jl's
asset assets/attenuation_length_straw_fit.parquet (the STRAW absorption-length
fit used by CascadiaMediumProperties, src/water_properties.jl:29-31,66-69).

Usage: python extract_abs_table.py <path to the reference checkout>
"""
import os
import sys

import pyarrow.parquet as pq


def main(ref_root: str) -> None:
    t = pq.read_table(os.path.join(ref_root, "assets", "attenuation_length_straw_fit.parquet"))
    d = t.to_pydict()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                       "attenuation_length_straw_fit.csv")
    with open(out, "w") as f:
        f.write("# wavelength_nm,abs_len_m (PhotonPropagation.jl assets/attenuation_length_straw_fit.parquet)\n")
        for wl, al in zip(d["wavelength"], d["abs_len"]):
            f.write(f"{wl!r},{al!r}\n")
    print(out, len(d["wavelength"]), "rows")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PP_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s <reference checkout> (or set PP_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
